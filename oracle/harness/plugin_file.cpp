// "File" plug-in for the reference harness: the per-case Level_Set_function
// and Initialize hooks (interfaces Src/Geometry/Level_Set_function.H:13-19 and
// Src/Base/Common/Initialize.H:12-23) read the level set phi and the initial
// conserved state from binary files written by the fixture generator, so any
// case defined in Python can be run through the reference's own solver.
// Test infrastructure only (built into oracle/_ref/ by oracle/build_ref.py).
//
// phi.bin: M*N doubles, index j*M+i.  U0.bin: M*N*4 doubles, index (j*M+i)*4+k.
#include <cstdio>
#include <cstdlib>
#include "Level_Set_function.H"
#include "Initialize.H"

extern const char *harness_phi_path;
extern const char *harness_u0_path;

static void read_all(const char *path, double *dst, long count)
{
    FILE *f = path ? fopen(path, "rb") : nullptr;
    if (!f || fread(dst, sizeof(double), count, f) != (size_t)count)
    {
        fprintf(stderr, "plugin_file: cannot read %ld doubles from %s\n", count, path ? path : "(null)");
        exit(4);
    }
    fclose(f);
}

void Level_Set_function(char *filename, const int N_x, const int N_y, const int num_ghost_cell,
                        double *XYCOORD, const int ndevices, const int device)
{
    const long cells = (long)(M) * (long)(N);
    double *phi = new double[cells];
    read_all(harness_phi_path, phi, cells);
    for (long c = 0; c < cells; c++)
        XYCOORD[c * num_coord + 2] = phi[c];
    delete[] phi;
}

void Initialize(char *filename, const double Psy_L, const double Psy_H, const int N_x, const int N_y,
                const int num_ghost_cell, const double gamma, double *U_OLD, double *U_NEW, double *XYCOORD,
                const int ndevices, const int device)
{
    const long cells = (long)(M) * (long)(N);
    read_all(harness_u0_path, U_OLD, cells * num_eq);
    for (long c = 0; c < cells * num_eq; c++)
        U_NEW[c] = U_OLD[c];
}
