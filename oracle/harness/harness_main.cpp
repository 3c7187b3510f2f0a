// Driver that runs the reference's own solver sources (compiled unmodified
// with g++ and the OpenACC stand-in header) and dumps every array the
// parity tests need in one binary record.
//
// Test infrastructure only: this file is compiled together with the
// reference's Src/ files by oracle/build_ref.py into oracle/_ref/, never
// shipped in the product library.
//
// The call sequence follows the reference time loop:
//   init   Test/InclineSod/InclineSod.cpp:97-105 (Psy_coord, Level_Set,
//          Scheme_Index, Initialize, Boundary), then ComputeDt and
//          CaculateMass (:116-128);
//   loop   Test/InclineSod/InclineSod.cpp:131-189 (TimeAdvance, Boundary,
//          Global_Boundary, ComputeDt, CaculateMass, now_t += new dt, iter++).
// Differences from the reference drivers, all deliberate:
//   * every array is zero-filled after allocation (the reference leaves them
//     uninitialised, Test/Sod/Sod.cpp:61-65), so never-written slots read 0;
//   * the loop stops after `nsteps` iterations (in addition to the reference's
//     now_t < Psy_time and iter < max_iter tests);
//   * no VTK output; Mass_start is initialised (InclineSod.cpp:65 does not).
//
// Usage: harness <case.inp> <nsteps> <out.bin> [phi.bin U0.bin]
//   phi.bin / U0.bin are read by the "file" plug-in (plugin_file.cpp).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>
#include <algorithm>

#include "openacc.h"
#include "EQDefine.H"
#include "CoordDefine.H"
#include "SchDefine.H"
#include "Initialize.H"
#include "CaculateMass.H"
#include "Psy_coord.H"
#include "Level_Set.H"
#include "TimeAdvance.H"
#include "ComputeDt.H"
#include "Boundary.H"
#include "ParamReader.H"
#ifdef HARNESS_HAS_SCHEME_INDEX
#include "Scheme_Index.H"
#endif

const char *harness_phi_path = nullptr;
const char *harness_u0_path = nullptr;

static void put(FILE *f, const void *p, size_t bytes)
{
    if (bytes && fwrite(p, 1, bytes, f) != bytes)
    {
        fprintf(stderr, "harness: short write\n");
        exit(3);
    }
}

int main(int argc, char **argv)
{
    if (argc < 4)
    {
        fprintf(stderr, "usage: %s case.inp nsteps out.bin [phi.bin U0.bin]\n", argv[0]);
        return 2;
    }
    char *filename = argv[1];
    const int nsteps = atoi(argv[2]);
    const char *out_path = argv[3];
    if (argc >= 6)
    {
        harness_phi_path = argv[4];
        harness_u0_path = argv[5];
    }

    ParamReader DetectParams;
    Params<double> para(DetectParams.open(filename).numbers());
    const int max_iter = int(para.get("max_iter", 100000));
    const double lo_x = para.get("lo_x", 0);
    const double lo_y = para.get("lo_y", 0);
    const double hi_x = para.get("hi_x", 1);
    const double hi_y = para.get("hi_y", 1);
    const int N_x = int(para.get("N_x", 500));
    const int N_y = int(para.get("N_y", 200));
    const double Psy_time = para.get("Psy_time", 1.0);
    const double CFL_number = para.get("CFL_number", 0.3);
    const int num_ghost_cell = int(para.get("num_ghost_cell", 2));
    const double gamma = para.get("gamma", 1.4);

    const double Psy_L = hi_x - lo_x;
    const double Psy_H = hi_y - lo_y;
    const long cells = (long)(M) * (long)(N);

    // value-initialised (zero) allocations
    double *U_OLD = new double[cells * num_eq]();
    double *U_NEW = new double[cells * num_eq]();
    double *U_TMP = new double[cells * num_tmp_size]();
    double *XYCOORD = new double[cells * num_coord]();
    double *SCHEME_IDX = new double[cells * num_sch]();
    std::vector<double> phi(cells), u_init(cells * num_eq);
    std::vector<double> dts, masses;

    const int ndevices = 1, device = 0;
    double TMP_DT[1] = {0.0}, MASS_DEVICE[1] = {0.0};
    double now_t = 0.0, dt = 0.0;
    int iter = 0;

    Psy_coord(lo_x, lo_y, Psy_L, Psy_H, N_x, N_y, num_ghost_cell, XYCOORD, ndevices, device);
    Level_Set(filename, N_x, N_y, num_ghost_cell, XYCOORD, ndevices, device);
    for (long c = 0; c < cells; c++)
        phi[c] = XYCOORD[c * num_coord + 2];
#ifdef HARNESS_HAS_SCHEME_INDEX
    Scheme_Index(N_x, N_y, num_ghost_cell, XYCOORD, SCHEME_IDX, ndevices, device);
#endif
    Initialize(filename, Psy_L, Psy_H, N_x, N_y, num_ghost_cell, gamma, U_OLD, U_NEW, XYCOORD, ndevices, device);
    std::memcpy(u_init.data(), U_OLD, sizeof(double) * cells * num_eq);
    Boundary(N_x, N_y, num_ghost_cell, gamma, U_OLD, U_NEW, XYCOORD, SCHEME_IDX, ndevices, device);

    ComputeDt(Psy_L, Psy_H, N_x, N_y, num_ghost_cell, gamma, CFL_number, U_OLD, XYCOORD, TMP_DT, ndevices, device);
    CaculateMass(Psy_L, Psy_H, N_x, N_y, num_ghost_cell, U_OLD, XYCOORD, MASS_DEVICE, ndevices, device);
    dt = TMP_DT[0];
    dts.push_back(dt);
    masses.push_back(MASS_DEVICE[0]);

    while (now_t < Psy_time && iter < max_iter && iter < nsteps)
    {
        TimeAdvance(Psy_L, Psy_H, N_x, N_y, num_ghost_cell, gamma, dt, U_OLD, U_TMP, U_NEW, XYCOORD, SCHEME_IDX, ndevices, device);
        Boundary(N_x, N_y, num_ghost_cell, gamma, U_OLD, U_NEW, XYCOORD, SCHEME_IDX, ndevices, device);
        Global_Boundary(N_x, N_y, num_ghost_cell, gamma, U_OLD, U_NEW, ndevices, device);
        ComputeDt(Psy_L, Psy_H, N_x, N_y, num_ghost_cell, gamma, CFL_number, U_OLD, XYCOORD, TMP_DT, ndevices, device);
        CaculateMass(Psy_L, Psy_H, N_x, N_y, num_ghost_cell, U_OLD, XYCOORD, MASS_DEVICE, ndevices, device);
        dt = TMP_DT[0];
        now_t = now_t + dt;
        iter++;
        dts.push_back(dt);
        masses.push_back(MASS_DEVICE[0]);
    }

    FILE *f = fopen(out_path, "wb");
    if (!f)
    {
        perror(out_path);
        return 3;
    }
    const char magic[8] = {'I', 'B', 'T', 'F', 'O', 'R', 'E', 'F'};
    int32_t hdr[6] = {(int32_t)(M), (int32_t)(N), num_ghost_cell, num_sch, iter, 1};
    put(f, magic, 8);
    put(f, hdr, sizeof(hdr));
    double tail[2] = {now_t, dt};
    put(f, tail, sizeof(tail));
    put(f, dts.data(), sizeof(double) * dts.size());
    put(f, masses.data(), sizeof(double) * masses.size());
    put(f, phi.data(), sizeof(double) * cells);
    put(f, u_init.data(), sizeof(double) * cells * num_eq);
    put(f, XYCOORD, sizeof(double) * cells * num_coord);
    put(f, SCHEME_IDX, sizeof(double) * cells * num_sch);
    put(f, U_OLD, sizeof(double) * cells * num_eq);
    put(f, U_NEW, sizeof(double) * cells * num_eq);
    fclose(f);
    return 0;
}
