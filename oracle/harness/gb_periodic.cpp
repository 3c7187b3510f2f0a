// Periodic Global_Boundary plug-in (same interface as
// Src/BoundaryCondition/Boundary.H:22-29).  The reference ships only the
// transmissive-x / reflective-y version (Test/Sod/Global_Boudary.cpp:9-77);
// the periodic isentropic-vortex case needs wrap-around ghost layers, defined
// here as: (1) ghost rows of interior columns take U_NEW from the opposite
// interior rows; (2) ghost columns of every row take U_OLD from the opposite
// interior columns (so corner cells come from the diagonal interior cells).
// Test infrastructure only.
#include "Boundary.H"

void Global_Boundary(const int N_x, const int N_y, const int num_ghost_cell, const double gamma,
                     double *U_OLD, double *U_NEW, const int ndevices, const int device)
{
    const int ng = num_ghost_cell;
    for (int j = 0; j < N; j++)
        for (int i = ng; i < N_x + ng; i++)
            for (int k = 0; k < num_eq; k++)
            {
                if (j < ng)
                    U_OLD[Index(i, j, k)] = U_NEW[Index(i, j + N_y, k)];
                if (j >= N_y + ng)
                    U_OLD[Index(i, j, k)] = U_NEW[Index(i, j - N_y, k)];
            }
    for (int j = 0; j < N; j++)
        for (int i = 0; i < ng; i++)
            for (int k = 0; k < num_eq; k++)
            {
                U_OLD[Index(i, j, k)] = U_OLD[Index(i + N_x, j, k)];
                U_OLD[Index(N_x + ng + i, j, k)] = U_OLD[Index(ng + i, j, k)];
            }
}
