// Geometry set-up: level-set normals and cell types (Src/Geometry/
// Level_Set.cpp:79-167), the compacted list of ghost-fluid cells, and the
// per-ghost boundary data of each variant (Scheme_Index: IDWBaseGFM/
// GFM_Method.cpp:5-113, LinearBaseGFM/GFM_Method.cpp:5-47, BCGFM/
// BCGFM_Method.cpp:7-210, HBCGFM/HBCGFM_Method.cpp).
//
// Coordinates are not stored: x_i = Li + i*dx and y_j = Hi + j*dx are
// recomputed with the same operations as Src/Geometry/Psy_coord.cpp:42-43,
// so every derived value is bit-identical to the reference's.  The image-
// point bracket search of Src/Geometry/Mirror_IDX.cpp:20-62 (a linear scan
// of the whole row/column, last match wins, unchanged when nothing matches)
// becomes index arithmetic plus a check of the neighbouring brackets with
// the exact coordinate values, which selects the same bracket.
#include <algorithm>
#include <vector>

#include "internal.h"

namespace ibtfo {

__device__ __forceinline__ double xc(const GridDesc &g, int i) { return g.Li + i * g.dx; }
__device__ __forceinline__ double yc(const GridDesc &g, int j) { return g.Hi + j * g.dx; }

__global__ void normals_kernel(GridDesc g, const double *__restrict__ phi, double *nx, double *ny)
{
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)g.M * g.N)
        return;
    int j = (int)(c / g.M), i = (int)(c - (long long)j * g.M);
    long long o = (long long)j * g.pitch + i;
    double vx = 0.0, vy = 0.0;
    if (j >= 1 && j < g.N - 1 && i >= 1 && i < g.M - 1)
    {
        vx = (phi[o + 1] - phi[o - 1]) / ((xc(g, i + 1) - xc(g, i - 1)));
        vy = (phi[o + g.pitch] - phi[o - g.pitch]) / ((yc(g, j + 1) - yc(g, j - 1)));
    }
    nx[o] = vx;
    ny[o] = vy;
}

// 0 fluid (phi >= 0), 1 solid, 2 ghost: a solid cell within ng cells of an
// interior fluid cell along x or y, and every cell of the domain-edge ring.
__global__ void types_kernel(GridDesc g, const double *__restrict__ phi, uint8_t *type)
{
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)g.M * g.N)
        return;
    int j = (int)(c / g.M), i = (int)(c - (long long)j * g.M);
    long long o = (long long)j * g.pitch + i;
    auto interior = [&](int ii, int jj) { return ii >= g.ng && ii < g.ng + g.n_x && jj >= g.ng && jj < g.ng + g.n_y; };
    uint8_t t;
    if (!interior(i, j))
        t = 2;
    else if (phi[o] >= 0)
        t = 0;
    else
    {
        t = 1;
        for (int k = 1; k <= g.ng && t == 1; k++)
        {
            const int ci[4] = {i + k, i - k, i, i};
            const int cj[4] = {j, j, j + k, j - k};
            for (int q = 0; q < 4; q++)
                if (interior(ci[q], cj[q]) && phi[(long long)cj[q] * g.pitch + ci[q]] >= 0)
                    t = 2;
        }
    }
    type[o] = t;
}

// one warp per interior row: number of ghost cells (type 2) in the row
__global__ void ghost_count_kernel(GridDesc g, const uint8_t *__restrict__ type, int *counts)
{
    int j = g.ng + blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (j >= g.ng + g.n_y)
        return;
    int n = 0;
    for (int i0 = g.ng; i0 < g.ng + g.n_x; i0 += 32)
    {
        int i = i0 + lane;
        bool gh = (i < g.ng + g.n_x) && type[(long long)j * g.pitch + i] == 2;
        n += __popc(__ballot_sync(0xffffffffu, gh));
    }
    if (lane == 0)
        counts[j - g.ng] = n;
}

// ordered compaction: ghost cells of row j go to offsets[j] onward, left to right
__global__ void ghost_list_kernel(GridDesc g, const uint8_t *__restrict__ type, const int *offsets, GhostRec *out)
{
    int j = g.ng + blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (j >= g.ng + g.n_y)
        return;
    int base = offsets[j - g.ng];
    for (int i0 = g.ng; i0 < g.ng + g.n_x; i0 += 32)
    {
        int i = i0 + lane;
        bool gh = (i < g.ng + g.n_x) && type[(long long)j * g.pitch + i] == 2;
        unsigned m = __ballot_sync(0xffffffffu, gh);
        if (gh)
        {
            GhostRec r = {};
            r.i = i;
            r.j = j;
            out[base + __popc(m & ((1u << lane) - 1u))] = r;
        }
        base += __popc(m);
    }
}

// Mirror_IDX.cpp:20-35: ii in [0, M-1) with x(ii) <= xm < x(ii+1); `keep` if none
__device__ int bracket_x(const GridDesc &g, double xm, int keep)
{
    double t = (xm - g.Li) / g.dx;
    if (!(t > -4.0 && t < g.M + 4.0))
        return keep;
    int k0 = (int)floor(t);
    int res = keep;
    for (int ii = k0 - 2; ii <= k0 + 2; ii++)
        if (ii >= 0 && ii < g.M - 1 && xm < xc(g, ii + 1) && xm >= xc(g, ii))
            res = ii;
    return res;
}

// Mirror_IDX.cpp:43-58 (column-0 y coordinates, jj in [0, N-1))
__device__ int bracket_y(const GridDesc &g, double ym, int keep)
{
    double t = (ym - g.Hi) / g.dx;
    if (!(t > -4.0 && t < g.N + 4.0))
        return keep;
    int k0 = (int)floor(t);
    int res = keep;
    for (int jj = k0 - 2; jj <= k0 + 2; jj++)
        if (jj >= 0 && jj < g.N - 1 && ym < yc(g, jj + 1) && ym >= yc(g, jj))
            res = jj;
    return res;
}

// inverse distance weights of the four corners (IDWBaseGFM/GFM_Method.cpp:77-116,
// BCGFM_Method.cpp:106-145 with the `!= 1` corner test)
__device__ void idw_weights(const GridDesc &g, const uint8_t *type, int idx, int idy, double xm, double ym,
                            bool ne_one, double w[4])
{
    const int ci[4] = {idx, idx, idx + 1, idx + 1};
    const int cj[4] = {idy, idy + 1, idy + 1, idy};
    for (int q = 0; q < 4; q++)
    {
        int t = type[(long long)cj[q] * g.pitch + ci[q]];
        w[q] = 0.0;
        if (ne_one ? (t != 1) : (t < 1))
        {
            double ddx = xc(g, ci[q]) - xm, ddy = yc(g, cj[q]) - ym;
            double d = sqrt(ddx * ddx + ddy * ddy);
            w[q] = 1 / d;
        }
    }
}

// LinearBaseGFM/GFM_Bound.cpp:116-575: corner chosen by the fluid pattern and
// by x_d (its y_d is also computed from x, :100-101); 0 when no corner is fluid
__device__ int linear_pick(int t1, int t2, int t3, int t4, bool xbig, bool ybig)
{
    const bool f1 = t1 < 1, f2 = t2 < 1, f3 = t3 < 1, f4 = t4 < 1;
    if (f1 && f4 && f2 && f3) return ybig ? (xbig ? 3 : 2) : (xbig ? 4 : 1);
    if (!f1 && f4 && f2 && f3) return ybig ? (xbig ? 3 : 2) : 4;
    if (f1 && !f4 && f2 && f3) return ybig ? (xbig ? 3 : 2) : 1;
    if (f1 && f4 && !f2 && f3) return ybig ? 3 : (xbig ? 4 : 1);
    if (f1 && f4 && f2 && !f3) return ybig ? 2 : (xbig ? 4 : 1);
    if (f1 && f4 && !f2 && !f3) return xbig ? 4 : 1;
    if (!f1 && !f4 && f2 && f3) return xbig ? 3 : 2;
    if (f1 && !f4 && f2 && !f3) return ybig ? 2 : 1;
    if (!f1 && f4 && !f2 && f3) return ybig ? 3 : 4;
    if (f1 && !f4 && !f2 && f3) return ybig ? 3 : 1;
    if (!f1 && f4 && f2 && !f3) return ybig ? 2 : 4;
    if (f1 && !f4 && !f2 && !f3) return 1;
    if (!f1 && !f4 && f2 && !f3) return 2;
    if (!f1 && !f4 && !f2 && f3) return 3;
    if (!f1 && f4 && !f2 && !f3) return 4;
    return 0;
}

// corners c = 0..3 of a bracket, (idx,idy), (idx,idy+1), (idx+1,idy+1),
// (idx+1,idy), whose value the boundary pass takes from the new state: the
// updated interior cells (a static property of the geometry)
__device__ int next_corners(const GridDesc &g, const uint8_t *type, int idx, int idy)
{
    int m = 0;
    for (int c = 0; c < 4; c++)
    {
        const int i = idx + (c >= 2), j = idy + (c == 1 || c == 2);
        const bool in = i >= g.ng && i < g.ng + g.n_x && j >= g.ng && j < g.ng + g.n_y;
        if (in && updated_cell(type[(long long)j * g.pitch + i]))
            m |= 1 << c;
    }
    return m;
}

__global__ void scheme_index_kernel(GridDesc g, int bc, const double *__restrict__ phi, const double *__restrict__ nxa,
                                    const double *__restrict__ nya, const uint8_t *__restrict__ type, GhostRec *gl,
                                    int n)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n)
        return;
    GhostRec r = gl[t];
    const long long o = (long long)r.j * g.pitch + r.i;
    const double x = xc(g, r.i), y = yc(g, r.j);
    const double p = phi[o], nx = nxa[o], ny = nya[o];
    const double ap = fabs(p);
    r.nx = nx;
    r.ny = ny;
    r.rg = ap;
    // grid spacings as the reference reads them from XYCOORD (cells (0,1),(1,1),(1,2))
    const double dxl = xc(g, 1) - xc(g, 0);
    const double dyl = yc(g, 2) - yc(g, 1);
    if (bc == BC_IDW || bc == BC_LINEAR || bc == BC_RIEMANNGFM)
    {
        r.xm = x + 2 * nx * ap;
        r.ym = y + 2 * ny * ap;
        r.idx = bracket_x(g, r.xm, 0);
        r.idy = bracket_y(g, r.ym, 0);
        if (bc == BC_IDW)
            idw_weights(g, type, r.idx, r.idy, r.xm, r.ym, false, r.w);
        else
        {
            auto T = [&](int ii, int jj) { return (int)type[(long long)jj * g.pitch + ii]; };
            double x_d = r.xm - xc(g, r.idx);
            double y_d = r.xm - xc(g, r.idx);
            r.pick = linear_pick(T(r.idx, r.idy), T(r.idx, r.idy + 1), T(r.idx + 1, r.idy + 1), T(r.idx + 1, r.idy),
                                 x_d > dxl / 2, y_d > dyl / 2);
        }
    }
    else
    {
        const double delta = sqrt(dxl * dxl + dyl * dyl) / 2;
        r.delta = delta;
        if (bc == BC_HBCGFM && ap > delta)
        {
            r.hmirror = 1;
            r.xm = x + nx * (2 * ap);
            r.ym = y + ny * (2 * ap);
            r.xm2 = x + nx * (2 * ap);
            r.ym2 = y + ny * (2 * ap);
        }
        else
        {
            r.xm = x + nx * (ap + delta);
            r.ym = y + ny * (ap + delta);
            r.xm2 = x + nx * (ap + 2 * delta);
            r.ym2 = y + ny * (ap + 2 * delta);
        }
        r.idx = bracket_x(g, r.xm, 0);
        r.idy = bracket_y(g, r.ym, 0);
        r.idx2 = bracket_x(g, r.xm2, 0);
        r.idy2 = bracket_y(g, r.ym2, 0);
        idw_weights(g, type, r.idx, r.idy, r.xm, r.ym, true, r.w);
        idw_weights(g, type, r.idx2, r.idy2, r.xm2, r.ym2, true, r.w2);
        r.snext = next_corners(g, type, r.idx2, r.idy2) << 4;
    }
    r.snext |= next_corners(g, type, r.idx, r.idy);
    gl[t] = r;
}

static inline unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// per tx x ty sweep tile: the number of interior fluid (or cut) cells it
// holds, plus TILE_COUNT_INTERIOR when every cell of the tile and of its
// one-cell ring is an interior fluid cell
constexpr int TILE_COUNT_INTERIOR = 1 << 30;
__global__ void tile_counts_kernel(GridDesc g, const uint8_t *__restrict__ type, int tx, int ty, int ntx, int nty,
                                   int *counts)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntx * nty)
        return;
    int bx = t % ntx, by = t / ntx;
    int i0 = g.ng + bx * tx, j0 = g.ng + by * ty;
    int n = 0;
    for (int j = j0; j < j0 + ty && j < g.ng + g.n_y; j++)
        for (int i = i0; i < i0 + tx && i < g.ng + g.n_x; i++)
            n += updated_cell(type[(long long)j * g.pitch + i]) ? 1 : 0;
    bool interior = i0 - 1 >= g.ng && j0 - 1 >= g.ng && i0 + tx < g.ng + g.n_x && j0 + ty < g.ng + g.n_y;
    for (int j = j0 - 1; j <= j0 + ty && interior; j++)
        for (int i = i0 - 1; i <= i0 + tx; i++)
            if (type[(long long)j * g.pitch + i] != CELL_FLUID)
            {
                interior = false;
                break;
            }
    counts[t] = n | (interior ? TILE_COUNT_INTERIOR : 0);
}

int active_tile_list(const GridDesc &g, const uint8_t *d_type, int tx, int ty, std::vector<unsigned> &list,
                     cudaStream_t s, bool row_order)
{
    const int ntx = (g.n_x + tx - 1) / tx, nty = (g.n_y + ty - 1) / ty;
    const int n = ntx * nty;
    int *d_counts = nullptr;
    if (cudaMallocAsync(&d_counts, sizeof(int) * n, s) != cudaSuccess)
        return 2;
    tile_counts_kernel<<<nblk(n, 256), 256, 0, s>>>(g, d_type, tx, ty, ntx, nty, d_counts);
    count_launch();
    std::vector<int> counts(n);
    cudaError_t e = cudaMemcpyAsync(counts.data(), d_counts, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d_counts, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return 5;
    list.clear();
    std::vector<int> work;
    for (int t = 0; t < n; t++)
        if (counts[t])
        {
            const bool interior = (counts[t] & TILE_COUNT_INTERIOR) != 0;
            list.push_back((unsigned)(t % ntx) | ((unsigned)(t / ntx) << 16) | (interior ? TILE_INTERIOR : 0u));
            work.push_back(counts[t] & (TILE_COUNT_INTERIOR - 1));
        }
    if (list.empty())
        list.push_back(0u); // a tile without fluid still runs the loop accounting
    else if (!row_order && tx == TILE_X && ty == FAST_TILE_Y)
    {
        // the 32x16 sweeps solve only the faces their fluid cells read, so a
        // tile's time follows its fluid count: longest first, so that the last
        // CTAs of a launch are the short ones (the row-band list of the
        // host-array step keeps row order)
        std::vector<int> idx(list.size());
        for (size_t k = 0; k < idx.size(); k++)
            idx[k] = (int)k;
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return work[a] > work[b]; });
        std::vector<unsigned> sorted(list.size());
        for (size_t k = 0; k < idx.size(); k++)
            sorted[k] = list[idx[k]];
        list.swap(sorted);
    }
    return 0;
}

int active_tiles(const GridDesc &g, const uint8_t *d_type, int ty, unsigned **d_tiles, int *ntiles, cudaStream_t s,
                 std::vector<unsigned> *host_list, bool row_order)
{
    std::vector<unsigned> list;
    int rc = active_tile_list(g, d_type, TILE_X, ty, list, s, row_order);
    if (rc)
        return rc;
    if (host_list)
        *host_list = list;
    if (*d_tiles)
        cudaFreeAsync(*d_tiles, s);
    *d_tiles = nullptr;
    if (cudaMallocAsync(d_tiles, sizeof(unsigned) * list.size(), s) != cudaSuccess)
        return 2;
    if (cudaMemcpyAsync(*d_tiles, list.data(), sizeof(unsigned) * list.size(), cudaMemcpyHostToDevice, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return 5;
    *ntiles = (int)list.size();
    return 0;
}

int setup_geometry(const GridDesc &g, int bc, const double *d_phi, double *d_nx, double *d_ny, uint8_t *d_type,
                   GhostRec **d_ghosts, int *nghost, cudaStream_t s)
{
    const long long cells = (long long)g.M * g.N;
    normals_kernel<<<nblk(cells, 256), 256, 0, s>>>(g, d_phi, d_nx, d_ny);
    types_kernel<<<nblk(cells, 256), 256, 0, s>>>(g, d_phi, d_type);
    count_launch(2);
    *nghost = 0;
    *d_ghosts = nullptr;
    if (bc == BC_REGULAR)
        return 0;
    int *d_counts = nullptr;
    if (cudaMallocAsync(&d_counts, sizeof(int) * (size_t)g.n_y, s) != cudaSuccess)
        return 2;
    const int rows_per_block = 8;
    ghost_count_kernel<<<nblk(g.n_y, rows_per_block), 32 * rows_per_block, 0, s>>>(g, d_type, d_counts);
    count_launch();
    std::vector<int> counts(g.n_y), offs(g.n_y);
    if (cudaMemcpyAsync(counts.data(), d_counts, sizeof(int) * g.n_y, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
    {
        cudaFreeAsync(d_counts, s);
        return 5;
    }
    long long tot = 0;
    for (int j = 0; j < g.n_y; j++)
    {
        offs[j] = (int)tot;
        tot += counts[j];
    }
    *nghost = (int)tot;
    if (tot == 0)
    {
        cudaFreeAsync(d_counts, s);
        return 0;
    }
    GhostRec *gl = nullptr;
    if (cudaMallocAsync(&gl, sizeof(GhostRec) * (size_t)tot, s) != cudaSuccess)
    {
        cudaFreeAsync(d_counts, s);
        return 2;
    }
    cudaMemcpyAsync(d_counts, offs.data(), sizeof(int) * g.n_y, cudaMemcpyHostToDevice, s);
    ghost_list_kernel<<<nblk(g.n_y, rows_per_block), 32 * rows_per_block, 0, s>>>(g, d_type, d_counts, gl);
    scheme_index_kernel<<<nblk(tot, 128), 128, 0, s>>>(g, bc, d_phi, d_nx, d_ny, d_type, gl, (int)tot);
    count_launch(2);
    cudaError_t e = cudaStreamSynchronize(s);
    cudaFreeAsync(d_counts, s);
    if (e != cudaSuccess)
    {
        cudaFreeAsync(gl, s);
        return 5;
    }
    *d_ghosts = gl;
    return 0;
}

} // namespace ibtfo
