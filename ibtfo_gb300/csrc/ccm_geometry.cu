// Cut-cell geometry and small-cell mixing (BC_CCM).  No counterpart in the
// reference, which has no cut-cell method; written from the Cartesian
// cut-cell literature.  All of it in FP64 (it divides by volume fractions).
//
// Geometry from the cell-centred level set phi (positive in the fluid):
//   * corner values: the mean of the four cells around each corner;
//   * aperture of a face: the fraction of the face where the linear
//     interpolation between its two corner values is >= 0;
//   * volume fraction alpha: the area of the polygon formed by the fluid
//     corners of the cell and the crossing points on its edges (shoelace);
//   * type: fluid (all four corners >= 0, alpha = 1), solid (all < 0, or
//     alpha < 1e-10), cut otherwise; faces beside a solid cell get aperture 0.
// Mixing: a cut cell with alpha < 0.5 exchanges with up to three neighbours
// on the fluid side of its wall (n = outward wall normal from the apertures:
// the x neighbour away from the wall with weight nx^2, the y neighbour with
// ny^2, the diagonal one with |nx ny|, solid neighbours dropped, weights
// renormalised): E = beta alpha_s alpha_t / (alpha_s + alpha_t) (U_t - U_s),
// alpha_s U_s += E, alpha_t U_t -= E.  Each exchange is antisymmetric, so the
// total of alpha U is conserved exactly; a single full-weight exchange merges
// the two cells.  The exchanges are computed from the swept state (one
// kernel) and summed per cell in a fixed order (a second kernel), so the
// result does not depend on thread timing.
#include <algorithm>
#include <vector>

#include "internal.h"
#include "physics.cuh"

namespace ibtfo {

static inline unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// fraction of a face with end values a, b where the linear interpolation is >= 0
__host__ __device__ inline double face_aperture(double a, double b)
{
    const bool fa = a >= 0.0, fb = b >= 0.0;
    if (fa && fb)
        return 1.0;
    if (!fa && !fb)
        return 0.0;
    const double t = a / (a - b); // crossing, measured from the a end
    return fa ? t : 1.0 - t;
}

// fluid area of the unit cell with corner values SW, SE, NE, NW
__host__ __device__ inline double cell_fraction(const double v[4])
{
    const double px[4] = {0.0, 1.0, 1.0, 0.0}, py[4] = {0.0, 0.0, 1.0, 1.0};
    double qx[8], qy[8];
    int n = 0;
    for (int k = 0; k < 4; k++)
    {
        const int k1 = (k + 1) & 3;
        if (v[k] >= 0.0)
        {
            qx[n] = px[k];
            qy[n] = py[k];
            n++;
        }
        if ((v[k] >= 0.0) != (v[k1] >= 0.0))
        {
            const double t = v[k] / (v[k] - v[k1]);
            qx[n] = px[k] + t * (px[k1] - px[k]);
            qy[n] = py[k] + t * (py[k1] - py[k]);
            n++;
        }
    }
    double a2 = 0.0;
    for (int k = 0; k < n; k++)
    {
        const int k1 = (k + 1 == n) ? 0 : k + 1;
        a2 += qx[k] * qy[k1] - qx[k1] * qy[k];
    }
    return 0.5 * a2;
}

__device__ inline double corner_phi(const GridDesc &g, const double *phi, int a, int b)
{
    // corner (a + 1/2, b + 1/2)
    const long long o = (long long)b * g.pitch + a;
    return 0.25 * (phi[o] + phi[o + 1] + phi[o + g.pitch] + phi[o + g.pitch + 1]);
}

// alpha, type, and the apertures of the east and north faces of each cell
__global__ void ccm_geom_kernel(GridDesc g, const double *__restrict__ phi, double *alpha, double *ax, double *ay,
                                uint8_t *type)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)g.M * g.N)
        return;
    const int j = (int)(q / g.M), i = (int)(q - (long long)j * g.M);
    const long long o = (long long)j * g.pitch + i;
    const bool interior = i >= g.ng && i < g.ng + g.n_x && j >= g.ng && j < g.ng + g.n_y;
    if (i < 1 || j < 1 || i >= g.M - 1 || j >= g.N - 1)
    {
        alpha[o] = 1.0;
        ax[o] = 1.0;
        ay[o] = 1.0;
        type[o] = CELL_GHOST;
        return;
    }
    const double sw = corner_phi(g, phi, i - 1, j - 1), se = corner_phi(g, phi, i, j - 1),
                 ne = corner_phi(g, phi, i, j), nw = corner_phi(g, phi, i - 1, j);
    ax[o] = face_aperture(se, ne);
    ay[o] = face_aperture(nw, ne);
    if (!interior)
    {
        alpha[o] = 1.0;
        type[o] = CELL_GHOST;
        return;
    }
    const double v[4] = {sw, se, ne, nw};
    const bool all_in = sw >= 0.0 && se >= 0.0 && ne >= 0.0 && nw >= 0.0;
    const bool all_out = sw < 0.0 && se < 0.0 && ne < 0.0 && nw < 0.0;
    double al = all_in ? 1.0 : (all_out ? 0.0 : cell_fraction(v));
    uint8_t t = all_in ? CELL_FLUID : CELL_CUT;
    if (all_out || al < 1e-10)
    {
        t = CELL_SOLID;
        al = 0.0;
    }
    alpha[o] = al;
    type[o] = t;
}

// faces beside a solid cell carry nothing
__global__ void ccm_aperture_fix_kernel(GridDesc g, const uint8_t *__restrict__ type, double *ax, double *ay)
{
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (long long)g.M * g.N)
        return;
    const int j = (int)(q / g.M), i = (int)(q - (long long)j * g.M);
    if (i >= g.M - 1 || j >= g.N - 1)
        return;
    const long long o = (long long)j * g.pitch + i;
    if (type[o] == CELL_SOLID || type[o + 1] == CELL_SOLID)
        ax[o] = 0.0;
    if (type[o] == CELL_SOLID || type[o + g.pitch] == CELL_SOLID)
        ay[o] = 0.0;
}

// one small cut cell's exchanges (up to 3), as the host builds the lists from
struct SmallExchanges
{
    long long s;
    long long t[3];
    double w[3];
    double alpha_s, alpha_t[3];
};

__device__ void small_exchanges(const GridDesc &g, const double *alpha, const double *ax, const double *ay,
                                const uint8_t *type, int i, int j, SmallExchanges &r)
{
    const long long o = (long long)j * g.pitch + i;
    const double as_ = alpha[o];
    r.s = o;
    r.alpha_s = as_;
    for (int k = 0; k < 3; k++)
    {
        r.t[k] = -1;
        r.w[k] = 0.0;
        r.alpha_t[k] = 0.0;
    }
    const double nLx = (ax[o - 1] - ax[o]) * g.dy, nLy = (ay[o - g.pitch] - ay[o]) * g.dx;
    const double L = sqrt(nLx * nLx + nLy * nLy);
    if (!(L > 0.0))
        return;
    const double nx = nLx / L, ny = nLy / L;
    const int sx = (nx > 0.0) ? -1 : 1, sy = (ny > 0.0) ? -1 : 1; // away from the wall
    const int ti[3] = {i + sx, i, i + sx}, tj[3] = {j, j + sy, j + sy};
    const double beta0[3] = {nx * nx, ny * ny, fabs(nx * ny)};
    double beta[3], bsum = 0.0;
    for (int k = 0; k < 3; k++)
    {
        const bool in = ti[k] >= g.ng && ti[k] < g.ng + g.n_x && tj[k] >= g.ng && tj[k] < g.ng + g.n_y;
        const long long ot = (long long)tj[k] * g.pitch + ti[k];
        const bool ok = in && updated_cell(type[ot]) && beta0[k] > 0.0;
        beta[k] = ok ? beta0[k] : 0.0;
        bsum += beta[k];
    }
    if (!(bsum > 0.0))
        return;
    for (int k = 0; k < 3; k++)
    {
        if (beta[k] == 0.0)
            continue;
        const long long ot = (long long)tj[k] * g.pitch + ti[k];
        const double at = alpha[ot];
        r.t[k] = ot;
        r.alpha_t[k] = at;
        r.w[k] = (beta[k] / bsum) * (as_ * at / (as_ + at));
    }
}

__global__ void small_count_kernel(GridDesc g, const double *__restrict__ alpha, const uint8_t *__restrict__ type,
                                   int *counts)
{
    const int row = blockIdx.x * blockDim.y + threadIdx.y;
    if (row >= g.n_y)
        return;
    const int j = row + g.ng;
    int n = 0;
    for (int i = g.ng + threadIdx.x; i < g.ng + g.n_x; i += 32)
    {
        const long long o = (long long)j * g.pitch + i;
        n += (type[o] == CELL_CUT && alpha[o] < 0.5) ? 1 : 0;
    }
    for (int d = 16; d > 0; d >>= 1)
        n += __shfl_xor_sync(0xffffffffu, n, d);
    if (threadIdx.x == 0)
        counts[row] = n;
}

// small cells of each row in column order (one warp per row)
__global__ void small_list_kernel(GridDesc g, const double *__restrict__ alpha, const double *__restrict__ ax,
                                  const double *__restrict__ ay, const uint8_t *__restrict__ type,
                                  const int *__restrict__ offsets, SmallExchanges *out)
{
    const int row = blockIdx.x * blockDim.y + threadIdx.y;
    if (row >= g.n_y)
        return;
    const int j = row + g.ng;
    int base = offsets[row];
    for (int i0 = g.ng; i0 < g.ng + g.n_x; i0 += 32)
    {
        const int i = i0 + threadIdx.x;
        bool small = false;
        if (i < g.ng + g.n_x)
        {
            const long long o = (long long)j * g.pitch + i;
            small = type[o] == CELL_CUT && alpha[o] < 0.5;
        }
        const unsigned m = __ballot_sync(0xffffffffu, small);
        if (small)
            small_exchanges(g, alpha, ax, ay, type, i, j, out[base + __popc(m & ((1u << threadIdx.x) - 1u))]);
        base += __popc(m);
    }
}

// E_k = w_k (U_t - U_s) from the swept state
__global__ void mix_exchange_kernel(const MixArgs a)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.nex || !a.st->fill_pending)
        return;
    const double *buf = a.st->cur ? a.buf1 : a.buf0;
    const MixExchange e = a.ex[k];
    for (int c = 0; c < 4; c++)
        a.e[4 * k + c] = e.w * (state_ld(buf, c, e.t, a.g) - state_ld(buf, c, e.s, a.g));
}

// U_p += sum of its exchanges (+E as the small cell, -E as a target) / alpha_p,
// summed in the fixed order of its link list
__global__ void mix_apply_kernel(const MixArgs a)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.npart || !a.st->fill_pending)
        return;
    double *buf = a.st->cur ? a.buf1 : a.buf0;
    const MixParticipant q = a.part[p];
    for (int c = 0; c < 4; c++)
    {
        double d = 0.0;
        for (int l = 0; l < q.count; l++)
        {
            const int x = a.links[q.first + l];
            const double e = a.e[4 * (x >> 1) + c];
            d += (x & 1) ? -e : e;
        }
        state_st(buf, c, q.o, state_ld(buf, c, q.o, a.g) + d * q.inv_alpha, a.g);
    }
}

void launch_mix(const MixArgs &a, cudaStream_t s)
{
    if (a.nex == 0)
        return;
    mix_exchange_kernel<<<nblk(a.nex, 128), 128, 0, s>>>(a);
    mix_apply_kernel<<<nblk(a.npart, 128), 128, 0, s>>>(a);
    count_launch(2);
}

int ccm_setup(const GridDesc &g, const double *d_phi, double *d_alpha, double *d_ax, double *d_ay, uint8_t *d_type,
              MixExchange **d_ex, int *nex, MixParticipant **d_part, int *npart, int **d_links, double **d_e,
              cudaStream_t s)
{
    const long long cells = (long long)g.M * g.N;
    ccm_geom_kernel<<<nblk(cells, 256), 256, 0, s>>>(g, d_phi, d_alpha, d_ax, d_ay, d_type);
    ccm_aperture_fix_kernel<<<nblk(cells, 256), 256, 0, s>>>(g, d_type, d_ax, d_ay);
    count_launch(2);
    *nex = 0;
    *npart = 0;
    // small cells, row by row
    int *d_counts = nullptr;
    if (cudaMallocAsync(&d_counts, sizeof(int) * (size_t)g.n_y, s) != cudaSuccess)
        return 2;
    const int rows_per_block = 8;
    small_count_kernel<<<nblk(g.n_y, rows_per_block), dim3(32, rows_per_block), 0, s>>>(g, d_alpha, d_type,
                                                                                         d_counts);
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
    std::vector<SmallExchanges> small((size_t)tot);
    if (tot > 0)
    {
        SmallExchanges *d_small = nullptr;
        if (cudaMallocAsync(&d_small, sizeof(SmallExchanges) * (size_t)tot, s) != cudaSuccess)
        {
            cudaFreeAsync(d_counts, s);
            return 2;
        }
        cudaMemcpyAsync(d_counts, offs.data(), sizeof(int) * g.n_y, cudaMemcpyHostToDevice, s);
        small_list_kernel<<<nblk(g.n_y, rows_per_block), dim3(32, rows_per_block), 0, s>>>(
            g, d_alpha, d_ax, d_ay, d_type, d_counts, d_small);
        count_launch();
        cudaError_t e = cudaMemcpyAsync(small.data(), d_small, sizeof(SmallExchanges) * (size_t)tot,
                                        cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        cudaFreeAsync(d_small, s);
        if (e != cudaSuccess)
        {
            cudaFreeAsync(d_counts, s);
            return 5;
        }
    }
    cudaFreeAsync(d_counts, s);

    // exchanges in small-cell order, then each participant's links in
    // exchange order (small side before target side)
    std::vector<MixExchange> ex;
    struct Link
    {
        long long o;
        int x;
        double alpha;
    };
    std::vector<Link> links;
    for (const SmallExchanges &r : small)
        for (int k = 0; k < 3; k++)
        {
            if (r.t[k] < 0)
                continue;
            const int id = (int)ex.size();
            ex.push_back(MixExchange{r.s, r.t[k], r.w[k]});
            links.push_back(Link{r.s, 2 * id, r.alpha_s});
            links.push_back(Link{r.t[k], 2 * id + 1, r.alpha_t[k]});
        }
    std::stable_sort(links.begin(), links.end(), [](const Link &a, const Link &b) { return a.o < b.o; });
    std::vector<MixParticipant> part;
    std::vector<int> lk(links.size());
    for (size_t n = 0; n < links.size(); n++)
    {
        lk[n] = links[n].x;
        if (part.empty() || part.back().o != links[n].o)
            part.push_back(MixParticipant{links[n].o, 1.0 / links[n].alpha, (int)n, 0});
        part.back().count++;
    }
    *nex = (int)ex.size();
    *npart = (int)part.size();
    if (ex.empty())
        return 0;
    if (cudaMallocAsync(d_ex, sizeof(MixExchange) * ex.size(), s) != cudaSuccess ||
        cudaMallocAsync(d_part, sizeof(MixParticipant) * part.size(), s) != cudaSuccess ||
        cudaMallocAsync(d_links, sizeof(int) * lk.size(), s) != cudaSuccess ||
        cudaMallocAsync(d_e, sizeof(double) * 4 * ex.size(), s) != cudaSuccess)
        return 2;
    if (cudaMemcpyAsync(*d_ex, ex.data(), sizeof(MixExchange) * ex.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(*d_part, part.data(), sizeof(MixParticipant) * part.size(), cudaMemcpyHostToDevice, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(*d_links, lk.data(), sizeof(int) * lk.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return 5;
    return 0;
}

CcmLaunch ccm_launcher_muscl_fast(int, int);
CcmLaunch ccm_launcher_mhm_fast(int, int);
CcmLaunch ccm_launcher_godunov_fast(int, int);
CcmLaunch ccm_launcher_muscl_f32(int, int);
CcmLaunch ccm_launcher_mhm_f32(int, int);
CcmLaunch ccm_launcher_godunov_f32(int, int);

// FP64 (both FP64 precision keys: the cut-cell method has no reference
// expression order to keep) or the FP32 compensated form
CcmLaunch ccm_launcher(int scheme, int riemann, int limiter, int precision)
{
    if (precision == 2)
    {
        switch (scheme)
        {
        case MHM: return ccm_launcher_mhm_f32(riemann, limiter);
        case GODUNOV: return ccm_launcher_godunov_f32(riemann, limiter);
        default: return ccm_launcher_muscl_f32(riemann, limiter);
        }
    }
    switch (scheme)
    {
    case MHM: return ccm_launcher_mhm_fast(riemann, limiter);
    case GODUNOV: return ccm_launcher_godunov_fast(riemann, limiter);
    default: return ccm_launcher_muscl_fast(riemann, limiter);
    }
}

} // namespace ibtfo
