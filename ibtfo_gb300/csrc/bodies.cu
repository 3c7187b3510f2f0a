// Device-side case set-up: level set of analytic bodies, piecewise initial
// states, and the density read-back used by the serving loop.
//
// The reference builds its level set on the host, either from a closed-form
// function per test (Test/InclineSod/Level_Set_function.cpp:8-52) or by a
// brute-force nearest-edge scan of a PNG outline (Test/PNGGeo/Level_Set.cpp:
// 31-142).  Here phi is the signed distance to a union of circles and
// ellipses, evaluated per cell on the GPU: phi = min over bodies of the
// distance to the body's outline, positive in the fluid (outside every body),
// with the reference's coordinates x_i = lo_x + (i - ng + 1/2) dx,
// y_j = lo_y + (j - ng + 1/2) dx (Psy_coord.cpp:33-43: dy := dx).
#include "../../include/ibtfo.h"
#include "internal.h"

namespace ibtfo {

// Distance from (y0, y1), y0, y1 >= 0, to the ellipse (x0/e0)^2 + (x1/e1)^2 = 1
// with e0 >= e1 > 0, by bisection on the root of
//   F(s) = (r0 z0 / (s + r0))^2 + (z1 / (s + 1))^2 - 1,  r0 = (e0/e1)^2, zk = yk/ek
// (D. Eberly, "Distance from a Point to an Ellipse, an Ellipsoid, or a
// Hyperellipsoid", Geometric Tools): the closest point is
// x0 = r0 y0 / (s + r0), x1 = y1 / (s + 1).  Points on the major axis inside
// the evolute (y1 = 0, y0 < (e0^2 - e1^2)/e0) take the closed form.
__device__ double ellipse_distance(double e0, double e1, double y0, double y1)
{
    if (y1 > 0.0)
    {
        if (y0 > 0.0)
        {
            const double z0 = y0 / e0, z1 = y1 / e1;
            const double gg = z0 * z0 + z1 * z1 - 1.0;
            if (gg == 0.0)
                return 0.0;
            const double r0 = (e0 / e1) * (e0 / e1);
            const double n0 = r0 * z0;
            double s0 = z1 - 1.0;
            double s1 = (gg < 0.0) ? 0.0 : sqrt(n0 * n0 + z1 * z1) - 1.0;
            double s = 0.0;
            for (int it = 0; it < 200; it++) // halves the bracket until it stops shrinking
            {
                s = 0.5 * (s0 + s1);
                if (s == s0 || s == s1)
                    break;
                const double a = n0 / (s + r0), b = z1 / (s + 1.0);
                const double f = a * a + b * b - 1.0;
                if (f > 0.0)
                    s0 = s;
                else if (f < 0.0)
                    s1 = s;
                else
                    break;
            }
            const double x0 = r0 * y0 / (s + r0), x1 = y1 / (s + 1.0);
            return sqrt((x0 - y0) * (x0 - y0) + (x1 - y1) * (x1 - y1));
        }
        return fabs(y1 - e1); // on the minor axis
    }
    const double num = e0 * y0, den = e0 * e0 - e1 * e1;
    if (num < den)
    {
        const double xr = num / den;
        const double x0 = e0 * xr, x1 = e1 * sqrt(fmax(0.0, 1.0 - xr * xr));
        return sqrt((x0 - y0) * (x0 - y0) + x1 * x1);
    }
    return fabs(y0 - e0);
}

// signed distance to one body, positive outside it; `band` = distance from
// the outline within which the exact distance is needed (farther cells get a
// lower bound with the right sign)
__device__ double body_distance(const ibtfo_body &b, double x, double y, double band)
{
    const double dx = x - b.xc, dy = y - b.yc;
    const double r = sqrt(dx * dx + dy * dy);
    if (b.kind == IBTFO_BODY_CIRCLE)
        return r - b.a;
    const double big = fmax(b.a, b.b), small = fmin(b.a, b.b);
    if (r - big > band)
        return r - big; // outside the bounding circle by more than the band
    if (r < small - band)
        return r - small; // inside the inscribed circle by more than the band
    // body frame: rotate by -theta, the major semi-axis along the first coordinate
    const double c = cos(b.theta), s = sin(b.theta);
    double u = c * dx + s * dy, v = -s * dx + c * dy;
    if (b.b > b.a)
    {
        const double t = u;
        u = v;
        v = -t;
    }
    const double y0 = fabs(u), y1 = fabs(v);
    const double d = ellipse_distance(big, small, y0, y1);
    const bool inside = (y0 / big) * (y0 / big) + (y1 / small) * (y1 / small) < 1.0;
    return inside ? -d : d;
}

__global__ void bodies_phi_kernel(GridDesc g, const ibtfo_body *__restrict__ bodies, int n, double band,
                                  double *phi)
{
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)g.M * g.N)
        return;
    const int j = (int)(c / g.M), i = (int)(c - (long long)j * g.M);
    const double x = g.Li + i * g.dx, y = g.Hi + j * g.dx;
    double p = 1e300;
    for (int k = 0; k < n; k++)
        p = fmin(p, body_distance(bodies[k], x, y, band));
    phi[(long long)j * g.pitch + i] = (n > 0) ? p : 1.0;
}

// U = left for x < x_split, right elsewhere (conserved variables); solid
// cells hold rho = -1, E = -1 (Test/InclineSod/Initialize.cpp:61-67)
__global__ void x_split_init_kernel(GridDesc g, const uint8_t *__restrict__ type, double x_split, double4 L,
                                    double4 R, double *buf)
{
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)g.M * g.N)
        return;
    const int j = (int)(c / g.M), i = (int)(c - (long long)j * g.M);
    const long long o = (long long)j * g.pitch + i;
    const double x = g.Li + i * g.dx;
    double4 u = (x < x_split) ? L : R;
    if (type[o] == 1)
        u = make_double4(-1.0, 0.0, 0.0, -1.0);
    state_st(buf, 0, o, u.x, g);
    state_st(buf, 1, o, u.y, g);
    state_st(buf, 2, o, u.z, g);
    state_st(buf, 3, o, u.w, g);
}

// initial values at the corner-column sources of the Regular domain edges
// (columns ng and N_x+ng-1, ghost rows): [2][2 ng][4]
__global__ void ring_ic_kernel(GridDesc g, const double *__restrict__ buf, double *ring)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * 2 * g.ng)
        return;
    const int side = t / (2 * g.ng), rr = t - side * 2 * g.ng;
    const int i = side ? g.n_x + g.ng - 1 : g.ng;
    const int j = (rr < g.ng) ? rr : g.n_y + rr;
    const long long o = (long long)j * g.pitch + i;
    for (int k = 0; k < 4; k++)
        ring[t * 4 + k] = state_ld(buf, k, o, g);
}

// interior density of the current state, row-major n_y x n_x
__global__ void density_kernel(GridDesc g, const double *__restrict__ b0, const double *__restrict__ b1,
                               const DevState *__restrict__ st, double *out)
{
    long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long long)g.n_x * g.n_y)
        return;
    const double *buf = st->cur ? b1 : b0;
    const int j = (int)(c / g.n_x), i = (int)(c - (long long)j * g.n_x);
    out[c] = state_ld(buf, 0, (long long)(j + g.ng) * g.pitch + i + g.ng, g);
}

static inline unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

void launch_bodies_phi(const GridDesc &g, const ibtfo_body *d_bodies, int n, double *phi, cudaStream_t s)
{
    const double band = 16.0 * g.dx;
    bodies_phi_kernel<<<nblk((long long)g.M * g.N, 256), 256, 0, s>>>(g, d_bodies, n, band, phi);
    count_launch();
}

void launch_x_split_init(const GridDesc &g, const uint8_t *type, double x_split, const double L[4],
                         const double R[4], double *buf, double *ring_ic, cudaStream_t s)
{
    x_split_init_kernel<<<nblk((long long)g.M * g.N, 256), 256, 0, s>>>(
        g, type, x_split, make_double4(L[0], L[1], L[2], L[3]), make_double4(R[0], R[1], R[2], R[3]), buf);
    ring_ic_kernel<<<1, 256, 0, s>>>(g, buf, ring_ic); // 4 ng <= 256 entries (ng <= 64)
    count_launch(2);
}

void launch_density(const GridDesc &g, const double *b0, const double *b1, const DevState *st, double *out,
                    cudaStream_t s)
{
    density_kernel<<<nblk((long long)g.n_x * g.n_y, 256), 256, 0, s>>>(g, b0, b1, st, out);
    count_launch();
}

} // namespace ibtfo
