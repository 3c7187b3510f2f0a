"""Case plug-ins: level set phi and initial conserved state for named problems.

The reference defines each problem with three per-case hooks compiled into
its driver (Src/Geometry/Level_Set_function.H:13-19, Src/Base/Common/
Initialize.H:12-23 and the Global_Boundary of Src/BoundaryCondition/
Boundary.H:22-29).  Here a case is plain data: `phi` (M*N doubles, index
j*M+i) and `u0` (M*N*4 doubles, index (j*M+i)*4+k, k = rho, rho u, rho v, E),
which both the GPU path and the CPU oracle consume unchanged.

Cell-centre coordinates follow Src/Geometry/Psy_coord.cpp:29-44: x_i =
Li + i*dx, y_j = Hi + j*dx with dx = (hi_x - lo_x)/N_x used in both
directions (the reference assumes square cells).

Cases that depend on the cell type (solid cells get rho = -1, E = -1, as in
Test/InclineSod/Initialize.cpp:43-67) take the type array returned by the
geometry set-up, in the same order as the reference calls Level_Set before
Initialize.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Grid:
    n_x: int
    n_y: int
    ng: int = 2
    lo_x: float = 0.0
    lo_y: float = 0.0
    hi_x: float = 1.0
    hi_y: float = 1.0

    @property
    def M(self):
        return self.n_x + 2 * self.ng

    @property
    def N(self):
        return self.n_y + 2 * self.ng

    def coords(self):
        """x, y arrays of shape (N, M), bit-identical to Psy_coord.cpp:29-44."""
        dx = (self.hi_x - self.lo_x) / self.n_x
        Li = -dx * self.ng + self.lo_x + dx / 2
        Hi = -dx * self.ng + self.lo_y + dx / 2
        i = np.arange(self.M, dtype=np.float64)
        j = np.arange(self.N, dtype=np.float64)
        x = Li + i * dx
        y = Hi + j * dx
        return np.broadcast_to(x[None, :], (self.N, self.M)), np.broadcast_to(y[:, None], (self.N, self.M))


def conserved(rho, u, v, p, gamma):
    """(rho, rho u, rho v, E) with E = p/(gamma-1) + 0.5 rho (u^2+v^2) (Test/Sod/Initialize.cpp:45-48)."""
    rho = np.asarray(rho, dtype=np.float64)
    out = np.empty(rho.shape + (4,))
    out[..., 0] = rho
    out[..., 1] = rho * u
    out[..., 2] = rho * v
    out[..., 3] = p / (gamma - 1) + 0.5 * rho * (u * u + v * v)
    return out


def _solid_fill(u, types):
    """solid cells (type 1) hold rho = -1, E = -1 (Test/InclineSod/Initialize.cpp:61-67)."""
    if types is None:
        return u
    solid = ~((types < 0.5) | (types > 1.5))
    u[solid] = (-1.0, 0.0, 0.0, -1.0)
    return u


# ------------------------------------------------------------------ problems


def sod_x(g: Grid, gamma=1.4, x0=0.5, left=(1.0, 0.0, 0.0, 1.0), right=(0.125, 0.0, 0.0, 0.1), types=None):
    """Sod shock tube split on x < x0, no immersed body (phi = 1)."""
    x, _ = g.coords()
    phi = np.ones((g.N, g.M))
    L = conserved(*left, gamma)
    R = conserved(*right, gamma)
    u = np.where((x < x0)[..., None], L, R)
    return phi.reshape(-1), _solid_fill(np.ascontiguousarray(u), types).reshape(-1)


def quadrants(g: Grid, gamma=1.4, xc=0.5, yc=0.5, states=None, types=None, downward=False):
    """Four-state 2D Riemann problem; states = upper-right, upper-left,
    lower-left, lower-right as (rho, u, v, p).  The default states move
    vertically faster than sound in three quadrants and slower in one, with
    small velocity jumps (no vacuum-forming expansions); `downward` reverses
    every vertical velocity."""
    if states is None:
        states = ((1.0, 0.1, 1.5, 1.0), (0.6, -0.1, 1.3, 0.7), (0.9, 0.0, 1.4, 0.9), (1.1, 0.2, 0.9, 1.1))
    if downward:
        states = tuple((r, u, -v, p) for (r, u, v, p) in states)
    x, y = g.coords()
    phi = np.ones((g.N, g.M))
    ur, ul, ll, lr = (conserved(*s, gamma) for s in states)
    right = x >= xc
    top = y >= yc
    u = np.where((top & right)[..., None], ur, np.where((top & ~right)[..., None], ul,
                 np.where((~top & ~right)[..., None], ll, lr)))
    return phi.reshape(-1), _solid_fill(np.ascontiguousarray(u), types).reshape(-1)


def channel_phi(g: Grid, angle_deg=30.0, width=0.25, center=None):
    """Inclined channel: signed distance min(d_lower, d_upper) to two walls
    parallel to an axis through `center` at `angle_deg` (fluid inside, phi > 0)."""
    x, y = g.coords()
    if center is None:
        center = (0.5 * (g.lo_x + g.hi_x), 0.5 * (g.lo_y + g.hi_y))
    th = math.radians(angle_deg)
    s = (x - center[0]) * (-math.sin(th)) + (y - center[1]) * math.cos(th)
    phi = np.minimum(s + 0.5 * width, 0.5 * width - s)
    return np.ascontiguousarray(phi).reshape(-1)


def channel_init(g: Grid, types, gamma=1.4, angle_deg=30.0, center=None, left=(1.0, 0.0, 0.0, 1.0),
                 right=(0.125, 0.0, 0.0, 0.1)):
    """Sod states split perpendicular to the channel axis at the channel midpoint."""
    x, y = g.coords()
    if center is None:
        center = (0.5 * (g.lo_x + g.hi_x), 0.5 * (g.lo_y + g.hi_y))
    th = math.radians(angle_deg)
    a = (x - center[0]) * math.cos(th) + (y - center[1]) * math.sin(th)
    u = np.where((a < 0)[..., None], conserved(*left, gamma), conserved(*right, gamma))
    u = np.ascontiguousarray(u)
    return _solid_fill(u, np.asarray(types).reshape(g.N, g.M)).reshape(-1)


def cylinder_phi(g: Grid, xc, yc, r):
    """Circular body of radius r centred at (xc, yc): phi = distance to the
    circle, positive in the fluid outside it."""
    x, y = g.coords()
    dx, dy = x - xc, y - yc
    return np.ascontiguousarray(np.sqrt(dx * dx + dy * dy) - r).reshape(-1)


def uniform_init(g: Grid, types, state=(1.0, 0.0, 0.0, 1.0), gamma=1.4):
    """One primitive state (rho, u, v, p) everywhere, solid cells filled as the reference does."""
    u = np.ascontiguousarray(np.broadcast_to(conserved(*state, gamma), (g.N, g.M, 4))).copy()
    return _solid_fill(u, np.asarray(types).reshape(g.N, g.M)).reshape(-1)


def post_shock(mach, gamma=1.4, pre=(1.0, 0.0, 0.0, 1.0)):
    """Rankine-Hugoniot state behind a normal shock moving in +x at Mach
    `mach` into the quiescent state `pre` (rho, u, v, p)."""
    rho1, _, _, p1 = pre
    a1 = math.sqrt(gamma * p1 / rho1)
    m2 = mach * mach
    rho2 = rho1 * (gamma + 1) * m2 / ((gamma - 1) * m2 + 2)
    p2 = p1 * (2 * gamma * m2 - (gamma - 1)) / (gamma + 1)
    u2 = 2 * a1 / (gamma + 1) * (mach - 1 / mach)
    return (rho2, u2, 0.0, p2)


def shock_init(g: Grid, types, mach, x_shock, gamma=1.4, pre=(1.0, 0.0, 0.0, 1.0)):
    """Normal shock at x = x_shock moving into `pre` (post-shock state behind it)."""
    x, _ = g.coords()
    u = np.where((x < x_shock)[..., None], conserved(*post_shock(mach, gamma, pre), gamma), conserved(*pre, gamma))
    u = np.ascontiguousarray(u)
    return _solid_fill(u, np.asarray(types).reshape(g.N, g.M)).reshape(-1)


def isentropic_vortex(g: Grid, gamma=1.4, beta=5.0, xc=5.0, yc=5.0, u_inf=1.0, v_inf=1.0, t=0.0, periodic=True):
    """Isentropic vortex of strength beta on a uniform (1, u_inf, v_inf, 1)
    stream; at time t the exact solution is the initial field moved by
    (u_inf t, v_inf t), wrapped periodically.  phi = 1 (no body)."""
    x, y = g.coords()
    Lx, Ly = g.hi_x - g.lo_x, g.hi_y - g.lo_y
    cx, cy = xc + u_inf * t, yc + v_inf * t
    dxv = x - cx
    dyv = y - cy
    if periodic:
        dxv = (dxv + 0.5 * Lx) % Lx - 0.5 * Lx
        dyv = (dyv + 0.5 * Ly) % Ly - 0.5 * Ly
    r2 = dxv * dxv + dyv * dyv
    f = np.exp(0.5 * (1.0 - r2))
    du = -beta / (2 * math.pi) * dyv * f
    dv = beta / (2 * math.pi) * dxv * f
    T = 1.0 - (gamma - 1.0) * beta * beta / (8.0 * gamma * math.pi * math.pi) * np.exp(1.0 - r2)
    rho = T ** (1.0 / (gamma - 1.0))
    p = rho * T
    u = conserved(rho, u_inf + du, v_inf + dv, p, gamma)
    return np.ones(g.N * g.M), np.ascontiguousarray(u).reshape(-1)


# reference C1/C2/C3 workloads --------------------------------------------------


@dataclass
class Workload:
    name: str
    grid: Grid
    gamma: float
    cfl: float
    t_end: float
    scheme: str
    riemann: str
    limiter: str
    boundary: str
    gbc: str = "walls"
    extra: dict = field(default_factory=dict)
    time: str = "SingleStep"


def sod_tube(n_x=400, n_y=100):
    """2D Sod tube, 400x100 on [0,1]x[0,0.25], CFL 0.5, t_end 0.2, no body."""
    return Workload("sod_tube_400x100", Grid(n_x, n_y, 2, 0.0, 0.0, 1.0, 0.25), 1.4, 0.5, 0.2,
                    "MUSCL", "HLL", "minmod", "Regular")


def inclined_channel(n_x=2048, n_y=1024, boundary="IDWBaseGFM"):
    """Inclined Sod channel, 2048x1024 on [0,2]x[0,1], width 0.25 at 30 deg,
    ghost-fluid walls, MUSCL + HLLC, CFL 0.45, t_end 0.2."""
    return Workload(f"inclined_channel_{n_x}x{n_y}", Grid(n_x, n_y, 2, 0.0, 0.0, 2.0, 1.0), 1.4, 0.45, 0.2,
                    "MUSCL", "HLLC", "minmod", boundary, extra={"angle": 30.0, "width": 0.25})


def vortex_periodic(n=4096, riemann="HLL_Toro", time="RK2"):
    """Isentropic vortex, periodic n x n on [0,10]^2, beta 5, MHM + HLLC
    (the reference's HLLC key is its HLL solver: here HLL_Toro), Time = RK2,
    CFL 0.25, advected one period (t 10).

    Solver: the vortex's vertical velocity exceeds the sound speed in part of
    the core; the reference's HLL, which reuses the X-face flux where
    S_D >= 0, turns the state to NaN there within a few dozen steps.
    HLL_Toro is the same HLL flux without that slot reuse and with wave-speed
    estimates defined everywhere.

    Time integration: with Time = SingleStep (forward Euler) the reference's
    MUSCL and MHM updates are unstable in smooth flow at any CFL; the limiter
    only bounds the growth.  Measured on this flow to t = 10 (FP64, 1024^2,
    CFL 0.25): a 1e-7 relative perturbation of the initial state ends at 1.8e-3
    (L1 density) after single steps, at 2.1e-5 after RK2 steps, against a
    distance of 1.6e-4 from the exact solution.  CFL 0.25: the reference's
    time step bounds one direction's Courant number (ComputeDt.cpp:49) while
    both directions update from the same state, and this stream is diagonal."""
    return Workload(f"isentropic_vortex_{n}", Grid(n, n, 2, 0.0, 0.0, 10.0, 10.0), 1.4, 0.25, 10.0,
                    "MHM", riemann, "minmod", "Regular", gbc="periodic", extra={"beta": 5.0}, time=time)


# served batch stream --------------------------------------------------------

# The served stream's solver, time integration and CFL number.  The
# reference's HLLC key is its HLL solver; HLL_Toro is that flux with
# wave-speed estimates that stay defined behind a Mach-4 body.  Measured on
# the stream's Mach 2-4 requests (FP64, a 1e-7 relative perturbation of the
# initial state, L1 density at t_end):
#   HLLC_Toro, single steps, CFL 0.3 or 0.45:  1e-2 (odd-even decoupling of
#     contact-restoring solvers at strong grid-aligned shocks)
#   HLL_Toro, single steps, CFL 0.45: up to 1e-3; CFL 0.3: 1e-7 on grids up
#     to 900 cells wide, but the forward-Euler update is unstable in smooth
#     flow, and on the larger grids the wake amplifies FP32 rounding to 1e-4
#   HLL_Toro, Time = RK2, CFL 0.45: 6e-7 to 1e-5 (the wake's own growth)
SERVE_RIEMANN = "HLL_Toro"
SERVE_TIME = "RK2"
SERVE_CFL = 0.45


@dataclass
class ServedRequest:
    id: int
    arrival: float        # seconds after the stream starts
    n_x: int
    n_y: int
    width: float
    height: float
    mach: float
    xc: float
    yc: float
    radius: float
    x_shock: float
    t_end: float
    cfl: float = SERVE_CFL


def served_stream(n_requests, rate, seed=42, min_cells=128 * 128, max_cells=2048 * 2048, crossings=1.5,
                  gamma=1.4):
    """Shock over an immersed cylinder, one request each, arriving as a
    Poisson stream of `rate` requests/s: cell count log-uniform in
    [min_cells, max_cells], aspect ratio n_x/n_y uniform in [1, 4], width 1
    and height n_y/n_x (square cells, as the reference's coordinates assume,
    Psy_coord.cpp:22), shock Mach uniform in [1.5, 4] starting at x = 0.1,
    cylinder radius uniform in [0.05, 0.2] of the height at a seeded position
    (x in [0.3, 0.7] of the width, y in [0.3, 0.7] of the height), run to
    t_end = `crossings` domain-crossing times of the shock."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    a1 = math.sqrt(gamma)  # sound speed of the quiescent (1, 0, 0, 1) gas
    for k in range(n_requests):
        t += rng.exponential(1.0 / rate)
        cells = math.exp(rng.uniform(math.log(min_cells), math.log(max_cells)))
        aspect = rng.uniform(1.0, 4.0)
        n_x = max(16, int(round(math.sqrt(cells * aspect))))
        n_y = max(16, int(round(cells / n_x)))
        mach = rng.uniform(1.5, 4.0)
        r_frac = rng.uniform(0.05, 0.2)
        fx, fy = rng.uniform(0.3, 0.7), rng.uniform(0.3, 0.7)
        W, H = 1.0, n_y / n_x
        out.append(ServedRequest(k, t, n_x, n_y, W, H, mach, fx * W, fy * H, r_frac * H, 0.1 * W,
                                 crossings * W / (mach * a1)))
    return out


def served_steps_estimate(r: ServedRequest, cfl=None, gamma=1.4):
    """Steps to t_end with the post-shock maximum wave speed (u2 + a2)."""
    rho2, u2, _, p2 = post_shock(r.mach, gamma)
    lam = u2 + math.sqrt(gamma * p2 / rho2)
    return int(math.ceil(r.t_end / ((cfl or r.cfl) * (r.width / r.n_x) / lam)))


# shock over random obstacles (cut cells) -----------------------------------


@dataclass
class Obstacle:
    kind: str      # "circle" or "ellipse"
    xc: float
    yc: float
    a: float       # radius, or the semi-axis along theta
    b: float       # the other semi-axis (= a for a circle)
    theta: float


def random_obstacles(n=24, seed=20261203, r_min=0.02, r_max=0.15, x_range=(1.0, 3.8), height=2.0, gap=0.01,
                     max_tries=100000):
    """`n` non-overlapping circles and ellipses: kind 50/50, radius (the
    ellipse's major semi-axis) uniform in [r_min, r_max], an ellipse's minor
    semi-axis 0.4-1.0 of it, orientation uniform in [0, pi), centre x uniform
    in `x_range` and y uniform in [r, height - r], drawn with rejection of any
    body whose bounding circle comes within `gap` of another's."""
    rng = np.random.default_rng(seed)
    out = []
    tries = 0
    while len(out) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place the obstacles without overlap")
        ellipse = rng.random() < 0.5
        r = rng.uniform(r_min, r_max)
        b = r * rng.uniform(0.4, 1.0) if ellipse else r
        th = rng.uniform(0.0, math.pi) if ellipse else 0.0
        x = rng.uniform(*x_range)
        y = rng.uniform(r, height - r)
        if any(math.hypot(x - o.xc, y - o.yc) < r + o.a + gap for o in out):
            continue
        out.append(Obstacle("ellipse" if ellipse else "circle", x, y, r, b, th))
    return out


def obstacles_phi(g: Grid, obstacles):
    """Host signed distance for circles only (ellipses: use the GPU set-up)."""
    phi = np.full(g.M * g.N, 1e300)
    for o in obstacles:
        if o.kind != "circle":
            raise ValueError("obstacles_phi handles circles; ellipses are built by Case.setup_bodies")
        phi = np.minimum(phi, cylinder_phi(g, o.xc, o.yc, o.a))
    return phi


def shock_obstacles(n_x=8192, n_y=4096):
    """Mach 3 shock over the 24 seeded obstacles, cut cells, [0,4] x [0,2],
    t_end 1.0, shock at x = 0.5 into (1, 0, 0, 1).  CFL 0.3: an unmixed cut
    cell (alpha >= 0.5) sees up to twice a full cell's Courant number in an
    unsplit update."""
    return Workload(f"shock_obstacles_{n_x}x{n_y}", Grid(n_x, n_y, 2, 0.0, 0.0, 4.0, 2.0), 1.4, 0.3, 1.0,
                    "MUSCL", "HLL_Toro", "minmod", "CCM", extra={"mach": 3.0, "x_shock": 0.5, "seed": 20261203})

