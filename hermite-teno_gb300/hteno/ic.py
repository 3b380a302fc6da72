"""Seeded initial data for the benchmark and test workloads (host side, numpy).

The reference hard-codes its initial conditions; the workloads here need seeded variants, so the
generators below are this project's definitions (the draw order is part of the definition):

* four_quadrant: Riemann data split at (0.5, 0.5) of [0,1]^2.  A numpy PCG64 stream seeded with
  `seed` draws, for the quadrants NE, NW, SW, SE in turn, rho ~ U[0.1, 1.5], u ~ U[-1, 1],
  v ~ U[-1, 1], p ~ U[0.03, 1.5].  Quadrant membership follows the reference's
  conservativeOfRiemann2D (Equations_Euler2D.cpp:530-617): x > 0.5 and y > 0.5 is NE, x < 0.5
  and y > 0.5 NW, x < 0.5 and y < 0.5 SW, everything else SE.
* sod: the reference's sodShock (Equations_Euler1D.cpp:317-332).
* gaussian_blobs_shock: density 1 + sum of 32 seeded Gaussian blobs, p = 1, u = v = 0, with a
  Mach 2 planar shock entering at x = 0 (Rankine-Hugoniot post-shock state for x < x_s).
"""
from __future__ import annotations

import numpy as np


def conservative2(rho, u, v, p, gamma=1.4):
    """Euler2D::conservative (Equations_Euler2D.cpp:28-34), elementwise."""
    q1 = rho * u
    q2 = rho * v
    return np.stack([rho, q1, q2, p / (gamma - 1.0) + 0.5 * (q1 * u + q2 * v)])


def quadrant_states(seed: int):
    rng = np.random.default_rng(seed)
    st = []
    for _ in range(4):  # NE, NW, SW, SE
        st.append((rng.uniform(0.1, 1.5), rng.uniform(-1.0, 1.0), rng.uniform(-1.0, 1.0),
                   rng.uniform(0.03, 1.5)))
    return np.array(st)


def four_quadrant(nx: int, ny: int, seed: int, gamma: float = 1.4):
    """Conserved state [4][ny][nx] of the seeded four-quadrant Riemann problem on [0,1]^2."""
    st = quadrant_states(seed)
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    quad = np.where((X > 0.5) & (Y > 0.5), 0,
                    np.where((X < 0.5) & (Y > 0.5), 1, np.where((X < 0.5) & (Y < 0.5), 2, 3)))
    w = st[quad]
    return np.ascontiguousarray(conservative2(w[..., 0], w[..., 1], w[..., 2], w[..., 3], gamma))


def cell_centres(nx: int, ny: int, xl: float, xr: float, yb: float, yt: float):
    """Cell centres as FV::System2D places them (FV_System2D.cpp:37-38): X, Y [ny][nx]."""
    dx, dy = (xr - xl) / nx, (yt - yb) / ny
    x = (np.arange(nx) + 0.5) * dx + xl
    y = (np.arange(ny) + 0.5) * dy + yb
    return np.meshgrid(x, y)


def rayleigh_taylor(nx: int, ny: int, xl: float = 0.0, xr: float = 0.25, yb: float = 0.0,
                    yt: float = 1.0, gamma: float = 1.4):
    """conservativeOfTaylorIns2D (Equations_Euler2D.cpp:619-635) at the cell centres: density 2
    below y = 0.5 and 1 above, hydrostatic-like pressure, a cos(8 pi x) vertical velocity
    perturbation.  Boundary HTENO_BC_TAYLOR (TaylorInstBc) holds the bottom / top states."""
    X, Y = cell_centres(nx, ny, xl, xr, yb, yt)
    low = Y < 0.5
    rho = np.where(low, 2.0, 1.0)
    p = np.where(low, 1.0 + 2.0 * Y, Y + 1.5)
    v = -0.025 * np.sqrt(gamma * p / rho) * np.cos(8.0 * (4.0 * np.arctan(1.0)) * X)
    return np.ascontiguousarray(conservative2(rho, 0.0 * X, v, p, gamma))


def double_mach(nx: int, ny: int, xl: float = 0.0, xr: float = 4.0, yb: float = 0.0,
                yt: float = 1.0, gamma: float = 1.4):
    """conservativeOfDoubleMach2D (Equations_Euler2D.cpp:637-655) at the cell centres: a Mach-10
    shock at 60 degrees through x = 1/6 on the wall.  Boundary HTENO_BC_DOUBLE_MACH
    (doubleMachBc)."""
    X, Y = cell_centres(nx, ny, xl, xr, yb, yt)
    post = X < 1.0 / 6.0 + Y / np.sqrt(3.0)
    rho = np.where(post, 8.0, 1.4)
    u = np.where(post, 8.25 * 0.5 * np.sqrt(3.0), 0.0)
    v = np.where(post, -8.25 * 0.5, 0.0)
    p = np.where(post, 116.5, 1.0)
    return np.ascontiguousarray(conservative2(rho, u, v, p, gamma))


def sod(nx: int, xl: float = 0.0, xr: float = 1.0, gamma: float = 1.4):
    """Conserved state [3][nx] of Sod's shock tube (sodShock, Equations_Euler1D.cpp:317-332)."""
    x = xl + (np.arange(nx) + 0.5) * (xr - xl) / nx
    rho = np.where(x < 0.5, 1.0, 0.125)
    p = np.where(x < 0.5, 1.0, 0.1)
    u = np.zeros(nx)
    return np.ascontiguousarray(np.stack([rho, rho * u, p / (gamma - 1.0) + 0.5 * rho * u * u]))


def blobs_shock_fn(seed: int, gamma: float = 1.4, nblob: int = 32, mach: float = 2.0,
                   x_shock: float = 0.02):
    """Pointwise conserved state q(X, Y) -> [4, ...] on [0,1]^2: rho = 1 + sum_b A_b
    exp(-|x - x_b|^2 / s_b^2), A ~ U[0.2, 1], s ~ U[0.01, 0.05], centres ~ U[0,1]^2 (drawn in
    that order per blob), p = 1, u = v = 0; points with x < x_shock hold the post-shock state of
    a Mach `mach` shock moving in +x into rho = 1, p = 1 (Rankine-Hugoniot)."""
    rng = np.random.default_rng(seed)
    blobs = []
    for _ in range(nblob):
        a = rng.uniform(0.2, 1.0)
        s = rng.uniform(0.01, 0.05)
        cx, cy = rng.uniform(0.0, 1.0, size=2)
        blobs.append((a, s, cx, cy))
    g, M = gamma, mach
    rho0, p0 = 1.0, 1.0
    c0 = np.sqrt(g * p0 / rho0)
    rho1 = rho0 * (g + 1) * M ** 2 / ((g - 1) * M ** 2 + 2)
    p1 = p0 * (2 * g * M ** 2 - (g - 1)) / (g + 1)
    u1 = M * c0 * (1 - rho0 / rho1)

    def q(X, Y):
        rho = np.ones_like(X)
        for a, s, cx, cy in blobs:
            rho = rho + a * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / s ** 2)
        post = X < x_shock
        rho = np.where(post, rho1, rho)
        p = np.where(post, p1, 1.0 + 0 * X)
        u = np.where(post, u1, 0 * X)
        return conservative2(rho, u, 0 * X, p, gamma)

    return q


def gaussian_blobs_shock(nx: int, ny: int, seed: int, gamma: float = 1.4, nblob: int = 32,
                         mach: float = 2.0, x_shock: float = 0.02):
    """Cell-centre values [4][ny][nx] of blobs_shock_fn on [0,1]^2."""
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(x, y)
    f = blobs_shock_fn(seed, gamma, nblob, mach, x_shock)
    return np.ascontiguousarray(f(X, Y))


def face_difference_moments(q_fn, nx, ny, xl, xr, yb, yt):
    """Hermite moments by face differences of an initial-data function, as
    FVHermite::System2D::Riemann2D does (FVHermite_System2D.cpp:94-100):
    v = (q(x + dx/2, y) - q(x - dx/2, y)) / dx, w likewise in y."""
    dx, dy = (xr - xl) / nx, (yt - yb) / ny
    x = xl + (np.arange(nx) + 0.5) * dx
    y = yb + (np.arange(ny) + 0.5) * dy
    X, Y = np.meshgrid(x, y)
    v = (q_fn(X + dx / 2.0, Y) - q_fn(X - dx / 2.0, Y)) / dx
    w = (q_fn(X, Y + dy / 2.0) - q_fn(X, Y - dy / 2.0)) / dy
    return np.ascontiguousarray(v), np.ascontiguousarray(w)


# ---- smooth cases with exact solutions (periodic) ----------------------------------------------
# Cell averages by the 9-point Gauss-Legendre rule per direction, as the reference's
# entropyWaves / isentropicVortex do (Equations_Euler2D.cpp:454-471, 513-528,
# Equations_Euler1D.cpp:263-277; nodes and weights of Schemes_Lagrange.cpp:22-42).

def _gauss9():
    a, w = np.polynomial.legendre.leggauss(9)
    return a, w


def cell_average_2d(f, nx, ny, xl, xr, yb, yt):
    """Cell averages [k][ny][nx] of f(X, Y) -> [k, ...] over the uniform grid."""
    a, w = _gauss9()
    dx, dy = (xr - xl) / nx, (yt - yb) / ny
    X, Y = np.meshgrid(xl + (np.arange(nx) + 0.5) * dx, yb + (np.arange(ny) + 0.5) * dy)
    acc = None
    for i in range(9):
        for j in range(9):
            v = w[i] * w[j] * np.asarray(f(X + dx * a[i] / 2.0, Y + dy * a[j] / 2.0)) / 4.0
            acc = v if acc is None else acc + v
    return np.ascontiguousarray(acc)


def cell_average_1d(f, nx, xl, xr):
    a, w = _gauss9()
    dx = (xr - xl) / nx
    X = xl + (np.arange(nx) + 0.5) * dx
    acc = None
    for i in range(9):
        v = w[i] * np.asarray(f(X + dx * a[i] / 2.0)) / 2.0
        acc = v if acc is None else acc + v
    return np.ascontiguousarray(acc)


def entropy_wave_2d(nx, ny, t=0.0, xl=-1.0, xr=1.0, yb=-1.0, yt=1.0, rho=1.0, u=1.0, v=1.0, p=1.0,
                    amp=0.5, gamma=1.4, derivative=False):
    """FV::System2D::entropyWave (FV_System2D.cpp:49-74): rho = rho_inf + A sin(pi (x + y)),
    constant u, v, p, advected to time t; derivative=True gives the cell averages of d/dx
    (= d/dy), the Hermite moments (dconservativeOfEntropyWave, Equations_Euler2D.cpp:442-452)."""
    def q(X, Y):
        xs, ys = X - u * t, Y - v * t
        if derivative:
            d = amp * np.cos(np.pi * (xs + ys)) * np.pi
            return np.stack([d, u * d, v * d, 0.5 * (u * u + v * v) * d])
        r = rho + amp * np.sin(np.pi * (xs + ys))
        return conservative2(r, u + 0 * r, v + 0 * r, p + 0 * r, gamma)
    return cell_average_2d(q, nx, ny, xl, xr, yb, yt)


def smooth_waves_2d(nx, ny, gamma=1.4):
    """Point values [4][ny][nx] of a smooth periodic flow on [0,1]^2 (a synthetic workload with no
    discontinuity): rho = 1 + 0.2 sin(2 pi x) sin(2 pi y), u = 0.5 + 0.1 sin(2 pi y),
    v = -0.3 + 0.1 cos(2 pi x), p = 1 + 0.1 cos(2 pi (x + y))."""
    X, Y = cell_centres(nx, ny, 0.0, 1.0, 0.0, 1.0)
    tp = 2 * np.pi
    rho = 1 + 0.2 * np.sin(tp * X) * np.sin(tp * Y)
    u = 0.5 + 0.1 * np.sin(tp * Y)
    v = -0.3 + 0.1 * np.cos(tp * X)
    p = 1 + 0.1 * np.cos(tp * (X + Y))
    return np.ascontiguousarray(conservative2(rho, u, v, p, gamma))


def isentropic_vortex_2d(nx, ny, t=0.0, xl=-5.0, xr=5.0, yb=-5.0, yt=5.0, gamma=1.4, b=5.0):
    """FV::System2D::isentropicVortex (FV_System2D.cpp:76-99; conservativeOfIsentropicVortex,
    Equations_Euler2D.cpp:656-666): the vortex of strength b on a (1, 1) mean flow, advected to
    time t (periodic domain of side L: positions wrap)."""
    L = xr - xl
    g1 = gamma - 1.0

    def q(X, Y):
        xs = (X - t - xl) % L + xl
        ys = (Y - t - yb) % (yt - yb) + yb
        r = xs ** 2 + ys ** 2
        rho = (1.0 - g1 * b ** 2 / 8.0 / gamma / np.pi ** 2 * np.exp(1 - r)) ** (1.0 / g1)
        uu = 1.0 - b * ys / 2.0 / np.pi * np.exp(0.5 * (1 - r))
        vv = 1.0 + b * xs / 2.0 / np.pi * np.exp(0.5 * (1 - r))
        return conservative2(rho, uu, vv, rho ** gamma, gamma)
    return cell_average_2d(q, nx, ny, xl, xr, yb, yt)


def entropy_wave_1d(nx, t=0.0, xl=-1.0, xr=1.0, rho=1.0, u=1.0, p=1.0, amp=0.5, gamma=1.4,
                    derivative=False):
    """FV::System1D / FVHermite::System1D entropyWave (Equations_Euler1D.cpp:243-294):
    rho = rho_inf + A sin(pi x), constant u, p, at time t; derivative=True: cell averages of
    d/dx (the Hermite moment)."""
    def q(X):
        xs = X - u * t
        if derivative:
            d = amp * np.cos(np.pi * xs) * np.pi
            return np.stack([d, u * d, 0.5 * u * u * d])
        r = rho + amp * np.sin(np.pi * xs)
        return np.stack([r, r * u, p / (gamma - 1.0) + 0.5 * r * u * u])
    return cell_average_1d(q, nx, xl, xr)
