"""Shared test cases: FEN's initial conditions and manufactured solutions.

Field arrays are numpy (k, j, i) views of FEN's f(0:nx+1, 0:ny+1, 0:nz+1); MAC placement
as in the reference test initialisers (test/small_test/navier_stokes/taylor_green_vortex/
taylor_green_vortex.f90:94-102): u at (i d, (j-1/2) d), v at ((i-1/2) d, j d), p at cell
centres, w at (., ., k d).
"""
import numpy as np

from oracle import oracle as O

PI = np.pi


def coords(n, d, kind):
    """Coordinates of ghosted indices 0..n+1: 'c' cell centre, 'f' face."""
    i = np.arange(n + 2, dtype=np.float64)
    return i * d if kind == "f" else (i - 0.5) * d


def mac_grids(dim, n, d):
    """Meshes (k, j, i) for u, v, w, p positions."""
    out = {}
    nz = n[2] if dim == 3 else 1
    for name, kinds in {"u": "fcc", "v": "cfc", "w": "ccf", "p": "ccc"}.items():
        x = coords(n[0], d[0], kinds[0])
        y = coords(n[1], d[1], kinds[1])
        z = coords(nz, d[2], kinds[2]) if dim == 3 else np.array([0.0, 0.5 * d[2], d[2]])
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        out[name] = (X, Y, Z)
    return out


def tgv2d_fields(n, L):
    """2D Taylor-Green vortex: u = sin x cos y, v = -cos x sin y, p = (cos 2x + cos 2y)/4."""
    d = L / n
    g = mac_grids(2, (n, n, 1), (d, d, d))
    X, Y, _ = g["u"]
    u = np.sin(X) * np.cos(Y)
    X, Y, _ = g["v"]
    v = -np.cos(X) * np.sin(Y)
    X, Y, _ = g["p"]
    p = (np.cos(2 * X) + np.cos(2 * Y)) / 4
    return u, v, p


def tgv3d_fields(n, L):
    """3D Taylor-Green vortex: u = sin x cos y cos z, v = -cos x sin y cos z, w = 0,
    p = (cos 2x + cos 2y)(cos 2z + 2)/16."""
    d = L / n
    g = mac_grids(3, (n, n, n), (d, d, d))
    X, Y, Z = g["u"]
    u = np.sin(X) * np.cos(Y) * np.cos(Z)
    X, Y, Z = g["v"]
    v = -np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(u)
    X, Y, Z = g["p"]
    p = (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2) / 16
    return u, v, w, p


def channel_fields(n, L, nu, seed=1234, noise=0.05):
    """Channel workload start (walls at y = -1, 1): laminar Poiseuille u = (1 - y^2)/(2 nu)
    at the u points plus seeded uniform noise of `noise` times the centreline velocity on the
    interiors of u, v, w (PCG64(seed), drawn per component in Fortran order, x fastest);
    p = 0.  Returns ghosted arrays (u, v, w, p)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = (n[2] + 2, n[1] + 2, n[0] + 2)
    dy = L[1] / n[1]
    yc = -1.0 + (np.arange(n[1] + 2) - 0.5) * dy
    Uc = 1.0 / (2 * nu)
    out = []
    for key in "uvw":
        a = np.zeros(shape)
        a[1:-1, 1:-1, 1:-1] = noise * Uc * rng.uniform(-1.0, 1.0, size=(n[2], n[1], n[0]))
        if key == "u":
            a[1:-1, 1:-1, 1:-1] += ((1 - yc[1:-1] ** 2) / (2 * nu))[None, :, None]
        out.append(a)
    out.append(np.zeros(shape))
    return tuple(out)


def random_interior(shape, rng, dim):
    a = np.zeros(shape)
    if dim == 3:
        a[1:-1, 1:-1, 1:-1] = rng.uniform(-1, 1, size=(shape[0] - 2, shape[1] - 2, shape[2] - 2))
    else:
        a[1, 1:-1, 1:-1] = rng.uniform(-1, 1, size=(shape[1] - 2, shape[2] - 2))
    return a


def interior(a, dim):
    return a[1:-1, 1:-1, 1:-1] if dim == 3 else a[1, 1:-1, 1:-1]


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


# Manufactured Poisson solutions of test/small_test/poisson/convergence_rate/
# convergence_rate.f90:167-223 (domain [0,1]^d, cell centres).
def poisson_case(name):
    s = lambda x: np.sin(2 * PI * x)
    c = lambda x: np.cos(2 * PI * x)
    cases = {
        "pp": (2, [O.PERIODIC] * 4, lambda X, Y, Z: -8 * PI * PI * s(X) * c(Y), lambda X, Y, Z: s(X) * c(Y)),
        "pn": (2, [O.PERIODIC, O.PERIODIC, O.WALL, O.WALL], lambda X, Y, Z: -4 * PI * PI * (s(X) + c(Y)),
               lambda X, Y, Z: s(X) + c(Y)),
        "nn": (2, [O.WALL] * 4, lambda X, Y, Z: -8 * PI * PI * c(X) * c(Y), lambda X, Y, Z: c(X) * c(Y)),
        "ppp": (3, [O.PERIODIC] * 6, lambda X, Y, Z: -12 * PI * PI * s(X) * c(Y) * s(Z),
                lambda X, Y, Z: s(X) * c(Y) * s(Z)),
        "ppn": (3, [O.PERIODIC] * 4 + [O.WALL] * 2, lambda X, Y, Z: -4 * PI * PI * (s(X) + s(Y) + c(Z)),
                lambda X, Y, Z: s(X) + s(Y) + c(Z)),
        "npn": (3, [O.WALL, O.WALL, O.PERIODIC, O.PERIODIC, O.WALL, O.WALL],
                lambda X, Y, Z: -12 * PI * PI * c(X) * c(Y) * c(Z), lambda X, Y, Z: c(X) * c(Y) * c(Z)),
        "nnn": (3, [O.WALL] * 6, lambda X, Y, Z: -12 * PI * PI * c(X) * c(Y) * c(Z),
                lambda X, Y, Z: c(X) * c(Y) * c(Z)),
        # walls in y with x, z periodic (the channel's solver; beyond the reference's dispatch)
        "pnp": (3, [O.PERIODIC, O.PERIODIC, O.WALL, O.WALL, O.PERIODIC, O.PERIODIC],
                lambda X, Y, Z: -4 * PI * PI * (s(X) + c(Y) + s(Z)), lambda X, Y, Z: s(X) + c(Y) + s(Z)),
    }
    return cases[name]


def poisson_rhs_grid(dim, N):
    d = 1.0 / N
    x = (np.arange(1, N + 1) - 0.5) * d
    if dim == 2:
        Y, X = np.meshgrid(x, x, indexing="ij")
        return X, Y, np.zeros_like(X)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    return X, Y, Z


def convergence_slope(Ns, errs):
    return -np.polyfit(np.log(np.asarray(Ns, float)), np.log(np.asarray(errs)), 1)[0]


def decaying_turbulence_2d(n, L, seed, kpeak=8.0):
    """Seeded 2D periodic velocity (u, v) interiors of shape (n, n) (axis 1 = x) with energy
    spectrum E(k) ~ k^4 exp(-(k/kpeak)^2), unit kinetic energy 1/2 <u^2 + v^2> = 1, and zero
    discrete divergence.

    A Gaussian streamfunction psi at the cell corners (i delta, j delta) with |psi_k|^2 ~
    k exp(-(k/kpeak)^2) gives E(k) ~ k |u_k|^2 ~ k^3 |psi_k|^2; u = (psi(i,j) - psi(i,j-1))/delta
    and v = -(psi(i,j) - psi(i-1,j))/delta on the MAC faces are then divergence-free to
    rounding, and the discrete projection below removes what rounding leaves."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = L / n
    k = np.fft.fftfreq(n, 1.0 / n)
    kk = np.sqrt(k[None, :] ** 2 + k[:, None] ** 2)
    amp = np.sqrt(kk * np.exp(-((kk / kpeak) ** 2)))
    amp[0, 0] = 0.0
    spec = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * amp
    psi = np.fft.ifft2(spec).real
    u = (psi - np.roll(psi, 1, axis=0)) / d
    v = -(psi - np.roll(psi, 1, axis=1)) / d
    s = 1.0 / np.sqrt(0.5 * np.mean(u ** 2 + v ** 2))
    return project_pp_2d(u * s, v * s, d)


def project_pp_2d(u, v, d):
    """Discrete projection of a periodic MAC velocity: v - G P D v with the 5-point
    Laplacian's modified wavenumbers (the pp solver's operator)."""
    n1, n0 = u.shape
    div = ((u - np.roll(u, 1, axis=1)) + (v - np.roll(v, 1, axis=0))) / d
    kx = 2.0 * (np.cos(2.0 * np.pi * np.arange(n0) / n0) - 1.0) / d ** 2
    ky = 2.0 * (np.cos(2.0 * np.pi * np.arange(n1) / n1) - 1.0) / d ** 2
    lam = kx[None, :] + ky[:, None]
    dh = np.fft.fft2(div)
    ph = np.where(lam == 0.0, 0.0, dh / np.where(lam == 0.0, 1.0, lam))
    phi = np.fft.ifft2(ph).real
    return u - (np.roll(phi, -1, axis=1) - phi) / d, v - (np.roll(phi, -1, axis=0) - phi) / d


def kolmogorov_ensemble(nruns=512, seed=5, sizes=(64, 96, 128, 192, 256), re_range=(50.0, 500.0), amp=1e-2):
    """Seeded ensemble of 2D Kolmogorov runs: N ~ U{sizes}, Re ~ U[re_range], nu = 1/Re
    (PCG64(seed)); the initial velocity of run q is uniform noise in [-amp, amp] from
    PCG64(seed + q).  Returns (n, nu, init) with init(q) -> (u, v) interiors (N, N)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = rng.choice(np.asarray(sizes), size=nruns)
    re = rng.uniform(re_range[0], re_range[1], size=nruns)

    def init(q):
        r = np.random.Generator(np.random.PCG64(seed + q))
        N = int(n[q])
        return amp * r.uniform(-1, 1, (N, N)), amp * r.uniform(-1, 1, (N, N))

    return n.astype(np.int32), 1.0 / re, init
