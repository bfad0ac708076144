"""CPU tests of the oracle against the reference's own known answers.

These restate FEN's tests (test/small_test/...) on the CPU restatement:
  * transforms vs FFTW's published definitions (golden vectors, tests/golden/transforms.npz)
  * poisson/convergence_rate: 2nd-order convergence of every fast direct solver
  * poisson/projection: max |div| < 1e-11 after projecting random fields (ppp, ppn)
  * fields/methods: ghost values of analytic fields exact to 1e-14
  * navier_stokes/taylor_green_vortex and advection: 2nd-order convergence
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import cases as C

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "transforms.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("n", [8, 12, 16, 24, 48, 96, 128, 192, 256, 384, 512])
def test_transforms_match_fftw_definitions(gold, n):
    x, z = gold[f"x_{n}"], gold[f"z_{n}"]
    sc = np.abs(x).sum()
    assert np.abs(O.fft(z, -1) - gold[f"fft_{n}"]).max() < 1e-13 * np.abs(z).sum()
    assert np.abs(O.fft(z, +1) - gold[f"bfft_{n}"]).max() < 1e-13 * np.abs(z).sum()
    assert np.abs(O.r2c(x) - gold[f"r2c_{n}"]).max() < 1e-13 * sc
    assert np.abs(O.c2r(gold[f"r2c_{n}"], n) - gold[f"c2r_{n}"]).max() < 1e-12 * sc
    assert np.abs(O.redft10(x) - gold[f"redft10_{n}"]).max() < 1e-13 * sc
    assert np.abs(O.redft01(x) - gold[f"redft01_{n}"]).max() < 1e-13 * sc


def _poisson_errors(name, Ns):
    dim, bc, rhs, sol = C.poisson_case(name)
    errs = []
    for N in Ns:
        n = (N, N, N if dim == 3 else 1)
        o = O.Oracle(dim, n, (1.0, 1.0, 1.0 if dim == 3 else 1.0 / N), bc=bc)
        assert o.solver == name
        X, Y, Z = C.poisson_rhs_grid(dim, N)
        ph = o.field(O.PHI)
        if dim == 2:
            ph[1, 1:-1, 1:-1] = rhs(X, Y, Z)
        else:
            ph[1:-1, 1:-1, 1:-1] = rhs(X, Y, Z)
        o.solve_poisson()
        errs.append(np.abs(C.interior(ph, dim) - sol(X, Y, Z)).max())
    return errs


@pytest.mark.parametrize("name", ["pp", "pn", "nn", "ppp", "ppn", "npn", "nnn", "pnp"])
def test_poisson_second_order(name):
    # poisson/convergence_rate/postpro.py:28 requires slope > 1.8
    Ns = [16, 32, 64] if name in ("pp", "pn", "nn") else [8, 16, 32]
    errs = _poisson_errors(name, Ns)
    assert C.convergence_slope(Ns, errs) > 1.8, errs


@pytest.mark.parametrize("bc", [[O.PERIODIC] * 6, [O.PERIODIC] * 4 + [O.WALL] * 2])
def test_projection_divergence_free(bc):
    # poisson/projection/projection.f90:84-126: v += grad(phi) with lap(phi) = -div(v)
    rng = np.random.Generator(np.random.PCG64(7))
    N = 16
    o = O.Oracle(3, (N, N, N), (1.0, 1.0, 1.0), bc=bc)
    worst = 0.0
    for _ in range(3):
        for f in (O.U, O.V, O.W):
            a = o.field(f)
            a[...] = 0.0
            a[1:-1, 1:-1, 1:-1] = rng.random((N, N, N))
            o.update_ghost_nodes(f)
        div = o.divergence()
        ph = o.field(O.PHI)
        ph[1:-1, 1:-1, 1:-1] = -div
        o.solve_poisson()
        o.update_ghost_nodes(O.PHI)
        d = N
        for f, ax in ((O.U, 2), (O.V, 1), (O.W, 0)):
            a = o.field(f)
            g = (np.roll(ph, -1, axis=ax) - ph) * d
            a[1:-1, 1:-1, 1:-1] += g[1:-1, 1:-1, 1:-1]
            o.update_ghost_nodes(f)
        worst = max(worst, np.abs(o.divergence()).max())
    assert worst < 1e-11


def test_ghost_values_exact():
    # fields/methods.f90:208-280: ghost values of periodic analytic fields to 1e-14
    N = 16
    L = 2 * np.pi
    o = O.Oracle(3, (N, N, N), (L, L, L))
    d = L / N
    g = C.mac_grids(3, (N, N, N), (d, d, d))
    for f, key in ((O.U, "u"), (O.V, "v"), (O.W, "w"), (O.P, "p")):
        X, Y, Z = g[key]
        exact = np.sin(X) * np.cos(Y) * np.sin(Z)
        a = o.field(f)
        a[...] = 0
        a[1:-1, 1:-1, 1:-1] = exact[1:-1, 1:-1, 1:-1]
        o.update_ghost_nodes(f)
        assert np.abs(a - exact).max() < 1e-14


def test_wall_ghost_rules():
    # scalar.f90:259-288 Dirichlet (tangential reflection, normal overwrite) and Neumann
    N = 8
    o = O.Oracle(2, (N, N, 1), (1.0, 1.0, 1.0 / N), bc=[O.WALL] * 4)
    rng = np.random.Generator(np.random.PCG64(3))
    u = o.field(O.U)
    u[1, 1:-1, 1:-1] = rng.random((N, N))
    top = o.bc_values(O.U, 3)
    top[...] = 1.0
    o.update_ghost_nodes(O.U)
    # u is tangential on top: ghost = 2*bc - interior; normal on right: f(hi) = f(hi+1) = bc = 0
    assert np.allclose(u[1, N + 1, 1:N], 2.0 - u[1, N, 1:N])
    assert np.all(u[1, 1:-1, N] == 0.0) and np.all(u[1, 1:-1, N + 1] == 0.0)
    p = o.field(O.P)
    p[1, 1:-1, 1:-1] = rng.random((N, N))
    o.update_ghost_nodes(O.P)
    assert np.all(p[1, 0, 1:-1] == p[1, 1, 1:-1]) and np.all(p[1, 1:-1, 0] == p[1, 1:-1, 1])


def test_tgv2d_second_order():
    # navier_stokes/taylor_green_vortex (taylor_green_vortex.f90:36-67): nu = 1 (module
    # default), dt from set_timestep(U = 2); u error vs exp(-2 nu t) decays at 2nd order
    nu, T = 1.0, 0.1
    Ns, errs = [16, 32, 64], []
    for N in Ns:
        L = 2 * np.pi
        o = O.Oracle(2, (N, N, 1), (L, L, L / N), viscosity=nu)
        u, v, p = C.tgv2d_fields(N, L)
        o.field(O.U)[...] = u
        o.field(O.V)[...] = v
        o.field(O.P)[...] = p
        for f in (O.U, O.V, O.P):
            o.update_ghost_nodes(f)
        dt = o.set_timestep(2.0)
        nst = int(np.ceil(T / dt))
        o.run(nst, dt)
        t = nst * dt
        err = np.abs(C.interior(o.field(O.U), 2) - C.interior(u, 2) * np.exp(-2 * nu * t)).max()
        errs.append(err)
    assert C.convergence_slope(Ns, errs) > 1.8, errs


def test_advection_second_order():
    # navier_stokes/advection: add_advection vs the analytic (u.grad)u, slope > 1.8
    Ns, ex, ey = [16, 32, 64, 128], [], []
    for N in Ns:
        L = 2 * np.pi
        o = O.Oracle(2, (N, N, 1), (L, L, L / N))
        d = L / N
        g = C.mac_grids(2, (N, N, 1), (d, d, d))
        X, Y, _ = g["u"]
        o.field(O.U)[...] = np.sin(X) * np.cos(Y)
        X, Y, _ = g["v"]
        o.field(O.V)[...] = -np.cos(X) * np.sin(Y)
        for f in (O.U, O.V):
            o.update_ghost_nodes(f)
        o.add_advection()
        X, Y, _ = g["u"]
        au = np.sin(X) * np.cos(Y) * np.cos(X) * np.cos(Y) + (-np.cos(X) * np.sin(Y)) * (-np.sin(X) * np.sin(Y))
        X, Y, _ = g["v"]
        av = np.sin(X) * np.cos(Y) * np.sin(X) * np.sin(Y) + (-np.cos(X) * np.sin(Y)) * (-np.cos(X) * np.cos(Y))
        ex.append(np.abs(C.interior(o.field(O.DV[0]), 2) + C.interior(au, 2)).max())
        ey.append(np.abs(C.interior(o.field(O.DV[1]), 2) + C.interior(av, 2)).max())
    assert C.convergence_slope(Ns, ex) > 1.8 and C.convergence_slope(Ns, ey) > 1.8


def test_zero_mode_pivot_exact():
    # poisson.f90:1112-1121: for power-of-two spacing the zero-mode last pivot cancels to
    # exactly 0 and the row is set to 0; the solution stays finite and mean-free (ppn)
    N = 16
    o = O.Oracle(3, (N, N, N), (1.0, 1.0, 1.0), bc=[O.PERIODIC] * 4 + [O.WALL] * 2)
    rng = np.random.Generator(np.random.PCG64(11))
    ph = o.field(O.PHI)
    r = rng.standard_normal((N, N, N))
    ph[1:-1, 1:-1, 1:-1] = r - r.mean()
    o.solve_poisson()
    sol = C.interior(ph, 3)
    assert np.all(np.isfinite(sol))
    assert abs(sol.mean()) < 1e-13


def test_unsupported_bc_rejected():
    # poisson.f90:91-95 aborts when no solver matches (here: walls in x only, 3D)
    with pytest.raises(ValueError):
        O.Oracle(3, (8, 8, 8), (1, 1, 1), bc=[O.WALL, O.WALL] + [O.PERIODIC] * 4)


def test_abc_flow_decay_second_order():
    # large_test/ABC (ABC.f90:40-166): the Arnold-Beltrami-Childress flow u = sin z + cos y,
    # v = sin x + cos z, w = sin y + cos x is a Beltrami field (advection is a gradient the
    # projection removes), so it decays as exp(-nu t); nu = 1 and dt = delta^2 / (16 nu) (the
    # 3D viscous limit delta^2 / (6 nu) of set_timestep sits outside AB2's stability interval
    # for the grid's highest Laplacian mode), errors at t = 0.1 converge at second order
    nu, T = 1.0, 0.1
    Ns, errs = [16, 32, 64], []
    for N in Ns:
        L = 2 * np.pi
        d = L / N
        g = C.mac_grids(3, (N, N, N), (d, d, d))
        X, Y, Z = g["u"]
        u = np.sin(Z) + np.cos(Y)
        X, Y, Z = g["v"]
        v = np.sin(X) + np.cos(Z)
        X, Y, Z = g["w"]
        w = np.sin(Y) + np.cos(X)
        o = O.Oracle(3, (N, N, N), (L, L, L), viscosity=nu)
        for f, a in ((O.U, u), (O.V, v), (O.W, w)):
            o.field(f)[...] = a
            o.update_ghost_nodes(f)
        dt = d * d / (16 * nu)
        o.dt_o = dt
        nst = int(np.ceil(T / dt))
        o.run(nst, dt)
        decay = np.exp(-nu * nst * dt)
        err = max(np.abs(C.interior(o.field(f), 3) - C.interior(a, 3) * decay).max()
                  for f, a in ((O.U, u), (O.V, v), (O.W, w)))
        errs.append(err)
    assert C.convergence_slope(Ns, errs) > 1.8, errs
