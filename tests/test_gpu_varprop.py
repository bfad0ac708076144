"""GPU parity of the variable-property momentum path against the oracle (FP64, 1e-12).

FEN's multiphase and non-Newtonian branches of navier_stokes_solver: density and viscosity
fields on the cells, face densities, the stress-divergence diffusion (2D) and the
Dodd-Ferrante split pressure (navier_stokes.f90:80-136, 140-213, 357-452, 505-566).
"""
import numpy as np
import pytest

import fen_gb300 as F
from oracle import oracle as O
from tests import cases as C

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _fields2d(n, L, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    u, v, p = C.tgv2d_fields(n, L)
    x = (np.arange(n + 2) - 0.5) * L / n
    X, Y = np.meshgrid(x, x)
    rho = np.zeros((3, n + 2, n + 2))
    mu = np.zeros((3, n + 2, n + 2))
    a, b = rng.uniform(0.2, 0.5, 2)
    rho[1] = 1.0 + a * (1 + np.sin(X) * np.cos(2 * Y))
    mu[1] = 0.02 * (1.0 + b * np.cos(X + Y) ** 2)
    return {"u": u, "v": v, "p": p, "rho": rho, "mu": mu}


def _run_pair(dim, n, L, bc_o, bc_g, f, nsteps, dt, var_mu=True, split=None, g=(0, 0, 0), constant_cfl=False):
    o = O.Oracle(dim, n, L, bc=bc_o, density=1.0, viscosity=0.02, g=g, cfl=0.3, constant_cfl=constant_cfl)
    grid = F.Grid(n[0], n[1], n[2], L[0], L[1], L[2], bc=bc_g, dim=dim)
    s = F.Solver(grid, density=1.0, viscosity=0.02, g=g, CFL=0.3, constant_CFL=constant_cfl)
    pairs = [("u", O.U, F.U), ("v", O.V, F.V), ("p", O.P, F.P), ("rho", O.RHO, F.RHO)]
    if dim == 3:
        pairs.insert(2, ("w", O.W, F.W))
    if var_mu:
        pairs.append(("mu", O.MU, F.MU))
    for key, fo, fg in pairs:
        o.field(fo)[...] = f[key]
        o.update_ghost_nodes(fo)
        s.set_field(fg, f[key])
        s.update_ghost_nodes(fg)
    o.set_properties(var_mu=var_mu, split=split is not None, rhomin=split or 1.0)
    if split is not None:
        s.set_split_pressure(split)
    if constant_cfl:
        dto = o.set_timestep(1.0)
        dtg = s.set_timestep(1.0)
        assert dto == dtg
        dt = dto
    else:
        o.dt_o = dt
        s.set_dt_o(dt)
    dto_ = o.run(nsteps, dt)
    dtg_ = s.advance_n(nsteps, dt)
    assert abs(dto_ - dtg_) <= 1e-12 * dto_
    return o, s


def _compare(o, s, dim):
    fids = [(O.U, F.U), (O.V, F.V)] + ([(O.W, F.W)] if dim == 3 else []) + [(O.P, F.P)]
    for fo, fg in fids:
        a = C.interior(s.get_field(fg), dim)
        b = C.interior(o.field(fo), dim)
        if fo == O.P:
            a, b = a - a.mean(), b - b.mean()
        assert C.rel_l2(a, b) < TOL, (fo, C.rel_l2(a, b))


def test_variable_density_and_viscosity_periodic(fen_lib):
    n, L = 32, 2 * np.pi
    f = _fields2d(n, L, 1)
    o, s = _run_pair(2, (n, n, 1), (L, L, L / n), [O.PERIODIC] * 4, ["Periodic"] * 4, f, 20, 5e-3)
    _compare(o, s, 2)


def test_variable_viscosity_channel_with_body_force(fen_lib):
    n = (16, 32, 1)
    L = (np.pi, 2 * np.pi, np.pi / 16)
    f = _fields2d(32, 2 * np.pi, 2)
    f = {k: a[:, :, :18] for k, a in f.items()}
    o, s = _run_pair(2, n, L, [O.PERIODIC, O.PERIODIC, O.WALL, O.WALL], ["Periodic", "Periodic", "Wall", "Wall"],
                     f, 20, 5e-3, g=(0.5, 0.0, 0.0))
    _compare(o, s, 2)


@pytest.mark.parametrize("constant_cfl", [False, True])
def test_split_pressure_with_variable_density(fen_lib, constant_cfl):
    n, L = 32, 2 * np.pi
    f = _fields2d(n, L, 3)
    o, s = _run_pair(2, (n, n, 1), (L, L, L / n), [O.PERIODIC] * 4, ["Periodic"] * 4, f, 20, 5e-3, var_mu=False,
                     split=1.0, constant_cfl=constant_cfl)
    _compare(o, s, 2)
    assert abs(s.status()["maxdiv"]) < 1e-10


def test_variable_density_3d(fen_lib):
    N, L = 16, 2 * np.pi
    u, v, w, p = C.tgv3d_fields(N, L)
    x = (np.arange(N + 2) - 0.5) * L / N
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    f = {"u": u, "v": v, "w": w, "p": p, "rho": 1.0 + 0.3 * np.sin(X) * np.cos(Y) * np.cos(Z)}
    o, s = _run_pair(3, (N, N, N), (L, L, L), [O.PERIODIC] * 6, ["Periodic"] * 6, f, 10, 5e-3, var_mu=False)
    _compare(o, s, 3)


def test_variable_property_errors(fen_lib):
    g3 = F.Grid(8, 8, 8, 1.0, 1.0, 1.0)
    s = F.Solver(g3)
    with pytest.raises(F.FenError, match="2D only"):
        s.set_field(F.MU, s.zeros())
    g2 = F.Grid(8, 8, 1, 1.0, 1.0, 1.0 / 8)
    m = F.Solver(g2, precision=F.MIXED)
    with pytest.raises(F.FenError, match="FP64"):
        m.set_field(F.RHO, m.zeros() + 1.0)
