"""navier_stokes/poiseuille (poiseuille.f90:36-40, 77; postpro.py:50, 62): a channel with walls
in y driven by the body force g(1) = 1 (nu = 1) settles to the parabola
u = g y (Ly - y) / (2 nu); the discrete steady state converges to it at second order
(slope > 1.8 over ny = 16, 32, 64).  The oracle is checked on the CPU; the same run through
the C ABI on the GPU."""
import numpy as np
import pytest

from oracle import oracle as O

NYS = (16, 32, 64)
NX = 4


def _setup(ny):
    dy = 1.0 / ny
    dt = 0.125 * dy * dy  # the 2D viscous limit delta^2 / (8 nu) at nu = 1
    nsteps = int(np.ceil(1.0 / dt))  # t = 1: the start-up transient decays as exp(-pi^2 t)
    yc = (np.arange(ny) + 0.5) * dy
    exact = 0.5 * yc * (1.0 - yc)
    return dy, dt, nsteps, exact


def _slope(errs):
    return float(np.log(errs[0] / errs[-1]) / np.log(NYS[-1] / NYS[0]))


def test_poiseuille_second_order_oracle():
    errs = []
    for ny in NYS:
        dy, dt, nsteps, exact = _setup(ny)
        o = O.Oracle(2, (NX, ny, 1), (NX * dy, 1.0, dy), bc=[O.PERIODIC, O.PERIODIC, O.WALL, O.WALL],
                     viscosity=1.0, g=(1.0, 0.0, 0.0))
        o.field(O.U)[1, 1:-1, 1:-1] = exact[:, None]
        o.update_ghost_nodes(O.U)
        o.dt_o = dt
        o.run(nsteps, dt)
        errs.append(np.abs(o.field(O.U)[1, 1:-1, 1:-1] - exact[:, None]).max())
    assert _slope(errs) > 1.8, errs


@pytest.mark.gpu
def test_poiseuille_second_order_gpu(fen_lib):
    import fen_gb300 as F

    errs = []
    for ny in NYS:
        dy, dt, nsteps, exact = _setup(ny)
        g = F.Grid(NX, ny, 1, NX * dy, 1.0, dy, bc=["Periodic", "Periodic", "Wall", "Wall"])
        s = F.Solver(g, viscosity=1.0, g=(1.0, 0.0, 0.0))
        u = s.zeros()
        u[1, 1:-1, 1:-1] = exact[:, None]
        s.set_field(F.U, u)
        s.update_ghost_nodes(F.U)
        s.set_dt_o(dt)
        s.advance_n(nsteps, dt)
        errs.append(np.abs(s.get_field(F.U)[1, 1:-1, 1:-1] - exact[:, None]).max())
    assert _slope(errs) > 1.8, errs
