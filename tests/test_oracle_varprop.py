"""CPU checks of the oracle's variable-property path (FEN's multiphase / non-Newtonian
branches of navier_stokes_solver: face densities, div(2 mu D), the Dodd-Ferrante split)."""
import numpy as np

from oracle import oracle as O
from tests import cases as C


def _channel(n, L, mu_y, g, rho=1.0):
    # FEN's stress-divergence branch uses the grid's single delta: an isotropic grid
    o = O.Oracle(2, (n[0], n[1], 1), (L[0], L[1], L[0] / n[0]), bc=[O.PERIODIC, O.PERIODIC, O.WALL, O.WALL],
                 density=rho, viscosity=float(np.max(mu_y)), g=(g, 0.0, 0.0))
    o.field(O.MU)[1, 1:-1, 1:-1] = mu_y[:, None]
    o.update_ghost_nodes(O.MU)
    o.set_properties(var_mu=True)
    return o


def test_variable_viscosity_channel_reaches_discrete_steady_state():
    # u(y) with d/dy(mu_e du/dy)/rho = -g, mu_e = (mu_j + mu_j+1)/2 on the edges, u = 0 at the
    # walls through the ghost u_0 = -u_1 (FEN's wall rule for the tangential component)
    n, L, g = (8, 16), (0.5, 1.0), 1.0
    y = (np.arange(n[1]) + 0.5) / n[1]
    mu_y = 0.05 + 0.1 * y ** 2
    o = _channel(n, L, mu_y, g)
    dt = 0.2 * (L[1] / n[1]) ** 2 / mu_y.max()
    o.dt_o = dt
    o.run(6000, dt)
    u = o.field(O.U)[1, 1:-1, 1:-1]
    d = L[1] / n[1]
    mg = np.concatenate([[mu_y[0]], mu_y, [mu_y[-1]]])  # Neumann ghosts of mu
    me = 0.5 * (mg[:-1] + mg[1:])                          # edges j-1/2, j = 1..n+1
    A = np.zeros((n[1], n[1]))
    for j in range(n[1]):
        lo, hi = me[j], me[j + 1]
        A[j, j] = -(lo + hi)
        if j > 0:
            A[j, j - 1] = lo
        else:
            A[j, j] -= lo  # u_0 = -u_1
        if j < n[1] - 1:
            A[j, j + 1] = hi
        else:
            A[j, j] -= hi  # u_{n+1} = -u_n
    want = np.linalg.solve(A / d ** 2, -g * np.ones(n[1]))
    assert np.abs(u - want[:, None]).max() < 1e-8 * np.abs(want).max()
    assert np.abs(o.field(O.V)[1, 1:-1, 1:-1]).max() < 1e-10


def _tgv(o, n, L):
    u, v, p = C.tgv2d_fields(n, L)
    for fid, a in ((O.U, u), (O.V, v), (O.P, p)):
        o.field(fid)[...] = a
        o.update_ghost_nodes(fid)


def test_split_with_uniform_density_equals_standard_step():
    n, L = 16, 2 * np.pi
    out = []
    for split in (False, True):
        o = O.Oracle(2, (n, n, 1), (L, L, L / n), density=2.0, viscosity=0.05)
        _tgv(o, n, L)
        if split:
            o.set_properties(split=True, rhomin=2.0)
        o.dt_o = 1e-2
        o.run(20, 1e-2)
        out.append([o.field(f)[1, 1:-1, 1:-1].copy() for f in (O.U, O.V, O.P)])
    for a, b in zip(*out):
        assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max())


def test_split_projection_is_divergence_free_with_variable_density():
    # the split projects with the constant rhomin (Poisson right-hand side and correction),
    # so the corrected velocity is divergence-free whatever rho(x); without the split FEN's
    # scaling (rho(i,j,k) in the right-hand side, rhof in the correction) is not an exact
    # projection for non-uniform rho, which the GPU path reproduces as it is
    n, L = 16, 2 * np.pi
    o = O.Oracle(2, (n, n, 1), (L, L, L / n), density=1.0, viscosity=0.02)
    _tgv(o, n, L)
    x = (np.arange(n + 2) - 0.5) * L / n
    o.field(O.RHO)[1] = 1.0 + 0.5 * np.sin(x)[None, :] * np.cos(x)[:, None]
    o.update_ghost_nodes(O.RHO)
    o.set_properties(split=True, rhomin=0.5)
    o.dt_o = 1e-2
    o.run(5, 1e-2)
    assert abs(o.diag()["maxdiv"]) < 1e-10
