"""FP64 path against the oracle at the workloads' own sizes and step counts.

2D Taylor-Green 128^2 (nu = 0.01, dt = dt_o = 1e-3, 1000 steps), also against the analytic
exp(-2 nu t) decay, and 3D Taylor-Green 256^3 (Re = 1600, constant CFL 0.5, 200 steps):
u, v, w and mean-free p within 1e-12 relative L2 of the oracle, and the same dt sequence.
The 3D oracle run takes about a minute on 16 host cores.
"""
import os

import numpy as np
import pytest

import fen_gb300 as F
from oracle import oracle as O
from tests import cases as C

pytestmark = pytest.mark.gpu


def _compare(s, o, dim, fids):
    for fg, fo in fids:
        a, b = C.interior(s.get_field(fg), dim), C.interior(o.field(fo), dim)
        if fo == O.P:
            a, b = a - a.mean(), b - b.mean()
        err = C.rel_l2(a, b)
        assert err < 1e-12, (fo, err)


def test_tgv2d_128_1000_steps(fen_lib):
    N, L, nu, dt, nsteps = 128, 2 * np.pi, 0.01, 1e-3, 1000
    u, v, p = C.tgv2d_fields(N, L)
    s = F.Solver(F.Grid(N, N, 1, L, L, L / N), viscosity=nu)
    o = O.Oracle(2, (N, N, 1), (L, L, L / N), viscosity=nu)
    for fg, fo, a in ((F.U, O.U, u), (F.V, O.V, v), (F.P, O.P, p)):
        s.set_field(fg, a)
        s.update_ghost_nodes(fg)
        o.field(fo)[...] = a
        o.update_ghost_nodes(fo)
    s.set_dt_o(dt)
    o.dt_o = dt
    s.advance_n(nsteps, dt)
    o.run(nsteps, dt)
    _compare(s, o, 2, [(F.U, O.U), (F.V, O.V), (F.P, O.P)])
    # analytic decay of the amplitude: exp(-2 nu t) at t = 1
    ug = C.interior(s.get_field(F.U), 2)
    u0 = C.interior(u, 2)
    ratio = np.sum(ug * u0) / np.sum(u0 * u0)
    assert abs(ratio - np.exp(-2 * nu * nsteps * dt)) < 1e-4


def test_tgv3d_256_200_steps(fen_lib):
    N, L, nsteps = 256, 2 * np.pi, 200
    u, v, w, p = C.tgv3d_fields(N, L)
    s = F.Solver(F.Grid(N, N, N, L, L, L), viscosity=1 / 1600, CFL=0.5, constant_CFL=True)
    o = O.Oracle(3, (N, N, N), (L, L, L), viscosity=1 / 1600, cfl=0.5, constant_cfl=True,
                 nthreads=os.cpu_count())
    for fg, fo, a in ((F.U, O.U, u), (F.V, O.V, v), (F.W, O.W, w), (F.P, O.P, p)):
        s.set_field(fg, a)
        s.update_ghost_nodes(fg)
        o.field(fo)[...] = a
        o.update_ghost_nodes(fo)
    dtg = s.set_timestep(1.0)
    dto = o.set_timestep(1.0)
    assert dtg == dto
    dtg = s.advance_n(nsteps, dtg)
    dto = o.run(nsteps, dto)
    assert abs(dtg - dto) <= 1e-12 * dto
    _compare(s, o, 3, [(F.U, O.U), (F.V, O.V), (F.W, O.W), (F.P, O.P)])
