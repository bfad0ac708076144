"""FP64 and mixed paths against the oracle at the workloads' own sizes.

2D Taylor-Green 128^2 (nu = 0.01, dt = dt_o = 1e-3, 1000 steps), also against the analytic
exp(-2 nu t) decay, and 3D Taylor-Green 256^3 (Re = 1600, constant CFL 0.5, 200 steps):
u, v, w and mean-free p within 1e-12 relative L2 of the oracle, and the same dt sequence.
The channel at its own size (512 x 256 x 384, Re_tau = 180, constant CFL 0.5, Poiseuille +
5% seeded noise): 10 steps of the FP64 path within 1e-12 of the oracle with the same dt
sequence, and the mixed form within 1e-6 of that oracle state.  The 3D oracle runs take
about a minute each on 16 host cores.
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


def test_channel_512x256x384_fp64_and_mixed(fen_lib):
    n, L, nu, nsteps = (512, 256, 384), (4 * np.pi, 2.0, 4 * np.pi / 3), 1.0 / 180, 10
    bc = ["Periodic", "Periodic", "Wall", "Wall", "Periodic", "Periodic"]
    Uc = 1.0 / (2 * nu)  # set_timestep(U) with the centreline velocity
    u, v, w, p = C.channel_fields(n, L, nu)
    o = O.Oracle(3, n, L, bc=[O.PERIODIC, O.PERIODIC, O.WALL, O.WALL, O.PERIODIC, O.PERIODIC], viscosity=nu,
                 g=(1.0, 0.0, 0.0), cfl=0.5, constant_cfl=True, aniso=True, nthreads=os.cpu_count())
    for fo, a in ((O.U, u), (O.V, v), (O.W, w), (O.P, p)):
        o.field(fo)[...] = a
        o.update_ghost_nodes(fo)
    dto = o.set_timestep(Uc)
    dts_o = []
    for _ in range(nsteps):
        dto = o.step(dto)
        dts_o.append(dto)
    fids = [(F.U, O.U), (F.V, O.V), (F.W, O.W), (F.P, O.P)]
    for prec, tol in ((F.FP64, 1e-12), (F.MIXED, 1e-6)):
        g = F.Grid(n[0], n[1], n[2], L[0], L[1], L[2], bc=bc, aniso=True)
        s = F.Solver(g, viscosity=nu, g=(1.0, 0.0, 0.0), CFL=0.5, constant_CFL=True, precision=prec)
        for fg, a in ((F.U, u), (F.V, v), (F.W, w), (F.P, p)):
            s.set_field(fg, a)
            s.update_ghost_nodes(fg)
        dtg = s.set_timestep(Uc)
        dts_g = []
        for step in range(1, nsteps + 1):
            dtg = s.advance_solution(step, dtg)
            dts_g.append(dtg)
        assert np.allclose(dts_g, dts_o, rtol=1e-12 if prec == F.FP64 else 1e-6, atol=0), (prec, dts_g, dts_o)
        for fg, fo in fids:
            a, b = C.interior(s.get_field(fg), 3), C.interior(o.field(fo), 3)
            if fo == O.P:
                a, b = a - a.mean(), b - b.mean()
            err = C.rel_l2(a, b)
            assert err < tol, (prec, fo, err)
        s.destroy_solver()
        del s
