"""Checkpoint/restart through the C ABI (FEN test/small_test/io: test_NS.f90 + run.sh).

The reference runs 10 steps saving at step 5, restarts from step 5, runs to 10 and requires
the two state files to be identical (`diff`, io/run.sh:7-11).  The FP64 form is bitwise.
The mixed form keeps its state as double-float pairs (about 48 bits), so the FP64 state
file rounds it once on reload; the FP32 transforms of the next steps then round the
slightly different right-hand sides differently and the two runs drift apart at about
1e-9, far inside the form's accuracy against FP64 (about 1e-7 on the channel workload):
the files agree to 1e-8 relative.
"""
import numpy as np
import pytest

import fen_gb300 as F
from tests import cases as C

pytestmark = pytest.mark.gpu


def _init(s, N, L):
    d = L / N
    g = C.mac_grids(3, (N, N, N), (d, d, d))
    X, Y, _ = g["u"]
    s.set_field(F.U, -np.cos(X) * np.sin(Y))
    X, Y, _ = g["v"]
    s.set_field(F.V, np.sin(X) * np.cos(Y))
    X, _, Z = g["w"]
    s.set_field(F.W, np.sin(X) * np.cos(Z))
    X, Y, _ = g["p"]
    s.set_field(F.P, -0.25 * (np.cos(2 * X) + np.cos(2 * Y)))
    for fid in (F.U, F.V, F.W, F.P):
        s.update_ghost_nodes(fid)


@pytest.mark.parametrize("prec", [F.FP64, F.MIXED])
def test_restart_is_bitwise(fen_lib, tmp_path, prec):
    N, L = 16, 2 * np.pi
    g = F.Grid(N, N, N, L, L, L)
    s = F.Solver(g, precision=prec)
    _init(s, N, L)
    dt = s.set_timestep(2.0)
    for step in range(1, 11):
        dt = s.advance_solution(step, dt)
        if step == 5:
            s.save_state(step, str(tmp_path))
    full = s.save_state(10, str(tmp_path))
    r = F.Solver(g, precision=prec)
    _init(r, N, L)
    dt = r.set_timestep(2.0)
    r.load_state(5, str(tmp_path))
    for step in range(6, 11):
        dt = r.advance_solution(step, dt)
    again = r.save_state(20, str(tmp_path))
    a = np.fromfile(full)
    b = np.fromfile(again)
    assert a.size == 7 * N ** 3
    if prec == F.FP64:
        assert np.array_equal(a, b)
    else:
        assert np.abs(a - b).max() <= 1e-8 * np.abs(a).max()


def test_save_fields_layout(fen_lib, tmp_path):
    N, L = 8, 2 * np.pi
    g = F.Grid(N, N, 1, L, L, L / N)
    s = F.Solver(g)
    u, v, p = C.tgv2d_fields(N, L)
    for fid, a in ((F.U, u), (F.V, v), (F.P, p)):
        s.set_field(fid, a)
        s.update_ghost_nodes(fid)
    s.save_fields(3, str(tmp_path))
    ufull = s.get_field(F.U)[1]
    vx = np.fromfile(tmp_path / "vx_0000003.raw").reshape(N, N)
    assert np.allclose(vx, 0.5 * (ufull[1:-1, 1:-1] + ufull[1:-1, :-2]), rtol=0, atol=1e-15)
    pr = np.fromfile(tmp_path / "p_0000003.raw").reshape(N, N)
    assert np.array_equal(pr, s.get_field(F.P)[1, 1:-1, 1:-1])


def test_multiphase_state_file(fen_lib, tmp_path):
    # FEN's -DMF state file (solver.f90:203-208, 296-304): p, u, v, dv_o%x, dv_o%y, vof, rho,
    # mu, p_o; a restart with variable density and viscosity and the split pressure is
    # bitwise, and vof (the caller's array) comes back as written
    N, L = 32, 2 * np.pi
    g = F.Grid(N, N, 1, L, L, L / N)
    rng = np.random.Generator(np.random.PCG64(12))
    u, v, p = C.tgv2d_fields(N, L)
    x = (np.arange(N + 2) - 0.5) * L / N
    X, Y = np.meshgrid(x, x)
    rho = np.zeros((3, N + 2, N + 2))
    mu = np.zeros((3, N + 2, N + 2))
    rho[1] = 1.0 + 0.4 * (1 + np.sin(X) * np.cos(2 * Y))
    mu[1] = 0.02 * (1.0 + 0.3 * np.cos(X + Y) ** 2)
    vof = rng.uniform(0, 1, g.interior_shape)

    def make():
        s = F.Solver(g, viscosity=0.02)
        for fid, a in ((F.U, u), (F.V, v), (F.P, p), (F.RHO, rho), (F.MU, mu)):
            s.set_field(fid, a)
            s.update_ghost_nodes(fid)
        s.set_split_pressure(1.0)
        s.set_dt_o(1e-3)
        return s

    s = make()
    for step in range(1, 11):
        s.advance_solution(step, 1e-3)
        if step == 5:
            s.save_state_mf(step, vof, str(tmp_path))
    full = s.save_state_mf(10, vof, str(tmp_path))
    data = np.fromfile(full)
    assert data.size == 9 * N * N
    seg = lambda q: data[q * N * N:(q + 1) * N * N].reshape(N, N)
    assert np.array_equal(seg(0), s.get_field(F.P)[1, 1:-1, 1:-1])
    assert np.array_equal(seg(5), vof[0])
    assert np.array_equal(seg(6), rho[1, 1:-1, 1:-1])
    assert np.array_equal(seg(7), mu[1, 1:-1, 1:-1])
    assert np.array_equal(seg(8), s.get_field(F.P_O)[1, 1:-1, 1:-1])
    r = F.Solver(g, viscosity=0.02)
    r.set_split_pressure(1.0)
    r.set_dt_o(1e-3)
    back = r.load_state_mf(5, str(tmp_path))
    assert np.array_equal(back, vof)
    for step in range(6, 11):
        r.advance_solution(step, 1e-3)
    again = np.fromfile(r.save_state_mf(20, vof, str(tmp_path)))
    assert np.array_equal(data, again)
