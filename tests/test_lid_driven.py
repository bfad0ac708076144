"""FEN's lid-driven cavity against the centreline profiles FEN ships with it.

test/small_test/navier_stokes/lid_driven/lid_driven.f90:26-75: unit square, 64^2, 'Wall' on
every side, viscosity 1e-3 (Re = 1000), u = 1 on the top wall, set_timestep(U = 1) with the
module default CFL = 1, steady when max|u - u_old| < 1e-8 over the whole u array.  FEN's
postpro.py:50-66 samples the steady u along the vertical centreline as the mean of the two
face columns i = nx/2, nx/2 + 1 (0.5 (u[nx/2] + u[nx/2 - 1]) with 0-based interior indices),
v along the horizontal centreline likewise, and plots them against uref/vref
(tests/golden/lid_driven_ghia.npz, made by tests/golden/make_ghia.py from FEN's files).

Here the profiles are compared at the reference points by linear interpolation between the
samples' cell-centre positions, with the wall values (u = 0 at y = 0, u = 1 at y = 1, v = 0
at x = 0, 1) at the ends.  Bound: at most 0.025 and an RMS of at most 0.015 (lid velocity
units) on each profile; the second-order 64^2 solution is measured at 0.018 / 0.012.

The CPU test pins the oracle itself to that data; the GPU test runs the same case through the
C ABI, holds it to 1e-12 of the oracle over the first 200 steps, reaches the steady state at
the oracle's step count (+-2) and meets the same bound.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

N, NU = 64, 1e-3
MAX_ERR, RMS_ERR = 0.025, 0.015
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lid_driven_ghia.npz")


def centreline_errors(u, v):
    """u, v: interior arrays (ny, nx) (axis 1 = x).  Returns the max and RMS deviation of the
    centreline profiles from FEN's reference points."""
    ref = np.load(GOLD)
    uref, vref = ref["uref"], ref["vref"]
    d = 1.0 / N
    uy = 0.5 * (u[:, N // 2] + u[:, N // 2 - 1])
    vx = 0.5 * (v[N // 2, :] + v[N // 2 - 1, :])
    pos = np.concatenate([[0.0], (np.arange(N) + 0.5) * d, [1.0]])
    ui = np.interp(uref[:, 0] + 0.5, pos, np.concatenate([[0.0], uy, [1.0]]))
    vi = np.interp(vref[:, 0] + 0.5, pos, np.concatenate([[0.0], vx, [0.0]]))
    eu, ev = ui - uref[:, 1], vi - vref[:, 1]
    return (np.abs(eu).max(), np.sqrt(np.mean(eu ** 2))), (np.abs(ev).max(), np.sqrt(np.mean(ev ** 2)))


def _oracle():
    o = O.Oracle(2, (N, N, 1), (1.0, 1.0, 1.0 / N), bc=[O.WALL] * 4, viscosity=NU, nthreads=1)
    o.bc_values(O.U, 3)[...] = 1.0  # v%x%bc%top = 1 (lid_driven.f90:59)
    for f in (O.U, O.V, O.P):
        o.update_ghost_nodes(f)
    return o


def run_oracle_to_steady(max_steps=20000):
    o = _oracle()
    dt = o.set_timestep(1.0)
    uo = o.field(O.U).copy()
    for step in range(1, max_steps + 1):
        o.step(dt)
        u = o.field(O.U)
        e = np.abs(u - uo).max()
        if e < 1e-8 and step > 1:
            return o, step
        uo = u.copy()
    raise AssertionError("no steady state")


def test_golden_profiles_are_fens():
    ref = np.load(GOLD)
    assert ref["uref"].shape == (17, 2) and ref["vref"].shape == (17, 2)
    # positions relative to the centre, inside the cavity up to the rounding of FEN's file
    for a in (ref["uref"], ref["vref"]):
        assert np.all(np.abs(a[:, 0]) <= 0.5 + 1e-3)
    # the lid row of the u profile carries the lid velocity, the bottom row about zero
    u = ref["uref"][np.argsort(ref["uref"][:, 0])]
    assert abs(u[-1, 1] - 1.0) < 1e-3 and abs(u[0, 1]) < 1e-3


def test_oracle_lid_driven_matches_fens_profiles():
    o, steps = run_oracle_to_steady()
    (mu, ru), (mv, rv) = centreline_errors(o.field(O.U)[1, 1:-1, 1:-1], o.field(O.V)[1, 1:-1, 1:-1])
    assert mu <= MAX_ERR and ru <= RMS_ERR, (mu, ru)
    assert mv <= MAX_ERR and rv <= RMS_ERR, (mv, rv)
    assert 5000 < steps < 10000, steps


@pytest.mark.gpu
def test_gpu_lid_driven_to_steady_state(fen_lib):
    import fen_gb300 as F
    from tests import cases as C

    o, steps_o = run_oracle_to_steady()
    # the GPU run through the C ABI, with the oracle alongside for the first 200 steps
    s = F.Solver(F.Grid(N, N, 1, 1.0, 1.0, 1.0 / N, bc=["Wall"] * 4), viscosity=NU)
    top = np.ones(_oracle().bc_values(O.U, 3).shape)
    s.set_bc_values(F.U, F.TOP, top)
    for f in (F.U, F.V, F.P):
        s.update_ghost_nodes(f)
    dt = s.set_timestep(1.0)
    o2 = _oracle()
    assert o2.set_timestep(1.0) == dt
    o2.run(200, dt)
    uo = s.get_field(F.U)
    steps_g = None
    for step in range(1, 20001):
        s.advance_solution(step, dt)
        u = s.get_field(F.U)
        if step == 200:
            for fid in (O.U, O.V, O.P):
                a, b = C.interior(s.get_field(fid), 2), C.interior(o2.field(fid), 2)
                if fid == O.P:
                    a, b = a - a.mean(), b - b.mean()
                assert C.rel_l2(a, b) < 1e-12, (fid, C.rel_l2(a, b))
        if np.abs(u - uo).max() < 1e-8 and step > 1:
            steps_g = step
            break
        uo = u
    assert steps_g is not None and abs(steps_g - steps_o) <= 2, (steps_g, steps_o)
    ug, vg = C.interior(s.get_field(F.U), 2), C.interior(s.get_field(F.V), 2)
    assert C.rel_l2(ug, C.interior(o.field(O.U), 2)) < 1e-9
    (mu, ru), (mv, rv) = centreline_errors(ug, vg)
    assert mu <= MAX_ERR and ru <= RMS_ERR, (mu, ru)
    assert mv <= MAX_ERR and rv <= RMS_ERR, (mv, rv)
    assert abs(s.status()["maxdiv"]) < 1e-10
