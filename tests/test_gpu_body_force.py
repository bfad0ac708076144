"""The body force S and the AB2 history dv_o through FEN's own field shapes.

FEN allocates S and dv_o without ghost nodes (navier_stokes.f90:759-768; the default gl = 0
of scalar.f90:76-81), and user programs write S%x%f between steps: the forced isotropic
turbulence case sets S = 0.1 (v - <v>) over the interior before every step
(test/large_test/isotropic_turbulence/isotropic.f90:114-152).  These tests do the same
through the C ABI with interior-only host arrays, in 2D and 3D, and hold the FP64 form to
1e-12 and the mixed form to 1e-6 relative L2 of the oracle (p mean-free), so the body-force
branch of the predictor (dv += S/rhof, navier_stokes.f90:245-255) is checked in both forms.
"""
import numpy as np
import pytest

import fen_gb300 as F
from oracle import oracle as O
from tests import cases as C

pytestmark = pytest.mark.gpu

RTOL_FP64 = 1e-12
RTOL_MIXED = 1e-6

CASES = {
    # 2D walls in y (pn solver), anisotropic spacing
    "2d": dict(dim=2, n=(32, 24, 1), L=(2.0, 1.0, 1.0 / 24), bc=[O.PERIODIC, O.PERIODIC, O.WALL, O.WALL]),
    # 3D channel form (walls in y, FFT in x and z, Thomas in y)
    "3d": dict(dim=3, n=(24, 16, 12), L=(2 * np.pi, 2.0, np.pi), bc=[O.PERIODIC, O.PERIODIC, O.WALL, O.WALL,
                                                                    O.PERIODIC, O.PERIODIC]),
}


def _vel_ids(dim):
    return [O.U, O.V] if dim == 2 else [O.U, O.V, O.W]


def _setup(case, prec):
    c = CASES[case]
    dim, n, L, bc = c["dim"], c["n"], c["L"], c["bc"]
    o = O.Oracle(dim, n, L, bc=bc, viscosity=0.02, aniso=True)
    g = F.Grid(n[0], n[1], n[2] if dim == 3 else 1, L[0], L[1], L[2], bc=bc, dim=dim, aniso=True)
    s = F.Solver(g, viscosity=0.02, precision=prec)
    rng = np.random.Generator(np.random.PCG64(17))
    for fid in _vel_ids(dim):
        a = C.random_interior(s.grid.shape, rng, dim)
        o.field(fid)[...] = a
        s.set_field(fid, a)
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)
    return o, s, dim


def _forcing(vel_interior):
    """S = 0.1 (v - <v>) per component over the interior (isotropic.f90:119-150)."""
    return [0.1 * (a - a.mean()) for a in vel_interior]


def _run(case, prec, nsteps=12, dt=2e-3):
    o, s, dim = _setup(case, prec)
    o.dt_o = dt
    s.set_dt_o(dt)
    for _ in range(nsteps):
        # host writes S%x%f between steps, FEN's interior-only shape (gl = 0)
        S_o = _forcing([C.interior(o.field(fid), dim) for fid in _vel_ids(dim)])
        S_g = _forcing([C.interior(s.get_field(fid), dim) for fid in _vel_ids(dim)])
        for q in range(dim):
            C.interior(o.field(O.S[q]), dim)[...] = S_o[q]
            h = S_g[q].reshape(s.field_shape(F.S_X + q))
            assert h.shape == s.grid.interior_shape
            s.set_field(F.S_X + q, h)
        o.step(dt)
        s.advance_solution(1, dt)
    return o, s, dim


def _errors(o, s, dim):
    err = {}
    for fid in _vel_ids(dim) + [O.P]:
        got, want = C.interior(s.get_field(fid), dim), C.interior(o.field(fid), dim)
        if fid == O.P:
            got, want = got - got.mean(), want - want.mean()
        err[fid] = C.rel_l2(got, want)
    return err


@pytest.mark.parametrize("case", list(CASES))
def test_body_force_fp64_matches_oracle(fen_lib, case):
    o, s, dim = _run(case, F.FP64)
    err = _errors(o, s, dim)
    assert max(err.values()) < RTOL_FP64, err
    # dv_o comes back in FEN's interior-only shape and equals the oracle's AB2 history
    for q in range(dim):
        got = s.get_field(F.DVO_X + q)
        assert got.shape == s.grid.interior_shape
        want = C.interior(o.field(O.DVO[q]), dim)
        assert C.rel_l2(got.reshape(want.shape), want) < RTOL_FP64


@pytest.mark.parametrize("case", list(CASES))
def test_body_force_mixed_matches_oracle(fen_lib, case):
    o, s, dim = _run(case, F.MIXED)
    err = _errors(o, s, dim)
    assert max(err.values()) < RTOL_MIXED, err


@pytest.mark.parametrize("prec", [F.FP64, F.MIXED])
def test_interior_only_round_trips(fen_lib, prec):
    """dv_o and S round-trip through interior-only host arrays; gl = 1 uploads of the same
    values agree; the device ghosts are untouched by a gl = 0 upload of u."""
    o, s, dim = _setup("3d", prec)
    rng = np.random.Generator(np.random.PCG64(5))
    tol = 0.0 if prec == F.FP64 else 1e-14
    for fid in (F.DVO_X, F.DVO_Y, F.DVO_Z, F.S_X, F.S_Z):
        a = rng.standard_normal(s.grid.interior_shape)
        s.set_field(fid, a)
        b = s.get_field(fid)
        if fid >= F.S_X and prec == F.MIXED:
            # the mixed form keeps S in FP32
            assert np.abs(b - a).max() <= 2 ** -23 * np.abs(a).max()
        else:
            assert np.abs(b - a).max() <= tol * np.abs(a).max()
        full = np.zeros(s.grid.shape)
        full[1:-1, 1:-1, 1:-1] = a
        s.set_field(fid, full, gl=1)
        assert np.array_equal(s.get_field(fid), b)
        assert np.array_equal(s.get_field(fid, gl=1)[1:-1, 1:-1, 1:-1], b)
    before = s.get_field(F.U)
    inner = rng.standard_normal(s.grid.interior_shape)
    s.set_field(F.U, inner, gl=0)
    after = s.get_field(F.U)
    ghost = np.ones(before.shape, dtype=bool)
    ghost[1:-1, 1:-1, 1:-1] = False
    assert np.abs(after[ghost] - before[ghost]).max() <= tol * max(1.0, np.abs(before).max())
    assert np.abs(after[1:-1, 1:-1, 1:-1] - inner).max() <= tol * np.abs(inner).max()


def test_field_bounds_follow_fen_allocation(fen_lib):
    for case in CASES:
        _, s, dim = _setup(case, F.FP64)
        nx, ny, nz = s.grid.Nx, s.grid.Ny, s.grid.Nz
        top = nz + 1 if dim == 3 else 2
        assert s.field_bounds(F.U) == ((0, 0, 0), (nx + 1, ny + 1, top))
        assert s.field_bounds(F.P) == ((0, 0, 0), (nx + 1, ny + 1, top))
        assert s.field_bounds(F.S_X) == ((1, 1, 1), (nx, ny, nz if dim == 3 else 1))
        assert s.field_bounds(F.DVO_Y) == ((1, 1, 1), (nx, ny, nz if dim == 3 else 1))
        with pytest.raises(ValueError):
            s.set_field(F.S_X, np.zeros(s.grid.shape))
