"""fields_mod generics and add_advection through the C ABI (fen_gradient, fen_laplacian,
fen_add_advection).

The device operators evaluate FEN's formulas (fields.f90:31-64, 256-343;
navier_stokes.f90:261-353) in the reference's operation order without FMA contraction, so
in FP64 contexts they are bit-identical to the same formulas evaluated here in numpy and to
the oracle's add_advection.  In mixed contexts the field is the double-float pair joined to
FP64 (about 48 bits), so the results agree to 1e-14 relative.
"""
import numpy as np
import pytest

import fen_gb300 as F
from oracle import oracle as O
from tests import cases as C

pytestmark = pytest.mark.gpu

CASES = {
    "2d_iso": dict(dim=2, n=(24, 16, 1), L=(1.5, 1.0, 1.0 / 16), aniso=False, bc=[O.PERIODIC, O.PERIODIC, O.WALL, O.WALL]),
    "3d_iso": dict(dim=3, n=(16, 12, 8), L=(2.0, 1.5, 1.0), aniso=False, bc=[O.PERIODIC] * 6),
    "3d_aniso": dict(dim=3, n=(16, 12, 8), L=(2.0, 1.0, 3.0), aniso=True,
                     bc=[O.PERIODIC, O.PERIODIC, O.WALL, O.WALL, O.PERIODIC, O.PERIODIC]),
}


def _make(case, prec=F.FP64):
    c = CASES[case]
    n, L = c["n"], c["L"]
    g = F.Grid(n[0], n[1], n[2] if c["dim"] == 3 else 1, L[0], L[1], L[2], bc=c["bc"], dim=c["dim"], aniso=c["aniso"])
    s = F.Solver(g, viscosity=0.01, precision=prec)
    o = O.Oracle(c["dim"], n, L, bc=c["bc"], viscosity=0.01, aniso=c["aniso"])
    return s, o, c["dim"]


def _plane(a, dim):
    """(k, j, i) ghosted array -> the arrays the formulas index (2D: the k = 1 plane)."""
    return a if dim == 3 else a[1:2]


def _ids(s):
    d = s.grid.deltas if s.grid.aniso else (s.grid.delta,) * 3
    return [1.0 / x for x in d], [1.0 / (x * x) for x in d]


def np_gradient(f, dim, id_):
    c = f[1:-1, 1:-1, 1:-1] if dim == 3 else f[:, 1:-1, 1:-1]
    sl = (lambda a: a[1:-1, 1:-1, 1:-1]) if dim == 3 else (lambda a: a[:, 1:-1, 1:-1])
    gx = (sl(np.roll(f, -1, axis=2)) - c) * id_[0]
    gy = (sl(np.roll(f, -1, axis=1)) - c) * id_[1]
    out = [gx, gy]
    if dim == 3:
        out.append((sl(np.roll(f, -1, axis=0)) - c) * id_[2])
    return out


def np_laplacian(f, dim, id2, iso, zform):
    sl = (lambda a: a[1:-1, 1:-1, 1:-1]) if dim == 3 else (lambda a: a[:, 1:-1, 1:-1])
    c = sl(f)
    two = 2.0 * c
    dx = (sl(np.roll(f, -1, axis=2)) - two) + sl(np.roll(f, 1, axis=2))
    dy = (sl(np.roll(f, -1, axis=1)) - two) + sl(np.roll(f, 1, axis=1))
    if dim == 2:
        return (dx + dy) * id2[0] if iso else dx * id2[0] + dy * id2[1]
    dz = (sl(np.roll(f, -1, axis=0)) - two) + sl(np.roll(f, 1, axis=0))
    if not iso:
        return dx * id2[0] + dy * id2[1] + dz * id2[2]
    return ((dx + dy) + dz) * id2[0] if zform else (dx + dy) * id2[0] + dz * id2[0]


@pytest.mark.parametrize("case", list(CASES))
def test_gradient_and_laplacian_bit_exact(fen_lib, case):
    s, _, dim = _make(case)
    rng = np.random.Generator(np.random.PCG64(3))
    id_, id2 = _ids(s)
    for fid in (F.P, F.PHI, F.U, F.V) + ((F.W,) if dim == 3 else ()):
        a = rng.standard_normal(s.grid.shape)
        s.set_field(fid, a)
        f = _plane(a, dim)
        if fid in (F.P, F.PHI):
            got = s.gradient(fid)
            want = np_gradient(f, dim, id_)
            for q in range(dim):
                assert np.array_equal(got[q], want[q]), (fid, q)
        lap = s.laplacian(fid)
        want = np_laplacian(f, dim, id2, not s.grid.aniso, fid == F.W)
        assert np.array_equal(lap, want), fid


@pytest.mark.parametrize("case", list(CASES))
def test_add_advection_matches_oracle(fen_lib, case):
    s, o, dim = _make(case)
    rng = np.random.Generator(np.random.PCG64(4))
    for fid in ([O.U, O.V] if dim == 2 else [O.U, O.V, O.W]):
        a = rng.standard_normal(s.grid.shape)
        o.field(fid)[...] = a
        s.set_field(fid, a)
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)
    o.add_advection()
    base = [rng.standard_normal(s.grid.interior_shape) for _ in range(dim)]
    got = s.add_advection([b.copy() for b in base])
    for q in range(dim):
        want = C.interior(o.field(O.DV[q]), dim).reshape(s.grid.interior_shape)
        # add_advection adds to the caller's RHS: RHS - 0 - terms, the same rounding as the
        # oracle's 0 - terms only when RHS is zero, so compare the increment to rounding
        assert np.abs((got[q] - base[q]) - want).max() <= 1e-12 * np.abs(want).max()
    zero = s.add_advection()
    for q in range(dim):
        want = C.interior(o.field(O.DV[q]), dim).reshape(s.grid.interior_shape)
        assert np.array_equal(zero[q], want), q


def test_operators_in_mixed_context(fen_lib):
    s32, _, dim = _make("3d_aniso", F.MIXED)
    s64, _, _ = _make("3d_aniso", F.FP64)
    rng = np.random.Generator(np.random.PCG64(6))
    for fid in (F.U, F.V, F.W, F.P):
        a = rng.standard_normal(s64.grid.shape)
        s32.set_field(fid, a)
        s64.set_field(fid, a)
    for fid in (F.U, F.W, F.P):
        a, b = s32.laplacian(fid), s64.laplacian(fid)
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
    ga, gb = s32.gradient(F.P), s64.gradient(F.P)
    for q in range(3):
        assert np.abs(ga[q] - gb[q]).max() <= 1e-13 * np.abs(gb[q]).max()
    ra, rb = s32.add_advection(), s64.add_advection()
    for q in range(3):
        assert np.abs(ra[q] - rb[q]).max() <= 1e-13 * np.abs(rb[q]).max()


def test_operator_argument_errors(fen_lib):
    s, _, _ = _make("3d_iso")
    with pytest.raises(F.FenError, match="scalar"):
        s.gradient(F.U)
    with pytest.raises(F.FenError, match="ghost"):
        s.laplacian(F.S_X)
