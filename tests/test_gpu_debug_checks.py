"""The debug library: every field index of the kernels checked against its array.

libfen_gb300_debug.so is compiled from the same sources with FEN_DEBUG_CHECKS: an index
outside its array is counted, the first one kept, and element 0 used in its place, so the
check records a fault without making one (fen_debug_checks).  Here each solver family,
both arithmetic forms, the transfers, the field operators and the adjoint run through the
debug library: the record must stay empty and every result must equal the release
library's bit for bit (the checks change no arithmetic).  The release library reports -1.
"""
import ctypes

import numpy as np
import pytest

import fen_gb300 as F
from fen_gb300 import build as B
from tests import cases as C

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def debug_lib(fen_lib):
    B.build()
    return F.load_library(B.DEBUG_LIB)


def _record(lib):
    n, first = ctypes.c_longlong(), ctypes.c_longlong()
    assert lib.fen_debug_checks(ctypes.byref(n), ctypes.byref(first)) == 0
    return n.value, first.value


CASES = [
    # (dim, n, L, bc, precision)
    (2, (24, 16, 1), (2.0, 1.0, 1.0 / 16), ["Periodic"] * 4, F.FP64),
    (2, (24, 16, 1), (2.0, 1.0, 1.0 / 16), ["Periodic", "Periodic", "Wall", "Wall"], F.MIXED),
    (2, (16, 32, 1), (1.0, 4.0, 4.0 / 32), ["Wall", "Wall", "Inflow", "Outflow"], F.FP64),
    (3, (16, 12, 8), (2.0, 1.5, 1.0), ["Periodic"] * 6, F.MIXED),
    (3, (16, 12, 8), (2.0, 2.0, 1.0), ["Periodic", "Periodic", "Wall", "Wall", "Periodic", "Periodic"], F.FP64),
    (3, (16, 12, 8), (2.0, 2.0, 1.0), ["Periodic", "Periodic", "Wall", "Wall", "Periodic", "Periodic"], F.MIXED),
    (3, (12, 8, 16), (1.0, 1.0, 1.0), ["Wall"] * 6, F.FP64),
    (3, (16, 12, 12), (1.0, 1.0, 1.0), ["Wall", "Wall", "Periodic", "Periodic", "Wall", "Wall"], F.FP64),
]


def _drive(lib, dim, n, L, bc, prec):
    g = F.Grid(n[0], n[1], n[2] if dim == 3 else 1, L[0], L[1], L[2], bc=bc, dim=dim, aniso=True)
    s = F.Solver(g, viscosity=0.02, g=(0.5, 0.0, 0.0), precision=prec, lib=lib)
    rng = np.random.Generator(np.random.PCG64(3))
    vel = [F.U, F.V] + ([F.W] if dim == 3 else [])
    for fid in vel + [F.P]:
        s.set_field(fid, C.random_interior(g.shape, rng, dim))
        s.update_ghost_nodes(fid)
    s.set_field(F.S_X, rng.standard_normal(g.interior_shape))
    s.set_dt_o(1e-3)
    s.advance_n(4, 1e-3)
    out = [s.get_field(fid) for fid in vel + [F.P, F.PHI]]
    out += [s.get_field(F.DVO_X), s.explicit_terms(), s.divergence(), s.laplacian(F.U)]
    if prec == F.FP64:
        out += list(s.gradient(F.P))
    return out


@pytest.mark.parametrize("case", range(len(CASES)))
def test_debug_library_records_nothing_and_matches_release(fen_lib, debug_lib, case):
    before = _record(debug_lib)
    rel = _drive(None, *CASES[case])
    dbg = _drive(B.DEBUG_LIB, *CASES[case])
    assert _record(debug_lib) == before == (0, 0)
    for a, b in zip(rel, dbg):
        assert np.array_equal(a, b)


def test_debug_library_adjoint_and_release_record(fen_lib, debug_lib):
    g = F.Grid(16, 12, 8, 2.0, 2.0, 1.0, bc=["Periodic", "Periodic", "Wall", "Wall", "Periodic", "Periodic"],
               aniso=True)
    s = F.Solver(g, viscosity=0.02, lib=B.DEBUG_LIB)
    rng = np.random.Generator(np.random.PCG64(4))
    for fid in (F.U, F.V, F.W):
        s.set_field(fid, C.random_interior(g.shape, rng, 3))
        s.update_ghost_nodes(fid)
    s.set_dt_o(1e-3)
    s.adjoint_setup(4, 2)
    s.adjoint_forward(1e-3)
    lam = [C.random_interior(g.shape, rng, 3) for _ in range(3)]
    s.adjoint_backward(*lam)
    assert _record(debug_lib) == (0, 0)
    assert _record(fen_lib)[0] == -1
