"""The mixed form's step diagnostics (max div, max |u|+|v|+|w|) against a host evaluation.

The mixed step's diagnostics pass (`k_checks_df`) takes the divergence of the velocity pairs
in FP32 pair arithmetic and the velocity sum of their leading words.  Here the same
arithmetic is evaluated on the host from the downloaded state: the pairs are recovered
exactly from the FP64 download (hi + lo is exact in FP64), every FP32 operation is an IEEE
float32 operation in numpy, and the fused multiply-add of the exact product is formed in
FP64, where the product and its rounding error are exact.  The device compiler may contract
other products and sums of the pair arithmetic into fused multiply-adds, which moves the
divergence by a rounding of its error terms (about 2^-48 of |u|/delta per term), so max div
is held to 2^-40 max|u| / delta_min; max |u|+|v|+|w| has no product and is held bit for bit
(navier_stokes.f90:568-640 prints these diagnostics).
"""
import numpy as np
import pytest

import fen_gb300 as F
from tests import cases as C

pytestmark = pytest.mark.gpu

f32 = np.float32


def _pairs(x):
    hi = x.astype(f32)
    lo = (x - hi.astype(np.float64)).astype(f32)
    return hi, lo


def _two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    e = ((a - (s - bb).astype(f32)).astype(f32) + (b - bb).astype(f32)).astype(f32)
    return s, e


def _mul_pair(ah, al, bh, bl):
    rh = (ah * bh).astype(f32)
    fma = (ah.astype(np.float64) * np.float64(bh) - rh.astype(np.float64)).astype(f32)
    rl = (fma + ((ah * bl).astype(f32) + (al * bh).astype(f32)).astype(f32)).astype(f32)
    return rh, rl


def _add_pair(a, b):
    s, e = _two_sum(a[0], b[0])
    return s, (e + (a[1] + b[1]).astype(f32)).astype(f32)


def _split(x):
    h = f32(x)
    return h, f32(np.float64(x) - np.float64(h))


def _deltas(g):
    return [g.Lx / g.Nx, g.Ly / g.Ny, g.Lz / g.Nz] if g.aniso else [g.Lx / g.Nx] * 3


def _host_checks(s, dim):
    g = s.grid
    d = _deltas(g)
    idp = [_split(1.0 / x) for x in d]
    fields = [_pairs(s.get_field(fid)) for fid in ([F.U, F.V, F.W] if dim == 3 else [F.U, F.V])]
    if dim == 2:
        fields = [(h[1:2], l[1:2]) for h, l in fields]  # the stored plane k = 1
    sl_c = (slice(1, -1),) * 3 if dim == 3 else (slice(0, 1), slice(1, -1), slice(1, -1))
    minus = [(slice(1, -1), slice(1, -1), slice(0, -2)), (slice(1, -1), slice(0, -2), slice(1, -1)),
             (slice(0, -2), slice(1, -1), slice(1, -1))]
    if dim == 2:
        minus = [(slice(0, 1), slice(1, -1), slice(0, -2)), (slice(0, 1), slice(0, -2), slice(1, -1))]
    terms = []
    for q in range(dim):
        h, l = fields[q]
        s0, e0 = _two_sum(h[sl_c], -h[minus[q]])
        e0 = (e0 + (l[sl_c] - l[minus[q]]).astype(f32)).astype(f32)
        terms.append(_mul_pair(s0, e0, *idp[q]))
    r = _add_pair(terms[0], terms[1])
    if dim == 3:
        r = _add_pair(r, terms[2])
    div = (r[0] + r[1]).astype(f32)
    vel = (np.abs(fields[0][0][sl_c]) + np.abs(fields[1][0][sl_c])).astype(f32)
    if dim == 3:
        vel = (vel + np.abs(fields[2][0][sl_c])).astype(f32)
    return div, vel


CASES = {
    "channel3d": dict(dim=3, n=(24, 16, 12), L=(2 * np.pi, 2.0, np.pi),
                      bc=["Periodic", "Periodic", "Wall", "Wall", "Periodic", "Periodic"]),
    "periodic3d": dict(dim=3, n=(16, 12, 18), L=(2 * np.pi, 1.5 * np.pi, 2.25 * np.pi), bc=["Periodic"] * 6),
    "cavity3d": dict(dim=3, n=(12, 16, 8), L=(1.0, 1.0, 1.0), bc=["Wall"] * 6),
    "channel2d": dict(dim=2, n=(32, 24, 1), L=(2.0, 1.0, 1.0 / 24), bc=["Periodic", "Periodic", "Wall", "Wall"]),
}


@pytest.mark.parametrize("case", list(CASES))
def test_mixed_step_diagnostics_match_host(fen_lib, case):
    c = CASES[case]
    dim, n, L, bc = c["dim"], c["n"], c["L"], c["bc"]
    g = F.Grid(n[0], n[1], n[2] if dim == 3 else 1, L[0], L[1], L[2], bc=bc, dim=dim, aniso=True)
    s = F.Solver(g, viscosity=0.02, precision=F.MIXED)
    rng = np.random.Generator(np.random.PCG64(8))
    for fid in [F.U, F.V] + ([F.W] if dim == 3 else []):
        s.set_field(fid, C.random_interior(g.shape, rng, dim))
        s.update_ghost_nodes(fid)
    s.set_dt_o(1e-3)
    for step in range(4):
        s.advance_n(1, 1e-3)
        st = s.status()
        div, vel = _host_checks(s, dim)
        tol = 2.0 ** -40 * float(vel.max()) / min(_deltas(g)[:dim])
        assert abs(st["maxdiv"] - float(div.max())) <= tol, (step, st["maxdiv"], float(div.max()))
        assert st["maxvel"] == float(vel.max())
    assert not st["nan"]
