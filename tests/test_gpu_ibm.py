"""GPU parity of the IBM forcing hook (apply_ibm_forcing, navier_stokes.f90:106-108) against
the oracle: solid points take the solid velocity, interface points an interpolation stencil
of nearby velocities; both are applied to v* between the predictor and the projection."""
import numpy as np
import pytest

import fen_gb300 as F
from oracle import oracle as O
from tests import cases as C

pytestmark = pytest.mark.gpu


def _forcing_lists(n, L, R, seed):
    """Points of each component inside a disc of radius R at the box centre: solid (at rest
    inside R - 2 delta, nn = 0) and interface (the ring, a stencil of the next points
    outward, seeded weights and a small boundary velocity)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = L / n
    out = []
    for comp in (0, 1):
        ijk, nn, nb, w, c0 = [], [], [], [], []
        for j in range(1, n + 1):
            for i in range(1, n + 1):
                x = (i - (0.0 if comp == 0 else 0.5)) * d - L / 2
                y = (j - (0.5 if comp == 0 else 0.0)) * d - L / 2
                r = np.hypot(x, y)
                if r < R - 2 * d:
                    ijk.append((i, j, 1)); nn.append(0); nb.append(np.zeros((8, 3))); w.append(np.zeros(8)); c0.append(0.0)
                elif r < R:
                    si, sj = int(np.sign(x) or 1), int(np.sign(y) or 1)
                    st = np.zeros((8, 3), dtype=int)
                    st[0] = (i + si, j, 1); st[1] = (i, j + sj, 1); st[2] = (i + si, j + sj, 1)
                    ww = np.zeros(8); ww[:3] = rng.uniform(0.1, 0.4, 3)
                    ijk.append((i, j, 1)); nn.append(3); nb.append(st); w.append(ww); c0.append(0.01 * rng.standard_normal())
        out.append((np.array(ijk), np.array(nn), np.array(nb), np.array(w), np.array(c0)))
    return out


def test_ibm_forcing_matches_oracle(fen_lib):
    n, L = 32, 2 * np.pi
    u, v, p = C.tgv2d_fields(n, L)
    o = O.Oracle(2, (n, n, 1), (L, L, L / n), viscosity=0.02)
    s = F.Solver(F.Grid(n, n, 1, L, L, L / n), viscosity=0.02)
    for fo, fg, a in ((O.U, F.U, u), (O.V, F.V, v), (O.P, F.P, p)):
        o.field(fo)[...] = a
        o.update_ghost_nodes(fo)
        s.set_field(fg, a)
        s.update_ghost_nodes(fg)
    lists = _forcing_lists(n, L, 1.2, 7)
    for comp, (ijk, nn, nb, w, c0) in enumerate(lists):
        o.set_ibm(comp, ijk, nn, nb, w, c0)
        s.set_ibm_forcing(comp, ijk, nn, nb, w, c0)
    dt = 5e-3
    o.dt_o = dt
    s.set_dt_o(dt)
    o.run(20, dt)
    s.advance_n(20, dt)
    for fo, fg in ((O.U, F.U), (O.V, F.V), (O.P, F.P)):
        a, b = C.interior(s.get_field(fg), 2), C.interior(o.field(fo), 2)
        if fo == O.P:
            a, b = a - a.mean(), b - b.mean()
        assert C.rel_l2(a, b) < 1e-12
    for comp, (ijk, *_rest) in enumerate(lists):
        fe_g, fe_o = s.ibm_force(comp), o.ibm_force(comp, len(ijk))
        assert np.abs(fe_g).max() > 0
        assert np.abs(fe_g - fe_o).max() <= 1e-11 * np.abs(fe_o).max()


def test_ibm_rejects_bad_points(fen_lib):
    s = F.Solver(F.Grid(8, 8, 1, 1.0, 1.0, 1.0 / 8))
    with pytest.raises(F.FenError, match="interior"):
        s.set_ibm_forcing(0, [(0, 3, 1)], [0])
    with pytest.raises(F.FenError, match="0..8"):
        s.set_ibm_forcing(0, [(2, 3, 1)], [9], np.zeros((1, 8, 3)), np.zeros((1, 8)), [0.0])
