"""CPU pin of the oracle's IBM forcing (apply_ibm_forcing, navier_stokes.f90:106-108;
eulerian_ibm.f90:194-268) independent of the GPU: after one step the recorded forcing of
every forced point equals (vs - v*)/dt, with v* = v + dt (-grad p / rhof + A dv + B dv_o + g)
formed here in numpy from the oracle's own explicit terms dv, vs = c0 for solid points and
vs = c0 + sum_q w_q v*(nbr_q) for interface points whose stencils reach unforced fluid."""
import numpy as np

from oracle import oracle as O
from tests import cases as C


def test_ibm_forcing_definition():
    n, L, nu, dt = 32, 2 * np.pi, 0.02, 4e-3
    d = L / n
    u, v, p = C.tgv2d_fields(n, L)
    o = O.Oracle(2, (n, n, 1), (L, L, d), viscosity=nu)
    for fid, a in ((O.U, u), (O.V, v), (O.P, p)):
        o.field(fid)[...] = a
        o.update_ghost_nodes(fid)
    o.dt_o = dt  # A = 3/2, B = -1/2; dv_o = 0 at the start
    o.compute_explicit_terms()
    dvx = o.field(O.DV[0])[1].copy()
    # v* at the u points (i + 1/2, j): arrays [j, i] with one ghost layer
    P = p[1]
    ustar = u[1].copy()
    ustar[1:-1, 1:-1] = u[1, 1:-1, 1:-1] + dt * (-(P[1:-1, 2:] - P[1:-1, 1:-1]) / d + 1.5 * dvx[1:-1, 1:-1])

    # solid points (at rest) inside a small box, interface points with stencils to the right
    ijk, nn, nb, w, c0, want = [], [], [], [], [], []
    rng = np.random.Generator(np.random.PCG64(3))
    for j in range(12, 16):
        for i in range(10, 14):
            ijk.append((i, j, 1)); nn.append(0); nb.append(np.zeros((8, 3), int)); w.append(np.zeros(8)); c0.append(0.0)
            want.append((0.0 - ustar[j, i]) / dt)
    for j in range(12, 16):
        i = 14
        st = np.zeros((8, 3), int)
        st[0] = (i + 1, j, 1)
        st[1] = (i + 2, j, 1)
        ww = np.zeros(8)
        ww[:2] = rng.uniform(0.1, 0.5, 2)
        cc = 0.01 * rng.standard_normal()
        ijk.append((i, j, 1)); nn.append(2); nb.append(st); w.append(ww); c0.append(cc)
        vs = cc + ww[0] * ustar[j, i + 1] + ww[1] * ustar[j, i + 2]
        want.append((vs - ustar[j, i]) / dt)
    o.set_ibm(0, np.array(ijk), np.array(nn), np.array(nb), np.array(w), np.array(c0))
    o.step(dt)
    fe = o.ibm_force(0, len(ijk))
    want = np.array(want)
    assert np.abs(fe - want).max() <= 1e-11 * np.abs(want).max()
    # no forcing is recorded for the unforced component
    assert np.all(o.ibm_force(1, 0) == 0)
