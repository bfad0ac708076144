"""GPU tests of the discrete adjoint of the 2D periodic FP64 step.

The gradient of J = 1/2 sum (u_T - u*)^2 + (v_T - v*)^2 with respect to the initial velocity
is checked against central finite differences along seeded random directions, against the
numpy adjoint reference, and for independence of the checkpoint interval.
"""
import numpy as np
import pytest

import fen_gb300 as F
from tests import adjoint_ref as R

pytestmark = pytest.mark.gpu

L = 2 * np.pi


def _smooth(rng, n, kmax=6):
    """Random band-limited periodic field of shape (n, n) (axis 1 = x)."""
    k = np.fft.fftfreq(n, 1.0 / n)
    kk = np.sqrt(k[None, :] ** 2 + k[:, None] ** 2)
    spec = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * (kk ** 4) * np.exp(-(kk / 3.0) ** 2)
    spec[kk > kmax] = 0.0
    f = np.fft.ifft2(spec).real
    return f / np.sqrt(np.mean(f ** 2))


def _full(s, interior, fid=0):
    a = s.zeros(fid)
    if a.shape[0] == 1:  # a field without ghosts (dv_o)
        a[0] = interior
    else:
        a[1, 1:-1, 1:-1] = interior
    return a


def _solver(n, nu):
    g = F.Grid(n, n, 1, L, L, L / n)
    return F.Solver(g, viscosity=nu)


def _state(s, u0, v0, p0):
    for fid, a in ((F.U, u0), (F.V, v0), (F.P, p0), (F.DVO_X, 0 * u0), (F.DVO_Y, 0 * u0)):
        s.set_field(fid, _full(s, a, fid))
        if fid in (F.U, F.V, F.P):
            s.update_ghost_nodes(fid)


def _rollout(s, u0, v0, p0, nsteps, dt):
    _state(s, u0, v0, p0)
    s.set_dt_o(dt)
    s.advance_n(nsteps, dt)
    return s.get_field(F.U)[1, 1:-1, 1:-1], s.get_field(F.V)[1, 1:-1, 1:-1]


def _problem(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    u0, v0, p0 = _smooth(rng, n), _smooth(rng, n), 0.1 * _smooth(rng, n)
    tu, tv = _smooth(rng, n), _smooth(rng, n)
    return rng, u0, v0, p0, tu, tv


def _gradient(s, u0, v0, p0, tu, tv, nsteps, dt, every):
    _state(s, u0, v0, p0)
    s.set_dt_o(dt)
    s.adjoint_setup(nsteps, every)
    s.adjoint_forward(dt)
    uT = s.get_field(F.U)[1, 1:-1, 1:-1]
    vT = s.get_field(F.V)[1, 1:-1, 1:-1]
    gu, gv, ms = s.adjoint_backward(_full(s, uT - tu), _full(s, vT - tv))
    J = 0.5 * (np.sum((uT - tu) ** 2) + np.sum((vT - tv) ** 2))
    return J, gu[1, 1:-1, 1:-1], gv[1, 1:-1, 1:-1], ms


def test_numpy_forward_matches_library(fen_lib):
    # pins the numpy reference to the library's forward step
    n, nu, dt = 32, 2e-3, 2e-3
    _, u0, v0, p0, _, _ = _problem(n, 1)
    s = _solver(n, nu)
    uT, vT = _rollout(s, u0, v0, p0, 1, dt)
    x = R.Step(n, L, nu, dt).forward([u0, v0, p0, 0 * u0, 0 * u0])
    assert np.abs(uT - x[0]).max() < 1e-12 * np.abs(x[0]).max()
    assert np.abs(vT - x[1]).max() < 1e-12 * np.abs(x[1]).max()


@pytest.mark.parametrize("nsteps", [1, 4])
def test_adjoint_matches_numpy_reference(fen_lib, nsteps):
    n, nu, dt = 32, 2e-3, 2e-3
    _, u0, v0, p0, tu, tv = _problem(n, 2)
    s = _solver(n, nu)
    J, gu, gv, _ = _gradient(s, u0, v0, p0, tu, tv, nsteps, dt, every=2)
    st = R.Step(n, L, nu, dt)
    xs = [[u0, v0, p0, 0 * u0, 0 * u0]]
    for _ in range(nsteps):
        xs.append(st.forward(xs[-1]))
    lam = [xs[-1][0] - tu, xs[-1][1] - tv, 0 * u0, 0 * u0, 0 * u0]
    for x in reversed(xs[:-1]):
        lam = st.adjoint(x, lam)
    scale = max(np.abs(lam[0]).max(), np.abs(lam[1]).max())
    assert np.abs(gu - lam[0]).max() < 1e-11 * scale
    assert np.abs(gv - lam[1]).max() < 1e-11 * scale


def test_gradient_matches_central_differences(fen_lib):
    n, nu, dt, nsteps = 32, 2e-3, 2e-3, 20
    rng, u0, v0, p0, tu, tv = _problem(n, 3)
    s = _solver(n, nu)
    J, gu, gv, _ = _gradient(s, u0, v0, p0, tu, tv, nsteps, dt, every=5)
    f = _solver(n, nu)
    norm = np.sqrt(np.sum(u0 ** 2) + np.sum(v0 ** 2))
    eps = 1e-6
    for _ in range(4):
        du, dv = _smooth(rng, n, kmax=8), _smooth(rng, n, kmax=8)
        dn = np.sqrt(np.sum(du ** 2) + np.sum(dv ** 2))
        du, dv = du * norm / dn, dv * norm / dn
        Jp = Jm = 0.0
        for sgn in (1.0, -1.0):
            uT, vT = _rollout(f, u0 + sgn * eps * du, v0 + sgn * eps * dv, p0, nsteps, dt)
            Jv = 0.5 * (np.sum((uT - tu) ** 2) + np.sum((vT - tv) ** 2))
            if sgn > 0:
                Jp = Jv
            else:
                Jm = Jv
        fd = (Jp - Jm) / (2 * eps)
        ad = np.sum(gu * du) + np.sum(gv * dv)
        # tolerance: central difference truncation O(eps^2) plus roundoff ~1e-16 J / eps
        assert abs(fd - ad) <= 1e-6 * abs(ad) + 1e-9 * J, (fd, ad)


def test_checkpoint_interval_does_not_change_gradient(fen_lib):
    n, nu, dt, nsteps = 32, 2e-3, 2e-3, 12
    _, u0, v0, p0, tu, tv = _problem(n, 4)
    s = _solver(n, nu)
    ref = None
    for every in (1, 5, 12):
        J, gu, gv, _ = _gradient(s, u0, v0, p0, tu, tv, nsteps, dt, every)
        if ref is None:
            ref = (gu, gv)
        else:
            assert np.array_equal(gu, ref[0]) and np.array_equal(gv, ref[1])


def test_autograd_rollout(fen_lib):
    import torch
    from fen_gb300.autograd import Rollout

    n, nu, dt, nsteps = 32, 2e-3, 2e-3, 6
    _, u0, v0, p0, tu, tv = _problem(n, 5)
    s = _solver(n, nu)
    _state(s, u0, v0, p0)
    U0 = torch.tensor(_full(s, u0), requires_grad=True)
    V0 = torch.tensor(_full(s, v0), requires_grad=True)
    uT, vT = Rollout.apply(U0, V0, s, nsteps, dt, 3)
    loss = 0.5 * (((uT[1, 1:-1, 1:-1] - torch.tensor(tu)) ** 2).sum() + ((vT[1, 1:-1, 1:-1] - torch.tensor(tv)) ** 2).sum())
    loss.backward()
    s2 = _solver(n, nu)
    J, gu, gv, _ = _gradient(s2, u0, v0, p0, tu, tv, nsteps, dt, 3)
    assert abs(loss.item() - J) <= 1e-12 * J
    assert np.array_equal(U0.grad.numpy()[1, 1:-1, 1:-1], gu)
    assert np.array_equal(V0.grad.numpy()[1, 1:-1, 1:-1], gv)
    assert np.all(U0.grad.numpy()[0] == 0) and np.all(U0.grad.numpy()[1, 0] == 0)


def test_adjoint_rejects_unsupported_contexts(fen_lib):
    # walls on every side (nnn) and the mixed form are outside the adjoint's scope
    g = F.Grid(16, 16, 16, L, L, L, bc=["Wall"] * 6)
    s = F.Solver(g)
    with pytest.raises(F.FenError, match="adjoint covers"):
        s.adjoint_setup(4, 2)
    m = F.Solver(F.Grid(16, 16, 1, L, L, L / 16), precision=F.MIXED)
    with pytest.raises(F.FenError, match="adjoint covers"):
        m.adjoint_setup(4, 2)
    s2 = _solver(16, 1e-2)
    s2.adjoint_setup(4, 2)
    s2.set_dt_o(1e-3)
    with pytest.raises(F.FenError, match="dt_o"):
        s2.adjoint_forward(2e-3)


def test_decaying_turbulence_gradient_16_directions(fen_lib):
    # 256^2, nu = 2e-3, dt = 2e-3, 500 steps, checkpoints every 50; central differences with
    # eps = 1e-6 |u0| along 16 seeded unit directions agree with the adjoint to 1e-6
    import bench

    out = bench.form_adjoint(F)
    assert out["fd_max_rel_err"] <= 1e-6, out
    assert out["ratio_backward_over_forward"] <= 3.0, out
