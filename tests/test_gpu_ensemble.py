"""GPU tests of the batched ensemble (2D periodic forced runs, FP32 with FP64 reductions).

Each run of the ensemble is checked against the FP64 oracle of the same run (FEN's 2D
periodic step with a source field S_x = sin(4y) and constant-CFL time stepping), and the
ensemble's own invariances are checked: the tile shape (CTAs per run) and the autotuner do
not change the results beyond FP32 rounding, and a low-Reynolds Kolmogorov run converges to
the discrete laminar solution.
"""
import numpy as np
import pytest

import fen_gb300 as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu

L = 2 * np.pi
KF = 4


def _noise(n, seed, amp=1e-2):
    rng = np.random.Generator(np.random.PCG64(seed))
    return amp * rng.uniform(-1, 1, (n, n)), amp * rng.uniform(-1, 1, (n, n))


def _oracle_run(n, nu, u0, v0, nsteps, cfl=0.4, U=1.0):
    o = O.Oracle(2, (n, n, 1), (L, L, L / n), viscosity=nu, cfl=cfl, constant_cfl=True)
    d = L / n
    y = (np.arange(n) + 0.5) * d
    o.field(O.S[0])[1, 1:-1, 1:-1] = np.sin(KF * y)[:, None]
    o.field(O.U)[1, 1:-1, 1:-1] = u0
    o.field(O.V)[1, 1:-1, 1:-1] = v0
    for fid in (O.U, O.V, O.P):
        o.update_ghost_nodes(fid)
    dt = o.set_timestep(U)
    for _ in range(nsteps):
        dt = o.step(dt)
    return [o.field(f)[1, 1:-1, 1:-1].copy() for f in (O.U, O.V, O.P)], dt


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _make(sizes, nus, seeds):
    e = F.Ensemble(sizes, nus, length=L, CFL=0.4, forcing=(1.0, KF))
    for q, (n, s) in enumerate(zip(sizes, seeds)):
        u0, v0 = _noise(n, s)
        e.upload(q, u0, v0)
    e.set_timestep(1.0)
    return e


SIZES = [64, 96, 128, 192, 256, 64, 128, 256]
NUS = [1 / 50, 1 / 500, 1 / 120, 1 / 300, 1 / 80, 1 / 400, 1 / 200, 1 / 500]
SEEDS = [5 + q for q in range(len(SIZES))]
# FP32 state against the FP64 oracle after 40 steps.  Velocity errors are FP32 rounding of
# the whole velocity: |u - u_o| / |(u_o, v_o)| and |v - v_o| / |(u_o, v_o)| stay below 1e-6
# (measured 2e-8 to 1.6e-7).  The mean-free pressure accumulates the FP32 rounding of each
# step's projection (p = sum of phi): below 1e-3 of |p| (measured up to 3.2e-4).
TOL_V, TOL_P = 1e-6, 1e-3


def _vel_err(ug, vg, uo, vo):
    nv = np.sqrt(np.sum(uo ** 2) + np.sum(vo ** 2))
    return float(np.linalg.norm(ug - uo) / nv), float(np.linalg.norm(vg - vo) / nv)


def test_ensemble_matches_oracle(fen_lib):
    nsteps = 40
    e = _make(SIZES, NUS, SEEDS)
    e.advance(nsteps)
    for q, (n, nu, s) in enumerate(zip(SIZES, NUS, SEEDS)):
        u0, v0 = _noise(n, s)
        (uo, vo, po), dto = _oracle_run(n, nu, u0, v0, nsteps)
        ug, vg, pg = e.download(q)
        st = e.status(q)
        eu, ev = _vel_err(ug, vg, uo, vo)
        assert eu < TOL_V and ev < TOL_V, (q, n, eu, ev)
        assert _rel(pg - pg.mean(), po - po.mean()) < TOL_P, (q, n)
        assert abs(st["dt"] - dto) <= 1e-5 * dto
        assert abs(st["maxdiv"]) < 1e-3 * np.abs(ug).max() * n / L
        assert not st["nan"]


def test_ensemble_tile_shape_does_not_change_results(fen_lib):
    sizes, nus, seeds = [128, 96, 64, 128], [1 / 100, 1 / 300, 1 / 60, 1 / 450], [11, 12, 13, 14]
    out = []
    for groups in ({128: 2, 96: 1, 64: 1}, {128: 8, 96: 4, 64: 2}):
        e = _make(sizes, nus, seeds)
        e.set_config(1024, groups)
        assert e.config()["groups"] == groups
        e.advance(30)
        out.append([e.download(q) for q in range(len(sizes))])
    for a, b in zip(*out):
        eu, ev = _vel_err(a[0], a[1], b[0], b[1])
        assert eu < 1e-6 and ev < 1e-6


def test_ensemble_tuner_and_cache(fen_lib, tmp_path):
    sizes = [64, 96, 128, 192, 256] * 2
    nus = list(np.linspace(1 / 500, 1 / 50, len(sizes)))
    cache = str(tmp_path / "tune.txt")
    e = _make(sizes, nus, range(len(sizes)))
    cfg = e.tune(steps=4, cache=cache)
    assert cfg["threads"] in (512, 1024)
    for n, g in cfg["groups"].items():
        assert n % g == 0 and F.ensemble_smem_bytes(n, g) <= 232448
    text = open(cache).read()
    assert "threads" in text
    # state restored: tuning then advancing equals advancing directly
    e.advance(5)
    f = _make(sizes, nus, range(len(sizes)))
    f.set_config(cfg["threads"], cfg["groups"])
    f.advance(5)
    for q in range(len(sizes)):
        assert np.array_equal(e.download(q)[0], f.download(q)[0])
    # cached configuration reused
    g = _make(sizes, nus, range(len(sizes)))
    assert g.tune(steps=4, cache=cache) == cfg


def test_kolmogorov_laminar_profile(fen_lib):
    # nu = 1/5: the laminar Kolmogorov flow is stable and the discrete steady state is
    # u_j = sin(4 y_j) / (nu lam_4) with lam_4 = (2 - 2 cos(4 d)) / d^2, v = 0.
    n, nu = 64, 1 / 5
    e = F.Ensemble([n], [nu], length=L, CFL=0.4, forcing=(1.0, KF))
    e.upload(0, np.zeros((n, n)), np.zeros((n, n)))
    e.set_timestep(1.0)
    e.advance(3000)
    u, v, _ = e.download(0)
    d = L / n
    y = (np.arange(n) + 0.5) * d
    lam4 = (2 - 2 * np.cos(KF * d)) / d ** 2
    want = np.broadcast_to((np.sin(KF * y) / (nu * lam4))[:, None], (n, n))
    assert _rel(u, want) < 1e-5
    assert np.abs(v).max() < 1e-5 * np.abs(want).max()


def test_ensemble_nan_reported(fen_lib):
    e = F.Ensemble([64, 64], [0.01, 0.01], length=L)
    u0, v0 = _noise(64, 1)
    u0[3, 3] = np.nan
    e.upload(0, u0, v0)
    e.upload(1, *_noise(64, 2))
    e.set_timestep(1.0)
    with pytest.raises(F.FenError, match="run 0"):
        e.advance(2)
    assert e.status(0)["nan"] and not e.status(1)["nan"]


def _np_adjoint(n, nu, u0, v0, dts, dtos, lam_u, lam_v):
    """FP64 numpy adjoint of the same rollout (recorded dt sequence, Kolmogorov forcing)."""
    from tests import adjoint_ref as R

    d = L / n
    S = np.broadcast_to(np.sin(KF * (np.arange(n) + 0.5) * d)[:, None], (n, n))
    xs = [[u0, v0, 0 * u0, 0 * u0, 0 * u0]]
    steps = [R.Step(n, L, nu, dt, dto) for dt, dto in zip(dts, dtos)]
    for st in steps:
        xs.append(st.forward(xs[-1], S))
    lam = [lam_u, lam_v, 0 * u0, 0 * u0, 0 * u0]
    for st, x in zip(reversed(steps), reversed(xs[:-1])):
        lam = st.adjoint(x, lam)
    return lam[0], lam[1], xs[-1]


ADJ_SIZES = [64, 96, 128, 192, 256]
ADJ_NUS = [1 / 60, 1 / 300, 1 / 120, 1 / 200, 1 / 90]


def _ens_gradients(every, nsteps=12, seeds=(21, 22, 23, 24, 25)):
    e = _make(ADJ_SIZES, ADJ_NUS, seeds)
    e.adjoint_setup(nsteps, every)
    e.adjoint_forward()
    tg = []
    for q, n in enumerate(ADJ_SIZES):
        uT, vT, _ = e.download(q)
        tu, tv = _noise(n, 100 + q, amp=1.0)
        e.adjoint_seed(q, uT - tu, vT - tv)
        tg.append((uT, vT, uT - tu, vT - tv))
    e.adjoint_backward()
    return e, tg, [e.adjoint_gradient(q) for q in range(len(ADJ_SIZES))]


def test_ensemble_adjoint_matches_numpy(fen_lib):
    # FP32 ensemble gradient against the FP64 numpy adjoint of the same rollout (the
    # recorded dt sequence); relative L2 within 1e-4 (FP32 transforms and state).
    nsteps = 12
    e, tg, grads = _ens_gradients(5, nsteps)
    for q, (n, nu) in enumerate(zip(ADJ_SIZES, ADJ_NUS)):
        u0, v0 = _noise(n, 21 + q)
        dts, dtos = e.adjoint_dts(q)
        gu_np, gv_np, xT = _np_adjoint(n, nu, u0, v0, dts, dtos, tg[q][2], tg[q][3])
        # the forward of the numpy reference matches the ensemble's final state
        assert np.linalg.norm(xT[0] - tg[q][0]) <= 1e-5 * np.linalg.norm(xT[0])
        gu, gv = grads[q]
        den = np.sqrt(np.sum(gu_np ** 2) + np.sum(gv_np ** 2))
        err = np.sqrt(np.sum((gu - gu_np) ** 2) + np.sum((gv - gv_np) ** 2)) / den
        assert err < 1e-4, (q, n, err)


def test_ensemble_adjoint_checkpoint_invariance_and_forward_state(fen_lib):
    e1, tg1, g1 = _ens_gradients(1)
    e2, tg2, g2 = _ens_gradients(12)
    for a, b in zip(g1, g2):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    # the checkpointing forward leaves the same state as a plain advance
    f = _make(ADJ_SIZES, ADJ_NUS, (21, 22, 23, 24, 25))
    f.advance(12)
    for q in range(len(ADJ_SIZES)):
        assert np.array_equal(f.download(q)[0], tg1[q][0])
