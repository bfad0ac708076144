"""The discrete adjoint beyond 2D periodic: 3D periodic (ppp) and walls in y (pn, pnp).

The step's transpose (fen_adjoint.cuh) is checked against central differences of the FP64
forward rollout through the C ABI: for a loss J = 1/2 |v_T - v_target|^2 over the interior
faces, dJ/dv_0 . d from the adjoint agrees with (J(v_0 + eps d) - J(v_0 - eps d)) / (2 eps)
along seeded smooth directions d, eps = 1e-6 |v_0|, to 1e-6 relative (plus the round-off
floor 1e-9 J).  Walls: the tangential ghosts are reflections of the first interior value
and the wall-normal face at the upper wall is overwritten by the boundary value; the
adjoint folds the first and has no sensitivity for the second.
"""
import numpy as np
import pytest

import fen_gb300 as F
from tests import cases as C

pytestmark = pytest.mark.gpu

PER3 = ["Periodic"] * 6
CHAN3 = ["Periodic", "Periodic", "Wall", "Wall", "Periodic", "Periodic"]
CHAN2 = ["Periodic", "Periodic", "Wall", "Wall"]


def _smooth(rng, shape, kmax=3):
    """A seeded smooth interior field: a few low Fourier modes."""
    nd = len(shape)
    grids = np.meshgrid(*[np.arange(s) / s for s in shape], indexing="ij")
    f = np.zeros(shape)
    for _ in range(6):
        k = rng.integers(0, kmax + 1, size=nd)
        ph = rng.uniform(0, 2 * np.pi, size=nd)
        term = rng.uniform(-1, 1) * np.ones(shape)
        for d in range(nd):
            term = term * np.cos(2 * np.pi * k[d] * grids[d] + ph[d])
        f += term
    return f


class Case:
    def __init__(self, n, L, bc, nu, dt, aniso=False):
        self.dim = 3 if len(bc) == 6 else 2
        self.n, self.L, self.bc, self.nu, self.dt, self.aniso = n, L, bc, nu, dt, aniso
        self.g = F.Grid(n[0], n[1], n[2] if self.dim == 3 else 1, L[0], L[1], L[2], bc=bc, dim=self.dim, aniso=aniso)
        self.vel = [F.U, F.V, F.W][: self.dim]

    def solver(self):
        return F.Solver(self.g, viscosity=self.nu)

    def interior_shape(self):
        return self.g.interior_shape if self.dim == 3 else self.g.interior_shape[1:]

    def full(self, s, interior):
        a = s.zeros()
        if self.dim == 3:
            a[1:-1, 1:-1, 1:-1] = interior
        else:
            a[1, 1:-1, 1:-1] = interior
        return a

    def load(self, s, x0):
        for fid, a in zip(self.vel + [F.P], x0):
            s.set_field(fid, self.full(s, a))
            s.update_ghost_nodes(fid)
        for q in range(self.dim):
            s.set_field(F.DVO_X + q, s.zeros(F.DVO_X + q))
        s.set_dt_o(self.dt)

    def final(self, s):
        return [C.interior(s.get_field(fid), self.dim) for fid in self.vel]

    def loss(self, vT, target):
        return 0.5 * sum(np.sum((a - b) ** 2) for a, b in zip(vT, target))

    def rollout(self, s, x0, nsteps):
        self.load(s, x0)
        s.advance_n(nsteps, self.dt)
        return self.final(s)

    def gradient(self, s, x0, target, nsteps, every):
        self.load(s, x0)
        s.adjoint_setup(nsteps, every)
        s.adjoint_forward(self.dt)
        vT = self.final(s)
        lam = [self.full(s, a - b) for a, b in zip(vT, target)]
        out = s.adjoint_backward(*lam)
        grads = [C.interior(g, self.dim) for g in out[:-1]]
        return self.loss(vT, target), grads, out[-1]


def _problem(case, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    shp = case.interior_shape()
    x0 = [_smooth(rng, shp) for _ in case.vel] + [0.1 * _smooth(rng, shp)]
    target = [_smooth(rng, shp) for _ in case.vel]
    return rng, x0, target


def _fd_check(case, nsteps, every, ndir, seed):
    rng, x0, target = _problem(case, seed)
    s = case.solver()
    J, grads, ms = case.gradient(s, x0, target, nsteps, every)
    f = case.solver()
    norm = np.sqrt(sum(np.sum(a ** 2) for a in x0[:-1]))
    eps = 1e-6
    worst = 0.0
    for _ in range(ndir):
        d = [_smooth(rng, case.interior_shape(), kmax=6) for _ in case.vel]
        dn = np.sqrt(sum(np.sum(a ** 2) for a in d))
        d = [a * norm / dn for a in d]
        Js = []
        for sgn in (1.0, -1.0):
            xp = [a + sgn * eps * b for a, b in zip(x0[:-1], d)] + [x0[-1]]
            Js.append(case.loss(case.rollout(f, xp, nsteps), target))
        fd = (Js[0] - Js[1]) / (2 * eps)
        ad = sum(np.sum(g * b) for g, b in zip(grads, d))
        assert abs(fd - ad) <= 1e-6 * abs(ad) + 1e-9 * J, (fd, ad)
        worst = max(worst, abs(fd - ad) / abs(ad))
    return worst, grads, ms


def test_adjoint_3d_periodic(fen_lib):
    case = Case((16, 12, 8), (2 * np.pi, 1.5 * np.pi, np.pi), PER3, 0.05, 1e-2, aniso=True)
    _fd_check(case, nsteps=8, every=3, ndir=4, seed=11)


@pytest.mark.parametrize("dim", [2, 3])
def test_adjoint_walls_in_y(fen_lib, dim):
    if dim == 2:
        case = Case((32, 24, 1), (2 * np.pi, 2.0, 2.0 / 24), CHAN2, 0.02, 2e-3, aniso=True)
    else:
        case = Case((16, 12, 8), (2 * np.pi, 2.0, np.pi), CHAN3, 0.02, 2e-3, aniso=True)
    worst, grads, _ = _fd_check(case, nsteps=10, every=4, ndir=4, seed=12 + dim)
    # the upper wall face of v carries no sensitivity
    gv = grads[1]
    top = gv[:, -1, :] if dim == 3 else gv[-1, :]
    assert np.all(top == 0.0)


def test_adjoint_checkpoints_do_not_change_3d_gradient(fen_lib):
    case = Case((12, 8, 8), (2 * np.pi, 2.0, np.pi), CHAN3, 0.02, 2e-3, aniso=True)
    _, x0, target = _problem(case, 21)
    s = case.solver()
    ref = None
    for every in (1, 4, 9):
        _, grads, _ = case.gradient(s, x0, target, 9, every)
        if ref is None:
            ref = grads
        else:
            for a, b in zip(grads, ref):
                assert np.array_equal(a, b)


def test_adjoint_tgv3d_64_rollout(fen_lib):
    # 64^3 Taylor-Green rollout (nu = 1/1600, fixed dt = 5e-3, 100 steps, checkpoints every
    # 10): central differences along 16 seeded directions agree to 1e-6, and the backward
    # sweep (with its checkpoint recomputation) costs at most 3 forward rollouts
    N, L = 64, 2 * np.pi
    case = Case((N, N, N), (L, L, L), PER3, 1.0 / 1600, 5e-3)
    u, v, w, p = C.tgv3d_fields(N, L)
    rng = np.random.Generator(np.random.PCG64(31))
    x0 = [C.interior(a, 3) for a in (u, v, w, p)]
    target = [_smooth(rng, case.interior_shape()) for _ in range(3)]
    s = case.solver()
    J, grads, ms = case.gradient(s, x0, target, 100, 10)
    f = case.solver()
    norm = np.sqrt(sum(np.sum(a ** 2) for a in x0[:-1]))
    eps = 1e-6
    for _ in range(16):
        d = [_smooth(rng, case.interior_shape(), kmax=6) for _ in range(3)]
        dn = np.sqrt(sum(np.sum(a ** 2) for a in d))
        d = [a * norm / dn for a in d]
        Js = [case.loss(case.rollout(f, [a + sg * eps * b for a, b in zip(x0[:-1], d)] + [x0[-1]], 100), target)
              for sg in (1.0, -1.0)]
        fd = (Js[0] - Js[1]) / (2 * eps)
        ad = sum(np.sum(g * b) for g, b in zip(grads, d))
        assert abs(fd - ad) <= 1e-6 * abs(ad) + 1e-9 * J, (fd, ad)
    # timing: best of three backward sweeps over the forward time of the same call
    ratios = [ms[0] / ms[1]]
    for _ in range(2):
        ratios.append(case.gradient(s, x0, target, 100, 10)[2])
        ratios[-1] = ratios[-1][0] / ratios[-1][1]
    assert min(ratios) <= 3.0, ratios
