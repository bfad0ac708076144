"""numpy reference of one 2D periodic FP64 step with its tangent-linear and adjoint maps.

Test infrastructure: an independent restatement (vectorised with np.roll) of FEN's
navier_stokes_solver (src/navier_stokes.f90:50-136) on a periodic 2D MAC grid with rho = 1,
used for the dot-product test of the adjoint and to check the library's adjoint step.
Arrays are interiors of shape (ny, nx), axis 1 = x.
"""
import numpy as np


def ip(f):
    return np.roll(f, -1, axis=1)


def im(f):
    return np.roll(f, 1, axis=1)


def jp(f):
    return np.roll(f, -1, axis=0)


def jm(f):
    return np.roll(f, 1, axis=0)


class Step:
    def __init__(self, n, L, nu, dt, dt_o=None):
        self.n, self.d, self.nu, self.dt = n, L / n, nu, dt
        dt_o = dt if dt_o is None else dt_o
        self.A = 1.0 + 0.5 * dt / dt_o
        self.B = -0.5 * dt / dt_o
        k = np.arange(n)
        mw = 2.0 * (np.cos(2.0 * np.pi * k / n) - 1.0) / self.d ** 2
        self.lam = mw[None, :] + mw[:, None]  # (ky, kx)

    # linear operators
    def lap(self, f):
        return (ip(f) + im(f) + jp(f) + jm(f) - 4.0 * f) / self.d ** 2

    def div(self, u, v):
        return ((u - im(u)) + (v - jm(v))) / self.d

    def grad(self, p):
        return (ip(p) - p) / self.d, (jp(p) - p) / self.d

    def poisson(self, b):
        bh = np.fft.fft2(b)
        lam = self.lam
        out = np.where(lam == 0.0, 0.0, bh / np.where(lam == 0.0, 1.0, lam))
        phi = np.fft.ifft2(out).real
        return phi - phi.mean()

    # advection and its linearisation / transpose
    def adv(self, u, v):
        d = self.d
        Fu = 0.25 * (ip(u) + u) ** 2
        Fv = 0.25 * (jp(v) + v) ** 2
        C = 0.25 * (jp(u) + u) * (ip(v) + v)
        Nu = -((Fu - im(Fu)) / d + (C - jm(C)) / d)
        Nv = -((C - im(C)) / d + (Fv - jm(Fv)) / d)
        return Nu, Nv

    def adv_tl(self, u, v, du, dv):
        d = self.d
        dFu = 0.5 * (ip(u) + u) * (ip(du) + du)
        dFv = 0.5 * (jp(v) + v) * (jp(dv) + dv)
        dC = 0.25 * ((jp(du) + du) * (ip(v) + v) + (jp(u) + u) * (ip(dv) + dv))
        return -((dFu - im(dFu)) / d + (dC - jm(dC)) / d), -((dC - im(dC)) / d + (dFv - jm(dFv)) / d)

    def adv_adj(self, u, v, hu, hv):
        d = self.d
        Fu_h = (ip(hu) - hu) / d
        Fv_h = (jp(hv) - hv) / d
        C_h = (jp(hu) - hu) / d + (ip(hv) - hv) / d
        gu = Fu_h * 0.5 * (ip(u) + u) + im(Fu_h * 0.5 * (ip(u) + u)) + C_h * 0.25 * (ip(v) + v) + jm(C_h * 0.25 * (ip(v) + v))
        gv = Fv_h * 0.5 * (jp(v) + v) + jm(Fv_h * 0.5 * (jp(v) + v)) + C_h * 0.25 * (jp(u) + u) + im(C_h * 0.25 * (jp(u) + u))
        return gu, gv

    # the step (S: optional constant body force on u, e.g. Kolmogorov forcing)
    def forward(self, x, S=None):
        u, v, p, ou, ov = x
        Nu, Nv = self.adv(u, v)
        du = Nu + self.nu * self.lap(u) + (0.0 if S is None else S)
        dv = Nv + self.nu * self.lap(v)
        gx, gy = self.grad(p)
        us = u + self.dt * (-gx + self.A * du + self.B * ou)
        vs = v + self.dt * (-gy + self.A * dv + self.B * ov)
        phi = self.poisson(self.div(us, vs) / self.dt)
        fx, fy = self.grad(phi)
        return [us - self.dt * fx, vs - self.dt * fy, p + phi, du, dv]

    def tangent(self, x, dx):
        u, v, p, ou, ov = x
        du_, dv_, dp, dou, dov = dx
        tNu, tNv = self.adv_tl(u, v, du_, dv_)
        ddu = tNu + self.nu * self.lap(du_)
        ddv = tNv + self.nu * self.lap(dv_)
        gx, gy = self.grad(dp)
        us = du_ + self.dt * (-gx + self.A * ddu + self.B * dou)
        vs = dv_ + self.dt * (-gy + self.A * ddv + self.B * dov)
        phi = self.poisson(self.div(us, vs) / self.dt)
        fx, fy = self.grad(phi)
        return [us - self.dt * fx, vs - self.dt * fy, dp + phi, ddu, ddv]

    def adjoint(self, x, lam):
        u, v = x[0], x[1]
        hu, hv, hp, hou, hov = lam
        dt = self.dt
        # G^T = -D, D^T = -G on the periodic MAC grid
        fh = hp + dt * self.div(hu, hv)
        bh = self.poisson(fh)
        gx, gy = self.grad(bh)
        ush, vsh = hu - gx / dt, hv - gy / dt
        ph = hp + dt * self.div(ush, vsh)
        dhu, dhv = hou + dt * self.A * ush, hov + dt * self.A * vsh
        ohu, ohv = dt * self.B * ush, dt * self.B * vsh
        au, av = self.adv_adj(u, v, dhu, dhv)
        return [ush + au + self.nu * self.lap(dhu), vsh + av + self.nu * self.lap(dhv), ph, ohu, ohv]


def dot(a, b):
    return sum(float(np.vdot(x, y)) for x, y in zip(a, b))
