// Discrete adjoint of the FP64 projection step: 2D and 3D, periodic, or periodic in x (and z)
// with no-slip walls in y (the pn and pnp solvers).
//
// FEN has no differentiation; this is the exact transpose of the discrete step of
// navier_stokes_solver (navier_stokes.f90:50-136) with constant density and viscosity and a
// fixed dt (dt_o = dt).  Forward, with G the forward-difference gradient to faces, D the
// backward-difference divergence, P the fast Poisson solve, N the divergence-form advection,
// L the Laplacian and E the ghost fill (scalar.f90:223-396):
//   dv   = N(E v) + mu/rhof L(E v)        v*  = v + dt(-G E p/rhof + A dv + B dv_o + g)
//   b    = rho/dt D E v*                  phi = P b
//   v'   = E v* - dt/rhof G E phi         p'  = p + phi            dv_o' = dv
// Backward, given the adjoint (^) of (v', p', dv_o'):
//   phi^ = p'^ + dt/rhof D v'^            b^  = P (phi^ - <phi^>)
//   v*^  = E^T (v'^ - rho/dt G b^)        p^  = p'^ + dt/rhof D v*^
//   dv^  = dv_o'^ + dt A v*^              dv_o^ = dt B v*^
//   v^   = v*^ + E^T (N'(v)^T dv^ + mu/rhof L dv^)
// G^T = -D where the adjoint fields are read with zero padding across the walls (they are
// defined on the interior only) and periodic copies along periodic axes; k_adj_ghost writes
// exactly those ghosts.  P is symmetric on mean-free right-hand sides (every b = D v* is mean
// free); with walls the solve's zero mode is a singular tridiagonal system whose particular
// solution depends on the mean, so phi^ loses its mean first.  E^T at the walls (y = 0, Ly):
// the wall-normal velocity at the upper wall face and outside is overwritten by the boundary
// value, so its adjoint is zero; the tangential ghosts are reflections 2 bc - u of the first
// interior value, which folds their sensitivity back with a minus sign (k_adj_state); p and
// phi ghosts (Neumann copies) receive no sensitivity, because the only reads of them (the
// wall-normal gradient at the upper wall face) feed an overwritten value.
#pragma once
#include "fen_types.cuh"

namespace fen {

struct AdjScales {
  double id[3];   // 1/delta per axis
  double id2[3];  // 1/delta^2 per axis
};

// The forward input velocity of the step being transposed, when the step is a graph replay:
// entry *slot of a device table of the segment's stored inputs (nv fields per entry).
struct AdjIn {
  const double* const* tab;
  const int* slot;
  int nv;
};
// *slot = value (value >= 0) or *slot - 1: the replays walk the segment backwards.
static __global__ void k_adj_slot(int* slot, int value) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *slot = (value >= 0) ? value : *slot - 1;
}

// Ghost layer of an adjoint field along one axis: periodic copies, or zeros (walls).  Axes
// are filled x, then y, then z, each over the full extent of the others.
template <int DIM>
__global__ void __launch_bounds__(256) k_adj_ghost(Layout L, double* __restrict__ f, int axis, int zero) {
  const int na = (axis == 0) ? L.n1 + 2 : L.n0 + 2;                               // first free extent
  const int nb = (DIM == 3) ? ((axis == 2) ? L.n1 + 2 : L.n2 + 2) : 1;             // second free extent
  const long long total = 2LL * na * nb;
  const int n = (axis == 0) ? L.n0 : (axis == 1) ? L.n1 : L.n2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int side = (int)(t & 1);
    const long long r = t >> 1;
    const int a = (int)(r % na), b = (int)(r / na);
    int i, j, k;
    const int g = side ? n + 1 : 0, s = side ? 1 : n;  // ghost index and its periodic source
    if (axis == 0) { i = g; j = a; k = b; }
    else if (axis == 1) { i = a; j = g; k = b; }
    else { i = a; j = b; k = g; }
    const long long dst = L.idx(i, j, DIM == 3 ? k : 0);
    double val = 0.0;
    if (!zero) {
      const long long src = (axis == 0) ? L.idx(s, j, DIM == 3 ? k : 0)
                                        : (axis == 1) ? L.idx(i, s, DIM == 3 ? k : 0) : L.idx(i, j, s);
      val = f[src];
    }
    f[dst] = val;
  }
}

// out = a + s D(x, y, z) over the interior (the transpose use of fields.f90:120-153).
template <int DIM>
__global__ void __launch_bounds__(256) k_adj_div(Layout L, const double* __restrict__ a, const double* __restrict__ x,
                                                 const double* __restrict__ y, const double* __restrict__ z, double s,
                                                 AdjScales q, double* __restrict__ out) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const long long c = L.idx(1 + cw.i, 1 + cw.j, kst<DIM>(1 + cw.k));
    double d = (x[c] - x[c - 1]) * q.id[0] + (y[c] - y[c - L.sx]) * q.id[1];
    if (DIM == 3) d += (z[c] - z[c - L.sp]) * q.id[2];
    out[c] = (a ? a[c] : 0.0) + s * d;
  }
}

// (uo, vo, wo) = (u, v, w) - f G(b) on the interior faces; with walls the upper wall face of
// v is not a degree of freedom (E^T) and gets zero.
template <int DIM>
__global__ void __launch_bounds__(256) k_adj_grad(Layout L, const double* __restrict__ u, const double* __restrict__ v,
                                                  const double* __restrict__ w, const double* __restrict__ b, double f,
                                                  AdjScales q, int wall, double* __restrict__ uo, double* __restrict__ vo,
                                                  double* __restrict__ wo) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int j = 1 + cw.j;
    const long long c = L.idx(1 + cw.i, j, kst<DIM>(1 + cw.k));
    uo[c] = u[c] - f * (b[c + 1] - b[c]) * q.id[0];
    vo[c] = (wall && j == L.n1) ? 0.0 : v[c] - f * (b[c + L.sx] - b[c]) * q.id[1];
    if (DIM == 3) wo[c] = w[c] - f * (b[c + L.sp] - b[c]) * q.id[2];
  }
}

// dv^ = dv_o'^ + dt A v*^ (to dh*), dv_o^ = dt B v*^ (in place).
template <int DIM>
__global__ void __launch_bounds__(256) k_adj_dv(Layout L, const double* __restrict__ us, const double* __restrict__ vs,
                                                const double* __restrict__ ws, double* __restrict__ dou,
                                                double* __restrict__ dov, double* __restrict__ dow, double dtA, double dtB,
                                                double* __restrict__ dhu, double* __restrict__ dhv, double* __restrict__ dhw) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const long long c = L.idx(1 + cw.i, 1 + cw.j, kst<DIM>(1 + cw.k));
    dhu[c] = dou[c] + dtA * us[c];
    dhv[c] = dov[c] + dtA * vs[c];
    dou[c] = dtB * us[c];
    dov[c] = dtB * vs[c];
    if (DIM == 3) {
      dhw[c] = dow[c] + dtA * ws[c];
      dow[c] = dtB * ws[c];
    }
  }
}

// Zero the upper wall face of an adjoint wall-normal velocity (E^T of the wall fill).
template <int DIM>
__global__ void k_adj_wall_face(Layout L, double* __restrict__ v) {
  const long long n = (long long)L.n0 * (DIM == 3 ? L.n2 : 1);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % L.n0), k = 1 + (int)(t / L.n0);
    v[L.idx(i, L.n1, kst<DIM>(k))] = 0.0;
  }
}

// Per-CTA interior sums of an adjoint field (for the mean removed before P).
template <int DIM>
__global__ void __launch_bounds__(256) k_adj_sum(Layout L, const double* __restrict__ f, double* __restrict__ partial) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  double s = 0.0;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) s += f[L.idx(1 + cw.i, 1 + cw.j, kst<DIM>(1 + cw.k))];
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// v^ = v*^ + E^T (N'(v)^T dv^ + mu/rhof L dv^)  (navier_stokes.f90:261-353, fields.f90:
// 298-343).  The advection is a sum of face and edge fluxes F = (product of two averages);
// the adjoint of each flux, F^, is the difference of the dv^ it feeds, and each velocity
// gathers F^ times the derivative of the fluxes it enters:
//   Fxx^(c) = (hu(c+1) - hu(c)) idx        Fxy^(c) = (hu(c+sy) - hu(c)) idy + (hv(c+1) - hv(c)) idx
//   Fyy^(c) = (hv(c+sy) - hv(c)) idy       Fxz^(c) = (hu(c+sz) - hu(c)) idz + (hw(c+1) - hw(c)) idx
//   Fzz^(c) = (hw(c+sz) - hw(c)) idz       Fyz^(c) = (hv(c+sz) - hv(c)) idz + (hw(c+sy) - hw(c)) idy
// With walls, the reflected tangential ghosts u(y = 0) = 2 bc - u(j = 1), u(ny + 1) = 2 bc -
// u(ny) (and w) fold the sensitivity they gather back into the first and last rows; only the
// wall-edge flux and the wall-normal diffusion read them (the dv^ of the ghost rows and of
// the wall faces is zero).
template <int DIM>
__global__ void __launch_bounds__(256) k_adj_state(Layout L, AdjIn in, const double* __restrict__ U, const double* __restrict__ V,
                                                   const double* __restrict__ W, const double* __restrict__ us,
                                                   const double* __restrict__ vs, const double* __restrict__ ws,
                                                   const double* __restrict__ hu, const double* __restrict__ hv,
                                                   const double* __restrict__ hw, AdjScales q, double mur, int wall,
                                                   double* __restrict__ uo, double* __restrict__ vo, double* __restrict__ wo) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const long long sy = L.sx, sz = L.sp;
  const double idx = q.id[0], idy = q.id[1], idz = q.id[2];
  if (in.tab) {
    const int e = *in.slot;
    U = in.tab[(long long)e * in.nv];
    V = in.tab[(long long)e * in.nv + 1];
    if (DIM == 3) W = in.tab[(long long)e * in.nv + 2];
  }
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int j = 1 + cw.j;
    const long long c = L.idx(1 + cw.i, j, kst<DIM>(1 + cw.k));
    const double Fxx_p = (hu[c + 1] - hu[c]) * idx, Fxx_m = (hu[c] - hu[c - 1]) * idx;
    const double Fyy_p = (hv[c + sy] - hv[c]) * idy, Fyy_m = (hv[c] - hv[c - sy]) * idy;
    const double Fxy_c = (hu[c + sy] - hu[c]) * idy + (hv[c + 1] - hv[c]) * idx;
    const double Fxy_jm = (hu[c] - hu[c - sy]) * idy + (hv[c + 1 - sy] - hv[c - sy]) * idx;
    const double Fxy_im = (hu[c - 1 + sy] - hu[c - 1]) * idy + (hv[c] - hv[c - 1]) * idx;
    double gu = Fxx_p * 0.5 * (U[c + 1] + U[c]) + Fxx_m * 0.5 * (U[c] + U[c - 1]) +
                Fxy_c * 0.25 * (V[c + 1] + V[c]) + Fxy_jm * 0.25 * (V[c + 1 - sy] + V[c - sy]);
    double gv = Fyy_p * 0.5 * (V[c + sy] + V[c]) + Fyy_m * 0.5 * (V[c] + V[c - sy]) +
                Fxy_c * 0.25 * (U[c + sy] + U[c]) + Fxy_im * 0.25 * (U[c - 1 + sy] + U[c - 1]);
    double lu = (hu[c + 1] - 2.0 * hu[c] + hu[c - 1]) * q.id2[0] + (hu[c + sy] - 2.0 * hu[c] + hu[c - sy]) * q.id2[1];
    double lv = (hv[c + 1] - 2.0 * hv[c] + hv[c - 1]) * q.id2[0] + (hv[c + sy] - 2.0 * hv[c] + hv[c - sy]) * q.id2[1];
    if (DIM == 3) {
      const double Fzz_p = (hw[c + sz] - hw[c]) * idz, Fzz_m = (hw[c] - hw[c - sz]) * idz;
      const double Fxz_c = (hu[c + sz] - hu[c]) * idz + (hw[c + 1] - hw[c]) * idx;
      const double Fxz_km = (hu[c] - hu[c - sz]) * idz + (hw[c + 1 - sz] - hw[c - sz]) * idx;
      const double Fxz_im = (hu[c - 1 + sz] - hu[c - 1]) * idz + (hw[c] - hw[c - 1]) * idx;
      const double Fyz_c = (hv[c + sz] - hv[c]) * idz + (hw[c + sy] - hw[c]) * idy;
      const double Fyz_km = (hv[c] - hv[c - sz]) * idz + (hw[c + sy - sz] - hw[c - sz]) * idy;
      const double Fyz_jm = (hv[c - sy + sz] - hv[c - sy]) * idz + (hw[c] - hw[c - sy]) * idy;
      gu += Fxz_c * 0.25 * (W[c + 1] + W[c]) + Fxz_km * 0.25 * (W[c + 1 - sz] + W[c - sz]);
      gv += Fyz_c * 0.25 * (W[c + sy] + W[c]) + Fyz_km * 0.25 * (W[c + sy - sz] + W[c - sz]);
      double gw = Fzz_p * 0.5 * (W[c + sz] + W[c]) + Fzz_m * 0.5 * (W[c] + W[c - sz]) +
                  Fxz_c * 0.25 * (U[c + sz] + U[c]) + Fxz_im * 0.25 * (U[c - 1 + sz] + U[c - 1]) +
                  Fyz_c * 0.25 * (V[c + sz] + V[c]) + Fyz_jm * 0.25 * (V[c - sy + sz] + V[c - sy]);
      lu += (hu[c + sz] - 2.0 * hu[c] + hu[c - sz]) * q.id2[2];
      lv += (hv[c + sz] - 2.0 * hv[c] + hv[c - sz]) * q.id2[2];
      double lw = (hw[c + 1] - 2.0 * hw[c] + hw[c - 1]) * q.id2[0] + (hw[c + sy] - 2.0 * hw[c] + hw[c - sy]) * q.id2[1] +
                  (hw[c + sz] - 2.0 * hw[c] + hw[c - sz]) * q.id2[2];
      double ow = ws[c] + gw + mur * lw;
      if (wall && j == 1) ow -= hw[c] * (idy * 0.25 * (V[c - sy] + V[c - sy + sz]) + mur * q.id2[1]);
      if (wall && j == L.n1) ow -= hw[c] * (-idy * 0.25 * (V[c] + V[c + sz]) + mur * q.id2[1]);
      wo[c] = ow;
    }
    double ou = us[c] + gu + mur * lu;
    if (wall && j == 1) ou -= hu[c] * (idy * 0.25 * (V[c - sy] + V[c - sy + 1]) + mur * q.id2[1]);
    if (wall && j == L.n1) ou -= hu[c] * (-idy * 0.25 * (V[c] + V[c + 1]) + mur * q.id2[1]);
    uo[c] = ou;
    vo[c] = (wall && j == L.n1) ? 0.0 : vs[c] + gv + mur * lv;
  }
}

}  // namespace fen
