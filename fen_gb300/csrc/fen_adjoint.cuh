// Discrete adjoint of the 2D periodic FP64 projection step.
//
// FEN has no differentiation; this is the exact transpose of the discrete step of
// navier_stokes_solver (navier_stokes.f90:50-136) for periodic 2D grids with constant
// density and viscosity.  Forward, with G the forward-difference gradient to faces, D the
// backward-difference divergence (G^T = -D on a periodic MAC grid), P the fast Poisson
// solve (symmetric: modified-wavenumber divide, zero mode and mean removed), N the
// divergence-form advection and L the 5-point Laplacian:
//   dv   = N(v) + mu/rhof L v            v*  = v + dt(-G p/rhof + A dv + B dv_o + g)
//   b    = rho/dt D v*                   phi = P b
//   v'   = v* - dt/rhof G phi            p'  = p + phi            dv_o' = dv
// Backward, given the adjoint (^) of (v', p', dv_o'):
//   phi^ = p'^ + dt/rhof D v'^           b^  = P phi^
//   v*^  = v'^ - rho/dt G b^             p^  = p'^ + dt/rhof D v*^
//   dv^  = dv_o'^ + dt A v*^             dv_o^ = dt B v*^
//   v^   = v*^ + N'(v)^T dv^ + mu/rhof L dv^
// Ghost cells hold periodic copies, so every gather below reads wrapped neighbours.
#pragma once
#include "fen_types.cuh"

namespace fen {

// out = a + s * D(x, y)  (fields.f90:144-145 transposed use)
__global__ void __launch_bounds__(256) k_adj_div2(Layout L, const double* __restrict__ a, const double* __restrict__ x,
                                                  const double* __restrict__ y, double s, double idx, double idy,
                                                  double* __restrict__ out) {
  const long long ncell = (long long)L.n0 * L.n1;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j;
    const long long c = L.idx(i, j, 0);
    const double d = (x[c] - x[c - 1]) * idx + (y[c] - y[c - L.sx]) * idy;
    out[c] = (a ? a[c] : 0.0) + s * d;
  }
}

// (uo, vo) = (u, v) - f * G(b)
__global__ void __launch_bounds__(256) k_adj_grad2(Layout L, const double* __restrict__ u, const double* __restrict__ v,
                                                   const double* __restrict__ b, double f, double idx, double idy,
                                                   double* __restrict__ uo, double* __restrict__ vo) {
  const long long ncell = (long long)L.n0 * L.n1;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j;
    const long long c = L.idx(i, j, 0);
    uo[c] = u[c] - f * (b[c + 1] - b[c]) * idx;
    vo[c] = v[c] - f * (b[c + L.sx] - b[c]) * idy;
  }
}

// dv^ = dv_o'^ + dtA v*^ (to dvh), dv_o^ = dtB v*^ (in place)
__global__ void __launch_bounds__(256) k_adj_dv2(Layout L, const double* __restrict__ us, const double* __restrict__ vs,
                                                 double* __restrict__ dou, double* __restrict__ dov, double dtA, double dtB,
                                                 double* __restrict__ dhu, double* __restrict__ dhv) {
  const long long ncell = (long long)L.n0 * L.n1;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j;
    const long long c = L.idx(i, j, 0);
    dhu[c] = dou[c] + dtA * us[c];
    dhv[c] = dov[c] + dtA * vs[c];
    dou[c] = dtB * us[c];
    dov[c] = dtB * vs[c];
  }
}

// v^ = v*^ + N'(v)^T dv^ + mu/rhof L dv^  (navier_stokes.f90:297-323, fields.f90:326-329)
__global__ void __launch_bounds__(256) k_adj_state2(Layout L, const double* __restrict__ u, const double* __restrict__ v,
                                                    const double* __restrict__ us, const double* __restrict__ vs,
                                                    const double* __restrict__ hu, const double* __restrict__ hv,
                                                    double idx, double idy, double id2x, double id2y, double mur,
                                                    double* __restrict__ uo, double* __restrict__ vo) {
  const long long ncell = (long long)L.n0 * L.n1;
  const long long sy = L.sx;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j;
    const long long c = L.idx(i, j, 0);
    // flux adjoints: F_u at i+1/2, i-1/2; F_v at j+1/2, j-1/2; C at (i,j), (i,j-1), (i-1,j)
    const double Fu_p = (hu[c + 1] - hu[c]) * idx, Fu_m = (hu[c] - hu[c - 1]) * idx;
    const double Fv_p = (hv[c + sy] - hv[c]) * idy, Fv_m = (hv[c] - hv[c - sy]) * idy;
    const double C_ij = (hu[c + sy] - hu[c]) * idy + (hv[c + 1] - hv[c]) * idx;
    const double C_ijm = (hu[c] - hu[c - sy]) * idy + (hv[c + 1 - sy] - hv[c - sy]) * idx;
    const double C_imj = (hu[c - 1 + sy] - hu[c - 1]) * idy + (hv[c] - hv[c - 1]) * idx;
    double gu = Fu_p * 0.5 * (u[c + 1] + u[c]) + Fu_m * 0.5 * (u[c] + u[c - 1]) +
                C_ij * 0.25 * (v[c + 1] + v[c]) + C_ijm * 0.25 * (v[c + 1 - sy] + v[c - sy]);
    double gv = Fv_p * 0.5 * (v[c + sy] + v[c]) + Fv_m * 0.5 * (v[c] + v[c - sy]) +
                C_ij * 0.25 * (u[c + sy] + u[c]) + C_imj * 0.25 * (u[c - 1 + sy] + u[c - 1]);
    const double lu = (hu[c + 1] - 2.0 * hu[c] + hu[c - 1]) * id2x + (hu[c + sy] - 2.0 * hu[c] + hu[c - sy]) * id2y;
    const double lv = (hv[c + 1] - 2.0 * hv[c] + hv[c - 1]) * id2x + (hv[c + sy] - 2.0 * hv[c] + hv[c - sy]) * id2y;
    uo[c] = us[c] + gu + mur * lu;
    vo[c] = vs[c] + gv + mur * lv;
  }
}

}  // namespace fen
