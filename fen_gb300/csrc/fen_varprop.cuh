// Variable-property momentum path of the FP64 step (FEN's multiphase / non-Newtonian branches
// of navier_stokes_solver, navier_stokes.f90:80-136, 140-213, 357-452, 505-566).
//
// Density rho and viscosity mu are cell-centred fields (navier_stokes.f90:36, 761-775)
// supplied by the caller (FEN's VoF or non-Newtonian modules update them between steps):
//   * face densities rhof = center_to_face(rho) (fields.f90:175-206) divide the pressure
//     gradient, the diffusion and the body force, and the correction;
//   * the Poisson right-hand side is div(v*) rho(i,j,k)/dt (navier_stokes.f90:115-121);
//   * with variable viscosity the diffusion is the stress divergence div(2 mu D)/rhof with
//     edge viscosities averaged over four cells (navier_stokes.f90:405-452; the reference
//     implements it in 2D only, so 3D contexts reject a viscosity field);
//   * the Dodd-Ferrante split (the MF branches, navier_stokes.f90:80-96, 174-184, 113,
//     526-531, 557): p_hat = p_o + (dt + dt_o)(p - p_o)/dt_o (constant CFL) or 2p - p_o,
//     RHS += grad p/rhof - grad p/rhomin - (1/rhof - 1/rhomin) grad p_hat, Poisson RHS
//     div(v*) rhomin/dt, correction dt grad(phi)/rhomin, and p_o = p before p += phi.
// Kernels follow the reference's operation order; one thread per cell.
#pragma once
#include "fen_types.cuh"

namespace fen {

struct VarArgs {
  const double *u, *v, *w, *p;
  double *us, *vs, *ws;
  double *dox, *doy, *doz;
  const double *Sx, *Sy, *Sz;
  const double* rho;  // cell density (null: constant `density`)
  const double* mu;   // cell viscosity (null: constant `viscosity`)
  const double* po;   // old pressure (split)
  double density, viscosity, g[3], id[3], id2[3];
  double irhomin;
  int iso, has_S, var_mu, split, constant_cfl;
};

__device__ __forceinline__ double rhof_q(const VarArgs& a, long long c, long long s) {
  return a.rho ? 0.5 * (a.rho[c + s] + a.rho[c]) : 0.5 * (a.density + a.density);
}

template <int DIM>
__global__ void __launch_bounds__(256) k_predictor_var(Layout L, const StepScalars* __restrict__ sc, VarArgs a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const double A = sc->A, B = sc->B, dt = sc->dt, dt_o = sc->dt_o;
  const double idx = a.id[0], idy = a.iso ? a.id[0] : a.id[1], idz = a.iso ? a.id[0] : a.id[2];
  const double id2x = a.id2[0], id2y = a.iso ? a.id2[0] : a.id2[1], id2z = a.iso ? a.id2[0] : a.id2[2];
  const long long sy = L.sx, sz = L.sp;
  const double* U = a.u;
  const double* V = a.v;
  const double* W = a.w;
  const double q = 0.25;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j, k = 1 + cw.k;
    const long long c = L.idx(i, j, kst<DIM>(k));
    const long long so[3] = {1, sy, sz};
    const double uc = U[c], vc = V[c];
    const double uip = U[c + 1], uim = U[c - 1], ujp = U[c + sy], ujm = U[c - sy];
    const double vip = V[c + 1], vim = V[c - 1], vjp = V[c + sy], vjm = V[c - sy];
    // add_advection (navier_stokes.f90:261-353)
    double dv[3] = {0.0, 0.0, 0.0};
    {
      const double uuip = q * ((uip + uc) * (uip + uc)), uuim = q * ((uim + uc) * (uim + uc));
      const double uvjp = (ujp + uc) * (vip + vc) * q, uvjm = (uc + ujm) * (V[c + 1 - sy] + vjm) * q;
      dv[0] = -((uuip - uuim) * idx) - (uvjp - uvjm) * idy;
      const double vuip = (vip + vc) * (ujp + uc) * q, vuim = (vc + vim) * (U[c - 1 + sy] + uim) * q;
      const double vvjp = q * ((vjp + vc) * (vjp + vc)), vvjm = q * ((vjm + vc) * (vjm + vc));
      dv[1] = -((vuip - vuim) * idx) - (vvjp - vvjm) * idy;
    }
    double wc = 0.0;
    if (DIM == 3) {
      wc = W[c];
      const double wip = W[c + 1], wim = W[c - 1], wjp = W[c + sy], wjm = W[c - sy], wkp = W[c + sz], wkm = W[c - sz];
      const double ukp = U[c + sz], ukm = U[c - sz], vkp = V[c + sz], vkm = V[c - sz];
      dv[0] = dv[0] - ((ukp + uc) * (wip + wc) * q - (uc + ukm) * (W[c + 1 - sz] + wkm) * q) * idz;
      dv[1] = dv[1] - ((vkp + vc) * (wjp + wc) * q - (vc + vkm) * (W[c + sy - sz] + wkm) * q) * idz;
      const double wuip = (wc + wip) * (uc + ukp) * q, wuim = (wc + wim) * (uim + U[c - 1 + sz]) * q;
      const double wvjp = (wc + wjp) * (vc + vkp) * q, wvjm = (wc + wjm) * (vjm + V[c - sy + sz]) * q;
      const double wwkp = (wc + wkp) * (wc + wkp) * q, wwkm = (wc + wkm) * (wc + wkm) * q;
      dv[2] = -((wuip - wuim) * idx) - (wvjp - wvjm) * idy - (wwkp - wwkm) * idz;
    }
    // add_diffusion (navier_stokes.f90:357-452)
    const double rfx = rhof_q(a, c, 1), rfy = rhof_q(a, c, sy), rfz = (DIM == 3) ? rhof_q(a, c, sz) : 1.0;
    if (!a.var_mu) {
      const double m = a.mu ? a.mu[c] : a.viscosity;  // mu%f(i,j,k) * lap(v) / rhof
      const double* F[3] = {U, V, W};
      for (int cq = 0; cq < DIM; ++cq) {
        const double* f = F[cq];
        const double two = 2.0 * f[c];
        double l;
        if (cq < 2) {
          if (a.iso) {
            l = ((f[c + 1] - two + f[c - 1]) + (f[c + sy] - two + f[c - sy])) * id2x;
            if (DIM == 3) l = l + (f[c + sz] - two + f[c - sz]) * id2x;
          } else {
            l = (f[c + 1] - two + f[c - 1]) * id2x + (f[c + sy] - two + f[c - sy]) * id2y;
            if (DIM == 3) l = l + (f[c + sz] - two + f[c - sz]) * id2z;
          }
        } else {  // the z component sums the three directions first (fields.f90:335-337)
          if (a.iso) l = ((f[c + 1] - two + f[c - 1]) + (f[c + sy] - two + f[c - sy]) + (f[c + sz] - two + f[c - sz])) * id2x;
          else l = (f[c + 1] - two + f[c - 1]) * id2x + (f[c + sy] - two + f[c - sy]) * id2y + (f[c + sz] - two + f[c - sz]) * id2z;
        }
        const double rf = (cq == 0) ? rfx : (cq == 1) ? rfy : rfz;
        dv[cq] = dv[cq] + m * l / rf;
      }
    } else {  // 2D stress divergence (navier_stokes.f90:419-447)
      const double* m = a.mu;
      const double id = idx;
      const long long ip = c + 1, im = c - 1, jp = c + sy, jm = c - sy;
      const double tauxxip = 2.0 * m[ip] * (U[ip] - U[c]) * id;
      const double tauxxim = 2.0 * m[c] * (U[c] - U[im]) * id;
      const double dtauxxdx = (tauxxip - tauxxim) * id;
      const double tauxyjp = 0.25 * (m[c] + m[ip] + m[jp] + m[ip + sy]) * ((U[jp] - U[c]) * id + (V[ip] - V[c]) * id);
      const double tauxyjm = 0.25 * (m[jm] + m[ip - sy] + m[c] + m[ip]) * ((U[c] - U[jm]) * id + (V[ip - sy] - V[jm]) * id);
      const double dtauxydy = (tauxyjp - tauxyjm) * id;
      dv[0] = dv[0] + (dtauxxdx + dtauxydy) / rfx;
      const double tauyxim = 0.25 * (m[im] + m[c] + m[im + sy] + m[jp]) * ((U[im + sy] - U[im]) * id + (V[c] - V[im]) * id);
      const double dtauyxdx = (tauxyjp - tauyxim) * id;
      const double tauyyjp = 2.0 * m[jp] * (V[jp] - V[c]) * id;
      const double tauyyjm = 2.0 * m[c] * (V[c] - V[jm]) * id;
      const double dtauyydy = (tauyyjp - tauyyjm) * id;
      dv[1] = dv[1] + (dtauyxdx + dtauyydy) / rfy;
    }
    const double rf[3] = {rfx, rfy, rfz};
    if (a.has_S) {
      const double* Sq[3] = {a.Sx, a.Sy, a.Sz};
      for (int cq = 0; cq < DIM; ++cq) dv[cq] = dv[cq] + Sq[cq][c] / rf[cq];
    }
    // predicted_velocity_field (navier_stokes.f90:160-198), with the split terms
    const double* P = a.p;
    double* out[3] = {a.us, a.vs, a.ws};
    double* dvo[3] = {a.dox, a.doy, a.doz};
    const double vel[3] = {uc, vc, wc};
    const double idq[3] = {idx, idy, idz};
    for (int cq = 0; cq < DIM; ++cq) {
      const long long s = so[cq];
      const double gp = (P[c + s] - P[c]) * idq[cq];
      double rhs = -gp / rf[cq] + A * dv[cq] + B * dvo[cq][c] + a.g[cq];
      if (a.split) {
        const double* po = a.po;
        const double ph0 = a.constant_cfl ? po[c] + (dt + dt_o) * (P[c] - po[c]) / dt_o : 2.0 * P[c] - po[c];
        const double ph1 = a.constant_cfl ? po[c + s] + (dt + dt_o) * (P[c + s] - po[c + s]) / dt_o : 2.0 * P[c + s] - po[c + s];
        const double gph = (ph1 - ph0) * idq[cq];
        rhs = rhs + gp / rf[cq] - a.irhomin * gp - (1.0 / rf[cq] - a.irhomin) * gph;
      }
      out[cq][c] = vel[cq] + dt * rhs;
      dvo[cq][c] = dv[cq];
    }
  }
}

// correct_velocity_field + update_pressure (navier_stokes.f90:505-566) with face densities
// or the split's 1/rhomin; p_o = p before p += phi under the split.
struct CorrVarArgs {
  const double *us, *vs, *ws, *phi;
  double *u, *v, *w, *p, *po;
  const double* rho;
  double density, irhomin, id[3];
  int iso, split;
};

template <int DIM>
__global__ void __launch_bounds__(256) k_correct_var(Layout L, const StepScalars* __restrict__ sc, CorrVarArgs a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const double dt = sc->dt;
  const double idx = a.id[0], idy = a.iso ? a.id[0] : a.id[1], idz = a.iso ? a.id[0] : a.id[2];
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j, k = 1 + cw.k;
    const long long c = L.idx(i, j, kst<DIM>(k));
    const long long so[3] = {1, L.sx, L.sp};
    const double idq[3] = {idx, idy, idz};
    const double* in[3] = {a.us, a.vs, a.ws};
    double* out[3] = {a.u, a.v, a.w};
    for (int q = 0; q < DIM; ++q) {
      const double gphi = (a.phi[c + so[q]] - a.phi[c]) * idq[q];
      if (a.split) {
        out[q][c] = in[q][c] - gphi * dt * a.irhomin;
      } else {
        const double rf = a.rho ? 0.5 * (a.rho[c + so[q]] + a.rho[c]) : 0.5 * (a.density + a.density);
        out[q][c] = in[q][c] - gphi * dt / rf;
      }
    }
    if (a.split) a.po[c] = a.p[c];
    a.p[c] = a.p[c] + a.phi[c];
  }
}

}  // namespace fen

namespace fen {

// IBM forcing hook (apply_ibm_forcing, navier_stokes.f90:106-108; eulerian_ibm.f90:194-268):
// after the predictor, each forced velocity point takes the target
//   vs = c0 + sum_k w_k v*(nbr_k)   (k < nn <= 8)
// (solid points: nn = 0 and c0 the solid velocity; interface points: the interpolation of
// the solid-boundary velocity and nearby fluid values), and the forcing Fe = (vs - v*)/dt
// is recorded.  All targets are evaluated from the unforced v* before any point is written.
struct IbmArgs {
  const long long* idx;   // forced point (layout index)
  const int* nn;          // stencil size
  const long long* nidx;  // [8 * point] neighbour layout indices
  const double* w;        // [8 * point] weights
  const double* c0;       // constant term
  double* vs;             // targets
  double* fe;             // forcing (vs - v*)/dt
  double* v;              // the velocity component v*
  int n;
};

__global__ void __launch_bounds__(256) k_ibm_target(IbmArgs a) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
    double s = a.c0[p];
    const int m = a.nn[p];
    for (int k = 0; k < m; ++k) s = s + a.w[8 * p + k] * a.v[a.nidx[8 * p + k]];
    a.vs[p] = s;
  }
}

__global__ void __launch_bounds__(256) k_ibm_apply(IbmArgs a, const StepScalars* __restrict__ sc) {
  const double dt = sc->dt;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
    const long long c = a.idx[p];
    a.fe[p] = (a.vs[p] - a.v[c]) / dt;
    a.v[c] = a.vs[p];
  }
}

}  // namespace fen
