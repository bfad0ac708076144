// Projection-step kernels (FEN src/navier_stokes.f90, src/fields.f90, src/poisson.f90).
#pragma once
#include "fen_fft.cuh"
#include "fen_ghost.cuh"
#include "fen_mixed.cuh"
#include "fen_types.cuh"

namespace fen {

// ------------------------------------------------------------------------------------
// Predictor: compute_explicit_terms + predicted_velocity_field fused
// (navier_stokes.f90:140-257, 261-353, 384-404; fields.f90:31-64, 175-206, 298-343).
// dv = -div(uu) + mu lap(v)/rhof + S/rhof;  v* = v + dt(-grad p/rhof + A dv + B dv_o + g);
// dv_o <- dv.  Operation order follows the reference; v* goes to separate buffers because
// the reference computes all of dv before updating v.
// ------------------------------------------------------------------------------------
template <typename T>
struct PredArgs {
  const T *u, *v, *w, *p;
  T *us, *vs, *ws;
  T *dox, *doy, *doz;
  const T *Sx, *Sy, *Sz;
  double id[3], id2[3];
  double mu, rhof, g[3];
  double dt_host;
  int iso, has_S, rhof_one, use_dev_dt;
};

// FP64 predictor: divergence-form advection (navier_stokes.f90:297-353), diffusion with
// constant mu (:384-404, fields.f90:326-337), body force (:245-255), pressure gradient
// (fields.f90:55-58) and the AB2 update with dv_o <- dv (:140-213); one thread per cell.
// FP64 issue is the bound on GB300, so the arithmetic is arranged to issue few FP64
// instructions: the edge products that two momentum equations of the same cell share
// (u v at (i+1/2, j+1/2), u w at (i+1/2, k+1/2), v w at (j+1/2, k+1/2)) are formed once,
// the factor 1/4 of every product is folded into the differencing scale, each Laplacian is
// the neighbour sum minus 2*DIM times the centre, and sums use fused multiply-adds.  The
// result differs from FEN's operation order by rounding only.
template <int DIM>
__global__ void __launch_bounds__(256) k_predictor(Layout L, const StepScalars* __restrict__ sc, PredArgs<double> a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const double A = sc->A, B = sc->B;
  const double dt = a.use_dev_dt ? sc->dt : a.dt_host;
  const double idx = a.id[0], idy = a.iso ? a.id[0] : a.id[1], idz = a.iso ? a.id[0] : a.id[2];
  const double qx = 0.25 * idx, qy = 0.25 * idy, qz = 0.25 * idz;
  const double irho = a.rhof_one ? 1.0 : 1.0 / a.rhof;
  // diffusion coefficients mu/rhof/delta^2 per axis (rhof = 1 keeps mu*id2 exactly)
  const double mx = a.rhof_one ? a.mu * a.id2[0] : a.mu * a.id2[0] / a.rhof;
  const double my = a.iso ? mx : (a.rhof_one ? a.mu * a.id2[1] : a.mu * a.id2[1] / a.rhof);
  const double mz = a.iso ? mx : (a.rhof_one ? a.mu * a.id2[2] : a.mu * a.id2[2] / a.rhof);
  const double gx = idx * irho, gy = idy * irho, gz = idz * irho;
  const double g0 = a.g[0], g1 = a.g[1], g2 = a.g[2];
  const long long sy = L.sx, sz = L.sp;
  const double* __restrict__ U = a.u;
  const double* __restrict__ V = a.v;
  const double* __restrict__ W = a.w;
  const double* __restrict__ P = a.p;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j, k = 1 + cw.k;
    const long long c = L.idx(i, j, kst<DIM>(k));
    const double uc = U[c], uip = U[c + 1], uim = U[c - 1], ujp = U[c + sy], ujm = U[c - sy];
    const double vc = V[c], vip = V[c + 1], vim = V[c - 1], vjp = V[c + sy], vjm = V[c - sy];
    const double su_p = uip + uc, su_m = uc + uim, sv_p = vjp + vc, sv_m = vc + vjm;
    const double uv_pp = (ujp + uc) * (vip + vc);               // (i+1/2, j+1/2)
    const double uv_pm = (uc + ujm) * (V[c + 1 - sy] + vjm);    // (i+1/2, j-1/2)
    const double uv_mp = (vc + vim) * (U[c - 1 + sy] + uim);    // (i-1/2, j+1/2)
    double ax = (su_p * su_p - su_m * su_m) * qx;
    ax = fma(uv_pp - uv_pm, qy, ax);
    double ay = (uv_pp - uv_mp) * qx;
    ay = fma(sv_p * sv_p - sv_m * sv_m, qy, ay);
    double lu = (uip + uim) + (ujp + ujm), lv = (vip + vim) + (vjp + vjm);
    double dvz = 0.0, wc = 0.0;
    double lux = 0.0, lvx = 0.0;
    if (DIM == 3) {
      wc = W[c];
      const double wip = W[c + 1], wim = W[c - 1], wjp = W[c + sy], wjm = W[c - sy], wkp = W[c + sz], wkm = W[c - sz];
      const double ukp = U[c + sz], ukm = U[c - sz], vkp = V[c + sz], vkm = V[c - sz];
      const double uw_pp = (ukp + uc) * (wip + wc);              // (i+1/2, k+1/2)
      const double uw_pm = (uc + ukm) * (W[c + 1 - sz] + wkm);   // (i+1/2, k-1/2)
      const double uw_mp = (wc + wim) * (uim + U[c - 1 + sz]);   // (i-1/2, k+1/2)
      const double vw_pp = (vkp + vc) * (wjp + wc);              // (j+1/2, k+1/2)
      const double vw_pm = (vc + vkm) * (W[c + sy - sz] + wkm);  // (j+1/2, k-1/2)
      const double vw_mp = (wc + wjm) * (vjm + V[c - sy + sz]);  // (j-1/2, k+1/2)
      const double sw_p = wc + wkp, sw_m = wc + wkm;
      ax = fma(uw_pp - uw_pm, qz, ax);
      ay = fma(vw_pp - vw_pm, qz, ay);
      double az = (uw_pp - uw_mp) * qx;
      az = fma(vw_pp - vw_mp, qy, az);
      az = fma(sw_p * sw_p - sw_m * sw_m, qz, az);
      double lw;
      if (a.iso) {
        lw = fma(-6.0, wc, ((wip + wim) + (wjp + wjm)) + (wkp + wkm));
        dvz = fma(mx, lw, -az);
      } else {
        dvz = fma(mx, fma(-2.0, wc, wip + wim), -az);
        dvz = fma(my, fma(-2.0, wc, wjp + wjm), dvz);
        dvz = fma(mz, fma(-2.0, wc, wkp + wkm), dvz);
      }
      lu = lu + (ukp + ukm);
      lv = lv + (vkp + vkm);
      lux = ukp + ukm;
      lvx = vkp + vkm;
    }
    double dvx, dvy;
    if (a.iso) {
      dvx = fma(mx, fma(-2.0 * DIM, uc, lu), -ax);
      dvy = fma(mx, fma(-2.0 * DIM, vc, lv), -ay);
    } else {
      dvx = fma(mx, fma(-2.0, uc, uip + uim), -ax);
      dvx = fma(my, fma(-2.0, uc, ujp + ujm), dvx);
      dvy = fma(mx, fma(-2.0, vc, vip + vim), -ay);
      dvy = fma(my, fma(-2.0, vc, vjp + vjm), dvy);
      if (DIM == 3) {
        dvx = fma(mz, fma(-2.0, uc, lux), dvx);
        dvy = fma(mz, fma(-2.0, vc, lvx), dvy);
      }
    }
    if (a.has_S) {
      dvx = fma(a.Sx[c], irho, dvx);
      dvy = fma(a.Sy[c], irho, dvy);
      if (DIM == 3) dvz = fma(a.Sz[c], irho, dvz);
    }
    const double pc = P[c];
    double rx = fma(-gx, P[c + 1] - pc, g0);
    double ry = fma(-gy, P[c + sy] - pc, g1);
    rx = fma(A, dvx, fma(B, a.dox[c], rx));
    ry = fma(A, dvy, fma(B, a.doy[c], ry));
    a.us[c] = fma(dt, rx, uc);
    a.vs[c] = fma(dt, ry, vc);
    a.dox[c] = dvx;
    a.doy[c] = dvy;
    if (DIM == 3) {
      double rz = fma(-gz, P[c + sz] - pc, g2);
      rz = fma(A, dvz, fma(B, a.doz[c], rz));
      a.ws[c] = fma(dt, rz, wc);
      a.doz[c] = dvz;
    }
  }
}

// 3D FP64 predictor with flux sharing between cells.  The six products a cell owns on its
// + faces/edges (1/4 folded into the scale q),
//   Fuu = (u(i+1) + u)^2, Fvv = (v(j+1) + v)^2, Fww = (w(k+1) + w)^2,
//   Euv = (u(j+1) + u)(v(i+1) + v), Euw = (u(k+1) + u)(w(i+1) + w), Evw = (v(k+1) + v)(w(j+1) + w),
// are formed once: the - face values come from the x neighbour lane (warp shuffle), the
// y neighbour row (shared memory) and the previous k of the z walk (registers); halo lanes,
// rows and the first k compute theirs directly (FP64 issue counts active lanes only).  The
// discrete operator is FEN's (navier_stokes.f90:297-353); diffusion and AB2 as k_predictor.
constexpr int kTX = 32, kTY = 8, kTZ = 16;

__device__ __forceinline__ void flux6(const double* __restrict__ U, const double* __restrict__ V,
                                      const double* __restrict__ W, long long c, long long sy, long long sz, double& fuu,
                                      double& fvv, double& fww, double& euv, double& euw, double& evw) {
  const double uc = U[c], vc = V[c], wc = W[c];
  const double su = U[c + 1] + uc, sv = V[c + sy] + vc, sw = W[c + sz] + wc;
  fuu = su * su;
  fvv = sv * sv;
  fww = sw * sw;
  euv = (U[c + sy] + uc) * (V[c + 1] + vc);
  euw = (U[c + sz] + uc) * (W[c + 1] + wc);
  evw = (V[c + sz] + vc) * (W[c + sy] + wc);
}

// The three + fluxes of cell c that the x, y or z neighbour needs as its - fluxes.
__device__ __forceinline__ void flux_x(const double* __restrict__ U, const double* __restrict__ V,
                                       const double* __restrict__ W, long long c, long long sy, long long sz, double& fuu,
                                       double& euv, double& euw) {
  const double uc = U[c], su = U[c + 1] + uc;
  fuu = su * su;
  euv = (U[c + sy] + uc) * (V[c + 1] + V[c]);
  euw = (U[c + sz] + uc) * (W[c + 1] + W[c]);
}
__device__ __forceinline__ void flux_y(const double* __restrict__ U, const double* __restrict__ V,
                                       const double* __restrict__ W, long long c, long long sy, long long sz, double& euv,
                                       double& fvv, double& evw) {
  const double vc = V[c], sv = V[c + sy] + vc;
  fvv = sv * sv;
  euv = (U[c + sy] + U[c]) * (V[c + 1] + vc);
  evw = (V[c + sz] + vc) * (W[c + sy] + W[c]);
}
__device__ __forceinline__ void flux_z(const double* __restrict__ U, const double* __restrict__ V,
                                       const double* __restrict__ W, long long c, long long sy, long long sz, double& euw,
                                       double& evw, double& fww) {
  const double wc = W[c], sw = W[c + sz] + wc;
  fww = sw * sw;
  euw = (U[c + sz] + U[c]) * (W[c + 1] + wc);
  evw = (V[c + sz] + V[c]) * (W[c + sy] + wc);
}

static __global__ void __launch_bounds__(kTX * kTY) k_predictor_tile(Layout L, const StepScalars* __restrict__ sc,
                                                              PredArgs<double> a) {
  __shared__ double sh[2][3][kTY][kTX];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = 1 + blockIdx.x * kTX + tx, j0 = 1 + blockIdx.y * kTY + ty;
  const bool act = (i0 <= L.n0) && (j0 <= L.n1);
  const int i = min(i0, L.n0), j = min(j0, L.n1);
  const int k0 = 1 + blockIdx.z * kTZ, k1 = min(L.n2, k0 + kTZ - 1);
  const double A = sc->A, B = sc->B;
  const double dt = a.use_dev_dt ? sc->dt : a.dt_host;
  const double idx = a.id[0], idy = a.iso ? a.id[0] : a.id[1], idz = a.iso ? a.id[0] : a.id[2];
  const double qx = 0.25 * idx, qy = 0.25 * idy, qz = 0.25 * idz;
  const double irho = a.rhof_one ? 1.0 : 1.0 / a.rhof;
  const double mx = a.rhof_one ? a.mu * a.id2[0] : a.mu * a.id2[0] / a.rhof;
  const double my = a.iso ? mx : (a.rhof_one ? a.mu * a.id2[1] : a.mu * a.id2[1] / a.rhof);
  const double mz = a.iso ? mx : (a.rhof_one ? a.mu * a.id2[2] : a.mu * a.id2[2] / a.rhof);
  const double gx = idx * irho, gy = idy * irho, gz = idz * irho;
  const long long sy = L.sx, sz = L.sp;
  const double* __restrict__ U = a.u;
  const double* __restrict__ V = a.v;
  const double* __restrict__ W = a.w;
  const double* __restrict__ P = a.p;
  // z-minus fluxes of the first k of the chunk
  double pww, puw, pvw;
  flux_z(U, V, W, L.idx(i, j, k0) - sz, sy, sz, puw, pvw, pww);
  int buf = 0;
  for (int k = k0; k <= k1; ++k, buf ^= 1) {
    const long long c = L.idx(i, j, k);
    double fuu, fvv, fww, euv, euw, evw;
    flux6(U, V, W, c, sy, sz, fuu, fvv, fww, euv, euw, evw);
    // x-minus: the lane to the left; lane 0 computes its own
    double xuu = __shfl_up_sync(0xffffffffu, fuu, 1);
    double xuv = __shfl_up_sync(0xffffffffu, euv, 1);
    double xuw = __shfl_up_sync(0xffffffffu, euw, 1);
    if (tx == 0) flux_x(U, V, W, c - 1, sy, sz, xuu, xuv, xuw);
    // y-minus: the row below through shared memory; row 0 computes its own
    sh[buf][0][ty][tx] = euv;
    sh[buf][1][ty][tx] = fvv;
    sh[buf][2][ty][tx] = evw;
    __syncthreads();
    double yuv, yvv, yvw;
    if (ty > 0) {
      yuv = sh[buf][0][ty - 1][tx];
      yvv = sh[buf][1][ty - 1][tx];
      yvw = sh[buf][2][ty - 1][tx];
    } else {
      flux_y(U, V, W, c - sy, sy, sz, yuv, yvv, yvw);
    }
    const double ax = fma(euw - puw, qz, fma(euv - yuv, qy, (fuu - xuu) * qx));
    const double ay = fma(evw - pvw, qz, fma(fvv - yvv, qy, (euv - xuv) * qx));
    const double az = fma(fww - pww, qz, fma(evw - yvw, qy, (euw - xuw) * qx));
    pww = fww;
    puw = euw;
    pvw = evw;
    if (act) {
      const double uc = U[c], vc = V[c], wc = W[c];
      const double uip = U[c + 1], uim = U[c - 1], ujp = U[c + sy], ujm = U[c - sy], ukp = U[c + sz], ukm = U[c - sz];
      const double vip = V[c + 1], vim = V[c - 1], vjp = V[c + sy], vjm = V[c - sy], vkp = V[c + sz], vkm = V[c - sz];
      const double wip = W[c + 1], wim = W[c - 1], wjp = W[c + sy], wjm = W[c - sy], wkp = W[c + sz], wkm = W[c - sz];
      double dvx, dvy, dvz;
      if (a.iso) {
        dvx = fma(mx, fma(-6.0, uc, ((uip + uim) + (ujp + ujm)) + (ukp + ukm)), -ax);
        dvy = fma(mx, fma(-6.0, vc, ((vip + vim) + (vjp + vjm)) + (vkp + vkm)), -ay);
        dvz = fma(mx, fma(-6.0, wc, ((wip + wim) + (wjp + wjm)) + (wkp + wkm)), -az);
      } else {
        dvx = fma(mz, fma(-2.0, uc, ukp + ukm), fma(my, fma(-2.0, uc, ujp + ujm), fma(mx, fma(-2.0, uc, uip + uim), -ax)));
        dvy = fma(mz, fma(-2.0, vc, vkp + vkm), fma(my, fma(-2.0, vc, vjp + vjm), fma(mx, fma(-2.0, vc, vip + vim), -ay)));
        dvz = fma(mz, fma(-2.0, wc, wkp + wkm), fma(my, fma(-2.0, wc, wjp + wjm), fma(mx, fma(-2.0, wc, wip + wim), -az)));
      }
      if (a.has_S) {
        dvx = fma(a.Sx[c], irho, dvx);
        dvy = fma(a.Sy[c], irho, dvy);
        dvz = fma(a.Sz[c], irho, dvz);
      }
      const double pc = P[c];
      double rx = fma(-gx, P[c + 1] - pc, a.g[0]);
      double ry = fma(-gy, P[c + sy] - pc, a.g[1]);
      double rz = fma(-gz, P[c + sz] - pc, a.g[2]);
      rx = fma(A, dvx, fma(B, a.dox[c], rx));
      ry = fma(A, dvy, fma(B, a.doy[c], ry));
      rz = fma(A, dvz, fma(B, a.doz[c], rz));
      a.us[c] = fma(dt, rx, uc);
      a.vs[c] = fma(dt, ry, vc);
      a.ws[c] = fma(dt, rz, wc);
      a.dox[c] = dvx;
      a.doy[c] = dvy;
      a.doz[c] = dvz;
    }
  }
}

// ------------------------------------------------------------------------------------
// Line transforms.  One kernel template covers every 1D stage of every solver:
//   CONTIG = true : lines along x (contiguous), the first and last stages;
//   CONTIG = false: lines along y or z (strided), a tile of consecutive columns per CTA.
// ------------------------------------------------------------------------------------
enum { OP_R2C = 0, OP_C2R, OP_C2C_F, OP_C2C_I, OP_C2C_SOLVE, OP_DCT2, OP_DCT3 };
enum { LD_FIELD = 0, LD_DIV, LD_REAL, LD_CPLX, LD_DIVMIX, LD_RESID };
enum { ST_FIELD = 0, ST_REAL, ST_CPLX };

template <typename T>
struct LineArgs {
  // geometry of the lines handled by this launch
  int n;                  // real length (R2C/C2R/DCT) or complex length (C2C) along the axis
  int nl;                 // lines per CTA
  int nlines;             // lines per outer index (columns for strided, rows for contiguous)
  // spectral input / output (element strides in units of their own type)
  const void* in;
  void* out;
  long long in_line, in_pos, in_outer;     // address = line*in_line + pos*in_pos + outer*in_outer
  long long out_line, out_pos, out_outer;
  // fields (LD_FIELD / LD_DIV / ST_FIELD)
  Layout L;
  const T *fu, *fv, *fw;  // predicted velocity for LD_DIV
  const float *ful, *fvl, *fwl;  // LD_DIVMIX: optional second pair added to pu, pv, pw
  const double* rho_c;           // LD_DIV with variable density: div * rho(i,j,k) * rho_over_dt (= 1/dt)
  DFField pu, pv, pw;     // pair v* of the mixed form (LD_DIVMIX)
  F2 idp[3];              // 1/delta per axis as float pairs (LD_DIVMIX, LD_RESID)
  F2 id2p[3];             // 1/delta^2 per axis as float pairs (LD_RESID)
  float *dvh, *dvl;       // pair divergence D v*: written by LD_DIVMIX when set, read by LD_RESID
  const T* fsrc;          // LD_FIELD source
  T* fdst;                // ST_FIELD destination
  double* partial;        // ST_FIELD: per-CTA line sums (mean removal), may be null
  double scale;
  float scale32;          // FP32 kernels: scale rounded on the host, and whether it is not 1
  int scaled;
  const StepScalars* sc;  // LD_DIV scaling rho/dt
  double id[3];
  int iso, dim;
  // OP_C2C_SOLVE eigenvalues: lam = lamA[col] + lamB[outer] + lamC[pos]
  const double* lamA; const double* lamB; const double* lamC;
  // optional tabulated scale/lam for OP_C2C_SOLVE, [(outer * n + pos) * nlines + col]
  const T* inv_lam;
  FFTPlan plan;
  // fast-division multipliers (fft_magic) of n, M, M + 1 and nl, computed on the host: an
  // integer division in the kernel runs through conversion instructions, which GB300 issues
  // on its FP64 pipe (every launcher sets them)
  unsigned mg[4];
  AxisTw tw;
};

// Global offset of (line, outer) of a contiguous launch: lines are x-rows j = 1..n1 of
// plane k = outer + 1; returns the Fortran (j, k).
template <int DIM>
__device__ __forceinline__ void row_jk(int line, int outer, int& j, int& k) { j = line + 1; k = outer + 1; }

template <typename T, int DIM>
__device__ __forceinline__ T div_at(const LineArgs<T>& a, int i, int j, int k) {
  // (u_i - u_{i-1}) / dx + (v_j - v_{j-1}) / dy + (w_k - w_{k-1}) / dz in FEN's operation
  // order (the Poisson right-hand side sets the pressure's rounding level)
  const Layout& L = a.L;
  const long long c = L.idx(i, j, kst<DIM>(k));
  const T* U = a.fu; const T* V = a.fv; const T* W = a.fw;
  T d;
  if (a.iso) {
    const T id = (T)a.id[0];
    d = (U[c] - U[c - 1]) * id + (V[c] - V[c - L.sx]) * id;
    if (DIM == 3) d = d + (W[c] - W[c - L.sp]) * id;
  } else {
    d = (U[c] - U[c - 1]) * (T)a.id[0] + (V[c] - V[c - L.sx]) * (T)a.id[1];
    if (DIM == 3) d = d + (W[c] - W[c - L.sp]) * (T)a.id[2];
  }
  return d;
}

// Elements loaded per thread before the first of them is stored to shared memory in the
// FP32 spectral loaders (memory-level parallelism of the load phase).
#ifndef FEN_LINE_LB
#define FEN_LINE_LB 4
#endif
constexpr int kLB = FEN_LINE_LB;
// Elements per thread of the batched FP32 r2c pair loaders (LD_DIVMIX, LD_RESID); 1: the
// element-at-a-time loop.
#ifndef FEN_R2C_LB
#define FEN_R2C_LB 2
#endif
constexpr int kLR = FEN_R2C_LB;
// ... of the pair-divergence loader (LD_DIVMIX): 3 (mixed channel forward x 0.514 -> 0.487
// ms; 3 in the residual loader spills and slows it, 4 in either spills more)
#ifndef FEN_R2C_LB_DIV
#define FEN_R2C_LB_DIV 3
#endif
constexpr int kLRD = FEN_R2C_LB_DIV;
// Strided (column) transforms: element addresses advanced by a constant stride per thread
// instead of divided out per element (needs nl | threads, true for the column tiles).
#ifndef FEN_STRIDED_IDX
#define FEN_STRIDED_IDX 1
#endif
constexpr bool kStridedIdx = FEN_STRIDED_IDX != 0;

template <typename T, int DIM, bool CONTIG, int OP, int LD, int ST>
__device__ __forceinline__ void line_body(const LineArgs<T>& a) {
  typedef typename cpx<T>::t T2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = a.n;
  const bool real_fft = (OP == OP_R2C || OP == OP_C2R || OP == OP_DCT2 || OP == OP_DCT3);
  const int M = real_fft ? n / 2 : n;
  const int nl = a.nl;
  T2* bufA = reinterpret_cast<T2*>(smem_raw);
  T2* bufB = bufA + (size_t)nl * M;
  const int line0 = blockIdx.x * nl;
  const int outer = blockIdx.y;
  const int nlv = min(nl, a.nlines - line0);  // valid lines in this CTA
  const int tid = threadIdx.x, nth = blockDim.x;
  // element -> (line, position) splits by multiply-high division with the host's multipliers
  // (a division here, even once per thread, compiles to conversions on the FP64 pipe)
  const FastDiv fN{(unsigned)n, a.mg[0]}, fM{(unsigned)M, a.mg[1]};
  const FastDiv fM1{(unsigned)(M + 1), a.mg[2]}, fL{(unsigned)nl, a.mg[3]};
  const int nth_l = fdivi(nth, fL);            // threads per line of the strided branches
  const bool nl_divides = nth_l * nl == nth;   // nl | threads
  // position-major smem: element (l, p) at p*nl + l
  auto S = [&](int l, int p) -> T2& { return bufA[(size_t)p * nl + l]; };
  T* Sr = reinterpret_cast<T*>(bufA);  // real view: real slot r of line l at (r/2 * nl + l)*2 + (r&1)
  auto RS = [&](int l, int r) -> T& { return Sr[((size_t)(r >> 1) * nl + l) * 2 + (r & 1)]; };

  const T* inR = reinterpret_cast<const T*>(a.in);
  const T2* inC = reinterpret_cast<const T2*>(a.in);
  // x lines: field index of (i + 1, row line0 + l) is rowbase + l*sx + i (the CTA's rows are
  // consecutive rows of one plane), formed without a per-element 64-bit index product
  long long rowbase = 0;
  if (CONTIG) {
    int j0, k0;
    row_jk<DIM>(line0, outer, j0, k0);
    rowbase = a.L.idx(1, j0, kst<DIM>(k0));
  }
  auto rc = [&](int l, int i) -> long long { return a.L.at(rowbase + (long long)(l * a.L.sx + i)); };
  // spectrum offsets of line l: x lines in 32-bit arithmetic from the CTA's base (a few rows
  // of one plane), strided lines in 64-bit
  const long long ibase = CONTIG ? (long long)line0 * a.in_line + (long long)outer * a.in_outer : 0;
  const long long obase = CONTIG ? (long long)line0 * a.out_line + (long long)outer * a.out_outer : 0;
  auto irow = [&](int l) -> long long {
    return CONTIG ? ibase + (long long)(l * (int)a.in_line) : (long long)(line0 + l) * a.in_line + (long long)outer * a.in_outer;
  };
  auto orow = [&](int l) -> long long {
    return CONTIG ? obase + (long long)(l * (int)a.out_line) : (long long)(line0 + l) * a.out_line + (long long)outer * a.out_outer;
  };
  auto ipos = [&](int p) -> long long { return CONTIG ? (long long)(p * (int)a.in_pos) : (long long)p * a.in_pos; };
  auto opos = [&](int p) -> long long { return CONTIG ? (long long)(p * (int)a.out_pos) : (long long)p * a.out_pos; };

  // ---------------- load ----------------
  if (OP == OP_R2C && CONTIG && sizeof(T) == 4 && (LD == LD_DIVMIX ? kLRD : kLR) > 1 &&
      (LD == LD_DIVMIX || LD == LD_RESID)) {
    constexpr int kB = (LD == LD_DIVMIX) ? kLRD : kLR;
    // FP32 r2c of the mixed form's pair loaders: kB elements per thread evaluated before any
    // store (their loads in flight together; the pair-divergence stores for the refinement
    // follow in the second pass so they cannot order the loads)
    const int work = nl * n;
    F2 rod{0.f, 0.f};
    if (LD == LD_RESID) rod = F2{a.sc->rdtp[0], a.sc->rdtp[1]};  // rho/dt as the prologue's pair
    const T rdt = (LD == LD_DIVMIX) ? (T)a.sc->rdtp[0] : T(0);
    const float* ph = (const float*)a.fsrc;
    for (int t0 = tid; t0 < work; t0 += nth * kB) {
      F2 v[kB];
#pragma unroll
      for (int b = 0; b < kB; ++b) {
        const int t = t0 + b * nth;
        v[b] = F2{0.f, 0.f};
        int l = 0, i = 0;
        if (t < work) divmod(t, fN, l, i);
        if (t < work && l < nlv) {
          const long long c = rc(l, i);
          if (LD == LD_DIVMIX) {
            v[b] = div_df_at<DIM>(a.L, a.pu, a.pv, a.pw, (const float*)a.fu, (const float*)a.fv, (const float*)a.fw,
                                  a.ful, a.fvl, a.fwl, a.idp, c);
          } else {
            // refinement right-hand side r = rho/dt D v* - L_h phi in double-float
            const F2 bb = mul_pair(a.dvh[c], a.dvl[c], rod);
            F2 lap = add_pair(lap_term(ph, c, 1, a.id2p[0]), lap_term(ph, c, a.L.sx, a.id2p[1]));
            if (DIM == 3) lap = add_pair(lap, lap_term(ph, c, a.L.sp, a.id2p[2]));
            float s, e;
            two_sum(bb.hi, -lap.hi, s, e);
            v[b] = F2{s, e + (bb.lo - lap.lo)};
          }
        }
      }
#pragma unroll
      for (int b = 0; b < kB; ++b) {
        const int t = t0 + b * nth;
        if (t < work) {
          int l, i;
          divmod(t, fN, l, i);
          T x = 0;
          if (l < nlv) {
            if (LD == LD_DIVMIX) {
              if (a.dvh) {  // kept for the refinement's residual
                const long long c = rc(l, i);
                a.dvh[c] = v[b].hi;
                a.dvl[c] = v[b].lo;
              }
              x = (T)(v[b].hi + v[b].lo) * rdt;
            } else {
              x = (T)(v[b].hi + v[b].lo);
            }
          }
          RS(l, i) = x;
        }
      }
    }
  } else if (OP == OP_R2C || OP == OP_DCT2) {
    // n reals per line -> packed complex (DCT2 reorders first: v_m = x_2m, v_{n-1-m} = x_2m+1)
    const int work = nl * n;
    F2 rod{0.f, 0.f};
    if (LD == LD_RESID) rod = F2{a.sc->rdtp[0], a.sc->rdtp[1]};
    // rho/dt read once (FP32 kernels: the prologue's FP32 rounding of it, so no conversion
    // is issued here): the field stores below may alias sc as far as the compiler knows
    T rdt = T(0);
    if (LD == LD_DIV || LD == LD_DIVMIX) {
      if constexpr (sizeof(T) == 4) rdt = a.sc->rdtp[0];
      else rdt = (T)a.sc->rho_over_dt;
    }
    for (int t = tid; t < work; t += nth) {
      int l, i;
      if (CONTIG) divmod(t, fN, l, i); else divmod(t, fL, i, l);
      T x = 0;
      if (l < nlv) {
        if (LD == LD_FIELD || LD == LD_DIV || LD == LD_DIVMIX || LD == LD_RESID) {
          int j, k;
          row_jk<DIM>(line0 + l, outer, j, k);
          if (LD == LD_FIELD) x = a.fsrc[a.L.idx(i + 1, j, kst<DIM>(k))];
          else if (LD == LD_DIV) {
            x = div_at<T, DIM>(a, i + 1, j, k);
            if (a.rho_c) x = x * (T)a.rho_c[a.L.idx(i + 1, j, kst<DIM>(k))];
            x = x * rdt;
          }
          else if (LD == LD_DIVMIX) {
            const F2 dd = div_df<DIM>(a.L, a.pu, a.pv, a.pw, (const float*)a.fu, (const float*)a.fv, (const float*)a.fw,
                                      a.ful, a.fvl, a.fwl,
                                      a.idp, i + 1, j, k);
            if (a.dvh) {  // kept for the refinement's residual
              const long long c = a.L.idx(i + 1, j, kst<DIM>(k));
              a.dvh[c] = dd.hi;
              a.dvl[c] = dd.lo;
            }
            x = (T)(dd.hi + dd.lo) * rdt;
          } else {
            // refinement right-hand side r = rho/dt D v* - L_h phi in double-float (phi = fsrc;
            // D v* as formed by this step's first transform)
            const long long c = a.L.idx(i + 1, j, kst<DIM>(k));
            const F2 b = mul_pair(a.dvh[c], a.dvl[c], rod);
            const float* ph = (const float*)a.fsrc;
            F2 lap = add_pair(lap_term(ph, c, 1, a.id2p[0]), lap_term(ph, c, a.L.sx, a.id2p[1]));
            if (DIM == 3) lap = add_pair(lap, lap_term(ph, c, a.L.sp, a.id2p[2]));
            float s, e;
            two_sum(b.hi, -lap.hi, s, e);
            x = (T)(s + (e + (b.lo - lap.lo)));
          }
        } else {
          x = inR[(long long)(line0 + l) * a.in_line + (long long)i * a.in_pos + (long long)outer * a.in_outer];
        }
      }
      int r = i;
      if (OP == OP_DCT2) r = (i & 1) ? (n - 1 - (i >> 1)) : (i >> 1);
      RS(l, r) = x;
    }
  } else if (OP == OP_C2R && sizeof(T) == 4) {
    // FP32 c2r: the same pre-processing with kLB elements (2 kLB loads) in flight per thread,
    // all loads of a batch issued before the first use (the kernel is bound by load latency)
    const int work = nl * M;
    for (int t0 = tid; t0 < work; t0 += nth * kLB) {
      T2 xk[kLB], xm[kLB];
#pragma unroll
      for (int b = 0; b < kLB; ++b) {
        const int t = t0 + b * nth;
        int l = 0, kk = 0;
        if (t < work) {
          if (CONTIG) divmod(t, fM, l, kk); else divmod(t, fL, kk, l);
        }
        if (t < work && l < nlv) {
          const long long base = irow(l);
          xk[b] = inC[base + ipos(kk)];
          xm[b] = inC[base + ipos(M - kk)];
        } else {
          xk[b] = mk<T2>(0, 0);
          xm[b] = xk[b];
        }
      }
#pragma unroll
      for (int b = 0; b < kLB; ++b) {
        const int t = t0 + b * nth;
        if (t < work) {
          int l, kk;
          if (CONTIG) divmod(t, fM, l, kk); else divmod(t, fL, kk, l);
          S(l, kk) = (l < nlv) ? c2r_pre(xk[b], xm[b], M, kk, a.tw.wN) : mk<T2>(0, 0);
        }
      }
    }
  } else if (OP == OP_C2R || OP == OP_DCT3) {
    // Hermitian half-spectrum X_0..X_M -> c2r pre-processed Z'_0..Z'_{M-1}
    const int work = nl * M;
    for (int t = tid; t < work; t += nth) {
      int l, kk;
      if (CONTIG) divmod(t, fM, l, kk); else divmod(t, fL, kk, l);
      T2 z = mk<T2>(0, 0);
      if (l < nlv) {
        const long long base = irow(l);
        T2 xk, xm;
        if (OP == OP_C2R) {
          xk = inC[base + ipos(kk)];
          xm = inC[base + ipos(M - kk)];
        } else {
          // V_k = (Y_k - i Y_{n-k}) exp(+i pi k / 2n), Y_n = 0  (Makhoul's DCT-III)
          auto Vk = [&](int q) -> T2 {
            const T yk = inR[base + (long long)q * a.in_pos];
            const T yr = (q == 0) ? T(0) : inR[base + (long long)(n - q) * a.in_pos];
            return cmulc(mk<T2>(yk, -yr), ldtw<T2>(a.tw.wD, q));
          };
          xk = Vk(kk);
          xm = Vk(M - kk);
        }
        z = c2r_pre(xk, xm, M, kk, a.tw.wN);
      }
      S(l, kk) = z;
    }
  } else if (kStridedIdx && !CONTIG && nl_divides) {
    // complex in, strided lines with nl dividing the thread count: every element a thread
    // loads belongs to the same line l = tid % nl, at positions p0, p0 + dp, ... (dp = nth / nl),
    // so the address advances by a constant stride (no per-element division or multiply)
    constexpr int B = (sizeof(T) == 4) ? kLB : 1;
    int l, p0;
    divmod(tid, fL, p0, l);
    const int dp = nth_l;
    const bool lok = l < nlv;
    const T2* src = inC + (long long)(line0 + (lok ? l : 0)) * a.in_line + (long long)outer * a.in_outer +
                    (long long)p0 * a.in_pos;
    const long long step = (long long)dp * a.in_pos;
    for (int p1 = p0; p1 < M; p1 += dp * B, src += step * B) {
      T2 zb[B];
#pragma unroll
      for (int b = 0; b < B; ++b) zb[b] = (p1 + b * dp < M && lok) ? src[step * b] : mk<T2>(0, 0);
#pragma unroll
      for (int b = 0; b < B; ++b)
        if (p1 + b * dp < M) S(l, p1 + b * dp) = zb[b];
    }
  } else {  // complex in: kLB loads in flight per thread (FP32; one in the FP64 kernels)
    const int work = nl * M;
    constexpr int B = (sizeof(T) == 4) ? kLB : 1;
    for (int t0 = tid; t0 < work; t0 += nth * B) {
      T2 zb[B];
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int t = t0 + b * nth;
        int l = 0, p = 0;
        if (t < work) {
          if (CONTIG) divmod(t, fM, l, p); else divmod(t, fL, p, l);
        }
        zb[b] = (t < work && l < nlv)
                    ? inC[(long long)(line0 + l) * a.in_line + (long long)p * a.in_pos + (long long)outer * a.in_outer]
                    : mk<T2>(0, 0);
      }
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int t = t0 + b * nth;
        if (t < work) {
          int l, p;
          if (CONTIG) divmod(t, fM, l, p); else divmod(t, fL, p, l);
          S(l, p) = zb[b];
        }
      }
    }
  }
  __syncthreads();

  // ---------------- transform ----------------
  T2* res;
  if (OP == OP_R2C || OP == OP_DCT2 || OP == OP_C2C_F || OP == OP_C2C_SOLVE)
    res = smem_fft<-1, fft_max_radix<T, CONTIG>()>(bufA, bufB, fL, 1, nl, a.plan, a.tw.wM);
  else
    res = smem_fft<+1, fft_max_radix<T, CONTIG>()>(bufA, bufB, fL, 1, nl, a.plan, a.tw.wM);

  if (OP == OP_C2C_SOLVE) {
    // normalise and divide by the eigenvalue sum, zero mode -> 0 (poisson.f90:458-471, 991-1005)
    const int work = nl * M;
    for (int t = tid; t < work; t += nth) {
      int l, p;
      divmod(t, fL, p, l);
      if (l < nlv) {
        T2& z = res[(size_t)p * nl + l];
        if (a.inv_lam) {
          const T f = a.inv_lam[((long long)outer * M + p) * a.nlines + line0 + l];
          z = mk<T2>(z.x * f, z.y * f);
        } else {
          const double lam = a.lamA[line0 + l] + (a.lamB ? a.lamB[outer] : 0.0) + a.lamC[p];
          if (lam == 0.0) z = mk<T2>(0, 0);
          else {
            const T f = (T)(a.scale / lam);
            z = mk<T2>(z.x * f, z.y * f);
          }
        }
      }
    }
    __syncthreads();
    T2* other = (res == bufA) ? bufB : bufA;
    res = smem_fft<+1, fft_max_radix<T, CONTIG>()>(res, other, fL, 1, nl, a.plan, a.tw.wM);
  }

  // ---------------- store ----------------
  // FP32 kernels take the scale as rounded on the host: a conversion or FP64 compare here
  // would be re-issued per element on the FP64 pipe wherever the compiler rematerialises it
  T scale;
  bool do_scale;
  if constexpr (sizeof(T) == 4) {
    scale = a.scale32;
    do_scale = a.scaled && (OP != OP_C2C_SOLVE);
  } else {
    scale = (T)a.scale;
    do_scale = (a.scale != 1.0) && (OP != OP_C2C_SOLVE);
  }
  T2* outC = reinterpret_cast<T2*>(a.out);
  T* outR = reinterpret_cast<T*>(a.out);
  auto R = [&](int l, int p) -> const T2& { return res[(size_t)p * nl + l]; };
  if (OP == OP_R2C) {
    const int work = nl * (M + 1);
    for (int t = tid; t < work; t += nth) {
      int l, kk;
      if (CONTIG) divmod(t, fM1, l, kk); else divmod(t, fL, kk, l);
      if (l < nlv) {
        T2 X = r2c_post(res + l, nl, M, kk, a.tw.wN);
        if (do_scale) X = mk<T2>(X.x * scale, X.y * scale);
        outC[orow(l) + opos(kk)] = X;
      }
    }
  } else if (OP == OP_DCT2) {
    const int work = nl * (M + 1);
    for (int t = tid; t < work; t += nth) {
      int l, kk;
      if (CONTIG) divmod(t, fM1, l, kk); else divmod(t, fL, kk, l);
      if (l < nlv) {
        const T2 Vk = r2c_post(res + l, nl, M, kk, a.tw.wN);
        const T2 qv = cmul(ldtw<T2>(a.tw.wD, kk), Vk);
        const long long base = orow(l);
        T y0 = T(2) * qv.x, y1 = T(-2) * qv.y;
        if (do_scale) { y0 = y0 * scale; y1 = y1 * scale; }
        if (kk < n) outR[base + opos(kk)] = y0;
        if (kk >= 1 && kk <= M - 1) outR[base + opos(n - kk)] = y1;
      }
    }
  } else if (OP == OP_C2R || OP == OP_DCT3) {
    // line sums for the mean removal: FP64 in the FP64 path; in FP32 kernels a compensated
    // pair per thread (two-sum on the FP32 pipe, the per-thread error far below FP64's),
    // converted once and reduced across the CTA in FP64
    const bool want_sum = (ST == ST_FIELD) && a.partial != nullptr;
    double lsum = 0.0;
    float lsh = 0.f, lsl = 0.f;
    const int work = nl * n;
    for (int t = tid; t < work; t += nth) {
      int l, i;
      if (CONTIG) divmod(t, fN, l, i); else divmod(t, fL, i, l);
      if (l < nlv) {
        int q = i;  // index into v (the c2r output)
        if (OP == OP_DCT3) q = (i & 1) ? (n - 1 - (i >> 1)) : (i >> 1);
        const T2 zz = R(l, q >> 1);
        T x = (q & 1) ? zz.y : zz.x;
        if (do_scale) x = x * scale;
        if (ST == ST_FIELD) {
          if constexpr (CONTIG) {
            a.fdst[rc(l, i)] = x;
          } else {
            int j, k;
            row_jk<DIM>(line0 + l, outer, j, k);
            a.fdst[a.L.idx(i + 1, j, kst<DIM>(k))] = x;
          }
          if (want_sum) {
            if constexpr (sizeof(T) == 8) {
              lsum += x;
            } else {
              float s, e;
              two_sum(lsh, (float)x, s, e);
              lsh = s;
              lsl += e;
            }
          }
        } else {
          outR[(long long)(line0 + l) * a.out_line + (long long)i * a.out_pos + (long long)outer * a.out_outer] = x;
        }
      }
    }
    if (want_sum) {
      // deterministic CTA sum (fixed order)
      if constexpr (sizeof(T) == 4) {
        // FP32 pairs through a warp butterfly, one FP64 value per warp, the warps summed
        // in order by thread 0 (the FP64 work of an FP32 kernel kept to a few instructions)
        for (int o = 16; o > 0; o >>= 1) {
          const float oh = __shfl_xor_sync(0xffffffffu, lsh, o), ol = __shfl_xor_sync(0xffffffffu, lsl, o);
          float s2, e2;
          two_sum(lsh, oh, s2, e2);
          lsh = s2;
          lsl = e2 + (lsl + ol);
        }
        __shared__ double redw[32];
        if ((tid & 31) == 0) redw[tid >> 5] = (double)lsh + (double)lsl;
        __syncthreads();
        if (tid == 0) {
          double t = 0.0;
          for (int w = 0; w < (nth + 31) / 32; ++w) t += redw[w];
          a.partial[(long long)blockIdx.y * gridDim.x + blockIdx.x] = t;
        }
      } else {
        __shared__ double red[256];
        red[tid] = lsum;
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
          if (tid < s) red[tid] += red[tid + s];
          __syncthreads();
        }
        if (tid == 0) a.partial[(long long)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
      }
    }
  } else if (kStridedIdx && !CONTIG && nl_divides) {  // complex out, strided lines (as the strided load)
    int l, p0;
    divmod(tid, fL, p0, l);
    if (l < nlv) {
      const int dp = nth_l;
      T2* dst = outC + (long long)(line0 + l) * a.out_line + (long long)outer * a.out_outer + (long long)p0 * a.out_pos;
      const long long step = (long long)dp * a.out_pos;
      for (int p = p0; p < M; p += dp, dst += step) {
        T2 z = R(l, p);
        if (do_scale) z = mk<T2>(z.x * scale, z.y * scale);
        *dst = z;
      }
    }
  } else {  // complex out
    const int work = nl * M;
    for (int t = tid; t < work; t += nth) {
      int l, p;
      if (CONTIG) divmod(t, fM, l, p); else divmod(t, fL, p, l);
      if (l < nlv) {
        T2 z = R(l, p);
        if (do_scale) z = mk<T2>(z.x * scale, z.y * scale);
        outC[(long long)(line0 + l) * a.out_line + (long long)p * a.out_pos + (long long)outer * a.out_outer] = z;
      }
    }
  }
}

template <typename T, int DIM, bool CONTIG, int OP, int LD, int ST>
__global__ void __launch_bounds__(256) k_line(LineArgs<T> a) {
  line_body<T, DIM, CONTIG, OP, LD, ST>(a);
}

// FP32 x-line transforms: compiled for 5 resident CTAs per SM (<= 48 registers, room for
// the radix-8 passes), where the default register choice would leave 4.
#ifndef FEN_ROW32_MINB
#define FEN_ROW32_MINB 5
#endif
template <int DIM, int OP, int LD, int ST>
__global__ void __launch_bounds__(256, FEN_ROW32_MINB) k_line_row32(LineArgs<float> a) {
  line_body<float, DIM, true, OP, LD, ST>(a);
}

// ------------------------------------------------------------------------------------
// Batched Thomas solve along one spectral axis (poisson.f90:348-385, 544-581, 1094-1135,
// 1233-1274, 1372-1413).  One thread per (column, outer) system.  The pivots depend only on
// the wavenumbers, so the forward-elimination coefficients c1 and the row factors are
// tabulated once at set-up with the reference's arithmetic; each solve then runs the
// right-hand-side recurrences.  FORM3 = the 3D solvers' reciprocal `factor` form, else the
// 2D solvers' division form.  Arithmetic uses explicitly rounded operations (no FMA
// contraction) so the zero-mode pivot cancels to exactly zero as in the reference.
//
// The interior rows share a, b and c, so each pivot is a function of the previous c1 alone;
// in FP64 that recurrence reaches an exact fixed point after a few rows for all but the
// lowest wavenumbers (channel 512 x 256 x 384: 11 rows on average, 43 at the 99th
// percentile, 12 of 98688 systems never).  conv[sys] is the first row whose (c1, factor)
// repeat the previous row's bit for bit; every later interior row then holds the same pair,
// so a sweep reads the tables for rows below conv only and keeps the fixed point in
// registers: the values used are the tabulated ones, and the results are unchanged.
// ------------------------------------------------------------------------------------
struct ThomasArgs {
  void* x;                    // spectral data (complex or real), in place
  long long s_col, s_row, s_outer;
  int ncol, nouter, n;
  const double* a;            // sub-diagonal a(row)
  double aval;                // a(row) of rows 1 .. n-1 (all equal: 1/delta^2)
  const double* c1;           // [sys][row] forward coefficients
  const double* fac;          // [sys][row] reciprocal factor (FORM3) or divisor (2D form); last row: raw pivot
  const int* conv;            // [sys] first interior row of the fixed point (n - 1: none)
  int form3;
  int split2;                 // complex data swept as two real systems: thread 2c + part, part 0 re / 1 im
  float avh, avl;             // aval as a (hi, lo) float pair (k_thomas_df)
};

// Elimination arithmetic: r - a d as one fused multiply-add, then the row factor.
template <typename V> struct ThomasOps;
template <> struct ThomasOps<double> {
  static __device__ __forceinline__ double sub_amul(double r, double a, double d) { return fma(-a, d, r); }
  static __device__ __forceinline__ double mul(double r, double f) { return __dmul_rn(r, f); }
  static __device__ __forceinline__ double div(double r, double f) { return __ddiv_rn(r, f); }
  static __device__ __forceinline__ double zero() { return 0.0; }
};
template <> struct ThomasOps<double2> {
  static __device__ __forceinline__ double2 sub_amul(double2 r, double a, double2 d) {
    return make_double2(fma(-a, d.x, r.x), fma(-a, d.y, r.y));
  }
  static __device__ __forceinline__ double2 mul(double2 r, double f) { return make_double2(__dmul_rn(r.x, f), __dmul_rn(r.y, f)); }
  static __device__ __forceinline__ double2 div(double2 r, double f) { return make_double2(__ddiv_rn(r.x, f), __ddiv_rn(r.y, f)); }
  static __device__ __forceinline__ double2 zero() { return make_double2(0.0, 0.0); }
};

// FP32 <-> FP64 conversions on the integer pipe.  GB300 issues FP64 at 1/64 of the FP32
// rate and its conversion instructions share that pipe, so the mixed form's tridiagonal
// solve (FP32 storage, FP64 elimination) widens and narrows by rewriting the IEEE fields:
// exact widening, round-to-nearest-even narrowing.  Zero, subnormal, infinite and NaN
// values (and results outside the normal FP32 range) take the hardware conversion.
// The rare cases go through calls that cannot be inlined: a plain conversion there would be
// if-converted into a select and then execute on the FP64 pipe for every element.
static __device__ __noinline__ double widen_rare(float f) { return (double)f; }
static __device__ __noinline__ float narrow_rare(double d) { return (float)d; }
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = u & 0x7F800000u;
  if (ex == 0u || ex == 0x7F800000u) return widen_rare(f);
  const unsigned hi = (u & 0x80000000u) | (((u & 0x7FFFFFFFu) >> 3) + 0x38000000u);
  return __hiloint2double((int)hi, (int)(u << 29));
}
__device__ __forceinline__ float narrow(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned e = (hi >> 20) & 0x7FFu;
  if (e < 897u || e > 1150u) return narrow_rare(d);  // FP32 exponent 1..254 only
  unsigned f = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  const unsigned rem = lo & 0x1FFFFFFFu;
  if (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) f += 1u;  // carries into the exponent
  return __uint_as_float(f);
}

// VS is the storage type (float/float2 in the mixed form), VC the FP64 compute type.
template <typename VS, typename VC>
__device__ __forceinline__ VC tconv(VS v);
template <> __device__ __forceinline__ double tconv<double, double>(double v) { return v; }
template <> __device__ __forceinline__ double2 tconv<double2, double2>(double2 v) { return v; }
template <> __device__ __forceinline__ double tconv<float, double>(float v) { return widen(v); }
template <> __device__ __forceinline__ double2 tconv<float2, double2>(float2 v) { return make_double2(widen(v.x), widen(v.y)); }
template <typename VC, typename VS>
__device__ __forceinline__ VS tback(VC v);
template <> __device__ __forceinline__ double tback<double, double>(double v) { return v; }
template <> __device__ __forceinline__ double2 tback<double2, double2>(double2 v) { return v; }
template <> __device__ __forceinline__ float tback<double, float>(double v) { return narrow(v); }
template <> __device__ __forceinline__ float2 tback<double2, float2>(double2 v) { return make_float2(narrow(v.x), narrow(v.y)); }

// One system per thread.  The rows are swept in batches of kTB: the batch's right-hand
// sides (and, below conv, its table values) are loaded first (independent loads, their
// latencies overlap), then the batch's dependent elimination steps run in registers.  The
// arithmetic and its order are the plain Thomas recurrence.
constexpr int kTB = 8;

// Resident 128-thread CTAs per SM the mixed-form 3D sweep (k_thomas_mixed) is compiled for:
// more systems in flight than the compiler's register choice (with the three-instruction
// sweep on the mixed channel 512x256x384: spectral stage 0.77 -> 0.75 ms at 8 CTAs, 0.76 ms
// at 6; 8 spills here, 6 does not).
#ifndef FEN_THOMAS_MINB
#define FEN_THOMAS_MINB 6
#endif
template <typename VS, typename VC>
__global__ void __launch_bounds__(128) k_thomas(ThomasArgs a) {
  typedef ThomasOps<VC> O;
  const int tcol = blockIdx.x * blockDim.x + threadIdx.x;
  const int col = a.split2 ? (tcol >> 1) : tcol;
  const int outer = blockIdx.y;
  if (col >= a.ncol) return;
  // split2: the real and imaginary parts of one complex system are two real systems with the
  // same coefficients, swept by neighbouring threads (twice the threads, coalesced loads)
  const int w = a.split2 ? 2 : 1;
  VS* X = reinterpret_cast<VS*>(a.x) + ((long long)col * a.s_col + (long long)outer * a.s_outer) * w + (tcol & (w - 1));
  const long long sys = (long long)outer * a.ncol + col;
  const long long ns = (long long)a.ncol * a.nouter;  // tables are [row][system]
  const double* c1 = a.c1 + sys;
  const double* f = a.fac + sys;
  const int n = a.n;
  const long long sr = a.s_row * w;
  const double av = a.aval;
  // the fixed point of the interior rows: rows >= T hold row T - 1's (c1, factor)
  const int T = a.conv[sys];
  const double ffix = f[(long long)(T - 1) * ns];
  const double cfix = c1[(long long)(T - 1) * ns];
  // forward sweep: d1 overwrites the right-hand side
  VC d = tconv<VS, VC>(X[0]);
  d = a.form3 ? O::mul(d, f[0]) : O::div(d, f[0]);
  X[0] = tback<VC, VS>(d);
  int t = 1;
  for (; t + kTB <= n - 1; t += kTB) {
    VS xb[kTB];
    double fb[kTB];
#pragma unroll
    for (int q = 0; q < kTB; ++q) {
      xb[q] = X[(long long)(t + q) * sr];
      fb[q] = (t + q < T) ? f[(long long)(t + q) * ns] : ffix;
    }
#pragma unroll
    for (int q = 0; q < kTB; ++q) {
      VC r = O::sub_amul(tconv<VS, VC>(xb[q]), av, d);
      d = a.form3 ? O::mul(r, fb[q]) : O::div(r, fb[q]);
      xb[q] = tback<VC, VS>(d);
    }
#pragma unroll
    for (int q = 0; q < kTB; ++q) X[(long long)(t + q) * sr] = xb[q];
  }
  for (; t < n - 1; ++t) {
    VC r = tconv<VS, VC>(X[(long long)t * sr]);
    r = O::sub_amul(r, av, d);
    const double ft = (t < T) ? f[(long long)t * ns] : ffix;
    d = a.form3 ? O::mul(r, ft) : O::div(r, ft);
    X[(long long)t * sr] = tback<VC, VS>(d);
  }
  {
    const double piv = f[(long long)(n - 1) * ns];
    VC r = tconv<VS, VC>(X[(long long)(n - 1) * sr]);
    if (piv != 0.0) d = O::div(O::sub_amul(r, a.a[n - 1], d), piv);
    else d = O::zero();
  }
  // backward sweep
  VC xn = d;
  X[(long long)(n - 1) * sr] = tback<VC, VS>(xn);
  t = n - 2;
  for (; t - kTB + 1 >= 0; t -= kTB) {
    VS xb[kTB];
    double cb[kTB];
#pragma unroll
    for (int q = 0; q < kTB; ++q) {
      xb[q] = X[(long long)(t - q) * sr];
      cb[q] = (t - q < T) ? c1[(long long)(t - q) * ns] : cfix;
    }
#pragma unroll
    for (int q = 0; q < kTB; ++q) {
      xn = O::sub_amul(tconv<VS, VC>(xb[q]), cb[q], xn);
      xb[q] = tback<VC, VS>(xn);
    }
#pragma unroll
    for (int q = 0; q < kTB; ++q) X[(long long)(t - q) * sr] = xb[q];
  }
  for (; t >= 0; --t) {
    VC dt = tconv<VS, VC>(X[(long long)t * sr]);
    xn = O::sub_amul(dt, (t < T) ? c1[(long long)t * ns] : cfix, xn);
    X[(long long)t * sr] = tback<VC, VS>(xn);
  }
}

// Mixed-form sweep (FP32 spectrum, FP64 elimination).  Above the fixed point (rows
// t0 = conv - 1 .. n - 2, where the factor f and c1 are the constants f*, c*) the forward
// sweep keeps the unscaled e_t = r_t - a d_(t-1), d_t = f* e_t, as one FMA per row,
// e_t = r_t - (a f*) e_(t-1); the backward sweep runs on y_t = x_t / f*, y_t = e_t - c* y_(t+1),
// again one FMA, and the stored result x_t = f* y_t is formed by an FP32 multiply of the
// narrowed y_t (an extra rounding of the order of the narrowing itself).  Rows below t0 and the
// last row take the tabulated recurrence of k_thomas.  Two FP64 instructions per row instead
// of three; FORM3 (the reciprocal factor form) only.
template <int SPLIT2>
__global__ void __launch_bounds__(128, FEN_THOMAS_MINB) k_thomas_mixed(ThomasArgs a) {
  const int tcol = blockIdx.x * blockDim.x + threadIdx.x;
  const int col = SPLIT2 ? (tcol >> 1) : tcol;
  const int outer = blockIdx.y;
  if (col >= a.ncol) return;
  const int w = SPLIT2 ? 2 : 1;
  float* X = reinterpret_cast<float*>(a.x) + ((long long)col * a.s_col + (long long)outer * a.s_outer) * w + (tcol & (w - 1));
  const long long sys = (long long)outer * a.ncol + col;
  const long long ns = (long long)a.ncol * a.nouter;
  const double* c1 = a.c1 + sys;
  const double* f = a.fac + sys;
  const int n = a.n;
  const long long sr = a.s_row * w;
  const double av = a.aval;
  const int T = a.conv[sys];
  const int t0 = (T < n - 1) ? T - 1 : n - 1;  // first row of the fixed point (n - 1: none)
  // forward sweep, tabulated rows [0, t0): d_t = (r_t - a d_(t-1)) f_t
  double d = 0.0;
  int t = 0;
  for (; t + kTB <= t0; t += kTB) {
    float xb[kTB];
    double fb[kTB];
#pragma unroll
    for (int q = 0; q < kTB; ++q) {
      xb[q] = X[(long long)(t + q) * sr];
      fb[q] = f[(long long)(t + q) * ns];
    }
#pragma unroll
    for (int q = 0; q < kTB; ++q) {
      const double r = (t + q == 0) ? widen(xb[q]) : fma(-av, d, widen(xb[q]));
      d = __dmul_rn(r, fb[q]);
      xb[q] = narrow(d);
    }
#pragma unroll
    for (int q = 0; q < kTB; ++q) X[(long long)(t + q) * sr] = xb[q];
  }
  for (; t < t0; ++t) {
    const double r = (t == 0) ? widen(X[0]) : fma(-av, d, widen(X[(long long)t * sr]));
    d = __dmul_rn(r, f[(long long)t * ns]);
    X[(long long)t * sr] = narrow(d);
  }
  const double piv = f[(long long)(n - 1) * ns];
  double xn;
  if (t0 < n - 1) {
    const double fs = f[(long long)t0 * ns], cs = c1[(long long)t0 * ns];
    const double g = __dmul_rn(av, fs);
    // converged rows [t0, n - 1): e_t, stored in place of d_t
    double e = (t0 == 0) ? widen(X[0]) : fma(-av, d, widen(X[(long long)t0 * sr]));
    X[(long long)t0 * sr] = narrow(e);
    t = t0 + 1;
    for (; t + kTB <= n - 1; t += kTB) {
      float xb[kTB];
#pragma unroll
      for (int q = 0; q < kTB; ++q) xb[q] = X[(long long)(t + q) * sr];
#pragma unroll
      for (int q = 0; q < kTB; ++q) {
        e = fma(-g, e, widen(xb[q]));
        xb[q] = narrow(e);
      }
#pragma unroll
      for (int q = 0; q < kTB; ++q) X[(long long)(t + q) * sr] = xb[q];
    }
    for (; t < n - 1; ++t) {
      e = fma(-g, e, widen(X[(long long)t * sr]));
      X[(long long)t * sr] = narrow(e);
    }
    // last row: a d_(n-2) = (a f*) e_(n-2); the zero mode's pivot cancels to exactly zero
    const double r = widen(X[(long long)(n - 1) * sr]);
    xn = (piv != 0.0) ? __ddiv_rn(fma(-g, e, r), piv) : 0.0;
    X[(long long)(n - 1) * sr] = narrow(xn);
    // backward sweep on y = x / f*: y_t = e_t - c* y_(t+1); x_t = f* y_t in FP32
    const float fs32 = narrow(fs);
    double y = __ddiv_rn(xn, fs);
    t = n - 2;
    for (; t - kTB + 1 >= t0; t -= kTB) {
      float xb[kTB];
#pragma unroll
      for (int q = 0; q < kTB; ++q) xb[q] = X[(long long)(t - q) * sr];
#pragma unroll
      for (int q = 0; q < kTB; ++q) {
        y = fma(-cs, y, widen(xb[q]));
        xb[q] = narrow(y) * fs32;
      }
#pragma unroll
      for (int q = 0; q < kTB; ++q) X[(long long)(t - q) * sr] = xb[q];
    }
    for (; t >= t0; --t) {
      y = fma(-cs, y, widen(X[(long long)t * sr]));
      X[(long long)t * sr] = narrow(y) * fs32;
    }
    xn = __dmul_rn(fs, y);  // x_(t0), the start of the tabulated rows below
  } else {
    const double r = widen(X[(long long)(n - 1) * sr]);
    xn = (piv != 0.0) ? __ddiv_rn(fma(-av, d, r), piv) : 0.0;
    X[(long long)(n - 1) * sr] = narrow(xn);
    t = n - 2;
  }
  // backward sweep, tabulated rows below t0: x_t = d_t - c1_t x_(t+1)
  for (t = t0 - 1; t - kTB + 1 >= 0; t -= kTB) {
    float xb[kTB];
    double cb[kTB];
#pragma unroll
    for (int q = 0; q < kTB; ++q) {
      xb[q] = X[(long long)(t - q) * sr];
      cb[q] = c1[(long long)(t - q) * ns];
    }
#pragma unroll
    for (int q = 0; q < kTB; ++q) {
      xn = fma(-cb[q], xn, widen(xb[q]));
      xb[q] = narrow(xn);
    }
#pragma unroll
    for (int q = 0; q < kTB; ++q) X[(long long)(t - q) * sr] = xb[q];
  }
  for (; t >= 0; --t) {
    xn = fma(-c1[(long long)t * ns], xn, widen(X[(long long)t * sr]));
    X[(long long)t * sr] = narrow(xn);
  }
}

// Mixed-form sweep in double-float arithmetic (FP32 pairs, about 48 significant bits): the
// recurrences of k_thomas_mixed with every per-row operation on the FP32 pipe.  GB300 issues
// FP64 at about 1/64 of its FP32 rate and the FP64 sweep is bound by that pipe; the pair form
// costs about fourteen FP32 instructions per row and recurrence instead of one FP64 FMA, and
// its rounding (2^-46 per operation) stays far below the FP32 spectrum it reads and writes.
// The tables c1 and factor are read as (hi, lo) float pairs of the FP64 values
// (k_thomas_pair_tables converts them in place at set-up).  FORM3 only.  Per system, the
// last row's division and the change of variables at the fixed point run in FP64 (a handful
// of instructions per system, not per row).
// Rows per load batch and resident 128-thread CTAs per SM of k_thomas_df.
// 8 rows in flight per thread at 70 registers (6 CTAs of 128 per SM).  Measured on the mixed
// channel (spectral stage, two sweeps): 0.52 ms; 4 rows at 40 registers (12 CTAs, the whole
// grid resident at once) 0.80 ms; 4 rows at 48 registers (10 CTAs) 0.63 ms; with the systems
// numbered across the outer rows instead of padded per row, 0.55 ms; with the rows 8, 16 or
// 32 ahead prefetched into L2, unchanged; 12 or 16 rows in flight at 86-112 registers (4-5
// CTAs), 0.49-0.52 ms; both parts of a complex system in one thread (two interleaved chains,
// 77 registers, the whole spectrum resident in one wave), 0.48 ms against 0.474.  Eight rows
// in flight at six CTAs is the balance.
#ifndef FEN_THOMAS_DF_TB
#define FEN_THOMAS_DF_TB 8
#endif
#ifndef FEN_THOMAS_DF_MINB
#define FEN_THOMAS_DF_MINB 6
#endif
constexpr int kTBD = FEN_THOMAS_DF_TB;
__device__ __forceinline__ DF df_of(float2 v) { return DF{v.x, v.y}; }
// x - g e for an FP32 x and pairs g, e (FMA-exact leading product, Knuth sum)
__device__ __forceinline__ DF df_xmy(float x, DF g, DF e) {
  const float p = g.h * e.h;
  float pe = fmaf(g.h, e.h, -p);
  pe = fmaf(g.h, e.l, pe);
  pe = fmaf(g.l, e.h, pe);
  float sh, sl;
  two_sum(x, -p, sh, sl);
  sl = sl - pe;
  const float h = sh + sl;
  return DF{h, sl - (h - sh)};
}
__device__ __forceinline__ double df_to_d(DF v) { return (double)v.h + (double)v.l; }
__device__ __forceinline__ DF df_from_d(double x) {
  const F2 q = split_d(x);
  return DF{q.hi, q.lo};
}

template <int SPLIT2>
__global__ void __launch_bounds__(128, FEN_THOMAS_DF_MINB) k_thomas_df(ThomasArgs a) {
  const int tcol = blockIdx.x * blockDim.x + threadIdx.x;
  const int col = SPLIT2 ? (tcol >> 1) : tcol;
  const int outer = blockIdx.y;
  if (col >= a.ncol) return;
  const int w = SPLIT2 ? 2 : 1;
  float* X = reinterpret_cast<float*>(a.x) + ((long long)col * a.s_col + (long long)outer * a.s_outer) * w + (tcol & (w - 1));
  const long long sys = (long long)outer * a.ncol + col;
  const long long ns = (long long)a.ncol * a.nouter;
  const float2* c1 = reinterpret_cast<const float2*>(a.c1) + sys;
  const float2* f = reinterpret_cast<const float2*>(a.fac) + sys;
  const int n = a.n;
  const long long sr = a.s_row * w;
  const DF av{a.avh, a.avl};
  const int T = a.conv[sys];
  const int t0 = (T < n - 1) ? T - 1 : n - 1;  // first row of the fixed point (n - 1: none)
  // forward sweep, tabulated rows [0, t0): d_t = (r_t - a d_(t-1)) f_t
  DF d{0.f, 0.f};
  int t = 0;
  for (; t + kTBD <= t0; t += kTBD) {
    float xb[kTBD];
    float2 fb[kTBD];
#pragma unroll
    for (int q = 0; q < kTBD; ++q) {
      xb[q] = X[(long long)(t + q) * sr];
      fb[q] = f[(long long)(t + q) * ns];
    }
#pragma unroll
    for (int q = 0; q < kTBD; ++q) {
      const DF r = (t + q == 0) ? DF{xb[q], 0.f} : df_xmy(xb[q], av, d);
      d = dmul(r, df_of(fb[q]));
      xb[q] = d.h;
    }
#pragma unroll
    for (int q = 0; q < kTBD; ++q) X[(long long)(t + q) * sr] = xb[q];
  }
  for (; t < t0; ++t) {
    const float x = X[(long long)t * sr];
    const DF r = (t == 0) ? DF{x, 0.f} : df_xmy(x, av, d);
    d = dmul(r, df_of(f[(long long)t * ns]));
    X[(long long)t * sr] = d.h;
  }
  const double piv = df_to_d(df_of(f[(long long)(n - 1) * ns]));
  DF xn;
  if (t0 < n - 1) {
    const double fsd = df_to_d(df_of(f[(long long)t0 * ns]));
    const DF cs = df_of(c1[(long long)t0 * ns]);
    const DF g = df_from_d(df_to_d(av) * fsd);
    // converged rows [t0, n - 1): e_t = r_t - a d_(t-1) unscaled, e_t = x_t - (a f*) e_(t-1)
    DF e = (t0 == 0) ? DF{X[0], 0.f} : df_xmy(X[(long long)t0 * sr], av, d);
    X[(long long)t0 * sr] = e.h;
    t = t0 + 1;
    for (; t + kTBD <= n - 1; t += kTBD) {
      float xb[kTBD];
#pragma unroll
      for (int q = 0; q < kTBD; ++q) xb[q] = X[(long long)(t + q) * sr];
#pragma unroll
      for (int q = 0; q < kTBD; ++q) {
        e = df_xmy(xb[q], g, e);
        xb[q] = e.h;
      }
#pragma unroll
      for (int q = 0; q < kTBD; ++q) X[(long long)(t + q) * sr] = xb[q];
    }
    for (; t < n - 1; ++t) {
      e = df_xmy(X[(long long)t * sr], g, e);
      X[(long long)t * sr] = e.h;
    }
    // last row: a d_(n-2) = (a f*) e_(n-2); the zero mode's pivot is exactly zero
    const DF r = df_xmy(X[(long long)(n - 1) * sr], g, e);
    const double xl = (piv != 0.0) ? df_to_d(r) / piv : 0.0;
    X[(long long)(n - 1) * sr] = (float)xl;
    // backward sweep on y = x / f*: y_t = e_t - c* y_(t+1); x_t = f* y_t in FP32
    const float fs32 = (float)fsd;
    DF y = df_from_d(xl / fsd);
    t = n - 2;
    for (; t - kTBD + 1 >= t0; t -= kTBD) {
      float xb[kTBD];
#pragma unroll
      for (int q = 0; q < kTBD; ++q) xb[q] = X[(long long)(t - q) * sr];
#pragma unroll
      for (int q = 0; q < kTBD; ++q) {
        y = df_xmy(xb[q], cs, y);
        xb[q] = y.h * fs32;
      }
#pragma unroll
      for (int q = 0; q < kTBD; ++q) X[(long long)(t - q) * sr] = xb[q];
    }
    for (; t >= t0; --t) {
      y = df_xmy(X[(long long)t * sr], cs, y);
      X[(long long)t * sr] = y.h * fs32;
    }
    xn = df_from_d(fsd * df_to_d(y));  // x_(t0), the start of the tabulated rows below
  } else {
    const DF r = df_xmy(X[(long long)(n - 1) * sr], av, d);
    const double xl = (piv != 0.0) ? df_to_d(r) / piv : 0.0;
    X[(long long)(n - 1) * sr] = (float)xl;
    xn = df_from_d(xl);
    t = n - 2;
  }
  // backward sweep, tabulated rows below t0: x_t = d_t - c1_t x_(t+1)
  for (t = t0 - 1; t - kTBD + 1 >= 0; t -= kTBD) {
    float xb[kTBD];
    float2 cb[kTBD];
#pragma unroll
    for (int q = 0; q < kTBD; ++q) {
      xb[q] = X[(long long)(t - q) * sr];
      cb[q] = c1[(long long)(t - q) * ns];
    }
#pragma unroll
    for (int q = 0; q < kTBD; ++q) {
      xn = df_xmy(xb[q], df_of(cb[q]), xn);
      xb[q] = xn.h;
    }
#pragma unroll
    for (int q = 0; q < kTBD; ++q) X[(long long)(t - q) * sr] = xb[q];
  }
  for (; t >= 0; --t) {
    xn = df_xmy(X[(long long)t * sr], df_of(c1[(long long)t * ns]), xn);
    X[(long long)t * sr] = xn.h;
  }
}

// The FP64 tables c1 and factor rewritten in place as (hi, lo) float pairs (k_thomas_df):
// hi = the FP64 value rounded to FP32, lo = the remainder rounded to FP32.
static __global__ void k_thomas_pair_tables(long long nt, double* c1, double* fac) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nt; i += (long long)gridDim.x * blockDim.x) {
    const F2 p = split_d(c1[i]), q = split_d(fac[i]);
    reinterpret_cast<float2*>(c1)[i] = make_float2(p.hi, p.lo);
    reinterpret_cast<float2*>(fac)[i] = make_float2(q.hi, q.lo);
  }
}

// Tabulate c1 and the row factors for every (col, outer) system with the reference's
// operation order, and the first interior row of their fixed point (conv, see k_thomas).
// lamA indexed by col, lamB by outer (nullptr in 2D).
static __global__ void k_thomas_tables(int ncol, int nouter, int n, const double* a, const double* b, const double* c,
                                const double* lamA, const double* lamB, int form3, double* c1, double* fac, int* conv) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  const int outer = blockIdx.y;
  if (col >= ncol) return;
  const long long sys = (long long)outer * ncol + col;
  const long long ns = (long long)ncol * nouter;  // [row][system]
  double* C1 = c1 + sys;
  double* F = fac + sys;
  const double mA = lamA[col];
  const double mB = lamB ? lamB[outer] : 0.0;
  int T = n - 1;
  if (form3) {
    // factor = 1/(b + mwn_x + mwn_y - a*c1)   (poisson.f90:1096, 1105, 1114)
    double fct = __ddiv_rn(1.0, __dadd_rn(__dadd_rn(b[0], mA), mB));
    C1[(0) * ns] = __dmul_rn(c[0], fct);
    F[(0) * ns] = fct;
    for (int t = 1; t < n - 1; ++t) {
      fct = __ddiv_rn(1.0, __dsub_rn(__dadd_rn(__dadd_rn(b[t], mA), mB), __dmul_rn(a[t], C1[(t - 1) * ns])));
      C1[(t) * ns] = __dmul_rn(c[t], fct);
      F[(t) * ns] = fct;
      if (T == n - 1 && C1[t * ns] == C1[(t - 1) * ns] && F[t * ns] == F[(t - 1) * ns]) T = t;
    }
    F[(n - 1) * ns] = __dsub_rn(__dadd_rn(__dadd_rn(b[n - 1], mA), mB), __dmul_rn(a[n - 1], C1[(n - 2) * ns]));
    C1[(n - 1) * ns] = 0.0;
  } else {
    // c1 = c/(b - a*c1 + mwn);  d1 = (r - a*d1)/(b + mwn - a*c1)   (poisson.f90:350-366)
    C1[(0) * ns] = __ddiv_rn(c[0], __dadd_rn(b[0], mA));
    F[(0) * ns] = __dadd_rn(b[0], mA);
    for (int t = 1; t < n - 1; ++t) {
      C1[(t) * ns] = __ddiv_rn(c[t], __dadd_rn(__dsub_rn(b[t], __dmul_rn(a[t], C1[(t - 1) * ns])), mA));
      F[(t) * ns] = __dsub_rn(__dadd_rn(b[t], mA), __dmul_rn(a[t], C1[(t - 1) * ns]));
      if (T == n - 1 && C1[t * ns] == C1[(t - 1) * ns] && F[t * ns] == F[(t - 1) * ns]) T = t;
    }
    F[(n - 1) * ns] = __dsub_rn(__dadd_rn(b[n - 1], mA), __dmul_rn(a[n - 1], C1[(n - 2) * ns]));
    C1[(n - 1) * ns] = 0.0;
  }
  conv[sys] = T;
}

// ------------------------------------------------------------------------------------
// Correction and pressure update (navier_stokes.f90:505-566): v = v* - dt grad(phi)/rhof,
// p = p + phi.  Ghosts of v and p are refilled afterwards.
// ------------------------------------------------------------------------------------
template <typename T>
struct CorrArgs {
  const T *us, *vs, *ws, *phi;
  T *u, *v, *w, *p;
  double id[3];
  double dt_host;
  int iso, use_dev_dt, rhof_one;
  double rhof;
};

template <typename T, int DIM>
__global__ void __launch_bounds__(256) k_correct(Layout L, const StepScalars* __restrict__ sc, CorrArgs<T> a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const T dt = (T)(a.use_dev_dt ? sc->dt : a.dt_host);
  const T f = a.rhof_one ? dt : (T)((double)dt / a.rhof);
  // v = v* - dt/rho (phi(+1) - phi) / delta as one FMA per component with g = dt/(rho delta)
  const T gx = -(T)a.id[0] * f;
  const T gy = a.iso ? gx : -(T)a.id[1] * f;
  const T gz = a.iso ? gx : -(T)a.id[2] * f;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j, k = 1 + cw.k;
    const long long c = L.idx(i, j, kst<DIM>(k));
    const T ph = a.phi[c];
    a.u[c] = fmx(a.phi[c + 1] - ph, gx, a.us[c]);
    a.v[c] = fmx(a.phi[c + L.sx] - ph, gy, a.vs[c]);
    if (DIM == 3) a.w[c] = fmx(a.phi[c + L.sp] - ph, gz, a.ws[c]);
    a.p[c] = a.p[c] + ph;
  }
}

// Mean removal over the interior (poisson.f90:491-503, 1159-1171): every CTA sums the
// per-line partials in the same order, then subtracts mean/float(nx*ny*nz).
// Mean of phi from the per-CTA partial sums of the inverse transform (one CTA; the result
// goes to sc->mean for k_mean_subtract and the host).
static __global__ void __launch_bounds__(1024) k_mean_reduce(const double* __restrict__ partial, int npart, double ncell_f,
                                                      StepScalars* sc) {
  __shared__ double red[1024];
  double s = 0.0;
  for (int q = threadIdx.x; q < npart; q += blockDim.x) s += partial[q];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) sc->mean = red[0] / ncell_f;
}

// Keep the mean of phi for the mixed form's correction (dir 0: mean_phi = mean), or bring it
// back for an explicit removal (dir 1: mean = mean_phi).
static __global__ void k_keep_mean(StepScalars* sc, int dir) {
  if (dir == 0) sc->mean_phi = sc->mean;
  else sc->mean = sc->mean_phi;
}

template <typename T, int DIM>
__global__ void __launch_bounds__(256) k_mean_subtract(Layout L, const StepScalars* __restrict__ sc, T* phi) {
  const T mt = (T)sc->mean;
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j, k = 1 + cw.k;
    const long long c = L.idx(i, j, kst<DIM>(k));
    phi[c] = phi[c] - mt;
  }
}

// ------------------------------------------------------------------------------------
// Diagnostics (navier_stokes.f90:570-619): signed max of div(v) and max(|u|+|v|+|w|),
// per-CTA partials reduced by k_finalize in a fixed order.
// ------------------------------------------------------------------------------------
template <typename T>
struct CheckArgs {
  const T *u, *v, *w;
  double id[3];
  int iso, want_div;
  double* pdiv;
  double* pvel;
  int* nan_flag;
};

// Order-preserving int64 key of a double's bits: key(x) < key(y) iff x < y for non-NaN x, y,
// and the map is its own inverse.  The diagnostics take their maxima on the integer pipe
// (GB300's FP64 pipe is narrow); NaNs are detected from the bits and left out of the maxima.
__device__ __forceinline__ long long okey(long long b) { return b ^ ((b >> 63) & 0x7fffffffffffffffLL); }
__device__ __forceinline__ bool nan_bits(long long b) { return (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }

template <int DIM>
__global__ void __launch_bounds__(256) k_checks(Layout L, CheckArgs<double> a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const long long kneg = okey(__double_as_longlong(-INFINITY));
  long long md = kneg, mv = 0;  // keys of -inf and +0
  bool bad = false;
  const double idx = a.id[0];
  const double idy = a.iso ? idx : a.id[1], idz = a.iso ? idx : a.id[2];
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j, k = 1 + cw.k;
    const long long c = L.idx(i, j, kst<DIM>(k));
    const double uc = a.u[c], vc = a.v[c];
    double vel = fabs(uc) + fabs(vc);
    double d = 0;
    if (a.want_div) d = fma(vc - a.v[c - L.sx], idy, (uc - a.u[c - 1]) * idx);
    if (DIM == 3) {
      const double wc = a.w[c];
      vel = vel + fabs(wc);
      if (a.want_div) d = fma(wc - a.w[c - L.sp], idz, d);
    }
    const long long bv = __double_as_longlong(vel), bd = __double_as_longlong(d);
    const bool nv = nan_bits(bv), nd = nan_bits(bd);
    bad |= nv | nd;
    mv = max(mv, nv ? 0LL : bv);  // vel >= +0: its bits are its key
    md = max(md, nd ? kneg : okey(bd));
  }
  __shared__ long long r1[256], r2[256];
  r1[threadIdx.x] = md;
  r2[threadIdx.x] = mv;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      r1[threadIdx.x] = max(r1[threadIdx.x], r1[threadIdx.x + h]);
      r2[threadIdx.x] = max(r2[threadIdx.x], r2[threadIdx.x + h]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.pdiv[blockIdx.x] = __longlong_as_double(okey(r1[0]));
    a.pvel[blockIdx.x] = __longlong_as_double(r2[0]);
  }
  if (bad) atomicOr(a.nan_flag, 1);
}

// Fold the check partials: maxdiv, maxvel, maxCFL = dt*maxvel/delta (navier_stokes.f90:593, 617).
static __global__ void k_finalize(const double* pdiv, const double* pvel, int np, StepScalars* sc, double delta, double dt_host,
                           int use_dev_dt, const int* nan_flag) {
  __shared__ double r1[256], r2[256];
  double md = -INFINITY, mv = 0.0;
  for (int q = threadIdx.x; q < np; q += blockDim.x) {
    md = fmax(md, pdiv[q]);
    mv = fmax(mv, pvel[q]);
  }
  r1[threadIdx.x] = md;
  r2[threadIdx.x] = mv;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      r1[threadIdx.x] = fmax(r1[threadIdx.x], r1[threadIdx.x + h]);
      r2[threadIdx.x] = fmax(r2[threadIdx.x], r2[threadIdx.x + h]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double dt = use_dev_dt ? sc->dt : dt_host;
    sc->maxdiv = r1[0];
    sc->maxvel = r2[0];
    sc->maxCFL = dt * r2[0] / delta;
    if (*nan_flag) sc->err = 1;
  }
}

// Start-of-step scalars: update_timestep when constant_CFL (navier_stokes.f90:670-730),
// then the AB2 coefficients (:157-158) and the Poisson right-hand-side scale (:118).
static __global__ void k_prologue(StepScalars* sc, int constant_cfl, double cfl, double delta, double density, double rhof) {
  if (threadIdx.x != 0) return;
  double dt;
  if (constant_cfl) {
    sc->dt_o = sc->dt;
    const double mv = sc->maxvel;
    if (mv > 0.0) sc->dt_conv = cfl * delta / mv;
    else sc->dt_conv = 1.0;
    dt = fmin(sc->dt_conv, sc->dt_visc);
    if (dt > 1.1 * sc->dt_o) dt = 1.1 * sc->dt_o;
    sc->dt = dt;
  } else {
    dt = sc->dt;  // written by the host before the step
  }
  sc->A = 1.0 + 0.5 * dt / sc->dt_o;
  sc->B = -0.5 * dt / sc->dt_o;
  sc->rho_over_dt = density / dt;
  sc->dt_over_rhof = dt / rhof;
  const double v[4] = {dt, sc->A, sc->B, sc->rho_over_dt};
  float* dst[4] = {sc->dtp, sc->Ap, sc->Bp, sc->rdtp};
  for (int q = 0; q < 4; ++q) {
    dst[q][0] = (float)v[q];
    dst[q][1] = (float)(v[q] - (double)dst[q][0]);
  }
}

// Tabulated scale/lam of the all-periodic spectral divide with the SOLVE kernel's formula
// (so FP64 results are bit-identical to computing it in place); zero mode -> 0.
template <typename T>
__global__ void k_inv_lam_table(int ncol, int n, int nouter, const double* lamA, const double* lamB, const double* lamC,
                                double scale, T* out) {
  const long long total = (long long)ncol * n * nouter;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const int col = (int)(t % ncol);
    const long long r = t / ncol;
    const int p = (int)(r % n);
    const int outer = (int)(r / n);
    const double lam = lamA[col] + (lamB ? lamB[outer] : 0.0) + lamC[p];
    out[t] = (lam == 0.0) ? T(0) : (T)(scale / lam);
  }
}

// Host-layout <-> HBM-layout copies.  The host array is FEN's contiguous Fortran array with
// gl ghost layers (x fastest): gl = 1 is f(0:nx+1, 0:ny+1, planes) as FEN allocates p, phi,
// v, rho and mu (scalar.f90:79-81 with l = 1); gl = 0 is the interior f(1:nx, 1:ny, 1:nz)
// that FEN allocates for dv, dv_o, grad_p, rhof and S (navier_stokes.f90:759-768, default
// gl = 0).  One contiguous copy moves it to a staging buffer and this kernel scatters rows
// into the padded layout (dir = 0) or gathers them back (dir = 1); with gl = 0 the device
// ghosts are left as they are.  `planes` counts the host array's planes (1 in 2D).
template <typename T>
__global__ void __launch_bounds__(256) k_relayout(Layout L, int planes, int gl, const double* __restrict__ src, T* dst_field,
                                                  const T* __restrict__ src_field, double* dst, int dir) {
  const int nxh = L.n0 + 2 * gl, nyh = L.n1 + 2 * gl;
  const int k0 = (L.dim == 3) ? 1 - gl : 0;  // storage plane of the host array's first plane
  const long long total = (long long)nxh * nyh * planes;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    const long long row = t / nxh;  // j + nyh * plane
    const int i = (int)(t - row * nxh) + 1 - gl;
    const int pl = (int)(row / nyh);
    const int j = (int)(row - (long long)pl * nyh) + 1 - gl;
    const long long d = L.idx(i, j, pl + k0);
    if (dir == 0) dst_field[d] = (T)src[t];
    else dst[t] = (double)src_field[d];
  }
}

}  // namespace fen
