// Mixed-precision form of the projection step.
//
// The state u, v, w, p is kept as double-float pairs (hi + lo, two FP32 words, about 48
// significant bits) and every kernel works with FP32 instructions.  GB300 issues FP64 at
// about 1/58 of its FP32 rate, and FP64 <-> FP32 conversions share the FP64 pipe, so the
// mixed step uses FP64 only where the form requires it: the tridiagonal solves, the mean
// removal and the diagnostics reductions.
//
// Accuracy: FP32 loses the small increments when large neighbouring values are combined
// first (e.g. the fluxes of a slow component advected by a fast mean flow).  Every stencil
// here is therefore evaluated in difference form: products of sums are expanded as
//   a1 b1 - a2 b2 = a1 (b1 - b2) + (a1 - a2) b2,
// and each neighbour difference is taken on the pairs, (hiA - hiB) + (loA - loB), which is
// exact up to one rounding of the difference itself.  The result is the same discrete
// operator as FEN's (navier_stokes.f90:261-404, fields.f90:31-153) evaluated to FP32
// relative accuracy of the increments rather than of the fluxes.
#pragma once
#include "fen_ghost.cuh"
#include "fen_types.cuh"

namespace fen {

// Knuth's error-free sum (no multiplications, so no FMA contraction).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (hi, lo) += x with renormalisation.
__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
  float s, e;
  two_sum(hi, x, s, e);
  e = e + lo;
  hi = s + e;
  lo = e - (hi - s);
}

// Pair arrays of one field.
struct DFField {
  const float* hi;
  const float* lo;
};
struct DFFieldW {
  float* hi;
  float* lo;
};

// Accurate difference A(ca) - A(cb) of a pair field.
__device__ __forceinline__ float dfd(const DFField& A, long long ca, long long cb) {
  return (A.hi[ca] - A.hi[cb]) + (A.lo[ca] - A.lo[cb]);
}

// ------------------------------------------------------------------------------------
// Predictor (mixed): writes the increment dt * rhs (FP32) and dv_o (FP32).
// ------------------------------------------------------------------------------------
struct PredDFArgs {
  DFField u, v, w, p;
  float *du, *dv, *dw;
  float *dox, *doy, *doz;
  const float *Sx, *Sy, *Sz;
  double id[3], id2[3];
  double mu, rhof, g[3];
  int iso, has_S, rhof_one;
};

template <int DIM>
__global__ void __launch_bounds__(256) k_predictor_df(Layout L, const StepScalars* __restrict__ sc, PredDFArgs a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const float A = (float)sc->A, B = (float)sc->B, dt = (float)sc->dt;
  const float idx = (float)a.id[0], idy = (float)a.id[1], idz = (float)a.id[2];
  const float id2x = (float)a.id2[0], id2y = (float)a.id2[1], id2z = (float)a.id2[2];
  const float mu = (float)a.mu, rhof = (float)a.rhof;
  const float qx = 0.25f * idx, qy = 0.25f * idy, qz = 0.25f * idz;
  const long long sy = L.sx, sz = L.sp;
  const DFField U = a.u, V = a.v, W = a.w, P = a.p;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ncell; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % L.n0);
    const long long r = t / L.n0;
    const int j = 1 + (int)(r % L.n1);
    const int k = 1 + (int)(r / L.n1);
    const long long c = L.idx(i, j, kst<DIM>(k));
    const long long ip = c + 1, im = c - 1, jp = c + sy, jm = c - sy;
    // ---- u: -(d(uu)/dx + d(uv)/dy [+ d(uw)/dz]) in difference form
    const float u_c = U.hi[c], u_ip = U.hi[ip], u_im = U.hi[im], u_jp = U.hi[jp], u_jm = U.hi[jm];
    const float v_c = V.hi[c], v_ip = V.hi[ip], v_im = V.hi[im], v_jp = V.hi[jp], v_jm = V.hi[jm];
    float dvx = -(dfd(U, ip, im) * (u_ip + 2.0f * u_c + u_im)) * qx;
    {
      const float a1 = u_jp + u_c, b2 = V.hi[ip - sy] + v_jm;
      const float db = dfd(V, ip, ip - sy) + dfd(V, c, jm);
      dvx = dvx - (a1 * db + dfd(U, jp, jm) * b2) * qy;
    }
    // ---- v
    float dvy;
    {
      const float a1 = v_ip + v_c, b2 = U.hi[im + sy] + u_im;
      const float db = dfd(U, jp, im + sy) + dfd(U, c, im);
      dvy = -((a1 * db + dfd(V, ip, im) * b2) * qx);
    }
    dvy = dvy - (dfd(V, jp, jm) * (v_jp + 2.0f * v_c + v_jm)) * qy;
    float dvz = 0.0f;
    float lux_z = 0.0f, lvy_z = 0.0f;
    if (DIM == 3) {
      const long long kp = c + sz, km = c - sz;
      const float w_c = W.hi[c], w_ip = W.hi[ip], w_im = W.hi[im], w_jp = W.hi[jp], w_jm = W.hi[jm];
      const float w_kp = W.hi[kp], w_km = W.hi[km];
      const float u_kp = U.hi[kp], v_kp = V.hi[kp];
      {  // d(uw)/dz for u
        const float a1 = u_kp + u_c, b2 = W.hi[ip - sz] + W.hi[km];
        const float db = dfd(W, ip, ip - sz) + dfd(W, c, km);
        dvx = dvx - (a1 * db + dfd(U, kp, km) * b2) * qz;
      }
      {  // d(vw)/dz for v
        const float a1 = v_kp + v_c, b2 = W.hi[jp - sz] + W.hi[km];
        const float db = dfd(W, jp, jp - sz) + dfd(W, c, km);
        dvy = dvy - (a1 * db + dfd(V, kp, km) * b2) * qz;
      }
      {  // w terms: d(wu)/dx, d(wv)/dy, d(ww)/dz
        const float a1x = w_c + w_ip, b2x = u_im + U.hi[im + sz];
        const float dbx = dfd(U, c, im) + dfd(U, kp, im + sz);
        const float a1y = w_c + w_jp, b2y = v_jm + V.hi[jm + sz];
        const float dby = dfd(V, c, jm) + dfd(V, kp, jm + sz);
        dvz = -((a1x * dbx + dfd(W, ip, im) * b2x) * qx) - (a1y * dby + dfd(W, jp, jm) * b2y) * qy -
              (dfd(W, kp, km) * (w_kp + 2.0f * w_c + w_km)) * qz;
        // w laplacian (fields.f90:335-337)
        const float lx = dfd(W, ip, c) - dfd(W, c, im);
        const float ly = dfd(W, jp, c) - dfd(W, c, jm);
        const float lz = dfd(W, kp, c) - dfd(W, c, km);
        const float lw = a.iso ? ((lx + ly) + lz) * id2x : lx * id2x + ly * id2y + lz * id2z;
        dvz = dvz + (a.rhof_one ? mu * lw : mu * lw / rhof);
      }
      lux_z = dfd(U, kp, c) - dfd(U, c, km);
      lvy_z = dfd(V, kp, c) - dfd(V, c, km);
    }
    {
      const float lx = dfd(U, ip, c) - dfd(U, c, im);
      const float ly = dfd(U, jp, c) - dfd(U, c, jm);
      float l = a.iso ? (lx + ly) * id2x : lx * id2x + ly * id2y;
      if (DIM == 3) l = l + lux_z * (a.iso ? id2x : id2z);
      dvx = dvx + (a.rhof_one ? mu * l : mu * l / rhof);
    }
    {
      const float lx = dfd(V, ip, c) - dfd(V, c, im);
      const float ly = dfd(V, jp, c) - dfd(V, c, jm);
      float l = a.iso ? (lx + ly) * id2x : lx * id2x + ly * id2y;
      if (DIM == 3) l = l + lvy_z * (a.iso ? id2x : id2z);
      dvy = dvy + (a.rhof_one ? mu * l : mu * l / rhof);
    }
    if (a.has_S) {
      dvx = dvx + (a.rhof_one ? a.Sx[c] : a.Sx[c] / rhof);
      dvy = dvy + (a.rhof_one ? a.Sy[c] : a.Sy[c] / rhof);
      if (DIM == 3) dvz = dvz + (a.rhof_one ? a.Sz[c] : a.Sz[c] / rhof);
    }
    const float gpx = dfd(P, ip, c) * idx;
    const float gpy = dfd(P, jp, c) * idy;
    const float rx = (a.rhof_one ? -gpx : -gpx / rhof) + A * dvx + B * a.dox[c] + (float)a.g[0];
    const float ry = (a.rhof_one ? -gpy : -gpy / rhof) + A * dvy + B * a.doy[c] + (float)a.g[1];
    a.du[c] = dt * rx;
    a.dv[c] = dt * ry;
    a.dox[c] = dvx;
    a.doy[c] = dvy;
    if (DIM == 3) {
      const float gpz = dfd(P, c + sz, c) * idz;
      const float rz = (a.rhof_one ? -gpz : -gpz / rhof) + A * dvz + B * a.doz[c] + (float)a.g[2];
      a.dw[c] = dt * rz;
      a.doz[c] = dvz;
    }
  }
}

// A double as a pair of floats.
struct F2 {
  float hi, lo;
};
__host__ __device__ inline F2 split_d(double x) {
  F2 r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}

// (a_hi + a_lo) * (b_hi + b_lo) as a pair (FMA-exact leading product).
__device__ __forceinline__ F2 mul_pair(float ah, float al, F2 b) {
  F2 r;
  r.hi = ah * b.hi;
  r.lo = fmaf(ah, b.hi, -r.hi) + (ah * b.lo + al * b.hi);
  return r;
}

// Pair sum of pairs.
__device__ __forceinline__ F2 add_pair(F2 a, F2 b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  F2 r;
  r.hi = s;
  r.lo = e + (a.lo + b.lo);
  return r;
}

// One axis term of div(v*) as a pair: ((vA - vB) + (dA - dB)) * id, the leading difference
// error-free.
__device__ __forceinline__ F2 div_term(const DFField& V, const float* d, long long ca, long long cb, F2 id) {
  float s, e;
  two_sum(V.hi[ca], -V.hi[cb], s, e);
  e = e + ((V.lo[ca] - V.lo[cb]) + (d ? d[ca] - d[cb] : 0.0f));
  return mul_pair(s, e, id);
}

// div(v*) at (i, j, k) as a pair, v* = v + dt*rhs (d* = the FP32 increment, or null for div(v)).
template <int DIM>
__device__ __forceinline__ F2 div_df(const Layout& L, const DFField& U, const DFField& V, const DFField& W,
                                     const float* du, const float* dv, const float* dw, const F2* id, int i, int j,
                                     int k) {
  const long long c = L.idx(i, j, kst<DIM>(k));
  F2 r = add_pair(div_term(U, du, c, c - 1, id[0]), div_term(V, dv, c, c - L.sx, id[1]));
  if (DIM == 3) r = add_pair(r, div_term(W, dw, c, c - L.sp, id[2]));
  return r;
}

// ------------------------------------------------------------------------------------
// Correction (mixed): v = v + (dt*rhs - dt grad(phi)/rhof), p = p + phi, on the pairs.
// ------------------------------------------------------------------------------------
struct CorrDFArgs {
  const float *du, *dv, *dw, *phi;
  const float* dphi;  // refinement correction of phi (or null)
  DFFieldW u, v, w, p;
  double id[3];
  int iso;
  double rhof;
};

template <int DIM>
__global__ void __launch_bounds__(256) k_correct_df(Layout L, const StepScalars* __restrict__ sc, CorrDFArgs a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const float f = (float)(sc->dt / a.rhof);
  const float idx = (float)a.id[0];
  const float idy = a.iso ? idx : (float)a.id[1];
  const float idz = a.iso ? idx : (float)a.id[2];
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ncell; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % L.n0);
    const long long r = t / L.n0;
    const int j = 1 + (int)(r % L.n1);
    const int k = 1 + (int)(r / L.n1);
    const long long c = L.idx(i, j, kst<DIM>(k));
    const float ph = a.phi[c];
    const float* q = a.dphi;
    const float qh = q ? q[c] : 0.0f;
    // grad(phi + dphi) by differences of each part
    const float gx = (a.phi[c + 1] - ph) + (q ? q[c + 1] - qh : 0.0f);
    const float gy = (a.phi[c + L.sx] - ph) + (q ? q[c + L.sx] - qh : 0.0f);
    float hi, lo;
    hi = a.u.hi[c]; lo = a.u.lo[c];
    df_add(hi, lo, a.du[c] - gx * idx * f);
    a.u.hi[c] = hi; a.u.lo[c] = lo;
    hi = a.v.hi[c]; lo = a.v.lo[c];
    df_add(hi, lo, a.dv[c] - gy * idy * f);
    a.v.hi[c] = hi; a.v.lo[c] = lo;
    if (DIM == 3) {
      const float gz = (a.phi[c + L.sp] - ph) + (q ? q[c + L.sp] - qh : 0.0f);
      hi = a.w.hi[c]; lo = a.w.lo[c];
      df_add(hi, lo, a.dw[c] - gz * idz * f);
      a.w.hi[c] = hi; a.w.lo[c] = lo;
    }
    hi = a.p.hi[c]; lo = a.p.lo[c];
    df_add(hi, lo, ph);
    if (q) df_add(hi, lo, qh);
    a.p.hi[c] = hi; a.p.lo[c] = lo;
  }
}

// ------------------------------------------------------------------------------------
// Diagnostics (mixed): signed max of div(v) and max(|u|+|v|+|w|) per CTA, folded in FP64
// by k_finalize.
// ------------------------------------------------------------------------------------
struct CheckDFArgs {
  DFField u, v, w;
  F2 idp[3];
  int want_div;
  double* pdiv;
  double* pvel;
  int* nan_flag;
};

template <int DIM>
__global__ void __launch_bounds__(256) k_checks_df(Layout L, CheckDFArgs a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  float md = -INFINITY, mv = 0.0f;
  bool bad = false;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ncell; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % L.n0);
    const long long r = t / L.n0;
    const int j = 1 + (int)(r % L.n1);
    const int k = 1 + (int)(r / L.n1);
    const long long c = L.idx(i, j, kst<DIM>(k));
    float vel = fabsf(a.u.hi[c]) + fabsf(a.v.hi[c]);
    float d = 0.0f;
    if (a.want_div) {
      const F2 dd = div_df<DIM>(L, a.u, a.v, a.w, nullptr, nullptr, nullptr, a.idp, i, j, k);
      d = dd.hi + dd.lo;
    }
    if (DIM == 3) vel = vel + fabsf(a.w.hi[c]);
    if (vel != vel || d != d) bad = true;
    mv = fmaxf(mv, vel);
    md = fmaxf(md, d);
  }
  __shared__ float r1[256], r2[256];
  r1[threadIdx.x] = md;
  r2[threadIdx.x] = mv;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) {
      r1[threadIdx.x] = fmaxf(r1[threadIdx.x], r1[threadIdx.x + h]);
      r2[threadIdx.x] = fmaxf(r2[threadIdx.x], r2[threadIdx.x + h]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.pdiv[blockIdx.x] = (double)r1[0];
    a.pvel[blockIdx.x] = (double)r2[0];
  }
  if (bad) atomicOr(a.nan_flag, 1);
}

// ------------------------------------------------------------------------------------
// Iterative refinement residual: r = b - L_h phi, b = div(v*) rho/dt, in double-float
// arithmetic.  L_h is the 3/5/7-point Laplacian the fast solver inverts exactly (periodic
// axes by their modified wavenumbers, wall axes by the Neumann/Dirichlet tridiagonal),
// applied with phi's ghost cells filled by its boundary rules.
// ------------------------------------------------------------------------------------
struct ResidualArgs {
  DFField u, v, w;
  const float *du, *dv, *dw;
  const float* phi;
  float* r;
  F2 idp[3];
  F2 id2p[3];
};

__device__ __forceinline__ F2 lap_term(const float* f, long long c, long long s, F2 id2) {
  float a, ea, b, eb;
  two_sum(f[c + s], -f[c], a, ea);
  two_sum(f[c], -f[c - s], b, eb);
  float d, ed;
  two_sum(a, -b, d, ed);
  return mul_pair(d, ed + (ea - eb), id2);
}

template <int DIM>
__global__ void __launch_bounds__(256) k_residual_df(Layout L, const StepScalars* __restrict__ sc, ResidualArgs a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const F2 rod = split_d(sc->rho_over_dt);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ncell; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % L.n0);
    const long long rr = t / L.n0;
    const int j = 1 + (int)(rr % L.n1);
    const int k = 1 + (int)(rr / L.n1);
    const long long c = L.idx(i, j, kst<DIM>(k));
    const F2 dv = div_df<DIM>(L, a.u, a.v, a.w, a.du, a.dv, a.dw, a.idp, i, j, k);
    const F2 b = mul_pair(dv.hi, dv.lo, rod);
    F2 lap = add_pair(lap_term(a.phi, c, 1, a.id2p[0]), lap_term(a.phi, c, L.sx, a.id2p[1]));
    if (DIM == 3) lap = add_pair(lap, lap_term(a.phi, c, L.sp, a.id2p[2]));
    float s, e;
    two_sum(b.hi, -lap.hi, s, e);
    a.r[c] = s + (e + (b.lo - lap.lo));
  }
}

// ------------------------------------------------------------------------------------
// Ghost fill of pair fields: the composed face rules of Resolve evaluated on hi + lo in FP64
// (surface cells only), split back into the pair.
// ------------------------------------------------------------------------------------
struct PairSrc {
  const float* hi;
  const float* lo;
  __device__ __forceinline__ double operator()(long long i) const { return (double)hi[i] + (double)lo[i]; }
};

struct GhostDFBatch {
  float* hi[4];
  float* lo[4];
  FieldBC bc[4];
  long long n[4];
};

template <int DIM>
__global__ void __launch_bounds__(256) k_ghost_fill_df(Layout L, GhostDFBatch G) {
  const int q = blockIdx.y;
  const long long total = G.n[q];
  Resolve<double, DIM, PairSrc> R{PairSrc{G.hi[q], G.lo[q]}, L, G.bc[q], 0.0};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    ghost_target<DIM>(L, G.bc[q], t, i, j, k);
    const double v = R.at(i, j, k);
    const long long o = L.idx(i, j, kst<DIM>(k));
    const float h = (float)v;
    G.hi[q][o] = h;
    G.lo[q][o] = (float)(v - (double)h);
  }
}

// FP64 field <-> pair (every stored element).
static __global__ void __launch_bounds__(256) k_split(long long n, const double* __restrict__ src, float* __restrict__ hi,
                                                      float* __restrict__ lo) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const double x = src[t];
    const float h = (float)x;
    hi[t] = h;
    lo[t] = (float)(x - (double)h);
  }
}
static __global__ void __launch_bounds__(256) k_join(long long n, const float* __restrict__ hi, const float* __restrict__ lo,
                                                     double* __restrict__ dst) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    dst[t] = (double)hi[t] + (double)lo[t];
}

}  // namespace fen
