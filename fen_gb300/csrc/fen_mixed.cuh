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

// ------------------------------------------------------------------------------------
// Double-float arithmetic on (hi, lo) pairs of FP32 words (about 48 significant bits).
// Sums use Knuth's two-sum, products the FMA-exact leading product; results are
// renormalised so that |lo| <= ulp(hi)/2.  Only FP32 instructions are issued.
// ------------------------------------------------------------------------------------
struct DF {
  float h, l;
};
__device__ __forceinline__ DF dfv(const DFField& A, long long c) { return DF{A.hi[c], A.lo[c]}; }
__device__ __forceinline__ DF dadd(DF a, DF b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e = e + (a.l + b.l);
  const float h = s + e;
  return DF{h, e - (h - s)};
}
__device__ __forceinline__ DF dsub(DF a, DF b) { return dadd(a, DF{-b.h, -b.l}); }
__device__ __forceinline__ DF dmul(DF a, DF b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  const float h = p + e;
  return DF{h, e - (h - p)};
}
__device__ __forceinline__ DF dsq(DF a) {
  const float p = a.h * a.h;
  float e = fmaf(a.h, a.h, -p);
  e = fmaf(2.0f * a.h, a.l, e);
  const float h = p + e;
  return DF{h, e - (h - p)};
}
// Second difference a(+) - 2 a(0) + a(-) of a pair field.
__device__ __forceinline__ DF d2(DF p, DF c, DF m) {
  float s1, e1, s2, e2;
  two_sum(p.h, m.h, s1, e1);
  two_sum(s1, -2.0f * c.h, s2, e2);
  float e = (e1 + e2) + ((p.l + m.l) - 2.0f * c.l);
  const float h = s2 + e;
  return DF{h, e - (h - s2)};
}

// Unnormalised forms for the intermediate values of the tiled predictor: the same error-free
// leading operations without the closing renormalisation (h = s + e, l = e - (h - s)).  A
// pair (s, e) whose e has not been folded into s represents the same value, and the next
// operation's error-free sum or product takes it as it is: e is at most a few ulp(s) (or,
// after an exact cancellation of the leading words, of the order of the operands' ulp), so
// each result keeps an absolute error of the order of 2^-46 of its operands, as the
// normalised forms do.  Pairs that are stored (v*, dv_o) are normalised first (dnorm).
// About a fifth fewer FP32 instructions in a kernel that is issue-bound once its planes are
// prefetched: channel 512x256x384 predictor 2.24 -> 1.85 ms, 500-step errors unchanged.
#ifndef FEN_DF_LAZY
#define FEN_DF_LAZY 1
#endif
__device__ __forceinline__ DF dnorm(DF a) {
  const float h = a.h + a.l;
  return DF{h, a.l - (h - a.h)};
}
#if FEN_DF_LAZY
__device__ __forceinline__ DF daddq(DF a, DF b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return DF{s, e + (a.l + b.l)};
}
__device__ __forceinline__ DF dsubq(DF a, DF b) { return daddq(a, DF{-b.h, -b.l}); }
__device__ __forceinline__ DF dmulq(DF a, DF b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return DF{p, e};
}
__device__ __forceinline__ DF dsqq(DF a) {
  const float p = a.h * a.h;
  float e = fmaf(a.h, a.h, -p);
  e = fmaf(2.0f * a.h, a.l, e);
  return DF{p, e};
}
__device__ __forceinline__ DF d2q(DF p, DF c, DF m) {
  float s1, e1, s2, e2;
  two_sum(p.h, m.h, s1, e1);
  two_sum(s1, -2.0f * c.h, s2, e2);
  return DF{s2, (e1 + e2) + ((p.l + m.l) - 2.0f * c.l)};
}
#else
__device__ __forceinline__ DF daddq(DF a, DF b) { return dadd(a, b); }
__device__ __forceinline__ DF dsubq(DF a, DF b) { return dsub(a, b); }
__device__ __forceinline__ DF dmulq(DF a, DF b) { return dmul(a, b); }
__device__ __forceinline__ DF dsqq(DF a) { return dsq(a); }
__device__ __forceinline__ DF d2q(DF p, DF c, DF m) { return d2(p, c, m); }
#endif

// ------------------------------------------------------------------------------------
// Predictor (mixed): v* = v + dt * rhs and dv_o, both as pairs.  Every term of
// navier_stokes.f90:140-404 (advection in divergence form, diffusion, body force, pressure
// gradient, AB2) is evaluated in double-float arithmetic and added to v as a pair, so v*
// keeps the state's pair accuracy: FP32 rounding of the increments (about 0.5 |v| per step
// at CFL 0.5) would otherwise random-walk into the solution.
// ------------------------------------------------------------------------------------
struct PredDFArgs {
  DFField u, v, w, p;
  float *du, *dv, *dw;        // v* hi
  float *dul, *dvl, *dwl;     // v* lo
  float *dox, *doy, *doz;     // dv_o hi
  float *doxl, *doyl, *dozl;  // dv_o lo
  const float *Sx, *Sy, *Sz;
  F2 qx, qy, qz;              // 1/(4 delta) per axis
  F2 mx, my, mz;              // mu/(rhof delta^2) per axis
  F2 gx, gy, gz;              // 1/(rhof delta) per axis (pressure gradient)
  F2 irho;                    // 1/rhof
  F2 g[3];                    // body acceleration
  int iso, has_S;
};

template <int DIM>
__global__ void __launch_bounds__(256) k_predictor_df(Layout L, const StepScalars* __restrict__ sc, PredDFArgs a) {
  const long long ncell = (long long)L.n0 * L.n1 * L.n2;
  const DF A = DF{sc->Ap[0], sc->Ap[1]}, B = DF{sc->Bp[0], sc->Bp[1]}, DT = DF{sc->dtp[0], sc->dtp[1]};
  const DF qx = DF{a.qx.hi, a.qx.lo}, qy = DF{a.qy.hi, a.qy.lo}, qz = DF{a.qz.hi, a.qz.lo};
  const DF mx = DF{a.mx.hi, a.mx.lo}, my = DF{a.my.hi, a.my.lo}, mz = DF{a.mz.hi, a.mz.lo};
  const long long sy = L.sx, sz = L.sp;
  const DFField U = a.u, V = a.v, W = a.w, P = a.p;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j, k = 1 + cw.k;
    const long long c = L.idx(i, j, kst<DIM>(k));
    const DF uc = dfv(U, c), uip = dfv(U, c + 1), uim = dfv(U, c - 1), ujp = dfv(U, c + sy), ujm = dfv(U, c - sy);
    const DF vc = dfv(V, c), vip = dfv(V, c + 1), vim = dfv(V, c - 1), vjp = dfv(V, c + sy), vjm = dfv(V, c - sy);
    // advection: products at faces and edges (1/4 folded into q); the (i+1/2, j+1/2) edge
    // product is shared by the u and v equations
    const DF uv_pp = dmul(dadd(ujp, uc), dadd(vip, vc));
    const DF uv_pm = dmul(dadd(uc, ujm), dadd(dfv(V, c + 1 - sy), vjm));
    const DF uv_mp = dmul(dadd(vc, vim), dadd(dfv(U, c - 1 + sy), uim));
    DF ax = dmul(dsub(dsq(dadd(uip, uc)), dsq(dadd(uc, uim))), qx);
    ax = dadd(ax, dmul(dsub(uv_pp, uv_pm), qy));
    DF ay = dmul(dsub(uv_pp, uv_mp), qx);
    ay = dadd(ay, dmul(dsub(dsq(dadd(vjp, vc)), dsq(dadd(vc, vjm))), qy));
    DF lu = dmul(d2(uip, uc, uim), mx), lv = dmul(d2(vip, vc, vim), mx);
    lu = dadd(lu, dmul(d2(ujp, uc, ujm), my));
    lv = dadd(lv, dmul(d2(vjp, vc, vjm), my));
    DF dz = DF{0.f, 0.f}, wc = DF{0.f, 0.f};
    if (DIM == 3) {
      wc = dfv(W, c);
      const DF wip = dfv(W, c + 1), wim = dfv(W, c - 1), wjp = dfv(W, c + sy), wjm = dfv(W, c - sy);
      const DF wkp = dfv(W, c + sz), wkm = dfv(W, c - sz);
      const DF ukp = dfv(U, c + sz), ukm = dfv(U, c - sz), vkp = dfv(V, c + sz), vkm = dfv(V, c - sz);
      const DF uw_pp = dmul(dadd(ukp, uc), dadd(wip, wc));
      const DF uw_pm = dmul(dadd(uc, ukm), dadd(dfv(W, c + 1 - sz), wkm));
      const DF uw_mp = dmul(dadd(wc, wim), dadd(uim, dfv(U, c - 1 + sz)));
      const DF vw_pp = dmul(dadd(vkp, vc), dadd(wjp, wc));
      const DF vw_pm = dmul(dadd(vc, vkm), dadd(dfv(W, c + sy - sz), wkm));
      const DF vw_mp = dmul(dadd(wc, wjm), dadd(vjm, dfv(V, c - sy + sz)));
      ax = dadd(ax, dmul(dsub(uw_pp, uw_pm), qz));
      ay = dadd(ay, dmul(dsub(vw_pp, vw_pm), qz));
      DF az = dmul(dsub(uw_pp, uw_mp), qx);
      az = dadd(az, dmul(dsub(vw_pp, vw_mp), qy));
      az = dadd(az, dmul(dsub(dsq(dadd(wc, wkp)), dsq(dadd(wc, wkm))), qz));
      lu = dadd(lu, dmul(d2(ukp, uc, ukm), mz));
      lv = dadd(lv, dmul(d2(vkp, vc, vkm), mz));
      DF lw = dmul(d2(wip, wc, wim), mx);
      lw = dadd(lw, dmul(d2(wjp, wc, wjm), my));
      lw = dadd(lw, dmul(d2(wkp, wc, wkm), mz));
      dz = dsub(lw, az);
    }
    DF dx = dsub(lu, ax), dy = dsub(lv, ay);
    if (a.has_S) {
      const DF ir = DF{a.irho.hi, a.irho.lo};
      dx = dadd(dx, dmul(DF{a.Sx[c], 0.f}, ir));
      dy = dadd(dy, dmul(DF{a.Sy[c], 0.f}, ir));
      if (DIM == 3) dz = dadd(dz, dmul(DF{a.Sz[c], 0.f}, ir));
    }
    // AB2 with the pressure gradient (fields.f90:55-58, navier_stokes.f90:169-198)
    const DF pc = dfv(P, c);
    DF rx = dsub(DF{a.g[0].hi, a.g[0].lo}, dmul(dsub(dfv(P, c + 1), pc), DF{a.gx.hi, a.gx.lo}));
    DF ry = dsub(DF{a.g[1].hi, a.g[1].lo}, dmul(dsub(dfv(P, c + sy), pc), DF{a.gy.hi, a.gy.lo}));
    rx = dadd(rx, dadd(dmul(A, dx), dmul(B, DF{a.dox[c], a.doxl[c]})));
    ry = dadd(ry, dadd(dmul(A, dy), dmul(B, DF{a.doy[c], a.doyl[c]})));
    const DF ix = dadd(uc, dmul(DT, rx)), iy = dadd(vc, dmul(DT, ry));  // v* pairs
    a.du[c] = ix.h; a.dul[c] = ix.l;
    a.dv[c] = iy.h; a.dvl[c] = iy.l;
    a.dox[c] = dx.h; a.doxl[c] = dx.l;
    a.doy[c] = dy.h; a.doyl[c] = dy.l;
    if (DIM == 3) {
      DF rz = dsub(DF{a.g[2].hi, a.g[2].lo}, dmul(dsub(dfv(P, c + sz), pc), DF{a.gz.hi, a.gz.lo}));
      rz = dadd(rz, dadd(dmul(A, dz), dmul(B, DF{a.doz[c], a.dozl[c]})));
      const DF iz = dadd(wc, dmul(DT, rz));
      a.dw[c] = iz.h; a.dwl[c] = iz.l;
      a.doz[c] = dz.h; a.dozl[c] = dz.l;
    }
  }
}

// ------------------------------------------------------------------------------------
// Tiled double-float predictor (3D): the face and edge products are formed once per face
// and shared (the - values from the left lane by shuffle, from the row below through shared
// memory and from the previous k in registers), as in the FP64 k_predictor_tile.  Each sum
// is formed upper + lower, so the sharing cell and the per-cell formula see the same pairs.
// ------------------------------------------------------------------------------------
#ifndef FEN_DFTILE_TY
#define FEN_DFTILE_TY 4
#endif
#ifndef FEN_DFTILE_TZ
#define FEN_DFTILE_TZ 16
#endif
constexpr int kDTX = 32, kDTY = FEN_DFTILE_TY, kDTZ = FEN_DFTILE_TZ;
// Planes ahead of the z-walk whose pair-field lines are prefetched (0: none).
#ifndef FEN_DFTILE_PF
#define FEN_DFTILE_PF 2
#endif
#ifndef FEN_DFTILE_PF_L1
#define FEN_DFTILE_PF_L1 0
#endif
__device__ __forceinline__ void pf_line(const float* p) {
#if FEN_DFTILE_PF_L1
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
#else
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
#endif
}

// Products on the + sides of cell c: fuu (i+1/2), fvv (j+1/2), fww (k+1/2), euv (i+1/2, j+1/2),
// euw (i+1/2, k+1/2), evw (j+1/2, k+1/2) (the 1/4 is folded into q).
__device__ __forceinline__ void dflux6(const DFField& U, const DFField& V, const DFField& W, long long c, long long sy,
                                       long long sz, DF& fuu, DF& fvv, DF& fww, DF& euv, DF& euw, DF& evw) {
  const DF uc = dfv(U, c), vc = dfv(V, c), wc = dfv(W, c);
  fuu = dsqq(daddq(dfv(U, c + 1), uc));
  fvv = dsqq(daddq(dfv(V, c + sy), vc));
  fww = dsqq(daddq(dfv(W, c + sz), wc));
  euv = dmulq(daddq(dfv(U, c + sy), uc), daddq(dfv(V, c + 1), vc));
  euw = dmulq(daddq(dfv(U, c + sz), uc), daddq(dfv(W, c + 1), wc));
  evw = dmulq(daddq(dfv(V, c + sz), vc), daddq(dfv(W, c + sy), wc));
}
// The three products a cell's +x neighbour needs (fuu, euv, euw of cell c).
__device__ __forceinline__ void dflux_x(const DFField& U, const DFField& V, const DFField& W, long long c, long long sy,
                                        long long sz, DF& fuu, DF& euv, DF& euw) {
  const DF uc = dfv(U, c);
  fuu = dsqq(daddq(dfv(U, c + 1), uc));
  euv = dmulq(daddq(dfv(U, c + sy), uc), daddq(dfv(V, c + 1), dfv(V, c)));
  euw = dmulq(daddq(dfv(U, c + sz), uc), daddq(dfv(W, c + 1), dfv(W, c)));
}
// ... its +y neighbour needs (euv, fvv, evw of cell c).
__device__ __forceinline__ void dflux_y(const DFField& U, const DFField& V, const DFField& W, long long c, long long sy,
                                        long long sz, DF& euv, DF& fvv, DF& evw) {
  const DF vc = dfv(V, c);
  fvv = dsqq(daddq(dfv(V, c + sy), vc));
  euv = dmulq(daddq(dfv(U, c + sy), dfv(U, c)), daddq(dfv(V, c + 1), vc));
  evw = dmulq(daddq(dfv(V, c + sz), vc), daddq(dfv(W, c + sy), dfv(W, c)));
}
// ... its +z neighbour needs (euw, evw, fww of cell c).
__device__ __forceinline__ void dflux_z(const DFField& U, const DFField& V, const DFField& W, long long c, long long sy,
                                        long long sz, DF& euw, DF& evw, DF& fww) {
  const DF wc = dfv(W, c);
  fww = dsqq(daddq(dfv(W, c + sz), wc));
  euw = dmulq(daddq(dfv(U, c + sz), dfv(U, c)), daddq(dfv(W, c + 1), wc));
  evw = dmulq(daddq(dfv(V, c + sz), dfv(V, c)), daddq(dfv(W, c + sy), wc));
}
__device__ __forceinline__ DF shfl_up_df(DF v) {
  return DF{__shfl_up_sync(0xffffffffu, v.h, 1), __shfl_up_sync(0xffffffffu, v.l, 1)};
}

// Tiles of 32 x 4 cells compiled for 6 resident 128-thread CTAs per SM (80 registers, no
// spills): 24 warps hide the loads better than the 16 of the compiler's 128-register choice
// (channel: 2.82 -> 2.36 ms with 32 x 8 tiles at 3 CTAs, 2.30 ms with 32 x 4 at 6); 64
// registers spill, and z-walks of 32 planes are slower.
#ifndef FEN_DFTILE_MINB
#define FEN_DFTILE_MINB 6
#endif
static __global__ void __launch_bounds__(kDTX * kDTY, FEN_DFTILE_MINB) k_predictor_df_tile(Layout L, const StepScalars* __restrict__ sc,
                                                                        PredDFArgs a) {
  __shared__ DF sh[2][3][kDTY][kDTX];
  __shared__ DF xsh[2][3][kDTY];  // x-minus products of each row's first lane
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = 1 + blockIdx.x * kDTX + tx, j0 = 1 + blockIdx.y * kDTY + ty;
  const bool act = (i0 <= L.n0) && (j0 <= L.n1);
  const int i = min(i0, L.n0), j = min(j0, L.n1);
  const int k0 = 1 + blockIdx.z * kDTZ, k1 = min(L.n2, k0 + kDTZ - 1);
  const DF A = DF{sc->Ap[0], sc->Ap[1]}, B = DF{sc->Bp[0], sc->Bp[1]}, DT = DF{sc->dtp[0], sc->dtp[1]};
  const DF qx = DF{a.qx.hi, a.qx.lo}, qy = DF{a.qy.hi, a.qy.lo}, qz = DF{a.qz.hi, a.qz.lo};
  const DF mx = DF{a.mx.hi, a.mx.lo}, my = DF{a.my.hi, a.my.lo}, mz = DF{a.mz.hi, a.mz.lo};
  const long long sy = L.sx, sz = L.sp;
  const DFField U = a.u, V = a.v, W = a.w, P = a.p;
  // z-minus products of the first k of the chunk
  DF puw, pvw, pww;
  dflux_z(U, V, W, L.idx(i, j, k0) - sz, sy, sz, puw, pvw, pww);
  int buf = 0;
  for (int k = k0; k <= k1; ++k, buf ^= 1) {
    const long long c = L.idx(i, j, k);
    DF fuu, fvv, fww, euv, euw, evw;
    dflux6(U, V, W, c, sy, sz, fuu, fvv, fww, euv, euw, evw);
    // x-minus: the lane to the left; for the first lane of every row, lanes 0 .. kDTY-1 of
    // row 0 form the products at i - 1 (one divergent pass per tile instead of one per row)
    DF xuu = shfl_up_df(fuu), xuv = shfl_up_df(euv), xuw = shfl_up_df(euw);
    if (ty == 0 && tx < kDTY) {
      const long long cx = L.idx(blockIdx.x * kDTX, min(1 + (int)blockIdx.y * kDTY + tx, L.n1), k);
      DF a0, a1, a2;
      dflux_x(U, V, W, cx, sy, sz, a0, a1, a2);
      xsh[buf][0][tx] = a0;
      xsh[buf][1][tx] = a1;
      xsh[buf][2][tx] = a2;
    }
    // y-minus: the row below through shared memory; row 0 forms its own
    sh[buf][0][ty][tx] = euv;
    sh[buf][1][ty][tx] = fvv;
    sh[buf][2][ty][tx] = evw;
    __syncthreads();
    if (tx == 0) {
      xuu = xsh[buf][0][ty];
      xuv = xsh[buf][1][ty];
      xuw = xsh[buf][2][ty];
    }
    DF yuv, yvv, yvw;
    if (ty > 0) {
      yuv = sh[buf][0][ty - 1][tx];
      yvv = sh[buf][1][ty - 1][tx];
      yvw = sh[buf][2][ty - 1][tx];
    } else {
      dflux_y(U, V, W, c - sy, sy, sz, yuv, yvv, yvw);
    }
    DF ax = dmulq(dsubq(fuu, xuu), qx);
    ax = daddq(ax, dmulq(dsubq(euv, yuv), qy));
    ax = daddq(ax, dmulq(dsubq(euw, puw), qz));
    DF ay = dmulq(dsubq(euv, xuv), qx);
    ay = daddq(ay, dmulq(dsubq(fvv, yvv), qy));
    ay = daddq(ay, dmulq(dsubq(evw, pvw), qz));
    DF az = dmulq(dsubq(euw, xuw), qx);
    az = daddq(az, dmulq(dsubq(evw, yvw), qy));
    az = daddq(az, dmulq(dsubq(fww, pww), qz));
    puw = euw;
    pvw = evw;
    pww = fww;
    if (act) {
      const DF uc = dfv(U, c), vc = dfv(V, c), wc = dfv(W, c);
      DF lu = dmulq(d2q(dfv(U, c + 1), uc, dfv(U, c - 1)), mx);
      lu = daddq(lu, dmulq(d2q(dfv(U, c + sy), uc, dfv(U, c - sy)), my));
      lu = daddq(lu, dmulq(d2q(dfv(U, c + sz), uc, dfv(U, c - sz)), mz));
      DF lv = dmulq(d2q(dfv(V, c + 1), vc, dfv(V, c - 1)), mx);
      lv = daddq(lv, dmulq(d2q(dfv(V, c + sy), vc, dfv(V, c - sy)), my));
      lv = daddq(lv, dmulq(d2q(dfv(V, c + sz), vc, dfv(V, c - sz)), mz));
      DF lw = dmulq(d2q(dfv(W, c + 1), wc, dfv(W, c - 1)), mx);
      lw = daddq(lw, dmulq(d2q(dfv(W, c + sy), wc, dfv(W, c - sy)), my));
      lw = daddq(lw, dmulq(d2q(dfv(W, c + sz), wc, dfv(W, c - sz)), mz));
      DF dx = dsubq(lu, ax), dy = dsubq(lv, ay), dz = dsubq(lw, az);
      if (a.has_S) {
        const DF ir = DF{a.irho.hi, a.irho.lo};
        dx = daddq(dx, dmulq(DF{a.Sx[c], 0.f}, ir));
        dy = daddq(dy, dmulq(DF{a.Sy[c], 0.f}, ir));
        dz = daddq(dz, dmulq(DF{a.Sz[c], 0.f}, ir));
      }
      // AB2 with the pressure gradient (fields.f90:55-58, navier_stokes.f90:169-198)
      const DF pc = dfv(P, c);
      DF rx = dsubq(DF{a.g[0].hi, a.g[0].lo}, dmulq(dsubq(dfv(P, c + 1), pc), DF{a.gx.hi, a.gx.lo}));
      DF ry = dsubq(DF{a.g[1].hi, a.g[1].lo}, dmulq(dsubq(dfv(P, c + sy), pc), DF{a.gy.hi, a.gy.lo}));
      DF rz = dsubq(DF{a.g[2].hi, a.g[2].lo}, dmulq(dsubq(dfv(P, c + sz), pc), DF{a.gz.hi, a.gz.lo}));
      rx = daddq(rx, daddq(dmulq(A, dx), dmulq(B, DF{a.dox[c], a.doxl[c]})));
      ry = daddq(ry, daddq(dmulq(A, dy), dmulq(B, DF{a.doy[c], a.doyl[c]})));
      rz = daddq(rz, daddq(dmulq(A, dz), dmulq(B, DF{a.doz[c], a.dozl[c]})));
      // v* = v + dt rhs as a pair; the stored pairs normalised
      const DF ix = dnorm(daddq(uc, dmulq(DT, rx))), iy = dnorm(daddq(vc, dmulq(DT, ry))), iz = dnorm(daddq(wc, dmulq(DT, rz)));
      dx = dnorm(dx);
      dy = dnorm(dy);
      dz = dnorm(dz);
      a.du[c] = ix.h; a.dul[c] = ix.l;
      a.dv[c] = iy.h; a.dvl[c] = iy.l;
      a.dw[c] = iz.h; a.dwl[c] = iz.l;
      a.dox[c] = dx.h; a.doxl[c] = dx.l;
      a.doy[c] = dy.h; a.doyl[c] = dy.l;
      a.doz[c] = dz.h; a.dozl[c] = dz.l;
    }
#if FEN_DFTILE_PF > 0
    {
      // the pair fields FEN_DFTILE_PF planes ahead of the next one (the last plane read is
      // n2 + 1) and the next plane of dv_o, requested now so the walk does not wait on them
      const long long cp = L.idx(i, j, min(k + 1 + FEN_DFTILE_PF, L.n2 + 1));
      const long long cn = L.idx(i, j, min(k + 1, L.n2));
      pf_line(U.hi + cp); pf_line(U.lo + cp); pf_line(V.hi + cp); pf_line(V.lo + cp);
      pf_line(W.hi + cp); pf_line(W.lo + cp); pf_line(P.hi + cp); pf_line(P.lo + cp);
      pf_line(a.dox + cn); pf_line(a.doxl + cn); pf_line(a.doy + cn); pf_line(a.doyl + cn);
      pf_line(a.doz + cn); pf_line(a.dozl + cn);
    }
#endif
  }
}

// One axis term of div(v*) as a pair: ((vA - vB) + (dA - dB)) * id with v* = v + d, both
// differences taken error-free on the pairs (d may be null: div(v)).
__device__ __forceinline__ F2 div_term(const DFField& V, const float* d, const float* dl, long long ca, long long cb,
                                       F2 id) {
  float s, e;
  two_sum(V.hi[ca], -V.hi[cb], s, e);
  e = e + (V.lo[ca] - V.lo[cb]);
  if (d) {
    float s2, e2;
    two_sum(d[ca], -d[cb], s2, e2);
    if (dl) e2 = e2 + (dl[ca] - dl[cb]);
    float s3, e3;
    two_sum(s, s2, s3, e3);
    s = s3;
    e = e3 + (e + e2);
  }
  return mul_pair(s, e, id);
}

// div at cell index c (div_df: at (i, j, k)) of the pair field V plus, when given, a second
// pair field (d, dl).
template <int DIM>
__device__ __forceinline__ F2 div_df_at(const Layout& L, const DFField& U, const DFField& V, const DFField& W,
                                        const float* du, const float* dv, const float* dw, const float* dul,
                                        const float* dvl, const float* dwl, const F2* id, long long c) {
  F2 r = add_pair(div_term(U, du, dul, c, c - 1, id[0]), div_term(V, dv, dvl, c, c - L.sx, id[1]));
  if (DIM == 3) r = add_pair(r, div_term(W, dw, dwl, c, c - L.sp, id[2]));
  return r;
}
template <int DIM>
__device__ __forceinline__ F2 div_df(const Layout& L, const DFField& U, const DFField& V, const DFField& W,
                                     const float* du, const float* dv, const float* dw, const float* dul,
                                     const float* dvl, const float* dwl, const F2* id, int i, int j, int k) {
  return div_df_at<DIM>(L, U, V, W, du, dv, dw, dul, dvl, dwl, id, L.idx(i, j, kst<DIM>(k)));
}

// ------------------------------------------------------------------------------------
// Correction (mixed): v = v + (dt*rhs - dt grad(phi)/rhof), p = p + phi, on the pairs.
// ------------------------------------------------------------------------------------
struct CorrDFArgs {
  const float *du, *dv, *dw, *phi;  // v* hi
  const float *dul, *dvl, *dwl;     // v* lo
  const float* dphi;  // refinement correction of phi (or null)
  int dphi_mean;      // subtract the mean of dphi (sc->mean) in the pressure update
  int phi_mean;       // subtract the mean of phi (sc->mean_phi) in the pressure update
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
  // the means of phi and dphi leave their gradients unchanged; they are removed only where
  // they enter p (the mean removal of the Poisson solve, poisson.f90:491-503, fused here)
  const float qm = a.dphi_mean ? (float)sc->mean : 0.0f;
  const float pm = a.phi_mean ? (float)sc->mean_phi : 0.0f;
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j, k = 1 + cw.k;
    const long long c = L.idx(i, j, kst<DIM>(k));
    const float ph = a.phi[c];
    const float* q = a.dphi;
    const float qh = q ? q[c] : 0.0f;
    // grad(phi + dphi) by differences of each part
    const float gx = (a.phi[c + 1] - ph) + (q ? q[c + 1] - qh : 0.0f);
    const float gy = (a.phi[c + L.sx] - ph) + (q ? q[c + L.sx] - qh : 0.0f);
    // v = v* - dt grad(phi)/rhof, summed as pairs
    {
      DF x = DF{a.du[c], a.dul[c]};  // v*
      x = dadd(x, DF{-gx * idx * f, 0.f});
      a.u.hi[c] = x.h; a.u.lo[c] = x.l;
      DF y = DF{a.dv[c], a.dvl[c]};
      y = dadd(y, DF{-gy * idy * f, 0.f});
      a.v.hi[c] = y.h; a.v.lo[c] = y.l;
      if (DIM == 3) {
        const float gz = (a.phi[c + L.sp] - ph) + (q ? q[c + L.sp] - qh : 0.0f);
        DF z = DF{a.dw[c], a.dwl[c]};
        z = dadd(z, DF{-gz * idz * f, 0.f});
        a.w.hi[c] = z.h; a.w.lo[c] = z.l;
      }
    }
    float hi, lo;
    hi = a.p.hi[c]; lo = a.p.lo[c];
    df_add(hi, lo, a.phi_mean ? ph - pm : ph);
    if (q) df_add(hi, lo, qh - qm);
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
  CellWalk cw(L, blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
  for (long long t = cw.t0; t < ncell; t += cw.stride, cw.next(L)) {
    const int i = 1 + cw.i, j = 1 + cw.j, k = 1 + cw.k;
    const long long c = L.idx(i, j, kst<DIM>(k));
    float vel = fabsf(a.u.hi[c]) + fabsf(a.v.hi[c]);
    float d = 0.0f;
    if (a.want_div) {
      const F2 dd = div_df<DIM>(L, a.u, a.v, a.w, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, a.idp, i, j, k);
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
// Iterative refinement residual r = b - L_h phi, b = div(v*) rho/dt, in double-float
// arithmetic (formed in the first transform's load, LD_RESID).  L_h is the 3/5/7-point
// Laplacian the fast solver inverts exactly (periodic axes by their modified wavenumbers,
// wall axes by the Neumann/Dirichlet tridiagonal), applied with phi's ghost cells filled by
// its boundary rules.  One axis' term (f[c+s] - 2 f[c] + f[c-s]) / delta^2:
// ------------------------------------------------------------------------------------
// formed as (f[c+s] + f[c-s]) - 2 f[c] by two error-free sums (2 f[c] is exact), the second
// difference to the rounding of its error term (13 FP32 instructions; the two one-sided
// differences and their difference took 20, refinement stage 2.02 -> 1.98 ms on the channel).
__device__ __forceinline__ F2 lap_term(const float* f, long long c, long long s, F2 id2) {
  float s1, e1, s2, e2;
  two_sum(f[c + s], f[c - s], s1, e1);
  two_sum(s1, -2.0f * f[c], s2, e2);
  return mul_pair(s2, e1 + e2, id2);
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
  GhostDiv gd[4];
  int low[4];  // 1: only the ghosts of v* the divergence reads (ghost_low_target)
};

template <int DIM>
__global__ void __launch_bounds__(256) k_ghost_fill_df(Layout L, GhostDFBatch G) {
  const int q = blockIdx.y;
  const long long total = G.n[q];
  Resolve<double, DIM, PairSrc> R{PairSrc{G.hi[q], G.lo[q]}, L, G.bc[q], 0.0};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    if (G.low[q]) ghost_low_target(L, G.bc[q], t, i, j, k);
    else if (G.gd[q].ok) ghost_target_fast<DIM>(L, G.bc[q], G.gd[q], t, i, j, k);
    else ghost_target<DIM>(L, G.bc[q], t, i, j, k);
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
