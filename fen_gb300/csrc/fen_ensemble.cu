// Batched ensemble of independent 2D periodic runs in one persistent launch.
//
// FEN advances one grid per program (navier_stokes_solver, navier_stokes.f90:50-136, with
// the pp Poisson solver, poisson.f90:416-505).  Here hundreds of 2D periodic runs of uneven
// sizes N x N advance together in FP32 (reductions in FP64) inside ONE kernel launch:
//
//  * The launch is persistent: clusters of 8 CTAs (one CTA per SM) take "packs" from a
//    global counter.  A pack holds 8/G runs of one size N; each run lives on G CTAs of the
//    cluster, every CTA holding N/G consecutive rows of u, v, p (plus one ghost row above
//    and below) in shared memory for all the steps of the launch.  HBM is touched only to
//    load and store the state once per launch and to stream dv_o (the AB2 history) once
//    per step.
//  * Inside a run, CTAs exchange data through distributed shared memory and synchronise
//    with the hardware cluster barrier (barrier.cluster), which cannot deadlock: all CTAs
//    of a cluster are co-scheduled and every CTA executes the same barrier sequence.
//  * Per step: predictor (advection, diffusion, forcing, AB2, pressure gradient) ->
//    divergence -> r2c FFT along x per row -> all-to-all of column blocks -> complex FFT
//    along y, divide by the modified wavenumbers, inverse FFT -> all-to-all back -> c2r
//    along x -> mean removal (FP64) -> correction, p update, max|u|+|v| (for the next dt)
//    -> ghost rows from the neighbouring CTAs.  Five cluster barriers per step.
//  * G (rows per CTA = N/G, the tile shape) is picked per N by the autotuner below, among
//    the G that fit the shared-memory budget.
//
// The time step follows FEN's constant-CFL update (navier_stokes.f90:680-696):
// dt_o = dt; dt = min(CFL delta / maxvel, dt_visc), capped at 1.1 dt_o; A = 1 + dt/(2 dt_o),
// B = -dt/(2 dt_o).  Density is 1.  The forcing is S_x = amp sin(kf y) at the u points.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fen_gpu.h"
#include "fen_fft.cuh"

namespace cg = cooperative_groups;
using namespace fen;

int fen_internal_fail(int code, const char* msg);

namespace fen {
namespace ens {

#ifndef FEN_ENS_CLUSTER
#define FEN_ENS_CLUSTER 8
#endif
constexpr int kCl = FEN_ENS_CLUSTER;   // CTAs per cluster (above 8: non-portable cluster size)
// 1: the SMs that kCl-CTA clusters leave idle run a second launch of 4-CTA clusters
#ifndef FEN_ENS_SPLIT
#define FEN_ENS_SPLIT 1
#endif
// Cells given to the 4-CTA launch, in percent of its SMs' proportional share (the small
// runs it takes cost more per cell; fen_ensemble_tune picks among 60..100 per device).  On the
// bench ensemble (512 runs, N in 64..256): 60: 34.0, 80: 36.7, 100: 32.6, 120: 28.3 Gcell-steps/s.
#ifndef FEN_ENS_SHARE
#define FEN_ENS_SHARE 80
#endif
// Elements per thread of the Poisson all-to-alls in the backward sweep's adjoint steps and
// recomputed forward steps (register pressure of the backward kernel, which carries both)
#ifndef FEN_ENS_ADJ_EPT
#define FEN_ENS_ADJ_EPT 4
#endif
#ifndef FEN_ENS_REC_EPT
#define FEN_ENS_REC_EPT 10
#endif
constexpr size_t kSmemLimit = 232448;  // opt-in dynamic shared memory per CTA (227 KB)
constexpr size_t kSmemReserve = 1024;  // static shared memory of the kernel + slack

// Division by a run-time constant: q = umulhi(n, m) with m = floor(2^32/d) + 1 is exact
// for n * d < 2^32 (all indices here are below 2^16).
struct FDiv {
  unsigned d, m;
};
__host__ __device__ inline FDiv make_fdiv(unsigned d) {
  FDiv f;
  f.d = d;
  f.m = (d > 1) ? (unsigned)(0x100000000ull / d) + 1u : 0u;
  return f;
}
__device__ __forceinline__ int fdiv(int n, FDiv f) { return f.d > 1 ? (int)__umulhi((unsigned)n, f.m) : n; }

// One grid size N of the ensemble.
struct ClassDesc {
  int N, G, M, SR, C, buf;  // rows per CTA M = N/G; spectrum row SR = N/2+1; column block C; buffer size (float2)
  FDiv fN, fSR, fC, fM, fNP;  // division by N, SR, C, M and the packing pairs N/4 + 1
  int tabs;                   // 1: tables copied into shared memory (when they fit), 0: read from global
  FFTPlan px, py;           // complex FFT lengths N/2 (x, real packing) and N (y)
  const float2* twx;        // exp(-2 pi i m/(N/2)), m < N/2
  const float2* twn;        // exp(-2 pi i k/N), k <= N/2
  const float2* twy;        // exp(-2 pi i m/N), m < N
  const float* lamx;        // 2 (cos(2 pi k/N) - 1)/delta^2, k <= N/2
  const float* lamy;        // same, k < N
  const float* force;       // amp sin(kf (j + 1/2) delta), j < N (u points)
  float idx, id2, inv_nn;   // 1/delta, 1/delta^2, 1/N^2
  double delta;
};

struct RunScal {
  double dt, dt_o, t, maxvel, nu, dt_visc, ke, maxdiv;
  int nan, pad[3];
};

struct Pack {
  int cls, nruns, first, pad;  // runs run_list[first .. first + nruns)
};

struct EnsArgs {
  const ClassDesc* cls;
  const Pack* packs;
  int npacks;
  const int* run_list;
  const long long* run_off;  // float offset of each run's state (u, v, p, dvo_x, dvo_y, N^2 each)
  float* state;
  RunScal* scal;
  int* counter;
  int nsteps;
  double cfl;
  // forward/adjoint pair (mode 1: forward with checkpoints, mode 2: backward sweep)
  int mode;                  // 0 advance, 1 forward with checkpoints, 2 backward
  int every, nseg;           // checkpoint interval, segments
  float* abuf;               // per-run adjoint storage, see AdjLayout
  const long long* aoff;     // float offset of each run's block in abuf
  double* rec;               // per run: nsteps x (dt, dt_o)
};

// Per-run adjoint storage (floats, N2 = N*N): checkpoints nseg x (u, v, p, dvo_x, dvo_y),
// the step inputs of one segment every x (u, v), a dv_o scratch for the recomputation
// (u, v), and the adjoint state (u^, v^, p^, dv_o^x, dv_o^y).
struct AdjLayout {
  long long ck, seg, dvo, adj;
  __host__ __device__ AdjLayout(long long N2, int nseg, int every) {
    ck = 0;
    seg = ck + (long long)nseg * 5 * N2;
    dvo = seg + (long long)every * 2 * N2;
    adj = dvo + 2 * N2;
  }
  __host__ __device__ static long long size(long long N2, int nseg, int every) { return AdjLayout(N2, nseg, every).adj + 5 * N2; }
};

__host__ __device__ inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

// Shared-memory footprint of one CTA for grid size N on G CTAs (bytes, dynamic part):
// u, v, p rows with one ghost row each side; three work buffers; the transform twiddles,
// modified wavenumbers and forcing of this N; eight FP64 reduction slots.
__host__ __device__ inline int tw_count(int N) { return round_up(N / 2 + (N / 2 + 1) + N, 2); }
__host__ __device__ inline int tab_count(int N, int G) { return round_up((N / 2 + 1) + N + N / G, 4); }
__host__ __device__ inline size_t smem_bytes(int N, int G, int* buf_out = nullptr, bool tables = false) {
  const int M = N / G, SR = N / 2 + 1, C = (SR + G - 1) / G;
  const int buf = round_up(M * SR > N * C ? M * SR : N * C, 2);
  if (buf_out) *buf_out = buf;
  const size_t fields = (size_t)round_up(3 * (M + 2) * N, 4) * sizeof(float);
  const size_t tabs = tables ? (size_t)tw_count(N) * sizeof(float2) + (size_t)tab_count(N, G) * sizeof(float) : 0;
  return fields + (size_t)3 * buf * sizeof(float2) + tabs + 8 * sizeof(double);
}

struct Carve {
  float *u, *v, *p;
  float2 *X, *Y, *Z;
  float2 *twx, *twn, *twy;
  float *lamx, *lamy, *force;
  double* red;
};

__device__ inline Carve carve(unsigned char* s, const ClassDesc& D) {
  Carve c;
  const int N = D.N, rows = (D.M + 2) * N;
  c.u = reinterpret_cast<float*>(s);
  c.v = c.u + rows;
  c.p = c.v + rows;
  float2* b = reinterpret_cast<float2*>(s + (size_t)round_up(3 * rows, 4) * sizeof(float));
  c.X = b;
  c.Y = b + D.buf;
  c.Z = b + 2 * D.buf;
  if (D.tabs) {
    c.twx = b + 3 * D.buf;
    c.twn = c.twx + N / 2;
    c.twy = c.twn + (N / 2 + 1);
    c.lamx = reinterpret_cast<float*>(c.twx + tw_count(N));
    c.lamy = c.lamx + (N / 2 + 1);
    c.force = c.lamy + N;
    c.red = reinterpret_cast<double*>(c.lamx + tab_count(N, D.G));
  } else {  // tables stay in global memory (generic pointers; read through L1)
    c.twx = const_cast<float2*>(D.twx);
    c.twn = const_cast<float2*>(D.twn);
    c.twy = const_cast<float2*>(D.twy);
    c.lamx = const_cast<float*>(D.lamx);
    c.lamy = const_cast<float*>(D.lamy);
    c.force = nullptr;  // set per CTA from D.force + r M
    c.red = reinterpret_cast<double*>(b + 3 * D.buf);
  }
  return c;
}

template <int NT>
__device__ inline double block_sum(double v, double* scratch) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) scratch[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (l < NT / 32) ? scratch[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

template <int NT>
__device__ inline float block_max(float v, float* scratch) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) scratch[w] = v;
  __syncthreads();
  float r = -INFINITY;
  if (w == 0) {
    r = (l < NT / 32) ? scratch[l] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) r = fmaxf(r, __shfl_down_sync(0xffffffffu, r, o));
  }
  return r;
}

__device__ inline const double2* tw64(const float2* p) { return reinterpret_cast<const double2*>(p); }

// Twiddle constants of the in-register radix-8/16 DFTs: cos(2 pi m/16), m = 0..15.
__device__ __forceinline__ float cos16(int m) {
  switch (m & 15) {
    case 0: return 1.0f;
    case 1: case 15: return 0.92387953251128674f;
    case 2: case 14: return 0.70710678118654752f;
    case 3: case 13: return 0.38268343236508977f;
    case 4: case 12: return 0.0f;
    case 5: case 11: return -0.38268343236508977f;
    case 6: case 10: return -0.70710678118654752f;
    default: return -0.92387953251128674f;  // 7, 9
    case 8: return -1.0f;
  }
}

// v * exp(DIR 2 pi i m / R) for a compile-time R | 16 (m known after unrolling).
template <int DIR, int R>
__device__ __forceinline__ float2 rot(float2 v, int m) {
  const int e = (m * (16 / R)) & 15;
  if (e == 0) return v;
  if (e == 4) return DIR < 0 ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
  if (e == 8) return make_float2(-v.x, -v.y);
  if (e == 12) return DIR < 0 ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  const float c = cos16(e), s = (float)DIR * cos16(e + 12);  // sin(2 pi e/16) = cos(2 pi (e-4)/16)
  return make_float2(v.x * c - v.y * s, v.x * s + v.y * c);
}

// In-register DFT of size R in natural order (R = 2, 3, 4, 8, 16); sizes 8 and 16 are
// A x B compositions: DFT-A over the stride-B subsequences, twiddles w_R^(n2 k1), DFT-B.
template <int DIR, int R>
__device__ __forceinline__ void dftr(float2 (&x)[16]);
template <int DIR, int A, int B>
__device__ __forceinline__ void dft_comp(float2 (&x)[16]) {
  float2 y[A * B];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    float2 tt[16];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) tt[n1] = x[B * n1 + n2];
    dftr<DIR, A>(tt);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = rot<DIR, A * B>(tt[k1], n2 * k1);
  }
#pragma unroll
  for (int k1 = 0; k1 < A; ++k1) {
    float2 tt[16];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) tt[n2] = y[n2 * A + k1];
    dftr<DIR, B>(tt);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) x[k1 + A * k2] = tt[k2];
  }
}
template <int DIR, int R>
__device__ __forceinline__ void dftr(float2 (&x)[16]) {
  if (R == 2) dft2<DIR>(x[0], x[1]);
  else if (R == 3) dft3<DIR>(x[0], x[1], x[2]);
  else if (R == 4) dft4<DIR>(x[0], x[1], x[2], x[3]);
  else if (R == 8) dft_comp<DIR, 4, 2>(x);
  else if (R == 16) dft_comp<DIR, 4, 4>(x);
}

// One radix-R pass of a Stockham FFT over nl lines (element (line l, position p) at
// buf[l*ls + p*es]); lines fastest over threads, so strided layouts stay bank-conflict free.
// Ns (product of the earlier radices) is a power of two: radices run 16s, 8, 4, 2, then one 3.
template <int DIR, int R, int NT>
__device__ __forceinline__ void fft_pass(const float2* __restrict__ src0, float2* __restrict__ dst0, int work, FDiv fnl,
                                         int ls, int es, int Ns, int nb, int tstep, const float2* __restrict__ tw) {
#pragma unroll 1
  for (int t = threadIdx.x; t < work; t += NT) {
    const int j = fdiv(t, fnl);
    const int l = t - j * (int)fnl.d;
    const int k = j & (Ns - 1);
    const float2* src = src0 + l * ls;
    float2* dst = dst0 + l * ls;
    float2 v[16];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = src[(j + q * nb) * es];
    if (Ns > 1) {
#pragma unroll
      for (int q = 1; q < R; ++q) {
        const float2 w = tw[q * k * tstep];
        v[q] = (DIR < 0) ? cmul(v[q], w) : cmulc(v[q], w);
      }
    }
    dftr<DIR, R>(v);
    const int o = (j - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) dst[(o + q * Ns) * es] = v[q];
  }
}

// Complex FFT of length P.M on nl lines; returns the buffer holding the result (a or b).
template <int DIR, int NT>
__device__ float2* ens_fft(float2* a, float2* b, int nl, FDiv fnl, int ls, int es, const FFTPlan& P, const float2* tw) {
  int Ns = 1;
  for (int s = 0; s < P.nst; ++s) {
    const int R = P.R[s];
    const int nb = P.nb[s], tstep = P.ts[s];  // host-computed spans (no run-time division)
    const int work = nl * nb;
    switch (R) {
      case 16: fft_pass<DIR, 16, NT>(a, b, work, fnl, ls, es, Ns, nb, tstep, tw); break;
      case 8: fft_pass<DIR, 8, NT>(a, b, work, fnl, ls, es, Ns, nb, tstep, tw); break;
      case 4: fft_pass<DIR, 4, NT>(a, b, work, fnl, ls, es, Ns, nb, tstep, tw); break;
      case 2: fft_pass<DIR, 2, NT>(a, b, work, fnl, ls, es, Ns, nb, tstep, tw); break;
      default: fft_pass<DIR, 3, NT>(a, b, work, fnl, ls, es, Ns, nb, tstep, tw); break;
    }
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

// Real-FFT packing on a row of shared memory (complex length Mh = N/2, twiddles wN =
// exp(-2 pi i k/N) in shared memory): the same relations as r2c_post / c2r_pre.
__device__ __forceinline__ float2 pack_r2c(const float2* Z, int Mh, int k, const float2* wN) {
  const float2 zk = Z[k == Mh ? 0 : k];
  const float2 zc = cconj(Z[k == 0 ? 0 : Mh - k]);
  const float2 E = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
  const float2 Dd = csub(zk, zc);
  const float2 O = make_float2(0.5f * Dd.y, -0.5f * Dd.x);
  return cadd(E, cmul(wN[k], O));
}
__device__ __forceinline__ float2 pack_c2r(float2 xk, float2 xmk, int k, const float2* wN) {
  if (k == 0) { xk.y = 0.f; xmk.y = 0.f; }
  const float2 b = cconj(xmk);
  const float2 s = cadd(xk, b);
  const float2 d = cmulc(csub(xk, b), wN[k]);
  return make_float2(s.x - d.y, s.y + d.x);
}

// Elements handled per thread per batch: loads of a batch are issued before any use, so
// their latencies (HBM for dv_o, distributed shared memory for the all-to-alls) overlap.
template <int NT>
struct Batch {
  static constexpr int kCells = (NT >= 1024) ? 9 : 18;
  static constexpr int kElems = (NT >= 1024) ? 5 : 10;
};

// One pack seen from one CTA: the run this CTA belongs to, its rows, the shared-memory
// carve, and the steps (forward, Poisson solve, adjoint) on the G CTAs of the run.
template <int NT>
struct Pk {
  const EnsArgs& a;
  const ClassDesc& D;
  cg::cluster_group& cl;
  Carve S;
  double* s_sc;  // dt, dt_o, t, maxvel, nu, dt_visc, nan
  float* s_f;    // dt, A, B, 1/dt, mean
  double* s_rd;
  float* s_rf;
  int N, G, M, SR, C, slot, r, base, run, cells, Mh, npair, rp, rm, c0, Cr;
  bool active;
  float idx, id2, q4, mu;
  const float* force;
  FDiv fN;
  float *gu, *gv, *gp, *gdx, *gdy;  // run state in HBM (dv_o may point at the recompute scratch)
  float* ablk;                      // run's adjoint block (mode 1, 2)
  double* rec;                      // run's (dt, dt_o) record
  float *Xf, *Yf, *Zf;

  __device__ Pk(const EnsArgs& a_, const Pack& P, const ClassDesc& D_, int q, cg::cluster_group& cl_, unsigned char* smem,
                double* s_sc_, float* s_f_, double* s_rd_, float* s_rf_)
      : a(a_), D(D_), cl(cl_), S(carve(smem, D_)), s_sc(s_sc_), s_f(s_f_), s_rd(s_rd_), s_rf(s_rf_) {
    N = D.N; G = D.G; M = D.M; SR = D.SR; C = D.C;
    slot = q / G;
    r = q - slot * G;
    active = slot < P.nruns;
    run = active ? a.run_list[P.first + slot] : 0;
    base = slot * G;
    cells = M * N;
    Mh = N / 2;
    npair = Mh / 2 + 1;
    rp = (r + 1) % G;
    rm = (r - 1 + G) % G;
    c0 = r * C;
    Cr = max(0, min(C, SR - c0));
    idx = D.idx; id2 = D.id2; q4 = 0.25f * D.idx;
    fN = D.fN;
    const size_t NN = (size_t)N * N;
    gu = a.state + (active ? a.run_off[run] : 0);
    gv = gu + NN; gp = gv + NN; gdx = gp + NN; gdy = gdx + NN;
    ablk = (a.mode && active) ? a.abuf + a.aoff[run] : nullptr;
    rec = (a.mode && active) ? a.rec + (size_t)run * a.nsteps * 2 : nullptr;
    Xf = reinterpret_cast<float*>(S.X); Yf = reinterpret_cast<float*>(S.Y); Zf = reinterpret_cast<float*>(S.Z);
    force = nullptr;
    mu = 0.f;
  }
  __device__ void gsync() {
    if (G > 1) cl.sync();
    else __syncthreads();
  }
  template <typename T>
  __device__ T* peer(T* p, int g) { return G == 1 ? p : cl.map_shared_rank(p, base + g); }
  __device__ int wrapj(int jg) const { return jg < 0 ? jg + N : (jg >= N ? jg - N : jg); }

  // rows r*M-1 .. r*M+M of a global N x N array into shared rows 0 .. M+1
  __device__ void load_rows(const float* g, float* s) {
    const int rows = (M + 2) * N;
    for (int t = threadIdx.x; t < rows; t += NT) {
      const int mm = fdiv(t, fN), i = t - mm * N;
      s[t] = active ? g[(size_t)wrapj(r * M + mm - 1) * N + i] : 0.f;
    }
  }
  __device__ void store_rows(const float* s, float* g) {
    if (!active) return;
    for (int t = threadIdx.x; t < cells; t += NT) g[(size_t)r * M * N + t] = s[t + N];
  }
  // global -> global copy of this CTA's rows
  __device__ void copy_rows(const float* src, float* dst) {
    if (!active) return;
    for (int t = threadIdx.x; t < cells; t += NT) dst[(size_t)r * M * N + t] = src[(size_t)r * M * N + t];
  }
  // ghost rows 0 and M+1 of up to three row arrays from the neighbouring CTAs (after a
  // cluster barrier that made the neighbours' interior rows final)
  __device__ void ghosts(float* f0, float* f1, float* f2) {
    float* fs[3] = {f0, f1, f2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      if (!fs[q]) continue;
      const float* Fm = peer(fs[q], rm);
      const float* Fn = peer(fs[q], rp);
      for (int t = threadIdx.x; t < N; t += NT) {
        const float x0 = Fm[M * N + t], x1 = Fn[N + t];
        fs[q][t] = x0;
        fs[q][(M + 1) * N + t] = x1;
      }
    }
  }

  // ---- the Poisson solve: rhs in Z (real rows of stride 2 SR); returns phi's buffer and
  // leaves the FP64 mean of phi in s_f[4] (poisson.f90:416-505 with the mean removal) ----
  template <int EPT = Batch<NT>::kElems>
  __device__ float2* poisson() {
    float2* SPEC = ens_fft<-1, NT>(S.Z, S.X, M, D.fM, SR, 1, D.px, S.twx);
    for (int t = threadIdx.x; t < M * npair; t += NT) {
      const int m = fdiv(t, D.fNP), k = t - m * npair;
      float2* row = SPEC + m * SR;
      if (k == 0) {
        const float2 x0 = pack_r2c(row, Mh, 0, S.twn);
        const float2 xm = pack_r2c(row, Mh, Mh, S.twn);
        row[0] = x0;
        row[Mh] = xm;
      } else {
        const float2 xa = pack_r2c(row, Mh, k, S.twn);
        const float2 xb = pack_r2c(row, Mh, Mh - k, S.twn);
        row[k] = xa;
        row[Mh - k] = xb;
      }
    }
    gsync();  // every row spectrum complete
    // all-to-all: the column block [c0, c0+Cr) of every row into T (= Y)
    float2* T = S.Y;
    float2* F = (SPEC == S.Z) ? S.X : S.Z;
    for (int b0 = 0; b0 < N * C; b0 += EPT * NT) {
      float2 val[EPT];
#pragma unroll
      for (int k = 0; k < EPT; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        val[k] = make_float2(0.f, 0.f);
        if (t < N * C) {
          const int y = fdiv(t, D.fC), cc = t - y * C;
          if (cc < Cr) {
            const int g = fdiv(y, D.fM), m = y - g * M;
            val[k] = peer(SPEC, g)[m * SR + c0 + cc];
          }
        }
      }
#pragma unroll
      for (int k = 0; k < EPT; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        if (t < N * C) T[t] = val[k];
      }
    }
    __syncthreads();
    float2* R1 = ens_fft<-1, NT>(T, F, C, D.fC, 1, C, D.py, S.twy);
    for (int t = threadIdx.x; t < N * C; t += NT) {
      const int y = fdiv(t, D.fC), cc = t - y * C;
      if (cc < Cr) {
        const int kx = c0 + cc;
        const float lam = S.lamx[kx] + S.lamy[y];
        const float s = (kx == 0 && y == 0) ? 0.f : D.inv_nn / lam;
        float2 z = R1[t];
        z.x *= s;
        z.y *= s;
        R1[t] = z;
      }
    }
    __syncthreads();
    float2* R2 = ens_fft<1, NT>(R1, (R1 == T) ? F : T, C, D.fC, 1, C, D.py, S.twy);
    gsync();  // column solves complete; row spectra no longer read
    for (int b0 = 0; b0 < M * SR; b0 += EPT * NT) {
      float2 val[EPT];
#pragma unroll
      for (int k = 0; k < EPT; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        if (t < M * SR) {
          const int m = fdiv(t, D.fSR), cc = t - m * SR;
          const int o = fdiv(cc, D.fC), cl_ = cc - o * C;
          val[k] = peer(R2, o)[(r * M + m) * C + cl_];
        }
      }
#pragma unroll
      for (int k = 0; k < EPT; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        if (t < M * SR) SPEC[t] = val[k];
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < M * npair; t += NT) {
      const int m = fdiv(t, D.fNP), k = t - m * npair;
      float2* row = SPEC + m * SR;
      if (k == 0) {
        row[0] = pack_c2r(row[0], row[Mh], 0, S.twn);
      } else {
        const float2 xa = row[k], xb = row[Mh - k];
        const float2 za = pack_c2r(xa, xb, k, S.twn);
        const float2 zb = pack_c2r(xb, xa, Mh - k, S.twn);
        row[k] = za;
        if (Mh - k != k) row[Mh - k] = zb;
      }
    }
    __syncthreads();
    float2* W3 = (SPEC != S.X && R2 != S.X) ? S.X : ((SPEC != S.Y && R2 != S.Y) ? S.Y : S.Z);
    float2* PHI = ens_fft<1, NT>(SPEC, W3, M, D.fM, SR, 1, D.px, S.twx);
    const float* Phf = reinterpret_cast<const float*>(PHI);
    {  // FP64 sum of phi for the mean removal
      float part = 0.f;
      for (int t = threadIdx.x; t < cells; t += NT) {
        const int m = fdiv(t, fN), i = t - m * N;
        part += Phf[m * 2 * SR + i];
      }
      const double s = block_sum<NT>((double)part, s_rd);
      if (threadIdx.x == 0) S.red[0] = s;
    }
    gsync();  // phi and the partial sums visible
    if (threadIdx.x < 32) {  // lanes read the G partial sums; fixed-order butterfly sum
      double s = (threadIdx.x < G) ? peer(S.red, threadIdx.x)[0] : 0.0;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0) s_f[4] = (float)(s / ((double)N * N));
    }
    __syncthreads();
    return PHI;
  }

  // ---- one forward step (navier_stokes.f90:50-136, constant CFL) ----
  // rec_step >= 0 replays the recorded (dt, dt_o) of that step instead of the CFL update;
  // rec_out >= 0 records this step's (dt, dt_o).
  template <int EPT = Batch<NT>::kElems>
  __device__ void fwd_step(int rec_step, int rec_out) {
    constexpr int CPT = Batch<NT>::kCells;
    if (threadIdx.x == 0) {
      double dt, dt_o;
      if (rec_step >= 0 && rec) {
        dt = rec[2 * rec_step];
        dt_o = rec[2 * rec_step + 1];
      } else {
        dt_o = s_sc[0];
        const double mv = s_sc[3];
        const double dt_conv = (mv > 0.0) ? a.cfl * D.delta / mv : 1.0;
        dt = fmin(dt_conv, s_sc[5]);
        if (dt > 1.1 * dt_o) dt = 1.1 * dt_o;
      }
      if (rec_out >= 0 && rec && r == 0) {
        rec[2 * rec_out] = dt;
        rec[2 * rec_out + 1] = dt_o;
      }
      s_sc[0] = dt;
      s_sc[1] = dt_o;
      const float rf = (float)dt / (float)dt_o;  // the FP32 stencils take A, B and 1/dt in FP32
      s_f[0] = (float)dt;
      s_f[1] = 1.0f + 0.5f * rf;
      s_f[2] = -0.5f * rf;
      s_f[3] = 1.0f / (float)dt;
    }
    __syncthreads();
    const float dt = s_f[0], A = s_f[1], B = s_f[2], rdt = s_f[3];

    // predictor: u* -> X, v* -> Y (FP32), dv_o streamed from/to HBM
    for (int b0 = 0; b0 < cells; b0 += CPT * NT) {
      float ox[CPT], oy[CPT];
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        ox[k] = 0.f;
        oy[k] = 0.f;
        if (active && t < cells) {
          const size_t gi = (size_t)r * M * N + t;
          ox[k] = gdx[gi];
          oy[k] = gdy[gi];
        }
      }
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        if (t < cells) {
          const int m = fdiv(t, fN), i = t - m * N;
          const int ip = (i + 1 == N) ? 1 - N : 1;
          const int im = (i == 0) ? N - 1 : -1;
          const int c = t + N;
          const float* U = S.u;
          const float* V = S.v;
          const float* Pp = S.p;
          const float uc = U[c], uip = U[c + ip], uim = U[c + im], ujp = U[c + N], ujm = U[c - N], uimjp = U[c + N + im];
          const float vc = V[c], vip = V[c + ip], vim = V[c + im], vjp = V[c + N], vjm = V[c - N], vipjm = V[c - N + ip];
          // u: -(d(uu)/dx + d(uv)/dy) + nu lap(u) + S_x      (navier_stokes.f90:297-323, fields.f90:326-329)
          const float fe = (uip + uc) * (uip + uc), fw = (uc + uim) * (uc + uim);
          const float cn = (ujp + uc) * (vip + vc), cs = (uc + ujm) * (vipjm + vjm);
          const float dvx = -((fe - fw) + (cn - cs)) * q4 + mu * (((uip + uim) + (ujp + ujm)) - 4.0f * uc) * id2 + force[m];
          // v: -(d(uv)/dx + d(vv)/dy) + nu lap(v)
          const float cw = (uimjp + uim) * (vc + vim);
          const float fn = (vjp + vc) * (vjp + vc), fs = (vc + vjm) * (vc + vjm);
          const float dvy = -((cn - cw) + (fn - fs)) * q4 + mu * (((vip + vim) + (vjp + vjm)) - 4.0f * vc) * id2;
          if (active) {
            const size_t gi = (size_t)r * M * N + t;
            gdx[gi] = dvx;
            gdy[gi] = dvy;
          }
          Xf[t] = uc + dt * (-(Pp[c + ip] - Pp[c]) * idx + A * dvx + B * ox[k]);
          Yf[t] = vc + dt * (-(Pp[c + N] - Pp[c]) * idx + A * dvy + B * oy[k]);
        }
      }
    }
    gsync();  // v* rows visible to the next CTA

    // divergence * rho/dt -> Z; u, v <- u*, v*
    {
      const float* Yprev = peer(Yf, rm);
      const float sc = idx * rdt;
      for (int t = threadIdx.x; t < cells; t += NT) {
        const int m = fdiv(t, fN), i = t - m * N;
        const int im = (i == 0) ? N - 1 : -1;
        const float us = Xf[t], usm = Xf[t + im], vs = Yf[t];
        const float vsm = (m > 0) ? Yf[t - N] : Yprev[(M - 1) * N + i];
        Zf[m * 2 * SR + i] = ((us - usm) + (vs - vsm)) * sc;
        S.u[t + N] = us;
        S.v[t + N] = vs;
      }
    }
    __syncthreads();
    float2* PHI = poisson<EPT>();
    const float* Phf = reinterpret_cast<const float*>(PHI);

    // correction, p update, max(|u| + |v|)
    {
      const float meanf = s_f[4];
      const float* Phn = reinterpret_cast<const float*>(peer(PHI, rp));
      float vmax = 0.f;
      int bad = 0;
      for (int t = threadIdx.x; t < cells; t += NT) {
        const int m = fdiv(t, fN), i = t - m * N;
        const int ip = (i + 1 == N) ? 1 - N : 1;
        const int o = m * 2 * SR + i;
        const float ph = Phf[o], phip = Phf[o + ip];
        const float phjp = (m + 1 < M) ? Phf[o + 2 * SR] : Phn[i];
        const int c = t + N;
        const float un = S.u[c] - dt * (phip - ph) * idx;
        const float vn = S.v[c] - dt * (phjp - ph) * idx;
        S.u[c] = un;
        S.v[c] = vn;
        S.p[c] = S.p[c] + (ph - meanf);
        const float vel = fabsf(un) + fabsf(vn);
        if (vel != vel) bad = 1;
        vmax = fmaxf(vmax, vel);
      }
      const float mx = block_max<NT>(vmax, s_rf);
      bad = __syncthreads_or(bad);
      if (threadIdx.x == 0) {
        S.red[1] = (double)mx;
        S.red[2] = (double)bad;
      }
    }
    gsync();  // corrected rows, maxima visible
    if (threadIdx.x < 32) {
      double mv = 0.0, bd = 0.0;
      if (threadIdx.x < G) {
        const double* rr = peer(S.red, threadIdx.x);
        mv = rr[1];
        bd = rr[2];
      }
      for (int o = 16; o > 0; o >>= 1) {
        mv = fmax(mv, __shfl_xor_sync(0xffffffffu, mv, o));
        bd = fmax(bd, __shfl_xor_sync(0xffffffffu, bd, o));
      }
      if (threadIdx.x == 0) {
        s_sc[3] = mv;
        s_sc[2] += s_sc[0];
        if (bd != 0.0) s_sc[6] = 1.0;
      }
    }
    ghosts(S.u, S.v, S.p);
    __syncthreads();
  }

  // ---- one adjoint step (the transpose of fwd_step for fixed dt; see fen_adjoint.cuh) ----
  // Adjoint state: u^, v^ (rows with ghosts) in S.u, S.v, p^ in S.p, dv_o^ in HBM (ax, ay);
  // the forward step's input velocity (u, v) in HBM (fu, fv, full N x N arrays).
  // Step s of the record; its forward input (u, v) is slot sl of the segment's step inputs.
  // The coefficients and the HBM pointers are re-derived after the Poisson solve instead of
  // being held across it (registers).
  __device__ void adj_coef(int s, float& dt, float& A, float& B, float& rdt) const {
    const double dtd = rec ? __ldg(rec + 2 * s) : 1.0, dt_od = rec ? __ldg(rec + 2 * s + 1) : 1.0;
    dt = (float)dtd;
    const float rf = (float)dtd / (float)dt_od;
    A = 1.0f + 0.5f * rf;
    B = -0.5f * rf;
    rdt = 1.0f / dt;
  }
  __device__ void adj_step(int s, int sl) {
    float dt, A, B, rdt;
    adj_coef(s, dt, A, B, rdt);
    // phi^ = p^ + dt D(v^)  -> Z
    for (int t = threadIdx.x; t < cells; t += NT) {
      const int m = fdiv(t, fN), i = t - m * N;
      const int im = (i == 0) ? N - 1 : -1;
      const int c = t + N;
      Zf[m * 2 * SR + i] = S.p[c] + dt * (((S.u[c] - S.u[c + im]) + (S.v[c] - S.v[c - N])) * idx);
    }
    __syncthreads();
    // b^ = P phi^ (symmetric); v*^ = v^ - (rho/dt) G b^  (in place)
    float2* PHI = poisson<FEN_ENS_ADJ_EPT>();
    adj_coef(s, dt, A, B, rdt);
    const long long N2 = (long long)N * N;
    const AdjLayout AL(N2, a.nseg, a.every);
    float* ax = ablk ? ablk + AL.adj + 3 * N2 : nullptr;
    float* ay = ablk ? ablk + AL.adj + 4 * N2 : nullptr;
    const float* fu = ablk ? ablk + AL.seg + (long long)sl * 2 * N2 : nullptr;
    const float* fv = ablk ? fu + N2 : nullptr;
    {
      const float* Phf = reinterpret_cast<const float*>(PHI);
      const float* Phn = reinterpret_cast<const float*>(peer(PHI, rp));
      for (int t = threadIdx.x; t < cells; t += NT) {
        const int m = fdiv(t, fN), i = t - m * N;
        const int ip = (i + 1 == N) ? 1 - N : 1;
        const int o = m * 2 * SR + i;
        const float b = Phf[o], bip = Phf[o + ip];
        const float bjp = (m + 1 < M) ? Phf[o + 2 * SR] : Phn[i];
        const int c = t + N;
        S.u[c] = S.u[c] - rdt * (bip - b) * idx;
        S.v[c] = S.v[c] - rdt * (bjp - b) * idx;
      }
    }
    gsync();
    ghosts(S.u, S.v, nullptr);
    __syncthreads();
    // p^ += dt D(v*^); dv^ = dv_o^ + dt A v*^ -> X, Y (rows with ghosts); dv_o^ = dt B v*^.
    // The HBM reads of dv_o^ are issued kAB cells at a time before any is used.
    constexpr int kAB = (NT >= 1024) ? 4 : 8;
    for (int b0 = 0; b0 < cells; b0 += kAB * NT) {
      float ox[kAB], oy[kAB];
#pragma unroll
      for (int k = 0; k < kAB; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        ox[k] = 0.f;
        oy[k] = 0.f;
        if (active && t < cells) {
          const size_t gi = (size_t)r * M * N + t;
          ox[k] = ax[gi];
          oy[k] = ay[gi];
        }
      }
#pragma unroll
      for (int k = 0; k < kAB; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        if (t < cells) {
          const int m = fdiv(t, fN), i = t - m * N;
          const int im = (i == 0) ? N - 1 : -1;
          const int c = t + N;
          const float us = S.u[c], vs = S.v[c];
          S.p[c] = S.p[c] + dt * (((us - S.u[c + im]) + (vs - S.v[c - N])) * idx);
          if (active) {
            const size_t gi = (size_t)r * M * N + t;
            ax[gi] = dt * B * us;
            ay[gi] = dt * B * vs;
          }
          Xf[c] = ox[k] + dt * A * us;
          Yf[c] = oy[k] + dt * A * vs;
        }
      }
    }
    gsync();
    ghosts(Xf, Yf, nullptr);
    __syncthreads();
    // v^ = v*^ + N'(v)^T dv^ + mu L dv^   (navier_stokes.f90:297-323 transposed).  The forward
    // input velocity around (i, j) comes from HBM (periodic in both directions); its reads are
    // issued kAS cells at a time before any is used, the u and v components in two passes so
    // each keeps only its own seven forward values per cell live.
    constexpr int kAS = (NT >= 1024) ? 2 : 4;
    const float mur = mu;
    const float* hu = Xf;
    const float* hv = Yf;
    for (int b0 = 0; b0 < cells; b0 += kAS * NT) {
      float f[kAS][7];
#pragma unroll
      for (int k = 0; k < kAS; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
#pragma unroll
        for (int e = 0; e < 7; ++e) f[k][e] = 0.f;
        if (active && t < cells) {
          const int m = fdiv(t, fN), i = t - m * N;
          const int ip = (i + 1 == N) ? 1 - N : 1;
          const int im = (i == 0) ? N - 1 : -1;
          const int jg = r * M + m;
          const size_t row = (size_t)jg * N, rowm = (size_t)wrapj(jg - 1) * N;
          f[k][0] = fu[row + i]; f[k][1] = fu[row + i + ip]; f[k][2] = fu[row + i + im];
          f[k][3] = fv[row + i]; f[k][4] = fv[row + i + ip]; f[k][5] = fv[rowm + i]; f[k][6] = fv[rowm + i + ip];
        }
      }
#pragma unroll
      for (int k = 0; k < kAS; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        if (t < cells) {
          const int m = fdiv(t, fN), i = t - m * N;
          const int ip = (i + 1 == N) ? 1 - N : 1;
          const int im = (i == 0) ? N - 1 : -1;
          const int c = t + N;
          const float u0 = f[k][0], uip = f[k][1], uim = f[k][2];
          const float v0 = f[k][3], vip = f[k][4], vjm = f[k][5], vipjm = f[k][6];
          const float Fu_p = (hu[c + ip] - hu[c]) * idx, Fu_m = (hu[c] - hu[c + im]) * idx;
          const float C_ij = (hu[c + N] - hu[c]) * idx + (hv[c + ip] - hv[c]) * idx;
          const float C_ijm = (hu[c] - hu[c - N]) * idx + (hv[c + ip - N] - hv[c - N]) * idx;
          const float gu_ = Fu_p * 0.5f * (uip + u0) + Fu_m * 0.5f * (u0 + uim) + C_ij * 0.25f * (vip + v0) +
                            C_ijm * 0.25f * (vipjm + vjm);
          const float lu = ((hu[c + ip] + hu[c + im]) + (hu[c + N] + hu[c - N]) - 4.0f * hu[c]) * id2;
          S.u[c] = S.u[c] + gu_ + mur * lu;
        }
      }
    }
    for (int b0 = 0; b0 < cells; b0 += kAS * NT) {
      float f[kAS][7];
#pragma unroll
      for (int k = 0; k < kAS; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
#pragma unroll
        for (int e = 0; e < 7; ++e) f[k][e] = 0.f;
        if (active && t < cells) {
          const int m = fdiv(t, fN), i = t - m * N;
          const int im = (i == 0) ? N - 1 : -1;
          const int jg = r * M + m;
          const size_t row = (size_t)jg * N, rowp = (size_t)wrapj(jg + 1) * N, rowm = (size_t)wrapj(jg - 1) * N;
          f[k][0] = fu[row + i]; f[k][1] = fu[row + i + im]; f[k][2] = fu[rowp + i]; f[k][3] = fu[rowp + i + im];
          f[k][4] = fv[row + i]; f[k][5] = fv[rowp + i]; f[k][6] = fv[rowm + i];
        }
      }
#pragma unroll
      for (int k = 0; k < kAS; ++k) {
        const int t = b0 + threadIdx.x + k * NT;
        if (t < cells) {
          const int m = fdiv(t, fN), i = t - m * N;
          const int ip = (i + 1 == N) ? 1 - N : 1;
          const int im = (i == 0) ? N - 1 : -1;
          const int c = t + N;
          const float u0 = f[k][0], uim = f[k][1], ujp = f[k][2], uimjp = f[k][3];
          const float v0 = f[k][4], vjp = f[k][5], vjm = f[k][6];
          const float Fv_p = (hv[c + N] - hv[c]) * idx, Fv_m = (hv[c] - hv[c - N]) * idx;
          const float C_ij = (hu[c + N] - hu[c]) * idx + (hv[c + ip] - hv[c]) * idx;
          const float C_imj = (hu[c + im + N] - hu[c + im]) * idx + (hv[c] - hv[c + im]) * idx;
          const float gv_ = Fv_p * 0.5f * (vjp + v0) + Fv_m * 0.5f * (v0 + vjm) + C_ij * 0.25f * (ujp + u0) +
                            C_imj * 0.25f * (uimjp + uim);
          const float lv = ((hv[c + ip] + hv[c + im]) + (hv[c + N] + hv[c - N]) - 4.0f * hv[c]) * id2;
          S.v[c] = S.v[c] + gv_ + mur * lv;
        }
      }
    }
    gsync();
    ghosts(S.u, S.v, nullptr);
    __syncthreads();
  }
};

// MODE 0: advance; 1: advance with checkpoints and the dt record; 2: backward sweep.  The
// mode is a template parameter so the advance kernel carries no adjoint code (registers).
template <int NT, int MODE>
__device__ void run_pack(const EnsArgs& a, const Pack& P, const ClassDesc& D, int q, cg::cluster_group& cl,
                         unsigned char* smem, double* s_sc, float* s_f, double* s_rd, float* s_rf) {
  Pk<NT> k(a, P, D, q, cl, smem, s_sc, s_f, s_rd, s_rf);
  if (!k.active && k.G == 1) return;  // no partner waits on this CTA
  const int N = k.N, M = k.M, r = k.r;
  const Carve& S = k.S;
  const long long N2 = (long long)N * N;
  // tables of this grid size
  if (D.tabs) {
    for (int t = threadIdx.x; t < N / 2; t += NT) S.twx[t] = D.twx[t];
    for (int t = threadIdx.x; t <= N / 2; t += NT) {
      S.twn[t] = D.twn[t];
      S.lamx[t] = D.lamx[t];
    }
    for (int t = threadIdx.x; t < N; t += NT) {
      S.twy[t] = D.twy[t];
      S.lamy[t] = D.lamy[t];
    }
    for (int t = threadIdx.x; t < M; t += NT) S.force[t] = D.force[r * M + t];
  }
  k.force = D.tabs ? S.force : D.force + r * M;
  if (threadIdx.x == 0) {
    RunScal rs;
    if (k.active) rs = a.scal[k.run];
    else { rs.dt = rs.dt_o = 1.0; rs.t = 0.0; rs.maxvel = 1.0; rs.nu = 1.0; rs.dt_visc = 1.0; rs.nan = 0; }
    s_sc[0] = rs.dt;
    s_sc[1] = rs.dt_o;
    s_sc[2] = rs.t;
    s_sc[3] = rs.maxvel;
    s_sc[4] = rs.nu;
    s_sc[5] = rs.dt_visc;
    s_sc[6] = rs.nan;
  }
  __syncthreads();
  k.mu = (float)s_sc[4];

  if (MODE == 2) {
    // ---- backward sweep: per segment, recompute from the checkpoint, then adjoint steps ----
    const AdjLayout AL(N2, a.nseg, a.every);
    float* ab = k.ablk;
    float* dscr = ab ? ab + AL.dvo : nullptr;
    float* adj = ab ? ab + AL.adj : nullptr;
    for (int seg = a.nseg - 1; seg >= 0; --seg) {
      const int s0 = seg * a.every, s1 = min(a.nsteps, s0 + a.every);
      float* ck = ab ? ab + AL.ck + (long long)seg * 5 * N2 : nullptr;
      k.gsync();  // partners are done with this CTA's rows of the previous segment
      k.load_rows(ck, S.u);
      k.load_rows(ck ? ck + N2 : nullptr, S.v);
      k.load_rows(ck ? ck + 2 * N2 : nullptr, S.p);
      if (ab) {
        k.copy_rows(ck + 3 * N2, dscr);
        k.copy_rows(ck + 4 * N2, dscr + N2);
      }
      k.gdx = dscr;
      k.gdy = dscr ? dscr + N2 : nullptr;
      __syncthreads();
      for (int s = s0; s < s1; ++s) {
        float* in = ab ? ab + AL.seg + (long long)(s - s0) * 2 * N2 : nullptr;
        if (in) {
          k.store_rows(S.u, in);
          k.store_rows(S.v, in + N2);
        }
        k.template fwd_step<FEN_ENS_REC_EPT>(s, -1);
      }
      k.gsync();  // step inputs of the segment written by every CTA of the run
      k.load_rows(adj, S.u);
      k.load_rows(adj ? adj + N2 : nullptr, S.v);
      k.load_rows(adj ? adj + 2 * N2 : nullptr, S.p);
      __syncthreads();
      for (int s = s1 - 1; s >= s0; --s) k.adj_step(s, s - s0);
      k.store_rows(S.u, adj);
      k.store_rows(S.v, adj ? adj + N2 : nullptr);
      k.store_rows(S.p, adj ? adj + 2 * N2 : nullptr);
    }
    k.gsync();
    return;
  }

  // ---- advance (mode 0) or forward with checkpoints (mode 1) ----
  k.load_rows(k.gu, S.u);
  k.load_rows(k.gv, S.v);
  k.load_rows(k.gp, S.p);
  __syncthreads();
  const AdjLayout AL(N2, a.nseg, a.every);
  for (int step = 0; step < a.nsteps; ++step) {
    if (MODE == 1 && step % a.every == 0 && k.ablk) {
      float* ck = k.ablk + AL.ck + (long long)(step / a.every) * 5 * N2;
      k.store_rows(S.u, ck);
      k.store_rows(S.v, ck + N2);
      k.store_rows(S.p, ck + 2 * N2);
      k.copy_rows(k.gdx, ck + 3 * N2);
      k.copy_rows(k.gdy, ck + 4 * N2);
    }
    k.fwd_step(-1, MODE == 1 ? step : -1);
  }

  // ---- store the state; kinetic energy and max div (FP64 across the run) ----
  {
    const float idx = k.idx;
    float kpart = 0.f, dmax = -INFINITY;
    for (int t = threadIdx.x; t < k.cells; t += NT) {
      const int m = fdiv(t, k.fN), i = t - m * N;
      const int im = (i == 0) ? N - 1 : -1;
      const int c = t + N;
      const float uu = S.u[c], vv = S.v[c];
      if (k.active) {
        const size_t gi = (size_t)r * M * N + t;
        k.gu[gi] = uu;
        k.gv[gi] = vv;
        k.gp[gi] = S.p[c];
      }
      kpart += uu * uu + vv * vv;
      dmax = fmaxf(dmax, ((uu - S.u[c + im]) + (vv - S.v[c - N])) * idx);
    }
    const double ks = block_sum<NT>((double)kpart, s_rd);
    const float dm = block_max<NT>(dmax, s_rf);
    if (threadIdx.x == 0) {
      S.red[3] = ks;
      S.red[4] = (double)dm;
    }
    k.gsync();
    if (threadIdx.x == 0 && r == 0 && k.active) {
      double kk = 0.0, d = -INFINITY;
      for (int g = 0; g < k.G; ++g) {
        const double* rr = k.peer(S.red, g);
        kk += rr[3];
        d = fmax(d, rr[4]);
      }
      RunScal rs = a.scal[k.run];
      rs.dt = s_sc[0];
      rs.dt_o = s_sc[1];
      rs.t = s_sc[2];
      rs.maxvel = s_sc[3];
      rs.nan = (int)s_sc[6];
      rs.ke = 0.5 * kk / ((double)N * N);
      rs.maxdiv = d;
      a.scal[k.run] = rs;
    }
    k.gsync();  // partners finished reading this CTA's partial sums
  }
}

template <int NT, int MODE>
__global__ void __launch_bounds__(NT, 1) k_ensemble(EnsArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_pack;
  __shared__ ClassDesc s_D;
  __shared__ double s_sc[8];
  __shared__ float s_f[8];
  __shared__ double s_rd[32];
  __shared__ float s_rf[32];
  cg::cluster_group cl = cg::this_cluster();
  const int q = (int)cl.block_rank();
  for (;;) {
    if (q == 0 && threadIdx.x == 0) s_pack = atomicAdd(a.counter, 1);
    cl.sync();
    const int pk = *cl.map_shared_rank(&s_pack, 0);
    cl.sync();  // every CTA has read the pack index before rank 0 fetches the next one
    if (pk >= a.npacks) break;
    const Pack P = a.packs[pk];
    if (threadIdx.x == 0) s_D = a.cls[P.cls];
    __syncthreads();
    run_pack<NT, MODE>(a, P, s_D, q, cl, smem, s_sc, s_f, s_rd, s_rf);
    __syncthreads();
  }
}

}  // namespace ens
}  // namespace fen

using namespace fen::ens;

// ------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------
struct fen_ensemble {
  int nruns = 0;
  int dev = 0;
  std::vector<int> n;
  std::vector<double> nu;
  double L = 0, cfl = 0, famp = 0;
  int fk = 0;
  std::vector<int> cls_n;                // distinct grid sizes, largest first
  std::vector<int> cls_g;                // CTAs per run for each size
  std::vector<int> run_cls;              // class of each run
  std::vector<ClassDesc> cls_host;
  std::vector<void*> bufs;
  std::vector<long long> off;
  float* state = nullptr;
  long long* d_off = nullptr;
  RunScal* d_scal = nullptr;
  std::vector<RunScal> scal;
  ClassDesc* d_cls = nullptr;
  Pack* d_packs = nullptr;
  int* d_runlist = nullptr;
  int* d_counter = nullptr;               // [0] the 8-CTA launch, [1] the 4-CTA launch
  int npacks = 0;
  int threads = 1024;
  size_t smem = 0;
  int nclusters = 0;
  // the SMs that kCl-CTA clusters leave idle take a second, concurrent launch of 4-CTA
  // clusters over the small grids (classes with G <= 4)
  Pack* d_packs4 = nullptr;
  int* d_runlist4 = nullptr;
  int npacks4 = 0;
  size_t smem4 = 0;
  int nclusters4 = 0;
  bool split = FEN_ENS_SPLIT != 0;
  int share = FEN_ENS_SHARE;  // percent of the 4-CTA launch's proportional share of the cells
  cudaStream_t stream2 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int exec_steps = -1;
  long long launches = 0;
  bool scal_dirty = false;
  // forward/adjoint pair
  int adj_nsteps = 0, adj_every = 0, adj_nseg = 0;
  bool adj_ready = false;
  float* abuf = nullptr;
  long long* d_aoff = nullptr;
  std::vector<long long> aoff;
  double* rec = nullptr;
};

namespace {

#define EK(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess)                                                                      \
      return fen_internal_fail(FEN_ERR_CUDA, (std::string(#x) + ": " + cudaGetErrorString(e_)).c_str()); \
  } while (0)

// Radix schedule of the in-register passes: 16s first, then one 8, 4 or 2, then a 3.
bool plan_len(int M, FFTPlan& P) {
  P.M = M;
  P.nst = 0;
  int m = M;
  while (m % 16 == 0) { P.R[P.nst++] = 16; m /= 16; }
  if (m % 8 == 0) { P.R[P.nst++] = 8; m /= 8; }
  if (m % 4 == 0) { P.R[P.nst++] = 4; m /= 4; }
  if (m % 2 == 0) { P.R[P.nst++] = 2; m /= 2; }
  if (m % 3 == 0) { P.R[P.nst++] = 3; m /= 3; }
  fft_plan_magic(P);
  return m == 1 && P.nst <= kMaxStages;
}

bool g_feasible(int N, int G) {
  if (G < 1 || G > kCl || (G & (G - 1)) != 0) return false;
  if (N % G != 0 || N / G < 2) return false;
  return smem_bytes(N, G) + kSmemReserve <= kSmemLimit;
}

template <typename T>
int dev_upload(fen_ensemble* e, const std::vector<T>& h, const T** out) {
  void* d = nullptr;
  EK(cudaMalloc(&d, std::max<size_t>(h.size(), 1) * sizeof(T)));
  e->bufs.push_back(d);
  EK(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  *out = (const T*)d;
  return 0;
}

int build_class(fen_ensemble* e, int N, ClassDesc& D) {
  D = ClassDesc{};
  D.N = N;
  if (!plan_len(N / 2, D.px) || !plan_len(N, D.py)) return fen_internal_fail(FEN_ERR_ARG, "ensemble grid size must be 2^a 3^b, a >= 2");
  const double d = e->L / N;
  D.delta = d;
  D.idx = (float)(1.0 / d);
  D.id2 = (float)(1.0 / (d * d));
  D.inv_nn = (float)(1.0 / ((double)N * N));
  std::vector<float2> twx(N / 2), twn(N / 2 + 1), twy(N);
  for (int m = 0; m < N / 2; ++m) { const double t = 2.0 * M_PI * m / (N / 2); twx[m] = make_float2((float)cos(t), (float)-sin(t)); }
  for (int k = 0; k <= N / 2; ++k) { const double t = 2.0 * M_PI * k / N; twn[k] = make_float2((float)cos(t), (float)-sin(t)); }
  for (int m = 0; m < N; ++m) { const double t = 2.0 * M_PI * m / N; twy[m] = make_float2((float)cos(t), (float)-sin(t)); }
  std::vector<float> lx(N / 2 + 1), ly(N), fo(N);
  for (int k = 0; k <= N / 2; ++k) lx[k] = (float)(2.0 * (cos(2.0 * M_PI * k / N) - 1.0) / (d * d));
  for (int k = 0; k < N; ++k) ly[k] = (float)(2.0 * (cos(2.0 * M_PI * k / N) - 1.0) / (d * d));
  for (int j = 0; j < N; ++j) fo[j] = (float)(e->famp * sin(e->fk * (j + 0.5) * d));
  int r;
  if ((r = dev_upload(e, twx, &D.twx)) || (r = dev_upload(e, twn, &D.twn)) || (r = dev_upload(e, twy, &D.twy)) ||
      (r = dev_upload(e, lx, &D.lamx)) || (r = dev_upload(e, ly, &D.lamy)) || (r = dev_upload(e, fo, &D.force)))
    return r;
  return 0;
}

void set_g(ClassDesc& D, int G) {
  D.G = G;
  D.M = D.N / G;
  D.SR = D.N / 2 + 1;
  D.C = (D.SR + G - 1) / G;
  int buf = 0;
  smem_bytes(D.N, G, &buf);
  D.buf = buf;
  D.fN = make_fdiv(D.N);
  D.fSR = make_fdiv(D.SR);
  D.fC = make_fdiv(D.C);
  D.fM = make_fdiv(D.M);
  D.fNP = make_fdiv(D.N / 4 + 1);
  D.tabs = smem_bytes(D.N, G, nullptr, true) + kSmemReserve <= kSmemLimit;
}

const void* kernel_ptr(int threads, int mode = 0) {
  if (threads == 512) return mode == 0 ? (const void*)k_ensemble<512, 0> : mode == 1 ? (const void*)k_ensemble<512, 1> : (const void*)k_ensemble<512, 2>;
  return mode == 0 ? (const void*)k_ensemble<1024, 0> : mode == 1 ? (const void*)k_ensemble<1024, 1> : (const void*)k_ensemble<1024, 2>;
}

// Pack the runs `subset` (all runs when empty) with the current G per class; uploads the
// class table, the packs and the run lists, and sizes the launches.  With the split on, the
// smallest runs of classes with G <= 4 go to 4-CTA clusters on the SMs the kCl-CTA clusters
// leave idle, up to that share of the SMs (cost N^2 per run).
int upload_packs(const std::vector<Pack>& packs, const std::vector<int>& list, Pack** dp, int** dl) {
  if (*dp) cudaFree(*dp);
  if (*dl) cudaFree(*dl);
  *dp = nullptr;
  *dl = nullptr;
  EK(cudaMalloc(dp, std::max<size_t>(packs.size(), 1) * sizeof(Pack)));
  EK(cudaMalloc(dl, std::max<size_t>(list.size(), 1) * sizeof(int)));
  if (!packs.empty()) EK(cudaMemcpy(*dp, packs.data(), packs.size() * sizeof(Pack), cudaMemcpyHostToDevice));
  if (!list.empty()) EK(cudaMemcpy(*dl, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice));
  return 0;
}

int max_clusters(fen_ensemble* e, int csize, size_t smem, int* out) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(csize, 1, 1);
  cfg.blockDim = dim3(e->threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  EK(cudaOccupancyMaxActiveClusters(out, kernel_ptr(e->threads), &cfg));
  return 0;
}

int build_packs(fen_ensemble* e, const std::vector<int>& subset) {
  for (size_t c = 0; c < e->cls_n.size(); ++c) set_g(e->cls_host[c], e->cls_g[c]);
  std::vector<int> runs;
  if (subset.empty()) {
    for (int q = 0; q < e->nruns; ++q) runs.push_back(q);
  } else {
    runs = subset;
  }
  // SMs left idle by the kCl-CTA clusters
  int sms = 0, dev = 0;
  EK(cudaGetDevice(&dev));
  EK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  size_t smem_all = 0;
  for (int q : runs) {
    const int c = e->run_cls[q];
    smem_all = std::max(smem_all, smem_bytes(e->cls_n[c], e->cls_g[c], nullptr, e->cls_host[c].tabs != 0));
  }
  for (int m = 0; m < 3; ++m) {
    EK(cudaFuncSetAttribute(kernel_ptr(e->threads, m), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(smem_all, 1)));
    if (kCl > 8) EK(cudaFuncSetAttribute(kernel_ptr(e->threads, m), cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  }
  // assignment: smallest eligible runs to the 4-CTA launch up to its share of the SMs
  std::vector<char> small(e->nruns, 0);
  int n4 = 0;
  if (e->split && kCl == 8) {
    int nc = 0;
    int r;
    if ((r = max_clusters(e, kCl, smem_all, &nc))) return r;
    const int idle = sms - kCl * nc;
    n4 = idle >= 4 ? idle / 4 : 0;
    if (n4 > 0) {
      std::vector<int> order(runs);
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return e->n[a] < e->n[b]; });
      double total = 0.0;
      for (int q : order) total += (double)e->n[q] * e->n[q];
      const double target = 0.01 * e->share * total * (4.0 * n4) / (4.0 * n4 + (double)kCl * nc);
      double acc = 0.0;
      for (int q : order) {
        const double w = (double)e->n[q] * e->n[q];
        if (e->cls_g[e->run_cls[q]] > 4 || acc + 0.5 * w > target) continue;
        small[q] = 1;
        acc += w;
      }
    }
  }
  std::vector<Pack> packs[2];
  std::vector<int> list[2];
  size_t smem[2] = {0, 0};
  for (size_t c = 0; c < e->cls_n.size(); ++c) {
    const int G = e->cls_g[c];
    for (int part = 0; part < 2; ++part) {
      const int csize = part ? 4 : kCl, per = csize / G;
      std::vector<int> rr;
      for (int q : runs)
        if (e->run_cls[q] == (int)c && (int)small[q] == part) rr.push_back(q);
      if (rr.empty()) continue;
      smem[part] = std::max(smem[part], smem_bytes(e->cls_n[c], G, nullptr, e->cls_host[c].tabs != 0));
      for (size_t s = 0; s < rr.size(); s += per) {
        Pack p;
        p.cls = (int)c;
        p.first = (int)list[part].size();
        p.nruns = (int)std::min<size_t>(per, rr.size() - s);
        p.pad = 0;
        for (int k = 0; k < p.nruns; ++k) list[part].push_back(rr[s + k]);
        packs[part].push_back(p);
      }
    }
  }
  EK(cudaMemcpy(e->d_cls, e->cls_host.data(), e->cls_host.size() * sizeof(ClassDesc), cudaMemcpyHostToDevice));
  int r;
  if ((r = upload_packs(packs[0], list[0], &e->d_packs, &e->d_runlist))) return r;
  if ((r = upload_packs(packs[1], list[1], &e->d_packs4, &e->d_runlist4))) return r;
  e->npacks = (int)packs[0].size();
  e->npacks4 = (int)packs[1].size();
  e->smem = smem[0];
  e->smem4 = smem[1];
  int nc = 0;
  if (e->npacks) {
    if ((r = max_clusters(e, kCl, e->smem, &nc))) return r;
    if (nc < 1)
      return fen_internal_fail(FEN_ERR_CUDA, ("no cluster of " + std::to_string(kCl) +
                                              " CTAs fits this device with the ensemble's shared memory").c_str());
  }
  e->nclusters = nc;
  e->nclusters4 = e->npacks4 ? std::max(1, n4) : 0;
  if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
  if (e->graph) { cudaGraphDestroy(e->graph); e->graph = nullptr; }
  e->exec_steps = -1;
  return 0;
}

int launch_one(fen_ensemble* e, EnsArgs a, int csize, int nclusters, size_t smem, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(csize * std::max(1, std::min(nclusters, a.npacks)), 1, 1);
  cfg.blockDim = dim3(e->threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  const int mode = a.mode;
  if (e->threads == 512) {
    if (mode == 0) EK(cudaLaunchKernelEx(&cfg, k_ensemble<512, 0>, a));
    else if (mode == 1) EK(cudaLaunchKernelEx(&cfg, k_ensemble<512, 1>, a));
    else EK(cudaLaunchKernelEx(&cfg, k_ensemble<512, 2>, a));
  } else {
    if (mode == 0) EK(cudaLaunchKernelEx(&cfg, k_ensemble<1024, 0>, a));
    else if (mode == 1) EK(cudaLaunchKernelEx(&cfg, k_ensemble<1024, 1>, a));
    else EK(cudaLaunchKernelEx(&cfg, k_ensemble<1024, 2>, a));
  }
  EK(cudaGetLastError());
  return 0;
}

// Kernels one ensemble pass launches.
int pass_kernels(const fen_ensemble* e) { return (e->npacks ? 1 : 0) + (e->npacks4 ? 1 : 0); }

// One ensemble pass: the kCl-CTA launch on e->stream and, when the split placed runs there,
// the 4-CTA launch on stream2 beside it (fork/join events, so a captured graph holds the two
// as parallel nodes).  The runs are independent and no CTA waits on the other launch.
int launch(fen_ensemble* e, int nsteps, int mode = 0) {
  EnsArgs a;
  memset(&a, 0, sizeof(a));
  a.cls = e->d_cls;
  a.packs = e->d_packs;
  a.npacks = e->npacks;
  a.run_list = e->d_runlist;
  a.run_off = e->d_off;
  a.state = e->state;
  a.scal = e->d_scal;
  a.counter = e->d_counter;
  a.nsteps = nsteps;
  a.cfl = e->cfl;
  a.mode = mode;
  a.every = mode ? e->adj_every : 1;
  a.nseg = mode ? e->adj_nseg : 1;
  a.abuf = e->abuf;
  a.aoff = e->d_aoff;
  a.rec = e->rec;
  EK(cudaMemsetAsync(e->d_counter, 0, 2 * sizeof(int), e->stream));
  const bool two = e->npacks4 > 0;
  if (two) EK(cudaEventRecord(e->fork, e->stream));
  // the kCl-CTA launch is issued first so that its clusters are placed before the small ones
  int r;
  if (e->npacks && (r = launch_one(e, a, kCl, e->nclusters, e->smem, e->stream))) return r;
  if (two) {
    EK(cudaStreamWaitEvent(e->stream2, e->fork, 0));
    EnsArgs b = a;
    b.packs = e->d_packs4;
    b.npacks = e->npacks4;
    b.run_list = e->d_runlist4;
    b.counter = e->d_counter + 1;
    if ((r = launch_one(e, b, 4, e->nclusters4, e->smem4, e->stream2))) return r;
    EK(cudaEventRecord(e->join, e->stream2));
    EK(cudaStreamWaitEvent(e->stream, e->join, 0));
  }
  return 0;
}

int push_scal(fen_ensemble* e) {
  if (e->scal_dirty) {
    EK(cudaMemcpyAsync(e->d_scal, e->scal.data(), e->scal.size() * sizeof(RunScal), cudaMemcpyHostToDevice, e->stream));
    e->scal_dirty = false;
  }
  return 0;
}

int pull_scal(fen_ensemble* e) {
  EK(cudaMemcpyAsync(e->scal.data(), e->d_scal, e->scal.size() * sizeof(RunScal), cudaMemcpyDeviceToHost, e->stream));
  EK(cudaStreamSynchronize(e->stream));
  return 0;
}

int advance_graph(fen_ensemble* e, int nsteps, float* ms) {
  int r;
  if ((r = push_scal(e))) return r;
  if (e->exec_steps != nsteps) {
    if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
    if (e->graph) { cudaGraphDestroy(e->graph); e->graph = nullptr; }
    EK(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    r = launch(e, nsteps);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    if (r) { if (g) cudaGraphDestroy(g); return r; }
    EK(ce);
    e->graph = g;
    EK(cudaGraphInstantiate(&e->exec, e->graph, 0));
    e->exec_steps = nsteps;
  }
  cudaEvent_t e0, e1;
  EK(cudaEventCreate(&e0));
  EK(cudaEventCreate(&e1));
  EK(cudaEventRecord(e0, e->stream));
  EK(cudaGraphLaunch(e->exec, e->stream));
  EK(cudaEventRecord(e1, e->stream));
  EK(cudaEventSynchronize(e1));
  EK(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  e->launches += pass_kernels(e);
  return pull_scal(e);
}

std::string device_key(int dev) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "unknown";
  std::string s = p.name;
  for (auto& ch : s)
    if (ch == ' ') ch = '_';
  return s + "_sm" + std::to_string(p.multiProcessorCount);
}

}  // namespace

extern "C" {

size_t fen_ensemble_smem_bytes(int n, int groups) {
  if (n <= 0 || groups <= 0 || n % groups) return 0;
  return smem_bytes(n, groups) + kSmemReserve;
}

int fen_ensemble_create(int nruns, const int* n, const double* viscosity, double length, double cfl, double forcing_amplitude,
                        int forcing_wavenumber, fen_ensemble** out) {
  if (!out || nruns < 1 || !n || !viscosity || !(length > 0) || !(cfl > 0)) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  *out = nullptr;
  for (int q = 0; q < nruns; ++q) {
    FFTPlan P;
    if (n[q] < 8 || n[q] % 4 != 0 || n[q] % 9 == 0 || !plan_len(n[q], P) || !plan_len(n[q] / 2, P))
      return fen_internal_fail(FEN_ERR_ARG,
                               ("ensemble run " + std::to_string(q) + ": N must be 2^a 3^b with a >= 2, b <= 1, N >= 8").c_str());
    if (!(viscosity[q] > 0)) return fen_internal_fail(FEN_ERR_ARG, "viscosity must be positive");
    bool ok = false;
    for (int G = 1; G <= kCl; G *= 2) ok = ok || g_feasible(n[q], G);
    if (!ok) return fen_internal_fail(FEN_ERR_ARG, ("ensemble run " + std::to_string(q) + ": N = " + std::to_string(n[q]) +
                                                    " does not fit a cluster's shared memory").c_str());
  }
  fen_ensemble* e = new fen_ensemble();
  e->nruns = nruns;
  e->n.assign(n, n + nruns);
  e->nu.assign(viscosity, viscosity + nruns);
  e->L = length;
  e->cfl = cfl;
  e->famp = forcing_amplitude;
  e->fk = forcing_wavenumber;
  cudaError_t ce = cudaGetDevice(&e->dev);
  if (ce != cudaSuccess) { delete e; return fen_internal_fail(FEN_ERR_CUDA, cudaGetErrorString(ce)); }
  int cc = 0;
  cudaDeviceGetAttribute(&cc, cudaDevAttrClusterLaunch, e->dev);
  if (!cc) { delete e; return fen_internal_fail(FEN_ERR_CUDA, "device has no thread-block cluster launch"); }
  std::vector<int> sizes(e->n);
  std::sort(sizes.begin(), sizes.end(), std::greater<int>());
  sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
  e->cls_n = sizes;
  e->run_cls.resize(nruns);
  for (int q = 0; q < nruns; ++q) e->run_cls[q] = (int)(std::find(sizes.begin(), sizes.end(), e->n[q]) - sizes.begin());
  e->cls_host.resize(sizes.size());
  e->cls_g.resize(sizes.size());
  int r = 0;
  for (size_t c = 0; c < sizes.size() && !r; ++c) {
    r = build_class(e, sizes[c], e->cls_host[c]);
    int G = 1;  // default tile: the fewest CTAs per run that fit
    while (!g_feasible(sizes[c], G)) G *= 2;
    e->cls_g[c] = G;
  }
  if (r) { fen_ensemble_destroy(e); return r; }
  e->off.resize(nruns);
  long long tot = 0;
  for (int q = 0; q < nruns; ++q) {
    e->off[q] = tot;
    tot += 5LL * e->n[q] * e->n[q];
  }
  e->scal.assign(nruns, RunScal{});
  for (int q = 0; q < nruns; ++q) {
    const double d = length / e->n[q];
    e->scal[q].nu = e->nu[q];
    e->scal[q].dt_visc = 0.125 * d * d / e->nu[q];
    e->scal[q].dt = e->scal[q].dt_o = std::min(cfl * d, e->scal[q].dt_visc);
    e->scal[q].maxvel = 0.0;
  }
  e->scal_dirty = true;
  auto fail_cuda = [&](cudaError_t err, const char* what) {
    fen_ensemble_destroy(e);
    return fen_internal_fail(FEN_ERR_CUDA, (std::string(what) + ": " + cudaGetErrorString(err)).c_str());
  };
  if ((ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail_cuda(ce, "stream");
  if ((ce = cudaStreamCreateWithFlags(&e->stream2, cudaStreamNonBlocking)) != cudaSuccess) return fail_cuda(ce, "stream");
  if ((ce = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming)) != cudaSuccess ||
      (ce = cudaEventCreateWithFlags(&e->join, cudaEventDisableTiming)) != cudaSuccess)
    return fail_cuda(ce, "events");
  if ((ce = cudaMalloc(&e->state, tot * sizeof(float))) != cudaSuccess) return fail_cuda(ce, "state");
  if ((ce = cudaMemset(e->state, 0, tot * sizeof(float))) != cudaSuccess) return fail_cuda(ce, "state");
  if ((ce = cudaMalloc(&e->d_off, nruns * sizeof(long long))) != cudaSuccess) return fail_cuda(ce, "offsets");
  if ((ce = cudaMemcpy(e->d_off, e->off.data(), nruns * sizeof(long long), cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail_cuda(ce, "offsets");
  if ((ce = cudaMalloc(&e->d_scal, nruns * sizeof(RunScal))) != cudaSuccess) return fail_cuda(ce, "scalars");
  if ((ce = cudaMalloc(&e->d_cls, sizes.size() * sizeof(ClassDesc))) != cudaSuccess) return fail_cuda(ce, "classes");
  if ((ce = cudaMalloc(&e->d_counter, 2 * sizeof(int))) != cudaSuccess) return fail_cuda(ce, "counter");
  if ((r = build_packs(e, {}))) { fen_ensemble_destroy(e); return r; }
  *out = e;
  return 0;
}

int fen_ensemble_destroy(fen_ensemble* e) {
  if (!e) return 0;
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  for (void* b : e->bufs) cudaFree(b);
  if (e->stream2) cudaStreamSynchronize(e->stream2);
  void* ptrs[] = {e->state, e->d_off, e->d_scal, e->d_cls, e->d_packs, e->d_runlist, e->d_counter, e->abuf, e->d_aoff, e->rec,
                  e->d_packs4, e->d_runlist4};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->join) cudaEventDestroy(e->join);
  if (e->stream2) cudaStreamDestroy(e->stream2);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return 0;
}

int fen_ensemble_upload(fen_ensemble* e, int run, const double* u, const double* v, const double* p) {
  if (!e || run < 0 || run >= e->nruns || !u || !v) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  const int N = e->n[run];
  const size_t NN = (size_t)N * N;
  std::vector<float> h(5 * NN, 0.f);
  double mv = 0.0;
  for (size_t k = 0; k < NN; ++k) {
    h[k] = (float)u[k];
    h[NN + k] = (float)v[k];
    h[2 * NN + k] = p ? (float)p[k] : 0.f;
    const double vel = fabs((double)h[k]) + fabs((double)h[NN + k]);
    if (vel > mv || vel != vel) mv = vel;
  }
  EK(cudaMemcpyAsync(e->state + e->off[run], h.data(), 5 * NN * sizeof(float), cudaMemcpyHostToDevice, e->stream));
  EK(cudaStreamSynchronize(e->stream));
  e->scal[run].maxvel = mv;
  e->scal[run].t = 0.0;
  e->scal[run].nan = 0;
  e->scal_dirty = true;
  return 0;
}

int fen_ensemble_download(fen_ensemble* e, int run, double* u, double* v, double* p) {
  if (!e || run < 0 || run >= e->nruns) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  const int N = e->n[run];
  const size_t NN = (size_t)N * N;
  std::vector<float> h(3 * NN);
  EK(cudaMemcpyAsync(h.data(), e->state + e->off[run], 3 * NN * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
  EK(cudaStreamSynchronize(e->stream));
  for (size_t k = 0; k < NN; ++k) {
    if (u) u[k] = h[k];
    if (v) v[k] = h[NN + k];
    if (p) p[k] = h[2 * NN + k];
  }
  return 0;
}

int fen_ensemble_set_timestep(fen_ensemble* e, double U) {
  if (!e || !(U > 0)) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  for (int q = 0; q < e->nruns; ++q) {
    const double d = e->L / e->n[q];
    e->scal[q].dt = e->scal[q].dt_o = std::min(e->cfl * d / U, e->scal[q].dt_visc);
  }
  e->scal_dirty = true;
  return 0;
}

int fen_ensemble_advance(fen_ensemble* e, int nsteps, double* ms) {
  if (!e || nsteps < 1) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  float f = 0.f;
  int r;
  if ((r = advance_graph(e, nsteps, &f))) return r;
  if (ms) *ms = f;
  for (int q = 0; q < e->nruns; ++q)
    if (e->scal[q].nan) return fen_internal_fail(FEN_ERR_NAN, ("NaN in the velocity of ensemble run " + std::to_string(q)).c_str());
  return 0;
}

int fen_ensemble_status(fen_ensemble* e, int run, double* out) {
  if (!e || run < 0 || run >= e->nruns || !out) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  const RunScal& s = e->scal[run];
  out[0] = s.t;
  out[1] = s.dt;
  out[2] = s.dt_o;
  out[3] = s.maxvel;
  out[4] = s.ke;
  out[5] = s.maxdiv;
  out[6] = s.nan;
  out[7] = s.nu;
  return 0;
}

int fen_ensemble_config(fen_ensemble* e, int* threads, int* sizes, int* groups, int* nclasses, int* nclusters) {
  if (!e) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  if (threads) *threads = e->threads;
  if (nclasses) *nclasses = (int)e->cls_n.size();
  if (nclusters) *nclusters = e->nclusters;
  for (size_t c = 0; c < e->cls_n.size(); ++c) {
    if (sizes) sizes[c] = e->cls_n[c];
    if (groups) groups[c] = e->cls_g[c];
  }
  return 0;
}

int fen_ensemble_set_config(fen_ensemble* e, int threads, const int* groups) {
  if (!e || (threads != 512 && threads != 1024)) return fen_internal_fail(FEN_ERR_ARG, "threads must be 512 or 1024");
  if (groups)
    for (size_t c = 0; c < e->cls_n.size(); ++c)
      if (!g_feasible(e->cls_n[c], groups[c]))
        return fen_internal_fail(FEN_ERR_ARG, ("N = " + std::to_string(e->cls_n[c]) + " on " + std::to_string(groups[c]) +
                                               " CTAs does not fit").c_str());
  e->threads = threads;
  if (groups)
    for (size_t c = 0; c < e->cls_n.size(); ++c) e->cls_g[c] = groups[c];
  return build_packs(e, {});
}

long long fen_ensemble_launches(fen_ensemble* e) { return e ? e->launches : 0; }

}  // extern "C"

// ---- forward/adjoint pair -----------------------------------------------------------------
namespace {
int timed_launch(fen_ensemble* e, int nsteps, int mode, float* ms) {
  int r;
  if ((r = push_scal(e))) return r;
  cudaEvent_t e0, e1;
  EK(cudaEventCreate(&e0));
  EK(cudaEventCreate(&e1));
  EK(cudaEventRecord(e0, e->stream));
  if ((r = launch(e, nsteps, mode))) return r;
  EK(cudaEventRecord(e1, e->stream));
  EK(cudaEventSynchronize(e1));
  EK(cudaEventElapsedTime(ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  e->launches += pass_kernels(e);
  return pull_scal(e);
}
}  // namespace

extern "C" {

int fen_ensemble_adjoint_setup(fen_ensemble* e, int nsteps, int every) {
  if (!e || nsteps < 1 || every < 1) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  every = std::min(every, nsteps);
  const int nseg = (nsteps + every - 1) / every;
  if (e->abuf) cudaFree(e->abuf);
  if (e->d_aoff) cudaFree(e->d_aoff);
  if (e->rec) cudaFree(e->rec);
  e->abuf = nullptr;
  e->d_aoff = nullptr;
  e->rec = nullptr;
  e->aoff.resize(e->nruns);
  long long tot = 0;
  for (int q = 0; q < e->nruns; ++q) {
    e->aoff[q] = tot;
    tot += AdjLayout::size((long long)e->n[q] * e->n[q], nseg, every);
    tot = (tot + 63) / 64 * 64;
  }
  cudaError_t ce;
  if ((ce = cudaMalloc(&e->abuf, tot * sizeof(float))) != cudaSuccess)
    return fen_internal_fail(FEN_ERR_NOMEM, (std::string("adjoint storage: ") + cudaGetErrorString(ce)).c_str());
  EK(cudaMemset(e->abuf, 0, tot * sizeof(float)));
  EK(cudaMalloc(&e->d_aoff, e->nruns * sizeof(long long)));
  EK(cudaMemcpy(e->d_aoff, e->aoff.data(), e->nruns * sizeof(long long), cudaMemcpyHostToDevice));
  EK(cudaMalloc(&e->rec, (size_t)e->nruns * nsteps * 2 * sizeof(double)));
  e->adj_nsteps = nsteps;
  e->adj_every = every;
  e->adj_nseg = nseg;
  e->adj_ready = false;
  return 0;
}

int fen_ensemble_adjoint_forward(fen_ensemble* e, double* ms) {
  if (!e || !e->abuf) return fen_internal_fail(FEN_ERR_STATE, "fen_ensemble_adjoint_setup first");
  float f = 0.f;
  int r;
  if ((r = timed_launch(e, e->adj_nsteps, 1, &f))) return r;
  if (ms) *ms = f;
  e->adj_ready = true;
  for (int q = 0; q < e->nruns; ++q)
    if (e->scal[q].nan) return fen_internal_fail(FEN_ERR_NAN, ("NaN in the velocity of ensemble run " + std::to_string(q)).c_str());
  return 0;
}

int fen_ensemble_adjoint_seed(fen_ensemble* e, int run, const double* lam_u, const double* lam_v) {
  if (!e || run < 0 || run >= e->nruns || !lam_u || !lam_v) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  if (!e->abuf) return fen_internal_fail(FEN_ERR_STATE, "fen_ensemble_adjoint_setup first");
  const long long N2 = (long long)e->n[run] * e->n[run];
  const AdjLayout AL(N2, e->adj_nseg, e->adj_every);
  std::vector<float> h(5 * N2, 0.f);
  for (long long k = 0; k < N2; ++k) {
    h[k] = (float)lam_u[k];
    h[N2 + k] = (float)lam_v[k];
  }
  EK(cudaMemcpy(e->abuf + e->aoff[run] + AL.adj, h.data(), 5 * N2 * sizeof(float), cudaMemcpyHostToDevice));
  return 0;
}

int fen_ensemble_adjoint_backward(fen_ensemble* e, double* ms) {
  if (!e || !e->adj_ready) return fen_internal_fail(FEN_ERR_STATE, "fen_ensemble_adjoint_forward first");
  float f = 0.f;
  int r;
  if ((r = timed_launch(e, e->adj_nsteps, 2, &f))) return r;
  if (ms) *ms = f;
  return 0;
}

int fen_ensemble_adjoint_gradient(fen_ensemble* e, int run, double* g_u, double* g_v) {
  if (!e || run < 0 || run >= e->nruns || !g_u || !g_v) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  if (!e->abuf) return fen_internal_fail(FEN_ERR_STATE, "fen_ensemble_adjoint_setup first");
  const long long N2 = (long long)e->n[run] * e->n[run];
  const AdjLayout AL(N2, e->adj_nseg, e->adj_every);
  std::vector<float> h(2 * N2);
  EK(cudaMemcpy(h.data(), e->abuf + e->aoff[run] + AL.adj, 2 * N2 * sizeof(float), cudaMemcpyDeviceToHost));
  for (long long k = 0; k < N2; ++k) {
    g_u[k] = h[k];
    g_v[k] = h[N2 + k];
  }
  return 0;
}

int fen_ensemble_adjoint_dts(fen_ensemble* e, int run, double* dt, double* dt_o) {
  if (!e || run < 0 || run >= e->nruns || !dt || !dt_o) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  if (!e->adj_ready) return fen_internal_fail(FEN_ERR_STATE, "fen_ensemble_adjoint_forward first");
  std::vector<double> h((size_t)2 * e->adj_nsteps);
  EK(cudaMemcpy(h.data(), e->rec + (size_t)run * e->adj_nsteps * 2, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int s = 0; s < e->adj_nsteps; ++s) {
    dt[s] = h[2 * s];
    dt_o[s] = h[2 * s + 1];
  }
  return 0;
}

}  // extern "C"

extern "C" {

// Autotuner: per grid size, the CTAs per run G (tile = N/G rows) among those that fit; then
// the CTA size.  Each candidate advances a sample of the ensemble's own runs for `steps`
// steps (the state is restored afterwards) and the fastest is kept.  Results are cached in
// `cache_path` (one "device N G" or "device threads T" line each) and reused when present.
int fen_ensemble_tune(fen_ensemble* e, int steps, const char* cache_path) {
  if (!e || steps < 1) return fen_internal_fail(FEN_ERR_ARG, "bad argument");
  const std::string key = device_key(e->dev);
  std::map<int, int> cached_g;
  int cached_t = 0, cached_s = 0;
  if (cache_path && cache_path[0]) {
    std::ifstream f(cache_path);
    std::string line;
    while (std::getline(f, line)) {
      std::istringstream ss(line);
      std::string k, what;
      int a = 0, b = 0;
      if (!(ss >> k >> what >> a)) continue;
      if (k != key) continue;
      if (what == "threads") cached_t = a;
      else if (what == "share") cached_s = a;
      else if (what == "N" && (ss >> b)) cached_g[a] = b;
    }
  }
  bool all = (cached_t == 512 || cached_t == 1024) && cached_s > 0;
  for (int N : e->cls_n) all = all && cached_g.count(N) && g_feasible(N, cached_g[N]);
  int r;
  if (all) {
    for (size_t c = 0; c < e->cls_n.size(); ++c) e->cls_g[c] = cached_g[e->cls_n[c]];
    e->threads = cached_t;
    e->share = cached_s;
    return build_packs(e, {});
  }
  // back up the state and the scalars
  const long long tot = e->off.back() + 5LL * e->n.back() * e->n.back();
  float* backup = nullptr;
  EK(cudaMalloc(&backup, tot * sizeof(float)));
  auto restore = [&]() -> int {
    EK(cudaMemcpyAsync(e->state, backup, tot * sizeof(float), cudaMemcpyDeviceToDevice, e->stream));
    EK(cudaStreamSynchronize(e->stream));
    return 0;
  };
  EK(cudaMemcpyAsync(backup, e->state, tot * sizeof(float), cudaMemcpyDeviceToDevice, e->stream));
  if ((r = push_scal(e))) { cudaFree(backup); return r; }
  std::vector<RunScal> scal0 = e->scal;
  auto trial = [&](const std::vector<int>& subset, float* ms) -> int {
    int rr;
    if ((rr = build_packs(e, subset))) return rr;
    e->scal = scal0;
    e->scal_dirty = true;
    if ((rr = push_scal(e))) return rr;
    if ((rr = launch(e, 1))) return rr;  // warm-up
    EK(cudaStreamSynchronize(e->stream));
    cudaEvent_t a0, a1;
    EK(cudaEventCreate(&a0));
    EK(cudaEventCreate(&a1));
    EK(cudaEventRecord(a0, e->stream));
    if ((rr = launch(e, steps))) return rr;
    EK(cudaEventRecord(a1, e->stream));
    EK(cudaEventSynchronize(a1));
    EK(cudaEventElapsedTime(ms, a0, a1));
    cudaEventDestroy(a0);
    cudaEventDestroy(a1);
    e->launches += 2 * pass_kernels(e);
    return restore();
  };
  e->threads = 1024;
  const std::vector<int> g0 = e->cls_g;
  for (size_t c = 0; c < e->cls_n.size() && !r; ++c) {
    std::vector<int> subset;
    for (int q = 0; q < e->nruns && (int)subset.size() < 4 * kCl * std::max(1, e->nclusters); ++q)
      if (e->run_cls[q] == (int)c) subset.push_back(q);
    float best = 1e30f;
    int bestG = g0[c];
    for (int G = 1; G <= kCl && !r; G *= 2) {
      if (!g_feasible(e->cls_n[c], G)) continue;
      e->cls_g[c] = G;
      float ms = 0.f;
      r = trial(subset, &ms);
      if (!r && ms < best) { best = ms; bestG = G; }
    }
    e->cls_g[c] = bestG;
  }
  float best_t = 1e30f;
  int bt = 1024;
  for (int T : {1024, 512}) {
    if (r) break;
    e->threads = T;
    float ms = 0.f;
    r = trial({}, &ms);
    if (!r && ms < best_t) { best_t = ms; bt = T; }
  }
  e->threads = bt;
  // the 4-CTA launch's share of the cells: the two concurrent launches should end together
  if (!r && e->split && kCl == 8) {
    float best_s = 1e30f;
    int bs = e->share;
    for (int sh : {60, 70, 80, 90, 100}) {
      e->share = sh;
      float ms = 0.f;
      r = trial({}, &ms);
      if (r) break;
      if (ms < best_s) { best_s = ms; bs = sh; }
    }
    e->share = bs;
  }
  e->scal = scal0;
  e->scal_dirty = true;
  cudaFree(backup);
  if (r) return r;
  if ((r = build_packs(e, {}))) return r;
  if (cache_path && cache_path[0]) {
    std::ofstream f(cache_path, std::ios::app);
    for (size_t c = 0; c < e->cls_n.size(); ++c) f << key << " N " << e->cls_n[c] << " " << e->cls_g[c] << "\n";
    f << key << " threads " << e->threads << "\n";
    f << key << " share " << e->share << "\n";
  }
  return 0;
}

}  // extern "C"
