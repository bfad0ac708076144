// Batched shared-memory FFTs for the fast direct Poisson solve (FEN src/poisson.f90).
//
// FEN calls FFTW once per 1D line (dfftw_execute_dft_r2c / dft / dft_c2r / r2r with
// REDFT10 and REDFT01, poisson.f90:336-593, 967-1432).  Here one CTA transforms a batch of
// lines staged in shared memory with a mixed-radix (16, 8, 4, 2, 3) Stockham autosort FFT.  Real
// transforms use the half-length complex FFT with the usual even/odd packing, and the DCTs
// use Makhoul's reordering, so every transform costs one complex FFT of length n/2.
// Transform definitions follow FFTW's documented ones: unnormalised, forward sign -1,
// REDFT10 Y_k = 2 sum x_j cos(pi (2j+1) k / 2n), REDFT01 Y_k = x_0 + 2 sum_{j>=1} x_j
// cos(pi j (2k+1) / 2n).
#pragma once
#include "fen_types.cuh"

namespace fen {

constexpr int kMaxStages = 16;
// Largest FFT radices compiled (build-time tuning knobs; see fft_max_radix).
#ifndef FEN_FFT_MAXR64
#define FEN_FFT_MAXR64 8
#endif
#ifndef FEN_FFT_MAXR32_ROW
#define FEN_FFT_MAXR32_ROW 8
#endif
#ifndef FEN_FFT_MAXR32_COL
#define FEN_FFT_MAXR32_COL 16
#endif

// Radix schedule of one complex FFT length, built on the host.
struct FFTPlan {
  int M;                       // complex length
  int nst;                     // stages
  int R[kMaxStages];           // radices: 16s or 8s first, then at most one 4 and one 2, then 3s
  unsigned nsm[kMaxStages];    // fast-division multiplier of the stage's span Ns (fft_magic)
  int nb[kMaxStages];          // M / R: butterflies of the stage per line
  int ts[kMaxStages];          // M / (Ns R): the stage's twiddle stride
};

// Multiplier m of the fast division n / d = umulhi(n, m), m = floor(2^32 / d) + 1 (0 for
// d = 1); exact for n * d < 2^32, which holds for every index here.  32-bit arithmetic only:
// floor(2^32 / d) = floor((2^32 - 1) / d) unless d is a power of two.
__host__ __device__ inline unsigned fft_magic(unsigned d) {
  return d > 1 ? 0xffffffffu / d + 1u + ((d & (d - 1)) == 0 ? 1u : 0u) : 0u;
}

// Fill the fast-division multipliers of a plan's radix schedule.
inline void fft_plan_magic(FFTPlan& P) {
  unsigned ns = 1;
  for (int s = 0; s < P.nst; ++s) {
    P.nsm[s] = fft_magic(ns);
    P.nb[s] = P.M / P.R[s];
    P.ts[s] = P.M / ((int)ns * P.R[s]);
    ns *= (unsigned)P.R[s];
  }
}

// Twiddle tables of one transform axis (device pointers; values computed on the host in
// FP64 with libm cos/sin, stored as double2 for FP64 kernels and rounded to float2 for FP32).
struct AxisTw {
  const double2* wM;   // exp(-2 pi i m / M),      m < M   (complex FFT of length M = n/2)
  const double2* wN;   // exp(-2 pi i k / n),      k <= n/2 (real-FFT packing)
  const double2* wD;   // exp(-i pi k / (2n)),     k < n   (DCT packing)
};

// Twiddle load.  FP64 kernels read double2 tables; FP32 kernels are handed float2 tables
// through the same pointer slot (no FP64 conversion inside the transform loops).
template <typename T2>
__device__ __forceinline__ T2 ldtw(const double2* p, int m);
template <>
__device__ __forceinline__ double2 ldtw<double2>(const double2* p, int m) { return __ldg(p + m); }
template <>
__device__ __forceinline__ float2 ldtw<float2>(const double2* p, int m) {
  return __ldg(reinterpret_cast<const float2*>(p) + m);
}

// In-register DFT of size R (R = 2, 3, 4), sign DIR (-1 forward, +1 backward).
template <int DIR, typename T2>
__device__ __forceinline__ void dft2(T2& a, T2& b) {
  T2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}
template <int DIR, typename T2>
__device__ __forceinline__ void dft4(T2& a, T2& b, T2& c, T2& d) {
  T2 s0 = cadd(a, c), s1 = csub(a, c), s2 = cadd(b, d), s3 = cmul_mi<DIR>(csub(b, d));
  a = cadd(s0, s2);
  c = csub(s0, s2);
  b = cadd(s1, s3);
  d = csub(s1, s3);
}
template <int DIR, typename T2>
__device__ __forceinline__ void dft3(T2& a, T2& b, T2& c) {
  typedef decltype(T2::x) T;
  const T h = (T)0.86602540378443864676;  // sqrt(3)/2
  T2 s = cadd(b, c), d = csub(b, c);
  T2 m = mk<T2>(a.x - (T)0.5 * s.x, a.y - (T)0.5 * s.y);
  a = cadd(a, s);
  // q = -i*h*d (forward) or +i*h*d (backward)
  T2 q = (DIR < 0) ? mk<T2>(h * d.y, -h * d.x) : mk<T2>(-h * d.y, h * d.x);
  b = cadd(m, q);
  c = csub(m, q);
}

// Division by a run-time constant d with multiplier fft_magic(d).
struct FastDiv {
  unsigned d, m;
};
__device__ __forceinline__ int fdivi(int n, FastDiv f) { return f.d > 1 ? (int)__umulhi((unsigned)n, f.m) : n; }
// (q, r) = (t / d, t % d) for 0 <= t, t * d < 2^32.
__device__ __forceinline__ void divmod(int t, FastDiv f, int& q, int& r) {
  q = fdivi(t, f);
  r = t - q * (int)f.d;
}

// cos(2 pi m/16), m = 0..15 (the in-register radix-8/16 rotations), as a constant of the
// kernel's own type: a double narrowed at run time would be a conversion on the FP64 pipe
// wherever the unrolled index is not folded.
template <typename T>
__device__ __forceinline__ T cos16(int m) {
  switch (m & 15) {
    case 0: return T(1.0);
    case 1: case 15: return T(0.92387953251128674);
    case 2: case 14: return T(0.70710678118654752);
    case 3: case 13: return T(0.38268343236508977);
    case 4: case 12: return T(0.0);
    case 5: case 11: return T(-0.38268343236508977);
    case 6: case 10: return T(-0.70710678118654752);
    case 8: return T(-1.0);
    default: return T(-0.92387953251128674);  // 7, 9
  }
}

// v * exp(DIR 2 pi i m / R) for R | 16 and m known at compile time after unrolling.
template <int DIR, int R, typename T2>
__device__ __forceinline__ T2 rot16(T2 v, int m) {
  typedef decltype(T2::x) T;
  const int e = (m * (16 / R)) & 15;
  if (e == 0) return v;
  if (e == 4) return DIR < 0 ? mk<T2>(v.y, -v.x) : mk<T2>(-v.y, v.x);
  if (e == 8) return mk<T2>(-v.x, -v.y);
  if (e == 12) return DIR < 0 ? mk<T2>(-v.y, v.x) : mk<T2>(v.y, -v.x);
  const T c = cos16<T>(e), s = (T)DIR * cos16<T>(e + 12);
  return mk<T2>(fmx(v.x, c, -(v.y * s)), fmx(v.x, s, v.y * c));
}

// In-register DFT of size R in natural order (R = 2, 3, 4, 8, 16); 8 and 16 are A x B
// compositions (DFT-A over the stride-B subsequences, twiddles w_R^(n2 k1), DFT-B).
template <int DIR, int R, typename T2>
__device__ __forceinline__ void dft_r(T2 (&x)[16]);
template <int DIR, int A, int B, typename T2>
__device__ __forceinline__ void dft_ab(T2 (&x)[16]) {
  T2 y[A * B];
#pragma unroll
  for (int n2 = 0; n2 < B; ++n2) {
    T2 tt[16];
#pragma unroll
    for (int n1 = 0; n1 < A; ++n1) tt[n1] = x[B * n1 + n2];
    dft_r<DIR, A, T2>(tt);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = rot16<DIR, A * B, T2>(tt[k1], n2 * k1);
  }
#pragma unroll
  for (int k1 = 0; k1 < A; ++k1) {
    T2 tt[16];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) tt[n2] = y[n2 * A + k1];
    dft_r<DIR, B, T2>(tt);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) x[k1 + A * k2] = tt[k2];
  }
}
template <int DIR, int R, typename T2>
__device__ __forceinline__ void dft_r(T2 (&x)[16]) {
  if (R == 2) dft2<DIR>(x[0], x[1]);
  else if (R == 3) dft3<DIR>(x[0], x[1], x[2]);
  else if (R == 4) dft4<DIR>(x[0], x[1], x[2], x[3]);
  else if (R == 8) dft_ab<DIR, 4, 2, T2>(x);
  else if (R == 16) dft_ab<DIR, 4, 4, T2>(x);
}

// One radix-R Stockham pass over nl lines (element (line l, position p) at buf[l*ls + p*es]),
// lines fastest over threads (strided layouts stay bank-conflict free).
template <int DIR, int R, typename T2>
__device__ __forceinline__ void fft_pass_r(const T2* __restrict__ src0, T2* __restrict__ dst0, int work, FastDiv fnl,
                                           int ls, int es, int Ns, FastDiv fns, bool ns_pow2, int nb, int tstep,
                                           const double2* __restrict__ tw) {
  for (int t = threadIdx.x; t < work; t += blockDim.x) {
    const int j = fdivi(t, fnl);
    const int l = t - j * (int)fnl.d;
    const int k = ns_pow2 ? (j & (Ns - 1)) : j - fdivi(j, fns) * Ns;
    const T2* src = src0 + l * ls;
    T2* dst = dst0 + l * ls;
    T2 v[16];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = src[(j + q * nb) * es];
    if (Ns > 1) {
#pragma unroll
      for (int q = 1; q < R; ++q) {
        const T2 w = ldtw<T2>(tw, q * k * tstep);
        v[q] = (DIR < 0) ? cmul(v[q], w) : cmulc(v[q], w);
      }
    }
    dft_r<DIR, R, T2>(v);
    const int o = (j - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) dst[(o + q * Ns) * es] = v[q];
  }
}

// Largest radix compiled per kernel; the host's plans (make_plan's maxr) match.  FP64
// transforms are FP64-issue bound and gain from radix 8 (fewer twiddle products and adds).
// FP32 column transforms take radix 16; FP32 x-line transforms radix 8 at 5 CTAs per SM
// (measured on the mixed channel step, 512-point rows: radix 4 at 6 CTAs 5.31 ms, radix 8 at
// 5 CTAs 5.22, at 4 CTAs 5.27, radix 16 at 3 CTAs 5.50).
constexpr int kFftMaxR64 = FEN_FFT_MAXR64;
constexpr int kFftMaxR32Row = FEN_FFT_MAXR32_ROW;
constexpr int kFftMaxR32Col = FEN_FFT_MAXR32_COL;
template <typename T, bool CONTIG>
__host__ __device__ constexpr int fft_max_radix() {
  return sizeof(T) == 8 ? kFftMaxR64 : (CONTIG ? kFftMaxR32Row : kFftMaxR32Col);
}

// One complex FFT of length P.M on `nl` lines held in shared memory, radix schedule P.R
// (16, 8, 4, 2, 3; none above MAXR).  Returns the buffer holding the result (a or b).
template <int DIR, int MAXR, typename T2>
__device__ T2* smem_fft(T2* a, T2* b, FastDiv fnl, int ls, int es, const FFTPlan& P, const double2* tw) {
  const int nl = (int)fnl.d;
  int Ns = 1;
  for (int s = 0; s < P.nst; ++s) {
    // per-stage spans come from the host plan: a run-time division here would compile to
    // conversions on the FP64 pipe, issued by every thread at every stage
    const int R = P.R[s];
    const int nb = P.nb[s];
    const int tstep = P.ts[s];
    const int work = nl * nb;
    const bool p2 = (Ns & (Ns - 1)) == 0;
    const FastDiv fns{(unsigned)Ns, P.nsm[s]};
    if (MAXR >= 16 && R == 16) fft_pass_r<DIR, (MAXR >= 16 ? 16 : 2), T2>(a, b, work, fnl, ls, es, Ns, fns, p2, nb, tstep, tw);
    else if (MAXR >= 8 && R == 8) fft_pass_r<DIR, (MAXR >= 8 ? 8 : 2), T2>(a, b, work, fnl, ls, es, Ns, fns, p2, nb, tstep, tw);
    else if (R == 4) fft_pass_r<DIR, 4, T2>(a, b, work, fnl, ls, es, Ns, fns, p2, nb, tstep, tw);
    else if (R == 2) fft_pass_r<DIR, 2, T2>(a, b, work, fnl, ls, es, Ns, fns, p2, nb, tstep, tw);
    else fft_pass_r<DIR, 3, T2>(a, b, work, fnl, ls, es, Ns, fns, p2, nb, tstep, tw);
    __syncthreads();
    T2* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

// ------------------------------------------------------------------------------------
// Real-transform packings on lines in shared memory (complex length M = n/2).
// ------------------------------------------------------------------------------------

// r2c post-processing: Z = FFT_M(x_even + i x_odd) -> X_k, k = 0..M.
template <typename T2>
__device__ __forceinline__ T2 r2c_post(const T2* Z, int es, int M, int k, const double2* wN) {
  typedef decltype(T2::x) T;
  const T2 zk = Z[(k % M) * es];
  const T2 zc = cconj(Z[((M - k) % M) * es]);
  const T2 E = mk<T2>((T)0.5 * (zk.x + zc.x), (T)0.5 * (zk.y + zc.y));
  const T2 D = csub(zk, zc);
  const T2 O = mk<T2>((T)0.5 * D.y, (T)-0.5 * D.x);  // -i/2 * D
  return cadd(E, cmul(ldtw<T2>(wN, k), O));
}

// c2r pre-processing: X_k (k = 0..M, Hermitian half-spectrum) -> Z'_k, k = 0..M-1, such that
// IFFT_M(Z') = x_even + i x_odd of the unnormalised c2r.  X0 and XM imaginary parts ignored.
template <typename T2>
__device__ __forceinline__ T2 c2r_pre(T2 xk, T2 xmk, int M, int k, const double2* wN) {
  if (k == 0) { xk.y = 0; xmk.y = 0; }
  const T2 b = cconj(xmk);
  const T2 s = cadd(xk, b);
  const T2 d = cmulc(csub(xk, b), ldtw<T2>(wN, k));  // (X_k - conj X_{M-k}) e^{+2 pi i k/n}
  return mk<T2>(s.x - d.y, s.y + d.x);                // s + i d
}

}  // namespace fen
