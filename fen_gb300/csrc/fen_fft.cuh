// Batched shared-memory FFTs for the fast direct Poisson solve (FEN src/poisson.f90).
//
// FEN calls FFTW once per 1D line (dfftw_execute_dft_r2c / dft / dft_c2r / r2r with
// REDFT10 and REDFT01, poisson.f90:336-593, 967-1432).  Here one CTA transforms a batch of
// lines staged in shared memory with a mixed-radix (4, 2, 3) Stockham autosort FFT.  Real
// transforms use the half-length complex FFT with the usual even/odd packing, and the DCTs
// use Makhoul's reordering, so every transform costs one complex FFT of length n/2.
// Transform definitions follow FFTW's documented ones: unnormalised, forward sign -1,
// REDFT10 Y_k = 2 sum x_j cos(pi (2j+1) k / 2n), REDFT01 Y_k = x_0 + 2 sum_{j>=1} x_j
// cos(pi j (2k+1) / 2n).
#pragma once
#include "fen_types.cuh"

namespace fen {

constexpr int kMaxStages = 16;

// Radix schedule of one complex FFT length, built on the host.
struct FFTPlan {
  int M;                       // complex length
  int nst;                     // stages
  int R[kMaxStages];           // radices, 4s first, then 2, then 3
};

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

// One complex FFT of length P.M on `nl` lines held in shared memory.  Element (line l,
// position p) lives at buf[l * ls + p * es].  Threads are mapped line-fastest so that, with
// es = number of lines and ls = 1, every load and store is bank-conflict free.  Returns the
// buffer holding the result (a or b).
template <int DIR, typename T2>
__device__ T2* smem_fft(T2* a, T2* b, int nl, int ls, int es, const FFTPlan& P, const double2* tw) {
  const int M = P.M;
  int Ns = 1;
  for (int s = 0; s < P.nst; ++s) {
    const int R = P.R[s];
    const int nb = M / R;
    const int tstep = M / (Ns * R);
    const int work = nl * nb;
    for (int t = threadIdx.x; t < work; t += blockDim.x) {
      const int l = t % nl;
      const int j = t / nl;
      const int k = j % Ns;
      const T2* src = a + l * ls;
      T2* dst = b + l * ls;
      const int idxD = (j - k) * R + k;
      if (R == 4) {
        T2 v0 = src[(j) * es], v1 = src[(j + nb) * es], v2 = src[(j + 2 * nb) * es], v3 = src[(j + 3 * nb) * es];
        if (Ns > 1) {
          T2 w1 = ldtw<T2>(tw, k * tstep), w2 = ldtw<T2>(tw, 2 * k * tstep), w3 = ldtw<T2>(tw, 3 * k * tstep);
          if (DIR < 0) { v1 = cmul(v1, w1); v2 = cmul(v2, w2); v3 = cmul(v3, w3); }
          else { v1 = cmulc(v1, w1); v2 = cmulc(v2, w2); v3 = cmulc(v3, w3); }
        }
        dft4<DIR>(v0, v1, v2, v3);
        dst[(idxD) * es] = v0; dst[(idxD + Ns) * es] = v1; dst[(idxD + 2 * Ns) * es] = v2; dst[(idxD + 3 * Ns) * es] = v3;
      } else if (R == 2) {
        T2 v0 = src[(j) * es], v1 = src[(j + nb) * es];
        if (Ns > 1) {
          T2 w1 = ldtw<T2>(tw, k * tstep);
          v1 = (DIR < 0) ? cmul(v1, w1) : cmulc(v1, w1);
        }
        dft2<DIR>(v0, v1);
        dst[(idxD) * es] = v0; dst[(idxD + Ns) * es] = v1;
      } else {  // R == 3
        T2 v0 = src[(j) * es], v1 = src[(j + nb) * es], v2 = src[(j + 2 * nb) * es];
        if (Ns > 1) {
          T2 w1 = ldtw<T2>(tw, k * tstep), w2 = ldtw<T2>(tw, 2 * k * tstep);
          if (DIR < 0) { v1 = cmul(v1, w1); v2 = cmul(v2, w2); }
          else { v1 = cmulc(v1, w1); v2 = cmulc(v2, w2); }
        }
        dft3<DIR>(v0, v1, v2);
        dst[(idxD) * es] = v0; dst[(idxD + Ns) * es] = v1; dst[(idxD + 2 * Ns) * es] = v2;
      }
    }
    __syncthreads();
    T2* t = a; a = b; b = t;
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
