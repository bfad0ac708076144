// Shared device types for the FEN projection-step kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fen {

// Field boundary-condition types (FEN src/scalar.f90:17-22).
enum { FT_PERIODIC = 0, FT_DIRICHLET = 1, FT_NEUMANN = 2 };
// Faces in the reference order (scalar.f90:24-36).
enum { F_LEFT = 0, F_RIGHT = 1, F_BOTTOM = 2, F_TOP = 3, F_FRONT = 4, F_BACK = 5 };

#ifdef FEN_DEBUG_CHECKS
// Debug build (FEN_DEBUG_CHECKS): every field index passes a bounds check against its array.
// An index outside it is counted, the first one is kept, and element 0 is used instead, so no
// out-of-range access is made and nothing traps; fen_debug_checks() reports the record of
// this translation unit (the library's stepping, transfer and operator kernels).
static __device__ unsigned long long g_fen_oob_count;
static __device__ long long g_fen_oob_first;
__device__ __forceinline__ long long fen_checked(long long r, long long total) {
  if (r < 0 || r >= total) {
    if (atomicAdd(&g_fen_oob_count, 1ull) == 0ull) g_fen_oob_first = r;
    return 0;
  }
  return r;
}
#endif

// Ghosted field in HBM.  Fortran index (i, j, k), i in [0, n0+1], j in [0, n1+1] and, in
// 3D, k in [0, n2+1] (gl = 1, scalar.f90:79-81).  Rows are padded to a multiple of four
// elements and shifted by `off` = 3 so the first interior element of every row (i = 1)
// starts on a 32-byte sector.  In 2D only the k = 1 plane is stored (storage plane 0):
// FEN allocates z ghost planes there but never reads or fills them (scalar.f90:344).
struct Layout {
  int dim;
  int n0, n1, n2;   // interior cells (n2 = 1 in 2D)
  int sx;           // row pitch, elements
  int sy;           // rows per plane (n1 + 2)
  long long sp;     // plane pitch, elements
  int off;
  long long total;  // elements to allocate
  // multipliers m of the division by n0 and n1 as umulhi(x, m) (fft_magic, exact for x * n <
  // 2^32), set on the host when n0, n1 <= 4096 (fastdiv = 1): CellWalk's start-up divisions
  // then use no conversion instructions, which GB300 issues on its slow FP64 pipe
  unsigned mg0 = 0, mg1 = 0;
  int fastdiv = 0;
  // an index formed by the caller (a row base plus offsets), checked as idx checks its own
  __host__ __device__ __forceinline__ long long at(long long r) const {
#if defined(FEN_DEBUG_CHECKS) && defined(__CUDA_ARCH__)
    return fen_checked(r, total);
#else
    return r;
#endif
  }
  __host__ __device__ __forceinline__ long long idx(int i, int j, int ks) const {
    const long long r = (long long)off + i + (long long)sx * j + sp * ks;
#if defined(FEN_DEBUG_CHECKS) && defined(__CUDA_ARCH__)
    return fen_checked(r, total);
#else
    return r;
#endif
  }
};

// Interior-cell walk of a grid-stride loop over t = t0, t0 + stride, ... (Fortran order, i
// fastest).  The 0-based (i, j, k) advance by the stride's own (si, sj, sk) with carries, so
// the 64-bit divisions by n0 and n1 happen once per thread instead of once per cell.
struct CellWalk {
  long long t0, stride;
  int i, j, k, si, sj, sk;
  __device__ __forceinline__ CellWalk(const Layout& L, long long t, long long s) : t0(t), stride(s) {
    if (L.fastdiv && t < (1LL << 20) && s < (1LL << 20)) {
      // thread index and stride below 2^20, n0 and n1 at most 4096: the products stay below 2^32
      const unsigned tt = (unsigned)t, ss = (unsigned)s;
      const unsigned r = (L.n0 > 1) ? __umulhi(tt, L.mg0) : tt;
      const unsigned q = (L.n1 > 1) ? __umulhi(r, L.mg1) : r;
      i = (int)(tt - r * (unsigned)L.n0);
      j = (int)(r - q * (unsigned)L.n1);
      k = (int)q;
      const unsigned r2 = (L.n0 > 1) ? __umulhi(ss, L.mg0) : ss;
      const unsigned q2 = (L.n1 > 1) ? __umulhi(r2, L.mg1) : r2;
      si = (int)(ss - r2 * (unsigned)L.n0);
      sj = (int)(r2 - q2 * (unsigned)L.n1);
      sk = (int)q2;
      return;
    }
    long long r = t / L.n0;
    i = (int)(t - r * L.n0);
    j = (int)(r % L.n1);
    k = (int)(r / L.n1);
    r = s / L.n0;
    si = (int)(s - r * L.n0);
    sj = (int)(r % L.n1);
    sk = (int)(r / L.n1);
  }
  __device__ __forceinline__ void next(const Layout& L) {
    i += si;
    int c = i >= L.n0;
    if (c) i -= L.n0;
    j += sj + c;
    c = j >= L.n1;
    if (c) j -= L.n1;
    k += sk + c;
  }
};

// Storage plane of Fortran plane k.
template <int DIM>
__host__ __device__ __forceinline__ int kst(int k) { return DIM == 3 ? k : 0; }

// Boundary description of one ghosted field.
struct FieldBC {
  int type[6];
  const double* val[6];  // Dirichlet values over the ghosted face extents; nullptr = 0
  int c;                 // location: 'c', 'x', 'y', 'z'
};

template <typename T> struct cpx;
template <> struct cpx<double> { typedef double2 t; };
template <> struct cpx<float> { typedef float2 t; };

template <typename T2> __device__ __forceinline__ T2 mk(decltype(T2::x) a, decltype(T2::x) b) { T2 r; r.x = a; r.y = b; return r; }
template <typename T2> __device__ __forceinline__ T2 cadd(T2 a, T2 b) { return mk<T2>(a.x + b.x, a.y + b.y); }
template <typename T2> __device__ __forceinline__ T2 csub(T2 a, T2 b) { return mk<T2>(a.x - b.x, a.y - b.y); }
// Complex products with one fused multiply-add per component (two instructions fewer than
// four multiplies and two adds; the FP64 transforms are bound by FP64 issue).
__device__ __forceinline__ double fmx(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmx(float a, float b, float c) { return fmaf(a, b, c); }
template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b) {
  return mk<T2>(fmx(a.x, b.x, -(a.y * b.y)), fmx(a.x, b.y, a.y * b.x));
}
// a * conj(b)
template <typename T2> __device__ __forceinline__ T2 cmulc(T2 a, T2 b) {
  return mk<T2>(fmx(a.x, b.x, a.y * b.y), fmx(a.y, b.x, -(a.x * b.y)));
}
template <typename T2> __device__ __forceinline__ T2 cconj(T2 a) { return mk<T2>(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <int DIR, typename T2> __device__ __forceinline__ T2 cmul_mi(T2 a) { return DIR < 0 ? mk<T2>(a.y, -a.x) : mk<T2>(-a.y, a.x); }

// Per-step scalars kept on the device so a captured step needs no host round trip.
struct StepScalars {
  double dt, dt_o;          // navier_stokes.f90:24-33
  double A, B;              // AB2 coefficients (:157-158)
  double rho_over_dt;       // phi = div * rho / dt (:118)
  double dt_over_rhof;      // correction factor (:533)
  double maxvel;            // max(|u|+|v|+|w|) of the current velocity (:599-611)
  double maxdiv, maxCFL;    // checks (:570-619)
  double mean;              // Poisson mean removal (poisson.f90:491-503)
  double mean_phi;          // mixed form with refinement: mean of phi, removed where phi enters p
  double dt_visc, dt_conv;
  int err;                  // NaN detected in the reductions
  int pad;
  // the same scalars as float pairs (hi + lo) for the mixed form's double-float stencils
  float dtp[2], Ap[2], Bp[2], rdtp[2];
};

}  // namespace fen
