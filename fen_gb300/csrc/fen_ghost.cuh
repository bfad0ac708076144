// Ghost-cell fill (FEN src/scalar.f90:223-396 with src/halo.f90:12-43 on one device).
//
// The reference fills faces in the order left, right, bottom, top, front, back, each over
// the full ghosted extent of the other axes, so edges and corners see the faces filled
// before them, and a Dirichlet face-normal component also overwrites its last interior
// plane (f(hi) = bc, scalar.f90:282-283, 331-332, 377-378).  The final value of every
// written cell is therefore a composition of at most three face rules applied to ONE
// interior value.  `Resolve` evaluates that composition directly, so one launch fills all
// ghosts of several fields without ordering passes: threads write only ghost cells and
// overwritten cells and read only interior cells that no thread writes.
#pragma once
#include "fen_fft.cuh"
#include "fen_types.cuh"

namespace fen {

// Interior value source: a plain array (the default) or any functor returning T for an
// element index (the mixed form reads hi + lo pairs through one).
template <typename T>
struct PtrSrc {
  const T* f;
  __device__ __forceinline__ T operator()(long long i) const { return f[i]; }
};

template <typename T, int DIM, typename Src = PtrSrc<T>>
struct Resolve {
  Src f;
  Layout L;
  FieldBC bc;
  double shift;  // subtracted from every interior value read (0 = none)

  __device__ __forceinline__ T bcv(int face, int a, int b) const {
    const double* p = bc.val[face];
    if (!p) return T(0);
    // face arrays cover the ghosted extents: left/right (j,k), bottom/top (i,k), front/back (i,j)
    int na = (face < 2) ? L.n1 + 2 : L.n0 + 2;
    if (DIM == 2 && face < 4) b = 0;  // 2D: single stored k plane
    return (T)p[a + (long long)na * b];
  }
  __device__ __forceinline__ T state(int i, int j, int k) const {
    T v = f(L.idx(i, j, kst<DIM>(k)));
    return shift != 0.0 ? (T)(v - (T)shift) : v;
  }
  __device__ __forceinline__ T after_x(int i, int j, int k) const {
    const int N = L.n0;
    const bool nrm = (bc.c == 'x');
    if (i == 0) {
      const int t = bc.type[F_LEFT];
      if (t == FT_PERIODIC) return state(N, j, k);
      if (t == FT_DIRICHLET) return nrm ? bcv(F_LEFT, j, k) : (T)(T(2) * bcv(F_LEFT, j, k) - state(1, j, k));
      return state(1, j, k);
    }
    if (i == N + 1) {
      const int t = bc.type[F_RIGHT];
      if (t == FT_PERIODIC) return state(1, j, k);
      if (t == FT_DIRICHLET) return nrm ? bcv(F_RIGHT, j, k) : (T)(T(2) * bcv(F_RIGHT, j, k) - state(N, j, k));
      return state(N, j, k);
    }
    if (i == N && nrm && bc.type[F_RIGHT] == FT_DIRICHLET) return bcv(F_RIGHT, j, k);
    return state(i, j, k);
  }
  __device__ __forceinline__ T after_y(int i, int j, int k) const {
    const int N = L.n1;
    const bool nrm = (bc.c == 'y');
    if (j == 0) {
      const int t = bc.type[F_BOTTOM];
      if (t == FT_PERIODIC) return after_x(i, N, k);
      if (t == FT_DIRICHLET) return nrm ? bcv(F_BOTTOM, i, k) : (T)(T(2) * bcv(F_BOTTOM, i, k) - after_x(i, 1, k));
      return after_x(i, 1, k);
    }
    if (j == N + 1) {
      const int t = bc.type[F_TOP];
      if (t == FT_PERIODIC) return after_x(i, 1, k);
      if (t == FT_DIRICHLET) return nrm ? bcv(F_TOP, i, k) : (T)(T(2) * bcv(F_TOP, i, k) - after_x(i, N, k));
      return after_x(i, N, k);
    }
    if (j == N && nrm && bc.type[F_TOP] == FT_DIRICHLET) return bcv(F_TOP, i, k);
    return after_x(i, j, k);
  }
  __device__ __forceinline__ T after_z(int i, int j, int k) const {
    if (DIM == 2) return after_y(i, j, k);
    const int N = L.n2;
    const bool nrm = (bc.c == 'z');
    if (k == 0) {
      const int t = bc.type[F_FRONT];
      if (t == FT_PERIODIC) return after_y(i, j, N);
      if (t == FT_DIRICHLET) return nrm ? bcv(F_FRONT, i, j) : (T)(T(2) * bcv(F_FRONT, i, j) - after_y(i, j, 1));
      return after_y(i, j, 1);
    }
    if (k == N + 1) {
      const int t = bc.type[F_BACK];
      if (t == FT_PERIODIC) return after_y(i, j, 1);
      if (t == FT_DIRICHLET) return nrm ? bcv(F_BACK, i, j) : (T)(T(2) * bcv(F_BACK, i, j) - after_y(i, j, N));
      return after_y(i, j, N);
    }
    if (k == N && nrm && bc.type[F_BACK] == FT_DIRICHLET) return bcv(F_BACK, i, j);
    return after_y(i, j, k);
  }
  // Final value of any cell after update_ghost_nodes.
  __device__ __forceinline__ T at(int i, int j, int k) const { return after_z(i, j, k); }
};

// Number of cells one field's ghost fill writes (see ghost_target).
struct GhostCount {
  long long a, b, c;  // segments: x columns, y rows, z planes
};

template <int DIM>
__host__ __device__ inline GhostCount ghost_count(const Layout& L, const FieldBC& bc) {
  const int xov = (bc.c == 'x' && bc.type[F_RIGHT] == FT_DIRICHLET);
  const int yov = (bc.c == 'y' && bc.type[F_TOP] == FT_DIRICHLET);
  const int zov = (DIM == 3 && bc.c == 'z' && bc.type[F_BACK] == FT_DIRICHLET);
  const long long nk = (DIM == 3) ? (L.n2 - zov) : 1;
  GhostCount g;
  g.a = (long long)(2 + xov) * (L.n1 - yov) * nk;
  g.b = (long long)(2 + yov) * (L.n0 + 2) * nk;
  g.c = (DIM == 3) ? (long long)(2 + zov) * (L.n0 + 2) * (L.n1 + 2) : 0;
  return g;
}

// Maps a linear work index of one field to the (i, j, k) cell it writes.
template <int DIM>
__device__ __forceinline__ void ghost_target(const Layout& L, const FieldBC& bc, long long t, int& i, int& j, int& k) {
  const int xov = (bc.c == 'x' && bc.type[F_RIGHT] == FT_DIRICHLET);
  const int yov = (bc.c == 'y' && bc.type[F_TOP] == FT_DIRICHLET);
  const int zov = (DIM == 3 && bc.c == 'z' && bc.type[F_BACK] == FT_DIRICHLET);
  const long long nk = (DIM == 3) ? (L.n2 - zov) : 1;
  const GhostCount g = ghost_count<DIM>(L, bc);
  if (t < g.a) {  // x faces: j in [1, n1-yov], k in [1, nk]
    const int w = 2 + xov;
    const int s = (int)(t % w);
    long long r = t / w;
    j = 1 + (int)(r % (L.n1 - yov));
    k = 1 + (int)(r / (L.n1 - yov));
    i = (s == 0) ? 0 : (s == 1) ? L.n0 + 1 : L.n0;
    return;
  }
  t -= g.a;
  if (t < g.b) {  // y faces: i in [0, n0+1], k in [1, nk]
    const int ni = L.n0 + 2;
    i = (int)(t % ni);
    long long r = t / ni;
    const int w = 2 + yov;
    const int s = (int)(r % w);
    k = 1 + (int)(r / w);
    j = (s == 0) ? 0 : (s == 1) ? L.n1 + 1 : L.n1;
    return;
  }
  t -= g.b;  // z faces: i in [0, n0+1], j in [0, n1+1]
  const int ni = L.n0 + 2, nj = L.n1 + 2;
  i = (int)(t % ni);
  long long r = t / ni;
  j = (int)(r % nj);
  const int s = (int)(r / nj);
  k = (s == 0) ? 0 : (s == 1) ? L.n2 + 1 : L.n2;
  (void)nk;
}

// ghost_target with 32-bit multiply-high divisions (fft_magic multipliers set on the host):
// the 64-bit divisions by run-time divisors compile to conversion sequences, which GB300
// issues on its narrow FP64 pipe.  Valid when every quotient's numerator times its divisor
// stays below 2^32 (ghost_fast_ok); the cell is the same.
struct GhostDiv {
  int ok;
  unsigned a0, a1, b0, b1, c0, c1;  // x faces: 2 + xov, n1 - yov; y faces: n0 + 2, 2 + yov; z faces: n0 + 2, n1 + 2
};
__device__ __forceinline__ unsigned gdiv(unsigned x, unsigned d, unsigned m) { return d > 1 ? __umulhi(x, m) : x; }

template <int DIM>
__host__ inline GhostDiv ghost_div(const Layout& L, const FieldBC& bc) {
  const int xov = (bc.c == 'x' && bc.type[F_RIGHT] == FT_DIRICHLET);
  const int yov = (bc.c == 'y' && bc.type[F_TOP] == FT_DIRICHLET);
  const GhostCount g = ghost_count<DIM>(L, bc);
  GhostDiv d;
  const unsigned long long lim = 1ull << 32;
  const unsigned long long wa = 2 + xov, na = L.n1 - yov, ni = L.n0 + 2, wb = 2 + yov, nj = L.n1 + 2;
  // numerators: t < g.a (by wa), t / wa (by na); t < g.b (by ni), t / ni (by wb); t < g.c (by ni), t / ni (by nj)
  d.ok = ((unsigned long long)g.a * wa < lim) && ((unsigned long long)(g.a / wa + 1) * na < lim) &&
         ((unsigned long long)g.b * ni < lim) && ((unsigned long long)(g.b / ni + 1) * wb < lim) &&
         ((unsigned long long)g.c * ni < lim) && ((unsigned long long)(g.c / ni + 1) * nj < lim);
  d.a0 = fft_magic((unsigned)wa); d.a1 = fft_magic((unsigned)na);
  d.b0 = fft_magic((unsigned)ni); d.b1 = fft_magic((unsigned)wb);
  d.c0 = fft_magic((unsigned)ni); d.c1 = fft_magic((unsigned)nj);
  return d;
}

template <int DIM>
__device__ __forceinline__ void ghost_target_fast(const Layout& L, const FieldBC& bc, const GhostDiv& D, long long t64,
                                                  int& i, int& j, int& k) {
  const unsigned xov = (bc.c == 'x' && bc.type[F_RIGHT] == FT_DIRICHLET);
  const unsigned yov = (bc.c == 'y' && bc.type[F_TOP] == FT_DIRICHLET);
  const unsigned zov = (DIM == 3 && bc.c == 'z' && bc.type[F_BACK] == FT_DIRICHLET);
  const unsigned nk = (DIM == 3) ? (unsigned)L.n2 - zov : 1u;
  const unsigned wa = 2 + xov, na = (unsigned)L.n1 - yov, ni = (unsigned)L.n0 + 2, wb = 2 + yov, nj = (unsigned)L.n1 + 2;
  const unsigned ga = wa * na * nk, gb = wb * ni * nk;
  unsigned t = (unsigned)t64;
  if (t < ga) {
    const unsigned r = gdiv(t, wa, D.a0), s = t - r * wa;
    const unsigned q = gdiv(r, na, D.a1);
    j = 1 + (int)(r - q * na);
    k = 1 + (int)q;
    i = (s == 0) ? 0 : (s == 1) ? L.n0 + 1 : L.n0;
    return;
  }
  t -= ga;
  if (t < gb) {
    const unsigned r = gdiv(t, ni, D.b0);
    i = (int)(t - r * ni);
    const unsigned q = gdiv(r, wb, D.b1), s = r - q * wb;
    k = 1 + (int)q;
    j = (s == 0) ? 0 : (s == 1) ? L.n1 + 1 : L.n1;
    return;
  }
  t -= gb;
  const unsigned r = gdiv(t, ni, D.c0);
  i = (int)(t - r * ni);
  const unsigned q = gdiv(r, nj, D.c1);
  j = (int)(r - q * nj);
  k = (q == 0) ? 0 : (q == 1) ? L.n2 + 1 : L.n2;
}

// Up to four fields per launch (blockIdx.y selects the field).
template <typename T>
struct GhostBatch {
  T* f[4];
  FieldBC bc[4];
  long long n[4];
  double shift[4];
  GhostDiv gd[4];
  int low[4];  // 1: only the ghosts of v* the divergence reads (ghost_low_target)
};

// The ghosts of v* the divergence reads (its minus neighbours) and the faces a wall overwrites:
// the low face of a velocity component's own axis, interior extent -- u(0, j, k), v(i, 0, k),
// w(i, j, 0) -- and, where that axis' high face is Dirichlet, the overwritten last face
// u(n0, j, k), v(i, n1, k), w(i, j, n2) (the face-normal rule of Resolve).
__host__ __device__ inline long long ghost_low_count(const Layout& L, const FieldBC& bc) {
  const char c = bc.c;
  const long long face = c == 'x' ? (long long)L.n1 * L.n2 : c == 'y' ? (long long)L.n0 * L.n2 : (long long)L.n0 * L.n1;
  const int hi = c == 'x' ? F_RIGHT : c == 'y' ? F_TOP : F_BACK;
  return face * (bc.type[hi] == FT_DIRICHLET ? 2 : 1);
}
__device__ __forceinline__ void ghost_low_target(const Layout& L, const FieldBC& bc, long long t, int& i, int& j, int& k) {
  const char c = bc.c;
  const unsigned face = c == 'x' ? (unsigned)(L.n1 * L.n2) : c == 'y' ? (unsigned)(L.n0 * L.n2) : (unsigned)(L.n0 * L.n1);
  unsigned u = (unsigned)t;
  const bool high = u >= face;  // the overwritten last face
  if (high) u -= face;
  if (c == 'x') {
    i = high ? L.n0 : 0;
    j = 1 + (int)(u % (unsigned)L.n1);
    k = 1 + (int)(u / (unsigned)L.n1);
  } else if (c == 'y') {
    i = 1 + (int)(u % (unsigned)L.n0);
    j = high ? L.n1 : 0;
    k = 1 + (int)(u / (unsigned)L.n0);
  } else {
    i = 1 + (int)(u % (unsigned)L.n0);
    j = 1 + (int)(u / (unsigned)L.n0);
    k = high ? L.n2 : 0;
  }
}

template <typename T, int DIM>
__global__ void __launch_bounds__(256) k_ghost_fill(Layout L, GhostBatch<T> G) {
  const int q = blockIdx.y;
  const long long total = G.n[q];
  Resolve<T, DIM> R{PtrSrc<T>{G.f[q]}, L, G.bc[q], G.shift[q]};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    if (G.low[q]) ghost_low_target(L, G.bc[q], t, i, j, k);
    else if (G.gd[q].ok) ghost_target_fast<DIM>(L, G.bc[q], G.gd[q], t, i, j, k);
    else ghost_target<DIM>(L, G.bc[q], t, i, j, k);
    const T v = R.at(i, j, k);
    G.f[q][L.idx(i, j, kst<DIM>(k))] = v;
  }
}

}  // namespace fen
