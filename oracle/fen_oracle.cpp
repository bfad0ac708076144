// FEN projection-step oracle: a CPU FP64 restatement of the reference algorithm.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or calls this
// file.  It is used by tests/ (as the checker), by __graft_entry__.smoke() (as the
// checker) and by bench.py's CPU-baseline leg (timed as the "port" baseline).
//
// Every routine below restates one FEN routine in the same floating-point operation
// order (the Fortran is evaluated left to right; `x**2` is `x*x`; `float(n)` is a
// single-precision conversion).  Build with -ffp-contract=off so no FMA contraction
// happens on any host (x86 or Arm): the reference's default x86 build has none either.
//
// Parity status: the reference (Fortran + MPI + FFTW + 2decomp) cannot be built here,
// so this restatement is pinned against the reference's own known-answer tests
// (analytic manufactured solutions, projection bound, TGV decay, ghost exactness) and
// its transforms against numpy.fft / scipy.fft (FFTW's published definitions).
// Bit-level parity with the reference binary is therefore unpinned.
//
// Reference files (paths inside the FEN project):
//   src/grid.f90, src/scalar.f90, src/fields.f90, src/navier_stokes.f90, src/poisson.f90
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cplx;

// Physical boundary conditions of the grid (grid.f90:41-46: 'Periodic' | 'Wall' |
// 'Inflow' | 'Outflow').
enum { PB_PERIODIC = 0, PB_WALL = 1, PB_INFLOW = 2, PB_OUTFLOW = 3 };
// Field boundary-condition types (scalar.f90:17-22).
enum { FT_PERIODIC = 0, FT_DIRICHLET = 1, FT_NEUMANN = 2, FT_ERROR = 9 };
// Faces in the reference order: left, right, bottom, top, front, back.
enum { F_LEFT = 0, F_RIGHT, F_BOTTOM, F_TOP, F_FRONT, F_BACK };

static inline double ffloat(long n) { return (double)(float)n; }  // Fortran float(n)

// ------------------------------------------------------------------------------------
// FFT: mixed-radix recursive Cooley-Tukey (twiddles from cos/sin in FP64).  Implements
// FFTW's published definitions: forward = sum x e^{-2 pi i jk/n}, backward = e^{+...},
// both unnormalised (FFTW manual, "What FFTW Really Computes").
// ------------------------------------------------------------------------------------
struct FFTPlan {
  int n = 0;
  std::vector<int> factors;
  std::vector<cplx> w;  // w[m] = exp(-2 pi i m / n)
  explicit FFTPlan(int n_ = 1) : n(n_) {
    int m = n;
    for (int r : {4, 2, 3, 5}) {
      while (m % r == 0 && !(r == 4 && false)) { factors.push_back(r); m /= r; }
    }
    for (int r = 7; m > 1; r += 2) while (m % r == 0) { factors.push_back(r); m /= r; }
    w.resize(n);
    for (int k = 0; k < n; ++k) {
      double a = 2.0 * M_PI * (double)k / (double)n;
      w[k] = cplx(cos(a), -sin(a));
    }
  }
};

static void fft_rec(const cplx* in, cplx* out, int n, int stride, const FFTPlan& p, int fi,
                    int sign) {
  if (n == 1) { out[0] = in[0]; return; }
  const int r = p.factors[fi];
  const int m = n / r;
  for (int q = 0; q < r; ++q) fft_rec(in + (size_t)q * stride, out + (size_t)q * m, m, stride * r, p, fi + 1, sign);
  const int N = p.n;
  const int step = N / n;
  cplx t[16];
  std::vector<cplx> tb;
  cplx* tt = t;
  if (r > 16) { tb.resize(r); tt = tb.data(); }
  for (int k = 0; k < m; ++k) {
    for (int q = 0; q < r; ++q) {
      cplx v = out[(size_t)q * m + k];
      if (q && k) {
        cplx wq = p.w[((size_t)q * k * step) % N];
        if (sign > 0) wq = std::conj(wq);
        v = v * wq;
      }
      tt[q] = v;
    }
    for (int s = 0; s < r; ++s) {
      cplx acc = tt[0];
      for (int q = 1; q < r; ++q) {
        cplx wr = p.w[((size_t)((q * s) % r)) * (N / r)];
        if (sign > 0) wr = std::conj(wr);
        acc += tt[q] * wr;
      }
      out[k + (size_t)s * m] = acc;
    }
  }
}

static void fft(const FFTPlan& p, const cplx* in, cplx* out, int sign) {
  fft_rec(in, out, p.n, 1, p, 0, sign);
}

// r2c (FFTW dft_r2c_1d): out[k] = sum_j x_j e^{-2 pi i jk/n}, k = 0..n/2.
static void r2c(const FFTPlan& p, const double* x, cplx* out) {
  const int n = p.n;
  std::vector<cplx> a(n), b(n);
  for (int j = 0; j < n; ++j) a[j] = cplx(x[j], 0.0);
  fft(p, a.data(), b.data(), -1);
  for (int k = 0; k <= n / 2; ++k) out[k] = b[k];
}

// c2r (FFTW dft_c2r_1d): x_j = sum_{k=0}^{n-1} X_k e^{+2 pi i jk/n} with X Hermitian
// extended from k = 0..n/2; the imaginary parts of X_0 (and X_{n/2}, n even) are ignored.
static void c2r(const FFTPlan& p, const cplx* in, double* x) {
  const int n = p.n;
  std::vector<cplx> a(n), b(n);
  a[0] = cplx(in[0].real(), 0.0);
  for (int k = 1; k <= (n - 1) / 2; ++k) { a[k] = in[k]; a[n - k] = std::conj(in[k]); }
  if (n % 2 == 0) a[n / 2] = cplx(in[n / 2].real(), 0.0);
  fft(p, a.data(), b.data(), +1);
  for (int j = 0; j < n; ++j) x[j] = b[j].real();
}

// REDFT10 (DCT-II): Y_k = 2 sum_j x_j cos(pi (2j+1) k / 2n), via a 2n complex FFT of
// the even extension.  p2 is the plan of length 2n.
static void redft10(const FFTPlan& p2, const double* x, double* y) {
  const int n = p2.n / 2;
  std::vector<cplx> a(2 * n), b(2 * n);
  for (int j = 0; j < n; ++j) { a[j] = cplx(x[j], 0.0); a[2 * n - 1 - j] = cplx(x[j], 0.0); }
  fft(p2, a.data(), b.data(), -1);
  for (int k = 0; k < n; ++k) {
    double ang = M_PI * (double)k / (2.0 * n);
    y[k] = (b[k] * cplx(cos(ang), -sin(ang))).real();
  }
}

// REDFT01 (DCT-III): Y_k = x_0 + 2 sum_{j>=1} x_j cos(pi j (2k+1) / 2n).
static void redft01(const FFTPlan& p2, const double* x, double* y) {
  const int n = p2.n / 2;
  std::vector<cplx> a(2 * n, cplx(0.0, 0.0)), b(2 * n);
  for (int j = 0; j < n; ++j) {
    double ang = M_PI * (double)j / (2.0 * n);
    double c = (j == 0) ? 1.0 : 2.0;
    a[j] = c * x[j] * cplx(cos(ang), sin(ang));
  }
  fft(p2, a.data(), b.data(), +1);
  for (int k = 0; k < n; ++k) y[k] = b[k].real();
}

// ------------------------------------------------------------------------------------
// Fields: ghosted arrays f(0:n1+1, 0:n2+1, 0:n3+1) (gl = 1), x fastest, as in
// scalar.f90:79-84.  In 2D the z extent is 0:2 with k = 1 the only plane used.
// ------------------------------------------------------------------------------------
struct Field {
  char c = 'c';               // location: 'c' centre, 'x'/'y'/'z' face (vector.f90:57-62)
  int type[6] = {0, 0, 0, 0, 0, 0};
  std::vector<double> f;
  std::vector<double> bc[6];  // per-face Dirichlet values over the ghosted face extents
};

struct Oracle {
  int dim = 2;
  int n[3] = {1, 1, 1};
  double L[3] = {1, 1, 1};
  double x0[3] = {0, 0, 0};
  double d[3] = {1, 1, 1};  // grid spacing per axis (the reference has one delta)
  int iso = 1;              // all spacings identical: use the reference's single-delta forms
  int pbc[6] = {0, 0, 0, 0, 0, 0};
  int periodic[3] = {1, 1, 1};
  int ng[3];
  // navier_stokes_mod state (navier_stokes.f90:17-45)
  double density = 1.0, viscosity = 1.0, g[3] = {0, 0, 0};
  double maxdiv = 0, maxCFL = 0, CFL = 1.0, dt_visc = 0, dt_conv = 0, dt_o = 0;
  int constant_CFL = 0;
  Field u, v, w, p, phi;
  std::vector<double> dv[3], dvo[3], S[3];
  // variable-property path: cell-centred rho and mu (navier_stokes.f90:36, 761-775), the old
  // pressure p_o of the Dodd-Ferrante split (multiphase.f90:25, navier_stokes.f90:80-96)
  Field rho, mu, p_o;
  int var_mu = 0;          // constant_viscosity = .false. (navier_stokes.f90:45, 405-452)
  // IBM forcing lists per component (apply_ibm_forcing, navier_stokes.f90:106-108):
  // target vs = c0 + sum_q w_q v*(nbr_q), evaluated from the unforced v*, and Fe = (vs - v*)/dt
  struct Ibm {
    std::vector<size_t> idx, nidx;
    std::vector<int> nn;
    std::vector<double> w, c0, fe;
  } ibm[3];
  int split = 0;           // Dodd-Ferrante split pressure with rhomin (the MF branches)
  double rhomin = 1.0, irhomin = 1.0;
  // poisson_mod state (poisson.f90:31-49)
  int solver = -1;
  std::vector<double> mwn[3];
  std::vector<double> a, b, c;
  FFTPlan plan[3], plan2[3];
  int nthreads = 1;

  size_t nx() const { return (size_t)ng[0]; }
  size_t plane() const { return (size_t)ng[0] * ng[1]; }
  size_t total() const { return (size_t)ng[0] * ng[1] * ng[2]; }
  size_t I(int i, int j, int k) const { return (size_t)i + (size_t)ng[0] * ((size_t)j + (size_t)ng[1] * k); }
};

enum { S_PP = 0, S_PN, S_NN, S_PPP, S_PPN, S_NPN, S_NNN, S_PNP };

// Field bc-type mapping from the physical bc strings (navier_stokes.f90:780-1016).
// comp: 0 = p/phi, 1 = v%x, 2 = v%y, 3 = v%z.
static int field_type(int face, int pb, int comp) {
  if (pb == PB_PERIODIC) return FT_PERIODIC;
  if (pb == PB_WALL) return comp == 0 ? FT_NEUMANN : FT_DIRICHLET;
  if (pb == PB_INFLOW) {
    if (face == F_BACK) return FT_ERROR;  // navier_stokes.f90:990-1016 has no Inflow branch
    if (comp == 0) return FT_NEUMANN;
    if (face == F_LEFT || face == F_RIGHT) return comp == 1 ? FT_DIRICHLET : FT_NEUMANN;
    return FT_DIRICHLET;  // bottom/top/front: all components Dirichlet (:890-899, :977-984)
  }
  if (pb == PB_OUTFLOW) {
    if (face == F_FRONT) return FT_ERROR;  // :961-987 has no Outflow branch
    return comp == 0 ? FT_DIRICHLET : FT_NEUMANN;
  }
  return FT_ERROR;
}

static void alloc_field(Oracle& o, Field& F, char c, int comp) {
  F.c = c;
  F.f.assign(o.total(), 0.0);
  for (int f = 0; f < 6; ++f) {
    F.type[f] = (f < 2 * o.dim) ? field_type(f, o.pbc[f], comp) : FT_PERIODIC;
    size_t sz = (f < 2) ? (size_t)o.ng[1] * o.ng[2] : (f < 4) ? (size_t)o.ng[0] * o.ng[2] : (size_t)o.ng[0] * o.ng[1];
    F.bc[f].assign(sz, 0.0);
  }
}

// scalar%update_ghost_nodes (scalar.f90:223-396), single rank (prow = pcol = 1), gl = 1.
static void update_ghost_nodes(Oracle& o, Field& F) {
  const int N1 = o.n[0], N2 = o.n[1], N3 = o.n[2];
  const int g1 = o.ng[0], g2 = o.ng[1], g3 = o.ng[2];
  double* f = F.f.data();
  const char c = F.c;
  // Left / right faces over the full (j, k) ghosted range.
  for (int k = 0; k < g3; ++k)
    for (int j = 0; j < g2; ++j) {
      const double bl = F.bc[F_LEFT][j + (size_t)g2 * k], br = F.bc[F_RIGHT][j + (size_t)g2 * k];
      double* r = f + o.I(0, j, k);
      if (F.type[F_LEFT] == FT_PERIODIC) r[0] = r[N1];
      else if (F.type[F_LEFT] == FT_DIRICHLET) r[0] = (c == 'x') ? bl : 2.0 * bl - r[1];
      else if (F.type[F_LEFT] == FT_NEUMANN) r[0] = r[1];
      if (F.type[F_RIGHT] == FT_PERIODIC) r[N1 + 1] = r[1];
      else if (F.type[F_RIGHT] == FT_DIRICHLET) {
        if (c == 'x') { r[N1] = br; r[N1 + 1] = br; }
        else r[N1 + 1] = 2.0 * br - r[N1];
      } else if (F.type[F_RIGHT] == FT_NEUMANN) r[N1 + 1] = r[N1];
    }
  // Bottom / top faces over the full (i, k) ghosted range.
  for (int k = 0; k < g3; ++k)
    for (int i = 0; i < g1; ++i) {
      const double bb = F.bc[F_BOTTOM][i + (size_t)g1 * k], bt = F.bc[F_TOP][i + (size_t)g1 * k];
      double& lo = f[o.I(i, 0, k)];
      const double in1 = f[o.I(i, 1, k)];
      if (F.type[F_BOTTOM] == FT_PERIODIC) lo = f[o.I(i, N2, k)];
      else if (F.type[F_BOTTOM] == FT_DIRICHLET) lo = (c == 'y') ? bb : 2.0 * bb - in1;
      else if (F.type[F_BOTTOM] == FT_NEUMANN) lo = in1;
      double& hi = f[o.I(i, N2 + 1, k)];
      if (F.type[F_TOP] == FT_PERIODIC) hi = f[o.I(i, 1, k)];
      else if (F.type[F_TOP] == FT_DIRICHLET) {
        if (c == 'y') { f[o.I(i, N2, k)] = bt; hi = bt; }
        else hi = 2.0 * bt - f[o.I(i, N2, k)];
      } else if (F.type[F_TOP] == FT_NEUMANN) hi = f[o.I(i, N2, k)];
    }
  if (o.dim == 3) {
    for (int j = 0; j < g2; ++j)
      for (int i = 0; i < g1; ++i) {
        const double bf = F.bc[F_FRONT][i + (size_t)g1 * j], bk = F.bc[F_BACK][i + (size_t)g1 * j];
        double& lo = f[o.I(i, j, 0)];
        const double in1 = f[o.I(i, j, 1)];
        if (F.type[F_FRONT] == FT_PERIODIC) lo = f[o.I(i, j, N3)];
        else if (F.type[F_FRONT] == FT_DIRICHLET) lo = (c == 'z') ? bf : 2.0 * bf - in1;
        else if (F.type[F_FRONT] == FT_NEUMANN) lo = in1;
        double& hi = f[o.I(i, j, N3 + 1)];
        if (F.type[F_BACK] == FT_PERIODIC) hi = f[o.I(i, j, 1)];
        else if (F.type[F_BACK] == FT_DIRICHLET) {
          if (c == 'z') { f[o.I(i, j, N3)] = bk; hi = bk; }
          else hi = 2.0 * bk - f[o.I(i, j, N3)];
        } else if (F.type[F_BACK] == FT_NEUMANN) hi = f[o.I(i, j, N3)];
      }
  }
}

// ------------------------------------------------------------------------------------
// Operators (fields.f90, navier_stokes.f90).  `iso` selects the reference's single-delta
// evaluation order; anisotropic grids use one spacing per axis (a generalisation).
// ------------------------------------------------------------------------------------
#define OMP_FOR _Pragma("omp parallel for schedule(static) num_threads(o.nthreads)")

// add_advection (navier_stokes.f90:261-353), accumulating into R (no ghosts, same indexing).
static void add_advection(Oracle& o, std::vector<double>* R) {
  const double idx = 1.0 / o.d[0], idy = 1.0 / o.d[1], idz = 1.0 / o.d[2];
  const double* U = o.u.f.data(); const double* V = o.v.f.data(); const double* W = o.w.f.data();
  const size_t sx = 1, sy = o.ng[0], sz = o.plane();
  const int K = (o.dim == 3) ? o.n[2] : 1;
  OMP_FOR
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= o.n[1]; ++j)
      for (int i = 1; i <= o.n[0]; ++i) {
        const size_t c = o.I(i, j, k);
        const size_t ip = c + sx, im = c - sx, jp = c + sy, jm = c - sy;
        // u terms
        double uuip = 0.25 * ((U[ip] + U[c]) * (U[ip] + U[c]));
        double uuim = 0.25 * ((U[im] + U[c]) * (U[im] + U[c]));
        double uvjp = (U[jp] + U[c]) * (V[ip] + V[c]) * 0.25;
        double uvjm = (U[c] + U[jm]) * (V[ip - sy] + V[jm]) * 0.25;
        R[0][c] = R[0][c] - (uuip - uuim) * idx - (uvjp - uvjm) * idy;
        if (o.dim == 3) {
          const size_t kp = c + sz, km = c - sz;
          double uwkp = (U[kp] + U[c]) * (W[ip] + W[c]) * 0.25;
          double uwkm = (U[c] + U[km]) * (W[ip - sz] + W[km]) * 0.25;
          R[0][c] = R[0][c] - (uwkp - uwkm) * idz;
        }
        // v terms
        double vuip = (V[ip] + V[c]) * (U[jp] + U[c]) * 0.25;
        double vuim = (V[c] + V[im]) * (U[im + sy] + U[im]) * 0.25;
        double vvjp = 0.25 * ((V[jp] + V[c]) * (V[jp] + V[c]));
        double vvjm = 0.25 * ((V[jm] + V[c]) * (V[jm] + V[c]));
        R[1][c] = R[1][c] - (vuip - vuim) * idx - (vvjp - vvjm) * idy;
        if (o.dim == 3) {
          const size_t kp = c + sz, km = c - sz;
          double vwkp = (V[kp] + V[c]) * (W[jp] + W[c]) * 0.25;
          double vwkm = (V[c] + V[km]) * (W[jp - sz] + W[km]) * 0.25;
          R[1][c] = R[1][c] - (vwkp - vwkm) * idz;
          // w terms
          double wuip = (W[c] + W[ip]) * (U[c] + U[kp]) * 0.25;
          double wuim = (W[c] + W[im]) * (U[im] + U[im + sz]) * 0.25;
          double wvjp = (W[c] + W[jp]) * (V[c] + V[kp]) * 0.25;
          double wvjm = (W[c] + W[jm]) * (V[jm] + V[jm + sz]) * 0.25;
          double wwkp = (W[c] + W[kp]) * (W[c] + W[kp]) * 0.25;
          double wwkm = (W[c] + W[km]) * (W[c] + W[km]) * 0.25;
          R[2][c] = R[2][c] - (wuip - wuim) * idx - (wvjp - wvjm) * idy - (wwkp - wwkm) * idz;
        }
      }
}

// laplacian of one ghosted component at cell c (fields.f90:298-343).
static inline double lap_at(const Oracle& o, const double* F, size_t c) {
  const size_t sy = o.ng[0], sz = o.plane();
  const double two = 2.0 * F[c];
  if (o.iso) {
    const double id2 = 1.0 / (o.d[0] * o.d[0]);
    double l = ((F[c + 1] - two + F[c - 1]) + (F[c + sy] - two + F[c - sy])) * id2;
    if (o.dim == 3) l = l + (F[c + sz] - two + F[c - sz]) * id2;
    return l;
  }
  double l = (F[c + 1] - two + F[c - 1]) * (1.0 / (o.d[0] * o.d[0])) +
             (F[c + sy] - two + F[c - sy]) * (1.0 / (o.d[1] * o.d[1]));
  if (o.dim == 3) l = l + (F[c + sz] - two + F[c - sz]) * (1.0 / (o.d[2] * o.d[2]));
  return l;
}

// The z component of laplacian_of_vector sums the three directions before scaling
// (fields.f90:335-337), unlike x and y.
static inline double lap_w_at(const Oracle& o, const double* F, size_t c) {
  const size_t sy = o.ng[0], sz = o.plane();
  const double two = 2.0 * F[c];
  if (o.iso) {
    const double id2 = 1.0 / (o.d[0] * o.d[0]);
    return ((F[c + 1] - two + F[c - 1]) + (F[c + sy] - two + F[c - sy]) + (F[c + sz] - two + F[c - sz])) * id2;
  }
  return (F[c + 1] - two + F[c - 1]) * (1.0 / (o.d[0] * o.d[0])) +
         (F[c + sy] - two + F[c - sy]) * (1.0 / (o.d[1] * o.d[1])) +
         (F[c + sz] - two + F[c - sz]) * (1.0 / (o.d[2] * o.d[2]));
}

// compute_explicit_terms (navier_stokes.f90:217-257) with the constant-viscosity
// center_to_face(rho, rhof) (fields.f90:175-206) at the q-face of cell c.
static inline double rhof_at(const Oracle& o, size_t c, int q) {
  const size_t so[3] = {1, o.nx(), o.plane()};
  return 0.5 * (o.rho.f[c + so[q]] + o.rho.f[c]);
}

// compute_explicit_terms (navier_stokes.f90:217-257): advection, then add_diffusion
// (:357-452): mu%f(i,j,k)*lap(v)/rhof with constant viscosity, the stress divergence
// div(2 mu D)/rhof with variable viscosity (2D only: the reference's 3D branch is empty),
// then S/rhof.
static void compute_explicit_terms(Oracle& o, std::vector<double>* R) {
  for (int c = 0; c < o.dim; ++c) std::fill(R[c].begin(), R[c].end(), 0.0);
  add_advection(o, R);
  const int K = (o.dim == 3) ? o.n[2] : 1;
  const double* F[3] = {o.u.f.data(), o.v.f.data(), o.w.f.data()};
  const double* mu = o.mu.f.data();
  if (!o.var_mu) {
    OMP_FOR
    for (int k = 1; k <= K; ++k)
      for (int j = 1; j <= o.n[1]; ++j)
        for (int i = 1; i <= o.n[0]; ++i) {
          const size_t c = o.I(i, j, k);
          R[0][c] = R[0][c] + mu[c] * lap_at(o, F[0], c) / rhof_at(o, c, 0);
          R[1][c] = R[1][c] + mu[c] * lap_at(o, F[1], c) / rhof_at(o, c, 1);
          if (o.dim == 3) R[2][c] = R[2][c] + mu[c] * lap_w_at(o, F[2], c) / rhof_at(o, c, 2);
        }
  } else if (o.dim == 2) {
    const double idelta = 1.0 / o.d[0];
    const size_t sy = o.nx();
    const double* U = F[0];
    const double* V = F[1];
    OMP_FOR
    for (int k = 1; k <= K; ++k)
      for (int j = 1; j <= o.n[1]; ++j)
        for (int i = 1; i <= o.n[0]; ++i) {
          const size_t c = o.I(i, j, k);
          const size_t ip = c + 1, im = c - 1, jp = c + sy, jm = c - sy;
          const double tauxxip = 2.0 * mu[ip] * (U[ip] - U[c]) * idelta;
          const double tauxxim = 2.0 * mu[c] * (U[c] - U[im]) * idelta;
          const double dtauxxdx = (tauxxip - tauxxim) * idelta;
          const double tauxyjp = 0.25 * (mu[c] + mu[ip] + mu[jp] + mu[ip + sy]) *
                                 ((U[jp] - U[c]) * idelta + (V[ip] - V[c]) * idelta);
          const double tauxyjm = 0.25 * (mu[jm] + mu[ip - sy] + mu[c] + mu[ip]) *
                                 ((U[c] - U[jm]) * idelta + (V[ip - sy] - V[jm]) * idelta);
          const double dtauxydy = (tauxyjp - tauxyjm) * idelta;
          R[0][c] = R[0][c] + (dtauxxdx + dtauxydy) / rhof_at(o, c, 0);
          const double tauyxip = tauxyjp;
          const double tauyxim = 0.25 * (mu[im] + mu[c] + mu[im + sy] + mu[jp]) *
                                 ((U[im + sy] - U[im]) * idelta + (V[c] - V[im]) * idelta);
          const double dtauyxdx = (tauyxip - tauyxim) * idelta;
          const double tauyyjp = 2.0 * mu[jp] * (V[jp] - V[c]) * idelta;
          const double tauyyjm = 2.0 * mu[c] * (V[c] - V[jm]) * idelta;
          const double dtauyydy = (tauyyjp - tauyyjm) * idelta;
          R[1][c] = R[1][c] + (dtauyxdx + dtauyydy) / rhof_at(o, c, 1);
        }
  }
  OMP_FOR
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= o.n[1]; ++j)
      for (int i = 1; i <= o.n[0]; ++i) {
        const size_t c = o.I(i, j, k);
        for (int q = 0; q < o.dim; ++q) R[q][c] = R[q][c] + o.S[q][c] / rhof_at(o, c, q);
      }
}

// divergence_of_vector (fields.f90:120-153) at cell c.
static inline double div_at(const Oracle& o, size_t c) {
  const size_t sy = o.ng[0], sz = o.plane();
  const double* U = o.u.f.data(); const double* V = o.v.f.data(); const double* W = o.w.f.data();
  if (o.iso) {
    const double id = 1.0 / o.d[0];
    double dv = (U[c] - U[c - 1]) * id + (V[c] - V[c - sy]) * id;
    if (o.dim == 3) dv = dv + (W[c] - W[c - sz]) * id;
    return dv;
  }
  double dv = (U[c] - U[c - 1]) * (1.0 / o.d[0]) + (V[c] - V[c - sy]) * (1.0 / o.d[1]);
  if (o.dim == 3) dv = dv + (W[c] - W[c - sz]) * (1.0 / o.d[2]);
  return dv;
}

// ------------------------------------------------------------------------------------
// Poisson fast direct solvers (poisson.f90).
// ------------------------------------------------------------------------------------
static double mwn_periodic(int i1, int n, double delta) {  // poisson.f90:141
  return 2.0 * (cos(2.0 * M_PI * (i1 - 1.0) / ffloat(n)) - 1.0) / (delta * delta);
}
static double mwn_neumann(int i1, int n, double delta) {  // poisson.f90:265
  return 2.0 * (cos(1.0 * M_PI * (i1 - 1.0) / ffloat(n)) - 1.0) / (delta * delta);
}

// Tridiagonal coefficients (poisson.f90:216-232): along axis ax, physical faces fl/fh.
static void init_tridiag(Oracle& o, int ax) {
  const int n = o.n[ax];
  const double dl = o.d[ax];
  o.a.assign(n, 0); o.b.assign(n, 0); o.c.assign(n, 0);
  for (int j = 0; j < n; ++j) {
    o.a[j] = 1.0 / (dl * dl);
    o.b[j] = -2.0 / (dl * dl);
    o.c[j] = 1.0 / (dl * dl);
  }
  o.b[0] = o.b[0] + o.a[0];
  if (o.pbc[2 * ax] == PB_INFLOW && o.pbc[2 * ax + 1] == PB_OUTFLOW) o.b[n - 1] = o.b[n - 1] - o.c[n - 1];
  else o.b[n - 1] = o.b[n - 1] + o.c[n - 1];
  o.a[0] = 0.0;
  o.c[n - 1] = 0.0;
}

static int init_poisson(Oracle& o) {
  // Dispatch on periodicity (poisson.f90:57-113); (P,N,P) is a generalisation used for
  // wall-bounded channels (walls in y, x and z periodic).
  const int* P = o.periodic;
  if (o.dim == 3) {
    if (P[0] && P[1] && P[2]) o.solver = S_PPP;
    else if (P[0] && P[1] && !P[2]) o.solver = S_PPN;
    else if (!P[0] && P[1] && !P[2]) o.solver = S_NPN;
    else if (!P[0] && !P[1] && !P[2]) o.solver = S_NNN;
    else if (P[0] && !P[1] && P[2]) o.solver = S_PNP;
    else return -1;
  } else {
    if (P[0] && P[1]) o.solver = S_PP;
    else if (P[0] && !P[1]) o.solver = S_PN;
    else if (!P[0] && !P[1]) o.solver = S_NN;
    else return -1;
  }
  for (int ax = 0; ax < o.dim; ++ax) {
    o.mwn[ax].assign(o.n[ax], 0.0);
    o.plan[ax] = FFTPlan(o.n[ax]);
    o.plan2[ax] = FFTPlan(2 * o.n[ax]);
  }
  const int s = o.solver;
  auto setm = [&](int ax, bool neu) {
    for (int i = 1; i <= o.n[ax]; ++i)
      o.mwn[ax][i - 1] = neu ? mwn_neumann(i, o.n[ax], o.d[ax]) : mwn_periodic(i, o.n[ax], o.d[ax]);
  };
  switch (s) {
    case S_PP: setm(0, false); setm(1, false); break;
    case S_PN: setm(0, false); init_tridiag(o, 1); break;
    case S_NN: setm(0, true); init_tridiag(o, 1); break;
    case S_PPP: setm(0, false); setm(1, false); setm(2, false); break;
    case S_PPN: setm(0, false); setm(1, false); init_tridiag(o, 2); break;
    case S_NPN: setm(0, true); setm(1, false); init_tridiag(o, 2); break;
    case S_NNN: setm(0, true); setm(1, true); init_tridiag(o, 2); break;
    case S_PNP: setm(0, false); setm(2, false); init_tridiag(o, 1); break;
  }
  return 0;
}

// Line helpers over a 3D complex/real spectral array A(i, j, k), i fastest, sizes m0,m1,m2.
struct Spec {
  int m0, m1, m2;
  std::vector<cplx> c;
  std::vector<double> r;
  size_t I(int i, int j, int k) const { return (size_t)i + (size_t)m0 * ((size_t)j + (size_t)m1 * k); }
};

// Complex FFT of all lines along axis ax (1 or 2) of S.c, in place.
static void lines_c2c(Oracle& o, Spec& S, int ax, int sign) {
  const FFTPlan& p = o.plan[ax];
  const int n = p.n;
  const int outer = (ax == 1) ? S.m2 : S.m1;
  OMP_FOR
  for (int q = 0; q < outer; ++q) {
    std::vector<cplx> a(n), b(n);
    for (int i = 0; i < S.m0; ++i) {
      for (int t = 0; t < n; ++t) a[t] = S.c[ax == 1 ? S.I(i, t, q) : S.I(i, q, t)];
      fft(p, a.data(), b.data(), sign);
      for (int t = 0; t < n; ++t) S.c[ax == 1 ? S.I(i, t, q) : S.I(i, q, t)] = b[t];
    }
  }
}

// Tridiagonal solve along axis ax of S (complex or real), with eigenvalue sums lam(i,j).
// `ppn_form`: the 3D reference solvers use a reciprocal factor (poisson.f90:1094-1135);
// the 2D ones divide (poisson.f90:348-385), with two different association orders.
template <typename T>
static void thomas_lines(Oracle& o, std::vector<T>& X, const Spec& S, int ax,
                         const std::vector<double>& lamA, const std::vector<double>& lamB,
                         int axA, int axB, bool ppn_form) {
  const int n = o.n[ax];
  const double* a = o.a.data(); const double* b = o.b.data(); const double* c = o.c.data();
  const int ma = (axA == 0) ? S.m0 : (axA == 1) ? S.m1 : S.m2;
  const int mb = (axB < 0) ? 1 : (axB == 0) ? S.m0 : (axB == 1) ? S.m1 : S.m2;
  auto idx = [&](int ia, int ib, int t) -> size_t {
    int ijk[3] = {0, 0, 0};
    ijk[axA] = ia;
    if (axB >= 0) ijk[axB] = ib;
    ijk[ax] = t;
    return S.I(ijk[0], ijk[1], ijk[2]);
  };
  OMP_FOR
  for (int ib = 0; ib < mb; ++ib) {
    std::vector<double> c1(n);
    std::vector<T> d1(n);
    for (int ia = 0; ia < ma; ++ia) {
      const double mA = lamA[ia];
      const double mB = (axB >= 0) ? lamB[ib] : 0.0;
      if (ppn_form) {
        double factor = 1.0 / (b[0] + mA + mB);
        c1[0] = c[0] * factor;
        d1[0] = X[idx(ia, ib, 0)] * factor;
        for (int t = 1; t < n - 1; ++t) {
          factor = 1.0 / (b[t] + mA + mB - a[t] * c1[t - 1]);
          c1[t] = c[t] * factor;
          d1[t] = (X[idx(ia, ib, t)] - a[t] * d1[t - 1]) * factor;
        }
        factor = (b[n - 1] + mA + mB - a[n - 1] * c1[n - 2]);
        if (factor != 0.0) d1[n - 1] = (X[idx(ia, ib, n - 1)] - a[n - 1] * d1[n - 2]) / factor;
        else d1[n - 1] = T(0.0);
      } else {
        c1[0] = c[0] / (b[0] + mA);
        d1[0] = X[idx(ia, ib, 0)] / (b[0] + mA);
        for (int t = 1; t < n - 1; ++t) {
          c1[t] = c[t] / (b[t] - a[t] * c1[t - 1] + mA);
          d1[t] = (X[idx(ia, ib, t)] - a[t] * d1[t - 1]) / (b[t] + mA - a[t] * c1[t - 1]);
        }
        double frac = (b[n - 1] + mA - a[n - 1] * c1[n - 2]);
        if (frac != 0.0) d1[n - 1] = (X[idx(ia, ib, n - 1)] - a[n - 1] * d1[n - 2]) / frac;
        else d1[n - 1] = T(0.0);
      }
      X[idx(ia, ib, n - 1)] = d1[n - 1];
      for (int t = n - 2; t >= 0; --t) X[idx(ia, ib, t)] = d1[t] - c1[t] * X[idx(ia, ib, t + 1)];
    }
  }
}

// Complex division by a real as gfortran lowers it: component-wise.
static inline cplx cdivr(cplx z, double r) { return cplx(z.real() / r, z.imag() / r); }
static inline cplx cmulr(cplx z, double r) { return cplx(z.real() * r, z.imag() * r); }

static double interior_sum(const Oracle& o, const double* f) {
  double s = 0.0;
  const int K = (o.dim == 3) ? o.n[2] : 1;
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= o.n[1]; ++j)
      for (int i = 1; i <= o.n[0]; ++i) s = s + f[o.I(i, j, k)];
  return s;
}

// solve_poisson on the interior of phi (poisson.f90:306-1451).
static void solve_poisson(Oracle& o, Field& PHI) {
  const int nx = o.n[0], ny = o.n[1], nz = (o.dim == 3) ? o.n[2] : 1;
  const int K = nz;
  double* phi = PHI.f.data();
  const int s = o.solver;
  const int h = nx / 2 + 1;
  if (s == S_PP || s == S_PPP || s == S_PN || s == S_PPN || s == S_PNP) {
    Spec S{h, ny, nz, {}, {}};
    S.c.assign((size_t)h * ny * nz, cplx(0, 0));
    // x: r2c per line (poisson.f90:441-445)
    OMP_FOR
    for (int k = 1; k <= K; ++k) {
      std::vector<double> line(nx);
      std::vector<cplx> out(h);
      for (int j = 1; j <= ny; ++j) {
        for (int i = 0; i < nx; ++i) line[i] = phi[o.I(i + 1, j, k)];
        r2c(o.plan[0], line.data(), out.data());
        for (int i = 0; i < h; ++i) S.c[S.I(i, j - 1, k - 1)] = out[i];
      }
    }
    if (s == S_PN || s == S_PPN || s == S_PNP)
      for (auto& z : S.c) z = cdivr(z, ffloat(nx));  // :341, :1074
    if (s == S_PP) {
      lines_c2c(o, S, 1, -1);
      for (auto& z : S.c) z = cdivr(z, ffloat((long)nx * ny));  // :458
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < h; ++i) {
          const double lam = o.mwn[0][i] + o.mwn[1][j];
          cplx& z = S.c[S.I(i, j, 0)];
          z = (lam == 0.0) ? cplx(0, 0) : cdivr(z, lam);
        }
      lines_c2c(o, S, 1, +1);
    } else if (s == S_PPP) {
      lines_c2c(o, S, 1, -1);
      lines_c2c(o, S, 2, -1);
      for (auto& z : S.c) z = cdivr(z, ffloat((long)nx * ny * nz));  // :992
      for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < h; ++i) {
            const double lam = o.mwn[0][i] + o.mwn[1][j] + o.mwn[2][k];
            cplx& z = S.c[S.I(i, j, k)];
            z = (lam == 0.0) ? cplx(0, 0) : cdivr(z, lam);
          }
      lines_c2c(o, S, 2, +1);
      lines_c2c(o, S, 1, +1);
    } else if (s == S_PN) {
      thomas_lines(o, S.c, S, 1, o.mwn[0], o.mwn[0], 0, -1, false);
    } else if (s == S_PPN) {
      lines_c2c(o, S, 1, -1);
      for (auto& z : S.c) z = cdivr(z, ffloat(ny));  // :1087
      thomas_lines(o, S.c, S, 2, o.mwn[0], o.mwn[1], 0, 1, true);
      lines_c2c(o, S, 1, +1);
    } else {  // S_PNP: FFT in z (normalised by nz), Thomas in y
      lines_c2c(o, S, 2, -1);
      for (auto& z : S.c) z = cdivr(z, ffloat(nz));
      thomas_lines(o, S.c, S, 1, o.mwn[0], o.mwn[2], 0, 2, true);
      lines_c2c(o, S, 2, +1);
    }
    if (s == S_PPN || s == S_PNP) std::fill(PHI.f.begin(), PHI.f.end(), 0.0);  // :1151
    // x: c2r per line (:484-488)
    OMP_FOR
    for (int k = 1; k <= K; ++k) {
      std::vector<double> line(nx);
      std::vector<cplx> in(h);
      for (int j = 1; j <= ny; ++j) {
        for (int i = 0; i < h; ++i) in[i] = S.c[S.I(i, j - 1, k - 1)];
        c2r(o.plan[0], in.data(), line.data());
        for (int i = 0; i < nx; ++i) phi[o.I(i + 1, j, k)] = line[i];
      }
    }
    if (s == S_PP || s == S_PN || s == S_PPN || s == S_PNP) {
      const double mean = interior_sum(o, phi);
      const double m = mean / ffloat((long)nx * ny * nz);
      if (s == S_PN) {  // interior only (:409-410)
        for (int k = 1; k <= K; ++k)
          for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) phi[o.I(i, j, k)] = phi[o.I(i, j, k)] - m;
      } else {
        for (auto& x : PHI.f) x = x - m;  // whole array (:503, :1171)
      }
    }
    return;
  }
  // DCT-based solvers: nn (2D), npn, nnn (3D).
  if (s == S_NN) {
    Spec S{nx, ny, 1, {}, {}};
    S.r.assign((size_t)nx * ny, 0.0);
    for (int j = 1; j <= ny; ++j) {
      std::vector<double> line(nx), out(nx);
      for (int i = 0; i < nx; ++i) line[i] = phi[o.I(i + 1, j, 1)];
      redft10(o.plan2[0], line.data(), out.data());
      for (int i = 0; i < nx; ++i) S.r[S.I(i, j - 1, 0)] = out[i];
    }
    thomas_lines(o, S.r, S, 1, o.mwn[0], o.mwn[0], 0, -1, false);
    for (int j = 1; j <= ny; ++j) {
      std::vector<double> line(nx), out(nx);
      for (int i = 0; i < nx; ++i) line[i] = S.r[S.I(i, j - 1, 0)];
      redft01(o.plan2[0], line.data(), out.data());
      for (int i = 0; i < nx; ++i) phi[o.I(i + 1, j, 1)] = out[i];
    }
    for (auto& x : PHI.f) x = x / ffloat((long)nx * 2);  // :594
    return;
  }
  // npn / nnn
  Spec R{nx, ny, nz, {}, {}};
  R.r.assign((size_t)nx * ny * nz, 0.0);
  OMP_FOR
  for (int k = 1; k <= nz; ++k) {
    std::vector<double> line(nx), out(nx);
    for (int j = 1; j <= ny; ++j) {
      for (int i = 0; i < nx; ++i) line[i] = phi[o.I(i + 1, j, k)];
      redft10(o.plan2[0], line.data(), out.data());
      for (int i = 0; i < nx; ++i) R.r[R.I(i, j - 1, k - 1)] = out[i] / (double)(nx * 2);  // :1213
    }
  }
  if (s == S_NPN) {
    const int hy = ny / 2 + 1;
    Spec C{nx, hy, nz, {}, {}};
    C.c.assign((size_t)nx * hy * nz, cplx(0, 0));
    OMP_FOR
    for (int k = 0; k < nz; ++k) {
      std::vector<double> line(ny);
      std::vector<cplx> out(hy);
      for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < ny; ++j) line[j] = R.r[R.I(i, j, k)];
        r2c(o.plan[1], line.data(), out.data());
        for (int j = 0; j < hy; ++j) C.c[C.I(i, j, k)] = cdivr(out[j], (double)ny);  // :1226
      }
    }
    thomas_lines(o, C.c, C, 2, o.mwn[0], o.mwn[1], 0, 1, true);
    OMP_FOR
    for (int k = 0; k < nz; ++k) {
      std::vector<double> line(ny);
      std::vector<cplx> in(hy);
      for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < hy; ++j) in[j] = C.c[C.I(i, j, k)];
        c2r(o.plan[1], in.data(), line.data());
        for (int j = 0; j < ny; ++j) R.r[R.I(i, j, k)] = line[j];
      }
    }
  } else {  // nnn
    OMP_FOR
    for (int k = 0; k < nz; ++k) {
      std::vector<double> line(ny), out(ny);
      for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < ny; ++j) line[j] = R.r[R.I(i, j, k)];
        redft10(o.plan2[1], line.data(), out.data());
        for (int j = 0; j < ny; ++j) R.r[R.I(i, j, k)] = out[j] / (double)(ny * 2);  // :1365
      }
    }
    thomas_lines(o, R.r, R, 2, o.mwn[0], o.mwn[1], 0, 1, true);
    OMP_FOR
    for (int k = 0; k < nz; ++k) {
      std::vector<double> line(ny), out(ny);
      for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < ny; ++j) line[j] = R.r[R.I(i, j, k)];
        redft01(o.plan2[1], line.data(), out.data());
        for (int j = 0; j < ny; ++j) R.r[R.I(i, j, k)] = out[j];
      }
    }
  }
  std::fill(PHI.f.begin(), PHI.f.end(), 0.0);  // :1290, :1429
  OMP_FOR
  for (int k = 1; k <= nz; ++k) {
    std::vector<double> line(nx), out(nx);
    for (int j = 1; j <= ny; ++j) {
      for (int i = 0; i < nx; ++i) line[i] = R.r[R.I(i, j - 1, k - 1)];
      redft01(o.plan2[0], line.data(), out.data());
      for (int i = 0; i < nx; ++i) phi[o.I(i + 1, j, k)] = out[i];
    }
  }
  // npn / nnn compute the mean but do not subtract it (:1297-1310, :1436-1449).
}

// ------------------------------------------------------------------------------------
// Time stepping (navier_stokes.f90:50-213, 505-730).
// ------------------------------------------------------------------------------------
static double dmin(const Oracle& o) {
  double m = o.d[0];
  for (int a = 1; a < o.dim; ++a) m = std::min(m, o.d[a]);
  return m;
}

static double max_vel(const Oracle& o) {
  double mv = 0.0;
  const int K = (o.dim == 3) ? o.n[2] : 1;
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= o.n[1]; ++j)
      for (int i = 1; i <= o.n[0]; ++i) {
        const size_t c = o.I(i, j, k);
        double vel = std::fabs(o.u.f[c]) + std::fabs(o.v.f[c]);
        if (o.dim == 3) vel = vel + std::fabs(o.w.f[c]);
        if (vel > mv) mv = vel;
      }
  return mv;
}

// set_timestep (navier_stokes.f90:623-666)
static double set_timestep(Oracle& o, double U) {
  const double dl = dmin(o);
  o.dt_conv = o.CFL * dl / U;
  o.dt_visc = 0.125 * dl * dl * o.density / o.viscosity;
  if (o.dim == 3) o.dt_visc = (1.0 / 6.0) * dl * dl * o.density / o.viscosity;
  double dt = std::min(o.dt_conv, o.dt_visc);
  o.dt_o = dt;
  return dt;
}

// update_timestep (navier_stokes.f90:670-730)
static void update_timestep(Oracle& o, double* dt) {
  o.dt_o = *dt;
  const double mv = max_vel(o);
  if (mv > 0.0) o.dt_conv = o.CFL * dmin(o) / mv;
  else o.dt_conv = 1.0;
  *dt = std::min(o.dt_conv, o.dt_visc);
  if (*dt > 1.1 * o.dt_o) *dt = 1.1 * o.dt_o;
}

static void step(Oracle& o, double* dtp) {
  if (o.constant_CFL) update_timestep(o, dtp);
  const double dt = *dtp;
  const int K = (o.dim == 3) ? o.n[2] : 1;
  const double idx = 1.0 / o.d[0], idy = 1.0 / o.d[1], idz = 1.0 / o.d[2];
  // Dodd-Ferrante approximate pressure (:87-95), whole array then ghosts
  std::vector<double> p_hat;
  if (o.split) {
    p_hat.resize(o.p.f.size());
    for (size_t t = 0; t < p_hat.size(); ++t) {
      if (o.constant_CFL) p_hat[t] = o.p_o.f[t] + (dt + o.dt_o) * (o.p.f[t] - o.p_o.f[t]) / o.dt_o;
      else p_hat[t] = 2.0 * o.p.f[t] - o.p_o.f[t];
    }
    Field ph = o.p;
    ph.f = p_hat;
    update_ghost_nodes(o, ph);
    p_hat = ph.f;
  }
  // predicted_velocity_field (:140-213)
  const double A = 1.0 + 0.5 * dt / o.dt_o;
  const double B = -0.5 * dt / o.dt_o;
  compute_explicit_terms(o, o.dv);
  Field* Vc[3] = {&o.u, &o.v, &o.w};
  const double* P = o.p.f.data();
  const size_t so[3] = {1, o.nx(), o.plane()};
  const double id[3] = {idx, idy, idz};
  OMP_FOR
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= o.n[1]; ++j)
      for (int i = 1; i <= o.n[0]; ++i) {
        const size_t c = o.I(i, j, k);
        for (int q = 0; q < o.dim; ++q) {
          const double rhof = rhof_at(o, c, q);
          const double gp = (P[c + so[q]] - P[c]) * (o.iso ? idx : id[q]);  // gradient (fields.f90:55-58)
          double rhs = -gp / rhof + A * o.dv[q][c] + B * o.dvo[q][c] + o.g[q];
          if (o.split) {
            const double gph = (p_hat[c + so[q]] - p_hat[c]) * (o.iso ? idx : id[q]);
            rhs = rhs + gp / rhof - o.irhomin * gp - (1.0 / rhof - o.irhomin) * gph;
          }
          Vc[q]->f[c] = Vc[q]->f[c] + dt * rhs;
        }
      }
  for (int q = 0; q < o.dim; ++q) o.dvo[q] = o.dv[q];
  for (int q = 0; q < o.dim; ++q) update_ghost_nodes(o, *Vc[q]);
  // apply_ibm_forcing (:106-108): targets from the unforced v*, then the forcing, then bcs
  bool forced = false;
  for (int q = 0; q < o.dim; ++q) {
    Oracle::Ibm& I = o.ibm[q];
    const size_t np = I.idx.size();
    if (!np) continue;
    forced = true;
    std::vector<double> vs(np);
    for (size_t p = 0; p < np; ++p) {
      double s = I.c0[p];
      for (int k = 0; k < I.nn[p]; ++k) s = s + I.w[8 * p + k] * Vc[q]->f[I.nidx[8 * p + k]];
      vs[p] = s;
    }
    I.fe.assign(np, 0.0);
    for (size_t p = 0; p < np; ++p) {
      I.fe[p] = (vs[p] - Vc[q]->f[I.idx[p]]) / dt;
      Vc[q]->f[I.idx[p]] = vs[p];
    }
  }
  if (forced)
    for (int q = 0; q < o.dim; ++q) update_ghost_nodes(o, *Vc[q]);
  // phi = div(v) * rho / dt (:111-122); rhomin/dt with the split
  double* phi = o.phi.f.data();
  OMP_FOR
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= o.n[1]; ++j)
      for (int i = 1; i <= o.n[0]; ++i) {
        const size_t c = o.I(i, j, k);
        phi[c] = div_at(o, c);
        phi[c] = o.split ? phi[c] * o.rhomin / dt : phi[c] * o.rho.f[c] / dt;
      }
  solve_poisson(o, o.phi);
  update_ghost_nodes(o, o.phi);
  // correct_velocity_field (:505-546)
  OMP_FOR
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= o.n[1]; ++j)
      for (int i = 1; i <= o.n[0]; ++i) {
        const size_t c = o.I(i, j, k);
        for (int q = 0; q < o.dim; ++q) {
          const double gphi = (phi[c + so[q]] - phi[c]) * (o.iso ? idx : id[q]);
          if (o.split) Vc[q]->f[c] = Vc[q]->f[c] - gphi * dt * o.irhomin;
          else Vc[q]->f[c] = Vc[q]->f[c] - gphi * dt / rhof_at(o, c, q);
        }
      }
  for (int q = 0; q < o.dim; ++q) update_ghost_nodes(o, *Vc[q]);
  // update_pressure (:550-566): p_o = p with the split; whole array, then ghosts
  if (o.split) o.p_o.f = o.p.f;
  for (size_t t = 0; t < o.p.f.size(); ++t) o.p.f[t] = o.p.f[t] + o.phi.f[t];
  update_ghost_nodes(o, o.p);
  // checks (:570-619)
  double md = -HUGE_VAL;
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= o.n[1]; ++j)
      for (int i = 1; i <= o.n[0]; ++i) {
        const double dv = div_at(o, o.I(i, j, k));
        if (dv > md) md = dv;
      }
  o.maxdiv = md;
  o.maxCFL = dt * max_vel(o) / dmin(o);
}

// ------------------------------------------------------------------------------------
// C API (ctypes).  Field ids: 0 u, 1 v, 2 w, 3 p, 4 phi, 5..7 dv_o, 8..10 S, 11..13 dv.
// ------------------------------------------------------------------------------------
extern "C" {

struct or_params {
  int dim, nx, ny, nz;
  double lx, ly, lz;
  double x0[3];
  int bc[6];
  double density, viscosity, g[3], cfl;
  int constant_cfl;
  int aniso;     // 0: delta = Lx/Nx on every axis (reference); 1: one spacing per axis
  int nthreads;
};

void* or_create(const or_params* P) {
  Oracle* o = new Oracle();
  o->dim = P->dim;
  o->n[0] = P->nx; o->n[1] = P->ny; o->n[2] = (P->dim == 3) ? P->nz : 1;
  o->L[0] = P->lx; o->L[1] = P->ly; o->L[2] = P->lz;
  for (int a = 0; a < 3; ++a) o->x0[a] = P->x0[a];
  // grid%setup (grid.f90:140): a single delta = Lx/float(Nx)
  const double delta = P->lx / ffloat(P->nx);
  if (P->aniso) {
    o->d[0] = P->lx / ffloat(P->nx);
    o->d[1] = P->ly / ffloat(P->ny);
    o->d[2] = (P->dim == 3) ? P->lz / ffloat(P->nz) : delta;
    o->iso = (o->d[0] == o->d[1]) && (P->dim == 2 || o->d[0] == o->d[2]);
  } else {
    o->d[0] = o->d[1] = o->d[2] = delta;
    o->iso = 1;
  }
  for (int f = 0; f < 6; ++f) o->pbc[f] = (f < 2 * P->dim) ? P->bc[f] : PB_PERIODIC;
  for (int a = 0; a < 3; ++a) o->periodic[a] = (o->pbc[2 * a] == PB_PERIODIC && o->pbc[2 * a + 1] == PB_PERIODIC);
  o->ng[0] = o->n[0] + 2; o->ng[1] = o->n[1] + 2; o->ng[2] = o->n[2] + 2;
  o->density = P->density; o->viscosity = P->viscosity;
  for (int a = 0; a < 3; ++a) o->g[a] = P->g[a];
  o->CFL = P->cfl; o->constant_CFL = P->constant_cfl;
  o->nthreads = P->nthreads > 0 ? P->nthreads : 1;
  alloc_field(*o, o->u, 'x', 1);
  alloc_field(*o, o->v, 'y', 2);
  alloc_field(*o, o->w, 'z', 3);
  alloc_field(*o, o->p, 'c', 0);
  alloc_field(*o, o->phi, 'c', 0);
  alloc_field(*o, o->rho, 'c', 0);  // rho, mu, p_o take p's boundary types (navier_stokes.f90:780-1016)
  alloc_field(*o, o->mu, 'c', 0);
  alloc_field(*o, o->p_o, 'c', 0);
  std::fill(o->rho.f.begin(), o->rho.f.end(), P->density);   // rho%f = density
  std::fill(o->mu.f.begin(), o->mu.f.end(), P->viscosity);   // mu%f = viscosity
  for (int q = 0; q < 3; ++q) {
    o->dv[q].assign(o->total(), 0.0);
    o->dvo[q].assign(o->total(), 0.0);
    o->S[q].assign(o->total(), 0.0);
  }
  if (init_poisson(*o) != 0) { delete o; return nullptr; }
  return o;
}

void or_destroy(void* h) { delete (Oracle*)h; }

double* or_field(void* h, int id) {
  Oracle* o = (Oracle*)h;
  switch (id) {
    case 0: return o->u.f.data();
    case 1: return o->v.f.data();
    case 2: return o->w.f.data();
    case 3: return o->p.f.data();
    case 4: return o->phi.f.data();
    case 5: case 6: case 7: return o->dvo[id - 5].data();
    case 8: case 9: case 10: return o->S[id - 8].data();
    case 11: case 12: case 13: return o->dv[id - 11].data();
    case 14: return o->rho.f.data();
    case 15: return o->mu.f.data();
    case 16: return o->p_o.f.data();
  }
  return nullptr;
}

void or_set_ibm(void* h, int comp, int np, const int* ijk, const int* nnbr, const int* nbr_ijk, const double* w,
                const double* c0) {
  Oracle* o = (Oracle*)h;
  Oracle::Ibm& I = o->ibm[comp];
  I = Oracle::Ibm();
  for (int p = 0; p < np; ++p) {
    const int k = (o->dim == 3) ? ijk[3 * p + 2] : 1;
    I.idx.push_back(o->I(ijk[3 * p], ijk[3 * p + 1], k));
    I.nn.push_back(nnbr[p]);
    I.c0.push_back(c0[p]);
    for (int q = 0; q < 8; ++q) {
      if (q < nnbr[p]) {
        const int* n3 = nbr_ijk + 3 * (8 * p + q);
        I.nidx.push_back(o->I(n3[0], n3[1], (o->dim == 3) ? n3[2] : 1));
        I.w.push_back(w[8 * p + q]);
      } else {
        I.nidx.push_back(0);
        I.w.push_back(0.0);
      }
    }
  }
}

const double* or_ibm_force(void* h, int comp) {
  Oracle* o = (Oracle*)h;
  return o->ibm[comp].fe.empty() ? nullptr : o->ibm[comp].fe.data();
}

// constant_viscosity = .not. var_mu; split: the MF pressure split with rhomin (solver.f90:91-92)
void or_set_properties(void* h, int var_mu, int split, double rhomin) {
  Oracle* o = (Oracle*)h;
  o->var_mu = var_mu;
  o->split = split;
  o->rhomin = rhomin;
  o->irhomin = 1.0 / rhomin;
}

static Field* fld(Oracle* o, int id) {
  switch (id) {
    case 0: return &o->u; case 1: return &o->v; case 2: return &o->w; case 3: return &o->p; case 4: return &o->phi;
    case 14: return &o->rho; case 15: return &o->mu; case 16: return &o->p_o;
  }
  return nullptr;
}

double* or_bc(void* h, int id, int face) { Field* F = fld((Oracle*)h, id); return F ? F->bc[face].data() : nullptr; }
int or_bc_type(void* h, int id, int face) { Field* F = fld((Oracle*)h, id); return F ? F->type[face] : -1; }
void or_set_bc_type(void* h, int id, int face, int t) { Field* F = fld((Oracle*)h, id); if (F) F->type[face] = t; }
void or_update_ghost_nodes(void* h, int id) { Oracle* o = (Oracle*)h; Field* F = fld(o, id); if (F) update_ghost_nodes(*o, *F); }
void or_solve_poisson(void* h) { Oracle* o = (Oracle*)h; solve_poisson(*o, o->phi); }
int or_solver_kind(void* h) { return ((Oracle*)h)->solver; }
void or_compute_explicit_terms(void* h) { Oracle* o = (Oracle*)h; compute_explicit_terms(*o, o->dv); }
void or_add_advection(void* h) {
  Oracle* o = (Oracle*)h;
  for (int c = 0; c < 3; ++c) std::fill(o->dv[c].begin(), o->dv[c].end(), 0.0);
  add_advection(*o, o->dv);
}
double or_set_timestep(void* h, double U) { return set_timestep(*(Oracle*)h, U); }
void or_set_dt_o(void* h, double dto) { ((Oracle*)h)->dt_o = dto; }
double or_get_dt_o(void* h) { return ((Oracle*)h)->dt_o; }
void or_step(void* h, double* dt) { step(*(Oracle*)h, dt); }
void or_run(void* h, int nsteps, double* dt) { for (int s = 0; s < nsteps; ++s) step(*(Oracle*)h, dt); }
void or_diag(void* h, double* out) {
  Oracle* o = (Oracle*)h;
  out[0] = o->maxdiv; out[1] = o->maxCFL; out[2] = o->dt_o; out[3] = o->dt_visc;
}
void or_delta(void* h, double* out) { Oracle* o = (Oracle*)h; out[0] = o->d[0]; out[1] = o->d[1]; out[2] = o->d[2]; }
void or_divergence(void* h, double* out) {  // interior divergence, x fastest, no ghosts
  Oracle* o = (Oracle*)h;
  const int K = (o->dim == 3) ? o->n[2] : 1;
  size_t t = 0;
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= o->n[1]; ++j)
      for (int i = 1; i <= o->n[0]; ++i) out[t++] = div_at(*o, o->I(i, j, k));
}

// Transform kernels exposed for pinning against numpy.fft / scipy.fft.
void or_fft(int n, const double* in_ri, double* out_ri, int sign) {
  FFTPlan p(n);
  std::vector<cplx> a(n), b(n);
  for (int j = 0; j < n; ++j) a[j] = cplx(in_ri[2 * j], in_ri[2 * j + 1]);
  fft(p, a.data(), b.data(), sign);
  for (int j = 0; j < n; ++j) { out_ri[2 * j] = b[j].real(); out_ri[2 * j + 1] = b[j].imag(); }
}
void or_r2c(int n, const double* x, double* out_ri) {
  FFTPlan p(n);
  std::vector<cplx> o(n / 2 + 1);
  r2c(p, x, o.data());
  for (int k = 0; k <= n / 2; ++k) { out_ri[2 * k] = o[k].real(); out_ri[2 * k + 1] = o[k].imag(); }
}
void or_c2r(int n, const double* in_ri, double* x) {
  FFTPlan p(n);
  std::vector<cplx> i(n / 2 + 1);
  for (int k = 0; k <= n / 2; ++k) i[k] = cplx(in_ri[2 * k], in_ri[2 * k + 1]);
  c2r(p, i.data(), x);
}
void or_redft10(int n, const double* x, double* y) { FFTPlan p(2 * n); redft10(p, x, y); }
void or_redft01(int n, const double* x, double* y) { FFTPlan p(2 * n); redft01(p, x, y); }

}  // extern "C"
