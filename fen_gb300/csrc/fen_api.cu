// Host runtime and C ABI of the GB300 projection step (see include/fen_gpu.h).
//
// One fen_ctx holds what FEN keeps in module state: the grid (src/grid.f90), the
// navier_stokes_mod fields (src/navier_stokes.f90:17-45) and the poisson_mod plan
// (src/poisson.f90:31-49), all resident in HBM, plus one CUDA stream and a captured graph
// of one time step.  The step is the sequence of navier_stokes_solver
// (navier_stokes.f90:50-136) as kernels; see fen_kernels.cuh.
//
// Two arithmetic forms share the plan:
//   FP64  : every field and transform in FP64 (the reference's arithmetic);
//   MIXED : state u, v, w, p as double-float pairs (fen_mixed.cuh); predictor, divergence,
//           transforms, correction in FP32 instructions; tridiagonal solves, mean removal
//           and the diagnostics reductions in FP64.  The FP64 arrays u, v, w, p then only
//           stage host transfers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fen_gpu.h"
#include "fen_adjoint.cuh"
#include "fen_fields.cuh"
#include "fen_kernels.cuh"
#include "fen_varprop.cuh"
#include "fen_types.cuh"

using namespace fen;

// Build knobs (on by default): the mixed form's two-instruction tridiagonal sweep, the mean of
// phi removed in the correction, the half-spectrum pitch padded to 64 bytes.
#ifndef FEN_CHECK_CTAS_PER_SM
#define FEN_CHECK_CTAS_PER_SM 16  // 256-thread CTAs per SM of the diagnostics pass (k_checks*; 4: FP64 256^3 0.357 -> 0.337 ms)
#endif
#ifndef FEN_VSTAR_LOW
#define FEN_VSTAR_LOW 1  // 1: the ghost fill of v* covers only the faces the divergence reads
#endif
#ifndef FEN_THOMAS_DF
#define FEN_THOMAS_DF 1  // mixed form, 3D solvers: the double-float sweep (k_thomas_df)
#endif
#ifndef FEN_THOMAS_FAST
#define FEN_THOMAS_FAST 1
#endif
#ifndef FEN_DEFER_MEAN
#define FEN_DEFER_MEAN 1
#endif
#ifndef FEN_SPEC_PAD
#define FEN_SPEC_PAD 1
#endif

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(FEN_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

enum { S_PP = 0, S_PN, S_NN, S_PPP, S_PPN, S_NPN, S_NNN, S_PNP };

// Field bc-type mapping from the physical bc strings (navier_stokes.f90:780-1016).
// comp: 0 = p/phi, 1 = v%x, 2 = v%y, 3 = v%z.  Returns -1 where the reference reports an
// error ('Inflow' on the back face, 'Outflow' on the front face).
int field_type(int face, int pb, int comp) {
  if (pb == FEN_BC_PERIODIC) return FT_PERIODIC;
  if (pb == FEN_BC_WALL) return comp == 0 ? FT_NEUMANN : FT_DIRICHLET;
  if (pb == FEN_BC_INFLOW) {
    if (face == F_BACK) return -1;
    if (comp == 0) return FT_NEUMANN;
    if (face == F_LEFT || face == F_RIGHT) return comp == 1 ? FT_DIRICHLET : FT_NEUMANN;
    return FT_DIRICHLET;
  }
  if (pb == FEN_BC_OUTFLOW) {
    if (face == F_FRONT) return -1;
    return comp == 0 ? FT_DIRICHLET : FT_NEUMANN;
  }
  return -1;
}

double ffloat(long long n) { return (double)(float)n; }  // Fortran float(n)

// One stage of the Poisson plan.  `la` is a precision-neutral descriptor; typed pointers
// are attached at launch (fdst_v, invlam_v, loader inputs).
struct Stage {
  int kind;          // 0 = line transform, 1 = Thomas
  int op, ld, st, contig;
  LineArgs<double> la;
  void* fdst_v;
  void* invlam_v;
  dim3 grid;
  size_t smem;
  ThomasArgs ta;
  dim3 tgrid;
};

}  // namespace

struct fen_ctx {
  fen_params prm{};
  int mixed = 0;
  int dim = 2;
  int n[3] = {1, 1, 1};
  double d[3] = {1, 1, 1};
  double dmin = 1;
  int iso = 1;
  int pbc[6] = {0, 0, 0, 0, 0, 0};
  int periodic[3] = {1, 1, 1};
  Layout L{};
  int ftype[5][6];
  double* bcval[5][6];
  // FP64 state (both forms) and FP64-form work fields
  double *u = nullptr, *v = nullptr, *w = nullptr, *p = nullptr, *phi = nullptr;
  double *us = nullptr, *vs = nullptr, *ws = nullptr;
  double* dvo[3] = {nullptr, nullptr, nullptr};
  double* S[3] = {nullptr, nullptr, nullptr};
  // mixed-form FP32 fields: the state as hi/lo pairs, phi, v* (pairs), dv_o, S
  float *u32 = nullptr, *v32 = nullptr, *w32 = nullptr, *p32 = nullptr, *phi32 = nullptr;
  float *u32l = nullptr, *v32l = nullptr, *w32l = nullptr, *p32l = nullptr;
  float* dphi32 = nullptr;  // refinement: correction of phi
  float *dv32h = nullptr, *dv32l = nullptr;  // refinement: pair divergence of v* from the first transform
  int refine = 0;
  int phi_offset = 0;  // phi32 still holds its mean (deferred_mean) until the next download
  float* d32[3] = {nullptr, nullptr, nullptr};
  float* dvo32[3] = {nullptr, nullptr, nullptr};
  float* d32l[3] = {nullptr, nullptr, nullptr};    // v* lo (pairs with d32)
  float* dvo32l[3] = {nullptr, nullptr, nullptr};  // dv_o lo (pairs with dvo32)
  double* tmp64 = nullptr;                         // FP64 staging of dv_o pairs
  // variable-property path (FP64)
  double *rho = nullptr, *mu = nullptr, *p_o = nullptr;
  int var_rho = 0, var_mu = 0, split = 0;
  double rhomin = 1.0;
  // IBM forcing lists per velocity component (device arrays)
  struct Ibm {
    long long *idx = nullptr, *nidx = nullptr;
    int* nn = nullptr;
    double *w = nullptr, *c0 = nullptr, *vs = nullptr, *fe = nullptr;
    int n = 0;
  } ibm[3];
  float* S32[3] = {nullptr, nullptr, nullptr};
  int has_S = 0;
  // poisson
  int solver = -1;
  double* mwn[3] = {nullptr, nullptr, nullptr};
  double *ta = nullptr, *tb = nullptr, *tc = nullptr;  // tridiagonal a, b, c (device)
  double *c1 = nullptr, *fac = nullptr;
  int* conv = nullptr;        // first row of the pivots' fixed point per system
  double tri_a = 0.0;         // sub-diagonal of the interior rows
  int tab_pairs = 0;          // c1 / fac hold (hi, lo) float pairs (the double-float sweep)
  void* specC = nullptr;
  void* specR = nullptr;
  void* inv_lam = nullptr;
  std::vector<void*> twbufs;
  AxisTw tw[3], twf[3];
  const double2* wfull[3] = {nullptr, nullptr, nullptr};   // exp(-2 pi i m/n), c2c stages
  const double2* wfullf[3] = {nullptr, nullptr, nullptr};  // the same as float2
  FFTPlan plan_half[3], plan_full[3];
  std::vector<Stage> stages;
  int needs_mean = 0;
  double mean_div = 1;
  double* partial = nullptr;
  int npartial = 0;
  // reductions
  double *pdiv = nullptr, *pvel = nullptr;
  int nred = 0;
  int* nan_flag = nullptr;
  StepScalars* sc = nullptr;
  StepScalars* sc_host = nullptr;  // pinned mirror
  int have_dt = 0;
  int vel_dirty = 1;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  long long launches = 0;
  long long launches_per_step = 0;
  double* stage_scratch = nullptr;  // host-layout staging for upload/download (one field)
  double* util = nullptr;           // fields_mod operators: 3 interior arrays + one FP64 field
  // discrete adjoint (2D periodic FP64): checkpoints, recomputed step inputs, adjoint fields
  struct Adjoint {
    int nsteps = 0, every = 0, nckpt = 0, nf = 0, nv = 0;
    double dt = 0;
    std::vector<double*> ckpt;    // nckpt+1 checkpoints x nf fields (u, v, [w,] p, dv_o x, y[, z])
    std::vector<double*> inputs;  // every x nv fields (the velocity at the start of each step)
    double *uh = nullptr, *vh = nullptr, *wh = nullptr, *ph = nullptr, *dou = nullptr, *dov = nullptr, *dow = nullptr;
    double *fh = nullptr, *bh = nullptr, *ush = nullptr, *vsh = nullptr, *wsh = nullptr;
    double *dhu = nullptr, *dhv = nullptr, *dhw = nullptr, *part = nullptr;
    const double** dtab = nullptr;  // device copy of `inputs` (the graph-replayed step reads its entry)
    int* dslot = nullptr;           // entry of the step being transposed
    double fwd_ms = 0, bwd_ms = 0;
    bool ready = false;
  } adj;
};

namespace {

int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

// Radix schedule: the largest power-of-two radices up to maxr first (fft_max_radix gives the
// kernels' limits), then 3s; the earlier radices' product is then a power of two at every
// power-of-two pass.
bool make_plan(int M, FFTPlan& P, int maxr) {
  P.M = M;
  P.nst = 0;
  int m = M;
  if (maxr >= 16)
    while (m % 16 == 0) { P.R[P.nst++] = 16; m /= 16; }
  if (maxr >= 8)
    while (m % 8 == 0) { P.R[P.nst++] = 8; m /= 8; }
  while (m % 4 == 0) { P.R[P.nst++] = 4; m /= 4; }
  if (m % 2 == 0) { P.R[P.nst++] = 2; m /= 2; }
  while (m % 3 == 0) { P.R[P.nst++] = 3; m /= 3; }
  fft_plan_magic(P);
  return m == 1 && P.nst <= kMaxStages;
}

template <typename V>
int upload_vec(fen_ctx* c, const std::vector<V>& h, const double2** out) {
  void* d = nullptr;
  CK(cudaMalloc(&d, std::max<size_t>(h.size(), 1) * sizeof(V)));
  CK(cudaMemcpy(d, h.data(), h.size() * sizeof(V), cudaMemcpyHostToDevice));
  c->twbufs.push_back(d);
  *out = (const double2*)d;
  return 0;
}

int upload_table(fen_ctx* c, const std::vector<double2>& h, const double2** out64, const double2** out32) {
  int r;
  if ((r = upload_vec(c, h, out64))) return r;
  std::vector<float2> f(h.size());
  for (size_t q = 0; q < h.size(); ++q) f[q] = make_float2((float)h[q].x, (float)h[q].y);
  return upload_vec(c, f, out32);
}

// Twiddles of one axis of real length n (periodic: r2c/c2c; Neumann: DCT).
int make_axis(fen_ctx* c, int ax, int n) {
  FFTPlan ph, pf;
  const int maxr = c->mixed ? (ax == 0 ? kFftMaxR32Row : kFftMaxR32Col) : kFftMaxR64;
  if (n % 2 != 0 || !make_plan(n / 2, ph, maxr) || !make_plan(n, pf, maxr))
    return fail(FEN_ERR_ARG, "grid size " + std::to_string(n) + " must be 2^a 3^b with a >= 1");
  c->plan_half[ax] = ph;
  c->plan_full[ax] = pf;
  std::vector<double2> wh(n / 2), wf(n), wn(n / 2 + 1), wd(n);
  for (int m = 0; m < n / 2; ++m) { double a = 2.0 * M_PI * m / (double)(n / 2); wh[m] = make_double2(cos(a), -sin(a)); }
  for (int m = 0; m < n; ++m) { double a = 2.0 * M_PI * m / (double)n; wf[m] = make_double2(cos(a), -sin(a)); }
  for (int k = 0; k <= n / 2; ++k) { double a = 2.0 * M_PI * k / (double)n; wn[k] = make_double2(cos(a), -sin(a)); }
  for (int k = 0; k < n; ++k) { double a = M_PI * k / (2.0 * n); wd[k] = make_double2(cos(a), -sin(a)); }
  int r;
  if ((r = upload_table(c, wh, &c->tw[ax].wM, &c->twf[ax].wM))) return r;
  if ((r = upload_table(c, wf, &c->wfull[ax], &c->wfullf[ax]))) return r;
  if ((r = upload_table(c, wn, &c->tw[ax].wN, &c->twf[ax].wN))) return r;
  if ((r = upload_table(c, wd, &c->tw[ax].wD, &c->twf[ax].wD))) return r;
  return 0;
}

// Modified wavenumbers (poisson.f90:141, 265).
std::vector<double> mwn_host(int n, double delta, bool neumann) {
  std::vector<double> m(n);
  for (int i = 1; i <= n; ++i) {
    const double num = neumann ? 1.0 * M_PI * (i - 1.0) / ffloat(n) : 2.0 * M_PI * (i - 1.0) / ffloat(n);
    volatile double cs = cos(num);
    volatile double t1 = cs - 1.0;
    volatile double t2 = 2.0 * t1;
    volatile double dd = delta * delta;
    m[i - 1] = t2 / dd;
  }
  return m;
}

template <typename T>
int alloc(T** p, long long n) {
  CK(cudaMalloc((void**)p, (size_t)std::max<long long>(n, 1) * sizeof(T)));
  CK(cudaMemset(*p, 0, (size_t)std::max<long long>(n, 1) * sizeof(T)));
  return 0;
}

size_t cplx_size(fen_ctx* c) { return c->mixed ? sizeof(float2) : sizeof(double2); }
size_t real_size(fen_ctx* c) { return c->mixed ? sizeof(float) : sizeof(double); }

LineArgs<double> base_line(fen_ctx* c) {
  LineArgs<double> a;
  memset(&a, 0, sizeof(a));
  a.L = c->L;
  a.scale = 1.0;
  a.sc = c->sc;
  for (int q = 0; q < 3; ++q) a.id[q] = 1.0 / c->d[q];
  a.iso = c->iso;
  a.dim = c->dim;
  return a;
}

// Contiguous x-line stage: lines = rows (ny per plane), outer = planes.
Stage x_stage(fen_ctx* c, int op, int ld, int st) {
  Stage s;
  memset(&s, 0, sizeof(s));
  s.kind = 0; s.op = op; s.ld = ld; s.st = st; s.contig = 1;
  s.la = base_line(c);
  const int nx = c->n[0];
  const int M = nx / 2;
// (measured: 2048 against 1024 and 512 complex elements per CTA; mixed channel inverse x
// 0.44 -> 0.38 ms, the FP64 x transforms unchanged or slightly faster)
#ifndef FEN_ROW_ELEMS
#define FEN_ROW_ELEMS 2048
#endif
  int nl = std::max(1, std::min(16, FEN_ROW_ELEMS / M));  // lines per CTA: about FEN_ROW_ELEMS complex elements
  // small grids (2D): fewer lines per CTA so that the launch still spreads over the SMs
  const long long rows = (long long)c->n[1] * (c->dim == 3 ? c->n[2] : 1);
  while (nl > 1 && cdiv(rows, nl) < 2 * 152) nl /= 2;
  s.la.n = nx;
  s.la.nl = nl;
  s.la.nlines = c->n[1];
  s.la.plan = c->plan_half[0];
  s.la.tw = c->mixed ? c->twf[0] : c->tw[0];
  s.grid = dim3(cdiv(c->n[1], nl), c->dim == 3 ? c->n[2] : 1);
  s.smem = 2 * (size_t)nl * M * cplx_size(c);
  return s;
}

// Strided stage along axis ax (1 or 2) over `ncol` consecutive columns.
Stage s_stage(fen_ctx* c, int op, int ld, int st, int ax, int ncol, int nouter, long long in_pos, long long in_outer,
              long long out_pos, long long out_outer, const void* in, void* out) {
  Stage s;
  memset(&s, 0, sizeof(s));
  s.kind = 0; s.op = op; s.ld = ld; s.st = st; s.contig = 0;
  s.la = base_line(c);
  const int n = c->n[ax];
  const bool cc = (op == OP_C2C_F || op == OP_C2C_I || op == OP_C2C_SOLVE);
  const int M = cc ? n : n / 2;
  // columns per CTA (build-time knobs): 8 FP32 complex columns (64-byte row segments) or 4
  // FP64 ones (64 bytes); measured against 16/8 and 4/8: FP32 column transforms 1.10 -> 0.90
  // ms per mixed channel step, FP64 1.82 -> 1.77 ms per 256^3 TGV step
#ifndef FEN_COL32_NL
#define FEN_COL32_NL 8
#endif
#ifndef FEN_COL64_NL
#define FEN_COL64_NL 4
#endif
  // long columns take fewer per CTA, down to one (two ping-pong buffers of nl * M complex
  // values in at most 200 KB of shared memory): FP64 columns up to 6144 points, FP32 up to
  // 12288 (x lines: FP64 12288 points, FP32 24576)
  int nl = c->mixed ? FEN_COL32_NL : FEN_COL64_NL;
  while (nl > 1 && 2 * (size_t)nl * M * cplx_size(c) > 200 * 1024) nl /= 2;
  s.la.n = n;
  s.la.nl = nl;
  s.la.nlines = ncol;
  s.la.in = in; s.la.out = out;
  s.la.in_line = 1; s.la.in_pos = in_pos; s.la.in_outer = in_outer;
  s.la.out_line = 1; s.la.out_pos = out_pos; s.la.out_outer = out_outer;
  s.la.plan = cc ? c->plan_full[ax] : c->plan_half[ax];
  s.la.tw = c->mixed ? c->twf[ax] : c->tw[ax];
  if (cc) s.la.tw.wM = c->mixed ? c->wfullf[ax] : c->wfull[ax];
  s.grid = dim3(cdiv(ncol, nl), nouter);
  s.smem = 2 * (size_t)nl * M * cplx_size(c);
  return s;
}

Stage t_stage(fen_ctx* c, void* x, long long s_col, long long s_row, long long s_outer, int ncol, int nouter, int n, int form3) {
  Stage s;
  memset(&s, 0, sizeof(s));
  s.kind = 1;
  s.ta.x = x;
  s.ta.s_col = s_col; s.ta.s_row = s_row; s.ta.s_outer = s_outer;
  s.ta.ncol = ncol; s.ta.nouter = nouter; s.ta.n = n;
  s.ta.a = c->ta;
  s.ta.c1 = c->c1;
  s.ta.fac = c->fac;
  s.ta.conv = c->conv;
  s.ta.aval = c->tri_a;
  s.ta.form3 = form3;
  s.tgrid = dim3(cdiv(ncol, 128), nouter);
  return s;
}

// Tridiagonal coefficients along axis ax (poisson.f90:216-232) and their tables.
int init_tridiag(fen_ctx* c, int ax, int ncol, int nouter, const double* lamA, const double* lamB, int form3) {
  const int n = c->n[ax];
  const double dl = c->d[ax];
  std::vector<double> a(n), b(n), cc(n);
  for (int j = 0; j < n; ++j) {
    volatile double dd = dl * dl;
    a[j] = 1.0 / dd;
    b[j] = -2.0 / dd;
    cc[j] = 1.0 / dd;
  }
  b[0] = b[0] + a[0];
  if (c->pbc[2 * ax] == FEN_BC_INFLOW && c->pbc[2 * ax + 1] == FEN_BC_OUTFLOW) b[n - 1] = b[n - 1] - cc[n - 1];
  else b[n - 1] = b[n - 1] + cc[n - 1];
  a[0] = 0.0;
  cc[n - 1] = 0.0;
  int r;
  if ((r = alloc(&c->ta, n)) || (r = alloc(&c->tb, n)) || (r = alloc(&c->tc, n))) return r;
  CK(cudaMemcpy(c->ta, a.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->tb, b.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->tc, cc.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  const long long nt = (long long)n * ncol * nouter;
  if ((r = alloc(&c->c1, nt)) || (r = alloc(&c->fac, nt)) || (r = alloc(&c->conv, (long long)ncol * nouter))) return r;
  c->tri_a = a[n - 1];  // rows 1 .. n-1 share a = 1/delta^2
  k_thomas_tables<<<dim3(cdiv(ncol, 128), nouter), 128>>>(ncol, nouter, n, c->ta, c->tb, c->tc, lamA, lamB, form3, c->c1, c->fac,
                                                        c->conv);
  CK(cudaGetLastError());
  // the mixed form's 3D solves sweep in double-float and read the tables as float pairs
  c->tab_pairs = (FEN_THOMAS_DF && c->mixed && form3) ? 1 : 0;
  if (c->tab_pairs) {
    k_thomas_pair_tables<<<(int)std::min<long long>(cdiv(nt, 256), 4096), 256>>>(nt, c->c1, c->fac);
    CK(cudaGetLastError());
  }
  CK(cudaDeviceSynchronize());
  return 0;
}

// Tabulate scale/lam for a SOLVE stage (same arithmetic as the in-kernel division).
int init_inv_lam(fen_ctx* c, Stage& s, int nouter) {
  const long long total = (long long)s.la.nlines * s.la.n * nouter;
  const int grid = std::min(cdiv(total, 256), 152 * 16);
  if (c->mixed) {
    float* t;
    int r;
    if ((r = alloc(&t, total))) return r;
    k_inv_lam_table<float><<<grid, 256>>>(s.la.nlines, s.la.n, nouter, s.la.lamA, s.la.lamB, s.la.lamC, s.la.scale, t);
    c->inv_lam = t;
  } else {
    double* t;
    int r;
    if ((r = alloc(&t, total))) return r;
    k_inv_lam_table<double><<<grid, 256>>>(s.la.nlines, s.la.n, nouter, s.la.lamA, s.la.lamB, s.la.lamC, s.la.scale, t);
    c->inv_lam = t;
  }
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  s.invlam_v = c->inv_lam;
  return 0;
}

int launch_stage(fen_ctx* c, const Stage& s, int first_from_field, const void* field_src, void* dst = nullptr);

// With g_attr_only set, the launch helpers only raise the kernel's dynamic shared-memory
// limit (done once per context, before any stream capture) instead of launching.
bool g_attr_only = false;

int init_poisson(fen_ctx* c) {
  const int* P = c->periodic;
  if (c->dim == 3) {
    if (P[0] && P[1] && P[2]) c->solver = S_PPP;
    else if (P[0] && P[1] && !P[2]) c->solver = S_PPN;
    else if (!P[0] && P[1] && !P[2]) c->solver = S_NPN;
    else if (!P[0] && !P[1] && !P[2]) c->solver = S_NNN;
    else if (P[0] && !P[1] && P[2]) c->solver = S_PNP;
    else return fail(FEN_ERR_BC, "no fast direct Poisson solver for this combination of periodic axes");
  } else {
    if (P[0] && P[1]) c->solver = S_PP;
    else if (P[0] && !P[1]) c->solver = S_PN;
    else if (!P[0] && !P[1]) c->solver = S_NN;
    else return fail(FEN_ERR_BC, "no fast direct Poisson solver for this combination of periodic axes");
  }
  int r;
  for (int ax = 0; ax < c->dim; ++ax)
    if ((r = make_axis(c, ax, c->n[ax]))) return r;
  const int s = c->solver;
  const bool neu[3] = {!P[0], !P[1], !P[2]};
  for (int ax = 0; ax < c->dim; ++ax) {
    std::vector<double> m = mwn_host(c->n[ax], c->d[ax], neu[ax]);
    if ((r = alloc(&c->mwn[ax], c->n[ax]))) return r;
    CK(cudaMemcpy(c->mwn[ax], m.data(), m.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  const int nx = c->n[0], ny = c->n[1], nz = (c->dim == 3) ? c->n[2] : 1;
  const int h = nx / 2 + 1;
  // complex pitch along x: the h = nx/2 + 1 half-spectrum columns padded to 64 bytes, so the
  // column transforms and tridiagonal sweeps move whole 64-byte segments of every row
  const int padc = FEN_SPEC_PAD ? (c->mixed ? 8 : 4) : 1;
  const long long hp = (h + padc - 1) / padc * padc;
  c->stages.clear();
  c->needs_mean = (s == S_PP || s == S_PN || s == S_PPN || s == S_PNP);
  c->mean_div = ffloat((long long)nx * ny * nz);
  if (s == S_PP || s == S_PN || s == S_PPP || s == S_PPN || s == S_PNP) {
    CK(cudaMalloc(&c->specC, (size_t)hp * ny * nz * cplx_size(c)));
    void* C = c->specC;
    Stage x0 = x_stage(c, OP_R2C, LD_DIV, ST_CPLX);
    x0.la.out = C;
    x0.la.out_line = hp; x0.la.out_pos = 1; x0.la.out_outer = hp * ny;
    if (s == S_PN || s == S_PPN || s == S_PNP) x0.la.scale = 1.0 / ffloat(nx);  // poisson.f90:341, 1074
    c->stages.push_back(x0);
    if (s == S_PP) {
      Stage y = s_stage(c, OP_C2C_SOLVE, LD_CPLX, ST_CPLX, 1, h, 1, hp, 0, hp, 0, C, C);
      y.la.scale = 1.0 / ffloat((long long)nx * ny);  // :458
      y.la.lamA = c->mwn[0]; y.la.lamB = nullptr; y.la.lamC = c->mwn[1];
      if ((r = init_inv_lam(c, y, 1))) return r;
      c->stages.push_back(y);
    } else if (s == S_PPP) {
      c->stages.push_back(s_stage(c, OP_C2C_F, LD_CPLX, ST_CPLX, 1, h, nz, hp, hp * ny, hp, hp * ny, C, C));
      Stage z = s_stage(c, OP_C2C_SOLVE, LD_CPLX, ST_CPLX, 2, h, ny, hp * ny, hp, hp * ny, hp, C, C);
      z.la.scale = 1.0 / ffloat((long long)nx * ny * nz);  // :992
      z.la.lamA = c->mwn[0]; z.la.lamB = c->mwn[1]; z.la.lamC = c->mwn[2];
      if ((r = init_inv_lam(c, z, ny))) return r;
      c->stages.push_back(z);
      c->stages.push_back(s_stage(c, OP_C2C_I, LD_CPLX, ST_CPLX, 1, h, nz, hp, hp * ny, hp, hp * ny, C, C));
    } else if (s == S_PN) {
      if ((r = init_tridiag(c, 1, h, 1, c->mwn[0], nullptr, 0))) return r;
      c->stages.push_back(t_stage(c, C, 1, hp, 0, h, 1, ny, 0));
    } else if (s == S_PPN) {
      Stage y = s_stage(c, OP_C2C_F, LD_CPLX, ST_CPLX, 1, h, nz, hp, hp * ny, hp, hp * ny, C, C);
      y.la.scale = 1.0 / ffloat(ny);  // :1087
      c->stages.push_back(y);
      if ((r = init_tridiag(c, 2, h, ny, c->mwn[0], c->mwn[1], 1))) return r;
      c->stages.push_back(t_stage(c, C, 1, hp * ny, hp, h, ny, nz, 1));
      c->stages.push_back(s_stage(c, OP_C2C_I, LD_CPLX, ST_CPLX, 1, h, nz, hp, hp * ny, hp, hp * ny, C, C));
    } else {  // S_PNP: FFT in z (normalised by nz), Thomas in y
      Stage z = s_stage(c, OP_C2C_F, LD_CPLX, ST_CPLX, 2, h, ny, hp * ny, hp, hp * ny, hp, C, C);
      z.la.scale = 1.0 / ffloat(nz);
      c->stages.push_back(z);
      if ((r = init_tridiag(c, 1, h, nz, c->mwn[0], c->mwn[2], 1))) return r;
      c->stages.push_back(t_stage(c, C, 1, hp, hp * ny, h, nz, ny, 1));
      c->stages.push_back(s_stage(c, OP_C2C_I, LD_CPLX, ST_CPLX, 2, h, ny, hp * ny, hp, hp * ny, hp, C, C));
    }
    Stage xi = x_stage(c, OP_C2R, LD_CPLX, ST_FIELD);
    xi.la.in = C;
    xi.la.in_line = hp; xi.la.in_pos = 1; xi.la.in_outer = hp * ny;
    c->stages.push_back(xi);
  } else {
    // DCT-based: nn (2D), npn, nnn
    CK(cudaMalloc(&c->specR, (size_t)nx * ny * nz * real_size(c)));
    void* R = c->specR;
    const long long px = nx;
    Stage x0 = x_stage(c, OP_DCT2, LD_DIV, ST_REAL);
    x0.la.out = R;
    x0.la.out_line = px; x0.la.out_pos = 1; x0.la.out_outer = px * ny;
    if (s != S_NN) x0.la.scale = 1.0 / (double)(nx * 2);  // :1213, :1352
    c->stages.push_back(x0);
    if (s == S_NN) {
      if ((r = init_tridiag(c, 1, nx, 1, c->mwn[0], nullptr, 0))) return r;
      c->stages.push_back(t_stage(c, R, 1, px, 0, nx, 1, ny, 0));
    } else if (s == S_NPN) {
      const int hy = ny / 2 + 1;
      CK(cudaMalloc(&c->specC, (size_t)nx * hy * nz * cplx_size(c)));
      void* C = c->specC;
      Stage y = s_stage(c, OP_R2C, LD_REAL, ST_CPLX, 1, nx, nz, px, px * ny, px, px * hy, R, C);
      y.la.scale = 1.0 / (double)ny;  // :1226
      c->stages.push_back(y);
      if ((r = init_tridiag(c, 2, nx, hy, c->mwn[0], c->mwn[1], 1))) return r;
      c->stages.push_back(t_stage(c, C, 1, px * hy, px, nx, hy, nz, 1));
      c->stages.push_back(s_stage(c, OP_C2R, LD_CPLX, ST_REAL, 1, nx, nz, px, px * hy, px, px * ny, C, R));
    } else {  // nnn
      Stage y = s_stage(c, OP_DCT2, LD_REAL, ST_REAL, 1, nx, nz, px, px * ny, px, px * ny, R, R);
      y.la.scale = 1.0 / (double)(ny * 2);  // :1365
      c->stages.push_back(y);
      if ((r = init_tridiag(c, 2, nx, ny, c->mwn[0], c->mwn[1], 1))) return r;
      c->stages.push_back(t_stage(c, R, 1, px * ny, px, nx, ny, nz, 1));
      c->stages.push_back(s_stage(c, OP_DCT3, LD_REAL, ST_REAL, 1, nx, nz, px, px * ny, px, px * ny, R, R));
    }
    Stage xi = x_stage(c, OP_DCT3, LD_REAL, ST_FIELD);
    xi.la.in = R;
    xi.la.in_line = px; xi.la.in_pos = 1; xi.la.in_outer = px * ny;
    if (s == S_NN) xi.la.scale = 1.0 / ffloat((long long)nx * 2);  // :594
    c->stages.push_back(xi);
  }
  // raise the shared-memory limit of every transform kernel this plan uses (both loaders
  // of the first stage)
  g_attr_only = true;
  for (size_t q = 0; q < c->stages.size(); ++q) {
    if (c->stages[q].kind != 0) continue;
    if ((r = launch_stage(c, c->stages[q], 0, nullptr)) || (q == 0 && (r = launch_stage(c, c->stages[q], 1, nullptr)))) {
      g_attr_only = false;
      return r;
    }
  }
  g_attr_only = false;
  // per-CTA partial sums of the last stage (mean removal)
  Stage& last = c->stages.back();
  c->npartial = (int)(last.grid.x * last.grid.y);
  if ((r = alloc(&c->partial, c->npartial))) return r;
  last.la.partial = c->needs_mean ? c->partial : nullptr;
  last.fdst_v = c->mixed ? (void*)c->phi32 : (void*)c->phi;
  return 0;
}

// ---------------------------------------------------------------------------------------
// Launch helpers
// ---------------------------------------------------------------------------------------
template <typename T>
LineArgs<T> typed_args(const Stage& s);

template <>
LineArgs<double> typed_args<double>(const Stage& s) {
  LineArgs<double> a = s.la;
  a.fdst = (double*)s.fdst_v;
  a.inv_lam = (const double*)s.invlam_v;
  return a;
}

template <>
LineArgs<float> typed_args<float>(const Stage& s) {
  const LineArgs<double>& d = s.la;
  LineArgs<float> a;
  memset(&a, 0, sizeof(a));
  a.n = d.n; a.nl = d.nl; a.nlines = d.nlines;
  a.in = d.in; a.out = d.out;
  a.in_line = d.in_line; a.in_pos = d.in_pos; a.in_outer = d.in_outer;
  a.out_line = d.out_line; a.out_pos = d.out_pos; a.out_outer = d.out_outer;
  a.L = d.L;
  a.partial = d.partial;
  a.scale = d.scale;
  a.scale32 = (float)d.scale;
  a.scaled = d.scale != 1.0;
  a.sc = d.sc;
  for (int q = 0; q < 3; ++q) a.id[q] = d.id[q];
  a.iso = d.iso; a.dim = d.dim;
  a.lamA = d.lamA; a.lamB = d.lamB; a.lamC = d.lamC;
  a.plan = d.plan;
  a.tw = d.tw;
  a.fdst = (float*)s.fdst_v;
  a.inv_lam = (const float*)s.invlam_v;
  return a;
}

template <typename T, int DIM, bool CONTIG, int OP, int LD, int ST>
int launch_line_t(fen_ctx* c, const Stage& s, const LineArgs<T>& a) {
  void (*kern)(LineArgs<T>);
  if constexpr (sizeof(T) == 4 && CONTIG) kern = k_line_row32<DIM, OP, LD, ST>;
  else kern = k_line<T, DIM, CONTIG, OP, LD, ST>;
  if (s.smem > 200 * 1024) return fail(FEN_ERR_ARG, "transform length too large for one CTA");
  if (g_attr_only) {
    CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    return 0;
  }
  LineArgs<T> b = a;
  constexpr bool real_fft = (OP == OP_R2C || OP == OP_C2R || OP == OP_DCT2 || OP == OP_DCT3);
  const int M = real_fft ? b.n / 2 : b.n;
  b.mg[0] = fft_magic((unsigned)b.n);
  b.mg[1] = fft_magic((unsigned)M);
  b.mg[2] = fft_magic((unsigned)(M + 1));
  b.mg[3] = fft_magic((unsigned)b.nl);
  kern<<<s.grid, 256, s.smem, c->stream>>>(b);
  c->launches++;
  CK(cudaGetLastError());
  return 0;
}

template <typename T, int DIM>
int launch_line_dim(fen_ctx* c, const Stage& s, int ld, const LineArgs<T>& a) {
  if (s.contig) {
    if (s.op == OP_R2C && ld == LD_DIV) return launch_line_t<T, DIM, true, OP_R2C, LD_DIV, ST_CPLX>(c, s, a);
    if (s.op == OP_R2C && ld == LD_DIVMIX) return launch_line_t<T, DIM, true, OP_R2C, LD_DIVMIX, ST_CPLX>(c, s, a);
    if (s.op == OP_R2C && ld == LD_FIELD) return launch_line_t<T, DIM, true, OP_R2C, LD_FIELD, ST_CPLX>(c, s, a);
    if (s.op == OP_DCT2 && ld == LD_DIV) return launch_line_t<T, DIM, true, OP_DCT2, LD_DIV, ST_REAL>(c, s, a);
    if (s.op == OP_DCT2 && ld == LD_DIVMIX) return launch_line_t<T, DIM, true, OP_DCT2, LD_DIVMIX, ST_REAL>(c, s, a);
    if (s.op == OP_DCT2 && ld == LD_FIELD) return launch_line_t<T, DIM, true, OP_DCT2, LD_FIELD, ST_REAL>(c, s, a);
    if constexpr (sizeof(T) == 4) {
      if (s.op == OP_R2C && ld == LD_RESID) return launch_line_t<T, DIM, true, OP_R2C, LD_RESID, ST_CPLX>(c, s, a);
      if (s.op == OP_DCT2 && ld == LD_RESID) return launch_line_t<T, DIM, true, OP_DCT2, LD_RESID, ST_REAL>(c, s, a);
    }
    if (s.op == OP_C2R) return launch_line_t<T, DIM, true, OP_C2R, LD_CPLX, ST_FIELD>(c, s, a);
    if (s.op == OP_DCT3) return launch_line_t<T, DIM, true, OP_DCT3, LD_REAL, ST_FIELD>(c, s, a);
  } else {
    if (s.op == OP_C2C_F) return launch_line_t<T, 3, false, OP_C2C_F, LD_CPLX, ST_CPLX>(c, s, a);
    if (s.op == OP_C2C_I) return launch_line_t<T, 3, false, OP_C2C_I, LD_CPLX, ST_CPLX>(c, s, a);
    if (s.op == OP_C2C_SOLVE) return launch_line_t<T, 3, false, OP_C2C_SOLVE, LD_CPLX, ST_CPLX>(c, s, a);
    if (s.op == OP_R2C) return launch_line_t<T, 3, false, OP_R2C, LD_REAL, ST_CPLX>(c, s, a);
    if (s.op == OP_C2R) return launch_line_t<T, 3, false, OP_C2R, LD_CPLX, ST_REAL>(c, s, a);
    if (s.op == OP_DCT2) return launch_line_t<T, 3, false, OP_DCT2, LD_REAL, ST_REAL>(c, s, a);
    if (s.op == OP_DCT3) return launch_line_t<T, 3, false, OP_DCT3, LD_REAL, ST_REAL>(c, s, a);
  }
  return fail(FEN_ERR_ARG, "unsupported transform stage");
}

// launch_stage's first_from_field: 1 loads the first transform from a field, kFirstResidual
// forms the mixed refinement's residual from v* and the field phi.
constexpr int kFirstResidual = 2;

template <typename T>
int launch_stage_t(fen_ctx* c, const Stage& s, int first_from_field, const void* field_src, void* dst) {
  LineArgs<T> a = typed_args<T>(s);
  if (dst && s.st == ST_FIELD) a.fdst = (T*)dst;
  for (int q = 0; q < 3; ++q) a.idp[q] = split_d(1.0 / c->d[q]);
  int ld = s.ld;
  if (first_from_field == kFirstResidual) {
    // mixed refinement: the first transform forms its own right-hand side from v* and phi
    if (!c->dv32h) return fail(FEN_ERR_STATE, "refinement without its divergence buffer");
    ld = LD_RESID;
    a.fsrc = (const T*)field_src;
    a.dvh = c->dv32h; a.dvl = c->dv32l;
    for (int q = 0; q < 3; ++q) a.id2p[q] = split_d(1.0 / (c->d[q] * c->d[q]));
  } else if (first_from_field) {
    ld = LD_FIELD;
    a.fsrc = (const T*)field_src;
  } else if (s.ld == LD_DIV) {
    if (c->mixed) {
      ld = LD_DIVMIX;
      a.pu = DFField{c->d32[0], c->d32l[0]}; a.pv = DFField{c->d32[1], c->d32l[1]}; a.pw = DFField{c->d32[2], c->d32l[2]};
      if (c->refine) { a.dvh = c->dv32h; a.dvl = c->dv32l; }
    } else {
      a.fu = (const T*)c->us; a.fv = (const T*)c->vs; a.fw = (const T*)c->ws;
      if (c->var_rho && !c->split) a.rho_c = c->rho;
    }
  }
  return (c->dim == 3) ? launch_line_dim<T, 3>(c, s, ld, a) : launch_line_dim<T, 2>(c, s, ld, a);
}

int launch_thomas(fen_ctx* c, const Stage& s) {
  const bool real = (c->solver == S_NN || c->solver == S_NNN);
  ThomasArgs ta = s.ta;
  ta.split2 = 0;
  constexpr int kTh = 128;  // (64-thread CTAs measured no faster)
  // the mixed form's reciprocal-factor (3D) solves take the two-FMA sweep above the pivots'
  // fixed point; the FP64 form keeps the reference's operation order
  const bool fast = FEN_THOMAS_FAST && c->mixed && ta.form3;
  const bool pairs = c->tab_pairs != 0;
  {
    const F2 av = split_d(ta.aval);
    ta.avh = av.hi;
    ta.avl = av.lo;
  }
  if (real) {
    const dim3 g(cdiv(ta.ncol, kTh), s.tgrid.y, s.tgrid.z);
    if (pairs) k_thomas_df<0><<<g, kTh, 0, c->stream>>>(ta);
    else if (fast) k_thomas_mixed<0><<<g, kTh, 0, c->stream>>>(ta);
    else if (c->mixed) k_thomas<float, double><<<g, kTh, 0, c->stream>>>(ta);
    else k_thomas<double, double><<<g, kTh, 0, c->stream>>>(ta);
  } else {
    // complex right-hand sides: real and imaginary parts as two real systems per column
    ta.split2 = 1;
    const dim3 g(cdiv(2LL * ta.ncol, kTh), s.tgrid.y, s.tgrid.z);
    if (pairs) k_thomas_df<1><<<g, kTh, 0, c->stream>>>(ta);
    else if (fast) k_thomas_mixed<1><<<g, kTh, 0, c->stream>>>(ta);
    else if (c->mixed) k_thomas<float, double><<<g, kTh, 0, c->stream>>>(ta);
    else k_thomas<double, double><<<g, kTh, 0, c->stream>>>(ta);
  }
  c->launches++;
  CK(cudaGetLastError());
  return 0;
}

int launch_stage(fen_ctx* c, const Stage& s, int first_from_field, const void* field_src, void* dst) {
  if (s.kind == 1) return g_attr_only ? 0 : launch_thomas(c, s);
  return c->mixed ? launch_stage_t<float>(c, s, first_from_field, field_src, dst)
                  : launch_stage_t<double>(c, s, first_from_field, field_src, dst);
}

FieldBC field_bc(fen_ctx* c, int f, bool homogeneous = false) {
  FieldBC b;
  for (int q = 0; q < 6; ++q) {
    b.type[q] = c->ftype[f][q];
    b.val[q] = homogeneous ? nullptr : c->bcval[f][q];
  }
  b.c = (f == FEN_U) ? 'x' : (f == FEN_V) ? 'y' : (f == FEN_W) ? 'z' : 'c';
  return b;
}

// Fill ghosts of up to four ghosted fields; `ids` give the bc set of each pointer.
// `homogeneous` uses zero Dirichlet values (increments of fields that satisfy the BCs).
template <typename T>
int ghost(fen_ctx* c, int nf, T* const* ptr, const int* ids, bool homogeneous = false, bool low_only = false) {
  GhostBatch<T> G;
  memset(&G, 0, sizeof(G));
  long long mx = 0;
  for (int q = 0; q < nf; ++q) {
    G.f[q] = ptr[q];
    G.bc[q] = field_bc(c, ids[q], homogeneous);
    GhostCount g = (c->dim == 3) ? ghost_count<3>(c->L, G.bc[q]) : ghost_count<2>(c->L, G.bc[q]);
    G.n[q] = g.a + g.b + g.c;
    G.shift[q] = 0.0;
    G.gd[q] = (c->dim == 3) ? ghost_div<3>(c->L, G.bc[q]) : ghost_div<2>(c->L, G.bc[q]);
    G.low[q] = (low_only && G.bc[q].c != 'c') ? 1 : 0;
    if (G.low[q]) G.n[q] = ghost_low_count(c->L, G.bc[q]);
    mx = std::max(mx, G.n[q]);
  }
  dim3 grid(std::min(cdiv(mx, 256), 4096), nf);
  if (c->dim == 3) k_ghost_fill<T, 3><<<grid, 256, 0, c->stream>>>(c->L, G);
  else k_ghost_fill<T, 2><<<grid, 256, 0, c->stream>>>(c->L, G);
  c->launches++;
  CK(cudaGetLastError());
  return 0;
}

// Remove the mean of phi (poisson.f90:491-503): reduce the inverse transform's partials, then
// subtract.
int launch_mean(fen_ctx* c) {
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  const int grid = std::min(cdiv(ncell, 256), 152 * 8);
  k_mean_reduce<<<1, 1024, 0, c->stream>>>(c->partial, c->npartial, c->mean_div, c->sc);
  if (c->mixed) {
    if (c->dim == 3) k_mean_subtract<float, 3><<<grid, 256, 0, c->stream>>>(c->L, c->sc, c->phi32);
    else k_mean_subtract<float, 2><<<grid, 256, 0, c->stream>>>(c->L, c->sc, c->phi32);
  } else {
    if (c->dim == 3) k_mean_subtract<double, 3><<<grid, 256, 0, c->stream>>>(c->L, c->sc, c->phi);
    else k_mean_subtract<double, 2><<<grid, 256, 0, c->stream>>>(c->L, c->sc, c->phi);
  }
  c->launches += 2;
  CK(cudaGetLastError());
  return 0;
}

int run_poisson(fen_ctx* c, bool from_field) {
  int r;
  const void* src = c->mixed ? (const void*)c->phi32 : (const void*)c->phi;
  for (size_t q = 0; q < c->stages.size(); ++q)
    if ((r = launch_stage(c, c->stages[q], from_field && q == 0, src))) return r;
  if (c->needs_mean && (r = launch_mean(c))) return r;
  return 0;
}

double rhof_of(fen_ctx* c) { return 0.5 * (c->prm.density + c->prm.density); }

// The step takes FEN's variable-property branches when a density or viscosity field was
// uploaded or the split pressure is on.
bool var_path(const fen_ctx* c) { return c->var_rho || c->var_mu || c->split; }

// Mixed form with refinement: the step keeps the mean of phi (removed in the correction's
// pressure update instead of by a separate pass over phi).
bool deferred_mean(const fen_ctx* c) { return FEN_DEFER_MEAN && c->mixed && c->refine && c->needs_mean; }

// Density of the Poisson scaling rho_over_dt: 1 with a density field (the loader multiplies
// by rho(i,j,k)), rhomin with the split, else the constant density.
double rho_scale(const fen_ctx* c) { return c->split ? c->rhomin : (c->var_rho ? 1.0 : c->prm.density); }

template <typename T>
PredArgs<T> pred_args(fen_ctx* c) {
  PredArgs<T> a;
  memset(&a, 0, sizeof(a));
  if (c->mixed) {
    a.u = (const T*)c->u32; a.v = (const T*)c->v32; a.w = (const T*)c->w32; a.p = (const T*)c->p32;
    a.us = (T*)c->d32[0]; a.vs = (T*)c->d32[1]; a.ws = (T*)c->d32[2];
    a.dox = (T*)c->dvo32[0]; a.doy = (T*)c->dvo32[1]; a.doz = (T*)c->dvo32[2];
    a.Sx = (const T*)c->S32[0]; a.Sy = (const T*)c->S32[1]; a.Sz = (const T*)c->S32[2];
  } else {
    a.u = (const T*)c->u; a.v = (const T*)c->v; a.w = (const T*)c->w; a.p = (const T*)c->p;
    a.us = (T*)c->us; a.vs = (T*)c->vs; a.ws = (T*)c->ws;
    a.dox = (T*)c->dvo[0]; a.doy = (T*)c->dvo[1]; a.doz = (T*)c->dvo[2];
    a.Sx = (const T*)c->S[0]; a.Sy = (const T*)c->S[1]; a.Sz = (const T*)c->S[2];
  }
  for (int q = 0; q < 3; ++q) {
    a.id[q] = 1.0 / c->d[q];
    a.id2[q] = 1.0 / (c->d[q] * c->d[q]);
  }
  a.mu = c->prm.viscosity;
  a.rhof = rhof_of(c);  // center_to_face of a constant density
  a.rhof_one = (a.rhof == 1.0);
  for (int q = 0; q < 3; ++q) a.g[q] = c->prm.g[q];
  a.iso = c->iso;
  a.has_S = c->has_S;
  a.use_dev_dt = 1;
  return a;
}

int launch_predictor(fen_ctx* c, const StepScalars* sc) {
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  const int grid = std::min(cdiv(ncell, 256), 152 * 16);
  if (c->mixed) {
    PredDFArgs pa;
    memset(&pa, 0, sizeof(pa));
    pa.u = DFField{c->u32, c->u32l}; pa.v = DFField{c->v32, c->v32l};
    pa.w = DFField{c->w32, c->w32l}; pa.p = DFField{c->p32, c->p32l};
    pa.du = c->d32[0]; pa.dv = c->d32[1]; pa.dw = c->d32[2];
    pa.dul = c->d32l[0]; pa.dvl = c->d32l[1]; pa.dwl = c->d32l[2];
    pa.dox = c->dvo32[0]; pa.doy = c->dvo32[1]; pa.doz = c->dvo32[2];
    pa.doxl = c->dvo32l[0]; pa.doyl = c->dvo32l[1]; pa.dozl = c->dvo32l[2];
    pa.Sx = c->S32[0]; pa.Sy = c->S32[1]; pa.Sz = c->S32[2];
    const double rhof = rhof_of(c);
    double id[3], id2[3];
    for (int q = 0; q < 3; ++q) {
      id[q] = 1.0 / c->d[q];
      id2[q] = 1.0 / (c->d[q] * c->d[q]);
    }
    if (c->iso)
      for (int q = 1; q < 3; ++q) { id[q] = id[0]; id2[q] = id2[0]; }
    F2* qs[3] = {&pa.qx, &pa.qy, &pa.qz};
    F2* ms[3] = {&pa.mx, &pa.my, &pa.mz};
    F2* gs[3] = {&pa.gx, &pa.gy, &pa.gz};
    for (int q = 0; q < 3; ++q) {
      *qs[q] = split_d(0.25 * id[q]);
      *ms[q] = split_d(c->prm.viscosity * id2[q] / rhof);
      *gs[q] = split_d(id[q] / rhof);
      pa.g[q] = split_d(c->prm.g[q]);
    }
    pa.irho = split_d(1.0 / rhof);
    pa.iso = c->iso;
    pa.has_S = c->has_S;
    if (c->dim == 3) {
      const dim3 tg(cdiv(c->n[0], kDTX), cdiv(c->n[1], kDTY), cdiv(c->n[2], kDTZ));
      k_predictor_df_tile<<<tg, dim3(kDTX, kDTY), 0, c->stream>>>(c->L, sc, pa);
    } else {
      k_predictor_df<2><<<grid, 256, 0, c->stream>>>(c->L, sc, pa);
    }
  } else if (var_path(c)) {
    VarArgs va;
    memset(&va, 0, sizeof(va));
    va.u = c->u; va.v = c->v; va.w = c->w; va.p = c->p;
    va.us = c->us; va.vs = c->vs; va.ws = c->ws;
    va.dox = c->dvo[0]; va.doy = c->dvo[1]; va.doz = c->dvo[2];
    va.Sx = c->S[0]; va.Sy = c->S[1]; va.Sz = c->S[2];
    va.rho = c->var_rho ? c->rho : nullptr;
    va.mu = c->mu;
    va.po = c->p_o;
    va.density = c->prm.density;
    va.viscosity = c->prm.viscosity;
    for (int q = 0; q < 3; ++q) {
      va.g[q] = c->prm.g[q];
      va.id[q] = 1.0 / c->d[q];
      va.id2[q] = 1.0 / (c->d[q] * c->d[q]);
    }
    va.irhomin = 1.0 / c->rhomin;
    va.iso = c->iso;
    va.has_S = c->has_S;
    va.var_mu = c->var_mu;
    va.split = c->split;
    va.constant_cfl = c->prm.constant_cfl;
    if (c->dim == 3) k_predictor_var<3><<<grid, 256, 0, c->stream>>>(c->L, sc, va);
    else k_predictor_var<2><<<grid, 256, 0, c->stream>>>(c->L, sc, va);
  } else {
    PredArgs<double> pa = pred_args<double>(c);
    if (c->dim == 3) {
      const dim3 tg(cdiv(c->n[0], kTX), cdiv(c->n[1], kTY), cdiv(c->n[2], kTZ));
      k_predictor_tile<<<tg, dim3(kTX, kTY), 0, c->stream>>>(c->L, sc, pa);
    } else {
      k_predictor<2><<<grid, 256, 0, c->stream>>>(c->L, sc, pa);
    }
  }
  c->launches++;
  CK(cudaGetLastError());
  return 0;
}

int launch_checks(fen_ctx* c, int want_div) {
  if (c->mixed) {
    CheckDFArgs a;
    memset(&a, 0, sizeof(a));
    a.u = DFField{c->u32, c->u32l}; a.v = DFField{c->v32, c->v32l}; a.w = DFField{c->w32, c->w32l};
    for (int q = 0; q < 3; ++q) a.idp[q] = split_d(1.0 / c->d[q]);
    a.want_div = want_div;
    a.pdiv = c->pdiv; a.pvel = c->pvel; a.nan_flag = c->nan_flag;
    if (c->dim == 3) k_checks_df<3><<<c->nred, 256, 0, c->stream>>>(c->L, a);
    else k_checks_df<2><<<c->nred, 256, 0, c->stream>>>(c->L, a);
    c->launches++;
    CK(cudaGetLastError());
    k_finalize<<<1, 256, 0, c->stream>>>(c->pdiv, c->pvel, c->nred, c->sc, c->dmin, 0.0, 1, c->nan_flag);
    c->launches++;
    CK(cudaGetLastError());
    return 0;
  }
  CheckArgs<double> a;
  memset(&a, 0, sizeof(a));
  a.u = c->u; a.v = c->v; a.w = c->w;
  for (int q = 0; q < 3; ++q) a.id[q] = 1.0 / c->d[q];
  a.iso = c->iso;
  a.want_div = want_div;
  a.pdiv = c->pdiv; a.pvel = c->pvel; a.nan_flag = c->nan_flag;
  if (c->dim == 3) k_checks<3><<<c->nred, 256, 0, c->stream>>>(c->L, a);
  else k_checks<2><<<c->nred, 256, 0, c->stream>>>(c->L, a);
  c->launches++;
  CK(cudaGetLastError());
  k_finalize<<<1, 256, 0, c->stream>>>(c->pdiv, c->pvel, c->nred, c->sc, c->dmin, 0.0, 1, c->nan_flag);
  c->launches++;
  CK(cudaGetLastError());
  return 0;
}

// Mixed form: the pair (hi, lo) arrays of a state field.
bool pair_of(fen_ctx* c, int f, float** hi, float** lo, double** d) {
  switch (f) {
    case FEN_U: *hi = c->u32; *lo = c->u32l; *d = c->u; return true;
    case FEN_V: *hi = c->v32; *lo = c->v32l; *d = c->v; return true;
    case FEN_W: *hi = c->w32; *lo = c->w32l; *d = c->w; return true;
    case FEN_P: *hi = c->p32; *lo = c->p32l; *d = c->p; return true;
  }
  return false;
}

// FP64 staging array <-> pairs (every stored element); dir 0: split, 1: join.
int pair_convert(fen_ctx* c, int f, int dir) {
  float *hi, *lo;
  double* d;
  if (!pair_of(c, f, &hi, &lo, &d)) return 0;
  const int grid = std::min(cdiv(c->L.total, 256), 152 * 16);
  if (dir == 0) k_split<<<grid, 256, 0, c->stream>>>(c->L.total, d, hi, lo);
  else k_join<<<grid, 256, 0, c->stream>>>(c->L.total, hi, lo, d);
  c->launches++;
  CK(cudaGetLastError());
  return 0;
}

// Ghost fill of up to four pair fields.
// Ghost fill of pair fields: the state pairs of `ids`, or the pairs (hi[q], lo[q]) with the
// boundary rules of ids[q] when hi is given.
int ghost_pairs(fen_ctx* c, int nf, const int* ids, float* const* hi = nullptr, float* const* lo = nullptr,
                bool low_only = false) {
  GhostDFBatch G;
  memset(&G, 0, sizeof(G));
  long long mx = 0;
  for (int q = 0; q < nf; ++q) {
    if (hi) {
      G.hi[q] = hi[q];
      G.lo[q] = lo[q];
    } else {
      double* d;
      pair_of(c, ids[q], &G.hi[q], &G.lo[q], &d);
    }
    G.bc[q] = field_bc(c, ids[q]);
    GhostCount g = (c->dim == 3) ? ghost_count<3>(c->L, G.bc[q]) : ghost_count<2>(c->L, G.bc[q]);
    G.n[q] = g.a + g.b + g.c;
    G.gd[q] = (c->dim == 3) ? ghost_div<3>(c->L, G.bc[q]) : ghost_div<2>(c->L, G.bc[q]);
    G.low[q] = (low_only && G.bc[q].c != 'c') ? 1 : 0;
    if (G.low[q]) G.n[q] = ghost_low_count(c->L, G.bc[q]);
    mx = std::max(mx, G.n[q]);
  }
  dim3 grid(std::min(cdiv(mx, 256), 4096), nf);
  if (c->dim == 3) k_ghost_fill_df<3><<<grid, 256, 0, c->stream>>>(c->L, G);
  else k_ghost_fill_df<2><<<grid, 256, 0, c->stream>>>(c->L, G);
  c->launches++;
  CK(cudaGetLastError());
  return 0;
}

// One navier_stokes_solver step as a launch sequence on c->stream.  `ev` (optional) gets
// an event after each stage for fen_profile_step.
int enqueue_step(fen_ctx* c, cudaEvent_t* ev) {
  int r;
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  const int grid = std::min(cdiv(ncell, 256), 152 * 16);
  int e = 0;
  auto mark = [&]() { if (ev) cudaEventRecord(ev[e++], c->stream); };
  mark();
  k_prologue<<<1, 32, 0, c->stream>>>(c->sc, c->prm.constant_cfl, c->prm.cfl, c->dmin, rho_scale(c), rhof_of(c));
  c->launches++;
  if ((r = launch_predictor(c, c->sc))) return r;
  mark();  // 1: predictor
  // v* takes the velocity boundary rules (update_ghost_nodes on v*).  Of its ghosts only the
  // divergence's minus neighbours are read -- u*(0, j, k), v*(i, 0, k), w*(i, j, 0) -- besides
  // the last face a wall overwrites, so only those are filled, unless the IBM hook or the
  // variable-property path runs, whose stencils may read others.  Every ghost of the new
  // velocity is filled after the correction.
  const bool v_low = FEN_VSTAR_LOW && !var_path(c) && (c->ibm[0].n + c->ibm[1].n + c->ibm[2].n == 0);
  if (c->mixed) {
    float* f[3] = {c->d32[0], c->d32[1], c->d32[2]};
    float* fl[3] = {c->d32l[0], c->d32l[1], c->d32l[2]};
    int ids[3] = {FEN_U, FEN_V, FEN_W};
    if ((r = ghost_pairs(c, c->dim, ids, f, fl, v_low))) return r;
  } else {
    double* f[3] = {c->us, c->vs, c->ws};
    int ids[3] = {FEN_U, FEN_V, FEN_W};
    if ((r = ghost<double>(c, c->dim, f, ids, false, v_low))) return r;
    if (c->ibm[0].n + c->ibm[1].n + c->ibm[2].n > 0) {
      // apply_ibm_forcing (navier_stokes.f90:106-108), then the boundary conditions again
      for (int q = 0; q < c->dim; ++q) {
        auto& I = c->ibm[q];
        if (!I.n) continue;
        IbmArgs ia{I.idx, I.nn, I.nidx, I.w, I.c0, I.vs, I.fe, f[q], I.n};
        const int g = std::min(cdiv(I.n, 256), 152 * 8);
        k_ibm_target<<<g, 256, 0, c->stream>>>(ia);
        k_ibm_apply<<<g, 256, 0, c->stream>>>(ia, c->sc);
        c->launches += 2;
      }
      CK(cudaGetLastError());
      if ((r = ghost<double>(c, c->dim, f, ids))) return r;
    }
  }
  mark();  // 2: ghost v*
  {
    const size_t ns = c->stages.size();
    for (size_t q = 0; q < ns; ++q) {
      if ((r = launch_stage(c, c->stages[q], 0, nullptr))) return r;
      if (q == 0) mark();       // 3: first (fused divergence) transform
      if (q + 2 == ns) mark();  // 4: spectral middle stages
    }
    if (deferred_mean(c)) {
      // the mean of phi is removed where phi enters p (k_correct_df); the gradient and the
      // refinement's residual do not see it
      k_mean_reduce<<<1, 1024, 0, c->stream>>>(c->partial, c->npartial, c->mean_div, c->sc);
      k_keep_mean<<<1, 1, 0, c->stream>>>(c->sc, 0);
      c->launches += 2;
      CK(cudaGetLastError());
    } else if (c->needs_mean && (r = launch_mean(c))) {
      return r;
    }
  }
  mark();  // 5: inverse x transform (+ mean)
  if (c->mixed) {
    float* f[1] = {c->phi32};
    int ids[1] = {FEN_PHI};
    if ((r = ghost<float>(c, 1, f, ids))) return r;
    if (c->refine) {
      // one iterative-refinement solve: r = b - L_h phi (double-float), L_h dphi = r (FP32)
      // (the residual is formed inside the first transform's load, kFirstResidual)
      const size_t ns = c->stages.size();
      for (size_t q = 0; q < ns; ++q)
        if ((r = launch_stage(c, c->stages[q], q == 0 ? kFirstResidual : 0, c->phi32, c->dphi32))) return r;
      if (c->needs_mean) {  // mean of dphi only: k_correct_df removes it in the pressure update
        k_mean_reduce<<<1, 1024, 0, c->stream>>>(c->partial, c->npartial, c->mean_div, c->sc);
        c->launches++;
        CK(cudaGetLastError());
      }
      float* g[1] = {c->dphi32};
      if ((r = ghost<float>(c, 1, g, ids))) return r;
    }
    CorrDFArgs ca;
    memset(&ca, 0, sizeof(ca));
    ca.du = c->d32[0]; ca.dv = c->d32[1]; ca.dw = c->d32[2]; ca.phi = c->phi32;
    ca.dul = c->d32l[0]; ca.dvl = c->d32l[1]; ca.dwl = c->d32l[2];
    ca.dphi = c->refine ? c->dphi32 : nullptr;
    ca.dphi_mean = c->refine && c->needs_mean;
    ca.phi_mean = deferred_mean(c);
    ca.u = DFFieldW{c->u32, c->u32l}; ca.v = DFFieldW{c->v32, c->v32l};
    ca.w = DFFieldW{c->w32, c->w32l}; ca.p = DFFieldW{c->p32, c->p32l};
    for (int q = 0; q < 3; ++q) ca.id[q] = 1.0 / c->d[q];
    ca.iso = c->iso;
    ca.rhof = rhof_of(c);
    if (c->dim == 3) k_correct_df<3><<<grid, 256, 0, c->stream>>>(c->L, c->sc, ca);
    else k_correct_df<2><<<grid, 256, 0, c->stream>>>(c->L, c->sc, ca);
    c->launches++;
    CK(cudaGetLastError());
  } else {
    double* f[1] = {c->phi};
    int ids[1] = {FEN_PHI};
    if ((r = ghost<double>(c, 1, f, ids))) return r;
    if (var_path(c)) {
      CorrVarArgs va;
      memset(&va, 0, sizeof(va));
      va.us = c->us; va.vs = c->vs; va.ws = c->ws; va.phi = c->phi;
      va.u = c->u; va.v = c->v; va.w = c->w; va.p = c->p; va.po = c->p_o;
      va.rho = c->var_rho ? c->rho : nullptr;
      va.density = c->prm.density;
      va.irhomin = 1.0 / c->rhomin;
      for (int q = 0; q < 3; ++q) va.id[q] = 1.0 / c->d[q];
      va.iso = c->iso;
      va.split = c->split;
      if (c->dim == 3) k_correct_var<3><<<grid, 256, 0, c->stream>>>(c->L, c->sc, va);
      else k_correct_var<2><<<grid, 256, 0, c->stream>>>(c->L, c->sc, va);
      c->launches++;
      CK(cudaGetLastError());
      if (c->split) {
        double* f[1] = {c->p_o};
        int ids[1] = {FEN_P};
        if ((r = ghost<double>(c, 1, f, ids))) return r;
      }
    } else {
      CorrArgs<double> ca;
      memset(&ca, 0, sizeof(ca));
      ca.us = c->us; ca.vs = c->vs; ca.ws = c->ws; ca.phi = c->phi;
      ca.u = c->u; ca.v = c->v; ca.w = c->w; ca.p = c->p;
      for (int q = 0; q < 3; ++q) ca.id[q] = 1.0 / c->d[q];
      ca.iso = c->iso;
      ca.use_dev_dt = 1;
      ca.rhof = rhof_of(c);
      ca.rhof_one = (ca.rhof == 1.0);
      if (c->dim == 3) k_correct<double, 3><<<grid, 256, 0, c->stream>>>(c->L, c->sc, ca);
      else k_correct<double, 2><<<grid, 256, 0, c->stream>>>(c->L, c->sc, ca);
      c->launches++;
      CK(cudaGetLastError());
    }
  }
  mark();  // 6: phi ghost + correction
  {
    double* f[4] = {c->u, c->v, c->w, c->p};
    int ids[4] = {FEN_U, FEN_V, FEN_W, FEN_P};
    double* f2[3] = {c->u, c->v, c->p};
    int ids2[3] = {FEN_U, FEN_V, FEN_P};
    if (c->mixed) {
      if ((r = ghost_pairs(c, c->dim == 3 ? 4 : 3, c->dim == 3 ? ids : ids2))) return r;
    } else if (c->dim == 3) {
      if ((r = ghost<double>(c, 4, f, ids))) return r;
    } else {
      if ((r = ghost<double>(c, 3, f2, ids2))) return r;
    }
  }
  mark();  // 7: ghosts
  if ((r = launch_checks(c, 1))) return r;
  mark();  // 8: checks
  return 0;
}

int host_planes(fen_ctx* c) { return c->dim == 3 ? c->n[2] + 2 : 3; }

// Copy one field between FEN's host layout (gl ghost layers, see k_relayout) and the padded
// HBM layout through a contiguous staging buffer (one memcpy + one relayout kernel).  dir 0:
// host -> device, 1: back.
template <typename T>
int relayout(fen_ctx* c, T* dfield, double* host_rw, int dir, int gl) {
  const int nxh = c->n[0] + 2 * gl, nyh = c->n[1] + 2 * gl;
  const int planes = (c->dim == 3) ? c->n[2] + 2 * gl : 1;
  const size_t cnt = (size_t)nxh * nyh * planes;
  double* h = host_rw + ((c->dim == 2 && gl == 1) ? (size_t)nxh * nyh : 0);  // 2D, gl = 1: plane k = 1
  if (!c->stage_scratch) {
    int r;
    const long long full = (long long)(c->n[0] + 2) * (c->n[1] + 2) * ((c->dim == 3) ? c->n[2] + 2 : 1);
    if ((r = alloc(&c->stage_scratch, full))) return r;
  }
  const int grid = std::min(cdiv((long long)cnt, 256), 152 * 16);
  if (dir == 0) {
    CK(cudaMemcpyAsync(c->stage_scratch, h, cnt * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    k_relayout<T><<<grid, 256, 0, c->stream>>>(c->L, planes, gl, c->stage_scratch, dfield, nullptr, nullptr, 0);
    c->launches++;
    CK(cudaGetLastError());
  } else {
    k_relayout<T><<<grid, 256, 0, c->stream>>>(c->L, planes, gl, nullptr, nullptr, dfield, c->stage_scratch, 1);
    c->launches++;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h, c->stage_scratch, cnt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

// Ghost level of FEN's allocation of each field (navier_stokes.f90:759-768): p, phi, rho,
// mu and v with one layer; dv_o and S with none (scalar.f90:76-81, default gl = 0); p_o with
// one (multiphase.f90:55).
int fen_gl(int f) { return (f >= FEN_DVO_X && f <= FEN_S_Z) ? 0 : 1; }

// Host elements of a field array with gl ghost layers (2D: gl = 1 arrays have 3 planes).
size_t host_count(fen_ctx* c, int gl) {
  const size_t pl = (c->dim == 3) ? (size_t)c->n[2] + 2 * gl : (size_t)(1 + 2 * gl);
  return (size_t)(c->n[0] + 2 * gl) * (c->n[1] + 2 * gl) * pl;
}

int pre_step(fen_ctx* c, double dt) {
  if (!c->have_dt) return fail(FEN_ERR_STATE, "set_timestep (or set_dt_o) must be called before advancing");
  // dt: previous dt for constant CFL, the step's dt otherwise
  c->sc_host->dt = dt;
  CK(cudaMemcpyAsync(&c->sc->dt, &c->sc_host->dt, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  // NaN status covers the steps of this call only
  CK(cudaMemsetAsync(&c->sc->err, 0, sizeof(int), c->stream));
  CK(cudaMemsetAsync(c->nan_flag, 0, sizeof(int), c->stream));
  if (c->prm.constant_cfl && c->vel_dirty) {
    int r;
    if ((r = launch_checks(c, 0))) return r;
  }
  c->vel_dirty = 0;
  if (deferred_mean(c)) c->phi_offset = 1;
  return 0;
}

void drop_graph(fen_ctx* c) {
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
}

int capture_graph(fen_ctx* c) {
  if (c->graph) return 0;
  cudaGraph_t g;
  const long long before = c->launches;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int r = enqueue_step(c, nullptr);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (r) return r;
  if (e != cudaSuccess) return fail(FEN_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  CK(cudaGraphInstantiate(&c->graph, g, 0));
  CK(cudaGraphDestroy(g));
  c->launches_per_step = c->launches - before;
  c->launches = before;
  return 0;
}

int read_back(fen_ctx* c) {
  CK(cudaMemcpyAsync(c->sc_host, c->sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

}  // namespace

// Error reporting for entry points defined in other translation units.
int fen_internal_fail(int code, const char* msg) { return fail(code, msg); }

// ---------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------
extern "C" {

const char* fen_last_error(void) { return g_err.c_str(); }

int fen_ctx_destroy(fen_ctx* c) {
  if (!c) return 0;
  drop_graph(c);
  double* bufs[] = {c->u, c->v, c->w, c->p, c->phi, c->us, c->vs, c->ws, c->dvo[0], c->dvo[1], c->dvo[2],
                    c->S[0], c->S[1], c->S[2], c->mwn[0], c->mwn[1], c->mwn[2], c->ta, c->tb, c->tc, c->c1,
                    c->fac, c->partial, c->pdiv, c->pvel, c->stage_scratch, c->util};
  for (double* b : bufs) if (b) cudaFree(b);
  float* fb[] = {c->u32, c->v32, c->w32, c->p32, c->u32l, c->v32l, c->w32l, c->p32l, c->phi32, c->d32[0],
                 c->d32[1], c->d32[2], c->dvo32[0], c->dvo32[1], c->dvo32[2], c->S32[0], c->S32[1], c->S32[2],
                 c->dphi32, c->dv32h, c->dv32l, c->d32l[0], c->d32l[1], c->d32l[2], c->dvo32l[0], c->dvo32l[1], c->dvo32l[2]};
  for (float* b : fb) if (b) cudaFree(b);
  if (c->tmp64) cudaFree(c->tmp64);
  for (double* b : {c->rho, c->mu, c->p_o}) if (b) cudaFree(b);
  if (c->conv) cudaFree(c->conv);
  for (auto& I : c->ibm) {
    void* bs[] = {I.idx, I.nidx, I.nn, I.w, I.c0, I.vs, I.fe};
    for (void* b : bs) if (b) cudaFree(b);
  }
  for (int f = 0; f < 5; ++f) for (int q = 0; q < 6; ++q) if (c->bcval[f][q]) cudaFree(c->bcval[f][q]);
  if (c->specC) cudaFree(c->specC);
  if (c->specR) cudaFree(c->specR);
  if (c->inv_lam) cudaFree(c->inv_lam);
  for (void* b : c->twbufs) cudaFree(b);
  if (c->nan_flag) cudaFree(c->nan_flag);
  if (c->sc) cudaFree(c->sc);
  if (c->sc_host) cudaFreeHost(c->sc_host);
  for (double* b : c->adj.ckpt) if (b) cudaFree(b);
  for (double* b : c->adj.inputs) if (b) cudaFree(b);
  if (c->adj.dtab) cudaFree(c->adj.dtab);
  if (c->adj.dslot) cudaFree(c->adj.dslot);
  double* ab[] = {c->adj.uh, c->adj.vh, c->adj.wh, c->adj.ph, c->adj.dou, c->adj.dov, c->adj.dow, c->adj.fh,
                  c->adj.bh, c->adj.ush, c->adj.vsh, c->adj.wsh, c->adj.dhu, c->adj.dhv, c->adj.dhw, c->adj.part};
  for (double* b : ab) if (b) cudaFree(b);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return 0;
}

int fen_ctx_create(const fen_params* P, fen_ctx** out) {
  if (!P || !out) return fail(FEN_ERR_ARG, "null argument");
  *out = nullptr;
  if (P->dim != 2 && P->dim != 3) return fail(FEN_ERR_ARG, "dim must be 2 or 3");
  if (P->nx < 2 || P->ny < 2 || (P->dim == 3 && P->nz < 2)) return fail(FEN_ERR_ARG, "grid sizes must be >= 2");
  if (P->precision != FEN_FP64 && P->precision != FEN_MIXED) return fail(FEN_ERR_ARG, "unknown precision form");
  auto pos = [](double x) { return x > 0.0 && !std::isinf(x); };
  if (!pos(P->lx) || !pos(P->ly) || (P->dim == 3 && !pos(P->lz))) return fail(FEN_ERR_ARG, "domain lengths must be positive");
  if (!pos(P->density) || !(P->viscosity >= 0.0) || std::isinf(P->viscosity))
    return fail(FEN_ERR_ARG, "density must be positive and viscosity non-negative");
  if (P->constant_cfl && !pos(P->cfl)) return fail(FEN_ERR_ARG, "CFL must be positive");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(FEN_ERR_CUDA, "no CUDA device");
  fen_ctx* c = new fen_ctx();
  memset(c->ftype, 0, sizeof(c->ftype));
  memset(c->bcval, 0, sizeof(c->bcval));
  c->prm = *P;
  c->mixed = (P->precision == FEN_MIXED);
  if (P->refine < 0 || P->refine > 1) {
    delete c;
    return fail(FEN_ERR_ARG, "refine must be 0 or 1");
  }
  c->refine = c->mixed ? P->refine : 0;
  c->dim = P->dim;
  c->n[0] = P->nx; c->n[1] = P->ny; c->n[2] = (P->dim == 3) ? P->nz : 1;
  // grid%setup: delta = Lx/float(Nx) (grid.f90:140); per-axis spacing when aniso
  const double delta = P->lx / ffloat(P->nx);
  if (P->aniso) {
    c->d[0] = P->lx / ffloat(P->nx);
    c->d[1] = P->ly / ffloat(P->ny);
    c->d[2] = (P->dim == 3) ? P->lz / ffloat(P->nz) : delta;
    c->iso = (c->d[0] == c->d[1]) && (P->dim == 2 || c->d[0] == c->d[2]);
  } else {
    c->d[0] = c->d[1] = c->d[2] = delta;
    c->iso = 1;
  }
  c->dmin = c->d[0];
  for (int a = 1; a < c->dim; ++a) c->dmin = std::min(c->dmin, c->d[a]);
  for (int f = 0; f < 6; ++f) c->pbc[f] = (f < 2 * c->dim) ? P->bc[f] : FEN_BC_PERIODIC;
  for (int a = 0; a < 3; ++a) c->periodic[a] = (c->pbc[2 * a] == FEN_BC_PERIODIC && c->pbc[2 * a + 1] == FEN_BC_PERIODIC);
  for (int f = 0; f < 2 * c->dim; ++f)
    if ((c->pbc[f] == FEN_BC_PERIODIC) != (c->pbc[f ^ 1] == FEN_BC_PERIODIC)) {
      delete c;
      return fail(FEN_ERR_BC, "a periodic face needs a periodic opposite face");
    }
  // field bc types: u, v, w, p, phi
  const int comp[5] = {1, 2, 3, 0, 0};
  for (int fi = 0; fi < 5; ++fi)
    for (int q = 0; q < 6; ++q) {
      int t = (q < 2 * c->dim) ? field_type(q, c->pbc[q], comp[fi]) : FT_PERIODIC;
      if (t < 0) { delete c; return fail(FEN_ERR_BC, "boundary condition not supported on this face"); }
      c->ftype[fi][q] = t;
    }
  // layout
  Layout& L = c->L;
  L.dim = c->dim;
  L.n0 = c->n[0]; L.n1 = c->n[1]; L.n2 = c->n[2];
  L.sx = ((c->n[0] + 2 + 3) / 4) * 4;
  L.sy = c->n[1] + 2;
  L.sp = (long long)L.sx * L.sy;
  L.off = 3;
  const int planes = (c->dim == 3) ? c->n[2] + 2 : 1;
  L.total = L.off + L.sp * planes + 4;
  L.fastdiv = (L.n0 <= 4096 && L.n1 <= 4096) ? 1 : 0;
  L.mg0 = fft_magic((unsigned)L.n0);
  L.mg1 = fft_magic((unsigned)L.n1);
  int r = 0;
  double** state[] = {&c->u, &c->v, &c->w, &c->p};
  for (double** f : state)
    if ((r = alloc(f, L.total))) { fen_ctx_destroy(c); return r; }
  if (c->mixed) {
    float** fl[] = {&c->u32, &c->v32, &c->w32, &c->p32, &c->u32l, &c->v32l, &c->w32l, &c->p32l, &c->phi32,
                    &c->d32[0], &c->d32[1], &c->d32[2], &c->dvo32[0], &c->dvo32[1], &c->dvo32[2],
                    &c->d32l[0], &c->d32l[1], &c->d32l[2], &c->dvo32l[0], &c->dvo32l[1], &c->dvo32l[2]};
    for (float** f : fl)
      if ((r = alloc(f, L.total))) { fen_ctx_destroy(c); return r; }
    if ((r = alloc(&c->tmp64, L.total))) { fen_ctx_destroy(c); return r; }
    if (c->refine && ((r = alloc(&c->dphi32, L.total)) || (r = alloc(&c->dv32h, L.total)) || (r = alloc(&c->dv32l, L.total)))) {
      fen_ctx_destroy(c);
      return r;
    }
  } else {
    double** fl[] = {&c->phi, &c->us, &c->vs, &c->ws, &c->dvo[0], &c->dvo[1], &c->dvo[2]};
    for (double** f : fl)
      if ((r = alloc(f, L.total))) { fen_ctx_destroy(c); return r; }
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { fen_ctx_destroy(c); return fail(FEN_ERR_CUDA, "stream"); }
  if (cudaMalloc((void**)&c->sc, sizeof(StepScalars)) != cudaSuccess ||
      cudaMallocHost((void**)&c->sc_host, sizeof(StepScalars)) != cudaSuccess) { fen_ctx_destroy(c); return fail(FEN_ERR_NOMEM, "scalars"); }
  memset(c->sc_host, 0, sizeof(StepScalars));
  cudaMemset(c->sc, 0, sizeof(StepScalars));
  c->nred = 152 * FEN_CHECK_CTAS_PER_SM;
  if ((r = alloc(&c->pdiv, c->nred)) || (r = alloc(&c->pvel, c->nred))) { fen_ctx_destroy(c); return r; }
  if (cudaMalloc((void**)&c->nan_flag, sizeof(int)) != cudaSuccess) { fen_ctx_destroy(c); return fail(FEN_ERR_NOMEM, "flag"); }
  cudaMemset(c->nan_flag, 0, sizeof(int));
  if ((r = init_poisson(c))) { fen_ctx_destroy(c); return r; }
  *out = c;
  return 0;
}

// Density, viscosity and old-pressure fields of the variable-property path, allocated on
// first use with FEN's initial values (rho%f = density, mu%f = viscosity, p_o = 0).
int prop_field(fen_ctx* c, int f, double** out) {
  double** slot = (f == FEN_RHO) ? &c->rho : (f == FEN_MU) ? &c->mu : &c->p_o;
  if (!*slot) {
    if (c->mixed) return fail(FEN_ERR_ARG, "the variable-property path runs in FP64 contexts only");
    if (f == FEN_MU && c->dim == 3)
      return fail(FEN_ERR_ARG, "variable viscosity is 2D only (FEN's 3D stress-divergence branch is empty)");
    int r;
    if ((r = alloc(slot, c->L.total))) return r;
    const double v0 = (f == FEN_RHO) ? c->prm.density : (f == FEN_MU) ? c->prm.viscosity : 0.0;
    if (v0 != 0.0) {
      std::vector<double> h((size_t)c->L.total, v0);
      CK(cudaMemcpy(*slot, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    drop_graph(c);
  }
  *out = *slot;
  return 0;
}

int fen_upload_gl(fen_ctx* c, int f, const double* host, int gl) {
  if (!c || !host) return fail(FEN_ERR_ARG, "null argument");
  if (f < FEN_U || f > FEN_P_O || (f == FEN_W && c->dim == 2)) return fail(FEN_ERR_ARG, "bad field id");
  if (gl != 0 && gl != 1) return fail(FEN_ERR_ARG, "ghost level must be 0 or 1");
  double* hrw = const_cast<double*>(host);
  int r;
  if (f >= FEN_RHO) {
    double* d;
    if ((r = prop_field(c, f, &d))) return r;
    if (f == FEN_RHO && !c->var_rho) { c->var_rho = 1; drop_graph(c); }
    if (f == FEN_MU && !c->var_mu) { c->var_mu = 1; drop_graph(c); }
    return relayout<double>(c, d, hrw, 0, gl);
  }
  if (f >= FEN_S_X && f <= FEN_S_Z) {
    // S is used in every component once any is set (dv += S/rhof, navier_stokes.f90:245-255)
    for (int q = 0; q < 3; ++q) {
      if (c->mixed && !c->S32[q] && (r = alloc(&c->S32[q], c->L.total))) return r;
      if (!c->mixed && !c->S[q] && (r = alloc(&c->S[q], c->L.total))) return r;
    }
    if (!c->has_S) { c->has_S = 1; drop_graph(c); }
    return c->mixed ? relayout<float>(c, c->S32[f - FEN_S_X], hrw, 0, gl) : relayout<double>(c, c->S[f - FEN_S_X], hrw, 0, gl);
  }
  if (f >= FEN_DVO_X && f <= FEN_DVO_Z) {
    if (!c->mixed) return relayout<double>(c, c->dvo[f - FEN_DVO_X], hrw, 0, gl);
    // dv_o is a pair in the mixed form: FP64 staging, then split
    if ((r = relayout<double>(c, c->tmp64, hrw, 0, gl))) return r;
    const int grid = std::min(cdiv(c->L.total, 256), 152 * 16);
    k_split<<<grid, 256, 0, c->stream>>>(c->L.total, c->tmp64, c->dvo32[f - FEN_DVO_X], c->dvo32l[f - FEN_DVO_X]);
    c->launches++;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return 0;
  }
  if (f == FEN_PHI) {
    c->phi_offset = 0;
    return c->mixed ? relayout<float>(c, c->phi32, hrw, 0, gl) : relayout<double>(c, c->phi, hrw, 0, gl);
  }
  double* d = (f == FEN_U) ? c->u : (f == FEN_V) ? c->v : (f == FEN_W) ? c->w : c->p;
  if (c->mixed && gl == 0 && (r = pair_convert(c, f, 1))) return r;  // keep the device ghosts
  if ((r = relayout<double>(c, d, hrw, 0, gl))) return r;
  if (c->mixed && (r = pair_convert(c, f, 0))) return r;
  if (f == FEN_U || f == FEN_V || f == FEN_W) c->vel_dirty = 1;
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int fen_download_gl(fen_ctx* c, int f, double* host, int gl) {
  if (!c || !host) return fail(FEN_ERR_ARG, "null argument");
  if (f < FEN_U || f > FEN_P_O || (f == FEN_W && c->dim == 2)) return fail(FEN_ERR_ARG, "bad field id");
  if (gl != 0 && gl != 1) return fail(FEN_ERR_ARG, "ghost level must be 0 or 1");
  if (f >= FEN_RHO) {
    double* d;
    int r;
    if ((r = prop_field(c, f, &d))) return r;
    return relayout<double>(c, d, host, 1, gl);
  }
  if (f >= FEN_S_X && f <= FEN_S_Z) {
    if (!c->has_S) {
      memset(host, 0, host_count(c, gl) * sizeof(double));
      return 0;
    }
    return c->mixed ? relayout<float>(c, c->S32[f - FEN_S_X], host, 1, gl) : relayout<double>(c, c->S[f - FEN_S_X], host, 1, gl);
  }
  if (f >= FEN_DVO_X && f <= FEN_DVO_Z) {
    if (!c->mixed) return relayout<double>(c, c->dvo[f - FEN_DVO_X], host, 1, gl);
    const int grid = std::min(cdiv(c->L.total, 256), 152 * 16);
    k_join<<<grid, 256, 0, c->stream>>>(c->L.total, c->dvo32[f - FEN_DVO_X], c->dvo32l[f - FEN_DVO_X], c->tmp64);
    c->launches++;
    CK(cudaGetLastError());
    return relayout<double>(c, c->tmp64, host, 1, gl);
  }
  if (f == FEN_PHI && c->mixed && c->phi_offset) {
    // the last step left the mean of phi in place: remove it and refill the ghosts
    const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
    const int grid = std::min(cdiv(ncell, 256), 152 * 8);
    k_keep_mean<<<1, 1, 0, c->stream>>>(c->sc, 1);
    if (c->dim == 3) k_mean_subtract<float, 3><<<grid, 256, 0, c->stream>>>(c->L, c->sc, c->phi32);
    else k_mean_subtract<float, 2><<<grid, 256, 0, c->stream>>>(c->L, c->sc, c->phi32);
    c->launches += 2;
    CK(cudaGetLastError());
    float* pf[1] = {c->phi32};
    int ids[1] = {FEN_PHI};
    int r;
    if ((r = ghost<float>(c, 1, pf, ids))) return r;
    c->phi_offset = 0;
  }
  if (f == FEN_PHI) return c->mixed ? relayout<float>(c, c->phi32, host, 1, gl) : relayout<double>(c, c->phi, host, 1, gl);
  double* d = (f == FEN_U) ? c->u : (f == FEN_V) ? c->v : (f == FEN_W) ? c->w : c->p;
  int r;
  if (c->mixed && (r = pair_convert(c, f, 1))) return r;
  return relayout<double>(c, d, host, 1, gl);
}

int fen_upload(fen_ctx* c, int f, const double* host) { return fen_upload_gl(c, f, host, fen_gl(f)); }
int fen_download(fen_ctx* c, int f, double* host) { return fen_download_gl(c, f, host, fen_gl(f)); }

int fen_field_bounds(fen_ctx* c, int f, int* lo, int* hi) {
  if (!c || !lo || !hi) return fail(FEN_ERR_ARG, "null argument");
  if (f < FEN_U || f > FEN_P_O || (f == FEN_W && c->dim == 2)) return fail(FEN_ERR_ARG, "bad field id");
  const int gl = fen_gl(f);
  for (int q = 0; q < 3; ++q) {
    lo[q] = 1 - gl;
    hi[q] = c->n[q] + gl;
  }
  return 0;
}

int fen_update_ghost_nodes(fen_ctx* c, int f) {
  if (!c) return fail(FEN_ERR_ARG, "null argument");
  if (f >= FEN_RHO && f <= FEN_P_O) {  // rho, mu, p_o take p's boundary types
    double* d;
    int r;
    if ((r = prop_field(c, f, &d))) return r;
    double* p[1] = {d};
    int ids[1] = {FEN_P};
    if ((r = ghost<double>(c, 1, p, ids))) return r;
    CK(cudaStreamSynchronize(c->stream));
    return 0;
  }
  if (f < FEN_U || f > FEN_PHI || (f == FEN_W && c->dim == 2)) return fail(FEN_ERR_ARG, "field has no ghost nodes");
  int ids[1] = {f};
  int r;
  if (f == FEN_PHI) {
    if (c->mixed) { float* p[1] = {c->phi32}; r = ghost<float>(c, 1, p, ids); }
    else { double* p[1] = {c->phi}; r = ghost<double>(c, 1, p, ids); }
  } else {
    double* p[1] = {(f == FEN_U) ? c->u : (f == FEN_V) ? c->v : (f == FEN_W) ? c->w : c->p};
    r = c->mixed ? ghost_pairs(c, 1, ids) : ghost<double>(c, 1, p, ids);
  }
  if (r) return r;
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int fen_set_bc_values(fen_ctx* c, int f, int face, const double* vals) {
  if (!c || !vals || f < FEN_U || f > FEN_PHI || face < 0 || face >= 2 * c->dim) return fail(FEN_ERR_ARG, "bad argument");
  const int nxg = c->n[0] + 2, nyg = c->n[1] + 2, nzg = (c->dim == 3) ? c->n[2] + 2 : 3;
  int na, nb;
  if (face < 2) { na = nyg; nb = nzg; }
  else if (face < 4) { na = nxg; nb = nzg; }
  else { na = nxg; nb = nyg; }
  // device copy: 3D keeps the whole face; 2D keeps the k = 1 column of the (a, 0:2) array
  const int nbd = (c->dim == 3 || face >= 4) ? nb : 1;
  const double* src = vals + ((c->dim == 2 && face < 4) ? (size_t)na : 0);
  if (!c->bcval[f][face]) {
    // a new device array: the captured step must be rebuilt to read it
    int r;
    if ((r = alloc(&c->bcval[f][face], (long long)na * nbd))) return r;
    drop_graph(c);
  }
  // stream-ordered after the previous step (the graph reads these values in place)
  CK(cudaMemcpyAsync(c->bcval[f][face], src, (size_t)na * nbd * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int fen_set_bc_type(fen_ctx* c, int f, int face, int t) {
  if (!c || f < FEN_U || f > FEN_PHI || face < 0 || face >= 2 * c->dim || t < 0 || t > 2)
    return fail(FEN_ERR_ARG, "bad argument");
  c->ftype[f][face] = t;
  drop_graph(c);
  return 0;
}

int fen_set_timestep(fen_ctx* c, double U, double* dt) {
  if (!c || !dt) return fail(FEN_ERR_ARG, "null argument");
  if (!(U >= 0.0)) return fail(FEN_ERR_ARG, "reference velocity U must be >= 0");
  // set_timestep (navier_stokes.f90:641-664)
  const double dl = c->dmin;
  const double dt_conv = c->prm.cfl * dl / U;
  double dt_visc = 0.125 * dl * dl * c->prm.density / c->prm.viscosity;
  if (c->dim == 3) dt_visc = (1.0 / 6.0) * dl * dl * c->prm.density / c->prm.viscosity;
  *dt = std::min(dt_conv, dt_visc);
  c->sc_host->dt = *dt;
  c->sc_host->dt_o = *dt;
  c->sc_host->dt_visc = dt_visc;
  c->sc_host->dt_conv = dt_conv;
  CK(cudaMemcpyAsync(c->sc, c->sc_host, sizeof(StepScalars), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->have_dt = 1;
  return 0;
}

int fen_set_dt_o(fen_ctx* c, double dt_o) {
  if (!c) return fail(FEN_ERR_ARG, "null argument");
  if (!(dt_o > 0.0) || std::isinf(dt_o)) return fail(FEN_ERR_ARG, "dt_o must be positive and finite");
  CK(cudaStreamSynchronize(c->stream));
  // keep dt_visc consistent with set_timestep's formula
  const double dl = c->dmin;
  double dt_visc = 0.125 * dl * dl * c->prm.density / c->prm.viscosity;
  if (c->dim == 3) dt_visc = (1.0 / 6.0) * dl * dl * c->prm.density / c->prm.viscosity;
  c->sc_host->dt_o = dt_o;
  if (!c->have_dt) { c->sc_host->dt_visc = dt_visc; c->sc_host->dt = dt_o; }
  CK(cudaMemcpyAsync(c->sc, c->sc_host, sizeof(StepScalars), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->have_dt = 1;
  return 0;
}

int fen_advance_solution(fen_ctx* c, int step, double* dt) {
  (void)step;
  if (!c || !dt) return fail(FEN_ERR_ARG, "null argument");
  if (!(*dt > 0.0) || std::isinf(*dt)) return fail(FEN_ERR_ARG, "dt must be positive and finite");
  int r;
  if ((r = pre_step(c, *dt))) return r;
  if ((r = capture_graph(c))) return r;
  CK(cudaGraphLaunch(c->graph, c->stream));
  c->launches += c->launches_per_step;
  if ((r = read_back(c))) return r;
  *dt = c->sc_host->dt;
  if (c->sc_host->err) return fail(FEN_ERR_NAN, "NaN in the velocity field");
  return 0;
}

int fen_advance_n(fen_ctx* c, int nsteps, double* dt) {
  if (!c || !dt || nsteps < 0) return fail(FEN_ERR_ARG, "bad argument");
  if (!(*dt > 0.0) || std::isinf(*dt)) return fail(FEN_ERR_ARG, "dt must be positive and finite");
  int r;
  if ((r = pre_step(c, *dt))) return r;
  if ((r = capture_graph(c))) return r;
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(c->graph, c->stream));
  c->launches += c->launches_per_step * nsteps;
  if ((r = read_back(c))) return r;
  *dt = c->sc_host->dt;
  if (c->sc_host->err) return fail(FEN_ERR_NAN, "NaN in the velocity field");
  return 0;
}

int fen_get_status(fen_ctx* c, fen_status* o) {
  if (!c || !o) return fail(FEN_ERR_ARG, "null argument");
  int r;
  if ((r = read_back(c))) return r;
  o->dt = c->sc_host->dt;
  o->dt_o = c->sc_host->dt_o;
  o->maxdiv = c->sc_host->maxdiv;
  o->maxcfl = c->sc_host->maxCFL;
  o->maxvel = c->sc_host->maxvel;
  o->dt_visc = c->sc_host->dt_visc;
  o->nan_detected = c->sc_host->err;
  o->poisson_solver = c->solver;
  return 0;
}

int fen_solve_poisson(fen_ctx* c) {
  if (!c) return fail(FEN_ERR_ARG, "null argument");
  int r;
  if ((r = run_poisson(c, true))) return r;
  c->phi_offset = 0;  // the solve removes the mean itself
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int fen_divergence(fen_ctx* c, double* out) {
  if (!c || !out) return fail(FEN_ERR_ARG, "null argument");
  // divergence_of_vector of the FP64 velocity (fields.f90:120-153), evaluated on the host
  // from a download (a test and post-processing aid, not on the step path)
  std::vector<double> hu((size_t)(c->n[0] + 2) * (c->n[1] + 2) * host_planes(c));
  std::vector<double> hv(hu.size()), hw(hu.size());
  int r;
  if ((r = fen_download(c, FEN_U, hu.data())) || (r = fen_download(c, FEN_V, hv.data()))) return r;
  if (c->dim == 3 && (r = fen_download(c, FEN_W, hw.data()))) return r;
  const int nxg = c->n[0] + 2, nyg = c->n[1] + 2;
  auto I = [&](int i, int j, int k) { return (size_t)i + (size_t)nxg * ((size_t)j + (size_t)nyg * k); };
  size_t t = 0;
  const int K = (c->dim == 3) ? c->n[2] : 1;
  for (int k = 1; k <= K; ++k)
    for (int j = 1; j <= c->n[1]; ++j)
      for (int i = 1; i <= c->n[0]; ++i) {
        double d;
        if (c->iso) {
          const double id = 1.0 / c->d[0];
          d = (hu[I(i, j, k)] - hu[I(i - 1, j, k)]) * id + (hv[I(i, j, k)] - hv[I(i, j - 1, k)]) * id;
          if (c->dim == 3) d = d + (hw[I(i, j, k)] - hw[I(i, j, k - 1)]) * id;
        } else {
          d = (hu[I(i, j, k)] - hu[I(i - 1, j, k)]) * (1.0 / c->d[0]) + (hv[I(i, j, k)] - hv[I(i, j - 1, k)]) * (1.0 / c->d[1]);
          if (c->dim == 3) d = d + (hw[I(i, j, k)] - hw[I(i, j, k - 1)]) * (1.0 / c->d[2]);
        }
        out[t++] = d;
      }
  return 0;
}

int fen_explicit_terms(fen_ctx* c, double* out) {
  if (!c || !out) return fail(FEN_ERR_ARG, "null argument");
  // Run the predictor with A = 1, B = 0, dt = 1 and read dv_o back: dv_o <- dv is exactly
  // compute_explicit_terms (navier_stokes.f90:217-257).  dv_o is restored afterwards.
  int r;
  const long long tot = c->L.total;
  const size_t es = c->mixed ? sizeof(float) : sizeof(double);
  std::vector<void*> save(3, nullptr);
  for (int q = 0; q < c->dim; ++q) {
    CK(cudaMalloc(&save[q], 2 * tot * es));
    void* src = c->mixed ? (void*)c->dvo32[q] : (void*)c->dvo[q];
    CK(cudaMemcpyAsync(save[q], src, tot * es, cudaMemcpyDeviceToDevice, c->stream));
    if (c->mixed)
      CK(cudaMemcpyAsync((char*)save[q] + tot * es, c->dvo32l[q], tot * es, cudaMemcpyDeviceToDevice, c->stream));
  }
  StepScalars s = *c->sc_host;
  s.A = 1.0; s.B = 0.0; s.dt = 1.0;
  s.Ap[0] = 1.0f; s.Ap[1] = 0.0f; s.Bp[0] = 0.0f; s.Bp[1] = 0.0f; s.dtp[0] = 1.0f; s.dtp[1] = 0.0f;
  StepScalars* dsc;
  CK(cudaMalloc((void**)&dsc, sizeof(StepScalars)));
  CK(cudaMemcpyAsync(dsc, &s, sizeof(s), cudaMemcpyHostToDevice, c->stream));
  if ((r = launch_predictor(c, dsc))) return r;
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  for (int q = 0; q < c->dim; ++q) {
    if ((r = fen_download_gl(c, FEN_DVO_X + q, out + (size_t)q * ncell, 0))) return r;
    void* dst = c->mixed ? (void*)c->dvo32[q] : (void*)c->dvo[q];
    CK(cudaMemcpyAsync(dst, save[q], tot * es, cudaMemcpyDeviceToDevice, c->stream));
    if (c->mixed)
      CK(cudaMemcpyAsync(c->dvo32l[q], (char*)save[q] + tot * es, tot * es, cudaMemcpyDeviceToDevice, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  for (int q = 0; q < c->dim; ++q) cudaFree(save[q]);
  cudaFree(dsc);
  return 0;
}

// ---- fields_mod generics and add_advection (fields.f90:13-26; navier_stokes.f90:261-353) ----
namespace {
// Scratch of the field operators: three interior arrays and one ghosted FP64 field.
int util_scratch(fen_ctx* c, double** out3, double** field) {
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  if (!c->util) {
    int r;
    if ((r = alloc(&c->util, 3 * ncell + c->L.total))) return r;
  }
  *out3 = c->util;
  *field = c->util + 3 * ncell;
  return 0;
}

// Device FP64 copy of a ghosted scalar or velocity field (pairs joined in the mixed form).
int fp64_field(fen_ctx* c, int f, double* spare, const double** out) {
  int r;
  switch (f) {
    case FEN_U: case FEN_V: case FEN_W: case FEN_P:
      if (c->mixed && (r = pair_convert(c, f, 1))) return r;
      *out = (f == FEN_U) ? c->u : (f == FEN_V) ? c->v : (f == FEN_W) ? c->w : c->p;
      return 0;
    case FEN_PHI:
      if (!c->mixed) { *out = c->phi; return 0; }
      k_widen_field<<<std::min(cdiv(c->L.total, 256), 152 * 16), 256, 0, c->stream>>>(c->L.total, c->phi32, spare);
      c->launches++;
      CK(cudaGetLastError());
      *out = spare;
      return 0;
    case FEN_RHO: case FEN_MU: case FEN_P_O: {
      double* d;
      if ((r = prop_field(c, f, &d))) return r;
      *out = d;
      return 0;
    }
  }
  return fail(FEN_ERR_ARG, "field has no ghost nodes (gradient and laplacian need a ghosted field)");
}

FieldOpArgs field_args(fen_ctx* c) {
  FieldOpArgs a;
  memset(&a, 0, sizeof(a));
  for (int q = 0; q < 3; ++q) {
    a.id[q] = 1.0 / c->d[q];
    a.id2[q] = 1.0 / (c->d[q] * c->d[q]);
  }
  a.iso = c->iso;
  return a;
}

int launch_field_op(fen_ctx* c, const FieldOpArgs& a) {
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  const int grid = std::min(cdiv(ncell, 256), 152 * 16);
  if (c->dim == 3) k_field_op<3><<<grid, 256, 0, c->stream>>>(c->L, a);
  else k_field_op<2><<<grid, 256, 0, c->stream>>>(c->L, a);
  c->launches++;
  CK(cudaGetLastError());
  return 0;
}
}  // namespace

int fen_gradient(fen_ctx* c, int f, double* gx, double* gy, double* gz) {
  if (!c || !gx || !gy || (c->dim == 3 && !gz)) return fail(FEN_ERR_ARG, "null argument");
  if (f == FEN_U || f == FEN_V || f == FEN_W) return fail(FEN_ERR_ARG, "gradient of a scalar field (p, phi, rho, mu, p_o)");
  double *o, *spare;
  const double* s;
  int r;
  if ((r = util_scratch(c, &o, &spare)) || (r = fp64_field(c, f, spare, &s))) return r;
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  FieldOpArgs a = field_args(c);
  a.op = FOP_GRADIENT;
  a.s = s;
  a.o0 = o; a.o1 = o + ncell; a.o2 = o + 2 * ncell;
  if ((r = launch_field_op(c, a))) return r;
  double* dst[3] = {gx, gy, gz};
  for (int q = 0; q < c->dim; ++q)
    CK(cudaMemcpyAsync(dst[q], o + q * ncell, ncell * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int fen_laplacian(fen_ctx* c, int f, double* out) {
  if (!c || !out) return fail(FEN_ERR_ARG, "null argument");
  double *o, *spare;
  const double* s;
  int r;
  if ((r = util_scratch(c, &o, &spare)) || (r = fp64_field(c, f, spare, &s))) return r;
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  FieldOpArgs a = field_args(c);
  a.op = FOP_LAPLACIAN;
  a.s = s;
  a.comp = (f == FEN_W) ? 2 : 0;
  a.o0 = o;
  if ((r = launch_field_op(c, a))) return r;
  CK(cudaMemcpyAsync(out, o, ncell * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

int fen_add_advection(fen_ctx* c, double* rx, double* ry, double* rz) {
  if (!c || !rx || !ry || (c->dim == 3 && !rz)) return fail(FEN_ERR_ARG, "null argument");
  double *o, *spare;
  const double *u, *v, *w = nullptr;
  int r;
  if ((r = util_scratch(c, &o, &spare)) || (r = fp64_field(c, FEN_U, spare, &u)) || (r = fp64_field(c, FEN_V, spare, &v)))
    return r;
  if (c->dim == 3 && (r = fp64_field(c, FEN_W, spare, &w))) return r;
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  double* rr[3] = {rx, ry, rz};
  for (int q = 0; q < c->dim; ++q)
    CK(cudaMemcpyAsync(o + q * ncell, rr[q], ncell * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  FieldOpArgs a = field_args(c);
  a.op = FOP_ADVECTION;
  a.u = u; a.v = v; a.w = w;
  a.o0 = o; a.o1 = o + ncell; a.o2 = o + 2 * ncell;
  if ((r = launch_field_op(c, a))) return r;
  for (int q = 0; q < c->dim; ++q)
    CK(cudaMemcpyAsync(rr[q], o + q * ncell, ncell * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

// ---- checkpoint / restart (solver.f90:103-329) ----------------------------------------
namespace {
// Interior of one field (x fastest), FEN's f(lo(1):hi(1), lo(2):hi(2), lo(3):hi(3)).
int interior_get(fen_ctx* c, int f, std::vector<double>& out) {
  out.resize(host_count(c, 0));
  return fen_download_gl(c, f, out.data(), 0);
}

int interior_set(fen_ctx* c, int f, const double* in) { return fen_upload_gl(c, f, in, 0); }

// save_state / load_state field order (solver.f90:195-208, 277-292).
std::vector<int> state_order(fen_ctx* c) {
  std::vector<int> o = {FEN_P, FEN_U, FEN_V, FEN_DVO_X, FEN_DVO_Y};
  if (c->dim == 3) { o.push_back(FEN_W); o.push_back(FEN_DVO_Z); }
  return o;
}
}  // namespace

int fen_save_state(fen_ctx* c, const char* path) {
  if (!c || !path) return fail(FEN_ERR_ARG, "null argument");
  FILE* fp = fopen(path, "wb");
  if (!fp) return fail(FEN_ERR_ARG, std::string("cannot open ") + path + ": " + strerror(errno));
  std::vector<double> buf;
  for (int f : state_order(c)) {
    int r;
    if ((r = interior_get(c, f, buf))) { fclose(fp); return r; }
    if (fwrite(buf.data(), sizeof(double), buf.size(), fp) != buf.size()) { fclose(fp); return fail(FEN_ERR_ARG, "short write"); }
  }
  fclose(fp);
  return 0;
}

int fen_load_state(fen_ctx* c, const char* path) {
  if (!c || !path) return fail(FEN_ERR_ARG, "null argument");
  FILE* fp = fopen(path, "rb");
  if (!fp) return fail(FEN_ERR_ARG, std::string("cannot open ") + path + ": " + strerror(errno));
  const size_t cnt = (size_t)c->n[0] * c->n[1] * ((c->dim == 3) ? c->n[2] : 1);
  std::vector<double> buf(cnt);
  for (int f : state_order(c)) {
    if (fread(buf.data(), sizeof(double), cnt, fp) != cnt) { fclose(fp); return fail(FEN_ERR_ARG, "state file too short"); }
    int r;
    if ((r = interior_set(c, f, buf.data()))) { fclose(fp); return r; }
  }
  fclose(fp);
  // ghost nodes of p and v (solver.f90:293-294)
  int r;
  if ((r = fen_update_ghost_nodes(c, FEN_P)) || (r = fen_update_ghost_nodes(c, FEN_U)) ||
      (r = fen_update_ghost_nodes(c, FEN_V)))
    return r;
  if (c->dim == 3 && (r = fen_update_ghost_nodes(c, FEN_W))) return r;
  return 0;
}

// save_state / load_state of FEN's multiphase build (solver.f90:203-208, 296-304): after the
// fields above come vof (the caller's array), rho, mu and p_o.
int fen_save_state_mf(fen_ctx* c, const char* path, const double* vof) {
  if (!c || !path || !vof) return fail(FEN_ERR_ARG, "null argument");
  if (c->mixed) return fail(FEN_ERR_ARG, "the variable-property path runs in FP64 contexts only");
  int r;
  if ((r = fen_save_state(c, path))) return r;
  FILE* fp = fopen(path, "ab");
  if (!fp) return fail(FEN_ERR_ARG, std::string("cannot open ") + path + ": " + strerror(errno));
  const size_t cnt = host_count(c, 0);
  std::vector<double> buf(cnt);
  bool ok = fwrite(vof, sizeof(double), cnt, fp) == cnt;
  for (int f : {FEN_RHO, FEN_MU, FEN_P_O}) {
    if (!ok) break;
    if (f == FEN_MU && c->dim == 3) {
      // FEN's 3D step has no variable-viscosity branch: mu is the constant viscosity
      std::fill(buf.begin(), buf.end(), c->prm.viscosity);
    } else if ((r = interior_get(c, f, buf))) {
      fclose(fp);
      return r;
    }
    ok = fwrite(buf.data(), sizeof(double), cnt, fp) == cnt;
  }
  fclose(fp);
  return ok ? 0 : fail(FEN_ERR_ARG, "short write");
}

int fen_load_state_mf(fen_ctx* c, const char* path, double* vof) {
  if (!c || !path || !vof) return fail(FEN_ERR_ARG, "null argument");
  if (c->mixed) return fail(FEN_ERR_ARG, "the variable-property path runs in FP64 contexts only");
  int r;
  if ((r = fen_load_state(c, path))) return r;
  FILE* fp = fopen(path, "rb");
  if (!fp) return fail(FEN_ERR_ARG, std::string("cannot open ") + path + ": " + strerror(errno));
  const size_t cnt = host_count(c, 0);
  const long skip = (long)(cnt * sizeof(double) * state_order(c).size());
  std::vector<double> buf(cnt);
  bool ok = fseek(fp, skip, SEEK_SET) == 0 && fread(vof, sizeof(double), cnt, fp) == cnt;
  for (int f : {FEN_RHO, FEN_MU, FEN_P_O}) {
    if (!ok) break;
    ok = fread(buf.data(), sizeof(double), cnt, fp) == cnt;
    if (!ok || (f == FEN_MU && c->dim == 3)) continue;
    if ((r = interior_set(c, f, buf.data())) || (r = fen_update_ghost_nodes(c, f))) {
      fclose(fp);
      return r;
    }
  }
  fclose(fp);
  return ok ? 0 : fail(FEN_ERR_ARG, "state file too short for the multiphase fields");
}

int fen_save_fields(fen_ctx* c, const char* dir, int step) {
  if (!c || !dir) return fail(FEN_ERR_ARG, "null argument");
  char sn[16];
  snprintf(sn, sizeof(sn), "%07d", step);
  const int nxg = c->n[0] + 2, nyg = c->n[1] + 2;
  const int K = (c->dim == 3) ? c->n[2] : 1;
  std::vector<double> h((size_t)nxg * nyg * host_planes(c)), out((size_t)c->n[0] * c->n[1] * K);
  const char* names[4] = {"vx_", "vy_", "vz_", "p_"};
  const int fids[4] = {FEN_U, FEN_V, FEN_W, FEN_P};
  const long long so[3] = {1, nxg, (long long)nxg * nyg};
  for (int q = 0; q < 4; ++q) {
    if (q == 2 && c->dim == 2) continue;
    int r;
    if ((r = fen_download(c, fids[q], h.data()))) return r;
    size_t t = 0;
    for (int k = 1; k <= K; ++k)
      for (int j = 1; j <= c->n[1]; ++j)
        for (int i = 1; i <= c->n[0]; ++i) {
          const size_t ci = (size_t)i + (size_t)nxg * ((size_t)j + (size_t)nyg * k);
          // face_to_center (fields.f90:210-252) for the velocity components
          out[t++] = (q < 3) ? 0.5 * (h[ci] + h[ci - so[q]]) : h[ci];
        }
    const std::string path = std::string(dir) + "/" + names[q] + sn + ".raw";
    FILE* fp = fopen(path.c_str(), "wb");
    if (!fp) return fail(FEN_ERR_ARG, "cannot open " + path);
    const size_t wr = fwrite(out.data(), sizeof(double), out.size(), fp);
    fclose(fp);
    if (wr != out.size()) return fail(FEN_ERR_ARG, "short write");
  }
  return 0;
}

// ---- discrete adjoint (fen_adjoint.cuh) ------------------------------------------------
namespace {
constexpr int kAdjParts = 152 * 4;  // CTAs of the adjoint mean reduction

int adj_copy(fen_ctx* c, double* dst, const double* src) {
  CK(cudaMemcpyAsync(dst, src, c->L.total * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  return 0;
}

// The state a checkpoint holds: u, v, [w,] p, dv_o.
std::vector<double*> adj_state(fen_ctx* c) {
  if (c->dim == 3) return {c->u, c->v, c->w, c->p, c->dvo[0], c->dvo[1], c->dvo[2]};
  return {c->u, c->v, c->p, c->dvo[0], c->dvo[1]};
}

int adj_save(fen_ctx* c, int q) {
  const auto src = adj_state(c);
  for (size_t f = 0; f < src.size(); ++f) {
    int r;
    if ((r = adj_copy(c, c->adj.ckpt[c->adj.nf * q + f], src[f]))) return r;
  }
  return 0;
}

int adj_restore(fen_ctx* c, int q) {
  const auto dst = adj_state(c);
  for (size_t f = 0; f < dst.size(); ++f) {
    int r;
    if ((r = adj_copy(c, dst[f], c->adj.ckpt[c->adj.nf * q + f]))) return r;
  }
  return 0;
}

// Walls in y (pn, pnp), else periodic on every axis.
bool adj_walls(const fen_ctx* c) { return c->solver == S_PN || c->solver == S_PNP; }

// Ghosts of adjoint fields: periodic copies, zeros across the walls.
int adj_ghost(fen_ctx* c, std::initializer_list<double*> fs) {
  const int wall = adj_walls(c) ? 1 : 0;
  for (double* f : fs) {
    if (!f) continue;
    for (int ax = 0; ax < c->dim; ++ax) {
      const long long n = 2LL * ((ax == 0) ? c->n[1] + 2 : c->n[0] + 2) * (c->dim == 3 ? ((ax == 2) ? c->n[1] + 2 : c->n[2] + 2) : 1);
      const int g = std::min(cdiv(n, 256), 152 * 8);
      const int zero = (ax == 1) ? wall : 0;
      if (c->dim == 3) k_adj_ghost<3><<<g, 256, 0, c->stream>>>(c->L, f, ax, zero);
      else k_adj_ghost<2><<<g, 256, 0, c->stream>>>(c->L, f, ax, zero);
      c->launches++;
    }
  }
  CK(cudaGetLastError());
  return 0;
}

AdjScales adj_scales(const fen_ctx* c) {
  AdjScales q;
  for (int a = 0; a < 3; ++a) {
    q.id[a] = 1.0 / c->d[a];
    q.id2[a] = 1.0 / (c->d[a] * c->d[a]);
  }
  return q;
}

// One adjoint step with the stored forward input velocity (u, v, w) of that step, or, when
// in.tab is set, the entry *in.slot of the table of stored inputs.
int adj_step(fen_ctx* c, const double* u, const double* v, const double* w, AdjIn in) {
  auto& A = c->adj;
  int r;
  const long long ncell = (long long)c->n[0] * c->n[1] * c->n[2];
  const int grid = std::min(cdiv(ncell, 256), 152 * 16);
  const AdjScales q = adj_scales(c);
  const double rhof = rhof_of(c), rho = c->prm.density, dt = A.dt;
  const double Acoef = 1.0 + 0.5 * dt / c->sc_host->dt_o, Bcoef = -0.5 * dt / c->sc_host->dt_o;
  const int wall = adj_walls(c) ? 1 : 0;
  const bool d3 = (c->dim == 3);
#define ADJ_LAUNCH(kern, ...) \
  do { if (d3) kern<3><<<grid, 256, 0, c->stream>>>(__VA_ARGS__); else kern<2><<<grid, 256, 0, c->stream>>>(__VA_ARGS__); c->launches++; } while (0)
  // phi^ = p'^ + dt/rhof D v'^
  if ((r = adj_ghost(c, {A.uh, A.vh, d3 ? A.wh : nullptr}))) return r;
  ADJ_LAUNCH(k_adj_div, c->L, A.ph, A.uh, A.vh, A.wh, dt / rhof, q, A.fh);
  if (wall) {
    // b^ = P (phi^ - <phi^>): the walls' solve is symmetric on mean-free right-hand sides
    const int gp = kAdjParts;
    if (d3) k_adj_sum<3><<<gp, 256, 0, c->stream>>>(c->L, A.fh, A.part);
    else k_adj_sum<2><<<gp, 256, 0, c->stream>>>(c->L, A.fh, A.part);
    k_mean_reduce<<<1, 1024, 0, c->stream>>>(A.part, gp, (double)ncell, c->sc);
    if (d3) k_mean_subtract<double, 3><<<grid, 256, 0, c->stream>>>(c->L, c->sc, A.fh);
    else k_mean_subtract<double, 2><<<grid, 256, 0, c->stream>>>(c->L, c->sc, A.fh);
    c->launches += 3;
  }
  // b^ = P phi^ (the forward's Poisson plan, loaded from phi^, written to b^)
  for (size_t s = 0; s < c->stages.size(); ++s)
    if ((r = launch_stage(c, c->stages[s], s == 0, A.fh, A.bh))) return r;
  if (c->needs_mean) {
    const int g2 = std::min(cdiv(ncell, 256), 152 * 8);
    k_mean_reduce<<<1, 1024, 0, c->stream>>>(c->partial, c->npartial, c->mean_div, c->sc);
    if (d3) k_mean_subtract<double, 3><<<g2, 256, 0, c->stream>>>(c->L, c->sc, A.bh);
    else k_mean_subtract<double, 2><<<g2, 256, 0, c->stream>>>(c->L, c->sc, A.bh);
    c->launches += 2;
  }
  if ((r = adj_ghost(c, {A.bh}))) return r;
  // v*^ = E^T (v'^ - rho/dt G b^)
  ADJ_LAUNCH(k_adj_grad, c->L, A.uh, A.vh, A.wh, A.bh, rho / dt, q, wall, A.ush, A.vsh, A.wsh);
  // p^ = p'^ + dt/rhof D v*^
  if ((r = adj_ghost(c, {A.ush, A.vsh, d3 ? A.wsh : nullptr}))) return r;
  ADJ_LAUNCH(k_adj_div, c->L, A.ph, A.ush, A.vsh, A.wsh, dt / rhof, q, A.ph);
  // dv^ = dv_o'^ + dt A v*^, dv_o^ = dt B v*^
  ADJ_LAUNCH(k_adj_dv, c->L, A.ush, A.vsh, A.wsh, A.dou, A.dov, A.dow, dt * Acoef, dt * Bcoef, A.dhu, A.dhv, A.dhw);
  // v^ = v*^ + E^T (N'^T dv^ + mu/rhof L dv^)
  if ((r = adj_ghost(c, {A.dhu, A.dhv, d3 ? A.dhw : nullptr}))) return r;
  ADJ_LAUNCH(k_adj_state, c->L, in, u, v, w, A.ush, A.vsh, A.wsh, A.dhu, A.dhv, A.dhw, q, c->prm.viscosity / rhof, wall,
             A.uh, A.vh, A.wh);
#undef ADJ_LAUNCH
  CK(cudaGetLastError());
  return 0;
}
}  // namespace

int fen_adjoint_setup(fen_ctx* c, int nsteps, int every) {
  if (!c || nsteps < 1 || every < 1) return fail(FEN_ERR_ARG, "bad argument");
  const bool solver_ok = c->solver == S_PP || c->solver == S_PPP || c->solver == S_PN || c->solver == S_PNP;
  if (c->mixed || !solver_ok || c->prm.constant_cfl || c->has_S || var_path(c))
    return fail(FEN_ERR_ARG,
                "the adjoint covers FP64 runs with fixed dt and no source field, periodic or with walls in y only "
                "(solvers pp, ppp, pn, pnp)");
  // the adjoint folds the ghosts of 'Wall' faces (reflected tangential, overwritten normal)
  if (adj_walls(c) && (c->pbc[FEN_BOTTOM] != FEN_BC_WALL || c->pbc[FEN_TOP] != FEN_BC_WALL))
    return fail(FEN_ERR_ARG, "the adjoint's walls in y must be 'Wall' faces");
  auto& A = c->adj;
  for (double* b : A.ckpt) if (b) cudaFree(b);
  for (double* b : A.inputs) if (b) cudaFree(b);
  A.ckpt.clear();
  A.inputs.clear();
  A.nsteps = nsteps;
  A.every = std::min(every, nsteps);
  A.nckpt = (nsteps + A.every - 1) / A.every;
  A.nf = (c->dim == 3) ? 7 : 5;
  A.nv = c->dim;
  int r;
  A.ckpt.assign((size_t)A.nf * (A.nckpt + 1), nullptr);
  for (auto& b : A.ckpt) if ((r = alloc(&b, c->L.total))) return r;
  A.inputs.assign((size_t)A.nv * A.every, nullptr);
  for (auto& b : A.inputs) if ((r = alloc(&b, c->L.total))) return r;
  if (A.dtab) cudaFree(A.dtab);
  if (A.dslot) cudaFree(A.dslot);
  A.dtab = nullptr;
  A.dslot = nullptr;
  CK(cudaMalloc(&A.dtab, A.inputs.size() * sizeof(double*)));
  CK(cudaMalloc(&A.dslot, sizeof(int)));
  CK(cudaMemcpy(A.dtab, A.inputs.data(), A.inputs.size() * sizeof(double*), cudaMemcpyHostToDevice));
  double** ab[] = {&A.uh, &A.vh, &A.wh, &A.ph, &A.dou, &A.dov, &A.dow, &A.fh, &A.bh, &A.ush, &A.vsh, &A.wsh,
                   &A.dhu, &A.dhv, &A.dhw};
  for (double** b : ab)
    if (!*b && (r = alloc(b, c->L.total))) return r;
  if (!A.part && (r = alloc(&A.part, kAdjParts))) return r;
  A.ready = false;
  return 0;
}

int fen_adjoint_forward(fen_ctx* c, double dt) {
  if (!c || c->adj.nsteps < 1) return fail(FEN_ERR_STATE, "fen_adjoint_setup first");
  auto& A = c->adj;
  // the adjoint applies one (A, B) pair to every step, which holds when dt_o == dt
  if (!(dt > 0.0) || c->sc_host->dt_o != dt) return fail(FEN_ERR_ARG, "the adjoint rollout needs dt_o == dt (fen_set_dt_o)");
  int r;
  if ((r = pre_step(c, dt))) return r;
  if ((r = capture_graph(c))) return r;
  A.dt = dt;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, c->stream));
  for (int s = 0; s < A.nsteps; ++s) {
    if (s % A.every == 0 && (r = adj_save(c, s / A.every))) return r;
    CK(cudaGraphLaunch(c->graph, c->stream));
  }
  c->launches += c->launches_per_step * A.nsteps;
  if ((r = adj_save(c, A.nckpt))) return r;  // final state, restored after the backward sweep
  CK(cudaEventRecord(e1, c->stream));
  CK(cudaEventSynchronize(e1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  A.fwd_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if ((r = read_back(c))) return r;
  if (c->sc_host->err) return fail(FEN_ERR_NAN, "NaN in the velocity field");
  A.ready = true;
  return 0;
}

int fen_adjoint_backward3(fen_ctx* c, const double* lam_u, const double* lam_v, const double* lam_w, double* g_u,
                          double* g_v, double* g_w, double* ms) {
  if (!c || !lam_u || !lam_v || !g_u || !g_v || (c->dim == 3 && (!lam_w || !g_w))) return fail(FEN_ERR_ARG, "null argument");
  auto& A = c->adj;
  if (!A.ready) return fail(FEN_ERR_STATE, "fen_adjoint_forward first");
  int r;
  const bool d3 = (c->dim == 3);
  // adjoint of the final state: (lam_u, lam_v, lam_w), p^ = 0, dv_o^ = 0
  if ((r = relayout<double>(c, A.uh, const_cast<double*>(lam_u), 0, 1)) ||
      (r = relayout<double>(c, A.vh, const_cast<double*>(lam_v), 0, 1)) ||
      (d3 && (r = relayout<double>(c, A.wh, const_cast<double*>(lam_w), 0, 1))))
    return r;
  for (double* f : {A.ph, A.dou, A.dov, A.dow}) CK(cudaMemsetAsync(f, 0, c->L.total * sizeof(double), c->stream));
  if (adj_walls(c)) {
    // the upper wall face of v is overwritten by the boundary value: no sensitivity
    const long long nf = (long long)c->n[0] * (d3 ? c->n[2] : 1);
    if (d3) k_adj_wall_face<3><<<cdiv(nf, 256), 256, 0, c->stream>>>(c->L, A.vh);
    else k_adj_wall_face<2><<<cdiv(nf, 256), 256, 0, c->stream>>>(c->L, A.vh);
    c->launches++;
  }
  // the adjoint step as one graph (a step of small grids is a few dozen short launches): its
  // forward input comes from the entry *dslot of the stored inputs, stepped down per replay
  cudaGraphExec_t ag = nullptr;
  long long per_adj = 0;
  {
    cudaGraph_t g;
    const long long before = c->launches;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    r = adj_step(c, nullptr, nullptr, nullptr, AdjIn{A.dtab, A.dslot, A.nv});
    if (!r) {
      k_adj_slot<<<1, 32, 0, c->stream>>>(A.dslot, -1);
      c->launches++;
    }
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (r) return r;
    if (e != cudaSuccess) return fail(FEN_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    CK(cudaGraphInstantiate(&ag, g, 0));
    CK(cudaGraphDestroy(g));
    per_adj = c->launches - before;
    c->launches = before;
  }
  // ghost entries of the seed carry no sensitivity: the first adjoint step overwrites them
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, c->stream));
  for (int seg = A.nckpt - 1; seg >= 0 && !r; --seg) {
    const int s0 = seg * A.every, s1 = std::min(A.nsteps, s0 + A.every);
    if ((r = adj_restore(c, seg))) break;
    for (int s = s0; s < s1 && !r; ++s) {
      const double* cur[3] = {c->u, c->v, c->w};  // the step's input velocity, kept for its adjoint
      for (int q = 0; q < A.nv && !r; ++q) r = adj_copy(c, A.inputs[(size_t)A.nv * (s - s0) + q], cur[q]);
      if (!r && cudaGraphLaunch(c->graph, c->stream) != cudaSuccess) r = fail(FEN_ERR_CUDA, "graph launch");
    }
    if (r) break;
    c->launches += c->launches_per_step * (s1 - s0);
    k_adj_slot<<<1, 32, 0, c->stream>>>(A.dslot, s1 - 1 - s0);
    c->launches++;
    for (int s = s1 - 1; s >= s0 && !r; --s)
      if (cudaGraphLaunch(ag, c->stream) != cudaSuccess) r = fail(FEN_ERR_CUDA, "graph launch");
    c->launches += per_adj * (s1 - s0);
  }
  cudaGraphExecDestroy(ag);
  if (r) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return r;
  }
  CK(cudaEventRecord(e1, c->stream));
  CK(cudaEventSynchronize(e1));
  float f = 0;
  CK(cudaEventElapsedTime(&f, e0, e1));
  A.bwd_ms = f;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if ((r = adj_restore(c, A.nckpt))) return r;
  // gradient: interior of v^ at step 0, ghost entries zero
  double* gout[3] = {g_u, g_v, g_w};
  double* gdev[3] = {A.uh, A.vh, A.wh};
  const int nxg = c->n[0] + 2, nyg = c->n[1] + 2, nzg = d3 ? c->n[2] + 2 : 3;
  for (int q = 0; q < c->dim; ++q) {
    if ((r = relayout<double>(c, gdev[q], gout[q], 1, 1))) return r;
    double* g = gout[q];
    for (int k = 0; k < nzg; ++k)
      for (int j = 0; j < nyg; ++j)
        for (int i = 0; i < nxg; ++i) {
          const bool in_k = d3 ? (k >= 1 && k <= c->n[2]) : (k == 1);
          if (!in_k || i == 0 || j == 0 || i == nxg - 1 || j == nyg - 1) g[i + (size_t)nxg * (j + (size_t)nyg * k)] = 0.0;
        }
  }
  if (ms) {
    ms[0] = A.bwd_ms;
    ms[1] = A.fwd_ms;
  }
  return 0;
}

int fen_adjoint_backward(fen_ctx* c, const double* lam_u, const double* lam_v, double* g_u, double* g_v, double* ms) {
  if (c && c->dim == 3) return fail(FEN_ERR_ARG, "3D contexts take fen_adjoint_backward3 (three components)");
  return fen_adjoint_backward3(c, lam_u, lam_v, nullptr, g_u, g_v, nullptr, ms);
}

int fen_set_ibm_forcing(fen_ctx* c, int comp, int npoints, const int* ijk, const int* nnbr, const int* nbr_ijk,
                        const double* w, const double* c0) {
  if (!c || comp < 0 || comp >= c->dim || npoints < 0) return fail(FEN_ERR_ARG, "bad argument");
  if (c->mixed) return fail(FEN_ERR_ARG, "the IBM forcing hook runs in FP64 contexts only");
  if (npoints > 0 && (!ijk || !nnbr || !c0)) return fail(FEN_ERR_ARG, "null argument");
  auto& I = c->ibm[comp];
  void* bs[] = {I.idx, I.nidx, I.nn, I.w, I.c0, I.vs, I.fe};
  for (void* b : bs) if (b) cudaFree(b);
  I = fen_ctx::Ibm();
  drop_graph(c);
  if (npoints == 0) return 0;
  const int K = (c->dim == 3) ? c->n[2] : 1;
  auto lin = [&](const int* q, long long* out) -> bool {
    const int i = q[0], j = q[1], k = (c->dim == 3) ? q[2] : 1;
    if (i < 0 || i > c->n[0] + 1 || j < 0 || j > c->n[1] + 1 || k < 0 || k > K + 1) return false;
    *out = c->L.idx(i, j, c->dim == 3 ? k : 0);
    return true;
  };
  std::vector<long long> idx(npoints), nidx((size_t)8 * npoints, 0);
  std::vector<int> nn(npoints);
  std::vector<double> ww((size_t)8 * npoints, 0.0), cc(c0, c0 + npoints);
  for (int p = 0; p < npoints; ++p) {
    if (!lin(ijk + 3 * p, &idx[p])) return fail(FEN_ERR_ARG, "forced point outside the grid");
    const int i = ijk[3 * p], j = ijk[3 * p + 1], k = (c->dim == 3) ? ijk[3 * p + 2] : 1;
    if (i < 1 || i > c->n[0] || j < 1 || j > c->n[1] || k < 1 || k > K) return fail(FEN_ERR_ARG, "forced point is not interior");
    nn[p] = nnbr[p];
    if (nn[p] < 0 || nn[p] > 8 || (nn[p] > 0 && (!nbr_ijk || !w))) return fail(FEN_ERR_ARG, "stencil size must be 0..8");
    for (int q = 0; q < nn[p]; ++q) {
      if (!lin(nbr_ijk + 3 * (8 * p + q), &nidx[(size_t)8 * p + q])) return fail(FEN_ERR_ARG, "stencil point outside the grid");
      ww[(size_t)8 * p + q] = w[(size_t)8 * p + q];
    }
  }
  int r;
  if ((r = alloc(&I.idx, npoints)) || (r = alloc(&I.nidx, 8LL * npoints)) || (r = alloc(&I.nn, npoints)) ||
      (r = alloc(&I.w, 8LL * npoints)) || (r = alloc(&I.c0, npoints)) || (r = alloc(&I.vs, npoints)) ||
      (r = alloc(&I.fe, npoints)))
    return r;
  CK(cudaMemcpy(I.idx, idx.data(), idx.size() * sizeof(long long), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(I.nidx, nidx.data(), nidx.size() * sizeof(long long), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(I.nn, nn.data(), nn.size() * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(I.w, ww.data(), ww.size() * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(I.c0, cc.data(), cc.size() * sizeof(double), cudaMemcpyHostToDevice));
  I.n = npoints;
  return 0;
}

int fen_get_ibm_force(fen_ctx* c, int comp, double* fe) {
  if (!c || comp < 0 || comp >= c->dim || !fe) return fail(FEN_ERR_ARG, "bad argument");
  const auto& I = c->ibm[comp];
  if (I.n) {
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(fe, I.fe, I.n * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return 0;
}

int fen_set_split_pressure(fen_ctx* c, double rhomin) {
  if (!c || !(rhomin > 0.0)) return fail(FEN_ERR_ARG, "bad argument");
  if (c->mixed) return fail(FEN_ERR_ARG, "the variable-property path runs in FP64 contexts only");
  double* d;
  int r;
  if ((r = prop_field(c, FEN_P_O, &d))) return r;
  c->split = 1;
  c->rhomin = rhomin;
  drop_graph(c);
  return 0;
}

int fen_debug_checks(long long* count, long long* first) {
  if (!count || !first) return fail(FEN_ERR_ARG, "null argument");
#ifdef FEN_DEBUG_CHECKS
  unsigned long long n = 0;
  long long f = 0;
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpyFromSymbol(&n, g_fen_oob_count, sizeof(n)));
  CK(cudaMemcpyFromSymbol(&f, g_fen_oob_first, sizeof(f)));
  *count = (long long)n;
  *first = n ? f : 0;
#else
  *count = -1;
  *first = 0;
#endif
  return 0;
}

int fen_sync(fen_ctx* c) {
  if (!c) return fail(FEN_ERR_ARG, "null argument");
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

long long fen_kernel_launches(fen_ctx* c) { return c ? c->launches : 0; }

int fen_time_steps(fen_ctx* c, int nsteps, double dt, double* ms) {
  if (!c || !ms) return fail(FEN_ERR_ARG, "null argument");
  int r;
  if ((r = pre_step(c, dt))) return r;
  if ((r = capture_graph(c))) return r;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaEventRecord(e0, c->stream));
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(c->graph, c->stream));
  CK(cudaEventRecord(e1, c->stream));
  CK(cudaEventSynchronize(e1));
  float f = 0;
  CK(cudaEventElapsedTime(&f, e0, e1));
  *ms = f;
  c->launches += c->launches_per_step * nsteps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 0;
}

int fen_profile_step(fen_ctx* c, int reps, double dt, double* out) {
  if (!c || !out || reps < 1) return fail(FEN_ERR_ARG, "bad argument");
  int r;
  if ((r = pre_step(c, dt))) return r;
  cudaEvent_t ev[9];
  for (int q = 0; q < 9; ++q) CK(cudaEventCreate(&ev[q]));
  for (int q = 0; q < 8; ++q) out[q] = 0;
  for (int rep = 0; rep < reps; ++rep) {
    if ((r = enqueue_step(c, ev))) return r;
    CK(cudaEventSynchronize(ev[8]));
    for (int q = 0; q < 8; ++q) {
      float f = 0;
      CK(cudaEventElapsedTime(&f, ev[q], ev[q + 1]));
      out[q] += f / reps;
    }
  }
  for (int q = 0; q < 9; ++q) cudaEventDestroy(ev[q]);
  return 0;
}

}  // extern "C"
