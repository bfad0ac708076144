// Allocation-free 2D periodic Poisson solve (FEN's pp solver, src/poisson.f90:416-505).
//
// Some callers cannot allocate device memory: host codes that run inside a framework which
// owns every device allocation through its own pool, or embedded solvers whose memory budget
// is fixed up front.  They already hold their input and output arrays, but cannot give the
// solver the scratch it needs.  fen_poisson_pp2d_noalloc therefore keeps its scratch (half spectrum, twiddles,
// eigenvalues, mean-removal partial sums) in one file-scope static device array of a fixed
// maximum size, which every GPU that loads this library holds until the process exits.
//
// The array name is only a host-side stand-in in host code; its device address is fetched
// with cudaGetSymbolAddress on the first call on each device (with that device current) and
// passed to the kernels.  Later calls fetch it again (no allocation) and redo the set-up
// when it changed, which happens after cudaDeviceReset reloads the module.  Every call
// shares the array and leaves its contents behind, so calls that overlap on the GPU
// (different streams, or different host threads on the same device) race; serialise them.
// Nothing in the array needs to start at zero: each call rewrites the tables it uses and
// every partial-sum slot it reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/fen_gpu.h"
#include "fen_kernels.cuh"

using namespace fen;

// Error reporting shared with the rest of the C ABI (fen_last_error).
int fen_internal_fail(int code, const char* msg);

namespace {

constexpr int kMaxN = FEN_NOALLOC_MAX_N;
constexpr long long kSpec = (long long)(kMaxN / 2 + 1) * kMaxN;  // complex half spectrum
constexpr long long kTwM = kMaxN / 2;                              // exp(-2 pi i m/(nx/2))
constexpr long long kTwN = kMaxN / 2 + 1;                          // exp(-2 pi i k/nx)
constexpr long long kTwY = kMaxN;                                  // exp(-2 pi i m/ny)
constexpr long long kLam = kMaxN;                                  // mwn_x and mwn_y (one double2 slot each pair)
constexpr long long kPart = 512;                                   // 1024 partial sums (doubles)
constexpr long long kScal = 16;                                    // StepScalars
constexpr long long kTotal = kSpec + kTwM + kTwN + kTwY + kLam + kPart + kScal;

}  // namespace

// The static scratch: 8.5 MB per device (see include/fen_gpu.h, FEN_NOALLOC_MAX_N).
static __device__ __align__(256) double2 g_noalloc_scratch[kTotal];

namespace {

std::mutex g_mu;
double2* g_addr[256] = {nullptr};

// Per-device set-up: the device address of the static array and the shared-memory limits of
// the transform kernels used here.  Runs on the first call on each device, and again when
// the array's address changed (a device reset reloads the module and drops the limits).
int setup_device(int dev, double2** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= 256) return fen_internal_fail(FEN_ERR_ARG, "fen_poisson_pp2d_noalloc: device index out of range");
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return fen_internal_fail(FEN_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
  if (g_addr[dev] != (double2*)p) {
    const int lim = 200 * 1024;
    e = cudaFuncSetAttribute(k_line<double, 2, true, OP_R2C, LD_FIELD, ST_CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_line<double, 3, false, OP_C2C_SOLVE, LD_CPLX, ST_CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_line<double, 2, true, OP_C2R, LD_CPLX, ST_FIELD>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e != cudaSuccess) return fen_internal_fail(FEN_ERR_CUDA, (std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e)).c_str());
    g_addr[dev] = (double2*)p;
  }
  *out = g_addr[dev];
  return 0;
}

bool radix_ok(int n) {
  if (n < 2 || n % 2) return false;
  int m = n;
  while (m % 2 == 0) m /= 2;
  while (m % 3 == 0) m /= 3;
  return m == 1;
}

bool make_plan_local(int M, FFTPlan& P) {
  P.M = M;
  P.nst = 0;
  int m = M;
  if (kFftMaxR64 >= 8)
    while (m % 8 == 0) { P.R[P.nst++] = 8; m /= 8; }
  while (m % 4 == 0) { P.R[P.nst++] = 4; m /= 4; }
  if (m % 2 == 0) { P.R[P.nst++] = 2; m /= 2; }
  while (m % 3 == 0) { P.R[P.nst++] = 3; m /= 3; }
  fft_plan_magic(P);
  return m == 1 && P.nst <= kMaxStages;
}

// Twiddles and modified wavenumbers 2(cos(2 pi i/n) - 1)/delta^2 (poisson.f90:141, 159).
__global__ void k_noalloc_tables(int nx, int ny, double delta, double2* wM, double2* wN, double2* wY, double* lamx,
                                 double* lamy) {
  const int h = nx / 2;
  const double d2 = delta * delta;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ny + nx + 2; t += gridDim.x * blockDim.x) {
    double s, c;
    if (t < h) { sincospi(2.0 * t / (double)h, &s, &c); wM[t] = make_double2(c, -s); }
    if (t <= h) { sincospi(2.0 * t / (double)nx, &s, &c); wN[t] = make_double2(c, -s); lamx[t] = 2.0 * (c - 1.0) / d2; }
    if (t < ny) { sincospi(2.0 * t / (double)ny, &s, &c); wY[t] = make_double2(c, -s); lamy[t] = 2.0 * (c - 1.0) / d2; }
  }
}

int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace

extern "C" int fen_poisson_pp2d_noalloc(const double* rhs, double* phi, int nx, int ny, double lx, void* stream) {
  if (!rhs || !phi) return fen_internal_fail(FEN_ERR_ARG, "fen_poisson_pp2d_noalloc: null array");
  if (nx > kMaxN || ny > kMaxN)
    return fen_internal_fail(FEN_ERR_ARG, ("fen_poisson_pp2d_noalloc: nx=" + std::to_string(nx) + ", ny=" + std::to_string(ny) +
                                           " exceeds the static scratch limit FEN_NOALLOC_MAX_N=" + std::to_string(kMaxN)).c_str());
  if (!radix_ok(nx) || !radix_ok(ny))
    return fen_internal_fail(FEN_ERR_ARG, "fen_poisson_pp2d_noalloc: nx and ny must be 2^a 3^b with a >= 1");
  if (!(lx > 0.0)) return fen_internal_fail(FEN_ERR_ARG, "fen_poisson_pp2d_noalloc: lx must be positive");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fen_internal_fail(FEN_ERR_CUDA, "fen_poisson_pp2d_noalloc: no current device");
  double2* base = nullptr;
  int r;
  if ((r = setup_device(dev, &base))) return r;
  cudaStream_t st = (cudaStream_t)stream;

  // carve the static array
  double2* spec = base;
  double2* wM = spec + kSpec;
  double2* wN = wM + kTwM;
  double2* wY = wN + kTwN;
  double* lamx = (double*)(wY + kTwY);
  double* lamy = lamx + (kMaxN / 2 + 1);
  double* part = (double*)(wY + kTwY + kLam);
  StepScalars* sc = (StepScalars*)(wY + kTwY + kLam + kPart);

  const int h = nx / 2 + 1;
  const long long hp = h;
  const double delta = lx / (double)(float)nx;  // grid.f90:140
  k_noalloc_tables<<<cdiv(nx + ny + 2, 256), 256, 0, st>>>(nx, ny, delta, wM, wN, wY, lamx, lamy);

  // interior-only arrays seen as a 2D field: idx(i, j) = (i - 1) + nx (j - 1)
  Layout L;
  L.dim = 2; L.n0 = nx; L.n1 = ny; L.n2 = 1;
  L.sx = nx; L.sy = ny; L.sp = (long long)nx * ny; L.off = -1 - nx; L.total = (long long)nx * ny;

  FFTPlan half, fully;
  if (!make_plan_local(nx / 2, half) || !make_plan_local(ny, fully))
    return fen_internal_fail(FEN_ERR_ARG, "fen_poisson_pp2d_noalloc: unsupported size");

  LineArgs<double> a;
  memset(&a, 0, sizeof(a));
  a.L = L;
  a.scale = 1.0;
  a.iso = 1;
  a.dim = 2;
  // x: r2c of every row (poisson.f90:441-445)
  LineArgs<double> ax = a;
  const int Mx = nx / 2;
  const int nlx = std::max(1, std::min(16, 1024 / Mx));
  ax.n = nx; ax.nl = nlx; ax.nlines = ny;
  ax.fsrc = rhs;
  ax.out = spec; ax.out_line = hp; ax.out_pos = 1; ax.out_outer = hp * ny;
  ax.plan = half;
  ax.tw.wM = wM; ax.tw.wN = wN; ax.tw.wD = nullptr;
  ax.mg[0] = fft_magic((unsigned)nx); ax.mg[1] = fft_magic((unsigned)Mx);
  ax.mg[2] = fft_magic((unsigned)(Mx + 1)); ax.mg[3] = fft_magic((unsigned)nlx);
  const dim3 gx(cdiv(ny, nlx), 1);
  const size_t smx = 2 * (size_t)nlx * Mx * sizeof(double2);
  k_line<double, 2, true, OP_R2C, LD_FIELD, ST_CPLX><<<gx, 256, smx, st>>>(ax);
  // y: forward FFT, /(nx ny), divide by mwn_x + mwn_y (zero mode -> 0), inverse (:451-478)
  LineArgs<double> ay = a;
  const int nly = (ny <= 512) ? 8 : 4;
  ay.n = ny; ay.nl = nly; ay.nlines = h;
  ay.in = spec; ay.out = spec;
  ay.in_line = 1; ay.in_pos = hp; ay.in_outer = 0;
  ay.out_line = 1; ay.out_pos = hp; ay.out_outer = 0;
  ay.scale = 1.0 / (double)(float)((long long)nx * ny);
  ay.lamA = lamx; ay.lamB = nullptr; ay.lamC = lamy;
  ay.plan = fully;
  ay.tw.wM = wY;
  ay.mg[0] = fft_magic((unsigned)ny); ay.mg[1] = fft_magic((unsigned)ny);
  ay.mg[2] = fft_magic((unsigned)(ny + 1)); ay.mg[3] = fft_magic((unsigned)nly);
  const dim3 gy(cdiv(h, nly), 1);
  const size_t smy = 2 * (size_t)nly * ny * sizeof(double2);
  k_line<double, 3, false, OP_C2C_SOLVE, LD_CPLX, ST_CPLX><<<gy, 256, smy, st>>>(ay);
  // x: c2r into phi with per-CTA line sums (:484-488)
  LineArgs<double> ai = ax;
  ai.in = spec; ai.in_line = hp; ai.in_pos = 1; ai.in_outer = hp * ny;
  ai.out = nullptr;
  ai.fdst = phi;
  ai.partial = part;
  k_line<double, 2, true, OP_C2R, LD_CPLX, ST_FIELD><<<gx, 256, smx, st>>>(ai);
  // subtract the mean (:491-503)
  const int npart = (int)(gx.x * gx.y);
  const int gm = std::min(cdiv((long long)nx * ny, 256), 152 * 8);
  k_mean_reduce<<<1, 1024, 0, st>>>(part, npart, (double)(float)((long long)nx * ny), sc);
  k_mean_subtract<double, 2><<<gm, 256, 0, st>>>(L, sc, phi);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fen_internal_fail(FEN_ERR_CUDA, (std::string("fen_poisson_pp2d_noalloc: ") + cudaGetErrorString(e)).c_str());
  return 0;
}
