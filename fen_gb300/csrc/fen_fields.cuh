// fields_mod generics and add_advection as stand-alone device operators (FP64).
//
// FEN's fields_mod exports gradient, divergence and laplacian (src/fields.f90:13-26), and
// user programs call navier_stokes_mod::add_advection directly
// (test/small_test/navier_stokes/advection/advection.f90:50).  The time step fuses these into
// its own kernels; the operators here serve callers of the module interfaces.  They read a
// ghosted field in the padded HBM layout and write interior arrays f(1:nx, 1:ny, 1:nz)
// (x fastest), the shape FEN allocates for grad_p, dv and RHS (gl = 0).  Arithmetic follows
// the reference's operation order with explicitly rounded operations (no FMA contraction), so
// the results are bit-identical to a plain FP64 evaluation of the same formulas.
#pragma once
#include "fen_types.cuh"

namespace fen {

struct FieldOpArgs {
  const double *s, *u, *v, *w;  // ghosted inputs
  double *o0, *o1, *o2;         // interior outputs (o1, o2 unused where not needed)
  double id[3];                 // 1/delta per axis
  double id2[3];                // 1/delta^2 per axis
  int iso;
  int op;                       // see below
  int comp;                     // laplacian: 0 scalar / x, y component form, 2: z component form
};
enum { FOP_GRADIENT = 0, FOP_LAPLACIAN = 1, FOP_ADVECTION = 2 };

// 0-based interior index t -> Fortran (i, j, k) and the padded-layout offset.
template <int DIM>
__device__ __forceinline__ long long field_cell(const Layout& L, long long t) {
  const long long r = t / L.n0;
  const int i = (int)(t - r * L.n0) + 1;
  const int j = (int)(r % L.n1) + 1;
  const int k = (int)(r / L.n1) + 1;
  return L.idx(i, j, kst<DIM>(k));
}

// s(ip) - 2 s(i) + s(im), evaluated left to right as in fields.f90:283-284.
__device__ __forceinline__ double second_diff(double p, double two, double m) { return __dadd_rn(__dsub_rn(p, two), m); }

template <int DIM>
__global__ void __launch_bounds__(256) k_field_op(Layout L, FieldOpArgs a) {
  const long long ncell = (long long)L.n0 * L.n1 * (DIM == 3 ? L.n2 : 1);
  const long long sy = L.sx, sz = L.sp;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ncell; t += (long long)gridDim.x * blockDim.x) {
    const long long c = field_cell<DIM>(L, t);
    if (a.op == FOP_GRADIENT) {
      // gradient_of_scalar (fields.f90:31-64): forward differences to the faces
      const double* s = a.s;
      a.o0[t] = __dmul_rn(__dsub_rn(s[c + 1], s[c]), a.id[0]);
      a.o1[t] = __dmul_rn(__dsub_rn(s[c + sy], s[c]), a.id[1]);
      if (DIM == 3) a.o2[t] = __dmul_rn(__dsub_rn(s[c + sz], s[c]), a.id[2]);
    } else if (a.op == FOP_LAPLACIAN) {
      // laplacian_of_scalar (fields.f90:256-290) and the component forms of
      // laplacian_of_vector (:294-343): the z component sums its three second differences
      // before the scaling; per-axis scaling when the spacing is anisotropic
      const double* s = a.s;
      const double two = __dmul_rn(2.0, s[c]);
      const double dx = second_diff(s[c + 1], two, s[c - 1]);
      const double dy = second_diff(s[c + sy], two, s[c - sy]);
      double l;
      if (DIM == 3) {
        const double dz = second_diff(s[c + sz], two, s[c - sz]);
        if (a.iso) {
          l = (a.comp == 2) ? __dmul_rn(__dadd_rn(__dadd_rn(dx, dy), dz), a.id2[0])
                            : __dadd_rn(__dmul_rn(__dadd_rn(dx, dy), a.id2[0]), __dmul_rn(dz, a.id2[0]));
        } else {
          l = __dadd_rn(__dadd_rn(__dmul_rn(dx, a.id2[0]), __dmul_rn(dy, a.id2[1])), __dmul_rn(dz, a.id2[2]));
        }
      } else {
        l = a.iso ? __dmul_rn(__dadd_rn(dx, dy), a.id2[0]) : __dadd_rn(__dmul_rn(dx, a.id2[0]), __dmul_rn(dy, a.id2[1]));
      }
      a.o0[t] = l;
    } else {
      // add_advection (navier_stokes.f90:261-353): RHS -= div(u u) in divergence form with
      // the quarter products of the face and edge averages
      const double *U = a.u, *V = a.v, *W = a.w;
      const long long ip = c + 1, im = c - 1, jp = c + sy, jm = c - sy;
      const double uuip = __dmul_rn(0.25, __dmul_rn(__dadd_rn(U[ip], U[c]), __dadd_rn(U[ip], U[c])));
      const double uuim = __dmul_rn(0.25, __dmul_rn(__dadd_rn(U[im], U[c]), __dadd_rn(U[im], U[c])));
      const double uvjp = __dmul_rn(__dmul_rn(__dadd_rn(U[jp], U[c]), __dadd_rn(V[ip], V[c])), 0.25);
      const double uvjm = __dmul_rn(__dmul_rn(__dadd_rn(U[c], U[jm]), __dadd_rn(V[ip - sy], V[jm])), 0.25);
      double rx = __dsub_rn(__dsub_rn(a.o0[t], __dmul_rn(__dsub_rn(uuip, uuim), a.id[0])),
                            __dmul_rn(__dsub_rn(uvjp, uvjm), a.id[1]));
      const double vuip = __dmul_rn(__dmul_rn(__dadd_rn(V[ip], V[c]), __dadd_rn(U[jp], U[c])), 0.25);
      const double vuim = __dmul_rn(__dmul_rn(__dadd_rn(V[c], V[im]), __dadd_rn(U[im + sy], U[im])), 0.25);
      const double vvjp = __dmul_rn(0.25, __dmul_rn(__dadd_rn(V[jp], V[c]), __dadd_rn(V[jp], V[c])));
      const double vvjm = __dmul_rn(0.25, __dmul_rn(__dadd_rn(V[jm], V[c]), __dadd_rn(V[jm], V[c])));
      double ry = __dsub_rn(__dsub_rn(a.o1[t], __dmul_rn(__dsub_rn(vuip, vuim), a.id[0])),
                            __dmul_rn(__dsub_rn(vvjp, vvjm), a.id[1]));
      if (DIM == 3) {
        const long long kp = c + sz, km = c - sz;
        const double uwkp = __dmul_rn(__dmul_rn(__dadd_rn(U[kp], U[c]), __dadd_rn(W[ip], W[c])), 0.25);
        const double uwkm = __dmul_rn(__dmul_rn(__dadd_rn(U[c], U[km]), __dadd_rn(W[ip - sz], W[km])), 0.25);
        rx = __dsub_rn(rx, __dmul_rn(__dsub_rn(uwkp, uwkm), a.id[2]));
        const double vwkp = __dmul_rn(__dmul_rn(__dadd_rn(V[kp], V[c]), __dadd_rn(W[jp], W[c])), 0.25);
        const double vwkm = __dmul_rn(__dmul_rn(__dadd_rn(V[c], V[km]), __dadd_rn(W[jp - sz], W[km])), 0.25);
        ry = __dsub_rn(ry, __dmul_rn(__dsub_rn(vwkp, vwkm), a.id[2]));
        const double wuip = __dmul_rn(__dmul_rn(__dadd_rn(W[c], W[ip]), __dadd_rn(U[c], U[kp])), 0.25);
        const double wuim = __dmul_rn(__dmul_rn(__dadd_rn(W[c], W[im]), __dadd_rn(U[im], U[im + sz])), 0.25);
        const double wvjp = __dmul_rn(__dmul_rn(__dadd_rn(W[c], W[jp]), __dadd_rn(V[c], V[kp])), 0.25);
        const double wvjm = __dmul_rn(__dmul_rn(__dadd_rn(W[c], W[jm]), __dadd_rn(V[jm], V[jm + sz])), 0.25);
        const double wwkp = __dmul_rn(__dmul_rn(__dadd_rn(W[c], W[kp]), __dadd_rn(W[c], W[kp])), 0.25);
        const double wwkm = __dmul_rn(__dmul_rn(__dadd_rn(W[c], W[km]), __dadd_rn(W[c], W[km])), 0.25);
        a.o2[t] = __dsub_rn(__dsub_rn(__dsub_rn(a.o2[t], __dmul_rn(__dsub_rn(wuip, wuim), a.id[0])),
                                      __dmul_rn(__dsub_rn(wvjp, wvjm), a.id[1])),
                            __dmul_rn(__dsub_rn(wwkp, wwkm), a.id[2]));
      }
      a.o0[t] = rx;
      a.o1[t] = ry;
    }
  }
}

// FP32 field -> FP64 (the mixed form's phi, for the operators above).
static __global__ void k_widen_field(long long n, const float* __restrict__ src, double* __restrict__ dst) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    dst[t] = (double)src[t];
}

}  // namespace fen
