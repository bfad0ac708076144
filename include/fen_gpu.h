/*
 * fen_gpu.h — C ABI of the GB300 projection-step library (libfen_gb300.so).
 *
 * Drop-in boundary for FEN's incompressible projection step: the Fortran modules
 * solver_mod, navier_stokes_mod, poisson_mod and fields_mod keep their public interfaces
 * and bind these entry points through iso_c_binding.  Plain pointers and sizes only.
 *
 * Conventions
 *   - Every entry point returns 0 on success or a negative FEN_ERR_* code; the message of
 *     the last failure on the calling thread is returned by fen_last_error().
 *   - Host field arrays use FEN's Fortran layout, x fastest, with the ghost level FEN
 *     allocates for that field (src/navier_stokes.f90:759-768, src/scalar.f90:76-81):
 *       gl = 1: f(0:nx+1, 0:ny+1, 0:nz+1) for v (u, v, w), p, phi, rho, mu, p_o;
 *       gl = 0: f(1:nx, 1:ny, 1:nz) for dv_o and S (FEN's default, no ghosts).
 *     In 2D the z extent is 0:2 (gl = 1; only plane k = 1 is read or written) or 1:1
 *     (gl = 0).  fen_field_bounds returns the bounds; fen_upload_gl/fen_download_gl take
 *     an explicit ghost level for callers whose host copy is laid out otherwise.
 *   - One context = one grid + one solver instance on the current CUDA device, with one
 *     stream.  Calls on one context must be serialised by the caller; distinct contexts are
 *     independent.  Device state persists between calls; host arrays are never retained.
 */
#ifndef FEN_GPU_H
#define FEN_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* Physical boundary conditions (src/grid.f90:41-46). */
enum { FEN_BC_PERIODIC = 0, FEN_BC_WALL = 1, FEN_BC_INFLOW = 2, FEN_BC_OUTFLOW = 3 };
/* Faces in the reference order (src/scalar.f90:24-36). */
enum { FEN_LEFT = 0, FEN_RIGHT = 1, FEN_BOTTOM = 2, FEN_TOP = 3, FEN_FRONT = 4, FEN_BACK = 5 };
/* Field identifiers (module state of navier_stokes_mod, src/navier_stokes.f90:36-37). */
enum {
  FEN_U = 0, FEN_V = 1, FEN_W = 2, FEN_P = 3, FEN_PHI = 4,
  FEN_DVO_X = 5, FEN_DVO_Y = 6, FEN_DVO_Z = 7,
  FEN_S_X = 8, FEN_S_Y = 9, FEN_S_Z = 10,
  /* cell-centred density and viscosity fields and the old pressure of the split
   * (navier_stokes.f90:36, multiphase.f90:25): uploading FEN_RHO or FEN_MU switches the
   * FP64 step to FEN's variable-property branches */
  FEN_RHO = 11, FEN_MU = 12, FEN_P_O = 13
};
/* Arithmetic forms. */
enum { FEN_FP64 = 0, FEN_MIXED = 1 };
/* Error codes. */
enum {
  FEN_OK = 0,
  FEN_ERR_ARG = -1,      /* invalid argument or size */
  FEN_ERR_BC = -2,       /* boundary-condition combination without a Poisson solver */
  FEN_ERR_CUDA = -3,     /* CUDA runtime failure */
  FEN_ERR_NAN = -4,      /* NaN detected by the step diagnostics */
  FEN_ERR_NOMEM = -5,    /* device allocation failed */
  FEN_ERR_STATE = -6     /* call out of order (e.g. step before set_timestep) */
};

typedef struct fen_ctx fen_ctx;

/* Grid + solver parameters: grid%setup (src/grid.f90:67-200) and the navier_stokes_mod
 * module variables density, viscosity, g, CFL, constant_CFL (src/navier_stokes.f90:18-45). */
typedef struct {
  int dim;              /* 2 or 3 (the reference's -DDIM) */
  int nx, ny, nz;       /* interior cells; nz = 1 in 2D */
  double lx, ly, lz;    /* domain lengths */
  double origin[3];
  int bc[6];            /* FEN_BC_* per face (left, right, bottom, top, front, back) */
  int aniso;            /* 0: delta = Lx/Nx on every axis (grid.f90:140); 1: Li/Ni per axis */
  double density, viscosity;
  double g[3];
  double cfl;
  int constant_cfl;
  int precision;        /* FEN_FP64 or FEN_MIXED */
  int refine;           /* FEN_MIXED: iterative-refinement solves per step (0 or 1) */
} fen_params;

/* Per-step diagnostics (navier_stokes.f90:24-33, 570-619). */
typedef struct {
  double dt, dt_o, maxdiv, maxcfl, maxvel, dt_visc;
  int nan_detected;
  int poisson_solver;   /* 0 pp, 1 pn, 2 nn, 3 ppp, 4 ppn, 5 npn, 6 nnn, 7 pnp */
} fen_status;

/* grid%setup + init_solver: allocate_navier_stokes_fields + init_poisson_solver
 * (src/solver.f90:34-99, src/navier_stokes.f90:752-1067, src/poisson.f90:57-113).
 * Sizes: every axis 2^a 3^b with a >= 1.  Each line transform holds its lines in shared
 * memory, so an axis is limited to 12288 points for FP64 x lines (24576 in FEN_MIXED) and
 * to 6144 for FP64 periodic columns (12288 in FEN_MIXED); beyond that the call returns
 * FEN_ERR_ARG ("transform length too large for one CTA"). */
int fen_ctx_create(const fen_params* params, fen_ctx** out);
/* destroy_solver (src/solver.f90:333-357) + destroy_poisson_solver (poisson.f90:1456). */
int fen_ctx_destroy(fen_ctx* ctx);
const char* fen_last_error(void);

/* Host <-> device transfer of one field in FEN's allocation of it (layout above), like a
 * Fortran assignment to v%x%f or S%x%f: the host array is c_loc(f%f) of the FEN field.
 * fen_upload of a gl = 1 field copies interior and ghosts; a gl = 0 field (dv_o, S) has no
 * ghosts to copy. */
int fen_upload(fen_ctx* ctx, int field, const double* host);
int fen_download(fen_ctx* ctx, int field, double* host);
/* The same with the host array's ghost level given explicitly (0: interior f(1:nx, 1:ny,
 * 1:nz) only, the device ghosts are left as they are; 1: f(0:nx+1, 0:ny+1, 0:nz+1)). */
int fen_upload_gl(fen_ctx* ctx, int field, const double* host, int gl);
int fen_download_gl(fen_ctx* ctx, int field, double* host, int gl);
/* Fortran bounds lbound(f%f) / ubound(f%f) of FEN's allocation of `field` (scalar.f90:
 * 76-81): lo = 1 - gl, hi = n + gl per axis (in 2D the z bounds are 0:2 or 1:1). */
int fen_field_bounds(fen_ctx* ctx, int field, int lo[3], int hi[3]);
/* scalar%update_ghost_nodes (src/scalar.f90:223-396) on the device copy. */
int fen_update_ghost_nodes(fen_ctx* ctx, int field);
/* Dirichlet values of one face of one field: field%bc%left ... (scalar.f90:28-36).  The
 * array covers the ghosted face extents as FEN allocates them (scalar.f90:89-95). */
int fen_set_bc_values(fen_ctx* ctx, int field, int face, const double* values);
/* Override a field boundary type (-1 halo is not used on one device): field%bc%type_* */
int fen_set_bc_type(fen_ctx* ctx, int field, int face, int type);

/* set_timestep (src/navier_stokes.f90:623-666): dt = min(CFL delta/U, dt_visc); dt_o = dt. */
int fen_set_timestep(fen_ctx* ctx, double U, double* dt);
/* Set dt_o explicitly (module variable navier_stokes_mod::dt_o, navier_stokes.f90:33). */
int fen_set_dt_o(fen_ctx* ctx, double dt_o);
/* advance_solution => navier_stokes_solver (src/navier_stokes.f90:50-136).  dt is
 * intent(inout): updated when constant_cfl is set. */
int fen_advance_solution(fen_ctx* ctx, int step, double* dt);
/* nsteps consecutive navier_stokes_solver calls without host synchronisation between them
 * (one captured CUDA graph replayed); dt as above after the last step. */
int fen_advance_n(fen_ctx* ctx, int nsteps, double* dt);
/* Diagnostics of the last step (maxdiv, maxCFL, dt, dt_o). */
int fen_get_status(fen_ctx* ctx, fen_status* out);

/* solve_poisson(phi) on the device copy of FEN_PHI (src/poisson.f90:21-29, 306-1451). */
int fen_solve_poisson(fen_ctx* ctx);
/* divergence(v, div) over the interior (src/fields.f90:120-153); out is nx*ny*nz, x fastest. */
int fen_divergence(fen_ctx* ctx, double* out);
/* compute_explicit_terms(dv) with the current v, p (src/navier_stokes.f90:217-257); the
 * three components go to out (3 * nx*ny*nz, x fastest). */
int fen_explicit_terms(fen_ctx* ctx, double* out);

/* fields_mod generics on the device copy of a field (src/fields.f90:13-26), FP64 results in
 * interior arrays f(1:nx, 1:ny, 1:nz), the shape FEN allocates for grad_p and lap_v (gl = 0).
 * fen_gradient: gradient_of_scalar (fields.f90:31-64) of p, phi, rho, mu or p_o, forward
 * differences to the faces (gz unused in 2D).  fen_laplacian: laplacian_of_scalar (:256-290)
 * of a scalar field, or the component formula of laplacian_of_vector (:294-343) for u, v, w.
 * fen_add_advection: add_advection(comp_grid, RHS) (navier_stokes.f90:261-353, called by
 * test/small_test/navier_stokes/advection/advection.f90:50): adds the advection terms of the
 * current velocity to the caller's RHS arrays (in/out). */
int fen_gradient(fen_ctx* ctx, int field, double* gx, double* gy, double* gz);
int fen_laplacian(fen_ctx* ctx, int field, double* out);
int fen_add_advection(fen_ctx* ctx, double* rhs_x, double* rhs_y, double* rhs_z);

/* save_state / load_state (src/solver.f90:160-329): raw FP64 global interiors, x fastest,
 * no header, in the order p, u, v, dv_o%x, dv_o%y[, w, dv_o%z]; load_state refreshes the
 * ghost nodes of p and v.  FEN names the file data/state_<step:7>.raw. */
int fen_save_state(fen_ctx* ctx, const char* path);
int fen_load_state(fen_ctx* ctx, const char* path);
/* The same files of FEN's multiphase build (-DMF, solver.f90:203-208, 296-304): the fields
 * above followed by vof, rho, mu and p_o (FP64 contexts).  The volume fraction belongs to the
 * caller (VoF advection stays with FEN): vof is its interior array f(1:nx, 1:ny, 1:nz),
 * written as given and filled by the load.  rho, mu and p_o come from the device (their
 * initial values density, viscosity and 0 when never uploaded); the load uploads them, which
 * puts the context on the variable-property path, and refreshes their ghosts.  In 3D FEN has
 * no variable-viscosity branch: mu is written as the constant viscosity and not read back. */
int fen_save_state_mf(fen_ctx* ctx, const char* path, const double* vof);
int fen_load_state_mf(fen_ctx* ctx, const char* path, double* vof);
/* save_fields (src/solver.f90:103-156): <dir>/vx_<step:7>.raw, vy_, [vz_], p_ with the
 * velocity interpolated to cell centres (face_to_center, src/fields.f90:210-252). */
int fen_save_fields(fen_ctx* ctx, const char* dir, int step);

/* Discrete adjoint of the step (no counterpart in FEN, which has no differentiation): FP64
 * contexts with fixed dt (dt_o = dt), no source field and constant properties, 2D or 3D,
 * periodic (pp, ppp) or periodic with 'Wall' faces in y (pn, pnp: the channel).
 * fen_adjoint_setup sizes an nsteps rollout with a checkpoint every `every` steps;
 * fen_adjoint_forward runs the rollout from the current state (which ends at step nsteps);
 * fen_adjoint_backward3 takes the sensitivity of a scalar loss to the final velocity and
 * returns its gradient with respect to the initial velocity, recomputing each checkpoint
 * segment (lam_w, g_w unused in 2D).  Arrays use the host field layout (gl = 1); ghost
 * entries of the gradient are zero, as is the upper wall face of v (overwritten by the
 * boundary value in every step).  ms (optional, 2 doubles): backward and forward device
 * times.  fen_adjoint_backward is the 2D form. */
int fen_adjoint_setup(fen_ctx* ctx, int nsteps, int every);
int fen_adjoint_forward(fen_ctx* ctx, double dt);
int fen_adjoint_backward3(fen_ctx* ctx, const double* lam_u, const double* lam_v, const double* lam_w, double* g_u,
                          double* g_v, double* g_w, double* ms);
int fen_adjoint_backward(fen_ctx* ctx, const double* lam_u, const double* lam_v, double* g_u, double* g_v,
                         double* ms);

/* Variable-property momentum path (FP64 contexts).  Upload FEN_RHO (cell density) and/or
 * FEN_MU (cell viscosity; 2D only, as FEN's stress-divergence branch, navier_stokes.f90:
 * 405-452) and fill their ghosts with fen_update_ghost_nodes (p's boundary rules).  The step
 * then divides by the face densities center_to_face(rho) (fields.f90:175-206) and scales the
 * Poisson right-hand side by rho(i,j,k)/dt.  fen_set_split_pressure turns on the Dodd-
 * Ferrante split of FEN's multiphase step (navier_stokes.f90:80-96, 113, 174-184, 526-531,
 * 557) with the minimum density rhomin; the old pressure is FEN_P_O (zero until uploaded). */
int fen_set_split_pressure(fen_ctx* ctx, double rhomin);

/* IBM forcing hook (apply_ibm_forcing, navier_stokes.f90:106-108; eulerian_ibm.f90:194-268),
 * FP64 contexts.  After the predictor, every listed point of velocity component comp
 * (0 x, 1 y, 2 z; Fortran indices ijk[3p..3p+2], interior) takes the target
 *   vs = c0[p] + sum_{q < nnbr[p]} w[8p+q] * v*(nbr_ijk[3(8p+q)..])    (nnbr <= 8)
 * computed from the unforced v*: solid points carry nnbr = 0 and the solid velocity in c0,
 * interface points the interpolation the caller's solid geometry defines.  The velocity
 * ghosts are refilled afterwards.  npoints = 0 removes the component's list.
 * fen_get_ibm_force returns FEN's forcing Fe = (vs - v*)/dt of the last step (npoints values). */
int fen_set_ibm_forcing(fen_ctx* ctx, int comp, int npoints, const int* ijk, const int* nnbr, const int* nbr_ijk,
                        const double* w, const double* c0);
int fen_get_ibm_force(fen_ctx* ctx, int comp, double* fe);

/* Bounds record of the debug build (libfen_gb300_debug.so, compiled with FEN_DEBUG_CHECKS):
 * every field index of the library's kernels is checked against its array; an index outside
 * is counted (count), the first is kept (first, an element offset), and element 0 is used in
 * its place, so nothing is read or written out of range and nothing traps.  The release
 * library reports count = -1 (no checks compiled).  No counterpart in FEN, whose debug builds
 * rely on gfortran's -fcheck=all (src/Makefile.defs:13). */
int fen_debug_checks(long long* count, long long* first);
/* Synchronise the context stream. */
int fen_sync(fen_ctx* ctx);
/* Number of kernels this library launched on the context since creation. */
long long fen_kernel_launches(fen_ctx* ctx);
/* Time `nsteps` steps on the device with CUDA events on the context stream (graph replay,
 * no host work inside the timed region); returns milliseconds. */
int fen_time_steps(fen_ctx* ctx, int nsteps, double dt, double* ms);
/* Per-stage device time of one step, measured with CUDA events on the context stream:
 * out[0..7] = predictor, ghost(v*), forward transforms, spectral solve, inverse
 * transform(s), correction, ghost(v,p,phi), checks (milliseconds, averaged over reps). */
int fen_profile_step(fen_ctx* ctx, int reps, double dt, double* out);

/* Allocation-free 2D periodic Poisson solve.  No counterpart in the reference: it serves
 * callers that cannot allocate device memory (a host framework that owns every device
 * allocation through its own pool, or a solver embedded under a fixed memory budget).  It
 * solves lap(phi) = rhs as FEN's pp solver does (FFT in x and y, zero mode set to 0, mean
 * removed) with grid spacing lx/nx on both axes.  rhs and phi are caller-owned
 * device-accessible arrays of nx*ny doubles (interior only, x fastest); they may alias.  The
 * call allocates nothing: its scratch lives in a static device array of about 8.5 MB that
 * every GPU loading this library holds until exit, sized for nx, ny <= FEN_NOALLOC_MAX_N;
 * larger sizes are rejected with FEN_ERR_ARG.  The first call on each device fetches that
 * array's device address (the set-up); every later call checks the address again and
 * repeats the set-up if it changed (after cudaDeviceReset).  All calls share the array, so
 * calls that overlap on the GPU race and must be serialised.  Work is queued on `stream`
 * (NULL = default stream) and the call returns after synchronising it.  The eigenvalues
 * come from device sincospi here, not from the host cosine table of the context path, so
 * the result matches fen_solve_poisson on the same grid to rounding (1e-13 relative L2), not
 * bit for bit. */
#define FEN_NOALLOC_MAX_N 1024
int fen_poisson_pp2d_noalloc(const double* rhs, double* phi, int nx, int ny, double lx, void* stream);

/* ---- Batched ensemble of 2D periodic runs (no counterpart in the reference) ------------
 * FEN runs one grid per program (solver_mod::advance_solution, solver.f90:333, with the pp
 * Poisson solver, poisson.f90:416-505).  An ensemble holds `nruns` independent 2D periodic
 * runs on [0, length]^2, run q on an n[q] x n[q] grid (n = 2^a 3^b, a >= 2, b <= 1) with its own
 * viscosity, density 1, forcing S_x = forcing_amplitude sin(forcing_wavenumber y) at the
 * u points, and FEN's constant-CFL time step (CFL = cfl).  Fields are FP32 on the device,
 * reductions FP64.  One fen_ensemble_advance is ONE persistent kernel launch (captured in a
 * CUDA graph) that advances every run by nsteps steps.
 * Host arrays are interiors of n*n doubles, x fastest: u(i,j) at ((i+1) d, (j+1/2) d),
 * v(i,j) at ((i+1/2) d, (j+1) d), p(i,j) at the cell centres (0-based i, j; d = length/n). */
typedef struct fen_ensemble fen_ensemble;
int fen_ensemble_create(int nruns, const int* n, const double* viscosity, double length, double cfl,
                        double forcing_amplitude, int forcing_wavenumber, fen_ensemble** out);
int fen_ensemble_destroy(fen_ensemble* ens);
/* State of one run; p may be NULL (zero).  dv_o restarts at zero, time at zero. */
int fen_ensemble_upload(fen_ensemble* ens, int run, const double* u, const double* v, const double* p);
int fen_ensemble_download(fen_ensemble* ens, int run, double* u, double* v, double* p);
/* set_timestep(U) of every run (navier_stokes.f90:623-665): dt = dt_o = min(cfl d / U, dt_visc). */
int fen_ensemble_set_timestep(fen_ensemble* ens, double U);
/* Advance every run by nsteps steps in one launch; *ms = device time (CUDA events). */
int fen_ensemble_advance(fen_ensemble* ens, int nsteps, double* ms);
/* out[8] = time, dt, dt_o, maxvel, kinetic energy 1/2 <u^2+v^2>, max div, NaN flag, viscosity. */
int fen_ensemble_status(fen_ensemble* ens, int run, double* out);
/* Launch shape: CTA size, the distinct grid sizes (largest first), CTAs per run for each. */
int fen_ensemble_config(fen_ensemble* ens, int* threads, int* sizes, int* groups, int* nclasses, int* nclusters);
int fen_ensemble_set_config(fen_ensemble* ens, int threads, const int* groups);
/* Autotuner: times each feasible CTAs-per-run choice per grid size, then the CTA size, on
 * the ensemble's own runs (state restored afterwards); caches results in cache_path (may be
 * NULL or empty: no cache) and reuses them when present. */
int fen_ensemble_tune(fen_ensemble* ens, int steps, const char* cache_path);
long long fen_ensemble_launches(fen_ensemble* ens);
/* Forward/adjoint pair of every run: the discrete adjoint of the ensemble step (FP32, the
 * transpose of the step for the recorded dt sequence, as fen_adjoint_* does for one FP64
 * context).  setup sizes an nsteps rollout with checkpoints every `every` steps (device
 * storage of about (5 nsteps/every + 2 every + 7) n^2 floats per run); forward advances every
 * run nsteps steps in one launch, saving checkpoints and the (dt, dt_o) of each step;
 * seed sets the sensitivity of each run's loss to its final (u, v); backward sweeps every run
 * back in one launch (recomputing each segment from its checkpoint) and gradient returns the
 * gradient with respect to the run's initial (u, v).  Arrays are n*n doubles, x fastest. */
int fen_ensemble_adjoint_setup(fen_ensemble* ens, int nsteps, int every);
int fen_ensemble_adjoint_forward(fen_ensemble* ens, double* ms);
int fen_ensemble_adjoint_seed(fen_ensemble* ens, int run, const double* lam_u, const double* lam_v);
int fen_ensemble_adjoint_backward(fen_ensemble* ens, double* ms);
int fen_ensemble_adjoint_gradient(fen_ensemble* ens, int run, double* g_u, double* g_v);
/* The recorded (dt, dt_o) of each step of the last forward (nsteps doubles each). */
int fen_ensemble_adjoint_dts(fen_ensemble* ens, int run, double* dt, double* dt_o);
/* Dynamic + static shared memory per CTA for an n x n run on `groups` CTAs (0 if invalid);
 * host-only, no device needed. */
size_t fen_ensemble_smem_bytes(int n, int groups);

#ifdef __cplusplus
}
#endif
#endif /* FEN_GPU_H */
