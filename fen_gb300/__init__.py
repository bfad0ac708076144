"""fen_gb300 — GB300-native incompressible projection step with FEN's interfaces.

Python face of ``libfen_gb300.so`` (C ABI in ``include/fen_gpu.h``).  The names mirror the
FEN Fortran modules the C ABI replaces:

    grid_mod            Grid(...)                         (src/grid.f90:67-200)
    solver_mod          Solver.init_solver / advance_solution / destroy_solver
                                                           (src/solver.f90:34-99, 333)
    navier_stokes_mod   set_timestep, module state v, p, phi, dv_o, S, maxdiv, maxCFL
                                                           (src/navier_stokes.f90:17-45, 623)
    poisson_mod         solve_poisson                      (src/poisson.f90:21-29)
    fields_mod          gradient, divergence, laplacian    (src/fields.f90:13-26)
                        add_advection                      (src/navier_stokes.f90:261-353)

Fields are exchanged as numpy arrays in FEN's allocation of each field, x fastest: v, p, phi,
rho, mu with one ghost layer, f(0:nx+1, 0:ny+1, 0:nz+1), viewed in numpy as shape
(nz+2, ny+2, nx+2) (in 2D the z extent is 0:2, 3 planes); dv_o and S without ghosts,
f(1:nx, 1:ny, 1:nz), shape (nz, ny, nx) (1 plane in 2D).  ``Solver.field_shape(fid)`` gives
the shape.

The CUDA library is required: there is no CPU fallback, and loading fails loudly when the
shared library or a GPU is missing.
"""
import ctypes
import os

import numpy as np

__all__ = ["Grid", "Solver", "Ensemble", "FenError", "PERIODIC", "WALL", "INFLOW", "OUTFLOW", "load_library"]

PERIODIC, WALL, INFLOW, OUTFLOW = 0, 1, 2, 3
BC_NAMES = {"Periodic": PERIODIC, "Wall": WALL, "Inflow": INFLOW, "Outflow": OUTFLOW}
LEFT, RIGHT, BOTTOM, TOP, FRONT, BACK = range(6)
U, V, W, P, PHI = 0, 1, 2, 3, 4
DVO_X, DVO_Y, DVO_Z = 5, 6, 7
S_X, S_Y, S_Z = 8, 9, 10
RHO, MU, P_O = 11, 12, 13  # cell density, cell viscosity, old pressure of the split
FP64, MIXED = 0, 1
SOLVER_NAMES = ["pp", "pn", "nn", "ppp", "ppn", "npn", "nnn", "pnp"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfen_gb300.so")


class FenError(RuntimeError):
    pass


class _Params(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("lz", ctypes.c_double),
        ("origin", ctypes.c_double * 3), ("bc", ctypes.c_int * 6), ("aniso", ctypes.c_int),
        ("density", ctypes.c_double), ("viscosity", ctypes.c_double), ("g", ctypes.c_double * 3),
        ("cfl", ctypes.c_double), ("constant_cfl", ctypes.c_int), ("precision", ctypes.c_int),
        ("refine", ctypes.c_int),
    ]


class _Status(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double), ("dt_o", ctypes.c_double), ("maxdiv", ctypes.c_double),
        ("maxcfl", ctypes.c_double), ("maxvel", ctypes.c_double), ("dt_visc", ctypes.c_double),
        ("nan_detected", ctypes.c_int), ("poisson_solver", ctypes.c_int),
    ]


_lib = None
_EXPORTS = [
    "fen_ctx_create", "fen_ctx_destroy", "fen_last_error", "fen_upload", "fen_download",
    "fen_update_ghost_nodes", "fen_set_bc_values", "fen_set_bc_type", "fen_set_timestep",
    "fen_set_dt_o", "fen_advance_solution", "fen_advance_n", "fen_get_status", "fen_solve_poisson",
    "fen_divergence", "fen_explicit_terms", "fen_sync", "fen_kernel_launches", "fen_time_steps",
    "fen_profile_step", "fen_save_state", "fen_load_state", "fen_save_fields", "fen_adjoint_setup",
    "fen_adjoint_forward", "fen_adjoint_backward", "fen_ensemble_create", "fen_ensemble_destroy",
    "fen_ensemble_upload", "fen_ensemble_download", "fen_ensemble_set_timestep", "fen_ensemble_advance",
    "fen_ensemble_status", "fen_ensemble_config", "fen_ensemble_set_config", "fen_ensemble_tune",
    "fen_ensemble_launches", "fen_ensemble_smem_bytes", "fen_ensemble_adjoint_setup", "fen_ensemble_adjoint_forward",
    "fen_ensemble_adjoint_seed", "fen_ensemble_adjoint_backward", "fen_ensemble_adjoint_gradient",
    "fen_ensemble_adjoint_dts", "fen_set_split_pressure", "fen_set_ibm_forcing", "fen_get_ibm_force",
    "fen_upload_gl", "fen_download_gl", "fen_field_bounds", "fen_gradient", "fen_laplacian", "fen_add_advection",
    "fen_save_state_mf", "fen_load_state_mf", "fen_adjoint_backward3", "fen_debug_checks",
]


def load_library(path=None):
    """Load libfen_gb300.so and declare the C ABI.  Raises FenError if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise FenError(f"{path} not built: run `python -m fen_gb300.build` (needs nvcc)")
    L = ctypes.CDLL(path)
    vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
    L.fen_ctx_create.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(vp)]
    L.fen_ctx_destroy.argtypes = [vp]
    L.fen_last_error.restype = ctypes.c_char_p
    L.fen_upload.argtypes = [vp, ip, dp]
    L.fen_download.argtypes = [vp, ip, dp]
    L.fen_upload_gl.argtypes = [vp, ip, dp, ip]
    L.fen_download_gl.argtypes = [vp, ip, dp, ip]
    L.fen_field_bounds.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.fen_update_ghost_nodes.argtypes = [vp, ip]
    L.fen_set_bc_values.argtypes = [vp, ip, ip, dp]
    L.fen_set_bc_type.argtypes = [vp, ip, ip, ip]
    L.fen_set_timestep.argtypes = [vp, ctypes.c_double, dp]
    L.fen_set_dt_o.argtypes = [vp, ctypes.c_double]
    L.fen_advance_solution.argtypes = [vp, ip, dp]
    L.fen_advance_n.argtypes = [vp, ip, dp]
    L.fen_get_status.argtypes = [vp, ctypes.POINTER(_Status)]
    L.fen_solve_poisson.argtypes = [vp]
    L.fen_divergence.argtypes = [vp, dp]
    L.fen_explicit_terms.argtypes = [vp, dp]
    L.fen_gradient.argtypes = [vp, ip, dp, dp, dp]
    L.fen_laplacian.argtypes = [vp, ip, dp]
    L.fen_add_advection.argtypes = [vp, dp, dp, dp]
    L.fen_sync.argtypes = [vp]
    L.fen_kernel_launches.argtypes = [vp]
    L.fen_kernel_launches.restype = ctypes.c_longlong
    L.fen_time_steps.argtypes = [vp, ip, ctypes.c_double, dp]
    L.fen_profile_step.argtypes = [vp, ip, ctypes.c_double, dp]
    L.fen_save_state.argtypes = [vp, ctypes.c_char_p]
    L.fen_load_state.argtypes = [vp, ctypes.c_char_p]
    L.fen_save_fields.argtypes = [vp, ctypes.c_char_p, ip]
    L.fen_save_state_mf.argtypes = [vp, ctypes.c_char_p, dp]
    L.fen_load_state_mf.argtypes = [vp, ctypes.c_char_p, dp]
    L.fen_adjoint_setup.argtypes = [vp, ip, ip]
    L.fen_set_split_pressure.argtypes = [vp, ctypes.c_double]
    cip_ = ctypes.POINTER(ctypes.c_int)
    L.fen_set_ibm_forcing.argtypes = [vp, ip, ip, cip_, cip_, cip_, dp, dp]
    L.fen_get_ibm_force.argtypes = [vp, ip, dp]
    L.fen_adjoint_forward.argtypes = [vp, ctypes.c_double]
    L.fen_adjoint_backward.argtypes = [vp, dp, dp, dp, dp, dp]
    L.fen_adjoint_backward3.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp]
    cip = ctypes.POINTER(ctypes.c_int)
    L.fen_ensemble_create.argtypes = [ctypes.c_int, cip, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int, ctypes.POINTER(vp)]
    L.fen_ensemble_destroy.argtypes = [vp]
    L.fen_ensemble_upload.argtypes = [vp, ctypes.c_int, dp, dp, dp]
    L.fen_ensemble_download.argtypes = [vp, ctypes.c_int, dp, dp, dp]
    L.fen_ensemble_set_timestep.argtypes = [vp, ctypes.c_double]
    L.fen_ensemble_advance.argtypes = [vp, ctypes.c_int, dp]
    L.fen_ensemble_status.argtypes = [vp, ctypes.c_int, dp]
    L.fen_ensemble_config.argtypes = [vp, cip, cip, cip, cip, cip]
    L.fen_ensemble_set_config.argtypes = [vp, ctypes.c_int, cip]
    L.fen_ensemble_tune.argtypes = [vp, ctypes.c_int, ctypes.c_char_p]
    L.fen_ensemble_launches.argtypes = [vp]
    L.fen_ensemble_launches.restype = ctypes.c_longlong
    L.fen_ensemble_smem_bytes.argtypes = [ctypes.c_int, ctypes.c_int]
    L.fen_ensemble_smem_bytes.restype = ctypes.c_size_t
    L.fen_ensemble_adjoint_setup.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.fen_ensemble_adjoint_forward.argtypes = [vp, dp]
    L.fen_ensemble_adjoint_seed.argtypes = [vp, ctypes.c_int, dp, dp]
    L.fen_ensemble_adjoint_backward.argtypes = [vp, dp]
    L.fen_ensemble_adjoint_gradient.argtypes = [vp, ctypes.c_int, dp, dp]
    L.fen_ensemble_adjoint_dts.argtypes = [vp, ctypes.c_int, dp, dp]
    L.fen_debug_checks.argtypes = [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
    if path == LIB_PATH:
        _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Grid:
    """grid%setup(Nx, Ny, Nz, Lx, Ly, Lz, x0, prow, pcol, bc) (src/grid.f90:67-200).

    prow/pcol are accepted for interface parity and ignored: one device holds the domain.
    ``bc`` is a list of 'Periodic' | 'Wall' | 'Inflow' | 'Outflow' (or the integer codes) for
    left, right, bottom, top[, front, back]; all periodic when omitted (grid.f90:96-104).
    ``aniso`` enables one spacing per axis (the reference uses delta = Lx/Nx everywhere).
    """

    def __init__(self, Nx, Ny, Nz, Lx, Ly, Lz, x0=(0.0, 0.0, 0.0), prow=1, pcol=1, bc=None, dim=None, aniso=False):
        self.dim = dim if dim is not None else (2 if Nz == 1 else 3)
        self.Nx, self.Ny, self.Nz = int(Nx), int(Ny), int(Nz) if self.dim == 3 else 1
        self.Lx, self.Ly, self.Lz = float(Lx), float(Ly), float(Lz)
        self.origin = tuple(float(v) for v in x0)
        bc = list(bc) if bc is not None else ["Periodic"] * (2 * self.dim)
        self.bc = [BC_NAMES[b] if isinstance(b, str) else int(b) for b in bc]
        self.aniso = bool(aniso)
        self.delta = self.Lx / float(np.float32(self.Nx))
        if aniso:
            self.deltas = (self.Lx / self.Nx, self.Ly / self.Ny, (self.Lz / self.Nz) if self.dim == 3 else self.delta)
        else:
            self.deltas = (self.delta,) * 3

    @property
    def shape(self):
        """numpy shape (k, j, i) of a ghosted field."""
        return ((self.Nz + 2) if self.dim == 3 else 3, self.Ny + 2, self.Nx + 2)

    @property
    def interior_shape(self):
        """numpy shape (k, j, i) of a field without ghosts (FEN's default gl = 0)."""
        return (self.Nz if self.dim == 3 else 1, self.Ny, self.Nx)


# Ghost level of FEN's allocation of each field (navier_stokes.f90:759-768): dv_o and S have
# none (scalar.f90:76-81), the others one.
def field_gl(fid):
    return 0 if DVO_X <= fid <= S_Z else 1


class Solver:
    """One solver instance: init_solver + the navier_stokes_mod/poisson_mod module state.

    Module variables of navier_stokes_mod (density, viscosity, g, CFL, constant_CFL,
    navier_stokes.f90:18-45) are constructor arguments.  ``precision`` selects the FP64 form
    or the mixed form (``MIXED``: FP32 stencils/transforms, double-float state, FP64
    tridiagonal and reductions); ``refine`` is the mixed form's number of iterative-
    refinement solves per step.
    """

    def __init__(self, grid, density=1.0, viscosity=1.0, g=(0.0, 0.0, 0.0), CFL=1.0, constant_CFL=False,
                 precision=FP64, refine=1, lib=None):
        self._L = load_library(lib)
        self.grid = grid
        p = _Params()
        p.dim, p.nx, p.ny, p.nz = grid.dim, grid.Nx, grid.Ny, grid.Nz
        p.lx, p.ly, p.lz = grid.Lx, grid.Ly, grid.Lz
        p.origin = (ctypes.c_double * 3)(*grid.origin)
        bc = grid.bc + [PERIODIC] * (6 - len(grid.bc))
        p.bc = (ctypes.c_int * 6)(*bc)
        p.aniso = int(grid.aniso)
        p.density, p.viscosity = float(density), float(viscosity)
        p.g = (ctypes.c_double * 3)(*[float(x) for x in g])
        p.cfl, p.constant_cfl, p.precision = float(CFL), int(bool(constant_CFL)), int(precision)
        p.refine = int(refine) if precision == MIXED else 0
        self._h = ctypes.c_void_p()
        self._check(self._L.fen_ctx_create(ctypes.byref(p), ctypes.byref(self._h)))
        self.dt_o = None

    # -- lifecycle -----------------------------------------------------------------------
    def _check(self, rc):
        if rc != 0:
            msg = self._L.fen_last_error().decode()
            raise FenError(f"fen error {rc}: {msg}")

    def destroy_solver(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.fen_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy_solver()
        except Exception:
            pass

    # -- fields ----------------------------------------------------------------------------
    def zeros(self, fid=None):
        """A zero host array shaped like field `fid` (a ghosted field when omitted)."""
        return np.zeros(self.field_shape(fid if fid is not None else U))

    def field_shape(self, fid, gl=None):
        """numpy shape of field `fid` with ghost level `gl` (FEN's allocation when None)."""
        gl = field_gl(fid) if gl is None else gl
        return self.grid.shape if gl == 1 else self.grid.interior_shape

    def field_bounds(self, fid):
        """Fortran (lbound, ubound) of FEN's allocation of field `fid`."""
        lo, hi = (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
        self._check(self._L.fen_field_bounds(self._h, fid, lo, hi))
        return tuple(lo), tuple(hi)

    def set_field(self, fid, arr, gl=None):
        """Upload field `fid` from a host array in FEN's allocation of it (or with ghost level
        `gl`: 0 interior only, 1 with one ghost layer)."""
        a = np.ascontiguousarray(arr, dtype=np.float64)
        shape = self.field_shape(fid, gl)
        if a.shape != shape:
            raise ValueError(f"field {fid}: shape {a.shape} != {shape}")
        g = field_gl(fid) if gl is None else int(gl)
        self._check(self._L.fen_upload_gl(self._h, fid, _dp(a), g))

    def get_field(self, fid, out=None, gl=None):
        """Download field `fid`; into `out` (a C-contiguous float64 array of the field's shape,
        e.g. a pinned host buffer) when given, else into a new array."""
        shape = self.field_shape(fid, gl)
        if out is None:
            a = np.zeros(shape)
        else:
            a = out
            if a.shape != shape or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
                raise ValueError(f"out must be a C-contiguous float64 array of shape {shape}")
        g = field_gl(fid) if gl is None else int(gl)
        self._check(self._L.fen_download_gl(self._h, fid, _dp(a), g))
        return a

    def update_ghost_nodes(self, fid):
        self._check(self._L.fen_update_ghost_nodes(self._h, fid))

    def set_bc_values(self, fid, face, values):
        a = np.ascontiguousarray(values, dtype=np.float64)
        self._check(self._L.fen_set_bc_values(self._h, fid, face, _dp(a)))

    def set_bc_type(self, fid, face, t):
        self._check(self._L.fen_set_bc_type(self._h, fid, face, t))

    # -- navier_stokes_mod / solver_mod ----------------------------------------------------
    def set_timestep(self, U):
        dt = ctypes.c_double()
        self._check(self._L.fen_set_timestep(self._h, float(U), ctypes.byref(dt)))
        self.dt_o = dt.value
        return dt.value

    def set_dt_o(self, dt_o):
        self._check(self._L.fen_set_dt_o(self._h, float(dt_o)))
        self.dt_o = float(dt_o)

    def advance_solution(self, step, dt):
        d = ctypes.c_double(dt)
        self._check(self._L.fen_advance_solution(self._h, int(step), ctypes.byref(d)))
        return d.value

    def advance_n(self, nsteps, dt):
        d = ctypes.c_double(dt)
        self._check(self._L.fen_advance_n(self._h, int(nsteps), ctypes.byref(d)))
        return d.value

    def status(self):
        s = _Status()
        self._check(self._L.fen_get_status(self._h, ctypes.byref(s)))
        return {"dt": s.dt, "dt_o": s.dt_o, "maxdiv": s.maxdiv, "maxCFL": s.maxcfl, "maxvel": s.maxvel,
                "dt_visc": s.dt_visc, "nan": bool(s.nan_detected), "poisson_solver": SOLVER_NAMES[s.poisson_solver]}

    def print_solver_status(self, step, time, dt):
        """print_navier_stokes_solver_status line (navier_stokes.f90:743-746)."""
        s = self.status()
        return "step: %7d time: %13.6E dt: %13.6E maxdiv: %13.6E maxCFL:  %13.6E" % (
            step, time, dt, s["maxdiv"], s["maxCFL"])

    # -- poisson_mod / fields_mod ----------------------------------------------------------
    def solve_poisson(self, phi=None):
        """solve_poisson(phi): solves in place on the device copy of phi; with an array
        argument it uploads it first and returns the solution."""
        if phi is not None:
            self.set_field(PHI, phi)
        self._check(self._L.fen_solve_poisson(self._h))
        if phi is not None:
            return self.get_field(PHI)

    def divergence(self):
        g = self.grid
        out = np.zeros(g.Nx * g.Ny * g.Nz)
        self._check(self._L.fen_divergence(self._h, _dp(out)))
        return out.reshape(g.Nz, g.Ny, g.Nx)

    def gradient(self, fid):
        """gradient_of_scalar of field `fid` (p, phi, rho, mu, p_o): interior arrays
        (gx, gy[, gz]) at the faces (fields.f90:31-64)."""
        g = self.grid
        out = [np.zeros(g.interior_shape) for _ in range(3)]
        self._check(self._L.fen_gradient(self._h, fid, _dp(out[0]), _dp(out[1]), _dp(out[2])))
        return tuple(out[: g.dim])

    def laplacian(self, fid):
        """laplacian of field `fid` over the interior: laplacian_of_scalar for p, phi, rho, mu,
        p_o; the laplacian_of_vector component formula for u, v, w (fields.f90:256-343)."""
        out = np.zeros(self.grid.interior_shape)
        self._check(self._L.fen_laplacian(self._h, fid, _dp(out)))
        return out

    def add_advection(self, rhs=None):
        """add_advection(comp_grid, RHS) (navier_stokes.f90:261-353): RHS += the advection
        terms of the current velocity; rhs is a list of interior arrays (zeros if None),
        updated in place and returned."""
        g = self.grid
        if rhs is None:
            rhs = [np.zeros(g.interior_shape) for _ in range(g.dim)]
        rr = [np.ascontiguousarray(a, dtype=np.float64) for a in rhs]
        for a in rr:
            if a.shape != g.interior_shape:
                raise ValueError(f"rhs shape {a.shape} != {g.interior_shape}")
        z = rr[2] if g.dim == 3 else np.zeros(1)
        self._check(self._L.fen_add_advection(self._h, _dp(rr[0]), _dp(rr[1]), _dp(z)))
        for a, b in zip(rhs, rr):
            if a is not b:
                a[...] = b
        return rhs

    def explicit_terms(self):
        g = self.grid
        out = np.zeros(3 * g.Nx * g.Ny * g.Nz)
        self._check(self._L.fen_explicit_terms(self._h, _dp(out)))
        return out.reshape(3, g.Nz, g.Ny, g.Nx)[: g.dim]

    # -- solver_mod checkpoint / snapshots (solver.f90:103-329) ---------------------------
    def save_state(self, step, directory="data", path=None):
        """save_state(step): data/state_<step:7>.raw in FEN's raw layout; returns the path."""
        path = path or os.path.join(directory, "state_%07d.raw" % step)
        self._check(self._L.fen_save_state(self._h, path.encode()))
        return path

    def load_state(self, step, directory="data", path=None):
        path = path or os.path.join(directory, "state_%07d.raw" % step)
        self._check(self._L.fen_load_state(self._h, path.encode()))
        return path

    def save_state_mf(self, step, vof, directory="data", path=None):
        """save_state of FEN's multiphase build: the state file plus vof (the caller's interior
        array), rho, mu and p_o; returns the path."""
        path = path or os.path.join(directory, "state_%07d.raw" % step)
        a = np.ascontiguousarray(vof, dtype=np.float64)
        if a.shape != self.grid.interior_shape:
            raise ValueError(f"vof shape {a.shape} != {self.grid.interior_shape}")
        self._check(self._L.fen_save_state_mf(self._h, path.encode(), _dp(a)))
        return path

    def load_state_mf(self, step, directory="data", path=None):
        """load_state of FEN's multiphase build; returns the volume fraction read."""
        path = path or os.path.join(directory, "state_%07d.raw" % step)
        vof = np.zeros(self.grid.interior_shape)
        self._check(self._L.fen_load_state_mf(self._h, path.encode(), _dp(vof)))
        return vof

    def save_fields(self, step, directory="data"):
        self._check(self._L.fen_save_fields(self._h, directory.encode(), int(step)))

    # -- variable-property path (navier_stokes.f90:80-136, 357-452; FP64) ---------------------
    def set_split_pressure(self, rhomin):
        """Dodd-Ferrante split pressure of FEN's multiphase step with minimum density rhomin
        (p_o = FEN field P_O); density and viscosity fields are RHO and MU (set_field)."""
        self._check(self._L.fen_set_split_pressure(self._h, float(rhomin)))

    def set_ibm_forcing(self, comp, ijk, nnbr, nbr_ijk=None, w=None, c0=None):
        """apply_ibm_forcing hook (navier_stokes.f90:106-108): forced points of one velocity
        component (Fortran (i, j, k) per row of ijk), each taking c0 + sum w_q v*(nbr_q) with
        up to 8 neighbours (nbr_ijk shape (n, 8, 3), w shape (n, 8)); nnbr = 0 with c0 the
        solid velocity forces a solid point."""
        ijk = np.ascontiguousarray(ijk, dtype=np.int32).reshape(-1, 3)
        n = ijk.shape[0]
        nn = np.ascontiguousarray(nnbr, dtype=np.int32).reshape(n)
        nb = np.ascontiguousarray(nbr_ijk if nbr_ijk is not None else np.zeros((n, 8, 3)), dtype=np.int32).reshape(n, 8, 3)
        ww = np.ascontiguousarray(w if w is not None else np.zeros((n, 8)), dtype=np.float64).reshape(n, 8)
        cc = np.ascontiguousarray(c0 if c0 is not None else np.zeros(n), dtype=np.float64).reshape(n)
        cip = ctypes.POINTER(ctypes.c_int)
        self._check(self._L.fen_set_ibm_forcing(self._h, int(comp), n, ijk.ctypes.data_as(cip), nn.ctypes.data_as(cip),
                                                nb.ctypes.data_as(cip), _dp(ww), _dp(cc)))
        self._ibm_n = getattr(self, "_ibm_n", {})
        self._ibm_n[comp] = n

    def ibm_force(self, comp):
        """Fe = (vs - v*)/dt of the forced points of the last step."""
        out = np.zeros(getattr(self, "_ibm_n", {}).get(comp, 0))
        if out.size:
            self._check(self._L.fen_get_ibm_force(self._h, int(comp), _dp(out)))
        return out

    # -- discrete adjoint (FP64; periodic, or walls in y) ------------------------------------
    def adjoint_setup(self, nsteps, every):
        self._check(self._L.fen_adjoint_setup(self._h, int(nsteps), int(every)))

    def adjoint_forward(self, dt):
        """Run the configured rollout from the current state, keeping checkpoints."""
        self._check(self._L.fen_adjoint_forward(self._h, float(dt)))

    def adjoint_backward(self, lam_u, lam_v, lam_w=None):
        """Gradient w.r.t. the initial velocity of a loss with sensitivity (lam_u, lam_v[,
        lam_w]) to the final velocity (ghosted arrays).  Returns (g_u, g_v, times_ms) in 2D and
        (g_u, g_v, g_w, times_ms) in 3D, times = (backward, forward) in ms."""
        lu = np.ascontiguousarray(lam_u, dtype=np.float64)
        lv = np.ascontiguousarray(lam_v, dtype=np.float64)
        d3 = self.grid.dim == 3
        lw = np.ascontiguousarray(lam_w if lam_w is not None else self.zeros(), dtype=np.float64)
        gu, gv, gw, ms = self.zeros(), self.zeros(), self.zeros(), np.zeros(2)
        self._check(self._L.fen_adjoint_backward3(self._h, _dp(lu), _dp(lv), _dp(lw), _dp(gu), _dp(gv), _dp(gw), _dp(ms)))
        return (gu, gv, gw, ms) if d3 else (gu, gv, ms)

    # -- measurement -------------------------------------------------------------------------
    def kernel_launches(self):
        return int(self._L.fen_kernel_launches(self._h))

    def time_steps(self, nsteps, dt):
        ms = ctypes.c_double()
        self._check(self._L.fen_time_steps(self._h, int(nsteps), float(dt), ctypes.byref(ms)))
        return ms.value

    def profile_step(self, reps, dt):
        out = np.zeros(8)
        self._check(self._L.fen_profile_step(self._h, int(reps), float(dt), _dp(out)))
        return out

    def sync(self):
        self._check(self._L.fen_sync(self._h))


class Ensemble:
    """Batched ensemble of independent 2D periodic runs advanced by one persistent launch.

    No counterpart in FEN, which runs one grid per program; each run follows FEN's 2D
    periodic projection step (navier_stokes_solver, navier_stokes.f90:50-136, pp Poisson
    solver) with density 1, constant-CFL time stepping and the forcing
    S_x = forcing[0] sin(forcing[1] y).  Fields are FP32 on the device, reductions FP64.
    Arrays exchanged with the host are interiors of shape (N, N), axis 1 = x.
    """

    def __init__(self, n, viscosity, length=2 * np.pi, CFL=0.4, forcing=(1.0, 4), lib=None):
        self._L = load_library(lib) if (lib is None or isinstance(lib, str)) else lib
        n = np.ascontiguousarray(n, dtype=np.int32)
        nu = np.ascontiguousarray(viscosity, dtype=np.float64)
        if n.shape != nu.shape or n.ndim != 1:
            raise ValueError("n and viscosity must be 1D arrays of the same length")
        self.n = n.copy()
        self.nruns = len(n)
        self.length = float(length)
        self._h = ctypes.c_void_p()
        rc = self._L.fen_ensemble_create(int(self.nruns), n.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(nu),
                                         self.length, float(CFL), float(forcing[0]), int(forcing[1]),
                                         ctypes.byref(self._h))
        self._check(rc)

    def _check(self, rc):
        if rc != 0:
            raise FenError(f"fen error {rc}: {self._L.fen_last_error().decode()}")

    def destroy(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.fen_ensemble_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def upload(self, run, u, v, p=None):
        N = int(self.n[run])
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u, v)]
        for a in arrs:
            if a.shape != (N, N):
                raise ValueError(f"run {run}: expected shape {(N, N)}, got {a.shape}")
        pp = None if p is None else np.ascontiguousarray(p, dtype=np.float64)
        self._check(self._L.fen_ensemble_upload(self._h, int(run), _dp(arrs[0]), _dp(arrs[1]),
                                                _dp(pp) if pp is not None else None))

    def download(self, run):
        N = int(self.n[run])
        u, v, p = np.zeros((N, N)), np.zeros((N, N)), np.zeros((N, N))
        self._check(self._L.fen_ensemble_download(self._h, int(run), _dp(u), _dp(v), _dp(p)))
        return u, v, p

    def set_timestep(self, U):
        self._check(self._L.fen_ensemble_set_timestep(self._h, float(U)))

    def advance(self, nsteps):
        """Advance every run by nsteps steps (one launch); returns the device time in ms."""
        ms = ctypes.c_double()
        self._check(self._L.fen_ensemble_advance(self._h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def status(self, run):
        o = np.zeros(8)
        self._check(self._L.fen_ensemble_status(self._h, int(run), _dp(o)))
        return {"time": o[0], "dt": o[1], "dt_o": o[2], "maxvel": o[3], "ke": o[4], "maxdiv": o[5],
                "nan": bool(o[6]), "viscosity": o[7]}

    def config(self):
        ci = ctypes.c_int
        t, nc, ncl = ci(), ci(), ci()
        sizes = (ci * 64)()
        groups = (ci * 64)()
        self._check(self._L.fen_ensemble_config(self._h, ctypes.byref(t), sizes, groups, ctypes.byref(nc),
                                                ctypes.byref(ncl)))
        return {"threads": t.value, "clusters": ncl.value,
                "groups": {int(sizes[c]): int(groups[c]) for c in range(nc.value)}}

    def set_config(self, threads, groups=None):
        """groups: {N: CTAs per run} for every grid size of the ensemble."""
        arr = None
        if groups is not None:
            order = list(self.config()["groups"].keys())
            arr = (ctypes.c_int * len(order))(*[int(groups[N]) for N in order])
        self._check(self._L.fen_ensemble_set_config(self._h, int(threads), arr))

    def tune(self, steps=20, cache=None):
        self._check(self._L.fen_ensemble_tune(self._h, int(steps), cache.encode() if cache else None))
        return self.config()

    def launches(self):
        return int(self._L.fen_ensemble_launches(self._h))

    # -- forward/adjoint pair ----------------------------------------------------------------
    def adjoint_setup(self, nsteps, every):
        self.adj_nsteps = int(nsteps)
        self._check(self._L.fen_ensemble_adjoint_setup(self._h, int(nsteps), int(every)))

    def adjoint_forward(self):
        """Advance every run adj_nsteps steps in one launch, keeping checkpoints; returns ms."""
        ms = ctypes.c_double()
        self._check(self._L.fen_ensemble_adjoint_forward(self._h, ctypes.byref(ms)))
        return ms.value

    def adjoint_seed(self, run, lam_u, lam_v):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (lam_u, lam_v)]
        self._check(self._L.fen_ensemble_adjoint_seed(self._h, int(run), _dp(a[0]), _dp(a[1])))

    def adjoint_backward(self):
        """Backward sweep of every run in one launch; returns ms."""
        ms = ctypes.c_double()
        self._check(self._L.fen_ensemble_adjoint_backward(self._h, ctypes.byref(ms)))
        return ms.value

    def adjoint_gradient(self, run):
        N = int(self.n[run])
        gu, gv = np.zeros((N, N)), np.zeros((N, N))
        self._check(self._L.fen_ensemble_adjoint_gradient(self._h, int(run), _dp(gu), _dp(gv)))
        return gu, gv

    def adjoint_dts(self, run):
        dt, dto = np.zeros(self.adj_nsteps), np.zeros(self.adj_nsteps)
        self._check(self._L.fen_ensemble_adjoint_dts(self._h, int(run), _dp(dt), _dp(dto)))
        return dt, dto


def ensemble_smem_bytes(n, groups, lib=None):
    """Shared memory per CTA of an n x n run held by `groups` CTAs (0 if invalid)."""
    L = lib or load_library()
    return int(L.fen_ensemble_smem_bytes(int(n), int(groups)))


def partition_runs(n, world_size):
    """Split ensemble runs across `world_size` GPUs (one process each) by cost: longest
    processing time first on the per-run cost N^2 (the runs are independent, so no data-path
    collective is needed).  Returns one array of run indices per rank, each sorted."""
    n = np.asarray(n, dtype=np.int64)
    order = np.argsort(-(n * n), kind="stable")
    load = np.zeros(world_size, dtype=np.int64)
    parts = [[] for _ in range(world_size)]
    for q in order:
        r = int(np.argmin(load))
        parts[r].append(int(q))
        load[r] += int(n[q]) * int(n[q])
    return [np.array(sorted(p), dtype=np.int64) for p in parts]
