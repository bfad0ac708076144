"""ctypes wrapper around the CPU FP64 oracle (oracle/fen_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` (as the
checker) and by ``bench.py``'s CPU-baseline leg.  The product library never loads it.

The oracle restates FEN's projection step (src/navier_stokes.f90, src/fields.f90,
src/scalar.f90, src/poisson.f90) in the reference's floating-point operation order.
Fields are Fortran-ordered ghosted arrays f(0:nx+1, 0:ny+1, 0:nz+1), x fastest; in 2D the
z extent is 0:2 with k = 1 the only plane used (scalar.f90:79-81).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "fen_oracle.cpp")
_LIB = os.path.join(_HERE, "liboracle.so")

# Physical boundary conditions (grid.f90:41-46)
PERIODIC, WALL, INFLOW, OUTFLOW = 0, 1, 2, 3
# Field ids
U, V, W, P, PHI = 0, 1, 2, 3, 4
DVO = (5, 6, 7)
S = (8, 9, 10)
RHO, MU, P_O = 14, 15, 16  # cell-centred density, viscosity, old pressure (split)
DV = (11, 12, 13)
SOLVERS = ["pp", "pn", "nn", "ppp", "ppn", "npn", "nnn", "pnp"]


def build(force=False):
    """Compile the oracle with g++ (-ffp-contract=off: no FMA contraction on any host)."""
    if not force and os.path.exists(_LIB) and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC):
        return _LIB
    cmd = ["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", _LIB, _SRC]
    subprocess.check_call(cmd)
    return _LIB


class _Params(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("lx", ctypes.c_double), ("ly", ctypes.c_double), ("lz", ctypes.c_double),
        ("x0", ctypes.c_double * 3), ("bc", ctypes.c_int * 6),
        ("density", ctypes.c_double), ("viscosity", ctypes.c_double), ("g", ctypes.c_double * 3),
        ("cfl", ctypes.c_double), ("constant_cfl", ctypes.c_int), ("aniso", ctypes.c_int),
        ("nthreads", ctypes.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        L = _lib
        dp_ = ctypes.POINTER(ctypes.c_double)
        L.or_create.restype = ctypes.c_void_p
        L.or_create.argtypes = [ctypes.POINTER(_Params)]
        L.or_destroy.argtypes = [ctypes.c_void_p]
        L.or_field.restype = ctypes.POINTER(ctypes.c_double)
        L.or_field.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.or_bc.restype = ctypes.POINTER(ctypes.c_double)
        L.or_bc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.or_bc_type.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.or_set_bc_type.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        for f in ("or_update_ghost_nodes",):
            getattr(L, f).argtypes = [ctypes.c_void_p, ctypes.c_int]
        for f in ("or_solve_poisson", "or_compute_explicit_terms", "or_add_advection"):
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.or_solver_kind.argtypes = [ctypes.c_void_p]
        L.or_set_timestep.restype = ctypes.c_double
        L.or_set_timestep.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.or_set_dt_o.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.or_set_properties.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        ip_ = ctypes.POINTER(ctypes.c_int)
        L.or_set_ibm.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ip_, ip_, ip_, dp_, dp_]
        L.or_ibm_force.restype = dp_
        L.or_ibm_force.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.or_get_dt_o.restype = ctypes.c_double
        L.or_get_dt_o.argtypes = [ctypes.c_void_p]
        L.or_step.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        L.or_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.or_diag.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        L.or_delta.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        L.or_divergence.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
        dp = ctypes.POINTER(ctypes.c_double)
        L.or_fft.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int]
        L.or_r2c.argtypes = [ctypes.c_int, dp, dp]
        L.or_c2r.argtypes = [ctypes.c_int, dp, dp]
        L.or_redft10.argtypes = [ctypes.c_int, dp, dp]
        L.or_redft01.argtypes = [ctypes.c_int, dp, dp]
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One FEN solver instance (grid + navier_stokes_mod + poisson_mod state) on the CPU."""

    def __init__(self, dim, n, L, bc=None, density=1.0, viscosity=1.0, g=(0, 0, 0), cfl=1.0,
                 constant_cfl=False, aniso=False, nthreads=None, origin=(0, 0, 0)):
        self.dim = dim
        n = list(n) + [1] * (3 - len(n))
        L = list(L) + [1.0] * (3 - len(L))
        if dim == 2:
            n[2] = 1
        self.n = n
        bc = list(bc) if bc is not None else [PERIODIC] * (2 * dim)
        bc = bc + [PERIODIC] * (6 - len(bc))
        p = _Params()
        p.dim, p.nx, p.ny, p.nz = dim, n[0], n[1], n[2]
        p.lx, p.ly, p.lz = L
        p.x0 = (ctypes.c_double * 3)(*origin)
        p.bc = (ctypes.c_int * 6)(*bc)
        p.density, p.viscosity = density, viscosity
        p.g = (ctypes.c_double * 3)(*g)
        p.cfl, p.constant_cfl, p.aniso = cfl, int(constant_cfl), int(aniso)
        p.nthreads = nthreads or min(os.cpu_count() or 1, 16)
        self._h = lib().or_create(ctypes.byref(p))
        if not self._h:
            raise ValueError("unsupported boundary-condition combination for the Poisson solver")
        self.shape = (n[2] + 2, n[1] + 2, n[0] + 2)  # numpy (k, j, i) view of f(i, j, k)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().or_destroy(self._h)
            self._h = None

    def field(self, fid):
        """Writable numpy view (k, j, i) of a ghosted Fortran array."""
        ptr = lib().or_field(self._h, fid)
        return np.ctypeslib.as_array(ptr, shape=self.shape)

    def bc_values(self, fid, face):
        n = self.n
        sizes = [(n[2] + 2, n[1] + 2)] * 2 + [(n[2] + 2, n[0] + 2)] * 2 + [(n[1] + 2, n[0] + 2)] * 2
        return np.ctypeslib.as_array(lib().or_bc(self._h, fid, face), shape=sizes[face])

    def bc_type(self, fid, face):
        return lib().or_bc_type(self._h, fid, face)

    def set_bc_type(self, fid, face, t):
        lib().or_set_bc_type(self._h, fid, face, t)

    def update_ghost_nodes(self, fid):
        lib().or_update_ghost_nodes(self._h, fid)

    def solve_poisson(self):
        lib().or_solve_poisson(self._h)

    @property
    def solver(self):
        return SOLVERS[lib().or_solver_kind(self._h)]

    def compute_explicit_terms(self):
        lib().or_compute_explicit_terms(self._h)

    def add_advection(self):
        lib().or_add_advection(self._h)

    def set_properties(self, var_mu=False, split=False, rhomin=1.0):
        """constant_viscosity = not var_mu; split: the Dodd-Ferrante pressure split with rhomin.
        Density and viscosity fields are the writable views field(RHO), field(MU)."""
        lib().or_set_properties(self._h, int(var_mu), int(split), float(rhomin))

    def set_ibm(self, comp, ijk, nnbr, nbr_ijk, w, c0):
        """IBM forcing list of one velocity component (see include/fen_gpu.h fen_set_ibm_forcing)."""
        a = [np.ascontiguousarray(x, dtype=np.int32) for x in (ijk, nnbr, nbr_ijk)]
        b = [np.ascontiguousarray(x, dtype=np.float64) for x in (w, c0)]
        self._ibm_keep = getattr(self, "_ibm_keep", {})
        self._ibm_keep[comp] = (a, b)
        ip_ = ctypes.POINTER(ctypes.c_int)
        lib().or_set_ibm(self._h, int(comp), len(b[1]), a[0].ctypes.data_as(ip_), a[1].ctypes.data_as(ip_),
                         a[2].ctypes.data_as(ip_), _dp(b[0]), _dp(b[1]))

    def ibm_force(self, comp, npoints):
        ptr = lib().or_ibm_force(self._h, int(comp))
        return np.ctypeslib.as_array(ptr, shape=(npoints,)).copy() if ptr else np.zeros(npoints)

    def set_timestep(self, U):
        return lib().or_set_timestep(self._h, U)

    @property
    def dt_o(self):
        return lib().or_get_dt_o(self._h)

    @dt_o.setter
    def dt_o(self, v):
        lib().or_set_dt_o(self._h, v)

    def step(self, dt):
        d = ctypes.c_double(dt)
        lib().or_step(self._h, ctypes.byref(d))
        return d.value

    def run(self, nsteps, dt):
        d = ctypes.c_double(dt)
        lib().or_run(self._h, nsteps, ctypes.byref(d))
        return d.value

    def diag(self):
        out = np.zeros(4)
        lib().or_diag(self._h, _dp(out))
        return {"maxdiv": out[0], "maxCFL": out[1], "dt_o": out[2], "dt_visc": out[3]}

    def delta(self):
        out = np.zeros(3)
        lib().or_delta(self._h, _dp(out))
        return out

    def divergence(self):
        out = np.zeros(self.n[0] * self.n[1] * self.n[2])
        lib().or_divergence(self._h, _dp(out))
        return out.reshape(self.n[2], self.n[1], self.n[0])


def fft(x, sign=-1):
    x = np.ascontiguousarray(x, dtype=complex)
    out = np.zeros_like(x)
    lib().or_fft(len(x), _dp(x.view(np.float64)), _dp(out.view(np.float64)), sign)
    return out


def r2c(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(len(x) // 2 + 1, complex)
    lib().or_r2c(len(x), _dp(x), _dp(out.view(np.float64)))
    return out


def c2r(X, n):
    X = np.ascontiguousarray(X, dtype=complex)
    out = np.zeros(n)
    lib().or_c2r(n, _dp(X.view(np.float64)), _dp(out))
    return out


def redft10(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    lib().or_redft10(len(x), _dp(x), _dp(out))
    return out


def redft01(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    lib().or_redft01(len(x), _dp(x), _dp(out))
    return out
