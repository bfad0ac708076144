"""GPU parity: the CUDA path through the C ABI against the CPU oracle and FEN's known answers.

Tolerances: ghost fills are copies and 2*bc - f, so they are bit-exact.  Everything else
differs from the oracle only by rounding (FMA contraction on the GPU, FFT summation order,
reciprocal-multiply instead of division), so single operators are held to 1e-13 relative
L2 and multi-step runs to the 1e-12 relative L2 target of the FP64 form.
"""
import numpy as np
import pytest

import fen_gb300 as F
from oracle import oracle as O
from tests import cases as C

pytestmark = pytest.mark.gpu

RTOL_OP = 1e-13
RTOL_RUN = 1e-12


def pair(dim, n, L, bc=None, **kw):
    """An oracle and a GPU solver with identical parameters."""
    n = tuple(n) + (1,) * (3 - len(n))
    L = tuple(L) + (1.0,) * (3 - len(L))
    aniso = kw.pop("aniso", False)
    o = O.Oracle(dim, n, L, bc=bc, aniso=aniso, **{k: v for k, v in kw.items() if k in (
        "density", "viscosity", "g", "cfl", "constant_cfl")})
    bcn = list(bc) if bc is not None else [O.PERIODIC] * (2 * dim)
    g = F.Grid(n[0], n[1], n[2] if dim == 3 else 1, L[0], L[1], L[2], bc=bcn, dim=dim, aniso=aniso)
    s = F.Solver(g, density=kw.get("density", 1.0), viscosity=kw.get("viscosity", 1.0), g=kw.get("g", (0, 0, 0)),
                 CFL=kw.get("cfl", 1.0), constant_CFL=kw.get("constant_cfl", False))
    return o, s


def load_both(o, s, fid, arr):
    o.field(fid)[...] = arr
    s.set_field(fid, arr)


BC_SETS_2D = {
    "pp": [O.PERIODIC] * 4,
    "pn": [O.PERIODIC, O.PERIODIC, O.WALL, O.WALL],
    "nn": [O.WALL] * 4,
    "pn_io": [O.PERIODIC, O.PERIODIC, O.INFLOW, O.OUTFLOW],
}
BC_SETS_3D = {
    "ppp": [O.PERIODIC] * 6,
    "ppn": [O.PERIODIC] * 4 + [O.WALL] * 2,
    "npn": [O.WALL, O.WALL, O.PERIODIC, O.PERIODIC, O.WALL, O.WALL],
    "nnn": [O.WALL] * 6,
    "pnp": [O.PERIODIC, O.PERIODIC, O.WALL, O.WALL, O.PERIODIC, O.PERIODIC],
    "io": [O.INFLOW, O.OUTFLOW, O.WALL, O.WALL, O.PERIODIC, O.PERIODIC],
}


@pytest.mark.parametrize("name", list(BC_SETS_2D) + list(BC_SETS_3D))
def test_ghost_fill_bit_exact(fen_lib, name):
    dim = 2 if name in BC_SETS_2D else 3
    bc = (BC_SETS_2D if dim == 2 else BC_SETS_3D)[name]
    n = (12, 8, 1) if dim == 2 else (8, 12, 6)
    try:
        o, s = pair(dim, n, (1.0, 1.0, 1.0), bc=bc)
    except ValueError:
        pytest.skip("no Poisson solver for this combination")
    rng = np.random.Generator(np.random.PCG64(5))
    for fid in ([O.U, O.V, O.P] if dim == 2 else [O.U, O.V, O.W, O.P]):
        a = rng.standard_normal(s.grid.shape)
        load_both(o, s, fid, a)
        # non-zero Dirichlet values on every face
        for face in range(2 * dim):
            vals = o.bc_values(fid, face)
            vals[...] = rng.standard_normal(vals.shape)
            full = vals.copy()
            s.set_bc_values(fid, face, full)
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)
        got = s.get_field(fid)
        want = o.field(fid)
        if dim == 2:
            assert np.array_equal(got[1], want[1])
        else:
            assert np.array_equal(got, want)


@pytest.mark.parametrize("name", ["pp", "nn", "ppp", "pnp"])
def test_explicit_terms(fen_lib, name):
    dim = 2 if name in BC_SETS_2D else 3
    bc = (BC_SETS_2D if dim == 2 else BC_SETS_3D)[name]
    n = (16, 12, 1) if dim == 2 else (12, 8, 6)
    o, s = pair(dim, n, (1.3, 0.9, 1.1), bc=bc, viscosity=0.03, aniso=True)
    rng = np.random.Generator(np.random.PCG64(9))
    for fid in ([O.U, O.V] if dim == 2 else [O.U, O.V, O.W]):
        a = rng.standard_normal(s.grid.shape)
        load_both(o, s, fid, a)
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)
    o.compute_explicit_terms()
    got = s.explicit_terms()
    for q in range(dim):
        want = C.interior(o.field(O.DV[q]), dim)
        assert C.rel_l2(got[q].reshape(want.shape), want) < RTOL_OP


POISSON_SIZES = {"pp": (24, 16, 1), "pn": (16, 24, 1), "nn": (24, 12, 1), "ppp": (16, 12, 24),
                 "ppn": (12, 16, 8), "npn": (16, 12, 12), "nnn": (12, 8, 16), "pnp": (16, 24, 12)}


@pytest.mark.parametrize("name", list(POISSON_SIZES))
def test_poisson_matches_oracle(fen_lib, name):
    dim, bc, _, _ = C.poisson_case(name)
    n = POISSON_SIZES[name]
    o, s = pair(dim, n, (1.0, 1.0, 1.0), bc=bc)
    assert s.status()["poisson_solver"] == name
    rng = np.random.Generator(np.random.PCG64(13))
    rhs = C.random_interior(s.grid.shape, rng, dim)
    r = C.interior(rhs, dim)
    r -= r.mean()
    load_both(o, s, O.PHI, rhs)
    o.solve_poisson()
    got = C.interior(s.solve_poisson(rhs), dim)
    want = C.interior(o.field(O.PHI), dim)
    assert C.rel_l2(got, want) < RTOL_OP, C.rel_l2(got, want)


@pytest.mark.parametrize("dim,n", [(2, (8, 4096, 1)), (3, (8, 4, 6144)), (2, (8192, 8, 1)), (3, (12288, 4, 4))])
def test_poisson_long_lines(fen_lib, dim, n):
    # periodic columns too long for two per CTA (4096 and 6144 points: one column per CTA,
    # two FP64 buffers of the whole line in shared memory) and x lines of 8192 and 12288
    # points (one line per CTA) against the oracle
    h = 1.0 / max(n)
    L = tuple(m * h for m in n)
    bc = [O.PERIODIC] * (2 * dim)
    o, s = pair(dim, n, L, bc=bc)
    rng = np.random.Generator(np.random.PCG64(17))
    rhs = C.random_interior(s.grid.shape, rng, dim)
    load_both(o, s, O.PHI, rhs)
    o.solve_poisson()
    got = C.interior(s.solve_poisson(rhs), dim)
    want = C.interior(o.field(O.PHI), dim)
    assert C.rel_l2(got, want) < RTOL_OP, C.rel_l2(got, want)


def test_transform_length_limit(fen_lib):
    # an FP64 column of 8192 points (256 KB of buffers) exceeds one CTA: refused at set-up
    with pytest.raises(F.FenError, match="too large"):
        F.Solver(F.Grid(8, 8192, 1, 8 / 8192, 1.0, 1.0 / 8192))


@pytest.mark.parametrize("name", ["pp", "pn", "nn", "ppp", "ppn", "npn", "nnn", "pnp"])
def test_poisson_second_order_gpu(fen_lib, name):
    # test/small_test/poisson/convergence_rate through the C ABI: slope > 1.8
    dim, bc, rhsf, solf = C.poisson_case(name)
    Ns = [16, 32, 64] if dim == 2 else [8, 16, 32]
    errs = []
    for N in Ns:
        g = F.Grid(N, N, N if dim == 3 else 1, 1.0, 1.0, 1.0, bc=bc, dim=dim)
        s = F.Solver(g)
        X, Y, Z = C.poisson_rhs_grid(dim, N)
        a = s.zeros()
        if dim == 2:
            a[1, 1:-1, 1:-1] = rhsf(X, Y, Z)
        else:
            a[1:-1, 1:-1, 1:-1] = rhsf(X, Y, Z)
        phi = s.solve_poisson(a)
        errs.append(np.abs(C.interior(phi, dim) - solf(X, Y, Z)).max())
    assert C.convergence_slope(Ns, errs) > 1.8, errs


@pytest.mark.parametrize("bc", [[O.PERIODIC] * 6, [O.PERIODIC] * 4 + [O.WALL] * 2])
def test_projection_gpu(fen_lib, bc):
    # poisson/projection/projection.f90:84-126 through the C ABI: max |div| < 1e-11
    N = 32
    g = F.Grid(N, N, N, 1.0, 1.0, 1.0, bc=bc)
    s = F.Solver(g)
    rng = np.random.Generator(np.random.PCG64(21))
    worst = 0.0
    for _ in range(3):
        vel = {}
        for fid in (F.U, F.V, F.W):
            a = s.zeros()
            a[1:-1, 1:-1, 1:-1] = rng.random((N, N, N))
            s.set_field(fid, a)
            s.update_ghost_nodes(fid)
            vel[fid] = s.get_field(fid)
        div = s.divergence()
        a = s.zeros()
        a[1:-1, 1:-1, 1:-1] = -div
        s.solve_poisson(a)
        s.update_ghost_nodes(F.PHI)
        ph = s.get_field(F.PHI)
        for fid, ax in ((F.U, 2), (F.V, 1), (F.W, 0)):
            gphi = (np.roll(ph, -1, axis=ax) - ph) * N
            v = vel[fid]
            v[1:-1, 1:-1, 1:-1] += gphi[1:-1, 1:-1, 1:-1]
            s.set_field(fid, v)
            s.update_ghost_nodes(fid)
        worst = max(worst, np.abs(s.divergence()).max())
    assert worst < 1e-11


def _init_tgv2d(o, s, N, L):
    u, v, p = C.tgv2d_fields(N, L)
    for fid, a in ((O.U, u), (O.V, v), (O.P, p)):
        load_both(o, s, fid, a)
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)


def _compare_state(o, s, dim, tol):
    fids = [O.U, O.V, O.P] if dim == 2 else [O.U, O.V, O.W, O.P]
    out = {}
    for fid in fids:
        got = C.interior(s.get_field(fid), dim)
        want = C.interior(o.field(fid), dim)
        if fid == O.P:
            got = got - got.mean()
            want = want - want.mean()
        out[fid] = C.rel_l2(got, want)
        assert out[fid] < tol, (fid, out[fid])
    return out


def test_step_tgv2d(fen_lib):
    # the 2D TGV workload at reduced length: 128^2, nu = 0.01, dt = dt_o = 1e-3
    N, L = 128, 2 * np.pi
    o, s = pair(2, (N, N, 1), (L, L, L / N), viscosity=0.01)
    _init_tgv2d(o, s, N, L)
    dt = 1e-3
    o.dt_o = dt
    s.set_dt_o(dt)
    o.run(50, dt)
    s.advance_n(50, dt)
    _compare_state(o, s, 2, RTOL_RUN)
    so, sg = o.diag(), s.status()
    assert abs(sg["maxdiv"]) < 1e-11 and abs(so["maxdiv"]) < 1e-11
    assert abs(sg["maxCFL"] - so["maxCFL"]) <= 1e-12 * so["maxCFL"]


def test_step_tgv3d_constant_cfl(fen_lib):
    # the 3D TGV workload at reduced size: Re = 1600, CFL = 0.5, dt from set_timestep(U = 1)
    N, L = 32, 2 * np.pi
    o, s = pair(3, (N, N, N), (L, L, L), viscosity=1.0 / 1600, cfl=0.5, constant_cfl=True)
    u, v, w, p = C.tgv3d_fields(N, L)
    for fid, a in ((O.U, u), (O.V, v), (O.W, w), (O.P, p)):
        load_both(o, s, fid, a)
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)
    dto = o.set_timestep(1.0)
    dtg = s.set_timestep(1.0)
    assert dto == dtg
    dts_o, dts_g = [], []
    for step in range(1, 21):
        dto = o.step(dto)
        dtg = s.advance_solution(step, dtg)
        dts_o.append(dto)
        dts_g.append(dtg)
    assert np.allclose(dts_o, dts_g, rtol=1e-13, atol=0)
    _compare_state(o, s, 3, RTOL_RUN)


def test_step_channel_small(fen_lib):
    # channel form (walls in y, x/z periodic, anisotropic spacing, body force g(1))
    n = (32, 16, 24)
    L = (4 * np.pi, 2.0, 4 * np.pi / 3)
    bc = BC_SETS_3D["pnp"]
    o, s = pair(3, n, L, bc=bc, aniso=True, viscosity=1.0 / 180, g=(1.0, 0.0, 0.0), cfl=0.5,
                constant_cfl=True)
    rng = np.random.Generator(np.random.PCG64(1234))
    d = o.delta()
    yc = -1.0 + (np.arange(n[1] + 2) - 0.5) * d[1]
    u = np.zeros(s.grid.shape)
    u[1:-1, 1:-1, 1:-1] = ((1 - yc[1:-1] ** 2) / (2 * (1.0 / 180)))[None, :, None]
    Uc = 90.0
    vel = [u, np.zeros(s.grid.shape), np.zeros(s.grid.shape)]
    for a in vel:
        a[1:-1, 1:-1, 1:-1] += 0.05 * Uc * rng.uniform(-1, 1, size=(n[2], n[1], n[0]))
    for fid, a in zip((O.U, O.V, O.W), vel):
        load_both(o, s, fid, a)
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)
    dto = o.set_timestep(Uc)
    dtg = s.set_timestep(Uc)
    for step in range(1, 11):
        dto = o.step(dto)
        dtg = s.advance_solution(step, dtg)
    assert abs(dto - dtg) <= 1e-13 * dto
    _compare_state(o, s, 3, RTOL_RUN)


def test_step_lid_driven_walls(fen_lib):
    # lid-driven cavity form (lid_driven.f90:35-59): walls everywhere, u = 1 on the top
    N = 32
    o, s = pair(2, (N, N, 1), (1.0, 1.0, 1.0 / N), bc=[O.WALL] * 4, viscosity=1e-2)
    top = o.bc_values(O.U, 3)
    top[...] = 1.0
    s.set_bc_values(F.U, F.TOP, np.ones(top.shape))
    for fid in (O.U, O.V, O.P):
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)
    dto = o.set_timestep(1.0)
    dtg = s.set_timestep(1.0)
    assert dto == dtg
    for step in range(1, 31):
        o.step(dto)
        s.advance_solution(step, dtg)
    _compare_state(o, s, 2, RTOL_RUN)


def test_step_poiseuille_inflow_outflow(fen_lib):
    # navier_stokes/poiseuille_io (poiseuille_io.f90:27-60): walls in x, Inflow at the
    # bottom with v = -x(x-1)/2, Outflow at the top (phi Dirichlet there, b(ny) - c(ny) in
    # the tridiagonal, poisson.f90:225-230); nu = 1 (module default); nn solver
    Nx, Ny = 16, 64
    Lx, Ly = 1.0, 4.0
    bc = [O.WALL, O.WALL, O.INFLOW, O.OUTFLOW]
    o, s = pair(2, (Nx, Ny, 1), (Lx, Ly, Ly / Ny), bc=bc)
    assert s.status()["poisson_solver"] == "nn"
    vin = o.bc_values(O.V, 2)
    xc = (np.arange(Nx + 2) - 0.5) * (Lx / Nx)
    vin[...] = (-0.5 * (xc ** 2 - xc))[None, :]
    s.set_bc_values(F.V, F.BOTTOM, vin.copy())
    for fid in (O.U, O.V, O.P):
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)
    dto = o.set_timestep(1.0)
    dtg = s.set_timestep(1.0)
    for step in range(1, 31):
        o.step(dto)
        s.advance_solution(step, dtg)
    assert np.all(np.isfinite(o.field(O.V)))
    _compare_state(o, s, 2, RTOL_RUN)


@pytest.mark.parametrize("n", [(24, 48, 1), (96, 96, 1), (48, 24, 36)])
def test_step_radix3_sizes(fen_lib, n):
    dim = 2 if n[2] == 1 else 3
    L = (2 * np.pi,) * 3
    o, s = pair(dim, n, L, viscosity=0.05, aniso=True)
    rng = np.random.Generator(np.random.PCG64(77))
    fids = [O.U, O.V] if dim == 2 else [O.U, O.V, O.W]
    for fid in fids:
        a = C.random_interior(s.grid.shape, rng, dim) * 0.5
        load_both(o, s, fid, a)
        o.update_ghost_nodes(fid)
        s.update_ghost_nodes(fid)
    dt = 1e-3
    o.dt_o = dt
    s.set_dt_o(dt)
    o.run(5, dt)
    s.advance_n(5, dt)
    _compare_state(o, s, dim, RTOL_RUN)


def test_nan_is_reported_not_faulted(fen_lib):
    N = 16
    g = F.Grid(N, N, 1, 1.0, 1.0, 1.0 / N)
    s = F.Solver(g)
    a = s.zeros()
    a[1, 5, 5] = np.nan
    s.set_field(F.U, a)
    s.set_dt_o(1e-3)
    with pytest.raises(F.FenError, match="NaN"):
        s.advance_solution(1, 1e-3)
    # the context stays usable once the state (including the AB2 history dv_o, which
    # carries the NaN as it would in the reference) is re-initialised
    for fid in (F.U, F.V, F.P, F.DVO_X, F.DVO_Y):
        s.set_field(fid, s.zeros(fid))
    s.advance_solution(2, 1e-3)


def test_errors_are_codes(fen_lib):
    with pytest.raises(F.FenError, match="fen error -2"):
        F.Solver(F.Grid(8, 8, 8, 1, 1, 1, bc=["Wall", "Wall"] + ["Periodic"] * 4))
    with pytest.raises(F.FenError, match="fen error -1"):
        F.Solver(F.Grid(10, 10, 1, 1, 1, 0.1))  # 10 is not 2^a 3^b
    g = F.Grid(8, 8, 1, 1.0, 1.0, 1.0 / 8)
    s = F.Solver(g)
    with pytest.raises(F.FenError, match="fen error -6"):
        s.advance_solution(1, 1e-3)  # no set_timestep yet


def test_launch_counter(fen_lib):
    g = F.Grid(16, 16, 1, 1.0, 1.0, 1.0 / 16)
    s = F.Solver(g)
    s.set_dt_o(1e-3)
    before = s.kernel_launches()
    s.advance_n(3, 1e-3)
    per = (s.kernel_launches() - before) / 3
    assert per >= 8


def test_get_field_into_caller_buffer(fen_lib):
    # download into a caller-owned buffer (the Fortran host array / a pinned buffer) gives the
    # same bytes as a fresh array; wrong shapes and dtypes are rejected
    g = F.Grid(16, 12, 8, 1.0, 1.0, 1.0)
    s = F.Solver(g)
    rng = np.random.Generator(np.random.PCG64(3))
    a = rng.standard_normal(g.shape)
    s.set_field(F.U, a)
    out = np.empty(g.shape)
    got = s.get_field(F.U, out=out)
    assert got is out and np.array_equal(out, s.get_field(F.U))
    with pytest.raises(ValueError):
        s.get_field(F.U, out=np.empty(g.shape, dtype=np.float32))


def test_invalid_time_steps_rejected(fen_lib):
    g = F.Grid(16, 16, 1, 1.0, 1.0, 1.0 / 16)
    s = F.Solver(g)
    for bad in (0.0, -1e-3, float("nan"), float("inf")):
        with pytest.raises(F.FenError, match="dt_o"):
            s.set_dt_o(bad)
    s.set_dt_o(1e-3)
    for bad in (0.0, -1e-3, float("nan")):
        with pytest.raises(F.FenError, match="dt must be positive"):
            s.advance_solution(1, bad)
        with pytest.raises(F.FenError, match="dt must be positive"):
            s.advance_n(2, bad)
    with pytest.raises(F.FenError, match="U must be"):
        s.set_timestep(-1.0)
    # the context stays usable
    s.advance_n(2, 1e-3)
    assert not s.status()["nan"]
