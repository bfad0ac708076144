"""The allocation-free entry point fen_poisson_pp2d_noalloc, called through the C ABI.

It exists for callers that cannot allocate device memory: they hand over their own input
and output arrays and the solver works in a static device array instead of cudaMalloc'd
scratch.  Its result must match the regular entry point (fen_solve_poisson on a context
with periodic x and y) to the same 1e-13 relative L2 used for single operators, on two
calls in a row (the second reuses the static scratch the first left behind), and a repeat
call must not change the device's free memory.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import fen_gb300 as F

pytestmark = pytest.mark.gpu

RTOL = 1e-13


def _bind(lib):
    f = lib.fen_poisson_pp2d_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _regular(rhs, lx):
    ny, nx = rhs.shape
    s = F.Solver(F.Grid(nx, ny, 1, lx, lx * ny / nx, lx / nx))
    a = s.zeros()
    a[1, 1:-1, 1:-1] = rhs
    return s.solve_poisson(a)[1, 1:-1, 1:-1].copy()


def test_noalloc_matches_regular_entry(fen_lib):
    import torch

    solve = _bind(fen_lib)
    torch.cuda.init()
    for call, (nx, ny, seed) in enumerate([(64, 48, 1), (96, 128, 2)]):
        rng = np.random.Generator(np.random.PCG64(seed))
        rhs = rng.standard_normal((ny, nx))
        rhs -= rhs.mean()
        lx = 2 * np.pi
        want = _regular(rhs, lx)
        d_rhs = torch.from_numpy(rhs).cuda()
        d_phi = torch.empty_like(d_rhs)
        torch.cuda.synchronize()
        rc = solve(d_rhs.data_ptr(), d_phi.data_ptr(), nx, ny, lx, None)
        assert rc == 0, fen_lib.fen_last_error()
        got = d_phi.cpu().numpy()
        err = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert err < RTOL, (call, err)


def test_noalloc_in_place_and_on_a_caller_stream(fen_lib):
    """rhs and phi may be the same array, and the work goes on the caller's stream."""
    import torch

    solve = _bind(fen_lib)
    nx, ny, lx = 96, 64, 2 * np.pi
    rng = np.random.Generator(np.random.PCG64(4))
    rhs = rng.standard_normal((ny, nx))
    want = _regular(rhs, lx)
    st = torch.cuda.Stream()
    for call in range(2):
        with torch.cuda.stream(st):
            d = torch.from_numpy(rhs).cuda()
        st.synchronize()
        rc = solve(d.data_ptr(), d.data_ptr(), nx, ny, lx, ctypes.c_void_p(st.cuda_stream))
        assert rc == 0, fen_lib.fen_last_error()
        got = d.cpu().numpy()
        err = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert err < RTOL, (call, err)


def test_noalloc_allocates_nothing_and_rejects_large_sizes(fen_lib):
    import torch

    solve = _bind(fen_lib)
    nx, ny, lx = 128, 128, 1.0
    rng = np.random.Generator(np.random.PCG64(3))
    d_rhs = torch.from_numpy(rng.standard_normal((ny, nx))).cuda()
    d_phi = torch.empty_like(d_rhs)
    assert solve(d_rhs.data_ptr(), d_phi.data_ptr(), nx, ny, lx, None) == 0  # first call does the set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert solve(d_rhs.data_ptr(), d_phi.data_ptr(), nx, ny, lx, None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    rc = solve(d_rhs.data_ptr(), d_phi.data_ptr(), 2048, 64, lx, None)
    assert rc == -1
    assert b"FEN_NOALLOC_MAX_N" in fen_lib.fen_last_error()
