"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports every entry
point declared in include/fen_gpu.h.  No compute call is made here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fen_gpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fen_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("fen_ctx_create", "fen_advance_solution", "fen_solve_poisson", "fen_update_ghost_nodes"):
        assert s in syms


def test_library_exports_every_declared_symbol(fen_lib):
    missing = [s for s in declared_symbols() if not hasattr(fen_lib, s)]
    assert not missing, missing


def test_error_path_without_device(fen_lib):
    import fen_gb300 as F

    p = F._Params()
    p.dim, p.nx, p.ny, p.nz = 5, 8, 8, 1
    h = ctypes.c_void_p()
    rc = fen_lib.fen_ctx_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == -1
    assert b"dim" in fen_lib.fen_last_error()


def test_python_api_fails_loudly_when_library_missing(tmp_path):
    import fen_gb300 as F

    with pytest.raises(F.FenError):
        F.load_library(str(tmp_path / "missing.so"))


@pytest.mark.parametrize("field,value,msg", [("lx", 0.0, b"domain lengths"), ("ly", -1.0, b"domain lengths"),
                                             ("density", 0.0, b"density"), ("viscosity", -1.0, b"viscosity"),
                                             ("cfl", 0.0, b"CFL")])
def test_invalid_parameters_rejected_before_device_use(fen_lib, field, value, msg):
    # parameter checks come before any CUDA call, so they run without a device
    import fen_gb300 as F

    p = F._Params()
    p.dim, p.nx, p.ny, p.nz = 2, 8, 8, 1
    p.lx = p.ly = p.lz = 1.0
    p.density, p.viscosity, p.cfl, p.constant_cfl = 1.0, 0.01, 0.5, 1
    setattr(p, field, value)
    h = ctypes.c_void_p()
    assert fen_lib.fen_ctx_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert msg in fen_lib.fen_last_error()


def declared_prototypes():
    """{name: number of arguments} of every entry point in include/fen_gpu.h."""
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for name, args in re.findall(r"\b(fen_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt, flags=re.S):
        a = args.strip()
        out[name] = 0 if a in ("", "void") else a.count(",") + 1
    return out


FORTRAN = os.path.join(ROOT, "fen_gb300", "fortran")


def test_fortran_binding_covers_the_header():
    # the iso_c_binding module (fen_gb300/fortran/fen_gpu_mod.f90) binds every entry point
    # with the C prototype's number of arguments and its C name
    txt = open(os.path.join(FORTRAN, "fen_gpu_mod.f90")).read()
    body = txt[txt.index("module fen_gpu_mod"):txt.index("end module fen_gpu_mod")]
    bound = {}
    for name, args, cname in re.findall(
            r"function\s+(fen_[a-z0-9_]+)\s*\(([^)]*)\)\s*(?:&\s*)?bind\s*\(\s*C\s*,\s*name\s*=\s*'([a-z0-9_]+)'",
            body):
        bound[name] = (0 if not args.strip() else args.count(",") + 1, cname)
    protos = declared_prototypes()
    assert len(protos) >= 50
    missing = [s for s in protos if s not in bound]
    assert not missing, missing
    wrong = {s: (bound[s], protos[s]) for s in protos if bound[s][0] != protos[s] or bound[s][1] != s}
    assert not wrong, wrong


def test_fortran_routing_uses_only_bound_entry_points():
    # the FEN-side routing module calls entry points that fen_gpu_mod binds, and re-points
    # FEN's two procedure pointers
    route = open(os.path.join(FORTRAN, "fen_gpu_route.f90")).read()
    mod = open(os.path.join(FORTRAN, "fen_gpu_mod.f90")).read()
    called = set(re.findall(r"\b(fen_[a-z0-9_]+)\s*\(", route))
    for s in called - {"fen_check"}:
        assert f"function {s}(" in mod, s
    assert "advance_solution => gpu_advance_solution" in route
    assert "solve_poisson => gpu_solve_poisson" in route
    # every module and program unit is closed
    for f in (route, mod):
        assert f.count("module fen_gpu") == 2 * len(re.findall(r"^module ", f, flags=re.M))
