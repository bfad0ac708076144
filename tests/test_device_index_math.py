"""CPU restatements of the integer and index arithmetic the CUDA kernels rely on.

Like test_conversions.py, these apply the device formulas to Python/numpy integers and check
them against exact references:

* the multiply-high division of the transforms (fft_magic / FastDiv in
  fen_gb300/csrc/fen_fft.cuh): multiplier floor(2^32/d) + 1 formed in 32-bit arithmetic,
  exact for n * d < 2^32;
* the mixed-radix Stockham schedule (16 or 8 first, then at most one 4 and one 2, then 3s)
  with radix-8 and radix-16 butterflies composed as 4 x 2 and 4 x 4 with exact 16th-root
  rotations, against numpy.fft for every length 2^a 3^b the line kernels take;
* the incremental cell walk of the grid-stride loops (CellWalk in fen_types.cuh);
* the order-preserving int64 keys and NaN test of the FP64 diagnostics (okey / nan_bits in
  fen_kernels.cuh);
* the ghost fills' work-index mappings (ghost_target, ghost_target_fast, and the v* fill of
  only the faces the divergence reads, ghost_low_target, in fen_ghost.cuh).
"""
import cmath
import math

import numpy as np
import pytest


def fft_magic(d):
    if d <= 1:
        return 0
    return (0xFFFFFFFF // d + 1 + (1 if (d & (d - 1)) == 0 else 0)) & 0xFFFFFFFF


def fdiv(n, d):
    return n if d <= 1 else (n * fft_magic(d)) >> 32


def test_fast_division_exact():
    rng = np.random.Generator(np.random.PCG64(0))
    for d in list(range(1, 600)) + [768, 1024, 1025, 2048, 3072, 4097]:
        assert d <= 1 or fft_magic(d) == 2 ** 32 // d + 1
        top = (2 ** 32 - 1) // d
        ns = np.unique(np.concatenate([np.arange(0, min(top, 5000)), rng.integers(0, top, 2000), [top]]))
        for n in ns:
            assert fdiv(int(n), d) == int(n) // d, (n, d)


def plan(M, maxr):
    R, m = [], M
    if maxr >= 16:
        while m % 16 == 0:
            R.append(16)
            m //= 16
    if maxr >= 8:
        while m % 8 == 0:
            R.append(8)
            m //= 8
    while m % 4 == 0:
        R.append(4)
        m //= 4
    if m % 2 == 0:
        R.append(2)
        m //= 2
    while m % 3 == 0:
        R.append(3)
        m //= 3
    assert m == 1
    return R


def cos16(m):
    return math.cos(2 * math.pi * (m % 16) / 16)


def rot16(sign, R, v, m):
    e = (m * (16 // R)) % 16
    c, s = cos16(e), sign * cos16(e + 12)
    return complex(v.real * c - v.imag * s, v.real * s + v.imag * c)


def dft_r(sign, R, x):
    if R in (2, 3, 4):
        x[:R] = [sum(x[n] * cmath.exp(sign * 2j * math.pi * n * k / R) for n in range(R)) for k in range(R)]
        return
    A, B = (4, 2) if R == 8 else (4, 4)
    y = [0j] * (A * B)
    for n2 in range(B):
        t = [x[B * n1 + n2] for n1 in range(A)]
        dft_r(sign, A, t)
        for k1 in range(A):
            y[n2 * A + k1] = rot16(sign, A * B, t[k1], n2 * k1)
    for k1 in range(A):
        t = [y[n2 * A + k1] for n2 in range(B)]
        dft_r(sign, B, t)
        for k2 in range(B):
            x[k1 + A * k2] = t[k2]


def stockham(x, sign, maxr, nl=1):
    """One transform per line of x (nl lines, line-fastest like the kernels)."""
    M = x.shape[0]
    a = [complex(v) for v in x.ravel(order="C")]
    b = [0j] * len(a)
    w = [cmath.exp(-2j * math.pi * m / M) for m in range(M)]
    Ns = 1
    for R in plan(M, maxr):
        nb, tstep = M // R, M // (Ns * R)
        p2 = (Ns & (Ns - 1)) == 0
        for t in range(nl * nb):
            j = fdiv(t, nl)
            line = t - j * nl
            k = (j & (Ns - 1)) if p2 else j - fdiv(j, Ns) * Ns
            v = [a[(j + q * nb) * nl + line] for q in range(R)]
            if Ns > 1:
                for q in range(1, R):
                    tw = w[q * k * tstep]
                    v[q] = v[q] * (tw if sign < 0 else tw.conjugate())
            dft_r(sign, R, v)
            o = (j - k) * R + k
            for q in range(R):
                b[(o + q * Ns) * nl + line] = v[q]
        a, b = b, a
        Ns *= R
    return np.array(a).reshape(M, nl)


@pytest.mark.parametrize("M", [2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512])
def test_stockham_schedule_matches_numpy(M):
    rng = np.random.Generator(np.random.PCG64(M))
    nl = 3
    x = rng.standard_normal((M, nl)) + 1j * rng.standard_normal((M, nl))
    want_f = np.fft.fft(x, axis=0)
    want_b = np.fft.ifft(x, axis=0) * M
    scale = np.abs(want_f).max()
    for maxr in (4, 8, 16):
        assert np.abs(stockham(x, -1, maxr, nl) - want_f).max() < 1e-12 * scale
        assert np.abs(stockham(x, +1, maxr, nl) - want_b).max() < 1e-12 * scale


def cell_walk(n0, n1, t0, s, ncell):
    r = t0 // n0
    i, j, k = t0 - r * n0, r % n1, r // n1
    r = s // n0
    si, sj, sk = s - r * n0, r % n1, r // n1
    t = t0
    while t < ncell:
        yield t, i, j, k
        t += s
        i += si
        c = int(i >= n0)
        i -= n0 * c
        j += sj + c
        c = int(j >= n1)
        j -= n1 * c
        k += sk + c


@pytest.mark.parametrize("n", [(256, 256, 256), (512, 256, 384), (96, 64, 1), (7, 5, 3), (1, 1, 1), (33, 1, 2)])
def test_cell_walk_matches_division(n):
    n0, n1, n2 = n
    ncell = n0 * n1 * n2
    rng = np.random.Generator(np.random.PCG64(ncell))
    for grid in (1, 3, 152 * 4, 152 * 16):
        s = grid * 256
        for t0 in rng.integers(0, min(s, ncell), 6):
            for t, i, j, k in cell_walk(n0, n1, int(t0), s, ncell):
                assert (i, j, k) == (t % n0, (t // n0) % n1, t // (n0 * n1))


def okey(b):
    b = np.asarray(b, dtype=np.int64)
    return b ^ ((b >> 63) & np.int64(0x7FFFFFFFFFFFFFFF))


def nan_bits(b):
    return (np.asarray(b, dtype=np.int64) & np.int64(0x7FFFFFFFFFFFFFFF)) > np.int64(0x7FF0000000000000)


def test_order_preserving_keys_and_nan_bits():
    rng = np.random.Generator(np.random.PCG64(5))
    x = np.concatenate([rng.standard_normal(50000) * 10.0 ** rng.integers(-300, 300, 50000),
                        [0.0, -0.0, np.inf, -np.inf, 5e-324, -5e-324, np.finfo(float).max, -np.finfo(float).max]])
    bits = x.view(np.int64)
    k = okey(bits)
    # sorting by key sorts by value (-0 lands just below +0)
    assert np.all(np.diff(x[np.argsort(k, kind="stable")]) >= 0)
    # the map is its own inverse, so the reduced key converts back to the maximum
    assert np.array_equal(okey(k), bits)
    assert x[np.argmax(k)] == x.max() and x[np.argmin(k)] == x.min()
    # NaNs of either sign and any payload are caught; no finite or infinite value is
    assert not nan_bits(bits).any()
    nan = np.array([0x7FF8000000000000, 0x7FF0000000000001, 0xFFF8000000000000 - 2 ** 64,
                    0xFFFFFFFFFFFFFFFF - 2 ** 64], dtype=np.int64)
    assert nan_bits(nan).all() and np.isnan(nan.view(np.float64)).all()


# ---- ghost fill: work index -> ghost cell (ghost_count / ghost_target / ghost_div /
# ghost_target_fast in fen_gb300/csrc/fen_ghost.cuh) ----

def _ghost_count(dim, n0, n1, n2, c, right, top, back):
    xov = int(c == "x" and right == "D")
    yov = int(c == "y" and top == "D")
    zov = int(dim == 3 and c == "z" and back == "D")
    nk = n2 - zov if dim == 3 else 1
    a = (2 + xov) * (n1 - yov) * nk
    b = (2 + yov) * (n0 + 2) * nk
    cc = (2 + zov) * (n0 + 2) * (n1 + 2) if dim == 3 else 0
    return a, b, cc, xov, yov, zov, nk


def _ghost_target(dim, n0, n1, n2, c, right, top, back, t):
    a, b, cc, xov, yov, zov, nk = _ghost_count(dim, n0, n1, n2, c, right, top, back)
    if t < a:
        w = 2 + xov
        s, r = t % w, t // w
        j, k = 1 + r % (n1 - yov), 1 + r // (n1 - yov)
        return (0 if s == 0 else n0 + 1 if s == 1 else n0), j, k
    t -= a
    if t < b:
        ni = n0 + 2
        i, r = t % ni, t // ni
        w = 2 + yov
        s, k = r % w, 1 + r // w
        return i, (0 if s == 0 else n1 + 1 if s == 1 else n1), k
    t -= b
    ni, nj = n0 + 2, n1 + 2
    i, r = t % ni, t // ni
    j, s = r % nj, r // nj
    return i, j, (0 if s == 0 else n2 + 1 if s == 1 else n2)


def _ghost_fast(dim, n0, n1, n2, c, right, top, back):
    """ghost_div's validity test and ghost_target_fast's 32-bit multiply-high mapping."""
    a, b, cc, xov, yov, zov, nk = _ghost_count(dim, n0, n1, n2, c, right, top, back)
    wa, na, ni, wb, nj = 2 + xov, n1 - yov, n0 + 2, 2 + yov, n1 + 2
    lim = 2 ** 32
    ok = (a * wa < lim and (a // wa + 1) * na < lim and b * ni < lim and (b // ni + 1) * wb < lim
          and cc * ni < lim and (cc // ni + 1) * nj < lim)

    def target(t):
        if t < a:
            r = fdiv(t, wa)
            s = t - r * wa
            q = fdiv(r, na)
            return (0 if s == 0 else n0 + 1 if s == 1 else n0), 1 + r - q * na, 1 + q
        t -= a
        if t < b:
            r = fdiv(t, ni)
            q = fdiv(r, wb)
            s = r - q * wb
            return t - r * ni, (0 if s == 0 else n1 + 1 if s == 1 else n1), 1 + q
        t -= b
        r = fdiv(t, ni)
        q = fdiv(r, nj)
        return t - r * ni, r - q * nj, (0 if q == 0 else n2 + 1 if q == 1 else n2)

    return ok, a + b + cc, target


@pytest.mark.parametrize("dim,n", [(3, (12, 16, 10)), (3, (24, 6, 9)), (2, (32, 24, 1)), (3, (2, 2, 2)),
                                   (2, (3, 2, 1))])
@pytest.mark.parametrize("c", ["x", "y", "z", "c"])
@pytest.mark.parametrize("walls", ["PPP", "DDD", "PDP", "DPD"])
def test_ghost_target_fast_matches(dim, n, c, walls):
    right, top, back = walls
    ok, total, fast = _ghost_fast(dim, *n, c, right, top, back)
    assert ok
    for t in range(total):
        assert fast(t) == _ghost_target(dim, *n, c, right, top, back, t), t


def test_ghost_fast_bound_covers_bench_grids():
    # the 512 x 256 x 384 channel and the 256^3 box take the fast mapping; 4096^3 does not
    for n in [(512, 256, 384), (256, 256, 256), (1024, 1024, 1024)]:
        for c in "xyzc":
            ok, total, fast = _ghost_fast(3, *n, c, "P", "D", "P")
            assert ok
            for t in [0, 1, total // 3, total // 2, total - 1]:
                assert fast(t) == _ghost_target(3, *n, c, "P", "D", "P", t)
    assert not _ghost_fast(3, 4096, 4096, 4096, "x", "P", "P", "P")[0]


# ---- ghosts of v* after the predictor (ghost_low_count / ghost_low_target in
# fen_gb300/csrc/fen_ghost.cuh): the divergence's minus neighbours plus the last face a
# wall overwrites ----

def _ghost_low_count(dim, n0, n1, n2, c, right, top, back):
    face = {"x": n1 * n2, "y": n0 * n2, "z": n0 * n1}[c]
    hi = {"x": right, "y": top, "z": back}[c]
    return face * (2 if hi == "D" else 1)


def _ghost_low_target(n0, n1, n2, c, t):
    face = {"x": n1 * n2, "y": n0 * n2, "z": n0 * n1}[c]
    high = t >= face
    u = t - face if high else t
    if c == "x":
        return (n0 if high else 0), 1 + u % n1, 1 + u // n1
    if c == "y":
        return 1 + u % n0, (n1 if high else 0), 1 + u // n0
    return 1 + u % n0, 1 + u // n0, (n2 if high else 0)


@pytest.mark.parametrize("dim,n", [(3, (12, 16, 10)), (3, (24, 6, 9)), (2, (32, 24, 1)), (2, (3, 2, 1))])
@pytest.mark.parametrize("walls", ["PPP", "DDD", "PDP", "DPD"])
def test_ghost_low_faces_cover_what_the_divergence_reads(dim, n, walls):
    # the cells filled are exactly the minus neighbours the divergence of cell (1..n0, 1..n1,
    # 1..n2) reads outside the interior computed by the predictor, plus the face-normal wall
    # face, each once; all of them are ghosts of the full fill (the same rule evaluates there)
    right, top, back = walls
    n0, n1, n2 = n
    comps = ["x", "y"] + (["z"] if dim == 3 else [])
    for c in comps:
        total = _ghost_low_count(dim, n0, n1, n2, c, right, top, back)
        cells = [_ghost_low_target(n0, n1, n2, c, t) for t in range(total)]
        assert len(set(cells)) == total
        ks = range(1, n2 + 1) if dim == 3 else [1]
        want = set()
        for k in ks:
            for j in range(1, n1 + 1):
                for i in range(1, n0 + 1):
                    m = {"x": (i - 1, j, k), "y": (i, j - 1, k), "z": (i, j, k - 1)}[c]
                    if m[{"x": 0, "y": 1, "z": 2}[c]] == 0:
                        want.add(m)
        hi = {"x": right, "y": top, "z": back}[c]
        if hi == "D":
            for k in ks:
                for j in range(1, n1 + 1):
                    for i in range(1, n0 + 1):
                        want.add({"x": (n0, j, k), "y": (i, n1, k), "z": (i, j, n2)}[c])
        assert set(cells) == want, c
        full_total = sum(_ghost_count(dim, n0, n1, n2, c, right, top, back)[:3])
        full = {_ghost_target(dim, n0, n1, n2, c, right, top, back, t) for t in range(full_total)}
        assert set(cells) <= full, c
