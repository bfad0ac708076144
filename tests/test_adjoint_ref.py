"""CPU checks of the numpy adjoint reference (FP64 adjoint-by-dot-product test)."""
import numpy as np

from tests import adjoint_ref as R


def _rand(rng, n, k=5):
    return [rng.standard_normal((n, n)) for _ in range(k)]


def test_dot_product_identity():
    # <TLM dx, lam> = <dx, ADJ lam> to rounding
    rng = np.random.Generator(np.random.PCG64(3))
    n = 24
    st = R.Step(n, 2 * np.pi, nu=2e-3, dt=2e-3)
    x = _rand(rng, n)
    for _ in range(4):
        dx, lam = _rand(rng, n), _rand(rng, n)
        a = R.dot(st.tangent(x, dx), lam)
        b = R.dot(dx, st.adjoint(x, lam))
        assert abs(a - b) <= 1e-12 * max(abs(a), 1.0)


def test_tangent_matches_finite_differences():
    rng = np.random.Generator(np.random.PCG64(4))
    n = 16
    st = R.Step(n, 2 * np.pi, nu=2e-3, dt=2e-3)
    x = _rand(rng, n)
    dx = _rand(rng, n)
    eps = 1e-6
    xp = [a + eps * b for a, b in zip(x, dx)]
    xm = [a - eps * b for a, b in zip(x, dx)]
    fd = [(a - b) / (2 * eps) for a, b in zip(st.forward(xp), st.forward(xm))]
    tl = st.tangent(x, dx)
    num = np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(fd, tl)))
    den = np.sqrt(sum(np.sum(b ** 2) for b in tl))
    assert num / den < 1e-8
