"""The pair-data updates of the finite-difference gradient kernel (csrc/eri_grad_fd.cuh)
against primitive pairs recomputed from scratch at the displaced centre (no GPU).

For exponents alpha (centre A), beta (centre B), p = alpha + beta, mu = alpha beta / p:
moving A by delta gives P' = P + (alpha/p) delta, P' - A' = PA - (beta/p) delta,
A' - B = AB + delta, K' = K exp(-mu (2 AB.delta + |delta|^2)); moving B gives
P' = P + (beta/p) delta, P' - A = PA + (beta/p) delta, A - B' = AB - delta,
K' = K exp(-mu (-2 AB.delta + |delta|^2))."""
import numpy as np
import pytest


def pair(alpha, beta, A, B, c=0.7):
    p = alpha + beta
    AB = A - B
    K = c * np.exp(-alpha * beta / p * AB.dot(AB)) / p
    P = (alpha * A + beta * B) / p
    return K, P, P - A, AB


@pytest.mark.parametrize("seed", range(5))
@pytest.mark.parametrize("which", ["A", "B"])
def test_displaced_pair_updates(seed, which):
    rng = np.random.default_rng(seed)
    alpha, beta = rng.uniform(0.05, 50.0, size=2)
    A, B = rng.normal(size=3) * 2, rng.normal(size=3) * 2
    K, P, PA, AB = pair(alpha, beta, A, B)
    p = alpha + beta
    mu = alpha * beta / p
    for axis in range(3):
        for h in (2e-4, -4e-4):
            d = np.zeros(3)
            d[axis] = h
            if which == "A":
                K2, P2, PA2, AB2 = pair(alpha, beta, A + d, B)
                Kf = K * np.exp(-mu * (2 * AB[axis] * h + h * h))
                Pf = P + alpha / p * d
                PAf = PA - beta / p * d
                ABf = AB + d
            else:
                K2, P2, PA2, AB2 = pair(alpha, beta, A, B + d)
                Kf = K * np.exp(-mu * (-2 * AB[axis] * h + h * h))
                Pf = P + beta / p * d
                PAf = PA + beta / p * d
                ABf = AB - d
            assert abs(Kf - K2) <= 1e-13 * abs(K2)
            assert np.allclose(Pf, P2, rtol=0, atol=1e-13)
            assert np.allclose(PAf, PA2, rtol=0, atol=1e-13)
            assert np.allclose(ABf, AB2, rtol=0, atol=1e-15)


def test_fourth_order_stencil():
    """(8 (f(h) - f(-h)) - (f(2h) - f(-2h))) / (12 h) of a Gaussian-type function at the
    kernel's step: error far below the gradient tolerance."""
    f = lambda x: np.exp(-0.8 * (x - 0.3) ** 2) * (x + 1.1) ** 2
    df = lambda x: np.exp(-0.8 * (x - 0.3) ** 2) * (2 * (x + 1.1) - 1.6 * (x - 0.3) * (x + 1.1) ** 2)
    h = 2e-4
    for x in np.linspace(-2, 2, 9):
        g = (8 * (f(x + h) - f(x - h)) - (f(x + 2 * h) - f(x - 2 * h))) / (12 * h)
        assert abs(g - df(x)) < 1e-10
