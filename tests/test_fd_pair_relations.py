"""The pair data of the gradient kernels against primitive pairs recomputed from
scratch (no GPU): the seeds of the dual-number kernel (csrc/eri_grad_ad.cuh,
the derivatives of P, P - A, K and A - B along the pair's centres), and the
displaced-pair updates of the finite-difference kernel of (dd|dd)
(csrc/eri_grad_fd.cuh).

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
def test_dual_number_seeds(seed, which):
    """dP/dX, d(P - A)/dX, dK/dX, d(A - B)/dX of the seeds against complex-step derivatives."""
    rng = np.random.default_rng(seed + 10)
    alpha, beta = rng.uniform(0.05, 50.0, size=2)
    A, B = rng.normal(size=3) * 2, rng.normal(size=3) * 2
    K, P, PA, AB = pair(alpha, beta, A, B)
    p = alpha + beta
    mu = alpha * beta / p
    h = 1e-30
    for j in range(3):
        d = np.zeros(3, dtype=complex)
        d[j] = 1j * h
        if which == "A":
            Kc, Pc, PAc, ABc = pair(alpha, beta, A + d, B.astype(complex))
            seed_P, seed_PA, seed_K, seed_AB = alpha / p, -beta / p, -2 * mu * AB[j] * K, 1.0
        else:
            Kc, Pc, PAc, ABc = pair(alpha, beta, A.astype(complex), B + d)
            seed_P, seed_PA, seed_K, seed_AB = beta / p, beta / p, 2 * mu * AB[j] * K, -1.0
        e = np.zeros(3)
        e[j] = 1.0
        assert np.allclose(Pc.imag / h, seed_P * e, rtol=0, atol=1e-14)
        assert np.allclose(PAc.imag / h, seed_PA * e, rtol=0, atol=1e-14)
        assert np.allclose(ABc.imag / h, seed_AB * e, rtol=0, atol=1e-14)
        assert abs(Kc.imag / h - seed_K) <= 1e-13 * max(abs(seed_K), abs(K))


def test_boys_derivative_relation(oracle_lib):
    """dF_m/dT = -F_{m+1}, the Boys seed of the dual-number kernel (oracle's exact Boys)."""
    for T in (1e-3, 0.5, 3.0, 17.0, 40.0):
        for m in range(10):
            h = 1e-5 * max(1.0, T)
            fd = (oracle_lib.boys(T + h, m, oracle_lib.EXACT) - oracle_lib.boys(T - h, m, oracle_lib.EXACT)) / (2 * h)
            assert abs(fd + oracle_lib.boys(T, m + 1, oracle_lib.EXACT)) < 1e-8 * max(1e-3, abs(fd))


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
