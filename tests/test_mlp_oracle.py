"""The network oracle itself (CPU): its backward formulas against finite differences, its BF16 rounding
against the definition, and the rounded gradient against the exact one."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5, 0.0, 3.0e-39], dtype=np.float32)
    b = mo.bf16(x)
    # bf16's ulp at 1 is 2^-7: 1 + 2^-8 is the midpoint (a tie, to the even mantissa 1.0), 1 + 3 * 2^-9
    # lies above it, 1 + 2^-9 below it
    assert b[0] == 1.0 and b[1] == 1.0
    assert b[2] == 1.0 + 2 ** -7
    assert b[3] == 1.0
    assert b[4] == -2.5 and b[5] == 0.0
    # every result has a zero low half
    assert np.all((b.view(np.uint32) & 0xFFFF) == 0)
    # and is within half an ulp of bf16
    rel = np.abs(b[:5] - x[:5]) / np.maximum(np.abs(x[:5]), 1e-30)
    assert np.all(rel <= 2 ** -8)


def test_exact_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    P = mo.init_params(seed=1, out_scale=0.3).astype(np.float64)
    P[mo.OFF_B1:mo.OFF_W2] = rng.normal(0, 0.1, mo.HID)
    P[mo.OFF_B2:mo.OFF_W3] = rng.normal(0, 0.1, mo.HID)
    S = mo.random_samples(40, seed=5).astype(np.float64)
    G = mo.grad_exact(P, S, 0.1, 0.05)
    idx = rng.choice(mo.NPARAMS, 60, replace=False)
    idx = np.concatenate([idx, [mo.OFF_B1 + 3, mo.OFF_B2 + 7, mo.OFF_B3, mo.OFF_B3 + 3, mo.OFF_W3 + 5]])
    h = 1e-6
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (mo.loss_exact(Pp, S, 0.1, 0.05) - mo.loss_exact(Pm, S, 0.1, 0.05)) / (2 * h)
        assert abs(fd - G[i]) <= 1e-6 + 1e-4 * abs(G[i]), (i, fd, G[i])


def test_rounded_gradient_close_to_exact():
    P = mo.init_params(seed=2, out_scale=0.5)
    S = mo.random_samples(512, seed=6)
    Gr, J = mo.grad(P, S, 0.1, 0.02)
    Ge = mo.grad_exact(P.astype(np.float64), S.astype(np.float64), 0.1, 0.02)
    # BF16 operands (features, weights, activations, back-propagated errors) cost a few per cent
    for lo, hi in ((mo.OFF_W1, mo.OFF_B1), (mo.OFF_W2, mo.OFF_B2), (mo.OFF_W3, mo.OFF_B3)):
        a, b = Gr[lo:hi], Ge[lo:hi]
        assert np.linalg.norm(a - b) <= 0.1 * np.linalg.norm(b)
        assert np.corrcoef(a, b)[0, 1] > 0.995
    assert np.isfinite(J)


def test_mixture_floor_keeps_the_plain_component():
    z = np.array([[-50.0, 10.0, 10.0, 10.0], [0.0, 0.0, 0.0, 0.0]])
    pi = mo.mixture(z, 0.1)
    assert np.allclose(pi.sum(1), 1.0)
    assert pi[0, 0] >= 0.1 and abs(pi[1, 0] - (0.1 + 0.9 / 4)) < 1e-12
