"""The learned proposal's network on the tensor cores against the CPU oracle (oracle/mlp_oracle.py):
forward logits and training gradients, through the C-ABI (pp_mlp_forward, pp_mlp_grad)."""
import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _params(seed, out_scale=0.5):
    rng = np.random.default_rng(seed + 100)
    P = mo.init_params(seed=seed, out_scale=out_scale)
    P[mo.OFF_B1:mo.OFF_W2] = rng.normal(0, 0.2, mo.HID)
    P[mo.OFF_B2:mo.OFF_W3] = rng.normal(0, 0.2, mo.HID)
    P[mo.OFF_B3:] = rng.normal(0, 0.3, mo.OUT)
    return P.astype(np.float32)


@pytest.mark.parametrize("n", [1, 127, 128, 129, 1000, 4096])
def test_forward_matches_oracle(built, n):
    P = _params(1)
    X = mo.random_samples(n, seed=n)[:, :mo.IN]
    z = pp.mlp_forward(P, X)
    zr = mo.forward(P, X)
    # tensor-core FP32 accumulation order differs from the oracle's; a hidden activation then rounds to
    # the neighbouring BF16 value now and then, which moves a logit by ~1e-3 at most
    err = np.abs(z - zr)
    assert err.max() <= 1e-2 * (1 + np.abs(zr).max()), err.max()
    assert np.median(err) <= 1e-4 * (1 + np.abs(zr).max())


def test_forward_is_row_independent(built):
    """A row's logits do not depend on the other rows of its 128-row tile (exactness of the MH ratio
    relies on the network being a function of the particle's own features)."""
    P = _params(2)
    X = mo.random_samples(256, seed=9)[:, :mo.IN]
    z1 = pp.mlp_forward(P, X)
    X2 = X.copy()
    X2[1::2] = mo.random_samples(128, seed=10)[:, :mo.IN]
    z2 = pp.mlp_forward(P, X2)
    assert np.array_equal(z1[0::2], z2[0::2])
    z3 = pp.mlp_forward(P, X[:1])
    assert np.array_equal(z3[0], z1[0])


@pytest.mark.parametrize("n,tpc", [(128, 1), (1000, 1), (4096, 4), (3000, 3)])
def test_gradient_matches_oracle(built, n, tpc):
    P = _params(3)
    S = mo.random_samples(n, seed=n + 7)
    g, J = pp.mlp_grad(P, S, floor=0.1, tau=0.02, tiles_per_cta=tpc)
    gr, Jr = mo.grad(P, S, 0.1, 0.02)
    assert abs(J - Jr) <= 1e-3 * (1 + abs(Jr))
    for name, lo, hi in (("W1", mo.OFF_W1, mo.OFF_B1), ("b1", mo.OFF_B1, mo.OFF_W2), ("W2", mo.OFF_W2, mo.OFF_B2), ("b2", mo.OFF_B2, mo.OFF_W3),
                         ("W3", mo.OFF_W3, mo.OFF_B3), ("b3", mo.OFF_B3, mo.NPARAMS)):
        a, b = g[lo:hi].astype(np.float64), gr[lo:hi]
        scale = np.abs(b).max() + 1e-12
        # same BF16 operands; FP32 accumulation order and the odd neighbouring-BF16 rounding differ
        assert np.abs(a - b).max() <= 3e-2 * scale, (name, np.abs(a - b).max(), scale)
        assert np.linalg.norm(a - b) <= 1e-2 * np.linalg.norm(b), name


def test_gradient_of_zero_utilities_with_no_entropy_is_zero(built):
    P = _params(4)
    S = mo.random_samples(300, seed=1)
    S[:, mo.IN:] = 0
    g, J = pp.mlp_grad(P, S, floor=0.1, tau=0.0)
    assert np.all(g == 0) and J == 0


def test_tensor_core_wait_that_runs_out_is_reported_and_the_gpu_stays_usable(built):
    """The bounded mbarrier wait of the network's kernels: with an arrival it completes; with none (no
    tensor-core work issued, a barrier nothing arrives at) it gives up after its limit, the host reads
    PP_ERR_CUDA, and the context still runs the network."""
    limit = 2_000_000  # ~1 ms at the SM clock
    rc, gave_up, cycles = pp.mlp_wait_test(limit, arrive=True)
    assert rc == pp.PP_OK and not gave_up and 0 <= cycles < limit
    rc, gave_up, cycles = pp.mlp_wait_test(limit, arrive=False)
    assert rc == pp.PP_ERR_CUDA and gave_up and cycles > limit
    P = _params(3)
    X = mo.random_samples(300, seed=5)[:, :mo.IN]
    z = pp.mlp_forward(P, X)
    zr = mo.forward(P, X)
    assert np.abs(z - zr).max() <= 1e-2 * (1 + np.abs(zr).max())
