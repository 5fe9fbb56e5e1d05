"""The learned proposal inside the engine: features against the oracle, exactness of the Metropolis-
Hastings chain (tracked energy and observables against the plain move), collection and training on the
GPU with gradients checked against the oracle."""
import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import mlp_oracle as mo
from oracle import pyoracle as po
from tests.helpers import config

pytestmark = pytest.mark.gpu


def _engine(name="c5", T=0.12, **kw):
    r, R, box = config(name)
    e = pp.Engine(pp.default_params(temperature=T, **kw))
    e.upload(r, R, box)
    return e, (r, R, box)


def _compare_features(f_gpu, f_ref):
    same = np.all(f_gpu == f_ref, axis=1)
    # rows can differ only where two candidates tie exactly in FP32 distance or an FP64 value rounds
    # exactly halfway between two FP32 numbers
    assert same.mean() >= 0.999, same.mean()
    assert np.abs(f_gpu - f_ref).max() <= 1e-5 or (~same).sum() <= 2


def test_features_match_oracle_after_upload(built):
    e, (r, R, box) = _engine()
    e.learned_init()
    f = e.learned_features()
    fr = mo.features(r, R, box, 0.12)
    assert (np.abs(fr).sum(1) > 0).mean() > 0.2  # a real test: many particles have neighbours
    _compare_features(f, fr)
    e.close()


def test_features_follow_the_fp64_state_after_learned_moves(built):
    """After moves the engine's image evaluates R0 . Q(q) in FP32 (deterministic in the FP64 state) where
    the oracle rounds the downloaded FP64 R: equal to ~1e-6, and the same neighbours."""
    e, _ = _engine()
    e.learned_init(seed=3)
    e.set_learned_weights(mo.init_params(seed=3, out_scale=2.0))
    e.set_proposal(True)
    e.sweeps(20)
    r2, R2, b2 = e.download()
    f = e.learned_features()
    fr = mo.features(r2, R2, b2, 0.12)
    close = np.all(np.abs(f - fr) <= 2e-5, axis=1)
    assert close.mean() >= 0.999, close.mean()
    assert np.array_equal(np.abs(f).sum(1) > 0, np.abs(fr).sum(1) > 0) or (~close).sum() <= 3
    e.close()


@pytest.mark.parametrize("name,T,prec", [("c5", 0.12, pp.PREC_FP32_GUARD), ("c2", 0.13, pp.PREC_FP32_GUARD), ("small", 0.11, pp.PREC_FP64)])
def test_learned_sweeps_keep_the_tracked_energy_exact(built, name, T, prec):
    e, _ = _engine(name, T, precision=prec)
    e.learned_init(seed=5)
    e.set_learned_weights(mo.init_params(seed=5, out_scale=2.0))
    e.set_proposal(True)
    e.sweeps(30)
    e.sync()
    r2, R2, b2 = e.download()
    s = po.System(po.params(T=T), arrays=(r2, R2, b2))
    E, ov = s.init_energy()
    assert not ov and E == e.tracked_energy()
    tries, acc = e.learned_stats()
    assert sum(tries) > 0 and 0 < sum(acc) <= sum(tries)
    assert all(t > 0 for t in tries)  # every component is drawn
    t0, a0 = e.counters()
    assert a0[0] == sum(acc)
    e.close()


def test_learned_audit_mode_has_no_mismatches(built):
    e, _ = _engine("c2", 0.13, audit=1)
    e.learned_init(seed=6)
    e.set_learned_weights(mo.init_params(seed=6, out_scale=2.0))
    e.set_proposal(True)
    e.sweeps(5)
    g = e.guard_stats()
    assert g["mismatches"] == 0 and g["pairs"] > 0
    e.close()


def _bonds_series(learned, weights, nrep=16, N=1000, rho=0.3, T=0.2, sweeps=8000, every=20, burn=6000):
    prm = [pp.default_params(temperature=T, seed=100 + k, disp_max=0.1, theta_max=0.2) for k in range(nrep)]
    e = pp.Engine(prm)
    for k in range(nrep):
        r, R, box = pp.generate(N, rho, 700 + k)
        e.upload(r, R, box, replica=k)
    e.learned_init(seed=9, scale_disp=[1, 2, 4, 1], scale_theta=[1, 2, 4, 10])
    e.set_learned_weights(weights)
    e.set_proposal(learned)
    e.sweeps(burn)
    vals = []
    for s in range(0, sweeps, every):
        e.sweeps(every)
        vals.append([-e.tracked_energy(k) / N for k in range(nrep)])
    e.close()
    return np.array(vals)


def test_learned_chain_samples_the_plain_chains_distribution(built):
    """Exactness of the MH correction: with a network whose mixture depends strongly on the environment,
    the equilibrium bonds per particle equal the plain move's within two standard errors (16 independent
    replicas each, 8000 sweeps after 6000 of burn-in; the per-replica time averages are the samples). The
    burn-in is long enough for the plain chain: after 1500 sweeps from the random insertion its bonds per
    particle still rise by ~4 % between the two halves of the run, which biases the comparison towards the
    faster-relaxing learned chain."""
    W = mo.init_params(seed=11, out_scale=3.0)
    W[mo.OFF_B3:] = [0.0, 1.0, 1.5, 0.5]
    a = _bonds_series(False, W)
    b = _bonds_series(True, W)
    ma, mb = a.mean(0), b.mean(0)  # per-replica time averages: independent estimates
    diff = mb.mean() - ma.mean()
    se = np.sqrt(ma.var(ddof=1) / len(ma) + mb.var(ddof=1) / len(mb))
    print("bonds per particle: plain %.5f learned %.5f se %.5f z %.2f" % (ma.mean(), mb.mean(), se, diff / se))
    assert abs(diff) < 2 * se, (ma.mean(), mb.mean(), se)


def test_collect_and_train_on_the_gpu(built):
    e, _ = _engine("c1", 0.12)
    e.learned_init(seed=21, draws=2)
    e.learned_collect(n_configs=40, sweeps_between=2, samples_per_config=128)
    S = e.learned_samples()
    assert S.shape == (40 * 128, mo.SAMPLE)
    assert np.all(np.isfinite(S)) and (S[:, mo.IN:] > 0).any()
    # gradient of the engine's own samples: tensor cores against the oracle
    W0 = e.learned_weights()
    g, J = pp.mlp_grad(W0, S[:1024], floor=0.1, tau=0.01)
    gr, Jr = mo.grad(W0, S[:1024], 0.1, 0.01)
    assert abs(J - Jr) <= 1e-3 * (1 + abs(Jr))
    assert np.linalg.norm(g - gr) <= 2e-2 * np.linalg.norm(gr)
    _, J0 = pp.mlp_grad(W0, S, floor=0.1, tau=0.01)
    obj = e.learned_train(epochs=20, lr=3e-3)
    W1 = e.learned_weights()
    assert np.all(np.isfinite(W1)) and not np.array_equal(W0, W1)
    _, J1 = pp.mlp_grad(W1, S, floor=0.1, tau=0.01)
    assert J1 > J0, (J0, J1, obj)
    e.close()
