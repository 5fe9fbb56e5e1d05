"""GPU sweeps: determinism, FP32-guard vs FP64 identity, energy bookkeeping, NPT, batched replicas."""
import numpy as np
import pytest

from tests import helpers
import patchyparticles_gb300 as pp
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def run(r, R, box, sweeps, **kw):
    e = pp.Engine(pp.default_params(**kw))
    e.upload(r, R, box)
    e.sweeps(sweeps)
    e.sync()
    out = e.download()
    res = dict(state=out, E=e.tracked_energy(), counters=e.counters(), guard=e.guard_stats(), box=e.box())
    e.close()
    return res


def oracle_energy(r, R, box):
    s = po.System(po.params(), arrays=(r, R, box))
    return s.init_energy()


def test_deterministic(built):
    r, R, box = helpers.config("c2")
    a = run(r, R, box, 10, seed=11)
    b = run(r, R, box, 10, seed=11)
    for x, y in zip(a["state"], b["state"]):
        assert np.array_equal(x, y)
    c = run(r, R, box, 10, seed=12)
    assert not np.array_equal(a["state"][0], c["state"][0])


@pytest.mark.parametrize("name,T", [("c2", 0.13), ("c5", 0.11), ("c3", 0.1)])
def test_fp32_guard_and_fp64_trajectories_identical(built, name, T):
    """Identical decisions for every pair -> bit-identical trajectories of the two precisions."""
    r, R, box = helpers.config(name)
    a = run(r, R, box, 30, temperature=T, precision=pp.PREC_FP32_GUARD, audit=1)
    b = run(r, R, box, 30, temperature=T, precision=pp.PREC_FP64)
    assert a["guard"]["mismatches"] == 0
    for x, y in zip(a["state"], b["state"]):
        assert np.array_equal(x, y)
    assert a["E"] == b["E"]
    assert a["counters"] == b["counters"]


@pytest.mark.parametrize("name,T", [("c1", 0.12), ("c2", 0.13), ("c5", 0.11), ("fcc", 0.12)])
def test_tracked_energy_equals_reference_energy_after_sweeps(built, name, T):
    """After sweeps the reference's routines, run on the downloaded state, find no overlap and the same energy."""
    r, R, box = helpers.config(name)
    res = run(r, R, box, 50, temperature=T)
    r2, R2, b2 = res["state"]
    E, ov = oracle_energy(r2, R2, b2)
    assert not ov
    assert E == res["E"]
    tries, acc = res["counters"]
    N = len(r)
    # one attempt per non-empty cell per checkerboard round: between 10% and 100% of N per sweep
    assert 0.1 * 50 * N < tries[0] <= 50 * N
    assert 0 < acc[0] < tries[0]
    # orientations stay orthonormal (FP64 accumulation)
    M = R2.reshape(-1, 3, 3)
    assert np.abs(np.einsum("nij,nkj->nik", M, M) - np.eye(3)).max() < 1e-13


def test_moves_are_small_and_local(built):
    r, R, box = helpers.config("c5")
    res = run(r, R, box, 1, disp_max=0.05)
    r2, _, _ = res["state"]
    d = np.abs(r2 - r)
    # one round per sweep, at most one attempt per particle per round, displacement in [-Disp_max/2, Disp_max/2)
    assert d.max() <= 0.025 + 1e-12
    assert (d.max(axis=1) > 0).sum() > 0.2 * len(r)


@pytest.mark.parametrize("name", ["c5", "small"])
def test_npt_volume_moves(built, name):
    r, R, box = helpers.config(name)
    res = run(r, R, box, 100, ensemble=pp.NPT, temperature=0.11, pressure=0.05, rescale_factor_max=0.01)
    tries, acc = res["counters"]
    assert tries[pp.MOVE_VOLUME] == 100
    assert 0 < acc[pp.MOVE_VOLUME] <= 100
    r2, R2, b2 = res["state"]
    assert not np.array_equal(b2, box)
    E, ov = oracle_energy(r2, R2, b2)
    assert not ov and E == res["E"]


def test_batch_replicas_equal_single_runs(built):
    confs = [helpers.config(n) for n in ("c1", "c3", "small")]
    prms = [pp.default_params(temperature=T, seed=s, kf_cosmax=c) for T, s, c in ((0.12, 5, 0.92), (0.09, 6, 0.9), (0.2, 7, 0.95))]
    e = pp.Engine(prms)
    for i, (r, R, box) in enumerate(confs):
        e.upload(r, R, box, replica=i)
    e.sweeps(20)
    e.sync()
    for i, (r, R, box) in enumerate(confs):
        p = prms[i]
        single = run(r, R, box, 20, temperature=p.temperature, seed=p.seed, kf_cosmax=p.kf_cosmax)
        got = e.download(i)
        for x, y in zip(got, single["state"]):
            assert np.array_equal(x, y)
        assert e.tracked_energy(i) == single["E"]
    e.close()


def test_check_energy_after_sweeps(built):
    r, R, box = helpers.config("c2")
    e = pp.Engine(pp.default_params(temperature=0.13))
    e.upload(r, R, box)
    e.sweeps(20)
    e.check_energy()
    E1 = e.tracked_energy()
    assert e.energy() == (E1, False)
    _, R2, _ = e.download()
    M = R2.reshape(-1, 3, 3)
    assert np.abs(np.einsum("nij,nkj->nik", M, M) - np.eye(3)).max() < 1e-15
    e.close()


def test_overlapping_configuration_is_rejected(built):
    r, R, box = helpers.config("c1")
    r = r.copy()
    r[1] = r[0] + np.array([0.5, 0.0, 0.0])
    e = pp.Engine(pp.default_params())
    with pytest.raises(pp.PPError) as ei:
        e.upload(r, R, box)
    assert ei.value.code == pp.PP_ERR_OVERLAP
