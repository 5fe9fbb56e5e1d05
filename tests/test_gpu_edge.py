"""Edge cases the reference handles: an empty system (no attempt at all, energy 0; with N = 0 the loops of
do_NVT / do_NPT, MC.c:19-68, run no iteration) and a single particle (no neighbours: every move that stays in
its cell is accepted), alone and inside a batch with an ordinary replica."""
import numpy as np
import pytest

import patchyparticles_gb300 as pp
from tests.helpers import config
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

BOX = np.array([8.0, 8.0, 8.0])


@pytest.mark.parametrize("ens", [pp.NVT, pp.NPT])
def test_empty_system(built, ens):
    e = pp.Engine(pp.default_params(ensemble=ens, pressure=0.05))
    e.upload(np.zeros((0, 3)), np.zeros((0, 9)), BOX)
    e.sweeps(9)
    e.sync()
    assert e.tracked_energy() == 0 and e.energy() == (0.0, False)
    tries, acc = e.counters()
    assert sum(tries) == 0 and sum(acc) == 0
    r, R, b = e.download()
    assert r.shape == (0, 3) and np.array_equal(b, BOX)
    e.close()


def test_single_particle(built):
    e = pp.Engine(pp.default_params())
    e.upload(np.array([[4.0, 4.0, 4.0]]), np.eye(3).reshape(1, 9), BOX)
    e.sweeps(50)
    e.sync()
    tries, acc = e.counters()
    assert tries[pp.MOVE_ROTO_TRASL] == 50 and acc[pp.MOVE_ROTO_TRASL] >= 45  # one non-empty cell per round
    assert e.tracked_energy() == 0
    r, R, _ = e.download()
    assert np.abs(r[0] - 4.0).max() < 50 * 0.05 and np.allclose(R.reshape(3, 3) @ R.reshape(3, 3).T, np.eye(3), atol=1e-12)
    e.close()


def test_batch_with_an_empty_replica(built):
    r, R, box = config("small")
    e = pp.Engine([pp.default_params(seed=1), pp.default_params(seed=2)])
    e.upload(r, R, box, replica=0)
    e.upload(np.zeros((0, 3)), np.zeros((0, 9)), BOX, replica=1)
    e.sweeps(20)
    e.sync()
    t0, _ = e.counters(0)
    t1, _ = e.counters(1)
    assert t0[pp.MOVE_ROTO_TRASL] > 0 and sum(t1) == 0 and e.tracked_energy(1) == 0
    single = pp.Engine(pp.default_params(seed=1))
    single.upload(r, R, box)
    single.sweeps(20)
    single.sync()
    for x, y in zip(e.download(0), single.download()):
        assert np.array_equal(x, y)
    e.close()
    single.close()


@pytest.mark.parametrize("where", ["position", "orientation", "box"])
def test_non_finite_input_is_refused_and_a_new_upload_recovers(built, where):
    r, R, box = config("c2")
    bad_r, bad_R, bad_box = r.copy(), R.copy(), box.copy()
    if where == "position":
        bad_r[len(r) // 2, 1] = np.nan
    elif where == "orientation":
        bad_R[7, 4] = np.inf
    else:
        bad_box[2] = np.inf
    e = pp.Engine(pp.default_params(temperature=0.2, seed=5))
    e.upload(r, R, box)
    with pytest.raises(pp.PPError) as ei:
        e.upload(bad_r, bad_R, bad_box)
    assert ei.value.code == pp.PP_ERR_ARG and "finite" in ei.value.message
    if where != "box":  # a refused configuration leaves the replica without one
        with pytest.raises(pp.PPError) as ei:
            e.sweeps(1)
        assert ei.value.code == pp.PP_ERR_STATE
    e.upload(r, R, box)
    e.sweeps(4)
    e.sync()
    r2, R2, b2 = e.download()
    s = po.System(po.params(T=0.2), arrays=(r2, R2, b2))
    E, ov = s.init_energy()
    assert not ov and E == e.tracked_energy()
    e.close()
