"""The persistent round kernel (the 8 colours of a plain round over the neighbour lists in one cooperative
launch, a grid barrier between colours) against one launch per colour: the same trajectory bit for bit
(NVT, NPT, a batch of uneven replicas, a dense system whose pairs need several chunks; stream launches and
graph replays). And its bounded barrier: a barrier that can never complete makes every wait run out, the
next call that reads the state reports it, and the GPU stays usable (fault detection without a fault)."""
import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import pyoracle as po
from tests.helpers import config

pytestmark = pytest.mark.gpu


def _run(persist, graphs, names, ens=pp.NVT, temps=(0.11,), sweeps=(37, 8, 3)):
    prm = [pp.default_params(temperature=temps[k % len(temps)], ensemble=ens, pressure=0.05, rescale_factor_max=0.01, seed=77 + k)
           for k in range(len(names))]
    e = pp.Engine(prm)
    e.set_persistent(persist)
    e.set_graphs(graphs)
    for k, n in enumerate(names):
        e.upload(*config(n), replica=k)
    for n in sweeps:
        e.sweeps(n)
    e.sync()
    out = []
    for k in range(len(names)):
        out.append(e.download(k) + (e.tracked_energy(k), e.counters(k)))
    e.close()
    return out


@pytest.mark.parametrize("graphs", [False, True])
@pytest.mark.parametrize("names,ens,temps", [
    (("c5",), pp.NVT, (0.11,)),
    (("c5",), pp.NPT, (0.11,)),
    (("c2",), pp.NVT, (0.13,)),  # rho = 0.5: more listed pairs per warp iteration than one chunk holds
    (("c1", "c3", "small"), pp.NVT, (0.12, 0.2, 0.09)),
])
def test_persistent_round_equals_one_launch_per_colour(built, graphs, names, ens, temps):
    a = _run(False, graphs, names, ens, temps)
    b = _run(True, graphs, names, ens, temps)
    for x, y in zip(a, b):
        for u, v in zip(x[:3], y[:3]):
            assert np.array_equal(u, v)
        assert x[3] == y[3] and x[4] == y[4]
        assert x[4][0][0] > 0  # attempts were made


def test_persistent_round_state_agrees_with_the_oracle(built):
    r, R, box = config("c5")
    e = pp.Engine(pp.default_params(temperature=0.11, ensemble=pp.NPT, pressure=0.05, seed=5))
    e.set_persistent(True)
    e.upload(r, R, box)
    e.sweeps(24)
    e.sync()
    r2, R2, b2 = e.download()
    s = po.System(po.params(T=0.11), arrays=(r2, R2, b2))
    E, ov = s.init_energy()
    assert not ov and E == e.tracked_energy()
    e.close()


def test_barrier_wait_that_runs_out_is_reported_and_the_gpu_stays_usable(built):
    r, R, box = config("c5")
    e = pp.Engine(pp.default_params(temperature=0.11, seed=3))
    e.set_persistent(True)
    e.upload(r, R, box)
    # ~1 ms per wait; the first barrier of every round waits for one arrival more than the grid makes
    e.set_barrier_test(limit_cycles=2_000_000, unreachable=True)
    e.sweeps(4)
    with pytest.raises(pp.PPError) as ei:
        e.counters()
    assert ei.value.code == pp.PP_ERR_CUDA and "grid barrier" in str(ei.value)
    e.close()
    # the context is intact: a new engine runs, and its state agrees with the oracle
    e = pp.Engine(pp.default_params(temperature=0.11, seed=4))
    e.upload(r, R, box)
    e.sweeps(8)
    e.sync()
    r2, R2, b2 = e.download()
    s = po.System(po.params(T=0.11), arrays=(r2, R2, b2))
    E, ov = s.init_energy()
    assert not ov and E == e.tracked_energy() and e.counters()[0][0] > 0
    e.close()
