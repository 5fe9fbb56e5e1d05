"""Captured sweep graphs replay exactly the stream launches: the same trajectory bit for bit (plain, NPT,
learned, audit), with periods and leftover sweeps mixed."""
import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import mlp_oracle as mo
from tests.helpers import config

pytestmark = pytest.mark.gpu


def _run(graphs, ens=pp.NVT, learned=False, audit=0, sweeps=(37, 8, 3)):
    r, R, box = config("c5")
    e = pp.Engine(pp.default_params(temperature=0.11, ensemble=ens, pressure=0.05, audit=audit, seed=77))
    e.set_graphs(graphs)
    e.upload(r, R, box)
    if learned:
        e.learned_init(seed=5)
        e.set_learned_weights(mo.init_params(seed=5, out_scale=2.0))
        e.set_proposal(True)
    for n in sweeps:
        e.sweeps(n)
    e.sync()
    out = e.download() + (e.tracked_energy(), e.counters())
    e.close()
    return out


@pytest.mark.parametrize("ens,learned,audit", [(pp.NVT, False, 0), (pp.NPT, False, 0), (pp.NVT, True, 0), (pp.NPT, True, 0), (pp.NVT, False, 1)])
def test_graph_replay_equals_stream_launches(built, ens, learned, audit):
    a = _run(False, ens, learned, audit)
    b = _run(True, ens, learned, audit)
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert a[3] == b[3] and a[4] == b[4]
