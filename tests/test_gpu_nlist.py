"""Per-epoch neighbour lists: the colour pass over the lists makes the decisions of the 27-cell scan, so the
trajectory is the same bit for bit (NVT, NPT with accepted volume moves, re-sort periods 1 to 16, dense and
crystalline configurations, lists forced to overflow, learned moves mid-epoch), and at short periods it tests
fewer pairs. The NPT cases also cover the volume pass over the epoch's flat pair list."""
import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import mlp_oracle as mo
from oracle import pyoracle as po
from tests.helpers import config

pytestmark = pytest.mark.gpu


def _run(name, lists, sweeps=(24, 5), graphs=True, learned_first=0, **kw):
    r, R, box = config(name)
    e = pp.Engine(pp.default_params(**kw))
    e.set_neighbour_lists(lists)
    e.set_graphs(graphs)
    e.upload(r, R, box)
    if learned_first:
        e.learned_init(seed=3)
        e.set_learned_weights(mo.init_params(seed=3, out_scale=2.0))
        e.set_proposal(True)
        e.sweeps(learned_first)
        e.set_proposal(False)
    for n in sweeps:
        e.sweeps(n)
    e.sync()
    out = dict(state=e.download(), E=e.tracked_energy(), counters=e.counters(), guard=e.guard_stats(), box=e.box())
    e.close()
    return out


def _same(a, b):
    for x, y in zip(a["state"], b["state"]):
        assert np.array_equal(x, y)
    assert a["E"] == b["E"] and a["counters"] == b["counters"]
    assert np.array_equal(a["box"], b["box"])


@pytest.mark.parametrize("name,T,ens,P,resort", [
    ("c2", 0.13, pp.NVT, 0.05, 4),
    ("c5", 0.11, pp.NPT, 0.05, 4),
    ("c1", 0.12, pp.NVT, 0.05, 1),
    ("c3", 0.10, pp.NVT, 0.05, 16),
    ("fcc", 0.12, pp.NVT, 0.05, 8),
    ("bcc", 0.12, pp.NVT, 0.05, 2),
    ("small", 0.12, pp.NPT, 2.0, 16),
])
def test_lists_reproduce_the_cell_scan(built, name, T, ens, P, resort):
    kw = dict(temperature=T, ensemble=ens, pressure=P, resort_every=resort, seed=5)
    a = _run(name, False, **kw)
    b = _run(name, True, **kw)
    _same(a, b)
    if resort <= 8:  # at longer periods the radius spans the 27 cells
        assert b["guard"]["pairs"] < a["guard"]["pairs"]
    assert b["guard"]["nl_overflows"] == 0
    if name == "small":
        tries, acc = b["counters"]
        assert acc[pp.MOVE_VOLUME] > 0  # the lists' radius covered accepted rescalings


def test_lists_with_stream_launches_and_odd_sweep_counts(built):
    kw = dict(temperature=0.11, ensemble=pp.NPT, pressure=0.05, seed=9)
    a = _run("c5", False, sweeps=(3, 7, 1, 13), graphs=False, **kw)
    b = _run("c5", True, sweeps=(3, 7, 1, 13), graphs=True, **kw)
    _same(a, b)


def test_overflowing_lists_take_the_exact_path(built, monkeypatch):
    monkeypatch.setenv("PPGPU_NL_CAP", "4")
    kw = dict(temperature=0.13, seed=21)
    a = _run("c2", False, **kw)
    b = _run("c2", True, **kw)
    _same(a, b)
    assert b["guard"]["nl_overflows"] > 0


def test_learned_moves_invalidate_the_epochs_lists(built):
    """Learned moves reach beyond the lists' radius: plain moves later in the same epoch scan the cells."""
    kw = dict(temperature=0.12, resort_every=8, seed=4)
    a = _run("c5", False, sweeps=(5, 16), learned_first=3, **kw)
    b = _run("c5", True, sweeps=(5, 16), learned_first=3, **kw)
    _same(a, b)


def test_lists_keep_the_reference_energy(built):
    r, R, box = config("c2")
    e = pp.Engine(pp.default_params(temperature=0.13, resort_every=2))
    e.upload(r, R, box)
    e.sweeps(40)
    e.sync()
    r2, R2, b2 = e.download()
    s = po.System(po.params(T=0.13), arrays=(r2, R2, b2))
    E, ov = s.init_energy()
    assert not ov and E == e.tracked_energy()
    e.close()
