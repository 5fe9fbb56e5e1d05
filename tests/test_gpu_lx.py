"""The NVT box-shape move (Lx_move, MC_change_Lx, MC.c:515-585) on the GPU: one attempt per sweep, Ly = Lz at
constant volume, the tracked energy equal to the reference routines' energy of the downloaded state,
the same trajectory with and without neighbour lists and CUDA graphs, the reference's validation errors,
and box-shape statistics against the reference's sequential MC (the oracle, pinned by a reference
trajectory with Lx_move = 1)."""
import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import pyoracle as po
from tests.helpers import config
from tests.test_gpu_stats import RUNS, equilibrated, zscore

pytestmark = pytest.mark.gpu

LX = dict(lx_move=1, lx_change_max=0.5, lyz_min=8.0, lyz_max=12.0)


def _run(sweeps, lists=True, graphs=True, **kw):
    r, R, box = config("small")
    e = pp.Engine(pp.default_params(temperature=0.11, seed=3, **dict(LX, **kw)))
    e.set_neighbour_lists(lists)
    e.set_graphs(graphs)
    e.upload(r, R, box)
    for n in sweeps:
        e.sweeps(n)
    e.sync()
    out = dict(state=e.download(), E=e.tracked_energy(), counters=e.counters(), box=e.box())
    e.close()
    return out


def test_lx_move_keeps_volume_shape_and_energy(built):
    res = _run((120, 80))
    tries, acc = res["counters"]
    assert tries[pp.MOVE_LX] == 200 and 0 < acc[pp.MOVE_LX] < 200  # one attempt per sweep
    b = res["box"]
    assert b[1] == b[2] and 8.0 <= b[1] <= 12.0
    assert abs(b[0] * b[1] * b[2] / 1000.0 - 1.0) < 1e-12
    assert b[0] != 10.0  # the shape moved
    r2, R2, b2 = res["state"]
    s = po.System(po.params(T=0.11), arrays=(r2, R2, b2))
    E, ov = s.init_energy()
    assert not ov and E == res["E"]


@pytest.mark.parametrize("lists,graphs", [(False, True), (True, False)])
def test_lx_move_with_and_without_lists_and_graphs(built, lists, graphs):
    a = _run((40, 7, 13))
    b = _run((40, 7, 13), lists=lists, graphs=graphs)
    for x, y in zip(a["state"], b["state"]):
        assert np.array_equal(x, y)
    assert a["E"] == b["E"] and a["counters"] == b["counters"] and np.array_equal(a["box"], b["box"])


def test_boltzmann_acceptance_variant(built):
    res = _run((100,), lx_move=2)
    r2, R2, b2 = res["state"]
    s = po.System(po.params(T=0.11), arrays=(r2, R2, b2))
    E, ov = s.init_energy()
    assert not ov and E == res["E"] and res["counters"][0][pp.MOVE_LX] == 100


def test_reference_validation_errors(built):
    r, R, box = config("small")
    for kw, msg in ((dict(lyz_min=10.0), "Lyz_min should be smaller"), (dict(lyz_max=10.0), "Lyz_max should be larger")):
        e = pp.Engine(pp.default_params(**dict(LX, **kw)))
        with pytest.raises(pp.PPError, match=msg):
            e.upload(r, R, box)
        e.close()
    e = pp.Engine(pp.default_params(**LX))
    with pytest.raises(pp.PPError, match="requires Ly = Lz"):
        e.upload(r, R, np.array([10.0, 10.0, 10.5]))
    e.close()


def test_box_shape_statistics_match_the_reference(built):
    N = 500
    L = (N / 0.3) ** (1.0 / 3.0)
    lx = dict(lx_move=1, lx_change_max=0.25, lyz_min=0.95 * L, lyz_max=1.05 * L)
    kw = dict(T=0.2, disp_max=0.3, theta_max=0.5, **lx)
    gkw = dict(temperature=0.2, disp_max=0.3, theta_max=0.5, **lx)
    r, R, box = equilibrated(N, 0.3, 79, kw, 1000)
    from tests.test_gpu_stats import gpu_runs, oracle_runs

    o = oracle_runs(r, R, box, kw, 200, 4000, 10, lambda s: s.box()[0])
    g = gpu_runs(r, R, box, gkw, 200, 4000, 10, lambda e, k: e.box(k)[0])
    z, se = zscore(g, o)
    print("Lx move <Lx>: gpu %.4f oracle %.4f se %.4f z %.2f" % (g.mean(), o.mean(), se, z))
    assert abs(z) < 2.0  # two combined standard errors of the 16 + 16 run means
