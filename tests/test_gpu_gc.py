"""Grand canonical (Ensemble = 1) and successive-umbrella-sampling (Ensemble = 3) insertions and removals
on the GPU (MC_add_remove, MC.c:342-448) against the oracle, which reproduces the reference's GC and SUS
trajectories byte for byte (tests/test_oracle.py):
- bookkeeping: after GC sweeps the particles are 0 .. N-1, the tracked energy equals the oracle's energy of
  the downloaded state, and MC_check_energy passes;
- statistics: <N> and <E/N> (GC) and the mean of the SUS window's histogram agree with the oracle's
  sequential runs within two combined standard errors (16 independent runs per side);
- the reference's stop when a GC insertion finds the system full ("increase GC_N_max").
"""
import threading

import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

RUNS = 16


def zscore(a, b):
    se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    return (a.mean() - b.mean()) / se, se


def gc_params(ens, seed, T, z, n_min, n_max):
    return pp.default_params(ensemble=ens, temperature=T, activity=z, n_min=n_min, n_max=n_max, disp_max=0.1, theta_max=0.2, seed=seed)


def test_gc_bookkeeping_and_exact_energy(built):
    r, R, box = pp.generate(300, 0.3, 4242, round_like_file=False)
    e = pp.Engine(gc_params(pp.GC, 11, 0.12, 0.1, 0, 600))
    e.upload(r, R, box)
    e.sweeps(200)
    e.sync()
    N = e.num_particles()
    t, a = e.counters()
    assert N != 300 and t[pp.MOVE_ADD] > 0 and t[pp.MOVE_REMOVE] > 0 and a[pp.MOVE_ADD] + a[pp.MOVE_REMOVE] > 0
    r2, R2, b2 = e.download()  # fails on ids that are not exactly 0 .. N-1
    assert r2.shape == (N, 3)
    s = po.System(po.params(T=0.12), arrays=(r2, R2, b2))
    E, ov = s.init_energy()
    assert not ov and E == e.tracked_energy()
    e.check_energy()
    nb, no = e.bonds()
    assert nb.sum() == -2 * E and no.sum() == 0
    e.close()


def _oracle_runs(kw, r, R, box, eq, prod, every, obs):
    out = [None] * RUNS

    def work(k):
        s = po.System(po.params(seed=2000 + k, **kw), arrays=(r, R, box))
        s.init_energy()
        s.sweeps(eq)
        vals = []
        for _ in range(prod // every):
            s.sweeps(every)
            vals.append(obs(s))
        out[k] = np.mean(vals, axis=0)
        s.close()

    th = [threading.Thread(target=work, args=(k,)) for k in range(RUNS)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    return np.array(out)


def test_gc_density_and_energy_match_the_reference(built):
    T, z, n_max = 0.2, 0.05, 400
    r, R, box = pp.generate(200, 0.2, 77, round_like_file=False)
    eq, prod, every = 2000, 20000, 20
    okw = dict(ensemble=po.GC, T=T, activity=z, n_max=n_max, disp_max=0.1, theta_max=0.2)

    def obs_o(s):
        n = s.num_particles()
        return [n, s.energy() / n if n else 0.0]

    res = [None]
    th = threading.Thread(target=lambda: res.__setitem__(0, _oracle_runs(okw, r, R, box, eq, prod, every, obs_o)))
    th.start()
    g = []
    for k in range(RUNS):
        e = pp.Engine(gc_params(pp.GC, 5000 + k, T, z, 0, n_max))
        e.upload(r, R, box)
        e.sweeps(eq)
        vals = []
        for _ in range(prod // every):
            e.sweeps(every)
            n = e.num_particles()
            vals.append([n, e.tracked_energy() / n if n else 0.0])
        g.append(np.mean(vals, axis=0))
        e.close()
    th.join()
    g, o = np.array(g), res[0]
    for i, name in enumerate(("N", "E/N")):
        zz, se = zscore(g[:, i], o[:, i])
        print("GC <%s>: gpu %.4f oracle %.4f se %.4f z %.2f" % (name, g[:, i].mean(), o[:, i].mean(), se, zz))
        assert abs(zz) < 2.0, name


def test_sus_window_histogram_matches_the_reference(built):
    T, z, n_min, n_max = 0.2, 0.05, 90, 110
    r, R, box = pp.generate(100, 0.1, 78, round_like_file=False)
    eq, prod = 1000, 20000
    okw = dict(ensemble=po.SUS, T=T, activity=z, n_min=n_min, n_max=n_max, disp_max=0.1, theta_max=0.2)
    bins = np.arange(n_min, n_max + 1)
    out_o = [None] * RUNS

    def work(k):
        s = po.System(po.params(seed=3000 + k, **okw), arrays=(r, R, box))
        s.init_energy()
        s.sweeps(eq)
        s.sus_histogram(reset=True)
        s.sweeps(prod)
        h = np.array(s.sus_histogram())
        out_o[k] = (h * bins).sum() / h.sum()
        assert s.num_particles() >= n_min and s.num_particles() <= n_max
        s.close()

    th = [threading.Thread(target=work, args=(k,)) for k in range(RUNS)]
    for t in th:
        t.start()
    g = []
    for k in range(RUNS):
        e = pp.Engine(gc_params(pp.SUS, 6000 + k, T, z, n_min, n_max))
        e.upload(r, R, box)
        e.sweeps(eq)
        e.sus_histogram(reset=True)
        e.sweeps(prod)
        h = np.array(e.sus_histogram())
        # one count per insertion / removal attempt: round(0.01 N_max) per sweep
        assert h.sum() == prod * round(0.01 * n_max) and n_min <= e.num_particles() <= n_max
        g.append((h * bins).sum() / h.sum())
        e.close()
    for t in th:
        t.join()
    g, o = np.array(g), np.array(out_o)
    zz, se = zscore(g, o)
    print("SUS window <N>: gpu %.4f oracle %.4f se %.4f z %.2f" % (g.mean(), o.mean(), se, zz))
    assert abs(zz) < 2.0


def test_gc_insertion_into_a_full_system_stops_with_the_references_message(built):
    r, R, box = pp.generate(300, 0.3, 4242, round_like_file=False)
    e = pp.Engine(gc_params(pp.GC, 3, 0.12, 50.0, 0, 301))  # a high activity fills the system at once
    e.upload(r, R, box)
    with pytest.raises(pp.PPError) as ei:
        e.sweeps(50)
        e.counters()
    assert ei.value.code == pp.PP_ERR_CAPACITY and "increase GC_N_max" in str(ei.value)
    e.close()


def test_gc_parameters_are_checked(built):
    with pytest.raises(pp.PPError):
        pp.Engine(gc_params(pp.GC, 1, 0.12, 0.0, 0, 10))  # activity must be > 0
    with pytest.raises(pp.PPError):
        pp.Engine([gc_params(pp.GC, 1, 0.12, 0.1, 0, 10)] * 2)  # one GC system per engine
    r, R, box = pp.generate(100, 0.1, 5, round_like_file=False)
    e = pp.Engine(gc_params(pp.SUS, 1, 0.12, 0.1, 110, 120))
    with pytest.raises(pp.PPError, match="smaller than Umbrella_sampling_min"):
        e.upload(r, R, box)
    e.close()
