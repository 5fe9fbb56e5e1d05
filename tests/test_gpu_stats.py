"""Statistical parity: observables of the GPU checkerboard engine against the reference's sequential MC.

The checkerboard engine visits particles in a different order from the reference (MC.c:312 picks one
uniformly at random per attempt), so trajectories differ and parity is statistical: run-averaged
energy per particle (NVT) and density (NPT) of independent GPU replicas and independent oracle runs
must agree within two combined standard errors. Both start from a configuration the oracle has already
equilibrated at a state point that relaxes within a few hundred sweeps (T = 0.2; at T = 0.15 the
reference's own energy still drifts after 2e4 sweeps, so run averages there measure kinetics, which
legitimately differ between the sequential and the checkerboard schedules).
"""
import threading

import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

RUNS = 16


def oracle_runs(r, R, box, prm_kw, eq, prod, every, observable):
    out = [None] * RUNS

    def work(k):
        s = po.System(po.params(seed=1000 + k, **prm_kw), arrays=(r, R, box))
        s.init_energy()
        s.sweeps(eq)
        vals = []
        for _ in range(prod // every):
            s.sweeps(every)
            vals.append(observable(s))
        out[k] = np.mean(vals)
        s.close()

    th = [threading.Thread(target=work, args=(k,)) for k in range(RUNS)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    return np.array(out)


def gpu_runs(r, R, box, prm_kw, eq, prod, every, observable):
    e = pp.Engine([pp.default_params(seed=5000 + k, **prm_kw) for k in range(RUNS)])
    for k in range(RUNS):
        e.upload(r, R, box, replica=k)
    e.sweeps(eq)
    vals = [[] for _ in range(RUNS)]
    for _ in range(prod // every):
        e.sweeps(every)
        e.sync()
        for k in range(RUNS):
            vals[k].append(observable(e, k))
    e.close()
    return np.array([np.mean(v) for v in vals])


def zscore(a, b):
    se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    return (a.mean() - b.mean()) / se, se


def equilibrated(N, rho, seed, kw, sweeps):
    r, R, box = pp.generate(N, rho, seed, round_like_file=True)
    s = po.System(po.params(seed=seed, **kw), arrays=(r, R, box))
    s.init_energy()
    s.sweeps(sweeps)
    r2, R2 = s.state()
    b2 = s.box()
    s.close()
    return r2, R2, b2


def test_nvt_energy_per_particle(built):
    N = 500
    kw = dict(T=0.2, disp_max=0.3, theta_max=0.5)
    gkw = dict(temperature=0.2, disp_max=0.3, theta_max=0.5)
    r, R, box = equilibrated(N, 0.3, 77, kw, 2000)
    o = oracle_runs(r, R, box, kw, 200, 4000, 10, lambda s: s.energy() / N)
    g = gpu_runs(r, R, box, gkw, 200, 4000, 10, lambda e, k: e.tracked_energy(k) / N)
    z, se = zscore(g, o)
    print("NVT <E/N>: gpu %.5f oracle %.5f se %.5f z %.2f" % (g.mean(), o.mean(), se, z))
    assert abs(z) < 2.0


def test_npt_density(built):
    N = 400
    kw = dict(ensemble=po.NPT, T=0.2, P=0.3, disp_max=0.3, theta_max=0.5, rescale_factor_max=0.05)
    gkw = dict(ensemble=pp.NPT, temperature=0.2, pressure=0.3, disp_max=0.3, theta_max=0.5, rescale_factor_max=0.05)
    r, R, box = equilibrated(N, 0.3, 78, kw, 2000)
    o = oracle_runs(r, R, box, kw, 200, 4000, 10, lambda s: N / np.prod(s.box()))
    g = gpu_runs(r, R, box, gkw, 200, 4000, 10, lambda e, k: N / np.prod(e.box(k)))
    z, se = zscore(g, o)
    print("NPT <rho>: gpu %.5f oracle %.5f se %.5f z %.2f" % (g.mean(), o.mean(), se, z))
    assert abs(z) < 2.0
