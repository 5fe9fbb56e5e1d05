"""Statistical parity: observables of the GPU checkerboard engine against the reference's sequential MC.

The checkerboard engine visits particles in a different order from the reference (MC.c:312 picks one
uniformly at random per attempt), so trajectories differ and parity is statistical: run-averaged
energy per particle (NVT) and density (NPT) of independent GPU replicas and independent oracle runs
must agree within two combined standard errors. Both start from a configuration the oracle has already
equilibrated at a state point that relaxes within a few hundred sweeps (T = 0.2; at T = 0.15 the
reference's own energy still drifts after 2e4 sweeps, so run averages there measure kinetics, which
legitimately differ between the sequential and the checkerboard schedules).
"""
import os
import threading

import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import pyoracle as po
from tests import helpers

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


# ---------------------------------------------------------------- the benchmark state points
# c1's point (N = 1000, rho = 0.1, T = 0.12, Disp_max 0.05, Theta_max 0.1) and an NPT system at c5's
# point (T = 0.11, P = 0.05, rescale_factor_max 0.01). The bond network ages there for millions of sweeps
# after a random insertion, so every run starts from one of the equilibrated fixtures of
# tests/golden/equilibrated (tests/golden/make_equilibrated.py: a long pre-equilibration, then the
# reference's sequential dynamics, which leave them stationary). Per side 16 runs (8 fixtures x 2 seeds),
# each 20 blocks of PROD / 20 sweeps; a run's value is the mean of its block averages, and the GPU and
# oracle means of the 16 run values must agree within two combined standard errors.
EQ_K = 8
PROD = 20000
BLOCKS = 20
EVERY = 50


def eq_fixture(name, k):
    import gzip
    import tempfile

    src = os.path.join(helpers.GOLDEN, "equilibrated", "%s_%d.rrr.gz" % (name, k))
    dst = os.path.join(tempfile.mkdtemp(prefix="ppeq_"), "%s_%d.rrr" % (name, k))
    with gzip.open(src, "rb") as f:
        open(dst, "wb").write(f.read())
    _, r, R, box = pp.read_rrr(dst)
    return r, R, box


def blocked(samples):
    """Mean of BLOCKS block averages of a run's samples (equal-size consecutive blocks)."""
    s = np.asarray(samples, dtype=np.float64)
    return s[: len(s) // BLOCKS * BLOCKS].reshape(BLOCKS, -1).mean(axis=1).mean()


def state_point_runs(name, okw, gkw, observables):
    """16 GPU replicas (one engine) and 16 oracle runs from the fixtures; observables: name -> (oracle fn,
    gpu fn). Returns {name: (gpu run values, oracle run values)}."""
    cfgs = [eq_fixture(name, k) for k in range(EQ_K)]
    runs = [(k, j) for k in range(EQ_K) for j in range(2)]
    out_o = {n: [None] * len(runs) for n in observables}

    def work(i):
        k, j = runs[i]
        s = po.System(po.params(seed=7000 + 10 * k + j, **okw), arrays=cfgs[k])
        s.init_energy()
        vals = {n: [] for n in observables}
        for _ in range(PROD // EVERY):
            s.sweeps(EVERY)
            for n, (fo, _) in observables.items():
                vals[n].append(fo(s))
        for n in observables:
            out_o[n][i] = blocked(vals[n])
        s.close()

    th = [threading.Thread(target=work, args=(i,)) for i in range(len(runs))]
    for t in th:
        t.start()
    e = pp.Engine([pp.default_params(seed=9000 + 10 * k + j, **gkw) for k, j in runs])
    for i, (k, j) in enumerate(runs):
        e.upload(*cfgs[k], replica=i)
    vals_g = {n: [[] for _ in runs] for n in observables}
    for _ in range(PROD // EVERY):
        e.sweeps(EVERY)
        e.sync()
        for n, (_, fg) in observables.items():
            for i in range(len(runs)):
                vals_g[n][i].append(fg(e, i))
    e.close()
    for t in th:
        t.join()
    return {n: (np.array([blocked(v) for v in vals_g[n]]), np.array(out_o[n])) for n in observables}


def test_c1_state_point_energy_and_bonds_per_particle(built):
    N = 1000
    okw = dict(T=0.12, disp_max=0.05, theta_max=0.1)
    gkw = dict(temperature=0.12, disp_max=0.05, theta_max=0.1)

    def o_bonds(s):
        return s.energies()[3].mean()  # bonded partners per particle, from the 27-cell walk

    def g_bonds(e, i):
        return e.bonds(i)[0].mean()  # per-particle bond counts from the energy kernel

    res = state_point_runs("c1", okw, gkw, {"E/N": (lambda s: s.energy() / N, lambda e, i: e.tracked_energy(i) / N),
                                             "bonds/N": (o_bonds, g_bonds)})
    for name, (g, o) in res.items():
        z, se = zscore(g, o)
        print("c1 <%s>: gpu %.5f oracle %.5f se %.5f z %.2f" % (name, g.mean(), o.mean(), se, z))
        assert abs(z) < 2.0, name
    # the two observables are one: bonds per particle = -2 E / N, on both sides
    assert np.allclose(res["bonds/N"][0], -2 * res["E/N"][0], atol=0.02) and np.allclose(res["bonds/N"][1], -2 * res["E/N"][1], atol=0.02)


def test_npt_density_at_the_large_scale_state_point(built):
    N = 1000
    okw = dict(ensemble=po.NPT, T=0.11, P=0.05, disp_max=0.05, theta_max=0.1, rescale_factor_max=0.01)
    gkw = dict(ensemble=pp.NPT, temperature=0.11, pressure=0.05, disp_max=0.05, theta_max=0.1, rescale_factor_max=0.01)
    res = state_point_runs("npt", okw, gkw, {"rho": (lambda s: N / np.prod(s.box()), lambda e, i: N / np.prod(e.box(i))),
                                              "E/N": (lambda s: s.energy() / N, lambda e, i: e.tracked_energy(i) / N)})
    for name, (g, o) in res.items():
        z, se = zscore(g, o)
        print("NPT T=0.11 P=0.05 <%s>: gpu %.5f oracle %.5f se %.5f z %.2f" % (name, g.mean(), o.mean(), se, z))
        assert abs(z) < 2.0, name
