"""Virtual-move Monte Carlo cluster moves (Dynamics = 1, VMMC_dynamics vmmc.c:258-483) on the GPU against the
oracle, which reproduces the reference's VMMC trajectories byte for byte (tests/test_oracle.py):
- bookkeeping: N VMMC moves per MC step, and after them the tracked energy equals the oracle's energy of the
  downloaded state and MC_check_energy passes (NVT and NPT);
- statistics: from the equilibrated fixtures of c1's state point (N = 1000, rho = 0.1, T = 0.12), the run
  averages of E/N and the VMMC acceptance of 16 GPU replicas and 16 oracle runs agree within two combined
  standard errors;
- the parameter checks.
"""
import threading

import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import pyoracle as po
from tests.test_gpu_stats import EQ_K, blocked, eq_fixture, zscore

pytestmark = pytest.mark.gpu

MAX_CLUSTER = 20


def test_vmmc_keeps_the_tracked_energy_exact(built):
    r, R, box = pp.generate(300, 0.3, 4242, round_like_file=False)
    for ens, extra in ((pp.NVT, {}), (pp.NPT, dict(pressure=0.05, rescale_factor_max=0.01))):
        e = pp.Engine(pp.default_params(ensemble=ens, temperature=0.11, dynamics=pp.VMMC, vmmc_max_cluster=MAX_CLUSTER, seed=41, **extra))
        e.upload(r, R, box)
        e.sweeps(40)
        e.sync()
        t, a = e.counters()
        assert t[pp.MOVE_VMMC] == 40 * 300 and 0 < a[pp.MOVE_VMMC] < t[pp.MOVE_VMMC]
        assert t[pp.MOVE_ROTO_TRASL] == 0  # every attempt is a cluster move
        r2, R2, b2 = e.download()
        s = po.System(po.params(T=0.11), arrays=(r2, R2, b2))
        E, ov = s.init_energy()
        assert not ov and E == e.tracked_energy()
        e.check_energy()
        e.close()


def test_vmmc_energy_and_acceptance_match_the_reference(built):
    N = 1000
    prod = 1000
    every = 20
    cfgs = [eq_fixture("c1", k) for k in range(EQ_K)]
    runs = [(k, j) for k in range(EQ_K) for j in range(2)]
    okw = dict(T=0.12, disp_max=0.05, theta_max=0.1, dynamics=po.VMMC, vmmc_max_cluster=MAX_CLUSTER)
    gkw = dict(temperature=0.12, disp_max=0.05, theta_max=0.1, dynamics=pp.VMMC, vmmc_max_cluster=MAX_CLUSTER)
    o_e, o_acc = [None] * len(runs), [None] * len(runs)

    def work(i):
        k, j = runs[i]
        s = po.System(po.params(seed=5000 + 10 * k + j, **okw), arrays=cfgs[k])
        s.init_energy()
        vals = []
        for _ in range(prod // every):
            s.sweeps(every)
            vals.append(s.energy() / N)
        t, a = s.counters()
        o_e[i] = blocked(vals)
        o_acc[i] = a[po.MOVE_VMMC] / t[po.MOVE_VMMC]
        s.close()

    th = [threading.Thread(target=work, args=(i,)) for i in range(len(runs))]
    for t in th:
        t.start()
    e = pp.Engine([pp.default_params(seed=9500 + 10 * k + j, **gkw) for k, j in runs])
    for i, (k, j) in enumerate(runs):
        e.upload(*cfgs[k], replica=i)
    vals = [[] for _ in runs]
    for _ in range(prod // every):
        e.sweeps(every)
        e.sync()
        for i in range(len(runs)):
            vals[i].append(e.tracked_energy(i) / N)
    g_e = np.array([blocked(v) for v in vals])
    g_acc = []
    for i in range(len(runs)):
        t, a = e.counters(i)
        g_acc.append(a[pp.MOVE_VMMC] / t[pp.MOVE_VMMC])
    e.check_energy(0)
    e.close()
    for t in th:
        t.join()
    for name, g, o in (("E/N", g_e, np.array(o_e)), ("VMMC acceptance", np.array(g_acc), np.array(o_acc))):
        z, se = zscore(g, o)
        print("VMMC c1 <%s>: gpu %.5f oracle %.5f se %.5f z %.2f" % (name, g.mean(), o.mean(), se, z))
        assert abs(z) < 2.0, name


def test_vmmc_parameters_are_checked(built):
    with pytest.raises(pp.PPError, match="vmmc_max_cluster"):
        pp.Engine(pp.default_params(dynamics=pp.VMMC, vmmc_max_cluster=0))
    with pytest.raises(pp.PPError, match="NVT and NPT"):
        pp.Engine(pp.default_params(dynamics=pp.VMMC, vmmc_max_cluster=5, ensemble=pp.GC, activity=0.1, n_max=400))
    with pytest.raises(pp.PPError, match="share an engine"):
        pp.Engine([pp.default_params(dynamics=pp.VMMC, vmmc_max_cluster=5), pp.default_params()])
    r, R, box = pp.generate(300, 0.3, 4242, round_like_file=False)
    e = pp.Engine(pp.default_params(dynamics=pp.VMMC, vmmc_max_cluster=5))
    e.upload(r, R, box)
    with pytest.raises(pp.PPError, match="no graphs"):
        e.set_graphs(True)
    e.close()
