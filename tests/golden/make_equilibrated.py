"""Equilibrated configurations at two of the benchmark state points, for the statistical parity tests
(tests/test_gpu_stats.py), written to tests/golden/equilibrated/:

  c1_<k>.rrr.gz    N = 1000 NVT, rho = 0.1, T = 0.12, Disp_max 0.05, Theta_max 0.1
  npt_<k>.rrr.gz   N = 1000 NPT, T = 0.11, P = 0.05, rescale_factor_max 0.01 (from rho = 0.3)

At these temperatures the bond network ages for millions of sweeps after a random insertion, far more than
the reference's sequential code can run in a test, so the fixtures are made in two stages:

  1. gpu: K replicas from seeded random insertions, pre-equilibrated by the GB300 engine for a fixed
     wall-clock budget (batched in one engine, ~10^6-10^7 sweeps), written as .rrr files;
  2. cpu: each configuration then runs S sweeps of the oracle (the reference's sequential algorithm,
     restated bit for bit), which reports the first- and second-half averages of E/N (and rho) of every
     run: stationarity under the reference's own dynamics. The oracle's final state is the fixture.

  python tests/golden/make_equilibrated.py gpu <dir> [seconds]   # on a GPU machine
  python tests/golden/make_equilibrated.py cpu <dir> [sweeps]    # writes tests/golden/equilibrated/
"""
import gzip
import os
import shutil
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

K = 8
POINTS = {
    "c1": dict(N=1000, rho=0.1, seed=6100, T=0.12, ensemble=0, P=0.0),
    "npt": dict(N=1000, rho=0.3, seed=6200, T=0.11, ensemble=5, P=0.05),
}
OUT = os.path.join(HERE, "equilibrated")


def gpu_stage(outdir, seconds):
    import patchyparticles_gb300 as pp
    from patchyparticles_gb300 import build

    build.build()
    os.makedirs(outdir, exist_ok=True)
    for name, pt in POINTS.items():
        prm = [pp.default_params(ensemble=pt["ensemble"], temperature=pt["T"], pressure=pt["P"], disp_max=0.05, theta_max=0.1,
                                 rescale_factor_max=0.01, seed=pt["seed"] + k) for k in range(K)]
        e = pp.Engine(prm)
        for k in range(K):
            e.upload(*pp.generate(pt["N"], pt["rho"], pt["seed"] + k, round_like_file=False), replica=k)
        t0, done = time.time(), 0
        while time.time() - t0 < seconds:
            e.sweeps(20000)
            e.sync()
            done += 20000
        for k in range(K):
            r, R, box = e.download(k)
            pp.write_rrr(os.path.join(outdir, "%s_%d.rrr" % (name, k)), done, r, R, box)
            print("%s replica %d: %d sweeps, E/N %.4f rho %.4f" % (name, k, done, e.tracked_energy(k) / pt["N"], pt["N"] / np.prod(box)), flush=True)
        e.close()


def cpu_stage(indir, sweeps):
    from oracle import pyoracle as po

    po.build(with_reference=False)
    os.makedirs(OUT, exist_ok=True)
    lines = []
    for name, pt in POINTS.items():
        res = [None] * K

        def work(k):
            s = po.System(po.params(ensemble=pt["ensemble"], T=pt["T"], P=pt["P"], disp_max=0.05, theta_max=0.1, rescale_factor_max=0.01,
                                    seed=pt["seed"] + 100 + k), path=os.path.join(indir, "%s_%d.rrr" % (name, k)))
            s.init_energy()
            E, rho = [], []
            for _ in range(100):
                s.sweeps(sweeps // 100)
                E.append(s.energy() / s.N)
                rho.append(s.N / np.prod(s.box()))
            tmp = os.path.join(OUT, "%s_%d.rrr" % (name, k))
            s.save(tmp, 0)
            with open(tmp, "rb") as f, open(tmp + ".gz", "wb") as raw, gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as g:
                shutil.copyfileobj(f, g)
            os.remove(tmp)
            res[k] = (np.mean(E[:50]), np.mean(E[50:]), np.mean(rho[:50]), np.mean(rho[50:]))
            s.close()

        th = [threading.Thread(target=work, args=(k,)) for k in range(K)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for k, (e1, e2, r1, r2) in enumerate(res):
            lines.append("%s_%d: E/N first half %.4f second half %.4f | rho %.4f %.4f" % (name, k, e1, e2, r1, r2))
        d = np.array([x[1] - x[0] for x in res])
        lines.append("%s: mean E/N drift (second - first half) %.4f +- %.4f over %d oracle sweeps" % (name, d.mean(), d.std(ddof=1) / np.sqrt(K), sweeps))
        if pt["ensemble"] == 5:
            d = np.array([x[3] - x[2] for x in res])
            lines.append("%s: mean rho drift %.5f +- %.5f" % (name, d.mean(), d.std(ddof=1) / np.sqrt(K)))
    print("\n".join(lines))


if __name__ == "__main__":
    stage, where = sys.argv[1], sys.argv[2]
    if stage == "gpu":
        gpu_stage(where, float(sys.argv[3]) if len(sys.argv) > 3 else 240.0)
    else:
        cpu_stage(where, int(sys.argv[3]) if len(sys.argv) > 3 else 200000)
