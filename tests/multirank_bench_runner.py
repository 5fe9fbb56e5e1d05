"""Runs bench.py's GPU arm with the engine replaced by a host-side stand-in, so that its multi-rank logic
(per-rank seeds, the barrier, the max-over-ranks time, the sum of attempts, one line from rank 0) runs as
gloo ranks on a machine without a GPU. Test infrastructure for tests/test_multirank.py only.

The stand-in's rank r makes 1000 + r attempts per sweep and takes 0.5 (1 + r) ms per sweep, and writes the
seeds it was given to $PP_FAKE_OUT/rank<r>.json.
"""
import json
import os
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

RANK = int(os.environ.get("RANK", "0"))
SEEN = {"generate_seeds": [], "engine_seeds": [], "device": None}


class _Engine:
    def __init__(self, prm):
        SEEN["engine_seeds"].append(prm["seed"])
        self.att = 0
        self.launches = 0

    def upload(self, r, R, box):
        pass

    def autotune(self, n):
        return None

    def sweeps(self, n):
        self.att += n * (1000 + RANK)
        self.launches += 8 * n

    def time_sweeps(self, n):
        self.sweeps(n)
        return 0.5 * (1 + RANK) * n

    def sync(self):
        pass

    def counters(self, reset=False):
        t = [0] * 8
        t[0] = self.att
        if reset:
            self.att = 0
        return t, list(t)

    def launch_count(self):
        return self.launches

    def set_timing(self, on):
        pass

    def kernel_stats(self, reset=False):
        return {"sweep_ms": 1.0, "sweep_launches": 1, "sort_ms": 0.0, "sort_launches": 0, "volume_ms": 0.0, "volume_launches": 0}

    def guard_stats(self, reset=False):
        return {"pairs": 0, "fallbacks": 0, "mismatches": 0, "max_err_r2": 0.0, "max_err_cos": 0.0, "nl_overflows": 0}

    def close(self):
        pass


def _fake_package():
    pp = types.ModuleType("patchyparticles_gb300")
    pp.MOVE_ROTO_TRASL, pp.MOVE_VOLUME, pp.PREC_FP32_GUARD, pp.PREC_FP64 = 0, 6, 0, 1
    pp.select_device = lambda d: SEEN.__setitem__("device", d)

    def generate(N, rho, seed, round_like_file=True):
        import numpy as np

        SEEN["generate_seeds"].append(seed)
        return np.zeros((1, 3)), np.eye(3).reshape(1, 9), np.ones(3)

    pp.generate = generate
    pp.default_params = lambda **kw: kw
    pp.Engine = _Engine
    b = types.ModuleType("patchyparticles_gb300.build")
    b.build = lambda *a, **k: None
    pp.build = b
    sys.modules["patchyparticles_gb300"] = pp
    sys.modules["patchyparticles_gb300.build"] = b


if __name__ == "__main__":
    _fake_package()
    import bench

    sys.argv = [os.path.abspath(__file__)] + sys.argv[1:]  # bench.py relaunches argv[0] when it spawns its ranks
    bench.main()
    with open(os.path.join(os.environ["PP_FAKE_OUT"], "rank%d.json" % RANK), "w") as f:
        json.dump(SEEN, f)
