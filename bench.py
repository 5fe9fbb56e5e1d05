#!/usr/bin/env python
"""Throughput benchmark of the roto-translation Monte Carlo hot path (Kern-Frenkel 4-patch, Dynamics = 0).

Metric: MC move attempts per second. Default workload: N = 1,048,576 particles, NPT (T = 0.11, P = 0.05,
rescale_factor_max = 0.01) from a seeded random insertion at rho = 0.3 with uniform orientations,
KF_delta = 0.12, KF_cosmax = 0.92, Disp_max = 0.05, Theta_max = 0.1, FP32 pair tests with an FP64 guard
band (eps = 1e-5), FP64 state. One step = one MC sweep: one checkerboard round (one attempt per non-empty cell) plus one NPT volume
attempt.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload c5|c2|c4|c1]

--impl gb300 (default) times the CUDA engine through its C-ABI; --impl reference times the reference's
CPU implementation of the same path on the host cores (oracle/_ref when the reference was compiled on
this machine, otherwise the oracle restatement of it, oracle/pp_oracle.c, which reproduces the reference
trajectory bit for bit), one independent system per core.

Under torchrun (N > 1) every rank runs an independent replica of the workload on its own GPU (the path
does not shard; there is no collective in the data path); rank 0 prints the aggregate.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "MC move attempts/sec at N=1M (frac of HBM peak); eff. samples/sec learned vs plain"
UNIT = "attempts/s"
# algorithmic bytes of one attempt: read + write of one particle's FP64 state as the reference keeps it,
# position (24 B) + orientation matrix (72 B); the unit of the HBM roofline of the sweep kernel
BYTES_PER_ATTEMPT = 192

WORKLOADS = {
    "c5": dict(N=1048576, rho=0.3, T=0.11, P=0.05, ensemble=5, rescale=0.01, disp=0.05, theta=0.1, seed=1005,
               name="N=1048576 NPT rho0=0.3 T=0.11 P=0.05 rescale_factor_max=0.01, plain roto-translation"),
    "c2": dict(N=32768, rho=0.5, T=0.13, P=0.0, ensemble=0, rescale=0.01, disp=0.05, theta=0.1, seed=1002,
               name="N=32768 NVT rho=0.5 T=0.13, plain roto-translation"),
    "c4": dict(N=32768, rho=0.1, T=0.09, P=0.0, ensemble=0, rescale=0.01, disp=0.05, theta=0.1, seed=1004,
               name="N=32768 NVT rho=0.1 T=0.09, plain roto-translation"),
    "c1": dict(N=1000, rho=0.1, T=0.12, P=0.0, ensemble=0, rescale=0.01, disp=0.05, theta=0.1, seed=1001,
               name="N=1000 NVT rho=0.1 T=0.12, plain roto-translation"),
}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def profiled_traffic(workload):
    """DRAM bytes per launch of the sweep kernel from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", "k_colour_%s.txt" % workload)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch_full_size"):
            try:
                return float(line.split("=")[1].split()[0])
            except Exception:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.out = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return ws, rank, local, dist
    return 1, 0, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allreduce(dist, value, op):
    if dist is None:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=op)
    return float(t.item())


def batch_configs(n=256, seed=3000):
    """The batched-replica workload: n NVT replicas, N log-uniform in [500, 8000], T uniform in [0.09, 0.20],
    rho uniform in [0.05, 0.6], KF_cosmax uniform in [0.89, 0.95] (seeded), each a seeded random insertion."""
    import patchyparticles_gb300 as pp

    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        N = int(round(np.exp(rng.uniform(np.log(500), np.log(8000)))))
        T, rho, cm = rng.uniform(0.09, 0.20), rng.uniform(0.05, 0.6), rng.uniform(0.89, 0.95)
        r, R, box = pp.generate(N, rho, seed + k, round_like_file=False)
        out.append(dict(N=N, T=T, rho=rho, cosmax=cm, seed=seed + k, arrays=(r, R, box)))
    return out


def run_batch(args, ws, rank, local, dist):
    """Batched replicas in one engine: every launch advances all of them."""
    import patchyparticles_gb300 as pp
    from patchyparticles_gb300 import build

    if rank == 0 or ws == 1:
        build.build()
    barrier(dist)
    pp.select_device(local)
    reps = batch_configs(seed=3000 + 1000 * rank)
    prm = [pp.default_params(temperature=c["T"], kf_cosmax=c["cosmax"], seed=c["seed"]) for c in reps]
    e = pp.Engine(prm)
    for k, c in enumerate(reps):
        e.upload(*c["arrays"], replica=k)
    tune = e.autotune(args.tune_sweeps) if args.tune_sweeps > 0 else None
    for _ in range(args.warmup):
        e.sweeps(args.sweeps_per_step)
    e.sync()
    for k in range(len(reps)):
        e.counters(replica=k, reset=True)
    launches0 = e.launch_count()
    sampler = ClockSampler(local)
    barrier(dist)
    sampler.start()
    ms = e.time_sweeps(args.steps * args.sweeps_per_step)
    clocks = sampler.stop()
    barrier(dist)
    att = sum(e.counters(replica=k)[0][pp.MOVE_ROTO_TRASL] for k in range(len(reps)))
    t_max = allreduce(dist, ms / 1000.0, _max_op(dist))
    att = allreduce(dist, att, _sum_op(dist))
    ntot = sum(c["N"] for c in reps)
    launches = e.launch_count() - launches0
    e.close()
    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    achieved = att / t_max * BYTES_PER_ATTEMPT / 1e9
    line = {
        "metric": "MC move attempts/sec, 256 batched replicas", "value": att / t_max, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic (seeded random insertion per replica)",
        "config": {"workload": "256 NVT replicas, N log-uniform 500-8000 (%d particles), T U[0.09,0.20], rho U[0.05,0.6], KF_cosmax U[0.89,0.95]" % ntot,
                   "schedule": tune, "l2": "the whole batch (%.0f MB of FP64 state) fits in L2" % (ntot * 128 / 1e6)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_source": peak_kind, "bytes_per_attempt": BYTES_PER_ATTEMPT, "note": "whole sweep, not one kernel"},
        "clocks": clocks, "e2e": None, "cpu_baseline": None, "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


def make_config(wl, seed_offset=0):
    """The workload's seeded random insertion, built by the product's generator (the GPU arm)."""
    import patchyparticles_gb300 as pp

    return pp.generate(wl["N"], wl["rho"], wl["seed"] + seed_offset, round_like_file=False)


def workload_config(wl, args):
    """The `config` object of both arms' lines: the workload alone (no implementation detail), so that the
    GPU line and the reference line describe the same thing."""
    prop = "plain" if args.proposal == "plain" else "learned mixture (36-64-64-4 network trained at N=32768 rho=0.1 T=0.09)"
    return {"workload": wl["name"] if args.proposal == "plain" else wl["name"].replace("plain roto-translation", "learned proposal"),
            "N": wl["N"], "sweeps_per_step": args.sweeps_per_step, "proposal": prop,
            "l2": "inputs larger than L2 (FP64 state %.0f MB + FP32 mirror %.0f MB per GPU)" % (wl["N"] * 128 / 1e6, wl["N"] * 64 / 1e6)}


def cpu_reference_impl():
    """Which CPU implementation is timed: the reference compiled here, or the oracle restatement."""
    return "port"


def cpu_throughput(wl, r, R, box, seconds, threads, samples=1):
    from oracle import pyoracle as po

    po.build(with_reference=False)
    prm = po.params(ensemble=wl["ensemble"], T=wl["T"], P=wl["P"], disp_max=wl["disp"], theta_max=wl["theta"],
                    rescale_factor_max=wl["rescale"], seed=wl["seed"])
    pool = po.Pool(r, R, box, prm, threads)
    tot_att, tot_t = 0, 0.0
    for _ in range(samples):
        t0 = time.perf_counter()
        _, att = pool.run(seconds)
        tot_t += time.perf_counter() - t0
        tot_att += att
    pool.close()
    return tot_att / tot_t, tot_att, tot_t


def run_reference(args, wl, ws, rank, dist):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    from oracle import pyoracle as po

    po.build(with_reference=False)
    # the input comes from the oracle's restatement of the reference generator (generator.c:43-68), which
    # equals the product's generator bit for bit: nothing of the GPU engine is loaded on this arm
    r, R, box = po.generate(wl["N"], wl["rho"], wl["seed"])
    prm = po.params(ensemble=wl["ensemble"], T=wl["T"], P=wl["P"], disp_max=wl["disp"], theta_max=wl["theta"],
                    rescale_factor_max=wl["rescale"], seed=wl["seed"])
    pool = po.Pool(r, R, box, prm, threads)
    # warm-up, then the K steps as one continuous all-core sample of ~20 s (a restart per step would cost
    # the pool ~0.1 s each): value = attempts / elapsed over the whole timed region
    pool.run(min(2.0, 0.2 * max(1, args.warmup)))
    sample = max(1.0, min(20.0, 0.2 * args.steps))
    t0 = time.perf_counter()
    _, att = pool.run(sample)
    el = time.perf_counter() - t0
    pool.close()
    value = att / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * el / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random insertion, uniform orientations)",
        "config": workload_config(wl, args),
        "implementation": "the reference's sequential CPU Monte Carlo (MC.c do_NVT/do_NPT) as restated by the oracle (oracle/pp_oracle.c, "
                          "trajectories byte-identical to the reference built from its sources); every pair test in FP64",
        "sample": "one continuous %.1f s all-core sample over the %d steps" % (el, args.steps),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": cpu_reference_impl(),
                         "sample": "%d independent %d-particle systems (one per host thread), %.1f s" % (threads, wl["N"], el)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args, wl, ws, rank, local, dist):
    import patchyparticles_gb300 as pp
    from patchyparticles_gb300 import build

    if rank == 0 or ws == 1:
        build.build()
    barrier(dist)
    pp.select_device(local)
    r, R, box = make_config(wl, seed_offset=rank)
    prep, audit = None, None
    if args.workload == "c2":
        # the configuration's 10^3-sweep hard-sphere equilibration (T = 1e9: every move without an overlap is
        # accepted, bonds do not matter) before the timed run; both precisions start from this state
        h = pp.Engine(pp.default_params(temperature=1e9, disp_max=wl["disp"], theta_max=wl["theta"], seed=wl["seed"] + 100 + rank))
        h.upload(r, R, box)
        h.sweeps(1000)
        r, R, box = h.download()
        h.close()
        prep = "1000 hard-sphere sweeps (T = 1e9) from the seeded random insertion"
        # the guard band's check on this state: every pair of 5 sweeps decided in FP32 and in FP64 (audit mode)
        a = pp.Engine(pp.default_params(temperature=wl["T"], disp_max=wl["disp"], theta_max=wl["theta"], seed=wl["seed"] + rank, audit=1))
        a.upload(r, R, box)
        a.sweeps(5)
        g = a.guard_stats()
        a.close()
        audit = {"sweeps": 5, "pairs": g["pairs"], "fallbacks": g["fallbacks"], "mismatches": g["mismatches"],
                 "max_err_r2": g["max_err_r2"], "max_err_cos": g["max_err_cos"]}
    prm = pp.default_params(ensemble=wl["ensemble"], temperature=wl["T"], pressure=wl["P"], disp_max=wl["disp"],
                            theta_max=wl["theta"], rescale_factor_max=wl["rescale"], seed=wl["seed"] + rank,
                            precision=pp.PREC_FP64 if args.precision == "fp64" else pp.PREC_FP32_GUARD)
    e = pp.Engine(prm)
    e.upload(r, R, box)
    spsw = args.sweeps_per_step
    train = None
    if args.proposal == "learned":
        # the large-scale configuration with the learned proposal: the network trained on the GPU on the
        # learned-comparison workload (N=32768, rho=0.1, T=0.09, plain-move samples), then used here
        W, train = train_network(args)
        e.learned_init(seed=7, **json.loads(args.learn_params))
        e.set_learned_weights(W)
        e.set_proposal(True)
        args.tune_sweeps = 0
    tune = e.autotune(args.tune_sweeps) if args.tune_sweeps > 0 else None  # schedule choice, before the timed region
    # warm-up
    for _ in range(args.warmup):
        e.sweeps(spsw)
    e.sync()
    e.counters(reset=True)
    launches0 = e.launch_count()
    sampler = ClockSampler(local)
    barrier(dist)
    e.sync()
    sampler.start()
    ms = e.time_sweeps(args.steps * spsw)  # CUDA events on the engine's stream around the K steps (graph replays)
    clocks = sampler.stop()
    barrier(dist)
    launches = e.launch_count() - launches0
    tries, acc = e.counters()
    attempts = tries[pp.MOVE_ROTO_TRASL] + tries[pp.MOVE_VOLUME]
    t_max = allreduce(dist, ms / 1000.0, _max_op(dist))
    att_sum = allreduce(dist, attempts, _sum_op(dist))
    value = att_sum / t_max

    # roofline of the dominant kernel: k_colour. A separate pass of the same sweeps with per-group CUDA events
    # on the engine stream (stream launches; the 8 colour launches of a round form one group), 192 B per attempt
    e.counters(reset=True)
    e.set_timing(True)
    e.kernel_stats(reset=True)
    e.guard_stats(reset=True)
    e.sweeps(args.roofline_sweeps)
    e.sync()
    ks = e.kernel_stats()
    gs = e.guard_stats()
    e.set_timing(False)
    rtries, _ = e.counters()
    peak, peak_kind = measured_peaks()
    sweep_launches = max(1, ks["sweep_launches"])
    avg_ms = ks["sweep_ms"] / sweep_launches
    att_per_launch = rtries[pp.MOVE_ROTO_TRASL] / sweep_launches
    achieved = att_per_launch * BYTES_PER_ATTEMPT / (avg_ms / 1000.0) / 1e9
    traffic = profiled_traffic(args.workload)

    # end to end through the C-ABI with host buffers: upload (H2D) + sweeps + download (D2H) per step
    e2e = None
    if not args.no_e2e:
        r_h, R_h, b_h = e.download()
        e2e_steps = args.e2e_steps
        att_e2e = 0
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e.upload(r_h, R_h, b_h)
            e.counters(reset=True)
            e.sweeps(args.e2e_sweeps)
            r_h, R_h, b_h = e.download()
            _ = e.tracked_energy()
            t, _a = e.counters()
            att_e2e += t[pp.MOVE_ROTO_TRASL] + t[pp.MOVE_VOLUME]
        el = time.perf_counter() - t0
        el = allreduce(dist, el, _max_op(dist))
        att_e2e = allreduce(dist, att_e2e, _sum_op(dist))
        N = wl["N"]
        # upload: 16-double canonical records + particle index; download: x y z R (12 doubles) + index
        e2e = {"value": att_e2e / el, "unit": UNIT, "h2d_bytes_per_step": N * (128 + 4), "d2h_bytes_per_step": N * (96 + 4),
               "sweeps_per_step": args.e2e_sweeps, "steps": e2e_steps,
               "step": "upload (H2D, initial energy check) + sweeps + download (D2H) + tracked energy, through the C-ABI with host arrays"}

    learned, learned_large = None, None
    if rank == 0 and ws == 1 and not args.no_learned and args.proposal == "plain":
        e.close()
        learned = learned_comparison(args)
        if args.workload == "c5":  # the large-scale configuration with the learned proposal, the same network
            learned_large = large_learned(args, wl, learned.pop("_weights"))
        else:
            learned.pop("_weights")

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, a, t = cpu_throughput(wl, r, R, box, args.cpu_seconds, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": cpu_reference_impl(),
               "sample": "%d independent %d-particle systems for %.1f s (%d attempts)" % (threads, wl["N"], t, a)}
    e.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic (seeded random insertion, uniform orientations)",
        "config": workload_config(wl, args),
        "precision": "FP64 pair tests" if args.precision == "fp64" else "FP32 pair tests with the FP64 guard band (eps 1e-5), FP64 state",
        "parallelism": "independent replicas, one per GPU" if ws > 1 else "single GPU",
        "launch": "CUDA graph per re-sort period, programmatic dependent launch between its kernels",
        "schedule": tune if tune else "defaults (resort_every 4, reorder_every 16, cell_scale 1.0)",
        "acceptance": acc[pp.MOVE_ROTO_TRASL] / max(1, tries[pp.MOVE_ROTO_TRASL]),
        "volume_acceptance": acc[pp.MOVE_VOLUME] / max(1, tries[pp.MOVE_VOLUME]) if tries[pp.MOVE_VOLUME] else None,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": sweep_kernel_name(args, tune), "peak_source": peak_kind,
                     "bytes_per_attempt": BYTES_PER_ATTEMPT, "avg_launch_ms": avg_ms, "attempts_per_launch": att_per_launch,
                     # pairs inside the FP32 guard band, decided in FP64 (colour and volume passes), per MC step
                     "guard_band_pairs_per_step": gs["fallbacks"] / max(1, args.roofline_sweeps)},
        "kernel_ms_per_step": {"sort": ks["sort_ms"] / max(1, ks["sort_launches"]), "sweep": avg_ms,
                               "volume": ks["volume_ms"] / max(1, ks["volume_launches"]) if ks["volume_launches"] else 0.0},
        "clocks": clocks,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "gpu_launches": launches,
        "learned": learned,
        "learned_large_scale": learned_large,
        "training": train,
        "preparation": prep,
        "fp32_vs_fp64_audit": audit,
    }
    print(json.dumps(line), flush=True)


def sweep_kernel_name(args, tune):
    if args.proposal == "learned":
        return "k_colour_learned (8 launches per round, one event group)"
    if os.environ.get("PPGPU_PERSIST") == "1":
        return "k_round (one persistent cooperative launch per round over the neighbour lists)"
    return "k_colour%s (8 launches per round, one event group)" % (" over neighbour lists" if (tune is None or tune.get("neighbour_lists", 1)) else "")


def train_network(args):
    """Trains the proposal network on the GPU as the learned comparison does (samples of the plain move at
    N=32768, rho=0.1, T=0.09); returns (weights, training record)."""
    import patchyparticles_gb300 as pp

    wl = WORKLOADS["c4"]
    r, R, box = pp.generate(wl["N"], wl["rho"], wl["seed"], round_like_file=False)
    e = pp.Engine(pp.default_params(temperature=wl["T"], disp_max=wl["disp"], theta_max=wl["theta"], seed=wl["seed"]))
    e.upload(r, R, box)
    e.learned_init(seed=7, **json.loads(args.learn_params))
    t0 = time.perf_counter()
    e.learned_collect(args.learn_configs, args.learn_sweeps_between, 128)
    obj = e.learned_train(args.learn_epochs, lr=3e-3)
    e.sync()
    W = e.learned_weights()
    e.close()
    return W, {"workload": wl["name"], "configs": args.learn_configs, "epochs": args.learn_epochs, "objective": obj, "seconds": time.perf_counter() - t0}


# ---------------------------------------------------------------- learned proposal vs plain (N=32768, T=0.09)
def _acf_particles(B):
    """Autocorrelation of per-particle bond counts B[t][i] (the per-time mean over particles removed, so a
    slow drift of the whole system does not count as correlation), averaged over particles."""
    T = B.shape[0]
    gm = B.mean(axis=1, keepdims=True)
    a = np.zeros(T)
    for c0 in range(0, B.shape[1], 4096):  # particles in chunks (memory)
        d = B[:, c0:c0 + 4096].astype(np.float64) - gm
        d -= d.mean(axis=0, keepdims=True)
        f = np.fft.rfft(d, 2 * T, axis=0)
        a += np.fft.irfft(f * np.conj(f), axis=0)[:T].sum(axis=1)
    a /= np.arange(T, 0, -1)
    return a / a[0]


def tau_int(acf, n, c=5.0):
    """Sokal's windowed integrated autocorrelation time, in samples: tau = 1 + 2 sum_{t=1..M} C(t) with the
    window M the smallest lag with M >= c tau. Returns (tau, M, window_limited, sigma): window_limited when
    no such M exists within the series (tau is then a lower bound) or M > n / 50 (the run is shorter than 50
    tau windows, Sokal's reliability rule); sigma from Sokal's variance 2 (2M + 1) / n tau^2."""
    tau, M = 1.0, len(acf) - 1
    found = False
    for m in range(1, len(acf)):
        tau = 1.0 + 2.0 * float(acf[1:m + 1].sum())
        if m >= c * tau:
            M, found = m, True
            break
    sigma = tau * np.sqrt(2.0 * (2 * M + 1) / n)
    return tau, M, (not found) or M > n / 50, sigma


def _chains(engines, sweeps, every):
    """Runs the chains side by side (each engine on its own stream, so their launches overlap) and samples
    every particle's bond count every `every` sweeps. Returns one (n, N) int8 array per engine."""
    n = sweeps // every
    out = [np.zeros((n, e.num_particles()), dtype=np.int8) for e in engines]
    for k in range(n):
        for e in engines:
            e.sweeps(every)
        for e, B in zip(engines, out):
            B[k] = e.bonds()[0]
    return out


def _chain_result(B, every, ms_per_sweep, N):
    acf = _acf_particles(B)
    tau, M, limited, sig = tau_int(acf, len(B))
    tau_sw, sig_sw = tau * every, sig * every
    sps = 1000.0 / ms_per_sweep
    g = B.mean(axis=1) / 2.0  # bonded pairs per particle at each snapshot
    half = len(g) // 2
    m1, m2 = g[:half].mean(), g[half:].mean()
    # standard error of the difference of the two halves' means, from 20 block averages
    nb = 20 if len(g) >= 20 else max(2, len(g))
    blk = g[: len(g) // nb * nb].reshape(nb, -1).mean(axis=1)
    drift_se = blk.std(ddof=1) / np.sqrt(nb / 2.0) * np.sqrt(2.0)
    ess = N * sps / (2.0 * tau_sw)
    return {"ms_per_sweep": ms_per_sweep, "sweeps": len(B) * every, "snapshot_every": every,
            "bonds_per_particle_halves": [float(m1), float(m2)], "drift": float(m2 - m1), "drift_se_blocks": float(drift_se),
            "tau_int_sweeps": float(tau_sw), "tau_int_sigma_sweeps": float(sig_sw), "window_sweeps": int(M * every),
            "tau_window_limited": bool(limited), "ess_per_s": float(ess), "ess_per_s_sigma": float(ess * sig_sw / tau_sw)}


def learned_comparison(args, T=None, N=None, rho=None):
    """The learned proposal against the plain move (default N=32768, rho=0.1, T=0.09). The network is trained
    on the GPU on samples of configurations generated by the plain move; both chains then start from the
    same configuration (the plain chain's state after the training samples) and run side by side.
    Effective samples/s of the per-particle bond count = N x sweeps/s / (2 tau_int), tau_int Sokal's
    windowed integrated autocorrelation time (with its window flag and error bar); the bonds-per-particle
    averages of the two halves of each chain show whether it was stationary."""
    import patchyparticles_gb300 as pp

    wl = dict(WORKLOADS["c4"])
    wl["T"] = T if T is not None else args.learn_T
    wl["N"] = N if N is not None else args.learn_N
    wl["rho"] = rho if rho is not None else wl["rho"]
    r, R, box = pp.generate(wl["N"], wl["rho"], wl["seed"], round_like_file=False)
    prm = pp.default_params(temperature=wl["T"], disp_max=wl["disp"], theta_max=wl["theta"], seed=wl["seed"])
    e = pp.Engine(prm)
    e.upload(r, R, box)
    e.learned_init(seed=7, **json.loads(args.learn_params))
    t0 = time.perf_counter()
    e.learned_collect(args.learn_configs, args.learn_sweeps_between, 128)
    t1 = time.perf_counter()
    obj = e.learned_train(args.learn_epochs, lr=3e-3)
    e.sync()
    t2 = time.perf_counter()
    W = e.learned_weights()
    r0, R0, b0 = e.download()
    e.close()
    res = {"workload": "N=%d NVT rho=%g T=%g KF_delta=0.12 KF_cosmax=0.92, Disp_max=0.05, Theta_max=0.1 (plain component)" % (wl["N"], wl["rho"], wl["T"]),
           "start": "both chains from the plain chain's state after %d sweeps (the training samples' run)" % (args.learn_configs * args.learn_sweeps_between),
           "training": {"configs": args.learn_configs, "sweeps_between": args.learn_sweeps_between, "samples": args.learn_configs * 128,
                        "epochs": args.learn_epochs, "objective": obj, "collect_s": t1 - t0, "train_s": t2 - t1,
                        "network": "36-64-64-4 ReLU, BF16 tcgen05 GEMMs, FP32 accumulation"}}
    engines = []
    for learned in (False, True):
        x = pp.Engine(prm)
        x.upload(r0, R0, b0)
        x.learned_init(seed=7, **json.loads(args.learn_params))
        x.set_learned_weights(W)
        x.set_proposal(learned)
        engines.append(x)
    # cost per sweep of each chain on its own (CUDA events on the engine's stream)
    ms = [x.time_sweeps(args.learn_time_sweeps) / args.learn_time_sweeps for x in engines]
    engines[1].learned_stats(reset=True)
    Bs = _chains(engines, args.learn_measure_sweeps, args.learn_every)
    for name, x, B, m in zip(("plain", "learned"), engines, Bs, ms):
        res[name] = _chain_result(B, args.learn_every, m, wl["N"])
    t, a = engines[1].learned_stats(reset=True)
    tt = max(1, sum(t))
    res["learned"]["component_share"] = [v / tt for v in t]
    res["learned"]["component_acceptance"] = [a[k] / max(1, t[k]) for k in range(len(t))]
    for x in engines:
        x.close()
    p, l = res["plain"], res["learned"]
    res["ess_ratio"] = l["ess_per_s"] / p["ess_per_s"]
    res["ess_ratio_sigma"] = res["ess_ratio"] * float(np.hypot(p["tau_int_sigma_sweeps"] / p["tau_int_sweeps"], l["tau_int_sigma_sweeps"] / l["tau_int_sweeps"]))
    res["per_sweep_ratio"] = p["tau_int_sweeps"] / l["tau_int_sweeps"]
    res["resolved"] = not (p["tau_window_limited"] or l["tau_window_limited"])
    res["_weights"] = W
    return res


def large_learned(args, wl, W):
    """Learned-proposal sweeps of the main workload (N=1M NPT): the network of the learned comparison, its
    attempts/s through the same timed sweeps as the main line, and the learned colour kernel's roofline."""
    import patchyparticles_gb300 as pp

    r, R, box = make_config(wl)
    e = pp.Engine(pp.default_params(ensemble=wl["ensemble"], temperature=wl["T"], pressure=wl["P"], disp_max=wl["disp"],
                                    theta_max=wl["theta"], rescale_factor_max=wl["rescale"], seed=wl["seed"]))
    e.upload(r, R, box)
    e.learned_init(seed=7, **json.loads(args.learn_params))
    e.set_learned_weights(W)
    e.set_proposal(True)
    for _ in range(3):
        e.sweeps(1)
    e.sync()
    e.counters(reset=True)
    e.learned_stats(reset=True)
    n = args.learn_large_sweeps
    ms = e.time_sweeps(n)
    tries, acc = e.counters()
    att = tries[pp.MOVE_ROTO_TRASL] + tries[pp.MOVE_VOLUME]
    e.counters(reset=True)
    e.set_timing(True)
    e.kernel_stats(reset=True)
    e.sweeps(8)
    e.sync()
    ks = e.kernel_stats()
    e.set_timing(False)
    rt, _ = e.counters()
    t, a = e.learned_stats()
    e.close()
    peak, kind = measured_peaks()
    avg = ks["sweep_ms"] / max(1, ks["sweep_launches"])
    achieved = rt[pp.MOVE_ROTO_TRASL] / max(1, ks["sweep_launches"]) * BYTES_PER_ATTEMPT / (avg / 1000.0) / 1e9
    return {"workload": wl["name"].replace("plain roto-translation", "learned proposal"), "value": att / (ms / 1000.0), "unit": UNIT,
            "ms_per_sweep": ms / n, "sweeps": n, "acceptance": acc[pp.MOVE_ROTO_TRASL] / max(1, tries[pp.MOVE_ROTO_TRASL]),
            "component_share": [x / max(1, sum(t)) for x in t],
            "roofline": {"kernel": "k_colour_learned (8 launches per round)", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": kind, "avg_round_ms": avg}}


def _max_op(dist):
    if dist is None:
        return None
    return dist.ReduceOp.MAX


def _sum_op(dist):
    if dist is None:
        return None
    return dist.ReduceOp.SUM


def _spawn_ranks(n):
    """Runs this command as n ranks on this node (127.0.0.1 rendezvous) and returns their exit status."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n), "--master-addr", "127.0.0.1",
           "--master-port", str(port), os.path.abspath(sys.argv[0])] + sys.argv[1:]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)  # ~0.85 s timed at N = 1M: the clock sampler sees it
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c5", choices=sorted(WORKLOADS) + ["c3"])
    ap.add_argument("--proposal", default="plain", choices=["plain", "learned"],
                    help="the moves of the timed sweeps: the plain roto-translation (default) or the learned mixture")
    ap.add_argument("--precision", default="fp32-guard", choices=["fp32-guard", "fp64"],
                    help="pair tests in FP32 with the FP64 guard band (default) or every pair in FP64")
    ap.add_argument("--sweeps-per-step", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--e2e-sweeps", type=int, default=1000,
                    help="sweeps between upload and download of an end-to-end step (1000 = Print_every of the reference's example inputs)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-plain effective-sample comparison")
    ap.add_argument("--tune-sweeps", type=int, default=10, help="sweeps per autotuner trial before the run (0: default schedule)")
    ap.add_argument("--roofline-sweeps", type=int, default=32, help="sweeps of the per-kernel event-timed pass")
    ap.add_argument("--learned-only", action="store_true", help="run only the learned-vs-plain comparison (one JSON object)")
    ap.add_argument("--learn-configs", type=int, default=10000)
    ap.add_argument("--learn-params", default="{}", help="JSON overrides of pp_learned_params (e.g. {\"jump\": 1e-3})")
    ap.add_argument("--learn-sweeps-between", type=int, default=5)
    ap.add_argument("--learn-epochs", type=int, default=30)
    ap.add_argument("--learn-measure-sweeps", type=int, default=200000, help="sweeps of each chain (plain and learned side by side)")
    ap.add_argument("--learn-every", type=int, default=100, help="sweeps between bond-count snapshots")
    ap.add_argument("--learn-time-sweeps", type=int, default=2000, help="sweeps of the per-chain cost measurement")
    ap.add_argument("--learn-T", type=float, default=0.09)
    ap.add_argument("--learn-large-sweeps", type=int, default=20, help="timed learned sweeps of the main workload")
    ap.add_argument("--learn-N", type=int, default=32768)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one rank per GPU: relaunch this command under torch.distributed.run (each rank runs an independent
        # replica; rank 0 prints the aggregate line)
        sys.exit(_spawn_ranks(args.gpus))
    ws_env = int(os.environ.get("WORLD_SIZE", "1"))
    if ws_env != args.gpus:
        sys.exit("bench.py: --gpus %d but WORLD_SIZE=%d: launch one rank per GPU" % (args.gpus, ws_env))
    wl = WORKLOADS.get(args.workload, WORKLOADS["c2"])
    ws, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, wl, ws, rank, dist)
    elif args.workload == "c3":
        run_batch(args, ws, rank, local, dist)
    elif args.learned_only:
        from patchyparticles_gb300 import build

        build.build()
        res = learned_comparison(args)
        res.pop("_weights")
        print(json.dumps({"learned": res}), flush=True)
    else:
        run_gpu(args, wl, ws, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
