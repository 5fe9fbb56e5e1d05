"""Python view of the ppgpu C-ABI (include/ppgpu.h) for tests and benchmarks.

This module only binds the shared library libppgpu.so with ctypes: every computation runs in the CUDA
kernels behind the C-ABI. If the library has not been built (patchyparticles_gb300.build.build()), importing
works but any engine call raises, so a missing extension can never fall back to another implementation.

The names mirror the reference's per-step interface: an Engine replaces the System + do_ensemble pair of
PatchyParticles (defs.h:58-112, MC.c:85-131) for Dynamics = 0 in the NVT/NPT ensembles.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libppgpu.so")

PP_OK = 0
PP_ERR_ARG = -1
PP_ERR_CUDA = -2
PP_ERR_OVERLAP = -3
PP_ERR_CAPACITY = -4
PP_ERR_IO = -5
PP_ERR_STATE = -6
PP_ERR_DRIFT = -7

NVT = 0
GC = 1
SUS = 3
NPT = 5
RTMC = 0  # Dynamics: roto-translations
VMMC = 1  # Dynamics: virtual-move cluster moves
AVBMC = 2  # Dynamics: aggregation-volume-bias moves and roto-translations
PREC_FP32_GUARD = 0
PREC_FP64 = 1
MOVE_ROTO_TRASL = 0
MOVE_ADD = 2
MOVE_REMOVE = 3
MOVE_AVB = 1
MOVE_VMMC = 5
MOVE_VOLUME = 6
MOVE_LX = 7
N_MOVES = 8


class PPParams(ctypes.Structure):
    _fields_ = [
        ("ensemble", ctypes.c_int),
        ("temperature", ctypes.c_double),
        ("pressure", ctypes.c_double),
        ("disp_max", ctypes.c_double),
        ("theta_max", ctypes.c_double),
        ("rescale_factor_max", ctypes.c_double),
        ("kf_delta", ctypes.c_double),
        ("kf_cosmax", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("precision", ctypes.c_int),
        ("guard_eps", ctypes.c_double),
        ("resort_every", ctypes.c_int),
        ("audit", ctypes.c_int),
        ("lx_move", ctypes.c_int),
        ("lx_change_max", ctypes.c_double),
        ("lyz_min", ctypes.c_double),
        ("lyz_max", ctypes.c_double),
        ("activity", ctypes.c_double),
        ("n_min", ctypes.c_int),
        ("n_max", ctypes.c_int),
        ("dynamics", ctypes.c_int),
        ("avb_p", ctypes.c_double),
        ("vmmc_max_cluster", ctypes.c_int),
        ("vmmc_max_move", ctypes.c_double),
    ]


class PPCounters(ctypes.Structure):
    _fields_ = [("tries", ctypes.c_longlong * N_MOVES), ("accepted", ctypes.c_longlong * N_MOVES)]


class PPGuardStats(ctypes.Structure):
    _fields_ = [
        ("pairs", ctypes.c_longlong),
        ("fallbacks", ctypes.c_longlong),
        ("mismatches", ctypes.c_longlong),
        ("max_err_r2", ctypes.c_double),
        ("max_err_cos", ctypes.c_double),
        ("nl_overflows", ctypes.c_longlong),
    ]


class PPKernelStats(ctypes.Structure):
    _fields_ = [
        ("sweep_ms", ctypes.c_double),
        ("sweep_launches", ctypes.c_longlong),
        ("sort_ms", ctypes.c_double),
        ("sort_launches", ctypes.c_longlong),
        ("volume_ms", ctypes.c_double),
        ("volume_launches", ctypes.c_longlong),
    ]


class PPLearnedParams(ctypes.Structure):
    _fields_ = [
        ("scale_disp", ctypes.c_double * 4),
        ("scale_theta", ctypes.c_double * 4),
        ("floor", ctypes.c_double),
        ("entropy", ctypes.c_double),
        ("kappa", ctypes.c_double),
        ("jump", ctypes.c_double),
        ("draws", ctypes.c_int),
        ("seed", ctypes.c_uint64),
    ]


PROPOSAL_PLAIN = 0
PROPOSAL_LEARNED = 1


class PPTuneResult(ctypes.Structure):
    _fields_ = [
        ("resort_every", ctypes.c_int),
        ("reorder_every", ctypes.c_int),
        ("cell_scale", ctypes.c_double),
        ("attempts_per_s", ctypes.c_double),
        ("baseline_attempts_per_s", ctypes.c_double),
        ("n_tried", ctypes.c_int),
        ("neighbour_lists", ctypes.c_int),
    ]


class PPError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"ppgpu error {code}: {message}")
        self.code = code
        self.message = message


_lib = None

# exported symbols of include/ppgpu.h
EXPORTED = [
    "pp_default_params", "pp_gpu_create", "pp_gpu_create_batch", "pp_gpu_upload", "pp_gpu_upload_replica",
    "pp_gpu_sweeps", "pp_gpu_sync", "pp_gpu_get_energy", "pp_gpu_energy", "pp_gpu_check_energy",
    "pp_gpu_orthonormalise", "pp_gpu_counters", "pp_gpu_download", "pp_gpu_download_replica", "pp_gpu_bonds",
    "pp_gpu_bond_lists", "pp_gpu_guard_stats", "pp_gpu_num_replicas", "pp_gpu_num_particles", "pp_gpu_box",
    "pp_gpu_launch_count", "pp_gpu_last_error", "pp_gpu_destroy", "pp_rrr_header", "pp_rrr_read", "pp_rrr_write",
    "pp_generate", "pp_gpu_select_device", "pp_gpu_set_timing", "pp_gpu_kernel_stats", "pp_gpu_time_sweeps",
    "pp_gpu_energy_noalloc", "pp_mlp_forward", "pp_mlp_grad", "pp_default_learned_params", "pp_gpu_learned_init",
    "pp_gpu_learned_set_weights", "pp_gpu_learned_get_weights", "pp_gpu_set_proposal", "pp_gpu_learned_collect",
    "pp_gpu_learned_train", "pp_gpu_learned_samples", "pp_gpu_learned_clear_samples", "pp_gpu_learned_features",
    "pp_gpu_learned_stats", "pp_gpu_autotune", "pp_gpu_set_graphs", "pp_gpu_set_neighbour_lists",
    "pp_gpu_set_persistent", "pp_gpu_set_barrier_test", "pp_gpu_sus_histogram", "pp_mlp_wait_test",
]


def load_library(path=None):
    """Loads libppgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libppgpu.so not found at {p}: build it with patchyparticles_gb300.build.build()")
    lib = ctypes.CDLL(p)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    fp = ctypes.POINTER(ctypes.c_float)
    vp = ctypes.c_void_p
    sig = {
        "pp_default_params": (None, [ctypes.POINTER(PPParams)]),
        "pp_gpu_create": (ctypes.c_int, [ctypes.POINTER(PPParams), ctypes.POINTER(vp)]),
        "pp_gpu_create_batch": (ctypes.c_int, [ctypes.POINTER(PPParams), ctypes.c_int, ctypes.POINTER(vp)]),
        "pp_gpu_upload": (ctypes.c_int, [vp, ctypes.c_int, dp, dp, dp]),
        "pp_gpu_upload_replica": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, dp, dp, dp]),
        "pp_gpu_sweeps": (ctypes.c_int, [vp, ctypes.c_longlong]),
        "pp_gpu_sync": (ctypes.c_int, [vp]),
        "pp_gpu_get_energy": (ctypes.c_int, [vp, ctypes.c_int, dp]),
        "pp_gpu_energy": (ctypes.c_int, [vp, ctypes.c_int, dp, ip]),
        "pp_gpu_check_energy": (ctypes.c_int, [vp, ctypes.c_int]),
        "pp_gpu_orthonormalise": (ctypes.c_int, [vp, ctypes.c_int]),
        "pp_gpu_counters": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(PPCounters), ctypes.c_int]),
        "pp_gpu_download": (ctypes.c_int, [vp, dp, dp, dp]),
        "pp_gpu_download_replica": (ctypes.c_int, [vp, ctypes.c_int, dp, dp, dp]),
        "pp_gpu_bonds": (ctypes.c_int, [vp, ctypes.c_int, ip, ip]),
        "pp_gpu_bond_lists": (ctypes.c_int, [vp, ctypes.c_int, ip, ip, ctypes.c_int]),
        "pp_gpu_guard_stats": (ctypes.c_int, [vp, ctypes.POINTER(PPGuardStats), ctypes.c_int]),
        "pp_gpu_num_replicas": (ctypes.c_int, [vp]),
        "pp_gpu_num_particles": (ctypes.c_int, [vp, ctypes.c_int]),
        "pp_gpu_box": (ctypes.c_int, [vp, ctypes.c_int, dp]),
        "pp_gpu_launch_count": (ctypes.c_longlong, [vp]),
        "pp_gpu_last_error": (ctypes.c_char_p, [vp]),
        "pp_gpu_destroy": (None, [vp]),
        "pp_rrr_header": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong), ip, dp]),
        "pp_rrr_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, dp, dp, dp, ctypes.c_char_p, ctypes.c_int]),
        "pp_rrr_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_longlong, ctypes.c_int, dp, dp, dp]),
        "pp_generate": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, dp, dp, dp]),
        "pp_gpu_select_device": (ctypes.c_int, [ctypes.c_int]),
        "pp_gpu_set_timing": (ctypes.c_int, [vp, ctypes.c_int]),
        "pp_gpu_kernel_stats": (ctypes.c_int, [vp, ctypes.POINTER(PPKernelStats), ctypes.c_int]),
        "pp_gpu_time_sweeps": (ctypes.c_int, [vp, ctypes.c_longlong, dp]),
        "pp_mlp_forward": (ctypes.c_int, [fp, ctypes.c_int, fp, fp]),
        "pp_default_learned_params": (None, [ctypes.POINTER(PPLearnedParams)]),
        "pp_gpu_learned_init": (ctypes.c_int, [vp, ctypes.POINTER(PPLearnedParams)]),
        "pp_gpu_learned_set_weights": (ctypes.c_int, [vp, fp]),
        "pp_gpu_learned_get_weights": (ctypes.c_int, [vp, fp]),
        "pp_gpu_set_proposal": (ctypes.c_int, [vp, ctypes.c_int]),
        "pp_gpu_learned_collect": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "pp_gpu_learned_train": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp]),
        "pp_gpu_learned_samples": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_longlong), fp]),
        "pp_gpu_learned_clear_samples": (ctypes.c_int, [vp]),
        "pp_gpu_learned_features": (ctypes.c_int, [vp, ctypes.c_int, fp]),
        "pp_gpu_learned_stats": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
        "pp_gpu_autotune": (ctypes.c_int, [vp, ctypes.c_int, ctypes.POINTER(PPTuneResult)]),
        "pp_gpu_set_graphs": (ctypes.c_int, [vp, ctypes.c_int]),
        "pp_gpu_set_neighbour_lists": (ctypes.c_int, [vp, ctypes.c_int]),
        "pp_gpu_set_persistent": (ctypes.c_int, [vp, ctypes.c_int]),
        "pp_gpu_sus_histogram": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
        "pp_gpu_set_barrier_test": (ctypes.c_int, [vp, ctypes.c_longlong, ctypes.c_int]),
        "pp_mlp_grad": (ctypes.c_int, [fp, ctypes.c_int, fp, ctypes.c_double, ctypes.c_double, ctypes.c_int, fp, dp]),
        "pp_mlp_wait_test": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def default_params(**kw):
    lib = load_library()
    p = PPParams()
    lib.pp_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


class Engine:
    """One engine = one or several independent systems (replicas) on the GPU."""

    def __init__(self, params):
        self.lib = load_library()
        plist = params if isinstance(params, (list, tuple)) else [params]
        arr = (PPParams * len(plist))(*plist)
        h = ctypes.c_void_p()
        rc = self.lib.pp_gpu_create_batch(arr, len(plist), ctypes.byref(h))
        self.h = h
        if rc != PP_OK:
            msg = self.lib.pp_gpu_last_error(h).decode() if h.value else "create failed"
            if h.value:
                self.lib.pp_gpu_destroy(h)
            self.h = ctypes.c_void_p()
            raise PPError(rc, msg)
        self.nrep = len(plist)
        self.params = list(plist)

    def _check(self, rc):
        if rc != PP_OK:
            raise PPError(rc, self.lib.pp_gpu_last_error(self.h).decode())

    def close(self):
        if self.h and self.h.value:
            self.lib.pp_gpu_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, r, R, box, replica=0):
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(-1, 3)
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(-1, 9)
        box = np.ascontiguousarray(box, dtype=np.float64).reshape(3)
        assert r.shape[0] == R.shape[0]
        self._check(self.lib.pp_gpu_upload_replica(self.h, replica, r.shape[0], _dp(r), _dp(R), _dp(box)))

    def sweeps(self, n):
        self._check(self.lib.pp_gpu_sweeps(self.h, n))

    def sync(self):
        self._check(self.lib.pp_gpu_sync(self.h))

    def energy(self, replica=0):
        E = ctypes.c_double()
        ov = ctypes.c_int()
        self._check(self.lib.pp_gpu_energy(self.h, replica, ctypes.byref(E), ctypes.byref(ov)))
        return E.value, bool(ov.value)

    def tracked_energy(self, replica=0):
        E = ctypes.c_double()
        self._check(self.lib.pp_gpu_get_energy(self.h, replica, ctypes.byref(E)))
        return E.value

    def check_energy(self, replica=0):
        self._check(self.lib.pp_gpu_check_energy(self.h, replica))

    def orthonormalise(self, replica=0):
        self._check(self.lib.pp_gpu_orthonormalise(self.h, replica))

    def counters(self, replica=0, reset=False):
        c = PPCounters()
        self._check(self.lib.pp_gpu_counters(self.h, replica, ctypes.byref(c), 1 if reset else 0))
        return list(c.tries), list(c.accepted)

    def num_particles(self, replica=0):
        """Current particle count (changes in the GC and SUS ensembles)."""
        return self.lib.pp_gpu_num_particles(self.h, replica)

    def sus_histogram(self, reset=False):
        """SUS: counts of N after every insertion / removal attempt, bins n_min .. n_max."""
        n = self.params[0].n_max - self.params[0].n_min + 1
        h = (ctypes.c_longlong * n)()
        self._check(self.lib.pp_gpu_sus_histogram(self.h, h, 1 if reset else 0))
        return list(h)

    def box(self, replica=0):
        b = np.zeros(3)
        self._check(self.lib.pp_gpu_box(self.h, replica, _dp(b)))
        return b

    def download(self, replica=0):
        N = self.num_particles(replica)
        r = np.zeros((N, 3))
        R = np.zeros((N, 9))
        b = np.zeros(3)
        self._check(self.lib.pp_gpu_download_replica(self.h, replica, _dp(r), _dp(R), _dp(b)))
        return r, R, b

    def bonds(self, replica=0):
        N = self.num_particles(replica)
        nb = np.zeros(N, dtype=np.int32)
        no = np.zeros(N, dtype=np.int32)
        self._check(self.lib.pp_gpu_bonds(self.h, replica, _ip(nb), _ip(no)))
        return nb, no

    def bond_lists(self, replica=0):
        N = self.num_particles(replica)
        nb, _ = self.bonds(replica)
        cap = int(nb.sum()) + 1
        off = np.zeros(N + 1, dtype=np.int32)
        part = np.zeros(cap, dtype=np.int32)
        rc = self.lib.pp_gpu_bond_lists(self.h, replica, _ip(off), _ip(part), cap)
        if rc < 0:
            self._check(rc)
        return off, part[:rc]

    def guard_stats(self, reset=False):
        g = PPGuardStats()
        self._check(self.lib.pp_gpu_guard_stats(self.h, ctypes.byref(g), 1 if reset else 0))
        return {k: getattr(g, k) for k, _ in PPGuardStats._fields_}

    def launch_count(self):
        return self.lib.pp_gpu_launch_count(self.h)

    def set_timing(self, enable=True):
        self._check(self.lib.pp_gpu_set_timing(self.h, 1 if enable else 0))

    def kernel_stats(self, reset=False):
        k = PPKernelStats()
        self._check(self.lib.pp_gpu_kernel_stats(self.h, ctypes.byref(k), 1 if reset else 0))
        return {f: getattr(k, f) for f, _ in PPKernelStats._fields_}

    def time_sweeps(self, n):
        ms = ctypes.c_double()
        self._check(self.lib.pp_gpu_time_sweeps(self.h, n, ctypes.byref(ms)))
        return ms.value

    def set_graphs(self, enable=True):
        self._check(self.lib.pp_gpu_set_graphs(self.h, 1 if enable else 0))

    def set_neighbour_lists(self, enable=True):
        self._check(self.lib.pp_gpu_set_neighbour_lists(self.h, 1 if enable else 0))

    def set_persistent(self, enable=True):
        """Plain rounds over the neighbour lists as one persistent cooperative launch (default) or one launch
        per colour; the trajectory is the same."""
        self._check(self.lib.pp_gpu_set_persistent(self.h, 1 if enable else 0))

    def set_barrier_test(self, limit_cycles=0, unreachable=False):
        """Failure-detection hook of the persistent kernel's grid barrier (see include/ppgpu.h)."""
        self._check(self.lib.pp_gpu_set_barrier_test(self.h, int(limit_cycles), 1 if unreachable else 0))

    def autotune(self, trial_sweeps=20):
        t = PPTuneResult()
        self._check(self.lib.pp_gpu_autotune(self.h, trial_sweeps, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in PPTuneResult._fields_}

    # ---------------------------------------------------------------- learned proposal
    def learned_init(self, **kw):
        p = default_learned_params(**kw)
        self._check(self.lib.pp_gpu_learned_init(self.h, ctypes.byref(p)))

    def set_proposal(self, learned):
        self._check(self.lib.pp_gpu_set_proposal(self.h, PROPOSAL_LEARNED if learned else PROPOSAL_PLAIN))

    def learned_weights(self):
        P = np.zeros(MLP_NPARAMS, dtype=np.float32)
        self._check(self.lib.pp_gpu_learned_get_weights(self.h, _fp(P)))
        return P

    def set_learned_weights(self, P):
        P = np.ascontiguousarray(P, dtype=np.float32).reshape(MLP_NPARAMS)
        self._check(self.lib.pp_gpu_learned_set_weights(self.h, _fp(P)))

    def learned_collect(self, n_configs, sweeps_between, samples_per_config):
        self._check(self.lib.pp_gpu_learned_collect(self.h, n_configs, sweeps_between, samples_per_config))

    def learned_train(self, epochs, lr=3e-3, tiles_per_cta=2):
        obj = ctypes.c_double()
        self._check(self.lib.pp_gpu_learned_train(self.h, epochs, tiles_per_cta, lr, ctypes.byref(obj)))
        return obj.value

    def learned_samples(self):
        n = ctypes.c_longlong()
        self._check(self.lib.pp_gpu_learned_samples(self.h, ctypes.byref(n), None))
        out = np.zeros((n.value, MLP_SAMPLE), dtype=np.float32)
        if n.value:
            self._check(self.lib.pp_gpu_learned_samples(self.h, ctypes.byref(n), _fp(out)))
        return out

    def learned_clear_samples(self):
        self._check(self.lib.pp_gpu_learned_clear_samples(self.h))

    def learned_features(self, replica=0):
        N = self.num_particles(replica)
        f = np.zeros((N, MLP_IN), dtype=np.float32)
        self._check(self.lib.pp_gpu_learned_features(self.h, replica, _fp(f)))
        return f

    def learned_stats(self, reset=False):
        t = (ctypes.c_longlong * 4)()
        a = (ctypes.c_longlong * 4)()
        self._check(self.lib.pp_gpu_learned_stats(self.h, t, a, 1 if reset else 0))
        return list(t), list(a)


def default_learned_params(**kw):
    lib = load_library()
    p = PPLearnedParams()
    lib.pp_default_learned_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        if k in ("scale_disp", "scale_theta"):
            for i, x in enumerate(v):
                getattr(p, k)[i] = x
        else:
            setattr(p, k, v)
    return p


def select_device(dev):
    rc = load_library().pp_gpu_select_device(dev)
    if rc != PP_OK:
        raise PPError(rc, f"cannot select CUDA device {dev}")


def rrr_header(path):
    lib = load_library()
    st = ctypes.c_longlong()
    n = ctypes.c_int()
    b = np.zeros(3)
    rc = lib.pp_rrr_header(path.encode(), ctypes.byref(st), ctypes.byref(n), _dp(b))
    if rc != PP_OK:
        raise PPError(rc, f"cannot read header of {path}")
    return st.value, n.value, b


def read_rrr(path):
    """Reads a .rrr file exactly as the reference's system_init does. Returns (step, r, R, box)."""
    lib = load_library()
    step, N, _ = rrr_header(path)
    r = np.zeros((N, 3))
    R = np.zeros((N, 9))
    b = np.zeros(3)
    err = ctypes.create_string_buffer(512)
    rc = lib.pp_rrr_read(path.encode(), N, _dp(r), _dp(R), _dp(b), err, 512)
    if rc != PP_OK:
        raise PPError(rc, err.value.decode())
    return step, r, R, b


def write_rrr(path, step, r, R, box):
    lib = load_library()
    r = np.ascontiguousarray(r, dtype=np.float64)
    R = np.ascontiguousarray(R, dtype=np.float64)
    box = np.ascontiguousarray(box, dtype=np.float64)
    rc = lib.pp_rrr_write(path.encode(), step, r.shape[0], _dp(r), _dp(R), _dp(box))
    if rc != PP_OK:
        raise PPError(rc, f"cannot write {path}")


def generate(N, density, seed, round_like_file=True):
    """Seeded random sequential insertion (the reference generator's algorithm). Returns (r, R, box)."""
    lib = load_library()
    r = np.zeros((N, 3))
    R = np.zeros((N, 9))
    b = np.zeros(3)
    rc = lib.pp_generate(N, density, seed, 1 if round_like_file else 0, _dp(r), _dp(R), _dp(b))
    if rc != PP_OK:
        raise PPError(rc, "generation failed (density must be in (0, 0.7])")
    return r, R, b


# ---------------------------------------------------------------- learned proposal: the network
MLP_IN = 36
MLP_HIDDEN = 64
MLP_OUT = 4
MLP_NPARAMS = 6788
MLP_SAMPLE = 40


def mlp_forward(params, x):
    """Logits z[n][4] of the per-particle network on the tensor cores (x: n x 36 FP32)."""
    lib = load_library()
    P = np.ascontiguousarray(params, dtype=np.float32).reshape(MLP_NPARAMS)
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_IN)
    z = np.zeros((x.shape[0], MLP_OUT), dtype=np.float32)
    rc = lib.pp_mlp_forward(_fp(P), x.shape[0], _fp(x), _fp(z))
    if rc != PP_OK:
        raise PPError(rc, "pp_mlp_forward failed")
    return z


def mlp_grad(params, samples, floor=0.1, tau=0.01, tiles_per_cta=1):
    """(gradient[6788], mean objective) of one training batch (samples: n x 40) on the tensor cores."""
    lib = load_library()
    P = np.ascontiguousarray(params, dtype=np.float32).reshape(MLP_NPARAMS)
    S = np.ascontiguousarray(samples, dtype=np.float32).reshape(-1, MLP_SAMPLE)
    g = np.zeros(MLP_NPARAMS, dtype=np.float32)
    obj = ctypes.c_double()
    rc = lib.pp_mlp_grad(_fp(P), S.shape[0], _fp(S), floor, tau, tiles_per_cta, _fp(g), ctypes.byref(obj))
    if rc != PP_OK:
        raise PPError(rc, "pp_mlp_grad failed")
    return g, obj.value


def mlp_wait_test(limit_cycles, arrive):
    """Runs the tensor-core kernels' bounded mbarrier wait alone (pp_mlp_wait_test): returns
    (status code, whether the wait gave up, cycles waited). arrive=False makes the wait run out."""
    lib = load_library()
    t = ctypes.c_int(-1)
    c = ctypes.c_longlong(-1)
    rc = lib.pp_mlp_wait_test(int(limit_cycles), 1 if arrive else 0, ctypes.byref(t), ctypes.byref(c))
    if rc not in (PP_OK, PP_ERR_CUDA):
        raise PPError(rc, "pp_mlp_wait_test failed")
    return rc, bool(t.value), c.value
