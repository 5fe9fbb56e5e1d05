"""ctypes view of the oracle restatement (oracle/pp_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
never by the product. build() compiles the restatement with oracle/Makefile (and the reference build
under oracle/_ref when the reference sources are present).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libpporacle.so")
CLI = os.path.join(HERE, "_build", "pporacle")
REF_DIR = os.path.join(HERE, "_ref")

NVT = 0
GC = 1
SUS = 3
NPT = 5
RTMC = 0  # Dynamics (defs.h:27-29)
AVBMC = 2
AVB = 1  # tries / accepted slot of the AVB move (defs.h:13)
VMMC = 1  # Dynamics = 1: virtual-move cluster moves
MOVE_VMMC = 5  # its tries / accepted slot (defs.h:17)


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("ensemble", ctypes.c_int),
        ("T", ctypes.c_double),
        ("P", ctypes.c_double),
        ("disp_max", ctypes.c_double),
        ("theta_max", ctypes.c_double),
        ("rescale_factor_max", ctypes.c_double),
        ("kf_delta", ctypes.c_double),
        ("kf_cosmax", ctypes.c_double),
        ("seed", ctypes.c_int),
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
    ]


def reference_dir():
    """Directory of the reference's C sources: $PP_REFERENCE_DIR, else a checkout named `reference` beside
    this repository; None where neither holds them (e.g. on a machine that only runs the GPU tests)."""
    for d in (os.environ.get("PP_REFERENCE_DIR"), os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")):
        if d and os.path.isfile(os.path.join(d, "MC.c")):
            return os.path.abspath(d)
    return None


def build(with_reference=True):
    subprocess.check_call(["make", "-s", "-C", HERE, "port"])
    ref = reference_dir() if with_reference else None
    if ref is not None:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", "REF=" + ref])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(with_reference=False)
        L = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        llp = ctypes.POINTER(ctypes.c_longlong)
        sig = {
            "orc_load_rrr": (vp, [ctypes.c_char_p, ctypes.POINTER(OrcParams), ctypes.c_char_p, ctypes.c_int]),
            "orc_from_arrays": (vp, [ctypes.c_int, dp, dp, dp, ctypes.POINTER(OrcParams)]),
            "orc_free": (None, [vp]),
            "orc_N": (ctypes.c_int, [vp]),
            "orc_box": (None, [vp, dp]),
            "orc_volume": (ctypes.c_double, [vp]),
            "orc_get_energy": (ctypes.c_double, [vp]),
            "orc_set_energy": (None, [vp, ctypes.c_double]),
            "orc_get_state": (None, [vp, dp, dp]),
            "orc_get_patches": (None, [vp, dp]),
            "orc_counters": (None, [vp, llp, llp]),
            "orc_reset_counters": (None, [vp]),
            "orc_interact": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
            "orc_particle_energy": (ctypes.c_double, [vp, ctypes.c_int, ip]),
            "orc_energies": (ctypes.c_double, [vp, dp, ip, ip, ip]),
            "orc_bond_lists": (ctypes.c_int, [vp, ip, ip, ctypes.c_int]),
            "orc_sweep": (None, [vp]),
            "orc_sweeps": (None, [vp, ctypes.c_longlong]),
            "orc_check_energy": (ctypes.c_int, [vp]),
            "orc_save_rrr": (ctypes.c_int, [vp, ctypes.c_longlong, ctypes.c_char_p]),
            "orc_drand48_sequence": (None, [ctypes.c_int, ctypes.c_int, dp]),
            "orc_generate": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_int, dp, dp, dp]),
            "orc_error": (ctypes.c_int, [vp]),
            "orc_sus_hist": (ctypes.c_int, [vp, llp, ctypes.c_int]),
            "orc_parallel_throughput": (ctypes.c_double, [ctypes.c_int, dp, dp, dp, ctypes.POINTER(OrcParams), ctypes.c_int, ctypes.c_double, llp]),
            "orc_pool_create": (vp, [ctypes.c_int, dp, dp, dp, ctypes.POINTER(OrcParams), ctypes.c_int]),
            "orc_pool_run": (ctypes.c_double, [vp, ctypes.c_double, llp]),
            "orc_pool_free": (None, [vp]),
        }
        for k, (res, args) in sig.items():
            f = getattr(L, k)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def params(ensemble=NVT, T=0.12, P=0.0, disp_max=0.05, theta_max=0.1, rescale_factor_max=0.01, kf_delta=0.12, kf_cosmax=0.92, seed=1,
           lx_move=0, lx_change_max=0.0, lyz_min=0.0, lyz_max=0.0, activity=0.0, n_min=0, n_max=0, dynamics=0, avb_p=0.5, vmmc_max_cluster=0):
    return OrcParams(ensemble, T, P, disp_max, theta_max, rescale_factor_max, kf_delta, kf_cosmax, seed, lx_move, lx_change_max, lyz_min, lyz_max,
                     activity, n_min, n_max, dynamics, avb_p, vmmc_max_cluster)


class System:
    """One oracle system (a restated reference System)."""

    def __init__(self, prm, path=None, arrays=None):
        L = lib()
        self.L = L
        if path is not None:
            err = ctypes.create_string_buffer(512)
            self.h = L.orc_load_rrr(path.encode(), ctypes.byref(prm), err, 512)
            if not self.h:
                raise RuntimeError(err.value.decode())
        else:
            r, R, box = arrays
            r = np.ascontiguousarray(r, dtype=np.float64)
            R = np.ascontiguousarray(R, dtype=np.float64)
            box = np.ascontiguousarray(box, dtype=np.float64)
            self.h = L.orc_from_arrays(r.shape[0], _dp(r), _dp(R), _dp(box), ctypes.byref(prm))
            if not self.h:
                raise RuntimeError("oracle allocation failed")
        self.N = L.orc_N(self.h)

    def close(self):
        if self.h:
            self.L.orc_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def energies(self):
        N = self.N
        E = np.zeros(N)
        ov = np.zeros(N, dtype=np.int32)
        nb = np.zeros(N, dtype=np.int32)
        no = np.zeros(N, dtype=np.int32)
        tot = self.L.orc_energies(self.h, _dp(E), _ip(ov), _ip(nb), _ip(no))
        return tot, E, ov, nb, no

    def init_energy(self):
        """main.c:55-64: energy = 0.5 sum MC_energy; returns (E, overlap_any)."""
        tot, E, ov, _, _ = self.energies()
        self.L.orc_set_energy(self.h, tot)
        return tot, bool(ov.any())

    def bond_lists(self):
        _, _, _, nb, _ = self.energies()
        cap = int(nb.sum()) + 1
        off = np.zeros(self.N + 1, dtype=np.int32)
        part = np.zeros(cap, dtype=np.int32)
        n = self.L.orc_bond_lists(self.h, _ip(off), _ip(part), cap)
        return off, part[:n]

    def interact(self, i, j):
        return self.L.orc_interact(self.h, i, j)

    def sweeps(self, n):
        self.L.orc_sweeps(self.h, n)

    def energy(self):
        return self.L.orc_get_energy(self.h)

    def volume(self):
        return self.L.orc_volume(self.h)

    def box(self):
        b = np.zeros(3)
        self.L.orc_box(self.h, _dp(b))
        return b

    def state(self):
        r = np.zeros((self.N, 3))
        R = np.zeros((self.N, 9))
        self.L.orc_get_state(self.h, _dp(r), _dp(R))
        return r, R

    def patches(self):
        P = np.zeros((self.N, 12))
        self.L.orc_get_patches(self.h, _dp(P))
        return P

    def counters(self, reset=False):
        t = (ctypes.c_longlong * 8)()
        a = (ctypes.c_longlong * 8)()
        self.L.orc_counters(self.h, t, a)
        if reset:
            self.L.orc_reset_counters(self.h)
        return list(t), list(a)

    def check_energy(self):
        return self.L.orc_check_energy(self.h)

    def num_particles(self):
        """Current particle count (changes in the GC and SUS ensembles)."""
        return self.L.orc_N(self.h)

    def error(self):
        return self.L.orc_error(self.h)

    def sus_histogram(self, reset=False):
        n = self.L.orc_sus_hist(self.h, None, 0)
        h = (ctypes.c_longlong * max(n, 1))()
        self.L.orc_sus_hist(self.h, h, 1 if reset else 0)
        return list(h)[:n]

    def save(self, path, step=0):
        return self.L.orc_save_rrr(self.h, step, path.encode())


def generate(N, density, seed):
    """The reference generator's seeded random sequential insertion (generator.c:43-68): (r, R, box)."""
    r = np.zeros((N, 3))
    R = np.zeros((N, 9))
    b = np.zeros(3)
    if lib().orc_generate(N, density, seed, _dp(r), _dp(R), _dp(b)) != 0:
        raise ValueError("density must be in (0, 0.7]")
    return r, R, b


def generated_text(r, R, box):
    """generated.rrr as the reference generator prints it (generator.c:70-82)."""
    out = ["0 %d %f %f %f" % (len(r), box[0], box[1], box[2])]
    for i in range(len(r)):
        out.append("%f %f %f" % tuple(R[i, 0:3]))
        out.append("%f %f %f" % tuple(R[i, 3:6]))
        out.append("%.12f %.12f %.12f" % tuple(r[i]))
    return "\n".join(out) + "\n"


def drand48_sequence(seed, n):
    out = np.zeros(n)
    lib().orc_drand48_sequence(seed, n, _dp(out))
    return out


def parallel_throughput(r, R, box, prm, threads, seconds):
    r = np.ascontiguousarray(r, dtype=np.float64)
    R = np.ascontiguousarray(R, dtype=np.float64)
    box = np.ascontiguousarray(box, dtype=np.float64)
    att = ctypes.c_longlong()
    rate = lib().orc_parallel_throughput(r.shape[0], _dp(r), _dp(R), _dp(box), ctypes.byref(prm), threads, seconds, ctypes.byref(att))
    return rate, att.value


class Pool:
    """Independent oracle systems, one per thread, kept alive across bounded throughput samples."""

    def __init__(self, r, R, box, prm, threads):
        r = np.ascontiguousarray(r, dtype=np.float64)
        R = np.ascontiguousarray(R, dtype=np.float64)
        box = np.ascontiguousarray(box, dtype=np.float64)
        self.L = lib()
        self.threads = threads
        self.h = self.L.orc_pool_create(r.shape[0], _dp(r), _dp(R), _dp(box), ctypes.byref(prm), threads)
        if not self.h:
            raise RuntimeError("oracle pool allocation failed")

    def run(self, seconds):
        att = ctypes.c_longlong()
        rate = self.L.orc_pool_run(self.h, seconds, ctypes.byref(att))
        return rate, att.value

    def close(self):
        if self.h:
            self.L.orc_pool_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
