"""pp_gpu_energy_noalloc: the energy entry point for callers that may not allocate device memory (hosts
running inside a device-memory budget or pool they do not own, latency-sensitive loops that cannot
afford cudaMalloc/cudaFree and their implicit device synchronisation).

The caller owns every buffer (here torch allocates them, as a host application's pool would); the
entry point only uses its static scratch array. Its results must equal the engine's own energy and
per-particle bond/overlap counts exactly (integers), on consecutive calls with different
configurations, and sizes beyond the static limit must be refused with PP_ERR_CAPACITY.
"""
import ctypes

import numpy as np
import pytest

from tests import helpers
import patchyparticles_gb300 as pp

pytestmark = pytest.mark.gpu


def _bind():
    lib = pp.load_library()
    f = lib.pp_gpu_energy_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, ctypes.c_int]
    return f


def _call(f, torch, r, R, box, with_outputs=True):
    N = len(r)
    r_t = torch.tensor(np.ascontiguousarray(r), dtype=torch.float64, device="cuda")
    R_t = torch.tensor(np.ascontiguousarray(R), dtype=torch.float64, device="cuda")
    nb_t = torch.full((max(N, 1),), -1, dtype=torch.int32, device="cuda")
    no_t = torch.full((max(N, 1),), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    E = ctypes.c_double()
    ov = ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    b = (ctypes.c_double * 3)(*[float(x) for x in box])
    rc = f(N, r_t.data_ptr(), R_t.data_ptr(), b, 0.12, 0.92, nb_t.data_ptr() if with_outputs else None, no_t.data_ptr() if with_outputs else None,
           ctypes.byref(E), ctypes.byref(ov), err, 256)
    return rc, E.value, bool(ov.value), nb_t.cpu().numpy()[:N], no_t.cpu().numpy()[:N], err.value.decode()


def _engine_reference(r, R, box):
    e = pp.Engine(pp.default_params())
    try:
        e.upload(r, R, box)
    except pp.PPError as x:
        if x.code != pp.PP_ERR_OVERLAP:
            raise
    nb, no = e.bonds()
    E, ov = e.energy()
    e.close()
    return E, ov, nb, no


def test_noalloc_energy_equals_engine_on_consecutive_calls(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    f = _bind()
    # three calls in a row, different sizes and densities: nothing of a previous call may leak into the next
    for name in ("c2", "c3", "adversarial", "c2"):
        r, R, box = helpers.config(name)
        E_ref, ov_ref, nb_ref, no_ref = _engine_reference(r, R, box)
        rc, E, ov, nb, no, msg = _call(f, torch, r, R, box)
        assert rc == pp.PP_OK, msg
        assert ov == ov_ref
        assert np.array_equal(nb, nb_ref) and np.array_equal(no, no_ref)
        if not ov_ref:
            assert E == E_ref
    # the per-particle outputs are optional
    r, R, box = helpers.config("c5")
    E_ref, _, _, _ = _engine_reference(r, R, box)
    rc, E, ov, _, _, msg = _call(f, torch, r, R, box, with_outputs=False)
    assert rc == pp.PP_OK, msg
    assert E == E_ref and not ov


def test_noalloc_rejects_sizes_beyond_the_static_limit(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    f = _bind()
    r, R, box = pp.generate(32769, 0.3, 9, round_like_file=False)
    rc, _, _, _, _, msg = _call(f, torch, r, R, box)
    assert rc == pp.PP_ERR_CAPACITY and "32768" in msg
    r, R, box = pp.generate(20000, 0.05, 9, round_like_file=False)  # box of ~73.7: 64^3 > 131072 cells
    rc, _, _, _, _, msg = _call(f, torch, r, R, box)
    assert rc == pp.PP_ERR_CAPACITY and "cells" in msg
