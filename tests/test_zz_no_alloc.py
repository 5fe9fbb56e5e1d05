"""pp_gpu_energy_noalloc: the energy entry point for callers that may not allocate device memory (hosts
running inside a device-memory budget or pool they do not own, latency-sensitive loops that cannot
afford cudaMalloc/cudaFree and their implicit device synchronisation).

The caller owns every buffer (here torch allocates them, as a host application's pool would); the
entry point only uses its static scratch array. Checked here:
- per-particle bond and overlap counts and the energy equal the reference's own probes (tests/golden),
  exactly (integers);
- two calls in a row, on different configurations, equal the engine's own entry points
  (pp_gpu_bonds / pp_gpu_energy) exactly: nothing of one call leaks into the next;
- the calls change the device's free memory by nothing;
- N = 0 gives E = 0 and no overlap; sizes beyond the static limits are refused with PP_ERR_CAPACITY.

This file is collected last, so that a run that stops at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

from tests import helpers
import patchyparticles_gb300 as pp

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return torch


def _bind():
    lib = pp.load_library()
    f = lib.pp_gpu_energy_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, ctypes.c_int]
    return f


class _Buffers:
    """The caller's device buffers of one configuration (allocated before any call)."""

    def __init__(self, torch, r, R, box):
        self.N = len(r)
        self.box = box
        self.r = torch.tensor(np.ascontiguousarray(r).reshape(-1), dtype=torch.float64, device="cuda")
        self.R = torch.tensor(np.ascontiguousarray(R).reshape(-1), dtype=torch.float64, device="cuda")
        self.nb = torch.full((max(self.N, 1),), -1, dtype=torch.int32, device="cuda")
        self.no = torch.full((max(self.N, 1),), -1, dtype=torch.int32, device="cuda")


def _call(f, B, with_outputs=True):
    E = ctypes.c_double()
    ov = ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    b = (ctypes.c_double * 3)(*[float(x) for x in B.box])
    rc = f(B.N, B.r.data_ptr() if B.N else None, B.R.data_ptr() if B.N else None, b, 0.12, 0.92,
           B.nb.data_ptr() if with_outputs else None, B.no.data_ptr() if with_outputs else None,
           ctypes.byref(E), ctypes.byref(ov), err, 256)
    return rc, E.value, bool(ov.value), err.value.decode()


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


@pytest.mark.parametrize("name", ["c1", "c2", "c3", "c5", "small", "fcc", "adversarial"])
def test_noalloc_equals_the_reference_probes(built, name):
    torch = _torch()
    f = _bind()
    r, R, box = helpers.config(name)
    N, Etot, anyov, _, _, nb_ref, no_ref, _ = helpers.parse_probe(name)
    B = _Buffers(torch, r, R, box)
    torch.cuda.synchronize()
    rc, E, ov, msg = _call(f, B)
    assert rc == pp.PP_OK, msg
    assert ov == bool(anyov)
    assert np.array_equal(B.nb.cpu().numpy()[:N], nb_ref) and np.array_equal(B.no.cpu().numpy()[:N], no_ref)
    if not anyov:
        assert E == Etot


def test_noalloc_two_calls_in_a_row_equal_the_engine_and_allocate_nothing(built):
    torch = _torch()
    f = _bind()
    names = ("c2", "c3", "adversarial", "c2")
    cfgs = [helpers.config(n) for n in names]
    refs = [_engine_reference(*c) for c in cfgs]  # the engine allocates: before the measured calls
    bufs = [_Buffers(torch, *c) for c in cfgs]
    empty = _Buffers(torch, np.zeros((0, 3)), np.zeros((0, 9)), cfgs[0][2])
    torch.cuda.synchronize()
    rc, _, _, msg = _call(f, bufs[0])  # warm-up: the module is loaded by now, the array exists
    assert rc == pp.PP_OK, msg
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    results = []
    for B in bufs:  # consecutive calls, different sizes and densities
        results.append(_call(f, B))
    rc0, E0, ov0, msg0 = _call(f, empty)
    rc1, E1, ov1, msg1 = _call(f, bufs[1], with_outputs=False)  # the per-particle outputs are optional
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "device free memory changed by %d bytes across the calls" % (free0 - free1)
    for (rc, E, ov, msg), B, (E_ref, ov_ref, nb_ref, no_ref) in zip(results, bufs, refs):
        assert rc == pp.PP_OK, msg
        assert ov == ov_ref
        assert np.array_equal(B.nb.cpu().numpy()[:B.N], nb_ref) and np.array_equal(B.no.cpu().numpy()[:B.N], no_ref)
        if not ov_ref:
            assert E == E_ref
    assert rc0 == pp.PP_OK and E0 == 0.0 and not ov0, msg0
    assert rc1 == pp.PP_OK and E1 == refs[1][0] and ov1 == refs[1][1], msg1


def test_noalloc_rejects_sizes_beyond_the_static_limit(built):
    torch = _torch()
    f = _bind()
    r, R, box = pp.generate(32769, 0.3, 9, round_like_file=False)
    rc, _, _, msg = _call(f, _Buffers(torch, r, R, box))
    assert rc == pp.PP_ERR_CAPACITY and "32768" in msg
    r, R, box = pp.generate(20000, 0.05, 9, round_like_file=False)  # box of ~73.7: 64^3 > 131072 cells
    rc, _, _, msg = _call(f, _Buffers(torch, r, R, box))
    assert rc == pp.PP_ERR_CAPACITY and "cells" in msg
