"""The C-ABI library: loads, exports every declared symbol, validates parameters without a GPU."""
import ctypes
import os
import re

import pytest

import patchyparticles_gb300 as pp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "ppgpu.h")).read()
    return sorted(set(re.findall(r"^[a-z][\w \*]*?\b(pp_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("pp_gpu_create", "pp_gpu_upload", "pp_gpu_sweeps", "pp_gpu_energy", "pp_gpu_download", "pp_gpu_orthonormalise", "pp_gpu_bonds", "pp_gpu_last_error", "pp_gpu_destroy", "pp_gpu_create_batch"):
        assert n in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(pp.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_functions()) <= set(pp.EXPORTED) | set(declared_functions())


def test_default_params(built):
    p = pp.default_params()
    assert p.ensemble == pp.NVT and p.precision == pp.PREC_FP32_GUARD and p.guard_eps == 1e-5
    assert p.kf_delta == 0.12 and p.kf_cosmax == 0.92


@pytest.mark.parametrize("field,value", [("ensemble", 3), ("temperature", -1.0), ("kf_delta", 1.5), ("precision", 7), ("resort_every", 100)])
def test_invalid_parameters_are_rejected_before_device_use(built, field, value):
    p = pp.default_params(**{field: value})
    with pytest.raises(pp.PPError) as ei:
        pp.Engine(p)
    assert ei.value.code == pp.PP_ERR_ARG


def test_tensor_core_wait_hook_checks_its_limits_before_device_use(built):
    lib = pp.load_library()
    assert lib.pp_mlp_wait_test(0, 0, None, None) == pp.PP_ERR_ARG
    assert lib.pp_mlp_wait_test(1 << 40, 0, None, None) == pp.PP_ERR_ARG
    assert lib.pp_mlp_wait_test(1000, 2, None, None) == pp.PP_ERR_ARG
