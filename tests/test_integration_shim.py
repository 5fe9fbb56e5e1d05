"""The reference-side shim (patchyparticles_gb300/csrc/ppgpu_reference_shim.c, the binding a maintainer
adds to the reference as gpu_ensemble.c) compiles against the reference's own headers and this
repository's C-ABI header, and links against the reference's own library sources and libppgpu.so. Runs
only where the reference sources are present (oracle.pyoracle.reference_dir()); it compiles and links
them, never runs them."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.pyoracle import reference_dir

REF = reference_dir()
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
# the reference's library sources (makefile.common's object list without main.o)
REF_LIB_SRC = ["parse_input.c", "output.c", "system.c", "MC.c", "utils.c", "avb.c", "vmmc.c", "cells.c"]

# stands in for the reference's main.c and MC_init, which a maintainer's edits (MC_init selects the GPU
# ensemble, main.c syncs before output) make call these hooks
DRIVER = r"""
#include "defs.h"
#include "output.h"
int gpu_ensemble_init(System *syst, Output *IO, int seed);
void gpu_do_ensemble(System *syst, Output *IO);
void gpu_sync_system(System *syst, Output *IO);
void gpu_check_energy(System *syst, Output *IO);
int main(int argc, char *argv[]) {
	void (*hooks[])(System *, Output *) = { gpu_do_ensemble, gpu_sync_system, gpu_check_energy };
	(void) argv;
	return argc > 1000 ? gpu_ensemble_init(NULL, NULL, 0) + (hooks[argc % 3] == NULL) : 0;
}
"""

needs_ref = pytest.mark.skipif(REF is None or not os.path.isfile(os.path.join(REF, "defs.h")), reason="reference sources not present")


def shim_source():
    return open(os.path.join(ROOT, "patchyparticles_gb300", "csrc", "ppgpu_reference_shim.c")).read()


def gcc(args):
    return subprocess.run(["gcc", "-std=gnu99", "-Wall"] + args, capture_output=True, text=True)


@needs_ref
def test_shim_compiles_against_the_reference_headers():
    work = tempfile.mkdtemp(prefix="ppshim_")
    src = os.path.join(work, "gpu_ensemble.c")
    open(src, "w").write(shim_source())
    p = gcc(["-c", src, "-I", REF, "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
             "-o", os.path.join(work, "gpu_ensemble.o")])
    shutil.rmtree(work)
    assert p.returncode == 0, p.stderr
    assert "warning" not in p.stderr, p.stderr


@needs_ref
def test_shim_links_with_the_reference_and_the_engine(built):
    lib = os.path.join(ROOT, "patchyparticles_gb300", "libppgpu.so")
    assert os.path.isfile(lib)
    work = tempfile.mkdtemp(prefix="ppshim_")
    src = os.path.join(work, "gpu_ensemble.c")
    drv = os.path.join(work, "driver.c")
    open(src, "w").write(shim_source())
    open(drv, "w").write(DRIVER)
    p = gcc(["-w", "-o", os.path.join(work, "PatchyParticles_gpu"), drv, src] + [os.path.join(REF, f) for f in REF_LIB_SRC] +
            ["-I", REF, "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
             "-L", os.path.dirname(lib), "-lppgpu", "-Wl,-rpath-link," + os.path.join(CUDA, "lib64"), "-lm"])
    shutil.rmtree(work)
    assert p.returncode == 0, p.stderr
