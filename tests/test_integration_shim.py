"""The reference-side shim shown in INTEGRATION.md compiles against the reference's own headers and this
repository's C-ABI header (the binding a maintainer would add). Runs only where the reference sources are
present (the container that builds the oracle from them); it reads them, never runs them."""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("PP_REFERENCE_DIR", "/root/reference")


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "defs.h")), reason="reference sources not present")
def test_shim_compiles_against_the_reference_headers():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```c\n(.*?)```", text, re.S)
    shim = [b for b in blocks if "gpu_do_ensemble" in b]
    assert shim, "the shim is missing from INTEGRATION.md"
    work = tempfile.mkdtemp(prefix="ppshim_")
    src = os.path.join(work, "gpu_ensemble.c")
    open(src, "w").write(shim[0])
    p = subprocess.run(["gcc", "-std=gnu99", "-Wall", "-c", src, "-I", REF, "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
                        "-o", os.path.join(work, "gpu_ensemble.o")], capture_output=True, text=True)
    shutil.rmtree(work)
    assert p.returncode == 0, p.stderr
