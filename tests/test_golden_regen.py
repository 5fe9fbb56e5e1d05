"""The committed golden fixtures are the reference's own outputs: tests/golden/make_golden.py rebuilds the
reference from its sources (oracle/Makefile), reruns its programs into a scratch directory, and every
fixture it writes must equal the committed one byte for byte. Runs only where the reference sources are
present (oracle.pyoracle.reference_dir())."""
import filecmp
import os
import shutil
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
from oracle.pyoracle import reference_dir

REF = reference_dir()


def fixture_files(top):
    out = []
    for d, dirs, files in os.walk(top):
        # equilibrated/ comes from make_equilibrated.py (a GPU pre-equilibration), not from the reference
        dirs[:] = [x for x in dirs if x not in ("__pycache__", "equilibrated")]
        for f in files:
            if f.endswith((".py", ".pyc")):
                continue
            out.append(os.path.relpath(os.path.join(d, f), top))
    return sorted(out)


@pytest.mark.skipif(REF is None or not os.path.isfile(os.path.join(REF, "MC.c")), reason="reference sources not present")
def test_fixtures_regenerate_byte_for_byte():
    out = tempfile.mkdtemp(prefix="ppgolden_")
    try:
        subprocess.run([sys.executable, os.path.join(GOLDEN, "make_golden.py"), REF, out], check=True,
                       capture_output=True, cwd=ROOT, timeout=600)
        made = fixture_files(out)
        assert made == fixture_files(GOLDEN)
        _, mismatch, errors = filecmp.cmpfiles(GOLDEN, out, made, shallow=False)
        assert not mismatch and not errors, (mismatch, errors)
    finally:
        shutil.rmtree(out)
