"""Shared test helpers: golden fixture access and small oracle/engine utilities."""
import gzip
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

# synthetic configurations whose reference probes are in tests/golden (see make_golden.py)
GENERATED = {
    "c1": (1000, 0.1, 1001),
    "c2": (4000, 0.5, 1002),
    "c3": (2000, 0.6, 1003),
    "c5": (4000, 0.3, 1005),
    "small": (300, 0.3, 4242),
}
SHIPPED = ("fcc", "bcc", "adversarial")


def golden_path(name):
    return os.path.join(GOLDEN, name)


def unpack_golden(name, dst_dir=None):
    """Decompresses tests/golden/<name>.gz into a temporary file and returns its path."""
    d = dst_dir or tempfile.mkdtemp(prefix="ppgold_")
    out = os.path.join(d, name)
    with gzip.open(golden_path(name + ".gz"), "rb") as f:
        open(out, "wb").write(f.read())
    return out


def parse_probe(name):
    """Reference per-particle results: (N, E_total, overlap_any, E[i], ov[i], nbonds[i], noverlaps[i], bonded lists)."""
    with gzip.open(golden_path("probe_%s.txt.gz" % name), "rt") as f:
        lines = f.read().splitlines()
    N, Etot, anyov = lines[0].split()
    N = int(N)
    E = np.zeros(N)
    ov = np.zeros(N, dtype=np.int32)
    nb = np.zeros(N, dtype=np.int32)
    no = np.zeros(N, dtype=np.int32)
    bonded = []
    for i, line in enumerate(lines[1:]):
        head, tail = line.split(":")
        idx, e, o, b, x = head.split()
        assert int(idx) == i
        E[i], ov[i], nb[i], no[i] = float(e), int(o), int(b), int(x)
        left = tail.split("|")[0].split()
        bonded.append([int(v) for v in left])
    return N, float(Etot), int(anyov), E, ov, nb, no, bonded


def config(name):
    """(r, R, box) of a golden configuration, read exactly as the reference reads it."""
    import patchyparticles_gb300 as pp

    if name in SHIPPED:
        p = unpack_golden(name + ".rrr")
        _, r, R, box = pp.read_rrr(p)
        return r, R, box
    N, rho, seed = GENERATED[name]
    return pp.generate(N, rho, seed, round_like_file=True)


def normalise_nan(text):
    return text.replace("-nan", "nan")
