"""The oracle restatement (oracle/pp_oracle.c) against the reference's own outputs (tests/golden/)."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from tests import helpers
from oracle import pyoracle as po


def test_drand48_recurrence_matches_libc(built):
    import ctypes

    libc = ctypes.CDLL("libc.so.6")
    libc.drand48.restype = ctypes.c_double
    libc.srand48.argtypes = [ctypes.c_long]
    for seed in (0, 1, 12345, -7, 2**31 - 1):
        libc.srand48(seed)
        want = [libc.drand48() for _ in range(50)]
        got = po.drand48_sequence(seed, 50)
        assert np.array_equal(np.array(want), got)


@pytest.mark.parametrize("name", ["fcc", "bcc", "adversarial", "c1", "c2", "c3", "c5", "small"])
def test_oracle_energies_match_reference_probe(built, name):
    N, Etot, anyov, E, ov, nb, no, bonded = helpers.parse_probe(name)
    r, R, box = helpers.config(name)
    s = po.System(po.params(), arrays=(r, R, box))
    tot, e, o, b, x = s.energies()
    assert s.N == N
    assert np.array_equal(e, E)
    assert np.array_equal(o, ov)
    assert np.array_equal(b, nb)
    assert np.array_equal(x, no)
    assert tot == Etot
    off, part = s.bond_lists()
    for i in range(0, N, max(1, N // 200)):
        assert list(part[off[i]:off[i + 1]]) == bonded[i]


def test_known_answers(built):
    # fcc.rrr: E/N = -1.828 (914 bonds); bcc.rrr: E = 0 without overlaps (delta = 0.12, cosmax = 0.92)
    for name, want in (("fcc", -914.0), ("bcc", 0.0)):
        r, R, box = helpers.config(name)
        s = po.System(po.params(), arrays=(r, R, box))
        E, ov = s.init_energy()
        assert E == want and not ov


@pytest.mark.parametrize("name", ["fcc_nvt", "bcc_npt", "small_nvt", "small_npt", "small_lx", "small_gc", "small_sus", "small_avb", "small_avb_npt", "small_vmmc", "small_vmmc_npt"])
def test_oracle_trajectory_matches_reference(built, name):
    """The restated main loop reproduces the reference's output files line for line (NVT, NPT, the Lx
    move, grand canonical insertions and removals, successive umbrella sampling with its histograms, the
    aggregation-volume-bias dynamics and the virtual-move cluster dynamics in NVT and NPT)."""
    src = helpers.golden_path("traj_" + name)
    work = tempfile.mkdtemp(prefix="pptraj_")
    os.makedirs(os.path.join(work, "confs"))
    if os.path.isdir(os.path.join(src, "sus")):
        os.makedirs(os.path.join(work, "sus"))
    shutil.copy(os.path.join(src, "input"), work)
    conf = [l.split("=")[1].strip() for l in open(os.path.join(src, "input")) if l.startswith("Initial_conditions_file")][0]
    helpers.unpack_golden(conf, work)
    out = subprocess.check_output([po.CLI, "input"], cwd=work, stderr=subprocess.DEVNULL).decode()
    assert out == open(os.path.join(src, "stdout.txt")).read()
    for fn in ("energy.dat", "acceptance.dat", "density.dat", "boxshape.dat"):
        p = os.path.join(src, fn)
        if os.path.exists(p):
            assert helpers.normalise_nan(open(os.path.join(work, fn)).read()) == helpers.normalise_nan(open(p).read()), fn
    import gzip

    assert open(os.path.join(work, "last.rrr"), "rb").read() == gzip.open(os.path.join(src, "last.rrr.gz")).read()
    if os.path.isdir(os.path.join(src, "sus")):
        want = sorted(os.listdir(os.path.join(src, "sus")))
        assert want and sorted(os.listdir(os.path.join(work, "sus"))) == want
        for fn in want:
            assert open(os.path.join(work, "sus", fn)).read() == open(os.path.join(src, "sus", fn)).read(), fn
    shutil.rmtree(work)


def test_check_energy_orthonormalises(built):
    r, R, box = helpers.config("fcc")
    s = po.System(po.params(), arrays=(r, R, box))
    s.init_energy()
    assert s.check_energy() == 0
    _, R2 = s.state()
    M = R2.reshape(-1, 3, 3)
    assert np.allclose(np.einsum("nij,nkj->nik", M, M), np.eye(3), atol=1e-14)


@pytest.mark.parametrize("N,rho,seed", [(300, 0.3, 4242), (1000, 0.1, 1001)])
def test_oracle_generator_prints_the_reference_generators_file(built, N, rho, seed):
    """orc_generate (generator.c:43-68 restated) against the seeded reference generator's own output."""
    import gzip

    want = gzip.open(helpers.golden_path("generator_%d_%s_%d.rrr.gz" % (N, rho, seed)), "rt").read()
    r, R, box = po.generate(N, rho, seed)
    assert po.generated_text(r, R, box) == want


def test_oracle_generator_equals_the_products(built):
    """The reference arm of bench.py builds its inputs with the oracle's generator, the GPU arm with the
    product's: both must give the same configuration bit for bit."""
    import patchyparticles_gb300 as pp

    for N, rho, seed in ((2000, 0.3, 1005), (500, 0.6, 7)):
        a = po.generate(N, rho, seed)
        b = pp.generate(N, rho, seed, round_like_file=False)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    with pytest.raises(ValueError):
        po.generate(10, 0.75, 1)
