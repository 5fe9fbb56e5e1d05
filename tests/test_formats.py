"""The reference file formats and the seeded generator of the product (include/ppgpu.h, host-only functions)."""
import gzip
import os
import tempfile

import numpy as np
import pytest

from tests import helpers
import patchyparticles_gb300 as pp
from oracle import pyoracle as po


@pytest.mark.parametrize("N,rho,seed", [(300, 0.3, 4242), (1000, 0.1, 1001)])
def test_generator_reproduces_reference_generator(built, N, rho, seed):
    p = helpers.unpack_golden("generator_%d_%s_%d.rrr" % (N, rho, seed))
    _, r, R, box = pp.read_rrr(p)
    g_r, g_R, g_box = pp.generate(N, rho, seed, round_like_file=True)
    assert np.array_equal(r, g_r) and np.array_equal(R, g_R) and np.array_equal(box, g_box)


def test_generator_rejects_dense(built):
    with pytest.raises(pp.PPError):
        pp.generate(100, 0.75, 1)


def test_generated_config_has_no_overlap(built):
    r, R, box = pp.generate(2000, 0.6, 3, round_like_file=False)
    s = po.System(po.params(), arrays=(r, R, box))
    _, ov = s.init_energy()
    assert not ov
    M = R.reshape(-1, 3, 3)
    assert np.allclose(np.linalg.det(M), 1.0, atol=1e-12)


@pytest.mark.parametrize("name", ["fcc", "bcc", "adversarial"])
def test_reader_bit_identical_to_reference_loader(built, name):
    path = helpers.unpack_golden(name + ".rrr")
    _, r, R, box = pp.read_rrr(path)
    s = po.System(po.params(), path=path)
    orr, oR = s.state()
    assert np.array_equal(r, orr) and np.array_equal(R, oR) and np.array_equal(box, s.box())


def test_rrr_write_format_and_roundtrip(built):
    r, R, box = helpers.config("small")
    d = tempfile.mkdtemp()
    p = os.path.join(d, "x.rrr")
    pp.write_rrr(p, 123, r, R, box)
    s = po.System(po.params(), arrays=(r, R, box))
    q = os.path.join(d, "y.rrr")
    s.save(q, 123)
    assert open(p).read() == open(q).read()
    step, N, b = pp.rrr_header(p)
    assert step == 123 and N == len(r)


def test_reader_rejects_short_file(built):
    d = tempfile.mkdtemp()
    p = os.path.join(d, "bad.rrr")
    open(p, "w").write("0 3 10 10 10\n1 0 0\n0 1 0\n1 1 1\n")
    with pytest.raises(pp.PPError):
        pp.read_rrr(p)
    open(p, "w").write("")
    with pytest.raises(pp.PPError):
        pp.rrr_header(p)


def test_reader_messages_are_the_reference_loaders(built):
    """pp_rrr_read reports the reference loader's three failures with its messages (system.c:77-81, 245):
    an unreadable file, a malformed header, and a record count different from the header's, in either
    direction (the reference would write past its particle array for extra records; the reader counts them)."""
    import ctypes
    lib = pp.load_library()
    d = tempfile.mkdtemp()
    rec = "1 0 0\n0 1 0\n{0} {0} {0}\n"

    def read(path, N):
        r = np.zeros((max(N, 1), 3))
        R = np.zeros((max(N, 1), 9))
        b = np.zeros(3)
        err = ctypes.create_string_buffer(512)
        rc = lib.pp_rrr_read(path.encode(), N, pp._dp(r), pp._dp(R), pp._dp(b), err, 512)
        return rc, err.value.decode()

    missing = os.path.join(d, "missing.rrr")
    rc, msg = read(missing, 1)
    assert rc == pp.PP_ERR_IO and msg == f"Initial_conditions_file '{missing}' is not readable"

    empty = os.path.join(d, "empty.rrr")
    open(empty, "w").close()
    rc, msg = read(empty, 1)
    assert rc == pp.PP_ERR_IO and msg == f"The initial configuration file '{empty}' is empty or its headers are malformed"

    short = os.path.join(d, "short.rrr")
    open(short, "w").write("0 3 10 10 10\n" + rec.format(1))
    rc, msg = read(short, 3)
    assert rc == pp.PP_ERR_IO
    assert msg == "Number of particles found in configuration (1) is different from the value found in the header (3)"

    extra = os.path.join(d, "extra.rrr")
    open(extra, "w").write("0 1 10 10 10\n" + "".join(rec.format(k + 1) for k in range(3)))
    rc, msg = read(extra, 1)
    assert rc == pp.PP_ERR_IO
    assert msg == "Number of particles found in configuration (3) is different from the value found in the header (1)"

    good = os.path.join(d, "good.rrr")
    open(good, "w").write("0 2 10 10 10\n" + "".join(rec.format(k + 1) for k in range(2)))
    assert read(good, 2) == (pp.PP_OK, "")

    # the oracle's loader reports the same failures with the same messages
    for path, N in ((missing, 1), (empty, 1), (short, 3), (extra, 1)):
        with pytest.raises(RuntimeError) as ex:
            po.System(po.params(), path=path)
        assert str(ex.value) == read(path, N)[1]


def test_writer_reports_a_failed_write(built):
    """A configuration that could not be written in full is an error, not a saved file (a full disk:
    /dev/full accepts the open and fails the writes)."""
    r = np.zeros((4, 3))
    R = np.tile(np.eye(3).reshape(9), (4, 1))
    box = np.full(3, 10.0)
    if os.path.exists("/dev/full"):
        with pytest.raises(pp.PPError) as ei:
            pp.write_rrr("/dev/full", 0, r, R, box)
        assert ei.value.code == pp.PP_ERR_IO
    with tempfile.TemporaryDirectory() as d:
        with pytest.raises(pp.PPError) as ei:
            pp.write_rrr(os.path.join(d, "missing", "x.rrr"), 0, r, R, box)
        assert ei.value.code == pp.PP_ERR_IO


def test_reader_and_writer_refuse_missing_arrays(built):
    lib = pp.load_library()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "c.rrr").encode()
        assert lib.pp_rrr_write(path, 0, 2, None, None, None) == pp.PP_ERR_ARG
        assert lib.pp_rrr_read(path, 2, None, None, None, None, 0) == pp.PP_ERR_ARG
