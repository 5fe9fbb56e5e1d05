"""GPU energy / bond / overlap parity with the reference's own routines (bit-exact, integer results)."""
import numpy as np
import pytest

from tests import helpers
import patchyparticles_gb300 as pp
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

PROBES = ["fcc", "bcc", "adversarial", "c1", "c2", "c3", "c5", "small"]


def _engine(r, R, box, **kw):
    e = pp.Engine(pp.default_params(**kw))
    return e


@pytest.mark.parametrize("precision", [pp.PREC_FP32_GUARD, pp.PREC_FP64])
@pytest.mark.parametrize("name", PROBES)
def test_bonds_and_overlaps_match_reference_probe(built, name, precision):
    """Per-particle bond and overlap counts equal the reference's MC_interact walk (golden probe)."""
    N, Etot, anyov, E, ov, nb, no, bonded = helpers.parse_probe(name)
    r, R, box = helpers.config(name)
    e = pp.Engine(pp.default_params(precision=precision, audit=1))
    if anyov:
        with pytest.raises(pp.PPError) as ei:
            e.upload(r, R, box)
        assert ei.value.code == pp.PP_ERR_OVERLAP
        # the upload still left the state on the device: per-particle results are available
    else:
        e.upload(r, R, box)
    gb, go = e.bonds()
    assert np.array_equal(gb, nb)
    assert np.array_equal(go, no)
    Eg, ovg = e.energy()
    assert ovg == bool(anyov)
    if not anyov:
        assert Eg == Etot
        assert e.tracked_energy() == Etot
    g = e.guard_stats()
    assert g["mismatches"] == 0
    assert g["max_err_r2"] < 1e-5 / 4 and g["max_err_cos"] < 1e-5 / 4
    if precision == pp.PREC_FP32_GUARD and name == "adversarial":
        assert g["fallbacks"] > 0  # the near-threshold pairs did go through FP64
    e.close()


@pytest.mark.parametrize("N,rho,seed", [(32768, 0.5, 2002), (32768, 0.1, 2004), (1048576, 0.3, 2005)])
def test_full_size_energy_matches_oracle(built, N, rho, seed):
    """Bench-size configurations: total energy and every particle's bond count against the oracle."""
    r, R, box = pp.generate(N, rho, seed, round_like_file=False)
    s = po.System(po.params(), arrays=(r, R, box))
    tot, E, ov, nb, no = s.energies()
    e = pp.Engine(pp.default_params())
    e.upload(r, R, box)
    gb, go = e.bonds()
    assert np.array_equal(gb, nb) and not go.any() and not ov.any()
    assert e.energy() == (tot, False)
    e.close()


def test_audit_zero_mismatches_all_pairs(built):
    """FP32 decisions outside the guard band never contradict FP64 over all candidate pairs."""
    for (N, rho, seed) in [(32768, 0.5, 3002), (65536, 0.3, 3005), (8000, 0.6, 3003)]:
        r, R, box = pp.generate(N, rho, seed, round_like_file=False)
        e = pp.Engine(pp.default_params(audit=1))
        e.upload(r, R, box)
        e.bonds()
        e.sweeps(5)
        e.sync()
        g = e.guard_stats()
        assert g["pairs"] > 10 * N
        assert g["mismatches"] == 0, g
        assert g["max_err_r2"] < 2.5e-6 and g["max_err_cos"] < 2.5e-6, g
        e.close()


def test_orthonormalise_bit_identical_to_reference_gram_schmidt(built):
    r, R, box = helpers.config("c2")
    # perturb orientations so that gram_schmidt has work to do
    rng = np.random.default_rng(5)
    R = R + rng.normal(scale=1e-6, size=R.shape)
    e = pp.Engine(pp.default_params())
    e.upload(r, R, box)
    e.orthonormalise()
    _, R_gpu, _ = e.download()
    s = po.System(po.params(), arrays=(r, R, box))
    s.init_energy()
    assert s.check_energy() == 0  # MC_check_energy runs gram_schmidt on every orientation (MC.c:774)
    _, R_orc = s.state()
    assert np.array_equal(R_gpu, R_orc)
    e.close()


def test_upload_download_roundtrip(built):
    r, R, box = helpers.config("c3")
    e = pp.Engine(pp.default_params())
    e.upload(r, R, box)
    r2, R2, b2 = e.download()
    assert np.array_equal(r, r2) and np.array_equal(R, R2) and np.array_equal(box, b2)
    e.close()


def test_too_small_box_is_rejected(built):
    r, R, box = pp.generate(20, 0.5, 1)
    e = pp.Engine(pp.default_params())
    with pytest.raises(pp.PPError) as ei:
        e.upload(r, R, box)
    assert ei.value.code == pp.PP_ERR_CAPACITY


@pytest.mark.parametrize("name", ["fcc", "c2", "c3"])
def test_bond_lists_match_reference_probe(built, name):
    """Bonded partner lists (output_print_bonds, output.c:213-268) against the reference's, particle by particle."""
    N, Etot, anyov, E, ov, nb, no, bonded = helpers.parse_probe(name)
    r, R, box = helpers.config(name)
    e = pp.Engine(pp.default_params())
    e.upload(r, R, box)
    off, part = e.bond_lists()
    assert off[-1] == nb.sum()
    for i in range(N):
        assert list(part[off[i]:off[i + 1]]) == bonded[i]
    e.close()
