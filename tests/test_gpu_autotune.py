"""The autotuner: it keeps a valid schedule, the trajectory stays exact afterwards (tracked energy against
the oracle), and NPT boxes keep a legal cell grid."""
import numpy as np
import pytest

import patchyparticles_gb300 as pp
from oracle import pyoracle as po
from tests.helpers import config

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ens", [pp.NVT, pp.NPT])
def test_autotune_keeps_the_chain_exact(built, ens):
    r, R, box = config("c5")
    prm = pp.default_params(temperature=0.11, ensemble=ens, pressure=0.05)
    e = pp.Engine(prm)
    e.upload(r, R, box)
    t = e.autotune(trial_sweeps=4)
    assert t["resort_every"] in (1, 2, 4, 8, 16) and t["reorder_every"] in (4, 16, 64) and t["cell_scale"] in (1.0, 1.2, 1.5)
    assert t["neighbour_lists"] in (0, 1)
    assert t["n_tried"] == 90 and t["attempts_per_s"] >= t["baseline_attempts_per_s"] > 0
    e.sweeps(20)
    e.sync()
    r2, R2, b2 = e.download()
    s = po.System(po.params(T=0.11), arrays=(r2, R2, b2))
    E, ov = s.init_energy()
    assert not ov and E == e.tracked_energy()
    e.close()


def test_autotune_rejects_bad_arguments(built):
    r, R, box = config("small")
    e = pp.Engine(pp.default_params())
    e.upload(r, R, box)
    with pytest.raises(pp.PPError):
        e.autotune(trial_sweeps=0)
    e.close()
