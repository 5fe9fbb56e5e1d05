"""Parameter validation of the C-ABI (pp_gpu_create / pp_gpu_create_batch): every invalid key is refused with
PP_ERR_ARG and a message before any CUDA call, so these run on the CPU. Valid parameters only fail later,
at the CUDA stream, where no GPU is present."""
import pytest

import patchyparticles_gb300 as pp


@pytest.mark.parametrize("kw,msg", [
    (dict(ensemble=4), "Ensemble 4 not supported"),
    (dict(ensemble=pp.GC, activity=0.0, n_max=10), "Activity must be > 0"),
    (dict(ensemble=pp.GC, activity=0.1, n_max=0), "GC_N_max >= 1"),
    (dict(ensemble=pp.SUS, activity=0.1, n_min=20, n_max=10), "Umbrella_sampling_min <= Umbrella_sampling_max"),
    (dict(ensemble=pp.GC, activity=0.1, n_max=10, lx_move=1, lx_change_max=0.5, lyz_min=1.0, lyz_max=2.0), "Lx_move is not supported"),
    (dict(temperature=0.0), "Temperature must be > 0"),
    (dict(disp_max=-0.1), "Disp_max and Theta_max must be >= 0"),
    (dict(kf_delta=1.5), "KF_delta must lie in (0, 1)"),
    (dict(kf_cosmax=1.0), "KF_cosmax must lie in (-1, 1)"),
    (dict(precision=7), "unknown precision 7"),
    (dict(guard_eps=0.5), "guard_eps too large"),
    (dict(resort_every=65), "resort_every"),
    (dict(ensemble=pp.NPT, rescale_factor_max=1.0), "rescale_factor_max must lie in (0, 1)"),
    (dict(lx_move=3), "Lx_move must be 0, 1"),
    (dict(lx_move=1, lx_change_max=0.0, lyz_min=1.0, lyz_max=2.0), "Lx_change_max must be > 0"),
    (dict(lx_move=1, lx_change_max=0.5, lyz_min=3.0, lyz_max=2.0), "0 < Lyz_min < Lyz_max"),
])
def test_invalid_parameters_are_refused(built, kw, msg):
    with pytest.raises(pp.PPError) as ex:
        pp.Engine(pp.default_params(**kw))
    assert ex.value.code == pp.PP_ERR_ARG and msg in ex.value.message


def test_a_batch_reports_its_invalid_replica(built):
    with pytest.raises(pp.PPError) as ex:
        pp.Engine([pp.default_params(), pp.default_params(temperature=-1.0)])
    assert ex.value.code == pp.PP_ERR_ARG and "Temperature" in ex.value.message


def test_lx_move_is_ignored_for_npt(built):
    """The reference sets Lx_move = 0 for NPT (system.c:165-169): its Lx keys are not validated there."""
    try:
        pp.Engine(pp.default_params(ensemble=pp.NPT, lx_move=1, lx_change_max=0.0)).close()
    except pp.PPError as ex:  # without a GPU the engine stops at the CUDA stream, not at the parameters
        assert ex.code == pp.PP_ERR_CUDA


def test_a_nan_guard_band_is_refused(built):
    with pytest.raises(pp.PPError) as ex:
        pp.Engine(pp.default_params(guard_eps=float("nan")))
    assert ex.value.code == pp.PP_ERR_ARG and "guard_eps" in ex.value.message
