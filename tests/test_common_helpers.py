"""The remaining rustalgos helpers against the reference's own checks (tests/rustalgos/test_common.py):
check_numerical_data, distances_from_seconds round trips and ordering errors,
avg_distances_for_betas and clip_wts_curve golden values, clipped_beta_wt."""
import numpy as np
import pytest

from cityseer_gb300 import rustalgos

ATOL, RTOL = 0.01, 1e-4  # the reference tests' tolerances (config.ATOL / config.RTOL)
SPEED = 1.33333


def test_check_numerical_data():
    with pytest.raises(TypeError):
        rustalgos.check_numerical_data(np.ones(5, np.float32))
    ok = np.random.default_rng(0).random((10, 2)).astype(np.float32)
    rustalgos.check_numerical_data(ok)
    ok[0, 0] = np.inf
    with pytest.raises(ValueError, match="must be finite"):
        rustalgos.check_numerical_data(ok)


def test_distances_from_seconds_round_trip():
    distances = [400, 600, 800, 1600, 2000, 2400]
    seconds = [round(t * 60) for t in (5, 7.5, 10, 20, 25, 30)]
    for d, t in zip(distances, seconds):
        assert rustalgos.distances_from_seconds([t], SPEED) == [d]
    ds = rustalgos.distances_from_seconds(seconds, SPEED)
    assert ds == distances and rustalgos.seconds_from_distances(ds, SPEED) == seconds
    for bad in ([10, 10], [10, 5]):
        with pytest.raises(ValueError, match="strictly increasing"):
            rustalgos.distances_from_seconds(bad, SPEED)
    with pytest.raises(ValueError, match="positive integers"):
        rustalgos.distances_from_seconds([0, 5], SPEED)


def test_avg_distances_and_clipped_curves():
    betas = rustalgos.betas_from_distances([100, 200, 400, 800, 1600])
    np.testing.assert_allclose(rustalgos.avg_distances_for_betas(betas),
                               [35.11949, 70.23898, 140.47797, 280.95593, 561.91187], atol=ATOL, rtol=RTOL)
    distances = [400, 800, 1600]
    betas = rustalgos.betas_from_distances(distances)
    np.testing.assert_allclose(rustalgos.clip_wts_curve(distances, betas, 0), [1, 1, 1], atol=ATOL, rtol=RTOL)
    np.testing.assert_allclose(rustalgos.clip_wts_curve(distances, betas, 50), [0.60653067, 0.7788008, 0.8824969],
                               atol=ATOL, rtol=RTOL)
    with pytest.raises(ValueError, match="cannot be greater"):
        rustalgos.clip_wts_curve(distances, betas, 401)
    for tol in (0, 50, 400):
        for d, b, mw in zip(distances, betas, rustalgos.clip_wts_curve(distances, betas, tol)):
            for dd in (0, 25, 50, 100, 400, 800, 1600):
                if dd > d:
                    continue
                got = rustalgos.clipped_beta_wt(b, mw, dd)
                assert np.isclose(got, min(np.exp(-b * dd), mw) / mw, atol=ATOL, rtol=RTOL)
                if tol == 0 or dd == 0 or dd <= tol:
                    assert np.isclose(got, 1.0 if dd <= tol else np.exp(-b * dd), atol=ATOL, rtol=RTOL)
    with pytest.raises(ValueError, match=r"\[0, 1\]"):
        rustalgos.clipped_beta_wt(0.01, 1.5, 10.0)


def test_config_helpers():
    """pysrc/cityseer/config.py:21-83: column keys, debug flag, threshold logging."""
    from cityseer_gb300 import config

    assert config.prep_gdf_key("density", 400) == "cc_density_400"
    assert config.prep_gdf_key("harmonic", 800, angular=True) == "cc_harmonic_800_ang"
    assert config.prep_gdf_key("beta", 200, weighted=False) == "cc_beta_200_nw"
    assert config.log_thresholds(betas=[0.01, 0.005]) == [400, 800]
    assert isinstance(config.DEBUG_MODE, bool)
