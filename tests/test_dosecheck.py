"""The dose-comparison statistics every parity test and the benchmark use
(dpm-g4cpp_gb300/dosecheck.py), on synthetic batch tallies whose truth is
known: the batch estimate, the t-corrected 2-sigma coverage, the signed and
absolute differences, and the absence of a selection bias."""
import importlib

import numpy as np
import pytest

dc = importlib.import_module("dpm-g4cpp_gb300.dosecheck")


def tallies(mu, rel_sd, B, H, rng, bias=1.0):
    """dose, dose2 of B batches of H / B histories: batch sums normal around
    mu * H / B with relative sd rel_sd * sqrt(B) (so the mean's relative
    standard error is rel_sd)"""
    t = rng.normal(1.0, rel_sd * np.sqrt(B), (B,) + mu.shape) * (bias * mu * H / B)
    return t.sum(0), (t * t).sum(0), t / (H / B)


def test_batch_estimate_is_the_batch_mean_and_its_standard_error():
    rng = np.random.default_rng(1)
    mu = rng.uniform(1.0, 5.0, 1000)
    d, q, per = tallies(mu, 0.05, 10, 10000, rng)
    m, s = dc.batch_estimate(d, q, 10, 10000)
    mb, sb = dc.batches_estimate(per)
    np.testing.assert_allclose(m, mb, rtol=1e-12)
    np.testing.assert_allclose(s, sb, rtol=1e-9)


@pytest.mark.parametrize("B", [10, 40])
def test_coverage_of_equal_distributions(B):
    """two independent estimates of the same dose: about 95.45 % of the voxels
    within the t-corrected combined 2 sigma, no signed difference, no excess
    of the absolute difference over the noise, the totals within their
    errors"""
    rng = np.random.default_rng(2 + B)
    mu = np.exp(-np.linspace(0.0, 3.0, 60000))
    da, qa, _ = tallies(mu, 0.03, B, 100000, rng)
    db, qb, _ = tallies(mu, 0.05, B, 40000, rng)
    ma, sa = dc.batch_estimate(da, qa, B, 100000)
    mb, sb = dc.batch_estimate(db, qb, B, 40000)
    c = dc.compare(ma, sa, B, mb, sb, B)
    assert abs(c["within_2sigma"] - c["expected_within_2sigma"]) < 0.006, c
    assert abs(c["mean_signed_pct"]) < 0.1, c
    assert c["mean_abs_excess_pct"] < 0.1, c
    assert abs(c["total_z"]) < 4.0, c


def test_a_planted_bias_is_measured():
    """one estimate 1 % high everywhere, 0.5 % standard error each: the signed
    difference reads +1 % and the coverage falls to P(|N(1.41, 1)| < t) ~ 0.75"""
    rng = np.random.default_rng(7)
    mu = np.exp(-np.linspace(0.0, 3.0, 60000))
    da, qa, _ = tallies(mu, 0.005, 10, 100000, rng, bias=1.01)
    db, qb, _ = tallies(mu, 0.005, 10, 100000, rng)
    c = dc.compare(*dc.batch_estimate(da, qa, 10, 100000), 10, *dc.batch_estimate(db, qb, 10, 100000), 10)
    assert abs(c["mean_signed_pct"] - 1.0) < 0.05, c
    assert abs(c["total_ratio"] - 1.01) < 5e-4, c
    assert 0.70 < c["within_2sigma"] < 0.80, c


def test_no_selection_bias_at_low_signal():
    """voxels chosen on the inverse-variance-weighted mean of the two
    estimates: at 30 % relative noise near the 10 % threshold the signed
    difference stays near zero, where choosing on one estimate's own value
    would bias it"""
    rng = np.random.default_rng(11)
    mu = np.concatenate([np.full(1000, 1.0), np.full(200000, 0.1)])
    da, qa, _ = tallies(mu, 0.3, 10, 10000, rng)
    db, qb, _ = tallies(mu, 0.3, 10, 10000, rng)
    c = dc.compare(*dc.batch_estimate(da, qa, 10, 10000), 10, *dc.batch_estimate(db, qb, 10, 10000), 10)
    assert abs(c["mean_signed_voxel_pct"]) < 1.0, c
