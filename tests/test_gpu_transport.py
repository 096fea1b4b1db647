"""Tier 2: full transport on the GPU against the CPU oracle.

* FP64 plain form, history by history: with the same per-history Philox
  stream, a GPU history and the oracle history consume identical uniforms, so
  their deposited energies agree to rounding unless a 1-ulp difference of a
  transcendental flips a branch.
* FP32 event form, statistically: the depth dose per bin agrees with the FP64
  oracle within combined 2 sigma (t-corrected for sigmas from 10 batches, so
  95.45 % of the bins above 10 % of Dmax are expected within it; with ~100
  bins the observed share may fall 3 binomial standard deviations below that,
  and no further), mean |diff| beyond statistics <= 1 % there, and every
  history conserves energy.
"""
import importlib
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def batch_sigma(dose, dose2, nb):
    """standard error of the summed dose from nb batch sums"""
    mean = dose / nb
    var = np.maximum(dose2 / nb - mean * mean, 0.0)
    return np.sqrt(var / max(nb - 1, 1)) * nb


@pytest.mark.parametrize("ise,e,geom", [(True, 15.0, 3), (False, 15.0, 3), (True, 6.0, 0), (True, 12.0, 1),
                                        (False, 10.0, 2)])
def test_fp64_histories_match_oracle(tables_c3, oracle_c3, dpm, ise, e, geom):
    n = 400
    he, _ = dpm.simulate_histories(tables_c3, n, e, ise, 1.0, geom, seed=2468)
    _, _, ho, _ = oracle_c3.simulate_slab_philox(n, e, ise, 1.0, geom, seed=2468)
    same = np.isclose(he, ho, rtol=1e-9, atol=1e-12)
    assert same.mean() >= 0.95, same.mean()


def oracle_batches(oracle, nb, per, e, ise, geom, seed0):
    """per-history mean depth dose, its standard error, and the per-batch
    arrays (nb x bins) from nb oracle runs of `per` histories"""
    runs = [oracle.simulate_slab(per, e, ise, 1.0, geom, seed0 + k)[0] for k in range(nb)]
    m = max(len(r) for r in runs)
    a = np.zeros((nb, m))
    for k, r in enumerate(runs):
        a[k, :len(r)] = r / per
    return a.mean(0), a.std(0, ddof=1) / np.sqrt(nb), a


def total_dose_z(g, n_g, batches, per):
    """z-score of the GPU total dose (bins above 10% Dmax) against the oracle's;
    the per-history spread measured on the oracle batches gives both sigmas"""
    o = batches.mean(0)
    m = min(len(g), len(o))
    mask = o[:m] > 0.1 * o.max()
    tot_b = batches[:, :m][:, mask].sum(1)
    sd_hist = tot_b.std(ddof=1) * np.sqrt(per)
    s = np.sqrt(sd_hist ** 2 / n_g + tot_b.var(ddof=1) / len(tot_b))
    return (g[:m][mask].sum() - tot_b.mean()) / s


def compare_depth_dose(g, sg, o, so, batches=10):
    """For the bins above 10% of Dmax: the fraction within the t-corrected
    combined 2 sigma, the lowest fraction that 3 binomial standard deviations
    allow for that many bins, the mean |relative difference| in excess of the
    statistical expectation, and the mean signed relative difference."""
    dc = importlib.import_module("dpm-g4cpp_gb300.dosecheck")
    m = min(len(g), len(o))
    r = dc.compare(g[:m], sg[:m], batches, o[:m], so[:m], batches)
    p, n = r["expected_within_2sigma"], r["voxels"]
    floor = p - 3.0 * math.sqrt(p * (1.0 - p) / n)
    return r["within_2sigma"], floor, r["mean_abs_excess_pct"] / 100.0, r["mean_signed_voxel_pct"] / 100.0


@pytest.mark.parametrize("ise", [True, False])
def test_fp64_depth_dose_statistical(tables_c3, oracle_c3, dpm, ise):
    n = 200000
    ph = dpm.Phantom.slab(tables_c3, 3, 1.0)
    src = dpm.Source(particle=-1 if ise else 0, e0=15.0, e1=15.0)
    res = dpm.run(tables_c3, [dpm.Job(ph, src, n, 11)], precision=dpm.FP64_PLAIN, batches=10)
    d, d2, _ = res.tally(0)
    assert res.stats(0).lost == 0
    per = 10000 if ise else 20000
    o, so, ob = oracle_batches(oracle_c3, 10, per, 15.0, ise, 3, 100)
    frac, floor, excess, bias = compare_depth_dose(d / n, batch_sigma(d, d2, 10) / n, o, so)
    assert frac >= floor, (frac, floor)
    assert excess < 0.01, excess    # mean |diff| beyond statistics: <= 1 %
    z = total_dose_z(d / n, n, ob, per)
    assert abs(z) < 3.5, (z, bias)  # no systematic offset of the integral dose


@pytest.mark.parametrize("ise", [True, False])
def test_fp32_depth_dose_vs_oracle(tables_c3, oracle_c3, dpm, ise):
    n = 1000000
    ph = dpm.Phantom.slab(tables_c3, 3, 1.0)
    src = dpm.Source(particle=-1 if ise else 0, e0=15.0, e1=15.0)
    res = dpm.run(tables_c3, [dpm.Job(ph, src, n, 31)], batches=10)
    d, d2, steps = res.tally(0)
    st = res.stats(0)
    assert st.lost == 0 and st.residual_violations == 0, st
    per = 10000 if ise else 20000
    o, so, ob = oracle_batches(oracle_c3, 10, per, 15.0, ise, 3, 200)
    frac, floor, excess, bias = compare_depth_dose(d / n, batch_sigma(d, d2, 10) / n, o, so)
    assert frac >= floor, (frac, floor)
    assert excess < 0.01, excess    # mean |diff| beyond statistics: <= 1 %
    z = total_dose_z(d / n, n, ob, per)
    assert abs(z) < 3.5, (z, bias)  # no systematic offset of the integral dose


def test_fp32_energy_conservation(tables_wlb, dpm):
    from importlib import import_module
    wl = import_module("dpm-g4cpp_gb300.workloads")
    m = wl.precision_phantom(nx=32, ny=32, nz=64, v=4.0)
    ph = dpm.Phantom.voxels(tables_wlb, m, 4.0)
    res = dpm.run(tables_wlb, [dpm.Job(ph, wl.precision_source(field=60.0), 50000, 7)], batches=5)
    st = res.stats(0)
    assert st.lost == 0
    assert st.residual_violations == 0
    assert st.max_residual < 1e-3 * 20.0
    assert st.histories == 50000
    assert abs(st.edep + st.escaped - st.primary_energy) < 1e-6 * st.primary_energy


@pytest.mark.parametrize("geom,ise,e", [(0, True, 6.0), (1, True, 12.0), (2, False, 10.0), (1, False, 15.0)])
def test_fp32_depth_dose_other_slabs(tables_c3, dpm, geom, ise, e):
    """the other slab presets (homogeneous water; Ti at 10-30 and 20-40 mm):
    the FP32 depth dose agrees with the FP64 form's bin by bin, and the FP32
    form conserves energy. Depth bins share histories, so their differences
    are correlated and the within-2-sigma share of ~20 bins scatters far
    more than a binomial count (0.81-0.96 measured on independent seeds):
    the share must reach 75 %. The dose-weighted signed difference of
    correlated bins has a standard error no larger than the mean relative
    error of a bin: it must stay below 3 of those, and below 0.5 % where
    that is smaller; the excess over noise below 0.5 %"""
    dc = importlib.import_module("dpm-g4cpp_gb300.dosecheck")
    ph = dpm.Phantom.slab(tables_c3, geom, 1.0)
    src = dpm.Source(particle=-1 if ise else 0, e0=e, e1=e)
    est = {}
    for prec, n in ((dpm.FP64_PLAIN, 100000), (dpm.FP32_EVENT, 1000000)):
        r = dpm.run(tables_c3, [dpm.Job(ph, src, n, 40 + geom)], precision=prec, batches=10)
        st = r.stats(0)
        assert st.lost == 0 and st.residual_violations == 0
        assert abs(st.edep + st.escaped - st.primary_energy) <= 1e-6 * st.primary_energy
        d, q, _ = r.tally(0)
        est[prec] = dc.batch_estimate(d, q, 10, n)
    c = dc.compare(est[dpm.FP32_EVENT][0], est[dpm.FP32_EVENT][1], 10,
                   est[dpm.FP64_PLAIN][0], est[dpm.FP64_PLAIN][1], 10)
    assert c["voxels"] >= 10
    assert c["within_2sigma"] >= 0.75, c
    assert abs(c["mean_signed_pct"]) < max(0.5, 3.0 * c["mean_rel_sigma_pct"]), c
    assert c["mean_abs_excess_pct"] < 0.5, c
