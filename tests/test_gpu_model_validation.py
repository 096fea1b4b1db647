"""GPU model-validation histograms (the reference's modelValidationTests,
testAPI.cc:92-198) against the same histograms made from the CPU oracle's
samplers, and FP32 against FP64: same shapes within statistics (chi^2)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

E0 = 15.0
EMC2 = 0.510991


def chi2_per_dof(a, b):
    """two-sample chi^2 of count histograms a, b (different totals) per degree of freedom"""
    na, nb = a.sum(), b.sum()
    m = (a + b) > 0
    num = (a[m] / na - b[m] / nb) ** 2
    den = a[m] / na ** 2 + b[m] / nb ** 2
    return float((num / den).sum() / max(1, m.sum() - 1))


def oracle_hist(oracle, model, imat, n, gcut, hbins=101, seed=5):
    """testAPI's two histograms from the oracle's samplers fed with numpy uniforms"""
    rng = np.random.default_rng(seed)
    E = np.full(n, E0)
    R = rng.random((n, 3))
    if model == 0:
        k = oracle.sampler(2, E, R, imat)
        dum0 = EMC2 * 0.7071067812 / (E0 + EMC2)
        cost = np.full(n, max(-1.0, min(1.0, 1.0 - dum0 * dum0)))
    elif model == 1:
        k = oracle.sampler(1, E, R, imat)
        cost = np.minimum(1.0, np.sqrt(k * (E0 + 2 * EMC2) / (E0 * (k + 2 * EMC2))))
    else:
        k = E.copy()
        cost = np.clip(oracle.sampler(3, E, R, imat), -1.0, 1.0)
    xmin = math.log10(gcut / E0)
    ihdel = 1.0 / ((0.1 - xmin) / (hbins - 1))
    hx = np.zeros(hbins)
    hc = np.zeros(hbins)
    red = k / E0
    ix = ((np.log10(red[red > 0]) - xmin) * ihdel).astype(int)
    np.add.at(hx, ix[(ix >= 0) & (ix < hbins)], 1)
    ic = (cost * (hbins // 2) + hbins // 2).astype(int)
    np.add.at(hc, ic[(ic >= 0) & (ic < hbins)], 1)
    return hx, hc


@pytest.mark.parametrize("model,imat", [(0, 0), (0, 1), (0, 2), (1, 0), (2, 0)])
def test_gpu_histograms_match_oracle(tables_c3, oracle_c3, dpm, model, imat):
    _, gx, _, gc = tables_c3.model_histogram(model, E0, 2_000_000, imat=imat, seed=11)
    ox, oc = oracle_hist(oracle_c3, model, imat, 200_000, tables_c3.gamma_cut)
    assert gx.sum() > 0 and gc.sum() == 2_000_000
    assert chi2_per_dof(gx, ox) < 2.0
    assert chi2_per_dof(gc, oc) < 2.0


@pytest.mark.parametrize("model", [0, 1, 2])
def test_fp32_histograms_match_fp64(tables_c3, dpm, model):
    _, ax, _, ac = tables_c3.model_histogram(model, E0, 2_000_000, seed=3, precision=dpm.FP64_PLAIN)
    _, bx, _, bc = tables_c3.model_histogram(model, E0, 2_000_000, seed=4, precision=dpm.FP32_EVENT)
    assert chi2_per_dof(ax, bx) < 2.0
    assert chi2_per_dof(ac, bc) < 2.0
