"""Tier 1: table interpolation and the four samplers on the GPU, fed with the
same inputs and uniforms as the reference.

FP64 form: the golden vectors of the reference build, within a few ulp (the
only differences are CUDA's log/exp against glibc's).

FP32 form, against the tolerances the target states for it:
* tables: relative error <= 1e-5 of max(|value|, 1 % of the curve's maximum)
  and <= 1e-6 relative wherever the value exceeds 5 % of the maximum. The two
  curves that vanish at a threshold (Moller IMFP just above 2 Ecut, pair IMFP
  just above 2 mc^2) lose digits to cancellation in FP32 there (up to 2e-5
  relative at 1e-4 of the curve's maximum, an absolute error near 1e-9 of it);
  everywhere else the measured error is below 3e-7;
* samplers, on 10^6 fresh draws per sampler and material against the oracle
  (the reference's FP64 samplers, pinned bit for bit to the reference build):
  both sides get the same inputs, the float values (energies and uniforms)
  the FP32 form works on. A draw whose uniform falls within FP32 rounding of
  an alias-bin or energy-bin edge takes the neighbouring bin (a "flip"). KN,
  Moller, SB: a relative difference above 1e-4 is a flip; flips are counted
  as a rate (a few per 10^6 draws) and every other draw agrees to 1e-5
  relative. GS (the MSC cosine crosses 0, and an energy-bin flip near mu = 1
  moves mu very little): draws within 1e-4 of an energy-bin or ratin-bin edge
  are the ones that may flip, and every other draw agrees to 1e-6 in mu.
  On the reference build's own golden vectors (double uniforms, rounded to
  float on the GPU) the same bounds hold, except that GS may move by up to
  2e-5 where rounding a uniform near a bin's upper edge moves the draw.
"""
import os

import numpy as np
import pytest

from conftest import DATA_C3

pytestmark = pytest.mark.gpu

FP64_RTOL = 4 * 2.0 ** -52 * 8   # a few ulp through log/exp/sqrt chains
# energy ranges where the reference samplers are defined (KN, Moller, SB, GS)
RANGES = {0: (0.0501, 20.99), 1: (0.4001, 20.99), 2: (0.0501, 20.99), 3: (0.2001, 20.99)}
N_DRAWS = 1_000_000
FLIP_REL = 1e-4              # KN, Moller, SB: a larger relative difference is a flip
NONFLIP_REL = 1e-5
FLIP_RATE_MAX = 2e-5         # flips per draw
GS_EDGE = 1e-4               # GS: distance to a bin edge within which a draw may flip
GS_ABS = 1e-6                # GS: every other draw, |d mu|
GS_ABS_GOLDEN = 2e-5         # GS on double uniforms rounded to float by the GPU


def gs_grid():
    """(log of the lowest energy, 1 / log spacing, cumulative points) of the
    GS tables (el_GSDtrData.dat header: #E, Emin, Emax, #cumulative)"""
    with open(os.path.join(DATA_C3, "el_GSDtrData.dat")) as f:
        for _ in range(4):
            f.readline()
        ne, emin, emax, nc = f.readline().split()
    ne, emin, emax, nc = int(ne), float(emin), float(emax), int(nc)
    return np.log(emin), (ne - 1) / np.log(emax / emin), nc


def gs_near_edge(E, R):
    """draws whose energy-bin uniform (r1) or ratin-bin uniform (r2) lies
    within GS_EDGE of a decision edge"""
    lmin, ild, nc = gs_grid()
    ph = (np.log(E) - lmin) * ild
    frac = ph - np.floor(ph)
    x = R[:, 1] * (nc - 1)
    return (np.abs(R[:, 0] - frac) < GS_EDGE) | (np.abs(x - np.round(x)) < GS_EDGE * (nc - 1))


@pytest.mark.parametrize("q", range(9))
def test_tables_fp64(golden, tables_c3, dpm, q):
    E = golden["tab_E"]
    for im in range(3):
        g = tables_c3.eval_table(q, E, im, dpm.FP64_PLAIN)
        ref = golden["tab_%d_%d" % (q, im)]
        np.testing.assert_allclose(g, ref, rtol=1e-13, atol=0)


@pytest.mark.parametrize("q", range(9))
def test_tables_fp32(golden, tables_c3, dpm, q):
    E = golden["tab_E"]
    for im in range(3):
        g = tables_c3.eval_table(q, E, im, dpm.FP32_EVENT)
        ref = golden["tab_%d_%d" % (q, im)]
        scale = np.maximum(np.abs(ref), 0.01 * np.abs(ref).max())
        rel = np.abs(g - ref) / scale
        assert rel.max() <= 1e-5, (q, im, rel.max(), E[np.argmax(rel)])
        away = np.abs(ref) > 0.05 * np.abs(ref).max()
        assert (np.abs(g - ref)[away] / np.abs(ref)[away]).max() <= 1e-6, (q, im)


@pytest.mark.parametrize("s", range(4))
def test_samplers_fp64(golden, tables_c3, dpm, s):
    for im in range(3):
        k = "smp_%d_%d_" % (s, im)
        g = tables_c3.eval_sampler(s, golden[k + "E"], golden[k + "R"], im, dpm.FP64_PLAIN)
        ref = golden[k + "out"]
        np.testing.assert_allclose(g, ref, rtol=FP64_RTOL, atol=1e-15)


def _check_fp32(s, E, R, g, ref, max_flips, gs_abs=GS_ABS):
    """returns (flip rate, worst error of the other draws)"""
    if s == 3:
        err = np.abs(g - ref)
        edge = gs_near_edge(E, R)
        flips = edge & (err > gs_abs)
        worst = err[~edge].max()
        assert worst <= gs_abs, (s, worst)
    else:
        err = np.abs(g - ref) / np.abs(ref)
        flips = err > FLIP_REL
        worst = err[~flips].max()
        assert worst <= NONFLIP_REL, (s, worst)
    assert flips.sum() <= max_flips, (s, int(flips.sum()))
    return flips.mean(), worst


@pytest.mark.parametrize("s", range(4))
def test_samplers_fp32_golden(golden, tables_c3, dpm, s):
    """the reference build's own vectors (1500 draws each): at most one flip"""
    for im in range(3):
        k = "smp_%d_%d_" % (s, im)
        E, R = golden[k + "E"], golden[k + "R"]
        g = tables_c3.eval_sampler(s, E, R, im, dpm.FP32_EVENT)
        _check_fp32(s, E, R, g, golden[k + "out"], 1, GS_ABS_GOLDEN)


@pytest.mark.parametrize("s", range(4))
def test_samplers_fp32_flip_rate(tables_c3, oracle_c3, dpm, s):
    lo, hi = RANGES[s]
    for im in range(3):
        rng = np.random.default_rng(1000 * s + im)
        # float-representable inputs, uniforms below 1 as the FP32 form draws them
        E = np.exp(rng.uniform(np.log(lo), np.log(hi), N_DRAWS)).astype(np.float32).astype(np.float64)
        R = np.minimum(rng.random((N_DRAWS, 3)).astype(np.float32), np.float32(1 - 2.0 ** -24)).astype(np.float64)
        g = tables_c3.eval_sampler(s, E, R, im, dpm.FP32_EVENT)
        ref = oracle_c3.sampler(s, E, R, im)
        rate, worst = _check_fp32(s, E, R, g, ref, int(FLIP_RATE_MAX * N_DRAWS))
        print("sampler %d material %d: flip rate %.2e, max error of the other draws %.2e" % (s, im, rate, worst))
