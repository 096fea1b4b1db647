"""Tier 1: table interpolation and the four samplers on the GPU, fed with the
same inputs and uniforms as the reference (golden vectors from the reference
build). FP64 form: within 4 ulp-scale relative error (the only differences are
CUDA's log/exp against glibc's). FP32 form: relative 2e-4 on smooth maps, with
alias-bin / energy-bin flips counted as a rate."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_RTOL = 4 * 2.0 ** -52 * 8   # a few ulp through log/exp/sqrt chains


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
        big = ref > 1e-15
        rel = np.abs(g[big] - ref[big]) / ref[big]
        assert np.max(rel) < 2e-4, (q, im, np.max(rel))


@pytest.mark.parametrize("s", range(4))
def test_samplers_fp64(golden, tables_c3, dpm, s):
    for im in range(3):
        k = "smp_%d_%d_" % (s, im)
        g = tables_c3.eval_sampler(s, golden[k + "E"], golden[k + "R"], im, dpm.FP64_PLAIN)
        ref = golden[k + "out"]
        np.testing.assert_allclose(g, ref, rtol=FP64_RTOL, atol=1e-15)


@pytest.mark.parametrize("s", range(4))
def test_samplers_fp32(golden, tables_c3, dpm, s):
    for im in range(3):
        k = "smp_%d_%d_" % (s, im)
        g = tables_c3.eval_sampler(s, golden[k + "E"], golden[k + "R"], im, dpm.FP32_EVENT)
        ref = golden[k + "out"]
        rel = np.abs(g - ref) / np.maximum(np.abs(ref), 1e-6)
        # a uniform within FP32 rounding of an alias or energy-bin edge may
        # select the neighbouring bin: allowed at a small rate
        flips = np.mean(rel > 2e-3)
        assert flips < 0.01, (s, im, flips)
        assert np.median(rel) < 1e-5, (s, im, np.median(rel))
