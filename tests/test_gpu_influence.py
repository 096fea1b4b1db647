"""Differentiation form: a beamlet-tagged run builds the CSR influence matrix
A (voxels x beamlets); D = A w is an autograd function whose hand-written
backward is A^T g. Checked against the untagged dose, against products with the
same A on the CPU (scipy), and against central finite differences."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(tables_wlb, dpm):
    wl = importlib.import_module("dpm-g4cpp_gb300.workloads")
    m, src, target = wl.differentiation_setup(n=32, v=4.0)
    src.nbx = src.nby = 4
    src.fx = src.fy = 10.0
    ph = dpm.Phantom.voxels(tables_wlb, m, 4.0)
    res = dpm.run(tables_wlb, [dpm.Job(ph, src, 64000, 3)], batches=4, tag_beamlets=True)
    A = res.influence(0)
    return dict(res=res, A=A, ph=ph, target=target)


def test_columns_sum_to_dose(setup):
    A = setup["A"].to_scipy()
    dose = setup["res"].tally(0)[0].reshape(-1)
    np.testing.assert_allclose(np.asarray(A.sum(axis=1)).ravel(), dose, rtol=2e-6, atol=1e-6 * dose.max())
    assert A.shape == (dose.size, 16)
    assert setup["A"].nnz > 0


def test_tagged_dose_equals_untagged(setup, tables_wlb, dpm):
    """the tagged run (kernels of the tagged tally form) and the same job
    untagged (the plain form) give the same dose up to the order of FP64
    additions: the beamlet tally does not touch the transport"""
    res = setup["res"]
    job = res._jobs[0]
    plain = dpm.run(tables_wlb, [job], batches=4)
    (dt, qt, _), (dp, qp, _) = res.tally(0), plain.tally(0)
    np.testing.assert_allclose(dt, dp, rtol=1e-10, atol=1e-12 * dp.max())
    np.testing.assert_allclose(qt, qp, rtol=1e-10, atol=1e-12 * qp.max())


def test_products_match_cpu(setup):
    import torch
    A = setup["A"]
    S = A.to_scipy().astype(np.float64)
    rng = np.random.default_rng(0)
    w = rng.random(A.cols)
    g = rng.random(A.rows)
    y = A.matvec(torch.tensor(w, device="cuda")).cpu().numpy()
    x = A.rmatvec(torch.tensor(g, device="cuda")).cpu().numpy()
    np.testing.assert_allclose(y, S @ w, rtol=1e-12, atol=1e-12 * np.abs(S @ w).max())
    np.testing.assert_allclose(x, S.T @ g, rtol=1e-10)


def test_backward_matches_finite_differences(setup):
    import torch
    inf = importlib.import_module("dpm-g4cpp_gb300.influence")
    A = setup["A"]
    T = torch.tensor(setup["target"].reshape(-1) * 1e-9, device="cuda", dtype=torch.float64)
    D0 = A.matvec(torch.ones(A.cols, device="cuda", dtype=torch.float64))
    T = T * (D0.max() / max(T.max(), 1e-30))      # target on the dose scale

    def loss(w):
        return 0.5 * ((inf.dose(A, w) - T) ** 2).sum()

    w = torch.rand(A.cols, device="cuda", dtype=torch.float64, requires_grad=True)
    L = loss(w)
    L.backward()
    grad = w.grad.detach().cpu().numpy()
    eps = 1e-3
    fd = np.zeros(A.cols)
    with torch.no_grad():
        for i in range(A.cols):
            e = torch.zeros_like(w)
            e[i] = eps
            fd[i] = (loss(w + e).item() - loss(w - e).item()) / (2 * eps)
    np.testing.assert_allclose(grad, fd, rtol=1e-5, atol=1e-8 * np.abs(fd).max())


def test_influence_matrix_vs_cpu_built(tables_wlb, dpm, orc):
    """A built on the CPU by the oracle (the reference's FP64 transport with
    each history's deposits tallied under its beamlet) against A built on the
    GPU (FP32 transport, FP64 accumulation, FP32 CSR values), both as dose per
    history from independent random streams: column by column, voxel by voxel
    within the t-corrected combined 2 sigma in each column's voxels above 10 %
    of its maximum, and the products A^T g for a target-shaped g within 4
    combined standard deviations per beamlet and 1 % on average."""
    from conftest import DATA_WLB
    wl = importlib.import_module("dpm-g4cpp_gb300.workloads")
    dc = importlib.import_module("dpm-g4cpp_gb300.dosecheck")
    m, src, target = wl.differentiation_setup(n=32, v=4.0)
    src.nbx = src.nby = 4
    src.fx = src.fy = 10.0
    nb = 16
    s = dict(particle=src.particle, spectrum=src.spectrum, e0=src.e0, e1=src.e1, shape=src.shape, cx=src.cx,
             cy=src.cy, fx=src.fx, fy=src.fy, nbx=src.nbx, nby=src.nby)
    KO, PER_O = 32, 200_000
    o, so, _, ob = orc.voxel_batches(DATA_WLB, m, 4.0, s, PER_O, KO, 1007, tagged=True, keep=True)
    o, so, ob = o.reshape(nb, -1), so.reshape(nb, -1), ob.reshape(KO, nb, -1)
    ph = dpm.Phantom.voxels(tables_wlb, m, 4.0)
    KG, PER_G = 16, 400_000
    gb = []
    for k in range(KG):
        res = dpm.run(tables_wlb, [dpm.Job(ph, src, PER_G, 3, first_history=k * PER_G)], batches=1,
                      tag_beamlets=True)
        A = res.influence(0).to_scipy().toarray().astype(np.float64)      # [voxels, beamlets]
        gb.append(A.T / PER_G)
        res.close()
    gb = np.stack(gb)                                                      # [KG, beamlets, voxels]
    g, sg = gb.mean(0), gb.std(0, ddof=1) / np.sqrt(KG)
    within, voxels = 0.0, 0
    for b in range(nb):
        r = dc.compare(g[b], sg[b], KG, o[b], so[b], KO)
        within += r["within_2sigma"] * r["voxels"]
        voxels += r["voxels"]
        assert abs(r["mean_signed_pct"]) < 2.0, (b, r)
    p = dc.P_2SIGMA
    floor = p - 3.0 * np.sqrt(p * (1 - p) / voxels)
    assert within / voxels >= floor, (within / voxels, floor, voxels)
    # A^T g per batch on both sides
    w = target.reshape(-1) + 0.1
    xo, xg = ob @ w, gb @ w                                                # [K, beamlets]
    mo, mg = xo.mean(0), xg.mean(0)
    se = np.sqrt(xo.var(0, ddof=1) / KO + xg.var(0, ddof=1) / KG)
    z = (mg - mo) / se
    print("A^T g z-scores", np.round(z, 2), "coverage", within / voxels)
    assert np.all(np.abs(z) < 4.0), z
    assert abs(np.mean((mg - mo) / mo)) < 0.01


def test_torch_operators(setup, tables_wlb, dpm):
    """torch.ops.dpmx (the registered C++ operators over the library's matrix
    handle) give the same matrix and the same products as the ctypes path"""
    import torch
    inf = importlib.import_module("dpm-g4cpp_gb300.influence")
    ops = inf.torch_ops()
    A = setup["A"]
    S = A.to_scipy()
    T = A.to_torch()
    assert T.layout == torch.sparse_csr and tuple(T.shape) == (A.rows, A.cols)
    np.testing.assert_array_equal(T.crow_indices().cpu().numpy(), S.indptr)
    np.testing.assert_array_equal(T.col_indices().cpu().numpy(), S.indices)
    np.testing.assert_array_equal(T.values().cpu().numpy(), S.data)
    # a second matrix built through the operators from the same run
    res = setup["res"]
    rh = res._h.value if hasattr(res._h, "value") else res._h
    h = ops.influence_build(int(rh), 0, 0.0)
    try:
        rng = np.random.default_rng(3)
        x = torch.tensor(rng.random(A.cols), device="cuda")
        g = torch.tensor(rng.random(A.rows), device="cuda")
        assert torch.equal(ops.csr_matvec(h, x), A.matvec(x))
        assert torch.equal(ops.csr_rmatvec(h, g), A.rmatvec(g))
    finally:
        ops.csr_free(h)


def test_largest_beamlet_grid(tables_wlb, dpm):
    """65535 beamlets (255 x 257, the largest grid) on a small phantom: the
    tagged run's columns still sum to its dose, the matrix has one column
    per beamlet, products match the CPU; a 65536-beamlet grid is refused"""
    import torch
    ph = dpm.Phantom.voxels(tables_wlb, np.zeros((8, 8, 8), dtype=np.uint8), 2.0)
    src = dpm.Source(particle=0, e0=6.0, e1=6.0, shape=2, nbx=255, nby=257, fx=0.06, fy=0.06)
    res = dpm.run(tables_wlb, [dpm.Job(ph, src, 4 * 65535, 5)], batches=4, tag_beamlets=True)
    A = res.influence(0)
    S = A.to_scipy().astype(np.float64)
    dose = res.tally(0)[0].reshape(-1)
    assert (A.rows, A.cols) == (512, 65535) and S.shape == (512, 65535) and S.nnz > 0
    np.testing.assert_allclose(np.asarray(S.sum(axis=1)).ravel(), dose, rtol=2e-6, atol=1e-6 * dose.max())
    w = np.random.default_rng(1).random(S.shape[1])
    y = A.matvec(torch.tensor(w, device="cuda")).cpu().numpy()
    np.testing.assert_allclose(y, S @ w, rtol=1e-12, atol=1e-12 * np.abs(S @ w).max())
    big = dpm.Source(particle=0, e0=6.0, e1=6.0, shape=2, nbx=256, nby=256, fx=0.06, fy=0.06)
    with pytest.raises(dpm.DpmxError) as e:
        dpm.run(tables_wlb, [dpm.Job(ph, big, 1000, 5)], batches=2, tag_beamlets=True)
    assert e.value.code == dpm.ERR_ARG
