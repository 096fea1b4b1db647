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
