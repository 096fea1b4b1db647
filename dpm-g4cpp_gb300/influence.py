"""Differentiable dose from a beamlet influence matrix.

A beamlet-tagged run (run(..., tag_beamlets=True) with a beamlet-grid source)
tallies the dose of every beamlet separately; `Result.influence()` compresses
that tally on the GPU into a CSR matrix A (rows: voxels, columns: beamlets,
FP32 values). `dose(A, w)` is the autograd function D = A w whose hand-written
backward is A^T g; both products run in the library's CUDA kernels on torch's
current stream, with FP64 vectors and FP64 accumulation.
"""
import ctypes as C
import os

import numpy as np

from . import _check, library

_OPS = None


def torch_ops():
    """torch.ops.dpmx (lib/libdpmx_torch.so, built with the library): the
    influence matrix as registered operators on the library's matrix handle:
    influence_build(result, job, threshold) -> handle, csr_tensor(handle) ->
    sparse CSR tensor, csr_matvec(handle, x), csr_rmatvec(handle, y),
    csr_free(handle)."""
    global _OPS
    if _OPS is None:
        import torch
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libdpmx_torch.so")
        if not os.path.exists(path):
            raise RuntimeError("torch operators %s not built (run build())" % path)
        torch.ops.load_library(path)
        _OPS = torch.ops.dpmx
    return _OPS


class InfluenceMatrix:
    def __init__(self, handle):
        self._h = handle
        r, c, n = C.c_longlong(), C.c_longlong(), C.c_longlong()
        _check(library().dpmx_csr_shape(self._h, C.byref(r), C.byref(c), C.byref(n)))
        self.rows, self.cols, self.nnz = r.value, c.value, n.value

    @property
    def handle(self):
        return self._h

    def device_arrays(self):
        rp, col, val = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(library().dpmx_csr_device(self._h, C.byref(rp), C.byref(col), C.byref(val)))
        return rp.value, col.value, val.value

    def to_host(self):
        """(indptr int64, indices int32, data float32) copied to the host."""
        indptr = np.zeros(self.rows + 1, dtype=np.int64)
        indices = np.zeros(max(1, self.nnz), dtype=np.int32)
        data = np.zeros(max(1, self.nnz), dtype=np.float32)
        _check(library().dpmx_csr_download(self._h, indptr.ctypes.data, indices.ctypes.data, data.ctypes.data))
        return indptr, indices[:self.nnz], data[:self.nnz]

    def to_torch(self):
        """A as a torch sparse CSR tensor on the GPU (torch.ops.dpmx.csr_tensor)."""
        h = self._h.value if hasattr(self._h, "value") else self._h
        return torch_ops().csr_tensor(int(h))

    def to_scipy(self):
        """A as a scipy.sparse.csr_matrix on the host (FP32 values)."""
        import scipy.sparse as sp
        indptr, indices, data = self.to_host()
        return sp.csr_matrix((data, indices, indptr), shape=(self.rows, self.cols))

    def matvec(self, x):
        """y = A x for a CUDA float64 tensor x of length cols."""
        import torch
        x = x.contiguous()
        y = torch.empty(self.rows, dtype=torch.float64, device=x.device)
        st = torch.cuda.current_stream().cuda_stream
        _check(library().dpmx_csr_spmv(self._h, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(st)))
        return y

    def rmatvec(self, y):
        """x = A^T y for a CUDA float64 tensor y of length rows."""
        import torch
        y = y.contiguous()
        x = torch.empty(self.cols, dtype=torch.float64, device=y.device)
        st = torch.cuda.current_stream().cuda_stream
        _check(library().dpmx_csr_spmv_t(self._h, C.c_void_p(y.data_ptr()), C.c_void_p(x.data_ptr()), C.c_void_p(st)))
        return x

    def close(self):
        if self._h:
            library().dpmx_csr_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _make_function():
    import torch

    class DoseFunction(torch.autograd.Function):
        """D = A w; backward: dL/dw = A^T dL/dD."""

        @staticmethod
        def forward(ctx, w, A):
            ctx.A = A
            return A.matvec(w.to(torch.float64))

        @staticmethod
        def backward(ctx, g):
            return ctx.A.rmatvec(g.to(torch.float64).contiguous()), None

    return DoseFunction


_dose_fn = None


def dose(A, w):
    """Differentiable D = A w (torch CUDA tensors, float64)."""
    global _dose_fn
    if _dose_fn is None:
        _dose_fn = _make_function()
    return _dose_fn.apply(w, A)
