// torch.ops.dpmx: the beamlet influence matrix of the library as registered
// PyTorch operators (loaded with torch.ops.load_library; nothing here is on
// the transport path). They call the C ABI of libdpmx.so; a matrix is the
// library's dpmx_csr object, passed between operators as an integer handle,
// which carries A by rows and the same entries by columns for A^T y.
//
//   dpmx::influence_build(int result, int job, float threshold) -> int
//       dpmx_influence_build on the dpmx_result* `result` (an integer): the
//       handle of A (rows: voxels, columns: beamlets)
//   dpmx::csr_tensor(int a) -> Tensor
//       A as a sparse CSR tensor on the GPU (int64 crow and column indices,
//       FP32 values; a copy owned by PyTorch)
//   dpmx::csr_matvec(int a, Tensor x) -> Tensor       y = A x
//   dpmx::csr_rmatvec(int a, Tensor y) -> Tensor      x = A^T y (no atomics:
//       the result does not depend on scheduling)
//       FP64 vectors and accumulation, on torch's current stream
//   dpmx::csr_free(int a) -> ()
//
// Errors of the library raise a c10::Error with dpmx_last_error's text.
#include <ATen/ATen.h>
#include <c10/cuda/CUDAFunctions.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/library.h>

#include "dpmx.h"

namespace {

void Check(int rc, const char* what) {
  TORCH_CHECK(rc == DPMX_OK, what, " failed: ", dpmx_last_error());
}

dpmx_csr* Csr(int64_t h) {
  TORCH_CHECK(h != 0, "dpmx: null matrix handle");
  return reinterpret_cast<dpmx_csr*>(h);
}

void Shape(dpmx_csr* a, long long& rows, long long& cols, long long& nnz) {
  Check(dpmx_csr_shape(a, &rows, &cols, &nnz), "dpmx_csr_shape");
}

int64_t InfluenceBuild(int64_t result, int64_t job, double threshold) {
  TORCH_CHECK(result != 0, "dpmx::influence_build: null result");
  dpmx_csr* a = nullptr;
  Check(dpmx_influence_build(reinterpret_cast<const dpmx_result*>(result), int(job), threshold, &a),
        "dpmx_influence_build");
  return reinterpret_cast<int64_t>(a);
}

at::Tensor CsrTensor(int64_t h) {
  dpmx_csr* a = Csr(h);
  long long rows = 0, cols = 0, nnz = 0;
  Shape(a, rows, cols, nnz);
  const int64_t* rp = nullptr;
  const int32_t* col = nullptr;
  const float* val = nullptr;
  Check(dpmx_csr_device(a, &rp, &col, &val), "dpmx_csr_device");
  const auto dev = at::TensorOptions().device(at::kCUDA, c10::cuda::current_device());
  at::Tensor crow = at::from_blob(const_cast<int64_t*>(rp), {rows + 1}, dev.dtype(at::kLong)).clone();
  at::Tensor ci = at::from_blob(const_cast<int32_t*>(col), {nnz}, dev.dtype(at::kInt)).to(at::kLong);
  at::Tensor v = at::from_blob(const_cast<float*>(val), {nnz}, dev.dtype(at::kFloat)).clone();
  return at::sparse_csr_tensor(crow, ci, v, {rows, cols}, dev.dtype(at::kFloat));
}

at::Tensor CsrMatvec(int64_t h, const at::Tensor& x) {
  dpmx_csr* a = Csr(h);
  long long rows = 0, cols = 0, nnz = 0;
  Shape(a, rows, cols, nnz);
  TORCH_CHECK(x.is_cuda() && x.dim() == 1 && x.size(0) == cols, "dpmx::csr_matvec: x must be a CUDA vector of ",
              cols, " elements");
  const at::Tensor xd = x.to(at::kDouble).contiguous();
  at::Tensor y = at::empty({rows}, xd.options());
  Check(dpmx_csr_spmv(a, xd.data_ptr<double>(), y.data_ptr<double>(), c10::cuda::getCurrentCUDAStream().stream()),
        "dpmx_csr_spmv");
  return y;
}

at::Tensor CsrRmatvec(int64_t h, const at::Tensor& y) {
  dpmx_csr* a = Csr(h);
  long long rows = 0, cols = 0, nnz = 0;
  Shape(a, rows, cols, nnz);
  TORCH_CHECK(y.is_cuda() && y.dim() == 1 && y.size(0) == rows, "dpmx::csr_rmatvec: y must be a CUDA vector of ",
              rows, " elements");
  const at::Tensor yd = y.to(at::kDouble).contiguous();
  at::Tensor x = at::empty({cols}, yd.options());
  Check(dpmx_csr_spmv_t(a, yd.data_ptr<double>(), x.data_ptr<double>(), c10::cuda::getCurrentCUDAStream().stream()),
        "dpmx_csr_spmv_t");
  return x;
}

void CsrFree(int64_t h) {
  if (h) dpmx_csr_free(reinterpret_cast<dpmx_csr*>(h));
}

}  // namespace

TORCH_LIBRARY(dpmx, m) {
  m.def("influence_build(int result, int job, float threshold) -> int", &InfluenceBuild);
  m.def("csr_tensor(int a) -> Tensor", &CsrTensor);
  m.def("csr_matvec(int a, Tensor x) -> Tensor", &CsrMatvec);
  m.def("csr_rmatvec(int a, Tensor y) -> Tensor", &CsrRmatvec);
  m.def("csr_free(int a) -> ()", &CsrFree);
}
