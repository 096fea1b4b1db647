// Beamlet influence matrix A (rows: voxels, columns: beamlets) built from the
// beamlet-tagged FP64 tally of an FP32 run, stored as CSR with FP32 values,
// and the two products of the differentiable dose D = A w:
//   forward  y = A x     one thread per row, FP64 accumulation
//   backward x = A^T y   per-block column partial sums in shared memory,
//                        one FP64 atomic per column and block
// These are HBM-bound: each product streams the CSR arrays once
// (4 B value + 4 B column per entry + 8 B row pointer per row).
#include <cstring>
#include <memory>

#include <cub/cub.cuh>

#include "host_util.h"

namespace dpmx {
namespace {

__global__ void CountNnzKernel(const double* dense, long long nvox, int nb, double thr, long long* cnt) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nvox; i += (long long)gridDim.x * blockDim.x) {
    long long c = 0;
    for (int b = 0; b < nb; ++b) c += fabs(dense[(long long)b * nvox + i]) > thr ? 1 : 0;
    cnt[i] = c;
  }
}

__global__ void FillCsrKernel(const double* dense, long long nvox, int nb, double thr, const long long* rowPtr,
                              int32_t* col, float* val) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nvox; i += (long long)gridDim.x * blockDim.x) {
    long long k = rowPtr[i];
    for (int b = 0; b < nb; ++b) {
      const double v = dense[(long long)b * nvox + i];
      if (fabs(v) > thr) { col[k] = b; val[k] = float(v); ++k; }
    }
  }
}

__global__ void SpmvKernel(const int64_t* rowPtr, const int32_t* col, const float* val, long long rows, const double* x,
                           double* y) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    const int64_t e = rowPtr[i + 1];
    for (int64_t k = rowPtr[i]; k < e; ++k) s += double(__ldg(val + k)) * __ldg(x + __ldg(col + k));
    y[i] = s;
  }
}

__global__ void SpmvTKernel(const int64_t* rowPtr, const int32_t* col, const float* val, long long rows,
                            long long cols, const double* y, double* x, int useShared) {
  extern __shared__ double part[];
  if (useShared) {
    for (long long c = threadIdx.x; c < cols; c += blockDim.x) part[c] = 0.0;
    __syncthreads();
  }
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x) {
    const double yi = y[i];
    if (yi == 0.0) continue;
    const int64_t e = rowPtr[i + 1];
    for (int64_t k = rowPtr[i]; k < e; ++k) {
      const double v = double(__ldg(val + k)) * yi;
      if (useShared) atomicAdd(part + __ldg(col + k), v);
      else atomicAdd(x + __ldg(col + k), v);
    }
  }
  if (useShared) {
    __syncthreads();
    for (long long c = threadIdx.x; c < cols; c += blockDim.x)
      if (part[c] != 0.0) atomicAdd(x + c, part[c]);
  }
}

__global__ void MaxAbsKernel(const double* a, long long n, unsigned long long* out) {
  double m = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    m = fmax(m, fabs(a[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

int Grid(long long n) { return int(std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 32))); }

}  // namespace

cudaError_t LaunchCountNnz(const double* dense, long long nvox, int nb, double thr, long long* rowCount,
                           cudaStream_t st) {
  CountNnzKernel<<<Grid(nvox), 256, 0, st>>>(dense, nvox, nb, thr, rowCount);
  return cudaGetLastError();
}
cudaError_t LaunchFillCsr(const double* dense, long long nvox, int nb, double thr, const long long* rowPtr,
                          int32_t* col, float* val, cudaStream_t st) {
  FillCsrKernel<<<Grid(nvox), 256, 0, st>>>(dense, nvox, nb, thr, rowPtr, col, val);
  return cudaGetLastError();
}
cudaError_t LaunchSpmv(const int64_t* rowPtr, const int32_t* col, const float* val, long long rows, const double* x,
                       double* y, cudaStream_t st) {
  SpmvKernel<<<Grid(rows), 256, 0, st>>>(rowPtr, col, val, rows, x, y);
  return cudaGetLastError();
}
cudaError_t LaunchSpmvT(const int64_t* rowPtr, const int32_t* col, const float* val, long long rows, long long cols,
                        const double* y, double* x, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(x, 0, cols * sizeof(double), st);
  if (e != cudaSuccess) return e;
  const int useShared = cols <= 4096 ? 1 : 0;
  const size_t smem = useShared ? size_t(cols) * sizeof(double) : 0;
  SpmvTKernel<<<std::min(Grid(rows), 152 * 4), 256, smem, st>>>(rowPtr, col, val, rows, cols, y, x, useShared);
  return cudaGetLastError();
}
cudaError_t LaunchMaxAbs(const double* a, long long n, unsigned long long* outBits, cudaStream_t st) {
  MaxAbsKernel<<<Grid(n), 256, 0, st>>>(a, n, outBits);
  return cudaGetLastError();
}

}  // namespace dpmx

using namespace dpmx;

extern "C" {

int dpmx_influence_build(const dpmx_result* r, int job, double threshold, dpmx_csr** out) {
  if (!r || !out || job < 0 || job >= int(r->jobs.size())) return Fail(DPMX_ERR_ARG, "bad job index");
  *out = nullptr;
  const JobOut& o = r->jobs[job];
  if (!o.d_btally) return Fail(DPMX_ERR_ARG, "the run did not tag beamlets (tag_beamlets = 0)");
  const long long nvox = o.nvox;
  const int nb = o.nbeamlets;
  unsigned long long* dmax = nullptr;
  CK(cudaMalloc(&dmax, sizeof(unsigned long long)));
  CK(cudaMemset(dmax, 0, sizeof(unsigned long long)));
  CK(LaunchMaxAbs(o.d_btally, nvox * nb, dmax, 0));
  unsigned long long bits = 0;
  CK(cudaMemcpy(&bits, dmax, sizeof(bits), cudaMemcpyDeviceToHost));
  cudaFree(dmax);
  double mx;
  std::memcpy(&mx, &bits, sizeof(mx));
  const double thr = threshold > 0.0 ? threshold * mx : 0.0;
  std::unique_ptr<dpmx_csr> a(new dpmx_csr());
  a->rows = nvox;
  a->cols = nb;
  CK(cudaMalloc(&a->rowPtr, (nvox + 1) * sizeof(int64_t)));
  long long* cnt = nullptr;
  CK(cudaMalloc(&cnt, (nvox + 1) * sizeof(long long)));
  CK(cudaMemset(cnt, 0, (nvox + 1) * sizeof(long long)));
  CK(LaunchCountNnz(o.d_btally, nvox, nb, thr, cnt, 0));
  size_t tmpBytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmpBytes, cnt, reinterpret_cast<long long*>(a->rowPtr), nvox + 1);
  void* tmp = nullptr;
  CK(cudaMalloc(&tmp, tmpBytes));
  CK(cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, cnt, reinterpret_cast<long long*>(a->rowPtr), nvox + 1));
  cudaFree(tmp);
  cudaFree(cnt);
  long long nnz = 0;
  CK(cudaMemcpy(&nnz, a->rowPtr + nvox, sizeof(long long), cudaMemcpyDeviceToHost));
  a->nnz = nnz;
  CK(cudaMalloc(&a->col, std::max<long long>(1, nnz) * sizeof(int32_t)));
  CK(cudaMalloc(&a->val, std::max<long long>(1, nnz) * sizeof(float)));
  CK(LaunchFillCsr(o.d_btally, nvox, nb, thr, reinterpret_cast<const long long*>(a->rowPtr), a->col, a->val, 0));
  CK(cudaDeviceSynchronize());
  *out = a.release();
  return DPMX_OK;
}

int dpmx_csr_shape(const dpmx_csr* a, long long* rows, long long* cols, long long* nnz) {
  if (!a) return Fail(DPMX_ERR_ARG, "null matrix");
  if (rows) *rows = a->rows;
  if (cols) *cols = a->cols;
  if (nnz) *nnz = a->nnz;
  return DPMX_OK;
}

int dpmx_csr_device(const dpmx_csr* a, const int64_t** row_ptr, const int32_t** col, const float** val) {
  if (!a) return Fail(DPMX_ERR_ARG, "null matrix");
  if (row_ptr) *row_ptr = a->rowPtr;
  if (col) *col = a->col;
  if (val) *val = a->val;
  return DPMX_OK;
}

int dpmx_csr_spmv(const dpmx_csr* a, const double* x, double* y, void* stream) {
  if (!a || !x || !y) return Fail(DPMX_ERR_ARG, "null argument");
  CK(LaunchSpmv(a->rowPtr, a->col, a->val, a->rows, x, y, static_cast<cudaStream_t>(stream)));
  return DPMX_OK;
}

int dpmx_csr_spmv_t(const dpmx_csr* a, const double* y, double* x, void* stream) {
  if (!a || !x || !y) return Fail(DPMX_ERR_ARG, "null argument");
  CK(LaunchSpmvT(a->rowPtr, a->col, a->val, a->rows, a->cols, y, x, static_cast<cudaStream_t>(stream)));
  return DPMX_OK;
}

int dpmx_csr_download(const dpmx_csr* a, int64_t* row_ptr, int32_t* col, float* val) {
  if (!a) return Fail(DPMX_ERR_ARG, "null matrix");
  if (row_ptr) CK(cudaMemcpy(row_ptr, a->rowPtr, (a->rows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost));
  if (col && a->nnz) CK(cudaMemcpy(col, a->col, a->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (val && a->nnz) CK(cudaMemcpy(val, a->val, a->nnz * sizeof(float), cudaMemcpyDeviceToHost));
  return DPMX_OK;
}

void dpmx_csr_free(dpmx_csr* a) { delete a; }

}  // extern "C"
