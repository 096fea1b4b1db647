// Beamlet influence matrix A (rows: voxels, columns: beamlets) built from the
// beamlet-tagged FP64 tally of an FP32 run, stored as CSR with FP32 values,
// plus the same entries grouped by column (CSR of A^T), and the two products
// of the differentiable dose D = A w:
//   forward  y = A x     2-16 lanes per row by the matrix's mean row length,
//                        x staged in shared memory, FP64 accumulation
//   backward x = A^T y   CSR of A^T: `splits` blocks per column each reduce a
//                        slice of the column, then one pass sums the slices
//                        (no atomics: the result does not depend on timing)
// Each streams its CSR arrays once (4 B value + 4 B index per entry + 8 B
// pointer per row) and gathers the dense vector from L2 or shared memory; the
// FP64 conversion and multiply-add of every entry run on GB300's FP64 units
// (1/64 of the FP32 rate), which bound them about as much as the traffic.
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

constexpr int kColChunk = 2048;    // rows per block when grouping entries by column

// y = A x with LANES lanes per row, chosen per matrix from its mean row length
// (a lane sums its share of the row, then the lanes reduce); config 4's matrix
// (53 entries a row) runs y = A x in 0.73 ms with 2 lanes, 0.77 with 4, 1.05
// with 8, 1.18 with 16 and 0.83 with 1
template <int LANES>
__global__ void __launch_bounds__(256) SpmvKernel(const int64_t* rowPtr, const int32_t* col, const float* val,
                                                  long long rows, long long cols, const double* x, double* y,
                                                  int stageX) {
  extern __shared__ double xs[];
  if (stageX) {
    for (long long c = threadIdx.x; c < cols; c += blockDim.x) xs[c] = x[c];
    __syncthreads();
  }
  const double* xv = stageX ? xs : x;
  const int sub = threadIdx.x % LANES;
  const long long first = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / LANES;
  const long long stride = (long long)gridDim.x * blockDim.x / LANES;
  for (long long i = first; i < rows; i += stride) {
    double s = 0.0;
    const int64_t e = rowPtr[i + 1];
    for (int64_t k = rowPtr[i] + sub; k < e; k += LANES) s += double(__ldg(val + k)) * xv[__ldg(col + k)];
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, LANES);
    if (sub == 0) y[i] = s;
  }
}

// block (c, s): slice s of column c of A^T y
__global__ void __launch_bounds__(256) SpmvTSliceKernel(const int64_t* colPtr, const int32_t* rowT, const float* valT,
                                                        const double* y, int splits, double* partial) {
  __shared__ double red[8];
  const int c = blockIdx.x / splits, sl = blockIdx.x % splits;
  const int64_t b0 = colPtr[c], b1 = colPtr[c + 1];
  const int64_t len = b1 - b0;
  const int64_t lo = b0 + len * sl / splits, hi = b0 + len * (sl + 1) / splits;
  double s = 0.0;
  for (int64_t k = lo + threadIdx.x; k < hi; k += blockDim.x) s += double(__ldg(valT + k)) * __ldg(y + __ldg(rowT + k));
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < int(blockDim.x >> 5); ++w) s += red[w];
    partial[blockIdx.x] = s;
  }
}

__global__ void SumSlicesKernel(const double* partial, long long cols, int splits, double* x) {
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < splits; ++k) s += partial[c * splits + k];
    x[c] = s;
  }
}

// entries of column b in rows [chunk * kColChunk, +kColChunk): count
__global__ void __launch_bounds__(256) ColCountKernel(const double* dense, long long nvox, int nchunks, double thr,
                                                      long long* cnt) {
  using BR = cub::BlockReduce<long long, 256>;
  __shared__ typename BR::TempStorage tmp;
  const int b = blockIdx.x / nchunks, ch = blockIdx.x % nchunks;
  const double* d = dense + (long long)b * nvox;
  long long n = 0;
  for (int j = 0; j < kColChunk; j += 256) {
    const long long i = (long long)ch * kColChunk + j + threadIdx.x;
    if (i < nvox && fabs(d[i]) > thr) ++n;
  }
  n = BR(tmp).Sum(n);
  if (threadIdx.x == 0) cnt[blockIdx.x] = n;
}

// ... and their row indices and values in row order, from offset off[block]
__global__ void __launch_bounds__(256) ColFillKernel(const double* dense, long long nvox, int nchunks, double thr,
                                                     const long long* off, int32_t* rowT, float* valT) {
  using BS = cub::BlockScan<int, 256>;
  __shared__ typename BS::TempStorage tmp;
  const int b = blockIdx.x / nchunks, ch = blockIdx.x % nchunks;
  const double* d = dense + (long long)b * nvox;
  long long base = off[blockIdx.x];
  for (int j = 0; j < kColChunk; j += 256) {
    const long long i = (long long)ch * kColChunk + j + threadIdx.x;
    const double v = i < nvox ? d[i] : 0.0;
    const int f = (i < nvox && fabs(v) > thr) ? 1 : 0;
    int pos = 0, tot = 0;
    BS(tmp).ExclusiveSum(f, pos, tot);
    if (f) {
      rowT[base + pos] = int32_t(i);
      valT[base + pos] = float(v);
    }
    base += tot;
    __syncthreads();   // the scan storage is reused
  }
}

// column pointers from the per-(column, chunk) offsets
__global__ void ColPtrKernel(const long long* off, int cols, int nchunks, long long nnz, int64_t* colPtr) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c <= cols; c += gridDim.x * blockDim.x)
    colPtr[c] = c < cols ? off[(long long)c * nchunks] : nnz;
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
cudaError_t LaunchSpmv(const int64_t* rowPtr, const int32_t* col, const float* val, long long rows, long long cols,
                       long long nnz, const double* x, double* y, cudaStream_t st) {
  const int stageX = cols <= 6144 ? 1 : 0;
  const double mean = rows > 0 ? double(nnz) / double(rows) : 0.0;
  const int lanes = mean < 64 ? 2 : mean < 256 ? 4 : mean < 1024 ? 8 : 16;
  const long long threads = rows * lanes;
  const int blocks = int(std::max<long long>(1, std::min<long long>((threads + 255) / 256, 152LL * 8)));
  const size_t smem = stageX ? cols * sizeof(double) : 0;
  switch (lanes) {
    case 2: SpmvKernel<2><<<blocks, 256, smem, st>>>(rowPtr, col, val, rows, cols, x, y, stageX); break;
    case 4: SpmvKernel<4><<<blocks, 256, smem, st>>>(rowPtr, col, val, rows, cols, x, y, stageX); break;
    case 8: SpmvKernel<8><<<blocks, 256, smem, st>>>(rowPtr, col, val, rows, cols, x, y, stageX); break;
    default: SpmvKernel<16><<<blocks, 256, smem, st>>>(rowPtr, col, val, rows, cols, x, y, stageX); break;
  }
  return cudaGetLastError();
}
cudaError_t LaunchSpmvT(const dpmx_csr* a, const double* y, double* x, cudaStream_t st) {
  if (a->cols == 0) return cudaSuccess;
  SpmvTSliceKernel<<<int(a->cols * a->splits), 256, 0, st>>>(a->colPtr, a->rowT, a->valT, y, a->splits, a->partial);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  SumSlicesKernel<<<int(std::min<long long>((a->cols + 255) / 256, 152LL)), 256, 0, st>>>(a->partial, a->cols,
                                                                                          a->splits, x);
  return cudaGetLastError();
}
cudaError_t LaunchMaxAbs(const double* a, long long n, unsigned long long* outBits, cudaStream_t st) {
  MaxAbsKernel<<<Grid(n), 256, 0, st>>>(a, n, outBits);
  return cudaGetLastError();
}

}  // namespace dpmx

using namespace dpmx;

namespace {

// stream-ordered temporaries of one call: freed on its stream where the call
// frees them, or when it leaves early on an error
struct AsyncTemps {
  cudaStream_t st;
  std::vector<void*> v;
  explicit AsyncTemps(cudaStream_t s) : st(s) {}
  template <class T> cudaError_t Get(T** p, size_t bytes) {
    void* q = nullptr;
    const cudaError_t e = cudaMallocAsync(&q, bytes, st);
    if (e == cudaSuccess) {
      v.push_back(q);
      *p = static_cast<T*>(q);
    }
    return e;
  }
  cudaError_t Free(void* p) {
    for (void*& q : v)
      if (q == p) {
        q = nullptr;
        return cudaFreeAsync(p, st);
      }
    return cudaSuccess;
  }
  ~AsyncTemps() {
    for (void* q : v)
      if (q) cudaFreeAsync(q, st);
  }
};

}  // namespace

extern "C" {

int dpmx_influence_build(const dpmx_result* r, int job, double threshold, dpmx_csr** out) {
  if (!r || !out || job < 0 || job >= int(r->jobs.size())) return Fail(DPMX_ERR_ARG, "bad job index");
  *out = nullptr;
  const JobOut& o = r->jobs[job];
  if (!o.d_btally) return Fail(DPMX_ERR_ARG, "the run did not tag beamlets (tag_beamlets = 0)");
  // the build runs on a stream of its own and takes its temporaries from the
  // stream-ordered allocator, so it waits for nothing but its own work
  StreamGuard sg;
  CK(sg.Create());
  const cudaStream_t st = sg.st;
  AsyncTemps tmps(st);
  const long long nvox = o.nvox;
  const int nb = o.nbeamlets;
  unsigned long long* dmax = nullptr;
  CK(tmps.Get(&dmax, sizeof(unsigned long long)));
  CK(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), st));
  CK(LaunchMaxAbs(o.d_btally, nvox * nb, dmax, st));
  unsigned long long bits = 0;
  CK(cudaMemcpyAsync(&bits, dmax, sizeof(bits), cudaMemcpyDeviceToHost, st));
  CK(tmps.Free(dmax));
  CK(cudaStreamSynchronize(st));
  double mx;
  std::memcpy(&mx, &bits, sizeof(mx));
  const double thr = threshold > 0.0 ? threshold * mx : 0.0;
  std::unique_ptr<dpmx_csr> a(new dpmx_csr());
  a->rows = nvox;
  a->cols = nb;
  CK(cudaMalloc(&a->rowPtr, (nvox + 1) * sizeof(int64_t)));
  long long* cnt = nullptr;
  CK(tmps.Get(&cnt, (nvox + 1) * sizeof(long long)));
  CK(cudaMemsetAsync(cnt, 0, (nvox + 1) * sizeof(long long), st));
  CK(LaunchCountNnz(o.d_btally, nvox, nb, thr, cnt, st));
  size_t tmpBytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmpBytes, cnt, reinterpret_cast<long long*>(a->rowPtr), nvox + 1, st);
  void* tmp = nullptr;
  CK(tmps.Get(&tmp, tmpBytes));
  CK(cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, cnt, reinterpret_cast<long long*>(a->rowPtr), nvox + 1, st));
  CK(tmps.Free(tmp));
  CK(tmps.Free(cnt));
  long long nnz = 0;
  CK(cudaMemcpyAsync(&nnz, a->rowPtr + nvox, sizeof(long long), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  a->nnz = nnz;
  CK(cudaMalloc(&a->col, std::max<long long>(1, nnz) * sizeof(int32_t)));
  CK(cudaMalloc(&a->val, std::max<long long>(1, nnz) * sizeof(float)));
  CK(LaunchFillCsr(o.d_btally, nvox, nb, thr, reinterpret_cast<const long long*>(a->rowPtr), a->col, a->val, st));
  // the same entries by column, in row order within a column
  const int nchunks = int((nvox + kColChunk - 1) / kColChunk);
  const long long nblk = (long long)nb * nchunks;
  long long* ccnt = nullptr;
  long long* coff = nullptr;
  CK(tmps.Get(&ccnt, nblk * sizeof(long long)));
  CK(tmps.Get(&coff, nblk * sizeof(long long)));
  ColCountKernel<<<int(nblk), 256, 0, st>>>(o.d_btally, nvox, nchunks, thr, ccnt);
  CK(cudaGetLastError());
  tmpBytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmpBytes, ccnt, coff, nblk, st);
  CK(tmps.Get(&tmp, tmpBytes));
  CK(cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, ccnt, coff, nblk, st));
  CK(tmps.Free(tmp));
  CK(cudaMalloc(&a->colPtr, (nb + 1) * sizeof(int64_t)));
  CK(cudaMalloc(&a->rowT, std::max<long long>(1, nnz) * sizeof(int32_t)));
  CK(cudaMalloc(&a->valT, std::max<long long>(1, nnz) * sizeof(float)));
  ColFillKernel<<<int(nblk), 256, 0, st>>>(o.d_btally, nvox, nchunks, thr, coff, a->rowT, a->valT);
  CK(cudaGetLastError());
  ColPtrKernel<<<1, 256, 0, st>>>(coff, nb, nchunks, nnz, a->colPtr);
  CK(cudaGetLastError());
  // enough column slices to fill the GPU with blocks of A^T y
  a->splits = int(std::max<long long>(1, (4LL * 152 * 4 + nb - 1) / nb));
  CK(cudaMalloc(&a->partial, (long long)nb * a->splits * sizeof(double)));
  CK(tmps.Free(ccnt));
  CK(tmps.Free(coff));
  CK(cudaStreamSynchronize(st));
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
  CK(LaunchSpmv(a->rowPtr, a->col, a->val, a->rows, a->cols, a->nnz, x, y, static_cast<cudaStream_t>(stream)));
  return DPMX_OK;
}

int dpmx_csr_spmv_t(const dpmx_csr* a, const double* y, double* x, void* stream) {
  if (!a || !x || !y) return Fail(DPMX_ERR_ARG, "null argument");
  CK(LaunchSpmvT(a, y, x, static_cast<cudaStream_t>(stream)));
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
