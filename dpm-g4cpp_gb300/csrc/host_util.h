// Host-side helpers shared by the C ABI translation units: error reporting and
// the result / matrix objects behind the opaque handles.
#pragma once

#include <string>
#include <vector>

#include "kernels.h"

namespace dpmx {

// records the message of the calling thread's last failure and returns code
int Fail(int code, const std::string& msg);
int NumSMs();
// Geom::GetMaterialIndex / GetVoxelMaterialDensity of the slab presets (Geom.cc:133-164)
int SlabMaterialAt(int geomIndex, double invL, int iz);
double SlabDensityAt(const dpmx_tables* t, int geomIndex, double invL, int iz);
// the reference's depth-histogram length for the deepest bin reached (Geom.cc:120-130)
int HistLen(int maxIz);

#define CK(call)                                                                               \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) {                                                                   \
      return ::dpmx::Fail(e_ == cudaErrorMemoryAllocation ? DPMX_ERR_NOMEM : DPMX_ERR_CUDA,    \
                          std::string(#call) + ": " + cudaGetErrorString(e_));                 \
    }                                                                                          \
  } while (0)

// a non-blocking stream owned by one call, destroyed with it (after its work
// has finished, also when the call leaves early on an error: buffers it used
// may go back to a pool next)
struct StreamGuard {
  cudaStream_t st = nullptr;
  cudaError_t Create() { return cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking); }
  ~StreamGuard() {
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
  }
};

// CUDA events made by one call, destroyed with it (also when the call leaves
// early on an error)
struct EventSet {
  std::vector<cudaEvent_t> v;
  cudaError_t Add(cudaEvent_t* out, unsigned flags = cudaEventDefault) {
    cudaEvent_t e = nullptr;
    const cudaError_t r = cudaEventCreateWithFlags(&e, flags);
    if (r == cudaSuccess) {
      v.push_back(e);
      *out = e;
    }
    return r;
  }
  ~EventSet() {
    for (cudaEvent_t e : v) cudaEventDestroy(e);
  }
};

struct JobOut;
// returns a job's device buffers to the scratch pool. A run has finished all
// its own work on them when dpmx_run returns, so this waits for nothing; the
// caller's own use of dpmx_result_tally_device pointers must be complete
// before the result is freed.
void ReleaseJobOut(JobOut& o);
// a device block of the run scratch pool (no cudaMalloc once the pool holds
// one that fits, and no device-wide synchronisation when it goes back): for
// buffers whose last device use has completed when ScratchPut is called
cudaError_t ScratchGet(size_t bytes, void** out);
void ScratchPut(void* p);

struct JobOut {
  long long tallySize = 0;
  int slab = 0;              // depth tally of a slab preset
  double* d_dose = nullptr;
  double* d_dose2 = nullptr;
  double* d_steps = nullptr;
  double* d_btally = nullptr;
  int nbeamlets = 0;
  long long nvox = 0;
  int maxIz = 0;
  RunCounters cnt{};
  GridGeom grid{};                                      // for the dose outputs
  double lbox = 1.0;
  std::shared_ptr<const std::vector<float>> binDensity;
  std::shared_ptr<const std::vector<uint8_t>> binMaterial;
  std::shared_ptr<uint8_t> matDev;                     // material ids on the device (voxel phantoms)
  std::shared_ptr<const std::vector<float>> materialDensity;
  float BinDensity(long long i) const {
    return binDensity ? (*binDensity)[i] : (*materialDensity)[(*binMaterial)[i]];
  }
};

}  // namespace dpmx

struct dpmx_result {
  std::vector<dpmx::JobOut> jobs;
  double ms = 0.0;
  long long launches = 0;
  long long cfg[4] = {0, 0, 0, 0};
  int batches = 1;
  double prof[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  ~dpmx_result() {
    for (auto& j : jobs) dpmx::ReleaseJobOut(j);
  }
};

struct dpmx_csr {
  long long rows = 0, cols = 0, nnz = 0;
  int64_t* rowPtr = nullptr;   // CSR of A (rows: voxels)
  int32_t* col = nullptr;
  float* val = nullptr;
  int64_t* colPtr = nullptr;   // the same entries by column (CSR of A^T), for A^T y
  int32_t* rowT = nullptr;
  float* valT = nullptr;
  int splits = 1;              // blocks per column of A^T y
  double* partial = nullptr;   // [cols][splits] block sums of A^T y
  ~dpmx_csr() {
    cudaFree(rowPtr);
    cudaFree(col);
    cudaFree(val);
    cudaFree(colPtr);
    cudaFree(rowT);
    cudaFree(valT);
    cudaFree(partial);
  }
};
