// dpmx_simulate_noalloc: the reference Simulate workload in the plain FP64
// form without any device allocation by the library.
//
// Some integrations cannot let a plug-in allocate device memory: a dose engine
// hosted inside a treatment-planning or scheduling framework that owns every
// device byte through its own pool (and accounts for it), or a caller on a
// latency-critical path where a cudaMalloc / cudaFree would synchronise the
// device. For them this entry point takes its inputs (the tables loaded
// earlier) and its outputs (caller-owned device arrays) and keeps its few
// kilobytes of scratch - material densities, run counters, the deepest bin
// reached, and the batch tally - in one fixed file-scope device array.
//
// That array exists once per device that loads the library and lives until
// the process exits; every call shares it and finds the previous call's
// contents, so each call clears the parts that must start at zero. Calls that
// overlap on the GPU (on different streams or host threads) race on it and
// must be serialised by the caller. The first call on a device looks the
// array's device address up (cudaGetSymbolAddress) and keeps it for the life
// of the process; make that first call before any stream capture. A
// cudaDeviceReset destroys the array with the context, so no reset may come
// between calls. Each call synchronises its stream before it returns.
#include <cmath>
#include <mutex>
#include <string>

#include "host_util.h"

namespace dpmx {
namespace {

// scratch layout (bytes): [0, 256) RunCounters, [256, 512) deepest bin (int),
// [512, 1024) material densities, [1024, ...) batch tally of kNoAllocMaxBins bins
constexpr int kNoAllocMaxBins = 8192;
constexpr int kSlabMaxBins = 1023;       // the depth-bin limit of dpmx_phantom_slab
constexpr size_t kOffCounters = 0, kOffMaxIz = 256, kOffDensity = 512, kOffTally = 1024;
constexpr size_t kScratchBytes = kOffTally + size_t(kNoAllocMaxBins) * sizeof(double);
static_assert(sizeof(RunCounters) <= 256, "counters must fit their scratch slot");
static_assert(kMaxMat * sizeof(double) <= 512, "densities must fit their scratch slot");

static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratchMutex;
void* g_scratchAddr[kMaxDevices] = {nullptr};

// device address of the scratch array on the current device (set up once per device)
int ScratchAddress(unsigned char** out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return Fail(DPMX_ERR_ARG, "device index beyond the supported range");
  std::lock_guard<std::mutex> lock(g_scratchMutex);
  if (!g_scratchAddr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if (e != cudaSuccess) return Fail(DPMX_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratchAddr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_scratchAddr[dev]);
  return DPMX_OK;
}

}  // namespace
}  // namespace dpmx

using namespace dpmx;

extern "C" int dpmx_simulate_noalloc(const dpmx_tables* t, int nprimary, double eprimary, int iselectron, double lbox,
                                     int geom_index, uint64_t seed, double* edep, double* edep2, double* steps,
                                     int bins, int* hist_len, void* stream) {
  if (!t || nprimary < 0 || !(lbox > 0.0) || geom_index < 0 || !edep || !steps)
    return Fail(DPMX_ERR_ARG, "bad dpmx_simulate_noalloc arguments");
  if (bins > kNoAllocMaxBins)
    return Fail(DPMX_ERR_ARG, "dpmx_simulate_noalloc: bins = " + std::to_string(bins) + " exceeds the maximum of " +
                                  std::to_string(kNoAllocMaxBins) + " depth bins of its fixed scratch");
  // depth bins the reference world needs (z <= 100 mm), with the same limit
  // as dpmx_phantom_slab so that both entry points accept the same voxel sizes
  const int need = int(std::ceil((100.0 - 0.5 * lbox) / lbox - 1.0e-9)) + 1;
  if (need > kSlabMaxBins) return Fail(DPMX_ERR_ARG, "voxel size too small for the slab geometry");
  if (bins < need)
    return Fail(DPMX_ERR_ARG, "dpmx_simulate_noalloc: bins = " + std::to_string(bins) + " is below the " +
                                  std::to_string(need) + " depth bins of a " + std::to_string(lbox) + " mm geometry");
  for (int iz = 0; iz < need; ++iz)
    if (SlabMaterialAt(geom_index, 1.0 / lbox, iz) >= t->h.nmat)
      return Fail(DPMX_ERR_ARG, "the data set has fewer materials than the slab geometry needs");
  const double emin = iselectron ? t->h.ecut : t->h.gcut, emax = t->h.dedx[0].x.back();
  if (!(eprimary > emin) || !(eprimary < emax)) return Fail(DPMX_ERR_ARG, "primary energy outside the data-set grids");
  unsigned char* scratch = nullptr;
  if (int rc = ScratchAddress(&scratch)) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  RunCounters* cnt = reinterpret_cast<RunCounters*>(scratch + kOffCounters);
  int* maxIz = reinterpret_cast<int*>(scratch + kOffMaxIz);
  double* density = reinterpret_cast<double*>(scratch + kOffDensity);
  double* tally = reinterpret_cast<double*>(scratch + kOffTally);
  // the scratch keeps the previous call's contents: clear what accumulates
  CK(cudaMemsetAsync(scratch, 0, kOffDensity, st));
  CK(cudaMemsetAsync(tally, 0, size_t(bins) * sizeof(double), st));
  CK(cudaMemcpyAsync(density, t->h.density.data(), t->h.nmat * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(edep, 0, size_t(bins) * sizeof(double), st));
  CK(cudaMemsetAsync(steps, 0, size_t(bins) * sizeof(double), st));
  if (edep2) CK(cudaMemsetAsync(edep2, 0, size_t(bins) * sizeof(double), st));
  SourceD src{};
  src.particle = iselectron ? -1 : 0;
  src.e0 = src.e1 = eprimary;
  const SlabGeomD g{geom_index, lbox, 1.0 / lbox, 0.5 * lbox};
  CK(LaunchFp64Slab(t->t64, g, density, src, 0, nprimary, seed, tally, steps, bins, maxIz, nullptr, cnt,
                    NumSMs() * 16, st));
  // one statistical batch: dose += t, dose^2 += t^2 into the caller's arrays
  if (edep2) {
    CK(LaunchFold(tally, edep, edep2, bins, st));
  } else {
    CK(cudaMemcpyAsync(edep, tally, size_t(bins) * sizeof(double), cudaMemcpyDeviceToDevice, st));
  }
  RunCounters hc;
  int hz = 0;
  CK(cudaMemcpyAsync(&hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&hz, maxIz, sizeof(hz), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (hist_len) *hist_len = HistLen(hz);
  if (hc.lost > 0) return Fail(DPMX_ERR_OVERFLOW, "secondary stack overflow or step limit reached");
  return DPMX_OK;
}
