// Model-validation histograms on the GPU: the reference's modelValidationTests
// (testAPI.cc:92-198, AbstractTest set-up :1-40) sample one interaction many
// times for a primary of fixed energy moving along +z and histogram
//   x = log10(k / E0) on [log10(gamma cut / E0), 0.1] in hbins - 1 intervals
//       (k: the secondary's energy for brem and Moller, the primary's for MSC)
//   the direction cosine of the secondary (brem, Moller) or of the primary
//   (MSC), bin = (int)(cost * (hbins / 2) + hbins / 2)
// Here every sample has its own Philox stream (key = seed, history = sample
// index); the interaction formulas are those of the transport kernels, in FP64
// or FP32. Counts are summed per block in shared memory.
#include <algorithm>

#include "device_common.cuh"
#include "host_util.h"
#include "kernels.h"

namespace dpmx {
namespace {

template <class R>
__device__ __forceinline__ R Uniform(HistoryRng& rng) {
  const double u = rng.U();
  // a 53-bit uniform below 1 may round up to 1 in FP32
  return sizeof(R) == sizeof(float) ? R(fmin(u, 0.99999994)) : R(u);
}

template <class R>
__global__ void __launch_bounds__(256) ModelHistKernel(DevTables<R> T, int model, int imat, R e0, long long n,
                                                       uint64_t seed, int hbins, double xmin, double ihdel,
                                                       unsigned long long* hx, unsigned long long* hc) {
  extern __shared__ unsigned int counts[];   // [x bins | cosine bins]
  for (int b = threadIdx.x; b < 2 * hbins; b += blockDim.x) counts[b] = 0u;
  __syncthreads();
  const R kEMC2 = Consts<R>::kEMC2;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    HistoryRng rng;
    rng.Init(seed, uint32_t(i));
    R k = e0, cost = R(1);
    if (model == DPMX_MODEL_BREM) {            // SimDPMLike.cc:661-695 (sampler arguments drawn last-first)
      const R r3 = Uniform<R>(rng), r2 = Uniform<R>(rng), r1 = Uniform<R>(rng);
      k = SampleSB(T.sb[imat], e0, r1, r2, r3);
      const R dum0 = kEMC2 * R(0.7071067812) / (e0 + kEMC2);
      cost = mmax(R(-1), mmin(R(1), R(1) - dum0 * dum0));
    } else if (model == DPMX_MODEL_MOLLER) {   // SimDPMLike.cc:699-728
      const R r3 = Uniform<R>(rng), r2 = Uniform<R>(rng), r1 = Uniform<R>(rng);
      k = SampleMoller(T.mol, e0, r1, r2, r3);
      cost = mmin(R(1), msqrt(k * (e0 + R(2) * kEMC2) / (e0 * (k + R(2) * kEMC2))));
    } else {                                   // SimDPMLike.cc:731-750: the primary is deflected
      const R r2 = Uniform<R>(rng), r1 = Uniform<R>(rng);
      cost = mmax(R(-1), mmin(R(1), SampleGS(T.gs, e0, r1, r2)));
    }
    const int ic = int(double(cost) * (hbins / 2) + (hbins / 2));
    if (ic >= 0 && ic < hbins) atomicAdd(&counts[hbins + ic], 1u);
    const double red = double(k) / double(e0);
    if (red > 0.0) {
      const int ix = int((log10(red) - xmin) * ihdel);
      if (ix >= 0 && ix < hbins) atomicAdd(&counts[ix], 1u);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < hbins; b += blockDim.x) {
    if (counts[b]) atomicAdd(hx + b, (unsigned long long)counts[b]);
    if (counts[hbins + b]) atomicAdd(hc + b, (unsigned long long)counts[hbins + b]);
  }
}

}  // namespace
}  // namespace dpmx

using namespace dpmx;

extern "C" int dpmx_model_histogram(const dpmx_tables* t, int precision, int model, int imat, double e0,
                                    long long n, uint64_t seed, int hbins, double* hist_x, double* hist_cos) {
  if (!t || !hist_x || !hist_cos || n < 0 || n > 0xffffffffLL || hbins < 3 || hbins > 4096)
    return Fail(DPMX_ERR_ARG, "bad model-histogram arguments");
  if (model != DPMX_MODEL_BREM && model != DPMX_MODEL_MOLLER && model != DPMX_MODEL_MSC)
    return Fail(DPMX_ERR_ARG, "unknown interaction model");
  if (imat < 0 || imat >= t->h.nmat) return Fail(DPMX_ERR_ARG, "bad material index");
  if (!(e0 > t->h.gcut) || !(e0 < t->h.dedx[0].x.back())) return Fail(DPMX_ERR_ARG, "energy outside the tables");
  // AbstractTest::AbstractTest (testAPI.cc:19-24)
  const double xmin = std::log10(t->h.gcut / e0), xmax = 0.1;
  const double ihdel = 1.0 / ((xmax - xmin) / (hbins - 1));
  unsigned long long* d = nullptr;
  CK(cudaMalloc(&d, 2 * size_t(hbins) * sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, 2 * size_t(hbins) * sizeof(unsigned long long));
  const int blocks = int(std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 8)));
  const size_t smem = 2 * size_t(hbins) * sizeof(unsigned int);
  if (e == cudaSuccess) {
    if (precision == DPMX_FP64_PLAIN)
      ModelHistKernel<double><<<blocks, 256, smem>>>(t->t64, model, imat, e0, n, seed, hbins, xmin, ihdel, d, d + hbins);
    else
      ModelHistKernel<float><<<blocks, 256, smem>>>(t->t32, model, imat, float(e0), n, seed, hbins, xmin, ihdel, d,
                                                    d + hbins);
    e = cudaGetLastError();
  }
  std::vector<unsigned long long> h(2 * size_t(hbins));
  if (e == cudaSuccess) e = cudaMemcpy(h.data(), d, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  CK(e);
  for (int b = 0; b < hbins; ++b) {
    hist_x[b] = double(h[b]);
    hist_cos[b] = double(h[hbins + b]);
  }
  return DPMX_OK;
}

extern "C" int dpmx_ring_selftest(int blocks, int nslots, int rounds, uint64_t seed, long long probe_cycles,
                                  long long* out) {
  if (!out || blocks < 1 || blocks > 152 * 64 || nslots < 1 || nslots > 512 || rounds < 1 || rounds > (1 << 20) ||
      probe_cycles < 0 || probe_cycles > (1LL << 32))
    return Fail(DPMX_ERR_ARG, "bad ring self-test arguments");
  unsigned long long* d = nullptr;
  CK(cudaMalloc(&d, 4 * sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, 4 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = LaunchRingSelfTest(blocks, nslots, rounds, uint32_t(seed), probe_cycles, d, 0);
  unsigned long long h[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  CK(e);
  for (int i = 0; i < 4; ++i) out[i] = (long long)h[i];
  return DPMX_OK;
}
