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

// ---------------------------------------------------------------------------
// Random-number hook: the Philox-4x32-10 block of each (counter, key) and the
// uniforms both transport forms make of it (UniformF32 of each word,
// UniformF64 of each word pair), for known-answer tests
// ---------------------------------------------------------------------------
namespace dpmx {
namespace {
__global__ void RngEvalKernel(const uint32_t* ctr, const uint32_t* key, int n, uint32_t* words, float* u32,
                              double* u64) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 c = make_uint4(ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3]);
  const uint4 w = philox(c, key[2 * i], key[2 * i + 1]);
  words[4 * i] = w.x; words[4 * i + 1] = w.y; words[4 * i + 2] = w.z; words[4 * i + 3] = w.w;
  u32[4 * i] = UniformF32(w.x); u32[4 * i + 1] = UniformF32(w.y);
  u32[4 * i + 2] = UniformF32(w.z); u32[4 * i + 3] = UniformF32(w.w);
  u64[2 * i] = UniformF64(w.x, w.y);
  u64[2 * i + 1] = UniformF64(w.z, w.w);
}

// FP64 atomicAdd throughput into an L2-resident array: the roof of the dose
// tally (one FP64 atomic per deposit). Every thread adds to pseudo-random bins
// of `nbins` doubles; the launch fills the GPU (8 blocks of 256 per SM).
__global__ void __launch_bounds__(256) AtomicRoofKernel(double* bins, uint32_t nbins, int per) {
  uint32_t x = (blockIdx.x * blockDim.x + threadIdx.x) * 0x9E3779B9u + 1u;
  for (int k = 0; k < per; ++k) {
    x ^= x << 13; x ^= x >> 17; x ^= x << 5;     // xorshift32
    atomicAdd(bins + (x % nbins), 1.0);
  }
}
}  // namespace
}  // namespace dpmx

extern "C" int dpmx_rng_eval(const uint32_t* counters, const uint32_t* keys, int n, uint32_t* words, float* u32,
                             double* u64) {
  if (n < 0 || (n > 0 && (!counters || !keys || !words || !u32 || !u64)))
    return Fail(DPMX_ERR_ARG, "bad random-number hook arguments");
  if (n == 0) return DPMX_OK;
  // one allocation: counters (4n), keys (2n), words (4n) as uint32, u32 (4n), u64 (2n)
  const size_t bytes = size_t(n) * (10 * sizeof(uint32_t) + 4 * sizeof(float) + 2 * sizeof(double));
  unsigned char* d = nullptr;
  CK(cudaMalloc(&d, bytes));
  uint32_t* dc = reinterpret_cast<uint32_t*>(d);
  uint32_t* dk = dc + 4 * size_t(n);
  uint32_t* dw = dk + 2 * size_t(n);
  float* df = reinterpret_cast<float*>(dw + 4 * size_t(n));
  double* dd = reinterpret_cast<double*>(df + 4 * size_t(n));   // 56n bytes in: 8-byte aligned
  cudaError_t e = cudaMemcpy(dc, counters, 4 * size_t(n) * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dk, keys, 2 * size_t(n) * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    RngEvalKernel<<<(n + 255) / 256, 256>>>(dc, dk, n, dw, df, dd);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(words, dw, 4 * size_t(n) * sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(u32, df, 4 * size_t(n) * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(u64, dd, 2 * size_t(n) * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d);
  CK(e);
  return DPMX_OK;
}

extern "C" int dpmx_atomic_roof(int nbins, int per_thread, double* atomics_per_s) {
  if (nbins < 1 || nbins > (1 << 26) || per_thread < 1 || per_thread > (1 << 16) || !atomics_per_s)
    return Fail(DPMX_ERR_ARG, "bad atomic-roof arguments");
  StreamGuard sg;
  CK(sg.Create());
  double* d = nullptr;
  CK(cudaMallocAsync(&d, size_t(nbins) * sizeof(double), sg.st));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMemsetAsync(d, 0, size_t(nbins) * sizeof(double), sg.st);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int blocks = NumSMs() * 8;
  if (e == cudaSuccess) {
    AtomicRoofKernel<<<blocks, 256, 0, sg.st>>>(d, uint32_t(nbins), per_thread);   // warm-up
    cudaEventRecord(e0, sg.st);
    AtomicRoofKernel<<<blocks, 256, 0, sg.st>>>(d, uint32_t(nbins), per_thread);
    cudaEventRecord(e1, sg.st);
    e = cudaGetLastError();
  }
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaStreamSynchronize(sg.st);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaFreeAsync(d, sg.st);
  cudaStreamSynchronize(sg.st);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  CK(e);
  *atomics_per_s = double(blocks) * 256.0 * per_thread / (ms * 1e-3);
  return DPMX_OK;
}
