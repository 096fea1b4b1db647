// Kernel launch interfaces between the host orchestration (api.cu) and the
// transport translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dpmx_internal.h"

namespace dpmx {

// run counters accumulated on the device (one set per job)
struct RunCounters {
  double deposited;
  double escaped;
  double primaryEnergy;
  unsigned long long maxResidualBits;   // max residual as ordered double bits
  unsigned long long steps;
  unsigned long long violations;
  unsigned long long lost;
  unsigned long long histories;
  unsigned long long photonSteps;   // Woodcock steps (FP32 form, accumulated on job 0)
};

// warp-reduced accumulation of per-thread counters (FP64 plain form)
__device__ inline void AccumulateCounters(RunCounters* c, double dep, double esc, double e0, double maxres,
                                          long long steps, long long viol, int lost) {
  const unsigned full = 0xffffffffu;
  for (int o = 16; o > 0; o >>= 1) {
    dep += __shfl_down_sync(full, dep, o);
    esc += __shfl_down_sync(full, esc, o);
    e0 += __shfl_down_sync(full, e0, o);
    maxres = fmax(maxres, __shfl_down_sync(full, maxres, o));
    steps += __shfl_down_sync(full, steps, o);
    viol += __shfl_down_sync(full, viol, o);
    lost += __shfl_down_sync(full, lost, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&c->deposited, dep);
    atomicAdd(&c->escaped, esc);
    atomicAdd(&c->primaryEnergy, e0);
    atomicMax(&c->maxResidualBits, (unsigned long long)__double_as_longlong(maxres));
    atomicAdd(&c->steps, (unsigned long long)steps);
    atomicAdd(&c->violations, (unsigned long long)viol);
    atomicAdd(&c->lost, (unsigned long long)lost);
  }
}

// ---- FP64 plain form (transport_fp64.cu) ----
cudaError_t LaunchFp64Slab(const DevTables<double>& T, const SlabGeomD& g, const double* density, const SourceD& src,
                           long long first, long long n, uint64_t seed, double* edep, double* steps, int cap,
                           int* maxIz, double* histEdep, RunCounters* cnt, int blocks, cudaStream_t st);
cudaError_t LaunchFp64Grid(const DevTables<double>& T, const GridGeom& g, const double* density, const SourceD& src,
                           long long first, long long n, uint64_t seed, double* tally, double* histEdep,
                           RunCounters* cnt, int blocks, cudaStream_t st);
cudaError_t LaunchSamplerEval64(const DevTables<double>& T, int s, int imat, const double* e, const double* r,
                                double* out, int n, cudaStream_t st);
cudaError_t LaunchTableEval64(const DevTables<double>& T, int q, int imat, const double* e, double* out, int n,
                              cudaStream_t st);

// ---- FP32 event-based form (transport_fp32.cu) ----
constexpr int kMaxJobs = 256;
constexpr int kMaxGenerations = 48;

struct JobF {                  // per-job geometry, source and tally (device view)
  int nx, ny, nz, tallyDepth;
  int matByDepth;              // material array indexed by iz only (slab presets)
  float vx, vy, vz, ivx, ivy, ivz;
  double x0, y0, z0;           // lower corner of voxel (0,0,0) [mm]
  const uint8_t* mat;
  double* tally;               // batch tally of this job: bin i of slice r at tally[r * sstride + i * tstride]
  long long tstride;
  long long sstride;
  double* steps;               // scoring-step counts (depth tally only) or null
  double* btally;              // beamlet-tagged tally [beamlet][nvox] or null
  int nbeamlets;
  int particle, spectrum, shape, nbx, nby;
  float e0, e1, cx, cy, fx, fy;
  uint32_t k0, k1;             // Philox key (job seed)
  RunCounters* cnt;
  int dbase;                   // first bin of this job (slice 0) in a block's shared depth tally, or -1
  const float* rho;            // per-voxel density [g/cm3] or null
  float wscale;                // Woodcock majorant scale (>= 1)
};

struct Segment {               // a run of primaries of one job inside a chunk
  int job;
  int pad;
  long long firstHist;         // first history index of the run within the job
  long long count;
  long long prefix;            // index of the run's first primary within the phase
  long long slotBase;          // energy-check slot of the run's first primary
};

// A queue is split into kStripes stripes, each with its own append counter
// (chosen by the appending warp), so that appends from all SMs do not meet on
// one atomic. Stripe s holds entries [s*stripeCap, s*stripeCap + count[s]).
constexpr int kStripes = 16;
constexpr int kWorkGrab = 64;  // queue items a warp claims per atomic

struct Queue {                 // SoA particle queue
  float *lx, *ly, *lz, *dx, *dy, *dz, *e;
  uint32_t *vox, *hist, *slot, *uidlo, *uidhi, *meta;
  unsigned long long capacity;   // total entries
  unsigned long long stripeCap;  // entries per stripe
};

struct PhaseArgs {
  DevTables<float> T;
  const JobF* jobs;
  int njobs;
  const Segment* segs;         // primaries of this phase (may be empty)
  int nsegs;
  long long nPrimaries;
  Queue in;                    // particles to transport in this phase
  const unsigned long long* inCount;   // kStripes counters
  Queue outE, outP;            // secondaries: electrons, photons
  unsigned long long* outECount;       // kStripes counters each
  unsigned long long* outPCount;
  unsigned long long* head;    // work counter of this phase
  double* histE;               // per-slot energy accounted (deposit + escape)
  double* histE0;              // per-slot primary energy
  unsigned long long* overflow;
  unsigned long long* fault;   // blocks that abandoned a bounded wait (results incomplete)
  int aggregate;               // warp-aggregated tally atomics
  int depthBins;               // > 0: depth tallies summed per block in shared memory first
  int depthStride;             //      (bins per job; job j at j * depthStride)
  int plainTally;              // 1: every job scores a 3-D voxel tally only (depthBins 0, no
                               //    tallyDepth, step counts or beamlet tally): the block kernels
                               //    built for that form run
  int plainGeom;               // 1: every job is a voxel phantom of material ids with nominal
                               //    densities (no slab preset, no per-voxel density array), and
                               //    the electron splines of all materials share one grid
  int slabForm;                // 1: every job is a slab preset whose depth bins fit the block's
                               //    shared depth tally (depthBins > 0), no beamlet tally, and the
                               //    electron splines of all materials share one grid
  int tagForm;                 // 1: every job scores a 3-D voxel tally and a beamlet tally only
  int soloJob;                 // 1: every particle of this launch belongs to one job, job0
  JobF job0;                   // that job's record (read from the kernel parameters), else job 0's
};

// shared-memory depth tally of a block (slab jobs): bins of all jobs of a run
constexpr int kDepthBins = 1024;

cudaError_t PreparePhotonPhase(const DevTables<float>& T);   // shared-memory limit, once per run
cudaError_t LaunchPhotonPhase(const PhaseArgs& a, int blocks, int threads, cudaStream_t st);
// block-batched photon phase (256 threads per block, shared-memory slots)
int PhotonBlockBlocksPerSM();
cudaError_t LaunchPhotonPhaseBlock(const PhaseArgs& a, int blocks, cudaStream_t st);
cudaError_t LaunchElectronPhase(const PhaseArgs& a, int blocks, int threads, cudaStream_t st);
// dose += t, dose2 += t^2, t = 0 over n bins
cudaError_t LaunchFold(double* t, double* dose, double* dose2, long long n, cudaStream_t st);
// the same over m batch slices, bin i of slice b at t[i * binStride + b * sliceStride]:
// dose[i] += sum_b t, dose2[i] += sum_b t^2; clear: zero the slices after
cudaError_t LaunchFoldSlices(double* t, double* dose, double* dose2, long long n, long long binStride,
                             long long sliceStride, int m, bool clear, cudaStream_t st);
// *sum += sum of d[0..n), *lastNz = max(*lastNz, 1 + index of the last non-zero bin)
cudaError_t LaunchTallySummary(const double* d, long long n, double* sum, unsigned long long* lastNz,
                               cudaStream_t st);
// per-slot energy check against the primary energy, per-job counters
cudaError_t LaunchEnergyCheck(const double* histE, const double* histE0, long long nslots, const Segment* segs,
                              int nsegs, const JobF* jobs, cudaStream_t st);
cudaError_t LaunchSamplerEval32(const DevTables<float>& T, int s, int imat, const double* e, const double* r,
                                double* out, int n, cudaStream_t st);
cudaError_t LaunchTableEval32(const DevTables<float>& T, int q, int imat, const double* e, double* out, int n,
                              cudaStream_t st);
// self-test of the block kernels' slot rings; out[4] (device, zeroed):
// visits, slots with a wrong visit count, warps that gave up, probe waits that
// ran out (one per block expected)
cudaError_t LaunchRingSelfTest(int blocks, int nslots, int rounds, uint32_t seed, long long probeCycles,
                               unsigned long long* out, cudaStream_t st);
int ElectronPhaseSmemBytes(const DevTables<float>& T);
// block-batched electron phase (320 threads per block, shared-memory slots)
int BlockPhaseSmemBytes(const DevTables<float>& T);
int BlockPhaseBlocksPerSM();
// the slots per block a run gets for a requested count (0: the default; the
// instantiated sizes are 448 and 384)
int BlockPhaseSlots(int requested);
cudaError_t PrepareBlockPhase(const DevTables<float>& T);
cudaError_t LaunchElectronPhaseBlock(const PhaseArgs& a, int blocks, int slots, cudaStream_t st);

// ---- influence matrix (influence.cu) ----
cudaError_t LaunchCountNnz(const double* dense, long long nvox, int nb, double thr, long long* rowCount,
                           cudaStream_t st);
cudaError_t LaunchFillCsr(const double* dense, long long nvox, int nb, double thr, const long long* rowPtr,
                          int32_t* col, float* val, cudaStream_t st);
cudaError_t LaunchSpmv(const int64_t* rowPtr, const int32_t* col, const float* val, long long rows, long long cols,
                       long long nnz, const double* x, double* y, cudaStream_t st);
cudaError_t LaunchMaxAbs(const double* a, long long n, unsigned long long* outBits, cudaStream_t st);

}  // namespace dpmx
