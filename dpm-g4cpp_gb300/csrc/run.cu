// Run orchestration behind dpmx_run / dpmx_simulate and the remaining C ABI:
//
//  * FP64 plain form: per job and statistical batch, one launch of the
//    one-thread-per-history kernel into a batch tally, then a fold
//    (dose += t, dose2 += t^2).
//  * FP32 event form: the statistical batches of every job score into
//    separate tally slices (as many as fit a memory budget; more batches run
//    group after group), so the histories of a group are cut into chunks of
//    at most `chunk` histories regardless of batch boundaries; a chunk runs
//    kGen generations of (photon phase, electron phase) over double-buffered
//    queues, then the per-history energy check. After a group every slice is
//    folded (dose += t, dose2 += t^2). The launches of the whole run are
//    captured into one CUDA graph and launched once. Empty phases return at
//    once (their input count is read on the device).
//  * Tuning: a short sample of the jobs is timed for a few launch shapes
//    (lane or block electron kernel, threads per block and blocks per SM of
//    the lane kernels, warp-aggregated tally), and the fastest is used for
//    the run.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "host_util.h"

using namespace dpmx;

namespace {

// generations per chunk: the deepest generation that held particles was the
// 5th in every workload measured (slab presets, 64-job batches, 2e8 histories
// on the CT-like phantom); particles left after the last one fail the run
constexpr int kGen = 16;
// per chunk: striped counts of the electron and photon queues of every
// generation, the two work counters of every generation, the overflow count
// and the count of blocks that abandoned a bounded wait
constexpr int kCntStride = (kGen + 1) * kStripes;
constexpr int kCtrPerChunk = 2 * kCntStride + 2 * (kGen + 1) + 2;
constexpr long long kMaxChunk = 1LL << 24;            // default upper bound of histories per chunk
constexpr long long kLaneMinHistories = 1LL << 23;    // runs of at least this many histories get two chunk lanes
constexpr int kQueuePerPrimary = 6;                   // queue entries per primary of a chunk and generation
constexpr bool kInterleaveSlices = false;             // batch slices: per bin (true) or one after another

struct Cfg {
  int threads = 256;
  int blocksPerSM = 3;
  long long chunk = 1 << 20;
  int aggregate = 0;
  int eblock = 1;          // electron phase: 0 lane-refill kernel, 1 block-batched kernel
  int pblock = 1;          // photon phase: 0 one photon per lane, 1 block-batched kernel
  int eslots = 0;          // electron slots per block of the block-batched kernel (0: default)
};

// Device scratch kept across runs. A run of the FP32 form needs GBs of queues,
// energy-check slots and batch tallies; cudaMalloc / cudaFree of them on every
// run would cost milliseconds and synchronise the device. A block is lent to
// one run at a time and returns to the pool when the run ends; idle blocks are
// released when an allocation fails, or by dpmx_scratch_release.
class ScratchPool {
 public:
  static ScratchPool& Instance() {
    static ScratchPool* p = new ScratchPool;   // never destroyed: no CUDA calls at process exit
    return *p;
  }
  cudaError_t Get(size_t bytes, void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    bytes = (std::max<size_t>(bytes, 1) + kGrain - 1) / kGrain * kGrain;
    {
      std::lock_guard<std::mutex> g(m_);
      Block* best = nullptr;
      for (auto& b : blocks_)
        if (!b.busy && b.dev == dev && b.bytes >= bytes && b.bytes <= 2 * bytes && (!best || b.bytes < best->bytes))
          best = &b;
      if (best) {
        best->busy = true;
        *out = best->p;
        return cudaSuccess;
      }
    }
    void* p = nullptr;
    e = cudaMalloc(&p, bytes);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      Release(dev);
      e = cudaMalloc(&p, bytes);
    }
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(m_);
    blocks_.push_back({dev, p, bytes, true});
    *out = p;
    return cudaSuccess;
  }
  void Put(void* p) {
    std::lock_guard<std::mutex> g(m_);
    for (auto& b : blocks_)
      if (b.p == p) b.busy = false;
  }
  // frees the idle blocks of device dev (all devices when dev < 0)
  void Release(int dev) {
    std::vector<Block> f;
    {
      std::lock_guard<std::mutex> g(m_);
      std::vector<Block> keep;
      for (auto& b : blocks_) ((!b.busy && (dev < 0 || b.dev == dev)) ? f : keep).push_back(b);
      blocks_.swap(keep);
    }
    int cur = 0;
    cudaGetDevice(&cur);
    for (auto& b : f) {
      cudaSetDevice(b.dev);
      cudaFree(b.p);
    }
    cudaSetDevice(cur);
  }

 private:
  static constexpr size_t kGrain = size_t(1) << 18;
  struct Block { int dev; void* p; size_t bytes; bool busy; };
  std::mutex m_;
  std::vector<Block> blocks_;
};

struct DevBuf {       // scratch of one run, lent by the pool
  cudaStream_t st = nullptr;
  std::vector<void*> v;
  explicit DevBuf(cudaStream_t s) : st(s) {}
  ~DevBuf() {
    // nothing of this run may still use a block when it goes back
    cudaStreamSynchronize(st);
    for (void* p : v) ScratchPool::Instance().Put(p);
  }
  template <class T> int Get(T** p, size_t n) {
    void* q = nullptr;
    CK(ScratchPool::Instance().Get(std::max<size_t>(n, 1) * sizeof(T), &q));
    v.push_back(q);
    *p = static_cast<T*>(q);
    return DPMX_OK;
  }
};

int AllocQueue(DevBuf& b, Queue& q, unsigned long long cap) {
  q.stripeCap = (cap + kStripes - 1) / kStripes;
  cap = q.stripeCap * kStripes;
  q.capacity = cap;
  float** f[7] = {&q.lx, &q.ly, &q.lz, &q.dx, &q.dy, &q.dz, &q.e};
  uint32_t** u[6] = {&q.vox, &q.hist, &q.slot, &q.uidlo, &q.uidhi, &q.meta};
  for (auto x : f) if (int rc = b.Get(x, cap)) return rc;
  for (auto x : u) if (int rc = b.Get(x, cap)) return rc;
  return DPMX_OK;
}

struct Chunk {
  std::vector<Segment> segP, segE, segAll;   // photon primaries, electron primaries, all by slot
  long long nP = 0, nE = 0, nslots = 0;
  int job = -1;   // the chunk's only job, or -1 (none yet, or several)
  bool mixed = false;
};

// a job with at least this many histories in a batch group fills the GPU on
// its own: it gets chunks of its own, which run the single-job kernel forms
constexpr long long kSoloJobHistories = 1LL << 20;

// Cuts batches [b0, b1) (of B) of every job into chunks of at most `chunk`
// histories. Batch b of job j runs as sub-job ((b - b0) << 8) | j, which
// scores into its own tally slice; a chunk may span several batches. Jobs
// come one after another (all their batches together), so that a chunk holds
// few jobs and their tallies stay in L2; a job of kSoloJobHistories or more
// starts and ends on chunk boundaries.
std::vector<Chunk> PlanGroup(const dpmx_job* jobs, int njobs, int b0, int b1, int B, long long chunk) {
  std::vector<Chunk> out;
  Chunk cur;
  for (int j = 0; j < njobs; ++j) {
    const long long N = jobs[j].histories;
    const bool solo = N * b1 / B - N * b0 / B >= std::min(chunk, kSoloJobHistories);
    if (solo && cur.nslots > 0) { out.push_back(cur); cur = Chunk(); }
    for (int b = b0; b < b1; ++b) {
      const long long N = jobs[j].histories;
      long long first = N * b / B;
      long long left = N * (b + 1) / B - first;
      while (left > 0) {
        const long long take = std::min(left, chunk - cur.nslots);
        Segment s{};
        s.job = ((b - b0) << 8) | j;   // sub-job: job (low 8 bits) and tally slice
        s.firstHist = jobs[j].first_history + first;
        s.count = take;
        s.slotBase = cur.nslots;
        if (jobs[j].source.particle == 0) { s.prefix = cur.nP; cur.nP += take; cur.segP.push_back(s); }
        else { s.prefix = cur.nE; cur.nE += take; cur.segE.push_back(s); }
        cur.segAll.push_back(s);
        if (cur.nslots == 0 && !cur.mixed) cur.job = j;
        else if (cur.job != j) { cur.job = -1; cur.mixed = true; }
        cur.nslots += take;
        first += take;
        left -= take;
        if (cur.nslots == chunk) { out.push_back(cur); cur = Chunk(); }
      }
    }
    if (solo && cur.nslots > 0) { out.push_back(cur); cur = Chunk(); }
  }
  if (cur.nslots > 0) out.push_back(cur);
  return out;
}

// ---------------------------------------------------------------------------
// FP32 event form
// ---------------------------------------------------------------------------
int RunFp32(const dpmx_tables* T, const dpmx_job* jobs, int njobs, int batches, const Cfg& cfg, bool tag,
            bool useGraph, cudaStream_t st, std::vector<JobOut>& outs, double* ms, long long* launches,
            double* prof = nullptr) {
  // prof (optional, launches not captured): events around every phase launch
  // give the electron / photon phase times; see dpmx_result_profile
  const bool profile = prof != nullptr && !useGraph;
  std::vector<cudaEvent_t> evE, evP;
  DevBuf buf(st);
  const int nsm = NumSMs();
  // concatenated tallies of all jobs: batch tally slices (interleaved per
  // bin, so that the batches of one bin share cache lines), dose, dose2
  std::vector<long long> off(njobs);
  long long total = 0;
  for (int j = 0; j < njobs; ++j) { off[j] = total; total += outs[j].tallySize; }
  // tally slices: all batches at once when they fit an eighth of the free
  // memory (at most 16 GB), else groups of as many as fit
  size_t freeB = 0, totB = 0;
  CK(cudaMemGetInfo(&freeB, &totB));
  const double budget = std::min(16.0e9, double(freeB) / 8.0);
  const int R = int(std::max(1.0, std::min(double(batches), budget / (8.0 * double(std::max(1LL, total))))));
  const int ngroups = (batches + R - 1) / R;
  // the phase kernels address bins and slices with 32-bit offsets
  if (double(R) * double(total) >= 4294967296.0 || double(total) >= 4294967296.0)
    return Fail(DPMX_ERR_ARG, "the tallies of one run exceed 2^32 bins; run the jobs in smaller groups");
  const long long binStride = kInterleaveSlices ? R : 1, sliceStride = kInterleaveSlices ? 1 : total;
  double *tB, *dose, *dose2;
  if (int rc = buf.Get(&tB, size_t(R) * total)) return rc;
  if (int rc = buf.Get(&dose, total)) return rc;
  if (int rc = buf.Get(&dose2, total)) return rc;
  CK(cudaMemsetAsync(tB, 0, size_t(R) * total * sizeof(double), st));
  CK(cudaMemsetAsync(dose, 0, total * sizeof(double), st));
  CK(cudaMemsetAsync(dose2, 0, total * sizeof(double), st));
  RunCounters* cnt;
  if (int rc = buf.Get(&cnt, njobs)) return rc;
  CK(cudaMemsetAsync(cnt, 0, njobs * sizeof(RunCounters), st));
  // per job: deposited energy and 1 + the last non-zero tally bin
  double* dsum;
  unsigned long long* dlast;
  if (int rc = buf.Get(&dsum, njobs)) return rc;
  if (int rc = buf.Get(&dlast, njobs)) return rc;
  // one JobF per job; a particle's sub-job (slice << 8 | job) selects the
  // job's tally slice
  const int nsub = R * njobs;
  std::vector<JobF> hj(njobs);
  for (int j = 0; j < njobs; ++j) {
    const dpmx_phantom* ph = jobs[j].phantom;
    const GridGeom& g = ph->grid;
    JobF& J = hj[j];
    std::memset(&J, 0, sizeof(J));
    J.nx = g.nx; J.ny = g.ny; J.nz = g.nz;
    J.tallyDepth = g.tallyDepth;
    J.matByDepth = g.matByDepth;
    J.vx = float(g.vx); J.vy = float(g.vy); J.vz = float(g.vz);
    J.ivx = float(1.0 / g.vx); J.ivy = float(1.0 / g.vy); J.ivz = float(1.0 / g.vz);
    J.x0 = g.x0; J.y0 = g.y0; J.z0 = g.z0;
    J.mat = g.mat;
    J.rho = g.rho;
    J.wscale = float(g.wscale);
    J.tally = tB + off[j] * binStride;
    J.tstride = binStride;
    J.sstride = sliceStride;
    J.steps = outs[j].d_steps;
    J.btally = tag ? outs[j].d_btally : nullptr;
    J.nbeamlets = std::max(1, outs[j].nbeamlets);
    const dpmx_source& s = jobs[j].source;
    J.particle = s.particle; J.spectrum = s.spectrum; J.shape = s.shape; J.nbx = s.nbx; J.nby = s.nby;
    J.e0 = float(s.e0); J.e1 = float(s.e1);
    J.cx = float(s.cx); J.cy = float(s.cy); J.fx = float(s.fx); J.fy = float(s.fy);
    if (ph->kind == 0) { J.shape = 0; J.cx = 0.f; J.cy = 0.f; }   // the reference's pencil beam
    J.k0 = uint32_t(jobs[j].seed);
    J.k1 = uint32_t(jobs[j].seed >> 32) ^ 0x5bd1e995u;
    J.cnt = cnt + j;
  }
  // slab jobs: the depth tallies are summed per block in shared memory first
  // when the bins of all sub-jobs fit
  bool allSlab = true;
  int maxNz = 1;
  for (int j = 0; j < njobs; ++j) {
    allSlab = allSlab && outs[j].slab;
    maxNz = std::max(maxNz, jobs[j].phantom->grid.nz);
  }
  // bins: (slice * njobs + job) * maxNz + iz
  const int depthBins = (allSlab && (long long)nsub * maxNz <= kDepthBins) ? nsub * maxNz : 0;
  for (int j = 0; j < njobs; ++j) hj[j].dbase = depthBins ? j * maxNz : -1;
  // jobs that all score a 3-D voxel tally only run the block kernels built
  // for that tally form
  bool plainTally = depthBins == 0;
  bool plainGeom = true;
  for (int j = 0; j < njobs; ++j) {
    plainTally = plainTally && hj[j].tallyDepth == 0 && hj[j].steps == nullptr && hj[j].btally == nullptr;
    plainGeom = plainGeom && hj[j].matByDepth == 0 && hj[j].rho == nullptr;
  }
  plainGeom = plainGeom && T->t32.elecUniform != 0;
  // slab presets whose depth tallies stay in the blocks' shared memory run
  // the slab kernel forms
  // beamlet-tagged runs of 3-D voxel jobs run the tagged tally forms
  bool tagForm = depthBins == 0 && njobs > 0;
  for (int j = 0; j < njobs; ++j)
    tagForm = tagForm && hj[j].tallyDepth == 0 && hj[j].steps == nullptr && hj[j].btally != nullptr;
  bool slabForm = depthBins > 0 && T->t32.elecUniform != 0;
  for (int j = 0; j < njobs; ++j)
    slabForm = slabForm && hj[j].tallyDepth == 1 && hj[j].matByDepth == 1 && hj[j].rho == nullptr &&
               hj[j].btally == nullptr && hj[j].dbase >= 0;
  JobF* dj;
  if (int rc = buf.Get(&dj, njobs)) return rc;
  CK(cudaMemcpyAsync(dj, hj.data(), njobs * sizeof(JobF), cudaMemcpyHostToDevice, st));

  // plan and segment tables
  std::vector<std::vector<Chunk>> plan(ngroups);
  std::vector<Segment> segs;
  size_t nchunks = 0;
  long long maxSlots = 1;
  for (int gi = 0; gi < ngroups; ++gi) {
    plan[gi] = PlanGroup(jobs, njobs, gi * R, std::min(batches, (gi + 1) * R), batches, cfg.chunk);
    for (auto& c : plan[gi]) {
      segs.insert(segs.end(), c.segP.begin(), c.segP.end());
      segs.insert(segs.end(), c.segE.begin(), c.segE.end());
      segs.insert(segs.end(), c.segAll.begin(), c.segAll.end());
      maxSlots = std::max(maxSlots, c.nslots);
      ++nchunks;
    }
  }
  Segment* dsegs;
  if (int rc = buf.Get(&dsegs, segs.size())) return rc;
  if (!segs.empty()) CK(cudaMemcpyAsync(dsegs, segs.data(), segs.size() * sizeof(Segment), cudaMemcpyHostToDevice, st));
  // chunk lanes: consecutive chunks alternate between two streams (forked
  // and joined inside the captured graph), each lane with its own queues and
  // energy-check slots, so that one chunk's phases fill the SMs the other's
  // leave idle at the end of each phase (a phase-profiled run keeps one lane)
  const int nlanes = (nchunks >= 2 && !profile) ? 2 : 1;
  StreamGuard lane2;
  if (nlanes == 2) CK(lane2.Create());
  double *histE[2] = {nullptr, nullptr}, *histE0[2] = {nullptr, nullptr};
  for (int l = 0; l < nlanes; ++l) {
    if (int rc = buf.Get(&histE[l], maxSlots)) return rc;
    if (int rc = buf.Get(&histE0[l], maxSlots)) return rc;
  }
  unsigned long long* ctr;
  if (int rc = buf.Get(&ctr, nchunks * kCtrPerChunk)) return rc;
  CK(cudaMemsetAsync(ctr, 0, nchunks * kCtrPerChunk * sizeof(unsigned long long), st));
  // queues: double-buffered electrons and photons; a generation holds well
  // under kQueuePerPrimary secondaries of each kind per primary
  const unsigned long long cap = (unsigned long long)std::max<long long>(maxSlots * kQueuePerPrimary, 1 << 18);
  Queue qeL[2][2], qpL[2][2];   // [lane][generation parity]
  for (int l = 0; l < nlanes; ++l)
    for (int k = 0; k < 2; ++k) {
      if (int rc = AllocQueue(buf, qeL[l][k], cap)) return rc;
      if (int rc = AllocQueue(buf, qpL[l][k], cap)) return rc;
    }
  // every event of the run (lane fork and join, phase timing, run timing)
  EventSet evs;
  // fork and join events of the lanes, one pair per batch group
  std::vector<cudaEvent_t> evFork, evJoin;
  if (nlanes == 2)
    for (int gi = 0; gi < ngroups; ++gi) {
      cudaEvent_t f, j;
      CK(evs.Add(&f, cudaEventDisableTiming));
      evFork.push_back(f);
      CK(evs.Add(&j, cudaEventDisableTiming));
      evJoin.push_back(j);
    }
  const int blocks = nsm * cfg.blocksPerSM;
  const int eblocks = nsm * BlockPhaseBlocksPerSM();   // block-batched electron phase: one wave
  if (cfg.eblock) CK(PrepareBlockPhase(T->t32));
  CK(PreparePhotonPhase(T->t32));
  long long nl = 0;
  auto enqueue = [&](cudaStream_t s0) -> int {
    size_t segCur = 0, ci = 0;
    for (int gi = 0; gi < ngroups; ++gi) {
      if (nlanes == 2) {
        CK(cudaEventRecord(evFork[gi], s0));
        CK(cudaStreamWaitEvent(lane2.st, evFork[gi], 0));
      }
      for (auto& c : plan[gi]) {
        const int lane = int(ci % size_t(nlanes));
        const cudaStream_t s = lane == 0 ? s0 : lane2.st;
        Queue* qe = qeL[lane];
        Queue* qp = qpL[lane];
        unsigned long long* cc = ctr + ci * kCtrPerChunk;
        unsigned long long* cntE = cc;                       // [gen][stripe]
        unsigned long long* cntP = cc + kCntStride;
        unsigned long long* headE = cc + 2 * kCntStride;     // [gen]
        unsigned long long* headP = headE + (kGen + 1);
        unsigned long long* ovf = headP + (kGen + 1);
        unsigned long long* fault = ovf + 1;
        const Segment* sP = dsegs + segCur;
        const Segment* sE = sP + c.segP.size();
        const Segment* sA = sE + c.segE.size();
        CK(cudaMemsetAsync(histE[lane], 0, c.nslots * sizeof(double), s));
        for (int g = 0; g < kGen; ++g) {
          PhaseArgs a;
          std::memset(&a, 0, sizeof(a));
          a.T = T->t32;
          a.jobs = dj;
          a.njobs = njobs;
          a.histE = histE[lane];
          a.histE0 = histE0[lane];
          a.overflow = ovf;
          a.fault = fault;
          a.aggregate = cfg.aggregate;
          a.depthBins = depthBins;
          a.depthStride = maxNz;
          a.plainTally = plainTally ? 1 : 0;
          a.plainGeom = plainGeom ? 1 : 0;
          a.slabForm = slabForm ? 1 : 0;
          a.tagForm = tagForm ? 1 : 0;
          // a chunk of one job runs the single-job forms with that job's record
          a.soloJob = c.job >= 0 ? 1 : 0;
          if (njobs > 0) a.job0 = hj[c.job >= 0 ? c.job : 0];
          // photons of generation g; their electrons join generation g
          a.segs = sP; a.nsegs = int(c.segP.size()); a.nPrimaries = (g == 0) ? c.nP : 0;
          a.in = qp[g & 1]; a.inCount = cntP + g * kStripes;
          a.outE = qe[g & 1]; a.outECount = cntE + g * kStripes;
          a.outP = qp[(g + 1) & 1]; a.outPCount = cntP + (g + 1) * kStripes;
          a.head = headP + g;
          if (profile) {
            evP.resize(evP.size() + 2);
            CK(evs.Add(&evP[evP.size() - 2]));
            CK(evs.Add(&evP.back()));
            CK(cudaEventRecord(evP[evP.size() - 2], s));
          }
          if (cfg.pblock) CK(LaunchPhotonPhaseBlock(a, nsm * PhotonBlockBlocksPerSM(), s));
          else CK(LaunchPhotonPhase(a, blocks, cfg.threads, s));
          if (profile) CK(cudaEventRecord(evP.back(), s));
          ++nl;
          // electrons of generation g; their secondaries form generation g+1
          a.segs = sE; a.nsegs = int(c.segE.size()); a.nPrimaries = (g == 0) ? c.nE : 0;
          a.in = qe[g & 1]; a.inCount = cntE + g * kStripes;
          a.outE = qe[(g + 1) & 1]; a.outECount = cntE + (g + 1) * kStripes;
          a.outP = qp[(g + 1) & 1]; a.outPCount = cntP + (g + 1) * kStripes;
          a.head = headE + g;
          if (profile) {
            evE.resize(evE.size() + 2);
            CK(evs.Add(&evE[evE.size() - 2]));
            CK(evs.Add(&evE.back()));
            CK(cudaEventRecord(evE[evE.size() - 2], s));
          }
          if (cfg.eblock) CK(LaunchElectronPhaseBlock(a, eblocks, cfg.eslots, s));
          else CK(LaunchElectronPhase(a, blocks, cfg.threads, s));
          if (profile) CK(cudaEventRecord(evE.back(), s));
          ++nl;
        }
        CK(LaunchEnergyCheck(histE[lane], histE0[lane], c.nslots, sA, int(c.segAll.size()), dj, s));
        ++nl;
        segCur += c.segP.size() + c.segE.size() + c.segAll.size();
        ++ci;
      }
      if (nlanes == 2) {
        CK(cudaEventRecord(evJoin[gi], lane2.st));
        CK(cudaStreamWaitEvent(s0, evJoin[gi], 0));
      }
      const int nslice = std::min(batches, (gi + 1) * R) - gi * R;
      if (R == 1) CK(LaunchFold(tB, dose, dose2, total, s0));
      else CK(LaunchFoldSlices(tB, dose, dose2, total, binStride, sliceStride, nslice, gi + 1 < ngroups, s0));
      ++nl;
    }
    const cudaStream_t s = s0;
    // results into the per-job buffers, with their sums
    CK(cudaMemsetAsync(dsum, 0, njobs * sizeof(double), s));
    CK(cudaMemsetAsync(dlast, 0, njobs * sizeof(unsigned long long), s));
    for (int j = 0; j < njobs; ++j) {
      const size_t n = outs[j].tallySize * sizeof(double);
      CK(cudaMemcpyAsync(outs[j].d_dose, dose + off[j], n, cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(outs[j].d_dose2, dose2 + off[j], n, cudaMemcpyDeviceToDevice, s));
      CK(LaunchTallySummary(dose + off[j], outs[j].tallySize, dsum + j, dlast + j, s));
      ++nl;
    }
    return DPMX_OK;
  };

  cudaEvent_t e0, e1;
  CK(evs.Add(&e0));
  CK(evs.Add(&e1));
  int rc = DPMX_OK;
  if (useGraph) {
    // The executable graph of the calling thread's previous run is kept: a new
    // run of the same shape (jobs, chunk plan, buffers) only differs in kernel
    // and copy parameters, which cudaGraphExecUpdate applies without
    // instantiating again; any other run instantiates and replaces it. Runs of
    // one thread do not overlap (each ends with a synchronisation), so the
    // executable is never updated while in flight. It is not destroyed at
    // thread exit (no CUDA calls while the process shuts down).
    static thread_local cudaGraphExec_t tlExec = nullptr;
    static thread_local int tlDev = -1;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    rc = enqueue(st);
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
    CK(ce);
    bool updated = false;
    if (tlExec && tlDev != dev) {   // made on another device: not updatable here
      cudaGraphExecDestroy(tlExec);
      tlExec = nullptr;
    }
    if (tlExec) {
      cudaGraphExecUpdateResultInfo info;
      if (cudaGraphExecUpdate(tlExec, graph, &info) == cudaSuccess) {
        updated = true;
      } else {
        cudaGetLastError();
        cudaGraphExecDestroy(tlExec);
        tlExec = nullptr;
      }
    }
    if (!updated) {
      const cudaError_t ie = cudaGraphInstantiate(&tlExec, graph, 0);
      if (ie != cudaSuccess) { tlExec = nullptr; cudaGraphDestroy(graph); CK(ie); }
      tlDev = dev;
    }
    cudaGraphDestroy(graph);
    CK(cudaEventRecord(e0, st));
    CK(cudaGraphLaunch(tlExec, st));
    CK(cudaEventRecord(e1, st));
    CK(cudaStreamSynchronize(st));
  } else {
    CK(cudaEventRecord(e0, st));
    rc = enqueue(st);
    if (rc) return rc;
    CK(cudaEventRecord(e1, st));
    CK(cudaStreamSynchronize(st));
  }
  float fms = 0.f;
  CK(cudaEventElapsedTime(&fms, e0, e1));
  *ms = fms;
  *launches = nl;
  // results: leftovers beyond the last generation and queue overflows are losses
  std::vector<unsigned long long> hc(nchunks * kCtrPerChunk);
  CK(cudaMemcpy(hc.data(), ctr, hc.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  unsigned long long lost = 0, leftover = 0, overflowed = 0, faults = 0;
  double nElec = 0, nPhot = 0;
  for (size_t ci = 0; ci < nchunks; ++ci) {
    const unsigned long long* cc = hc.data() + ci * kCtrPerChunk;
    for (int k = 0; k < kStripes; ++k) leftover += cc[kGen * kStripes + k] + cc[kCntStride + kGen * kStripes + k];
    overflowed += cc[2 * kCntStride + 2 * (kGen + 1)];
    faults += cc[2 * kCntStride + 2 * (kGen + 1) + 1];
    for (int g = 0; g < kGen; ++g)
      for (int k = 0; k < kStripes; ++k) {
        nElec += double(cc[g * kStripes + k]);
        nPhot += double(cc[kCntStride + g * kStripes + k]);
      }
  }
  if (prof) {
    double te = 0, tp = 0;
    for (size_t k = 0; k + 1 < evE.size(); k += 2) {
      float x = 0.f;
      CK(cudaEventElapsedTime(&x, evE[k], evE[k + 1]));
      te += x;
    }
    for (size_t k = 0; k + 1 < evP.size(); k += 2) {
      float x = 0.f;
      CK(cudaEventElapsedTime(&x, evP[k], evP[k + 1]));
      tp += x;
    }
    double hist = 0, primE = 0, primP = 0;
    for (int j = 0; j < njobs; ++j) {
      hist += double(jobs[j].histories);
      (jobs[j].source.particle == 0 ? primP : primE) += double(jobs[j].histories);
    }
    RunCounters c0{};
    CK(cudaMemcpy(&c0, cnt, sizeof(RunCounters), cudaMemcpyDeviceToHost));
    prof[0] = te;
    prof[1] = tp;
    prof[2] = double(evE.size() / 2);
    prof[3] = double(evP.size() / 2);
    prof[4] = double(c0.steps);
    prof[5] = double(c0.photonSteps);
    prof[6] = nElec + primE;
    prof[7] = nPhot + primP;
    prof[8] = hist;
    prof[9] = fms;
  }
  std::vector<RunCounters> hcnt(njobs);
  std::vector<double> hsum(njobs);
  std::vector<unsigned long long> hlast(njobs);
  CK(cudaMemcpy(hcnt.data(), cnt, njobs * sizeof(RunCounters), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hsum.data(), dsum, njobs * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hlast.data(), dlast, njobs * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  for (int j = 0; j < njobs; ++j) {
    outs[j].cnt = hcnt[j];
    outs[j].cnt.deposited = hsum[j];
    if (outs[j].slab) outs[j].maxIz = hlast[j] > 0 ? int(hlast[j] - 1) : 0;
  }
  if (faults > 0)
    return Fail(DPMX_ERR_CUDA, std::to_string(faults) + " warps of a transport phase gave up a bounded wait; run incomplete");
  lost = leftover + overflowed;
  // losses of the queues are reported on job 0
  if (njobs > 0) outs[0].cnt.lost += lost;
  if (lost > 0)
    return Fail(DPMX_ERR_OVERFLOW, std::to_string(overflowed) + " secondaries dropped on full queues, " +
                                       std::to_string(leftover) + " particles left after " + std::to_string(kGen) +
                                       " generations");
  return DPMX_OK;
}

// ---------------------------------------------------------------------------
// FP64 plain form
// ---------------------------------------------------------------------------
int RunFp64(const dpmx_tables* T, const dpmx_job* jobs, int njobs, int batches, bool fixedSeedSlab, cudaStream_t st,
            std::vector<JobOut>& outs, double* ms, long long* launches, double* histEdep) {
  DevBuf buf(st);
  const int blocks = NumSMs() * 16;
  double* density;
  if (int rc = buf.Get(&density, kMaxMat)) return rc;
  CK(cudaMemcpyAsync(density, T->h.density.data(), T->h.nmat * sizeof(double), cudaMemcpyHostToDevice, st));
  RunCounters* cnt;
  if (int rc = buf.Get(&cnt, njobs)) return rc;
  CK(cudaMemsetAsync(cnt, 0, njobs * sizeof(RunCounters), st));
  int* maxIz;
  if (int rc = buf.Get(&maxIz, njobs)) return rc;
  CK(cudaMemsetAsync(maxIz, 0, njobs * sizeof(int), st));
  long long maxT = 1;
  for (auto& o : outs) maxT = std::max(maxT, o.tallySize);
  double* tB;
  if (int rc = buf.Get(&tB, maxT)) return rc;
  EventSet evs;
  cudaEvent_t e0, e1;
  CK(evs.Add(&e0));
  CK(evs.Add(&e1));
  CK(cudaEventRecord(e0, st));
  long long nl = 0;
  long long histOff = 0;
  for (int j = 0; j < njobs; ++j) {
    const dpmx_phantom* ph = jobs[j].phantom;
    JobOut& o = outs[j];
    CK(cudaMemsetAsync(o.d_dose, 0, o.tallySize * sizeof(double), st));
    CK(cudaMemsetAsync(o.d_dose2, 0, o.tallySize * sizeof(double), st));
    SourceD src{};
    const dpmx_source& s = jobs[j].source;
    src.particle = s.particle; src.spectrum = s.spectrum; src.shape = s.shape; src.nbx = s.nbx; src.nby = s.nby;
    src.e0 = s.e0; src.e1 = s.e1; src.cx = s.cx; src.cy = s.cy; src.fx = s.fx; src.fy = s.fy;
    src.zEntry = ph->grid.z0;
    const long long N = jobs[j].histories;
    for (int b = 0; b < batches; ++b) {
      const long long lo = N * b / batches, hi = N * (b + 1) / batches;
      if (hi <= lo) continue;
      CK(cudaMemsetAsync(tB, 0, o.tallySize * sizeof(double), st));
      double* he = histEdep ? histEdep + histOff + lo : nullptr;
      if (ph->kind == 0) {
        SlabGeomD g{ph->geomIndex, ph->lbox, 1.0 / ph->lbox, 0.5 * ph->lbox};
        CK(LaunchFp64Slab(T->t64, g, density, src, jobs[j].first_history + lo, hi - lo, jobs[j].seed, tB, o.d_steps,
                          int(o.tallySize),
                          maxIz + j, he, cnt + j, blocks, st));
      } else {
        GridGeom g = ph->grid;
        CK(LaunchFp64Grid(T->t64, g, density, src, jobs[j].first_history + lo, hi - lo, jobs[j].seed, tB, he,
                          cnt + j, blocks, st));
      }
      CK(LaunchFold(tB, o.d_dose, o.d_dose2, o.tallySize, st));
      nl += 2;
    }
    histOff += N;
  }
  (void)fixedSeedSlab;
  CK(cudaEventRecord(e1, st));
  CK(cudaStreamSynchronize(st));
  float fms = 0.f;
  CK(cudaEventElapsedTime(&fms, e0, e1));
  *ms = fms;
  *launches = nl;
  std::vector<RunCounters> hcnt(njobs);
  std::vector<int> hmz(njobs);
  CK(cudaMemcpy(hcnt.data(), cnt, njobs * sizeof(RunCounters), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hmz.data(), maxIz, njobs * sizeof(int), cudaMemcpyDeviceToHost));
  for (int j = 0; j < njobs; ++j) {
    outs[j].cnt = hcnt[j];
    outs[j].cnt.histories = (unsigned long long)jobs[j].histories;
    outs[j].maxIz = hmz[j];
  }
  long long lost = 0;
  for (auto& o : outs) lost += (long long)o.cnt.lost;
  if (lost > 0) return Fail(DPMX_ERR_OVERFLOW, "secondary stack overflow or step limit reached");
  return DPMX_OK;
}

int PrepareOutputs(const dpmx_job* jobs, int njobs, bool tag, cudaStream_t st, std::vector<JobOut>& outs) {
  outs.assign(njobs, JobOut());
  for (int j = 0; j < njobs; ++j) {
    const dpmx_phantom* ph = jobs[j].phantom;
    JobOut& o = outs[j];
    o.tallySize = ph->tallySize;
    o.slab = ph->kind == 0;
    o.nvox = (long long)ph->grid.nx * ph->grid.ny * ph->grid.nz;
    o.grid = ph->grid;
    o.lbox = ph->lbox;
    o.binDensity = ph->binDensity;
    o.binMaterial = ph->binMaterial;
    o.matDev = ph->matOwner;
    o.materialDensity = ph->materialDensity;
    // dose and dose^2 come from the scratch pool; every run writes them whole
    void* p = nullptr;
    CK(ScratchPool::Instance().Get(o.tallySize * sizeof(double), &p));
    o.d_dose = static_cast<double*>(p);
    CK(ScratchPool::Instance().Get(o.tallySize * sizeof(double), &p));
    o.d_dose2 = static_cast<double*>(p);
    if (o.slab) {
      CK(ScratchPool::Instance().Get(o.tallySize * sizeof(double), &p));
      o.d_steps = static_cast<double*>(p);
      CK(cudaMemsetAsync(o.d_steps, 0, o.tallySize * sizeof(double), st));
    }
    if (tag && !o.slab) {
      const dpmx_source& s = jobs[j].source;
      o.nbeamlets = (s.shape == 2) ? std::max(1, s.nbx * s.nby) : 1;
      const size_t n = size_t(o.nbeamlets) * size_t(o.nvox);
      CK(ScratchPool::Instance().Get(n * sizeof(double), &p));
      o.d_btally = static_cast<double*>(p);
      CK(cudaMemsetAsync(o.d_btally, 0, n * sizeof(double), st));
    }
  }
  return DPMX_OK;
}

int CheckJobs(const dpmx_tables* t, const dpmx_job* jobs, int njobs) {
  if (!t || !jobs || njobs < 1) return Fail(DPMX_ERR_ARG, "no jobs");
  if (njobs > kMaxJobs) return Fail(DPMX_ERR_ARG, "too many jobs in one run");
  for (int j = 0; j < njobs; ++j) {
    const dpmx_job& J = jobs[j];
    if (!J.phantom || J.phantom->tables != t) return Fail(DPMX_ERR_ARG, "job phantom missing or built on other tables");
    if (J.histories < 0 || J.first_history < 0 || J.first_history + J.histories > (1LL << 32))
      return Fail(DPMX_ERR_ARG, "history indices must lie in [0, 2^32)");
    const dpmx_source& s = J.source;
    if (s.particle != -1 && s.particle != 0) return Fail(DPMX_ERR_ARG, "source particle must be -1 (e-) or 0 (photon)");
    const double emax = t->h.dedx[0].x.back();
    const double emin = s.particle == 0 ? t->h.gcut : t->h.ecut;
    const double hi = s.spectrum == 0 ? s.e0 : std::max(s.e0, s.e1);
    const double lo = s.spectrum == 0 ? s.e0 : std::min(s.e0, s.e1);
    if (!(lo > emin) || !(hi < emax)) return Fail(DPMX_ERR_ARG, "source energies must lie inside the data-set grids");
    if (s.shape == 2 && (s.nbx < 1 || s.nby < 1 || s.nbx * s.nby > 65535))
      return Fail(DPMX_ERR_ARG, "beamlet grid must have 1..65535 beamlets");
    if (s.spectrum < 0 || s.spectrum > 2 || s.shape < 0 || s.shape > 2) return Fail(DPMX_ERR_ARG, "bad source spec");
  }
  return DPMX_OK;
}

Cfg DefaultCfg(const dpmx_run_options* o, long long totalHist) {
  // The block-batched photon phase is the default for every run. It is faster
  // with photon beams and somewhat slower when photons are few (electron
  // beams), but the two photon kernels round some FP32 results differently, so
  // a choice that depended on the job mix would make a batched run differ
  // (slightly) from the same jobs run alone.
  Cfg c;
  if (o && o->block_size > 0) c.threads = std::min(256, std::max(32, o->block_size / 32 * 32));
  if (o && o->blocks_per_sm > 0) c.blocksPerSM = o->blocks_per_sm;
  if (o && o->chunk_histories > 0) c.chunk = o->chunk_histories;
  else {
    // as few chunks as the bound allows, of equal size, and at least two
    // (one per lane) for runs of kLaneMinHistories or more
    const long long n = std::max(1LL, totalHist);
    const long long k = std::max((n + kMaxChunk - 1) / kMaxChunk, n >= kLaneMinHistories ? 2LL : 1LL);
    c.chunk = std::max<long long>(1 << 14, (n + k - 1) / k);
  }
  if (o && o->tally_aggregate >= 0) c.aggregate = o->tally_aggregate;
  if (o && o->electron_kernel >= 0) c.eblock = o->electron_kernel;
  if (o && o->photon_kernel >= 0) c.pblock = o->photon_kernel;
  if (o && o->electron_slots > 0) c.eslots = o->electron_slots;
  c.eslots = BlockPhaseSlots(c.eslots);
  return c;
}

// times a few launch shapes on a sample of the jobs and returns the fastest
int Autotune(const dpmx_tables* t, const dpmx_job* jobs, int njobs, const Cfg base, cudaStream_t st, Cfg* best) {
  long long total = 0;
  for (int j = 0; j < njobs; ++j) total += jobs[j].histories;
  const long long sample = std::min<long long>(total, 1 << 18);
  std::vector<dpmx_job> sj(jobs, jobs + njobs);
  for (auto& j : sj) j.histories = std::max<long long>(1, (long long)(double(j.histories) * sample / std::max(1LL, total)));
  // threads and blocks per SM of the lane kernels, tally aggregation, the
  // electron kernel and the block kernel's slots per block (its queue
  // depth); the photon kernel stays the run's (the two photon kernels round
  // some FP32 results differently)
  struct Cand { int threads, bps, agg, eblock, pblock, eslots; };
  // (threads and blocks per SM shape the lane kernels, compiled for at most
  // 256 threads per block; the block-batched kernels have fixed block shapes)
  const int sDef = BlockPhaseSlots(0), sSmall = 384;
  const Cand cands[] = {{256, 3, 0, 0, -1, sDef},   {256, 3, 1, 0, -1, sDef},   {256, 2, 0, 0, -1, sDef},
                        {128, 6, 0, 0, -1, sDef},   {256, 3, 0, 1, -1, sDef},   {256, 3, 1, 1, -1, sDef},
                        {256, 3, 0, 1, -1, sSmall}, {256, 3, 1, 1, -1, sSmall}};
  double bestMs = 1e30;
  *best = base;
  for (const Cand& c : cands) {
    Cfg cfg = base;
    cfg.threads = c.threads;
    cfg.blocksPerSM = c.bps;
    cfg.aggregate = c.agg;
    cfg.eblock = c.eblock;
    cfg.eslots = BlockPhaseSlots(c.eslots);
    if (c.pblock >= 0) cfg.pblock = c.pblock;
    cfg.chunk = sample;
    std::vector<JobOut> outs;
    if (int rc = PrepareOutputs(sj.data(), njobs, false, st, outs)) return rc;
    double ms = 0;
    long long nl = 0;
    const int rc = RunFp32(t, sj.data(), njobs, 1, cfg, false, false, st, outs, &ms, &nl);
    for (auto& o : outs) ReleaseJobOut(o);
    if (rc) return rc;
    if (ms < bestMs) { bestMs = ms; *best = cfg; }
  }
  best->chunk = base.chunk;
  return DPMX_OK;
}

}  // namespace

namespace dpmx {
void ReleaseJobOut(JobOut& o) {
  // every run synchronises its stream before it returns, so no library work
  // still uses these blocks: they go back to the pool without a device-wide wait
  for (double* p : {o.d_dose, o.d_dose2, o.d_steps, o.d_btally})
    if (p) ScratchPool::Instance().Put(p);
  o.d_dose = o.d_dose2 = o.d_steps = o.d_btally = nullptr;
}
cudaError_t ScratchGet(size_t bytes, void** out) { return ScratchPool::Instance().Get(bytes, out); }
void ScratchPut(void* p) {
  if (p) ScratchPool::Instance().Put(p);
}
}  // namespace dpmx

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int dpmx_run(const dpmx_tables* t, const dpmx_job* jobs, int njobs, const dpmx_run_options* opt, dpmx_result** out) {
  if (!out) return Fail(DPMX_ERR_ARG, "null result pointer");
  *out = nullptr;
  if (int rc = CheckJobs(t, jobs, njobs)) return rc;
  dpmx_run_options o;
  if (opt) o = *opt; else dpmx_run_options_default(&o);
  if (o.batches < 1) o.batches = 1;
  if (o.batches > 65536) return Fail(DPMX_ERR_ARG, "at most 65536 statistical batches");
  if (o.precision != DPMX_FP64_PLAIN && o.precision != DPMX_FP32_EVENT) return Fail(DPMX_ERR_ARG, "bad precision");
  cudaStream_t st = static_cast<cudaStream_t>(o.stream);
  bool ownStream = false;
  if (!st) { CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)); ownStream = true; }
  std::unique_ptr<dpmx_result> r(new dpmx_result());
  r->batches = o.batches;
  const bool tag = o.tag_beamlets && o.precision == DPMX_FP32_EVENT;
  int rc = PrepareOutputs(jobs, njobs, tag, st, r->jobs);
  if (!rc) {
    if (o.precision == DPMX_FP64_PLAIN) {
      rc = RunFp64(t, jobs, njobs, o.batches, true, st, r->jobs, &r->ms, &r->launches, nullptr);
      r->cfg[0] = 128; r->cfg[1] = 16; r->cfg[2] = 0; r->cfg[3] = 0;
    } else {
      long long total = 0;
      for (int j = 0; j < njobs; ++j) total += jobs[j].histories;
      Cfg cfg = DefaultCfg(&o, total);
      if (o.autotune) rc = Autotune(t, jobs, njobs, cfg, st, &cfg);
      if (!rc)
        rc = RunFp32(t, jobs, njobs, o.batches, cfg, tag, o.use_graph != 0 && !o.profile_phases, st, r->jobs, &r->ms,
                     &r->launches, o.profile_phases ? r->prof : nullptr);
      r->cfg[0] = cfg.threads; r->cfg[1] = cfg.blocksPerSM; r->cfg[2] = cfg.chunk;
      r->cfg[3] = cfg.aggregate | (cfg.eblock << 1) | (cfg.pblock << 2) | ((long long)cfg.eslots << 3);
    }
  }
  if (ownStream) cudaStreamDestroy(st);
  if (rc && rc != DPMX_ERR_OVERFLOW) return rc;
  *out = r.release();
  return rc;
}

int dpmx_result_tally(const dpmx_result* r, int job, double* dose, double* dose2, double* steps) {
  if (!r || job < 0 || job >= int(r->jobs.size())) return Fail(DPMX_ERR_ARG, "bad job index");
  const JobOut& o = r->jobs[job];
  const size_t n = size_t(o.tallySize) * sizeof(double);
  // on a stream of this call (no wait on other streams); into pinned memory
  // the copies run at the host link's rate (GB300: ~190 GB/s device to host,
  // the same for one or two streams and for a kernel storing to mapped memory)
  StreamGuard s0;
  CK(s0.Create());
  if (dose) CK(cudaMemcpyAsync(dose, o.d_dose, n, cudaMemcpyDeviceToHost, s0.st));
  if (dose2) CK(cudaMemcpyAsync(dose2, o.d_dose2, n, cudaMemcpyDeviceToHost, s0.st));
  if (steps) {
    if (o.d_steps) CK(cudaMemcpyAsync(steps, o.d_steps, n, cudaMemcpyDeviceToHost, s0.st));
    else std::memset(steps, 0, n);
  }
  CK(cudaStreamSynchronize(s0.st));
  return DPMX_OK;
}

const double* dpmx_result_tally_device(const dpmx_result* r, int job) {
  if (!r || job < 0 || job >= int(r->jobs.size())) return nullptr;
  return r->jobs[job].d_dose;
}

int dpmx_result_stats(const dpmx_result* r, int job, dpmx_job_stats* s) {
  if (!r || !s || job < 0 || job >= int(r->jobs.size())) return Fail(DPMX_ERR_ARG, "bad job index");
  const RunCounters& c = r->jobs[job].cnt;
  s->edep = c.deposited;
  s->escaped = c.escaped;
  s->primary_energy = c.primaryEnergy;
  double mr;
  std::memcpy(&mr, &c.maxResidualBits, sizeof(double));
  s->max_residual = mr;
  s->residual_violations = (long long)c.violations;
  s->lost = (long long)c.lost;
  s->steps = (long long)c.steps;
  s->histories = (long long)c.histories;
  return DPMX_OK;
}

double dpmx_result_elapsed_ms(const dpmx_result* r) { return r ? r->ms : 0.0; }
long long dpmx_result_launches(const dpmx_result* r) { return r ? r->launches : 0; }
int dpmx_result_config(const dpmx_result* r, long long* cfg4) {
  if (!r || !cfg4) return Fail(DPMX_ERR_ARG, "null argument");
  for (int i = 0; i < 4; ++i) cfg4[i] = r->cfg[i];
  return DPMX_OK;
}
int dpmx_result_profile(const dpmx_result* r, double* out10) {
  if (!r || !out10) return Fail(DPMX_ERR_ARG, "null argument");
  for (int i = 0; i < 10; ++i) out10[i] = r->prof[i];
  return DPMX_OK;
}

void dpmx_result_free(dpmx_result* r) { delete r; }

void dpmx_scratch_release(void) { ScratchPool::Instance().Release(-1); }

int dpmx_result_write(const dpmx_result* r, int job, const char* path, int format) {
  if (!r || !path || job < 0 || job >= int(r->jobs.size())) return Fail(DPMX_ERR_ARG, "bad result, job or path");
  if (format != DPMX_DOSE_RAW && format != DPMX_DOSE_DEPTH) return Fail(DPMX_ERR_ARG, "unknown dose format");
  JobOut o = r->jobs[job];
  if (format == DPMX_DOSE_RAW && o.slab) return Fail(DPMX_ERR_ARG, "raw 3-D output needs a voxel phantom");
  if (!o.binDensity && !o.binMaterial) {
    // the material ids of a voxel phantom are kept on the device only
    if (!o.matDev) return Fail(DPMX_ERR_ARG, "the job's phantom has no material ids");
    auto ids = std::make_shared<std::vector<uint8_t>>(size_t(o.tallySize));
    CK(cudaMemcpy(ids->data(), o.matDev.get(), ids->size(), cudaMemcpyDeviceToHost));
    o.binMaterial = ids;
  }
  const long long n = o.tallySize;
  std::vector<double> d(n), d2(n), st;
  CK(cudaMemcpy(d.data(), o.d_dose, n * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(d2.data(), o.d_dose2, n * sizeof(double), cudaMemcpyDeviceToHost));
  if (o.slab && o.d_steps) {
    st.resize(n);
    CK(cudaMemcpy(st.data(), o.d_steps, n * sizeof(double), cudaMemcpyDeviceToHost));
  }
  const double hist = double(o.cnt.histories);
  if (!(hist > 0)) return Fail(DPMX_ERR_ARG, "the job ran no histories");
  FILE* f = std::fopen(path, format == DPMX_DOSE_RAW ? "wb" : "w");
  if (!f) return Fail(DPMX_ERR_FILE, std::string("file ") + path + " could not be created");
  bool ok = true;
  if (format == DPMX_DOSE_RAW) {
    // header, then dose [Gy per history] and its relative 1-sigma uncertainty
    // (from the statistical batches) per voxel, x fastest
    const GridGeom& g = o.grid;
    const char magic[8] = {'D', 'P', 'M', 'X', 'D', 'O', 'S', 'E'};
    const int32_t head[4] = {1, g.nx, g.ny, g.nz};
    const double geo[6] = {g.vx, g.vy, g.vz, g.x0, g.y0, g.z0};
    const int64_t hb[2] = {int64_t(o.cnt.histories), int64_t(r->batches)};
    ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(head, 4, 4, f) == 4 && std::fwrite(geo, 8, 6, f) == 6 &&
         std::fwrite(hb, 8, 2, f) == 2;
    const double mevToJ = 1.602176634e-13, volCm3 = g.vx * g.vy * g.vz * 1.0e-3;
    const int B = r->batches;
    std::vector<double> dose(n), rel(n);
    for (long long i = 0; i < n; ++i) {
      const double massKg = double(o.BinDensity(i)) * volCm3 * 1.0e-3;
      dose[i] = massKg > 0.0 ? d[i] * mevToJ / massKg / hist : 0.0;
      // batch sums t_b: sum_b t_b = d, sum_b t_b^2 = d2; error of the mean of B batches
      const double var = B > 1 ? std::max(0.0, (d2[i] - d[i] * d[i] / B) / (B - 1)) * B : 0.0;
      rel[i] = d[i] > 0.0 ? std::sqrt(var) / d[i] : 0.0;
    }
    ok = ok && std::fwrite(dose.data(), 8, n, f) == size_t(n) && std::fwrite(rel.data(), 8, n, f) == size_t(n);
  } else {
    // Geom::Write's columns (Geom.cc:167-192) for any phantom: the energy of a
    // depth slice per primary over the slice's mean density times its
    // thickness [MeV cm2/g], and the scoring steps per primary (slab presets)
    const GridGeom& g = o.grid;
    const int nz = o.slab ? int(n) : g.nz;
    const double dz = o.slab ? o.lbox : g.vz;
    std::vector<double> ez(nz, 0.0), rz(nz, 0.0), sz(nz, 0.0);
    if (o.slab) {
      for (int i = 0; i < nz; ++i) { ez[i] = d[i]; rz[i] = o.BinDensity(i); sz[i] = st.empty() ? 0.0 : st[i]; }
    } else {
      const long long plane = (long long)g.nx * g.ny;
      for (int iz = 0; iz < nz; ++iz) {
        double e = 0.0, r0 = 0.0;
        for (long long k = 0; k < plane; ++k) { e += d[iz * plane + k]; r0 += o.BinDensity(iz * plane + k); }
        ez[iz] = e;
        rz[iz] = r0 / double(plane);
      }
    }
    int len = nz;
    if (o.slab) len = std::min(nz, HistLen(o.maxIz));
    double sum = 0.0;
    for (int i = 0; i < nz; ++i) sum += ez[i];
    std::fprintf(f, "# === Mean energy deposit in the target: %13.4e  [MeV/event]\n", sum / hist);
    std::fprintf(f, "# === Energy deposit as a function of the depth: \n");
    std::fprintf(f, "# === Index       Depth [cm]    Edep [MeV cm2/g]  #Simulation-Steps \n");
    const double norm = 1.0 / (hist * dz * 0.1);
    for (int i = 0; i < len; ++i)
      std::fprintf(f, " %10d    %13.4e    %13.4e    %13.4e\n", i, (i + 0.5) * dz * 0.1,
                   rz[i] > 0.0 ? ez[i] * norm / rz[i] : 0.0, sz[i] / hist);
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? DPMX_OK : Fail(DPMX_ERR_FILE, std::string("writing ") + path + " failed");
}

int dpmx_simulate(const dpmx_tables* t, int nprimary, double eprimary, int iselectron, double lbox, int geom_index,
                  uint64_t seed, int precision, double* edep_hist, double* step_hist, int cap, int* hist_len) {
  if (!t || nprimary < 0 || !(lbox > 0.0)) return Fail(DPMX_ERR_ARG, "bad simulate arguments");
  dpmx_phantom* ph = nullptr;
  if (int rc = dpmx_phantom_slab(t, geom_index, lbox, &ph)) return rc;
  dpmx_job job;
  std::memset(&job, 0, sizeof(job));
  job.phantom = ph;
  job.source.particle = iselectron ? -1 : 0;
  job.source.e0 = job.source.e1 = eprimary;
  job.histories = nprimary;
  job.seed = seed;
  dpmx_run_options o;
  dpmx_run_options_default(&o);
  o.precision = precision;
  o.batches = 1;
  dpmx_result* r = nullptr;
  int rc = dpmx_run(t, &job, 1, &o, &r);
  if (r) {
    const JobOut& jo = r->jobs[0];
    std::vector<double> d(jo.tallySize), s(jo.tallySize);
    int rc2 = dpmx_result_tally(r, 0, d.data(), nullptr, s.data());
    if (!rc && rc2) rc = rc2;
    const int n = std::min<int>(cap, int(jo.tallySize));
    for (int i = 0; i < n; ++i) {
      if (edep_hist) edep_hist[i] = d[i];
      if (step_hist) step_hist[i] = s[i];
    }
    int mz = 0;
    for (int i = 0; i < int(d.size()); ++i) if (d[i] != 0.0 || s[i] != 0.0) mz = i;
    if (hist_len) *hist_len = HistLen(mz);
    dpmx_result_free(r);
  }
  dpmx_phantom_free(ph);
  return rc;
}

int dpmx_write_hist(const dpmx_tables* t, const char* fname, int geom_index, double lbox, int nprimary,
                    const double* edep, const double* steps, int len) {
  // Geom::Write (Geom.cc:167-192)
  if (!t || !fname || !edep || !steps || nprimary <= 0 || len < 0) return Fail(DPMX_ERR_ARG, "bad write arguments");
  FILE* f = std::fopen(fname, "w");
  if (!f) return Fail(DPMX_ERR_FILE, std::string("file ") + fname + " could not be created");
  const double toCm = 0.1;
  const double norm = 1. / (nprimary * lbox * toCm);
  double sum = 0.0;
  for (int i = 0; i < len; ++i) sum += edep[i];
  std::fprintf(f, "# === Mean energy deposit in the target: %13.4e  [MeV/event]\n", sum / nprimary);
  std::fprintf(f, "# === Energy deposit as a function of the depth: \n");
  std::fprintf(f, "# === Index       Depth [cm]    Edep [MeV cm2/g]  #Simulation-Steps \n");
  const double invL = 1.0 / lbox;
  for (int i = 0; i < len; ++i) {
    const double rho = SlabDensityAt(t, geom_index, invL, i);
    std::fprintf(f, " %10d    %13.4e    %13.4e    %13.4e\n", i, (i + 0.5) * lbox * toCm, edep[i] * norm / rho,
                 steps[i] / nprimary);
  }
  std::fclose(f);
  return DPMX_OK;
}

int dpmx_sampler_eval(const dpmx_tables* t, int precision, int sampler, int imat, const double* e, const double* r,
                      double* out, int n) {
  if (!t || !e || !r || !out || n < 0 || sampler < 0 || sampler > 3) return Fail(DPMX_ERR_ARG, "bad sampler arguments");
  if (imat < 0 || imat >= t->h.nmat) return Fail(DPMX_ERR_ARG, "bad material index");
  if (n == 0) return DPMX_OK;
  DevBuf b(nullptr);
  double *de, *dr, *dout;
  if (int rc = b.Get(&de, n)) return rc;
  if (int rc = b.Get(&dr, 3 * size_t(n))) return rc;
  if (int rc = b.Get(&dout, n)) return rc;
  CK(cudaMemcpy(de, e, n * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dr, r, 3 * size_t(n) * sizeof(double), cudaMemcpyHostToDevice));
  if (precision == DPMX_FP64_PLAIN) CK(LaunchSamplerEval64(t->t64, sampler, imat, de, dr, dout, n, 0));
  else CK(LaunchSamplerEval32(t->t32, sampler, imat, de, dr, dout, n, 0));
  CK(cudaMemcpy(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost));
  return DPMX_OK;
}

int dpmx_table_eval(const dpmx_tables* t, int precision, int q, int imat, const double* e, double* out, int n) {
  if (!t || !e || !out || n < 0 || q < 0 || q > 8) return Fail(DPMX_ERR_ARG, "bad table arguments");
  if (imat < 0 || imat >= t->h.nmat) return Fail(DPMX_ERR_ARG, "bad material index");
  if (n == 0) return DPMX_OK;
  DevBuf b(nullptr);
  double *de, *dout;
  if (int rc = b.Get(&de, n)) return rc;
  if (int rc = b.Get(&dout, n)) return rc;
  CK(cudaMemcpy(de, e, n * sizeof(double), cudaMemcpyHostToDevice));
  if (precision == DPMX_FP64_PLAIN) CK(LaunchTableEval64(t->t64, q, imat, de, dout, n, 0));
  else CK(LaunchTableEval32(t->t32, q, imat, de, dout, n, 0));
  CK(cudaMemcpy(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost));
  return DPMX_OK;
}

// test hook: the FP64 slab workload with per-history deposited energies
int dpmx_simulate_histories(const dpmx_tables* t, int nprimary, double eprimary, int iselectron, double lbox,
                            int geom_index, uint64_t seed, double* hist_edep, double* edep_hist, int cap) {
  if (!t || nprimary < 0 || !hist_edep) return Fail(DPMX_ERR_ARG, "bad arguments");
  dpmx_phantom* ph = nullptr;
  if (int rc = dpmx_phantom_slab(t, geom_index, lbox, &ph)) return rc;
  dpmx_job job;
  std::memset(&job, 0, sizeof(job));
  job.phantom = ph;
  job.source.particle = iselectron ? -1 : 0;
  job.source.e0 = job.source.e1 = eprimary;
  job.histories = nprimary;
  job.seed = seed;
  std::vector<JobOut> outs;
  int rc = PrepareOutputs(&job, 1, false, 0, outs);
  double* d_he = nullptr;
  if (!rc && cudaMalloc(&d_he, std::max(1, nprimary) * sizeof(double)) != cudaSuccess) rc = Fail(DPMX_ERR_NOMEM, "alloc");
  double ms = 0;
  long long nl = 0;
  if (!rc) rc = RunFp64(t, &job, 1, 1, true, 0, outs, &ms, &nl, d_he);
  if (!rc || rc == DPMX_ERR_OVERFLOW) {
    cudaMemcpy(hist_edep, d_he, nprimary * sizeof(double), cudaMemcpyDeviceToHost);
    if (edep_hist) {
      std::vector<double> d(outs[0].tallySize);
      cudaMemcpy(d.data(), outs[0].d_dose, d.size() * sizeof(double), cudaMemcpyDeviceToHost);
      for (int i = 0; i < std::min<int>(cap, int(d.size())); ++i) edep_hist[i] = d[i];
    }
  }
  cudaFree(d_he);
  for (auto& o : outs) ReleaseJobOut(o);
  dpmx_phantom_free(ph);
  return rc;
}

// test hook: one job of any phantom in the FP64 form, with each history's
// deposited energy
int dpmx_job_histories(const dpmx_tables* t, const dpmx_job* job, double* hist_edep, double* dose) {
  if (!t || !job || !hist_edep) return Fail(DPMX_ERR_ARG, "bad arguments");
  if (int rc = CheckJobs(t, job, 1)) return rc;
  if (job->histories > (1LL << 26)) return Fail(DPMX_ERR_ARG, "at most 2^26 histories per call");
  std::vector<JobOut> outs;
  int rc = PrepareOutputs(job, 1, false, 0, outs);
  double* d_he = nullptr;
  const long long n = job->histories;
  if (!rc && cudaMalloc(&d_he, std::max(1LL, n) * sizeof(double)) != cudaSuccess) rc = Fail(DPMX_ERR_NOMEM, "alloc");
  double ms = 0;
  long long nl = 0;
  if (!rc) rc = RunFp64(t, job, 1, 1, true, 0, outs, &ms, &nl, d_he);
  if (!rc || rc == DPMX_ERR_OVERFLOW) {
    if (cudaMemcpy(hist_edep, d_he, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess && !rc)
      rc = Fail(DPMX_ERR_CUDA, "copy of the per-history energies failed");
    if (dose && cudaMemcpy(dose, outs[0].d_dose, outs[0].tallySize * sizeof(double), cudaMemcpyDeviceToHost) !=
                    cudaSuccess && !rc)
      rc = Fail(DPMX_ERR_CUDA, "copy of the dose failed");
  }
  cudaFree(d_he);
  for (auto& o : outs) ReleaseJobOut(o);
  return rc;
}

}  // extern "C"
