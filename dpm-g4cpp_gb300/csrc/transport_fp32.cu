// Event-based FP32 transport with FP64 tallies.
//
// Particles of one generation live in SoA queues in HBM. A generation is
// transported in two phases: all photons (Woodcock tracking), then all
// electrons/positrons (condensed-history stepping). Each phase is one
// persistent launch, in one of two forms:
//  * block-batched (the default): a block keeps a few hundred particles in
//    shared memory, each waiting on a ring (a shared-memory queue) by what it
//    does next; a warp takes up to 32 particles of one ring whenever it is
//    free, runs that interaction (or refills them from the phase's work
//    counter) and one step, and puts each on the ring of its next action, so
//    a warp runs one kind of interaction at a time and no warp waits for
//    another (ElectronPhaseB, PhotonPhaseB);
//  * one particle per lane, refilled from the work counter when it ends
//    (ElectronPhase, PhotonPhase).
// Secondaries are appended to the next generation's queues with
// warp-aggregated atomics on striped counters.
//
// Geometry is tracked as an integer voxel index plus an FP32 offset inside the
// voxel, which keeps the 1e-4 mm boundary tolerance of the reference
// (Geom.hh:107) meaningful at any phantom size. Electron spline tables are read
// through L1 (or staged in shared memory); photon and sampling tables are read
// in place. Energy deposits are tallied in FP64 (optionally warp-aggregated on
// equal voxels; slab depth tallies per block in shared memory first), and every
// particle's deposited plus escaped energy is added to its history's FP64 slot
// once, at the end of the particle, for the per-history energy check.
//
// The physics of each step and interaction is the reference's
// (SimDPMLike.cc:254-791) evaluated in FP32; the order in which particles of a
// history are processed differs from the reference's LIFO stack, so results
// agree with it statistically.
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "device_common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace dpmx {
namespace {

constexpr float kEMC2f = 0.510991f;
constexpr float kPIf = 3.1415926535897932f;
constexpr float kHalfTolF = 0.5e-4f;
constexpr unsigned kFull = 0xffffffffu;
constexpr unsigned kMaxPhotonSteps = 1u << 22;     // per particle: a lane never loops without bound
// A particle's sub-job (meta >> 2) is its job (low 8 bits) and the statistical
// batch slice of the job's tally it scores into (the bits above).
__device__ __forceinline__ int JobOfSub(uint32_t sub) { return int(sub & 0xffu); }
__device__ __forceinline__ uint32_t SliceOfSub(uint32_t sub) { return sub >> 8; }
constexpr unsigned kMaxElectronSteps = 1u << 24;

// ---------------------------------------------------------------------------
// per-particle random numbers: Philox key = job seed, counter =
// {block, uid_lo, uid_hi, history}; 4 uniforms per block (UniformF32: one word
// each, on the open interval (0,1))
// ---------------------------------------------------------------------------
struct PRng {
  uint32_t k0, k1, ctr, ulo, uhi, hist;
  uint4 w;
  int have;
  __device__ __forceinline__ void Init(uint32_t a, uint32_t b, uint32_t h, uint32_t lo, uint32_t hi) {
    k0 = a; k1 = b; hist = h; ulo = lo; uhi = hi; ctr = 0; have = 0;
  }
  __device__ __forceinline__ float U() {
    if (have == 0) {
      w = philox(make_uint4(ctr++, ulo, uhi, hist), k0, k1);
      have = 4;
    }
    const uint32_t x = w.x;
    w.x = w.y; w.y = w.z; w.z = w.w;
    --have;
    return UniformF32(x);
  }
  // stream id of the k-th secondary created at the current stream position
  __device__ __forceinline__ void Child(int k, uint32_t& lo, uint32_t& hi) const {
    uint64_t z = ((uint64_t(uhi) << 32) | ulo) +
                 0x9E3779B97F4A7C15ull * (uint64_t(ctr) * 8u + uint64_t(4 - have) * 2u + uint64_t(k) + 1u);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    lo = uint32_t(z);
    hi = uint32_t(z >> 32);
  }
};

// photon linear tables, staged in shared memory or read in place
constexpr bool kPhotonTablesInSmem = false;   // no measured gain: the photon phase waits on the phantom
struct PTables {
  LinearT<float> imfpMax, tot[kMaxMat], comp[kMaxMat], pair[kMaxMat];
};

// shared-memory copies of the electron spline tables
struct ETables {
  SplineT<float> dedx[kMaxMat], itr1[kMaxMat], brem[kMaxMat], k1, moller;
  SplinePairT<float> di[kMaxMat];   // dE/dx and 1/lambda_1 in one record per bin (read in place)
  // nominal density and Moller scaling of each material: shared memory serves
  // lanes in different materials in one access, the kernel parameters would
  // serialise them
  float density[kMaxMat], mollerScale[kMaxMat];
};

__device__ __forceinline__ SplineT<float> Rebase(const SplineT<float>& s, const float* gbase, float* sbase) {
  SplineT<float> r = s;
  r.p = sbase + (s.p - gbase);
  return r;
}

// stage the electron tables of T into shared memory (whole block)
__device__ void StageElectronTables(const DevTables<float>& T, float* sdata, ETables* et) {
  for (int i = threadIdx.x; i < T.elecCount; i += blockDim.x) sdata[i] = T.elecBase[i];
  if (threadIdx.x == 0) {
    for (int m = 0; m < T.nmat; ++m) {
      et->dedx[m] = Rebase(T.dedx[m], T.elecBase, sdata);
      et->itr1[m] = Rebase(T.itr1[m], T.elecBase, sdata);
      et->brem[m] = Rebase(T.brem[m], T.elecBase, sdata);
      et->di[m] = T.di[m];   // read in place
      et->density[m] = T.density[m];
      et->mollerScale[m] = T.mollerScale[m];
    }
    et->k1 = Rebase(T.k1, T.elecBase, sdata);
    et->moller = Rebase(T.moller, T.elecBase, sdata);
  }
  __syncthreads();
}

__device__ __forceinline__ LinearT<float> RebaseL(const LinearT<float>& s, const float* gbase, float* sbase) {
  LinearT<float> r = s;
  r.p = sbase + (s.p - gbase);
  return r;
}

// the photon tables of T into shared memory at sdata (whole block; no barrier:
// the caller's next barrier publishes them), or their global addresses
__device__ void StagePhotonTables(const DevTables<float>& T, bool stage, float* sdata, PTables* pt) {
  if (stage)
    for (int i = threadIdx.x; i < T.photCount; i += blockDim.x) sdata[i] = T.photBase[i];
  if (threadIdx.x == 0) {
    pt->imfpMax = stage ? RebaseL(T.imfpMax, T.photBase, sdata) : T.imfpMax;
    for (int m = 0; m < T.nmat; ++m) {
      pt->tot[m] = stage ? RebaseL(T.tot[m], T.photBase, sdata) : T.tot[m];
      pt->comp[m] = stage ? RebaseL(T.comp[m], T.photBase, sdata) : T.comp[m];
      pt->pair[m] = stage ? RebaseL(T.pair[m], T.photBase, sdata) : T.pair[m];
    }
  }
}

// bytes of dynamic shared memory the photon phase stages its tables in
__host__ __device__ inline size_t PhotonTableBytes(const DevTables<float>& T) {
  return kPhotonTablesInSmem ? ((size_t(T.photCount) * sizeof(float) + 15) & ~size_t(15)) : 0;
}

// the same tables read in place (global memory, cached in L1); one thread
__device__ void BindElectronTables(const DevTables<float>& T, ETables* et) {
  for (int m = 0; m < T.nmat; ++m) {
    et->dedx[m] = T.dedx[m];
    et->itr1[m] = T.itr1[m];
    et->brem[m] = T.brem[m];
    et->di[m] = T.di[m];
  }
  et->k1 = T.k1;
  et->moller = T.moller;
  for (int m = 0; m < T.nmat; ++m) {
    et->density[m] = T.density[m];
    et->mollerScale[m] = T.mollerScale[m];
  }
}

// spline value at e whose log (of the unclamped value) is le
__device__ __forceinline__ float SplineLe(const SplineT<float>& s, float e, float le) {
  const float ec = fminf(s.emaxm, fmaxf(s.emin, e));
  const float lc = (ec == e) ? le : __logf(ec);
  int il = int((lc - s.logMin) * s.invLogDelta);
  il = il < 0 ? 0 : (il > s.n - 2 ? s.n - 2 : il);
  const float4 q = reinterpret_cast<const float4*>(s.p)[il];   // y, b, c, d
  const float xv = ec - s.p[4 * s.n + il];
  return fmaxf(1.0E-20f, q.x + xv * (q.y + xv * (q.z + xv * q.w)));
}

// dE/dx and 1/lambda_1 at e (log le) from one 32-byte record: the same
// arithmetic as SplineLe on each, one index computation and one grid point
struct DedxItr1 {
  float dedx, itr1;
};
__device__ __forceinline__ DedxItr1 SplinePairLe(const SplinePairT<float>& s, float e, float le) {
  const float ec = fminf(s.emaxm, fmaxf(s.emin, e));
  const float lc = (ec == e) ? le : __logf(ec);
  int il = int((lc - s.logMin) * s.invLogDelta);
  il = il < 0 ? 0 : (il > s.n - 2 ? s.n - 2 : il);
  const float4* r = reinterpret_cast<const float4*>(s.p) + 2 * il;
  const float4 q = r[0], t = r[1];
  const float xv = ec - s.p[8 * s.n + il];
  DedxItr1 o;
  o.dedx = fmaxf(1.0E-20f, q.x + xv * (q.y + xv * (q.z + xv * q.w)));
  o.itr1 = fmaxf(1.0E-20f, t.x + xv * (t.y + xv * (t.z + xv * t.w)));
  return o;
}

// ---------------------------------------------------------------------------
// queues
// ---------------------------------------------------------------------------
struct PState {           // a particle as stored in a queue
  int ix, iy, iz;
  float lx, ly, lz, dx, dy, dz, e;
  uint32_t hist, slot, ulo, uhi, meta;   // meta: type (2 bits: 0 photon, 1 e-, 2 e+) | job << 2
};

__device__ __forceinline__ uint32_t PackVox(int ix, int iy, int iz) {
  return uint32_t(ix) | (uint32_t(iy) << 11) | (uint32_t(iz) << 22);
}

// queue entry of the item-th particle of a striped queue (prefix: kStripes+1
// running counts of the stripes)
__device__ __forceinline__ unsigned long long StripedIndex(const Queue& q, const unsigned long long* prefix,
                                                           unsigned long long item) {
  int s = 0;
#pragma unroll
  for (int k = 1; k < kStripes; ++k) s += (item >= prefix[k]) ? 1 : 0;
  return (unsigned long long)s * q.stripeCap + (item - prefix[s]);
}

// queue records are written once and read once, a generation's worth at a
// time (hundreds of MB): loads and stores carry the streaming (evict-first)
// hint, so that they do not push the phantom, tables and tallies out of L2
__device__ __forceinline__ void LoadParticle(const Queue& q, unsigned long long i, PState& p) {
  const uint32_t v = __ldcs(q.vox + i);
  p.ix = int(v & 0x7ffu); p.iy = int((v >> 11) & 0x7ffu); p.iz = int(v >> 22);
  p.lx = __ldcs(q.lx + i); p.ly = __ldcs(q.ly + i); p.lz = __ldcs(q.lz + i);
  p.dx = __ldcs(q.dx + i); p.dy = __ldcs(q.dy + i); p.dz = __ldcs(q.dz + i);
  p.e = __ldcs(q.e + i);
  p.hist = __ldcs(q.hist + i); p.slot = __ldcs(q.slot + i); p.ulo = __ldcs(q.uidlo + i); p.uhi = __ldcs(q.uidhi + i);
  p.meta = __ldcs(q.meta + i);
}

// appends p to q with one atomic per group of converged lanes; returns false
// (and counts the overflow) when the queue is full
__device__ __forceinline__ bool Append(const Queue& q, unsigned long long* count, unsigned long long* overflow,
                                       const PState& p) {
  cg::coalesced_group g = cg::coalesced_threads();
  // blocks and warps spread over all stripes (7 is coprime with kStripes, so
  // the first warp of consecutive blocks, which does most block-stage appends,
  // still cycles through every stripe)
  const int stripe = int((blockIdx.x * 7u + (threadIdx.x >> 5)) & (kStripes - 1));
  unsigned long long base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(count + stripe, (unsigned long long)g.size());
  base = g.shfl(base, 0);
  const unsigned long long j = base + g.thread_rank();
  if (j >= q.stripeCap) {
    atomicAdd(overflow, 1ull);
    return false;
  }
  const unsigned long long i = (unsigned long long)stripe * q.stripeCap + j;
  __stcs(q.vox + i, PackVox(p.ix, p.iy, p.iz));
  __stcs(q.lx + i, p.lx); __stcs(q.ly + i, p.ly); __stcs(q.lz + i, p.lz);
  __stcs(q.dx + i, p.dx); __stcs(q.dy + i, p.dy); __stcs(q.dz + i, p.dz);
  __stcs(q.e + i, p.e);
  __stcs(q.hist + i, p.hist); __stcs(q.slot + i, p.slot); __stcs(q.uidlo + i, p.ulo); __stcs(q.uidhi + i, p.uhi);
  __stcs(q.meta + i, p.meta);
  return true;
}

// ---------------------------------------------------------------------------
// tallies
// ---------------------------------------------------------------------------
// a block's shared-memory depth tally (energy and scoring steps per bin), or none
struct DepthAcc {
  double* e = nullptr;
  unsigned* n = nullptr;
  int sliceStride = 0;   // bins between the batch slices of a job
};

// adds de to bin idx of batch slice `slice` of the job's tally. Bins and
// slices of a run stay below 2^32 doubles (checked when the run is planned):
// 32-bit index arithmetic, one widening for the address
__device__ __forceinline__ void ScoreBin(const JobF& J, uint32_t slice, uint32_t idx, double de, int agg) {
  double* ptr = J.tally + (slice * uint32_t(J.sstride) + idx * uint32_t(J.tstride));
  if (agg) {
    cg::coalesced_group g = cg::coalesced_threads();
    cg::coalesced_group peers = cg::labeled_partition(g, (unsigned long long)ptr);
    const double sum = cg::reduce(peers, de, cg::plus<double>());
    if (peers.thread_rank() == 0) atomicAdd(ptr, sum);
  } else {
    atomicAdd(ptr, de);
  }
}

// deposit e of a particle (meta: its type and sub-job) in voxel (ix, iy, iz)
__device__ __forceinline__ void Score(const JobF& J, uint32_t meta, int ix, int iy, int iz, uint32_t hist, float e,
                                      int agg, const DepthAcc& d = DepthAcc()) {
  const double de = double(e);
  const uint32_t slice = SliceOfSub(meta >> 2);
  if (d.e != nullptr && J.dbase >= 0) {   // depth tally of a slab job: block-local first
    const int b = J.dbase + int(slice) * d.sliceStride + iz;
    atomicAdd(d.e + b, de);
    atomicAdd(d.n + b, 1u);
    return;
  }
  const uint32_t idx = J.tallyDepth ? uint32_t(iz) : (uint32_t(iz) * uint32_t(J.ny) + uint32_t(iy)) * uint32_t(J.nx) + uint32_t(ix);
  ScoreBin(J, slice, idx, de, agg);
  if (J.steps) atomicAdd(J.steps + iz, 1.0);
  if (J.btally) {
    const long long nvox = (long long)J.nx * J.ny * J.nz;
    atomicAdd(J.btally + (long long)(hist % uint32_t(J.nbeamlets)) * nvox + (long long)idx, de);
  }
}

// tally forms of the block kernels, as template flags: warp-aggregated
// atomics, and the plain 3-D tally. A run whose jobs all score voxel dose only
// (no slab depth tally, no step counts, no beamlet tally) gets kernels
// without the other forms' code at every deposit site (smaller kernels: the
// phases are instruction-fetch bound)
constexpr int kTallyAgg = 1, kTallyPlain = 2;
// geometry form flag (set only together with kTallyPlain): every job is a
// voxel phantom of material ids with the materials' nominal densities (no
// slab preset indexed by depth, no per-voxel density array), and the electron
// splines of all materials lie on one grid at a fixed stride (DevTables::
// elecUniform)
constexpr int kGeomPlain = 4;
// single-job form flag (electron block kernel): every particle of the launch
// belongs to one job (a single-job run, or a chunk of one job in a batched
// run), whose record the kernel reads from its parameter block
// (constant-bank operands) instead of loading it from shared memory at every
// use
constexpr int kSingleJob = 8;
// slab form flags (set together): every job is a slab preset (materials by
// depth, nominal densities, electron splines on one grid) whose depth bins
// fit the block's shared-memory depth tally, and no beamlet tally
constexpr int kTallyDepth = 16, kGeomSlab = 32;
// tagged tally form flag: every job scores a 3-D voxel tally and a beamlet
// tally (influence matrix), nothing else
constexpr int kTallyTag = 64;
template <int TF>
__device__ __forceinline__ const JobF& JobRec(const PhaseArgs& a, const JobF* jobs, int job) {
  if constexpr ((TF & kSingleJob) != 0) return a.job0;
  else return jobs[job];
}
template <int TF>
__device__ __forceinline__ void ScoreT(const JobF& J, uint32_t meta, int ix, int iy, int iz, uint32_t hist, float e,
                                       const DepthAcc& d) {
  if constexpr ((TF & kTallyDepth) != 0) {
    const int b = J.dbase + int(SliceOfSub(meta >> 2)) * d.sliceStride + iz;
    atomicAdd(d.e + b, double(e));
    atomicAdd(d.n + b, 1u);
  } else if constexpr ((TF & kTallyTag) != 0) {
    const uint32_t idx = (uint32_t(iz) * uint32_t(J.ny) + uint32_t(iy)) * uint32_t(J.nx) + uint32_t(ix);
    const double de = double(e);
    ScoreBin(J, SliceOfSub(meta >> 2), idx, de, 0);
    const long long nvox = (long long)J.nx * J.ny * J.nz;
    atomicAdd(J.btally + (long long)(hist % uint32_t(J.nbeamlets)) * nvox + (long long)idx, de);
  } else if constexpr ((TF & kTallyPlain) != 0) {
    const uint32_t idx = (uint32_t(iz) * uint32_t(J.ny) + uint32_t(iy)) * uint32_t(J.nx) + uint32_t(ix);
    ScoreBin(J, SliceOfSub(meta >> 2), idx, double(e), TF & kTallyAgg);
  } else {
    Score(J, meta, ix, iy, iz, hist, e, TF & kTallyAgg, d);
  }
}

// bytes of a depth tally of `bins` bins (energy, then step counts)
__host__ __device__ constexpr size_t DepthAccBytes(int bins) { return size_t(bins) * (sizeof(double) + sizeof(unsigned)); }

// the block's depth tally at `mem` (dynamic shared memory, 8-byte aligned),
// zeroed; before the block's first barrier
__device__ __forceinline__ DepthAcc DepthAccInit(const PhaseArgs& a, unsigned char* mem) {
  DepthAcc d;
  if (a.depthBins > 0) {
    d.sliceStride = a.njobs * a.depthStride;
    d.e = reinterpret_cast<double*>(mem);
    d.n = reinterpret_cast<unsigned*>(mem + size_t(a.depthBins) * sizeof(double));
    for (int b = threadIdx.x; b < a.depthBins; b += blockDim.x) { d.e[b] = 0.0; d.n[b] = 0u; }
  }
  return d;
}

// adds the block's depth tally to the jobs' tallies (whole block, at its end)
__device__ __forceinline__ void DepthAccFlush(const PhaseArgs& a, const JobF* jobs, const DepthAcc& d) {
  if (d.e == nullptr) return;
  __syncthreads();
  for (int b = threadIdx.x; b < a.depthBins; b += blockDim.x) {
    const unsigned n = d.n[b];
    if (n == 0u) continue;
    // bin b = (slice * njobs + job) * depthStride + iz
    const int q = b / a.depthStride, iz = b % a.depthStride;
    const JobF& J = jobs[q % a.njobs];
    atomicAdd(J.tally + (long long)(q / a.njobs) * J.sstride + (long long)iz * J.tstride, d.e[b]);
    if (J.steps) atomicAdd(J.steps + iz, double(n));
  }
}

// density of voxel (ix, iy, iz) of material im (Geom::GetVoxelMaterialDensity)
__device__ __forceinline__ float VoxelRho(const JobF& J, const DevTables<float>& T, int ix, int iy, int iz, int im) {
  return J.rho ? __ldg(J.rho + (uint32_t(iz) * uint32_t(J.ny) + uint32_t(iy)) * uint32_t(J.nx) + uint32_t(ix))
               : T.density[im];
}

__device__ __forceinline__ bool InBox(const JobF& J, int ix, int iy, int iz) {
  return (unsigned)ix < (unsigned)J.nx && (unsigned)iy < (unsigned)J.ny && (unsigned)iz < (unsigned)J.nz;
}

__device__ __forceinline__ int MaterialAt(const JobF& J, int ix, int iy, int iz) {
  const uint8_t m = J.matByDepth ? __ldg(J.mat + iz)
                                 : __ldg(J.mat + (uint32_t(iz) * uint32_t(J.ny) + uint32_t(iy)) * uint32_t(J.nx) + uint32_t(ix));
  return m == kVacuum ? -1 : int(m);
}

// MaterialAt and VoxelRho for the kernels' geometry form (TF & kGeomPlain:
// the 3-D id array and the material's nominal density only)
template <int TF>
__device__ __forceinline__ int MaterialAtT(const JobF& J, int ix, int iy, int iz) {
  if constexpr ((TF & kGeomSlab) != 0) {
    const uint8_t m = __ldg(J.mat + iz);
    return m == kVacuum ? -1 : int(m);
  } else if constexpr ((TF & kGeomPlain) != 0) {
    const uint8_t m = __ldg(J.mat + (uint32_t(iz) * uint32_t(J.ny) + uint32_t(iy)) * uint32_t(J.nx) + uint32_t(ix));
    return m == kVacuum ? -1 : int(m);
  } else {
    return MaterialAt(J, ix, iy, iz);
  }
}
template <int TF>
__device__ __forceinline__ float VoxelRhoT(const JobF& J, const DevTables<float>& T, int ix, int iy, int iz, int im) {
  if constexpr ((TF & (kGeomPlain | kGeomSlab)) != 0) return T.density[im];
  else return VoxelRho(J, T, ix, iy, iz, im);
}

// Distance to the voxel walls along d. A face closer than half the tolerance
// ahead is crossed first (the push of Geom::DistanceToBoundary, Geom.cc:46-52).
// Returns false when the particle leaves the box.
__device__ __forceinline__ bool Settle(const JobF& J, PState& p, float& s, int& axis) {
  for (int it = 0; it < 6; ++it) {
    float sx = 1.0e20f, sy = 1.0e20f, sz = 1.0e20f;
    if (p.dx > 0.f) {
      const float pd = J.vx - p.lx;
      if (pd < kHalfTolF) { ++p.ix; p.lx = 0.f; if (p.ix >= J.nx) return false; continue; }
      sx = pd / p.dx;
    } else if (p.dx < 0.f) {
      const float pd = p.lx;
      if (pd < kHalfTolF) { --p.ix; p.lx = J.vx; if (p.ix < 0) return false; continue; }
      sx = -pd / p.dx;
    }
    if (p.dy > 0.f) {
      const float pd = J.vy - p.ly;
      if (pd < kHalfTolF) { ++p.iy; p.ly = 0.f; if (p.iy >= J.ny) return false; continue; }
      sy = pd / p.dy;
    } else if (p.dy < 0.f) {
      const float pd = p.ly;
      if (pd < kHalfTolF) { --p.iy; p.ly = J.vy; if (p.iy < 0) return false; continue; }
      sy = -pd / p.dy;
    }
    if (p.dz > 0.f) {
      const float pd = J.vz - p.lz;
      if (pd < kHalfTolF) { ++p.iz; p.lz = 0.f; if (p.iz >= J.nz) return false; continue; }
      sz = pd / p.dz;
    } else if (p.dz < 0.f) {
      const float pd = p.lz;
      if (pd < kHalfTolF) { --p.iz; p.lz = J.vz; if (p.iz < 0) return false; continue; }
      sz = -pd / p.dz;
    }
    s = sx; axis = 0;
    if (sy < s) { s = sy; axis = 1; }
    if (sz < s) { s = sz; axis = 2; }
    return true;
  }
  return false;
}

// move s along d, crossing the face of `axis` exactly when the step is
// geometry limited; false when the particle leaves the box
__device__ __forceinline__ bool MoveToFace(const JobF& J, PState& p, float s, int axis) {
  if (axis != 0) p.lx += s * p.dx;
  if (axis != 1) p.ly += s * p.dy;
  if (axis != 2) p.lz += s * p.dz;
  if (axis == 0) { if (p.dx > 0.f) { ++p.ix; p.lx = 0.f; } else { --p.ix; p.lx = J.vx; } }
  else if (axis == 1) { if (p.dy > 0.f) { ++p.iy; p.ly = 0.f; } else { --p.iy; p.ly = J.vy; } }
  else { if (p.dz > 0.f) { ++p.iz; p.lz = 0.f; } else { --p.iz; p.lz = J.vz; } }
  return InBox(J, p.ix, p.iy, p.iz);
}

// free flight of s (photons): may cross many voxels
__device__ __forceinline__ bool Fly(const JobF& J, PState& p, float s) {
  const float gx = p.lx + s * p.dx, gy = p.ly + s * p.dy, gz = p.lz + s * p.dz;
  // (clamped so that a very long flight cannot overflow the integer voxel index)
  const int kx = int(fmaxf(-1.0e6f, fminf(1.0e6f, floorf(gx * J.ivx))));
  const int ky = int(fmaxf(-1.0e6f, fminf(1.0e6f, floorf(gy * J.ivy))));
  const int kz = int(fmaxf(-1.0e6f, fminf(1.0e6f, floorf(gz * J.ivz))));
  p.ix += kx; p.iy += ky; p.iz += kz;
  p.lx = gx - float(kx) * J.vx;
  p.ly = gy - float(ky) * J.vy;
  p.lz = gz - float(kz) * J.vz;
  return InBox(J, p.ix, p.iy, p.iz);
}

// ---------------------------------------------------------------------------
// primaries
// ---------------------------------------------------------------------------
__device__ __forceinline__ int FindSegment(const Segment* segs, int n, long long i) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (segs[mid].prefix <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ void MakePrimary(const PhaseArgs& a, const Segment* segs, long long i, PState& p, PRng& rng) {
  const Segment& sg = segs[FindSegment(segs, a.nsegs, i)];
  const JobF& J = a.jobs[JobOfSub(uint32_t(sg.job))];
  const long long h = sg.firstHist + (i - sg.prefix);
  p.hist = uint32_t(h);
  p.slot = uint32_t(sg.slotBase + (i - sg.prefix));
  p.ulo = 0; p.uhi = 0;
  rng.Init(J.k0, J.k1, p.hist, 0u, 0u);
  double x = J.cx, y = J.cy;
  if (J.shape == 1) {
    x = J.cx + (rng.U() - 0.5f) * J.fx;
    y = J.cy + (rng.U() - 0.5f) * J.fy;
  } else if (J.shape == 2) {
    const int b = int(h % (long long)(J.nbx * J.nby));
    const int bx = b % J.nbx, by = b / J.nbx;
    x = J.cx + (bx - 0.5f * J.nbx) * J.fx + rng.U() * J.fx;
    y = J.cy + (by - 0.5f * J.nby) * J.fy + rng.U() * J.fy;
  }
  float e = J.e0;
  if (J.spectrum == 1) e = J.e0 + rng.U() * (J.e1 - J.e0);
  else if (J.spectrum == 2) e = J.e1 - (J.e1 - J.e0) * sqrtf(1.0f - rng.U());
  // entry plane z = z0 (face of the first voxel layer); x, y relative to the box
  const double rx = (x - J.x0) * J.ivx, ry = (y - J.y0) * J.ivy;
  p.ix = int(floor(rx)); p.iy = int(floor(ry)); p.iz = 0;
  p.lx = float((x - J.x0) - p.ix * double(J.vx));
  p.ly = float((y - J.y0) - p.iy * double(J.vy));
  p.lz = 0.f;
  p.dx = 0.f; p.dy = 0.f; p.dz = 1.f;
  p.e = e;
  p.meta = (J.particle == 0 ? 0u : 1u) | (uint32_t(sg.job) << 2);
  a.histE0[p.slot] = double(e);
}

// ---------------------------------------------------------------------------
// photon phase: Woodcock tracking (SimDPMLike.cc:463-635)
// ---------------------------------------------------------------------------
// Work distribution of a persistent phase kernel. A warp claims kWorkGrab
// consecutive items per atomic on the phase's work counter and hands them to
// its idle lanes over later iterations (warp-uniform state).
struct WorkPool {
  unsigned long long lo = 0, hi = 0, total = 0;
  bool exhausted = false;
  // returns the item for this lane (or ~0ull); `need` is the ballot of idle lanes
  __device__ __forceinline__ unsigned long long Take(unsigned need, bool idle, unsigned long long* head, int lane) {
    unsigned long long item = ~0ull;
    if (need == 0 || exhausted) return item;
    if (lo >= hi) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(head, (unsigned long long)kWorkGrab);
      base = __shfl_sync(kFull, base, 0);
      lo = base;
      hi = base + kWorkGrab < total ? base + kWorkGrab : total;
      if (base >= total) { exhausted = true; return item; }
    }
    const unsigned long long my = lo + __popc(need & ((1u << lane) - 1u));
    if (idle && my < hi) item = my;
    const unsigned long long n = __popc(need);
    lo = lo + n < hi ? lo + n : hi;
    return item;
  }
};

// escaped energy summed in the lane and flushed once per job change
// (keyed by the job's counters: the statistical batches of one job share them,
// so particles of different batches do not force a flush)
struct EscTally {
  double e = 0.0;
  RunCounters* c = nullptr;
  __device__ __forceinline__ void Add(const JobF* jobs, int j, double x) {
    RunCounters* cj = jobs[j].cnt;
    if (cj != c) {
      if (c && e != 0.0) atomicAdd(&c->escaped, e);
      e = 0.0;
      c = cj;
    }
    e += x;
  }
  __device__ __forceinline__ void Flush(const JobF*) {
    if (c && e != 0.0) atomicAdd(&c->escaped, e);
    e = 0.0;
  }
};

// running counts of the input stripes into shared memory; returns the total
__device__ __forceinline__ unsigned long long StripePrefix(const unsigned long long* counts, unsigned long long* pre) {
  if (threadIdx.x == 0) {
    unsigned long long s = 0;
    for (int k = 0; k < kStripes; ++k) { pre[k] = s; s += counts[k]; }
    pre[kStripes] = s;
  }
  __syncthreads();
  return pre[kStripes];
}

__global__ void __launch_bounds__(256) PhotonPhase(PhaseArgs a) {
  extern __shared__ __align__(16) unsigned char pdyn[];   // photon tables, then the depth tally
  __shared__ JobF sjobs[16];
  __shared__ unsigned long long spre[kStripes + 1];
  __shared__ PTables pt;
  const bool fewJobs = a.njobs <= 16;
  if (fewJobs) {
    for (int j = threadIdx.x; j < a.njobs; j += blockDim.x) sjobs[j] = a.jobs[j];
  }
  const unsigned long long nQ = StripePrefix(a.inCount, spre);
  const JobF* jobs = fewJobs ? sjobs : a.jobs;
  const unsigned long long total = (unsigned long long)a.nPrimaries + nQ;
  if (total == 0) return;   // an empty generation skips the table staging
  StagePhotonTables(a.T, kPhotonTablesInSmem, reinterpret_cast<float*>(pdyn), &pt);
  const DepthAcc dacc = DepthAccInit(a, pdyn + PhotonTableBytes(a.T));
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const DevTables<float>& T = a.T;

  bool active = false;
  WorkPool pool;
  pool.total = total;
  EscTally esc;
  PState p;
  PRng rng;
  double acc = 0.0;
  unsigned pst = 0;
  unsigned long long nph = 0;
  float lmax = 0.f, lmaxE = -1.f;   // Woodcock mean free path, kept while energy and job do not change
  int lmaxJob = -1;
  for (;;) {
    const unsigned need = __ballot_sync(kFull, !active);
    const unsigned long long my = pool.Take(need, !active, a.head, lane);
    if (my != ~0ull) {
      if (my < (unsigned long long)a.nPrimaries) {
        MakePrimary(a, a.segs, (long long)my, p, rng);
      } else {
        LoadParticle(a.in, StripedIndex(a.in, spre, my - a.nPrimaries), p);
        const JobF& J = jobs[JobOfSub(p.meta >> 2)];
        rng.Init(J.k0, J.k1, p.hist, p.ulo, p.uhi);
      }
      acc = 0.0;
      pst = 0;
      active = true;
      const JobF& J = jobs[JobOfSub(p.meta >> 2)];
      if (!InBox(J, p.ix, p.iy, p.iz) || MaterialAt(J, p.ix, p.iy, p.iz) < 0) {
        acc += p.e;
        esc.Add(jobs, JobOfSub(p.meta >> 2), double(p.e));
        atomicAdd(a.histE + p.slot, acc);
        active = false;
      }
    }
    if (!__any_sync(kFull, active)) {
      if (pool.exhausted) break;
      continue;
    }
    if (!active) continue;

    // one Woodcock step
    const int job = JobOfSub(p.meta >> 2);
    const JobF& J = jobs[job];
    bool done = false;
    if (++pst > kMaxPhotonSteps) {   // cannot happen for finite cross sections; bounded anyway
      acc += p.e;
      atomicAdd(&J.cnt->lost, 1ull);
      atomicAdd(a.histE + p.slot, acc);
      active = false;
      continue;
    }
    ++nph;
    if (p.e != lmaxE || job != lmaxJob) {
      lmax = 1.0f / (LinearGet(pt.imfpMax, p.e) * J.wscale);
      lmaxE = p.e;
      lmaxJob = job;
    }
    const float step = -lmax * __logf(rng.U());
    int im = -1;
    if (Fly(J, p, step)) im = MaterialAt(J, p.ix, p.iy, p.iz);
    if (im < 0) {
      acc += p.e;
      esc.Add(jobs, job, double(p.e));
      done = true;
    } else {
      const float rho = VoxelRho(J, T, p.ix, p.iy, p.iz, im);
      const float r1 = rng.U();
      float prob = 1.0f - LinearGet(pt.tot[im], p.e) * rho * lmax;
      if (r1 >= prob) {
        prob += LinearGet(pt.comp[im], p.e) * rho * lmax;
        if (r1 < prob) {
          // Compton (SimDPMLike.cc:512-570)
          const float a3 = rng.U(), a2 = rng.U(), a1 = rng.U();
          const float eps = SampleKN(T.kn, p.e, a1, a2, a3);
          const float kappa = p.e * (1.0f / kEMC2f);
          const float phCost = 1.0f - (1.0f - eps) / (eps * kappa);
          const float phE = eps * p.e;
          const float phPhi = 2.0f * kPIf * rng.U();
          const float elE = p.e - phE;
          float sn, cs;
          __sincosf(phPhi, &sn, &cs);
          if (elE < T.ecut) {
            Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, elE, a.aggregate, dacc);
            acc += elE;
          } else {
            const float e0 = kappa;
            const float elCost = (1.0f + e0) * sqrtf((1.0f - eps) / (e0 * (2.0f + e0 * (1.0f - eps))));
            const float sint = sqrtf(fmaxf(0.f, (1.0f + elCost) * (1.0f - elCost)));
            PState c = p;
            c.dx = -sint * cs; c.dy = -sint * sn; c.dz = elCost;   // phi + pi
            RotateToLab(c.dx, c.dy, c.dz, p.dx, p.dy, p.dz);
            c.e = elE;
            c.meta = 1u | (p.meta & ~3u);
            rng.Child(0, c.ulo, c.uhi);
            if (!Append(a.outE, a.outECount, a.overflow, c)) acc += elE;
          }
          p.e = phE;
          if (p.e < T.gcut) {
            Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, p.e, a.aggregate, dacc);
            acc += p.e;
            done = true;
          } else {
            const float phSint = sqrtf(fmaxf(0.f, (1.0f - phCost) * (1.0f + phCost)));
            float u1 = phSint * cs, u2 = phSint * sn, u3 = phCost;
            RotateToLab(u1, u2, u3, p.dx, p.dy, p.dz);
            p.dx = u1; p.dy = u2; p.dz = u3;
          }
        } else {
          prob += LinearGet(pt.pair[im], p.e) * rho * lmax;
          if (r1 < prob && p.e > 2.0f * kEMC2f) {
            // pair production (SimDPMLike.cc:573-627)
            const float sum = p.e - 2.0f * kEMC2f;
            const float e1 = rng.U() * sum;
            const float e2 = sum - e1;
            if (e2 < T.ecut) {
              Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, e2, a.aggregate, dacc);
              acc += e2;
            } else {
              PState c = p;
              c.e = e2; c.meta = 1u | (p.meta & ~3u);
              rng.Child(0, c.ulo, c.uhi);
              if (!Append(a.outE, a.outECount, a.overflow, c)) acc += e2;
            }
            if (e1 < T.ecut) {
              Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, e1, a.aggregate, dacc);
              acc += e1;
              // annihilation at rest (SimDPMLike.cc:753-791)
              const float cost = 1.0f - 2.0f * rng.U();
              const float sint = sqrtf(fmaxf(0.f, (1.0f - cost) * (1.0f + cost)));
              const float phi = 2.0f * kPIf * rng.U();
              float s2, c2;
              __sincosf(phi, &s2, &c2);
              PState g = p;
              g.e = kEMC2f; g.meta = 0u | (p.meta & ~3u);
              g.dx = sint * c2; g.dy = sint * s2; g.dz = cost;
              rng.Child(0, g.ulo, g.uhi);
              if (!Append(a.outP, a.outPCount, a.overflow, g)) acc += kEMC2f;
              g.dx = -g.dx; g.dy = -g.dy; g.dz = -g.dz;
              rng.Child(1, g.ulo, g.uhi);
              if (!Append(a.outP, a.outPCount, a.overflow, g)) acc += kEMC2f;
            } else {
              PState c = p;
              c.e = e1; c.meta = 2u | (p.meta & ~3u);
              rng.Child(1, c.ulo, c.uhi);
              if (!Append(a.outE, a.outECount, a.overflow, c)) acc += e1 + 2.0f * kEMC2f;
            }
            done = true;
          } else if (r1 < prob) {
            // below threshold (pair IMFP floor): treated as photoelectric
            Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, p.e, a.aggregate, dacc);
            acc += p.e;
            done = true;
          } else {
            // photoelectric absorption
            Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, p.e, a.aggregate, dacc);
            acc += p.e;
            done = true;
          }
        }
      }
    }
    if (done) {
      atomicAdd(a.histE + p.slot, acc);
      active = false;
    }
  }
  esc.Flush(jobs);
  DepthAccFlush(a, jobs, dacc);
  for (int o = 16; o > 0; o >>= 1) nph += __shfl_down_sync(kFull, nph, o);
  if (lane == 0 && a.njobs > 0) atomicAdd(&a.jobs[0].cnt->photonSteps, nph);
}

// ---------------------------------------------------------------------------
// electron phase: condensed-history stepping (SimDPMLike.cc:81-460)
// ---------------------------------------------------------------------------
struct EState {
  float nTr1, nTr10, nMol, invMol, nBrem, ekin0, sGeom;
  int axis;
  bool hinge, needGeom;
};

__device__ __forceinline__ void InitElectron(const ETables& et, const PState& p, PRng& rng, EState& s) {
  // SimDPMLike.cc:113-146
  s.hinge = true;
  s.ekin0 = p.e;
  const float le = __logf(p.e);
  s.nTr1 = SplineLe(et.k1, p.e, le);
  s.nTr10 = rng.U() * s.nTr1;
  s.nTr1 -= s.nTr10;
  s.nMol = -__logf(rng.U());
  s.invMol = SplineLe(et.moller, p.e, le);
  s.nBrem = -__logf(rng.U());
  s.needGeom = true;
}

__global__ void __launch_bounds__(256) ElectronPhase(PhaseArgs a) {
  extern __shared__ __align__(16) float sdata[];   // 16-byte spline records
  __shared__ ETables et;
  __shared__ JobF sjobs[16];
  const bool fewJobs = a.njobs <= 16;
  if (fewJobs)
    for (int j = threadIdx.x; j < a.njobs; j += blockDim.x) sjobs[j] = a.jobs[j];
  __shared__ unsigned long long spre[kStripes + 1];
  const unsigned long long nQ = StripePrefix(a.inCount, spre);
  const JobF* jobs = fewJobs ? sjobs : a.jobs;
  const unsigned long long total = (unsigned long long)a.nPrimaries + nQ;
  if (total == 0) return;   // an empty generation skips the table staging
  StageElectronTables(a.T, sdata, &et);
  const int lane = threadIdx.x & 31;
  const DevTables<float>& T = a.T;
  const float ecut = T.ecut, gcut = T.gcut;

  bool active = false;
  WorkPool pool;
  pool.total = total;
  EscTally esc;
  PState p;
  PRng rng;
  EState s;
  double acc = 0.0;
  unsigned pst = 0;
  unsigned long long nsteps = 0;
  for (;;) {
    const unsigned need = __ballot_sync(kFull, !active);
    const unsigned long long my = pool.Take(need, !active, a.head, lane);
    if (my != ~0ull) {
      if (my < (unsigned long long)a.nPrimaries) {
        MakePrimary(a, a.segs, (long long)my, p, rng);
      } else {
        LoadParticle(a.in, StripedIndex(a.in, spre, my - a.nPrimaries), p);
        const JobF& J = jobs[JobOfSub(p.meta >> 2)];
        rng.Init(J.k0, J.k1, p.hist, p.ulo, p.uhi);
      }
      acc = 0.0;
      pst = 0;
      active = true;
      const JobF& J = jobs[JobOfSub(p.meta >> 2)];
      if (!InBox(J, p.ix, p.iy, p.iz) || MaterialAt(J, p.ix, p.iy, p.iz) < 0) {
        acc += p.e + ((p.meta & 3u) == 2u ? 2.0f * kEMC2f : 0.f);
        esc.Add(jobs, JobOfSub(p.meta >> 2), acc);
        atomicAdd(a.histE + p.slot, acc);
        active = false;
      } else {
        InitElectron(et, p, rng, s);
      }
    }
    if (!__any_sync(kFull, active)) {
      if (pool.exhausted) break;
      continue;
    }
    if (!active) continue;

    // ---- one condensed-history sub-step (SimDPMLike.cc:273-458) ----
    const int job = JobOfSub(p.meta >> 2);
    const JobF& J = jobs[job];
    const bool positron = (p.meta & 3u) == 2u;
    bool done = false;
    int im = -1;
    if (s.needGeom) {
      if (Settle(J, p, s.sGeom, s.axis)) im = MaterialAt(J, p.ix, p.iy, p.iz);
      s.needGeom = false;
    } else {
      im = MaterialAt(J, p.ix, p.iy, p.iz);
    }
    if (im < 0) {
      const float out = p.e + (positron ? 2.0f * kEMC2f : 0.f);
      acc += out;
      esc.Add(jobs, job, double(out));
      done = true;
    } else if (++pst > kMaxElectronSteps) {   // bounded: every step loses energy or moves >= 5e-5 mm
      acc += p.e + (positron ? 2.0f * kEMC2f : 0.f);
      atomicAdd(&J.cnt->lost, 1ull);
      done = true;
    } else {
      ++nsteps;
      const float rho = VoxelRho(J, T, p.ix, p.iy, p.iz, im);
      float step = s.sGeom;
      int what = 0;
      const float le = __logf(p.e);
      float dedx = SplineLe(et.dedx[im], p.e, le) * rho;
      float emid = fmaxf(p.e - 0.5f * step * dedx, ecut);
      float lm = __logf(emid);
      float dTr1 = SplineLe(et.itr1[im], emid, lm) * rho;
      const float dMol = s.invMol * T.mollerScale[im] * rho;
      const float dBrem = SplineLe(et.brem[im], emid, lm) * rho;
      const float sBrem = s.nBrem / dBrem;
      if (sBrem < step) { step = sBrem; what = 1; }
      const float sMol = s.nMol / dMol;
      if (sMol < step) { step = sMol; what = 2; }
      float sEl = s.nTr1 / dTr1;
      if (sEl < step) {
        sEl = s.nTr1 / (SplineLe(et.itr1[im], p.e, le) * rho);
        emid = fmaxf(p.e - 0.5f * sEl * dedx, ecut);
        dTr1 = SplineLe(et.itr1[im], emid, __logf(emid)) * rho;
        sEl = fminf(step, s.nTr1 / dTr1);
        step = sEl;
        what = 3;
      }
      s.nBrem = (what == 1) ? 0.f : s.nBrem - step * dBrem;
      s.nMol = (what == 2) ? 0.f : s.nMol - step * dMol;
      s.nTr1 = (what == 3) ? 0.f : s.nTr1 - step * dTr1;
      emid = fmaxf(p.e - 0.5f * step * dedx, ecut);
      dedx = SplineLe(et.dedx[im], emid, __logf(emid)) * rho;
      const float de = step * dedx;
      const float ef = p.e - de;
      if (ef < ecut) {
        // stops in this step: deposit all (SimDPMLike.cc:401-422)
        const float edep = p.e;
        p.e = 0.f;
        if (!positron) {
          Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, edep, a.aggregate);
          acc += edep;
        } else {
          // e+: move to the end of the step, annihilate there
          bool inside;
          if (what == 0) inside = MoveToFace(J, p, step, s.axis);
          else { p.lx += step * p.dx; p.ly += step * p.dy; p.lz += step * p.dz; inside = true; }
          const int im2 = inside ? MaterialAt(J, p.ix, p.iy, p.iz) : -1;
          if (im2 < 0) {
            acc += edep + 2.0f * kEMC2f;
            esc.Add(jobs, job, double(edep + 2.0f * kEMC2f));
          } else {
            const float cost = 1.0f - 2.0f * rng.U();
            const float sint = sqrtf(fmaxf(0.f, (1.0f - cost) * (1.0f + cost)));
            const float phi = 2.0f * kPIf * rng.U();
            float sn, cs;
            __sincosf(phi, &sn, &cs);
            PState g = p;
            g.e = kEMC2f; g.meta = 0u | (p.meta & ~3u);
            g.dx = sint * cs; g.dy = sint * sn; g.dz = cost;
            rng.Child(0, g.ulo, g.uhi);
            if (!Append(a.outP, a.outPCount, a.overflow, g)) acc += kEMC2f;
            g.dx = -g.dx; g.dy = -g.dy; g.dz = -g.dz;
            rng.Child(1, g.ulo, g.uhi);
            if (!Append(a.outP, a.outPCount, a.overflow, g)) acc += kEMC2f;
            Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, edep, a.aggregate);
            acc += edep;
          }
        }
        done = true;
      } else {
        p.e = ef;
        // score in the voxel of the step, then move
        Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, de, a.aggregate);
        acc += de;
        if (what == 0) {
          if (!MoveToFace(J, p, step, s.axis)) {
            acc += p.e + (positron ? 2.0f * kEMC2f : 0.f);
            esc.Add(jobs, job, double(p.e + (positron ? 2.0f * kEMC2f : 0.f)));
            done = true;
          } else if (!Settle(J, p, s.sGeom, s.axis)) {
            acc += p.e + (positron ? 2.0f * kEMC2f : 0.f);
            esc.Add(jobs, job, double(p.e + (positron ? 2.0f * kEMC2f : 0.f)));
            done = true;
          }
        } else {
          p.lx += step * p.dx; p.ly += step * p.dy; p.lz += step * p.dz;
          s.needGeom = true;
          // the interaction (SimDPMLike.cc:169-244)
          if (what == 1) {
            if (p.e > gcut) {
              // bremsstrahlung photon (SimDPMLike.cc:661-695)
              const float r3 = rng.U(), r2 = rng.U(), r1 = rng.U();
              const float eg = SampleSB(T.sb[im], p.e, r1, r2, r3);
              const float dum0 = (kEMC2f * 0.7071067812f) / (p.e + kEMC2f);
              const float cost = fmaxf(-1.0f, fminf(1.0f, 1.0f - dum0 * dum0));
              const float sint = sqrtf(fmaxf(0.f, (1.0f + cost) * (1.0f - cost)));
              const float phi = 2.0f * kPIf * rng.U();
              float sn, cs;
              __sincosf(phi, &sn, &cs);
              PState g = p;
              g.e = eg; g.meta = 0u | (p.meta & ~3u);
              g.dx = sint * cs; g.dy = sint * sn; g.dz = cost;
              RotateToLab(g.dx, g.dy, g.dz, p.dx, p.dy, p.dz);
              rng.Child(0, g.ulo, g.uhi);
              if (!Append(a.outP, a.outPCount, a.overflow, g)) acc += eg;
              p.e -= eg;
            }
            if (p.e < ecut) {
              Score(J, p.meta, p.ix, p.iy, p.iz, p.hist, p.e, a.aggregate);
              acc += p.e;
              if (positron) {
                const float cost = 1.0f - 2.0f * rng.U();
                const float sint = sqrtf(fmaxf(0.f, (1.0f - cost) * (1.0f + cost)));
                const float phi = 2.0f * kPIf * rng.U();
                float sn, cs;
                __sincosf(phi, &sn, &cs);
                PState g = p;
                g.e = kEMC2f; g.meta = 0u | (p.meta & ~3u);
                g.dx = sint * cs; g.dy = sint * sn; g.dz = cost;
                rng.Child(0, g.ulo, g.uhi);
                if (!Append(a.outP, a.outPCount, a.overflow, g)) acc += kEMC2f;
                g.dx = -g.dx; g.dy = -g.dy; g.dz = -g.dz;
                rng.Child(1, g.ulo, g.uhi);
                if (!Append(a.outP, a.outPCount, a.overflow, g)) acc += kEMC2f;
              }
              p.e = 0.f;
              done = true;
            } else {
              s.nBrem = -__logf(rng.U());
            }
          } else if (what == 2) {
            if (p.e > 2.0f * ecut) {
              // Moller delta electron (SimDPMLike.cc:699-728)
              const float r3 = rng.U(), r2 = rng.U(), r1 = rng.U();
              const float se = SampleMoller(T.mol, p.e, r1, r2, r3);
              const float k2 = 2.0f * kEMC2f;
              const float cost = fminf(1.0f, sqrtf(se * (p.e + k2) / (p.e * (se + k2))));
              const float sint = sqrtf(fmaxf(0.f, (1.0f + cost) * (1.0f - cost)));
              const float phi = 2.0f * kPIf * rng.U();
              float sn, cs;
              __sincosf(phi, &sn, &cs);
              PState c = p;
              c.e = se; c.meta = 1u | (p.meta & ~3u);
              c.dx = sint * cs; c.dy = sint * sn; c.dz = cost;
              RotateToLab(c.dx, c.dy, c.dz, p.dx, p.dy, p.dz);
              rng.Child(0, c.ulo, c.uhi);
              if (!Append(a.outE, a.outECount, a.overflow, c)) acc += se;
              p.e -= se;
            }
            s.nMol = -__logf(rng.U());
            s.invMol = SplineLe(et.moller, p.e, __logf(p.e));
          } else if (what == 3) {
            if (s.hinge) {
              // GS angular deflection at the hinge (SimDPMLike.cc:731-750)
              const float r2 = rng.U(), r1 = rng.U();
              float cost, sint;
              SampleGSAngle(T.gs, s.ekin0, r1, r2, cost, sint);
              const float phi = 2.0f * kPIf * rng.U();
              float sn, cs;
              __sincosf(phi, &sn, &cs);
              float u1 = sint * cs, u2 = sint * sn, u3 = cost;
              RotateToLab(u1, u2, u3, p.dx, p.dy, p.dz);
              const float inv = rsqrtf(u1 * u1 + u2 * u2 + u3 * u3);
              p.dx = u1 * inv; p.dy = u2 * inv; p.dz = u3 * inv;
              s.nTr1 = s.nTr10;
              s.hinge = false;
            } else {
              s.ekin0 = p.e;
              s.nTr1 = SplineLe(et.k1, p.e, __logf(p.e));
              s.nTr10 = rng.U() * s.nTr1;
              s.nTr1 -= s.nTr10;
              s.hinge = true;
            }
          }
        }
      }
    }
    if (done) {
      atomicAdd(a.histE + p.slot, acc);
      active = false;
    }
  }
  // step counters: one atomic per warp
  for (int o = 16; o > 0; o >>= 1) nsteps += __shfl_down_sync(kFull, nsteps, o);
  esc.Flush(jobs);
  if (lane == 0 && a.njobs > 0) atomicAdd(&a.jobs[0].cnt->steps, nsteps);
}

// ---------------------------------------------------------------------------
// electron phase, block-batched: kSlots electrons per block live in shared
// memory, each waiting in one of six rings (shared memory) by what it does
// next: MSC hinge, MSC step end, brem, Moller, plain sub-step or refill. A
// warp takes up to 32 entries of one ring whenever it is free, runs that
// interaction (or the refill) and one condensed-history sub-step on them, and
// puts each slot on the ring of its next action. The code of one interaction
// thus runs with full warps, and no warp waits for another between sub-steps.
// A particle's history does not depend on this order: every particle draws
// from its own random stream.
//
// A ring has kRingSize (512) cells, at least one per slot, and two counters
// (head: entries taken, tail: entries reserved); every slot is on at most one
// ring, so no ring holds more than kSlots entries. The cell of position pos
// holds (lap << 10 | full << 9 | slot) with lap = pos / 512 mod 64, the
// bounded-queue scheme of D. Vyukov: a producer waits until its cell is empty
// for its lap, a consumer until it is full for its lap, so neither can take
// the other lap's entry. At most one operation of each warp is pending on a
// cell, so a cell never lags its newest reservation by more laps than the
// block has warps (at most 32), and 6 bits tell the laps apart.
// ---------------------------------------------------------------------------
// Slots per block: a compile-time size of the shared-memory state, instantiated
// for kSlots (the default: 3 blocks, ~157 KB, fit the 164 KB shared-memory
// carve-out and leave the rest to L1) and kSlotsSmall (more L1), and chosen per
// run (dpmx_run_options::electron_slots, tried by the autotuner)
constexpr int kSlots = 448;
constexpr int kSlotsSmall = 384;
constexpr int kBlockMinBlocks = 3;      // resident blocks per SM the kernel is compiled for
constexpr int kBlockThreads = 320;      // threads per block (a multiple of 32): 64 registers, 30 warps per SM
constexpr int kSecondStepLanes = 20;    // lanes that must go on for a second sub-step in the same turn
constexpr bool kTablesInSmem = false;  // electron tables staged per block, else read through L1
constexpr uint32_t kFHinge = 4u, kFPositron = 16u;
constexpr int8_t kMatUnknown = -2;   // the slot's voxel changed since its material was read

// shared-memory state of the NS resident electrons, in 16-byte records that a
// lane reads or writes with one 128-bit access
template <int NS>
struct SlotArraysT {
  float4 pos[NS];   // offset in the voxel lx, ly, lz; kinetic energy
  float4 dir[NS];   // direction dx, dy, dz; voxel (PackVox, as float bits)
  float4 mfp[NS];   // nTr1, nMol, invMol, nBrem
  uint4 id[NS];     // flags (hinge, positron; sub-job << 8), history, energy-check slot, sub-steps
  uint4 rs[NS];     // random stream uid lo, uid hi, counter; ekin0 (float bits)
  float nTr10[NS];
  double acc[NS];
  int8_t mat[NS];   // material of the slot's current voxel (-1: vacuum)
};
constexpr long long kWaitCycles = 4LL << 30;   // bound of one wait (~2 s): then the warp gives up
constexpr int kRingBits = 9;
constexpr int kRingSize = 1 << kRingBits;   // cells per ring: at least the slots of a block
constexpr uint32_t kCellSlot = uint32_t(kRingSize) - 1u, kCellFull = uint32_t(kRingSize);

static_assert(kBlockThreads <= 32 * 32, "a ring cell's 6-bit lap covers at most 32 pending warps");
template <int NR>
struct Rings {
  uint16_t cell[NR][kRingSize];
  unsigned int head[NR], tail[NR];
  int live;        // slots not retired: queued or held by a warp
  int exhausted;   // every work item of the generation has been claimed
};

__device__ __forceinline__ uint32_t CellEmpty(uint32_t pos) { return ((pos >> kRingBits) & 63u) << (kRingBits + 1); }
__device__ __forceinline__ uint32_t CellFull(uint32_t pos) { return CellEmpty(pos) | kCellFull; }

__device__ __forceinline__ uint32_t CellLoad(const uint16_t* c) {
  uint16_t v;
  asm volatile("ld.acquire.cta.shared::cta.u16 %0, [%1];"
               : "=h"(v)
               : "r"(uint32_t(__cvta_generic_to_shared(c)))
               : "memory");
  return v;
}
// publishes a cell: the slot's state written before it is visible to the
// warp that loads the cell
__device__ __forceinline__ void CellStore(uint16_t* c, uint32_t v) {
  asm volatile("st.release.cta.shared::cta.u16 [%0], %1;" ::"r"(uint32_t(__cvta_generic_to_shared(c))),
               "h"(uint16_t(v))
               : "memory");
}
// waits until (cell & m) == want; false after `limit` cycles
__device__ __forceinline__ bool CellWait(const uint16_t* c, uint32_t want, uint32_t m, uint32_t& v,
                                         long long limit = kWaitCycles) {
  v = CellLoad(c);
  if ((v & m) == want) return true;
  const long long t0 = clock64();
  for (;;) {
    __nanosleep(32);
    v = CellLoad(c);
    if ((v & m) == want) return true;
    if (clock64() - t0 > limit) return false;
  }
}

// slots 0 .. nslots - 1 on ring `idle` (lap 0, full), every other cell empty
// for lap 0; before a barrier
template <int NR>
__device__ __forceinline__ void RingsInit(Rings<NR>& R, int idle, int nslots) {
  for (int i = threadIdx.x; i < NR * kRingSize; i += blockDim.x) {
    const int r = i / kRingSize, k = i % kRingSize;
    R.cell[r][k] = uint16_t(r == idle && k < nslots ? (kCellFull | uint32_t(k)) : 0u);
  }
  if (threadIdx.x < NR) {
    R.head[threadIdx.x] = 0u;
    R.tail[threadIdx.x] = int(threadIdx.x) == idle ? unsigned(nslots) : 0u;
  }
  if (threadIdx.x == 0) {
    R.live = nslots;
    R.exhausted = 0;
  }
}

// the calling warp (all lanes) takes up to 32 entries of the fullest ring
// (the longest wait, and the fullest warps). Returns the ring, with
// the slot of each lane < n in k, or -1 when no slot is queued or live (done)
// or a wait gave up (gaveUp set).
template <int NR>
__device__ __forceinline__ int RingTake(Rings<NR>& R, int lane, int& n, int& k, bool& gaveUp) {
  static_assert(NR <= 6, "ring index packed in 3 bits");
  volatile unsigned int* vhead = R.head;
  volatile unsigned int* vtail = R.tail;
  int ring = -1;
  uint32_t h = 0;
  long long t0 = 0;
  bool waited = false;
  n = 0;
  for (;;) {
    uint32_t hh = 0;
    int av = 0;
    if (lane < NR) {
      hh = vhead[lane];
      av = int(vtail[lane] - hh);
    }
    // the fullest ring; of equally full ones, the first
    const int pick =
        7 - int(__reduce_max_sync(kFull, lane < NR ? (uint32_t(av) << 3) | uint32_t(7 - lane) : 0u) & 7u);
    const int pav = __shfl_sync(kFull, av, pick);
    if (pav > 0) {
      const int take = min(pav, 32);
      int ok = 0;
      if (lane == pick) ok = atomicCAS(&R.head[pick], hh, hh + uint32_t(take)) == hh;
      if (__shfl_sync(kFull, ok, pick)) {
        ring = pick;
        h = __shfl_sync(kFull, hh, pick);
        n = take;
        break;
      }
      continue;   // another warp took them first
    }
    if (__shfl_sync(kFull, *(volatile int*)&R.live, 0) == 0) return -1;
    // the rings are empty while other warps hold slots: wait for their puts
    if (!waited) {
      t0 = clock64();
      waited = true;
    } else if (clock64() - t0 > kWaitCycles) {
      gaveUp = true;
      return -1;
    }
    __nanosleep(128);
  }
  bool bad = false;
  if (lane < n) {
    const uint32_t pos = h + uint32_t(lane);
    uint16_t* c = &R.cell[ring][pos & kCellSlot];
    uint32_t v;
    if (CellWait(c, CellFull(pos), ~kCellSlot, v)) {
      k = int(v & kCellSlot);
      CellStore(c, CellEmpty(pos + kRingSize));
    } else {
      bad = true;
    }
  }
  if (__any_sync(kFull, bad)) {
    gaveUp = true;
    return -1;
  }
  return ring;
}

// the calling warp (all lanes) puts slot k on ring q (q == NR: the slot
// retires; q < 0: nothing to put); one reservation per ring and warp
template <int NR>
__device__ __forceinline__ void RingPut(Rings<NR>& R, int lane, int q, int k, bool& gaveUp) {
  const unsigned grp = __match_any_sync(kFull, q);
  const int leader = __ffs(grp) - 1;
  uint32_t base = 0;
  if (lane == leader && q >= 0) {
    if (q < NR) base = atomicAdd(&R.tail[q], uint32_t(__popc(grp)));
    else atomicSub(&R.live, __popc(grp));
  }
  base = __shfl_sync(kFull, base, leader);
  bool bad = false;
  if (q >= 0 && q < NR) {
    const uint32_t pos = base + uint32_t(__popc(grp & ((1u << lane) - 1u)));
    uint16_t* c = &R.cell[q][pos & kCellSlot];
    uint32_t v;
    if (CellWait(c, CellEmpty(pos), 0xffffu, v)) CellStore(c, CellFull(pos) | uint32_t(k));
    else bad = true;
  }
  if (__any_sync(kFull, bad)) gaveUp = true;
}

// electron rings (of equally full rings the first is taken)
enum : int { kRBrem, kRMoller, kRHinge, kRMscEnd, kRIdle, kRStep, kRings };
static_assert(kSlots <= kRingSize && kSlotsSmall <= kRingSize, "a ring holds every slot");
// ring of a sub-step's result code (0 step, 1 brem, 2 Moller, 3 hinge, 4 MSC
// step end, 5 finished), four bits per code
constexpr uint32_t kRingOfCode = 0x432105u;
using SlotRings = Rings<kRings>;

template <int NS>
__host__ __device__ constexpr size_t BlockPhaseStaticBytes() {
  return (sizeof(SlotArraysT<NS>) + sizeof(SlotRings) + 15) & ~size_t(15);   // staged tables start 16-byte aligned
}

// dynamic shared memory of the block kernel: slots, rings, the electron tables
// when staged, then the depth tally of `depthBins` bins
template <int NS>
__host__ __device__ inline size_t BlockPhaseSmemBytesFor(const DevTables<float>& T, int depthBins) {
  const size_t b = BlockPhaseStaticBytes<NS>() + (kTablesInSmem ? size_t(T.elecCount) * sizeof(float) : 0);
  return ((b + 15) & ~size_t(15)) + DepthAccBytes(depthBins);
}

__device__ __forceinline__ void UnpackVox(uint32_t v, PState& p) {
  p.ix = int(v & 0x7ffu); p.iy = int((v >> 11) & 0x7ffu); p.iz = int(v >> 22);
}

template <class SA>
__device__ __forceinline__ void LoadSlot(const SA& S, int k, PState& p, EState& s, uint32_t& fl) {
  const float4 a = S.pos[k], b = S.dir[k], c = S.mfp[k];
  const uint4 d = S.id[k], r = S.rs[k];
  p.lx = a.x; p.ly = a.y; p.lz = a.z; p.e = a.w;
  p.dx = b.x; p.dy = b.y; p.dz = b.z;
  UnpackVox(__float_as_uint(b.w), p);
  s.nTr1 = c.x; s.nMol = c.y; s.invMol = c.z; s.nBrem = c.w;
  fl = d.x; p.hist = d.y; p.slot = d.z;
  p.ulo = r.x; p.uhi = r.y;
  s.ekin0 = __uint_as_float(r.w);
  s.nTr10 = S.nTr10[k];
  p.meta = ((fl >> 8) << 2) | ((fl & kFPositron) ? 2u : 1u);
  s.hinge = (fl & kFHinge) != 0;
}

// a new particle in slot k, its random stream at counter ctr
template <class SA>
__device__ __forceinline__ void StoreSlot(SA& S, int k, const PState& p, const EState& s, uint32_t ctr) {
  S.pos[k] = make_float4(p.lx, p.ly, p.lz, p.e);
  S.dir[k] = make_float4(p.dx, p.dy, p.dz, __uint_as_float(PackVox(p.ix, p.iy, p.iz)));
  S.mfp[k] = make_float4(s.nTr1, s.nMol, s.invMol, s.nBrem);
  S.id[k] = make_uint4((s.hinge ? kFHinge : 0u) | ((p.meta & 3u) == 2u ? kFPositron : 0u) | ((p.meta >> 2) << 8),
                       p.hist, p.slot, 0u);
  S.rs[k] = make_uint4(p.ulo, p.uhi, ctr, __float_as_uint(s.ekin0));
  S.nTr10[k] = s.nTr10;
}

// the part of slot k a plain sub-step reads (the random stream, the MSC hinge
// state and nTr10 stay as they are; pst: sub-steps taken), and the part it
// writes back
template <class SA>
__device__ __forceinline__ void LoadStepState(const SA& S, int k, PState& p, EState& s, uint32_t& fl,
                                              uint32_t& pst) {
  const float4 a = S.pos[k], b = S.dir[k], c = S.mfp[k];
  const uint4 d = S.id[k];
  p.lx = a.x; p.ly = a.y; p.lz = a.z; p.e = a.w;
  p.dx = b.x; p.dy = b.y; p.dz = b.z;
  UnpackVox(__float_as_uint(b.w), p);
  s.nTr1 = c.x; s.nMol = c.y; s.invMol = c.z; s.nBrem = c.w;
  fl = d.x; p.hist = d.y; p.slot = d.z; pst = d.w;
  p.meta = ((fl >> 8) << 2) | ((fl & kFPositron) ? 2u : 1u);
  s.hinge = (fl & kFHinge) != 0;
}

template <class SA>
__device__ __forceinline__ void StoreStepState(SA& S, int k, const PState& p, const EState& s) {
  S.pos[k] = make_float4(p.lx, p.ly, p.lz, p.e);
  S.dir[k].w = __uint_as_float(PackVox(p.ix, p.iy, p.iz));
  S.mfp[k] = make_float4(s.nTr1, s.nMol, s.invMol, s.nBrem);
}

// random stream of slot k (a fresh Philox block per use; the counter advances)
template <class SA>
__device__ __forceinline__ void SlotRng(const SA& S, int k, const JobF& J, uint32_t hist, PRng& r) {
  const uint4 q = S.rs[k];
  r.Init(J.k0, J.k1, hist, q.x, q.y);
  r.ctr = q.z;
}

// e+ annihilation at rest: two back-to-back 0.511 MeV photons (SimDPMLike.cc:753-791)
__device__ __forceinline__ void AnnihilateF(const PhaseArgs& a, const PState& p, PRng& rng, double& acc) {
  const float cost = 1.0f - 2.0f * rng.U();
  const float sint = sqrtf(fmaxf(0.f, (1.0f - cost) * (1.0f + cost)));
  const float phi = 2.0f * kPIf * rng.U();
  float sn, cs;
  __sincosf(phi, &sn, &cs);
  PState g = p;
  g.e = kEMC2f; g.meta = 0u | (p.meta & ~3u);
  g.dx = sint * cs; g.dy = sint * sn; g.dz = cost;
#pragma unroll 1
  for (int c = 0; c < 2; ++c) {   // child c; the second photon opposite the first
    rng.Child(c, g.ulo, g.uhi);
    if (!Append(a.outP, a.outPCount, a.overflow, g)) acc += kEMC2f;
    g.dx = -g.dx; g.dy = -g.dy; g.dz = -g.dz;
  }
}

// one condensed-history sub-step of slot k. Returns 0 to keep stepping,
// 1 brem, 2 Moller, 3 MSC hinge, 4 MSC step end, 5 finished.
// Every sub-step starts by settling the electron in its voxel (distance to the
// walls, a face within the tolerance crossed first); a sub-step that ends on
// a voxel face only moves onto it, and the next one settles. One deposit at
// most is scored, and one escape counted, per sub-step, at one place in the
// code each (fewer inlined copies: the kernel is instruction-fetch bound).
// the dE/dx + 1/lambda_1 and brem descriptors of material im: in the plain
// form material 0's (kernel parameters, constant bank) with the records moved
// by im strides, else the block's shared copies
template <int TF>
__device__ __forceinline__ SplinePairT<float> DiOf(const PhaseArgs& a, const ETables& et, int im) {
  if constexpr ((TF & (kGeomPlain | kGeomSlab)) != 0) {
    SplinePairT<float> d = a.T.di[0];
    d.p += im * a.T.diStride;
    return d;
  } else {
    return et.di[im];
  }
}
template <int TF>
__device__ __forceinline__ SplineT<float> BremOf(const PhaseArgs& a, const ETables& et, int im) {
  if constexpr ((TF & (kGeomPlain | kGeomSlab)) != 0) {
    SplineT<float> d = a.T.brem[0];
    d.p += im * a.T.bremStride;
    return d;
  } else {
    return et.brem[im];
  }
}

template <int TF, class SA>
__device__ __forceinline__ int StepSlot(const PhaseArgs& a, const ETables& et, const JobF* jobs, SA& S,
                                        int k, EscTally& esc, unsigned long long& nsteps, const DepthAcc& dacc) {
  const DevTables<float>& T = a.T;
  PState p;
  EState s;
  uint32_t fl, pst;
  LoadStepState(S, k, p, s, fl, pst);
  const int job = JobOfSub(fl >> 8);
  const JobF& J = JobRec<TF>(a, jobs, job);
  const bool positron = (fl & kFPositron) != 0;
  double acc = S.acc[k];
  int code = 0;
  int im = -1;
  {
    const int ox = p.ix, oy = p.iy, oz = p.iz;
    if (Settle(J, p, s.sGeom, s.axis)) {
      im = S.mat[k];
      if (im == kMatUnknown || p.ix != ox || p.iy != oy || p.iz != oz) {
        im = MaterialAtT<TF>(J, p.ix, p.iy, p.iz);
        S.mat[k] = int8_t(im);
      }
    }
  }
  ++pst;
  S.id[k].w = pst;
  float step = 0.f, scored = 0.f, out = 0.f;
  int what = 0;
  bool score = false, moves = false, escapes = false;
  if (im < 0) {
    out = p.e + (positron ? 2.0f * kEMC2f : 0.f);
    escapes = true;
    code = 5;
  } else if (pst > kMaxElectronSteps) {
    acc += p.e + (positron ? 2.0f * kEMC2f : 0.f);
    atomicAdd(&J.cnt->lost, 1ull);
    code = 5;
  } else {
    ++nsteps;
    const float ecut = T.ecut;
    const float rho = ((TF & (kGeomPlain | kGeomSlab)) != 0) ? et.density[im] : VoxelRhoT<TF>(J, T, p.ix, p.iy, p.iz, im);
    step = s.sGeom;
    // dE/dx and 1/lambda_1 at E and at the mid-step energy, each pair from
    // one record; a step that no event shortens ends with the same mid-step
    // energy, whose dE/dx is then already at hand
    const float le = __logf(p.e);
    const DedxItr1 atE = SplinePairLe(DiOf<TF>(a, et, im), p.e, le);
    float dedx = atE.dedx * rho;
    float emid = fmaxf(p.e - 0.5f * step * dedx, ecut);
    const float lm = __logf(emid);
    const DedxItr1 atMid = SplinePairLe(DiOf<TF>(a, et, im), emid, lm);
    float dTr1 = atMid.itr1 * rho;
    const float dMol = s.invMol * et.mollerScale[im] * rho;
    const float dBrem = SplineLe(BremOf<TF>(a, et, im), emid, lm) * rho;
    const float sBrem = s.nBrem / dBrem;
    if (sBrem < step) { step = sBrem; what = 1; }
    const float sMol = s.nMol / dMol;
    if (sMol < step) { step = sMol; what = 2; }
    float sEl = s.nTr1 / dTr1;
    if (sEl < step) {
      sEl = s.nTr1 / (atE.itr1 * rho);
      emid = fmaxf(p.e - 0.5f * sEl * dedx, ecut);
      dTr1 = SplinePairLe(DiOf<TF>(a, et, im), emid, __logf(emid)).itr1 * rho;
      sEl = fminf(step, s.nTr1 / dTr1);
      step = sEl;
      what = 3;
    }
    s.nBrem = (what == 1) ? 0.f : s.nBrem - step * dBrem;
    s.nMol = (what == 2) ? 0.f : s.nMol - step * dMol;
    s.nTr1 = (what == 3) ? 0.f : s.nTr1 - step * dTr1;
    emid = fmaxf(p.e - 0.5f * step * dedx, ecut);
    dedx = SplinePairLe(DiOf<TF>(a, et, im), emid, __logf(emid)).dedx * rho;
    const float de = step * dedx;
    const float ef = p.e - de;
    if (ef < ecut) {
      // the electron stops: its energy is deposited here; a positron moves
      // to the end of the step first and annihilates there
      scored = p.e;
      p.e = 0.f;
      score = true;
      if (positron) {
        bool inside;
        if (what == 0) inside = MoveToFace(J, p, step, s.axis);
        else { p.lx += step * p.dx; p.ly += step * p.dy; p.lz += step * p.dz; inside = true; }
        const int im2 = inside ? MaterialAtT<TF>(J, p.ix, p.iy, p.iz) : -1;
        if (im2 < 0) {
          out = scored + 2.0f * kEMC2f;
          escapes = true;
          score = false;
        } else {
          PRng rng;
          SlotRng(S, k, J, p.hist, rng);
          AnnihilateF(a, p, rng, acc);
        }
      }
      code = 5;
    } else {
      p.e = ef;
      scored = de;
      score = true;
      moves = true;
    }
  }
  if (score) {
    ScoreT<TF>(J, p.meta, p.ix, p.iy, p.iz, p.hist, scored, dacc);
    acc += scored;
  }
  if (moves) {
    if (what == 0) {
      if (MoveToFace(J, p, step, s.axis)) {
        S.mat[k] = kMatUnknown;   // the voxel just entered; read when the next sub-step settles
      } else {
        out = p.e + (positron ? 2.0f * kEMC2f : 0.f);
        escapes = true;
        code = 5;
      }
    } else {
      p.lx += step * p.dx; p.ly += step * p.dy; p.lz += step * p.dz;
      code = (what == 3) ? (s.hinge ? 3 : 4) : what;
    }
  }
  if (escapes) {
    acc += out;
    esc.Add(jobs, job, double(out));
  }
  if (code == 5) {
    atomicAdd(a.histE + p.slot, acc);
    S.id[k].x = 0u;
  } else {
    S.acc[k] = acc;
    StoreStepState(S, k, p, s);
  }
  return code;
}

// GS angular deflection at the MSC hinge (SimDPMLike.cc:216-226, :731-750)
template <int TF, class SA>
__device__ __forceinline__ void EventHinge(const PhaseArgs& a, const JobF* jobs, SA& S, int k) {
  PState p;
  EState s;
  uint32_t fl;
  LoadSlot(S, k, p, s, fl);
  PRng rng;
  SlotRng(S, k, JobRec<TF>(a, jobs, JobOfSub(fl >> 8)), p.hist, rng);
  const float r2 = rng.U(), r1 = rng.U();
  float cost, sint;
  SampleGSAngle(a.T.gs, s.ekin0, r1, r2, cost, sint);
  const float phi = 2.0f * kPIf * rng.U();
  float sn, cs;
  __sincosf(phi, &sn, &cs);
  float u1 = sint * cs, u2 = sint * sn, u3 = cost;
  RotateToLab(u1, u2, u3, p.dx, p.dy, p.dz);
  const float inv = rsqrtf(u1 * u1 + u2 * u2 + u3 * u3);
  S.dir[k] = make_float4(u1 * inv, u2 * inv, u3 * inv, __uint_as_float(PackVox(p.ix, p.iy, p.iz)));
  S.mfp[k].x = s.nTr10;
  S.id[k].x = fl & ~kFHinge;
  S.rs[k].z = rng.ctr;
}

// end of an MSC step: new scattering strength and hinge (SimDPMLike.cc:227-237)
template <int TF, class SA>
__device__ __forceinline__ void EventMscEnd(const PhaseArgs& a, const ETables& et, const JobF* jobs, SA& S,
                                            int k) {
  const uint4 d = S.id[k], q = S.rs[k];
  const uint32_t fl = d.x;
  const JobF& J = JobRec<TF>(a, jobs, JobOfSub(fl >> 8));
  PRng rng;
  rng.Init(J.k0, J.k1, d.y, q.x, q.y);
  rng.ctr = q.z;
  const float e = S.pos[k].w;
  const float k1 = SplineLe(et.k1, e, __logf(e));
  const float n0 = rng.U() * k1;
  S.rs[k] = make_uint4(q.x, q.y, rng.ctr, __float_as_uint(e));   // ekin0 = e
  S.nTr10[k] = n0;
  S.mfp[k].x = k1 - n0;
  S.id[k].x = fl | kFHinge;
}

// bremsstrahlung (SimDPMLike.cc:172-194, :661-695); false when the electron
// fell below the tracking cut and finished
template <int TF, class SA>
__device__ __forceinline__ bool EventBrem(const PhaseArgs& a, const JobF* jobs, SA& S, int k,
                                         const DepthAcc& dacc) {
  PState p;
  EState s;
  uint32_t fl;
  LoadSlot(S, k, p, s, fl);
  const JobF& J = JobRec<TF>(a, jobs, JobOfSub(fl >> 8));
  const DevTables<float>& T = a.T;
  PRng rng;
  SlotRng(S, k, J, p.hist, rng);
  double acc = S.acc[k];
  const int im = S.mat[k];
  if (p.e > T.gcut && im >= 0) {
    const float r3 = rng.U(), r2 = rng.U(), r1 = rng.U();
    const float eg = SampleSB(T.sb[im], p.e, r1, r2, r3);
    const float dum0 = (kEMC2f * 0.7071067812f) / (p.e + kEMC2f);
    const float cost = fmaxf(-1.0f, fminf(1.0f, 1.0f - dum0 * dum0));
    const float sint = sqrtf(fmaxf(0.f, (1.0f + cost) * (1.0f - cost)));
    const float phi = 2.0f * kPIf * rng.U();
    float sn, cs;
    __sincosf(phi, &sn, &cs);
    PState g = p;
    g.e = eg; g.meta = 0u | (p.meta & ~3u);
    g.dx = sint * cs; g.dy = sint * sn; g.dz = cost;
    RotateToLab(g.dx, g.dy, g.dz, p.dx, p.dy, p.dz);
    rng.Child(0, g.ulo, g.uhi);
    if (!Append(a.outP, a.outPCount, a.overflow, g)) acc += eg;
    p.e -= eg;
  }
  if (p.e < T.ecut) {
    ScoreT<TF>(J, p.meta, p.ix, p.iy, p.iz, p.hist, p.e, dacc);
    acc += p.e;
    if ((fl & kFPositron) != 0) AnnihilateF(a, p, rng, acc);
    atomicAdd(a.histE + p.slot, acc);
    S.id[k].x = 0u;
    return false;
  }
  S.pos[k].w = p.e;
  S.mfp[k].w = -__logf(rng.U());
  S.acc[k] = acc;
  S.rs[k].z = rng.ctr;
  return true;
}

// Moller delta electron (SimDPMLike.cc:204-214, :699-728)
template <int TF, class SA>
__device__ __forceinline__ void EventMoller(const PhaseArgs& a, const ETables& et, const JobF* jobs, SA& S,
                                            int k) {
  PState p;
  EState s;
  uint32_t fl;
  LoadSlot(S, k, p, s, fl);
  const JobF& J = JobRec<TF>(a, jobs, JobOfSub(fl >> 8));
  PRng rng;
  SlotRng(S, k, J, p.hist, rng);
  double acc = S.acc[k];
  if (p.e > 2.0f * a.T.ecut) {
    const float r3 = rng.U(), r2 = rng.U(), r1 = rng.U();
    const float se = SampleMoller(a.T.mol, p.e, r1, r2, r3);
    const float k2 = 2.0f * kEMC2f;
    const float cost = fminf(1.0f, sqrtf(se * (p.e + k2) / (p.e * (se + k2))));
    const float sint = sqrtf(fmaxf(0.f, (1.0f + cost) * (1.0f - cost)));
    const float phi = 2.0f * kPIf * rng.U();
    float sn, cs;
    __sincosf(phi, &sn, &cs);
    PState c = p;
    c.e = se; c.meta = 1u | (p.meta & ~3u);
    c.dx = sint * cs; c.dy = sint * sn; c.dz = cost;
    RotateToLab(c.dx, c.dy, c.dz, p.dx, p.dy, p.dz);
    rng.Child(0, c.ulo, c.uhi);
    if (!Append(a.outE, a.outECount, a.overflow, c)) acc += se;
    p.e -= se;
  }
  S.pos[k].w = p.e;
  const float nMol = -__logf(rng.U());
  S.mfp[k] = make_float4(s.nTr1, nMol, SplineLe(et.moller, p.e, __logf(p.e)), s.nBrem);
  S.acc[k] = acc;
  S.rs[k].z = rng.ctr;
}

// first sub-step state of a claimed work item (a primary or a queued
// electron) in slot k; false when it starts outside the phantom
template <int TF, class SA>
__device__ __forceinline__ bool RefillSlot(const PhaseArgs& a, const ETables& et, const JobF* jobs,
                                           const unsigned long long* spre, SA& S, int k,
                                           unsigned long long item, EscTally& esc) {
  PState p;
  PRng rng;
  if (item < (unsigned long long)a.nPrimaries) {
    MakePrimary(a, a.segs, (long long)item, p, rng);
  } else {
    LoadParticle(a.in, StripedIndex(a.in, spre, item - a.nPrimaries), p);
    const JobF& J = JobRec<TF>(a, jobs, JobOfSub(p.meta >> 2));
    rng.Init(J.k0, J.k1, p.hist, p.ulo, p.uhi);
  }
  const int job = JobOfSub(p.meta >> 2);
  const JobF& J = JobRec<TF>(a, jobs, job);
  const int im0 = InBox(J, p.ix, p.iy, p.iz) ? MaterialAtT<TF>(J, p.ix, p.iy, p.iz) : -1;
  if (im0 < 0) {
    const double out = p.e + ((p.meta & 3u) == 2u ? 2.0 * kEMC2f : 0.0);
    esc.Add(jobs, job, out);
    atomicAdd(a.histE + p.slot, out);
    return false;
  }
  EState s;
  InitElectron(et, p, rng, s);
  StoreSlot(S, k, p, s, rng.ctr);
  S.acc[k] = 0.0;
  S.mat[k] = int8_t(im0);
  return true;
}

// TF: form flags (kTallyAgg, kTallyPlain, kGeomPlain, kSingleJob); NS: slots per block
template <int TF, int NS>
__global__ void __launch_bounds__(kBlockThreads, kBlockMinBlocks) ElectronPhaseB(PhaseArgs a) {
  using SlotArrays = SlotArraysT<NS>;
  extern __shared__ __align__(16) unsigned char dyn[];
  SlotArrays& S = *reinterpret_cast<SlotArrays*>(dyn);
  SlotRings& R = *reinterpret_cast<SlotRings*>(dyn + sizeof(SlotArrays));
  float* sdata = reinterpret_cast<float*>(dyn + BlockPhaseStaticBytes<NS>());
  __shared__ ETables et;
  __shared__ JobF sjobs[16];
  __shared__ unsigned long long spre[kStripes + 1];
  const bool fewJobs = a.njobs <= 16;
  if (fewJobs)
    for (int j = threadIdx.x; j < a.njobs; j += blockDim.x) sjobs[j] = a.jobs[j];
  const DepthAcc dacc = DepthAccInit(a, dyn + BlockPhaseSmemBytesFor<NS>(a.T, 0));
  const unsigned long long nQ = StripePrefix(a.inCount, spre);
  const JobF* jobs = fewJobs ? sjobs : a.jobs;
  const unsigned long long total = (unsigned long long)a.nPrimaries + nQ;
  if (total == 0) return;   // an empty generation skips the table staging
  if (kTablesInSmem) StageElectronTables(a.T, sdata, &et);
  else if (threadIdx.x == 0) BindElectronTables(a.T, &et);   // visible after the barrier below
  const int tid = threadIdx.x, lane = tid & 31;
  RingsInit(R, kRIdle, NS);
  for (int k = tid; k < NS; k += blockDim.x) S.id[k] = make_uint4(0u, 0u, 0u, 0u);
  __syncthreads();
  volatile int* vexh = &R.exhausted;
  EscTally esc;
  unsigned long long nsteps = 0;
  bool gaveUp = false;
  for (;;) {
    int n = 0, k = 0;
    const int ring = RingTake(R, lane, n, k, gaveUp);
    if (ring < 0) break;
    const bool have = lane < n;
    bool live = have;
    switch (ring) {   // the same on every lane
      case kRHinge:
        if (have) EventHinge<TF>(a, jobs, S, k);
        break;
      case kRMscEnd:
        if (have) EventMscEnd<TF>(a, et, jobs, S, k);
        break;
      case kRBrem:
        if (have) live = EventBrem<TF>(a, jobs, S, k, dacc);
        break;
      case kRMoller:
        if (have) EventMoller<TF>(a, et, jobs, S, k);
        break;
      case kRIdle:
        live = false;
        if (have && *vexh == 0) {
          // one claim on the work counter per warp
          cg::coalesced_group g = cg::coalesced_threads();
          unsigned long long base = 0;
          if (g.thread_rank() == 0) base = atomicAdd(a.head, (unsigned long long)g.size());
          base = g.shfl(base, 0);
          const unsigned long long item = base + g.thread_rank();
          if (base + g.size() >= total) *vexh = 1;
          if (item < total) live = RefillSlot<TF>(a, et, jobs, spre, S, k, item, esc);
        }
        break;
      default:
        break;
    }
    // a slot that keeps stepping takes a second sub-step before it goes back
    // to a ring when at least kSecondStepLanes lanes of the warp do (one call
    // site; lanes whose slot had an event wait). With fewer, they go back to
    // the step ring and join a fuller warp.
    int code = live ? 0 : 5;
    for (int rep = 0; rep < 2 && (rep == 0 ? __any_sync(kFull, code == 0)
                                           : __popc(__ballot_sync(kFull, code == 0)) >= kSecondStepLanes);
         ++rep)
      if (code == 0) code = StepSlot<TF>(a, et, jobs, S, k, esc, nsteps, dacc);
    // the ring of the slot's next action; a finished slot goes back to the
    // idle ring while there is work left, else it retires (q == kRings)
    int q = -1;
    if (have) {
      q = int((kRingOfCode >> (4 * code)) & 15u);
      if (q == kRIdle && *vexh != 0) q = kRings;
    }
    RingPut(R, lane, q, k, gaveUp);
    if (gaveUp) break;
  }
  // a warp that gave up a wait leaves electrons unfinished: reported
  if (gaveUp && lane == 0) atomicAdd(a.fault, 1ull);
  esc.Flush(jobs);
  DepthAccFlush(a, jobs, dacc);
  for (int o = 16; o > 0; o >>= 1) nsteps += __shfl_down_sync(kFull, nsteps, o);
  if (lane == 0 && a.njobs > 0) atomicAdd(&a.jobs[0].cnt->steps, nsteps);
}

// ---------------------------------------------------------------------------
// photon phase, block-batched: kPSlots photons per block live in shared
// memory with their random-number state, each waiting on one of four rings
// (Compton, pair, refill, plain step); a warp takes up to 32 slots of one ring,
// runs that interaction or the refill, then one Woodcock step on them, as in
// the electron phase. The uniforms are drawn in the order of PhotonPhase, so
// both kernels give the same histories.
// ---------------------------------------------------------------------------
// 3 blocks of 448 slots: 80 registers a thread (4 blocks of 352 slots: 64,
// with spills) and 1344 photons per SM; the photon phase 1.4 % faster
constexpr int kPSlots = 448;
constexpr int kPhotonStepsPerTake = 3;   // Woodcock steps a photon takes per turn while they are delta steps
constexpr int kPBlockMinBlocks = 3;
constexpr int kPBlockThreads = 256;   // threads per block (a multiple of 32)

// shared-memory state of the resident photons, in 16-byte records
struct PSlotArrays {
  float4 pos[kPSlots];   // offset in the voxel lx, ly, lz; energy
  float4 dir[kPSlots];   // direction dx, dy, dz; voxel (PackVox, as float bits)
  uint4 id[kPSlots];     // meta (type, sub-job), history, energy-check slot, steps taken
  uint4 rs[kPSlots];     // random stream uid lo, uid hi, counter, buffered words left
  uint4 w[kPSlots];      // the buffered Philox words
  double acc[kPSlots];
};
// photon rings (of equally full rings the first is taken)
enum : int { kPRComp, kPRPair, kPRIdle, kPRStep, kPRings };
static_assert(kPSlots <= kRingSize, "a ring holds every slot");
// ring of a Woodcock step's result code (0 step, 1 Compton, 2 pair, 3 finished)
constexpr uint32_t kPRingOfCode = 0x2103u;
using PSlotRings = Rings<kPRings>;

__host__ __device__ constexpr size_t PhotonBlockStaticBytes() { return sizeof(PSlotArrays) + sizeof(PSlotRings); }

__device__ __forceinline__ void LoadPhoton(const PSlotArrays& S, int k, const JobF* jobs, PState& p, PRng& rng) {
  const float4 a = S.pos[k], b = S.dir[k];
  const uint4 d = S.id[k], q = S.rs[k];
  p.lx = a.x; p.ly = a.y; p.lz = a.z; p.e = a.w;
  p.dx = b.x; p.dy = b.y; p.dz = b.z;
  UnpackVox(__float_as_uint(b.w), p);
  p.meta = d.x; p.hist = d.y; p.slot = d.z; p.ulo = q.x; p.uhi = q.y;
  const JobF& J = jobs[JobOfSub(p.meta >> 2)];
  rng.Init(J.k0, J.k1, p.hist, p.ulo, p.uhi);
  rng.ctr = q.z;
  rng.have = int(q.w);
  rng.w = S.w[k];
}

__device__ __forceinline__ void StorePhoton(PSlotArrays& S, int k, const PState& p, const PRng& rng) {
  S.pos[k] = make_float4(p.lx, p.ly, p.lz, p.e);
  S.dir[k] = make_float4(p.dx, p.dy, p.dz, __uint_as_float(PackVox(p.ix, p.iy, p.iz)));
  S.rs[k] = make_uint4(p.ulo, p.uhi, rng.ctr, uint32_t(rng.have));
  S.w[k] = rng.w;
}

// Woodcock steps of slot k (SimDPMLike.cc:471-508), up to kPhotonStepsPerTake
// while they are delta steps: 0 delta step, 1 Compton, 2 pair, 3 finished
// (escaped, absorbed, or over the step cap)
template <int TF>
__device__ __forceinline__ int PhotonStepSlot(const PhaseArgs& a, const PTables& pt, const JobF* jobs, PSlotArrays& S,
                                              int k, EscTally& esc, unsigned long long& nph, const DepthAcc& dacc) {
  const DevTables<float>& T = a.T;
  PState p;
  PRng rng;
  LoadPhoton(S, k, jobs, p, rng);
  const int job = JobOfSub(p.meta >> 2);
  const JobF& J = jobs[job];
  double acc = S.acc[k];
  int code = 0;
  uint32_t pst = S.id[k].w;
  // the majorant IMFP at the photon's energy, which delta steps keep
  const float lmax = 1.0f / (LinearGet(pt.imfpMax, p.e) * J.wscale);
#pragma unroll 1
  for (int it = 0; it < kPhotonStepsPerTake && code == 0; ++it) {
    if (++pst > kMaxPhotonSteps) {   // cannot happen for finite cross sections; bounded anyway
      acc += p.e;
      atomicAdd(&J.cnt->lost, 1ull);
      code = 3;
    } else {
      ++nph;
      const float step = -lmax * __logf(rng.U());
      int im = -1;
      if (Fly(J, p, step)) im = MaterialAtT<TF>(J, p.ix, p.iy, p.iz);
      if (im < 0) {
        acc += p.e;
        esc.Add(jobs, job, double(p.e));
        code = 3;
      } else {
        const float rho = VoxelRhoT<TF>(J, T, p.ix, p.iy, p.iz, im);
        const float r1 = rng.U();
        float prob = 1.0f - LinearGet(pt.tot[im], p.e) * rho * lmax;
        if (r1 >= prob) {
          prob += LinearGet(pt.comp[im], p.e) * rho * lmax;
          if (r1 < prob) {
            code = 1;
          } else {
            prob += LinearGet(pt.pair[im], p.e) * rho * lmax;
            if (r1 < prob && p.e > 2.0f * kEMC2f) {
              code = 2;
            } else {
              // photoelectric absorption (also below the pair threshold)
              ScoreT<TF>(J, p.meta, p.ix, p.iy, p.iz, p.hist, p.e, dacc);
              acc += p.e;
              code = 3;
            }
          }
        }
      }
    }
  }
  S.id[k].w = pst;
  if (code == 3) {
    atomicAdd(a.histE + p.slot, acc);
  } else {
    S.acc[k] = acc;
    StorePhoton(S, k, p, rng);
  }
  return code;
}

// Compton scattering at the slot's position (SimDPMLike.cc:512-570); false
// when the scattered photon falls below the cut and is absorbed
template <int TF>
__device__ __forceinline__ bool PhotonComptonSlot(const PhaseArgs& a, const JobF* jobs, PSlotArrays& S, int k,
                                                  const DepthAcc& dacc) {
  const DevTables<float>& T = a.T;
  PState p;
  PRng rng;
  LoadPhoton(S, k, jobs, p, rng);
  const JobF& J = jobs[JobOfSub(p.meta >> 2)];
  double acc = S.acc[k];
  const float a3 = rng.U(), a2 = rng.U(), a1 = rng.U();
  const float eps = SampleKN(T.kn, p.e, a1, a2, a3);
  const float kappa = p.e * (1.0f / kEMC2f);
  const float phCost = 1.0f - (1.0f - eps) / (eps * kappa);
  const float phE = eps * p.e;
  const float phPhi = 2.0f * kPIf * rng.U();
  const float elE = p.e - phE;
  float sn, cs;
  __sincosf(phPhi, &sn, &cs);
  if (elE < T.ecut) {
    ScoreT<TF>(J, p.meta, p.ix, p.iy, p.iz, p.hist, elE, dacc);
    acc += elE;
  } else {
    const float e0 = kappa;
    const float elCost = (1.0f + e0) * sqrtf((1.0f - eps) / (e0 * (2.0f + e0 * (1.0f - eps))));
    const float sint = sqrtf(fmaxf(0.f, (1.0f + elCost) * (1.0f - elCost)));
    PState c = p;
    c.dx = -sint * cs; c.dy = -sint * sn; c.dz = elCost;   // phi + pi
    RotateToLab(c.dx, c.dy, c.dz, p.dx, p.dy, p.dz);
    c.e = elE;
    c.meta = 1u | (p.meta & ~3u);
    rng.Child(0, c.ulo, c.uhi);
    if (!Append(a.outE, a.outECount, a.overflow, c)) acc += elE;
  }
  p.e = phE;
  if (p.e < T.gcut) {
    ScoreT<TF>(J, p.meta, p.ix, p.iy, p.iz, p.hist, p.e, dacc);
    acc += p.e;
    atomicAdd(a.histE + p.slot, acc);
    return false;
  }
  const float phSint = sqrtf(fmaxf(0.f, (1.0f - phCost) * (1.0f + phCost)));
  float u1 = phSint * cs, u2 = phSint * sn, u3 = phCost;
  RotateToLab(u1, u2, u3, p.dx, p.dy, p.dz);
  p.dx = u1; p.dy = u2; p.dz = u3;
  S.acc[k] = acc;
  StorePhoton(S, k, p, rng);
  return true;
}

// pair production at the slot's position (SimDPMLike.cc:573-627); the photon ends
template <int TF>
__device__ __forceinline__ void PhotonPairSlot(const PhaseArgs& a, const JobF* jobs, PSlotArrays& S, int k,
                                               const DepthAcc& dacc) {
  const DevTables<float>& T = a.T;
  PState p;
  PRng rng;
  LoadPhoton(S, k, jobs, p, rng);
  const JobF& J = jobs[JobOfSub(p.meta >> 2)];
  double acc = S.acc[k];
  const float sum = p.e - 2.0f * kEMC2f;
  const float e1 = rng.U() * sum;
  const float e2 = sum - e1;
  if (e2 < T.ecut) {
    ScoreT<TF>(J, p.meta, p.ix, p.iy, p.iz, p.hist, e2, dacc);
    acc += e2;
  } else {
    PState c = p;
    c.e = e2; c.meta = 1u | (p.meta & ~3u);
    rng.Child(0, c.ulo, c.uhi);
    if (!Append(a.outE, a.outECount, a.overflow, c)) acc += e2;
  }
  if (e1 < T.ecut) {
    ScoreT<TF>(J, p.meta, p.ix, p.iy, p.iz, p.hist, e1, dacc);
    acc += e1;
    AnnihilateF(a, p, rng, acc);   // at rest (SimDPMLike.cc:753-791)
  } else {
    PState c = p;
    c.e = e1; c.meta = 2u | (p.meta & ~3u);
    rng.Child(1, c.ulo, c.uhi);
    if (!Append(a.outE, a.outECount, a.overflow, c)) acc += e1 + 2.0f * kEMC2f;
  }
  atomicAdd(a.histE + p.slot, acc);
}

// a new photon (primary or queued) in slot k; false when it starts outside
template <int TF>
__device__ __forceinline__ bool PhotonRefillSlot(const PhaseArgs& a, const JobF* jobs,
                                                 const unsigned long long* spre, PSlotArrays& S, int k,
                                                 unsigned long long item, EscTally& esc) {
  PState p;
  PRng rng;
  if (item < (unsigned long long)a.nPrimaries) {
    MakePrimary(a, a.segs, (long long)item, p, rng);
  } else {
    LoadParticle(a.in, StripedIndex(a.in, spre, item - a.nPrimaries), p);
    const JobF& J = jobs[JobOfSub(p.meta >> 2)];
    rng.Init(J.k0, J.k1, p.hist, p.ulo, p.uhi);
  }
  const JobF& J = jobs[JobOfSub(p.meta >> 2)];
  if (!InBox(J, p.ix, p.iy, p.iz) || MaterialAtT<TF>(J, p.ix, p.iy, p.iz) < 0) {
    esc.Add(jobs, JobOfSub(p.meta >> 2), double(p.e));
    atomicAdd(a.histE + p.slot, double(p.e));
    return false;
  }
  S.id[k] = make_uint4(p.meta, p.hist, p.slot, 0u);
  S.acc[k] = 0.0;
  StorePhoton(S, k, p, rng);
  return true;
}

// TF: form flags (kTallyAgg, kTallyPlain, kGeomPlain)
template <int TF>
__global__ void __launch_bounds__(kPBlockThreads, kPBlockMinBlocks) PhotonPhaseB(PhaseArgs a) {
  extern __shared__ __align__(16) unsigned char dyn[];
  PSlotArrays& S = *reinterpret_cast<PSlotArrays*>(dyn);
  PSlotRings& R = *reinterpret_cast<PSlotRings*>(dyn + sizeof(PSlotArrays));
  __shared__ JobF sjobs[16];
  __shared__ unsigned long long spre[kStripes + 1];
  __shared__ PTables pt;
  const bool fewJobs = a.njobs <= 16;
  if (fewJobs)
    for (int j = threadIdx.x; j < a.njobs; j += blockDim.x) sjobs[j] = a.jobs[j];
  const unsigned long long nQ = StripePrefix(a.inCount, spre);
  const JobF* jobs = fewJobs ? sjobs : a.jobs;
  const unsigned long long total = (unsigned long long)a.nPrimaries + nQ;
  if (total == 0) return;
  StagePhotonTables(a.T, false, nullptr, &pt);
  const DepthAcc dacc = DepthAccInit(a, dyn + ((PhotonBlockStaticBytes() + 15) & ~size_t(15)));
  const int tid = threadIdx.x, lane = tid & 31;
  RingsInit(R, kPRIdle, kPSlots);
  __syncthreads();
  volatile int* vexh = &R.exhausted;
  EscTally esc;
  unsigned long long nph = 0;
  bool gaveUp = false;
  for (;;) {
    int n = 0, k = 0;
    const int ring = RingTake(R, lane, n, k, gaveUp);
    if (ring < 0) break;
    const bool have = lane < n;
    bool live = have;
    if (ring == kPRComp) {
      if (have) live = PhotonComptonSlot<TF>(a, jobs, S, k, dacc);
    } else if (ring == kPRPair) {
      if (have) PhotonPairSlot<TF>(a, jobs, S, k, dacc);
      live = false;
    } else if (ring == kPRIdle) {
      live = false;
      if (have && *vexh == 0) {
        cg::coalesced_group g = cg::coalesced_threads();
        unsigned long long base = 0;
        if (g.thread_rank() == 0) base = atomicAdd(a.head, (unsigned long long)g.size());
        base = g.shfl(base, 0);
        const unsigned long long item = base + g.thread_rank();
        if (base + g.size() >= total) *vexh = 1;
        if (item < total) live = PhotonRefillSlot<TF>(a, jobs, spre, S, k, item, esc);
      }
    }
    const int code = live ? PhotonStepSlot<TF>(a, pt, jobs, S, k, esc, nph, dacc) : 3;
    int q = -1;
    if (have) {
      q = int((kPRingOfCode >> (4 * code)) & 15u);
      if (q == kPRIdle && *vexh != 0) q = kPRings;
    }
    RingPut(R, lane, q, k, gaveUp);
    if (gaveUp) break;
  }
  // a warp that gave up a wait leaves photons unfinished: reported
  if (gaveUp && lane == 0) atomicAdd(a.fault, 1ull);
  esc.Flush(jobs);
  DepthAccFlush(a, jobs, dacc);
  for (int o = 16; o > 0; o >>= 1) nph += __shfl_down_sync(kFull, nph, o);
  if (lane == 0 && a.njobs > 0) atomicAdd(&a.jobs[0].cnt->photonSteps, nph);
}

__global__ void FoldKernel(double* t, double* dose, double* dose2, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = t[i];
    if (v != 0.0) {
      dose[i] += v;
      dose2[i] += v * v;
      t[i] = 0.0;
    }
  }
}

// adds the m batch slices of each bin to dose and dose^2 (slices in order);
// ZERO: clears the slices for the next batch group (the last group's slices
// are cleared by the next run's memset: without the stores the loads of a
// bin's slices overlap, 0.26 against 0.33 ms for 10 slices of 4.2 M bins)
template <bool ZERO>
__global__ void FoldSlicesKernel(double* t, double* dose, double* dose2, long long n, long long binStride,
                                 long long sliceStride, int m) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double* ti = t + i * binStride;
    double s = 0.0, s2 = 0.0;
    bool any = false;
    for (int b = 0; b < m; ++b) {
      const double v = ti[b * sliceStride];
      if (v != 0.0) {
        s += v;
        s2 += v * v;
        if (ZERO) ti[b * sliceStride] = 0.0;
        any = true;
      }
    }
    if (any) {
      dose[i] += s;
      dose2[i] += s2;
    }
  }
}

__global__ void __launch_bounds__(256) TallySummaryKernel(const double* d, long long n, double* sum,
                                                          unsigned long long* lastNz) {
  __shared__ double ws[8];
  __shared__ unsigned long long wl[8];
  double s = 0.0;
  unsigned long long last = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = d[i];
    s += v;
    if (v != 0.0) last = (unsigned long long)i + 1;
  }
  cg::thread_block_tile<32> w = cg::tiled_partition<32>(cg::this_thread_block());
  s = cg::reduce(w, s, cg::plus<double>());
  last = cg::reduce(w, last, cg::greater<unsigned long long>());
  if (w.thread_rank() == 0) { ws[threadIdx.x >> 5] = s; wl[threadIdx.x >> 5] = last; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < int(blockDim.x >> 5); ++k) { s += ws[k]; last = last > wl[k] ? last : wl[k]; }
    atomicAdd(sum, s);
    atomicMax(lastNz, last);
  }
}

__global__ void EnergyCheckKernel(const double* histE, const double* histE0, long long nslots, const Segment* segs,
                                  int nsegs, const JobF* jobs) {
  // per-thread sums for the current job's counters (the batches of a job
  // share them), flushed when they change; the final flush is reduced over
  // the lanes of a warp that share the counters
  RunCounters* cur = nullptr;
  double se0 = 0.0, mres = 0.0;
  unsigned long long nh = 0, nv = 0;
  auto flush = [&](RunCounters* c) {
    if (nh) {
      atomicAdd(&c->primaryEnergy, se0);
      atomicAdd(&c->histories, nh);
      atomicMax(&c->maxResidualBits, (unsigned long long)__double_as_longlong(mres));
      if (nv) atomicAdd(&c->violations, nv);
    }
    se0 = mres = 0.0;
    nh = nv = 0;
  };
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nslots;
       i += (long long)gridDim.x * blockDim.x) {
    // slots are laid out segment after segment
    int lo = 0, hi = nsegs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (segs[mid].slotBase <= i) lo = mid; else hi = mid - 1;
    }
    RunCounters* c = jobs[JobOfSub(uint32_t(segs[lo].job))].cnt;
    if (c != cur) {
      if (cur) flush(cur);
      cur = c;
    }
    const double e0 = histE0[i];
    const double res = fabs(e0 - histE[i]);
    se0 += e0;
    ++nh;
    mres = fmax(mres, res);
    if (res > 1.0e-3 * e0) ++nv;
  }
  cg::coalesced_group g = cg::coalesced_threads();
  cg::coalesced_group peers = cg::labeled_partition(g, (unsigned long long)cur);
  se0 = cg::reduce(peers, se0, cg::plus<double>());
  nh = cg::reduce(peers, nh, cg::plus<unsigned long long>());
  nv = cg::reduce(peers, nv, cg::plus<unsigned long long>());
  mres = cg::reduce(peers, mres, cg::greater<double>());
  if (peers.thread_rank() == 0 && cur) flush(cur);
}

__global__ void SamplerKernel32(DevTables<float> T, int s, int imat, const double* e, const double* r, double* out,
                                int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ei = float(e[i]);
  const float u0 = float(r[3 * i]), u1 = float(r[3 * i + 1]), u2 = float(r[3 * i + 2]);
  float v = 0.f;
  switch (s) {
    case 0: v = SampleKN(T.kn, ei, u0, u1, u2); break;
    case 1: v = SampleMoller(T.mol, ei, u0, u1, u2); break;
    case 2: v = SampleSB(T.sb[imat], ei, u0, u1, u2); break;
    case 3: v = SampleGS(T.gs, ei, u0, u1); break;
    default: break;
  }
  out[i] = double(v);
}

__global__ void TableKernel32(DevTables<float> T, int q, int imat, const double* e, double* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ei = float(e[i]);
  const float le = __logf(ei);
  float v = 0.f;
  switch (q) {
    case 0: v = SplineLe(T.dedx[imat], ei, le); break;
    case 1: v = SplineLe(T.itr1[imat], ei, le); break;
    case 2: v = SplineLe(T.brem[imat], ei, le); break;
    case 3: v = SplineLe(T.moller, ei, le); break;
    case 4: v = SplineLe(T.k1, ei, le); break;
    case 5: v = LinearGet(T.imfpMax, ei); break;
    case 6: v = LinearGet(T.tot[imat], ei); break;
    case 7: v = LinearGet(T.comp[imat], ei); break;
    case 8: v = LinearGet(T.pair[imat], ei); break;
    default: break;
  }
  out[i] = double(v);
}

// Self-test of the slot rings (one independent run per block): slots
// 0 .. nslots - 1 start on ring 0; a warp that takes a slot counts a visit
// and puts it on the ring picked by a hash of (seed, slot, visit), until the
// slot has `rounds` visits and retires. out[0] += visits, out[1] += slots
// whose visit count is not `rounds`, out[2] += warps that gave up a wait,
// out[3] += blocks whose probe wait on a cell nothing fills gave up after
// `probeCycles` (as it must).
__global__ void __launch_bounds__(256) RingSelfTestKernel(int nslots, int rounds, uint32_t seed, long long probeCycles,
                                                          unsigned long long* out) {
  __shared__ Rings<4> R;
  __shared__ unsigned int visits[kRingSize];
  __shared__ uint16_t probe;
  const int lane = threadIdx.x & 31;
  RingsInit(R, 0, nslots);
  for (int k = threadIdx.x; k < kRingSize; k += blockDim.x) visits[k] = 0u;
  if (threadIdx.x == 0) probe = uint16_t(CellEmpty(0));
  __syncthreads();
  bool gaveUp = false;
  unsigned long long taken = 0;
  for (;;) {
    int n = 0, k = 0;
    const int ring = RingTake(R, lane, n, k, gaveUp);
    if (ring < 0) break;
    int q = -1;
    if (lane < n) {
      const unsigned v = atomicAdd(&visits[k], 1u) + 1u;
      ++taken;
      uint32_t h = seed ^ (uint32_t(k) * 0x9E3779B1u) ^ (v * 0x85EBCA77u);
      h ^= h >> 15;
      h *= 0x2C1B3C6Du;
      h ^= h >> 12;
      q = v >= unsigned(rounds) ? 4 : int(h & 3u);
    }
    RingPut(R, lane, q, k, gaveUp);
    if (gaveUp) break;
  }
  __syncthreads();
  unsigned long long bad = 0;
  for (int k = threadIdx.x; k < nslots; k += blockDim.x) bad += visits[k] != unsigned(rounds);
  for (int o = 16; o > 0; o >>= 1) {
    taken += __shfl_down_sync(kFull, taken, o);
    bad += __shfl_down_sync(kFull, bad, o);
  }
  if (lane == 0) {
    atomicAdd(out, taken);
    atomicAdd(out + 1, bad);
    if (gaveUp) atomicAdd(out + 2, 1ull);
  }
  if (threadIdx.x == 0) {
    uint32_t v;
    if (!CellWait(&probe, CellFull(0), ~kCellSlot, v, probeCycles)) atomicAdd(out + 3, 1ull);
  }
}

}  // namespace

int ElectronPhaseSmemBytes(const DevTables<float>& T) { return int(T.elecCount * sizeof(float)); }

// template flags of the block kernels a run's phase arguments select: 0 or
// kTallyAgg (the general forms), kTallyPlain, kTallyPlain | kGeomPlain,
// kTallyDepth | kGeomSlab, kTallyTag | kGeomPlain (warp aggregation,
// measured slower on every workload, is built for the general form only)
static int KernelForm(const PhaseArgs& a) {
  if (a.aggregate) return kTallyAgg;
  if (a.slabForm) return kTallyDepth | kGeomSlab;
  if (a.tagForm) return a.plainGeom ? (kTallyTag | kGeomPlain) : 0;
  if (!a.plainTally) return 0;
  return a.plainGeom ? (kTallyPlain | kGeomPlain) : kTallyPlain;
}

// dynamic shared memory of the block-batched photon phase
__host__ __device__ inline size_t PhotonBlockSmemBytes(int depthBins) {
  return ((PhotonBlockStaticBytes() + 15) & ~size_t(15)) + DepthAccBytes(depthBins);
}

cudaError_t PreparePhotonPhase(const DevTables<float>& T) {
  cudaError_t e = cudaFuncSetAttribute(PhotonPhase, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(PhotonTableBytes(T) + DepthAccBytes(kDepthBins)));
  const int sb = int(PhotonBlockSmemBytes(kDepthBins));
  if (e == cudaSuccess) e = cudaFuncSetAttribute(PhotonPhaseB<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(PhotonPhaseB<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(PhotonPhaseB<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(PhotonPhaseB<6>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(PhotonPhaseB<48>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(PhotonPhaseB<68>, cudaFuncAttributeMaxDynamicSharedMemorySize, sb);
  return e;
}

int PhotonBlockBlocksPerSM() { return kPBlockMinBlocks; }

cudaError_t LaunchPhotonPhaseBlock(const PhaseArgs& a, int blocks, cudaStream_t st) {
  const size_t smem = PhotonBlockSmemBytes(a.depthBins);
  switch (KernelForm(a)) {
    case 1: PhotonPhaseB<1><<<blocks, kPBlockThreads, smem, st>>>(a); break;
    case 2: PhotonPhaseB<2><<<blocks, kPBlockThreads, smem, st>>>(a); break;
    case 6: PhotonPhaseB<6><<<blocks, kPBlockThreads, smem, st>>>(a); break;
    case 48: PhotonPhaseB<48><<<blocks, kPBlockThreads, smem, st>>>(a); break;
    case 68: PhotonPhaseB<68><<<blocks, kPBlockThreads, smem, st>>>(a); break;
    default: PhotonPhaseB<0><<<blocks, kPBlockThreads, smem, st>>>(a); break;   // the general form
  }
  return cudaGetLastError();
}

cudaError_t LaunchPhotonPhase(const PhaseArgs& a, int blocks, int threads, cudaStream_t st) {
  PhotonPhase<<<blocks, threads, PhotonTableBytes(a.T) + DepthAccBytes(a.depthBins), st>>>(a);
  return cudaGetLastError();
}

int BlockPhaseSmemBytes(const DevTables<float>& T) { return int(BlockPhaseSmemBytesFor<kSlots>(T, kDepthBins)); }

int BlockPhaseBlocksPerSM() { return kBlockMinBlocks; }

int BlockPhaseSlots(int requested) { return requested == kSlotsSmall ? kSlotsSmall : kSlots; }

template <int NS>
static cudaError_t PrepareBlockPhaseFor(const DevTables<float>& T) {
  const int smem = int(BlockPhaseSmemBytesFor<NS>(T, kDepthBins));
  cudaError_t e = cudaFuncSetAttribute(ElectronPhaseB<0, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<1, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<2, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<6, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<48, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<68, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if constexpr (NS == kSlots) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<8, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<10, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<14, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<56, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(ElectronPhaseB<76, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  }
  return e;
}

cudaError_t PrepareBlockPhase(const DevTables<float>& T) {
  const cudaError_t e = PrepareBlockPhaseFor<kSlots>(T);
  return e != cudaSuccess ? e : PrepareBlockPhaseFor<kSlotsSmall>(T);
}

template <int NS>
static void LaunchElectronPhaseBlockFor(const PhaseArgs& a, int blocks, cudaStream_t st) {
  const size_t smem = BlockPhaseSmemBytesFor<NS>(a.T, a.depthBins);
  // the single-job forms are built for the default slot count
  const int f = KernelForm(a) | ((NS == kSlots && a.soloJob && !a.aggregate) ? kSingleJob : 0);
  switch (f) {
    case 1: ElectronPhaseB<1, NS><<<blocks, kBlockThreads, smem, st>>>(a); break;
    case 2: ElectronPhaseB<2, NS><<<blocks, kBlockThreads, smem, st>>>(a); break;
    case 6: ElectronPhaseB<6, NS><<<blocks, kBlockThreads, smem, st>>>(a); break;
    case 8: ElectronPhaseB<8, kSlots><<<blocks, kBlockThreads, smem, st>>>(a); break;
    case 10: ElectronPhaseB<10, kSlots><<<blocks, kBlockThreads, smem, st>>>(a); break;
    case 14: ElectronPhaseB<14, kSlots><<<blocks, kBlockThreads, smem, st>>>(a); break;
    case 48: ElectronPhaseB<48, NS><<<blocks, kBlockThreads, smem, st>>>(a); break;
    case 56: ElectronPhaseB<56, kSlots><<<blocks, kBlockThreads, smem, st>>>(a); break;
    case 68: ElectronPhaseB<68, NS><<<blocks, kBlockThreads, smem, st>>>(a); break;
    case 76: ElectronPhaseB<76, kSlots><<<blocks, kBlockThreads, smem, st>>>(a); break;
    default: ElectronPhaseB<0, NS><<<blocks, kBlockThreads, smem, st>>>(a); break;   // the general form
  }
}

cudaError_t LaunchElectronPhaseBlock(const PhaseArgs& a, int blocks, int slots, cudaStream_t st) {
  if (BlockPhaseSlots(slots) == kSlotsSmall) LaunchElectronPhaseBlockFor<kSlotsSmall>(a, blocks, st);
  else LaunchElectronPhaseBlockFor<kSlots>(a, blocks, st);
  return cudaGetLastError();
}

cudaError_t LaunchElectronPhase(const PhaseArgs& a, int blocks, int threads, cudaStream_t st) {
  const int smem = ElectronPhaseSmemBytes(a.T);
  ElectronPhase<<<blocks, threads, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t LaunchFold(double* t, double* dose, double* dose2, long long n, cudaStream_t st) {
  const int blocks = int(std::min<long long>((n + 255) / 256, 152LL * 16));
  FoldKernel<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(t, dose, dose2, n);
  return cudaGetLastError();
}

cudaError_t LaunchFoldSlices(double* t, double* dose, double* dose2, long long n, long long binStride,
                             long long sliceStride, int m, bool clear, cudaStream_t st) {
  const int blocks = int(std::min<long long>((n + 255) / 256, 152LL * 16));
  if (clear) FoldSlicesKernel<true><<<blocks > 0 ? blocks : 1, 256, 0, st>>>(t, dose, dose2, n, binStride, sliceStride, m);
  else FoldSlicesKernel<false><<<blocks > 0 ? blocks : 1, 256, 0, st>>>(t, dose, dose2, n, binStride, sliceStride, m);
  return cudaGetLastError();
}

cudaError_t LaunchTallySummary(const double* d, long long n, double* sum, unsigned long long* lastNz,
                               cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int blocks = int(std::min<long long>((n + 255) / 256, 152LL * 8));
  TallySummaryKernel<<<blocks, 256, 0, st>>>(d, n, sum, lastNz);
  return cudaGetLastError();
}

cudaError_t LaunchEnergyCheck(const double* histE, const double* histE0, long long nslots, const Segment* segs,
                              int nsegs, const JobF* jobs, cudaStream_t st) {
  if (nslots <= 0) return cudaSuccess;
  const int blocks = int(std::min<long long>((nslots + 255) / 256, 152LL * 4));
  EnergyCheckKernel<<<blocks, 256, 0, st>>>(histE, histE0, nslots, segs, nsegs, jobs);
  return cudaGetLastError();
}

cudaError_t LaunchSamplerEval32(const DevTables<float>& T, int s, int imat, const double* e, const double* r,
                                double* out, int n, cudaStream_t st) {
  SamplerKernel32<<<(n + 127) / 128, 128, 0, st>>>(T, s, imat, e, r, out, n);
  return cudaGetLastError();
}

cudaError_t LaunchTableEval32(const DevTables<float>& T, int q, int imat, const double* e, double* out, int n,
                              cudaStream_t st) {
  TableKernel32<<<(n + 127) / 128, 128, 0, st>>>(T, q, imat, e, out, n);
  return cudaGetLastError();
}

cudaError_t LaunchRingSelfTest(int blocks, int nslots, int rounds, uint32_t seed, long long probeCycles,
                               unsigned long long* out, cudaStream_t st) {
  RingSelfTestKernel<<<blocks, 256, 0, st>>>(nslots, rounds, seed, probeCycles, out);
  return cudaGetLastError();
}

}  // namespace dpmx
