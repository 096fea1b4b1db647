/*
 * dpmx.h - C ABI of the GB300-native dpm_Simulate transport library
 * (libdpmx.so). Plain pointers and sizes only; every call returns an int
 * status (DPMX_OK = 0, negative on error) and dpmx_last_error() gives the
 * message of the calling thread's last failure. Nothing in the library exits
 * or aborts the process.
 *
 * The calls replace these reference interfaces (paths inside bl406/dpm-g4cpp):
 *   dpmx_tables_load      SimElectronData::Load, SimPhotonData::Load,
 *                         SimMaterialData::Load (dpm_Simulate.cc:71-78,
 *                         SimElectronData.cc:44-115, SimPhotonData.cc:28-78,
 *                         SimMaterialData.cc:6-53) - same 14 data files
 *   dpmx_phantom_slab     Geom::Geom(lbox, matData, geomIndex) (Geom.cc:9-17)
 *                         with the pre-defined slab geometries (Geom.cc:133-164)
 *   dpmx_phantom_voxels   the extension point of Geom::GetMaterialIndex /
 *                         GetVoxelMaterialDensity (Geom.hh:64-95) for 3-D
 *                         voxel phantoms
 *   dpmx_simulate         Simulate(nprimary, eprimary, iselectron, lbox, ...,
 *                         geomIndex, filename) (SimDPMLike.hh:46,
 *                         SimDPMLike.cc:40-251), histograms returned in memory
 *   dpmx_write_hist       Geom::Write (Geom.cc:167-192), the hist.sim format
 *   dpmx_run              many Simulate calls (jobs) batched in one run
 *   dpmx_sampler_eval     the per-interaction samplers SimKNTables.cc:69-90,
 *                         SimMollerTables.cc:69-89, SimSBTables.cc:93-114,
 *                         SimGSTables.cc:84-119 fed with given uniforms
 *   dpmx_table_eval       the loaders' interpolators, e.g.
 *                         SimStoppingPower::GetDEDXPerDensity (SimStoppingPower.hh:43)
 *   dpmx_influence_*      no reference counterpart: the beamlet influence matrix
 */
#ifndef DPMX_H
#define DPMX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DPMX_OK 0
#define DPMX_ERR_FILE (-1)      /* a data file is missing or unreadable */
#define DPMX_ERR_PARSE (-2)     /* a data file does not have the expected layout */
#define DPMX_ERR_CUDA (-3)      /* a CUDA call failed (no device, launch error...) */
#define DPMX_ERR_ARG (-4)       /* an argument is out of range */
#define DPMX_ERR_OVERFLOW (-5)  /* a particle queue or stack overflowed; result incomplete */
#define DPMX_ERR_NOMEM (-6)     /* device memory exhausted */

/* precision / algorithm of a run */
#define DPMX_FP64_PLAIN 0       /* one thread per history, FP64, reference order */
#define DPMX_FP32_EVENT 1       /* event-based FP32 transport, FP64 tallies */

typedef struct dpmx_tables dpmx_tables;
typedef struct dpmx_phantom dpmx_phantom;
typedef struct dpmx_result dpmx_result;
typedef struct dpmx_csr dpmx_csr;

const char* dpmx_last_error(void);
const char* dpmx_version(void);

/* ---- data tables (the reference's data-file format) ---- */
int dpmx_tables_load(const char* data_dir, dpmx_tables** out);
void dpmx_tables_free(dpmx_tables* t);
int dpmx_tables_num_materials(const dpmx_tables* t);
/* which: 0 electron cut, 1 gamma cut, 2 MSC s-low, 3 s-high, 4 e-cross [MeV/mm] */
double dpmx_tables_param(const dpmx_tables* t, int which);
double dpmx_tables_density(const dpmx_tables* t, int imat);
/* copies the material name (NUL-terminated, truncated to cap) */
int dpmx_tables_material_name(const dpmx_tables* t, int imat, char* name, int cap);

/* ---- geometry ---- */
/* reference pre-defined geometry geom_index (0-3) with cubic voxels of lbox mm;
 * depth tally (bins of lbox along +z) */
int dpmx_phantom_slab(const dpmx_tables* t, int geom_index, double lbox_mm, dpmx_phantom** out);
/* nx*ny*nz voxels (x fastest) of vx*vy*vz mm, material ids from the host array
 * mat (255 = vacuum: as in the reference's transport, SimDPMLike.cc:88-93 and
 * :282-287, a track that enters a vacuum voxel ends there); the phantom spans
 * x in [-nx*vx/2, nx*vx/2], y likewise, z in [0, nz*vz]; 3-D tally */
int dpmx_phantom_voxels(const dpmx_tables* t, int nx, int ny, int nz, double vx, double vy, double vz,
                        const uint8_t* mat, dpmx_phantom** out);
/* the same with a density per voxel [g/cm3] (the material id keeps the
 * composition): Geom::GetVoxelMaterialDensity(iVoxel) (Geom.hh:75-92) as the
 * reference designed it for fractional densities; the photon majorant is
 * scaled by the largest density / nominal density ratio */
int dpmx_phantom_voxels_density(const dpmx_tables* t, int nx, int ny, int nz, double vx, double vy, double vz,
                                const uint8_t* mat, const float* density, dpmx_phantom** out);
void dpmx_phantom_free(dpmx_phantom* p);
/* number of tally bins of a phantom (slab: depth bins; voxels: nx*ny*nz) */
long long dpmx_phantom_tally_size(const dpmx_phantom* p);

/* ---- sources and jobs ---- */
typedef struct {
  int particle;       /* -1 electron, 0 photon */
  int spectrum;       /* 0 mono e0; 1 uniform on [e0,e1]; 2 p(E) ~ (e1-E) on [e0,e1] */
  double e0, e1;      /* MeV */
  int shape;          /* 0 pencil at (cx,cy); 1 rectangle fx*fy centred at (cx,cy);
                         2 grid of nbx*nby beamlets fx*fy each, centred at (cx,cy) */
  double cx, cy, fx, fy;  /* mm */
  int nbx, nby;       /* shape 2: nbx * nby <= 65535 */
} dpmx_source;

typedef struct {
  const dpmx_phantom* phantom;
  dpmx_source source;
  long long histories;
  uint64_t seed;
  long long first_history;   /* index of the job's first history: history h always
                                uses random stream h, so a job split into ranges
                                (e.g. across GPUs) sums to the unsplit result;
                                indices lie in [0, 2^32): first_history +
                                histories <= 2^32, else DPMX_ERR_ARG */
} dpmx_job;

typedef struct {
  int precision;             /* DPMX_FP64_PLAIN or DPMX_FP32_EVENT */
  int batches;               /* statistical batches for dose^2 (default 10, at most 65536) */
  int block_size;            /* threads per block (0: default / tuned) */
  int blocks_per_sm;         /* resident blocks per SM (0: default / tuned) */
  long long chunk_histories; /* histories per transport chunk (0: as few equal chunks of at most
                                2^24 as the run needs, and at least two for runs of 2^23 or more;
                                a run of two or more chunks runs them on two streams) */
  int tally_aggregate;       /* FP32: -1 default, 0 plain atomics, 1 warp-aggregated */
  int use_graph;             /* FP32: capture each batch in a CUDA graph (default 1) */
  int tag_beamlets;          /* FP32: also tally dose per beamlet (influence matrix) */
  int autotune;              /* 1: time the candidate kernel shapes (electron kernel, block
                                size, tally aggregation, electron slots per block) on a
                                sample of the jobs and run the fastest */
  int profile_phases;        /* FP32: time every phase launch (no graph); see dpmx_result_profile */
  int electron_kernel;       /* FP32 electron phase: -1 default, 0 one electron per lane with
                                refill, 1 block-batched (shared-memory slots on rings by their
                                next interaction, one interaction kind per warp) */
  int photon_kernel;         /* FP32 photon phase: -1 default, 0 one photon per lane, 1
                                block-batched (shared-memory slots on rings by their next
                                interaction); both draw the same random numbers per photon */
  void* stream;              /* cudaStream_t to run on, NULL = library stream */
  int electron_slots;        /* FP32 block-batched electron phase: electrons resident per block
                                (its ring depth): 0 default (448), or 384 */
} dpmx_run_options;

void dpmx_run_options_default(dpmx_run_options* o);

typedef struct {
  double edep;               /* total energy deposited in the tally [MeV] */
  double escaped;            /* energy that left the phantom [MeV] */
  double primary_energy;     /* sum of primary kinetic energies [MeV] */
  double max_residual;       /* max |E_primary - E_deposited - E_escaped| of a history [MeV] */
  long long residual_violations; /* histories with residual > 1e-3 E_primary */
  long long lost;            /* particles dropped (queue/stack overflow, step cap) */
  long long steps;           /* electron condensed-history sub-steps */
  long long histories;
} dpmx_job_stats;

/* runs njobs jobs (1..256) as one run; DPMX_ERR_ARG beyond the limits: at
 * most 65536 batches, history indices in [0, 2^32), source energies strictly
 * inside the data set's range. Safe to call from several host threads at once
 * (each run has its own stream unless opt->stream is given). */
int dpmx_run(const dpmx_tables* t, const dpmx_job* jobs, int njobs, const dpmx_run_options* opt,
             dpmx_result** out);
/* host copies of a job's tallies; any output pointer may be NULL.
 * dose: energy per bin [MeV], summed over histories; dose2: sum over batches of
 * the squared batch sums; steps: number of scoring steps per bin (slab only) */
int dpmx_result_tally(const dpmx_result* r, int job, double* dose, double* dose2, double* steps);
/* device pointer of a job's dose tally (valid until dpmx_result_free) */
const double* dpmx_result_tally_device(const dpmx_result* r, int job);
int dpmx_result_stats(const dpmx_result* r, int job, dpmx_job_stats* s);
/* wall time of the transport (device events) [ms] and kernel launches issued */
double dpmx_result_elapsed_ms(const dpmx_result* r);
long long dpmx_result_launches(const dpmx_result* r);
/* chosen launch configuration: [block_size, blocks_per_sm, chunk_histories,
 * tally_aggregate + 2 * electron_kernel + 4 * photon_kernel + 8 * electron_slots] */
int dpmx_result_config(const dpmx_result* r, long long* cfg4);
/* phase profile of a run with profile_phases = 1 (zeros otherwise), 10 values:
 * electron-phase ms, photon-phase ms, electron-phase launches, photon-phase
 * launches, electron sub-steps, photon steps, electrons transported, photons
 * transported, histories, total ms */
int dpmx_result_profile(const dpmx_result* r, double* out10);
void dpmx_result_free(dpmx_result* r);
/* dose outputs of a job:
 *  DPMX_DOSE_RAW   voxel phantoms: "DPMXDOSE", int32 {version 1, nx, ny, nz},
 *                  float64 {vx, vy, vz, x0, y0, z0} [mm], int64 {histories,
 *                  batches}, then float64 dose [Gy per history] and float64
 *                  relative 1-sigma uncertainty per voxel (x fastest)
 *  DPMX_DOSE_DEPTH the hist.sim text of Geom::Write (Geom.cc:167-192) for any
 *                  phantom: per depth slice the energy per primary over the
 *                  slice's mean density and thickness [MeV cm2/g], and the
 *                  scoring steps per primary (slab presets; 0 for voxels) */
#define DPMX_DOSE_RAW 0
#define DPMX_DOSE_DEPTH 1
int dpmx_result_write(const dpmx_result* r, int job, const char* path, int format);
/* Runs keep their device scratch (particle queues, batch tallies) in a pool
 * for later runs on the same device; this frees the blocks no run is using. */
void dpmx_scratch_release(void);

/* ---- drop-in for Simulate(...) ---- */
/* pencil beam from (0,0,-lbox/2) along +z through geometry geom_index; fills
 * edep_hist/step_hist (cap bins) with the reference's depth histograms and
 * sets *hist_len to the number of bins the reference would write */
int dpmx_simulate(const dpmx_tables* t, int nprimary, double eprimary, int iselectron, double lbox,
                  int geom_index, uint64_t seed, int precision, double* edep_hist, double* step_hist,
                  int cap, int* hist_len);
/* The same workload in the FP64 plain form for callers that must not have the
 * library allocate device memory (a plug-in inside a framework that owns all
 * device memory through its own pool, or a latency-critical caller for whom a
 * cudaMalloc would synchronise the device). No counterpart in the reference.
 * edep, edep2 (may be NULL) and steps are caller-owned DEVICE arrays of `bins`
 * doubles (depth bins of lbox); bins must cover the geometry's depth bins and
 * may not exceed 8192; lbox has the same lower limit as dpmx_phantom_slab
 * (at most 1023 depth bins). The library's scratch is a fixed 65 KB device
 * array shared by all calls: calls that overlap on the GPU race and must be
 * serialised. The first call on a device looks the array up (and keeps its
 * address until the process exits, so no cudaDeviceReset may come between
 * calls); it should come before any stream capture. Runs on `stream` (NULL:
 * default stream), synchronises that stream and reads the run's counters
 * back before it returns. */
int dpmx_simulate_noalloc(const dpmx_tables* t, int nprimary, double eprimary, int iselectron, double lbox,
                          int geom_index, uint64_t seed, double* edep, double* edep2, double* steps, int bins,
                          int* hist_len, void* stream);
/* writes hist.sim exactly as Geom::Write */
int dpmx_write_hist(const dpmx_tables* t, const char* fname, int geom_index, double lbox, int nprimary,
                    const double* edep_hist, const double* step_hist, int hist_len);

/* ---- tier-1 hooks ---- */
/* sampler: 0 KN eps, 1 Moller T', 2 SB k (imat), 3 GS mu. e: n energies,
 * r: 3n uniforms (sampler arguments in order), out: n results; host arrays */
int dpmx_sampler_eval(const dpmx_tables* t, int precision, int sampler, int imat, const double* e,
                      const double* r, double* out, int n);
/* quantity: 0 dE/dx, 1 1/lambda_1, 2 brem IMFP, 3 Moller IMFP, 4 K1,
 * 5 global max photon IMFP, 6 total, 7 Compton, 8 pair IMFP (per density) */
int dpmx_table_eval(const dpmx_tables* t, int precision, int quantity, int imat, const double* e,
                    double* out, int n);
/* FP64 form of the Simulate workload (SimDPMLike.cc:57-247) that also returns
 * each history's deposited energy (hist_edep, nprimary values) and the depth
 * histogram; history h uses the per-history random stream with index h */
int dpmx_simulate_histories(const dpmx_tables* t, int nprimary, double eprimary, int iselectron, double lbox,
                            int geom_index, uint64_t seed, double* hist_edep, double* edep_hist, int cap);

/* FP64 form of one job on any phantom (voxels included) with each history's
 * deposited energy in hist_edep (job->histories values, at most 2^26) and,
 * if dose is not NULL, the job's tally (dpmx_phantom_tally_size values);
 * history h uses the per-history random stream with index first_history + h,
 * as the oracle's Philox mode does */
int dpmx_job_histories(const dpmx_tables* t, const dpmx_job* job, double* hist_edep, double* dose);
/* random numbers (replaces the reference's global mt19937, Random.hh:10-12,
 * Random.cc:3-4, by counter-based Philox-4x32-10, Salmon et al. SC'11): for
 * each i, the block philox(counters[4i..4i+3], keys[2i..2i+1]) into
 * words[4i..], the FP32 transport's uniform of each word into u32[4i..], and
 * the FP64 form's uniform of each word pair into u64[2i..]; host arrays */
int dpmx_rng_eval(const uint32_t* counters, const uint32_t* keys, int n, uint32_t* words, float* u32,
                  double* u64);
/* measurement hook: FP64 atomicAdd throughput into `nbins` doubles (kept in
 * L2 when nbins * 8 B fits it), every thread of a GPU-filling launch adding to
 * per_thread pseudo-random bins; the roof of the dose tally's one atomic per
 * deposit. No reference counterpart. */
int dpmx_atomic_roof(int nbins, int per_thread, double* atomics_per_s);

/* ---- model validation (the reference's modelValidationTests, testAPI.cc) ---- */
#define DPMX_MODEL_BREM 0
#define DPMX_MODEL_MOLLER 1
#define DPMX_MODEL_MSC 2
/* n interactions of `model` for a primary of energy e0 [MeV] along +z in
 * material imat, sampled on the GPU (a Philox stream per sample, key `seed`),
 * histogrammed as testAPI does: hist_x[hbins] counts x = log10(k/e0) on
 * [log10(gamma cut/e0), 0.1] (hbins - 1 intervals; k the secondary's energy,
 * the primary's for MSC), hist_cos[hbins] counts the direction cosine of the
 * secondary (the primary for MSC) in bin (int)(cost*(hbins/2) + hbins/2) */
int dpmx_model_histogram(const dpmx_tables* t, int precision, int model, int imat, double e0, long long n,
                         uint64_t seed, int hbins, double* hist_x, double* hist_cos);

/* ---- self-test of the block kernels' slot rings ---- */
/* `blocks` independent blocks of 256 threads each pass `nslots` slots (1..512)
 * through four slot rings (the shared-memory queues the block-batched phases
 * schedule with) until every slot has been taken `rounds` times; then each
 * block waits `probe_cycles` clock cycles on a ring cell that nothing fills.
 * out[0] = slots taken, out[1] = slots taken a number of times other than
 * `rounds`, out[2] = warps that gave up a wait, out[3] = blocks whose probe
 * wait ran out. A correct ring gives blocks * nslots * rounds, 0, 0, blocks. */
int dpmx_ring_selftest(int blocks, int nslots, int rounds, uint64_t seed, long long probe_cycles, long long* out);

/* ---- influence matrix (beamlet-tagged run with tag_beamlets = 1) ---- */
/* builds A (rows: voxels, cols: beamlets, FP32 values from the FP64 tally,
 * entries <= threshold * max dropped) on the device */
int dpmx_influence_build(const dpmx_result* r, int job, double threshold, dpmx_csr** out);
int dpmx_csr_shape(const dpmx_csr* a, long long* rows, long long* cols, long long* nnz);
/* device arrays: row_ptr (rows+1, int64), col (nnz, int32), val (nnz, float) */
int dpmx_csr_device(const dpmx_csr* a, const int64_t** row_ptr, const int32_t** col, const float** val);
/* y[rows] = A x[cols]; device pointers, FP64 vectors, FP64 accumulation */
int dpmx_csr_spmv(const dpmx_csr* a, const double* x, double* y, void* stream);
/* x[cols] = A^T y[rows]; device pointers. Uses per-matrix scratch: calls on
 * one matrix must not overlap (same stream, or ordered by the caller). The
 * result does not depend on scheduling (no atomics). */
int dpmx_csr_spmv_t(const dpmx_csr* a, const double* y, double* x, void* stream);
/* host copies of the three CSR arrays (sizes from dpmx_csr_shape) */
int dpmx_csr_download(const dpmx_csr* a, int64_t* row_ptr, int32_t* col, float* val);
void dpmx_csr_free(dpmx_csr* a);

#ifdef __cplusplus
}
#endif
#endif /* DPMX_H */
