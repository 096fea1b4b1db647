// Internal definitions shared by the host library code and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#include "dpmx.h"

namespace dpmx {

constexpr int kMaxMat = 8;         // materials per data set
constexpr uint8_t kVacuum = 255;   // material id of vacuum voxels

// ---------------------------------------------------------------------------
// Device table views, templated on the arithmetic type R (double for the plain
// FP64 form, float for the event-based form). All arrays live in one device
// allocation per precision.
// ---------------------------------------------------------------------------
template <class R>
struct SplineT {       // natural cubic spline on a log-uniform grid: n x {x,y,b,c,d} (FP64);
                       // n x {y,b,c,d} then n x x, 16-byte aligned (FP32)
  const R* p;
  int n;
  R logMin, invLogDelta, emin, emaxm;   // emaxm = emax - 1e-6 (loader clamp)
};
template <class R>
struct SplinePairT {   // FP32 only: two splines of a material on one log-uniform grid (dE/dx and
                       // 1/lambda_1), n x {y,b,c,d of the first, y,b,c,d of the second} in
                       // 32-byte records, then the n grid points
  const R* p;
  int n;
  R logMin, invLogDelta, emin, emaxm;
};
template <class R>
struct LinearT {       // linear interpolation on a uniform grid: n x {x,y} (FP64), n x y (FP32)
  const R* p;
  int n;
  R xmin, invDelta, emin, emaxm;
};
template <class R>
struct alignas(sizeof(R) * 4) AliasEntry {   // one point of an alias + linear-pdf table
  R x, y, w;
  int32_t idx;
};
template <class R>
struct AliasSetT {     // numE tables of numS points on a log energy grid
  const AliasEntry<R>* p;
  int numE, numS;
  R minE, logMinE, invLogDeltaE;
};
template <class R>
struct GSSetT {        // GS ratin tables: numE x numS x {u, a, b, 1 - u}
  const R* uab;
  const R* e;          // energy grid
  const R* a;          // transformation parameter per energy
  int numE, numS;
  R logMinE, invLogDeltaE, deltaCum;
  R deltaCumLo;        // 1/(numS-1) - deltaCum (FP32: the rest of the bin width)
};

template <class R>
struct DevTables {
  int nmat;
  R ecut, gcut;
  R density[kMaxMat], mollerScale[kMaxMat];
  SplineT<R> dedx[kMaxMat], itr1[kMaxMat], brem[kMaxMat], k1, moller;
  SplinePairT<R> di[kMaxMat];   // FP32: dedx and itr1 of each material in one record per bin
  LinearT<R> imfpMax, tot[kMaxMat], comp[kMaxMat], pair[kMaxMat];
  AliasSetT<R> kn, mol, sb[kMaxMat];
  GSSetT<R> gs;
  const R* elecBase;   // electron spline data are contiguous from here ...
  int elecCount;       // ... for this many values (shared-memory staging)
  const R* photBase;   // the photon linear tables likewise
  int photCount;
  // FP32: 1 when every material's dE/dx + 1/lambda_1 records and brem spline
  // lie on material 0's grid, one material after another at a fixed stride
  // (values between consecutive materials' records): material m's descriptor
  // is then material 0's with its records moved by m strides
  int elecUniform;
  int diStride, bremStride;
};

// ---------------------------------------------------------------------------
// Host-side parsed data (FP64, as read from the files)
// ---------------------------------------------------------------------------
struct Curve {
  std::vector<double> x, y;
};
struct AliasTab {
  double e = 0;
  std::vector<double> x, y, w;
  std::vector<int> idx;
};

struct HostTables {
  double ecut = 0, gcut = 0, slow = 0, shigh = 0, ecross = 0;
  int nmat = 0;
  std::vector<std::string> names;
  std::vector<double> density, mollerScale;
  std::vector<Curve> dedx, itr1, brem;
  Curve k1, moller;
  Curve imfpMax;
  std::vector<Curve> tot, comp, pair;
  std::vector<AliasTab> kn, mol;
  std::vector<double> sbE;
  std::vector<std::vector<AliasTab>> sb;
  int gsNumE = 0, gsNumS = 0;
  std::vector<double> gsE, gsA, gsU, gsPA, gsPB;   // [e*numS + s]
};

int LoadHostTables(const std::string& dir, HostTables& h, std::string& err);

// natural cubic spline coefficients (b, c, d per point), the recurrence of the
// reference loader
void SplineCoefficients(const std::vector<double>& x, const std::vector<double>& y, std::vector<double>& b,
                        std::vector<double>& c, std::vector<double>& d);

// ---------------------------------------------------------------------------
// Geometry and source descriptors passed to kernels
// ---------------------------------------------------------------------------
struct GridGeom {          // voxel box; world = the box
  int nx, ny, nz;
  double x0, y0, z0;       // lower corner of voxel (0,0,0) [mm]
  double vx, vy, vz;       // voxel size [mm]
  const uint8_t* mat;      // nx*ny*nz material ids (kVacuum outside any material)
  int tallyDepth;          // 1: tally by iz only (slab workload), 0: 3-D
  int matByDepth;          // 1: mat has nz entries, indexed by iz (slab presets)
  const float* rho;        // per-voxel density [g/cm3] or null (the material's nominal density)
  double wscale;           // >= 1: max over voxels of density / nominal density (Woodcock majorant)
};

struct SlabGeomD {         // the reference's pre-defined slab geometry (Geom.cc)
  int geomIndex;
  double L, invL, halfL;
};

struct SourceD {
  int particle, spectrum, shape, nbx, nby;
  double e0, e1, cx, cy, fx, fy;
  double zEntry;           // z of the entry plane [mm]
};

}  // namespace dpmx

// opaque handles of the C ABI
struct dpmx_tables {
  dpmx::HostTables h;
  int device = 0;
  void* d64 = nullptr;
  void* d32 = nullptr;
  dpmx::DevTables<double> t64;
  dpmx::DevTables<float> t32;
};

struct dpmx_phantom {
  const dpmx_tables* tables = nullptr;
  int kind = 0;             // 0 slab preset, 1 voxel array
  int geomIndex = 0;
  double lbox = 1.0;
  dpmx::GridGeom grid{};    // voxel box (slab presets are materialised too)
  uint8_t* d_mat = nullptr;
  std::shared_ptr<uint8_t> matOwner;   // owns d_mat; results keep it for their dose outputs
  float* d_rho = nullptr;   // per-voxel densities (dpmx_phantom_voxels_density) or null
  long long tallySize = 0;
  // for the dose outputs, shared with the results that outlive the phantom:
  // the density of every tally bin [g/cm3] (0 for vacuum), either given per
  // bin or as material ids (a host copy for slab presets; voxel phantoms keep
  // theirs on the device, matOwner) and a density per material
  std::shared_ptr<const std::vector<float>> binDensity;
  std::shared_ptr<const std::vector<uint8_t>> binMaterial;
  std::shared_ptr<const std::vector<float>> materialDensity;   // 256 entries
};
