// Host side of libdpmx.so: the C ABI (include/dpmx.h), device table upload,
// phantoms, and the orchestration of both transport forms (batches, chunks,
// generations, CUDA-graph capture, launch-configuration tuning).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "host_util.h"

using namespace dpmx;

namespace {
thread_local std::string g_error;
}  // namespace

namespace dpmx {
int Fail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}
int NumSMs() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}
}  // namespace dpmx

namespace {

// ---------------------------------------------------------------------------
// device table images
// ---------------------------------------------------------------------------
template <class R>
struct Image {
  std::vector<unsigned char> bytes;
  size_t Put(const void* p, size_t n) {
    size_t off = (bytes.size() + 255) & ~size_t(255);
    bytes.resize(off + n);
    std::memcpy(bytes.data() + off, p, n);
    return off;
  }
};

struct Fixup {      // pointer fields patched after upload: (address of field, offset)
  std::vector<std::pair<const void**, size_t>> v;
  void Add(const void** f, size_t off) { v.push_back({f, off}); }
  void Apply(void* base) {
    for (auto& x : v) *x.first = static_cast<unsigned char*>(base) + x.second;
  }
};

template <class R>
void PutSplines(const std::vector<const Curve*>& curves, std::vector<SplineT<R>*> outs, Image<R>& img, Fixup& fx,
                double emin, double emax, size_t& first, size_t& count) {
  // all splines of the list are written back to back (one contiguous range)
  std::vector<R> all;
  std::vector<size_t> offs;
  for (const Curve* c : curves) {
    std::vector<double> b, cc, d;
    SplineCoefficients(c->x, c->y, b, cc, d);
    offs.push_back(all.size());
    if (sizeof(R) == sizeof(double)) {   // FP64: n x {x, y, b, c, d}
      for (size_t i = 0; i < c->x.size(); ++i) {
        all.push_back(R(c->x[i])); all.push_back(R(c->y[i]));
        all.push_back(R(b[i])); all.push_back(R(cc[i])); all.push_back(R(d[i]));
      }
    } else {   // FP32: n 16-byte records {y, b, c, d}, then the n grid points
      for (size_t i = 0; i < c->x.size(); ++i) {
        all.push_back(R(c->y[i])); all.push_back(R(b[i])); all.push_back(R(cc[i])); all.push_back(R(d[i]));
      }
      for (size_t i = 0; i < c->x.size(); ++i) all.push_back(R(c->x[i]));
      while (all.size() % 4 != 0) all.push_back(R(0));   // the next spline's records stay 16-byte aligned
    }
  }
  const size_t base = img.Put(all.data(), all.size() * sizeof(R));
  first = base;
  count = all.size();
  for (size_t k = 0; k < curves.size(); ++k) {
    const Curve* c = curves[k];
    SplineT<R>* s = outs[k];
    s->n = int(c->x.size());
    const double lmin = std::log(c->x[0]);
    s->logMin = R(lmin);
    s->invLogDelta = R(1.0 / (std::log(c->x[1]) - lmin));
    s->emin = R(emin);
    s->emaxm = R(emax - 1.0E-6);
    fx.Add(reinterpret_cast<const void**>(&s->p), base + offs[k] * sizeof(R));
  }
}

template <class R>
void PutLinear(const Curve& c, LinearT<R>& s, Image<R>& img, Fixup& fx, double emin, double emax) {
  // FP64 keeps the file's grid points (the reference interpolates between
  // them); FP32 keeps the values only and places them on the uniform grid
  std::vector<R> v;
  for (size_t i = 0; i < c.x.size(); ++i) {
    if (sizeof(R) == sizeof(double)) v.push_back(R(c.x[i]));
    v.push_back(R(c.y[i]));
  }
  fx.Add(reinterpret_cast<const void**>(&s.p), img.Put(v.data(), v.size() * sizeof(R)));
  s.n = int(c.x.size());
  s.xmin = R(c.x[0]);
  s.invDelta = R(1.0 / (c.x[1] - c.x[0]));
  s.emin = R(emin);
  s.emaxm = R(emax - 1.0E-6);
}

template <class R>
void PutAlias(const std::vector<AliasTab>& tabs, const std::vector<double>& energies, AliasSetT<R>& s, Image<R>& img,
              Fixup& fx) {
  std::vector<AliasEntry<R>> v;
  for (const AliasTab& t : tabs)
    for (size_t i = 0; i < t.x.size(); ++i) v.push_back(AliasEntry<R>{R(t.x[i]), R(t.y[i]), R(t.w[i]), t.idx[i]});
  fx.Add(reinterpret_cast<const void**>(&s.p), img.Put(v.data(), v.size() * sizeof(AliasEntry<R>)));
  s.numE = int(tabs.size());
  s.numS = int(tabs[0].x.size());
  s.minE = R(energies[0]);
  const double lmin = std::log(energies[0]);
  s.logMinE = R(lmin);
  s.invLogDeltaE = R(1.0 / (std::log(energies[1]) - lmin));
}

template <class R>
int BuildImage(const HostTables& h, DevTables<R>& T, void** dptr) {
  Image<R> img;
  Fixup fx;
  std::memset(&T, 0, sizeof(T));
  T.nmat = h.nmat;
  T.ecut = R(h.ecut);
  T.gcut = R(h.gcut);
  for (int m = 0; m < h.nmat; ++m) { T.density[m] = R(h.density[m]); T.mollerScale[m] = R(h.mollerScale[m]); }
  // electron splines, contiguous (Emin/Emax taken from material 0's grid as the loaders do)
  std::vector<const Curve*> cs;
  std::vector<SplineT<R>*> outs;
  std::vector<std::pair<double, double>> lim;
  for (int m = 0; m < h.nmat; ++m) { cs.push_back(&h.dedx[m]); outs.push_back(&T.dedx[m]); }
  size_t f0, n0, f1, n1, f2, n2, f3, n3, f4, n4;
  PutSplines<R>(cs, outs, img, fx, h.dedx[0].x.front(), h.dedx[0].x.back(), f0, n0);
  cs.clear(); outs.clear();
  for (int m = 0; m < h.nmat; ++m) { cs.push_back(&h.itr1[m]); outs.push_back(&T.itr1[m]); }
  PutSplines<R>(cs, outs, img, fx, h.itr1[0].x.front(), h.itr1[0].x.back(), f1, n1);
  cs.clear(); outs.clear();
  for (int m = 0; m < h.nmat; ++m) { cs.push_back(&h.brem[m]); outs.push_back(&T.brem[m]); }
  PutSplines<R>(cs, outs, img, fx, h.brem[0].x.front(), h.brem[0].x.back(), f2, n2);
  PutSplines<R>({&h.k1}, {&T.k1}, img, fx, h.k1.x.front(), h.k1.x.back(), f3, n3);
  PutSplines<R>({&h.moller}, {&T.moller}, img, fx, h.moller.x.front(), h.moller.x.back(), f4, n4);
  size_t elecEnd = f4 + n4 * sizeof(R);
  if (sizeof(R) == sizeof(float)) {
    // dE/dx and 1/lambda_1 share the electron energy grid (the reference's data
    // files write both on it): one 32-byte record per bin serves a sub-step's
    // two lookups at one energy
    std::vector<R> all;
    std::vector<size_t> offs;
    for (int m = 0; m < h.nmat; ++m) {
      const Curve& a = h.dedx[m];
      const Curve& b = h.itr1[m];
      bool same = a.x.size() == b.x.size();
      for (size_t i = 0; same && i < a.x.size(); ++i) same = std::abs(a.x[i] - b.x[i]) <= 1e-12 * a.x[i];
      if (!same)
        return Fail(DPMX_ERR_PARSE, "eloss_rdedx.dat and el_itr1mfp.dat of material " + std::to_string(m) +
                                        " are not on one energy grid");
      std::vector<double> ab, ac, ad, bb, bc, bd;
      SplineCoefficients(a.x, a.y, ab, ac, ad);
      SplineCoefficients(b.x, b.y, bb, bc, bd);
      offs.push_back(all.size());
      for (size_t i = 0; i < a.x.size(); ++i) {
        all.push_back(R(a.y[i])); all.push_back(R(ab[i])); all.push_back(R(ac[i])); all.push_back(R(ad[i]));
        all.push_back(R(b.y[i])); all.push_back(R(bb[i])); all.push_back(R(bc[i])); all.push_back(R(bd[i]));
      }
      for (size_t i = 0; i < a.x.size(); ++i) all.push_back(R(a.x[i]));
      while (all.size() % 4 != 0) all.push_back(R(0));
    }
    const size_t base = img.Put(all.data(), all.size() * sizeof(R));
    for (int m = 0; m < h.nmat; ++m) {
      SplinePairT<R>& s = T.di[m];
      const Curve& a = h.dedx[m];
      s.n = int(a.x.size());
      const double lmin = std::log(a.x[0]);
      s.logMin = R(lmin);
      s.invLogDelta = R(1.0 / (std::log(a.x[1]) - lmin));
      s.emin = R(h.dedx[0].x.front());
      s.emaxm = R(h.dedx[0].x.back() - 1.0E-6);
      fx.Add(reinterpret_cast<const void**>(&s.p), base + offs[m] * sizeof(R));
    }
    elecEnd = base + all.size() * sizeof(R);
    // one grid and a fixed record stride for all materials (the data files
    // write every material on the same energies)
    bool uniform = h.nmat >= 1;
    for (int m = 1; m < h.nmat && uniform; ++m) {
      uniform = T.di[m].n == T.di[0].n && T.di[m].logMin == T.di[0].logMin &&
                T.di[m].invLogDelta == T.di[0].invLogDelta && offs[m] == m * offs[1] &&
                T.brem[m].n == T.brem[0].n && T.brem[m].logMin == T.brem[0].logMin &&
                T.brem[m].invLogDelta == T.brem[0].invLogDelta && T.brem[m].emin == T.brem[0].emin &&
                T.brem[m].emaxm == T.brem[0].emaxm;
      const Curve& a = h.dedx[m];
      for (size_t i = 0; uniform && i < a.x.size(); ++i) uniform = a.x[i] == h.dedx[0].x[i];
      for (size_t i = 0; uniform && i < h.brem[m].x.size(); ++i) uniform = h.brem[m].x[i] == h.brem[0].x[i];
    }
    // the brem splines follow one another at (5n + padding) values each
    const size_t bremStride = (size_t(5 * T.brem[0].n) + 3) & ~size_t(3);
    T.elecUniform = uniform ? 1 : 0;
    T.diStride = uniform && h.nmat > 1 ? int(offs[1]) : 0;
    T.bremStride = uniform ? int(bremStride) : 0;
  }
  // photon linear tables, contiguous
  const size_t photBegin = (img.bytes.size() + 255) & ~size_t(255);
  PutLinear<R>(h.imfpMax, T.imfpMax, img, fx, h.imfpMax.x.front(), h.imfpMax.x.back());
  for (int m = 0; m < h.nmat; ++m) {
    PutLinear<R>(h.tot[m], T.tot[m], img, fx, h.tot[0].x.front(), h.tot[0].x.back());
    PutLinear<R>(h.comp[m], T.comp[m], img, fx, h.comp[0].x.front(), h.comp[0].x.back());
    PutLinear<R>(h.pair[m], T.pair[m], img, fx, h.pair[0].x.front(), h.pair[0].x.back());
  }
  const size_t photEnd = img.bytes.size();
  // sampling tables
  std::vector<double> knE, molE;
  for (auto& t : h.kn) knE.push_back(t.e);
  for (auto& t : h.mol) molE.push_back(t.e);
  PutAlias<R>(h.kn, knE, T.kn, img, fx);
  PutAlias<R>(h.mol, molE, T.mol, img, fx);
  for (int m = 0; m < h.nmat; ++m) PutAlias<R>(h.sb[m], h.sbE, T.sb[m], img, fx);
  {
    const int ne = h.gsNumE, ns = h.gsNumS;
    std::vector<R> uab(size_t(ne) * ns * 4, R(0));
    for (size_t i = 0; i < size_t(ne) * ns; ++i) {
      uab[4 * i] = R(h.gsU[i]); uab[4 * i + 1] = R(h.gsPA[i]); uab[4 * i + 2] = R(h.gsPB[i]);
      uab[4 * i + 3] = R(1.0 - h.gsU[i]);   // 1 - u for the FP32 sampler's well-conditioned form
    }
    std::vector<R> e(h.gsE.begin(), h.gsE.end()), a(h.gsA.begin(), h.gsA.end());
    fx.Add(reinterpret_cast<const void**>(&T.gs.uab), img.Put(uab.data(), uab.size() * sizeof(R)));
    fx.Add(reinterpret_cast<const void**>(&T.gs.e), img.Put(e.data(), e.size() * sizeof(R)));
    fx.Add(reinterpret_cast<const void**>(&T.gs.a), img.Put(a.data(), a.size() * sizeof(R)));
    T.gs.numE = ne;
    T.gs.numS = ns;
    const double lmin = std::log(h.gsE[0]);
    T.gs.logMinE = R(lmin);
    T.gs.invLogDeltaE = R(1.0 / (std::log(h.gsE[1]) - lmin));
    T.gs.deltaCum = R(1.0 / (ns - 1));
    T.gs.deltaCumLo = R(1.0 / (ns - 1) - double(T.gs.deltaCum));
  }
  fx.Add(reinterpret_cast<const void**>(&T.elecBase), f0);
  T.elecCount = int((elecEnd - f0) / sizeof(R));
  fx.Add(reinterpret_cast<const void**>(&T.photBase), photBegin);
  T.photCount = int((photEnd - photBegin) / sizeof(R));
  void* d = nullptr;
  CK(cudaMalloc(&d, img.bytes.size()));
  CK(cudaMemcpy(d, img.bytes.data(), img.bytes.size(), cudaMemcpyHostToDevice));
  fx.Apply(d);
  *dptr = d;
  return DPMX_OK;
}

// the largest material id of m[0..n) other than vacuum, into *out (zeroed
// before); m 16-byte aligned, read 16 bytes per thread
__device__ __forceinline__ unsigned MaxNonVacuum(uint32_t w) {
  unsigned best = 0;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const unsigned v = (w >> (8 * b)) & 0xffu;
    best = max(best, v == kVacuum ? 0u : v);
  }
  return best;
}
__global__ void __launch_bounds__(256) MaxMaterialKernel(const uint8_t* m, unsigned long long n, unsigned* out) {
  unsigned best = 0;
  const unsigned long long n16 = n / 16;
  const uint4* q = reinterpret_cast<const uint4*>(m);
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) {
    const uint4 w = q[i];
    best = max(best, max(max(MaxNonVacuum(w.x), MaxNonVacuum(w.y)), max(MaxNonVacuum(w.z), MaxNonVacuum(w.w))));
  }
  if (blockIdx.x == 0 && threadIdx.x < n - n16 * 16) {   // the last n % 16 bytes
    const unsigned v = m[n16 * 16 + threadIdx.x];
    best = max(best, v == kVacuum ? 0u : v);
  }
  best = __reduce_max_sync(0xffffffffu, best);
  if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(out, best);
}

}  // namespace

namespace dpmx {

double SlabDensityAt(const dpmx_tables* t, int geomIndex, double invL, int iz) {
  // Geom::GetMaterialIndex (Geom.cc:133-164) + GetVoxelMaterialDensity
  int m = 0;
  if (iz < 0) return 1.0E-40;
  switch (geomIndex) {
    case 1: m = (iz < 10.0 * invL) ? 0 : (iz < 30.0 * invL ? 1 : 0); break;
    case 2: m = (iz < 20.0 * invL) ? 0 : (iz < 40.0 * invL ? 1 : 0); break;
    case 3: m = (iz < 10.0 * invL) ? 0 : (iz < 15.0 * invL ? 1 : (iz < 25.0 * invL ? 2 : 0)); break;
    default: m = 0;
  }
  return t->h.density[m];
}
int SlabMaterialAt(int geomIndex, double invL, int iz) {
  switch (geomIndex) {
    case 1: return (iz < 10.0 * invL) ? 0 : (iz < 30.0 * invL ? 1 : 0);
    case 2: return (iz < 20.0 * invL) ? 0 : (iz < 40.0 * invL ? 1 : 0);
    case 3: return (iz < 10.0 * invL) ? 0 : (iz < 15.0 * invL ? 1 : (iz < 25.0 * invL ? 2 : 0));
    default: return 0;
  }
}

// the reference's depth-histogram length: starts at 20 bins, grows by +10
// past the deepest bin reached (Geom.cc:120-130)
int HistLen(int maxIz) {
  int size = 20;
  while (size <= maxIz) size += 10;
  return size;
}

}  // namespace dpmx

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* dpmx_last_error(void) { return g_error.c_str(); }
const char* dpmx_version(void) { return "dpmx 1.0 (sm_103a)"; }

int dpmx_tables_load(const char* dir, dpmx_tables** out) {
  if (!dir || !out) return Fail(DPMX_ERR_ARG, "null argument");
  *out = nullptr;
  std::unique_ptr<dpmx_tables> t(new dpmx_tables());
  std::string err;
  int rc = LoadHostTables(dir, t->h, err);
  if (rc) return Fail(rc, err);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return Fail(DPMX_ERR_CUDA, "no CUDA device");
  CK(cudaGetDevice(&t->device));
  if ((rc = BuildImage<double>(t->h, t->t64, &t->d64))) return rc;
  if ((rc = BuildImage<float>(t->h, t->t32, &t->d32))) return rc;
  *out = t.release();
  return DPMX_OK;
}

void dpmx_tables_free(dpmx_tables* t) {
  if (!t) return;
  cudaFree(t->d64);
  cudaFree(t->d32);
  delete t;
}

int dpmx_tables_num_materials(const dpmx_tables* t) { return t ? t->h.nmat : 0; }

double dpmx_tables_param(const dpmx_tables* t, int which) {
  if (!t) return 0.0;
  switch (which) {
    case 0: return t->h.ecut;
    case 1: return t->h.gcut;
    case 2: return t->h.slow;
    case 3: return t->h.shigh;
    case 4: return t->h.ecross;
    default: return 0.0;
  }
}

double dpmx_tables_density(const dpmx_tables* t, int imat) {
  if (!t || imat < 0 || imat >= t->h.nmat) return 0.0;
  return t->h.density[imat];
}

int dpmx_tables_material_name(const dpmx_tables* t, int imat, char* name, int cap) {
  if (!t || imat < 0 || imat >= t->h.nmat || !name || cap < 1) return Fail(DPMX_ERR_ARG, "bad material index");
  std::snprintf(name, size_t(cap), "%s", t->h.names[imat].c_str());
  return DPMX_OK;
}

// the material ids of a phantom: a block of the scratch pool (no cudaMalloc or
// device-wide cudaFree per phantom), shared by the phantom and the results
// that write its dose; back to the pool when the last of them lets go (every
// device use of it has completed by then: runs and dose writers synchronise)
static int NewDeviceIds(dpmx_phantom* p, size_t bytes) {
  void* q = nullptr;
  CK(ScratchGet(bytes, &q));
  p->d_mat = static_cast<uint8_t*>(q);
  p->matOwner.reset(p->d_mat, [](uint8_t* m) { ScratchPut(m); });
  return DPMX_OK;
}

int dpmx_phantom_slab(const dpmx_tables* t, int geom_index, double lbox, dpmx_phantom** out) {
  if (!t || !out || !(lbox > 0.0)) return Fail(DPMX_ERR_ARG, "bad slab phantom arguments");
  if (geom_index < 0) return Fail(DPMX_ERR_ARG, "geometry index must be >= 0");
  const double invL = 1.0 / lbox;
  // the voxel box enclosing the reference world |x|,|y| <= 100 mm, z <= 100 mm
  const int ixmax = int(std::ceil((100.0 - 0.5 * lbox) * invL - 1.0e-9));
  const int nx = 2 * ixmax + 1;
  const int nz = int(std::ceil((100.0 - 0.5 * lbox) * invL - 1.0e-9)) + 1;
  if (nx > 2047 || nz > 1023) return Fail(DPMX_ERR_ARG, "voxel size too small for the slab geometry");
  for (int iz = 0; iz < nz; ++iz)
    if (SlabMaterialAt(geom_index, invL, iz) >= t->h.nmat)
      return Fail(DPMX_ERR_ARG, "the data set has fewer materials than the slab geometry needs");
  auto rho = std::make_shared<std::vector<float>>(size_t(nz) + 16, 0.0f);
  for (int iz = 0; iz < nz + 16; ++iz) (*rho)[iz] = float(SlabDensityAt(t, geom_index, invL, iz));
  std::unique_ptr<dpmx_phantom> p(new dpmx_phantom());
  p->tables = t;
  p->kind = 0;
  p->geomIndex = geom_index;
  p->lbox = lbox;
  std::vector<uint8_t> m(nz);
  for (int iz = 0; iz < nz; ++iz) m[iz] = uint8_t(SlabMaterialAt(geom_index, invL, iz));
  if (int rc = NewDeviceIds(p.get(), nz)) return rc;
  CK(cudaMemcpy(p->d_mat, m.data(), nz, cudaMemcpyHostToDevice));
  GridGeom& g = p->grid;
  g.nx = nx; g.ny = nx; g.nz = nz;
  g.vx = g.vy = g.vz = lbox;
  g.x0 = -(ixmax + 0.5) * lbox;
  g.y0 = g.x0;
  g.z0 = -0.5 * lbox;
  g.mat = p->d_mat;
  g.tallyDepth = 1;
  g.matByDepth = 1;
  g.rho = nullptr;
  g.wscale = 1.0;
  p->tallySize = nz + 16;
  p->binDensity = rho;
  *out = p.release();
  return DPMX_OK;
}

int dpmx_phantom_voxels(const dpmx_tables* t, int nx, int ny, int nz, double vx, double vy, double vz,
                        const uint8_t* mat, dpmx_phantom** out) {
  if (!t || !out || !mat) return Fail(DPMX_ERR_ARG, "null argument");
  if (nx < 1 || ny < 1 || nz < 1 || nx > 2047 || ny > 2047 || nz > 1023)
    return Fail(DPMX_ERR_ARG, "phantom dimensions must be 1..2047 (x, y) and 1..1023 (z)");
  if (!(vx > 0 && vy > 0 && vz > 0)) return Fail(DPMX_ERR_ARG, "voxel sizes must be positive");
  const size_t n = size_t(nx) * ny * nz;
  std::unique_ptr<dpmx_phantom, void (*)(dpmx_phantom*)> p(new dpmx_phantom(), dpmx_phantom_free);
  p->tables = t;
  p->kind = 1;
  // the material ids, and after them (16-byte aligned) the slot where the
  // device writes the largest id other than vacuum: checked on the GPU
  const size_t nal = (n + 15) & ~size_t(15);
  if (int rc = NewDeviceIds(p.get(), nal + 16)) return rc;
  CK(cudaMemcpy(p->d_mat, mat, n, cudaMemcpyHostToDevice));
  unsigned* dworst = reinterpret_cast<unsigned*>(p->d_mat + nal);
  CK(cudaMemset(dworst, 0, sizeof(unsigned)));
  const unsigned long long n16 = n / 16;
  const int blocks = int(std::max<unsigned long long>(1, std::min<unsigned long long>((n16 + 255) / 256, 152ULL * 8)));
  MaxMaterialKernel<<<blocks, 256>>>(p->d_mat, n, dworst);
  CK(cudaGetLastError());
  unsigned worst = 0;
  CK(cudaMemcpy(&worst, dworst, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (int(worst) >= t->h.nmat) return Fail(DPMX_ERR_ARG, "material id beyond the data set");
  auto lut = std::make_shared<std::vector<float>>(256, 0.0f);
  for (int m = 0; m < t->h.nmat; ++m) (*lut)[m] = float(t->h.density[m]);
  GridGeom& g = p->grid;
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.vx = vx; g.vy = vy; g.vz = vz;
  g.x0 = -0.5 * nx * vx;
  g.y0 = -0.5 * ny * vy;
  g.z0 = 0.0;
  g.mat = p->d_mat;
  g.tallyDepth = 0;
  g.matByDepth = 0;
  g.rho = nullptr;
  g.wscale = 1.0;
  p->tallySize = (long long)n;
  p->materialDensity = lut;   // the ids stay on the device (matOwner)
  *out = p.release();
  return DPMX_OK;
}

int dpmx_phantom_voxels_density(const dpmx_tables* t, int nx, int ny, int nz, double vx, double vy, double vz,
                                const uint8_t* mat, const float* density, dpmx_phantom** out) {
  if (!density) return Fail(DPMX_ERR_ARG, "null density array");
  dpmx_phantom* p = nullptr;
  if (int rc = dpmx_phantom_voxels(t, nx, ny, nz, vx, vy, vz, mat, &p)) return rc;
  std::unique_ptr<dpmx_phantom, void (*)(dpmx_phantom*)> guard(p, dpmx_phantom_free);
  const size_t n = size_t(nx) * ny * nz;
  // the Woodcock majorant of the photon tables holds for the nominal
  // densities; denser voxels scale it (SimDPMLike.cc:471-474 uses it as is)
  double ws = 1.0;
  auto rho = std::make_shared<std::vector<float>>(n);
  for (size_t i = 0; i < n; ++i) {
    if (mat[i] == kVacuum) { (*rho)[i] = 0.0f; continue; }
    const float r = density[i];
    if (!(r > 0.0f) || !(r < 1.0e4f)) return Fail(DPMX_ERR_ARG, "voxel densities must be positive and finite");
    (*rho)[i] = r;
    ws = std::max(ws, double(r) / t->h.density[mat[i]]);
  }
  {
    void* q = nullptr;
    CK(ScratchGet(n * sizeof(float), &q));
    p->d_rho = static_cast<float*>(q);
  }
  CK(cudaMemcpy(p->d_rho, rho->data(), n * sizeof(float), cudaMemcpyHostToDevice));
  p->grid.rho = p->d_rho;
  p->grid.wscale = ws;
  p->binDensity = rho;
  *out = guard.release();
  return DPMX_OK;
}

void dpmx_phantom_free(dpmx_phantom* p) {
  if (!p) return;
  p->matOwner.reset();   // the device ids go when no result holds them either
  ScratchPut(p->d_rho);
  delete p;
}

long long dpmx_phantom_tally_size(const dpmx_phantom* p) { return p ? p->tallySize : 0; }

void dpmx_run_options_default(dpmx_run_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->precision = DPMX_FP32_EVENT;
  o->batches = 10;
  o->tally_aggregate = -1;
  o->electron_kernel = -1;
  o->photon_kernel = -1;
  o->use_graph = 1;
}

}  // extern "C"

