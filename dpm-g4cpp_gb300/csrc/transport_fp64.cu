// Plain FP64 GPU form of the dpm_Simulate transport: one thread per history,
// a per-thread LIFO secondary stack in local memory, and the reference's
// control flow and random-number consumption order (SimDPMLike.cc:40-791).
// Random numbers come from one Philox stream per history (HistoryRng), so a
// history computed here can be compared with the CPU oracle history by history.
// This translation unit is compiled without FMA contraction to keep the
// double-precision arithmetic in the reference's operation order.
#include "device_common.cuh"
#include "kernels.h"

namespace dpmx {
namespace {

constexpr int kStackDepth = 64;   // secondary stack per thread (overflow drops + counts)

struct TrackD {
  double pos[3], dir[3];
  int box[3];
  int type, mat;
  double ekin;
};

// The reference's pre-defined slab geometry (Geom.cc:20-164)
struct SlabGeo {
  SlabGeomD g;
  const double* density;
  double* edep;     // depth histograms
  double* steps;
  int cap;
  int* maxIz;
  __device__ double DistanceToBoundary(double* r, const double* v, int* i) const {
    const double kTol = 1.0E-4, kHalfTol = 0.5 * kTol, kExtent = 100.0;
    for (int guard = 0; guard < 64; ++guard) {
      if (fabs(r[0]) > kExtent || fabs(r[1]) > kExtent || r[2] > kExtent || r[2] < -g.L) return -1.0;
      i[0] = int(floor((r[0] + g.halfL) * g.invL));
      i[1] = int(floor((r[1] + g.halfL) * g.invL));
      i[2] = int(floor((r[2] + g.halfL) * g.invL));
      double snext = 1.0E+20;
      bool pushed = false;
      for (int a = 0; a < 3 && !pushed; ++a) {
        const double tr = r[a] - i[a] * g.L;
        if (v[a] > 0.0) {
          const double pd = g.halfL - tr;
          if (pd < kHalfTol) { r[a] += kTol; pushed = true; }
          else { const double s = pd / v[a]; if (a == 0 || s < snext) snext = s; }
        } else if (v[a] < 0.0) {
          const double pd = g.halfL + tr;
          if (pd < kHalfTol) { r[a] -= kTol; pushed = true; }
          else { const double s = -pd / v[a]; if (a == 0 || s < snext) snext = s; }
        }
      }
      if (!pushed) return snext;
    }
    return -1.0;   // cannot happen for finite directions; treated as leaving the world
  }
  __device__ int MaterialIndex(const int* i) const {
    const int iz = i[2];
    if (iz < 0) return -1;
    switch (g.geomIndex) {
      case 1: if (iz < 10.0 * g.invL) return 0; if (iz < 30.0 * g.invL) return 1; return 0;
      case 2: if (iz < 20.0 * g.invL) return 0; if (iz < 40.0 * g.invL) return 1; return 0;
      case 3: if (iz < 10.0 * g.invL) return 0; if (iz < 15.0 * g.invL) return 1; if (iz < 25.0 * g.invL) return 2; return 0;
      default: return 0;
    }
  }
  __device__ double Density(int im) const { return im > -1 ? density[im] : 1.0E-40; }
  __device__ double DensityAt(const int*, int im) const { return Density(im); }
  __device__ double Wscale() const { return 1.0; }
  __device__ void Score(double e, const int* i) const {
    const int iz = i[2];
    if (iz >= 0 && iz < cap) {
      atomicAdd(edep + iz, e);
      atomicAdd(steps + iz, 1.0);
      if (iz >= 20) atomicMax(maxIz, iz);
    }
  }
};

// Voxel box: the world is the box, vacuum outside (same push semantics)
// Geom::DistanceToBoundary (Geom.cc:20-117) on the phantom's lattice: the
// index from the position relative to the centre of voxel 0 (lower corner +
// half a voxel), the distance to the walls from the position relative to the
// voxel's centre, as the reference computes both for its own lattice
struct GridGeo {
  GridGeom g;
  double ivx, ivy, ivz;
  const double* density;
  double* tally;
  __device__ double DistanceToBoundary(double* r, const double* v, int* i) const {
    const double kTol = 1.0E-4, kHalfTol = 0.5 * kTol;
    const double o[3] = {g.x0, g.y0, g.z0}, s[3] = {g.vx, g.vy, g.vz}, is[3] = {ivx, ivy, ivz};
    const int n[3] = {g.nx, g.ny, g.nz};
    for (int guard = 0; guard < 64; ++guard) {
      for (int a = 0; a < 3; ++a)
        if (r[a] < o[a] || r[a] > o[a] + n[a] * s[a]) return -1.0;
      double tr[3];
      for (int a = 0; a < 3; ++a) {
        const double h = 0.5 * s[a];
        const double q = r[a] - (o[a] + 0.5 * s[a]);
        i[a] = int(floor((q + h) * is[a]));
        tr[a] = q - i[a] * s[a];
      }
      double snext = 1.0E+20;
      bool pushed = false;
      for (int a = 0; a < 3 && !pushed; ++a) {
        const double h = 0.5 * s[a];
        if (v[a] > 0.0) {
          const double pd = h - tr[a];
          if (pd < kHalfTol) { r[a] += kTol; pushed = true; }
          else { const double q = pd / v[a]; if (q < snext) snext = q; }
        } else if (v[a] < 0.0) {
          const double pd = h + tr[a];
          if (pd < kHalfTol) { r[a] -= kTol; pushed = true; }
          else { const double q = -pd / v[a]; if (q < snext) snext = q; }
        }
      }
      if (!pushed) return snext;
    }
    return -1.0;
  }
  __device__ bool Inside(const int* i) const {
    return i[0] >= 0 && i[0] < g.nx && i[1] >= 0 && i[1] < g.ny && i[2] >= 0 && i[2] < g.nz;
  }
  __device__ int MaterialIndex(const int* i) const {
    if (!Inside(i)) return -1;
    const uint8_t m = g.mat[(size_t(i[2]) * g.ny + i[1]) * g.nx + i[0]];
    return m == kVacuum ? -1 : int(m);
  }
  __device__ double Density(int im) const { return im > -1 ? density[im] : 1.0E-40; }
  // Geom::GetVoxelMaterialDensity(iVoxel) (Geom.hh:89-92) with per-voxel densities
  __device__ double DensityAt(const int* i, int im) const {
    if (g.rho && im > -1) return double(g.rho[(size_t(i[2]) * g.ny + i[1]) * g.nx + i[0]]);
    return Density(im);
  }
  __device__ double Wscale() const { return g.wscale; }
  __device__ void Score(double e, const int* i) const {
    if (Inside(i)) atomicAdd(tally + (size_t(i[2]) * g.ny + i[1]) * g.nx + i[0], e);
  }
};

template <class G>
struct HistorySim {
  const DevTables<double>& T;
  const G& geom;
  HistoryRng& rng;
  TrackD* stack;
  int sp = 0;
  double deposited = 0.0, escaped = 0.0;
  long long steps = 0;
  int lost = 0;
  __device__ HistorySim(const DevTables<double>& t, const G& g, HistoryRng& r, TrackD* s)
      : T(t), geom(g), rng(r), stack(s) {}

  __device__ TrackD* Push(const TrackD& parent, int type, double e) {
    if (sp >= kStackDepth) {          // overflow: the secondary is dropped and counted
      ++lost;
      escaped += e;
      return nullptr;
    }
    TrackD& t = stack[sp++];
    t = parent;
    t.type = type;
    t.ekin = e;
    return &t;
  }
  __device__ void Score(double e, const int* box) { geom.Score(e, box); deposited += e; }
  __device__ void Escape(const TrackD& t) { escaped += t.ekin + (t.type == +1 ? 2.0 * 0.510991 : 0.0); }

  // SimDPMLike.cc:753-791
  __device__ void Annihilate(const TrackD& t) {
    const double kPI = 3.1415926535897932, kEMC2 = 0.510991;
    const double cost = 1.0 - 2.0 * rng.U();
    const double sint = sqrt((1.0 - cost) * (1.0 + cost));
    const double phi = 2.0 * kPI * rng.U();
    double sn, cs;
    sincos(phi, &sn, &cs);
    const double rx = sint * cs, ry = sint * sn, rz = cost;
    if (TrackD* a = Push(t, 0, kEMC2)) { a->dir[0] = rx; a->dir[1] = ry; a->dir[2] = rz; }
    if (TrackD* b = Push(t, 0, kEMC2)) { b->dir[0] = -rx; b->dir[1] = -ry; b->dir[2] = -rz; }
  }
  // SimDPMLike.cc:661-695 (the three sampler arguments are drawn last-first)
  __device__ void Brem(TrackD& t) {
    const double kPI = 3.1415926535897932, kEMC2 = 0.510991, kHalfSqrt2EMC2 = kEMC2 * 0.7071067812;
    const double r3 = rng.U(), r2 = rng.U(), r1 = rng.U();
    const double eg = SampleSB(T.sb[t.mat], t.ekin, r1, r2, r3);
    TrackD* a = Push(t, 0, eg);
    const double dum0 = kHalfSqrt2EMC2 / (t.ekin + kEMC2);
    const double cost = fmax(-1.0, fmin(1.0, 1.0 - dum0 * dum0));
    const double sint = sqrt((1.0 + cost) * (1.0 - cost));
    const double phi = 2.0 * kPI * rng.U();
    if (a) {
      double sn, cs;
      sincos(phi, &sn, &cs);
      a->dir[0] = sint * cs; a->dir[1] = sint * sn; a->dir[2] = cost;
      RotateToLab(a->dir[0], a->dir[1], a->dir[2], t.dir[0], t.dir[1], t.dir[2]);
    }
    t.ekin = t.ekin - eg;
  }
  // SimDPMLike.cc:699-728
  __device__ void Moller(TrackD& t) {
    const double kPI = 3.1415926535897932, k2EMC2 = 2.0 * 0.510991;
    const double r3 = rng.U(), r2 = rng.U(), r1 = rng.U();
    const double se = SampleMoller(T.mol, t.ekin, r1, r2, r3);
    const double cost = sqrt(se * (t.ekin + k2EMC2) / (t.ekin * (se + k2EMC2)));
    const double sc = fmin(1.0, cost);
    TrackD* a = Push(t, -1, se);
    const double sint = sqrt((1.0 + sc) * (1.0 - sc));
    const double phi = 2.0 * kPI * rng.U();
    if (a) {
      double sn, cs;
      sincos(phi, &sn, &cs);
      a->dir[0] = sint * cs; a->dir[1] = sint * sn; a->dir[2] = sc;
      RotateToLab(a->dir[0], a->dir[1], a->dir[2], t.dir[0], t.dir[1], t.dir[2]);
    }
    t.ekin -= se;
  }
  // SimDPMLike.cc:731-750
  __device__ void MSC(TrackD& t, double ekin0) {
    const double kPI = 3.1415926535897932;
    const double r2 = rng.U(), r1 = rng.U();
    const double d = SampleGS(T.gs, ekin0, r1, r2);
    const double cost = fmax(-1.0, fmin(1.0, d));
    const double sint = sqrt((1.0 - cost) * (1.0 + cost));
    const double phi = 2.0 * kPI * rng.U();
    double sn, cs;
    sincos(phi, &sn, &cs);
    double u1 = sint * cs, u2 = sint * sn, u3 = cost;
    RotateToLab(u1, u2, u3, t.dir[0], t.dir[1], t.dir[2]);
    t.dir[0] = u1; t.dir[1] = u2; t.dir[2] = u3;
  }

  // SimDPMLike.cc:254-460
  __device__ int KeepTrackingElectron(TrackD& t, double& nTr1, double& nMol, double invMol, double& nBrem) {
    int what = 0;
    double sGeom = geom.DistanceToBoundary(t.pos, t.dir, t.box);
    if (sGeom < 0.0) { Escape(t); t.ekin = 0.0; return 4; }
    for (int guard = 0; what == 0; ++guard) {
      if (guard > 1000000) { ++lost; escaped += t.ekin; t.ekin = 0.0; return 4; }
      double step = sGeom;
      int im = geom.MaterialIndex(t.box);
      if (im < 0) { Escape(t); t.ekin = 0.0; return 4; }
      t.mat = im;
      ++steps;
      const double scal = T.mollerScale[im];
      const double rho = geom.DensityAt(t.box, im);
      double dedx = SplineGet(T.dedx[im], t.ekin) * rho;
      double emid = fmax(t.ekin - 0.5 * step * dedx, T.ecut);
      double dTr1 = SplineGet(T.itr1[im], emid) * rho;
      const double dMol = invMol * scal * rho;
      const double dBrem = SplineGet(T.brem[im], emid) * rho;
      const double sBrem = nBrem / dBrem;
      if (sBrem < step) { step = sBrem; what = 1; }
      const double sMol = nMol / dMol;
      if (sMol < step) { step = sMol; what = 2; }
      double sEl = nTr1 / dTr1;
      if (sEl < step) {
        sEl = nTr1 / (SplineGet(T.itr1[im], t.ekin) * rho);
        emid = fmax(t.ekin - 0.5 * sEl * dedx, T.ecut);
        dTr1 = SplineGet(T.itr1[im], emid) * rho;
        sEl = fmin(step, nTr1 / dTr1);
        step = sEl;
        what = 3;
      }
      nBrem = (what == 1) ? 0 : nBrem - step * dBrem;
      nMol = (what == 2) ? 0 : nMol - step * dMol;
      nTr1 = (what == 3) ? 0 : nTr1 - step * dTr1;
      emid = fmax(t.ekin - 0.5 * step * dedx, T.ecut);
      dedx = SplineGet(T.dedx[im], emid) * rho;
      const double de = step * dedx;
      const double ef = t.ekin - de;
      double edep;
      if (ef < T.ecut) {
        edep = t.ekin;
        t.ekin = 0.0;
        if (t.type == +1) {
          t.pos[0] += t.dir[0] * step; t.pos[1] += t.dir[1] * step; t.pos[2] += t.dir[2] * step;
          geom.DistanceToBoundary(t.pos, t.dir, t.box);
          im = geom.MaterialIndex(t.box);
          if (im < 0) { escaped += edep + 2.0 * 0.510991; return 4; }
          t.mat = im;
          Annihilate(t);
        }
        what = 4;
      } else {
        t.ekin = ef;
        edep = de;
      }
      t.pos[0] += t.dir[0] * step; t.pos[1] += t.dir[1] * step; t.pos[2] += t.dir[2] * step;
      Score(edep, t.box);
      if (what == 0) {
        sGeom = geom.DistanceToBoundary(t.pos, t.dir, t.box);
        if (sGeom < 0.0) { Escape(t); t.ekin = 0.0; return 4; }
      }
    }
    return what;
  }

  // SimDPMLike.cc:463-635
  __device__ void KeepTrackingPhoton(TrackD& t) {
    const double kPI = 3.1415926535897932, kEMC2 = 0.510991, kInvEMC2 = 1.0 / kEMC2;
    for (int guard = 0; t.ekin > 0.0; ++guard) {
      if (guard > 1000000) { ++lost; escaped += t.ekin; t.ekin = 0.0; return; }
      const double lmax = 1.0 / (LinearGet(T.imfpMax, t.ekin) * geom.Wscale());
      const double step = -lmax * log(rng.U());
      t.pos[0] += t.dir[0] * step; t.pos[1] += t.dir[1] * step; t.pos[2] += t.dir[2] * step;
      if (geom.DistanceToBoundary(t.pos, t.dir, t.box) < 0) { Escape(t); t.ekin = 0.0; return; }
      const int im = geom.MaterialIndex(t.box);
      if (im < 0) { Escape(t); t.ekin = 0.0; return; }
      t.mat = im;
      const double rho = geom.DensityAt(t.box, im);
      const double tot = LinearGet(T.tot[im], t.ekin) * rho;
      const double r1 = rng.U();
      double prob = 1.0 - tot * lmax;
      if (r1 < prob) continue;
      prob += LinearGet(T.comp[im], t.ekin) * rho * lmax;
      if (r1 < prob) {
        const double a3 = rng.U(), a2 = rng.U(), a1 = rng.U();
        const double eps = SampleKN(T.kn, t.ekin, a1, a2, a3);
        const double kappa = t.ekin * kInvEMC2;
        const double phCost = 1.0 - (1.0 - eps) / (eps * kappa);
        const double phE = eps * t.ekin;
        const double phPhi = 2.0 * kPI * rng.U();
        const double elE = t.ekin - phE;
        if (elE < T.ecut) {
          Score(elE, t.box);
        } else {
          const double e0 = t.ekin * kInvEMC2;
          const double elCost = (1.0 + e0) * sqrt((1.0 - eps) / (e0 * (2.0 + e0 * (1.0 - eps))));
          if (TrackD* a = Push(t, -1, elE)) {
            const double sint = sqrt((1.0 + elCost) * (1.0 - elCost));
            const double phi = phPhi + kPI;
            double sn, cs;
            sincos(phi, &sn, &cs);
            a->dir[0] = sint * cs; a->dir[1] = sint * sn; a->dir[2] = elCost;
            RotateToLab(a->dir[0], a->dir[1], a->dir[2], t.dir[0], t.dir[1], t.dir[2]);
          }
        }
        t.ekin = phE;
        if (t.ekin < T.gcut) {
          Score(t.ekin, t.box);
          t.ekin = 0.0;
          return;
        }
        const double phSint = sqrt((1.0 - phCost) * (1.0 + phCost));
        double sn, cs;
        sincos(phPhi, &sn, &cs);
        double u1 = phSint * cs, u2 = phSint * sn, u3 = phCost;
        RotateToLab(u1, u2, u3, t.dir[0], t.dir[1], t.dir[2]);
        t.dir[0] = u1; t.dir[1] = u2; t.dir[2] = u3;
        continue;
      }
      prob += LinearGet(T.pair[im], t.ekin) * rho * lmax;
      if (r1 < prob) {
        const double sum = t.ekin - 2.0 * kEMC2;
        const double e1 = rng.U() * sum;
        const double e2 = sum - e1;
        if (e2 < T.ecut) Score(e2, t.box);
        else Push(t, -1, e2);
        if (e1 < T.ecut) { Score(e1, t.box); Annihilate(t); }
        else Push(t, +1, e1);
        t.ekin = 0.0;
        return;
      }
      Score(t.ekin, t.box);
      t.ekin = 0.0;
    }
  }

  // SimDPMLike.cc:81-246
  __device__ void History(const TrackD& primary) {
    sp = 0;
    stack[sp++] = primary;
    while (sp > 0) {
      TrackD t = stack[--sp];
      geom.DistanceToBoundary(t.pos, t.dir, t.box);
      int im = geom.MaterialIndex(t.box);
      if (im < 0) { Escape(t); continue; }
      t.mat = im;
      if (t.type == 0) { KeepTrackingPhoton(t); continue; }
      bool hinge = true;
      double ekin0 = t.ekin;
      double nTr1 = SplineGet(T.k1, t.ekin);
      double nTr10 = rng.U() * nTr1;
      nTr1 -= nTr10;
      double nMol = -log(rng.U());
      double invMol = SplineGet(T.moller, t.ekin);
      double nBrem = -log(rng.U());
      while (t.ekin > 0.0) {
        const int what = KeepTrackingElectron(t, nTr1, nMol, invMol, nBrem);
        switch (what) {
          case 1:
            if (t.ekin > T.gcut) Brem(t);
            if (t.ekin < T.ecut) {
              Score(t.ekin, t.box);
              t.ekin = 0.0;
              if (t.type == +1) Annihilate(t);
              break;
            }
            nBrem = -log(rng.U());
            break;
          case 2:
            if (t.ekin > 2. * T.ecut) Moller(t);
            nMol = -log(rng.U());
            invMol = SplineGet(T.moller, t.ekin);
            break;
          case 3:
            if (hinge) {
              MSC(t, ekin0);
              nTr1 = nTr10;
              hinge = false;
            } else {
              ekin0 = t.ekin;
              nTr1 = SplineGet(T.k1, ekin0);
              nTr10 = rng.U() * nTr1;
              nTr1 -= nTr10;
              hinge = true;
            }
            break;
          default:
            break;
        }
      }
    }
  }
};

// primary of history h for a voxel job (same draw order as the oracle's SamplePrimary)
__device__ void SamplePrimaryD(const SourceD& s, long long h, HistoryRng& rng, TrackD& t) {
  double x = s.cx, y = s.cy;
  if (s.shape == 1) {
    x = s.cx + (rng.U() - 0.5) * s.fx;
    y = s.cy + (rng.U() - 0.5) * s.fy;
  } else if (s.shape == 2) {
    const int nb = s.nbx * s.nby;
    const int b = int(h % nb);
    const int bx = b % s.nbx, by = b / s.nbx;
    x = s.cx + (bx - 0.5 * s.nbx) * s.fx + rng.U() * s.fx;
    y = s.cy + (by - 0.5 * s.nby) * s.fy + rng.U() * s.fy;
  }
  double e = s.e0;
  if (s.spectrum == 1) e = s.e0 + rng.U() * (s.e1 - s.e0);
  else if (s.spectrum == 2) e = s.e1 - (s.e1 - s.e0) * sqrt(1.0 - rng.U());
  t.pos[0] = x; t.pos[1] = y; t.pos[2] = s.zEntry;
  t.dir[0] = 0.0; t.dir[1] = 0.0; t.dir[2] = 1.0;
  t.box[0] = t.box[1] = t.box[2] = 0;
  t.type = s.particle;
  t.mat = -1;
  t.ekin = e;
}

template <class G>
__device__ void RunHistories(const DevTables<double>& T, const G& geom, const SourceD& src, long long first,
                             long long n, uint64_t seed, bool slabSource, double lbox, double* histEdep,
                             RunCounters* cnt) {
  TrackD stack[kStackDepth];
  double dep = 0.0, esc = 0.0, e0sum = 0.0, maxres = 0.0;
  long long steps = 0, viol = 0;
  int lost = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
    const long long h = first + k;
    HistoryRng rng;
    rng.Init(seed, uint32_t(h));
    TrackD p;
    if (slabSource) {   // SimDPMLike.cc:64-75
      p.pos[0] = 0.0; p.pos[1] = 0.0; p.pos[2] = -0.5 * lbox;
      p.dir[0] = 0.0; p.dir[1] = 0.0; p.dir[2] = 1.0;
      p.box[0] = p.box[1] = p.box[2] = 0;
      p.type = src.particle; p.mat = -1; p.ekin = src.e0;
    } else {
      SamplePrimaryD(src, h, rng, p);
    }
    HistorySim<G> sim(T, geom, rng, stack);
    sim.History(p);
    if (histEdep) histEdep[k] = sim.deposited;
    dep += sim.deposited;
    esc += sim.escaped;
    e0sum += p.ekin;
    steps += sim.steps;
    lost += sim.lost;
    const double res = fabs(p.ekin - sim.deposited - sim.escaped);
    maxres = fmax(maxres, res);
    if (res > 1.0e-3 * p.ekin) ++viol;
  }
  AccumulateCounters(cnt, dep, esc, e0sum, maxres, steps, viol, lost);
}

// six blocks of 128 threads per SM (80 registers, 24 warps): the history
// loop waits on its FP64 arithmetic and its local-memory secondary stack, and
// more resident warps hide it (slab workload 1.35e6 against 9.0e5 histories/s
// at 4 blocks and 128 registers; 8 blocks spill 1 KB)
__global__ void __launch_bounds__(128, 6) SlabKernel(DevTables<double> T, SlabGeo geom, SourceD src, long long first,
                                                  long long n, uint64_t seed, double lbox, double* histEdep,
                                                  RunCounters* cnt) {
  RunHistories(T, geom, src, first, n, seed, true, lbox, histEdep, cnt);
}

__global__ void __launch_bounds__(128, 6) GridKernel(DevTables<double> T, GridGeo geom, SourceD src, long long first,
                                                  long long n, uint64_t seed, double* histEdep, RunCounters* cnt) {
  RunHistories(T, geom, src, first, n, seed, false, 0.0, histEdep, cnt);
}

// ---- tier-1 evaluation kernels (FP64) ----
__global__ void SamplerKernel64(DevTables<double> T, int s, int imat, const double* e, const double* r, double* out,
                                int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* u = r + 3 * i;
  double v = 0.0;
  switch (s) {
    case 0: v = SampleKN(T.kn, e[i], u[0], u[1], u[2]); break;
    case 1: v = SampleMoller(T.mol, e[i], u[0], u[1], u[2]); break;
    case 2: v = SampleSB(T.sb[imat], e[i], u[0], u[1], u[2]); break;
    case 3: v = SampleGS(T.gs, e[i], u[0], u[1]); break;
    default: break;
  }
  out[i] = v;
}

__global__ void TableKernel64(DevTables<double> T, int q, int imat, const double* e, double* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = 0.0;
  switch (q) {
    case 0: v = SplineGet(T.dedx[imat], e[i]); break;
    case 1: v = SplineGet(T.itr1[imat], e[i]); break;
    case 2: v = SplineGet(T.brem[imat], e[i]); break;
    case 3: v = SplineGet(T.moller, e[i]); break;
    case 4: v = SplineGet(T.k1, e[i]); break;
    case 5: v = LinearGet(T.imfpMax, e[i]); break;
    case 6: v = LinearGet(T.tot[imat], e[i]); break;
    case 7: v = LinearGet(T.comp[imat], e[i]); break;
    case 8: v = LinearGet(T.pair[imat], e[i]); break;
    default: break;
  }
  out[i] = v;
}

}  // namespace

cudaError_t LaunchFp64Slab(const DevTables<double>& T, const SlabGeomD& g, const double* density, const SourceD& src,
                           long long first, long long n, uint64_t seed, double* edep, double* steps, int cap,
                           int* maxIz, double* histEdep, RunCounters* cnt, int blocks, cudaStream_t st) {
  SlabGeo geo{g, density, edep, steps, cap, maxIz};
  SlabKernel<<<blocks, 128, 0, st>>>(T, geo, src, first, n, seed, g.L, histEdep, cnt);
  return cudaGetLastError();
}

cudaError_t LaunchFp64Grid(const DevTables<double>& T, const GridGeom& g, const double* density, const SourceD& src,
                           long long first, long long n, uint64_t seed, double* tally, double* histEdep,
                           RunCounters* cnt, int blocks, cudaStream_t st) {
  GridGeo geo{g, 1.0 / g.vx, 1.0 / g.vy, 1.0 / g.vz, density, tally};
  GridKernel<<<blocks, 128, 0, st>>>(T, geo, src, first, n, seed, histEdep, cnt);
  return cudaGetLastError();
}

cudaError_t LaunchSamplerEval64(const DevTables<double>& T, int s, int imat, const double* e, const double* r,
                                double* out, int n, cudaStream_t st) {
  SamplerKernel64<<<(n + 127) / 128, 128, 0, st>>>(T, s, imat, e, r, out, n);
  return cudaGetLastError();
}

cudaError_t LaunchTableEval64(const DevTables<double>& T, int q, int imat, const double* e, double* out, int n,
                              cudaStream_t st) {
  TableKernel64<<<(n + 127) / 128, 128, 0, st>>>(T, q, imat, e, out, n);
  return cudaGetLastError();
}

}  // namespace dpmx
