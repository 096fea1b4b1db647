// CPU oracle for the dpm_Simulate transport path. TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain double-precision C++, the reference's
// simulation phase so that the GPU implementation can be checked against it:
//   * data loaders   Simulation/src/Sim*.cc (LoadData / Load), SimDataSpline.cc:33-67
//   * samplers       SimLinAliasData.cc:25-42, SimKNTables.cc:69-90,
//                    SimMollerTables.cc:69-89, SimSBTables.cc:93-114,
//                    SimGSTables.cc:84-119
//   * geometry       Geom.cc:20-164 (pre-defined slab geometries), plus a 3-D
//                    voxel geometry with the same boundary/push semantics
//   * transport      SimDPMLike.cc:40-791 (Simulate, KeepTrackingElectron,
//                    KeepTrackingPhoton, RotateToLabFrame, Perform*)
// Only the tests, the smoke check and the benchmark's CPU-baseline leg use it;
// the product path never does.
//
// The reference passes three fresh uniforms as the arguments of each sampler
// call (e.g. SimDPMLike.cc:666-670); g++ evaluates call arguments right to
// left, so the LAST parameter receives the FIRST draw. The draw order here is
// written out explicitly to match that build.
//
// Two random-number streams are provided:
//   * "mt"     : one global std::mt19937 + uniform_real_distribution<double>,
//                consumed in the reference's order (Random.cc:3-4). With the same
//                seed this reproduces the reference bit for bit.
//   * "philox" : one Philox-4x32-10 stream per history (key = seed, counter =
//                {block, 0, 0, history}), the stream the FP64 GPU kernel uses,
//                so GPU and oracle histories can be compared one by one.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------------------
// Interpolation tables
// ---------------------------------------------------------------------------
// Natural cubic spline on a log-uniform grid (SimDataSpline.hh:38-50,
// coefficients as in SimDataSpline.cc:33-67).
struct Spline {
  int n = 0;
  double logMin = 0, invLogDelta = 0;
  std::vector<double> x, y, b, c, d;
  void Set(const std::vector<double>& xs, const std::vector<double>& ys) {
    n = int(xs.size());
    x = xs; y = ys;
    b.assign(n, 0.0); c.assign(n, 0.0); d.assign(n, 0.0);
    logMin = std::log(x[0]);
    invLogDelta = 1. / (std::log(x[1]) - logMin);
    // tridiagonal elimination of the natural spline, then the cubic coefficients
    const int m2 = n - 1;
    double s = 0.0, r = 0.0;
    for (int m = 0; m < m2; ++m) {
      d[m] = x[m + 1] - x[m];
      r = (y[m + 1] - y[m]) / d[m];
      c[m] = r - s;
      s = r;
    }
    r = 0.0; s = 0.0;
    c[0] = 0.0; c[m2] = 0.0;
    for (int m = 1; m < m2; ++m) {
      c[m] = c[m] + r * c[m - 1];
      b[m] = 2.0 * (x[m - 1] - x[m + 1]) - r * s;
      s = d[m];
      r = s / b[m];
    }
    int mr = m2 - 1;
    for (int m = 1; m < m2; ++m) {
      c[mr] = (d[mr] * c[mr + 1] - c[mr]) / b[mr];
      --mr;
    }
    for (int m = 0; m < m2; ++m) {
      s = d[m];
      r = c[m + 1] - c[m];
      d[m] = r / s;
      c[m] = 3.0 * c[m];
      b[m] = (y[m + 1] - y[m]) / s - (c[m] + r) * s;
    }
  }
  double At(double xv, int il) const {
    xv -= x[il];
    return y[il] + xv * (b[il] + xv * (c[il] + xv * d[il]));
  }
  double Value(double xv) const {
    const double lx = std::log(xv);
    int il = (int)((lx - logMin) * invLogDelta);
    il = std::max(0, std::min(n - 2, il));
    return At(xv, il);
  }
};

// Linear interpolation on a linear-uniform grid (SimDataLinear.hh:38-45)
struct Linear {
  int n = 0;
  double xMin = 0, invDelta = 0;
  std::vector<double> x, y;
  void Set(const std::vector<double>& xs, const std::vector<double>& ys) {
    n = int(xs.size()); x = xs; y = ys;
    xMin = x[0];
    invDelta = 1. / (x[1] - xMin);
  }
  double Value(double xv) const {
    int il = (int)((xv - xMin) * invDelta);
    il = std::max(0, std::min(n - 2, il));
    return (y[il + 1] - y[il]) * (xv - x[il]) / (x[il + 1] - x[il]) + y[il];
  }
};

// Walker alias + linear pdf sampling table (SimLinAliasData.cc:25-42)
struct LinAlias {
  std::vector<double> x, y, w;
  std::vector<int> idx;
  double Sample(double r1, double r2) const {
    const int n = int(x.size());
    const double rest = r1 * (n - 1);
    int il = (int)(rest);
    if (w[il] < rest - il) il = idx[il];
    const double xv = x[il];
    const double xd = x[il + 1] - xv;
    if (y[il] > 0.0) {
      const double dum = (y[il + 1] - y[il]) / y[il];
      if (std::abs(dum) > 0.1) return xv - xd / dum * (1.0 - std::sqrt(1.0 + r2 * dum * (dum + 2.0)));
      return xv + r2 * xd * (1.0 - 0.5 * dum * (r2 - 1.0) * (1.0 + dum * r2));
    }
    return xv + xd * std::sqrt(r2);
  }
};

// A spline quantity with the loaders' energy clamp and 1e-20 floor, e.g.
// SimStoppingPower.hh:43-49: e = min(Emax-1e-6, max(Emin, E)).
struct Clamped {
  Spline sp;
  double emin = 0, emax = 0;
  double Get(double e) const { return std::max(1.0E-20, sp.Value(std::min(emax - 1.0E-6, std::max(emin, e)))); }
};
struct ClampedLin {
  Linear li;
  double emin = 0, emax = 0;
  double Get(double e) const { return std::max(1.0E-20, li.Value(std::min(emax - 1.0E-6, std::max(emin, e)))); }
};

struct EGridTables {         // shared layout of the KN / Moller / SB / GS energy grids
  int numE = 0, numS = 0;
  double minE = 0, logMinE = 0, invLogDeltaE = 0;
};

struct Tables {
  // mat.dat (SimMaterialData.cc:6-53)
  double ecut = 0, gcut = 0, slow = 0, shigh = 0, ecross = 0;
  int nmat = 0;
  std::vector<std::string> names;
  std::vector<double> density, mollerScale;
  // electron spline data
  std::vector<Clamped> itr1, dedx, brem;   // per material
  Clamped k1, moller;                      // reference material only
  // photon linear data
  ClampedLin imfpMax;
  std::vector<ClampedLin> imfpTot, imfpCompton, imfpPair;
  // sampling tables
  EGridTables kn, mol, sb, gs;
  std::vector<LinAlias> knT, molT;
  std::vector<std::vector<LinAlias>> sbT;  // [mat][E]
  std::vector<double> gsE, gsA;            // per-E transform parameter
  std::vector<std::vector<double>> gsU, gsPA, gsPB;
  double gsDeltaCum = 0;
  std::string error;
};

// ---------------------------------------------------------------------------
// Loaders: the same header-skip and field order as the reference readers.
// ---------------------------------------------------------------------------
struct File {
  FILE* f = nullptr;
  char buf[512];
  bool ok = true;
  File(const std::string& dir, const char* name) {
    std::string p = dir + "/" + name;
    f = std::fopen(p.c_str(), "r");
    ok = f != nullptr;
  }
  ~File() { if (f) std::fclose(f); }
  void Skip(int n) { for (int i = 0; i < n && ok; ++i) ok = std::fgets(buf, sizeof(buf), f) != nullptr; }
  int I() { int v = 0; if (ok && std::fscanf(f, "%d", &v) != 1) ok = false; return v; }
  double D() { double v = 0; if (ok && std::fscanf(f, "%lg", &v) != 1) ok = false; return v; }
  std::string S() { char s[256] = {0}; if (ok && std::fscanf(f, "%255s", s) != 1) ok = false; return s; }
  void EatLine() { if (ok) { int ch; while ((ch = std::fgetc(f)) != EOF && ch != '\n') {} } }
};

bool LoadSplinePerMat(const std::string& dir, const char* name, int nskip, int valCol, std::vector<Clamped>& out) {
  // el_itr1mfp (3 columns, value = 3rd), eloss_rdedx, imfp_brem (2 columns)
  File f(dir, name);
  if (!f.ok) return false;
  f.Skip(nskip);
  const int n = f.I(), nm = f.I();
  f.EatLine();
  f.Skip(1);
  out.resize(nm);
  for (int im = 0; im < nm; ++im) {
    f.Skip(3);
    std::vector<double> xs(n), ys(n);
    for (int i = 0; i < n; ++i) {
      xs[i] = f.D();
      double a = f.D();
      if (valCol == 3) a = f.D();
      ys[i] = a;
      f.EatLine();
    }
    if (!f.ok) return false;
    out[im].sp.Set(xs, ys);
    out[im].emin = xs[0];
    out[im].emax = xs[n - 1];
  }
  // the reference takes Emin/Emax from material 0's grid
  for (auto& c : out) { c.emin = out[0].emin; c.emax = out[0].emax; }
  return f.ok;
}

bool LoadSplineRef(const std::string& dir, const char* name, int nskip1, int nskip2, Clamped& out) {
  // el_scatStrength (4 + N + 4), imfp_moller (3 + N + 4): only the first block
  File f(dir, name);
  if (!f.ok) return false;
  f.Skip(nskip1);
  const int n = f.I();
  f.EatLine();
  f.Skip(nskip2);
  std::vector<double> xs(n), ys(n);
  for (int i = 0; i < n; ++i) { xs[i] = f.D(); ys[i] = f.D(); }
  if (!f.ok) return false;
  out.sp.Set(xs, ys);
  out.emin = xs[0];
  out.emax = xs[n - 1];
  return true;
}

bool LoadLinearPerMat(const std::string& dir, const char* name, std::vector<ClampedLin>& out) {
  File f(dir, name);   // SimIMFPPhoton.cc:19-62
  if (!f.ok) return false;
  f.Skip(3);
  const int n = f.I(), nm = f.I();
  f.EatLine();
  f.Skip(1);
  out.resize(nm);
  for (int im = 0; im < nm; ++im) {
    f.Skip(3);
    std::vector<double> xs(n), ys(n);
    for (int i = 0; i < n; ++i) { xs[i] = f.D(); ys[i] = f.D(); f.EatLine(); }
    if (!f.ok) return false;
    out[im].li.Set(xs, ys);
    out[im].emin = xs[0];
    out[im].emax = xs[n - 1];
  }
  for (auto& c : out) { c.emin = out[0].emin; c.emax = out[0].emax; }
  return true;
}

bool LoadAliasTables(const std::string& dir, const char* name, EGridTables& g, std::vector<LinAlias>& out) {
  File f(dir, name);   // SimKNTables.cc:20-66, SimMollerTables.cc:20-66
  if (!f.ok) return false;
  f.Skip(5);
  g.numE = f.I(); g.numS = f.I();
  out.resize(g.numE);
  for (int ie = 0; ie < g.numE; ++ie) {
    const double e = f.D();
    if (ie == 0) { g.minE = e; g.logMinE = std::log(e); }
    if (ie == 1) g.invLogDeltaE = 1. / (std::log(e) - g.logMinE);
    LinAlias& t = out[ie];
    t.x.resize(g.numS); t.y.resize(g.numS); t.w.resize(g.numS); t.idx.resize(g.numS);
    for (int is = 0; is < g.numS; ++is) { t.x[is] = f.D(); t.y[is] = f.D(); t.w[is] = f.D(); t.idx[is] = f.I(); }
  }
  return f.ok;
}

bool LoadSB(const std::string& dir, Tables& T) {
  File f(dir, "brem_SBDtrData.dat");   // SimSBTables.cc:21-90
  if (!f.ok) return false;
  f.Skip(5);
  T.sb.numE = f.I(); T.sb.numS = f.I();
  const int nm = f.I();
  for (int ie = 0; ie < T.sb.numE; ++ie) {
    const double e = f.D();
    if (ie == 0) { T.sb.minE = e; T.sb.logMinE = std::log(e); }
    if (ie == 1) T.sb.invLogDeltaE = 1. / (std::log(e) - T.sb.logMinE);
  }
  f.EatLine();
  T.sbT.assign(nm, std::vector<LinAlias>(T.sb.numE));
  for (int im = 0; im < nm; ++im) {
    f.Skip(3);
    for (int ie = 0; ie < T.sb.numE; ++ie) {
      LinAlias& t = T.sbT[im][ie];
      const int n = T.sb.numS;
      t.x.resize(n); t.y.resize(n); t.w.resize(n); t.idx.resize(n);
      for (int is = 0; is < n; ++is) { t.x[is] = f.D(); t.y[is] = f.D(); t.w[is] = f.D(); t.idx[is] = f.I(); }
    }
    f.EatLine();
  }
  return f.ok;
}

bool LoadGS(const std::string& dir, Tables& T) {
  File f(dir, "el_GSDtrData.dat");     // SimGSTables.cc:19-81
  if (!f.ok) return false;
  f.Skip(4);
  T.gs.numE = f.I();
  f.D(); f.D();
  T.gs.numS = f.I();
  f.EatLine();
  T.gsDeltaCum = 1.0 / (T.gs.numS - 1);
  f.Skip(6);
  const int ne = T.gs.numE, ns = T.gs.numS;
  T.gsE.resize(ne); T.gsA.resize(ne);
  T.gsU.assign(ne, std::vector<double>(ns));
  T.gsPA = T.gsU; T.gsPB = T.gsU;
  for (int ie = 0; ie < ne; ++ie) {
    f.I();
    const double e = f.D();
    T.gsA[ie] = f.D();
    T.gsE[ie] = e;
    if (ie == 0) { T.gs.minE = e; T.gs.logMinE = std::log(e); }
    if (ie == 1) T.gs.invLogDeltaE = 1. / (std::log(e) - T.gs.logMinE);
    for (int is = 0; is < ns; ++is) { T.gsU[ie][is] = f.D(); T.gsPA[ie][is] = f.D(); T.gsPB[ie][is] = f.D(); }
  }
  return f.ok;
}

bool LoadMaterials(const std::string& dir, Tables& T) {
  File f(dir, "mat.dat");              // SimMaterialData.cc:6-53
  if (!f.ok) return false;
  f.Skip(1);
  T.ecut = f.D(); T.gcut = f.D(); f.EatLine();
  f.Skip(1);
  T.slow = f.D(); T.shigh = f.D(); T.ecross = f.D(); f.EatLine();
  f.Skip(1);
  T.nmat = f.I(); f.EatLine();
  for (int im = 0; im < T.nmat; ++im) {
    f.Skip(2);
    f.I();
    T.names.push_back(f.S());
    T.density.push_back(f.D());
    f.EatLine();
    f.Skip(3);
    T.mollerScale.push_back(f.D());
    f.D();
    f.EatLine();
  }
  return f.ok;
}

Tables* Load(const std::string& dir) {
  Tables* T = new Tables();
  bool ok = LoadMaterials(dir, *T)
         && LoadSplinePerMat(dir, "el_itr1mfp.dat", 4, 3, T->itr1)
         && LoadSplineRef(dir, "el_scatStrength.dat", 4, 4, T->k1)
         && LoadSplineRef(dir, "imfp_moller.dat", 3, 4, T->moller)
         && LoadSplinePerMat(dir, "imfp_brem.dat", 3, 2, T->brem)
         && LoadSplinePerMat(dir, "eloss_rdedx.dat", 2, 2, T->dedx)
         && LoadAliasTables(dir, "ioni_MollerDtrData.dat", T->mol, T->molT)
         && LoadSB(dir, *T)
         && LoadGS(dir, *T);
  if (ok) {
    std::vector<ClampedLin> one;
    File f(dir, "imfp_globalMax.dat");   // SimIMFPMaxPhoton.cc:6-38
    ok = f.ok;
    if (ok) {
      f.Skip(3);
      const int n = f.I();
      f.EatLine();
      f.Skip(1);
      std::vector<double> xs(n), ys(n);
      for (int i = 0; i < n; ++i) { xs[i] = f.D(); ys[i] = f.D(); }
      ok = f.ok;
      if (ok) { T->imfpMax.li.Set(xs, ys); T->imfpMax.emin = xs[0]; T->imfpMax.emax = xs[n - 1]; }
    }
  }
  ok = ok && LoadLinearPerMat(dir, "imfp_total.dat", T->imfpTot)
          && LoadLinearPerMat(dir, "imfp_compton.dat", T->imfpCompton)
          && LoadLinearPerMat(dir, "imfp_pairp.dat", T->imfpPair)
          && LoadAliasTables(dir, "compton_KNDtrData.dat", T->kn, T->knT);
  if (!ok) { delete T; return nullptr; }
  return T;
}

// ---------------------------------------------------------------------------
// Samplers
// ---------------------------------------------------------------------------
constexpr double kPI = 3.1415926535897932;
constexpr double kEMC2 = 0.510991;

// SimKNTables.cc:69-90
double SampleKN(const Tables& T, double eg, double r1, double r2, double r3) {
  const double lp = std::log(eg);
  double ph = (lp - T.kn.logMinE) * T.kn.invLogDeltaE;
  int ie = (int)ph;
  ph -= ie;
  if (r1 < ph) ++ie;
  const double xi = T.knT[ie].Sample(r2, r3);
  const double kappa = eg / kEMC2;
  return std::exp(std::log(1. + 2. * kappa) * (xi - 1.));
}
// SimMollerTables.cc:69-89
double SampleMoller(const Tables& T, double ep, double r1, double r2, double r3) {
  const double lp = std::log(ep);
  double ph = (lp - T.mol.logMinE) * T.mol.invLogDeltaE;
  int ie = (int)ph;
  ph -= ie;
  if (r1 < ph) ++ie;
  const double xi = T.molT[ie].Sample(r2, r3);
  const double dum1 = lp - T.mol.logMinE;
  return std::exp(xi * dum1) * 0.5 * T.mol.minE;
}
// SimSBTables.cc:93-114
double SampleSB(const Tables& T, double ep, int imat, double r1, double r2, double r3) {
  if (imat < 0) return 0.0;
  const double lp = std::log(ep);
  double ph = (lp - T.sb.logMinE) * T.sb.invLogDeltaE;
  int ie = (int)ph;
  ph -= ie;
  if (r1 < ph) ++ie;
  const double xi = T.sbT[imat][ie].Sample(r2, r3);
  const double kc = T.sb.minE / ep;
  const double kappa = kc * std::exp(-xi * (T.sb.logMinE - lp));
  return kappa * ep;
}
// SimGSTables.cc:84-119
double SampleGS(const Tables& T, double ep, double r1, double r2) {
  const double lp = std::log(ep);
  double ph = (lp - T.gs.logMinE) * T.gs.invLogDeltaE;
  int ie = (int)ph;
  const int ielow = ie;
  ph -= ie;
  if (r1 < ph) ++ie;
  const double dc = T.gsDeltaCum;
  const int il = (int)(r2 / dc);
  const double resid = r2 - il * dc;
  const double pa = T.gsPA[ie][il], pb = T.gsPB[ie][il];
  const double u0 = T.gsU[ie][il], u1 = T.gsU[ie][il + 1];
  const double dum1 = (1.0 + pa + pb) * dc * resid;
  const double dum2 = dc * dc + pa * dc * resid + pb * resid * resid;
  const double u = u0 + dum1 / dum2 * (u1 - u0);
  const double a0 = T.gsA[ielow], a1 = T.gsA[ielow + 1];
  const double e0 = T.gsE[ielow], e1 = T.gsE[ielow + 1];
  const double a = (a1 - a0) / (e1 - e0) * (ep - e0) + a0;
  return 1. - 2. * a * u / (1. - u + a);
}

// ---------------------------------------------------------------------------
// Random numbers
// ---------------------------------------------------------------------------
struct MtRng {    // Random.cc:3-4
  std::mt19937 gen;
  std::uniform_real_distribution<double> dis{0.0, 1.0};
  explicit MtRng(uint32_t s) : gen(s) {}
  double U() { return dis(gen); }
  void BeginHistory(uint64_t) {}
};

// Philox-4x32-10 (Salmon et al., SC'11)
inline void Philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = uint64_t(0xD2511F53u) * c[0];
    const uint64_t p1 = uint64_t(0xCD9E8D57u) * c[2];
    const uint32_t n0 = uint32_t(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n1 = uint32_t(p1);
    const uint32_t n2 = uint32_t(p0 >> 32) ^ c[3] ^ k1;
    const uint32_t n3 = uint32_t(p0);
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
}
// draw k of history h: Philox block k/2 at counter {k/2, 0, 0, h}, words
// (2(k%2), 2(k%2)+1) -> 52-bit uniform on the open interval (0,1)
struct PhiloxRng {
  uint32_t k0, k1, hist = 0, block = 0;
  uint32_t w[4];
  int have = 0;
  explicit PhiloxRng(uint64_t seed) : k0(uint32_t(seed)), k1(uint32_t(seed >> 32)) {}
  void BeginHistory(uint64_t h) { hist = uint32_t(h); block = 0; have = 0; }
  double U() {
    if (have == 0) {
      w[0] = block++; w[1] = 0; w[2] = 0; w[3] = hist;
      Philox(w, k0, k1);
      have = 2;
    }
    const int j = 2 - have;
    --have;
    const uint64_t bits = (uint64_t(w[2 * j + 1]) << 32) | w[2 * j];
    return double((bits >> 11) | 1u) * (1.0 / 9007199254740992.0);
  }
};

// ---------------------------------------------------------------------------
// Geometry
// ---------------------------------------------------------------------------
// The reference's pre-defined slab geometries with its 1-D depth tally
// (Geom.cc:9-192, Geom.hh:107-109).
struct SlabGeom {
  int gi;
  double L, invL, halfL;
  const Tables* T;
  std::vector<double> edep, steps;
  static constexpr double kTol = 1.0E-4, kExtent = 100.0;
  SlabGeom(double lbox, const Tables* t, int geomIndex) : gi(geomIndex), L(lbox), invL(1. / lbox), halfL(0.5 * lbox), T(t) {
    edep.assign(20, 0.0); steps.assign(20, 0.0);
  }
  double DistanceToBoundary(double* r, const double* v, int* i) const {
    const double kHalfTol = 0.5 * kTol;
    for (;;) {   // the reference recurses after a push; loop instead
      if (std::abs(r[0]) > kExtent || std::abs(r[1]) > kExtent || r[2] > kExtent || r[2] < -L) return -1.0;
      i[0] = (int)std::floor((r[0] + halfL) * invL);
      i[1] = (int)std::floor((r[1] + halfL) * invL);
      i[2] = (int)std::floor((r[2] + halfL) * invL);
      const double tr[3] = {r[0] - i[0] * L, r[1] - i[1] * L, r[2] - i[2] * L};
      double snext = 1.0E+20;
      bool pushed = false;
      for (int a = 0; a < 3 && !pushed; ++a) {
        if (v[a] > 0.0) {
          const double pd = halfL - tr[a];
          if (pd < kHalfTol) { r[a] += kTol; pushed = true; }
          else { const double s = pd / v[a]; if (a == 0 || s < snext) snext = s; }
        } else if (v[a] < 0.0) {
          const double pd = halfL + tr[a];
          if (pd < kHalfTol) { r[a] -= kTol; pushed = true; }
          else { const double s = -pd / v[a]; if (a == 0 || s < snext) snext = s; }
        }
      }
      if (!pushed) return snext;
    }
  }
  int MaterialIndex(const int* i) const {
    const int iz = i[2];
    if (iz < 0) return -1;
    switch (gi) {
      case 1: if (iz < 10.0 * invL) return 0; if (iz < 30.0 * invL) return 1; return 0;
      case 2: if (iz < 20.0 * invL) return 0; if (iz < 40.0 * invL) return 1; return 0;
      case 3: if (iz < 10.0 * invL) return 0; if (iz < 15.0 * invL) return 1; if (iz < 25.0 * invL) return 2; return 0;
      default: return 0;
    }
  }
  double Density(int imat) const { return imat > -1 ? T->density[imat] : 1.0E-40; }
  double DensityAt(const int*, int imat) const { return Density(imat); }
  double Wscale() const { return 1.0; }
  void Score(double e, const int* i) {
    const int iz = i[2];
    if (iz >= 0) {
      const size_t k = size_t(iz);
      if (k >= edep.size()) { edep.resize(k + 10, 0.0); steps.resize(k + 10, 0.0); }
      edep[k] += e;
      steps[k] += 1.0;
    }
  }
};

// A 3-D voxel phantom: nx*ny*nz voxels of size (vx,vy,vz) whose lower corner
// is at (x0,y0,z0). Outside the world box is vacuum. The boundary arithmetic
// is Geom::DistanceToBoundary's (Geom.cc:20-117) on a lattice whose voxel of
// index 0 is centred at c (index = floor((r - c + s/2) / s), position relative
// to the voxel centre, distance s/2 -/+ that), so that the reference's own
// lattice (c = 0, world |x|,|y| <= 100 mm, -lbox <= z <= 100 mm) reproduces
// Geom bit for bit. By default c is the centre of the phantom's first voxel,
// the array starts at index 0 and the world is the phantom box.
struct VoxelGeom {
  int nx, ny, nz;
  double x0, y0, z0, vx, vy, vz;
  double ivx, ivy, ivz;
  const uint8_t* mat;
  const Tables* T;
  double* dose;      // [nvox] energy deposit
  double* tag;       // optional per-history accumulator (energy check)
  const float* rho = nullptr;   // per-voxel density or null
  double wscale = 1.0;          // Woodcock majorant scale for densities above nominal
  double c[3] = {0, 0, 0};      // centre of the voxel of lattice index 0
  int lo[3] = {0, 0, 0};        // lattice index of the array's first voxel
  double wlo[3] = {0, 0, 0}, whi[3] = {0, 0, 0};   // world box
  double* depth = nullptr;      // optional depth tally (energy, steps) in Geom::Score's order
  double* dsteps = nullptr;
  int dsize = 20;               // its length by Geom::Score's growth rule (+10 past a bin beyond it)
  double* btally = nullptr;     // optional beamlet-tagged tally [beamlet][voxel]
  int beamlet = 0;              // beamlet of the current history
  static constexpr double kTol = 1.0E-4;
  void SetDefaultLattice() {
    const double o[3] = {x0, y0, z0}, s[3] = {vx, vy, vz};
    const int n[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
      c[a] = o[a] + 0.5 * s[a];
      lo[a] = 0;
      wlo[a] = o[a];
      whi[a] = o[a] + n[a] * s[a];
    }
  }
  double DistanceToBoundary(double* r, const double* v, int* i) const {
    const double kHalfTol = 0.5 * kTol;
    const double s[3] = {vx, vy, vz}, is[3] = {ivx, ivy, ivz};
    for (;;) {   // Geom.cc recurses after a push; loop instead
      for (int a = 0; a < 3; ++a) {
        if (r[a] < wlo[a] || r[a] > whi[a]) return -1.0;
      }
      double tr[3];
      for (int a = 0; a < 3; ++a) {
        const double h = 0.5 * s[a];
        const double q = r[a] - c[a];
        i[a] = (int)std::floor((q + h) * is[a]);
        tr[a] = q - i[a] * s[a];     // in [-h, h)
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
  }
  size_t Flat(const int* i) const {
    return (size_t(i[2] - lo[2]) * ny + size_t(i[1] - lo[1])) * nx + size_t(i[0] - lo[0]);
  }
  bool Inside(const int* i) const {
    return i[0] >= lo[0] && i[0] < lo[0] + nx && i[1] >= lo[1] && i[1] < lo[1] + ny && i[2] >= lo[2] &&
           i[2] < lo[2] + nz;
  }
  // material 255 is vacuum: index -1 (SimDPMLike.cc:88-93)
  int MaterialIndex(const int* i) const {
    if (!Inside(i)) return -1;
    const uint8_t m = mat[Flat(i)];
    return m == 255 ? -1 : int(m);
  }
  double Density(int imat) const { return imat > -1 ? T->density[imat] : 1.0E-40; }
  // Geom::GetVoxelMaterialDensity(iVoxel) (Geom.hh:89-92), with per-voxel
  // densities when given
  double DensityAt(const int* i, int imat) const {
    if (rho && imat > -1) return double(rho[Flat(i)]);
    return Density(imat);
  }
  double Wscale() const { return wscale; }
  void Score(double e, const int* i) {
    if (!Inside(i)) return;
    dose[Flat(i)] += e;
    if (btally) btally[size_t(beamlet) * nx * ny * nz + Flat(i)] += e;
    if (depth) {   // Geom::Score (Geom.cc:120-130): by depth bin, in deposit order
      const int iz = i[2] - lo[2];
      if (iz >= dsize) dsize = iz + 10;
      depth[iz] += e;
      dsteps[iz] += 1.0;
    }
  }
};

// ---------------------------------------------------------------------------
// Transport (SimDPMLike.cc)
// ---------------------------------------------------------------------------
struct Track {
  double pos[3], dir[3];
  int box[3];
  int type, mat;
  double ekin;
};

struct Stats {
  double escaped = 0.0;     // kinetic (+rest for e+) energy that left the geometry
  double deposited = 0.0;
  long long steps = 0;      // electron condensed-history sub-steps
  int maxDepth = 0;
};

template <class G, class R>
struct Sim {
  const Tables& T;
  G& geom;
  R& rng;
  Stats st;
  std::vector<Track> stack;
  Sim(const Tables& t, G& g, R& r) : T(t), geom(g), rng(r) {}

  Track& Push(const Track& parent, int type, double e) {
    stack.push_back(parent);
    Track& t = stack.back();
    t.type = type;
    t.ekin = e;
    if (int(stack.size()) > st.maxDepth) st.maxDepth = int(stack.size());
    return t;
  }
  void Score(double e, const int* box) { geom.Score(e, box); st.deposited += e; }

  // SimDPMLike.cc:638-652
  static void Rotate(double& u, double& v, double& w, double u1, double u2, double u3) {
    double up = u1 * u1 + u2 * u2;
    if (up > 0.) {
      up = std::sqrt(up);
      const double px = u, py = v, pz = w;
      u = (u1 * u3 * px - u2 * py) / up + u1 * pz;
      v = (u2 * u3 * px + u1 * py) / up + u2 * pz;
      w = -up * px + u3 * pz;
    } else if (u3 < 0.) {
      u = -u;
      w = -w;
    }
  }
  // SimDPMLike.cc:753-791
  void Annihilate(const Track& t) {
    const double cost = 1.0 - 2.0 * rng.U();
    const double sint = std::sqrt((1.0 - cost) * (1.0 + cost));
    const double phi = 2.0 * kPI * rng.U();
    const double rx = sint * std::cos(phi), ry = sint * std::sin(phi), rz = cost;
    Track& a = Push(t, 0, kEMC2);
    a.dir[0] = rx; a.dir[1] = ry; a.dir[2] = rz;
    Track& b = Push(t, 0, kEMC2);
    b.dir[0] = -rx; b.dir[1] = -ry; b.dir[2] = -rz;
  }
  // SimDPMLike.cc:661-695
  void Brem(Track& t) {
    const double kHalfSqrt2EMC2 = kEMC2 * 0.7071067812;
    const double r3 = rng.U(), r2 = rng.U(), r1 = rng.U();
    const double eg = SampleSB(T, t.ekin, t.mat, r1, r2, r3);
    Track& a = Push(t, 0, eg);
    const double dum0 = kHalfSqrt2EMC2 / (t.ekin + kEMC2);
    const double cost = std::max(-1.0, std::min(1.0, 1.0 - dum0 * dum0));
    const double sint = std::sqrt((1.0 + cost) * (1.0 - cost));
    const double phi = 2.0 * kPI * rng.U();
    a.dir[0] = sint * std::cos(phi); a.dir[1] = sint * std::sin(phi); a.dir[2] = cost;
    Rotate(a.dir[0], a.dir[1], a.dir[2], t.dir[0], t.dir[1], t.dir[2]);
    t.ekin = t.ekin - eg;
  }
  // SimDPMLike.cc:699-728
  void Moller(Track& t) {
    const double k2EMC2 = 2.0 * kEMC2;
    const double r3 = rng.U(), r2 = rng.U(), r1 = rng.U();
    const double se = SampleMoller(T, t.ekin, r1, r2, r3);
    const double cost = std::sqrt(se * (t.ekin + k2EMC2) / (t.ekin * (se + k2EMC2)));
    const double sc = std::min(1.0, cost);
    Track& a = Push(t, -1, se);
    const double sint = std::sqrt((1.0 + sc) * (1.0 - sc));
    const double phi = 2.0 * kPI * rng.U();
    a.dir[0] = sint * std::cos(phi); a.dir[1] = sint * std::sin(phi); a.dir[2] = sc;
    Rotate(a.dir[0], a.dir[1], a.dir[2], t.dir[0], t.dir[1], t.dir[2]);
    t.ekin -= se;
  }
  // SimDPMLike.cc:731-750
  void MSC(Track& t, double ekin0) {
    const double r2 = rng.U(), r1 = rng.U();
    const double d = SampleGS(T, ekin0, r1, r2);
    const double cost = std::max(-1.0, std::min(1.0, d));
    const double sint = std::sqrt((1.0 - cost) * (1.0 + cost));
    const double phi = 2.0 * kPI * rng.U();
    double u1 = sint * std::cos(phi), u2 = sint * std::sin(phi), u3 = cost;
    Rotate(u1, u2, u3, t.dir[0], t.dir[1], t.dir[2]);
    t.dir[0] = u1; t.dir[1] = u2; t.dir[2] = u3;
  }

  // SimDPMLike.cc:254-460; returns 1 brem, 2 Moller, 3 msc, 4 stopped/left
  int KeepTrackingElectron(Track& t, double& nTr1, double& nMol, double invMol, double& nBrem) {
    int what = 0;
    double sGeom = geom.DistanceToBoundary(t.pos, t.dir, t.box);
    if (sGeom < 0.0) { Escape(t); t.ekin = 0.0; return 4; }
    while (what == 0) {
      double step = sGeom;
      what = 0;
      int im = geom.MaterialIndex(t.box);
      if (im < 0) { Escape(t); t.ekin = 0.0; return 4; }
      t.mat = im;
      ++st.steps;
      const double scal = T.mollerScale[im];
      const double rho = geom.DensityAt(t.box, im);
      double dedx = T.dedx[im].Get(t.ekin) * rho;
      double emid = std::max(t.ekin - 0.5 * step * dedx, T.ecut);
      double dTr1 = T.itr1[im].Get(emid) * rho;
      const double dMol = invMol * scal * rho;
      const double dBrem = T.brem[im].Get(emid) * rho;
      const double sBrem = nBrem / dBrem;
      if (sBrem < step) { step = sBrem; what = 1; }
      const double sMol = nMol / dMol;
      if (sMol < step) { step = sMol; what = 2; }
      double sEl = nTr1 / dTr1;
      if (sEl < step) {
        sEl = nTr1 / (T.itr1[im].Get(t.ekin) * rho);
        emid = std::max(t.ekin - 0.5 * sEl * dedx, T.ecut);
        dTr1 = T.itr1[im].Get(emid) * rho;
        sEl = std::min(step, nTr1 / dTr1);
        step = sEl;
        what = 3;
      }
      nBrem = (what == 1) ? 0 : nBrem - step * dBrem;
      nMol = (what == 2) ? 0 : nMol - step * dMol;
      nTr1 = (what == 3) ? 0 : nTr1 - step * dTr1;
      emid = std::max(t.ekin - 0.5 * step * dedx, T.ecut);
      dedx = T.dedx[im].Get(emid) * rho;
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
          if (im < 0) {   // the reference returns here without scoring the deposit
            st.escaped += edep + 2.0 * kEMC2;
            return 4;
          }
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

  void Escape(const Track& t) { st.escaped += t.ekin + (t.type == +1 ? 2.0 * kEMC2 : 0.0); }

  // SimDPMLike.cc:463-635
  void KeepTrackingPhoton(Track& t) {
    const double kInvEMC2 = 1.0 / kEMC2;
    while (t.ekin > 0.0) {
      const double lmax = 1.0 / (T.imfpMax.Get(t.ekin) * geom.Wscale());
      const double step = -lmax * std::log(rng.U());
      t.pos[0] += t.dir[0] * step; t.pos[1] += t.dir[1] * step; t.pos[2] += t.dir[2] * step;
      if (geom.DistanceToBoundary(t.pos, t.dir, t.box) < 0) { Escape(t); t.ekin = 0.0; return; }
      const int im = geom.MaterialIndex(t.box);
      if (im < 0) { Escape(t); t.ekin = 0.0; return; }
      t.mat = im;
      const double rho = geom.DensityAt(t.box, im);
      const double tot = T.imfpTot[im].Get(t.ekin) * rho;
      const double r1 = rng.U();
      double prob = 1.0 - tot * lmax;
      if (r1 < prob) continue;
      prob += T.imfpCompton[im].Get(t.ekin) * rho * lmax;
      if (r1 < prob) {
        const double a3 = rng.U(), a2 = rng.U(), a1 = rng.U();
        const double eps = SampleKN(T, t.ekin, a1, a2, a3);
        const double kappa = t.ekin * kInvEMC2;
        const double phCost = 1.0 - (1.0 - eps) / (eps * kappa);
        const double phE = eps * t.ekin;
        const double phPhi = 2.0 * kPI * rng.U();
        const double elE = t.ekin - phE;
        if (elE < T.ecut) {
          Score(elE, t.box);
        } else {
          const double e0 = t.ekin * kInvEMC2;
          const double elCost = (1.0 + e0) * std::sqrt((1.0 - eps) / (e0 * (2.0 + e0 * (1.0 - eps))));
          Track& a = Push(t, -1, elE);
          const double sint = std::sqrt((1.0 + elCost) * (1.0 - elCost));
          const double phi = phPhi + kPI;
          a.dir[0] = sint * std::cos(phi); a.dir[1] = sint * std::sin(phi); a.dir[2] = elCost;
          Rotate(a.dir[0], a.dir[1], a.dir[2], t.dir[0], t.dir[1], t.dir[2]);
        }
        t.ekin = phE;
        if (t.ekin < T.gcut) {
          Score(t.ekin, t.box);
          t.ekin = 0.0;
          return;
        }
        const double phSint = std::sqrt((1.0 - phCost) * (1.0 + phCost));
        double u1 = phSint * std::cos(phPhi), u2 = phSint * std::sin(phPhi), u3 = phCost;
        Rotate(u1, u2, u3, t.dir[0], t.dir[1], t.dir[2]);
        t.dir[0] = u1; t.dir[1] = u2; t.dir[2] = u3;
        continue;
      }
      prob += T.imfpPair[im].Get(t.ekin) * rho * lmax;
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

  // SimDPMLike.cc:81-246: one history, starting from the given primary track
  void History(const Track& primary) {
    stack.clear();
    stack.push_back(primary);
    if (st.maxDepth < 1) st.maxDepth = 1;
    while (!stack.empty()) {
      Track t = stack.back();
      stack.pop_back();
      geom.DistanceToBoundary(t.pos, t.dir, t.box);
      int im = geom.MaterialIndex(t.box);
      if (im < 0) { Escape(t); continue; }
      t.mat = im;
      if (t.type == 0) { KeepTrackingPhoton(t); continue; }
      bool hinge = true;
      double ekin0 = t.ekin;
      double nTr1 = T.k1.Get(t.ekin);
      double nTr10 = rng.U() * nTr1;
      nTr1 -= nTr10;
      double nMol = -std::log(rng.U());
      double invMol = T.moller.Get(t.ekin);
      double nBrem = -std::log(rng.U());
      while (t.ekin > 0.0) {
        const int what = KeepTrackingElectron(t, nTr1, nMol, invMol, nBrem);
        if (t.mat < 0) continue;
        switch (what) {
          case 1:
            if (t.ekin > T.gcut) Brem(t);
            if (t.ekin < T.ecut) {
              Score(t.ekin, t.box);
              t.ekin = 0.0;
              if (t.type == +1) Annihilate(t);
              break;
            }
            nBrem = -std::log(rng.U());
            break;
          case 2:
            if (t.ekin > 2. * T.ecut) Moller(t);
            nMol = -std::log(rng.U());
            invMol = T.moller.Get(t.ekin);
            break;
          case 3:
            if (hinge) {
              MSC(t, ekin0);
              nTr1 = nTr10;
              hinge = false;
            } else {
              ekin0 = t.ekin;
              nTr1 = T.k1.Get(ekin0);
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

// ---------------------------------------------------------------------------
// Sources for the voxel-phantom runs
// ---------------------------------------------------------------------------
struct Source {
  int particle;        // -1 e-, 0 photon
  int spectrum;        // 0 mono e0, 1 uniform [e0,e1], 2 linear falling p(E) ~ (e1-E) on [e0,e1]
  double e0, e1;
  int shape;           // 0 pencil at (cx,cy), 1 rectangle fx*fy centred at (cx,cy), 2 beamlet grid
  double cx, cy, fx, fy;
  int nbx, nby;        // beamlet grid (shape 2): nbx*nby beamlets of fx*fy, pitch fx, fy
};

// samples the primary of history h into t; returns the beamlet index (or 0)
template <class R>
int SamplePrimary(const Source& s, double zEntry, R& rng, long long h, Track& t) {
  double x = s.cx, y = s.cy;
  int beamlet = 0;
  if (s.shape == 1) {
    x = s.cx + (rng.U() - 0.5) * s.fx;
    y = s.cy + (rng.U() - 0.5) * s.fy;
  } else if (s.shape == 2) {
    const int nb = s.nbx * s.nby;
    beamlet = int(h % nb);
    const int bx = beamlet % s.nbx, by = beamlet / s.nbx;
    x = s.cx + (bx - 0.5 * s.nbx) * s.fx + rng.U() * s.fx;
    y = s.cy + (by - 0.5 * s.nby) * s.fy + rng.U() * s.fy;
  }
  double e = s.e0;
  if (s.spectrum == 1) e = s.e0 + rng.U() * (s.e1 - s.e0);
  else if (s.spectrum == 2) e = s.e1 - (s.e1 - s.e0) * std::sqrt(1.0 - rng.U());
  t.pos[0] = x; t.pos[1] = y; t.pos[2] = zEntry;
  t.dir[0] = 0.0; t.dir[1] = 0.0; t.dir[2] = 1.0;
  t.box[0] = t.box[1] = t.box[2] = 0;
  t.type = s.particle;
  t.mat = -1;
  t.ekin = e;
  return beamlet;
}

}  // namespace oracle

// ===========================================================================
// C interface (used through ctypes by the tests and the benchmark)
// ===========================================================================
using namespace oracle;

extern "C" {

void* oracle_load(const char* dir) { return Load(dir); }
void oracle_free(void* h) { delete static_cast<Tables*>(h); }
int oracle_num_materials(void* h) { return static_cast<Tables*>(h)->nmat; }
double oracle_density(void* h, int im) { return static_cast<Tables*>(h)->density[im]; }
double oracle_cut(void* h, int which) { auto* T = static_cast<Tables*>(h); return which == 0 ? T->ecut : T->gcut; }

// Philox-4x32-10 blocks: out[4i..] = philox(ctr[4i..], key[2i..])
void oracle_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out, int n) {
  for (int i = 0; i < n; ++i) {
    uint32_t c[4] = {ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3]};
    Philox(c, key[2 * i], key[2 * i + 1]);
    for (int j = 0; j < 4; ++j) out[4 * i + j] = c[j];
  }
}

// quantity codes: 0 dedx, 1 itr1, 2 brem, 3 moller, 4 k1, 5 imfpMax, 6 tot, 7 compton, 8 pair
void oracle_eval_table(void* h, int q, int imat, const double* e, double* out, int n) {
  auto* T = static_cast<Tables*>(h);
  for (int i = 0; i < n; ++i) {
    double v = 0;
    switch (q) {
      case 0: v = T->dedx[imat].Get(e[i]); break;
      case 1: v = T->itr1[imat].Get(e[i]); break;
      case 2: v = T->brem[imat].Get(e[i]); break;
      case 3: v = T->moller.Get(e[i]); break;
      case 4: v = T->k1.Get(e[i]); break;
      case 5: v = T->imfpMax.Get(e[i]); break;
      case 6: v = T->imfpTot[imat].Get(e[i]); break;
      case 7: v = T->imfpCompton[imat].Get(e[i]); break;
      case 8: v = T->imfpPair[imat].Get(e[i]); break;
      default: break;
    }
    out[i] = v;
  }
}

// sampler codes: 0 KN eps, 1 Moller T', 2 SB k (imat), 3 GS mu; r has 3 uniforms per sample
void oracle_eval_sampler(void* h, int s, int imat, const double* e, const double* r, double* out, int n) {
  auto* T = static_cast<Tables*>(h);
  for (int i = 0; i < n; ++i) {
    const double* u = r + 3 * i;
    double v = 0;
    switch (s) {
      case 0: v = SampleKN(*T, e[i], u[0], u[1], u[2]); break;
      case 1: v = SampleMoller(*T, e[i], u[0], u[1], u[2]); break;
      case 2: v = SampleSB(*T, e[i], imat, u[0], u[1], u[2]); break;
      case 3: v = SampleGS(*T, e[i], u[0], u[1]); break;
      default: break;
    }
    out[i] = v;
  }
}

// Reference CLI workload: pencil beam along +z from (0,0,-lbox/2) through the
// pre-defined slab geometry, mt19937 stream. edep/steps are resized by the
// reference rule; the first `cap` bins are returned and the used length too.
int oracle_simulate_slab(void* h, int nprimary, double eprimary, int iselectron, double lbox, int geomIndex,
                         uint32_t seed, double* edep, double* steps, int cap, double* stats) {
  auto* T = static_cast<Tables*>(h);
  SlabGeom g(lbox, T, geomIndex);
  MtRng rng(seed);
  Sim<SlabGeom, MtRng> sim(*T, g, rng);
  for (int ip = 0; ip < nprimary; ++ip) {
    Track p{};
    p.ekin = eprimary;
    p.type = iselectron ? -1 : 0;
    p.dir[2] = 1.0;
    p.pos[2] = -0.5 * lbox;
    p.mat = -1;
    sim.History(p);
  }
  const int n = int(g.edep.size());
  for (int i = 0; i < std::min(n, cap); ++i) { edep[i] = g.edep[i]; steps[i] = g.steps[i]; }
  if (stats) { stats[0] = sim.st.deposited; stats[1] = sim.st.escaped; stats[2] = double(sim.st.steps); stats[3] = sim.st.maxDepth; }
  return n;
}

// Same slab workload with the per-history Philox stream (history ids
// first..first+n-1) the FP64 GPU kernel uses. hist_edep (optional, length n)
// receives each history's total deposited energy.
int oracle_simulate_slab_philox(void* h, long long first, int nprimary, double eprimary, int iselectron, double lbox,
                                int geomIndex, uint64_t seed, double* edep, double* steps, int cap,
                                double* hist_edep, double* stats) {
  auto* T = static_cast<Tables*>(h);
  SlabGeom g(lbox, T, geomIndex);
  PhiloxRng rng(seed);
  Sim<SlabGeom, PhiloxRng> sim(*T, g, rng);
  for (int ip = 0; ip < nprimary; ++ip) {
    rng.BeginHistory(uint64_t(first + ip));
    Track p{};
    p.ekin = eprimary;
    p.type = iselectron ? -1 : 0;
    p.dir[2] = 1.0;
    p.pos[2] = -0.5 * lbox;
    p.mat = -1;
    const double before = sim.st.deposited;
    sim.History(p);
    if (hist_edep) hist_edep[ip] = sim.st.deposited - before;
  }
  const int n = int(g.edep.size());
  for (int i = 0; i < std::min(n, cap); ++i) { edep[i] = g.edep[i]; steps[i] = g.steps[i]; }
  if (stats) { stats[0] = sim.st.deposited; stats[1] = sim.st.escaped; stats[2] = double(sim.st.steps); stats[3] = sim.st.maxDepth; }
  return n;
}

// The reference CLI workload (pencil beam from (0,0,-lbox/2) along +z,
// mt19937 stream, SimDPMLike.cc:57-247) on a 3-D voxel phantom laid out as the
// reference's own lattice: voxels of lbox centred at integer multiples of lbox
// (lattice index 0 at the origin), x and y indices -k..k and z indices 0..nz-1
// covering the world |x|,|y| <= 100 mm, -lbox <= z <= 100 mm (Geom.cc:20-28,
// Geom.hh:107-109), each voxel holding the slab material of its depth
// (Geom.cc:133-164). The depth tally (Geom::Score order) is returned in
// edep/steps (cap bins), its length by Geom::Score's rule as the return value.
int oracle_simulate_voxel_slabref(void* h, int nprimary, double eprimary, int iselectron, double lbox,
                                  int geomIndex, uint32_t seed, double* edep, double* steps, int cap, double* stats) {
  auto* T = static_cast<Tables*>(h);
  const double invL = 1.0 / lbox, halfL = 0.5 * lbox;
  const int k = int(std::ceil((100.0 - halfL) * invL - 1.0e-9));       // lateral indices -k..k
  const int nz = int(std::ceil((100.0 - halfL) * invL - 1.0e-9)) + 1;  // depth indices 0..nz-1
  const int nx = 2 * k + 1;
  SlabGeom slab(lbox, T, geomIndex);
  std::vector<uint8_t> mat(size_t(nx) * nx * nz);
  for (int iz = 0; iz < nz; ++iz) {
    const int ib[3] = {0, 0, iz};
    const int m = slab.MaterialIndex(ib);
    std::fill(mat.begin() + size_t(iz) * nx * nx, mat.begin() + size_t(iz + 1) * nx * nx,
              uint8_t(m < 0 ? 255 : m));
  }
  std::vector<double> dose(mat.size(), 0.0), depth(nz, 0.0), dsteps(nz, 0.0);
  VoxelGeom g{nx, nx, nz, -(k + 0.5) * lbox, -(k + 0.5) * lbox, -halfL, lbox, lbox, lbox, invL, invL, invL,
              mat.data(), T, dose.data(), nullptr};
  for (int a = 0; a < 3; ++a) g.c[a] = 0.0;
  g.lo[0] = g.lo[1] = -k;
  g.lo[2] = 0;
  g.wlo[0] = g.wlo[1] = -100.0;
  g.whi[0] = g.whi[1] = 100.0;
  g.wlo[2] = -lbox;
  g.whi[2] = 100.0;
  g.depth = depth.data();
  g.dsteps = dsteps.data();
  MtRng rng(seed);
  Sim<VoxelGeom, MtRng> sim(*T, g, rng);
  for (int ip = 0; ip < nprimary; ++ip) {
    Track p{};
    p.ekin = eprimary;
    p.type = iselectron ? -1 : 0;
    p.dir[2] = 1.0;
    p.pos[2] = -halfL;
    p.mat = -1;
    sim.History(p);
  }
  const int n = g.dsize;
  for (int i = 0; i < std::min(n, cap); ++i) {
    edep[i] = i < nz ? depth[i] : 0.0;
    steps[i] = i < nz ? dsteps[i] : 0.0;
  }
  if (stats) { stats[0] = sim.st.deposited; stats[1] = sim.st.escaped; stats[2] = double(sim.st.steps); stats[3] = sim.st.maxDepth; }
  return n;
}

// Voxel-phantom run with a beam source, Philox stream per history. The dose
// array (nx*ny*nz, zero-filled by the caller) receives the deposited energy
// [MeV] and hist_edep (optional) each history's deposited energy; btally
// (optional, nbx*nby*nx*ny*nz) the dose per beamlet of a beamlet-grid source,
// each history's deposits under its beamlet.
int oracle_simulate_voxel(void* h, int nx, int ny, int nz, double vx, double vy, double vz, const uint8_t* mat,
                          int particle, int spectrum, double e0, double e1, int shape, double cx, double cy,
                          double fx, double fy, int nbx, int nby, long long first, long long nhist, uint64_t seed,
                          double* dose, double* hist_edep, double* stats, const float* rho, double* btally) {
  auto* T = static_cast<Tables*>(h);
  VoxelGeom g{nx, ny, nz, -0.5 * nx * vx, -0.5 * ny * vy, 0.0, vx, vy, vz, 1.0 / vx, 1.0 / vy, 1.0 / vz, mat, T, dose, nullptr};
  g.SetDefaultLattice();
  g.btally = btally;
  if (rho) {
    // the same majorant scale as the library: max density / nominal density
    g.rho = rho;
    const size_t n = size_t(nx) * ny * nz;
    for (size_t i = 0; i < n; ++i)
      if (mat[i] != 255) g.wscale = std::max(g.wscale, double(rho[i]) / T->density[mat[i]]);
  }
  PhiloxRng rng(seed);
  Sim<VoxelGeom, PhiloxRng> sim(*T, g, rng);
  Source s{particle, spectrum, e0, e1, shape, cx, cy, fx, fy, nbx, nby};
  for (long long i = 0; i < nhist; ++i) {
    const long long hid = first + i;
    rng.BeginHistory(uint64_t(hid));
    Track p{};
    g.beamlet = SamplePrimary(s, 0.0, rng, hid, p);
    const double before = sim.st.deposited;
    sim.History(p);
    if (hist_edep) hist_edep[i] = sim.st.deposited - before;
  }
  if (stats) { stats[0] = sim.st.deposited; stats[1] = sim.st.escaped; stats[2] = double(sim.st.steps); stats[3] = sim.st.maxDepth; }
  return 0;
}

}  // extern "C"
