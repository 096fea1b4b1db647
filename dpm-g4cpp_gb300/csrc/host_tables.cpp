// Reader of the reference's simulation data files (the 14 files written by
// dpm_GenerateData, layouts in ElectronData.hh:439-663, PhotonData.hh:170-257,
// KNTableBuilder.cc:149-178, MollerTableBuilder.cc:120-149,
// SBTableBuilder.cc:296-344). Every file is a sequence of '#' comment lines and
// whitespace-separated values; the values are consumed in the order the
// reference loaders read them (Simulation/src/Sim*.cc LoadData).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "dpmx_internal.h"

namespace dpmx {
namespace {

// all value tokens of a file, comment lines dropped
struct Tokens {
  std::vector<std::string> v;
  size_t i = 0;
  bool bad = false;
  bool Read(const std::string& path) {
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    while (std::getline(f, line)) {
      size_t k = line.find_first_not_of(" \t\r");
      if (k == std::string::npos || line[k] == '#') continue;
      std::istringstream ss(line);
      std::string t;
      while (ss >> t) v.push_back(t);
    }
    return true;
  }
  double D() {
    if (i >= v.size()) { bad = true; return 0.0; }
    char* end = nullptr;
    const double x = std::strtod(v[i].c_str(), &end);
    if (end == v[i].c_str()) bad = true;
    ++i;
    return x;
  }
  int I() { return int(std::lround(D())); }
  std::string S() {
    if (i >= v.size()) { bad = true; return ""; }
    return v[i++];
  }
};

int Open(const std::string& dir, const char* name, Tokens& t, std::string& err) {
  const std::string p = dir + "/" + name;
  if (!t.Read(p)) {
    err = "data file " + p + " not found";
    return DPMX_ERR_FILE;
  }
  return DPMX_OK;
}

int Bad(const char* name, std::string& err) {
  err = std::string("unexpected layout of data file ") + name;
  return DPMX_ERR_PARSE;
}

// N nmat, then nmat blocks of N rows with `cols` columns; value column `vc`
int PerMaterial(const std::string& dir, const char* name, int cols, int vc, std::vector<Curve>& out,
                std::string& err) {
  Tokens t;
  int rc = Open(dir, name, t, err);
  if (rc) return rc;
  const int n = t.I(), nm = t.I();
  if (t.bad || n < 2 || nm < 1 || nm > kMaxMat) return Bad(name, err);
  out.assign(nm, Curve());
  for (int m = 0; m < nm; ++m) {
    out[m].x.resize(n);
    out[m].y.resize(n);
    for (int i = 0; i < n; ++i) {
      double row[3] = {0, 0, 0};
      for (int c = 0; c < cols; ++c) row[c] = t.D();
      out[m].x[i] = row[0];
      out[m].y[i] = row[vc];
    }
  }
  return t.bad ? Bad(name, err) : DPMX_OK;
}

// N, then the first block of N (E, value) rows (reference material only)
int FirstBlock(const std::string& dir, const char* name, Curve& out, std::string& err) {
  Tokens t;
  int rc = Open(dir, name, t, err);
  if (rc) return rc;
  const int n = t.I();
  if (t.bad || n < 2) return Bad(name, err);
  out.x.resize(n);
  out.y.resize(n);
  for (int i = 0; i < n; ++i) { out.x[i] = t.D(); out.y[i] = t.D(); }
  return t.bad ? Bad(name, err) : DPMX_OK;
}

void ReadAlias(Tokens& t, int ns, AliasTab& a) {
  a.x.resize(ns); a.y.resize(ns); a.w.resize(ns); a.idx.resize(ns);
  for (int s = 0; s < ns; ++s) { a.x[s] = t.D(); a.y[s] = t.D(); a.w[s] = t.D(); a.idx[s] = t.I(); }
}

// alias indices of the ns-1 bins must name a bin (the sampler reads idx+1)
bool AliasOk(const AliasTab& a) {
  const int ns = int(a.x.size());
  for (int s = 0; s + 1 < ns; ++s)
    if (a.idx[s] < 0 || a.idx[s] > ns - 2) return false;
  return true;
}

int EnergyAlias(const std::string& dir, const char* name, std::vector<AliasTab>& out, std::string& err) {
  Tokens t;
  int rc = Open(dir, name, t, err);
  if (rc) return rc;
  const int ne = t.I(), ns = t.I();
  if (t.bad || ne < 2 || ns < 2) return Bad(name, err);
  out.assign(ne, AliasTab());
  for (int e = 0; e < ne; ++e) {
    out[e].e = t.D();
    ReadAlias(t, ns, out[e]);
  }
  for (auto& a : out)
    if (!AliasOk(a)) return Bad(name, err);
  return t.bad ? Bad(name, err) : DPMX_OK;
}

}  // namespace

void SplineCoefficients(const std::vector<double>& x, const std::vector<double>& y, std::vector<double>& b,
                        std::vector<double>& c, std::vector<double>& d) {
  // natural cubic spline as set up by SimDataSpline::SetUp (SimDataSpline.cc:33-67):
  // forward elimination on the interval slopes, back substitution for the
  // second-derivative terms, then the per-interval cubic coefficients
  const int n = int(x.size());
  b.assign(n, 0.0); c.assign(n, 0.0); d.assign(n, 0.0);
  const int last = n - 1;
  double prevSlope = 0.0;
  for (int m = 0; m < last; ++m) {
    d[m] = x[m + 1] - x[m];
    const double slope = (y[m + 1] - y[m]) / d[m];
    c[m] = slope - prevSlope;
    prevSlope = slope;
  }
  double ratio = 0.0, h = 0.0;
  c[0] = 0.0;
  c[last] = 0.0;
  for (int m = 1; m < last; ++m) {
    c[m] = c[m] + ratio * c[m - 1];
    b[m] = 2.0 * (x[m - 1] - x[m + 1]) - ratio * h;
    h = d[m];
    ratio = h / b[m];
  }
  for (int m = last - 1; m >= 1; --m) c[m] = (d[m] * c[m + 1] - c[m]) / b[m];
  for (int m = 0; m < last; ++m) {
    const double hm = d[m];
    const double dc = c[m + 1] - c[m];
    d[m] = dc / hm;
    c[m] = 3.0 * c[m];
    b[m] = (y[m + 1] - y[m]) / hm - (c[m] + dc) * hm;
  }
}

int LoadHostTables(const std::string& dir, HostTables& h, std::string& err) {
  int rc;
  {  // mat.dat (SimMaterialData.cc:6-53)
    Tokens t;
    if ((rc = Open(dir, "mat.dat", t, err))) return rc;
    h.ecut = t.D(); h.gcut = t.D();
    h.slow = t.D(); h.shigh = t.D(); h.ecross = t.D();
    h.nmat = t.I();
    if (t.bad || h.nmat < 1 || h.nmat > kMaxMat) return Bad("mat.dat", err);
    for (int m = 0; m < h.nmat; ++m) {
      t.I();
      h.names.push_back(t.S());
      h.density.push_back(t.D());
      for (int k = 0; k < 6; ++k) t.D();
      h.mollerScale.push_back(t.D());
      t.D();
    }
    if (t.bad) return Bad("mat.dat", err);
  }
  if ((rc = PerMaterial(dir, "el_itr1mfp.dat", 3, 2, h.itr1, err))) return rc;       // SimITr1MFPElastic.cc:13-55 (3rd column)
  if ((rc = FirstBlock(dir, "el_scatStrength.dat", h.k1, err))) return rc;          // SimMaxScatStrength.cc:6-42
  if ((rc = FirstBlock(dir, "imfp_moller.dat", h.moller, err))) return rc;          // SimIMFPMoller.cc:6-43
  if ((rc = PerMaterial(dir, "imfp_brem.dat", 2, 1, h.brem, err))) return rc;       // SimIMFPBrem.cc:18-60
  if ((rc = PerMaterial(dir, "eloss_rdedx.dat", 2, 1, h.dedx, err))) return rc;     // SimStoppingPower.cc:18-60
  if ((rc = EnergyAlias(dir, "ioni_MollerDtrData.dat", h.mol, err))) return rc;     // SimMollerTables.cc:20-66
  if ((rc = EnergyAlias(dir, "compton_KNDtrData.dat", h.kn, err))) return rc;       // SimKNTables.cc:20-66
  {  // brem_SBDtrData.dat (SimSBTables.cc:21-90)
    Tokens t;
    if ((rc = Open(dir, "brem_SBDtrData.dat", t, err))) return rc;
    const int ne = t.I(), ns = t.I(), nm = t.I();
    if (t.bad || ne < 2 || ns < 2 || nm < h.nmat) return Bad("brem_SBDtrData.dat", err);
    h.sbE.resize(ne);
    for (int e = 0; e < ne; ++e) h.sbE[e] = t.D();
    h.sb.assign(nm, std::vector<AliasTab>(ne));
    for (int m = 0; m < nm; ++m)
      for (int e = 0; e < ne; ++e) {
        h.sb[m][e].e = h.sbE[e];
        ReadAlias(t, ns, h.sb[m][e]);
        if (!AliasOk(h.sb[m][e])) return Bad("brem_SBDtrData.dat", err);
      }
    if (t.bad) return Bad("brem_SBDtrData.dat", err);
  }
  {  // el_GSDtrData.dat (SimGSTables.cc:19-81): material 0's tables only
    Tokens t;
    if ((rc = Open(dir, "el_GSDtrData.dat", t, err))) return rc;
    h.gsNumE = t.I();
    t.D(); t.D();
    h.gsNumS = t.I();
    if (t.bad || h.gsNumE < 2 || h.gsNumS < 2) return Bad("el_GSDtrData.dat", err);
    const int ne = h.gsNumE, ns = h.gsNumS;
    h.gsE.resize(ne); h.gsA.resize(ne);
    h.gsU.resize(size_t(ne) * ns); h.gsPA.resize(size_t(ne) * ns); h.gsPB.resize(size_t(ne) * ns);
    for (int e = 0; e < ne; ++e) {
      t.I();
      h.gsE[e] = t.D();
      h.gsA[e] = t.D();
      for (int s = 0; s < ns; ++s) {
        h.gsU[size_t(e) * ns + s] = t.D();
        h.gsPA[size_t(e) * ns + s] = t.D();
        h.gsPB[size_t(e) * ns + s] = t.D();
      }
    }
    if (t.bad) return Bad("el_GSDtrData.dat", err);
  }
  if ((rc = FirstBlock(dir, "imfp_globalMax.dat", h.imfpMax, err))) return rc;      // SimIMFPMaxPhoton.cc:6-38
  if ((rc = PerMaterial(dir, "imfp_total.dat", 2, 1, h.tot, err))) return rc;       // SimIMFPPhoton.cc:19-62
  if ((rc = PerMaterial(dir, "imfp_compton.dat", 2, 1, h.comp, err))) return rc;
  if ((rc = PerMaterial(dir, "imfp_pairp.dat", 2, 1, h.pair, err))) return rc;
  if (int(h.itr1.size()) < h.nmat || int(h.dedx.size()) < h.nmat || int(h.brem.size()) < h.nmat ||
      int(h.tot.size()) < h.nmat || int(h.comp.size()) < h.nmat || int(h.pair.size()) < h.nmat) {
    err = "data files hold fewer materials than mat.dat";
    return DPMX_ERR_PARSE;
  }
  return DPMX_OK;
}

}  // namespace dpmx
