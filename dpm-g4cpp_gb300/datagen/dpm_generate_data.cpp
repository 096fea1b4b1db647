// dpm_generate_data: a Geant4-free writer of the simulation-phase data files.
//
// The reference `dpm_GenerateData` (dpm_GenerateData.cc:52-128) extracts its
// physics through Geant4, which is not available to this project. This program
// writes the same 18 ASCII files, with the same grids, header line counts and
// column layouts, so that any reader of the reference format (the reference's
// own `Sim*::LoadData` functions, or this project's loaders) can use them:
//
//   mat.dat                 ElectronData.hh:444-480
//   el_iemfp.dat            ElectronData.hh:483-497      (not read by the simulation)
//   el_itr1mfp.dat          ElectronData.hh:500-515
//   el_screeningPar.dat     ElectronData.hh:519-533      (not read by the simulation)
//   el_scatStrength.dat     ElectronData.hh:536-550
//   el_GSDtrData.dat        ElectronData.hh:553-585
//   eloss_rdedx.dat         ElectronData.hh:588-602
//   eloss_rRange.dat        ElectronData.hh:605-618      (not read by the simulation)
//   imfp_brem.dat           ElectronData.hh:621-636
//   imfp_moller.dat         ElectronData.hh:639-654
//   ioni_MollerDtrData.dat  MollerTableBuilder.cc:120-149
//   brem_SBDtrData.dat      SBTableBuilder.cc:296-344
//   imfp_compton.dat, imfp_pairp.dat, imfp_photoe.dat, imfp_total.dat,
//   imfp_globalMax.dat      PhotonData.hh:170-257
//   compton_KNDtrData.dat   KNTableBuilder.cc:149-178
//
// Physics used in place of the Geant4 models (each is a published, analytic or
// tabulated description; none is a port of Geant4 code):
//   * elastic e- scattering: screened Rutherford cross section per element
//     with Moliere's screening parameter, times the Mott (spin) factor of
//     McKinley and Feshbach (Phys. Rev. 74 (1948) 1759) in place of the
//     partial-wave cross sections the reference takes from Geant4; the
//     inelastic Z(Z+1)/Z^2 scattering power correction is applied as in the
//     reference (ElectronData.hh:219-221);
//   * collision stopping power: the restricted Berger-Seltzer (ICRU Report 37)
//     formula for electrons with the density effect of Sternheimer, Berger and
//     Seltzer (At. Data Nucl. Data Tables 30 (1984) 261) for the tabulated
//     materials, Sternheimer-Peierls' general formula for the others;
//   * bremsstrahlung: the Seltzer-Berger scaled DCS tables (NIST, the same data
//     the reference ships in SBTables/data/NIST_BREM) read from --sb-dir; the
//     restricted radiative stopping power, the brem IMFP and the brem sampling
//     tables are all built from them;
//   * Moller: the Moller DCS (restricted IMFP in closed form, sampling tables);
//   * Compton: Klein-Nishina per electron (no binding);
//   * pair production: Bethe-Heitler DCS with Butcher-Messel screening
//     functions, integrated numerically, Z^2 -> Z(Z+1) for triplet production;
//   * photoelectric: Heitler's non-relativistic K-shell Born cross section
//     times 1.25 for the outer shells;
//   * GS multiple scattering: Goudsmit-Saunderson angular distributions for the
//     screened Rutherford DCS, with the Legendre transport coefficients from the
//     small-angle Bessel-function approximation of Kawrakow and Bielajew
//     (NIM B 134 (1998) 325, Eq. 42), in the transformed variable
//     mu(u) = 1 - 2au/(1-u+a) and a rational-interpolation inverse CDF on a
//     64-point cumulative grid (the table layout SimGSTables.cc:84-119 reads).
//
// Usage: dpm_generate_data -d <outdir> -c <config-index> -s <sb-data-dir> [-m name,name,...]
//   config indices 0-5 are the reference's Configuration.hh:69-111 presets;
//   index 6 is this project's water / lung / compact-bone set used for the
//   voxel phantoms.  -m overrides the material list.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

constexpr double kPi      = 3.14159265358979323846;
constexpr double kEMC2    = 0.510998950;        // electron rest energy [MeV]
constexpr double kAlpha   = 1.0 / 137.035999084;
constexpr double kRe      = 2.8179403262e-12;   // classical electron radius [mm]
constexpr double kNA      = 6.02214076e23;
constexpr double kBarnMM2 = 1.0e-22;            // 1 barn in mm^2
constexpr double kMBarnMM2 = 1.0e-25;           // 1 mbarn in mm^2

// ---------------------------------------------------------------------------
// Elements and materials (compositions by mass fraction, densities in g/cm3 and
// mean excitation energies from the NIST/ICRU material tables that Geant4's
// G4_* materials are defined from).
// ---------------------------------------------------------------------------
struct Element { int Z; double A; double I_eV; };

const std::map<int, Element>& Elements() {
  static const std::map<int, Element> e = {
    {1,  {1,  1.008,   19.2}}, {6,  {6,  12.011,  81.0}}, {7,  {7,  14.007,  82.0}},
    {8,  {8,  15.999,  95.0}}, {11, {11, 22.990, 149.0}}, {12, {12, 24.305, 156.0}},
    {15, {15, 30.974, 173.0}}, {16, {16, 32.06,  180.0}}, {17, {17, 35.45,  174.0}},
    {18, {18, 39.948, 188.0}}, {19, {19, 39.098, 190.0}}, {20, {20, 40.078, 191.0}},
    {22, {22, 47.867, 233.0}}, {26, {26, 55.845, 286.0}}, {30, {30, 65.38,  330.0}},
    {74, {74, 183.84, 727.0}},
  };
  return e;
}

struct MaterialDef {
  std::string name;
  double density;                              // g/cm3
  double I_eV;                                 // mean excitation energy of the material
  std::vector<std::pair<int, double>> comp;    // (Z, mass fraction)
};

const std::vector<MaterialDef>& MaterialLibrary() {
  static const std::vector<MaterialDef> lib = {
    {"G4_WATER", 1.0, 78.0, {{1, 0.111894}, {8, 0.888106}}},
    {"G4_AIR", 0.00120479, 85.7, {{6, 0.000124}, {7, 0.755268}, {8, 0.231781}, {18, 0.012827}}},
    {"G4_Ti", 4.54, 233.0, {{22, 1.0}}},
    {"G4_W", 19.3, 727.0, {{74, 1.0}}},
    {"G4_BONE_COMPACT_ICRU", 1.85, 91.9,
      {{1, 0.063984}, {6, 0.278}, {7, 0.027}, {8, 0.410016}, {12, 0.002}, {15, 0.07}, {16, 0.002}, {20, 0.147}}},
    {"G4_BONE_CORTICAL_ICRP", 1.92, 110.0,
      {{1, 0.034}, {6, 0.155}, {7, 0.042}, {8, 0.435}, {11, 0.001}, {12, 0.002}, {15, 0.103}, {16, 0.003}, {20, 0.225}}},
    {"G4_LUNG_ICRP", 1.04, 75.3,
      {{1, 0.105}, {6, 0.083}, {7, 0.023}, {8, 0.779}, {11, 0.002}, {15, 0.001}, {16, 0.002}, {17, 0.003}, {19, 0.002}}},
  };
  return lib;
}

struct Material {
  MaterialDef def;
  std::vector<int>    Z;       // element atomic numbers
  std::vector<double> nAtoms;  // atoms per mm3 of each element
  double nElectrons = 0.0;     // electrons per mm3
  // per-material averages written to mat.dat (ElectronData.hh:116-123)
  double zMean = 0, z2 = 0, zs = 0, wMean = 0, zw = 0, iMeanMeV = 0, scpc = 0;
};

Material BuildMaterial(const MaterialDef& d) {
  Material m;
  m.def = d;
  double tot = 0.0, sZ = 0, sZ2 = 0, sZs = 0, sW = 0, sZW = 0, sLnI = 0;
  for (auto& c : d.comp) {
    const Element& el = Elements().at(c.first);
    // atoms per mm3: rho[g/cm3] * N_A * w/A / 1000 [mm3/cm3]
    const double n = d.density * kNA * c.second / el.A * 1.0e-3;
    m.Z.push_back(el.Z);
    m.nAtoms.push_back(n);
    m.nElectrons += n * el.Z;
    tot  += n;
    sZ   += n * el.Z;
    sZ2  += n * el.Z * el.Z;
    sZs  += n * el.Z * (el.Z + 1.0);
    sW   += n * el.A;
    sZW  += n * el.A * el.Z;
    sLnI += n * std::log(el.I_eV * 1.0e-6);
  }
  m.zMean = sZ / tot; m.z2 = sZ2 / tot; m.zs = sZs / tot; m.wMean = sW / tot;
  m.zw = sZW / tot;   m.iMeanMeV = std::exp(sLnI / tot);
  m.scpc = sZs / sZ2;  // scattering power correction Z(Z+1)/Z^2
  return m;
}

// ---------------------------------------------------------------------------
// Elastic scattering: screened Rutherford DCS with Moliere's screening, times
// the McKinley-Feshbach ratio of the Mott to the Rutherford cross section,
//   dsigma/dmu = pi k^2 R(mu) / (mu + A)^2,   k = Z r_e mc^2/(p beta c),
//   R(mu) = 1 + pi alpha Z beta sqrt(mu) (1 - sqrt(mu)) - beta^2 mu,
//   mu = (1-cos)/2 = sin^2(theta/2).
// With K_p = int_0^1 mu^p / (mu + A)^2 dmu (closed forms below):
//   sigma_el = pi k^2 [K_0 + c (K_1/2 - K_1) - beta^2 K_1]
//   sigma_1  = 2 pi k^2 [K_1 + c (K_3/2 - K_2) - beta^2 K_2],  c = pi alpha Z beta
// (R = 1 gives the screened Rutherford sigma_el = pi k^2/(A(1+A)) and
// sigma_1 = 2 pi k^2 [ln((1+A)/A) - 1/(1+A)].) The factor lowers the first
// transport cross section of water by 4-6 % at 0.2-5 MeV.
// ---------------------------------------------------------------------------
double MoliereA(int Z, double T) {
  const double pc2   = T * (T + 2.0 * kEMC2);            // (pc)^2
  const double beta2 = pc2 / ((T + kEMC2) * (T + kEMC2));
  const double aTF   = 0.88534 * std::pow(double(Z), -1.0 / 3.0);   // in Bohr radii
  // (hbar/(2 p a))^2 = (alpha mc^2 / (2 pc aTF))^2 with a in Bohr radii
  const double f     = kAlpha * kEMC2 / (2.0 * aTF);
  return f * f / pc2 * (1.13 + 3.76 * (kAlpha * Z) * (kAlpha * Z) / beta2);
}

void ElasticXS(int Z, double T, double& sEl, double& sTr1) {
  const double pc2   = T * (T + 2.0 * kEMC2);
  const double beta2 = pc2 / ((T + kEMC2) * (T + kEMC2));
  const double k     = Z * kRe * kEMC2 / std::sqrt(pc2 * beta2);
  const double A     = MoliereA(Z, T);
  const double c     = kPi * kAlpha * Z * std::sqrt(beta2);
  const double sa    = std::sqrt(A), at = std::atan(1.0 / sa), L = std::log1p(1.0 / A);
  const double K0  = 1.0 / (A * (1.0 + A));
  const double Kh  = at / sa - 1.0 / (1.0 + A);               // p = 1/2 (mu = t^2)
  const double K1  = L - 1.0 / (1.0 + A);
  const double K3h = 2.0 - 3.0 * sa * at + A / (1.0 + A);     // p = 3/2
  const double K2  = 1.0 - 2.0 * A * L + A / (1.0 + A);
  sEl  = kPi * k * k * (K0 + c * (Kh - K1) - beta2 * K1);
  sTr1 = 2.0 * kPi * k * k * (K1 + c * (K3h - K2) - beta2 * K2);
}

// macroscopic elastic and first transport cross sections [1/mm] (no scpc)
void MacroElastic(const Material& m, double T, double& mEl, double& mTr1) {
  mEl = mTr1 = 0.0;
  for (size_t i = 0; i < m.Z.size(); ++i) {
    double a, b;
    ElasticXS(m.Z[i], T, a, b);
    mEl  += m.nAtoms[i] * a;
    mTr1 += m.nAtoms[i] * b;
  }
}

// solves G1(x) = 2x[(1+x) ln(1+1/x) - 1] = g for x (Newton on a bracketed start)
double ScreeningFromG1(double g) {
  double lo = 1.0e-16, hi = 1.0e6;
  auto G1 = [](double x) { return 2.0 * x * ((1.0 + x) * std::log1p(1.0 / x) - 1.0); };
  // G1 is increasing in x: bisection in log space, then a few Newton polishes
  for (int it = 0; it < 200; ++it) {
    const double mid = std::sqrt(lo * hi);
    if (G1(mid) < g) lo = mid; else hi = mid;
    if (hi / lo < 1.0 + 1.0e-13) break;
  }
  return std::sqrt(lo * hi);
}

// ---------------------------------------------------------------------------
// Seltzer-Berger scaled brem DCS chi(Z,T,kappa) = beta^2/Z^2 k dsigma/dk [mb]
// ---------------------------------------------------------------------------
struct SBData {
  std::vector<double> T;       // 113 electron kinetic energies [MeV]
  std::vector<double> kappa;   // 32 reduced photon energies
  std::map<int, std::vector<double>> chi;  // Z -> [iT * nk + ik]
  bool Load(const std::string& dir, const std::vector<int>& zs) {
    const std::string base = dir + "/NIST_BREM/nist_brems_";
    FILE* f = std::fopen((base + "grid").c_str(), "r");
    if (!f) { std::fprintf(stderr, "cannot open %sgrid\n", base.c_str()); return false; }
    int a, nT, nk;
    if (std::fscanf(f, "%d %d %d", &a, &nT, &nk) != 3) { std::fclose(f); return false; }
    T.resize(nT); kappa.resize(nk);
    for (int i = 0; i < nT; ++i) if (std::fscanf(f, "%lg", &T[i]) != 1) { std::fclose(f); return false; }
    for (int i = 0; i < nk; ++i) if (std::fscanf(f, "%lg", &kappa[i]) != 1) { std::fclose(f); return false; }
    std::fclose(f);
    for (int Z : zs) {
      if (chi.count(Z)) continue;
      FILE* g = std::fopen((base + std::to_string(Z)).c_str(), "r");
      if (!g) { std::fprintf(stderr, "cannot open SB data for Z=%d\n", Z); return false; }
      std::vector<double> v(size_t(nT) * nk);
      for (auto& x : v) if (std::fscanf(g, "%lg", &x) != 1) { std::fclose(g); return false; }
      std::fclose(g);
      chi[Z] = v;
    }
    return true;
  }
  // chi at kinetic energy T for table kappa index ik, log-log in T
  double ChiAt(int Z, double t, int ik) const {
    const int nT = int(T.size()), nk = int(kappa.size());
    int j = int(std::upper_bound(T.begin(), T.end(), t) - T.begin()) - 1;
    j = std::max(0, std::min(nT - 2, j));
    const std::vector<double>& v = chi.at(Z);
    const double y0 = v[size_t(j) * nk + ik], y1 = v[size_t(j + 1) * nk + ik];
    const double w = std::log(t / T[j]) / std::log(T[j + 1] / T[j]);
    return std::exp(std::log(y0) + w * (std::log(y1) - std::log(y0)));
  }
};

// material-weighted sum_i n_i Z_i^2 chi_i(T, kappa_k) over the SB kappa grid
std::vector<double> MaterialChi(const Material& m, const SBData& sb, double T) {
  std::vector<double> out(sb.kappa.size(), 0.0);
  for (size_t ik = 0; ik < sb.kappa.size(); ++ik) {
    for (size_t i = 0; i < m.Z.size(); ++i) {
      out[ik] += m.nAtoms[i] * double(m.Z[i]) * m.Z[i] * sb.ChiAt(m.Z[i], T, int(ik));
    }
  }
  return out;
}

// piecewise-linear chi(kappa) evaluated at kappa
double InterpChi(const std::vector<double>& kap, const std::vector<double>& c, double k) {
  int j = int(std::upper_bound(kap.begin(), kap.end(), k) - kap.begin()) - 1;
  j = std::max(0, std::min(int(kap.size()) - 2, j));
  const double w = (k - kap[j]) / (kap[j + 1] - kap[j]);
  return c[j] + w * (c[j + 1] - c[j]);
}

// Integrals of the piecewise-linear chi: I0 = int_a^b chi dk, I1 = int_a^b chi/k dk
void IntegrateChi(const std::vector<double>& kap, const std::vector<double>& c,
                  double a, double b, double& I0, double& I1) {
  I0 = I1 = 0.0;
  for (size_t j = 0; j + 1 < kap.size(); ++j) {
    const double lo = std::max(a, kap[j]), hi = std::min(b, kap[j + 1]);
    if (hi <= lo) continue;
    const double s  = (c[j + 1] - c[j]) / (kap[j + 1] - kap[j]);
    const double c0 = c[j] - s * kap[j];              // chi = c0 + s k on this piece
    I0 += c0 * (hi - lo) + 0.5 * s * (hi * hi - lo * lo);
    I1 += c0 * std::log(hi / lo) + s * (hi - lo);
  }
}

// restricted radiative stopping power [MeV/mm] and brem IMFP [1/mm] for k > kc
void BremQuantities(const Material& m, const SBData& sb, double T, double gcut,
                    double& radDEDX, double& imfp) {
  const double beta2 = T * (T + 2.0 * kEMC2) / ((T + kEMC2) * (T + kEMC2));
  const std::vector<double> c = MaterialChi(m, sb, T);
  const double kc = std::min(1.0, gcut / T);
  double I0a, I1a, I0b, I1b;
  IntegrateChi(sb.kappa, c, sb.kappa.front(), kc, I0a, I1a);
  IntegrateChi(sb.kappa, c, kc, 1.0, I0b, I1b);
  radDEDX = T * I0a * kMBarnMM2 / beta2;
  imfp    = I1b * kMBarnMM2 / beta2;
}

// ---------------------------------------------------------------------------
// Collision stopping power (restricted Berger-Seltzer formula, ICRU 37)
// ---------------------------------------------------------------------------
// density-effect parameters of Sternheimer, Berger and Seltzer (At. Data
// Nucl. Data Tables 30 (1984) 261): the table's I [eV], Cbar, x0, x1, a, m,
// delta0. Cbar = 1 + 2 ln(I / plasma energy) moves with the material's I.
struct SternheimerParams { double I, C, x0, x1, a, m, d0; };
const std::map<std::string, SternheimerParams>& SternheimerTable() {
  static const std::map<std::string, SternheimerParams> t = {
    {"G4_WATER", {75.0, 3.5017, 0.2400, 2.8004, 0.09116, 3.4773, 0.0}},
    {"G4_AIR", {85.7, 10.5961, 1.7418, 4.2759, 0.10914, 3.3994, 0.0}},
    {"G4_Ti", {233.0, 4.4450, 0.0957, 3.0386, 0.15643, 3.0302, 0.12}},
    {"G4_W", {727.0, 5.4059, 0.2167, 3.4960, 0.15509, 2.8447, 0.14}},
    {"G4_BONE_COMPACT_ICRU", {91.9, 3.3390, 0.0944, 3.0201, 0.05822, 3.6419, 0.0}},
    {"G4_BONE_CORTICAL_ICRP", {106.4, 3.6488, 0.1161, 3.0919, 0.06198, 3.5919, 0.0}},
    {"G4_LUNG_ICRP", {75.3, 3.4708, 0.2261, 2.8001, 0.08588, 3.5353, 0.0}},
  };
  return t;
}

double DensityEffect(const Material& m, double T) {
  const double I = m.def.I_eV;
  const double x = std::log10(std::sqrt(T * (T + 2.0 * kEMC2)) / kEMC2);
  const auto it = SternheimerTable().find(m.def.name);
  if (it != SternheimerTable().end()) {
    const SternheimerParams& p = it->second;
    const double C = p.C + 2.0 * std::log(I / p.I);
    if (x < p.x0) return p.d0 > 0.0 ? p.d0 * std::pow(10.0, 2.0 * (x - p.x0)) : 0.0;
    if (x < p.x1) return 4.606 * x - C + p.a * std::pow(p.x1 - x, p.m);
    return 4.606 * x - C;
  }
  // Sternheimer-Peierls general parameters (condensed media unless rho < 0.01)
  // plasma energy 28.816 sqrt(rho <Z/A>) eV, with rho <Z/A> = electrons per cm3 / N_A
  const double plasma = 28.816 * std::sqrt(m.nElectrons * 1.0e3 / kNA);
  const double Cbar = 1.0 + 2.0 * std::log(I / plasma);
  double x0, x1;
  if (m.def.density < 0.01) {              // gases (Sternheimer-Peierls 1971)
    if (Cbar < 10.0)      { x0 = 1.6; x1 = 4.0; }
    else if (Cbar < 10.5) { x0 = 1.7; x1 = 4.0; }
    else if (Cbar < 11.0) { x0 = 1.8; x1 = 4.0; }
    else if (Cbar < 11.5) { x0 = 1.9; x1 = 4.0; }
    else if (Cbar < 12.25){ x0 = 2.0; x1 = 4.0; }
    else if (Cbar < 13.804){ x0 = 2.0; x1 = 5.0; }
    else                  { x0 = 0.326 * Cbar - 2.5; x1 = 5.0; }
  } else if (I < 100.0) {
    x1 = 2.0; x0 = (Cbar < 3.681) ? 0.2 : 0.326 * Cbar - 1.0;
  } else {
    x1 = 3.0; x0 = (Cbar < 5.215) ? 0.2 : 0.326 * Cbar - 1.5;
  }
  const double mexp = 3.0;
  const double a = (Cbar - 4.606 * x0) / std::pow(x1 - x0, mexp);
  if (x < x0) return 0.0;
  if (x < x1) return 4.606 * x - Cbar + a * std::pow(x1 - x, mexp);
  return 4.606 * x - Cbar;
}

double CollisionDEDX(const Material& m, double T, double ecut) {
  const double tau   = T / kEMC2;
  const double gamma = tau + 1.0;
  const double beta2 = tau * (tau + 2.0) / (gamma * gamma);
  const double d     = std::min(ecut, 0.5 * T) / kEMC2;
  const double ie    = m.def.I_eV * 1.0e-6 / kEMC2;
  double f = std::log(2.0 * (tau + 2.0) / (ie * ie)) - 1.0 - beta2 + std::log((tau - d) * d)
             + tau / (tau - d) + (0.5 * d * d + (2.0 * tau + 1.0) * std::log(1.0 - d / tau)) / (gamma * gamma);
  f -= DensityEffect(m, T);
  const double val = 2.0 * kPi * kRe * kRe * kEMC2 * m.nElectrons / beta2 * f;
  return std::max(0.0, val);
}

// Moller restricted macroscopic cross section for T' > ecut [1/mm]
double MollerIMFP(const Material& m, double T, double ecut) {
  if (T <= 2.0 * ecut) return 0.0;
  const double gamma = T / kEMC2 + 1.0;
  const double beta2 = 1.0 - 1.0 / (gamma * gamma);
  const double x = ecut / T;
  const double g2 = gamma * gamma;
  const double s = (gamma - 1.0) * (gamma - 1.0) / g2 * (0.5 - x) + 1.0 / x - 1.0 / (1.0 - x)
                   - (2.0 * gamma - 1.0) / g2 * std::log((1.0 - x) / x);
  return 2.0 * kPi * kRe * kRe * kEMC2 / (beta2 * T) * s * m.nElectrons;
}

// ---------------------------------------------------------------------------
// Photon cross sections per atom [mm^2]
// ---------------------------------------------------------------------------
double KleinNishinaPerElectron(double k) {
  const double x = k / kEMC2;
  const double l = std::log1p(2.0 * x);
  const double s = (1.0 + x) / (x * x) * (2.0 * (1.0 + x) / (1.0 + 2.0 * x) - l / x)
                   + l / (2.0 * x) - (1.0 + 3.0 * x) / ((1.0 + 2.0 * x) * (1.0 + 2.0 * x));
  return 2.0 * kPi * kRe * kRe * s;
}

double PairPerAtom(int Z, double k) {
  if (k <= 2.0 * kEMC2 * (1.0 + 1.0e-9)) return 0.0;
  const double emin = kEMC2 / k, emax = 1.0 - emin;
  const double z13 = std::pow(double(Z), 1.0 / 3.0);
  const double lz3 = std::log(double(Z)) / 3.0;
  auto dcs = [&](double e) {
    const double delta = 136.0 * kEMC2 / (z13 * k * e * (1.0 - e));
    double p1, p2;
    if (delta <= 1.0) {
      p1 = 20.867 - 3.242 * delta + 0.625 * delta * delta;
      p2 = 20.209 - 1.930 * delta - 0.086 * delta * delta;
    } else {
      p1 = p2 = 21.12 - 4.184 * std::log(delta + 0.952);
    }
    const double v = (e * e + (1.0 - e) * (1.0 - e)) * (0.25 * p1 - lz3)
                     + (2.0 / 3.0) * e * (1.0 - e) * (0.25 * p2 - lz3);
    return std::max(0.0, v);
  };
  // composite Simpson over the allowed energy fraction
  const int n = 400;
  const double h = (emax - emin) / n;
  double s = dcs(emin) + dcs(emax);
  for (int i = 1; i < n; ++i) s += (i % 2 ? 4.0 : 2.0) * dcs(emin + i * h);
  s *= h / 3.0;
  return 4.0 * kAlpha * kRe * kRe * Z * (Z + 1.0) * s;
}

double PhotoelectricPerAtom(int Z, double k) {
  const double sigmaT = 8.0 * kPi * kRe * kRe / 3.0;
  const double a4 = std::pow(kAlpha, 4.0);
  return 1.25 * 4.0 * std::sqrt(2.0) * std::pow(double(Z), 5.0) * a4 * sigmaT * std::pow(kEMC2 / k, 3.5);
}

// ---------------------------------------------------------------------------
// Walker alias tables over the bins of a piecewise-linear pdf (Vose's method).
// W[i] is the probability of keeping bin i, I[i] its alias; the layout is the
// one SimLinAliasData::Sample (SimLinAliasData.cc:25-42) consumes.
// ---------------------------------------------------------------------------
void BuildLinearAlias(const std::vector<double>& x, const std::vector<double>& y,
                      std::vector<double>& W, std::vector<int>& I) {
  const int n = int(x.size());
  const int nb = n - 1;
  std::vector<double> p(nb);
  double sum = 0.0;
  for (int i = 0; i < nb; ++i) {
    p[i] = std::max(1.0e-40, 0.5 * (x[i + 1] - x[i]) * (y[i] + y[i + 1]));
    sum += p[i];
  }
  for (auto& v : p) v *= nb / sum;
  W.assign(n, 1.0);
  I.assign(n, 0);
  std::vector<int> small, large;
  for (int i = 0; i < nb; ++i) (p[i] < 1.0 ? small : large).push_back(i);
  while (!small.empty() && !large.empty()) {
    const int s = small.back(); small.pop_back();
    const int l = large.back();
    W[s] = p[s];
    I[s] = l;
    p[l] -= 1.0 - p[s];
    if (p[l] < 1.0) { large.pop_back(); small.push_back(l); }
  }
  for (int s : small) { W[s] = 1.0; I[s] = s; }
  for (int l : large) { W[l] = 1.0; I[l] = l; }
  for (int i = 0; i < nb; ++i) if (W[i] >= 1.0) I[i] = i;
}

// adaptive point insertion: start from the given abscissas and bisect the bin
// whose midpoint linear-interpolation error (relative or absolute) is largest
template <class F>
void AdaptiveGrid(std::vector<double>& x, std::vector<double>& y, int n, F pdf, bool relative) {
  while (int(x.size()) < n) {
    double best = -1.0, bx = 0, by = 0;
    int bi = 0;
    for (size_t i = 0; i + 1 < x.size(); ++i) {
      const double xm = 0.5 * (x[i] + x[i + 1]);
      const double ym = 0.5 * (y[i] + y[i + 1]);
      const double v  = pdf(xm);
      const double e  = relative ? std::fabs(1.0 - ym / v) : std::fabs(ym - v);
      if (e > best) { best = e; bi = int(i); bx = xm; by = v; }
    }
    x.insert(x.begin() + bi + 1, bx);
    y.insert(y.begin() + bi + 1, by);
  }
}

struct AliasTable1 { double E; std::vector<double> x, y, w; std::vector<int> idx; };

void WriteAliasRows(FILE* f, const AliasTable1& t) {
  const int n = int(t.x.size());
  for (int i = 0; i < n; ++i) {
    std::fprintf(f, "%22.14E  %22.14E  %22.14E  %d ", t.x[i], t.y[i], t.w[i], t.idx[i]);
    if ((i + 1) % 2 == 0 || i == n - 1) std::fprintf(f, "\n");
  }
}

std::vector<double> LogGrid(double a, double b, int n) {
  std::vector<double> g(n);
  const double la = std::log(a), d = std::log(b / a) / (n - 1);
  g[0] = a;
  for (int i = 1; i < n - 1; ++i) g[i] = std::exp(la + i * d);
  g[n - 1] = b;
  return g;
}

// ---------------------------------------------------------------------------
// Goudsmit-Saunderson distributions
// ---------------------------------------------------------------------------
double Digamma1p(int n) {   // psi(n+1) for integer n >= 1
  if (n < 8) {
    double h = 0.0;
    for (int i = 1; i <= n; ++i) h += 1.0 / i;
    return h - 0.5772156649015329;
  }
  const double in2 = 1.0 / (double(n) * n);
  return std::log(double(n)) + 0.5 / n - in2 / 12.0 + in2 * in2 / 120.0;
}

// xi_l = [exp(-nel G_l) - exp(-nel)]/[1 - exp(-nel)]: the Legendre coefficients
// of the angular distribution after `nel` elastic collisions on average, with
// the no-scattering term removed; G_l from the Bessel-K1 approximation.
std::vector<double> GSCoefficients(double nel, double A) {
  std::vector<double> xi;
  xi.reserve(4096);
  const double en = std::exp(-nel);
  xi.push_back(1.0);
  for (int l = 1; l < 400000; ++l) {
    const double ll = double(l) * (l + 1.0);
    const double y  = 2.0 * std::sqrt(ll * A);
    double G = 1.0;
    if (y < 30.0) {
      const double k1 = std::cyl_bessel_k(1.0, y);
      G = 1.0 - y * k1 * (1.0 + 0.5 * y * y * (Digamma1p(l) - 0.5 * std::log(ll)));
    }
    const double v = (std::exp(-nel * G) - en) / (1.0 - en);
    xi.push_back(v);
    if (y > 30.0 || (l > 20 && std::fabs(v) * (l + 0.5) < 1.0e-13)) break;
  }
  return xi;
}

// q(u) for the transformed variable u, mu(u) = 1 - 2au/(1-u+a)
double GSTransformedPDF(const std::vector<double>& xi, double a, double u) {
  const double k  = 1.0 / (1.0 - u + a);
  const double mu = 1.0 - 2.0 * a * u * k;
  double p0 = 1.0, p1 = mu;
  double sum = 0.5 * xi[0] + 1.5 * mu * xi[1];
  for (size_t l = 1; l + 1 < xi.size(); ++l) {
    const double p2 = ((2.0 * l + 1.0) * mu * p1 - double(l) * p0) / (l + 1.0);
    sum += (l + 1.5) * p2 * xi[l + 1];
    p0 = p1; p1 = p2;
  }
  return 2.0 * a * (1.0 + a) * k * k * std::max(sum, 0.0);
}

// natural cubic spline (second-derivative form) used for the dense q(u) curve
struct Cubic {
  std::vector<double> x, y, m;
  void Set(const std::vector<double>& xx, const std::vector<double>& yy) {
    x = xx; y = yy;
    const int n = int(x.size());
    m.assign(n, 0.0);
    std::vector<double> c(n, 0.0), d(n, 0.0);
    for (int i = 1; i < n - 1; ++i) {
      const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
      const double r  = 6.0 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
      const double b  = 2.0 * (h0 + h1) - h0 * c[i - 1];
      c[i] = h1 / b;
      d[i] = (r - h0 * d[i - 1]) / b;
    }
    for (int i = n - 2; i > 0; --i) m[i] = d[i] - c[i] * m[i + 1];
  }
  double operator()(double t) const {
    int j = int(std::upper_bound(x.begin(), x.end(), t) - x.begin()) - 1;
    j = std::max(0, std::min(int(x.size()) - 2, j));
    const double h = x[j + 1] - x[j], a = (x[j + 1] - t) / h, b = (t - x[j]) / h;
    return a * y[j] + b * y[j + 1] + ((a * a * a - a) * m[j] + (b * b * b - b) * m[j + 1]) * h * h / 6.0;
  }
};

struct GSTable { double E, a; std::vector<double> u, pa, pb; };

GSTable BuildGSTable(double E, double nel, double A, int nCum) {
  GSTable t;
  t.E = E;
  std::vector<double> xi = GSCoefficients(nel, A);
  // transformation parameter: the `a` for which a flat q(u) reproduces the mean
  // of (1-mu) of the distribution, i.e. G1(a) = 1 - <mu> = 1 - xi_1
  t.a = ScreeningFromG1(std::max(1.0e-14, 1.0 - xi[1]));
  const int nu = 1024;
  std::vector<double> ug(nu), qg(nu);
  for (int i = 0; i < nu; ++i) {
    ug[i] = (i == nu - 1) ? 1.0 : i / double(nu - 1);
    qg[i] = GSTransformedPDF(xi, t.a, ug[i]);
  }
  // keep the pdf strictly positive so that the rational-interpolation
  // parameters stay finite where the Legendre sum was clipped at zero
  const double qmax = *std::max_element(qg.begin(), qg.end());
  for (auto& q : qg) q = std::max(q, 1.0e-12 * qmax);
  Cubic sp;
  sp.Set(ug, qg);
  // CDF by 8-point Gauss-Legendre on each dense interval of the spline
  static const double gx[8] = {0.0198550717512319, 0.1016667612931866, 0.2372337950418355, 0.4082826787521751,
                               0.5917173212478249, 0.7627662049581645, 0.8983332387068134, 0.9801449282487681};
  static const double gw[8] = {0.0506142681451881, 0.1111905172266872, 0.1568533229389436, 0.1813418916891810,
                               0.1813418916891810, 0.1568533229389436, 0.1111905172266872, 0.0506142681451881};
  std::vector<double> cdf(nu, 0.0);
  for (int i = 1; i < nu; ++i) {
    const double h = ug[i] - ug[i - 1];
    double s = 0.0;
    for (int j = 0; j < 8; ++j) s += gw[j] * std::max(0.0, sp(ug[i - 1] + gx[j] * h));
    cdf[i] = cdf[i - 1] + s * h;
  }
  const double norm = 1.0 / cdf[nu - 1];
  for (int i = 0; i < nu; ++i) { cdf[i] *= norm; qg[i] *= norm; }
  sp.Set(ug, qg);
  // rational-interpolation parameters on the dense grid, then the u values at
  // the equally spaced cumulative grid, then the parameters on that grid
  auto ratinAB = [](double dc, double du, double p0, double p1, double& pa, double& pb) {
    const double r = dc / du;
    pb = 1.0 - r * r / (p0 * p1);
    pa = r / p0 - 1.0 - pb;
  };
  std::vector<double> da(nu - 1), db(nu - 1);
  for (int i = 0; i + 1 < nu; ++i) ratinAB(cdf[i + 1] - cdf[i], ug[i + 1] - ug[i], qg[i], qg[i + 1], da[i], db[i]);
  t.u.assign(nCum, 0.0);
  t.u[nCum - 1] = 1.0;
  const double dc = 1.0 / (nCum - 1);
  for (int c = 1; c < nCum - 1; ++c) {
    const double cv = c * dc;
    int j = int(std::upper_bound(cdf.begin(), cdf.end(), cv) - cdf.begin()) - 1;
    j = std::max(0, std::min(nu - 2, j));
    const double del = cdf[j + 1] - cdf[j], r = cv - cdf[j];
    const double n1 = (1.0 + da[j] + db[j]) * del * r;
    const double n2 = del * del + da[j] * del * r + db[j] * r * r;
    t.u[c] = ug[j] + n1 / n2 * (ug[j + 1] - ug[j]);
  }
  t.pa.assign(nCum, 0.0);
  t.pb.assign(nCum, 0.0);
  for (int c = 0; c + 1 < nCum; ++c) {
    const double p0 = std::max(1.0e-300, sp(t.u[c])), p1 = std::max(1.0e-300, sp(t.u[c + 1]));
    ratinAB(dc, t.u[c + 1] - t.u[c], p0, p1, t.pa[c], t.pb[c]);
  }
  return t;
}

// ---------------------------------------------------------------------------
FILE* OpenOut(const std::string& dir, const char* name) {
  const std::string p = dir + "/" + name;
  FILE* f = std::fopen(p.c_str(), "w");
  if (!f) { std::fprintf(stderr, "cannot create %s\n", p.c_str()); std::exit(2); }
  return f;
}

struct Config {
  std::vector<std::string> mats{"G4_WATER"};
  double ecut = 0.2, gcut = 0.05, slow = 5.0, shigh = 10.0, ecross = 12.0, emax = 21.0;
  int nEl = 128, nPh = 1024;
};

Config PresetConfig(int idx) {   // Configuration.hh:69-111, plus index 6
  Config c;
  switch (idx) {
    case 1: c.mats = {"G4_WATER", "G4_AIR"}; break;
    case 2: c.mats = {"G4_WATER", "G4_BONE_CORTICAL_ICRP"}; break;
    case 3: c.mats = {"G4_WATER", "G4_Ti", "G4_BONE_COMPACT_ICRU"}; break;
    case 4: c.slow = 2.0; c.shigh = 5.0; c.mats = {"G4_Ti"}; break;
    case 5: c.slow = 1.0; c.shigh = 1.0; c.mats = {"G4_W"}; break;
    case 6: c.mats = {"G4_WATER", "G4_LUNG_ICRP", "G4_BONE_COMPACT_ICRU"}; break;
    default: break;
  }
  return c;
}

}  // namespace

int main(int argc, char** argv) {
  std::string outDir = "./data", sbDir;
  int cfgIdx = 0;
  std::string matOverride;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) { std::fprintf(stderr, "missing value for %s\n", a.c_str()); std::exit(1); }
      return argv[++i];
    };
    if (a == "-d") outDir = next();
    else if (a == "-c") cfgIdx = std::atoi(next().c_str());
    else if (a == "-s") sbDir = next();
    else if (a == "-m") matOverride = next();
    else { std::fprintf(stderr, "usage: %s -d outdir -c idx -s sb-data-dir [-m m1,m2]\n", argv[0]); return 1; }
  }
  if (sbDir.empty()) { std::fprintf(stderr, "the Seltzer-Berger data directory (-s) is required\n"); return 1; }
  Config cfg = PresetConfig(cfgIdx);
  if (!matOverride.empty()) {
    cfg.mats.clear();
    size_t p = 0;
    while (p <= matOverride.size()) {
      size_t q = matOverride.find(',', p);
      if (q == std::string::npos) q = matOverride.size();
      cfg.mats.push_back(matOverride.substr(p, q - p));
      p = q + 1;
    }
  }
  std::vector<Material> mats;
  std::vector<int> allZ;
  for (auto& nm : cfg.mats) {
    const MaterialDef* d = nullptr;
    for (auto& m : MaterialLibrary()) if (m.name == nm) d = &m;
    if (!d) { std::fprintf(stderr, "unknown material %s\n", nm.c_str()); return 1; }
    mats.push_back(BuildMaterial(*d));
    for (int z : mats.back().Z) allZ.push_back(z);
  }
  SBData sb;
  if (!sb.Load(sbDir, allZ)) return 2;
  const int nmat = int(mats.size());
  const double ecut = cfg.ecut, gcut = cfg.gcut, emax = cfg.emax;

  // electron grid (ElectronData.hh:161-179): 128 log points on [0.99 ecut, emax]
  const std::vector<double> eg = LogGrid(0.99 * ecut, emax, cfg.nEl);
  const int ne = cfg.nEl;
  std::vector<std::vector<double>> el(nmat, std::vector<double>(ne)), tr1(nmat, std::vector<double>(ne)),
      scr(nmat, std::vector<double>(ne)), k1(nmat, std::vector<double>(ne)), dedx(nmat, std::vector<double>(ne)),
      range(nmat, std::vector<double>(ne)), bremE(nmat), brem(nmat), molE(nmat), mol(nmat);
  auto allowedK1 = [&](const Material& m, double E) {
    double mEl, mTr1;
    MacroElastic(m, E, mEl, mTr1);
    const double fx = std::atan(5.0 * std::log(E / cfg.ecross)) / kPi + 0.5;
    return m.scpc * mTr1 * cfg.slow * std::pow(cfg.shigh / cfg.slow, fx);
  };
  for (int im = 0; im < nmat; ++im) {
    const Material& m = mats[im];
    for (int ie = 0; ie < ne; ++ie) {
      const double E = eg[ie];
      double mEl, mTr1;
      MacroElastic(m, E, mEl, mTr1);
      el[im][ie]  = 1.0 / mEl;
      tr1[im][ie] = 1.0 / mTr1;
      scr[im][ie] = ScreeningFromG1(mTr1 / mEl);
      k1[im][ie]  = allowedK1(m, E);
      double rad, bimfp;
      BremQuantities(m, sb, E, gcut, rad, bimfp);
      dedx[im][ie] = CollisionDEDX(m, E, ecut) + rad;
    }
    // restricted range: trapezoid of 1/dedx on a fine log grid from the lowest energy
    {
      std::vector<double> fg = LogGrid(eg.front(), emax, 4096);
      std::vector<double> fr(fg.size(), 0.0);
      auto sp = [&](double E) { double r, b; BremQuantities(m, sb, E, gcut, r, b); return CollisionDEDX(m, E, ecut) + r; };
      double prev = 1.0 / sp(fg[0]);
      for (size_t j = 1; j < fg.size(); ++j) {
        const double cur = 1.0 / sp(fg[j]);
        fr[j] = fr[j - 1] + 0.5 * (prev + cur) * (fg[j] - fg[j - 1]);
        prev = cur;
      }
      for (int ie = 0; ie < ne; ++ie) {
        int j = int(std::upper_bound(fg.begin(), fg.end(), eg[ie]) - fg.begin()) - 1;
        j = std::max(0, std::min(int(fg.size()) - 2, j));
        const double w = (eg[ie] - fg[j]) / (fg[j + 1] - fg[j]);
        range[im][ie] = fr[j] + w * (fr[j + 1] - fr[j]);
      }
    }
    bremE[im] = LogGrid(std::max(ecut, gcut), emax, ne);
    molE[im]  = LogGrid(2.0 * ecut, emax, ne);
    for (int ie = 0; ie < ne; ++ie) {
      double rad, bimfp;
      BremQuantities(m, sb, bremE[im][ie], gcut, rad, bimfp);
      brem[im].push_back(std::max(1.0e-20, bimfp));
      mol[im].push_back(std::max(1.0e-20, MollerIMFP(m, molE[im][ie], ecut)));
    }
  }

  // --- mat.dat
  {
    FILE* f = OpenOut(outDir, "mat.dat");
    std::fprintf(f, "# Secondary electron and gamma production thresholds:\n %.8E %.8E\n", ecut, gcut);
    std::fprintf(f, "# MSC maximum step length parameters:\n %.8E %.8E %.8E\n", cfg.slow, cfg.shigh, cfg.ecross);
    std::fprintf(f, "# Number of materials:\n %d\n", nmat);
    for (int im = 0; im < nmat; ++im) {
      const Material& m = mats[im];
      std::fprintf(f, "# \n# Material index, name and density [g/cm3] data:\n");
      std::fprintf(f, " %d %16s %.8E\n", im, m.def.name.c_str(), m.def.density);
      std::fprintf(f, "# Z, Z^2, Z(Z+1), w [amu], wZ [amu], I [MeV] (all are weighted for molecules)\n");
      std::fprintf(f, " %.8E  %.8E  %.8E  %.8E  %.8E  %.8E\n", m.zMean, m.z2, m.zs, m.wMean, m.zw, m.iMeanMeV);
      std::fprintf(f, "# [Z/w]/[Z/w]_ref, [Z^2/w]/[Z^2/w]_ref (all are weighted for molecules) ref: im=0\n");
      std::fprintf(f, " %.8E  %.8E\n", m.zMean / m.wMean * mats[0].wMean / mats[0].zMean,
                   m.z2 / m.wMean * mats[0].wMean / mats[0].z2);
    }
    std::fclose(f);
  }
  auto matHeader = [&](FILE* f, int im) { std::fprintf(f, "#\n# Material name: %s\n#\n", mats[im].def.name.c_str()); };
  // --- el_iemfp.dat (not read by the simulation)
  {
    FILE* f = OpenOut(outDir, "el_iemfp.dat");
    std::fprintf(f, "# Inverse elastic mean free path, i.e. macroscopic cross section, data\n");
    std::fprintf(f, "# The `_scpc` are the scattering power corrected, i.e. inelastic scattering correected, data) \n");
    std::fprintf(f, "# E [MeV]   1/Lambda_elastic [1/mm] 1/Lambda_elastic_scpc [1/mm]  \n");
    std::fprintf(f, "# number of data per materials\n %d\n", ne);
    std::fprintf(f, "# -----------------------------\n");
    for (int im = 0; im < nmat; ++im) {
      matHeader(f, im);
      for (int ie = 0; ie < ne; ++ie)
        std::fprintf(f, "%.8E  %.8E  %.8E\n", eg[ie], 1.0 / el[im][ie], mats[im].scpc / el[im][ie]);
    }
    std::fclose(f);
  }
  // --- el_itr1mfp.dat
  {
    FILE* f = OpenOut(outDir, "el_itr1mfp.dat");
    std::fprintf(f, "# Inverse 1-rst transport mean free path, i.e. macroscopic cross section, data\n");
    std::fprintf(f, "# The `scpc` are the scattering power corrected, i.e. inelastic scattering correected, data) \n");
    std::fprintf(f, "# E [MeV]   1/Lambda_1 [1/mm][cm3/g] 1/Lambda_1^{scpc} [1/mm][cm3/g]  \n");
    std::fprintf(f, "# number of data per materials and #material\n %d %d\n", ne, nmat);
    std::fprintf(f, "# -----------------------------\n");
    for (int im = 0; im < nmat; ++im) {
      const double rho = mats[im].def.density;
      matHeader(f, im);
      for (int ie = 0; ie < ne; ++ie)
        std::fprintf(f, "%.8E  %.8E  %.8E\n", eg[ie], 1.0 / tr1[im][ie] / rho, mats[im].scpc / tr1[im][ie] / rho);
    }
    std::fclose(f);
  }
  // --- el_screeningPar.dat (not read by the simulation)
  {
    FILE* f = OpenOut(outDir, "el_screeningPar.dat");
    std::fprintf(f, "# Screening parameter of the screened Rutherford DCS\n");
    std::fprintf(f, "# (i.e. \\eta(E_i), such that the accurate G_1(\\eta) = mfp_el/mfp_tr1) \n");
    std::fprintf(f, "# E [MeV]   Screening_parameter [] \n");
    std::fprintf(f, "# number of data per materials\n %d\n", ne);
    std::fprintf(f, "# -----------------------------\n");
    for (int im = 0; im < nmat; ++im) {
      matHeader(f, im);
      for (int ie = 0; ie < ne; ++ie) std::fprintf(f, "%.8E  %.8E\n", eg[ie], scr[im][ie]);
    }
    std::fclose(f);
  }
  // --- el_scatStrength.dat
  {
    FILE* f = OpenOut(outDir, "el_scatStrength.dat");
    std::fprintf(f, "# The max scattering strength `K_1(E)` allowed in a given MSC step.\n");
    std::fprintf(f, "# Max K_1(E) is approximated as max-MSC-step-length(E)/tr1-mfp(E).\n");
    std::fprintf(f, "# E [MeV]   Max-scattering-strength [] \n");
    std::fprintf(f, "# number of data per materials\n %d\n", ne);
    std::fprintf(f, "# -----------------------------\n");
    for (int im = 0; im < nmat; ++im) {
      matHeader(f, im);
      for (int ie = 0; ie < ne; ++ie) std::fprintf(f, "%.8E  %.8E\n", eg[ie], k1[im][ie]);
    }
    std::fclose(f);
  }
  // --- el_GSDtrData.dat: 256 log energies on [ecut, emax] x 64 cumulative values
  {
    const int nGS = 256, nCum = 64;
    std::vector<double> gsE(nGS);
    const double lmin = std::log(ecut), dl = std::log(emax / ecut) / (nGS - 1);
    for (int i = 0; i < nGS - 1; ++i) gsE[i] = std::exp(lmin + i * dl);
    gsE[nGS - 1] = emax;
    FILE* f = OpenOut(outDir, "el_GSDtrData.dat");
    std::fprintf(f, "# Data related to the transformed GS angular distributions:\n");
    std::fprintf(f, "# (optimal transformation parameters `a` and tables for fast,\n");
    std::fprintf(f, "#  rejection free sampling from the q(u;s/emfp,scrPar,a) pdf-s)\n");
    std::fprintf(f, "# #ekin, emin [MeV], emax [MeV] and #cumulative:\n");
    std::fprintf(f, "%d  %.14E  %.14E  %d\n", nGS, gsE[0], gsE[nGS - 1], nCum);
    std::fprintf(f, "# For each materials: #ekin tables and 3x#cumulative data in each table,\n");
    std::fprintf(f, "# i, E_i [MeV] and transformation parameter are given before each table.\n");
    std::fprintf(f, "# -----------------------------\n");
    for (int im = 0; im < nmat; ++im) {
      const Material& m = mats[im];
      matHeader(f, im);
      for (int ie = 0; ie < nGS; ++ie) {
        const double E = gsE[ie];
        double mEl, mTr1;
        MacroElastic(m, E, mEl, mTr1);
        const double g1  = mTr1 / mEl;                 // lambda_el / lambda_1
        const double nel = allowedK1(m, E) / g1;       // s / lambda_el (scpc both)
        const double A   = ScreeningFromG1(g1);
        GSTable t = BuildGSTable(E, nel, A, nCum);
        std::fprintf(f, "%d  %.14E  %.14E\n", ie, E, t.a);
        for (int iu = 0; iu < nCum; ++iu) {
          std::fprintf(f, "%22.14E  %22.14E  %22.14E ", t.u[iu], t.pa[iu], t.pb[iu]);
          if ((iu + 1) % 2 == 0 || iu == nCum - 1) std::fprintf(f, "\n");
        }
      }
    }
    std::fclose(f);
  }
  // --- eloss_rdedx.dat (its first header line has no newline: 2-line header)
  {
    FILE* f = OpenOut(outDir, "eloss_rdedx.dat");
    std::fprintf(f, "# The restricted, total (collisonal and radiative) stopping power");
    std::fprintf(f, "# E [MeV]   dE/dx [MeV/mm][cm3/g] \n");
    std::fprintf(f, "# number of data per materials and #material\n %d %d\n", ne, nmat);
    std::fprintf(f, "# -----------------------------\n");
    for (int im = 0; im < nmat; ++im) {
      matHeader(f, im);
      for (int ie = 0; ie < ne; ++ie)
        std::fprintf(f, "%.8E  %.8E\n", eg[ie], dedx[im][ie] / mats[im].def.density);
    }
    std::fclose(f);
  }
  // --- eloss_rRange.dat (not read by the simulation)
  {
    FILE* f = OpenOut(outDir, "eloss_rRange.dat");
    std::fprintf(f, "# The restricted, total (collisonal and radiative) range");
    std::fprintf(f, "# E [MeV]   Range [mm] \n");
    std::fprintf(f, "# number of data per materials\n %d\n", ne);
    std::fprintf(f, "# -----------------------------\n");
    for (int im = 0; im < nmat; ++im) {
      matHeader(f, im);
      for (int ie = 0; ie < ne; ++ie) std::fprintf(f, "%.8E  %.8E\n", eg[ie], range[im][ie]);
    }
    std::fclose(f);
  }
  // --- imfp_brem.dat
  {
    FILE* f = OpenOut(outDir, "imfp_brem.dat");
    std::fprintf(f, "# The restricted imfp for bremsstrahlung interaction\n");
    std::fprintf(f, "# E [MeV]   Brem_IMFP [1/mm][cm3/g] \n");
    std::fprintf(f, "# number of data per materials and #materials\n %d %d\n", ne, nmat);
    std::fprintf(f, "# -----------------------------\n");
    for (int im = 0; im < nmat; ++im) {
      matHeader(f, im);
      for (int ie = 0; ie < ne; ++ie)
        std::fprintf(f, "%.8E  %.8E\n", bremE[im][ie], brem[im][ie] / mats[im].def.density);
    }
    std::fclose(f);
  }
  // --- imfp_moller.dat
  {
    FILE* f = OpenOut(outDir, "imfp_moller.dat");
    std::fprintf(f, "# The restricted imfp for Moller interaction\n");
    std::fprintf(f, "# E [MeV]   Moller_IMFP [1/mm][cm3/g] \n");
    std::fprintf(f, "# number of data per materials\n %d\n", ne);
    std::fprintf(f, "# -----------------------------\n");
    for (int im = 0; im < nmat; ++im) {
      matHeader(f, im);
      for (int ie = 0; ie < ne; ++ie)
        std::fprintf(f, "%.8E  %.8E\n", molE[im][ie], mol[im][ie] / mats[im].def.density);
    }
    std::fclose(f);
  }
  // --- ioni_MollerDtrData.dat: 128 log energies on [2 ecut, emax] x 64 uniform xi
  {
    const int nP = 128, nS = 64;
    std::vector<double> pe = LogGrid(2.0 * ecut, emax, nP);
    FILE* f = OpenOut(outDir, "ioni_MollerDtrData.dat");
    std::fprintf(f, "# Tables for rejection free sampling of the energy transferred to the\n");
    std::fprintf(f, "# secondary electron in Moller scattering (transformed variable xi).\n");
    std::fprintf(f, "# The size of the discrete primary (np) and secondary (ns) energies first \n");
    std::fprintf(f, "# then the primary energy and the corresponding (4 x ns) sampling table data \n");
    std::fprintf(f, "# each of the (np) discrete primary energies. \n");
    std::fprintf(f, "%d %d\n", nP, nS);
    for (int ie = 0; ie < nP; ++ie) {
      double T = pe[ie];
      if (ie == 0) T += 1.0e-6;
      if (ie == nP - 1) T -= 1.0e-6;
      const double gamma = T / kEMC2 + 1.0, g2 = gamma * gamma;
      const double C1 = (gamma - 1.0) * (gamma - 1.0) / g2, C2 = (2.0 * gamma - 1.0) / g2;
      const double e0 = ecut / T, lr = std::log(0.5 / e0);
      AliasTable1 t;
      t.E = pe[ie];
      for (int i = 0; i < nS; ++i) {
        const double xi = (i == nS - 1) ? 1.0 : i / double(nS - 1);
        const double a = e0 * std::exp(xi * lr), b = 1.0 - a;
        // eps * dsigma/deps of the Moller DCS (up to constants): pdf in xi
        t.x.push_back(xi);
        t.y.push_back(((1.0 / a - C2) + a * C1 + a / b * (1.0 / b - C2)) * e0);
      }
      BuildLinearAlias(t.x, t.y, t.w, t.idx);
      std::fprintf(f, "%22.14E\n", t.E);
      WriteAliasRows(f, t);
    }
    std::fclose(f);
  }
  // --- brem_SBDtrData.dat: per material 128 log energies on [gcut, emax] x 64
  {
    const int nP = 128, nS = 64;
    std::vector<double> pe = LogGrid(gcut, emax, nP);
    FILE* f = OpenOut(outDir, "brem_SBDtrData.dat");
    std::fprintf(f, "# Tables for rejection free sampling of the emitted photon energy\n");
    std::fprintf(f, "# in electron bremsstrahlung interaction according to the Seltzer-Berger DCS.\n");
    std::fprintf(f, "# The size of the discrete primary (np), secondary (ns) energies and #materials first \n");
    std::fprintf(f, "# followed by the discrete primary energy grid and for each material (np) tables with \n");
    std::fprintf(f, "# (4 x ns) sampling table data each. \n");
    std::fprintf(f, "%d %d %d\n", nP, nS, nmat);
    for (int ie = 0; ie < nP; ++ie) {
      std::fprintf(f, "%22.14E ", pe[ie]);
      if ((ie + 1) % 6 == 0 || ie == nP - 1) std::fprintf(f, "\n");
    }
    for (int im = 0; im < nmat; ++im) {
      matHeader(f, im);
      for (int ie = 0; ie < nP; ++ie) {
        double T = pe[ie];
        if (ie == 0) T += 1.0e-6;
        if (ie == nP - 1) T -= 1.0e-6;
        const std::vector<double> c = MaterialChi(mats[im], sb, T);
        const double kc = gcut / T, lkc = std::log(kc);
        // pdf in xi = 1 - ln(kappa)/ln(kappa_c) is proportional to chi(kappa(xi))
        auto pdf = [&](double xi) { return InterpChi(sb.kappa, c, kc * std::exp(-xi * lkc)); };
        AliasTable1 t;
        t.E = pe[ie];
        t.x = {0.0};
        t.y = {pdf(0.0)};
        for (size_t k = 0; k + 1 < sb.kappa.size(); ++k) {
          if (sb.kappa[k] <= kc) continue;
          const double xi = 1.0 - std::log(sb.kappa[k]) / lkc;
          if (xi >= 1.0) continue;
          t.x.push_back(xi);
          t.y.push_back(c[k]);
        }
        t.x.push_back(1.0);
        t.y.push_back(c.back());
        AdaptiveGrid(t.x, t.y, nS, pdf, false);
        BuildLinearAlias(t.x, t.y, t.w, t.idx);
        WriteAliasRows(f, t);
      }
    }
    std::fclose(f);
  }
  // --- photon data: 1024 linear points on [0.99 gcut, emax]
  {
    const int np = cfg.nPh;
    std::vector<double> pg(np);
    const double pmin = 0.99 * gcut, inv = 1.0 / ((emax - pmin) / (np - 1));
    pg[0] = pmin;
    for (int i = 1; i < np - 1; ++i) pg[i] = pmin + i / inv;
    pg[np - 1] = emax;
    std::vector<std::vector<double>> comp(nmat, std::vector<double>(np)), pair(nmat, std::vector<double>(np)),
        phot(nmat, std::vector<double>(np)), tot(nmat, std::vector<double>(np));
    std::vector<double> gmax(np, 0.0);
    for (int im = 0; im < nmat; ++im) {
      const Material& m = mats[im];
      for (int ie = 0; ie < np; ++ie) {
        const double k = pg[ie];
        double c = 0, p = 0, ph = 0;
        for (size_t i = 0; i < m.Z.size(); ++i) {
          c  += m.nAtoms[i] * m.Z[i] * KleinNishinaPerElectron(k);
          p  += m.nAtoms[i] * PairPerAtom(m.Z[i], k);
          ph += m.nAtoms[i] * PhotoelectricPerAtom(m.Z[i], k);
        }
        comp[im][ie] = std::max(1.0e-20, c);
        pair[im][ie] = std::max(1.0e-20, p);
        phot[im][ie] = std::max(1.0e-20, ph);
        tot[im][ie]  = comp[im][ie] + pair[im][ie] + phot[im][ie];
        if (im == 0 || gmax[ie] < tot[im][ie]) gmax[ie] = tot[im][ie];
      }
    }
    auto writePh = [&](const char* fname, const char* l1, const char* l2, const std::vector<std::vector<double>>& v) {
      FILE* f = OpenOut(outDir, fname);
      std::fprintf(f, "%s", l1);
      std::fprintf(f, "%s", l2);
      std::fprintf(f, "# number of data per materials and #material\n %d %d\n", np, nmat);
      std::fprintf(f, "# -----------------------------\n");
      for (int im = 0; im < nmat; ++im) {
        matHeader(f, im);
        for (int ie = 0; ie < np; ++ie) std::fprintf(f, "%.8E  %.8E\n", pg[ie], v[im][ie] / mats[im].def.density);
      }
      std::fclose(f);
    };
    writePh("imfp_compton.dat", "# The imfp for Compton scattering\n", "# E [MeV]   Compton_IMFP [1/mm] \n", comp);
    writePh("imfp_pairp.dat", "# The imfp for e- e+ pair production.\n", "# E [MeV]   Pair_IMFP [1/mm] \n", pair);
    writePh("imfp_photoe.dat", "# The imfp for photoelectric effect.\n", "# E [MeV]   PhotoEl_IMFP [1/mm] \n", phot);
    writePh("imfp_total.dat", "# The total imfp = compton + pair + photoe  .\n", "# E [MeV]   Total_IMFP [1/mm] \n", tot);
    FILE* f = OpenOut(outDir, "imfp_globalMax.dat");
    std::fprintf(f, "# The global max tota-imfp.\n");
    std::fprintf(f, "# E [MeV]   Max-Total_IMFP [1/mm] \n");
    std::fprintf(f, "# number of data per materials\n %d\n", np);
    std::fprintf(f, "# -----------------------------\n");
    for (int ie = 0; ie < np; ++ie) std::fprintf(f, "%.8E  %.8E\n", pg[ie], gmax[ie]);
    std::fclose(f);
  }
  // --- compton_KNDtrData.dat: 32 log energies on [gcut, emax] x 64 adaptive xi
  {
    const int nP = 32, nS = 64;
    std::vector<double> pe = LogGrid(gcut, emax, nP);
    FILE* f = OpenOut(outDir, "compton_KNDtrData.dat");
    std::fprintf(f, "# Tables for rejection free sampling of reduced energy transfer\n");
    std::fprintf(f, "# in Compton scattering according to the Klein-Nishina DCS.\n");
    std::fprintf(f, "# The size of the discrete primary (np) and secondary (ns) energies first \n");
    std::fprintf(f, "# then the primary energy and the corresponding (4 x ns) sampling table data \n");
    std::fprintf(f, "# each of the (np) discrete primary energies. \n");
    std::fprintf(f, "%d %d\n", nP, nS);
    for (int ie = 0; ie < nP; ++ie) {
      double k = pe[ie];
      if (ie == 0) k += 1.0e-6;
      if (ie == nP - 1) k -= 1.0e-6;
      const double kappa = k / kEMC2;
      // pdf in xi, eps = exp(ln(1/(1+2 kappa)) (1 - xi)): eps * dsigma_KN/deps
      auto pdf = [kappa](double xi) {
        const double l = std::log(1.0 / (1.0 + 2.0 * kappa));
        const double eps = std::exp(l * (1.0 - xi)), ie_ = 1.0 / eps;
        const double beta = (1.0 - ie_) / kappa;
        return eps * (eps + ie_) * (1.0 + eps * beta * (2.0 + beta) / (1.0 + eps * eps));
      };
      AliasTable1 t;
      t.E = pe[ie];
      t.x = {0.0, 0.5, 1.0};
      t.y = {pdf(0.0), pdf(0.5), pdf(1.0)};
      AdaptiveGrid(t.x, t.y, nS, pdf, true);
      BuildLinearAlias(t.x, t.y, t.w, t.idx);
      std::fprintf(f, "%22.14E\n", t.E);
      WriteAliasRows(f, t);
    }
    std::fclose(f);
  }
  std::printf("dpm_generate_data: wrote %d materials to %s\n", nmat, outDir.c_str());
  return 0;
}
