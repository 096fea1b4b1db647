// C entry points into the reference's own simulation code, compiled from the
// unmodified reference sources (Simulation/src/*.cc) by oracle/build_ref.sh.
// TEST INFRASTRUCTURE ONLY: used to generate the golden vectors under
// tests/golden/ and to pin the CPU oracle (oracle/dpm_oracle.cc) bit for bit.
//
// Two transport entry points:
//   ref_simulate_cli  : the unmodified `Simulate` (SimDPMLike.cc:40-251), which
//                       writes the reference's hist.sim text file;
//   ref_simulate_full : the same history loop (SimDPMLike.cc:57-247) restated
//                       here around the reference's own KeepTrackingElectron /
//                       KeepTrackingPhoton / Perform* functions and the
//                       reference's own Geom, returning the full-precision
//                       depth histograms (the hist.sim file keeps 5 digits).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#define private public
#include "Geom.hh"
#undef private

#include "Random.hh"
#include "SimDPMLike.hh"
#include "SimElectronData.hh"
#include "SimGSTables.hh"
#include "SimIMFPBrem.hh"
#include "SimIMFPMaxPhoton.hh"
#include "SimIMFPMoller.hh"
#include "SimIMFPPhoton.hh"
#include "SimITr1MFPElastic.hh"
#include "SimKNTables.hh"
#include "SimMaterialData.hh"
#include "SimMaxScatStrength.hh"
#include "SimMollerTables.hh"
#include "SimPhotonData.hh"
#include "SimSBTables.hh"
#include "SimStoppingPower.hh"
#include "Track.hh"
#include "TrackStack.hh"

namespace {
struct RefData {
  SimElectronData el;
  SimPhotonData ph;
  SimMaterialData mat;
};
}  // namespace

extern "C" {

void* ref_load(const char* dir) {
  RefData* d = new RefData();
  d->el.Load(dir, 0);
  d->ph.Load(dir, 0);
  d->mat.Load(dir, 0);
  return d;
}
void ref_free(void* h) { delete static_cast<RefData*>(h); }
void ref_seed(uint32_t s) { Random::generator.seed(s); }
double ref_uniform() { return Random::UniformRand(); }

// quantity codes as oracle_eval_table: 0 dedx, 1 itr1, 2 brem, 3 moller, 4 k1,
// 5 imfpMax, 6 total, 7 compton, 8 pair
void ref_eval_table(void* h, int q, int imat, const double* e, double* out, int n) {
  RefData* d = static_cast<RefData*>(h);
  for (int i = 0; i < n; ++i) {
    double v = 0;
    switch (q) {
      case 0: v = d->el.GetDEDX()->GetDEDXPerDensity(e[i], imat); break;
      case 1: v = d->el.GetITr1MFPElastic()->GetITr1MFPPerDensity(e[i], imat); break;
      case 2: v = d->el.GetIMFPBrem()->GetIMFPPerDensity(e[i], imat); break;
      case 3: v = d->el.GetIMFPMoller()->GetIMFPPerDensity(e[i]); break;
      case 4: v = d->el.GetMaxScatStrength()->GetMaxScatStrength(e[i]); break;
      case 5: v = d->ph.GetIMFPTotalMax()->GetIMFP(e[i]); break;
      case 6: v = d->ph.GetIMFPTotal()->GetIMFPPerDensity(e[i], imat); break;
      case 7: v = d->ph.GetIMFPCompton()->GetIMFPPerDensity(e[i], imat); break;
      case 8: v = d->ph.GetIMFPPairProd()->GetIMFPPerDensity(e[i], imat); break;
      default: break;
    }
    out[i] = v;
  }
}

// sampler codes: 0 KN eps, 1 Moller T', 2 SB k (imat), 3 GS mu; 3 uniforms per sample
void ref_eval_sampler(void* h, int s, int imat, const double* e, const double* r, double* out, int n) {
  RefData* d = static_cast<RefData*>(h);
  for (int i = 0; i < n; ++i) {
    const double* u = r + 3 * i;
    double v = 0;
    switch (s) {
      case 0: v = d->ph.GetTheKNTables()->SampleEnergyTransfer(e[i], u[0], u[1], u[2]); break;
      case 1: v = d->el.GetTheMollerTables()->SampleEnergyTransfer(e[i], u[0], u[1], u[2]); break;
      case 2: v = d->el.GetTheSBTables()->SampleEnergyTransfer(e[i], imat, u[0], u[1], u[2]); break;
      case 3: v = d->el.GetTheGSTables()->SampleAngularDeflection(e[i], u[0], u[1]); break;
      default: break;
    }
    out[i] = v;
  }
}

// Geom::DistanceToBoundary on n (r, v) pairs; r is updated in place (pushes)
void ref_distance(double lbox, int geomIndex, void* h, double* r, const double* v, int* ibox, double* s, int n) {
  RefData* d = static_cast<RefData*>(h);
  Geom g(lbox, &d->mat, geomIndex);
  for (int i = 0; i < n; ++i) {
    double vv[3] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
    s[i] = g.DistanceToBoundary(r + 3 * i, vv, ibox + 3 * i);
  }
}

void ref_simulate_cli(void* h, int n, double e, int isElectron, double lbox, int geomIndex, const char* fname) {
  RefData* d = static_cast<RefData*>(h);
  Simulate(n, e, isElectron != 0, lbox, d->mat, d->el, d->ph, geomIndex, fname);
}

int ref_simulate_full(void* h, int n, double e, int isElectron, double lbox, int geomIndex,
                      double* edep, double* steps, int cap) {
  RefData* d = static_cast<RefData*>(h);
  SimMaterialData& matData = d->mat;
  SimElectronData& elData = d->el;
  SimPhotonData& phData = d->ph;
  Geom geom(lbox, &matData, geomIndex);
  const double theElectronCut = matData.fElectronCut;
  const double theGammaCut = matData.fGammaCut;
  for (int ip = 0; ip < n; ++ip) {
    Track& p = TrackStack::Instance().Insert();
    p.fEkin = e;
    p.fType = isElectron ? -1 : 0;
    p.fDirection[0] = 0.0; p.fDirection[1] = 0.0; p.fDirection[2] = 1.0;
    p.fPosition[0] = 0.0;  p.fPosition[1] = 0.0;  p.fPosition[2] = -0.5 * lbox;
    Track track;
    while (-1 < TrackStack::Instance().PopIntoThisTrack(track)) {
      geom.DistanceToBoundary(track.fPosition, track.fDirection, track.fBoxIndx);
      int im = geom.GetMaterialIndex(track.fBoxIndx);
      if (im < 0) continue;
      track.fMatIndx = im;
      if (track.fType == 0) {
        KeepTrackingPhoton(phData, matData, geom, track);
        continue;
      }
      bool isMSCHinge = true;
      double theEkin0 = track.fEkin;
      double numTr1MFP = elData.GetMaxScatStrength()->GetMaxScatStrength(track.fEkin);
      double numTr1MFP0 = Random::UniformRand() * numTr1MFP;
      numTr1MFP -= numTr1MFP0;
      double numMollerMFP = -std::log(Random::UniformRand());
      double invMollerMFP = elData.GetIMFPMoller()->GetIMFPPerDensity(track.fEkin);
      double numBremMFP = -std::log(Random::UniformRand());
      while (track.fEkin > 0.0) {
        int what = KeepTrackingElectron(elData, matData, geom, track, numTr1MFP, numMollerMFP, invMollerMFP, numBremMFP);
        if (track.fMatIndx < 0) continue;
        switch (what) {
          case 1:
            if (track.fEkin > theGammaCut) PerformBrem(track, elData.GetTheSBTables());
            if (track.fEkin < theElectronCut) {
              geom.Score(track.fEkin, track.fBoxIndx[2]);
              track.fEkin = 0.0;
              if (track.fType == +1) PerformAnnihilation(track);
              break;
            }
            numBremMFP = -std::log(Random::UniformRand());
            break;
          case 2:
            if (track.fEkin > 2. * theElectronCut) PerformMoller(track, elData.GetTheMollerTables());
            numMollerMFP = -std::log(Random::UniformRand());
            invMollerMFP = elData.GetIMFPMoller()->GetIMFPPerDensity(track.fEkin);
            break;
          case 3:
            if (isMSCHinge) {
              PerformMSCAngularDeflection(track, theEkin0, elData.GetTheGSTables());
              numTr1MFP = numTr1MFP0;
              isMSCHinge = false;
            } else {
              theEkin0 = track.fEkin;
              numTr1MFP = elData.GetMaxScatStrength()->GetMaxScatStrength(theEkin0);
              numTr1MFP0 = Random::UniformRand() * numTr1MFP;
              numTr1MFP -= numTr1MFP0;
              isMSCHinge = true;
            }
            break;
          default:
            break;
        }
      }
    }
  }
  const int len = int(geom.fEdepHist.size());
  for (int i = 0; i < len && i < cap; ++i) {
    edep[i] = geom.fEdepHist[i];
    steps[i] = geom.fStepHist[i];
  }
  return len;
}

}  // extern "C"
