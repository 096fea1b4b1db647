// Device building blocks shared by the FP64 and FP32 transport kernels:
// counter-based random numbers, table interpolation and the rejection-free
// samplers, all templated on the arithmetic type R.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dpmx_internal.h"

namespace dpmx {

// ---------------------------------------------------------------------------
// math wrappers (float overloads map to the single-precision functions)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double mlog(double x) { return log(x); }
__device__ __forceinline__ float mlog(float x) { return __logf(x); }
__device__ __forceinline__ double mexp(double x) { return exp(x); }
__device__ __forceinline__ float mexp(float x) { return __expf(x); }
__device__ __forceinline__ double msqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float msqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ void msincos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void msincos(float x, float* s, float* c) { __sincosf(x, s, c); }
__device__ __forceinline__ double mfloor(double x) { return floor(x); }
__device__ __forceinline__ float mfloor(float x) { return floorf(x); }
template <class R> __device__ __forceinline__ R mmin(R a, R b) { return a < b ? a : b; }
template <class R> __device__ __forceinline__ R mmax(R a, R b) { return a > b ? a : b; }
template <class R> __device__ __forceinline__ R mabs(R a) { return a < R(0) ? -a : a; }

template <class R> struct Consts {
  static constexpr R kPI = R(3.1415926535897932);
  static constexpr R kEMC2 = R(0.510991);
};

// ---------------------------------------------------------------------------
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw; SC'11)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// Philox words to uniforms on the open interval (0,1).
// FP64: two words give 53 bits, the lowest forced to 1: (bits | 1) * 2^-53.
__device__ __forceinline__ double UniformF64(uint32_t lo, uint32_t hi) {
  const uint64_t bits = (uint64_t(hi) << 32) | lo;
  return double((bits >> 11) | 1ull) * (1.0 / 9007199254740992.0);
}
// FP32: one word, converted with rounding toward zero and scaled by 2^-32, so
// small uniforms keep all 32 bits of resolution (the smallest is 2^-32, and
// -ln U reaches 22.2 mean free paths) while the largest, 1 - 2^-24, stays
// below 1.
__device__ __forceinline__ float UniformF32(uint32_t x) {
  return __uint2float_rz(x | 1u) * 2.3283064365386963e-10f;
}

// One stream per history for the FP64 form: draw k of history h comes from
// Philox block k/2 at counter {k/2, 0, 0, h}; two 32-bit words make a 53-bit
// uniform on the open interval (0,1).
struct HistoryRng {
  uint32_t k0, k1, hist, block;
  uint4 w;
  int have;
  __device__ void Init(uint64_t seed, uint32_t h) {
    k0 = uint32_t(seed); k1 = uint32_t(seed >> 32); hist = h; block = 0; have = 0;
  }
  __device__ __forceinline__ double U() {
    if (have == 0) {
      w = philox(make_uint4(block++, 0u, 0u, hist), k0, k1);
      have = 2;
    }
    uint32_t lo, hi;
    if (have == 2) { lo = w.x; hi = w.y; } else { lo = w.z; hi = w.w; }
    --have;
    return UniformF64(lo, hi);
  }
};

// ---------------------------------------------------------------------------
// Table interpolation (reference loader semantics)
// ---------------------------------------------------------------------------
// SimDataSpline::GetValue (SimDataSpline.hh:38-50) behind the loaders' clamp
// and 1e-20 floor (e.g. SimStoppingPower.hh:43-49)
template <class R>
__device__ __forceinline__ R SplineAt(const R* p, int n, R logMin, R invLogDelta, R e) {
  int il = int((mlog(e) - logMin) * invLogDelta);
  il = il < 0 ? 0 : (il > n - 2 ? n - 2 : il);
  const R* q = p + 5 * il;
  const R xv = e - q[0];
  return q[1] + xv * (q[2] + xv * (q[3] + xv * q[4]));
}
template <class R>
__device__ __forceinline__ R SplineGet(const SplineT<R>& s, R e) {
  e = mmin(s.emaxm, mmax(s.emin, e));
  return mmax(R(1.0E-20), SplineAt(s.p, s.n, s.logMin, s.invLogDelta, e));
}
// SimDataLinear::GetValue (SimDataLinear.hh:38-45) behind the same clamp
__device__ __forceinline__ double LinearGet(const LinearT<double>& s, double e) {
  e = mmin(s.emaxm, mmax(s.emin, e));
  int il = int((e - s.xmin) * s.invDelta);
  il = il < 0 ? 0 : (il > s.n - 2 ? s.n - 2 : il);
  const double* q = s.p + 2 * il;
  return mmax(1.0E-20, (q[3] - q[1]) * (e - q[0]) / (q[2] - q[0]) + q[1]);
}
// FP32 form: values on the uniform grid x_i = xmin + i / invDelta; the
// position inside the interval comes from the grid, not from stored points
__device__ __forceinline__ float LinearGet(const LinearT<float>& s, float e) {
  e = mmin(s.emaxm, mmax(s.emin, e));
  const float t = (e - s.xmin) * s.invDelta;
  int il = int(t);
  il = il < 0 ? 0 : (il > s.n - 2 ? s.n - 2 : il);
  const float y0 = s.p[il], y1 = s.p[il + 1];
  return mmax(1.0E-20f, (y1 - y0) * (t - float(il)) + y0);
}

// ---------------------------------------------------------------------------
// Samplers
// ---------------------------------------------------------------------------
// SimLinAliasData::Sample (SimLinAliasData.cc:25-42)
template <class R>
__device__ __forceinline__ R LinAliasSample(const AliasEntry<R>* t, int n, R r1, R r2) {
  const R rest = r1 * R(n - 1);
  int il = int(rest);
  if (t[il].w < rest - R(il)) il = t[il].idx;
  const R xv = t[il].x;
  const R xd = t[il + 1].x - xv;
  const R y0 = t[il].y;
  if (y0 > R(0)) {
    const R dum = (t[il + 1].y - y0) / y0;
    if (mabs(dum) > R(0.1)) return xv - xd / dum * (R(1) - msqrt(R(1) + r2 * dum * (dum + R(2))));
    return xv + r2 * xd * (R(1) - R(0.5) * dum * (r2 - R(1)) * (R(1) + dum * r2));
  }
  return xv + xd * msqrt(r2);
}

// pick the lower or upper energy grid table with probability linear in ln E
template <class R>
__device__ __forceinline__ int EnergyBin(R logMin, R invLogDelta, R le, R r1, int numE) {
  R ph = (le - logMin) * invLogDelta;
  int ie = int(ph);
  ph -= R(ie);
  if (r1 < ph) ++ie;
  return ie < 0 ? 0 : (ie > numE - 1 ? numE - 1 : ie);
}

// SimKNTables.cc:69-90: reduced photon energy eps = E'/E of Compton scattering
template <class R>
__device__ __forceinline__ R SampleKN(const AliasSetT<R>& s, R eg, R r1, R r2, R r3) {
  const R le = mlog(eg);
  const int ie = EnergyBin(s.logMinE, s.invLogDeltaE, le, r1, s.numE);
  const R xi = LinAliasSample(s.p + size_t(ie) * s.numS, s.numS, r2, r3);
  const R kappa = eg / Consts<R>::kEMC2;
  return mexp(mlog(R(1) + R(2) * kappa) * (xi - R(1)));
}
// SimMollerTables.cc:69-89: kinetic energy of the delta electron
template <class R>
__device__ __forceinline__ R SampleMoller(const AliasSetT<R>& s, R ep, R r1, R r2, R r3) {
  const R le = mlog(ep);
  const int ie = EnergyBin(s.logMinE, s.invLogDeltaE, le, r1, s.numE);
  const R xi = LinAliasSample(s.p + size_t(ie) * s.numS, s.numS, r2, r3);
  return mexp(xi * (le - s.logMinE)) * R(0.5) * s.minE;
}
// SimSBTables.cc:93-114: bremsstrahlung photon energy
template <class R>
__device__ __forceinline__ R SampleSB(const AliasSetT<R>& s, R ep, R r1, R r2, R r3) {
  const R le = mlog(ep);
  const int ie = EnergyBin(s.logMinE, s.invLogDeltaE, le, r1, s.numE);
  const R xi = LinAliasSample(s.p + size_t(ie) * s.numS, s.numS, r2, r3);
  const R kc = s.minE / ep;
  return kc * mexp(-xi * (s.logMinE - le)) * ep;
}
// SimGSTables.cc:84-119: cosine of the MSC angular deflection
template <class R>
__device__ __forceinline__ R SampleGS(const GSSetT<R>& g, R ep, R r1, R r2) {
  const R le = mlog(ep);
  R ph = (le - g.logMinE) * g.invLogDeltaE;
  int ielow = int(ph);
  ielow = ielow < 0 ? 0 : (ielow > g.numE - 2 ? g.numE - 2 : ielow);
  int ie = ielow;
  ph -= R(ielow);
  if (r1 < ph) ++ie;
  const R dc = g.deltaCum;
  int il = int(r2 / dc);
  il = il > g.numS - 2 ? g.numS - 2 : il;
  const R resid = r2 - R(il) * dc;
  const R* q = g.uab + (size_t(ie) * g.numS + il) * 4;
  const R pa = q[1], pb = q[2], u0 = q[0], u1 = q[4];
  const R dum1 = (R(1) + pa + pb) * dc * resid;
  const R dum2 = dc * dc + pa * dc * resid + pb * resid * resid;
  const R u = u0 + dum1 / dum2 * (u1 - u0);
  const R a0 = g.a[ielow], a1 = g.a[ielow + 1];
  const R e0 = g.e[ielow], e1 = g.e[ielow + 1];
  const R a = (a1 - a0) / (e1 - e0) * (ep - e0) + a0;
  return R(1) - R(2) * a * u / (R(1) - u + a);
}

// FP32 form of the GS deflection: the same bin choices and ratin
// interpolation, carried out both for u and for w = 1 - u (the table keeps
// 1 - u, rounded from FP64, in each record's fourth slot). The transform
// mu = 1 - 2 a u / (1 - u + a) magnifies an error of u near u = 1 by ~2/a
// (a is ~1e-3 at high energies), so:
//  * the position in the ratin bin and its distance to the bin's upper edge,
//    r2 - il/(n-1) and (il+1)/(n-1) - r2, come from FMAs with the bin width
//    split into a float and its rest (an FP32 product il * dc alone is off by
//    ~3e-8, all of the distance near the bin's edge);
//  * the interpolation weight f and 1 - f = (s (dc - b r)) / dum2 are both
//    formed without cancellation, and u = u0 + f (u1 - u0),
//    w = w1 + (1 - f) (w0 - w1) add terms of one sign;
//  * mu comes from 1 - mu = 2 a u / (w + a) and 1 + mu = 2 w (1 + a) / (w + a),
//    and sin(theta) = sqrt((1 - mu)(1 + mu)) from those two.
__device__ __forceinline__ void SampleGSAngle(const GSSetT<float>& g, float ep, float r1, float r2, float& cost,
                                              float& sint) {
  const float le = mlog(ep);
  float ph = (le - g.logMinE) * g.invLogDeltaE;
  int ielow = int(ph);
  ielow = ielow < 0 ? 0 : (ielow > g.numE - 2 ? g.numE - 2 : ielow);
  int ie = ielow;
  ph -= float(ielow);
  if (r1 < ph) ++ie;
  const float dc = g.deltaCum, dcl = g.deltaCumLo;
  int il = int(r2 / dc);
  il = il > g.numS - 2 ? g.numS - 2 : il;
  const float fil = float(il), fil1 = float(il + 1);
  const float resid = fmaf(-fil, dc, r2) - fil * dcl;           // r2 - il / (n-1)
  const float rest = fmaxf(0.0f, fmaf(fil1, dc, -r2) + fil1 * dcl);   // (il+1) / (n-1) - r2
  const float4 q0 = reinterpret_cast<const float4*>(g.uab)[size_t(ie) * g.numS + il];
  const float4 q1 = reinterpret_cast<const float4*>(g.uab)[size_t(ie) * g.numS + il + 1];
  const float pa = q0.y, pb = q0.z;
  const float dum1 = (1.0f + pa + pb) * dc * resid;
  const float dum2 = dc * dc + pa * dc * resid + pb * resid * resid;
  const float idum2 = 1.0f / dum2;
  const float f = dum1 * idum2;
  const float fc = fmaxf(0.0f, rest * (dc - pb * resid) * idum2);   // 1 - f
  const float u = q0.x + f * (q1.x - q0.x);
  const float w = q1.w + fc * (q0.w - q1.w);
  const float a0 = g.a[ielow], a1 = g.a[ielow + 1];
  const float e0 = g.e[ielow], e1 = g.e[ielow + 1];
  const float a = (a1 - a0) / (e1 - e0) * (ep - e0) + a0;
  const float inv = 1.0f / (w + a);
  const float om = fmaxf(0.0f, 2.0f * a * u * inv);             // 1 - mu
  const float op = fmaxf(0.0f, 2.0f * w * (1.0f + a) * inv);    // 1 + mu
  cost = u < 0.5f ? 1.0f - om : op - 1.0f;
  cost = fmaxf(-1.0f, fminf(1.0f, cost));
  sint = fminf(1.0f, sqrtf(om * op));
}
template <>
__device__ __forceinline__ float SampleGS<float>(const GSSetT<float>& g, float ep, float r1, float r2) {
  float c, s;
  SampleGSAngle(g, ep, r1, r2, c, s);
  return c;
}

// SimDPMLike.cc:638-652: rotate (u,v,w) from the frame of (u1,u2,u3) to the lab
template <class R>
__device__ __forceinline__ void RotateToLab(R& u, R& v, R& w, R u1, R u2, R u3) {
  R up = u1 * u1 + u2 * u2;
  if (up > R(0)) {
    up = msqrt(up);
    const R px = u, py = v, pz = w;
    u = (u1 * u3 * px - u2 * py) / up + u1 * pz;
    v = (u2 * u3 * px + u1 * py) / up + u2 * pz;
    w = -up * px + u3 * pz;
  } else if (u3 < R(0)) {
    u = -u;
    w = -w;
  }
}

}  // namespace dpmx
