// Device-side types and physics building blocks shared by the transport kernels.
//
// The formulas restate the reference's frame algebra and Stokes / Jones updates
// (MonteCarloRadiativeTransfer.jl src/utils.jl) in forms that are mathematically equal
// but better conditioned in FP32:
//   * sin(theta) of a unit vector is taken from its transverse part sqrt(x^2 + y^2)
//     instead of sqrt(1 - z^2) (src/utils.jl:17, :56);
//   * the Rayleigh cube-root sampler uses cbrt(b - |r|) = 1 / cbrt(b + |r|)
//     (src/scatterers/rayleigh.jl:11);
//   * the RT peel-off's rotation into the ray frame of the incoming direction is
//     written with the azimuth difference of bin and ray (src/utils.jl:91-112).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mcrt {

constexpr int MAX_LAYERS = 8;
constexpr int MAX_SCAT = 4;
constexpr double PI_D = 3.14159265358979323846;
constexpr double LOG2E_D = 1.4426950408889634074;
// |k_z| > 1 - eps(Float64) of get_basis (src/utils.jl:53) expressed through the
// transverse part of a unit vector: 1 - |z| ~ s^2 / 2.
constexpr double POLE_S2 = 3.3e-16;

// Accumulator slots kept per thread and per instance (all FP64 raw sums).
enum Acc {
  ACC_ADT = 0, ACC_AABS, ACC_AREF, ACC_ATRANS, ACC_AREM,
  ACC_PEAK, ACC_PEAK2, ACC_PHOTONS, ACC_EVENTS, ACC_ATTEMPTS,
  ACC_RT, ACC_CB1, ACC_CBN, ACC_KEPLER_CAP, ACC_REJECT_CAP, ACC_NONFINITE,
  NACC
};

// ------------------------------------------------------------------ device views
struct DevScatterer {
  int kind;        // 0 Rayleigh, 1 Mie
  int ntheta;      // Mie table length (the device tables carry one zero pad entry)
  int rp;          // Mie random_points
  float scalef;    // (ntheta - 1) / pi, the table index per radian, in each precision
  double kl;
  const float4* F; // (F11, F12, F33, F34) per angle, ntheta + 1
  const float4* S; // (S11re, S11im, S22re, S22im) per angle, ntheta + 1
  const float* csrn; // rp + 1 (+1 pad)
  double scaled;
  double pad;
};

template <typename T>
__host__ __device__ __forceinline__ T table_scale(const DevScatterer& s);
template <>
__host__ __device__ __forceinline__ float table_scale<float>(const DevScatterer& s) { return s.scalef; }
template <>
__host__ __device__ __forceinline__ double table_scale<double>(const DevScatterer& s) { return s.scaled; }

struct DevLayer {
  double tau, omega;
  int inf, scat;
};

// One simulate() instance as seen by the kernels. Plain data, copied into shared
// memory by the block that works on it.
struct __align__(16) DevInstance {
  int geom;  // 0 plane, 1 sphere
  int n_layers;
  int n_scat;
  int compute_cb;
  DevLayer layers[MAX_LAYERS];
  DevScatterer scat[MAX_SCAT];
  double k0[3];
  double inc[4];   // (cos, sin) of the incidence theta and phi (src/gpu.jl:50-52)
  double I0[4];
  double Ei[4];    // E_from_I(I0): E1 (re, im), E2 (re, im)
  double kfs[4];   // spherical frame of -k0
  double kf0[3];   // backscatter direction ray_to_norm(e_z, kfs)
  double eh0[2];   // get_basis(kf0).Eh (x, y)
  double Rkfs[9];  // norm_to_ray matrix of the frame kfs (row major)
  double kl1;      // mean free path of layer 1's scatterer (CB phase scale)
  double min_int, tau0;
  long long max_scat;
  long long n_photons;     // photons of this instance in this launch
  long long photon_begin;  // first photon index (Philox counter)
  long long nrays;         // number_of_rays (stratified test mode)
  long long max_attempts;  // cap of every rejection loop (a loop reaching it sets MCRT_FLAG_REJECT_LIMIT)
  unsigned key0, key1;
  int rng_mode;
  int rt_fourier;          // plane with Rayleigh scatterers only: RT bins by azimuthal Fourier modes
  const void* bins;        // BinTables<T> in device memory
  double* Irt;
  double* Icb;
  double* ladder;
  double* acc;             // NACC raw sums
  double* Frt;             // Fourier RT coefficients [ntheta][4 Stokes][5 modes] (rt_fourier)
  unsigned long long* claim;  // [0] photons claimed, [1] photons finished by blocks, this launch
};
static_assert(sizeof(DevInstance) % 16 == 0, "DevInstance is copied as 16-byte words");

template <typename T>
struct BinTables {
  int ntheta, nphi, nthetab, nphib;
  int up0, up1, lo0, lo1;
  // RT, per theta index: sin, cos, log2(e)/|cos|, inorm; per phi index: cos, sin.
  const T *st, *ct, *g, *w, *cp, *sp;
  // CB, per bin b = j2 * nthetab + j1.
  const T *kfx, *kfy, *kfz, *ehx, *ehy, *gb, *cf2, *sf2, *c1, *c2, *c3;
  const int* upb;
  // CB grid itself: per theta_b index sin, cos; per phi_b index cos, sin.
  const T *stb, *ctb, *cpb, *spb;
  // RT polar bins in pairs for the packed FP32 tiles, read per event through L1 rather
  // than held in registers: per pair {st0, st1, ct0, ct1}, {g0, g1, w0, w1}. The upper
  // then the lower hemisphere, each padded with zero-weight pairs to a multiple of
  // RTP_PAD pairs, then RTP_PAD zero-weight pairs for lanes without bins.
  const float4* rtp;
  int rtp_lo;    // first pair of the lower hemisphere
  int rtp_zero;  // first of the trailing zero-weight pairs
};
constexpr int RTP_PAD = 4;  // a multiple of every tile's pairs per lane (2 or 4)

// ------------------------------------------------------------------ Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11.
struct U4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

__host__ __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// Uniform (0,1) from 32 bits: (x + 0.5) * 2^-32; the complement 1 - u is exact as ~x.
template <typename T>
__device__ __forceinline__ T u01(uint32_t x);
template <>
__device__ __forceinline__ float u01<float>(uint32_t x) {
  return __fmaf_rn((float)(x >> 8), 5.9604644775390625e-08f, 2.98023223876953125e-08f);
}
template <>
__device__ __forceinline__ double u01<double>(uint32_t x) {
  return ((double)x + 0.5) * 2.3283064365386962890625e-10;
}

// The three draws of one rejection attempt, in the reference's call order.
struct Draw {
  uint32_t r[4];
};
__device__ __forceinline__ Draw draw(unsigned k0, unsigned k1, unsigned long long photon,
                                     uint32_t event, uint32_t attempt) {
  U4 o = philox4x32_10(U4{(uint32_t)photon, (uint32_t)(photon >> 32), event, attempt}, k0, k1);
  return Draw{{o.x, o.y, o.z, o.w}};
}

// ------------------------------------------------------------------ math traits
template <typename T>
struct MT;
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// arccos from Hastings' approximation, Abramowitz & Stegun (1964) formula 4.4.46:
// acos(x) = sqrt(1 - x) (a0 + a1 x + ... + a7 x^7) + e(x), |e| <= 2e-8 for 0 <= x <= 1,
// and acos(-x) = pi - acos(x).
__device__ __forceinline__ float acos_as4446(float x) {
  const float ax = fabsf(x);
  float p = -0.0012624911f;
  p = p * ax + 0.0066700901f;
  p = p * ax - 0.0170881256f;
  p = p * ax + 0.0308918810f;
  p = p * ax - 0.0501743046f;
  p = p * ax + 0.0889789874f;
  p = p * ax - 0.2145988016f;
  p = p * ax + 1.5707963050f;
  const float y = fmaxf(1.0f - ax, 0.0f);
  const float r = y > 0.0f ? y * rsqrt_approx(y) * p : 0.0f;
  return x < 0.0f ? 3.14159265358979f - r : r;
}

// FP32 transport uses the hardware approximations (MUFU) in the hot loops; their
// errors (about 2^-22 relative for rsqrt and exp2, 2^-20.5 absolute for sin and cos on
// [-pi, pi]) sit far below the 1e-4 agreement required of FP32 against FP64.
template <>
struct MT<float> {
  static __device__ __forceinline__ float rsqrt(float x) { return rsqrt_approx(x); }
  static __device__ __forceinline__ float sqrt(float x) { return sqrtf(x); }
  static __device__ __forceinline__ float exp2n(float x) {  // exp2(-x)
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(-x));
    return r;
  }
  static __device__ __forceinline__ float log(float x) { return logf(x); }
  static __device__ __forceinline__ float exp(float x) { return expf(x); }
  static __device__ __forceinline__ float acos(float x) { return acos_as4446(x); }
  static __device__ __forceinline__ float cbrt(float x) { return cbrtf(x); }
  static __device__ __forceinline__ void sincos(float x, float* s, float* c) { sincosf(x, s, c); }
  // sin and cos of 2 pi t for a phase t in turns with |t| <= 1/2
  static __device__ __forceinline__ void sincos_turns(float t, float* s, float* c) {
    __sincosf(6.28318530717958647692f * t, s, c);
  }
  static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
  static __device__ __forceinline__ float rint(float x) { return rintf(x); }
  static __device__ __forceinline__ float floor(float x) { return floorf(x); }
  static __device__ __forceinline__ float fabs(float x) { return fabsf(x); }
  static __device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }
  // Natural log of a positive FP32 norm, accumulated into an FP64 log scale: the MUFU
  // log2 (relative error about 2^-22) instead of an FP64 log on the FP64 pipe.
  static __device__ __forceinline__ double logscale(float x) { return (double)(__log2f(x) * 0.693147180559945309f); }
  // exp of an FP64 log-scale difference, returned in FP32 (underflows to 0 as the cast would).
  static __device__ __forceinline__ float expscale(double d) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"((float)(d * 1.4426950408889634)));
    return r;
  }
  static constexpr float KEPLER_TOL = 4e-6f;
  static constexpr int KEPLER_CAP = 32;
};
template <>
struct MT<double> {
  static __device__ __forceinline__ double rsqrt(double x) { return ::rsqrt(x); }
  static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
  static __device__ __forceinline__ double exp2n(double x) { return ::exp2(-x); }
  static __device__ __forceinline__ double log(double x) { return ::log(x); }
  static __device__ __forceinline__ double exp(double x) { return ::exp(x); }
  static __device__ __forceinline__ double logscale(double x) { return ::log(x); }
  static __device__ __forceinline__ double expscale(double d) { return ::exp(d); }
  static __device__ __forceinline__ double acos(double x) { return ::acos(x); }
  static __device__ __forceinline__ double cbrt(double x) { return ::cbrt(x); }
  static __device__ __forceinline__ void sincos(double x, double* s, double* c) { ::sincos(x, s, c); }
  static __device__ __forceinline__ void sincospi(double x, double* s, double* c) {
    ::sincospi(x, s, c);
  }
  static __device__ __forceinline__ void sincos_turns(double t, double* s, double* c) {
    ::sincospi(2.0 * t, s, c);
  }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ double rint(double x) { return ::rint(x); }
  static __device__ __forceinline__ double floor(double x) { return ::floor(x); }
  static __device__ __forceinline__ double fabs(double x) { return ::fabs(x); }
  static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
  static constexpr double KEPLER_TOL = 1e-12;
  static constexpr int KEPLER_CAP = 100;
};

template <typename T>
__device__ __forceinline__ T clamp1(T c) {
  return c > T(1) ? T(1) : (c < T(-1) ? T(-1) : c);
}

// ------------------------------------------------------------------ frames
template <typename T>
struct Frame {
  T ct, st, cp, sp;
};

// spherical_from_cartesian (src/utils.jl:9-23), pole branch at s^2 < 1e-24.
template <typename T>
__device__ __forceinline__ Frame<T> spherical(T x, T y, T z) {
  T s2 = x * x + y * y;
  Frame<T> f;
  if (s2 < T(1e-24)) {
    f.ct = z > T(0) ? T(1) : (z < T(0) ? T(-1) : T(0));
    f.st = T(0);
    f.cp = T(1);
    f.sp = T(0);
  } else {
    T r = MT<T>::rsqrt(s2);
    f.ct = z;
    f.st = s2 * r;
    f.cp = x * r;
    f.sp = y * r;
  }
  return f;
}

// ray_to_norm (src/utils.jl:30-34)
template <typename T>
__device__ __forceinline__ void ray_to_norm(const Frame<T>& f, T x, T y, T z, T& ox, T& oy, T& oz) {
  ox = x * f.ct * f.cp - y * f.sp + z * f.st * f.cp;
  oy = x * f.ct * f.sp + y * f.cp + z * f.st * f.sp;
  oz = -x * f.st + z * f.ct;
}

// norm_to_ray (src/utils.jl:41-45)
template <typename T>
__device__ __forceinline__ void norm_to_ray(const Frame<T>& f, T x, T y, T z, T& ox, T& oy, T& oz) {
  ox = x * f.ct * f.cp + y * f.ct * f.sp - z * f.st;
  oy = -x * f.sp + y * f.cp;
  oz = x * f.st * f.cp + y * f.st * f.sp + z * f.ct;
}

// get_basis(k).Eh (src/utils.jl:52-62), x and y components (z is 0).
template <typename T>
__device__ __forceinline__ void basis_h(T kx, T ky, T& ehx, T& ehy) {
  T s2 = kx * kx + ky * ky;
  if (s2 < T(POLE_S2)) {
    ehx = T(0);
    ehy = T(-1);
  } else {
    T r = MT<T>::rsqrt(s2);
    ehx = ky * r;
    ehy = -kx * r;
  }
}

// ------------------------------------------------------------------ scatterers
template <typename T>
struct PMat {
  T p11, p12, p33, p34;
};

// phase_matrix evaluated at a given cosine (src/scatterers/rayleigh.jl:13-16,
// src/scatterers/mie.jl:53-71); Mie reads the padded FP32 table F.
template <typename T>
__device__ __forceinline__ PMat<T> phase_eval(int kind, const float4* F, int ntheta, T scale, T mu) {
  if (kind == 0) {
    T m2 = mu * mu;
    return PMat<T>{T(0.75) + T(0.75) * m2, T(-0.75) + T(0.75) * m2, T(1.5) * mu, T(0)};
  }
  T th = MT<T>::acos(clamp1(mu));
  T sn = th * scale;
  int i0 = (int)sn;
  i0 = i0 > ntheta - 1 ? ntheta - 1 : i0;
  T f = sn - (T)i0;
  f = f > T(1) ? T(1) : f;
  float4 a = F[i0], b = F[i0 + 1];
  T w0 = T(1) - f;
  return PMat<T>{w0 * (T)a.x + f * (T)b.x, w0 * (T)a.y + f * (T)b.y, w0 * (T)a.z + f * (T)b.z,
                 w0 * (T)a.w + f * (T)b.w};
}

// amplitude_matrix diagonal (src/scatterers/rayleigh.jl:20-23, src/scatterers/mie.jl:76-92,
// keeping the reference's (2 - f, f - 1) interpolation weights of mie.jl:80-85).
template <typename T>
__device__ __forceinline__ void amp_eval(int kind, const float4* S, int ntheta, T scale, T mu, T& s1r,
                                         T& s1i, T& s2r, T& s2i) {
  if (kind == 0) {
    s1r = T(0);
    s1i = T(1);
    s2r = T(0);
    s2i = mu;
    return;
  }
  T th = MT<T>::acos(clamp1(mu));
  T sn = th * scale;
  int i0 = (int)sn;
  i0 = i0 > ntheta - 1 ? ntheta - 1 : i0;
  T f = sn - (T)i0;
  f = f > T(1) ? T(1) : f;
  float4 a = S[i0], b = S[i0 + 1];
  T w0 = T(2) - f, w1 = f - T(1);
  s1r = w0 * (T)a.x + w1 * (T)b.x;
  s1i = w0 * (T)a.y + w1 * (T)b.y;
  s2r = w0 * (T)a.z + w1 * (T)b.z;
  s2i = w0 * (T)a.w + w1 * (T)b.w;
}

// Sampled cos(theta): Rayleigh closed form (rayleigh.jl:10-11) or Mie inverse CDF
// (mie.jl:47-51).
template <typename T>
__device__ __forceinline__ T sample_mu(int kind, const float* csrn, int rp, T u) {
  if (kind == 0) {
    T rn = T(2) * (T(1) - T(2) * u);
    T b = MT<T>::sqrt(T(1) + rn * rn);
    T p = MT<T>::cbrt(b + MT<T>::fabs(rn));
    T c = p - T(1) / p;
    return rn < T(0) ? -c : c;
  }
  T rn = u * (T)rp;
  int m = (int)rn;
  m = m > rp - 1 ? rp - 1 : m;
  T f = rn - (T)m;
  return (T(1) - f) * (T)csrn[m] + f * (T)csrn[m + 1];
}

// Stokes rotation (src/utils.jl:82-84)
template <typename T>
__device__ __forceinline__ void rotate(T c2, T s2, T& q, T& u) {
  T nq = c2 * q + s2 * u;
  T nu = -s2 * q + c2 * u;
  q = nq;
  u = nu;
}

// kepler_solver (src/utils.jl:243-261) with an iteration cap.
template <typename T>
__device__ __forceinline__ T kepler(T M, T e, int& capped) {
  const T TWO_PI = (T)(2 * PI_D);
  T MM = M - MT<T>::floor(M / TWO_PI) * TWO_PI;
  T s, c;
  MT<T>::sincos(MM, &s, &c);
  T ea = M + T(0.85) * e * (s > T(0) ? T(1) : (s < T(0) ? T(-1) : T(0)));
  T dea = T(1);
  int it = 0;
  while (MT<T>::fabs(dea) > MT<T>::KEPLER_TOL) {
    if (++it > MT<T>::KEPLER_CAP) {
      capped = 1;
      break;
    }
    T se, ce;
    MT<T>::sincos(ea, &se, &ce);
    T f3 = e * ce, f2 = e * se, f1 = T(1) - f3;
    T f = ea - f2 - M;
    dea = -f / f1;
    dea = -f / (f1 + f2 * dea / T(2));
    dea = -f / (f1 + f2 * dea / T(2) + f3 * dea * dea / T(6));
    ea += dea;
  }
  return ea;
}

// The rotation angle pair (cos psi, sin psi) of update_I / update_E for an outgoing
// direction whose ray-frame spherical angles are ks, in the frame f, with basis Eh of
// the outgoing direction. sign = -1 for update_I (src/utils.jl:105), +1 for update_E
// (src/utils.jl:183).
template <typename T>
__device__ __forceinline__ void psi_angles(const Frame<T>& f, const Frame<T>& ks, T ehx, T ehy,
                                           T sign, T& cpsi, T& spsi) {
  T hx = ks.sp * f.ct * f.cp + ks.cp * f.sp;
  T hy = ks.sp * f.ct * f.sp - ks.cp * f.cp;
  T vx = ks.ct * ks.cp * f.ct * f.cp - ks.ct * ks.sp * f.sp - ks.st * f.st * f.cp;
  T vy = ks.ct * ks.cp * f.ct * f.sp + ks.ct * ks.sp * f.cp - ks.st * f.st * f.sp;
  cpsi = ehx * hx + ehy * hy;
  spsi = sign * (ehx * vx + ehy * vy);
}

// update_I (src/utils.jl:91-112) for a general outgoing direction k with basis Eh.
template <typename T>
__device__ __forceinline__ void update_I(const Frame<T>& f, const T I[4], T kx, T ky, T kz, T ehx,
                                         T ehy, int kind, const float4* F, int ntheta, T scale,
                                         T out[4]) {
  T rx, ry, rz;
  norm_to_ray(f, kx, ky, kz, rx, ry, rz);
  Frame<T> ks = spherical(rx, ry, rz);
  T cpsi, spsi;
  psi_angles(f, ks, ehx, ehy, T(-1), cpsi, spsi);
  PMat<T> P = phase_eval<T>(kind, F, ntheta, scale, rz);
  T q = I[1], u = I[2];
  rotate(ks.cp * ks.cp - ks.sp * ks.sp, T(-2) * ks.sp * ks.cp, q, u);
  out[0] = P.p11 * I[0] + P.p12 * q;
  out[1] = P.p12 * I[0] + P.p11 * q;
  out[2] = P.p33 * u + P.p34 * I[3];
  out[3] = -P.p34 * u + P.p33 * I[3];
  rotate(cpsi * cpsi - spsi * spsi, T(2) * spsi * cpsi, out[1], out[2]);
}

// update_E (src/utils.jl:170-192) on E = (E1re, E1im, E2re, E2im), in place.
template <typename T>
__device__ __forceinline__ void update_E(const Frame<T>& f, T E[4], T kx, T ky, T kz, T ehx, T ehy,
                                         int kind, const float4* S, int ntheta, T scale) {
  T rx, ry, rz;
  norm_to_ray(f, kx, ky, kz, rx, ry, rz);
  Frame<T> ks = spherical(rx, ry, rz);
  T cpsi, spsi;
  psi_angles(f, ks, ehx, ehy, T(1), cpsi, spsi);
  T s1r, s1i, s2r, s2i;
  amp_eval<T>(kind, S, ntheta, scale, rz, s1r, s1i, s2r, s2i);
  T ar = E[0] * ks.cp + E[2] * ks.sp, ai = E[1] * ks.cp + E[3] * ks.sp;
  T br = -E[0] * ks.sp + E[2] * ks.cp, bi = -E[1] * ks.sp + E[3] * ks.cp;
  T sar = s1r * ar - s1i * ai, sai = s1r * ai + s1i * ar;
  T sbr = s2r * br - s2i * bi, sbi = s2r * bi + s2i * br;
  E[0] = sar * cpsi + sbr * spsi;
  E[1] = sai * cpsi + sbi * spsi;
  E[2] = -sar * spsi + sbr * cpsi;
  E[3] = -sai * spsi + sbi * cpsi;
}

// 2x2 complex matrix of update_E(., k, f): M = R(psi) diag(S11, S22) R(phi_k).
// Stored as m[8] = (m11r, m11i, m12r, m12i, m21r, m21i, m22r, m22i).
template <typename T>
__device__ __forceinline__ void update_E_matrix(const Frame<T>& f, T kx, T ky, T kz, int kind,
                                                const float4* S, int ntheta, T scale, T m[8]) {
  T ehx, ehy;
  basis_h(kx, ky, ehx, ehy);
  T rx, ry, rz;
  norm_to_ray(f, kx, ky, kz, rx, ry, rz);
  Frame<T> ks = spherical(rx, ry, rz);
  T cpsi, spsi;
  psi_angles(f, ks, ehx, ehy, T(1), cpsi, spsi);
  T s1r, s1i, s2r, s2i;
  amp_eval<T>(kind, S, ntheta, scale, rz, s1r, s1i, s2r, s2i);
  T c = ks.cp, s = ks.sp;
  // M11 = cpsi S11 c - spsi S22 s ; M12 = cpsi S11 s + spsi S22 c
  // M21 = -spsi S11 c - cpsi S22 s ; M22 = -spsi S11 s + cpsi S22 c
  m[0] = cpsi * c * s1r - spsi * s * s2r;
  m[1] = cpsi * c * s1i - spsi * s * s2i;
  m[2] = cpsi * s * s1r + spsi * c * s2r;
  m[3] = cpsi * s * s1i + spsi * c * s2i;
  m[4] = -spsi * c * s1r - cpsi * s * s2r;
  m[5] = -spsi * c * s1i - cpsi * s * s2i;
  m[6] = -spsi * s * s1r + cpsi * c * s2r;
  m[7] = -spsi * s * s1i + cpsi * c * s2i;
}

template <typename T>
__device__ __forceinline__ void cmul(T ar, T ai, T br, T bi, T& cr, T& ci) {
  cr = ar * br - ai * bi;
  ci = ar * bi + ai * br;
}

// C = A * B for 2x2 complex matrices in the m[8] layout.
template <typename T>
__device__ __forceinline__ void mat2_mul(const T A[8], const T B[8], T C[8]) {
  T r[8];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      T xr, xi, yr, yi;
      cmul(A[(2 * i + 0) * 2], A[(2 * i + 0) * 2 + 1], B[(0 * 2 + j) * 2], B[(0 * 2 + j) * 2 + 1], xr,
           xi);
      cmul(A[(2 * i + 1) * 2], A[(2 * i + 1) * 2 + 1], B[(1 * 2 + j) * 2], B[(1 * 2 + j) * 2 + 1], yr,
           yi);
      r[(2 * i + j) * 2] = xr + yr;
      r[(2 * i + j) * 2 + 1] = xi + yi;
    }
#pragma unroll
  for (int k = 0; k < 8; ++k) C[k] = r[k];
}

// y = M x for a 2-vector of complex numbers x = (x1r, x1i, x2r, x2i).
template <typename T>
__device__ __forceinline__ void mat2_vec(const T M[8], const T x[4], T y[4]) {
  T ar, ai, br, bi;
  cmul(M[0], M[1], x[0], x[1], ar, ai);
  cmul(M[2], M[3], x[2], x[3], br, bi);
  T y0 = ar + br, y1 = ai + bi;
  cmul(M[4], M[5], x[0], x[1], ar, ai);
  cmul(M[6], M[7], x[2], x[3], br, bi);
  y[0] = y0;
  y[1] = y1;
  y[2] = ar + br;
  y[3] = ai + bi;
}

// ------------------------------------------------------------------ geometry (FP64)
// distance_to_boundary (src/geometries/plane.jl:97-105, sphere.jl:69-73)
__device__ __forceinline__ double dist_d(const DevInstance& in, const double x[3], double kx, double ky,
                                         double kz, int idx) {
  if (in.geom == 0) {
    if (kz > 0) return -x[2] / kz;
    if (!in.layers[idx].inf) return (x[2] + in.layers[idx].tau) / -kz;
    return INFINITY;
  }
  double kxv = kx * x[0] + ky * x[1] + kz * x[2];
  double xx = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  double tau = in.layers[0].tau;
  double D = tau * tau - xx;
  D = D > 0 ? D : 0;
  return -kxv + sqrt(kxv * kxv + D);
}

}  // namespace mcrt
