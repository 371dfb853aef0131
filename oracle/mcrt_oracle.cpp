// CPU oracle for the polarised Monte Carlo transport with coherent backscattering.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in FP64 C++, the reference's CPU path
// (MonteCarloRadiativeTransfer.jl: src/cpu.jl, src/utils.jl, src/geometries/plane.jl,
// src/geometries/sphere.jl, src/scatterers/rayleigh.jl, src/scatterers/mie.jl) so that
// the CUDA library can be checked against it. Only tests/, __graft_entry__.smoke() and
// bench.py (CPU baseline and the reference arm) load it; the library never does.
//
// Parity status: UNPINNED by the reference itself. The reference ships no golden
// vectors (test/runtests.jl:1-6 is an empty testset) and Julia is not installed, so
// the reference cannot be run here. The restatement is instead pinned by known-answer
// tests derived from the reference's semantics: published Philox4x32-10 vectors,
// exact per-photon energy closure, the analytic single-scattering slab reflection,
// the Rayleigh sampler's density, an independent Mie evaluation, agreement of the
// reference's O(n) reciprocal-path walk with the incremental form, reciprocity of the
// slab reflection function at the 3-sigma level, agreement at all scattering orders
// with an independently written analog polarised Monte Carlo on Rayleigh slabs and on a
// slab of absorbing Mie spheres, and agreement at all orders with an exact vector
// adding-doubling solution (tests/doubling.py): every RT bin's full Stokes vector for
// four incident polarisation states, and the CB ladder, CB intensity and enhancement
// factor at exact backscatter, where reciprocity fixes the interference term; and for the
// sphere, agreement at first order with an exact geometric integral (every RT bin, and
// the CB bins near backscatter); and the CB cone at second order for Rayleigh scatterers,
// exactly twice the ladder at exact backscatter and equal to an exact integral off it.
//
// Random numbers: the reference calls an unseeded rand(). Here every draw comes from
// Philox4x32-10 keyed by (seed, instance) with counter (photon, event, attempt), and
// the draws of one rejection attempt are consumed in the reference's call order:
//   u0 -> phase_matrix sampling (rayleigh.jl:10 / mie.jl:48),
//   u1 -> azimuth (utils.jl:309 or :313),
//   u2 -> free path (cpu.jl:199).
// Event 0 holds the start-up draws: u0,u1 for the sphere entry point (sphere.jl:43-46)
// and u2 of attempt a for the a-th initial-propagation draw (plane.jl:88-94,
// sphere.jl:56-63).
//
// Deliberate, documented deviations (all affect only measure-zero or NaN cases):
//   * cosines that round outside [-1, 1] are clamped before acos / sqrt(1 - c^2)
//     (the reference would throw a DomainError or produce NaN there);
//   * a rotated cosine that rounds below -1 is clamped instead of being read as the
//     "sample a new angle" sentinel of phase_matrix (rayleigh.jl:9, mie.jl:47);
//   * the unbounded loops (rejection loop cpu.jl:194-235, kepler_solver utils.jl:249)
//     are capped; hitting a cap is counted and reported;
//   * the reciprocal-path amplitude scale raa = sqrt(Iaf / |Eaf|^2) (gpu.jl:84,
//     cpu.jl:77) is taken as zero where the rounded backscattered intensity is negative
//     or the field vanishes (a fully polarised photon scattered at 90 degrees by
//     Rayleigh scatterers), where the reference's sqrt throws a DomainError.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double PI = 3.14159265358979323846;
constexpr double EPS = 2.220446049250313e-16;  // Julia eps(Float64)
constexpr long MAX_ATTEMPTS = 1000000;
constexpr int MAX_KEPLER = 100;  // same cap as the FP64 kernels

// The per-bin arithmetic (frames, update_I, update_E, the bin bodies) is templated on
// the scalar type R. The oracle instantiates it with double; opcount.cpp instantiates
// it with an operation-counting type to fix the algorithmic flops per bin evaluation.
// Elementary functions are called unqualified, so the counting type supplies its own.
inline double Sqrt(double x) { return std::sqrt(x); }
inline double Exp(double x) { return std::exp(x); }
inline double Log(double x) { return std::log(x); }
inline double Cos(double x) { return std::cos(x); }
inline double Sin(double x) { return std::sin(x); }
inline double Acos(double x) { return std::acos(x); }
inline double Cbrt(double x) { return std::cbrt(x); }
inline double Fabs(double x) { return std::fabs(x); }
inline double Max(double a, double b) { return std::max(a, b); }
inline long Trunc(double x) { return (long)std::trunc(x); }

template <class R>
struct V3T {
  R x, y, z;
};
template <class R>
inline V3T<R> operator+(V3T<R> a, V3T<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R>
inline V3T<R> operator-(V3T<R> a, V3T<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R>
inline V3T<R> operator-(V3T<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R>
inline V3T<R> operator*(R s, V3T<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R>
inline R dot(V3T<R> a, V3T<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R>
inline R norm3(V3T<R> a) { return Sqrt(dot(a, a)); }

template <class R>
struct V4T {
  R v[4];
};
template <class R>
inline V4T<R> scale4(V4T<R> a, R s) { return {{a.v[0] * s, a.v[1] * s, a.v[2] * s, a.v[3] * s}}; }

template <class R>
struct SphT {
  R ct, st, cp, sp;
};

using V3 = V3T<double>;
using V4 = V4T<double>;
using Sph = SphT<double>;
using cplx = std::complex<double>;

template <class R>
inline R jsign(R x) { return x > 0 ? R(1.0) : (x < 0 ? R(-1.0) : R(0.0)); }
template <class R>
inline R clamp1(R c) { return c > 1.0 ? R(1.0) : (c < -1.0 ? R(-1.0) : c); }

// ---------------------------------------------------------------- Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11.
inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

struct Draws {
  double u[4];
};

struct Rng {
  uint32_t key[2];
  int mode;          // 0: Philox everywhere; 1: stratified first-collision depth
  int64_t n_total;   // photons in the run (stratified mode)
  Draws at(uint64_t photon, uint32_t event, uint32_t attempt) const {
    uint32_t ctr[4] = {(uint32_t)photon, (uint32_t)(photon >> 32), event, attempt};
    uint32_t o[4];
    philox4x32_10(ctr, key, o);
    Draws d;
    for (int i = 0; i < 4; ++i) d.u[i] = ((double)o[i] + 0.5) * 2.3283064365386962890625e-10;
    if (mode == 1 && event == 0 && attempt == 0) d.u[2] = ((double)photon + 0.5) / (double)n_total;
    return d;
  }
};

// ---------------------------------------------------------------- frame algebra
// utils.jl:9-23
template <class R>
inline SphT<R> spherical_from_cartesian(V3T<R> x) {
  R s2 = x.x * x.x + x.y * x.y;
  if (s2 < 1e-24) return {jsign(x.z), R(0.0), R(1.0), R(0.0)};
  R ct = clamp1(x.z);
  R st = Sqrt(R(1.0) - ct * ct);
  R si = R(1.0) / Sqrt(s2);
  return {ct, st, x.x * si, x.y * si};
}

// utils.jl:30-34
template <class R>
inline V3T<R> ray_to_norm(V3T<R> x, R ct, R st, R cp, R sp) {
  return {x.x * ct * cp - x.y * sp + x.z * st * cp, x.x * ct * sp + x.y * cp + x.z * st * sp,
          -x.x * st + x.z * ct};
}
template <class R>
inline V3T<R> ray_to_norm(V3T<R> x, const SphT<R>& s) { return ray_to_norm(x, s.ct, s.st, s.cp, s.sp); }

// utils.jl:41-45
template <class R>
inline V3T<R> norm_to_ray(V3T<R> x, R ct, R st, R cp, R sp) {
  return {x.x * ct * cp + x.y * ct * sp - x.z * st, -x.x * sp + x.y * cp,
          x.x * st * cp + x.y * st * sp + x.z * ct};
}
template <class R>
inline V3T<R> norm_to_ray(V3T<R> x, const SphT<R>& s) { return norm_to_ray(x, s.ct, s.st, s.cp, s.sp); }

// utils.jl:52-62 (the y component of Ev keeps the reference's sign, utils.jl:60)
template <class R>
inline void get_basis(V3T<R> k, V3T<R>& Eh, V3T<R>& Ev) {
  if (Fabs(k.z) > 1.0 - EPS) {
    Eh = {R(0.0), R(-1.0), R(0.0)};
    Ev = {jsign(k.z), R(0.0), R(0.0)};
  } else {
    R ev3 = -Sqrt(R(1.0) - k.z * k.z);
    R inv = R(1.0) / ev3;
    R eh1 = k.y * -inv;
    R eh2 = k.x * inv;
    Eh = {eh1, eh2, R(0.0)};
    Ev = {-k.z * eh2, -k.z * eh1, ev3};
  }
}

// utils.jl:82-84
template <class R>
inline V4T<R> rotate(V4T<R> I, R c2, R s2) {
  return {{I.v[0], c2 * I.v[1] + s2 * I.v[2], -s2 * I.v[1] + c2 * I.v[2], I.v[3]}};
}

// ---------------------------------------------------------------- scatterers
struct Scat {
  int kind = 0;  // 0 Rayleigh, 1 Mie
  double omega = 1, kl = 1;
  int ntheta = 0, random_points = 0;
  std::vector<double> F11, F12, F33, F34, csrn;
  std::vector<cplx> S11, S22;
};

template <class R>
struct PMT {  // phase matrix in the reference's block form
  R p11, p12, p33, p34;
};
using PM = PMT<double>;

// rayleigh.jl:8-18 and mie.jl:46-74; u < 0 means "do not sample" (cos given).
template <class R>
inline PMT<R> phase_matrix(const Scat& s, R& c, R u, bool sample) {
  if (s.kind == 0) {
    if (sample) {
      R rn = 2.0 * (1.0 - 2.0 * u);
      R r = Sqrt(1.0 + rn * rn);
      c = Cbrt(r + rn) - Cbrt(r - rn);
    }
    R c2 = c * c;
    return {0.75 * (1 + c2), -0.75 * (1 - c2), 1.5 * c, R(0.0)};
  }
  if (sample) {
    R rn = u * (double)s.random_points;
    long mrn = Trunc(rn);
    if (mrn > s.random_points - 1) mrn = s.random_points - 1;
    c = ((double)(mrn + 1) - rn) * s.csrn[mrn] + (rn - (double)mrn) * s.csrn[mrn + 1];
  }
  R th = Acos(clamp1(c));
  R sn = th / PI * (double)(s.ntheta - 1);
  long msn = Trunc(sn) + 1;  // 1-based as in mie.jl:55
  if (msn > s.ntheta) msn = s.ntheta;
  R w0 = (double)msn - sn;
  PMT<R> p{w0 * s.F11[msn - 1], w0 * s.F12[msn - 1], w0 * s.F33[msn - 1], w0 * s.F34[msn - 1]};
  if (msn + 1 <= s.ntheta) {
    R w1 = sn - (double)msn + 1.0;
    p.p11 += w1 * s.F11[msn];
    p.p12 += w1 * s.F12[msn];
    p.p33 += w1 * s.F33[msn];
    p.p34 += w1 * s.F34[msn];
  }
  return p;
}

template <class R>
inline V4T<R> pm_apply(const PMT<R>& p, V4T<R> I) {
  return {{p.p11 * I.v[0] + p.p12 * I.v[1], p.p12 * I.v[0] + p.p11 * I.v[1],
           p.p33 * I.v[2] + p.p34 * I.v[3], -p.p34 * I.v[2] + p.p33 * I.v[3]}};
}

// rayleigh.jl:20-23 and mie.jl:76-92 (keeps the (2-f, f-1) weights of mie.jl:80-85)
template <class R>
inline void amplitude_matrix(const Scat& s, R c, std::complex<R>& S11, std::complex<R>& S22) {
  using C = std::complex<R>;
  if (s.kind == 0) {
    S11 = C(R(0.0), R(1.0));
    S22 = C(R(0.0), c);
    return;
  }
  R th = Acos(clamp1(c));
  R sn = th / PI * (double)(s.ntheta - 1);
  long msn = Trunc(sn) + 1;
  if (msn > s.ntheta) msn = s.ntheta;
  R w0 = (double)(msn + 1) - sn;
  S11 = w0 * C(R(s.S11[msn - 1].real()), R(s.S11[msn - 1].imag()));
  S22 = w0 * C(R(s.S22[msn - 1].real()), R(s.S22[msn - 1].imag()));
  if (msn + 1 <= s.ntheta) {
    R w1 = sn - (double)msn;
    S11 += w1 * C(R(s.S11[msn].real()), R(s.S11[msn].imag()));
    S22 += w1 * C(R(s.S22[msn].real()), R(s.S22[msn].imag()));
  }
}

// utils.jl:91-112
template <class R>
inline V4T<R> update_I(const Scat& sca, V4T<R> I, V3T<R> k, const SphT<R>& f, V3T<R>* Eh_out = nullptr,
                       V3T<R>* Ev_out = nullptr) {
  V3T<R> Eh, Ev;
  get_basis(k, Eh, Ev);
  V3T<R> kr = norm_to_ray(k, f);
  SphT<R> ks = spherical_from_cartesian(kr);
  V3T<R> Ehk = ray_to_norm(V3T<R>{ks.sp, -ks.cp, R(0.0)}, f);
  V3T<R> Evk = ray_to_norm(V3T<R>{ks.ct * ks.cp, ks.ct * ks.sp, -ks.st}, f);
  R cpsi = Eh.x * Ehk.x + Eh.y * Ehk.y;
  R spsi = -Eh.x * Evk.x - Eh.y * Evk.y;
  R c = Max(kr.z, R(-1.0));
  PMT<R> P = phase_matrix(sca, c, R(0.0), false);
  V4T<R> Ip = pm_apply(P, rotate(I, ks.cp * ks.cp - ks.sp * ks.sp, -2.0 * ks.sp * ks.cp));
  Ip = rotate(Ip, cpsi * cpsi - spsi * spsi, 2.0 * spsi * cpsi);
  if (Eh_out) *Eh_out = Eh;
  if (Ev_out) *Ev_out = Ev;
  return Ip;
}

// utils.jl:119-150
template <class R>
inline void E_from_I(V4T<R> I, std::complex<R>& E1, std::complex<R>& E2) {
  const double tol = 1e-14;
  R A1, A2, phi2;
  if (I.v[0] - Fabs(I.v[1]) > tol * I.v[0]) {
    A1 = Sqrt(0.5 * (I.v[0] - I.v[1]));
    A2 = Sqrt(0.5 * (I.v[0] + I.v[1]));
    R q = Sqrt(I.v[0] * I.v[0] - I.v[1] * I.v[1]);
    if (I.v[2] >= q) {
      phi2 = 0.0;
    } else if (I.v[2] <= -q) {
      phi2 = PI;
    } else {
      phi2 = Acos(I.v[2] / q);
      if (I.v[3] > 0.0) phi2 = 2 * PI - phi2;
    }
  } else if (I.v[0] + I.v[1] <= tol * I.v[0]) {
    A1 = Sqrt(I.v[0]);
    A2 = 0.0;
    phi2 = 0.0;
  } else {
    A1 = 0.0;
    A2 = Sqrt(I.v[0]);
    phi2 = 0.0;
  }
  E1 = std::complex<R>(A1, R(0.0));
  E2 = A2 * std::complex<R>(Cos(phi2), Sin(phi2));
}

// utils.jl:157-163
template <class R>
inline V4T<R> I_from_E(std::complex<R> E1, std::complex<R> E2) {
  R qh = E1.real() * E1.real() + E1.imag() * E1.imag();
  R qv = E2.real() * E2.real() + E2.imag() * E2.imag();
  std::complex<R> x = E2 * std::conj(E1);
  return {{qh + qv, -qh + qv, 2.0 * x.real(), -2.0 * x.imag()}};
}

// utils.jl:170-192
template <class R>
inline void update_E(const Scat& sca, std::complex<R>& E1, std::complex<R>& E2, V3T<R> k, const SphT<R>& f,
                     V3T<R>* Eh_out = nullptr, V3T<R>* Ev_out = nullptr) {
  V3T<R> Eh, Ev;
  get_basis(k, Eh, Ev);
  V3T<R> kr = norm_to_ray(k, f);
  SphT<R> ks = spherical_from_cartesian(kr);
  V3T<R> Ehk = ray_to_norm(V3T<R>{ks.sp, -ks.cp, R(0.0)}, f);
  V3T<R> Evk = ray_to_norm(V3T<R>{ks.ct * ks.cp, ks.ct * ks.sp, -ks.st}, f);
  R cpsi = Eh.x * Ehk.x + Eh.y * Ehk.y;
  R spsi = Eh.x * Evk.x + Eh.y * Evk.y;
  std::complex<R> S11, S22;
  amplitude_matrix(sca, kr.z, S11, S22);
  std::complex<R> a = E1 * ks.cp + E2 * ks.sp, b = -E1 * ks.sp + E2 * ks.cp;
  a = S11 * a;
  b = S22 * b;
  E1 = a * cpsi + b * spsi;
  E2 = -a * spsi + b * cpsi;
  if (Eh_out) *Eh_out = Eh;
  if (Ev_out) *Ev_out = Ev;
}

// utils.jl:243-261 (iteration cap added)
inline double kepler_solver(double M, double e, long* capped) {
  const double tol = 1e-12;
  double MM = M - std::floor(M / (2 * PI)) * 2 * PI;
  double ea = M + 0.85 * e * jsign(std::sin(MM));
  double dea = 1.0;
  int it = 0;
  while (std::fabs(dea) > tol) {
    if (++it > MAX_KEPLER) {
      ++*capped;
      break;
    }
    double f3 = e * std::cos(ea), f2 = e * std::sin(ea), f1 = 1.0 - f3;
    double f = ea - f2 - M;
    dea = -f / f1;
    dea = -f / (f1 + f2 * dea / 2.0);
    dea = -f / (f1 + f2 * dea / 2.0 + f3 * dea * dea / 6.0);
    ea += dea;
  }
  return ea;
}

// ---------------------------------------------------------------- geometry
struct Layer {
  double tau, omega;
  bool inf;
  int scat;
};

struct Geom {
  int kind = 0;  // 0 plane, 1 sphere
  double theta = PI, phi = 0.0;
  std::vector<Layer> layers;  // sphere: exactly one, tau = optical radius
  std::vector<Scat> scats;
  int nl() const { return (int)layers.size(); }
};

template <class R>
inline R distance_to_boundary(const Geom& g, V3T<R> x, V3T<R> k, int idx) {
  if (g.kind == 0) {  // plane.jl:97-105
    if (k.z > 0) return -x.z / k.z;
    if (!g.layers[idx].inf) return (x.z + g.layers[idx].tau) / -k.z;
    return R(INFINITY);
  }
  R kx = dot(k, x), xx = dot(x, x);  // sphere.jl:69-73
  double tau = g.layers[0].tau;
  return -kx + Sqrt(Max(kx * kx + tau * tau - xx, R(0.0)));
}

inline int pass_boundary(const Geom& g, V3 x, int idx) {
  if (g.kind == 0) {  // plane.jl:107-115
    if (x.z > 0) return -1;
    if (!g.layers[idx].inf && x.z < -g.layers[idx].tau) return 1;
    return 0;
  }
  return norm3(x) > g.layers[0].tau ? -2 : 0;  // sphere.jl:75
}

inline double min_dist_first(const Geom& g, V3 x, int idx) {
  if (g.kind == 0) return idx == 0 ? std::fabs(x.z) : INFINITY;  // plane.jl:117
  return g.layers[0].tau - norm3(x);                              // sphere.jl:77
}

inline double min_dist_last(const Geom& g, V3 x, int idx) {
  if (g.kind == 0) {  // plane.jl:121-127
    if (idx == g.nl() - 1 && !g.layers[idx].inf) return g.layers[idx].tau - std::fabs(x.z);
    return INFINITY;
  }
  return INFINITY;  // sphere.jl:81
}

inline bool can_direct_transmit(const Geom& g) {
  if (g.kind == 0) return g.nl() == 1 && !g.layers[0].inf;  // plane.jl:64
  return true;                                               // sphere.jl:39
}

inline void incidence_angle(const Geom& g, double& th, double& ph) {
  if (g.kind == 0) {
    th = g.theta;
    ph = g.phi;
  } else {
    th = PI;
    ph = 0.0;
  }
}

// ---------------------------------------------------------------- configuration
struct Cfg {
  int64_t nrays;
  double min_int;
  int64_t max_scat;
  bool compute_cb;
  double tau0;
  int nphi, ntheta, nthetab, nphib;
  const double *cphi, *sphi, *ctheta, *stheta, *inorm, *cthetab, *sthetab, *cphib, *sphib;
  int up0, up1, lo0, lo1;  // theta ranges [a, b)
};

struct Tally {
  double A[5] = {0, 0, 0, 0, 0};
  std::vector<double> Irt, Icb, ladder;
  double peak_sum = 0, peak_sq = 0, photons = 0;
  double events = 0, attempts = 0, rt_evals = 0, cb1_evals = 0, cbn_evals = 0;
  long kepler_capped = 0, attempts_capped = 0;
};

struct Ctx {
  const Cfg* cfg;
  const Geom* g;
  V4 I0;
  V3 k0;
  Sph inc;  // incidence angle trig, as used by forward_E/backward_E (cpu.jl:47-49)
  Rng rng;
  int cb_form;  // 0: reference O(n) walk, 1: incremental
};

// utils.jl:294-323, with the three draws of one attempt passed in
inline V4 scatter(const Ctx& C, V4 I, V3 k, int idx, double u0, double u1, V3& kp, Tally& T) {
  const Scat& sca = C.g->scats[C.g->layers[idx].scat];
  Sph ks = spherical_from_cartesian(k);
  double ct = 0;
  PM P = phase_matrix(sca, ct, u0, true);
  double eq = -P.p12 * I.v[1] / (P.p11 * I.v[0]);
  double eu = -P.p12 * I.v[2] / (P.p11 * I.v[0]);
  double ee = std::sqrt(eq * eq + eu * eu);
  double phi;
  if (ee > 1e-12) {
    double gam = std::acos(clamp1(eq / ee));
    if (eu < 0) gam = 2 * PI - gam;
    double ma = 4 * PI * u1 + gam - ee * std::sin(gam);
    double ea = kepler_solver(ma, ee, &T.kepler_capped);
    phi = 0.5 * (ea - gam);
  } else {
    phi = 2 * PI * u1;
  }
  double st = std::sqrt(std::max(1 - ct * ct, 0.0));
  kp = ray_to_norm(V3{st * std::cos(phi), st * std::sin(phi), ct}, ks);
  V4 Ip = update_I(sca, I, kp, ks);
  return scale4(Ip, I.v[0] / Ip.v[0]);
}

// One RT bin of cpu.jl:13-26: the peel-off Stokes vector into the direction
// (st cos(phi), st sin(phi), ct) with its attenuation and quadrature weight. Returns
// false when the path to the boundary is longer than tau0 (no contribution).
template <class R>
inline bool rt_bin(const Scat& sca, const Geom& g, double tau0, V4T<R> I, const SphT<R>& ks, V3T<R> x, int idx,
                   R st, R ct, R cphi, R sphi, R inorm, V4T<R>& Ipp) {
  V3T<R> kk{st * cphi, st * sphi, ct};
  V4T<R> Ip = update_I(sca, I, kk, ks);
  R t = distance_to_boundary(g, x, kk, idx);
  if (!(t <= tau0)) return false;
  R nx = Exp(-t);
  Ipp = scale4(Ip, inorm * nx);
  return true;
}

// cpu.jl:6-31
inline double collect_rt(const Ctx& C, Tally& T, V4 I, V3 k, V3 x, int idx, int j1a, int j1b) {
  const Cfg& cfg = *C.cfg;
  const Scat& sca = C.g->scats[C.g->layers[idx].scat];
  Sph ks = spherical_from_cartesian(k);
  double acc = 0.0;
  for (int j2 = 0; j2 < cfg.nphi; ++j2) {
    for (int j1 = j1a; j1 < j1b; ++j1) {
      V4 Ipp;
      if (rt_bin(sca, *C.g, cfg.tau0, I, ks, x, idx, cfg.stheta[j1], cfg.ctheta[j1], cfg.cphi[j2], cfg.sphi[j2],
                 cfg.inorm[j1], Ipp)) {
        double* dst = &T.Irt[4 * ((size_t)j2 * cfg.ntheta + j1)];
        for (int s = 0; s < 4; ++s) dst[s] += Ipp.v[s];
        acc += Ipp.v[0];
      }
    }
  }
  T.rt_evals += (double)cfg.nphi * (j1b - j1a);
  return acc;
}

// utils.jl:199-216: field along the path, first to last scatterer
inline void forward_E(const Scat& sca, cplx& E1, cplx& E2, const std::vector<V3>& kpath, int n,
                      Sph ks, double& enorm) {
  enorm = 0.0;
  double norm0 = std::sqrt(std::norm(E1) + std::norm(E2));
  for (int k = 2; k <= n; ++k) {
    update_E(sca, E1, E2, kpath[k], ks);
    double norm2 = std::sqrt(std::norm(E1) + std::norm(E2));
    E1 *= norm0 / norm2;
    E2 *= norm0 / norm2;
    enorm += std::log(norm0 / norm2);
    ks = spherical_from_cartesian(kpath[k]);
  }
}

// utils.jl:223-241: field along the reversed path
inline void backward_E(const Scat& sca, cplx& E1, cplx& E2, const std::vector<V3>& kpath, int n,
                       Sph ks, double& enorm) {
  enorm = 0.0;
  double norm0 = std::sqrt(std::norm(E1) + std::norm(E2));
  for (int k = n; k >= 2; --k) {
    update_E(sca, E1, E2, -kpath[k], ks);
    double norm2 = std::sqrt(std::norm(E1) + std::norm(E2));
    E1 *= norm0 / norm2;
    E2 *= norm0 / norm2;
    enorm += std::log(norm0 / norm2);
    ks = spherical_from_cartesian(-kpath[k]);
  }
}

// 2x2 complex matrix of update_E(sca, ., k, f): columns are the images of (1,0), (0,1).
struct M2 {
  cplx a, b, c, d;  // [[a, b], [c, d]]
};
inline M2 update_E_matrix(const Scat& sca, V3 k, const Sph& f) {
  cplx x1(1, 0), x2(0, 0), y1(0, 0), y2(1, 0);
  update_E(sca, x1, x2, k, f);
  update_E(sca, y1, y2, k, f);
  return {x1, y1, x2, y2};
}
inline M2 mul(const M2& p, const M2& q) {
  return {p.a * q.a + p.b * q.c, p.a * q.b + p.b * q.d, p.c * q.a + p.d * q.c,
          p.c * q.b + p.d * q.d};
}

// Incremental reciprocal-path state: the forward field is advanced one scatterer per
// event exactly as forward_E does; the backward field is L_n * M(-k_n | incidence) * E_i
// with L_{n+1} = L_n * M(-k_n | frame(-k_{n+1})), kept scaled with a log factor.
struct CBState {
  cplx A1, A2;       // forward field, norm kept at norm0
  double enorma;     // sum of log(norm0 / norm2) as in forward_E
  M2 L;              // backward prefix product, scaled
  double logL;       // log of the scale removed from L
};

struct PathBuf {
  std::vector<V3> kpath, xpath;
  std::vector<int> idxpath;
};

// Per-event inputs of one reciprocal-path CB bin (computed once per event, cpu.jl:42-81).
template <class R>
struct CBNIn {
  SphT<R> kfs, kas, kbs;
  V3T<R> ki, xa, xb;
  int idxa, idxb;
  R kl, tab;
  std::complex<R> Ea1, Ea2, Eb1, Eb2;
};

// One reciprocal-path CB bin of cpu.jl:85-126: the forward and backward fields into the
// bin direction, their attenuations, the interference with phase kl (ki + kf).(xa - xb),
// and the rotation into the bin's frame. Returns false when tau0 cuts the forward path.
template <class R>
inline bool cbn_bin(const Scat& sca, const Geom& g, double tau0, const CBNIn<R>& e, R stb, R ctb, R cpb, R spb,
                    V4T<R>& I1, R& ladder) {
  V3T<R> kfb{stb * cpb, stb * spb, ctb};
  kfb = ray_to_norm(kfb, e.kfs);
  std::complex<R> a1 = e.Ea1, a2 = e.Ea2, b1 = e.Eb1, b2 = e.Eb2;
  update_E(sca, a1, a2, kfb, e.kas);
  V3T<R> Eh, Ev;
  update_E(sca, b1, b2, kfb, e.kbs, &Eh, &Ev);
  R dphi = e.kl * dot(e.ki + kfb, e.xa - e.xb);
  R tya = distance_to_boundary(g, e.xa, kfb, e.idxa);
  if (!(tya <= tau0)) return false;
  R nexta = Exp(-0.5 * tya);
  a1 *= nexta;
  a2 *= nexta;
  V4T<R> Ia = I_from_E(a1, a2);
  R tyb = distance_to_boundary(g, e.xb, kfb, e.idxb);
  if (Fabs(tyb + e.tab) <= tau0) {
    R nextb = Exp(-0.5 * (tyb + e.tab));
    b1 *= nextb;
    b2 *= nextb;
  } else {
    b1 = R(0.0);
    b2 = R(0.0);
  }
  V4T<R> Ib = I_from_E(b1, b2);
  std::complex<R> ph(Cos(dphi), Sin(dphi));
  V4T<R> Iab = I_from_E(a1 * ph + b1, a2 * ph + b2);
  Iab = scale4(Iab, Ia.v[0] / (Ia.v[0] + Ib.v[0]));
  Eh = norm_to_ray(Eh, e.kfs);
  Ev = norm_to_ray(Ev, e.kfs);
  R cpsi = spb * Eh.x - cpb * Eh.y;
  R spsi = -spb * Ev.x + cpb * Ev.y;
  I1 = rotate(Iab, cpsi * cpsi - spsi * spsi, 2.0 * cpsi * spsi);
  ladder = Ia.v[0];
  return true;
}

// One single-scattering CB bin of cpu.jl:132-156.
template <class R>
inline bool cb1_bin(const Scat& sca, const Geom& g, double tau0, V4T<R> I, const SphT<R>& kfs, const SphT<R>& kas,
                    V3T<R> xa, int idxa, R stb, R ctb, R cpb, R spb, V4T<R>& I1) {
  V3T<R> kfb{stb * cpb, stb * spb, ctb};
  kfb = ray_to_norm(kfb, kfs);
  V3T<R> Eh, Ev;
  V4T<R> Iaf = update_I(sca, I, kfb, kas, &Eh, &Ev);
  R tya = distance_to_boundary(g, xa, kfb, idxa);
  if (!(tya <= tau0)) return false;
  Iaf = scale4(Iaf, Exp(-tya));
  Eh = norm_to_ray(Eh, kfs);
  Ev = norm_to_ray(Ev, kfs);
  R cpsi = spb * Eh.x - cpb * Eh.y;
  R spsi = -spb * Ev.x + cpb * Ev.y;
  I1 = rotate(Iaf, cpsi * cpsi - spsi * spsi, 2.0 * cpsi * spsi);
  return true;
}

// cpu.jl:38-160, plus the ladder (incoherent) s11 and the per-photon CB-peak value.
inline void collect_cb(const Ctx& C, Tally& T, V4 I, V3 k, V3 x, int idx, const PathBuf& pb, int n,
                       const CBState* inc, double& peak) {
  const Cfg& cfg = *C.cfg;
  const Geom& g = *C.g;
  V3 xa = x, ka = k;
  int idxa = idx;
  Sph kas = spherical_from_cartesian(ka);
  V3 kf = -pb.kpath[1];
  Sph kfs = spherical_from_cartesian(kf);
  const Scat& sca = g.scats[g.layers[0].scat];  // cpu.jl:50 (layer 1 always)
  double kl = sca.kl;                           // cpu.jl:94 (layer 1 always)
  if (n > 1) {
    V3 ki = pb.kpath[1];
    V3 xb = pb.xpath[1];
    V3 kb = -pb.kpath[2];
    int idxb = pb.idxpath[1];
    Sph kbs = spherical_from_cartesian(kb);
    double ta = distance_to_boundary(g, xa, kf, idxa);
    double tb = distance_to_boundary(g, xb, kf, idxb);
    double tab = ta - tb;
    V4 Iaf = update_I(sca, I, kf, kas);
    cplx Ei1, Ei2;
    E_from_I(C.I0, Ei1, Ei2);
    cplx Ea1, Ea2, Eb1, Eb2;
    double enorma, enormb;
    if (!inc) {
      Ea1 = Ei1;
      Ea2 = Ei2;
      forward_E(sca, Ea1, Ea2, pb.kpath, n, C.inc, enorma);
      Eb1 = Ei1;
      Eb2 = Ei2;
      backward_E(sca, Eb1, Eb2, pb.kpath, n, C.inc, enormb);
    } else {
      Ea1 = inc->A1;
      Ea2 = inc->A2;
      enorma = inc->enorma;
      M2 Mn = update_E_matrix(sca, -pb.kpath[n], C.inc);
      M2 B = mul(inc->L, Mn);
      cplx b1 = B.a * Ei1 + B.b * Ei2, b2 = B.c * Ei1 + B.d * Ei2;
      double norm0 = std::sqrt(std::norm(Ei1) + std::norm(Ei2));
      double nb = std::sqrt(std::norm(b1) + std::norm(b2));
      Eb1 = b1 * (norm0 / nb);
      Eb2 = b2 * (norm0 / nb);
      enormb = std::log(norm0 / nb) - inc->logL;
    }
    double sc = std::exp(enorma - enormb);
    Eb1 *= sc;
    Eb2 *= sc;
    cplx Eaf1 = Ea1, Eaf2 = Ea2;
    update_E(sca, Eaf1, Eaf2, kf, kas);
    // gpu.jl:84; a rounded, slightly negative intensity (90-degree Rayleigh scattering of
    // a fully polarised photon, P11 = -P12) or a vanishing field norm gives zero here,
    // where the reference's sqrt would throw a DomainError.
    const double nef = std::norm(Eaf1) + std::norm(Eaf2);
    double raa = nef > 0 ? std::sqrt(std::max(Iaf.v[0], 0.0) / nef) : 0.0;
    Ea1 *= raa;
    Ea2 *= raa;
    Eb1 *= raa;
    Eb2 *= raa;
    const CBNIn<double> e{kfs, kas, kbs, ki, xa, xb, idxa, idxb, kl, tab, Ea1, Ea2, Eb1, Eb2};
    for (int j2 = 0; j2 < cfg.nphib; ++j2) {
      for (int j1 = 0; j1 < cfg.nthetab; ++j1) {
        V4 I1;
        double lad;
        if (cbn_bin(sca, g, cfg.tau0, e, cfg.sthetab[j1], cfg.cthetab[j1], cfg.cphib[j2], cfg.sphib[j2], I1, lad)) {
          size_t b = (size_t)j2 * cfg.nthetab + j1;
          for (int s = 0; s < 4; ++s) T.Icb[4 * b + s] += I1.v[s];
          T.ladder[b] += lad;
          if (b == 0) peak += I1.v[0];
        }
      }
    }
    T.cbn_evals += (double)cfg.nphib * cfg.nthetab;
  } else {
    for (int j2 = 0; j2 < cfg.nphib; ++j2) {
      for (int j1 = 0; j1 < cfg.nthetab; ++j1) {
        V4 I1;
        if (cb1_bin(sca, g, cfg.tau0, I, kfs, kas, xa, idxa, cfg.sthetab[j1], cfg.cthetab[j1], cfg.cphib[j2],
                    cfg.sphib[j2], I1)) {
          size_t b = (size_t)j2 * cfg.nthetab + j1;
          for (int s = 0; s < 4; ++s) T.Icb[4 * b + s] += I1.v[s];
          T.ladder[b] += I1.v[0];
          if (b == 0) peak += I1.v[0];
        }
      }
    }
    T.cb1_evals += (double)cfg.nphib * cfg.nthetab;
  }
}

// plane.jl:77-95 and sphere.jl:54-67
inline V3 initial_propagation(const Ctx& C, V3 x, V3 k, uint64_t photon, Tally& T) {
  const Cfg& cfg = *C.cfg;
  const Geom& g = *C.g;
  double t;
  Draws d0 = C.rng.at(photon, 0, 0);
  if (g.kind == 0) {
    if (g.layers[0].inf) {
      t = -std::log(d0.u[2]);
    } else {
      bool has_dt = can_direct_transmit(g);
      double tp = distance_to_boundary(g, x, k, 0);
      if (has_dt && tp <= cfg.tau0) {
        t = -std::log(1 - d0.u[2] * (1 - std::exp(-tp)));
      } else {
        t = tp + 1;
        for (uint32_t a = 0; t > tp; ++a) {
          if (a >= MAX_ATTEMPTS) {
            ++T.attempts_capped;
            t = tp;
            break;
          }
          t = -std::log(a == 0 ? d0.u[2] : C.rng.at(photon, 0, a).u[2]);
        }
      }
    }
  } else {
    double tp = 2.0 * x.z;
    if (tp <= cfg.tau0) {
      t = -std::log(1 - d0.u[2] * (1 - std::exp(-tp)));
    } else {
      t = tp + 1;
      for (uint32_t a = 0; t > tp; ++a) {
        if (a >= MAX_ATTEMPTS) {
          ++T.attempts_capped;
          t = tp;
          break;
        }
        t = -std::log(1 - (a == 0 ? d0.u[2] : C.rng.at(photon, 0, a).u[2]));
      }
    }
  }
  return x + t * k;
}

// cpu.jl:162-273 for one photon
void trace_photon(const Ctx& C, uint64_t photon, PathBuf& pb, Tally& T) {
  const Cfg& cfg = *C.cfg;
  const Geom& g = *C.g;
  V4 I = C.I0;
  V3 k = C.k0;
  V3 x{0, 0, 0};
  if (g.kind == 1) {  // sphere.jl:43-47
    Draws d0 = C.rng.at(photon, 0, 0);
    double tau = g.layers[0].tau;
    double r = tau * std::sqrt(d0.u[0]);
    double ph = 2 * PI * d0.u[1];
    x = {r * std::cos(ph), r * std::sin(ph), std::sqrt(tau * tau - r * r)};
  }
  int idx = 0;
  int n = 0;
  if (can_direct_transmit(g)) {
    double tp = distance_to_boundary(g, x, k, idx);
    double dt = tp <= cfg.tau0 ? std::exp(-tp) : 0.0;
    T.A[0] += I.v[0] * dt;
    I = scale4(I, 1 - dt);
  }
  x = initial_propagation(C, x, k, photon, T);

  CBState cbs;
  const Scat& sca1 = g.scats[g.layers[0].scat];
  bool use_inc = C.cb_form == 1 && cfg.compute_cb;
  double peak = 0.0;

  while (I.v[0] >= cfg.min_int && n < cfg.max_scat) {
    ++n;
    pb.kpath[n] = k;
    pb.xpath[n] = x;
    pb.idxpath[n] = idx;
    if (use_inc) {
      if (n == 1) {
        E_from_I(C.I0, cbs.A1, cbs.A2);
        cbs.enorma = 0.0;
        cbs.L = {1.0, 0.0, 0.0, 1.0};
        cbs.logL = 0.0;
      } else {
        Sph fr = n == 2 ? C.inc : spherical_from_cartesian(pb.kpath[n - 1]);
        cplx Ei1, Ei2;
        E_from_I(C.I0, Ei1, Ei2);
        double norm0 = std::sqrt(std::norm(Ei1) + std::norm(Ei2));
        update_E(sca1, cbs.A1, cbs.A2, pb.kpath[n], fr);
        double norm2 = std::sqrt(std::norm(cbs.A1) + std::norm(cbs.A2));
        cbs.A1 *= norm0 / norm2;
        cbs.A2 *= norm0 / norm2;
        cbs.enorma += std::log(norm0 / norm2);
        if (n >= 3) {
          M2 step = update_E_matrix(sca1, -pb.kpath[n - 1], spherical_from_cartesian(-pb.kpath[n]));
          cbs.L = mul(cbs.L, step);
          double s = std::sqrt(std::norm(cbs.L.a) + std::norm(cbs.L.b) + std::norm(cbs.L.c) +
                               std::norm(cbs.L.d));
          cbs.L = {cbs.L.a / s, cbs.L.b / s, cbs.L.c / s, cbs.L.d / s};
          cbs.logL += std::log(s);
        }
      }
    }

    V4 Ip = I;
    V3 kp = k, xp = x;
    int idxp = idx;
    for (uint32_t a = 0;; ++a) {
      if (a >= MAX_ATTEMPTS) {
        ++T.attempts_capped;
        I.v[0] = -INFINITY;  // terminate the photon; its weight is reported as capped
        break;
      }
      Draws d = C.rng.at(photon, (uint32_t)n, a);
      T.attempts += 1;
      Ip = scatter(C, I, k, idx, d.u[0], d.u[1], kp, T);
      double t = -std::log(d.u[2]);
      xp = x + t * kp;
      int pbv = pass_boundary(g, xp, idx);
      idxp = idx + pbv;
      if (pbv == -2) continue;
      if (pbv == -1) {
        if (idxp < 0) continue;
        xp = {x.x, x.y, -g.layers[idx].tau};
        break;
      }
      if (pbv == 1) {
        if (idxp > g.nl() - 1) continue;
        xp = {x.x, x.y, 0.0};
        break;
      }
      break;
    }
    if (!(I.v[0] > -INFINITY)) break;
    T.events += 1;

    double om = g.layers[idx].omega;
    T.A[1] += (1.0 - om) * I.v[0];
    I = scale4(I, om);

    double Iref = 0.0, Itrans = 0.0;
    bool near_upper = min_dist_first(g, x, idx) <= cfg.tau0;
    bool near_lower = min_dist_last(g, x, idx) <= cfg.tau0;
    if (cfg.compute_cb && (near_upper || near_lower))
      collect_cb(C, T, I, k, x, idx, pb, n, use_inc ? &cbs : nullptr, peak);
    if (near_upper) Iref = collect_rt(C, T, I, k, x, idx, cfg.up0, cfg.up1);
    if (near_lower) Itrans = collect_rt(C, T, I, k, x, idx, cfg.lo0, cfg.lo1);
    T.A[2] += Iref;
    T.A[3] += Itrans;
    double Iesc = Iref + Itrans;
    I = scale4(Ip, (I.v[0] - Iesc) / Ip.v[0]);
    k = kp;
    x = xp;
    idx = idxp;
  }
  if (I.v[0] > -INFINITY) T.A[4] += I.v[0];
  T.peak_sum += peak;
  T.peak_sq += peak * peak;
  T.photons += 1;
}

}  // namespace

// ==================================================================== C interface
extern "C" {

typedef struct {
  int kind;
  double omega, kl;
  int n_theta;
  const double *F11, *F12, *F33, *F34;
  const double *S11, *S22;  // interleaved (re, im), n_theta pairs each
  int random_points;
  const double* csrn;       // random_points + 1 entries
} orc_scatterer;

typedef struct {
  double tau, omega;
  int infinite;
  int scatterer;
} orc_layer;

typedef struct {
  int kind;  // 0 plane, 1 sphere
  double theta, phi;
  int n_layers;
  const orc_layer* layers;
  int n_scatterers;
  const orc_scatterer* scatterers;
} orc_geometry;

typedef struct {
  int64_t number_of_rays;
  double minimum_intensity;
  int64_t maximum_scattering_times;
  int compute_cb;
  double tau0;
  int n_phi;
  const double *cos_phi, *sin_phi;
  int n_theta;
  const double *cos_theta, *sin_theta, *inorm;
  int n_theta_b;
  const double *cos_theta_b, *sin_theta_b;
  int n_phi_b;
  const double *cos_phi_b, *sin_phi_b;
} orc_config;

typedef struct {
  uint64_t seed;
  uint32_t instance;
  int rng_mode;  // 0 Philox, 1 stratified first-collision depth
  int cb_form;   // 0 reference walk, 1 incremental
  int n_threads; // <= 0: all
  int64_t photon_begin, photon_count;
} orc_run;

// Raw sums (not divided by the number of rays). stats = {sum peak, sum peak^2, photons};
// counters = {events, attempts, rt_evals, cb1_evals, cbn_evals, kepler_capped,
// attempts_capped}.
int orc_simulate(const orc_config* c, const orc_geometry* gd, const double I0[4], const orc_run* run,
                 double A_out[5], double* Irt, double* Icb, double* ladder, double* stats,
                 double* counters) {
  if (!c || !gd || !I0 || !run) return 1;
  if (gd->n_layers < 1 || gd->n_scatterers < 1) return 1;
  Geom g;
  g.kind = gd->kind;
  g.theta = gd->theta;
  g.phi = gd->phi;
  for (int i = 0; i < gd->n_layers; ++i) {
    const orc_layer& L = gd->layers[i];
    if (L.scatterer < 0 || L.scatterer >= gd->n_scatterers) return 1;
    g.layers.push_back({L.tau, L.omega, L.infinite != 0, L.scatterer});
  }
  for (int i = 0; i < gd->n_scatterers; ++i) {
    const orc_scatterer& s = gd->scatterers[i];
    Scat S;
    S.kind = s.kind;
    S.omega = s.omega;
    S.kl = s.kl;
    if (s.kind == 1) {
      S.ntheta = s.n_theta;
      S.random_points = s.random_points;
      S.F11.assign(s.F11, s.F11 + s.n_theta);
      S.F12.assign(s.F12, s.F12 + s.n_theta);
      S.F33.assign(s.F33, s.F33 + s.n_theta);
      S.F34.assign(s.F34, s.F34 + s.n_theta);
      S.csrn.assign(s.csrn, s.csrn + s.random_points + 1);
      for (int j = 0; j < s.n_theta; ++j) {
        S.S11.emplace_back(s.S11[2 * j], s.S11[2 * j + 1]);
        S.S22.emplace_back(s.S22[2 * j], s.S22[2 * j + 1]);
      }
    }
    g.scats.push_back(std::move(S));
  }
  Cfg cfg{};
  cfg.nrays = c->number_of_rays;
  cfg.min_int = c->minimum_intensity;
  cfg.max_scat = c->maximum_scattering_times;
  cfg.compute_cb = c->compute_cb != 0;
  cfg.tau0 = c->tau0;
  cfg.nphi = c->n_phi;
  cfg.cphi = c->cos_phi;
  cfg.sphi = c->sin_phi;
  cfg.ntheta = c->n_theta;
  cfg.ctheta = c->cos_theta;
  cfg.stheta = c->sin_theta;
  cfg.inorm = c->inorm;
  cfg.nthetab = c->n_theta_b;
  cfg.cthetab = c->cos_theta_b;
  cfg.sthetab = c->sin_theta_b;
  cfg.nphib = c->n_phi_b;
  cfg.cphib = c->cos_phi_b;
  cfg.sphib = c->sin_phi_b;
  if (g.kind == 0) {  // plane.jl:119,129
    cfg.up0 = cfg.ntheta / 2;
    cfg.up1 = cfg.ntheta;
    cfg.lo0 = 0;
    cfg.lo1 = cfg.ntheta / 2;
  } else {  // sphere.jl:79,83
    cfg.up0 = 0;
    cfg.up1 = cfg.ntheta;
    cfg.lo0 = 0;
    cfg.lo1 = 0;
  }

  Ctx C;
  C.cfg = &cfg;
  C.g = &g;
  for (int s = 0; s < 4; ++s) C.I0.v[s] = I0[s];
  double th0, ph0;
  incidence_angle(g, th0, ph0);
  C.inc = {std::cos(th0), std::sin(th0), std::cos(ph0), std::sin(ph0)};
  C.k0 = ray_to_norm(V3{0.0, 0.0, 1.0}, C.inc);  // MonteCarloRadiativeTransfer.jl:32
  C.rng.key[0] = (uint32_t)run->seed;
  C.rng.key[1] = (uint32_t)(run->seed >> 32) + 0x632BE5ABu * run->instance;
  C.rng.mode = run->rng_mode;
  C.rng.n_total = cfg.nrays;
  C.cb_form = run->cb_form;

  int nthr = 1;
#ifdef _OPENMP
  nthr = run->n_threads > 0 ? run->n_threads : omp_get_max_threads();
#endif
  std::vector<Tally> tallies(nthr);
  size_t nrt = 4 * (size_t)cfg.ntheta * cfg.nphi, ncb = 4 * (size_t)cfg.nthetab * cfg.nphib;
  for (auto& T : tallies) {
    T.Irt.assign(nrt, 0.0);
    T.Icb.assign(ncb, 0.0);
    T.ladder.assign(ncb / 4, 0.0);
  }
  int64_t p0 = run->photon_begin, pn = run->photon_count;
#pragma omp parallel num_threads(nthr)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    PathBuf pb;
    pb.kpath.resize(cfg.max_scat + 2);
    pb.xpath.resize(cfg.max_scat + 2);
    pb.idxpath.resize(cfg.max_scat + 2);
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = 0; i < pn; ++i) trace_photon(C, (uint64_t)(p0 + i), pb, tallies[tid]);
  }
  for (int s = 0; s < 5; ++s) A_out[s] = 0;
  std::memset(Irt, 0, nrt * sizeof(double));
  std::memset(Icb, 0, ncb * sizeof(double));
  if (ladder) std::memset(ladder, 0, ncb / 4 * sizeof(double));
  double st[3] = {0, 0, 0}, ct[7] = {0, 0, 0, 0, 0, 0, 0};
  for (auto& T : tallies) {
    for (int s = 0; s < 5; ++s) A_out[s] += T.A[s];
    for (size_t i = 0; i < nrt; ++i) Irt[i] += T.Irt[i];
    for (size_t i = 0; i < ncb; ++i) Icb[i] += T.Icb[i];
    if (ladder)
      for (size_t i = 0; i < ncb / 4; ++i) ladder[i] += T.ladder[i];
    st[0] += T.peak_sum;
    st[1] += T.peak_sq;
    st[2] += T.photons;
    ct[0] += T.events;
    ct[1] += T.attempts;
    ct[2] += T.rt_evals;
    ct[3] += T.cb1_evals;
    ct[4] += T.cbn_evals;
    ct[5] += (double)T.kepler_capped;
    ct[6] += (double)T.attempts_capped;
  }
  if (stats)
    for (int i = 0; i < 3; ++i) stats[i] = st[i];
  if (counters)
    for (int i = 0; i < 7; ++i) counters[i] = ct[i];
  return 0;
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  philox4x32_10(ctr, key, out);
}

// Rayleigh cos(theta) sampler of rayleigh.jl:10-11 for a given uniform draw.
double orc_rayleigh_sample(double u) {
  Scat s;
  double c = 0;
  phase_matrix(s, c, u, true);
  return c;
}

double orc_kepler_solver(double M, double e) {
  long capped = 0;
  return kepler_solver(M, e, &capped);
}

// MieScatterer's tables (src/scatterers/mie.jl:36-44): bhmie (mie.jl:129-216) for the
// amplitude functions S1, S2 and the normalised Mueller elements F11, F12, F33, F34 on
// Nθ uniform angles over [0, π], then calculate_csrn (src/utils.jl:263-287) for the
// inverse CDF of cos(Θ) on random_points + 1 uniform probabilities. S1, S2 are
// interleaved (re, im). q = {q_ext, q_sca, q_abs, q_back, asymm}. Returns 0, or 1 for
// invalid sizes.
int orc_mie_tables(double x, double m_re, double m_im, int n_theta, int random_points, double* F11,
                   double* F12, double* F33, double* F34, double* S1_out, double* S2_out, double* csrn,
                   double* q) {
  if (!(x > 0) || n_theta < 2 || random_points < 1) return 1;
  const cplx m(m_re, m_im);
  const cplx y = m * x;
  const int nstop = (int)std::floor(std::max(x + 4 * std::cbrt(x) + 2, x * std::abs(m)));  // mie.jl:133
  const int nmax = nstop + 15;                                                             // nextra = 15
  const int N = n_theta;
  // θ = range(0, π, Nθ); μ = cos.(θ). Arrays below are 1-based as in the reference.
  std::vector<double> mu(N + 1);
  for (int i = 1; i <= N; ++i) mu[i] = std::cos(PI * (double)(i - 1) / (double)(N - 1));
  std::vector<cplx> d(nmax + 1, cplx(0.0, 0.0));  // d[nmax] = 0; downward recursion (mie.jl:138-141)
  for (int n = nmax - 1; n >= 1; --n) d[n] = (double)(n + 1) / y - 1.0 / (d[n + 1] + (double)(n + 1) / y);
  std::vector<double> pin(N + 1, 0.0), tn(N + 1, 0.0), pi0(N + 1, 0.0), pi1(N + 1, 1.0);
  std::vector<cplx> S1(N + 1, cplx(0.0, 0.0)), S2(N + 1, cplx(0.0, 0.0));
  double psi0 = std::cos(x), psi1 = std::sin(x), chi0 = -std::sin(x), chi1 = std::cos(x);
  cplx xi1(psi1, -chi1), a_prev(0.0, 0.0), b_prev(0.0, 0.0);
  double qsca = 0.0, g = 0.0;
  for (int n = 1; n <= nstop; ++n) {
    const double dn = (double)n;
    const double fn = (2.0 * dn + 1.0) / (dn * (dn + 1.0));
    const double psi = (2.0 * dn - 1.0) * psi1 / x - psi0;
    const double chi = (2.0 * dn - 1.0) * chi1 / x - chi0;
    const cplx xi(psi, -chi);
    const cplx da = d[n] / m + dn / x, db = d[n] * m + dn / x;
    const cplx an = (da * psi - psi1) / (da * xi - xi1);  // mie.jl:163-165
    const cplx bn = (db * psi - psi1) / (db * xi - xi1);
    qsca += (std::norm(an) + std::norm(bn)) * (2.0 * dn + 1.0);
    g += (an.real() * bn.real() + an.imag() * bn.imag()) * fn;
    if (n > 1)
      g += (a_prev.real() * an.real() + a_prev.imag() * an.imag() + b_prev.real() * bn.real() +
            b_prev.imag() * bn.imag()) * (dn - 1.0) * (dn + 1.0) / dn;
    for (int i = 1; i <= (N + 1) / 2; ++i) {  // mie.jl:173-184: half range, mirrored by parity
      const int ii = N + 1 - i;
      pin[i] = pi1[i];
      tn[i] = dn * mu[i] * pin[i] - (dn + 1.0) * pi0[i];
      S1[i] += fn * (an * pin[i] + bn * tn[i]);
      S2[i] += fn * (an * tn[i] + bn * pin[i]);
      if (i < ii) {
        const double p = (n & 1) == 0 ? -1.0 : 1.0;
        S1[ii] += fn * (an * pin[i] - bn * tn[i]) * p;
        S2[ii] += fn * (-an * tn[i] + bn * pin[i]) * p;
      }
    }
    psi0 = psi1;
    psi1 = psi;
    chi0 = chi1;
    chi1 = chi;
    xi1 = cplx(psi1, -chi1);
    a_prev = an;
    b_prev = bn;
    for (int i = 1; i <= N; ++i) pi1[i] = ((2.0 * dn + 1.0) * mu[i] * pin[i] - (dn + 1.0) * pi0[i]) / dn;
    for (int i = 1; i <= N; ++i) pi0[i] = pin[i];
  }
  g *= 2.0 / qsca;
  qsca *= 2.0 / (x * x);
  const double qext = 4.0 / (x * x) * S1[1].real();
  if (q) {
    q[0] = qext;
    q[1] = qsca;
    q[2] = qext - qsca;
    q[3] = 4.0 / (x * x) * std::norm(S1[N]);
    q[4] = g;
  }
  const double coeff = 4.0 / (qsca * x * x);  // mie.jl:201-212
  for (int i = 1; i <= N; ++i) {
    const double s1 = std::norm(S1[i]), s2 = std::norm(S2[i]);
    const cplx c = S2[i] * std::conj(S1[i]);
    F11[i - 1] = (s1 + s2) * 0.5 * coeff;
    F12[i - 1] = -(s1 - s2) * 0.5 * coeff;
    F33[i - 1] = c.real() * coeff;
    F34[i - 1] = c.imag() * coeff;
    S1_out[2 * (i - 1)] = S1[i].real();
    S1_out[2 * (i - 1) + 1] = S1[i].imag();
    S2_out[2 * (i - 1)] = S2[i].real();
    S2_out[2 * (i - 1) + 1] = S2[i].imag();
  }

  // calculate_csrn(itpf11, n) with itpf11 the linear interpolant of F11 on the θ grid.
  const int n = random_points;
  const double hstep = PI / (double)(N - 1);
  auto itp11 = [&](double t) {  // linear_interpolation(range(0, π, Nθ), F11)
    double s = t / hstep;
    int j = (int)std::floor(s);
    if (j < 0) j = 0;
    if (j > N - 2) j = N - 2;
    const double w = s - j;
    return (1.0 - w) * F11[j] + w * F11[j + 1];
  };
  std::vector<double> xv(n + 1), yv(n + 1);
  double run = 0.0;
  for (int i = 0; i <= n; ++i) {  // xv = (0:n) ./ (n / π); yv = cumsum(itp11(xv) .* sin.(xv))
    xv[i] = (double)i / ((double)n / PI);
    run += itp11(xv[i]) * std::sin(xv[i]);
    yv[i] = run;
  }
  const double total = yv[n];
  for (int i = 0; i <= n; ++i) {
    xv[i] = PI - xv[i];
    yv[i] = 1.0 - yv[i] / total;
  }
  // swap roles: knots are the probabilities, values the cosines; then reverse both
  std::vector<double> kx(n + 1), ky(n + 1);
  for (int i = 0; i <= n; ++i) {
    kx[n - i] = yv[i];
    ky[n - i] = -std::cos(xv[i]);
  }
  // linear_interpolation(xv[2:end], yv[2:end]) evaluated at ex = (0:n) ./ n; the first
  // reversed knot duplicates the second (sin π rounds the last increment away)
  for (int j = 0; j <= n; ++j) {
    const double e = (double)j / (double)n;
    int lo = 1, hi = n;  // knots kx[1..n]; find the last k with kx[k] <= e, clamped to [1, n-1]
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (kx[mid] <= e) lo = mid;
      else hi = mid;
    }
    int k = lo;
    if (k > n - 1) k = n - 1;
    const double w = (e - kx[k]) / (kx[k + 1] - kx[k]);
    csrn[j] = (1.0 - w) * ky[k] + w * ky[k + 1];
  }
  return 0;
}

int orc_version(void) { return 2; }

}  // extern "C"
