// Host-side FP64 helpers: Mie table producer and the precomputation of the per-bin
// constants the kernels read. Everything here runs once per scatterer or per solve.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

namespace mcrt {
namespace host {

using cplx = std::complex<double>;
constexpr double PI = 3.14159265358979323846;
constexpr double EPS = 2.220446049250313e-16;

struct V3 {
  double x, y, z;
};
struct Sph {
  double ct, st, cp, sp;
};

// spherical_from_cartesian (src/utils.jl:9-23)
inline Sph spherical(V3 v) {
  double s2 = v.x * v.x + v.y * v.y;
  if (s2 < 1e-24) return {v.z > 0 ? 1.0 : (v.z < 0 ? -1.0 : 0.0), 0.0, 1.0, 0.0};
  double ct = v.z > 1 ? 1.0 : (v.z < -1 ? -1.0 : v.z);
  double si = 1.0 / std::sqrt(s2);
  return {ct, std::sqrt(1.0 - ct * ct), v.x * si, v.y * si};
}
// ray_to_norm (src/utils.jl:30-34)
inline V3 ray_to_norm(V3 x, const Sph& f) {
  return {x.x * f.ct * f.cp - x.y * f.sp + x.z * f.st * f.cp,
          x.x * f.ct * f.sp + x.y * f.cp + x.z * f.st * f.sp, -x.x * f.st + x.z * f.ct};
}
// norm_to_ray (src/utils.jl:41-45)
inline V3 norm_to_ray(V3 x, const Sph& f) {
  return {x.x * f.ct * f.cp + x.y * f.ct * f.sp - x.z * f.st, -x.x * f.sp + x.y * f.cp,
          x.x * f.st * f.cp + x.y * f.st * f.sp + x.z * f.ct};
}
// get_basis (src/utils.jl:52-62), Ev with the reference's y sign (src/utils.jl:60)
inline void get_basis(V3 k, V3& Eh, V3& Ev) {
  if (std::fabs(k.z) > 1.0 - EPS) {
    Eh = {0.0, -1.0, 0.0};
    Ev = {k.z > 0 ? 1.0 : (k.z < 0 ? -1.0 : 0.0), 0.0, 0.0};
  } else {
    double ev3 = -std::sqrt(1.0 - k.z * k.z);
    double inv = 1.0 / ev3;
    double eh1 = k.y * -inv, eh2 = k.x * inv;
    Eh = {eh1, eh2, 0.0};
    Ev = {-k.z * eh2, -k.z * eh1, ev3};
  }
}

// E_from_I (src/utils.jl:119-150): returns (E1re, E1im, E2re, E2im)
inline void E_from_I(const double I[4], double E[4]) {
  const double tol = 1e-14;
  double A1, A2, phi2;
  if (I[0] - std::fabs(I[1]) > tol * I[0]) {
    A1 = std::sqrt(0.5 * (I[0] - I[1]));
    A2 = std::sqrt(0.5 * (I[0] + I[1]));
    double q = std::sqrt(I[0] * I[0] - I[1] * I[1]);
    if (I[2] >= q) {
      phi2 = 0.0;
    } else if (I[2] <= -q) {
      phi2 = PI;
    } else {
      phi2 = std::acos(I[2] / q);
      if (I[3] > 0.0) phi2 = 2 * PI - phi2;
    }
  } else if (I[0] + I[1] <= tol * I[0]) {
    A1 = std::sqrt(I[0]);
    A2 = 0.0;
    phi2 = 0.0;
  } else {
    A1 = 0.0;
    A2 = std::sqrt(I[0]);
    phi2 = 0.0;
  }
  E[0] = A1;
  E[1] = 0.0;
  E[2] = A2 * std::cos(phi2);
  E[3] = A2 * std::sin(phi2);
}

struct MieResult {
  double q_ext, q_sca, q_abs, q_back, asymm;
  std::vector<cplx> S1, S2;
  std::vector<double> F11, F12, F33, F34;
};

// bhmie (src/scatterers/mie.jl:129-216): Bohren & Huffman's recurrences.
inline MieResult bhmie(double x, cplx m, int ntheta, int nextra = 15, int custom_nstop = 0) {
  cplx y = m * x;
  int nstop = custom_nstop ? custom_nstop
                           : (int)std::floor(std::max(x + 4 * std::cbrt(x) + 2, x * std::abs(m)));
  int nmax = nstop + nextra;
  std::vector<double> mu(ntheta);
  for (int i = 0; i < ntheta; ++i) {
    double th = ntheta > 1 ? PI * i / (ntheta - 1) : 0.0;
    mu[i] = std::cos(th);
  }
  std::vector<cplx> d(nmax + 1, cplx(0, 0));  // 1-based, d[nmax] = 0
  for (int n = nmax - 1; n >= 1; --n) d[n] = (double)(n + 1) / y - 1.0 / (d[n + 1] + (double)(n + 1) / y);
  std::vector<double> pi_(ntheta, 0.0), tau(ntheta, 0.0), pi0(ntheta, 0.0), pi1(ntheta, 1.0);
  MieResult R;
  R.S1.assign(ntheta, cplx(0, 0));
  R.S2.assign(ntheta, cplx(0, 0));
  double psi0 = std::cos(x), psi1 = std::sin(x), chi0 = -std::sin(x), chi1 = std::cos(x);
  cplx xi1(psi1, -chi1);
  cplx a(0, 0), b(0, 0);
  double q_sca = 0, asymm = 0;
  for (int n = 1; n <= nstop; ++n) {
    double fn = (2.0 * n + 1) / (n * (n + 1.0));
    double psi = (2.0 * n - 1) * psi1 / x - psi0;
    double chi = (2.0 * n - 1) * chi1 / x - chi0;
    cplx xi(psi, -chi);
    cplx an = ((d[n] / m + n / x) * psi - psi1);
    an /= ((d[n] / m + n / x) * xi - xi1);
    cplx bn = ((d[n] * m + n / x) * psi - psi1) / ((d[n] * m + n / x) * xi - xi1);
    q_sca += (std::norm(an) + std::norm(bn)) * (2 * n + 1);
    asymm += (an.real() * bn.real() + an.imag() * bn.imag()) * fn;
    if (n > 1)
      asymm += (a.real() * an.real() + a.imag() * an.imag() + b.real() * bn.real() + b.imag() * bn.imag()) *
               (n - 1.0) * (n + 1.0) / n;
    for (int i = 1; i <= (ntheta + 1) / 2; ++i) {
      int ii = ntheta + 1 - i;
      pi_[i - 1] = pi1[i - 1];
      tau[i - 1] = n * mu[i - 1] * pi_[i - 1] - (n + 1) * pi0[i - 1];
      R.S1[i - 1] += fn * (an * pi_[i - 1] + bn * tau[i - 1]);
      R.S2[i - 1] += fn * (an * tau[i - 1] + bn * pi_[i - 1]);
      if (i < ii) {
        double p = (n & 1) == 0 ? -1.0 : 1.0;
        R.S1[ii - 1] += fn * (an * pi_[i - 1] - bn * tau[i - 1]) * p;
        R.S2[ii - 1] += fn * (-an * tau[i - 1] + bn * pi_[i - 1]) * p;
      }
    }
    psi0 = psi1;
    psi1 = psi;
    chi0 = chi1;
    chi1 = chi;
    xi1 = cplx(psi1, -chi1);
    a = an;
    b = bn;
    for (int i = 0; i < ntheta; ++i) pi1[i] = ((2.0 * n + 1) * mu[i] * pi_[i] - (n + 1.0) * pi0[i]) / n;
    pi0 = pi_;
  }
  asymm *= 2 / q_sca;
  q_sca *= 2 / (x * x);
  R.q_ext = 4 / (x * x) * R.S1[0].real();
  R.q_sca = q_sca;
  R.q_abs = R.q_ext - q_sca;
  R.q_back = 4 / (x * x) * std::norm(R.S1[ntheta - 1]);
  R.asymm = asymm;
  double coeff = 4.0 / (q_sca * x * x);
  R.F11.resize(ntheta);
  R.F12.resize(ntheta);
  R.F33.resize(ntheta);
  R.F34.resize(ntheta);
  for (int i = 0; i < ntheta; ++i) {
    double a2 = std::norm(R.S1[i]), b2 = std::norm(R.S2[i]);
    cplx c = R.S2[i] * std::conj(R.S1[i]);
    R.F11[i] = (a2 + b2) * 0.5 * coeff;
    R.F12[i] = -(a2 - b2) * 0.5 * coeff;
    R.F33[i] = c.real() * coeff;
    R.F34[i] = c.imag() * coeff;
  }
  return R;
}

// Piecewise-linear interpolation on increasing knots (linear_interpolation).
inline double lerp_knots(const std::vector<double>& X, const std::vector<double>& Y, double x) {
  size_t n = X.size();
  if (x <= X[0]) return Y[0];
  if (x >= X[n - 1]) return Y[n - 1];
  size_t lo = 0, hi = n - 1;  // X[lo] <= x < X[hi]
  while (hi - lo > 1) {
    size_t mid = (lo + hi) / 2;
    if (X[mid] <= x)
      lo = mid;
    else
      hi = mid;
  }
  double dx = X[hi] - X[lo];
  double w = dx > 0 ? (x - X[lo]) / dx : 0.0;
  return Y[lo] + w * (Y[hi] - Y[lo]);
}

// calculate_csrn (src/utils.jl:263-287): inverse CDF of cos(theta) for the phase
// function F11 tabulated on the uniform grid 0..pi.
inline std::vector<double> calculate_csrn(const std::vector<double>& F11, int n) {
  int nt = (int)F11.size();
  auto itp11 = [&](double th) {
    double pos = th / (PI / (nt - 1));
    if (pos <= 0) return F11[0];
    if (pos >= nt - 1) return F11[nt - 1];
    int i = (int)std::floor(pos);
    double f = pos - i;
    return (1 - f) * F11[i] + f * F11[i + 1];
  };
  std::vector<double> xv(n + 1), yv(n + 1);
  double acc = 0;
  for (int i = 0; i <= n; ++i) {
    xv[i] = i / (n / PI);
    acc += itp11(xv[i]) * std::sin(xv[i]);
    yv[i] = acc;
  }
  double total = yv[n];
  std::vector<double> X(n + 1), Y(n + 1);
  for (int i = 0; i <= n; ++i) {
    double th = PI - xv[i];
    double p = 1 - yv[i] / total;
    X[i] = p;
    Y[i] = -std::cos(th);
  }
  std::reverse(X.begin(), X.end());
  std::reverse(Y.begin(), Y.end());
  std::vector<double> Xk(X.begin() + 1, X.end()), Yk(Y.begin() + 1, Y.end());
  std::vector<double> csrn(n + 1);
  for (int i = 0; i <= n; ++i) csrn[i] = lerp_knots(Xk, Yk, (double)i / n);
  return csrn;
}

}  // namespace host
}  // namespace mcrt
