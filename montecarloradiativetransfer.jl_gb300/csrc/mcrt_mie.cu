// Mie table producer on the device (see mcrt_mie.cuh). FP64 throughout: it runs once
// per scatterer, and its outputs must match the host producer to rounding.
#include "mcrt_mie.cuh"

namespace mcrt {
namespace {

constexpr double PI_M = 3.14159265358979323846;

struct Z {
  double re, im;
};
__device__ __forceinline__ Z operator+(Z a, Z b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ Z operator-(Z a, Z b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ Z operator-(Z a) { return {-a.re, -a.im}; }
__device__ __forceinline__ Z operator+(Z a, double s) { return {a.re + s, a.im}; }
__device__ __forceinline__ Z operator-(Z a, double s) { return {a.re - s, a.im}; }
__device__ __forceinline__ Z operator*(Z a, Z b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ Z operator*(Z a, double s) { return {a.re * s, a.im * s}; }
__device__ __forceinline__ Z operator*(double s, Z a) { return {s * a.re, s * a.im}; }
// Smith's algorithm (R. L. Smith, "Algorithm 116: Complex division", CACM 5(8), 1962).
__device__ __forceinline__ Z operator/(Z a, Z b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, den = b.re + b.im * r;
    return {(a.re + a.im * r) / den, (a.im - a.re * r) / den};
  }
  const double r = b.re / b.im, den = b.re * r + b.im;
  return {(a.re * r + a.im) / den, (a.im * r - a.re) / den};
}
__device__ __forceinline__ Z operator/(double a, Z b) { return Z{a, 0.0} / b; }
__device__ __forceinline__ double norm2(Z a) { return a.re * a.re + a.im * a.im; }

__global__ void __launch_bounds__(256) k_mie_tables(const MieJob* jobs) {
  const MieJob J = jobs[blockIdx.x];
  __shared__ double s_qsca;
  const double x = J.x;
  const Z m{J.m_re, J.m_im};
  const int nt = J.nt, rp = J.rp, tid = threadIdx.x, nthr = blockDim.x;
  double* out = J.out;
  double* F11 = out + 7;
  double* F12 = F11 + nt;
  double* F33 = F12 + nt;
  double* F34 = F33 + nt;
  double* S11 = F34 + nt;
  double* S22 = S11 + 2 * nt;
  double* csrn = S22 + 2 * nt;
  Z* ab = reinterpret_cast<Z*>(J.ab);

  // Coefficients a_n, b_n (mie.jl:133-171): D_n by downward recurrence from nmax, then
  // the Riccati-Bessel functions upward. Sequential; one thread.
  if (tid == 0) {
    const Z y = m * x;
    Z* d = reinterpret_cast<Z*>(J.d);
    d[J.nmax] = Z{0.0, 0.0};
    for (int n = J.nmax - 1; n >= 1; --n) d[n] = (double)(n + 1) / y - 1.0 / (d[n + 1] + (double)(n + 1) / y);
    double psi0 = cos(x), psi1 = sin(x), chi0 = -sin(x), chi1 = cos(x);
    Z xi1{psi1, -chi1};
    Z a{0.0, 0.0}, b{0.0, 0.0};
    double q_sca = 0.0, asymm = 0.0;
    for (int n = 1; n <= J.nstop; ++n) {
      const double fn = (2.0 * n + 1) / (n * (n + 1.0));
      const double psi = (2.0 * n - 1) * psi1 / x - psi0;
      const double chi = (2.0 * n - 1) * chi1 / x - chi0;
      const Z xi{psi, -chi};
      const Z t = d[n] / m + (double)n / x;
      const Z an = (t * psi - psi1) / (t * xi - xi1);
      const Z u = d[n] * m + (double)n / x;
      const Z bn = (u * psi - psi1) / (u * xi - xi1);
      q_sca += (norm2(an) + norm2(bn)) * (2 * n + 1);
      asymm += (an.re * bn.re + an.im * bn.im) * fn;
      if (n > 1) asymm += (a.re * an.re + a.im * an.im + b.re * bn.re + b.im * bn.im) * (n - 1.0) * (n + 1.0) / n;
      ab[2 * n] = an;
      ab[2 * n + 1] = bn;
      psi0 = psi1;
      psi1 = psi;
      chi0 = chi1;
      chi1 = chi;
      xi1 = Z{psi1, -chi1};
      a = an;
      b = bn;
    }
    asymm *= 2 / q_sca;
    q_sca *= 2 / (x * x);
    s_qsca = q_sca;
    out[6] = asymm;
  }
  __syncthreads();
  const double q_sca = s_qsca;
  const double coeff = 4.0 / (q_sca * x * x);

  // Amplitudes S1, S2 and the phase matrix per angle (mie.jl:173-192, 201-212): angle i and its
  // mirror nt + 1 - i share the angular functions pi_n, tau_n (1-based as the reference).
  auto store = [&](int k, Z s1, Z s2) {
    const double a2 = norm2(s1), b2 = norm2(s2);
    const Z c = s2 * Z{s1.re, -s1.im};
    F11[k] = (a2 + b2) * 0.5 * coeff;
    F12[k] = -(a2 - b2) * 0.5 * coeff;
    F33[k] = c.re * coeff;
    F34[k] = c.im * coeff;
    S11[2 * k] = s1.re;
    S11[2 * k + 1] = s1.im;
    S22[2 * k] = s2.re;
    S22[2 * k + 1] = s2.im;
    J.F[k] = make_float4((float)F11[k], (float)F12[k], (float)F33[k], (float)F34[k]);
    J.S[k] = make_float4((float)s1.re, (float)s1.im, (float)s2.re, (float)s2.im);
  };
  const int half = (nt + 1) / 2;
  for (int i = 1 + tid; i <= half; i += nthr) {
    const int ii = nt + 1 - i;
    const double mu = cos(nt > 1 ? PI_M * (i - 1) / (nt - 1) : 0.0);
    double pi0 = 0.0, pi1 = 1.0;
    Z s1{0.0, 0.0}, s2{0.0, 0.0}, s1m{0.0, 0.0}, s2m{0.0, 0.0};
    for (int n = 1; n <= J.nstop; ++n) {
      const double fn = (2.0 * n + 1) / (n * (n + 1.0));
      const Z an = ab[2 * n], bn = ab[2 * n + 1];
      const double pin = pi1;
      const double tau = n * mu * pin - (n + 1) * pi0;
      s1 = s1 + fn * (an * pin + bn * tau);
      s2 = s2 + fn * (an * tau + bn * pin);
      if (i < ii) {
        const double p = (n & 1) == 0 ? -1.0 : 1.0;
        s1m = s1m + fn * (an * pin - bn * tau) * p;
        s2m = s2m + fn * (-an * tau + bn * pin) * p;
      }
      pi1 = ((2.0 * n + 1) * mu * pin - (n + 1.0) * pi0) / n;
      pi0 = pin;
    }
    store(i - 1, s1, s2);
    if (i < ii) store(ii - 1, s1m, s2m);
  }
  __syncthreads();
  if (tid == 0) {
    const double q_ext = 4 / (x * x) * S11[0];
    out[0] = q_sca / q_ext;                         // omega (mie.jl:39)
    out[1] = ((4.0 / 3.0) * J.r) / (J.nu * q_ext);  // kl (mie.jl:40)
    out[2] = q_ext;
    out[3] = q_sca;
    out[4] = q_ext - q_sca;
    out[5] = 4 / (x * x) * (S11[2 * (nt - 1)] * S11[2 * (nt - 1)] + S11[2 * (nt - 1) + 1] * S11[2 * (nt - 1) + 1]);
    J.F[nt] = make_float4(0.f, 0.f, 0.f, 0.f);
    J.S[nt] = make_float4(0.f, 0.f, 0.f, 0.f);
  }

  // calculate_csrn (utils.jl:263-287): running integral of F11 sin(theta) on rp + 1
  // points, inverted by piecewise-linear interpolation at i / rp.
  double* term = J.terms;
  double* yv = J.terms + rp + 1;
  for (int i = tid; i <= rp; i += nthr) {
    const double xv = i / (rp / PI_M);
    const double pos = xv / (PI_M / (nt - 1));
    double f11;
    if (pos <= 0) {
      f11 = F11[0];
    } else if (pos >= nt - 1) {
      f11 = F11[nt - 1];
    } else {
      const int k = (int)floor(pos);
      const double f = pos - k;
      f11 = (1 - f) * F11[k] + f * F11[k + 1];
    }
    term[i] = f11 * sin(xv);
  }
  __syncthreads();
  if (tid == 0) {
    double acc = 0.0;  // the reference's summation order
    for (int i = 0; i <= rp; ++i) {
      acc += term[i];
      yv[i] = acc;
    }
  }
  __syncthreads();
  const double total = yv[rp];
  // knots j = 0 .. rp - 1: X = 1 - yv[rp - 1 - j] / total (increasing), Y = -cos(pi - xv)
  auto Xk = [&](int j) { return 1 - yv[rp - 1 - j] / total; };
  auto Yk = [&](int j) { return -cos(PI_M - (rp - 1 - j) / (rp / PI_M)); };
  for (int i = tid; i <= rp; i += nthr) {
    const double q = (double)i / rp;
    double v;
    if (q <= Xk(0)) {
      v = Yk(0);
    } else if (q >= Xk(rp - 1)) {
      v = Yk(rp - 1);
    } else {
      int lo = 0, hi = rp - 1;
      while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (Xk(mid) <= q)
          lo = mid;
        else
          hi = mid;
      }
      const double dx = Xk(hi) - Xk(lo);
      const double w = dx > 0 ? (q - Xk(lo)) / dx : 0.0;
      v = Yk(lo) + w * (Yk(hi) - Yk(lo));
    }
    csrn[i] = v;
    J.C[i] = (float)v;
  }
  __syncthreads();
  for (int i = rp + 1 + tid; i < J.nc; i += nthr) J.C[i] = i == rp + 1 ? (float)csrn[rp] : 0.0f;
}

}  // namespace

cudaError_t launch_mie_tables(const MieJob* jobs, int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_mie_tables<<<n, 256, 0, st>>>(jobs);
  return cudaGetLastError();
}

}  // namespace mcrt
