// Operation count of one bin evaluation of the reference's algorithm.
//
// TEST INFRASTRUCTURE ONLY. Instantiates the oracle's templated per-bin arithmetic
// (rt_bin: cpu.jl:13-26; cbn_bin: cpu.jl:85-126; cb1_bin: cpu.jl:132-156, with the
// update_I / update_E / frame functions of utils.jl they call) with a scalar type that
// counts its operations, and prints the mean counts per bin evaluation as JSON:
//   add  additions and subtractions (a fused multiply-add counts here and in mul,
//        so FMA = 2 flops), mul  multiplications, flops = add + mul;
//   div, sqrt, exp, sincos (one per sin or cos), acos, cbrt: the special-function
//        operations, counted separately; cmp  comparisons (branch tests, max).
// Sign flips and |x| are free (operand modifiers on the GPU) and are not counted.
// Usage: opcount [samples]. Inputs are seeded pseudo-random photon states in the
// workloads' geometries (a tau = 5 slab at 30 degrees zenith incidence, and the same
// slab for Rayleigh scatterers), with the reference's default bin grids.

#include <cstdio>
#include <cstdlib>
#include <random>

namespace opc {

struct Ops {
  double add = 0, mul = 0, div = 0, sqrt = 0, exp = 0, log = 0, sincos = 0, acos = 0, cbrt = 0, cmp = 0;
};
inline Ops& ops() {
  static Ops o;
  return o;
}

struct Counted {
  double v;
  Counted() : v(0.0) {}
  Counted(double x) : v(x) {}
};
inline Counted operator+(Counted a, Counted b) {
  ops().add += 1;
  return a.v + b.v;
}
inline Counted operator-(Counted a, Counted b) {
  ops().add += 1;
  return a.v - b.v;
}
inline Counted operator*(Counted a, Counted b) {
  ops().mul += 1;
  return a.v * b.v;
}
inline Counted operator/(Counted a, Counted b) {
  ops().div += 1;
  return a.v / b.v;
}
inline Counted operator-(Counted a) { return -a.v; }
inline Counted operator+(Counted a) { return a; }
inline Counted& operator+=(Counted& a, Counted b) { return a = a + b; }
inline Counted& operator-=(Counted& a, Counted b) { return a = a - b; }
inline Counted& operator*=(Counted& a, Counted b) { return a = a * b; }
inline Counted& operator/=(Counted& a, Counted b) { return a = a / b; }
inline bool cmp(bool r) {
  ops().cmp += 1;
  return r;
}
inline bool operator<(Counted a, Counted b) { return cmp(a.v < b.v); }
inline bool operator>(Counted a, Counted b) { return cmp(a.v > b.v); }
inline bool operator<=(Counted a, Counted b) { return cmp(a.v <= b.v); }
inline bool operator>=(Counted a, Counted b) { return cmp(a.v >= b.v); }
inline bool operator==(Counted a, Counted b) { return cmp(a.v == b.v); }
inline bool operator!=(Counted a, Counted b) { return cmp(a.v != b.v); }
inline Counted Sqrt(Counted x) {
  ops().sqrt += 1;
  return std::sqrt(x.v);
}
inline Counted Exp(Counted x) {
  ops().exp += 1;
  return std::exp(x.v);
}
inline Counted Log(Counted x) {
  ops().log += 1;
  return std::log(x.v);
}
inline Counted Cos(Counted x) {
  ops().sincos += 1;
  return std::cos(x.v);
}
inline Counted Sin(Counted x) {
  ops().sincos += 1;
  return std::sin(x.v);
}
inline Counted Acos(Counted x) {
  ops().acos += 1;
  return std::acos(x.v);
}
inline Counted Cbrt(Counted x) {
  ops().cbrt += 1;
  return std::cbrt(x.v);
}
inline Counted Fabs(Counted x) { return std::fabs(x.v); }
inline Counted Max(Counted a, Counted b) { return cmp(a.v > b.v) ? a : b; }
inline long Trunc(Counted x) { return (long)std::trunc(x.v); }

}  // namespace opc

#include <cmath>
#include <complex>

#include "mcrt_oracle.cpp"

namespace {

using opc::Counted;
using R = Counted;

struct Grid {
  std::vector<double> ct, st, w, cp, sp, ctb, stb, cpb, spb;
  int up0, up1;
};

// The reference's default bins for a plane (config.jl:55-124, plane.jl:131-142):
// Ntheta = 64 half-range Gauss-Legendre nodes, Nphi = 48, Nphi_b = 8, and 51
// backscattering polar angles up to 2 degrees (the count of DEFAULT_THEB).
Grid default_grid() {
  Grid G;
  const int nt = 64, h = nt / 2, np = 48, ntb = 51, npb = 8;
  // Gauss-Legendre nodes on [-1, 1] by Newton iteration on P_h.
  std::vector<double> x(h), w(h);
  for (int i = 0; i < h; ++i) {
    double z = std::cos(PI * (i + 0.75) / (h + 0.5)), dp = 0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1, p1 = z;
      for (int k = 2; k <= h; ++k) {
        double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = h * (z * p1 - p0) / (z * z - 1);
      double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-15) break;
    }
    x[i] = z;
    w[i] = 2 / ((1 - z * z) * dp * dp);
  }
  G.ct.resize(nt);
  G.w.resize(nt);
  for (int i = 0; i < h; ++i) {
    G.ct[i] = (x[i] - 1) / 2;
    G.w[i] = w[i] / 2 / (2 * np);
    G.ct[nt - 1 - i] = -G.ct[i];
    G.w[nt - 1 - i] = G.w[i];
  }
  for (double c : G.ct) G.st.push_back(std::sqrt(1 - c * c));
  for (int j = 0; j < np; ++j) {
    G.cp.push_back(std::cos(2 * PI * j / np));
    G.sp.push_back(std::sin(2 * PI * j / np));
  }
  for (int j = 0; j < ntb; ++j) {
    double t = 2.0 * PI / 180.0 * j / (ntb - 1);
    G.ctb.push_back(std::cos(t));
    G.stb.push_back(std::sin(t));
  }
  for (int j = 0; j < npb; ++j) {
    G.cpb.push_back(std::cos(2 * PI * j / npb));
    G.spb.push_back(std::sin(2 * PI * j / npb));
  }
  G.up0 = h;
  G.up1 = nt;
  return G;
}

Scat mie_like() {
  // Table values do not change the operation count; 1801 angles as in the workload.
  Scat s;
  s.kind = 1;
  s.ntheta = 1801;
  s.random_points = 1000;
  s.F11.assign(s.ntheta, 1.0);
  s.F12.assign(s.ntheta, -0.1);
  s.F33.assign(s.ntheta, 0.9);
  s.F34.assign(s.ntheta, 0.05);
  s.S11.assign(s.ntheta, cplx(1.0, 0.2));
  s.S22.assign(s.ntheta, cplx(0.8, -0.1));
  s.csrn.assign(s.random_points + 1, 0.0);
  return s;
}

V3T<R> rand_dir(std::mt19937_64& rng) {
  std::uniform_real_distribution<double> U(0.0, 1.0);
  double mu = 2 * U(rng) - 1, ph = 2 * PI * U(rng), s = std::sqrt(1 - mu * mu);
  return {R(s * std::cos(ph)), R(s * std::sin(ph)), R(mu)};
}

V4T<R> rand_stokes(std::mt19937_64& rng) {
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  double q = 0.5 * U(rng), u = 0.5 * U(rng), v = 0.5 * U(rng);
  return {{R(1.0), R(q), R(u), R(v)}};
}

std::complex<R> rand_c(std::mt19937_64& rng) {
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  return {R(U(rng)), R(U(rng))};
}

struct Mean {
  opc::Ops sum;
  double n = 0;
  void add(const opc::Ops& o, double bins) {
    sum.add += o.add;
    sum.mul += o.mul;
    sum.div += o.div;
    sum.sqrt += o.sqrt;
    sum.exp += o.exp;
    sum.log += o.log;
    sum.sincos += o.sincos;
    sum.acos += o.acos;
    sum.cbrt += o.cbrt;
    sum.cmp += o.cmp;
    n += bins;
  }
  void print(const char* name, bool last) const {
    auto m = [&](double v) { return v / n; };
    std::printf(
        "  \"%s\": {\"flops\": %.3f, \"add\": %.3f, \"mul\": %.3f, \"div\": %.3f, \"sqrt\": %.3f, "
        "\"exp\": %.3f, \"log\": %.3f, \"sincos\": %.3f, \"acos\": %.3f, \"cbrt\": %.3f, \"cmp\": %.3f}%s\n",
        name, m(sum.add + sum.mul), m(sum.add), m(sum.mul), m(sum.div), m(sum.sqrt), m(sum.exp), m(sum.log),
        m(sum.sincos), m(sum.acos), m(sum.cbrt), m(sum.cmp), last ? "" : ",");
  }
};

}  // namespace

int main(int argc, char** argv) {
  const int samples = argc > 1 ? std::atoi(argv[1]) : 200;
  const Grid G = default_grid();
  Geom g;
  g.kind = 0;
  g.layers.push_back({5.0, 0.99, false, 0});
  const double tau0 = 50.0;
  std::mt19937_64 rng(20240601);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  std::printf("{\n");
  for (int kind = 0; kind < 2; ++kind) {
    g.scats.clear();
    if (kind == 0) {
      Scat s;
      s.kind = 0;
      g.scats.push_back(s);
    } else {
      g.scats.push_back(mie_like());
    }
    const Scat& sca = g.scats[0];
    Mean rt, cbn, cb1;
    for (int it = 0; it < samples; ++it) {
      V3T<R> k = rand_dir(rng), x{R(0.0), R(0.0), R(-5.0 * U(rng))};
      V4T<R> I = rand_stokes(rng);
      SphT<R> ks = spherical_from_cartesian(k);
      opc::ops() = opc::Ops();
      for (int j2 = 0; j2 < (int)G.cp.size(); ++j2)
        for (int j1 = G.up0; j1 < G.up1; ++j1) {
          V4T<R> o;
          rt_bin(sca, g, tau0, I, ks, x, 0, R(G.st[j1]), R(G.ct[j1]), R(G.cp[j2]), R(G.sp[j2]), R(G.w[j1]), o);
        }
      rt.add(opc::ops(), (double)G.cp.size() * (G.up1 - G.up0));

      // reciprocal-path and single-scattering CB bins around the backscattering direction
      V3T<R> kf = {R(0.5), R(0.0), R(std::sqrt(0.75))};
      CBNIn<R> e{spherical_from_cartesian(kf), ks, spherical_from_cartesian(rand_dir(rng)), rand_dir(rng), x,
                 V3T<R>{R(U(rng)), R(U(rng)), R(-5.0 * U(rng))}, 0, 0, R(100.0), R(0.3 * U(rng)),
                 rand_c(rng), rand_c(rng), rand_c(rng), rand_c(rng)};
      opc::ops() = opc::Ops();
      for (int j2 = 0; j2 < (int)G.cpb.size(); ++j2)
        for (int j1 = 0; j1 < (int)G.ctb.size(); ++j1) {
          V4T<R> o;
          R lad;
          cbn_bin(sca, g, tau0, e, R(G.stb[j1]), R(G.ctb[j1]), R(G.cpb[j2]), R(G.spb[j2]), o, lad);
        }
      cbn.add(opc::ops(), (double)G.cpb.size() * G.ctb.size());
      opc::ops() = opc::Ops();
      for (int j2 = 0; j2 < (int)G.cpb.size(); ++j2)
        for (int j1 = 0; j1 < (int)G.ctb.size(); ++j1) {
          V4T<R> o;
          cb1_bin(sca, g, tau0, I, e.kfs, ks, x, 0, R(G.stb[j1]), R(G.ctb[j1]), R(G.cpb[j2]), R(G.spb[j2]), o);
        }
      cb1.add(opc::ops(), (double)G.cpb.size() * G.ctb.size());
    }
    std::printf(" \"%s\": {\n", kind == 0 ? "rayleigh" : "mie");
    rt.print("rt_bin", false);
    cbn.print("cb_reciprocal_bin", false);
    cb1.print("cb_single_bin", true);
    std::printf(" }%s\n", kind == 0 ? "," : "");
  }
  std::printf("}\n");
  return 0;
}
