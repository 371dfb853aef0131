// Plain per-ray kernel: the structure of the reference's gpu_kernel
// (MonteCarloRadiativeTransfer.jl src/gpu.jl:177-296) written in CUDA C++.
//
// One thread per ray in a grid-stride loop, path history (kpath, xpath, idxpath) in
// global memory, the reciprocal-path fields rebuilt by walking the whole path at every
// CB event (src/utils.jl:199-241), and one global FP64 atomic per Stokes component per
// bin per event (src/gpu.jl:24-27, :135-138, :167-170). All arithmetic is in T.
// It is the baseline the persistent kernel is measured against and a second,
// independent check of it; it draws the same Philox streams.
#pragma once

#include "mcrt_device.cuh"

namespace mcrt {

struct PlainParams {
  const DevInstance* inst;
  double* kpath;   // [maxorders + 1][threads][3] in T (reinterpreted)
  double* xpath;
  int* idxpath;
  long long threads;
  long long maxord;
  unsigned* status;
};

template <typename T>
struct PV3 {
  T x, y, z;
};

template <typename T>
__device__ __forceinline__ T plain_dist(const DevInstance& in, PV3<T> x, PV3<T> k, int idx) {
  if (in.geom == 0) {
    if (k.z > T(0)) return -x.z / k.z;
    if (!in.layers[idx].inf) return (x.z + (T)in.layers[idx].tau) / -k.z;
    return (T)INFINITY;
  }
  T kx = k.x * x.x + k.y * x.y + k.z * x.z, xx = x.x * x.x + x.y * x.y + x.z * x.z;
  T tau = (T)in.layers[0].tau;
  T D = kx * kx + tau * tau - xx;
  return -kx + MT<T>::sqrt(D > T(0) ? D : T(0));
}

// get_basis (src/utils.jl:52-62) including its Ev, used by the CB bins' final rotation.
template <typename T>
__device__ __forceinline__ void plain_basis(PV3<T> k, PV3<T>& Eh, PV3<T>& Ev) {
  if (MT<T>::fabs(k.z) > T(1) - (T)2.220446049250313e-16) {
    Eh = {T(0), T(-1), T(0)};
    Ev = {k.z > T(0) ? T(1) : (k.z < T(0) ? T(-1) : T(0)), T(0), T(0)};
  } else {
    T ev3 = -MT<T>::sqrt(T(1) - k.z * k.z);
    T inv = T(1) / ev3;
    T eh1 = k.y * -inv, eh2 = k.x * inv;
    Eh = {eh1, eh2, T(0)};
    Ev = {-k.z * eh2, -k.z * eh1, ev3};
  }
}

template <typename T>
__device__ __forceinline__ Frame<T> plain_sph(PV3<T> x) {
  T s2 = x.x * x.x + x.y * x.y;
  if (s2 < T(1e-24)) return Frame<T>{x.z > T(0) ? T(1) : (x.z < T(0) ? T(-1) : T(0)), T(0), T(1), T(0)};
  T ct = clamp1(x.z);
  T si = T(1) / MT<T>::sqrt(s2);
  return Frame<T>{ct, MT<T>::sqrt(T(1) - ct * ct), x.x * si, x.y * si};
}

template <typename T>
__device__ __forceinline__ PV3<T> plain_r2n(PV3<T> v, const Frame<T>& f) {
  PV3<T> o;
  ray_to_norm(f, v.x, v.y, v.z, o.x, o.y, o.z);
  return o;
}

template <typename T>
__device__ __forceinline__ PV3<T> plain_n2r(PV3<T> v, const Frame<T>& f) {
  PV3<T> o;
  norm_to_ray(f, v.x, v.y, v.z, o.x, o.y, o.z);
  return o;
}

// update_I as written in src/utils.jl:91-112 (recomputes the ray-frame direction).
template <typename T>
__device__ __forceinline__ void plain_update_I(const DevScatterer& s, const T I[4], PV3<T> k,
                                               const Frame<T>& f, T out[4]) {
  PV3<T> Eh, Ev;
  plain_basis(k, Eh, Ev);
  update_I<T>(f, I, k.x, k.y, k.z, Eh.x, Eh.y, s.kind, s.F, s.ntheta, table_scale<T>(s), out);
}

template <typename T>
__device__ __forceinline__ void plain_update_E(const DevScatterer& s, T E[4], PV3<T> k,
                                               const Frame<T>& f) {
  PV3<T> Eh, Ev;
  plain_basis(k, Eh, Ev);
  update_E<T>(f, E, k.x, k.y, k.z, Eh.x, Eh.y, s.kind, s.S, s.ntheta, table_scale<T>(s));
}

template <typename T>
__global__ void __launch_bounds__(256) k_plain(PlainParams p) {
  const DevInstance& in = *p.inst;
  const BinTables<T>& B = *reinterpret_cast<const BinTables<T>*>(in.bins);
  const long long nid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)blockDim.x * gridDim.x;
  if (nid >= p.threads) return;
  PV3<T>* kpath = reinterpret_cast<PV3<T>*>(p.kpath);
  PV3<T>* xpath = reinterpret_cast<PV3<T>*>(p.xpath);
  const DevScatterer& s1 = in.scat[in.layers[0].scat];
  const T tau0 = (T)in.tau0;
  const Frame<T> inc{(T)in.inc[0], (T)in.inc[1], (T)in.inc[2], (T)in.inc[3]};
  const PV3<T> k0{(T)in.k0[0], (T)in.k0[1], (T)in.k0[2]};
  double lacc[NACC];
  for (int i = 0; i < NACC; ++i) lacc[i] = 0.0;

  for (long long r = nid; r < in.n_photons; r += stride) {
    const unsigned long long ph = (unsigned long long)(in.photon_begin + r);
    T I[4] = {(T)in.I0[0], (T)in.I0[1], (T)in.I0[2], (T)in.I0[3]};
    PV3<T> k = k0, x{T(0), T(0), T(0)};
    int idx = 0, n = 0;
    double peak = 0.0;
    Draw d0 = draw(in.key0, in.key1, ph, 0, 0);
    T tau1 = (T)in.layers[0].tau;
    if (in.geom == 1) {
      T rr = tau1 * MT<T>::sqrt(u01<T>(d0.r[0]));
      T phi = (T)(2 * PI_D) * u01<T>(d0.r[1]);
      T s, c;
      MT<T>::sincos(phi, &s, &c);
      x = {rr * c, rr * s, MT<T>::sqrt(tau1 * tau1 - rr * rr)};
    }
    bool cdt = in.geom == 1 || (in.n_layers == 1 && !in.layers[0].inf);
    if (cdt) {  // src/gpu.jl:196-201
      T tp = plain_dist(in, x, k, 0);
      T dt = tp <= tau0 ? MT<T>::exp(-tp) : T(0);
      atomicAdd(in.acc + ACC_ADT, (double)(I[0] * dt));
      for (int s = 0; s < 4; ++s) I[s] *= T(1) - dt;
    }
    {  // initial_propagation (plane.jl:77-95, sphere.jl:54-67)
      T u2 = in.rng_mode == 1 ? (T)(((double)ph + 0.5) / (double)in.nrays) : u01<T>(d0.r[2]);
      T t;
      if (in.geom == 0) {
        if (in.layers[0].inf) {
          t = -MT<T>::log(u2);
        } else {
          T tp = plain_dist(in, x, k, 0);
          if (cdt && tp <= tau0) {
            t = -MT<T>::log(T(1) - u2 * (T(1) - MT<T>::exp(-tp)));
          } else {
            t = tp + T(1);
            for (unsigned a = 0; t > tp; ++a) {
              if ((long long)a >= in.max_attempts) {
                atomicOr(p.status, 1u);
                t = tp;
                break;
              }
              T u = a == 0 ? u2 : u01<T>(draw(in.key0, in.key1, ph, 0, a).r[2]);
              t = -MT<T>::log(u);
            }
          }
        }
      } else {
        T tp = T(2) * x.z;
        if (tp <= tau0) {
          t = -MT<T>::log(T(1) - u2 * (T(1) - MT<T>::exp(-tp)));
        } else {
          t = tp + T(1);
          for (unsigned a = 0; t > tp; ++a) {
            if ((long long)a >= in.max_attempts) {
              atomicOr(p.status, 1u);
              t = tp;
              break;
            }
            uint32_t rr = a == 0 ? d0.r[2] : draw(in.key0, in.key1, ph, 0, a).r[2];
            T uc = in.rng_mode == 1 && a == 0 ? T(1) - u2 : u01<T>(~rr);
            t = -MT<T>::log(uc);
          }
        }
      }
      x = {x.x + t * k.x, x.y + t * k.y, x.z + t * k.z};
    }
    bool dead = false;
    while (I[0] >= (T)in.min_int && n < in.max_scat) {
      ++n;
      const size_t slot = (size_t)n * p.threads + nid;
      kpath[slot] = k;
      xpath[slot] = x;
      p.idxpath[slot] = idx;
      // rejection loop (src/gpu.jl:215-256)
      const DevLayer& L = in.layers[idx];
      const DevScatterer& sc = in.scat[L.scat];
      const Frame<T> ks = plain_sph(k);
      T Ip[4];
      PV3<T> kp = k, xp = x;
      int idxp = idx;
      unsigned a = 0;
      int kcap = 0;
      for (;; ++a) {
        if ((long long)a >= in.max_attempts) {
          atomicOr(p.status, 1u);
          dead = true;
          break;
        }
        Draw d = draw(in.key0, in.key1, ph, (uint32_t)n, a);
        T u0 = u01<T>(d.r[0]), u1 = u01<T>(d.r[1]), u2 = u01<T>(d.r[2]);
        T mu;
        if (sc.kind == 0) {  // rayleigh.jl:10-11 as written
          T rn = T(2) * (T(1) - T(2) * u0);
          T b = MT<T>::sqrt(T(1) + rn * rn);
          mu = MT<T>::cbrt(b + rn) - MT<T>::cbrt(b - rn);
        } else {
          mu = sample_mu<T>(1, sc.csrn, sc.rp, u0);
        }
        PMat<T> P = phase_eval<T>(sc.kind, sc.F, sc.ntheta, table_scale<T>(sc), mu);
        T eq = -P.p12 * I[1] / (P.p11 * I[0]), eu = -P.p12 * I[2] / (P.p11 * I[0]);
        T ee = MT<T>::sqrt(eq * eq + eu * eu);
        T phi;
        if (ee > T(1e-12)) {
          T gam = MT<T>::acos(clamp1(eq / ee));
          if (eu < T(0)) gam = (T)(2 * PI_D) - gam;
          T sg, cg;
          MT<T>::sincos(gam, &sg, &cg);
          T ma = (T)(4 * PI_D) * u1 + gam - ee * sg;
          phi = T(0.5) * (kepler<T>(ma, ee, kcap) - gam);
        } else {
          phi = (T)(2 * PI_D) * u1;
        }
        T st = MT<T>::sqrt(fmax(T(1) - mu * mu, T(0)));
        T sp, cp;
        MT<T>::sincos(phi, &sp, &cp);
        kp = plain_r2n(PV3<T>{st * cp, st * sp, mu}, ks);
        plain_update_I(sc, I, kp, ks, Ip);
        T sc1 = I[0] / Ip[0];
        for (int s = 0; s < 4; ++s) Ip[s] *= sc1;
        T t = -MT<T>::log(u2);
        xp = {x.x + t * kp.x, x.y + t * kp.y, x.z + t * kp.z};
        int pb;
        if (in.geom == 0)
          pb = xp.z > T(0) ? -1 : ((!L.inf && xp.z < -(T)L.tau) ? 1 : 0);
        else
          pb = MT<T>::sqrt(xp.x * xp.x + xp.y * xp.y + xp.z * xp.z) > (T)in.layers[0].tau ? -2 : 0;
        idxp = idx + pb;
        if (pb == -2) continue;
        if (pb == -1) {
          if (idxp < 0) continue;
          xp = {x.x, x.y, -(T)L.tau};
          break;
        }
        if (pb == 1) {
          if (idxp > in.n_layers - 1) continue;
          xp = {x.x, x.y, T(0)};
          break;
        }
        break;
      }
      if (dead) break;
      if (kcap) atomicOr(p.status, 2u);
      lacc[ACC_EVENTS] += 1;
      lacc[ACC_ATTEMPTS] += a + 1;
      const T om = (T)L.omega;
      atomicAdd(in.acc + ACC_AABS, (double)((T(1) - om) * I[0]));
      for (int s = 0; s < 4; ++s) I[s] *= om;
      T Iref = T(0), Itrans = T(0);
      T mdf, mdl;
      if (in.geom == 0) {
        mdf = idx == 0 ? MT<T>::fabs(x.z) : (T)INFINITY;
        mdl = (idx == in.n_layers - 1 && !L.inf) ? (T)L.tau - MT<T>::fabs(x.z) : (T)INFINITY;
      } else {
        mdf = (T)in.layers[0].tau - MT<T>::sqrt(x.x * x.x + x.y * x.y + x.z * x.z);
        mdl = (T)INFINITY;
      }
      const bool up = mdf <= tau0, dn = mdl <= tau0;
      // ---- CB (src/gpu.jl:41-175)
      if (in.compute_cb && (up || dn)) {
        const Frame<T> kas = plain_sph(k);
        const PV3<T> k1 = kpath[(size_t)1 * p.threads + nid];
        const PV3<T> kf0{-k1.x, -k1.y, -k1.z};
        const Frame<T> kfs = plain_sph(kf0);
        if (n > 1) {
          const PV3<T> xb = xpath[(size_t)1 * p.threads + nid];
          const int idxb = p.idxpath[(size_t)1 * p.threads + nid];
          const PV3<T> k2 = kpath[(size_t)2 * p.threads + nid];
          const Frame<T> kbs = plain_sph(PV3<T>{-k2.x, -k2.y, -k2.z});
          T ta = plain_dist(in, x, kf0, idx), tb = plain_dist(in, xb, kf0, idxb), tab = ta - tb;
          T Iaf[4];
          plain_update_I(s1, I, kf0, kas, Iaf);
          T Ea[4] = {(T)in.Ei[0], (T)in.Ei[1], (T)in.Ei[2], (T)in.Ei[3]};
          T Eb[4] = {Ea[0], Ea[1], Ea[2], Ea[3]};
          const T norm0 = MT<T>::sqrt(Ea[0] * Ea[0] + Ea[1] * Ea[1] + Ea[2] * Ea[2] + Ea[3] * Ea[3]);
          T enorma = T(0), enormb = T(0);
          Frame<T> f = inc;
          for (int j = 2; j <= n; ++j) {  // forward_E
            const PV3<T> kj = kpath[(size_t)j * p.threads + nid];
            plain_update_E(s1, Ea, kj, f);
            T n2 = MT<T>::sqrt(Ea[0] * Ea[0] + Ea[1] * Ea[1] + Ea[2] * Ea[2] + Ea[3] * Ea[3]);
            for (int s = 0; s < 4; ++s) Ea[s] *= norm0 / n2;
            enorma += MT<T>::log(norm0 / n2);
            f = plain_sph(kj);
          }
          f = inc;
          for (int j = n; j >= 2; --j) {  // backward_E
            const PV3<T> kj = kpath[(size_t)j * p.threads + nid];
            const PV3<T> mk{-kj.x, -kj.y, -kj.z};
            plain_update_E(s1, Eb, mk, f);
            T n2 = MT<T>::sqrt(Eb[0] * Eb[0] + Eb[1] * Eb[1] + Eb[2] * Eb[2] + Eb[3] * Eb[3]);
            for (int s = 0; s < 4; ++s) Eb[s] *= norm0 / n2;
            enormb += MT<T>::log(norm0 / n2);
            f = plain_sph(mk);
          }
          const T sc = MT<T>::exp(enorma - enormb);
          for (int s = 0; s < 4; ++s) Eb[s] *= sc;
          T Eaf[4] = {Ea[0], Ea[1], Ea[2], Ea[3]};
          plain_update_E(s1, Eaf, kf0, kas);
          // src/gpu.jl:84, with a slightly negative rounded intensity (90-degree Rayleigh
          // scattering of a fully polarised photon) or a vanishing field clamped to zero.
          const T nef = Eaf[0] * Eaf[0] + Eaf[1] * Eaf[1] + Eaf[2] * Eaf[2] + Eaf[3] * Eaf[3];
          const T raa = nef > T(0) ? MT<T>::sqrt(fmax(Iaf[0], T(0)) / nef) : T(0);
          for (int s = 0; s < 4; ++s) {
            Ea[s] *= raa;
            Eb[s] *= raa;
          }
          const T kl = (T)in.kl1;
          for (int j2 = 0; j2 < B.nphib; ++j2) {
            for (int j1 = 0; j1 < B.nthetab; ++j1) {
              // The bin direction, recomputed per bin as src/gpu.jl:92-94 does.
              const size_t b = (size_t)j2 * B.nthetab + j1;
              const PV3<T> kf = plain_r2n(
                  PV3<T>{B.stb[j1] * B.cpb[j2], B.stb[j1] * B.spb[j2], B.ctb[j1]}, kfs);
              T a4[4] = {Ea[0], Ea[1], Ea[2], Ea[3]}, b4[4] = {Eb[0], Eb[1], Eb[2], Eb[3]};
              plain_update_E(s1, a4, kf, kas);
              PV3<T> Eh, Ev;
              plain_basis(kf, Eh, Ev);
              plain_update_E(s1, b4, kf, kbs);
              const T dphi = kl * ((k1.x + kf.x) * (x.x - xb.x) + (k1.y + kf.y) * (x.y - xb.y) +
                                   (k1.z + kf.z) * (x.z - xb.z));
              const T tya = plain_dist(in, x, kf, idx);
              if (tya <= tau0) {
                const T na = MT<T>::exp(T(-0.5) * tya);
                for (int s = 0; s < 4; ++s) a4[s] *= na;
                const T Ia0 = a4[0] * a4[0] + a4[1] * a4[1] + a4[2] * a4[2] + a4[3] * a4[3];
                const T tyb = plain_dist(in, xb, kf, idxb);
                if (MT<T>::fabs(tyb + tab) <= tau0) {
                  const T nb = MT<T>::exp(T(-0.5) * (tyb + tab));
                  for (int s = 0; s < 4; ++s) b4[s] *= nb;
                } else {
                  for (int s = 0; s < 4; ++s) b4[s] = T(0);
                }
                const T Ib0 = b4[0] * b4[0] + b4[1] * b4[1] + b4[2] * b4[2] + b4[3] * b4[3];
                T sn, cs;
                MT<T>::sincos(dphi, &sn, &cs);
                const T c1r = a4[0] * cs - a4[1] * sn + b4[0], c1i = a4[0] * sn + a4[1] * cs + b4[1];
                const T c2r = a4[2] * cs - a4[3] * sn + b4[2], c2i = a4[2] * sn + a4[3] * cs + b4[3];
                const T qh = c1r * c1r + c1i * c1i, qv = c2r * c2r + c2i * c2i;
                const T scl = Ia0 / (Ia0 + Ib0);
                T S[4] = {(qh + qv) * scl, (qv - qh) * scl, T(2) * (c2r * c1r + c2i * c1i) * scl,
                          T(-2) * (c2i * c1r - c2r * c1i) * scl};
                const PV3<T> eh = plain_n2r(Eh, kfs), ev = plain_n2r(Ev, kfs);
                const T cpsi = B.spb[j2] * eh.x - B.cpb[j2] * eh.y;
                const T spsi = -B.spb[j2] * ev.x + B.cpb[j2] * ev.y;
                rotate(cpsi * cpsi - spsi * spsi, T(2) * cpsi * spsi, S[1], S[2]);
                double* dst = in.Icb + 4 * b;
                for (int s = 0; s < 4; ++s) atomicAdd(dst + s, (double)S[s]);
                atomicAdd(in.ladder + b, (double)Ia0);
                if (b == 0) peak += (double)S[0];
              }
            }
          }
          lacc[ACC_CBN] += (double)B.nphib * B.nthetab;
        } else {
          for (int j2 = 0; j2 < B.nphib; ++j2) {
            for (int j1 = 0; j1 < B.nthetab; ++j1) {
              const size_t b = (size_t)j2 * B.nthetab + j1;
              const PV3<T> kf = plain_r2n(
                  PV3<T>{B.stb[j1] * B.cpb[j2], B.stb[j1] * B.spb[j2], B.ctb[j1]}, kfs);
              T o[4];
              PV3<T> Eh, Ev;
              plain_basis(kf, Eh, Ev);
              plain_update_I(s1, I, kf, kas, o);
              const T tya = plain_dist(in, x, kf, idx);
              if (tya <= tau0) {
                const T na = MT<T>::exp(-tya);
                for (int s = 0; s < 4; ++s) o[s] *= na;
                const PV3<T> eh = plain_n2r(Eh, kfs), ev = plain_n2r(Ev, kfs);
                const T cpsi = B.spb[j2] * eh.x - B.cpb[j2] * eh.y;
                const T spsi = -B.spb[j2] * ev.x + B.cpb[j2] * ev.y;
                rotate(cpsi * cpsi - spsi * spsi, T(2) * cpsi * spsi, o[1], o[2]);
                double* dst = in.Icb + 4 * b;
                for (int s = 0; s < 4; ++s) atomicAdd(dst + s, (double)o[s]);
                atomicAdd(in.ladder + b, (double)o[0]);
                if (b == 0) peak += (double)o[0];
              }
            }
          }
          lacc[ACC_CB1] += (double)B.nphib * B.nthetab;
        }
      }
      // ---- RT (src/gpu.jl:6-34)
      for (int rng = 0; rng < 2; ++rng) {
        if (!(rng == 0 ? up : dn)) continue;
        const int r0 = rng == 0 ? B.up0 : B.lo0, r1 = rng == 0 ? B.up1 : B.lo1;
        const Frame<T> ksr = plain_sph(k);
        T accv = T(0);
        for (int j2 = 0; j2 < B.nphi; ++j2) {
          for (int j1 = r0; j1 < r1; ++j1) {
            const PV3<T> kk{B.st[j1] * B.cp[j2], B.st[j1] * B.sp[j2], B.ct[j1]};
            T o[4];
            plain_update_I(sc, I, kk, ksr, o);
            const T t = plain_dist(in, x, kk, idx);
            if (t <= tau0) {
              const T w = B.w[j1] * MT<T>::exp(-t);
              double* dst = in.Irt + 4 * ((size_t)j2 * B.ntheta + j1);
              for (int s = 0; s < 4; ++s) atomicAdd(dst + s, (double)(o[s] * w));
              accv += o[0] * w;
            }
          }
        }
        lacc[ACC_RT] += (double)B.nphi * (r1 - r0);
        if (rng == 0)
          Iref = accv;
        else
          Itrans = accv;
      }
      atomicAdd(in.acc + ACC_AREF, (double)Iref);
      atomicAdd(in.acc + ACC_ATRANS, (double)Itrans);
      const T Iesc = Iref + Itrans;
      const T sc2 = (I[0] - Iesc) / Ip[0];
      for (int s = 0; s < 4; ++s) I[s] = Ip[s] * sc2;
      k = kp;
      x = xp;
      idx = idxp;
    }
    if (!dead) {
      atomicAdd(in.acc + ACC_AREM, (double)I[0]);
      lacc[ACC_PEAK] += peak;
      lacc[ACC_PEAK2] += peak * peak;
    }
    lacc[ACC_PHOTONS] += 1;
  }
  for (int i = ACC_PEAK; i < NACC; ++i)
    if (lacc[i] != 0.0) atomicAdd(in.acc + i, lacc[i]);
}

}  // namespace mcrt
