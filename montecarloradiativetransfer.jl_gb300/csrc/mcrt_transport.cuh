// Persistent event-batched transport kernel.
//
// Replaces the reference's per-ray gpu_kernel (MonteCarloRadiativeTransfer.jl
// src/gpu.jl:177-296) with the same physics organised for sm_103a:
//
//  * One thread owns one photon path at a time and, in a *sample* phase, advances it
//    by one scattering event: Philox draws, scatter(), the free-path rejection loop,
//    absorption, and the incremental reciprocal-path (CB) state (src/gpu.jl:207-260).
//    The event's parameters go to shared memory.
//  * In the *collect* phase the whole block sweeps the peel-off bins. Lanes own bins,
//    not photons: a warp takes a tile of 32 x NB bins (RT: one azimuth and NB polar
//    angles per lane; CB: one bin pair per lane) and loops over every event of the
//    batch, reading the event (a shared-memory broadcast) and accumulating the bins'
//    Stokes contributions in registers. This is src/gpu.jl:6-34 (RT) and :41-175 (CB)
//    with the event loop and the bin loop exchanged, so tallies need no atomics per
//    contribution: each lane flushes its bins once per batch with FP64 reductions.
//    The per-event escaped intensity (the return value of collect_rt_gpu!) is summed
//    with __shfl_xor_sync across the warp and added per warp into shared memory.
//    For Rayleigh slabs the RT lanes own polar bins and tally the exact azimuthal
//    Fourier modes of the peel-off instead (rt_fourier_tile).
//  * The *finish* phase renormalises each photon by its escaped intensity
//    (src/gpu.jl:288-291), ends finished paths and claims new photons from the
//    instance's work queue (a global counter, claimed warp-aggregated).
//
// Work: one launch serves any number of instances (simulate() calls). Blocks start
// spread over the instances in proportion to their photons; a block works on one
// instance at a time and moves on (cyclically) when the current one has no photons left
// to claim, so uneven batches run in one persistent launch.
#pragma once

#include <type_traits>

#include "mcrt_device.cuh"

namespace mcrt {

constexpr int EV_UP = 1, EV_DN = 2, EV_CB = 4, EV_CBN = 8;

template <typename T>
struct __align__(16) EventP {
  T I[4];                 // Stokes after absorption
  T fct, fst, fcp, fsp;   // spherical frame of the incoming direction (ka)
  T a_up, a_dn;           // plane: distance numerators of xa (up: -z, down: z + tau)
  T xax, xay, xaz, Da;    // sphere: xa and tau^2 - |xa|^2
  T bct, bst, bcp, bsp;   // CB: frame of kb = -k_2
  T ea[4], eb[4];         // CB: reciprocal-path fields at xa and xb
  T b_up, b_dn, tab2;     // CB: distance numerators of xb; (tau_a - tau_b) * log2(e)
  T v1, v2, v3;           // CB: phase coefficients, kl (xa - xb) in the backscatter frame / 2 pi
  T xbx, xby, xbz, Db;    // CB sphere: xb and tau^2 - |xb|^2
  int flags, layer, pad0, pad1;
};

template <typename T>
struct __align__(16) PState {
  double x[3], x1[3];
  double logA, logL, peak;
  unsigned long long id;
  T I[4];
  T k[3], wI;
  T Ih[4];
  T k2[3], pad0;
  T kprev[3], pad1;
  T A[4];
  T L[8];
  int n, idx, idx1, pad2;
};

template <typename T, int BS>
struct __align__(16) Shared {
  DevInstance inst;
  EventP<T> ev[BS];
  T esc_up[BS], esc_dn[BS], peak[BS];
  unsigned short list[4][BS];  // 0 up, 1 down, 2 CB order > 1, 3 CB order 1
  int cnt[2][4];
  int item_next;
  int cur;
  int exhausted;
  int taken;   // photons of the current instance this block claimed in this launch
  int expand;  // this block finished the instance's last photon (Fourier expansion)
};

struct KParams {
  const DevInstance* inst;
  int n_inst;
  uint4* state;          // photon state pool, SoA of 16-byte words
  double* tacc;          // per-thread accumulators, SoA [NACC][slots]
  unsigned* status;      // status flags (mcrt_status_flags)
  int table_f4;          // shared-memory table capacity in float4
};

template <typename T>
__device__ __forceinline__ void ps_load(PState<T>& s, const uint4* base, size_t stride, size_t g) {
  constexpr int N = sizeof(PState<T>) / 16;
  union U {
    PState<T> p;
    uint4 q[N];
    __device__ U() {}
  } u;
#pragma unroll
  for (int i = 0; i < N; ++i) u.q[i] = base[(size_t)i * stride + g];
  s = u.p;
}

template <typename T>
__device__ __forceinline__ void ps_store(const PState<T>& s, uint4* base, size_t stride, size_t g) {
  constexpr int N = sizeof(PState<T>) / 16;
  union U {
    PState<T> p;
    uint4 q[N];
    __device__ U() {}
  } u;
  u.p = s;
#pragma unroll
  for (int i = 0; i < N; ++i) base[(size_t)i * stride + g] = u.q[i];
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sphere distance to the boundary along a unit direction with k.x = kx and
// D = tau^2 - |x|^2 >= 0, in a cancellation-free form of sphere.jl:69-73.
template <typename T>
__device__ __forceinline__ T sphere_t(T kx, T D) {
  T r = MT<T>::sqrt(kx * kx + D);
  return kx > T(0) ? MT<T>::div(D, kx + r) : r - kx;
}

// ------------------------------------------------------------------ instance staging
// Copies the instance into shared memory and stages its Mie tables there with
// coalesced 16-byte loads; the shared copy's table pointers are redirected.
template <typename T, int BS>
__device__ void stage_instance(Shared<T, BS>& sh, float4* tables, const KParams& p, int cur) {
  const int tid = threadIdx.x;
  {
    const int4* src = reinterpret_cast<const int4*>(&p.inst[cur]);
    int4* dst = reinterpret_cast<int4*>(&sh.inst);
    constexpr int N = sizeof(DevInstance) / 16;
    for (int i = tid; i < N; i += BS) dst[i] = src[i];
  }
  __syncthreads();
  int off = 0;
  const DevInstance& src = p.inst[cur];
  for (int s = 0; s < src.n_scat; ++s) {
    const DevScatterer& d = src.scat[s];
    if (d.kind != 1) continue;
    int nf = d.ntheta + 1;
    int nc4 = (d.rp + 2 + 3) / 4;
    if (off + 2 * nf + nc4 > p.table_f4) continue;  // stays in global memory (L1/L2)
    float4* F = tables + off;
    float4* S = F + nf;
    float4* C = S + nf;
    for (int i = tid; i < nf; i += BS) {
      F[i] = d.F[i];
      S[i] = d.S[i];
    }
    const float4* c4 = reinterpret_cast<const float4*>(d.csrn);
    for (int i = tid; i < nc4; i += BS) C[i] = c4[i];
    if (tid == 0) {
      sh.inst.scat[s].F = F;
      sh.inst.scat[s].S = S;
      sh.inst.scat[s].csrn = reinterpret_cast<const float*>(C);
    }
    off += 2 * nf + nc4;
  }
  __syncthreads();
}

// The next instance after cur (cyclically) that still has photons to claim, or -1.
__device__ __forceinline__ int next_instance(const KParams& p, int cur) {
  for (int k = 1; k <= p.n_inst; ++k) {
    const int i = (cur + k) % p.n_inst;
    unsigned long long c = atomicAdd(p.inst[i].claim, 0ull);
    if ((long long)c < p.inst[i].n_photons) return i;
  }
  return -1;
}

// Where a block starts: blocks are spread over the instances in proportion to their
// photons (instances come largest first), so a small instance is worked by a few full
// blocks rather than by every block with a few photons each.
__device__ __forceinline__ int start_instance(const KParams& p) {
  double total = 0.0;
  for (int i = 0; i < p.n_inst; ++i) total += (double)p.inst[i].n_photons;
  if (!(total > 0.0)) return -1;
  const double target = (blockIdx.x + 0.5) / gridDim.x * total;
  double cum = 0.0;
  int first = p.n_inst - 1;
  for (int i = 0; i < p.n_inst; ++i) {
    cum += (double)p.inst[i].n_photons;
    if (cum > target) {
      first = i;
      break;
    }
  }
  return next_instance(p, first - 1 < 0 ? p.n_inst - 1 : first - 1);
}

__device__ __forceinline__ void acc_add(double* tacc, size_t stride, size_t g, int k, double v) {
  tacc[(size_t)k * stride + g] += v;
}

// ------------------------------------------------------------------ photon start
// Start of cpu_kernel / gpu_kernel for one photon: initial_x, direct transmission and
// initial_propagation (src/gpu.jl:187-204; plane.jl:64-95; sphere.jl:39-67), in FP64.
template <typename T>
__device__ bool start_photon(PState<T>& ps, const DevInstance& in, unsigned long long ph,
                             double* tacc, size_t stride, size_t g, unsigned* status) {
  ps.id = ph;
  ps.n = 0;
  ps.idx = 0;
  ps.idx1 = 0;
  ps.peak = 0.0;
  double I[4] = {in.I0[0], in.I0[1], in.I0[2], in.I0[3]};
  double k[3] = {in.k0[0], in.k0[1], in.k0[2]};
  double x[3] = {0.0, 0.0, 0.0};
  Draw d0 = draw(in.key0, in.key1, ph, 0, 0);
  double tau1 = in.layers[0].tau;
  if (in.geom == 1) {
    double r = tau1 * sqrt(u01<double>(d0.r[0]));
    double phi = 2 * PI_D * u01<double>(d0.r[1]);
    double s, c;
    sincos(phi, &s, &c);
    x[0] = r * c;
    x[1] = r * s;
    x[2] = sqrt(tau1 * tau1 - r * r);
  }
  bool cdt = in.geom == 1 || (in.n_layers == 1 && !in.layers[0].inf);
  if (cdt) {
    double tp = dist_d(in, x, k[0], k[1], k[2], 0);
    double dt = tp <= in.tau0 ? exp(-tp) : 0.0;
    acc_add(tacc, stride, g, ACC_ADT, I[0] * dt);
    for (int s = 0; s < 4; ++s) I[s] *= 1 - dt;
  }
  double u2 = in.rng_mode == 1 ? ((double)ph + 0.5) / (double)in.nrays : u01<double>(d0.r[2]);
  double t;
  if (in.geom == 0) {
    if (in.layers[0].inf) {
      t = -log(u2);
    } else {
      double tp = dist_d(in, x, k[0], k[1], k[2], 0);
      if (cdt && tp <= in.tau0) {
        t = -log(1 - u2 * (1 - exp(-tp)));
      } else {
        t = tp + 1;
        for (unsigned a = 0; t > tp; ++a) {
          if ((long long)a >= in.max_attempts) {
            atomicOr(status, 1u);
            acc_add(tacc, stride, g, ACC_REJECT_CAP, 1.0);
            t = tp;
            break;
          }
          double u = a == 0 ? u2 : u01<double>(draw(in.key0, in.key1, ph, 0, a).r[2]);
          t = -log(u);
        }
      }
    }
  } else {
    double tp = 2.0 * x[2];
    if (tp <= in.tau0) {
      t = -log(1 - u2 * (1 - exp(-tp)));
    } else {
      t = tp + 1;
      for (unsigned a = 0; t > tp; ++a) {
        if ((long long)a >= in.max_attempts) {
          atomicOr(status, 1u);
          acc_add(tacc, stride, g, ACC_REJECT_CAP, 1.0);
          t = tp;
          break;
        }
        uint32_t r = a == 0 ? d0.r[2] : draw(in.key0, in.key1, ph, 0, a).r[2];
        double uc = in.rng_mode == 1 && a == 0 ? 1.0 - u2 : u01<double>(~r);  // 1 - u (sphere.jl:61)
        t = -log(uc);
      }
    }
  }
  for (int s = 0; s < 3; ++s) {
    ps.x[s] = x[s] + t * k[s];
    ps.k[s] = (T)k[s];
  }
  for (int s = 0; s < 4; ++s) ps.I[s] = (T)I[s];
  if (!((double)ps.I[0] >= in.min_int && 0 < in.max_scat)) {
    acc_add(tacc, stride, g, ACC_AREM, (double)ps.I[0]);
    acc_add(tacc, stride, g, ACC_PHOTONS, 1.0);
    return false;
  }
  return true;
}

// ------------------------------------------------------------------ sample phase
// One scattering event of src/gpu.jl:209-291 up to the collection: records the
// reciprocal-path state, runs the rejection loop (scatter + free path + boundary test),
// absorbs, and writes the event's collection parameters. The move to the new position
// is applied here; the escaped-intensity renormalisation waits for the collect phase.
template <typename T>
__device__ int sample_event(PState<T>& ps, const DevInstance& in, const BinTables<T>& B,
                            EventP<T>& ev, double* tacc, size_t stride, size_t g,
                            unsigned* status, bool& dead, unsigned& attempts) {
  dead = false;
  const int n = ++ps.n;
  const DevScatterer& s1 = in.scat[in.layers[0].scat];
  const Frame<T> inc{(T)in.inc[0], (T)in.inc[1], (T)in.inc[2], (T)in.inc[3]};

  // Incremental forward / backward fields (forward_E, backward_E of src/utils.jl:199-241).
  if (in.compute_cb) {
    if (n == 1) {
      ps.x1[0] = ps.x[0];
      ps.x1[1] = ps.x[1];
      ps.x1[2] = ps.x[2];
      ps.idx1 = ps.idx;
      double nr = sqrt(in.Ei[0] * in.Ei[0] + in.Ei[1] * in.Ei[1] + in.Ei[2] * in.Ei[2] +
                       in.Ei[3] * in.Ei[3]);
      for (int s = 0; s < 4; ++s) ps.A[s] = (T)(in.Ei[s] / nr);
      ps.logA = log(nr);
      for (int s = 0; s < 8; ++s) ps.L[s] = T(0);
      ps.L[0] = T(1);
      ps.L[6] = T(1);
      ps.logL = 0.0;
    } else {
      if (n == 2) {
        ps.k2[0] = ps.k[0];
        ps.k2[1] = ps.k[1];
        ps.k2[2] = ps.k[2];
      }
      Frame<T> fr = n == 2 ? inc : spherical(ps.kprev[0], ps.kprev[1], ps.kprev[2]);
      T m[8], a[4];
      update_E_matrix(fr, ps.k[0], ps.k[1], ps.k[2], s1.kind, s1.S, s1.ntheta, table_scale<T>(s1), m);
      mat2_vec(m, ps.A, a);
      T na = MT<T>::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3]);
      T ina = T(1) / na;
      for (int s = 0; s < 4; ++s) ps.A[s] = a[s] * ina;
      ps.logA += MT<T>::logscale(na);
      if (n >= 3) {
        Frame<T> fm = spherical(-ps.k[0], -ps.k[1], -ps.k[2]);
        update_E_matrix(fm, -ps.kprev[0], -ps.kprev[1], -ps.kprev[2], s1.kind, s1.S, s1.ntheta, table_scale<T>(s1), m);
        mat2_mul(ps.L, m, ps.L);
        T nl = T(0);
        for (int s = 0; s < 8; ++s) nl += ps.L[s] * ps.L[s];
        nl = MT<T>::sqrt(nl);
        T inl = T(1) / nl;
        for (int s = 0; s < 8; ++s) ps.L[s] *= inl;
        ps.logL += MT<T>::logscale(nl);
      }
    }
    ps.kprev[0] = ps.k[0];
    ps.kprev[1] = ps.k[1];
    ps.kprev[2] = ps.k[2];
  }

  // Rejection loop (src/gpu.jl:215-256).
  const int idx = ps.idx;
  const DevLayer& L = in.layers[idx];
  const DevScatterer& sc = in.scat[L.scat];
  const Frame<T> ks = spherical(ps.k[0], ps.k[1], ps.k[2]);
  const T* I = ps.I;
  T Ip[4], kp[3];
  double xp[3];
  int idxp = idx;
  unsigned a = 0;
  int kcap = 0;
  for (;; ++a) {
    if ((long long)a >= in.max_attempts) {
      atomicOr(status, 1u);
      acc_add(tacc, stride, g, ACC_REJECT_CAP, 1.0);
      dead = true;
      return 0;
    }
    Draw d = draw(in.key0, in.key1, ps.id, (uint32_t)n, a);
    T u0 = u01<T>(d.r[0]), u1 = u01<T>(d.r[1]), u2 = u01<T>(d.r[2]);
    // scatter (src/utils.jl:294-323)
    T mu = sample_mu<T>(sc.kind, sc.csrn, sc.rp, u0);
    PMat<T> P = phase_eval<T>(sc.kind, sc.F, sc.ntheta, table_scale<T>(sc), mu);
    T den = P.p11 * I[0];
    T eq = -P.p12 * I[1] / den, eu = -P.p12 * I[2] / den;
    T ee = MT<T>::sqrt(eq * eq + eu * eu);
    T phi;
    if (ee > T(1e-12)) {
      T gam = MT<T>::acos(clamp1(eq / ee));
      if (eu < T(0)) gam = (T)(2 * PI_D) - gam;
      T sg, cg;
      MT<T>::sincos(gam, &sg, &cg);
      T ma = (T)(4 * PI_D) * u1 + gam - ee * sg;
      T ea = kepler<T>(ma, ee, kcap);
      phi = T(0.5) * (ea - gam);
    } else {
      phi = (T)(2 * PI_D) * u1;
    }
    T st = MT<T>::sqrt(fmax(T(1) - mu * mu, T(0)));
    T sphi, cphi;
    MT<T>::sincos(phi, &sphi, &cphi);
    T lx = st * cphi, ly = st * sphi, lz = mu;
    ray_to_norm(ks, lx, ly, lz, kp[0], kp[1], kp[2]);
    // update_I(sca, I, k', ks) with the ray-frame direction known exactly
    Frame<T> kls = spherical(lx, ly, lz);
    T ehx, ehy;
    basis_h(kp[0], kp[1], ehx, ehy);
    T cpsi, spsi;
    psi_angles(ks, kls, ehx, ehy, T(-1), cpsi, spsi);
    T q = I[1], u = I[2];
    rotate(kls.cp * kls.cp - kls.sp * kls.sp, T(-2) * kls.sp * kls.cp, q, u);
    Ip[0] = P.p11 * I[0] + P.p12 * q;
    Ip[1] = P.p12 * I[0] + P.p11 * q;
    Ip[2] = P.p33 * u + P.p34 * I[3];
    Ip[3] = -P.p34 * u + P.p33 * I[3];
    rotate(cpsi * cpsi - spsi * spsi, T(2) * spsi * cpsi, Ip[1], Ip[2]);
    // free path and boundary test
    T t = -MT<T>::log(u2);
    for (int s = 0; s < 3; ++s) xp[s] = ps.x[s] + (double)t * (double)kp[s];
    int pb;
    if (in.geom == 0) {
      pb = xp[2] > 0 ? -1 : ((!L.inf && xp[2] < -L.tau) ? 1 : 0);
    } else {
      double r2 = xp[0] * xp[0] + xp[1] * xp[1] + xp[2] * xp[2];
      pb = sqrt(r2) > in.layers[0].tau ? -2 : 0;
    }
    idxp = idx + pb;
    if (pb == -2) continue;
    if (pb == -1) {
      if (idxp < 0) continue;
      xp[0] = ps.x[0];
      xp[1] = ps.x[1];
      xp[2] = -L.tau;
      break;
    }
    if (pb == 1) {
      if (idxp > in.n_layers - 1) continue;
      xp[0] = ps.x[0];
      xp[1] = ps.x[1];
      xp[2] = 0.0;
      break;
    }
    break;
  }
  if (kcap) {
    atomicOr(status, 2u);
    acc_add(tacc, stride, g, ACC_KEPLER_CAP, 1.0);
  }

  // Absorption (src/gpu.jl:259-260)
  T Ia[4];
  const T om = (T)L.omega;
  acc_add(tacc, stride, g, ACC_AABS, (1.0 - L.omega) * (double)I[0]);
  for (int s = 0; s < 4; ++s) Ia[s] = I[s] * om;

  // Proximity tests (src/gpu.jl:266-267)
  double mdf, mdl;
  if (in.geom == 0) {
    mdf = idx == 0 ? fabs(ps.x[2]) : INFINITY;
    mdl = (idx == in.n_layers - 1 && !L.inf) ? L.tau - fabs(ps.x[2]) : INFINITY;
  } else {
    mdf = in.layers[0].tau -
          sqrt(ps.x[0] * ps.x[0] + ps.x[1] * ps.x[1] + ps.x[2] * ps.x[2]);
    mdl = INFINITY;
  }
  const bool up = mdf <= in.tau0, dn = mdl <= in.tau0;
  const bool cb = in.compute_cb && (up || dn);
  int flags = (up ? EV_UP : 0) | (dn ? EV_DN : 0) | (cb ? EV_CB : 0) | ((cb && n > 1) ? EV_CBN : 0);

  // Event parameters shared by RT and CB.
  for (int s = 0; s < 4; ++s) ev.I[s] = Ia[s];
  ev.fct = ks.ct;
  ev.fst = ks.st;
  ev.fcp = ks.cp;
  ev.fsp = ks.sp;
  if (in.geom == 0) {
    ev.a_up = (T)(-ps.x[2]);
    ev.a_dn = L.inf ? (T)INFINITY : (T)(ps.x[2] + L.tau);
  } else {
    double tau = in.layers[0].tau;
    ev.xax = (T)ps.x[0];
    ev.xay = (T)ps.x[1];
    ev.xaz = (T)ps.x[2];
    double D = tau * tau - (ps.x[0] * ps.x[0] + ps.x[1] * ps.x[1] + ps.x[2] * ps.x[2]);
    ev.Da = (T)(D > 0 ? D : 0);
  }
  ev.flags = flags;
  ev.layer = L.scat;

  if (cb && n > 1) {
    // Reciprocal-path setup of collect_cb_gpu! (src/gpu.jl:55-88).
    const Frame<T> kbs = spherical(-ps.k2[0], -ps.k2[1], -ps.k2[2]);
    ev.bct = kbs.ct;
    ev.bst = kbs.st;
    ev.bcp = kbs.cp;
    ev.bsp = kbs.sp;
    T m[8], Ei[4], tmp[4], b[4];
    for (int s = 0; s < 4; ++s) Ei[s] = (T)in.Ei[s];
    update_E_matrix(inc, -ps.k[0], -ps.k[1], -ps.k[2], s1.kind, s1.S, s1.ntheta, table_scale<T>(s1), m);
    mat2_vec(m, Ei, tmp);
    mat2_vec(ps.L, tmp, b);
    const T kf0x = (T)in.kf0[0], kf0y = (T)in.kf0[1], kf0z = (T)in.kf0[2];
    const T eh0x = (T)in.eh0[0], eh0y = (T)in.eh0[1];
    T Iaf0[4];
    update_I(ks, Ia, kf0x, kf0y, kf0z, eh0x, eh0y, s1.kind, s1.F, s1.ntheta, table_scale<T>(s1), Iaf0);
    T Ef[4] = {ps.A[0], ps.A[1], ps.A[2], ps.A[3]};
    update_E(ks, Ef, kf0x, kf0y, kf0z, eh0x, eh0y, s1.kind, s1.S, s1.ntheta, table_scale<T>(s1));
    T nf = Ef[0] * Ef[0] + Ef[1] * Ef[1] + Ef[2] * Ef[2] + Ef[3] * Ef[3];
    // raa of src/gpu.jl:84. The backscattered intensity vanishes in exact arithmetic for a
    // fully polarised photon scattered at 90 degrees by Rayleigh scatterers (P11 = -P12),
    // where rounding can leave it slightly negative: clamped at zero (the reference's
    // sqrt would throw there), as is a vanishing field norm.
    T c = nf > T(0) ? MT<T>::sqrt(fmax(Iaf0[0], T(0)) / nf) : T(0);
    T rb = (T)MT<T>::expscale(ps.logL - ps.logA) * c;
    for (int s = 0; s < 4; ++s) {
      ev.ea[s] = ps.A[s] * c;
      ev.eb[s] = b[s] * rb;
    }
    double ta0 = dist_d(in, ps.x, in.kf0[0], in.kf0[1], in.kf0[2], idx);
    double tb0 = dist_d(in, ps.x1, in.kf0[0], in.kf0[1], in.kf0[2], ps.idx1);
    ev.tab2 = (T)((ta0 - tb0) * LOG2E_D);
    double dx = in.kl1 * (ps.x[0] - ps.x1[0]) / (2 * PI_D);
    double dy = in.kl1 * (ps.x[1] - ps.x1[1]) / (2 * PI_D);
    double dz = in.kl1 * (ps.x[2] - ps.x1[2]) / (2 * PI_D);
    ev.v1 = (T)(in.Rkfs[0] * dx + in.Rkfs[1] * dy + in.Rkfs[2] * dz);
    ev.v2 = (T)(in.Rkfs[3] * dx + in.Rkfs[4] * dy + in.Rkfs[5] * dz);
    ev.v3 = (T)(in.Rkfs[6] * dx + in.Rkfs[7] * dy + in.Rkfs[8] * dz);
    if (in.geom == 0) {
      const DevLayer& L1 = in.layers[ps.idx1];
      ev.b_up = (T)(-ps.x1[2]);
      ev.b_dn = L1.inf ? (T)INFINITY : (T)(ps.x1[2] + L1.tau);
    } else {
      double tau = in.layers[0].tau;
      ev.xbx = (T)ps.x1[0];
      ev.xby = (T)ps.x1[1];
      ev.xbz = (T)ps.x1[2];
      double D = tau * tau - (ps.x1[0] * ps.x1[0] + ps.x1[1] * ps.x1[1] + ps.x1[2] * ps.x1[2]);
      ev.Db = (T)(D > 0 ? D : 0);
    }
  }

  // The pending state change (applied now; the weight waits). The event counters are
  // kept by the caller from the returned flags and attempts.
  attempts = a + 1;

  T inv = T(1) / Ip[0];
  ps.Ih[0] = T(1);
  ps.Ih[1] = Ip[1] * inv;
  ps.Ih[2] = Ip[2] * inv;
  ps.Ih[3] = Ip[3] * inv;
  ps.wI = Ia[0];
  for (int s = 0; s < 3; ++s) {
    ps.k[s] = kp[s];
    ps.x[s] = xp[s];
  }
  ps.idx = idxp;
  return flags;
}

// ------------------------------------------------------------------ collect: RT tile
template <typename T, int NB>
struct RTLane {
  T st[NB], ct[NB], g[NB], w[NB];
  T cb, sb;
  T acc[NB][4];
};

template <typename T, int NB, bool MIE, bool SPHERE>
__device__ __forceinline__ T rt_event(RTLane<T, NB>& R, const EventP<T>& E, const float4* F,
                                      int ntheta, T scale, T tau0l, bool upper) {
  const T fct = E.fct, fst = E.fst, fcp = E.fcp, fsp = E.fsp;
  const T sD = R.sb * fcp - R.cb * fsp, cD = R.cb * fcp + R.sb * fsp;
  const T a1 = fct * cD, a3 = fst * cD, bq = fct * sD, c4 = fst * sD;
  const T I0 = E.I[0], I1 = E.I[1], I2 = E.I[2], I3 = E.I[3];
  T a = upper ? E.a_up : E.a_dn;
  T qx = T(0), xz = T(0), D = T(0);
  if (SPHERE) {
    qx = R.cb * E.xax + R.sb * E.xay;
    xz = E.xaz;
    D = E.Da;
  }
  T esc = T(0);
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const T k1 = R.st[i] * a1 - R.ct[i] * fst;
    const T k2 = R.st[i] * sD;
    const T k3 = R.st[i] * a3 + R.ct[i] * fct;
    const T s2 = k1 * k1 + k2 * k2;
    T cpk, spk, stk, ctk;
    if (s2 < T(1e-24)) {
      cpk = T(1);
      spk = T(0);
      stk = T(0);
      ctk = k3 > T(0) ? T(1) : (k3 < T(0) ? T(-1) : T(0));
    } else {
      const T r = MT<T>::rsqrt(s2);
      cpk = k1 * r;
      spk = k2 * r;
      stk = s2 * r;
      ctk = k3;
    }
    const T c2 = cpk * cpk - spk * spk, sr = T(-2) * spk * cpk;
    const T q = c2 * I1 + sr * I2, u = -sr * I1 + c2 * I2;
    const T cpsi = spk * bq + cpk * cD;
    const T spsi = ctk * (spk * cD - cpk * bq) + stk * c4;
    const T c2p = cpsi * cpsi - spsi * spsi, s2p = T(2) * spsi * cpsi;
    PMat<T> P;
    if (MIE) {
      P = phase_eval<T>(1, F, ntheta, scale, k3);
    } else {
      const T m2 = k3 * k3;
      P = PMat<T>{T(0.75) + T(0.75) * m2, T(-0.75) + T(0.75) * m2, T(1.5) * k3, T(0)};
    }
    const T o0 = P.p11 * I0 + P.p12 * q;
    const T o1 = P.p12 * I0 + P.p11 * q;
    const T o2 = P.p33 * u + P.p34 * I3;
    const T o3 = -P.p34 * u + P.p33 * I3;
    const T r1 = c2p * o1 + s2p * o2, r2 = -s2p * o1 + c2p * o2;
    T t2;
    if (SPHERE) {
      const T kx = R.st[i] * qx + R.ct[i] * xz;
      t2 = sphere_t(kx, D) * T(LOG2E_D);
    } else {
      t2 = a * R.g[i];
    }
    const T wgt = t2 <= tau0l ? MT<T>::exp2n(t2) * R.w[i] : T(0);
    R.acc[i][0] += o0 * wgt;
    R.acc[i][1] += r1 * wgt;
    R.acc[i][2] += r2 * wgt;
    R.acc[i][3] += o3 * wgt;
    esc += o0 * wgt;
  }
  return esc;
}

template <typename T, int NB, int BS>
__device__ void rt_tile(Shared<T, BS>& sh, const BinTables<T>& B, int tile, bool upper, int pc, int q0,
                        int q1) {
  const int lane = threadIdx.x & 31;
  const int r0 = upper ? B.up0 : B.lo0, r1 = upper ? B.up1 : B.lo1;
  const int ngrp = (r1 - r0 + NB - 1) / NB;
  const int item = tile * 32 + lane;
  const bool lane_ok = item < ngrp * B.nphi;
  const int it = lane_ok ? item : 0;
  const int j2 = it % B.nphi, grp = it / B.nphi;
  RTLane<T, NB> R;
  R.cb = B.cp[j2];
  R.sb = B.sp[j2];
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    int j1 = r0 + grp * NB + i;
    bool ok = lane_ok && j1 < r1;
    int jj = ok ? j1 : r0;
    R.st[i] = B.st[jj];
    R.ct[i] = B.ct[jj];
    R.g[i] = B.g[jj];
    R.w[i] = ok ? B.w[jj] : T(0);
#pragma unroll
    for (int s = 0; s < 4; ++s) R.acc[i][s] = T(0);
  }
  const DevInstance& in = sh.inst;
  const T tau0l = (T)(in.tau0 * LOG2E_D);
  const int li = upper ? 0 : 1;
  T* escarr = upper ? sh.esc_up : sh.esc_dn;
  const bool sphere = in.geom == 1;
  for (int q = q0; q < q1; ++q) {
    const int e = sh.list[li][q];
    const EventP<T>& E = sh.ev[e];
    const DevScatterer& sc = in.scat[E.layer];
    T esc;
    if (sc.kind == 1) {
      const T scale = table_scale<T>(sc);
      esc = sphere ? rt_event<T, NB, true, true>(R, E, sc.F, sc.ntheta, scale, tau0l, upper)
                   : rt_event<T, NB, true, false>(R, E, sc.F, sc.ntheta, scale, tau0l, upper);
    } else {
      esc = sphere ? rt_event<T, NB, false, true>(R, E, sc.F, sc.ntheta, T(0), tau0l, upper)
                   : rt_event<T, NB, false, false>(R, E, sc.F, sc.ntheta, T(0), tau0l, upper);
    }
    esc = warp_sum(esc);
    if (lane == 0) atomicAdd(&escarr[e], esc);
  }
  if (lane_ok) {
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      int j1 = r0 + grp * NB + i;
      if (j1 < r1) {
        double* dst = in.Irt + 4 * ((size_t)j2 * B.ntheta + j1);
#pragma unroll
        for (int s = 0; s < 4; ++s) atomicAdd(dst + s, (double)R.acc[i][s]);
      }
    }
  }
}

// ------------------------------------------------------------------ collect: RT, Fourier modes
// For Rayleigh scatterers the peel-off Stokes vector into a bin, expressed in the bin's
// meridian frame, is a trigonometric polynomial of degree 2 in the bin azimuth
// (dipole scattering is quadratic in the field), and in a slab the attenuation
// inorm * exp(-t) depends on the polar bin only. So per (event, polar bin) the 5
// Fourier coefficients of each Stokes component are taken from update_I at 5 equally
// spaced azimuths (an exact 5-point DFT) and summed over events with the attenuation
// weight. The block that finishes the launch's last photon of the instance expands the
// coefficients into every configured azimuth (fourier_expand). This equals the per-bin
// evaluation of src/gpu.jl:11-31 up to rounding and costs 5 evaluations per polar bin
// instead of Nphi.

// cos and sin of 2*pi*j/5 and of 4*pi*j/5, j = 0..4.
template <typename T>
__device__ __forceinline__ void fourier_node(int j, T& c1, T& s1, T& c2, T& s2) {
  constexpr double C1 = 0.30901699437494742, S1 = 0.95105651629515357;   // 2*pi/5
  constexpr double C2 = -0.80901699437494742, S2 = 0.58778525229247313;  // 4*pi/5
  switch (j) {
    case 0: c1 = T(1), s1 = T(0), c2 = T(1), s2 = T(0); break;
    case 1: c1 = T(C1), s1 = T(S1), c2 = T(C2), s2 = T(S2); break;
    case 2: c1 = T(C2), s1 = T(S2), c2 = T(C1), s2 = T(-S1); break;
    case 3: c1 = T(C2), s1 = T(-S2), c2 = T(C1), s2 = T(S1); break;
    default: c1 = T(C1), s1 = T(-S1), c2 = T(C2), s2 = T(-S2); break;
  }
}

// Unweighted Rayleigh update_I into the direction (st cos(phib), st sin(phib), ct): the
// arithmetic of rt_event with the Rayleigh phase matrix.
template <typename T>
__device__ __forceinline__ void rayleigh_peel(T st, T ct, T cb, T sb, const Frame<T>& f, const T I[4],
                                              T o[4]) {
  const T sDe = sb * f.cp - cb * f.sp, cD = cb * f.cp + sb * f.sp;
  const T k1 = st * (f.ct * cD) - ct * f.st;
  const T k2 = st * sDe;
  const T k3 = st * (f.st * cD) + ct * f.ct;
  T s2 = k1 * k1 + k2 * k2;
  const bool pole = s2 < T(1e-24);
  s2 = pole ? T(1) : s2;
  const T r = MT<T>::rsqrt(s2);
  const T cpk = pole ? T(1) : k1 * r, spk = pole ? T(0) : k2 * r, stk = pole ? T(0) : s2 * r;
  const T ctk = pole ? (k3 > T(0) ? T(1) : (k3 < T(0) ? T(-1) : T(0))) : k3;
  const T c2 = cpk * cpk - spk * spk, sr = T(-2) * spk * cpk;
  const T q = c2 * I[1] + sr * I[2], u = -sr * I[1] + c2 * I[2];
  const T bq = f.ct * sDe, c4 = f.st * sDe;
  const T cpsi = spk * bq + cpk * cD;
  const T spsi = ctk * (spk * cD - cpk * bq) + stk * c4;
  const T c2p = cpsi * cpsi - spsi * spsi, s2p = T(2) * spsi * cpsi;
  const T m2 = k3 * k3;
  const T p11 = T(0.75) + T(0.75) * m2, p12 = T(-0.75) + T(0.75) * m2, p33 = T(1.5) * k3;
  const T o1 = p12 * I[0] + p11 * q, o2 = p33 * u;
  o[0] = p11 * I[0] + p12 * q;
  o[1] = c2p * o1 + s2p * o2;
  o[2] = -s2p * o1 + c2p * o2;
  o[3] = p33 * I[3];
}

// One lane per polar bin of the hemisphere; events q0..q1 of the batch's list.
template <typename T, int BS>
__device__ void rt_fourier_tile(Shared<T, BS>& sh, const BinTables<T>& B, int tile, bool upper, int q0,
                                int q1) {
  const int lane = threadIdx.x & 31;
  const int r0 = upper ? B.up0 : B.lo0, r1 = upper ? B.up1 : B.lo1;
  const int j1 = r0 + tile * 32 + lane;
  const bool ok = j1 < r1;
  const int jj = ok ? j1 : r0;
  const T st = B.st[jj], ct = B.ct[jj], g = B.g[jj], w = ok ? B.w[jj] : T(0);
  // sums over the configured azimuths of the 4 non-constant modes (for the escaped intensity)
  T fs1 = T(0), fs2 = T(0), fs3 = T(0), fs4 = T(0);
  for (int j2 = 0; j2 < B.nphi; ++j2) {
    const T cp = B.cp[j2], sp = B.sp[j2];
    fs1 += cp;
    fs2 += sp;
    fs3 += cp * cp - sp * sp;
    fs4 += T(2) * sp * cp;
  }
  const T fs0 = T(B.nphi);
  T acc[4][5];
#pragma unroll
  for (int s = 0; s < 4; ++s)
#pragma unroll
    for (int m = 0; m < 5; ++m) acc[s][m] = T(0);
  const DevInstance& in = sh.inst;
  const T tau0l = (T)(in.tau0 * LOG2E_D);
  const int li = upper ? 0 : 1;
  T* escarr = upper ? sh.esc_up : sh.esc_dn;
  for (int q = q0; q < q1; ++q) {
    const int e = sh.list[li][q];
    const EventP<T>& E = sh.ev[e];
    const Frame<T> f{E.fct, E.fst, E.fcp, E.fsp};
    const T t2 = (upper ? E.a_up : E.a_dn) * g;
    const T wgt = t2 <= tau0l ? MT<T>::exp2n(t2) * w : T(0);
    T c[4][5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      T n1, m1, n2, m2;
      fourier_node<T>(j, n1, m1, n2, m2);
      T o[4];
      rayleigh_peel<T>(st, ct, n1, m1, f, E.I, o);
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        if (j == 0) {
          c[s][0] = o[s];
          c[s][1] = o[s];
          c[s][2] = T(0);
          c[s][3] = o[s];
          c[s][4] = T(0);
        } else {
          c[s][0] += o[s];
          c[s][1] += o[s] * n1;
          c[s][2] += o[s] * m1;
          c[s][3] += o[s] * n2;
          c[s][4] += o[s] * m2;
        }
      }
    }
    // f(phi) = c0/5 + (2/5) (c1 cos phi + c2 sin phi + c3 cos 2phi + c4 sin 2phi)
    const T w0 = wgt * T(0.2), w1 = wgt * T(0.4);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      acc[s][0] += w0 * c[s][0];
#pragma unroll
      for (int m = 1; m < 5; ++m) acc[s][m] += w1 * c[s][m];
    }
    T esc = w0 * c[0][0] * fs0 + w1 * (c[0][1] * fs1 + c[0][2] * fs2 + c[0][3] * fs3 + c[0][4] * fs4);
    esc = warp_sum(esc);
    if (lane == 0) atomicAdd(&escarr[e], esc);
  }
  if (ok) {
    double* dst = in.Frt + 20 * (size_t)j1;
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
      for (int m = 0; m < 5; ++m) atomicAdd(dst + 5 * s + m, (double)acc[s][m]);
  }
}

// Irt of every bin from the Fourier coefficients (plain stores: the Fourier path writes
// Irt nowhere else). Coefficients are read through L2, after the caller's fence.
template <typename T>
__device__ void fourier_expand(const DevInstance& in, const BinTables<T>& B, int tid, int nthreads) {
  const int nt = B.ntheta, nb = B.ntheta * B.nphi;
  for (int b = tid; b < nb; b += nthreads) {
    const int j1 = b % nt, j2 = b / nt;
    const double cp = (double)B.cp[j2], sp = (double)B.sp[j2];
    const double c2 = cp * cp - sp * sp, s2 = 2.0 * sp * cp;
    const double* f = in.Frt + 20 * (size_t)j1;
    double* dst = in.Irt + 4 * (size_t)b;
#pragma unroll
    for (int s = 0; s < 4; ++s)
      dst[s] = __ldcg(f + 5 * s) + __ldcg(f + 5 * s + 1) * cp + __ldcg(f + 5 * s + 2) * sp +
               __ldcg(f + 5 * s + 3) * c2 + __ldcg(f + 5 * s + 4) * s2;
  }
}

// ------------------------------------------------------------------ collect: RT tile, FP32x2
// The FP32 RT peel-off with two polar bins per packed FP32x2 instruction (FFMA2, FMUL2,
// FADD2 of sm_100 and later): same arithmetic as rt_event, half the issued FP32
// instructions. Steps without a packed form (MUFU, conversions, table loads, selects)
// run per bin.
struct P2 {
  float2 v;
};
__device__ __forceinline__ P2 p2(float a, float b) { return P2{make_float2(a, b)}; }
__device__ __forceinline__ P2 p2s(float a) { return P2{make_float2(a, a)}; }
__device__ __forceinline__ P2 operator*(P2 a, P2 b) { return P2{__fmul2_rn(a.v, b.v)}; }
__device__ __forceinline__ P2 operator+(P2 a, P2 b) { return P2{__fadd2_rn(a.v, b.v)}; }
__device__ __forceinline__ P2 fma2(P2 a, P2 b, P2 c) { return P2{__ffma2_rn(a.v, b.v, c.v)}; }

// acos_as4446 (Abramowitz & Stegun 4.4.46) on two values at once, times `scale` (the
// Mie table index per radian): the factor rides on the sign and offset selects, which
// run on the ALU pipe, instead of costing a multiply on the busy FMA pipe.
__device__ __forceinline__ P2 acos2_scaled(P2 x, float scale) {
  const P2 ax = p2(fabsf(x.v.x), fabsf(x.v.y));
  P2 p = fma2(p2s(-0.0012624911f), ax, p2s(0.0066700901f));
  p = fma2(p, ax, p2s(-0.0170881256f));
  p = fma2(p, ax, p2s(0.0308918810f));
  p = fma2(p, ax, p2s(-0.0501743046f));
  p = fma2(p, ax, p2s(0.0889789874f));
  p = fma2(p, ax, p2s(-0.2145988016f));
  p = fma2(p, ax, p2s(1.5707963050f));
  P2 y = fma2(ax, p2s(-1.0f), p2s(1.0f));
  y.v.x = fmaxf(y.v.x, 1e-30f);  // |x| = 1 gives acos = 0 or pi
  y.v.y = fmaxf(y.v.y, 1e-30f);
  const P2 r = (y * p2(rsqrt_approx(y.v.x), rsqrt_approx(y.v.y))) * p;
  const float pis = 3.14159265358979f * scale;
  const P2 sg = p2(x.v.x < 0.f ? -scale : scale, x.v.y < 0.f ? -scale : scale);
  const P2 off = p2(x.v.x < 0.f ? pis : 0.f, x.v.y < 0.f ? pis : 0.f);
  return fma2(sg, r, off);
}

template <int NP>
struct RTLaneF2 {
  const float4* pc;  // this lane's first pair of polar-bin constants (BinTables::rtp)
  float cb, sb;
  P2 acc[NP][4];
};

template <int NP, bool MIE, bool SPHERE>
__device__ __forceinline__ float rt_event_f2(RTLaneF2<NP>& R, const EventP<float>& E, const float4* F,
                                             int ntheta, float scale, float tau0l, bool upper) {
  const float fct = E.fct, fst = E.fst, fcp = E.fcp, fsp = E.fsp;
  const float sD = R.sb * fcp - R.cb * fsp, cD = R.cb * fcp + R.sb * fsp;
  const P2 A1 = p2s(fct * cD), A3 = p2s(fst * cD), NFST = p2s(-fst), FCT = p2s(fct), SD = p2s(sD);
  const P2 BQ = p2s(fct * sD), NBQ = p2s(-fct * sD), CD = p2s(cD), C4 = p2s(fst * sD);
  const float I0 = E.I[0], I1 = E.I[1], I2 = E.I[2], I3 = E.I[3];
  const P2 PI0 = p2s(I0), PI1 = p2s(I1), PI2 = p2s(I2), PI3 = p2s(I3), NPI3 = p2s(-I3);
  const P2 M2I2 = p2s(-2.0f * I2), P2I1 = p2s(2.0f * I1), M1 = p2s(-1.0f), ONE = p2s(1.0f);
  const P2 A = p2s(upper ? E.a_up : E.a_dn);
  P2 QX = p2s(0.f), XZ = p2s(0.f);
  if (SPHERE) {
    QX = p2s(R.cb * E.xax + R.sb * E.xay);
    XZ = p2s(E.xaz);
  }
  P2 esc = p2s(0.f);
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    // the pair's polar constants come through L1 each event, which frees the registers
    // that holding them would take (fewer spills at the 128-register cap)
    const float4 pa = R.pc[2 * i], pb = R.pc[2 * i + 1];
    const P2 Rst = p2(pa.x, pa.y), Rct = p2(pa.z, pa.w), Rg = p2(pb.x, pb.y), Rw = p2(pb.z, pb.w);
    const P2 k1 = fma2(Rst, A1, Rct * NFST);
    const P2 k2 = Rst * SD;
    const P2 k3 = fma2(Rst, A3, Rct * FCT);
    P2 s2 = fma2(k1, k1, k2 * k2);
    // An RT bin exactly along the photon direction has probability zero; the clamp only
    // keeps the arithmetic finite there.
    s2.v.x = fmaxf(s2.v.x, 1e-30f);
    s2.v.y = fmaxf(s2.v.y, 1e-30f);
    const P2 r = p2(rsqrt_approx(s2.v.x), rsqrt_approx(s2.v.y));
    const P2 cpk = k1 * r, spk = k2 * r, stk = s2 * r;
    const P2 c2 = fma2(cpk + cpk, cpk, M1);  // cos 2phi = 2 cos^2 - 1 (cpk^2 + spk^2 = 1)
    const P2 srn = spk * cpk;  // -sr / 2
    const P2 q = fma2(c2, PI1, srn * M2I2);
    const P2 u = fma2(c2, PI2, srn * P2I1);
    const P2 cpsi = fma2(spk, BQ, cpk * CD);
    const P2 spsi = fma2(k3, fma2(spk, CD, cpk * NBQ), stk * C4);
    const P2 c2p = fma2(cpsi + cpsi, cpsi, M1);  // cos 2psi (cpsi^2 + spsi^2 = 1)
    const P2 s2p = (spsi * cpsi) * p2s(2.0f);
    P2 p11, p12, p33, p34;
    if (MIE) {
      const P2 sn = acos2_scaled(k3, scale);
      int i0 = min((int)sn.v.x, ntheta - 1), i1 = min((int)sn.v.y, ntheta - 1);
      const P2 f = fma2(p2((float)i0, (float)i1), M1, sn);
      const float4 a0 = F[i0], b0 = F[i0 + 1], a1 = F[i1], b1 = F[i1 + 1];
      p11 = fma2(f, p2(b0.x - a0.x, b1.x - a1.x), p2(a0.x, a1.x));
      p12 = fma2(f, p2(b0.y - a0.y, b1.y - a1.y), p2(a0.y, a1.y));
      p33 = fma2(f, p2(b0.z - a0.z, b1.z - a1.z), p2(a0.z, a1.z));
      p34 = fma2(f, p2(a0.w - b0.w, a1.w - b1.w), p2(-a0.w, -a1.w));  // holds -p34
    } else {
      const P2 m2 = k3 * k3;
      p11 = fma2(m2, p2s(0.75f), p2s(0.75f));
      p12 = fma2(m2, p2s(0.75f), p2s(-0.75f));
      p33 = k3 * p2s(1.5f);
      p34 = p2s(0.f);
    }
    const P2 o0 = fma2(p11, PI0, p12 * q);
    const P2 o1 = fma2(p12, PI0, p11 * q);
    P2 o2, o3;
    if (MIE) {
      o2 = fma2(p33, u, p34 * NPI3);  // p34 holds -p34 here
      o3 = fma2(p34, u, p33 * PI3);
    } else {
      o2 = p33 * u;
      o3 = p33 * PI3;
    }
    const P2 r1 = fma2(c2p, o1, s2p * o2);
    const P2 r2 = fma2(c2p, o2, (s2p * o1) * M1);
    P2 t2;
    if (SPHERE) {
      const P2 kx = fma2(Rst, QX, Rct * XZ);
      t2 = p2(sphere_t(kx.v.x, E.Da), sphere_t(kx.v.y, E.Da)) * p2s((float)LOG2E_D);
    } else {
      t2 = A * Rg;
    }
    const P2 ex = p2(t2.v.x <= tau0l ? MT<float>::exp2n(t2.v.x) : 0.f,
                     t2.v.y <= tau0l ? MT<float>::exp2n(t2.v.y) : 0.f);
    const P2 wgt = ex * Rw;
    R.acc[i][0] = fma2(o0, wgt, R.acc[i][0]);
    R.acc[i][1] = fma2(r1, wgt, R.acc[i][1]);
    R.acc[i][2] = fma2(r2, wgt, R.acc[i][2]);
    R.acc[i][3] = fma2(o3, wgt, R.acc[i][3]);
    esc = fma2(o0, wgt, esc);
  }
  return esc.v.x + esc.v.y;
}

// The RT events [q0, q1) of one list for a lane, all of one scatterer kind and geometry.
template <int NP, bool MIE, bool SPHERE, typename SH>
__device__ __forceinline__ void rt_events_f2(RTLaneF2<NP>& R, SH& sh, const DevInstance& in, int li, int q0,
                                             int q1, float tau0l, bool upper, float* escarr, int lane) {
  for (int q = q0; q < q1; ++q) {
    const int e = sh.list[li][q];
    const EventP<float>& E = sh.ev[e];
    const DevScatterer& sc = in.scat[E.layer];
    float esc = rt_event_f2<NP, MIE, SPHERE>(R, E, sc.F, sc.ntheta, MIE ? table_scale<float>(sc) : 0.f, tau0l,
                                             upper);
    esc = warp_sum(esc);
    if (lane == 0) atomicAdd(&escarr[e], esc);
  }
}

template <int NB, int BS>
__device__ void rt_tile_f2(Shared<float, BS>& sh, const BinTables<float>& B, int tile, bool upper, int pc,
                           int q0, int q1) {
  static_assert(NB % 2 == 0, "bins are paired");
  constexpr int NP = NB / 2;
  static_assert(RTP_PAD % NP == 0, "a lane's pairs lie within a hemisphere's padded pairs");
  const int lane = threadIdx.x & 31;
  const int r0 = upper ? B.up0 : B.lo0, r1 = upper ? B.up1 : B.lo1;
  const int ngrp = (r1 - r0 + NB - 1) / NB;
  const int item = tile * 32 + lane;
  const bool lane_ok = item < ngrp * B.nphi;
  const int it = lane_ok ? item : 0;
  const int j2 = it % B.nphi, grp = it / B.nphi;
  RTLaneF2<NP> R;
  R.cb = B.cp[j2];
  R.sb = B.sp[j2];
  R.pc = B.rtp + 2 * (lane_ok ? (upper ? 0 : B.rtp_lo) + grp * NP : B.rtp_zero);
#pragma unroll
  for (int i = 0; i < NP; ++i)
#pragma unroll
    for (int s = 0; s < 4; ++s) R.acc[i][s] = p2s(0.f);
  const DevInstance& in = sh.inst;
  const float tau0l = (float)(in.tau0 * LOG2E_D);
  const int li = upper ? 0 : 1;
  float* escarr = upper ? sh.esc_up : sh.esc_dn;
  const bool sphere = in.geom == 1;
  bool one_kind = true;
  for (int k = 1; k < in.n_scat; ++k) one_kind = one_kind && in.scat[k].kind == in.scat[0].kind;
  if (one_kind) {
    // every scatterer of the instance is of one kind: the event loop carries no branch
    // on the kind or the geometry (measured 3.3% faster on the Mie slab, 1.5% on the
    // Mie sphere, than branching per event)
    const int kind = in.scat[0].kind;
    if (kind == 1)
      sphere ? rt_events_f2<NP, true, true>(R, sh, in, li, q0, q1, tau0l, upper, escarr, lane)
             : rt_events_f2<NP, true, false>(R, sh, in, li, q0, q1, tau0l, upper, escarr, lane);
    else
      sphere ? rt_events_f2<NP, false, true>(R, sh, in, li, q0, q1, tau0l, upper, escarr, lane)
             : rt_events_f2<NP, false, false>(R, sh, in, li, q0, q1, tau0l, upper, escarr, lane);
  } else {
    for (int q = q0; q < q1; ++q) {
      const int e = sh.list[li][q];
      const EventP<float>& E = sh.ev[e];
      const DevScatterer& sc = in.scat[E.layer];
      float esc;
      if (sc.kind == 1) {
        const float scale = table_scale<float>(sc);
        esc = sphere ? rt_event_f2<NP, true, true>(R, E, sc.F, sc.ntheta, scale, tau0l, upper)
                     : rt_event_f2<NP, true, false>(R, E, sc.F, sc.ntheta, scale, tau0l, upper);
      } else {
        esc = sphere ? rt_event_f2<NP, false, true>(R, E, sc.F, sc.ntheta, 0.f, tau0l, upper)
                     : rt_event_f2<NP, false, false>(R, E, sc.F, sc.ntheta, 0.f, tau0l, upper);
      }
      esc = warp_sum(esc);
      if (lane == 0) atomicAdd(&escarr[e], esc);
    }
  }
  if (lane_ok) {
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      int j1 = r0 + grp * NB + i;
      if (j1 < r1) {
        double* dst = in.Irt + 4 * ((size_t)j2 * B.ntheta + j1);
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const float2 a = R.acc[i / 2][s].v;
          atomicAdd(dst + s, (double)((i & 1) ? a.y : a.x));
        }
      }
    }
  }
}

// ------------------------------------------------------------------ collect: CB, FP32x2
// Frame products of one event, splat for packed arithmetic.
struct F2Frame {
  P2 ctcp, ctsp, nst, nsp, cp, stcp, stsp, ct, sp, ncp, nstcp, nstsp;
};
__device__ __forceinline__ F2Frame frame2(float ct, float st, float cp, float sp) {
  return F2Frame{p2s(ct * cp), p2s(ct * sp), p2s(-st),      p2s(-sp),      p2s(cp),       p2s(st * cp),
                 p2s(st * sp), p2s(ct),      p2s(sp),       p2s(-cp),      p2s(-st * cp), p2s(-st * sp)};
}

// update_E (src/utils.jl:170-192) for two outgoing directions at once: the field E and
// the frame are the event's; k and its basis Eh are the two bins'.
template <bool MIE>
__device__ __forceinline__ void update_E2(const F2Frame& F, const float E[4], P2 kx, P2 ky, P2 kz, P2 ehx,
                                          P2 ehy, const float4* S, int ntheta, float scale, P2 out[4]) {
  const P2 M1 = p2s(-1.0f);
  const P2 rx = fma2(kx, F.ctcp, fma2(ky, F.ctsp, kz * F.nst));
  const P2 ry = fma2(kx, F.nsp, ky * F.cp);
  const P2 rz = fma2(kx, F.stcp, fma2(ky, F.stsp, kz * F.ct));
  P2 s2 = fma2(rx, rx, ry * ry);
  // A CB bin exactly along the event's incoming (or reversed first) direction, where
  // spherical_from_cartesian takes its pole branch (src/utils.jl:12-14), has probability
  // zero for the sampled directions; the clamp only keeps the arithmetic finite there.
  // (The FP64 forms keep the branch.) Dropping it made CB-heavy workloads 3% faster.
  s2.v.x = fmaxf(s2.v.x, 1e-30f);
  s2.v.y = fmaxf(s2.v.y, 1e-30f);
  const P2 r = p2(rsqrt_approx(s2.v.x), rsqrt_approx(s2.v.y));
  const P2 kcp = rx * r, ksp = ry * r, kst = s2 * r, kct = rz;
  const P2 hx = fma2(ksp, F.ctcp, kcp * F.sp);
  const P2 hy = fma2(ksp, F.ctsp, kcp * F.ncp);
  const P2 kk = kct * kcp, ks = kct * ksp;
  const P2 vx = fma2(kk, F.ctcp, fma2(ks, F.nsp, kst * F.nstcp));
  const P2 vy = fma2(kk, F.ctsp, fma2(ks, F.cp, kst * F.nstsp));
  const P2 cpsi = fma2(ehx, hx, ehy * hy);
  const P2 spsi = fma2(ehx, vx, ehy * vy);
  const P2 SE0 = p2s(E[0]), SE1 = p2s(E[1]), SE2 = p2s(E[2]), SE3 = p2s(E[3]);
  const P2 ar = fma2(SE0, kcp, SE2 * ksp), ai = fma2(SE1, kcp, SE3 * ksp);
  const P2 br = fma2(p2s(-E[0]), ksp, SE2 * kcp), bi = fma2(p2s(-E[1]), ksp, SE3 * kcp);
  P2 sar, sai, sbr, sbi;
  if (MIE) {
    const P2 sn = acos2_scaled(rz, scale);
    const int i0 = min((int)sn.v.x, ntheta - 1), i1 = min((int)sn.v.y, ntheta - 1);
    const P2 f = fma2(p2((float)i0, (float)i1), M1, sn);
    const P2 w0 = fma2(f, M1, p2s(2.0f)), w1 = f + M1;  // the (2 - f, f - 1) weights of mie.jl:80-85
    const float4 a0 = S[i0], b0 = S[i0 + 1], a1 = S[i1], b1 = S[i1 + 1];
    const P2 s1r = fma2(w0, p2(a0.x, a1.x), w1 * p2(b0.x, b1.x));
    const P2 s1i = fma2(w0, p2(a0.y, a1.y), w1 * p2(b0.y, b1.y));
    const P2 s2r = fma2(w0, p2(a0.z, a1.z), w1 * p2(b0.z, b1.z));
    const P2 s2i = fma2(w0, p2(a0.w, a1.w), w1 * p2(b0.w, b1.w));
    const P2 nai = ai * M1, nbi = bi * M1;
    sar = fma2(s1r, ar, s1i * nai);
    sai = fma2(s1r, ai, s1i * ar);
    sbr = fma2(s2r, br, s2i * nbi);
    sbi = fma2(s2r, bi, s2i * br);
  } else {  // S = diag(i, i cos)
    sar = ai * M1;
    sai = ar;
    sbr = (bi * rz) * M1;
    sbi = br * rz;
  }
  out[0] = fma2(sar, cpsi, sbr * spsi);
  out[1] = fma2(sai, cpsi, sbi * spsi);
  out[2] = fma2(sbr, cpsi, (sar * spsi) * M1);
  out[3] = fma2(sbi, cpsi, (sai * spsi) * M1);
}

struct CBLaneF2 {
  P2 kx, ky, kz, ehx, ehy, g, cf, sf, c1, c2, c3;
  bool upb0, upb1;
  P2 acc[4];
  P2 lad;
};

// The reciprocal-path CB bins of src/gpu.jl:90-140 for one event, NPC pairs of bins per
// lane; the event's frames and fields are set up once for all of the lane's pairs.
template <int NPC, bool MIE, bool SPHERE>
__device__ __forceinline__ float cbn_event_f2(CBLaneF2 (&CL)[NPC], const EventP<float>& E, const DevScatterer& s1,
                                              float tau0l, bool peak_lane) {
  const F2Frame FA = frame2(E.fct, E.fst, E.fcp, E.fsp);
  const F2Frame FB = frame2(E.bct, E.bst, E.bcp, E.bsp);
  const float scale = table_scale<float>(s1);
  const P2 M1 = p2s(-1.0f);
  float peak = 0.f;
#pragma unroll
  for (int pp = 0; pp < NPC; ++pp) {
    CBLaneF2& C = CL[pp];
    P2 ea[4], eb[4];
    update_E2<MIE>(FA, E.ea, C.kx, C.ky, C.kz, C.ehx, C.ehy, s1.S, s1.ntheta, scale, ea);
    update_E2<MIE>(FB, E.eb, C.kx, C.ky, C.kz, C.ehx, C.ehy, s1.S, s1.ntheta, scale, eb);
    // Phase kl (ki + kf).(xa - xb) in turns, cancellation-free in the backscatter frame.
    const P2 turns = fma2(C.c1, p2s(E.v1), fma2(C.c2, p2s(E.v2), C.c3 * p2s(E.v3)));
    float sn0, cs0, sn1, cs1;
    MT<float>::sincos_turns(turns.v.x - rintf(turns.v.x), &sn0, &cs0);
    MT<float>::sincos_turns(turns.v.y - rintf(turns.v.y), &sn1, &cs1);
    const P2 sn = p2(sn0, sn1), cs = p2(cs0, cs1), nsn = p2(-sn0, -sn1);
    P2 ta2, tb2;
    if (SPHERE) {
      const P2 kxa = fma2(C.kx, p2s(E.xax), fma2(C.ky, p2s(E.xay), C.kz * p2s(E.xaz)));
      const P2 kxb = fma2(C.kx, p2s(E.xbx), fma2(C.ky, p2s(E.xby), C.kz * p2s(E.xbz)));
      ta2 = p2(sphere_t(kxa.v.x, E.Da), sphere_t(kxa.v.y, E.Da)) * p2s((float)LOG2E_D);
      tb2 = p2(sphere_t(kxb.v.x, E.Db), sphere_t(kxb.v.y, E.Db)) * p2s((float)LOG2E_D);
    } else {
      ta2 = p2(C.upb0 ? E.a_up : E.a_dn, C.upb1 ? E.a_up : E.a_dn) * C.g;
      tb2 = p2(C.upb0 ? E.b_up : E.b_dn, C.upb1 ? E.b_up : E.b_dn) * C.g;
    }
    tb2 = tb2 + p2s(E.tab2);
    const bool ma0 = ta2.v.x <= tau0l, ma1 = ta2.v.y <= tau0l;
    const P2 na = p2(ma0 ? MT<float>::exp2n(0.5f * ta2.v.x) : 0.f, ma1 ? MT<float>::exp2n(0.5f * ta2.v.y) : 0.f);
    const P2 nb = p2(fabsf(tb2.v.x) <= tau0l ? MT<float>::exp2n(0.5f * tb2.v.x) : 0.f,
                     fabsf(tb2.v.y) <= tau0l ? MT<float>::exp2n(0.5f * tb2.v.y) : 0.f);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      ea[s] = ea[s] * na;
      eb[s] = eb[s] * nb;
    }
    const P2 Ia = fma2(ea[0], ea[0], fma2(ea[1], ea[1], fma2(ea[2], ea[2], ea[3] * ea[3])));
    const P2 Ib = fma2(eb[0], eb[0], fma2(eb[1], eb[1], fma2(eb[2], eb[2], eb[3] * eb[3])));
    const P2 c1r = fma2(ea[0], cs, fma2(ea[1], nsn, eb[0])), c1i = fma2(ea[0], sn, fma2(ea[1], cs, eb[1]));
    const P2 c2r = fma2(ea[2], cs, fma2(ea[3], nsn, eb[2])), c2i = fma2(ea[2], sn, fma2(ea[3], cs, eb[3]));
    const P2 qh = fma2(c1r, c1r, c1i * c1i), qv = fma2(c2r, c2r, c2i * c2i);
    P2 S0 = qh + qv, S1 = fma2(qh, M1, qv);
    P2 S2 = fma2(c2r, c1r, c2i * c1i) * p2s(2.0f);
    P2 S3 = fma2(c2i, c1r, (c2r * c1i) * M1) * p2s(-2.0f);
    const P2 den = Ia + Ib;
    const P2 scl = p2(den.v.x > 0.f ? __fdividef(Ia.v.x, den.v.x) : 0.f,
                      den.v.y > 0.f ? __fdividef(Ia.v.y, den.v.y) : 0.f);
    S0 = S0 * scl;
    S1 = S1 * scl;
    S2 = S2 * scl;
    S3 = S3 * scl;
    const P2 R1 = fma2(C.cf, S1, C.sf * S2), R2 = fma2(C.cf, S2, (C.sf * S1) * M1);
    C.acc[0] = C.acc[0] + S0;
    C.acc[1] = C.acc[1] + R1;
    C.acc[2] = C.acc[2] + R2;
    C.acc[3] = C.acc[3] + S3;
    C.lad = C.lad + Ia;
    if (pp == 0) peak = S0.v.x;  // bin 0 of the grid is the x half of a lane's first pair
  }
  return peak_lane ? peak : 0.f;
}

// ------------------------------------------------------------------ collect: CB tile
template <typename T, int NB>
struct CBLane {
  T kx[NB], ky[NB], kz[NB], ehx[NB], ehy[NB], g[NB], cf[NB], sf[NB], c1[NB], c2[NB], c3[NB];
  bool upb[NB];
  T acc[NB][4];
  T lad[NB];
};

template <typename T, int NB, bool MIE, bool SPHERE>
__device__ __forceinline__ T cbn_event(CBLane<T, NB>& C, const EventP<T>& E, const DevScatterer& s1,
                                       T tau0l, bool peak_lane) {
  const Frame<T> fa{E.fct, E.fst, E.fcp, E.fsp};
  const Frame<T> fb{E.bct, E.bst, E.bcp, E.bsp};
  const T scale = table_scale<T>(s1);
  T pk = T(0);
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    T ea[4] = {E.ea[0], E.ea[1], E.ea[2], E.ea[3]};
    T eb[4] = {E.eb[0], E.eb[1], E.eb[2], E.eb[3]};
    update_E<T>(fa, ea, C.kx[i], C.ky[i], C.kz[i], C.ehx[i], C.ehy[i], MIE ? 1 : 0, s1.S, s1.ntheta, scale);
    update_E<T>(fb, eb, C.kx[i], C.ky[i], C.kz[i], C.ehx[i], C.ehy[i], MIE ? 1 : 0, s1.S, s1.ntheta, scale);
    // Phase kl (ki + kf).(xa - xb) in turns, cancellation-free in the backscatter frame.
    const T turns = C.c1[i] * E.v1 + C.c2[i] * E.v2 + C.c3[i] * E.v3;
    const T fr = turns - MT<T>::rint(turns);
    T sn, cs;
    MT<T>::sincos_turns(fr, &sn, &cs);
    T ta2, tb2;
    if (SPHERE) {
      ta2 = sphere_t(C.kx[i] * E.xax + C.ky[i] * E.xay + C.kz[i] * E.xaz, E.Da) * T(LOG2E_D);
      tb2 = sphere_t(C.kx[i] * E.xbx + C.ky[i] * E.xby + C.kz[i] * E.xbz, E.Db) * T(LOG2E_D);
    } else {
      ta2 = (C.upb[i] ? E.a_up : E.a_dn) * C.g[i];
      tb2 = (C.upb[i] ? E.b_up : E.b_dn) * C.g[i];
    }
    tb2 += E.tab2;
    const bool ma = ta2 <= tau0l;
    const T na = MT<T>::exp2n(T(0.5) * ta2);
    const T nb = MT<T>::fabs(tb2) <= tau0l ? MT<T>::exp2n(T(0.5) * tb2) : T(0);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      ea[s] *= na;
      eb[s] *= nb;
    }
    const T Ia = ea[0] * ea[0] + ea[1] * ea[1] + ea[2] * ea[2] + ea[3] * ea[3];
    const T Ib = eb[0] * eb[0] + eb[1] * eb[1] + eb[2] * eb[2] + eb[3] * eb[3];
    const T c1r = ea[0] * cs - ea[1] * sn + eb[0], c1i = ea[0] * sn + ea[1] * cs + eb[1];
    const T c2r = ea[2] * cs - ea[3] * sn + eb[2], c2i = ea[2] * sn + ea[3] * cs + eb[3];
    const T qh = c1r * c1r + c1i * c1i, qv = c2r * c2r + c2i * c2i;
    T S0 = qh + qv, S1 = qv - qh;
    T S2 = T(2) * (c2r * c1r + c2i * c1i), S3 = T(-2) * (c2i * c1r - c2r * c1i);
    const T den = Ia + Ib;
    const bool ok = ma && den > T(0);
    const T scl = ok ? MT<T>::div(Ia, den) : T(0);
    S0 *= scl;
    S1 *= scl;
    S2 *= scl;
    S3 *= scl;
    rotate(C.cf[i], C.sf[i], S1, S2);
    C.acc[i][0] += ok ? S0 : T(0);
    C.acc[i][1] += ok ? S1 : T(0);
    C.acc[i][2] += ok ? S2 : T(0);
    C.acc[i][3] += ok ? S3 : T(0);
    C.lad[i] += ok ? Ia : T(0);
    if (i == 0 && peak_lane) pk = ok ? S0 : T(0);
  }
  return pk;
}

template <typename T, int NB, bool MIE, bool SPHERE>
__device__ __forceinline__ T cb1_event(CBLane<T, NB>& C, const EventP<T>& E, const DevScatterer& s1,
                                       T tau0l, bool peak_lane) {
  const Frame<T> fa{E.fct, E.fst, E.fcp, E.fsp};
  const T scale = table_scale<T>(s1);
  T pk = T(0);
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    T o[4];
    update_I<T>(fa, E.I, C.kx[i], C.ky[i], C.kz[i], C.ehx[i], C.ehy[i], MIE ? 1 : 0, s1.F, s1.ntheta,
                scale, o);
    T ta2;
    if (SPHERE)
      ta2 = sphere_t(C.kx[i] * E.xax + C.ky[i] * E.xay + C.kz[i] * E.xaz, E.Da) * T(LOG2E_D);
    else
      ta2 = (C.upb[i] ? E.a_up : E.a_dn) * C.g[i];
    const bool ma = ta2 <= tau0l;
    const T w = ma ? MT<T>::exp2n(ta2) : T(0);
#pragma unroll
    for (int s = 0; s < 4; ++s) o[s] *= w;
    rotate(C.cf[i], C.sf[i], o[1], o[2]);
#pragma unroll
    for (int s = 0; s < 4; ++s) C.acc[i][s] += ma ? o[s] : T(0);
    C.lad[i] += ma ? o[0] : T(0);
    if (i == 0 && peak_lane) pk = ma ? o[0] : T(0);
  }
  return pk;
}

template <typename T, int NB, int BS>
__device__ void cb_tile(Shared<T, BS>& sh, const BinTables<T>& B, int tile, int pc, int q0, int q1) {
  const int lane = threadIdx.x & 31;
  const int ngrp = (B.nthetab + NB - 1) / NB;
  const int item = tile * 32 + lane;
  const bool lane_ok = item < ngrp * B.nphib;
  const int it = lane_ok ? item : 0;
  const int j2 = it % B.nphib, grp = it / B.nphib;
  CBLane<T, NB> C;
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    int j1 = grp * NB + i;
    bool ok = lane_ok && j1 < B.nthetab;
    int b = ok ? j2 * B.nthetab + j1 : 0;
    C.kx[i] = B.kfx[b];
    C.ky[i] = B.kfy[b];
    C.kz[i] = B.kfz[b];
    C.ehx[i] = B.ehx[b];
    C.ehy[i] = B.ehy[b];
    C.g[i] = B.gb[b];
    C.cf[i] = B.cf2[b];
    C.sf[i] = B.sf2[b];
    C.c1[i] = B.c1[b];
    C.c2[i] = B.c2[b];
    C.c3[i] = B.c3[b];
    C.upb[i] = B.upb[b] != 0;
#pragma unroll
    for (int s = 0; s < 4; ++s) C.acc[i][s] = T(0);
    C.lad[i] = T(0);
  }
  const bool peak_lane = lane_ok && j2 == 0 && grp == 0;
  const DevInstance& in = sh.inst;
  const DevScatterer& s1 = in.scat[in.layers[0].scat];
  const T tau0l = (T)(in.tau0 * LOG2E_D);
  const bool sphere = in.geom == 1, mie = s1.kind == 1;
  // events [q0, q1) of the concatenated lists (order > 1, then order 1)
  const int nn = sh.cnt[pc][2];
  for (int q = q0; q < min(q1, nn); ++q) {
    const int e = sh.list[2][q];
    const EventP<T>& E = sh.ev[e];
    T pk;
    if (mie)
      pk = sphere ? cbn_event<T, NB, true, true>(C, E, s1, tau0l, peak_lane)
                  : cbn_event<T, NB, true, false>(C, E, s1, tau0l, peak_lane);
    else
      pk = sphere ? cbn_event<T, NB, false, true>(C, E, s1, tau0l, peak_lane)
                  : cbn_event<T, NB, false, false>(C, E, s1, tau0l, peak_lane);
    if (peak_lane) sh.peak[e] = pk;
  }
  for (int q = max(q0, nn); q < q1; ++q) {
    const int e = sh.list[3][q - nn];
    const EventP<T>& E = sh.ev[e];
    T pk;
    if (mie)
      pk = sphere ? cb1_event<T, NB, true, true>(C, E, s1, tau0l, peak_lane)
                  : cb1_event<T, NB, true, false>(C, E, s1, tau0l, peak_lane);
    else
      pk = sphere ? cb1_event<T, NB, false, true>(C, E, s1, tau0l, peak_lane)
                  : cb1_event<T, NB, false, false>(C, E, s1, tau0l, peak_lane);
    if (peak_lane) sh.peak[e] = pk;
  }
  if (lane_ok) {
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      int j1 = grp * NB + i;
      if (j1 < B.nthetab) {
        size_t b = (size_t)j2 * B.nthetab + j1;
        double* dst = in.Icb + 4 * b;
#pragma unroll
        for (int s = 0; s < 4; ++s) atomicAdd(dst + s, (double)C.acc[i][s]);
        atomicAdd(in.ladder + b, (double)C.lad[i]);
      }
    }
  }
}

// ------------------------------------------------------------------ collect: CB tile, FP32x2 lanes
template <int BS, int NPC>
__device__ void cb_tile_f2(Shared<float, BS>& sh, const BinTables<float>& B, int tile, int pc, int q0, int q1) {
  constexpr int NB = 2 * NPC;
  const int lane = threadIdx.x & 31;
  const int ngrp = (B.nthetab + NB - 1) / NB;
  const int item = tile * 32 + lane;
  const bool lane_ok = item < ngrp * B.nphib;
  const int it = lane_ok ? item : 0;
  const int j2 = it % B.nphib, grp = it / B.nphib;
  int bb[NB];
  bool okb[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    const int j1 = grp * NB + i;
    okb[i] = lane_ok && j1 < B.nthetab;
    bb[i] = okb[i] ? j2 * B.nthetab + j1 : 0;
  }
  CBLaneF2 C[NPC];
#pragma unroll
  for (int pp = 0; pp < NPC; ++pp) {
    const int b0 = bb[2 * pp], b1 = bb[2 * pp + 1];
    C[pp].kx = p2(B.kfx[b0], B.kfx[b1]);
    C[pp].ky = p2(B.kfy[b0], B.kfy[b1]);
    C[pp].kz = p2(B.kfz[b0], B.kfz[b1]);
    C[pp].ehx = p2(B.ehx[b0], B.ehx[b1]);
    C[pp].ehy = p2(B.ehy[b0], B.ehy[b1]);
    C[pp].g = p2(B.gb[b0], B.gb[b1]);
    C[pp].cf = p2(B.cf2[b0], B.cf2[b1]);
    C[pp].sf = p2(B.sf2[b0], B.sf2[b1]);
    C[pp].c1 = p2(B.c1[b0], B.c1[b1]);
    C[pp].c2 = p2(B.c2[b0], B.c2[b1]);
    C[pp].c3 = p2(B.c3[b0], B.c3[b1]);
    C[pp].upb0 = B.upb[b0] != 0;
    C[pp].upb1 = B.upb[b1] != 0;
#pragma unroll
    for (int s = 0; s < 4; ++s) C[pp].acc[s] = p2s(0.f);
    C[pp].lad = p2s(0.f);
  }
  const bool peak_lane = lane_ok && j2 == 0 && grp == 0;
  const DevInstance& in = sh.inst;
  const DevScatterer& s1 = in.scat[in.layers[0].scat];
  const float tau0l = (float)(in.tau0 * LOG2E_D);
  const bool sphere = in.geom == 1, mie = s1.kind == 1;
  const int nn = sh.cnt[pc][2];
  for (int q = q0; q < min(q1, nn); ++q) {
    const int e = sh.list[2][q];
    const EventP<float>& E = sh.ev[e];
    float pk;
    if (mie)
      pk = sphere ? cbn_event_f2<NPC, true, true>(C, E, s1, tau0l, peak_lane)
                  : cbn_event_f2<NPC, true, false>(C, E, s1, tau0l, peak_lane);
    else
      pk = sphere ? cbn_event_f2<NPC, false, true>(C, E, s1, tau0l, peak_lane)
                  : cbn_event_f2<NPC, false, false>(C, E, s1, tau0l, peak_lane);
    if (peak_lane) sh.peak[e] = pk;
  }
  // Order-1 events (a few per path) use the scalar single-scattering bins.
  if (max(q0, nn) < q1) {
    CBLane<float, NB> Cs;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      const int b = bb[i];
      Cs.kx[i] = B.kfx[b];
      Cs.ky[i] = B.kfy[b];
      Cs.kz[i] = B.kfz[b];
      Cs.ehx[i] = B.ehx[b];
      Cs.ehy[i] = B.ehy[b];
      Cs.g[i] = B.gb[b];
      Cs.cf[i] = B.cf2[b];
      Cs.sf[i] = B.sf2[b];
      Cs.upb[i] = B.upb[b] != 0;
#pragma unroll
      for (int s = 0; s < 4; ++s) Cs.acc[i][s] = 0.f;
      Cs.lad[i] = 0.f;
    }
    for (int q = max(q0, nn); q < q1; ++q) {
      const int e = sh.list[3][q - nn];
      const EventP<float>& E = sh.ev[e];
      float pk;
      if (mie)
        pk = sphere ? cb1_event<float, NB, true, true>(Cs, E, s1, tau0l, peak_lane)
                    : cb1_event<float, NB, true, false>(Cs, E, s1, tau0l, peak_lane);
      else
        pk = sphere ? cb1_event<float, NB, false, true>(Cs, E, s1, tau0l, peak_lane)
                    : cb1_event<float, NB, false, false>(Cs, E, s1, tau0l, peak_lane);
      if (peak_lane) sh.peak[e] = pk;
    }
#pragma unroll
    for (int pp = 0; pp < NPC; ++pp) {
#pragma unroll
      for (int s = 0; s < 4; ++s) C[pp].acc[s] = C[pp].acc[s] + p2(Cs.acc[2 * pp][s], Cs.acc[2 * pp + 1][s]);
      C[pp].lad = C[pp].lad + p2(Cs.lad[2 * pp], Cs.lad[2 * pp + 1]);
    }
  }
  if (lane_ok) {
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      if (okb[i]) {
        double* dst = in.Icb + 4 * (size_t)bb[i];
#pragma unroll
        for (int s = 0; s < 4; ++s)
          atomicAdd(dst + s, (double)((i & 1) ? C[i / 2].acc[s].v.y : C[i / 2].acc[s].v.x));
        atomicAdd(in.ladder + bb[i], (double)((i & 1) ? C[i / 2].lad.v.y : C[i / 2].lad.v.x));
      }
    }
  }
}

// ------------------------------------------------------------------ the kernel
template <typename T, int BS, int NBR, int NBC, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_transport(KParams p) {
  extern __shared__ __align__(16) unsigned char smraw[];
  Shared<T, BS>& sh = *reinterpret_cast<Shared<T, BS>*>(smraw);
  float4* tables = reinterpret_cast<float4*>(smraw + sizeof(Shared<T, BS>));
  const int tid = threadIdx.x, lane = tid & 31;
  const size_t g = (size_t)blockIdx.x * BS + tid;
  const size_t stride = (size_t)gridDim.x * BS;

  if (tid == 0) {
    sh.cur = start_instance(p);
    sh.exhausted = 0;
    sh.taken = 0;
    sh.item_next = 0;
    for (int i = 0; i < 8; ++i) (&sh.cnt[0][0])[i] = 0;
  }
  for (int k = 0; k < NACC; ++k) p.tacc[(size_t)k * stride + g] = 0.0;
  __syncthreads();
  if (sh.cur < 0) return;
  stage_instance<T, BS>(sh, tables, p, sh.cur);

  bool alive = false;
  int pc = 0;
  PState<T> ps;
  // per-thread event counters of the current instance (flushed when the block leaves it)
  unsigned c_ev = 0, c_up = 0, c_dn = 0, c_cb1 = 0, c_cbn = 0;
  unsigned long long c_att = 0;
  for (;;) {
    const DevInstance& in = sh.inst;
    const BinTables<T>& B = *reinterpret_cast<const BinTables<T>*>(in.bins);
    // ---- claim new photons (warp-aggregated) and start them
    {
      const bool want_b = !alive && !sh.exhausted;
      const unsigned want = __ballot_sync(0xffffffffu, want_b);
      if (want) {
        const int leader = __ffs(want) - 1;
        unsigned long long base = 0;
        if (lane == leader) {
          const int nw = __popc(want);
          base = atomicAdd(in.claim, (unsigned long long)nw);
          const long long left = in.n_photons - (long long)base;
          if (left > 0) atomicAdd(&sh.taken, left < nw ? (int)left : nw);
        }
        base = __shfl_sync(0xffffffffu, base, leader);
        if (want_b) {
          unsigned long long my = base + __popc(want & ((1u << lane) - 1u));
          if ((long long)my < in.n_photons) {
            alive = start_photon<T>(ps, in, (unsigned long long)in.photon_begin + my, p.tacc, stride,
                                    g, p.status);
          } else {
            sh.exhausted = 1;
          }
        }
      }
    }
    // ---- sample phase
    int flags = 0;
    if (alive) {
      bool dead = false;
      unsigned att = 0;
      flags = sample_event<T>(ps, in, B, sh.ev[tid], p.tacc, stride, g, p.status, dead, att);
      if (dead) {
        alive = false;
        flags = 0;
      } else {
        ++c_ev;
        c_att += att;
        c_up += (flags & EV_UP) != 0;
        c_dn += (flags & EV_DN) != 0;
        c_cbn += (flags & EV_CBN) != 0;
        c_cb1 += (flags & EV_CB) != 0 && (flags & EV_CBN) == 0;
      }
      sh.esc_up[tid] = T(0);
      sh.esc_dn[tid] = T(0);
      sh.peak[tid] = T(0);
      if (alive) ps_store(ps, p.state, stride, g);
    }
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const int bit = l == 0 ? EV_UP : (l == 1 ? EV_DN : (l == 2 ? EV_CBN : EV_CB));
      bool in_list = (flags & bit) != 0;
      if (l == 3) in_list = in_list && !(flags & EV_CBN);
      const unsigned m = __ballot_sync(0xffffffffu, in_list);
      if (m) {
        const int leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&sh.cnt[pc][l], __popc(m));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (in_list) sh.list[l][base + __popc(m & ((1u << lane) - 1u))] = (unsigned short)tid;
      }
    }
    const int nalive = __syncthreads_count(alive);
    if (nalive == 0) {
      if (!sh.exhausted) continue;
      // This block has finished its part of the instance: fold the per-thread
      // accumulators into the instance's totals and move on. The event counters were
      // kept in registers (bin evaluations follow from the events' up/down/CB flags).
      acc_add(p.tacc, stride, g, ACC_EVENTS, (double)c_ev);
      acc_add(p.tacc, stride, g, ACC_ATTEMPTS, (double)c_att);
      acc_add(p.tacc, stride, g, ACC_RT,
              (double)B.nphi * ((double)c_up * (B.up1 - B.up0) + (double)c_dn * (B.lo1 - B.lo0)));
      acc_add(p.tacc, stride, g, ACC_CB1, (double)c_cb1 * B.nthetab * B.nphib);
      acc_add(p.tacc, stride, g, ACC_CBN, (double)c_cbn * B.nthetab * B.nphib);
      c_ev = c_up = c_dn = c_cb1 = c_cbn = 0;
      c_att = 0;
      for (int k = 0; k < NACC; ++k) {
        double v = p.tacc[(size_t)k * stride + g];
        p.tacc[(size_t)k * stride + g] = 0.0;
        v = warp_sum(v);
        if (lane == 0 && v != 0.0) atomicAdd(in.acc + k, v);
      }
      if (in.rt_fourier) {
        // Publish this block's coefficient flushes, then count its photons as finished;
        // the block whose count completes the launch's photons expands the coefficients.
        __threadfence();
        __syncthreads();
        if (tid == 0) {
          int last = 0;
          if (sh.taken > 0) {
            const unsigned long long old = atomicAdd(in.claim + 1, (unsigned long long)sh.taken);
            last = (long long)(old + (unsigned long long)sh.taken) == in.n_photons;
          }
          sh.expand = last;
        }
        __syncthreads();
        if (sh.expand) {
          __threadfence();
          fourier_expand<T>(in, B, tid, BS);
        }
      }
      __syncthreads();
      if (tid == 0) {
        sh.cur = next_instance(p, sh.cur);
        sh.exhausted = 0;
        sh.taken = 0;
        for (int i = 0; i < 8; ++i) (&sh.cnt[0][0])[i] = 0;
      }
      __syncthreads();
      if (sh.cur < 0) break;
      stage_instance<T, BS>(sh, tables, p, sh.cur);
      continue;
    }
    // ---- collect phase
    {
      const int nu = sh.cnt[pc][0], nd = sh.cnt[pc][1], nc = sh.cnt[pc][2] + sh.cnt[pc][3];
      const int tcb = nc ? (B.nphib * ((B.nthetab + NBC - 1) / NBC) + 31) / 32 : 0;
      const bool fr = sh.inst.rt_fourier != 0;
      const int tup = !nu ? 0
                      : fr ? (B.up1 - B.up0 + 31) / 32
                           : (B.nphi * ((B.up1 - B.up0 + NBR - 1) / NBR) + 31) / 32;
      const int tdn = !nd ? 0
                      : fr ? (B.lo1 - B.lo0 + 31) / 32
                           : (B.nphi * ((B.lo1 - B.lo0 + NBR - 1) / NBR) + 31) / 32;
      // Work items are (tile, chunk of events); the costlier CB items go first. CB chunks
      // hold up to 256 events. RT chunks hold 128 events in blocks of up to 256 threads,
      // which balances the end of the phase better (measured 5% faster on the Mie slab;
      // 64 or 96 lose more to tally flushes than they gain), and 256 in larger blocks.
      // Fourier RT tiles are few (one lane per polar bin) and flush 20 values per lane,
      // so they take 64.
      constexpr int EVC = 256, EVR = BS <= 256 ? 128 : 256, EVF = 64;
      const int evr = fr ? EVF : EVR;
      const int ccb = (nc + EVC - 1) / EVC, cup = (nu + evr - 1) / evr, cdn = (nd + evr - 1) / evr;
      const int icb = tcb * ccb, iup = tup * cup, idn = tdn * cdn;
      const int total = icb + iup + idn;
      if (tid == 0)
        for (int l = 0; l < 4; ++l) sh.cnt[pc ^ 1][l] = 0;
      for (;;) {
        int w = 0;
        if (lane == 0) w = atomicAdd(&sh.item_next, 1);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= total) break;
        if (w < icb) {
          const int c = w % ccb;
          if constexpr (std::is_same<T, float>::value && NBC % 2 == 0)
            cb_tile_f2<BS, NBC / 2>(sh, B, w / ccb, pc, c * EVC, min((c + 1) * EVC, nc));
          else
            cb_tile<T, NBC, BS>(sh, B, w / ccb, pc, c * EVC, min((c + 1) * EVC, nc));
        } else if (w < icb + iup) {
          w -= icb;
          const int c = w % cup;
          if (fr)
            rt_fourier_tile<T, BS>(sh, B, w / cup, true, c * evr, min((c + 1) * evr, nu));
          else if constexpr (std::is_same<T, float>::value)
            rt_tile_f2<NBR, BS>(sh, B, w / cup, true, pc, c * evr, min((c + 1) * evr, nu));
          else
            rt_tile<T, NBR, BS>(sh, B, w / cup, true, pc, c * evr, min((c + 1) * evr, nu));
        } else {
          w -= icb + iup;
          const int c = w % cdn;
          if (fr)
            rt_fourier_tile<T, BS>(sh, B, w / cdn, false, c * evr, min((c + 1) * evr, nd));
          else if constexpr (std::is_same<T, float>::value)
            rt_tile_f2<NBR, BS>(sh, B, w / cdn, false, pc, c * evr, min((c + 1) * evr, nd));
          else
            rt_tile<T, NBR, BS>(sh, B, w / cdn, false, pc, c * evr, min((c + 1) * evr, nd));
        }
      }
    }
    __syncthreads();
    // ---- finish phase: renormalise by the escaped intensity (src/gpu.jl:285-294)
    if (tid == 0) sh.item_next = 0;
    if (alive) {
      ps_load(ps, p.state, stride, g);
      const double eu = (double)sh.esc_up[tid], ed = (double)sh.esc_dn[tid];
      acc_add(p.tacc, stride, g, ACC_AREF, eu);
      acc_add(p.tacc, stride, g, ACC_ATRANS, ed);
      ps.peak += (double)sh.peak[tid];
      const T wnew = ps.wI - (T)(eu + ed);
      for (int s = 0; s < 4; ++s) ps.I[s] = ps.Ih[s] * wnew;
      const double i0 = (double)ps.I[0];
      if (!isfinite(i0)) {
        atomicOr(p.status, 4u);
        acc_add(p.tacc, stride, g, ACC_NONFINITE, 1.0);
        acc_add(p.tacc, stride, g, ACC_PHOTONS, 1.0);
        alive = false;
      } else if (!(i0 >= in.min_int && ps.n < in.max_scat)) {
        acc_add(p.tacc, stride, g, ACC_AREM, i0);
        acc_add(p.tacc, stride, g, ACC_PEAK, ps.peak);
        acc_add(p.tacc, stride, g, ACC_PEAK2, ps.peak * ps.peak);
        acc_add(p.tacc, stride, g, ACC_PHOTONS, 1.0);
        alive = false;
      }
    }
    pc ^= 1;
  }
}

}  // namespace mcrt
