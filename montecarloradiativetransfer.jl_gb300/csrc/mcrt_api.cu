// C ABI of libmcrt (declared in include/mcrt.h): device context, scatterer upload,
// resident solves, batched persistent launches and the drop-in mcrt_simulate.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "mcrt.h"
#include "mcrt_device.cuh"
#include "mcrt_host.h"
#include "mcrt_kernels.h"
#include "mcrt_mie.cuh"

using namespace mcrt;

namespace {
// NVTX range for the host-side phases (upload, launch, read-back, serving waves), so a
// timeline profiler shows them beside the kernels. Costs nothing without a tool attached.
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
};
}  // namespace

namespace {

thread_local std::string g_err;

int set_err(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return set_err(e_ == cudaErrorMemoryAllocation ? MCRT_ENOMEM : MCRT_ECUDA,          \
                     std::string(#call) + ": " + cudaGetErrorString(e_));                 \
  } while (0)

// A host-to-device copy that has landed when it returns, ordered on `st`. A plain
// cudaMemcpy from pageable memory may return before its DMA reaches the device, and it
// runs on the legacy default stream, which a context's non-blocking stream does not wait
// for: a later copy to the same buffer on that stream could then be overwritten by the
// earlier one (seen as a solve's first launch running its creation-time photon range
// while another process shared the GPU).
inline cudaError_t upload_sync(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
  return e != cudaSuccess ? e : cudaStreamSynchronize(st);
}

struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t bytes) {
    release();
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) n = bytes;
    else p = nullptr;
    return e;
  }
  template <typename U>
  U* as() const {
    return reinterpret_cast<U*>(p);
  }
};

}  // namespace

// ================================================================== context / scatterers
struct mcrt_ctx {
  int device = 0;
  int sms = 0;
  int smem_optin = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::mutex mu;
  struct Tuned {
    int bs, bpsm, staging;
    double paths_per_ms;
  };
  std::map<std::string, Tuned> tuned;  // workload signature -> fastest launch shape
  unsigned char* noalloc_scratch = nullptr;  // device address of mcrt_simulate_noalloc's array
};

struct mcrt_scatterer {
  mcrt_ctx* ctx = nullptr;
  int kind = 0;
  double omega = 1, kl = 1;
  int ntheta = 0, rp = 0;
  DevBuf F, S, C;
  DevScatterer view() const {
    DevScatterer d{};
    d.kind = kind;
    d.ntheta = ntheta;
    d.rp = rp;
    d.kl = kl;
    d.scaled = ntheta > 1 ? (ntheta - 1) / host::PI : 0.0;
    d.scalef = (float)d.scaled;
    d.F = F.as<const float4>();
    d.S = S.as<const float4>();
    d.csrn = C.as<const float>();
    return d;
  }
};

extern "C" {

int mcrt_abi_version(void) { return MCRT_ABI_VERSION; }

const char* mcrt_last_error(void) { return g_err.c_str(); }

int mcrt_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

namespace {
int noalloc_prepare(mcrt_ctx* ctx);
}

int mcrt_ctx_create(int device, mcrt_ctx** out) {
  if (!out) return set_err(MCRT_EINVAL, "mcrt_ctx_create: out is NULL");
  *out = nullptr;
  int n = mcrt_device_count();
  if (n <= 0) return set_err(MCRT_ENODEV, "no CUDA device is visible");
  if (device < 0 || device >= n) return set_err(MCRT_EINVAL, "device index out of range");
  std::unique_ptr<mcrt_ctx> c(new mcrt_ctx());
  c->device = device;
  CK(cudaSetDevice(device));
  CK(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device));
  CK(cudaDeviceGetAttribute(&c->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CK(cudaEventCreate(&c->e0));
  CK(cudaEventCreate(&c->e1));
  // Everything mcrt_simulate_noalloc needs on the device is made resident now, so that
  // its calls allocate nothing even where modules load lazily.
  int rc = noalloc_prepare(c.get());
  if (rc) return rc;
  *out = c.release();
  return MCRT_OK;
}

int mcrt_ctx_destroy(mcrt_ctx* ctx) {
  if (!ctx) return MCRT_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->e0) cudaEventDestroy(ctx->e0);
  if (ctx->e1) cudaEventDestroy(ctx->e1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MCRT_OK;
}

int mcrt_scatterer_create(mcrt_ctx* ctx, const mcrt_scatterer_desc* d, mcrt_scatterer** out) {
  if (!ctx || !d || !out) return set_err(MCRT_EINVAL, "mcrt_scatterer_create: NULL argument");
  *out = nullptr;
  if (d->kind != MCRT_RAYLEIGH && d->kind != MCRT_MIE)
    return set_err(MCRT_EINVAL, "unknown scatterer kind");
  if (!(d->kl > 0) || !std::isfinite(d->kl))
    return set_err(MCRT_EINVAL, "scatterer mean free path kl must be positive");
  std::unique_ptr<mcrt_scatterer> s(new mcrt_scatterer());
  s->ctx = ctx;
  s->kind = d->kind;
  s->omega = d->omega;
  s->kl = d->kl;
  CK(cudaSetDevice(ctx->device));
  if (d->kind == MCRT_MIE) {
    if (d->n_theta < 2 || d->random_points < 1)
      return set_err(MCRT_EINVAL, "Mie tables need n_theta >= 2 and random_points >= 1");
    if (!d->F11 || !d->F12 || !d->F33 || !d->F34 || !d->S11 || !d->S22 || !d->csrn)
      return set_err(MCRT_EINVAL, "Mie table pointer is NULL");
    s->ntheta = d->n_theta;
    s->rp = d->random_points;
    const int nf = d->n_theta + 1;
    std::vector<float4> F(nf, make_float4(0, 0, 0, 0)), S(nf, make_float4(0, 0, 0, 0));
    for (int i = 0; i < d->n_theta; ++i) {
      F[i] = make_float4((float)d->F11[i], (float)d->F12[i], (float)d->F33[i], (float)d->F34[i]);
      S[i] = make_float4((float)d->S11[2 * i], (float)d->S11[2 * i + 1], (float)d->S22[2 * i],
                         (float)d->S22[2 * i + 1]);
    }
    const int nc = ((d->random_points + 2 + 3) / 4) * 4;
    std::vector<float> C(nc, 0.0f);
    for (int i = 0; i <= d->random_points; ++i) C[i] = (float)d->csrn[i];
    C[d->random_points + 1] = C[d->random_points];
    CK(s->F.alloc(nf * sizeof(float4)));
    CK(s->S.alloc(nf * sizeof(float4)));
    CK(s->C.alloc(nc * sizeof(float)));
    CK(upload_sync(s->F.p, F.data(), nf * sizeof(float4), ctx->stream));
    CK(upload_sync(s->S.p, S.data(), nf * sizeof(float4), ctx->stream));
    CK(upload_sync(s->C.p, C.data(), nc * sizeof(float), ctx->stream));
  }
  *out = s.release();
  return MCRT_OK;
}

int mcrt_scatterer_params(const mcrt_scatterer* s, double* omega, double* kl) {
  if (!s) return set_err(MCRT_EINVAL, "mcrt_scatterer_params: NULL scatterer");
  if (omega) *omega = s->omega;
  if (kl) *kl = s->kl;
  return MCRT_OK;
}

int mcrt_scatterer_destroy(mcrt_scatterer* s) {
  if (!s) return MCRT_OK;
  cudaSetDevice(s->ctx->device);
  delete s;
  return MCRT_OK;
}

int mcrt_mie_tables(double r, double m_re, double m_im, double lambda, double nu, int n_theta,
                    int random_points, double* omega, double* kl, double* F11, double* F12,
                    double* F33, double* F34, double* S11, double* S22, double* csrn, double* q) {
  if (!(r > 0) || !(lambda > 0) || !(nu > 0) || n_theta < 2 || random_points < 1)
    return set_err(MCRT_EINVAL, "mcrt_mie_tables: need r, lambda, nu > 0, n_theta >= 2, random_points >= 1");
  const double x = 2 * host::PI * r / lambda;  // mie.jl:37
  host::MieResult R = host::bhmie(x, host::cplx(m_re, m_im), n_theta);
  if (omega) *omega = R.q_sca / R.q_ext;                   // mie.jl:39
  if (kl) *kl = ((4.0 / 3.0) * r) / (nu * R.q_ext);        // mie.jl:40
  for (int i = 0; i < n_theta; ++i) {
    if (F11) F11[i] = R.F11[i];
    if (F12) F12[i] = R.F12[i];
    if (F33) F33[i] = R.F33[i];
    if (F34) F34[i] = R.F34[i];
    if (S11) {
      S11[2 * i] = R.S1[i].real();
      S11[2 * i + 1] = R.S1[i].imag();
    }
    if (S22) {
      S22[2 * i] = R.S2[i].real();
      S22[2 * i + 1] = R.S2[i].imag();
    }
  }
  if (csrn) {
    std::vector<double> c = host::calculate_csrn(R.F11, random_points);  // mie.jl:41-42
    std::copy(c.begin(), c.end(), csrn);
  }
  if (q) {
    q[0] = R.q_ext;
    q[1] = R.q_sca;
    q[2] = R.q_abs;
    q[3] = R.q_back;
    q[4] = R.asymm;
  }
  return MCRT_OK;
}

int mcrt_mie_scatterers_create(mcrt_ctx* ctx, int n, const double* r, const double* m_re, const double* m_im,
                               const double* lambda, const double* nu, int n_theta, int random_points,
                               mcrt_scatterer** out, double* tables) {
  if (!ctx || n < 1 || !r || !m_re || !m_im || !lambda || !nu || !out)
    return set_err(MCRT_EINVAL, "mcrt_mie_scatterers_create: bad argument");
  if (n_theta < 2 || random_points < 1)
    return set_err(MCRT_EINVAL, "mcrt_mie_scatterers_create: need n_theta >= 2 and random_points >= 1");
  for (int i = 0; i < n; ++i) {
    out[i] = nullptr;
    if (!(r[i] > 0) || !(lambda[i] > 0) || !(nu[i] > 0) || !std::isfinite(m_re[i]) || !std::isfinite(m_im[i]))
      return set_err(MCRT_EINVAL, "mcrt_mie_scatterers_create: need r, lambda, nu > 0 and a finite m");
  }
  CK(cudaSetDevice(ctx->device));
  const size_t nres = mie_result_doubles(n_theta, random_points);
  std::vector<MieJob> jobs(n);
  std::vector<size_t> scratch_off(n);
  size_t scratch = 0;
  for (int i = 0; i < n; ++i) {
    MieJob& J = jobs[i];
    J.x = 2 * host::PI * r[i] / lambda[i];  // mie.jl:37
    J.m_re = m_re[i];
    J.m_im = m_im[i];
    J.r = r[i];
    J.nu = nu[i];
    J.nt = n_theta;
    J.rp = random_points;
    // the series length of bhmie (mie.jl:133-135), computed on the host as there
    J.nstop = (int)std::floor(std::max(J.x + 4 * std::cbrt(J.x) + 2, J.x * std::hypot(m_re[i], m_im[i])));
    J.nmax = J.nstop + 15;
    if (J.nstop < 1 || J.nstop > (1 << 20))
      return set_err(MCRT_EINVAL, "mcrt_mie_scatterers_create: size parameter out of range");
    scratch_off[i] = scratch;
    scratch += 2 * (size_t)(J.nmax + 1) + 4 * (size_t)(J.nstop + 1) + 2 * (size_t)(random_points + 1);
    J.nc = ((random_points + 2 + 3) / 4) * 4;
  }
  DevBuf d_scr, d_res, d_jobs;
  CK(d_scr.alloc(scratch * sizeof(double)));
  CK(d_res.alloc(nres * n * sizeof(double)));
  std::vector<std::unique_ptr<mcrt_scatterer>> made(n);
  for (int i = 0; i < n; ++i) {
    MieJob& J = jobs[i];
    made[i].reset(new mcrt_scatterer());
    mcrt_scatterer& s = *made[i];
    s.ctx = ctx;
    s.kind = MCRT_MIE;
    s.ntheta = n_theta;
    s.rp = random_points;
    CK(s.F.alloc((n_theta + 1) * sizeof(float4)));
    CK(s.S.alloc((n_theta + 1) * sizeof(float4)));
    CK(s.C.alloc(J.nc * sizeof(float)));
    double* base = d_scr.as<double>() + scratch_off[i];
    J.d = base;
    J.ab = base + 2 * (size_t)(J.nmax + 1);
    J.terms = J.ab + 4 * (size_t)(J.nstop + 1);
    J.out = d_res.as<double>() + nres * i;
    J.F = s.F.as<float4>();
    J.S = s.S.as<float4>();
    J.C = s.C.as<float>();
  }
  CK(d_jobs.alloc(n * sizeof(MieJob)));
  cudaStream_t st = ctx->stream;
  Range rr("mcrt mie tables");
  CK(cudaMemcpyAsync(d_jobs.p, jobs.data(), n * sizeof(MieJob), cudaMemcpyHostToDevice, st));
  CK(launch_mie_tables(d_jobs.as<const MieJob>(), n, st));
  std::vector<double> h(nres * n);
  CK(cudaMemcpyAsync(h.data(), d_res.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (int i = 0; i < n; ++i) {
    const double* R = h.data() + nres * i;
    if (!(R[0] >= 0) || !(R[1] > 0) || !std::isfinite(R[1]))
      return set_err(MCRT_ENONCONV, "mcrt_mie_scatterers_create: the Mie series gave no finite omega and kl");
    made[i]->omega = R[0];
    made[i]->kl = R[1];
  }
  if (tables) std::memcpy(tables, h.data(), h.size() * sizeof(double));
  for (int i = 0; i < n; ++i) out[i] = made[i].release();
  return MCRT_OK;
}

}  // extern "C"

// ================================================================== validation
namespace {

constexpr double PI = host::PI;

// Tally doubles of one instance: Irt | Icb | ladder | acc (NACC) | Fourier RT coefficients.
struct TallyLayout {
  size_t nrt, ncb, per_inst;
};
TallyLayout tally_layout(const mcrt_config* c) {
  TallyLayout t;
  t.nrt = 4 * (size_t)c->n_theta * c->n_phi;
  t.ncb = 4 * (size_t)c->n_theta_b * c->n_phi_b;
  t.per_inst = t.nrt + t.ncb + t.ncb / 4 + NACC + 20 * (size_t)c->n_theta;
  return t;
}
void assign_tally(DevInstance& D, double* t, const TallyLayout& L) {
  D.Irt = t;
  D.Icb = t + L.nrt;
  D.ladder = t + L.nrt + L.ncb;
  D.acc = D.ladder + L.ncb / 4;
  D.Frt = D.acc + NACC;
}

int validate_config(const mcrt_config* c, int geom) {
  if (!c) return set_err(MCRT_EINVAL, "config is NULL");
  if (c->number_of_rays < 0) return set_err(MCRT_EINVAL, "number_of_rays must be >= 0");
  if (c->maximum_scattering_times < 0)
    return set_err(MCRT_EINVAL, "maximum_scattering_times must be >= 0");
  if (c->n_phi < 1 || c->n_theta < 1 || c->n_theta_b < 1 || c->n_phi_b < 1)
    return set_err(MCRT_EINVAL, "bin counts must be >= 1");
  if (geom == MCRT_PLANE && (c->n_theta % 2) != 0)
    return set_err(MCRT_EINVAL, "a plane geometry needs an even Ntheta (two half-range quadratures)");
  if (!c->cos_phi || !c->sin_phi || !c->cos_theta || !c->sin_theta || !c->inorm || !c->cos_theta_b ||
      !c->sin_theta_b || !c->cos_phi_b || !c->sin_phi_b)
    return set_err(MCRT_EINVAL, "config array pointer is NULL");
  if (!(c->tau0 >= 0)) return set_err(MCRT_EINVAL, "tau0 must be >= 0");
  return MCRT_OK;
}

// validate(p::PlaneGeometry) (plane.jl:52-62) and validate(s::SphereGeometry)
// (sphere.jl:35-37), with the reference's messages.
int validate_geometry(const mcrt_geometry* g) {
  if (!g) return set_err(MCRT_EINVAL, "geometry is NULL");
  if (g->kind == MCRT_PLANE) {
    if (!(PI / 2 < g->theta && g->theta <= PI)) return set_err(MCRT_EINVAL, "θ must be in (π/2, π]");
    if (!(0 <= g->phi && g->phi < 2 * PI)) return set_err(MCRT_EINVAL, "ϕ must be in [0, 2π)");
    if (g->n_layers < 1 || !g->layers)
      return set_err(MCRT_EINVAL, "There needs to be at least one layer");
    if (g->n_layers > MAX_LAYERS) return set_err(MCRT_EINVAL, "too many layers (at most 8)");
    for (int i = 0; i < g->n_layers; ++i) {
      if (i != g->n_layers - 1 && g->layers[i].infinite)
        return set_err(MCRT_EINVAL, "Only the last layer can be infinite");
      if (!g->layers[i].scatterer) return set_err(MCRT_EINVAL, "layer scatterer is NULL");
      if (!g->layers[i].infinite && !(g->layers[i].tau > 0))
        return set_err(MCRT_EINVAL, "layer optical thickness must be positive");
    }
  } else if (g->kind == MCRT_SPHERE) {
    if (g->n_layers != 1 || !g->layers || !g->layers[0].scatterer)
      return set_err(MCRT_EINVAL, "a sphere has exactly one region with a scatterer");
    if (!(g->layers[0].tau > 0)) return set_err(MCRT_EINVAL, "Radius must be positive");
  } else {
    return set_err(MCRT_EINVAL, "unknown geometry kind");
  }
  return MCRT_OK;
}

// ================================================================== bin tables
struct HostBins {
  std::vector<double> st, ct, g, w, cp, sp;
  std::vector<double> kfx, kfy, kfz, ehx, ehy, gb, cf2, sf2, c1, c2, c3;
  std::vector<int> upb;
  std::vector<double> stb, ctb, cpb, spb;
  int ntheta, nphi, nthetab, nphib, up0, up1, lo0, lo1;
  std::vector<float> rtp;  // BinTables::rtp, 8 floats per pair
  int rtp_lo = 0, rtp_zero = 0;
};

// Per-bin constants of the RT grid (config.jl:78-99) and of the CB grid rotated into
// the backscatter frame kfs (src/gpu.jl:92-94), including the CB bins' final rotation
// into their own meridian planes (src/gpu.jl:127-133).
HostBins make_bins(const mcrt_config* c, int geom, const host::Sph& kfs) {
  HostBins H;
  H.ntheta = c->n_theta;
  H.nphi = c->n_phi;
  H.nthetab = c->n_theta_b;
  H.nphib = c->n_phi_b;
  if (geom == MCRT_PLANE) {  // plane.jl:119,129
    H.up0 = c->n_theta / 2;
    H.up1 = c->n_theta;
    H.lo0 = 0;
    H.lo1 = c->n_theta / 2;
  } else {  // sphere.jl:79,83
    H.up0 = 0;
    H.up1 = c->n_theta;
    H.lo0 = 0;
    H.lo1 = 0;
  }
  for (int j = 0; j < c->n_theta; ++j) {
    H.st.push_back(c->sin_theta[j]);
    H.ct.push_back(c->cos_theta[j]);
    H.g.push_back(LOG2E_D / std::fabs(c->cos_theta[j]));
    H.w.push_back(c->inorm[j]);
  }
  for (int j = 0; j < c->n_phi; ++j) {
    H.cp.push_back(c->cos_phi[j]);
    H.sp.push_back(c->sin_phi[j]);
  }
  {
    auto pairs = [&](int r0, int r1) {
      const int np = (r1 - r0 + 1) / 2, npad = (np + RTP_PAD - 1) / RTP_PAD * RTP_PAD;
      for (int p = 0; p < npad; ++p) {
        const int ja = r0 + 2 * p, jb = ja + 1;
        const bool oka = ja < r1, okb = jb < r1;
        const int ia = oka ? ja : r0, ib = okb ? jb : r0;
        const float v[8] = {(float)H.st[ia], (float)H.st[ib], (float)H.ct[ia], (float)H.ct[ib],
                            (float)H.g[ia],  (float)H.g[ib],  oka ? (float)H.w[ia] : 0.f, okb ? (float)H.w[ib] : 0.f};
        H.rtp.insert(H.rtp.end(), v, v + 8);
      }
    };
    if (H.up1 > H.up0) pairs(H.up0, H.up1);
    H.rtp_lo = (int)(H.rtp.size() / 8);
    if (H.lo1 > H.lo0) pairs(H.lo0, H.lo1);
    H.rtp_zero = (int)(H.rtp.size() / 8);
    // lanes without bins evaluate a real bin at zero weight, so their arithmetic stays finite
    const int i0 = H.up1 > H.up0 ? H.up0 : H.lo0;
    const float z[8] = {(float)H.st[i0], (float)H.st[i0], (float)H.ct[i0], (float)H.ct[i0],
                        (float)H.g[i0],  (float)H.g[i0],  0.f, 0.f};
    for (int p = 0; p < RTP_PAD; ++p) H.rtp.insert(H.rtp.end(), z, z + 8);
  }
  for (int j = 0; j < c->n_theta_b; ++j) {
    H.stb.push_back(c->sin_theta_b[j]);
    H.ctb.push_back(c->cos_theta_b[j]);
  }
  for (int j = 0; j < c->n_phi_b; ++j) {
    H.cpb.push_back(c->cos_phi_b[j]);
    H.spb.push_back(c->sin_phi_b[j]);
  }
  for (int j2 = 0; j2 < c->n_phi_b; ++j2) {
    for (int j1 = 0; j1 < c->n_theta_b; ++j1) {
      const double stb = c->sin_theta_b[j1], ctb = c->cos_theta_b[j1];
      const double cpb = c->cos_phi_b[j2], spb = c->sin_phi_b[j2];
      host::V3 kf = host::ray_to_norm({stb * cpb, stb * spb, ctb}, kfs);
      host::V3 Eh, Ev;
      host::get_basis(kf, Eh, Ev);
      host::V3 eh = host::norm_to_ray(Eh, kfs), ev = host::norm_to_ray(Ev, kfs);
      const double cpsi = spb * eh.x - cpb * eh.y;
      const double spsi = -spb * ev.x + cpb * ev.y;
      H.kfx.push_back(kf.x);
      H.kfy.push_back(kf.y);
      H.kfz.push_back(kf.z);
      H.ehx.push_back(Eh.x);
      H.ehy.push_back(Eh.y);
      H.gb.push_back(LOG2E_D / std::fabs(kf.z));
      H.upb.push_back(kf.z > 0 ? 1 : 0);
      H.cf2.push_back(cpsi * cpsi - spsi * spsi);
      H.sf2.push_back(2.0 * cpsi * spsi);
      H.c1.push_back(stb * cpb);
      H.c2.push_back(stb * spb);
      // cos(theta_b) - 1 without cancellation near the backscatter direction
      H.c3.push_back(ctb > 0 ? -(stb * stb) / (1.0 + ctb) : ctb - 1.0);
    }
  }
  return H;
}

struct Packer {
  std::vector<unsigned char> bytes;
  size_t add(const void* src, size_t n) {
    size_t off = (bytes.size() + 255) & ~size_t(255);
    bytes.resize(off + n);
    std::memcpy(bytes.data() + off, src, n);
    return off;
  }
};

template <typename T>
int upload_bins(const HostBins& H, DevBuf& buf, cudaStream_t st) {
  Packer P;
  BinTables<T> hdr{};
  P.add(&hdr, sizeof(hdr));
  auto addv = [&](const std::vector<double>& v) {
    std::vector<T> t(v.begin(), v.end());
    if (t.empty()) t.push_back(T(0));
    return P.add(t.data(), t.size() * sizeof(T));
  };
  size_t o_st = addv(H.st), o_ct = addv(H.ct), o_g = addv(H.g), o_w = addv(H.w), o_cp = addv(H.cp),
         o_sp = addv(H.sp);
  size_t o_kfx = addv(H.kfx), o_kfy = addv(H.kfy), o_kfz = addv(H.kfz), o_ehx = addv(H.ehx),
         o_ehy = addv(H.ehy), o_gb = addv(H.gb), o_cf2 = addv(H.cf2), o_sf2 = addv(H.sf2),
         o_c1 = addv(H.c1), o_c2 = addv(H.c2), o_c3 = addv(H.c3);
  size_t o_upb = P.add(H.upb.data(), H.upb.size() * sizeof(int));
  size_t o_stb = addv(H.stb), o_ctb = addv(H.ctb), o_cpb = addv(H.cpb), o_spb = addv(H.spb);
  size_t o_rtp = P.add(H.rtp.data(), H.rtp.size() * sizeof(float));
  CK(buf.alloc(P.bytes.size()));
  unsigned char* base = buf.as<unsigned char>();
  hdr.ntheta = H.ntheta;
  hdr.nphi = H.nphi;
  hdr.nthetab = H.nthetab;
  hdr.nphib = H.nphib;
  hdr.up0 = H.up0;
  hdr.up1 = H.up1;
  hdr.lo0 = H.lo0;
  hdr.lo1 = H.lo1;
  auto at = [&](size_t o) { return reinterpret_cast<const T*>(base + o); };
  hdr.st = at(o_st);
  hdr.ct = at(o_ct);
  hdr.g = at(o_g);
  hdr.w = at(o_w);
  hdr.cp = at(o_cp);
  hdr.sp = at(o_sp);
  hdr.kfx = at(o_kfx);
  hdr.kfy = at(o_kfy);
  hdr.kfz = at(o_kfz);
  hdr.ehx = at(o_ehx);
  hdr.ehy = at(o_ehy);
  hdr.gb = at(o_gb);
  hdr.cf2 = at(o_cf2);
  hdr.sf2 = at(o_sf2);
  hdr.c1 = at(o_c1);
  hdr.c2 = at(o_c2);
  hdr.c3 = at(o_c3);
  hdr.upb = reinterpret_cast<const int*>(base + o_upb);
  hdr.stb = at(o_stb);
  hdr.ctb = at(o_ctb);
  hdr.cpb = at(o_cpb);
  hdr.spb = at(o_spb);
  hdr.rtp = reinterpret_cast<const float4*>(base + o_rtp);
  hdr.rtp_lo = H.rtp_lo;
  hdr.rtp_zero = H.rtp_zero;
  std::memcpy(P.bytes.data(), &hdr, sizeof(hdr));
  CK(upload_sync(buf.p, P.bytes.data(), P.bytes.size(), st));
  return MCRT_OK;
}

// Host copy of one instance: geometry, incidence frame, CB constants, RNG key.
int make_instance(const mcrt_config* c, const mcrt_geometry* g, const double I0[4], uint64_t seed,
                  uint32_t instance, int rng_mode, long long n_photons, long long photon_begin,
                  DevInstance& D, host::Sph& kfs_out) {
  std::memset(&D, 0, sizeof(D));
  D.max_attempts = 1LL << 20;
  D.geom = g->kind;
  D.n_layers = g->n_layers;
  std::vector<const mcrt_scatterer*> sc;
  for (int i = 0; i < g->n_layers; ++i) {
    const mcrt_scatterer* s = g->layers[i].scatterer;
    int k = -1;
    for (size_t j = 0; j < sc.size(); ++j)
      if (sc[j] == s) k = (int)j;
    if (k < 0) {
      if ((int)sc.size() >= MAX_SCAT) return set_err(MCRT_EINVAL, "at most 4 distinct scatterers");
      sc.push_back(s);
      k = (int)sc.size() - 1;
    }
    D.layers[i].tau = g->layers[i].tau;
    D.layers[i].omega = g->layers[i].omega;
    D.layers[i].inf = g->kind == MCRT_PLANE && g->layers[i].infinite ? 1 : 0;
    D.layers[i].scat = k;
  }
  D.n_scat = (int)sc.size();
  for (size_t j = 0; j < sc.size(); ++j) D.scat[j] = sc[j]->view();
  double th0 = g->kind == MCRT_PLANE ? g->theta : PI, ph0 = g->kind == MCRT_PLANE ? g->phi : 0.0;
  host::Sph inc{std::cos(th0), std::sin(th0), std::cos(ph0), std::sin(ph0)};
  host::V3 k0 = host::ray_to_norm({0, 0, 1}, inc);  // MonteCarloRadiativeTransfer.jl:32
  D.k0[0] = k0.x;
  D.k0[1] = k0.y;
  D.k0[2] = k0.z;
  D.inc[0] = inc.ct;
  D.inc[1] = inc.st;
  D.inc[2] = inc.cp;
  D.inc[3] = inc.sp;
  for (int s = 0; s < 4; ++s) D.I0[s] = I0[s];
  host::E_from_I(I0, D.Ei);
  host::V3 kf{-k0.x, -k0.y, -k0.z};  // kf = -kpath[1] (src/gpu.jl:48)
  host::Sph kfs = host::spherical(kf);
  kfs_out = kfs;
  D.kfs[0] = kfs.ct;
  D.kfs[1] = kfs.st;
  D.kfs[2] = kfs.cp;
  D.kfs[3] = kfs.sp;
  D.kf0[0] = kf.x;
  D.kf0[1] = kf.y;
  D.kf0[2] = kf.z;
  host::V3 Eh, Ev;
  host::get_basis(kf, Eh, Ev);
  D.eh0[0] = Eh.x;
  D.eh0[1] = Eh.y;
  // rows of norm_to_ray for the frame kfs
  D.Rkfs[0] = kfs.ct * kfs.cp;
  D.Rkfs[1] = kfs.ct * kfs.sp;
  D.Rkfs[2] = -kfs.st;
  D.Rkfs[3] = -kfs.sp;
  D.Rkfs[4] = kfs.cp;
  D.Rkfs[5] = 0.0;
  D.Rkfs[6] = kfs.st * kfs.cp;
  D.Rkfs[7] = kfs.st * kfs.sp;
  D.Rkfs[8] = kfs.ct;
  D.kl1 = g->layers[0].scatterer->kl;  // mean_free_path(g, 1) (src/gpu.jl:102)
  D.min_int = c->minimum_intensity;
  D.tau0 = c->tau0;
  D.max_scat = c->maximum_scattering_times;
  D.compute_cb = c->compute_cb ? 1 : 0;
  D.n_photons = n_photons;
  D.photon_begin = photon_begin;
  D.nrays = c->number_of_rays > 0 ? c->number_of_rays : 1;
  D.key0 = (unsigned)seed;
  D.key1 = (unsigned)(seed >> 32) + 0x632BE5ABu * instance;
  D.rng_mode = rng_mode;
  // Rayleigh peel-off in a slab: the bin's Stokes vector is a degree-2 trigonometric
  // polynomial in its azimuth and its attenuation depends on the polar angle only.
  bool all_rayleigh = true;
  for (int s = 0; s < D.n_scat; ++s) all_rayleigh = all_rayleigh && D.scat[s].kind == 0;
  D.rt_fourier = (g->kind == MCRT_PLANE && all_rayleigh && c->n_phi >= 5) ? 1 : 0;
  return MCRT_OK;
}

// ================================================================== kernel dispatch
bool kernel_info(int prec, int bs, KInfo& k) {
  return prec == MCRT_FP32 ? kernel_info_fp32(bs, k) : kernel_info_fp64(bs, k);
}

int table_f4_of(const DevInstance& D) {
  int f4 = 0;
  for (int s = 0; s < D.n_scat; ++s)
    if (D.scat[s].kind == 1) f4 += 2 * (D.scat[s].ntheta + 1) + (D.scat[s].rp + 2 + 3) / 4;
  return f4;
}

}  // namespace

// ================================================================== launches
using ctx_t = mcrt_ctx;

struct Launch {
  int precision = MCRT_FP32, kernel = MCRT_KERNEL_PERSISTENT;
  int bs = 256, bpsm = 0, blocks = 0;
  size_t smem = 0;
  int table_f4 = 0;
};

// Everything a group of instances needs on the device: descriptors, bin tables,
// tallies, counters and the photon-state pool.
struct Group {
  mcrt_ctx* ctx = nullptr;
  Launch L;
  int n_inst = 0;
  std::vector<DevInstance> hinst;   // host copies (device pointers filled in)
  std::vector<int> order;           // device slot -> user index
  std::vector<std::unique_ptr<DevBuf>> bins;
  DevBuf d_inst, d_tally, d_claim, d_status, d_state, d_tacc;
  DevBuf d_kpath, d_xpath, d_idx;  // plain kernel path history
  long long plain_threads = 0;
  size_t nrt = 0, ncb = 0, per_inst = 0;  // tally doubles per instance
  float last_ms = 0.f;
  double photons = 0;
};

namespace {

int size_launch(mcrt_ctx* ctx, Group& G, const mcrt_run_opts* o, const std::string& sig) {
  Launch& L = G.L;
  L.precision = o ? o->precision : MCRT_FP32;
  L.kernel = o ? o->kernel : MCRT_KERNEL_PERSISTENT;
  if (L.precision != MCRT_FP32 && L.precision != MCRT_FP64)
    return set_err(MCRT_EINVAL, "precision must be MCRT_FP32 or MCRT_FP64");
  if (L.kernel != MCRT_KERNEL_PERSISTENT && L.kernel != MCRT_KERNEL_PLAIN)
    return set_err(MCRT_EINVAL, "unknown kernel kind");
  if (L.kernel == MCRT_KERNEL_PLAIN) return MCRT_OK;
  int bs = o && o->block_size ? o->block_size : 0;
  int bpsm = o && o->blocks_per_sm ? o->blocks_per_sm : 0;
  int staging = o ? o->table_staging : 0;
  if (staging < 0 || staging > 2) return set_err(MCRT_EINVAL, "table_staging must be 0, 1 or 2");
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->tuned.find(sig);
    if (it != ctx->tuned.end()) {
      if (!bs) {
        bs = it->second.bs;
        if (!bpsm) bpsm = it->second.bpsm;
      }
      if (!staging) staging = it->second.staging;
    }
  }
  if (!bs) bs = L.precision == MCRT_FP32 ? 256 : 128;
  KInfo ki;
  if (!kernel_info(L.precision, bs, ki))
    return set_err(MCRT_EINVAL, "unsupported block size for this precision (FP32: 128/256/512/768, FP64: 128/256)");
  int tf4 = 0;
  if (staging != 2)  // 2: Mie tables stay in global memory and are read through L1
    for (auto& D : G.hinst) tf4 = std::max(tf4, table_f4_of(D));
  size_t smem = ki.shared_static + (size_t)tf4 * 16;
  if (smem > (size_t)ctx->smem_optin) {
    // the tables that do not fit are read from global memory through L1
    tf4 = (int)((ctx->smem_optin - ki.shared_static) / 16);
    if (tf4 < 0) return set_err(MCRT_EINVAL, "block size too large for shared memory");
    smem = ki.shared_static + (size_t)tf4 * 16;
  }
  CK(cudaFuncSetAttribute(ki.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ki.fn, bs, smem));
  if (occ < 1) return set_err(MCRT_EINVAL, "kernel does not fit on an SM with this block size");
  if (!bpsm || bpsm > occ) bpsm = occ;
  L.bs = bs;
  L.bpsm = bpsm;
  L.blocks = ctx->sms * bpsm;
  L.smem = smem;
  L.table_f4 = tf4;
  return MCRT_OK;
}

int autotune(mcrt_ctx* ctx, const mcrt_config* c, const mcrt_geometry* g, const double* I0, uint64_t seed,
             uint32_t inst, long long nph, long long photon_begin, int rng_mode, const mcrt_run_opts* o,
             const std::string& sig);

// Allocates tallies, counters, bins and state for the group's instances.
int build_group(mcrt_ctx* ctx, const mcrt_config* c, const mcrt_geometry* const* geoms,
                const double (*I0)[4], const uint64_t* seeds, const uint32_t* insts,
                const long long* nph, long long photon_begin, int rng_mode, int n,
                const mcrt_run_opts* o, Group& G) {
  Range r("mcrt build group");
  G.ctx = ctx;
  G.n_inst = n;
  G.hinst.resize(n);
  std::vector<host::Sph> kfs(n);
  for (int i = 0; i < n; ++i) {
    int rc = make_instance(c, geoms[i], I0[i], seeds[i], insts[i], rng_mode, nph[i], photon_begin,
                           G.hinst[i], kfs[i]);
    if (rc) return rc;
    if (o && o->max_attempts > 0) G.hinst[i].max_attempts = o->max_attempts;
  }
  // order instances by photon budget, largest first (blocks walk the list in order)
  G.order.resize(n);
  for (int i = 0; i < n; ++i) G.order[i] = i;
  std::stable_sort(G.order.begin(), G.order.end(),
                   [&](int a, int b) { return G.hinst[a].n_photons > G.hinst[b].n_photons; });
  const DevInstance& D0 = G.hinst[G.order[0]];
  std::string sig = std::to_string(D0.geom) + "/" + std::to_string(c->n_theta) + "x" +
                    std::to_string(c->n_phi) + "/" + std::to_string(c->n_theta_b) + "x" +
                    std::to_string(c->n_phi_b) + "/" + std::to_string(D0.scat[0].kind) + ":" +
                    std::to_string(D0.scat[0].ntheta) + "/" + std::to_string(o ? o->precision : 0);
  const bool persistent = !o || o->kernel == MCRT_KERNEL_PERSISTENT;
  if (persistent && (!o || !o->block_size || !o->table_staging)) {
    bool have;
    {
      std::lock_guard<std::mutex> lk(ctx->mu);
      have = ctx->tuned.count(sig) > 0;
    }
    if (!have) {
      const int big = G.order[0];
      int rc = autotune(ctx, c, geoms[big], I0[big], seeds[big], insts[big], nph[big], photon_begin,
                        rng_mode, o, sig);
      if (rc) return rc;
    }
  }
  int rc = size_launch(ctx, G, o, sig);
  if (rc) return rc;
  // bin tables, one per distinct (geometry kind, incidence)
  std::map<std::string, const void*> bin_cache;
  for (int i = 0; i < n; ++i) {
    char key[128];
    std::snprintf(key, sizeof key, "%d/%.17g/%.17g/%.17g/%.17g", geoms[i]->kind, kfs[i].ct, kfs[i].st,
                  kfs[i].cp, kfs[i].sp);
    auto it = bin_cache.find(key);
    if (it == bin_cache.end()) {
      HostBins H = make_bins(c, geoms[i]->kind, kfs[i]);
      std::unique_ptr<DevBuf> b(new DevBuf());
      rc = G.L.precision == MCRT_FP32 ? upload_bins<float>(H, *b, ctx->stream)
                                      : upload_bins<double>(H, *b, ctx->stream);
      if (rc) return rc;
      bin_cache[key] = b->p;
      G.bins.push_back(std::move(b));
      it = bin_cache.find(key);
    }
    G.hinst[i].bins = it->second;
  }
  const TallyLayout TL = tally_layout(c);
  G.nrt = TL.nrt;
  G.ncb = TL.ncb;
  G.per_inst = TL.per_inst;
  CK(G.d_tally.alloc(G.per_inst * n * sizeof(double)));
  CK(G.d_claim.alloc(2 * n * sizeof(unsigned long long)));
  CK(G.d_status.alloc(sizeof(unsigned)));
  for (int i = 0; i < n; ++i) {
    assign_tally(G.hinst[i], G.d_tally.as<double>() + G.per_inst * i, TL);
    G.hinst[i].claim = G.d_claim.as<unsigned long long>() + 2 * i;
  }
  std::vector<DevInstance> dev(n);
  for (int s = 0; s < n; ++s) dev[s] = G.hinst[G.order[s]];
  CK(G.d_inst.alloc(n * sizeof(DevInstance)));
  CK(upload_sync(G.d_inst.p, dev.data(), n * sizeof(DevInstance), ctx->stream));
  if (G.L.kernel == MCRT_KERNEL_PERSISTENT) {
    KInfo ki;
    kernel_info(G.L.precision, G.L.bs, ki);
    size_t slots = (size_t)G.L.blocks * G.L.bs;
    CK(G.d_state.alloc(slots * ki.state_bytes));
    CK(G.d_tacc.alloc(slots * NACC * sizeof(double)));
  } else {
    if (n != 1) return set_err(MCRT_EINVAL, "the plain kernel runs one instance per launch");
    long long th = o && o->plain_threads > 0 ? o->plain_threads
                                             : std::min<long long>(c->maximum_threads > 0 ? c->maximum_threads : 8192,
                                                                   std::max<long long>(nph[0], 1));
    G.plain_threads = th;
    size_t rows = (size_t)c->maximum_scattering_times + 1;
    size_t vb = G.L.precision == MCRT_FP32 ? 3 * sizeof(float) : 3 * sizeof(double);
    CK(G.d_kpath.alloc(rows * th * vb));
    CK(G.d_xpath.alloc(rows * th * vb));
    CK(G.d_idx.alloc(rows * th * sizeof(int)));
  }
  return MCRT_OK;
}

int launch_group(Group& G) {
  Range r("mcrt launch");
  mcrt_ctx* ctx = G.ctx;
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  CK(cudaMemsetAsync(G.d_tally.p, 0, G.d_tally.n, st));
  CK(cudaMemsetAsync(G.d_claim.p, 0, G.d_claim.n, st));
  CK(cudaMemsetAsync(G.d_status.p, 0, G.d_status.n, st));
  G.photons = 0;
  for (auto& D : G.hinst) G.photons += (double)D.n_photons;
  CK(cudaEventRecord(ctx->e0, st));
  if (G.L.kernel == MCRT_KERNEL_PERSISTENT) {
    KInfo ki;
    kernel_info(G.L.precision, G.L.bs, ki);
    KParams p;
    p.inst = G.d_inst.as<const DevInstance>();
    p.n_inst = G.n_inst;
    p.state = G.d_state.as<uint4>();
    p.tacc = G.d_tacc.as<double>();
    p.status = G.d_status.as<unsigned>();
    p.table_f4 = G.L.table_f4;
    CK(launch_transport(ki, G.L.blocks, G.L.bs, G.L.smem, st, p));
  } else {
    PlainParams p;
    p.inst = G.d_inst.as<const DevInstance>();
    p.kpath = G.d_kpath.as<double>();
    p.xpath = G.d_xpath.as<double>();
    p.idxpath = G.d_idx.as<int>();
    p.threads = G.plain_threads;
    p.maxord = (long long)(G.d_idx.n / sizeof(int) / std::max<long long>(G.plain_threads, 1));
    p.status = G.d_status.as<unsigned>();
    int blocks = (int)((G.plain_threads + 255) / 256);
    CK(launch_plain(G.L.precision == MCRT_FP64, blocks, st, p));
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(ctx->e1, st));
  return MCRT_OK;
}

int finish_group(Group& G) {
  CK(cudaEventSynchronize(G.ctx->e1));
  CK(cudaEventElapsedTime(&G.last_ms, G.ctx->e0, G.ctx->e1));
  return MCRT_OK;
}

int read_instance(Group& G, int user_index, double A_out[5], double* Irt, double* Icb, double* lad,
                  mcrt_stats* stats) {
  Range r("mcrt read tallies");
  CK(cudaStreamSynchronize(G.ctx->stream));
  std::vector<double> h(G.per_inst);
  const double* src = G.hinst[user_index].Irt;
  CK(cudaMemcpy(h.data(), src, G.per_inst * sizeof(double), cudaMemcpyDeviceToHost));
  unsigned status = 0;
  CK(cudaMemcpy(&status, G.d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
  const double* acc = h.data() + G.nrt + G.ncb + G.ncb / 4;
  if (A_out)
    for (int s = 0; s < 5; ++s) A_out[s] = acc[s];
  if (Irt) std::memcpy(Irt, h.data(), G.nrt * sizeof(double));
  if (Icb) std::memcpy(Icb, h.data() + G.nrt, G.ncb * sizeof(double));
  if (lad) std::memcpy(lad, h.data() + G.nrt + G.ncb, G.ncb / 4 * sizeof(double));
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->cb_peak_sum = acc[ACC_PEAK];
    stats->cb_peak_sumsq = acc[ACC_PEAK2];
    stats->photons = acc[ACC_PHOTONS];
    stats->events = acc[ACC_EVENTS];
    stats->attempts = acc[ACC_ATTEMPTS];
    stats->rt_evals = acc[ACC_RT];
    stats->cb1_evals = acc[ACC_CB1];
    stats->cbn_evals = acc[ACC_CBN];
    stats->kernel_ms = G.last_ms;
    stats->status_flags = (int)status;
    stats->block_size = G.L.kernel == MCRT_KERNEL_PERSISTENT ? G.L.bs : 256;
    stats->blocks = G.L.kernel == MCRT_KERNEL_PERSISTENT ? G.L.blocks : (int)((G.plain_threads + 255) / 256);
  }
  return MCRT_OK;
}

// The autotuner: times the candidate launch shapes (threads per block, blocks per SM)
// and, for Mie scatterers, the table staging (shared memory or global memory through
// L1) on the same sample of the workload's own photons, and keeps the fastest for this
// workload signature in the context. User-given fields are kept fixed.
int autotune(mcrt_ctx* ctx, const mcrt_config* c, const mcrt_geometry* g, const double* I0, uint64_t seed,
             uint32_t inst, long long nph, long long photon_begin, int rng_mode, const mcrt_run_opts* o,
             const std::string& sig) {
  Range r("mcrt autotune");
  const int prec = o ? o->precision : MCRT_FP32;
  std::vector<std::pair<int, int>> shapes;
  if (prec == MCRT_FP32)
    shapes = {{256, 2}, {256, 1}, {512, 1}, {768, 1}};
  else
    shapes = {{128, 2}, {128, 1}, {256, 1}};
  if (o && o->block_size) {
    shapes.clear();
    shapes.push_back({o->block_size, o->blocks_per_sm});
  }
  bool mie = false;
  for (int l = 0; l < g->n_layers; ++l) mie = mie || g->layers[l].scatterer->kind == MCRT_MIE;
  std::vector<int> stagings = mie ? std::vector<int>{1, 2} : std::vector<int>{1};
  if (o && o->table_staging) stagings = {o->table_staging};
  const double I[1][4] = {{I0[0], I0[1], I0[2], I0[3]}};
  ctx_t::Tuned best{0, 0, 0, -1.0};
  std::vector<std::string> seen;
  bool warmed = false;
  // Every candidate runs the same photons, so the rates compare steady-state throughput
  // rather than the end-of-launch tail: up to 4 per thread of the largest shape, fewer
  // when a probe launch (which also warms up the device) counts more than 2e11 bin
  // evaluations for them (about a second). The count, unlike a time, does not change
  // under a profiler.
  long long ns = std::max<long long>(1, std::min<long long>(nph, 4LL * ctx->sms * 768));
  {
    mcrt_run_opts oo{};
    if (o) oo = *o;
    oo.kernel = MCRT_KERNEL_PERSISTENT;
    oo.block_size = shapes[0].first;
    oo.blocks_per_sm = shapes[0].second;
    oo.table_staging = stagings[0];
    Group T;
    const mcrt_geometry* gs[1] = {g};
    long long n1 = std::min<long long>(ns, (long long)ctx->sms * 256);
    if (!build_group(ctx, c, gs, I, &seed, &inst, &n1, photon_begin, rng_mode, 1, &oo, T)) {
      if (launch_group(T) || finish_group(T)) return MCRT_ECUDA;
      warmed = true;
      mcrt_stats st;
      double Ap[5];
      if (read_instance(T, 0, Ap, nullptr, nullptr, nullptr, &st)) return MCRT_ECUDA;
      const double per_photon = (st.rt_evals + st.cb1_evals + st.cbn_evals) / std::max<double>(n1, 1.0);
      if (per_photon > 0)
        ns = std::max<long long>(n1, std::min<long long>(ns, (long long)(2e11 / per_photon)));
    }
  }
  auto trial = [&](std::pair<int, int> sh, int st) -> int {
    mcrt_run_opts oo{};
    if (o) oo = *o;
    oo.kernel = MCRT_KERNEL_PERSISTENT;
    oo.block_size = sh.first;
    oo.blocks_per_sm = sh.second;
    oo.table_staging = st;
    Group T;
    const mcrt_geometry* gs[1] = {g};
    long long n1 = ns;
    if (build_group(ctx, c, gs, I, &seed, &inst, &n1, photon_begin, rng_mode, 1, &oo, T)) return MCRT_OK;
    std::string key = std::to_string(T.L.bs) + "x" + std::to_string(T.L.bpsm) + "/" + std::to_string(T.L.table_f4);
    if (std::find(seen.begin(), seen.end(), key) != seen.end()) return MCRT_OK;  // occupancy folded it
    seen.push_back(key);
    for (int rep = warmed ? 1 : 0; rep < 2; ++rep) {  // the first launch also warms up the device
      if (launch_group(T) || finish_group(T)) return MCRT_ECUDA;
    }
    warmed = true;
    const double rate = ns / std::max(T.last_ms, 1e-3f);
    if (rate > best.paths_per_ms) best = ctx_t::Tuned{T.L.bs, T.L.bpsm, st, rate};
    return MCRT_OK;
  };
  // launch shapes with the first staging choice, then the other stagings on the best shape
  for (auto sh : shapes)
    if (trial(sh, stagings[0])) return MCRT_ECUDA;
  const std::pair<int, int> best_shape{best.bs, best.bpsm};
  for (size_t k = 1; k < stagings.size(); ++k)
    if (best.bs && trial(best_shape, stagings[k])) return MCRT_ECUDA;
  if (best.bs == 0) return set_err(MCRT_EINVAL, "autotune: no launch shape fits this workload");
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->tuned[sig] = best;
  return MCRT_OK;
}

}  // namespace

// ================================================================== public entry points
struct mcrt_solve {
  Group G;
};
struct mcrt_batch {
  Group G;
};

extern "C" {

int mcrt_solve_create(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_geometry* g,
                      const double I0[4], const mcrt_run_opts* opts, mcrt_solve** out) {
  if (!ctx || !out || !I0) return set_err(MCRT_EINVAL, "mcrt_solve_create: NULL argument");
  *out = nullptr;
  int rc = validate_geometry(g);
  if (rc) return rc;
  rc = validate_config(cfg, g->kind);
  if (rc) return rc;
  CK(cudaSetDevice(ctx->device));
  std::unique_ptr<mcrt_solve> s(new mcrt_solve());
  const mcrt_geometry* gs[1] = {g};
  double I[1][4] = {{I0[0], I0[1], I0[2], I0[3]}};
  uint64_t seed = opts ? opts->seed : 0;
  uint32_t inst = opts ? opts->instance : 0;
  long long nph = cfg->number_of_rays;
  rc = build_group(ctx, cfg, gs, I, &seed, &inst, &nph, opts ? opts->photon_begin : 0,
                   opts ? opts->rng_mode : 0, 1, opts, s->G);
  if (rc) return rc;
  *out = s.release();
  return MCRT_OK;
}

int mcrt_solve_launch(mcrt_solve* s, int64_t photon_begin, int64_t n_photons) {
  if (!s || n_photons < 0) return set_err(MCRT_EINVAL, "mcrt_solve_launch: bad argument");
  DevInstance& D = s->G.hinst[0];
  if (D.n_photons != n_photons || D.photon_begin != photon_begin) {
    D.n_photons = n_photons;
    D.photon_begin = photon_begin;
    CK(cudaMemcpyAsync(s->G.d_inst.p, &D, sizeof(DevInstance), cudaMemcpyHostToDevice, s->G.ctx->stream));
    CK(cudaStreamSynchronize(s->G.ctx->stream));
  }
  return launch_group(s->G);
}

int mcrt_solve_read(mcrt_solve* s, double A_out[5], double* Irt, double* Icb, double* Icb_ladder,
                    mcrt_stats* stats) {
  if (!s) return set_err(MCRT_EINVAL, "mcrt_solve_read: NULL solve");
  int rc = finish_group(s->G);
  if (rc) return rc;
  return read_instance(s->G, 0, A_out, Irt, Icb, Icb_ladder, stats);
}

int mcrt_solve_destroy(mcrt_solve* s) {
  if (!s) return MCRT_OK;
  cudaSetDevice(s->G.ctx->device);
  cudaStreamSynchronize(s->G.ctx->stream);
  delete s;
  return MCRT_OK;
}

int mcrt_simulate(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_geometry* g, const double I0[4],
                  const mcrt_run_opts* opts, double A_out[5], double* Irt, double* Icb,
                  double* Icb_ladder, mcrt_stats* stats) {
  if (!A_out || !Irt || !Icb) return set_err(MCRT_EINVAL, "mcrt_simulate: output pointer is NULL");
  mcrt_solve* s = nullptr;
  int rc = mcrt_solve_create(ctx, cfg, g, I0, opts, &s);
  if (rc) return rc;
  std::unique_ptr<mcrt_solve, int (*)(mcrt_solve*)> guard(s, mcrt_solve_destroy);
  rc = mcrt_solve_launch(s, opts ? opts->photon_begin : 0, cfg->number_of_rays);
  if (rc) return rc;
  rc = mcrt_solve_read(s, A_out, Irt, Icb, Icb_ladder, stats);
  if (rc) return rc;
  // divide by the number of rays (MonteCarloRadiativeTransfer.jl:78-84)
  const double inv = cfg->number_of_rays > 0 ? 1.0 / (double)cfg->number_of_rays : 0.0;
  for (int i = 0; i < 5; ++i) A_out[i] *= inv;
  for (size_t i = 0; i < s->G.nrt; ++i) Irt[i] *= inv;
  for (size_t i = 0; i < s->G.ncb; ++i) Icb[i] *= inv;
  if (Icb_ladder)
    for (size_t i = 0; i < s->G.ncb / 4; ++i) Icb_ladder[i] *= inv;
  if (stats && (stats->status_flags & MCRT_FLAG_REJECT_LIMIT))
    return set_err(MCRT_ENONCONV, "a rejection loop hit its iteration cap; see stats.status_flags");
  return MCRT_OK;
}

int mcrt_batch_create(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_instance* inst, int n_inst,
                      const mcrt_run_opts* opts, mcrt_batch** out) {
  if (!ctx || !inst || !out || n_inst < 1) return set_err(MCRT_EINVAL, "mcrt_batch_create: bad argument");
  *out = nullptr;
  if (opts && opts->kernel == MCRT_KERNEL_PLAIN)
    return set_err(MCRT_EINVAL, "batches run on the persistent kernel");
  std::vector<const mcrt_geometry*> gs(n_inst);
  std::vector<double> I(4 * (size_t)n_inst);
  std::vector<uint64_t> seeds(n_inst);
  std::vector<uint32_t> ids(n_inst);
  std::vector<long long> nph(n_inst);
  for (int i = 0; i < n_inst; ++i) {
    int rc = validate_geometry(inst[i].geometry);
    if (rc) return rc;
    rc = validate_config(cfg, inst[i].geometry->kind);
    if (rc) return rc;
    if (inst[i].n_photons < 0) return set_err(MCRT_EINVAL, "n_photons must be >= 0");
    gs[i] = inst[i].geometry;
    for (int s = 0; s < 4; ++s) I[4 * i + s] = inst[i].I0[s];
    seeds[i] = inst[i].seed;
    ids[i] = inst[i].instance;
    nph[i] = inst[i].n_photons;
  }
  CK(cudaSetDevice(ctx->device));
  std::unique_ptr<mcrt_batch> b(new mcrt_batch());
  int rc = build_group(ctx, cfg, gs.data(), reinterpret_cast<const double(*)[4]>(I.data()), seeds.data(),
                       ids.data(), nph.data(), 0, opts ? opts->rng_mode : 0, n_inst, opts, b->G);
  if (rc) return rc;
  *out = b.release();
  return MCRT_OK;
}

int mcrt_batch_launch(mcrt_batch* b) {
  if (!b) return set_err(MCRT_EINVAL, "mcrt_batch_launch: NULL batch");
  return launch_group(b->G);
}

int mcrt_batch_read(mcrt_batch* b, int i, double A_out[5], double* Irt, double* Icb, double* lad,
                    mcrt_stats* stats) {
  if (!b || i < 0 || i >= b->G.n_inst) return set_err(MCRT_EINVAL, "mcrt_batch_read: bad index");
  int rc = finish_group(b->G);
  if (rc) return rc;
  return read_instance(b->G, i, A_out, Irt, Icb, lad, stats);
}

int mcrt_batch_timing(mcrt_batch* b, double* kernel_ms, double* photons) {
  if (!b) return set_err(MCRT_EINVAL, "mcrt_batch_timing: NULL batch");
  int rc = finish_group(b->G);
  if (rc) return rc;
  if (kernel_ms) *kernel_ms = b->G.last_ms;
  if (photons) *photons = b->G.photons;
  return MCRT_OK;
}

int mcrt_batch_destroy(mcrt_batch* b) {
  if (!b) return MCRT_OK;
  cudaSetDevice(b->G.ctx->device);
  cudaStreamSynchronize(b->G.ctx->stream);
  delete b;
  return MCRT_OK;
}

}  // extern "C"

// ================================================================== run_rt
namespace {

// Inputs of the Mueller assembly epilogue. The tallies of state i start at
// tally + i * per_inst (Irt | Icb | ladder | acc, raw sums).
struct RunRtArgs {
  int kind;
  int n_states;
  int nt, np, ntb, npb;
  size_t per_inst, nrt, ncb;
  const double* tally;
  double inv_n;            // 1 / number_of_rays
  const double* norm_rt;   // per theta: plane |1/(4 cos inorm)|, sphere 1/inorm
  const double* norm_cb;   // per theta_b: plane 1/|4 cos|, sphere 1
  double* out_rt;          // plane [16][np][nt], sphere [16][nt]
  double* out_cb;          // plane [16][npb][ntb], sphere [16][ntb]
  double coef[6][4];       // plane: weight of state i's tally in Mueller column b
  int vstate[2];           // sphere: state i has V != 0
  int nfi[8], nfib[8];     // sphere: the 8 azimuth indices i * Nphi / 8
};

// Plane assembly of MonteCarloRadiativeTransfer.jl:186-291: one thread per RT or CB bin.
__global__ void k_run_rt_plane(RunRtArgs a) {
  const int nrt = a.nt * a.np, ncb = a.ntb * a.npb;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrt + ncb) return;
  const bool rt = t < nrt;
  const int b = rt ? t : t - nrt;  // bin index j2 * ntheta + j1
  const size_t off = rt ? 0 : a.nrt;
  const double nrm = (rt ? a.norm_rt[b % a.nt] : a.norm_cb[b % a.ntb]) * a.inv_n;
  double m[4][4] = {};
  for (int i = 0; i < a.n_states; ++i) {
    const double* x = a.tally + (size_t)i * a.per_inst + off + 4 * (size_t)b;
    for (int s = 0; s < 4; ++s)
      for (int c = 0; c < 4; ++c) m[s][c] += a.coef[i][c] * x[s];
  }
  double* out = rt ? a.out_rt : a.out_cb;
  const int nb = rt ? nrt : ncb;
  for (int s = 0; s < 4; ++s)
    for (int c = 0; c < 4; ++c) out[(size_t)(4 * s + c) * nb + b] = m[s][c] * nrm;
}

// Sphere assembly of MonteCarloRadiativeTransfer.jl:87-184: one thread per RT or CB
// polar bin, summing over azimuths; renormalised by the scattered energy.
__global__ void k_run_rt_sphere(RunRtArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.nt + a.ntb) return;
  const bool rt = t < a.nt;
  const int j1 = rt ? t : t - a.nt;
  const int nt = rt ? a.nt : a.ntb, np = rt ? a.np : a.npb;
  const int* N = rt ? a.nfi : a.nfib;
  const size_t off = rt ? 0 : a.nrt;
  double gsca = 0.0;
  for (int i = 0; i < a.n_states; ++i)
    if (!a.vstate[i]) {
      const double* acc = a.tally + (size_t)i * a.per_inst + a.nrt + a.ncb + a.ncb / 4;
      gsca += (acc[ACC_ADT] + acc[ACC_AREF]) * a.inv_n;
    }
  double m[4][4] = {};
  for (int i = 0; i < a.n_states; ++i) {
    const double* x = a.tally + (size_t)i * a.per_inst + off;
    auto X = [&](int s, int p) { return x[4 * ((size_t)p * nt + j1) + s] * a.inv_n; };
    if (!a.vstate[i]) {
      for (int s = 0; s < 4; ++s) {
        m[s][0] += (X(s, N[0]) + X(s, N[2]) + X(s, N[4]) + X(s, N[6])) * 0.25;
        m[s][1] += (-X(s, N[0]) + X(s, N[2]) - X(s, N[4]) + X(s, N[6])) * 0.25;
        m[s][2] += (X(s, N[1]) - X(s, N[3]) + X(s, N[5]) - X(s, N[7])) * 0.25;
      }
    } else {
      m[2][3] -= (X(2, N[0]) + X(2, N[4])) * 0.5;
      double s3 = 0.0;
      for (int p = 0; p < np; ++p) s3 += X(3, p);
      m[3][3] -= s3 / np;
    }
  }
  const double nrm = (rt ? a.norm_rt[j1] : a.norm_cb[j1]) / gsca;
  double* out = rt ? a.out_rt : a.out_cb;
  for (int s = 0; s < 4; ++s)
    for (int c = 0; c < 4; ++c) out[(size_t)(4 * s + c) * nt + j1] = m[s][c] * nrm;
}

}  // namespace

extern "C" {

int mcrt_run_rt(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_geometry* g, const mcrt_run_opts* opts,
                double* M_rt, double* M_cb, double energy[5], mcrt_stats* stats) {
  if (!ctx || !cfg || !g || !M_rt || !M_cb || !energy)
    return set_err(MCRT_EINVAL, "mcrt_run_rt: NULL argument");
  if (opts && opts->kernel == MCRT_KERNEL_PLAIN)
    return set_err(MCRT_EINVAL, "mcrt_run_rt runs the persistent kernel (one batched launch)");
  int rc = validate_geometry(g);
  if (rc) return rc;
  rc = validate_config(cfg, g->kind);
  if (rc) return rc;
  // incident states: plane.jl:70-75 (6, columns) and sphere.jl:49-52 (2)
  static const double IP[6][4] = {{1, -1, 0, 0}, {1, 1, 0, 0}, {1, 0, -1, 0},
                                  {1, 0, 1, 0},  {1, 0, 0, -1}, {1, 0, 0, 1}};
  static const double IS[2][4] = {{1, -1, 0, 0}, {1, 0, 0, -1}};
  const bool plane = g->kind == MCRT_PLANE;
  const int n = plane ? 6 : 2;
  std::vector<const mcrt_geometry*> gs(n, g);
  std::vector<double> I(4 * (size_t)n);
  std::vector<uint64_t> seeds(n, opts ? opts->seed : 0);
  std::vector<uint32_t> ids(n);
  std::vector<long long> nph(n, cfg->number_of_rays);
  for (int i = 0; i < n; ++i) {
    for (int s = 0; s < 4; ++s) I[4 * i + s] = plane ? IP[i][s] : IS[i][s];
    ids[i] = (opts ? opts->instance : 0) + (uint32_t)i;
  }
  CK(cudaSetDevice(ctx->device));
  Group G;
  rc = build_group(ctx, cfg, gs.data(), reinterpret_cast<const double(*)[4]>(I.data()), seeds.data(), ids.data(),
                   nph.data(), opts ? opts->photon_begin : 0, opts ? opts->rng_mode : 0, n, opts, G);
  if (rc) return rc;
  rc = launch_group(G);
  if (rc) return rc;

  RunRtArgs a{};
  a.kind = g->kind;
  a.n_states = n;
  a.nt = cfg->n_theta;
  a.np = cfg->n_phi;
  a.ntb = cfg->n_theta_b;
  a.npb = cfg->n_phi_b;
  a.per_inst = G.per_inst;
  a.nrt = G.nrt;
  a.ncb = G.ncb;
  a.tally = G.d_tally.as<double>();
  a.inv_n = cfg->number_of_rays > 0 ? 1.0 / (double)cfg->number_of_rays : 0.0;
  std::vector<double> nrm(a.nt + a.ntb);
  for (int j = 0; j < a.nt; ++j)
    nrm[j] = plane ? std::fabs(1.0 / (4.0 * cfg->cos_theta[j] * cfg->inorm[j])) : 1.0 / cfg->inorm[j];
  for (int j = 0; j < a.ntb; ++j) nrm[a.nt + j] = plane ? 1.0 / std::fabs(4.0 * cfg->cos_theta_b[j]) : 1.0;
  // first polarisation of each plane state (MonteCarloRadiativeTransfer.jl:208-215)
  int k1s[6] = {0};
  double k2s[6] = {0};
  for (int i = 0; plane && i < n; ++i) {
    for (int j = 1; j < 4; ++j)
      if (std::fabs(I[4 * i + j]) > 1.0 - 2.220446049250313e-16) {
        k1s[i] = j;
        k2s[i] = I[4 * i + j];
        break;
      }
    if (k1s[i] == 1) a.coef[i][0] += 0.5;
    a.coef[i][k1s[i]] += 0.5 * k2s[i];
  }
  for (int i = 0; !plane && i < n; ++i) a.vstate[i] = I[4 * i + 3] != 0.0;
  for (int i = 0; i < 8; ++i) {
    a.nfi[i] = i * a.np / 8;
    a.nfib[i] = i * a.npb / 8;
  }
  const size_t n_rt = 16 * (size_t)a.nt * (plane ? a.np : 1), n_cb = 16 * (size_t)a.ntb * (plane ? a.npb : 1);
  DevBuf d_out;
  CK(d_out.alloc((nrm.size() + n_rt + n_cb) * sizeof(double)));
  double* dn = d_out.as<double>();
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpyAsync(dn, nrm.data(), nrm.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  a.norm_rt = dn;
  a.norm_cb = dn + a.nt;
  a.out_rt = dn + nrm.size();
  a.out_cb = a.out_rt + n_rt;
  Range rr("mcrt run_rt epilogue");
  const int items = plane ? a.nt * a.np + a.ntb * a.npb : a.nt + a.ntb;
  if (plane)
    k_run_rt_plane<<<(items + 127) / 128, 128, 0, st>>>(a);
  else
    k_run_rt_sphere<<<(items + 127) / 128, 128, 0, st>>>(a);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(M_rt, a.out_rt, n_rt * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(M_cb, a.out_cb, n_cb * sizeof(double), cudaMemcpyDeviceToHost, st));
  rc = finish_group(G);
  if (rc) return rc;
  // energies from the per-state A tallies
  double e[5] = {0, 0, 0, 0, 0};
  unsigned flags = 0;
  mcrt_stats tot;
  std::memset(&tot, 0, sizeof tot);
  for (int i = 0; i < n; ++i) {
    double A[5];
    mcrt_stats si;
    rc = read_instance(G, i, A, nullptr, nullptr, nullptr, &si);
    if (rc) return rc;
    flags |= (unsigned)si.status_flags;
    tot.photons += si.photons;
    tot.events += si.events;
    tot.attempts += si.attempts;
    tot.rt_evals += si.rt_evals;
    tot.cb1_evals += si.cb1_evals;
    tot.cbn_evals += si.cbn_evals;
    tot.cb_peak_sum += si.cb_peak_sum;
    tot.cb_peak_sumsq += si.cb_peak_sumsq;
    tot.block_size = si.block_size;
    tot.blocks = si.blocks;
    tot.kernel_ms = si.kernel_ms;
    if (plane && k1s[i] == 1)
      for (int s = 0; s < 5; ++s) e[s] += 0.5 * A[s] * a.inv_n;
    if (!plane && !a.vstate[i]) {
      e[0] += A[0] * a.inv_n;
      e[1] += A[1] * a.inv_n;
      e[2] += A[2] * a.inv_n;
      e[4] += A[4] * a.inv_n;
    }
  }
  for (int s = 0; s < 5; ++s) energy[s] = e[s];
  tot.status_flags = (int)flags;
  if (stats) *stats = tot;
  if (flags & MCRT_FLAG_REJECT_LIMIT)
    return set_err(MCRT_ENONCONV, "a rejection loop hit its iteration cap; see stats.status_flags");
  return MCRT_OK;
}

}  // extern "C"

// ================================================================== FP32 peak
namespace {
// Eight independent FMA chains per thread; the result is stored only if it is
// impossible, so nothing is elided.
__global__ void k_fma_peak(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
        x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      x0 = fmaf(x0, a, b);
      x1 = fmaf(x1, a, b);
      x2 = fmaf(x2, a, b);
      x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b);
      x5 = fmaf(x5, a, b);
      x6 = fmaf(x6, a, b);
      x7 = fmaf(x7, a, b);
    }
  }
  float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == -1.2345f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" int mcrt_measure_fp32_peak(mcrt_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return set_err(MCRT_EINVAL, "mcrt_measure_fp32_peak: NULL argument");
  CK(cudaSetDevice(ctx->device));
  DevBuf out;
  const int threads = 256, blocks = ctx->sms * 8, iters = 4096;
  CK(out.alloc((size_t)threads * blocks * sizeof(float)));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    CK(cudaEventRecord(ctx->e0, ctx->stream));
    k_fma_peak<<<blocks, threads, 0, ctx->stream>>>(out.as<float>(), iters, 0.9999f, 0.0001f);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->e1, ctx->stream));
    CK(cudaEventSynchronize(ctx->e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ctx->e0, ctx->e1));
    if (rep > 0) best = std::min(best, ms);
  }
  const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  return MCRT_OK;
}

// ================================================================== serving loop
// Continuous batching in front of the persistent kernel (declared in include/mcrt.h).
namespace {

// Bin tables laid out for a given device address (defined with the no-allocation path).
template <typename T>
std::vector<unsigned char> pack_bins_at(const HostBins& H, const unsigned char* dev);

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Device memory owned by one resident request, released stream-ordered so that freeing
// never waits for the wave still running on the device.
struct AsyncBuf {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  ~AsyncBuf() {
    if (p) cudaFreeAsync(p, st);
  }
};

struct SrvReq {
  uint64_t id = 0;
  mcrt_config cfg{};
  std::vector<double> arrays[9];
  mcrt_geometry geom{};
  std::vector<mcrt_layer> layers;
  double I0[4] = {0, 0, 0, 0};
  uint64_t seed = 0;
  uint32_t inst = 0;
  long long nph = 0;
  DevInstance D{};
  std::vector<unsigned char> binbytes;
  AsyncBuf tally, bins;
  size_t nrt = 0, ncb = 0, per_inst = 0;
  double footprint = 0;
  long long next = 0;       // next photon index to hand to a wave
  long long last_wave = -1; // last wave that carried photons of this request
  int waves = 0;
  int state = 0;            // 0 pending, 1 resident, 2 done, 3 failed
  unsigned status = 0;
  double t_sub = 0, t_adm = 0, t_done = 0;
  std::vector<double> result;  // raw sums once done
  double bins_per_event = 0;   // RT + CB bin evaluations of one event (CB weighted by its cost)
  double cost = 0;             // estimated bin evaluations per photon (measured after each wave)
  double meas[2] = {0, 0};     // photons and events finished so far (read back after a wave)
};

}  // namespace

struct mcrt_server {
  mcrt_ctx* ctx = nullptr;
  mcrt_server_opts o{};
  KInfo ki{};
  int bs = 256, blocks = 0, tf4 = 0;
  size_t smem = 0;
  cudaStream_t stream = nullptr;
  // Read-backs after a wave (results, cost counters) run here, so that they do not queue
  // behind the wave that waits on `stream`.
  cudaStream_t copy_stream = nullptr;
  struct Slot {
    DevBuf d_wave, d_claim, d_status, d_state, d_tacc;
    DevInstance* h_wave = nullptr;  // pinned; read by the wave's copy when it runs
    cudaGraphExec_t gexec = nullptr;
    cudaEvent_t start = nullptr, done = nullptr;
    long long wave_id = -1;
    std::vector<SrvReq*> members;
    bool in_flight = false;
  } slot[2];
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  int fatal = 0;
  std::string fatal_msg;
  uint64_t next_id = 1;
  long long next_wave = 0;
  std::deque<SrvReq*> pending;
  std::vector<SrvReq*> active;
  std::map<uint64_t, std::unique_ptr<SrvReq>> reqs;
  double resident = 0, peak_resident = 0, busy_s = 0, completed = 0, photons_done = 0;
};

namespace {

// Footprint of a request: its tallies, bin tables and Mie tables.
double request_footprint(const SrvReq& r) {
  double b = (double)r.per_inst * sizeof(double) + (double)r.binbytes.size() + 4096.0;
  for (int s = 0; s < r.D.n_scat; ++s)
    if (r.D.scat[s].kind == 1) b += 32.0 * (r.D.scat[s].ntheta + 1) + 4.0 * (r.D.scat[s].rp + 4);
  return b;
}

// Bin evaluations of one event: every RT bin (a slab event near both faces peels off into
// both hemispheres) and every CB bin, a reciprocal-path CB bin counted as 3.2 RT bins (its
// measured cost ratio in the transport kernel).
double request_bins_per_event(const SrvReq& r) {
  return (double)r.cfg.n_theta * r.cfg.n_phi + (r.cfg.compute_cb ? 3.2 * r.cfg.n_theta_b * r.cfg.n_phi_b : 0.0);
}

// Events per photon before any has been measured: the fewer of the events that
// absorption alone takes to bring the weight to minimum_intensity and a diffusion
// estimate (2 + tau^2 for the total optical size), capped by maximum_scattering_times.
double request_events_prior(const SrvReq& r) {
  double tau = 0.0, om = 0.0;
  for (int i = 0; i < r.geom.n_layers; ++i) {
    tau += r.layers[i].infinite ? 50.0 : r.layers[i].tau;
    om = std::max(om, r.layers[i].omega);
  }
  const double absorb = std::log(1.0 / std::max(r.cfg.minimum_intensity, 1e-300)) / std::max(1.0 - om, 1e-4);
  return std::max(1.0, std::min({(double)r.cfg.maximum_scattering_times, absorb, 2.0 + tau * tau}));
}

// Admits pending requests while the cap and slot count allow (under the lock).
int srv_admit(mcrt_server* S) {
  while (!S->pending.empty() && (int)S->active.size() < S->o.max_active) {
    SrvReq* r = S->pending.front();
    if (S->resident + r->footprint > S->o.memory_cap_bytes && !S->active.empty()) break;
    S->pending.pop_front();
    r->tally.st = r->bins.st = S->stream;
    if (cudaMallocAsync(&r->tally.p, r->per_inst * sizeof(double), S->stream) != cudaSuccess ||
        cudaMallocAsync(&r->bins.p, r->binbytes.size(), S->stream) != cudaSuccess)
      return set_err(MCRT_ENOMEM, "server: device allocation for a request failed");
    // bin tables carry absolute pointers: rebuild them for the final address
    HostBins H = make_bins(&r->cfg, r->geom.kind,
                           host::Sph{r->D.kfs[0], r->D.kfs[1], r->D.kfs[2], r->D.kfs[3]});
    r->binbytes = S->o.precision == MCRT_FP32 ? pack_bins_at<float>(H, (unsigned char*)r->bins.p)
                                              : pack_bins_at<double>(H, (unsigned char*)r->bins.p);
    CK(cudaMemcpyAsync(r->bins.p, r->binbytes.data(), r->binbytes.size(), cudaMemcpyHostToDevice, S->stream));
    CK(cudaMemsetAsync(r->tally.p, 0, r->per_inst * sizeof(double), S->stream));
    r->D.bins = r->bins.p;
    assign_tally(r->D, (double*)r->tally.p, tally_layout(&r->cfg));
    r->state = 1;
    r->t_adm = now_s();
    S->active.push_back(r);
    S->resident += r->footprint;
    S->peak_resident = std::max(S->peak_resident, S->resident);
  }
  return MCRT_OK;
}

// Waits for the wave in slot b and retires the requests whose last photons it carried.
int srv_retire(mcrt_server* S, int b) {
  auto& sl = S->slot[b];
  if (!sl.in_flight) return MCRT_OK;
  CK(cudaEventSynchronize(sl.done));
  float ms = 0;
  cudaEventElapsedTime(&ms, sl.start, sl.done);
  unsigned status = 0;
  CK(cudaMemcpy(&status, sl.d_status.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
  std::vector<SrvReq*> finished;
  for (SrvReq* r : sl.members) {
    r->status |= status;
    if (r->last_wave == sl.wave_id && r->next >= r->nph) finished.push_back(r);
  }
  // The wave has finished (its event was waited on), so the finished requests' tallies
  // are complete; the next wave, queued on S->stream, does not touch them.
  for (SrvReq* r : finished) {
    r->result.resize(r->per_inst);
    CK(cudaMemcpyAsync(r->result.data(), r->tally.p, r->per_inst * sizeof(double), cudaMemcpyDeviceToHost,
                       S->copy_stream));
  }
  // The photons and events each unfinished member has completed so far (a wave still
  // running may be adding to them; the value is only an estimate): its measured cost per
  // photon sizes its quanta in later waves.
  if (S->o.wave_work > 0)
    for (SrvReq* r : sl.members)
      if (!(r->last_wave == sl.wave_id && r->next >= r->nph))
        CK(cudaMemcpyAsync(r->meas, r->D.acc + ACC_PHOTONS, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                           S->copy_stream));
  CK(cudaStreamSynchronize(S->copy_stream));
  for (SrvReq* r : sl.members)
    if (r->meas[0] > 0) r->cost = r->bins_per_event * std::max(r->meas[1] / r->meas[0], 1.0);
  std::lock_guard<std::mutex> lk(S->mu);
  S->busy_s += ms * 1e-3;
  for (SrvReq* r : finished) {
    r->tally.~AsyncBuf();
    new (&r->tally) AsyncBuf();
    r->bins.~AsyncBuf();
    new (&r->bins) AsyncBuf();
    r->state = 2;
    r->t_done = now_s();
    S->resident -= r->footprint;
    S->completed += 1;
    S->photons_done += (double)r->nph;
    S->active.erase(std::find(S->active.begin(), S->active.end(), r));
  }
  sl.in_flight = false;
  sl.members.clear();
  S->cv.notify_all();
  return MCRT_OK;
}

int srv_launch(mcrt_server* S, int b) {
  Range r("mcrt serve wave");
  auto& sl = S->slot[b];
  if (S->o.use_graphs) {
    CK(cudaEventRecord(sl.start, S->stream));
    CK(cudaGraphLaunch(sl.gexec, S->stream));
    CK(cudaEventRecord(sl.done, S->stream));
  } else {
    CK(cudaEventRecord(sl.start, S->stream));
    CK(cudaMemcpyAsync(sl.d_wave.p, sl.h_wave, S->o.max_active * sizeof(DevInstance), cudaMemcpyHostToDevice,
                       S->stream));
    CK(cudaMemsetAsync(sl.d_claim.p, 0, sl.d_claim.n, S->stream));
    CK(cudaMemsetAsync(sl.d_status.p, 0, sl.d_status.n, S->stream));
    KParams p{sl.d_wave.as<const DevInstance>(), S->o.max_active, sl.d_state.as<uint4>(),
              sl.d_tacc.as<double>(), sl.d_status.as<unsigned>(), S->tf4};
    CK(launch_transport(S->ki, S->blocks, S->bs, S->smem, S->stream, p));
    CK(cudaEventRecord(sl.done, S->stream));
  }
  sl.in_flight = true;
  return MCRT_OK;
}

// Builds the next wave in slot b from the resident requests with photons left.
int srv_build_wave(mcrt_server* S, int b, bool& launched) {
  launched = false;
  auto& sl = S->slot[b];
  std::vector<SrvReq*> members;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    for (SrvReq* r : S->active)
      if (r->next < r->nph) members.push_back(r);
  }
  if (members.empty()) return MCRT_OK;
  std::stable_sort(members.begin(), members.end(),
                   [](SrvReq* a, SrvReq* c) { return a->nph - a->next > c->nph - c->next; });
  // Each member's quantum: an equal share of wave_photons (at least min_quantum), or,
  // with wave_work > 0, its equal share of the wave's bin evaluations over its cost per
  // photon. The photon quanta measured better on the mixed request stream (lower median
  // and tail latency, fewer GPU-busy seconds for the same work).
  const long long q = std::max<long long>(S->o.min_quantum, S->o.wave_photons / (long long)members.size());
  const double share = S->o.wave_work / (double)members.size();
  const long long wid = S->next_wave++;
  for (int i = 0; i < S->o.max_active; ++i) {
    DevInstance& W = sl.h_wave[i];
    if (i < (int)members.size()) {
      SrvReq* r = members[i];
      long long qi = q;
      if (S->o.wave_work > 0)
        qi = std::max<long long>(32, (long long)std::min(share / std::max(r->cost, 1.0), 1e15));
      W = r->D;
      W.photon_begin = r->next;
      W.n_photons = std::min<long long>(qi, r->nph - r->next);
      r->next += W.n_photons;
      r->last_wave = wid;
      r->waves += 1;
    } else {
      W.n_photons = 0;  // padding: skipped by the kernel
    }
    W.claim = sl.d_claim.as<unsigned long long>() + 2 * i;
  }
  sl.members = members;
  sl.wave_id = wid;
  int rc = srv_launch(S, b);
  if (rc) return rc;
  launched = true;
  return MCRT_OK;
}

void srv_fail(mcrt_server* S, int rc) {
  std::lock_guard<std::mutex> lk(S->mu);
  S->fatal = rc;
  S->fatal_msg = g_err;
  for (auto& kv : S->reqs)
    if (kv.second->state < 2) kv.second->state = 3;
  S->cv.notify_all();
}

void srv_loop(mcrt_server* S) {
  cudaSetDevice(S->ctx->device);
  int cur = 0;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->stop) break;
      int rc = srv_admit(S);
      if (rc) {
        lk.unlock();
        srv_fail(S, rc);
        return;
      }
      if (S->active.empty() && !S->slot[0].in_flight && !S->slot[1].in_flight) {
        S->cv.wait_for(lk, std::chrono::milliseconds(5));
        continue;
      }
    }
    // Slot cur held the wave before last; retire it, then refill it, so one wave always
    // waits queued behind the running one.
    int rc = srv_retire(S, cur);
    if (rc) return srv_fail(S, rc);
    {
      std::lock_guard<std::mutex> lk(S->mu);
      rc = srv_admit(S);
    }
    if (rc) return srv_fail(S, rc);
    bool launched = false;
    rc = srv_build_wave(S, cur, launched);
    if (rc) return srv_fail(S, rc);
    if (!launched) {
      rc = srv_retire(S, cur ^ 1);
      if (rc) return srv_fail(S, rc);
    }
    cur ^= 1;
  }
  srv_retire(S, 0);
  srv_retire(S, 1);
}

}  // namespace

extern "C" int mcrt_server_create(mcrt_ctx* ctx, const mcrt_server_opts* opts, mcrt_server** out) {
  if (!ctx || !out) return set_err(MCRT_EINVAL, "mcrt_server_create: NULL argument");
  *out = nullptr;
  std::unique_ptr<mcrt_server> S(new mcrt_server());
  S->ctx = ctx;
  if (opts) S->o = *opts;
  if (S->o.memory_cap_bytes <= 0) S->o.memory_cap_bytes = 20e9;
  if (S->o.max_active <= 0) S->o.max_active = 256;
  if (S->o.wave_photons <= 0) S->o.wave_photons = 1 << 20;
  if (S->o.min_quantum <= 0) S->o.min_quantum = 4096;
  if (S->o.precision != MCRT_FP32 && S->o.precision != MCRT_FP64)
    return set_err(MCRT_EINVAL, "precision must be MCRT_FP32 or MCRT_FP64");
  CK(cudaSetDevice(ctx->device));
  S->bs = S->o.precision == MCRT_FP32 ? 256 : 128;
  kernel_info(S->o.precision, S->bs, S->ki);
  // room for one 1801-angle Mie table set in shared memory; larger sets read through L1
  S->tf4 = 2 * 1802 + (1002 + 3) / 4;
  S->smem = S->ki.shared_static + (size_t)S->tf4 * 16;
  CK(cudaFuncSetAttribute(S->ki.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S->smem));
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, S->ki.fn, S->bs, S->smem));
  if (occ < 1) return set_err(MCRT_EINVAL, "server: kernel does not fit");
  S->blocks = ctx->sms * occ;
  CK(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&S->copy_stream, cudaStreamNonBlocking));
  const size_t slots = (size_t)S->blocks * S->bs;
  for (auto& sl : S->slot) {
    CK(sl.d_wave.alloc(S->o.max_active * sizeof(DevInstance)));
    CK(sl.d_claim.alloc(2 * S->o.max_active * sizeof(unsigned long long)));
    CK(sl.d_status.alloc(sizeof(unsigned)));
    CK(sl.d_state.alloc(slots * S->ki.state_bytes));
    CK(sl.d_tacc.alloc(slots * NACC * sizeof(double)));
    CK(cudaMallocHost(&sl.h_wave, S->o.max_active * sizeof(DevInstance)));
    std::memset(sl.h_wave, 0, S->o.max_active * sizeof(DevInstance));
    for (int i = 0; i < S->o.max_active; ++i) sl.h_wave[i].claim = sl.d_claim.as<unsigned long long>() + 2 * i;
    CK(cudaEventCreate(&sl.start));
    CK(cudaEventCreate(&sl.done));
    if (S->o.use_graphs) {
      // One graph per slot: copy the wave table, clear the counters, run the wave.
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
      cudaMemcpyAsync(sl.d_wave.p, sl.h_wave, S->o.max_active * sizeof(DevInstance), cudaMemcpyHostToDevice,
                      S->stream);
      cudaMemsetAsync(sl.d_claim.p, 0, sl.d_claim.n, S->stream);
      cudaMemsetAsync(sl.d_status.p, 0, sl.d_status.n, S->stream);
      KParams p{sl.d_wave.as<const DevInstance>(), S->o.max_active, sl.d_state.as<uint4>(), sl.d_tacc.as<double>(),
                sl.d_status.as<unsigned>(), S->tf4};
      launch_transport(S->ki, S->blocks, S->bs, S->smem, S->stream, p);
      CK(cudaStreamEndCapture(S->stream, &g));
      cudaError_t e = cudaGraphInstantiate(&sl.gexec, g, 0);
      cudaGraphDestroy(g);
      CK(e);
    }
  }
  mcrt_server* raw = S.release();
  raw->worker = std::thread(srv_loop, raw);
  *out = raw;
  return MCRT_OK;
}

extern "C" int mcrt_server_submit(mcrt_server* S, const mcrt_request* q, uint64_t* ticket) {
  if (!S || !q || !ticket || !q->config || !q->geometry)
    return set_err(MCRT_EINVAL, "mcrt_server_submit: NULL argument");
  int rc = validate_geometry(q->geometry);
  if (rc) return rc;
  rc = validate_config(q->config, q->geometry->kind);
  if (rc) return rc;
  if (q->n_photons < 0) return set_err(MCRT_EINVAL, "n_photons must be >= 0");
  std::unique_ptr<SrvReq> r(new SrvReq());
  const mcrt_config* c = q->config;
  r->cfg = *c;
  const double* src[9] = {c->cos_phi, c->sin_phi, c->cos_theta, c->sin_theta, c->inorm,
                          c->cos_theta_b, c->sin_theta_b, c->cos_phi_b, c->sin_phi_b};
  const int len[9] = {c->n_phi, c->n_phi, c->n_theta, c->n_theta, c->n_theta,
                      c->n_theta_b, c->n_theta_b, c->n_phi_b, c->n_phi_b};
  for (int i = 0; i < 9; ++i) r->arrays[i].assign(src[i], src[i] + len[i]);
  r->cfg.cos_phi = r->arrays[0].data();
  r->cfg.sin_phi = r->arrays[1].data();
  r->cfg.cos_theta = r->arrays[2].data();
  r->cfg.sin_theta = r->arrays[3].data();
  r->cfg.inorm = r->arrays[4].data();
  r->cfg.cos_theta_b = r->arrays[5].data();
  r->cfg.sin_theta_b = r->arrays[6].data();
  r->cfg.cos_phi_b = r->arrays[7].data();
  r->cfg.sin_phi_b = r->arrays[8].data();
  r->cfg.number_of_rays = q->n_photons;
  r->layers.assign(q->geometry->layers, q->geometry->layers + q->geometry->n_layers);
  r->geom = *q->geometry;
  r->geom.layers = r->layers.data();
  for (int s = 0; s < 4; ++s) r->I0[s] = q->I0[s];
  r->seed = q->seed;
  r->inst = q->instance;
  r->nph = q->n_photons;
  host::Sph kfs;
  rc = make_instance(&r->cfg, &r->geom, r->I0, r->seed, r->inst, 0, r->nph, 0, r->D, kfs);
  if (rc) return rc;
  HostBins H = make_bins(&r->cfg, r->geom.kind, kfs);
  r->binbytes = S->o.precision == MCRT_FP32 ? pack_bins_at<float>(H, nullptr) : pack_bins_at<double>(H, nullptr);
  const TallyLayout TL = tally_layout(c);
  r->nrt = TL.nrt;
  r->ncb = TL.ncb;
  r->per_inst = TL.per_inst;
  r->footprint = request_footprint(*r);
  if (r->footprint > S->o.memory_cap_bytes)
    return set_err(MCRT_EBUSY, "request footprint exceeds the server's memory cap");
  r->bins_per_event = request_bins_per_event(*r);
  r->cost = r->bins_per_event * request_events_prior(*r);
  r->t_sub = now_s();
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->fatal) return set_err(S->fatal, "server stopped: " + S->fatal_msg);
  r->id = S->next_id++;
  *ticket = r->id;
  if (r->nph == 0) {  // nothing to run
    r->state = 2;
    r->result.assign(r->per_inst, 0.0);
    r->t_adm = r->t_done = r->t_sub;
  } else {
    S->pending.push_back(r.get());
  }
  S->reqs[r->id] = std::move(r);
  S->cv.notify_all();
  return MCRT_OK;
}

extern "C" int mcrt_server_wait(mcrt_server* S, uint64_t ticket, double timeout_ms) {
  if (!S) return set_err(MCRT_EINVAL, "mcrt_server_wait: NULL server");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return set_err(MCRT_ENOTFOUND, "unknown ticket");
  SrvReq* r = it->second.get();
  const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double, std::milli>(timeout_ms);
  while (r->state < 2) {
    if (S->cv.wait_until(lk, until) == std::cv_status::timeout && r->state < 2)
      return set_err(MCRT_ETIMEDOUT, "mcrt_server_wait: timed out");
  }
  if (r->state == 3) return set_err(S->fatal ? S->fatal : MCRT_ECUDA, "server failed: " + S->fatal_msg);
  return MCRT_OK;
}

extern "C" int mcrt_server_result(mcrt_server* S, uint64_t ticket, double A_out[5], double* Irt, double* Icb,
                                  double* lad, mcrt_ticket_info* info) {
  if (!S) return set_err(MCRT_EINVAL, "mcrt_server_result: NULL server");
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return set_err(MCRT_ENOTFOUND, "unknown ticket");
  SrvReq* r = it->second.get();
  if (r->state != 2) return set_err(MCRT_EBUSY, "result not ready");
  const double inv = r->nph > 0 ? 1.0 / (double)r->nph : 0.0;
  const double* h = r->result.data();
  const double* acc = h + r->nrt + r->ncb + r->ncb / 4;
  if (A_out)
    for (int s = 0; s < 5; ++s) A_out[s] = acc[s] * inv;
  if (Irt)
    for (size_t i = 0; i < r->nrt; ++i) Irt[i] = h[i] * inv;
  if (Icb)
    for (size_t i = 0; i < r->ncb; ++i) Icb[i] = h[r->nrt + i] * inv;
  if (lad)
    for (size_t i = 0; i < r->ncb / 4; ++i) lad[i] = h[r->nrt + r->ncb + i] * inv;
  if (info) {
    info->submitted_s = r->t_sub;
    info->admitted_s = r->t_adm;
    info->completed_s = r->t_done;
    info->footprint_bytes = r->footprint;
    info->photons = r->nph;
    info->waves = r->waves;
    info->status_flags = (int)r->status;
  }
  S->reqs.erase(it);
  return MCRT_OK;
}

extern "C" int mcrt_server_stats(mcrt_server* S, double out[8]) {
  if (!S || !out) return set_err(MCRT_EINVAL, "mcrt_server_stats: NULL argument");
  std::lock_guard<std::mutex> lk(S->mu);
  out[0] = S->completed;
  out[1] = S->photons_done;
  out[2] = (double)S->next_wave;
  out[3] = S->busy_s;
  out[4] = S->peak_resident;
  out[5] = S->resident;
  out[6] = (double)S->pending.size();
  out[7] = (double)S->active.size();
  return MCRT_OK;
}

extern "C" int mcrt_server_destroy(mcrt_server* S) {
  if (!S) return MCRT_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv.notify_all();
  }
  if (S->worker.joinable()) S->worker.join();
  cudaSetDevice(S->ctx->device);
  cudaStreamSynchronize(S->stream);
  S->reqs.clear();
  cudaStreamSynchronize(S->stream);
  for (auto& sl : S->slot) {
    if (sl.gexec) cudaGraphExecDestroy(sl.gexec);
    if (sl.h_wave) cudaFreeHost(sl.h_wave);
    if (sl.start) cudaEventDestroy(sl.start);
    if (sl.done) cudaEventDestroy(sl.done);
  }
  cudaStreamDestroy(S->stream);
  if (S->copy_stream) cudaStreamDestroy(S->copy_stream);
  delete S;
  return MCRT_OK;
}

// ================================================================== no device allocation
// mcrt_simulate_noalloc: the persistent-kernel simulate for callers that must not
// allocate device memory at call time (declared in include/mcrt.h, which states the
// contract). All call-time device storage lives in g_noalloc_scratch below.
namespace {

// The device array every mcrt_simulate_noalloc call works in. Each GPU that loads the
// library holds it until the process exits; calls reuse it, so overlapping calls race.
static __device__ __align__(256) unsigned char g_noalloc_scratch[MCRT_NOALLOC_SCRATCH_BYTES];

// In host code g_noalloc_scratch names a host-side stand-in, not a device address, so
// the device address is looked up once per device (with that device current) and kept.
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_base[NOALLOC_MAX_DEVICES] = {};

int noalloc_base(int device, unsigned char** out) {
  if (device < 0 || device >= NOALLOC_MAX_DEVICES)
    return set_err(MCRT_EINVAL, "mcrt_simulate_noalloc: device index out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_base[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_err(MCRT_ECUDA, std::string("mcrt_simulate_noalloc: cudaGetSymbolAddress failed: ") +
                                     cudaGetErrorString(e));
    g_noalloc_base[device] = static_cast<unsigned char*>(p);
  }
  *out = g_noalloc_base[device];
  return MCRT_OK;
}

// The launch shape of mcrt_simulate_noalloc: one block per SM of this many threads.
int noalloc_block_size(int prec) { return prec == MCRT_FP32 ? 256 : 128; }

// Called by mcrt_ctx_create with the context's device current. Looking up the array's
// address loads the module that holds it (and so creates the array on the device where
// modules load lazily); querying the two kernels it launches loads theirs. Afterwards a
// call allocates nothing on the device.
int noalloc_prepare(mcrt_ctx* ctx) {
  int rc = noalloc_base(ctx->device, &ctx->noalloc_scratch);
  if (rc) return rc;
  for (int prec : {MCRT_FP32, MCRT_FP64}) {
    KInfo ki;
    if (!kernel_info(prec, noalloc_block_size(prec), ki)) return set_err(MCRT_EINVAL, "no kernel for this precision");
    cudaFuncAttributes fa;
    CK(cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(ki.fn)));
  }
  return MCRT_OK;
}

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// The bin tables of upload_bins laid out at a given device address, as host bytes.
template <typename T>
std::vector<unsigned char> pack_bins_at(const HostBins& H, const unsigned char* dev) {
  Packer P;
  BinTables<T> hdr{};
  P.add(&hdr, sizeof(hdr));
  auto addv = [&](const std::vector<double>& v) {
    std::vector<T> t(v.begin(), v.end());
    if (t.empty()) t.push_back(T(0));
    return P.add(t.data(), t.size() * sizeof(T));
  };
  size_t o_st = addv(H.st), o_ct = addv(H.ct), o_g = addv(H.g), o_w = addv(H.w), o_cp = addv(H.cp),
         o_sp = addv(H.sp);
  size_t o_kfx = addv(H.kfx), o_kfy = addv(H.kfy), o_kfz = addv(H.kfz), o_ehx = addv(H.ehx),
         o_ehy = addv(H.ehy), o_gb = addv(H.gb), o_cf2 = addv(H.cf2), o_sf2 = addv(H.sf2),
         o_c1 = addv(H.c1), o_c2 = addv(H.c2), o_c3 = addv(H.c3);
  size_t o_upb = P.add(H.upb.data(), H.upb.size() * sizeof(int));
  size_t o_stb = addv(H.stb), o_ctb = addv(H.ctb), o_cpb = addv(H.cpb), o_spb = addv(H.spb);
  size_t o_rtp = P.add(H.rtp.data(), H.rtp.size() * sizeof(float));
  hdr.ntheta = H.ntheta;
  hdr.nphi = H.nphi;
  hdr.nthetab = H.nthetab;
  hdr.nphib = H.nphib;
  hdr.up0 = H.up0;
  hdr.up1 = H.up1;
  hdr.lo0 = H.lo0;
  hdr.lo1 = H.lo1;
  auto at = [&](size_t o) { return reinterpret_cast<const T*>(dev + o); };
  hdr.st = at(o_st);
  hdr.ct = at(o_ct);
  hdr.g = at(o_g);
  hdr.w = at(o_w);
  hdr.cp = at(o_cp);
  hdr.sp = at(o_sp);
  hdr.kfx = at(o_kfx);
  hdr.kfy = at(o_kfy);
  hdr.kfz = at(o_kfz);
  hdr.ehx = at(o_ehx);
  hdr.ehy = at(o_ehy);
  hdr.gb = at(o_gb);
  hdr.cf2 = at(o_cf2);
  hdr.sf2 = at(o_sf2);
  hdr.c1 = at(o_c1);
  hdr.c2 = at(o_c2);
  hdr.c3 = at(o_c3);
  hdr.upb = reinterpret_cast<const int*>(dev + o_upb);
  hdr.stb = at(o_stb);
  hdr.ctb = at(o_ctb);
  hdr.cpb = at(o_cpb);
  hdr.spb = at(o_spb);
  hdr.rtp = reinterpret_cast<const float4*>(dev + o_rtp);
  hdr.rtp_lo = H.rtp_lo;
  hdr.rtp_zero = H.rtp_zero;
  std::memcpy(P.bytes.data(), &hdr, sizeof(hdr));
  return P.bytes;
}

}  // namespace

extern "C" int mcrt_simulate_noalloc(mcrt_ctx* ctx, const mcrt_config* cfg, const mcrt_geometry* g,
                                     const double I0[4], const mcrt_run_opts* opts, double A_out[5],
                                     double* Irt, double* Icb, double* Icb_ladder, mcrt_stats* stats) {
  if (!ctx || !I0 || !A_out || !Irt || !Icb)
    return set_err(MCRT_EINVAL, "mcrt_simulate_noalloc: NULL argument");
  int rc = validate_geometry(g);
  if (rc) return rc;
  rc = validate_config(cfg, g->kind);
  if (rc) return rc;
  const int prec = opts ? opts->precision : MCRT_FP32;
  if (prec != MCRT_FP32 && prec != MCRT_FP64)
    return set_err(MCRT_EINVAL, "precision must be MCRT_FP32 or MCRT_FP64");
  if (opts && opts->kernel != MCRT_KERNEL_PERSISTENT)
    return set_err(MCRT_EINVAL, "mcrt_simulate_noalloc runs the persistent kernel only");
  const int bs = noalloc_block_size(prec);
  if (opts && opts->block_size != 0 && opts->block_size != bs)
    return set_err(MCRT_EINVAL, "mcrt_simulate_noalloc runs 256 threads per block (FP32) or 128 (FP64); "
                                "block_size must be 0 or that value");
  if (opts && opts->blocks_per_sm != 0 && opts->blocks_per_sm != 1)
    return set_err(MCRT_EINVAL, "mcrt_simulate_noalloc runs one block per SM; blocks_per_sm must be 0 or 1");
  if (opts && opts->table_staging != 0 && opts->table_staging != 1)
    return set_err(MCRT_EINVAL, "mcrt_simulate_noalloc stages Mie tables in shared memory; table_staging "
                                "must be 0 or 1");
  CK(cudaSetDevice(ctx->device));
  unsigned char* base = ctx->noalloc_scratch;
  if (!base) return set_err(MCRT_EINVAL, "mcrt_simulate_noalloc: the context has no scratch array");

  DevInstance D;
  host::Sph kfs;
  rc = make_instance(cfg, g, I0, opts ? opts->seed : 0, opts ? opts->instance : 0, opts ? opts->rng_mode : 0,
                     cfg->number_of_rays, opts ? opts->photon_begin : 0, D, kfs);
  if (rc) return rc;
  if (opts && opts->max_attempts > 0) D.max_attempts = opts->max_attempts;
  HostBins H = make_bins(cfg, g->kind, kfs);

  // Launch shape: one block per SM.
  KInfo ki;
  if (!kernel_info(prec, bs, ki)) return set_err(MCRT_EINVAL, "no kernel for this precision");
  int tf4 = table_f4_of(D);
  size_t smem = ki.shared_static + (size_t)tf4 * 16;
  if (smem > (size_t)ctx->smem_optin) {
    // the tables that do not fit are read from global memory through L1
    tf4 = (int)(((long long)ctx->smem_optin - (long long)ki.shared_static) / 16);
    if (tf4 < 0) return set_err(MCRT_EINVAL, "block size too large for shared memory");
    smem = ki.shared_static + (size_t)tf4 * 16;
  }
  CK(cudaFuncSetAttribute(ki.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ki.fn, bs, smem));
  if (occ < 1) return set_err(MCRT_EINVAL, "kernel does not fit on an SM with this block size");
  const int blocks = ctx->sms;
  const size_t slots = (size_t)blocks * bs;

  // Layout of the scratch array.
  const TallyLayout TL = tally_layout(cfg);
  const size_t nrt = TL.nrt, ncb = TL.ncb, per_inst = TL.per_inst;
  std::vector<unsigned char> binbytes;
  const size_t off_inst = 0;
  const size_t off_bins = align256(sizeof(DevInstance));
  binbytes = prec == MCRT_FP32 ? pack_bins_at<float>(H, base + off_bins) : pack_bins_at<double>(H, base + off_bins);
  const size_t off_tally = align256(off_bins + binbytes.size());
  const size_t off_claim = align256(off_tally + per_inst * sizeof(double));
  const size_t off_status = off_claim + 2 * sizeof(unsigned long long);
  const size_t off_state = align256(off_status + sizeof(unsigned));
  const size_t off_tacc = align256(off_state + slots * ki.state_bytes);
  const size_t need = off_tacc + slots * NACC * sizeof(double);
  if (need > MCRT_NOALLOC_SCRATCH_BYTES) {
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "mcrt_simulate_noalloc: this config needs %zu bytes of device scratch; the array holds %u "
                  "(MCRT_NOALLOC_SCRATCH_BYTES); use mcrt_simulate",
                  need, (unsigned)MCRT_NOALLOC_SCRATCH_BYTES);
    return set_err(MCRT_EINVAL, msg);
  }
  double* tally = reinterpret_cast<double*>(base + off_tally);
  D.bins = base + off_bins;
  assign_tally(D, tally, TL);
  D.claim = reinterpret_cast<unsigned long long*>(base + off_claim);

  // The array keeps the previous call's contents: write the inputs and clear the
  // tallies, the claim counter and the status word (the kernel clears its per-thread
  // accumulators itself).
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpyAsync(base + off_inst, &D, sizeof(DevInstance), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(base + off_bins, binbytes.data(), binbytes.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(base + off_tally, 0, off_state - off_tally, st));
  KParams p;
  p.inst = reinterpret_cast<const DevInstance*>(base + off_inst);
  p.n_inst = 1;
  p.state = reinterpret_cast<uint4*>(base + off_state);
  p.tacc = reinterpret_cast<double*>(base + off_tacc);
  p.status = reinterpret_cast<unsigned*>(base + off_status);
  p.table_f4 = tf4;
  CK(cudaEventRecord(ctx->e0, st));
  CK(launch_transport(ki, blocks, bs, smem, st, p));
  CK(cudaEventRecord(ctx->e1, st));
  CK(cudaEventSynchronize(ctx->e1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->e0, ctx->e1));
  std::vector<double> h(per_inst);
  unsigned status = 0;
  CK(cudaMemcpy(h.data(), tally, per_inst * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&status, base + off_status, sizeof(unsigned), cudaMemcpyDeviceToHost));

  const double inv = cfg->number_of_rays > 0 ? 1.0 / (double)cfg->number_of_rays : 0.0;
  const double* acc = h.data() + nrt + ncb + ncb / 4;
  for (int s = 0; s < 5; ++s) A_out[s] = acc[s] * inv;
  for (size_t i = 0; i < nrt; ++i) Irt[i] = h[i] * inv;
  for (size_t i = 0; i < ncb; ++i) Icb[i] = h[nrt + i] * inv;
  if (Icb_ladder)
    for (size_t i = 0; i < ncb / 4; ++i) Icb_ladder[i] = h[nrt + ncb + i] * inv;
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->cb_peak_sum = acc[ACC_PEAK];
    stats->cb_peak_sumsq = acc[ACC_PEAK2];
    stats->photons = acc[ACC_PHOTONS];
    stats->events = acc[ACC_EVENTS];
    stats->attempts = acc[ACC_ATTEMPTS];
    stats->rt_evals = acc[ACC_RT];
    stats->cb1_evals = acc[ACC_CB1];
    stats->cbn_evals = acc[ACC_CBN];
    stats->kernel_ms = ms;
    stats->status_flags = (int)status;
    stats->block_size = bs;
    stats->blocks = blocks;
  }
  if (status & MCRT_FLAG_REJECT_LIMIT)
    return set_err(MCRT_ENONCONV, "a rejection loop hit its iteration cap; see stats.status_flags");
  return MCRT_OK;
}
