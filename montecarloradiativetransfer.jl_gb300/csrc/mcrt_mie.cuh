// Mie table producer on the device: bhmie (src/scatterers/mie.jl:129-216) and
// calculate_csrn (src/utils.jl:263-287) for a batch of scatterers in one launch, one
// thread block per scatterer. It writes the FP32 tables the transport kernels read
// (float4 F = (F11, F12, F33, F34) and S = (S11, S22) per angle, plus the inverse-CDF
// knots) and the FP64 results, so a new (x, m) never round-trips through the host.
#pragma once

#include <cuda_runtime.h>

namespace mcrt {

// FP64 results of one scatterer, in this order (doubles):
//   [0] omega, [1] kl, [2..6] q_ext, q_sca, q_abs, q_back, asymm,
//   then F11, F12, F33, F34 (nt each), S11, S22 (2 nt each, re/im), csrn (rp + 1).
inline size_t mie_result_doubles(int nt, int rp) { return 7 + 8 * (size_t)nt + (size_t)rp + 1; }

struct MieJob {
  double x, m_re, m_im, r, nu;
  int nt, rp, nstop, nmax;
  double* d;      // scratch: 2 (nmax + 1) doubles, the log-derivative D_n (re, im)
  double* ab;     // scratch: 4 (nstop + 1) doubles, a_n and b_n (re, im)
  double* terms;  // scratch: 2 (rp + 1) doubles, the CDF terms and their running sums
  double* out;    // FP64 results (mie_result_doubles)
  float4* F;      // nt + 1 (last entry zero)
  float4* S;      // nt + 1
  float* C;       // nc = round_up(rp + 2, 4): rp + 1 knots, then the last repeated
  int nc;
};

cudaError_t launch_mie_tables(const MieJob* jobs, int n, cudaStream_t st);

}  // namespace mcrt
