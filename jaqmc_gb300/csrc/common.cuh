// Internal declarations shared by the qmc CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <stdio.h>

#include <string>

#include "../../include/qmc.h"

namespace qmc {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
qmc_status cuda_status(cudaError_t e, const char* what);

#define QMC_CUDA(call)                                                     \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) return ::qmc::cuda_status(e_, #call);           \
  } while (0)
#define QMC_LAUNCH(what)                                                   \
  do {                                                                     \
    cudaError_t e_ = cudaGetLastError();                                   \
    if (e_ != cudaSuccess) return ::qmc::cuda_status(e_, what);            \
  } while (0)
#define QMC_TRY(expr)                                                      \
  do {                                                                     \
    qmc_status s_ = (expr);                                                \
    if (s_ != QMC_OK) return s_;                                           \
  } while (0)

__host__ __device__ inline int round_up(int x, int m) { return (x + m - 1) / m * m; }
__host__ __device__ inline size_t align_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

constexpr float kRsqrt2 = 0.70710678118654752440f;

// Orbital matrices A (row i = electron, column j = orbital, determinant k).
// Value passes (Tp == 1): A[w][k][i][j].  Tangent passes: A[w][t][i][k][j],
// so the K*n columns (k, j) of one electron row and tangent are contiguous
// (a warp's output columns store as one run); a matrix then has row stride
// K*n and tangent stride n*K*n.
__host__ __device__ inline size_t amat_index(int Tp, int n, int K, size_t w, int k, int t, int i, int j) {
  return Tp == 1 ? ((w * K + k) * n + i) * (size_t)n + j : (((w * Tp + t) * n + i) * (size_t)K + k) * n + j;
}
__host__ __device__ inline int amat_row_stride(int Tp, int n, int K) { return Tp == 1 ? n : K * n; }
__host__ __device__ inline size_t amat_tangent_stride(int n, int K) { return (size_t)n * K * n; }
constexpr int kMaxAtoms = 64;

// Floats of one envelope channel's pi and sigma (the reference's shapes:
// pi (n_orb, A, K); sigma (n_orb, A, K), or (n_orb, A, 3, K) for the diagonal
// envelope; the null envelope has neither).
__host__ __device__ inline size_t env_pi_floats(int kind, int n, int A, int K) {
  return kind == QMC_ENVELOPE_NULL ? 0 : (size_t)n * A * K;
}
__host__ __device__ inline size_t env_sigma_floats(int kind, int n, int A, int K) {
  return kind == QMC_ENVELOPE_NULL ? 0 : (size_t)n * A * K * (kind == QMC_ENVELOPE_DIAGONAL ? 3 : 1);
}
// The orbital GEMM epilogues apply the isotropic envelopes themselves; the
// diagonal envelope is applied afterwards by launch_envelope_diag and the
// null envelope not at all.
__host__ __device__ inline bool env_in_epilogue(int kind) {
  return kind == QMC_ENVELOPE_ISOTROPIC || kind == QMC_ENVELOPE_ABS_ISOTROPIC;
}

// ---------------------------------------------------------------- model
// Dimensions derived from qmc_ferminet_config.  Widths with a trailing `p`
// are padded to a multiple of 8 (the K step of the SIMT GEMM); padded
// activation columns and weight rows are kept at zero.
struct Dims {
  int n_up, n_dn, n, A, K, L, C;  // C: non-empty spin channels
  int split;                      // per-spin orbitals/envelopes
  int env_abs;                    // isotropic envelopes: |sigma| (abs_isotropic)
  int env_kind;                   // QMC_ENVELOPE_*
  int d1_in[QMC_MAX_LAYERS], d2_in[QMC_MAX_LAYERS];
  int d1[QMC_MAX_LAYERS], d2[QMC_MAX_LAYERS];
  int upd2[QMC_MAX_LAYERS];
  int d1_in_p[QMC_MAX_LAYERS];   // padded one-electron input width
  int g1_p[QMC_MAX_LAYERS];      // padded width of the spin means of h1 (C*d1_in)
  int g2_p[QMC_MAX_LAYERS];      // padded width of the spin means of h2 (C*d2_in)
  int d_last;                    // width of the last one-electron layer
  int norb;                      // K*n orbital columns per electron
  int norb_p;                    // norb padded to a multiple of 8 (weight row stride)
};

// Device arena layout (float offsets) of the derived parameters.
struct ArenaLayout {
  size_t w_main[QMC_MAX_LAYERS];  // [(d1_in_p + g2_p) x d1]   rows: W_h ; W_g2
  size_t w_g1[QMC_MAX_LAYERS];    // [g1_p x d1]
  size_t b1[QMC_MAX_LAYERS];      // [d1]
  size_t w2[QMC_MAX_LAYERS];      // [d2_in x d2]
  size_t b2[QMC_MAX_LAYERS];      // [d2]
  size_t w_orb[2];                // [d_last x norb_p] per channel (zero padded columns)
  size_t env_pi[2], env_sigma[2]; // [n x A x K] per channel (reference layout)
  size_t atoms, charges;          // [A x 3], [A]
  // FP32 transposes for the adjoint's input-gradient GEMMs
  size_t wt_main[QMC_MAX_LAYERS]; // [d1 x (d1_in_p + g2_p)]
  size_t wt_g1[QMC_MAX_LAYERS];   // [d1 x g1_p]
  size_t wt2[QMC_MAX_LAYERS];     // [d2 x d2_in]
  size_t wt_orb[2];               // [norb_p x d_last]
  size_t total;                   // floats
  // bf16 arena (element offsets) for the mixed form: transposed weights
  size_t t_main[QMC_MAX_LAYERS];  // [d1 x (d1_in_p + g2_p)] K-major
  size_t t_g1[QMC_MAX_LAYERS];    // [d1 x g1_p]
  size_t t_orb[2];                // [norb_p x d_last]
  // first layer on the tensor cores: its kernel with each source (features,
  // pair means) padded to whole 64-column chunks, as fp32 [k0w][d1] and as
  // bf16 planes [d1][k0w]
  size_t w0_pad, t0_pad;
  int k0w;
  // 32-wide two-electron layers as split-BF16 m16n8k16 B fragments
  // (bf16 offsets; 256 x 16 bytes per layer, in per-lane order)
  size_t pfrag[QMC_MAX_LAYERS];
  size_t total_bf16;
};

// Source offsets of each leaf in the flat parameter vector.
struct ParamLayout {
  size_t dense1_k[QMC_MAX_LAYERS], dense1_b[QMC_MAX_LAYERS];
  size_t dense2_k[QMC_MAX_LAYERS], dense2_b[QMC_MAX_LAYERS];
  size_t orb_k[2];
  size_t env_pi[2], env_sigma[2];
  size_t total;
};

}  // namespace qmc

namespace qmc {
struct PsiModel;
}

struct qmc_model {
  int kind = 0;                    // QMC_KIND_FERMINET or QMC_KIND_PSIFORMER
  qmc::PsiModel* psi = nullptr;    // Psiformer dims and layouts (kind == PSIFORMER)
  qmc::Dims d;
  qmc::ArenaLayout a;
  qmc::ParamLayout p;
  int precision;
  int device;
  float* arena = nullptr;          // derived fp32 parameters
  __nv_bfloat16* arena_bf16 = nullptr;
  float atoms_host[3 * qmc::kMaxAtoms];
  float charges_host[qmc::kMaxAtoms];
  double nuclear_repulsion = 0.0;  // sum_{I<J} Z_I Z_J / R_IJ
  int* dev_err = nullptr;          // device error word of bounded waits
  bool params_set = false;
  size_t grad_budget = (size_t)8 << 30;  // bytes for the adjoint's chunked workspace
  size_t energy_budget = (size_t)32 << 30;  // bytes for the chunked Psiformer local-energy workspace
  int n_sms = 0;
  // FP64 re-evaluation of determinants whose FP32 kinetic term cancels
  // (qmc_model_set_det_guard): -1 = by precision (on for FP32, off for mixed)
  int det_guard = -1;
  bool det_guard_on() const { return det_guard < 0 ? precision == QMC_PRECISION_FP32 : det_guard != 0; }
};

namespace qmc {

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11): 10 rounds of the
// multiply/xor-swap round function with the published multipliers and Weyl
// key increments.
struct U4 { uint32_t x, y, z, w; };

__host__ __device__ inline uint32_t mulhilo(uint32_t a, uint32_t b, uint32_t* hi) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  return (uint32_t)p;
}

__host__ __device__ inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, hi1;
    uint32_t lo0 = mulhilo(M0, c.x, &hi0);
    uint32_t lo1 = mulhilo(M1, c.z, &hi1);
    U4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// Open-interval uniform from the top 24 bits: ((x >> 8) + 0.5) * 2^-24.
__host__ __device__ inline float u01(uint32_t x) {
  return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// Draw layout of one MH step for one walker: Philox blocks b = 0..nb-1 with
// counter (b, walker, step_lo, step_hi) give 4 words each.  Words are
// consumed in pairs by Box-Muller for the 3n normals (block 0 .. ceil(3n/4)-1);
// the accept uniform is word x of block ceil(3n/4).
__host__ __device__ inline int normal_blocks(int n) { return (3 * n + 3) / 4; }

}  // namespace qmc
