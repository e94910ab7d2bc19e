// Split-BF16 tcgen05 GEMMs of the mixed form (stream_tc.cu).
//
// All three GEMMs are computed transposed, D[f][c] = sum_k W^T[f][k] X[c][k]:
// output features f sit on the 128 TMEM lanes of a CTA's accumulator and the
// tile's activation rows c (whole tangent groups) on TMEM columns, so one
// epilogue thread owns every tangent of one output element.  Operands are
// two-plane split BF16 (hi, lo) in HBM; the MMA issues hi*hi + hi*lo + lo*hi
// with FP32 accumulation in TMEM.
#pragma once
#include "act.cuh"
#include "common.cuh"

namespace qmc {

// Padded tangent count used by the tensor-core tiles (a multiple of 4 such
// that whole groups fill a tile whose width is a multiple of 16 and <= 256).
int tc_padded_tangents(int T);
// Groups per column tile for padded tangent count Tp.
int tc_groups_per_tile(int Tp);
// Whether the one-electron layer with these padded widths runs on tcgen05.
bool tc_layer_supported(int k1, int k2, int n_out);

struct TcLayerArgs {
  int n_groups, n, Tp, T;
  const __nv_bfloat16* X; int k1; size_t x_plane;   // [rows][k1] split planes
  const __nv_bfloat16* G2; int k2; size_t g2_plane; // [rows][k2] split planes
  const __nv_bfloat16* Wt; int n_out;               // [n_out][w_ld] split planes
  int w_ld;  // weight row: 0 = k1 + k2 (k1 a multiple of 64); else 64 * (chunks of k1 + chunks of k2),
             // the second source's weights starting at column 64 * ceil(k1 / 64)
  const float* Gb; const float* bias;
  bool residual;
  __nv_bfloat16* out; size_t out_plane;             // [rows][n_out] split planes
  int* err;
};
// z = [X | G2] W + Gb + b; tanh with the forward-Laplacian tangent rules;
// residual (X + h)/sqrt(2) when `residual`.
qmc_status tc_stream_layer(cudaStream_t s, const TcLayerArgs& a);

struct TcStoreArgs {
  int n_rows;
  const __nv_bfloat16* X; int k; size_t x_plane;    // [n_rows][k] split planes
  const __nv_bfloat16* Wt; int n_out;               // [n_out][k] split planes
  float* out;                                       // [n_rows][ld_out] fp32
  int* err;
  int ld_out = 0;                                   // row stride of out (0: n_out)
};
// out = X W (the spin-mean broadcast term of a layer).
qmc_status tc_store_gemm(cudaStream_t s, const TcStoreArgs& a);

struct TcOrbitalArgs {
  int B, n, n_up, split, Tp, T, K, natom, env_abs;
  const __nv_bfloat16* X; int k; size_t x_plane;    // [rows][k] split planes (last layer)
  const __nv_bfloat16* Wt[2]; int norb;             // per channel [norb][k] split planes
  const float* pi[2]; const float* sigma[2];        // per channel [n][A][K]
  const float* rae; const float* aevec;
  float* A;                                         // [w][k][Tp][n][n]
  int raw;           // T == 1: store orbitals without the envelope (applied by the LU pass)
  int unit_env;      // T > 1: orbitals without an envelope (diagonal / null envelopes)
  int* err;
};
// orbital projection x envelope with the product rule.
qmc_status tc_orbitals(cudaStream_t s, const TcOrbitalArgs& a);

}  // namespace qmc
