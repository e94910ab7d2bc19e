// Declarations of the FermiNet / MH / reduction kernels (kernels.cu).
#pragma once
#include "act.cuh"
#include "common.cuh"

namespace qmc {

// Value-only determinant passes whose orbital matrices arrive without the
// envelope factor: the factors (launch_envelope_value, laid out like the
// matrices) are multiplied in, and written back, as the matrices are loaded.
struct EnvArgs {
  const float* env;  // [B][K][n][n]
};
// Split n contiguous fp32 values into bf16 hi / lo planes (`plane` elements apart).
cudaError_t launch_to_split(cudaStream_t s, size_t n, const float* src, __nv_bfloat16* dst, size_t plane);

// Multiply raw value-only orbital matrices [w][k][i][j] by their envelopes in place.
cudaError_t launch_envelope_apply(cudaStream_t s, int B, int n, int n_up, int split, int K, int A, int env_abs,
                                  const float* pi0, const float* sg0, const float* pi1, const float* sg1,
                                  const float* rae, float* Amat);
// Diagonal envelope with the product rule, in place on orbital matrices stored
// without an envelope (value layout for Tp == 1, tangent layout otherwise).
cudaError_t launch_envelope_diag(cudaStream_t s, int B, int n, int n_up, int split, int K, int A, int Tp, int T,
                                 const float* pi0, const float* sg0, const float* pi1, const float* sg1,
                                 const float* aevec, float* Amat);
// Envelopes [w][k][i][j] of the value-only orbital matrices.
cudaError_t launch_envelope_value(cudaStream_t s, int B, int n, int n_up, int split, int K, int A, int env_abs,
                                  const float* pi0, const float* sg0, const float* pi1, const float* sg1,
                                  const float* rae, float* env);


// Features of MoleculeFeatures (input/atomic.py:46-79) with tangents.
//  X0    [(w*n+i)*Tp + t][K0p]   one-electron rows (ae features)
//  H2    [(w*n+i)*n + j][P2][4]  two-electron rows, compact tangents
//  rae   [w*n+i][A], aevec [w*n+i][A][3]
//  pe    [w] Coulomb potential (may be null)
// P2 = 5 (value, Laplacian wrt r_i-r_j, d/d(r_i-r_j)_{x,y,z}) when T > 1, else 1.
cudaError_t launch_features(cudaStream_t s, int B, int n, int A, int Tp, int T, int K0p,
                            const float* electrons, const float* atoms, const float* charges,
                            double nuc, float* X0, float* H2, float* rae, float* aevec, float* pe,
                            int n_up = 0, int C = 0, int g2p = 0, float* G2 = nullptr);

// Value-only inputs of the mixed form's first layer, one block per walker:
// rae / aevec / pe and H2 as launch_features (P2 = 1); X0 as split bf16
// [w*n+i][K0p]; the pair rows' spin means G2 as split bf16 [w*n+i][g2p]; and
// the broadcast term Gb [w][dout] = (spin means of X0) W_g1 [g1p][dout].
size_t inputs_value_smem(int n, int A, int g1p);
cudaError_t launch_inputs_value(cudaStream_t s, int B, int n, int A, int n_up, int C, int K0p, int g1p, int g2p,
                                int dout, const float* electrons, const float* atoms, const float* charges,
                                double nuc, const float* Wg1, float* rae, float* aevec, float* H2, StSplit X0s,
                                StSplit G2s, float* Gb, float* pe);

// Forward-Laplacian inputs of the mixed form's first layer, one block per
// walker: rae / aevec / pe and H2 (P2 = 5) as launch_features; X0 as split
// bf16 [(w*n+i)*Tp + t][K0p]; the pair rows' spin means G2 (split) with their
// tangent rules as launch_mean_h2; Gb [w*Tp + t][dout] = (spin means of X0) W_g1.
bool inputs_fl_supported(int n, int A, int Tp, int g1p);
cudaError_t launch_inputs_fl(cudaStream_t s, int B, int n, int A, int n_up, int C, int Tp, int T, int K0p, int g1p,
                             int g2p, int dout, const float* electrons, const float* atoms, const float* charges,
                             double nuc, const float* Wg1, float* rae, float* aevec, float* H2, StSplit X0s,
                             StSplit G2s, float* Gb, float* pe);

// Tangent two-electron layer (P2 = 5, 32 outputs) fused with the next
// one-electron layer's pair means: Hout as launch_pair_layer (skipped when
// null), G2 [(w*n+i)*Tp + t][g2p] as launch_mean_h2 on Hout; one block per
// walker (16 n threads, n <= 32).  cudaErrorNotSupported for shapes it does
// not cover.
template <class Out>
cudaError_t launch_pair_layer_mean_fl(cudaStream_t s, int B, int n, int n_up, int C, int Tp, int T, int d_in,
                                      int d_out, const float* Hin, const float* W, const float* b, float* Hout,
                                      int g2p, Out G2);

// Two-electron layer h2' = residual(tanh(h2 W + b)) on compact tangent rows.
cudaError_t launch_pair_layer(cudaStream_t s, int npairs, int P2, int d_in, int d_out,
                              const float* Hin, const float* W, const float* b, float* Hout);

// Value-only two-electron layer fused with the spin means of its output
// (written as the next layer's G2 rows [w*n+i][s*d_out + f]); returns
// cudaErrorNotSupported for widths or electron counts it does not cover.
template <class Out>
cudaError_t launch_pair_layer_mean(cudaStream_t s, int B, int n, int n_up, int C, int d_in, int d_out,
                                   const float* Hin, const float* W, const float* b, float* Hout, int g2p,
                                   Out G2);

// Spin-channel means of the one-electron rows: G1[(w*Tp+t)][s*d + f]
// (padding columns up to the output row width are written as zero).
template <class In, class Out>
cudaError_t launch_mean_h1(cudaStream_t s, int B, int n, int n_up, int C, int Tp, int d, In X, int g1p,
                           Out G1);

// Spin-channel means of the two-electron rows expanded to full tangents:
// G2[(w*n+i)*Tp + t][s*d2 + f].
template <class Out>
cudaError_t launch_mean_h2(cudaStream_t s, int B, int n, int n_up, int C, int Tp, int T, int d2,
                           int P2, const float* H2, int g2p, Out G2);

// Per-walker determinant stage: LU/log|det| of the K value matrices, FP64
// signed log-sum-exp and, when T > 1, the slogdet forward-Laplacian traces
// combined into the kinetic energy.  A: [w][k][Tp][n][n].  gl_add [B][T-1]
// (optional, tangent passes): gradient (T-2) and Laplacian of a log term added
// to log|det| before the kinetic energy (the Psiformer's Jastrow).
// fl_scratch (optional, logdet_fl_scratch_bytes): with it, tangent passes with
// 16 < n <= 64 run the FP32 block-per-walker kernel and recompute only the
// determinants it marks in FP64.
// cancel64 (tangent passes): also evaluate in FP64 every determinant whose
// FP32 kinetic term cancels beyond kCancelScore (the FP32 form's accuracy
// guard; see kernels.cu).
cudaError_t launch_logdet(cudaStream_t s, int B, int n, int K, int Tp, int T, const float* A,
                          const float* pe, float* logpsi, float* sign, float* ke, float* el,
                          uint8_t* flags, int* n_refactor, const EnvArgs* env = nullptr,
                          const float* gl_add = nullptr, void* fl_scratch = nullptr, bool cancel64 = false);
size_t logdet_fl_scratch_bytes(int B, int K, int T);

// Cotangent of log|psi| with respect to the value orbital matrices:
// Abar[w][k] = w_k A_k^{-T}; also writes log|psi| (may be null).
cudaError_t launch_logdet_bwd(cudaStream_t s, int B, int n, int K, const float* A, float* Abar, float* logpsi);

// Value-only two-electron stream fused over all its layers (see kernels.cu).
constexpr int kPairStreamMax = 8;
struct PairStreamArgs {
  int n, n_up, C, nl;
  int din[kPairStreamMax];                  // 4 or 32; outputs are 32 wide
  const float* W[kPairStreamMax];           // [din][32]
  const float* b[kPairStreamMax];           // [32]
  const float* H0;                          // [B][n][n][din[0]] pair features
  int g2p[kPairStreamMax];                  // padded width of the means after layer l
  const uint4* Wf[kPairStreamMax];          // split-BF16 fragments of W (mixed form), launch_pair_frags
};
template <class Out>
struct PairStreamOut {
  Out G2[kPairStreamMax];                   // means after pair layer l (input of layer l+1)
};
size_t pair_stream_smem(int n, int nl);
// B fragments of one 32-wide pair layer W [din][32] (din <= 32) for the
// mixed-form stream: out[ks][nt][lane] = {b0 hi, b1 hi, b0 lo, b1 lo}.
cudaError_t launch_pair_frags(cudaStream_t s, const float* W, int din, uint4* out);
template <class Out>
cudaError_t launch_pair_stream_value(cudaStream_t s, int B, const PairStreamArgs& a, const PairStreamOut<Out>& o);


// Several jobs of one model in one MH batch (device tables): job j owns
// walkers [offsets[j], offsets[j + 1]) and draws from seeds[j] with update
// index counters[j] + step, indexed by the walker's position in its job.
struct MhGroup {
  int n_jobs = 0;
  const int* offsets = nullptr;
  const uint64_t* seeds = nullptr;
  const uint64_t* counters = nullptr;
};

// MH proposal x' = x + stddev * N(0,1) for update `step` of a call.
// The update index is ctr (+ *ctr_dev when ctr_dev is not null).
cudaError_t launch_mh_propose(cudaStream_t s, int B, int n, const float* x, float* xp,
                              float stddev, uint64_t seed, uint64_t ctr, const uint64_t* ctr_dev,
                              const float* inj_normals, const MhGroup& grp = MhGroup{});
// Accept/reject with 2 log|psi| and the draw for update `ctr` (+ *ctr_dev).
cudaError_t launch_mh_accept(cudaStream_t s, int B, int n, float* x, const float* xp, float* lp,
                             const float* logpsi_p, uint64_t seed, uint64_t ctr, const uint64_t* ctr_dev,
                             const float* inj_uniforms, uint32_t* accepts, const MhGroup& grp = MhGroup{});
// ctr[0 .. count) += inc on the stream.
cudaError_t launch_counter_add(cudaStream_t s, uint64_t* ctr, uint64_t inc, int count = 1);
cudaError_t launch_mh_draws(cudaStream_t s, int B, int n, int steps, uint64_t seed, uint64_t ctr,
                            float* normals, float* uniforms);
cudaError_t launch_scale(cudaStream_t s, int B, const float* in, float c, float* out);

// FP64 mean/variance of x[0, B), or per segment [offsets[s], offsets[s + 1])
// (device offsets, `segments` of them) into out[2 s], out[2 s + 1].
cudaError_t launch_reduce_mean_var(cudaStream_t s, int B, const float* x, double* out,
                                   const int* offsets = nullptr, int segments = 1);

// fp32 [rows][cols] (row stride ld_in) -> fp32 transposed [cols][rows]
cudaError_t launch_transpose_f32(cudaStream_t s, const float* in, int rows, int cols, int ld_in, float* out);

// fp32 [rows][cols] -> transposed split-bf16 planes hi/lo of [cols_p][rows_p]
// (zero padded; the lo plane starts cols_p*rows_p elements after hi)
cudaError_t launch_transpose_split(cudaStream_t s, const float* in, int rows, int cols, int ld_in,
                                   __nv_bfloat16* out, int rows_p, int cols_p);

}  // namespace qmc
