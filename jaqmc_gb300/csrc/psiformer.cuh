// Psiformer + SimpleEE Jastrow (value path): layouts shared by psiformer.cu
// and the entry points of api.cu.
#pragma once
#include "common.cuh"
#include "plan.cuh"

namespace qmc {

constexpr int kPsiMaxLayers = 8;
constexpr int kPsiMaxMlp = 4;  // hidden MLP widths per layer (plus the final one back to D)
constexpr int kLapMaxLocal = 4;  // LapNet: local updates of the individual stream per layer

// The attention-backbone models share this description: the Psiformer
// (arch 0) and LapNet (arch 1, src/jaqmc/wavefunction/backbone/lapnet/
// _backbone.py: an individual stream hs giving queries and keys, a dense
// stream hd giving values and carrying the attention and update residuals).
enum { kArchPsiformer = 0, kArchLapNet = 1 };

struct PsiDims {
  int arch;
  int n, n_up, n_dn, A, K;
  int L, H, Dh, D;                // layers, heads, head width, attention width H*Dh
  int n_dense;                    // MLP dense layers per block (hidden widths + 1)
  int mlp[kPsiMaxMlp + 1];        // output widths of the MLP dense layers (last = D)
  int split, env_abs, jastrow;
  int K0, K0p;                    // 4A + 1 input features, padded to a multiple of 8
  int n_local;                    // LapNet: local updates per layer (not in the last layer)
  int in_bias, bb_bias;           // LapNet: input / backbone projections have biases
};

// Offsets (floats) of each leaf in the flat parameter vector (reference leaf
// order of PsiformerWavefunction); the arena starts with a verbatim copy.
struct PsiParams {
  size_t in_k, in_b;
  size_t ln0_s[kPsiMaxLayers], ln0_b[kPsiMaxLayers];
  size_t q_k[kPsiMaxLayers], q_b[kPsiMaxLayers], k_k[kPsiMaxLayers], k_b[kPsiMaxLayers];
  size_t v_k[kPsiMaxLayers], v_b[kPsiMaxLayers], o_k[kPsiMaxLayers], o_b[kPsiMaxLayers];
  size_t ln1_s[kPsiMaxLayers], ln1_b[kPsiMaxLayers];
  size_t mlp_k[kPsiMaxLayers][kPsiMaxMlp + 1], mlp_b[kPsiMaxLayers][kPsiMaxMlp + 1];
  size_t orb_k[2], env_pi[2], env_sigma[2];
  size_t alpha_par, alpha_anti;
  // LapNet (arch 1): query|key, value, output, value-update and local-update
  // projections per layer (bias offsets only when the model has biases)
  size_t qk_k[kPsiMaxLayers], qk_b[kPsiMaxLayers], lv_k[kPsiMaxLayers], lv_b[kPsiMaxLayers];
  size_t lo_k[kPsiMaxLayers], lo_b[kPsiMaxLayers], vu_k[kPsiMaxLayers], vu_b[kPsiMaxLayers];
  size_t ul_k[kPsiMaxLayers][kLapMaxLocal], ul_b[kPsiMaxLayers][kLapMaxLocal];
  size_t total;
};

// Derived parameters after the verbatim copy (float offsets into the arena)
// and the split-bf16 K-major copies of the GEMM weights (bf16 offsets).
struct PsiArena {
  size_t w_in;                    // [K0p][D] input kernel, zero rows past K0
  size_t w_qkv[kPsiMaxLayers];    // [D][3D]: query | key | value kernels side by side
  size_t b_qkv[kPsiMaxLayers];    // [3D]
  // FP32 transposes for the adjoint's input-cotangent GEMMs
  size_t t32_qkv[kPsiMaxLayers];  // [3D][D]
  size_t t32_o[kPsiMaxLayers];    // [D][D]
  size_t t32_mlp[kPsiMaxLayers][kPsiMaxMlp + 1];  // [dout][din]
  // LapNet: biases (zero when the model has none): input, output,
  // value-update and local-update projections; b_qkv holds query|key|value
  size_t lb_in, lb_o[kPsiMaxLayers], lb_vu[kPsiMaxLayers], lb_ul[kPsiMaxLayers][kLapMaxLocal];
  // LapNet FP32 transposes for the adjoint ([dout][din]; t32_qkv holds query|key, t32_o the output)
  size_t t32_v[kPsiMaxLayers], t32_vu[kPsiMaxLayers], t32_ul[kPsiMaxLayers][kLapMaxLocal];
  size_t total;
  size_t t_qkv[kPsiMaxLayers];    // [3D][D] (LapNet: query|key [2D][D])
  size_t t_o[kPsiMaxLayers];      // [D][D]
  size_t t_mlp[kPsiMaxLayers][kPsiMaxMlp + 1];
  size_t t_v[kPsiMaxLayers], t_vu[kPsiMaxLayers], t_ul[kPsiMaxLayers][kLapMaxLocal];  // LapNet [D][D]
  size_t total_bf16;
};

struct PsiModel {
  PsiDims d;
  PsiParams p;
  PsiArena a;
};

// Workspace of a Psiformer value pass: the shared fields of Plan (orbital
// matrices, envelope scratch, MH buffers, the backbone output in h1[0]) plus
// the backbone's own buffers.
struct PsiPlan {
  Plan base;
  size_t x;     // [rows][D] f32 residual stream
  size_t xn;    // [rows][D] GEMM input (f32, or two bf16 planes)
  size_t z;     // [rows][max(3D, mlp)] f32 GEMM output
  size_t att;   // [rows][D] attention output, GEMM input
  size_t jas;   // [B] Jastrow
  size_t jgl;   // [B][3n+1] Jastrow gradient and Laplacian (forward-Laplacian passes)
  size_t in_plane;  // bf16 elements between planes of xn / att / h1[0]
  size_t x2, xn2, z2;  // LapNet: individual stream (f32), its GEMM operand, projection outputs [rows][D]
};

PsiPlan psi_make_plan(const qmc_model* m, int B);

// Forward-Laplacian local energy (psiformer.cu driver, psiformer_fl.cu kernels).
// Rows carry T = 3n+2 tangents (padded to the tensor-core tile in the mixed
// form); walkers run in chunks of psi_fl_chunk so the workspace stays bounded.
PsiPlan psi_fl_plan(const qmc_model* m, int B);
int psi_fl_chunk(const qmc_model* m, int batch);
qmc_status psi_fl_check(const qmc_model* m);
qmc_status psi_local_energy(qmc_model* m, int batch, const float* electrons, float* e_local, float* ke,
                            float* pe, float* logpsi, uint8_t* flags, void* ws, cudaStream_t s);

cudaError_t launch_psi_features_fl(cudaStream_t s, int B, int n, int n_up, int A, int Tp, int T, int K0p,
                                   const float* x, const float* atoms, const float* charges, double nuc,
                                   const float* alpha, float* X0, float* rae, float* aevec, float* pe,
                                   float* jas, float* jgl);
template <class Out>
cudaError_t launch_psi_group_fl(cudaStream_t s, int groups, int Tp, int D, const float* z, int ldz,
                                const float* bias, int act, float* x, int xmode, const float* ln_s,
                                const float* ln_b, Out out);
// The input layer of a tangent pass in one kernel: z = x0 W_in formed per
// electron for its nonzero tangent rows (value, Laplacian, its own three
// Jacobian rows), then launch_psi_group_fl's act 0 / xmode 1 rules.
template <class Out>
cudaError_t launch_psi_input_fl(cudaStream_t s, int groups, int n, int Tp, int D, const float* x0, int k0,
                                int k0p, const float* w_in, const float* bias, float* x, const float* ln_s,
                                const float* ln_b, Out out);
template <class Out>
cudaError_t launch_psi_attention_fl(cudaStream_t s, int B, int n, int Tp, int T, int H, int Dh, const float* qkv,
                                    const float* bqkv, Out out);
bool psi_attention_fl_supported(int n, int Dh);
// The split-BF16 warp-MMA variant of the forward-Laplacian attention
// (attention_mma.cu), used by the mixed form when the shape allows it.
bool psi_attention_fl_mma_supported(int n, int Dh);
template <class Out>
cudaError_t launch_psi_attention_fl_mma(cudaStream_t s, int B, int n, int Tp, int T, int H, int Dh, const float* qkv,
                                        const float* bqkv, Out out);
qmc_status psi_evaluate(qmc_model* m, const PsiPlan& pp, void* ws, const float* electrons, float* logpsi,
                        float* sign, uint8_t* flags, cudaStream_t s);
qmc_status psi_set_params(qmc_model* m, const float* params, cudaStream_t s);
// Value-pass features (log-rescaled ae features + spin column, rae, aevec) and
// the SimpleEE Jastrow per walker (alpha == nullptr: no Jastrow).
cudaError_t launch_psi_features(cudaStream_t s, int B, int n, int n_up, int A, int K0p, const float* x,
                                const float* atoms, const float* alpha, float* X0, float* rae, float* aevec,
                                float* jas);

}  // namespace qmc
