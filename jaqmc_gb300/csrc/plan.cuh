// Workspace plan and evaluation driver shared by the C-ABI entry points.
#pragma once
#include "common.cuh"

namespace qmc {

// Byte offsets of every scratch buffer of one call inside the workspace.
struct Plan {
  int B, T, Tp, P2, K0p;
  bool mixed;
  size_t x0, h1[2], h2[2], g1, gb, g2, rae, aevec, amat, pe, lpsi, sgn, xp, lp, refac, total;
  size_t redo;  // determinant-stage scratch of tangent passes (logdet_fl_scratch_bytes)
  size_t x0s, g2s0;  // mixed form: the first layer's features / pair means as bf16 planes
  size_t act_bytes;  // bytes per one-electron activation (fp32, or two bf16 planes)
  size_t h1_plane, g1_plane, g2_plane;  // bf16 elements between split planes
  int dmax, g1max, g2max;
};


Plan make_plan(const qmc_model* m, int op, int B);

// sum_{I<J} Z_I Z_J / |R_I - R_J| in FP64
double nuclear_repulsion(const float* atoms, const float* charges, int A);

// Validates a call: parameters set, batch >= 1, workspace large enough,
// supported shapes, model on the current device.
qmc_status check_call(qmc_model* m, int batch, const void* ws, size_t ws_bytes, int op);

// features -> backbone -> orbitals -> determinants for p.B walkers using the
// scratch buffers of plan p inside ws.
qmc_status evaluate(qmc_model* m, const Plan& p, void* ws, const float* electrons, bool want_pe,
                    float* logpsi, float* sign, float* ke, float* el, uint8_t* flags, cudaStream_t s);

// The orbital (x envelope) stage reading the backbone output in h1[hb], and the
// determinant stage; shared by the FermiNet and Psiformer drivers.
qmc_status run_orbitals(qmc_model* m, const Plan& p, void* ws, int hb, cudaStream_t s);
qmc_status run_logdet(qmc_model* m, const Plan& p, void* ws, const float* pe, float* logpsi, float* sign,
                      float* ke, float* el, uint8_t* flags, cudaStream_t s);

// Adjoint (adjoint.cu): workspace bytes for `batch` walkers under the model's
// gradient budget, and the chunked forward + backward driver.
size_t grad_workspace(const qmc_model* m, int batch);
qmc_status run_grad(qmc_model* m, int batch, const float* electrons, const double* weights, float* per_walker,
                    double* grad, float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s);
// Psiformer adjoint: workspace under the gradient budget and the chunked driver.
size_t psi_grad_workspace(const qmc_model* m, int batch);
qmc_status run_psi_grad(qmc_model* m, int batch, const float* electrons, const double* weights, float* per_walker,
                        double* grad, float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s);
// Layer taps of the adjoint (KFAC statistics): descriptors and the chunked run.
int attn_layer_taps(const qmc_model* m, int batch, qmc_layer_tap* taps, int max_taps, size_t* total);
qmc_status run_attn_grad_taps(qmc_model* m, int batch, const float* electrons, float* taps, size_t taps_floats,
                              float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s);
int layer_taps(const qmc_model* m, int batch, qmc_layer_tap* taps, int max_taps, size_t* total);
qmc_status run_grad_taps(qmc_model* m, int batch, const float* electrons, float* taps, size_t taps_floats,
                         float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s);

}  // namespace qmc
