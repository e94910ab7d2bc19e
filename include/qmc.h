/*
 * qmc.h — C ABI of the GB300 (sm_103a) VMC inner loop: FermiNet and
 * Psiformer log|psi|, forward-Laplacian local energy and the all-electron
 * Metropolis-Hastings walker step, plus the walker-batch reductions and the
 * FermiNet parameter adjoint.
 *
 * Conventions
 *  - Every array argument is caller-owned DEVICE memory unless the name ends
 *    in `_host`.  Electrons are float32 (batch, n, 3), spin-up electrons first.
 *  - Calls are stream-ordered on the given cudaStream_t and never synchronise
 *    the device; results are valid once the stream reaches them.
 *  - Scratch memory is a caller-provided workspace whose size comes from
 *    qmc_workspace_size(); no entry point below allocates on the hot path.
 *  - A model handle is thread-compatible, not thread-safe: one host thread
 *    (or one serving slot) drives it at a time.
 *  - Every entry point returns a qmc_status; qmc_last_error() gives the text of
 *    the calling thread's last failure.  Kernels never trap: numerical trouble
 *    is reported per walker in a flag array (QMC_FLAG_*).
 */
#ifndef QMC_H_
#define QMC_H_

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int qmc_status;
enum {
  QMC_OK = 0,
  QMC_ERR_ARG = 1,         /* bad pointer / value                         */
  QMC_ERR_SHAPE = 2,       /* unsupported size (electrons, widths, batch) */
  QMC_ERR_NUMERIC = 3,     /* reserved: hard numerical failure            */
  QMC_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up          */
  QMC_ERR_CUDA = 5,        /* a CUDA runtime call failed                  */
  QMC_ERR_WORKSPACE = 6,   /* workspace smaller than qmc_workspace_size() */
  QMC_ERR_UNSUPPORTED = 7  /* feature not built / not on this device      */
};

/* per-walker flag bits written by qmc_forward / qmc_local_energy / qmc_mh_steps */
enum {
  QMC_FLAG_NONFINITE = 1,  /* log|psi| or E_L is NaN/Inf                      */
  QMC_FLAG_REFACTOR = 2,   /* a determinant was re-factorised in FP64          */
  QMC_FLAG_SINGULAR = 4    /* a determinant has an exactly zero pivot          */
};

enum { QMC_PRECISION_FP32 = 0, QMC_PRECISION_MIXED_BF16 = 1 };
/* Envelope types (src/jaqmc/wavefunction/output/envelope.py:16-35):
 * isotropic exp(-sigma r), abs_isotropic exp(-|sigma| r), diagonal
 * exp(-||sigma (.) (r - R)||) with a decay rate per dimension (sigma has shape
 * (n_orb, A, 3, K) per channel), null (no envelope and no envelope
 * parameters). */
enum { QMC_ENVELOPE_ISOTROPIC = 0, QMC_ENVELOPE_ABS_ISOTROPIC = 1, QMC_ENVELOPE_DIAGONAL = 2,
       QMC_ENVELOPE_NULL = 3 };
enum { QMC_OP_FORWARD = 0, QMC_OP_LOCAL_ENERGY = 1, QMC_OP_MH = 2, QMC_OP_GRAD = 3 };

#define QMC_MAX_LAYERS 8

/* Hyper-parameters of FermiNetWavefunction
 * (src/jaqmc/app/molecule/wavefunction/ferminet.py:44-50). */
typedef struct {
  int n_up, n_down;                     /* nspins                               */
  int n_atoms;
  int ndets;                            /* K                                    */
  int n_layers;                         /* len(hidden_dims_single)              */
  int hidden_single[QMC_MAX_LAYERS];
  int hidden_double[QMC_MAX_LAYERS];
  int envelope;                         /* QMC_ENVELOPE_*                       */
  int orbitals_spin_split;              /* 0/1                                  */
  int precision;                        /* QMC_PRECISION_*                      */
} qmc_ferminet_config;

/* Psiformer with the SimpleEE Jastrow (PsiformerWavefunction,
 * src/jaqmc/app/molecule/wavefunction/psiformer.py:38-94): Pre-LN layers,
 * biased attention projections and input layer, log-rescaled input features,
 * no orbital bias.  qmc_forward, qmc_mh_steps(_resident), qmc_mh_draws, the
 * forward-Laplacian qmc_local_energy (at most 42 electrons) and the FP32
 * parameter adjoint qmc_grad (at most 64 electrons, head width <= 64). */
typedef struct {
  int n_up, n_down, n_atoms;
  int ndets;                            /* K                                    */
  int n_layers;                         /* <= 8                                 */
  int n_heads, head_dim;                /* attention width n_heads*head_dim     */
  int n_mlp;                            /* hidden MLP widths per layer (<= 4)   */
  int mlp_dims[4];
  int envelope;                         /* QMC_ENVELOPE_*                       */
  int orbitals_spin_split;              /* 0/1                                  */
  int jastrow;                          /* 0 none, 1 SimpleEE                   */
  int precision;                        /* QMC_PRECISION_*                      */
} qmc_psiformer_config;

/* LapNet with the SimpleEE Jastrow (LapNetWavefunction,
 * src/jaqmc/app/molecule/wavefunction/lapnet.py:27-140; backbone
 * src/jaqmc/wavefunction/backbone/lapnet/_backbone.py:15-250): an individual
 * stream giving queries and keys and taking num_local_updates tanh updates
 * per layer (none in the last), a dense stream giving values and taking the
 * attention and value-update residuals, log-rescaled input features, spin-
 * split orbitals.  use_layernorm is not supported.  qmc_forward,
 * qmc_mh_steps(_resident), qmc_mh_draws, qmc_ecp_energy, the forward-
 * Laplacian qmc_local_energy (at most 42 electrons) and the FP32 parameter
 * adjoint qmc_grad (at most 64 electrons, head width <= 64). */
typedef struct {
  int n_up, n_down, n_atoms;
  int ndets;                            /* K                                    */
  int n_layers;                         /* num_layers, <= 8                     */
  int n_heads, head_dim;                /* num_heads, heads_dim                 */
  int num_local_updates;                /* <= 4                                 */
  int use_input_bias;                   /* 0/1                                  */
  int use_backbone_bias;                /* 0/1                                  */
  int envelope;                         /* QMC_ENVELOPE_*                       */
  int orbitals_spin_split;              /* 0/1                                  */
  int jastrow;                          /* 0 none, 1 SimpleEE                   */
  int precision;                        /* QMC_PRECISION_*                      */
} qmc_lapnet_config;

/* Model kinds: FermiNet, and the attention backbones (Psiformer, LapNet). */
enum { QMC_KIND_FERMINET = 0, QMC_KIND_PSIFORMER = 1 };

typedef struct qmc_model qmc_model;

/* Text of the calling thread's last error ("" if none). */
const char* qmc_last_error(void);

/* Library / device information; returns QMC_ERR_UNSUPPORTED when the current
 * device is not an sm_103 part. */
qmc_status qmc_device_check(int* sm_major, int* sm_minor, int* n_sms);

/* Create a FermiNet model on the current device.  atoms_host (A*3, bohr) and
 * charges_host (A) are host arrays.  Replaces the construction of
 * FermiNetWavefunction + its wiring (src/jaqmc/app/molecule/workflow.py:119-136). */
qmc_status qmc_ferminet_create(const qmc_ferminet_config* cfg, const float* atoms_host,
                               const float* charges_host, qmc_model** out);
/* Create a Psiformer model on the current device (see qmc_psiformer_config).
 * Replaces the construction of PsiformerWavefunction + its wiring
 * (src/jaqmc/app/molecule/workflow.py:119-136). */
qmc_status qmc_psiformer_create(const qmc_psiformer_config* cfg, const float* atoms_host,
                                const float* charges_host, qmc_model** out);
/* Create a LapNet model on the current device (see qmc_lapnet_config).
 * Replaces the construction of LapNetWavefunction + its wiring
 * (src/jaqmc/app/molecule/workflow.py:119-136).  The flat parameter vector
 * holds, in order: the input projection kernel (4A+1, D) [and bias], per
 * layer qk_projection (D, 2D) [bias], value_projection, output_projection,
 * value_update (D, D) [bias] and qk_update_layers_j (D, D) [bias] for
 * j < num_local_updates except in the last layer, then the orbitals,
 * envelope and Jastrow leaves as for the Psiformer. */
qmc_status qmc_lapnet_create(const qmc_lapnet_config* cfg, const float* atoms_host, const float* charges_host,
                             qmc_model** out);
qmc_status qmc_model_destroy(qmc_model* m);

/* Number of float32 entries of the flat parameter vector (leaf order:
 * per layer single kernel, bias, [two-electron kernel, bias]; orbital kernels
 * per spin channel; envelope pi, sigma per channel). */
size_t qmc_param_count(const qmc_model* m);

/* Load parameters from a flat float32 DEVICE vector (qmc_param_count entries)
 * into the model's device arena (reordered, padded and, for the mixed form,
 * converted to bf16).  Replaces the params pytree handed to
 * Wavefunction.evaluate (src/jaqmc/wavefunction/base.py:94-104). */
qmc_status qmc_model_set_params(qmc_model* m, const float* params, cudaStream_t stream);

/* Switch between QMC_PRECISION_FP32 and QMC_PRECISION_MIXED_BF16. */
qmc_status qmc_model_set_precision(qmc_model* m, int precision);

/* Determinant accuracy guard of qmc_local_energy: determinants whose FP32
 * kinetic term w_k (tr(A^-1 L) - sum_d tr((A^-1 J_d)^2) + sum_d tr(A^-1 J_d)^2)
 * loses too many digits to cancellation are evaluated again in FP64 (and the
 * walker flagged QMC_FLAG_REFACTOR).  mode 1 = on, 0 = off, -1 = the default:
 * on for QMC_PRECISION_FP32, off for QMC_PRECISION_MIXED_BF16.  No
 * counterpart in the reference (it evaluates slogdet's rule,
 * src/jaqmc/laplacian/primitives/slogdet.py:25-72, in the working precision). */
qmc_status qmc_model_set_det_guard(qmc_model* m, int mode);

/* Bytes of workspace needed by `op` (QMC_OP_*) for `batch` walkers.  For
 * QMC_OP_GRAD, and QMC_OP_LOCAL_ENERGY on a Psiformer model, the call runs in
 * chunks under the model's byte budget (qmc_model_set_grad_budget /
 * qmc_model_set_energy_budget) and this is one chunk's workspace.  0 for an
 * op the model does not support. */
size_t qmc_workspace_size(const qmc_model* m, int op, int batch);

/* log|psi| and sign for a batch: the vmapped FermiNetWavefunction.evaluate /
 * phase_logpsi (src/jaqmc/app/molecule/wavefunction/ferminet.py:76-122,
 * src/jaqmc/wavefunction/output/logdet.py:53-80).
 * logpsi, sign: (batch,) float32; flags: (batch,) uint8 or NULL. */
qmc_status qmc_forward(qmc_model* m, int batch, const float* electrons, float* logpsi,
                       float* sign, uint8_t* flags, void* workspace, size_t workspace_bytes,
                       cudaStream_t stream);

/* The same forward pass as qmc_forward, for callers that may not allocate
 * device memory while they run (for example code executing inside another
 * framework's step or a serving loop that reserves all memory up front).  The
 * intermediate buffers live in a 64 MiB device array inside this library;
 * batches whose forward pass needs more are rejected with QMC_ERR_WORKSPACE.
 * The array is shared by all calls on a device: calls whose GPU work overlaps
 * race, so serialise them.  The first call on a device resolves the array's
 * address; make it before any stream capture.  That address stays valid only
 * while the CUDA context that resolved it lives: after cudaDeviceReset do not
 * call this entry point again in the same process.  Both model families
 * (FermiNet and Psiformer) are served.  This entry point has no counterpart
 * in the reference. */
qmc_status qmc_forward_noalloc(qmc_model* m, int batch, const float* electrons, float* logpsi,
                               float* sign, uint8_t* flags, cudaStream_t stream);

/* Local energy E_L = KE + V per walker with the forward-Laplacian kinetic
 * energy KE = -1/2 (lap log|psi| + |grad log|psi||^2)
 * (src/jaqmc/estimator/kinetic/euclidean.py:114-135, _common.py:61-73) and the
 * Coulomb potential (src/jaqmc/app/molecule/hamiltonian.py:9-22).
 * Outputs (batch,) float32 each; any of ke / pe / logpsi / flags may be NULL. */
qmc_status qmc_local_energy(qmc_model* m, int batch, const float* electrons, float* e_local,
                            float* ke, float* pe, float* logpsi, uint8_t* flags,
                            void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* Rows per electron that `op` propagates: 1 for QMC_OP_FORWARD / QMC_OP_MH,
 * the 3n+2 forward-Laplacian tangents (padded to the tensor-core tile in the
 * mixed form) for QMC_OP_LOCAL_ENERGY; -1 for an invalid model or op.  No
 * counterpart in the reference (its tangents live inside the jaxpr
 * interpreter, src/jaqmc/laplacian/interpreter.py:392-438). */
int qmc_tangent_rows(const qmc_model* m, int op);

/* `steps` all-electron Gaussian MH updates (src/jaqmc/sampler/mcmc.py:96-199):
 * x' = x + stddev * N(0,1); accept iff 2 log|psi(x')| - 2 log|psi(x)| > log u.
 * Draws come from Philox4x32-10 keyed by `seed`, counter (step = counter + s,
 * walker, block), unless inj_normals (steps,batch,n,3) / inj_uniforms
 * (steps,batch) are given.  electrons is updated in place; log_prob (batch,)
 * receives 2 log|psi| of the final walkers; accepts (batch,) uint32 receives the
 * number of accepted moves per walker (added to its previous value). */
qmc_status qmc_mh_steps(qmc_model* m, int batch, int steps, float stddev, uint64_t seed,
                        uint64_t counter, float* electrons, float* log_prob, uint32_t* accepts,
                        const float* inj_normals, const float* inj_uniforms, uint8_t* flags,
                        void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* qmc_mh_steps with the Philox update counter resident in device memory:
 * update s of the call uses step = *counter + s, and *counter is advanced by
 * `steps` on the stream when the call's work is done.  Nothing on the host
 * depends on the counter, so a request (this call, qmc_local_energy and
 * qmc_reduce_mean_var on fixed buffers) can be captured once into a CUDA graph
 * and replayed: every replay continues the job's random stream.  No draw
 * injection.  Reference counterpart: the sampler state's PRNG key threaded
 * through MCMCSampler.step (src/jaqmc/sampler/mcmc.py:160-199). */
qmc_status qmc_mh_steps_resident(qmc_model* m, int batch, int steps, float stddev, uint64_t seed,
                                 uint64_t* counter, float* electrons, float* log_prob, uint32_t* accepts,
                                 uint8_t* flags, void* workspace, size_t workspace_bytes,
                                 cudaStream_t stream);

/* Several jobs of one model in one MH batch: their walkers concatenated in
 * `electrons` (batch = offsets[n_jobs] walkers; offsets, seeds and counters
 * are device arrays of n_jobs + 1, n_jobs and n_jobs entries).  Job j's
 * walkers [offsets[j], offsets[j + 1]) take exactly the proposals and
 * acceptances of qmc_mh_steps_resident on that job alone with seed seeds[j]
 * and counter counters[j]; every counter advances by `steps`.  This is the
 * grouped launch of the serving loop, which packs queued requests of jobs
 * that share a model into one launch set.  Each walker's log|psi| depends
 * only on its own electrons, so the batch's composition does not change any
 * job's results.  No counterpart in the reference (one process runs one
 * job there). */
qmc_status qmc_mh_steps_grouped(qmc_model* m, int n_jobs, const int* offsets, const uint64_t* seeds,
                                uint64_t* counters, int batch, int steps, float stddev, float* electrons,
                                float* log_prob, uint32_t* accepts, uint8_t* flags, void* workspace,
                                size_t workspace_bytes, cudaStream_t stream);

/* The draws qmc_mh_steps would use for (seed, counter, steps): normals
 * (steps,batch,n,3) and uniforms (steps,batch), either may be NULL. */
qmc_status qmc_mh_draws(const qmc_model* m, int batch, int steps, uint64_t seed,
                        uint64_t counter, float* normals, float* uniforms, cudaStream_t stream);

/* Parameter adjoint of log|psi| (FP32), replacing the per-walker
 * jax.value_and_grad of LossAndGrad (src/jaqmc/estimator/loss_grad.py:70-91)
 * and its gradient algebra (:113-128):
 *   per_walker (batch x qmc_param_count, may be NULL): row w = d log|psi_w| / d theta
 *     in the flat parameter layout of qmc_model_set_params;
 *   grad (qmc_param_count doubles, may be NULL): sum_w weights[w] * d log|psi_w| / d theta,
 *     e.g. weights = 2 (E_c,w - <E_c>) / batch for the VMC energy gradient;
 *   logpsi (batch, may be NULL).
 * Walkers are processed in chunks sized by the gradient budget; every chunk
 * recomputes its forward activations.  Workspace: qmc_workspace_size(m, QMC_OP_GRAD, batch).
 * FermiNet, Psiformer and LapNet models (for a Psiformer: the backward of
 * the input Dense, LayerNorms, attention, tanh MLP, orbitals, envelope and
 * Jastrow, src/jaqmc/app/molecule/wavefunction/psiformer.py:38-146; for
 * LapNet: of both streams, the local updates, attention, value updates,
 * orbitals, envelope and Jastrow, .../wavefunction/lapnet.py:27-140). */
qmc_status qmc_grad(qmc_model* m, int batch, const float* electrons, const double* weights, float* per_walker,
                    double* grad, float* logpsi, void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* Byte budget of the adjoint's workspace (default 8 GiB); sets the chunk size. */
qmc_status qmc_model_set_grad_budget(qmc_model* m, size_t bytes);

/* Layer taps of the parameter adjoint, the statistics a Kronecker-factored
 * curvature (KFAC) needs: for every dense layer the inputs x and the output
 * cotangents dy = d log|psi_w| / d(layer output) of each of its applications,
 * and for the remaining parameters (the envelope's) the per-walker gradients.
 * Replaces the layer-tag registration and the curvature statistics that
 * kfac_jax collects from the jaxpr of vmap(log|psi|)
 * (src/jaqmc/optimizer/kfac/kfac.py:162-186,
 *  src/jaqmc/optimizer/kfac/curvature_blocks.py:94-137,
 *  src/jaqmc/optimizer/kfac/tag_registration.py:22-259).
 * FermiNet tap order: per layer l the one-electron Dense (input [h1 | spin means of h1
 * | spin means of h2], n applications per walker, bias) then, when layer l
 * updates the two-electron stream, the two-electron Dense (n^2 applications,
 * bias); the orbital projection of each spin channel (n_s applications, no
 * bias); last the envelope parameters as one diagonal tap (rows_per_walker 1,
 * in_cols 0, out_cols = their count).
 * Psiformer tap order: the input Dense (n applications, bias); per layer the
 * first LayerNorm (diagonal: scale then shift, 2 D), the q, k, v and output
 * projections (n applications each, bias), the second LayerNorm (diagonal)
 * and the MLP Dense layers (n applications, bias); the orbital projection
 * of each spin channel; the envelope and Jastrow parameters as one diagonal
 * tap.  LapNet: the input Dense (bias when use_input_bias); per layer the
 * fused query/key projection [D][2D], the value, attention-output and
 * update projections and each local update (n applications, bias when
 * use_backbone_bias); then orbitals and the diagonal tail as above.
 * A tap's inputs are a row-major
 * [batch * rows_per_walker][in_cols] block at float offset in_offset of the
 * taps buffer and its cotangents (or per-walker gradients) a
 * [batch * rows_per_walker][out_cols] block at out_offset; walker w's rows are
 * w * rows_per_walker ... (w + 1) * rows_per_walker - 1. */
enum { QMC_TAP_DENSE = 0, QMC_TAP_DIAGONAL = 1 };
typedef struct {
  int kind;              /* QMC_TAP_*                                          */
  int rows_per_walker;   /* applications per walker                            */
  int in_cols, out_cols; /* input width (no bias column) and output width       */
  int has_bias;
  size_t kernel_offset;  /* flat parameter offset of the kernel [in_cols][out] (or of the diagonal block) */
  size_t bias_offset;    /* flat parameter offset of the bias (has_bias)        */
  size_t in_offset, out_offset;  /* float offsets in the taps buffer            */
} qmc_layer_tap;
/* Fills up to max_taps descriptors for `batch` walkers; returns the number of
 * taps (or -1 for a model without taps) and the taps buffer size in floats. */
int qmc_layer_taps(const qmc_model* m, int batch, qmc_layer_tap* taps, int max_taps, size_t* total_floats);
/* Runs the adjoint (forward with saved activations + backward, chunked under
 * the gradient budget; workspace = qmc_workspace_size(QMC_OP_GRAD)) and writes
 * the taps of every walker into `taps` (total_floats floats); logpsi
 * (batch,) may be NULL. */
qmc_status qmc_grad_taps(qmc_model* m, int batch, const float* electrons, float* taps, size_t taps_floats,
                         float* logpsi, void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* Byte budget of the Psiformer local-energy workspace (default 32 GiB): walkers
 * run in balanced chunks whose forward-Laplacian activations fit it.  FermiNet
 * models ignore it. */
qmc_status qmc_model_set_energy_budget(qmc_model* m, size_t bytes);

/* FP64 walker-batch mean and variance <x^2> - <x>^2 of a float32 vector,
 * NaNs skipped (src/jaqmc/estimator/base.py:27-53).  mean_var: 2 doubles. */
qmc_status qmc_reduce_mean_var(int batch, const float* x, double* mean_var, cudaStream_t stream);
/* The same per segment [offsets[s], offsets[s + 1]) of x (device offsets,
 * n_segments + 1 entries) into mean_var[2 s], mean_var[2 s + 1]: each
 * segment's result is bitwise that of qmc_reduce_mean_var on the segment
 * alone (the per-job statistics of a grouped request). */
qmc_status qmc_reduce_mean_var_segments(int n_segments, const int* offsets, const float* x, double* mean_var,
                                        cudaStream_t stream);

/* Effective-core-potential energy per walker: the reference's ECPEnergy
 * estimator (src/jaqmc/estimator/ecp/estimator.py:33-155, nonlocal integral
 * src/jaqmc/estimator/ecp/nonlocal_integral.py:17-130).  e_local (batch,) =
 * sum_{i,I} V_0(r_iI); e_nonlocal (batch,) = sum_i sum over the max_core
 * nearest ECP atoms of sum_l V_{l+1}(r) (2l+1) sum_q w_q P_l(cos theta_q)
 * psi(r_i -> R + r Rot_i x_q) / psi, each displaced configuration one forward
 * pass of the model (run in chunks inside the workspace).  Device tables:
 * ecp_atoms [n_ecp_atoms] indices into the model's atoms; radial
 * [n_ecp_atoms][n_channels][max_terms][3] = (alpha, coeff, power) with
 * V_c(r) = sum_t coeff r^power exp(-alpha r^2), channel 0 local and channel
 * l + 1 the semi-local l (zero coefficients pad); quad [n_quad][4] = (x, y,
 * z, weight), weights summing to 1; rotations [batch][n][9] row-major or NULL
 * (then drawn from Philox4x32-10 with seed / counter: phi = 2 pi u1,
 * cos theta = 1 - 2 u2 per walker and electron).  n_channels <= 5, max_core
 * <= 8, n_quad <= 256. */
size_t qmc_ecp_workspace_size(const qmc_model* m, int batch, int n_channels, int max_core, int n_quad);
qmc_status qmc_ecp_energy(qmc_model* m, int batch, const float* electrons, int n_ecp_atoms, const int* ecp_atoms,
                          int n_channels, int max_terms, const float* radial, int max_core, int n_quad,
                          const float* quad, const float* rotations, uint64_t seed, uint64_t counter,
                          float* e_local, float* e_nonlocal, void* workspace, size_t workspace_bytes,
                          cudaStream_t stream);

/* Reads and clears the model's device error word (synchronises the device).
 * Returns QMC_ERR_TIMEOUT with *code != 0 when a bounded wait inside a
 * tensor-core kernel expired since the last check. */
qmc_status qmc_model_check_error(qmc_model* m, int* code);

/* Built-in launch profiler.  While enabled, every kernel the library launches
 * is counted per class and bracketed by CUDA events on its stream (stream
 * capture must not be active).  qmc_profile_read synchronises on the recorded
 * events and returns, per class, the number of launches and their summed
 * device time in ms, then clears the record.  Classes: QMC_KC_*. */
enum {
  QMC_KC_STREAM_LAYER = 0, /* one-electron layers >= 1: GEMM + tangent epilogue */
  QMC_KC_BROADCAST = 1,    /* spin-mean broadcast GEMM                    */
  QMC_KC_ORBITAL = 2,      /* orbital GEMM x envelope                     */
  QMC_KC_LOGDET = 3,       /* LU / log-sum-exp / slogdet traces           */
  QMC_KC_FEATURES = 4,     /* input features + potential                  */
  QMC_KC_MEANS = 5,        /* spin means of both streams                  */
  QMC_KC_PAIR = 6,         /* two-electron layers                         */
  QMC_KC_MH = 7,           /* proposal / accept                           */
  QMC_KC_OTHER = 8,
  QMC_KC_LAYER0 = 9,       /* first one-electron layer (4A-wide input)    */
  QMC_KC_COUNT = 10
};
qmc_status qmc_profile_enable(int on);
qmc_status qmc_profile_read(int n_classes, int64_t* launches, double* ms);

/* FP32 FMA throughput probe: one launch of `blocks` blocks of 256 threads,
 * each thread running 8 independent chains of 16 x iters FMAs; `out` receives
 * blocks x 256 floats (a sink).  *fma_per_launch = the FMAs issued.  Timed
 * with CUDA events by the caller, it measures the FP32 SIMT peak that the
 * plain-form rooflines divide by.  No counterpart in the reference. */
qmc_status qmc_ffma_throughput(int blocks, int iters, float* out, double* fma_per_launch,
                               cudaStream_t stream);

/* Warp-level BF16 MMA throughput probe (mma.m16n8k16, FP32 accumulate, the
 * legacy warp tensor path that the mixed form's forward-Laplacian attention
 * uses): `blocks` blocks of 256 threads, `iters` rounds of 8 independent
 * MMAs per warp into blocks x 256 floats (a sink); *flop_per_launch = the
 * FLOPs issued.  Timed with CUDA events by the caller, it is the roofline
 * denominator of that kernel.  No counterpart in the reference. */
qmc_status qmc_mma_throughput(int blocks, int iters, float* out, double* flop_per_launch,
                              cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* QMC_H_ */
