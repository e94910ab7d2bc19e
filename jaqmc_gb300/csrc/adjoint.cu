// Hand-written adjoint of log|psi| with respect to the FermiNet parameters
// (FP32).  Replaces the per-walker jax.value_and_grad of LossAndGrad
// (src/jaqmc/estimator/loss_grad.py:70-91) and the VMC gradient algebra
// (:113-128): per-walker Jacobian rows d log|psi_w| / d theta in the flat
// parameter layout of qmc_model_set_params, and sum_w c_w d log|psi_w|/d theta.
//
// Walkers are processed in chunks sized to a byte budget; each chunk re-runs
// the forward pass keeping every layer's activations, then runs the backward
// pass (recomputation instead of storing activations for the whole batch).
#include <algorithm>

#include "gemm_simt.cuh"
#include "kernels.cuh"
#include "plan.cuh"
#include "profile.cuh"
#include "psiformer.cuh"

namespace qmc {

template <typename T>
static T* at(void* ws, size_t off) { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }

// ------------------------------------------------------------ kernels
// y = tanh(z) saved next to the layer output (value-only one-electron layer)
struct EpiLayerSave {
  const float* Gb;
  const float* bias;
  const float* resid;  // nullptr: no residual
  float* out;
  float* y;
  int ld;
  __device__ void operator()(const float* Cs, int ng, int g0, int n0, int N, const RowMap& m) const {
    for (int p = threadIdx.x; p < ng * kBN; p += blockDim.x) {
      int lg = p / kBN, c = p % kBN, col = n0 + c;
      if (col >= N) continue;
      int g = g0 + lg;
      size_t r = m.row(g, 0);
      float h = tanhf(Cs[lg * kCsLd + c] + Gb[(size_t)m.w(g) * N + col] + bias[col]);
      y[r * ld + col] = h;
      out[r * ld + col] = resid ? (h + resid[r * ld + col]) * kRsqrt2 : h;
    }
  }
};

// two-electron layer with saved tanh outputs
__global__ void k_pair_fwd_save(int npairs, int d_in, int d_out, const float* __restrict__ Hin,
                                const float* __restrict__ W, const float* __restrict__ b, float* __restrict__ Hout,
                                float* __restrict__ Y) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)npairs * d_out) return;
  const int f = (int)(e % d_out);
  const size_t pr = e / d_out;
  const float* x = Hin + pr * d_in;
  float z = b[f];
  for (int k = 0; k < d_in; ++k) z = fmaf(x[k], W[k * d_out + f], z);
  const float y = tanhf(z);
  Y[e] = y;
  Hout[e] = d_in == d_out ? (y + x[f]) * kRsqrt2 : y;
}

// orbital / envelope cotangents from Abar (value-only pass)
// Envelope value of column (k, j) at electron (w, i) for every envelope kind
// (src/jaqmc/wavefunction/output/envelope.py:123-163); 1 for the null envelope.
__device__ float env_value(int kind, int env_abs, int natom, int K, int k, int j, size_t wi, const float* pi,
                           const float* sg, const float* rae, const float* aevec) {
  if (kind == QMC_ENVELOPE_NULL) return 1.f;
  float env = 0.f;
  for (int I = 0; I < natom; ++I) {
    const size_t q = (size_t)j * natom + I;
    if (kind == QMC_ENVELOPE_DIAGONAL) {
      float s2 = 0.f;
      for (int c = 0; c < 3; ++c) {
        const float t = sg[(q * 3 + c) * K + k] * aevec[(wi * natom + I) * 3 + c];
        s2 = fmaf(t, t, s2);
      }
      env += pi[q * K + k] * expf(-sqrtf(s2));
    } else {
      const float sv = sg[q * K + k];
      const float se = env_abs ? fabsf(sv) : sv;
      env += pi[q * K + k] * expf(-se * rae[wi * natom + I]);
    }
  }
  return env;
}

__global__ void k_orb_bwd(int B, int n, int n_up, int split, int K, int natom, int env_abs, int env_kind, int norb_p,
                          const float* __restrict__ Abar, const float* __restrict__ orb,
                          const float* __restrict__ rae, const float* __restrict__ aevec, const float* __restrict__ pi0,
                          const float* __restrict__ sg0, const float* __restrict__ pi1,
                          const float* __restrict__ sg1, float* __restrict__ orbbar, float* __restrict__ envbar) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)B * n * norb_p) return;
  const int col = (int)(e % norb_p);
  const size_t wi = e / norb_p;
  const int i = (int)(wi % n), w = (int)(wi / n);
  if (col >= K * n) {
    orbbar[e] = 0.f;
    return;
  }
  const int k = col / n, j = col % n;
  const bool c1 = split && i >= n_up;
  const float* pi = c1 ? pi1 : pi0;
  const float* sg = c1 ? sg1 : sg0;
  const float env = env_value(env_kind, env_abs, natom, K, k, j, wi, pi, sg, rae, aevec);
  const size_t ai = (((size_t)w * K + k) * n + i) * n + j;
  const float ab = Abar[ai];
  orbbar[e] = ab * env;
  envbar[ai] = ab * orb[ai];
}

// envelope parameter rows of the Jacobian: d/dpi, d/dsigma for channel c
__global__ void k_env_jac(int B, int n, int i0, int ns, int K, int natom, int env_abs, const float* __restrict__ envbar,
                          const float* __restrict__ rae, const float* __restrict__ pi, const float* __restrict__ sg,
                          float* __restrict__ J, size_t P, size_t off_pi, size_t off_sg) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per_w = (size_t)n * natom * K;
  if (e >= (size_t)B * per_w) return;
  const int w = (int)(e / per_w);
  const size_t q = e % per_w;  // (j, I, k) in the reference layout
  const int k = (int)(q % K), I = (int)((q / K) % natom), j = (int)(q / ((size_t)K * natom));
  const float pv = pi[q], sv = sg[q];
  const float se = env_abs ? fabsf(sv) : sv;
  const float dse = env_abs ? (sv > 0.f ? 1.f : (sv < 0.f ? -1.f : 0.f)) : 1.f;
  float dpi = 0.f, dsg = 0.f;
  for (int i = i0; i < i0 + ns; ++i) {
    const float r = rae[((size_t)w * n + i) * natom + I];
    const float ex = expf(-se * r);
    const float eb = envbar[(((size_t)w * K + k) * n + i) * n + j];
    dpi = fmaf(eb, ex, dpi);
    dsg = fmaf(eb, -pv * ex * r * dse, dsg);
  }
  J[(size_t)w * P + off_pi + q] = dpi;
  J[(size_t)w * P + off_sg + q] = dsg;
}

// Diagonal envelope parameter rows: d/dpi[j,I,k] = sum_i Ebar e^{-s},
// d/dsigma[j,I,c,k] = sum_i Ebar (-pi e^{-s} sigma_c v_c^2 / s), v = r_i - R_I,
// s = ||sigma (.) v|| (src/jaqmc/wavefunction/output/envelope.py:143-163).
__global__ void k_env_jac_diag(int B, int n, int i0, int ns, int K, int natom, const float* __restrict__ envbar,
                               const float* __restrict__ aevec, const float* __restrict__ pi,
                               const float* __restrict__ sg, float* __restrict__ J, size_t P, size_t off_pi,
                               size_t off_sg) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per_w = (size_t)n * natom * K;
  if (e >= (size_t)B * per_w) return;
  const int w = (int)(e / per_w);
  const size_t q = e % per_w;  // (j, I, k)
  const int k = (int)(q % K), I = (int)((q / K) % natom), j = (int)(q / ((size_t)K * natom));
  const size_t jI = (size_t)j * natom + I;
  const float pv = pi[q];
  float sc[3];
  for (int c = 0; c < 3; ++c) sc[c] = sg[(jI * 3 + c) * K + k];
  float dpi = 0.f, ds[3] = {0.f, 0.f, 0.f};
  for (int i = i0; i < i0 + ns; ++i) {
    const float* v = aevec + (((size_t)w * n + i) * natom + I) * 3;
    float s2 = 0.f;
    for (int c = 0; c < 3; ++c) s2 = fmaf(sc[c] * v[c], sc[c] * v[c], s2);
    const float s = sqrtf(s2);
    const float ex = expf(-s);
    const float eb = envbar[(((size_t)w * K + k) * n + i) * n + j];
    dpi = fmaf(eb, ex, dpi);
    const float f = s > 0.f ? -eb * pv * ex / s : 0.f;
    for (int c = 0; c < 3; ++c) ds[c] = fmaf(f * sc[c] * v[c], v[c], ds[c]);
  }
  J[(size_t)w * P + off_pi + q] = dpi;
  for (int c = 0; c < 3; ++c) J[(size_t)w * P + off_sg + (jI * 3 + c) * K + k] = ds[c];
}

// Jacobian block of a dense layer: J[w][off + kx*N + c] =
//   sum_{r<R} X[w*Rs + row0 + r][kx] * Z[w*Rs + row0 + r][c]
__global__ void k_jac_outer(int B, int R, int Rs, int row0, const float* __restrict__ X, int ldx, int Kx,
                            const float* __restrict__ Z, int ldz, int N, float* __restrict__ J, size_t P,
                            size_t off) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t per_w = (size_t)Kx * N;
  if (e >= (size_t)B * per_w) return;
  const int w = (int)(e / per_w);
  const int kx = (int)((e % per_w) / N), c = (int)(e % N);
  const size_t base = (size_t)w * Rs + row0;
  float acc = 0.f;
  for (int r = 0; r < R; ++r) acc = fmaf(X[(base + r) * ldx + kx], Z[(base + r) * ldz + c], acc);
  J[(size_t)w * P + off + (size_t)kx * N + c] = acc;
}

// The same Jacobian block with the walker's rows staged in shared memory:
// one block per (walker, 32 columns of X); Z [R][N] and X [R][32] are read
// from global memory once per block, and a thread forms 4 consecutive kx of
// one output column c per pass (consecutive threads take consecutive c, so the
// X float4 reads are broadcasts and the J stores are coalesced).
constexpr int kJacKT = 32;
__global__ void __launch_bounds__(256) k_jac_outer_tiled(int R, int Rs, int row0, const float* __restrict__ X, int ldx,
                                                         int Kx, const float* __restrict__ Z, int ldz, int N,
                                                         float* __restrict__ J, size_t P, size_t off) {
  extern __shared__ __align__(16) float sj[];
  const int w = blockIdx.x, kx0 = blockIdx.y * kJacKT;
  const int kt = min(kJacKT, Kx - kx0);
  float* Xs = sj;                   // [R][kJacKT]
  float* Zs = sj + R * kJacKT;      // [R][N]
  const size_t base = (size_t)w * Rs + row0;
  for (int e = threadIdx.x; e < R * N; e += blockDim.x) {
    const int r = e / N, c = e - r * N;
    Zs[e] = Z[(base + r) * ldz + c];
  }
  for (int e = threadIdx.x; e < R * kJacKT; e += blockDim.x) {
    const int r = e / kJacKT, k = e - r * kJacKT;
    Xs[e] = k < kt ? X[(base + r) * ldx + kx0 + k] : 0.f;
  }
  __syncthreads();
  float* Jw = J + (size_t)w * P + off;
  const int pairs = (kJacKT / 4) * N;
  for (int p = threadIdx.x; p < pairs; p += blockDim.x) {
    const int kq = p / N, c = p - kq * N;
    if (4 * kq >= kt) continue;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    for (int r = 0; r < R; ++r) {
      const float z = Zs[r * N + c];
      const float4 x = *reinterpret_cast<const float4*>(Xs + r * kJacKT + 4 * kq);
      a0 = fmaf(x.x, z, a0);
      a1 = fmaf(x.y, z, a1);
      a2 = fmaf(x.z, z, a2);
      a3 = fmaf(x.w, z, a3);
    }
    const int k = kx0 + 4 * kq;
    Jw[(size_t)k * N + c] = a0;
    if (4 * kq + 1 < kt) Jw[(size_t)(k + 1) * N + c] = a1;
    if (4 * kq + 2 < kt) Jw[(size_t)(k + 2) * N + c] = a2;
    if (4 * kq + 3 < kt) Jw[(size_t)(k + 3) * N + c] = a3;
  }
}

// J[w][off + kx N + c] = sum_r X[..][kx] Z[..][c]: the staged kernel when a
// walker's rows fit in shared memory, else the plain one.
static cudaError_t jac_outer(cudaStream_t s, int B, int R, int Rs, int row0, const float* X, int ldx, int Kx,
                             const float* Z, int ldz, int N, float* J, size_t P, size_t off) {
  const size_t sm = sizeof(float) * (size_t)R * (kJacKT + N);
  if (sm <= 160 * 1024) {
    int dev;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    static int set_dev = -1;
    if (set_dev != dev) {
      e = cudaFuncSetAttribute(k_jac_outer_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
      if (e != cudaSuccess) return e;
      set_dev = dev;
    }
    k_jac_outer_tiled<<<dim3((unsigned)B, (unsigned)((Kx + kJacKT - 1) / kJacKT)), 256, sm, s>>>(
        R, Rs, row0, X, ldx, Kx, Z, ldz, N, J, P, off);
    return cudaGetLastError();
  }
  const size_t total = (size_t)B * Kx * N;
  k_jac_outer<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(B, R, Rs, row0, X, ldx, Kx, Z, ldz, N, J, P, off);
  return cudaGetLastError();
}

// per-walker column sums Zs[w][c] = sum_{r<R} Z[w*R + r][c]; optionally also
// written as Jacobian rows (bias gradients)
__global__ void k_colsum(int B, int R, const float* __restrict__ Z, int ldz, int N, float* __restrict__ Zs,
                         float* __restrict__ J, size_t P, size_t off) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)B * N) return;
  const int w = (int)(e / N), c = (int)(e % N);
  float acc = 0.f;
  for (int r = 0; r < R; ++r) acc += Z[((size_t)w * R + r) * ldz + c];
  if (Zs) Zs[e] = acc;
  if (J) J[(size_t)w * P + off + c] = acc;
}

// z = hbar * s * (1 - y^2), hres = hbar * s (residual path)
__global__ void k_tanh_bwd(size_t count, float s, const float* __restrict__ hbar, const float* __restrict__ y,
                           float* __restrict__ zbar) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= count) return;
  const float v = y[e];
  zbar[e] = hbar[e] * s * (1.f - v * v);
}

// hbar_in[w,i,f] = T[w,i,f] + res * hbar_out[w,i,f] / sqrt(2) + g1bar[w][s(i)*din + f] / n_s
__global__ void k_input_grad(int B, int n, int n_up, int C, int din, const float* __restrict__ Tm, int ldt,
                             const float* __restrict__ hbar_out, int residual, const float* __restrict__ g1bar,
                             int g1p, float* __restrict__ hbar_in) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)B * n * din) return;
  const int f = (int)(e % din);
  const size_t wi = e / din;
  const int i = (int)(wi % n), w = (int)(wi / n);
  const int sc = (C == 2 && i >= n_up) ? 1 : 0;
  const int ns = C == 1 ? n : (sc == 0 ? n_up : n - n_up);
  float v = Tm[wi * ldt + f] + g1bar[(size_t)w * g1p + sc * din + f] / (float)ns;
  if (residual) v += hbar_out[wi * din + f] * kRsqrt2;
  hbar_in[e] = v;
}

// h2bar[w,a,i,f] (+)= g2bar[w,i][s(a)*d2 + f] / n_{s(a)}  (G2 averages over the first index)
__global__ void k_h2_from_g2(int B, int n, int n_up, int C, int d2, const float* __restrict__ Tm, int ldt,
                             int col0, float* __restrict__ h2bar, int accumulate) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)B * n * n * d2) return;
  const int f = (int)(e % d2);
  const size_t pr = e / d2;
  const int i = (int)(pr % n), a = (int)((pr / n) % n), w = (int)(pr / ((size_t)n * n));
  const int sc = (C == 2 && a >= n_up) ? 1 : 0;
  const int ns = C == 1 ? n : (sc == 0 ? n_up : n - n_up);
  const float v = Tm[((size_t)w * n + i) * ldt + col0 + sc * d2 + f] / (float)ns;
  h2bar[e] = accumulate ? h2bar[e] + v : v;
}

// two-electron layer backward data path: h2bar_in = z2bar W2^T (+ residual)
__global__ void k_pair_bwd_data(size_t npairs, int d_in, int d_out, const float* __restrict__ z2bar,
                                const float* __restrict__ Wt, const float* __restrict__ h2bar_out,
                                float* __restrict__ h2bar_in) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= npairs * d_in) return;
  const int k = (int)(e % d_in);
  const size_t pr = e / d_in;
  float acc = 0.f;
  for (int f = 0; f < d_out; ++f) acc = fmaf(z2bar[pr * d_out + f], Wt[(size_t)f * d_in + k], acc);
  if (d_in == d_out) acc += h2bar_out[pr * d_out + k] * kRsqrt2;
  h2bar_in[e] = acc;
}

// grad[p] += sum_w c_w J[w][p]  (FP64 accumulation)
__global__ void k_weighted_sum(int B, size_t P, const float* __restrict__ J, const double* __restrict__ c,
                               double* __restrict__ grad) {
  size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  double acc = 0.0;
  for (int w = 0; w < B; ++w) acc += c[w] * (double)J[(size_t)w * P + p];
  grad[p] += acc;
}

static inline unsigned blocks(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------------------ layer taps
// Input rows of one-electron layer l for a chunk: [h1 (din) | spin means of
// h1 (C din, the walker's) | spin means of h2 (C d2in, the row's)], the order
// of the reference's Dense kernel rows (backbone/ferminet.py:82-90).
__global__ void k_tap_x1(int B, int n, int din, int dinp, int c_din, int g1p, int c_d2, int g2p,
                         const float* __restrict__ in, const float* __restrict__ g1m, const float* __restrict__ G2,
                         float* __restrict__ dst) {
  const int cols = din + c_din + c_d2;
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)B * n * cols) return;
  const int c = (int)(e % cols);
  const size_t r = e / cols;
  float v;
  if (c < din) v = in[r * dinp + c];
  else if (c < din + c_din) v = g1m[(r / n) * g1p + (c - din)];
  else v = G2[r * g2p + (c - din - c_din)];
  dst[e] = v;
}

// dst[(w ns + ii) cols + c] = scale * src[(w n + i0 + ii) ld + c]
__global__ void k_tap_gather(int B, int n, int i0, int ns, const float* __restrict__ src, int ld, int cols,
                             float* __restrict__ dst) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)B * ns * cols) return;
  const int c = (int)(e % cols);
  const size_t r = e / cols;
  const size_t w = r / ns;
  const int ii = (int)(r % ns);
  dst[e] = src[(w * n + i0 + ii) * (size_t)ld + c];
}

constexpr int kMaxTaps = 128;
struct TapPlan {
  int count = 0;
  qmc_layer_tap t[kMaxTaps];
  size_t total = 0;
};

static TapPlan make_taps(const qmc_model* m, int B) {
  const Dims& d = m->d;
  const ParamLayout& pl = m->p;
  TapPlan tp;
  size_t o = 0;
  auto add = [&](int kind, int rpw, int in_cols, int out_cols, int bias, size_t k_off, size_t b_off) {
    qmc_layer_tap& t = tp.t[tp.count++];
    t.kind = kind;
    t.rows_per_walker = rpw;
    t.in_cols = in_cols;
    t.out_cols = out_cols;
    t.has_bias = bias;
    t.kernel_offset = k_off;
    t.bias_offset = b_off;
    t.in_offset = o;
    o += (size_t)B * rpw * in_cols;
    t.out_offset = o;
    o += (size_t)B * rpw * out_cols;
  };
  for (int l = 0; l < d.L; ++l) {
    add(QMC_TAP_DENSE, d.n, d.d1_in[l] + d.C * d.d1_in[l] + d.C * d.d2_in[l], d.d1[l], 1, pl.dense1_k[l],
        pl.dense1_b[l]);
    if (d.upd2[l]) add(QMC_TAP_DENSE, d.n * d.n, d.d2_in[l], d.d2[l], 1, pl.dense2_k[l], pl.dense2_b[l]);
  }
  const int nch = d.split ? 2 : 1;
  for (int c = 0; c < nch; ++c) {
    const int ns = d.split ? (c == 0 ? d.n_up : d.n_dn) : d.n;
    add(QMC_TAP_DENSE, ns, d.d_last, d.norb, 0, pl.orb_k[c], 0);
  }
  const size_t env0 = pl.env_pi[0];
  if (pl.total > env0) add(QMC_TAP_DIAGONAL, 1, 0, (int)(pl.total - env0), 0, env0, 0);
  tp.total = o;
  return tp;
}

// Where backward() writes the taps of a chunk: the call's plan and the
// chunk's first walker.
struct TapOut {
  float* base = nullptr;
  const TapPlan* plan = nullptr;
  int w0 = 0;
  float* in(int k) const { return base + plan->t[k].in_offset + (size_t)w0 * plan->t[k].rows_per_walker * plan->t[k].in_cols; }
  float* out(int k) const {
    return base + plan->t[k].out_offset + (size_t)w0 * plan->t[k].rows_per_walker * plan->t[k].out_cols;
  }
};

// ------------------------------------------------------------ plan
struct GradPlan {
  int B;
  size_t x0, h1[QMC_MAX_LAYERS], y1[QMC_MAX_LAYERS], g1m[QMC_MAX_LAYERS], G2[QMC_MAX_LAYERS], gb;
  size_t h2[QMC_MAX_LAYERS], y2[QMC_MAX_LAYERS], amat, orb, abar, envbar, rae, aevec, lpsi;
  size_t hbar[2], zbar, tmp, zsum, g1bar, h2bar[2], z2bar, orbbar, J, total;
};

static GradPlan make_grad_plan(const qmc_model* m, int B) {
  const Dims& d = m->d;
  GradPlan p{};
  p.B = B;
  size_t o = 0;
  auto take = [&](size_t floats) { size_t r = o; o += align_up(floats * 4, 256); return r; };
  const size_t rows = (size_t)B * d.n, pairs = rows * d.n;
  int dmax = 8, kmax = 8, g1max = 8, d2max = 4;
  p.x0 = take(rows * d.d1_in_p[0]);
  for (int l = 0; l < d.L; ++l) {
    p.h1[l] = take(rows * d.d1[l]);
    p.y1[l] = take(rows * d.d1[l]);
    p.g1m[l] = take((size_t)B * d.g1_p[l]);
    p.G2[l] = take(rows * d.g2_p[l]);
    p.h2[l] = take(pairs * d.d2_in[l]);
    if (d.upd2[l]) p.y2[l] = take(pairs * d.d2[l]);
    dmax = std::max(dmax, std::max(d.d1[l], d.d1_in_p[l]));
    kmax = std::max(kmax, d.d1_in_p[l] + d.g2_p[l]);
    g1max = std::max(g1max, d.g1_p[l]);
    d2max = std::max(d2max, std::max(d.d2[l], d.d2_in[l]));
  }
  p.gb = take((size_t)B * dmax);
  const size_t am = (size_t)B * d.K * d.n * d.n;
  p.amat = take(am);
  p.orb = take(am);
  p.abar = take(am);
  p.envbar = take(am);
  p.rae = take(rows * d.A);
  p.aevec = take(rows * d.A * 3);
  p.lpsi = take(B);
  p.hbar[0] = take(rows * dmax);
  p.hbar[1] = take(rows * dmax);
  p.zbar = take(rows * dmax);
  p.tmp = take(rows * std::max(kmax, d.norb_p));
  p.zsum = take((size_t)B * dmax);
  p.g1bar = take((size_t)B * g1max);
  p.h2bar[0] = take(pairs * d2max);
  p.h2bar[1] = take(pairs * d2max);
  p.z2bar = take(pairs * d2max);
  p.orbbar = take(rows * d.norb_p);
  p.J = take((size_t)B * m->p.total);
  p.total = o;
  return p;
}

// walkers per chunk under the model's byte budget
static int grad_chunk(const qmc_model* m, int B) {
  const size_t one = make_grad_plan(m, 1).total;
  const size_t two = make_grad_plan(m, 2).total;
  const size_t per = two > one ? two - one : one;
  size_t c = m->grad_budget > one ? 1 + (m->grad_budget - one) / per : 1;
  return (int)std::max<size_t>(1, std::min<size_t>(c, (size_t)B));
}

size_t grad_workspace(const qmc_model* m, int B) { return make_grad_plan(m, grad_chunk(m, B)).total; }

#define QMC_PROF(cls, call)         \
  do {                              \
    ::qmc::ProfScope ps_((cls), s); \
    QMC_CUDA(call);                 \
  } while (0)

// Forward pass of `B` walkers keeping every layer's activations.
static qmc_status forward_save(qmc_model* m, const GradPlan& p, void* ws, const float* electrons, cudaStream_t s) {
  const Dims& d = m->d;
  const ArenaLayout& a = m->a;
  const float* ar = m->arena;
  const int B = p.B, n = d.n;
  const RowMap rows_map{n, 0, n, 1};
  const RowMap w_map{1, 0, 1, 1};
  QMC_PROF(QMC_KC_FEATURES, launch_features(s, B, n, d.A, 1, 1, d.d1_in_p[0], electrons, ar + a.atoms, ar + a.charges,
                                            m->nuclear_repulsion, at<float>(ws, p.x0), at<float>(ws, p.h2[0]),
                                            at<float>(ws, p.rae), at<float>(ws, p.aevec), nullptr));
  for (int l = 0; l < d.L; ++l) {
    const int din = d.d1_in[l], dinp = d.d1_in_p[l], dout = d.d1[l];
    const float* in = l == 0 ? at<float>(ws, p.x0) : at<float>(ws, p.h1[l - 1]);
    float* g1m = at<float>(ws, p.g1m[l]);
    float* G2 = at<float>(ws, p.G2[l]);
    float* Gb = at<float>(ws, p.gb);
    QMC_PROF(QMC_KC_MEANS, launch_mean_h1(s, B, n, d.n_up, d.C, 1, din, StF32{const_cast<float*>(in), dinp}, d.g1_p[l],
                                          StF32{g1m, d.g1_p[l]}));
    QMC_PROF(QMC_KC_BROADCAST, launch_gemm_simt(s, B, w_map, g1m, d.g1_p[l], d.g1_p[l], nullptr, 0, 0, ar + a.w_g1[l],
                                                dout, dout, EpiStore{Gb, dout, nullptr}));
    QMC_PROF(QMC_KC_MEANS, launch_mean_h2(s, B, n, d.n_up, d.C, 1, 1, d.d2_in[l], 1, at<float>(ws, p.h2[l]), d.g2_p[l],
                                          StF32{G2, d.g2_p[l]}));
    EpiLayerSave epi{Gb, ar + a.b1[l], (l > 0 && din == dout) ? in : nullptr, at<float>(ws, p.h1[l]),
                     at<float>(ws, p.y1[l]), dout};
    QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rows_map, in, dinp, dinp, G2, d.g2_p[l], d.g2_p[l],
                                                   ar + a.w_main[l], dout, dout, epi));
    if (d.upd2[l]) {
      const size_t np = (size_t)B * n * n;
      ::qmc::ProfScope ps_(QMC_KC_PAIR, s);
      k_pair_fwd_save<<<blocks(np * d.d2[l]), 256, 0, s>>>((int)np, d.d2_in[l], d.d2[l], at<float>(ws, p.h2[l]),
                                                            ar + a.w2[l], ar + a.b2[l], at<float>(ws, p.h2[l + 1]),
                                                            at<float>(ws, p.y2[l]));
      QMC_CUDA(cudaGetLastError());
    }
  }
  const int nch = d.split ? 2 : 1;
  for (int c = 0; c < nch; ++c) {
    const int ns = d.split ? (c == 0 ? d.n_up : d.n_dn) : d.n;
    const int i0 = (d.split && c == 1) ? d.n_up : 0;
    RowMap map{ns, i0, n, 1};
    EpiOrbital epi{at<float>(ws, p.amat), at<float>(ws, p.rae), at<float>(ws, p.aevec), ar + a.env_pi[c],
                   ar + a.env_sigma[c], n, d.A, d.K, 1, d.env_abs};
    epi.orb = at<float>(ws, p.orb);
    epi.unit_env = !env_in_epilogue(d.env_kind);
    QMC_PROF(QMC_KC_ORBITAL, launch_gemm_simt(s, B * ns, map, at<float>(ws, p.h1[d.L - 1]), d.d_last, d.d_last, nullptr,
                                              0, 0, ar + a.w_orb[c], d.norb_p, d.norb, epi));
  }
  if (d.env_kind == QMC_ENVELOPE_DIAGONAL) {
    const int c1 = nch - 1;
    QMC_PROF(QMC_KC_ORBITAL, launch_envelope_diag(s, B, n, d.n_up, d.split, d.K, d.A, 1, 1, ar + a.env_pi[0],
                                                  ar + a.env_sigma[0], ar + a.env_pi[c1], ar + a.env_sigma[c1],
                                                  at<float>(ws, p.aevec), at<float>(ws, p.amat)));
  }
  return QMC_OK;
}

// Backward pass of one chunk: per-walker Jacobian rows into J (row stride P).
static qmc_status backward(qmc_model* m, const GradPlan& p, void* ws, float* J, float* logpsi, cudaStream_t s,
                           const TapOut* taps = nullptr) {
  const Dims& d = m->d;
  const ArenaLayout& a = m->a;
  const ParamLayout& pl = m->p;
  const float* ar = m->arena;
  const int B = p.B, n = d.n;
  const size_t P = pl.total, rows = (size_t)B * n, pairs = rows * n;
  const RowMap rows_map{n, 0, n, 1};
  const RowMap w_map{1, 0, 1, 1};
  QMC_PROF(QMC_KC_LOGDET, launch_logdet_bwd(s, B, n, d.K, at<float>(ws, p.amat), at<float>(ws, p.abar), logpsi));
  const int nch = d.split ? 2 : 1;
  {
    ::qmc::ProfScope ps_(QMC_KC_ORBITAL, s);
    k_orb_bwd<<<blocks(rows * d.norb_p), 256, 0, s>>>(
        B, n, d.n_up, d.split, d.K, d.A, d.env_abs, d.env_kind, d.norb_p, at<float>(ws, p.abar), at<float>(ws, p.orb),
        at<float>(ws, p.rae), at<float>(ws, p.aevec), ar + a.env_pi[0], ar + a.env_sigma[0], ar + a.env_pi[nch - 1],
        ar + a.env_sigma[nch - 1], at<float>(ws, p.orbbar), at<float>(ws, p.envbar));
    QMC_CUDA(cudaGetLastError());
  }
  float* hbar = at<float>(ws, p.hbar[0]);
  for (int c = 0; c < nch; ++c) {
    const int ns = d.split ? (c == 0 ? d.n_up : d.n_dn) : d.n;
    const int i0 = (d.split && c == 1) ? d.n_up : 0;
    {
      ::qmc::ProfScope ps_(QMC_KC_OTHER, s);
      if (d.env_kind == QMC_ENVELOPE_DIAGONAL)
        k_env_jac_diag<<<blocks((size_t)B * n * d.A * d.K), 256, 0, s>>>(
            B, n, i0, ns, d.K, d.A, at<float>(ws, p.envbar), at<float>(ws, p.aevec), ar + a.env_pi[c],
            ar + a.env_sigma[c], J, P, pl.env_pi[c], pl.env_sigma[c]);
      else if (d.env_kind != QMC_ENVELOPE_NULL)
        k_env_jac<<<blocks((size_t)B * n * d.A * d.K), 256, 0, s>>>(B, n, i0, ns, d.K, d.A, d.env_abs,
                                                                   at<float>(ws, p.envbar), at<float>(ws, p.rae),
                                                                   ar + a.env_pi[c], ar + a.env_sigma[c], J, P,
                                                                   pl.env_pi[c], pl.env_sigma[c]);
      QMC_CUDA(cudaGetLastError());
      QMC_CUDA(jac_outer(s,
          B, ns, n, i0, at<float>(ws, p.h1[d.L - 1]), d.d_last, d.d_last, at<float>(ws, p.orbbar), d.norb_p, d.norb, J,
          P, pl.orb_k[c]));
    }
    if (taps) {  // orbital projection of channel c: inputs h1[L-1] and cotangents orbbar, its rows only
      int k = 0;
      for (int l = 0; l < d.L; ++l) k += d.upd2[l] ? 2 : 1;
      k += c;
      k_tap_gather<<<blocks((size_t)B * ns * d.d_last), 256, 0, s>>>(B, n, i0, ns, at<float>(ws, p.h1[d.L - 1]),
                                                                    d.d_last, d.d_last, taps->in(k));
      QMC_CUDA(cudaGetLastError());
      k_tap_gather<<<blocks((size_t)B * ns * d.norb), 256, 0, s>>>(B, n, i0, ns, at<float>(ws, p.orbbar), d.norb_p,
                                                                  d.norb, taps->out(k));
      QMC_CUDA(cudaGetLastError());
    }
    // hbar of the last layer's rows of this channel = orbbar W_orb^T
    RowMap map{ns, i0, n, 1};
    QMC_PROF(QMC_KC_ORBITAL, launch_gemm_simt(s, B * ns, map, at<float>(ws, p.orbbar), d.norb_p, d.norb_p, nullptr, 0, 0,
                                              ar + a.wt_orb[c], d.d_last, d.d_last, EpiStore{hbar, d.d_last, nullptr}));
  }
  int hb = 0, h2b = 0;
  for (int l = d.L - 1; l >= 0; --l) {
    const int din = d.d1_in[l], dinp = d.d1_in_p[l], dout = d.d1[l];
    const bool res = l > 0 && din == dout;
    const float* in = l == 0 ? at<float>(ws, p.x0) : at<float>(ws, p.h1[l - 1]);
    float* hb_out = at<float>(ws, p.hbar[hb]);
    float* zbar = at<float>(ws, p.zbar);
    float* zsum = at<float>(ws, p.zsum);
    {
      ::qmc::ProfScope ps_(QMC_KC_STREAM_LAYER, s);
      k_tanh_bwd<<<blocks(rows * dout), 256, 0, s>>>(rows * dout, res ? kRsqrt2 : 1.f, hb_out, at<float>(ws, p.y1[l]),
                                                     zbar);
      QMC_CUDA(cudaGetLastError());
      if (taps) {  // one-electron Dense l: inputs [h1 | means] and output cotangents zbar
        int k = 0;
        for (int q = 0; q < l; ++q) k += d.upd2[q] ? 2 : 1;
        const int cols = din + d.C * din + d.C * d.d2_in[l];
        k_tap_x1<<<blocks(rows * cols), 256, 0, s>>>(B, n, din, dinp, d.C * din, d.g1_p[l], d.C * d.d2_in[l], d.g2_p[l],
                                                     in, at<float>(ws, p.g1m[l]), at<float>(ws, p.G2[l]), taps->in(k));
        QMC_CUDA(cudaGetLastError());
        QMC_CUDA(cudaMemcpyAsync(taps->out(k), zbar, sizeof(float) * rows * dout, cudaMemcpyDeviceToDevice, s));
      }
      const size_t k0 = pl.dense1_k[l];
      QMC_CUDA(jac_outer(s, B, n, n, 0, in, dinp, din, zbar, dout, dout, J, P, k0));
      QMC_CUDA(jac_outer(s,
          B, n, n, 0, at<float>(ws, p.G2[l]), d.g2_p[l], d.C * d.d2_in[l], zbar, dout, dout, J, P,
          k0 + (size_t)(din + d.C * din) * dout));
      k_colsum<<<blocks((size_t)B * dout), 256, 0, s>>>(B, n, zbar, dout, dout, zsum, J, P, pl.dense1_b[l]);
      QMC_CUDA(cudaGetLastError());
      QMC_CUDA(jac_outer(s, B, 1, 1, 0, at<float>(ws, p.g1m[l]), d.g1_p[l],
                                                                      d.C * din, zsum, dout, dout, J, P,
                                                                      k0 + (size_t)din * dout));
    }
    float* tmp = at<float>(ws, p.tmp);
    const int kmain = dinp + d.g2_p[l];
    if (l > 0) {
      // [h | g2] input cotangents = zbar W_main^T ; spin-mean cotangent = zsum W_g1^T
      QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rows_map, zbar, dout, dout, nullptr, 0, 0,
                                                     ar + a.wt_main[l], kmain, kmain, EpiStore{tmp, kmain, nullptr}));
      float* g1bar = at<float>(ws, p.g1bar);
      QMC_PROF(QMC_KC_BROADCAST, launch_gemm_simt(s, B, w_map, zsum, dout, dout, nullptr, 0, 0, ar + a.wt_g1[l],
                                                  d.g1_p[l], d.g1_p[l], EpiStore{g1bar, d.g1_p[l], nullptr}));
      ::qmc::ProfScope ps_(QMC_KC_MEANS, s);
      k_input_grad<<<blocks(rows * din), 256, 0, s>>>(B, n, d.n_up, d.C, din, tmp, kmain, hb_out, res ? 1 : 0, g1bar,
                                                      d.g1_p[l], at<float>(ws, p.hbar[hb ^ 1]));
      QMC_CUDA(cudaGetLastError());
    }
    // two-electron stream: h2[l+1] = pair_l(h2[l]) for l < L-1; G2[l] = means of h2[l]
    {
      ::qmc::ProfScope ps_(QMC_KC_PAIR, s);
      float* h2b_next = at<float>(ws, p.h2bar[h2b]);  // cotangent of h2[l+1]
      float* h2b_cur = at<float>(ws, p.h2bar[h2b ^ 1]);
      bool have_cur = false;
      if (d.upd2[l]) {
        float* z2 = at<float>(ws, p.z2bar);
        k_tanh_bwd<<<blocks(pairs * d.d2[l]), 256, 0, s>>>(pairs * d.d2[l], d.d2_in[l] == d.d2[l] ? kRsqrt2 : 1.f,
                                                          h2b_next, at<float>(ws, p.y2[l]), z2);
        QMC_CUDA(cudaGetLastError());
        if (taps) {  // two-electron Dense l: inputs h2[l] and output cotangents z2 (contiguous pair rows)
          int k = 1;
          for (int q = 0; q < l; ++q) k += d.upd2[q] ? 2 : 1;
          QMC_CUDA(cudaMemcpyAsync(taps->in(k), at<float>(ws, p.h2[l]), sizeof(float) * pairs * d.d2_in[l],
                                   cudaMemcpyDeviceToDevice, s));
          QMC_CUDA(cudaMemcpyAsync(taps->out(k), z2, sizeof(float) * pairs * d.d2[l], cudaMemcpyDeviceToDevice, s));
        }
        QMC_CUDA(jac_outer(s,
            B, n * n, n * n, 0, at<float>(ws, p.h2[l]), d.d2_in[l], d.d2_in[l], z2, d.d2[l], d.d2[l], J, P,
            pl.dense2_k[l]));
        k_colsum<<<blocks((size_t)B * d.d2[l]), 256, 0, s>>>(B, n * n, z2, d.d2[l], d.d2[l], nullptr, J, P,
                                                             pl.dense2_b[l]);
        QMC_CUDA(cudaGetLastError());
        if (l > 0) {
          k_pair_bwd_data<<<blocks(pairs * d.d2_in[l]), 256, 0, s>>>(pairs, d.d2_in[l], d.d2[l], z2, ar + a.wt2[l],
                                                                    h2b_next, h2b_cur);
          QMC_CUDA(cudaGetLastError());
          have_cur = true;
        }
      }
      if (l > 0) {
        k_h2_from_g2<<<blocks(pairs * d.d2_in[l]), 256, 0, s>>>(B, n, d.n_up, d.C, d.d2_in[l], tmp, kmain, dinp, h2b_cur,
                                                               have_cur ? 1 : 0);
        QMC_CUDA(cudaGetLastError());
        h2b ^= 1;
      }
    }
    hb ^= 1;
  }
  return QMC_OK;
}

// qmc_grad_taps: the adjoint's chunks with the layer taps written out; the
// envelope tap is the envelope columns of each chunk's per-walker Jacobian.
qmc_status run_grad_taps(qmc_model* m, int batch, const float* electrons, float* taps, size_t taps_floats,
                         float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s) {
  const int chunk = grad_chunk(m, batch);
  const GradPlan p = make_grad_plan(m, chunk);
  if (ws_bytes < p.total) {
    set_error("workspace too small for the adjoint: %zu bytes given, %zu needed", ws_bytes, p.total);
    return QMC_ERR_WORKSPACE;
  }
  const TapPlan tp = make_taps(m, batch);
  if (taps_floats < tp.total) {
    set_error("taps buffer too small: %zu floats given, %zu needed", taps_floats, tp.total);
    return QMC_ERR_WORKSPACE;
  }
  const size_t P = m->p.total;
  for (int w0 = 0; w0 < batch; w0 += chunk) {
    const int B = std::min(chunk, batch - w0);
    GradPlan q = make_grad_plan(m, B);
    float* J = at<float>(ws, q.J);
    TapOut to;
    to.base = taps;
    to.plan = &tp;
    to.w0 = w0;
    QMC_TRY(forward_save(m, q, ws, electrons + (size_t)w0 * m->d.n * 3, s));
    QMC_TRY(backward(m, q, ws, J, logpsi ? logpsi + w0 : nullptr, s, &to));
    const qmc_layer_tap& et = tp.t[tp.count - 1];
    if (et.kind == QMC_TAP_DIAGONAL)
      QMC_CUDA(cudaMemcpy2DAsync(to.out(tp.count - 1), sizeof(float) * et.out_cols, J + et.kernel_offset,
                                 sizeof(float) * P, sizeof(float) * et.out_cols, B, cudaMemcpyDeviceToDevice, s));
  }
  return QMC_OK;
}

int layer_taps(const qmc_model* m, int batch, qmc_layer_tap* taps, int max_taps, size_t* total) {
  const TapPlan tp = make_taps(m, batch);
  for (int k = 0; k < tp.count && k < max_taps; ++k) taps[k] = tp.t[k];
  if (total) *total = tp.total;
  return tp.count;
}

qmc_status run_grad(qmc_model* m, int batch, const float* electrons, const double* weights, float* per_walker,
                    double* grad, float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s) {
  const int chunk = grad_chunk(m, batch);
  const GradPlan p = make_grad_plan(m, chunk);
  if (ws_bytes < p.total) {
    set_error("workspace too small for the adjoint: %zu bytes given, %zu needed", ws_bytes, p.total);
    return QMC_ERR_WORKSPACE;
  }
  const size_t P = m->p.total;
  if (grad) QMC_CUDA(cudaMemsetAsync(grad, 0, P * sizeof(double), s));
  for (int w0 = 0; w0 < batch; w0 += chunk) {
    const int B = std::min(chunk, batch - w0);
    GradPlan q = make_grad_plan(m, B);
    // the chunk's plan lays out fewer walkers inside the same workspace
    float* J = per_walker ? per_walker + (size_t)w0 * P : at<float>(ws, q.J);
    QMC_TRY(forward_save(m, q, ws, electrons + (size_t)w0 * m->d.n * 3, s));
    QMC_TRY(backward(m, q, ws, J, logpsi ? logpsi + w0 : nullptr, s));
    if (grad && weights) {
      ::qmc::ProfScope ps_(QMC_KC_OTHER, s);
      k_weighted_sum<<<blocks(P), 256, 0, s>>>(B, P, J, weights + w0, grad);
      QMC_CUDA(cudaGetLastError());
    }
  }
  return QMC_OK;
}


// =====================================================================
// Psiformer parameter adjoint (FP32 SIMT): per-walker d log|psi| / d theta of
// PsiformerWavefunction (src/jaqmc/app/molecule/wavefunction/psiformer.py:
// 38-146, backbone src/jaqmc/wavefunction/backbone/psiformer.py:29-187,
// Jastrow src/jaqmc/wavefunction/jastrow.py:48-122), the reverse of the value
// forward: input Dense, per layer LayerNorm -> multi-head attention (QKV
// Dense, softmax(q k^T / sqrt(Dh)) v, output Dense) -> residual -> LayerNorm
// -> tanh MLP -> residual, orbitals x envelope, log-sum-exp of determinants,
// plus the Jastrow.  The forward keeps every layer's activations (the
// backward needs them all); walkers run in chunks under the gradient budget.
// =====================================================================

// LayerNorm of one row per warp (D <= 512, a multiple of 32): y = (x - mu) rs s + b,
// rs = 1 / sqrt(var + 1e-5) with the biased two-pass variance; mu and rs kept.
__global__ void k_psi_ln_fwd(int rows, int D, const float* __restrict__ x, const float* __restrict__ sc,
                             const float* __restrict__ bi, float* __restrict__ y, float* __restrict__ mu,
                             float* __restrict__ rs) {
  const int lane = threadIdx.x & 31;
  const size_t r = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= (size_t)rows) return;
  const float* xr = x + r * D;
  float s = 0.f;
  for (int f = lane; f < D; f += 32) s += xr[f];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const float m = s / (float)D;
  float q = 0.f;
  for (int f = lane; f < D; f += 32) q += (xr[f] - m) * (xr[f] - m);
  for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
  const float inv = rsqrtf(q / (float)D + 1e-5f);
  for (int f = lane; f < D; f += 32) y[r * D + f] = (xr[f] - m) * inv * sc[f] + bi[f];
  if (lane == 0) {
    mu[r] = m;
    rs[r] = inv;
  }
}

// dx += rs (g - mean(g) - xhat mean(g xhat)), g = dy s, xhat = (x - mu) rs (one warp per row).
__global__ void k_psi_ln_bwd(int rows, int D, const float* __restrict__ x, const float* __restrict__ mu,
                             const float* __restrict__ rs, const float* __restrict__ sc, const float* __restrict__ dy,
                             float* __restrict__ dx) {
  const int lane = threadIdx.x & 31;
  const size_t r = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= (size_t)rows) return;
  const float m = mu[r], inv = rs[r];
  float sg = 0.f, sgx = 0.f;
  for (int f = lane; f < D; f += 32) {
    const float g = dy[r * D + f] * sc[f];
    sg += g;
    sgx += g * (x[r * D + f] - m) * inv;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sg += __shfl_xor_sync(0xffffffffu, sg, o);
    sgx += __shfl_xor_sync(0xffffffffu, sgx, o);
  }
  sg /= (float)D;
  sgx /= (float)D;
  for (int f = lane; f < D; f += 32) {
    const float xh = (x[r * D + f] - m) * inv;
    dx[r * D + f] += inv * (dy[r * D + f] * sc[f] - sg - xh * sgx);
  }
}

// Per-walker LayerNorm parameter rows: J[scale_f] = sum_i xhat_if dy_if, J[bias_f] = sum_i dy_if.
__global__ void k_psi_ln_jac(int B, int n, int D, const float* __restrict__ x, const float* __restrict__ mu,
                             const float* __restrict__ rs, const float* __restrict__ dy, float* __restrict__ J,
                             size_t P, size_t off_s, size_t off_b) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)B * D) return;
  const int w = (int)(e / D), f = (int)(e % D);
  float js = 0.f, jb = 0.f;
  for (int i = 0; i < n; ++i) {
    const size_t r = (size_t)w * n + i;
    const float g = dy[r * D + f];
    js = fmaf((x[r * D + f] - mu[r]) * rs[r], g, js);
    jb += g;
  }
  J[(size_t)w * P + off_s + f] = js;
  J[(size_t)w * P + off_b + f] = jb;
}

__global__ void k_psi_add_jas(int B, float* __restrict__ lp, const float* __restrict__ jas) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < B) lp[w] += jas[w];
}

__global__ void k_psi_tanh_add(size_t count, float* __restrict__ z, const float* __restrict__ res,
                               float* __restrict__ out, int act) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= count) return;
  float v = z[e];
  if (act) v = tanhf(v);
  z[e] = v;
  if (out) out[e] = v + res[e];
}

// Attention of one (walker, head) per block, keeping the probabilities:
// qkv rows [q | k | v] with biases (q unscaled); P[w][h][i][j] = softmax_j(q_i . k_j / sqrt(Dh));
// o[w n + i][h Dh + d] = sum_j P_ij v_jd.  n <= 64, Dh <= 64.
__global__ void __launch_bounds__(128) k_psi_attn_save(int n, int H, int Dh, const float* __restrict__ qkv,
                                                       float* __restrict__ Pr, float* __restrict__ o) {
  extern __shared__ float sm[];
  const int w = blockIdx.x / H, h = blockIdx.x % H, D = H * Dh;
  float* q = sm;              // [n][Dh]
  float* k = q + n * Dh;      // [n][Dh]
  float* v = k + n * Dh;      // [n][Dh]
  float* S = v + n * Dh;      // [n][n]
  for (int e = threadIdx.x; e < n * Dh; e += blockDim.x) {
    const int i = e / Dh, d = e % Dh;
    const float* r = qkv + ((size_t)w * n + i) * 3 * D + h * Dh + d;
    q[e] = r[0];
    k[e] = r[D];
    v[e] = r[2 * D];
  }
  __syncthreads();
  const float sc = 1.0f / sqrtf((float)Dh);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    float a = 0.f;
    for (int d = 0; d < Dh; ++d) a = fmaf(q[i * Dh + d], k[j * Dh + d], a);
    S[e] = a * sc;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int i = threadIdx.x >> 5; i < n; i += nw) {
    float mx = -INFINITY;
    for (int j = lane; j < n; j += 32) mx = fmaxf(mx, S[i * n + j]);
    for (int of = 16; of > 0; of >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, of));
    float sum = 0.f;
    for (int j = lane; j < n; j += 32) {
      const float e = expf(S[i * n + j] - mx);
      S[i * n + j] = e;
      sum += e;
    }
    for (int of = 16; of > 0; of >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, of);
    for (int j = lane; j < n; j += 32) S[i * n + j] /= sum;
  }
  __syncthreads();
  float* Pw = Pr + ((size_t)w * H + h) * n * n;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) Pw[e] = S[e];
  for (int e = threadIdx.x; e < n * Dh; e += blockDim.x) {
    const int i = e / Dh, d = e % Dh;
    float a = 0.f;
    for (int j = 0; j < n; ++j) a = fmaf(S[i * n + j], v[j * Dh + d], a);
    o[((size_t)w * n + i) * D + h * Dh + d] = a;
  }
}

// Attention backward of one (walker, head): from do (the cotangent of o),
//   dv = P^T do, dP = do v^T, dS = P (dP - rowsum(dP P)),
//   dq = dS k / sqrt(Dh), dk = dS^T q / sqrt(Dh), written into qkvbar rows [dq | dk | dv].
__global__ void __launch_bounds__(128) k_psi_attn_bwd(int n, int H, int Dh, const float* __restrict__ qkv,
                                                      const float* __restrict__ Pr, const float* __restrict__ dout,
                                                      float* __restrict__ qkvbar) {
  extern __shared__ float sm[];
  const int w = blockIdx.x / H, h = blockIdx.x % H, D = H * Dh;
  float* q = sm;
  float* k = q + n * Dh;
  float* v = k + n * Dh;
  float* g = v + n * Dh;      // do [n][Dh]
  float* P = g + n * Dh;      // [n][n]
  float* dS = P + n * n;      // [n][n]
  for (int e = threadIdx.x; e < n * Dh; e += blockDim.x) {
    const int i = e / Dh, d = e % Dh;
    const float* r = qkv + ((size_t)w * n + i) * 3 * D + h * Dh + d;
    q[e] = r[0];
    k[e] = r[D];
    v[e] = r[2 * D];
    g[e] = dout[((size_t)w * n + i) * D + h * Dh + d];
  }
  const float* Pw = Pr + ((size_t)w * H + h) * n * n;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) P[e] = Pw[e];
  __syncthreads();
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {  // dP_ij = do_i . v_j
    const int i = e / n, j = e % n;
    float a = 0.f;
    for (int d = 0; d < Dh; ++d) a = fmaf(g[i * Dh + d], v[j * Dh + d], a);
    dS[e] = a;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int i = threadIdx.x >> 5; i < n; i += nw) {
    float t = 0.f;
    for (int j = lane; j < n; j += 32) t += dS[i * n + j] * P[i * n + j];
    for (int of = 16; of > 0; of >>= 1) t += __shfl_xor_sync(0xffffffffu, t, of);
    for (int j = lane; j < n; j += 32) dS[i * n + j] = P[i * n + j] * (dS[i * n + j] - t);
  }
  __syncthreads();
  const float sc = 1.0f / sqrtf((float)Dh);
  for (int e = threadIdx.x; e < n * Dh; e += blockDim.x) {
    const int i = e / Dh, d = e % Dh;
    float dq = 0.f, dk = 0.f, dv = 0.f;
    for (int j = 0; j < n; ++j) {
      dq = fmaf(dS[i * n + j], k[j * Dh + d], dq);
      dk = fmaf(dS[j * n + i], q[j * Dh + d], dk);
      dv = fmaf(P[j * n + i], g[j * Dh + d], dv);
    }
    float* out = qkvbar + ((size_t)w * n + i) * 3 * D + h * Dh + d;
    out[0] = dq * sc;
    out[D] = dk * sc;
    out[2 * D] = dv;
  }
}

// SimpleEE Jastrow parameter rows: d/d alpha of -c alpha^2 / (alpha + r) is
// -c alpha (alpha + 2 r) / (alpha + r)^2 (c = 1/4 same spin, 1/2 opposite).
__global__ void k_psi_jas_jac(int B, int n, int n_up, const float* __restrict__ x, const float* __restrict__ alpha,
                              float* __restrict__ J, size_t P, size_t off_par, size_t off_anti) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  const float ap = alpha[0], aa = alpha[1];
  float jp = 0.f, ja = 0.f;
  const float* xw = x + (size_t)w * n * 3;
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      const float dx = xw[3 * i] - xw[3 * j], dy = xw[3 * i + 1] - xw[3 * j + 1], dz = xw[3 * i + 2] - xw[3 * j + 2];
      const float r = sqrtf(dx * dx + dy * dy + dz * dz);
      if ((i < n_up) == (j < n_up)) jp += -0.25f * ap * (ap + 2.f * r) / ((ap + r) * (ap + r));
      else ja += -0.5f * aa * (aa + 2.f * r) / ((aa + r) * (aa + r));
    }
  J[(size_t)w * P + off_par] = jp;
  J[(size_t)w * P + off_anti] = ja;
}

struct PsiGradPlan {
  int B;
  size_t x0, rae, aevec, jas, h[kPsiMaxLayers + 1], mu0[kPsiMaxLayers], rs0[kPsiMaxLayers], xn0[kPsiMaxLayers],
      qkv[kPsiMaxLayers], pr[kPsiMaxLayers], o[kPsiMaxLayers], hm[kPsiMaxLayers], mu1[kPsiMaxLayers],
      rs1[kPsiMaxLayers], xn1[kPsiMaxLayers], y[kPsiMaxLayers][kPsiMaxMlp + 1];
  size_t amat, orb, abar, envbar, hbar, hmbar, zbar, tmp, obar, qkvbar, orbbar, J, total;
};

static PsiGradPlan make_psi_grad_plan(const qmc_model* m, int B) {
  const PsiDims& d = m->psi->d;
  PsiGradPlan p{};
  p.B = B;
  size_t o = 0;
  auto take = [&](size_t floats) { size_t r = o; o += align_up(floats * 4, 256); return r; };
  const size_t rows = (size_t)B * d.n, D = d.D;
  int wmax = d.D;
  for (int k = 0; k < d.n_dense; ++k) wmax = std::max(wmax, d.mlp[k]);
  p.x0 = take(rows * d.K0p);
  p.rae = take(rows * d.A);
  p.aevec = take(rows * d.A * 3);
  p.jas = take(B);
  for (int l = 0; l <= d.L; ++l) p.h[l] = take(rows * D);
  for (int l = 0; l < d.L; ++l) {
    p.mu0[l] = take(rows);
    p.rs0[l] = take(rows);
    p.xn0[l] = take(rows * D);
    p.qkv[l] = take(rows * 3 * D);
    p.pr[l] = take((size_t)B * d.H * d.n * d.n);
    p.o[l] = take(rows * D);
    p.hm[l] = take(rows * D);
    p.mu1[l] = take(rows);
    p.rs1[l] = take(rows);
    p.xn1[l] = take(rows * D);
    for (int k = 0; k < d.n_dense; ++k) p.y[l][k] = take(rows * d.mlp[k]);
  }
  const size_t am = (size_t)B * d.K * d.n * d.n;
  p.amat = take(am);
  p.orb = take(am);
  p.abar = take(am);
  p.envbar = take(am);
  p.hbar = take(rows * D);
  p.hmbar = take(rows * D);
  p.zbar = take(rows * wmax);
  p.tmp = take(rows * std::max<size_t>(3 * D, std::max<size_t>(wmax, m->d.norb_p)));
  p.obar = take(rows * D);
  p.qkvbar = take(rows * 3 * D);
  p.orbbar = take(rows * m->d.norb_p);
  p.J = take((size_t)B * m->psi->p.total);
  p.total = o;
  return p;
}

static size_t attn_grad_total(const qmc_model* m, int B);

static int psi_grad_chunk(const qmc_model* m, int B) {
  const size_t one = attn_grad_total(m, 1);
  const size_t two = attn_grad_total(m, 2);
  const size_t per = two > one ? two - one : one;
  const size_t c = m->grad_budget > one ? 1 + (m->grad_budget - one) / per : 1;
  return (int)std::max<size_t>(1, std::min<size_t>(c, (size_t)B));
}

size_t psi_grad_workspace(const qmc_model* m, int B) { return attn_grad_total(m, psi_grad_chunk(m, B)); }

// Layer taps of the attention backbones (KFAC statistics): the dense layers'
// inputs and output cotangents per application (n rows per walker; the
// orbital projection per spin channel), the LayerNorm scales / shifts and the
// trailing envelope / Jastrow parameters as diagonal taps (per-walker rows of
// the Jacobian).  The indices say where each layer's tap sits in the plan.
struct AttnTaps {
  TapPlan plan;
  int in = -1, orb[2] = {-1, -1}, tail = -1;
  int ln0[kPsiMaxLayers], ln1[kPsiMaxLayers], q[kPsiMaxLayers], k[kPsiMaxLayers], v[kPsiMaxLayers];
  int o[kPsiMaxLayers], mlp[kPsiMaxLayers][kPsiMaxMlp + 1];
  int qk[kPsiMaxLayers], lv[kPsiMaxLayers], lo[kPsiMaxLayers], vu[kPsiMaxLayers], ul[kPsiMaxLayers][kLapMaxLocal];
};

static int lap_local(const PsiDims& d, int l);

static AttnTaps make_attn_taps(const qmc_model* m, int B) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const Dims& fd = m->d;
  AttnTaps a{};
  TapPlan& tp = a.plan;
  size_t o = 0;
  auto add = [&](int kind, int rpw, int in_cols, int out_cols, int bias, size_t k_off, size_t b_off) {
    qmc_layer_tap& t = tp.t[tp.count];
    t.kind = kind;
    t.rows_per_walker = rpw;
    t.in_cols = in_cols;
    t.out_cols = out_cols;
    t.has_bias = bias;
    t.kernel_offset = k_off;
    t.bias_offset = b_off;
    t.in_offset = o;
    o += (size_t)B * rpw * in_cols;
    t.out_offset = o;
    o += (size_t)B * rpw * out_cols;
    return tp.count++;
  };
  const int n = d.n, D = d.D;
  const bool lap = d.arch == kArchLapNet;
  const int in_bias = lap ? d.in_bias : 1;
  a.in = add(QMC_TAP_DENSE, n, d.K0, D, in_bias, P.in_k, in_bias ? P.in_b : 0);
  for (int l = 0; l < d.L; ++l) {
    if (lap) {
      const int bb = d.bb_bias;
      a.qk[l] = add(QMC_TAP_DENSE, n, D, 2 * D, bb, P.qk_k[l], bb ? P.qk_b[l] : 0);
      a.lv[l] = add(QMC_TAP_DENSE, n, D, D, bb, P.lv_k[l], bb ? P.lv_b[l] : 0);
      a.lo[l] = add(QMC_TAP_DENSE, n, D, D, bb, P.lo_k[l], bb ? P.lo_b[l] : 0);
      a.vu[l] = add(QMC_TAP_DENSE, n, D, D, bb, P.vu_k[l], bb ? P.vu_b[l] : 0);
      for (int j = 0; j < lap_local(d, l); ++j)
        a.ul[l][j] = add(QMC_TAP_DENSE, n, D, D, bb, P.ul_k[l][j], bb ? P.ul_b[l][j] : 0);
      continue;
    }
    a.ln0[l] = add(QMC_TAP_DIAGONAL, 1, 0, 2 * D, 0, P.ln0_s[l], 0);  // scale then shift
    a.q[l] = add(QMC_TAP_DENSE, n, D, D, 1, P.q_k[l], P.q_b[l]);
    a.k[l] = add(QMC_TAP_DENSE, n, D, D, 1, P.k_k[l], P.k_b[l]);
    a.v[l] = add(QMC_TAP_DENSE, n, D, D, 1, P.v_k[l], P.v_b[l]);
    a.o[l] = add(QMC_TAP_DENSE, n, D, D, 1, P.o_k[l], P.o_b[l]);
    a.ln1[l] = add(QMC_TAP_DIAGONAL, 1, 0, 2 * D, 0, P.ln1_s[l], 0);
    int din = D;
    for (int k = 0; k < d.n_dense; ++k) {
      a.mlp[l][k] = add(QMC_TAP_DENSE, n, din, d.mlp[k], 1, P.mlp_k[l][k], P.mlp_b[l][k]);
      din = d.mlp[k];
    }
  }
  const int nch = fd.split ? 2 : 1;
  for (int c = 0; c < nch; ++c) {
    const int ns = fd.split ? (c == 0 ? fd.n_up : fd.n_dn) : n;
    a.orb[c] = add(QMC_TAP_DENSE, ns, D, fd.norb, 0, P.orb_k[c], 0);
  }
  const size_t env0 = P.env_pi[0];
  if (P.total > env0) a.tail = add(QMC_TAP_DIAGONAL, 1, 0, (int)(P.total - env0), 0, env0, 0);
  tp.total = o;
  return a;
}

// dst [rows][cols] (contiguous) = src [rows][cols] with row stride ld
static cudaError_t tap_copy(cudaStream_t s, float* dst, int cols, const float* src, int ld, size_t rows) {
  return cudaMemcpy2DAsync(dst, sizeof(float) * cols, src, sizeof(float) * ld, sizeof(float) * cols, rows,
                           cudaMemcpyDeviceToDevice, s);
}

// Orbitals x envelope of an attention backbone's output hL [B n][D] into
// amat (the raw orbitals kept in orb for the envelope cotangent).
static qmc_status attn_orbitals_fwd(qmc_model* m, int B, void* ws, const float* hL, size_t amat, size_t orb,
                                    size_t rae, size_t aevec, cudaStream_t s) {
  const Dims& fd = m->d;
  const ArenaLayout& fa = m->a;
  const float* ar = m->arena;
  const int n = fd.n, D = fd.d_last;
  const int nch = fd.split ? 2 : 1;
  for (int c = 0; c < nch; ++c) {
    const int ns = fd.split ? (c == 0 ? fd.n_up : fd.n_dn) : n;
    const int i0 = (fd.split && c == 1) ? fd.n_up : 0;
    RowMap map{ns, i0, n, 1};
    EpiOrbital epi{at<float>(ws, amat), at<float>(ws, rae), at<float>(ws, aevec), ar + fa.env_pi[c],
                   ar + fa.env_sigma[c], n, fd.A, fd.K, 1, fd.env_abs};
    epi.orb = at<float>(ws, orb);
    epi.unit_env = !env_in_epilogue(fd.env_kind);
    QMC_PROF(QMC_KC_ORBITAL, launch_gemm_simt(s, B * ns, map, hL, D, D, nullptr, 0, 0, ar + fa.w_orb[c], fd.norb_p,
                                              fd.norb, epi));
  }
  if (fd.env_kind == QMC_ENVELOPE_DIAGONAL) {
    const int c1 = nch - 1;
    QMC_PROF(QMC_KC_ORBITAL, launch_envelope_diag(s, B, n, fd.n_up, fd.split, fd.K, fd.A, 1, 1, ar + fa.env_pi[0],
                                                  ar + fa.env_sigma[0], ar + fa.env_pi[c1], ar + fa.env_sigma[c1],
                                                  at<float>(ws, aevec), at<float>(ws, amat)));
  }
  return QMC_OK;
}

// Determinant, orbital and envelope backward of an attention backbone:
// log|psi| (+ Jastrow) into lp, the orbital and envelope Jacobian rows, and
// the cotangent hbar [B n][D] of the backbone output hL.
static qmc_status attn_orbitals_bwd(qmc_model* m, int B, void* ws, const float* hL, size_t amat, size_t orb,
                                    size_t abar, size_t envbar, size_t rae, size_t aevec, size_t orbbar, size_t jas,
                                    float* hbar, float* J, float* lp, cudaStream_t s, const TapOut* taps = nullptr,
                                    const int* orb_tap = nullptr) {
  const PsiParams& P = m->psi->p;
  const Dims& fd = m->d;
  const ArenaLayout& fa = m->a;
  const float* ar = m->arena;
  const int n = fd.n, D = fd.d_last;
  const size_t rows = (size_t)B * n, Pn = P.total;
  QMC_PROF(QMC_KC_LOGDET, launch_logdet_bwd(s, B, n, fd.K, at<float>(ws, amat), at<float>(ws, abar), lp));
  const int nch = fd.split ? 2 : 1;
  {
    ::qmc::ProfScope ps_(QMC_KC_ORBITAL, s);
    if (lp) {
      k_psi_add_jas<<<blocks(B), 256, 0, s>>>(B, lp, at<float>(ws, jas));
      QMC_CUDA(cudaGetLastError());
    }
    k_orb_bwd<<<blocks(rows * fd.norb_p), 256, 0, s>>>(
        B, n, fd.n_up, fd.split, fd.K, fd.A, fd.env_abs, fd.env_kind, fd.norb_p, at<float>(ws, abar),
        at<float>(ws, orb), at<float>(ws, rae), at<float>(ws, aevec), ar + fa.env_pi[0], ar + fa.env_sigma[0],
        ar + fa.env_pi[nch - 1], ar + fa.env_sigma[nch - 1], at<float>(ws, orbbar), at<float>(ws, envbar));
    QMC_CUDA(cudaGetLastError());
  }
  for (int c = 0; c < nch; ++c) {
    const int ns = fd.split ? (c == 0 ? fd.n_up : fd.n_dn) : n;
    const int i0 = (fd.split && c == 1) ? fd.n_up : 0;
    ::qmc::ProfScope ps_(QMC_KC_OTHER, s);
    if (fd.env_kind == QMC_ENVELOPE_DIAGONAL)
      k_env_jac_diag<<<blocks((size_t)B * n * fd.A * fd.K), 256, 0, s>>>(
          B, n, i0, ns, fd.K, fd.A, at<float>(ws, envbar), at<float>(ws, aevec), ar + fa.env_pi[c],
          ar + fa.env_sigma[c], J, Pn, P.env_pi[c], P.env_sigma[c]);
    else if (fd.env_kind != QMC_ENVELOPE_NULL)
      k_env_jac<<<blocks((size_t)B * n * fd.A * fd.K), 256, 0, s>>>(B, n, i0, ns, fd.K, fd.A, fd.env_abs,
                                                                   at<float>(ws, envbar), at<float>(ws, rae),
                                                                   ar + fa.env_pi[c], ar + fa.env_sigma[c], J, Pn,
                                                                   P.env_pi[c], P.env_sigma[c]);
    QMC_CUDA(cudaGetLastError());
    QMC_CUDA(jac_outer(s, B, ns, n, i0, hL, D, D, at<float>(ws, orbbar), fd.norb_p, fd.norb, J, Pn, P.orb_k[c]));
    if (taps) {
      k_tap_gather<<<blocks((size_t)B * ns * D), 256, 0, s>>>(B, n, i0, ns, hL, D, D, taps->in(orb_tap[c]));
      k_tap_gather<<<blocks((size_t)B * ns * fd.norb), 256, 0, s>>>(B, n, i0, ns, at<float>(ws, orbbar), fd.norb_p,
                                                                    fd.norb, taps->out(orb_tap[c]));
      QMC_CUDA(cudaGetLastError());
    }
    RowMap map{ns, i0, n, 1};
    QMC_CUDA(launch_gemm_simt(s, B * ns, map, at<float>(ws, orbbar), fd.norb_p, fd.norb_p, nullptr, 0, 0,
                              ar + fa.wt_orb[c], D, D, EpiStore{hbar, D, nullptr}));
  }
  return QMC_OK;
}

static qmc_status psi_forward_save(qmc_model* m, const PsiGradPlan& p, void* ws, const float* electrons,
                                   cudaStream_t s) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const PsiArena& a = m->psi->a;
  const Dims& fd = m->d;
  const ArenaLayout& fa = m->a;
  const float* ar = m->arena;
  const int B = p.B, n = d.n, D = d.D;
  const size_t rows = (size_t)B * n;
  const RowMap rmap{n, 0, n, 1};
  const unsigned wb = (unsigned)((rows + 7) / 8);  // warp-per-row kernels, 8 rows per block
  QMC_PROF(QMC_KC_FEATURES, launch_psi_features(s, B, n, d.n_up, d.A, d.K0p, electrons, ar + fa.atoms,
                                                d.jastrow ? ar + P.alpha_par : nullptr, at<float>(ws, p.x0),
                                                at<float>(ws, p.rae), at<float>(ws, p.aevec), at<float>(ws, p.jas)));
  QMC_PROF(QMC_KC_LAYER0, launch_gemm_simt(s, B * n, rmap, at<float>(ws, p.x0), d.K0p, d.K0p, nullptr, 0, 0,
                                           ar + a.w_in, D, D, EpiStore{at<float>(ws, p.h[0]), D, ar + P.in_b}));
  float* tmp = at<float>(ws, p.tmp);
  for (int l = 0; l < d.L; ++l) {
    float* h = at<float>(ws, p.h[l]);
    {
      ::qmc::ProfScope ps_(QMC_KC_MEANS, s);
      k_psi_ln_fwd<<<wb, 256, 0, s>>>((int)rows, D, h, ar + P.ln0_s[l], ar + P.ln0_b[l], at<float>(ws, p.xn0[l]),
                                     at<float>(ws, p.mu0[l]), at<float>(ws, p.rs0[l]));
      QMC_CUDA(cudaGetLastError());
    }
    QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rmap, at<float>(ws, p.xn0[l]), D, D, nullptr, 0, 0,
                                                   ar + a.w_qkv[l], 3 * D, 3 * D,
                                                   EpiStore{at<float>(ws, p.qkv[l]), 3 * D, ar + a.b_qkv[l]}));
    {
      ::qmc::ProfScope ps_(QMC_KC_PAIR, s);
      const size_t sm = sizeof(float) * (3 * (size_t)n * d.Dh + (size_t)n * n);
      k_psi_attn_save<<<B * d.H, 128, sm, s>>>(n, d.H, d.Dh, at<float>(ws, p.qkv[l]), at<float>(ws, p.pr[l]),
                                               at<float>(ws, p.o[l]));
      QMC_CUDA(cudaGetLastError());
    }
    QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rmap, at<float>(ws, p.o[l]), D, D, nullptr, 0, 0,
                                                   ar + P.o_k[l], D, D, EpiStore{tmp, D, ar + P.o_b[l]}));
    {
      ::qmc::ProfScope ps_(QMC_KC_MEANS, s);
      k_psi_tanh_add<<<blocks(rows * D), 256, 0, s>>>(rows * D, tmp, h, at<float>(ws, p.hm[l]), 0);
      QMC_CUDA(cudaGetLastError());
      k_psi_ln_fwd<<<wb, 256, 0, s>>>((int)rows, D, at<float>(ws, p.hm[l]), ar + P.ln1_s[l], ar + P.ln1_b[l],
                                     at<float>(ws, p.xn1[l]), at<float>(ws, p.mu1[l]), at<float>(ws, p.rs1[l]));
      QMC_CUDA(cudaGetLastError());
    }
    const float* in = at<float>(ws, p.xn1[l]);
    int din = D;
    for (int k = 0; k < d.n_dense; ++k) {
      float* y = at<float>(ws, p.y[l][k]);
      QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rmap, in, din, din, nullptr, 0, 0,
                                                     ar + P.mlp_k[l][k], d.mlp[k], d.mlp[k],
                                                     EpiStore{y, d.mlp[k], ar + P.mlp_b[l][k]}));
      const bool last = k == d.n_dense - 1;
      ::qmc::ProfScope ps_(QMC_KC_MEANS, s);
      k_psi_tanh_add<<<blocks(rows * d.mlp[k]), 256, 0, s>>>(rows * d.mlp[k], y, at<float>(ws, p.hm[l]),
                                                            last ? at<float>(ws, p.h[l + 1]) : nullptr, 1);
      QMC_CUDA(cudaGetLastError());
      in = y;
      din = d.mlp[k];
    }
  }
  return attn_orbitals_fwd(m, B, ws, at<float>(ws, p.h[d.L]), p.amat, p.orb, p.rae, p.aevec, s);
}

static qmc_status psi_backward(qmc_model* m, const PsiGradPlan& p, void* ws, const float* electrons, float* J,
                               float* logpsi, cudaStream_t s, const TapOut* taps = nullptr,
                               const AttnTaps* ti = nullptr) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const PsiArena& a = m->psi->a;
  const Dims& fd = m->d;
  const ArenaLayout& fa = m->a;
  const float* ar = m->arena;
  const int B = p.B, n = d.n, D = d.D;
  const size_t rows = (size_t)B * n, Pn = P.total;
  const RowMap rmap{n, 0, n, 1};
  const unsigned wb = (unsigned)((rows + 7) / 8);
  float* hbar = at<float>(ws, p.hbar);
  QMC_TRY(attn_orbitals_bwd(m, B, ws, at<float>(ws, p.h[d.L]), p.amat, p.orb, p.abar, p.envbar, p.rae, p.aevec,
                            p.orbbar, p.jas, hbar, J, logpsi, s, taps, ti ? ti->orb : nullptr));
  float* hmbar = at<float>(ws, p.hmbar);
  float* zbar = at<float>(ws, p.zbar);
  float* tmp = at<float>(ws, p.tmp);
  float* obar = at<float>(ws, p.obar);
  float* qkvbar = at<float>(ws, p.qkvbar);
  for (int l = d.L - 1; l >= 0; --l) {
    // h[l+1] = hm + y_last: both branches take hbar
    QMC_CUDA(cudaMemcpyAsync(hmbar, hbar, sizeof(float) * rows * D, cudaMemcpyDeviceToDevice, s));
    const float* ybar = hbar;
    for (int k = d.n_dense - 1; k >= 0; --k) {
      const int dout = d.mlp[k], din = k == 0 ? D : d.mlp[k - 1];
      const float* x = k == 0 ? at<float>(ws, p.xn1[l]) : at<float>(ws, p.y[l][k - 1]);
      ::qmc::ProfScope ps_(QMC_KC_STREAM_LAYER, s);
      k_tanh_bwd<<<blocks(rows * dout), 256, 0, s>>>(rows * dout, 1.f, ybar, at<float>(ws, p.y[l][k]), zbar);
      QMC_CUDA(cudaGetLastError());
      QMC_CUDA(jac_outer(s, B, n, n, 0, x, din, din, zbar, dout, dout, J, Pn,
                                                                P.mlp_k[l][k]));
      if (taps) {
        QMC_CUDA(tap_copy(s, taps->in(ti->mlp[l][k]), din, x, din, rows));
        QMC_CUDA(tap_copy(s, taps->out(ti->mlp[l][k]), dout, zbar, dout, rows));
      }
      k_colsum<<<blocks((size_t)B * dout), 256, 0, s>>>(B, n, zbar, dout, dout, nullptr, J, Pn, P.mlp_b[l][k]);
      QMC_CUDA(cudaGetLastError());
      // input cotangent zbar W^T into tmp (the next k's ybar, or the LayerNorm output's)
      QMC_CUDA(launch_gemm_simt(s, B * n, rmap, zbar, dout, dout, nullptr, 0, 0, ar + a.t32_mlp[l][k], din, din,
                                EpiStore{tmp, din, nullptr}));
      ybar = tmp;
    }
    {
      ::qmc::ProfScope ps_(QMC_KC_MEANS, s);
      // LayerNorm 1: parameters and the cotangent of hm (tmp holds the cotangent of xn1)
      k_psi_ln_jac<<<blocks((size_t)B * D), 256, 0, s>>>(B, n, D, at<float>(ws, p.hm[l]), at<float>(ws, p.mu1[l]),
                                                        at<float>(ws, p.rs1[l]), tmp, J, Pn, P.ln1_s[l], P.ln1_b[l]);
      QMC_CUDA(cudaGetLastError());
      k_psi_ln_bwd<<<wb, 256, 0, s>>>((int)rows, D, at<float>(ws, p.hm[l]), at<float>(ws, p.mu1[l]),
                                     at<float>(ws, p.rs1[l]), ar + P.ln1_s[l], tmp, hmbar);
      QMC_CUDA(cudaGetLastError());
    }
    {
      // att = o Wo + bo; hm = h + att
      ::qmc::ProfScope ps_(QMC_KC_STREAM_LAYER, s);
      QMC_CUDA(jac_outer(s, B, n, n, 0, at<float>(ws, p.o[l]), D, D, hmbar, D, D, J,
                                                            Pn, P.o_k[l]));
      if (taps) {
        QMC_CUDA(tap_copy(s, taps->in(ti->o[l]), D, at<float>(ws, p.o[l]), D, rows));
        QMC_CUDA(tap_copy(s, taps->out(ti->o[l]), D, hmbar, D, rows));
      }
      k_colsum<<<blocks((size_t)B * D), 256, 0, s>>>(B, n, hmbar, D, D, nullptr, J, Pn, P.o_b[l]);
      QMC_CUDA(cudaGetLastError());
      QMC_CUDA(launch_gemm_simt(s, B * n, rmap, hmbar, D, D, nullptr, 0, 0, ar + a.t32_o[l], D, D,
                                EpiStore{obar, D, nullptr}));
    }
    {
      ::qmc::ProfScope ps_(QMC_KC_PAIR, s);
      const size_t sm = sizeof(float) * (4 * (size_t)n * d.Dh + 2 * (size_t)n * n);
      k_psi_attn_bwd<<<B * d.H, 128, sm, s>>>(n, d.H, d.Dh, at<float>(ws, p.qkv[l]), at<float>(ws, p.pr[l]), obar,
                                              qkvbar);
      QMC_CUDA(cudaGetLastError());
    }
    {
      ::qmc::ProfScope ps_(QMC_KC_STREAM_LAYER, s);
      const float* xn0 = at<float>(ws, p.xn0[l]);
      const size_t kofs[3] = {P.q_k[l], P.k_k[l], P.v_k[l]}, bofs[3] = {P.q_b[l], P.k_b[l], P.v_b[l]};
      for (int c = 0; c < 3; ++c) {
        QMC_CUDA(jac_outer(s, B, n, n, 0, xn0, D, D, qkvbar + (size_t)c * D, 3 * D, D,
                                                              J, Pn, kofs[c]));
        if (taps) {
          const int tk = c == 0 ? ti->q[l] : (c == 1 ? ti->k[l] : ti->v[l]);
          QMC_CUDA(tap_copy(s, taps->in(tk), D, xn0, D, rows));
          QMC_CUDA(tap_copy(s, taps->out(tk), D, qkvbar + (size_t)c * D, 3 * D, rows));
        }
        k_colsum<<<blocks((size_t)B * D), 256, 0, s>>>(B, n, qkvbar + (size_t)c * D, 3 * D, D, nullptr, J, Pn,
                                                       bofs[c]);
        QMC_CUDA(cudaGetLastError());
      }
      QMC_CUDA(launch_gemm_simt(s, B * n, rmap, qkvbar, 3 * D, 3 * D, nullptr, 0, 0, ar + a.t32_qkv[l], D, D,
                                EpiStore{tmp, D, nullptr}));
    }
    {
      // LayerNorm 0 on h[l]; hbar(h[l]) = hmbar (residual) + its input cotangent
      ::qmc::ProfScope ps_(QMC_KC_MEANS, s);
      k_psi_ln_jac<<<blocks((size_t)B * D), 256, 0, s>>>(B, n, D, at<float>(ws, p.h[l]), at<float>(ws, p.mu0[l]),
                                                        at<float>(ws, p.rs0[l]), tmp, J, Pn, P.ln0_s[l], P.ln0_b[l]);
      QMC_CUDA(cudaGetLastError());
      QMC_CUDA(cudaMemcpyAsync(hbar, hmbar, sizeof(float) * rows * D, cudaMemcpyDeviceToDevice, s));
      k_psi_ln_bwd<<<wb, 256, 0, s>>>((int)rows, D, at<float>(ws, p.h[l]), at<float>(ws, p.mu0[l]),
                                     at<float>(ws, p.rs0[l]), ar + P.ln0_s[l], tmp, hbar);
      QMC_CUDA(cudaGetLastError());
    }
  }
  {
    ::qmc::ProfScope ps_(QMC_KC_LAYER0, s);
    QMC_CUDA(jac_outer(s, B, n, n, 0, at<float>(ws, p.x0), d.K0p, d.K0, hbar, D, D,
                                                             J, Pn, P.in_k));
    k_colsum<<<blocks((size_t)B * D), 256, 0, s>>>(B, n, hbar, D, D, nullptr, J, Pn, P.in_b);
    QMC_CUDA(cudaGetLastError());
    if (taps) {
      QMC_CUDA(tap_copy(s, taps->in(ti->in), d.K0, at<float>(ws, p.x0), d.K0p, rows));
      QMC_CUDA(tap_copy(s, taps->out(ti->in), D, hbar, D, rows));
    }
    if (d.jastrow) {
      k_psi_jas_jac<<<blocks(B), 256, 0, s>>>(B, n, d.n_up, electrons, ar + P.alpha_par, J, Pn, P.alpha_par,
                                              P.alpha_anti);
      QMC_CUDA(cudaGetLastError());
    }
  }
  return QMC_OK;
}

// ------------------------------------------------------------ LapNet adjoint
// Saved activations of a chunk of B walkers: the individual stream hs before
// each local update (hs[l][0] = the layer's query/key input), the update
// outputs u = tanh(hs Wu + bu), the dense stream hd[l] (hd[L] = the backbone
// output), q|k|v with biases, the attention probabilities and output, the
// post-attention residual r and the value update y = tanh(r Wvu + bvu).
struct LapGradPlan {
  int B;
  size_t x0, rae, aevec, jas;
  size_t hs[kPsiMaxLayers][kLapMaxLocal + 1], u[kPsiMaxLayers][kLapMaxLocal], hd[kPsiMaxLayers + 1];
  size_t qkv[kPsiMaxLayers], pr[kPsiMaxLayers], o[kPsiMaxLayers], r[kPsiMaxLayers], y[kPsiMaxLayers];
  size_t amat, orb, abar, envbar, hbar, hsbar, zbar, obar, qkvbar, orbbar, J, total;
};

// y += x
__global__ void k_add_to(size_t count, const float* __restrict__ x, float* __restrict__ y) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < count) y[e] += x[e];
}

static int lap_local(const PsiDims& d, int l) { return l + 1 < d.L ? d.n_local : 0; }

static LapGradPlan make_lap_grad_plan(const qmc_model* m, int B) {
  const PsiDims& d = m->psi->d;
  LapGradPlan p{};
  p.B = B;
  size_t o = 0;
  auto take = [&](size_t floats) { size_t r = o; o += align_up(floats * 4, 256); return r; };
  const size_t rows = (size_t)B * d.n, D = d.D;
  p.x0 = take(rows * d.K0p);
  p.rae = take(rows * d.A);
  p.aevec = take(rows * d.A * 3);
  p.jas = take(B);
  for (int l = 0; l <= d.L; ++l) p.hd[l] = take(rows * D);
  for (int l = 0; l < d.L; ++l) {
    for (int j = 0; j <= lap_local(d, l); ++j) p.hs[l][j] = take(rows * D);
    for (int j = 0; j < lap_local(d, l); ++j) p.u[l][j] = take(rows * D);
    p.qkv[l] = take(rows * 3 * D);
    p.pr[l] = take((size_t)B * d.H * d.n * d.n);
    p.o[l] = take(rows * D);
    p.r[l] = take(rows * D);
    p.y[l] = take(rows * D);
  }
  const size_t am = (size_t)B * d.K * d.n * d.n;
  p.amat = take(am);
  p.orb = take(am);
  p.abar = take(am);
  p.envbar = take(am);
  p.hbar = take(rows * D);
  p.hsbar = take(rows * D);
  p.zbar = take(rows * D);
  p.obar = take(rows * D);
  p.qkvbar = take(rows * 3 * D);
  p.orbbar = take(rows * m->d.norb_p);
  p.J = take((size_t)B * m->psi->p.total);
  p.total = o;
  return p;
}

static qmc_status lap_forward_save(qmc_model* m, const LapGradPlan& p, void* ws, const float* electrons,
                                   cudaStream_t s) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const PsiArena& a = m->psi->a;
  const ArenaLayout& fa = m->a;
  const float* ar = m->arena;
  const int B = p.B, n = d.n, D = d.D;
  const size_t rows = (size_t)B * n;
  const RowMap rmap{n, 0, n, 1};
  QMC_PROF(QMC_KC_FEATURES, launch_psi_features(s, B, n, d.n_up, d.A, d.K0p, electrons, ar + fa.atoms,
                                                d.jastrow ? ar + P.alpha_par : nullptr, at<float>(ws, p.x0),
                                                at<float>(ws, p.rae), at<float>(ws, p.aevec), at<float>(ws, p.jas)));
  QMC_PROF(QMC_KC_LAYER0, launch_gemm_simt(s, B * n, rmap, at<float>(ws, p.x0), d.K0p, d.K0p, nullptr, 0, 0,
                                           ar + a.w_in, D, D, EpiStore{at<float>(ws, p.hd[0]), D, ar + a.lb_in}));
  QMC_CUDA(cudaMemcpyAsync(at<float>(ws, p.hs[0][0]), at<float>(ws, p.hd[0]), sizeof(float) * rows * D,
                           cudaMemcpyDeviceToDevice, s));
  for (int l = 0; l < d.L; ++l) {
    float* qkv = at<float>(ws, p.qkv[l]);
    QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rmap, at<float>(ws, p.hs[l][0]), D, D, nullptr, 0, 0,
                                                   ar + P.qk_k[l], 2 * D, 2 * D,
                                                   EpiStore{qkv, 3 * D, ar + a.b_qkv[l]}));
    QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rmap, at<float>(ws, p.hd[l]), D, D, nullptr, 0, 0,
                                                   ar + P.lv_k[l], D, D,
                                                   EpiStore{qkv + 2 * D, 3 * D, ar + a.b_qkv[l] + 2 * D}));
    const int nl = lap_local(d, l);
    for (int j = 0; j < nl; ++j) {
      float* u = at<float>(ws, p.u[l][j]);
      QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rmap, at<float>(ws, p.hs[l][j]), D, D, nullptr, 0,
                                                     0, ar + P.ul_k[l][j], D, D, EpiStore{u, D, ar + a.lb_ul[l][j]}));
      // u = tanh(u); next hs = hs + u (into the next layer's first state after the last update)
      float* next = j + 1 < nl ? at<float>(ws, p.hs[l][j + 1]) : at<float>(ws, p.hs[l + 1][0]);
      ::qmc::ProfScope ps_(QMC_KC_MEANS, s);
      k_psi_tanh_add<<<blocks(rows * D), 256, 0, s>>>(rows * D, u, at<float>(ws, p.hs[l][j]), next, 1);
      QMC_CUDA(cudaGetLastError());
    }
    if (nl == 0 && l + 1 < d.L)
      QMC_CUDA(cudaMemcpyAsync(at<float>(ws, p.hs[l + 1][0]), at<float>(ws, p.hs[l][0]), sizeof(float) * rows * D,
                               cudaMemcpyDeviceToDevice, s));
    {
      ::qmc::ProfScope ps_(QMC_KC_PAIR, s);
      const size_t sm = sizeof(float) * (3 * (size_t)n * d.Dh + (size_t)n * n);
      k_psi_attn_save<<<B * d.H, 128, sm, s>>>(n, d.H, d.Dh, qkv, at<float>(ws, p.pr[l]), at<float>(ws, p.o[l]));
      QMC_CUDA(cudaGetLastError());
    }
    float* r = at<float>(ws, p.r[l]);
    float* y = at<float>(ws, p.y[l]);
    // r = hd + o Wo + bo
    QMC_CUDA(cudaMemcpyAsync(r, at<float>(ws, p.hd[l]), sizeof(float) * rows * D, cudaMemcpyDeviceToDevice, s));
    QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rmap, at<float>(ws, p.o[l]), D, D, nullptr, 0, 0,
                                                   ar + P.lo_k[l], D, D, EpiStore{r, D, ar + a.lb_o[l], 1}));
    QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, B * n, rmap, r, D, D, nullptr, 0, 0, ar + P.vu_k[l], D, D,
                                                   EpiStore{y, D, ar + a.lb_vu[l]}));
    {
      ::qmc::ProfScope ps_(QMC_KC_MEANS, s);
      k_psi_tanh_add<<<blocks(rows * D), 256, 0, s>>>(rows * D, y, r, at<float>(ws, p.hd[l + 1]), 1);
      QMC_CUDA(cudaGetLastError());
    }
  }
  return attn_orbitals_fwd(m, B, ws, at<float>(ws, p.hd[d.L]), p.amat, p.orb, p.rae, p.aevec, s);
}

static qmc_status lap_backward(qmc_model* m, const LapGradPlan& p, void* ws, const float* electrons, float* J,
                               float* logpsi, cudaStream_t s, const TapOut* taps = nullptr,
                               const AttnTaps* ti = nullptr) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const PsiArena& a = m->psi->a;
  const float* ar = m->arena;
  const int B = p.B, n = d.n, D = d.D;
  const size_t rows = (size_t)B * n, Pn = P.total;
  const RowMap rmap{n, 0, n, 1};
  float* hbar = at<float>(ws, p.hbar);    // cotangent of the dense stream
  float* hsbar = at<float>(ws, p.hsbar);  // cotangent of the individual stream
  float* zbar = at<float>(ws, p.zbar);
  float* obar = at<float>(ws, p.obar);
  float* qkvbar = at<float>(ws, p.qkvbar);
  QMC_TRY(attn_orbitals_bwd(m, B, ws, at<float>(ws, p.hd[d.L]), p.amat, p.orb, p.abar, p.envbar, p.rae, p.aevec,
                            p.orbbar, p.jas, hbar, J, logpsi, s, taps, ti ? ti->orb : nullptr));
  QMC_CUDA(cudaMemsetAsync(hsbar, 0, sizeof(float) * rows * D, s));
  auto tap = [&](int k, const float* x, int in_cols, int ldx, const float* dy, int out_cols, int ldy) -> qmc_status {
    if (!taps) return QMC_OK;
    QMC_CUDA(tap_copy(s, taps->in(k), in_cols, x, ldx, rows));
    QMC_CUDA(tap_copy(s, taps->out(k), out_cols, dy, ldy, rows));
    return QMC_OK;
  };
  auto bias_rows = [&](const float* z, int ldz, int N, size_t off) -> qmc_status {
    if (!d.bb_bias) return QMC_OK;
    k_colsum<<<blocks((size_t)B * N), 256, 0, s>>>(B, n, z, ldz, N, nullptr, J, Pn, off);
    QMC_CUDA(cudaGetLastError());
    return QMC_OK;
  };
  for (int l = d.L - 1; l >= 0; --l) {
    ::qmc::ProfScope ps_(QMC_KC_STREAM_LAYER, s);
    // hd[l+1] = r + y, y = tanh(r Wvu + bvu): rbar = hbar + zbar Wvu^T, zbar = hbar (1 - y^2)
    const float* r = at<float>(ws, p.r[l]);
    k_tanh_bwd<<<blocks(rows * D), 256, 0, s>>>(rows * D, 1.f, hbar, at<float>(ws, p.y[l]), zbar);
    QMC_CUDA(cudaGetLastError());
    QMC_CUDA(jac_outer(s, B, n, n, 0, r, D, D, zbar, D, D, J, Pn, P.vu_k[l]));
    QMC_TRY(bias_rows(zbar, D, D, P.vu_b[l]));
    if (taps) QMC_TRY(tap(ti->vu[l], r, D, D, zbar, D, D));
    QMC_CUDA(launch_gemm_simt(s, B * n, rmap, zbar, D, D, nullptr, 0, 0, ar + a.t32_vu[l], D, D,
                              EpiStore{hbar, D, nullptr, 1}));  // hbar now holds rbar
    // r = hd[l] + o Wo + bo
    QMC_CUDA(jac_outer(s, B, n, n, 0, at<float>(ws, p.o[l]), D, D, hbar, D, D, J, Pn, P.lo_k[l]));
    QMC_TRY(bias_rows(hbar, D, D, P.lo_b[l]));
    if (taps) QMC_TRY(tap(ti->lo[l], at<float>(ws, p.o[l]), D, D, hbar, D, D));
    QMC_CUDA(launch_gemm_simt(s, B * n, rmap, hbar, D, D, nullptr, 0, 0, ar + a.t32_o[l], D, D,
                              EpiStore{obar, D, nullptr}));
    {
      ::qmc::ProfScope ps2_(QMC_KC_PAIR, s);
      const size_t sm = sizeof(float) * (4 * (size_t)n * d.Dh + 2 * (size_t)n * n);
      k_psi_attn_bwd<<<B * d.H, 128, sm, s>>>(n, d.H, d.Dh, at<float>(ws, p.qkv[l]), at<float>(ws, p.pr[l]), obar,
                                              qkvbar);
      QMC_CUDA(cudaGetLastError());
    }
    // v = hd[l] Wv + bv: hd[l]'s cotangent = rbar (residual) + vbar Wv^T
    const float* hd = at<float>(ws, p.hd[l]);
    QMC_CUDA(jac_outer(s, B, n, n, 0, hd, D, D, qkvbar + 2 * D, 3 * D, D, J, Pn, P.lv_k[l]));
    QMC_TRY(bias_rows(qkvbar + 2 * D, 3 * D, D, P.lv_b[l]));
    if (taps) QMC_TRY(tap(ti->lv[l], hd, D, D, qkvbar + 2 * D, D, 3 * D));
    QMC_CUDA(launch_gemm_simt(s, B * n, rmap, qkvbar + 2 * D, 3 * D, D, nullptr, 0, 0, ar + a.t32_v[l], D, D,
                              EpiStore{hbar, D, nullptr, 1}));
    // local updates, last first: hs_{j+1} = hs_j + u_j, u_j = tanh(hs_j Wu_j + bu_j)
    for (int j = lap_local(d, l) - 1; j >= 0; --j) {
      k_tanh_bwd<<<blocks(rows * D), 256, 0, s>>>(rows * D, 1.f, hsbar, at<float>(ws, p.u[l][j]), zbar);
      QMC_CUDA(cudaGetLastError());
      QMC_CUDA(jac_outer(s, B, n, n, 0, at<float>(ws, p.hs[l][j]), D, D, zbar, D, D, J, Pn, P.ul_k[l][j]));
      QMC_TRY(bias_rows(zbar, D, D, P.ul_b[l][j]));
      if (taps) QMC_TRY(tap(ti->ul[l][j], at<float>(ws, p.hs[l][j]), D, D, zbar, D, D));
      QMC_CUDA(launch_gemm_simt(s, B * n, rmap, zbar, D, D, nullptr, 0, 0, ar + a.t32_ul[l][j], D, D,
                                EpiStore{hsbar, D, nullptr, 1}));
    }
    // q|k = hs[l][0] Wqk + bqk
    QMC_CUDA(jac_outer(s, B, n, n, 0, at<float>(ws, p.hs[l][0]), D, D, qkvbar, 3 * D, 2 * D, J, Pn, P.qk_k[l]));
    QMC_TRY(bias_rows(qkvbar, 3 * D, 2 * D, P.qk_b[l]));
    if (taps) QMC_TRY(tap(ti->qk[l], at<float>(ws, p.hs[l][0]), D, D, qkvbar, 2 * D, 3 * D));
    QMC_CUDA(launch_gemm_simt(s, B * n, rmap, qkvbar, 3 * D, 2 * D, nullptr, 0, 0, ar + a.t32_qkv[l], D, D,
                              EpiStore{hsbar, D, nullptr, 1}));
  }
  {
    // both streams start as the input projection
    ::qmc::ProfScope ps_(QMC_KC_LAYER0, s);
    k_add_to<<<blocks(rows * D), 256, 0, s>>>(rows * D, hsbar, hbar);
    QMC_CUDA(cudaGetLastError());
    QMC_CUDA(jac_outer(s, B, n, n, 0, at<float>(ws, p.x0), d.K0p, d.K0, hbar, D, D, J, Pn, P.in_k));
    if (taps) QMC_TRY(tap(ti->in, at<float>(ws, p.x0), d.K0, d.K0p, hbar, D, D));
    if (d.in_bias) {
      k_colsum<<<blocks((size_t)B * D), 256, 0, s>>>(B, n, hbar, D, D, nullptr, J, Pn, P.in_b);
      QMC_CUDA(cudaGetLastError());
    }
    if (d.jastrow) {
      k_psi_jas_jac<<<blocks(B), 256, 0, s>>>(B, n, d.n_up, electrons, ar + P.alpha_par, J, Pn, P.alpha_par,
                                              P.alpha_anti);
      QMC_CUDA(cudaGetLastError());
    }
  }
  return QMC_OK;
}

static size_t attn_grad_total(const qmc_model* m, int B) {
  return m->psi->d.arch == kArchLapNet ? make_lap_grad_plan(m, B).total : make_psi_grad_plan(m, B).total;
}

qmc_status run_psi_grad(qmc_model* m, int batch, const float* electrons, const double* weights, float* per_walker,
                        double* grad, float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s) {
  const PsiDims& pd = m->psi->d;
  if (pd.n > 64 || pd.Dh > 64) {
    set_error("the attention-backbone adjoint supports at most 64 electrons and head width 64");
    return QMC_ERR_SHAPE;
  }
  {
    int dev;
    QMC_CUDA(cudaGetDevice(&dev));
    static int set_dev = -1;
    if (set_dev != dev) {
      QMC_CUDA(cudaFuncSetAttribute(k_psi_attn_save, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
      QMC_CUDA(cudaFuncSetAttribute(k_psi_attn_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
      set_dev = dev;
    }
  }
  const int chunk = psi_grad_chunk(m, batch);
  const size_t need = attn_grad_total(m, chunk);
  if (ws_bytes < need) {
    set_error("workspace too small for the adjoint: %zu bytes given, %zu needed", ws_bytes, need);
    return QMC_ERR_WORKSPACE;
  }
  const size_t P = m->psi->p.total;
  const int n = m->psi->d.n;
  if (grad) QMC_CUDA(cudaMemsetAsync(grad, 0, P * sizeof(double), s));
  for (int w0 = 0; w0 < batch; w0 += chunk) {
    const int B = std::min(chunk, batch - w0);
    const bool lapnet = pd.arch == kArchLapNet;
    const PsiGradPlan q = lapnet ? PsiGradPlan{} : make_psi_grad_plan(m, B);
    const LapGradPlan ql = lapnet ? make_lap_grad_plan(m, B) : LapGradPlan{};
    float* J = per_walker ? per_walker + (size_t)w0 * P : at<float>(ws, lapnet ? ql.J : q.J);
    // parameters without a term (the Jastrow when it is off) stay zero
    QMC_CUDA(cudaMemsetAsync(J, 0, sizeof(float) * B * P, s));
    const float* x = electrons + (size_t)w0 * n * 3;
    if (lapnet) {
      QMC_TRY(lap_forward_save(m, ql, ws, x, s));
      QMC_TRY(lap_backward(m, ql, ws, x, J, logpsi ? logpsi + w0 : nullptr, s));
    } else {
      QMC_TRY(psi_forward_save(m, q, ws, x, s));
      QMC_TRY(psi_backward(m, q, ws, x, J, logpsi ? logpsi + w0 : nullptr, s));
    }
    if (grad && weights) {
      ::qmc::ProfScope ps_(QMC_KC_OTHER, s);
      k_weighted_sum<<<blocks(P), 256, 0, s>>>(B, P, J, weights + w0, grad);
      QMC_CUDA(cudaGetLastError());
    }
  }
  return QMC_OK;
}

// Layer taps of a Psiformer / LapNet model: the adjoint chunk by chunk with
// each dense layer's inputs and output cotangents copied out as they are
// formed, then the diagonal taps from the chunk's Jacobian rows.
qmc_status run_attn_grad_taps(qmc_model* m, int batch, const float* electrons, float* taps, size_t taps_floats,
                              float* logpsi, void* ws, size_t ws_bytes, cudaStream_t s) {
  const PsiDims& pd = m->psi->d;
  if (pd.n > 64 || pd.Dh > 64) {
    set_error("the attention-backbone adjoint supports at most 64 electrons and head width 64");
    return QMC_ERR_SHAPE;
  }
  {
    int dev;
    QMC_CUDA(cudaGetDevice(&dev));
    static int set_dev = -1;
    if (set_dev != dev) {
      QMC_CUDA(cudaFuncSetAttribute(k_psi_attn_save, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
      QMC_CUDA(cudaFuncSetAttribute(k_psi_attn_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
      set_dev = dev;
    }
  }
  const int chunk = psi_grad_chunk(m, batch);
  const size_t need = attn_grad_total(m, chunk);
  if (ws_bytes < need) {
    set_error("workspace too small for the adjoint: %zu bytes given, %zu needed", ws_bytes, need);
    return QMC_ERR_WORKSPACE;
  }
  const AttnTaps ti = make_attn_taps(m, batch);
  const TapPlan& tp = ti.plan;
  if (taps_floats < tp.total) {
    set_error("taps buffer too small: %zu floats given, %zu needed", taps_floats, tp.total);
    return QMC_ERR_WORKSPACE;
  }
  const size_t P = m->psi->p.total;
  const int n = pd.n;
  const bool lapnet = pd.arch == kArchLapNet;
  for (int w0 = 0; w0 < batch; w0 += chunk) {
    const int B = std::min(chunk, batch - w0);
    const PsiGradPlan q = lapnet ? PsiGradPlan{} : make_psi_grad_plan(m, B);
    const LapGradPlan ql = lapnet ? make_lap_grad_plan(m, B) : LapGradPlan{};
    float* J = at<float>(ws, lapnet ? ql.J : q.J);
    QMC_CUDA(cudaMemsetAsync(J, 0, sizeof(float) * B * P, s));
    TapOut to;
    to.base = taps;
    to.plan = &tp;
    to.w0 = w0;
    const float* x = electrons + (size_t)w0 * n * 3;
    float* lp = logpsi ? logpsi + w0 : nullptr;
    if (lapnet) {
      QMC_TRY(lap_forward_save(m, ql, ws, x, s));
      QMC_TRY(lap_backward(m, ql, ws, x, J, lp, s, &to, &ti));
    } else {
      QMC_TRY(psi_forward_save(m, q, ws, x, s));
      QMC_TRY(psi_backward(m, q, ws, x, J, lp, s, &to, &ti));
    }
    for (int k = 0; k < tp.count; ++k) {
      const qmc_layer_tap& t = tp.t[k];
      if (t.kind != QMC_TAP_DIAGONAL) continue;
      QMC_CUDA(cudaMemcpy2DAsync(to.out(k), sizeof(float) * t.out_cols, J + t.kernel_offset, sizeof(float) * P,
                                 sizeof(float) * t.out_cols, B, cudaMemcpyDeviceToDevice, s));
    }
  }
  return QMC_OK;
}

int attn_layer_taps(const qmc_model* m, int batch, qmc_layer_tap* taps, int max_taps, size_t* total) {
  const AttnTaps ti = make_attn_taps(m, batch);
  for (int k = 0; k < ti.plan.count && k < max_taps; ++k) taps[k] = ti.plan.t[k];
  if (total) *total = ti.plan.total;
  return ti.plan.count;
}

}  // namespace qmc
