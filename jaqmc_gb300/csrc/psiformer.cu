// Psiformer + SimpleEE Jastrow, value path: log|psi| of a walker batch and,
// through the shared MH driver, the all-electron Metropolis-Hastings step.
//
//   features (rescaled ae features + spin)      k_psi_features
//   x = Dense(features)                          GEMM + k_psi_row
//   per layer (Pre-LN, backbone/psiformer.py:61-99):
//     xn = LN0(x)                                (fused into the previous row kernel)
//     qkv = xn Wqkv                              one GEMM, 3D outputs
//     att = MHA(qkv + bqkv)                      k_psi_attention, one block per (walker, head)
//     x += att Wo + bo ; xn = LN1(x)             GEMM + k_psi_row
//     h = tanh(xn W_k + b_k) ... ; x += h        GEMMs + k_psi_row
//   orbitals x envelope, LU, log-sum-exp         shared with FermiNet
//   log|psi| += Jastrow                          k_psi_add
//
// GEMMs are plain stores: split-BF16 tcgen05 (mixed form) or FP32 SIMT; bias,
// tanh, residual, LayerNorm and the operand format of the next GEMM are one
// warp-per-row kernel.
#include <algorithm>
#include <cmath>
#include <utility>

#include "gemm_simt.cuh"
#include "kernels.cuh"
#include "profile.cuh"
#include "psiformer.cuh"
#include "stream_tc.cuh"

#define QMC_PROF(cls, call)         \
  do {                              \
    ::qmc::ProfScope ps_((cls), s); \
    QMC_CUDA(call);                 \
  } while (0)
#define QMC_PROF_TRY(cls, call)     \
  do {                              \
    ::qmc::ProfScope ps_((cls), s); \
    QMC_TRY(call);                  \
  } while (0)

namespace qmc {

template <typename T>
static T* at(void* ws, size_t off) { return reinterpret_cast<T*>(static_cast<char*>(ws) + off); }

// ------------------------------------------------------------------ kernels
// One block (256 threads) per walker.  X0 row (w, i): per atom
// [log(1+r), vec * log(1+r) / r] (src/jaqmc/wavefunction/input/atomic.py:58-66),
// then the spin (+1 up, -1 down, backbone/psiformer.py:170-176), zeros up to
// K0p.  rae / aevec feed the envelope.  jas[w] is the SimpleEE Jastrow
// (src/jaqmc/wavefunction/jastrow.py:48-122), reduced in a fixed order.
__global__ void __launch_bounds__(256) k_psi_features(int n, int n_up, int A, int K0p, const float* __restrict__ x,
                                                      const float* __restrict__ atoms,
                                                      const float* __restrict__ alpha, float* __restrict__ X0,
                                                      float* __restrict__ rae, float* __restrict__ aevec,
                                                      float* __restrict__ jas) {
  __shared__ float red[256];
  extern __shared__ float xs[];  // [n][3]
  const int w = blockIdx.x;
  for (int e = threadIdx.x; e < 3 * n; e += blockDim.x) xs[e] = x[(size_t)w * 3 * n + e];
  __syncthreads();
  for (int e = threadIdx.x; e < n * K0p; e += blockDim.x) {
    const int i = e / K0p, c = e % K0p;
    float v = 0.f;
    if (c < 4 * A) {
      const int I = c >> 2, q = c & 3;
      const float dx = xs[3 * i] - atoms[3 * I], dy = xs[3 * i + 1] - atoms[3 * I + 1],
                  dz = xs[3 * i + 2] - atoms[3 * I + 2];
      const float r = sqrtf(dx * dx + dy * dy + dz * dz);
      const float lr = log1pf(r);
      v = q == 0 ? lr : (q == 1 ? dx : q == 2 ? dy : dz) * lr / r;
    } else if (c == 4 * A) {
      v = i < n_up ? 1.f : -1.f;
    }
    X0[((size_t)w * n + i) * K0p + c] = v;
  }
  for (int e = threadIdx.x; e < n * A; e += blockDim.x) {
    const int i = e / A, I = e % A;
    const float dx = xs[3 * i] - atoms[3 * I], dy = xs[3 * i + 1] - atoms[3 * I + 1],
                dz = xs[3 * i + 2] - atoms[3 * I + 2];
    const size_t o = (size_t)w * n * A + e;
    rae[o] = sqrtf(dx * dx + dy * dy + dz * dz);
    aevec[3 * o] = dx;
    aevec[3 * o + 1] = dy;
    aevec[3 * o + 2] = dz;
  }
  float acc = 0.f;
  if (alpha) {
    const float ap = alpha[0], aa = alpha[1];
    for (int p = threadIdx.x; p < n * n; p += blockDim.x) {
      const int i = p / n, j = p % n;
      if (j <= i) continue;
      const float dx = xs[3 * i] - xs[3 * j], dy = xs[3 * i + 1] - xs[3 * j + 1], dz = xs[3 * i + 2] - xs[3 * j + 2];
      const float r = sqrtf(dx * dx + dy * dy + dz * dz);
      const bool same = (i < n_up) == (j < n_up);
      acc += same ? -(0.25f * ap * ap) / (ap + r) : -(0.5f * aa * aa) / (aa + r);
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) jas[w] = red[0];
}

// One warp per row of D <= 512 features (multiple of 32):
//   v = z + bias; v = tanh(v) if act; v += x if resid; x = v if write_x;
//   out = LayerNorm(v) (eps 1e-5, biased two-pass variance) if ln_s, else v.
template <class Out>
__global__ void k_psi_row(int rows, int D, const float* __restrict__ z, int ldz, const float* __restrict__ bias,
                          int act, float* __restrict__ x, int resid, int write_x, const float* __restrict__ ln_s,
                          const float* __restrict__ ln_b, Out out) {
  constexpr int kMax = 16;
  const int lane = threadIdx.x & 31;
  const size_t row = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= (size_t)rows) return;
  const int per = D >> 5;
  float v[kMax];
  float sum = 0.f;
#pragma unroll
  for (int k = 0; k < kMax; ++k) {
    if (k < per) {
      const int f = lane + 32 * k;
      float t = z[row * ldz + f] + bias[f];
      if (act) t = tanhf(t);
      if (resid) t += x[row * D + f];
      if (write_x) x[row * D + f] = t;
      v[k] = t;
      sum += t;
    }
  }
  if (!ln_s) {
#pragma unroll
    for (int k = 0; k < kMax; ++k)
      if (k < per) out.put(row, lane + 32 * k, v[k]);
    return;
  }
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  const float mean = sum / (float)D;
  float sq = 0.f;
#pragma unroll
  for (int k = 0; k < kMax; ++k)
    if (k < per) sq += (v[k] - mean) * (v[k] - mean);
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
  const float inv = rsqrtf(sq / (float)D + 1e-5f);
#pragma unroll
  for (int k = 0; k < kMax; ++k) {
    if (k < per) {
      const int f = lane + 32 * k;
      out.put(row, f, (v[k] - mean) * inv * ln_s[f] + ln_b[f]);
    }
  }
}

// Multi-head dot-product attention of one (walker, head) per block
// (flax MultiHeadDotProductAttention semantics, backbone/psiformer.py:74-81):
// q, k, v = projections + biases, q / sqrt(Dh), softmax over keys, o = p v.
// Scores and outputs are computed in 2 x 4 register tiles from 16-byte shared
// loads.  A thread's four keys (and its two query rows) are strided, so the
// eight lanes of a 16-byte access phase read consecutive rows and distinct
// banks.  Rows past n are zero.
struct AttnShape {
  int n, Dh, n2, np, ld, lds;
  __host__ __device__ AttnShape(int n_, int Dh_) : n(n_), Dh(Dh_) {
    n2 = (n + 1) / 2 * 2;  // query rows padded to pairs
    np = (n + 3) / 4 * 4;  // key / value rows padded to quads
    ld = Dh + 4;           // row stride (16-byte aligned rows)
    lds = np + 1;          // score row stride
  }
  __host__ __device__ size_t floats() const {
    return (size_t)(n2 + 2 * np) * ld + (size_t)n2 * lds;
  }
};

template <class Out>
__global__ void __launch_bounds__(128) k_psi_attention(int n, int H, int Dh, const float* __restrict__ qkv,
                                                       const float* __restrict__ bqkv, Out out) {
  extern __shared__ __align__(16) float sa[];
  const AttnShape sh(n, Dh);
  const int ld = sh.ld, lds = sh.lds, n2 = sh.n2, np = sh.np;
  float* Q = sa;
  float* Kt = Q + (size_t)n2 * ld;
  float* V = Kt + (size_t)np * ld;
  float* S = V + (size_t)np * ld;
  const int w = blockIdx.x / H, h = blockIdx.x % H;
  const int D = H * Dh;
  const float scale = 1.0f / sqrtf((float)Dh);
  // 16-byte loads of q, k, v (Dh, D and the row strides are multiples of 4)
  const int dq = Dh / 4;
#pragma unroll 2
  for (int e = threadIdx.x; e < np * dq; e += blockDim.x) {
    const int i = e / dq, d = 4 * (e % dq);
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f), k = q, v = q;
    if (i < n) {
      const float* r = qkv + ((size_t)w * n + i) * 3 * D + h * Dh + d;
      const int c = h * Dh + d;
      const float4 rq = *reinterpret_cast<const float4*>(r), rk = *reinterpret_cast<const float4*>(r + D),
                   rv = *reinterpret_cast<const float4*>(r + 2 * D);
      const float4 bq = *reinterpret_cast<const float4*>(bqkv + c),
                   bk = *reinterpret_cast<const float4*>(bqkv + D + c),
                   bv = *reinterpret_cast<const float4*>(bqkv + 2 * D + c);
      q = make_float4((rq.x + bq.x) * scale, (rq.y + bq.y) * scale, (rq.z + bq.z) * scale, (rq.w + bq.w) * scale);
      k = make_float4(rk.x + bk.x, rk.y + bk.y, rk.z + bk.z, rk.w + bk.w);
      v = make_float4(rv.x + bv.x, rv.y + bv.y, rv.z + bv.z, rv.w + bv.w);
    }
    if (i < n2) *reinterpret_cast<float4*>(Q + i * ld + d) = q;
    *reinterpret_cast<float4*>(Kt + i * ld + d) = k;
    *reinterpret_cast<float4*>(V + i * ld + d) = v;
  }
  __syncthreads();
  // scores: thread (ti, tj) -> rows {ti, ti + n2/2} x keys {tj + c * np/4}
  const int hi = n2 / 2, hj = np / 4;
  for (int t = threadIdx.x; t < hi * hj; t += blockDim.x) {
    const int ti = t / hj, tj = t % hj;
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    for (int d = 0; d < Dh; d += 4) {
      const float4 q0 = *reinterpret_cast<const float4*>(Q + ti * ld + d);
      const float4 q1 = *reinterpret_cast<const float4*>(Q + (ti + hi) * ld + d);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float4 kk = *reinterpret_cast<const float4*>(Kt + (tj + c * hj) * ld + d);
        acc[0][c] = fmaf(q0.x, kk.x, fmaf(q0.y, kk.y, fmaf(q0.z, kk.z, fmaf(q0.w, kk.w, acc[0][c]))));
        acc[1][c] = fmaf(q1.x, kk.x, fmaf(q1.y, kk.y, fmaf(q1.z, kk.z, fmaf(q1.w, kk.w, acc[1][c]))));
      }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      S[ti * lds + tj + c * hj] = acc[0][c];
      S[(ti + hi) * lds + tj + c * hj] = acc[1][c];
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int i = threadIdx.x >> 5; i < n; i += nw) {
    float mx = -INFINITY;
    for (int j = lane; j < n; j += 32) mx = fmaxf(mx, S[i * lds + j]);
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    float sum = 0.f;
    for (int j = lane; j < n; j += 32) {
      const float e = expf(S[i * lds + j] - mx);
      S[i * lds + j] = e;
      sum += e;
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    const float inv = 1.0f / sum;
    for (int j = lane; j < n; j += 32) S[i * lds + j] *= inv;
  }
  __syncthreads();
  // outputs: thread (ti, td) -> rows {ti, ti + n2/2} x features 4 td .. 4 td + 3
  const int hd = Dh / 4;
  for (int t = threadIdx.x; t < hi * hd; t += blockDim.x) {
    const int ti = t / hd, d0 = 4 * (t % hd);
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    for (int j = 0; j < n; ++j) {
      const float p0 = S[ti * lds + j], p1 = S[(ti + hi) * lds + j];
      const float4 v = *reinterpret_cast<const float4*>(V + j * ld + d0);
      acc[0][0] = fmaf(p0, v.x, acc[0][0]);
      acc[0][1] = fmaf(p0, v.y, acc[0][1]);
      acc[0][2] = fmaf(p0, v.z, acc[0][2]);
      acc[0][3] = fmaf(p0, v.w, acc[0][3]);
      acc[1][0] = fmaf(p1, v.x, acc[1][0]);
      acc[1][1] = fmaf(p1, v.y, acc[1][1]);
      acc[1][2] = fmaf(p1, v.z, acc[1][2]);
      acc[1][3] = fmaf(p1, v.w, acc[1][3]);
    }
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      const int i = ti + a * hi;
      if (i < n)
#pragma unroll
        for (int c = 0; c < 4; ++c) out.put((size_t)w * n + i, h * Dh + d0 + c, acc[a][c]);
    }
  }
}

__global__ void k_psi_add(int B, float* __restrict__ lp, const float* __restrict__ jas) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < B) lp[w] += jas[w];
}

static size_t attention_smem(int n, int Dh) { return sizeof(float) * AttnShape(n, Dh).floats(); }

cudaError_t launch_psi_features(cudaStream_t s, int B, int n, int n_up, int A, int K0p, const float* x,
                                const float* atoms, const float* alpha, float* X0, float* rae, float* aevec,
                                float* jas) {
  k_psi_features<<<B, 256, sizeof(float) * 3 * n, s>>>(n, n_up, A, K0p, x, atoms, alpha, X0, rae, aevec, jas);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ host side
PsiPlan psi_make_plan(const qmc_model* m, int B) {
  const PsiDims& d = m->psi->d;
  PsiPlan pp{};
  Plan& p = pp.base;
  p.B = B;
  p.T = 1;
  p.Tp = 1;
  p.P2 = 1;
  p.K0p = d.K0p;
  p.mixed = m->precision == QMC_PRECISION_MIXED_BF16;
  p.act_bytes = 4;
  const size_t rows = (size_t)B * d.n;
  int W = d.D;
  for (int k = 0; k < d.n_dense; ++k) W = std::max(W, d.mlp[k]);
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += align_up(bytes, 256); return r; };
  p.x0 = take(rows * d.K0p * 4);
  p.h1[0] = p.h1[1] = take(rows * d.D * 4);
  p.h1_plane = rows * d.D;
  const size_t env = (size_t)B * d.K * d.n * d.n * 4;
  p.h2[0] = take(env);  // envelope factors of the value-only LU path
  p.h2[1] = p.g1 = p.gb = p.g2 = o;
  p.rae = take(rows * d.A * 4);
  p.aevec = take(rows * d.A * 12);
  p.amat = take(env);
  p.pe = take((size_t)B * 4);
  p.lpsi = take((size_t)B * 4);
  p.sgn = take((size_t)B * 4);
  p.xp = take(rows * 12);
  p.lp = take((size_t)B * 4);
  p.refac = take(16);
  p.redo = take((size_t)B);
  pp.x = take(rows * d.D * 4);
  pp.in_plane = rows * W;
  pp.xn = take(rows * W * 4);
  pp.att = take(rows * W * 4);
  pp.z = take(rows * std::max(3 * d.D, W) * 4);
  pp.jas = take((size_t)B * 4);
  if (d.arch == kArchLapNet) {
    pp.x2 = take(rows * d.D * 4);
    pp.xn2 = take(rows * W * 4);
    pp.z2 = take(rows * d.D * 4);
  }
  p.dmax = d.D;
  p.total = o;
  return pp;
}

// out[rows][n_out] (row stride ldo; default the z buffer, ldo = n_out) =
// X[rows][k] W[k][n_out] (X: GEMM-input buffer at `xoff`)
static qmc_status psi_gemm(qmc_model* m, const PsiPlan& pp, void* ws, cudaStream_t s, size_t xoff, int k,
                           size_t w_f32, size_t t_bf16, int n_out, float* out = nullptr, int ldo = 0) {
  const int rows = pp.base.B * m->psi->d.n * pp.base.Tp;
  float* z = out ? out : at<float>(ws, pp.z);
  const int ld = ldo > 0 ? ldo : n_out;
  if (pp.base.mixed) {
    TcStoreArgs a{rows, at<__nv_bfloat16>(ws, xoff), k, pp.in_plane, m->arena_bf16 + t_bf16, n_out, z, m->dev_err};
    a.ld_out = ld;
    QMC_PROF_TRY(QMC_KC_STREAM_LAYER, tc_store_gemm(s, a));
  } else {
    const RowMap map{1, 0, 1, 1};
    QMC_PROF(QMC_KC_STREAM_LAYER, launch_gemm_simt(s, rows, map, at<float>(ws, xoff), k, k, nullptr, 0, 0,
                                                   m->arena + w_f32, n_out, n_out, EpiStore{z, ld, nullptr}));
  }
  return QMC_OK;
}

template <class Out>
static cudaError_t launch_row(cudaStream_t s, int rows, int D, const float* z, int ldz, const float* bias, int act,
                              float* x, int resid, int write_x, const float* ln_s, const float* ln_b, Out out) {
  const int wpb = 8;
  k_psi_row<Out><<<(unsigned)((rows + wpb - 1) / wpb), 32 * wpb, 0, s>>>(rows, D, z, ldz, bias, act, x, resid,
                                                                        write_x, ln_s, ln_b, out);
  return cudaGetLastError();
}

template <class Out>
static cudaError_t launch_attention(cudaStream_t s, int B, int n, int H, int Dh, const float* qkv,
                                    const float* bqkv, Out out) {
  const size_t sm = attention_smem(n, Dh);
  static int attr_dev = -1;
  int dev;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (sm > 48 * 1024 && attr_dev != dev) {
    e = cudaFuncSetAttribute(k_psi_attention<Out>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    attr_dev = dev;
  }
  k_psi_attention<Out><<<(unsigned)(B * H), 128, sm, s>>>(n, H, Dh, qkv, bqkv, out);
  return cudaGetLastError();
}

template <class Out>
static qmc_status psi_backbone(qmc_model* m, const PsiPlan& pp, void* ws, cudaStream_t s,
                               Out (*fmt)(void*, const PsiPlan&, size_t, int)) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const PsiArena& a = m->psi->a;
  const float* ar = m->arena;
  const int B = pp.base.B, rows = B * d.n, D = d.D;
  float* x = at<float>(ws, pp.x);
  float* z = at<float>(ws, pp.z);
  // input Dense (FP32 SIMT in both forms: K = 4A + 1 is small)
  {
    const RowMap map{1, 0, 1, 1};
    QMC_PROF(QMC_KC_LAYER0, launch_gemm_simt(s, rows, map, at<float>(ws, pp.base.x0), d.K0p, d.K0p, nullptr, 0, 0,
                                             ar + a.w_in, D, D, EpiStore{z, D, nullptr}));
  }
  QMC_PROF(QMC_KC_LAYER0, launch_row(s, rows, D, z, D, ar + P.in_b, 0, x, 0, 1, ar + P.ln0_s[0], ar + P.ln0_b[0],
                                     fmt(ws, pp, pp.xn, D)));
  for (int l = 0; l < d.L; ++l) {
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn, D, a.w_qkv[l], a.t_qkv[l], 3 * D));
    QMC_PROF(QMC_KC_PAIR, launch_attention(s, B, d.n, d.H, d.Dh, z, ar + a.b_qkv[l], fmt(ws, pp, pp.att, D)));
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.att, D, P.o_k[l], a.t_o[l], D));
    QMC_PROF(QMC_KC_MEANS, launch_row(s, rows, D, z, D, ar + P.o_b[l], 0, x, 1, 1, ar + P.ln1_s[l], ar + P.ln1_b[l],
                                      fmt(ws, pp, pp.xn, D)));
    size_t in = pp.xn, other = pp.att;
    int din = D;
    for (int k = 0; k < d.n_dense; ++k) {
      const int dout = d.mlp[k];
      QMC_TRY(psi_gemm(m, pp, ws, s, in, din, P.mlp_k[l][k], a.t_mlp[l][k], dout));
      if (k + 1 < d.n_dense) {
        QMC_PROF(QMC_KC_MEANS, launch_row(s, rows, dout, z, dout, ar + P.mlp_b[l][k], 1, x, 0, 0, nullptr, nullptr,
                                          fmt(ws, pp, other, dout)));
        std::swap(in, other);
        din = dout;
      } else if (l + 1 < d.L) {
        QMC_PROF(QMC_KC_MEANS, launch_row(s, rows, D, z, D, ar + P.mlp_b[l][k], 1, x, 1, 1, ar + P.ln0_s[l + 1],
                                          ar + P.ln0_b[l + 1], fmt(ws, pp, pp.xn, D)));
      } else {  // backbone output, in the orbital GEMM's operand format
        QMC_PROF(QMC_KC_MEANS, launch_row(s, rows, D, z, D, ar + P.mlp_b[l][k], 1, x, 1, 1, nullptr, nullptr,
                                          fmt(ws, pp, pp.base.h1[0], D)));
      }
    }
  }
  return QMC_OK;
}

// LapNet backbone, value pass (src/jaqmc/wavefunction/backbone/lapnet/
// _backbone.py:68-150, no LayerNorm).  Two residual streams: hs (x2, GEMM
// operand xn2) gives queries and keys and takes the local updates; hd (x,
// operand xn) gives values and takes the attention and value-update
// residuals.  Per layer:
//   z[:, 0:2D]  = hs Wqk                      (before the local updates)
//   hs += tanh(hs Wu_j + bu_j), j < n_local   (not in the last layer)
//   z[:, 2D:3D] = hd Wv
//   att = MHA(z + [bqk | bv])                 the Psiformer attention kernel
//   r = hd + att Wo + bo;  hd = r + tanh(r Wvu + bvu)
template <class Out>
static qmc_status lapnet_backbone(qmc_model* m, const PsiPlan& pp, void* ws, cudaStream_t s,
                                  Out (*fmt)(void*, const PsiPlan&, size_t, int)) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const PsiArena& a = m->psi->a;
  const float* ar = m->arena;
  const int B = pp.base.B, rows = B * d.n, D = d.D;
  float* x = at<float>(ws, pp.x);
  float* x2 = at<float>(ws, pp.x2);
  float* z = at<float>(ws, pp.z);
  float* z2 = at<float>(ws, pp.z2);
  {
    const RowMap map{1, 0, 1, 1};
    QMC_PROF(QMC_KC_LAYER0, launch_gemm_simt(s, rows, map, at<float>(ws, pp.base.x0), d.K0p, d.K0p, nullptr, 0, 0,
                                             ar + a.w_in, D, D, EpiStore{z, D, nullptr}));
  }
  QMC_PROF(QMC_KC_LAYER0, launch_row(s, rows, D, z, D, ar + a.lb_in, 0, x, 0, 1, nullptr, nullptr,
                                     fmt(ws, pp, pp.xn, D)));
  QMC_PROF(QMC_KC_LAYER0, launch_row(s, rows, D, z, D, ar + a.lb_in, 0, x2, 0, 1, nullptr, nullptr,
                                     fmt(ws, pp, pp.xn2, D)));
  for (int l = 0; l < d.L; ++l) {
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn2, D, P.qk_k[l], a.t_qkv[l], 2 * D, z, 3 * D));
    for (int j = 0; l + 1 < d.L && j < d.n_local; ++j) {
      QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn2, D, P.ul_k[l][j], a.t_ul[l][j], D, z2, D));
      QMC_PROF(QMC_KC_MEANS, launch_row(s, rows, D, z2, D, ar + a.lb_ul[l][j], 1, x2, 1, 1, nullptr, nullptr,
                                        fmt(ws, pp, pp.xn2, D)));
    }
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn, D, P.lv_k[l], a.t_v[l], D, z + 2 * D, 3 * D));
    QMC_PROF(QMC_KC_PAIR, launch_attention(s, B, d.n, d.H, d.Dh, z, ar + a.b_qkv[l], fmt(ws, pp, pp.att, D)));
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.att, D, P.lo_k[l], a.t_o[l], D));
    QMC_PROF(QMC_KC_MEANS, launch_row(s, rows, D, z, D, ar + a.lb_o[l], 0, x, 1, 1, nullptr, nullptr,
                                      fmt(ws, pp, pp.xn, D)));
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn, D, P.vu_k[l], a.t_vu[l], D));
    QMC_PROF(QMC_KC_MEANS, launch_row(s, rows, D, z, D, ar + a.lb_vu[l], 1, x, 1, 1, nullptr, nullptr,
                                      fmt(ws, pp, l + 1 < d.L ? pp.xn : pp.base.h1[0], D)));
  }
  return QMC_OK;
}

static StSplit fmt_split(void* ws, const PsiPlan& pp, size_t off, int ld) {
  return StSplit{at<__nv_bfloat16>(ws, off), ld, off == pp.base.h1[0] ? pp.base.h1_plane : pp.in_plane};
}
static StF32 fmt_f32(void* ws, const PsiPlan&, size_t off, int ld) { return StF32{at<float>(ws, off), ld}; }

qmc_status psi_evaluate(qmc_model* m, const PsiPlan& pp, void* ws, const float* electrons, float* logpsi,
                        float* sign, uint8_t* flags, cudaStream_t s) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const Plan& p = pp.base;
  const size_t sm = sizeof(float) * 3 * d.n;
  QMC_PROF(QMC_KC_FEATURES,
           (k_psi_features<<<p.B, 256, sm, s>>>(d.n, d.n_up, d.A, d.K0p, electrons, m->arena + m->a.atoms,
                                                d.jastrow ? m->arena + P.alpha_par : nullptr, at<float>(ws, p.x0),
                                                at<float>(ws, p.rae), at<float>(ws, p.aevec), at<float>(ws, pp.jas)),
            cudaGetLastError()));
  if (d.arch == kArchLapNet) {
    if (p.mixed) QMC_TRY(lapnet_backbone<StSplit>(m, pp, ws, s, fmt_split));
    else QMC_TRY(lapnet_backbone<StF32>(m, pp, ws, s, fmt_f32));
  } else {
    if (p.mixed) QMC_TRY(psi_backbone<StSplit>(m, pp, ws, s, fmt_split));
    else QMC_TRY(psi_backbone<StF32>(m, pp, ws, s, fmt_f32));
  }
  QMC_TRY(run_orbitals(m, p, ws, 0, s));
  QMC_TRY(run_logdet(m, p, ws, nullptr, logpsi, sign, nullptr, nullptr, flags, s));
  QMC_PROF(QMC_KC_OTHER, (k_psi_add<<<(p.B + 255) / 256, 256, 0, s>>>(p.B, logpsi, at<float>(ws, pp.jas)),
                          cudaGetLastError()));
  return QMC_OK;
}

// ------------------------------------------------------------ forward Laplacian
PsiPlan psi_fl_plan(const qmc_model* m, int B) {
  const PsiDims& d = m->psi->d;
  PsiPlan pp{};
  Plan& p = pp.base;
  p.B = B;
  p.mixed = m->precision == QMC_PRECISION_MIXED_BF16;
  p.T = 3 * d.n + 2;
  p.Tp = p.mixed ? tc_padded_tangents(p.T) : p.T;
  p.P2 = 1;
  p.K0p = d.K0p;
  p.act_bytes = 4;
  const size_t rows = (size_t)B * d.n * p.Tp;
  int W = d.D;
  for (int k = 0; k < d.n_dense; ++k) W = std::max(W, d.mlp[k]);
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += align_up(bytes, 256); return r; };
  p.x0 = take(rows * d.K0p * 4);
  pp.x = take(rows * d.D * 4);
  pp.in_plane = rows * W;
  pp.xn = take(rows * W * 4);
  pp.att = take(rows * W * 4);
  // the backbone output (orbital GEMM operand) reuses the attention buffer,
  // free once the last layer's MLP has read it
  p.h1[0] = p.h1[1] = pp.att;
  p.h1_plane = pp.in_plane;
  pp.z = take(rows * std::max(3 * d.D, W) * 4);
  p.rae = take((size_t)B * d.n * d.A * 4);
  p.aevec = take((size_t)B * d.n * d.A * 12);
  p.amat = take((size_t)B * d.K * p.Tp * d.n * d.n * 4);
  p.pe = take((size_t)B * 4);
  p.lpsi = take((size_t)B * 4);
  p.sgn = take((size_t)B * 4);
  p.refac = take(16);
  p.redo = take(logdet_fl_scratch_bytes(B, d.K, p.T));
  pp.jas = take((size_t)B * 4);
  pp.jgl = take((size_t)B * (3 * d.n + 1) * 4);
  if (d.arch == kArchLapNet) {
    pp.x2 = take(rows * d.D * 4);
    pp.xn2 = take(rows * W * 4);
    pp.z2 = take(rows * d.D * 4);
  }
  p.h2[0] = p.h2[1] = p.g1 = p.gb = p.g2 = p.xp = p.lp = o;  // unused by these passes
  p.dmax = d.D;
  p.total = o;
  return pp;
}

// Walkers per chunk: at most the model's energy budget of workspace, chunks balanced.
int psi_fl_chunk(const qmc_model* m, int batch) {
  const size_t per = psi_fl_plan(m, 1).base.total;
  const int cap = (int)std::max<size_t>(1, std::min<size_t>((size_t)batch, m->energy_budget / per));
  const int nch = (batch + cap - 1) / cap;
  return (batch + nch - 1) / nch;
}

qmc_status psi_fl_check(const qmc_model* m) {
  const PsiDims& d = m->psi->d;
  const PsiPlan pp = psi_fl_plan(m, 1);
  if (pp.base.Tp <= 0 || pp.base.Tp > 128) {
    set_error("local energy supports at most 42 electrons (3n+2 <= 128 tangents per tile)");
    return QMC_ERR_SHAPE;
  }
  if (!psi_attention_fl_supported(d.n, d.Dh)) {
    set_error("psiformer local energy: %d electrons x head width %d exceed the attention kernel", d.n, d.Dh);
    return QMC_ERR_UNSUPPORTED;
  }
  return QMC_OK;
}

template <class Out>
static qmc_status psi_backbone_fl(qmc_model* m, const PsiPlan& pp, void* ws, cudaStream_t s,
                                  Out (*fmt)(void*, const PsiPlan&, size_t, int)) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const PsiArena& a = m->psi->a;
  const float* ar = m->arena;
  const Plan& p = pp.base;
  const int groups = p.B * d.n, rows = groups * p.Tp, Tp = p.Tp, D = d.D;
  float* x = at<float>(ws, pp.x);
  float* z = at<float>(ws, pp.z);
  (void)rows;
  // input Dense fused into its group pass (the inputs' tangent rows are
  // sparse: an electron's features depend on its own position only)
  QMC_PROF(QMC_KC_LAYER0, launch_psi_input_fl(s, groups, d.n, Tp, D, at<float>(ws, p.x0), d.K0, d.K0p,
                                              ar + a.w_in, ar + P.in_b, x, ar + P.ln0_s[0], ar + P.ln0_b[0],
                                              fmt(ws, pp, pp.xn, D)));
  for (int l = 0; l < d.L; ++l) {
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn, D, a.w_qkv[l], a.t_qkv[l], 3 * D));
    QMC_PROF(QMC_KC_PAIR, launch_psi_attention_fl(s, p.B, d.n, Tp, p.T, d.H, d.Dh, z, ar + a.b_qkv[l],
                                                  fmt(ws, pp, pp.att, D)));
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.att, D, P.o_k[l], a.t_o[l], D));
    QMC_PROF(QMC_KC_MEANS, launch_psi_group_fl(s, groups, Tp, D, z, D, ar + P.o_b[l], 0, x, 2, ar + P.ln1_s[l],
                                               ar + P.ln1_b[l], fmt(ws, pp, pp.xn, D)));
    size_t in = pp.xn, other = pp.att;
    int din = D;
    for (int k = 0; k < d.n_dense; ++k) {
      const int dout = d.mlp[k];
      QMC_TRY(psi_gemm(m, pp, ws, s, in, din, P.mlp_k[l][k], a.t_mlp[l][k], dout));
      if (k + 1 < d.n_dense) {
        QMC_PROF(QMC_KC_MEANS, launch_psi_group_fl(s, groups, Tp, dout, z, dout, ar + P.mlp_b[l][k], 1, x, 0,
                                                   nullptr, nullptr, fmt(ws, pp, other, dout)));
        std::swap(in, other);
        din = dout;
      } else if (l + 1 < d.L) {
        QMC_PROF(QMC_KC_MEANS, launch_psi_group_fl(s, groups, Tp, D, z, D, ar + P.mlp_b[l][k], 1, x, 2,
                                                   ar + P.ln0_s[l + 1], ar + P.ln0_b[l + 1], fmt(ws, pp, pp.xn, D)));
      } else {
        QMC_PROF(QMC_KC_MEANS, launch_psi_group_fl(s, groups, Tp, D, z, D, ar + P.mlp_b[l][k], 1, x, 2, nullptr,
                                                   nullptr, fmt(ws, pp, p.h1[0], D)));
      }
    }
  }
  return QMC_OK;
}

// LapNet backbone with forward-Laplacian tangents: lapnet_backbone's steps on
// groups of Tp tangent rows (the group kernel carries value, Laplacian and
// Jacobian rows through bias, tanh and the residuals; the tangent attention
// kernel propagates through softmax and the bilinear products).
template <class Out>
static qmc_status lapnet_backbone_fl(qmc_model* m, const PsiPlan& pp, void* ws, cudaStream_t s,
                                     Out (*fmt)(void*, const PsiPlan&, size_t, int)) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const PsiArena& a = m->psi->a;
  const float* ar = m->arena;
  const Plan& p = pp.base;
  const int groups = p.B * d.n, rows = groups * p.Tp, Tp = p.Tp, D = d.D;
  float* x = at<float>(ws, pp.x);
  float* x2 = at<float>(ws, pp.x2);
  float* z = at<float>(ws, pp.z);
  float* z2 = at<float>(ws, pp.z2);
  (void)rows;
  // the input Dense of both streams fused into their group passes
  QMC_PROF(QMC_KC_LAYER0, launch_psi_input_fl(s, groups, d.n, Tp, D, at<float>(ws, p.x0), d.K0, d.K0p,
                                              ar + a.w_in, ar + a.lb_in, x, nullptr, nullptr,
                                              fmt(ws, pp, pp.xn, D)));
  QMC_PROF(QMC_KC_LAYER0, launch_psi_input_fl(s, groups, d.n, Tp, D, at<float>(ws, p.x0), d.K0, d.K0p,
                                              ar + a.w_in, ar + a.lb_in, x2, nullptr, nullptr,
                                              fmt(ws, pp, pp.xn2, D)));
  for (int l = 0; l < d.L; ++l) {
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn2, D, P.qk_k[l], a.t_qkv[l], 2 * D, z, 3 * D));
    for (int j = 0; l + 1 < d.L && j < d.n_local; ++j) {
      QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn2, D, P.ul_k[l][j], a.t_ul[l][j], D, z2, D));
      QMC_PROF(QMC_KC_MEANS, launch_psi_group_fl(s, groups, Tp, D, z2, D, ar + a.lb_ul[l][j], 1, x2, 2, nullptr,
                                                 nullptr, fmt(ws, pp, pp.xn2, D)));
    }
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn, D, P.lv_k[l], a.t_v[l], D, z + 2 * D, 3 * D));
    QMC_PROF(QMC_KC_PAIR, launch_psi_attention_fl(s, p.B, d.n, Tp, p.T, d.H, d.Dh, z, ar + a.b_qkv[l],
                                                  fmt(ws, pp, pp.att, D)));
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.att, D, P.lo_k[l], a.t_o[l], D));
    QMC_PROF(QMC_KC_MEANS, launch_psi_group_fl(s, groups, Tp, D, z, D, ar + a.lb_o[l], 0, x, 2, nullptr, nullptr,
                                               fmt(ws, pp, pp.xn, D)));
    QMC_TRY(psi_gemm(m, pp, ws, s, pp.xn, D, P.vu_k[l], a.t_vu[l], D));
    QMC_PROF(QMC_KC_MEANS, launch_psi_group_fl(s, groups, Tp, D, z, D, ar + a.lb_vu[l], 1, x, 2, nullptr, nullptr,
                                               fmt(ws, pp, l + 1 < d.L ? pp.xn : p.h1[0], D)));
  }
  return QMC_OK;
}

qmc_status psi_local_energy(qmc_model* m, int batch, const float* electrons, float* e_local, float* ke,
                            float* pe, float* logpsi, uint8_t* flags, void* ws, cudaStream_t s) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const float* ar = m->arena;
  const int chunk = psi_fl_chunk(m, batch);
  for (int b0 = 0; b0 < batch; b0 += chunk) {
    const int Bc = std::min(chunk, batch - b0);
    const PsiPlan pp = psi_fl_plan(m, Bc);
    const Plan& p = pp.base;
    float* pe_ws = at<float>(ws, p.pe);
    QMC_PROF(QMC_KC_FEATURES,
             launch_psi_features_fl(s, Bc, d.n, d.n_up, d.A, p.Tp, p.T, d.K0p, electrons + (size_t)b0 * 3 * d.n,
                                    ar + m->a.atoms, ar + m->a.charges, m->nuclear_repulsion,
                                    d.jastrow ? ar + P.alpha_par : nullptr, at<float>(ws, p.x0), at<float>(ws, p.rae),
                                    at<float>(ws, p.aevec), pe_ws, at<float>(ws, pp.jas), at<float>(ws, pp.jgl)));
    if (d.arch == kArchLapNet) {
      if (p.mixed) QMC_TRY(lapnet_backbone_fl<StSplit>(m, pp, ws, s, fmt_split));
      else QMC_TRY(lapnet_backbone_fl<StF32>(m, pp, ws, s, fmt_f32));
    } else {
      if (p.mixed) QMC_TRY(psi_backbone_fl<StSplit>(m, pp, ws, s, fmt_split));
      else QMC_TRY(psi_backbone_fl<StF32>(m, pp, ws, s, fmt_f32));
    }
    QMC_TRY(run_orbitals(m, p, ws, 0, s));
    float* lp = logpsi ? logpsi + b0 : at<float>(ws, p.lpsi);
    QMC_PROF(QMC_KC_LOGDET, launch_logdet(s, Bc, d.n, d.K, p.Tp, p.T, at<float>(ws, p.amat), pe_ws, lp,
                                          at<float>(ws, p.sgn), ke ? ke + b0 : nullptr, e_local + b0,
                                          flags ? flags + b0 : nullptr, nullptr, nullptr, at<float>(ws, pp.jgl),
                                          at<void>(ws, p.redo), m->det_guard_on()));
    QMC_PROF(QMC_KC_OTHER, (k_psi_add<<<(Bc + 255) / 256, 256, 0, s>>>(Bc, lp, at<float>(ws, pp.jas)),
                            cudaGetLastError()));
    if (pe) QMC_CUDA(cudaMemcpyAsync(pe + b0, pe_ws, sizeof(float) * Bc, cudaMemcpyDeviceToDevice, s));
  }
  return QMC_OK;
}

qmc_status psi_set_params(qmc_model* m, const float* params, cudaStream_t s) {
  const PsiDims& d = m->psi->d;
  const PsiParams& P = m->psi->p;
  const PsiArena& a = m->psi->a;
  const ArenaLayout& oa = m->a;
  float* ar = m->arena;
  __nv_bfloat16* ab = m->arena_bf16;
  const int D = d.D;
  QMC_CUDA(cudaMemcpyAsync(ar, params, P.total * sizeof(float), cudaMemcpyDeviceToDevice, s));
  // input kernel [K0][D] zero-padded to [K0p][D]
  QMC_CUDA(cudaMemsetAsync(ar + a.w_in, 0, sizeof(float) * d.K0p * D, s));
  QMC_CUDA(cudaMemcpyAsync(ar + a.w_in, params + P.in_k, sizeof(float) * d.K0 * D, cudaMemcpyDeviceToDevice, s));
  auto copy = [&](size_t dst, size_t src, size_t count) {
    return cudaMemcpyAsync(ar + dst, params + src, sizeof(float) * count, cudaMemcpyDeviceToDevice, s);
  };
  for (int l = 0; d.arch == kArchLapNet && l < d.L; ++l) {
    // biases stay zero (arena initialisation) when the model has none
    if (d.bb_bias) {
      QMC_CUDA(copy(a.b_qkv[l], P.qk_b[l], 2 * (size_t)D));
      QMC_CUDA(copy(a.b_qkv[l] + 2 * (size_t)D, P.lv_b[l], D));
      QMC_CUDA(copy(a.lb_o[l], P.lo_b[l], D));
      QMC_CUDA(copy(a.lb_vu[l], P.vu_b[l], D));
    }
    QMC_CUDA(launch_transpose_split(s, ar + P.qk_k[l], D, 2 * D, 2 * D, ab + a.t_qkv[l], D, 2 * D));
    QMC_CUDA(launch_transpose_split(s, ar + P.lv_k[l], D, D, D, ab + a.t_v[l], D, D));
    QMC_CUDA(launch_transpose_split(s, ar + P.lo_k[l], D, D, D, ab + a.t_o[l], D, D));
    QMC_CUDA(launch_transpose_split(s, ar + P.vu_k[l], D, D, D, ab + a.t_vu[l], D, D));
    QMC_CUDA(launch_transpose_f32(s, ar + P.qk_k[l], D, 2 * D, 2 * D, ar + a.t32_qkv[l]));
    QMC_CUDA(launch_transpose_f32(s, ar + P.lv_k[l], D, D, D, ar + a.t32_v[l]));
    QMC_CUDA(launch_transpose_f32(s, ar + P.lo_k[l], D, D, D, ar + a.t32_o[l]));
    QMC_CUDA(launch_transpose_f32(s, ar + P.vu_k[l], D, D, D, ar + a.t32_vu[l]));
    for (int j = 0; l + 1 < d.L && j < d.n_local; ++j) {
      if (d.bb_bias) QMC_CUDA(copy(a.lb_ul[l][j], P.ul_b[l][j], D));
      QMC_CUDA(launch_transpose_split(s, ar + P.ul_k[l][j], D, D, D, ab + a.t_ul[l][j], D, D));
      QMC_CUDA(launch_transpose_f32(s, ar + P.ul_k[l][j], D, D, D, ar + a.t32_ul[l][j]));
    }
  }
  if (d.arch == kArchLapNet && d.in_bias) QMC_CUDA(copy(a.lb_in, P.in_b, D));
  for (int l = 0; d.arch == kArchPsiformer && l < d.L; ++l) {
    const size_t src[3] = {P.q_k[l], P.k_k[l], P.v_k[l]}, bsrc[3] = {P.q_b[l], P.k_b[l], P.v_b[l]};
    for (int c = 0; c < 3; ++c) {
      QMC_CUDA(cudaMemcpy2DAsync(ar + a.w_qkv[l] + (size_t)c * D, sizeof(float) * 3 * D, params + src[c],
                                 sizeof(float) * D, sizeof(float) * D, D, cudaMemcpyDeviceToDevice, s));
      QMC_CUDA(cudaMemcpyAsync(ar + a.b_qkv[l] + (size_t)c * D, params + bsrc[c], sizeof(float) * D,
                               cudaMemcpyDeviceToDevice, s));
    }
    QMC_CUDA(launch_transpose_split(s, ar + a.w_qkv[l], D, 3 * D, 3 * D, ab + a.t_qkv[l], D, 3 * D));
    QMC_CUDA(launch_transpose_split(s, ar + P.o_k[l], D, D, D, ab + a.t_o[l], D, D));
    QMC_CUDA(launch_transpose_f32(s, ar + a.w_qkv[l], D, 3 * D, 3 * D, ar + a.t32_qkv[l]));
    QMC_CUDA(launch_transpose_f32(s, ar + P.o_k[l], D, D, D, ar + a.t32_o[l]));
    int din = D;
    for (int k = 0; k < d.n_dense; ++k) {
      QMC_CUDA(launch_transpose_split(s, ar + P.mlp_k[l][k], din, d.mlp[k], d.mlp[k], ab + a.t_mlp[l][k], din,
                                      d.mlp[k]));
      QMC_CUDA(launch_transpose_f32(s, ar + P.mlp_k[l][k], din, d.mlp[k], d.mlp[k], ar + a.t32_mlp[l][k]));
      din = d.mlp[k];
    }
  }
  const int nch = d.split ? 2 : 1;
  for (int c = 0; c < nch; ++c) {
    QMC_CUDA(cudaMemsetAsync(ar + oa.w_orb[c], 0, sizeof(float) * D * m->d.norb_p, s));
    QMC_CUDA(cudaMemcpy2DAsync(ar + oa.w_orb[c], sizeof(float) * m->d.norb_p, params + P.orb_k[c],
                               sizeof(float) * m->d.norb, sizeof(float) * m->d.norb, D, cudaMemcpyDeviceToDevice,
                               s));
    if (m->d.env_kind != QMC_ENVELOPE_NULL) {
      QMC_CUDA(cudaMemcpyAsync(ar + oa.env_pi[c], params + P.env_pi[c],
                               sizeof(float) * env_pi_floats(m->d.env_kind, d.n, d.A, d.K), cudaMemcpyDeviceToDevice,
                               s));
      QMC_CUDA(cudaMemcpyAsync(ar + oa.env_sigma[c], params + P.env_sigma[c],
                               sizeof(float) * env_sigma_floats(m->d.env_kind, d.n, d.A, d.K),
                               cudaMemcpyDeviceToDevice, s));
    }
    QMC_CUDA(launch_transpose_split(s, ar + oa.w_orb[c], D, m->d.norb, m->d.norb_p, ab + oa.t_orb[c], D,
                                    m->d.norb));
    QMC_CUDA(cudaMemsetAsync(ar + oa.wt_orb[c], 0, sizeof(float) * m->d.norb_p * D, s));
    QMC_CUDA(launch_transpose_f32(s, ar + oa.w_orb[c], D, m->d.norb, m->d.norb_p, ar + oa.wt_orb[c]));
  }
  m->params_set = true;
  return QMC_OK;
}

}  // namespace qmc

namespace qmc {

// Flat parameter offsets (C-ABI leaf order), derived arena fields and the
// bf16 K-major weight copies of an attention-backbone model whose dims are
// filled in; allocates and initialises the device arenas.
static qmc_status psi_layout_alloc(qmc_model* m, int env_kind, const float* atoms_host, const float* charges_host) {
  PsiDims& d = m->psi->d;
  const int n = d.n, A = d.A, D = d.D;
  PsiParams& P = m->psi->p;
  size_t o = 0;
  auto take = [&](size_t count) { size_t r = o; o += count; return r; };
  P.in_k = take((size_t)d.K0 * D);
  if (d.arch == kArchPsiformer || d.in_bias) P.in_b = take(D);
  for (int l = 0; l < d.L; ++l) {
    if (d.arch == kArchLapNet) {
      auto dense = [&](size_t* k, size_t* b, int dout) {
        *k = take((size_t)D * dout);
        if (d.bb_bias) *b = take(dout);
      };
      dense(&P.qk_k[l], &P.qk_b[l], 2 * D);
      dense(&P.lv_k[l], &P.lv_b[l], D);
      dense(&P.lo_k[l], &P.lo_b[l], D);
      dense(&P.vu_k[l], &P.vu_b[l], D);
      for (int j = 0; l + 1 < d.L && j < d.n_local; ++j) dense(&P.ul_k[l][j], &P.ul_b[l][j], D);
      continue;
    }
    P.ln0_s[l] = take(D);
    P.ln0_b[l] = take(D);
    P.q_k[l] = take((size_t)D * D);
    P.q_b[l] = take(D);
    P.k_k[l] = take((size_t)D * D);
    P.k_b[l] = take(D);
    P.v_k[l] = take((size_t)D * D);
    P.v_b[l] = take(D);
    P.o_k[l] = take((size_t)D * D);
    P.o_b[l] = take(D);
    P.ln1_s[l] = take(D);
    P.ln1_b[l] = take(D);
    int din = D;
    for (int k = 0; k < d.n_dense; ++k) {
      P.mlp_k[l][k] = take((size_t)din * d.mlp[k]);
      P.mlp_b[l][k] = take(d.mlp[k]);
      din = d.mlp[k];
    }
  }
  const int nch = d.split ? 2 : 1;
  for (int c = 0; c < nch; ++c) P.orb_k[c] = take((size_t)D * d.K * n);
  for (int c = 0; c < nch; ++c) {
    P.env_pi[c] = take(env_pi_floats(env_kind, n, A, d.K));
    P.env_sigma[c] = take(env_sigma_floats(env_kind, n, A, d.K));
  }
  if (nch == 1) {
    P.orb_k[1] = P.orb_k[0];
    P.env_pi[1] = P.env_pi[0];
    P.env_sigma[1] = P.env_sigma[0];
  }
  if (d.jastrow) {
    P.alpha_par = take(1);
    P.alpha_anti = take(1);
  }
  P.total = o;
  // arena: verbatim params, then derived fp32 parameters, each block 64-byte
  // aligned (vector loads and TMA need 16-byte aligned bases)
  PsiArena& a = m->psi->a;
  o = align_up(P.total, 64);
  auto takea = [&](size_t count) { size_t r = o; o += align_up(count, 16); return r; };
  a.w_in = takea((size_t)d.K0p * D);
  if (d.arch == kArchLapNet) {
    a.lb_in = takea(D);
    for (int l = 0; l < d.L; ++l) {
      a.b_qkv[l] = takea((size_t)3 * D);
      a.lb_o[l] = takea(D);
      a.lb_vu[l] = takea(D);
      a.t32_qkv[l] = takea((size_t)2 * D * D);
      a.t32_o[l] = takea((size_t)D * D);
      a.t32_v[l] = takea((size_t)D * D);
      a.t32_vu[l] = takea((size_t)D * D);
      for (int j = 0; l + 1 < d.L && j < d.n_local; ++j) {
        a.lb_ul[l][j] = takea(D);
        a.t32_ul[l][j] = takea((size_t)D * D);
      }
    }
  }
  for (int l = 0; d.arch == kArchPsiformer && l < d.L; ++l) {
    a.w_qkv[l] = takea((size_t)D * 3 * D);
    a.b_qkv[l] = takea((size_t)3 * D);
    a.t32_qkv[l] = takea((size_t)3 * D * D);
    a.t32_o[l] = takea((size_t)D * D);
    int din = D;
    for (int k = 0; k < d.n_dense; ++k) {
      a.t32_mlp[l][k] = takea((size_t)d.mlp[k] * din);
      din = d.mlp[k];
    }
  }
  // FermiNet-shared orbital / envelope fields of the model
  Dims& fd = m->d;
  fd.n = n;
  fd.n_up = d.n_up;
  fd.n_dn = d.n_dn;
  fd.A = A;
  fd.K = d.K;
  fd.L = 0;
  fd.C = (d.n_up > 0) + (d.n_dn > 0);
  fd.split = d.split;
  fd.env_abs = d.env_abs;
  fd.env_kind = env_kind;
  fd.d_last = D;
  fd.norb = d.K * n;
  fd.norb_p = align_up(fd.norb, 8);
  ArenaLayout& fa = m->a;
  for (int c = 0; c < 2; ++c) {
    if (c < nch) {
      fa.w_orb[c] = takea((size_t)D * fd.norb_p);
      fa.wt_orb[c] = takea((size_t)fd.norb_p * D);
      fa.env_pi[c] = takea(env_pi_floats(env_kind, n, A, d.K));
      fa.env_sigma[c] = takea(env_sigma_floats(env_kind, n, A, d.K));
    } else {
      fa.w_orb[1] = fa.w_orb[0];
      fa.wt_orb[1] = fa.wt_orb[0];
      fa.env_pi[1] = fa.env_pi[0];
      fa.env_sigma[1] = fa.env_sigma[0];
    }
  }
  fa.atoms = takea((size_t)3 * A);
  fa.charges = takea(A);
  a.total = fa.total = o;
  size_t ob = 0;
  auto takeb = [&](size_t count) { size_t r = ob; ob += align_up(count, 64); return r; };
  for (int l = 0; l < d.L; ++l) {
    if (d.arch == kArchLapNet) {
      a.t_qkv[l] = takeb((size_t)2 * D * 2 * D);
      a.t_v[l] = takeb((size_t)2 * D * D);
      a.t_o[l] = takeb((size_t)2 * D * D);
      a.t_vu[l] = takeb((size_t)2 * D * D);
      for (int j = 0; l + 1 < d.L && j < d.n_local; ++j) a.t_ul[l][j] = takeb((size_t)2 * D * D);
      continue;
    }
    a.t_qkv[l] = takeb((size_t)2 * D * 3 * D);
    a.t_o[l] = takeb((size_t)2 * D * D);
    int din = D;
    for (int k = 0; k < d.n_dense; ++k) {
      a.t_mlp[l][k] = takeb((size_t)2 * din * d.mlp[k]);
      din = d.mlp[k];
    }
  }
  for (int c = 0; c < 2; ++c) fa.t_orb[c] = c < nch ? takeb((size_t)2 * fd.norb_p * D) : fa.t_orb[0];
  a.total_bf16 = fa.total_bf16 = ob;
  cudaError_t e = cudaGetDevice(&m->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->n_sms, cudaDevAttrMultiProcessorCount, m->device);
  if (e == cudaSuccess) e = cudaMalloc(&m->arena, fa.total * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->arena_bf16, fa.total_bf16 * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMalloc(&m->dev_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m->dev_err, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(m->arena, 0, fa.total * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(m->arena_bf16, 0, fa.total_bf16 * sizeof(__nv_bfloat16));
  memcpy(m->atoms_host, atoms_host, sizeof(float) * 3 * A);
  memcpy(m->charges_host, charges_host, sizeof(float) * A);
  m->nuclear_repulsion = nuclear_repulsion(atoms_host, charges_host, A);
  if (e == cudaSuccess) e = cudaMemcpy(m->arena + fa.atoms, atoms_host, sizeof(float) * 3 * A, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(m->arena + fa.charges, charges_host, sizeof(float) * A, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(m->arena);
    cudaFree(m->arena_bf16);
    cudaFree(m->dev_err);
    m->arena = nullptr;
    m->arena_bf16 = nullptr;
    m->dev_err = nullptr;
    return cuda_status(e, "attention-backbone model create");
  }
  return QMC_OK;
}

// Shared validation of the attention sizes, precision and envelope.
static qmc_status psi_check_common(const char* who, int n, int A, int ndets, int n_layers, int n_heads,
                                   int head_dim, int precision, int envelope) {
  if (n < 1 || n > 64 || A < 1 || A > kMaxAtoms || ndets < 1 || n_layers < 1 || n_layers > kPsiMaxLayers ||
      n_heads < 1 || head_dim < 1) {
    set_error("%s: bad sizes (n=%d atoms=%d layers=%d heads=%d)", who, n, A, n_layers, n_heads);
    return QMC_ERR_SHAPE;
  }
  const int D = n_heads * head_dim;
  if (!(D % 64 == 0 && D <= 512 && head_dim % 4 == 0)) {
    set_error("%s: attention width must be a multiple of 64 (at most 512), head width a multiple of 4", who);
    return QMC_ERR_UNSUPPORTED;
  }
  if (attention_smem(n, head_dim) > 200 * 1024) {
    set_error("%s: %d electrons x head width %d exceed the attention kernel's shared memory", who, n, head_dim);
    return QMC_ERR_UNSUPPORTED;
  }
  if (precision != QMC_PRECISION_FP32 && precision != QMC_PRECISION_MIXED_BF16) {
    set_error("unknown precision %d", precision);
    return QMC_ERR_ARG;
  }
  if (envelope < QMC_ENVELOPE_ISOTROPIC || envelope > QMC_ENVELOPE_NULL) {
    set_error("unsupported envelope %d", envelope);
    return QMC_ERR_UNSUPPORTED;
  }
  return QMC_OK;
}

static void psi_common_dims(PsiDims& d, int n_up, int n_down, int A, int K, int L, int H, int Dh, int split,
                            int envelope, int jastrow) {
  d.n = n_up + n_down;
  d.n_up = n_up;
  d.n_dn = n_down;
  d.A = A;
  d.K = K;
  d.L = L;
  d.H = H;
  d.Dh = Dh;
  d.D = H * Dh;
  d.split = split && n_up > 0 && n_down > 0;
  d.env_abs = envelope == QMC_ENVELOPE_ABS_ISOTROPIC;
  d.jastrow = jastrow != 0;
  d.K0 = 4 * A + 1;
  d.K0p = (d.K0 + 7) / 8 * 8;  // the SIMT GEMM walks K in steps of 8
}

static qmc_status psi_finish(qmc_model* m, int precision, int envelope, const float* atoms_host,
                             const float* charges_host, qmc_model** out) {
  m->precision = precision;
  const qmc_status st = psi_layout_alloc(m, envelope, atoms_host, charges_host);
  if (st != QMC_OK) {
    delete m->psi;
    delete m;
    return st;
  }
  *out = m;
  return QMC_OK;
}

}  // namespace qmc

using namespace qmc;

extern "C" qmc_status qmc_psiformer_create(const qmc_psiformer_config* cfg, const float* atoms_host,
                                           const float* charges_host, qmc_model** out) {
  if (!cfg || !atoms_host || !charges_host || !out) {
    set_error("null argument");
    return QMC_ERR_ARG;
  }
  *out = nullptr;
  if (cfg->n_up < 0 || cfg->n_down < 0 || cfg->n_mlp < 0 || cfg->n_mlp > kPsiMaxMlp) {
    set_error("psiformer: bad sizes (n_up=%d n_down=%d mlp=%d)", cfg->n_up, cfg->n_down, cfg->n_mlp);
    return QMC_ERR_SHAPE;
  }
  QMC_TRY(psi_check_common("psiformer", cfg->n_up + cfg->n_down, cfg->n_atoms, cfg->ndets, cfg->n_layers,
                           cfg->n_heads, cfg->head_dim, cfg->precision, cfg->envelope));
  for (int k = 0; k < cfg->n_mlp; ++k) {
    if (cfg->mlp_dims[k] % 64 || cfg->mlp_dims[k] < 64 || cfg->mlp_dims[k] > 512) {
      set_error("psiformer: MLP widths must be multiples of 64 (at most 512)");
      return QMC_ERR_UNSUPPORTED;
    }
  }
  qmc_model* m = new qmc_model();
  m->kind = QMC_KIND_PSIFORMER;
  m->psi = new PsiModel();
  PsiDims& d = m->psi->d;
  d.arch = kArchPsiformer;
  psi_common_dims(d, cfg->n_up, cfg->n_down, cfg->n_atoms, cfg->ndets, cfg->n_layers, cfg->n_heads, cfg->head_dim,
                  cfg->orbitals_spin_split, cfg->envelope, cfg->jastrow);
  d.n_dense = cfg->n_mlp + 1;
  for (int k = 0; k < cfg->n_mlp; ++k) d.mlp[k] = cfg->mlp_dims[k];
  d.mlp[cfg->n_mlp] = d.D;
  return psi_finish(m, cfg->precision, cfg->envelope, atoms_host, charges_host, out);
}

extern "C" qmc_status qmc_lapnet_create(const qmc_lapnet_config* cfg, const float* atoms_host,
                                        const float* charges_host, qmc_model** out) {
  if (!cfg || !atoms_host || !charges_host || !out) {
    set_error("null argument");
    return QMC_ERR_ARG;
  }
  *out = nullptr;
  if (cfg->n_up < 0 || cfg->n_down < 0 || cfg->num_local_updates < 0 || cfg->num_local_updates > kLapMaxLocal) {
    set_error("lapnet: bad sizes (n_up=%d n_down=%d local updates=%d, at most %d)", cfg->n_up, cfg->n_down,
              cfg->num_local_updates, kLapMaxLocal);
    return QMC_ERR_SHAPE;
  }
  QMC_TRY(psi_check_common("lapnet", cfg->n_up + cfg->n_down, cfg->n_atoms, cfg->ndets, cfg->n_layers,
                           cfg->n_heads, cfg->head_dim, cfg->precision, cfg->envelope));
  qmc_model* m = new qmc_model();
  m->kind = QMC_KIND_PSIFORMER;
  m->psi = new PsiModel();
  PsiDims& d = m->psi->d;
  d.arch = kArchLapNet;
  psi_common_dims(d, cfg->n_up, cfg->n_down, cfg->n_atoms, cfg->ndets, cfg->n_layers, cfg->n_heads, cfg->head_dim,
                  cfg->orbitals_spin_split, cfg->envelope, cfg->jastrow);
  d.n_dense = 0;
  d.n_local = cfg->num_local_updates;
  d.in_bias = cfg->use_input_bias != 0;
  d.bb_bias = cfg->use_backbone_bias != 0;
  return psi_finish(m, cfg->precision, cfg->envelope, atoms_host, charges_host, out);
}
