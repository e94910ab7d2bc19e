// FermiNet features, two-electron stream, spin means, determinant stage,
// Metropolis-Hastings and reductions for sm_103a.
#include <algorithm>

#include "kernels.cuh"
#include "tc_ptx.cuh"

namespace qmc {

// =====================================================================
// features (src/jaqmc/wavefunction/input/atomic.py:46-79,
//           src/jaqmc/geometry/obc.py:7-88,
//           src/jaqmc/app/molecule/hamiltonian.py:9-22)
// =====================================================================
__global__ void k_features(int n, int A, int Tp, int T, int K0p, const float* __restrict__ elec,
                           const float* __restrict__ atoms, const float* __restrict__ charges,
                           double nuc, float* __restrict__ X0, float* __restrict__ H2,
                           float* __restrict__ rae_g, float* __restrict__ aevec_g,
                           float* __restrict__ pe, int n_up, int C, int g2p, float* __restrict__ G2) {
  extern __shared__ float sh[];
  float* xs = sh;                // [n][3]
  float* rs = xs + 3 * n;        // [n][A]
  float* vs = rs + n * A;        // [n][A][3]
  __shared__ double red[32];
  const int w = blockIdx.x;
  const float* ew = elec + (size_t)w * n * 3;
  for (int e = threadIdx.x; e < 3 * n; e += blockDim.x) xs[e] = ew[e];
  __syncthreads();
  double vpot = 0.0;
  for (int e = threadIdx.x; e < n * A; e += blockDim.x) {
    int i = e / A, I = e % A;
    float dx = xs[3 * i] - atoms[3 * I], dy = xs[3 * i + 1] - atoms[3 * I + 1],
          dz = xs[3 * i + 2] - atoms[3 * I + 2];
    float r = sqrtf(dx * dx + dy * dy + dz * dz);
    rs[e] = r;
    vs[3 * e] = dx;
    vs[3 * e + 1] = dy;
    vs[3 * e + 2] = dz;
    size_t gi = (size_t)w * n * A + e;
    rae_g[gi] = r;
    aevec_g[3 * gi] = dx;
    aevec_g[3 * gi + 1] = dy;
    aevec_g[3 * gi + 2] = dz;
    if (pe) vpot -= (double)charges[I] / (double)r;
  }
  __syncthreads();
  // one-electron rows (32-bit index arithmetic within a walker)
  const int A4 = 4 * A;
  const int per_w = n * Tp * K0p;
  float* Xw = X0 + (size_t)w * per_w;
  for (int e = threadIdx.x; e < per_w; e += blockDim.x) {
    const int f = e % K0p;
    const int it = e / K0p;
    const int t = it % Tp;
    const int i = it / Tp;
    float v = 0.f;
    if (f < A4 && t < T) {
      int I = f >> 2, comp = f & 3;
      float r = rs[i * A + I];
      const float* vec = vs + 3 * (i * A + I);
      if (t == 0) {
        v = comp == 0 ? r : vec[comp - 1];
      } else if (t == 1) {
        v = comp == 0 ? 2.0f / r : 0.f;
      } else {
        int d = t - 2, el = d / 3, c = d % 3;
        if (el == i) v = comp == 0 ? vec[c] / r : (comp - 1 == c ? 1.f : 0.f);
      }
    }
    Xw[e] = v;
  }
  // two-electron rows
  const int P2 = T > 1 ? 5 : 1;
  const int per_w2 = n * n * P2 * 4;
  float* Hw = H2 + (size_t)w * per_w2;
  for (int e = threadIdx.x; e < per_w2; e += blockDim.x) {
    const int comp = e & 3;
    const int p = (e >> 2) % P2;
    const int pr = e / (4 * P2);
    const int i = pr / n, j = pr % n;
    float v = 0.f;
    if (i != j) {
      float d[3] = {xs[3 * i] - xs[3 * j], xs[3 * i + 1] - xs[3 * j + 1], xs[3 * i + 2] - xs[3 * j + 2]};
      float r = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      if (p == 0) v = comp == 0 ? r : d[comp - 1];
      else if (p == 1) v = comp == 0 ? 2.0f / r : 0.f;
      else {
        int c = p - 2;
        v = comp == 0 ? d[c] / r : (comp - 1 == c ? 1.f : 0.f);
      }
      if (pe && p == 0 && comp == 0 && i < j) vpot += 1.0 / (double)r;
    }
    Hw[e] = v;
  }
  if (G2 && T == 1) {
    // spin means of the ee features over the first electron index:
    // G2[w*n+i][s*4 + comp] = mean_{a in s} ee[a, i, comp]
    for (int e = threadIdx.x; e < n * g2p; e += blockDim.x) {
      const int i = e / g2p, col = e % g2p;
      float v = 0.f;
      if (col < 4 * C) {
        const int sc = col / 4, comp = col % 4;
        const int a0 = C == 1 ? 0 : (sc == 0 ? 0 : n_up), a1 = C == 1 ? n : (sc == 0 ? n_up : n);
        float acc = 0.f;
        for (int a = a0; a < a1; ++a) {
          if (a == i) continue;
          float d0 = xs[3 * a] - xs[3 * i], d1 = xs[3 * a + 1] - xs[3 * i + 1], d2 = xs[3 * a + 2] - xs[3 * i + 2];
          acc += comp == 0 ? sqrtf(d0 * d0 + d1 * d1 + d2 * d2) : (comp == 1 ? d0 : (comp == 2 ? d1 : d2));
        }
        v = acc / (float)(a1 - a0);
      }
      G2[((size_t)w * n + i) * g2p + col] = v;
    }
  }
  if (pe) {
    // block reduction of the potential
    for (int o = 16; o > 0; o >>= 1) vpot += __shfl_xor_sync(0xffffffffu, vpot, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vpot;
    __syncthreads();
    if (threadIdx.x < 32) {
      double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0) pe[w] = (float)(v + nuc);
    }
  }
}

cudaError_t launch_features(cudaStream_t s, int B, int n, int A, int Tp, int T, int K0p,
                            const float* electrons, const float* atoms, const float* charges,
                            double nuc, float* X0, float* H2, float* rae, float* aevec, float* pe,
                            int n_up, int C, int g2p, float* G2) {
  size_t sm = sizeof(float) * (3 * n + 4 * n * A);
  k_features<<<B, 256, sm, s>>>(n, A, Tp, T, K0p, electrons, atoms, charges, nuc, X0, H2, rae,
                                aevec, pe, n_up, C, g2p, G2);
  return cudaGetLastError();
}

// 2^x by the hardware base-2 exponential (relative error ~2^-22).  Used by
// the mixed form's envelope factors: exp(-|sigma| r) = 2^(-log2(e) |sigma| r)
// with log2(e) |sigma| rounded to FP32 adds at most ~1e-6 relative error for
// the arguments that matter, below the form's split-BF16 operand error.
__device__ __forceinline__ float fast_exp2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Envelope factor of every value-only orbital matrix element (walker w,
// determinant k, electron i, orbital j): sum_I pi[j,I,k] exp(-s r_iI) with
// s = |sigma[j,I,k]| (abs_isotropic) or sigma (isotropic), per spin channel
// of electron i (src/jaqmc/wavefunction/output/envelope.py:98-140).  Same
// terms in the same order as the tangent epilogues, the exponentials by
// fast_exp2 (the kernel serves the mixed form only).  One block per
// kEnvWalkers walkers, thread (walker, i, j) looping over k with its electron's
// distances in registers (NA atoms at compile time; NA = 0: any count); the
// parameters are staged once per block as (pi, log2(e) s) pairs
// [channel][k][I][j], so a warp reads consecutive j.
constexpr int kEnvWalkers = 8;
template <int NA>
__global__ void k_envelope_value(int B, int n, int n_up, int split, int K, int A, int env_abs,
                                 const float* __restrict__ pi0, const float* __restrict__ sg0,
                                 const float* __restrict__ pi1, const float* __restrict__ sg1,
                                 const float* __restrict__ rae, float* __restrict__ env) {
  extern __shared__ float2 she2[];
  const int nch = split ? 2 : 1, per = K * A * n, kan = A * n;
  for (int e = threadIdx.x; e < nch * per; e += blockDim.x) {
    const int c = e / per, rem = e - c * per;
    const int k = rem / kan, rem2 = rem - k * kan;
    const int I = rem2 / n, j = rem2 - I * n;
    const size_t q = ((size_t)j * A + I) * K + k;
    const float sv = (c ? sg1 : sg0)[q];
    she2[e] = make_float2((c ? pi1 : pi0)[q], (env_abs ? fabsf(sv) : sv) * 1.4426950408889634f);
  }
  __syncthreads();
  const int nn = n * n;
  const int na = NA > 0 ? NA : A;
  for (int e = threadIdx.x; e < kEnvWalkers * nn; e += blockDim.x) {
    const int wl = e / nn, ij = e - wl * nn;
    const int w = blockIdx.x * kEnvWalkers + wl;
    if (w >= B) break;
    const int i = ij / n, j = ij - i * n;
    const int c = split && i >= n_up ? 1 : 0;
    const float* ra = rae + ((size_t)w * n + i) * A;
    float* out = env + (size_t)w * K * nn + ij;
    const float2* q = she2 + (size_t)c * per + j;
    if constexpr (NA > 0) {
      float r[NA];
#pragma unroll
      for (int I = 0; I < NA; ++I) r[I] = __ldg(ra + I);
      for (int k = 0; k < K; ++k, q += kan) {
        float acc = 0.f;
#pragma unroll
        for (int I = 0; I < NA; ++I) {
          const float2 v = q[I * n];
          acc += v.x * fast_exp2(-v.y * r[I]);
        }
        out[(size_t)k * nn] = acc;
      }
    } else {
      for (int k = 0; k < K; ++k, q += kan) {
        float acc = 0.f;
        for (int I = 0; I < na; ++I) {
          const float2 v = q[I * n];
          acc += v.x * fast_exp2(-v.y * __ldg(ra + I));
        }
        out[(size_t)k * nn] = acc;
      }
    }
  }
}

cudaError_t launch_envelope_value(cudaStream_t s, int B, int n, int n_up, int split, int K, int A, int env_abs,
                                  const float* pi0, const float* sg0, const float* pi1, const float* sg1,
                                  const float* rae, float* env) {
  const size_t sm = sizeof(float2) * (split ? 2 : 1) * (size_t)A * K * n;
  if (sm > 48 * 1024) return cudaErrorNotSupported;
  const unsigned grid = (unsigned)((B + kEnvWalkers - 1) / kEnvWalkers);
#define QMC_ENV_CASE(NA_)                                                                                       \
  case NA_:                                                                                                     \
    k_envelope_value<NA_><<<grid, 256, sm, s>>>(B, n, n_up, split, K, A, env_abs, pi0, sg0, pi1, sg1, rae, env); \
    break;
  switch (A) {
    QMC_ENV_CASE(1)
    QMC_ENV_CASE(2)
    QMC_ENV_CASE(3)
    QMC_ENV_CASE(4)
    QMC_ENV_CASE(6)
    QMC_ENV_CASE(12)
    default:
      k_envelope_value<0><<<grid, 256, sm, s>>>(B, n, n_up, split, K, A, env_abs, pi0, sg0, pi1, sg1, rae, env);
  }
#undef QMC_ENV_CASE
  return cudaGetLastError();
}

// The same factors multiplied into raw value-only orbital matrices in place:
// one block per (walker, determinant k), the parameters of k staged as
// [channel][I][j] and the walker's electron-atom distances in shared memory.
__global__ void k_envelope_apply(int n, int n_up, int split, int K, int A, int env_abs,
                                 const float* __restrict__ pi0, const float* __restrict__ sg0,
                                 const float* __restrict__ pi1, const float* __restrict__ sg1,
                                 const float* __restrict__ rae, float* __restrict__ Amat) {
  extern __shared__ float sha[];
  const int nch = split ? 2 : 1, per = A * n;
  float* ps = sha;                  // [nch][A][n]
  float* ss = ps + nch * per;       // [nch][A][n]
  float* ra = ss + nch * per;       // [n][A]
  const int w = blockIdx.x / K, k = blockIdx.x % K;
  for (int e = threadIdx.x; e < nch * per; e += blockDim.x) {
    const int c = e / per, I = (e / n) % A, j = e % n;
    const size_t q = ((size_t)j * A + I) * K + k;
    ps[e] = (c ? pi1 : pi0)[q];
    const float sv = (c ? sg1 : sg0)[q];
    ss[e] = env_abs ? fabsf(sv) : sv;
  }
  for (int e = threadIdx.x; e < n * A; e += blockDim.x) ra[e] = rae[(size_t)w * n * A + e];
  __syncthreads();
  float* Am = Amat + ((size_t)w * K + k) * n * n;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    const int c = split && i >= n_up ? 1 : 0;
    float acc = 0.f;
    for (int I = 0; I < A; ++I) {
      const int o = (c * A + I) * n + j;
      acc += ps[o] * expf(-ss[o] * ra[i * A + I]);
    }
    Am[e] *= acc;
  }
}

cudaError_t launch_envelope_apply(cudaStream_t s, int B, int n, int n_up, int split, int K, int A, int env_abs,
                                  const float* pi0, const float* sg0, const float* pi1, const float* sg1,
                                  const float* rae, float* Amat) {
  const size_t sm = sizeof(float) * ((size_t)2 * (split ? 2 : 1) * A * n + (size_t)n * A);
  if (sm > 48 * 1024) return cudaErrorNotSupported;
  k_envelope_apply<<<(unsigned)((size_t)B * K), 256, sm, s>>>(n, n_up, split, K, A, env_abs, pi0, sg0, pi1, sg1,
                                                               rae, Amat);
  return cudaGetLastError();
}

// Diagonal envelope (src/jaqmc/wavefunction/output/envelope.py:143-163),
// applied in place to orbital matrices that the orbital GEMM stored without
// an envelope.  For column (k, j) at electron i, with v = r_i - R_I,
//   s_I = ||sigma_I (.) v||,  E = sum_I pi_I e^{-s_I},
//   dE/dv_c = -sum_I pi_I e^{-s_I} sigma_Ic^2 v_c / s_I,
//   lap E = sum_I pi_I e^{-s_I} (|grad s_I|^2 - lap s_I),
//   lap s = sum_c (sigma_c^2 / s - sigma_c^4 v_c^2 / s^3).
// Value rows become O E; tangent rows O_t E, plus O_0 dE/dv_c on electron i's
// own three gradient rows; the Laplacian row O_L E + 2 sum_c O_c dE_c + O_0 lap E
// (the product rule of the tangent epilogues).  One block per (walker,
// electron); thread (k, j) over the K n columns of the electron's row, so a
// warp reads and writes consecutive columns of each tangent row.
__global__ void __launch_bounds__(256) k_envelope_diag(int n, int n_up, int split, int K, int A, int Tp, int T,
                                                       const float* __restrict__ pi0, const float* __restrict__ sg0,
                                                       const float* __restrict__ pi1, const float* __restrict__ sg1,
                                                       const float* __restrict__ aevec, float* __restrict__ Amat) {
  __shared__ float av[3 * kMaxAtoms];
  const int w = blockIdx.x / n, i = blockIdx.x % n;
  const int ch = split && i >= n_up ? 1 : 0;
  const float* pi = ch ? pi1 : pi0;
  const float* sg = ch ? sg1 : sg0;
  for (int e = threadIdx.x; e < 3 * A; e += blockDim.x) av[e] = aevec[((size_t)w * n + i) * A * 3 + e];
  __syncthreads();
  const size_t ts = amat_tangent_stride(n, K);
  for (int col = threadIdx.x; col < K * n; col += blockDim.x) {
    const int k = col / n, j = col - k * n;
    float e0 = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f, el = 0.f;
    for (int I = 0; I < A; ++I) {
      const size_t q = (size_t)j * A + I;
      const float pv = pi[q * K + k];
      float s2[3], sq = 0.f;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float sc = sg[(q * 3 + c) * K + k];
        s2[c] = sc * sc;
        sq = fmaf(s2[c] * av[3 * I + c], av[3 * I + c], sq);
      }
      const float s = sqrtf(sq);
      const float ev = pv * expf(-s);
      e0 += ev;
      if (T > 1) {
        const float inv = 1.f / s;
        float d[3], gsq = 0.f, lap_s = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          d[c] = s2[c] * av[3 * I + c] * inv;
          gsq = fmaf(d[c], d[c], gsq);
          lap_s += s2[c] * inv - d[c] * d[c] * inv;
        }
        g0 = fmaf(-ev, d[0], g0);
        g1 = fmaf(-ev, d[1], g1);
        g2 = fmaf(-ev, d[2], g2);
        el = fmaf(ev, gsq - lap_s, el);
      }
    }
    float* dst = Amat + amat_index(Tp, n, K, w, k, 0, i, j);
    if (T == 1) {
      dst[0] *= e0;
      continue;
    }
    const int t3 = 2 + 3 * i;
    const float o0 = dst[0], oL = dst[ts];
    const float oc0 = dst[(size_t)t3 * ts], oc1 = dst[(size_t)(t3 + 1) * ts], oc2 = dst[(size_t)(t3 + 2) * ts];
    for (int t = 0; t < T; ++t) dst[(size_t)t * ts] *= e0;  // rows T..Tp-1 are zero and stay so
    dst[(size_t)t3 * ts] = fmaf(o0, g0, oc0 * e0);
    dst[(size_t)(t3 + 1) * ts] = fmaf(o0, g1, oc1 * e0);
    dst[(size_t)(t3 + 2) * ts] = fmaf(o0, g2, oc2 * e0);
    dst[ts] = oL * e0 + 2.f * (oc0 * g0 + oc1 * g1 + oc2 * g2) + o0 * el;
  }
}

cudaError_t launch_envelope_diag(cudaStream_t s, int B, int n, int n_up, int split, int K, int A, int Tp, int T,
                                 const float* pi0, const float* sg0, const float* pi1, const float* sg1,
                                 const float* aevec, float* Amat) {
  if (A > kMaxAtoms) return cudaErrorNotSupported;
  k_envelope_diag<<<(unsigned)((size_t)B * n), 256, 0, s>>>(n, n_up, split, K, A, Tp, T, pi0, sg0, pi1, sg1, aevec,
                                                            Amat);
  return cudaGetLastError();
}

// hi = bf16(v), lo = bf16(v - hi) for n contiguous values (planes `plane` apart).
__global__ void k_to_split(size_t n, const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, size_t plane) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float v = src[e];
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  dst[e] = hi;
  dst[e + plane] = __float2bfloat16_rn(v - __bfloat162float(hi));
}

cudaError_t launch_to_split(cudaStream_t s, size_t n, const float* src, __nv_bfloat16* dst, size_t plane) {
  k_to_split<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, src, dst, plane);
  return cudaGetLastError();
}

// =====================================================================
// two-electron layer (src/jaqmc/wavefunction/backbone/ferminet.py:55-63)
// rows p: 0 value, 1 Laplacian wrt the pair difference, 2..4 its gradient.
// =====================================================================
__global__ void k_pair_layer(int npairs, int P2, int d_in, int d_out, const float* __restrict__ Hin,
                             const float* __restrict__ W, const float* __restrict__ b,
                             float* __restrict__ Hout) {
  extern __shared__ float sh[];
  float* Ws = sh;                     // [d_in][d_out], loaded once per block
  float* Is = Ws + d_in * d_out;      // [ppb][P2][d_in] of the current chunk
  const int ppb = blockDim.x / d_out;
  for (int e = threadIdx.x; e < d_in * d_out; e += blockDim.x) Ws[e] = W[e];
  const int lp = threadIdx.x / d_out, f = threadIdx.x % d_out;
  const float bf = b[f];
  const bool res = d_in == d_out;
  const int nchunks = (npairs + ppb - 1) / ppb;
  for (int chunk = blockIdx.x; chunk < nchunks; chunk += gridDim.x) {
    const int p0 = chunk * ppb;
    const int np = min(ppb, npairs - p0);
    __syncthreads();  // previous chunk done with Is (and Ws loaded on entry)
    for (int e = threadIdx.x; e < np * P2 * d_in; e += blockDim.x) Is[e] = Hin[(size_t)p0 * P2 * d_in + e];
    __syncthreads();
    if (lp >= np) continue;
    const float* in = Is + lp * P2 * d_in;
    float z[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int k = 0; k < d_in; ++k) {
      float wv = Ws[k * d_out + f];
#pragma unroll
      for (int p = 0; p < 5; ++p)
        if (p < P2) z[p] = fmaf(in[p * d_in + k], wv, z[p]);
    }
    float h = tanhf(z[0] + bf);
    float out[5];
    out[0] = h;
    if (P2 > 1) {
      float d1 = 1.f - h * h, d2 = -2.f * h * d1;
      float S = z[2] * z[2] + z[3] * z[3] + z[4] * z[4];
      out[1] = d1 * z[1] + d2 * S;
      out[2] = d1 * z[2];
      out[3] = d1 * z[3];
      out[4] = d1 * z[4];
    }
    float* o = Hout + ((size_t)(p0 + lp) * P2) * d_out + f;
    for (int p = 0; p < P2; ++p) {
      float v = out[p];
      if (res) v = (v + in[p * d_in + f]) * kRsqrt2;
      o[p * d_out] = v;
    }
  }
}

// Value-only two-electron layer: one thread per pair, all d_out features in
// registers, weights broadcast from shared memory.
template <int DIN, int DOUT>
__global__ void __launch_bounds__(128) k_pair_layer_value(int npairs, const float* __restrict__ Hin,
                                                          const float* __restrict__ W,
                                                          const float* __restrict__ b,
                                                          float* __restrict__ Hout) {
  __shared__ float Ws[DIN * DOUT];
  __shared__ float bs[DOUT];
  for (int e = threadIdx.x; e < DIN * DOUT; e += blockDim.x) Ws[e] = W[e];
  for (int e = threadIdx.x; e < DOUT; e += blockDim.x) bs[e] = b[e];
  __syncthreads();
  const int pr = blockIdx.x * blockDim.x + threadIdx.x;
  if (pr >= npairs) return;
  float x[DIN];
  const float4* src = reinterpret_cast<const float4*>(Hin + (size_t)pr * DIN);
#pragma unroll
  for (int q = 0; q < DIN / 4; ++q) {
    float4 v = src[q];
    x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
  }
  float4* dst = reinterpret_cast<float4*>(Hout + (size_t)pr * DOUT);
#pragma unroll
  for (int f4 = 0; f4 < DOUT / 4; ++f4) {
    float z[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) z[e] = bs[4 * f4 + e];
#pragma unroll
    for (int k = 0; k < DIN; ++k) {
      const float4 w = *reinterpret_cast<const float4*>(&Ws[k * DOUT + 4 * f4]);
      z[0] = fmaf(x[k], w.x, z[0]);
      z[1] = fmaf(x[k], w.y, z[1]);
      z[2] = fmaf(x[k], w.z, z[2]);
      z[3] = fmaf(x[k], w.w, z[3]);
    }
    float4 o;
    o.x = tanhf(z[0]); o.y = tanhf(z[1]); o.z = tanhf(z[2]); o.w = tanhf(z[3]);
    if (DIN == DOUT) {
      o.x = (o.x + x[4 * f4]) * kRsqrt2;
      o.y = (o.y + x[4 * f4 + 1]) * kRsqrt2;
      o.z = (o.z + x[4 * f4 + 2]) * kRsqrt2;
      o.w = (o.w + x[4 * f4 + 3]) * kRsqrt2;
    }
    dst[f4] = o;
  }
}

// Value-only two-electron layer fused with the spin means of its output (the
// next layer's <h2>): one block per walker.  Outputs are staged in shared
// memory and reduced in a fixed order, so the means are deterministic.
template <int DIN, int DOUT, class Out>
__global__ void __launch_bounds__(256) k_pair_layer_mean(int n, int n_up, int C, const float* __restrict__ Hin,
                                                         const float* __restrict__ W, const float* __restrict__ b,
                                                         float* __restrict__ Hout, int g2p, Out G2) {
  extern __shared__ float shp[];
  float* Ws = shp;                  // [DIN][DOUT]
  float* Os = Ws + DIN * DOUT;      // [n*n][DOUT]
  for (int e = threadIdx.x; e < DIN * DOUT; e += blockDim.x) Ws[e] = W[e];
  __syncthreads();
  const int w = blockIdx.x;
  const int np = n * n;
  for (int pr = threadIdx.x; pr < np; pr += blockDim.x) {
    const size_t gp = (size_t)w * np + pr;
    float x[DIN];
    const float4* src = reinterpret_cast<const float4*>(Hin + gp * DIN);
#pragma unroll
    for (int q = 0; q < DIN / 4; ++q) {
      float4 v = src[q];
      x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
    }
    float4* dst = reinterpret_cast<float4*>(Hout + gp * DOUT);
#pragma unroll
    for (int f4 = 0; f4 < DOUT / 4; ++f4) {
      float z[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) z[e] = b[4 * f4 + e];
#pragma unroll
      for (int k = 0; k < DIN; ++k) {
        const float4 wv = *reinterpret_cast<const float4*>(&Ws[k * DOUT + 4 * f4]);
        z[0] = fmaf(x[k], wv.x, z[0]);
        z[1] = fmaf(x[k], wv.y, z[1]);
        z[2] = fmaf(x[k], wv.z, z[2]);
        z[3] = fmaf(x[k], wv.w, z[3]);
      }
      float4 o;
      o.x = tanhf(z[0]); o.y = tanhf(z[1]); o.z = tanhf(z[2]); o.w = tanhf(z[3]);
      if (DIN == DOUT) {
        o.x = (o.x + x[4 * f4]) * kRsqrt2;
        o.y = (o.y + x[4 * f4 + 1]) * kRsqrt2;
        o.z = (o.z + x[4 * f4 + 2]) * kRsqrt2;
        o.w = (o.w + x[4 * f4 + 3]) * kRsqrt2;
      }
      dst[f4] = o;
      *reinterpret_cast<float4*>(&Os[pr * DOUT + 4 * f4]) = o;
    }
  }
  __syncthreads();
  // <h2>_s[i] = mean over a in channel s of h2[a, i]  (first index averaged)
  for (int e = threadIdx.x; e < n * g2p; e += blockDim.x) {
    const int i = e / g2p, col = e % g2p;
    float v = 0.f;
    if (col < C * DOUT) {
      const int sc = col / DOUT, f = col % DOUT;
      const int a0 = C == 1 ? 0 : (sc == 0 ? 0 : n_up), a1 = C == 1 ? n : (sc == 0 ? n_up : n);
      float acc = 0.f;
      for (int a = a0; a < a1; ++a) acc += Os[(a * n + i) * DOUT + f];
      v = acc / (float)(a1 - a0);
    }
    G2.put((size_t)w * n + i, col, v);
  }
}

// Whole value-only two-electron stream of one walker per block: every pair
// layer h2 <- tanh(W2 h2 + b2) (+ residual) with the activations kept in
// shared memory, and after each layer the spin means over the first electron
// index that the next one-electron layer reads (G2 of layers 1..nl).  Pair
// activations never leave the SM.  Widths: input 4 or 32, output 32.
// z[0..3] += x * W[0..7] as packed pairs (8 consecutive weights of one row).
__device__ __forceinline__ void pair_fma8(float x, const float* __restrict__ w, float2* z) {
  const float2 xx = make_float2(x, x);
  const float4* w4 = reinterpret_cast<const float4*>(w);
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const float4 wv = w4[q];
    z[2 * q] = __ffma2_rn(xx, make_float2(wv.x, wv.y), z[2 * q]);
    z[2 * q + 1] = __ffma2_rn(xx, make_float2(wv.z, wv.w), z[2 * q + 1]);
  }
}

// tanh for the two-electron stream: split_tanh in the mixed form (FAST),
// otherwise tanhf.
template <bool FAST>
__device__ __forceinline__ float pair_tanh(float x) {
  if constexpr (FAST) return split_tanh(x);
  else return tanhf(x);
}

template <class Out>
__global__ void __launch_bounds__(256) k_pair_stream_value(PairStreamArgs a, PairStreamOut<Out> o) {
  constexpr bool kFastTanh = std::is_same<Out, StSplit>::value;
  extern __shared__ float shs[];
  constexpr int DO = 32, RS = 36;  // row stride 36 floats: conflict-free 16-byte accesses
  float* Ws = shs;                         // [nl][32][32]
  float* bs = Ws + a.nl * DO * DO;         // [nl][32]
  float* Os = bs + a.nl * DO;              // [n*n][RS]
  for (int l = 0; l < a.nl; ++l) {
    for (int e = threadIdx.x; e < a.din[l] * DO; e += blockDim.x) Ws[l * DO * DO + e] = a.W[l][e];
    for (int e = threadIdx.x; e < DO; e += blockDim.x) bs[l * DO + e] = a.b[l][e];
  }
  __syncthreads();
  const int n = a.n, np = n * n, w = blockIdx.x;
  for (int l = 0; l < a.nl; ++l) {
    const float* Wl = Ws + l * DO * DO;
    const float* bl = bs + l * DO;
    const int din = a.din[l];
    for (int pr = threadIdx.x; pr < np; pr += blockDim.x) {
      float x[DO];
      float* row = Os + pr * RS;
      if (l == 0) {
        const float4* src = reinterpret_cast<const float4*>(a.H0 + ((size_t)w * np + pr) * din);
#pragma unroll
        for (int q = 0; q < DO / 4; ++q) {
          const float4 v = q < din / 4 ? __ldg(src + q) : make_float4(0.f, 0.f, 0.f, 0.f);
          x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
        }
      } else {
#pragma unroll
        for (int q = 0; q < DO / 4; ++q) {
          const float4 v = *reinterpret_cast<const float4*>(row + 4 * q);
          x[4 * q] = v.x; x[4 * q + 1] = v.y; x[4 * q + 2] = v.z; x[4 * q + 3] = v.w;
        }
      }
      // 8 outputs per pass: each input broadcast feeds 4 packed FMAs
      // (__ffma2_rn rounds each lane like fmaf, so the sums are unchanged)
#pragma unroll
      for (int f8 = 0; f8 < DO / 8; ++f8) {
        float2 z[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) z[e] = make_float2(bl[8 * f8 + 2 * e], bl[8 * f8 + 2 * e + 1]);
        if (din == 4) {
#pragma unroll
          for (int k = 0; k < 4; ++k) pair_fma8(x[k], Wl + k * DO + 8 * f8, z);
        } else {
#pragma unroll
          for (int k = 0; k < DO; ++k) pair_fma8(x[k], Wl + k * DO + 8 * f8, z);
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          float4 v;
          v.x = pair_tanh<kFastTanh>(z[2 * q].x);
          v.y = pair_tanh<kFastTanh>(z[2 * q].y);
          v.z = pair_tanh<kFastTanh>(z[2 * q + 1].x);
          v.w = pair_tanh<kFastTanh>(z[2 * q + 1].y);
          if (din == DO) {  // residual: this thread's own row, not yet overwritten
            const float4 r = *reinterpret_cast<const float4*>(row + 8 * f8 + 4 * q);
            v.x = (v.x + r.x) * kRsqrt2;
            v.y = (v.y + r.y) * kRsqrt2;
            v.z = (v.z + r.z) * kRsqrt2;
            v.w = (v.w + r.w) * kRsqrt2;
          }
          *reinterpret_cast<float4*>(row + 8 * f8 + 4 * q) = v;
        }
      }
    }
    __syncthreads();
    // <h2>_s[i] = mean over a in channel s of h2[a, i]  (first index averaged)
    const int g2p = a.g2p[l];
    for (int e = threadIdx.x; e < n * g2p; e += blockDim.x) {
      const int i = e / g2p, col = e % g2p;
      float v = 0.f;
      if (col < a.C * DO) {
        const int sc = col / DO, f = col % DO;
        const int a0 = a.C == 1 ? 0 : (sc == 0 ? 0 : a.n_up), a1 = a.C == 1 ? n : (sc == 0 ? a.n_up : n);
        float acc = 0.f;
        for (int aa = a0; aa < a1; ++aa) acc += Os[(aa * n + i) * RS + f];
        v = acc / (float)(a1 - a0);
      }
      o.G2[l].put((size_t)w * n + i, col, v);
    }
    __syncthreads();
  }
}

size_t pair_stream_smem(int n, int nl) { return sizeof(float) * ((size_t)nl * (32 * 32 + 32) + (size_t)n * n * 36); }

// ---------------------------------------------------------------------
// Mixed form of the same stream on the tensor cores: every 32-wide pair
// layer of a 16-pair tile is a 16 x 32 x K product done by warp-level
// m16n8k16 BF16 MMAs, each operand split into hi + lo BF16 parts
// (lo*hi + hi*lo + hi*hi, FP32 accumulation), like the split-BF16 one-electron
// layers.  The layers are a chain of tiny products whose operands live in
// registers: an accumulator tile maps element for element onto the next
// layer's A operand, so no shared-memory operand staging is needed.  The
// activations pass through shared memory only for the spin means between
// layers.  Fragment layouts (PTX ISA, mma.m16n8k16 .bf16): g = lane / 4,
// t = lane % 4; A regs (row g | g+8, cols 2t..2t+1 | 2t+8..2t+9), B regs
// (k 2t..2t+1 | 2t+8..2t+9, col g), C (row g | g+8, cols 2t..2t+1).
// ---------------------------------------------------------------------
constexpr int kPairMmaWarps = 8;
constexpr int kPairRS = 40;  // activation row stride (floats): conflict-free 8-byte fragment accesses

__device__ __forceinline__ void split_bf16x2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

__device__ __forceinline__ void mma_16816_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__global__ void k_pair_frags(const float* __restrict__ W, int din, uint4* __restrict__ out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 256) return;
  const int ks = (e >> 7) & 1, nt = (e >> 5) & 3, ln = e & 31;
  const int col = 8 * nt + (ln >> 2), k0 = 16 * ks + 2 * (ln & 3);
  auto wv = [&](int k) { return k < din ? W[k * 32 + col] : 0.f; };
  uint32_t h0, l0, h1, l1;
  split_bf16x2(wv(k0), wv(k0 + 1), h0, l0);
  split_bf16x2(wv(k0 + 8), wv(k0 + 9), h1, l1);
  out[e] = make_uint4(h0, h1, l0, l1);
}

cudaError_t launch_pair_frags(cudaStream_t s, const float* W, int din, uint4* out) {
  if (din < 1 || din > 32) return cudaErrorInvalidValue;
  k_pair_frags<<<1, 256, 0, s>>>(W, din, out);
  return cudaGetLastError();
}

static size_t pair_stream_mma_smem(int n, int nl) {
  const size_t mt = ((size_t)n * n + 15) / 16;
  return sizeof(uint4) * (size_t)nl * 256 + sizeof(float) * ((size_t)nl * 32 + mt * 16 * kPairRS);
}

__global__ void __launch_bounds__(kPairMmaWarps * 32, 4) k_pair_stream_mma(PairStreamArgs a, PairStreamOut<StSplit> o) {
  extern __shared__ uint4 shq[];
  uint4* Wf = shq;                                          // [nl][ks 2][nt 4][lane 32] {b0 hi, b1 hi, b0 lo, b1 lo}
  float* bs = reinterpret_cast<float*>(Wf + a.nl * 256);   // [nl][32]
  float* Os = bs + a.nl * 32;                               // [tiles * 16][kPairRS]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int n = a.n, np = n * n, mt = (np + 15) / 16, w = blockIdx.x;
  for (int e = threadIdx.x; e < a.nl * 256; e += blockDim.x) Wf[e] = __ldg(a.Wf[e >> 8] + (e & 255));
  for (int e = threadIdx.x; e < a.nl * 32; e += blockDim.x) bs[e] = a.b[e >> 5][e & 31];
  __syncthreads();
  for (int l = 0; l < a.nl; ++l) {
    const uint4* Wl = Wf + l * 256;
    const float* bl = bs + l * 32;
    const int din = a.din[l];
    const int nks = din > 16 ? 2 : 1;
    float2 bias[4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) bias[nt] = *reinterpret_cast<const float2*>(bl + 8 * nt + 2 * t);
    for (int tile = warp; tile < mt; tile += kPairMmaWarps) {
      const int r0 = tile * 16 + g, r1 = r0 + 8;
      // x[ks] = {(r0, c), (r0, c+1), (r1, c), (r1, c+1), (r0, c+8), (r0, c+9), (r1, c+8), (r1, c+9)},
      // c = 16 ks + 2t: the A operand and, for 32-wide inputs, the residual
      float x[2][8];
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int r = (q & 1) ? r1 : r0;
          const int c = 16 * ks + 2 * t + ((q & 2) ? 8 : 0);
          float2 v = make_float2(0.f, 0.f);
          if (ks < nks) {
            if (l == 0) {
              if (r < np && c < din)
                v = __ldg(reinterpret_cast<const float2*>(a.H0 + ((size_t)w * np + r) * din + c));
            } else {
              v = *reinterpret_cast<const float2*>(Os + r * kPairRS + c);
            }
          }
          x[ks][2 * q] = v.x;
          x[ks][2 * q + 1] = v.y;
        }
      }
      uint32_t ahi[2][4], alo[2][4];
#pragma unroll
      for (int ks = 0; ks < 2; ++ks)
#pragma unroll
        for (int q = 0; q < 4; ++q) split_bf16x2(x[ks][2 * q], x[ks][2 * q + 1], ahi[ks][q], alo[ks][q]);
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        float acc[4];
        acc[0] = acc[2] = bias[nt].x;
        acc[1] = acc[3] = bias[nt].y;
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
          if (ks < nks) {
            const uint4 bw = Wl[(ks * 4 + nt) * 32 + lane];
            mma_16816_bf16(acc, alo[ks], bw.x, bw.y);
            mma_16816_bf16(acc, ahi[ks], bw.z, bw.w);
            mma_16816_bf16(acc, ahi[ks], bw.x, bw.y);
          }
        }
        float v[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) v[e] = pair_tanh<true>(acc[e]);
        if (din == 32) {
          // the input at this output's position: k-slice nt / 2, column half nt % 2
          const float* xr = &x[nt >> 1][(nt & 1) * 4];
          v[0] = (v[0] + xr[0]) * kRsqrt2;
          v[1] = (v[1] + xr[1]) * kRsqrt2;
          v[2] = (v[2] + xr[2]) * kRsqrt2;
          v[3] = (v[3] + xr[3]) * kRsqrt2;
        }
        *reinterpret_cast<float2*>(Os + r0 * kPairRS + 8 * nt + 2 * t) = make_float2(v[0], v[1]);
        *reinterpret_cast<float2*>(Os + r1 * kPairRS + 8 * nt + 2 * t) = make_float2(v[2], v[3]);
      }
    }
    __syncthreads();
    // <h2>_s[i] = mean over a in channel s of h2[a, i]  (first index
    // averaged): one (i, feature) per thread, both channels in one pass
    const int g2p = a.g2p[l];
    for (int e = threadIdx.x; e < n * 32; e += blockDim.x) {
      const int i = e >> 5, f = e & 31;
      const size_t row = (size_t)w * n + i;
      if (a.C == 1) {
        float acc = 0.f;
        for (int aa = 0; aa < n; ++aa) acc += Os[(aa * n + i) * kPairRS + f];
        o.G2[l].put(row, f, acc / (float)n);
      } else {
        float s0 = 0.f, s1 = 0.f;
        for (int aa = 0; aa < a.n_up; ++aa) s0 += Os[(aa * n + i) * kPairRS + f];
        for (int aa = a.n_up; aa < n; ++aa) s1 += Os[(aa * n + i) * kPairRS + f];
        o.G2[l].put(row, f, s0 / (float)a.n_up);
        o.G2[l].put(row, 32 + f, s1 / (float)(n - a.n_up));
      }
    }
    const int padc = g2p - a.C * 32;  // zero padding columns
    for (int e = threadIdx.x; e < n * padc; e += blockDim.x)
      o.G2[l].put((size_t)w * n + e / padc, a.C * 32 + e % padc, 0.f);
    __syncthreads();
  }
}

template <class Out>
cudaError_t launch_pair_stream_value(cudaStream_t s, int B, const PairStreamArgs& a, const PairStreamOut<Out>& o) {
  if (a.nl < 1 || a.nl > kPairStreamMax) return cudaErrorNotSupported;
  int dev;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if constexpr (std::is_same<Out, StSplit>::value) {
    bool ok = pair_stream_mma_smem(a.n, a.nl) <= 200 * 1024;
    for (int l = 0; l < a.nl; ++l) ok = ok && (a.din[l] == 32 || (a.din[l] == 4 && l == 0));
    if (ok) {
      static int mma_dev = -1;
      if (mma_dev != dev) {
        e = cudaFuncSetAttribute(k_pair_stream_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        mma_dev = dev;
      }
      k_pair_stream_mma<<<B, kPairMmaWarps * 32, pair_stream_mma_smem(a.n, a.nl), s>>>(a, o);
      return cudaGetLastError();
    }
  }
  const size_t sm = pair_stream_smem(a.n, a.nl);
  if (sm > 200 * 1024) return cudaErrorNotSupported;
  static int attr_dev = -1;
  if (attr_dev != dev) {
    e = cudaFuncSetAttribute(k_pair_stream_value<Out>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    attr_dev = dev;
  }
  k_pair_stream_value<Out><<<B, 256, sm, s>>>(a, o);
  return cudaGetLastError();
}
template cudaError_t launch_pair_stream_value<StF32>(cudaStream_t, int, const PairStreamArgs&,
                                                     const PairStreamOut<StF32>&);
template cudaError_t launch_pair_stream_value<StSplit>(cudaStream_t, int, const PairStreamArgs&,
                                                       const PairStreamOut<StSplit>&);

template <class Out>
cudaError_t launch_pair_layer_mean(cudaStream_t s, int B, int n, int n_up, int C, int d_in, int d_out,
                                   const float* Hin, const float* W, const float* b, float* Hout, int g2p,
                                   Out G2) {
  const size_t sm = sizeof(float) * ((size_t)d_in * d_out + (size_t)n * n * d_out);
  if (sm > 200 * 1024) return cudaErrorNotSupported;
  static int attr_dev = -1;
  int dev;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
#define QMC_PLM(DI, DO)                                                                              \
  if (d_in == DI && d_out == DO) {                                                                   \
    if (attr_dev != dev) {                                                                           \
      e = cudaFuncSetAttribute(k_pair_layer_mean<DI, DO, Out>,                                       \
                               cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);             \
      if (e != cudaSuccess) return e;                                                                \
    }                                                                                                \
    k_pair_layer_mean<DI, DO, Out><<<B, 256, sm, s>>>(n, n_up, C, Hin, W, b, Hout, g2p, G2);         \
    attr_dev = dev;                                                                                  \
    return cudaGetLastError();                                                                       \
  }
  QMC_PLM(4, 32)
  QMC_PLM(32, 32)
#undef QMC_PLM
  return cudaErrorNotSupported;
}
template cudaError_t launch_pair_layer_mean<StF32>(cudaStream_t, int, int, int, int, int, int, const float*,
                                                   const float*, const float*, float*, int, StF32);
template cudaError_t launch_pair_layer_mean<StSplit>(cudaStream_t, int, int, int, int, int, int, const float*,
                                                     const float*, const float*, float*, int, StSplit);

// Tangent form (P2 = 5 planes: value, Laplacian, three gradient components),
// 32 outputs: 32 pairs per block, each thread four features of one pair, so
// every 4 inputs cost 5 + 4 16-byte shared loads for 80 FMAs and the outputs
// leave as 16-byte stores.  Same arithmetic order per output as k_pair_layer.
template <int DIN>
__global__ void __launch_bounds__(256) k_pair_layer_t5(int npairs, const float* __restrict__ Hin,
                                                       const float* __restrict__ W, const float* __restrict__ b,
                                                       float* __restrict__ Hout) {
  constexpr int P2 = 5, DO = 32, PPB = 32;
  constexpr int IS = P2 * DIN + 4;  // per-pair stride (floats): four pairs per warp on distinct banks
  __shared__ __align__(16) float Ws[DIN * DO];
  __shared__ __align__(16) float Is[PPB * IS];
  for (int e = threadIdx.x; e < DIN * DO; e += blockDim.x) Ws[e] = W[e];
  const int p0 = blockIdx.x * PPB;
  const int np = min(PPB, npairs - p0);
  constexpr int V4 = P2 * DIN / 4;  // float4 per pair
  const float4* src = reinterpret_cast<const float4*>(Hin + (size_t)p0 * P2 * DIN);
  for (int e = threadIdx.x; e < np * V4; e += blockDim.x) {
    const int pr = e / V4, q = e - pr * V4;
    *reinterpret_cast<float4*>(Is + pr * IS + 4 * q) = __ldg(src + e);
  }
  __syncthreads();
  const int lp = threadIdx.x >> 3, f0 = 4 * (threadIdx.x & 7);
  if (lp >= np) return;
  const float* in = Is + lp * IS;
  float z[P2][4];
#pragma unroll
  for (int p = 0; p < P2; ++p)
#pragma unroll
    for (int c = 0; c < 4; ++c) z[p][c] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < DIN; k0 += 4) {
    float4 x[P2];
#pragma unroll
    for (int p = 0; p < P2; ++p) x[p] = *reinterpret_cast<const float4*>(in + p * DIN + k0);
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const float4 w = *reinterpret_cast<const float4*>(Ws + (k0 + kk) * DO + f0);
#pragma unroll
      for (int p = 0; p < P2; ++p) {
        const float xv = kk == 0 ? x[p].x : kk == 1 ? x[p].y : kk == 2 ? x[p].z : x[p].w;
        z[p][0] = fmaf(xv, w.x, z[p][0]);
        z[p][1] = fmaf(xv, w.y, z[p][1]);
        z[p][2] = fmaf(xv, w.z, z[p][2]);
        z[p][3] = fmaf(xv, w.w, z[p][3]);
      }
    }
  }
  float out[P2][4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float h = tanhf(z[0][c] + b[f0 + c]);
    const float d1 = 1.f - h * h, d2 = -2.f * h * d1;
    const float S = z[2][c] * z[2][c] + z[3][c] * z[3][c] + z[4][c] * z[4][c];
    out[0][c] = h;
    out[1][c] = d1 * z[1][c] + d2 * S;
    out[2][c] = d1 * z[2][c];
    out[3][c] = d1 * z[3][c];
    out[4][c] = d1 * z[4][c];
  }
  float* o = Hout + (size_t)(p0 + lp) * P2 * DO + f0;
#pragma unroll
  for (int p = 0; p < P2; ++p) {
    float4 v = make_float4(out[p][0], out[p][1], out[p][2], out[p][3]);
    if (DIN == DO) {
      const float4 r = *reinterpret_cast<const float4*>(in + p * DIN + f0);
      v.x = (v.x + r.x) * kRsqrt2;
      v.y = (v.y + r.y) * kRsqrt2;
      v.z = (v.z + r.z) * kRsqrt2;
      v.w = (v.w + r.w) * kRsqrt2;
    }
    *reinterpret_cast<float4*>(o + p * DO) = v;
  }
}

// Tangent pair layer fused with the next one-electron layer's pair means
// (k_pair_layer_t5 followed by k_mean_h2 on its output), one block of 16 n
// threads per walker: thread (i, q) owns features 2q, 2q+1 of every pair
// (a, i) and walks a in electron order, with pair row a (all i) staged in
// shared memory by cp.async one row ahead (two buffers).  It writes the pair outputs (same arithmetic order as
// k_pair_layer_t5), scatters each pair's gradient planes into the Jacobian
// rows t = 2 + 3a + c of row i of G2 (channel of a, times 1/n_s; zeros in
// the other channel), and keeps the channel sums of the five planes over a
// in registers for rows t = 0 (mean), 1 (twice the mean Laplacian) and the
// rows of electron i itself (minus the mean gradient), as k_mean_h2 forms
// them.  Padding rows T..Tp-1 are written as zeros.  Every G2 element is
// written once, so no atomics and no ordering between threads are involved.
// Two adjacent features of one row (c even): one 8-byte (FP32) or two 4-byte
// (split bf16 planes) stores.
__device__ __forceinline__ void put2(const StF32& Y, size_t r, int c, float x0, float x1) {
  *reinterpret_cast<float2*>(Y.p + r * Y.ld + c) = make_float2(x0, x1);
}
__device__ __forceinline__ void put2(const StSplit& Y, size_t r, int c, float x0, float x1) {
  const __nv_bfloat162 hi = __floats2bfloat162_rn(x0, x1);
  const __nv_bfloat162 lo = __floats2bfloat162_rn(x0 - __low2float(hi), x1 - __high2float(hi));
  __nv_bfloat16* p = Y.p + r * Y.ld + c;
  *reinterpret_cast<__nv_bfloat162*>(p) = hi;
  *reinterpret_cast<__nv_bfloat162*>(p + Y.plane) = lo;
}

template <int DIN, class Out>
__global__ void __launch_bounds__(512) k_pair_layer_t5_mean(int n, int n_up, int C, int Tp, int T,
                                                             const float* __restrict__ Hin,
                                                             const float* __restrict__ W,
                                                             const float* __restrict__ b, float* __restrict__ Hout,
                                                             int g2p, Out G2) {
  constexpr int P2 = 5, DO = 32;
  constexpr int RS = P2 * DIN + 4;  // staged pair stride (floats)
  extern __shared__ __align__(16) float smp[];
  float* Ws = smp;               // [DIN][32]
  float* Is0 = Ws + DIN * DO;    // [2][n][RS]: pairs (a, i) of rows a and a + 1
  const int w = blockIdx.x;
  const int i = threadIdx.x >> 4, q = threadIdx.x & 15, f0 = 2 * q;
  for (int e = threadIdx.x; e < DIN * DO; e += blockDim.x) Ws[e] = W[e];
  const float b0 = b[f0], b1 = b[f0 + 1];
  // channel sums of the five planes (channel 0 / 1 of the first electron)
  float acc0[P2][2], acc1[P2][2];
#pragma unroll
  for (int p = 0; p < P2; ++p) acc0[p][0] = acc0[p][1] = acc1[p][0] = acc1[p][1] = 0.f;
  const size_t row_i = ((size_t)w * n + i) * Tp;  // G2 rows of electron i
  const float inv0 = 1.0f / (float)(C == 1 ? n : n_up), inv1 = C == 1 ? 0.f : 1.0f / (float)(n - n_up);
  constexpr int V4 = P2 * DIN / 4;
  auto stage = [&](int a, float* dst) {
    const float* src = Hin + ((size_t)w * n + a) * n * P2 * DIN;
    for (int e = threadIdx.x; e < n * V4; e += blockDim.x) {
      const int pi = e / V4, qq = e - pi * V4;
      ptx::cp_async16(dst + pi * RS + 4 * qq, src + 4 * e);
    }
  };
  stage(0, Is0);
  ptx::cp_async_commit();
  for (int a = 0; a < n; ++a) {
    __syncthreads();  // every thread is done with row a - 1, whose buffer row a + 1 takes
    if (a + 1 < n) stage(a + 1, Is0 + ((a + 1) & 1) * n * RS);
    ptx::cp_async_commit();  // (possibly empty) group of row a + 1
    ptx::cp_async_wait<1>();  // this thread's copies of row a have landed
    __syncthreads();          // and every thread's
    const float* in = Is0 + (a & 1) * n * RS + i * RS;
    float z[P2][2];
#pragma unroll
    for (int p = 0; p < P2; ++p) z[p][0] = z[p][1] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < DIN; k0 += 4) {
      float4 x[P2];
#pragma unroll
      for (int p = 0; p < P2; ++p) x[p] = *reinterpret_cast<const float4*>(in + p * DIN + k0);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const float2 wv = *reinterpret_cast<const float2*>(Ws + (k0 + kk) * DO + f0);
#pragma unroll
        for (int p = 0; p < P2; ++p) {
          const float xv = kk == 0 ? x[p].x : kk == 1 ? x[p].y : kk == 2 ? x[p].z : x[p].w;
          z[p][0] = fmaf(xv, wv.x, z[p][0]);
          z[p][1] = fmaf(xv, wv.y, z[p][1]);
        }
      }
    }
    float out[P2][2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const float h = tanhf(z[0][c] + (c == 0 ? b0 : b1));
      const float d1 = 1.f - h * h, d2 = -2.f * h * d1;
      const float S = z[2][c] * z[2][c] + z[3][c] * z[3][c] + z[4][c] * z[4][c];
      out[0][c] = h;
      out[1][c] = d1 * z[1][c] + d2 * S;
      out[2][c] = d1 * z[2][c];
      out[3][c] = d1 * z[3][c];
      out[4][c] = d1 * z[4][c];
    }
    float* o = Hout ? Hout + (((size_t)w * n + a) * n + i) * P2 * DO + f0 : nullptr;
    const int sa = (C == 2 && a >= n_up) ? 1 : 0;
    const float inva = sa ? inv1 : inv0;
#pragma unroll
    for (int p = 0; p < P2; ++p) {
      float2 v = make_float2(out[p][0], out[p][1]);
      if (DIN == DO) {
        const float2 r = *reinterpret_cast<const float2*>(in + p * DIN + f0);
        v.x = (v.x + r.x) * kRsqrt2;
        v.y = (v.y + r.y) * kRsqrt2;
      }
      if (o) *reinterpret_cast<float2*>(o + p * DO) = v;
      if (sa == 0) {  // uniform over the block: keeps both sums in registers
        acc0[p][0] += v.x;
        acc0[p][1] += v.y;
      } else {
        acc1[p][0] += v.x;
        acc1[p][1] += v.y;
      }
      if (p >= 2 && a != i && 2 + 3 * a + (p - 2) < T) {
        // Jacobian row of electron a, direction p - 2: the pair's gradient
        const size_t r = row_i + 2 + 3 * a + (p - 2);
        put2(G2, r, sa * DO + f0, v.x * inva, v.y * inva);
        if (C == 2) put2(G2, r, (1 - sa) * DO + f0, 0.f, 0.f);
      }
    }
  }
  // rows 0 (value), 1 (Laplacian) and electron i's own Jacobian rows
  auto emit = [&](const float (&A)[P2][2], int sc, float inv) {
    const int col = sc * DO + f0;
    put2(G2, row_i, col, A[0][0] * inv, A[0][1] * inv);
    put2(G2, row_i + 1, col, 2.0f * A[1][0] * inv, 2.0f * A[1][1] * inv);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (2 + 3 * i + d < T) put2(G2, row_i + 2 + 3 * i + d, col, -A[2 + d][0] * inv, -A[2 + d][1] * inv);
  };
  emit(acc0, 0, inv0);
  if (C == 2) emit(acc1, 1, inv1);
  // padding columns and rows (g2p is even)
  for (int col = C * DO + 2 * q; col < g2p; col += 32)
    for (int t = 0; t < T; ++t) put2(G2, row_i + t, col, 0.f, 0.f);
  for (int t = T; t < Tp; ++t)
    for (int col = 2 * q; col < g2p; col += 32) put2(G2, row_i + t, col, 0.f, 0.f);
}

template <class Out>
cudaError_t launch_pair_layer_mean_fl(cudaStream_t s, int B, int n, int n_up, int C, int Tp, int T, int d_in,
                                      int d_out, const float* Hin, const float* W, const float* b, float* Hout,
                                      int g2p, Out G2) {
  if (d_out != 32 || (d_in != 4 && d_in != 32) || n < 1 || 16 * n > 512 || T != 3 * n + 2 ||
      ((uintptr_t)Hin & 15) != 0)
    return cudaErrorNotSupported;
  const size_t sm = sizeof(float) * ((size_t)d_in * 32 + 2 * (size_t)n * (5 * d_in + 4));
  if (sm > 48 * 1024) return cudaErrorNotSupported;
  if (d_in == 4)
    k_pair_layer_t5_mean<4, Out><<<B, 16 * n, sm, s>>>(n, n_up, C, Tp, T, Hin, W, b, Hout, g2p, G2);
  else
    k_pair_layer_t5_mean<32, Out><<<B, 16 * n, sm, s>>>(n, n_up, C, Tp, T, Hin, W, b, Hout, g2p, G2);
  return cudaGetLastError();
}
template cudaError_t launch_pair_layer_mean_fl<StF32>(cudaStream_t, int, int, int, int, int, int, int, int,
                                                      const float*, const float*, const float*, float*, int, StF32);
template cudaError_t launch_pair_layer_mean_fl<StSplit>(cudaStream_t, int, int, int, int, int, int, int, int,
                                                        const float*, const float*, const float*, float*, int,
                                                        StSplit);

cudaError_t launch_pair_layer(cudaStream_t s, int npairs, int P2, int d_in, int d_out,
                              const float* Hin, const float* W, const float* b, float* Hout) {
  if (P2 == 5 && d_out == 32 && (d_in == 4 || d_in == 32) && ((uintptr_t)Hin & 15) == 0 &&
      ((uintptr_t)Hout & 15) == 0) {
    const unsigned grid = (unsigned)((npairs + 31) / 32);
    if (d_in == 4) k_pair_layer_t5<4><<<grid, 256, 0, s>>>(npairs, Hin, W, b, Hout);
    else k_pair_layer_t5<32><<<grid, 256, 0, s>>>(npairs, Hin, W, b, Hout);
    return cudaGetLastError();
  }
  if (P2 == 1) {
    const unsigned grid = (unsigned)((npairs + 127) / 128);
    if (d_in == 4 && d_out == 32) {
      k_pair_layer_value<4, 32><<<grid, 128, 0, s>>>(npairs, Hin, W, b, Hout);
      return cudaGetLastError();
    }
    if (d_in == 32 && d_out == 32) {
      k_pair_layer_value<32, 32><<<grid, 128, 0, s>>>(npairs, Hin, W, b, Hout);
      return cudaGetLastError();
    }
  }
  int ppb = 256 / d_out;
  if (ppb < 1) return cudaErrorInvalidValue;
  size_t sm = sizeof(float) * (d_in * d_out + ppb * P2 * d_in);
  static int n_sms = 0;
  if (!n_sms) cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, 0);
  int nchunks = (npairs + ppb - 1) / ppb;
  int grid = std::min(nchunks, std::max(1, n_sms) * 8);
  k_pair_layer<<<grid, ppb * d_out, sm, s>>>(npairs, P2, d_in, d_out, Hin, W, b, Hout);
  return cudaGetLastError();
}

// =====================================================================
// spin-channel means (src/jaqmc/wavefunction/backbone/ferminet.py:65-90)
// =====================================================================
__device__ __forceinline__ void channel_range(int s, int C, int n, int n_up, int* a0, int* a1) {
  if (C == 1) { *a0 = 0; *a1 = n; return; }
  *a0 = s == 0 ? 0 : n_up;
  *a1 = s == 0 ? n_up : n;
}

template <class In, class Out>
__global__ void k_mean_h1(int B, int n, int n_up, int C, int Tp, int d, In X, int g1p, Out G1) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t total = (size_t)B * Tp * g1p;
  if (e >= total) return;
  int col = (int)(e % g1p);
  size_t wt = e / g1p;
  int t = (int)(wt % Tp);
  int w = (int)(wt / Tp);
  float v = 0.f;
  if (col < C * d) {
    int s = col / d, f = col % d, a0, a1;
    channel_range(s, C, n, n_up, &a0, &a1);
    float acc = 0.f;
    for (int i = a0; i < a1; ++i) acc += X.get(((size_t)w * n + i) * Tp + t, f);
    v = acc / (float)(a1 - a0);
  }
  G1.put(wt, col, v);
}

// 8 consecutive features of one row (16-byte aligned) <-> registers.
__device__ __forceinline__ void load8(const StF32& X, size_t r, int c, float* v) {
  const float4* p = reinterpret_cast<const float4*>(X.p + r * X.ld + c);
  const float4 a = __ldg(p), b = __ldg(p + 1);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void load8(const StSplit& X, size_t r, int c, float* v) {
  const __nv_bfloat16* p = X.p + r * X.ld + c;
  const uint4 h = __ldg(reinterpret_cast<const uint4*>(p));
  const uint4 l = __ldg(reinterpret_cast<const uint4*>(p + X.plane));
  const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[2 * k] = __uint_as_float(hw[k] << 16) + __uint_as_float(lw[k] << 16);
    v[2 * k + 1] = __uint_as_float(hw[k] & 0xffff0000u) + __uint_as_float(lw[k] & 0xffff0000u);
  }
}
__device__ __forceinline__ void store8(const StF32& Y, size_t r, int c, const float* v) {
  float4* p = reinterpret_cast<float4*>(Y.p + r * Y.ld + c);
  p[0] = make_float4(v[0], v[1], v[2], v[3]);
  p[1] = make_float4(v[4], v[5], v[6], v[7]);
}
__device__ __forceinline__ void store8(const StSplit& Y, size_t r, int c, const float* v) {
  uint32_t hw[4], lw[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const __nv_bfloat162 hi = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
    const __nv_bfloat162 lo = __floats2bfloat162_rn(v[2 * k] - __low2float(hi), v[2 * k + 1] - __high2float(hi));
    hw[k] = *reinterpret_cast<const uint32_t*>(&hi);
    lw[k] = *reinterpret_cast<const uint32_t*>(&lo);
  }
  __nv_bfloat16* p = Y.p + r * Y.ld + c;
  *reinterpret_cast<uint4*>(p) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
  *reinterpret_cast<uint4*>(p + Y.plane) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
}
static bool vec8_ok(const StF32& X) { return ((uintptr_t)X.p & 15) == 0 && X.ld % 4 == 0; }
static bool vec8_ok(const StSplit& X) {
  return ((uintptr_t)X.p & 15) == 0 && X.ld % 8 == 0 && X.plane % 8 == 0;
}

// Spin means of 8 features per thread (16-byte loads), one electron row at a
// time: the small register footprint keeps five blocks per SM, which measured
// faster than batching rows per thread.
// (32-bit index arithmetic: the launcher keeps B * Tp * g1p / 8 below 2^31)
template <class In, class Out>
__global__ void k_mean_h1_vec(int B, int n, int n_up, int C, int Tp, int d, In X, int g1p, Out G1) {
  const unsigned nv = (unsigned)g1p / 8u;
  const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (unsigned)B * (unsigned)Tp * nv) return;
  const unsigned wt32 = e / nv;
  const int col = 8 * (int)(e - wt32 * nv);
  const size_t wt = wt32;
  const int w = (int)(wt32 / (unsigned)Tp);
  const int t = (int)(wt32 - (unsigned)w * (unsigned)Tp);
  float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (col < C * d) {
    const int s = col / d, f = col % d;
    int a0, a1;
    channel_range(s, C, n, n_up, &a0, &a1);
    for (int i = a0; i < a1; ++i) {
      float v[8];
      load8(X, ((size_t)w * n + i) * Tp + t, f, v);
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[j] += v[j];
    }
    const float inv = 1.0f / (float)(a1 - a0);
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] *= inv;
  }
  store8(G1, wt, col, acc);
}

template <class In, class Out>
cudaError_t launch_mean_h1(cudaStream_t s, int B, int n, int n_up, int C, int Tp, int d, In X, int g1p,
                           Out G1) {
  if (d % 8 == 0 && g1p % 8 == 0 && vec8_ok(X) && vec8_ok(G1) && (size_t)B * Tp * (g1p / 8) < (1ull << 31)) {
    const size_t total = (size_t)B * Tp * (g1p / 8);
    k_mean_h1_vec<In, Out><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(B, n, n_up, C, Tp, d, X, g1p, G1);
    return cudaGetLastError();
  }
  size_t total = (size_t)B * Tp * g1p;
  k_mean_h1<In, Out><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(B, n, n_up, C, Tp, d, X, g1p, G1);
  return cudaGetLastError();
}
template cudaError_t launch_mean_h1<StF32, StF32>(cudaStream_t, int, int, int, int, int, int, StF32, int,
                                                  StF32);
template cudaError_t launch_mean_h1<StSplit, StSplit>(cudaStream_t, int, int, int, int, int, int, StSplit,
                                                      int, StSplit);

// Value-only passes of the mixed form: everything the first layer reads, from
// the electron positions, in one block per walker.  The electron-atom and
// electron-electron vectors (input/atomic.py:46-79) go to shared memory once;
// from there the block writes the one-electron rows X0 as split bf16, the
// pair rows H2 (fp32, read by the two-electron stream), the spin means of the
// pair rows over their first electron (split bf16, the first layer's second
// GEMM source) and the first layer's broadcast term Gb[w] = g1[w] W_g1, where
// g1 holds the spin means of X0 (backbone/ferminet.py:65-90).  The means sum
// electrons in index order, as k_mean_h1_vec and k_features do.
__device__ __forceinline__ float f4_comp(const float4& v, int c) {
  return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w));
}

__global__ void k_inputs_value(int n, int A, int n_up, int C, int K0p, int g1p, int g2p, int dout,
                               const float* __restrict__ elec, const float* __restrict__ atoms,
                               const float* __restrict__ charges, double nuc, const float* __restrict__ Wg1,
                               float* __restrict__ rae_g, float* __restrict__ aevec_g, float* __restrict__ H2,
                               StSplit X0s, StSplit G2s, float* __restrict__ Gb, float* __restrict__ pe) {
  extern __shared__ float4 shin[];
  float4* ea = shin;                                  // [n][A]: |r_i - R_I|, r_i - R_I
  float4* pr = ea + n * A;                            // [n][n]: |r_i - r_j|, r_i - r_j (zero for i == j)
  float* g1 = reinterpret_cast<float*>(pr + n * n);   // [g1p]
  float* xs = g1 + g1p;                               // [n][3]
  __shared__ double red[32];
  const int w = blockIdx.x;
  const float* ew = elec + (size_t)w * n * 3;
  for (int e = threadIdx.x; e < 3 * n; e += blockDim.x) xs[e] = ew[e];
  __syncthreads();
  double vpot = 0.0;
  for (int e = threadIdx.x; e < n * A; e += blockDim.x) {
    const int i = e / A, I = e - i * A;
    const float dx = xs[3 * i] - atoms[3 * I], dy = xs[3 * i + 1] - atoms[3 * I + 1],
                dz = xs[3 * i + 2] - atoms[3 * I + 2];
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    ea[e] = make_float4(r, dx, dy, dz);
    const size_t gi = (size_t)w * n * A + e;
    rae_g[gi] = r;
    aevec_g[3 * gi] = dx;
    aevec_g[3 * gi + 1] = dy;
    aevec_g[3 * gi + 2] = dz;
    if (pe) vpot -= (double)charges[I] / (double)r;
  }
  float4* h2w = reinterpret_cast<float4*>(H2) + (size_t)w * n * n;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i != j) {
      const float d0 = xs[3 * i] - xs[3 * j], d1 = xs[3 * i + 1] - xs[3 * j + 1], d2 = xs[3 * i + 2] - xs[3 * j + 2];
      const float r = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
      v = make_float4(r, d0, d1, d2);
      if (pe && i < j) vpot += 1.0 / (double)r;
    }
    pr[e] = v;
    h2w[e] = v;
  }
  __syncthreads();
  const size_t row0 = (size_t)w * n;
  const int A4 = 4 * A;
  const int k2 = K0p / 2;  // two features per thread, paired stores
  for (int e = threadIdx.x; e < n * k2; e += blockDim.x) {
    const int i = e / k2, f0 = 2 * (e - i * k2);
    put2(X0s, row0 + i, f0, f0 < A4 ? f4_comp(ea[i * A + (f0 >> 2)], f0 & 3) : 0.f,
         f0 + 1 < A4 ? f4_comp(ea[i * A + ((f0 + 1) >> 2)], (f0 + 1) & 3) : 0.f);
  }
  for (int col = threadIdx.x; col < g1p; col += blockDim.x) {
    float acc = 0.f;
    if (col < C * A4) {
      const int sc = col / A4, f = col - sc * A4;
      int a0, a1;
      channel_range(sc, C, n, n_up, &a0, &a1);
      for (int a = a0; a < a1; ++a) acc += f4_comp(ea[a * A + (f >> 2)], f & 3);
      acc *= 1.0f / (float)(a1 - a0);
    }
    g1[col] = acc;
  }
  const int c2 = g2p / 2;  // two columns per thread, paired stores
  for (int e = threadIdx.x; e < n * c2; e += blockDim.x) {
    const int i = e / c2, col0 = 2 * (e - i * c2);
    float vv[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int col = col0 + q;
      float v = 0.f;
      if (col < 4 * C) {
        const int sc = col >> 2, c4 = col & 3;
        int a0, a1;
        channel_range(sc, C, n, n_up, &a0, &a1);
        float acc = 0.f;
        for (int a = a0; a < a1; ++a)
          if (a != i) acc += f4_comp(pr[a * n + i], c4);  // pair (a, i): r_a - r_i
        v = acc / (float)(a1 - a0);
      }
      vv[q] = v;
    }
    put2(G2s, row0 + i, col0, vv[0], vv[1]);
  }
  __syncthreads();
  for (int f = threadIdx.x; f < dout; f += blockDim.x) {
    float acc = 0.f;
    for (int k = 0; k < g1p; ++k) acc = fmaf(g1[k], __ldg(Wg1 + (size_t)k * dout + f), acc);
    Gb[(size_t)w * dout + f] = acc;
  }
  if (pe) {
    for (int o = 16; o > 0; o >>= 1) vpot += __shfl_xor_sync(0xffffffffu, vpot, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vpot;
    __syncthreads();
    if (threadIdx.x < 32) {
      double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0) pe[w] = (float)(v + nuc);
    }
  }
}

// Forward-Laplacian passes of the mixed form: the same per-walker fusion with
// T tangent rows (value, Laplacian, 3n Jacobian rows; Tp padded) -- the rows
// k_features writes (X0 as split bf16, H2 with P2 = 5 tangent planes), the
// first layer's broadcast term Gb[w, t] = g1[w, t] W_g1 with g1 the spin means
// of X0 (k_mean_h1_vec's order: electrons in index order, then times 1/n_s),
// and the spin means of the pair rows with their tangent rules (k_mean_h2):
// rows t = 0, 1 average pair values and Laplacians (the latter doubled), a
// Jacobian row of electron el either subtracts the gradients of every pair
// (el, i) with i the row's electron, or takes the one pair (el, i) of el's
// channel.  W_g1's column of a thread stays in registers (g1p <= kFlG1Max).
constexpr int kFlG1Max = 32;

__global__ void __launch_bounds__(256, 1) k_inputs_fl(int n, int A, int n_up, int C, int Tp, int T, int K0p, int g1p,
                                                   int g2p, int dout, const float* __restrict__ elec,
                                                   const float* __restrict__ atoms, const float* __restrict__ charges,
                                                   double nuc, const float* __restrict__ Wg1,
                                                   float* __restrict__ rae_g, float* __restrict__ aevec_g,
                                                   float* __restrict__ H2, StSplit X0s, StSplit G2s,
                                                   float* __restrict__ Gb, float* __restrict__ pe) {
  // shared tables of the walker (every quotient formed once):
  //   ea [n][A]      (|r_i - R_I|, r_i - R_I)
  //   ed [n][A]      (2 / |r_i - R_I|, (r_i - R_I) / |r_i - R_I|)
  //   pl [n][n][5]   the five planes of pair (a, b) (r_a - r_b), rows of H2
  //   ps [C][n][5]   per channel s and electron b: sum over a in s of pl[a][b]
  //   g1 [Tp][g1p]   spin means of the one-electron rows
  extern __shared__ float4 shfl4[];
  float4* ea = shfl4;
  float4* ed = ea + n * A;
  float4* pl = ed + n * A;
  float4* ps = pl + (size_t)n * n * 5;
  float* g1 = reinterpret_cast<float*>(ps + (size_t)C * n * 5);
  float* xs = g1 + Tp * g1p;
  __shared__ double red[8];
  const int w = blockIdx.x;
  const float* ew = elec + (size_t)w * n * 3;
  for (int e = threadIdx.x; e < 3 * n; e += blockDim.x) xs[e] = ew[e];
  __syncthreads();
  double vpot = 0.0;
  for (int e = threadIdx.x; e < n * A; e += blockDim.x) {
    const int i = e / A, I = e - i * A;
    const float dx = xs[3 * i] - atoms[3 * I], dy = xs[3 * i + 1] - atoms[3 * I + 1],
                dz = xs[3 * i + 2] - atoms[3 * I + 2];
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    ea[e] = make_float4(r, dx, dy, dz);
    ed[e] = make_float4(2.0f / r, dx / r, dy / r, dz / r);
    const size_t gi = (size_t)w * n * A + e;
    rae_g[gi] = r;
    aevec_g[3 * gi] = dx;
    aevec_g[3 * gi + 1] = dy;
    aevec_g[3 * gi + 2] = dz;
    if (pe) vpot -= (double)charges[I] / (double)r;
  }
  float4* h2w = reinterpret_cast<float4*>(H2) + (size_t)w * n * n * 5;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    float4 v[5];
#pragma unroll
    for (int p = 0; p < 5; ++p) v[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i != j) {
      const float d0 = xs[3 * i] - xs[3 * j], d1 = xs[3 * i + 1] - xs[3 * j + 1], d2 = xs[3 * i + 2] - xs[3 * j + 2];
      const float r = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
      v[0] = make_float4(r, d0, d1, d2);
      v[1] = make_float4(2.0f / r, 0.f, 0.f, 0.f);
      v[2] = make_float4(d0 / r, 1.f, 0.f, 0.f);
      v[3] = make_float4(d1 / r, 0.f, 1.f, 0.f);
      v[4] = make_float4(d2 / r, 0.f, 0.f, 1.f);
      if (pe && i < j) vpot += 1.0 / (double)r;
    }
#pragma unroll
    for (int p = 0; p < 5; ++p) {
      pl[(size_t)e * 5 + p] = v[p];
      h2w[(size_t)e * 5 + p] = v[p];
    }
  }
  __syncthreads();
  // channel sums of the pair planes over the first electron, in electron order
  for (int e = threadIdx.x; e < C * n * 5; e += blockDim.x) {
    const int sc = e / (n * 5), rem = e - sc * n * 5;
    const int b = rem / 5, p = rem - b * 5;
    int a0, a1;
    channel_range(sc, C, n, n_up, &a0, &a1);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int a = a0; a < a1; ++a) {
      const float4 v = pl[((size_t)a * n + b) * 5 + p];
      acc.x += v.x;
      acc.y += v.y;
      acc.z += v.z;
      acc.w += v.w;
    }
    ps[e] = acc;
  }
  const int A4 = 4 * A;
  // one-electron feature f of electron i, tangent row t (k_features' rows)
  auto x0v = [&](int i, int t, int f) -> float {
    if (f >= A4 || t >= T) return 0.f;
    const int I = f >> 2, comp = f & 3;
    if (t == 0) return f4_comp(ea[i * A + I], comp);
    if (t == 1) return comp == 0 ? ed[i * A + I].x : 0.f;
    const int dd = t - 2, el = dd / 3, c = dd - 3 * el;
    if (el != i) return 0.f;
    return comp == 0 ? f4_comp(ed[i * A + I], 1 + c) : (comp - 1 == c ? 1.f : 0.f);
  };
  const size_t rowb = (size_t)w * n * Tp;
  // 1 / n_s of the two channels (the same quotient every mean kernel forms)
  const float invc[2] = {1.0f / (float)(C == 1 ? n : n_up), C == 1 ? 0.f : 1.0f / (float)(n - n_up)};
  const int k8 = K0p / 8;  // one-electron rows: 8 features per thread, 16-byte stores
  for (int e = threadIdx.x; e < n * Tp * k8; e += blockDim.x) {
    const int it = e / k8, f0 = 8 * (e - it * k8);
    const int i = it / Tp, t = it - i * Tp;
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = x0v(i, t, f0 + q);
    store8(X0s, rowb + it, f0, v);
  }
  // spin means of the one-electron rows: rows t <= 1 sum the channel's
  // electrons; a Jacobian row of electron el has el's row alone (the other
  // electrons' rows are zero)
  for (int e = threadIdx.x; e < Tp * g1p; e += blockDim.x) {
    const int t = e / g1p, col = e - t * g1p;
    float acc = 0.f;
    if (col < C * A4 && t < T) {
      const int sc = col / A4, f = col - sc * A4;
      int a0, a1;
      channel_range(sc, C, n, n_up, &a0, &a1);
      if (t <= 1) {
        for (int a = a0; a < a1; ++a) acc += x0v(a, t, f);
      } else {
        const int el = (t - 2) / 3;
        if (el >= a0 && el < a1) acc = x0v(el, t, f);
      }
      acc *= invc[sc];
    }
    g1[e] = acc;
  }
  // pair rows' spin means over the first electron a of pair (a, i), per
  // tangent row (k_mean_h2's rules), 8 columns per thread
  const int c8 = g2p / 8;
  for (int e = threadIdx.x; e < n * Tp * c8; e += blockDim.x) {
    const int it = e / c8, col0 = 8 * (e - it * c8);
    const int i = it / Tp, t = it - i * Tp;
    const int dd = t - 2, el = t >= 2 ? dd / 3 : -1, c = t >= 2 ? dd - 3 * el : 0;
    float vv[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int col = col0 + q;
      float v = 0.f;
      if (col < 4 * C && t < T) {
        const int sc = col >> 2, f = col & 3;
        int a0, a1;
        channel_range(sc, C, n, n_up, &a0, &a1);
        const float inv = invc[sc];
        if (t == 0) {
          v = f4_comp(ps[((size_t)sc * n + i) * 5], f) * inv;
        } else if (t == 1) {
          v = 2.0f * f4_comp(ps[((size_t)sc * n + i) * 5 + 1], f) * inv;
        } else if (el == i) {
          v = -f4_comp(ps[((size_t)sc * n + i) * 5 + 2 + c], f) * inv;
        } else if (el >= a0 && el < a1) {
          v = f4_comp(pl[((size_t)el * n + i) * 5 + 2 + c], f) * inv;
        }
      }
      vv[q] = v;
    }
    store8(G2s, rowb + it, col0, vv);
  }
  __syncthreads();
  // broadcast term of the first layer: one output column per thread, its
  // weights in registers, the spin-mean rows read four at a time
  for (int f = threadIdx.x; f < dout; f += blockDim.x) {
    float wc[kFlG1Max];
#pragma unroll
    for (int k = 0; k < kFlG1Max; ++k) wc[k] = k < g1p ? __ldg(Wg1 + (size_t)k * dout + f) : 0.f;
    float* gbw = Gb + (size_t)w * Tp * dout + f;
    for (int t = 0; t < Tp; ++t) {
      const float4* gr = reinterpret_cast<const float4*>(g1 + t * g1p);
      float acc = 0.f;
#pragma unroll
      for (int k4 = 0; k4 < kFlG1Max / 4; ++k4) {
        if (4 * k4 < g1p) {
          const float4 gv = gr[k4];
          acc = fmaf(gv.x, wc[4 * k4], acc);
          acc = fmaf(gv.y, wc[4 * k4 + 1], acc);
          acc = fmaf(gv.z, wc[4 * k4 + 2], acc);
          acc = fmaf(gv.w, wc[4 * k4 + 3], acc);
        }
      }
      gbw[(size_t)t * dout] = acc;
    }
  }
  if (pe) {
    for (int o = 16; o > 0; o >>= 1) vpot += __shfl_xor_sync(0xffffffffu, vpot, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vpot;
    __syncthreads();
    if (threadIdx.x < 32) {
      double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (threadIdx.x == 0) pe[w] = (float)(v + nuc);
    }
  }
}

size_t inputs_fl_smem(int n, int A, int Tp, int g1p, int C) {
  return sizeof(float4) * (2 * (size_t)n * A + (size_t)n * n * 5 + (size_t)C * n * 5) +
         sizeof(float) * ((size_t)Tp * g1p + 3 * n);
}

bool inputs_fl_supported(int n, int A, int Tp, int g1p) {
  return g1p <= kFlG1Max && g1p % 4 == 0 && inputs_fl_smem(n, A, Tp, g1p, 2) <= 48 * 1024;
}
// (K0p and g2p are multiples of 8 and the split planes 16-byte aligned: the
// rows go out as 16-byte stores)

cudaError_t launch_inputs_fl(cudaStream_t s, int B, int n, int A, int n_up, int C, int Tp, int T, int K0p, int g1p,
                             int g2p, int dout, const float* electrons, const float* atoms, const float* charges,
                             double nuc, const float* Wg1, float* rae, float* aevec, float* H2, StSplit X0s,
                             StSplit G2s, float* Gb, float* pe) {
  if (!inputs_fl_supported(n, A, Tp, g1p)) return cudaErrorNotSupported;
  k_inputs_fl<<<B, 256, inputs_fl_smem(n, A, Tp, g1p, C), s>>>(n, A, n_up, C, Tp, T, K0p, g1p, g2p, dout, electrons,
                                                            atoms, charges, nuc, Wg1, rae, aevec, H2, X0s, G2s, Gb,
                                                            pe);
  return cudaGetLastError();
}

size_t inputs_value_smem(int n, int A, int g1p) {
  return sizeof(float4) * ((size_t)n * A + (size_t)n * n) + sizeof(float) * ((size_t)g1p + 3 * n);
}

cudaError_t launch_inputs_value(cudaStream_t s, int B, int n, int A, int n_up, int C, int K0p, int g1p, int g2p,
                                int dout, const float* electrons, const float* atoms, const float* charges,
                                double nuc, const float* Wg1, float* rae, float* aevec, float* H2, StSplit X0s,
                                StSplit G2s, float* Gb, float* pe) {
  const size_t sm = inputs_value_smem(n, A, g1p);
  if (sm > 48 * 1024) return cudaErrorNotSupported;
  k_inputs_value<<<B, 128, sm, s>>>(n, A, n_up, C, K0p, g1p, g2p, dout, electrons, atoms, charges, nuc, Wg1, rae,
                                    aevec, H2, X0s, G2s, Gb, pe);
  return cudaGetLastError();
}

// d/dr_e of h2[a, i] = (delta_{ae} - delta_{ie}) d/dDelta (pair (a,i), a != i);
// the full Laplacian of a pair feature is twice its Laplacian in Delta.
template <class Out>
__global__ void k_mean_h2(int B, int n, int n_up, int C, int Tp, int T, int d2, int P2,
                          const float* __restrict__ H2, int g2p, Out G2) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t total = (size_t)B * n * Tp * g2p;
  if (e >= total) return;
  int col = (int)(e % g2p);
  size_t r = e / g2p;
  int t = (int)(r % Tp);
  size_t wi = r / Tp;
  int i = (int)(wi % n);
  int w = (int)(wi / n);
  float v = 0.f;
  if (col < C * d2 && t < T) {
    int s = col / d2, f = col % d2, a0, a1;
    channel_range(s, C, n, n_up, &a0, &a1);
    const float inv = 1.0f / (float)(a1 - a0);
    auto at = [&](int a, int p) { return H2[((((size_t)w * n + a) * n + i) * P2 + p) * d2 + f]; };
    if (t == 0) {
      float acc = 0.f;
      for (int a = a0; a < a1; ++a) acc += at(a, 0);
      v = acc * inv;
    } else if (t == 1) {
      float acc = 0.f;
      for (int a = a0; a < a1; ++a) acc += at(a, 1);
      v = 2.0f * acc * inv;
    } else {
      int dd = t - 2, el = dd / 3, c = dd % 3;
      float acc = 0.f;
      if (el == i) {
        for (int a = a0; a < a1; ++a) acc -= at(a, 2 + c);
      } else if (el >= a0 && el < a1) {
        acc = at(el, 2 + c);
      }
      v = acc * inv;
    }
  }
  G2.put(r, col, v);
}

// k_mean_h2 with 8 features per thread (16-byte loads and stores).
template <class Out>
__global__ void k_mean_h2_vec(int B, int n, int n_up, int C, int Tp, int T, int d2, int P2,
                              const float* __restrict__ H2, int g2p, Out G2) {
  // 32-bit index arithmetic: the launcher keeps B * n * Tp * g2p / 8 below 2^31
  const unsigned nv = (unsigned)g2p / 8u;
  const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (unsigned)B * (unsigned)n * (unsigned)Tp * nv) return;
  const unsigned r32 = e / nv;
  const int col = 8 * (int)(e - r32 * nv);
  const size_t r = r32;
  const unsigned wi = r32 / (unsigned)Tp;
  const int t = (int)(r32 - wi * (unsigned)Tp);
  const int w = (int)(wi / (unsigned)n);
  const int i = (int)(wi - (unsigned)w * (unsigned)n);
  float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (col < C * d2 && t < T) {
    const int sc = col / d2, f = col % d2;
    int a0, a1;
    channel_range(sc, C, n, n_up, &a0, &a1);
    const float inv = 1.0f / (float)(a1 - a0);
    // row of pair (a, i), tangent slot p
    auto row = [&](int a, int p) { return ((((size_t)w * n + a) * n + i) * P2 + p) * d2 + f; };
    auto add8 = [&](size_t o, float sgn) {
      const float4 x = __ldg(reinterpret_cast<const float4*>(H2 + o));
      const float4 y = __ldg(reinterpret_cast<const float4*>(H2 + o + 4));
      acc[0] += sgn * x.x; acc[1] += sgn * x.y; acc[2] += sgn * x.z; acc[3] += sgn * x.w;
      acc[4] += sgn * y.x; acc[5] += sgn * y.y; acc[6] += sgn * y.z; acc[7] += sgn * y.w;
    };
    float scale = inv;
    if (t <= 1) {
      for (int a = a0; a < a1; ++a) add8(row(a, t), 1.f);
      if (t == 1) scale = 2.0f * inv;
    } else {
      const int dd = t - 2, el = dd / 3, c = dd % 3;
      if (el == i) {
        for (int a = a0; a < a1; ++a) add8(row(a, 2 + c), -1.f);
      } else if (el >= a0 && el < a1) {
        add8(row(el, 2 + c), 1.f);
      }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] *= scale;
  }
  store8(G2, r, col, acc);
}

template <class Out>
cudaError_t launch_mean_h2(cudaStream_t s, int B, int n, int n_up, int C, int Tp, int T, int d2,
                           int P2, const float* H2, int g2p, Out G2) {
  if (d2 % 8 == 0 && g2p % 8 == 0 && ((uintptr_t)H2 & 15) == 0 && vec8_ok(G2) &&
      (size_t)B * n * Tp * (g2p / 8) < (1ull << 31)) {
    const size_t total = (size_t)B * n * Tp * (g2p / 8);
    k_mean_h2_vec<Out><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(B, n, n_up, C, Tp, T, d2, P2, H2, g2p, G2);
    return cudaGetLastError();
  }
  size_t total = (size_t)B * n * Tp * g2p;
  k_mean_h2<Out><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(B, n, n_up, C, Tp, T, d2, P2, H2,
                                                                  g2p, G2);
  return cudaGetLastError();
}
template cudaError_t launch_mean_h2<StF32>(cudaStream_t, int, int, int, int, int, int, int, int,
                                           const float*, int, StF32);
template cudaError_t launch_mean_h2<StSplit>(cudaStream_t, int, int, int, int, int, int, int, int,
                                             const float*, int, StSplit);

// =====================================================================
// determinant stage (src/jaqmc/wavefunction/output/logdet.py:53-80,
//                    src/jaqmc/laplacian/primitives/slogdet.py:25-72,
//                    src/jaqmc/estimator/kinetic/_common.py:61-73)
// One CTA per walker; each warp factorises determinants k = warp, warp+nw, ...
// =====================================================================
// FP64 re-factorisation threshold on the pivot growth factor max|U| / max|A|.
constexpr float kRefactorGrowth = 1e6f;
// Tangent passes with n > 16 also re-factorise in FP64 when the smallest
// pivot is below kRefactorPivot x max|A| (condition number >~ 1e4): the traces
// tr(P_d^2) of such a determinant lose to FP32 inversion error what the
// kinetic energy needs (measured on 42-electron walkers: FP32 errors of up to
// 20 Ha fall to 0.03 Ha).
constexpr float kRefactorPivot = 1e-4f;

// Cancellation trigger of the tangent passes.  Determinant k enters the
// kinetic energy as w_k (tL_k - t2_k + q_k) (w_k = s_k e^{l_k} / psi), and
// the FP32 rounding errors of its traces are about eps32 times their
// magnitudes, so its error in Ha is about eps32 times
//   |w_k| (|tL| + |t2| + |q|)^2 / |tL - t2 + q|
// (the weight, the magnitude and the cancellation between the traces).  A
// determinant whose score exceeds kCancelScore is evaluated again in FP64.
// On burnt-in N2 walkers (FermiNet 4 x (256, 32), K = 16) this re-evaluates
// about one determinant in eight and takes the share of walkers whose FP32
// E_L is within 1e-4 Ha of an FP64 evaluation from ~0.84 to ~0.98.
constexpr float kCancelScore = 1e3f;
__device__ __forceinline__ bool cancel_marks(float wk, float tL, float t2, float q) {
  const float mag = fabsf(tL) + fabsf(t2) + fabsf(q);
  const float net = fabsf(tL - t2 + q);
  return fabsf(wk) * mag * mag > kCancelScore * net;  // also true for net == 0 with mag > 0
}

// w_k = s_k exp(l_k - lmax) / sum_k s_k exp(l_k - lmax) for the K
// determinants (warp-cooperative; singular determinants have s_k = 0).
__device__ void det_weights(int K, const double* lds, const float* sgs, float* wts) {
  const int lane = threadIdx.x & 31;
  double lmax = -INFINITY;
  for (int k = lane; k < K; k += 32)
    if (sgs[k] != 0.f) lmax = fmax(lmax, lds[k]);
  for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  double S = 0.0;
  for (int k = lane; k < K; k += 32)
    if (sgs[k] != 0.f) S += (double)sgs[k] * exp(lds[k] - lmax);
  for (int o = 16; o > 0; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
  for (int k = lane; k < K; k += 32)
    wts[k] = (sgs[k] != 0.f && S != 0.0) ? (float)((double)sgs[k] * exp(lds[k] - lmax) / S) : 0.f;
  __syncwarp();
}

__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

struct DetOut {
  double ld;
  float sgn;
  float tL, t2, q;
  double kin;  // tL - t2 + q, formed in the precision the traces were computed in
  int refactor, singular;
};

// LU with partial pivoting of the n x n matrix in S (row stride ld) by one
// warp; perm[i] = source row of pivoted row i.  log|det| is accumulated as a
// normalised mantissa/exponent product (one FP64 log per determinant).
// Returns the pivot growth factor max|U| / max|A| in *growth.
template <typename S>
__device__ void warp_lu(S* LU, int n, int ld, int* perm, double* logabs, float* sgn, double* growth,
                        int* singular, double* pivmin = nullptr) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < n; i += 32) perm[i] = i;
  S amax = (S)0;
  for (int e = lane; e < n * n; e += 32) amax = fmax(amax, (S)fabs(LU[(e / n) * ld + (e % n)]));
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  __syncwarp();
  S mant = (S)1;
  int ex = 0;
  float sg = 1.f;
  int sing = 0;
  S pmn = (S)INFINITY;
  for (int k = 0; k < n; ++k) {
    S best = (S)-1;
    int bi = k;
    for (int i = k + lane; i < n; i += 32) {
      S v = fabs(LU[i * ld + k]);
      if (v > best) { best = v; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      S ob = __shfl_xor_sync(0xffffffffu, best, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (bi != k) {
      for (int j = lane; j < n; j += 32) {
        S tmp = LU[k * ld + j];
        LU[k * ld + j] = LU[bi * ld + j];
        LU[bi * ld + j] = tmp;
      }
      if (lane == 0) {
        int tp = perm[k];
        perm[k] = perm[bi];
        perm[bi] = tp;
      }
      sg = -sg;
    }
    __syncwarp();
    S piv = LU[k * ld + k];
    if (!(fabs(piv) > (S)0)) { sing = 1; break; }
    pmn = fmin(pmn, (S)fabs(piv));
    if (piv < (S)0) sg = -sg;
    int e2;
    mant = frexp(mant * (S)fabs(piv), &e2);
    ex += e2;
    for (int i = k + 1 + lane; i < n; i += 32) LU[i * ld + k] /= piv;
    __syncwarp();
    for (int j = k + 1 + lane; j < n; j += 32) {
      S ukj = LU[k * ld + j];
      for (int i = k + 1; i < n; ++i) LU[i * ld + j] -= LU[i * ld + k] * ukj;
    }
    __syncwarp();
  }
  S umax = (S)0;
  if (!sing)
    for (int j = lane; j < n; j += 32)
      for (int i = 0; i <= j; ++i) umax = fmax(umax, (S)fabs(LU[i * ld + j]));
  for (int o = 16; o > 0; o >>= 1) umax = fmax(umax, __shfl_xor_sync(0xffffffffu, umax, o));
  // one FP64 log per determinant (FP64 is scarce on this part): lane 0 only
  *logabs = sing ? -INFINITY : (lane == 0 ? log((double)mant) + (double)ex * 0.69314718055994530942 : 0.0);
  *sgn = sg;
  *growth = sing ? INFINITY : (double)umax / (double)amax;
  *singular = sing;
  if (pivmin) *pivmin = sing ? 0.0 : (double)pmn / (double)amax;
}

// Per-warp scratch for one determinant: LU and A^-1 (row stride ld), the
// products M_t = A^-1 A_t (row stride ldm, odd, so that transposed reads are
// bank-conflict free) and the staged A_t for the FP64 path.
struct DetScratch {
  int ld, ldm;
  size_t bytes;  // per warp, FP64 worst case
  __host__ __device__ DetScratch(int n) {
    ld = (n + 3) / 4 * 4;
    ldm = (n % 2 == 0) ? n + 1 : n + 2;
    bytes = align_up((size_t)(2 * n * ld + 2 * n * ldm) * 8 + (size_t)n * 4, 16);
  }
};

// A^-1 column by column (lane j solves L U x = P e_j in place in column j).
template <typename S>
__device__ void warp_inverse(const S* LU, S* Ainv, const int* perm, int n, int ld) {
  const int lane = threadIdx.x & 31;
  for (int j = lane; j < ld; j += 32) {
    if (j >= n) {  // zero padding columns
      for (int i = 0; i < n; ++i) Ainv[i * ld + j] = (S)0;
      continue;
    }
    for (int i = 0; i < n; ++i) {
      S v = perm[i] == j ? (S)1 : (S)0;
      for (int m = 0; m < i; ++m) v -= LU[i * ld + m] * Ainv[m * ld + j];
      Ainv[i * ld + j] = v;
    }
    for (int i = n - 1; i >= 0; --i) {
      S v = Ainv[i * ld + j];
      for (int m = i + 1; m < n; ++m) v -= LU[i * ld + m] * Ainv[m * ld + j];
      Ainv[i * ld + j] = v / LU[i * ld + i];
    }
  }
  __syncwarp();
}

// M = A^-1 A_t into Ms; returns tr(M) (warp-reduced).  FP32: columns of A_t
// held in registers, rows of A^-1 read as float4 broadcasts.
template <int NMAX>
__device__ float warp_product_f32(const float* Ainv, const float* __restrict__ At, float* Ms, int n,
                                  int ld, int ldm, int rs) {
  const int lane = threadIdx.x & 31;
  float tr = 0.f;
  for (int j = lane; j < n; j += 32) {
    float x[NMAX];
#pragma unroll
    for (int m = 0; m < NMAX; ++m) x[m] = m < n ? At[m * rs + j] : 0.f;
#pragma unroll 4
    for (int i = 0; i < n; ++i) {
      const float4* a4 = reinterpret_cast<const float4*>(Ainv + i * ld);
      float acc = 0.f;
#pragma unroll
      for (int m4 = 0; m4 < NMAX / 4; ++m4) {
        if (4 * m4 < n) {
          float4 a = a4[m4];
          acc = fmaf(a.x, x[4 * m4], acc);
          acc = fmaf(a.y, x[4 * m4 + 1], acc);
          acc = fmaf(a.z, x[4 * m4 + 2], acc);
          acc = fmaf(a.w, x[4 * m4 + 3], acc);
        }
      }
      Ms[i * ldm + j] = acc;
      if (i == j) tr += acc;
    }
  }
  tr = warp_sum(tr);
  __syncwarp();
  return tr;
}

// FP64 variant (re-factorised determinants only): A_t staged in shared memory.
__device__ double warp_product_f64(const double* Ainv, const float* __restrict__ At, double* Ms,
                                   double* Xs, int n, int ld, int ldm, int rs) {
  const int lane = threadIdx.x & 31;
  for (int e = lane; e < n * n; e += 32) Xs[(e / n) * ldm + (e % n)] = (double)At[(e / n) * rs + (e % n)];
  __syncwarp();
  double tr = 0.0;
  for (int j = lane; j < n; j += 32) {
    for (int i = 0; i < n; ++i) {
      double acc = 0.0;
      for (int m = 0; m < n; ++m) acc += Ainv[i * ld + m] * Xs[m * ldm + j];
      Ms[i * ldm + j] = acc;
      if (i == j) tr += acc;
    }
  }
  tr = warp_sum(tr);
  __syncwarp();
  return tr;
}

template <typename S>
__device__ S warp_trace_sq(const S* Ms, int n, int ldm) {
  const int lane = threadIdx.x & 31;
  S t2 = (S)0;
  for (int j = lane; j < n; j += 32)
    for (int i = 0; i < n; ++i) t2 += Ms[i * ldm + j] * Ms[j * ldm + i];
  t2 = warp_sum(t2);
  __syncwarp();
  return t2;
}

// Tangent traces of one determinant for n <= 16 (FP32):
//   tL = tr(A^-1 L_A) as one dot product, and for every Jacobian direction d
//   P_d = A^-1 J_d A, t1_d = tr(P_d), t2 += tr(P_d^2), q += t1_d^2.
// Each half-warp owns one direction per pass with lane j computing column j
// of P_d, and every lane carries two directions, so a warp pass covers four
// directions and each broadcast row of A^-1 feeds 2 x NMAX FMAs.  P_d goes
// to shared memory (row stride ldm, odd) for tr(P_d^2) = sum_i P_ij P_ji.
// (Packing the two directions into f32x2 FMAs needs a duplicated A^-1 and
// more shared-memory loads per row, which measured slower.)
template <int NMAX>
__device__ void det_tangents_f32(const float* Ainv, const float* __restrict__ Ak, int n, int T, size_t ts,
                                 int rs, int ld, int ldm, float* Ms, float* t1s, DetOut& o) {
  static_assert(NMAX <= 16 && NMAX % 4 == 0, "half-warp columns");
  const int lane = threadIdx.x & 31;
  const int h = lane >> 4, j = lane & 15;
  const bool colv = j < n;
  // tL = sum_{i,m} A^-1_im L_mi
  {
    const float* L = Ak + ts;
    float acc = 0.f;
    for (int e = lane; e < n * n; e += 32) {
      const int m = e / n, i = e - m * n;
      acc = fmaf(Ainv[i * ld + m], L[m * rs + i], acc);
    }
    o.tL = warp_sum(acc);
  }
  const int D = T - 2;
  float t2acc = 0.f, qacc = 0.f;
  float* Ma = Ms + (size_t)h * n * ldm;        // direction 4g + h
  float* Mb = Ms + (size_t)(2 + h) * n * ldm;  // direction 4g + 2 + h
  float xa[NMAX], xb[NMAX];
  auto load_cols = [&](int g) {
    const int da = 4 * g + h, db = 4 * g + 2 + h;
    const float* Ja = Ak + (size_t)(2 + da) * ts;
    const float* Jb = Ak + (size_t)(2 + db) * ts;
    const bool va = colv && da < D, vb = colv && db < D;
#pragma unroll
    for (int m = 0; m < NMAX; ++m) {
      xa[m] = (va && m < n) ? __ldg(Ja + m * rs + j) : 0.f;
      xb[m] = (vb && m < n) ? __ldg(Jb + m * rs + j) : 0.f;
    }
  };
  const int G = (D + 3) / 4;
  if (G > 0) load_cols(0);
  for (int g = 0; g < G; ++g) {
    float tra = 0.f, trb = 0.f;
#pragma unroll
    for (int i = 0; i < NMAX; ++i) {
      if (i < n) {
        const float4* a4 = reinterpret_cast<const float4*>(Ainv + i * ld);
        float acc_a = 0.f, acc_b = 0.f;
#pragma unroll
        for (int m4 = 0; m4 < NMAX / 4; ++m4) {
          if (4 * m4 < n) {
            const float4 a = a4[m4];
            acc_a = fmaf(a.x, xa[4 * m4], acc_a);
            acc_a = fmaf(a.y, xa[4 * m4 + 1], acc_a);
            acc_a = fmaf(a.z, xa[4 * m4 + 2], acc_a);
            acc_a = fmaf(a.w, xa[4 * m4 + 3], acc_a);
            acc_b = fmaf(a.x, xb[4 * m4], acc_b);
            acc_b = fmaf(a.y, xb[4 * m4 + 1], acc_b);
            acc_b = fmaf(a.z, xb[4 * m4 + 2], acc_b);
            acc_b = fmaf(a.w, xb[4 * m4 + 3], acc_b);
          }
        }
        if (colv) {
          Ma[i * ldm + j] = acc_a;
          Mb[i * ldm + j] = acc_b;
        }
        if (i == j) {
          tra = acc_a;
          trb = acc_b;
        }
      }
    }
    // next pass's columns are in flight while this pass is reduced
    if (g + 1 < G) load_cols(g + 1);
    __syncwarp();
    float sq = 0.f;
    if (colv) {
      const float* ra = Ma + j * ldm;
      const float* rb = Mb + j * ldm;
#pragma unroll
      for (int i = 0; i < NMAX; ++i)
        if (i < n) sq = fmaf(Ma[i * ldm + j], ra[i], fmaf(Mb[i * ldm + j], rb[i], sq));
    }
    t2acc += sq;
    // per-half sums of the diagonals (lanes j >= n contribute zero)
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) {
      tra += __shfl_xor_sync(0xffffffffu, tra, off);
      trb += __shfl_xor_sync(0xffffffffu, trb, off);
    }
    const int da = 4 * g + h, db = 4 * g + 2 + h;
    if (j == 0) {
      if (da < D) {
        t1s[da] = tra;
        qacc = fmaf(tra, tra, qacc);
      }
      if (db < D) {
        t1s[db] = trb;
        qacc = fmaf(trb, trb, qacc);
      }
    }
    __syncwarp();
  }
  o.t2 = warp_sum(t2acc);
  o.q = warp_sum(qacc);
}

// Factorise determinant k of a walker and, for T > 1, the slogdet traces
//   tL = tr(A^-1 L_A),  t1_d = tr(A^-1 J_d A),  t2 = sum_d tr((A^-1 J_d A)^2),
//   q = sum_d t1_d^2.
// Ak: the matrix (row stride rs floats); tangent t at Ak + t * ts.
template <typename S, int NMAX>
__device__ DetOut det_stage(const float* __restrict__ Ak, int n, int T, int rs, size_t ts, char* scratch,
                            float* t1s, bool fp64_pass) {
  const int lane = threadIdx.x & 31;
  const DetScratch sc(n);
  const int ld = sc.ld, ldm = sc.ldm;
  S* LU = reinterpret_cast<S*>(scratch);
  S* Ainv = LU + n * ld;
  S* Ms = Ainv + n * ld;
  S* Xs = Ms + n * ldm;
  int* perm = reinterpret_cast<int*>(scratch + (size_t)(2 * n * ld + 2 * n * ldm) * 8);
  DetOut o{};
  for (int e = lane; e < n * n; e += 32) LU[(e / n) * ld + (e % n)] = (S)Ak[(e / n) * rs + (e % n)];
  __syncwarp();
  double growth;
  warp_lu<S>(LU, n, ld, perm, &o.ld, &o.sgn, &growth, &o.singular);
  o.refactor = (!fp64_pass && !o.singular && !(growth <= (double)kRefactorGrowth)) ? 1 : 0;
  if (T <= 1 || o.singular || o.refactor) return o;
  warp_inverse<S>(LU, Ainv, perm, n, ld);
  if constexpr (sizeof(S) == 4 && NMAX <= 16) {
    det_tangents_f32<NMAX>(reinterpret_cast<const float*>(Ainv), Ak, n, T, ts, rs, ld, ldm,
                           reinterpret_cast<float*>(Ms), t1s, o);
    o.kin = (double)o.tL - (double)o.t2 + (double)o.q;
    return o;
  }
  S tl = (S)0, t2acc = (S)0, qacc = (S)0;
  for (int t = 1; t < T; ++t) {
    const float* At = Ak + (size_t)t * ts;
    S tr;
    if constexpr (sizeof(S) == 4) tr = warp_product_f32<NMAX>(Ainv, At, Ms, n, ld, ldm, rs);
    else tr = warp_product_f64(Ainv, At, Ms, Xs, n, ld, ldm, rs);
    if (t == 1) {
      tl = tr;
    } else {
      S t2 = warp_trace_sq<S>(Ms, n, ldm);
      if (lane == 0) t1s[t - 2] = (float)tr;
      t2acc += t2;
      qacc += tr * tr;
    }
  }
  o.tL = (float)tl;
  o.t2 = (float)t2acc;
  o.q = (float)qacc;
  o.kin = (double)tl - (double)t2acc + (double)qacc;
  return o;
}

// The tangent traces of one determinant with the products in double-float
// arithmetic (the determinant guard's re-evaluation; FP64 runs at about 1/64
// of the FP32 rate on this part).  LU and inverse in FP64; A^-1 split into
// hi + lo floats; each entry of M_d = A^-1 J_d (J_d exact in FP32) summed as
// s + c with TwoProduct (p = a x, e = fma(a, x, -p)) and TwoSum error-free
// transformations (Ogita, Rump & Oishi, "Accurate sum and dot product", SIAM
// J. Sci. Comput. 26, 2005), so an entry errs by ~n eps32^2 relative to
// sum |A^-1| |J| instead of n eps32; the traces tr M, tr M^2, tr(A^-1 L) and
// their combination tL - t2 + q are then accumulated in FP64.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// One tangent direction of the double-float stage: M = A^-1 J (A^-1 as the
// FP32 pair Ah + Al, J in FP32) with error-free products and sums into the
// hi/lo tiles Mh / Ml; returns tr M and tr M^2 in FP64 (every lane).
template <int NMAX>
__device__ void df_direction(const float* Ah, const float* Al, const float* __restrict__ J, float* Mh, float* Ml,
                             int n, int ld, int ldm, int rs, double* tr_out, double* t2_out) {
  const int lane = threadIdx.x & 31;
  double tr = 0.0;
  for (int j = lane; j < n; j += 32) {
    float x[NMAX];
#pragma unroll
    for (int m = 0; m < NMAX; ++m) x[m] = m < n ? J[m * rs + j] : 0.f;
    for (int i = 0; i < n; ++i) {
      float sh = 0.f, sl = 0.f;
#pragma unroll
      for (int m = 0; m < NMAX; ++m) {
        if (m < n) {
          const float a = Ah[i * ld + m];
          const float p = a * x[m];
          const float pe = fmaf(a, x[m], -p);
          float s2, se;
          two_sum(sh, p, s2, se);
          sh = s2;
          sl += se + fmaf(Al[i * ld + m], x[m], pe);
        }
      }
      const float hv = sh + sl;
      const float lv = sl - (hv - sh);
      Mh[i * ldm + j] = hv;
      Ml[i * ldm + j] = lv;
      if (i == j) tr += (double)hv + (double)lv;
    }
  }
  tr = warp_sum(tr);
  __syncwarp();
  double t2 = 0.0;
  for (int j = lane; j < n; j += 32)
    for (int i = 0; i < n; ++i)
      t2 = fma((double)Mh[i * ldm + j] + (double)Ml[i * ldm + j], (double)Mh[j * ldm + i] + (double)Ml[j * ldm + i],
               t2);
  t2 = warp_sum(t2);
  __syncwarp();
  *tr_out = tr;
  *t2_out = t2;
}

// FP64 LU and inverse of A_k by one warp into the scratch (LU, A^-1 as
// doubles), then A^-1 split into the FP32 pair Ah + Al over the LU space and
// tr(A^-1 L) in FP64.  Returns the determinant's log, sign and singularity.
__device__ DetOut df_factor(const float* __restrict__ Ak, int n, int T, int rs, size_t ts, double* LU, int* perm,
                            float** Ah_out, float** Al_out, double* tl_out) {
  const int lane = threadIdx.x & 31;
  const DetScratch sc(n);
  const int ld = sc.ld;
  double* Ai = LU + n * ld;
  DetOut o{};
  for (int e = lane; e < n * n; e += 32) LU[(e / n) * ld + (e % n)] = (double)Ak[(e / n) * rs + (e % n)];
  __syncwarp();
  double growth;
  warp_lu<double>(LU, n, ld, perm, &o.ld, &o.sgn, &growth, &o.singular);
  o.refactor = 1;
  *tl_out = 0.0;
  if (o.singular || T <= 1) return o;
  warp_inverse<double>(LU, Ai, perm, n, ld);
  float* Ah = reinterpret_cast<float*>(LU);  // the factors are no longer needed
  float* Al = Ah + n * ld;
  for (int e = lane; e < n * ld; e += 32) {
    const double v = Ai[e];
    const float hv = (float)v;
    Ah[e] = hv;
    Al[e] = (float)(v - (double)hv);
  }
  __syncwarp();
  double tl = 0.0;
  const float* L = Ak + ts;
  for (int e = lane; e < n * n; e += 32) {
    const int m = e / n, i = e - m * n;
    tl = fma(Ai[i * ld + m], (double)L[m * rs + i], tl);
  }
  *tl_out = warp_sum(tl);
  *Ah_out = Ah;
  *Al_out = Al;
  return o;
}

template <int NMAX>
__device__ DetOut det_stage_df(const float* __restrict__ Ak, int n, int T, int rs, size_t ts, char* scratch,
                               float* t1s) {
  const int lane = threadIdx.x & 31;
  const DetScratch sc(n);
  const int ld = sc.ld, ldm = sc.ldm;
  double* LU = reinterpret_cast<double*>(scratch);
  float* Mh = reinterpret_cast<float*>(LU + 2 * n * ld);  // [n][ldm]
  float* Ml = Mh + n * ldm;                               // [n][ldm] (both inside the 2 n ldm doubles)
  int* perm = reinterpret_cast<int*>(scratch + (size_t)(2 * n * ld + 2 * n * ldm) * 8);
  float *Ah = nullptr, *Al = nullptr;
  double tl;
  DetOut o = df_factor(Ak, n, T, rs, ts, LU, perm, &Ah, &Al, &tl);
  if (o.singular || T <= 1) return o;
  double t2acc = 0.0, qacc = 0.0;
  for (int t = 2; t < T; ++t) {
    double tr, t2;
    df_direction<NMAX>(Ah, Al, Ak + (size_t)t * ts, Mh, Ml, n, ld, ldm, rs, &tr, &t2);
    if (lane == 0) t1s[t - 2] = (float)tr;
    t2acc += t2;
    qacc = fma(tr, tr, qacc);
  }
  o.tL = (float)tl;
  o.t2 = (float)t2acc;
  o.q = (float)qacc;
  o.kin = tl - t2acc + qacc;
  return o;
}

// Warp 0 of a walker's block: FP64 signed log-sum-exp over the K
// determinants and, for T > 1, the gradient, Laplacian and kinetic energy
// from the per-determinant traces (lds / sgs / tLs / t2s / qs / t1s in shared
// memory; ints = {any refactored, any singular}).
__device__ void logdet_finish(int w, int K, int T, double* lds, const double* kins, float* sgs, float* tLs,
                              const float* t2s, const float* qs, const float* t1s, const int* ints,
                              const float* __restrict__ pe,
                              float* __restrict__ logpsi, float* __restrict__ sign, float* __restrict__ ke,
                              float* __restrict__ el, uint8_t* __restrict__ flags, int* __restrict__ n_refactor,
                              const float* __restrict__ gl_add) {
  const int lane = threadIdx.x & 31;
  const int D = T > 1 ? T - 2 : 0;
  // FP64 signed log-sum-exp over determinants, one determinant per lane
  double lmax = -INFINITY;
  for (int k = lane; k < K; k += 32)
    if (sgs[k] != 0.f) lmax = fmax(lmax, lds[k]);
  for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  double Ssum = 0.0;
  for (int k = lane; k < K; k += 32)
    if (sgs[k] != 0.f) Ssum += (double)sgs[k] * exp(lds[k] - lmax);
  Ssum = warp_sum(Ssum);
  double lp = lane == 0 ? log(fabs(Ssum)) + lmax : 0.0;
  float sg = Ssum > 0 ? 1.f : (Ssum < 0 ? -1.f : 0.f);
  bool bad = lane == 0 && !isfinite(lp);
  if (T > 1) {
    // w_k = s_k exp(ld_k - max) / S, once per determinant (FP64)
    float* wk = tLs;  // reuse: tL_k is folded into the per-det term below
    for (int k = lane; k < K; k += 32) {
      const double wt = sgs[k] != 0.f ? (double)sgs[k] * exp(lds[k] - lmax) / Ssum : 0.0;
      lds[k] = wt * kins[k];
      wk[k] = (float)wt;
    }
    __syncwarp();
    // grad_d = sum_k w_k t1_kd ; lap = sum_k w_k (tL - t2 + q) - |grad|^2
    // an additive log term (gl_add: its gradient, then its Laplacian) joins
    // the gradient before it is squared
    const float* ga = gl_add ? gl_add + (size_t)w * (D + 1) : nullptr;
    double g2 = 0.0, gt2 = 0.0;
    for (int d = lane; d < D; d += 32) {
      double g = 0.0;
      for (int k = 0; k < K; ++k) g += (double)wk[k] * (double)t1s[(size_t)k * D + d];
      g2 += g * g;
      const double gt = ga ? g + (double)ga[d] : g;
      gt2 += gt * gt;
    }
    g2 = warp_sum(g2);
    gt2 = warp_sum(gt2);
    double lap = 0.0;
    for (int k = 0; k < K; ++k) lap += lds[k];
    lap -= g2;
    if (ga) lap += (double)ga[D];
    double kin = -0.5 * (lap + gt2);
    if (lane == 0) {
      if (ke) ke[w] = (float)kin;
      if (el) el[w] = (float)(kin + (pe ? (double)pe[w] : 0.0));
    }
    bad = bad || (lane == 0 && !isfinite(kin));
  }
  if (lane == 0) {
    if (logpsi) logpsi[w] = (float)lp;
    if (sign) sign[w] = sg;
    uint8_t f = (bad ? QMC_FLAG_NONFINITE : 0) | (ints[0] ? QMC_FLAG_REFACTOR : 0) |
                (ints[1] ? QMC_FLAG_SINGULAR : 0);
    if (flags) flags[w] = f;
    if (ints[0] && n_refactor) atomicAdd(n_refactor, 1);
  }
}

// Shared-memory bytes of k_logdet's per-walker head (the launcher and the
// kernel both size it here): lds, kins [K] (double); sgs, tLs, t2s, qs [K];
// t1s [K][D]; ints [2]; wts [K]; done64 [K].
__host__ __device__ inline size_t logdet_head_bytes(int K, int D) {
  return align_up((size_t)2 * K * 8 + (size_t)4 * K * 4 + (size_t)K * D * 4 + 8 + (size_t)K * 8, 16);
}

template <int NMAX>
__global__ void __launch_bounds__(256, NMAX <= 16 ? 3 : 2) k_logdet(int n, int K, int Tp, int T, const float* __restrict__ A,
                         const float* __restrict__ pe, float* __restrict__ logpsi,
                         float* __restrict__ sign, float* __restrict__ ke, float* __restrict__ el,
                         uint8_t* __restrict__ flags, int* __restrict__ n_refactor,
                         const float* __restrict__ gl_add, int cancel) {
  extern __shared__ double shd[];
  const int w = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const int D = T > 1 ? T - 2 : 0;
  // shared layout: per-det results, then per-warp scratch
  double* lds = shd;                                    // [K]
  double* kins = lds + K;                               // [K] tL - t2 + q
  float* sgs = reinterpret_cast<float*>(kins + K);      // [K]
  float* tLs = sgs + K;                                 // [K]
  float* t2s = tLs + K;                                 // [K]
  float* qs = t2s + K;                                  // [K]
  float* t1s = qs + K;                                  // [K][D]
  int* ints = reinterpret_cast<int*>(t1s + (size_t)K * D);  // flags [2]
  float* wts = reinterpret_cast<float*>(ints + 2);          // [K] determinant weights
  int* done64 = reinterpret_cast<int*>(wts + K);            // [K] already evaluated in FP64
  const size_t head = logdet_head_bytes(K, D);
  const DetScratch sc(n);
  char* scratch = reinterpret_cast<char*>(shd) + head + sc.bytes * warp;
  if (threadIdx.x < 2) ints[threadIdx.x] = 0;
  __syncthreads();
  for (int k = warp; k < K; k += nw) {
    const float* Ak = A + amat_index(Tp, n, K, w, k, 0, 0, 0);
    const int rs = amat_row_stride(Tp, n, K);
    const size_t ts = amat_tangent_stride(n, K);
    float* t1k = t1s + (size_t)k * D;
    DetOut o = det_stage<float, NMAX>(Ak, n, T, rs, ts, scratch, t1k, false);
    if (o.refactor) {
      o = det_stage<double, NMAX>(Ak, n, T, rs, ts, scratch, t1k, true);
      o.refactor = 1;
    }
    if (lane == 0) {
      lds[k] = o.ld;
      kins[k] = o.singular ? 0.0 : o.kin;
      sgs[k] = o.singular ? 0.f : o.sgn;
      tLs[k] = o.tL;
      t2s[k] = o.t2;
      qs[k] = o.q;
      done64[k] = o.refactor;
      if (o.refactor) atomicOr(&ints[0], 1);
      if (o.singular) atomicOr(&ints[1], 1);
    }
    __syncwarp();
  }
  __syncthreads();
  if (cancel && T > 1) {
    // determinants whose FP32 kinetic term cancels too much: again, with the
    // products in double-float and the traces in FP64
    if (warp == 0) det_weights(K, lds, sgs, wts);
    __syncthreads();
    for (int k = warp; k < K; k += nw) {
      if (sgs[k] == 0.f || done64[k] || !cancel_marks(wts[k], tLs[k], t2s[k], qs[k])) continue;
      const float* Ak = A + amat_index(Tp, n, K, w, k, 0, 0, 0);
      DetOut o = det_stage_df<NMAX>(Ak, n, T, amat_row_stride(Tp, n, K), amat_tangent_stride(n, K), scratch,
                                    t1s + (size_t)k * D);
      if (lane == 0) {
        lds[k] = o.ld;
        kins[k] = o.singular ? 0.0 : o.kin;
        sgs[k] = o.singular ? 0.f : o.sgn;
        tLs[k] = o.singular ? 0.f : o.tL;
        t2s[k] = o.singular ? 0.f : o.t2;
        qs[k] = o.singular ? 0.f : o.q;
        atomicOr(&ints[0], 1);
        if (o.singular) atomicOr(&ints[1], 1);
      }
      if (o.singular)
        for (int d = lane; d < D; d += 32) t1s[(size_t)k * D + d] = 0.f;
      __syncwarp();
    }
    __syncthreads();
  }
  if (warp != 0) return;
  logdet_finish(w, K, T, lds, kins, sgs, tLs, t2s, qs, t1s, ints, pe, logpsi, sign, ke, el, flags, n_refactor,
                gl_add);
}

// Tangent determinant stage for 16 < n <= 64: three launches.
//
// k_logdet_fl_wide (FP32, one block of 8 warps per walker, the K
// determinants in turn): warp 0 factorises and inverts A_k; then every warp
// takes a share of the Jacobian directions d, computing
// P_d = A_k^-1 J_d A_k column by column into its own shared-memory tile for
// t1_d = tr P_d and tr(P_d^2), while all threads share tL = tr(A_k^-1 L A_k).
// A determinant whose pivot growth exceeds kRefactorGrowth, or whose smallest
// pivot is below kRefactorPivot x max|A|, is marked instead: inverting it in
// FP64 and forming its products in FP32 is not enough (the products cancel),
// so it goes whole to FP64.  A walker without marked determinants finishes in
// this kernel; one with marks leaves its per-determinant results in a record
// in global memory.
//
// k_logdet_fl_det64 (one warp per marked (walker, determinant)) recomputes
// the marked determinants in FP64 into the records, spread over the GPU, and
// k_logdet_fl_finish completes the marked walkers from their records.
struct WideShape {
  int ld, ldm;
  size_t head, bytes;
  __host__ __device__ WideShape(int n, int K, int D, int nw) {
    ld = (n + 3) / 4 * 4;
    ldm = (n % 2 == 0) ? n + 1 : n + 2;
    // lds[K], kins[K] (double), sgs, tLs, t2s, qs [K], t1s [K][D], ints[4], then
    // red: [nw][3] partial traces, later [K] weights
    head = align_up((size_t)2 * K * 8 + (size_t)4 * K * 4 + (size_t)K * D * 4 + 16 +
                        (size_t)(3 * nw > K ? 3 * nw : K) * 4,
                    16);
    bytes = head + (size_t)2 * n * ld * 4 + align_up((size_t)n * 4, 16) + (size_t)nw * n * ldm * 4;
  }
};

// Per-walker record of the determinant results (global scratch):
// ld[K], kin[K] (double), sg[K], tL[K], t2[K], q[K], t1[K][D] (float),
// mark[K] (byte), any-singular (int).
struct DetRecord {
  size_t kin, sg, tL, t2, q, t1, mark, sing, bytes;
  __host__ __device__ DetRecord(int K, int D) {
    kin = (size_t)K * 8;
    sg = kin + (size_t)K * 8;
    tL = sg + (size_t)K * 4;
    t2 = tL + (size_t)K * 4;
    q = t2 + (size_t)K * 4;
    t1 = q + (size_t)K * 4;
    mark = t1 + (size_t)K * D * 4;
    sing = align_up(mark + (size_t)K, 4);
    bytes = align_up(sing + 4, 16);
  }
};

size_t logdet_fl_scratch_bytes(int B, int K, int T) {
  const int D = T > 1 ? T - 2 : 0;
  return align_up((size_t)B, 16) + (size_t)B * DetRecord(K, D).bytes;
}

template <int NMAX>
__global__ void __launch_bounds__(256, 2) k_logdet_fl_wide(int n, int K, int Tp, int T, const float* __restrict__ A,
                                                            const float* __restrict__ pe, float* __restrict__ logpsi,
                                                            float* __restrict__ sign, float* __restrict__ ke,
                                                            float* __restrict__ el, uint8_t* __restrict__ flags,
                                                            uint8_t* __restrict__ redo, char* __restrict__ records,
                                                            const float* __restrict__ gl_add, int cancel) {
  extern __shared__ double shd[];
  const int w = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int D = T - 2;
  const WideShape sh(n, K, D, nw);
  const DetRecord rec(K, D);
  char* rw = records + (size_t)w * rec.bytes;
  const int ld = sh.ld, ldm = sh.ldm;
  double* lds = shd;                                         // [K]
  double* kins = lds + K;                                    // [K] tL - t2 + q
  float* sgs = reinterpret_cast<float*>(kins + K);           // [K]
  float* tLs = sgs + K;                                      // [K]
  float* t2s = tLs + K;                                      // [K]
  float* qs = t2s + K;                                       // [K]
  float* t1s = qs + K;                                       // [K][D]
  int* ints = reinterpret_cast<int*>(t1s + (size_t)K * D);   // any marked, any singular, skip this det
  float* red = reinterpret_cast<float*>(ints + 4);           // [nw][3]
  float* LU = reinterpret_cast<float*>(reinterpret_cast<char*>(shd) + sh.head);
  float* Ainv = LU + (size_t)n * ld;
  int* perm = reinterpret_cast<int*>(Ainv + (size_t)n * ld);
  float* Ms = reinterpret_cast<float*>(reinterpret_cast<char*>(perm) + align_up((size_t)n * 4, 16)) +
              (size_t)warp * n * ldm;
  if (threadIdx.x < 3) ints[threadIdx.x] = 0;
  const int rs = amat_row_stride(Tp, n, K);
  const size_t ts = amat_tangent_stride(n, K);
  for (int k = 0; k < K; ++k) {
    const float* Ak = A + amat_index(Tp, n, K, w, k, 0, 0, 0);
    __syncthreads();  // the previous determinant is done with LU / Ainv / red
    if (warp == 0) {
      for (int e = lane; e < n * n; e += 32) LU[(e / n) * ld + (e % n)] = Ak[(e / n) * rs + (e % n)];
      __syncwarp();
      double ldv, growth, pivmin;
      float sg;
      int sing;
      warp_lu<float>(LU, n, ld, perm, &ldv, &sg, &growth, &sing, &pivmin);
      const bool mark = !sing && (!(growth <= (double)kRefactorGrowth) || pivmin < (double)kRefactorPivot);
      if (!sing && !mark) warp_inverse<float>(LU, Ainv, perm, n, ld);
      if (lane == 0) {
        lds[k] = ldv;
        sgs[k] = sing ? 0.f : sg;
        ints[2] = sing || mark;
        if (mark) ints[0] = 1;
        if (sing) ints[1] = 1;
        reinterpret_cast<uint8_t*>(rw + rec.mark)[k] = mark ? 1 : 0;
      }
    }
    __syncthreads();
    if (ints[2]) {  // singular (zero weight) or marked (recomputed in FP64)
      for (int d = threadIdx.x; d < D; d += blockDim.x) t1s[(size_t)k * D + d] = 0.f;
      if (threadIdx.x == 0) {
        tLs[k] = t2s[k] = qs[k] = 0.f;
        kins[k] = 0.0;
      }
      continue;
    }
    float tl = 0.f;
    {
      const float* L = Ak + ts;
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int m = e / n, i = e - m * n;
        tl = fmaf(Ainv[i * ld + m], L[m * rs + i], tl);
      }
    }
    tl = warp_sum(tl);
    float t2acc = 0.f, qacc = 0.f;
    for (int d = warp; d < D; d += nw) {
      const float tr = warp_product_f32<NMAX>(Ainv, Ak + (size_t)(2 + d) * ts, Ms, n, ld, ldm, rs);
      const float t2 = warp_trace_sq<float>(Ms, n, ldm);
      if (lane == 0) t1s[(size_t)k * D + d] = tr;
      t2acc += t2;
      qacc = fmaf(tr, tr, qacc);
    }
    if (lane == 0) {
      red[3 * warp] = tl;
      red[3 * warp + 1] = t2acc;
      red[3 * warp + 2] = qacc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      float a = 0.f, b = 0.f, c = 0.f;
      for (int v = 0; v < nw; ++v) {
        a += red[3 * v];
        b += red[3 * v + 1];
        c += red[3 * v + 2];
      }
      tLs[k] = a;
      t2s[k] = b;
      qs[k] = c;
      kins[k] = (double)a - (double)b + (double)c;
    }
  }
  __syncthreads();
  if (cancel) {
    // determinants whose FP32 kinetic term cancels too much join the FP64 pass
    float* wts = red;  // [K] (red is sized for 3 nw >= K floats: see WideShape)
    if (warp == 0) {
      det_weights(K, lds, sgs, wts);
      uint8_t* mk = reinterpret_cast<uint8_t*>(rw + rec.mark);
      bool any = false;
      for (int k = lane; k < K; k += 32)
        if (sgs[k] != 0.f && !mk[k] && cancel_marks(wts[k], tLs[k], t2s[k], qs[k])) {
          mk[k] = 1;
          any = true;
        }
      if (__any_sync(0xffffffffu, any) && lane == 0) ints[0] = 1;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) redo[w] = ints[0] ? 1 : 0;
  if (ints[0]) {  // leave the record for the FP64 pass
    double* rld = reinterpret_cast<double*>(rw);
    double* rkin = reinterpret_cast<double*>(rw + rec.kin);
    float* rsg = reinterpret_cast<float*>(rw + rec.sg);
    float* rtL = reinterpret_cast<float*>(rw + rec.tL);
    float* rt2 = reinterpret_cast<float*>(rw + rec.t2);
    float* rq = reinterpret_cast<float*>(rw + rec.q);
    float* rt1 = reinterpret_cast<float*>(rw + rec.t1);
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
      rld[k] = lds[k];
      rkin[k] = kins[k];
      rsg[k] = sgs[k];
      rtL[k] = tLs[k];
      rt2[k] = t2s[k];
      rq[k] = qs[k];
    }
    for (int e = threadIdx.x; e < K * D; e += blockDim.x) rt1[e] = t1s[e];
    if (threadIdx.x == 0) *reinterpret_cast<int*>(rw + rec.sing) = ints[1];
    return;
  }
  if (warp != 0) return;
  logdet_finish(w, K, T, lds, kins, sgs, tLs, t2s, qs, t1s, ints, pe, logpsi, sign, ke, el, flags, nullptr, gl_add);
}

// Double-float re-evaluation of a marked (walker, determinant): a block of
// kDet64Warps warps; warp 0 factorises and inverts A_k in FP64 and forms
// tr(A^-1 L), then every warp takes a share of the Jacobian directions with
// its own product tiles; the FP64 sums over directions are combined in warp
// order.  Shared memory: LU and A^-1 (doubles), the permutation, then the
// per-warp hi/lo product tiles.
constexpr int kDet64Warps = 4;
struct Det64Shape {
  size_t head, per_warp, bytes;
  __host__ __device__ Det64Shape(int n) {
    const DetScratch sc(n);
    head = align_up((size_t)2 * n * sc.ld * 8 + (size_t)n * 4, 16) + 64;
    per_warp = align_up((size_t)2 * n * sc.ldm * 4, 16);
    bytes = head + kDet64Warps * per_warp + (size_t)kDet64Warps * 2 * 8;
  }
};

template <int NMAX>
__global__ void __launch_bounds__(kDet64Warps * 32) k_logdet_fl_det64(int n, int K, int Tp, int T,
                                                                       const float* __restrict__ A,
                                                                       const uint8_t* __restrict__ redo,
                                                                       char* __restrict__ records) {
  extern __shared__ double shd[];
  const int w = blockIdx.x / K, k = blockIdx.x % K;
  if (!redo[w]) return;
  const int D = T - 2;
  const DetRecord rec(K, D);
  char* rw = records + (size_t)w * rec.bytes;
  if (!reinterpret_cast<const uint8_t*>(rw + rec.mark)[k]) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const DetScratch sc(n);
  const Det64Shape sh(n);
  char* base = reinterpret_cast<char*>(shd);
  double* LU = reinterpret_cast<double*>(base);
  int* perm = reinterpret_cast<int*>(base + (size_t)2 * n * sc.ld * 8);
  int* flag = reinterpret_cast<int*>(base + sh.head - 64);  // singular
  double* red = reinterpret_cast<double*>(base + sh.head + kDet64Warps * sh.per_warp);  // [warps][2]
  float* Mh = reinterpret_cast<float*>(base + sh.head + warp * sh.per_warp);
  float* Ml = Mh + n * sc.ldm;
  const float* Ak = A + amat_index(Tp, n, K, w, k, 0, 0, 0);
  const int rs = amat_row_stride(Tp, n, K);
  const size_t ts = amat_tangent_stride(n, K);
  float* t1k = reinterpret_cast<float*>(rw + rec.t1) + (size_t)k * D;
  DetOut o{};
  double tl = 0.0;
  if (warp == 0) {
    float *Ah = nullptr, *Al = nullptr;
    o = df_factor(Ak, n, T, rs, ts, LU, perm, &Ah, &Al, &tl);
    if (lane == 0) *flag = o.singular;
  }
  __syncthreads();
  if (*flag) {
    if (threadIdx.x == 0) {
      reinterpret_cast<double*>(rw)[k] = o.ld;
      reinterpret_cast<double*>(rw + rec.kin)[k] = 0.0;
      reinterpret_cast<float*>(rw + rec.sg)[k] = 0.f;
      reinterpret_cast<float*>(rw + rec.tL)[k] = 0.f;
      reinterpret_cast<float*>(rw + rec.t2)[k] = 0.f;
      reinterpret_cast<float*>(rw + rec.q)[k] = 0.f;
      atomicOr(reinterpret_cast<int*>(rw + rec.sing), 1);
    }
    for (int d = threadIdx.x; d < D; d += blockDim.x) t1k[d] = 0.f;
    return;
  }
  const float* Ah = reinterpret_cast<const float*>(LU);
  const float* Al = Ah + n * sc.ld;
  double t2acc = 0.0, qacc = 0.0;
  for (int d = warp; d < D; d += kDet64Warps) {
    double tr, t2;
    df_direction<NMAX>(Ah, Al, Ak + (size_t)(2 + d) * ts, Mh, Ml, n, sc.ld, sc.ldm, rs, &tr, &t2);
    if (lane == 0) t1k[d] = (float)tr;
    t2acc += t2;
    qacc = fma(tr, tr, qacc);
  }
  if (lane == 0) {
    red[2 * warp] = t2acc;
    red[2 * warp + 1] = qacc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t2s = 0.0, qs = 0.0;
    for (int v = 0; v < kDet64Warps; ++v) {
      t2s += red[2 * v];
      qs += red[2 * v + 1];
    }
    reinterpret_cast<double*>(rw)[k] = o.ld;
    reinterpret_cast<double*>(rw + rec.kin)[k] = tl - t2s + qs;
    reinterpret_cast<float*>(rw + rec.sg)[k] = o.sgn;
    reinterpret_cast<float*>(rw + rec.tL)[k] = (float)tl;
    reinterpret_cast<float*>(rw + rec.t2)[k] = (float)t2s;
    reinterpret_cast<float*>(rw + rec.q)[k] = (float)qs;
  }
}

__global__ void __launch_bounds__(32) k_logdet_fl_finish(int K, int T, const uint8_t* __restrict__ redo,
                                                          const char* __restrict__ records,
                                                          const float* __restrict__ pe, float* __restrict__ logpsi,
                                                          float* __restrict__ sign, float* __restrict__ ke,
                                                          float* __restrict__ el, uint8_t* __restrict__ flags,
                                                          const float* __restrict__ gl_add) {
  extern __shared__ double shd[];
  const int w = blockIdx.x;
  if (!redo[w]) return;
  const int D = T - 2;
  const DetRecord rec(K, D);
  const char* rw = records + (size_t)w * rec.bytes;
  double* lds = shd;
  double* kins = lds + K;
  float* sgs = reinterpret_cast<float*>(kins + K);
  float* tLs = sgs + K;
  float* t2s = tLs + K;
  float* qs = t2s + K;
  float* t1s = qs + K;
  int* ints = reinterpret_cast<int*>(t1s + (size_t)K * D);
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    lds[k] = reinterpret_cast<const double*>(rw)[k];
    kins[k] = reinterpret_cast<const double*>(rw + rec.kin)[k];
    sgs[k] = reinterpret_cast<const float*>(rw + rec.sg)[k];
    tLs[k] = reinterpret_cast<const float*>(rw + rec.tL)[k];
    t2s[k] = reinterpret_cast<const float*>(rw + rec.t2)[k];
    qs[k] = reinterpret_cast<const float*>(rw + rec.q)[k];
  }
  for (int e = threadIdx.x; e < K * D; e += blockDim.x) t1s[e] = reinterpret_cast<const float*>(rw + rec.t1)[e];
  if (threadIdx.x == 0) {
    ints[0] = 1;
    ints[1] = *reinterpret_cast<const int*>(rw + rec.sing);
  }
  __syncwarp();
  logdet_finish(w, K, T, lds, kins, sgs, tLs, t2s, qs, t1s, ints, pe, logpsi, sign, ke, el, flags, nullptr, gl_add);
}

// Value-only determinant stage (MH passes): LU in registers.  A segment of
// SEG lanes factorises one matrix, lane i holding row i, so a warp works on
// 32/SEG matrices at once.  Rows stay in their lanes: step k picks the pivot
// among the lanes not yet used (one packed |value|:lane key, SEG-lane max by
// shuffles), the pivot lane writes its row to a per-segment shared-memory
// buffer that every lane reads back, and the permutation's parity comes from
// the used-lane mask.  |det| is a running FP32 product of the pivots kept as
// mantissa and exponent; the multipliers are not kept.  Matrices whose pivot
// growth exceeds the threshold are re-factorised in FP64 afterwards by warp 0.
template <int SEG>
__device__ __forceinline__ unsigned pivot_key(float v, int i, bool cand) {
  constexpr unsigned IB = SEG <= 4 ? 2 : SEG <= 8 ? 3 : SEG <= 16 ? 4 : 5;  // lane index bits
  constexpr unsigned MARK = 1u << IB;
  constexpr unsigned KEEP = ~((MARK << 1) - 1u);
  // |v| bit patterns order like the values; ties (to 2^-(23-IB-1) relative)
  // go to the lower lane, and any candidate beats a non-candidate (key 0)
  return cand ? ((__float_as_uint(fabsf(v)) & KEEP) | MARK | (unsigned)(SEG - 1 - i)) : 0u;
}

template <int SEG>
__global__ void __launch_bounds__(256) k_logdet_value(int B, int n, int K, int WB, float* __restrict__ A,
                                                      float* __restrict__ logpsi, float* __restrict__ sign,
                                                      uint8_t* __restrict__ flags, EnvArgs env) {
  extern __shared__ double shv[];
  const int nmat = WB * K;
  double* lds = shv;                                       // [nmat]
  float* sgs = reinterpret_cast<float*>(lds + nmat);       // [nmat]
  int* redo = reinterpret_cast<int*>(sgs + nmat);          // [nmat] re-factorise flags
  int* singular = redo + nmat;                             // [nmat]
  float* rowbuf = reinterpret_cast<float*>(reinterpret_cast<char*>(shv) + align_up((size_t)nmat * 20, 16));
  char* scratch = reinterpret_cast<char*>(rowbuf + 8 * 64);  // FP64 re-factorisation
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / SEG, i = lane % SEG;
  // two pivot-row buffers per segment, used on alternate steps
  float* rb0 = rowbuf + warp * 64 + sub * SEG;
  float* rb1 = rb0 + 32;
  const int w0 = blockIdx.x * WB;
  const int mpw = 32 / SEG;
  const unsigned all_rows = n >= 32 ? 0xffffffffu : ((1u << n) - 1u);
  int my_redo = 0;
  for (int base = warp * mpw; base < nmat; base += 8 * mpw) {
    const int mloc = base + sub;
    const int w = w0 + mloc / K;
    const bool active = mloc < nmat && w < B;
    float r[SEG];
    float* Am = A + ((size_t)w * K + (mloc % K)) * n * n;
#pragma unroll
    for (int j = 0; j < SEG; ++j) r[j] = (active && i < n && j < n) ? Am[i * n + j] : 0.f;
    if (env.env && active && i < n) {  // envelope factors of row i
      const float* Em = env.env + ((size_t)w * K + (mloc % K)) * n * n;
#pragma unroll
      for (int j = 0; j < SEG; ++j)
        if (j < n) r[j] *= __ldg(Em + i * n + j);
    }
    float amax = 0.f;
#pragma unroll
    for (int j = 0; j < SEG; ++j) amax = fmaxf(amax, fabsf(r[j]));
#pragma unroll
    for (int o = SEG / 2; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o, SEG));
    bool cand = active && i < n;
    unsigned unused = all_rows;
    __syncwarp();  // the previous matrix's last pivot rows have been read
    int inversions = 0, ex = 0, sing = 0;
    float mant = 1.f, sg = 1.f, umax = 0.f;
#pragma unroll
    for (int k = 0; k < SEG; ++k) {
      if (k < n) {
        unsigned key = pivot_key<SEG>(r[k], i, cand);
#pragma unroll
        for (int o = SEG / 2; o > 0; o >>= 1) key = max(key, __shfl_xor_sync(0xffffffffu, key, o, SEG));
        const int p = SEG - 1 - (int)(key & (unsigned)(SEG - 1));
        inversions += __popc(unused & ((1u << p) - 1u));
        unused &= ~(1u << p);
        float* rb = (k & 1) ? rb1 : rb0;
        if (i == p) {
#pragma unroll
          for (int q = 0; q < SEG / 4; ++q)
            if (4 * q + 3 >= k)
              *reinterpret_cast<float4*>(rb + 4 * q) = make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
          cand = false;
        }
        __syncwarp();
        float u[SEG];
#pragma unroll
        for (int q = 0; q < SEG / 4; ++q)
          if (4 * q + 3 >= k) {
            const float4 v = *reinterpret_cast<const float4*>(rb + 4 * q);
            u[4 * q] = v.x; u[4 * q + 1] = v.y; u[4 * q + 2] = v.z; u[4 * q + 3] = v.w;
          }
        const float ukk = u[k];
#pragma unroll
        for (int j = 0; j < SEG; ++j)
          if (j >= k) umax = fmaxf(umax, fabsf(u[j]));
        if (ukk == 0.f) sing = 1;
        if (ukk < 0.f) sg = -sg;
        int e2;
        mant = frexpf(mant * fabsf(ukk), &e2);
        ex += e2;
        if (cand && ukk != 0.f) {
          const float l = r[k] / ukk;
#pragma unroll
          for (int j = 0; j < SEG; ++j)
            if (j > k) r[j] = fmaf(-l, u[j], r[j]);
        }
      }
    }
    if (inversions & 1) sg = -sg;
    if (active && i == 0) {
      lds[mloc] = sing ? -INFINITY : (double)logf(mant) + (double)ex * 0.69314718055994530942;
      sgs[mloc] = sing ? 0.f : sg;
      singular[mloc] = sing;
      const int rd = (!sing && !(umax <= kRefactorGrowth * amax)) ? 1 : 0;
      redo[mloc] = rd;
      my_redo |= rd;
    }
  }
  // rare: FP64 re-factorisation of matrices with large pivot growth
  if (__syncthreads_or(my_redo)) {
    if (warp == 0) {
      for (int mloc = 0; mloc < nmat; ++mloc) {
        const int w = w0 + mloc / K;
        if (w >= B || !redo[mloc]) continue;
        float* Am = A + ((size_t)w * K + (mloc % K)) * n * n;
        if (env.env) {  // the FP64 pass reads the matrix with its envelope factors
          const float* Em = env.env + ((size_t)w * K + (mloc % K)) * n * n;
          for (int e = lane; e < n * n; e += 32) Am[e] *= Em[e];
          __syncwarp();
        }
        DetOut o = det_stage<double, 16>(Am, n, 1, n, (size_t)n * n, scratch, nullptr, true);
        if (lane == 0) {
          lds[mloc] = o.ld;
          sgs[mloc] = o.singular ? 0.f : o.sgn;
          singular[mloc] = o.singular;
        }
        __syncwarp();
      }
    }
    __syncthreads();
  }
  // signed log-sum-exp per walker, one warp per walker: FP64 determinant
  // logs and sum, FP32 exponentials of the (non-positive) differences
  for (int wl = warp; wl < WB; wl += 8) {
    const int w = w0 + wl;
    if (w >= B) break;
    const double* ldw = lds + wl * K;
    const float* sgw = sgs + wl * K;
    double lmax = -INFINITY;
    for (int k = lane; k < K; k += 32)
      if (sgw[k] != 0.f) lmax = fmax(lmax, ldw[k]);
    for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    double S = 0.0;
    int anyredo = 0, anysing = 0;
    for (int k = lane; k < K; k += 32) {
      if (sgw[k] != 0.f) S += (double)(sgw[k] * expf((float)(ldw[k] - lmax)));
      anyredo |= redo[wl * K + k];
      anysing |= singular[wl * K + k];
    }
    S = warp_sum(S);
    anyredo = __any_sync(0xffffffffu, anyredo);
    anysing = __any_sync(0xffffffffu, anysing);
    if (lane == 0) {
      const double aS = fabs(S);
      double lp = (aS > 1e-30 ? (double)logf((float)aS) : log(aS)) + lmax;
      if (logpsi) logpsi[w] = (float)lp;
      if (sign) sign[w] = S > 0 ? 1.f : (S < 0 ? -1.f : 0.f);
      if (flags)
        flags[w] = (!isfinite(lp) ? QMC_FLAG_NONFINITE : 0) | (anyredo ? QMC_FLAG_REFACTOR : 0) |
                   (anysing ? QMC_FLAG_SINGULAR : 0);
    }
  }
}

static cudaError_t launch_logdet_value(cudaStream_t s, int B, int n, int K, float* A, float* logpsi,
                                       float* sign, uint8_t* flags, const EnvArgs* envp) {
  EnvArgs env{};
  if (envp) env = *envp;
  const int seg = n <= 4 ? 4 : n <= 8 ? 8 : n <= 16 ? 16 : 32;
  const int per_pass = 8 * (32 / seg);
  const int WB = std::max(1, per_pass / K);
  const size_t sm = align_up((size_t)WB * K * 20, 16) + 8 * 64 * sizeof(float) + DetScratch(n).bytes;
  const unsigned grid = (unsigned)((B + WB - 1) / WB);
  switch (seg) {
    case 4: k_logdet_value<4><<<grid, 256, sm, s>>>(B, n, K, WB, A, logpsi, sign, flags, env); break;
    case 8: k_logdet_value<8><<<grid, 256, sm, s>>>(B, n, K, WB, A, logpsi, sign, flags, env); break;
    case 16: k_logdet_value<16><<<grid, 256, sm, s>>>(B, n, K, WB, A, logpsi, sign, flags, env); break;
    default: k_logdet_value<32><<<grid, 256, sm, s>>>(B, n, K, WB, A, logpsi, sign, flags, env); break;
  }
  return cudaGetLastError();
}

// Value-only determinants for 32 < n <= 64: one block per walker, one warp
// per matrix at a time, FP32 LU in shared memory (warp_lu, partial pivoting),
// matrices with pivot growth above the threshold re-factorised in FP64 by
// warp 0, then the FP64 signed log-sum-exp.  Shared memory holds one FP32
// matrix per warp, so blocks stay small (the tangent kernel k_logdet sizes
// its scratch for the FP64 inverse and products).
constexpr int kLuWarps = 8;
__global__ void __launch_bounds__(kLuWarps * 32) k_logdet_value_smem(int n, int K, const float* __restrict__ A,
                                                                     float* __restrict__ logpsi,
                                                                     float* __restrict__ sign,
                                                                     uint8_t* __restrict__ flags) {
  extern __shared__ double sml[];
  const int ld = (n + 3) / 4 * 4;
  double* lds = sml;                                         // [K]
  float* sgs = reinterpret_cast<float*>(lds + K);            // [K]
  int* redo = reinterpret_cast<int*>(sgs + K);               // [K]
  int* sing = redo + K;                                      // [K]
  char* base = reinterpret_cast<char*>(sml) + align_up((size_t)K * 20, 16);  // lds, sgs, redo, sing
  const size_t per_warp = align_up((size_t)n * ld * 4 + (size_t)n * 4, 16);
  const int w = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* LU = reinterpret_cast<float*>(base + per_warp * warp);
  int* perm = reinterpret_cast<int*>(LU + (size_t)n * ld);
  for (int k = warp; k < K; k += kLuWarps) {
    const float* Ak = A + ((size_t)w * K + k) * n * n;
    for (int e = lane; e < n * n; e += 32) LU[(e / n) * ld + (e % n)] = Ak[e];
    __syncwarp();
    double la, growth;
    float sg;
    int sgl = 0;
    warp_lu<float>(LU, n, ld, perm, &la, &sg, &growth, &sgl);
    if (lane == 0) {
      lds[k] = sgl ? -INFINITY : la;
      sgs[k] = sgl ? 0.f : sg;
      sing[k] = sgl;
      redo[k] = (!sgl && !(growth <= (double)kRefactorGrowth)) ? 1 : 0;
    }
    __syncwarp();
  }
  __syncthreads();
  if (warp != 0) return;
  double* LU64 = reinterpret_cast<double*>(base + per_warp * kLuWarps);
  int* perm64 = reinterpret_cast<int*>(LU64 + (size_t)n * ld);
  for (int k = 0; k < K; ++k) {
    if (!redo[k]) continue;
    const float* Ak = A + ((size_t)w * K + k) * n * n;
    for (int e = lane; e < n * n; e += 32) LU64[(e / n) * ld + (e % n)] = (double)Ak[e];
    __syncwarp();
    double la, growth;
    float sg;
    int sgl = 0;
    warp_lu<double>(LU64, n, ld, perm64, &la, &sg, &growth, &sgl);
    if (lane == 0) {
      lds[k] = sgl ? -INFINITY : la;
      sgs[k] = sgl ? 0.f : sg;
      sing[k] = sgl;
    }
    __syncwarp();
  }
  double lmax = -INFINITY;
  int anyredo = 0, anysing = 0;
  for (int k = lane; k < K; k += 32) {
    if (sgs[k] != 0.f) lmax = fmax(lmax, lds[k]);
    anyredo |= redo[k];
    anysing |= sing[k];
  }
  for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  double S = 0.0;
  for (int k = lane; k < K; k += 32)
    if (sgs[k] != 0.f) S += (double)sgs[k] * exp(lds[k] - lmax);
  S = warp_sum(S);
  anyredo = __any_sync(0xffffffffu, anyredo);
  anysing = __any_sync(0xffffffffu, anysing);
  if (lane == 0) {
    const double lp = log(fabs(S)) + lmax;
    if (logpsi) logpsi[w] = (float)lp;
    if (sign) sign[w] = S > 0 ? 1.f : (S < 0 ? -1.f : 0.f);
    if (flags)
      flags[w] = (isfinite(lp) ? 0 : QMC_FLAG_NONFINITE) | (anyredo ? QMC_FLAG_REFACTOR : 0) |
                 (anysing ? QMC_FLAG_SINGULAR : 0);
  }
}

static cudaError_t launch_logdet_value_smem(cudaStream_t s, int B, int n, int K, const float* A, float* logpsi,
                                            float* sign, uint8_t* flags) {
  const size_t ld = (n + 3) / 4 * 4;
  const size_t per_warp = align_up((size_t)n * ld * 4 + (size_t)n * 4, 16);
  const size_t sm = align_up((size_t)K * 20, 16) + per_warp * kLuWarps + (size_t)n * ld * 8 + (size_t)n * 4;
  if (sm > 200 * 1024) return cudaErrorInvalidValue;
  static int attr_dev = -1;
  int dev;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (attr_dev != dev) {
    e = cudaFuncSetAttribute(k_logdet_value_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    attr_dev = dev;
  }
  k_logdet_value_smem<<<B, kLuWarps * 32, sm, s>>>(n, K, A, logpsi, sign, flags);
  return cudaGetLastError();
}

cudaError_t launch_logdet(cudaStream_t s, int B, int n, int K, int Tp, int T, const float* A,
                          const float* pe, float* logpsi, float* sign, float* ke, float* el,
                          uint8_t* flags, int* n_refactor, const EnvArgs* env, const float* gl_add,
                          void* fl_scratch, bool cancel64) {
  if (T > 1 && n > 16 && n <= 64 && fl_scratch && !env) {
    const int nw = 8;
    const WideShape sh(n, K, T - 2, nw);
    const size_t fin = (size_t)2 * K * 8 + (size_t)4 * K * 4 + (size_t)K * (T - 2) * 4 + 16;
    if (sh.bytes <= 110 * 1024 && Det64Shape(n).bytes <= 220 * 1024 && fin <= 110 * 1024) {
      uint8_t* redo = static_cast<uint8_t*>(fl_scratch);
      char* records = static_cast<char*>(fl_scratch) + align_up((size_t)B, 16);
      int dev;
      cudaError_t e = cudaGetDevice(&dev);
      if (e != cudaSuccess) return e;
#define QMC_LDW(NM)                                                                                         \
  {                                                                                                         \
    static int set_dev = -1;                                                                                \
    if (set_dev != dev) {                                                                                   \
      e = cudaFuncSetAttribute(k_logdet_fl_wide<NM>, cudaFuncAttributeMaxDynamicSharedMemorySize, 110 * 1024); \
      if (e == cudaSuccess)                                                                                 \
        e = cudaFuncSetAttribute(k_logdet_fl_det64<NM>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                                 220 * 1024);                                                               \
      if (e == cudaSuccess)                                                                                 \
        e = cudaFuncSetAttribute(k_logdet_fl_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, 110 * 1024); \
      if (e != cudaSuccess) return e;                                                                       \
      set_dev = dev;                                                                                        \
    }                                                                                                       \
    k_logdet_fl_wide<NM><<<B, 32 * nw, sh.bytes, s>>>(n, K, Tp, T, A, pe, logpsi, sign, ke, el, flags, redo, \
                                                      records, gl_add, cancel64 ? 1 : 0);                   \
    k_logdet_fl_det64<NM><<<B * K, kDet64Warps * 32, Det64Shape(n).bytes, s>>>(n, K, Tp, T, A, redo, records); \
  }
      if (n <= 32) QMC_LDW(32)
      else QMC_LDW(64)
#undef QMC_LDW
      k_logdet_fl_finish<<<B, 32, fin, s>>>(K, T, redo, records, pe, logpsi, sign, ke, el, flags, gl_add);
      return cudaGetLastError();
    }
  }
  if (T == 1 && n <= 32) return launch_logdet_value(s, B, n, K, const_cast<float*>(A), logpsi, sign, flags, env);
  if (T == 1 && n <= 64 && !env) return launch_logdet_value_smem(s, B, n, K, A, logpsi, sign, flags);
  if (env) return cudaErrorInvalidValue;  // tangent passes take enveloped matrices
  const int D = T > 1 ? T - 2 : 0;
  const size_t head = logdet_head_bytes(K, D);
  const DetScratch sc(n);
  int nw = (int)((200 * 1024 - head) / sc.bytes);
  nw = nw < 1 ? 1 : nw;
  nw = nw > 8 ? 8 : nw;
  nw = nw > K ? K : nw;
  size_t sm = head + sc.bytes * nw;
  if (sm > 220 * 1024) return cudaErrorInvalidValue;
  int dev;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
#define QMC_LD(NM)                                                                          \
  {                                                                                         \
    static int set_dev = -1;                                                                \
    if (set_dev != dev) {                                                                   \
      e = cudaFuncSetAttribute(k_logdet<NM>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                               220 * 1024);                                                 \
      if (e != cudaSuccess) return e;                                                       \
      set_dev = dev;                                                                        \
    }                                                                                       \
    k_logdet<NM><<<B, 32 * nw, sm, s>>>(n, K, Tp, T, A, pe, logpsi, sign, ke, el, flags,    \
                                        n_refactor, gl_add, cancel64 ? 1 : 0);              \
  }
  if (n <= 8) QMC_LD(8)
  else if (n <= 16) QMC_LD(16)
  else if (n <= 32) QMC_LD(32)
  else if (n <= 64) QMC_LD(64)
  else return cudaErrorInvalidValue;
#undef QMC_LD
  return cudaGetLastError();
}

// =====================================================================
// determinant backward: dlog|psi| / dA_k = w_k A_k^{-T}, w_k = D_k / psi
// (the cotangent of slogdet + signed log-sum-exp,
//  src/jaqmc/wavefunction/output/logdet.py:53-80)
// =====================================================================
template <typename S>
__device__ void det_inverse(const float* __restrict__ Ak, int n, char* scratch, double* ld, float* sg, int* sing,
                            double* growth) {
  const int lane = threadIdx.x & 31;
  const DetScratch sc(n);
  S* LU = reinterpret_cast<S*>(scratch);
  S* Ainv = LU + n * sc.ld;
  int* perm = reinterpret_cast<int*>(scratch + (size_t)(2 * n * sc.ld + 2 * n * sc.ldm) * 8);
  for (int e = lane; e < n * n; e += 32) LU[(e / n) * sc.ld + (e % n)] = (S)Ak[e];
  __syncwarp();
  warp_lu<S>(LU, n, sc.ld, perm, ld, sg, growth, sing);
  if (!*sing) warp_inverse<S>(LU, Ainv, perm, n, sc.ld);
}

__global__ void k_logdet_bwd(int n, int K, const float* __restrict__ A, float* __restrict__ Abar,
                             float* __restrict__ logpsi) {
  extern __shared__ double shb[];
  const int w = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  double* lds = shb;                                   // [K]
  float* sgs = reinterpret_cast<float*>(lds + K);      // [K]
  int* dbl = reinterpret_cast<int*>(sgs + K);          // [K] factorise in FP64
  float* wk = reinterpret_cast<float*>(dbl + K);       // [K]
  const DetScratch sc(n);
  char* scratch = reinterpret_cast<char*>(shb) + align_up((size_t)K * 20 + 16, 16) + sc.bytes * warp;
  const size_t ts = (size_t)n * n;
  for (int k = warp; k < K; k += nw) {
    const float* Ak = A + ((size_t)w * K + k) * ts;
    double ld, growth;
    float sg;
    int sing;
    det_inverse<float>(Ak, n, scratch, &ld, &sg, &sing, &growth);
    int use64 = !sing && !(growth <= (double)kRefactorGrowth);
    if (use64) det_inverse<double>(Ak, n, scratch, &ld, &sg, &sing, &growth);
    if (lane == 0) {
      lds[k] = ld;
      sgs[k] = sing ? 0.f : sg;
      dbl[k] = use64;
    }
    __syncwarp();
  }
  __syncthreads();
  if (warp == 0) {
    double lmax = -INFINITY;
    for (int k = lane; k < K; k += 32)
      if (sgs[k] != 0.f) lmax = fmax(lmax, lds[k]);
    for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    double S = 0.0;
    for (int k = lane; k < K; k += 32)
      if (sgs[k] != 0.f) S += (double)sgs[k] * exp(lds[k] - lmax);
    S = warp_sum(S);
    for (int k = lane; k < K; k += 32) wk[k] = sgs[k] != 0.f ? (float)((double)sgs[k] * exp(lds[k] - lmax) / S) : 0.f;
    if (lane == 0 && logpsi) logpsi[w] = (float)(log(fabs(S)) + lmax);
  }
  __syncthreads();
  // second pass: A_k^{-1} again (the scratch holds one determinant per warp)
  for (int k = warp; k < K; k += nw) {
    const float* Ak = A + ((size_t)w * K + k) * ts;
    float* Bk = Abar + ((size_t)w * K + k) * ts;
    if (sgs[k] == 0.f) {
      for (int e = lane; e < n * n; e += 32) Bk[e] = 0.f;
      continue;
    }
    double ld, growth;
    float sg;
    int sing;
    if (dbl[k]) {
      det_inverse<double>(Ak, n, scratch, &ld, &sg, &sing, &growth);
      const double* Ainv = reinterpret_cast<const double*>(scratch) + n * sc.ld;
      for (int e = lane; e < n * n; e += 32) Bk[e] = (float)((double)wk[k] * Ainv[(e % n) * sc.ld + e / n]);
    } else {
      det_inverse<float>(Ak, n, scratch, &ld, &sg, &sing, &growth);
      const float* Ainv = reinterpret_cast<const float*>(scratch) + n * sc.ld;
      for (int e = lane; e < n * n; e += 32) Bk[e] = wk[k] * Ainv[(e % n) * sc.ld + e / n];
    }
    __syncwarp();
  }
}

cudaError_t launch_logdet_bwd(cudaStream_t s, int B, int n, int K, const float* A, float* Abar, float* logpsi) {
  const DetScratch sc(n);
  const size_t head = align_up((size_t)K * 20 + 16, 16);
  int nw = (int)((200 * 1024 - head) / sc.bytes);
  nw = std::max(1, std::min(std::min(nw, 8), K));
  const size_t sm = head + sc.bytes * nw;
  static int attr_dev = -1;
  int dev;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (attr_dev != dev) {
    e = cudaFuncSetAttribute(k_logdet_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 210 * 1024);
    if (e != cudaSuccess) return e;
    attr_dev = dev;
  }
  k_logdet_bwd<<<B, 32 * nw, sm, s>>>(n, K, A, Abar, logpsi);
  return cudaGetLastError();
}

// =====================================================================
// Metropolis-Hastings (src/jaqmc/sampler/mcmc.py:53-54, 96-137)
// =====================================================================
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float* z0, float* z1) {
  float u1 = u01(a), u2 = u01(b);
  float rad = sqrtf(-2.0f * logf(u1));
  float sn, cs;
  sincospif(2.0f * u2, &sn, &cs);
  *z0 = rad * cs;
  *z1 = rad * sn;
}

__device__ __forceinline__ U4 draw_block(uint64_t seed, uint64_t step, int w, int b) {
  U4 c{(uint32_t)b, (uint32_t)w, (uint32_t)step, (uint32_t)(step >> 32)};
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// Grouped MH (several jobs of one model in one batch): walker w belongs to the
// job j with offsets[j] <= w < offsets[j + 1] and draws from that job's seed,
// counter and its index within the job -- the draws of the job run alone.
__device__ __forceinline__ int mh_stream(const MhGroup& g, int w, uint64_t* seed, uint64_t* step) {
  if (g.n_jobs <= 0) return w;
  int lo = 0, hi = g.n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.offsets[mid] <= w) lo = mid;
    else hi = mid - 1;
  }
  *seed = g.seeds[lo];
  *step += g.counters[lo];
  return w - g.offsets[lo];
}

__global__ void k_mh_propose(int B, int n, const float* __restrict__ x, float* __restrict__ xp,
                             float stddev, uint64_t seed, uint64_t step,
                             const uint64_t* __restrict__ ctr_dev, const float* __restrict__ inj, MhGroup grp) {
  const int nb = normal_blocks(n);
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)B * nb) return;
  if (ctr_dev) step += *ctr_dev;
  int w = (int)(e / nb), b = (int)(e % nb);
  float z[4];
  if (inj) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int c = 4 * b + q;
      z[q] = c < 3 * n ? inj[(size_t)w * 3 * n + c] : 0.f;
    }
  } else {
    const int wl = mh_stream(grp, w, &seed, &step);
    U4 r = draw_block(seed, step, wl, b);
    box_muller(r.x, r.y, &z[0], &z[1]);
    box_muller(r.z, r.w, &z[2], &z[3]);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int c = 4 * b + q;
    if (c < 3 * n) {
      size_t o = (size_t)w * 3 * n + c;
      xp[o] = x[o] + stddev * z[q];
    }
  }
}

cudaError_t launch_mh_propose(cudaStream_t s, int B, int n, const float* x, float* xp,
                              float stddev, uint64_t seed, uint64_t ctr, const uint64_t* ctr_dev,
                              const float* inj, const MhGroup& grp) {
  size_t total = (size_t)B * normal_blocks(n);
  k_mh_propose<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(B, n, x, xp, stddev, seed, ctr, ctr_dev, inj, grp);
  return cudaGetLastError();
}

__global__ void k_mh_accept(int B, int n, float* __restrict__ x, const float* __restrict__ xp,
                            float* __restrict__ lp, const float* __restrict__ logpsi_p,
                            uint64_t seed, uint64_t step, const uint64_t* __restrict__ ctr_dev,
                            const float* __restrict__ inj, uint32_t* __restrict__ accepts, MhGroup grp) {
  int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  if (ctr_dev) step += *ctr_dev;
  float u;
  if (inj) {
    u = inj[w];
  } else {
    const int wl = mh_stream(grp, w, &seed, &step);
    u = u01(draw_block(seed, step, wl, normal_blocks(n)).x);
  }
  float lp2 = 2.0f * logpsi_p[w];
  float ratio = lp2 - lp[w];
  bool cond = ratio > logf(u);
  if (cond) {
    for (int c = 0; c < 3 * n; ++c) x[(size_t)w * 3 * n + c] = xp[(size_t)w * 3 * n + c];
    lp[w] = lp2;
    if (accepts) accepts[w] += 1u;
  }
}

cudaError_t launch_mh_accept(cudaStream_t s, int B, int n, float* x, const float* xp, float* lp,
                             const float* logpsi_p, uint64_t seed, uint64_t ctr, const uint64_t* ctr_dev,
                             const float* inj_uniforms, uint32_t* accepts, const MhGroup& grp) {
  k_mh_accept<<<(B + 127) / 128, 128, 0, s>>>(B, n, x, xp, lp, logpsi_p, seed, ctr, ctr_dev, inj_uniforms,
                                              accepts, grp);
  return cudaGetLastError();
}

__global__ void k_counter_add(int count, uint64_t* ctr, uint64_t inc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) ctr[i] += inc;
}

cudaError_t launch_counter_add(cudaStream_t s, uint64_t* ctr, uint64_t inc, int count) {
  k_counter_add<<<(count + 255) / 256, 256, 0, s>>>(count, ctr, inc);
  return cudaGetLastError();
}

__global__ void k_mh_draws(int B, int n, int steps, uint64_t seed, uint64_t ctr,
                           float* __restrict__ normals, float* __restrict__ uniforms) {
  const int nb = normal_blocks(n);
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)steps * B * (nb + 1)) return;
  int b = (int)(e % (nb + 1));
  size_t sw = e / (nb + 1);
  int w = (int)(sw % B), st = (int)(sw / B);
  U4 r = draw_block(seed, ctr + st, w, b);
  if (b == nb) {
    if (uniforms) uniforms[(size_t)st * B + w] = u01(r.x);
    return;
  }
  if (!normals) return;
  float z[4];
  box_muller(r.x, r.y, &z[0], &z[1]);
  box_muller(r.z, r.w, &z[2], &z[3]);
  for (int q = 0; q < 4; ++q) {
    int c = 4 * b + q;
    if (c < 3 * n) normals[((size_t)st * B + w) * 3 * n + c] = z[q];
  }
}

cudaError_t launch_mh_draws(cudaStream_t s, int B, int n, int steps, uint64_t seed, uint64_t ctr,
                            float* normals, float* uniforms) {
  size_t total = (size_t)steps * B * (normal_blocks(n) + 1);
  k_mh_draws<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(B, n, steps, seed, ctr, normals, uniforms);
  return cudaGetLastError();
}

__global__ void k_scale(int B, const float* __restrict__ in, float c, float* __restrict__ out) {
  int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < B) out[w] = c * in[w];
}
cudaError_t launch_scale(cudaStream_t s, int B, const float* in, float c, float* out) {
  k_scale<<<(B + 255) / 256, 256, 0, s>>>(B, in, c, out);
  return cudaGetLastError();
}

// =====================================================================
// FP64 batch mean / variance (src/jaqmc/estimator/base.py:27-53)
// =====================================================================
// FP64 mean and variance of x[0, B) (offsets null), or one block per segment
// [offsets[s], offsets[s + 1]) into out[2 s], out[2 s + 1] in the same order
// of summation, so a segment's result equals the call on that segment alone.
__global__ void k_reduce_mean_var(int B, const float* __restrict__ x, double* __restrict__ out,
                                  const int* __restrict__ offsets) {
  __shared__ double s1[32], s2[32];
  __shared__ int sc[32];
  if (offsets) {
    const int o0 = offsets[blockIdx.x];
    B = offsets[blockIdx.x + 1] - o0;
    x += o0;
    out += 2 * blockIdx.x;
  }
  double a = 0.0, b = 0.0;
  int c = 0;
  for (int i = threadIdx.x; i < B; i += blockDim.x) {
    float v = x[i];
    if (!isnan(v)) { a += v; b += (double)v * v; ++c; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  int wp = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) { s1[wp] = a; s2[wp] = b; sc[wp] = c; }
  __syncthreads();
  if (wp == 0) {
    int nw = blockDim.x >> 5;
    a = ln < nw ? s1[ln] : 0.0;
    b = ln < nw ? s2[ln] : 0.0;
    c = ln < nw ? sc[ln] : 0;
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (ln == 0) {
      double m = c ? a / c : NAN;
      out[0] = m;
      out[1] = c ? b / c - m * m : NAN;
    }
  }
}

cudaError_t launch_reduce_mean_var(cudaStream_t s, int B, const float* x, double* out, const int* offsets,
                                   int segments) {
  k_reduce_mean_var<<<offsets ? segments : 1, 1024, 0, s>>>(B, x, out, offsets);
  return cudaGetLastError();
}

// =====================================================================
// parameter preparation
// =====================================================================
__global__ void k_transpose_f32(const float* __restrict__ in, int rows, int cols, int ld_in,
                                float* __restrict__ out) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)rows * cols) return;
  int r = (int)(e % rows), c = (int)(e / rows);  // out[c][r]
  out[e] = in[(size_t)r * ld_in + c];
}

cudaError_t launch_transpose_f32(cudaStream_t s, const float* in, int rows, int cols, int ld_in, float* out) {
  size_t total = (size_t)rows * cols;
  k_transpose_f32<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(in, rows, cols, ld_in, out);
  return cudaGetLastError();
}

__global__ void k_transpose_split(const float* __restrict__ in, int rows, int cols, int ld_in,
                                  __nv_bfloat16* __restrict__ out, int rows_p, int cols_p) {
  size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t plane = (size_t)rows_p * cols_p;
  if (e >= plane) return;
  int r = (int)(e % rows_p), c = (int)(e / rows_p);  // out[c][r]
  float v = (r < rows && c < cols) ? in[(size_t)r * ld_in + c] : 0.f;
  __nv_bfloat16 hi = __float2bfloat16_rn(v);
  out[e] = hi;
  out[e + plane] = __float2bfloat16_rn(v - __bfloat162float(hi));
}

cudaError_t launch_transpose_split(cudaStream_t s, const float* in, int rows, int cols, int ld_in,
                                   __nv_bfloat16* out, int rows_p, int cols_p) {
  size_t total = (size_t)rows_p * cols_p;
  k_transpose_split<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(in, rows, cols, ld_in, out, rows_p,
                                                                   cols_p);
  return cudaGetLastError();
}

}  // namespace qmc
