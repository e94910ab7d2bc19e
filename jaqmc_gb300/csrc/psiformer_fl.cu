// Psiformer forward Laplacian: the value, the Laplacian and the Jacobian over
// the 3n electron coordinates carried through every layer of the network, in
// the tangent-row layout of the FermiNet passes: row (w, i, t) of an
// activation holds, for electron i of walker w, t = 0 the value, t = 1 the
// Laplacian and t = 2 + 3e + c the derivative along coordinate c of electron e
// (rows T..Tp-1 are zero padding).  The rules are those of the reference's
// forward-Laplacian interpreter: linear maps act row by row, elementwise
// functions use L f(u) = f'(u) L u + f''(u) sum_d (J_d u)^2, and bilinear maps
// (attention scores and mixing) the product rule
// L(ab) = L a b + a L b + 2 sum_d J_d a J_d b
// (src/jaqmc/laplacian/primitives/elementwise.py:42-72,
//  src/jaqmc/laplacian/primitives/dot_general.py:713+,
//  src/jaqmc/laplacian/primitives/arithmetic.py:385).
//
//   k_psi_features_fl   log-rescaled ae features with tangents, envelope
//                       inputs, Coulomb potential, SimpleEE Jastrow with its
//                       gradient and Laplacian
//   k_psi_group_fl      one electron's tangent group: bias, tanh, residual and
//                       LayerNorm with their tangent rules
//   k_psi_attention_fl  one (walker, head): scores, softmax and mixing with
//                       their tangent rules, directions streamed one by one
#include <cmath>
#include <type_traits>

#include "act.cuh"
#include "psiformer.cuh"

namespace qmc {

namespace {

__device__ __forceinline__ float wsum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double wsum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over a block of blockDim.x (a multiple of 32, at most 1024) threads;
// every thread gets the total.  `red` holds 32 values of T.
template <typename T>
__device__ T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = wsum(v);
  __syncthreads();  // red may still be read by a previous call
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T t = 0;
  for (int k = 0; k < nw; ++k) t += red[k];
  return t;
}

__device__ __forceinline__ float dot4(float4 a, float4 b) {
  return fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, a.w * b.w)));
}

}  // namespace

// ------------------------------------------------------------------ features
// One block per walker.  Per (electron i, atom I), d = r_i - R_I, r = |d|:
//   value     l = log(1+r),  d_a g with g = l / r
//                                 (src/jaqmc/wavefunction/input/atomic.py:58-66)
//   d/dx_c    l: d_c / (r (1+r));  d_a g: delta_ac g + d_a d_c g'(r) / r
//   Laplacian l: l'' + 2 l'/r;     d_a g: d_a (g'' + 4 g'/r)
// with l' = 1/(1+r), l'' = -1/(1+r)^2, g' = l'/r - l/r^2,
// g'' + 4 g'/r = (l'' + 2 l'/r - 2 l/r^2) / r.  Only the three Jacobian rows of
// electron i's own coordinates are nonzero; the spin feature is constant.
// pe[w] = sum_{i<j} 1/r_ij - sum_{i,I} Z_I / r_iI + nuc in FP64
// (src/jaqmc/app/molecule/hamiltonian.py:9-22).  SimpleEE Jastrow
// J = sum_{i<j} f(r_ij), f = -c a^2 / (a + r) (src/jaqmc/wavefunction/jastrow.py:48-122):
// jgl[w] = [grad_{r_i} J for all i (3n), Laplacian 2 sum_{i<j} (f'' + 2 f'/r)].
constexpr int kAeStride = 9;  // dx dy dz l g a0 b0 lapl lapv

__global__ void __launch_bounds__(256) k_psi_features_fl(int n, int n_up, int A, int Tp, int T, int K0p,
                                                         const float* __restrict__ x,
                                                         const float* __restrict__ atoms,
                                                         const float* __restrict__ charges, double nuc,
                                                         const float* __restrict__ alpha, float* __restrict__ X0,
                                                         float* __restrict__ rae, float* __restrict__ aevec,
                                                         float* __restrict__ pe, float* __restrict__ jas,
                                                         float* __restrict__ jgl) {
  __shared__ double redd[32];
  __shared__ float redf[32];
  extern __shared__ float sf[];
  float* xs = sf;          // [n][3]
  float* ae = xs + 3 * n;  // [n][A][kAeStride]
  const int w = blockIdx.x;
  for (int e = threadIdx.x; e < 3 * n; e += blockDim.x) xs[e] = x[(size_t)w * 3 * n + e];
  __syncthreads();
  double vpot = 0.0;
  for (int e = threadIdx.x; e < n * A; e += blockDim.x) {
    const int i = e / A, I = e % A;
    const float dx = xs[3 * i] - atoms[3 * I], dy = xs[3 * i + 1] - atoms[3 * I + 1],
                dz = xs[3 * i + 2] - atoms[3 * I + 2];
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    const float l = log1pf(r), ip = 1.f / (1.f + r), ir = 1.f / r;
    const float g = l * ir;
    float* P = ae + (size_t)e * kAeStride;
    P[0] = dx;
    P[1] = dy;
    P[2] = dz;
    P[3] = l;
    P[4] = g;
    P[5] = ip * ir;                                 // l'/r
    P[6] = (ip - g) * ir * ir;                      // g'/r
    P[7] = -ip * ip + 2.f * ip * ir;                // l'' + 2 l'/r
    P[8] = (-ip * ip + 2.f * ip * ir - 2.f * g * ir) * ir;  // g'' + 4 g'/r
    const size_t o = (size_t)w * n * A + e;
    rae[o] = r;
    aevec[3 * o] = dx;
    aevec[3 * o + 1] = dy;
    aevec[3 * o + 2] = dz;
    vpot -= (double)charges[I] / (double)r;
  }
  __syncthreads();
  const int per = Tp * K0p;
  for (int e = threadIdx.x; e < n * per; e += blockDim.x) {
    const int i = e / per, rem = e % per, t = rem / K0p, c = rem % K0p;
    float v = 0.f;
    if (c < 4 * A) {
      const int I = c >> 2, q = c & 3;
      const float* P = ae + (size_t)(i * A + I) * kAeStride;
      if (t == 0) {
        v = q == 0 ? P[3] : P[q - 1] * P[4];
      } else if (t == 1) {
        v = q == 0 ? P[7] : P[q - 1] * P[8];
      } else if (t < T) {
        const int dir = t - 2, ee = dir / 3, comp = dir % 3;
        if (ee == i) v = q == 0 ? P[comp] * P[5] : (q - 1 == comp ? P[4] : 0.f) + P[q - 1] * P[comp] * P[6];
      }
    } else if (c == 4 * A && t == 0) {
      v = i < n_up ? 1.f : -1.f;
    }
    X0[(size_t)w * n * per + e] = v;
  }
  const float ap = alpha ? alpha[0] : 1.f, aa = alpha ? alpha[1] : 1.f;
  float jv = 0.f, jl = 0.f;
  for (int p = threadIdx.x; p < n * n; p += blockDim.x) {
    const int i = p / n, j = p % n;
    if (j <= i) continue;
    const float dx = xs[3 * i] - xs[3 * j], dy = xs[3 * i + 1] - xs[3 * j + 1], dz = xs[3 * i + 2] - xs[3 * j + 2];
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    vpot += 1.0 / (double)r;
    if (alpha) {
      const bool same = (i < n_up) == (j < n_up);
      const float a = same ? ap : aa, cf = same ? 0.25f : 0.5f;
      const float ia = 1.f / (a + r), ca2 = cf * a * a;
      jv -= ca2 * ia;                                           // f
      jl += 2.f * (-2.f * ca2 * ia * ia * ia + 2.f * ca2 * ia * ia / r);  // 2 (f'' + 2 f'/r)
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    float g[3] = {0.f, 0.f, 0.f};
    if (alpha)
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        const float dx = xs[3 * i] - xs[3 * j], dy = xs[3 * i + 1] - xs[3 * j + 1],
                    dz = xs[3 * i + 2] - xs[3 * j + 2];
        const float r = sqrtf(dx * dx + dy * dy + dz * dz);
        const bool same = (i < n_up) == (j < n_up);
        const float a = same ? ap : aa, cf = same ? 0.25f : 0.5f;
        const float ia = 1.f / (a + r);
        const float s = cf * a * a * ia * ia / r;  // f'(r) / r
        g[0] = fmaf(s, dx, g[0]);
        g[1] = fmaf(s, dy, g[1]);
        g[2] = fmaf(s, dz, g[2]);
      }
    float* o = jgl + (size_t)w * (3 * n + 1) + 3 * i;
    o[0] = g[0];
    o[1] = g[1];
    o[2] = g[2];
  }
  const double v = block_sum(vpot, redd);
  const float J = block_sum(jv, redf);
  const float JL = block_sum(jl, redf);
  if (threadIdx.x == 0) {
    pe[w] = (float)(v + nuc);
    jas[w] = J;
    jgl[(size_t)w * (3 * n + 1) + 3 * n] = JL;
  }
}

cudaError_t launch_psi_features_fl(cudaStream_t s, int B, int n, int n_up, int A, int Tp, int T, int K0p,
                                   const float* x, const float* atoms, const float* charges, double nuc,
                                   const float* alpha, float* X0, float* rae, float* aevec, float* pe,
                                   float* jas, float* jgl) {
  const size_t sm = sizeof(float) * (3 * n + (size_t)n * A * kAeStride);
  if (sm > 48 * 1024) return cudaErrorInvalidValue;
  k_psi_features_fl<<<B, 256, sm, s>>>(n, n_up, A, Tp, T, K0p, x, atoms, charges, nuc, alpha, X0, rae, aevec, pe,
                                       jas, jgl);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ group pass
// One block (8 warps) per tangent group (w, i) of Tp rows x D features:
//   h = z + bias (bias on the value row only); with `act`, h = tanh with
//     J h = h' J z, L h = h' L z + h'' sum_d (J_d z)^2, h' = 1 - h^2, h'' = -2 h h';
//   xmode 0: v = h;  1: x = v = h;  2: x = v = x + h;
//   out = LayerNorm(v) (eps 1e-5, src/jaqmc/wavefunction/backbone/psiformer.py:61-99)
//   when ln_s is set, else v.
// LayerNorm with u = v - mu, var = mean(u^2), r = (var + eps)^-1/2, y = s u r + b:
//   J_d mu = mean(J_d v),  J_d var = 2 mean(u J_d v),  J_d r = -r^3 mean(u J_d v)
//   L mu = mean(L v),  L var = 2 mean(u L v) + 2 (mean(sum_d (J_d v)^2) - sum_d (J_d mu)^2)
//   L r = -r^3/2 L var + 3/4 r^5 sum_d (J_d var)^2
//   J_d y = s (J_d u r + u J_d r),  L y = s (L u r + u L r + 2 sum_d J_d u J_d r),
// the last sum written sum_d J_d v J_d r - sum_d J_d mu J_d r.
constexpr int kGrpMaxD = 512;
constexpr int kGrpMaxTp = 256;
constexpr int kGrpWarps = 8;

__device__ __forceinline__ void put4(const StF32& o, size_t r, int c, float4 v) {
  *reinterpret_cast<float4*>(o.p + r * o.ld + c) = v;
}
__device__ __forceinline__ void put4(const StSplit& o, size_t r, int c, float4 v) {
  const __nv_bfloat162 h0 = __floats2bfloat162_rn(v.x, v.y), h1 = __floats2bfloat162_rn(v.z, v.w);
  const float2 f0 = __bfloat1622float2(h0), f1 = __bfloat1622float2(h1);
  const __nv_bfloat162 l0 = __floats2bfloat162_rn(v.x - f0.x, v.y - f0.y),
                       l1 = __floats2bfloat162_rn(v.z - f1.x, v.w - f1.y);
  const size_t i = r * o.ld + c;
  uint2 hi, lo;
  hi.x = *reinterpret_cast<const uint32_t*>(&h0);
  hi.y = *reinterpret_cast<const uint32_t*>(&h1);
  lo.x = *reinterpret_cast<const uint32_t*>(&l0);
  lo.y = *reinterpret_cast<const uint32_t*>(&l1);
  *reinterpret_cast<uint2*>(o.p + i) = hi;
  *reinterpret_cast<uint2*>(o.p + i + o.plane) = lo;
}

// The pass reads each z row once: the value row first (h, h'), then the
// Jacobian rows t >= 2 (J h = h' J z, accumulating sum_d (J_d z)^2 per
// feature), then the Laplacian row, which needs that sum.  A warp takes
// whole rows, a lane four consecutive features per 128 (16-byte accesses).
//
// Input layer (in.x0 set): z = x0 W_in is formed here instead of read.  An
// electron's input features depend on its own position only, so of its
// tangent rows only the value row, the Laplacian row and its own three
// Jacobian rows t = 2 + 3i + c are nonzero; the others have z = 0 exactly.
struct PsiInput {
  const float* x0;  // [group * Tp + t][k0p] input features with tangents (null: read z)
  const float* w;   // [k0][D] input Dense kernel
  int k0, k0p, n;   // features, their row stride, electrons per walker
};

__device__ __forceinline__ float xw_dot(const float* __restrict__ xr, const float* __restrict__ W, int k0, int D,
                                        int c) {
  float acc = 0.f;
  for (int k = 0; k < k0; ++k) acc = fmaf(__ldg(xr + k), __ldg(W + (size_t)k * D + c), acc);
  return acc;
}
__device__ __forceinline__ float4 xw_dot4(const float* __restrict__ xr, const float* __restrict__ W, int k0, int D,
                                          int c) {
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int k = 0; k < k0; ++k) {
    const float xv = __ldg(xr + k);
    const float4 w = __ldg(reinterpret_cast<const float4*>(W + (size_t)k * D + c));
    acc.x = fmaf(xv, w.x, acc.x);
    acc.y = fmaf(xv, w.y, acc.y);
    acc.z = fmaf(xv, w.z, acc.z);
    acc.w = fmaf(xv, w.w, acc.w);
  }
  return acc;
}

template <class Out>
__global__ void __launch_bounds__(kGrpWarps * 32) k_psi_group_fl(int Tp, int D, const float* __restrict__ z,
                                                                  int ldz, const float* __restrict__ bias, int act,
                                                                  float* __restrict__ x, int xmode,
                                                                  const float* __restrict__ ln_s,
                                                                  const float* __restrict__ ln_b, Out out,
                                                                  PsiInput in) {
  constexpr int kV = kGrpMaxD / 128;
  __shared__ __align__(16) float colacc[kGrpWarps][kGrpMaxD];
  __shared__ __align__(16) float hv[2][kGrpMaxD];  // h, h' of the value row
  __shared__ __align__(16) float v0[kGrpMaxD];
  __shared__ float S1[kGrpMaxTp], S2[kGrpMaxTp];
  __shared__ float redf[32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t r0 = (size_t)blockIdx.x * Tp;
  const float invD = 1.f / (float)D;
  const int t_own = in.x0 ? 2 + 3 * (int)(blockIdx.x % (unsigned)in.n) : 0;  // first nonzero Jacobian row
  // value row
  float s = 0.f;
  for (int c = threadIdx.x; c < D; c += blockDim.x) {
    float v = (in.x0 ? xw_dot(in.x0 + r0 * in.k0p, in.w, in.k0, D, c) : z[r0 * ldz + c]) + bias[c];
    if (act) {
      v = tanhf(v);
      hv[0][c] = v;
      hv[1][c] = 1.f - v * v;
    }
    if (xmode == 2) v += x[r0 * D + c];
    if (xmode) x[r0 * D + c] = v;
    v0[c] = v;
    s += v;
  }
  float mu0 = 0.f, var = 0.f;
  if (ln_s) {
    mu0 = block_sum(s, redf) * invD;
    float q = 0.f;
    for (int c = threadIdx.x; c < D; c += blockDim.x) q += (v0[c] - mu0) * (v0[c] - mu0);
    var = block_sum(q, redf) * invD;
  } else {
    __syncthreads();
  }
  // Jacobian rows
  float4 qa[kV];
#pragma unroll
  for (int k = 0; k < kV; ++k) qa[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  float Qs = 0.f;
  for (int t = 2 + warp; t < Tp; t += kGrpWarps) {
    const float* zr = z + (r0 + t) * ldz;
    float* xr = x + (r0 + t) * D;
    float s1 = 0.f, s2 = 0.f;
    const bool live = !in.x0 || (unsigned)(t - t_own) < 3u;
#pragma unroll
    for (int k = 0; k < kV; ++k) {
      const int c = 4 * lane + 128 * k;
      if (c < D) {
        const float4 zz = !in.x0 ? *reinterpret_cast<const float4*>(zr + c)
                                 : (live ? xw_dot4(in.x0 + (r0 + t) * in.k0p, in.w, in.k0, D, c)
                                         : make_float4(0.f, 0.f, 0.f, 0.f));
        float4 v = zz;
        if (act) {
          const float4 h1 = *reinterpret_cast<const float4*>(&hv[1][c]);
          v = make_float4(h1.x * zz.x, h1.y * zz.y, h1.z * zz.z, h1.w * zz.w);
          qa[k].x = fmaf(zz.x, zz.x, qa[k].x);
          qa[k].y = fmaf(zz.y, zz.y, qa[k].y);
          qa[k].z = fmaf(zz.z, zz.z, qa[k].z);
          qa[k].w = fmaf(zz.w, zz.w, qa[k].w);
        }
        if (xmode == 2) {
          const float4 xx = *reinterpret_cast<const float4*>(xr + c);
          v = make_float4(v.x + xx.x, v.y + xx.y, v.z + xx.z, v.w + xx.w);
        }
        if (xmode) *reinterpret_cast<float4*>(xr + c) = v;
        if (!ln_s) {
          put4(out, r0 + t, c, v);
        } else {
          const float4 u = *reinterpret_cast<const float4*>(&v0[c]);
          s1 += (v.x + v.y) + (v.z + v.w);
          s2 = fmaf(u.x - mu0, v.x, fmaf(u.y - mu0, v.y, fmaf(u.z - mu0, v.z, fmaf(u.w - mu0, v.w, s2))));
          Qs = fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, fmaf(v.w, v.w, Qs))));
        }
      }
    }
    if (ln_s) {
      s1 = wsum(s1);
      s2 = wsum(s2);
      if (lane == 0) {
        S1[t] = s1;
        S2[t] = s2;
      }
    }
  }
  // Laplacian row: L h = h' L z + h'' sum_d (J_d z)^2, h'' = -2 h h'
  if (act) {
#pragma unroll
    for (int k = 0; k < kV; ++k) {
      const int c = 4 * lane + 128 * k;
      if (c < D) *reinterpret_cast<float4*>(&colacc[warp][c]) = qa[k];
    }
  }
  __syncthreads();
  float s1 = 0.f, s2 = 0.f;
  for (int c = threadIdx.x; c < D; c += blockDim.x) {
    float v = in.x0 ? xw_dot(in.x0 + (r0 + 1) * in.k0p, in.w, in.k0, D, c) : z[(r0 + 1) * ldz + c];
    if (act) {
      float q = 0.f;
#pragma unroll
      for (int wv = 0; wv < kGrpWarps; ++wv) q += colacc[wv][c];
      const float h = hv[0][c], h1 = hv[1][c];
      v = fmaf(h1, v, -2.f * h * h1 * q);
    }
    if (xmode == 2) v += x[(r0 + 1) * D + c];
    if (xmode) x[(r0 + 1) * D + c] = v;
    if (!ln_s) {
      out.put(r0 + 1, c, v);
      out.put(r0, c, v0[c]);
    } else {
      s1 += v;
      s2 = fmaf(v0[c] - mu0, v, s2);
    }
  }
  if (!ln_s) return;
  s1 = block_sum(s1, redf);
  s2 = block_sum(s2, redf);
  if (threadIdx.x == 0) {
    S1[1] = s1;
    S2[1] = s2;
  }
  const float Q = block_sum(Qs, redf);  // also publishes S1 / S2
  const float r = rsqrtf(var + 1e-5f);
  const float r3 = r * r * r;
  float a1 = 0.f, a2 = 0.f, a3 = 0.f;  // sum_d (J mu)^2, (J var)^2, J mu J r
  for (int t = 2 + threadIdx.x; t < Tp; t += blockDim.x) {
    const float dmu = S1[t] * invD, dv = 2.f * S2[t] * invD, dr = -0.5f * r3 * dv;
    a1 = fmaf(dmu, dmu, a1);
    a2 = fmaf(dv, dv, a2);
    a3 = fmaf(dmu, dr, a3);
  }
  const float Sdmu2 = block_sum(a1, redf);
  const float Sdv2 = block_sum(a2, redf);
  const float Smd = block_sum(a3, redf);
  const float Lmu = S1[1] * invD;
  const float Lv = 2.f * S2[1] * invD + 2.f * (Q * invD - Sdmu2);
  const float Lr = -0.5f * r3 * Lv + 0.75f * r3 * r * r * Sdv2;
  float4 cacc[kV];
#pragma unroll
  for (int k = 0; k < kV; ++k) cacc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int t = 2 + warp; t < Tp; t += kGrpWarps) {
    const float dmu = S1[t] * invD, dr = -r3 * S2[t] * invD;
    const float* xr = x + (r0 + t) * D;
#pragma unroll
    for (int k = 0; k < kV; ++k) {
      const int c = 4 * lane + 128 * k;
      if (c < D) {
        const float4 J = *reinterpret_cast<const float4*>(xr + c);
        const float4 u = *reinterpret_cast<const float4*>(&v0[c]);
        const float4 sc = *reinterpret_cast<const float4*>(ln_s + c);
        const float4 y = make_float4(sc.x * fmaf(J.x - dmu, r, (u.x - mu0) * dr),
                                     sc.y * fmaf(J.y - dmu, r, (u.y - mu0) * dr),
                                     sc.z * fmaf(J.z - dmu, r, (u.z - mu0) * dr),
                                     sc.w * fmaf(J.w - dmu, r, (u.w - mu0) * dr));
        put4(out, r0 + t, c, y);
        cacc[k].x = fmaf(J.x, dr, cacc[k].x);
        cacc[k].y = fmaf(J.y, dr, cacc[k].y);
        cacc[k].z = fmaf(J.z, dr, cacc[k].z);
        cacc[k].w = fmaf(J.w, dr, cacc[k].w);
      }
    }
  }
  __syncthreads();  // every warp is done with colacc's sums of squares
#pragma unroll
  for (int k = 0; k < kV; ++k) {
    const int c = 4 * lane + 128 * k;
    if (c < D) *reinterpret_cast<float4*>(&colacc[warp][c]) = cacc[k];
  }
  __syncthreads();
  for (int c = threadIdx.x; c < D; c += blockDim.x) {
    float C = -Smd;
#pragma unroll
    for (int wv = 0; wv < kGrpWarps; ++wv) C += colacc[wv][c];
    const float u = v0[c] - mu0;
    out.put(r0, c, fmaf(ln_s[c] * u, r, ln_b[c]));
    const float x1 = x[(r0 + 1) * D + c];
    out.put(r0 + 1, c, ln_s[c] * ((x1 - Lmu) * r + u * Lr + 2.f * C));
  }
}

template <class Out>
cudaError_t launch_psi_group_fl(cudaStream_t s, int groups, int Tp, int D, const float* z, int ldz,
                                const float* bias, int act, float* x, int xmode, const float* ln_s,
                                const float* ln_b, Out out) {
  if (D % 64 || D > kGrpMaxD || Tp > kGrpMaxTp || Tp < 2 || ldz % 4 || (ln_s && !xmode)) return cudaErrorInvalidValue;
  k_psi_group_fl<Out><<<groups, kGrpWarps * 32, 0, s>>>(Tp, D, z, ldz, bias, act, x, xmode, ln_s, ln_b, out,
                                                        PsiInput{nullptr, nullptr, 0, 0, 1});
  return cudaGetLastError();
}

// ------------------------------------------------------------------ attention
// One block per (walker, head).  With q scaled by 1/sqrt(Dh) (value and
// tangent rows), S = q k^T, a = softmax_j(S), o = a v
// (flax MultiHeadDotProductAttention, src/jaqmc/wavefunction/backbone/psiformer.py:74-81):
//   J_d S = J_d q k0^T + q0 J_d k^T
//   J_d a_ij = a_ij b_ij,  b_ij = J_d S_ij - sum_k a_ik J_d S_ik
//   J_d o = J_d a v0 + a J_d v
//   L S = L q k0^T + q0 L k^T + 2 sum_d J_d q J_d k^T
//   L a_ij = a_ij (sum_d b_ij^2 - sum_k a_ik sum_d b_ik^2 + L S_ij - sum_k a_ik L S_ik)
//   L o = L a v0 + a L v + 2 sum_d J_d a J_d v.
// The directions d stream through shared memory one at a time (the next
// direction's rows are loaded into registers while the current one is
// computed); sum_d J_d q J_d k^T, sum_d b^2 and sum_d J_d a J_d v accumulate
// across them, the last in registers of the thread that owns the output tile.
struct AttnFlShape {
  int n, Dh, n2, np, ld, lds;
  __host__ __device__ AttnFlShape(int n_, int Dh_) : n(n_), Dh(Dh_) {
    n2 = (n + 1) / 2 * 2;
    np = (n + 3) / 4 * 4;
    ld = Dh + 4;
    lds = np + 1;
  }
  // Q0 K0 V0 dQ dK dV [np][ld]; A dS XS Bsq [n2][lds]
  __host__ __device__ size_t floats() const { return (size_t)6 * np * ld + (size_t)4 * n2 * lds; }
};
constexpr int kAttnFlThreads = 256;
constexpr int kAttnFlPf = 4;  // prefetch float4 registers per tensor per thread

// Output-tile rows per thread: the smallest RT in 1..4 whose tiles
// (ceil(n / RT) rows x Dh/4 feature quads) fit one tile per thread.
static int attention_fl_rows(int n, int Dh) {
  for (int rt = 1; rt <= 4; ++rt)
    if ((size_t)((n + rt - 1) / rt) * (Dh / 4) <= kAttnFlThreads) return rt;
  return 0;
}

size_t psi_attention_fl_smem(int n, int Dh) { return sizeof(float) * AttnFlShape(n, Dh).floats(); }

bool psi_attention_fl_supported(int n, int Dh) {
  const AttnFlShape sh(n, Dh);
  return Dh % 4 == 0 && attention_fl_rows(n, Dh) > 0 && (size_t)sh.np * (Dh / 4) <= (size_t)kAttnFlPf * kAttnFlThreads &&
         psi_attention_fl_smem(n, Dh) <= 200 * 1024;
}

template <int RT, class Out>
__global__ void __launch_bounds__(kAttnFlThreads, 2) k_psi_attention_fl(int n, int Tp, int T, int H, int Dh,
                                                                         const float* __restrict__ qkv,
                                                                         const float* __restrict__ bqkv, Out out) {
  extern __shared__ __align__(16) float sa[];
  const AttnFlShape sh(n, Dh);
  const int ld = sh.ld, lds = sh.lds, n2 = sh.n2, np = sh.np;
  float* Q0 = sa;
  float* K0 = Q0 + (size_t)np * ld;
  float* V0 = K0 + (size_t)np * ld;
  float* dQ = V0 + (size_t)np * ld;
  float* dK = dQ + (size_t)np * ld;
  float* dV = dK + (size_t)np * ld;
  float* Am = dV + (size_t)np * ld;
  float* dS = Am + (size_t)n2 * lds;
  float* XS = dS + (size_t)n2 * lds;
  float* Bq = XS + (size_t)n2 * lds;
  const int w = blockIdx.x / H, h = blockIdx.x % H;
  const int D = H * Dh, ld3 = 3 * D;
  const float scale = 1.0f / sqrtf((float)Dh);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int dq4 = Dh / 4, tot = np * dq4;
  const size_t grow = (size_t)w * n * Tp;  // first row of the walker
  auto rowp = [&](int i, int t) { return qkv + (grow + (size_t)i * Tp + t) * ld3 + h * Dh; };
  // value rows with the projection biases
  for (int e = tid; e < tot; e += blockDim.x) {
    const int i = e / dq4, d = 4 * (e % dq4);
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f), k = q, v = q;
    if (i < n) {
      const float* r = rowp(i, 0) + d;
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
    *reinterpret_cast<float4*>(Q0 + i * ld + d) = q;
    *reinterpret_cast<float4*>(K0 + i * ld + d) = k;
    *reinterpret_cast<float4*>(V0 + i * ld + d) = v;
  }
  for (int e = tid; e < n2 * lds; e += blockDim.x) {
    XS[e] = 0.f;
    Bq[e] = 0.f;
  }
  __syncthreads();
  const int hi = n2 / 2, hj = np / 4;
  // value scores and softmax
  for (int tt = tid; tt < hi * hj; tt += blockDim.x) {
    const int ti = tt / hj, tj = tt % hj;
    float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    for (int d = 0; d < Dh; d += 4) {
      const float4 qa = *reinterpret_cast<const float4*>(Q0 + ti * ld + d);
      const float4 qb = *reinterpret_cast<const float4*>(Q0 + (ti + hi) * ld + d);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float4 kk = *reinterpret_cast<const float4*>(K0 + (tj + c * hj) * ld + d);
        acc[0][c] += dot4(qa, kk);
        acc[1][c] += dot4(qb, kk);
      }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      Am[ti * lds + tj + c * hj] = acc[0][c];
      Am[(ti + hi) * lds + tj + c * hj] = acc[1][c];
    }
  }
  __syncthreads();
  for (int i = warp; i < n; i += nw) {
    float mx = -INFINITY;
    for (int j = lane; j < n; j += 32) mx = fmaxf(mx, Am[i * lds + j]);
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    float sum = 0.f;
    for (int j = lane; j < n; j += 32) {
      const float e = expf(Am[i * lds + j] - mx);
      Am[i * lds + j] = e;
      sum += e;
    }
    sum = wsum(sum);
    const float inv = 1.0f / sum;
    for (int j = lane; j < n; j += 32) Am[i * lds + j] *= inv;
  }
  // output tile of this thread: rows ti + a * nR (a < RT), features 4 td .. 4 td + 3
  const int nR = (n + RT - 1) / RT;
  const bool own = tid < nR * dq4;
  const int oti = own ? tid / dq4 : 0, od = own ? 4 * (tid % dq4) : 0;
  float xo[RT][4];
#pragma unroll
  for (int a = 0; a < RT; ++a)
#pragma unroll
    for (int f = 0; f < 4; ++f) xo[a][f] = 0.f;
  float4 pf[3][kAttnFlPf];
  auto prefetch = [&](int t) {
#pragma unroll
    for (int u = 0; u < kAttnFlPf; ++u) {
      const int e = tid + u * kAttnFlThreads;
      const int i = e / dq4, d = 4 * (e % dq4);
      float4 zq = make_float4(0.f, 0.f, 0.f, 0.f), zk = zq, zv = zq;
      if (e < tot && i < n) {
        const float* r = rowp(i, t) + d;
        zq = *reinterpret_cast<const float4*>(r);
        zk = *reinterpret_cast<const float4*>(r + D);
        zv = *reinterpret_cast<const float4*>(r + 2 * D);
      }
      pf[0][u] = make_float4(zq.x * scale, zq.y * scale, zq.z * scale, zq.w * scale);
      pf[1][u] = zk;
      pf[2][u] = zv;
    }
  };
  auto commit = [&]() {
#pragma unroll
    for (int u = 0; u < kAttnFlPf; ++u) {
      const int e = tid + u * kAttnFlThreads;
      if (e < tot) {
        const int i = e / dq4, d = 4 * (e % dq4);
        *reinterpret_cast<float4*>(dQ + i * ld + d) = pf[0][u];
        *reinterpret_cast<float4*>(dK + i * ld + d) = pf[1][u];
        *reinterpret_cast<float4*>(dV + i * ld + d) = pf[2][u];
      }
    }
  };
  // out rows of this thread's tile: sum_j P[i][j] v0[j] + R[i][j] v1[j] (R may
  // be null), and cr = sum_j P[i][j] v1[j] when cr is set
  auto mix = [&](const float* P, const float* R, const float* v1, float (*o)[4], float (*cr)[4]) {
#pragma unroll
    for (int a = 0; a < RT; ++a)
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        o[a][f] = 0.f;
        if (cr) cr[a][f] = 0.f;
      }
    for (int j = 0; j < n; ++j) {
      const float4 va = *reinterpret_cast<const float4*>(V0 + j * ld + od);
      const float4 vb = v1 ? *reinterpret_cast<const float4*>(v1 + j * ld + od) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int a = 0; a < RT; ++a) {
        const int i = oti + a * nR;
        const float p = i < n ? P[i * lds + j] : 0.f, q = (R && i < n) ? R[i * lds + j] : 0.f;
        o[a][0] = fmaf(p, va.x, fmaf(q, vb.x, o[a][0]));
        o[a][1] = fmaf(p, va.y, fmaf(q, vb.y, o[a][1]));
        o[a][2] = fmaf(p, va.z, fmaf(q, vb.z, o[a][2]));
        o[a][3] = fmaf(p, va.w, fmaf(q, vb.w, o[a][3]));
        if (cr) {
          cr[a][0] = fmaf(p, vb.x, cr[a][0]);
          cr[a][1] = fmaf(p, vb.y, cr[a][1]);
          cr[a][2] = fmaf(p, vb.z, cr[a][2]);
          cr[a][3] = fmaf(p, vb.w, cr[a][3]);
        }
      }
    }
  };
  auto put_tile = [&](int t, float (*o)[4]) {
#pragma unroll
    for (int a = 0; a < RT; ++a) {
      const int i = oti + a * nR;
      if (own && i < n)
#pragma unroll
        for (int f = 0; f < 4; ++f) out.put(grow + (size_t)i * Tp + t, h * Dh + od + f, o[a][f]);
    }
  };
  // score tangents of the rows in dQ / dK against the value rows:
  // S' = dQ K0^T + Q0 dK^T into dS, and (cross) XS += dQ dK^T
  auto scores = [&](bool cross) {
    for (int tt = tid; tt < hi * hj; tt += blockDim.x) {
      const int ti = tt / hj, tj = tt % hj;
      float ds[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
      float xs[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
      for (int d = 0; d < Dh; d += 4) {
        const float4 qa = *reinterpret_cast<const float4*>(Q0 + ti * ld + d);
        const float4 qb = *reinterpret_cast<const float4*>(Q0 + (ti + hi) * ld + d);
        const float4 ga = *reinterpret_cast<const float4*>(dQ + ti * ld + d);
        const float4 gb = *reinterpret_cast<const float4*>(dQ + (ti + hi) * ld + d);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int j = tj + c * hj;
          const float4 k0 = *reinterpret_cast<const float4*>(K0 + j * ld + d);
          const float4 gk = *reinterpret_cast<const float4*>(dK + j * ld + d);
          ds[0][c] += dot4(ga, k0) + dot4(qa, gk);
          ds[1][c] += dot4(gb, k0) + dot4(qb, gk);
          if (cross) {
            xs[0][c] += dot4(ga, gk);
            xs[1][c] += dot4(gb, gk);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int j = tj + c * hj;
        dS[ti * lds + j] = ds[0][c];
        dS[(ti + hi) * lds + j] = ds[1][c];
        if (cross) {
          XS[ti * lds + j] += xs[0][c];
          XS[(ti + hi) * lds + j] += xs[1][c];
        }
      }
    }
  };
  float o[RT][4], cr[RT][4];
  if (T > 2) prefetch(2);
  for (int t = 2; t < T; ++t) {
    __syncthreads();  // the previous direction is done with dQ / dK / dV / dS
    commit();
    __syncthreads();
    if (t + 1 < T) prefetch(t + 1);
    scores(true);
    __syncthreads();
    for (int i = warp; i < n; i += nw) {
      float ab = 0.f;
      for (int j = lane; j < n; j += 32) ab = fmaf(Am[i * lds + j], dS[i * lds + j], ab);
      ab = wsum(ab);
      for (int j = lane; j < n; j += 32) {
        const float b = dS[i * lds + j] - ab;
        Bq[i * lds + j] = fmaf(b, b, Bq[i * lds + j]);
        dS[i * lds + j] = Am[i * lds + j] * b;
      }
    }
    __syncthreads();
    if (own) {
      mix(dS, Am, dV, o, cr);
#pragma unroll
      for (int a = 0; a < RT; ++a)
#pragma unroll
        for (int f = 0; f < 4; ++f) xo[a][f] += cr[a][f];
      put_tile(t, o);
    }
  }
  // Laplacian rows
  __syncthreads();
  prefetch(1);
  commit();
  __syncthreads();
  scores(false);
  __syncthreads();
  for (int e = tid; e < n2 * lds; e += blockDim.x) dS[e] += 2.f * XS[e];
  __syncthreads();
  for (int i = warp; i < n; i += nw) {
    float m1 = 0.f, m2 = 0.f;
    for (int j = lane; j < n; j += 32) {
      m1 = fmaf(Am[i * lds + j], Bq[i * lds + j], m1);
      m2 = fmaf(Am[i * lds + j], dS[i * lds + j], m2);
    }
    m1 = wsum(m1);
    m2 = wsum(m2);
    for (int j = lane; j < n; j += 32)
      dS[i * lds + j] = Am[i * lds + j] * (Bq[i * lds + j] - m1 + dS[i * lds + j] - m2);
  }
  __syncthreads();
  if (own) {
    mix(dS, Am, dV, o, nullptr);
#pragma unroll
    for (int a = 0; a < RT; ++a)
#pragma unroll
      for (int f = 0; f < 4; ++f) o[a][f] += 2.f * xo[a][f];
    put_tile(1, o);
    mix(Am, nullptr, nullptr, o, nullptr);
    put_tile(0, o);
  }
  // zero padding rows
  for (int e = tid; e < n * (Tp - T) * Dh; e += blockDim.x) {
    const int i = e / ((Tp - T) * Dh), r = e % ((Tp - T) * Dh);
    out.put(grow + (size_t)i * Tp + T + r / Dh, h * Dh + r % Dh, 0.f);
  }
}

template <class Out>
cudaError_t launch_psi_input_fl(cudaStream_t s, int groups, int n, int Tp, int D, const float* x0, int k0,
                                int k0p, const float* w_in, const float* bias, float* x, const float* ln_s,
                                const float* ln_b, Out out) {
  if (D % 64 || D > kGrpMaxD || Tp > kGrpMaxTp || Tp < 5 || n < 1 || k0 > k0p ||
      ((uintptr_t)w_in & 15) != 0)
    return cudaErrorInvalidValue;
  k_psi_group_fl<Out><<<groups, kGrpWarps * 32, 0, s>>>(Tp, D, nullptr, 0, bias, 0, x, 1, ln_s, ln_b, out,
                                                        PsiInput{x0, w_in, k0, k0p, n});
  return cudaGetLastError();
}
template cudaError_t launch_psi_input_fl<StF32>(cudaStream_t, int, int, int, int, const float*, int, int,
                                                const float*, const float*, float*, const float*, const float*,
                                                StF32);
template cudaError_t launch_psi_input_fl<StSplit>(cudaStream_t, int, int, int, int, const float*, int, int,
                                                  const float*, const float*, float*, const float*, const float*,
                                                  StSplit);

template <class Out>
cudaError_t launch_psi_attention_fl(cudaStream_t s, int B, int n, int Tp, int T, int H, int Dh, const float* qkv,
                                    const float* bqkv, Out out) {
  // split-BF16 operands (the mixed form): the warp-MMA kernel
  if constexpr (std::is_same<Out, StSplit>::value) {
    if (psi_attention_fl_mma_supported(n, Dh)) return launch_psi_attention_fl_mma(s, B, n, Tp, T, H, Dh, qkv, bqkv, out);
  }
  if (!psi_attention_fl_supported(n, Dh) || T < 2 || Tp < T) return cudaErrorInvalidValue;
  const size_t sm = psi_attention_fl_smem(n, Dh);
  const int rt = attention_fl_rows(n, Dh);
  int dev;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
#define QMC_ATT(RT)                                                                                       \
  {                                                                                                       \
    static int attr_dev = -1;                                                                             \
    if (attr_dev != dev) {                                                                                \
      e = cudaFuncSetAttribute(k_psi_attention_fl<RT, Out>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                               200 * 1024);                                                               \
      if (e != cudaSuccess) return e;                                                                     \
      attr_dev = dev;                                                                                     \
    }                                                                                                     \
    k_psi_attention_fl<RT, Out><<<(unsigned)(B * H), kAttnFlThreads, sm, s>>>(n, Tp, T, H, Dh, qkv, bqkv, out); \
  }
  if (rt == 1) QMC_ATT(1)
  else if (rt == 2) QMC_ATT(2)
  else if (rt == 3) QMC_ATT(3)
  else QMC_ATT(4)
#undef QMC_ATT
  return cudaGetLastError();
}

template cudaError_t launch_psi_group_fl<StF32>(cudaStream_t, int, int, int, const float*, int, const float*, int,
                                                float*, int, const float*, const float*, StF32);
template cudaError_t launch_psi_group_fl<StSplit>(cudaStream_t, int, int, int, const float*, int, const float*, int,
                                                  float*, int, const float*, const float*, StSplit);
template cudaError_t launch_psi_attention_fl<StF32>(cudaStream_t, int, int, int, int, int, int, const float*,
                                                    const float*, StF32);
template cudaError_t launch_psi_attention_fl<StSplit>(cudaStream_t, int, int, int, int, int, int, const float*,
                                                      const float*, StSplit);

}  // namespace qmc
