// FP32 SIMT GEMM over "tangent rows" with group-aware epilogues.
//
// Rows of every activation buffer are (walker w, electron i, tangent t) with
// t = 0 value, t = 1 Laplacian, t = 2 + 3e + c the derivative along
// coordinate c of electron e, and t in [T, Tp) zero padding.  A "group" is
// the Tp rows of one (w, i).  A thread block owns whole groups
// (G = 128 / Tp of them), so the epilogue sees every tangent of an output
// element and can apply the forward-Laplacian activation rule
//   h = f(z0),  J_t h = f'(z0) z_t,  L h = f'(z0) z_L + f''(z0) sum_t z_t^2
// without another pass over memory.
#pragma once
#include "act.cuh"
#include "common.cuh"

namespace qmc {

// group g -> (walker, electron); rows are ((w*n + i) * Tp + t)
struct RowMap {
  int gpw;  // groups per walker
  int i0;   // electron index of a walker's first group
  int n;    // electrons per walker in the row layout
  int Tp;   // padded tangents per group
  __device__ __forceinline__ int w(int g) const { return g / gpw; }
  __device__ __forceinline__ int i(int g) const { return i0 + g % gpw; }
  __device__ __forceinline__ size_t row(int g, int t) const {
    return ((size_t)w(g) * n + i(g)) * Tp + t;
  }
};

constexpr int kBM = 128, kBN = 128, kBK = 8, kCsLd = kBN + 4;
constexpr size_t kSimtSmem = (size_t)kBM * kCsLd * sizeof(float);  // epilogue staging

// out[row][col] = acc (+bias[col]); rows of the plain map.
struct EpiStore {
  float* out;
  int ld;
  const float* bias;
  int accumulate = 0;  // out += result instead of out = result
  __device__ void operator()(const float* Cs, int ng, int g0, int n0, int N, const RowMap& m) const {
    const int Tp = m.Tp;
    for (int p = threadIdx.x; p < ng * Tp * kBN; p += blockDim.x) {
      int r = p / kBN, c = p % kBN, col = n0 + c;
      if (col >= N) continue;
      int lg = r / Tp, t = r % Tp;
      float v = Cs[r * kCsLd + c];
      if (bias) v += bias[col];
      float* o = out + m.row(g0 + lg, t) * ld + col;
      *o = accumulate ? *o + v : v;
    }
  }
};

// FermiNet one-electron layer: z = acc + Gb[w,t] + (t==0) b; tanh with the
// tangent rules; residual (h_in + h)/sqrt(2) when `resid` is set.  `Out` is
// the storage policy of the activations (StF32 or StSplit).
template <class Out>
struct EpiLayer {
  const float* Gb;   // [walkers*Tp][N] broadcast (spin-mean) term
  const float* bias; // [N]
  Out resid;         // rows like out; resid.p == nullptr: no residual
  Out out;
  int T;             // real tangents (1 = value only)
  __device__ __forceinline__ void put(size_t row, int col, float v) const {
    if (resid.valid()) v = (v + resid.get(row, col)) * kRsqrt2;
    out.put(row, col, v);
  }
  __device__ void operator()(const float* Cs, int ng, int g0, int n0, int N, const RowMap& m) const {
    const int Tp = m.Tp;
    for (int p = threadIdx.x; p < ng * kBN; p += blockDim.x) {
      int lg = p / kBN, c = p % kBN, col = n0 + c;
      if (col >= N) continue;
      int g = g0 + lg;
      const float* cs = Cs + (lg * Tp) * kCsLd + c;
      const float* gb = Gb + (size_t)m.w(g) * Tp * N + col;
      size_t r0 = m.row(g, 0);
      float h = tanhf(cs[0] + gb[0] + bias[col]);
      put(r0, col, h);
      if (T > 1) {
        float d1 = 1.0f - h * h, d2 = -2.0f * h * d1, S = 0.0f;
        for (int t = 2; t < T; ++t) {
          float z = cs[t * kCsLd] + gb[(size_t)t * N];
          S = fmaf(z, z, S);
          put(r0 + t, col, d1 * z);
        }
        float zL = cs[kCsLd] + gb[N];
        put(r0 + 1, col, d1 * zL + d2 * S);
        for (int t = T; t < Tp; ++t) out.put(r0 + t, col, 0.0f);
      }
    }
  }
};

// Orbitals x envelope with the product rule; writes the orbital matrices
// (fp32, layout of amat_index).  Columns are (k, j) = k*n + j.
struct EpiOrbital {
  float* A;
  const float* rae;    // [walkers*n][A]
  const float* aevec;  // [walkers*n][A][3]
  const float* pi;     // this spin channel: [n][A][K]
  const float* sigma;  // [n][A][K]
  int n, natom, K, T, env_abs;
  float* orb = nullptr;  // value-only passes: also store the orbitals before the envelope
  int unit_env = 0;      // store the orbitals without an envelope (diagonal / null envelopes)
  __device__ void operator()(const float* Cs, int ng, int g0, int n0, int N, const RowMap& m) const {
    const int Tp = m.Tp;
    for (int p = threadIdx.x; p < ng * kBN; p += blockDim.x) {
      int lg = p / kBN, c = p % kBN, col = n0 + c;
      if (col >= N) continue;
      int g = g0 + lg, w = m.w(g), i = m.i(g);
      int k = col / n, j = col % n;
      const float* ra = rae + ((size_t)w * n + i) * natom;
      const float* av = aevec + (((size_t)w * n + i) * natom) * 3;
      float e0 = 0.f, ex = 0.f, ey = 0.f, ez = 0.f, el = 0.f;
      // all atoms' parameters first, so their loads are in flight together
      float pvs[8], svs[8];
#pragma unroll
      for (int I = 0; I < 8; ++I) {
        pvs[I] = I < natom && !unit_env ? pi[((size_t)j * natom + I) * K + k] : 0.f;
        svs[I] = I < natom && !unit_env ? sigma[((size_t)j * natom + I) * K + k] : 0.f;
      }
      if (unit_env) e0 = 1.f;
      for (int I = 0; I < (unit_env ? 0 : natom); ++I) {
        float pv = I < 8 ? pvs[I] : pi[((size_t)j * natom + I) * K + k];
        float sv = I < 8 ? svs[I] : sigma[((size_t)j * natom + I) * K + k];
        float r = ra[I];
        float se = env_abs ? fabsf(sv) : sv;
        float ev = pv * expf(-se * r);
        e0 += ev;
        if (T > 1) {
          float gr = -se * ev / r;
          ex = fmaf(gr, av[3 * I + 0], ex);
          ey = fmaf(gr, av[3 * I + 1], ey);
          ez = fmaf(gr, av[3 * I + 2], ez);
          el += ev * (se * se - 2.0f * se / r);
        }
      }
      const float* cs = Cs + (lg * Tp) * kCsLd + c;
      float* dst = A + amat_index(Tp, n, K, w, k, 0, i, j);
      const size_t ts = amat_tangent_stride(n, K);
      float o0 = cs[0];
      dst[0] = o0 * e0;
      if (orb) orb[amat_index(1, n, K, w, k, 0, i, j)] = o0;
      if (T > 1) {
        int ti = 2 + 3 * i;
        for (int t = 2; t < T; ++t) {
          float v = cs[t * kCsLd] * e0;
          if (t == ti) v = fmaf(o0, ex, v);
          else if (t == ti + 1) v = fmaf(o0, ey, v);
          else if (t == ti + 2) v = fmaf(o0, ez, v);
          dst[t * ts] = v;
        }
        float cross = cs[ti * kCsLd] * ex + cs[(ti + 1) * kCsLd] * ey + cs[(ti + 2) * kCsLd] * ez;
        dst[ts] = cs[kCsLd] * e0 + 2.0f * cross + o0 * el;
        for (int t = T; t < Tp; ++t) dst[t * ts] = 0.0f;
      }
    }
  }
};

// The kernel and its launcher have internal linkage: every translation unit
// that includes this header owns its own instantiations, and with them its own
// record of which device already has the shared-memory opt-in set.
namespace {

// C[rows x N] = [A1 | A2][rows x (K1+K2)] * W[(K1+K2) x N].  K1 and K2 are
// multiples of 8; W rows are read as float4, so ldw is a multiple of 4 with
// zero columns from N up to round_up(N, 4); A1/A2/W are 16-byte aligned.
template <class Epi>
__global__ void __launch_bounds__(256)
k_gemm_simt(int n_groups, RowMap map, const float* __restrict__ A1, int lda1, int K1,
            const float* __restrict__ A2, int lda2, int K2, const float* __restrict__ W, int ldw,
            int N, Epi epi) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  float* As = smem;                  // [2][kBK][kBM]
  float* Bs = smem + 2 * kBK * kBM;  // [2][kBK][kBN]
  const int tid = threadIdx.x;
  const int Tp = map.Tp;
  const int G = kBM / Tp;
  const int g0 = blockIdx.x * G;
  const int ng = min(G, n_groups - g0);
  const int n0 = blockIdx.y * kBN;
  const int K = K1 + K2;

  // loader coordinates
  const int a_r = tid >> 1, a_k = (tid & 1) * 4;
  const int a_lg = a_r / Tp, a_t = a_r % Tp;
  const bool a_ok = a_lg < ng;
  const size_t a_row = a_ok ? map.row(g0 + a_lg, a_t) : 0;
  const int b_k = tid >> 5, b_c = (tid & 31) * 4;
  const bool b_ok = (n0 + b_c) < N;

  auto load_a = [&](int k0, float4& v) {
    v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!a_ok) return;
    int k = k0 + a_k;
    const float* src = (k < K1) ? (A1 + a_row * lda1 + k) : (A2 + a_row * lda2 + (k - K1));
    v = *reinterpret_cast<const float4*>(src);
  };
  auto load_b = [&](int k0, float4& v) {
    v = b_ok ? *reinterpret_cast<const float4*>(W + (size_t)(k0 + b_k) * ldw + n0 + b_c)
             : make_float4(0.f, 0.f, 0.f, 0.f);
  };
  auto store_tiles = [&](int buf, const float4& va, const float4& vb) {
    float* as = As + buf * kBK * kBM;
    as[(a_k + 0) * kBM + a_r] = va.x;
    as[(a_k + 1) * kBM + a_r] = va.y;
    as[(a_k + 2) * kBM + a_r] = va.z;
    as[(a_k + 3) * kBM + a_r] = va.w;
    *reinterpret_cast<float4*>(Bs + buf * kBK * kBN + b_k * kBN + b_c) = vb;
  };

  const int ty = tid >> 4, tx = tid & 15;
  float acc[8][8];
#pragma unroll
  for (int r = 0; r < 8; ++r)
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[r][c] = 0.f;

  float4 va, vb;
  load_a(0, va);
  load_b(0, vb);
  store_tiles(0, va, vb);
  __syncthreads();
  int buf = 0;
  for (int k0 = 0; k0 < K; k0 += kBK) {
    const bool more = k0 + kBK < K;
    if (more) {
      load_a(k0 + kBK, va);
      load_b(k0 + kBK, vb);
    }
    const float* as = As + buf * kBK * kBM;
    const float* bs = Bs + buf * kBK * kBN;
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      float4 a0 = *reinterpret_cast<const float4*>(as + kk * kBM + ty * 4);
      float4 a1 = *reinterpret_cast<const float4*>(as + kk * kBM + 64 + ty * 4);
      float4 b0 = *reinterpret_cast<const float4*>(bs + kk * kBN + tx * 4);
      float4 b1 = *reinterpret_cast<const float4*>(bs + kk * kBN + 64 + tx * 4);
      float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int r = 0; r < 8; ++r)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
    }
    if (more) {
      store_tiles(buf ^ 1, va, vb);
      __syncthreads();
      buf ^= 1;
    }
  }
  __syncthreads();
  // stage the accumulator tile for the group-aware epilogue
  float* Cs = smem;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    int row = (r < 4) ? (ty * 4 + r) : (64 + ty * 4 + r - 4);
    *reinterpret_cast<float4*>(Cs + row * kCsLd + tx * 4) =
        make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
    *reinterpret_cast<float4*>(Cs + row * kCsLd + 64 + tx * 4) =
        make_float4(acc[r][4], acc[r][5], acc[r][6], acc[r][7]);
  }
  __syncthreads();
  if (ng > 0) epi(Cs, ng, g0, n0, N, map);
}

template <class Epi>
cudaError_t launch_gemm_simt(cudaStream_t s, int n_groups, RowMap map, const float* A1, int lda1,
                             int K1, const float* A2, int lda2, int K2, const float* W, int ldw,
                             int N, const Epi& epi) {
  if (n_groups <= 0) return cudaSuccess;
  if (map.Tp > kBM) return cudaErrorInvalidValue;
  static int attr_dev = -1;  // the attribute is per device
  int dev;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (attr_dev != dev) {
    e = cudaFuncSetAttribute(k_gemm_simt<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSimtSmem);
    if (e != cudaSuccess) return e;
    attr_dev = dev;
  }
  int G = kBM / map.Tp;
  dim3 grid((n_groups + G - 1) / G, (N + kBN - 1) / kBN);
  k_gemm_simt<Epi><<<grid, 256, kSimtSmem, s>>>(n_groups, map, A1, lda1, K1, A2, lda2, K2, W, ldw, N, epi);
  return cudaGetLastError();
}

}  // namespace

}  // namespace qmc
