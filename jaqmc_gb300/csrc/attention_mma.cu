// Forward-Laplacian multi-head attention on warp-level split-BF16 MMAs
// (mixed form).  The same rules as k_psi_attention_fl (psiformer_fl.cu):
// with q scaled by 1/sqrt(Dh), S = q k^T, a = softmax_j(S), o = a v,
//   J_d S = J_d q k0^T + q0 J_d k^T
//   J_d a = a (J_d S - sum_k a J_d S)
//   J_d o = J_d a v0 + a J_d v
//   L S = L q k0^T + q0 L k^T + 2 sum_d J_d q J_d k^T
//   L a = a (sum_d b^2 - sum_k a sum_d b^2 + L S - sum_k a L S),  b = J_d S - sum_k a J_d S
//   L o = L a v0 + a L v + 2 sum_d J_d a J_d v,
// but every product of an n x Dh by Dh x n (scores) or n x n by n x Dh
// (mixing) block is formed by mma.m16n8k16 with both operands split into
// hi + lo bf16 and three products (hi hi + hi lo + lo hi, FP32 accumulate).
// The value-row scores and softmax stay FP32.
//
// One block (8 warps) per (walker, head).  Warp w owns the 16-row query tile
// it = w % mt of every direction in its group gi = w / mt (G = 8 / mt groups;
// group gi takes directions t = 2 + gi, 2 + gi + G, ...).  A group stages the
// q, k and v tangent rows of its next direction in shared memory with
// cp.async while it computes the current one, and synchronises on its own
// named barrier.  The cross sums sum_d J_d q J_d k^T, sum_d b^2 and
// sum_d J_d a J_d v stay in the owning warp's registers and are reduced over
// the groups in a fixed order at the end, so results do not depend on timing.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdlib>
#include <cstring>

#include "act.cuh"
#include "psiformer.cuh"

namespace qmc {

namespace {

constexpr int kAmThreads = 256;
constexpr int kAmWarps = kAmThreads / 32;

__device__ __forceinline__ void am_split(float x0, float x1, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - hf.x, x1 - hf.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

__device__ __forceinline__ void am_mma(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                       uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// d += A B with A = ah + al, B = bh + bl (the lo x lo product dropped)
__device__ __forceinline__ void am_mma3(float (&d)[4], const uint32_t (&ah)[4], const uint32_t (&al)[4], uint32_t bh0,
                                        uint32_t bh1, uint32_t bl0, uint32_t bl1) {
  am_mma(d, ah[0], ah[1], ah[2], ah[3], bh0, bh1);
  am_mma(d, ah[0], ah[1], ah[2], ah[3], bl0, bl1);
  am_mma(d, al[0], al[1], al[2], al[3], bh0, bh1);
}

__device__ __forceinline__ void am_cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void am_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void am_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void am_bar(int id, int count) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(count) : "memory");
}

__device__ __forceinline__ void am_put2(const StSplit& o, size_t r, int c, float v0, float v1) {
  uint32_t hi, lo;
  am_split(v0, v1, hi, lo);
  const size_t i = r * o.ld + c;
  *reinterpret_cast<uint32_t*>(o.p + i) = hi;
  *reinterpret_cast<uint32_t*>(o.p + i + o.plane) = lo;
}
__device__ __forceinline__ void am_put2(const StF32& o, size_t r, int c, float v0, float v1) {
  *reinterpret_cast<float2*>(o.p + r * o.ld + c) = make_float2(v0, v1);
}

}  // namespace

// Shared-memory plan of one block (byte offsets).  NP = n rounded up to 16,
// mt = NP / 16 query tiles, G direction groups.  Row strides: LDQ = Dh + 8
// (q and k tangent rows, 8-byte fragment reads conflict free), LDV = Dh + 4
// (v rows and the value-row arrays, column reads conflict free), LA = NP + 8
// (probabilities and the cross sums).
struct AmShape {
  int n, Dh, NP, mt, G, KE, NT8, KJ, ND8, LDQ, LDV, LA;
  size_t qfrag, kfrag, vfrag, afrag, A, U, stage, red, lap, bytes;
  __host__ __device__ AmShape(int n_, int Dh_, int G_) : n(n_), Dh(Dh_), G(G_) {
    NP = (n + 15) / 16 * 16;
    mt = NP / 16;
    KE = Dh / 16;
    NT8 = NP / 8;
    KJ = NP / 16;
    ND8 = Dh / 8;
    LDQ = Dh + 8;
    LDV = Dh + 4;
    LA = NP + 8;
    size_t o = 0;
    qfrag = o;
    o += (size_t)mt * KE * 32 * 32;  // [it][ks][lane] {hi[4], lo[4]}
    kfrag = o;
    o += (size_t)KE * NT8 * 32 * 16;  // [ks][nt][lane] {bh0, bh1, bl0, bl1}
    vfrag = o;
    o += (size_t)KJ * ND8 * 32 * 16;  // [kj][nd][lane]
    afrag = o;
    o += (size_t)mt * KJ * 32 * 32;  // [it][kj][lane]
    A = o;
    o += (size_t)NP * LA * 4;
    U = o;
    const size_t setup = (size_t)3 * NP * LDV * 4;  // Q0 K0 V0 (fp32, value rows)
    stage = (size_t)(2 * NP * LDQ + NP * LDV) * 4;  // dQ dK dV of one direction
    red = (size_t)(2 * NP * LA + NP * LDV) * 4;     // XS, Bq, XO of one group
    lap = stage;                                    // the Laplacian rows
    size_t u = setup;
    if ((size_t)G * 2 * stage > u) u = (size_t)G * 2 * stage;
    if ((size_t)G * red + lap > u) u = (size_t)G * red + lap;
    bytes = U + u;
  }
};

template <int MT, int DHT, class Out>
__global__ void __launch_bounds__(kAmThreads, 1) k_attention_fl_mma(int n, int Tp, int T, int H, int G,
                                                                     const float* __restrict__ qkv,
                                                                     const float* __restrict__ bqkv, Out out) {
  constexpr int Dh = 16 * DHT, NP = 16 * MT, KE = DHT, NT8 = 2 * MT, KJ = MT, ND8 = 2 * DHT;
  extern __shared__ __align__(16) uint8_t sm[];
  const AmShape sh(n, Dh, G);
  const int LDQ = sh.LDQ, LDV = sh.LDV, LA = sh.LA;
  uint32_t* qfrag = reinterpret_cast<uint32_t*>(sm + sh.qfrag);
  uint4* kfrag = reinterpret_cast<uint4*>(sm + sh.kfrag);
  uint4* vfrag = reinterpret_cast<uint4*>(sm + sh.vfrag);
  uint32_t* afrag = reinterpret_cast<uint32_t*>(sm + sh.afrag);
  float* Am = reinterpret_cast<float*>(sm + sh.A);
  uint8_t* U = sm + sh.U;
  const int w = blockIdx.x / H, h = blockIdx.x % H;
  const int D = H * Dh, ld3 = 3 * D;
  const float scale = 1.0f / sqrtf((float)Dh);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, c = lane & 3;
  const size_t grow = (size_t)w * n * Tp;
  auto rowp = [&](int i, int t) { return qkv + (grow + (size_t)i * Tp + t) * ld3 + h * Dh; };

  // ---- value rows (with biases; q scaled) and the FP32 softmax
  float* Q0f = reinterpret_cast<float*>(U);
  float* K0f = Q0f + NP * LDV;
  float* V0f = K0f + NP * LDV;
  for (int e = tid; e < NP * (Dh / 4); e += kAmThreads) {
    const int i = e / (Dh / 4), d = 4 * (e % (Dh / 4));
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f), k = q, v = q;
    if (i < n) {
      const float* r = rowp(i, 0) + d;
      const int cc = h * Dh + d;
      const float4 rq = *reinterpret_cast<const float4*>(r), rk = *reinterpret_cast<const float4*>(r + D),
                   rv = *reinterpret_cast<const float4*>(r + 2 * D);
      const float4 bq = *reinterpret_cast<const float4*>(bqkv + cc),
                   bk = *reinterpret_cast<const float4*>(bqkv + D + cc),
                   bv = *reinterpret_cast<const float4*>(bqkv + 2 * D + cc);
      q = make_float4((rq.x + bq.x) * scale, (rq.y + bq.y) * scale, (rq.z + bq.z) * scale, (rq.w + bq.w) * scale);
      k = make_float4(rk.x + bk.x, rk.y + bk.y, rk.z + bk.z, rk.w + bk.w);
      v = make_float4(rv.x + bv.x, rv.y + bv.y, rv.z + bv.z, rv.w + bv.w);
    }
    *reinterpret_cast<float4*>(Q0f + i * LDV + d) = q;
    *reinterpret_cast<float4*>(K0f + i * LDV + d) = k;
    *reinterpret_cast<float4*>(V0f + i * LDV + d) = v;
  }
  for (int e = tid; e < NP * LA; e += kAmThreads) Am[e] = 0.f;
  __syncthreads();
  for (int e = tid; e < n * n; e += kAmThreads) {
    const int i = e / n, j = e % n;
    float acc = 0.f;
    for (int d = 0; d < Dh; d += 4) {
      const float4 a = *reinterpret_cast<const float4*>(Q0f + i * LDV + d);
      const float4 b = *reinterpret_cast<const float4*>(K0f + j * LDV + d);
      acc = fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, fmaf(a.w, b.w, acc))));
    }
    Am[i * LA + j] = acc;
  }
  __syncthreads();
  for (int i = warp; i < n; i += kAmWarps) {
    float mx = -INFINITY;
    for (int j = lane; j < n; j += 32) mx = fmaxf(mx, Am[i * LA + j]);
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    float sum = 0.f;
    for (int j = lane; j < n; j += 32) {
      const float e = expf(Am[i * LA + j] - mx);
      Am[i * LA + j] = e;
      sum += e;
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    const float inv = 1.0f / sum;
    for (int j = lane; j < n; j += 32) Am[i * LA + j] *= inv;
  }
  __syncthreads();

  // ---- fixed operands in fragment order (hi/lo split once per block)
  for (int e = tid; e < MT * KE * 32; e += kAmThreads) {  // q0: A operand, k = feature
    const int it = e / (KE * 32), ks = (e / 32) % KE, ln = e % 32;
    const int r0 = 16 * it + (ln >> 2), k0 = 16 * ks + 2 * (ln & 3);
    uint32_t* f = qfrag + (size_t)e * 8;
    am_split(Q0f[r0 * LDV + k0], Q0f[r0 * LDV + k0 + 1], f[0], f[4]);
    am_split(Q0f[(r0 + 8) * LDV + k0], Q0f[(r0 + 8) * LDV + k0 + 1], f[1], f[5]);
    am_split(Q0f[r0 * LDV + k0 + 8], Q0f[r0 * LDV + k0 + 9], f[2], f[6]);
    am_split(Q0f[(r0 + 8) * LDV + k0 + 8], Q0f[(r0 + 8) * LDV + k0 + 9], f[3], f[7]);
  }
  for (int e = tid; e < KE * NT8 * 32; e += kAmThreads) {  // k0: B operand, k = feature, n = key
    const int ks = e / (NT8 * 32), nt = (e / 32) % NT8, ln = e % 32;
    const int j = 8 * nt + (ln >> 2), k0 = 16 * ks + 2 * (ln & 3);
    uint32_t bh0, bh1, bl0, bl1;
    am_split(K0f[j * LDV + k0], K0f[j * LDV + k0 + 1], bh0, bl0);
    am_split(K0f[j * LDV + k0 + 8], K0f[j * LDV + k0 + 9], bh1, bl1);
    kfrag[e] = make_uint4(bh0, bh1, bl0, bl1);
  }
  for (int e = tid; e < KJ * ND8 * 32; e += kAmThreads) {  // v0: B operand, k = key, n = feature
    const int kj = e / (ND8 * 32), nd = (e / 32) % ND8, ln = e % 32;
    const int d = 8 * nd + (ln >> 2), j0 = 16 * kj + 2 * (ln & 3);
    uint32_t bh0, bh1, bl0, bl1;
    am_split(V0f[j0 * LDV + d], V0f[(j0 + 1) * LDV + d], bh0, bl0);
    am_split(V0f[(j0 + 8) * LDV + d], V0f[(j0 + 9) * LDV + d], bh1, bl1);
    vfrag[e] = make_uint4(bh0, bh1, bl0, bl1);
  }
  for (int e = tid; e < MT * KJ * 32; e += kAmThreads) {  // a: A operand, k = key
    const int it = e / (KJ * 32), kj = (e / 32) % KJ, ln = e % 32;
    const int r0 = 16 * it + (ln >> 2), k0 = 16 * kj + 2 * (ln & 3);
    uint32_t* f = afrag + (size_t)e * 8;
    am_split(Am[r0 * LA + k0], Am[r0 * LA + k0 + 1], f[0], f[4]);
    am_split(Am[(r0 + 8) * LA + k0], Am[(r0 + 8) * LA + k0 + 1], f[1], f[5]);
    am_split(Am[r0 * LA + k0 + 8], Am[r0 * LA + k0 + 9], f[2], f[6]);
    am_split(Am[(r0 + 8) * LA + k0 + 8], Am[(r0 + 8) * LA + k0 + 9], f[3], f[7]);
  }
  __syncthreads();
  // the value-row arrays are dead: zero the staging buffers (rows past n stay zero)
  {
    float* z = reinterpret_cast<float*>(U);
    const size_t cnt = (size_t)G * 2 * sh.stage / 4;
    for (size_t e = tid; e < cnt; e += kAmThreads) z[e] = 0.f;
  }
  __syncthreads();

  const int it = warp % MT, gi = warp / MT;
  const int i0 = 16 * it;
  const int r0 = i0 + g, r1 = r0 + 8;
  float XS[NT8][4], BQ[NT8][4], XO[ND8][4];
#pragma unroll
  for (int a = 0; a < NT8; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) XS[a][b] = BQ[a][b] = 0.f;
#pragma unroll
  for (int a = 0; a < ND8; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) XO[a][b] = 0.f;

  // S (tile rows r0 / r1, all keys) = dQ k0^T + q0 dK^T [+ XS += dQ dK^T]
  auto scores = [&](const float* dQs, const float* dKs, float qscale, bool cross, float (&S)[NT8][4]) {
#pragma unroll
    for (int a = 0; a < NT8; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) S[a][b] = 0.f;
#pragma unroll
    for (int ks = 0; ks < KE; ++ks) {
      const int k0 = 16 * ks + 2 * c;
      uint32_t qh[4], ql[4];
      {
        const float2 x0 = *reinterpret_cast<const float2*>(dQs + r0 * LDQ + k0);
        const float2 x1 = *reinterpret_cast<const float2*>(dQs + r1 * LDQ + k0);
        const float2 x2 = *reinterpret_cast<const float2*>(dQs + r0 * LDQ + k0 + 8);
        const float2 x3 = *reinterpret_cast<const float2*>(dQs + r1 * LDQ + k0 + 8);
        am_split(x0.x * qscale, x0.y * qscale, qh[0], ql[0]);
        am_split(x1.x * qscale, x1.y * qscale, qh[1], ql[1]);
        am_split(x2.x * qscale, x2.y * qscale, qh[2], ql[2]);
        am_split(x3.x * qscale, x3.y * qscale, qh[3], ql[3]);
      }
      uint32_t q0h[4], q0l[4];
      {
        const uint4* f = reinterpret_cast<const uint4*>(qfrag + ((size_t)(it * KE + ks) * 32 + lane) * 8);
        const uint4 hh = f[0], ll = f[1];
        q0h[0] = hh.x, q0h[1] = hh.y, q0h[2] = hh.z, q0h[3] = hh.w;
        q0l[0] = ll.x, q0l[1] = ll.y, q0l[2] = ll.z, q0l[3] = ll.w;
      }
#pragma unroll
      for (int nt = 0; nt < NT8; ++nt) {
        const uint4 kb = kfrag[(ks * NT8 + nt) * 32 + lane];
        const float* kr = dKs + (8 * nt + g) * LDQ + k0;
        const float2 y0 = *reinterpret_cast<const float2*>(kr);
        const float2 y1 = *reinterpret_cast<const float2*>(kr + 8);
        uint32_t dh0, dl0, dh1, dl1;
        am_split(y0.x, y0.y, dh0, dl0);
        am_split(y1.x, y1.y, dh1, dl1);
        am_mma3(S[nt], qh, ql, kb.x, kb.y, kb.z, kb.w);
        am_mma3(S[nt], q0h, q0l, dh0, dh1, dl0, dl1);
        if (cross) am_mma3(XS[nt], qh, ql, dh0, dh1, dl0, dl1);
      }
    }
  };
  // O (tile rows, all features) = P v0 + a dV [+ XO += P dV]; P given as
  // accumulator tiles (the softmax tangent of S)
  auto mix = [&](const float (&P)[NT8][4], const float* dVs, bool cross, float (&O)[ND8][4]) {
#pragma unroll
    for (int a = 0; a < ND8; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) O[a][b] = 0.f;
#pragma unroll
    for (int kj = 0; kj < KJ; ++kj) {
      uint32_t ph[4], pl[4];
      am_split(P[2 * kj][0], P[2 * kj][1], ph[0], pl[0]);
      am_split(P[2 * kj][2], P[2 * kj][3], ph[1], pl[1]);
      am_split(P[2 * kj + 1][0], P[2 * kj + 1][1], ph[2], pl[2]);
      am_split(P[2 * kj + 1][2], P[2 * kj + 1][3], ph[3], pl[3]);
      uint32_t ah[4], al[4];
      {
        const uint4* f = reinterpret_cast<const uint4*>(afrag + ((size_t)(it * KJ + kj) * 32 + lane) * 8);
        const uint4 hh = f[0], ll = f[1];
        ah[0] = hh.x, ah[1] = hh.y, ah[2] = hh.z, ah[3] = hh.w;
        al[0] = ll.x, al[1] = ll.y, al[2] = ll.z, al[3] = ll.w;
      }
      const int j0 = 16 * kj + 2 * c;
#pragma unroll
      for (int nd = 0; nd < ND8; ++nd) {
        const uint4 vb = vfrag[(kj * ND8 + nd) * 32 + lane];
        const int d = 8 * nd + g;
        uint32_t vh0, vl0, vh1, vl1;
        am_split(dVs[j0 * LDV + d], dVs[(j0 + 1) * LDV + d], vh0, vl0);
        am_split(dVs[(j0 + 8) * LDV + d], dVs[(j0 + 9) * LDV + d], vh1, vl1);
        am_mma3(O[nd], ph, pl, vb.x, vb.y, vb.z, vb.w);
        am_mma3(O[nd], ah, al, vh0, vh1, vl0, vl1);
        if (cross) am_mma3(XO[nd], ph, pl, vh0, vh1, vl0, vl1);
      }
    }
  };
  auto put_rows = [&](int t, const float (&O)[ND8][4]) {
#pragma unroll
    for (int nd = 0; nd < ND8; ++nd) {
      const int col = h * Dh + 8 * nd + 2 * c;
      if (r0 < n) am_put2(out, grow + (size_t)r0 * Tp + t, col, O[nd][0], O[nd][1]);
      if (r1 < n) am_put2(out, grow + (size_t)r1 * Tp + t, col, O[nd][2], O[nd][3]);
    }
  };
  auto aval = [&](int r, int j) { return Am[r * LA + j]; };

  // ---- directions
  if (gi < G) {
    const int nthr = MT * 32, lid = it * 32 + lane, bar = 1 + gi;
    uint8_t* gbase = U + (size_t)gi * 2 * sh.stage;
    auto bufQ = [&](int b) { return reinterpret_cast<float*>(gbase + (size_t)b * sh.stage); };
    auto bufK = [&](int b) { return bufQ(b) + NP * LDQ; };
    auto bufV = [&](int b) { return bufQ(b) + 2 * NP * LDQ; };
    auto prefetch = [&](int t, int b) {
      float* q = bufQ(b);
      float* k = bufK(b);
      float* v = bufV(b);
      for (int e = lid; e < n * (Dh / 4); e += nthr) {
        const int j = e / (Dh / 4), d = 4 * (e % (Dh / 4));
        const float* src = rowp(j, t) + d;
        am_cp16(q + j * LDQ + d, src);
        am_cp16(k + j * LDQ + d, src + D);
        am_cp16(v + j * LDV + d, src + 2 * D);
      }
      am_commit();
    };
    int t = 2 + gi, b = 0;
    if (t < T) prefetch(t, 0);
    for (; t < T; t += G, b ^= 1) {
      const bool more = t + G < T;
      if (more) prefetch(t + G, b ^ 1);
      if (more) am_wait<1>();
      else am_wait<0>();
      am_bar(bar, nthr);
      float S[NT8][4];
      scores(bufQ(b), bufK(b), scale, true, S);
      // softmax tangent: b = S - sum_k a S; sum_d b^2; S <- a b
      float ab0 = 0.f, ab1 = 0.f;
#pragma unroll
      for (int nt = 0; nt < NT8; ++nt) {
        const int j = 8 * nt + 2 * c;
        ab0 = fmaf(aval(r0, j), S[nt][0], fmaf(aval(r0, j + 1), S[nt][1], ab0));
        ab1 = fmaf(aval(r1, j), S[nt][2], fmaf(aval(r1, j + 1), S[nt][3], ab1));
      }
      ab0 += __shfl_xor_sync(0xffffffffu, ab0, 1);
      ab0 += __shfl_xor_sync(0xffffffffu, ab0, 2);
      ab1 += __shfl_xor_sync(0xffffffffu, ab1, 1);
      ab1 += __shfl_xor_sync(0xffffffffu, ab1, 2);
#pragma unroll
      for (int nt = 0; nt < NT8; ++nt) {
        const int j = 8 * nt + 2 * c;
        const float a00 = aval(r0, j), a01 = aval(r0, j + 1), a10 = aval(r1, j), a11 = aval(r1, j + 1);
        const float b0 = S[nt][0] - ab0, b1 = S[nt][1] - ab0, b2 = S[nt][2] - ab1, b3 = S[nt][3] - ab1;
        BQ[nt][0] = fmaf(b0, b0, BQ[nt][0]);
        BQ[nt][1] = fmaf(b1, b1, BQ[nt][1]);
        BQ[nt][2] = fmaf(b2, b2, BQ[nt][2]);
        BQ[nt][3] = fmaf(b3, b3, BQ[nt][3]);
        S[nt][0] = a00 * b0;
        S[nt][1] = a01 * b1;
        S[nt][2] = a10 * b2;
        S[nt][3] = a11 * b3;
      }
      float O[ND8][4];
      mix(S, bufV(b), true, O);
      put_rows(t, O);
      am_bar(bar, nthr);  // the group is done with buffer b
    }
  }
  __syncthreads();

  // ---- cross sums of the groups, reduced in group order
  float* red = reinterpret_cast<float*>(U);
  const size_t redf = sh.red / 4;
  if (gi < G) {
    float* xs = red + (size_t)gi * redf;
    float* bq = xs + NP * LA;
    float* xo = bq + NP * LA;
#pragma unroll
    for (int nt = 0; nt < NT8; ++nt) {
      const int j = 8 * nt + 2 * c;
      xs[r0 * LA + j] = XS[nt][0];
      xs[r0 * LA + j + 1] = XS[nt][1];
      xs[r1 * LA + j] = XS[nt][2];
      xs[r1 * LA + j + 1] = XS[nt][3];
      bq[r0 * LA + j] = BQ[nt][0];
      bq[r0 * LA + j + 1] = BQ[nt][1];
      bq[r1 * LA + j] = BQ[nt][2];
      bq[r1 * LA + j + 1] = BQ[nt][3];
    }
#pragma unroll
    for (int nd = 0; nd < ND8; ++nd) {
      const int d = 8 * nd + 2 * c;
      xo[r0 * LDV + d] = XO[nd][0];
      xo[r0 * LDV + d + 1] = XO[nd][1];
      xo[r1 * LDV + d] = XO[nd][2];
      xo[r1 * LDV + d + 1] = XO[nd][3];
    }
  }
  __syncthreads();
  for (size_t e = tid; e < redf; e += kAmThreads) {
    float s = red[e];
    for (int q = 1; q < G; ++q) s += red[(size_t)q * redf + e];
    red[e] = s;
  }
  // the Laplacian rows (t = 1) into the space after the group partials
  float* lQ = reinterpret_cast<float*>(U + (size_t)G * sh.red);
  float* lK = lQ + NP * LDQ;
  float* lV = lK + NP * LDQ;
  for (int e = tid; e < NP * (Dh / 4); e += kAmThreads) {
    const int j = e / (Dh / 4), d = 4 * (e % (Dh / 4));
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f), k = q, v = q;
    if (j < n) {
      const float* r = rowp(j, 1) + d;
      q = *reinterpret_cast<const float4*>(r);
      k = *reinterpret_cast<const float4*>(r + D);
      v = *reinterpret_cast<const float4*>(r + 2 * D);
    }
    *reinterpret_cast<float4*>(lQ + j * LDQ + d) = q;
    *reinterpret_cast<float4*>(lK + j * LDQ + d) = k;
    *reinterpret_cast<float4*>(lV + j * LDV + d) = v;
  }
  __syncthreads();

  // ---- Laplacian and value rows: one warp per query tile
  if (warp < MT) {
    const float* xs = red;
    const float* bq = xs + NP * LA;
    const float* xo = bq + NP * LA;
    float S[NT8][4];
    scores(lQ, lK, scale, false, S);
    float m1a = 0.f, m1b = 0.f, m2a = 0.f, m2b = 0.f;
#pragma unroll
    for (int nt = 0; nt < NT8; ++nt) {
      const int j = 8 * nt + 2 * c;
      S[nt][0] += 2.f * xs[r0 * LA + j];
      S[nt][1] += 2.f * xs[r0 * LA + j + 1];
      S[nt][2] += 2.f * xs[r1 * LA + j];
      S[nt][3] += 2.f * xs[r1 * LA + j + 1];
      m1a = fmaf(aval(r0, j), bq[r0 * LA + j], fmaf(aval(r0, j + 1), bq[r0 * LA + j + 1], m1a));
      m1b = fmaf(aval(r1, j), bq[r1 * LA + j], fmaf(aval(r1, j + 1), bq[r1 * LA + j + 1], m1b));
      m2a = fmaf(aval(r0, j), S[nt][0], fmaf(aval(r0, j + 1), S[nt][1], m2a));
      m2b = fmaf(aval(r1, j), S[nt][2], fmaf(aval(r1, j + 1), S[nt][3], m2b));
    }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
      m1a += __shfl_xor_sync(0xffffffffu, m1a, o);
      m1b += __shfl_xor_sync(0xffffffffu, m1b, o);
      m2a += __shfl_xor_sync(0xffffffffu, m2a, o);
      m2b += __shfl_xor_sync(0xffffffffu, m2b, o);
    }
#pragma unroll
    for (int nt = 0; nt < NT8; ++nt) {
      const int j = 8 * nt + 2 * c;
      S[nt][0] = aval(r0, j) * (bq[r0 * LA + j] - m1a + S[nt][0] - m2a);
      S[nt][1] = aval(r0, j + 1) * (bq[r0 * LA + j + 1] - m1a + S[nt][1] - m2a);
      S[nt][2] = aval(r1, j) * (bq[r1 * LA + j] - m1b + S[nt][2] - m2b);
      S[nt][3] = aval(r1, j + 1) * (bq[r1 * LA + j + 1] - m1b + S[nt][3] - m2b);
    }
    float O[ND8][4];
    mix(S, lV, false, O);
#pragma unroll
    for (int nd = 0; nd < ND8; ++nd) {
      const int d = 8 * nd + 2 * c;
      O[nd][0] += 2.f * xo[r0 * LDV + d];
      O[nd][1] += 2.f * xo[r0 * LDV + d + 1];
      O[nd][2] += 2.f * xo[r1 * LDV + d];
      O[nd][3] += 2.f * xo[r1 * LDV + d + 1];
    }
    put_rows(1, O);
    // value rows: o = a v0
#pragma unroll
    for (int a = 0; a < ND8; ++a)
#pragma unroll
      for (int q = 0; q < 4; ++q) O[a][q] = 0.f;
#pragma unroll
    for (int kj = 0; kj < KJ; ++kj) {
      const uint4* f = reinterpret_cast<const uint4*>(afrag + ((size_t)(it * KJ + kj) * 32 + lane) * 8);
      const uint4 hh = f[0], ll = f[1];
      const uint32_t ah[4] = {hh.x, hh.y, hh.z, hh.w}, al[4] = {ll.x, ll.y, ll.z, ll.w};
#pragma unroll
      for (int nd = 0; nd < ND8; ++nd) {
        const uint4 vb = vfrag[(kj * ND8 + nd) * 32 + lane];
        am_mma3(O[nd], ah, al, vb.x, vb.y, vb.z, vb.w);
      }
    }
    put_rows(0, O);
  }
  // padding rows past T
  for (int e = tid; e < n * (Tp - T) * (Dh / 2); e += kAmThreads) {
    const int i = e / ((Tp - T) * (Dh / 2)), r = e % ((Tp - T) * (Dh / 2));
    am_put2(out, grow + (size_t)i * Tp + T + r / (Dh / 2), h * Dh + 2 * (r % (Dh / 2)), 0.f, 0.f);
  }
}

// Direction groups: as many as the warps allow (8 / query tiles), fewer when
// the staging buffers would not fit.
static int am_groups(int n, int Dh) {
  const int mt = (n + 15) / 16;
  for (int G = kAmWarps / mt; G >= 1; --G)
    if (AmShape(n, Dh, G).bytes <= 220 * 1024) return G;
  return 0;
}

// QMC_ATTENTION_FL=simt in the environment keeps the FP32 SIMT kernel in the
// mixed form too (a diagnostic switch, read once per process).
static bool am_disabled() {
  static const int off = [] {
    const char* v = std::getenv("QMC_ATTENTION_FL");
    return v && std::strcmp(v, "simt") == 0 ? 1 : 0;
  }();
  return off != 0;
}

bool psi_attention_fl_mma_supported(int n, int Dh) {
  return !am_disabled() && n >= 1 && n <= 48 && (Dh == 16 || Dh == 32 || Dh == 64) && am_groups(n, Dh) > 0;
}

template <class Out>
cudaError_t launch_psi_attention_fl_mma(cudaStream_t s, int B, int n, int Tp, int T, int H, int Dh, const float* qkv,
                                        const float* bqkv, Out out) {
  if (!psi_attention_fl_mma_supported(n, Dh) || T < 2 || Tp < T || (H * Dh) % 8) return cudaErrorInvalidValue;
  const int G = am_groups(n, Dh);
  const size_t sm = AmShape(n, Dh, G).bytes;
  const int mt = (n + 15) / 16;
  int dev;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
#define QMC_AM(MT, DHT)                                                                                          \
  {                                                                                                              \
    static int attr_dev = -1;                                                                                    \
    if (attr_dev != dev) {                                                                                       \
      e = cudaFuncSetAttribute(k_attention_fl_mma<MT, DHT, Out>, cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                               220 * 1024);                                                                      \
      if (e != cudaSuccess) return e;                                                                            \
      attr_dev = dev;                                                                                            \
    }                                                                                                            \
    k_attention_fl_mma<MT, DHT, Out><<<(unsigned)(B * H), kAmThreads, sm, s>>>(n, Tp, T, H, G, qkv, bqkv, out); \
  }
#define QMC_AM_DH(MT)         \
  if (Dh == 16) QMC_AM(MT, 1) \
  else if (Dh == 32) QMC_AM(MT, 2) else QMC_AM(MT, 4)
  if (mt == 1) QMC_AM_DH(1)
  else if (mt == 2) QMC_AM_DH(2)
  else QMC_AM_DH(3)
#undef QMC_AM_DH
#undef QMC_AM
  return cudaGetLastError();
}

template cudaError_t launch_psi_attention_fl_mma<StSplit>(cudaStream_t, int, int, int, int, int, int, const float*,
                                                          const float*, StSplit);

}  // namespace qmc
