// Split-BF16 tcgen05 GEMMs (see stream_tc.cuh).
//
// One CTA computes a 128-feature x N-column accumulator (N = whole tangent
// groups, <= 256).  Warp roles: warp 0 issues the TMA loads of the K chunks
// (64 bf16 = one 128-byte swizzle row) into a ring of shared-memory stages;
// warp 1 owns the TMEM allocation and issues the MMAs (3 per K=16 step:
// hi*hi, hi*lo, lo*hi); warps 2-9 run the epilogue from TMEM, two warps per
// TMEM lane quarter splitting the tile's columns.  The kernel is persistent:
// one CTA per SM walks a static list of (column tile, 128-feature block) work
// items with two TMEM accumulators, so the epilogue of one item overlaps the
// loads and MMAs of the next.  Every
// mbarrier wait is bounded; on expiry the CTA records an error code, waits
// (bounded) for its own copies and MMAs, frees TMEM and exits.
#include <cudaTypedefs.h>

#include <algorithm>
#include <type_traits>

#include "stream_tc.cuh"
#include "tc_ptx.cuh"

namespace qmc {

constexpr int kTcThreads = 320;
constexpr int kEpiWarps = 8;
constexpr int kKChunk = 64;                      // bf16 per 128-byte swizzle row
constexpr int kATile = 128 * kKChunk * 2;        // bytes of one A plane tile
constexpr long long kWaitCycles = 1000000000LL;  // about 0.5 s at 2 GHz
constexpr int kErrTimeoutFull = 1, kErrTimeoutEmpty = 2, kErrTimeoutAcc = 3;
constexpr int kEnvRegs = 8;  // atoms whose envelope parameters stay in registers

struct TileInfo {
  int row0;   // first activation row of the tile (TMA y coordinate)
  int a_sel;  // which A tensor map (orbital spin channel)
  int g0;     // first group
  int ng;     // valid groups in the tile
  int w, i0;  // orbital tiles: walker and first electron
};

struct TcArgs {
  int n_tiles, n_mblocks;  // work items: (column tile, 128-feature block)
  int n_cols;     // columns per tile (G * Tp)
  int G, Tp, T;
  int k_chunks, k1_chunks;
  int stages;
  int tmem_cols;
  int n_out;
  int resid_last;  // order the K chunks so this CTA's residual features come last
  int ebuf_bytes;  // epilogue staging bytes per half (0: unused)
  int b4d;         // activation maps are 4-D (k, electron, walker, plane), one per spin channel
  int* err;
};

// K-chunk order: source B (0 = first, 1 = second), chunk index within it,
// and the A (weight) K offset.  With resid_last: second-source chunks first,
// then the first-source chunks outside [m0, m0+128), then those two.
__device__ __forceinline__ void chunk_src(const TcArgs& g, int m0, int c, int* b2, int* kx, int* ka) {
  const int nx = g.k1_chunks, n2 = g.k_chunks - g.k1_chunks;
  if (!g.resid_last) {
    *b2 = c >= nx;
    *kx = (c < nx ? c : c - nx) * kKChunk;
    *ka = c * kKChunk;
    return;
  }
  if (c < n2) {
    *b2 = 1;
    *kx = c * kKChunk;
    *ka = (nx + c) * kKChunk;
    return;
  }
  const int r0 = m0 / kKChunk;
  int idx = c - n2, j;
  if (idx >= nx - 2) {
    j = r0 + (idx - (nx - 2));
  } else {
    j = idx < r0 ? idx : idx + 2;
  }
  *b2 = 0;
  *kx = j * kKChunk;
  *ka = j * kKChunk;
}

__device__ __forceinline__ void report(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// 10 warps share the SM's four 16K-register sub-partitions (three warps on
// two of them), which caps a thread at 168 registers.
template <class Epi>
__global__ void __launch_bounds__(kTcThreads, 1)
k_tc_gemm(const __grid_constant__ CUtensorMap mapA0, const __grid_constant__ CUtensorMap mapA1,
          const __grid_constant__ CUtensorMap mapB1, const __grid_constant__ CUtensorMap mapB2, TcArgs g,
          Epi epi) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int stage_b = g.n_cols * kKChunk * 2;
  const int stage_bytes = 2 * kATile + 2 * stage_b;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)g.stages * stage_bytes);
  uint64_t* empty = full + g.stages;
  uint64_t* tfull = empty + g.stages;   // [2] accumulator ready
  uint64_t* tempty = tfull + 2;         // [2] accumulator drained by the epilogue
  uint64_t* done = tempty + 2;          // all MMAs of this CTA complete
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  int* aborted = reinterpret_cast<int*>(tmem_slot + 1);
  // per epilogue half: a staging tile of [2 planes][rows][128 features] bf16
  uint8_t* ebuf0 = smem + (size_t)g.stages * stage_bytes + 256;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_items = g.n_tiles * g.n_mblocks;
  const int acc_cols = g.tmem_cols / 2;  // column offset of the second accumulator

  // once any CTA of the call has given up on a wait, the rest skip their work
  __shared__ int skip;
  if (threadIdx.x == 0) skip = g.err ? *(volatile int*)g.err : 0;
  __syncthreads();
  if (skip) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < g.stages; ++s) {
      ptx::mbar_init(&full[s], 1);
      ptx::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      ptx::mbar_init(&tfull[b], 1);
      ptx::mbar_init(&tempty[b], kEpiWarps);
    }
    ptx::mbar_init(done, 1);
    *aborted = 0;
    ptx::fence_mbar_init();
  }
  if (warp == 1) {
    ptx::tmem_alloc(tmem_slot, (uint32_t)g.tmem_cols);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      ptx::prefetch_tmap(&mapA0);
      ptx::prefetch_tmap(&mapB1);
      int cg = 0;  // chunks issued by this CTA
      for (int it = blockIdx.x; it < n_items && !*(volatile int*)aborted; it += gridDim.x) {
        const int mb = it % g.n_mblocks, m0 = mb * 128;
        const TileInfo ti = epi.tile(it / g.n_mblocks, g);
        const CUtensorMap* A = ti.a_sel ? &mapA1 : &mapA0;
        for (int c = 0; c < g.k_chunks; ++c, ++cg) {
          const int s = cg % g.stages;
          const uint32_t ph = (uint32_t)(cg / g.stages) & 1u;
          if (!ptx::mbar_wait_bounded(&empty[s], ph ^ 1u, kWaitCycles)) {
            report(g.err, kErrTimeoutEmpty);
            atomicExch(aborted, 1);
            break;
          }
          uint8_t* base = smem + (size_t)s * stage_bytes;
          int b2, kx, ka;
          chunk_src(g, m0, c, &b2, &kx, &ka);
          ptx::mbar_expect_tx(&full[s], (uint32_t)stage_bytes);
          ptx::tma_load_3d(base, A, ka, m0, 0, &full[s]);
          ptx::tma_load_3d(base + kATile, A, ka, m0, 1, &full[s]);
          if (g.b4d) {  // one spin channel's electrons of walkers row0 ..
            const CUtensorMap* Bm = ti.a_sel ? &mapB2 : &mapB1;
            ptx::tma_load_4d(base + 2 * kATile, Bm, kx, 0, ti.row0, 0, &full[s]);
            ptx::tma_load_4d(base + 2 * kATile + stage_b, Bm, kx, 0, ti.row0, 1, &full[s]);
          } else {
            const CUtensorMap* Bm = b2 ? &mapB2 : &mapB1;
            ptx::tma_load_3d(base + 2 * kATile, Bm, kx, ti.row0, 0, &full[s]);
            ptx::tma_load_3d(base + 2 * kATile + stage_b, Bm, kx, ti.row0, 1, &full[s]);
          }
        }
      }
      // never leave with copies in flight: wait (bounded) for the last phase
      // armed on every stage
      for (int c = cg - g.stages; c < cg; ++c) {
        if (c < 0) continue;
        ptx::mbar_wait_bounded(&full[c % g.stages], (uint32_t)(c / g.stages) & 1u, kWaitCycles);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = ptx::idesc_bf16(128, g.n_cols);
      int cg = 0, j = 0;
      for (int it = blockIdx.x; it < n_items && !*(volatile int*)aborted; it += gridDim.x, ++j) {
        const int buf = j & 1;
        const uint32_t use = (uint32_t)(j >> 1);
        if (!ptx::mbar_wait_bounded(&tempty[buf], (use & 1u) ^ 1u, kWaitCycles)) {
          report(g.err, kErrTimeoutAcc);
          atomicExch(aborted, 1);
          break;
        }
        ptx::tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(buf * acc_cols);
        bool ok = true;
        for (int c = 0; c < g.k_chunks; ++c, ++cg) {
          const int s = cg % g.stages;
          const uint32_t ph = (uint32_t)(cg / g.stages) & 1u;
          if (!ptx::mbar_wait_bounded(&full[s], ph, kWaitCycles)) {
            report(g.err, kErrTimeoutFull);
            atomicExch(aborted, 1);
            ok = false;
            break;
          }
          ptx::tc_fence_after();
          uint8_t* base = smem + (size_t)s * stage_bytes;
          const uint64_t a_hi = ptx::sw128_desc(base), a_lo = ptx::sw128_desc(base + kATile);
          const uint64_t b_hi = ptx::sw128_desc(base + 2 * kATile);
          const uint64_t b_lo = ptx::sw128_desc(base + 2 * kATile + stage_b);
#pragma unroll
          for (int kk = 0; kk < kKChunk / 16; ++kk) {
            const uint64_t off = (uint64_t)(kk * 32) >> 4;  // 16 bf16 = 32 bytes
            ptx::mma_bf16(acc, a_hi + off, b_hi + off, idesc, (c | kk) != 0);
            ptx::mma_bf16(acc, a_hi + off, b_lo + off, idesc, 1u);
            ptx::mma_bf16(acc, a_lo + off, b_hi + off, idesc, 1u);
          }
          ptx::mma_commit(&empty[s]);
        }
        if (!ok) break;
        ptx::mma_commit(&tfull[buf]);
      }
      ptx::mma_commit(done);  // fires once every MMA issued here has completed
      ptx::mbar_wait_bounded(done, 0u, kWaitCycles);
    }
  } else {
    const int q = warp & 3;            // TMEM lane quarter accessible to this warp
    const int half = (warp - 2) >> 2;  // which of the two warps of this quarter
    int j = 0;
    for (int it = blockIdx.x; it < n_items; it += gridDim.x, ++j) {
      const int buf = j & 1;
      const uint32_t use = (uint32_t)(j >> 1);
      if (!ptx::mbar_wait_bounded(&tfull[buf], use & 1u, kWaitCycles)) {
        report(g.err, kErrTimeoutAcc);
        atomicExch(aborted, 1);
        break;
      }
      if (*(volatile int*)aborted) break;
      ptx::tc_fence_after();
      const int mb = it % g.n_mblocks, m0 = mb * 128;
      const TileInfo ti = epi.tile(it / g.n_mblocks, g);
      const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(buf * acc_cols);
      epi.run(ti, g, taddr, m0 + 32 * q + lane, half, ebuf0 + (size_t)half * g.ebuf_bytes);
      ptx::tc_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(ptx::smem_u32(&tempty[buf]))
                                  : "memory");
    }
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    ptx::tc_fence_after();
    ptx::tmem_dealloc(tmem, (uint32_t)g.tmem_cols);
  }
}

// ------------------------------------------------------------ epilogues
// contiguous tiles: groups [tile*G, tile*G + G), rows tile*G*Tp ...
struct ContigTiles {
  int n_groups;
  __device__ TileInfo tile(int tx, const TcArgs& g) const {
    TileInfo t{};
    t.g0 = tx * g.G;
    t.ng = min(g.G, n_groups - t.g0);
    t.row0 = t.g0 * g.Tp;
    return t;
  }
};

// One-electron layer epilogue.  Each warp owns 32 features (a TMEM lane
// quarter) and walks the rows of its tile in chunks of 16, reading the
// accumulators as 16x256b fragments (a thread: 4 features x 2 row pairs).
// Two shared-memory staging tiles per warp of [2 planes][16 rows][32
// features] bf16 take the residual rows of the next chunk by cp.async while
// the current chunk is computed; ldmatrix/stmatrix (.trans) move the residual
// into and the outputs out of the fragment layout, outputs replace the
// residual in place, and a chunk leaves with 16-byte stores per plane.  No
// barrier is wider than the warp.  Tangent rows past T come out as zeros.
template <bool RESID>
struct EpiTcLayer : ContigTiles {
  static constexpr int kCR = 16;                 // rows per chunk
  static constexpr int kBuf = 2 * kCR * 32;      // bf16 per chunk buffer
  static constexpr int kGbuf = kCR * 32;         // floats per broadcast-term chunk
  int n, ld;  // electrons per walker, activation row width (n_out)
  StSplit resid, out;
  const float* Gb;
  const float* bias;

  // Value-pass staging tiles [2 planes][16 rows][4 pieces of 8 features],
  // piece p of row r stored at p ^ ((r >> 1) & 3): the eight rows of an 8x8
  // ldmatrix / stmatrix tile then fall on distinct bank groups.
  static __device__ __forceinline__ int swz(int r, int p) { return p ^ ((r >> 1) & 3); }
  __device__ __forceinline__ void fetch_sw(const StSplit& st, size_t row0, int nrows, int col0, int nvec, int lane,
                                           __nv_bfloat16* buf) const {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int v = lane + 32 * q;
      const int pl = v >> 6, r = (v >> 2) & 15, vq = v & 3;
      if (r < nrows && vq < nvec)
        ptx::cp_async16(buf + (pl * kCR + r) * 32 + 8 * swz(r, vq),
                        st.p + pl * st.plane + (row0 + r) * (size_t)st.ld + col0 + 8 * vq);
    }
    ptx::cp_async_commit();
  }
  __device__ __forceinline__ void store_sw(const StSplit& st, size_t row0, int nrows, int col0, int nvec, int lane,
                                           const __nv_bfloat16* buf) const {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int v = lane + 32 * q;
      const int pl = v >> 6, r = (v >> 2) & 15, vq = v & 3;
      if (r < nrows && vq < nvec)
        *reinterpret_cast<uint4*>(st.p + pl * st.plane + (row0 + r) * (size_t)st.ld + col0 + 8 * vq) =
            *reinterpret_cast<const uint4*>(buf + (pl * kCR + r) * 32 + 8 * swz(r, vq));
    }
  }
  // tangent passes: staging rows [lo, hi) <-> rows row0 + [lo, hi) (row0 may
  // be negative; only rows in [lo, hi) are addressed)
  __device__ __forceinline__ void fetch_rows_sw(const StSplit& st, long long row0, int lo, int hi, int col0,
                                                int nvec, int lane, __nv_bfloat16* buf) const {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int v = lane + 32 * q;
      const int pl = v >> 6, r = (v >> 2) & 15, vq = v & 3;
      if (r >= lo && r < hi && vq < nvec)
        ptx::cp_async16(buf + (pl * kCR + r) * 32 + 8 * swz(r, vq),
                        st.p + pl * st.plane + (size_t)(row0 + r) * st.ld + col0 + 8 * vq);
    }
    ptx::cp_async_commit();
  }
  __device__ __forceinline__ void store_rows_sw(const StSplit& st, long long row0, int lo, int hi, int skip, int col0,
                                                int nvec, int lane, const __nv_bfloat16* buf) const {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int v = lane + 32 * q;
      const int pl = v >> 6, r = (v >> 2) & 15, vq = v & 3;
      if (r >= lo && r < hi && r != skip && vq < nvec)
        *reinterpret_cast<uint4*>(st.p + pl * st.plane + (size_t)(row0 + r) * st.ld + col0 + 8 * vq) =
            *reinterpret_cast<const uint4*>(buf + (pl * kCR + r) * 32 + 8 * swz(r, vq));
    }
  }
  // broadcast rows t0 + [lo, hi) of a walker (fp32, row stride N) -> gbuf,
  // committed with the next residual fetch
  __device__ __forceinline__ void fetch_gb_sw(const float* gbw, int t0, int lo, int hi, int col0, int N, int lane,
                                              float* gbuf) const {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int v = lane + 32 * q;
      const int r = v >> 3, p = v & 7;
      if (r >= lo && r < hi && col0 + 4 * p + 4 <= N)
        ptx::cp_async16(gbuf + r * 32 + 4 * (p ^ (((r >> 1) & 3) << 1)), gbw + (size_t)(t0 + r) * N + col0 + 4 * p);
    }
  }
  __device__ void run(const TileInfo& ti, const TcArgs& g, uint32_t taddr, int f, int half, uint8_t* ebuf) const {
    const int N = g.n_out;
    const int lane = f & 31, col0 = f - lane;
    const int q = (f & 127) >> 5;
    const int nvec = max(0, min(4, (N - col0) / 8));
    __nv_bfloat16* buf0 = reinterpret_cast<__nv_bfloat16*>(ebuf) + q * 2 * kBuf;  // value-only layout
    if (g.T == 1) {
      // Thread T holds features col0 + T/4 + 8 fb (fb = 0..3) of rows
      // 8 rb + 2(T%4) + {0, 1} (rb = 0, 1) of each 16-row chunk: the 16x256b
      // TMEM fragment, which ldmatrix / stmatrix (.trans) move to and from the
      // [row][feature] staging tile.
      const int T4 = lane >> 2, T2 = 2 * (lane & 3);
      float bq[4];
      int Fq[4];
#pragma unroll
      for (int fb = 0; fb < 4; ++fb) {
        Fq[fb] = col0 + T4 + 8 * fb;
        bq[fb] = Fq[fb] < N ? bias[Fq[fb]] : 0.f;
      }
      int c0 = 16 * half, k = 0;
      if (c0 >= ti.ng) return;
      const uint32_t tq = taddr;  // lane field: this warp's quarter
      if (RESID) fetch_sw(resid, (size_t)(ti.g0 + c0), min(16, ti.ng - c0), col0, nvec, lane, buf0);
      for (; c0 < ti.ng; c0 += 32, k ^= 1) {
        __nv_bfloat16* buf = buf0 + k * kBuf;
        const int nrows = min(16, ti.ng - c0);
        const size_t row0 = (size_t)(ti.g0 + c0);
        const bool more = c0 + 32 < ti.ng;
        if (RESID && more)
          fetch_sw(resid, row0 + 32, min(16, ti.ng - c0 - 32), col0, nvec, lane, buf0 + (k ^ 1) * kBuf);
        // r[4 (2 lh + rb) + q]: lane half lh (features + 16 lh), row block rb
        uint32_t r[16];
#pragma unroll
        for (int lh = 0; lh < 2; ++lh)
#pragma unroll
          for (int rb = 0; rb < 2; ++rb)
            ptx::tmem_ld16x256_nw(tq + ((uint32_t)(16 * lh) << 16) + (uint32_t)(c0 + 8 * rb), r + 4 * (2 * lh + rb));
        // broadcast terms of the rows' walkers (row0 = w0 n + e0; rows past
        // the chunk's first walker found by 32-bit division of e0 + rr)
        const unsigned row32 = (unsigned)(ti.g0 + c0);
        const unsigned w0 = row32 / (unsigned)n;
        const unsigned e0 = row32 - w0 * (unsigned)n;
        float gb[2][2][4];  // [rb][e][fb]
#pragma unroll
        for (int rb = 0; rb < 2; ++rb)
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int rr = 8 * rb + T2 + e;
            const size_t w = w0 + (e0 + (unsigned)rr) / (unsigned)n;
#pragma unroll
            for (int fb = 0; fb < 4; ++fb)
              gb[rb][e][fb] = (rr < nrows && Fq[fb] < N) ? __ldg(Gb + w * N + Fq[fb]) : 0.f;
          }
        ptx::tmem_wait16(r);
        if (more) ptx::cp_async_wait<1>();
        else ptx::cp_async_wait<0>();
        __syncwarp();
        const uint32_t sb = ptx::smem_u32(buf);
        // tile address of this lane: row 8 rb + (lane % 8) of piece (lane / 8)
        const int lr = lane & 7, lp = lane >> 3;
#pragma unroll
        for (int rb = 0; rb < 2; ++rb) {
          const int row = 8 * rb + lr;
          const uint32_t a_hi = sb + (uint32_t)(((0 * kCR + row) * 32 + 8 * swz(row, lp)) * 2);
          const uint32_t a_lo = sb + (uint32_t)(((1 * kCR + row) * 32 + 8 * swz(row, lp)) * 2);
          uint32_t rh[4], rl[4];
          if (RESID) {
            ptx::ldsm_x4_trans(a_hi, rh);
            ptx::ldsm_x4_trans(a_lo, rl);
          }
          uint32_t oh[4], ol[4];
#pragma unroll
          for (int fb = 0; fb < 4; ++fb) {
            // accumulator registers of (fb, rb): lane half fb / 2, rows even/odd at q = 2 (fb & 1) + e
            const uint32_t* ra = r + 4 * (2 * (fb >> 1) + rb) + 2 * (fb & 1);
            float2 y = make_float2(split_tanh(__uint_as_float(ra[0]) + gb[rb][0][fb] + bq[fb]),
                                   split_tanh(__uint_as_float(ra[1]) + gb[rb][1][fb] + bq[fb]));
            if (RESID) {
              const float2 h2 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&rh[fb]));
              const float2 l2 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&rl[fb]));
              y = __fmul2_rn(__fadd2_rn(y, __fadd2_rn(h2, l2)), make_float2(kRsqrt2, kRsqrt2));
            }
            const __nv_bfloat162 hi = __floats2bfloat162_rn(y.x, y.y);
            const float2 lo2 = __ffma2_rn(__bfloat1622float2(hi), make_float2(-1.f, -1.f), y);  // y - hi, exact
            const __nv_bfloat162 lo = __floats2bfloat162_rn(lo2.x, lo2.y);
            oh[fb] = *reinterpret_cast<const uint32_t*>(&hi);
            ol[fb] = *reinterpret_cast<const uint32_t*>(&lo);
          }
          ptx::stsm_x4_trans(a_hi, oh);
          ptx::stsm_x4_trans(a_lo, ol);
        }
        __syncwarp();
        store_sw(out, row0, nrows, col0, nvec, lane, buf);
        __syncwarp();
      }
      return;
    }
    const int Tp = g.Tp, T = g.T;
    // Tangent passes, same fragment layout as the value pass.  A group
    // (electron) occupies tile columns [lg*Tp, lg*Tp + Tp); its 16-column
    // chunks start at lg*Tp rounded down to a multiple of 8 (off = 0 or 4
    // columns earlier), so chunk c holds tangents t = 16c - off + [0, 16);
    // fragment rows outside [0, Tp) belong to the neighbouring groups and are
    // neither used nor stored.  The value row t = 0 sits in lane T%4 = off/2
    // of each quad (rb = 0, e = 0), the Laplacian row t = 1 next to it.
    // Per warp: two residual/output staging tiles and two broadcast-term tiles
    // (fp32 [16][32], piece p of row r at p ^ (2 ((r >> 1) & 3))), refilled by
    // cp.async one chunk ahead.
    buf0 = reinterpret_cast<__nv_bfloat16*>(ebuf) + q * (2 * kBuf + 2 * kGbuf * 2);
    float* gbuf0 = reinterpret_cast<float*>(buf0 + 2 * kBuf);
    const int T4 = lane >> 2, T2 = 2 * (lane & 3);
    float bq[4];
    int Fq[4];
#pragma unroll
    for (int fb = 0; fb < 4; ++fb) {
      Fq[fb] = col0 + T4 + 8 * fb;
      bq[fb] = Fq[fb] < N ? bias[Fq[fb]] : 0.f;
    }
    const int lr = lane & 7, lp = lane >> 3;
    for (int lg = half; lg < ti.ng; lg += 2) {
      const int gi = ti.g0 + lg;
      const size_t r0 = (size_t)gi * Tp;
      const int cs0 = lg * Tp, off = cs0 & 7;
      const uint32_t tca = taddr + (uint32_t)(cs0 - off);
      const float* gbw = Gb + (size_t)(gi / n) * Tp * N;  // this walker's broadcast rows
      const int nch = (Tp + off + 15) / 16;
      // staging rows of chunk c that hold this group's tangents
      auto sr_lo = [&](int c) { return max(0, off - 16 * c); };
      auto sr_hi = [&](int c) { return min(16, Tp + off - 16 * c); };
      auto prefetch = [&](int c, int kb) {
        const int t0 = 16 * c - off;  // tangent of staging row 0 (may be negative)
        fetch_gb_sw(gbw, t0, sr_lo(c), sr_hi(c), col0, N, lane, gbuf0 + kb * kGbuf);
        if (RESID) fetch_rows_sw(resid, (long long)r0 + t0, sr_lo(c), sr_hi(c), col0, nvec, lane, buf0 + kb * kBuf);
        else ptx::cp_async_commit();
      };
      prefetch(0, 0);
      float h[4], d1[4], S[4] = {0.f, 0.f, 0.f, 0.f}, zL[4] = {0.f, 0.f, 0.f, 0.f}, res1[4] = {0.f, 0.f, 0.f, 0.f};
      // |grad z|^2 partial sums: S from the checked chunks, S2 (rows e = 0, 1
      // apart) from the unchecked ones
      float2 S2[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
      const int src = (lane & ~3) | (off >> 1);  // quad lane holding t = 0 and t = 1
      int k = 0;
      for (int c = 0; c < nch; ++c, k ^= 1) {
        __nv_bfloat16* buf = buf0 + k * kBuf;
        const float* gbuf = gbuf0 + k * kGbuf;
        const bool more = c + 1 < nch;
        if (more) prefetch(c + 1, k ^ 1);
        uint32_t r[16];
#pragma unroll
        for (int lh = 0; lh < 2; ++lh)
#pragma unroll
          for (int rb = 0; rb < 2; ++rb)
            if (16 * c + 8 * rb - off < Tp)  // the block holds tangents of this group
              ptx::tmem_ld16x256_nw(tca + ((uint32_t)(16 * lh) << 16) + (uint32_t)(16 * c + 8 * rb),
                                    r + 4 * (2 * lh + rb));
        ptx::tmem_wait16(r);
        if (more) ptx::cp_async_wait<1>();
        else ptx::cp_async_wait<0>();
        __syncwarp();
        const uint32_t sb = ptx::smem_u32(buf);
        uint32_t rh[2][4], rl[2][4];
        if (RESID) {
#pragma unroll
          for (int rb = 0; rb < 2; ++rb) {
            const int row = 8 * rb + lr;
            ptx::ldsm_x4_trans(sb + (uint32_t)(((0 * kCR + row) * 32 + 8 * swz(row, lp)) * 2), rh[rb]);
            ptx::ldsm_x4_trans(sb + (uint32_t)(((1 * kCR + row) * 32 + 8 * swz(row, lp)) * 2), rl[rb]);
          }
        }
        // MODE 1: every row of the chunk is a Jacobian tangent or a padding
        // row (T <= t < Tp) of this group: padding rows have zero
        // accumulators, broadcast terms and residuals, so they come out as
        // the zeros they must be stored as with no per-row checks.  MODE 2:
        // the group's first chunk with off = 0, the same plus the value row
        // t = 0 and the Laplacian row t = 1 in fragment slot (rb 0, e 0 / 1)
        // of quad lane 0.  MODE 0: chunks that reach into a neighbouring
        // group (off > 0, or Tp not a multiple of 16), rows checked one by
        // one.
        auto compute = [&](auto mode_tag) {
          constexpr int MODE = decltype(mode_tag)::value;
          // pre-activations z of this thread's 16 elements [rb][e][fb]; the two
          // rows e = 0, 1 of a (rb, fb) slot are one packed f32x2 operand in
          // the unchecked modes
          float z[2][2][4];
  #pragma unroll
          for (int rb = 0; rb < 2; ++rb)
  #pragma unroll
            for (int fb = 0; fb < 4; ++fb) {
              const uint32_t* ra = r + 4 * (2 * (fb >> 1) + rb) + 2 * (fb & 1);
              float gv[2];
  #pragma unroll
              for (int e = 0; e < 2; ++e) {
                const int sr = 8 * rb + T2 + e;
                const int pz = ((T4 >> 2) + 2 * fb) ^ (((sr >> 1) & 3) << 1);
                gv[e] = gbuf[sr * 32 + 4 * pz + (T4 & 3)];
              }
              if (MODE != 0) {
                const float2 zp = __fadd2_rn(make_float2(__uint_as_float(ra[0]), __uint_as_float(ra[1])),
                                             make_float2(gv[0], gv[1]));
                z[rb][0][fb] = zp.x;
                z[rb][1][fb] = zp.y;
              } else {
  #pragma unroll
                for (int e = 0; e < 2; ++e) {
                  const int t = 16 * c - off + 8 * rb + T2 + e;
                  z[rb][e][fb] = (t >= 0 && t < T) ? __uint_as_float(ra[e]) + gv[e] : 0.f;
                }
              }
            }
          float res[2][2][4];
  #pragma unroll
          for (int rb = 0; rb < 2; ++rb)
  #pragma unroll
            for (int fb = 0; fb < 4; ++fb) {
              if (RESID) {
                const float2 h2 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&rh[rb][fb]));
                const float2 l2 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&rl[rb][fb]));
                const float2 rs = __fadd2_rn(h2, l2);
                res[rb][0][fb] = rs.x;
                res[rb][1][fb] = rs.y;
              } else {
                res[rb][0][fb] = res[rb][1][fb] = 0.f;
              }
            }
          if (MODE == 2 || (MODE == 0 && c == 0)) {
            // value row: h = tanh(z + b) on the source lane, then shared by the quad
  #pragma unroll
            for (int fb = 0; fb < 4; ++fb) {
              const float hv = tanhf(z[0][0][fb] + bq[fb]);
              h[fb] = __shfl_sync(0xffffffffu, hv, src);
              d1[fb] = 1.f - h[fb] * h[fb];
              zL[fb] = z[0][1][fb];
              res1[fb] = res[0][1][fb];
            }
          }
          const bool head = MODE == 2 && (lane & 3) == 0;  // this lane holds t = 0 and t = 1
          uint32_t oh[2][4], ol[2][4];
  #pragma unroll
          for (int rb = 0; rb < 2; ++rb)
  #pragma unroll
            for (int fb = 0; fb < 4; ++fb) {
              float2 y;
              if (MODE == 0) {
                float ys[2];
  #pragma unroll
                for (int e = 0; e < 2; ++e) {
                  const int t = 16 * c - off + 8 * rb + T2 + e;
                  const float zz = z[rb][e][fb];
                  float v;
                  if (t == 0) {
                    v = h[fb];
                  } else {
                    if (t >= 2) S[fb] = fmaf(zz, zz, S[fb]);  // zero for padding rows
                    v = d1[fb] * zz;                          // t = 1 rewritten at the end
                  }
                  if (RESID) v = (v + res[rb][e][fb]) * kRsqrt2;
                  ys[e] = t >= T ? 0.f : v;
                }
                y = make_float2(ys[0], ys[1]);
              } else {
                const float2 zz = make_float2(z[rb][0][fb], z[rb][1][fb]);
                // MODE 2, rb 0: the head lane's rows t = 0, 1 stay out of |grad z|^2
                const float2 zs = (MODE == 2 && rb == 0 && head) ? make_float2(0.f, 0.f) : zz;
                S2[fb] = __ffma2_rn(zs, zs, S2[fb]);
                y = __fmul2_rn(make_float2(d1[fb], d1[fb]), zz);  // t = 1 rewritten at the end
                if (MODE == 2 && rb == 0 && head) y.x = h[fb];
                if (RESID)
                  y = __fmul2_rn(__fadd2_rn(y, make_float2(res[rb][0][fb], res[rb][1][fb])),
                                 make_float2(kRsqrt2, kRsqrt2));
              }
              const __nv_bfloat162 hi = __floats2bfloat162_rn(y.x, y.y);
              const float2 lo2 = __ffma2_rn(__bfloat1622float2(hi), make_float2(-1.f, -1.f), y);  // y - hi, exact
              const __nv_bfloat162 lo = __floats2bfloat162_rn(lo2.x, lo2.y);
              oh[rb][fb] = *reinterpret_cast<const uint32_t*>(&hi);
              ol[rb][fb] = *reinterpret_cast<const uint32_t*>(&lo);
            }
  #pragma unroll
          for (int rb = 0; rb < 2; ++rb) {
            const int row = 8 * rb + lr;
            ptx::stsm_x4_trans(sb + (uint32_t)(((0 * kCR + row) * 32 + 8 * swz(row, lp)) * 2), oh[rb]);
            ptx::stsm_x4_trans(sb + (uint32_t)(((1 * kCR + row) * 32 + 8 * swz(row, lp)) * 2), ol[rb]);
          }
        };
        const int tc0 = 16 * c - off;
        const bool inside = tc0 >= 0 && tc0 + 16 <= Tp;
        if (inside && c > 0) compute(std::integral_constant<int, 1>{});
        else if (inside && off == 0) compute(std::integral_constant<int, 2>{});
        else compute(std::integral_constant<int, 0>{});
        __syncwarp();
        // rows of this group except the Laplacian row (written below)
        store_rows_sw(out, (long long)r0 + 16 * c - off, sr_lo(c), sr_hi(c), c == 0 ? off + 1 : -1, col0, nvec, lane,
                      buf);
        __syncwarp();
      }
      // Laplacian row: quad sums of sum_d z_d^2, then on the source lane
      // y = tanh'' |grad z|^2 + tanh' lap z  (tanh'' = -2 h tanh')
#pragma unroll
      for (int fb = 0; fb < 4; ++fb) {
        float st = S[fb] + (S2[fb].x + S2[fb].y);
        st += __shfl_xor_sync(0xffffffffu, st, 1);
        st += __shfl_xor_sync(0xffffffffu, st, 2);
        float y1 = d1[fb] * zL[fb] - 2.f * h[fb] * d1[fb] * st;
        if (RESID) y1 = (y1 + res1[fb]) * kRsqrt2;
        if (lane == src && Fq[fb] < N) {
          const __nv_bfloat16 hi = __float2bfloat16_rn(y1);
          __nv_bfloat16* o = out.p + (r0 + 1) * (size_t)out.ld + Fq[fb];
          o[0] = hi;
          o[out.plane] = __float2bfloat16_rn(y1 - __bfloat162float(hi));
        }
      }
    }
  }

};

struct EpiTcStore : ContigTiles {
  float* out;
  int ld;
  __device__ void run(const TileInfo& ti, const TcArgs& g, uint32_t taddr, int f, int half, uint8_t*) const {
    const bool fok = f < g.n_out;
    for (int c0 = 16 * half; c0 < g.n_cols; c0 += 32) {
      float v[16];
      ptx::tmem_ld16(taddr + c0, v);
      if (!fok) continue;
#pragma unroll
      for (int j = 0; j < 16; ++j)
        if (c0 + j < ti.ng) out[(size_t)(ti.row0 + c0 + j) * ld + f] = v[j];
    }
  }
};

// Orbital tiles never straddle a (walker, spin channel): tile -> (w, s, chunk).
struct EpiTcOrbital {
  int n, n_up, split, K, natom, env_abs, tiles_up, tiles_per_walker;
  const float* pi[2];
  const float* sigma[2];
  const float* rae;
  const float* aevec;
  float* A;
  int raw;           // value-only passes: store orbitals without the envelope factor
  int unit_env;      // tangent passes: envelope 1 (the diagonal / null envelopes come later)
  int n_rows;  // B * n (value-only passes)
  // value-only passes with split orbitals: tiles of W4[s] walkers x the
  // electrons of channel s (4-D activation maps), tpc4[s] tiles per channel
  int chan4d, B;
  int W4[2], tpc4[2];
  // channel selects (a runtime index into a kernel-parameter array would
  // copy the struct to local memory)
  __device__ __forceinline__ const float* pis(int s) const { return s ? pi[1] : pi[0]; }
  __device__ __forceinline__ const float* sigs(int s) const { return s ? sigma[1] : sigma[0]; }
  __device__ TileInfo tile(int tx, const TcArgs& g) const {
    TileInfo t{};
    if (g.T == 1 && chan4d) {
      const int s = tx < tpc4[0] ? 0 : 1;
      const int ns = s ? n - n_up : n_up;
      t.a_sel = s;
      t.w = (s ? tx - tpc4[0] : tx) * (s ? W4[1] : W4[0]);
      t.row0 = t.w;
      t.i0 = s ? n_up : 0;
      t.ng = min(s ? W4[1] : W4[0], B - t.w) * ns;
      return t;
    }
    if (g.T == 1) {
      // value-only: contiguous 256-row tiles over all walkers, one pass per
      // spin channel; rows of the other channel are skipped in the epilogue
      const int tpc = (n_rows + 255) / 256;
      t.a_sel = split ? tx / tpc : 0;
      t.g0 = (tx % tpc) * 256;
      t.ng = min(256, n_rows - t.g0);
      t.row0 = t.g0;
      return t;
    }
    const int w = tx / tiles_per_walker, r = tx % tiles_per_walker;
    int s = 0, chunk = r, i0 = 0, ns = n;
    if (split) {
      s = r < tiles_up ? 0 : 1;
      chunk = s == 0 ? r : r - tiles_up;
      i0 = s == 0 ? 0 : n_up;
      ns = s == 0 ? n_up : n - n_up;
    }
    t.a_sel = s;
    t.w = w;
    t.i0 = i0 + chunk * g.G;
    t.ng = min(g.G, ns - chunk * g.G);
    t.row0 = (w * n + t.i0) * g.Tp;
    return t;
  }
  // envelope parameters of column (k, j) for the first kEnvRegs atoms, held
  // in registers across the tile's rows
  struct EnvParams {
    float pv[kEnvRegs], se[kEnvRegs];
  };
  __device__ void load_params(int s, int k, int j, EnvParams& ep) const {
#pragma unroll
    for (int I = 0; I < kEnvRegs; ++I) {
      float pv = 0.f, se = 0.f;
      if (I < natom && !unit_env) {
        pv = pis(s)[((size_t)j * natom + I) * K + k];
        float sv = sigs(s)[((size_t)j * natom + I) * K + k];
        se = env_abs ? fabsf(sv) : sv;
      }
      ep.pv[I] = pv;
      ep.se[I] = se;
    }
  }
  // envelope value, gradient (wrt the electron) and Laplacian for column (k, j)
  __device__ void envelope(int s, int w, int i, int k, int j, int T, float* e, const EnvParams& ep) const {
    if (unit_env) {
      e[0] = 1.f; e[1] = 0.f; e[2] = 0.f; e[3] = 0.f; e[4] = 0.f;
      return;
    }
    const float* ra = rae + ((size_t)w * n + i) * natom;
    const float* av = aevec + ((size_t)w * n + i) * natom * 3;
    float e0 = 0.f, ex = 0.f, ey = 0.f, ez = 0.f, el = 0.f;
    auto term = [&](int I, float pv, float se) {
      float r = ra[I];
      float ev = pv * expf(-se * r);
      e0 += ev;
      if (T > 1) {
        float gr = -se * ev / r;
        ex = fmaf(gr, av[3 * I], ex);
        ey = fmaf(gr, av[3 * I + 1], ey);
        ez = fmaf(gr, av[3 * I + 2], ez);
        el += ev * (se * se - 2.0f * se / r);
      }
    };
    // constant indices keep the register-held parameters out of local memory
#pragma unroll
    for (int I = 0; I < kEnvRegs; ++I)
      if (I < natom) term(I, ep.pv[I], ep.se[I]);
    for (int I = kEnvRegs; I < natom; ++I) {
      float sv = sigs(s)[((size_t)j * natom + I) * K + k];
      term(I, pis(s)[((size_t)j * natom + I) * K + k], env_abs ? fabsf(sv) : sv);
    }
    e[0] = e0; e[1] = ex; e[2] = ey; e[3] = ez; e[4] = el;
  }
  __device__ void run(const TileInfo& ti, const TcArgs& g, uint32_t taddr, int f, int half, uint8_t*) const {
    const bool fok = f < g.n_out;
    const int k = fok ? f / n : 0, j = fok ? f % n : 0;
    const size_t ts = amat_tangent_stride(n, K);
    EnvParams ep;
    if (g.T == 1 && raw) {  // value-only raw stores use no envelope
#pragma unroll
      for (int I = 0; I < kEnvRegs; ++I) ep.pv[I] = ep.se[I] = 0.f;
    } else {
      load_params(ti.a_sel, k, j, ep);
    }
    if (g.T == 1 && chan4d) {
      const int ns = ti.a_sel ? n - n_up : n_up;
      // raw stores of whole chunks walk one pointer: column (wq, iq) of the
      // tile lands at base + wq*K*n*n + iq*n for this thread's (k, j)
      const int wstride = K * n * n;
      float* base = A + amat_index(1, n, K, ti.w, k, 0, ti.i0, j);
      for (int c0 = 16 * half; c0 < g.n_cols; c0 += 32) {
        float v[16];
        ptx::tmem_ld16(taddr + c0, v);
        if (!fok || c0 >= ti.ng) continue;
        int wq = c0 / ns, iq = c0 - wq * ns;
        if (raw && c0 + 16 <= ti.ng) {
          int off = wq * wstride + iq * n;
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) {
            base[off] = v[jj];
            off += n;
            if (++iq == ns) {
              iq = 0;
              off += wstride - ns * n;
            }
          }
          continue;
        }
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
          if (c0 + jj < ti.ng) {
            const int w = ti.w + wq, i = ti.i0 + iq;
            const size_t idx = amat_index(1, n, K, w, k, 0, i, j);
            if (raw) {
              A[idx] = v[jj];
            } else {
              float e[5];
              envelope(ti.a_sel, w, i, k, j, 1, e, ep);
              A[idx] = v[jj] * e[0];
            }
          }
          if (++iq == ns) {
            iq = 0;
            ++wq;
          }
        }
      }
      return;
    }
    if (g.T == 1) {
      for (int c0 = 16 * half; c0 < g.n_cols; c0 += 32) {
        float v[16];
        ptx::tmem_ld16(taddr + c0, v);
        if (!fok || c0 >= ti.ng) continue;
        const int gi0 = ti.g0 + c0;
        int w = gi0 / n, i = gi0 - w * n;
        if (raw && c0 + 16 <= ti.ng) {
          // column (w, i) lands at base + w*K*n*n + i*n for this thread's (k, j)
          float* base = A + amat_index(1, n, K, w, k, 0, 0, j);
          const int wstep = K * n * n - n * n;
          int off = i * n;
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) {
            if (!split || (i < n_up ? 0 : 1) == ti.a_sel) base[off] = v[jj];
            off += n;
            if (++i == n) {
              i = 0;
              off += wstep;
            }
          }
          continue;
        }
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
          if (c0 + jj < ti.ng && (!split || (i < n_up ? 0 : 1) == ti.a_sel)) {
            const size_t idx = amat_index(1, n, K, w, k, 0, i, j);
            if (raw) {
              A[idx] = v[jj];
            } else {
              float e[5];
              envelope(ti.a_sel, w, i, k, j, 1, e, ep);
              A[idx] = v[jj] * e[0];
            }
          }
          if (++i == n) {
            i = 0;
            ++w;
          }
        }
      }
      return;
    }
    for (int lg = half; lg < ti.ng; lg += 2) {
      const int i = ti.i0 + lg;
      float e[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      if (fok) envelope(ti.a_sel, ti.w, i, k, j, g.T, e, ep);
      float* dst = A + amat_index(g.Tp, n, K, ti.w, k, 0, i, j);
      const int ti3 = 2 + 3 * i;
      const uint32_t col0 = taddr + lg * g.Tp;
      // pass 1: every tangent row as o_t e (rows >= T padded with zeros); the
      // Laplacian row and electron i's own three gradient rows are rewritten
      // in pass 2 with their product-rule terms
      for (int q4 = 0; q4 < g.Tp / 4; ++q4) {
        float v[4];
        ptx::tmem_ld4(col0 + 4 * q4, v);
        if (!fok) continue;
        float* d4 = dst + (size_t)(4 * q4) * ts;
#pragma unroll
        for (int ee = 0; ee < 4; ++ee) d4[ee * ts] = (4 * q4 + ee < g.T) ? v[ee] * e[0] : 0.f;
      }
      // pass 2: value o_0 and Laplacian o_L (columns 0, 1) and o_c of the
      // gradient rows ti3 + c: grad row = o_c e + o_0 de_c,
      // Laplacian = o_L e + 2 sum_c o_c de_c + o_0 lap e
      float v01[4], oc[3];
      ptx::tmem_ld4_ld1x3(col0, col0 + ti3, col0 + ti3 + 1, col0 + ti3 + 2, v01, oc);
      if (fok) {
        const float o0 = v01[0], oL = v01[1];
        float cross = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          dst[(size_t)(ti3 + c) * ts] = fmaf(o0, e[1 + c], oc[c] * e[0]);
          cross = fmaf(oc[c], e[1 + c], cross);
        }
        dst[ts] = oL * e[0] + 2.0f * cross + o0 * e[4];
      }
    }
  }
};

// ------------------------------------------------------------ host side
int tc_padded_tangents(int T) {
  if (T <= 1) return 1;
  for (int Tp = (T + 3) / 4 * 4; Tp <= 256; Tp += 4)
    if (tc_groups_per_tile(Tp) > 0) return Tp;
  return -1;
}

// Pipeline stages that fit next to two epilogue staging buffers.
static int tc_stages_fitting(int n_cols, int ebuf_bytes) {
  const int stage_bytes = 2 * kATile + 2 * n_cols * kKChunk * 2;
  const long avail = 227L * 1024 - 1024 - 256 - 2L * ebuf_bytes - 64;
  return (int)std::min<long>(4, avail / stage_bytes);
}

// Epilogue staging bytes per half of a layer tile: four warps x two chunk
// buffers x [2 planes][16 rows][32 features] bf16, plus (tangent passes) two
// fp32 chunks [16][32] of the broadcast terms.
static int tc_layer_ebuf(int Tp) {
  const int per_warp = 2 * 2 * 16 * 32 * 2 + (Tp == 1 ? 0 : 2 * 16 * 32 * 4);
  return 4 * per_warp;
}

int tc_groups_per_tile(int Tp) {
  if (Tp == 1) return 128;  // value-only tiles: 128 rows, so short launches spread over all SMs
  for (int G = 256 / Tp; G >= 1; --G)
    if ((G * Tp) % 16 == 0 && tc_stages_fitting(G * Tp, tc_layer_ebuf(Tp)) >= 2) return G;
  return 0;
}

bool tc_layer_supported(int k1, int k2, int n_out) {
  return k1 % kKChunk == 0 && k2 > 0 && k2 <= 256 && n_out >= 16;
}

static PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 3-D map over two bf16 planes: dims (k_extent, rows, 2), box (64, box_rows, 1).
static qmc_status make_map(CUtensorMap* m, const void* base, int k_extent, size_t rows, int ld,
                           size_t plane, int box_rows) {
  auto enc = encoder();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled is unavailable");
    return QMC_ERR_UNSUPPORTED;
  }
  cuuint64_t dims[3] = {(cuuint64_t)k_extent, (cuuint64_t)rows, 2};
  cuuint64_t strides[2] = {(cuuint64_t)ld * 2, (cuuint64_t)plane * 2};
  cuuint32_t box[3] = {(cuuint32_t)kKChunk, (cuuint32_t)box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d): k=%d rows=%zu ld=%d plane=%zu box_rows=%d", (int)r,
              k_extent, rows, ld, plane, box_rows);
    return QMC_ERR_CUDA;
  }
  return QMC_OK;
}

// 4-D map over two bf16 planes of rows [walker][electron][ld] whose first
// electron row is `base`: dims (k_extent, ne, walkers, 2), box (64, ne,
// box_w, 1); a box lands in shared memory as box_w * ne consecutive rows.
static qmc_status make_map4(CUtensorMap* m, const void* base, int k_extent, int ne, size_t walkers, int ld, int n,
                            size_t plane, int box_w) {
  auto enc = encoder();
  if (!enc) {
    set_error("cuTensorMapEncodeTiled is unavailable");
    return QMC_ERR_UNSUPPORTED;
  }
  cuuint64_t dims[4] = {(cuuint64_t)k_extent, (cuuint64_t)ne, (cuuint64_t)walkers, 2};
  cuuint64_t strides[3] = {(cuuint64_t)ld * 2, (cuuint64_t)n * ld * 2, (cuuint64_t)plane * 2};
  cuuint32_t box[4] = {(cuuint32_t)kKChunk, (cuuint32_t)ne, (cuuint32_t)box_w, 1};
  cuuint32_t es[4] = {1, 1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled (4-D) failed (%d): k=%d ne=%d walkers=%zu box_w=%d", (int)r, k_extent, ne,
              walkers, box_w);
    return QMC_ERR_CUDA;
  }
  return QMC_OK;
}

static int tmem_cols_for(int n_cols) {
  int c = 32;
  while (c < n_cols) c <<= 1;
  return c;
}

template <class Epi>
static qmc_status launch(cudaStream_t s, const CUtensorMap& A0, const CUtensorMap& A1, const CUtensorMap& B1,
                         const CUtensorMap& B2, TcArgs g, int n_tiles, const Epi& epi) {
  if (n_tiles <= 0) return QMC_OK;
  const int stage_bytes = 2 * kATile + 2 * g.n_cols * kKChunk * 2;
  g.stages = tc_stages_fitting(g.n_cols, g.ebuf_bytes);
  if (g.stages < 2) {
    set_error("tile of %d columns does not fit two pipeline stages", g.n_cols);
    return QMC_ERR_SHAPE;
  }
  g.tmem_cols = 2 * tmem_cols_for(g.n_cols);  // two accumulators
  if (g.tmem_cols > 512) {
    set_error("tile of %d columns does not fit two TMEM accumulators", g.n_cols);
    return QMC_ERR_SHAPE;
  }
  g.n_tiles = n_tiles;
  g.n_mblocks = (g.n_out + 127) / 128;
  const size_t smem = 1024 + (size_t)g.stages * stage_bytes + 256 + 2 * (size_t)g.ebuf_bytes;
  // the opt-in attribute is per device and kernel; raise it to this launch's need
  static int attr_dev = -1;
  static size_t attr_bytes = 0;
  int dev;
  QMC_CUDA(cudaGetDevice(&dev));
  if (attr_dev != dev || attr_bytes < smem) {
    QMC_CUDA(cudaFuncSetAttribute(k_tc_gemm<Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_dev = dev;
    attr_bytes = smem;
  }
  static int n_sms = 0;
  if (!n_sms) QMC_CUDA(cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev));
  const int n_items = g.n_tiles * g.n_mblocks;
  k_tc_gemm<Epi><<<std::min(n_items, n_sms), kTcThreads, smem, s>>>(A0, A1, B1, B2, g, epi);
  QMC_CUDA(cudaGetLastError());
  return QMC_OK;
}

qmc_status tc_stream_layer(cudaStream_t s, const TcLayerArgs& a) {
  const int G = tc_groups_per_tile(a.Tp);
  const int c1 = (a.k1 + kKChunk - 1) / kKChunk, c2 = (a.k2 + kKChunk - 1) / kKChunk;
  // a first source narrower than whole chunks needs the chunk-padded weights;
  // rows of both sources are read with 16-byte aligned strides
  const bool shape_ok = a.w_ld ? (a.w_ld == kKChunk * (c1 + c2)) : tc_layer_supported(a.k1, a.k2, a.n_out);
  if (G <= 0 || !shape_ok || a.k1 % 8 || a.k2 % 8 || a.k2 <= 0 || a.k2 > 256 || a.n_out < 16) {
    set_error("tensor-core layer: unsupported shape (Tp=%d k1=%d k2=%d n_out=%d w_ld=%d)", a.Tp, a.k1, a.k2,
              a.n_out, a.w_ld);
    return QMC_ERR_SHAPE;
  }
  const size_t rows = (size_t)a.n_groups * a.Tp;
  TcArgs g{};
  g.G = G;
  g.Tp = a.Tp;
  g.T = a.T;
  g.n_cols = G * a.Tp;
  g.k1_chunks = c1;
  g.k_chunks = c1 + c2;
  g.n_out = a.n_out;
  g.err = a.err;
  CUtensorMap mA, mB1, mB2;
  const int kw = a.w_ld ? a.w_ld : a.k1 + a.k2;
  QMC_TRY(make_map(&mA, a.Wt, kw, a.n_out, kw, (size_t)a.n_out * kw, 128));
  QMC_TRY(make_map(&mB1, a.X, a.k1, rows, a.k1, a.x_plane, g.n_cols));
  QMC_TRY(make_map(&mB2, a.G2, a.k2, rows, a.k2, a.g2_plane, g.n_cols));
  if (a.residual && (a.k1 != a.n_out || a.k1 < 2 * kKChunk || a.n_out % 128)) {
    set_error("tensor-core layer: residual needs equal widths that are multiples of 128 (got %d -> %d)", a.k1,
              a.n_out);
    return QMC_ERR_SHAPE;
  }
  g.resid_last = 0;
  g.ebuf_bytes = tc_layer_ebuf(a.T == 1 ? 1 : a.Tp);
  if (a.n_out % 8) {
    set_error("tensor-core layer: output width %d is not a multiple of 8", a.n_out);
    return QMC_ERR_SHAPE;
  }
  auto fill = [&](auto& e) {
    e.n_groups = a.n_groups;
    e.n = a.n;
    e.ld = a.n_out;
    e.resid = StSplit{const_cast<__nv_bfloat16*>(a.X), a.k1, a.x_plane};
    e.out = StSplit{a.out, a.n_out, a.out_plane};
    e.Gb = a.Gb;
    e.bias = a.bias;
  };
  if (a.residual) {
    EpiTcLayer<true> e{};
    fill(e);
    return launch(s, mA, mA, mB1, mB2, g, (a.n_groups + G - 1) / G, e);
  }
  EpiTcLayer<false> e{};
  fill(e);
  return launch(s, mA, mA, mB1, mB2, g, (a.n_groups + G - 1) / G, e);
}

qmc_status tc_store_gemm(cudaStream_t s, const TcStoreArgs& a) {
  constexpr int kRows = 128;  // rows per tile
  TcArgs g{};
  g.G = kRows;
  g.Tp = 1;
  g.T = 1;
  g.n_cols = kRows;
  g.k1_chunks = (a.k + kKChunk - 1) / kKChunk;
  g.k_chunks = g.k1_chunks;
  g.n_out = a.n_out;
  g.err = a.err;
  CUtensorMap mA, mB;
  QMC_TRY(make_map(&mA, a.Wt, a.k, a.n_out, a.k, (size_t)a.n_out * a.k, 128));
  QMC_TRY(make_map(&mB, a.X, a.k, a.n_rows, a.k, a.x_plane, kRows));
  EpiTcStore e{};
  e.n_groups = a.n_rows;
  e.out = a.out;
  e.ld = a.ld_out > 0 ? a.ld_out : a.n_out;
  return launch(s, mA, mA, mB, mB, g, (a.n_rows + kRows - 1) / kRows, e);
}

qmc_status tc_orbitals(cudaStream_t s, const TcOrbitalArgs& a) {
  const int G = tc_groups_per_tile(a.Tp);
  if (G <= 0 || a.k % kKChunk) {
    set_error("tensor-core orbitals: unsupported shape (Tp=%d k=%d)", a.Tp, a.k);
    return QMC_ERR_SHAPE;
  }
  const size_t rows = (size_t)a.B * a.n * a.Tp;
  TcArgs g{};
  g.G = G;
  g.Tp = a.Tp;
  g.T = a.T;
  g.n_cols = a.T == 1 ? 256 : G * a.Tp;
  g.k1_chunks = a.k / kKChunk;
  g.k_chunks = g.k1_chunks;
  g.n_out = a.norb;
  g.err = a.err;
  CUtensorMap mA0, mA1, mB;
  QMC_TRY(make_map(&mA0, a.Wt[0], a.k, a.norb, a.k, (size_t)a.norb * a.k, 128));
  QMC_TRY(make_map(&mA1, a.split ? a.Wt[1] : a.Wt[0], a.k, a.norb, a.k, (size_t)a.norb * a.k, 128));
  QMC_TRY(make_map(&mB, a.X, a.k, rows, a.k, a.x_plane, g.n_cols));
  EpiTcOrbital e{};
  e.n = a.n;
  e.n_up = a.n_up;
  e.split = a.split;
  e.K = a.K;
  e.natom = a.natom;
  e.env_abs = a.env_abs;
  if (a.split) {
    e.tiles_up = (a.n_up + G - 1) / G;
    e.tiles_per_walker = e.tiles_up + (a.n - a.n_up + G - 1) / G;
  } else {
    e.tiles_up = (a.n + G - 1) / G;
    e.tiles_per_walker = e.tiles_up;
  }
  e.n_rows = a.B * a.n;
  const int n_tiles = a.T == 1 ? (a.split ? 2 : 1) * ((e.n_rows + 255) / 256) : a.B * e.tiles_per_walker;
  for (int c = 0; c < 2; ++c) {
    e.pi[c] = a.pi[a.split ? c : 0];
    e.sigma[c] = a.sigma[a.split ? c : 0];
  }
  e.rae = a.rae;
  e.aevec = a.aevec;
  e.A = a.A;
  e.raw = a.T == 1 ? a.raw : 0;
  e.unit_env = a.T == 1 ? 0 : a.unit_env;
  // value-only split orbitals: tiles of one channel's electrons only, N the
  // largest multiple of lcm(16, n_up, n_dn) up to 256
  const int nd = a.n - a.n_up;
  if (a.T == 1 && a.split && a.n_up > 0 && nd > 0) {
    auto gcd = [](int x, int y) { while (y) { const int t = x % y; x = y; y = t; } return x; };
    long L = 16;
    L = L / gcd((int)L, a.n_up) * a.n_up;
    L = L / gcd((int)L, nd) * nd;
    if (L <= 256) {
      const int N4 = (int)(256 / L * L);
      g.n_cols = N4;
      g.b4d = 1;
      e.chan4d = 1;
      e.B = a.B;
      e.W4[0] = N4 / a.n_up;
      e.W4[1] = N4 / nd;
      e.tpc4[0] = (a.B + e.W4[0] - 1) / e.W4[0];
      e.tpc4[1] = (a.B + e.W4[1] - 1) / e.W4[1];
      CUtensorMap m4u, m4d;
      QMC_TRY(make_map4(&m4u, a.X, a.k, a.n_up, a.B, a.k, a.n, a.x_plane, e.W4[0]));
      QMC_TRY(make_map4(&m4d, a.X + (size_t)a.n_up * a.k, a.k, nd, a.B, a.k, a.n, a.x_plane, e.W4[1]));
      return launch(s, mA0, mA1, m4u, m4d, g, e.tpc4[0] + e.tpc4[1], e);
    }
  }
  return launch(s, mA0, mA1, mB, mB, g, n_tiles, e);
}

}  // namespace qmc
