#include <mutex>
#include <vector>

#include "profile.cuh"

namespace qmc {

namespace {
struct ProfState {
  std::mutex mu;
  bool on = false;
  std::vector<cudaEvent_t> pool;
  struct Rec { int cls; int ev0; };
  std::vector<Rec> recs;
  int64_t launches[QMC_KC_COUNT] = {};
};
ProfState& st() {
  static ProfState s;
  return s;
}
cudaEvent_t event_at(ProfState& p, int i) {
  while ((int)p.pool.size() <= i) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    p.pool.push_back(e);
  }
  return p.pool[i];
}
}  // namespace

ProfScope::ProfScope(int c, cudaStream_t str) : cls(c), s(str), slot(-1) {
  ProfState& p = st();
  if (!p.on) return;
  std::lock_guard<std::mutex> g(p.mu);
  p.launches[cls] += 1;
  int ev0 = (int)p.recs.size() * 2;
  cudaEvent_t e = event_at(p, ev0);
  if (!e || !event_at(p, ev0 + 1)) return;
  cudaEventRecord(e, s);
  p.recs.push_back({cls, ev0});
  slot = ev0;
}

ProfScope::~ProfScope() {
  if (slot < 0) return;
  ProfState& p = st();
  std::lock_guard<std::mutex> g(p.mu);
  cudaEventRecord(p.pool[slot + 1], s);
}

// FP32 FMA throughput probe: every thread runs kFmaChains independent
// dependent chains of `iters` FMAs (enough independent work to hide the FMA
// latency on each SM sub-partition), and writes one value so that nothing is
// eliminated.  Work per launch: blocks x 256 x kFmaChains x iters FMAs.
constexpr int kFmaChains = 8;
__global__ void __launch_bounds__(256) k_ffma_throughput(int iters, float b, float c, float* __restrict__ out) {
  float a[kFmaChains];
#pragma unroll
  for (int k = 0; k < kFmaChains; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
#pragma unroll
      for (int k = 0; k < kFmaChains; ++k) a[k] = fmaf(a[k], b, c);
    }
  }
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < kFmaChains; ++k) acc += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// Warp-level BF16 MMA throughput probe (mma.m16n8k16, FP32 accumulate):
// every warp runs kMmaChains independent accumulators; the operands are
// register constants, so only the tensor pipe is measured.  Work per launch:
// blocks x 8 warps x kMmaChains x iters MMAs of 2 x 16 x 8 x 16 FLOPs.
constexpr int kMmaChains = 8;
__global__ void __launch_bounds__(256) k_mma_throughput(int iters, float* __restrict__ out) {
  const uint32_t a0 = threadIdx.x * 0x00010001u, a1 = a0 ^ 0x3f803f80u, a2 = a0 + 1u, a3 = a1 + 1u;
  const uint32_t b0 = a0 ^ 0x40004000u, b1 = a1 ^ 0x3c003c00u;
  float d[kMmaChains][4] = {};
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kMmaChains; ++k)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
          "{%0, %1, %2, %3};\n"
          : "+f"(d[k][0]), "+f"(d[k][1]), "+f"(d[k][2]), "+f"(d[k][3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < kMmaChains; ++k) acc += d[k][0] + d[k][1] + d[k][2] + d[k][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace qmc

extern "C" {

qmc_status qmc_mma_throughput(int blocks, int iters, float* out, double* flop_per_launch, cudaStream_t stream) {
  if (blocks < 1 || iters < 1 || !out) {
    qmc::set_error("qmc_mma_throughput: blocks, iters >= 1 and an output of blocks x 256 floats");
    return QMC_ERR_ARG;
  }
  qmc::k_mma_throughput<<<blocks, 256, 0, stream>>>(iters, out);
  if (flop_per_launch)
    *flop_per_launch = (double)blocks * 8.0 * qmc::kMmaChains * (double)iters * (2.0 * 16 * 8 * 16);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? QMC_OK : qmc::cuda_status(e, "k_mma_throughput");
}

qmc_status qmc_ffma_throughput(int blocks, int iters, float* out, double* fma_per_launch, cudaStream_t stream) {
  if (blocks < 1 || iters < 1 || !out) {
    qmc::set_error("qmc_ffma_throughput: blocks, iters >= 1 and an output of blocks x 256 floats");
    return QMC_ERR_ARG;
  }
  qmc::k_ffma_throughput<<<blocks, 256, 0, stream>>>(iters, 0.999999f, 1e-7f, out);
  if (fma_per_launch) *fma_per_launch = (double)blocks * 256.0 * qmc::kFmaChains * 16.0 * (double)iters;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? QMC_OK : qmc::cuda_status(e, "k_ffma_throughput");
}

qmc_status qmc_profile_enable(int on) {
  qmc::ProfState& p = qmc::st();
  std::lock_guard<std::mutex> g(p.mu);
  p.on = on != 0;
  return QMC_OK;
}

qmc_status qmc_profile_read(int n_classes, int64_t* launches, double* ms) {
  qmc::ProfState& p = qmc::st();
  std::lock_guard<std::mutex> g(p.mu);
  double acc[QMC_KC_COUNT] = {};
  for (auto& r : p.recs) {
    cudaError_t e = cudaEventSynchronize(p.pool[r.ev0 + 1]);
    if (e != cudaSuccess) return qmc::cuda_status(e, "qmc_profile_read");
    float t = 0.f;
    e = cudaEventElapsedTime(&t, p.pool[r.ev0], p.pool[r.ev0 + 1]);
    if (e != cudaSuccess) return qmc::cuda_status(e, "qmc_profile_read");
    acc[r.cls] += t;
  }
  for (int c = 0; c < n_classes && c < QMC_KC_COUNT; ++c) {
    if (launches) launches[c] = p.launches[c];
    if (ms) ms[c] = acc[c];
  }
  p.recs.clear();
  for (auto& l : p.launches) l = 0;
  return QMC_OK;
}

}  // extern "C"
