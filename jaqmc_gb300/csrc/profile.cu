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

}  // namespace qmc

extern "C" {

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
