// qmc_forward_noalloc: the forward pass with its scratch in a fixed device
// array owned by this library, for callers that must not allocate device
// memory while they run.
//
// Who needs it: code that evaluates log|psi| from inside a host callback or a
// plugin whose host framework forbids device allocation during execution (a
// custom call running inside another runtime's step, a real-time serving loop
// that pre-reserves all memory up front), and callers that cannot hold a
// workspace of their own across calls.  They still pass their own inputs and
// outputs; only the intermediate buffers come from the array below.
//
// Limits and behaviour:
//  * The array holds kNoAllocBytes (64 MiB).  A call whose forward pass needs
//    more (about 100 KB per walker for a 14-electron FermiNet of widths
//    256/32 and 16 determinants, i.e. roughly 650 such walkers) is rejected
//    with QMC_ERR_WORKSPACE before anything is launched.
//  * Every device that loads this part of the library keeps the 64 MiB
//    reserved until the process exits.
//  * All calls on a device share the one array and it keeps whatever the last
//    call left in it.  The forward pass writes every scratch element it reads
//    before reading it, so nothing has to be cleared between calls.  Calls whose
//    GPU work overlaps in time (different streams, or several host threads)
//    race on the array; serialise them.
//  * The first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current); make that first call
//    before any stream capture begins.  The address is kept for the life of
//    the process, so it is only valid while the CUDA context that first
//    resolved it lives: after cudaDeviceReset (or anything else that destroys
//    the device's primary context) do not call this entry point again in the
//    same process.
//  * FermiNet and Psiformer models are both served (the same forward pass as
//    qmc_forward for each); the batch limit depends on the model.
#include <mutex>

#include "plan.cuh"
#include "psiformer.cuh"

namespace qmc {

constexpr size_t kNoAllocBytes = 64ull << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device; the host-side symbol itself is not a device address).
static qmc_status noalloc_scratch(void** out) {
  int dev;
  QMC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device ordinal %d out of range for the built-in scratch", dev);
    return QMC_ERR_ARG;
  }
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(built-in scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return QMC_OK;
}

}  // namespace qmc

extern "C" qmc_status qmc_forward_noalloc(qmc_model* m, int batch, const float* electrons, float* logpsi,
                                          float* sign, uint8_t* flags, cudaStream_t stream) {
  using namespace qmc;
  // argument errors first, so that the size message below is only given when
  // the size is the cause
  if (!m) {
    set_error("null model");
    return QMC_ERR_ARG;
  }
  if (!m->params_set) {
    set_error("parameters not set (qmc_model_set_params)");
    return QMC_ERR_ARG;
  }
  if (batch < 1) {
    set_error("batch must be >= 1");
    return QMC_ERR_SHAPE;
  }
  if (!electrons || !logpsi) {
    set_error("null electrons/logpsi");
    return QMC_ERR_ARG;
  }
  int dev;
  QMC_CUDA(cudaGetDevice(&dev));
  if (dev != m->device) {
    set_error("model lives on device %d but device %d is current", m->device, dev);
    return QMC_ERR_ARG;
  }
  const bool psi = m->kind == QMC_KIND_PSIFORMER;
  const PsiPlan pp = psi ? psi_make_plan(m, batch) : PsiPlan{};
  const Plan p = psi ? pp.base : make_plan(m, QMC_OP_FORWARD, batch);
  if (p.total > kNoAllocBytes) {
    set_error("qmc_forward_noalloc: %d walkers need %zu bytes of scratch but the built-in array holds %zu; "
              "use a smaller batch or qmc_forward with a workspace",
              batch, p.total, kNoAllocBytes);
    return QMC_ERR_WORKSPACE;
  }
  void* ws = nullptr;
  QMC_TRY(noalloc_scratch(&ws));
  // the remaining shape checks of qmc_forward (mixed-form widths and the like)
  QMC_TRY(check_call(m, batch, ws, kNoAllocBytes, QMC_OP_FORWARD));
  if (psi) return psi_evaluate(m, pp, ws, electrons, logpsi, sign, flags, stream);
  return evaluate(m, p, ws, electrons, false, logpsi, sign, nullptr, nullptr, flags, stream);
}
