// XLA FFI handlers exposing the GB300 library to JAX (jax.ffi.ffi_call).
//
// Built only where jaxlib's FFI headers exist (jaqmc_gb300/jax_ffi.py:build);
// neither environment this library is developed in has jax, so these handlers
// are UNTESTED.  Each handler forwards XLA's buffers and CUDA stream to the
// C ABI of include/qmc.h.  The model handle and its workspace are 64-bit
// attributes created on the Python side; the flat parameter vector is an input
// buffer, uploaded into the model's arena on the same stream before the work,
// so the data dependency orders parameter updates and evaluations.
#include <cstdint>

#include "qmc.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

static ffi::Error status_to_error(qmc_status s) {
  if (s == QMC_OK) return ffi::Error::Success();
  return ffi::Error(ffi::ErrorCode::kInternal, qmc_last_error());
}

static qmc_model* M(int64_t h) { return reinterpret_cast<qmc_model*>(h); }

// log|psi| and sign for a (B, n, 3) batch.
static ffi::Error Forward(cudaStream_t stream, int64_t model, int64_t workspace, int64_t workspace_bytes,
                          ffi::Buffer<ffi::F32> params, ffi::Buffer<ffi::F32> electrons,
                          ffi::ResultBuffer<ffi::F32> logpsi, ffi::ResultBuffer<ffi::F32> sign) {
  const int batch = static_cast<int>(electrons.dimensions()[0]);
  qmc_status s = qmc_model_set_params(M(model), params.typed_data(), stream);
  if (s != QMC_OK) return status_to_error(s);
  return status_to_error(qmc_forward(M(model), batch, electrons.typed_data(), logpsi->typed_data(),
                                     sign->typed_data(), nullptr, reinterpret_cast<void*>(workspace),
                                     static_cast<size_t>(workspace_bytes), stream));
}

XLA_FFI_DEFINE_HANDLER_SYMBOL(QmcForward, Forward,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("model")
                                  .Attr<int64_t>("workspace")
                                  .Attr<int64_t>("workspace_bytes")
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>());

// E_L, kinetic and potential energy per walker.
static ffi::Error LocalEnergy(cudaStream_t stream, int64_t model, int64_t workspace, int64_t workspace_bytes,
                              ffi::Buffer<ffi::F32> params, ffi::Buffer<ffi::F32> electrons,
                              ffi::ResultBuffer<ffi::F32> e_local, ffi::ResultBuffer<ffi::F32> kinetic,
                              ffi::ResultBuffer<ffi::F32> potential) {
  const int batch = static_cast<int>(electrons.dimensions()[0]);
  qmc_status s = qmc_model_set_params(M(model), params.typed_data(), stream);
  if (s != QMC_OK) return status_to_error(s);
  return status_to_error(qmc_local_energy(M(model), batch, electrons.typed_data(), e_local->typed_data(),
                                          kinetic->typed_data(), potential->typed_data(), nullptr, nullptr,
                                          reinterpret_cast<void*>(workspace), static_cast<size_t>(workspace_bytes),
                                          stream));
}

XLA_FFI_DEFINE_HANDLER_SYMBOL(QmcLocalEnergy, LocalEnergy,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("model")
                                  .Attr<int64_t>("workspace")
                                  .Attr<int64_t>("workspace_bytes")
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>());

// `steps` MH updates.  The Philox update index is a device buffer (u64[1]):
// the handler returns the walkers, 2 log|psi|, per-walker accept counts and
// the advanced index, so the counter is threaded like the reference's PRNG
// key and no attribute changes between steps (no recompilation).
static ffi::Error MhSteps(cudaStream_t stream, int64_t model, int64_t workspace, int64_t workspace_bytes,
                          int64_t steps, float stddev, int64_t seed, ffi::Buffer<ffi::F32> params,
                          ffi::Buffer<ffi::F32> electrons, ffi::Buffer<ffi::U64> counter,
                          ffi::ResultBuffer<ffi::F32> electrons_out, ffi::ResultBuffer<ffi::F32> log_prob,
                          ffi::ResultBuffer<ffi::U32> accepts, ffi::ResultBuffer<ffi::U64> counter_out) {
  const int batch = static_cast<int>(electrons.dimensions()[0]);
  qmc_status s = qmc_model_set_params(M(model), params.typed_data(), stream);
  if (s != QMC_OK) return status_to_error(s);
  cudaError_t e = cudaMemcpyAsync(electrons_out->typed_data(), electrons.typed_data(), electrons.size_bytes(),
                                  cudaMemcpyDeviceToDevice, stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(counter_out->typed_data(), counter.typed_data(), sizeof(uint64_t), cudaMemcpyDeviceToDevice,
                        stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(accepts->typed_data(), 0, sizeof(uint32_t) * batch, stream);
  if (e != cudaSuccess) return ffi::Error(ffi::ErrorCode::kInternal, cudaGetErrorString(e));
  return status_to_error(qmc_mh_steps_resident(M(model), batch, static_cast<int>(steps), stddev,
                                               static_cast<uint64_t>(seed), counter_out->typed_data(),
                                               electrons_out->typed_data(), log_prob->typed_data(),
                                               accepts->typed_data(), nullptr, reinterpret_cast<void*>(workspace),
                                               static_cast<size_t>(workspace_bytes), stream));
}

XLA_FFI_DEFINE_HANDLER_SYMBOL(QmcMhSteps, MhSteps,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("model")
                                  .Attr<int64_t>("workspace")
                                  .Attr<int64_t>("workspace_bytes")
                                  .Attr<int64_t>("steps")
                                  .Attr<float>("stddev")
                                  .Attr<int64_t>("seed")
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Arg<ffi::Buffer<ffi::U64>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>()
                                  .Ret<ffi::Buffer<ffi::U64>>());
