// XLA FFI handlers exposing the GB300 library to JAX (jax.ffi.ffi_call).
//
// Built only where jaxlib's FFI headers exist (jaqmc_gb300/jax_ffi.py:build);
// neither environment this library is developed in has jax, so these handlers
// are UNTESTED.  Each handler forwards XLA's buffers and CUDA stream to the
// C ABI of include/qmc.h; the model handle and its workspace are passed as
// 64-bit attributes created on the Python side.
#include <cstdint>

#include "qmc.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

static ffi::Error status_to_error(qmc_status s) {
  if (s == QMC_OK) return ffi::Error::Success();
  return ffi::Error(ffi::ErrorCode::kInternal, qmc_last_error());
}

// log|psi| and sign for a (B, n, 3) batch.
static ffi::Error Forward(cudaStream_t stream, int64_t model, int64_t workspace, int64_t workspace_bytes,
                          ffi::Buffer<ffi::F32> electrons, ffi::ResultBuffer<ffi::F32> logpsi,
                          ffi::ResultBuffer<ffi::F32> sign) {
  const int batch = static_cast<int>(electrons.dimensions()[0]);
  return status_to_error(qmc_forward(reinterpret_cast<qmc_model*>(model), batch, electrons.typed_data(),
                                     logpsi->typed_data(), sign->typed_data(), nullptr,
                                     reinterpret_cast<void*>(workspace), static_cast<size_t>(workspace_bytes),
                                     stream));
}

XLA_FFI_DEFINE_HANDLER_SYMBOL(QmcForward, Forward,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("model")
                                  .Attr<int64_t>("workspace")
                                  .Attr<int64_t>("workspace_bytes")
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>());

// Local energy, kinetic and potential parts per walker.
static ffi::Error LocalEnergy(cudaStream_t stream, int64_t model, int64_t workspace, int64_t workspace_bytes,
                              ffi::Buffer<ffi::F32> electrons, ffi::ResultBuffer<ffi::F32> e_local,
                              ffi::ResultBuffer<ffi::F32> kinetic, ffi::ResultBuffer<ffi::F32> potential) {
  const int batch = static_cast<int>(electrons.dimensions()[0]);
  return status_to_error(qmc_local_energy(reinterpret_cast<qmc_model*>(model), batch, electrons.typed_data(),
                                          e_local->typed_data(), kinetic->typed_data(), potential->typed_data(),
                                          nullptr, nullptr, reinterpret_cast<void*>(workspace),
                                          static_cast<size_t>(workspace_bytes), stream));
}

XLA_FFI_DEFINE_HANDLER_SYMBOL(QmcLocalEnergy, LocalEnergy,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Attr<int64_t>("model")
                                  .Attr<int64_t>("workspace")
                                  .Attr<int64_t>("workspace_bytes")
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>());

// `steps` MH updates: electrons (in/out), log_prob (out), accepts (out).
static ffi::Error MhSteps(cudaStream_t stream, int64_t model, int64_t workspace, int64_t workspace_bytes,
                          int64_t steps, float stddev, int64_t seed, int64_t counter, ffi::Buffer<ffi::F32> electrons,
                          ffi::ResultBuffer<ffi::F32> electrons_out, ffi::ResultBuffer<ffi::F32> log_prob,
                          ffi::ResultBuffer<ffi::U32> accepts) {
  const int batch = static_cast<int>(electrons.dimensions()[0]);
  cudaError_t e = cudaMemcpyAsync(electrons_out->typed_data(), electrons.typed_data(),
                                  electrons.size_bytes(), cudaMemcpyDeviceToDevice, stream);
  if (e != cudaSuccess) return ffi::Error(ffi::ErrorCode::kInternal, cudaGetErrorString(e));
  e = cudaMemsetAsync(accepts->typed_data(), 0, sizeof(uint32_t) * batch, stream);
  if (e != cudaSuccess) return ffi::Error(ffi::ErrorCode::kInternal, cudaGetErrorString(e));
  return status_to_error(qmc_mh_steps(reinterpret_cast<qmc_model*>(model), batch, static_cast<int>(steps), stddev,
                                      static_cast<uint64_t>(seed), static_cast<uint64_t>(counter),
                                      electrons_out->typed_data(), log_prob->typed_data(), accepts->typed_data(),
                                      nullptr, nullptr, nullptr, reinterpret_cast<void*>(workspace),
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
                                  .Attr<int64_t>("counter")
                                  .Arg<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::F32>>()
                                  .Ret<ffi::Buffer<ffi::U32>>());
