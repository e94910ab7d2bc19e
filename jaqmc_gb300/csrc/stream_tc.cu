#include "stream_tc.cuh"

namespace qmc {
int tc_padded_tangents(int T) { return T; }
bool tc_layer_supported(int, int, int) { return false; }
qmc_status tc_stream_layer(cudaStream_t, int, int, int, int, const __nv_bfloat16*, int,
                           const __nv_bfloat16*, int, const __nv_bfloat16*, int, const float*,
                           const float*, bool, __nv_bfloat16*) {
  set_error("tensor-core stream layer not built");
  return QMC_ERR_UNSUPPORTED;
}
}  // namespace qmc
