// tcgen05 (5th-gen tensor core) BF16 path for the one-electron stream layers.
#pragma once
#include "common.cuh"

namespace qmc {

// Padded tangent count used by the tensor-core tiles.
int tc_padded_tangents(int T);
// Whether a layer with these padded widths runs on the tensor-core kernel.
bool tc_layer_supported(int k1, int k2, int n_out);
// z = [X | G2] W^T + Gb + b, tanh with tangent rules, optional residual.
qmc_status tc_stream_layer(cudaStream_t s, int n_groups, int n, int Tp, int T,
                           const __nv_bfloat16* X, int k1, const __nv_bfloat16* G2, int k2,
                           const __nv_bfloat16* Wt, int n_out, const float* Gb, const float* bias,
                           bool residual, __nv_bfloat16* out);

}  // namespace qmc
