// Internal interface of the learned cooling surrogate (mlp.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbhydro.h"

// pack the FP32 master weights into the BF16 tensor-core layout (once per
// weight update) and run inference y[i] = net(feat[4 i .. 4 i + 3])
int gb_mlp_pack(cudaStream_t s);
int gb_mlp_launch_infer(int64_t n, const float* feat, float* y, gb_status* st, cudaStream_t s);
