// Per-kernel CUDA-event timing recorded on the launching stream.
#pragma once

#include <cuda_runtime.h>

enum {
    GBP_GUARD = 0, GBP_RECON, GBP_FLUX, GBP_EMF, GBP_FACEB, GBP_UPDATE, GBP_DT, GBP_HEAT,
    GBP_SUR_FEAT, GBP_MLP, GBP_SUR_ACCEPT, GBP_SUR_FALLBACK, GBP_COPY, GBP_N
};

void gb_prof_begin(int id, cudaStream_t s);
void gb_prof_end(int id, cudaStream_t s);
