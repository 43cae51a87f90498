// Mixed-precision instantiation: FP32 reconstruction, characteristic
// projection and Riemann solve; FP64 flux accumulation, energy recovery
// and constrained-transport face update.
#include "hydro_launch.cuh"

size_t gb_hydro_scratch_bytes_mixed() { return gbh::scratch_layout<float>::bytes; }

int gb_hydro_chunk_mixed(const gbh::hydro_kparams& kp, int mhd, int cool, int nblk, const int* list,
                         void* scratch, gb_status* st, cudaStream_t s, cudaEvent_t ev_put,
                         const sur_feat_out* sf, cudaEvent_t ev_wait)
{
    return gbh::launch_chunk<float>(kp, mhd, cool, nblk, list, scratch, st, s, ev_put, sf, ev_wait);
}

// CFL limit of the mixed path: FP32 arithmetic on the FP64 state
int gb_dt_launch_f32(const gbh::hydro_kparams& kp, int mhd, int nblk, const int* list,
                     unsigned long long* bits, cudaStream_t s)
{
    dim3 g(4, nblk);
    gbh::k_dtlimit<float><<<g, 256, 0, s>>>(g_gb.grid, kp.gamma, mhd, kp.dx[0], kp.dx[1], kp.dx[2], list, bits,
                                            kp.cfl_sum, kp.cflc, kp.cflsc);
    return gb_check(cudaGetLastError(), "k_dtlimit<float>") ? GB_ERR_CUDA : GB_OK;
}
