// Plain FP64 instantiation of the unsplit step (compiled with -fmad=false
// so its rounding matches the CPU oracle operation by operation).
#include "hydro_launch.cuh"

size_t gb_hydro_scratch_bytes_fp64() { return gbh::scratch_layout<double>::bytes; }

int gb_fused_attr_fp64() { return gbh::fused_set_attr<double>(); }

int gb_hydro_chunk_fp64(const gbh::hydro_kparams& kp, int mhd, int cool, int nblk, const int* list,
                        void* scratch, gb_status* st, cudaStream_t s, cudaEvent_t ev_put,
                         const sur_feat_out* sf, cudaEvent_t ev_wait)
{
    return gbh::launch_chunk<double>(kp, mhd, cool, nblk, list, scratch, st, s, ev_put, sf, ev_wait);
}

int gb_dt_launch_f32(const gbh::hydro_kparams& kp, int mhd, int nblk, const int* list,
                     unsigned long long* bits, cudaStream_t s);

int gb_dt_launch(const gbh::hydro_kparams& kp, int mhd, int nblk, const int* list,
                 unsigned long long* bits, cudaStream_t s)
{
    dim3 g(4, nblk);
    if (g_gb.hp.precision == 1)
        return gb_dt_launch_f32(kp, mhd, nblk, list, bits, s);
    gbh::k_dtlimit<double><<<g, 256, 0, s>>>(g_gb.grid, kp.gamma, mhd, kp.dx[0], kp.dx[1], kp.dx[2], list, bits,
                                            kp.cfl_sum, kp.cflc, kp.cflsc);
    return gb_check(cudaGetLastError(), "k_dtlimit") ? GB_ERR_CUDA : GB_OK;
}
