// Mixed-precision instantiation: FP32 reconstruction, characteristic
// projection and Riemann solve; FP64 flux accumulation, energy recovery
// and constrained-transport face update.
#include <cudaTypedefs.h>

#include "hydro_launch.cuh"

size_t gb_hydro_scratch_bytes_mixed() { return gbh::scratch_layout<float>::bytes; }

int gb_fused_attr_mixed() { return gbh::fused_set_attr<float>(); }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// the chunk's FP32 copies: x (24, fastest), y (24), z (24), variable (9),
// block (nblk); the box is one plane of all nine variables of one block
// (x extent 24 floats = 96 bytes, a multiple of 16; every copy starts at
// x = 0)
int gb_encode_p32_map(CUtensorMap* map, const float* p32, int nblk, size_t stride_floats)
{
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) {
        gb_set_error("cuTensorMapEncodeTiled not available");
        return GB_ERR_CUDA;
    }
    const cuuint64_t dims[5] = {(cuuint64_t)GB_N, (cuuint64_t)GB_N, (cuuint64_t)GB_N, (cuuint64_t)gbh::NP32,
                                (cuuint64_t)nblk};
    const cuuint64_t strides[4] = {(cuuint64_t)GB_N * 4, (cuuint64_t)GB_N * GB_N * 4, (cuuint64_t)GB_N3 * 4,
                                   (cuuint64_t)stride_floats * 4};
    const cuuint32_t box[5] = {(cuuint32_t)GB_N, (cuuint32_t)GB_N, 1u, (cuuint32_t)gbh::NP32, 1u};
    const cuuint32_t estr[5] = {1u, 1u, 1u, 1u, 1u};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, (void*)p32, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        gb_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return GB_ERR_CUDA;
    }
    return GB_OK;
}

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
