// Mixed-precision instantiation: FP32 reconstruction, characteristic
// projection and Riemann solve; FP64 flux accumulation, energy recovery
// and constrained-transport face update.
#include "hydro_launch.cuh"

size_t gb_hydro_scratch_bytes_mixed() { return gbh::scratch_layout<float>::bytes; }

int gb_hydro_chunk_mixed(const gbh::hydro_kparams& kp, int mhd, int cool, int nblk, const int* list,
                         void* scratch, gb_status* st, cudaStream_t s)
{
    return gbh::launch_chunk<float>(kp, mhd, cool, nblk, list, scratch, st, s);
}
