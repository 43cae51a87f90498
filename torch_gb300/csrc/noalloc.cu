// Allocation-free variant of the plain FP64 unsplit step.
//
// Some callers cannot let this library call cudaMalloc: a Fortran or C
// host that hands all device memory out of its own pool and forbids other
// allocations, or a time-stepping loop that must not call cudaMalloc
// because it can synchronise the whole device and stall every other
// stream. For them gb_hydro_unsplit_noalloc runs the same FP64 kernels as
// gb_hydro_unsplit (precision 0, no fused cooling) with their scratch in a
// file-scope device array of GB_NOALLOC_MAX_BLOCKS blocks' worth, which
// every GPU that loads the library holds until the process exits.
//
// Host code must not pass the array's name to a kernel: on the host it is
// only a stand-in symbol, not a device address. The first call on each
// device (with that device current) looks the address up with
// cudaGetSymbolAddress and caches it; make that first call before any
// stream capture. All calls share the one array and it keeps the previous
// call's contents; nothing in it has to start at zero because each kernel
// reads only regions an earlier kernel of the same call wrote. Calls that
// overlap on the GPU (two streams, two host threads) race on the array.
// Compiled with -fmad=false, as the allocating FP64 path.
#include <atomic>

#include "hydro_launch.cuh"

namespace {

constexpr size_t kBlockBytes = gbh::scratch_layout<double>::bytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_MAX_BLOCKS * kBlockBytes];

constexpr int kMaxDevices = 64;
// looked up once per device; threads that race on the first call store the
// same address (atomics keep that free of a data race)
std::atomic<void*> g_scratch_addr[kMaxDevices];

// per-device set-up: the device address of the static scratch array
int scratch_for_current_device(void** out)
{
    int dev = -1;
    if (gb_check(cudaGetDevice(&dev), "cudaGetDevice")) return GB_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) {
        gb_set_error("gb_hydro_unsplit_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
        return GB_ERR_LIMIT;
    }
    void* p = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (!p) {
        if (gb_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(noalloc scratch)"))
            return GB_ERR_CUDA;
        g_scratch_addr[dev].store(p, std::memory_order_release);
    }
    *out = p;
    return GB_OK;
}

}  // namespace

int gb_prof_is_on();

extern "C" int gb_hydro_unsplit_noalloc(int blockCount, const int* blockList_dev, double dt, double dtOld,
                                        gb_status* st_dev, void* stream)
{
    (void)dtOld;
    if (!g_gb.grid_ok || !g_gb.hydro_ok) {
        gb_set_error("gb_hydro_unsplit_noalloc: call gb_register_grid and gb_hydro_init first");
        return GB_ERR_NOT_INIT;
    }
    if (blockCount < 0 || blockCount > GB_NOALLOC_MAX_BLOCKS) {
        gb_set_error("gb_hydro_unsplit_noalloc: blockCount %d outside 0..%d (the static scratch holds %d blocks)",
                     blockCount, GB_NOALLOC_MAX_BLOCKS, GB_NOALLOC_MAX_BLOCKS);
        return GB_ERR_LIMIT;
    }
    if ((blockCount > 0 && !blockList_dev) || !(dt > 0.0)) {
        gb_set_error("gb_hydro_unsplit_noalloc: bad block list or dt = %g", dt);
        return GB_ERR_ARG;
    }
    if (g_gb.hp.mhd && (!g_gb.grid.f[0] || !g_gb.grid.f[1] || !g_gb.grid.f[2] || g_gb.grid.slot[GB_MAGX] < 0 ||
                        g_gb.grid.slot[GB_MAGY] < 0 || g_gb.grid.slot[GB_MAGZ] < 0)) {
        gb_set_error("gb_hydro_unsplit_noalloc: MHD needs face fields and MAG slots");
        return GB_ERR_ARG;
    }
    if (gb_prof_is_on()) {
        gb_set_error("gb_hydro_unsplit_noalloc: disable the profiler first (it creates CUDA events)");
        return GB_ERR_ARG;
    }
    if (blockCount == 0) return GB_OK;
    void* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    // the allocating entry point's parameters; no flux registers (they
    // would need allocation)
    gbh::hydro_kparams kp = gb_make_kp(dt, nullptr);
    kp.fc_links = nullptr;
    kp.fc_reg = nullptr;
    kp.ec_reg = nullptr;
    return gbh::launch_chunk<double>(kp, g_gb.hp.mhd, 0, blockCount, blockList_dev, scratch, st_dev,
                                     (cudaStream_t)stream);
}
