// Host-side state of one gbhydro library instance (one registered grid,
// one parameter set). Internal header.
#pragma once

#include "cool_dev.cuh"
#include "gb_common.cuh"

struct gb_state_t {
    bool grid_ok = false;
    gb_grid_desc desc{};
    gb_dev_grid grid{};
    bool tree_ok = false;
    gb_tree_desc tree{};
    bool hydro_ok = false;
    gb_hydro_params hp{};
    bool cool_ok = false;
    gb_cool_ctx cool{};
    double* d_table = nullptr; // T axis, n axis, lambda (one allocation)
    // staging buffers reused across calls
    double* d_stage = nullptr;
    size_t stage_bytes = 0;
    void* d_scratch = nullptr;
    size_t scratch_bytes = 0;
    double* d_dtmin = nullptr;
    int* d_all_blocks = nullptr;
    int all_blocks_n = 0;
    // flux conservation at fine-coarse faces: face links (per store block
    // 6 x {type, 4 fine leaves}), boundary flux registers, level-sorted list
    bool fc_on = true;
    int* d_links = nullptr;
    int links_n = 0;
    bool links_ok = false;
    void* d_fcreg = nullptr;
    size_t fcreg_bytes = 0;
    int* d_fclist = nullptr;
    int fclist_cap = 0;
    // surface-edge electric-field registers (MHD): NSURF doubles per node
    double* d_ereg = nullptr;
    size_t ereg_bytes = 0;
    // guard-fill plan: the node covering each of the 27 regions around a
    // leaf (two int4 per entry)
    void* d_plan = nullptr;
    int plan_n = 0;
    bool plan_ok = false;
    // per-cell CFL codes of the interior cells (store block x 3 directions x
    // 4096 bytes): written by the reconstruction, read by the next CFL limit
    unsigned char* d_cflc = nullptr;
    size_t cflc_bytes = 0;
    // bumped by every call that changes what a captured step graph baked
    // in (grid, tree, parameters, tables, weights, modes)
    unsigned long long gen = 0;
};

extern gb_state_t g_gb;

// scratch allocation helper (grows, never shrinks)
int gb_ensure_scratch(size_t bytes);
int gb_ensure_stage(size_t bytes);

// kernels launched from other translation units
int gb_launch_cool_blocks(int nblk, const int* list, double dt, gb_status* st, cudaStream_t s);
int gb_launch_hydro(int nblk, const int* list, double dt, const double* dtp, int cool, gb_status* st,
                    cudaStream_t s);
int gb_launch_dt(int nblk, const int* list, double* dt_out, cudaStream_t s);
int gb_launch_guardfill(int nblk, const int* list, cudaStream_t s);
int gb_sur_prepare(int64_t ncell, cudaStream_t s);
int gb_guard_prepare(cudaStream_t s);
// launch shapes chosen by the autotuner (gb_set_launch_config)
int gb_chunk_blocks();
int gb_chunk_streams();
int gb_recon_tile();
int gb_recon_occupancy();
int gb_fused_step();
