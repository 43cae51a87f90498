/*
 * gbhydro: C ABI of the GB300 (sm_103a) hydro/MHD + heating/cooling step.
 *
 * The library replaces, for one GPU, the per-step hot path that Torch's
 * patched FLASH 4.6.2 runs:
 *   Hydro(blockCount, blockList, timeEndAdv, dt, dtOld, sweepOrder)
 *     -> hy_uhd_unsplit(blockCount, blockList, dt, dtOld)
 *        (src/flash/source/physics/Hydro/HydroMain/unsplit/hy_uhd_interface.F90:472-479;
 *         called at src/flash/source/Driver/DriverMain/Unsplit/Couple_AMUSE/Driver_evolveFlash.F90:406)
 *   Heat(blockCount, blockList, dt, time) -> RadHeat(...)
 *        (src/flash/source/physics/sourceTerms/Heat/HeatMain/HeatCool/phenHeat/Heat_interface.F90:10-16;
 *         .../phenHeat/mol_and_dust/solver/RadHeat.F90:45)
 * Plain pointers and sizes only; every pointer to grid data is a device
 * pointer unless the name says _host. Calls are stream-ordered on the
 * stream given (NULL = the legacy default stream) and return a gb_rc;
 * kernel-side failures land in a device gb_status the caller reads after
 * synchronising (gb_status_read). No call traps, asserts or aborts.
 */
#ifndef GBHYDRO_H
#define GBHYDRO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- codes */
typedef enum gb_rc {
    GB_OK = 0,
    GB_ERR_ARG = -1,        /* bad argument (null pointer, size out of range) */
    GB_ERR_CUDA = -2,       /* a CUDA runtime call failed */
    GB_ERR_NOT_INIT = -3,   /* gb_cool_init / gb_register_grid not called */
    GB_ERR_TABLE = -4,      /* cooling table missing or malformed */
    GB_ERR_LIMIT = -5       /* request beyond a documented maximum */
} gb_rc;

/* kernel status codes (gb_status.code holds the first; n_code[c] counts
 * every cell that raised code c, so a later or rarer code is never hidden) */
enum {
    GB_ST_OK = 0,
    GB_ST_NEG_DENS = 1,     /* density <= 0 after the update */
    GB_ST_NEG_PRES = 2,     /* pressure floored */
    GB_ST_NONFINITE = 3,    /* NaN/Inf in the updated state */
    GB_ST_ZERO_UNBRACKETED = 4, /* Brent entered without a sign change (Fortran `stop`) */
    GB_ST_ZERO_MAXITER = 5, /* Brent iteration cap (Fortran `stop`) */
    GB_ST_OVERHEAT = 6,     /* T > absTmax clamped (RadHeat.F90:380-405) */
    GB_ST_TIMEOUT = 7       /* a bounded wait for a tensor-memory copy gave up */
};

/* Device-resident status word: the first failure plus counters. */
typedef struct gb_status {
    int code;
    int block, i, j, k;     /* where the first failure happened */
    int pad;
    double value;           /* offending value */
    unsigned long long n_fallback;     /* reconstruction fell back to first order */
    unsigned long long n_bracket_fail; /* zbrac gave up; absolute bracket used */
    unsigned long long n_dust_noconv;  /* dust Newton hit its cap */
    unsigned long long n_clamped;      /* T clamped at absTmax */
    unsigned long long n_eint_switch;  /* dual-energy switch chose the advected e_int */
    unsigned long long n_surrogate;    /* cells cooled by the learned surrogate */
    unsigned long long n_surrogate_reject; /* surrogate rejected -> plain integrator */
    unsigned long long n_code[8];      /* cells that raised each status code (index = code) */
    unsigned long long n_rh_fallback;  /* hybrid order: face states of a direction that failed
                                          the Rankine-Hugoniot check -> first order */
} gb_status;

/* ---------------------------------------------------------------- grid */
#define GB_NXB 16
#define GB_NGUARD 4
#define GB_NB (GB_NXB + 2 * GB_NGUARD) /* 24 */

/* cell-variable roles; gb_grid_desc.slot[] maps each to a store slot or -1 */
enum {
    GB_DENS = 0, GB_VELX, GB_VELY, GB_VELZ, GB_PRES, GB_ENER, GB_EINT,
    GB_MAGX, GB_MAGY, GB_MAGZ, GB_TEMP, GB_TDUS, GB_PHHE, GB_PEFL, GB_IHP,
    GB_NROLE
};

/* Store layout. Cells: unk[block][slot][k][j][i] with i fastest and
 * 24^3 padded cells per (block, slot). Faces (MHD):
 *   facex[block][k][j][i], i in 0..24 (face i = low face of cell i),
 *   facey[block][k][j][i], j in 0..24, facez[block][k][j][i], k in 0..24. */
typedef struct gb_grid_desc {
    int nvar;               /* slots per block */
    int maxblocks;
    int slot[GB_NROLE];
    double* unk;
    double* facex;
    double* facey;
    double* facez;
} gb_grid_desc;

/* Block tree for guard filling. Arrays of length nnodes (device pointers):
 * level (0 = root level), integer lower corner in units of that level's
 * block size, child node ids (8 per node, -1 for leaves; child c has
 * offset (c&1, (c>>1)&1, (c>>2)&1)), and the root-grid lookup
 * root[rx + nrx*(ry + nry*rz)] -> node id. Leaf blocks are addressed in
 * the store by their node id. The domain is periodic. */
typedef struct gb_tree_desc {
    int nnodes;
    int nrx, nry, nrz;      /* root grid in blocks */
    int maxlevel;
    const int* level;
    const int* coord;       /* 3 ints per node */
    const int* child;       /* 8 ints per node */
    const int* root;
    double xmin[3];
    double root_dx[3];      /* cell size at level 0 */
} gb_tree_desc;

int gb_register_grid(const gb_grid_desc* grid, const gb_tree_desc* tree);

/* Fill the guard cells (and guard faces) of the listed blocks from their
 * neighbours: same-level copy, injection from a coarser neighbour,
 * restriction (8-cell mean) from a finer one, periodic domain. The role
 * FLASH's Grid_fillGuardCells plays before Hydro
 * (src/flash/source/Driver/DriverMain/Unsplit/Couple_AMUSE/Driver_computeDt.F90:243).
 * Cell variables filled: the ones the step reads (DENS, VEL*, PRES, ENER,
 * EINT, MAG*), as FLASH's Hydro fills with a variable mask; other slots
 * (TEMP, TDUS, ...) keep their guard values. */
int gb_fill_guardcells(int blockCount, const int* blockList_dev, void* stream);

/* ---------------------------------------------------------------- hydro */
typedef struct gb_hydro_params {
    double gamma;
    double cfl;             /* flash.par.turbsph_standard:163 */
    double cvisc;           /* :198 */
    int use_avisc;          /* :197 */
    int mhd;                /* 0 = hydro HLLC, 1 = USM MHD HLLD + CT */
    double eint_switch;     /* :164 */
    double smlrho, smallp;  /* floors in grid units */
    int precision;          /* 0 = all FP64, 1 = FP32 reconstruction/Riemann, FP64 update */
    int energy_fix;         /* energyFix (:213): the gas energy is taken from the total
                               energy less the magnetic energy of the flux-updated cell
                               field; the stored field is the staggered faces' mean */
    int hybrid_order;       /* use_hybridOrder (:206): first-order face states where the
                               flow compresses and a reconstructed state fails the
                               Rankine-Hugoniot check (hy_uhd_dataReconstOneStep.F90:934-999,
                               :1150-1218) */
    int fallback_lower_cfl; /* hy_fallbackLowerCFL (:207) */
    double hybrid_kappa;    /* hy_hybridOrderKappa: compression threshold, in units of the
                               cell's fast speed (FLASH's default 0) */
    double cfl_fallback_factor; /* hy_cflFallbackFactor (:208) */
    int cfl_sum;            /* 1: the CFL limit of a cell is 1 / sum_d (|v_d| + c_f,d) / dx_d
                               (stable for the unsplit step, whose transverse terms vanish
                               on grid-scale modes); 0: min_d dx_d / (|v_d| + c_f,d) */
    int shock_detect;       /* shockDetect + shockLowerCFL (:225-226): cells of a strong
                               compressive shock take a lowered CFL in the next dt */
} gb_hydro_params;

int gb_hydro_init(const gb_hydro_params* p);

/* One unsplit step over blockCount leaf blocks (blockList: device int
 * array of store block ids, 0-based). Replaces hy_uhd_unsplit; dtOld is
 * accepted for signature parity and unused (as in the second-order
 * unsplit scheme). Guard cells must have been filled. st: device status.
 * The ids of this and every other device block list index the store
 * unchecked: each must name a leaf block below maxblocks, once, as the
 * leaf lists FLASH passes to Hydro do (the Python layer checks host lists
 * before it copies them). */
int gb_hydro_unsplit(int blockCount, const int* blockList_dev, double dt, double dtOld,
                     gb_status* st_dev, void* stream);

/* Allocation-free FP64 unsplit step (no counterpart in the reference).
 * For callers that cannot let the library allocate device memory: a host
 * that owns all device memory through its own pool, or a step loop that
 * must not call cudaMalloc because it can synchronise the whole device.
 * Runs the same plain FP64 kernels as gb_hydro_unsplit (no fused cooling,
 * whatever gb_hydro_params.precision says) with their scratch in a static
 * device array sized for GB_NOALLOC_MAX_BLOCKS blocks (about 3.9 MiB per
 * block, ~15.7 MiB held on every GPU that loads the library until exit).
 * blockCount above GB_NOALLOC_MAX_BLOCKS returns GB_ERR_LIMIT. The first
 * call on each device looks up the array's device address (make it before
 * any stream capture). Calls share the array: calls that overlap on the GPU
 * race. The profiler must be off. */
#define GB_NOALLOC_MAX_BLOCKS 4
int gb_hydro_unsplit_noalloc(int blockCount, const int* blockList_dev, double dt, double dtOld,
                             gb_status* st_dev, void* stream);

/* Per-cell CFL codes: every step's reconstruction records, for each
 * interior cell, whether its states fell back to first order (positivity,
 * or the hybrid-order Rankine-Hugoniot checks), and the next CFL limit
 * scales that cell's limit by the lowered CFL over cfl (0.9 / 3 or 0.25;
 * hy_uhd_dataReconstOneStep.F90:972, :1207-1216, :1240, the cellCfl
 * argument). gb_register_grid clears them; this clears them again (e.g.
 * after the caller restored an earlier state). */
int gb_cfl_codes_reset(void* stream);

/* Copy the registered grid's CFL codes (maxblocks x 3 x 16^3 bytes, an
 * opaque per-cell record) to or from a caller buffer in host or device
 * memory, stream-ordered: what a checkpoint keeps so that a restart takes
 * the same next dt as the uninterrupted run. nbytes must equal that size. */
int gb_cfl_codes_save(void* dst, size_t nbytes, void* stream);
int gb_cfl_codes_load(const void* src, size_t nbytes, void* stream);

/* Blocks per launch chunk of the hydro kernels (scratch = chunk x per-block
 * scratch; the autotuner picks it). Default 16. */
int gb_set_chunk_blocks(int n);

/* Launch shapes of the hydro step: blocks per chunk (the scratch of one
 * chunk is reused across chunks), cells per reconstruction CTA per
 * direction (32 or 64), and for the mixed path's reconstruction a register
 * bound for occupancy (0: unbounded; 1: 5 / 2 resident CTAs per SM for tile
 * 32 / 64, no spills; 2: 6 / 3, with some spilling). Chosen by
 * torch_gb300.autotune; no counterpart in the reference. */
int gb_set_launch_config(int chunk_blocks, int recon_tile, int recon_occupancy);
int gb_get_launch_config(int* chunk_blocks, int* recon_tile, int* recon_occupancy);

/* Reconstruction and Riemann solve as one kernel per block (1, 2) or as
 * two kernels over a chunk with the face states in between in device
 * memory (0, the default). The fused kernel keeps each plane's face states
 * in shared memory; in the mixed path mode 1 stages a rolling window of the
 * block's FP32 primitives with the tensor memory accelerator (one CTA per
 * SM), mode 2 reads them through L1 (no window: two CTAs per SM); the FP64
 * path reads its stencils from the store in both. The same arithmetic
 * either way; chosen by torch_gb300.autotune; no counterpart in the
 * reference. */
int gb_set_fused(int on);
int gb_get_fused(void);

/* Streams the chunks of a step run on (1 or 2). With 2, consecutive chunks
 * alternate between the caller's stream and a library stream, each with its
 * own scratch, so that one chunk's FP64-bound kernels overlap the next
 * chunk's FP32-bound ones; under flux conservation a chunk waits for the
 * previous chunk's flux registration. Results are bitwise those of 1
 * stream. Default 1; chosen by torch_gb300.autotune; no counterpart in the
 * reference. */
int gb_set_chunk_streams(int n);
int gb_get_chunk_streams(void);

/* CFL time step: writes cfl * min over interior cells of the listed blocks
 * of dx_d / (|v_d| + c_f,d) to *dt_dev (device double). The per-block
 * Hydro_computeDt + MPI_AllReduce(MINLOC) of
 * src/flash/source/Driver/DriverMain/Unsplit/Couple_AMUSE/Driver_computeDt.F90:327-335,514-515. */
int gb_compute_dt(int blockCount, const int* blockList_dev, double* dt_dev, void* stream);

/* ---------------------------------------------------------------- cooling */
typedef struct gb_cool_params {
    /* Heat_data / Cool_data runtime parameters (phenHeat/Config, mol_and_dust/Config) */
    double tradmin, tradmax, dradmin, dradmax;
    double theatmin, theatmax, absTmin, absTmax;
    double Gzero, subfactor, smallp;
    int use_cr_heating;
    double crIonRate, crIonNH, crIonExp, crIonEnergy;
    double dust_sputter_temp;
    int pe_recipe;          /* 0 WD01, 1 BT94, 2 NOGF */
    double pe_norm;
    double boltz, mp;
    double T_cool_min, nd_cool_min, nd_cool_max;
    int useDustCool;
    int int_method;         /* 0 Implicit (the only one on the GPU), 1 Euler */
    double mu_mol;          /* 24/11, RadHeat.F90:278 */
    double xHp_const;       /* ionisation fraction when the grid has no IHP slot */
    /* grid units -> CGS (1.0 when the grid is in CGS) */
    double dens_unit, vel_unit, time_unit;
    double eos_abar;        /* mean molecular weight of the Gamma EOS (T from e) */
} gb_cool_params;

/* Load cool.dat (FLASH format, get_cooling_data.F90:20-55) or the compact
 * int32 form, and set the parameters. Replaces Cool_init/Heat_init. */
int gb_cool_init(const char* cool_dat_path, const gb_cool_params* p);

/* Temperature floor of the implicit step's Brent tolerance, in kelvin.
 * heatCool.F90 stops Brent's method at max(TtoEI * 1 K, 1e-6 e_old), so
 * the default, 1.0, is the reference integrator; a smaller value solves the
 * same backward-Euler equation more tightly (a diagnostic: it measures how
 * far the reference's answer sits from the equation's root). No counterpart
 * in the reference's interface. */
int gb_set_brent_tolerance(double kelvin);

/* Per-cell heating/cooling over the interior of the listed blocks:
 * RadHeat.F90:179-457 with heating_and_cooling's "Implicit" branch
 * (heatCool.F90:216-514). Updates EINT, ENER, TEMP, TDUS (and PRES via the
 * Gamma EOS); zeroes PHHE/PEFL when present. */
int gb_heat(int blockCount, const int* blockList_dev, double dt, double time,
            gb_status* st_dev, void* stream);

/* The same per-cell solve on plain CGS arrays of n cells (no grid): ei,
 * temp, tdust updated in place; dens, xhp, phhe (erg/cm^3/s), gflux may be
 * NULL for defaults (xHp_const, 0, 0). */
int gb_cool_cells(int64_t n, const double* dens, double* ei, double* temp, double* tdust,
                  const double* xhp, const double* phhe, const double* gflux, double dt,
                  gb_status* st_dev, void* stream);

/* Formulation of the rate function (de/dt) that gb_cool_cells integrates:
 * 0 (default) = heatCool.F90's terms as written (a pow per power law),
 * 1 = the same terms with the transcendentals shared (one ln T and one
 * sqrt T per evaluation, x^a as exp(a ln x), the column density and the
 * FUV field's logarithm from per-cell constants), 2 = the terms evaluated
 * in FP32 (Brent's iterates stay FP64). The mixed hydro path's fused
 * cooling epilogue uses form 1, or form 2 under gb_set_cooling_mode(2);
 * the FP64 path's epilogue and gb_heat always use form 0. No counterpart
 * in the reference's interface. */
int gb_set_rate_form(int form);

/* ---------------------------------------------------------------- step */
/* One full step over the registered grid as FLASH's Driver_evolveFlash
 * runs it: guard fill, hydro (or MHD), then the cooling source term fused
 * into the update's epilogue when cool != 0. */
int gb_evolve_step(int blockCount, const int* blockList_dev, double dt, int cool,
                   gb_status* st_dev, void* stream);

/* Device-resident driver clock of a run (Driver_data's dr_simTime, dr_dt,
 * dr_dtOld, dr_tmax, dr_nstep), read and advanced by gb_step_graph. */
typedef struct gb_driver_state {
    double sim_time;  /* time at the start of the next step */
    double dt;        /* dt of the last step taken */
    double dt_old;    /* dt of the step before it (0: none yet) */
    double t_max;     /* the step that would pass t_max is shortened to end on it */
    double nstep;     /* steps taken */
} gb_driver_state;

/* Flux conservation at fine-coarse block faces (FLASH's flux_correct:
 * Grid_putFluxData / Grid_conserveFluxes / Grid_getFluxData around the
 * update in hy_uhd_unsplit; interface in Grid_interface.F90:132-135,460-468).
 * On by default; it applies when the registered tree has more than one
 * level: the listed leaves are stepped finest level first, a block next to
 * a coarser one registers its boundary fluxes of rho, rho v, E, rho e_int
 * and the face velocity, and a block next to finer ones replaces its
 * boundary fluxes by the mean of the 2 x 2 fine fluxes before its update.
 * Face B is not matched across levels (no edge-EMF averaging). The
 * allocation-free entry point does not apply it. */
int gb_set_flux_correction(int on);

/* Limits applied to every CFL time step, as Driver_computeDt.F90:588,596:
 * dt = min(dt, dt_old * change_factor) when dt_old > 0, then
 * dt = min(max(dt, dtmin), dtmax). Defaults 0, +inf, +inf (no limit);
 * flash.par.turbsph_standard:106-109 sets dtmin 3.15e7 s, dtmax 3.15e12 s,
 * tstep_change_factor 2 (pass them in code units). */
int gb_set_dt_limits(double dtmin, double dtmax, double change_factor);

/* The same step with dt on the device, as one CUDA graph: the CFL limit of
 * the listed blocks (CFL * min dx / (|v| + c_f), as gb_compute_dt), limited
 * as gb_set_dt_limits says and shortened to end on drv->t_max, is written
 * to drv->dt; then guard fill, hydro/MHD and (cool != 0) cooling run with
 * that dt, read by the kernels from drv; then drv advances (sim_time += dt,
 * dt_old = dt, nstep += 1). The host does not wait.
 * The graph is captured on the first call and replayed while the
 * arguments and the library's configuration (grid, parameters, cooling
 * mode, tables, surrogate weights, chunk size) stay the same; any change
 * re-captures it. blockList_dev, drv_dev and st_dev must stay valid while
 * the graph may run. Replaces the Driver_computeDt + Hydro + Heat sequence
 * of one FLASH step (Driver_evolveFlash.F90:405-408, Driver_sourceTerms.F90:67,
 * Driver_computeDt.F90:327-335,514-515), with dt computed at the start of
 * the step. Not re-entrant. */
int gb_step_graph(int blockCount, const int* blockList_dev, int cool, gb_driver_state* drv_dev,
                  gb_status* st_dev, void* stream);

/* The state of a FLASH host that keeps unk and facevar{x,y,z} in its own
 * (pinned) arrays: the interior transfers below in one argument. */
typedef struct gb_host_io {
    double* unk;                 /* unk(nunk, 24, 24, 24, blocks), variable fastest */
    int nunk;
    int host_slot[GB_NROLE];     /* index of role r in unk's variable axis, or -1 */
    double* facex;               /* facevar{x,y,z}; all NULL without face fields */
    double* facey;
    double* facez;
} gb_host_io;

/* gb_step_graph for a host-resident state: the same graph also uploads the
 * listed blocks' interiors from io (cells and owned faces) before the CFL
 * reduction, and downloads each chunk's interiors as soon as that chunk's
 * update and cooling are done, while later chunks compute (a chunk's blocks
 * are final then: later chunks read only their own blocks, guard copies and
 * the flux / edge registers). The host arrays' guard cells and guard faces
 * are neither read nor written. The arrays must be pinned and must not be
 * touched by the host while the graph may run. No counterpart in the
 * reference (FLASH's Grid keeps unk on the host and calls Hydro on it). */
int gb_step_graph_host(int blockCount, const int* blockList_dev, int cool, gb_driver_state* drv_dev,
                       gb_status* st_dev, const gb_host_io* io, void* stream);
/* Drops the captured step graph. */
int gb_graph_reset(void);
/* Number of captures and replays of the step graph so far, and the kernel
 * launches one replay of the current graph makes. */
int gb_graph_info(long long* captures, long long* launches, long long* kernel_nodes);

/* Host<->device copies of the whole store in FLASH's unk(NUNK, i, j, k,
 * blk) order (variable fastest), transposed on the device. nunk = number
 * of variables in the host array; host_slot[r] = index of role r in the
 * host's variable axis or -1. */
int gb_grid_upload_flash(const double* unk_host, int nunk, const int* host_slot, int nblocks,
                         void* stream);
int gb_grid_download_flash(double* unk_host, int nunk, const int* host_slot, int nblocks,
                           void* stream);

/* The same for the listed store blocks only (host list of 0-based store
 * ids, e.g. the leaf blocks FLASH passes to Hydro): block list[q] of the
 * host unk array <-> store block list[q]. Runs of consecutive ids move as
 * one copy. */
int gb_grid_upload_flash_list(const double* unk_host, int nunk, const int* host_slot, int blockCount,
                              const int* blockList_host, void* stream);
int gb_grid_download_flash_list(double* unk_host, int nunk, const int* host_slot, int blockCount,
                                const int* blockList_host, void* stream);

/* Face-centred B of the listed blocks in FLASH's facevar{x,y,z}(1, ...,
 * blk) order (one face variable: the same element order as the store's
 * face arrays, so no transpose). */
int gb_grid_upload_faces_list(const double* fx_host, const double* fy_host, const double* fz_host,
                              int blockCount, const int* blockList_host, void* stream);
int gb_grid_download_faces_list(double* fx_host, double* fy_host, double* fz_host, int blockCount,
                                const int* blockList_host, void* stream);

/* The same two transfers for the interiors only: the 16^3 interior cells
 * of each listed block, and the faces each block owns (4..20 along the
 * normal, 4..19 across). The step rebuilds guard cells and guard faces on
 * the device from the neighbours' interiors (as Grid_fillGuardCells does
 * before Hydro, Driver_computeDt.F90:243), so a host that keeps the state
 * in its FLASH arrays between steps moves 30 % of the bytes. The host
 * arrays keep the full FLASH shape; their guard cells and guard faces are
 * neither read nor written. Host arrays must be pinned (the kernels read
 * and write them in place); no counterpart in the reference. */
int gb_grid_upload_flash_interior_list(const double* unk_host, int nunk, const int* host_slot, int blockCount,
                                       const int* blockList_host, void* stream);
int gb_grid_download_flash_interior_list(double* unk_host, int nunk, const int* host_slot, int blockCount,
                                         const int* blockList_host, void* stream);
int gb_grid_upload_faces_interior_list(const double* fx_host, const double* fy_host, const double* fz_host,
                                       int blockCount, const int* blockList_host, void* stream);
int gb_grid_download_faces_interior_list(double* fx_host, double* fy_host, double* fz_host, int blockCount,
                                         const int* blockList_host, void* stream);

/* ---------------------------------------------------------------- surrogate */
/* Learned cooling surrogate (no counterpart in the reference): an MLP
 * 4 -> 64 -> 64 -> 64 -> 1 with SiLU, BF16 weights, FP32 accumulation.
 * Inputs per cell, normalised: log10 n [cm^-3], log10 T [K],
 * log10(dt / t_cool) with t_cool = e / |de/dt| of the plain integrator's
 * rate function, log10 G [G0] (FUV field). Output: (log10 T_new -
 * log10 T) / 4. Parameters are one flat FP32 vector: W1[64][4], b1[64],
 * W2[64][64], b2[64], W3[64][64], b3[64], W4[1][64], b4[1]. */
#define GB_MLP_IN 4
#define GB_MLP_HIDDEN 64
#define GB_MLP_NPARAM (64 * 4 + 64 + 64 * 64 + 64 + 64 * 64 + 64 + 64 + 1)

int gb_mlp_init_random(uint64_t seed);
int gb_mlp_set_weights(const float* host, int n);
int gb_mlp_get_weights(float* host, int n);
/* Loss and gradient of the mean squared error on n <= 2^20 device samples
 * (feat: n x 4, 16-byte aligned; target: n) into host buffers, from the
 * tensor-core training pass (BF16 inputs, activations and gradient
 * operands, FP32 accumulation). */
int gb_mlp_grad(const float* feat_dev, const float* target_dev, int n, float* grad_host, float* loss_host,
                void* stream);
/* Adam training on device samples: `steps` mini-batches of `batch` drawn on
 * the device with a seeded counter hash, each step one tensor-core
 * forward/backward kernel and one Adam kernel (no host synchronisation
 * between steps); per-step loss written to loss_host (may be NULL). */
int gb_mlp_train(const float* feat_dev, const float* target_dev, int64_t n, int steps, int batch, float lr,
                 uint64_t seed, float* loss_host, void* stream);
/* Inference on n cells (feat 16-byte aligned); tensor_cores = 1 uses the
 * tcgen05 path (BF16 operands, FP32 accumulators in tensor memory), 0 a
 * CUDA-core FP32 reference with the same BF16-rounded weights. */
int gb_mlp_infer(int64_t n, const float* feat_dev, float* y_dev, int tensor_cores, void* stream);
/* Training samples from the plain implicit integrator: log n ~ U[-2, 6],
 * log T ~ U[1, 8], log(dt/t_cool) ~ U[-3, 3], log G ~ U[-1, 1]; writes
 * normalised features (n x 4) and targets (n); rows where the root finder
 * failed get target NaN. */
int gb_surrogate_samples(int64_t n, uint64_t seed, float* feat_dev, float* target_dev, gb_status* st_dev,
                         void* stream);
/* Cooling mode of gb_evolve_step(cool = 1): 0 = plain integrator fused in
 * the update, 1 = surrogate with per-cell acceptance test and plain
 * fallback, 2 = the plain integrator, as a pass of its own after the
 * update, with its rate function de/dt evaluated in FP32 (the mixed path; Brent's and the
 * bracket search's iterates and the residual stay FP64; the FP64 path
 * keeps its reference rates in every mode but 1). The network's prediction starts at most four FP32 secant-Newton
 * iterations on the backward-Euler residual; a cell is accepted when a
 * correction below rel_tol * e came from a local slope and the energy
 * moved the way the initial rate points. check_fp64 = 1 re-evaluates the
 * residual in FP64 at the converged state before accepting. */
int gb_set_cooling_mode(int mode, double rel_tol, int check_fp64);

/* ---------------------------------------------------------------- profiling */
/* Per-kernel CUDA-event timing on the launching stream (no counterpart in
 * the reference; FLASH's Timers_start/stop play this role). While enabled
 * every launch records an event pair; gb_prof_read synchronises and
 * returns per-kernel-group milliseconds and launch counts in the order
 * guard, recon, flux, emf, faceb, update, dt, heat, surrogate features,
 * mlp, surrogate accept, surrogate fallback, layout copies (n >= 13). */
int gb_prof_enable(int on);
int gb_prof_read(double* ms, long long* launches, int n);

/* Self-check of the bounded waits in the tcgen05 and TMA kernels: one
 * thread waits, for at most limit_cycles (1e3 .. 4e9) SM cycles, on an
 * mbarrier that nothing arrives on (arrive = 0) or on one it arrived on
 * itself (arrive = 1). *result_host: 1 the wait completed, 2 it gave up and
 * recorded GB_ST_TIMEOUT in st (may be NULL). Nothing is left in flight, so
 * the context stays usable. */
int gb_check_bounded_wait(long long limit_cycles, int arrive, gb_status* st, int* result_host, void* stream);
/* Measured FP64 FMA throughput of the current GPU in TFLOP/s (2 flops per
 * FMA; a few milliseconds of independent FMA chains on every SM): the
 * denominator of the FP64-pipe roofline. */
int gb_measure_fp64_peak(double* tflops);
/* The same for FP32 FMA (the denominator of the mixed path's FP32 work). */
int gb_measure_fp32_peak(double* tflops);

/* Self-check of the mixed path's integer-pipe FP64 <-> FP32 conversions
 * against the hardware conversions: for the n device values, counts into
 * mismatches_dev[0] the doubles whose float differs and into [1] the floats
 * whose double differs (NaN payloads aside). No counterpart in the
 * reference. */
int gb_selfcheck_conversions(int64_t n, const double* d_dev, const float* f_dev,
                             unsigned long long* mismatches_dev, void* stream);

/* ---------------------------------------------------------------- misc */
int gb_status_reset(gb_status* st_dev, void* stream);
int gb_status_read(const gb_status* st_dev, gb_status* st_host);
const char* gb_last_error(void);
int gb_version(void);

#ifdef __cplusplus
}
#endif
#endif
