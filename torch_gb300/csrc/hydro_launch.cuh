// Launch sequence of one unsplit step over a chunk of blocks for one
// reconstruction precision T. Included by hydro_fp64.cu (T = double,
// compiled with -fmad=false) and hydro_mixed.cu (T = float).
#pragma once

#include "gb_prof.h"
#include "gb_state.h"
#include "hydro_dev.cuh"
#include "hydro_fused.cuh"

namespace gbh {

// reconstruction at the tuned shape: tile 32 or 64, and in the mixed path a
// register bound for occupancy: 0 unbounded, 1 the bound that still avoids
// spills (5 / 2 resident CTAs per SM for tile 32 / 64), 2 a tighter one
// that spills (6 / 3)
template <typename T, bool MHD>
void launch_recon(int tile, dim3 rg, cudaStream_t s, const gb_dev_grid& g, const hydro_kparams& kp, const int* list,
                  T* rscr, const float* p32, gb_status* st)
{
    using SL = scratch_layout<T>;
    const int occ = std::is_same<T, float>::value ? gb_recon_occupancy() : 0;
    if (tile == 64) {
        if (occ == 2) k_recon<T, MHD, 64, 3><<<rg, 3 * 64, 0, s>>>(g, kp, list, rscr, SL::recon, p32, SL::prim32, st);
        else if (occ == 1) k_recon<T, MHD, 64, 2><<<rg, 3 * 64, 0, s>>>(g, kp, list, rscr, SL::recon, p32, SL::prim32, st);
        else k_recon<T, MHD, 64, 1><<<rg, 3 * 64, 0, s>>>(g, kp, list, rscr, SL::recon, p32, SL::prim32, st);
    } else {
        if (occ == 2) k_recon<T, MHD, 32, 6><<<rg, 3 * 32, 0, s>>>(g, kp, list, rscr, SL::recon, p32, SL::prim32, st);
        else if (occ == 1) k_recon<T, MHD, 32, 5><<<rg, 3 * 32, 0, s>>>(g, kp, list, rscr, SL::recon, p32, SL::prim32, st);
        else k_recon<T, MHD, 32, 1><<<rg, 3 * 32, 0, s>>>(g, kp, list, rscr, SL::recon, p32, SL::prim32, st);
    }
}

// the fused kernels' dynamic shared memory limit (both physics)
template <typename T>
int fused_set_attr()
{
    constexpr bool TMA = std::is_same<T, float>::value;
    const int bytes = (int)fused_layout<T, TMA>::bytes;
    if (gb_check(cudaFuncSetAttribute(k_recon_flux<T, true, TMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
                 "fused kernel shared memory") ||
        gb_check(cudaFuncSetAttribute(k_recon_flux<T, false, TMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
                 "fused kernel shared memory"))
        return GB_ERR_CUDA;
    if constexpr (TMA) {
        // mode 2: the mixed kernel without the window
        const int b2 = (int)fused_layout<T, false>::bytes;
        if (gb_check(cudaFuncSetAttribute(k_recon_flux<T, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b2),
                     "fused kernel shared memory") ||
            gb_check(cudaFuncSetAttribute(k_recon_flux<T, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b2),
                     "fused kernel shared memory"))
            return GB_ERR_CUDA;
    }
    return GB_OK;
}

// reconstruction then fluxes: fused per block, or the two chunk kernels
template <typename T, bool MHD>
int recon_and_flux(int tile, dim3 rg, dim3 fg, cudaStream_t s, const gb_dev_grid& g, const hydro_kparams& kp, int nblk,
                   const int* list, T* rscr, T* fscr, float* p32, gb_status* st)
{
    using SL = scratch_layout<T>;
    if (const int fm = gb_fused_step()) {
        constexpr bool TMA = std::is_same<T, float>::value;
        CUtensorMap tm;
        memset(&tm, 0, sizeof tm);
        gb_prof_begin(GBP_RECON, s);
        if (TMA && fm == 2) {
            // mixed path without the window: stencils through L1
            k_recon_flux<T, MHD, false><<<nblk, FUSED_THREADS, fused_layout<T, false>::bytes, s>>>(
                g, kp, list, fscr, SL::flux, p32, SL::prim32, tm, st);
        } else {
            if constexpr (TMA) {
                if (gb_encode_p32_map(&tm, p32, nblk, SL::prim32)) return GB_ERR_CUDA;
            }
            k_recon_flux<T, MHD, TMA><<<nblk, FUSED_THREADS, fused_layout<T, TMA>::bytes, s>>>(
                g, kp, list, fscr, SL::flux, p32, SL::prim32, tm, st);
        }
        gb_prof_end(GBP_RECON, s);
        return GB_OK;
    }
    gb_prof_begin(GBP_RECON, s);
    launch_recon<T, MHD>(tile, rg, s, g, kp, list, rscr, p32, st);
    gb_prof_end(GBP_RECON, s);
    gb_prof_begin(GBP_FLUX, s);
    k_flux<T, MHD><<<fg, 128, 0, s>>>(g, kp, list, rscr, SL::recon, fscr, SL::flux, p32, SL::prim32);
    gb_prof_end(GBP_FLUX, s);
    return GB_OK;
}

// fine-side boundary fluxes into the flux registers (as soon as the fluxes
// exist)
template <typename T>
void put_fluxes(const hydro_kparams& kp, int nblk, const int* list, T* fscr, cudaStream_t s)
{
    using SL = scratch_layout<T>;
    if (kp.fc_links) {
        dim3 rg2(1, 6, nblk);
        k_fc_put<T><<<rg2, GB_NXB * GB_NXB, 0, s>>>(list, kp.fc_links, (T*)kp.fc_reg, fscr, SL::flux);
    }
}

template <typename T>
int launch_chunk(const hydro_kparams& kp_in, int mhd, int cool, int nblk, const int* list,
                 void* scratch, gb_status* st, cudaStream_t s, cudaEvent_t ev_put = nullptr,
                 const sur_feat_out* sf = nullptr, cudaEvent_t ev_wait = nullptr)
{
    using SL = scratch_layout<T>;
    // scratch of the chunk: [recon | flux | emf | faceb | prim32 | divu |
    // ecc | edgen], each block-major
    char* base = (char*)scratch;
    T* rscr = (T*)base;
    T* fscr = (T*)(base + (size_t)nblk * SL::recon * sizeof(T));
    double* escr = (double*)(base + (size_t)nblk * (SL::recon + SL::flux) * sizeof(T));
    double* bscr = escr + (size_t)nblk * SL::emf;
    float* p32 = (float*)(bscr + (size_t)nblk * SL::fb);
    T* dscr = (T*)(p32 + (size_t)nblk * SL::prim32);
    T* cscr = dscr + (size_t)nblk * SL::divu;
    T* nscr = cscr + (size_t)nblk * SL::ecc;
    hydro_kparams kp = kp_in;
    kp.divu = dscr;
    kp.ecc = cscr;
    kp.edgen = nscr;
    const gb_dev_grid& g = g_gb.grid;
    if constexpr (SL::prim32 > 0) {
        dim3 pg((GB_STEP_CELLS / 4 + (mhd ? GB_STEP_FACES_ALL : 0) + 127) / 128, nblk);
        gb_prof_begin(GBP_RECON, s);
        if (mhd) k_prim32<true><<<pg, 128, 0, s>>>(g, list, p32, SL::prim32);
        else k_prim32<false><<<pg, 128, 0, s>>>(g, list, p32, SL::prim32);
        gb_prof_end(GBP_RECON, s);
    }
    if (kp.hybrid) {
        gb_prof_begin(GBP_RECON, s);
        if (mhd) k_divu<T, true><<<dim3(1, nblk), DIVU_THREADS, 0, s>>>(g, list, p32, SL::prim32, dscr, SL::divu);
        else k_divu<T, false><<<dim3(1, nblk), DIVU_THREADS, 0, s>>>(g, list, p32, SL::prim32, dscr, SL::divu);
        gb_prof_end(GBP_RECON, s);
    }
    if (mhd) {
        // time-n edge fields for the Riemann problems' half-step normal field
        // (timed with the edge-field kernels)
        gb_prof_begin(GBP_EMF, s);
        k_edge_n<T, true><<<dim3(6, nblk), EN_THREADS, 0, s>>>(g, list, p32, SL::prim32, nscr, SL::edgen);
        gb_prof_end(GBP_EMF, s);
    }
    const int tile = gb_recon_tile();
    dim3 rg((NRC + tile - 1) / tile, nblk);
    dim3 fg((NFC + 127) / 128, 3, nblk);
    if (mhd) {
        if (int rc = recon_and_flux<T, true>(tile, rg, fg, s, g, kp, nblk, list, rscr, fscr, p32, st)) return rc;
        put_fluxes<T>(kp, nblk, list, fscr, s);
        dim3 eg(GB_NXB, 3, nblk);
        gb_prof_begin(GBP_EMF, s);
        k_emf<T><<<eg, EMF_THREADS, 0, s>>>(list, cscr, SL::ecc, fscr, SL::flux, escr, SL::emf);
        if (kp.ec_reg)
            k_emf_put<<<dim3((NSURF + 127) / 128, nblk), 128, 0, s>>>(list, kp.ec_near, escr, SL::emf, kp.ec_reg);
        gb_prof_end(GBP_EMF, s);
        // the registers this chunk wrote are complete (a chunk on another
        // stream may read them now); the registers it reads next were
        // written by earlier chunks: wait for them only here, so that this
        // chunk's reconstruction, fluxes and edge fields overlap the
        // previous chunk's
        if (ev_put) cudaEventRecord(ev_put, s);
        if (ev_wait) cudaStreamWaitEvent(s, ev_wait, 0);
        if (kp.ec_reg) {
            gb_prof_begin(GBP_EMF, s);
            k_emf_get<<<dim3((GB_NXB * NRING + 127) / 128, 3, nblk), 128, 0, s>>>(
                list, kp.ec_plan, kp.ec_near, kp.ec_child, kp.ec_reg, escr, SL::emf);
            gb_prof_end(GBP_EMF, s);
        }
        dim3 bg((NFB + 127) / 128, 3, nblk);
        gb_prof_begin(GBP_FACEB, s);
        k_faceb<<<bg, 128, 0, s>>>(g, kp, list, escr, SL::emf, bscr, SL::fb);
        gb_prof_end(GBP_FACEB, s);
    } else {
        if (int rc = recon_and_flux<T, false>(tile, rg, fg, s, g, kp, nblk, list, rscr, fscr, p32, st)) return rc;
        put_fluxes<T>(kp, nblk, list, fscr, s);
        if (ev_put) cudaEventRecord(ev_put, s);
        if (ev_wait) cudaStreamWaitEvent(s, ev_wait, 0);
    }
    if (kp.fc_links) {
        // after the edge fields, which use the block's own fluxes
        dim3 rg2(1, 6, nblk);
        k_fc_get<T><<<rg2, GB_NXB * GB_NXB, 0, s>>>(list, kp.fc_links, (const T*)kp.fc_reg, fscr, SL::flux);
    }
    dim3 ug((GB_NXB * GB_NXB * GB_NXB + 127) / 128, nblk);
    gb_prof_begin(GBP_UPDATE, s);
    const sur_feat_out sfv = sf ? *sf : sur_feat_out{};
    const bool feat = !cool && sfv.feat;
    // cool 2 (the plain integrator on FP32 rates) exists for the mixed path,
    // as a pass of its own after the update (22.54 against 22.78 ms per
    // 4101-leaf step fused into it: the integrator's long code apart from the
    // update's); the FP64 path runs its reference rates in the update
    if (cool == 2 && std::is_same<T, float>::value) {
        if (mhd) k_update<T, true, 0, false><<<ug, 128, 0, s>>>(g, kp, g_gb.cool, list, fscr, SL::flux, bscr, SL::fb, st, sfv);
        else k_update<T, false, 0, false><<<ug, 128, 0, s>>>(g, kp, g_gb.cool, list, fscr, SL::flux, bscr, SL::fb, st, sfv);
        k_cool_pass<<<ug, 128, 0, s>>>(g, kp, g_gb.cool, list, st);
    } else if (mhd) {
        if (cool) k_update<T, true, 1, false><<<ug, 128, 0, s>>>(g, kp, g_gb.cool, list, fscr, SL::flux, bscr, SL::fb, st, sfv);
        else if (feat) k_update<T, true, 0, true><<<ug, 128, 0, s>>>(g, kp, g_gb.cool, list, fscr, SL::flux, bscr, SL::fb, st, sfv);
        else k_update<T, true, 0, false><<<ug, 128, 0, s>>>(g, kp, g_gb.cool, list, fscr, SL::flux, bscr, SL::fb, st, sfv);
    } else {
        if (cool) k_update<T, false, 1, false><<<ug, 128, 0, s>>>(g, kp, g_gb.cool, list, fscr, SL::flux, bscr, SL::fb, st, sfv);
        else if (feat) k_update<T, false, 0, true><<<ug, 128, 0, s>>>(g, kp, g_gb.cool, list, fscr, SL::flux, bscr, SL::fb, st, sfv);
        else k_update<T, false, 0, false><<<ug, 128, 0, s>>>(g, kp, g_gb.cool, list, fscr, SL::flux, bscr, SL::fb, st, sfv);
    }
    gb_prof_end(GBP_UPDATE, s);
    return gb_check(cudaGetLastError(), "hydro chunk launch") ? GB_ERR_CUDA : GB_OK;
}

}  // namespace gbh

// kernel parameters of a step with dt (or, with dtp, dt read from the
// device) from the registered grid and the hydro parameters (capi.cu)
gbh::hydro_kparams gb_make_kp(double dt, const double* dtp);
