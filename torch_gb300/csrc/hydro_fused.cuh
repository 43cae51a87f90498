// Reconstruction and Riemann solve fused per block: the face states never
// leave shared memory.
//
// One CTA per block of a chunk marches over the 18 planes of the
// reconstruction band (z = 3..20). For each plane it reconstructs the
// plane's 18 x 18 cells in all three directions (the same per-cell code as
// k_recon, three rounds of 128 cells per direction), keeps their face
// states in shared memory, and solves the Riemann problems of the plane's
// x and y faces and of the z faces between it and the previous plane (whose
// + states along z it kept). Only the fluxes (and the edge fields'
// reference) go to HBM, where the edge-field, flux-register and update
// kernels read them as before.
//
// The mixed path stages its inputs with the tensor memory accelerator: a
// window of five planes of the block's FP32 primitives (9 variables x 24 x
// 24 floats each, one cp.async.bulk.tensor per plane) rolls along z, the
// next plane loading while the current one computes; every wait on a
// plane's mbarrier is bounded. The FP64 path reads its stencils from the
// store (no room for a window of doubles beside the states).
#pragma once

#include <cuda.h>

#include "hydro_dev.cuh"

namespace gbh {

constexpr int FT = 128;                      // cells per direction and round
constexpr int FUSED_THREADS = 3 * FT;        // three directions
constexpr int NPL = RB * RB;                 // band cells per plane (324)
constexpr int NWIN = 5;                      // planes in the staged window
constexpr int WIN_PLANE = NP32 * GB_N * GB_N;  // floats per staged plane
constexpr int NXF = 17 * RB;                 // x (or y) faces of a plane (306)
constexpr unsigned FUSED_WAIT_LIMIT = 1u << 16;

// shared memory: mbarriers | window (TMA) | 7 state planes [NP][NPL]
// (x+, x-, y+, y-, z- and two z+ buffers) | transverse exchange
template <typename T, bool TMA>
struct fused_layout {
    static constexpr size_t bar = 128;
    static constexpr size_t win = TMA ? (size_t)NWIN * WIN_PLANE * sizeof(float) : 0;
    static constexpr size_t states = (size_t)7 * NP * NPL * sizeof(T);
    static constexpr size_t xch = ((size_t)6 * NP * FT + 3 * FT) * sizeof(T);
    static constexpr size_t bytes = bar + win + states + xch;
};
static_assert(fused_layout<float, true>::bytes <= 227 * 1024, "fused FP32 kernel fits shared memory");
static_assert(fused_layout<double, false>::bytes <= 227 * 1024, "fused FP64 kernel fits shared memory");
static_assert((WIN_PLANE * sizeof(float)) % 128 == 0, "window planes start on 128-byte boundaries");

// ---- TMA and mbarrier (inline PTX)
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// true once the phase of the given parity has completed (a suspended
// wait of at most about a microsecond per call)
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 1000;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// one box of a 5-D tensor map into shared memory, completing on bar
__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, unsigned long long* bar, int c0, int c1,
                                            int c2, int c3, int c4)
{
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
        : "memory");
}

// the FP32 copy's variable index of a role (as the flux kernel reads it)
__device__ __forceinline__ int p32_var(int role)
{
    return role == GB_EINT ? 8 : (role >= GB_MAGX ? 5 + (role - GB_MAGX) : role);
}

template <typename T, bool MHD, bool TMA>
__global__ void __launch_bounds__(FUSED_THREADS, 1)
k_recon_flux(gb_dev_grid g, hydro_kparams kp, const int* __restrict__ list, T* __restrict__ fscr, size_t fstride,
             const float* __restrict__ p32, size_t p32_stride, const __grid_constant__ CUtensorMap tmap, gb_status* st)
{
    using L = fused_layout<T, TMA>;
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem);
    float* win = reinterpret_cast<float*>(smem + L::bar);
    T* S = reinterpret_cast<T*>(smem + L::bar + L::win);
    T* X = S + (size_t)7 * NP * NPL;
    T(*s_sig)[NP][FT] = reinterpret_cast<T(*)[NP][FT]>(X);
    T(*s_abn)[NP][FT] = reinterpret_cast<T(*)[NP][FT]>(X + 3 * NP * FT);
    T(*s_dnb)[FT] = reinterpret_cast<T(*)[FT]>(X + 6 * NP * FT);
    auto plane = [&](int q) { return S + (size_t)q * NP * NPL; };

    const int tid = threadIdx.x, lane = tid % FT, d = tid / FT;
    const int cb = blockIdx.x;
    const int blk = list[cb];
    // the half-step normal field of the Riemann problems (k_edge_n's
    // time-n edge fields of this block)
    T dtdh[3];
    if constexpr (std::is_same<T, float>::value) kp_dtdxf(kp, gb_block_level(g, blk), dtdh);
    else kp_dtdx(kp, gb_block_level(g, blk), dtdh);
    const T* enb = (const T*)kp.edgen + (size_t)cb * scratch_layout<T>::edgen;
    T gam, dtd[3], hd[3];
    recon_consts<T>(g, kp, blk, gam, dtd, hd);
    const float* p32b = p32 + (size_t)cb * p32_stride;
    const int us[NP] = {0, rot_slot_rt<1>(d), rot_slot_rt<2>(d), rot_slot_rt<3>(d), 4,
                        rot_slot_rt<5>(d), rot_slot_rt<6>(d), rot_slot_rt<7>(d)};
    int off[NP];
    if constexpr (TMA) {
#pragma unroll
        for (int s = 0; s < NP; ++s) off[s] = us[s] * GB_N * GB_N;
    } else {
        rot_offsets<T, MHD>(g, d, off);
    }

    // the window: plane pl (z = 1..22) lives in slot pl % NWIN, its n-th
    // load there is n = (pl - 1) / NWIN
    bool timeout = false;
    auto issue = [&](int pl) {
        const int slot = pl % NWIN;
        mbar_expect_tx(&bars[slot], WIN_PLANE * (unsigned)sizeof(float));
        tma_load_5d(win + (size_t)slot * WIN_PLANE, &tmap, &bars[slot], 0, 0, pl, 0, cb);
    };
    auto wait = [&](int pl) {
        const int slot = pl % NWIN;
        const unsigned parity = (unsigned)((pl - 1) / NWIN) & 1u;
        unsigned n = 0;
        while (!mbar_try_wait(&bars[slot], parity))
            if (++n > FUSED_WAIT_LIMIT) {
                timeout = true;
                break;
            }
    };
    if constexpr (TMA) {
        if (tid == 0) {
#pragma unroll
            for (int q = 0; q < NWIN; ++q) mbar_init(&bars[q], 1);
            fence_mbar_init();
        }
        __syncthreads();
        if (tid == 0)
            for (int pl = 1; pl <= NWIN; ++pl) issue(pl);
    }

    for (int kz = 0; kz < RB; ++kz) {
        const int k = RLO + kz;
        if constexpr (TMA) {
            if (kz == 0) {
                for (int pl = 1; pl <= NWIN; ++pl) wait(pl);
            } else {
                wait(k + 2);
            }
        }
        const int zc = kz & 1;  // this plane's z+ buffer: 5 + zc
        // reconstruction: three rounds of FT cells per direction
        for (int r = 0; r < 3; ++r) {
            const int cell = r * FT + lane;
            const bool active = cell < NPL;
            const int cp = active ? cell : 0;
            const int i = RLO + cp % RB, j = RLO + cp / RB;
            const int band = cp + NPL * kz;
            auto ld = [&](int m, T* w) {
                if constexpr (TMA) {
                    const int pi = i + (d == 0 ? m - 2 : 0), pj = j + (d == 1 ? m - 2 : 0),
                              pk = k + (d == 2 ? m - 2 : 0);
                    const float* src = win + (size_t)(pk % NWIN) * WIN_PLANE + pj * GB_N + pi;
#pragma unroll
                    for (int s = 0; s < NP; ++s) w[s] = (MHD || s < 5) ? (T)src[off[s]] : (T)0;
                } else {
                    const int stride = d == 0 ? 1 : (d == 1 ? GB_N : GB_N * GB_N);
                    load_rot<T, MHD>(g, blk, gb_cidx(i, j, k) + (m - 2) * stride, p32b, off, w);
                }
            };
            T wp[NP], wn[NP];
            recon_item<T, MHD, FT>(g, kp, cb, blk, d, lane, band, band, active, i, j, k, gam, dtd, hd, p32b, ld,
                                   s_sig, s_abn, s_dnb, st, wp, wn);
            if (active) {
                T* qp = plane(d == 0 ? 0 : (d == 1 ? 2 : 5 + zc));
                T* qn = plane(d == 0 ? 1 : (d == 1 ? 3 : 4));
#pragma unroll
                for (int s = 0; s < NP; ++s) {
                    qp[(size_t)us[s] * NPL + cell] = wp[s];
                    qn[(size_t)us[s] * NPL + cell] = wn[s];
                }
            }
            __syncthreads();
        }
        // plane k - 2 has been read for the last time: its slot takes k + 3
        if constexpr (TMA) {
            if (tid == 0 && k + 3 <= GB_N - 2 && !timeout) issue(k + 3);
        }
        // Riemann problems: the plane's x and y faces, the z faces below it
        const int nface = kz == 0 ? 2 * NXF : 2 * NXF + NPL;
        for (int f = tid; f < nface; f += FUSED_THREADS) {
            int dir, I[3], cl, cr, ql, qr;
            if (f < NXF) {
                dir = 0;
                I[0] = LO + f % 17; I[1] = RLO + f / 17; I[2] = k;
                cl = (I[0] - 1 - RLO) + RB * (I[1] - RLO);
                cr = cl + 1;
                ql = 0; qr = 1;
            } else if (f < 2 * NXF) {
                const int e = f - NXF;
                dir = 1;
                I[0] = RLO + e % RB; I[1] = LO + e / RB; I[2] = k;
                cl = (I[0] - RLO) + RB * (I[1] - 1 - RLO);
                cr = cl + RB;
                ql = 2; qr = 3;
            } else {
                const int c = f - 2 * NXF;
                dir = 2;
                I[0] = RLO + c % RB; I[1] = RLO + c / RB; I[2] = k;
                cl = cr = c;
                ql = 5 + (zc ^ 1); qr = 4;
            }
            T wl[NP], wr[NP];
            const T* pl_ = plane(ql);
            const T* pr_ = plane(qr);
#pragma unroll
            for (int v = 0; v < NP; ++v) {
                wl[v] = pl_[(size_t)v * NPL + cl];
                wr[v] = pr_[(size_t)v * NPL + cr];
            }
            int Il[3] = {I[0], I[1], I[2]};
            Il[dir] -= 1;
            auto U = [&](int role, int ci) -> T {
                if constexpr (TMA) {
                    const int x = ci % GB_N, y = (ci / GB_N) % GB_N, z = ci / (GB_N * GB_N);
                    return (T)win[(size_t)(z % NWIN) * WIN_PLANE + p32_var(role) * GB_N * GB_N + y * GB_N + x];
                } else if constexpr (std::is_same<T, float>::value) {
                    return p32b[(size_t)p32_var(role) * GB_N3 + ci];
                } else {
                    return (T)g.unk[((int64_t)blk * g.nvar + g.slot[role]) * GB_N3 + ci];
                }
            };
            const int cil = gb_cidx(Il[0], Il[1], Il[2]), cir = gb_cidx(I[0], I[1], I[2]);
            T out[NP], feint, un;
            T* fs = fscr + (size_t)cb * fstride + (size_t)dir * NFLX * NFC;
            const int fi = flux_index(dir, I[0], I[1], I[2]);
            if (dir == 0) {
                const T bnf = MHD ? face_b_half<T, 0>(face_b<T>(g, 0, blk, gb_fidx(0, I[0], I[1], I[2]), p32b), enb, I, dtdh)
                                  : (T)0;
                face_flux_core<T, MHD, 0>(kp, wl, wr, bnf, U, cil, cir, out, feint, un);
                face_flux_store<T, MHD, 0>(fs, fi, out, feint, un);
            } else if (dir == 1) {
                const T bnf = MHD ? face_b_half<T, 1>(face_b<T>(g, 1, blk, gb_fidx(1, I[0], I[1], I[2]), p32b), enb, I, dtdh)
                                  : (T)0;
                face_flux_core<T, MHD, 1>(kp, wl, wr, bnf, U, cil, cir, out, feint, un);
                face_flux_store<T, MHD, 1>(fs, fi, out, feint, un);
            } else {
                const T bnf = MHD ? face_b_half<T, 2>(face_b<T>(g, 2, blk, gb_fidx(2, I[0], I[1], I[2]), p32b), enb, I, dtdh)
                                  : (T)0;
                face_flux_core<T, MHD, 2>(kp, wl, wr, bnf, U, cil, cir, out, feint, un);
                face_flux_store<T, MHD, 2>(fs, fi, out, feint, un);
            }
        }
        __syncthreads();
    }
    if constexpr (TMA) {
        // a wait that gave up left its copy in flight: wait for every plane
        // once more (bounded) so that nothing lands after the CTA is gone
        if (timeout) {
            for (int pl = GB_N - 2 - NWIN + 1; pl <= GB_N - 2; ++pl) wait(pl);
            if (tid == 0) gb_fail(st, GB_ST_TIMEOUT, blk, 0, 0, 0, 0.0);
        }
    }
}

}  // namespace gbh

// tensor map of a chunk's FP32 copies: 5-D (x, y, z, variable, block),
// boxes of one plane of all nine variables of one block (hydro_mixed.cu)
int gb_encode_p32_map(CUtensorMap* map, const float* p32, int nblk, size_t stride_floats);
