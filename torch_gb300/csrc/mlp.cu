// Learned cooling surrogate: a 4 -> 64 -> 64 -> 64 -> 1 SiLU MLP on the
// fifth-generation tensor cores (tcgen05, accumulators in tensor memory).
//
// Inference and training share one BF16 weight image in shared memory and
// one forward pass: BF16 operands, FP32 accumulation, activations rounded to
// BF16 between layers. Training adds the backward pass in the same kernel
// (the data gradients dz W and the weight gradients dz^T a on the tensor
// cores, the pre-activations and gradient accumulators kept in tensor
// memory) and an Adam step on FP32 master weights that also rewrites the
// weight images. A CUDA-core FP32 forward with the same BF16-rounded
// weights is kept as the reference for the tensor-core path.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include "gb_state.h"
#include "mlp.h"
#include "tc05.cuh"

namespace {

constexpr int H = GB_MLP_HIDDEN;  // 64
constexpr int NIN = GB_MLP_IN;    // 4

// parameter offsets in the flat FP32 vector
constexpr int OW1 = 0, OB1 = OW1 + H * NIN, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H,
              OB3 = OW3 + H * H, OW4 = OB3 + H, OB4 = OW4 + H, NPAR = OB4 + 1;
static_assert(NPAR == GB_MLP_NPARAM, "parameter count");
// per-CTA partial gradients: the NPAR gradients, then the loss
constexpr int PSTRIDE = NPAR + 1;

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z)
{
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// the hardware tanh approximation (one MUFU operation; its ~2^-11 relative
// error is below the BF16 rounding the activation gets next)
__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ------------------------------------------- inference on tcgen05 + TMEM
// A CTA holds the weights once in shared memory and runs four warpgroups,
// each on its own 128-cell tiles (M = 128) with its own 64 accumulator
// columns of tensor memory, A operands and mbarrier; two CTAs fill an SM's
// shared memory and its 512 TMEM columns, so eight tiles are in flight per
// SM. Every layer is one chain of K = 16 tcgen05 MMAs issued by one thread
// of the warpgroup; the epilogue reads the accumulator back (thread t of
// the warpgroup holds cell t's row), applies the SiLU, rounds to BF16 and
// writes the next layer's A operand into shared memory.
//
// The biases ride in the MMA: A carries a column of ones after the
// activations (column NIN of layer 1, column H of the hidden layers) and
// the weight image the bias in that column, so D = A W^T + b exactly (the
// BF16 bias times 1.0 enters the FP32 accumulator unrounded, as in the
// CUDA-core path). The hidden layers' ones column and its zero padding are
// one block shared by the warpgroups: the last MMA of a hidden layer points
// its A descriptor there. Layers 1-3 are stored scaled by 1/2 (exact in
// BF16), so the accumulator holds h = z / 2 and SiLU(z) = h (1 + tanh h)
// costs one tanh and one FMA.
struct tc_layout {
    static constexpr int M = 128;      // cells per tile
    static constexpr int WG = 4;       // warpgroups (tiles in flight) per CTA
    static constexpr int KH = H + 16;  // hidden K: activations, ones column, zero padding
    // weight images, [out][in] K-major (B operands), 16-byte core-matrix rows
    static constexpr int W1_LBO = H * 16, W1 = 0, W1_BYTES = 2 * W1_LBO;  // N 64, K 16
    static constexpr int WH_LBO = H * 16, WH_BYTES = (KH / 8) * WH_LBO;  // N 64, K 80
    static constexpr int W2 = W1 + W1_BYTES, W3 = W2 + WH_BYTES;
    static constexpr int W4_LBO = 16 * 16, W4 = W3 + WH_BYTES, W4_BYTES = (KH / 8) * W4_LBO;  // N 16, K 80
    static constexpr int WBYTES = W4 + W4_BYTES;
    // A operands, K-groups of 128 rows x 16 bytes
    static constexpr int A_LBO = M * 16;
    static constexpr int ONES = WBYTES;                // K-groups 8 (ones column) and 9 (zero)
    static constexpr int TILE0 = ONES + 2 * A_LBO;     // per warpgroup: A1 (2 groups) then A (8 groups)
    static constexpr int A1_OFF = 0, A_OFF = 2 * A_LBO, TILE_BYTES = 10 * A_LBO;
    // WG mbarriers, the TMEM address, the weight copy's mbarrier
    static constexpr int BAR = TILE0 + WG * TILE_BYTES;
    static constexpr int WBAR = BAR + 8 * WG + 8;
    static constexpr int BYTES = BAR + 8 * WG + 16;
    static constexpr uint32_t COLS_PER_WG = 64, TMEM_COLS = COLS_PER_WG * WG;
};
static_assert(tc_layout::WBYTES % 16 == 0 && tc_layout::TILE0 % 16 == 0 && tc_layout::TILE_BYTES % 16 == 0,
              "16-byte operands");
static_assert(2 * (tc_layout::BYTES + 1024) <= 228 * 1024, "two tcgen05 MLP CTAs fit an SM");
static_assert(2 * tc_layout::TMEM_COLS <= 512, "two tcgen05 MLP CTAs fit an SM's tensor memory");

// ----------------------------------------------------------- training
// The backward pass needs W3 and W2 as B operands of d_prev = dz W: their
// transposes, rows k_in, K = n_out (unscaled).
struct tr_layout {
    using L = tc_layout;
    static constexpr int M = 128;  // samples per tile
    static constexpr int WT_LBO = H * 16, WT_BYTES = (H / 8) * WT_LBO;
    static constexpr int WT3 = L::WBYTES, WT2 = WT3 + WT_BYTES;  // global image: WT3 then WT2
    static constexpr int ONES = WT2 + WT_BYTES;  // the forward's ones block (K-groups 8, 9)
    static constexpr int A_LBO = M * 16;
    static constexpr int X1 = ONES + 2 * A_LBO;  // layer-1 A: x, 1, zeros (2 K-groups)
    static constexpr int ACT = X1 + 2 * A_LBO;   // activations, sample rows (8 K-groups)
    static constexpr int DZ = ACT + 8 * A_LBO;   // dz, sample rows (8 K-groups)
    // sample-major operands of the weight gradients, K = the tile's 128
    // samples (16 K-groups); a K-group's stride is padded by 16 bytes so the
    // 2-byte stores of one row by a warp's 32 samples hit distinct banks
    static constexpr int AT_ROWS = H + 16, AT_LBO = AT_ROWS * 16 + 16;  // [a, 1, 0 ...] as rows
    static constexpr int XT_ROWS = 16, XT_LBO = XT_ROWS * 16 + 16;      // [x, 1, 0 ...] as rows
    static constexpr int DT_LBO = M * 16 + 16;                          // 128-row stacks
    static constexpr int AT1 = DZ + 8 * A_LBO, AT2 = AT1 + 16 * AT_LBO, AT3 = AT2 + 16 * AT_LBO;
    static constexpr int XT = AT3 + 16 * AT_LBO;
    static constexpr int DTA = XT + 16 * XT_LBO;  // rows: dz3^T (0-63), dy^T (64), zeros
    static constexpr int DTB = DTA + 16 * DT_LBO;  // rows: dz2^T (0-63), dz1^T (64-127)
    static constexpr int RED = DTB + 16 * DT_LBO;  // 4 floats: the warps' loss sums
    static constexpr int BAR = RED + 16;  // the MMA barrier, the TMEM address, the weight copy's barrier
    static constexpr int WBAR = BAR + 16;
    static constexpr int BYTES = BAR + 24;
    // tensor-memory columns: pre-activations (the data gradients overwrite
    // them once read), the output, and the weight-gradient accumulators
    // (128 lanes; only the rows the A stack makes meaningful are read)
    static constexpr uint32_t Z1 = 0, Z2 = 64, Z3 = 128, Y = 192, G1 = 208, G3 = 224, G2 = 320, G4 = 416;
    static constexpr uint32_t TMEM_COLS = 512;
};
static_assert(tr_layout::BYTES <= 227 * 1024, "tcgen05 MLP training fits shared memory");
static_assert(tr_layout::G4 + 80 <= tr_layout::TMEM_COLS, "training accumulators fit tensor memory");
static_assert(tr_layout::AT1 % 16 == 0 && tr_layout::XT % 16 == 0 && tr_layout::DTA % 16 == 0 && tr_layout::WT3 % 16 == 0 &&
                  tr_layout::DTB % 16 == 0 && tr_layout::RED % 16 == 0,
              "16-byte operands");

// the image entries of parameter i with value w: the forward image (layers
// 1-3 scaled by 1/2, biases in the ones column) and the W^T images of
// layers 3 and 2. Every other image entry is a zero set at allocation.
__device__ __forceinline__ void put_param(int i, float w, __nv_bfloat16* __restrict__ fw, __nv_bfloat16* __restrict__ wt)
{
    using L = tc_layout;
    using T = tr_layout;
    auto at = [](int base, int lbo, int r, int k) { return (base + (k / 8) * lbo + r * 16 + (k % 8) * 2) / 2; };
    const __nv_bfloat16 half = __float2bfloat16_rn(0.5f * w), full = __float2bfloat16_rn(w);
    if (i < OB1) {
        fw[at(L::W1, L::W1_LBO, (i - OW1) / NIN, (i - OW1) % NIN)] = half;
    } else if (i < OW2) {
        fw[at(L::W1, L::W1_LBO, i - OB1, NIN)] = half;
    } else if (i < OB2) {
        const int r = (i - OW2) / H, k = (i - OW2) % H;
        fw[at(L::W2, L::WH_LBO, r, k)] = half;
        wt[at(T::WT2 - T::WT3, T::WT_LBO, k, r)] = full;
    } else if (i < OW3) {
        fw[at(L::W2, L::WH_LBO, i - OB2, H)] = half;
    } else if (i < OB3) {
        const int r = (i - OW3) / H, k = (i - OW3) % H;
        fw[at(L::W3, L::WH_LBO, r, k)] = half;
        wt[at(0, T::WT_LBO, k, r)] = full;
    } else if (i < OW4) {
        fw[at(L::W3, L::WH_LBO, i - OB3, H)] = half;
    } else if (i < OB4) {
        fw[at(L::W4, L::W4_LBO, 0, i - OW4)] = full;
    } else {
        fw[at(L::W4, L::W4_LBO, 0, H)] = full;
    }
}

__global__ void k_put_images(const float* __restrict__ w, __nv_bfloat16* __restrict__ fw, __nv_bfloat16* __restrict__ wt)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < NPAR) put_param(i, w[i], fw, wt);
}

// a bounded wait for an MMA chain: about one second at the SM clock
constexpr long long TC_WAIT_CYCLES = 2000000000LL;

__global__ void __launch_bounds__(128 * tc_layout::WG) k_mlp_infer_tc(int64_t n, const float4* __restrict__ feat,
                                                                    const uint4* __restrict__ wimg,
                                                                    float* __restrict__ y, gb_status* st)
{
    using L = tc_layout;
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, wg = tid >> 7, t = tid & 127, warp = tid >> 5;
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm + L::BAR) + wg;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + L::BAR + 8 * L::WG);
    unsigned char* tile_sm = sm + L::TILE0 + wg * L::TILE_BYTES;

    // the weight image arrives by one bulk copy while the CTA sets up
    unsigned long long* wbar = reinterpret_cast<unsigned long long*>(sm + L::WBAR);
    if (tid == 0) {
        tc05::mbar_init(wbar, 1);
        tc05::mbar_expect_tx(wbar, L::WBYTES);
        tc05::bulk_g2s(sm, wimg, L::WBYTES, wbar);
    }
    // constant parts of the A operands: the shared ones block, and the zero
    // second K-group of each layer-1 A
    const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
    if (wg == 0) {
        reinterpret_cast<uint4*>(sm + L::ONES)[t] = make_uint4(pack2(1.0f, 0.0f), 0u, 0u, 0u);
        reinterpret_cast<uint4*>(sm + L::ONES + L::A_LBO)[t] = z4;
    }
    reinterpret_cast<uint4*>(tile_sm + L::A1_OFF + L::A_LBO)[t] = z4;
    if (warp == 0) tc05::alloc(tslot, L::TMEM_COLS);
    if (t == 0) tc05::mbar_init(bar, 1);
    tc05::fence_async_smem();
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();
    const uint32_t tacc = *tslot + (uint32_t)wg * L::COLS_PER_WG;  // this warpgroup's columns
    const uint32_t trow = tc05::tmem_at(tacc, (uint32_t)(warp & 3) * 32u, 0u);
    const uint32_t s0 = tc05::saddr(sm), sA1 = tc05::saddr(tile_sm + L::A1_OFF), sA = tc05::saddr(tile_sm + L::A_OFF);
    uint4* a_rows = reinterpret_cast<uint4*>(tile_sm + L::A_OFF) + t;  // row t of K-group 0
    constexpr uint32_t ID64 = tc05::idesc_bf16(L::M, H), ID16 = tc05::idesc_bf16(L::M, 16);
    const uint32_t bar_id = 1u + (uint32_t)wg;

    uint32_t phase = 0;
    // layer 1: one K = 16 MMA
    auto layer1 = [&]() {
        if (t == 0) {
            tc05::fence_after_sync();
            tc05::mma_bf16(tacc, tc05::sdesc(sA1, L::A_LBO, 128u), tc05::sdesc(s0 + L::W1, L::W1_LBO, 128u), ID64, 0u);
            tc05::commit(bar);
        }
    };
    // a hidden or the output layer: four MMAs over the activations and one
    // over the shared ones block
    auto layer = [&](uint32_t w, uint32_t w_lbo, uint32_t idesc) {
        if (t == 0) {
            tc05::fence_after_sync();
#pragma unroll
            for (int s = 0; s < 4; ++s)
                tc05::mma_bf16(tacc, tc05::sdesc(sA + 2u * s * L::A_LBO, L::A_LBO, 128u),
                               tc05::sdesc(w + 2u * s * w_lbo, w_lbo, 128u), idesc, s > 0);
            tc05::mma_bf16(tacc, tc05::sdesc(s0 + L::ONES, L::A_LBO, 128u), tc05::sdesc(w + 8u * w_lbo, w_lbo, 128u),
                           idesc, 1u);
            tc05::commit(bar);
        }
    };
    auto wait = [&]() -> bool {
        const bool done = tc05::mbar_wait(bar, phase, TC_WAIT_CYCLES);
        phase ^= 1u;
        tc05::fence_after_sync();
        return done;
    };
    // 16 accumulator columns -> SiLU -> BF16 -> two K-groups of row t
    auto silu16 = [&](const uint32_t (&v)[16], int c) {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            uint32_t q[4];
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const float h0 = __uint_as_float(v[j * 8 + 2 * p]), h1 = __uint_as_float(v[j * 8 + 2 * p + 1]);
                q[p] = pack2(fmaf(h0, tanh_approx(h0), h0), fmaf(h1, tanh_approx(h1), h1));
            }
            a_rows[(2 * c + j) * (L::A_LBO / 16)] = make_uint4(q[0], q[1], q[2], q[3]);
        }
    };
    // hidden epilogue: the next chunk's TMEM load is in flight while one
    // chunk is converted
    auto hidden_out = [&]() {
        uint32_t va[16], vb[16];
        tc05::ld16(trow, va);
        tc05::wait16(va);
        tc05::ld16(trow + 16u, vb);
        silu16(va, 0);
        tc05::wait16(vb);
        tc05::ld16(trow + 32u, va);
        silu16(vb, 1);
        tc05::wait16(va);
        tc05::ld16(trow + 48u, vb);
        silu16(va, 2);
        tc05::wait16(vb);
        silu16(vb, 3);
        tc05::fence_async_smem();
        tc05::fence_before_sync();
    };

    const int64_t ntiles = (n + L::M - 1) / L::M;
    const int64_t tstep = (int64_t)gridDim.x * L::WG;
    int64_t tile = (int64_t)blockIdx.x * L::WG + wg;
    float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tile < ntiles && tile * L::M + t < n) f = feat[tile * L::M + t];
    bool done = tc05::mbar_wait(wbar, 0u, TC_WAIT_CYCLES);  // the weights (a failure ends the loop at once)
    for (; tile < ntiles; tile += tstep) {
        const int64_t row = tile * L::M + t;
        reinterpret_cast<uint4*>(tile_sm + L::A1_OFF)[t] =
            make_uint4(pack2(f.x, f.y), pack2(f.z, f.w), pack2(1.0f, 0.0f), 0u);
        tc05::fence_async_smem();
        tc05::fence_before_sync();
        if (tc05::bar_or(bar_id, 128, !done)) break;  // also the previous tile's last wait
        layer1();
        // the next tile's features load while this tile runs
        const int64_t nrow = row + tstep * L::M;
        f = nrow < n ? feat[nrow] : make_float4(0.f, 0.f, 0.f, 0.f);
        done = wait();
        hidden_out();
        if (tc05::bar_or(bar_id, 128, !done)) break;
        layer(s0 + L::W2, L::WH_LBO, ID64);
        done = wait();
        hidden_out();
        if (tc05::bar_or(bar_id, 128, !done)) break;
        layer(s0 + L::W3, L::WH_LBO, ID64);
        done = wait();
        hidden_out();
        if (tc05::bar_or(bar_id, 128, !done)) break;
        layer(s0 + L::W4, L::W4_LBO, ID16);
        done = wait();
        const float out = __uint_as_float(tc05::ld1(trow));
        if (row < n) y[row] = done ? out : __int_as_float(0x7fc00000);
        tc05::fence_before_sync();
    }
    if (tc05::bar_or(bar_id, 128, !done)) {
        // a chain that did not complete in time: this warpgroup's remaining
        // predictions are NaN (the acceptance test sends those cells to the
        // integrator); wait once more, bounded, before the accumulator is
        // freed
        for (; tile < ntiles; tile += tstep)
            if (tile * L::M + t < n) y[tile * L::M + t] = __int_as_float(0x7fc00000);
        if (t == 0) gb_fail(st, GB_ST_TIMEOUT, -1, 0, 0, 0, 0.0);
        tc05::mbar_wait(bar, phase ^ 1u, TC_WAIT_CYCLES);
        tc05::mbar_wait(wbar, 0u, TC_WAIT_CYCLES);
    }
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();
    if (warp == 0) tc05::dealloc(*tslot, L::TMEM_COLS);
}

// a counter-based sample draw: row of sample b of training step `step`,
// uniform over [0, n)
__device__ __forceinline__ int64_t sample_row(uint64_t seed, int step, int batch, int b, int64_t n)
{
    uint64_t z = seed + 0x9E3779B97F4A7C15ULL * ((uint64_t)step * (uint64_t)batch + (uint64_t)b + 1u);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (int64_t)(z % (uint64_t)n);
}

// row r, sample t of a sample-major operand (one BF16 value)
__device__ __forceinline__ void put_t(unsigned char* base, int lbo, int r, int t, uint32_t bits)
{
    *reinterpret_cast<uint16_t*>(base + (t >> 3) * lbo + r * 16 + (t & 7) * 2) = (uint16_t)bits;
}

// One training pass over `batch` samples (drawn with sample_row when
// `sample`, else rows 0 .. batch-1): forward, squared-error loss, backward;
// each CTA runs 128-sample tiles and writes its partial gradients and loss
// sum (divided by batch) to part[blockIdx.x]. Per tile, on the tensor cores:
//   forward   Z_l = [a_{l-1}, 1] W_l'^T  (the inference image)
//   backward  d_{l-1} = dz_l W_l         (the W^T images, into Z_l's columns)
//             G_l += [dz_l^T ; ...] [a_{l-1}, 1]  (weight and bias gradients
//             summed over the tile's samples, K = 128)
// with dz_4 = dy = 2 (y - t) / batch, dz_3 = (dy W_4) silu'(z_3) and
// dz_l = d_l silu'(z_l), all rounded to BF16 as MMA operands. Two
// gradients share one M = 128 MMA where their A rows stack: [dz3^T ; dy^T]
// against a2 and a3 (layers 3 and 4), [dz2^T ; dz1^T] against a1 and x
// (layers 2 and 1).
__global__ void __launch_bounds__(128, 1)
k_mlp_train_tc(const float4* __restrict__ feat, const float* __restrict__ target, int64_t n, int batch, uint64_t seed,
               int step, int sample, const uint4* __restrict__ fw, const uint4* __restrict__ wt,
               float* __restrict__ part, gb_status* st)
{
    using L = tc_layout;
    using T = tr_layout;
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm + T::BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + T::BAR + 8);
    float* red = reinterpret_cast<float*>(sm + T::RED);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

    // the weight images arrive by two bulk copies while the CTA sets up
    unsigned long long* wbar = reinterpret_cast<unsigned long long*>(sm + T::WBAR);
    if (t == 0) {
        tc05::mbar_init(wbar, 1);
        tc05::mbar_expect_tx(wbar, L::WBYTES + 2 * T::WT_BYTES);
        tc05::bulk_g2s(sm, fw, L::WBYTES, wbar);
        tc05::bulk_g2s(sm + T::WT3, wt, 2 * T::WT_BYTES, wbar);
    }
    // constant operand parts: the forward ones block and layer 1's zero
    // K-group; rows 64 (ones) .. 79 of the activation operands, rows 4
    // (ones) .. 15 of x's, rows 65 .. 127 of the layer-3/4 stack (zeros)
    const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
    const uint4 ones8 = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
    reinterpret_cast<uint4*>(sm + T::ONES)[t] = make_uint4(pack2(1.0f, 0.0f), 0u, 0u, 0u);
    reinterpret_cast<uint4*>(sm + T::ONES + T::A_LBO)[t] = z4;
    reinterpret_cast<uint4*>(sm + T::X1 + T::A_LBO)[t] = z4;
    for (int i = t; i < 16 * 16; i += blockDim.x) {
        const int g = i >> 4, q = i & 15;
        for (int m = 0; m < 3; ++m)
            *reinterpret_cast<uint4*>(sm + T::AT1 + (m * 16 + g) * T::AT_LBO + (H + q) * 16) = q == 0 ? ones8 : z4;
    }
    for (int i = t; i < 16 * 12; i += blockDim.x) {
        const int g = i / 12, q = i % 12;
        *reinterpret_cast<uint4*>(sm + T::XT + g * T::XT_LBO + (NIN + q) * 16) = q == 0 ? ones8 : z4;
    }
    for (int i = t; i < 16 * 63; i += blockDim.x)
        *reinterpret_cast<uint4*>(sm + T::DTA + (i / 63) * T::DT_LBO + (65 + i % 63) * 16) = z4;
    if (warp == 0) tc05::alloc(tslot, T::TMEM_COLS);
    if (t == 0) tc05::mbar_init(bar, 1);
    tc05::fence_async_smem();
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();

    const uint32_t tm = *tslot;
    const uint32_t trow = tc05::tmem_at(tm, (uint32_t)warp * 32u, 0u);
    const uint32_t s0 = tc05::saddr(sm);
    constexpr uint32_t ID64 = tc05::idesc_bf16(128, H), ID16 = tc05::idesc_bf16(128, 16),
                       ID80 = tc05::idesc_bf16(128, T::AT_ROWS);
    uint4* act_row = reinterpret_cast<uint4*>(sm + T::ACT) + t;
    uint4* dz_row = reinterpret_cast<uint4*>(sm + T::DZ) + t;
    const __nv_bfloat16* w4 = reinterpret_cast<const __nv_bfloat16*>(sm + L::W4);  // row 0 of layer 4

    auto mma = [&](uint32_t d, int a, int a_lbo, int b, int b_lbo, uint32_t idesc, bool acc) {
        tc05::mma_bf16(tm + d, tc05::sdesc(s0 + a, a_lbo, 128u), tc05::sdesc(s0 + b, b_lbo, 128u), idesc, acc);
    };
    // forward layer: four K-steps over the activations, one over the ones
    auto fwd_layer = [&](uint32_t d, int w, int w_lbo, uint32_t idesc) {
        for (int s = 0; s < 4; ++s) mma(d, T::ACT + 2 * s * T::A_LBO, T::A_LBO, w + 2 * s * w_lbo, w_lbo, idesc, s > 0);
        mma(d, T::ONES, T::A_LBO, w + 8 * w_lbo, w_lbo, idesc, true);
    };
    // data gradient: D = dz (sample rows, K = 64) x W (the W^T image)
    auto data_grad = [&](uint32_t d, int wt_img) {
        for (int s = 0; s < 4; ++s)
            mma(d, T::DZ + 2 * s * T::A_LBO, T::A_LBO, wt_img + 2 * s * T::WT_LBO, T::WT_LBO, ID64, s > 0);
    };
    // weight gradient: D += stack (K = the tile's samples) x operand rows
    bool first = true;
    auto weight_grad = [&](uint32_t d, int stack, int b, int b_lbo, uint32_t idesc) {
        for (int s = 0; s < 8; ++s)
            mma(d, stack + 2 * s * T::DT_LBO, T::DT_LBO, b + 2 * s * b_lbo, b_lbo, idesc, !(first && s == 0));
    };
    uint32_t phase = 0;
    auto wait = [&]() -> bool {
        const bool done = tc05::mbar_wait(bar, phase, TC_WAIT_CYCLES);
        phase ^= 1u;
        tc05::fence_after_sync();
        return done;
    };
    auto to_mma = [&]() {
        tc05::fence_async_smem();
        tc05::fence_before_sync();
    };
    // forward epilogue: z = 2 h from the accumulator, a = BF16(silu z) into
    // the activation rows and the sample-major operand `at`
    auto fwd_epi = [&](uint32_t zcol, int at) {
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
            uint32_t v[16];
            tc05::ld16(trow + zcol + 16u * c, v);
            tc05::wait16(v);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                uint32_t q[4];
#pragma unroll
                for (int p = 0; p < 4; ++p)
                    q[p] = pack2(silu(2.0f * __uint_as_float(v[8 * j + 2 * p])),
                                 silu(2.0f * __uint_as_float(v[8 * j + 2 * p + 1])));
                act_row[(2 * c + j) * (T::A_LBO / 16)] = make_uint4(q[0], q[1], q[2], q[3]);
#pragma unroll
                for (int e = 0; e < 8; ++e) put_t(sm + at, T::AT_LBO, 16 * c + 8 * j + e, t, q[e >> 1] >> (16 * (e & 1)));
            }
        }
        to_mma();
    };
    // backward epilogue: dz = d silu'(2 h) from the data gradient's and the
    // pre-activation's columns (d = dy W4 for layer 3) into the dz rows
    // (when the next data gradient needs them) and rows row0.. of `stack`
    auto bwd_epi = [&](bool from_dy, float dy, uint32_t dcol, uint32_t zcol, bool rows, int stack, int row0) {
#pragma unroll 1
        for (int c = 0; c < 4; ++c) {
            uint32_t vd[16], vz[16];
            if (!from_dy) tc05::ld16(trow + dcol + 16u * c, vd);
            tc05::ld16(trow + zcol + 16u * c, vz);
            if (!from_dy) tc05::wait16(vd);
            tc05::wait16(vz);
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                uint32_t q[4];
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    float g[2];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int e = 8 * j + 2 * p + h, k = 16 * c + e;
                        const float d = from_dy ? dy * __bfloat162float(w4[(k / 8) * (L::W4_LBO / 2) + (k % 8)])
                                                : __uint_as_float(vd[e]);
                        g[h] = d * silu_grad(2.0f * __uint_as_float(vz[e]));
                    }
                    q[p] = pack2(g[0], g[1]);
                }
                if (rows) dz_row[(2 * c + j) * (T::A_LBO / 16)] = make_uint4(q[0], q[1], q[2], q[3]);
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    put_t(sm + stack, T::DT_LBO, row0 + 16 * c + 8 * j + e, t, q[e >> 1] >> (16 * (e & 1)));
            }
        }
        to_mma();
    };

    float loss = 0.0f;
    bool done = tc05::mbar_wait(wbar, 0u, TC_WAIT_CYCLES);  // the weights (a failure ends the loop at once)
    const int ntiles = (batch + 127) / 128;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int b = tile * 128 + t;
        const bool valid = b < batch;
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        float tg = 0.0f;
        if (valid) {
            const int64_t j = sample ? sample_row(seed, step, batch, b, n) : (int64_t)b;
            x = feat[j];
            tg = target[j];
        }
        const uint32_t x01 = pack2(x.x, x.y), x23 = pack2(x.z, x.w);
        reinterpret_cast<uint4*>(sm + T::X1)[t] = make_uint4(x01, x23, pack2(1.0f, 0.0f), 0u);
        put_t(sm + T::XT, T::XT_LBO, 0, t, x01);
        put_t(sm + T::XT, T::XT_LBO, 1, t, x01 >> 16);
        put_t(sm + T::XT, T::XT_LBO, 2, t, x23);
        put_t(sm + T::XT, T::XT_LBO, 3, t, x23 >> 16);
        to_mma();
        if (__syncthreads_or(!done)) break;
        if (t == 0) {
            tc05::fence_after_sync();
            mma(T::Z1, T::X1, T::A_LBO, L::W1, L::W1_LBO, ID64, false);
            tc05::commit(bar);
        }
        done = wait();
        fwd_epi(T::Z1, T::AT1);
        if (__syncthreads_or(!done)) break;
        if (t == 0) {
            tc05::fence_after_sync();
            fwd_layer(T::Z2, L::W2, L::WH_LBO, ID64);
            tc05::commit(bar);
        }
        done = wait();
        fwd_epi(T::Z2, T::AT2);
        if (__syncthreads_or(!done)) break;
        if (t == 0) {
            tc05::fence_after_sync();
            fwd_layer(T::Z3, L::W3, L::WH_LBO, ID64);
            tc05::commit(bar);
        }
        done = wait();
        fwd_epi(T::Z3, T::AT3);
        if (__syncthreads_or(!done)) break;
        if (t == 0) {
            tc05::fence_after_sync();
            fwd_layer(T::Y, L::W4, L::W4_LBO, ID16);
            tc05::commit(bar);
        }
        done = wait();
        // the TMEM load is warp-collective: every lane runs it, valid or not
        const float yv = __uint_as_float(tc05::ld1(trow + T::Y));
        const float r = valid ? yv - tg : 0.0f;
        loss += r * r;
        const float dy = 2.0f * r / (float)batch;
        put_t(sm + T::DTA, T::DT_LBO, H, t, pack2(dy, 0.0f));
        bwd_epi(true, dy, 0u, T::Z3, true, T::DTA, 0);
        if (__syncthreads_or(!done)) break;
        if (t == 0) {
            tc05::fence_after_sync();
            data_grad(T::Z3, T::WT3);
            weight_grad(T::G3, T::DTA, T::AT2, T::AT_LBO, ID80);
            weight_grad(T::G4, T::DTA, T::AT3, T::AT_LBO, ID80);
            tc05::commit(bar);
        }
        done = wait();
        bwd_epi(false, 0.0f, T::Z3, T::Z2, true, T::DTB, 0);
        if (__syncthreads_or(!done)) break;
        if (t == 0) {
            tc05::fence_after_sync();
            data_grad(T::Z2, T::WT2);
            weight_grad(T::G2, T::DTB, T::AT1, T::AT_LBO, ID80);
            tc05::commit(bar);
        }
        done = wait();
        bwd_epi(false, 0.0f, T::Z2, T::Z1, false, T::DTB, H);
        if (__syncthreads_or(!done)) break;
        if (t == 0) {
            tc05::fence_after_sync();
            weight_grad(T::G1, T::DTB, T::XT, T::XT_LBO, ID16);
            tc05::commit(bar);
        }
        done = wait();
        tc05::fence_before_sync();
        first = false;
    }

    float* out = part + (size_t)blockIdx.x * PSTRIDE;
    const bool failed = __syncthreads_or(!done);
    tc05::fence_after_sync();
    if (!failed) {
        // rows n of the layer-3 and layer-2 accumulators in warps 0-1 (lanes
        // 0-63), rows 64 + n of layer 1's and row 64 of layer 4's in warps 2-3
        uint32_t v[16];
        if (warp < 2) {
            const int nr = t;
#pragma unroll 1
            for (int g = 0; g < 2; ++g) {
                const uint32_t col = g == 0 ? T::G3 : T::G2;
                const int ow = g == 0 ? OW3 : OW2, ob = g == 0 ? OB3 : OB2;
#pragma unroll 1
                for (int c = 0; c < 5; ++c) {
                    tc05::ld16(trow + col + 16u * c, v);
                    tc05::wait16(v);
                    for (int e = 0; e < 16; ++e) {
                        const int k = 16 * c + e;
                        if (k < H) out[ow + nr * H + k] = __uint_as_float(v[e]);
                        else if (k == H) out[ob + nr] = __uint_as_float(v[e]);
                    }
                }
            }
        } else {
            const int nr = t - H;
            tc05::ld16(trow + T::G1, v);
            tc05::wait16(v);
            for (int k = 0; k < NIN; ++k) out[OW1 + nr * NIN + k] = __uint_as_float(v[k]);
            out[OB1 + nr] = __uint_as_float(v[NIN]);
#pragma unroll 1
            for (int c = 0; c < 5; ++c) {
                tc05::ld16(trow + T::G4 + 16u * c, v);
                tc05::wait16(v);
                if (t == H)
                    for (int e = 0; e < 16; ++e) {
                        const int k = 16 * c + e;
                        if (k < H) out[OW4 + k] = __uint_as_float(v[e]);
                        else if (k == H) out[OB4] = __uint_as_float(v[e]);
                    }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
        if (lane == 0) red[warp] = loss;
    } else {
        // a chain that did not complete in time: the partials are NaN, so
        // the step's loss and weights show it; wait once more, bounded,
        // before the accumulators are freed
        for (int i = t; i < PSTRIDE; i += blockDim.x) out[i] = __int_as_float(0x7fc00000);
        if (t == 0) gb_fail(st, GB_ST_TIMEOUT, -1, 0, 0, 0, 0.0);
        tc05::mbar_wait(bar, phase ^ 1u, TC_WAIT_CYCLES);
        tc05::mbar_wait(wbar, 0u, TC_WAIT_CYCLES);
    }
    tc05::fence_before_sync();
    __syncthreads();
    tc05::fence_after_sync();
    if (!failed && t == 0) out[NPAR] = (red[0] + red[1] + red[2] + red[3]) / (float)batch;
    if (warp == 0) tc05::dealloc(tm, T::TMEM_COLS);
}

// Adam on the FP32 master weights with the gradient summed over the
// training CTAs' partials (a fixed order: the result does not depend on
// scheduling), then the new value into the weight images; the last thread
// sums the loss
__global__ void k_adam_tc(int nparts, const float* __restrict__ part, float* __restrict__ w, float* __restrict__ m,
                          float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                          __nv_bfloat16* __restrict__ fw, __nv_bfloat16* __restrict__ wt, float* __restrict__ losses,
                          int it)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > NPAR) return;
    float g = 0.0f;
    for (int p = 0; p < nparts; ++p) g += part[(size_t)p * PSTRIDE + i];
    if (i == NPAR) {
        if (losses) losses[it] = g;
        return;
    }
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    put_param(i, wi, fw, wt);
}

// the gradient and loss of one pass: the partials summed in a fixed order
__global__ void k_reduce_parts(int nparts, const float* __restrict__ part, float* __restrict__ g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= PSTRIDE) return;
    float s = 0.0f;
    for (int p = 0; p < nparts; ++p) s += part[(size_t)p * PSTRIDE + i];
    g[i] = s;
}

// FP32 reference forward on CUDA cores with the same BF16-rounded weights
__global__ void k_mlp_infer_fp32(int64_t n, const float* __restrict__ feat, const float* __restrict__ w,
                                 float* __restrict__ y)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x[NIN], a[H], b[H];
    for (int c = 0; c < NIN; ++c) x[c] = bf16r(feat[i * NIN + c]);
    for (int o = 0; o < H; ++o) {
        float s = bf16r(w[OB1 + o]);
        for (int c = 0; c < NIN; ++c) s += bf16r(w[OW1 + o * NIN + c]) * x[c];
        a[o] = bf16r(silu(s));
    }
    for (int o = 0; o < H; ++o) {
        float s = bf16r(w[OB2 + o]);
        for (int c = 0; c < H; ++c) s += bf16r(w[OW2 + o * H + c]) * a[c];
        b[o] = bf16r(silu(s));
    }
    for (int o = 0; o < H; ++o) {
        float s = bf16r(w[OB3 + o]);
        for (int c = 0; c < H; ++c) s += bf16r(w[OW3 + o * H + c]) * b[c];
        a[o] = bf16r(silu(s));
    }
    float s = bf16r(w[OB4]);
    for (int c = 0; c < H; ++c) s += bf16r(w[OW4 + c]) * a[c];
    y[i] = s;
}

// ------------------------------------------------------------- state
struct mlp_state {
    float* w = nullptr;  // master FP32 params
    float* g = nullptr;  // gradient and loss of gb_mlp_grad (PSTRIDE)
    float* m = nullptr;
    float* v = nullptr;
    __nv_bfloat16* img = nullptr;  // forward weight image (inference and training)
    __nv_bfloat16* wt = nullptr;   // W^T images of layers 3 and 2 (training)
    float* part = nullptr;         // per-CTA partial gradients, one row per SM
    int sms = 0;
    int tc_blocks = 0;  // inference CTAs on the device
    int step = 0;
    bool packed = false;
} g_mlp;

int ensure_params()
{
    if (g_mlp.w) return GB_OK;
    int dev = 0, sms = 0;
    if (gb_check(cudaGetDevice(&dev), "device") ||
        gb_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count"))
        return GB_ERR_CUDA;
    const size_t b = sizeof(float) * NPAR;
    if (gb_check(cudaMalloc(&g_mlp.w, b), "mlp w") || gb_check(cudaMalloc(&g_mlp.g, sizeof(float) * PSTRIDE), "mlp g") ||
        gb_check(cudaMalloc(&g_mlp.m, b), "mlp m") || gb_check(cudaMalloc(&g_mlp.v, b), "mlp v") ||
        gb_check(cudaMalloc(&g_mlp.img, tc_layout::WBYTES), "mlp image") ||
        gb_check(cudaMalloc(&g_mlp.wt, 2 * tr_layout::WT_BYTES), "mlp transposed image") ||
        gb_check(cudaMalloc(&g_mlp.part, sizeof(float) * PSTRIDE * (size_t)sms), "mlp partials"))
        return GB_ERR_CUDA;
    // the inference CTAs: two fit an SM (shared memory, 512 TMEM columns,
    // registers); the grid is two per SM, and a CTA that finds no room
    // simply starts when another ends (they never wait on each other). A
    // training CTA holds a whole SM (shared memory and all 512 columns).
    if (gb_check(cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_layout::BYTES),
                 "k_mlp_infer_tc smem") ||
        gb_check(cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
                 "k_mlp_infer_tc carveout") ||
        gb_check(cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tr_layout::BYTES),
                 "k_mlp_train_tc smem"))
        return GB_ERR_CUDA;
    g_mlp.sms = sms;
    g_mlp.tc_blocks = 2 * sms;
    // the images' padding entries stay zero; the parameters' entries are
    // written by k_put_images and the Adam step
    cudaMemset(g_mlp.img, 0, tc_layout::WBYTES);
    cudaMemset(g_mlp.wt, 0, 2 * tr_layout::WT_BYTES);
    cudaMemset(g_mlp.m, 0, b);
    cudaMemset(g_mlp.v, 0, b);
    return GB_OK;
}

uint64_t splitmix(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// one training pass (forward, backward) over `batch` samples into the
// partials; returns the number of partial rows
int train_pass(const float* feat, const float* target, int64_t n, int batch, uint64_t seed, int step, int sample,
               cudaStream_t s)
{
    const int tiles = (batch + 127) / 128;
    const int grid = tiles < g_mlp.sms ? tiles : g_mlp.sms;
    k_mlp_train_tc<<<grid, 128, tr_layout::BYTES, s>>>(reinterpret_cast<const float4*>(feat), target, n, batch, seed,
                                                       step, sample, reinterpret_cast<const uint4*>(g_mlp.img),
                                                       reinterpret_cast<const uint4*>(g_mlp.wt), g_mlp.part, nullptr);
    return grid;
}

}  // namespace

extern "C" int gb_mlp_set_weights(const float* host, int n)
{
    if (!host || n != NPAR) return GB_ERR_ARG;
    int rc = ensure_params();
    if (rc) return rc;
    if (gb_check(cudaMemcpy(g_mlp.w, host, sizeof(float) * NPAR, cudaMemcpyHostToDevice), "mlp set")) return GB_ERR_CUDA;
    cudaMemset(g_mlp.m, 0, sizeof(float) * NPAR);
    cudaMemset(g_mlp.v, 0, sizeof(float) * NPAR);
    g_mlp.step = 0;
    g_mlp.packed = false;
    g_gb.gen += 1;
    return GB_OK;
}

extern "C" int gb_mlp_get_weights(float* host, int n)
{
    if (!host || n != NPAR || !g_mlp.w) return GB_ERR_ARG;
    return gb_check(cudaMemcpy(host, g_mlp.w, sizeof(float) * NPAR, cudaMemcpyDeviceToHost), "mlp get") ? GB_ERR_CUDA
                                                                                                       : GB_OK;
}

extern "C" int gb_mlp_init_random(uint64_t seed)
{
    // Glorot-uniform weights, zero biases
    float h[NPAR];
    uint64_t s = seed;
    auto uni = [&]() { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); };
    auto fill = [&](int off, int fan_in, int fan_out) {
        double a = sqrt(6.0 / (fan_in + fan_out));
        for (int i = 0; i < fan_in * fan_out; ++i) h[off + i] = (float)((2.0 * uni() - 1.0) * a);
    };
    memset(h, 0, sizeof h);
    fill(OW1, NIN, H);
    fill(OW2, H, H);
    fill(OW3, H, H);
    fill(OW4, H, 1);
    return gb_mlp_set_weights(h, NPAR);
}

extern "C" int gb_mlp_grad(const float* feat, const float* target, int n, float* grad_host, float* loss_host,
                           void* stream)
{
    if (!feat || !target || n <= 0 || n > (1 << 20) || !aligned16(feat) || !g_mlp.w) return GB_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = gb_mlp_pack(s);
    if (rc) return rc;
    const int parts = train_pass(feat, target, n, n, 0, 0, 0, s);
    k_reduce_parts<<<(PSTRIDE + 255) / 256, 256, 0, s>>>(parts, g_mlp.part, g_mlp.g);
    if (grad_host) cudaMemcpyAsync(grad_host, g_mlp.g, sizeof(float) * NPAR, cudaMemcpyDeviceToHost, s);
    if (loss_host) cudaMemcpyAsync(loss_host, g_mlp.g + NPAR, sizeof(float), cudaMemcpyDeviceToHost, s);
    return gb_check(cudaStreamSynchronize(s), "mlp grad") ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_mlp_train(const float* feat, const float* target, int64_t n, int steps, int batch, float lr,
                            uint64_t seed, float* loss_host, void* stream)
{
    if (!feat || !target || n <= 0 || steps <= 0 || batch <= 0 || batch > (1 << 20) || !aligned16(feat))
        return GB_ERR_ARG;
    int rc = ensure_params();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    rc = gb_mlp_pack(s);
    if (rc) return rc;
    float* dloss = nullptr;
    if (loss_host && gb_check(cudaMalloc(&dloss, sizeof(float) * (size_t)steps), "mlp losses")) return GB_ERR_CUDA;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < steps; ++it) {
        const int parts = train_pass(feat, target, n, batch, seed, it, 1, s);
        g_mlp.step += 1;
        // cosine decay of the learning rate over the run
        const float lrt = lr * 0.5f * (1.0f + cosf(3.14159265f * (float)it / (float)steps));
        const float c1 = 1.0f - powf(b1, (float)g_mlp.step), c2 = 1.0f - powf(b2, (float)g_mlp.step);
        k_adam_tc<<<(PSTRIDE + 255) / 256, 256, 0, s>>>(parts, g_mlp.part, g_mlp.w, g_mlp.m, g_mlp.v, lrt, b1, b2, eps,
                                                        c1, c2, g_mlp.img, g_mlp.wt, dloss, it);
    }
    if (dloss) cudaMemcpyAsync(loss_host, dloss, sizeof(float) * (size_t)steps, cudaMemcpyDeviceToHost, s);
    const bool bad = gb_check(cudaStreamSynchronize(s), "mlp train");
    if (dloss) cudaFree(dloss);
    g_mlp.packed = true;  // the Adam step keeps the images current
    g_gb.gen += 1;
    return bad ? GB_ERR_CUDA : GB_OK;
}

int gb_mlp_pack(cudaStream_t s)
{
    if (!g_mlp.w) {
        gb_set_error("surrogate has no weights");
        return GB_ERR_NOT_INIT;
    }
    if (g_mlp.packed) return GB_OK;
    k_put_images<<<(NPAR + 255) / 256, 256, 0, s>>>(g_mlp.w, g_mlp.img, g_mlp.wt);
    g_mlp.packed = true;
    return gb_check(cudaGetLastError(), "mlp pack") ? GB_ERR_CUDA : GB_OK;
}

int gb_mlp_launch_infer(int64_t n, const float* feat, float* y, gb_status* st, cudaStream_t s)
{
    int rc = gb_mlp_pack(s);
    if (rc) return rc;
    if (n <= 0) return GB_OK;
    const int64_t ctas = (n + tc_layout::M * tc_layout::WG - 1) / (tc_layout::M * tc_layout::WG);
    const unsigned grid = (unsigned)(ctas < g_mlp.tc_blocks ? ctas : g_mlp.tc_blocks);
    k_mlp_infer_tc<<<grid, 128 * tc_layout::WG, tc_layout::BYTES, s>>>(n, reinterpret_cast<const float4*>(feat),
                                                                      reinterpret_cast<const uint4*>(g_mlp.img), y, st);
    return gb_check(cudaGetLastError(), "k_mlp_infer_tc") ? GB_ERR_CUDA : GB_OK;
}

// Self-check of the bounded mbarrier wait the tcgen05 kernels use: one
// thread waits, for at most `limit` SM cycles, on a barrier that nothing
// arrives on (or, with `arrive`, on one it arrived on itself, which must
// complete at once) and records GB_ST_TIMEOUT when the wait gives up. No
// copy or MMA is in flight, so the context stays usable either way.
__global__ void k_wait_check(long long limit, int arrive, gb_status* st, int* result)
{
    __shared__ unsigned long long bar;
    if (threadIdx.x != 0) return;
    tc05::mbar_init(&bar, 1);
    if (arrive) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc05::saddr(&bar)) : "memory");
    const bool ok = tc05::mbar_wait(&bar, 0u, limit);
    if (!ok) gb_fail(st, GB_ST_TIMEOUT, -1, 0, 0, 0, (double)limit);
    *result = ok ? 1 : 2;
}

extern "C" int gb_check_bounded_wait(long long limit_cycles, int arrive, gb_status* st, int* result_host, void* stream)
{
    if (limit_cycles < 1000 || limit_cycles > 4000000000LL || !result_host) return GB_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int* d = nullptr;
    if (gb_check(cudaMalloc(&d, sizeof(int)), "wait check")) return GB_ERR_CUDA;
    k_wait_check<<<1, 32, 0, s>>>(limit_cycles, arrive, st, d);
    cudaMemcpyAsync(result_host, d, sizeof(int), cudaMemcpyDeviceToHost, s);
    const bool bad = gb_check(cudaStreamSynchronize(s), "k_wait_check");
    cudaFree(d);
    return bad ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_mlp_infer(int64_t n, const float* feat, float* y, int tensor_cores, void* stream)
{
    if (n < 0 || (n > 0 && (!feat || !y || !aligned16(feat)))) return GB_ERR_ARG;
    if (!g_mlp.w) {
        gb_set_error("gb_mlp_infer: no weights");
        return GB_ERR_NOT_INIT;
    }
    if (n == 0) return GB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (tensor_cores) return gb_mlp_launch_infer(n, feat, y, nullptr, s);
    k_mlp_infer_fp32<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(n, feat, g_mlp.w, y);
    return gb_check(cudaGetLastError(), "k_mlp_infer_fp32") ? GB_ERR_CUDA : GB_OK;
}
