// Learned cooling surrogate: a 4 -> 64 -> 64 -> 64 -> 1 SiLU MLP.
//
// Training runs in FP32 on CUDA cores with hand-written kernels (tiled
// GEMM, SiLU forward/backward, squared-error loss, Adam); the forward pass
// uses weights rounded to BF16 so training sees the inference weights.
// Inference keeps BF16 weights and FP32 accumulation on the tensor cores
// (mma.sync m16n8k16); the accumulator fragment of one layer is the A
// fragment of the next, so activations never leave registers.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include "gb_state.h"
#include "mlp.h"

namespace {

constexpr int H = GB_MLP_HIDDEN;  // 64
constexpr int NIN = GB_MLP_IN;    // 4

// parameter offsets in the flat FP32 vector
constexpr int OW1 = 0, OB1 = OW1 + H * NIN, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H,
              OB3 = OW3 + H * H, OW4 = OB3 + H, OB4 = OW4 + H, NPAR = OB4 + 1;
static_assert(NPAR == GB_MLP_NPARAM, "parameter count");

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z)
{
    float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// C[M x N] = act(A[M x K] * op(B) + bias), row-major; op(B) = B^T when
// tb (B stored N x K, the weight layout [out][in]) else B (K x N).
// ta: A stored K x M (used for weight gradients: A^T * dZ).
template <int TILE>
__global__ void k_gemm(int M, int N, int K, const float* __restrict__ A, int lda, int ta,
                       const float* __restrict__ B, int ldb, int tb, float* __restrict__ Cm, int ldc,
                       const float* __restrict__ bias, int round_b, float beta)
{
    __shared__ float sa[TILE][TILE + 1];
    __shared__ float sb[TILE][TILE + 1];
    const int tx = threadIdx.x % TILE, ty = threadIdx.x / TILE;
    const int row = blockIdx.y * TILE + ty, col = blockIdx.x * TILE + tx;
    float acc = 0.0f;
    for (int k0 = 0; k0 < K; k0 += TILE) {
        int ka = k0 + tx, kb = k0 + ty;
        float av = 0.0f, bv = 0.0f;
        if (row < M && ka < K) av = ta ? A[(size_t)ka * lda + row] : A[(size_t)row * lda + ka];
        int bcol = blockIdx.x * TILE + tx;
        if (kb < K && bcol < N) bv = tb ? B[(size_t)bcol * ldb + kb] : B[(size_t)kb * ldb + bcol];
        if (round_b) bv = bf16r(bv);
        sa[ty][tx] = av;
        sb[ty][tx] = bv;
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TILE; ++kk) acc += sa[ty][kk] * sb[kk][tx];
        __syncthreads();
    }
    if (row < M && col < N) {
        float v = acc + (bias ? (round_b ? bf16r(bias[col]) : bias[col]) : 0.0f);
        float* c = Cm + (size_t)row * ldc + col;
        *c = beta != 0.0f ? beta * *c + v : v;
    }
}

__global__ void k_silu(int n, const float* __restrict__ z, float* __restrict__ a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = silu(z[i]);
}

__global__ void k_silu_back(int n, const float* __restrict__ z, float* __restrict__ d)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] *= silu_grad(z[i]);
}

// dY = 2 (Y - T) / B over valid rows; loss sum -> *loss
__global__ void k_mse(int n, const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ dy,
                      float* __restrict__ loss)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < n) {
        float r = y[i] - t[i];
        dy[i] = 2.0f * r / (float)n;
        l = r * r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l / (float)n);
}

// column sums of dZ [M x N] -> db[N]
__global__ void k_colsum(int M, int N, const float* __restrict__ dz, float* __restrict__ db)
{
    int c = blockIdx.x;
    float s = 0.0f;
    for (int r = threadIdx.x; r < M; r += blockDim.x) s += dz[(size_t)r * N + c];
    __shared__ float red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[c] = red[0];
}

__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gi = g[i];
    float mi = b1 * m[i] + (1.0f - b1) * gi;
    float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_gather(int n, const int* __restrict__ idx, const float* __restrict__ feat,
                         const float* __restrict__ tgt, float* __restrict__ x, float* __restrict__ t)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int j = idx[i];
#pragma unroll
    for (int c = 0; c < NIN; ++c) x[(size_t)i * NIN + c] = feat[(size_t)j * NIN + c];
    t[i] = tgt[j];
}

// ------------------------------------------------------------- inference
// weights packed as BF16 in the B-operand order of mma.m16n8k16 (.col:
// element (k, n) at n * K + k), layer 1 padded to K = 16, layer 4 to N = 8.
// Rows of each matrix are padded by 8 elements (16 bytes): a B-fragment
// load then has the 8 rows of a warp start 4 banks apart, so the 32 lanes
// hit 32 distinct banks (unpadded 128-byte rows put all 8 rows on the same
// 4 banks, an 8-way conflict).
struct packed_layout {
    static constexpr int P1 = 16 + 8, PH = H + 8;  // row pitches (elements)
    static constexpr int W1 = 0;                 // 64 x 16
    static constexpr int W2 = W1 + H * P1;       // 64 x 64
    static constexpr int W3 = W2 + H * PH;       // 64 x 64
    static constexpr int W4 = W3 + H * PH;       // 8 x 64
    static constexpr int N = W4 + 8 * PH;
};

__global__ void k_pack_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ pk, float* __restrict__ pb)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    using PL = packed_layout;
    if (i < H * PL::P1) {
        int n = i / PL::P1, k = i % PL::P1;
        pk[PL::W1 + i] = __float2bfloat16_rn(k < NIN ? w[OW1 + n * NIN + k] : 0.0f);
    }
    if (i < H * PL::PH) {
        int n = i / PL::PH, k = i % PL::PH;
        pk[PL::W2 + i] = __float2bfloat16_rn(k < H ? w[OW2 + n * H + k] : 0.0f);
        pk[PL::W3 + i] = __float2bfloat16_rn(k < H ? w[OW3 + n * H + k] : 0.0f);
    }
    if (i < 8 * PL::PH) {
        int n = i / PL::PH, k = i % PL::PH;
        pk[PL::W4 + i] = __float2bfloat16_rn(n == 0 && k < H ? w[OW4 + k] : 0.0f);
    }
    // biases stay FP32 (they are added to the FP32 accumulator), rounded to
    // BF16 values to match training
    if (i < H) {
        pb[i] = bf16r(w[OB1 + i]);
        pb[H + i] = bf16r(w[OB2 + i]);
        pb[2 * H + i] = bf16r(w[OB3 + i]);
    }
    if (i == 0) pb[3 * H] = bf16r(w[OB4]);
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// B fragment (two .b32) for k-tile kt, n-tile nt of a layer whose rows
// are `pitch` elements apart
__device__ __forceinline__ void bfrag(const __nv_bfloat16* w, int pitch, int kt, int nt, int lane, uint32_t& b0,
                                      uint32_t& b1)
{
    int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* p = w + (nt * 8 + g) * pitch + kt * 16 + t * 2;
    b0 = *reinterpret_cast<const uint32_t*>(p);
    b1 = *reinterpret_cast<const uint32_t*>(p + 8);
}

// SiLU for inference: z sigmoid(z) = h (1 + tanh h), h = z / 2, with the
// hardware tanh approximation (one MUFU operation; its ~2^-11 relative
// error is below the BF16 rounding the activation gets next)
__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float silu_infer(float z)
{
    const float h = 0.5f * z;
    return fmaf(h, tanh_approx(h), h);
}

__device__ __forceinline__ uint32_t silu_pair(float z0, float z1) { return pack2(silu_infer(z0), silu_infer(z1)); }

// one hidden layer for NT 16-row tiles: acc[tile][8 n-tiles][4] = A(16 x K)
// W^T + bias, then SiLU and repack to the A fragments of the next layer.
// Each B fragment is read from shared memory once for all NT tiles.
template <int KT, int NT>
__device__ __forceinline__ void hidden_layer(const uint32_t (*afr)[4][4], const __nv_bfloat16* w, const float* bias,
                                             int lane, uint32_t (*anext)[4][4])
{
    const int t = lane & 3;
    float acc[NT][8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float b0 = bias[nt * 8 + t * 2], b1 = bias[nt * 8 + t * 2 + 1];
#pragma unroll
        for (int q = 0; q < NT; ++q) {
            acc[q][nt][0] = b0; acc[q][nt][1] = b1; acc[q][nt][2] = b0; acc[q][nt][3] = b1;
        }
    }
#pragma unroll
    for (int kt = 0; kt < KT; ++kt)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            uint32_t b0, b1;
            bfrag(w, KT * 16 + 8, kt, nt, lane, b0, b1);
#pragma unroll
            for (int q = 0; q < NT; ++q) mma_bf16(acc[q][nt], afr[q][kt], b0, b1);
        }
#pragma unroll
    for (int q = 0; q < NT; ++q)
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            anext[q][kt][0] = silu_pair(acc[q][2 * kt][0], acc[q][2 * kt][1]);
            anext[q][kt][1] = silu_pair(acc[q][2 * kt][2], acc[q][2 * kt][3]);
            anext[q][kt][2] = silu_pair(acc[q][2 * kt + 1][0], acc[q][2 * kt + 1][1]);
            anext[q][kt][3] = silu_pair(acc[q][2 * kt + 1][2], acc[q][2 * kt + 1][3]);
        }
}

constexpr int INFER_NT = 2;  // 16-row tiles per warp iteration

__global__ void __launch_bounds__(128, 4) k_mlp_infer(int64_t n, const float* __restrict__ feat,
                                                   const __nv_bfloat16* __restrict__ wpk,
                                                   const float* __restrict__ bias, float* __restrict__ y)
{
    __shared__ __align__(16) __nv_bfloat16 sw[packed_layout::N];
    __shared__ float sbias[3 * H + 1];
    for (int i = threadIdx.x; i < packed_layout::N / 2; i += blockDim.x)
        reinterpret_cast<uint32_t*>(sw)[i] = reinterpret_cast<const uint32_t*>(wpk)[i];
    for (int i = threadIdx.x; i < 3 * H + 1; i += blockDim.x) sbias[i] = bias[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    constexpr int NT = INFER_NT;
    const int64_t ngroups = (n + 16 * NT - 1) / (16 * NT);
    const int64_t gstep = (int64_t)gridDim.x * 4;
    // the features of a warp's next group are loaded while it computes the
    // current one (the only global loads of the kernel)
    auto load_feat = [&](int64_t grp, float4 (*fv)[2]) {
#pragma unroll
        for (int q = 0; q < NT; ++q) {
            const int64_t ra = (grp * NT + q) * 16 + g, rb = ra + 8;
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            fv[q][0] = (grp < ngroups && ra < n) ? reinterpret_cast<const float4*>(feat)[ra] : z;
            fv[q][1] = (grp < ngroups && rb < n) ? reinterpret_cast<const float4*>(feat)[rb] : z;
        }
    };
    float4 fnext[NT][2];
    load_feat((int64_t)blockIdx.x * 4 + warp, fnext);
    for (int64_t grp = (int64_t)blockIdx.x * 4 + warp; grp < ngroups; grp += gstep) {
        // layer 1 A fragments: features in columns 0..3, zero-padded to 16;
        // columns t*2, t*2+1 (only t < 2 carry features)
        uint32_t a1[NT][4][4];
        int64_t r0[NT];
#pragma unroll
        for (int q = 0; q < NT; ++q) {
            r0[q] = (grp * NT + q) * 16 + g;
            const float f0[4] = {fnext[q][0].x, fnext[q][0].y, fnext[q][0].z, fnext[q][0].w};
            const float f1[4] = {fnext[q][1].x, fnext[q][1].y, fnext[q][1].z, fnext[q][1].w};
            a1[q][0][0] = t < 2 ? pack2(f0[t * 2], f0[t * 2 + 1]) : 0u;
            a1[q][0][1] = t < 2 ? pack2(f1[t * 2], f1[t * 2 + 1]) : 0u;
            a1[q][0][2] = 0u;
            a1[q][0][3] = 0u;
        }
        load_feat(grp + gstep, fnext);
        uint32_t h1[NT][4][4], h2[NT][4][4];
        hidden_layer<1, NT>(a1, sw + packed_layout::W1, sbias, lane, h1);
        hidden_layer<4, NT>(h1, sw + packed_layout::W2, sbias + H, lane, h2);
        hidden_layer<4, NT>(h2, sw + packed_layout::W3, sbias + 2 * H, lane, h1);
        float out[NT][4];
#pragma unroll
        for (int q = 0; q < NT; ++q) {
            out[q][0] = sbias[3 * H]; out[q][1] = 0.0f; out[q][2] = sbias[3 * H]; out[q][3] = 0.0f;
        }
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            uint32_t b0, b1;
            bfrag(sw + packed_layout::W4, packed_layout::PH, kt, 0, lane, b0, b1);
#pragma unroll
            for (int q = 0; q < NT; ++q) mma_bf16(out[q], h1[q][kt], b0, b1);
        }
        // column 0 lives in the t == 0 lanes: out[0] row g, out[2] row g + 8
        if (t == 0) {
#pragma unroll
            for (int q = 0; q < NT; ++q) {
                if (r0[q] < n) y[r0[q]] = out[q][0];
                if (r0[q] + 8 < n) y[r0[q] + 8] = out[q][2];
            }
        }
    }
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
    float* w = nullptr;   // master FP32 params
    float* g = nullptr;   // gradients
    float* m = nullptr;
    float* v = nullptr;
    __nv_bfloat16* pk = nullptr;
    float* pb = nullptr;
    int step = 0;
    bool packed = false;
    // training buffers
    int cap = 0;
    float *x = nullptr, *t = nullptr, *z1 = nullptr, *a1 = nullptr, *z2 = nullptr, *a2 = nullptr, *z3 = nullptr,
          *a3 = nullptr, *yv = nullptr, *dy = nullptr, *d3 = nullptr, *d2 = nullptr, *d1 = nullptr,
          *loss = nullptr;
    int* idx = nullptr;
} g_mlp;

int ensure_params()
{
    if (g_mlp.w) return GB_OK;
    size_t b = sizeof(float) * NPAR;
    if (gb_check(cudaMalloc(&g_mlp.w, b), "mlp w") || gb_check(cudaMalloc(&g_mlp.g, b), "mlp g") ||
        gb_check(cudaMalloc(&g_mlp.m, b), "mlp m") || gb_check(cudaMalloc(&g_mlp.v, b), "mlp v") ||
        gb_check(cudaMalloc(&g_mlp.pk, sizeof(__nv_bfloat16) * packed_layout::N), "mlp pk") ||
        gb_check(cudaMalloc(&g_mlp.pb, sizeof(float) * (3 * H + 1)), "mlp pb"))
        return GB_ERR_CUDA;
    cudaMemset(g_mlp.m, 0, b);
    cudaMemset(g_mlp.v, 0, b);
    return GB_OK;
}

int ensure_batch(int B)
{
    if (B <= g_mlp.cap) return GB_OK;
    float** bufs[] = {&g_mlp.z1, &g_mlp.a1, &g_mlp.z2, &g_mlp.a2, &g_mlp.z3, &g_mlp.a3, &g_mlp.d3, &g_mlp.d2,
                      &g_mlp.d1};
    for (float** p : bufs) {
        if (*p) cudaFree(*p);
        if (gb_check(cudaMalloc(p, sizeof(float) * (size_t)B * H), "mlp batch")) return GB_ERR_CUDA;
    }
    float** small[] = {&g_mlp.x, &g_mlp.t, &g_mlp.yv, &g_mlp.dy};
    for (float** p : small) {
        if (*p) cudaFree(*p);
        if (gb_check(cudaMalloc(p, sizeof(float) * (size_t)B * NIN), "mlp batch")) return GB_ERR_CUDA;
    }
    if (g_mlp.idx) cudaFree(g_mlp.idx);
    if (!g_mlp.loss && gb_check(cudaMalloc(&g_mlp.loss, sizeof(float)), "mlp loss")) return GB_ERR_CUDA;
    if (gb_check(cudaMalloc(&g_mlp.idx, sizeof(int) * (size_t)B), "mlp idx")) return GB_ERR_CUDA;
    g_mlp.cap = B;
    return GB_OK;
}

void gemm(cudaStream_t s, int M, int N, int K, const float* A, int lda, int ta, const float* B, int ldb, int tb,
          float* Cm, int ldc, const float* bias, int round_b)
{
    constexpr int T = 16;
    dim3 grid((N + T - 1) / T, (M + T - 1) / T);
    k_gemm<T><<<grid, T * T, 0, s>>>(M, N, K, A, lda, ta, B, ldb, tb, Cm, ldc, bias, round_b, 0.0f);
}

// forward + backward of one batch already in g_mlp.x / g_mlp.t; gradients
// into g_mlp.g, loss into g_mlp.loss
void fwd_bwd(int B, cudaStream_t s)
{
    const float* w = g_mlp.w;
    float* gr = g_mlp.g;
    const int nb = (B * H + 255) / 256;
    gemm(s, B, H, NIN, g_mlp.x, NIN, 0, w + OW1, NIN, 1, g_mlp.z1, H, w + OB1, 1);
    k_silu<<<nb, 256, 0, s>>>(B * H, g_mlp.z1, g_mlp.a1);
    gemm(s, B, H, H, g_mlp.a1, H, 0, w + OW2, H, 1, g_mlp.z2, H, w + OB2, 1);
    k_silu<<<nb, 256, 0, s>>>(B * H, g_mlp.z2, g_mlp.a2);
    gemm(s, B, H, H, g_mlp.a2, H, 0, w + OW3, H, 1, g_mlp.z3, H, w + OB3, 1);
    k_silu<<<nb, 256, 0, s>>>(B * H, g_mlp.z3, g_mlp.a3);
    gemm(s, B, 1, H, g_mlp.a3, H, 0, w + OW4, H, 1, g_mlp.yv, 1, w + OB4, 1);
    cudaMemsetAsync(g_mlp.loss, 0, sizeof(float), s);
    k_mse<<<(B + 255) / 256, 256, 0, s>>>(B, g_mlp.yv, g_mlp.t, g_mlp.dy, g_mlp.loss);
    // layer 4: dW4 = dy^T a3 (1 x 64), db4 = sum dy, d3 = dy W4 (B x 64)
    gemm(s, 1, H, B, g_mlp.dy, 1, 1, g_mlp.a3, H, 0, gr + OW4, H, nullptr, 0);
    k_colsum<<<1, 256, 0, s>>>(B, 1, g_mlp.dy, gr + OB4);
    gemm(s, B, H, 1, g_mlp.dy, 1, 0, w + OW4, H, 0, g_mlp.d3, H, nullptr, 1);
    k_silu_back<<<nb, 256, 0, s>>>(B * H, g_mlp.z3, g_mlp.d3);
    gemm(s, H, H, B, g_mlp.d3, H, 1, g_mlp.a2, H, 0, gr + OW3, H, nullptr, 0);
    k_colsum<<<H, 256, 0, s>>>(B, H, g_mlp.d3, gr + OB3);
    gemm(s, B, H, H, g_mlp.d3, H, 0, w + OW3, H, 0, g_mlp.d2, H, nullptr, 1);
    k_silu_back<<<nb, 256, 0, s>>>(B * H, g_mlp.z2, g_mlp.d2);
    gemm(s, H, H, B, g_mlp.d2, H, 1, g_mlp.a1, H, 0, gr + OW2, H, nullptr, 0);
    k_colsum<<<H, 256, 0, s>>>(B, H, g_mlp.d2, gr + OB2);
    gemm(s, B, H, H, g_mlp.d2, H, 0, w + OW2, H, 0, g_mlp.d1, H, nullptr, 1);
    k_silu_back<<<nb, 256, 0, s>>>(B * H, g_mlp.z1, g_mlp.d1);
    gemm(s, H, NIN, B, g_mlp.d1, H, 1, g_mlp.x, NIN, 0, gr + OW1, NIN, nullptr, 0);
    k_colsum<<<H, 256, 0, s>>>(B, H, g_mlp.d1, gr + OB1);
}

uint64_t splitmix(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
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
    if (!feat || !target || n <= 0 || !g_mlp.w) return GB_ERR_ARG;
    int rc = ensure_batch(n);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemcpyAsync(g_mlp.x, feat, sizeof(float) * (size_t)n * NIN, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(g_mlp.t, target, sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    fwd_bwd(n, s);
    if (grad_host) cudaMemcpyAsync(grad_host, g_mlp.g, sizeof(float) * NPAR, cudaMemcpyDeviceToHost, s);
    if (loss_host) cudaMemcpyAsync(loss_host, g_mlp.loss, sizeof(float), cudaMemcpyDeviceToHost, s);
    return gb_check(cudaStreamSynchronize(s), "mlp grad") ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_mlp_train(const float* feat, const float* target, int64_t n, int steps, int batch, float lr,
                            uint64_t seed, float* loss_host, void* stream)
{
    if (!feat || !target || n <= 0 || steps <= 0 || batch <= 0 || batch > (1 << 20)) return GB_ERR_ARG;
    int rc = ensure_params();
    if (rc) return rc;
    rc = ensure_batch(batch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int* hidx = nullptr;
    if (gb_check(cudaMallocHost(&hidx, sizeof(int) * (size_t)batch), "pinned idx")) return GB_ERR_CUDA;
    uint64_t st = seed;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = 0; it < steps; ++it) {
        cudaStreamSynchronize(s);  // hidx is reused
        for (int i = 0; i < batch; ++i) hidx[i] = (int)(splitmix(st) % (uint64_t)n);
        cudaMemcpyAsync(g_mlp.idx, hidx, sizeof(int) * batch, cudaMemcpyHostToDevice, s);
        k_gather<<<(batch + 255) / 256, 256, 0, s>>>(batch, g_mlp.idx, feat, target, g_mlp.x, g_mlp.t);
        fwd_bwd(batch, s);
        g_mlp.step += 1;
        // cosine decay of the learning rate over the run
        float lrt = lr * 0.5f * (1.0f + cosf(3.14159265f * (float)it / (float)steps));
        float c1 = 1.0f - powf(b1, (float)g_mlp.step), c2 = 1.0f - powf(b2, (float)g_mlp.step);
        k_adam<<<(NPAR + 255) / 256, 256, 0, s>>>(NPAR, g_mlp.w, g_mlp.g, g_mlp.m, g_mlp.v, lrt, b1, b2, eps, c1, c2);
        if (loss_host) cudaMemcpyAsync(loss_host + it, g_mlp.loss, sizeof(float), cudaMemcpyDeviceToHost, s);
    }
    cudaStreamSynchronize(s);
    cudaFreeHost(hidx);
    g_mlp.packed = false;
    g_gb.gen += 1;
    return gb_check(cudaGetLastError(), "mlp train") ? GB_ERR_CUDA : GB_OK;
}

int gb_mlp_pack(cudaStream_t s)
{
    if (!g_mlp.w) {
        gb_set_error("surrogate has no weights");
        return GB_ERR_NOT_INIT;
    }
    if (g_mlp.packed) return GB_OK;
    k_pack_bf16<<<(H * packed_layout::PH + 255) / 256, 256, 0, s>>>(g_mlp.w, g_mlp.pk, g_mlp.pb);
    g_mlp.packed = true;
    return gb_check(cudaGetLastError(), "mlp pack") ? GB_ERR_CUDA : GB_OK;
}

int gb_mlp_launch_infer(int64_t n, const float* feat, float* y, cudaStream_t s)
{
    int rc = gb_mlp_pack(s);
    if (rc) return rc;
    int64_t groups = (n + 16 * INFER_NT - 1) / (16 * INFER_NT);
    int64_t blocks = (groups + 3) / 4;
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (blocks < 1) blocks = 1;
    k_mlp_infer<<<(unsigned)blocks, 128, 0, s>>>(n, feat, g_mlp.pk, g_mlp.pb, y);
    return gb_check(cudaGetLastError(), "k_mlp_infer") ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_mlp_infer(int64_t n, const float* feat, float* y, int tensor_cores, void* stream)
{
    if (n < 0 || (n > 0 && (!feat || !y))) return GB_ERR_ARG;
    if (!g_mlp.w) {
        gb_set_error("gb_mlp_infer: no weights");
        return GB_ERR_NOT_INIT;
    }
    if (n == 0) return GB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (tensor_cores) return gb_mlp_launch_infer(n, feat, y, s);
    k_mlp_infer_fp32<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(n, feat, g_mlp.w, y);
    return gb_check(cudaGetLastError(), "k_mlp_infer_fp32") ? GB_ERR_CUDA : GB_OK;
}
