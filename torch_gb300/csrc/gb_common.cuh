// Shared device-side definitions of the gbhydro library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbhydro.h"

#define GB_N GB_NB
#define GB_N3 (GB_NB * GB_NB * GB_NB)
#define GB_FSZ (GB_NB * GB_NB * (GB_NB + 1))

// Guard-fill plan entry flags (the plan: for every leaf and each of the 27
// block-sized regions around it, two int4 {node, level, flags, 0},
// {cx, cy, cz, 0}; region r = rx + 3 ry + 9 rz, offsets -1..1 per axis)
constexpr int GP_REFINED = 1;   // a node of the leaf's level with children
constexpr int GP_LEAFKIDS = 2;  // ... whose children are all leaves

// Record the first failure in the status word and count it.
__device__ __forceinline__ void gb_fail(gb_status* st, int code, int blk, int i, int j, int k,
                                        double v)
{
    if (!st) return;
    if (atomicCAS(&st->code, 0, code) == 0) {
        st->block = blk;
        st->i = i;
        st->j = j;
        st->k = k;
        st->value = v;
    }
}

__device__ __forceinline__ void gb_count(unsigned long long* c, unsigned long long n = 1)
{
    if (c) atomicAdd(c, n);
}

// Warp-aggregated counter increment (one atomic per warp).
__device__ __forceinline__ void gb_count_warp(unsigned long long* c, bool pred)
{
    unsigned m = __ballot_sync(__activemask(), pred);
    if (m && (threadIdx.x & 31) == (__ffs(__activemask()) - 1)) {
        if (c) atomicAdd(c, (unsigned long long)__popc(m));
    }
}

// Grid state shared by the kernels of one registration.
struct gb_dev_grid {
    int nvar;
    int maxblocks;
    int slot[GB_NROLE];
    double* unk;
    double* f[3];
    const int* level; // refinement level per store block (NULL: all level 0)
};

// cell size of a block: root cell size scaled by 2^-level (exact)
// FP64 <-> FP32 conversions on the integer pipe. GB300's FP64 pipe, which
// also executes the hardware conversions, is the bottleneck of the mixed
// path while the integer pipe idles. Both are IEEE conversions (float ->
// double exact, double -> float round-to-nearest-even), written from the
// binary64/binary32 encodings; zero and normal values take the integer
// path, everything else (subnormal results, overflow, inf, nan) the
// hardware one.
__device__ __forceinline__ float gb_d2f(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    if (((hi & 0x7FFFFFFFu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);  // +-0
    const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
    if (e <= 0 || e >= 255) return (float)x;
    // the top 23 of the 52 mantissa bits: 20 from hi, 3 from lo; 29 dropped
    unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1FFFFFFFu, half = 0x10000000u;
    m += (unsigned)((rem > half) | ((rem == half) & (m & 1u)));
    // a mantissa carry (m == 2^23) moves into the exponent; e == 254 with a
    // carry gives +-inf, the correctly rounded overflow
    return __uint_as_float((hi & 0x80000000u) | (((unsigned)e << 23) + m));
}

__device__ __forceinline__ double gb_f2d(float x)
{
    const unsigned u = __float_as_uint(x);
    const unsigned ex = (u >> 23) & 0xFFu;
    if ((u & 0x7FFFFFFFu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);  // +-0
    if (ex == 0u || ex == 255u) return (double)x;
    const unsigned hi = (u & 0x80000000u) | ((ex + (1023u - 127u)) << 20) | ((u & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}

// 2^l as a double, built from its exponent bits (0 <= l < 1023)
__device__ __forceinline__ double gb_pow2(int l) { return __longlong_as_double((long long)(1023 + l) << 52); }

__device__ __forceinline__ int gb_block_level(const gb_dev_grid& g, int blk) { return g.level ? __ldg(g.level + blk) : 0; }

__device__ __forceinline__ void gb_block_dx(const gb_dev_grid& g, const double* dx0, int blk, double* dx)
{
    double sc = g.level ? ldexp(1.0, -__ldg(g.level + blk)) : 1.0;
    dx[0] = dx0[0] * sc;
    dx[1] = dx0[1] * sc;
    dx[2] = dx0[2] * sc;
}

__device__ __forceinline__ double* gb_var(const gb_dev_grid& g, int blk, int role)
{
    return g.unk + ((int64_t)blk * g.nvar + g.slot[role]) * GB_N3;
}

__host__ __device__ __forceinline__ int gb_cidx(int i, int j, int k)
{
    return i + GB_N * (j + GB_N * k);
}

// face index of face array d (face coordinate along d runs 0..GB_N)
__host__ __device__ __forceinline__ int gb_fidx(int d, int i, int j, int k)
{
    return d == 0 ? i + (GB_N + 1) * (j + GB_N * k)
                  : (d == 1 ? i + GB_N * (j + (GB_N + 1) * k) : i + GB_N * (j + GB_N * k));
}

// ---- host-side helpers implemented in capi.cu
void gb_set_error(const char* fmt, ...);
int gb_check(cudaError_t e, const char* what);
