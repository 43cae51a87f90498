// Shared device-side definitions of the gbhydro library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbhydro.h"

#define GB_N GB_NB
#define GB_N3 (GB_NB * GB_NB * GB_NB)
#define GB_FSZ (GB_NB * GB_NB * (GB_NB + 1))

// ---------------------------------------------------------------- the step's read region
// Every cell and face a step reads, per block: the reconstruction band
// (cells 3..20 on every axis) and the 5-point stencil's reach along one
// axis at a time (cells 1, 2, 21, 22 on that axis, 3..20 on the others);
// faces 3..21 along their normal and 3..20 across. The step's guard fill
// and its FP32 primitive copy cover this region widened to whole 32-byte
// sectors along x (full rows, or the 4-cell groups at either end of a
// row): a partial sector would cost a read-modify-write of the sector in
// HBM, more than the few cells the widening adds.
constexpr int GB_BAND_LO = GB_NGUARD - 1, GB_BAND = GB_NXB + 2;  // 3, 18

// guard cells: z slabs (k = 3, 20 with j = 1..22; k = 1, 2, 21, 22 with
// j = 3..20), y slabs (k = 4..19; j = 1, 2, 3, 20, 21, 22), full rows in
// x; x slabs (j, k = 4..19; i = 0..3, 20..23)
constexpr int GSZ_A = 2 * (GB_N - 2) * GB_N, GSZ_B = 4 * GB_BAND * GB_N;
constexpr int GSY = GB_NXB * 6 * GB_N, GSX = GB_NXB * GB_NXB * 8;
constexpr int GB_STEP_GUARD_CELLS = GSZ_A + GSZ_B + GSY + GSX;  // 7136
__device__ __forceinline__ void gb_step_guard_cell(int q, int& i, int& j, int& k)
{
    if (q < GSZ_A) {
        const int zz = q / ((GB_N - 2) * GB_N), rr = q - zz * ((GB_N - 2) * GB_N);
        k = zz ? GB_BAND_LO + GB_BAND - 1 : GB_BAND_LO;
        j = 1 + rr / GB_N;
        i = rr % GB_N;
    } else if (q < GSZ_A + GSZ_B) {
        q -= GSZ_A;
        const int zz = q / (GB_BAND * GB_N), rr = q - zz * (GB_BAND * GB_N);
        k = zz < 2 ? 1 + zz : GB_N - 5 + zz;  // 1, 2, 21, 22
        j = GB_BAND_LO + rr / GB_N;
        i = rr % GB_N;
    } else if (q < GSZ_A + GSZ_B + GSY) {
        q -= GSZ_A + GSZ_B;
        const int kk = q / (6 * GB_N), rr = q - kk * (6 * GB_N);
        const int yy = rr / GB_N;
        k = GB_NGUARD + kk;
        j = yy < 3 ? 1 + yy : GB_N - 7 + yy;  // 1, 2, 3, 20, 21, 22
        i = rr % GB_N;
    } else {
        q -= GSZ_A + GSZ_B + GSY;
        const int xx = q & 7, rr = q >> 3;
        i = xx < 4 ? xx : GB_N - 8 + xx;  // 0..3, 20..23
        j = GB_NGUARD + rr % GB_NXB;
        k = GB_NGUARD + rr / GB_NXB;
    }
}

// cells of the FP32 copy: whole rows (j, k) in the band, the y arms and
// the z arms
constexpr int GB_STEP_ROWS = GB_BAND * GB_BAND + 2 * 4 * GB_BAND;  // 468
constexpr int GB_STEP_CELLS = GB_STEP_ROWS * GB_N;                  // 11232
static_assert(GB_N % 4 == 0 && (GB_N3 * 8) % 32 == 0, "four-cell groups of the FP32 copy are 16-byte aligned");
__device__ __forceinline__ void gb_step_cell(int q, int& i, int& j, int& k)
{
    const int row = q / GB_N;
    i = q - row * GB_N;
    if (row < GB_BAND * GB_BAND) {
        j = GB_BAND_LO + row % GB_BAND;
        k = GB_BAND_LO + row / GB_BAND;
    } else if (row < GB_BAND * GB_BAND + 4 * GB_BAND) {
        const int r = row - GB_BAND * GB_BAND, a = r / GB_BAND;
        j = a < 2 ? 1 + a : GB_N - 5 + a;
        k = GB_BAND_LO + r % GB_BAND;
    } else {
        const int r = row - GB_BAND * GB_BAND - 4 * GB_BAND, a = r / GB_BAND;
        j = GB_BAND_LO + r % GB_BAND;
        k = a < 2 ? 1 + a : GB_N - 5 + a;
    }
}

// faces of the FP32 copy, per axis a: whole x rows, j = 3..20 (..21 for
// a = 1), k = 3..20 (..21 for a = 2)
__host__ __device__ constexpr int gb_step_faces(int a)
{
    return (GB_N + (a == 0)) * (GB_BAND + (a == 1)) * (GB_BAND + (a == 2));
}
constexpr int GB_STEP_FACES_ALL = gb_step_faces(0) + gb_step_faces(1) + gb_step_faces(2);

// The q-th position of the shell of width W of an N0 x N1 x N2 box (box
// coordinates): the two z slabs, the two y slabs inside them, the two x
// slabs inside those, x fastest.
template <int N0, int N1, int N2, int W>
struct shell_slabs {
    static constexpr int NI0 = N0 - 2 * W, NI1 = N1 - 2 * W, NI2 = N2 - 2 * W;
    static constexpr int NZ = 2 * W * N1 * N0, NY = NI2 * 2 * W * N0, NX = NI2 * NI1 * 2 * W;
    static constexpr int COUNT = NZ + NY + NX;
    __device__ __forceinline__ static void at(int q, int& i, int& j, int& k)
    {
        if (q < NZ) {
            const int zz = q / (N1 * N0), rr = q - zz * (N1 * N0);
            k = zz < W ? zz : NI2 + zz;
            j = rr / N0;
            i = rr - j * N0;
        } else if (q < NZ + NY) {
            q -= NZ;
            const int kk = q / (2 * W * N0), rr = q - kk * (2 * W * N0);
            const int yy = rr / N0;
            k = W + kk;
            j = yy < W ? yy : NI1 + yy;
            i = rr - yy * N0;
        } else {
            q -= NZ + NY;
            const int xx = q % (2 * W), rr = q / (2 * W);
            i = xx < W ? xx : NI0 + xx;
            j = W + rr % NI1;
            k = W + rr / NI1;
        }
    }
};

// guard faces of axis A in the step's read region: the shell of the box
// normal 3..21, across 3..20
template <int A>
using step_face_shell = shell_slabs<GB_BAND + (A == 0), GB_BAND + (A == 1), GB_BAND + (A == 2), 1>;
constexpr int GB_STEP_GUARD_FACES = (GB_BAND + 1) * GB_BAND * GB_BAND - (GB_NXB + 1) * GB_NXB * GB_NXB;  // 1804

// Guard-fill plan entry flags (the plan: for every leaf and each of the 27
// block-sized regions around it, two int4 {node, level, flags, 0},
// {cx, cy, cz, 0}; region r = rx + 3 ry + 9 rz, offsets -1..1 per axis)
constexpr int GP_REFINED = 1;   // a node of the leaf's level with children
constexpr int GP_LEAFKIDS = 2;  // ... whose children are all leaves

// finite and positive (the cooling solve's input guard)
__device__ __forceinline__ bool gb_finite_pos(double x) { return isfinite(x) && x > 0.0; }

// Record the first failure in the status word and count it under its code.
__device__ __forceinline__ void gb_fail(gb_status* st, int code, int blk, int i, int j, int k,
                                        double v)
{
    if (!st) return;
    atomicAdd(&st->n_code[code & 7], 1ull);
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

// x 2^l for a normal, finite x whose scaled exponent stays normal (dt / dx
// of a level): the exponent field moves by l on the integer pipe, the same
// value as the FP64 multiplication, without an FP64 instruction
__device__ __forceinline__ double gb_scale_pow2(double x, int l)
{
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e == 0 || e == 0x7FF || e + l <= 0 || e + l >= 0x7FF) return x * gb_pow2(l);
    return __longlong_as_double(b + ((long long)l << 52));
}

__device__ __forceinline__ int gb_block_level(const gb_dev_grid& g, int blk) { return g.level ? __ldg(g.level + blk) : 0; }

__device__ __forceinline__ void gb_block_dx(const gb_dev_grid& g, const double* dx0, int blk, double* dx)
{
    const int l = g.level ? __ldg(g.level + blk) : 0;
    dx[0] = gb_scale_pow2(dx0[0], -l);
    dx[1] = gb_scale_pow2(dx0[1], -l);
    dx[2] = gb_scale_pow2(dx0[2], -l);
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
