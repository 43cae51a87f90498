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
// and its FP32 primitive copy cover only this region; guard layers 0 and
// 23 and the stencil-free corners are never read by a step.
constexpr int GB_BAND_LO = GB_NGUARD - 1, GB_BAND = GB_NXB + 2;            // 3, 18
constexpr int GB_ARM = 4 * GB_BAND * GB_BAND;                              // cells per axis arm set
constexpr int GB_STEP_CELLS = GB_BAND * GB_BAND * GB_BAND + 3 * GB_ARM;    // 9720
constexpr int GB_STEP_FACES = (GB_BAND + 1) * GB_BAND * GB_BAND;           // per axis, 6156

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

// arm cell a of the stencil reach (a < 3 GB_ARM): one axis at 1, 2, 21 or 22
__device__ __forceinline__ void gb_arm_cell(int a, int& i, int& j, int& k)
{
    const int d = a / GB_ARM, r = a - d * GB_ARM;
    auto arm = [](int l) { return l < 2 ? GB_BAND_LO - 2 + l : GB_BAND_LO + GB_BAND + (l - 2); };
    if (d == 0) {
        i = arm(r & 3);
        j = GB_BAND_LO + (r >> 2) % GB_BAND;
        k = GB_BAND_LO + (r >> 2) / GB_BAND;
    } else if (d == 1) {
        i = GB_BAND_LO + r % GB_BAND;
        j = arm((r / GB_BAND) & 3);
        k = GB_BAND_LO + r / (4 * GB_BAND);
    } else {
        i = GB_BAND_LO + r % GB_BAND;
        j = GB_BAND_LO + (r / GB_BAND) % GB_BAND;
        k = arm(r / (GB_BAND * GB_BAND));
    }
}

// q-th cell of the step's read region (q < GB_STEP_CELLS): band, then arms
__device__ __forceinline__ void gb_step_cell(int q, int& i, int& j, int& k)
{
    constexpr int NB = GB_BAND * GB_BAND * GB_BAND;
    if (q < NB) {
        i = GB_BAND_LO + q % GB_BAND;
        j = GB_BAND_LO + (q / GB_BAND) % GB_BAND;
        k = GB_BAND_LO + q / (GB_BAND * GB_BAND);
    } else {
        gb_arm_cell(q - NB, i, j, k);
    }
}

// guard cells of the step's read region: the band's shell, then the arms
using band_shell = shell_slabs<GB_BAND, GB_BAND, GB_BAND, 1>;
constexpr int GB_STEP_GUARD_CELLS = band_shell::COUNT + 3 * GB_ARM;  // 5624
__device__ __forceinline__ void gb_step_guard_cell(int q, int& i, int& j, int& k)
{
    if (q < band_shell::COUNT) {
        band_shell::at(q, i, j, k);
        i += GB_BAND_LO;
        j += GB_BAND_LO;
        k += GB_BAND_LO;
    } else {
        gb_arm_cell(q - band_shell::COUNT, i, j, k);
    }
}

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
