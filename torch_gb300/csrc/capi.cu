// C ABI entry points, registration, guard-cell fill and host-side driving
// of the hydro step.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "gb_prof.h"
#include "gb_state.h"
#include "hydro_dev.cuh"

gb_state_t g_gb;

// ---------------------------------------------------------------- profiler
namespace {
struct prof_state {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<int> ids;  // kernel id per recorded pair
    cudaEvent_t open[GBP_N];
} g_prof;

cudaEvent_t prof_event()
{
    if (g_prof.used == g_prof.pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        g_prof.pool.push_back(e);
    }
    return g_prof.pool[g_prof.used++];
}
}  // namespace

void gb_prof_begin(int id, cudaStream_t s)
{
    if (!g_prof.on) return;
    cudaEvent_t e = prof_event();
    cudaEventRecord(e, s);
    g_prof.open[id] = e;
}

void gb_prof_end(int id, cudaStream_t s)
{
    if (!g_prof.on) return;
    cudaEvent_t e = prof_event();
    cudaEventRecord(e, s);
    g_prof.ids.push_back(id);
    // the begin event of this pair is the one recorded just before the
    // kernel; keep pairs adjacent in the pool
    (void)g_prof.open[id];
}

int gb_prof_is_on() { return g_prof.on ? 1 : 0; }

extern "C" int gb_prof_enable(int on)
{
    g_prof.on = on != 0;
    g_prof.used = 0;
    g_prof.ids.clear();
    return GB_OK;
}

extern "C" int gb_prof_read(double* ms, long long* launches, int n)
{
    if (!ms || !launches || n < GBP_N) return GB_ERR_ARG;
    for (int i = 0; i < GBP_N; ++i) {
        ms[i] = 0.0;
        launches[i] = 0;
    }
    if (gb_check(cudaDeviceSynchronize(), "profiler sync")) return GB_ERR_CUDA;
    for (size_t q = 0; q < g_prof.ids.size(); ++q) {
        float t = 0.0f;
        cudaEventElapsedTime(&t, g_prof.pool[2 * q], g_prof.pool[2 * q + 1]);
        ms[g_prof.ids[q]] += t;
        launches[g_prof.ids[q]] += 1;
    }
    return GB_OK;
}

// FP64 FMA throughput probe: 8 independent dependency chains per thread
// NCH independent FMA chains per thread (enough to hide the pipe latency)
template <typename T, int NCH>
__global__ void __launch_bounds__(256) k_fma_peak(T* out, int iters, T a, T b)
{
    T x[NCH];
#pragma unroll
    for (int q = 0; q < NCH; ++q) x[q] = (T)1e-3 * (T)(threadIdx.x + q);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < NCH; ++q) x[q] = fma(x[q], a, b);
    }
    T s = (T)0;
#pragma unroll
    for (int q = 0; q < NCH; ++q) s += x[q];
    if (s == (T)-1) out[0] = s;  // keeps the chains live; never true
}

// FMA throughput of the current GPU in TFLOP/s (2 flops per FMA), best of
// five timed launches of a few milliseconds over 8 CTAs per SM
template <typename T, int NCH>
static int measure_fma_peak(double* tflops)
{
    if (!tflops) return GB_ERR_ARG;
    int dev = 0, nsm = 0;
    if (gb_check(cudaGetDevice(&dev), "device") ||
        gb_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "sm count"))
        return GB_ERR_CUDA;
    T* d = nullptr;
    if (gb_check(cudaMalloc(&d, sizeof(T)), "probe alloc")) return GB_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int iters = sizeof(T) == 8 ? 1 << 14 : 1 << 16, blocks = nsm * 8, threads = 256;
    const T a = (T)0.9999999, b = (T)1e-7;
    k_fma_peak<T, NCH><<<blocks, threads>>>(d, iters, a, b);
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(e0);
        k_fma_peak<T, NCH><<<blocks, threads>>>(d, iters, a, b);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    int rc = gb_check(cudaGetLastError(), "k_fma_peak") ? GB_ERR_CUDA : GB_OK;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    *tflops = 2.0 * NCH * (double)iters * (double)blocks * threads / (best * 1e-3) / 1e12;
    return rc;
}

extern "C" int gb_measure_fp64_peak(double* tflops) { return measure_fma_peak<double, 8>(tflops); }
extern "C" int gb_measure_fp32_peak(double* tflops) { return measure_fma_peak<float, 16>(tflops); }

// the integer-pipe conversions against the hardware ones, bit for bit
__global__ void k_check_conv(int64_t n, const double* __restrict__ d, const float* __restrict__ f,
                             unsigned long long* __restrict__ bad)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float a = gb_d2f(d[i]), b = (float)d[i];
    const double c = gb_f2d(f[i]), e = (double)f[i];
    const bool ok1 = __float_as_uint(a) == __float_as_uint(b) || (isnan(a) && isnan(b));
    const bool ok2 = __double_as_longlong(c) == __double_as_longlong(e) || (isnan(c) && isnan(e));
    if (!ok1) atomicAdd(bad, 1ull);
    if (!ok2) atomicAdd(bad + 1, 1ull);
}

extern "C" int gb_selfcheck_conversions(int64_t n, const double* d_dev, const float* f_dev,
                                        unsigned long long* mismatches_dev, void* stream)
{
    if (n < 0 || (n > 0 && (!d_dev || !f_dev || !mismatches_dev))) return GB_ERR_ARG;
    if (n == 0) return GB_OK;
    k_check_conv<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(n, d_dev, f_dev, mismatches_dev);
    return gb_check(cudaGetLastError(), "k_check_conv") ? GB_ERR_CUDA : GB_OK;
}

static char g_err[512] = "";

void gb_set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

int gb_check(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return 0;
    gb_set_error("%s: %s", what, cudaGetErrorString(e));
    return 1;
}

extern "C" const char* gb_last_error(void) { return g_err; }
extern "C" int gb_version(void) { return 1; }

int gb_ensure_scratch(size_t bytes)
{
    if (bytes <= g_gb.scratch_bytes) return GB_OK;
    if (g_gb.d_scratch) cudaFree(g_gb.d_scratch);
    g_gb.d_scratch = nullptr;
    g_gb.scratch_bytes = 0;
    if (gb_check(cudaMalloc(&g_gb.d_scratch, bytes), "cudaMalloc(scratch)")) return GB_ERR_CUDA;
    g_gb.scratch_bytes = bytes;
    return GB_OK;
}

int gb_ensure_stage(size_t bytes)
{
    if (bytes <= g_gb.stage_bytes) return GB_OK;
    if (g_gb.d_stage) cudaFree(g_gb.d_stage);
    g_gb.d_stage = nullptr;
    g_gb.stage_bytes = 0;
    if (gb_check(cudaMalloc(&g_gb.d_stage, bytes), "cudaMalloc(stage)")) return GB_ERR_CUDA;
    g_gb.stage_bytes = bytes;
    return GB_OK;
}

// ---------------------------------------------------------------- status
extern "C" int gb_status_reset(gb_status* st, void* stream)
{
    if (!st) return GB_ERR_ARG;
    return gb_check(cudaMemsetAsync(st, 0, sizeof(gb_status), (cudaStream_t)stream), "status reset")
               ? GB_ERR_CUDA
               : GB_OK;
}

extern "C" int gb_status_read(const gb_status* st, gb_status* host)
{
    if (!st || !host) return GB_ERR_ARG;
    return gb_check(cudaMemcpy(host, st, sizeof(gb_status), cudaMemcpyDeviceToHost), "status read")
               ? GB_ERR_CUDA
               : GB_OK;
}

// ---------------------------------------------------------------- registration
extern "C" int gb_register_grid(const gb_grid_desc* grid, const gb_tree_desc* tree)
{
    if (!grid || !grid->unk || grid->nvar <= 0 || grid->maxblocks <= 0) {
        gb_set_error("gb_register_grid: bad grid descriptor");
        return GB_ERR_ARG;
    }
    for (int r = 0; r < GB_NROLE; ++r)
        if (grid->slot[r] >= grid->nvar) {
            gb_set_error("gb_register_grid: slot of role %d beyond nvar", r);
            return GB_ERR_ARG;
        }
    for (int r = GB_DENS; r <= GB_EINT; ++r)
        if (grid->slot[r] < 0) {
            gb_set_error("gb_register_grid: hydro role %d has no slot", r);
            return GB_ERR_ARG;
        }
    g_gb.desc = *grid;
    g_gb.grid.nvar = grid->nvar;
    g_gb.grid.maxblocks = grid->maxblocks;
    memcpy(g_gb.grid.slot, grid->slot, sizeof grid->slot);
    g_gb.grid.unk = grid->unk;
    g_gb.grid.f[0] = grid->facex;
    g_gb.grid.f[1] = grid->facey;
    g_gb.grid.f[2] = grid->facez;
    g_gb.grid.level = nullptr;
    g_gb.grid_ok = true;
    g_gb.links_ok = false;
    g_gb.plan_ok = false;
    g_gb.gen += 1;
    g_gb.tree_ok = false;
    if (tree) {
        if (tree->nnodes < grid->maxblocks || !tree->level || !tree->coord || !tree->child || !tree->root ||
            tree->nrx <= 0 || tree->nry <= 0 || tree->nrz <= 0 || tree->maxlevel < 0 || tree->maxlevel > 20) {
            gb_set_error("gb_register_grid: bad tree descriptor");
            return GB_ERR_ARG;
        }
        g_gb.tree = *tree;
        g_gb.grid.level = tree->level;
        g_gb.tree_ok = true;
    }
    // per-cell CFL codes start at zero (no cell lowered) for a new grid
    const size_t cb = (size_t)grid->maxblocks * 3 * GB_NXB * GB_NXB * GB_NXB;
    if (cb > g_gb.cflc_bytes) {
        if (g_gb.d_cflc) cudaFree(g_gb.d_cflc);
        g_gb.d_cflc = nullptr;
        g_gb.cflc_bytes = 0;
        if (gb_check(cudaMalloc(&g_gb.d_cflc, cb), "cudaMalloc(cfl codes)")) return GB_ERR_CUDA;
        g_gb.cflc_bytes = cb;
    }
    if (gb_check(cudaMemset(g_gb.d_cflc, 0, cb), "cudaMemset(cfl codes)")) return GB_ERR_CUDA;
    return GB_OK;
}

extern "C" int gb_cfl_codes_reset(void* stream)
{
    if (!g_gb.grid_ok) {
        gb_set_error("gb_cfl_codes_reset: call gb_register_grid first");
        return GB_ERR_NOT_INIT;
    }
    return gb_check(cudaMemsetAsync(g_gb.d_cflc, 0, g_gb.cflc_bytes, (cudaStream_t)stream), "cfl codes reset")
               ? GB_ERR_CUDA
               : GB_OK;
}

// copies the registered grid's CFL codes between the library and a caller
// buffer (host or device memory, cudaMemcpyDefault)
static int cfl_codes_copy(void* dst, const void* src, size_t nbytes, void* stream, const char* who)
{
    if (!g_gb.grid_ok) {
        gb_set_error("%s: call gb_register_grid first", who);
        return GB_ERR_NOT_INIT;
    }
    const size_t need = (size_t)g_gb.grid.maxblocks * 3 * GB_NXB * GB_NXB * GB_NXB;
    if (nbytes != need || !dst || !src) {
        gb_set_error("%s: %zu bytes given, the registered grid's codes take %zu", who, nbytes, need);
        return GB_ERR_ARG;
    }
    return gb_check(cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyDefault, (cudaStream_t)stream), who) ? GB_ERR_CUDA
                                                                                                      : GB_OK;
}

extern "C" int gb_cfl_codes_save(void* dst, size_t nbytes, void* stream)
{
    return cfl_codes_copy(dst, g_gb.d_cflc, nbytes, stream, "gb_cfl_codes_save");
}

extern "C" int gb_cfl_codes_load(const void* src, size_t nbytes, void* stream)
{
    return cfl_codes_copy(g_gb.d_cflc, src, nbytes, stream, "gb_cfl_codes_load");
}

extern "C" int gb_hydro_init(const gb_hydro_params* p)
{
    if (!p || !(p->gamma > 1.0) || p->precision < 0 || p->precision > 1) {
        gb_set_error("gb_hydro_init: bad parameters");
        return GB_ERR_ARG;
    }
    g_gb.hp = *p;
    g_gb.hydro_ok = true;
    g_gb.gen += 1;
    // [0]: bits of the CFL minimum, [1..3]: dt / root_dx of the last dt,
    // [4..5]: the same as three floats
    if (!g_gb.d_dtmin && gb_check(cudaMalloc(&g_gb.d_dtmin, 8 * sizeof(double)), "cudaMalloc(dtmin)"))
        return GB_ERR_CUDA;
    return GB_OK;
}

// ---------------------------------------------------------------- guard fill
namespace {

struct leaf_hit {
    int node, level;
};

// All positions are non-negative finest-cell coordinates and every size is
// a power of two, so divisions are shifts: GB_NXB = 2^4 cells per block.
static_assert(GB_NXB == 16, "block size 16 assumed by the shifts below");
constexpr int LOG2_NXB = 4;

__device__ __forceinline__ leaf_hit find_leaf(const gb_tree_desc& t, long long X, long long Y, long long Z)
{
    const int sh0 = LOG2_NXB + t.maxlevel;
    int rx = (int)(X >> sh0), ry = (int)(Y >> sh0), rz = (int)(Z >> sh0);
    int node = t.root[rx + t.nrx * (ry + t.nry * rz)];
    int l = 0;
    for (int it = 0; it <= t.maxlevel && node >= 0; ++it) {
        int c0 = __ldg(t.child + 8 * node);
        if (c0 < 0) break;
        const int sh = sh0 - 1 - l;
        int cx = (int)((X >> sh) & 1), cy = (int)((Y >> sh) & 1), cz = (int)((Z >> sh) & 1);
        node = __ldg(t.child + 8 * node + (cx | (cy << 1) | (cz << 2)));
        ++l;
    }
    leaf_hit h;
    h.node = node;
    h.level = node >= 0 ? t.level[node] : 0;
    return h;
}

// periodic wrap of a guard position: x lies in (-n, 2n) (a guard region is
// narrower than the domain)
__device__ __forceinline__ long long wrap(long long x, long long n) { return x < 0 ? x + n : (x >= n ? x - n : x); }

// Guard-fill plan, built once per registered tree: for every leaf b and
// each of the 27 block-sized regions around it (offsets -1, 0, 1 per axis,
// periodic; region r = rx + 3 ry + 9 rz, r = 13 being b itself), the node
// covering the region, found by descending from the root no deeper than b's
// level: a leaf of b's level or coarser, or a refined node of b's level
// whose children cover the region. Two int4 per entry:
// {node, level, flags, 0} and {cx, cy, cz, 0}. A guard cell then reads its
// block's entry and its region's entry and takes at most one step down.

__global__ void k_guard_plan(gb_tree_desc t, int4* __restrict__ plan, int* __restrict__ near)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= t.nnodes * 27) return;
    const int b = idx / 27, r = idx % 27;
    int4 h = make_int4(-1, 0, 0, 0), c = make_int4(0, 0, 0, 0);
    if (t.child[8 * b] < 0) {
        const int L = t.level[b];
        const int off[3] = {r % 3 - 1, (r / 3) % 3 - 1, r / 9 - 1};
        const int nr[3] = {t.nrx, t.nry, t.nrz};
        int P[3];  // the region's block coordinates at level L, periodic
        for (int d = 0; d < 3; ++d) {
            const int n = nr[d] << L;
            P[d] = t.coord[3 * b + d] + off[d];
            P[d] = P[d] < 0 ? P[d] + n : (P[d] >= n ? P[d] - n : P[d]);
        }
        int node = t.root[(P[0] >> L) + t.nrx * ((P[1] >> L) + t.nry * (P[2] >> L))];
        for (int l = 0; l < L && node >= 0; ++l) {
            if (t.child[8 * node] < 0) break;
            const int sh = L - 1 - l;
            node = t.child[8 * node + ((P[0] >> sh) & 1) + 2 * ((P[1] >> sh) & 1) + 4 * ((P[2] >> sh) & 1)];
        }
        if (r == 13) node = b;
        if (node >= 0) {
            int flags = 0;
            if (t.child[8 * node] >= 0) {
                flags = GP_REFINED | GP_LEAFKIDS;
                for (int q = 0; q < 8; ++q) {
                    const int ch = t.child[8 * node + q];
                    if (ch < 0 || t.child[8 * ch] >= 0) flags &= ~GP_LEAFKIDS;
                }
            }
            h = make_int4(node, t.level[node], flags, 0);
            c = make_int4(t.coord[3 * node], t.coord[3 * node + 1], t.coord[3 * node + 2], 0);
            // per leaf: bit 0 a coarser leaf around it, bit 1 a finer one
            const int bits = (h.y < L ? 1 : 0) | (flags & GP_REFINED ? 2 : 0);
            if (bits) atomicOr(near + b, bits);
        }
    }
    plan[2 * (size_t)idx] = h;
    plan[2 * (size_t)idx + 1] = c;
}

__device__ __forceinline__ int region_of(int loc) { return loc < GB_NGUARD ? 0 : (loc >= GB_NGUARD + GB_NXB ? 2 : 1); }

// Periodic level-L index of the cell (or face) at padded index I of the
// block at coordinate c of level L; M = cells of level L across the domain.
// With the plan every position is such a 32-bit level-local index: the
// finest-cell position of the walk from the root is (A + 1/2) 2^(maxlevel-L)
// for a cell centre and A 2^(maxlevel-L) for a face, so every shift of the
// walk becomes a shift of A.
__device__ __forceinline__ int level_index(int c, int I, int M)
{
    const int A = (c << LOG2_NXB) + I - GB_NGUARD;
    return A < 0 ? A + M : (A >= M ? A - M : A);
}

struct plan_hit {
    int node, level, c[3];
};

// The leaf covering level-L position A (a face position along axis fa when
// fa >= 0, cell centres otherwise) from the plan entry {e, ec} of its region.
__device__ __forceinline__ plan_hit plan_leaf(const gb_tree_desc& t, int4 e, int4 ec, int L, const int* A, int fa)
{
    plan_hit h;
    h.node = e.x;
    h.level = e.y;
    h.c[0] = ec.x;
    h.c[1] = ec.y;
    h.c[2] = ec.z;
    if (h.node < 0 || !(e.z & GP_REFINED)) return h;
    for (int dl = 0; L + dl < t.maxlevel; ++dl) {
        const int half = (1 << dl) >> 1;
        int q = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) q |= ((((A[d] << dl) + (d == fa ? 0 : half)) >> 3) & 1) << d;
        h.node = __ldg(t.child + 8 * h.node + q);
        if (h.node < 0) return h;
        h.level = __ldg(t.level + h.node);
#pragma unroll
        for (int d = 0; d < 3; ++d) h.c[d] = __ldg(t.coord + 3 * h.node + d);
        if ((dl == 0 && (e.z & GP_LEAFKIDS)) || __ldg(t.child + 8 * h.node) < 0) break;
    }
    return h;
}

// The q-th guard position of an N0 x N1 x N2 padded array whose interior
// spans [GB_NGUARD, GB_NGUARD + NI) on each axis (N - NI = 2 GB_NGUARD):
// the two z slabs, the two y slabs inside them, the two x slabs inside
// those. x runs fastest everywhere; in the x slabs the 8 guard columns of a
// row are consecutive, so four neighbouring threads share a 32-byte sector.
template <int N0, int N1, int NI0, int NI1, int NI2>
struct guard_slabs {
    static constexpr int G = 2 * GB_NGUARD;
    static constexpr int NZ = G * N1 * N0, NY = NI2 * G * N0, NX = NI2 * NI1 * G;
    static constexpr int COUNT = NZ + NY + NX;
    __device__ __forceinline__ static void at(int q, int& i, int& j, int& k)
    {
        if (q < NZ) {
            const int zz = q / (N1 * N0), rr = q - zz * (N1 * N0);
            k = zz < GB_NGUARD ? zz : NI2 + zz;
            j = rr / N0;
            i = rr - j * N0;
        } else if (q < NZ + NY) {
            q -= NZ;
            const int kk = q / (G * N0), rr = q - kk * (G * N0);
            const int yy = rr / N0;
            k = GB_NGUARD + kk;
            j = yy < GB_NGUARD ? yy : NI1 + yy;
            i = rr - yy * N0;
        } else {
            q -= NZ + NY;
            const int xx = q % G, rr = q / G;
            i = xx < GB_NGUARD ? xx : NI0 + xx;
            j = GB_NGUARD + rr % NI1;
            k = GB_NGUARD + rr / NI1;
        }
    }
};
using cell_slabs = guard_slabs<GB_N, GB_N, GB_NXB, GB_NXB, GB_NXB>;
template <int AX>
using face_slabs = guard_slabs<GB_N + (AX == 0), GB_N + (AX == 1), GB_NXB + (AX == 0), GB_NXB + (AX == 1),
                               GB_NXB + (AX == 2)>;
static_assert(face_slabs<0>::COUNT == face_slabs<1>::COUNT && face_slabs<1>::COUNT == face_slabs<2>::COUNT,
              "guard faces per axis");
constexpr int GB_NGF = face_slabs<0>::COUNT;

// Face neighbours of every leaf: links[(b * 6 + f) * 5] = same (0), coarser
// (1) or finer (2) neighbour across face f = 2 d + side, then the four fine
// leaves (finer only; quadrant q: bit 0 the upper half along the first
// transverse axis, bit 1 along the second). The probe lies one finest cell
// across the face, at the face centre or the quadrant centres.
__global__ void k_face_links(gb_tree_desc t, int* __restrict__ links)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= t.nnodes * 6) return;
    const int b = idx / 6, f = idx % 6;
    int* out = links + (size_t)idx * 5;
    out[0] = 0;
    out[1] = out[2] = out[3] = out[4] = -1;
    if (t.child[8 * b] >= 0) return;
    const int d = f >> 1, side = f & 1;
    const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
    const long long N[3] = {(long long)t.nrx * GB_NXB << t.maxlevel, (long long)t.nry * GB_NXB << t.maxlevel,
                            (long long)t.nrz * GB_NXB << t.maxlevel};
    const int L = t.level[b];
    const long long E = (long long)GB_NXB << (t.maxlevel - L);
    const int* cd = t.coord + 3 * b;
    long long X[3];
    X[d] = wrap(side ? (cd[d] + 1) * E : cd[d] * E - 1, N[d]);
    X[t1] = cd[t1] * E + E / 2;
    X[t2] = cd[t2] * E + E / 2;
    leaf_hit h = find_leaf(t, X[0], X[1], X[2]);
    if (h.node < 0) return;
    if (h.level < L) {
        out[0] = 1;
    } else if (h.level > L) {
        out[0] = 2;
        for (int q = 0; q < 4; ++q) {
            long long Y[3] = {X[0], X[1], X[2]};
            Y[t1] = cd[t1] * E + E / 4 + (q & 1) * (E / 2);
            Y[t2] = cd[t2] * E + E / 4 + (q >> 1) * (E / 2);
            out[1 + q] = find_leaf(t, Y[0], Y[1], Y[2]).node;
        }
    }
}

// The block list reordered finest level first (one CTA; order within a
// level is arbitrary and does not change any result).
__global__ void __launch_bounds__(1024) k_sort_levels(const int* __restrict__ list, int n, const int* __restrict__ level,
                                                      int maxlevel, int* __restrict__ out)
{
    __shared__ int cnt[32], off[32];
    if (threadIdx.x < 32) cnt[threadIdx.x] = 0;
    __syncthreads();
    for (int q = threadIdx.x; q < n; q += blockDim.x) atomicAdd(&cnt[min(max(level[list[q]], 0), 31)], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int l = 31; l >= 0; --l) {
            off[l] = acc;
            acc += cnt[l];
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int b = list[q];
        out[atomicAdd(&off[min(max(level[b], 0), 31)], 1)] = b;
    }
    (void)maxlevel;
}

// The guard cells of a padded block, enumerated as slabs: the two z slabs
// (k < 4 or k >= 20, all j, i), the two y slabs inside them, the two x slabs
// inside those. 2 * 4 * 24 * 24 + 2 * 4 * 16 * 24 + 2 * 4 * 16 * 16 = 9728.
constexpr int GZ = 2 * GB_NGUARD * GB_N * GB_N, GY = 2 * GB_NGUARD * GB_NXB * GB_N, GX = 2 * GB_NGUARD * GB_NXB * GB_NXB;
constexpr int GB_NGC = GZ + GY + GX;
static_assert(GB_NGC == GB_N3 - GB_NXB * GB_NXB * GB_NXB, "guard cell count");

__device__ __forceinline__ void guard_cell(int q, int& i, int& j, int& k)
{
    const int lo = GB_NGUARD, hi = GB_NGUARD + GB_NXB;
    if (q < GZ) {
        const int zz = q / (GB_N * GB_N), r = q % (GB_N * GB_N);
        k = zz < GB_NGUARD ? zz : hi + (zz - GB_NGUARD);
        j = r / GB_N;
        i = r % GB_N;
    } else if (q < GZ + GY) {
        q -= GZ;
        const int yy = q / (GB_NXB * GB_N), r = q % (GB_NXB * GB_N);
        j = yy < GB_NGUARD ? yy : hi + (yy - GB_NGUARD);
        k = lo + r / GB_N;
        i = r % GB_N;
    } else {
        q -= GZ + GY;
        const int xx = q / (GB_NXB * GB_NXB), r = q % (GB_NXB * GB_NXB);
        i = xx < GB_NGUARD ? xx : hi + (xx - GB_NGUARD);
        k = lo + r / GB_NXB;
        j = lo + r % GB_NXB;
    }
}

// The variables the hydro step reads in guard cells (FLASH fills guard
// cells for Hydro with a variable mask the same way); store slots, -1 = absent
struct guard_vars {
    int n;
    int slot[GB_NROLE];
};

// Without a plan (a capture that did not prepare one, or a domain too wide
// for 32-bit level indices): 64-bit finest-cell positions and a walk from
// the root per guard cell.
__global__ void k_guard_cells(gb_dev_grid g, gb_tree_desc t, const int* __restrict__ list, guard_vars gv)
{
    const int blk = list[blockIdx.y];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= GB_NGC) return;
    int i, j, k;
    guard_cell(q, i, j, k);
    const int c = gb_cidx(i, j, k);
    const int L = t.level[blk];
    const int ls = t.maxlevel - L;  // log2 of this block's cell size in finest cells
    const long long s = 1LL << ls;
    const long long N[3] = {(long long)t.nrx * GB_NXB << t.maxlevel, (long long)t.nry * GB_NXB << t.maxlevel,
                            (long long)t.nrz * GB_NXB << t.maxlevel};
    const int* cd = t.coord + 3 * blk;
    const int loc[3] = {i, j, k};
    long long lo[3], X[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = wrap(((long long)cd[d] * GB_NXB + loc[d] - GB_NGUARD) * s, N[d]);
        X[d] = lo[d] + (s >> 1);
    }
    leaf_hit h = find_leaf(t, X[0], X[1], X[2]);
    if (h.node < 0) return;
    const int lsl = t.maxlevel - h.level;
    const int* sc = t.coord + 3 * h.node;
    double* dst = g.unk + (int64_t)blk * g.nvar * GB_N3 + c;
    const double* src = g.unk + (int64_t)h.node * g.nvar * GB_N3;
    if (h.level <= L) {
        // same level: copy; coarser: injection of the covering coarse cell
        int si = (int)((X[0] >> lsl) - (long long)sc[0] * GB_NXB) + GB_NGUARD;
        int sj = (int)((X[1] >> lsl) - (long long)sc[1] * GB_NXB) + GB_NGUARD;
        int sk = (int)((X[2] >> lsl) - (long long)sc[2] * GB_NXB) + GB_NGUARD;
        int sci = gb_cidx(si, sj, sk);
        // all loads first, then all stores: the loads are independent and in
        // flight together (a store between them could alias the next load)
        double val[GB_NROLE];
#pragma unroll
        for (int q2 = 0; q2 < GB_NROLE; ++q2)
            if (q2 < gv.n) val[q2] = src[(int64_t)gv.slot[q2] * GB_N3 + sci];
#pragma unroll
        for (int q2 = 0; q2 < GB_NROLE; ++q2)
            if (q2 < gv.n) dst[(int64_t)gv.slot[q2] * GB_N3] = val[q2];
    } else {
        // finer neighbour: mean of the fine cells covering this cell
        int r = 1 << (ls - lsl);
        int bi = (int)((lo[0] >> lsl) - (long long)sc[0] * GB_NXB) + GB_NGUARD;
        int bj = (int)((lo[1] >> lsl) - (long long)sc[1] * GB_NXB) + GB_NGUARD;
        int bk = (int)((lo[2] >> lsl) - (long long)sc[2] * GB_NXB) + GB_NGUARD;
        double inv = 1.0 / (double)(r * r * r);
        double val[GB_NROLE];
#pragma unroll
        for (int q2 = 0; q2 < GB_NROLE; ++q2) {
            if (q2 >= gv.n) continue;
            const int64_t v = gv.slot[q2];
            double acc = 0.0;
            for (int z = 0; z < r; ++z)
                for (int y = 0; y < r; ++y)
                    for (int x = 0; x < r; ++x) acc += src[(int64_t)v * GB_N3 + gb_cidx(bi + x, bj + y, bk + z)];
            val[q2] = acc * inv;
        }
#pragma unroll
        for (int q2 = 0; q2 < GB_NROLE; ++q2)
            if (q2 < gv.n) dst[(int64_t)gv.slot[q2] * GB_N3] = val[q2];
    }
}

__global__ void k_guard_faces(gb_dev_grid g, gb_tree_desc t, const int* __restrict__ list)
{
    const int a = blockIdx.z;
    const int blk = list[blockIdx.y];
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= GB_FSZ) return;
    int I[3];
    if (a == 0) { I[0] = f % (GB_N + 1); I[1] = (f / (GB_N + 1)) % GB_N; I[2] = f / ((GB_N + 1) * GB_N); }
    else if (a == 1) { I[0] = f % GB_N; I[1] = (f / GB_N) % (GB_N + 1); I[2] = f / (GB_N * (GB_N + 1)); }
    else { I[0] = f % GB_N; I[1] = (f / GB_N) % GB_N; I[2] = f / (GB_N * GB_N); }
    bool own = true;
    for (int e = 0; e < 3; ++e) {
        int top = GB_NGUARD + GB_NXB - 1 + (e == a);
        if (I[e] < GB_NGUARD || I[e] > top) own = false;
    }
    if (own) return;
    const int L = t.level[blk];
    const int ls = t.maxlevel - L;  // log2 of this block's cell size in finest cells
    const long long s = 1LL << ls;
    const long long N[3] = {(long long)t.nrx * GB_NXB << t.maxlevel, (long long)t.nry * GB_NXB << t.maxlevel,
                            (long long)t.nrz * GB_NXB << t.maxlevel};
    const int* cd = t.coord + 3 * blk;
    long long lo[3], X[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = wrap(((long long)cd[d] * GB_NXB + I[d] - GB_NGUARD) * s, N[d]);
        X[d] = lo[d] + (d == a ? 0 : (s >> 1));
    }
    leaf_hit h = find_leaf(t, X[0], X[1], X[2]);
    if (h.node < 0) return;
    if (h.level != L) {
        // a face on a level boundary: the copy owned by the leaf of this
        // block's level on the lower side, when there is one, so that every
        // block of a level reads the same face
        leaf_hit h2 = find_leaf(t, a == 0 ? wrap(X[0] - 1, N[0]) : X[0], a == 1 ? wrap(X[1] - 1, N[1]) : X[1],
                                a == 2 ? wrap(X[2] - 1, N[2]) : X[2]);
        if (h2.node >= 0 && h2.level == L) {
            X[a] = wrap(X[a] - 1, N[a]) + 1;  // its upper face, unwrapped at the domain edge
            h = h2;
        }
    }
    const int lsl = t.maxlevel - h.level;
    const int* sc = t.coord + 3 * h.node;
    const double* src = g.f[a] + (int64_t)h.node * GB_FSZ;
    double* dst = g.f[a] + (int64_t)blk * GB_FSZ + f;
    if (h.level <= L) {
        int S[3];
        for (int d = 0; d < 3; ++d) S[d] = (int)((X[d] >> lsl) - (long long)sc[d] * GB_NXB) + GB_NGUARD;
        if ((X[a] & ((1LL << lsl) - 1)) == 0) {
            *dst = src[gb_fidx(a, S[0], S[1], S[2])];
        } else {
            // fine face inside a coarse cell: mean of the two coarse faces
            int S1[3] = {S[0], S[1], S[2]};
            S1[a] += 1;
            *dst = 0.5 * (src[gb_fidx(a, S[0], S[1], S[2])] + src[gb_fidx(a, S1[0], S1[1], S1[2])]);
        }
    } else {
        // finer neighbour: area mean of the fine faces on this face
        int r = 1 << (ls - lsl);
        int B[3];
        for (int d = 0; d < 3; ++d) B[d] = (int)((lo[d] >> lsl) - (long long)sc[d] * GB_NXB) + GB_NGUARD;
        int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
        double acc = 0.0;
        for (int y = 0; y < r; ++y)
            for (int x = 0; x < r; ++x) {
                int Q[3] = {B[0], B[1], B[2]};
                Q[t1] += x;
                Q[t2] += y;
                acc += src[gb_fidx(a, Q[0], Q[1], Q[2])];
            }
        *dst = acc / (double)(r * r);
    }
}

// The same fills from the guard-fill plan: each guard cell reads two plan
// entries (its block, its region), computes 32-bit level-local indices and
// takes at most one step down the tree; the results are those of the walks
// from the root above, value for value.
// STEP: only the guard cells a step reads (the region of gb_step_cell);
// otherwise all of them (FLASH's guard fill)
template <bool STEP>
__global__ void __launch_bounds__(128) k_guard_cells_plan(gb_dev_grid g, gb_tree_desc t, const int* __restrict__ list,
                                                          guard_vars gv, const int4* __restrict__ plan)
{
    // every CTA serves one block: its 27 plan entries go to shared memory
    // once, so a guard cell's only global loads before its data are none
    // (or one child lookup next to a finer leaf)
    __shared__ int4 pb[54];
    const int blk = list[blockIdx.y];
    if (threadIdx.x < 54) pb[threadIdx.x] = __ldg(plan + (size_t)blk * 54 + threadIdx.x);
    __syncthreads();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (STEP ? GB_STEP_GUARD_CELLS : cell_slabs::COUNT)) return;
    int I[3];
    if (STEP) gb_step_guard_cell(q, I[0], I[1], I[2]);
    else cell_slabs::at(q, I[0], I[1], I[2]);
    const int r = region_of(I[0]) + 3 * region_of(I[1]) + 9 * region_of(I[2]);
    const int4 se = pb[26], sc = pb[27];  // region 13: the block itself
    const int4 e = pb[2 * r], ec = pb[2 * r + 1];
    const int L = se.y;
    const int cs[3] = {sc.x, sc.y, sc.z}, nr[3] = {t.nrx, t.nry, t.nrz};
    int A[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) A[d] = level_index(cs[d], I[d], nr[d] << (L + LOG2_NXB));
    const plan_hit h = plan_leaf(t, e, ec, L, A, -1);
    if (h.node < 0) return;
    double* dst = g.unk + (int64_t)blk * g.nvar * GB_N3 + gb_cidx(I[0], I[1], I[2]);
    const double* src = g.unk + (int64_t)h.node * g.nvar * GB_N3;
    const int k = L - h.level;
    double val[GB_NROLE];
    if (k >= 0) {
        // same level: copy; coarser: injection of the covering coarse cell
        const int sci = gb_cidx((A[0] >> k) - (h.c[0] << LOG2_NXB) + GB_NGUARD,
                                (A[1] >> k) - (h.c[1] << LOG2_NXB) + GB_NGUARD,
                                (A[2] >> k) - (h.c[2] << LOG2_NXB) + GB_NGUARD);
#pragma unroll
        for (int q2 = 0; q2 < GB_NROLE; ++q2)
            if (q2 < gv.n) val[q2] = src[(int64_t)gv.slot[q2] * GB_N3 + sci];
    } else {
        // finer neighbour: mean of the fine cells covering this cell
        const int m = -k, rr = 1 << m;
        const int bi = (A[0] << m) - (h.c[0] << LOG2_NXB) + GB_NGUARD;
        const int bj = (A[1] << m) - (h.c[1] << LOG2_NXB) + GB_NGUARD;
        const int bk = (A[2] << m) - (h.c[2] << LOG2_NXB) + GB_NGUARD;
        const double inv = 1.0 / (double)(rr * rr * rr);
        if (m == 1) {
            // one level finer (every 2:1-balanced tree): the 8 loads of a
            // variable are independent and issued together; the sum keeps
            // the z, y, x order of the general loop below
            const int c0 = gb_cidx(bi, bj, bk);
#pragma unroll
            for (int q2 = 0; q2 < GB_NROLE; ++q2) {
                if (q2 >= gv.n) continue;
                const double* sv = src + (int64_t)gv.slot[q2] * GB_N3 + c0;
                double w[8];
#pragma unroll
                for (int z = 0; z < 2; ++z)
#pragma unroll
                    for (int y = 0; y < 2; ++y)
#pragma unroll
                        for (int x = 0; x < 2; ++x) w[4 * z + 2 * y + x] = sv[x + GB_N * (y + GB_N * z)];
                double acc = 0.0;
#pragma unroll
                for (int e = 0; e < 8; ++e) acc += w[e];
                val[q2] = acc * inv;
            }
        } else {
#pragma unroll
            for (int q2 = 0; q2 < GB_NROLE; ++q2) {
                if (q2 >= gv.n) continue;
                const double* sv = src + (int64_t)gv.slot[q2] * GB_N3;
                double acc = 0.0;
                for (int z = 0; z < rr; ++z)
                    for (int y = 0; y < rr; ++y)
                        for (int x = 0; x < rr; ++x) acc += sv[gb_cidx(bi + x, bj + y, bk + z)];
                val[q2] = acc * inv;
            }
        }
    }
#pragma unroll
    for (int q2 = 0; q2 < GB_NROLE; ++q2)
        if (q2 < gv.n) dst[(int64_t)gv.slot[q2] * GB_N3] = val[q2];
}

template <int AX, bool STEP>
__device__ __forceinline__ void guard_face_plan(const gb_dev_grid& g, const gb_tree_desc& t, int blk, int q,
                                                const int4* __restrict__ pb)
{
    int I[3];
    if (STEP) {
        step_face_shell<AX>::at(q, I[0], I[1], I[2]);
        I[0] += GB_BAND_LO;
        I[1] += GB_BAND_LO;
        I[2] += GB_BAND_LO;
    } else {
        face_slabs<AX>::at(q, I[0], I[1], I[2]);
    }
    const int r = region_of(I[0]) + 3 * region_of(I[1]) + 9 * region_of(I[2]);
    const int4 se = pb[26], sc = pb[27];
    const int4 e = pb[2 * r], ec = pb[2 * r + 1];
    const int L = se.y;
    const int cs[3] = {sc.x, sc.y, sc.z}, nr[3] = {t.nrx, t.nry, t.nrz};
    int A[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) A[d] = level_index(cs[d], I[d], nr[d] << (L + LOG2_NXB));
    plan_hit h = plan_leaf(t, e, ec, L, A, AX);
    if (h.node < 0) return;
    if (h.level != L) {
        // a face on a level boundary: the copy owned by the leaf of this
        // block's level on the lower side, when there is one, so that every
        // block of a level reads the same face
        constexpr int stride = AX == 0 ? 1 : (AX == 1 ? 3 : 9);
        const int r2 = r + (region_of(I[AX] - 1) - region_of(I[AX])) * stride;
        if (r2 != r) {
            const int4 e2 = pb[2 * r2];
            if (e2.x >= 0 && !(e2.z & GP_REFINED) && e2.y == L) {
                const int4 ec2 = pb[2 * r2 + 1];
                h.node = e2.x;
                h.level = L;
                h.c[0] = ec2.x;
                h.c[1] = ec2.y;
                h.c[2] = ec2.z;
                const int M = nr[AX] << (L + LOG2_NXB);
                A[AX] = (A[AX] == 0 ? M : A[AX]);  // its upper face, unwrapped at the domain edge
            }
        }
    }
    const double* src = g.f[AX] + (int64_t)h.node * GB_FSZ;
    double* dst = g.f[AX] + (int64_t)blk * GB_FSZ + gb_fidx(AX, I[0], I[1], I[2]);
    const int k = L - h.level;
    if (k >= 0) {
        int S[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) S[d] = (A[d] >> k) - (h.c[d] << LOG2_NXB) + GB_NGUARD;
        if ((A[AX] & ((1 << k) - 1)) == 0) {
            *dst = src[gb_fidx(AX, S[0], S[1], S[2])];
        } else {
            // fine face inside a coarse cell: mean of the two coarse faces
            int S1[3] = {S[0], S[1], S[2]};
            S1[AX] += 1;
            *dst = 0.5 * (src[gb_fidx(AX, S[0], S[1], S[2])] + src[gb_fidx(AX, S1[0], S1[1], S1[2])]);
        }
    } else {
        // finer neighbour: area mean of the fine faces on this face
        const int m = -k, rr = 1 << m;
        int B[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) B[d] = (A[d] << m) - (h.c[d] << LOG2_NXB) + GB_NGUARD;
        constexpr int t1 = AX == 0 ? 1 : 0, t2 = AX == 2 ? 1 : 2;
        double acc = 0.0;
        if (m == 1) {
            // the four fine faces, loads issued together, summed in the
            // order of the general loop
            double w[4];
#pragma unroll
            for (int y = 0; y < 2; ++y)
#pragma unroll
                for (int x = 0; x < 2; ++x) {
                    int Q[3] = {B[0], B[1], B[2]};
                    Q[t1] += x;
                    Q[t2] += y;
                    w[2 * y + x] = src[gb_fidx(AX, Q[0], Q[1], Q[2])];
                }
            acc = ((acc + w[0]) + w[1]) + w[2];
            acc += w[3];
        } else {
            for (int y = 0; y < rr; ++y)
                for (int x = 0; x < rr; ++x) {
                    int Q[3] = {B[0], B[1], B[2]};
                    Q[t1] += x;
                    Q[t2] += y;
                    acc += src[gb_fidx(AX, Q[0], Q[1], Q[2])];
                }
        }
        *dst = acc / (double)(rr * rr);
    }
}

template <bool STEP>
__global__ void __launch_bounds__(128) k_guard_faces_plan(gb_dev_grid g, gb_tree_desc t, const int* __restrict__ list,
                                                          const int4* __restrict__ plan)
{
    __shared__ int4 pb[54];
    const int blk = list[blockIdx.y];
    if (threadIdx.x < 54) pb[threadIdx.x] = __ldg(plan + (size_t)blk * 54 + threadIdx.x);
    __syncthreads();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (STEP ? GB_STEP_GUARD_FACES : GB_NGF)) return;
    if (blockIdx.z == 0)
        guard_face_plan<0, STEP>(g, t, blk, q, pb);
    else if (blockIdx.z == 1)
        guard_face_plan<1, STEP>(g, t, blk, q, pb);
    else
        guard_face_plan<2, STEP>(g, t, blk, q, pb);
}

__global__ void k_dt_init(unsigned long long* bits) { *bits = 0x7FF0000000000000ULL; }  // +inf

struct dt_limits {
    double dtmin, dtmax, change_factor;
};

// dt = CFL x the minimum limit; with a driver clock, limited as
// Driver_computeDt.F90:588,596 and shortened to end on t_max. Also
// dt / root_dx for the step's kernels.
__global__ void k_dt_finish(const unsigned long long* bits, double cfl, double* out, double* dtdx, float* dtdxf,
                            double dx0, double dx1, double dx2, gb_driver_state* drv, dt_limits lim)
{
    double dt = cfl * __longlong_as_double((long long)*bits);
    if (drv) {
        if (drv->dt_old > 0.0) dt = fmin(dt, drv->dt_old * lim.change_factor);
        dt = fmin(fmax(dt, lim.dtmin), lim.dtmax);
        const double left = drv->t_max - drv->sim_time;
        if (dt > left) dt = left > 0.0 ? left : 0.0;
        drv->dt = dt;
    }
    *out = dt;
    dtdx[0] = dt / dx0;
    dtdx[1] = dt / dx1;
    dtdx[2] = dt / dx2;
    dtdxf[0] = (float)dtdx[0];
    dtdxf[1] = (float)dtdx[1];
    dtdxf[2] = (float)dtdx[2];
}

__global__ void k_advance_clock(gb_driver_state* drv)
{
    // a step shortened to end on t_max lands on it exactly
    const double left = drv->t_max - drv->sim_time;
    drv->sim_time = drv->dt >= left ? drv->t_max : drv->sim_time + drv->dt;
    drv->dt_old = drv->dt;
    drv->nstep += 1.0;
}

__global__ void k_flash_to_soa(const double* __restrict__ in, int nunk, const int* __restrict__ hslot,
                               gb_dev_grid g, int nblocks, const int* __restrict__ list)
{
    // in: unk(nunk, 24, 24, 24, nblocks) Fortran order (variable fastest);
    // staged block q goes to store block list[q] (q itself without a list)
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = (int64_t)nblocks * GB_N3;
    if (idx >= total) return;
    int q = (int)(idx / GB_N3), c = (int)(idx % GB_N3);
    int blk = list ? list[q] : q;
    const double* cell = in + idx * nunk;
    for (int r = 0; r < GB_NROLE; ++r) {
        int hs = hslot[r], ds = g.slot[r];
        if (hs >= 0 && ds >= 0) g.unk[((int64_t)blk * g.nvar + ds) * GB_N3 + c] = cell[hs];
    }
}

__global__ void k_soa_to_flash(double* __restrict__ out, int nunk, const int* __restrict__ hslot,
                               gb_dev_grid g, int nblocks, const int* __restrict__ list)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = (int64_t)nblocks * GB_N3;
    if (idx >= total) return;
    int q = (int)(idx / GB_N3), c = (int)(idx % GB_N3);
    int blk = list ? list[q] : q;
    double* cell = out + idx * nunk;
    for (int r = 0; r < GB_NROLE; ++r) {
        int hs = hslot[r], ds = g.slot[r];
        if (hs >= 0 && ds >= 0) cell[hs] = g.unk[((int64_t)blk * g.nvar + ds) * GB_N3 + c];
    }
}

// FLASH-layout transfers straight from / to host memory the device can
// address (pinned host memory; on GB300 it is read and written over
// NVLink-C2C): one CTA moves FT cells of one block; the host side is one
// contiguous run of FT * nunk values, the store side one coalesced row per
// variable, transposed through shared memory.
constexpr int FT = 64;
static_assert(GB_N3 % FT == 0, "tile");

template <bool UP>
__global__ void __launch_bounds__(FT) k_flash_direct(double* host, int nunk, const int* __restrict__ hslot, gb_dev_grid g,
                                                     const int* __restrict__ list, int read_first)
{
    extern __shared__ double tile[];  // FT * nunk
    const int q = blockIdx.y;
    const int blk = list ? list[q] : q;
    const int c0 = blockIdx.x * FT;
    double* h = host + ((size_t)blk * GB_N3 + c0) * nunk;
    const int tot = FT * nunk;
    if (UP || read_first)
        for (int e = threadIdx.x; e < tot; e += FT) tile[e] = h[e];
    __syncthreads();
    const int c = c0 + threadIdx.x;
    for (int r = 0; r < GB_NROLE; ++r) {
        const int hs = hslot[r], ds = g.slot[r];
        if (hs < 0 || ds < 0) continue;
        double* d = g.unk + ((size_t)blk * g.nvar + ds) * GB_N3 + c;
        if (UP) *d = tile[threadIdx.x * nunk + hs];
        else tile[threadIdx.x * nunk + hs] = *d;
    }
    if (!UP) {
        __syncthreads();
        for (int e = threadIdx.x; e < tot; e += FT) h[e] = tile[e];
    }
}

// Interior cells only: one CTA moves FT interior cells (FT / 16 rows of
// 16 cells along i) of one block; each row is one contiguous run of
// 16 * nunk host values.
constexpr int IROWS = FT / GB_NXB;
static_assert(FT % GB_NXB == 0 && (GB_NXB * GB_NXB) % IROWS == 0, "interior tile");

// Work items are (block, group of IROWS rows); a grid smaller than the
// item count strides over them (a download running beside compute kernels
// keeps a small footprint that way).
constexpr int ITEMS_PER_BLOCK = GB_NXB * GB_NXB / IROWS;

template <bool UP>
__global__ void __launch_bounds__(FT) k_flash_interior(double* host, int nunk, const int* __restrict__ hslot,
                                                       gb_dev_grid g, const int* __restrict__ list, int nblk,
                                                       int read_first)
{
    extern __shared__ double tile[];  // FT * nunk
    const int run = GB_NXB * nunk;
    const int tot = FT * nunk;
    for (int item = blockIdx.x; item < nblk * ITEMS_PER_BLOCK; item += gridDim.x) {
        const int blk = list[item / ITEMS_PER_BLOCK];
        const int row0 = (item % ITEMS_PER_BLOCK) * IROWS;  // rows (j, k) of the interior, j fastest
        auto hrow = [&](int r) {
            const int jk = row0 + r;
            const int ci = gb_cidx(GB_NGUARD, GB_NGUARD + jk % GB_NXB, GB_NGUARD + jk / GB_NXB);
            return host + ((size_t)blk * GB_N3 + ci) * nunk;
        };
        if (UP || read_first)
            for (int e = threadIdx.x; e < tot; e += FT) tile[e] = hrow(e / run)[e % run];
        __syncthreads();
        const int r = threadIdx.x / GB_NXB, i = threadIdx.x % GB_NXB;
        const int jk = row0 + r;
        const int c = gb_cidx(GB_NGUARD + i, GB_NGUARD + jk % GB_NXB, GB_NGUARD + jk / GB_NXB);
        for (int q = 0; q < GB_NROLE; ++q) {
            const int hs = hslot[q], ds = g.slot[q];
            if (hs < 0 || ds < 0) continue;
            double* d = g.unk + ((size_t)blk * g.nvar + ds) * GB_N3 + c;
            if (UP) *d = tile[threadIdx.x * nunk + hs];
            else tile[threadIdx.x * nunk + hs] = *d;
        }
        __syncthreads();
        if (!UP) {
            for (int e = threadIdx.x; e < tot; e += FT) hrow(e / run)[e % run] = tile[e];
            __syncthreads();
        }
    }
}

// The faces a block owns along each axis a: normal index 4..20 (17),
// transverse 4..19 (16 x 16); x fastest, so runs along x are contiguous on
// both sides.
constexpr int GB_NOWN = (GB_NXB + 1) * GB_NXB * GB_NXB;

template <bool UP>
__global__ void k_faces_interior(double* hx, double* hy, double* hz, gb_dev_grid g, const int* __restrict__ list,
                                 int nblk)
{
    const int64_t n = (int64_t)nblk * 3 * GB_NOWN;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t % GB_NOWN), a = (int)((t / GB_NOWN) % 3), q = (int)(t / (3 * GB_NOWN));
        const int blk = list[q];
        const int nx = GB_NXB + (a == 0), ny = GB_NXB + (a == 1);
        const int I = GB_NGUARD + e % nx, J = GB_NGUARD + (e / nx) % ny, K = GB_NGUARD + e / (nx * ny);
        const size_t off = (size_t)blk * GB_FSZ + gb_fidx(a, I, J, K);
        double* h = (a == 0 ? hx : a == 1 ? hy : hz) + off;
        double* d = (a == 0 ? g.f[0] : a == 1 ? g.f[1] : g.f[2]) + off;
        if (UP) *d = *h;
        else *h = *d;
    }
}

template <bool UP>
__global__ void k_faces_direct(double* hx, double* hy, double* hz, gb_dev_grid g, const int* __restrict__ list)
{
    const int a = blockIdx.z, q = blockIdx.y;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= GB_FSZ) return;
    const int blk = list ? list[q] : q;
    double* h = (a == 0 ? hx : a == 1 ? hy : hz) + (size_t)blk * GB_FSZ + e;
    double* d = g.f[a] + (size_t)blk * GB_FSZ + e;
    if (UP) *d = *h;
    else *h = *d;
}

}  // namespace

// The device address of host memory, when kernels may address it (pinned
// memory under unified addressing); nullptr otherwise.
static void* device_view(const void* host)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Allocations and the face-link table of flux conservation (before any
// capture). Returns whether flux conservation applies to the registered
// grid (a tree with more than one level).
static int fc_prepare(int nblk, cudaStream_t s, bool* active)
{
    *active = false;
    if (!g_gb.fc_on || !g_gb.tree_ok || g_gb.tree.maxlevel <= 0 || g_gb.hp.precision < 0) return GB_OK;
    const int nn = g_gb.tree.nnodes;
    if (!g_gb.links_ok || g_gb.links_n < nn) {
        if (g_gb.links_n < nn) {
            if (g_gb.d_links) cudaFree(g_gb.d_links);
            g_gb.d_links = nullptr;
            g_gb.links_n = 0;
            if (gb_check(cudaMalloc(&g_gb.d_links, (size_t)nn * 6 * 5 * sizeof(int)), "cudaMalloc(links)"))
                return GB_ERR_CUDA;
            g_gb.links_n = nn;
        }
        k_face_links<<<(nn * 6 + 255) / 256, 256, 0, s>>>(g_gb.tree, g_gb.d_links);
        if (gb_check(cudaGetLastError(), "k_face_links")) return GB_ERR_CUDA;
        g_gb.links_ok = true;
    }
    const size_t reg = (size_t)nn * 6 * GB_NXB * GB_NXB * gbh::NREG * sizeof(double);
    if (g_gb.fcreg_bytes < reg) {
        if (g_gb.d_fcreg) cudaFree(g_gb.d_fcreg);
        g_gb.d_fcreg = nullptr;
        g_gb.fcreg_bytes = 0;
        if (gb_check(cudaMalloc(&g_gb.d_fcreg, reg), "cudaMalloc(flux registers)")) return GB_ERR_CUDA;
        g_gb.fcreg_bytes = reg;
    }
    if (g_gb.hp.mhd) {
        const size_t ereg = (size_t)nn * gbh::NSURF * sizeof(double);
        if (g_gb.ereg_bytes < ereg) {
            if (g_gb.d_ereg) cudaFree(g_gb.d_ereg);
            g_gb.d_ereg = nullptr;
            g_gb.ereg_bytes = 0;
            if (gb_check(cudaMalloc(&g_gb.d_ereg, ereg), "cudaMalloc(edge registers)")) return GB_ERR_CUDA;
            g_gb.ereg_bytes = ereg;
        }
        // the edge matching finds the finer leaves through the guard-fill plan
        int rc = gb_guard_prepare(s);
        if (rc) return rc;
    }
    if (g_gb.fclist_cap < nblk) {
        if (g_gb.d_fclist) cudaFree(g_gb.d_fclist);
        g_gb.d_fclist = nullptr;
        g_gb.fclist_cap = 0;
        if (gb_check(cudaMalloc(&g_gb.d_fclist, (size_t)nblk * sizeof(int)), "cudaMalloc(level list)"))
            return GB_ERR_CUDA;
        g_gb.fclist_cap = nblk;
    }
    *active = true;
    return GB_OK;
}

int gb_fc_prepare(int nblk, cudaStream_t s)
{
    bool on = false;
    return fc_prepare(nblk, s, &on);
}

extern "C" int gb_set_flux_correction(int on)
{
    g_gb.fc_on = on != 0;
    g_gb.gen += 1;
    return GB_OK;
}

// Whether the plan's 32-bit level-local indices hold the tree: every
// position of the finest level, shifted once more, below 2^30.
static bool plan_fits(const gb_tree_desc& t)
{
    const long long n = (long long)std::max(t.nrx, std::max(t.nry, t.nrz)) << (LOG2_NXB + t.maxlevel);
    return n < (1LL << 29);
}

// The guard-fill plan of the registered tree (before any capture: it
// allocates once per registration).
int gb_guard_prepare(cudaStream_t s)
{
    if (!g_gb.tree_ok || g_gb.plan_ok || !plan_fits(g_gb.tree)) return GB_OK;
    const int nn = g_gb.tree.nnodes;
    if (g_gb.plan_n < nn) {
        if (g_gb.d_plan) cudaFree(g_gb.d_plan);
        g_gb.d_plan = nullptr;
        g_gb.plan_n = 0;
        if (gb_check(cudaMalloc(&g_gb.d_plan, (size_t)nn * (54 * sizeof(int4) + sizeof(int))), "cudaMalloc(guard plan)"))
            return GB_ERR_CUDA;
        g_gb.plan_n = nn;
    }
    // the per-node flags follow the entries of plan_n nodes (the allocation's
    // capacity, which a larger tree registered earlier may have set): the
    // edge matching reads them at the same place
    int* near = (int*)((int4*)g_gb.d_plan + (size_t)g_gb.plan_n * 54);
    cudaMemsetAsync(near, 0, (size_t)nn * sizeof(int), s);
    k_guard_plan<<<(nn * 27 + 255) / 256, 256, 0, s>>>(g_gb.tree, (int4*)g_gb.d_plan, near);
    if (gb_check(cudaGetLastError(), "k_guard_plan")) return GB_ERR_CUDA;
    g_gb.plan_ok = true;
    return GB_OK;
}

// the plan when it is ready; inside a capture that did not prepare it
// (nothing allocates there) the kernels walk from the root instead
static const int4* guard_plan(cudaStream_t s)
{
    if (!g_gb.tree_ok) return nullptr;
    if (!g_gb.plan_ok) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(s, &cs);
        if (cs != cudaStreamCaptureStatusNone || gb_guard_prepare(s) != GB_OK || !g_gb.plan_ok) return nullptr;
    }
    return (const int4*)g_gb.d_plan;
}

static guard_vars hydro_guard_vars();

// guard cells and (when face fields exist) guard faces of the listed
// blocks; step: only those a step reads
static void launch_guard_kernels(int nblk, const int* list, bool faces, bool step, cudaStream_t s)
{
    const int4* plan = guard_plan(s);
    gb_prof_begin(GBP_GUARD, s);
    if (plan && step) {
        k_guard_cells_plan<true><<<dim3((GB_STEP_GUARD_CELLS + 127) / 128, nblk), 128, 0, s>>>(
            g_gb.grid, g_gb.tree, list, hydro_guard_vars(), plan);
    } else if (plan) {
        k_guard_cells_plan<false><<<dim3((cell_slabs::COUNT + 127) / 128, nblk), 128, 0, s>>>(
            g_gb.grid, g_gb.tree, list, hydro_guard_vars(), plan);
    } else {
        k_guard_cells<<<dim3((GB_NGC + 127) / 128, nblk), 128, 0, s>>>(g_gb.grid, g_gb.tree, list,
                                                                        hydro_guard_vars());
    }
    gb_prof_end(GBP_GUARD, s);
    if (!faces) return;
    gb_prof_begin(GBP_GUARD, s);
    if (plan && step)
        k_guard_faces_plan<true><<<dim3((GB_STEP_GUARD_FACES + 127) / 128, nblk, 3), 128, 0, s>>>(g_gb.grid, g_gb.tree,
                                                                                                list, plan);
    else if (plan)
        k_guard_faces_plan<false><<<dim3((GB_NGF + 127) / 128, nblk, 3), 128, 0, s>>>(g_gb.grid, g_gb.tree, list,
                                                                                      plan);
    else
        k_guard_faces<<<dim3((GB_FSZ + 127) / 128, nblk, 3), 128, 0, s>>>(g_gb.grid, g_gb.tree, list);
    gb_prof_end(GBP_GUARD, s);
}

static guard_vars hydro_guard_vars()
{
    guard_vars gv;
    gv.n = 0;
    const int roles[] = {GB_DENS, GB_VELX, GB_VELY, GB_VELZ, GB_PRES, GB_ENER, GB_EINT, GB_MAGX, GB_MAGY, GB_MAGZ};
    for (int r : roles)
        if (g_gb.grid.slot[r] >= 0) gv.slot[gv.n++] = g_gb.grid.slot[r];
    return gv;
}

int gb_launch_guardfill(int nblk, const int* list, cudaStream_t s)
{
    launch_guard_kernels(nblk, list, g_gb.hp.mhd && g_gb.grid.f[0], true, s);
    return gb_check(cudaGetLastError(), "guard fill") ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_fill_guardcells(int blockCount, const int* list, void* stream)
{
    if (!g_gb.grid_ok || !g_gb.tree_ok) {
        gb_set_error("gb_fill_guardcells: register a grid with a block tree first");
        return GB_ERR_NOT_INIT;
    }
    if (blockCount < 0 || (blockCount > 0 && !list)) return GB_ERR_ARG;
    if (blockCount == 0) return GB_OK;
    // the face pass runs whenever the grid has face fields
    launch_guard_kernels(blockCount, list, g_gb.grid.f[0] && g_gb.grid.f[1] && g_gb.grid.f[2], false,
                         (cudaStream_t)stream);
    return gb_check(cudaGetLastError(), "guard fill") ? GB_ERR_CUDA : GB_OK;
}

// ---------------------------------------------------------------- hydro
size_t gb_hydro_scratch_bytes_fp64();
size_t gb_hydro_scratch_bytes_mixed();
int gb_hydro_chunk_fp64(const gbh::hydro_kparams& kp, int mhd, int cool, int nblk, const int* list,
                        void* scratch, gb_status* st, cudaStream_t s, cudaEvent_t ev_put, const sur_feat_out* sf,
                        cudaEvent_t ev_wait);
int gb_hydro_chunk_mixed(const gbh::hydro_kparams& kp, int mhd, int cool, int nblk, const int* list,
                         void* scratch, gb_status* st, cudaStream_t s, cudaEvent_t ev_put, const sur_feat_out* sf,
                         cudaEvent_t ev_wait);
int gb_dt_launch(const gbh::hydro_kparams& kp, int mhd, int nblk, const int* list,
                 unsigned long long* bits, cudaStream_t s);

static int g_chunk_blocks = 16;
static int g_chunk_streams = 1;
static int g_recon_tile = 32;
static int g_recon_occ = 0;

int gb_chunk_blocks() { return g_chunk_blocks; }
int gb_chunk_streams() { return g_chunk_streams; }
extern "C" int gb_get_chunk_streams(void) { return g_chunk_streams; }

// Chunks on two streams: consecutive chunks alternate between the caller's
// stream and a library stream, each with its own scratch, so that one
// chunk's FP64-bound kernels (update, face B, acceptance) run beside the
// next chunk's FP32-bound ones (reconstruction, fluxes, MLP). Results do not
// change: chunks touch disjoint blocks, and where flux conservation applies
// a chunk starts only after the previous chunk has registered its fluxes.
extern "C" int gb_set_chunk_streams(int n)
{
    if (n != 1 && n != 2) {
        gb_set_error("gb_set_chunk_streams: %d (1 or 2)", n);
        return GB_ERR_ARG;
    }
    g_chunk_streams = n;
    g_gb.gen += 1;
    return GB_OK;
}

namespace {
struct chunk_aux {
    cudaStream_t s2 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    std::vector<cudaEvent_t> put;  // one per chunk
    // per-chunk downloads of a host-resident step (gb_step_graph_host)
    cudaStream_t s3 = nullptr;
    cudaEvent_t dl = nullptr, dl_join = nullptr;
    // the step graph's CFL reduction beside its guard fill
    cudaStream_t s_dt = nullptr;
    cudaEvent_t dt_fork = nullptr, dt_join = nullptr;
} g_aux;

// The device views of a host-resident state while its step is recorded
// (nullptr otherwise).
struct host_io_dev {
    double* unk = nullptr;
    int nunk = 0, read_first = 0;
    double* f[3] = {nullptr, nullptr, nullptr};
    int* dslot = nullptr;  // device copy of the slot map
};
const host_io_dev* g_hio = nullptr;
}  // namespace

static int dt_stream_prepare()
{
    if (!g_aux.s_dt && gb_check(cudaStreamCreateWithFlags(&g_aux.s_dt, cudaStreamNonBlocking), "dt stream"))
        return GB_ERR_CUDA;
    if (!g_aux.dt_fork && (gb_check(cudaEventCreateWithFlags(&g_aux.dt_fork, cudaEventDisableTiming), "event") ||
                           gb_check(cudaEventCreateWithFlags(&g_aux.dt_join, cudaEventDisableTiming), "event")))
        return GB_ERR_CUDA;
    return GB_OK;
}

static int g_io_priority = 0;  // the device's greatest stream priority

static int io_streams_prepare()
{
    if (!g_aux.s3) {
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        g_io_priority = greatest;
        if (gb_check(cudaStreamCreateWithPriority(&g_aux.s3, cudaStreamNonBlocking, greatest), "download stream"))
            return GB_ERR_CUDA;
    }
    if (!g_aux.dl && (gb_check(cudaEventCreateWithFlags(&g_aux.dl, cudaEventDisableTiming), "event") ||
                      gb_check(cudaEventCreateWithFlags(&g_aux.dl_join, cudaEventDisableTiming), "event")))
        return GB_ERR_CUDA;
    return GB_OK;
}

// interior transfers of nblk listed blocks (device list) of a host-resident state
static void launch_io(bool up, const host_io_dev& io, int nblk, const int* list, cudaStream_t s);

// The second stream and the events of a step of nchunks chunks (before any
// capture: it creates them once).
int gb_streams_prepare(int nchunks)
{
    if (g_chunk_streams < 2) return GB_OK;
    if (!g_aux.s2 && gb_check(cudaStreamCreateWithFlags(&g_aux.s2, cudaStreamNonBlocking), "chunk stream"))
        return GB_ERR_CUDA;
    if (!g_aux.fork && (gb_check(cudaEventCreateWithFlags(&g_aux.fork, cudaEventDisableTiming), "event") ||
                        gb_check(cudaEventCreateWithFlags(&g_aux.join, cudaEventDisableTiming), "event")))
        return GB_ERR_CUDA;
    while ((int)g_aux.put.size() < nchunks) {
        cudaEvent_t e;
        if (gb_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event")) return GB_ERR_CUDA;
        g_aux.put.push_back(e);
    }
    return GB_OK;
}
int gb_recon_tile() { return g_recon_tile; }

static int g_fused = 0;
int gb_fused_step() { return g_fused; }
int gb_fused_attr_fp64();
int gb_fused_attr_mixed();

extern "C" int gb_set_fused(int on)
{
    if (on < 0 || on > 2) {
        gb_set_error("gb_set_fused: mode %d is not 0, 1 or 2", on);
        return GB_ERR_ARG;
    }
    if (on) {
        // the fused kernels' shared memory beyond the default 48 KB
        if (gb_fused_attr_fp64() || gb_fused_attr_mixed()) return GB_ERR_CUDA;
    }
    g_fused = on;
    g_gb.gen += 1;
    return GB_OK;
}

extern "C" int gb_get_fused(void) { return g_fused; }
int gb_recon_occupancy() { return g_recon_occ; }

extern "C" int gb_set_launch_config(int chunk_blocks, int recon_tile, int recon_occupancy)
{
    if (chunk_blocks < 1 || chunk_blocks > 65535 || (recon_tile != 32 && recon_tile != 64) || recon_occupancy < 0 ||
        recon_occupancy > 2) {
        gb_set_error("gb_set_launch_config: chunk %d (1..65535), recon tile %d (32 or 64), occupancy %d (0..2)",
                     chunk_blocks, recon_tile, recon_occupancy);
        return GB_ERR_ARG;
    }
    g_chunk_blocks = chunk_blocks;
    g_recon_tile = recon_tile;
    g_recon_occ = recon_occupancy;
    g_gb.gen += 1;
    return GB_OK;
}

extern "C" int gb_get_launch_config(int* chunk_blocks, int* recon_tile, int* recon_occupancy)
{
    if (chunk_blocks) *chunk_blocks = g_chunk_blocks;
    if (recon_tile) *recon_tile = g_recon_tile;
    if (recon_occupancy) *recon_occupancy = g_recon_occ;
    return GB_OK;
}

extern "C" int gb_set_chunk_blocks(int n)
{
    if (n < 1 || n > 65535) return GB_ERR_ARG;
    g_chunk_blocks = n;
    g_gb.gen += 1;
    return GB_OK;
}

gbh::hydro_kparams gb_make_kp(double dt, const double* dtp)
{
    gbh::hydro_kparams kp;
    kp.dtp = dtp;
    kp.dtdxp = dtp ? g_gb.d_dtmin + 1 : nullptr;  // written by k_dt_finish
    kp.fc_links = nullptr;
    kp.fc_reg = nullptr;
    kp.gammaf = (float)g_gb.hp.gamma;
    kp.inv_gm1 = 1.0 / (g_gb.hp.gamma - 1.0);
    kp.cviscf = (float)g_gb.hp.cvisc;
    kp.dtdxfp = dtp ? (const float*)(g_gb.d_dtmin + 4) : nullptr;  // written by k_dt_finish
    kp.gamma = g_gb.hp.gamma;
    kp.cvisc = g_gb.hp.cvisc;
    kp.eint_switch = g_gb.hp.eint_switch;
    kp.smlrho = g_gb.hp.smlrho;
    kp.smallp = g_gb.hp.smallp;
    kp.use_avisc = g_gb.hp.use_avisc;
    kp.energy_fix = g_gb.hp.mhd && g_gb.hp.energy_fix;
    kp.hybrid = g_gb.hp.hybrid_order;
    kp.lower_cfl = g_gb.hp.fallback_lower_cfl;
    kp.kappa = g_gb.hp.hybrid_kappa;
    kp.cflc = g_gb.d_cflc;
    kp.cfl_sum = g_gb.hp.cfl_sum;
    {
        // a code's scale: the lowered CFL over cfl, at most 1
        const double s1 = fmin(1.0, (g_gb.hp.cfl_fallback_factor / 3.0) / g_gb.hp.cfl);
        const double s2 = fmin(1.0, 0.25 / g_gb.hp.cfl);
        kp.cflsc = {{1.0, s1, s2, fmin(s1, s2)}};
    }
    kp.dt = dt;
    if (g_gb.tree_ok) {
        kp.dx[0] = g_gb.tree.root_dx[0];
        kp.dx[1] = g_gb.tree.root_dx[1];
        kp.dx[2] = g_gb.tree.root_dx[2];
    } else {
        kp.dx[0] = kp.dx[1] = kp.dx[2] = 1.0;
    }
    for (int d = 0; d < 3; ++d) {
        kp.dtdx0[d] = dt / kp.dx[d];
        kp.dtdxf0[d] = (float)kp.dtdx0[d];
        kp.iso = kp.dx[0] == kp.dx[1] && kp.dx[1] == kp.dx[2];
    }
    return kp;
}

int gb_cooling_mode();
int gb_launch_surrogate(int nblk, const int* list, double dt, const double* dtp, gb_status* st, cudaStream_t s,
                        int chain, bool feat_done);
int gb_sur_feat_target(int chain, int nblk, sur_feat_out* out);

int gb_launch_hydro(int nblk, const int* list, double dt, const double* dtp, int cool, gb_status* st,
                    cudaStream_t s)
{
    const int chunk = g_chunk_blocks < nblk ? g_chunk_blocks : nblk;
    const bool mixed = g_gb.hp.precision == 1;
    const int nchunks = (nblk + chunk - 1) / chunk;
    // the in-library profiler times launches one by one: one stream then
    const int ns = g_chunk_streams > 1 && nchunks > 1 && !g_prof.on ? 2 : 1;
    size_t per = mixed ? gb_hydro_scratch_bytes_mixed() : gb_hydro_scratch_bytes_fp64();
    const size_t chunk_bytes = (per * (size_t)chunk + 255) / 256 * 256;
    int rc = gb_ensure_scratch(chunk_bytes * ns);
    if (rc) return rc;
    if (ns > 1) {
        rc = gb_streams_prepare(nchunks);
        if (rc) return rc;
    }
    gbh::hydro_kparams kp = gb_make_kp(dt, dtp);
    bool fc = false;
    rc = fc_prepare(nblk, s, &fc);
    if (rc) return rc;
    if (fc) {
        // finest level first, so fine boundary fluxes are registered before
        // the coarse blocks next to them are updated
        k_sort_levels<<<1, 1024, 0, s>>>(list, nblk, g_gb.tree.level, g_gb.tree.maxlevel, g_gb.d_fclist);
        if (gb_check(cudaGetLastError(), "k_sort_levels")) return GB_ERR_CUDA;
        list = g_gb.d_fclist;
        kp.fc_links = g_gb.d_links;
        kp.fc_reg = g_gb.d_fcreg;
        if (g_gb.hp.mhd && g_gb.plan_ok && g_gb.d_ereg) {
            kp.ec_plan = (const int4*)g_gb.d_plan;
            kp.ec_near = (const int*)((const int4*)g_gb.d_plan + (size_t)g_gb.plan_n * 54);
            kp.ec_child = g_gb.tree.child;
            kp.ec_reg = g_gb.d_ereg;
        }
    }
    if (ns > 1) {
        cudaEventRecord(g_aux.fork, s);
        cudaStreamWaitEvent(g_aux.s2, g_aux.fork, 0);
    }
    for (int k = 0, b0 = 0; b0 < nblk; ++k, b0 += chunk) {
        int nb = nblk - b0 < chunk ? nblk - b0 : chunk;
        // the plain integrator after the update: 1 fused into it on the
        // precision path's own rates, 2 on FP32 rates (mixed path: a pass of
        // its own after the update; FP64 takes it as 1)
        const int fused = !cool ? 0 : gb_cooling_mode() == 0 ? 1 : gb_cooling_mode() == 2 ? 2 : 0;
        const int chain = ns > 1 ? (k & 1) : 0;
        cudaStream_t sk = chain ? g_aux.s2 : s;
        void* scr = (char*)g_gb.d_scratch + (size_t)chain * chunk_bytes;
        cudaEvent_t ev_put = nullptr, ev_wait = nullptr;
        if (ns > 1 && fc) {
            // the fine boundary fluxes and edge fields this chunk reads were
            // registered by earlier chunks: before its first register read it
            // waits for the previous chunk's registration event. That covers
            // every earlier chunk: the ones on the other stream ran before the
            // previous chunk there, the ones on this stream before this one.
            if (k > 0) ev_wait = g_aux.put[k - 1];
            ev_put = g_aux.put[k];
        }
        // the surrogate cools this chunk next: the update writes its features
        sur_feat_out sf;
        const bool feat = cool && !fused && gb_sur_feat_target(chain, nb, &sf) == GB_OK;
        rc = mixed ? gb_hydro_chunk_mixed(kp, g_gb.hp.mhd, fused, nb, list + b0, scr, st, sk, ev_put,
                                          feat ? &sf : nullptr, ev_wait)
                   : gb_hydro_chunk_fp64(kp, g_gb.hp.mhd, fused, nb, list + b0, scr, st, sk, ev_put,
                                         feat ? &sf : nullptr, ev_wait);
        if (rc) return rc;
        if (cool && !fused) {
            rc = gb_launch_surrogate(nb, list + b0, dt, dtp, st, sk, chain, feat);
            if (rc) return rc;
        }
        if (g_hio) {
            // this chunk's blocks are final: download them on the download
            // stream while later chunks compute
            cudaEventRecord(g_aux.dl, sk);
            cudaStreamWaitEvent(g_aux.s3, g_aux.dl, 0);
            launch_io(false, *g_hio, nb, list + b0, g_aux.s3);
        }
    }
    if (g_hio) {
        cudaEventRecord(g_aux.dl_join, g_aux.s3);
        cudaStreamWaitEvent(s, g_aux.dl_join, 0);
    }
    if (ns > 1) {
        cudaEventRecord(g_aux.join, g_aux.s2);
        cudaStreamWaitEvent(s, g_aux.join, 0);
    }
    return GB_OK;
}

extern "C" int gb_hydro_unsplit(int blockCount, const int* list, double dt, double dtOld, gb_status* st,
                                void* stream)
{
    (void)dtOld;
    if (!g_gb.grid_ok || !g_gb.hydro_ok) {
        gb_set_error("gb_hydro_unsplit: call gb_register_grid and gb_hydro_init first");
        return GB_ERR_NOT_INIT;
    }
    if (blockCount < 0 || (blockCount > 0 && !list) || !(dt > 0.0)) {
        gb_set_error("gb_hydro_unsplit: bad block list or dt = %g", dt);
        return GB_ERR_ARG;
    }
    if (g_gb.hp.mhd && (!g_gb.grid.f[0] || !g_gb.grid.f[1] || !g_gb.grid.f[2] || g_gb.grid.slot[GB_MAGX] < 0 ||
                        g_gb.grid.slot[GB_MAGY] < 0 || g_gb.grid.slot[GB_MAGZ] < 0)) {
        gb_set_error("gb_hydro_unsplit: MHD needs face fields and MAG slots");
        return GB_ERR_ARG;
    }
    if (blockCount == 0) return GB_OK;
    return gb_launch_hydro(blockCount, list, dt, nullptr, 0, st, (cudaStream_t)stream);
}

static dt_limits g_dt_limits = {0.0, __builtin_huge_val(), __builtin_huge_val()};

extern "C" int gb_set_dt_limits(double dtmin, double dtmax, double change_factor)
{
    if (!(dtmin >= 0.0) || !(dtmax > 0.0) || !(dtmin <= dtmax) || !(change_factor > 0.0)) {
        gb_set_error("gb_set_dt_limits: need 0 <= dtmin <= dtmax and change_factor > 0");
        return GB_ERR_ARG;
    }
    g_dt_limits = {dtmin, dtmax, change_factor};
    g_gb.gen += 1;
    return GB_OK;
}

static int launch_dt(int nblk, const int* list, double* dt_out, gb_driver_state* drv, cudaStream_t s)
{
    k_dt_init<<<1, 1, 0, s>>>((unsigned long long*)g_gb.d_dtmin);
    gbh::hydro_kparams kp = gb_make_kp(1.0, nullptr);
    gb_prof_begin(GBP_DT, s);
    int rc = gb_dt_launch(kp, g_gb.hp.mhd, nblk, list, (unsigned long long*)g_gb.d_dtmin, s);
    if (rc) return rc;
    k_dt_finish<<<1, 1, 0, s>>>((const unsigned long long*)g_gb.d_dtmin, g_gb.hp.cfl, dt_out, g_gb.d_dtmin + 1,
                                (float*)(g_gb.d_dtmin + 4), kp.dx[0], kp.dx[1], kp.dx[2], drv, g_dt_limits);
    gb_prof_end(GBP_DT, s);
    return gb_check(cudaGetLastError(), "k_dt_finish") ? GB_ERR_CUDA : GB_OK;
}

int gb_launch_dt(int nblk, const int* list, double* dt_out, cudaStream_t s)
{
    return launch_dt(nblk, list, dt_out, nullptr, s);
}

extern "C" int gb_compute_dt(int blockCount, const int* list, double* dt_dev, void* stream)
{
    if (!g_gb.grid_ok || !g_gb.hydro_ok) {
        gb_set_error("gb_compute_dt: call gb_register_grid and gb_hydro_init first");
        return GB_ERR_NOT_INIT;
    }
    if (blockCount <= 0 || !list || !dt_dev) return GB_ERR_ARG;
    return gb_launch_dt(blockCount, list, dt_dev, (cudaStream_t)stream);
}

extern "C" int gb_evolve_step(int blockCount, const int* list, double dt, int cool, gb_status* st,
                              void* stream)
{
    if (!g_gb.grid_ok || !g_gb.hydro_ok || !g_gb.tree_ok) {
        gb_set_error("gb_evolve_step: register grid + tree and call gb_hydro_init first");
        return GB_ERR_NOT_INIT;
    }
    if (cool && !g_gb.cool_ok) {
        gb_set_error("gb_evolve_step: cooling requested before gb_cool_init");
        return GB_ERR_NOT_INIT;
    }
    if (cool && (g_gb.grid.slot[GB_TEMP] < 0 || g_gb.grid.slot[GB_TDUS] < 0)) {
        gb_set_error("gb_evolve_step: cooling needs TEMP and TDUS slots");
        return GB_ERR_ARG;
    }
    if (blockCount <= 0 || !list || !(dt > 0.0)) {
        gb_set_error("gb_evolve_step: bad block list or dt = %g", dt);
        return GB_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int rc = gb_launch_guardfill(blockCount, list, s);
    if (rc) return rc;
    return gb_launch_hydro(blockCount, list, dt, nullptr, cool, st, s);
}

// ---------------------------------------------------------------- step graph
// The whole step -- CFL reduction into dt_dev, guard fill, every hydro
// chunk, cooling -- captured once as a CUDA graph on a private stream and
// replayed on the caller's stream. Kernels read dt from dt_dev, so the
// host never waits inside a step. The graph is re-captured whenever an
// argument or anything it baked in (gen) changes.
namespace {
struct step_graph {
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;
    const int* list = nullptr;
    int n = 0, cool = -1;
    gb_driver_state* drv = nullptr;
    gb_status* st = nullptr;
    unsigned long long gen = ~0ULL;
    long long launches = 0, captures = 0, kernel_nodes = 0;
    // the host-resident state the graph was recorded for (io.unk null: none)
    gb_host_io io = {};
    host_io_dev dio;
} g_graph;

bool same_io(const gb_host_io* a, const gb_host_io& b)
{
    if (!a) return b.unk == nullptr;
    return a->unk == b.unk && a->nunk == b.nunk && a->facex == b.facex && a->facey == b.facey &&
           a->facez == b.facez && memcmp(a->host_slot, b.host_slot, sizeof b.host_slot) == 0;
}

void graph_drop()
{
    if (g_graph.exec) cudaGraphExecDestroy(g_graph.exec);
    g_graph.exec = nullptr;
}

int record_step(int n, const int* list, int cool, gb_driver_state* drv, gb_status* st, cudaStream_t s)
{
    double* dt_dev = &drv->dt;
    if (g_hio) {
        launch_io(true, *g_hio, n, list, s);
        if (gb_check(cudaGetLastError(), "interior upload")) return GB_ERR_CUDA;
    }
    // the CFL reduction reads interiors, the guard fill writes guard cells:
    // they run side by side, and the chunks wait for both
    cudaEventRecord(g_aux.dt_fork, s);
    cudaStreamWaitEvent(g_aux.s_dt, g_aux.dt_fork, 0);
    int rc = launch_dt(n, list, dt_dev, drv, g_aux.s_dt);
    if (rc) return rc;
    cudaEventRecord(g_aux.dt_join, g_aux.s_dt);
    rc = gb_launch_guardfill(n, list, s);
    if (rc) return rc;
    cudaStreamWaitEvent(s, g_aux.dt_join, 0);
    rc = gb_launch_hydro(n, list, 1.0, dt_dev, cool, st, s);
    if (rc) return rc;
    k_advance_clock<<<1, 1, 0, s>>>(drv);
    return gb_check(cudaGetLastError(), "k_advance_clock") ? GB_ERR_CUDA : GB_OK;
}
}  // namespace

int gb_cooling_mode();

static int run_step_graph(int blockCount, const int* list, int cool, gb_driver_state* drv, gb_status* st,
                      const gb_host_io* io, void* stream)
{
    if (!g_gb.grid_ok || !g_gb.hydro_ok || !g_gb.tree_ok) {
        gb_set_error("gb_step_graph: register grid + tree and call gb_hydro_init first");
        return GB_ERR_NOT_INIT;
    }
    if (cool && (!g_gb.cool_ok || g_gb.grid.slot[GB_TEMP] < 0 || g_gb.grid.slot[GB_TDUS] < 0)) {
        gb_set_error("gb_step_graph: cooling needs gb_cool_init and TEMP/TDUS slots");
        return GB_ERR_NOT_INIT;
    }
    if (blockCount <= 0 || !list || !drv) {
        gb_set_error("gb_step_graph: bad block list or driver state pointer");
        return GB_ERR_ARG;
    }
    if (gb_prof_is_on()) {
        gb_set_error("gb_step_graph: the in-library profiler times launches one by one; disable it first");
        return GB_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const bool same = g_graph.exec && g_graph.list == list && g_graph.n == blockCount && g_graph.cool == cool &&
                      g_graph.drv == drv && g_graph.st == st && g_graph.gen == g_gb.gen && same_io(io, g_graph.io);
    if (!same) {
        graph_drop();
        g_graph.io = gb_host_io{};
        host_io_dev dio;
        if (io) {
            // device views of the pinned host arrays and a device copy of
            // the slot map (the graph bakes both in)
            dio.unk = (double*)device_view(io->unk);
            dio.nunk = io->nunk;
            const bool faces = io->facex || io->facey || io->facez;
            for (int a = 0; a < 3 && faces; ++a)
                dio.f[a] = (double*)device_view(a == 0 ? io->facex : a == 1 ? io->facey : io->facez);
            if (!dio.unk || io->nunk <= 0 || (size_t)FT * io->nunk * sizeof(double) > 48 * 1024 ||
                (faces && (!dio.f[0] || !dio.f[1] || !dio.f[2] || !g_gb.grid.f[0]))) {
                gb_set_error("gb_step_graph_host: host arrays must be pinned (nunk %d, up to %d)", io->nunk,
                             (int)(48 * 1024 / (FT * 8)));
                return GB_ERR_ARG;
            }
            int mapped = 0;
            for (int r = 0; r < GB_NROLE; ++r)
                if (io->host_slot[r] >= 0 && io->host_slot[r] < io->nunk && g_gb.grid.slot[r] >= 0) ++mapped;
            dio.read_first = mapped < io->nunk;
            if (!g_graph.dio.dslot && gb_check(cudaMalloc(&g_graph.dio.dslot, GB_NROLE * sizeof(int)), "slot map"))
                return GB_ERR_CUDA;
            dio.dslot = g_graph.dio.dslot;
            if (gb_check(cudaMemcpy(dio.dslot, io->host_slot, GB_NROLE * sizeof(int), cudaMemcpyHostToDevice),
                         "slot map") ||
                io_streams_prepare())
                return GB_ERR_CUDA;
        }
        if (!g_graph.cap && gb_check(cudaStreamCreateWithFlags(&g_graph.cap, cudaStreamNonBlocking), "graph stream"))
            return GB_ERR_CUDA;
        // everything that allocates or uploads happens before the capture
        const int chunk = gb_chunk_blocks() < blockCount ? gb_chunk_blocks() : blockCount;
        size_t per = g_gb.hp.precision == 1 ? gb_hydro_scratch_bytes_mixed() : gb_hydro_scratch_bytes_fp64();
        int rc = gb_ensure_scratch((per * (size_t)chunk + 255) / 256 * 256 * (size_t)g_chunk_streams);
        if (!rc && cool && gb_cooling_mode() == 1) rc = gb_sur_prepare((int64_t)chunk * 4096, s);
        if (!rc) rc = gb_fc_prepare(blockCount, s);
        if (!rc) rc = gb_guard_prepare(s);
        if (!rc) rc = gb_streams_prepare((blockCount + chunk - 1) / chunk);
        if (!rc) rc = dt_stream_prepare();
        if (rc) return rc;
        if (gb_check(cudaStreamSynchronize(s), "graph prepare")) return GB_ERR_CUDA;
        if (gb_check(cudaStreamBeginCapture(g_graph.cap, cudaStreamCaptureModeThreadLocal), "begin capture"))
            return GB_ERR_CUDA;
        g_graph.dio = dio.unk ? dio : host_io_dev{nullptr, 0, 0, {nullptr, nullptr, nullptr}, g_graph.dio.dslot};
        g_hio = io ? &g_graph.dio : nullptr;
        rc = record_step(blockCount, list, cool, drv, st, g_graph.cap);
        g_hio = nullptr;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(g_graph.cap, &graph);
        if (rc || gb_check(e, "end capture")) {
            if (graph) cudaGraphDestroy(graph);
            return rc ? rc : GB_ERR_CUDA;
        }
        size_t nn = 0;
        cudaGraphGetNodes(graph, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        long long kn = 0;
        if (nn && cudaGraphGetNodes(graph, nodes.data(), &nn) == cudaSuccess)
            for (size_t q = 0; q < nn; ++q) {
                cudaGraphNodeType ty;
                if (cudaGraphNodeGetType(nodes[q], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) ++kn;
            }
        g_graph.kernel_nodes = kn;
        e = cudaGraphInstantiate(&g_graph.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (gb_check(e, "graph instantiate")) {
            g_graph.exec = nullptr;
            return GB_ERR_CUDA;
        }
        g_graph.list = list;
        g_graph.n = blockCount;
        g_graph.cool = cool;
        g_graph.drv = drv;
        g_graph.st = st;
        g_graph.gen = g_gb.gen;
        g_graph.io = io ? *io : gb_host_io{};
        g_graph.captures += 1;
    }
    g_graph.launches += 1;
    return gb_check(cudaGraphLaunch(g_graph.exec, s), "graph launch") ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_step_graph(int blockCount, const int* list, int cool, gb_driver_state* drv, gb_status* st,
                             void* stream)
{
    return run_step_graph(blockCount, list, cool, drv, st, nullptr, stream);
}

extern "C" int gb_step_graph_host(int blockCount, const int* list, int cool, gb_driver_state* drv, gb_status* st,
                                  const gb_host_io* io, void* stream)
{
    if (!io) {
        gb_set_error("gb_step_graph_host: no host state");
        return GB_ERR_ARG;
    }
    return run_step_graph(blockCount, list, cool, drv, st, io, stream);
}

extern "C" int gb_graph_info(long long* captures, long long* launches, long long* kernel_nodes)
{
    if (captures) *captures = g_graph.captures;
    if (launches) *launches = g_graph.launches;
    if (kernel_nodes) *kernel_nodes = g_graph.exec ? g_graph.kernel_nodes : 0;
    return GB_OK;
}

extern "C" int gb_graph_reset(void)
{
    graph_drop();
    return GB_OK;
}

// ---------------------------------------------------------------- host I/O
static int flash_copy(bool up, double* host, int nunk, const int* host_slot, int nblocks, void* stream)
{
    if (!g_gb.grid_ok) {
        gb_set_error("grid transfer before gb_register_grid");
        return GB_ERR_NOT_INIT;
    }
    if (!host || !host_slot || nunk <= 0 || nblocks <= 0 || nblocks > g_gb.grid.maxblocks) return GB_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    size_t bytes = (size_t)nblocks * GB_N3 * nunk * sizeof(double);
    int rc = gb_ensure_stage(bytes + GB_NROLE * sizeof(int));
    if (rc) return rc;
    int* dslot = (int*)((char*)g_gb.d_stage + bytes);
    if (gb_check(cudaMemcpyAsync(dslot, host_slot, GB_NROLE * sizeof(int), cudaMemcpyHostToDevice, s), "slot copy"))
        return GB_ERR_CUDA;
    int64_t total = (int64_t)nblocks * GB_N3;
    unsigned nb = (unsigned)((total + 255) / 256);
    if (up) {
        if (gb_check(cudaMemcpyAsync(g_gb.d_stage, host, bytes, cudaMemcpyHostToDevice, s), "upload")) return GB_ERR_CUDA;
        gb_prof_begin(GBP_COPY, s);
        k_flash_to_soa<<<nb, 256, 0, s>>>(g_gb.d_stage, nunk, dslot, g_gb.grid, nblocks, nullptr);
        gb_prof_end(GBP_COPY, s);
        if (gb_check(cudaGetLastError(), "k_flash_to_soa")) return GB_ERR_CUDA;
    } else {
        gb_prof_begin(GBP_COPY, s);
        k_soa_to_flash<<<nb, 256, 0, s>>>(g_gb.d_stage, nunk, dslot, g_gb.grid, nblocks, nullptr);
        gb_prof_end(GBP_COPY, s);
        if (gb_check(cudaGetLastError(), "k_soa_to_flash")) return GB_ERR_CUDA;
        if (gb_check(cudaMemcpyAsync(host, g_gb.d_stage, bytes, cudaMemcpyDeviceToHost, s), "download"))
            return GB_ERR_CUDA;
    }
    return GB_OK;
}

extern "C" int gb_grid_upload_flash(const double* unk_host, int nunk, const int* host_slot, int nblocks,
                                    void* stream)
{
    return flash_copy(true, const_cast<double*>(unk_host), nunk, host_slot, nblocks, stream);
}

extern "C" int gb_grid_download_flash(double* unk_host, int nunk, const int* host_slot, int nblocks,
                                      void* stream)
{
    return flash_copy(false, unk_host, nunk, host_slot, nblocks, stream);
}

// Runs of consecutive store ids in a host block list: [q0, q0 + len) of the
// list covers store blocks list[q0] .. list[q0] + len - 1.
template <typename F>
static int for_each_run(int n, const int* list, F&& f)
{
    for (int q0 = 0; q0 < n;) {
        int len = 1;
        while (q0 + len < n && list[q0 + len] == list[q0] + len) ++len;
        int rc = f(q0, list[q0], len);
        if (rc) return rc;
        q0 += len;
    }
    return GB_OK;
}

static int check_host_list(int n, const int* list, const char* who)
{
    if (n < 0 || (n > 0 && !list)) {
        gb_set_error("%s: bad block list", who);
        return GB_ERR_ARG;
    }
    for (int q = 0; q < n; ++q)
        if (list[q] < 0 || list[q] >= g_gb.grid.maxblocks) {
            gb_set_error("%s: block id %d outside the store (maxblocks %d)", who, list[q], g_gb.grid.maxblocks);
            return GB_ERR_ARG;
        }
    return GB_OK;
}

static int flash_copy_list(bool up, double* host, int nunk, const int* host_slot, int n, const int* list,
                           void* stream)
{
    if (!g_gb.grid_ok) {
        gb_set_error("grid transfer before gb_register_grid");
        return GB_ERR_NOT_INIT;
    }
    if (!host || !host_slot || nunk <= 0) return GB_ERR_ARG;
    int rc = check_host_list(n, list, up ? "gb_grid_upload_flash_list" : "gb_grid_download_flash_list");
    if (rc || n == 0) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t per = (size_t)GB_N3 * nunk;  // doubles per FLASH block
    double* hd = (double*)device_view(host);
    // staging: the blocks themselves unless the kernel can address the host
    // array, then the slot map and the list
    const size_t bytes = hd ? 0 : (size_t)n * per * sizeof(double);
    rc = gb_ensure_stage(bytes + (GB_NROLE + (size_t)n) * sizeof(int));
    if (rc) return rc;
    double* stage = (double*)g_gb.d_stage;
    int* dslot = (int*)((char*)g_gb.d_stage + bytes);
    int* dlist = dslot + GB_NROLE;
    if (gb_check(cudaMemcpyAsync(dslot, host_slot, GB_NROLE * sizeof(int), cudaMemcpyHostToDevice, s), "slot copy") ||
        gb_check(cudaMemcpyAsync(dlist, list, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s), "list copy"))
        return GB_ERR_CUDA;
    if (hd) {
        // the kernel reads / writes the host array in place: no staging
        // copies, one launch for the whole list
        int mapped = 0;
        for (int r = 0; r < GB_NROLE; ++r)
            if (host_slot[r] >= 0 && host_slot[r] < nunk && g_gb.grid.slot[r] >= 0) ++mapped;
        const size_t smem = (size_t)FT * nunk * sizeof(double);
        if (smem > 48 * 1024) {
            gb_set_error("FLASH transfer: nunk %d above the %d variables one tile holds", nunk, (int)(48 * 1024 / (FT * 8)));
            return GB_ERR_ARG;
        }
        dim3 grid(GB_N3 / FT, n);
        gb_prof_begin(GBP_COPY, s);
        if (up) k_flash_direct<true><<<grid, FT, smem, s>>>(hd, nunk, dslot, g_gb.grid, dlist, 0);
        else k_flash_direct<false><<<grid, FT, smem, s>>>(hd, nunk, dslot, g_gb.grid, dlist, mapped < nunk);
        gb_prof_end(GBP_COPY, s);
        return gb_check(cudaGetLastError(), "k_flash_direct") ? GB_ERR_CUDA : GB_OK;
    }
    const unsigned nb = (unsigned)(((int64_t)n * GB_N3 + 255) / 256);
    if (up) {
        rc = for_each_run(n, list, [&](int q0, int b0, int len) {
            return gb_check(cudaMemcpyAsync(stage + (size_t)q0 * per, host + (size_t)b0 * per,
                                            (size_t)len * per * sizeof(double), cudaMemcpyHostToDevice, s),
                            "upload") ? GB_ERR_CUDA : GB_OK;
        });
        if (rc) return rc;
        gb_prof_begin(GBP_COPY, s);
        k_flash_to_soa<<<nb, 256, 0, s>>>(stage, nunk, dslot, g_gb.grid, n, dlist);
        gb_prof_end(GBP_COPY, s);
        return gb_check(cudaGetLastError(), "k_flash_to_soa") ? GB_ERR_CUDA : GB_OK;
    }
    gb_prof_begin(GBP_COPY, s);
    k_soa_to_flash<<<nb, 256, 0, s>>>(stage, nunk, dslot, g_gb.grid, n, dlist);
    gb_prof_end(GBP_COPY, s);
    if (gb_check(cudaGetLastError(), "k_soa_to_flash")) return GB_ERR_CUDA;
    return for_each_run(n, list, [&](int q0, int b0, int len) {
        return gb_check(cudaMemcpyAsync(host + (size_t)b0 * per, stage + (size_t)q0 * per,
                                        (size_t)len * per * sizeof(double), cudaMemcpyDeviceToHost, s),
                        "download") ? GB_ERR_CUDA : GB_OK;
    });
}

extern "C" int gb_grid_upload_flash_list(const double* unk_host, int nunk, const int* host_slot, int blockCount,
                                         const int* blockList_host, void* stream)
{
    return flash_copy_list(true, const_cast<double*>(unk_host), nunk, host_slot, blockCount, blockList_host, stream);
}

extern "C" int gb_grid_download_flash_list(double* unk_host, int nunk, const int* host_slot, int blockCount,
                                           const int* blockList_host, void* stream)
{
    return flash_copy_list(false, unk_host, nunk, host_slot, blockCount, blockList_host, stream);
}

// Interior transfers: the host arrays must be addressable by the device
// (pinned); the guard cells and guard faces of the host arrays stay as
// they are.
static int interior_prepare(const char* who, int n, const int* list, const int* host_slot, cudaStream_t s,
                            int** dslot, int** dlist)
{
    if (!g_gb.grid_ok) {
        gb_set_error("%s before gb_register_grid", who);
        return GB_ERR_NOT_INIT;
    }
    int rc = check_host_list(n, list, who);
    if (rc || n == 0) return rc;
    rc = gb_ensure_stage((GB_NROLE + (size_t)n) * sizeof(int));
    if (rc) return rc;
    *dslot = (int*)g_gb.d_stage;
    *dlist = *dslot + GB_NROLE;
    if (host_slot &&
        gb_check(cudaMemcpyAsync(*dslot, host_slot, GB_NROLE * sizeof(int), cudaMemcpyHostToDevice, s), "slot copy"))
        return GB_ERR_CUDA;
    return gb_check(cudaMemcpyAsync(*dlist, list, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s), "list copy")
               ? GB_ERR_CUDA
               : GB_OK;
}

static int flash_interior_list(bool up, double* host, int nunk, const int* host_slot, int n, const int* list,
                               void* stream)
{
    const char* who = up ? "gb_grid_upload_flash_interior_list" : "gb_grid_download_flash_interior_list";
    if (!host || !host_slot || nunk <= 0) return GB_ERR_ARG;
    double* hd = (double*)device_view(host);
    if (!hd) {
        gb_set_error("%s: the host array is not pinned", who);
        return GB_ERR_ARG;
    }
    const size_t smem = (size_t)FT * nunk * sizeof(double);
    if (smem > 48 * 1024) {
        gb_set_error("%s: nunk %d above the %d variables one tile holds", who, nunk, (int)(48 * 1024 / (FT * 8)));
        return GB_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int *dslot = nullptr, *dlist = nullptr;
    int rc = interior_prepare(who, n, list, host_slot, s, &dslot, &dlist);
    if (rc || n == 0) return rc;
    int mapped = 0;
    for (int r = 0; r < GB_NROLE; ++r)
        if (host_slot[r] >= 0 && host_slot[r] < nunk && g_gb.grid.slot[r] >= 0) ++mapped;
    const unsigned grid = (unsigned)(n * ITEMS_PER_BLOCK);
    gb_prof_begin(GBP_COPY, s);
    if (up) k_flash_interior<true><<<grid, FT, smem, s>>>(hd, nunk, dslot, g_gb.grid, dlist, n, 0);
    else k_flash_interior<false><<<grid, FT, smem, s>>>(hd, nunk, dslot, g_gb.grid, dlist, n, mapped < nunk);
    gb_prof_end(GBP_COPY, s);
    return gb_check(cudaGetLastError(), "k_flash_interior") ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_grid_upload_flash_interior_list(const double* unk_host, int nunk, const int* host_slot,
                                                  int blockCount, const int* blockList_host, void* stream)
{
    return flash_interior_list(true, const_cast<double*>(unk_host), nunk, host_slot, blockCount, blockList_host,
                               stream);
}

extern "C" int gb_grid_download_flash_interior_list(double* unk_host, int nunk, const int* host_slot,
                                                    int blockCount, const int* blockList_host, void* stream)
{
    return flash_interior_list(false, unk_host, nunk, host_slot, blockCount, blockList_host, stream);
}

static int faces_interior_list(bool up, double* const host[3], int n, const int* list, void* stream)
{
    const char* who = up ? "gb_grid_upload_faces_interior_list" : "gb_grid_download_faces_interior_list";
    if (!g_gb.grid_ok || !g_gb.grid.f[0] || !g_gb.grid.f[1] || !g_gb.grid.f[2]) {
        gb_set_error("%s: the registered grid has no face fields", who);
        return GB_ERR_NOT_INIT;
    }
    if (!host[0] || !host[1] || !host[2]) return GB_ERR_ARG;
    double* hv[3] = {(double*)device_view(host[0]), (double*)device_view(host[1]), (double*)device_view(host[2])};
    if (!hv[0] || !hv[1] || !hv[2]) {
        gb_set_error("%s: the host arrays are not pinned", who);
        return GB_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int *dslot = nullptr, *dlist = nullptr;
    int rc = interior_prepare(who, n, list, nullptr, s, &dslot, &dlist);
    if (rc || n == 0) return rc;
    const unsigned grid = (unsigned)(((int64_t)n * 3 * GB_NOWN + 255) / 256);
    gb_prof_begin(GBP_COPY, s);
    if (up) k_faces_interior<true><<<grid, 256, 0, s>>>(hv[0], hv[1], hv[2], g_gb.grid, dlist, n);
    else k_faces_interior<false><<<grid, 256, 0, s>>>(hv[0], hv[1], hv[2], g_gb.grid, dlist, n);
    gb_prof_end(GBP_COPY, s);
    return gb_check(cudaGetLastError(), "k_faces_interior") ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_grid_upload_faces_interior_list(const double* fx_host, const double* fy_host, const double* fz_host,
                                                  int blockCount, const int* blockList_host, void* stream)
{
    double* h[3] = {const_cast<double*>(fx_host), const_cast<double*>(fy_host), const_cast<double*>(fz_host)};
    return faces_interior_list(true, h, blockCount, blockList_host, stream);
}

extern "C" int gb_grid_download_faces_interior_list(double* fx_host, double* fy_host, double* fz_host,
                                                    int blockCount, const int* blockList_host, void* stream)
{
    double* h[3] = {fx_host, fy_host, fz_host};
    return faces_interior_list(false, h, blockCount, blockList_host, stream);
}

// Downloads run beside the compute kernels of later chunks: they are
// launched at the device's greatest priority, so the CTA scheduler hands
// them SM slots as compute CTAs retire instead of after the compute kernels
// queued before them (the priority is a launch attribute, kept by the
// graph's kernel nodes).
template <typename... P, typename... A>
static void launch_prio(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool prio, A... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributePriority;
    at[0].val.priority = g_io_priority;
    cfg.attrs = at;
    cfg.numAttrs = prio ? 1 : 0;
    cudaLaunchKernelEx(&cfg, k, args...);
}

// CTAs of a download running beside compute: enough rows in flight to
// keep the host link busy (about 190 GB/s device to host at a few
// microseconds of latency), few enough to leave the SMs to the compute
// kernels. Measured on the 4101-leaf host-resident step (256-block chunks):
// 128 CTAs 35.0 ms per step, 192 33.1 ms, 256 31.6 ms, 384 32.2 ms.
constexpr int g_io_ctas = 256;

static void launch_io(bool up, const host_io_dev& io, int nblk, const int* list, cudaStream_t s)
{
    const size_t smem = (size_t)FT * io.nunk * sizeof(double);
    const int items = nblk * ITEMS_PER_BLOCK;
    const int64_t faces = (int64_t)nblk * 3 * GB_NOWN;
    if (up) {
        launch_prio(k_flash_interior<true>, dim3(items), dim3(FT), smem, s, false, io.unk, io.nunk,
                    (const int*)io.dslot, g_gb.grid, list, nblk, 0);
        if (io.f[0])
            launch_prio(k_faces_interior<true>, dim3((unsigned)((faces + 255) / 256)), dim3(256), 0, s, false,
                        io.f[0], io.f[1], io.f[2], g_gb.grid, list, nblk);
        return;
    }
    launch_prio(k_flash_interior<false>, dim3(std::min(items, g_io_ctas)), dim3(FT), smem, s, true, io.unk,
                io.nunk, (const int*)io.dslot, g_gb.grid, list, nblk, io.read_first);
    if (io.f[0])
        launch_prio(k_faces_interior<false>, dim3((unsigned)std::min<int64_t>((faces + 255) / 256, g_io_ctas / 4)),
                    dim3(256), 0, s, true, io.f[0], io.f[1], io.f[2], g_gb.grid, list, nblk);
}

static int face_copy_list(bool up, double* const host[3], int n, const int* list, void* stream)
{
    if (!g_gb.grid_ok || !g_gb.grid.f[0] || !g_gb.grid.f[1] || !g_gb.grid.f[2]) {
        gb_set_error("face transfer: the registered grid has no face fields");
        return GB_ERR_NOT_INIT;
    }
    if (!host[0] || !host[1] || !host[2]) return GB_ERR_ARG;
    int rc = check_host_list(n, list, up ? "gb_grid_upload_faces_list" : "gb_grid_download_faces_list");
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (n == 0) return GB_OK;
    double* hv[3] = {(double*)device_view(host[0]), (double*)device_view(host[1]), (double*)device_view(host[2])};
    if (hv[0] && hv[1] && hv[2]) {
        rc = gb_ensure_stage((size_t)n * sizeof(int) + 16);
        if (rc) return rc;
        int* dlist = (int*)g_gb.d_stage;
        if (gb_check(cudaMemcpyAsync(dlist, list, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s), "list copy"))
            return GB_ERR_CUDA;
        dim3 grid((GB_FSZ + 255) / 256, n, 3);
        if (up) k_faces_direct<true><<<grid, 256, 0, s>>>(hv[0], hv[1], hv[2], g_gb.grid, dlist);
        else k_faces_direct<false><<<grid, 256, 0, s>>>(hv[0], hv[1], hv[2], g_gb.grid, dlist);
        return gb_check(cudaGetLastError(), "k_faces_direct") ? GB_ERR_CUDA : GB_OK;
    }
    for (int a = 0; a < 3; ++a) {
        double* dev = g_gb.grid.f[a];
        double* h = host[a];
        rc = for_each_run(n, list, [&](int, int b0, int len) {
            const size_t off = (size_t)b0 * GB_FSZ, cnt = (size_t)len * GB_FSZ * sizeof(double);
            return gb_check(up ? cudaMemcpyAsync(dev + off, h + off, cnt, cudaMemcpyHostToDevice, s)
                               : cudaMemcpyAsync(h + off, dev + off, cnt, cudaMemcpyDeviceToHost, s),
                            up ? "face upload" : "face download") ? GB_ERR_CUDA : GB_OK;
        });
        if (rc) return rc;
    }
    return GB_OK;
}

extern "C" int gb_grid_upload_faces_list(const double* fx_host, const double* fy_host, const double* fz_host,
                                         int blockCount, const int* blockList_host, void* stream)
{
    double* h[3] = {const_cast<double*>(fx_host), const_cast<double*>(fy_host), const_cast<double*>(fz_host)};
    return face_copy_list(true, h, blockCount, blockList_host, stream);
}

extern "C" int gb_grid_download_faces_list(double* fx_host, double* fy_host, double* fz_host, int blockCount,
                                           const int* blockList_host, void* stream)
{
    double* h[3] = {fx_host, fy_host, fz_host};
    return face_copy_list(false, h, blockCount, blockList_host, stream);
}
