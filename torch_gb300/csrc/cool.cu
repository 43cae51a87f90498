// Heating/cooling source term: table set-up and per-cell kernels.
// Compiled with -fmad=false (see cool_dev.cuh).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "cool_dev.cuh"
#include "gb_prof.h"
#include "gb_state.h"

using namespace gbcool;

namespace {

// Read cool.dat in FLASH's format (get_cooling_data.F90:20-55) or the
// compact int32 form ("GBCOOL01"). Values are log10 in units of 1e-4.
int read_table(const char* path, std::vector<int>& logT, std::vector<int>& logn,
               std::vector<int>& logL)
{
    FILE* f = fopen(path, "rb");
    if (!f) {
        gb_set_error("cannot open cooling table %s", path);
        return GB_ERR_TABLE;
    }
    char magic[8];
    size_t got = fread(magic, 1, 8, f);
    logT.assign(GB_TEMP_PTS, 0);
    logn.assign(GB_DENS_PTS, 0);
    logL.assign(GB_TEMP_PTS * GB_DENS_PTS, 0);
    if (got == 8 && memcmp(magic, "GBCOOL01", 8) == 0) {
        int dims[2];
        if (fread(dims, sizeof(int), 2, f) != 2 || dims[0] != GB_TEMP_PTS || dims[1] != GB_DENS_PTS ||
            fread(logT.data(), sizeof(int), GB_TEMP_PTS, f) != GB_TEMP_PTS ||
            fread(logn.data(), sizeof(int), GB_DENS_PTS, f) != GB_DENS_PTS ||
            fread(logL.data(), sizeof(int), logL.size(), f) != logL.size()) {
            fclose(f);
            gb_set_error("malformed compact cooling table %s", path);
            return GB_ERR_TABLE;
        }
        fclose(f);
        return GB_OK;
    }
    // FLASH text format
    rewind(f);
    char line[256];
    int nt = 0, nd = 0;
    if (!fgets(line, sizeof line, f) || sscanf(line, "%d %d", &nt, &nd) != 2 ||
        nt != GB_TEMP_PTS || nd != GB_DENS_PTS) {
        fclose(f);
        gb_set_error("wrong number of data points in %s", path);
        return GB_ERR_TABLE;
    }
    for (int j = 0; j < GB_TEMP_PTS; ++j)
        for (int i = 0; i < GB_DENS_PTS; ++i) {
            if (!fgets(line, sizeof line, f) || strlen(line) < 60) {
                fclose(f);
                gb_set_error("read error in %s at record %d", path, j * GB_DENS_PTS + i + 1);
                return GB_ERR_TABLE;
            }
            int v[6];
            for (int c = 0; c < 6; ++c) {
                char fld[11];
                memcpy(fld, line + 10 * c, 10);
                fld[10] = 0;
                char* end = nullptr;
                double x = strtod(fld, &end);
                if (end == fld) {
                    fclose(f);
                    gb_set_error("read error in %s at record %d", path, j * GB_DENS_PTS + i + 1);
                    return GB_ERR_TABLE;
                }
                v[c] = (int)lround(x * 1e4);
            }
            if (i == 0) logT[j] = v[0];
            if (j == 0) logn[i] = v[1];
            logL[i + GB_DENS_PTS * j] = v[5];
        }
    fclose(f);
    return GB_OK;
}

__device__ __forceinline__ bool finite_pos(double x) { return gb_finite_pos(x); }

// RadHeat.F90:223-423 for one cell of a registered grid.
__global__ void k_heat_blocks(gb_dev_grid g, gb_cool_ctx c, const int* __restrict__ list,
                              double dt, double gamma, gb_status* st)
{
    const int blk = list[blockIdx.y];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= GB_NXB * GB_NXB * GB_NXB) return;
    const int i = GB_NGUARD + t % GB_NXB, j = GB_NGUARD + (t / GB_NXB) % GB_NXB,
              k = GB_NGUARD + t / (GB_NXB * GB_NXB);
    const int ci = gb_cidx(i, j, k);
    const gb_cool_params& p = c.p;
    double rho_c = gb_var(g, blk, GB_DENS)[ci];
    double ei_c = gb_var(g, blk, GB_EINT)[ci];
    double temp = gb_var(g, blk, GB_TEMP)[ci];
    double vx = gb_var(g, blk, GB_VELX)[ci], vy = gb_var(g, blk, GB_VELY)[ci],
           vz = gb_var(g, blk, GB_VELZ)[ci];
    gb_cool_vars v;
    v.rho = rho_c * p.dens_unit;
    double ei = ei_c * (p.vel_unit * p.vel_unit);
    v.tdust = gb_var(g, blk, GB_TDUS)[ci];
    v.xHp = g.slot[GB_IHP] >= 0 ? gb_var(g, blk, GB_IHP)[ci] : p.xHp_const;
    double ek = 0.5e0 * (vx * vx + vy * vy + vz * vz);
    v.ephen = g.slot[GB_PHHE] >= 0 ? gb_var(g, blk, GB_PHHE)[ci] : 0.0;
    v.ephen = v.ephen / v.rho;
    v.Gflux = g.slot[GB_PEFL] >= 0 ? gb_var(g, blk, GB_PEFL)[ci] : 0.0;
    v.mu_mol = p.mu_mol;
    v.strat_factor = 1.0;
    gb_cool_diag d = {0, 0, 0, 0, 0};
    if (!(finite_pos(v.rho) && finite_pos(ei) && finite_pos(temp))) {
        gb_fail(st, GB_ST_NONFINITE, blk, i, j, k, temp);
        return;
    }
    heating_and_cooling(c, v, &ei, dt * p.time_unit, &temp, &d);
    bool clamped = false;
    if (temp > p.absTmax) {
        ei = p.absTmax * v.TtoEI;
        temp = p.absTmax;
        clamped = true;
    }
    if (ei < p.smallp / v.rho) ei = p.smallp / v.rho;
    double ei_out = ei / (p.vel_unit * p.vel_unit);
    gb_var(g, blk, GB_ENER)[ci] = ei_out + ek;
    gb_var(g, blk, GB_EINT)[ci] = ei_out;
    gb_var(g, blk, GB_TEMP)[ci] = temp;
    gb_var(g, blk, GB_TDUS)[ci] = v.tdust;
    gb_var(g, blk, GB_PRES)[ci] = (gamma - 1.0) * rho_c * ei_out;
    if (g.slot[GB_PHHE] >= 0) gb_var(g, blk, GB_PHHE)[ci] = 0.0;
    if (g.slot[GB_PEFL] >= 0) gb_var(g, blk, GB_PEFL)[ci] = 0.0;
    if (st) {
        gb_count_warp(&st->n_bracket_fail, d.bracket_fail != 0);
        gb_count_warp(&st->n_dust_noconv, d.dust_noconv != 0);
        gb_count_warp(&st->n_clamped, clamped);
        if (clamped) gb_fail(st, GB_ST_OVERHEAT, blk, i, j, k, temp);
        if (d.unbracketed) gb_fail(st, GB_ST_ZERO_UNBRACKETED, blk, i, j, k, ei);
        if (d.maxiter) gb_fail(st, GB_ST_ZERO_MAXITER, blk, i, j, k, ei);
    }
}

// The same per-cell solve on plain CGS arrays (FORM: the rate formulation,
// as heating_and_cooling's template argument).
template <int FORM>
__global__ void k_cool_cells(gb_cool_ctx c, int64_t n, const double* __restrict__ dens,
                             double* ei_a, double* temp_a, double* tdust_a,
                             const double* __restrict__ xhp, const double* __restrict__ phhe,
                             const double* __restrict__ gflux, double dt, gb_status* st)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    gb_cool_vars v;
    v.rho = dens[idx];
    double ei = ei_a[idx], temp = temp_a[idx];
    v.tdust = tdust_a[idx];
    v.xHp = xhp ? xhp[idx] : c.p.xHp_const;
    v.ephen = (phhe ? phhe[idx] : 0.0) / v.rho;
    v.Gflux = gflux ? gflux[idx] : 0.0;
    v.mu_mol = c.p.mu_mol;
    v.strat_factor = 1.0;
    gb_cool_diag d = {0, 0, 0, 0, 0};
    if (!(finite_pos(v.rho) && finite_pos(ei) && finite_pos(temp))) {
        gb_fail(st, GB_ST_NONFINITE, -1, (int)(idx & 0x7fffffff), 0, 0, temp);
        return;
    }
    heating_and_cooling<FORM>(c, v, &ei, dt, &temp, &d);
    bool clamped = false;
    if (temp > c.p.absTmax) {
        ei = c.p.absTmax * v.TtoEI;
        temp = c.p.absTmax;
        clamped = true;
    }
    if (ei < c.p.smallp / v.rho) ei = c.p.smallp / v.rho;
    ei_a[idx] = ei;
    temp_a[idx] = temp;
    tdust_a[idx] = v.tdust;
    if (st) {
        gb_count_warp(&st->n_bracket_fail, d.bracket_fail != 0);
        gb_count_warp(&st->n_dust_noconv, d.dust_noconv != 0);
        gb_count_warp(&st->n_clamped, clamped);
        if (d.unbracketed) gb_fail(st, GB_ST_ZERO_UNBRACKETED, -1, (int)(idx & 0x7fffffff), 0, 0, ei);
        if (d.maxiter) gb_fail(st, GB_ST_ZERO_MAXITER, -1, (int)(idx & 0x7fffffff), 0, 0, ei);
    }
}

}  // namespace

static double g_brent_tol_K = 1.0;
static int g_rate_form = 0;

namespace {
gb_cool_pf make_pf(const gb_cool_params& p);
}

extern "C" int gb_set_rate_form(int form)
{
    if (form < 0 || form > 2) {
        gb_set_error("gb_set_rate_form: form %d is not 0, 1 or 2", form);
        return GB_ERR_ARG;
    }
    g_rate_form = form;
    return GB_OK;
}

extern "C" int gb_set_brent_tolerance(double kelvin)
{
    if (!(kelvin > 0.0) || !(kelvin <= 1e6)) {
        gb_set_error("gb_set_brent_tolerance: tolerance %g K outside (0, 1e6]", kelvin);
        return GB_ERR_ARG;
    }
    g_brent_tol_K = kelvin;
    g_gb.cool.brent_tol_K = kelvin;
    g_gb.gen += 1;
    return GB_OK;
}

extern "C" int gb_cool_init(const char* path, const gb_cool_params* p)
{
    if (!path || !p) {
        gb_set_error("gb_cool_init: null argument");
        return GB_ERR_ARG;
    }
    std::vector<int> lt, ln, ll;
    int rc = read_table(path, lt, ln, ll);
    if (rc != GB_OK) return rc;
    // 10.e0**x on the host, as get_cooling_data computes it
    const size_t ntab = GB_TEMP_PTS + GB_DENS_PTS + (size_t)GB_TEMP_PTS * GB_DENS_PTS;
    std::vector<double> h(ntab);
    for (int j = 0; j < GB_TEMP_PTS; ++j) h[j] = pow(10.e0, (double)lt[j] / 10000.0);
    for (int i = 0; i < GB_DENS_PTS; ++i) h[GB_TEMP_PTS + i] = pow(10.e0, (double)ln[i] / 10000.0);
    for (size_t q = 0; q < ll.size(); ++q)
        h[GB_TEMP_PTS + GB_DENS_PTS + q] = pow(10.e0, (double)ll[q] / 10000.0);
    // FP32 copies: axes, and the molecular power per gram cool_dat / (mu_mol m_p)
    std::vector<float> hf(ntab);
    for (size_t q = 0; q < GB_TEMP_PTS + GB_DENS_PTS; ++q) hf[q] = (float)h[q];
    for (size_t q = GB_TEMP_PTS + GB_DENS_PTS; q < ntab; ++q) hf[q] = (float)(h[q] / (p->mu_mol * p->mp));
    if (!g_gb.d_table) {
        if (gb_check(cudaMalloc(&g_gb.d_table, ntab * (sizeof(double) + sizeof(float))), "cudaMalloc(table)"))
            return GB_ERR_CUDA;
    }
    float* d_tabf = (float*)(g_gb.d_table + ntab);
    if (gb_check(cudaMemcpy(g_gb.d_table, h.data(), ntab * sizeof(double), cudaMemcpyHostToDevice),
                 "cudaMemcpy(table)") ||
        gb_check(cudaMemcpy(d_tabf, hf.data(), ntab * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy(table f32)"))
        return GB_ERR_CUDA;
    g_gb.cool.Tf = d_tabf;
    g_gb.cool.nf = d_tabf + GB_TEMP_PTS;
    g_gb.cool.lamf = d_tabf + GB_TEMP_PTS + GB_DENS_PTS;
    g_gb.cool.p = *p;
    g_gb.cool.pf = make_pf(*p);
    g_gb.cool.T = g_gb.d_table;
    g_gb.cool.n = g_gb.d_table + GB_TEMP_PTS;
    g_gb.cool.lam = g_gb.d_table + GB_TEMP_PTS + GB_DENS_PTS;
    g_gb.cool.brent_tol_K = g_brent_tol_K;
    g_gb.cool.T_min = h[0];
    g_gb.cool.nd_min = h[GB_TEMP_PTS];
    g_gb.cool_ok = true;
    g_gb.gen += 1;
    return GB_OK;
}

int gb_launch_cool_blocks(int nblk, const int* list, double dt, gb_status* st, cudaStream_t s)
{
    dim3 grid((GB_NXB * GB_NXB * GB_NXB + 127) / 128, nblk);
    gb_prof_begin(GBP_HEAT, s);
    k_heat_blocks<<<grid, 128, 0, s>>>(g_gb.grid, g_gb.cool, list, dt, g_gb.hp.gamma, st);
    gb_prof_end(GBP_HEAT, s);
    return gb_check(cudaGetLastError(), "k_heat_blocks") ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_heat(int blockCount, const int* list, double dt, double time, gb_status* st,
                       void* stream)
{
    (void)time;
    if (!g_gb.cool_ok || !g_gb.grid_ok) {
        gb_set_error("gb_heat: call gb_cool_init and gb_register_grid first");
        return GB_ERR_NOT_INIT;
    }
    if (blockCount < 0 || (blockCount > 0 && !list)) return GB_ERR_ARG;
    if (g_gb.grid.slot[GB_TEMP] < 0 || g_gb.grid.slot[GB_TDUS] < 0 || g_gb.grid.slot[GB_EINT] < 0) {
        gb_set_error("gb_heat: grid lacks TEMP/TDUS/EINT slots");
        return GB_ERR_ARG;
    }
    if (blockCount == 0) return GB_OK;
    return gb_launch_cool_blocks(blockCount, list, dt, st, (cudaStream_t)stream);
}

extern "C" int gb_cool_cells(int64_t n, const double* dens, double* ei, double* temp, double* tdust,
                             const double* xhp, const double* phhe, const double* gflux, double dt,
                             gb_status* st, void* stream)
{
    if (!g_gb.cool_ok) {
        gb_set_error("gb_cool_cells: call gb_cool_init first");
        return GB_ERR_NOT_INIT;
    }
    if (n < 0 || (n > 0 && (!dens || !ei || !temp || !tdust))) return GB_ERR_ARG;
    if (n == 0) return GB_OK;
    int tpb = 128;
    int64_t nb = (n + tpb - 1) / tpb;
    if (g_rate_form == 2)
        k_cool_cells<2><<<(unsigned)nb, tpb, 0, (cudaStream_t)stream>>>(g_gb.cool, n, dens, ei, temp, tdust, xhp,
                                                                     phhe, gflux, dt, st);
    else if (g_rate_form == 1)
        k_cool_cells<1><<<(unsigned)nb, tpb, 0, (cudaStream_t)stream>>>(g_gb.cool, n, dens, ei, temp, tdust, xhp,
                                                                     phhe, gflux, dt, st);
    else
        k_cool_cells<0><<<(unsigned)nb, tpb, 0, (cudaStream_t)stream>>>(g_gb.cool, n, dens, ei, temp, tdust, xhp,
                                                                     phhe, gflux, dt, st);
    return gb_check(cudaGetLastError(), "k_cool_cells") ? GB_ERR_CUDA : GB_OK;
}

// ---------------------------------------------------------------- surrogate
#include "cool_f32.cuh"
#include "mlp.h"
#include "sur_common.cuh"
#include "sur_dev.cuh"

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double uni(uint64_t seed, int64_t i, int k)
{
    uint64_t z = mix64(seed + 0x9E3779B97F4A7C15ULL * (uint64_t)(4 * i + k + 1));
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// t_cool and the plain integrator's solution for one training sample
__global__ void k_sur_samples(gb_cool_ctx c, int64_t n, uint64_t seed, float* __restrict__ feat,
                              float* __restrict__ target, gb_status* st)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double lnn = -2.0 + 8.0 * uni(seed, i, 0), lT = 1.0 + 7.0 * uni(seed, i, 1),
                 lr = -3.0 + 6.0 * uni(seed, i, 2), lG = -1.0 + 2.0 * uni(seed, i, 3);
    const double nden = pow(10.0, lnn), T0 = pow(10.0, lT), G = pow(10.0, lG);
    gb_cool_ctx cc = c;
    cc.p.Gzero = G;
    const gb_cool_params& p = cc.p;
    const double TtoEI = p.boltz / ((5.0 / 3.0 - 1.0) * p.eos_abar * p.mp);
    gb_cool_vars v;
    v.rho = nden * p.mu_mol * p.mp;
    v.tdust = 15.0;
    v.xHp = p.xHp_const;
    v.ephen = 0.0;
    v.Gflux = 0.0;
    v.mu_mol = p.mu_mol;
    v.strat_factor = 1.0;
    double ei = T0 * TtoEI, temp = T0;
    v.ndens = v.rho / (v.mu_mol * p.mp);
    v.TtoEI = ei / temp;
    v.conf = v.ndens * v.ndens / v.rho;
    double gam, lam;
    double f0 = dei_parts(cc, v, cooling_floor(cc, v), ei, &gam, &lam);
    double tcool = ei / fmax(fabs(f0), 1e-300);
    double dt = pow(10.0, lr) * tcool;
    gb_cool_diag d = {0, 0, 0, 0, 0};
    heating_and_cooling(cc, v, &ei, dt, &temp, &d);
    if (temp > p.absTmax) temp = p.absTmax;
    float x[4];
    gbsur::features(nden, T0, dt / tcool, gam, lam, x);
    reinterpret_cast<float4*>(feat)[i] = make_float4(x[0], x[1], x[2], x[3]);
    bool bad = d.unbracketed || d.maxiter || !isfinite(temp) || !(temp > 0.0);
    target[i] = bad ? __int_as_float(0x7fc00000) : (float)((log10(temp) - lT) / gbsur::Y_SCALE);
    if (st) gb_count_warp(&st->n_bracket_fail, d.bracket_fail != 0);
}

struct sur_cell {
    double rho, ei, temp, TtoEI;
};

// state of one interior cell after the hydro update, in CGS
__device__ __forceinline__ void sur_load(const gb_dev_grid& g, const gb_cool_ctx& c, double gamma, int blk, int ci,
                                         gb_cool_vars& v, double& ei, double& temp)
{
    const gb_cool_params& p = c.p;
    v.rho = gb_var(g, blk, GB_DENS)[ci] * p.dens_unit;
    ei = gb_var(g, blk, GB_EINT)[ci] * (p.vel_unit * p.vel_unit);
    temp = ei * ((gamma - 1.0) * p.eos_abar * p.mp / p.boltz);
    v.tdust = gb_var(g, blk, GB_TDUS)[ci];
    v.xHp = g.slot[GB_IHP] >= 0 ? gb_var(g, blk, GB_IHP)[ci] : p.xHp_const;
    v.ephen = g.slot[GB_PHHE] >= 0 ? gb_var(g, blk, GB_PHHE)[ci] / v.rho : 0.0;
    v.Gflux = g.slot[GB_PEFL] >= 0 ? gb_var(g, blk, GB_PEFL)[ci] : 0.0;
    v.mu_mol = p.mu_mol;
    v.strat_factor = 1.0;
    v.ndens = v.rho / (v.mu_mol * p.mp);
    v.TtoEI = ei / temp;
    v.conf = v.ndens * v.ndens / v.rho;
}

__device__ __forceinline__ void sur_store(const gb_dev_grid& g, const gb_cool_ctx& c, double gamma, int blk, int ci,
                                          const gb_cool_vars& v, double ei, double temp)
{
    const gb_cool_params& p = c.p;
    if (ei < p.smallp / v.rho) ei = p.smallp / v.rho;
    double vx = gb_var(g, blk, GB_VELX)[ci], vy = gb_var(g, blk, GB_VELY)[ci], vz = gb_var(g, blk, GB_VELZ)[ci];
    double e = ei / (p.vel_unit * p.vel_unit);
    double rho = gb_var(g, blk, GB_DENS)[ci];
    gb_var(g, blk, GB_EINT)[ci] = e;
    gb_var(g, blk, GB_ENER)[ci] = e + 0.5 * (vx * vx + vy * vy + vz * vz);
    gb_var(g, blk, GB_PRES)[ci] = (gamma - 1.0) * rho * e;
    gb_var(g, blk, GB_TEMP)[ci] = temp;
    gb_var(g, blk, GB_TDUS)[ci] = v.tdust;
    if (g.slot[GB_PHHE] >= 0) gb_var(g, blk, GB_PHHE)[ci] = 0.0;
    if (g.slot[GB_PEFL] >= 0) gb_var(g, blk, GB_PEFL)[ci] = 0.0;
}

__device__ __forceinline__ void sur_load_fast(const gb_dev_grid& g, const gb_cool_ctx& c, const sur_units& u, int blk,
                                              int ci, gb_cool_vars& v, double& ei, double& temp)
{
    const gb_cool_params& p = c.p;
    v.rho = gb_var(g, blk, GB_DENS)[ci] * p.dens_unit;
    ei = gb_var(g, blk, GB_EINT)[ci] * u.vel2;
    temp = ei * u.T_of_e;
    v.tdust = gb_var(g, blk, GB_TDUS)[ci];
    v.xHp = g.slot[GB_IHP] >= 0 ? gb_var(g, blk, GB_IHP)[ci] : p.xHp_const;
    v.ephen = g.slot[GB_PHHE] >= 0 ? gb_var(g, blk, GB_PHHE)[ci] / v.rho : 0.0;
    v.Gflux = g.slot[GB_PEFL] >= 0 ? gb_var(g, blk, GB_PEFL)[ci] : 0.0;
    v.mu_mol = p.mu_mol;
    v.strat_factor = 1.0;
    v.ndens = v.rho * u.inv_mu_mp;
    v.TtoEI = u.e_of_T;
    v.conf = v.ndens * u.inv_mu_mp;  // ndens^2 / rho
}

__device__ __forceinline__ void sur_store_fast(const gb_dev_grid& g, const gb_cool_ctx& c, const sur_units& u,
                                               double gamma, int blk, int ci, const gb_cool_vars& v, double ei,
                                               double temp)
{
    const gb_cool_params& p = c.p;
    if (ei * v.rho < p.smallp) ei = p.smallp / v.rho;
    double vx = gb_var(g, blk, GB_VELX)[ci], vy = gb_var(g, blk, GB_VELY)[ci], vz = gb_var(g, blk, GB_VELZ)[ci];
    double e = ei * u.inv_vel2;
    double rho = gb_var(g, blk, GB_DENS)[ci];
    gb_var(g, blk, GB_EINT)[ci] = e;
    gb_var(g, blk, GB_ENER)[ci] = e + 0.5 * (vx * vx + vy * vy + vz * vz);
    gb_var(g, blk, GB_PRES)[ci] = (gamma - 1.0) * rho * e;
    gb_var(g, blk, GB_TEMP)[ci] = temp;
    gb_var(g, blk, GB_TDUS)[ci] = v.tdust;
    if (g.slot[GB_PHHE] >= 0) gb_var(g, blk, GB_PHHE)[ci] = 0.0;
    if (g.slot[GB_PEFL] >= 0) gb_var(g, blk, GB_PEFL)[ci] = 0.0;
}

// the accepted state of one cell: the FP64 update of the internal energy
// and what follows from it (total energy, pressure, temperature); the
// energy floor is tested in FP32 and taken in FP64 when it applies. The
// dust temperature is written only when it changed (new_tdust).
__device__ __forceinline__ void sur_store_f32(const gb_dev_grid& g, const sur_units& u, double gamma, int blk, int ci,
                                              float rhof, bool new_tdust, float tdust, double ei, double temp)
{
    double rho = gb_var(g, blk, GB_DENS)[ci];
    if (gb_d2f(ei) * rhof < u.smallp_f) ei = u.smallp / (rho * u.dens_unit);
    double vx = gb_var(g, blk, GB_VELX)[ci], vy = gb_var(g, blk, GB_VELY)[ci], vz = gb_var(g, blk, GB_VELZ)[ci];
    double e = ei * u.inv_vel2;
    gb_var(g, blk, GB_EINT)[ci] = e;
    gb_var(g, blk, GB_ENER)[ci] = e + 0.5 * (vx * vx + vy * vy + vz * vz);
    gb_var(g, blk, GB_PRES)[ci] = (gamma - 1.0) * rho * e;
    gb_var(g, blk, GB_TEMP)[ci] = temp;
    if (new_tdust) gb_var(g, blk, GB_TDUS)[ci] = gb_f2d(tdust);
    if (g.slot[GB_PHHE] >= 0) gb_var(g, blk, GB_PHHE)[ci] = 0.0;
    if (g.slot[GB_PEFL] >= 0) gb_var(g, blk, GB_PEFL)[ci] = 0.0;
}

__device__ __forceinline__ void cell_of(int64_t idx, const int* list, int& blk, int& ci, int& i, int& j, int& k)
{
    int cb = (int)(idx / 4096), t = (int)(idx % 4096);
    blk = list[cb];
    i = GB_NGUARD + t % GB_NXB;
    j = GB_NGUARD + (t / GB_NXB) % GB_NXB;
    k = GB_NGUARD + t / (GB_NXB * GB_NXB);
    ci = gb_cidx(i, j, k);
}

// features + the rate at the old state
__global__ void k_sur_feat(gb_dev_grid g, gb_cool_ctx c, gb_cool_pf pf, sur_units un, const int* __restrict__ list,
                           int64_t ncell, double dt_code, const double* __restrict__ dtp, float* __restrict__ feat,
                           float2* __restrict__ f0out)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncell) return;
    if (dtp) dt_code = *dtp;
    int blk, ci, i, j, k;
    cell_of(idx, list, blk, ci, i, j, k);
    gb_cool_varsf vf;
    double ei;
    float eif, tempf;
    sur_load_f32(g, pf, un, blk, ci, vf, ei, eif, tempf);
    float4 x;
    float2 f0fl;
    sur_features(c, pf, un, vf, eif, tempf, dt_code, x, f0fl);
    reinterpret_cast<float4*>(feat)[idx] = x;
    f0out[idx] = f0fl;
}

// acceptance test: starting from the network's prediction, at most four
// secant-Newton iterations on the backward-Euler residual
//   g(e) = e - dt f(e) - e_old   (heatCool.F90:1928-1950),
// the slope taken through the last two rate evaluations (the first pair is
// the old state, whose rate the feature kernel kept). A cell is accepted
// once a Newton correction below rel_tol of e was computed from a local
// slope (its two points within 5 % of each other) and the energy moved
// the way the rate at the old state points; otherwise it goes to the
// fallback list and the plain integrator solves it.
// eight resident CTAs per SM (64 registers, no spills; seven with the FP64
// re-check, which would spill at eight): the kernel waits on memory and on
// the rate evaluations' MUFU results, and more warps hide that
template <bool CHECK64>
__global__ void __launch_bounds__(128, CHECK64 ? 7 : 8) k_sur_accept(gb_dev_grid g, gb_cool_ctx c, gb_cool_pf pf, sur_units un, double gamma,
                             const int* __restrict__ list, int64_t ncell, double dt_code, const double* __restrict__ dtp,
                             const float* __restrict__ y, const float2* __restrict__ f0a, double rel_tol,
                             int* __restrict__ rej, int* __restrict__ nrej, gb_status* st)
{
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncell) return;
    if (dtp) dt_code = *dtp;
    int blk, ci, i, j, k;
    cell_of(idx, list, blk, ci, i, j, k);
    const gb_cool_params& p = c.p;
    gb_cool_varsf vf;
    double ei0;
    float e0f, temp0f;
    sur_load_f32(g, pf, un, blk, ci, vf, ei0, e0f, temp0f);
    const gb_cool_tabf tf = {c.Tf, c.nf, c.lamf, un.T_min_f, un.nd_min_f};
    const float dtf = gb_d2f(dt_code) * un.time_unit_f;
    const float rtol = (float)rel_tol;
    const float2 f0fl = f0a[idx];
    const float f0 = f0fl.x;
    const float flf = f0fl.y;
    const float Tp = temp0f * exp10f((float)gbsur::Y_SCALE * y[idx]);
    bool ok = isfinite(Tp) && Tp > 0.0f;
    double ein = 0.0;
    float xfin = 0.0f;
    if (ok) {
        // secant-Newton from the prediction, in FP32 on the change of the
        // energy x = e - e_old (the backward-Euler residual is then
        // g = x - dt f, with no cancellation against e_old); e is formed in
        // FP64 once at the end
        const float xmin = un.emin_f - e0f;
        float xa = 0.0f, fa = f0;
        float xb = fmaxf(Tp * un.e_of_T_f, un.emin_f) - e0f;
        float J = 1.0f;
        bool conv = false;
        for (int it = 0; it < 4; ++it) {
            float gm, lm;
            const float eb_f = e0f + xb;
            const float fb = gbcoolf::dei_parts(pf, tf, vf, flf, eb_f, &gm, &lm);
            const float gb = xb - dtf * fb;
            const float de = xb - xa;
            const float slope = fabsf(de) > 1e-7f * eb_f ? (fb - fa) / de : 0.0f;
            J = 1.0f - dtf * slope;
            if (!(J > 0.0f)) break;
            float xn = xb - gb / J;
            if (!isfinite(xn)) break;
            if (xn < xmin) xn = xmin;
            xa = xb;
            fa = fb;
            xb = xn;
            // the correction is small and the secant slope local (its two
            // points within 5 % of each other)
            if (fabsf(xb - xa) <= 0.25f * rtol * (e0f + xb) && fabsf(de) <= 0.05f * (e0f + xa)) {
                conv = true;
                break;
            }
        }
        const double eb = ei0 + gb_f2d(xb);
        xfin = xb;
        // the converged FP32 iterate is the answer; optionally re-check the
        // backward-Euler residual (heatCool.F90:1928-1950) in FP64 with the
        // last secant slope
        if (conv && CHECK64) {
            gb_cool_vars v;
            double e64, t64;
            sur_load_fast(g, c, un, blk, ci, v, e64, t64);
            const double dt = dt_code * p.time_unit;
            double f64 = dei_dt(c, v, cooling_floor(c, v), eb);
            double g64 = eb - dt * f64 - ei0;
            double delta = g64 / (double)J;
            ein = eb - delta;
            xfin = gb_d2f(ein - ei0);
            ok = isfinite(ein) && ein > 0.0 && fabs(delta) <= rel_tol * ein;
        } else {
            ein = eb;
            ok = conv && isfinite(xb) && e0f + xb > 0.0f;
        }
        // the solution moves the way the rate at the old state points
        if (ok && f0 < 0.0f && xfin > e0f * rtol) ok = false;
        if (ok && f0 > 0.0f && xfin < -e0f * rtol) ok = false;
    }
    if (ok) {
        double temp = ein * un.T_of_e;
        float tempf = gb_d2f(temp);
        if (tempf < un.absTmin_f) {
            temp = p.absTmin;
            tempf = un.absTmin_f;
            ein = p.absTmin * un.e_of_T;
        }
        const bool dust = p.useDustCool && tempf <= un.dust_sputter_f;
        const float tdust = dust ? gbcoolf::dust_temperature(pf, vf, tempf, vf.tdust) : 0.0f;
        if (tempf > un.absTmax_f) {
            ein = p.absTmax * un.e_of_T;
            temp = p.absTmax;
        }
        sur_store_f32(g, un, gamma, blk, ci, vf.rho, dust, tdust, ein, temp);
    } else {
        int slot = atomicAdd(nrej, 1);
        rej[slot] = (int)idx;
    }
    if (st) {
        gb_count_warp(&st->n_surrogate, ok);
        gb_count_warp(&st->n_surrogate_reject, !ok);
    }
}

// rejected cells: the plain implicit integrator (RadHeat.F90:223-423)
__device__ void sur_fallback_cell(const gb_dev_grid& g, const gb_cool_ctx& c, double gamma, const int* __restrict__ list,
                                  double dt_code, int64_t idx, gb_status* st)
{
    int blk, ci, i, j, k;
    cell_of(idx, list, blk, ci, i, j, k);
    gb_cool_vars v;
    double ei, temp;
    sur_load(g, c, gamma, blk, ci, v, ei, temp);
    gb_cool_diag d = {0, 0, 0, 0, 0};
    if (!(finite_pos(v.rho) && finite_pos(ei) && finite_pos(temp))) {
        gb_fail(st, GB_ST_NONFINITE, blk, i, j, k, temp);
        return;
    }
    heating_and_cooling(c, v, &ei, dt_code * c.p.time_unit, &temp, &d);
    bool clamped = false;
    if (temp > c.p.absTmax) {
        ei = c.p.absTmax * v.TtoEI;
        temp = c.p.absTmax;
        clamped = true;
    }
    sur_store(g, c, gamma, blk, ci, v, ei, temp);
    if (st) {
        gb_count_warp(&st->n_bracket_fail, d.bracket_fail != 0);
        gb_count_warp(&st->n_clamped, clamped);
        if (clamped) gb_fail(st, GB_ST_OVERHEAT, blk, i, j, k, temp);
        if (d.unbracketed) gb_fail(st, GB_ST_ZERO_UNBRACKETED, blk, i, j, k, ei);
        if (d.maxiter) gb_fail(st, GB_ST_ZERO_MAXITER, blk, i, j, k, ei);
    }
}

__global__ void k_sur_fallback(gb_dev_grid g, gb_cool_ctx c, double gamma, const int* __restrict__ list,
                               double dt_code, const double* __restrict__ dtp, const int* __restrict__ rej, const int* __restrict__ nrej,
                               gb_status* st)
{
    // a fixed grid striding over the compacted list: usually nothing is
    // rejected, and a grid sized for the worst case would launch thousands
    // of CTAs that only read the count
    const int n = *nrej;
    if (dtp) dt_code = *dtp;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
        sur_fallback_cell(g, c, gamma, list, dt_code, rej[q], st);
}

int g_cool_mode = 0;
double g_sur_tol = 2e-3;
int g_sur_check64 = 0;
struct sur_bufs {
    float* feat = nullptr;
    float* y = nullptr;
    float2* f0 = nullptr;
    int* rej = nullptr;
    int* nrej = nullptr;
    int64_t cap = 0;
} g_sbs[2];  // one set per chunk stream

gb_cool_pf make_pf(const gb_cool_params& p)
{
    gb_cool_pf f;
    f.theatmin = (float)p.theatmin;
    f.theatmax = (float)p.theatmax;
    f.tradmin = (float)p.tradmin;
    f.tradmax = (float)p.tradmax;
    f.dradmin = (float)p.dradmin;
    f.dradmax = (float)p.dradmax;
    f.dust_sputter_temp = (float)p.dust_sputter_temp;
    f.Gzero = (float)p.Gzero;
    f.pe_norm = (float)p.pe_norm;
    f.crIonExp = (float)p.crIonExp;
    f.crIonNH = (float)p.crIonNH;
    f.lnNH = (float)log(p.crIonNH);
    f.crRE = (float)(p.crIonRate * p.crIonEnergy);
    f.T_cool_min = (float)p.T_cool_min;
    f.nd_cool_min = (float)p.nd_cool_min;
    f.nd_cool_max = (float)p.nd_cool_max;
    f.absTmin = (float)p.absTmin;
    f.jeansK = (float)(5.0 / 3.0 * 3.1415926535897932384 * p.boltz / 6.6725985e-8);
    f.use_cr_heating = p.use_cr_heating;
    f.cr_uniform = (p.crIonNH == 1.0 && p.crIonExp == 1.0) ? 1 : 0;
    f.pe_recipe = p.pe_recipe;
    f.useDustCool = p.useDustCool;
    return f;
}

int sur_ensure(sur_bufs& g_sb, int64_t ncell)
{
    if (ncell <= g_sb.cap) return GB_OK;
    cudaFree(g_sb.feat);
    cudaFree(g_sb.y);
    cudaFree(g_sb.f0);
    cudaFree(g_sb.rej);
    if (!g_sb.nrej && gb_check(cudaMalloc(&g_sb.nrej, sizeof(int)), "sur nrej")) return GB_ERR_CUDA;
    if (gb_check(cudaMalloc(&g_sb.feat, sizeof(float) * 4 * ncell), "sur feat") ||
        gb_check(cudaMalloc(&g_sb.y, sizeof(float) * ncell), "sur y") ||
        gb_check(cudaMalloc(&g_sb.f0, sizeof(float2) * ncell), "sur f0") ||
        gb_check(cudaMalloc(&g_sb.rej, sizeof(int) * ncell), "sur rej"))
        return GB_ERR_CUDA;
    g_sb.cap = ncell;
    return GB_OK;
}

}  // namespace

int gb_cooling_mode() { return g_cool_mode; }

int gb_sur_prepare(int64_t ncell, cudaStream_t s)
{
    int rc = sur_ensure(g_sbs[0], ncell);
    if (!rc && gb_chunk_streams() > 1) rc = sur_ensure(g_sbs[1], ncell);
    return rc ? rc : gb_mlp_pack(s);
}

// the unit factors of the surrogate kernels
static sur_units make_units()
{
    sur_units un;
    {
        const gb_cool_params& p = g_gb.cool.p;
        un.T_of_e = (g_gb.hp.gamma - 1.0) * p.eos_abar * p.mp / p.boltz;
        un.e_of_T = 1.0 / un.T_of_e;
        un.inv_mu_mp = 1.0 / (p.mu_mol * p.mp);
        un.vel2 = p.vel_unit * p.vel_unit;
        un.inv_vel2 = 1.0 / un.vel2;
        un.dens_unit_f = (float)p.dens_unit;
        un.T_of_e_f = (float)un.T_of_e;
        un.e_of_T_f = (float)un.e_of_T;
        un.inv_mu_mp_f = (float)un.inv_mu_mp;
        un.time_unit_f = (float)p.time_unit;
        un.mu_mol_f = (float)p.mu_mol;
        un.xHp_const_f = (float)p.xHp_const;
        un.emin_f = (float)(0.5 * p.absTmin * un.e_of_T);
        un.absTmin_f = (float)p.absTmin;
        un.absTmax_f = (float)p.absTmax;
        un.dust_sputter_f = (float)p.dust_sputter_temp;
        un.smallp_f = (float)p.smallp;
        un.smallp = p.smallp;
        un.dens_unit = p.dens_unit;
        un.T_min_f = (float)g_gb.cool.T_min;
        un.nd_min_f = (float)g_gb.cool.nd_min;
    }
    return un;
}

// Where the hydro update of a chunk of nblk blocks on chain `chain` writes
// the surrogate's features (its buffers, allocated here when they are too
// small: callers inside a capture prepared them before)
int gb_sur_feat_target(int chain, int nblk, sur_feat_out* out)
{
    sur_bufs& g_sb = g_sbs[chain & 1];
    int rc = sur_ensure(g_sb, (int64_t)nblk * 4096);
    if (rc) return rc;
    out->feat = reinterpret_cast<float4*>(g_sb.feat);
    out->f0 = g_sb.f0;
    out->pf = make_pf(g_gb.cool.p);
    out->un = make_units();
    return GB_OK;
}

int gb_launch_surrogate(int nblk, const int* list, double dt, const double* dtp, gb_status* st, cudaStream_t s,
                        int chain, bool feat_done)
{
    sur_bufs& g_sb = g_sbs[chain & 1];
    const int64_t ncell = (int64_t)nblk * 4096;
    int rc = sur_ensure(g_sb, ncell);
    if (rc) return rc;
    const unsigned nb = (unsigned)((ncell + 127) / 128);
    const gb_cool_pf pf = make_pf(g_gb.cool.p);
    const sur_units un = make_units();
    if (!feat_done) {
        gb_prof_begin(GBP_SUR_FEAT, s);
        k_sur_feat<<<nb, 128, 0, s>>>(g_gb.grid, g_gb.cool, pf, un, list, ncell, dt, dtp, g_sb.feat, g_sb.f0);
        gb_prof_end(GBP_SUR_FEAT, s);
    }
    gb_prof_begin(GBP_MLP, s);
    rc = gb_mlp_launch_infer(ncell, g_sb.feat, g_sb.y, st, s);
    gb_prof_end(GBP_MLP, s);
    if (rc) return rc;
    cudaMemsetAsync(g_sb.nrej, 0, sizeof(int), s);
    gb_prof_begin(GBP_SUR_ACCEPT, s);
    if (g_sur_check64)
        k_sur_accept<true><<<nb, 128, 0, s>>>(g_gb.grid, g_gb.cool, pf, un, g_gb.hp.gamma, list, ncell, dt, dtp, g_sb.y, g_sb.f0,
                                              g_sur_tol, g_sb.rej, g_sb.nrej, st);
    else
        k_sur_accept<false><<<nb, 128, 0, s>>>(g_gb.grid, g_gb.cool, pf, un, g_gb.hp.gamma, list, ncell, dt, dtp, g_sb.y, g_sb.f0,
                                               g_sur_tol, g_sb.rej, g_sb.nrej, st);
    gb_prof_end(GBP_SUR_ACCEPT, s);
    gb_prof_begin(GBP_SUR_FALLBACK, s);
    k_sur_fallback<<<nb < 152 * 4 ? nb : 152 * 4, 128, 0, s>>>(g_gb.grid, g_gb.cool, g_gb.hp.gamma, list, dt, dtp,
                                                               g_sb.rej, g_sb.nrej, st);
    gb_prof_end(GBP_SUR_FALLBACK, s);
    return gb_check(cudaGetLastError(), "surrogate launch") ? GB_ERR_CUDA : GB_OK;
}

extern "C" int gb_set_cooling_mode(int mode, double rel_tol, int check_fp64)
{
    if (mode < 0 || mode > 2 || !(rel_tol > 0.0) || rel_tol > 0.5) return GB_ERR_ARG;
    g_cool_mode = mode;
    g_gb.gen += 1;
    g_sur_tol = rel_tol;
    g_sur_check64 = check_fp64 ? 1 : 0;
    return GB_OK;
}

extern "C" int gb_surrogate_samples(int64_t n, uint64_t seed, float* feat, float* target, gb_status* st, void* stream)
{
    if (!g_gb.cool_ok) {
        gb_set_error("gb_surrogate_samples: call gb_cool_init first");
        return GB_ERR_NOT_INIT;
    }
    if (n <= 0 || !feat || !target) return GB_ERR_ARG;
    k_sur_samples<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(g_gb.cool, n, seed, feat, target, st);
    return gb_check(cudaGetLastError(), "k_sur_samples") ? GB_ERR_CUDA : GB_OK;
}
