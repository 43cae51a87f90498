// Heating/cooling source term: table set-up and per-cell kernels.
// Compiled with -fmad=false (see cool_dev.cuh).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "cool_dev.cuh"
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

__device__ __forceinline__ bool finite_pos(double x) { return isfinite(x) && x > 0.0; }

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

// The same per-cell solve on plain CGS arrays.
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
    heating_and_cooling(c, v, &ei, dt, &temp, &d);
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
    std::vector<double> h(GB_TEMP_PTS + GB_DENS_PTS + (size_t)GB_TEMP_PTS * GB_DENS_PTS);
    for (int j = 0; j < GB_TEMP_PTS; ++j) h[j] = pow(10.e0, (double)lt[j] / 10000.0);
    for (int i = 0; i < GB_DENS_PTS; ++i) h[GB_TEMP_PTS + i] = pow(10.e0, (double)ln[i] / 10000.0);
    for (size_t q = 0; q < ll.size(); ++q)
        h[GB_TEMP_PTS + GB_DENS_PTS + q] = pow(10.e0, (double)ll[q] / 10000.0);
    if (!g_gb.d_table) {
        if (gb_check(cudaMalloc(&g_gb.d_table, h.size() * sizeof(double)), "cudaMalloc(table)"))
            return GB_ERR_CUDA;
    }
    if (gb_check(cudaMemcpy(g_gb.d_table, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice),
                 "cudaMemcpy(table)"))
        return GB_ERR_CUDA;
    g_gb.cool.p = *p;
    g_gb.cool.T = g_gb.d_table;
    g_gb.cool.n = g_gb.d_table + GB_TEMP_PTS;
    g_gb.cool.lam = g_gb.d_table + GB_TEMP_PTS + GB_DENS_PTS;
    g_gb.cool.T_min = h[0];
    g_gb.cool.nd_min = h[GB_TEMP_PTS];
    g_gb.cool_ok = true;
    return GB_OK;
}

int gb_launch_cool_blocks(int nblk, const int* list, double dt, gb_status* st, cudaStream_t s)
{
    dim3 grid((GB_NXB * GB_NXB * GB_NXB + 127) / 128, nblk);
    k_heat_blocks<<<grid, 128, 0, s>>>(g_gb.grid, g_gb.cool, list, dt, g_gb.hp.gamma, st);
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
    k_cool_cells<<<(unsigned)nb, tpb, 0, (cudaStream_t)stream>>>(g_gb.cool, n, dens, ei, temp, tdust,
                                                                  xhp, phhe, gflux, dt, st);
    return gb_check(cudaGetLastError(), "k_cool_cells") ? GB_ERR_CUDA : GB_OK;
}
