/*
 * Multi-block drivers over the oracle (test infrastructure only): the
 * block loop a FLASH rank runs, parallelised one block per OpenMP thread
 * for the timed CPU baseline.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#include <math.h>
#endif

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* params of block b: the per-cell CFL codes point at the block's own */
static orc_hydro_params at_block(const orc_hydro_params* p, int b)
{
    orc_hydro_params q = *p;
    if (p->cflc) q.cflc = p->cflc + (int64_t)b * ORC_CFLC;
    return q;
}

/* One unsplit step over nblocks consecutive blocks (block-major storage as
 * in hydro_oracle.h). Returns the total fallback-cell count. */
long orc_unsplit_blocks(const orc_hydro_params* p, int nblocks, double* u, double* bx, double* by,
                        double* bz, double dt, double dx, double dy, double dz)
{
    const int n = p->nxb + 2 * p->nguard;
    const int64_t n3 = (int64_t)n * n * n, fsz = n3 + (int64_t)n * n;
    long total = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
    for (int b = 0; b < nblocks; ++b) {
        double* ub = u + (int64_t)b * ORV_NVAR * n3;
        double* fx = p->mhd ? bx + (int64_t)b * fsz : NULL;
        double* fy = p->mhd ? by + (int64_t)b * fsz : NULL;
        double* fz = p->mhd ? bz + (int64_t)b * fsz : NULL;
        orc_hydro_params pb = at_block(p, b);
        total += orc_unsplit_block(&pb, ub, fx, fy, fz, dt, dx, dy, dz);
    }
    return total;
}

double orc_dt_limit_blocks(const orc_hydro_params* p, int nblocks, const double* u, double dx,
                           double dy, double dz)
{
    const int n = p->nxb + 2 * p->nguard;
    const int64_t n3 = (int64_t)n * n * n;
    double best = 1e300;
#pragma omp parallel for reduction(min : best)
    for (int b = 0; b < nblocks; ++b) {
        orc_hydro_params pb = at_block(p, b);
        double v = orc_block_dt_limit(&pb, u + (int64_t)b * ORV_NVAR * n3, dx, dy, dz);
        if (v < best) best = v;
    }
    return best;
}

/* RadHeat over many cells, one chunk per thread. */
int orc_radheat_cells_omp(const orc_cool_params* p, const orc_table* t, int64_t n, double dt,
                          const double* dens, const double* velx, const double* vely,
                          const double* velz, double* ener, double* eint, double* temp,
                          double* tdus, const double* xhp, double* phhe, double* pefl,
                          int* ncount_out, int* flags_out)
{
    int clamped = 0;
    const int64_t chunk = 256;
    int64_t nchunks = (n + chunk - 1) / chunk;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : clamped)
    for (int64_t c = 0; c < nchunks; ++c) {
        int64_t o = c * chunk;
        int64_t m = n - o < chunk ? n - o : chunk;
        clamped += orc_radheat_cells(p, t, m, dt, dens + o, velx ? velx + o : NULL,
                                     vely ? vely + o : NULL, velz ? velz + o : NULL, ener + o,
                                     eint + o, temp + o, tdus + o, xhp ? xhp + o : NULL,
                                     phhe ? phhe + o : NULL, pefl ? pefl + o : NULL,
                                     ncount_out ? ncount_out + o : NULL,
                                     flags_out ? flags_out + o : NULL);
    }
    return clamped;
}

/* ---------------------------------------------------- block-tree leaf lists */

void orc_fill_guards_list(const orc_hydro_params* p, int nlist, const int* list, const int* level,
                          const int* coord, const int* child, const int* root, int nr0, int nr1, int nr2,
                          int maxlevel, double* u, double* bx, double* by, double* bz)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (int q = 0; q < nlist; ++q)
        orc_fill_guards_leaf(p, list[q], level, coord, child, root, nr0, nr1, nr2, maxlevel, u, bx, by, bz);
}

double orc_dt_limit_list(const orc_hydro_params* p, int nlist, const int* list, const int* level,
                         const double* u, double root_dx)
{
    const int n = p->nxb + 2 * p->nguard;
    const int64_t n3 = (int64_t)n * n * n;
    double best = 1e300;
#pragma omp parallel for reduction(min : best)
    for (int q = 0; q < nlist; ++q) {
        const int b = list[q];
        const double dx = ldexp(root_dx, -level[b]);
        orc_hydro_params pb = at_block(p, b);
        double v = orc_block_dt_limit(&pb, u + (int64_t)b * ORV_NVAR * n3, dx, dx, dx);
        if (v < best) best = v;
    }
    return best;
}

long orc_unsplit_list(const orc_hydro_params* p, int nlist, const int* list, const int* level, double* u,
                      double* bx, double* by, double* bz, double dt, double root_dx)
{
    const int n = p->nxb + 2 * p->nguard;
    const int64_t n3 = (int64_t)n * n * n, fsz = n3 + (int64_t)n * n;
    long total = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
    for (int q = 0; q < nlist; ++q) {
        const int b = list[q];
        const double dx = ldexp(root_dx, -level[b]);
        double* ub = u + (int64_t)b * ORV_NVAR * n3;
        double* fx = p->mhd ? bx + (int64_t)b * fsz : NULL;
        double* fy = p->mhd ? by + (int64_t)b * fsz : NULL;
        double* fz = p->mhd ? bz + (int64_t)b * fsz : NULL;
        orc_hydro_params pb = at_block(p, b);
        total += orc_unsplit_block(&pb, ub, fx, fy, fz, dt, dx, dx, dx);
    }
    return total;
}

long orc_unsplit_tree(const orc_hydro_params* p, int nlist, const int* list, const int* level, const int* coord,
                      const int* child, const int* root, int nr0, int nr1, int nr2, int maxlevel, double* u,
                      double* bx, double* by, double* bz, double dt, double root_dx, int flux_correct)
{
    const int n = p->nxb + 2 * p->nguard;
    const int64_t n3 = (int64_t)n * n * n, fsz = n3 + (int64_t)n * n;
    int nnodes = 0;
    for (int q = 0; q < nlist; ++q)
        if (list[q] + 1 > nnodes) nnodes = list[q] + 1;
    const size_t per_face = (size_t)p->nxb * p->nxb * ORC_NREG;
    double* reg = NULL;
    double* ereg = NULL;
    if (flux_correct && maxlevel > 0) reg = (double*)calloc((size_t)nnodes * 6 * per_face, sizeof(double));
    if (reg && p->mhd) ereg = (double*)calloc((size_t)nnodes * ORC_NSURF, sizeof(double));
    long total = 0;
    for (int L = maxlevel; L >= 0; --L) {
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
        for (int q = 0; q < nlist; ++q) {
            const int b = list[q];
            if (level[b] != L) continue;
            const double dx = ldexp(root_dx, -level[b]);
            double* ub = u + (int64_t)b * ORV_NVAR * n3;
            double* fx = p->mhd ? bx + (int64_t)b * fsz : NULL;
            double* fy = p->mhd ? by + (int64_t)b * fsz : NULL;
            double* fz = p->mhd ? bz + (int64_t)b * fsz : NULL;
            orc_hydro_params pb = at_block(p, b);
            if (!reg) {
                total += orc_unsplit_block(&pb, ub, fx, fy, fz, dt, dx, dx, dx);
                continue;
            }
            orc_fluxfix ff;
            ff.ereg = ereg;
            ff.b = b;
            ff.nnodes = nnodes;
            ff.level = level;
            ff.coord = coord;
            ff.child = child;
            ff.root = root;
            ff.nr[0] = nr0;
            ff.nr[1] = nr1;
            ff.nr[2] = nr2;
            ff.maxlevel = maxlevel;
            int fine[24];
            orc_face_links(b, level, coord, child, root, nr0, nr1, nr2, maxlevel, ff.type, fine);
            for (int f = 0; f < 6; ++f) {
                ff.store[f] = reg + ((size_t)b * 6 + f) * per_face;
                for (int qq = 0; qq < 4; ++qq) {
                    const int m = fine[4 * f + qq];
                    /* the fine leaf's face that touches this block is the opposite one */
                    ff.fine[f][qq] = m >= 0 && m < nnodes ? reg + ((size_t)m * 6 + (f ^ 1)) * per_face : NULL;
                }
            }
            total += orc_unsplit_block_fc(&pb, ub, fx, fy, fz, dt, dx, dx, dx, &ff);
        }
    }
    free(reg);
    free(ereg);
    return total;
}
