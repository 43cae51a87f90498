/*
 * CPU oracle: heating/cooling source term. TEST INFRASTRUCTURE ONLY (see
 * oracle.h). Each function names the Fortran routine and lines it restates;
 * statement order and operand order follow the Fortran so that, compiled
 * with -ffp-contract=off, every rounding step is the one gfortran performs.
 *
 * Where the Fortran prints and `stop`s (root finder failures) this code
 * records a flag in orc_cool_diag and carries on with a defined value, so a
 * test can compare the flag with the GPU kernel's status word.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* Fortran MAX/MIN on non-NaN reals. */
static inline double fmx(double a, double b) { return a > b ? a : b; }
static inline double fmn(double a, double b) { return a < b ? a : b; }

static const double ORC_PI = 3.1415926535897932384;     /* heatCool.F90:1683 */
static const double ORC_NEWTON = 6.6725985e-8;          /* heatCool.F90:1683 */

void orc_cool_default_params(orc_cool_params* p)
{
    /* Values of flash.par.turbsph_standard:300-390 and :170, with the
     * Config defaults of phenHeat/Config for the rest. */
    memset(p, 0, sizeof(*p));
    p->tradmin = 10.0;
    p->tradmax = 1.e15;
    p->dradmin = 1e-99;
    p->dradmax = 1e10;
    p->theatmin = 1e-99;
    p->theatmax = 2.0e4;
    p->absTmin = 10.0;
    p->absTmax = 1e9;
    p->Gzero = 1.69e0;
    p->subfactor = 0.3;
    p->smallp = 1.3807e-19;
    p->use_cr_heating = 1;
    p->crIonRate = 2.0e-17;
    p->crIonNH = 1e20;
    p->crIonExp = 0.021;
    p->crIonEnergy = 20.0e0 * 1.6022e-12; /* Heat_init.F90:75 */
    p->dust_sputter_temp = 3e5;
    p->pe_recipe = 0; /* WD01 */
    p->pe_norm = 1.3e-24;
    /* CGS Boltzmann constant and proton mass (CODATA 2006). FLASH takes
     * them from its PhysicalConstants unit, which is not vendored. */
    p->boltz = 1.3806504e-16;
    p->mp = 1.672621637e-24;
    p->T_cool_min = 10.0;
    p->nd_cool_min = 1e1;
    p->nd_cool_max = 1e10;
    p->useDustCool = 1;
    p->int_method = 0; /* "Implicit", flash.par.turbsph_standard:314 */
    p->mu_mol = 24.0 / 11.0;
}

/* ------------------------------------------------------------- table */

int orc_table_load_flash(orc_table* t, const char* path)
{
    /* get_cooling_data.F90:20-55 */
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    char line[256];
    if (!fgets(line, sizeof line, f)) { fclose(f); return -2; }
    int ti = 0, dj = 0;
    if (sscanf(line, "%d %d", &ti, &dj) != 2 || ti != ORC_TEMP_PTS || dj != ORC_DENS_PTS) {
        fclose(f);
        return -2;
    }
    for (int j = 0; j < ORC_TEMP_PTS; ++j) {
        for (int i = 0; i < ORC_DENS_PTS; ++i) {
            if (!fgets(line, sizeof line, f)) { fclose(f); return -3; }
            double v[6];
            /* FORMAT(6(2X,F8.4)): six fields of ten columns */
            size_t len = strlen(line);
            if (len < 60) { fclose(f); return -3; }
            for (int c = 0; c < 6; ++c) {
                char fld[11];
                memcpy(fld, line + 10 * c, 10);
                fld[10] = 0;
                char* end = NULL;
                v[c] = strtod(fld, &end);
                if (end == fld) { fclose(f); return -3; }
            }
            double T = pow(10.e0, v[0]);
            double n = pow(10.e0, v[1]);
            double L = pow(10.e0, v[5]);
            if (i == 0) t->T[j] = T;
            if (j == 0) t->n[i] = n;
            t->lambda[i + ORC_DENS_PTS * j] = L;
        }
    }
    fclose(f);
    t->T_min = t->T[0];
    t->nd_min = t->n[0];
    return 0;
}

void orc_table_from_ilog(orc_table* t, const int32_t* logT_e4, const int32_t* logn_e4,
                         const int32_t* logL_e4)
{
    /* k / 10000.0 is the double nearest to the decimal k*1e-4, i.e. exactly
     * what a formatted read of the F8.4 field returns. */
    for (int j = 0; j < ORC_TEMP_PTS; ++j) t->T[j] = pow(10.e0, (double)logT_e4[j] / 10000.0);
    for (int i = 0; i < ORC_DENS_PTS; ++i) t->n[i] = pow(10.e0, (double)logn_e4[i] / 10000.0);
    for (int k = 0; k < ORC_DENS_PTS * ORC_TEMP_PTS; ++k)
        t->lambda[k] = pow(10.e0, (double)logL_e4[k] / 10000.0);
    t->T_min = t->T[0];
    t->nd_min = t->n[0];
}

int orc_find(const double* x, double x0, int N)
{
    /* find.F90:9-42. x is 0-based storage of the 1-based table. */
    if (x0 < x[0]) return 0;
    if (x0 > x[N - 1]) return N;
    int il = 1, ir = N;
    while (ir != il + 1) {
        int im = (il + ir) / 2;
        if (x[im - 1] > x0) ir = im;
        else il = im;
    }
    return il;
}

/* ------------------------------------------------------- rate terms */

double orc_lin_interp(double x1, double y1, double x2, double y2, double x)
{
    /* heatCool.F90:2379-2392 (the extrapolation warning is dropped) */
    double ms = (y2 - y1) / (x2 - x1);
    return ms * (x - x1) + y1;
}

double orc_radloss(double T)
{
    /* heatCool.F90:1590-1667 */
    double radia;
    if (T >= 1.70e4) {
        if (T >= 5.62e5) {
            if (T >= 2.75e6) {
                if (T >= 3.16e7) radia = 3.090e-27 * sqrt(T);
                else radia = 5.188e-21 / pow(T, 0.33);
            } else {
                if (T >= 1.78e6) radia = 3.890e-4 / pow(T, 2.95);
                else radia = 1.3e-22 * pow(T / 1.5e5, 0.01);
            }
        } else {
            if (T >= 7.94e4) {
                if (T >= 2.51e5) radia = 3.98e-11 / (T * T);
                else radia = 6.31e-22 * pow(T / 1.e6, 0.01);
            } else {
                if (T >= 3.98e4) radia = 1.e-31 * (T * T);
                else radia = 1.479e-21 / pow(T, 0.216);
            }
        }
    } else {
        if (T >= 1.e3) {
            if (T >= 6.31e3) {
                if (T >= 1.0e4) radia = 7.63e-81 * pow(T, 13.8);
                else radia = 3.13e-27 * pow(T, 0.396);
            } else {
                if (T >= 3.16e3) radia = 2.64e-26 * pow(T, 0.152);
                else radia = 5.28e-27 * pow(T, 0.352);
            }
        } else {
            if (T >= 3.98e1) {
                if (T >= 2.00e2) radia = 3.06e-27 * pow(T, 0.431);
                else radia = 1.52e-28 * pow(T, 0.997);
            } else {
                if (T >= 2.51e1) radia = 2.39e-29 * pow(T, 1.50);
                else radia = 1.095e-32 * pow(T, 3.885);
            }
        }
    }
    return radia;
}

static double lam_jeans(const orc_cool_params* p, double rho, double n, double T)
{
    /* heatCool.F90:1687 / :1717 */
    return 1.0 / (rho / n) * sqrt(5. / 3. * ORC_PI * p->boltz * T / n / ORC_NEWTON);
}

static double approx_column_dens(const orc_cool_params* p, double rho, double n, double T)
{
    /* heatCool.F90:1669-1691 */
    double lam_j = lam_jeans(p, rho, n, T);
    return lam_j * n;
}

static double f_ext(const orc_cool_params* p, double rho, double n, double T)
{
    /* heatCool.F90:1693-1722 */
    const double dust_gas_ratio = 0.01, N_H0 = 1.87e21;
    double lam_j = lam_jeans(p, rho, n, T);
    double Av = lam_j * n * dust_gas_ratio / N_H0;
    return exp(-3.5 * Av);
}

static double heating(const orc_cool_params* p, double T, double n, double rho, double strat)
{
    /* heatCool.F90:890-964 (ephen_in is unused by the routine) */
    double eplus = 0.0, lin;
    if ((T <= p->theatmax) && (T >= p->theatmin)) {
        if (p->use_cr_heating) {
            if (p->crIonNH == 1.0 && p->crIonExp == 1.0) {
                eplus = strat * p->crIonRate * p->crIonEnergy / (rho / n);
            } else {
                eplus = strat *
                        (p->crIonRate * p->crIonEnergy *
                         pow(fmx(p->crIonNH, approx_column_dens(p, rho, n, T)) / p->crIonNH,
                             -p->crIonExp)) /
                        (rho / n);
            }
        }
        double ll = p->theatmin, ll10 = ll + 0.1 * ll;
        double ul = p->theatmax, ul10 = ul - 0.1 * ul;
        if (T >= ul10) lin = orc_lin_interp(ul10, 1.0, ul, 0.0, T);
        else if (T <= ll10) lin = orc_lin_interp(ll, 0.0, ll10, 1.0, T);
        else lin = 1.0;
        eplus = eplus * lin;
    } else {
        eplus = 0.0;
    }
    return eplus;
}

static void pe_heating(const orc_cool_params* p, double G, double xHp, double n, double T,
                       double rho, double* PeHeat, double* dust_heating)
{
    /* heatCool.F90:970-1110 */
    const double C0 = 7.64, C1 = 4.52, C2 = 0.04371, C3 = 0.00557, C4 = 0.132, C5 = 0.452,
                 C6 = 0.675;
    *PeHeat = 0.0;
    *dust_heating = 0.0;
    if ((T <= fmn(p->theatmax, p->dust_sputter_temp)) && (T >= p->theatmin)) {
        double xl = (xHp == 0.0) ? 1e-8 : xHp;
        double Gfactor, eff;
        if (p->pe_recipe == 1) { /* BT94 */
            Gfactor = G * sqrt(T) / (xl * n * 0.5);
            eff = 4.9e-2 / (1.0 + 4.0e-3 * pow(Gfactor, 0.73)) +
                  (3.7e-2 * pow(T / 1.0e4, 0.7)) / (1.0 + 2.0e-4 * Gfactor);
            *PeHeat = p->pe_norm * eff * G / (rho / n);
            *dust_heating = p->pe_norm * fmx(0.0, (1.0 - eff)) * G * n;
        } else if (p->pe_recipe == 0) { /* WD01 */
            Gfactor = G * sqrt(T) / (xl * n);
            eff = (C0 + C1 * pow(T, C4)) /
                  (1.0 + (C2 * pow(Gfactor, C5)) * (1.0 + C3 * pow(Gfactor, C6)));
            *PeHeat = 1e-26 * eff * G / (rho / n);
            *dust_heating = (p->pe_norm - 1e-26 * eff) * G * n;
            *dust_heating = fmx(*dust_heating, 0.0);
        } else { /* NOGF */
            eff = 0.05;
            *PeHeat = p->pe_norm * eff * G / (rho / n);
            *dust_heating = p->pe_norm * (1.0 - eff) * G * n;
        }
        double ll = p->theatmin, ll10 = ll + 0.1 * ll;
        double ul = fmn(p->theatmax, p->dust_sputter_temp), ul10 = ul - 0.1 * ul, lin;
        if (T >= ul10) lin = orc_lin_interp(ul10, 1.0, ul, 0.0, T);
        else if (T <= ll10) lin = orc_lin_interp(ll, 0.0, ll10, 1.0, T);
        else lin = 1.0;
        *PeHeat = *PeHeat * lin;
    }
}

static double cooling(const orc_cool_params* p, double T, double n, double conf, double xHp)
{
    /* heatCool.F90:1116-1200 (DGionFix = .true.) */
    double emin = 0.0;
    if ((T <= p->tradmax && T >= p->tradmin) && (n >= p->dradmin && n <= p->dradmax)) {
        emin = orc_radloss(T);
        if (xHp > 1e-2 && T < 1.2e4) {
            double DG = orc_lin_interp(1e-2, 1.0, 1e-1, 5.0, fmn(1e-1, xHp));
            emin = emin * DG;
            if (T > 1e4) {
                double q = orc_lin_interp(1e4, 1.0, 1.2e4, pow(DG, 0.5), T);
                emin = emin / (q * q);
            }
        } else if (xHp < 1e-2 && T < 1e4) {
            double DG = orc_lin_interp(1e-4, 0.35, 1e-2, 1.0, fmx(1e-4, xHp));
            emin = emin * DG;
            if (T > 9e3) emin = emin / orc_lin_interp(9e3, 1.0, 1e4, DG, T);
        }
        double ll = p->tradmin, ll10 = ll + 0.1 * ll;
        double ul = p->tradmax, ul10 = ul - 0.1 * ul, lin;
        if (T >= ul10) lin = orc_lin_interp(ul10, 1.0, ul, 0.0, T);
        else if (T <= ll10) lin = orc_lin_interp(ll, 0.0, ll10, 1.0, T);
        else lin = 1.0;
        emin = emin * lin;
        emin = emin * conf;
    } else {
        emin = 0.0;
    }
    return emin;
}

static double molecular_cooling(const orc_cool_params* p, const orc_table* t, double n,
                                double T, double mu)
{
    /* heatCool.F90:1211-1303 */
    double cool_pw = 0.0;
    if ((n >= p->nd_cool_min) && (n <= p->nd_cool_max) && (T >= p->T_cool_min) &&
        (T <= p->theatmax)) {
        int ixtemp = orc_find(t->T, fmx(T, t->T_min), ORC_TEMP_PTS);
        int ixdens = orc_find(t->n, fmx(n, t->nd_min), ORC_DENS_PTS);
        if (ixtemp > 0 && ixtemp <= ORC_TEMP_PTS && ixdens > 0 && ixdens <= ORC_DENS_PTS)
            cool_pw = t->lambda[(ixdens - 1) + ORC_DENS_PTS * (ixtemp - 1)] / (mu * p->mp);
        else
            cool_pw = 0.0;
        double ll = p->T_cool_min, ll10 = ll + 0.1 * ll;
        double ul = p->theatmax, ul10 = ul - 0.1 * ul, lin;
        if (T >= ul10) lin = orc_lin_interp(ul10, 1.0, ul, 0.0, T);
        else if (T <= ll10) lin = orc_lin_interp(ll, 0.0, ll10, 1.0, T);
        else lin = 1.0;
        cool_pw = cool_pw * lin;
        ll = p->nd_cool_min; ll10 = ll + 0.1 * ll;
        ul = p->nd_cool_max; ul10 = ul - 0.1 * ul;
        if (n >= ul10) lin = orc_lin_interp(ul10, 1.0, ul, 0.0, n);
        else if (n <= ll10) lin = orc_lin_interp(ll, 0.0, ll10, 1.0, n);
        else lin = 1.0;
        cool_pw = cool_pw * lin;
    }
    return cool_pw;
}

static double dust_cooling(const orc_cool_params* p, double n, double T, double tdust, double rho)
{
    /* heatCool.F90:1305-1390 */
    double cool_dg = 0.0;
    if (T <= p->dust_sputter_temp) {
        double lambda_gd =
            3.8e-33 * (n * n) * (1.0 - 0.8 * exp(-75.0 / T)) * (T - tdust) * sqrt(T);
        cool_dg = lambda_gd / rho;
        double ul = p->dust_sputter_temp, ul10 = ul - 0.1 * ul, lin;
        if (T >= ul10) lin = orc_lin_interp(ul10, 1.0, ul, 0.0, T);
        else lin = 1.0;
        cool_dg = cool_dg * lin;
    }
    return cool_dg;
}

double orc_dust_cooling(const orc_cool_params* p, double n, double T, double tdust, double rho)
{
    return dust_cooling(p, n, T, tdust, rho);
}

double orc_dei_dt(const orc_cool_params* p, const orc_table* t, orc_cool_vars* v, double t_in,
                  double ei_in)
{
    /* heatCool.F90:1397-1588 */
    (void)t_in;
    double tmp_temp = ei_in / v->TtoEI;
    if (tmp_temp < 0.0) tmp_temp = 1.0;
    double eplus = heating(p, tmp_temp, v->ndens, v->rho, v->strat_factor);
    double total_local_FUV = v->Gflux + p->Gzero * f_ext(p, v->rho, v->ndens, tmp_temp) *
                                            v->strat_factor;
    double PeHeat, dust_heating;
    pe_heating(p, total_local_FUV, v->xHp, v->ndens, tmp_temp, v->rho, &PeHeat, &dust_heating);
    eplus = eplus + v->ephen;
    double emin = cooling(p, p->tradmin, v->ndens, v->conf, v->xHp);
    double cool_pw = 0.0, cool_dg = 0.0;
    if (p->useDustCool) cool_pw = molecular_cooling(p, t, v->ndens, p->T_cool_min, v->mu_mol);
    double cooling_floor = emin + cool_pw;
    emin = cooling(p, tmp_temp, v->ndens, v->conf, v->xHp);
    if (p->useDustCool) {
        cool_pw = molecular_cooling(p, t, v->ndens, tmp_temp, v->mu_mol);
        cool_dg = dust_cooling(p, v->ndens, tmp_temp, v->tdust, v->rho);
    }
    return eplus + PeHeat - emin - cool_pw - cool_dg + cooling_floor;
}

/* ------------------------------------------------------- dust solver */

static double get_dust_temperature(const orc_cool_params* p, double tdust_in, double temp_in,
                                   double nden, double phen_heat, orc_cool_diag* d)
{
    /* heatCool.F90:703-884 */
    const double tol = 1.e-4, smallt = .1;
    const int max_newton = 100;
    double error = 10. * tol;
    double tdust = tdust_in;
    if (tdust < p->absTmin) tdust = p->absTmin;
    double temp_gas = (temp_in < p->absTmin) ? p->absTmin : temp_in;
    double heat = phen_heat;
    int l = 1;
    while ((l <= max_newton) && (error > tol)) {
        double lambda_dust = 6.8 * pow(tdust, 6.0);
        double coll = 3.8 * nden * (1.0 - 0.8 * exp(-75.0 / temp_gas)) * (temp_gas - tdust) *
                      sqrt(temp_gas);
        double eqfunc = heat + coll - lambda_dust;
        double det = -(6.0 * lambda_dust / tdust) -
                     3.8 * nden * (1.0 - 0.8 * exp(-75.0 / temp_gas)) * sqrt(temp_gas);
        double tnew = tdust - eqfunc / det;
        error = fabs(tnew - tdust) / tdust;
        tdust = tnew;
        if (tdust < smallt) {
            tdust = smallt;
            error = 0.1 * tol;
        }
        l = l + 1;
    }
    if (l > max_newton && d) d->dust_noconv += 1;
    if (tdust < p->absTmin) tdust = p->absTmin;
    return tdust;
}

static void dust_update(const orc_cool_params* p, orc_cool_vars* v, double temp, double one_e33,
                        orc_cool_diag* d)
{
    /* the block repeated at heatCool.F90:325-338, :430-443, :570-583 */
    double total_local_FUV =
        v->Gflux + p->Gzero * f_ext(p, v->rho, v->ndens, temp) * v->strat_factor;
    double PeHeat, dust_heat;
    pe_heating(p, total_local_FUV, v->xHp, v->ndens, temp, v->rho, &PeHeat, &dust_heat);
    double dust_cr_heat = heating(p, temp, v->ndens, v->rho, v->strat_factor);
    dust_cr_heat = dust_cr_heat * v->rho;
    dust_heat = dust_heat + dust_cr_heat;
    dust_heat = dust_heat / (v->ndens * one_e33);
    v->tdust = get_dust_temperature(p, v->tdust, temp, v->ndens, dust_heat, d);
}

/* ------------------------------------------------------- root finders */

static double one_step(const orc_cool_params* p, const orc_table* t, orc_cool_vars* v,
                       double dx, double y, double yold)
{
    /* heatCool.F90:1928-1950 */
    return y - dx * orc_dei_dt(p, t, v, dx, y) - yold;
}

static double zero(const orc_cool_params* p, const orc_table* t, orc_cool_vars* v, double a,
                   double b, double a_old, double machep, double tt, double dt, orc_cool_diag* d)
{
    /* heatCool.F90:1981-2197 (Brent's method) */
    const int max_iter = 10000;
    double sa = a, sb = b;
    double fa = one_step(p, t, v, dt, sa, a_old);
    double fb = one_step(p, t, v, dt, sb, a_old);
    double c = sa, fc = fa, e = sb - sa, dd = e;
    int n_tries = 0;
    if ((fa > 0.0 && fb > 0.0) || (fa < 0.0 && fb < 0.0)) {
        /* The Fortran prints and stops here. */
        if (d) d->zero_unbracketed += 1;
        return sb;
    }
    for (;;) {
        if (fabs(fc) < fabs(fb)) {
            sa = sb; sb = c; c = sa;
            fa = fb; fb = fc; fc = fa;
        }
        double tol = 2.0 * machep * fabs(sb) + tt;
        double m = 0.5 * (c - sb);
        if (fabs(m) <= tol || fb == 0.0) break;
        if (fabs(e) < tol || fabs(fa) <= fabs(fb)) {
            e = m;
            dd = e;
        } else {
            double s = fb / fa, pp, q, r;
            if (sa == c) {
                pp = 2.0 * m * s;
                q = 1.0 - s;
            } else {
                q = fa / fc;
                r = fb / fc;
                pp = s * (2.0 * m * q * (q - r) - (sb - sa) * (r - 1.0));
                q = (q - 1.0) * (r - 1.0) * (s - 1.0);
            }
            if (0.0 < pp) q = -q;
            else pp = -pp;
            s = e;
            e = dd;
            if (2.0 * pp < 3.0 * m * q - fabs(tol * q) && pp < fabs(0.5 * s * q)) {
                dd = pp / q;
            } else {
                e = m;
                dd = e;
            }
        }
        sa = sb;
        fa = fb;
        if (tol < fabs(dd)) sb = sb + dd;
        else if (0.0 < m) sb = sb + tol;
        else sb = sb - tol;
        fb = one_step(p, t, v, dt, sb, a_old);
        if ((0.0 < fb && 0.0 < fc) || (fb <= 0.0 && fc <= 0.0)) {
            c = sa;
            fc = fa;
            e = sb - sa;
            dd = e;
        }
        n_tries = n_tries + 1;
        if (d) d->brent_iters = n_tries;
        if (n_tries > max_iter) {
            /* The Fortran prints and stops here. */
            if (d) d->zero_maxiter += 1;
            break;
        }
    }
    return sb;
}

static int zbrac(const orc_cool_params* p, const orc_table* t, orc_cool_vars* v, double* x1,
                 double* x2, double xold, double dt)
{
    /* heatCool.F90:2294-2348 */
    const double FACTOR = 1.6;
    const int NTRY = 5000;
    double f1 = one_step(p, t, v, dt, *x1, xold);
    double f2 = one_step(p, t, v, dt, *x2, xold);
    for (int j = 1; j <= NTRY; ++j) {
        if (f1 * f2 < 0.0) return 1;
        if (fabs(f1) < fabs(f2)) {
            *x1 = *x1 + FACTOR * (*x1 - *x2);
            if (*x1 < 0.0) *x1 = v->TtoEI * 1.0;
            f1 = one_step(p, t, v, dt, *x1, xold);
        } else {
            *x2 = *x2 + FACTOR * (*x2 - *x1);
            if (*x2 < 0.0) *x2 = v->TtoEI * 1.0;
            f2 = one_step(p, t, v, dt, *x2, xold);
        }
    }
    return 0;
}

/* ------------------------------------------------------- DoPr5 (RK4) */

typedef double (*orc_rhs)(void* ctx, double x, double y);

typedef struct dopr5_state {
    double atol, rtol, hmin, hmax;
    double k7; /* DoPr5's SAVEd k7 (OdeInt.F90:275); first_call is .false. */
} dopr5_state;

static void dopr5_step(dopr5_state* s, orc_rhs f, void* ctx, double x, double y, double h,
                       double* yn1, double* del)
{
    /* OdeInt.F90:245-327 */
    const double c2 = 1.0 / 5.0, c3 = 3.0 / 10.0, c4 = 4.0 / 5.0, c5 = 8.0 / 9.0, c6 = 1.0,
                 c7 = 1.0;
    const double a21 = 1.0 / 5.0, a31 = 3.0 / 40.0, a32 = 9.0 / 40.0, a41 = 44.0 / 45.0,
                 a42 = -56.0 / 15.0, a43 = 32.0 / 9.0, a51 = 19372.0 / 6561.0,
                 a52 = -25360.0 / 2187.0, a53 = 64448.0 / 6561.0, a54 = -212.0 / 729.0,
                 a61 = 9017.0 / 3168.0, a62 = -355.0 / 33.0, a63 = 46732.0 / 5247.0,
                 a64 = 49.0 / 176.0, a65 = -5103.0 / 18656.0, a71 = 35.0 / 384.0,
                 a72 = 0.0, a73 = 500.0 / 1113.0, a74 = 125.0 / 192.0,
                 a75 = -2187.0 / 6784.0, a76 = 11.0 / 84.0;
    const double b1 = 35.0 / 384.0, b2 = 0.0, b3 = 500.0 / 1113.0, b4 = 125.0 / 192.0,
                 b5 = -2187.0 / 6784.0, b6 = 11.0 / 84.0, b7 = 0.0;
    const double bs1 = 5179.0 / 57600.0, bs2 = 0.0, bs3 = 7571.0 / 16695.0,
                 bs4 = 393.0 / 640.0, bs5 = -92097.0 / 339200.0, bs6 = 187.0 / 2100.0,
                 bs7 = 1.0 / 40.0;
    (void)a72;
    double k1 = s->k7;
    double k2 = h * f(ctx, x + c2 * h, y + a21 * k1);
    double k3 = h * f(ctx, x + c3 * h, y + a31 * k1 + a32 * k2);
    double k4 = h * f(ctx, x + c4 * h, y + a41 * k1 + a42 * k2 + a43 * k3);
    double k5 = h * f(ctx, x + c5 * h, y + a51 * k1 + a52 * k2 + a53 * k3 + a54 * k4);
    double k6 = h * f(ctx, x + c6 * h, y + a61 * k1 + a62 * k2 + a63 * k3 + a64 * k4 + a65 * k5);
    double k7 = h * f(ctx, x + c7 * h,
                      y + a71 * k1 + 0.0 * k2 + a73 * k3 + a74 * k4 + a75 * k5 + a76 * k6);
    s->k7 = k7;
    *yn1 = y + b1 * k1 + b2 * k2 + b3 * k3 + b4 * k4 + b5 * k5 + b6 * k6 + b7 * k7;
    double ysn1 = y + bs1 * k1 + bs2 * k2 + bs3 * k3 + bs4 * k4 + bs5 * k5 + bs6 * k6 + bs7 * k7;
    *del = *yn1 - ysn1;
}

static int dopr5_stepper(dopr5_state* s, orc_rhs f, void* ctx, double ystart, double xx1,
                         double xmax, double* h1, double* xx2, double* yend)
{
    /* OdeInt.F90:125-243 */
    const int max_stepper_count = 100;
    const double order = 5.0, beta = 0.4 / order, alpha = 1.0 / order - 0.75 * beta;
    const double s1 = 0.9;
    int nbad = 0;
    double h = *h1, y = ystart, x = xx1, error = 1.0, yn1 = 0, del = 0;
    while (nbad < max_stepper_count) {
        double oldy = y, oldx = x, oldh = h, olderr = error;
        if ((x + h) > xmax) h = xmax - x;
        dopr5_step(s, f, ctx, x, y, h, &yn1, &del);
        error = fabs(del) / (s->atol + fabs(yn1) * s->rtol);
        if (error == 0.0) h = s->hmax;
        else h = fmx(s1 * oldh * pow(error, -alpha) * pow(olderr, beta), s->hmin);
        if (error <= 1.0) {
            *xx2 = x + oldh;
            *yend = yn1;
            *h1 = h;
            return 0;
        } else {
            y = oldy;
            x = oldx;
            h = fmn(h, s->hmax);
        }
        nbad = nbad + 1;
    }
    return -1; /* the Fortran stops: "nbad so bad" */
}

static int dopr5_driver(dopr5_state* s, orc_rhs f, void* ctx, double yinit, double x1,
                        double x2, double hinit, double* yend)
{
    /* OdeInt.F90:44-120 */
    double y = yinit, x = x1, h = hinit;
    long step = 0;
    while (x < x2) {
        double xn, yn;
        if (dopr5_stepper(s, f, ctx, y, x, x2, &h, &xn, &yn) != 0) return -1;
        x = xn;
        y = yn;
        if (y < 0.0) return -2;
        if (step > 10000000L) return -3;
        step = step + 1;
    }
    *yend = y;
    return 0;
}

static double rhs_line(void* ctx, double x, double y)
{
    (void)ctx;
    (void)y;
    return x; /* test.f95:83-90 */
}

int orc_dopr5_line_kat(double atol, double rtol, double hmin, int have_hmax, double hmax,
                       double dt_out, double t_end, double* out_x, double* out_t, int n_out)
{
    /* test.f95:17-38 with adpt = .true. OdeInit without hmax_in reads an
     * absent optional argument; the intended default hmin*1e5 of
     * OdeInit.F90:30-34 is used instead. */
    dopr5_state s;
    s.atol = atol;
    s.rtol = rtol;
    s.hmin = hmin;
    s.hmax = have_hmax ? hmax : hmin * 1e5;
    s.k7 = 0.0;
    double x = 0.0, t = 0.0, dt = 0.1;
    int k = 0;
    if (k < n_out) { out_x[k] = x; out_t[k] = t; k++; }
    while (t < t_end) {
        double t_new = t + dt_out, x_new = 0.0;
        if (dopr5_driver(&s, rhs_line, NULL, x, t, t_new, dt, &x_new) != 0) return -1;
        x = x_new;
        t = t_new;
        if (k < n_out) { out_x[k] = x; out_t[k] = t; k++; }
    }
    return k;
}

typedef struct cool_rhs_ctx {
    const orc_cool_params* p;
    const orc_table* t;
    orc_cool_vars* v;
} cool_rhs_ctx;

static double rhs_cool(void* ctx, double x, double y)
{
    cool_rhs_ctx* c = (cool_rhs_ctx*)ctx;
    return orc_dei_dt(c->p, c->t, c->v, x, y);
}

/* ------------------------------------------------------- integrator */

void orc_heating_and_cooling(const orc_cool_params* p, const orc_table* t, orc_cool_vars* v,
                             double* ei_io, double timestep, double* temp_io, orc_cool_diag* d)
{
    /* heatCool.F90:41-700 */
    const double err_tol = 1e-6;
    const int max_count = 100000;
    double ei = *ei_io, temp = *temp_io;
    double total_time = 0.0;
    int ncount = 0;

    v->ndens = v->rho / (v->mu_mol * p->mp);
    v->TtoEI = ei / temp;
    v->conf = v->ndens * v->ndens / v->rho;

    if (p->int_method == 1) {
        /* Euler, :119-214 */
        for (;;) {
            double eiold = ei;
            double dei = orc_dei_dt(p, t, v, timestep, eiold);
            double dt1 = p->subfactor * ei / fmx(fabs(dei), 1e-50);
            double dt0 = fmn((timestep - total_time), dt1);
            ei = ei + dei * dt0;
            temp = ei / v->TtoEI;
            total_time = total_time + dt0;
            ncount = ncount + 1;
            if (ncount > max_count) break; /* the Fortran aborts */
            if ((timestep - total_time) < 1e-6) break;
        }
        if (temp < p->absTmin) {
            temp = p->absTmin;
            ei = p->absTmin * v->TtoEI;
        }
        if (p->useDustCool && temp <= p->dust_sputter_temp)
            v->tdust = get_dust_temperature(p, v->tdust, temp, v->ndens, 0.0, d);
    } else if (p->int_method == 0) {
        /* Implicit (backward Euler), :216-514. The loop body runs once:
         * dt0 = timestep on the first pass (first_loop is never cleared). */
        while ((timestep - total_time) > (1e-6 * timestep)) {
            ncount = ncount + 1;
            double eiolder = ei;
            double eiold = ei;
            double dei = orc_dei_dt(p, t, v, timestep, eiold);
            double dt0 = timestep;
            eiold = eiolder + dei * dt0 * 1.0e-3;
            double ei1 = eiolder, ei2 = eiold;
            int bracket_found = 0;
            if (fabs((ei1 - ei2) / ei1) < (err_tol * dt0 / (timestep - total_time))) {
                dt0 = (timestep - total_time);
                ei = eiolder + dei * dt0;
                temp = ei / v->TtoEI;
                if (p->useDustCool && temp <= p->dust_sputter_temp)
                    dust_update(p, v, temp, 1e-33, d);
                total_time = total_time + dt0;
                if (d) d->early_euler += 1;
                continue;
            }
            bracket_found = zbrac(p, t, v, &ei1, &ei2, eiolder, dt0);
            if (!bracket_found && d) d->bracket_fail += 1;
            if (ei1 < 0.0 || ei2 < 0.0) {
                ei1 = fmx(ei1, v->TtoEI * 1.0);
                ei2 = fmx(ei2, v->TtoEI * 1.0);
            }
            if (bracket_found)
                ei = zero(p, t, v, ei1, ei2, eiolder, 3e-16, fmx(v->TtoEI * 1.0, eiold * err_tol),
                          dt0, d);
            else
                ei = zero(p, t, v, v->TtoEI * 1.0, v->TtoEI * 1.0e9, eiolder, 3e-16,
                          fmx(v->TtoEI * 1.0, eiold * err_tol), dt0, d);
            temp = ei / v->TtoEI;
            if (p->useDustCool && temp <= p->dust_sputter_temp) dust_update(p, v, temp, 1e-33, d);
            total_time = total_time + dt0;
        }
        if (temp < p->absTmin) {
            temp = p->absTmin;
            ei = p->absTmin * v->TtoEI;
        }
    } else if (p->int_method == 2) {
        /* trap, :516-610 */
        for (;;) {
            double eiold = ei;
            double dei = orc_dei_dt(p, t, v, timestep, eiold);
            double dt1 = p->subfactor * ei / fmx(fabs(dei), 1e-50);
            double dt0 = fmn((timestep - total_time), dt1);
            double ei1 = eiold + dei * dt0;
            double dei2 = orc_dei_dt(p, t, v, timestep, ei1);
            double ei2 = eiold + 0.5 * dt0 * (dei + dei2);
            temp = ei2 / v->TtoEI;
            total_time = total_time + dt0;
            if (p->useDustCool && temp <= p->dust_sputter_temp) dust_update(p, v, temp, 1e-33, d);
            ncount = ncount + 1;
            if ((timestep - total_time) < 1e-6 || ncount > max_count) break;
        }
        /* ei is not updated by the trap branch (only temp): kept as written. */
        if (temp < p->tradmin) {
            temp = p->tradmin;
            ei = p->tradmin * v->TtoEI;
        }
    } else {
        /* RK4 = adaptive DoPr5, :612-691 */
        dopr5_state s;
        s.atol = ei * 1e-6;
        s.rtol = 1e-6;
        s.hmin = 1.0;
        s.hmax = timestep * p->subfactor;
        s.k7 = 0.0;
        cool_rhs_ctx c = {p, t, v};
        double eiold = ei, out = ei;
        if (dopr5_driver(&s, rhs_cool, &c, eiold, total_time, timestep, 1e3, &out) == 0) ei = out;
        temp = ei / v->TtoEI;
        if (p->useDustCool && temp <= p->dust_sputter_temp) dust_update(p, v, temp, 1e-33, d);
        if (temp < p->absTmin) {
            temp = p->absTmin;
            ei = p->absTmin * v->TtoEI;
        }
    }
    if (d) d->ncount = ncount;
    *ei_io = ei;
    *temp_io = temp;
}

int orc_radheat_cells(const orc_cool_params* p, const orc_table* t, int64_t n, double dt,
                      const double* dens, const double* velx, const double* vely,
                      const double* velz, double* ener, double* eint, double* temp,
                      double* tdus, const double* xhp, double* phhe, double* pefl,
                      int* ncount_out, int* flags_out)
{
    /* RadHeat.F90:223-423, per cell; the block loop and EOS call are the
     * caller's. */
    int clamped = 0;
    for (int64_t c = 0; c < n; ++c) {
        orc_cool_vars v;
        memset(&v, 0, sizeof v);
        orc_cool_diag d;
        memset(&d, 0, sizeof d);
        double tmp = temp[c];
        v.rho = dens[c];
        double ei = eint[c];
        v.tdust = tdus[c];
        v.xHp = xhp ? xhp[c] : 1e-4;
        double ek = 0.0;
        if (velx && vely && velz)
            ek = 0.5e0 * (velx[c] * velx[c] + vely[c] * vely[c] + velz[c] * velz[c]);
        v.ephen = phhe ? phhe[c] : 0.0;
        v.ephen = v.ephen / v.rho;
        v.Gflux = pefl ? pefl[c] : 0.0;
        v.mu_mol = p->mu_mol;
        v.strat_factor = 1.0;
        orc_heating_and_cooling(p, t, &v, &ei, dt, &tmp, &d);
        int flags = 0;
        if (tmp > p->absTmax) {
            ei = p->absTmax * v.TtoEI;
            tmp = p->absTmax;
            clamped++;
            flags |= 1;
        }
        if (ei < p->smallp / dens[c]) ei = p->smallp / dens[c];
        ener[c] = ei + ek;
        eint[c] = ei;
        temp[c] = tmp;
        tdus[c] = v.tdust;
        if (phhe) phhe[c] = 0.0;
        if (pefl) pefl[c] = 0.0;
        if (d.bracket_fail) flags |= 2;
        if (d.zero_unbracketed) flags |= 4;
        if (d.zero_maxiter) flags |= 8;
        if (d.dust_noconv) flags |= 16;
        if (d.early_euler) flags |= 32;
        if (ncount_out) ncount_out[c] = d.brent_iters;
        if (flags_out) flags_out[c] = flags;
    }
    return clamped;
}
