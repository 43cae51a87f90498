// Per-cell heating/cooling solver on the device (FP64).
//
// Device restatement of heating_and_cooling's "Implicit" branch and the
// rate terms it calls, from
//   src/flash/source/physics/sourceTerms/Heat/HeatMain/HeatCool/phenHeat/
//   mol_and_dust/solver/heatCool.F90
// Operand order follows the Fortran; the file that includes this header is
// compiled with -fmad=false so rounding matches a plain -O2 Fortran build
// except where CUDA's pow/exp differ from the host libm by an ulp. Every
// loop has the Fortran's iteration cap; where the Fortran prints and stops
// the device records a status code and returns a defined value.
#pragma once

#include "gb_common.cuh"
#include "cool_types.cuh"
#include "cool_f32.cuh"

namespace gbcool {

__device__ __forceinline__ double fmx(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double fmn(double a, double b) { return a < b ? a : b; }

__device__ __forceinline__ double lin_interp(double x1, double y1, double x2, double y2, double x)
{
    // heatCool.F90:2379-2392
    double ms = (y2 - y1) / (x2 - x1);
    return ms * (x - x1) + y1;
}

__device__ __forceinline__ int find(const double* x, double x0, int N)
{
    // find.F90:9-42 (1-based result)
    if (x0 < __ldg(x)) return 0;
    if (x0 > __ldg(x + N - 1)) return N;
    int il = 1, ir = N;
    while (ir != il + 1) {
        int im = (il + ir) / 2;
        if (__ldg(x + im - 1) > x0) ir = im;
        else il = im;
    }
    return il;
}

static __device__ double radloss(double T)
{
    // heatCool.F90:1590-1667
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

__device__ __forceinline__ double lam_jeans(const gb_cool_params& p, double rho, double n, double T)
{
    // heatCool.F90:1687
    const double pi = 3.1415926535897932384, newton = 6.6725985e-8;
    return 1.0 / (rho / n) * sqrt(5. / 3. * pi * p.boltz * T / n / newton);
}

__device__ __forceinline__ double f_ext(const gb_cool_params& p, double rho, double n, double T)
{
    // heatCool.F90:1693-1722
    double lam_j = lam_jeans(p, rho, n, T);
    double Av = lam_j * n * 0.01 / 1.87e21;
    return exp(-3.5 * Av);
}

static __device__ double heating(const gb_cool_params& p, double T, double n, double rho, double strat)
{
    // heatCool.F90:890-964
    double eplus = 0.0, lin;
    if ((T <= p.theatmax) && (T >= p.theatmin)) {
        if (p.use_cr_heating) {
            if (p.crIonNH == 1.0 && p.crIonExp == 1.0) {
                eplus = strat * p.crIonRate * p.crIonEnergy / (rho / n);
            } else {
                double ncol = lam_jeans(p, rho, n, T) * n;
                eplus = strat * (p.crIonRate * p.crIonEnergy *
                                 pow(fmx(p.crIonNH, ncol) / p.crIonNH, -p.crIonExp)) /
                        (rho / n);
            }
        }
        double ll = p.theatmin, ll10 = ll + 0.1 * ll;
        double ul = p.theatmax, ul10 = ul - 0.1 * ul;
        if (T >= ul10) lin = lin_interp(ul10, 1.0, ul, 0.0, T);
        else if (T <= ll10) lin = lin_interp(ll, 0.0, ll10, 1.0, T);
        else lin = 1.0;
        eplus = eplus * lin;
    }
    return eplus;
}

static __device__ void pe_heating(const gb_cool_params& p, double G, double xHp, double n, double T,
                           double rho, double* PeHeat, double* dust_heating)
{
    // heatCool.F90:970-1110
    const double C0 = 7.64, C1 = 4.52, C2 = 0.04371, C3 = 0.00557, C4 = 0.132, C5 = 0.452,
                 C6 = 0.675;
    *PeHeat = 0.0;
    *dust_heating = 0.0;
    if ((T <= fmn(p.theatmax, p.dust_sputter_temp)) && (T >= p.theatmin)) {
        double xl = (xHp == 0.0) ? 1e-8 : xHp;
        double Gfactor, eff;
        if (p.pe_recipe == 1) {
            Gfactor = G * sqrt(T) / (xl * n * 0.5);
            eff = 4.9e-2 / (1.0 + 4.0e-3 * pow(Gfactor, 0.73)) +
                  (3.7e-2 * pow(T / 1.0e4, 0.7)) / (1.0 + 2.0e-4 * Gfactor);
            *PeHeat = p.pe_norm * eff * G / (rho / n);
            *dust_heating = p.pe_norm * fmx(0.0, (1.0 - eff)) * G * n;
        } else if (p.pe_recipe == 0) {
            Gfactor = G * sqrt(T) / (xl * n);
            eff = (C0 + C1 * pow(T, C4)) / (1.0 + (C2 * pow(Gfactor, C5)) * (1.0 + C3 * pow(Gfactor, C6)));
            *PeHeat = 1e-26 * eff * G / (rho / n);
            *dust_heating = (p.pe_norm - 1e-26 * eff) * G * n;
            *dust_heating = fmx(*dust_heating, 0.0);
        } else {
            eff = 0.05;
            *PeHeat = p.pe_norm * eff * G / (rho / n);
            *dust_heating = p.pe_norm * (1.0 - eff) * G * n;
        }
        double ll = p.theatmin, ll10 = ll + 0.1 * ll;
        double ul = fmn(p.theatmax, p.dust_sputter_temp), ul10 = ul - 0.1 * ul, lin;
        if (T >= ul10) lin = lin_interp(ul10, 1.0, ul, 0.0, T);
        else if (T <= ll10) lin = lin_interp(ll, 0.0, ll10, 1.0, T);
        else lin = 1.0;
        *PeHeat = *PeHeat * lin;
    }
}

static __device__ double cooling(const gb_cool_params& p, double T, double n, double conf, double xHp)
{
    // heatCool.F90:1116-1200
    double emin = 0.0;
    if ((T <= p.tradmax && T >= p.tradmin) && (n >= p.dradmin && n <= p.dradmax)) {
        emin = radloss(T);
        if (xHp > 1e-2 && T < 1.2e4) {
            double DG = lin_interp(1e-2, 1.0, 1e-1, 5.0, fmn(1e-1, xHp));
            emin = emin * DG;
            if (T > 1e4) {
                double q = lin_interp(1e4, 1.0, 1.2e4, pow(DG, 0.5), T);
                emin = emin / (q * q);
            }
        } else if (xHp < 1e-2 && T < 1e4) {
            double DG = lin_interp(1e-4, 0.35, 1e-2, 1.0, fmx(1e-4, xHp));
            emin = emin * DG;
            if (T > 9e3) emin = emin / lin_interp(9e3, 1.0, 1e4, DG, T);
        }
        double ll = p.tradmin, ll10 = ll + 0.1 * ll;
        double ul = p.tradmax, ul10 = ul - 0.1 * ul, lin;
        if (T >= ul10) lin = lin_interp(ul10, 1.0, ul, 0.0, T);
        else if (T <= ll10) lin = lin_interp(ll, 0.0, ll10, 1.0, T);
        else lin = 1.0;
        emin = emin * lin;
        emin = emin * conf;
    }
    return emin;
}

static __device__ double molecular_cooling(const gb_cool_ctx& c, double n, double T, double mu)
{
    // heatCool.F90:1211-1303
    const gb_cool_params& p = c.p;
    double cool_pw = 0.0;
    if ((n >= p.nd_cool_min) && (n <= p.nd_cool_max) && (T >= p.T_cool_min) && (T <= p.theatmax)) {
        int ixtemp = find(c.T, fmx(T, c.T_min), GB_TEMP_PTS);
        int ixdens = find(c.n, fmx(n, c.nd_min), GB_DENS_PTS);
        if (ixtemp > 0 && ixtemp <= GB_TEMP_PTS && ixdens > 0 && ixdens <= GB_DENS_PTS)
            cool_pw = __ldg(c.lam + (ixdens - 1) + GB_DENS_PTS * (ixtemp - 1)) / (mu * p.mp);
        double ll = p.T_cool_min, ll10 = ll + 0.1 * ll;
        double ul = p.theatmax, ul10 = ul - 0.1 * ul, lin;
        if (T >= ul10) lin = lin_interp(ul10, 1.0, ul, 0.0, T);
        else if (T <= ll10) lin = lin_interp(ll, 0.0, ll10, 1.0, T);
        else lin = 1.0;
        cool_pw = cool_pw * lin;
        ll = p.nd_cool_min; ll10 = ll + 0.1 * ll;
        ul = p.nd_cool_max; ul10 = ul - 0.1 * ul;
        if (n >= ul10) lin = lin_interp(ul10, 1.0, ul, 0.0, n);
        else if (n <= ll10) lin = lin_interp(ll, 0.0, ll10, 1.0, n);
        else lin = 1.0;
        cool_pw = cool_pw * lin;
    }
    return cool_pw;
}

__device__ __forceinline__ double dust_cooling(const gb_cool_params& p, double n, double T,
                                               double tdust, double rho)
{
    // heatCool.F90:1305-1390
    double cool_dg = 0.0;
    if (T <= p.dust_sputter_temp) {
        double lambda_gd = 3.8e-33 * (n * n) * (1.0 - 0.8 * exp(-75.0 / T)) * (T - tdust) * sqrt(T);
        cool_dg = lambda_gd / rho;
        double ul = p.dust_sputter_temp, ul10 = ul - 0.1 * ul, lin;
        if (T >= ul10) lin = lin_interp(ul10, 1.0, ul, 0.0, T);
        else lin = 1.0;
        cool_dg = cool_dg * lin;
    }
    return cool_dg;
}

// The state-independent part of dei_dt: cooling evaluated at the floors
// (heatCool.F90:1509-1519). It depends only on ndens/conf, so it is
// computed once per cell; the value is identical to recomputing it.
__device__ __forceinline__ double cooling_floor(const gb_cool_ctx& c, const gb_cool_vars& v)
{
    double emin = cooling(c.p, c.p.tradmin, v.ndens, v.conf, v.xHp);
    double pw = 0.0;
    if (c.p.useDustCool) pw = molecular_cooling(c, v.ndens, c.p.T_cool_min, v.mu_mol);
    return emin + pw;
}

static __device__ double dei_dt(const gb_cool_ctx& c, const gb_cool_vars& v, double floor_, double ei_in)
{
    // heatCool.F90:1397-1588
    const gb_cool_params& p = c.p;
    double tmp_temp = ei_in / v.TtoEI;
    if (tmp_temp < 0.0) tmp_temp = 1.0;
    double eplus = heating(p, tmp_temp, v.ndens, v.rho, v.strat_factor);
    double fuv = v.Gflux + p.Gzero * f_ext(p, v.rho, v.ndens, tmp_temp) * v.strat_factor;
    double PeHeat, dust_heating;
    pe_heating(p, fuv, v.xHp, v.ndens, tmp_temp, v.rho, &PeHeat, &dust_heating);
    eplus = eplus + v.ephen;
    double emin = cooling(p, tmp_temp, v.ndens, v.conf, v.xHp);
    double cool_pw = 0.0, cool_dg = 0.0;
    if (p.useDustCool) {
        cool_pw = molecular_cooling(c, v.ndens, tmp_temp, v.mu_mol);
        cool_dg = dust_cooling(p, v.ndens, tmp_temp, v.tdust, v.rho);
    }
    return eplus + PeHeat - emin - cool_pw - cool_dg + floor_;
}

// dei_dt split into its heating part (Gamma) and cooling part (Lambda):
// Gamma = CR + stellar + photoelectric heating + the floor term + any gas
// heating by warmer dust, Lambda = atomic + molecular + dust cooling. The
// return value is dei_dt itself, summed in dei_dt's order.
static __device__ double dei_parts(const gb_cool_ctx& c, const gb_cool_vars& v, double floor_, double ei_in,
                                   double* gam, double* lam)
{
    const gb_cool_params& p = c.p;
    double tmp_temp = ei_in / v.TtoEI;
    if (tmp_temp < 0.0) tmp_temp = 1.0;
    double eplus = heating(p, tmp_temp, v.ndens, v.rho, v.strat_factor);
    double fuv = v.Gflux + p.Gzero * f_ext(p, v.rho, v.ndens, tmp_temp) * v.strat_factor;
    double PeHeat, dust_heating;
    pe_heating(p, fuv, v.xHp, v.ndens, tmp_temp, v.rho, &PeHeat, &dust_heating);
    eplus = eplus + v.ephen;
    double emin = cooling(p, tmp_temp, v.ndens, v.conf, v.xHp);
    double cool_pw = 0.0, cool_dg = 0.0;
    if (p.useDustCool) {
        cool_pw = molecular_cooling(c, v.ndens, tmp_temp, v.mu_mol);
        cool_dg = dust_cooling(p, v.ndens, tmp_temp, v.tdust, v.rho);
    }
    *gam = eplus + PeHeat + floor_ + fmx(-cool_dg, 0.0);
    *lam = emin + cool_pw + fmx(cool_dg, 0.0);
    return eplus + PeHeat - emin - cool_pw - cool_dg + floor_;
}

template <int FORM = 0>
static __device__ double get_dust_temperature(const gb_cool_params& p, double tdust_in, double temp_in,
                                       double nden, double phen_heat, gb_cool_diag* d)
{
    // heatCool.F90:703-884; the gas temperature is fixed during the Newton
    // iterations, so its collision factor and square root are formed once
    // (the same values). FORM >= 1: T_dust^6 as a product instead of pow.
    const double tol = 1.e-4, smallt = .1;
    double error = 10. * tol;
    double tdust = tdust_in;
    if (tdust < p.absTmin) tdust = p.absTmin;
    double tg = (temp_in < p.absTmin) ? p.absTmin : temp_in;
    const double acoll = 3.8 * nden * (1.0 - 0.8 * exp(-75.0 / tg)), sq = sqrt(tg);
    int l = 1;
    while ((l <= 100) && (error > tol)) {
        double t6;
        if (FORM >= 1) {
            const double t2 = tdust * tdust;
            t6 = t2 * t2 * t2;
        } else {
            t6 = pow(tdust, 6.0);
        }
        double lambda_dust = 6.8 * t6;
        double coll = acoll * (tg - tdust) * sq;
        double eqfunc = phen_heat + coll - lambda_dust;
        double det = -(6.0 * lambda_dust / tdust) - acoll * sq;
        double tnew = tdust - eqfunc / det;
        error = fabs(tnew - tdust) / tdust;
        tdust = tnew;
        if (tdust < smallt) {
            tdust = smallt;
            error = 0.1 * tol;
        }
        l = l + 1;
    }
    if (l > 100) d->dust_noconv = 1;
    if (tdust < p.absTmin) tdust = p.absTmin;
    return tdust;
}

template <int FORM = 0>
static __device__ void dust_update(const gb_cool_ctx& c, gb_cool_vars& v, double temp, gb_cool_diag* d)
{
    // heatCool.F90:430-443
    const gb_cool_params& p = c.p;
    double fuv = v.Gflux + p.Gzero * f_ext(p, v.rho, v.ndens, temp) * v.strat_factor;
    double PeHeat, dust_heat;
    pe_heating(p, fuv, v.xHp, v.ndens, temp, v.rho, &PeHeat, &dust_heat);
    double cr = heating(p, temp, v.ndens, v.rho, v.strat_factor);
    cr = cr * v.rho;
    dust_heat = dust_heat + cr;
    dust_heat = dust_heat / (v.ndens * 1e-33);
    v.tdust = get_dust_temperature<FORM>(p, v.tdust, temp, v.ndens, dust_heat, d);
}

// ---- dei_dt restated for the mixed path (FR): the same rate terms with
// the transcendentals shared. Per evaluation one ln T and one sqrt(T);
// every power x^a becomes exp(a ln x); the column density (Jeans length
// times n, proportional to sqrt(T)) and the FUV field's logarithm (the
// shielding exponent when no external flux is given) come from per-cell
// constants. Algebraically the reference's rates; they round differently
// by a few ulp, which moves the implicit solve by far less than its
// tolerance.
struct fr_consts {
    double kJ;     // column density = kJ sqrt(T)
    double lnK;    // ln(column / crIonNH) - ln(T) / 2
    double lnG0;   // ln(Gzero strat) (used when Gflux == 0)
    double lnxn;   // ln(x_l n): the photoelectric grain-charging denominator
    double rn;     // rho / n
    // FORM 2: the cell's state and the cooling at the floors in FP32, and
    // the FP32 tables
    gb_cool_varsf vf;
    float fl32;
    gb_cool_tabf tf;
};

__device__ __forceinline__ fr_consts make_fr(const gb_cool_params& p, const gb_cool_vars& v)
{
    const double pi = 3.1415926535897932384, newton = 6.6725985e-8;
    fr_consts f;
    f.rn = v.rho / v.ndens;
    f.kJ = sqrt(5. / 3. * pi * p.boltz / v.ndens / newton) / f.rn * v.ndens;
    f.lnK = log(f.kJ) - log(p.crIonNH);
    f.lnG0 = log(p.Gzero * v.strat_factor);
    const double xl = (v.xHp == 0.0) ? 1e-8 : v.xHp;
    f.lnxn = log(xl * v.ndens);
    return f;
}

// FORM 2 (the plain integrator on FP32 rates): the backward-Euler residual
// and Brent's and zbrac's iterates stay FP64; only the rate function de/dt
// runs in FP32 (gbcoolf::dei_parts with the library's exp/log), from the
// cell's state converted once. The rate's relative error, about 1e-6 (1e-5
// on the steepest power law), moves the residual's root by far less than
// Brent's stopping tolerance max(TtoEI * 1 K, 1e-6 e) in most cells.
__device__ __forceinline__ void make_fr32(const gb_cool_ctx& c, const gb_cool_vars& v, fr_consts& f)
{
    gbcoolf::make_vars(c.pf, v, f.vf);
    f.tf = gb_cool_tabf{c.Tf, c.nf, c.lamf, gb_d2f(c.T_min), gb_d2f(c.nd_min)};
    f.fl32 = gbcoolf::cooling_floor<true>(c.pf, f.tf, f.vf);
}

// the dust temperature after the step (heatCool.F90:430-443): FORM 2 in
// FP32 (the same dust heating and Newton iteration, gbcoolf::dust_temperature)
template <int FORM>
__device__ __forceinline__ void dust_after_step(const gb_cool_ctx& c, gb_cool_vars& v, const fr_consts& f, double temp,
                                                gb_cool_diag* d)
{
    if (FORM == 2) v.tdust = gb_f2d(gbcoolf::dust_temperature<true>(c.pf, f.vf, gb_d2f(temp), gb_d2f(v.tdust)));
    else dust_update<FORM>(c, v, temp, d);
}

// radloss (heatCool.F90:1590-1667) from ln T and sqrt(T)
__device__ __forceinline__ double radloss_fr(double T, double lnT, double sqT)
{
    double radia;
    if (T >= 1.70e4) {
        if (T >= 5.62e5) {
            if (T >= 2.75e6) {
                if (T >= 3.16e7) radia = 3.090e-27 * sqT;
                else radia = 5.188e-21 * exp(-0.33 * lnT);
            } else {
                if (T >= 1.78e6) radia = 3.890e-4 * exp(-2.95 * lnT);
                else radia = 1.3e-22 * exp(0.01 * (lnT - 11.918390573078392));  // (T / 1.5e5)^0.01
            }
        } else {
            if (T >= 7.94e4) {
                if (T >= 2.51e5) radia = 3.98e-11 / (T * T);
                else radia = 6.31e-22 * exp(0.01 * (lnT - 13.815510557964274));  // (T / 1e6)^0.01
            } else {
                if (T >= 3.98e4) radia = 1.e-31 * (T * T);
                else radia = 1.479e-21 * exp(-0.216 * lnT);
            }
        }
    } else {
        if (T >= 1.e3) {
            if (T >= 6.31e3) {
                if (T >= 1.0e4) radia = 7.63e-81 * exp(13.8 * lnT);
                else radia = 3.13e-27 * exp(0.396 * lnT);
            } else {
                if (T >= 3.16e3) radia = 2.64e-26 * exp(0.152 * lnT);
                else radia = 5.28e-27 * exp(0.352 * lnT);
            }
        } else {
            if (T >= 3.98e1) {
                if (T >= 2.00e2) radia = 3.06e-27 * exp(0.431 * lnT);
                else radia = 1.52e-28 * exp(0.997 * lnT);
            } else {
                if (T >= 2.51e1) radia = 2.39e-29 * (T * sqT);
                else radia = 1.095e-32 * exp(3.885 * lnT);
            }
        }
    }
    return radia;
}

__device__ __forceinline__ double ramp(double x, double ll, double ul)
{
    const double ll10 = ll + 0.1 * ll, ul10 = ul - 0.1 * ul;
    if (x >= ul10) return lin_interp(ul10, 1.0, ul, 0.0, x);
    if (x <= ll10) return lin_interp(ll, 0.0, ll10, 1.0, x);
    return 1.0;
}

static __device__ double dei_dt_fr(const gb_cool_ctx& c, const gb_cool_vars& v, const fr_consts& f, double floor_,
                                   double ei_in)
{
    const gb_cool_params& p = c.p;
    double T = ei_in / v.TtoEI;
    if (T < 0.0) T = 1.0;
    const double lnT = log(T), sqT = sqrt(T);
    const double ncol = f.kJ * sqT;
    const double Av = ncol * 0.01 / 1.87e21;
    // CR heating (heatCool.F90:890-964)
    double eplus = 0.0;
    if ((T <= p.theatmax) && (T >= p.theatmin)) {
        if (p.use_cr_heating) {
            if (p.crIonNH == 1.0 && p.crIonExp == 1.0) {
                eplus = v.strat_factor * p.crIonRate * p.crIonEnergy / f.rn;
            } else {
                const double L = 0.5 * lnT + f.lnK;  // ln(column / NH)
                const double pw = L > 0.0 ? exp(-p.crIonExp * L) : 1.0;
                eplus = v.strat_factor * (p.crIonRate * p.crIonEnergy * pw) / f.rn;
            }
        }
        eplus = eplus * ramp(T, p.theatmin, p.theatmax);
    }
    // photoelectric heating, WD01 (:970-1110), with the shielded FUV field
    const double fext = exp(-3.5 * Av);
    const double fuv = v.Gflux + p.Gzero * fext * v.strat_factor;
    double PeHeat = 0.0;
    if (p.pe_recipe != 0) {
        double dh;
        pe_heating(p, fuv, v.xHp, v.ndens, T, v.rho, &PeHeat, &dh);
    } else if ((T <= fmn(p.theatmax, p.dust_sputter_temp)) && (T >= p.theatmin)) {
        const double C0 = 7.64, C1 = 4.52, C2 = 0.04371, C3 = 0.00557, C4 = 0.132, C5 = 0.452, C6 = 0.675;
        double den = 1.0;
        if (fuv > 0.0) {
            const double lnfuv = v.Gflux == 0.0 ? f.lnG0 - 3.5 * Av : log(fuv);
            const double lnGf = lnfuv + 0.5 * lnT - f.lnxn;
            den = 1.0 + (C2 * exp(C5 * lnGf)) * (1.0 + C3 * exp(C6 * lnGf));
        }
        const double eff = (C0 + C1 * exp(C4 * lnT)) / den;
        PeHeat = 1e-26 * eff * fuv / f.rn;
        PeHeat = PeHeat * ramp(T, p.theatmin, fmn(p.theatmax, p.dust_sputter_temp));
    }
    eplus = eplus + v.ephen;
    // atomic cooling (:1116-1200)
    double emin = 0.0;
    if ((T <= p.tradmax && T >= p.tradmin) && (v.ndens >= p.dradmin && v.ndens <= p.dradmax)) {
        emin = radloss_fr(T, lnT, sqT);
        if (v.xHp > 1e-2 && T < 1.2e4) {
            double DG = lin_interp(1e-2, 1.0, 1e-1, 5.0, fmn(1e-1, v.xHp));
            emin = emin * DG;
            if (T > 1e4) {
                double q = lin_interp(1e4, 1.0, 1.2e4, sqrt(DG), T);
                emin = emin / (q * q);
            }
        } else if (v.xHp < 1e-2 && T < 1e4) {
            double DG = lin_interp(1e-4, 0.35, 1e-2, 1.0, fmx(1e-4, v.xHp));
            emin = emin * DG;
            if (T > 9e3) emin = emin / lin_interp(9e3, 1.0, 1e4, DG, T);
        }
        emin = emin * ramp(T, p.tradmin, p.tradmax);
        emin = emin * v.conf;
    }
    double cool_pw = 0.0, cool_dg = 0.0;
    if (p.useDustCool) {
        cool_pw = molecular_cooling(c, v.ndens, T, v.mu_mol);
        if (T <= p.dust_sputter_temp) {
            const double lambda_gd = 3.8e-33 * (v.ndens * v.ndens) * (1.0 - 0.8 * exp(-75.0 / T)) * (T - v.tdust) * sqT;
            const double ul = p.dust_sputter_temp, ul10 = ul - 0.1 * ul;
            cool_dg = lambda_gd / v.rho * (T >= ul10 ? lin_interp(ul10, 1.0, ul, 0.0, T) : 1.0);
        }
    }
    return eplus + PeHeat - emin - cool_pw - cool_dg + floor_;
}

template <int FORM>
__device__ __forceinline__ double rate(const gb_cool_ctx& c, const gb_cool_vars& v, const fr_consts& f,
                                       double floor_, double y)
{
    if (FORM == 2) {
        float gam, lam;
        return gb_f2d(gbcoolf::dei_parts<true>(c.pf, f.tf, f.vf, f.fl32, gb_d2f(y), &gam, &lam));
    }
    if (FORM == 1) return dei_dt_fr(c, v, f, floor_, y);
    return dei_dt(c, v, floor_, y);
}

template <int FORM = 0>
__device__ __forceinline__ double one_step(const gb_cool_ctx& c, const gb_cool_vars& v, const fr_consts& f,
                                           double floor_, double dx, double y, double yold)
{
    // heatCool.F90:1928-1950
    return y - dx * rate<FORM>(c, v, f, floor_, y) - yold;
}

// |a| < |b| and friends on the integer pipe: for non-NaN doubles the
// magnitudes order as their bit patterns without the sign bit, and the
// sign tests read the sign bit, so these take exactly FP64's decisions
__device__ __forceinline__ unsigned long long mag_bits(double x)
{
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ bool pos_bits(double x) { return __double_as_longlong(x) > 0; }

template <int FORM = 0>
static __device__ double zero(const gb_cool_ctx& c, const gb_cool_vars& v, const fr_consts& f, double floor_,
                       double a, double b, double a_old, double machep, double tt, double dt,
                       gb_cool_diag* d)
{
    // heatCool.F90:1981-2197 (Brent). FORM 2 (the mixed path's integrator on
    // FP32 rates) takes every comparison on the integer pipe (the same
    // decisions) and forms the inverse-quadratic / secant trial step in FP32
    // (a trial point a few ulp of FP32 from FP64's, which Brent's own
    // acceptance test and bisection fallback then treat alike); the iterates,
    // the bracket and the tolerance stay FP64.
    double sa = a, sb = b;
    double fa = 0.0, fb = 0.0;
#pragma unroll 1
    for (int i = 0; i < 2; ++i) {  // one call site for both (see zbrac)
        const double fv = one_step<FORM>(c, v, f, floor_, dt, i == 0 ? sa : sb, a_old);
        if (i == 0) fa = fv;
        else fb = fv;
    }
    double cc = sa, fc = fa, e = sb - sa, dd = e;
    int n_tries = 0;
    if ((fa > 0.0 && fb > 0.0) || (fa < 0.0 && fb < 0.0)) {
        d->unbracketed = 1;
        return sb;
    }
    for (;;) {
        if (FORM == 2 ? mag_bits(fc) < mag_bits(fb) : fabs(fc) < fabs(fb)) {
            sa = sb; sb = cc; cc = sa;
            fa = fb; fb = fc; fc = fa;
        }
        double tol = 2.0 * machep * fabs(sb) + tt;
        double m = 0.5 * (cc - sb);
        if (FORM == 2) {
            if (mag_bits(m) <= mag_bits(tol) || mag_bits(fb) == 0ull) break;
        } else {
            if (fabs(m) <= tol || fb == 0.0) break;
        }
        if (FORM == 2 ? (mag_bits(e) < mag_bits(tol) || mag_bits(fa) <= mag_bits(fb))
                      : (fabs(e) < tol || fabs(fa) <= fabs(fb))) {
            e = m;
            dd = e;
        } else if (FORM == 2) {
            const float faf = gb_d2f(fa), fbf = gb_d2f(fb), fcf = gb_d2f(fc), mf = gb_d2f(m);
            float s = fbf / faf, pp, q, r;
            if (sa == cc) {
                pp = 2.0f * mf * s;
                q = 1.0f - s;
            } else {
                q = faf / fcf;
                r = fbf / fcf;
                pp = s * (2.0f * mf * q * (q - r) - gb_d2f(sb - sa) * (r - 1.0f));
                q = (q - 1.0f) * (r - 1.0f) * (s - 1.0f);
            }
            if (0.0f < pp) q = -q;
            else pp = -pp;
            const float sf = gb_d2f(e);
            e = dd;
            // non-finite FP32 intermediates fail the test: bisection
            if (2.0f * pp < 3.0f * mf * q - fabsf(gb_d2f(tol) * q) && pp < fabsf(0.5f * sf * q)) {
                dd = gb_f2d(pp / q);
            } else {
                e = m;
                dd = e;
            }
        } else {
            double s = fb / fa, pp, q, r;
            if (sa == cc) {
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
        if (FORM == 2 ? mag_bits(tol) < mag_bits(dd) : tol < fabs(dd)) sb = sb + dd;
        else if (FORM == 2 ? pos_bits(m) : 0.0 < m) sb = sb + tol;
        else sb = sb - tol;
        fb = one_step<FORM>(c, v, f, floor_, dt, sb, a_old);
        if (FORM == 2 ? pos_bits(fb) == pos_bits(fc)
                      : ((0.0 < fb && 0.0 < fc) || (fb <= 0.0 && fc <= 0.0))) {
            cc = sa;
            fc = fa;
            e = sb - sa;
            dd = e;
        }
        n_tries = n_tries + 1;
        if (n_tries > 10000) {
            d->maxiter = 1;
            break;
        }
    }
    d->iters = n_tries;
    return sb;
}

template <int FORM = 0>
static __device__ int zbrac(const gb_cool_ctx& c, const gb_cool_vars& v, const fr_consts& f, double floor_,
                     double* x1, double* x2, double xold, double dt)
{
    // heatCool.F90:2294-2348
    // FORM 2 takes the sign and magnitude tests on the integer pipe (the
    // same decisions: a product of two energies-sized residuals never
    // underflows, so f1 f2 < 0 is opposite nonzero signs)
    // The residual is evaluated at one call site in the loop (and one for
    // the two starting points): the rate function is long, and copies of it
    // at every call site overflowed the instruction cache.
    const double FACTOR = 1.6;
    double f1 = 0.0, f2 = 0.0;
#pragma unroll 1
    for (int i = 0; i < 2; ++i) {
        const double fv = one_step<FORM>(c, v, f, floor_, dt, i == 0 ? *x1 : *x2, xold);
        if (i == 0) f1 = fv;
        else f2 = fv;
    }
    for (int j = 1; j <= 5000; ++j) {
        if (FORM == 2 ? (((__double_as_longlong(f1) ^ __double_as_longlong(f2)) < 0) && mag_bits(f1) != 0ull &&
                         mag_bits(f2) != 0ull)
                      : f1 * f2 < 0.0)
            return 1;
        const bool first = FORM == 2 ? mag_bits(f1) < mag_bits(f2) : fabs(f1) < fabs(f2);
        double xn = first ? *x1 + FACTOR * (*x1 - *x2) : *x2 + FACTOR * (*x2 - *x1);
        if (FORM == 2 ? __double_as_longlong(xn) < 0 && mag_bits(xn) != 0ull : xn < 0.0) xn = v.TtoEI * 1.0;
        const double fn = one_step<FORM>(c, v, f, floor_, dt, xn, xold);
        if (first) {
            *x1 = xn;
            f1 = fn;
        } else {
            *x2 = xn;
            f2 = fn;
        }
    }
    return 0;
}

// heating_and_cooling, "Implicit" (default) or "Euler" branch, for one
// cell. v must hold rho, Gflux, ephen, tdust, xHp, strat_factor, mu_mol.
template <int FORM = 0>
static __device__ void heating_and_cooling(const gb_cool_ctx& c, gb_cool_vars& v, double* ei_io,
                                    double timestep, double* temp_io, gb_cool_diag* d)
{
    const gb_cool_params& p = c.p;
    const double err_tol = 1e-6;
    double ei = *ei_io, temp = *temp_io;
    double total_time = 0.0;
    v.ndens = v.rho / (v.mu_mol * p.mp);
    v.TtoEI = ei / temp;
    v.conf = v.ndens * v.ndens / v.rho;
    // FORM 2 forms the floors' cooling in FP32 with its rates
    double fl = FORM == 2 ? 0.0 : cooling_floor(c, v);
    fr_consts frc;
    if (FORM == 1) frc = make_fr(p, v);
    if (FORM == 2) make_fr32(c, v, frc);
    if (p.int_method == 1) {
        // Euler, heatCool.F90:119-214
        int ncount = 0;
        for (;;) {
            double dei = rate<FORM>(c, v, frc, fl, ei);
            double dt1 = p.subfactor * ei / fmx(fabs(dei), 1e-50);
            double dt0 = fmn((timestep - total_time), dt1);
            ei = ei + dei * dt0;
            temp = ei / v.TtoEI;
            total_time = total_time + dt0;
            ncount = ncount + 1;
            if (ncount > 100000) break;
            if ((timestep - total_time) < 1e-6) break;
        }
        if (temp < p.absTmin) {
            temp = p.absTmin;
            ei = p.absTmin * v.TtoEI;
        }
        if (p.useDustCool && temp <= p.dust_sputter_temp)
            v.tdust = get_dust_temperature<FORM>(p, v.tdust, temp, v.ndens, 0.0, d);
    } else {
        // Implicit, heatCool.F90:216-514 (one pass: dt0 = timestep)
        while ((timestep - total_time) > (1e-6 * timestep)) {
            double eiolder = ei;
            double eiold = ei;
            double dei = rate<FORM>(c, v, frc, fl, eiold);
            double dt0 = timestep;
            eiold = eiolder + dei * dt0 * 1.0e-3;
            double ei1 = eiolder, ei2 = eiold;
            if (fabs((ei1 - ei2) / ei1) < (err_tol * dt0 / (timestep - total_time))) {
                dt0 = (timestep - total_time);
                ei = eiolder + dei * dt0;
                temp = ei / v.TtoEI;
                if (p.useDustCool && temp <= p.dust_sputter_temp) dust_after_step<FORM>(c, v, frc, temp, d);
                total_time = total_time + dt0;
                continue;
            }
            int found = zbrac<FORM>(c, v, frc, fl, &ei1, &ei2, eiolder, dt0);
            if (!found) d->bracket_fail = 1;
            if (ei1 < 0.0 || ei2 < 0.0) {
                ei1 = fmx(ei1, v.TtoEI * 1.0);
                ei2 = fmx(ei2, v.TtoEI * 1.0);
            }
            if (found)
                ei = zero<FORM>(c, v, frc, fl, ei1, ei2, eiolder, 3e-16, fmx(v.TtoEI * c.brent_tol_K, eiold * err_tol), dt0, d);
            else
                ei = zero<FORM>(c, v, frc, fl, v.TtoEI * 1.0, v.TtoEI * 1.0e9, eiolder, 3e-16,
                          fmx(v.TtoEI * c.brent_tol_K, eiold * err_tol), dt0, d);
            temp = ei / v.TtoEI;
            if (p.useDustCool && temp <= p.dust_sputter_temp) dust_after_step<FORM>(c, v, frc, temp, d);
            total_time = total_time + dt0;
        }
        if (temp < p.absTmin) {
            temp = p.absTmin;
            ei = p.absTmin * v.TtoEI;
        }
    }
    *ei_io = ei;
    *temp_io = temp;
}

}  // namespace gbcool
