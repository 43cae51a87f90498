// Types shared by the FP64 cooling solver (cool_dev.cuh) and its FP32 rate
// function (cool_f32.cuh).
#pragma once

#include "gb_common.cuh"

#define GB_TEMP_PTS 320
#define GB_DENS_PTS 190

// the runtime parameters in FP32, converted once on the host (values far
// below FP32's range, such as 1e-99, become 0, which leaves every
// comparison they take part in unchanged)
struct gb_cool_pf {
    float theatmin, theatmax, tradmin, tradmax, dradmin, dradmax, dust_sputter_temp;
    float Gzero, pe_norm, crIonExp, crIonNH, lnNH, crRE, T_cool_min, nd_cool_min, nd_cool_max, absTmin;
    float jeansK;  // 5/3 pi k_B / G_Newton (heatCool.F90:1687)
    int use_cr_heating, cr_uniform, pe_recipe, useDustCool;
};

struct gb_cool_ctx {
    gb_cool_params p;
    const double* T;    // cool_dat(1, :, 1), TEMP_PTS
    const double* n;    // cool_dat(:, 1, 2), DENS_PTS
    const double* lam;  // cool_dat(:, :, 3), dens fastest
    double T_min, nd_min;
    // Brent tolerance floor of the implicit step in kelvin (heatCool.F90
    // passes TtoEI * 1 K; other values are a diagnostic of that tolerance)
    double brent_tol_K;
    // FP32 copies for the FP32 rate function: axes, and cool_dat(:, :, 3)
    // divided by mu_mol m_p (the molecular power per gram)
    const float* Tf;
    const float* nf;
    const float* lamf;
    gb_cool_pf pf;
};

struct gb_cool_vars {
    double ndens, rho, conf, Gflux, ephen, tdust, TtoEI, xHp, strat_factor, mu_mol;
};

struct gb_cool_diag {
    int bracket_fail, dust_noconv, unbracketed, maxiter, iters;
};

struct gb_cool_tabf {
    const float* T;    // TEMP_PTS
    const float* n;    // DENS_PTS
    const float* lam;  // cool_dat(:, :, 3) / (mu_mol m_p): molecular power per gram
    float T_min, nd_min;
};

struct gb_cool_varsf {
    float ndens, rho, conf, Gflux, ephen, tdust, TtoEI, xHp, mu_mol;
    float cr_pref;  // strat * crIonRate * crIonEnergy / (rho / n)
};
