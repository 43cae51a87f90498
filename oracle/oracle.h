/*
 * CPU oracle for the hydro/MHD + heating/cooling hot path.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product library links, loads or
 * calls this code; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it, as the reference the GPU results are compared against.
 *
 * Cooling part: a statement-level C restatement of the vendored Fortran
 *   src/flash/source/physics/sourceTerms/Heat/HeatMain/HeatCool/phenHeat/
 *     mol_and_dust/solver/heatCool.F90, RadHeat.F90,
 *     mol_and_dust/find.F90, get_cooling_data.F90, Cool_init.F90,
 *     phenHeat/Heat_init.F90
 * with every `real` as IEEE double (the reference builds with
 * -fdefault-real-8, support/Makefile.h.in:13) and this file compiled with
 * -O2 -ffp-contract=off so no fused multiply-adds change the rounding.
 *
 * Hydro part: see hydro_oracle.c.
 */
#ifndef GB_ORACLE_H
#define GB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_TEMP_PTS 320
#define ORC_DENS_PTS 190

/* Heat_data + Cool_data runtime parameters (phenHeat/Heat_data.F90,
 * mol_and_dust/Cool_data.F90). */
typedef struct orc_cool_params {
    double tradmin, tradmax, dradmin, dradmax;
    double theatmin, theatmax, absTmin, absTmax;
    double Gzero, subfactor, smallp;
    int use_cr_heating;
    double crIonRate, crIonNH, crIonExp, crIonEnergy; /* crIonEnergy already in erg */
    double dust_sputter_temp;
    int pe_recipe; /* 0 = WD01, 1 = BT94, 2 = NOGF */
    double pe_norm;
    double boltz, mp;
    double T_cool_min, nd_cool_min, nd_cool_max;
    int useDustCool;
    int int_method; /* 0 = Implicit, 1 = Euler, 2 = trap, 3 = RK4 (DoPr5) */
    double mu_mol;  /* RadHeat.F90:278 hard-codes 24/11 */
} orc_cool_params;

/* The molecular cooling table cool_dat(DENS_PTS, TEMP_PTS, 3) of
 * Cool_data.F90:27-29, stored as the two 1-D axes `find` searches plus the
 * power column. lambda[i_dens + DENS_PTS * i_temp] (0-based). */
typedef struct orc_table {
    double T[ORC_TEMP_PTS];     /* cool_dat(1, :, 1) */
    double n[ORC_DENS_PTS];     /* cool_dat(:, 1, 2) */
    double lambda[ORC_DENS_PTS * ORC_TEMP_PTS]; /* cool_dat(:, :, 3) */
    double T_min, nd_min;       /* Cool_init.F90:77-78 */
} orc_table;

/* Module variables of cool_vars (CoolVars.F90:7-8). */
typedef struct orc_cool_vars {
    double ndens, rho, conf, Gflux, ephen, tdust, TtoEI, xHp, strat_factor, mu_mol;
} orc_cool_vars;

/* Per-cell counters the Fortran prints instead of returning. */
typedef struct orc_cool_diag {
    int ncount;        /* heating_and_cooling's ncount */
    int bracket_fail;  /* zbrac gave up; absolute bracket used */
    int brent_iters;   /* iterations in `zero` */
    int dust_noconv;   /* get_dust_temperature hit max_newton */
    int early_euler;   /* the |ei1-ei2|/ei1 < tol explicit-Euler exit */
    int zero_unbracketed; /* `zero` entered without a sign change (Fortran stops) */
    int zero_maxiter;  /* `zero` exceeded max_iter (Fortran stops) */
} orc_cool_diag;

void orc_cool_default_params(orc_cool_params* p);

/* get_cooling_data.F90: parse a FLASH-format cool.dat. Returns 0 on success,
 * negative on open/format errors (the Fortran aborts). */
int orc_table_load_flash(orc_table* t, const char* path);
/* Build the table from log10 values given as integers in units of 1e-4
 * (lossless for the file's F8.4 fields). */
void orc_table_from_ilog(orc_table* t, const int32_t* logT_e4, const int32_t* logn_e4,
                         const int32_t* logL_e4);

int orc_find(const double* x, double x0, int N); /* find.F90:9-42, 1-based */
double orc_radloss(double T);                     /* heatCool.F90:1590-1667 */
/* dust_cooling, heatCool.F90:1305-1390: gas-dust cooling [erg/g/s] */
double orc_dust_cooling(const orc_cool_params* p, double n, double T, double tdust, double rho);
double orc_lin_interp(double x1, double y1, double x2, double y2, double x);

/* heating_and_cooling(ei, timestep, temp, ncount), heatCool.F90:41-700.
 * vars carries the cool_vars module state (rho, Gflux, ephen, tdust, xHp,
 * strat_factor, mu_mol in; ndens, conf, TtoEI, tdust out). */
void orc_heating_and_cooling(const orc_cool_params* p, const orc_table* t, orc_cool_vars* v,
                             double* ei, double timestep, double* temp, orc_cool_diag* d);

/* The per-cell body of RadHeat.F90:223-423 applied to n cells of plain
 * arrays. ener/eint/temp/tdus are updated in place; phhe/pefl are zeroed.
 * vel* may be NULL (ek = 0). Returns the number of cells clamped at absTmax. */
int orc_radheat_cells(const orc_cool_params* p, const orc_table* t, int64_t n, double dt,
                      const double* dens, const double* velx, const double* vely,
                      const double* velz, double* ener, double* eint, double* temp,
                      double* tdus, const double* xhp, double* phhe, double* pefl,
                      int* ncount_out, int* flags_out);

/* dei_dt at a given state (for tests of the rate function). */
double orc_dei_dt(const orc_cool_params* p, const orc_table* t, orc_cool_vars* v,
                  double t_in, double ei_in);

/* OdeInt.F90 DoPr5 driver, restated for the known-answer test in
 * IntegratorModule/test.f95 + test.dat. f(x, y) = x. Writes n_out rows of
 * (x_state, t) sampled every `dt_out`. Returns rows written. */
int orc_dopr5_line_kat(double atol, double rtol, double hmin, int have_hmax, double hmax,
                       double dt_out, double t_end, double* out_x, double* out_t, int n_out);

/* ---------------------------------------------------------------- hydro */
#include "hydro_oracle.h"

#ifdef __cplusplus
}
#endif
#endif
