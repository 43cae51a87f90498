/*
 * FLOP-counting build of the oracle. TEST INFRASTRUCTURE ONLY (see
 * oracle.h): it measures the arithmetic of the hot path per zone-update, it
 * is not the product and nothing in the product links it.
 *
 * The C restatement (hydro_oracle.c, cool_oracle.c) is compiled as C++ with
 * `double` replaced by `cdouble`, a one-field wrapper with the same size
 * and alignment whose operators count: + and - (add), * (mul), / (div),
 * sqrt; exp, log, pow as transcendentals. Negation, fabs, fmin/fmax and
 * comparisons are not counted. The counting build computes the same values
 * as the plain build (every operation is the double operation).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct fc_counts {
    unsigned long long add, mul, div, sqrt, trans;
};
static fc_counts g_fc;

struct cdouble {
    double v;
    cdouble() = default;
    constexpr cdouble(double x) : v(x) {}
    explicit operator double() const { return v; }
    explicit operator int() const { return (int)v; }
    explicit operator long() const { return (long)v; }
    explicit operator long long() const { return (long long)v; }
    explicit operator unsigned long long() const { return (unsigned long long)v; }
    explicit operator bool() const { return v != 0.0; }
    cdouble& operator+=(cdouble o) { ++g_fc.add; v += o.v; return *this; }
    cdouble& operator-=(cdouble o) { ++g_fc.add; v -= o.v; return *this; }
    cdouble& operator*=(cdouble o) { ++g_fc.mul; v *= o.v; return *this; }
    cdouble& operator/=(cdouble o) { ++g_fc.div; v /= o.v; return *this; }
};
static_assert(sizeof(cdouble) == sizeof(double), "layout");

static inline cdouble operator+(cdouble a, cdouble b) { ++g_fc.add; return cdouble(a.v + b.v); }
static inline cdouble operator-(cdouble a, cdouble b) { ++g_fc.add; return cdouble(a.v - b.v); }
static inline cdouble operator*(cdouble a, cdouble b) { ++g_fc.mul; return cdouble(a.v * b.v); }
static inline cdouble operator/(cdouble a, cdouble b) { ++g_fc.div; return cdouble(a.v / b.v); }
static inline cdouble operator-(cdouble a) { return cdouble(-a.v); }
static inline cdouble operator+(cdouble a) { return a; }
static inline bool operator<(cdouble a, cdouble b) { return a.v < b.v; }
static inline bool operator>(cdouble a, cdouble b) { return a.v > b.v; }
static inline bool operator<=(cdouble a, cdouble b) { return a.v <= b.v; }
static inline bool operator>=(cdouble a, cdouble b) { return a.v >= b.v; }
static inline bool operator==(cdouble a, cdouble b) { return a.v == b.v; }
static inline bool operator!=(cdouble a, cdouble b) { return a.v != b.v; }
static inline bool operator!(cdouble a) { return a.v == 0.0; }
static inline cdouble sqrt(cdouble a) { ++g_fc.sqrt; return cdouble(::sqrt(a.v)); }
static inline cdouble fabs(cdouble a) { return cdouble(::fabs(a.v)); }
static inline cdouble fmax(cdouble a, cdouble b) { return cdouble(::fmax(a.v, b.v)); }
static inline cdouble fmin(cdouble a, cdouble b) { return cdouble(::fmin(a.v, b.v)); }
static inline cdouble exp(cdouble a) { ++g_fc.trans; return cdouble(::exp(a.v)); }
static inline cdouble log(cdouble a) { ++g_fc.trans; return cdouble(::log(a.v)); }
static inline cdouble log10(cdouble a) { ++g_fc.trans; return cdouble(::log10(a.v)); }
static inline cdouble pow(cdouble a, cdouble b) { ++g_fc.trans; return cdouble(::pow(a.v, b.v)); }
static inline cdouble ldexp(cdouble a, int e) { return cdouble(::ldexp(a.v, e)); }
static inline bool isfinite(cdouble a) { return std::isfinite(a.v); }
static inline bool isnan(cdouble a) { return std::isnan(a.v); }

// per-phase counts of the block step (hydro_oracle.c's ORC_PHASE marks)
static fc_counts g_mark, g_phase[4];
static void fc_phase(int k)
{
    if (k >= 0 && k < 4) {
        g_phase[k].add += g_fc.add - g_mark.add;
        g_phase[k].mul += g_fc.mul - g_mark.mul;
        g_phase[k].div += g_fc.div - g_mark.div;
        g_phase[k].sqrt += g_fc.sqrt - g_mark.sqrt;
        g_phase[k].trans += g_fc.trans - g_mark.trans;
    }
    g_mark = g_fc;
}
#define ORC_PHASE(k) fc_phase(k)

#define double cdouble
#include "cool_oracle.c"
#include "hydro_oracle.c"
#undef double

#define FC_API extern "C" __attribute__((visibility("default")))

FC_API void fc_reset(void)
{
    memset(&g_fc, 0, sizeof g_fc);
    memset(&g_mark, 0, sizeof g_mark);
    memset(g_phase, 0, sizeof g_phase);
}
FC_API void fc_phase_read(unsigned long long* out)
{
    for (int k = 0; k < 4; ++k) {
        out[5 * k + 0] = g_phase[k].add;
        out[5 * k + 1] = g_phase[k].mul;
        out[5 * k + 2] = g_phase[k].div;
        out[5 * k + 3] = g_phase[k].sqrt;
        out[5 * k + 4] = g_phase[k].trans;
    }
}
FC_API void fc_read(unsigned long long* out)
{
    out[0] = g_fc.add;
    out[1] = g_fc.mul;
    out[2] = g_fc.div;
    out[3] = g_fc.sqrt;
    out[4] = g_fc.trans;
}

/* one unsplit step of each of n consecutive blocks (guard cells filled) */
FC_API void fc_unsplit_blocks(const orc_hydro_params* p, int n, double* u, double* bx, double* by, double* bz,
                              double dt, double dx)
{
    const int m = p->nxb + 2 * p->nguard;
    const int64_t n3 = (int64_t)m * m * m, fsz = n3 + (int64_t)m * m;
    for (int b = 0; b < n; ++b)
        orc_unsplit_block(p, (cdouble*)(u + (int64_t)b * ORV_NVAR * n3),
                          p->mhd ? (cdouble*)(bx + b * fsz) : nullptr, p->mhd ? (cdouble*)(by + b * fsz) : nullptr,
                          p->mhd ? (cdouble*)(bz + b * fsz) : nullptr, dt, dx, dx, dx);
}

FC_API void fc_dt_blocks(const orc_hydro_params* p, int n, const double* u, double dx)
{
    const int m = p->nxb + 2 * p->nguard;
    const int64_t n3 = (int64_t)m * m * m;
    for (int b = 0; b < n; ++b) orc_block_dt_limit(p, (const cdouble*)(u + (int64_t)b * ORV_NVAR * n3), dx, dx, dx);
}

FC_API void fc_radheat_cells(const orc_cool_params* p, const orc_table* t, int64_t n, double dt, const double* dens,
                             double* ener, double* eint, double* temp, double* tdus)
{
    orc_radheat_cells(p, t, n, dt, (const cdouble*)dens, nullptr, nullptr, nullptr, (cdouble*)ener, (cdouble*)eint,
                      (cdouble*)temp, (cdouble*)tdus, nullptr, nullptr, nullptr, nullptr, nullptr);
}
