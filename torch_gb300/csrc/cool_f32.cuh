// FP32 restatement of the heating/cooling rate function de/dt
// (heatCool.F90:1397-1588 and the terms it calls) for the learned-cooling
// path: the surrogate's features and its Newton iterations use it; the
// final acceptance check re-evaluates the residual in FP64 with
// cool_dev.cuh. Power laws are evaluated as exp(ln C + a ln T) so that
// terms such as 7.63e-81 T^13.8 stay inside FP32's range; intermediate
// quantities are scaled the same way where a product would leave it.
#pragma once

#include "cool_types.cuh"
#include "gb_common.cuh"

namespace gbcoolf {

__device__ __forceinline__ float lin(float x1, float y1, float x2, float y2, float x)
{
    return (y2 - y1) / (x2 - x1) * (x - x1) + y1;
}

// ACC: the correctly rounded-to-a-few-ulp library functions (expf, logf,
// powf) instead of the hardware approximations (__expf, whose error grows
// with |x|: about 60 ulp at the power laws' x ~ -50). The plain integrator
// run on FP32 rates takes ACC; the surrogate's features and Newton steps
// do not need it.
template <bool ACC>
__device__ __forceinline__ float ex(float x) { return ACC ? expf(x) : __expf(x); }
template <bool ACC>
__device__ __forceinline__ float lg(float x) { return ACC ? logf(x) : __logf(x); }
template <bool ACC>
__device__ __forceinline__ float pwr(float x, float y) { return ACC ? powf(x, y) : __powf(x, y); }

template <bool ACC = false>
__device__ __forceinline__ float pw(float lnC, float a, float lnT) { return ex<ACC>(lnC + a * lnT); }

// Radloss (heatCool.F90:1590-1667) in log space
template <bool ACC = false>
__device__ __forceinline__ float radloss(float T)
{
    const float l = lg<ACC>(T);
    if (T >= 1.70e4f) {
        if (T >= 5.62e5f) {
            if (T >= 2.75e6f) return T >= 3.16e7f ? pw<ACC>(-61.0416264f, 0.5f, l) : pw<ACC>(-46.7079387f, -0.33f, l);
            return T >= 1.78e6f ? pw<ACC>(-7.85193121f, -2.95f, l) : pw<ACC>(-50.5136917f, 0.01f, l);
        }
        if (T >= 7.94e4f) return T >= 2.51e5f ? pw<ACC>(-23.9471542f, -2.0f, l) : pw<ACC>(-48.9528915f, 0.01f, l);
        return T >= 3.98e4f ? pw<ACC>(-71.3801379f, 2.0f, l) : pw<ACC>(-47.9629208f, -0.216f, l);
    }
    if (T >= 1.e3f) {
        if (T >= 6.31e3f) return T >= 1.0e4f ? pw<ACC>(-184.477305f, 13.8f, l) : pw<ACC>(-61.0287645f, 0.396f, l);
        return T >= 3.16e3f ? pw<ACC>(-58.8964335f, 0.152f, l) : pw<ACC>(-60.5058714f, 0.352f, l);
    }
    if (T >= 3.98e1f) return T >= 2.00e2f ? pw<ACC>(-61.0513826f, 0.431f, l) : pw<ACC>(-64.0536723f, 0.997f, l);
    return T >= 2.51e1f ? pw<ACC>(-65.9036743f, 1.5f, l) : pw<ACC>(-73.5919686f, 3.885f, l);
}

__device__ __forceinline__ float fmx(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float fmn(float a, float b) { return a < b ? a : b; }

__device__ __forceinline__ float ramp_T(float T, float lo, float hi)
{
    float ll10 = lo + 0.1f * lo, ul10 = hi - 0.1f * hi;
    if (T >= ul10) return lin(ul10, 1.0f, hi, 0.0f, T);
    if (T <= ll10) return lin(lo, 0.0f, ll10, 1.0f, T);
    return 1.0f;
}

__device__ __forceinline__ int find(const float* x, float x0, int N)
{
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

// de/dt split into heating Gamma and cooling Lambda (as dei_parts);
// floor_ is the cooling at the floors (state-independent per cell)
template <bool ACC = false>
static __device__ float dei_parts(const gb_cool_pf& p, const gb_cool_tabf& t, const gb_cool_varsf& v, float floor_,
                           float ei, float* gam, float* lam)
{
    float T = ei / v.TtoEI;
    if (T < 0.0f) T = 1.0f;
    const float sqT = sqrtf(T);
    // Jeans-length column density (heatCool.F90:1669-1722)
    const float lam_j = v.ndens / v.rho * sqrtf(p.jeansK * T / v.ndens);
    const float ncol = lam_j * v.ndens;
    float eplus = 0.0f;
    if (T <= p.theatmax && T >= p.theatmin) {
        if (p.use_cr_heating) {
            if (p.cr_uniform) eplus = v.cr_pref;
            else eplus = v.cr_pref * ex<ACC>(-p.crIonExp * (lg<ACC>(fmx(p.crIonNH, ncol)) - p.lnNH));
        }
        eplus *= ramp_T(T, p.theatmin, p.theatmax);
    }
    const float fext = ex<ACC>(-3.5f * (ncol * 0.01f / 1.87e21f));
    const float G = v.Gflux + p.Gzero * fext;
    float PeHeat = 0.0f;
    const float ulpe = fmn(p.theatmax, p.dust_sputter_temp);
    if (T <= ulpe && T >= p.theatmin) {
        const float xl = v.xHp == 0.0f ? 1e-8f : v.xHp;
        float eff;
        if (p.pe_recipe == 1) {
            float Gf = G * sqT / (xl * v.ndens * 0.5f);
            eff = 4.9e-2f / (1.0f + 4.0e-3f * pwr<ACC>(Gf, 0.73f)) + 3.7e-2f * pwr<ACC>(T * 1e-4f, 0.7f) / (1.0f + 2.0e-4f * Gf);
            PeHeat = p.pe_norm * eff * G * (v.ndens / v.rho);
        } else if (p.pe_recipe == 0) {
            float Gf = G * sqT / (xl * v.ndens);
            float gp = Gf > 0.0f ? lg<ACC>(Gf) : -1e30f;
            eff = (7.64f + 4.52f * ex<ACC>(0.132f * lg<ACC>(T))) /
                  (1.0f + (0.04371f * ex<ACC>(0.452f * gp)) * (1.0f + 0.00557f * ex<ACC>(0.675f * gp)));
            // 1e-26 * eff * G / (rho / n), with rho/n ~ 4e-24 kept in range
            PeHeat = 1e-26f * eff * G * (v.ndens / v.rho);
        } else {
            PeHeat = p.pe_norm * 0.05f * G * (v.ndens / v.rho);
        }
        PeHeat *= ramp_T(T, p.theatmin, ulpe);
    }
    eplus += v.ephen;
    // atomic cooling (heatCool.F90:1116-1200)
    float emin = 0.0f;
    if (T <= p.tradmax && T >= p.tradmin && v.ndens >= p.dradmin && v.ndens <= p.dradmax) {
        emin = radloss<ACC>(T);
        if (v.xHp > 1e-2f && T < 1.2e4f) {
            float DG = lin(1e-2f, 1.0f, 1e-1f, 5.0f, fmn(1e-1f, v.xHp));
            emin *= DG;
            if (T > 1e4f) {
                float q = lin(1e4f, 1.0f, 1.2e4f, sqrtf(DG), T);
                emin /= q * q;
            }
        } else if (v.xHp < 1e-2f && T < 1e4f) {
            float DG = lin(1e-4f, 0.35f, 1e-2f, 1.0f, fmx(1e-4f, v.xHp));
            emin *= DG;
            if (T > 9e3f) emin /= lin(9e3f, 1.0f, 1e4f, DG, T);
        }
        emin *= ramp_T(T, p.tradmin, p.tradmax) * v.conf;
    }
    float cool_pw = 0.0f, cool_dg = 0.0f;
    if (p.useDustCool) {
        if (v.ndens >= p.nd_cool_min && v.ndens <= p.nd_cool_max && T >= p.T_cool_min &&
            T <= p.theatmax) {
            int it = find(t.T, fmx(T, t.T_min), GB_TEMP_PTS);
            int id = find(t.n, fmx(v.ndens, t.nd_min), GB_DENS_PTS);
            if (it > 0 && it <= GB_TEMP_PTS && id > 0 && id <= GB_DENS_PTS)
                cool_pw = __ldg(t.lam + (id - 1) + GB_DENS_PTS * (it - 1));
            cool_pw *= ramp_T(T, p.T_cool_min, p.theatmax) *
                       ramp_T(v.ndens, p.nd_cool_min, p.nd_cool_max);
        }
        if (T <= p.dust_sputter_temp) {
            // 3.8e-33 n^2 (...) / rho  ->  3.8e-33 n (n / rho) (...)
            cool_dg = 3.8e-33f * v.ndens * (v.ndens / v.rho) * (1.0f - 0.8f * ex<ACC>(-75.0f / T)) * (T - v.tdust) * sqT;
            float ul = p.dust_sputter_temp, ul10 = ul - 0.1f * ul;
            if (T >= ul10) cool_dg *= lin(ul10, 1.0f, ul, 0.0f, T);
        }
    }
    *gam = eplus + PeHeat + floor_ + fmx(-cool_dg, 0.0f);
    *lam = emin + cool_pw + fmx(cool_dg, 0.0f);
    return eplus + PeHeat - emin - cool_pw - cool_dg + floor_;
}

// T_dust after a step (heatCool.F90:430-443 + get_dust_temperature,
// :703-884) in FP32: dust heating by FUV photons that did not eject
// photo-electrons plus cosmic rays, Newton on the dust energy balance
template <bool ACC = false>
static __device__ float dust_temperature(const gb_cool_pf& p, const gb_cool_varsf& v, float T, float tdust_in)
{
    const float sqT = sqrtf(T);
    const float lam_j = v.ndens / v.rho * sqrtf(p.jeansK * T / v.ndens);
    const float ncol = lam_j * v.ndens;
    const float G = v.Gflux + p.Gzero * ex<ACC>(-3.5f * (ncol * 0.01f / 1.87e21f));
    // dust heating / (n 1e-33): photo-electric remainder + CR heating * rho
    float heat = 0.0f;
    const float ulpe = fmn(p.theatmax, p.dust_sputter_temp);
    if (T <= ulpe && T >= p.theatmin) {
        const float xl = v.xHp == 0.0f ? 1e-8f : v.xHp;
        float eff = 0.05f, dh;
        if (p.pe_recipe == 0) {
            float Gf = G * sqT / (xl * v.ndens);
            float gp = Gf > 0.0f ? lg<ACC>(Gf) : -1e30f;
            eff = (7.64f + 4.52f * ex<ACC>(0.132f * lg<ACC>(T))) /
                  (1.0f + (0.04371f * ex<ACC>(0.452f * gp)) * (1.0f + 0.00557f * ex<ACC>(0.675f * gp)));
            dh = fmx((p.pe_norm * 1e26f - eff) * G * 1e7f, 0.0f);  // (pe_norm - 1e-26 eff) G n / (n 1e-33)
        } else if (p.pe_recipe == 1) {
            float Gf = G * sqT / (xl * v.ndens * 0.5f);
            eff = 4.9e-2f / (1.0f + 4.0e-3f * pwr<ACC>(Gf, 0.73f)) + 3.7e-2f * pwr<ACC>(T * 1e-4f, 0.7f) / (1.0f + 2.0e-4f * Gf);
            dh = p.pe_norm * 1e33f * fmx(0.0f, 1.0f - eff) * G;
        } else {
            dh = p.pe_norm * 1e33f * 0.95f * G;
        }
        heat = dh;
    }
    if (p.use_cr_heating && T <= p.theatmax && T >= p.theatmin) {
        float cr = v.cr_pref;
        if (!p.cr_uniform)
            cr *= ex<ACC>(-p.crIonExp * (lg<ACC>(fmx(p.crIonNH, ncol)) - p.lnNH));
        cr *= ramp_T(T, p.theatmin, p.theatmax);
        heat += cr * (v.rho / v.ndens) * 1e33f;
    }
    const float absTmin = p.absTmin;
    float td = tdust_in < absTmin ? absTmin : tdust_in;
    const float tg = T < absTmin ? absTmin : T;
    const float cfac = 3.8f * v.ndens * (1.0f - 0.8f * ex<ACC>(-75.0f / tg)) * sqrtf(tg);
    float err = 1e-3f;
    for (int l = 0; l < 100 && err > 1e-4f; ++l) {
        float t3 = td * td * td;
        float lamd = 6.8f * t3 * t3;
        float eq = heat + cfac * (tg - td) - lamd;
        float det = -(6.0f * lamd / td) - cfac;
        float tn = td - eq / det;
        err = fabsf(tn - td) / td;
        td = tn;
        if (td < 0.1f) {
            td = 0.1f;
            err = 1e-5f;
        }
    }
    return td < absTmin ? absTmin : td;
}

__device__ __forceinline__ void make_vars(const gb_cool_pf& p, const gb_cool_vars& v, gb_cool_varsf& f)
{
    f.ndens = gb_d2f(v.ndens);
    f.rho = gb_d2f(v.rho);
    f.conf = gb_d2f(v.conf);
    f.Gflux = gb_d2f(v.Gflux);
    f.ephen = gb_d2f(v.ephen);
    f.tdust = gb_d2f(v.tdust);
    f.TtoEI = gb_d2f(v.TtoEI);
    f.xHp = gb_d2f(v.xHp);
    f.mu_mol = gb_d2f(v.mu_mol);
    f.cr_pref = p.crRE * (f.ndens / f.rho);
}

// cooling at the floors (heatCool.F90:1509-1519) in FP32
template <bool ACC = false>
static __device__ float cooling_floor(const gb_cool_pf& p, const gb_cool_tabf& t, const gb_cool_varsf& v)
{
    float emin = 0.0f;
    const float T = p.tradmin;
    if (T <= p.tradmax && T >= p.tradmin && v.ndens >= p.dradmin && v.ndens <= p.dradmax) {
        emin = radloss<ACC>(T);
        if (v.xHp > 1e-2f && T < 1.2e4f) {
            float DG = lin(1e-2f, 1.0f, 1e-1f, 5.0f, fmn(1e-1f, v.xHp));
            emin *= DG;
            if (T > 1e4f) {
                float q = lin(1e4f, 1.0f, 1.2e4f, sqrtf(DG), T);
                emin /= q * q;
            }
        } else if (v.xHp < 1e-2f && T < 1e4f) {
            float DG = lin(1e-4f, 0.35f, 1e-2f, 1.0f, fmx(1e-4f, v.xHp));
            emin *= DG;
            if (T > 9e3f) emin /= lin(9e3f, 1.0f, 1e4f, DG, T);
        }
        emin *= ramp_T(T, p.tradmin, p.tradmax) * v.conf;
    }
    float pw_ = 0.0f;
    const float Tm = p.T_cool_min;
    if (p.useDustCool && v.ndens >= p.nd_cool_min && v.ndens <= p.nd_cool_max && Tm >= p.T_cool_min &&
        Tm <= p.theatmax) {
        int it = find(t.T, fmx(Tm, t.T_min), GB_TEMP_PTS);
        int id = find(t.n, fmx(v.ndens, t.nd_min), GB_DENS_PTS);
        if (it > 0 && it <= GB_TEMP_PTS && id > 0 && id <= GB_DENS_PTS) pw_ = __ldg(t.lam + (id - 1) + GB_DENS_PTS * (it - 1));
        pw_ *= ramp_T(Tm, p.T_cool_min, p.theatmax) * ramp_T(v.ndens, p.nd_cool_min, p.nd_cool_max);
    }
    return emin + pw_;
}

}  // namespace gbcoolf
