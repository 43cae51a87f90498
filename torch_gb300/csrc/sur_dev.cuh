// Per-cell inputs and features of the learned cooling surrogate, shared by
// the surrogate kernels and the hydro update (which writes the features of
// the state it just produced, when the surrogate cools that state next).
#pragma once

#include "cool_f32.cuh"
#include "sur_common.cuh"

// Unit factors of the learned-cooling kernels, divided once on the host:
// their loads and stores multiply instead of dividing per cell (FP64
// division is a long sequence on the FP64 pipe). The fallback kernel, which
// is the plain integrator, keeps sur_load's divisions.
struct sur_units {
    double T_of_e;     // (gamma - 1) abar m_p / k_B
    double e_of_T;     // its inverse: TtoEI
    double inv_mu_mp;  // 1 / (mu_mol m_p)
    double vel2, inv_vel2;
    // FP32 copies for the surrogate kernels, whose per-cell inputs go
    // straight to FP32 (FP64 instructions are the scarce resource there)
    float dens_unit_f, T_of_e_f, e_of_T_f, inv_mu_mp_f, time_unit_f, mu_mol_f, xHp_const_f;
    float emin_f;  // 0.5 absTmin TtoEI, the energy floor of the iteration
    float absTmin_f, absTmax_f, dust_sputter_f, smallp_f, T_min_f, nd_min_f;
    double smallp, dens_unit;
};

// The inputs of the surrogate kernels for one cell in FP32: the FP64
// state is converted on the integer pipe and scaled in FP32. Only the
// internal energy is also kept in FP64 (the accepted energy is formed from
// it in FP64). Each FP32 input is within a couple of ulp of the rounded
// FP64 value the plain loader makes.
__device__ __forceinline__ void sur_load_f32(const gb_dev_grid& g, const gb_cool_pf& pf, const sur_units& u, int blk,
                                             int ci, gb_cool_varsf& f, double& ei, float& eif, float& tempf)
{
    ei = gb_var(g, blk, GB_EINT)[ci] * u.vel2;
    eif = gb_d2f(ei);
    tempf = eif * u.T_of_e_f;
    f.rho = gb_d2f(gb_var(g, blk, GB_DENS)[ci]) * u.dens_unit_f;
    f.ndens = f.rho * u.inv_mu_mp_f;
    f.conf = f.ndens * u.inv_mu_mp_f;  // ndens^2 / rho
    f.tdust = gb_d2f(gb_var(g, blk, GB_TDUS)[ci]);
    f.xHp = g.slot[GB_IHP] >= 0 ? gb_d2f(gb_var(g, blk, GB_IHP)[ci]) : u.xHp_const_f;
    f.ephen = g.slot[GB_PHHE] >= 0 ? gb_d2f(gb_var(g, blk, GB_PHHE)[ci]) / f.rho : 0.0f;
    f.Gflux = g.slot[GB_PEFL] >= 0 ? gb_d2f(gb_var(g, blk, GB_PEFL)[ci]) : 0.0f;
    f.TtoEI = u.e_of_T_f;
    f.mu_mol = u.mu_mol_f;
    f.cr_pref = pf.crRE * (f.ndens / f.rho);
}

// The surrogate's features of one cell and the rate at its state (with
// the cooling floor): x = (log n, log T, log dt / t_cool, log Gamma /
// Lambda) normalised (sur_common.cuh), f0fl = (de/dt, floor).
__device__ __forceinline__ void sur_features(const gb_cool_ctx& c, const gb_cool_pf& pf, const sur_units& un,
                                             const gb_cool_varsf& vf, float eif, float tempf, double dt_code,
                                             float4& x, float2& f0fl)
{
    const gb_cool_tabf tf = {c.Tf, c.nf, c.lamf, un.T_min_f, un.nd_min_f};
    const float fl = gbcoolf::cooling_floor(pf, tf, vf);
    float gam, lam;
    const float f0 = gbcoolf::dei_parts(pf, tf, vf, fl, eif, &gam, &lam);
    const float dt = gb_d2f(dt_code) * un.time_unit_f;
    // features in FP32: dt / t_cool = dt |f| / e
    const float r = dt * fabsf(f0) / eif;
    float lr = log10f(fmaxf(r, 1e-30f));
    lr = fminf(fmaxf(lr, (float)-gbsur::R_CLAMP), (float)gbsur::R_CLAMP);
    float lh = log10f(fmaxf(gam, 1e-30f)) - log10f(fmaxf(lam, 1e-30f));
    lh = fminf(fmaxf(lh, (float)-gbsur::H_CLAMP), (float)gbsur::H_CLAMP);
    x = make_float4((log10f(vf.ndens) - (float)gbsur::N_MID) / (float)gbsur::N_HALF,
                    (log10f(tempf) - (float)gbsur::T_MID) / (float)gbsur::T_HALF, lr / (float)gbsur::R_HALF,
                    lh / (float)gbsur::H_HALF);
    f0fl = make_float2(f0, fl);
}

// Where the hydro update writes the surrogate's inputs (null feat: it
// writes none; the feature kernel makes them)
struct sur_feat_out {
    float4* feat = nullptr;
    float2* f0 = nullptr;
    gb_cool_pf pf;
    sur_units un;
};
