// Feature and target normalisation of the learned cooling surrogate, shared
// by the sample generator, the inline feature kernel and the host code.
#pragma once

namespace gbsur {
// x0 = (log10 n - 2) / 4, x1 = (log10 T - 4.5) / 3.5,
// x2 = log10(dt / t_cool) / 3 (log clamped to [-12, 12]),
// x3 = log10(Gamma / Lambda) / 4, the heating rate in units of the cooling
//      rate at the current state (clamped to [-8, 8] decades): positive
//      where the gas heats, negative where it cools, zero at equilibrium,
// y  = (log10 T_new - log10 T) / 4
constexpr double N_MID = 2.0, N_HALF = 4.0;
constexpr double T_MID = 4.5, T_HALF = 3.5;
constexpr double R_HALF = 3.0, R_CLAMP = 12.0;
constexpr double Y_SCALE = 4.0;

constexpr double H_CLAMP = 8.0, H_HALF = 4.0;

__host__ __device__ inline void features(double nden, double T, double dt_over_tcool, double gam, double lam,
                                         float* x)
{
    double lr = log10(dt_over_tcool);
    lr = lr < -R_CLAMP ? -R_CLAMP : (lr > R_CLAMP ? R_CLAMP : lr);
    double lh = log10(fmax(gam, 1e-300)) - log10(fmax(lam, 1e-300));
    lh = lh < -H_CLAMP ? -H_CLAMP : (lh > H_CLAMP ? H_CLAMP : lh);
    x[0] = (float)((log10(nden) - N_MID) / N_HALF);
    x[1] = (float)((log10(T) - T_MID) / T_HALF);
    x[2] = (float)(lr / R_HALF);
    x[3] = (float)(lh / H_HALF);
}
}  // namespace gbsur
