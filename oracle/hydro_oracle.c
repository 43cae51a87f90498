/*
 * CPU oracle: unsplit PPM + HLLC hydro and staggered-mesh PPM + HLLD + CT
 * MHD for one guard-cell-padded block. TEST INFRASTRUCTURE ONLY.
 *
 * The per-cell reconstruction follows the control flow of
 *   src/flash/source/physics/Hydro/HydroMain/unsplit/hy_uhd_dataReconstOneStep.F90
 *   - multidimensional MHD terms aBn, dnBn            (:364-424)
 *   - normal-direction PPM per dimension              (:628-638 / :844-853)
 *   - transverse-flux corrections, hydro then MHD     (:1006-1089)
 *   - hybrid-order fallback to first order where the flow compresses and
 *     a face state fails the Rankine-Hugoniot check, before (:934-999) and
 *     after (:1150-1218) the transverse corrections, with the per-cell CFL
 *     lowering of hy_fallbackLowerCFL (:972, :1207-1216)
 *   - positivity fallback to first order              (:1230-1272)
 * hy_uhd_checkRHjumpCond's body is not vendored (interface
 * hy_uhd_interface.F90:798-807); rh_fail below writes it from the
 * Rankine-Hugoniot relations: no single shock compresses an ideal gas by
 * more than (gamma + 1) / (gamma - 1) (Toro 1997 eq. 3.58's strong-shock
 * limit), so a face state whose density differs from its cell's by more is
 * not shock-connected to it. Compression is Balsara & Spicer's (1999)
 * undivided velocity divergence below kappa times the cell's fast speed,
 * the minimum over the +-k4 box (k4 = 1 MHD, 2 hydro; :275-278) clipped to
 * the reconstruction band, whose cells all have filled neighbours.
 *
 * The normal-direction PPM (interface hy_uhd_interface.F90:200-228) is
 * written from Colella & Woodward (1984) eqs. 1.6, 1.10, 1.12 with
 * characteristic (minmod) limiting and characteristic tracing against a
 * reference state (Colella 1990; Stone et al. 2008, sec. 4.2). The
 * transverse term `sig` of one direction is A(W) . (W_R - W_L) of the
 * limited parabola. Riemann solvers: HLLC (Toro 1997 ch. 10, Davis wave
 * speeds) and HLLD (Miyoshi & Kusano 2005). Artificial viscosity follows
 * docs/torch_manual/main.tex:375-408. Electric fields: Gardiner & Stone
 * (2005) eq. 41/50 (contact-upwinded CT) with the cell-centred reference
 * field at t + dt/2 (from the cell's face states along the edge).
 * Internal energy: Bryan et al.
 * (1995) dual-energy formalism with eintSwitch.
 *
 * Every expression is written in the order the GPU kernels evaluate it;
 * build with -O2 -ffp-contract=off.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAXW 7 /* waves of the 1-D MHD system */
#define NP 8   /* primitive vars rho, vx, vy, vz, p, Bx, By, Bz */

static const double TWO3 = 2.0 / 3.0;

/* Phase marks of one block step for the flop-counting build (flopcount.cpp
 * attributes the arithmetic since the previous mark to phase k: 0
 * reconstruction, 1 Riemann fluxes, 2 edge electric fields, 3 face field
 * and cell update; -1 only sets the mark). No-ops otherwise. */
#ifndef ORC_PHASE
#define ORC_PHASE(k) ((void)0)
#endif

void orc_hydro_default_params(orc_hydro_params* p, int mhd)
{
    memset(p, 0, sizeof(*p));
    p->gamma = 5.0 / 3.0;
    p->cvisc = 0.1;
    p->use_avisc = 1;
    p->eint_switch = 1.e-4;
    p->smlrho = 1e-30;
    p->smallp = 1e-30;
    p->mhd = mhd;
    p->nxb = 16;
    p->nguard = 4;
    p->energy_fix = 1;
    p->cfl_sum = 1;
    p->hybrid_order = 1;
    p->fallback_lower_cfl = 1;
    p->hybrid_kappa = 0.0;
    p->cfl_fallback_factor = 0.9;
    p->cfl = 0.8;
    p->cflc = NULL;
}

double orc_cfl_scale(const orc_hydro_params* p, int code)
{
    double s = 1.0;
    if (code & 1) s = fmin(s, (p->cfl_fallback_factor / 3.0) / p->cfl);
    if (code & 2) s = fmin(s, 0.25 / p->cfl);
    return s;
}

/* ------------------------------------------------------------ indexing */
typedef struct blk {
    int n;  /* cells per side incl. guards */
    int ng, nxb;
    double* u; /* ORV_NVAR * n^3 */
    double* f[3];
} blk;

static inline int64_t cidx(int n, int i, int j, int k) { return i + (int64_t)n * (j + (int64_t)n * k); }
static inline int64_t fidx(int n, int d, int i, int j, int k)
{
    if (d == 0) return i + (int64_t)(n + 1) * (j + (int64_t)n * k);
    if (d == 1) return i + (int64_t)n * (j + (int64_t)(n + 1) * k);
    return i + (int64_t)n * (j + (int64_t)n * k);
}
static inline double U(const blk* b, int v, int i, int j, int k)
{
    return b->u[(int64_t)v * b->n * b->n * b->n + cidx(b->n, i, j, k)];
}

static inline double minmod(double a, double b)
{
    if (a * b <= 0.0) return 0.0;
    return (fabs(a) <= fabs(b)) ? a : b;
}

/* ------------------------------------------------------------ eigensystems */

/* Hydro, primitive (rho, vn, vt1, vt2, p). Waves: vn-a, vn, vn, vn, vn+a. */
static void eig_hydro(double gam, const double* q, double* lam, double R[MAXW][MAXW],
                      double L[MAXW][MAXW])
{
    double rho = q[0], vn = q[1], p = q[4];
    double a2 = gam * p / rho;
    double a = sqrt(a2);
    memset(R, 0, sizeof(double) * MAXW * MAXW);
    memset(L, 0, sizeof(double) * MAXW * MAXW);
    lam[0] = vn - a; lam[1] = vn; lam[2] = vn; lam[3] = vn; lam[4] = vn + a;
    /* R[var][wave] */
    R[0][0] = 1.0; R[1][0] = -a / rho; R[4][0] = a2;
    R[0][1] = 1.0;
    R[2][2] = 1.0;
    R[3][3] = 1.0;
    R[0][4] = 1.0; R[1][4] = a / rho; R[4][4] = a2;
    /* L[wave][var] */
    L[0][1] = -rho / (2.0 * a); L[0][4] = 1.0 / (2.0 * a2);
    L[1][0] = 1.0; L[1][4] = -1.0 / a2;
    L[2][2] = 1.0;
    L[3][3] = 1.0;
    L[4][1] = rho / (2.0 * a); L[4][4] = 1.0 / (2.0 * a2);
}

/* MHD, primitive (rho, vn, vt1, vt2, p, Bt1, Bt2) with parameter Bn
 * (q[5] = Bn, q[6] = Bt1, q[7] = Bt2 in the rotated 8-vector). Waves:
 * vn-cf, vn-ca, vn-cs, vn, vn+cs, vn+ca, vn+cf. Right eigenvectors in the
 * Roe & Balsara (1996) normalisation; left ones are their exact inverse. */
static void eig_mhd(double gam, const double* q, double* lam, double R[MAXW][MAXW],
                    double L[MAXW][MAXW])
{
    double rho = q[0], vn = q[1], p = q[4], bn = q[5], bt1 = q[6], bt2 = q[7];
    double a2 = gam * p / rho;
    double sr = sqrt(rho);
    double bnx2 = bn * bn / rho;
    double bt2s = (bt1 * bt1 + bt2 * bt2) / rho;
    double term = a2 + bnx2 + bt2s;
    /* (a^2+b^2)^2 - 4 a^2 bn^2 written without cancellation, and the
     * alpha_f, alpha_s of Roe & Balsara (1996) from differences that are
     * exact when the transverse field vanishes */
    double d1 = a2 - bnx2;
    double disc = sqrt(d1 * d1 + bt2s * (2.0 * (a2 + bnx2) + bt2s));
    double cf2 = 0.5 * (term + disc);
    double cs2 = a2 * bnx2 / cf2;
    double cf = sqrt(cf2), cs = sqrt(cs2), ca = sqrt(bnx2);
    double bperp = sqrt(bt1 * bt1 + bt2 * bt2);
    double by, bz;
    if (bperp > 0.0) { by = bt1 / bperp; bz = bt2 / bperp; }
    else { by = 0.70710678118654752440; bz = 0.70710678118654752440; }
    double af, as;
    if (disc > 0.0) {
        double af2 = ((d1 - bt2s) + disc) / (2.0 * disc);
        double as2 = ((bt2s - d1) + disc) / (2.0 * disc);
        af2 = af2 < 0.0 ? 0.0 : (af2 > 1.0 ? 1.0 : af2);
        as2 = as2 < 0.0 ? 0.0 : (as2 > 1.0 ? 1.0 : as2);
        af = sqrt(af2);
        as = sqrt(as2);
    } else {
        af = 1.0;
        as = 0.0;
    }
    double S = bn >= 0.0 ? 1.0 : -1.0;
    double a = sqrt(a2);
    double n2 = af * af * cf2 + as * as * cs2;
    double sra = sr * a;
    memset(R, 0, sizeof(double) * MAXW * MAXW);
    memset(L, 0, sizeof(double) * MAXW * MAXW);
    lam[0] = vn - cf; lam[1] = vn - ca; lam[2] = vn - cs; lam[3] = vn;
    lam[4] = vn + cs; lam[5] = vn + ca; lam[6] = vn + cf;
    /* var order: 0 rho, 1 vn, 2 vt1, 3 vt2, 4 p, 5 Bt1, 6 Bt2 */
    /* fast - */
    R[0][0] = rho * af; R[1][0] = -af * cf; R[2][0] = as * cs * by * S; R[3][0] = as * cs * bz * S;
    R[4][0] = rho * af * a2; R[5][0] = as * sra * by; R[6][0] = as * sra * bz;
    /* alfven - */
    R[2][1] = -bz; R[3][1] = by; R[5][1] = -S * sr * bz; R[6][1] = S * sr * by;
    /* slow - */
    R[0][2] = rho * as; R[1][2] = -as * cs; R[2][2] = -af * cf * by * S; R[3][2] = -af * cf * bz * S;
    R[4][2] = rho * as * a2; R[5][2] = -af * sra * by; R[6][2] = -af * sra * bz;
    /* entropy */
    R[0][3] = 1.0;
    /* slow + */
    R[0][4] = rho * as; R[1][4] = as * cs; R[2][4] = af * cf * by * S; R[3][4] = af * cf * bz * S;
    R[4][4] = rho * as * a2; R[5][4] = -af * sra * by; R[6][4] = -af * sra * bz;
    /* alfven + */
    R[2][5] = -bz; R[3][5] = by; R[5][5] = S * sr * bz; R[6][5] = -S * sr * by;
    /* fast + */
    R[0][6] = rho * af; R[1][6] = af * cf; R[2][6] = -as * cs * by * S; R[3][6] = -as * cs * bz * S;
    R[4][6] = rho * af * a2; R[5][6] = as * sra * by; R[6][6] = as * sra * bz;

    double hn = 0.5 / n2, hra = 0.5 / (rho * a2), hsa = 0.5 / sra, hs = 0.5 / sr;
    /* fast - */
    L[0][1] = -af * cf * hn; L[0][2] = as * cs * S * by * hn; L[0][3] = as * cs * S * bz * hn;
    L[0][4] = af * hra; L[0][5] = as * by * hsa; L[0][6] = as * bz * hsa;
    /* alfven - */
    L[1][2] = -0.5 * bz; L[1][3] = 0.5 * by; L[1][5] = -bz * S * hs; L[1][6] = by * S * hs;
    /* slow - */
    L[2][1] = -as * cs * hn; L[2][2] = -af * cf * S * by * hn; L[2][3] = -af * cf * S * bz * hn;
    L[2][4] = as * hra; L[2][5] = -af * by * hsa; L[2][6] = -af * bz * hsa;
    /* entropy */
    L[3][0] = 1.0; L[3][4] = -1.0 / a2;
    /* slow + */
    L[4][1] = as * cs * hn; L[4][2] = af * cf * S * by * hn; L[4][3] = af * cf * S * bz * hn;
    L[4][4] = as * hra; L[4][5] = -af * by * hsa; L[4][6] = -af * bz * hsa;
    /* alfven + */
    L[5][2] = -0.5 * bz; L[5][3] = 0.5 * by; L[5][5] = bz * S * hs; L[5][6] = -by * S * hs;
    /* fast + */
    L[6][1] = af * cf * hn; L[6][2] = -as * cs * S * by * hn; L[6][3] = -as * cs * S * bz * hn;
    L[6][4] = af * hra; L[6][5] = as * by * hsa; L[6][6] = as * bz * hsa;
}

/* rotated 8-vector slot -> unrotated primitive slot for direction d */
static inline int rot_slot(int d, int s)
{
    static const int m[3][NP] = {
        {0, 1, 2, 3, 4, 5, 6, 7},
        {0, 2, 3, 1, 4, 6, 7, 5},
        {0, 3, 1, 2, 4, 7, 5, 6},
    };
    return m[d][s];
}
/* wave-vector slot (7 MHD / 5 hydro) -> rotated 8-vector slot */
static inline int wslot(int s) { return s < 5 ? s : s + 1; }

/* ------------------------------------------------------------ PPM */

/* Normal-direction PPM at one cell. qs[m][s]: rotated primitive 8-vectors
 * of the 5-point stencil (m = 0..4, centre 2). Outputs rotated 8-vectors
 * wp (face +1/2), wn (face -1/2) and sig = A.(W_R - W_L). */
static void ppm_normal(const orc_hydro_params* p, const double qs[5][NP], double dtdx, double* wp,
                       double* wn, double* sig)
{
    const int nw = p->mhd ? 7 : 5;
    double lam[MAXW], R[MAXW][MAXW], L[MAXW][MAXW];
    if (p->mhd) eig_mhd(p->gamma, qs[2], lam, R, L);
    else eig_hydro(p->gamma, qs[2], lam, R, L);

    /* limited slopes at stencil points 1, 2, 3, projected with the centre
     * cell's eigenvectors */
    double dwm[3][MAXW];
    for (int m = 1; m <= 3; ++m) {
        double dal[MAXW], dar[MAXW], da[MAXW];
        for (int k = 0; k < nw; ++k) {
            double sl = 0.0, sr = 0.0;
            for (int s = 0; s < nw; ++s) {
                int qsl = wslot(s);
                sl = sl + L[k][s] * (qs[m][qsl] - qs[m - 1][qsl]);
                sr = sr + L[k][s] * (qs[m + 1][qsl] - qs[m][qsl]);
            }
            dal[k] = sl;
            dar[k] = sr;
            da[k] = minmod(dal[k], dar[k]);
        }
        for (int s = 0; s < nw; ++s) {
            double acc = 0.0;
            for (int k = 0; k < nw; ++k) acc = acc + R[s][k] * da[k];
            dwm[m - 1][s] = acc;
        }
    }
    double WL[MAXW], WR[MAXW], dW[MAXW], W6[MAXW];
    for (int s = 0; s < nw; ++s) {
        int qq = wslot(s);
        double qm = qs[1][qq], q0 = qs[2][qq], qp = qs[3][qq];
        double wl = 0.5 * (qm + q0) - (dwm[1][s] - dwm[0][s]) / 6.0;
        double wr = 0.5 * (q0 + qp) - (dwm[2][s] - dwm[1][s]) / 6.0;
        /* keep edge values between the neighbouring cell averages */
        wl = fmax(fmin(q0, qm), wl);
        wl = fmin(fmax(q0, qm), wl);
        wr = fmax(fmin(q0, qp), wr);
        wr = fmin(fmax(q0, qp), wr);
        /* CW84 eq. 1.10 */
        double qa = (wr - q0) * (q0 - wl);
        if (qa <= 0.0) {
            wl = q0;
            wr = q0;
        } else {
            double qb = wr - wl;
            double qc = 6.0 * (q0 - 0.5 * (wl + wr));
            if (qb * qc > qb * qb) wl = 3.0 * q0 - 2.0 * wr;
            else if (qb * qc < -(qb * qb)) wr = 3.0 * q0 - 2.0 * wl;
        }
        WL[s] = wl;
        WR[s] = wr;
        dW[s] = wr - wl;
        W6[s] = 6.0 * (q0 - 0.5 * (wl + wr));
    }
    /* characteristic projections of the parabola */
    double ldW[MAXW], lW6[MAXW];
    for (int k = 0; k < nw; ++k) {
        double a = 0.0, b = 0.0;
        for (int s = 0; s < nw; ++s) {
            a = a + L[k][s] * dW[s];
            b = b + L[k][s] * W6[s];
        }
        ldW[k] = a;
        lW6[k] = b;
    }
    /* + state (face i+1/2), reference = fastest right-moving wave */
    double sK = lam[nw - 1] * dtdx;
    int refK = lam[nw - 1] > 0.0;
    double Wp[MAXW], Wn[MAXW];
    for (int s = 0; s < nw; ++s)
        Wp[s] = refK ? WR[s] - 0.5 * sK * (dW[s] - (1.0 - TWO3 * sK) * W6[s]) : WR[s];
    for (int k = 0; k < nw; ++k) {
        if (lam[k] > 0.0) {
            double sg = lam[k] * dtdx;
            double gK = refK ? 0.5 * sK * (ldW[k] - (1.0 - TWO3 * sK) * lW6[k]) : 0.0;
            double c = gK - 0.5 * sg * (ldW[k] - (1.0 - TWO3 * sg) * lW6[k]);
            for (int s = 0; s < nw; ++s) Wp[s] = Wp[s] + c * R[s][k];
        }
    }
    /* - state (face i-1/2), reference = fastest left-moving wave */
    double s0 = lam[0] * dtdx;
    int ref0 = lam[0] < 0.0;
    for (int s = 0; s < nw; ++s)
        Wn[s] = ref0 ? WL[s] - 0.5 * s0 * (dW[s] + (1.0 + TWO3 * s0) * W6[s]) : WL[s];
    for (int k = 0; k < nw; ++k) {
        if (lam[k] < 0.0) {
            double sg = lam[k] * dtdx;
            double g0 = ref0 ? 0.5 * s0 * (ldW[k] + (1.0 + TWO3 * s0) * lW6[k]) : 0.0;
            double c = g0 - 0.5 * sg * (ldW[k] + (1.0 + TWO3 * sg) * lW6[k]);
            for (int s = 0; s < nw; ++s) Wn[s] = Wn[s] + c * R[s][k];
        }
    }
    /* transverse term A . dW */
    double sg7[MAXW];
    for (int s = 0; s < nw; ++s) {
        double acc = 0.0;
        for (int k = 0; k < nw; ++k) acc = acc + (lam[k] * ldW[k]) * R[s][k];
        sg7[s] = acc;
    }
    for (int s = 0; s < NP; ++s) { wp[s] = 0.0; wn[s] = 0.0; sig[s] = 0.0; }
    for (int s = 0; s < nw; ++s) {
        wp[wslot(s)] = Wp[s];
        wn[wslot(s)] = Wn[s];
        sig[wslot(s)] = sg7[s];
    }
    /* normal B is not reconstructed: the face value replaces it later */
    wp[5] = qs[2][5];
    wn[5] = qs[2][5];
}

/* ------------------------------------------------------------ reconstruction */

typedef struct recon_out {
    double wp[3][NP], wn[3][NP];
} recon_out;

/* hy_uhd_checkRHjumpCond for one face state: see the header */
static int rh_fail(double gam, double rho_c, double rho_f)
{
    const double lim = (gam + 1.0) / (gam - 1.0);
    return rho_f > lim * rho_c || rho_c > lim * rho_f;
}

/* flags: bit 0 positivity fallback, bit 1 first Rankine-Hugoniot fallback,
 * bit 2 second one (any direction); codes[d] the CFL code of direction d */
static int recon_cell(const orc_hydro_params* p, const blk* b, int i, int j, int k, double dt,
                      const double* del, double divu_min, recon_out* o, unsigned char* codes)
{
    const int nv = p->mhd ? 8 : 5;
    double wc[NP];
    for (int v = 0; v < NP; ++v) wc[v] = 0.0;
    wc[0] = U(b, ORV_DENS, i, j, k);
    wc[1] = U(b, ORV_VELX, i, j, k);
    wc[2] = U(b, ORV_VELY, i, j, k);
    wc[3] = U(b, ORV_VELZ, i, j, k);
    wc[4] = U(b, ORV_PRES, i, j, k);
    if (p->mhd) {
        wc[5] = U(b, ORV_MAGX, i, j, k);
        wc[6] = U(b, ORV_MAGY, i, j, k);
        wc[7] = U(b, ORV_MAGZ, i, j, k);
    }
    double hdt = 0.5 * dt;
    double hd[3] = {0.5 * dt / del[0], 0.5 * dt / del[1], 0.5 * dt / del[2]};
    (void)hdt;

    /* multidimensional MHD terms, hy_uhd_dataReconstOneStep.F90:364-424 */
    double aBn[3][NP], dnBn[3] = {0.0, 0.0, 0.0};
    memset(aBn, 0, sizeof aBn);
    if (p->mhd) {
        double uB = wc[1] * wc[5] + wc[2] * wc[6] + wc[3] * wc[7];
        double row[NP] = {0.0, -wc[5] / wc[0], -wc[6] / wc[0], -wc[7] / wc[0],
                          (p->gamma - 1.0) * uB, 0.0, -wc[2], -wc[3]};
        for (int v = 0; v < NP; ++v) { aBn[0][v] = row[v]; aBn[1][v] = row[v]; aBn[2][v] = row[v]; }
        aBn[1][5] = -wc[1]; aBn[1][6] = 0.0;
        aBn[2][5] = -wc[1]; aBn[2][7] = 0.0;
        aBn[2][6] = -wc[2];
        int n = b->n;
        dnBn[0] = b->f[0][fidx(n, 0, i + 1, j, k)] - b->f[0][fidx(n, 0, i, j, k)];
        dnBn[1] = b->f[1][fidx(n, 1, i, j + 1, k)] - b->f[1][fidx(n, 1, i, j, k)];
        dnBn[2] = b->f[2][fidx(n, 2, i, j, k + 1)] - b->f[2][fidx(n, 2, i, j, k)];
    }

    /* (I) normal-direction reconstruction */
    double sig[3][NP];
    for (int d = 0; d < 3; ++d) {
        double qs[5][NP];
        for (int m = 0; m < 5; ++m) {
            int ii = i + (d == 0 ? m - 2 : 0), jj = j + (d == 1 ? m - 2 : 0),
                kk = k + (d == 2 ? m - 2 : 0);
            double w[NP] = {U(b, ORV_DENS, ii, jj, kk), U(b, ORV_VELX, ii, jj, kk),
                            U(b, ORV_VELY, ii, jj, kk), U(b, ORV_VELZ, ii, jj, kk),
                            U(b, ORV_PRES, ii, jj, kk), 0.0, 0.0, 0.0};
            if (p->mhd) {
                w[5] = U(b, ORV_MAGX, ii, jj, kk);
                w[6] = U(b, ORV_MAGY, ii, jj, kk);
                w[7] = U(b, ORV_MAGZ, ii, jj, kk);
            }
            for (int s = 0; s < NP; ++s) qs[m][s] = w[rot_slot(d, s)];
        }
        double wp[NP], wn[NP], sg[NP];
        ppm_normal(p, qs, dt / del[d], wp, wn, sg);
        for (int s = 0; s < NP; ++s) {
            int v = rot_slot(d, s);
            o->wp[d][v] = wp[s];
            o->wn[d][v] = wn[s];
            sig[d][v] = sg[s];
        }
        if (p->mhd) {
            /* normal-direction dnBn source term inside the PPM call */
            for (int v = 0; v < nv; ++v) {
                o->wp[d][v] = o->wp[d][v] - hd[d] * aBn[d][v] * dnBn[d];
                o->wn[d][v] = o->wn[d][v] - hd[d] * aBn[d][v] * dnBn[d];
            }
        }
    }

    /* (Ia) hybrid order before the transverse corrections, :934-999 */
    int comp = 0, flags = 0;
    unsigned char code[3] = {0, 0, 0};
    if (p->hybrid_order) {
        double cs = p->gamma * wc[4] + (wc[5] * wc[5] + wc[6] * wc[6] + wc[7] * wc[7]);
        cs = sqrt(cs / wc[0]);
        comp = divu_min < p->hybrid_kappa * cs;
        if (comp) {
            for (int d = 0; d < 3; ++d) {
                if (rh_fail(p->gamma, wc[0], o->wp[d][0]) || rh_fail(p->gamma, wc[0], o->wn[d][0])) {
                    for (int v = 0; v < NP; ++v) {
                        o->wp[d][v] = wc[v];
                        o->wn[d][v] = wc[v];
                    }
                    if (p->fallback_lower_cfl) code[d] |= 1;
                    flags |= 2;
                }
            }
        }
    }

    /* (II) transverse corrections, :1006-1089 */
    for (int v = 0; v < nv; ++v) {
        o->wn[0][v] = o->wn[0][v] - hd[1] * sig[1][v];
        o->wp[0][v] = o->wp[0][v] - hd[1] * sig[1][v];
        o->wn[1][v] = o->wn[1][v] - hd[0] * sig[0][v];
        o->wp[1][v] = o->wp[1][v] - hd[0] * sig[0][v];
    }
    if (p->mhd) {
        for (int v = 0; v < nv; ++v) {
            o->wn[0][v] = o->wn[0][v] - hd[1] * aBn[1][v] * dnBn[1];
            o->wp[0][v] = o->wp[0][v] - hd[1] * aBn[1][v] * dnBn[1];
            o->wn[1][v] = o->wn[1][v] - hd[0] * aBn[0][v] * dnBn[0];
            o->wp[1][v] = o->wp[1][v] - hd[0] * aBn[0][v] * dnBn[0];
        }
    }
    for (int v = 0; v < nv; ++v) {
        o->wn[0][v] = o->wn[0][v] - hd[2] * sig[2][v];
        o->wp[0][v] = o->wp[0][v] - hd[2] * sig[2][v];
        o->wn[1][v] = o->wn[1][v] - hd[2] * sig[2][v];
        o->wp[1][v] = o->wp[1][v] - hd[2] * sig[2][v];
        o->wn[2][v] = o->wn[2][v] - hd[0] * sig[0][v] - hd[1] * sig[1][v];
        o->wp[2][v] = o->wp[2][v] - hd[0] * sig[0][v] - hd[1] * sig[1][v];
    }
    if (p->mhd) {
        for (int v = 0; v < nv; ++v) {
            o->wn[0][v] = o->wn[0][v] - hd[2] * aBn[2][v] * dnBn[2];
            o->wp[0][v] = o->wp[0][v] - hd[2] * aBn[2][v] * dnBn[2];
            o->wn[1][v] = o->wn[1][v] - hd[2] * aBn[2][v] * dnBn[2];
            o->wp[1][v] = o->wp[1][v] - hd[2] * aBn[2][v] * dnBn[2];
            o->wn[2][v] = o->wn[2][v] - hd[0] * aBn[0][v] * dnBn[0] - hd[1] * aBn[1][v] * dnBn[1];
            o->wp[2][v] = o->wp[2][v] - hd[0] * aBn[0][v] * dnBn[0] - hd[1] * aBn[1][v] * dnBn[1];
        }
    }

    /* (Ib) hybrid order after the transverse corrections, :1150-1218; any
     * direction's fallback lowers the cell's CFL to 0.25 (3-D) */
    if (comp) {
        for (int d = 0; d < 3; ++d) {
            if (rh_fail(p->gamma, wc[0], o->wp[d][0]) || rh_fail(p->gamma, wc[0], o->wn[d][0])) {
                for (int v = 0; v < NP; ++v) {
                    o->wp[d][v] = wc[v];
                    o->wn[d][v] = wc[v];
                }
                code[d] |= 2;
                flags |= 4;
            }
        }
    }

    /* (IV) positivity fallback, :1230-1272, lowering the cell's CFL */
    for (int d = 0; d < 3; ++d) {
        if (o->wn[d][0] < 0.0 || o->wp[d][0] < 0.0 || o->wn[d][4] < 0.0 || o->wp[d][4] < 0.0) {
            for (int v = 0; v < NP; ++v) {
                o->wn[d][v] = wc[v];
                o->wp[d][v] = wc[v];
            }
            code[d] |= 1;
            flags |= 1;
        }
    }
    if (codes) {
        codes[0] = code[0];
        codes[1] = code[1];
        codes[2] = code[2];
    }
    return flags;
}

/* ------------------------------------------------------------ Riemann */

typedef struct face_flux {
    double f[NP]; /* rho, mx, my, mz, E, Bx, By, Bz (unrotated) */
    double feint; /* rho*e_int */
    double un;    /* face normal velocity for div(v) */
} face_flux;

/* rotated conserved flux of one state: rho, vn, vt1, vt2, p, Bn, Bt1, Bt2 */
static void hllc(double gam, const double* L, const double* R, double* F, double* un)
{
    double gm1 = gam - 1.0;
    double aL = sqrt(gam * L[4] / L[0]), aR = sqrt(gam * R[4] / R[0]);
    double SL = fmin(L[1] - aL, R[1] - aR);
    double SR = fmax(L[1] + aL, R[1] + aR);
    double EL = L[4] / gm1 + 0.5 * L[0] * (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]);
    double ER = R[4] / gm1 + 0.5 * R[0] * (R[1] * R[1] + R[2] * R[2] + R[3] * R[3]);
    double FL[5] = {L[0] * L[1], L[0] * L[1] * L[1] + L[4], L[0] * L[1] * L[2], L[0] * L[1] * L[3],
                    L[1] * (EL + L[4])};
    double FR[5] = {R[0] * R[1], R[0] * R[1] * R[1] + R[4], R[0] * R[1] * R[2], R[0] * R[1] * R[3],
                    R[1] * (ER + R[4])};
    for (int s = 0; s < NP; ++s) F[s] = 0.0;
    if (SL >= 0.0) {
        for (int s = 0; s < 5; ++s) F[s] = FL[s];
        *un = L[1];
        return;
    }
    if (SR <= 0.0) {
        for (int s = 0; s < 5; ++s) F[s] = FR[s];
        *un = R[1];
        return;
    }
    double SM = (R[4] - L[4] + L[0] * L[1] * (SL - L[1]) - R[0] * R[1] * (SR - R[1])) /
                (L[0] * (SL - L[1]) - R[0] * (SR - R[1]));
    *un = SM;
    const double* W = SM >= 0.0 ? L : R;
    double S = SM >= 0.0 ? SL : SR;
    double E = SM >= 0.0 ? EL : ER;
    const double* FW = SM >= 0.0 ? FL : FR;
    double fac = W[0] * (S - W[1]) / (S - SM);
    double Us[5] = {fac, fac * SM, fac * W[2], fac * W[3],
                    fac * (E / W[0] + (SM - W[1]) * (SM + W[4] / (W[0] * (S - W[1]))))};
    double Uw[5] = {W[0], W[0] * W[1], W[0] * W[2], W[0] * W[3], E};
    for (int s = 0; s < 5; ++s) F[s] = FW[s] + S * (Us[s] - Uw[s]);
}

static void mhd_flux(const double* W, double bx, double E, double pT, double* F)
{
    double vB = W[1] * bx + W[2] * W[6] + W[3] * W[7];
    F[0] = W[0] * W[1];
    F[1] = W[0] * W[1] * W[1] + pT - bx * bx;
    F[2] = W[0] * W[1] * W[2] - bx * W[6];
    F[3] = W[0] * W[1] * W[3] - bx * W[7];
    F[4] = (E + pT) * W[1] - bx * vB;
    F[5] = 0.0;
    F[6] = W[6] * W[1] - bx * W[2];
    F[7] = W[7] * W[1] - bx * W[3];
}

static void hlld(double gam, const double* L, const double* R, double* F, double* un)
{
    const double gm1 = gam - 1.0;
    const double bx = L[5]; /* both states carry the face value */
    double bx2 = bx * bx;
    double BL2 = bx2 + L[6] * L[6] + L[7] * L[7];
    double BR2 = bx2 + R[6] * R[6] + R[7] * R[7];
    double pTL = L[4] + 0.5 * BL2, pTR = R[4] + 0.5 * BR2;
    double EL = L[4] / gm1 + 0.5 * L[0] * (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]) + 0.5 * BL2;
    double ER = R[4] / gm1 + 0.5 * R[0] * (R[1] * R[1] + R[2] * R[2] + R[3] * R[3]) + 0.5 * BR2;
    double gpl = gam * L[4], gpr = gam * R[4];
    double tl = (gpl + BL2) / L[0], tr = (gpr + BR2) / R[0];
    double cfL = sqrt(0.5 * (tl + sqrt(fmax(tl * tl - 4.0 * gpl * bx2 / (L[0] * L[0]), 0.0))));
    double cfR = sqrt(0.5 * (tr + sqrt(fmax(tr * tr - 4.0 * gpr * bx2 / (R[0] * R[0]), 0.0))));
    double cmax = fmax(cfL, cfR);
    double SL = fmin(L[1], R[1]) - cmax;
    double SR = fmax(L[1], R[1]) + cmax;
    double FL[NP], FR[NP];
    mhd_flux(L, bx, EL, pTL, FL);
    mhd_flux(R, bx, ER, pTR, FR);
    if (SL >= 0.0) {
        for (int s = 0; s < NP; ++s) F[s] = FL[s];
        *un = L[1];
        return;
    }
    if (SR <= 0.0) {
        for (int s = 0; s < NP; ++s) F[s] = FR[s];
        *un = R[1];
        return;
    }
    double sdl = SL - L[1], sdr = SR - R[1];
    double den = sdr * R[0] - sdl * L[0];
    double SM = (sdr * R[0] * R[1] - sdl * L[0] * L[1] - pTR + pTL) / den;
    double pTs = (sdr * R[0] * pTL - sdl * L[0] * pTR + L[0] * R[0] * sdr * sdl * (R[1] - L[1])) / den;
    *un = SM;
    /* single-star states */
    double Us[2][NP], Uo[2][NP], Fo[2][NP], Ss[2], sqs[2];
    double vst[2], wst[2], byst[2], bzst[2], vBst[2];
    const double* Ws[2] = {L, R};
    double Es[2] = {EL, ER}, Sx[2] = {SL, SR}, pTx[2] = {pTL, pTR};
    for (int a = 0; a < 2; ++a) {
        const double* W = Ws[a];
        double S = Sx[a];
        double sd = S - W[1];
        double rs = W[0] * sd / (S - SM);
        double t1 = W[0] * sd * (S - SM);
        double dd = t1 - bx2;
        double vs, ws, bys, bzs;
        if (fabs(dd) < 1e-12 * (fabs(t1) + bx2)) {
            vs = W[2];
            ws = W[3];
            bys = W[6];
            bzs = W[7];
        } else {
            double q = (SM - W[1]) / dd;
            vs = W[2] - bx * W[6] * q;
            ws = W[3] - bx * W[7] * q;
            double r = (W[0] * sd * sd - bx2) / dd;
            bys = W[6] * r;
            bzs = W[7] * r;
        }
        double vB = W[1] * bx + W[2] * W[6] + W[3] * W[7];
        double vBs = SM * bx + vs * bys + ws * bzs;
        double Est = (sd * Es[a] - pTx[a] * W[1] + pTs * SM + bx * (vB - vBs)) / (S - SM);
        Us[a][0] = rs; Us[a][1] = rs * SM; Us[a][2] = rs * vs; Us[a][3] = rs * ws;
        Us[a][4] = Est; Us[a][5] = bx; Us[a][6] = bys; Us[a][7] = bzs;
        Uo[a][0] = W[0]; Uo[a][1] = W[0] * W[1]; Uo[a][2] = W[0] * W[2]; Uo[a][3] = W[0] * W[3];
        Uo[a][4] = Es[a]; Uo[a][5] = bx; Uo[a][6] = W[6]; Uo[a][7] = W[7];
        for (int s = 0; s < NP; ++s) Fo[a][s] = (a == 0 ? FL[s] : FR[s]);
        sqs[a] = sqrt(rs);
        vst[a] = vs; wst[a] = ws; byst[a] = bys; bzst[a] = bzs; vBst[a] = vBs;
    }
    Ss[0] = SM - fabs(bx) / sqs[0];
    Ss[1] = SM + fabs(bx) / sqs[1];
    if (Ss[0] >= 0.0) {
        for (int s = 0; s < NP; ++s) F[s] = Fo[0][s] + SL * (Us[0][s] - Uo[0][s]);
        return;
    }
    if (Ss[1] <= 0.0) {
        for (int s = 0; s < NP; ++s) F[s] = Fo[1][s] + SR * (Us[1][s] - Uo[1][s]);
        return;
    }
    /* double-star states */
    double sgn = bx >= 0.0 ? 1.0 : -1.0;
    double isum = 1.0 / (sqs[0] + sqs[1]);
    double vss = (sqs[0] * vst[0] + sqs[1] * vst[1] + (byst[1] - byst[0]) * sgn) * isum;
    double wss = (sqs[0] * wst[0] + sqs[1] * wst[1] + (bzst[1] - bzst[0]) * sgn) * isum;
    double byss = (sqs[0] * byst[1] + sqs[1] * byst[0] + sqs[0] * sqs[1] * (vst[1] - vst[0]) * sgn) * isum;
    double bzss = (sqs[0] * bzst[1] + sqs[1] * bzst[0] + sqs[0] * sqs[1] * (wst[1] - wst[0]) * sgn) * isum;
    double vBss = SM * bx + vss * byss + wss * bzss;
    int a = SM >= 0.0 ? 0 : 1;
    double Ess = a == 0 ? Us[0][4] - sqs[0] * (vBst[0] - vBss) * sgn
                        : Us[1][4] + sqs[1] * (vBst[1] - vBss) * sgn;
    double Uss[NP] = {Us[a][0], Us[a][0] * SM, Us[a][0] * vss, Us[a][0] * wss, Ess, bx, byss, bzss};
    double S = Sx[a], Sst = Ss[a];
    for (int s = 0; s < NP; ++s)
        F[s] = Fo[a][s] + S * (Us[a][s] - Uo[a][s]) + Sst * (Uss[s] - Us[a][s]);
}

/* Riemann problem at a face of direction d between recon states wl (left
 * cell's + state) and wr (right cell's - state), unrotated primitive
 * 8-vectors; bnf is the face-centred normal B (mhd). */
static void face_solve(const orc_hydro_params* p, int d, const double* wl, const double* wr,
                       double bnf, face_flux* out)
{
    double L[NP], R[NP], Fr[NP];
    for (int s = 0; s < NP; ++s) {
        L[s] = wl[rot_slot(d, s)];
        R[s] = wr[rot_slot(d, s)];
    }
    double un;
    if (p->mhd) {
        L[5] = bnf;
        R[5] = bnf;
        hlld(p->gamma, L, R, Fr, &un);
    } else {
        hllc(p->gamma, L, R, Fr, &un);
    }
    for (int s = 0; s < NP; ++s) out->f[rot_slot(d, s)] = Fr[s];
    double gm1 = p->gamma - 1.0;
    double eL = L[4] / (gm1 * L[0]), eR = R[4] / (gm1 * R[0]);
    out->feint = Fr[0] * (Fr[0] >= 0.0 ? eL : eR);
    out->un = un;
}

/* ------------------------------------------------------------ block update */

/* Edge electric field at time n along c at edge (A, B, C): the mean of the
 * four cell-centred E_c = -(v x B)_c = v_b B_a - v_a B_b around it (a =
 * c + 1, b = c + 2 cyclically; the edge sits at A - 1/2 along a and B - 1/2
 * along b, C is its cell index along c), summed in a fixed order. */
static double edge_e_n(const blk* b, int c, int A, int B, int C)
{
    const int a = (c + 1) % 3, bb = (c + 2) % 3;
    double e[2][2];
    for (int ia = 0; ia < 2; ++ia)
        for (int ib = 0; ib < 2; ++ib) {
            int x[3];
            x[a] = A - 1 + ia;
            x[bb] = B - 1 + ib;
            x[c] = C;
            double va = U(b, ORV_VELX + a, x[0], x[1], x[2]), vb = U(b, ORV_VELX + bb, x[0], x[1], x[2]);
            double Ba = U(b, ORV_MAGX + a, x[0], x[1], x[2]), Bb = U(b, ORV_MAGX + bb, x[0], x[1], x[2]);
            e[ia][ib] = vb * Ba - va * Bb;
        }
    return 0.25 * (((e[0][0] + e[0][1]) + e[1][0]) + e[1][1]);
}

/* The normal field of face (I, J, K) of direction d at t + dt/2: a
 * constrained-transport half step, dB_d/dt = -(d_a E_b - d_b E_a), with the
 * time-n edge fields of edge_e_n (Gardiner & Stone 2005 sec. 4 and 2008
 * sec. 5: the longitudinal field of the Riemann problems at the half step).
 * Without it the face fluxes pair the normal field at time n with
 * time-centred transverse states, and the contact-upwinded edge fields
 * amplify: a weak field loop advected diagonally gains magnetic energy. */
static double face_b_half(const blk* b, int d, int I, int J, int K, const double* dtd)
{
    const int a = (d + 1) % 3, bb = (d + 2) % 3;
    int F[3] = {I, J, K};
    /* edges along bb (their a' = d, b' = a) at a -/+ 1/2; along a (a' = bb,
     * b' = d) at bb -/+ 1/2 */
    double eb_lo = edge_e_n(b, bb, F[d], F[a], F[bb]);
    double eb_hi = edge_e_n(b, bb, F[d], F[a] + 1, F[bb]);
    double ea_lo = edge_e_n(b, a, F[bb], F[d], F[a]);
    double ea_hi = edge_e_n(b, a, F[bb] + 1, F[d], F[a]);
    return b->f[d][fidx(b->n, d, I, J, K)] - 0.5 * (dtd[a] * (eb_hi - eb_lo) - dtd[bb] * (ea_hi - ea_lo));
}

static inline double upw(double f, double a, double b)
{
    return f > 0.0 ? a : (f < 0.0 ? b : 0.5 * (a + b));
}

/* Registers of one face: 16 x 16 face cells (first transverse axis
 * fastest, axes in x, y, z order) x ORC_NREG flux values. */
static const int reg_slots_note = ORC_NREG;

static void face_axes(int d, int* t1, int* t2)
{
    *t1 = d == 0 ? 1 : 0;
    *t2 = d == 2 ? 1 : 2;
}

/* Put this block's boundary fluxes (faces whose neighbour is coarser) and
 * take the fine-face means (faces whose neighbour is finer), as
 * Grid_putFluxData / Grid_conserveFluxes / Grid_getFluxData do on a
 * Cartesian mesh. `fl` are the block's face fluxes, n the padded size. */
static void flux_fix(const orc_fluxfix* fx, face_flux* const* fl, int n, int lo, int nxb)
{
#define FFX(d, i, j, k) fl[d][(i) + (int64_t)(n + 1) * ((j) + (int64_t)(n + 1) * (k))]
    for (int f = 0; f < 6; ++f) {
        const int d = f >> 1, side = f & 1;
        if (fx->type[f] == ORC_FACE_COARSER && fx->store[f]) {
            int t1, t2;
            face_axes(d, &t1, &t2);
            for (int c2 = 0; c2 < nxb; ++c2)
                for (int c1 = 0; c1 < nxb; ++c1) {
                    int I[3];
                    I[d] = side ? lo + nxb : lo;
                    I[t1] = lo + c1;
                    I[t2] = lo + c2;
                    const face_flux* o = &FFX(d, I[0], I[1], I[2]);
                    double* r = fx->store[f] + (size_t)(c1 + nxb * c2) * ORC_NREG;
                    for (int v = 0; v < 5; ++v) r[v] = o->f[v];
                    r[5] = o->feint;
                    r[6] = o->un;
                }
        }
    }
    for (int f = 0; f < 6; ++f) {
        const int d = f >> 1, side = f & 1;
        if (fx->type[f] != ORC_FACE_FINER) continue;
        int t1, t2;
        face_axes(d, &t1, &t2);
        const int h = nxb / 2;
        for (int c2 = 0; c2 < nxb; ++c2)
            for (int c1 = 0; c1 < nxb; ++c1) {
                const int q = (c1 >= h) + 2 * (c2 >= h);
                const double* r = fx->fine[f][q];
                if (!r) continue;
                const int g1 = 2 * (c1 - h * (c1 >= h)), g2 = 2 * (c2 - h * (c2 >= h));
                const double* r00 = r + (size_t)(g1 + nxb * g2) * ORC_NREG;
                const double* r10 = r + (size_t)(g1 + 1 + nxb * g2) * ORC_NREG;
                const double* r01 = r + (size_t)(g1 + nxb * (g2 + 1)) * ORC_NREG;
                const double* r11 = r + (size_t)(g1 + 1 + nxb * (g2 + 1)) * ORC_NREG;
                double m[ORC_NREG];
                for (int v = 0; v < ORC_NREG; ++v) m[v] = 0.25 * (((r00[v] + r10[v]) + r01[v]) + r11[v]);
                int I[3];
                I[d] = side ? lo + nxb : lo;
                I[t1] = lo + c1;
                I[t2] = lo + c2;
                face_flux* o = &FFX(d, I[0], I[1], I[2]);
                for (int v = 0; v < 5; ++v) o->f[v] = m[v];
                o->feint = m[5];
                o->un = m[6];
            }
    }
#undef FFX
    (void)reg_slots_note;
}

static int ring_index(int A, int B) { return B == 0 ? A : (B == 16 ? 17 + A : (A == 0 ? 33 + B : 48 + B)); }

static void ring_edge(int q, int* A, int* B)
{
    if (q < 17) { *A = q; *B = 0; }
    else if (q < 34) { *A = q - 17; *B = 16; }
    else if (q < 49) { *A = 0; *B = q - 33; }
    else { *A = 16; *B = q - 48; }
}

static int orc_leaf_at(const int* level, const int* child, const int* root, int nr0, int nr1, int maxlevel,
                       long long X, long long Y, long long Z);
static long long orc_wrap(long long x, long long n);

/* Edge electric fields at fine-coarse boundaries: store this block's
 * surface edges, then replace each surface edge that a leaf one level finer
 * also carries by the mean of its two fine edges. The surrounding cells of
 * an edge outside the block are tried in a fixed order ((A-1, B-1), (A,
 * B-1), (A-1, B), (A, B) in (a, b)); the first that lies in a leaf of level
 * L + 1 gives the fine edges (every such leaf carries the same values).
 * EE(c, i, j, k) addresses the block's edge fields, lo its first interior
 * index. */
static void edge_fix(const orc_fluxfix* fx, double* const* emf, int n, int lo)
{
#define EEF(c, i, j, k) emf[c][(i) + (int64_t)(n + 1) * ((j) + (int64_t)(n + 1) * (k))]
    const int b = fx->b, L = fx->level[b];
    double* mine = fx->ereg + (size_t)b * ORC_NSURF;
    for (int c = 0; c < 3; ++c)
        for (int C = 0; C < 16; ++C)
            for (int q = 0; q < ORC_NRING; ++q) {
                int A, B, I[3];
                ring_edge(q, &A, &B);
                I[(c + 1) % 3] = lo + A;
                I[(c + 2) % 3] = lo + B;
                I[c] = lo + C;
                mine[((size_t)c * 16 + C) * ORC_NRING + q] = EEF(c, I[0], I[1], I[2]);
            }
    const long long S = 1LL << (fx->maxlevel - L); /* level-L cell in finest cells */
    for (int c = 0; c < 3; ++c) {
        const int a = (c + 1) % 3, bb = (c + 2) % 3;
        for (int C = 0; C < 16; ++C)
            for (int q = 0; q < ORC_NRING; ++q) {
                int A, B;
                ring_edge(q, &A, &B);
                for (int cand = 0; cand < 4; ++cand) {
                    const int ia = cand & 1, ib = cand >> 1;
                    const int cell[2] = {A - 1 + ia, B - 1 + ib};
                    if (cell[0] >= 0 && cell[0] < 16 && cell[1] >= 0 && cell[1] < 16) continue;
                    /* centre of the outside cell, finest units, periodic */
                    int ci[3];
                    ci[a] = cell[0];
                    ci[bb] = cell[1];
                    ci[c] = C;
                    long long X[3], g[3];
                    for (int d = 0; d < 3; ++d) {
                        const long long M = (long long)fx->nr[d] * 16 << L; /* level-L cells across */
                        g[d] = orc_wrap((long long)fx->coord[3 * b + d] * 16 + ci[d], M);
                        X[d] = g[d] * S + S / 2;
                    }
                    const int F = orc_leaf_at(fx->level, fx->child, fx->root, fx->nr[0], fx->nr[1], fx->maxlevel,
                                              X[0], X[1], X[2]);
                    if (F < 0 || F >= fx->nnodes || fx->level[F] != L + 1) continue;
                    /* the fine cells of the outside coarse cell start at
                     * 2 g - 16 coord_F; the edge is on the upper side of
                     * the coarse cell when ia (ib) = 0 */
                    const int Af = (int)(2 * g[a] - 16LL * fx->coord[3 * F + a]) + (ia ? 0 : 2);
                    const int Bf = (int)(2 * g[bb] - 16LL * fx->coord[3 * F + bb]) + (ib ? 0 : 2);
                    const int Cf = (int)(2 * g[c] - 16LL * fx->coord[3 * F + c]);
                    const double* r = fx->ereg + (size_t)F * ORC_NSURF + ((size_t)c * 16 + Cf) * ORC_NRING +
                                      ring_index(Af, Bf);
                    int I[3];
                    I[a] = lo + A;
                    I[bb] = lo + B;
                    I[c] = lo + C;
                    EEF(c, I[0], I[1], I[2]) = 0.5 * (r[0] + r[ORC_NRING]);
                    break;
                }
            }
    }
#undef EEF
}

static int unsplit_block(const orc_hydro_params* p, double* u, double* bxf, double* byf, double* bzf,
                         double dt, double dx, double dy, double dz, const orc_fluxfix* fx);

int orc_unsplit_block(const orc_hydro_params* p, double* u, double* bxf, double* byf, double* bzf,
                      double dt, double dx, double dy, double dz)
{
    return unsplit_block(p, u, bxf, byf, bzf, dt, dx, dy, dz, NULL);
}

int orc_unsplit_block_fc(const orc_hydro_params* p, double* u, double* bxf, double* byf, double* bzf,
                         double dt, double dx, double dy, double dz, const orc_fluxfix* fx)
{
    return unsplit_block(p, u, bxf, byf, bzf, dt, dx, dy, dz, fx);
}

static int unsplit_block(const orc_hydro_params* p, double* u, double* bxf, double* byf, double* bzf,
                         double dt, double dx, double dy, double dz, const orc_fluxfix* fx)
{
    const int ng = p->nguard, nxb = p->nxb, n = nxb + 2 * ng;
    const int lo = ng, hi = ng + nxb - 1; /* interior cells */
    const int rlo = lo - 1, rhi = hi + 1;  /* reconstruction / flux band */
    const int64_t n3 = (int64_t)n * n * n;
    blk b = {n, ng, nxb, u, {bxf, byf, bzf}};
    double del[3] = {dx, dy, dz};
    const double gm1 = p->gamma - 1.0;

    ORC_PHASE(-1);
    recon_out* rec = (recon_out*)calloc((size_t)n3, sizeof(recon_out));
    /* undivided velocity divergence over the band (hybrid order) */
    double* divu = (double*)calloc((size_t)n3, sizeof(double));
    if (p->hybrid_order) {
        for (int k = rlo; k <= rhi; ++k)
            for (int j = rlo; j <= rhi; ++j)
                for (int i = rlo; i <= rhi; ++i)
                    divu[cidx(n, i, j, k)] = 0.5 * (U(&b, ORV_VELX, i + 1, j, k) - U(&b, ORV_VELX, i - 1, j, k)) +
                                             0.5 * (U(&b, ORV_VELY, i, j + 1, k) - U(&b, ORV_VELY, i, j - 1, k)) +
                                             0.5 * (U(&b, ORV_VELZ, i, j, k + 1) - U(&b, ORV_VELZ, i, j, k - 1));
    }
    const int k4 = p->mhd ? 1 : 2;
    int nfall = 0;
    for (int k = rlo; k <= rhi; ++k)
        for (int j = rlo; j <= rhi; ++j)
            for (int i = rlo; i <= rhi; ++i) {
                double dmin = 1e300;
                if (p->hybrid_order) {
                    for (int kk = k - k4; kk <= k + k4; ++kk)
                        for (int jj = j - k4; jj <= j + k4; ++jj)
                            for (int ii = i - k4; ii <= i + k4; ++ii) {
                                if (ii < rlo || ii > rhi || jj < rlo || jj > rhi || kk < rlo || kk > rhi) continue;
                                double x = divu[cidx(n, ii, jj, kk)];
                                if (x < dmin) dmin = x;
                            }
                }
                unsigned char codes[3];
                int fl = recon_cell(p, &b, i, j, k, dt, del, dmin, &rec[cidx(n, i, j, k)], codes);
                nfall += fl & 1;
                if (p->cflc && i >= lo && i <= hi && j >= lo && j <= hi && k >= lo && k <= hi)
                    p->cflc[(i - lo) + nxb * ((j - lo) + nxb * (k - lo))] = (unsigned char)(codes[0] | codes[1] | codes[2]);
            }
    free(divu);
    ORC_PHASE(0);

    /* fluxes: face index I = left face of cell I; faces lo..hi+1 in the
     * normal direction, cells rlo..rhi across */
    int64_t nf = (int64_t)(n + 1) * (n + 1) * (n + 1);
    const double dtdf[3] = {dt / dx, dt / dy, dt / dz};
    face_flux* fl[3];
    for (int d = 0; d < 3; ++d) fl[d] = (face_flux*)calloc((size_t)nf, sizeof(face_flux));
#define FF(d, i, j, k) fl[d][(i) + (int64_t)(n + 1) * ((j) + (int64_t)(n + 1) * (k))]
    for (int d = 0; d < 3; ++d) {
        for (int k = rlo; k <= rhi + (d == 2); ++k)
            for (int j = rlo; j <= rhi + (d == 1); ++j)
                for (int i = rlo; i <= rhi + (d == 0); ++i) {
                    int I = i, J = j, K = k;
                    int in = (d == 0 ? (I >= lo && I <= hi + 1) : (I >= rlo && I <= rhi)) &&
                             (d == 1 ? (J >= lo && J <= hi + 1) : (J >= rlo && J <= rhi)) &&
                             (d == 2 ? (K >= lo && K <= hi + 1) : (K >= rlo && K <= rhi));
                    if (!in) continue;
                    int il = I - (d == 0), jl = J - (d == 1), kl = K - (d == 2);
                    const double* wl = rec[cidx(n, il, jl, kl)].wp[d];
                    const double* wr = rec[cidx(n, I, J, K)].wn[d];
                    double bnf = p->mhd ? face_b_half(&b, d, I, J, K, dtdf) : 0.0;
                    face_flux* o = &FF(d, I, J, K);
                    face_solve(p, d, wl, wr, bnf, o);
                    if (p->use_avisc) {
                        int vn = ORV_VELX + d;
                        double dv = U(&b, vn, I, J, K) - U(&b, vn, il, jl, kl);
                        double vis = p->cvisc * fmax(-dv, 0.0);
                        if (vis > 0.0) {
                            /* conserved differences (left minus right) */
                            double rl = U(&b, ORV_DENS, il, jl, kl), rr = U(&b, ORV_DENS, I, J, K);
                            double ul[NP], ur[NP];
                            double vl[3] = {U(&b, ORV_VELX, il, jl, kl), U(&b, ORV_VELY, il, jl, kl), U(&b, ORV_VELZ, il, jl, kl)};
                            double vr[3] = {U(&b, ORV_VELX, I, J, K), U(&b, ORV_VELY, I, J, K), U(&b, ORV_VELZ, I, J, K)};
                            double Bl[3] = {0, 0, 0}, Br[3] = {0, 0, 0};
                            if (p->mhd) {
                                for (int c = 0; c < 3; ++c) {
                                    Bl[c] = U(&b, ORV_MAGX + c, il, jl, kl);
                                    Br[c] = U(&b, ORV_MAGX + c, I, J, K);
                                }
                            }
                            double pl = U(&b, ORV_PRES, il, jl, kl), pr = U(&b, ORV_PRES, I, J, K);
                            ul[0] = rl; ur[0] = rr;
                            for (int c = 0; c < 3; ++c) { ul[1 + c] = rl * vl[c]; ur[1 + c] = rr * vr[c]; }
                            ul[4] = pl / gm1 + 0.5 * rl * (vl[0] * vl[0] + vl[1] * vl[1] + vl[2] * vl[2]) +
                                    0.5 * (Bl[0] * Bl[0] + Bl[1] * Bl[1] + Bl[2] * Bl[2]);
                            ur[4] = pr / gm1 + 0.5 * rr * (vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2]) +
                                    0.5 * (Br[0] * Br[0] + Br[1] * Br[1] + Br[2] * Br[2]);
                            for (int c = 0; c < 3; ++c) { ul[5 + c] = Bl[c]; ur[5 + c] = Br[c]; }
                            for (int s = 0; s < NP; ++s) {
                                if (s == 5 + d) continue;
                                if (!p->mhd && s >= 5) continue;
                                o->f[s] = o->f[s] + vis * (ul[s] - ur[s]);
                            }
                            double el = rl * U(&b, ORV_EINT, il, jl, kl);
                            double er = rr * U(&b, ORV_EINT, I, J, K);
                            o->feint = o->feint + vis * (el - er);
                        }
                    }
                }
    }

    ORC_PHASE(1);
    /* edge electric fields (mhd), Gardiner & Stone 2005 eqs. 41, 50 */
    double* emf[3] = {NULL, NULL, NULL};
    if (p->mhd) {
        for (int c = 0; c < 3; ++c) emf[c] = (double*)calloc((size_t)nf, sizeof(double));
#define EE(c, i, j, k) emf[c][(i) + (int64_t)(n + 1) * ((j) + (int64_t)(n + 1) * (k))]
        for (int c = 0; c < 3; ++c) {
            int a = (c + 1) % 3, bb = (c + 2) % 3;
            /* edge along c at face index A in a and B in bb; cell index in c */
            for (int K = lo; K <= hi + 1; ++K)
                for (int J = lo; J <= hi + 1; ++J)
                    for (int I = lo; I <= hi + 1; ++I) {
                        int idx3[3] = {I, J, K};
                        if (idx3[c] > hi) continue; /* along-edge index is a cell index */
                        int A = idx3[a], B = idx3[bb], C = idx3[c];
                        /* helpers to address faces/cells by (a, b, c) coordinates */
#define AT(arr3, av, bv, cv) (arr3[a] = (av), arr3[bb] = (bv), arr3[c] = (cv))
                        int t[3];
                        /* a-face fluxes at (A, B-1), (A, B): E = -F_a(B_bb) */
                        AT(t, A, B - 1, C); face_flux* fa0 = &FF(a, t[0], t[1], t[2]);
                        AT(t, A, B, C);     face_flux* fa1 = &FF(a, t[0], t[1], t[2]);
                        /* b-face fluxes at (A-1, B), (A, B): E = +F_b(B_a) */
                        AT(t, A - 1, B, C); face_flux* fb0 = &FF(bb, t[0], t[1], t[2]);
                        AT(t, A, B, C);     face_flux* fb1 = &FF(bb, t[0], t[1], t[2]);
                        double ea0 = -fa0->f[5 + bb], ea1 = -fa1->f[5 + bb];
                        double eb0 = fb0->f[5 + a], eb1 = fb1->f[5 + a];
                        /* cell-centred reference E_c = -(v x B)_c at the four
                         * cells, at the fluxes' time level t + dt/2: from the
                         * mean of the cell's own two face states along c (time
                         * centred by the tracing and by the transverse terms of
                         * the other two directions; v_a, v_b, B_a, B_b are
                         * tangential to c). A plane-parallel flow then gets the
                         * 1-D Riemann flux at every edge, as the method requires
                         * (Gardiner & Stone 2005 sec. 3) */
                        double ecc[2][2];
                        for (int ia = 0; ia < 2; ++ia)
                            for (int ib = 0; ib < 2; ++ib) {
                                AT(t, A - 1 + ia, B - 1 + ib, C);
                                const recon_out* rc = &rec[cidx(n, t[0], t[1], t[2])];
                                double va = 0.5 * (rc->wp[c][1 + a] + rc->wn[c][1 + a]);
                                double vb = 0.5 * (rc->wp[c][1 + bb] + rc->wn[c][1 + bb]);
                                double Ba = 0.5 * (rc->wp[c][5 + a] + rc->wn[c][5 + a]);
                                double Bb = 0.5 * (rc->wp[c][5 + bb] + rc->wn[c][5 + bb]);
                                ecc[ia][ib] = vb * Ba - va * Bb;
                            }
                        double eavg = 0.25 * (ea0 + ea1 + eb0 + eb1);
                        /* derivatives along bb on the a-face line, upwinded by
                         * the mass flux through the a-faces */
                        double dbm = upw(fa0->f[0], 2.0 * (eb0 - ecc[0][0]), 2.0 * (eb1 - ecc[1][0]));
                        double dbp = upw(fa1->f[0], 2.0 * (ecc[0][1] - eb0), 2.0 * (ecc[1][1] - eb1));
                        /* derivatives along a on the b-face line */
                        double dam = upw(fb0->f[0], 2.0 * (ea0 - ecc[0][0]), 2.0 * (ea1 - ecc[0][1]));
                        double dap = upw(fb1->f[0], 2.0 * (ecc[1][0] - ea0), 2.0 * (ecc[1][1] - ea1));
                        EE(c, I, J, K) = p->emf_average ? eavg : eavg + 0.125 * (dbm - dbp) + 0.125 * (dam - dap);
#undef AT
                    }
        }
    }

    ORC_PHASE(2);
    /* flux conservation at fine-coarse faces (after the electric fields,
     * which use the block's own fluxes) */
    if (fx) flux_fix(fx, fl, n, lo, nxb);
    /* edge electric fields at fine-coarse boundaries */
    if (fx && fx->ereg && p->mhd) edge_fix(fx, emf, n, lo);

    /* conservative update of the interior cells */
    double* unew = (double*)malloc(sizeof(double) * (size_t)(ORV_NVAR * n3));
    memcpy(unew, u, sizeof(double) * (size_t)(ORV_NVAR * n3));
    double dtd[3] = {dt / dx, dt / dy, dt / dz};
    /* new face fields (interior faces) */
    double* fnew[3] = {NULL, NULL, NULL};
    if (p->mhd) {
        for (int d = 0; d < 3; ++d) {
            int64_t sz = (int64_t)n * n * n + (int64_t)n * n;
            fnew[d] = (double*)malloc(sizeof(double) * (size_t)sz);
            memcpy(fnew[d], b.f[d], sizeof(double) * (size_t)sz);
        }
        for (int a = 0; a < 3; ++a) {
            int bb = (a + 1) % 3, c = (a + 2) % 3;
            for (int k = lo; k <= hi + (a == 2); ++k)
                for (int j = lo; j <= hi + (a == 1); ++j)
                    for (int i = lo; i <= hi + (a == 0); ++i) {
                        int t0[3] = {i, j, k}, t1[3] = {i, j, k}, t2[3] = {i, j, k}, t3[3] = {i, j, k};
                        /* B_a -= dt/d_b (E_c[b+1] - E_c[b]) - dt/d_c (E_b[c+1] - E_b[c]) */
                        t1[bb] += 1;
                        t3[c] += 1;
                        double ec0 = EE(c, t0[0], t0[1], t0[2]), ec1 = EE(c, t1[0], t1[1], t1[2]);
                        double eb0 = EE(bb, t2[0], t2[1], t2[2]), eb1 = EE(bb, t3[0], t3[1], t3[2]);
                        int64_t fi = fidx(n, a, i, j, k);
                        fnew[a][fi] = b.f[a][fi] - dtd[bb] * (ec1 - ec0) + dtd[c] * (eb1 - eb0);
                    }
        }
    }
    for (int k = lo; k <= hi; ++k)
        for (int j = lo; j <= hi; ++j)
            for (int i = lo; i <= hi; ++i) {
                int64_t ci = cidx(n, i, j, k);
                double rho = U(&b, ORV_DENS, i, j, k);
                double vx = U(&b, ORV_VELX, i, j, k), vy = U(&b, ORV_VELY, i, j, k), vz = U(&b, ORV_VELZ, i, j, k);
                double pr = U(&b, ORV_PRES, i, j, k);
                double Bc[3] = {0, 0, 0};
                if (p->mhd) for (int c = 0; c < 3; ++c) Bc[c] = U(&b, ORV_MAGX + c, i, j, k);
                double Uc[NP];
                Uc[0] = rho;
                Uc[1] = rho * vx; Uc[2] = rho * vy; Uc[3] = rho * vz;
                Uc[4] = pr / gm1 + 0.5 * rho * (vx * vx + vy * vy + vz * vz) +
                        0.5 * (Bc[0] * Bc[0] + Bc[1] * Bc[1] + Bc[2] * Bc[2]);
                Uc[5] = Bc[0]; Uc[6] = Bc[1]; Uc[7] = Bc[2];
                double re = rho * U(&b, ORV_EINT, i, j, k);
                face_flux* fxm = &FF(0, i, j, k); face_flux* fxp = &FF(0, i + 1, j, k);
                face_flux* fym = &FF(1, i, j, k); face_flux* fyp = &FF(1, i, j + 1, k);
                face_flux* fzm = &FF(2, i, j, k); face_flux* fzp = &FF(2, i, j, k + 1);
                double Un[NP];
                for (int s = 0; s < NP; ++s)
                    Un[s] = Uc[s] - dtd[0] * (fxp->f[s] - fxm->f[s]) - dtd[1] * (fyp->f[s] - fym->f[s]) -
                            dtd[2] * (fzp->f[s] - fzm->f[s]);
                /* dt * div v from the face velocities, as sum_d (dt/dx_d) dv_d */
                double dtdivv = dtd[0] * (fxp->un - fxm->un) + dtd[1] * (fyp->un - fym->un) +
                                dtd[2] * (fzp->un - fzm->un);
                double ren = re - dtd[0] * (fxp->feint - fxm->feint) - dtd[1] * (fyp->feint - fym->feint) -
                             dtd[2] * (fzp->feint - fzm->feint) - pr * dtdivv;
                double Bn[3] = {0, 0, 0};
                if (p->mhd) {
                    Bn[0] = 0.5 * (fnew[0][fidx(n, 0, i, j, k)] + fnew[0][fidx(n, 0, i + 1, j, k)]);
                    Bn[1] = 0.5 * (fnew[1][fidx(n, 1, i, j, k)] + fnew[1][fidx(n, 1, i, j + 1, k)]);
                    Bn[2] = 0.5 * (fnew[2][fidx(n, 2, i, j, k)] + fnew[2][fidx(n, 2, i, j, k + 1)]);
                }
                double rn = fmax(Un[0], p->smlrho);
                double ek = 0.5 * (Un[1] * Un[1] + Un[2] * Un[2] + Un[3] * Un[3]) / rn;
                double em = 0.5 * (Bn[0] * Bn[0] + Bn[1] * Bn[1] + Bn[2] * Bn[2]);
                if (p->mhd && p->energy_fix) em = 0.5 * (Un[5] * Un[5] + Un[6] * Un[6] + Un[7] * Un[7]);
                double eiE = ((Un[4] - ek) - em) / rn;
                double eia = ren / rn;
                double ei = (eiE > p->eint_switch * (Un[4] / rn)) ? eiE : eia;
                double pn = gm1 * rn * ei;
                if (pn < p->smallp) {
                    pn = p->smallp;
                    ei = pn / (gm1 * rn);
                }
                double vxn = Un[1] / rn, vyn = Un[2] / rn, vzn = Un[3] / rn;
                unew[ORV_DENS * n3 + ci] = rn;
                unew[ORV_VELX * n3 + ci] = vxn;
                unew[ORV_VELY * n3 + ci] = vyn;
                unew[ORV_VELZ * n3 + ci] = vzn;
                unew[ORV_PRES * n3 + ci] = pn;
                unew[ORV_EINT * n3 + ci] = ei;
                unew[ORV_ENER * n3 + ci] = ei + 0.5 * (vxn * vxn + vyn * vyn + vzn * vzn);
                if (p->mhd) {
                    unew[ORV_MAGX * n3 + ci] = Bn[0];
                    unew[ORV_MAGY * n3 + ci] = Bn[1];
                    unew[ORV_MAGZ * n3 + ci] = Bn[2];
                }
            }
    ORC_PHASE(3);
    memcpy(u, unew, sizeof(double) * (size_t)(ORV_NVAR * n3));
    if (p->mhd) {
        for (int d = 0; d < 3; ++d) {
            int64_t sz = (int64_t)n * n * n + (int64_t)n * n;
            memcpy(b.f[d], fnew[d], sizeof(double) * (size_t)sz);
            free(fnew[d]);
            free(emf[d]);
        }
    }
    free(unew);
    for (int d = 0; d < 3; ++d) free(fl[d]);
    free(rec);
#undef FF
#undef EE
    return nfall;
}

double orc_block_dt_limit(const orc_hydro_params* p, const double* u, double dx, double dy, double dz)
{
    const int ng = p->nguard, nxb = p->nxb, n = nxb + 2 * ng;
    const int64_t n3 = (int64_t)n * n * n;
    double del[3] = {dx, dy, dz};
    double best = 1e300;
    for (int k = ng; k < ng + nxb; ++k)
        for (int j = ng; j < ng + nxb; ++j)
            for (int i = ng; i < ng + nxb; ++i) {
                int64_t c = cidx(n, i, j, k);
                double rho = u[ORV_DENS * n3 + c], pr = u[ORV_PRES * n3 + c];
                double gp = p->gamma * pr;
                double B[3] = {0, 0, 0};
                if (p->mhd) for (int q = 0; q < 3; ++q) B[q] = u[(ORV_MAGX + q) * n3 + c];
                double B2 = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
                double t = (gp + B2) / rho;
                double rate = 0.0, cell = 1e300;
                for (int d = 0; d < 3; ++d) {
                    double v = fabs(u[(ORV_VELX + d) * n3 + c]);
                    double cf = sqrt(0.5 * (t + sqrt(fmax(t * t - 4.0 * gp * B[d] * B[d] / (rho * rho), 0.0))));
                    if (p->cfl_sum) {
                        rate = rate + (v + cf) / del[d];
                    } else {
                        double dtc = del[d] / (v + cf);
                        if (dtc < cell) cell = dtc;
                    }
                }
                if (!p->cfl_sum) {
                    if (p->cflc) {
                        int code = p->cflc[(i - ng) + nxb * ((j - ng) + nxb * (k - ng))];
                        if (code) cell = cell * orc_cfl_scale(p, code);
                    }
                    if (cell < best) best = cell;
                }
                if (p->cfl_sum) {
                    double lim = 1.0 / rate;
                    if (p->cflc) {
                        int code = p->cflc[(i - ng) + nxb * ((j - ng) + nxb * (k - ng))];
                        if (code) lim = lim * orc_cfl_scale(p, code);
                    }
                    if (lim < best) best = lim;
                }
            }
    return best;
}

void orc_fill_guards_periodic(const orc_hydro_params* p, int nbx, int nby, int nbz, double* u,
                              double* bx, double* by, double* bz)
{
    const int ng = p->nguard, nxb = p->nxb, n = nxb + 2 * ng;
    const int64_t n3 = (int64_t)n * n * n, fsz = n3 + (int64_t)n * n;
    const int nv = p->mhd ? ORV_NVAR : ORV_MAGX;
    int nb[3] = {nbx, nby, nbz};
    int NX[3] = {nbx * nxb, nby * nxb, nbz * nxb};
    int nblk = nbx * nby * nbz;
    for (int b = 0; b < nblk; ++b) {
        int bc[3] = {b % nbx, (b / nbx) % nby, b / (nbx * nby)};
        for (int k = 0; k < n; ++k)
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < n; ++i) {
                    int l[3] = {i, j, k};
                    int guard = 0;
                    for (int d = 0; d < 3; ++d) if (l[d] < ng || l[d] >= ng + nxb) guard = 1;
                    if (!guard) continue;
                    int ob[3], ol[3];
                    for (int d = 0; d < 3; ++d) {
                        int g = bc[d] * nxb + l[d] - ng;
                        g = ((g % NX[d]) + NX[d]) % NX[d];
                        ob[d] = g / nxb;
                        ol[d] = g % nxb + ng;
                    }
                    int o = ob[0] + nb[0] * (ob[1] + nb[1] * ob[2]);
                    for (int v = 0; v < nv; ++v)
                        u[(int64_t)b * ORV_NVAR * n3 + v * n3 + cidx(n, i, j, k)] =
                            u[(int64_t)o * ORV_NVAR * n3 + v * n3 + cidx(n, ol[0], ol[1], ol[2])];
                }
        if (!p->mhd) continue;
        double* fa[3] = {bx, by, bz};
        for (int d = 0; d < 3; ++d) {
            for (int k = 0; k < n + (d == 2); ++k)
                for (int j = 0; j < n + (d == 1); ++j)
                    for (int i = 0; i < n + (d == 0); ++i) {
                        int l[3] = {i, j, k};
                        int own = 1;
                        for (int e = 0; e < 3; ++e) {
                            int top = ng + nxb - 1 + (e == d);
                            if (l[e] < ng || l[e] > top) own = 0;
                        }
                        if (own) continue;
                        int ob[3], ol[3];
                        for (int e = 0; e < 3; ++e) {
                            int g = bc[e] * nxb + l[e] - ng;
                            g = ((g % NX[e]) + NX[e]) % NX[e];
                            ob[e] = g / nxb;
                            ol[e] = g % nxb + ng;
                        }
                        int o = ob[0] + nb[0] * (ob[1] + nb[1] * ob[2]);
                        fa[d][(int64_t)b * fsz + fidx(n, d, i, j, k)] =
                            fa[d][(int64_t)o * fsz + fidx(n, d, ol[0], ol[1], ol[2])];
                    }
        }
    }
}

void orc_conserved_totals(const orc_hydro_params* p, int nblocks, const double* u, const double* bx,
                          const double* by, const double* bz, double dx, double dy, double dz,
                          double* out)
{
    const int ng = p->nguard, nxb = p->nxb, n = nxb + 2 * ng;
    const int64_t n3 = (int64_t)n * n * n, fsz = n3 + (int64_t)n * n;
    double M = 0, Px = 0, Py = 0, Pz = 0, E = 0, dmax = 0, bmax = 0;
    double gm1 = p->gamma - 1.0;
    for (int b = 0; b < nblocks; ++b) {
        const double* ub = u + (int64_t)b * ORV_NVAR * n3;
        for (int k = ng; k < ng + nxb; ++k)
            for (int j = ng; j < ng + nxb; ++j)
                for (int i = ng; i < ng + nxb; ++i) {
                    int64_t c = cidx(n, i, j, k);
                    double r = ub[ORV_DENS * n3 + c];
                    double v[3] = {ub[ORV_VELX * n3 + c], ub[ORV_VELY * n3 + c], ub[ORV_VELZ * n3 + c]};
                    double B2 = 0;
                    if (p->mhd) {
                        for (int q = 0; q < 3; ++q) {
                            double bq = ub[(ORV_MAGX + q) * n3 + c];
                            B2 += bq * bq;
                            if (fabs(bq) > bmax) bmax = fabs(bq);
                        }
                        double dv = (bx[(int64_t)b * fsz + fidx(n, 0, i + 1, j, k)] - bx[(int64_t)b * fsz + fidx(n, 0, i, j, k)]) / dx +
                                    (by[(int64_t)b * fsz + fidx(n, 1, i, j + 1, k)] - by[(int64_t)b * fsz + fidx(n, 1, i, j, k)]) / dy +
                                    (bz[(int64_t)b * fsz + fidx(n, 2, i, j, k + 1)] - bz[(int64_t)b * fsz + fidx(n, 2, i, j, k)]) / dz;
                        if (fabs(dv) > dmax) dmax = fabs(dv);
                    }
                    M += r;
                    Px += r * v[0];
                    Py += r * v[1];
                    Pz += r * v[2];
                    E += ub[ORV_PRES * n3 + c] / gm1 + 0.5 * r * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) + 0.5 * B2;
                }
    }
    double vol = dx * dy * dz;
    out[0] = M * vol; out[1] = Px * vol; out[2] = Py * vol; out[3] = Pz * vol; out[4] = E * vol;
    out[5] = bmax > 0 ? dmax * dx / bmax : 0.0;
}

/* Test hook: the eigensystem of one rotated primitive 8-vector, R and L as
 * row-major 7x7 (unused rows/columns zero). */
void orc_test_eig(int mhd, double gam, const double* q8, double* lam, double* Rout, double* Lout)
{
    double R[MAXW][MAXW], L[MAXW][MAXW];
    if (mhd) eig_mhd(gam, q8, lam, R, L);
    else eig_hydro(gam, q8, lam, R, L);
    memcpy(Rout, R, sizeof R);
    memcpy(Lout, L, sizeof L);
}

/* ------------------------------------------------------------ AMR guard fill */

static int orc_leaf_at(const int* level, const int* child, const int* root, int nr0, int nr1, int maxlevel,
                       long long X, long long Y, long long Z)
{
    const long long S0 = 16LL << maxlevel;
    long long r[3] = {X / S0, Y / S0, Z / S0};
    int node = root[r[0] + nr0 * (r[1] + nr1 * r[2])];
    for (int l = 0; l <= maxlevel; ++l) {
        if (child[8 * node] < 0) break;
        long long half = S0 >> (l + 1);
        int c = (int)((X / half) & 1) | ((int)((Y / half) & 1) << 1) | ((int)((Z / half) & 1) << 2);
        node = child[8 * node + c];
    }
    (void)level;
    return node;
}

static long long orc_wrap(long long x, long long n) { return ((x % n) + n) % n; }

/* Guard cells and guard faces of every leaf of a block tree (periodic
 * domain): same-level neighbours are copied, a coarser neighbour's covering
 * cell is injected, a finer neighbour's covering cells are averaged
 * (8 cells; faces: the 4 fine faces on the coarse face); a fine guard face
 * that falls inside a coarse cell takes the mean of the two coarse faces. */
void orc_fill_guards_leaf(const orc_hydro_params* p, int b, const int* level, const int* coord,
                          const int* child, const int* root, int nr0, int nr1, int nr2, int maxlevel,
                          double* u, double* bx, double* by, double* bz)
{
    const int ng = p->nguard, nxb = p->nxb, n = nxb + 2 * ng;
    const int64_t n3 = (int64_t)n * n * n, fsz = n3 + (int64_t)n * n;
    const int nv = p->mhd ? ORV_NVAR : ORV_MAGX;
    const long long N[3] = {(long long)nr0 * nxb << maxlevel, (long long)nr1 * nxb << maxlevel,
                            (long long)nr2 * nxb << maxlevel};
    double* fa[3] = {bx, by, bz};
    {
        const int L = level[b];
        const long long s = 1LL << (maxlevel - L);
        const int* cd = coord + 3 * b;
        for (int k = 0; k < n; ++k)
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < n; ++i) {
                    int l3[3] = {i, j, k};
                    int guard = 0;
                    for (int d = 0; d < 3; ++d) if (l3[d] < ng || l3[d] >= ng + nxb) guard = 1;
                    if (!guard) continue;
                    long long lo[3], X[3];
                    for (int d = 0; d < 3; ++d) {
                        lo[d] = orc_wrap(((long long)cd[d] * nxb + l3[d] - ng) * s, N[d]);
                        X[d] = lo[d] + s / 2;
                    }
                    int m = orc_leaf_at(level, child, root, nr0, nr1, maxlevel, X[0], X[1], X[2]);
                    const long long sl = 1LL << (maxlevel - level[m]);
                    const int* sc = coord + 3 * m;
                    double* dst = u + (int64_t)b * ORV_NVAR * n3 + cidx(n, i, j, k);
                    const double* src = u + (int64_t)m * ORV_NVAR * n3;
                    if (level[m] <= L) {
                        int si = (int)(X[0] / sl - (long long)sc[0] * nxb) + ng;
                        int sj = (int)(X[1] / sl - (long long)sc[1] * nxb) + ng;
                        int sk = (int)(X[2] / sl - (long long)sc[2] * nxb) + ng;
                        for (int v = 0; v < nv; ++v) dst[v * n3] = src[v * n3 + cidx(n, si, sj, sk)];
                    } else {
                        int r = (int)(s / sl);
                        int bi = (int)(lo[0] / sl - (long long)sc[0] * nxb) + ng;
                        int bj = (int)(lo[1] / sl - (long long)sc[1] * nxb) + ng;
                        int bk = (int)(lo[2] / sl - (long long)sc[2] * nxb) + ng;
                        double inv = 1.0 / (double)(r * r * r);
                        for (int v = 0; v < nv; ++v) {
                            double acc = 0.0;
                            for (int z = 0; z < r; ++z)
                                for (int y = 0; y < r; ++y)
                                    for (int x = 0; x < r; ++x) acc += src[v * n3 + cidx(n, bi + x, bj + y, bk + z)];
                            dst[v * n3] = acc * inv;
                        }
                    }
                }
        if (!p->mhd) return;
        for (int a = 0; a < 3; ++a)
            for (int k = 0; k < n + (a == 2); ++k)
                for (int j = 0; j < n + (a == 1); ++j)
                    for (int i = 0; i < n + (a == 0); ++i) {
                        int I[3] = {i, j, k};
                        int own = 1;
                        for (int e = 0; e < 3; ++e) {
                            int top = ng + nxb - 1 + (e == a);
                            if (I[e] < ng || I[e] > top) own = 0;
                        }
                        if (own) continue;
                        long long lo[3], X[3];
                        for (int d = 0; d < 3; ++d) {
                            lo[d] = orc_wrap(((long long)cd[d] * nxb + I[d] - ng) * s, N[d]);
                            X[d] = lo[d] + (d == a ? 0 : s / 2);
                        }
                        int m = orc_leaf_at(level, child, root, nr0, nr1, maxlevel, X[0], X[1], X[2]);
                        if (level[m] != L) {
                            /* a face on a level boundary: the copy owned by the leaf of this
                             * block's level on the lower side, when there is one, so that
                             * every block of a level reads the same face */
                            long long Y[3] = {X[0], X[1], X[2]};
                            Y[a] = orc_wrap(X[a] - 1, N[a]);
                            int m2 = orc_leaf_at(level, child, root, nr0, nr1, maxlevel, Y[0], Y[1], Y[2]);
                            if (level[m2] == L) {
                                m = m2;
                                X[a] = Y[a] + 1; /* its upper face, unwrapped at the domain edge */
                            }
                        }
                        const long long sl = 1LL << (maxlevel - level[m]);
                        const int* sc = coord + 3 * m;
                        const double* src = fa[a] + (int64_t)m * fsz;
                        double* dst = fa[a] + (int64_t)b * fsz + fidx(n, a, i, j, k);
                        if (level[m] <= L) {
                            int S[3];
                            for (int d = 0; d < 3; ++d) S[d] = (int)(X[d] / sl - (long long)sc[d] * nxb) + ng;
                            if (X[a] % sl == 0) {
                                *dst = src[fidx(n, a, S[0], S[1], S[2])];
                            } else {
                                int S1[3] = {S[0], S[1], S[2]};
                                S1[a] += 1;
                                *dst = 0.5 * (src[fidx(n, a, S[0], S[1], S[2])] + src[fidx(n, a, S1[0], S1[1], S1[2])]);
                            }
                        } else {
                            int r = (int)(s / sl);
                            int B[3];
                            for (int d = 0; d < 3; ++d) B[d] = (int)(lo[d] / sl - (long long)sc[d] * nxb) + ng;
                            int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
                            double acc = 0.0;
                            for (int y = 0; y < r; ++y)
                                for (int x = 0; x < r; ++x) {
                                    int Q[3] = {B[0], B[1], B[2]};
                                    Q[t1] += x;
                                    Q[t2] += y;
                                    acc += src[fidx(n, a, Q[0], Q[1], Q[2])];
                                }
                            *dst = acc / (double)(r * r);
                        }
                    }
    }
}

void orc_fill_guards_tree(const orc_hydro_params* p, int nnodes, const int* level, const int* coord,
                          const int* child, const int* root, int nr0, int nr1, int nr2, int maxlevel,
                          double* u, double* bx, double* by, double* bz)
{
    for (int b = 0; b < nnodes; ++b)
        if (child[8 * b] < 0)
            orc_fill_guards_leaf(p, b, level, coord, child, root, nr0, nr1, nr2, maxlevel, u, bx, by, bz);
}

/* Face neighbours of leaf b (see hydro_oracle.h). Positions are finest-cell
 * coordinates; the probe point lies one finest cell across the face, at the
 * face centre (same or coarser neighbour) or at the quadrant centres. */
void orc_face_links(int b, const int* level, const int* coord, const int* child, const int* root, int nr0,
                    int nr1, int nr2, int maxlevel, int* type, int* fine)
{
    const long long nxb = 16;
    const long long N[3] = {(long long)nr0 * nxb << maxlevel, (long long)nr1 * nxb << maxlevel,
                            (long long)nr2 * nxb << maxlevel};
    const int L = level[b];
    const long long E = nxb << (maxlevel - L); /* block extent in finest cells */
    for (int f = 0; f < 6; ++f) {
        const int d = f >> 1, side = f & 1;
        int t1, t2;
        face_axes(d, &t1, &t2);
        long long X[3];
        X[d] = orc_wrap(side ? (coord[3 * b + d] + 1) * E : coord[3 * b + d] * E - 1, N[d]);
        X[t1] = coord[3 * b + t1] * E + E / 2;
        X[t2] = coord[3 * b + t2] * E + E / 2;
        int m = orc_leaf_at(level, child, root, nr0, nr1, maxlevel, X[0], X[1], X[2]);
        for (int q = 0; q < 4; ++q) fine[4 * f + q] = -1;
        if (level[m] < L) {
            type[f] = ORC_FACE_COARSER;
        } else if (level[m] == L) {
            type[f] = ORC_FACE_SAME;
        } else {
            type[f] = ORC_FACE_FINER;
            for (int q = 0; q < 4; ++q) {
                long long Y[3] = {X[0], X[1], X[2]};
                Y[t1] = coord[3 * b + t1] * E + E / 4 + (q & 1) * (E / 2);
                Y[t2] = coord[3 * b + t2] * E + E / 4 + (q >> 1) * (E / 2);
                fine[4 * f + q] = orc_leaf_at(level, child, root, nr0, nr1, maxlevel, Y[0], Y[1], Y[2]);
            }
        }
    }
}
