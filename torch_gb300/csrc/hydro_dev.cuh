// Unsplit PPM + HLLC hydro / PPM + HLLD + CT MHD step, device code.
//
// One step over a chunk of blocks runs five kernels:
//   k_recon   per cell (18^3 band of each block, one warp per direction):
//             normal-direction PPM with characteristic limiting and tracing,
//             transverse corrections and multidimensional MHD terms in the
//             order of hy_uhd_dataReconstOneStep.F90:1006-1089, positivity
//             fallback (:1230-1272) -> face states in scratch
//   k_flux    per face: HLLC / HLLD + artificial viscosity -> fluxes
//   k_emf     per edge (MHD): contact-upwinded CT electric field
//   k_faceb   per face (MHD): Faraday update of the face-centred field
//   k_update  per interior cell: FP64 flux-difference update, dual-energy
//             recovery, Gamma-law EOS, optional fused cooling epilogue
// The reconstruction and Riemann solve run in T (double for the plain path,
// float for the mixed path); every accumulation into conserved variables,
// the electric fields and the face-field update run in double.
#pragma once

#include <type_traits>

#include "cool_dev.cuh"
#include "gb_common.cuh"
#include "sur_dev.cuh"

namespace gbh {

constexpr int NP = 8;      // rho, vx, vy, vz, p, Bx, By, Bz
constexpr int MAXW = 7;
constexpr int RB = 18;     // reconstruction band: cells 3..20
constexpr int RLO = GB_NGUARD - 1;
constexpr int NRC = RB * RB * RB;
// time-n edge fields for the half-step normal field of the Riemann
// problems: per direction c a box of 19^3 positions (3..21 on every axis;
// along c the index is a cell, across it an edge at index - 1/2), x fastest
// whatever c, so that faces next to each other along x read edges next to
// each other
constexpr int EB = RB + 1;
constexpr int NEN = EB * EB * EB;
constexpr int LO = GB_NGUARD, HI = GB_NGUARD + GB_NXB - 1;
constexpr int NFC = 17 * RB * RB;             // faces per direction in the flux box
constexpr int NFLX = 10;                      // 8 fluxes + rho*e_int flux + face velocity
constexpr int NEDGE = 16 * 17 * 17;           // edges per direction
constexpr int NFB = 17 * 16 * 16;             // interior faces per direction

constexpr int NP32 = 9;  // FP32 copy of the primitives: rho, vx, vy, vz, p, Bx, By, Bz, e_int

// scratch sizes per block (elements)
template <typename T>
struct scratch_layout {
    static constexpr size_t recon = (size_t)NRC * 6 * NP;     // T
    static constexpr size_t flux = (size_t)3 * NFC * NFLX;    // T
    static constexpr size_t emf = (size_t)3 * NEDGE;          // double
    static constexpr size_t fb = (size_t)3 * NFB;             // double
    // FP32 primitives of the padded block (mixed path only)
    // (+ the three face-B arrays, FP32, after the cell variables)
    static constexpr size_t prim32 = std::is_same<T, float>::value ? (size_t)NP32 * GB_N3 + 3 * GB_FSZ : 0;  // float
    // hybrid order: the minimum undivided velocity divergence over each
    // band cell's box (T)
    static constexpr size_t divu = (size_t)NRC;
    // the edge fields' cell-centred reference, -(v x B)_d of the mean face
    // state along d, per direction and band cell (T)
    static constexpr size_t ecc = (size_t)3 * NRC;
    // MHD: the time-n edge fields of the normal-field half step (T)
    static constexpr size_t edgen = (size_t)3 * NEN;
    static constexpr size_t bytes = recon * sizeof(T) + flux * sizeof(T) + (emf + fb) * sizeof(double) +
                                    prim32 * sizeof(float) + divu * sizeof(T) + ecc * sizeof(T) +
                                    edgen * sizeof(T);
};
// the FP32 copy of each block starts on a 16-byte boundary (k_prim32 stores
// four cells at a time): every section before it and its own stride are
// multiples of 16 bytes
static_assert((scratch_layout<float>::recon * 4 + scratch_layout<float>::flux * 4 +
               (scratch_layout<float>::emf + scratch_layout<float>::fb) * 8) % 16 == 0 &&
                  (scratch_layout<float>::prim32 * 4) % 16 == 0,
              "FP32 copy 16-byte aligned");

// FP32 copy of the primitive variables of the padded blocks: the mixed
// path converts each double once here instead of at every stencil read
// (conversions issue on the FP64 pipe)
template <bool MHD>
__global__ void __launch_bounds__(128)
k_prim32(gb_dev_grid g, const int* __restrict__ list, float* __restrict__ p32, size_t stride)
{
    // threads [0, GB_STEP_CELLS / 4): groups of four x-neighbouring cells of
    // the step's read region (rows are whole and a multiple of four long, so
    // a group is two 16-byte loads and one 16-byte store per variable); then
    // (MHD) its faces, axis by axis
    const int cb = blockIdx.y;
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < GB_STEP_CELLS / 4) {
        int i, j, k;
        gb_step_cell(4 * q, i, j, k);
        const int c = gb_cidx(i, j, k);
        const double* base = g.unk + (int64_t)list[cb] * g.nvar * GB_N3 + c;
        float* out = p32 + (size_t)cb * stride + c;
        const int roles[NP32] = {GB_DENS, GB_VELX, GB_VELY, GB_VELZ, GB_PRES, GB_MAGX, GB_MAGY, GB_MAGZ, GB_EINT};
#pragma unroll
        for (int v = 0; v < NP32; ++v) {
            if (!MHD && v >= 5 && v < 8) {
                *reinterpret_cast<float4*>(out + (size_t)v * GB_N3) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                continue;
            }
            const double* src = base + (int64_t)g.slot[roles[v]] * GB_N3;
            const double2 x0 = *reinterpret_cast<const double2*>(src);
            const double2 x1 = *reinterpret_cast<const double2*>(src + 2);
            *reinterpret_cast<float4*>(out + (size_t)v * GB_N3) =
                make_float4(gb_d2f(x0.x), gb_d2f(x0.y), gb_d2f(x1.x), gb_d2f(x1.y));
        }
        return;
    }
    q -= GB_STEP_CELLS / 4;
    if (!MHD || q >= GB_STEP_FACES_ALL) return;
    const int a = q < gb_step_faces(0) ? 0 : (q < gb_step_faces(0) + gb_step_faces(1) ? 1 : 2);
    const int e = q - (a == 0 ? 0 : (a == 1 ? gb_step_faces(0) : gb_step_faces(0) + gb_step_faces(1)));
    const int nx = GB_N + (a == 0), ny = GB_BAND + (a == 1);
    const int fi = gb_fidx(a, e % nx, GB_BAND_LO + (e / nx) % ny, GB_BAND_LO + e / (nx * ny));
    const double* fa = a == 0 ? g.f[0] : (a == 1 ? g.f[1] : g.f[2]);
    p32[(size_t)cb * stride + (size_t)NP32 * GB_N3 + (size_t)a * GB_FSZ + fi] =
        gb_d2f(fa[(int64_t)list[cb] * GB_FSZ + fi]);
}

// face B of the padded block for reconstruction precision T: the FP32
// copies of the mixed path, the FP64 store otherwise
template <typename T>
__device__ __forceinline__ T face_b(const gb_dev_grid& g, int a, int blk, int fi, const float* p32b)
{
    if constexpr (std::is_same<T, float>::value) return p32b[(size_t)NP32 * GB_N3 + (size_t)a * GB_FSZ + fi];
    else return (a == 0 ? g.f[0] : (a == 1 ? g.f[1] : g.f[2]))[(int64_t)blk * GB_FSZ + fi];  // no run-time index into the parameters
}

template <typename T>
__device__ __forceinline__ T two3() { return (T)(2.0 / 3.0); }
template <>
__device__ __forceinline__ float two3<float>() { return 2.0f / 3.0f; }

// x / 6: the oracle's division in FP64; in FP32 (whose divisions are
// approximate in the mixed path anyway) a product with the rounded 1/6
template <typename T>
__device__ __forceinline__ T over6(T x) { return x / (T)6; }
template <>
__device__ __forceinline__ float over6<float>(float x) { return x * (1.0f / 6.0f); }

template <typename T>
__device__ __forceinline__ T minmod(T a, T b)
{
    if (a * b <= (T)0) return (T)0;
    return (fabs(a) <= fabs(b)) ? a : b;
}

// rotated slot -> unrotated primitive slot
__device__ __forceinline__ int rot_slot(int d, int s)
{
    // d = 0: identity; 1: (0,2,3,1,4,6,7,5); 2: (0,3,1,2,4,7,5,6)
    if (d == 0 || s == 0 || s == 4) return s;
    int base = s < 4 ? 1 : 5, o = s - base;
    return base + (o + d) % 3;
}
__device__ __forceinline__ int wslot(int s) { return s < 5 ? s : s + 1; }

// ---------------------------------------------------------------- eigensystems
// Structural non-zeros of the eigenvector matrices that eig_hydro / eig_mhd
// fill (every other entry is 0). The projections below skip the zero
// entries at compile time: without fast-math the compiler cannot drop 0 * x,
// and for finite x a skipped term is +-0, which leaves every sum unchanged.
template <bool MHD>
__host__ __device__ constexpr bool nz_L(int k, int s)
{
    return MHD ? (k == 3 ? (s == 0 || s == 4)
                         : (k == 1 || k == 5) ? (s == 2 || s == 3 || s == 5 || s == 6) : (s >= 1 && s <= 6))
               : ((k == 0 || k == 4) ? (s == 1 || s == 4) : k == 1 ? (s == 0 || s == 4) : s == k);
}
template <bool MHD>
__host__ __device__ constexpr bool nz_R(int s, int k)
{
    return MHD ? (k == 3 ? s == 0 : (k == 1 || k == 5) ? (s == 2 || s == 3 || s == 5 || s == 6) : true)
               : ((k == 0 || k == 4) ? (s == 0 || s == 1 || s == 4) : k == 1 ? s == 0 : s == k);
}
template <typename T>
__device__ __forceinline__ void eig_hydro(T gam, const T* q, T* lam, T (*R)[MAXW], T (*L)[MAXW])
{
    T rho = q[0], vn = q[1], p = q[4];
    T a2 = gam * p / rho;
    T a = sqrt(a2);
#pragma unroll
    for (int r = 0; r < MAXW; ++r)
#pragma unroll
        for (int c = 0; c < MAXW; ++c) { R[r][c] = (T)0; L[r][c] = (T)0; }
    lam[0] = vn - a; lam[1] = vn; lam[2] = vn; lam[3] = vn; lam[4] = vn + a;
    R[0][0] = (T)1; R[1][0] = -a / rho; R[4][0] = a2;
    R[0][1] = (T)1;
    R[2][2] = (T)1;
    R[3][3] = (T)1;
    R[0][4] = (T)1; R[1][4] = a / rho; R[4][4] = a2;
    L[0][1] = -rho / ((T)2 * a); L[0][4] = (T)1 / ((T)2 * a2);
    L[1][0] = (T)1; L[1][4] = (T)-1 / a2;
    L[2][2] = (T)1;
    L[3][3] = (T)1;
    L[4][1] = rho / ((T)2 * a); L[4][4] = (T)1 / ((T)2 * a2);
}

template <typename T>
__device__ __forceinline__ void eig_mhd(T gam, const T* q, T* lam, T (*R)[MAXW], T (*L)[MAXW])
{
    T rho = q[0], vn = q[1], p = q[4], bn = q[5], bt1 = q[6], bt2 = q[7];
    T a2 = gam * p / rho;
    T sr = sqrt(rho);
    T bnx2 = bn * bn / rho;
    T bt2s = (bt1 * bt1 + bt2 * bt2) / rho;
    T term = a2 + bnx2 + bt2s;
    T d1 = a2 - bnx2;
    T disc = sqrt(d1 * d1 + bt2s * ((T)2 * (a2 + bnx2) + bt2s));
    T cf2 = (T)0.5 * (term + disc);
    T cs2 = a2 * bnx2 / cf2;
    T cf = sqrt(cf2), cs = sqrt(cs2), ca = sqrt(bnx2);
    T bperp = sqrt(bt1 * bt1 + bt2 * bt2);
    T by, bz;
    if (bperp > (T)0) { by = bt1 / bperp; bz = bt2 / bperp; }
    else { by = (T)0.70710678118654752440; bz = (T)0.70710678118654752440; }
    T af, as;
    if (disc > (T)0) {
        T af2 = ((d1 - bt2s) + disc) / ((T)2 * disc);
        T as2 = ((bt2s - d1) + disc) / ((T)2 * disc);
        af2 = af2 < (T)0 ? (T)0 : (af2 > (T)1 ? (T)1 : af2);
        as2 = as2 < (T)0 ? (T)0 : (as2 > (T)1 ? (T)1 : as2);
        af = sqrt(af2);
        as = sqrt(as2);
    } else {
        af = (T)1;
        as = (T)0;
    }
    T S = bn >= (T)0 ? (T)1 : (T)-1;
    T a = sqrt(a2);
    T n2 = af * af * cf2 + as * as * cs2;
    T sra = sr * a;
#pragma unroll
    for (int r = 0; r < MAXW; ++r)
#pragma unroll
        for (int c = 0; c < MAXW; ++c) { R[r][c] = (T)0; L[r][c] = (T)0; }
    lam[0] = vn - cf; lam[1] = vn - ca; lam[2] = vn - cs; lam[3] = vn;
    lam[4] = vn + cs; lam[5] = vn + ca; lam[6] = vn + cf;
    R[0][0] = rho * af; R[1][0] = -af * cf; R[2][0] = as * cs * by * S; R[3][0] = as * cs * bz * S;
    R[4][0] = rho * af * a2; R[5][0] = as * sra * by; R[6][0] = as * sra * bz;
    R[2][1] = -bz; R[3][1] = by; R[5][1] = -S * sr * bz; R[6][1] = S * sr * by;
    R[0][2] = rho * as; R[1][2] = -as * cs; R[2][2] = -af * cf * by * S; R[3][2] = -af * cf * bz * S;
    R[4][2] = rho * as * a2; R[5][2] = -af * sra * by; R[6][2] = -af * sra * bz;
    R[0][3] = (T)1;
    R[0][4] = rho * as; R[1][4] = as * cs; R[2][4] = af * cf * by * S; R[3][4] = af * cf * bz * S;
    R[4][4] = rho * as * a2; R[5][4] = -af * sra * by; R[6][4] = -af * sra * bz;
    R[2][5] = -bz; R[3][5] = by; R[5][5] = S * sr * bz; R[6][5] = -S * sr * by;
    R[0][6] = rho * af; R[1][6] = af * cf; R[2][6] = -as * cs * by * S; R[3][6] = -as * cs * bz * S;
    R[4][6] = rho * af * a2; R[5][6] = as * sra * by; R[6][6] = as * sra * bz;
    T hn = (T)0.5 / n2, hra = (T)0.5 / (rho * a2), hsa = (T)0.5 / sra, hs = (T)0.5 / sr;
    L[0][1] = -af * cf * hn; L[0][2] = as * cs * S * by * hn; L[0][3] = as * cs * S * bz * hn;
    L[0][4] = af * hra; L[0][5] = as * by * hsa; L[0][6] = as * bz * hsa;
    L[1][2] = (T)-0.5 * bz; L[1][3] = (T)0.5 * by; L[1][5] = -bz * S * hs; L[1][6] = by * S * hs;
    L[2][1] = -as * cs * hn; L[2][2] = -af * cf * S * by * hn; L[2][3] = -af * cf * S * bz * hn;
    L[2][4] = as * hra; L[2][5] = -af * by * hsa; L[2][6] = -af * bz * hsa;
    L[3][0] = (T)1; L[3][4] = (T)-1 / a2;
    L[4][1] = as * cs * hn; L[4][2] = af * cf * S * by * hn; L[4][3] = af * cf * S * bz * hn;
    L[4][4] = as * hra; L[4][5] = -af * by * hsa; L[4][6] = -af * bz * hsa;
    L[5][2] = (T)-0.5 * bz; L[5][3] = (T)0.5 * by; L[5][5] = bz * S * hs; L[5][6] = -by * S * hs;
    L[6][1] = af * cf * hn; L[6][2] = -as * cs * S * by * hn; L[6][3] = -as * cs * S * bz * hn;
    L[6][4] = af * hra; L[6][5] = as * by * hsa; L[6][6] = as * bz * hsa;
}

// ---------------------------------------------------------------- PPM
// qs[m][s]: rotated stencil (m = 0..4), outputs rotated wp, wn, sig.
template <typename T, bool MHD>
__device__ __forceinline__ void ppm_normal(T gam, const T (*qs)[NP], T dtdx, T* wp, T* wn, T* sig)
{
    constexpr int nw = MHD ? 7 : 5;
    T lam[MAXW], R[MAXW][MAXW], L[MAXW][MAXW];
    if (MHD) eig_mhd<T>(gam, qs[2], lam, R, L);
    else eig_hydro<T>(gam, qs[2], lam, R, L);
    // characteristic differences L (q[m+1] - q[m]) of the four stencil
    // intervals, each formed once: cell m's limited slope takes intervals
    // m - 1 and m (the same sums, in the same order, as forming both per cell)
    T ld[4][MAXW];
    T dwm[3][MAXW];
    if constexpr (std::is_same<T, float>::value) {
        // FP32: the projections that share a matrix row run as packed pairs
        // (fma.rn.f32x2: two lanes per instruction, each lane the same
        // rounding as the scalar fused multiply-add): intervals (0, 1) and
        // (2, 3) of L . dq, and cells 1 and 2 of R . da
        float2 d01[MAXW], d23[MAXW];
#pragma unroll
        for (int s = 0; s < nw; ++s) {
            const int qq = wslot(s);
            d01[s] = make_float2(qs[1][qq] - qs[0][qq], qs[2][qq] - qs[1][qq]);
            d23[s] = make_float2(qs[3][qq] - qs[2][qq], qs[4][qq] - qs[3][qq]);
        }
#pragma unroll
        for (int k = 0; k < nw; ++k) {
            float2 a01 = make_float2(0.0f, 0.0f), a23 = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int s = 0; s < nw; ++s) {
                if (!nz_L<MHD>(k, s)) continue;
                const float2 l2 = make_float2(L[k][s], L[k][s]);
                a01 = __ffma2_rn(l2, d01[s], a01);
                a23 = __ffma2_rn(l2, d23[s], a23);
            }
            ld[0][k] = a01.x;
            ld[1][k] = a01.y;
            ld[2][k] = a23.x;
            ld[3][k] = a23.y;
        }
        float2 da12[MAXW];
        float da3[MAXW];
#pragma unroll
        for (int k = 0; k < nw; ++k) {
            da12[k] = make_float2(minmod<float>(ld[0][k], ld[1][k]), minmod<float>(ld[1][k], ld[2][k]));
            da3[k] = minmod<float>(ld[2][k], ld[3][k]);
        }
#pragma unroll
        for (int s = 0; s < nw; ++s) {
            float2 a12 = make_float2(0.0f, 0.0f);
            float a3 = 0.0f;
#pragma unroll
            for (int k = 0; k < nw; ++k)
                if (nz_R<MHD>(s, k)) {
                    a12 = __ffma2_rn(make_float2(R[s][k], R[s][k]), da12[k], a12);
                    a3 = __fmaf_rn(R[s][k], da3[k], a3);
                }
            dwm[0][s] = a12.x;
            dwm[1][s] = a12.y;
            dwm[2][s] = a3;
        }
    } else {
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int k = 0; k < nw; ++k) {
                T acc = (T)0;
#pragma unroll
                for (int s = 0; s < nw; ++s) {
                    const int qq = wslot(s);
                    if (!nz_L<MHD>(k, s)) continue;
                    acc = acc + L[k][s] * (qs[m + 1][qq] - qs[m][qq]);
                }
                ld[m][k] = acc;
            }
#pragma unroll
        for (int m = 1; m <= 3; ++m) {
            T da[MAXW];
#pragma unroll
            for (int k = 0; k < nw; ++k) da[k] = minmod<T>(ld[m - 1][k], ld[m][k]);
#pragma unroll
            for (int s = 0; s < nw; ++s) {
                T acc = (T)0;
#pragma unroll
                for (int k = 0; k < nw; ++k)
                    if (nz_R<MHD>(s, k)) acc = acc + R[s][k] * da[k];
                dwm[m - 1][s] = acc;
            }
        }
    }
    T WL[MAXW], WR[MAXW], dW[MAXW], W6[MAXW];
#pragma unroll
    for (int s = 0; s < nw; ++s) {
        const int qq = wslot(s);
        T qm = qs[1][qq], q0 = qs[2][qq], qp = qs[3][qq];
        T wl = (T)0.5 * (qm + q0) - over6<T>(dwm[1][s] - dwm[0][s]);
        T wr = (T)0.5 * (q0 + qp) - over6<T>(dwm[2][s] - dwm[1][s]);
        wl = fmax(fmin(q0, qm), wl);
        wl = fmin(fmax(q0, qm), wl);
        wr = fmax(fmin(q0, qp), wr);
        wr = fmin(fmax(q0, qp), wr);
        T qa = (wr - q0) * (q0 - wl);
        if (qa <= (T)0) {
            wl = q0;
            wr = q0;
        } else {
            T qb = wr - wl;
            T qc = (T)6 * (q0 - (T)0.5 * (wl + wr));
            if (qb * qc > qb * qb) wl = (T)3 * q0 - (T)2 * wr;
            else if (qb * qc < -(qb * qb)) wr = (T)3 * q0 - (T)2 * wl;
        }
        WL[s] = wl;
        WR[s] = wr;
        dW[s] = wr - wl;
        W6[s] = (T)6 * (q0 - (T)0.5 * (wl + wr));
    }
    T ldW[MAXW], lW6[MAXW];
    if constexpr (std::is_same<T, float>::value) {
        // L . dW and L . W6 as one packed pair per matrix entry
        float2 w2[MAXW];
#pragma unroll
        for (int s = 0; s < nw; ++s) w2[s] = make_float2(dW[s], W6[s]);
#pragma unroll
        for (int k = 0; k < nw; ++k) {
            float2 ab = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int s = 0; s < nw; ++s) {
                if (!nz_L<MHD>(k, s)) continue;
                ab = __ffma2_rn(make_float2(L[k][s], L[k][s]), w2[s], ab);
            }
            ldW[k] = ab.x;
            lW6[k] = ab.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < nw; ++k) {
            T a = (T)0, b = (T)0;
#pragma unroll
            for (int s = 0; s < nw; ++s) {
                if (!nz_L<MHD>(k, s)) continue;
                a = a + L[k][s] * dW[s];
                b = b + L[k][s] * W6[s];
            }
            ldW[k] = a;
            lW6[k] = b;
        }
    }
    const T t3 = two3<T>();
    T sK = lam[nw - 1] * dtdx;
    bool refK = lam[nw - 1] > (T)0;
    T Wp[MAXW], Wn[MAXW];
#pragma unroll
    for (int s = 0; s < nw; ++s)
        Wp[s] = refK ? WR[s] - (T)0.5 * sK * (dW[s] - ((T)1 - t3 * sK) * W6[s]) : WR[s];
    T s0 = lam[0] * dtdx;
    bool ref0 = lam[0] < (T)0;
#pragma unroll
    for (int s = 0; s < nw; ++s)
        Wn[s] = ref0 ? WL[s] - (T)0.5 * s0 * (dW[s] + ((T)1 + t3 * s0) * W6[s]) : WL[s];
    if constexpr (std::is_same<T, float>::value) {
        // each wave corrects the + state (lam > 0) or the - state (lam < 0):
        // one packed pair per matrix entry with the other side's coefficient
        // 0 (adding 0 R leaves a state unchanged), and no branch on the wave
        // speeds' signs, which differ between the cells of a warp
        float2 wpn[MAXW];
#pragma unroll
        for (int s = 0; s < nw; ++s) wpn[s] = make_float2(Wp[s], Wn[s]);
#pragma unroll
        for (int k = 0; k < nw; ++k) {
            const T sg = lam[k] * dtdx;
            const T gK = refK ? (T)0.5 * sK * (ldW[k] - ((T)1 - t3 * sK) * lW6[k]) : (T)0;
            const T cp = gK - (T)0.5 * sg * (ldW[k] - ((T)1 - t3 * sg) * lW6[k]);
            const T g0 = ref0 ? (T)0.5 * s0 * (ldW[k] + ((T)1 + t3 * s0) * lW6[k]) : (T)0;
            const T cn = g0 - (T)0.5 * sg * (ldW[k] + ((T)1 + t3 * sg) * lW6[k]);
            const float2 c2 = make_float2(lam[k] > (T)0 ? cp : (T)0, lam[k] < (T)0 ? cn : (T)0);
#pragma unroll
            for (int s = 0; s < nw; ++s)
                if (nz_R<MHD>(s, k)) wpn[s] = __ffma2_rn(c2, make_float2(R[s][k], R[s][k]), wpn[s]);
        }
#pragma unroll
        for (int s = 0; s < nw; ++s) {
            Wp[s] = wpn[s].x;
            Wn[s] = wpn[s].y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < nw; ++k) {
            if (lam[k] > (T)0) {
                T sg = lam[k] * dtdx;
                T gK = refK ? (T)0.5 * sK * (ldW[k] - ((T)1 - t3 * sK) * lW6[k]) : (T)0;
                T c = gK - (T)0.5 * sg * (ldW[k] - ((T)1 - t3 * sg) * lW6[k]);
#pragma unroll
                for (int s = 0; s < nw; ++s)
                    if (nz_R<MHD>(s, k)) Wp[s] = Wp[s] + c * R[s][k];
            }
        }
#pragma unroll
        for (int k = 0; k < nw; ++k) {
            if (lam[k] < (T)0) {
                T sg = lam[k] * dtdx;
                T g0 = ref0 ? (T)0.5 * s0 * (ldW[k] + ((T)1 + t3 * s0) * lW6[k]) : (T)0;
                T c = g0 - (T)0.5 * sg * (ldW[k] + ((T)1 + t3 * sg) * lW6[k]);
#pragma unroll
                for (int s = 0; s < nw; ++s)
                    if (nz_R<MHD>(s, k)) Wn[s] = Wn[s] + c * R[s][k];
            }
        }
    }
#pragma unroll
    for (int s = 0; s < NP; ++s) { wp[s] = (T)0; wn[s] = (T)0; sig[s] = (T)0; }
    if constexpr (std::is_same<T, float>::value) {
        // rows s and s + 1 of R (lam ldW) as packed pairs (a row's structural
        // zero adds 0 to its lane, as skipping it would)
        float lw[MAXW];
#pragma unroll
        for (int k = 0; k < nw; ++k) lw[k] = lam[k] * ldW[k];
#pragma unroll
        for (int s = 0; s < nw; s += 2) {
            if (s + 1 < nw) {
                float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
                for (int k = 0; k < nw; ++k)
                    if (nz_R<MHD>(s, k) || nz_R<MHD>(s + 1, k))
                        acc = __ffma2_rn(make_float2(lw[k], lw[k]), make_float2(R[s][k], R[s + 1][k]), acc);
                sig[wslot(s)] = acc.x;
                sig[wslot(s + 1)] = acc.y;
            } else {
                float acc = 0.0f;
#pragma unroll
                for (int k = 0; k < nw; ++k)
                    if (nz_R<MHD>(s, k)) acc = __fmaf_rn(lw[k], R[s][k], acc);
                sig[wslot(s)] = acc;
            }
        }
#pragma unroll
        for (int s = 0; s < nw; ++s) {
            wp[wslot(s)] = Wp[s];
            wn[wslot(s)] = Wn[s];
        }
    } else {
#pragma unroll
        for (int s = 0; s < nw; ++s) {
            T acc = (T)0;
#pragma unroll
            for (int k = 0; k < nw; ++k)
                if (nz_R<MHD>(s, k)) acc = acc + (lam[k] * ldW[k]) * R[s][k];
            wp[wslot(s)] = Wp[s];
            wn[wslot(s)] = Wn[s];
            sig[wslot(s)] = acc;
        }
    }
    wp[5] = qs[2][5];
    wn[5] = qs[2][5];
}

// CFL limit scale of a cell's code (bit 0: the fallback factor / 3, bit 1:
// 0.25; a ratio to cfl, at most 1)
struct cfl_scale {
    double s[4];
};

struct hydro_kparams {
    double gamma, cvisc, eint_switch, smlrho, smallp;
    int use_avisc;
    double dt, dx[3];
    // when set, the step's dt is read from device memory (written by the
    // CFL reduction earlier in the same stream or graph) instead of dt
    const double* dtp;
    // dt / root_dx per direction (dtdxp: its device copy, used with dtp).
    // A level-l block has dx = root_dx 2^-l, so its dt/dx is this times 2^l,
    // exactly, with no division in the kernels.
    double dtdx0[3];
    const double* dtdxp;
    // flux conservation at fine-coarse faces (null: off): face links of
    // every store block (6 faces x {type, 4 fine leaves}) and the boundary
    // flux registers (store block x 6 faces x 256 face cells x NREG, in T)
    const int* fc_links;
    void* fc_reg;
    // FP32 copies for the mixed path: gamma, cvisc, dt / root_dx (and its
    // device copy, written with dtdxp)
    float gammaf, cviscf;
    double inv_gm1;  // 1 / (gamma - 1), for the mixed path's update
    float dtdxf0[3];
    const float* dtdxfp;
    // edge electric fields at fine-coarse boundaries (MHD with flux
    // conservation; null: off): the guard-fill plan, the tree's child
    // table and the surface-edge registers (NSURF doubles per tree node)
    // cubic cells (dx = dy = dz at every level): the mixed update sums the
    // three directions' flux differences before one FP64 scaling
    int iso = 0;
    int energy_fix = 0;  // energyFix: gas energy from the flux-updated cell field
    // hybrid order (use_hybridOrder): first-order states where the flow
    // compresses and a state fails the Rankine-Hugoniot check; the minimum
    // divergence per band cell comes from k_divu. lower_cfl: the first
    // check's fallback lowers the cell's CFL (hy_fallbackLowerCFL)
    int hybrid = 0, lower_cfl = 0;
    double kappa = 0.0;
    const void* divu = nullptr;
    // the edge fields' reference per direction and band cell (T, 3 x NRC
    // per chunk block), written by the reconstruction
    void* ecc = nullptr;
    // the time-n edge fields (T, 3 x NEN per chunk block), written by
    // k_edge_n, read by the Riemann solves for the half-step normal field
    const void* edgen = nullptr;
    // per-cell CFL codes of the interior cells (store block x 3 directions
    // x 4096 bytes; null: not kept), read by the next CFL limit
    unsigned char* cflc = nullptr;
    int cfl_sum = 0;
    cfl_scale cflsc = {{1.0, 1.0, 1.0, 1.0}};
    const int4* ec_plan = nullptr;
    const int* ec_near = nullptr;  // per node: bit 0 a coarser leaf around it, bit 1 a finer one
    const int* ec_child = nullptr;
    double* ec_reg = nullptr;
};

__device__ __forceinline__ double kp_dt(const hydro_kparams& kp) { return kp.dtp ? *kp.dtp : kp.dt; }

// dt/dx of a level-l block in FP32 (the exact power-of-two scaling of
// dt/root_dx, 2^l from the exponent bits)
__device__ __forceinline__ void kp_dtdxf(const hydro_kparams& kp, int level, float* out)
{
    const float sc = __int_as_float((127 + level) << 23);
    if (kp.dtdxfp) {
        out[0] = kp.dtdxfp[0] * sc;
        out[1] = kp.dtdxfp[1] * sc;
        out[2] = kp.dtdxfp[2] * sc;
    } else {
        out[0] = kp.dtdxf0[0] * sc;
        out[1] = kp.dtdxf0[1] * sc;
        out[2] = kp.dtdxf0[2] * sc;
    }
}

__device__ __forceinline__ void kp_dtdx(const hydro_kparams& kp, int level, double* out)
{
    const double* d = kp.dtdxp ? kp.dtdxp : kp.dtdx0;
    out[0] = gb_scale_pow2(d[0], level);
    out[1] = gb_scale_pow2(d[1], level);
    out[2] = gb_scale_pow2(d[2], level);
}

// primitive 8-vector of a cell of the padded block
template <typename T, bool MHD>
__device__ __forceinline__ void load_w(const gb_dev_grid& g, int blk, int ci, T* w)
{
    const double* base = g.unk + (int64_t)blk * g.nvar * GB_N3 + ci;
    w[0] = (T)base[(int64_t)g.slot[GB_DENS] * GB_N3];
    w[1] = (T)base[(int64_t)g.slot[GB_VELX] * GB_N3];
    w[2] = (T)base[(int64_t)g.slot[GB_VELY] * GB_N3];
    w[3] = (T)base[(int64_t)g.slot[GB_VELZ] * GB_N3];
    w[4] = (T)base[(int64_t)g.slot[GB_PRES] * GB_N3];
    if (MHD) {
        w[5] = (T)base[(int64_t)g.slot[GB_MAGX] * GB_N3];
        w[6] = (T)base[(int64_t)g.slot[GB_MAGY] * GB_N3];
        w[7] = (T)base[(int64_t)g.slot[GB_MAGZ] * GB_N3];
    } else {
        w[5] = (T)0; w[6] = (T)0; w[7] = (T)0;
    }
}

// primitives of a cell: FP32 copy on the mixed path, the FP64 store on the plain one
template <typename T, bool MHD>
__device__ __forceinline__ void load_prim(const gb_dev_grid& g, int blk, int ci, const float* p32, T* w)
{
    if constexpr (std::is_same<T, float>::value) {
#pragma unroll
        for (int v = 0; v < NP; ++v) w[v] = p32[(size_t)v * GB_N3 + ci];
    } else {
        load_w<T, MHD>(g, blk, ci, w);
    }
}

// ---------------------------------------------------------------- k_divu
// Hybrid order's compression measure (hy_uhd_dataReconstOneStep.F90:934-948,
// 1150-1164): the undivided velocity divergence (Balsara & Spicer 1999)
// sum_d (v_d(c + e_d) - v_d(c - e_d)) / 2 of every band cell, then per band
// cell its minimum over the +-k4 box (k4 = 1 MHD, 2 hydro) clipped to the
// band, whose cells all have filled neighbours. One CTA per block; the
// divergences stay in shared memory.
constexpr int DIVU_THREADS = 256;
template <typename T, bool MHD>
__global__ void __launch_bounds__(DIVU_THREADS)
k_divu(gb_dev_grid g, const int* __restrict__ list, const float* __restrict__ p32, size_t p32_stride,
       T* __restrict__ out, size_t out_stride)
{
    __shared__ T s_div[NRC];
    const int cb = blockIdx.y;
    const int blk = list[cb];
    const float* p32b = p32 + (size_t)cb * p32_stride;
    auto vel = [&](int d, int ci) -> T {
        if constexpr (std::is_same<T, float>::value) return p32b[(size_t)(1 + d) * GB_N3 + ci];
        else return g.unk[((int64_t)blk * g.nvar + g.slot[GB_VELX + d]) * GB_N3 + ci];
    };
    for (int c = threadIdx.x; c < NRC; c += DIVU_THREADS) {
        const int i = RLO + c % RB, j = RLO + (c / RB) % RB, k = RLO + c / (RB * RB);
        const int ci = gb_cidx(i, j, k);
        s_div[c] = (T)0.5 * (vel(0, ci + 1) - vel(0, ci - 1)) + (T)0.5 * (vel(1, ci + GB_N) - vel(1, ci - GB_N)) +
                   (T)0.5 * (vel(2, ci + GB_N * GB_N) - vel(2, ci - GB_N * GB_N));
    }
    __syncthreads();
    constexpr int K4 = MHD ? 1 : 2;
    T* o = out + (size_t)cb * out_stride;
    for (int c = threadIdx.x; c < NRC; c += DIVU_THREADS) {
        const int i = c % RB, j = (c / RB) % RB, k = c / (RB * RB);
        T m = (T)1e30;
        for (int kk = k - K4; kk <= k + K4; ++kk) {
            if (kk < 0 || kk >= RB) continue;
            for (int jj = j - K4; jj <= j + K4; ++jj) {
                if (jj < 0 || jj >= RB) continue;
                for (int ii = i - K4; ii <= i + K4; ++ii) {
                    if (ii < 0 || ii >= RB) continue;
                    const T x = s_div[ii + RB * (jj + RB * kk)];
                    if (x < m) m = x;
                }
            }
        }
        o[c] = m;
    }
}

// hy_uhd_checkRHjumpCond for one face state, written from the
// Rankine-Hugoniot relations: no single shock compresses an ideal gas by
// more than (gamma + 1) / (gamma - 1) (the strong-shock limit, Toro 1997
// eq. 3.58), so a face state whose density differs from its cell's by more
// is not shock-connected to it
//
// The check's arithmetic uses explicitly rounded operations: they share no
// subexpression with the reconstruction and are never contracted, so the
// check leaves the compiler's fusing of the reconstruction's own
// arithmetic (and with it the mixed path's results) the same in every
// launch-shape instantiation.
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float rn_sqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double rn_sqrt(double a) { return __dsqrt_rn(a); }

template <typename T>
__device__ __forceinline__ bool rh_fail(T gam, T rho_c, T rho_f)
{
    const T lim = rn_div(rn_add(gam, (T)1), rn_sub(gam, (T)1));
    return rho_f > rn_mul(lim, rho_c) || rho_c > rn_mul(lim, rho_f);
}

// ---------------------------------------------------------------- k_recon
// blockDim = 3 * TILE: threads [d TILE, (d + 1) TILE) reconstruct direction d
// for TILE cells (TILE a multiple of 32, so every warp has one direction).
// All three directions run the same instructions: a thread works in its
// direction's rotated frame (normal velocity and field first), rotating by
// where it loads and stores rather than by moving registers, so register
// arrays keep constant indices and the kernel holds one copy of the PPM and
// eigensystem code (three copies, one per direction, overflowed the
// instruction cache). The block barrier between the normal and the
// transverse part sits in the kernel.

// unrotated slot of rotated slot s for direction d (see rot_slot), for a
// compile-time s and a run-time d: an index computation, not a register move
template <int S>
__device__ __forceinline__ int rot_slot_rt(int d)
{
    if (S == 0 || S == 4) return S;
    constexpr int base = S < 4 ? 1 : 5, o = S - base;
    const int r = o + d;
    return base + (r >= 3 ? r - 3 : r);
}

template <typename T>
__device__ __forceinline__ T pick3(int d, T a, T b, T c) { return d == 0 ? a : (d == 1 ? b : c); }

// offsets (elements from the cell's first variable) of the rotated
// primitives of direction d: FP32 copy (mixed) or FP64 store slots (plain)
template <typename T, bool MHD>
__device__ __forceinline__ void rot_offsets(const gb_dev_grid& g, int d, int* off)
{
    int u[NP];
    u[0] = 0; u[1] = rot_slot_rt<1>(d); u[2] = rot_slot_rt<2>(d); u[3] = rot_slot_rt<3>(d); u[4] = 4;
    u[5] = rot_slot_rt<5>(d); u[6] = rot_slot_rt<6>(d); u[7] = rot_slot_rt<7>(d);
    if constexpr (std::is_same<T, float>::value) {
#pragma unroll
        for (int s = 0; s < NP; ++s) off[s] = u[s] * GB_N3;
    } else {
        // store slots of the primitive roles, picked by selects (the role
        // of rotated slot s is one of three)
        const int sv[3] = {g.slot[GB_VELX], g.slot[GB_VELY], g.slot[GB_VELZ]};
        off[0] = g.slot[GB_DENS] * GB_N3;
        off[4] = g.slot[GB_PRES] * GB_N3;
#pragma unroll
        for (int s = 1; s < 4; ++s) off[s] = pick3(u[s] - 1, sv[0], sv[1], sv[2]) * GB_N3;
        if (MHD) {
            const int sb[3] = {g.slot[GB_MAGX], g.slot[GB_MAGY], g.slot[GB_MAGZ]};
#pragma unroll
            for (int s = 5; s < 8; ++s) off[s] = pick3(u[s] - 5, sb[0], sb[1], sb[2]) * GB_N3;
        } else {
            off[5] = off[6] = off[7] = -1;
        }
    }
}

// rotated primitives of one cell (ci: padded cell index)
template <typename T, bool MHD>
__device__ __forceinline__ void load_rot(const gb_dev_grid& g, int blk, int ci, const float* p32b, const int* off, T* w)
{
    if constexpr (std::is_same<T, float>::value) {
#pragma unroll
        for (int s = 0; s < NP; ++s) w[s] = p32b[(size_t)off[s] + ci];
    } else {
        const double* base = g.unk + (int64_t)blk * g.nvar * GB_N3 + ci;
#pragma unroll
        for (int s = 0; s < NP; ++s) w[s] = (MHD || s < 5) ? (T)base[off[s]] : (T)0;
    }
}

// normal-direction PPM and the normal MHD term of direction d; wp, wn, wc
// come back in the rotated frame, s_sig / s_abn in the unrotated one
// ld(m, w): the rotated primitives of stencil point m (0..4, centre 2)
template <typename T, bool MHD, int TILE, typename LD>
__device__ __forceinline__ void recon_normal_ld(const gb_dev_grid& g, T gam, const T* dtd, const T* hd, int d, int blk,
                                                int i, int j, int k, int lane, const float* p32b, const LD& ld,
                                                T (*s_sig)[NP][TILE], T (*s_abn)[NP][TILE], T (*s_dnb)[TILE], T* wp,
                                                T* wn, T* wc)
{
    T qs[5][NP];
#pragma unroll
    for (int m = 0; m < 5; ++m) ld(m, qs[m]);
#pragma unroll
    for (int s = 0; s < NP; ++s) wc[s] = qs[2][s];
    T sgr[NP];
    ppm_normal<T, MHD>(gam, qs, pick3(d, dtd[0], dtd[1], dtd[2]), wp, wn, sgr);
    const int us[NP] = {0, rot_slot_rt<1>(d), rot_slot_rt<2>(d), rot_slot_rt<3>(d), 4,
                        rot_slot_rt<5>(d), rot_slot_rt<6>(d), rot_slot_rt<7>(d)};
#pragma unroll
    for (int s = 0; s < NP; ++s) s_sig[d][us[s]][lane] = sgr[s];
    if (MHD) {
        // multidimensional terms (hy_uhd_dataReconstOneStep.F90:364-424),
        // in the rotated frame; u.B sums in the unrotated order
        const T p1 = wc[1] * wc[5], p2 = wc[2] * wc[6], p3 = wc[3] * wc[7];
        const T uB = pick3(d, p1, p3, p2) + pick3(d, p2, p1, p3) + pick3(d, p3, p2, p1);
        const T row[NP] = {(T)0, -wc[5] / wc[0], -wc[6] / wc[0], -wc[7] / wc[0], (gam - (T)1) * uB,
                           (T)0, -wc[2], -wc[3]};
        const T hdd = pick3(d, hd[0], hd[1], hd[2]);
        const int fa = gb_fidx(d, i, j, k);
        T dnb = face_b<T>(g, d, blk, fa + (d == 0 ? 1 : (d == 1 ? GB_N : GB_N * GB_N)), p32b) -
                face_b<T>(g, d, blk, fa, p32b);
#pragma unroll
        for (int s = 0; s < NP; ++s) {
            s_abn[d][us[s]][lane] = row[s];
            wp[s] = wp[s] - hdd * row[s] * dnb;
            wn[s] = wn[s] - hdd * row[s] * dnb;
        }
        s_dnb[d][lane] = dnb;
    }
}

template <typename T, bool MHD, int TILE>
__device__ __forceinline__ void recon_normal(const gb_dev_grid& g, T gam, const T* dtd, const T* hd, int d, int blk,
                                             int i, int j, int k, int lane, const float* p32b, const int* off,
                                             T (*s_sig)[NP][TILE], T (*s_abn)[NP][TILE], T (*s_dnb)[TILE], T* wp,
                                             T* wn, T* wc)
{
    const int stride = d == 0 ? 1 : (d == 1 ? GB_N : GB_N * GB_N);
    const int c0 = gb_cidx(i, j, k);
    auto ld = [&](int m, T* w) { load_rot<T, MHD>(g, blk, c0 + (m - 2) * stride, p32b, off, w); };
    recon_normal_ld<T, MHD, TILE>(g, gam, dtd, hd, d, blk, i, j, k, lane, p32b, ld, s_sig, s_abn, s_dnb, wp, wn, wc);
}

// the cell-centred electric field along d, -(v x B)_d, of the mean of the
// cell's two face states along d (rotated frame: slots 2, 3 are the
// velocities along a = (d + 1) % 3 and b = (d + 2) % 3, slots 6, 7 their
// fields): the edge fields' reference at the fluxes' time level
template <typename T>
__device__ __forceinline__ T ecc_of(const T* wp, const T* wn)
{
    const T va = (T)0.5 * (wp[2] + wn[2]), vb = (T)0.5 * (wp[3] + wn[3]);
    const T Ba = (T)0.5 * (wp[6] + wn[6]), Bb = (T)0.5 * (wp[7] + wn[7]);
    return vb * Ba - va * Bb;
}

// wn[s] -= a b and wp[s] -= a b: both states take the same correction, so
// the mixed path applies it to the pair in one packed fma.rn.f32x2 (each
// lane the scalar fused multiply-add's rounding)
template <typename T>
__device__ __forceinline__ void sub_both(T* wn, T* wp, int s, T a, T b)
{
    if constexpr (std::is_same<T, float>::value) {
        const float2 r = __ffma2_rn(make_float2(-a, -a), make_float2(b, b), make_float2(wn[s], wp[s]));
        wn[s] = r.x;
        wp[s] = r.y;
    } else {
        wn[s] = wn[s] - a * b;
        wp[s] = wp[s] - a * b;
    }
}

// transverse corrections of direction d in the vendored order
// (hy_uhd_dataReconstOneStep.F90:1006-1089), wp / wn in d's rotated frame
template <typename T, bool MHD, int TILE>
__device__ __forceinline__ void recon_transverse(const T* hd, int d, int lane, T (*s_sig)[NP][TILE],
                                                 T (*s_abn)[NP][TILE], T (*s_dnb)[TILE], T* wp, T* wn)
{
    constexpr int nv = MHD ? 8 : 5;
    const int us[NP] = {0, rot_slot_rt<1>(d), rot_slot_rt<2>(d), rot_slot_rt<3>(d), 4,
                        rot_slot_rt<5>(d), rot_slot_rt<6>(d), rot_slot_rt<7>(d)};
    if (d < 2) {
        // the other in-plane direction first (x: y, y: x), then z
        const int o = d == 0 ? 1 : 0;
        const T ho = o == 0 ? hd[0] : hd[1];
#pragma unroll
        for (int s = 0; s < nv; ++s) sub_both<T>(wn, wp, s, ho, s_sig[o][us[s]][lane]);
        if (MHD) {
#pragma unroll
            for (int s = 0; s < nv; ++s) sub_both<T>(wn, wp, s, ho * s_abn[o][us[s]][lane], s_dnb[o][lane]);
        }
#pragma unroll
        for (int s = 0; s < nv; ++s) sub_both<T>(wn, wp, s, hd[2], s_sig[2][us[s]][lane]);
        if (MHD) {
#pragma unroll
            for (int s = 0; s < nv; ++s) sub_both<T>(wn, wp, s, hd[2] * s_abn[2][us[s]][lane], s_dnb[2][lane]);
        }
    } else {
#pragma unroll
        for (int s = 0; s < nv; ++s) {
            sub_both<T>(wn, wp, s, hd[0], s_sig[0][us[s]][lane]);
            sub_both<T>(wn, wp, s, hd[1], s_sig[1][us[s]][lane]);
        }
        if (MHD) {
#pragma unroll
            for (int s = 0; s < nv; ++s) {
                sub_both<T>(wn, wp, s, hd[0] * s_abn[0][us[s]][lane], s_dnb[0][lane]);
                sub_both<T>(wn, wp, s, hd[1] * s_abn[1][us[s]][lane], s_dnb[1][lane]);
            }
        }
    }
}

// gamma, dt/dx and dt/(2 dx) of a block for reconstruction precision T:
// FP32 throughout in the mixed path (no FP64 instruction), the oracle's
// FP64 values otherwise
template <typename T>
__device__ __forceinline__ void recon_consts(const gb_dev_grid& g, const hydro_kparams& kp, int blk, T& gam, T* dtd, T* hd)
{
    if constexpr (std::is_same<T, float>::value) {
        gam = kp.gammaf;
        kp_dtdxf(kp, gb_block_level(g, blk), dtd);
#pragma unroll
        for (int q = 0; q < 3; ++q) hd[q] = 0.5f * dtd[q];
    } else {
        gam = kp.gamma;
        kp_dtdx(kp, gb_block_level(g, blk), dtd);
#pragma unroll
        for (int q = 0; q < 3; ++q) hd[q] = 0.5 * dtd[q];
    }
}

// One cell and direction of the reconstruction (every thread of the CTA
// calls it together: it holds the barrier between the normal and the
// transverse part): normal-direction PPM and MHD term, hybrid-order check,
// transverse corrections, second hybrid-order check, positivity fallback;
// counts, the cell's CFL code and (MHD) the edge fields' reference. wp, wn
// come back in d's rotated frame. ld(m, w) loads stencil point m; cell is
// the band index (cc the one read when the thread has no cell).
template <typename T, bool MHD, int TILE, typename LD>
__device__ __forceinline__ void recon_item(const gb_dev_grid& g, const hydro_kparams& kp, int cb, int blk, int d,
                                           int lane, int cell, int cc, bool active, int i, int j, int k, T gam,
                                           const T* dtd, const T* hd, const float* p32b, const LD& ld,
                                           T (*s_sig)[NP][TILE], T (*s_abn)[NP][TILE], T (*s_dnb)[TILE],
                                           gb_status* st, T* wp, T* wn)
{
    T wc[NP];
    recon_normal_ld<T, MHD, TILE>(g, gam, dtd, hd, d, blk, i, j, k, lane, p32b, ld, s_sig, s_abn, s_dnb, wp, wn, wc);
    // hybrid order before the transverse corrections
    // (hy_uhd_dataReconstOneStep.F90:934-999): where the flow compresses, a
    // direction whose states fail the Rankine-Hugoniot check falls back to
    // the cell's state (the transverse terms already computed stay)
    bool comp = false, rh = false;
    unsigned code = 0;
    if (kp.hybrid) {
        // (gamma p + B.B) / rho, B.B summed in x, y, z order
        const T b0 = rn_mul(wc[5], wc[5]), b1 = rn_mul(wc[6], wc[6]), b2 = rn_mul(wc[7], wc[7]);
        T cs = rn_add(rn_mul(gam, wc[4]), rn_add(rn_add(pick3(d, b0, b2, b1), pick3(d, b1, b0, b2)), pick3(d, b2, b1, b0)));
        cs = rn_sqrt(rn_div(cs, wc[0]));
        comp = ((const T*)kp.divu)[(size_t)cb * NRC + cc] < rn_mul((T)kp.kappa, cs);
        if (comp && (rh_fail(gam, wc[0], wp[0]) || rh_fail(gam, wc[0], wn[0]))) {
#pragma unroll
            for (int v = 0; v < NP; ++v) { wn[v] = wc[v]; wp[v] = wc[v]; }
            if (kp.lower_cfl) code |= 1u;
            rh = true;
        }
    }
    __syncthreads();
    recon_transverse<T, MHD, TILE>(hd, d, lane, s_sig, s_abn, s_dnb, wp, wn);
    // hybrid order after them (:1150-1218): a fallback in any direction
    // lowers the cell's CFL to 0.25 (3-D)
    if (comp && (rh_fail(gam, wc[0], wp[0]) || rh_fail(gam, wc[0], wn[0]))) {
#pragma unroll
        for (int v = 0; v < NP; ++v) { wn[v] = wc[v]; wp[v] = wc[v]; }
        code |= 2u;
        rh = true;
    }
    // positivity fallback (density and pressure keep their slots in every
    // frame), lowering the cell's CFL (:1230-1272)
    bool fell = (wn[0] < (T)0 || wp[0] < (T)0 || wn[4] < (T)0 || wp[4] < (T)0);
    if (fell) {
#pragma unroll
        for (int v = 0; v < NP; ++v) { wn[v] = wc[v]; wp[v] = wc[v]; }
        code |= 1u;
    }
    if (!active) return;
    if (st) {
        gb_count_warp(&st->n_fallback, fell);
        if (kp.hybrid) gb_count_warp(&st->n_rh_fallback, rh);
    }
    if (kp.cflc && i >= LO && i <= HI && j >= LO && j <= HI && k >= LO && k <= HI)
        kp.cflc[((size_t)blk * 3 + d) * (GB_NXB * GB_NXB * GB_NXB) + (i - LO) + GB_NXB * ((j - LO) + GB_NXB * (k - LO))] =
            (unsigned char)code;
    if (MHD) ((T*)kp.ecc)[((size_t)cb * 3 + d) * NRC + cell] = ecc_of(wp, wn);
}

// MINB: resident CTAs per SM the register allocation must allow (1 = no
// bound); the autotuner chooses between the unbounded kernel and a bound
// that trades spills for occupancy
template <typename T, bool MHD, int TILE, int MINB>
__global__ void __launch_bounds__(3 * TILE, MINB)
k_recon(gb_dev_grid g, hydro_kparams kp, const int* __restrict__ list, T* __restrict__ scr,
        size_t scr_stride, const float* __restrict__ p32, size_t p32_stride, gb_status* st)
{
    __shared__ T s_sig[3][NP][TILE];
    __shared__ T s_abn[3][NP][TILE];
    __shared__ T s_dnb[3][TILE];
    const int lane = threadIdx.x % TILE;
    const int d = threadIdx.x / TILE;
    const int cb = blockIdx.y;
    const int blk = list[cb];
    const int cell = blockIdx.x * TILE + lane;
    const bool active = cell < NRC;
    const int cc = active ? cell : 0;
    const int i = RLO + cc % RB, j = RLO + (cc / RB) % RB, k = RLO + cc / (RB * RB);
    T gam, dtd[3], hd[3];
    recon_consts<T>(g, kp, blk, gam, dtd, hd);
    const float* p32b = p32 + (size_t)cb * p32_stride;
    int off[NP];
    rot_offsets<T, MHD>(g, d, off);
    const int stride = d == 0 ? 1 : (d == 1 ? GB_N : GB_N * GB_N);
    const int c0 = gb_cidx(i, j, k);
    auto ld = [&](int m, T* w) { load_rot<T, MHD>(g, blk, c0 + (m - 2) * stride, p32b, off, w); };
    T wp[NP], wn[NP];
    recon_item<T, MHD, TILE>(g, kp, cb, blk, d, lane, cell, cc, active, i, j, k, gam, dtd, hd, p32b, ld, s_sig, s_abn,
                             s_dnb, st, wp, wn);
    if (!active) return;
    T* out = scr + (size_t)cb * scr_stride;
    const int us[NP] = {0, rot_slot_rt<1>(d), rot_slot_rt<2>(d), rot_slot_rt<3>(d), 4,
                        rot_slot_rt<5>(d), rot_slot_rt<6>(d), rot_slot_rt<7>(d)};
    // the Riemann solver takes the normal field from the face, not from the
    // states (and hydro has no field): those planes are neither written here
    // nor read there
#pragma unroll
    for (int s = 0; s < (MHD ? NP : 5); ++s) {
        if (s == 5) continue;
        out[((size_t)(0 * 3 + d) * NP + us[s]) * NRC + cell] = wp[s];
        out[((size_t)(1 * 3 + d) * NP + us[s]) * NRC + cell] = wn[s];
    }
}

// ---------------------------------------------------------------- Riemann
template <typename T>
__device__ __forceinline__ void hllc(T gam, const T* L, const T* R, T* F, T* un)
{
    T gm1 = gam - (T)1;
    T aL = sqrt(gam * L[4] / L[0]), aR = sqrt(gam * R[4] / R[0]);
    T SL = fmin(L[1] - aL, R[1] - aR);
    T SR = fmax(L[1] + aL, R[1] + aR);
    T EL = L[4] / gm1 + (T)0.5 * L[0] * (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]);
    T ER = R[4] / gm1 + (T)0.5 * R[0] * (R[1] * R[1] + R[2] * R[2] + R[3] * R[3]);
    T FL[5] = {L[0] * L[1], L[0] * L[1] * L[1] + L[4], L[0] * L[1] * L[2], L[0] * L[1] * L[3], L[1] * (EL + L[4])};
    T FR[5] = {R[0] * R[1], R[0] * R[1] * R[1] + R[4], R[0] * R[1] * R[2], R[0] * R[1] * R[3], R[1] * (ER + R[4])};
#pragma unroll
    for (int s = 0; s < NP; ++s) F[s] = (T)0;
    if (SL >= (T)0) {
#pragma unroll
        for (int s = 0; s < 5; ++s) F[s] = FL[s];
        *un = L[1];
        return;
    }
    if (SR <= (T)0) {
#pragma unroll
        for (int s = 0; s < 5; ++s) F[s] = FR[s];
        *un = R[1];
        return;
    }
    T SM = (R[4] - L[4] + L[0] * L[1] * (SL - L[1]) - R[0] * R[1] * (SR - R[1])) /
           (L[0] * (SL - L[1]) - R[0] * (SR - R[1]));
    *un = SM;
    const bool left = SM >= (T)0;
    const T* W = left ? L : R;
    T S = left ? SL : SR;
    T E = left ? EL : ER;
    T fac = W[0] * (S - W[1]) / (S - SM);
    T Us[5] = {fac, fac * SM, fac * W[2], fac * W[3],
               fac * (E / W[0] + (SM - W[1]) * (SM + W[4] / (W[0] * (S - W[1]))))};
    T Uw[5] = {W[0], W[0] * W[1], W[0] * W[2], W[0] * W[3], E};
#pragma unroll
    for (int s = 0; s < 5; ++s) F[s] = (left ? FL[s] : FR[s]) + S * (Us[s] - Uw[s]);
}

template <typename T>
__device__ __forceinline__ void mhd_flux(const T* W, T bx, T E, T pT, T* F)
{
    T vB = W[1] * bx + W[2] * W[6] + W[3] * W[7];
    F[0] = W[0] * W[1];
    F[1] = W[0] * W[1] * W[1] + pT - bx * bx;
    F[2] = W[0] * W[1] * W[2] - bx * W[6];
    F[3] = W[0] * W[1] * W[3] - bx * W[7];
    F[4] = (E + pT) * W[1] - bx * vB;
    F[5] = (T)0;
    F[6] = W[6] * W[1] - bx * W[2];
    F[7] = W[7] * W[1] - bx * W[3];
}

template <typename T>
__device__ __forceinline__ T hlld_eps();
template <>
__device__ __forceinline__ double hlld_eps<double>() { return 1e-12; }
template <>
__device__ __forceinline__ float hlld_eps<float>() { return 1e-6f; }

template <typename T>
__device__ __forceinline__ void hlld(T gam, const T* L, const T* R, T* F, T* un)
{
    const T gm1 = gam - (T)1;
    const T bx = L[5];
    T bx2 = bx * bx;
    T BL2 = bx2 + L[6] * L[6] + L[7] * L[7];
    T BR2 = bx2 + R[6] * R[6] + R[7] * R[7];
    T pTL = L[4] + (T)0.5 * BL2, pTR = R[4] + (T)0.5 * BR2;
    T EL = L[4] / gm1 + (T)0.5 * L[0] * (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]) + (T)0.5 * BL2;
    T ER = R[4] / gm1 + (T)0.5 * R[0] * (R[1] * R[1] + R[2] * R[2] + R[3] * R[3]) + (T)0.5 * BR2;
    T gpl = gam * L[4], gpr = gam * R[4];
    T tl = (gpl + BL2) / L[0], tr = (gpr + BR2) / R[0];
    T cfL = sqrt((T)0.5 * (tl + sqrt(fmax(tl * tl - (T)4 * gpl * bx2 / (L[0] * L[0]), (T)0))));
    T cfR = sqrt((T)0.5 * (tr + sqrt(fmax(tr * tr - (T)4 * gpr * bx2 / (R[0] * R[0]), (T)0))));
    T cmax = fmax(cfL, cfR);
    T SL = fmin(L[1], R[1]) - cmax;
    T SR = fmax(L[1], R[1]) + cmax;
    T FL[NP], FR[NP];
    mhd_flux<T>(L, bx, EL, pTL, FL);
    mhd_flux<T>(R, bx, ER, pTR, FR);
    if (SL >= (T)0) {
#pragma unroll
        for (int s = 0; s < NP; ++s) F[s] = FL[s];
        *un = L[1];
        return;
    }
    if (SR <= (T)0) {
#pragma unroll
        for (int s = 0; s < NP; ++s) F[s] = FR[s];
        *un = R[1];
        return;
    }
    T sdl = SL - L[1], sdr = SR - R[1];
    T den = sdr * R[0] - sdl * L[0];
    T SM = (sdr * R[0] * R[1] - sdl * L[0] * L[1] - pTR + pTL) / den;
    T pTs = (sdr * R[0] * pTL - sdl * L[0] * pTR + L[0] * R[0] * sdr * sdl * (R[1] - L[1])) / den;
    *un = SM;
    T Us[2][NP], Uo[2][NP], sqs[2], vst[2], wst[2], byst[2], bzst[2], vBst[2];
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        const T* W = a == 0 ? L : R;
        T S = a == 0 ? SL : SR;
        T Ea = a == 0 ? EL : ER;
        T pTa = a == 0 ? pTL : pTR;
        T sd = S - W[1];
        T rs = W[0] * sd / (S - SM);
        T t1 = W[0] * sd * (S - SM);
        T dd = t1 - bx2;
        T vs, ws, bys, bzs;
        if (fabs(dd) < hlld_eps<T>() * (fabs(t1) + bx2)) {
            vs = W[2]; ws = W[3]; bys = W[6]; bzs = W[7];
        } else {
            T q = (SM - W[1]) / dd;
            vs = W[2] - bx * W[6] * q;
            ws = W[3] - bx * W[7] * q;
            T r = (W[0] * sd * sd - bx2) / dd;
            bys = W[6] * r;
            bzs = W[7] * r;
        }
        T vB = W[1] * bx + W[2] * W[6] + W[3] * W[7];
        T vBs = SM * bx + vs * bys + ws * bzs;
        T Est = (sd * Ea - pTa * W[1] + pTs * SM + bx * (vB - vBs)) / (S - SM);
        Us[a][0] = rs; Us[a][1] = rs * SM; Us[a][2] = rs * vs; Us[a][3] = rs * ws;
        Us[a][4] = Est; Us[a][5] = bx; Us[a][6] = bys; Us[a][7] = bzs;
        Uo[a][0] = W[0]; Uo[a][1] = W[0] * W[1]; Uo[a][2] = W[0] * W[2]; Uo[a][3] = W[0] * W[3];
        Uo[a][4] = Ea; Uo[a][5] = bx; Uo[a][6] = W[6]; Uo[a][7] = W[7];
        sqs[a] = sqrt(rs);
        vst[a] = vs; wst[a] = ws; byst[a] = bys; bzst[a] = bzs; vBst[a] = vBs;
    }
    T Ss0 = SM - fabs(bx) / sqs[0];
    T Ss1 = SM + fabs(bx) / sqs[1];
    if (Ss0 >= (T)0) {
#pragma unroll
        for (int s = 0; s < NP; ++s) F[s] = FL[s] + SL * (Us[0][s] - Uo[0][s]);
        return;
    }
    if (Ss1 <= (T)0) {
#pragma unroll
        for (int s = 0; s < NP; ++s) F[s] = FR[s] + SR * (Us[1][s] - Uo[1][s]);
        return;
    }
    T sgn = bx >= (T)0 ? (T)1 : (T)-1;
    T isum = (T)1 / (sqs[0] + sqs[1]);
    T vss = (sqs[0] * vst[0] + sqs[1] * vst[1] + (byst[1] - byst[0]) * sgn) * isum;
    T wss = (sqs[0] * wst[0] + sqs[1] * wst[1] + (bzst[1] - bzst[0]) * sgn) * isum;
    T byss = (sqs[0] * byst[1] + sqs[1] * byst[0] + sqs[0] * sqs[1] * (vst[1] - vst[0]) * sgn) * isum;
    T bzss = (sqs[0] * bzst[1] + sqs[1] * bzst[0] + sqs[0] * sqs[1] * (wst[1] - wst[0]) * sgn) * isum;
    T vBss = SM * bx + vss * byss + wss * bzss;
    const bool left = SM >= (T)0;
    // the side's states picked with selects (a runtime index into Us / Uo
    // would put both arrays in local memory)
    T Ua[NP], Uoa[NP];
#pragma unroll
    for (int s = 0; s < NP; ++s) {
        Ua[s] = left ? Us[0][s] : Us[1][s];
        Uoa[s] = left ? Uo[0][s] : Uo[1][s];
    }
    T Ess = left ? Us[0][4] - sqs[0] * (vBst[0] - vBss) * sgn : Us[1][4] + sqs[1] * (vBst[1] - vBss) * sgn;
    T Uss[NP] = {Ua[0], Ua[0] * SM, Ua[0] * vss, Ua[0] * wss, Ess, bx, byss, bzss};
    T S = left ? SL : SR;
    T Sst = left ? Ss0 : Ss1;
#pragma unroll
    for (int s = 0; s < NP; ++s)
        F[s] = (left ? FL[s] : FR[s]) + S * (Ua[s] - Uoa[s]) + Sst * (Uss[s] - Ua[s]);
}

// flux box of direction d: along d faces 4..20 (17), across d cells 3..20
// (18), x fastest whatever d is, so that neighbouring threads read
// neighbouring cells and faces in every direction (a normal-first order
// puts neighbouring y and z faces 18 and 324 cells apart)
// ---- the normal field of the Riemann problems at t + dt/2
// (Gardiner & Stone 2005 sec. 4, 2008 sec. 5): dB_d/dt = -(d_a E_b - d_b E_a)
// over half a step with time-n edge fields, each the mean of the four
// cell-centred E_c = v_b B_a - v_a B_b around the edge (a = c + 1, b = c + 2
// cyclically), summed in a fixed order. Only the edges some flux-box face
// needs are formed: at most one of A, B outside the interior faces 4..20,
// so every cell read lies in the step's filled read region.
__device__ __forceinline__ int en_index(int x, int y, int z)
{
    return (x - RLO) + EB * ((y - RLO) + EB * (z - RLO));
}

// One CTA per block, direction c and half of the band along c (9 cells):
// the cell-centred E_c of the 20 x 20 x 9 cells around its edges once into
// shared memory, then each edge the mean of its four, written x-fastest.
constexpr int EN_HALF = RB / 2;  // cells along c per CTA
constexpr int EN_THREADS = 256;

template <typename T, int C>
__device__ __forceinline__ void edge_n_dir(const gb_dev_grid& g, int blk, const float* __restrict__ pb,
                                           T* __restrict__ out, int half, T* ec)
{
    // ec: the cells' E_c over a box of 9 cells along c (this CTA's half)
    // and 20 across (2..21), x fastest like the store: both passes run x
    // fastest, so global loads coalesce and shared accesses do not conflict
    constexpr int c = C, a = (C + 1) % 3, bb = (C + 2) % 3;
    constexpr int X0 = c == 0 ? EN_HALF : 20, X1 = c == 1 ? EN_HALF : 20, X2 = c == 2 ? EN_HALF : 20;
    constexpr int NCELL = X0 * X1 * X2;
    constexpr int SA = a == 0 ? 1 : (a == 1 ? X0 : X0 * X1), SB = bb == 0 ? 1 : (bb == 1 ? X0 : X0 * X1);
    const int C0 = RLO + half * EN_HALF;
    const int o[3] = {c == 0 ? C0 : RLO - 1, c == 1 ? C0 : RLO - 1, c == 2 ? C0 : RLO - 1};
    const double* base = g.unk + (int64_t)blk * g.nvar * GB_N3;
    for (int t = threadIdx.x; t < NCELL; t += EN_THREADS) {
        int x[3];
        x[0] = o[0] + t % X0;
        x[1] = o[1] + (t / X0) % X1;
        x[2] = o[2] + t / (X0 * X1);
        T e = (T)0;
        // cells outside the band along both a and bb lie outside the step's
        // filled read region and feed only edges no face needs
        if ((x[a] >= RLO && x[a] <= RLO + RB - 1) || (x[bb] >= RLO && x[bb] <= RLO + RB - 1)) {
            const int cidx = gb_cidx(x[0], x[1], x[2]);
            T va, vb, Ba, Bb;
            if constexpr (std::is_same<T, float>::value) {
                va = pb[(size_t)(1 + a) * GB_N3 + cidx];
                vb = pb[(size_t)(1 + bb) * GB_N3 + cidx];
                Ba = pb[(size_t)(5 + a) * GB_N3 + cidx];
                Bb = pb[(size_t)(5 + bb) * GB_N3 + cidx];
            } else {
                va = base[(int64_t)g.slot[GB_VELX + a] * GB_N3 + cidx];
                vb = base[(int64_t)g.slot[GB_VELX + bb] * GB_N3 + cidx];
                Ba = base[(int64_t)g.slot[GB_MAGX + a] * GB_N3 + cidx];
                Bb = base[(int64_t)g.slot[GB_MAGX + bb] * GB_N3 + cidx];
            }
            e = vb * Ba - va * Bb;
        }
        ec[t] = e;
    }
    __syncthreads();
    // edge positions: 19 along each axis but c (9), x fastest
    constexpr int E0 = c == 0 ? EN_HALF : EB, E1 = c == 1 ? EN_HALF : EB;
    constexpr int NE = EN_HALF * EB * EB;
    for (int t = threadIdx.x; t < NE; t += EN_THREADS) {
        int X[3];
        X[0] = (c == 0 ? C0 : RLO) + t % E0;
        X[1] = (c == 1 ? C0 : RLO) + (t / E0) % E1;
        X[2] = (c == 2 ? C0 : RLO) + t / (E0 * E1);
        const int A = X[a], B = X[bb];
        T v = (T)0;
        if ((A >= LO && A <= HI + 1) || (B >= LO && B <= HI + 1)) {
            // the cell at A - 1, B - 1 and its neighbours +1 along a and bb
            const int s00 = (X[0] - o[0]) + X0 * ((X[1] - o[1]) + X1 * (X[2] - o[2])) - SA - SB;
            v = (T)0.25 * (((ec[s00] + ec[s00 + SB]) + ec[s00 + SA]) + ec[s00 + SA + SB]);
        }
        out[(size_t)c * NEN + en_index(X[0], X[1], X[2])] = v;
    }
}

template <typename T, bool MHD>
__global__ void __launch_bounds__(EN_THREADS)
k_edge_n(gb_dev_grid g, const int* __restrict__ list, const float* __restrict__ p32, size_t p32_stride,
         T* __restrict__ escr, size_t estride)
{
    if (!MHD) return;
    const int cb = blockIdx.y;
    const int blk = list[cb];
    const float* pb = p32 + (size_t)cb * p32_stride;
    T* out = escr + (size_t)cb * estride;
    __shared__ T ec[EN_HALF * 20 * 20];
    const int c = blockIdx.x >> 1, half = blockIdx.x & 1;
    if (c == 0) edge_n_dir<T, 0>(g, blk, pb, out, half, ec);
    else if (c == 1) edge_n_dir<T, 1>(g, blk, pb, out, half, ec);
    else edge_n_dir<T, 2>(g, blk, pb, out, half, ec);
}

// the half-step normal field of flux-box face (I) of direction D
template <typename T, int D>
__device__ __forceinline__ T face_b_half(T bnf, const T* en, const int* I, const T* dtd)
{
    constexpr int d = D, a = (D + 1) % 3, bb = (D + 2) % 3;
    // edges along bb at a -/+ 1/2 and along a at bb -/+ 1/2, each at the
    // face's own position otherwise (x, y, z addressing)
    int Ia[3] = {I[0], I[1], I[2]}, Ib[3] = {I[0], I[1], I[2]};
    Ia[a] += 1;
    Ib[bb] += 1;
    const T eb_lo = en[(size_t)bb * NEN + en_index(I[0], I[1], I[2])];
    const T eb_hi = en[(size_t)bb * NEN + en_index(Ia[0], Ia[1], Ia[2])];
    const T ea_lo = en[(size_t)a * NEN + en_index(I[0], I[1], I[2])];
    const T ea_hi = en[(size_t)a * NEN + en_index(Ib[0], Ib[1], Ib[2])];
    return bnf - (T)0.5 * (dtd[a] * (eb_hi - eb_lo) - dtd[bb] * (ea_hi - ea_lo));
}

__device__ __forceinline__ void flux_coords(int d, int f, int* I)
{
    const int n0 = d == 0 ? 17 : RB, n1 = d == 1 ? 17 : RB;
    const int e0 = f % n0, e1 = (f / n0) % n1, e2 = f / (n0 * n1);
    I[0] = (d == 0 ? LO : RLO) + e0;
    I[1] = (d == 1 ? LO : RLO) + e1;
    I[2] = (d == 2 ? LO : RLO) + e2;
}
__device__ __forceinline__ int flux_index(int d, int i, int j, int k)
{
    const int n0 = d == 0 ? 17 : RB, n1 = d == 1 ? 17 : RB;
    return (i - (d == 0 ? LO : RLO)) + n0 * ((j - (d == 1 ? LO : RLO)) + n1 * (k - (d == 2 ? LO : RLO)));
}
__device__ __forceinline__ int rc_index(int i, int j, int k)
{
    return (i - RLO) + RB * ((j - RLO) + RB * (k - RLO));
}

// ---------------------------------------------------------------- k_flux
// The flux at one face of direction D from the left cell's + state wl and
// the right cell's - state wr (unrotated; the normal field bnf from the
// face): HLLC / HLLD, the rho e_int flux upwinded by the mass flux, and
// artificial viscosity from the cell values U(role, ci) of the two cells
// (cell indices cil, cir). out is unrotated.
template <typename T, bool MHD, int D, typename UL>
__device__ __forceinline__ void face_flux_core(const hydro_kparams& kp, const T* wl, const T* wr, T bnf, const UL& U,
                                               int cil, int cir, T* out, T& feint, T& un)
{
    constexpr int d = D;
    T Lr[NP], Rr[NP], Fr[NP];
#pragma unroll
    for (int s = 0; s < NP; ++s) {
        Lr[s] = wl[rot_slot(d, s)];
        Rr[s] = wr[rot_slot(d, s)];
    }
    const T gam = std::is_same<T, float>::value ? (T)kp.gammaf : (T)kp.gamma;
    if (MHD) {
        Lr[5] = bnf;
        Rr[5] = bnf;
        hlld<T>(gam, Lr, Rr, Fr, &un);
    } else {
        hllc<T>(gam, Lr, Rr, Fr, &un);
    }
#pragma unroll
    for (int s = 0; s < NP; ++s) out[rot_slot(d, s)] = Fr[s];
    const T gm1 = gam - (T)1;
    T eL = Lr[4] / (gm1 * Lr[0]), eR = Rr[4] / (gm1 * Rr[0]);
    feint = Fr[0] * (Fr[0] >= (T)0 ? eL : eR);
    if (kp.use_avisc) {
        T dv = U(GB_VELX + d, cir) - U(GB_VELX + d, cil);
        T vis = (std::is_same<T, float>::value ? (T)kp.cviscf : (T)kp.cvisc) * fmax(-dv, (T)0);
        if (vis > (T)0) {
            T rl = U(GB_DENS, cil), rr = U(GB_DENS, cir);
            T vl[3] = {U(GB_VELX, cil), U(GB_VELY, cil), U(GB_VELZ, cil)};
            T vr[3] = {U(GB_VELX, cir), U(GB_VELY, cir), U(GB_VELZ, cir)};
            T Bl[3] = {(T)0, (T)0, (T)0}, Br[3] = {(T)0, (T)0, (T)0};
            if (MHD) {
#pragma unroll
                for (int c = 0; c < 3; ++c) { Bl[c] = U(GB_MAGX + c, cil); Br[c] = U(GB_MAGX + c, cir); }
            }
            T pl = U(GB_PRES, cil), pr = U(GB_PRES, cir);
            T ul[NP], ur[NP];
            ul[0] = rl; ur[0] = rr;
#pragma unroll
            for (int c = 0; c < 3; ++c) { ul[1 + c] = rl * vl[c]; ur[1 + c] = rr * vr[c]; }
            ul[4] = pl / gm1 + (T)0.5 * rl * (vl[0] * vl[0] + vl[1] * vl[1] + vl[2] * vl[2]) +
                    (T)0.5 * (Bl[0] * Bl[0] + Bl[1] * Bl[1] + Bl[2] * Bl[2]);
            ur[4] = pr / gm1 + (T)0.5 * rr * (vr[0] * vr[0] + vr[1] * vr[1] + vr[2] * vr[2]) +
                    (T)0.5 * (Br[0] * Br[0] + Br[1] * Br[1] + Br[2] * Br[2]);
#pragma unroll
            for (int c = 0; c < 3; ++c) { ul[5 + c] = Bl[c]; ur[5 + c] = Br[c]; }
#pragma unroll
            for (int s = 0; s < NP; ++s) {
                if (s == 5 + d) continue;
                if (!MHD && s >= 5) continue;
                out[s] = out[s] + vis * (ul[s] - ur[s]);
            }
            T el = rl * U(GB_EINT, cil), er = rr * U(GB_EINT, cir);
            feint = feint + vis * (el - er);
        }
    }
}

// the face's fluxes into the flux scratch of its block (f: index in the
// direction's flux box); the normal field's flux (and hydro's field
// fluxes) are never read: not stored
template <typename T, bool MHD, int D>
__device__ __forceinline__ void face_flux_store(T* fs, int f, const T* out, T feint, T un)
{
    constexpr int d = D;
#pragma unroll
    for (int s = 0; s < NP; ++s)
        if (s != 5 + d && (MHD || s < 5)) fs[(size_t)s * NFC + f] = out[s];
    fs[(size_t)8 * NFC + f] = feint;
    fs[(size_t)9 * NFC + f] = un;
}

template <typename T, bool MHD, int D>
__device__ __forceinline__ void flux_face(gb_dev_grid g, hydro_kparams kp, const int* __restrict__ list, const T* __restrict__ rscr,
       size_t rstride, T* __restrict__ fscr, size_t fstride, const float* __restrict__ p32, size_t p32_stride)
{
    constexpr int d = D;
    const int cb = blockIdx.z;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= NFC) return;
    const int blk = list[cb];
    int I[3];
    flux_coords(d, f, I);
    int Il[3] = {I[0], I[1], I[2]};
    Il[d] -= 1;
    const T* rs = rscr + (size_t)cb * rstride;
    const int cl = rc_index(Il[0], Il[1], Il[2]), cr = rc_index(I[0], I[1], I[2]);
    T wl[NP], wr[NP];
#pragma unroll
    for (int v = 0; v < NP; ++v) {
        // the normal field (v = 5 + d) comes from the face below; hydro has
        // no field: those state planes are not written
        if (v == 5 + d || (!MHD && v >= 5)) {
            wl[v] = (T)0;
            wr[v] = (T)0;
            continue;
        }
        wl[v] = rs[((size_t)(0 * 3 + d) * NP + v) * NRC + cl];
        wr[v] = rs[((size_t)(1 * 3 + d) * NP + v) * NRC + cr];
    }
    const float* pb = p32 + (size_t)cb * p32_stride;
    T bnf = (T)0;
    if (MHD) {
        T dtd[3];
        if constexpr (std::is_same<T, float>::value) kp_dtdxf(kp, gb_block_level(g, blk), dtd);
        else kp_dtdx(kp, gb_block_level(g, blk), dtd);
        bnf = face_b_half<T, D>(face_b<T>(g, d, blk, gb_fidx(d, I[0], I[1], I[2]), pb),
                                (const T*)kp.edgen + (size_t)cb * scratch_layout<T>::edgen, I, dtd);
    }
    const double* base = g.unk + (int64_t)blk * g.nvar * GB_N3;
    auto U = [&](int role, int ci) -> T {
        if constexpr (std::is_same<T, float>::value) {
            const int v = role == GB_EINT ? 8 : (role >= GB_MAGX ? 5 + (role - GB_MAGX) : role);
            return pb[(size_t)v * GB_N3 + ci];
        } else {
            return (T)base[(int64_t)g.slot[role] * GB_N3 + ci];
        }
    };
    T out[NP], feint, un;
    face_flux_core<T, MHD, D>(kp, wl, wr, bnf, U, gb_cidx(Il[0], Il[1], Il[2]), gb_cidx(I[0], I[1], I[2]), out, feint,
                              un);
    face_flux_store<T, MHD, D>(fscr + (size_t)cb * fstride + (size_t)d * NFLX * NFC, f, out, feint, un);
}

// mixed path: eight resident CTAs per SM (64 registers, no spills) to hide
// the latency of the face-state loads; the FP64 Riemann solvers need more
template <typename T, bool MHD>
__global__ void __launch_bounds__(128, std::is_same<T, float>::value ? 8 : 1)
k_flux(gb_dev_grid g, hydro_kparams kp, const int* __restrict__ list, const T* __restrict__ rscr,
       size_t rstride, T* __restrict__ fscr, size_t fstride, const float* __restrict__ p32, size_t p32_stride)
{
    // the direction is uniform over the CTA: a compile-time index in each branch
    if (blockIdx.y == 0) flux_face<T, MHD, 0>(g, kp, list, rscr, rstride, fscr, fstride, p32, p32_stride);
    else if (blockIdx.y == 1) flux_face<T, MHD, 1>(g, kp, list, rscr, rstride, fscr, fstride, p32, p32_stride);
    else flux_face<T, MHD, 2>(g, kp, list, rscr, rstride, fscr, fstride, p32, p32_stride);
}

// ---------------------------------------------------------------- k_emf
template <typename R>
__device__ __forceinline__ R upw(R f, R a, R b)
{
    return f > (R)0 ? a : (f < (R)0 ? b : (R)0.5 * (a + b));
}

// edge box of direction c: along c cells 4..19 (16), along a and b faces 4..20 (17).
// The electric field is computed in the reconstruction precision T from the
// Riemann fluxes and the cell-centred v x B (FP32 copies of the primitives
// in the mixed path); it is stored as double and the face-B update that
// consumes it stays FP64. Every edge value is shared by the four faces
// around the edge, so div B is kept to round-off in either precision.
// One CTA takes one plane C of the edges of direction CD (a compile-time
// axis, so the axis permutations of every index fold away): the cell-centred
// field of the plane's 18 x 18 cells is computed once into shared memory
// (each value serves four edges), then each thread makes one of the 17 x 17
// edges from its four face fluxes and four cell values.
constexpr int EMF_THREADS = 320;
constexpr int EMF_CELLS = RB * RB;     // cells 3..20 across the plane
constexpr int EMF_EDGES = 17 * 17;     // edges 4..20 across the plane

template <typename T, int CD>
__device__ __forceinline__ void emf_plane(const int* __restrict__ list, const T* __restrict__ rscr, size_t rstride,
                                          const T* __restrict__ fscr, size_t fstride, double* __restrict__ escr,
                                          size_t estride, T* s_ecc)
{
    using R = T;
    constexpr int c = CD;
    constexpr int a = (c + 1) % 3, b = (c + 2) % 3;
    const int cb = blockIdx.z;
    const int C = LO + blockIdx.x;
    int t[3];
    auto at = [&](int av, int bv, int cv) { t[a] = av; t[b] = bv; t[c] = cv; };
    // the cell-centred reference field at the fluxes' time level t + dt/2,
    // -(v x B)_c of the mean of the cell's two face states along c (time
    // centred by the tracing and the other directions' transverse terms; v
    // and B along a and b are tangential to c), written by the
    // reconstruction: a plane-parallel flow then gets the 1-D Riemann flux
    // at every edge (Gardiner & Stone 2005 sec. 3). x runs fastest across
    // the threads where the plane has an x axis (a for c = 2, b for c = 1).
    const T* es = rscr + (size_t)cb * rstride + (size_t)c * NRC;
    for (int q = threadIdx.x; q < EMF_CELLS; q += EMF_THREADS) {
        const int qa = c == 1 ? q / RB : q % RB, qb = c == 1 ? q % RB : q / RB;
        at(RLO + qa, RLO + qb, C);
        s_ecc[qa + RB * qb] = es[rc_index(t[0], t[1], t[2])];
    }
    __syncthreads();
    const int q = threadIdx.x;
    if (q >= EMF_EDGES) return;
    const int A = LO + (c == 1 ? q / 17 : q % 17), B = LO + (c == 1 ? q % 17 : q / 17);
    const int e = (A - LO) + 17 * (B - LO) + EMF_EDGES * (C - LO);
    const T* fs = fscr + (size_t)cb * fstride;
    auto fl = [&](int d, int var, int x0, int x1, int x2) -> R {
        return (R)fs[(size_t)d * NFLX * NFC + (size_t)var * NFC + flux_index(d, x0, x1, x2)];
    };
    at(A, B - 1, C); R ea0 = -fl(a, 5 + b, t[0], t[1], t[2]); R ma0 = fl(a, 0, t[0], t[1], t[2]);
    at(A, B, C);     R ea1 = -fl(a, 5 + b, t[0], t[1], t[2]); R ma1 = fl(a, 0, t[0], t[1], t[2]);
    at(A - 1, B, C); R eb0 = fl(b, 5 + a, t[0], t[1], t[2]);  R mb0 = fl(b, 0, t[0], t[1], t[2]);
    at(A, B, C);     R eb1 = fl(b, 5 + a, t[0], t[1], t[2]);  R mb1 = fl(b, 0, t[0], t[1], t[2]);
    R ecc[2][2];
#pragma unroll
    for (int ia = 0; ia < 2; ++ia)
#pragma unroll
        for (int ib = 0; ib < 2; ++ib) ecc[ia][ib] = s_ecc[(A - 1 + ia - RLO) + RB * (B - 1 + ib - RLO)];
    const R two = (R)2, eighth = (R)0.125;
    R eavg = (R)0.25 * (ea0 + ea1 + eb0 + eb1);
    R dbm = upw<R>(ma0, two * (eb0 - ecc[0][0]), two * (eb1 - ecc[1][0]));
    R dbp = upw<R>(ma1, two * (ecc[0][1] - eb0), two * (ecc[1][1] - eb1));
    R dam = upw<R>(mb0, two * (ea0 - ecc[0][0]), two * (ea1 - ecc[0][1]));
    R dap = upw<R>(mb1, two * (ecc[1][0] - ea0), two * (ecc[1][1] - ea1));
    const R ev = eavg + eighth * (dbm - dbp) + eighth * (dam - dap);
    if constexpr (std::is_same<R, float>::value) escr[(size_t)cb * estride + (size_t)c * NEDGE + e] = gb_f2d(ev);
    else escr[(size_t)cb * estride + (size_t)c * NEDGE + e] = ev;
}

// grid (16 planes, 3 directions, blocks)
template <typename T>
__global__ void __launch_bounds__(EMF_THREADS)
k_emf(const int* __restrict__ list, const T* __restrict__ rscr, size_t rstride, const T* __restrict__ fscr,
      size_t fstride, double* __restrict__ escr, size_t estride)
{
    __shared__ T s_ecc[EMF_CELLS];
    if (blockIdx.y == 0) emf_plane<T, 0>(list, rscr, rstride, fscr, fstride, escr, estride, s_ecc);
    else if (blockIdx.y == 1) emf_plane<T, 1>(list, rscr, rstride, fscr, fstride, escr, estride, s_ecc);
    else emf_plane<T, 2>(list, rscr, rstride, fscr, fstride, escr, estride, s_ecc);
}

__device__ __forceinline__ int edge_index(int c, int i, int j, int k)
{
    int I[3] = {i, j, k};
    int a = (c + 1) % 3, b = (c + 2) % 3;
    return (I[a] - LO) + 17 * ((I[b] - LO) + 17 * (I[c] - LO));
}

// interior face box of direction a: along a 4..20 (17), across a 4..19
// (16), x fastest whatever a is (neighbouring threads take neighbouring
// faces and cells)
__device__ __forceinline__ void fb_coords(int a, int f, int* I)
{
    const int n0 = a == 0 ? 17 : 16, n1 = a == 1 ? 17 : 16;
    I[0] = LO + f % n0;
    I[1] = LO + (f / n0) % n1;
    I[2] = LO + f / (n0 * n1);
}
__device__ __forceinline__ int fb_index(int a, int i, int j, int k)
{
    const int n0 = a == 0 ? 17 : 16, n1 = a == 1 ? 17 : 16;
    return (i - LO) + n0 * ((j - LO) + n1 * (k - LO));
}

template <int A>
__device__ __forceinline__ void faceb_face(const gb_dev_grid& g, const hydro_kparams& kp, const int* __restrict__ list,
                                           const double* __restrict__ escr, size_t estride, double* __restrict__ bscr,
                                           size_t bstride)
{
    constexpr int a = A;
    const int cb = blockIdx.z;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= NFB) return;
    const int blk = list[cb];
    const int bb = (a + 1) % 3, c = (a + 2) % 3;
    int I[3];
    fb_coords(a, f, I);
    int t1[3] = {I[0], I[1], I[2]}, t3[3] = {I[0], I[1], I[2]};
    t1[bb] += 1;
    t3[c] += 1;
    const double* es = escr + (size_t)cb * estride;
    double ec0 = es[(size_t)c * NEDGE + edge_index(c, I[0], I[1], I[2])];
    double ec1 = es[(size_t)c * NEDGE + edge_index(c, t1[0], t1[1], t1[2])];
    double eb0 = es[(size_t)bb * NEDGE + edge_index(bb, I[0], I[1], I[2])];
    double eb1 = es[(size_t)bb * NEDGE + edge_index(bb, t3[0], t3[1], t3[2])];
    double dtd[3];
    kp_dtdx(kp, gb_block_level(g, blk), dtd);
    double dtd_b = dtd[bb], dtd_c = dtd[c];
    double old = g.f[a][(int64_t)blk * GB_FSZ + gb_fidx(a, I[0], I[1], I[2])];
    bscr[(size_t)cb * bstride + (size_t)a * NFB + f] = old - dtd_b * (ec1 - ec0) + dtd_c * (eb1 - eb0);
}

static __global__ void __launch_bounds__(128)
k_faceb(gb_dev_grid g, hydro_kparams kp, const int* __restrict__ list, const double* __restrict__ escr,
        size_t estride, double* __restrict__ bscr, size_t bstride)
{
    if (blockIdx.y == 0) faceb_face<0>(g, kp, list, escr, estride, bscr, bstride);
    else if (blockIdx.y == 1) faceb_face<1>(g, kp, list, escr, estride, bscr, bstride);
    else faceb_face<2>(g, kp, list, escr, estride, bscr, bstride);
}

// ---------------------------------------------------------------- edge fields at fine-coarse boundaries
// The CT counterpart of the flux registers. Every leaf stores the electric
// fields of its surface edges; a leaf replaces each of its surface edges
// that a leaf one level finer also carries (across a face, an edge or a
// corner) by the mean of the two fine edges along it. The coarse face-B
// update on a fine-coarse face is then the mean of the four fine ones, and
// every coarse block around such an edge takes the same value. Surface
// edges of direction c: node positions (A, B) on the ring of the 17 x 17
// node grid across c (A along (c + 1) % 3, B along (c + 2) % 3, A or B in
// {0, 16}) times the 16 cells along c; register index (c 16 + C) 64 + ring.
constexpr int NRING = 64;
constexpr int NSURF = 3 * GB_NXB * NRING;

__device__ __forceinline__ int edge_ring(int A, int B)
{
    return B == 0 ? A : (B == GB_NXB ? 17 + A : (A == 0 ? 33 + B : 48 + B));
}

__device__ __forceinline__ void ring_edge(int q, int& A, int& B)
{
    if (q < 17) { A = q; B = 0; }
    else if (q < 34) { A = q - 17; B = GB_NXB; }
    else if (q < 49) { A = 0; B = q - 33; }
    else { A = GB_NXB; B = q - 48; }
}

static __global__ void __launch_bounds__(128)
k_emf_put(const int* __restrict__ list, const int* __restrict__ near, const double* __restrict__ escr, size_t estride,
          double* __restrict__ ereg)
{
    const int cb = blockIdx.y, t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= NSURF) return;
    const int blk = list[cb];
    if (!(__ldg(near + blk) & 1)) return;  // no coarser leaf reads this block's edges
    const int c = t / (GB_NXB * NRING), C = (t / NRING) % GB_NXB;
    int A, B;
    ring_edge(t % NRING, A, B);
    ereg[(size_t)blk * NSURF + t] = escr[(size_t)cb * estride + (size_t)c * NEDGE + A + 17 * (B + 17 * C)];
}

// The surrounding cells of a surface edge outside the block are tried in a
// fixed order ((A-1, B-1), (A, B-1), (A-1, B), (A, B)); the first lying in
// a leaf one level finer (its region's plan node is refined, the child
// holding the cell is a leaf) gives the fine edges (every such leaf carries
// the same values).
template <int CD>
__device__ __forceinline__ void emf_get_dir(const int4* __restrict__ pb, const int* __restrict__ child,
                                            const double* __restrict__ ereg, double* __restrict__ es, int C, int q)
{
    constexpr int a = (CD + 1) % 3, b = (CD + 2) % 3;
    int A, B;
    ring_edge(q, A, B);
#pragma unroll
    for (int cand = 0; cand < 4; ++cand) {
        const int ia = cand & 1, ib = cand >> 1;
        const int ca = A - 1 + ia, cbb = B - 1 + ib;
        const int ra = ca < 0 ? -1 : (ca >= GB_NXB ? 1 : 0), rb = cbb < 0 ? -1 : (cbb >= GB_NXB ? 1 : 0);
        if (ra == 0 && rb == 0) continue;
        const int r = (a == 0 ? ra + 1 : b == 0 ? rb + 1 : 1) + 3 * (a == 1 ? ra + 1 : b == 1 ? rb + 1 : 1) +
                      9 * (a == 2 ? ra + 1 : b == 2 ? rb + 1 : 1);
        const int4 e = __ldg(pb + 2 * r);
        if (e.x < 0 || !(e.z & GP_REFINED)) continue;
        const int la = ca - GB_NXB * ra, lb = cbb - GB_NXB * rb;
        const int ba = la >= GB_NXB / 2, bbit = lb >= GB_NXB / 2, bc = C >= GB_NXB / 2;
        const int q8 = (a == 0 ? ba : b == 0 ? bbit : bc) | ((a == 1 ? ba : b == 1 ? bbit : bc) << 1) |
                       ((a == 2 ? ba : b == 2 ? bbit : bc) << 2);
        const int F = __ldg(child + 8 * e.x + q8);
        if (F < 0) continue;
        if (!(e.z & GP_LEAFKIDS) && __ldg(child + 8 * F) >= 0) continue;
        const int Af = 2 * la + (ia ? 0 : 2) - GB_NXB * ba, Bf = 2 * lb + (ib ? 0 : 2) - GB_NXB * bbit;
        const int Cf = 2 * C - GB_NXB * bc;
        const double* rf = ereg + (size_t)F * NSURF + ((size_t)CD * GB_NXB + Cf) * NRING + edge_ring(Af, Bf);
        es[(size_t)CD * NEDGE + A + 17 * (B + 17 * C)] = 0.5 * (rf[0] + rf[NRING]);
        return;
    }
}

static __global__ void __launch_bounds__(128)
k_emf_get(const int* __restrict__ list, const int4* __restrict__ plan, const int* __restrict__ near,
          const int* __restrict__ child, const double* __restrict__ ereg, double* __restrict__ escr, size_t estride)
{
    const int cb = blockIdx.z, t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= GB_NXB * NRING) return;
    const int blk = list[cb];
    if (!(__ldg(near + blk) & 2)) return;  // no finer leaf around this block
    const int4* pb = plan + (size_t)blk * 54;
    double* es = escr + (size_t)cb * estride;
    const int C = t / NRING, q = t % NRING;
    if (blockIdx.y == 0) emf_get_dir<0>(pb, child, ereg, es, C, q);
    else if (blockIdx.y == 1) emf_get_dir<1>(pb, child, ereg, es, C, q);
    else emf_get_dir<2>(pb, child, ereg, es, C, q);
}

// ---------------------------------------------------------------- flux conservation
// Grid_putFluxData / Grid_conserveFluxes / Grid_getFluxData on a Cartesian
// mesh: a block whose neighbour across face f is coarser stores its
// boundary fluxes; a block whose neighbour is finer replaces its boundary
// fluxes by the mean of the 2 x 2 fine-face fluxes. Blocks are stepped
// finest level first, so the fine registers are written (put, an earlier
// chunk or earlier in this one) before a coarse block reads them (get).
constexpr int NREG = 7;  // rho, mx, my, mz, E, rho e_int, u_n
enum { FACE_SAME = 0, FACE_COARSER = 1, FACE_FINER = 2 };
__device__ __forceinline__ int reg_var(int v) { return v < 5 ? v : v + 3; }  // flux slots 0..4, 8, 9

template <typename T>
__global__ void __launch_bounds__(256)
k_fc_put(const int* __restrict__ list, const int* __restrict__ links, T* __restrict__ reg,
         const T* __restrict__ fscr, size_t fstride)
{
    const int f = blockIdx.y, cb = blockIdx.z, c = threadIdx.x;
    const int blk = list[cb];
    if (links[((size_t)blk * 6 + f) * 5] != FACE_COARSER) return;
    const int d = f >> 1, side = f & 1;
    const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
    int I[3];
    I[d] = side ? LO + GB_NXB : LO;
    I[t1] = LO + c % GB_NXB;
    I[t2] = LO + c / GB_NXB;
    const T* fs = fscr + (size_t)cb * fstride + (size_t)d * NFLX * NFC + flux_index(d, I[0], I[1], I[2]);
    T* r = reg + (((size_t)blk * 6 + f) * (GB_NXB * GB_NXB) + c) * NREG;
#pragma unroll
    for (int v = 0; v < NREG; ++v) r[v] = fs[(size_t)reg_var(v) * NFC];
}

template <typename T>
__global__ void __launch_bounds__(256)
k_fc_get(const int* __restrict__ list, const int* __restrict__ links, const T* __restrict__ reg,
         T* __restrict__ fscr, size_t fstride)
{
    const int f = blockIdx.y, cb = blockIdx.z, c = threadIdx.x;
    const int blk = list[cb];
    const int* lk = links + ((size_t)blk * 6 + f) * 5;
    if (lk[0] != FACE_FINER) return;
    const int d = f >> 1, side = f & 1;
    const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
    constexpr int h = GB_NXB / 2;
    const int c1 = c % GB_NXB, c2 = c / GB_NXB;
    const int q = (c1 >= h) + 2 * (c2 >= h);
    const int m = lk[1 + q];
    if (m < 0) return;
    const int g1 = 2 * (c1 - h * (c1 >= h)), g2 = 2 * (c2 - h * (c2 >= h));
    // the fine leaf's face touching this block is the opposite one (f ^ 1)
    const T* r = reg + ((size_t)m * 6 + (f ^ 1)) * (GB_NXB * GB_NXB) * NREG;
    const T* r00 = r + (size_t)(g1 + GB_NXB * g2) * NREG;
    const T* r10 = r + (size_t)(g1 + 1 + GB_NXB * g2) * NREG;
    const T* r01 = r + (size_t)(g1 + GB_NXB * (g2 + 1)) * NREG;
    const T* r11 = r + (size_t)(g1 + 1 + GB_NXB * (g2 + 1)) * NREG;
    int I[3];
    I[d] = side ? LO + GB_NXB : LO;
    I[t1] = LO + c1;
    I[t2] = LO + c2;
    T* fs = fscr + (size_t)cb * fstride + (size_t)d * NFLX * NFC + flux_index(d, I[0], I[1], I[2]);
#pragma unroll
    for (int v = 0; v < NREG; ++v) fs[(size_t)reg_var(v) * NFC] = (T)0.25 * (((r00[v] + r10[v]) + r01[v]) + r11[v]);
}

// ---------------------------------------------------------------- k_update
// Error-free transformation of an FP32 sum (Knuth's TwoSum): s + e == a + b
// exactly, s the rounded sum (needs round-to-nearest adds, no reassociation).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// (ap - am) + (bp - bm) + (cp - cm) of six FP32 fluxes as a double: the
// cascaded TwoSum of Ogita, Rump and Oishi (SIAM J. Sci. Comput. 26, 2005,
// "Sum2"), accurate as if summed in twice FP32's precision (relative error
// about 2^-48 of the sum of magnitudes), then one FP64 addition. It
// replaces three FP64 subtractions and two FP64 additions.
__device__ __forceinline__ double flux_div(float ap, float am, float bp, float bm, float cp, float cm)
{
    float s0, e0, s1, e1, s2, e2, t, e3, S, e4;
    two_sum(ap, -am, s0, e0);
    two_sum(bp, -bm, s1, e1);
    two_sum(cp, -cm, s2, e2);
    two_sum(s0, s1, t, e3);
    two_sum(t, s2, S, e4);
    const float E = (((e0 + e1) + e2) + e3) + e4;
    return gb_f2d(S) + gb_f2d(E);
}

// 1 / x in FP64 from an FP32 seed and two Newton-Raphson steps
// (y <- y + y (1 - x y); each step doubles the correct bits: about 2^-22,
// 2^-44, 2^-88), for x inside FP32's normal range; an FP64 division
// otherwise.
__device__ __forceinline__ double rcp_newton(double x)
{
    const float xf = gb_d2f(x);
    if (!(fabsf(xf) > 1e-30f && fabsf(xf) < 1e30f)) return 1.0 / x;
    double y = gb_f2d(1.0f / xf);
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

// FEAT: also write the learned-cooling surrogate's features of the new
// state (what the feature kernel would compute next): FP32 work beside this
// FP64-bound kernel instead of a kernel of its own
// mixed path without the fused plain cooling: eight resident CTAs per SM
// (64 registers, no spills); the FP64 path and the FP64-rate integrator need
// more registers (the FP32-rate integrator runs in k_cool_pass)
template <typename T, bool MHD, int COOL, bool FEAT>
__global__ void __launch_bounds__(128, (std::is_same<T, float>::value && !COOL) ? 8 : 1)
k_update(gb_dev_grid g, hydro_kparams kp, gb_cool_ctx cool, const int* __restrict__ list,
         const T* __restrict__ fscr, size_t fstride, const double* __restrict__ bscr, size_t bstride,
         gb_status* st, sur_feat_out sf)
{
    const int cb = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= GB_NXB * GB_NXB * GB_NXB) return;
    const int blk = list[cb];
    const int i = LO + t % GB_NXB, j = LO + (t / GB_NXB) % GB_NXB, k = LO + t / (GB_NXB * GB_NXB);
    const int ci = gb_cidx(i, j, k);
    double* base = g.unk + (int64_t)blk * g.nvar * GB_N3;
    auto UV = [&](int role) -> double& { return base[(int64_t)g.slot[role] * GB_N3 + ci]; };
    const double gm1 = kp.gamma - 1.0;
    double rho = UV(GB_DENS), vx = UV(GB_VELX), vy = UV(GB_VELY), vz = UV(GB_VELZ), pr = UV(GB_PRES);
    double Bc[3] = {0.0, 0.0, 0.0};
    if (MHD) { Bc[0] = UV(GB_MAGX); Bc[1] = UV(GB_MAGY); Bc[2] = UV(GB_MAGZ); }
    // the mixed path replaces the divisions of the conversions by one
    // reciprocal of the density (FP64 divisions are long instruction
    // sequences on the FP64 pipe); the FP64 path keeps the oracle's operations
    constexpr bool RCP = std::is_same<T, float>::value;
    double Uc[NP];
    Uc[0] = rho;
    Uc[1] = rho * vx; Uc[2] = rho * vy; Uc[3] = rho * vz;
    Uc[4] = (RCP ? pr * kp.inv_gm1 : pr / gm1) + 0.5 * rho * (vx * vx + vy * vy + vz * vz) +
            0.5 * (Bc[0] * Bc[0] + Bc[1] * Bc[1] + Bc[2] * Bc[2]);
    Uc[5] = Bc[0]; Uc[6] = Bc[1]; Uc[7] = Bc[2];
    double re = rho * UV(GB_EINT);
    const T* fs = fscr + (size_t)cb * fstride;
    const int fm[3] = {flux_index(0, i, j, k), flux_index(1, i, j, k), flux_index(2, i, j, k)};
    const int fp[3] = {flux_index(0, i + 1, j, k), flux_index(1, i, j + 1, k), flux_index(2, i, j, k + 1)};
    double dtd[3];
    kp_dtdx(kp, gb_block_level(g, blk), dtd);
    auto F = [&](int d, int var, int idx) -> double {
        const T x = fs[(size_t)d * NFLX * NFC + (size_t)var * NFC + idx];
        if constexpr (std::is_same<T, float>::value) return gb_f2d(x);  // exact, on the integer pipe
        else return x;
    };
    double Un[5], dtdivv, ren;
    if (RCP && kp.iso) {
        // cubic cells: one FP64 scaling of the summed flux differences
        auto Ff = [&](int d, int var, int idx) -> float {
            return (float)fs[(size_t)d * NFLX * NFC + (size_t)var * NFC + idx];
        };
        auto div = [&](int var) {
            return flux_div(Ff(0, var, fp[0]), Ff(0, var, fm[0]), Ff(1, var, fp[1]), Ff(1, var, fm[1]),
                            Ff(2, var, fp[2]), Ff(2, var, fm[2]));
        };
#pragma unroll
        for (int s = 0; s < 5; ++s) Un[s] = fma(-dtd[0], div(s), Uc[s]);
        dtdivv = dtd[0] * div(9);
        ren = fma(-dtd[0], div(8), re) - pr * dtdivv;
    } else {
#pragma unroll
        for (int s = 0; s < 5; ++s)
            Un[s] = Uc[s] - dtd[0] * (F(0, s, fp[0]) - F(0, s, fm[0])) - dtd[1] * (F(1, s, fp[1]) - F(1, s, fm[1])) -
                    dtd[2] * (F(2, s, fp[2]) - F(2, s, fm[2]));
        // dt * div v from the face velocities, as sum_d (dt/dx_d) dv_d
        dtdivv = dtd[0] * (F(0, 9, fp[0]) - F(0, 9, fm[0])) + dtd[1] * (F(1, 9, fp[1]) - F(1, 9, fm[1])) +
                 dtd[2] * (F(2, 9, fp[2]) - F(2, 9, fm[2]));
        ren = re - dtd[0] * (F(0, 8, fp[0]) - F(0, 8, fm[0])) - dtd[1] * (F(1, 8, fp[1]) - F(1, 8, fm[1])) -
              dtd[2] * (F(2, 8, fp[2]) - F(2, 8, fm[2])) - pr * dtdivv;
    }
    double Bn[3] = {0.0, 0.0, 0.0};
    if (MHD) {
        const double* bs = bscr + (size_t)cb * bstride;
        double blo[3] = {bs[0 * NFB + fb_index(0, i, j, k)], bs[1 * NFB + fb_index(1, i, j, k)],
                         bs[2 * NFB + fb_index(2, i, j, k)]};
        double bhi[3] = {bs[0 * NFB + fb_index(0, i + 1, j, k)], bs[1 * NFB + fb_index(1, i, j + 1, k)],
                         bs[2 * NFB + fb_index(2, i, j, k + 1)]};
#pragma unroll
        for (int d = 0; d < 3; ++d) Bn[d] = 0.5 * (blo[d] + bhi[d]);
        // write back the interior faces: low faces by every cell, high
        // faces by the cells on the upper boundary
        g.f[0][(int64_t)blk * GB_FSZ + gb_fidx(0, i, j, k)] = blo[0];
        g.f[1][(int64_t)blk * GB_FSZ + gb_fidx(1, i, j, k)] = blo[1];
        g.f[2][(int64_t)blk * GB_FSZ + gb_fidx(2, i, j, k)] = blo[2];
        if (i == HI) g.f[0][(int64_t)blk * GB_FSZ + gb_fidx(0, i + 1, j, k)] = bhi[0];
        if (j == HI) g.f[1][(int64_t)blk * GB_FSZ + gb_fidx(1, i, j + 1, k)] = bhi[1];
        if (k == HI) g.f[2][(int64_t)blk * GB_FSZ + gb_fidx(2, i, j, k + 1)] = bhi[2];
    }
    double rn = fmax(Un[0], kp.smlrho);
    const double irn = RCP ? rcp_newton(rn) : 0.0;
    auto over_rn = [&](double x) { return RCP ? x * irn : x / rn; };
    double ek = over_rn(0.5 * (Un[1] * Un[1] + Un[2] * Un[2] + Un[3] * Un[3]));
    double em = 0.5 * (Bn[0] * Bn[0] + Bn[1] * Bn[1] + Bn[2] * Bn[2]);
    if (MHD && kp.energy_fix) {
        // energyFix (Balsara & Spicer 1999): the gas energy is the updated
        // total energy less the magnetic energy of the cell field advanced by
        // the same fluxes (component c by the two directions across it; the
        // normal direction's flux of B_c is zero); the stored field and the
        // total energy built from it next step use the staggered faces' mean
        double Bf[3];
        if constexpr (std::is_same<T, float>::value) {
            // the field's change in FP32 (its relative error reaches em only
            // through the change), the field itself in FP64
            float dtf[3];
            kp_dtdxf(kp, gb_block_level(g, blk), dtf);
            auto Fq = [&](int d, int var, int idx) -> float {
                return (float)fs[(size_t)d * NFLX * NFC + (size_t)var * NFC + idx];
            };
            const float d0 = -(dtf[1] * (Fq(1, 5, fp[1]) - Fq(1, 5, fm[1]))) - dtf[2] * (Fq(2, 5, fp[2]) - Fq(2, 5, fm[2]));
            const float d1 = -(dtf[0] * (Fq(0, 6, fp[0]) - Fq(0, 6, fm[0]))) - dtf[2] * (Fq(2, 6, fp[2]) - Fq(2, 6, fm[2]));
            const float d2 = -(dtf[0] * (Fq(0, 7, fp[0]) - Fq(0, 7, fm[0]))) - dtf[1] * (Fq(1, 7, fp[1]) - Fq(1, 7, fm[1]));
            Bf[0] = Uc[5] + gb_f2d(d0);
            Bf[1] = Uc[6] + gb_f2d(d1);
            Bf[2] = Uc[7] + gb_f2d(d2);
        } else {
            Bf[0] = (Uc[5] - dtd[1] * (F(1, 5, fp[1]) - F(1, 5, fm[1]))) - dtd[2] * (F(2, 5, fp[2]) - F(2, 5, fm[2]));
            Bf[1] = (Uc[6] - dtd[0] * (F(0, 6, fp[0]) - F(0, 6, fm[0]))) - dtd[2] * (F(2, 6, fp[2]) - F(2, 6, fm[2]));
            Bf[2] = (Uc[7] - dtd[0] * (F(0, 7, fp[0]) - F(0, 7, fm[0]))) - dtd[1] * (F(1, 7, fp[1]) - F(1, 7, fm[1]));
        }
        em = 0.5 * (Bf[0] * Bf[0] + Bf[1] * Bf[1] + Bf[2] * Bf[2]);
    }
    const double xE = (Un[4] - ek) - em;  // rho e from the total energy
    double eiE = over_rn(xE);
    double eia = over_rn(ren);
    // the mixed path compares and forms the pressure before the division by
    // rho (the same quantities with two FP64 operations fewer); the FP64 path
    // keeps the oracle's operations
    bool use_E = RCP ? xE > kp.eint_switch * Un[4] : eiE > kp.eint_switch * over_rn(Un[4]);
    double ei = use_E ? eiE : eia;
    double pn = RCP ? gm1 * (use_E ? xE : ren) : gm1 * rn * ei;
    bool floored = false;
    if (pn < kp.smallp) {
        pn = kp.smallp;
        ei = pn / (gm1 * rn);
        floored = true;
    }
    double vxn = over_rn(Un[1]), vyn = over_rn(Un[2]), vzn = over_rn(Un[3]);
    // specific kinetic energy: ek / rho in the mixed path (one FP64 product
    // instead of four)
    double ekin_s = RCP ? ek * irn : 0.5 * (vxn * vxn + vyn * vyn + vzn * vzn);
    if (COOL) {
        // fused heating/cooling epilogue (RadHeat.F90:223-423 on the new state)
        const gb_cool_params& p = cool.p;
        gb_cool_vars v;
        v.rho = rn * p.dens_unit;
        double eic = ei * (p.vel_unit * p.vel_unit);
        double temp = eic * (gm1 * p.eos_abar * p.mp / p.boltz);
        v.tdust = UV(GB_TDUS);
        v.xHp = g.slot[GB_IHP] >= 0 ? UV(GB_IHP) : p.xHp_const;
        v.ephen = g.slot[GB_PHHE] >= 0 ? UV(GB_PHHE) / v.rho : 0.0;
        v.Gflux = g.slot[GB_PEFL] >= 0 ? UV(GB_PEFL) : 0.0;
        v.mu_mol = p.mu_mol;
        v.strat_factor = 1.0;
        gb_cool_diag dg = {0, 0, 0, 0, 0};
        // the input guard of gb_heat: a non-finite or non-positive state is
        // reported and keeps its hydro values (the root finder would spend
        // its whole iteration budget on it)
        const bool good = gb_finite_pos(v.rho) && gb_finite_pos(eic) && gb_finite_pos(temp);
        bool clamped = false;
        if (good) {
            // the mixed path evaluates the rates with shared transcendentals
            // (one ln T and one sqrt T per evaluation); the FP64 path keeps
            // the reference's formulation
            gbcool::heating_and_cooling<RCP ? COOL : 0>(cool, v, &eic, kp_dt(kp) * p.time_unit, &temp, &dg);
            if (temp > p.absTmax) {
                eic = p.absTmax * v.TtoEI;
                temp = p.absTmax;
                clamped = true;
            }
            if (eic < p.smallp / v.rho) eic = p.smallp / v.rho;
            ei = eic / (p.vel_unit * p.vel_unit);
            pn = gm1 * rn * ei;
            UV(GB_TEMP) = temp;
            UV(GB_TDUS) = v.tdust;
            if (g.slot[GB_PHHE] >= 0) UV(GB_PHHE) = 0.0;
            if (g.slot[GB_PEFL] >= 0) UV(GB_PEFL) = 0.0;
        }
        if (st) {
            if (!good) gb_fail(st, GB_ST_NONFINITE, blk, i, j, k, temp);
            gb_count_warp(&st->n_bracket_fail, dg.bracket_fail != 0);
            gb_count_warp(&st->n_clamped, clamped);
            if (clamped) gb_fail(st, GB_ST_OVERHEAT, blk, i, j, k, temp);
            if (dg.unbracketed) gb_fail(st, GB_ST_ZERO_UNBRACKETED, blk, i, j, k, eic);
            if (dg.maxiter) gb_fail(st, GB_ST_ZERO_MAXITER, blk, i, j, k, eic);
        }
    }
    UV(GB_DENS) = rn;
    UV(GB_VELX) = vxn;
    UV(GB_VELY) = vyn;
    UV(GB_VELZ) = vzn;
    UV(GB_PRES) = pn;
    UV(GB_EINT) = ei;
    UV(GB_ENER) = ei + ekin_s;
    if (MHD) { UV(GB_MAGX) = Bn[0]; UV(GB_MAGY) = Bn[1]; UV(GB_MAGZ) = Bn[2]; }
    if (st) {
        gb_count_warp(&st->n_eint_switch, !use_E);
        if (!(Un[0] > 0.0)) gb_fail(st, GB_ST_NEG_DENS, blk, i, j, k, Un[0]);
        else if (!isfinite(pn) || !isfinite(Un[4])) gb_fail(st, GB_ST_NONFINITE, blk, i, j, k, pn);
        else if (floored) gb_fail(st, GB_ST_NEG_PRES, blk, i, j, k, eiE);
    }
    if constexpr (FEAT) {
        // the inputs are read back as stored (this thread wrote them)
        gb_cool_varsf vf;
        double eid;
        float eif, tempf;
        sur_load_f32(g, sf.pf, sf.un, blk, ci, vf, eid, eif, tempf);
        float4 x;
        float2 f0fl;
        sur_features(cool, sf.pf, sf.un, vf, eif, tempf, kp_dt(kp), x, f0fl);
        const int64_t idx = (int64_t)cb * (GB_NXB * GB_NXB * GB_NXB) + t;
        sf.feat[idx] = x;
        sf.f0[idx] = f0fl;
    }
}

// The plain integrator on FP32 rates (the mixed path's cooling mode 2) as a
// pass of its own over a chunk's interior cells, after the update without
// it: the inputs of the fused epilogue of k_update (the new density and
// internal energy, the stored dust temperature and source terms) and its
// stores; the specific kinetic energy of the total energy comes from the
// stored velocities. Its own kernel keeps the integrator's long code apart
// from the update's. Five resident CTAs per SM (90 registers, no spills):
// 22.29 ms per 4101-leaf step against 22.53 at four and 22.58 at six
static __global__ void __launch_bounds__(128, 5)
k_cool_pass(gb_dev_grid g, hydro_kparams kp, gb_cool_ctx cool, const int* __restrict__ list, gb_status* st)
{
    const int cb = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= GB_NXB * GB_NXB * GB_NXB) return;
    const int blk = list[cb];
    const int i = LO + t % GB_NXB, j = LO + (t / GB_NXB) % GB_NXB, k = LO + t / (GB_NXB * GB_NXB);
    const int ci = gb_cidx(i, j, k);
    double* base = g.unk + (int64_t)blk * g.nvar * GB_N3;
    auto UV = [&](int role) -> double& { return base[(int64_t)g.slot[role] * GB_N3 + ci]; };
    const double gm1 = kp.gamma - 1.0;
    const double rn = UV(GB_DENS);
    const gb_cool_params& p = cool.p;
    gb_cool_vars v;
    v.rho = rn * p.dens_unit;
    double eic = UV(GB_EINT) * (p.vel_unit * p.vel_unit);
    double temp = eic * (gm1 * p.eos_abar * p.mp / p.boltz);
    v.tdust = UV(GB_TDUS);
    v.xHp = g.slot[GB_IHP] >= 0 ? UV(GB_IHP) : p.xHp_const;
    v.ephen = g.slot[GB_PHHE] >= 0 ? UV(GB_PHHE) / v.rho : 0.0;
    v.Gflux = g.slot[GB_PEFL] >= 0 ? UV(GB_PEFL) : 0.0;
    v.mu_mol = p.mu_mol;
    v.strat_factor = 1.0;
    gb_cool_diag dg = {0, 0, 0, 0, 0};
    const bool good = gb_finite_pos(v.rho) && gb_finite_pos(eic) && gb_finite_pos(temp);
    bool clamped = false;
    if (good) {
        gbcool::heating_and_cooling<2>(cool, v, &eic, kp_dt(kp) * p.time_unit, &temp, &dg);
        if (temp > p.absTmax) {
            eic = p.absTmax * v.TtoEI;
            temp = p.absTmax;
            clamped = true;
        }
        if (eic < p.smallp / v.rho) eic = p.smallp / v.rho;
        const double ei = eic / (p.vel_unit * p.vel_unit);
        const double vx = UV(GB_VELX), vy = UV(GB_VELY), vz = UV(GB_VELZ);
        UV(GB_TEMP) = temp;
        UV(GB_TDUS) = v.tdust;
        if (g.slot[GB_PHHE] >= 0) UV(GB_PHHE) = 0.0;
        if (g.slot[GB_PEFL] >= 0) UV(GB_PEFL) = 0.0;
        UV(GB_PRES) = gm1 * rn * ei;
        UV(GB_EINT) = ei;
        UV(GB_ENER) = ei + 0.5 * (vx * vx + vy * vy + vz * vz);
    }
    if (st) {
        if (!good) gb_fail(st, GB_ST_NONFINITE, blk, i, j, k, temp);
        gb_count_warp(&st->n_bracket_fail, dg.bracket_fail != 0);
        gb_count_warp(&st->n_clamped, clamped);
        if (clamped) gb_fail(st, GB_ST_OVERHEAT, blk, i, j, k, temp);
        if (dg.unbracketed) gb_fail(st, GB_ST_ZERO_UNBRACKETED, blk, i, j, k, eic);
        if (dg.maxiter) gb_fail(st, GB_ST_ZERO_MAXITER, blk, i, j, k, eic);
    }
}

// ---------------------------------------------------------------- CFL
// R = double: the oracle's arithmetic; R = float (mixed path): the same
// limit from FP32 arithmetic on the FP64 state (dt to ~1e-7 relative)
// Per cell the limit is min_d dx_d / (|v_d| + c_f,d), or with cfl_sum
// 1 / sum_d (|v_d| + c_f,d) / dx_d; a cell whose reconstruction fell back
// last step (its CFL code, the OR over the three directions) has it scaled
// by sc[code] (the lowered CFL over cfl).

template <typename R>
static __global__ void __launch_bounds__(256)
k_dtlimit(gb_dev_grid g, double gamma, int mhd, double dx0, double dx1, double dx2,
          const int* __restrict__ list, unsigned long long* __restrict__ out_bits, int cfl_sum,
          const unsigned char* __restrict__ cflc, cfl_scale sc)
{
    const int blk = list[blockIdx.y];
    const double root[3] = {dx0, dx1, dx2};
    double deld[3];
    gb_block_dx(g, root, blk, deld);
    const R del[3] = {(R)deld[0], (R)deld[1], (R)deld[2]};
    R best = (R)1e30;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < GB_NXB * GB_NXB * GB_NXB; t += gridDim.x * blockDim.x) {
        const int i = LO + t % GB_NXB, j = LO + (t / GB_NXB) % GB_NXB, k = LO + t / (GB_NXB * GB_NXB);
        const int ci = gb_cidx(i, j, k);
        const double* base = g.unk + (int64_t)blk * g.nvar * GB_N3 + ci;
        auto ld = [&](int role) -> R {
            const double x = base[(int64_t)g.slot[role] * GB_N3];
            if constexpr (std::is_same<R, float>::value) return gb_d2f(x);
            else return x;
        };
        R rho = ld(GB_DENS), p = ld(GB_PRES);
        R B[3] = {0, 0, 0};
        if (mhd) {
            B[0] = ld(GB_MAGX);
            B[1] = ld(GB_MAGY);
            B[2] = ld(GB_MAGZ);
        }
        R gp = (R)gamma * p;
        R B2 = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
        R tt = (gp + B2) / rho;
        R rate = (R)0, cell = (R)1e30;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            R v = fabs(ld(GB_VELX + d));
            R cf = sqrt((R)0.5 * (tt + sqrt(fmax(tt * tt - (R)4 * gp * B[d] * B[d] / (rho * rho), (R)0))));
            if (cfl_sum) {
                rate = rate + (v + cf) / del[d];
            } else {
                R dtc = del[d] / (v + cf);
                cell = fmin(cell, dtc);
            }
        }
        if (cfl_sum) cell = (R)1 / rate;
        if (cflc) {
            const unsigned char* cc = cflc + (size_t)blk * 3 * (GB_NXB * GB_NXB * GB_NXB) + t;
            const int code = cc[0] | cc[GB_NXB * GB_NXB * GB_NXB] | cc[2 * GB_NXB * GB_NXB * GB_NXB];
            if (code) cell = cell * (R)(code == 1 ? sc.s[1] : (code == 2 ? sc.s[2] : sc.s[3]));
        }
        best = fmin(best, cell);
    }
    // warp shuffle then block reduction of the minimum
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
    __shared__ R s_min[8];
    if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x < 32) {
        best = threadIdx.x < (blockDim.x >> 5) ? s_min[threadIdx.x] : (R)1e30;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
        // positive doubles order like their bit patterns
        if (threadIdx.x == 0) atomicMin(out_bits, (unsigned long long)__double_as_longlong((double)best));
    }
}

}  // namespace gbh
