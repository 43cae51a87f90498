/*
 * CPU oracle for the unsplit hydro / staggered-mesh MHD block update.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * FLASH 4.6.2's unsplit solver body is not in the reference tree; only the
 * per-cell reconstruction driver hy_uhd_dataReconstOneStep.F90 and the
 * interfaces in hy_uhd_interface.F90 are. This restatement follows that
 * driver's control flow (normal-direction PPM per dimension, transverse
 * corrections, multidimensional MHD terms, positivity fallback) and writes
 * the absent pieces from the published methods the reference cites:
 * Colella & Woodward 1984 (PPM), Stone et al. 2008 (characteristic tracing),
 * Toro 1997 / Batten et al. 1997 (HLLC), Miyoshi & Kusano 2005 (HLLD),
 * Gardiner & Stone 2005 (upwinded CT electric fields), Bryan et al. 1995
 * (dual energy). Parity against FLASH itself is unpinned.
 *
 * Block storage: NV cell variables, each a contiguous nxg*nyg*nzg array
 * (x fastest), guard cells included; face-centred B as three arrays of
 * (nxg+1)*nyg*nzg, nxg*(nyg+1)*nzg, nxg*nyg*(nzg+1).
 */
#ifndef GB_HYDRO_ORACLE_H
#define GB_HYDRO_ORACLE_H

#include <stdint.h>

/* cell-variable slots in the oracle's block layout */
enum {
    ORV_DENS = 0, ORV_VELX, ORV_VELY, ORV_VELZ, ORV_PRES, ORV_ENER, ORV_EINT,
    ORV_MAGX, ORV_MAGY, ORV_MAGZ, ORV_NVAR
};

typedef struct orc_hydro_params {
    double gamma;
    double cvisc;      /* use_avisc/cvisc, flash.par.turbsph_standard:197-198 */
    int use_avisc;
    double eint_switch;/* eintSwitch, :164 */
    double smlrho, smallp;
    int mhd;           /* 0: hydro (HLLC), 1: USM MHD (HLLD + CT) */
    int nxb, nguard;   /* 16, 4 */
    int energy_fix;    /* energyFix, :213: gas energy from the flux-updated cell field */
    int cfl_sum;       /* CFL limit 1 / sum_d (|v_d| + c_f,d) / dx_d instead of min_d */
    int hybrid_order;  /* use_hybridOrder, :206 */
    int fallback_lower_cfl; /* hy_fallbackLowerCFL, :207 */
    double hybrid_kappa;    /* hy_hybridOrderKappa (FLASH default 0) */
    double cfl_fallback_factor; /* hy_cflFallbackFactor, :208 */
    double cfl;        /* cfl, :163 (the lowered CFL of a cell is a ratio to it) */
    /* per-cell CFL codes (NULL: not kept): ORC_CFLC bytes per store block,
     * interior cells x fastest; written by the step, read by the CFL limit
     * of the next one. Bit 0: the fallback factor / 3 (first-order states
     * from the positivity check, or from the first Rankine-Hugoniot check
     * with fallback_lower_cfl); bit 1: 0.25 (second check). */
    unsigned char* cflc;
    /* edge electric fields: 0 = Gardiner & Stone (2005) eq. 41/50, the
     * arithmetic mean of the four face fields plus contact-upwinded
     * derivative terms (the scheme the GPU runs); 1 = the arithmetic mean
     * alone (Balsara & Spicer 1999), a comparison point only */
    int emf_average;
} orc_hydro_params;

#define ORC_CFLC 4096
/* CFL limit scale of a cell code (a ratio to p->cfl, at most 1) */
double orc_cfl_scale(const orc_hydro_params* p, int code);

void orc_hydro_default_params(orc_hydro_params* p, int mhd);

/* One unsplit step of one block. `u` holds the ORV_NVAR variables (those
 * beyond ORV_EINT only when mhd) with guard cells filled; bx/by/bz the face
 * fields (mhd only). Interior cells and interior faces are overwritten in
 * place with the state at t+dt. Returns the number of cells whose
 * reconstructed state fell back to first order. */
int orc_unsplit_block(const orc_hydro_params* p, double* u, double* bx, double* by, double* bz,
                      double dt, double dx, double dy, double dz);

/* Flux conservation at fine-coarse faces. Faces f = 2 d + side (side 0 =
 * low). A face whose neighbour is coarser stores the block's boundary
 * fluxes (rho, mx, my, mz, E, rho e_int, u_n: ORC_NREG values per face
 * cell, 16 x 16 face cells, first transverse axis fastest) into store[f];
 * a face whose neighbour is finer replaces its boundary fluxes by the mean
 * of the 2 x 2 fine-face fluxes held in fine[f][q] (q = quadrant: bit 0 the
 * upper half along the first transverse axis, bit 1 along the second). */
#define ORC_NREG 7
enum { ORC_FACE_SAME = 0, ORC_FACE_COARSER = 1, ORC_FACE_FINER = 2 };
typedef struct orc_fluxfix {
    int type[6];
    double* store[6];
    const double* fine[6][4];
    /* Edge electric fields at fine-coarse boundaries (MHD; ereg NULL: off).
     * ereg holds ORC_NSURF surface-edge fields per tree node; block b
     * stores its own and replaces each surface edge that a leaf one level
     * finer also carries (across a face, an edge or a corner) by the mean
     * of the two fine edges along it. The tree locates those leaves. */
    double* ereg;
    int b, nnodes;
    const int *level, *coord, *child, *root;
    int nr[3], maxlevel;
} orc_fluxfix;

/* Surface edges of a 16^3 block: per edge direction c, the 64 node
 * positions (A, B) on the ring of the 17 x 17 node grid across c (A along
 * (c + 1) % 3, B along (c + 2) % 3, A or B in {0, 16}; ring index A for
 * B = 0, 17 + A for B = 16, 33 + B for A = 0, 48 + B for A = 16) times the
 * 16 cells along c: index (c * 16 + C) * 64 + ring. */
#define ORC_NRING 64
#define ORC_NSURF (3 * 16 * ORC_NRING)

int orc_unsplit_block_fc(const orc_hydro_params* p, double* u, double* bx, double* by, double* bz,
                         double dt, double dx, double dy, double dz, const orc_fluxfix* fx);

/* Face neighbours of leaf b of a block tree: type[f] (ORC_FACE_*) and, for
 * finer neighbours, the four fine leaves (quadrant order as above). */
void orc_face_links(int b, const int* level, const int* coord, const int* child, const int* root, int nr0,
                    int nr1, int nr2, int maxlevel, int* type, int* fine);

/* One step of the listed leaves of a block tree with flux conservation at
 * fine-coarse faces (flux_correct): leaves are stepped finest level first,
 * each level OpenMP-parallel (omp_driver.c). */
long orc_unsplit_tree(const orc_hydro_params* p, int nlist, const int* list, const int* level, const int* coord,
                      const int* child, const int* root, int nr0, int nr1, int nr2, int maxlevel, double* u,
                      double* bx, double* by, double* bz, double dt, double root_dx, int flux_correct);

/* CFL limit over the interior cells of one block:
 * min_d dx_d / (|v_d| + c_f,d). */
double orc_block_dt_limit(const orc_hydro_params* p, const double* u, double dx, double dy,
                          double dz);

/* Periodic guard-cell fill for a uniform grid of nbx*nby*nbz blocks stored
 * consecutively (block id = bx + nbx*(by + nby*bz)). Fills all NV cell
 * variables and, when mhd, the three face arrays (guard faces and the
 * shared boundary face taken from the lower-index owner). */
void orc_fill_guards_periodic(const orc_hydro_params* p, int nbx, int nby, int nbz, double* u,
                              double* bx, double* by, double* bz);

/* Guard cells and faces of every leaf of a block tree (gb_tree_desc
 * arrays; node id = store block id): copy from a same-level neighbour,
 * injection from a coarser one, 8-cell (face: 4-face) mean from a finer
 * one, mean of two coarse faces for a fine face inside a coarse cell. */
void orc_fill_guards_tree(const orc_hydro_params* p, int nnodes, const int* level, const int* coord,
                          const int* child, const int* root, int nr0, int nr1, int nr2, int maxlevel,
                          double* u, double* bx, double* by, double* bz);

/* The same fill for one leaf b (reads only interior cells and owned faces
 * of other leaves, so leaves can be filled concurrently). */
void orc_fill_guards_leaf(const orc_hydro_params* p, int b, const int* level, const int* coord,
                          const int* child, const int* root, int nr0, int nr1, int nr2, int maxlevel,
                          double* u, double* bx, double* by, double* bz);

/* OpenMP drivers over a list of leaves of a block tree (omp_driver.c): guard
 * fill, CFL limit and one unsplit step with cell size root_dx / 2^level. */
void orc_fill_guards_list(const orc_hydro_params* p, int nlist, const int* list, const int* level,
                          const int* coord, const int* child, const int* root, int nr0, int nr1, int nr2,
                          int maxlevel, double* u, double* bx, double* by, double* bz);
double orc_dt_limit_list(const orc_hydro_params* p, int nlist, const int* list, const int* level,
                         const double* u, double root_dx);
long orc_unsplit_list(const orc_hydro_params* p, int nlist, const int* list, const int* level, double* u,
                      double* bx, double* by, double* bz, double dt, double root_dx);

/* Total mass, momentum, energy (E incl. magnetic) and max |div B| over the
 * interior of a uniform grid. out[0..4] = M, Px, Py, Pz, E; out[5] = max
 * |divB| * dx / max|B|. */
void orc_conserved_totals(const orc_hydro_params* p, int nblocks, const double* u,
                          const double* bx, const double* by, const double* bz, double dx,
                          double dy, double dz, double* out);

#endif
