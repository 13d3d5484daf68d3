/*
 * openmmpol_gb300.h -- C ABI of the GB300 induced-point-dipole library
 * (libommp_gb300.so).
 *
 * The first block repeats, with the same names, types and meaning, the subset
 * of OpenMMPol's C interface that drives the polarization path; each entry
 * cites the declaration it replaces in the reference's include/openmmpol.h
 * and the Fortran binding behind it in src/mod_c_interface.F90.  A host that
 * only uses these symbols links against this library instead of the
 * reference's and gets the same results (the direct O(N^2) sums, solved on
 * the GPU).  As in the reference, these calls print a message and terminate
 * the process (exit status 1) on any error.
 *
 * The second block (ommp_gpu_*) adds what the reference does not have:
 * status-returning variants, solver tolerance and iteration controls, the
 * FP32-inner / FP64-refinement precision mode, convergence history, kernel
 * timing, and direct access to the E_M2D field and the T matrix-vector
 * product for verification.
 *
 * Layout conventions (identical to the reference's Fortran arrays seen from C):
 *   coordinates   double [mm_atoms][3], atomic units (bohr)
 *   fields        double [pol_atoms][3], atomic units
 *   dipoles       double [n_ipd][pol_atoms][3]; set 0 = direct (D), set 1 =
 *                 polarization (P) for AMOEBA (include/f_cart_components.h)
 * Pointers returned by getters point into library memory and stay valid until
 * ommp_terminate(); input arrays are only read during the call.
 */
#ifndef OPENMMPOL_GB300_H
#define OPENMMPOL_GB300_H

#include <stdbool.h>
#include <stdint.h>

#ifndef _OPENMMPOL_CONST
/* values of config/openmmpol_const.h.in */
#define OMMP_VERBOSE_DEBUG 3
#define OMMP_VERBOSE_HIGH 2
#define OMMP_VERBOSE_LOW 1
#define OMMP_VERBOSE_NONE 0
#define OMMP_VERBOSE_DEFAULT OMMP_VERBOSE_LOW
#define OMMP_SOLVER_NONE 0
#define OMMP_SOLVER_CG 1
#define OMMP_SOLVER_DIIS 2
#define OMMP_SOLVER_INVERSION 3
#define OMMP_SOLVER_DEFAULT OMMP_SOLVER_CG
#define OMMP_MATV_NONE 0
#define OMMP_MATV_INCORE 1
#define OMMP_MATV_DIRECT 2
#define OMMP_MATV_DEFAULT OMMP_MATV_DIRECT
#define OMMP_AMOEBA_D 1
#define OMMP_AMOEBA_P 2
#define OMMP_STR_CHAR_MAX 4096
#endif

/* precision modes of ommp_gpu_set_precision */
#define OMMP_GPU_PREC_FP64 0  /* plain FP64 solver (default) */
#define OMMP_GPU_PREC_MIXED 1 /* FP32 inner CG + FP64 iterative refinement */
#define OMMP_GPU_PREC_MIXED_DS 2 /* as MIXED, refinement residual products in  \
                                    double-single arithmetic (~1e-13 relative) */

/* status codes of the ommp_gpu_* calls */
#define OMMP_GPU_OK 0
#define OMMP_GPU_ERR_INPUT 1
#define OMMP_GPU_ERR_NOT_CONVERGED 2
#define OMMP_GPU_ERR_BAD_ARG 3
#define OMMP_GPU_ERR_NUMERIC 4
#define OMMP_GPU_ERR_CUDA 5
#define OMMP_GPU_ERR_MEMORY 6
#define OMMP_GPU_ERR_CANCELLED 7

typedef void *OMMP_SYSTEM_PRT;
typedef void *OMMP_QM_HELPER_PRT;

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference-compatible subset ------------------------------------- */

/* include/openmmpol.h:17 ; src/mod_c_interface.F90:216-231 */
OMMP_SYSTEM_PRT ommp_init_mmp(const char *filename);
/* include/openmmpol.h:19 ; src/mod_c_interface.F90:59-69 */
void ommp_set_default_solver(OMMP_SYSTEM_PRT s, int32_t solver);
/* include/openmmpol.h:20 ; src/mod_c_interface.F90:71-81 */
void ommp_set_default_matv(OMMP_SYSTEM_PRT s, int32_t matv);
/* include/openmmpol.h:24 ; src/mod_c_interface.F90:274-282 */
void ommp_terminate(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:28 */
void ommp_set_verbose(int32_t level);
/* include/openmmpol.h:29 */
void ommp_set_outputfile(const char *path);
/* include/openmmpol.h:30 */
void ommp_close_outputfile(void);
/* include/openmmpol.h:31 */
void ommp_message(const char *msg, int32_t level, const char *tag);
/* include/openmmpol.h:32 */
void ommp_fatal(const char *msg);
/* include/openmmpol.h:33-34 (timers print at OMMP_VERBOSE_HIGH) */
void ommp_time_pull(const char *label);
void ommp_time_push(void);
/* include/openmmpol.h:38 ; src/mod_c_interface.F90:378-388 */
double ommp_get_polelec_energy(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:39 ; src/mod_c_interface.F90:390-401, energy_MM_MM
 * src/mod_electrostatics.F90:899-941.  Interaction energy of the static
 * multipoles (EM): the m-scaled pairs of the force field, no damping.
 * Computed on the GPU once per geometry. */
double ommp_get_fixedelec_energy(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:63 ; ommp_get_full_ele_energy src/mod_interface.F90:388-398.
 * The electrostatic energy: ommp_get_fixedelec_energy + ommp_get_polelec_energy. */
double ommp_get_full_ele_energy(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:40 ; src/mod_c_interface.F90:289-305.
 * ext_field: [pol_atoms][3].  Like the reference, `matv` is ignored on this
 * path and the default matrix-vector method is used (mod_interface.F90:222). */
void ommp_set_external_field(OMMP_SYSTEM_PRT s, const double *ext_field, int32_t solver, int32_t matv);
/* include/openmmpol.h:41 ; src/mod_c_interface.F90:307-325.  Solves the D
 * set only, from ext_field alone (no permanent-multipole field). */
void ommp_set_external_field_nomm(OMMP_SYSTEM_PRT s, const double *ext_field, int32_t solver,
                                  int32_t matv);
/* include/openmmpol.h:66 */
bool ommp_ff_is_amoeba(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:68-71 */
int32_t ommp_get_n_ipd(OMMP_SYSTEM_PRT s);
int32_t ommp_get_ld_cart(OMMP_SYSTEM_PRT s);
int32_t ommp_get_mm_atoms(OMMP_SYSTEM_PRT s);
int32_t ommp_get_pol_atoms(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:73 : [mm_atoms][3] */
double *ommp_get_cmm(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:76 : [pol_atoms][3] */
double *ommp_get_cpol(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:77 : [mm_atoms][ld_cart], lab frame */
double *ommp_get_q(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:78 ; src/mod_c_interface.F90:999-1008 : [n_ipd][pol_atoms][3] */
double *ommp_get_ipd(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:79 ; src/mod_c_interface.F90:1010-1028 : 0-based */
int32_t *ommp_get_polar_mm(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:86 : new coordinates [mm_atoms][3] */
void ommp_update_coordinates(OMMP_SYSTEM_PRT s, const double *cmm);
/* include/openmmpol.h:43-48 ; src/mod_c_interface.F90:327-376,1123-1176 ;
 * src/mod_interface.F90:250-330.  Potential v [n] or field E [n][3] at n
 * points cext [n][3] (bohr) of the static multipoles (mm), the induced
 * dipoles (pol: D set for the potential, (P + D)/2 for the AMOEBA field) or
 * both (mmpol); undamped, no screening.  The result is ADDED into v / E.
 * The induced part needs a solved system. */
void ommp_potential_mmpol2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *cext, double *v);
void ommp_potential_mm2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *cext, double *v);
void ommp_potential_pol2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *cext, double *v);
void ommp_field_mmpol2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *cext, double *E);
void ommp_field_mm2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *cext, double *E);
void ommp_field_pol2ext(OMMP_SYSTEM_PRT s, int32_t n, const double *cext, double *E);
/* include/openmmpol.h:91 ; src/mod_c_interface.F90:833-846, polelec_geomgrad
 * src/mod_geomgrad.F90:113-277.  Geometric gradient of the polarization
 * energy, grd [mm_atoms][3] (hartree/bohr), overwritten; the induced dipoles
 * are solved first (default solver) when the system has none.  FP64 on the
 * GPU whatever the precision mode. */
void ommp_polelec_geomgrad(OMMP_SYSTEM_PRT s, double *grd);
/* include/openmmpol.h:90 ; src/mod_c_interface.F90:818-831,
 * ommp_fixedelec_geomgrad src/mod_interface.F90:657-668, fixedelec_geomgrad
 * src/mod_geomgrad.F90:17-111.  Geometric gradient of the static multipole
 * energy (the m-scaled, undamped interaction of the static multipoles),
 * grd [mm_atoms][3] overwritten; FP64 on the GPU, computed once per
 * geometry. */
void ommp_fixedelec_geomgrad(OMMP_SYSTEM_PRT s, double *grd);
/* include/openmmpol.h:92 ; src/mod_c_interface.F90:606-624,
 * ommp_rotation_geomgrad src/mod_interface.F90:699-710, rotation_geomgrad
 * src/rotate_multipoles.F90:3-230.  Forces from the frame dependence of the
 * rotated static dipoles and quadrupoles in a caller's field E [mm_atoms][3]
 * and field gradient Egrd [mm_atoms][6] (xx, xy, yy, xz, yz, zz); grd
 * [mm_atoms][3] overwritten (zeros for point-charge force fields). */
void ommp_rotation_geomgrad(OMMP_SYSTEM_PRT s, const double *E, const double *Egrd, double *grd);
/* QM helper, include/openmmpol.h:106-127 ; src/mod_c_interface.F90:1179-1196,
 * 1374-1660 ; src/mod_qm_helper.F90:80-161,356-520.  A helper holds n QM
 * nuclei (coordinates cqm [n][3] bohr, charges qqm [n], atomic numbers zqm
 * [n]).  ommp_prepare_qm_ele_ene computes, once until the next
 * ommp_qm_helper_update_coord, the field of the nuclei at the polarizable
 * sites (E_n2p [pol_atoms][3]) and the potential of the static multipoles at
 * the nuclei (V_m2n [n]), and, once the system holds dipoles, that of the
 * induced dipoles (V_p2n [n]; like the reference, update_coord keeps it).
 * ommp_prepare_qm_ele_grd recomputes at every call the field, field gradient
 * and field Hessian of the nuclei at every static site (E_n2m [mm][3], G_n2m
 * [mm][6] xx,xy,yy,xz,yz,zz, H_n2m [mm][10] xxx,xxy,xxz,xyy,xyz,xzz,yyy,yyz,
 * yzz,zzz), G_n2p (G_n2m at the polarizable sites) and the field of the
 * static multipoles / induced dipoles at the nuclei (E_m2n, E_p2n [n][3];
 * E_p2n needs dipoles).  The getters return the helper's arrays, or NULL
 * before they are computed; get_npol / get_nmm return 0 until E_n2p / E_n2m
 * exist.  The QM-MM van der Waals terms, link atoms and frozen atoms of the
 * reference's helper are not part of this library. */
OMMP_QM_HELPER_PRT ommp_init_qm_helper(int32_t n, const double *cqm, const double *qqm, const int32_t *zqm);
void ommp_terminate_qm_helper(OMMP_QM_HELPER_PRT qm);
void ommp_qm_helper_update_coord(OMMP_QM_HELPER_PRT qm, const double *cqm);
void ommp_prepare_qm_ele_ene(OMMP_SYSTEM_PRT s, OMMP_QM_HELPER_PRT qm);
void ommp_prepare_qm_ele_grd(OMMP_SYSTEM_PRT s, OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_V_m2n(OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_V_p2n(OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_E_m2n(OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_E_p2n(OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_E_n2p(OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_G_n2p(OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_E_n2m(OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_G_n2m(OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_H_n2m(OMMP_QM_HELPER_PRT qm);
double *ommp_qm_helper_get_cqm(OMMP_QM_HELPER_PRT qm);
int32_t ommp_qm_helper_get_npol(OMMP_QM_HELPER_PRT qm);
int32_t ommp_qm_helper_get_nmm(OMMP_QM_HELPER_PRT qm);
int32_t ommp_qm_helper_get_qm_atoms(OMMP_QM_HELPER_PRT qm);
/* include/openmmpol.h:153-155 ; src/mod_c_interface.F90:1843-1879.  FMM
 * switch of the FP64 dipole-field products (T.mu of the FP64 solvers and of
 * the strict mixed mode's refinement residual) and of the permanent-multipole
 * field in the FP64 modes: a uniform octree with Cartesian expansions of total
 * order 10 (as accurate as the reference's default order-8 spherical FMM),
 * near pairs (neighbouring leaves, every damped pair among them) direct.  The
 * reference switches it on by itself above 1,000 atoms; here the direct sums
 * stay the default and the host asks for the FMM.  The FP32 inner products
 * and the double-single mode stay direct. */
void ommp_enable_fmm(OMMP_SYSTEM_PRT s);
void ommp_disable_fmm(OMMP_SYSTEM_PRT s);
bool ommp_use_fmm(OMMP_SYSTEM_PRT s);
/* include/openmmpol.h:156-160 ; src/mod_c_interface.F90:1781-1841.  The
 * reference's FMM settings.  lmax_pol: expansion order of the induced-dipole
 * (T.mu) products; lmax: order of the permanent-multipole field; both map to
 * the total order of this FMM's Cartesian expansions (2..12, default 10 each;
 * the reference's default 8 is a spherical-harmonic order, about as accurate
 * as 10 here).  distance (bohr): the reference treats leaf cells closer than
 * this as near; min_cell_size (bohr): it stops subdividing below this half
 * diagonal.  This FMM's near field is the 27 neighbouring leaves of a uniform
 * octree, so both become lower bounds of the leaf side (distance, and
 * 2 min_cell_size / sqrt 3), beside the Thole damping range; default 0 (the
 * damping range alone).  Out-of-range values stop the process like the
 * reference's errors. */
void ommp_set_fmm_lmax_pol(OMMP_SYSTEM_PRT s, int32_t l);
void ommp_set_fmm_lmax(OMMP_SYSTEM_PRT s, int32_t l);
void ommp_set_fmm_distance(OMMP_SYSTEM_PRT s, double d);
void ommp_set_fmm_min_cell_size(OMMP_SYSTEM_PRT s, double d);

/* ---- extensions (no counterpart in the reference) ---------------------- */

/* status-returning versions of the calls above (no process exit) */
int32_t ommp_gpu_init_mmp(const char *filename, OMMP_SYSTEM_PRT *out);
int32_t ommp_gpu_set_external_field(OMMP_SYSTEM_PRT s, const double *ext_field, int32_t solver,
                                    int32_t matv, int32_t add_mm_field);
/* the same call, named for hosts that look for an explicit status variant */
int32_t ommp_gpu_set_external_field_status(OMMP_SYSTEM_PRT s, const double *ext_field, int32_t solver,
                                           int32_t matv, int32_t add_mm_field);
/* same with a device pointer ext_field [pol_atoms][3] (no host copy) */
int32_t ommp_gpu_set_external_field_device(OMMP_SYSTEM_PRT s, const double *ext_field_dev,
                                           int32_t solver, int32_t matv, int32_t add_mm_field);
int32_t ommp_gpu_get_polelec_energy(OMMP_SYSTEM_PRT s, double *energy);
int32_t ommp_gpu_get_fixedelec_energy(OMMP_SYSTEM_PRT s, double *energy);
/* ommp_polelec_geomgrad returning a status instead of stopping the process */
int32_t ommp_gpu_polelec_geomgrad(OMMP_SYSTEM_PRT s, double *grd);
/* ommp_fixedelec_geomgrad returning a status */
int32_t ommp_gpu_fixedelec_geomgrad(OMMP_SYSTEM_PRT s, double *grd);
/* ommp_rotation_geomgrad returning a status */
int32_t ommp_gpu_rotation_geomgrad(OMMP_SYSTEM_PRT s, const double *E, const double *Egrd, double *grd);
/* FMM on (on != 0) or off, with expansion order 2..12 (both orders) */
int32_t ommp_gpu_set_fmm(OMMP_SYSTEM_PRT s, int32_t on, int32_t order);
/* the four FMM settings above returning a status instead of stopping */
int32_t ommp_gpu_set_fmm_lmax_pol(OMMP_SYSTEM_PRT s, int32_t l);
int32_t ommp_gpu_set_fmm_lmax(OMMP_SYSTEM_PRT s, int32_t l);
int32_t ommp_gpu_set_fmm_distance(OMMP_SYSTEM_PRT s, double d);
int32_t ommp_gpu_set_fmm_min_cell_size(OMMP_SYSTEM_PRT s, double d);
/* current orders and the leaf-side lower bound (bohr) from the settings */
void ommp_gpu_get_fmm_settings(OMMP_SYSTEM_PRT s, int32_t *lmax_pol, int32_t *lmax, double *min_leaf);
/* Process-wide, default off: systems created while on get the FMM switched
 * on when they have more than 1,000 MM atoms, as the reference does by
 * default (src/mod_electrostatics.F90:294-306).  Off, the direct sums stay
 * the default (the plain FP64 path then reproduces the reference's direct
 * results to 1e-9, which an FMM truncated at ~1e-4 cannot). */
void ommp_gpu_set_fmm_auto(int32_t on);
/* QM helper calls returning a status instead of stopping the process */
int32_t ommp_gpu_init_qm_helper(int32_t n, const double *cqm, const double *qqm, const int32_t *zqm,
                                OMMP_QM_HELPER_PRT *out);
int32_t ommp_gpu_prepare_qm_ele_ene(OMMP_SYSTEM_PRT s, OMMP_QM_HELPER_PRT qm);
int32_t ommp_gpu_prepare_qm_ele_grd(OMMP_SYSTEM_PRT s, OMMP_QM_HELPER_PRT qm);
int32_t ommp_gpu_update_coordinates(OMMP_SYSTEM_PRT s, const double *cmm);
int32_t ommp_gpu_set_default_solver(OMMP_SYSTEM_PRT s, int32_t solver);
int32_t ommp_gpu_set_default_matv(OMMP_SYSTEM_PRT s, int32_t matv);
/* text of the last error of any call (thread-local to the library) */
const char *ommp_gpu_last_error(void);

/* solver controls; the reference hard-codes tol 1e-8 / 200 iterations
 * (src/mod_solvers.F90:30-35) */
void ommp_gpu_set_solver_tol(OMMP_SYSTEM_PRT s, double tol);
void ommp_gpu_set_solver_maxiter(OMMP_SYSTEM_PRT s, int32_t maxiter);
void ommp_gpu_set_precision(OMMP_SYSTEM_PRT s, int32_t mode);
/* FP64 direct T.mu kernel: 0 auto (symmetric from 2048 sites), 1 all ordered
 * pairs, 2 symmetric (each unordered pair once, deterministic) */
int32_t ommp_gpu_set_fp64_kernel(OMMP_SYSTEM_PRT s, int32_t mode);
/* status-returning forms of ommp_{potential,field}_*2ext; which:
 * OMMP_GPU_EXT_MMPOL, OMMP_GPU_EXT_MM or OMMP_GPU_EXT_POL */
#define OMMP_GPU_EXT_MMPOL 0
#define OMMP_GPU_EXT_MM 1
#define OMMP_GPU_EXT_POL 2
int32_t ommp_gpu_potential_ext(OMMP_SYSTEM_PRT s, int32_t which, int32_t n, const double *cext, double *v);
int32_t ommp_gpu_field_ext(OMMP_SYSTEM_PRT s, int32_t which, int32_t n, const double *cext, double *E);
/* FP32 inner T.mu kernel: 0 autotuned (default), 1 one target per thread
 * with a per-pair damping test, 2 tile-classified (undamped inner loop for
 * tiles beyond the damping range, two targets per thread), 3 symmetric (each
 * unordered pair once for both directions, tile-classified, deterministic
 * fixed-point sums) */
int32_t ommp_gpu_set_fp32_kernel(OMMP_SYSTEM_PRT s, int32_t mode);
/* the FP32 launch shape the autotuner chose for ncol columns: shape[0] the
 * kernel (1, 2 or 3 as above), shape[1] the columns per launch, shape[2] the
 * source splits; zeros before the first mixed solve with ncol columns */
int32_t ommp_gpu_get_fp32_shape(OMMP_SYSTEM_PRT s, int32_t ncol, int32_t *shape);
/* preconditioner of the FP32 inner solver of the mixed modes: 0 the
 * reference's diagonal (alpha), 1 block Jacobi over runs of bonded sites,
 * 2 (default) block Jacobi with a first-order Neumann step over the
 * near-field couplings between the runs (z = B^-1 r - B^-1 N B^-1 r, N the
 * blocks of T between sites of different runs within 6.5 bohr).  The FP64
 * solver and the outer convergence test always use the reference's
 * diagonal. */
int32_t ommp_gpu_set_inner_preconditioner(OMMP_SYSTEM_PRT s, int32_t mode);
/* runs of the block-Jacobi inner preconditioner: at most max_sites (1..32)
 * consecutive polarizable sites, each within link_bohr of an earlier site of
 * its run (defaults 8 and 3.0); rebuilt at once and at every geometry */
int32_t ommp_gpu_set_inner_blocks(OMMP_SYSTEM_PRT s, int32_t max_sites, double link_bohr);
/* forget the last dipoles as a starting guess */
void ommp_gpu_clear_guess(OMMP_SYSTEM_PRT s);
/* capture the inner FP32 iteration as a CUDA graph (default on) */
void ommp_gpu_set_use_graphs(OMMP_SYSTEM_PRT s, int32_t on);
/* FP32 inner solve of batches (mixed modes, at least 4 columns): 1 (default)
 * block CG, the columns sharing one Krylov space; 0 the scalar PCG per
 * column */
void ommp_gpu_set_block_cg(OMMP_SYSTEM_PRT s, int32_t on);
/* refinement residuals of the mixed modes once one has been recomputed:
 * 0 recompute r = E - T mu with the mode's residual product (FP64 or
 * double-single) at every step; 1 update r -= T d with the FP32 product of
 * the step's correction d when the bound on its error (1e-5 of the residual,
 * the FP32 operator's tested accuracy) is below a tenth of the tolerance,
 * recomputing otherwise; -1 (default) by mode: 1 in mixed-ds, 0 in the
 * strict mixed mode, whose every residual stays an FP64 product */
int32_t ommp_gpu_set_residual_update(OMMP_SYSTEM_PRT s, int32_t mode);

/* Batched right-hand sides: nfields external fields (e.g. from several QM
 * densities) solved together, each as ommp_set_external_field would solve it
 * from a zero guess, in the system's precision mode; the columns of all
 * fields share every pair evaluation (mixed mode: one block of columns
 * through the FP32-inner / FP64-refinement solver).  fields [nfields]
 * [pol_atoms][3]; ipd_out [nfields][n_ipd][pol_atoms][3]; energies [nfields]
 * (host, may be NULL) = ommp_get_polelec_energy of each solution.  The
 * system's own dipoles and warm-start guess are not touched. */
int32_t ommp_gpu_set_external_fields_batch(OMMP_SYSTEM_PRT s, int32_t nfields, const double *fields,
                                           double *ipd_out, double *energies);
/* same with fields and ipd_out in device memory */
int32_t ommp_gpu_set_external_fields_batch_device(OMMP_SYSTEM_PRT s, int32_t nfields,
                                                  const double *fields_dev, double *ipd_out_dev,
                                                  double *energies);

/* results of the last solve: iterations of set k (CG/DIIS) or refinement
 * steps (mixed), residual history (returns the length, copies up to maxn) */
int32_t ommp_gpu_get_iterations(OMMP_SYSTEM_PRT s, int32_t set);
int32_t ommp_gpu_get_residual_history(OMMP_SYSTEM_PRT s, int32_t set, double *out, int32_t maxn);
/* counters of the last solve: 0 FP64 T.mu products, 1 FP32 products,
 * 2 refinement steps, 3 inner FP32 iterations, 4 double-single products,
 * 5 refinement residuals updated by an FP32 product */
int64_t ommp_gpu_get_counter(OMMP_SYSTEM_PRT s, int32_t which);
/* device time of the last polarization solve (ms, CUDA events) */
double ommp_gpu_last_solve_ms(OMMP_SYSTEM_PRT s);

/* verification hooks: E_M2D [n_ipd][pol_atoms][3]; y = T x for nrhs (1|2)
 * columns [nrhs][pol_atoms][3]; dodiag = 0 leaves out the 1/alpha diagonal */
int32_t ommp_gpu_get_e_m2d(OMMP_SYSTEM_PRT s, double *out);
int32_t ommp_gpu_tmatvec(OMMP_SYSTEM_PRT s, const double *x, double *y, int32_t nrhs, int32_t dodiag,
                         int32_t matv);
int32_t ommp_gpu_tmatvec_fp32(OMMP_SYSTEM_PRT s, const double *x, double *y, int32_t nrhs);
/* the double-single product of OMMP_GPU_PREC_MIXED_DS (diagonal included) */
int32_t ommp_gpu_tmatvec_ds(OMMP_SYSTEM_PRT s, const double *x, double *y, int32_t nrhs);

/* CUDA-event timing of the pair kernels: which 0 = FP64 T.mu, 1 = FP32 T.mu,
 * 2 = double-single T.mu;
 * columns = right-hand sides summed over the timed launches (may be NULL) */
void ommp_gpu_enable_kernel_timing(OMMP_SYSTEM_PRT s, int32_t on);
void ommp_gpu_kernel_stats(OMMP_SYSTEM_PRT s, int32_t which, int64_t *launches, double *total_ms,
                           int64_t *columns);
void ommp_gpu_reset_kernel_stats(OMMP_SYSTEM_PRT s);
int32_t ommp_gpu_synchronize(OMMP_SYSTEM_PRT s);
/* stream-ordered timers on the system's stream: record slot 0..7, then the
 * elapsed device time between two recorded slots (waits for the second) */
int32_t ommp_gpu_timer_record(OMMP_SYSTEM_PRT s, int32_t slot);
int32_t ommp_gpu_timer_elapsed(OMMP_SYSTEM_PRT s, int32_t a, int32_t b, double *ms);
/* overwrite `bytes` of a scratch buffer on the system's stream (L2 flush) */
int32_t ommp_gpu_flush_l2(OMMP_SYSTEM_PRT s, int64_t bytes);
/* kernels launched by this library since it was loaded */
int64_t ommp_gpu_kernel_launch_count(void);
/* device buffers for hosts without their own CUDA runtime (device-pointer API) */
int32_t ommp_gpu_device_alloc(int64_t bytes, void **ptr);
int32_t ommp_gpu_device_free(void *ptr);
int32_t ommp_gpu_copy_to_device(void *dst, const void *src, int64_t bytes);
int32_t ommp_gpu_copy_to_host(void *dst, const void *src, int64_t bytes);
/* free and total device memory of the current device, bytes */
int32_t ommp_gpu_device_mem_info(int64_t *free_bytes, int64_t *total_bytes);
/* measured FMA throughput of the FP64 (fp64 = 1) or FP32 pipe, TFLOP/s */
int32_t ommp_gpu_measure_pipe_peak(int32_t fp64, double *tflops);
/* SM count of the current device, 0 without a GPU */
int32_t ommp_gpu_device_sm_count(void);

/* No counterpart in the reference.  The solves of nsys systems (mixed or
 * mixed-ds precision, direct products), each with its own external field
 * fields[k] [pol_atoms][3] (host memory), advanced together on one stream:
 * every round, the pair products of all systems that need one share one
 * persistent launch per product kind and column width (work items: system,
 * super-tile, chunk of slots), each product getting a bounded share per round
 * (a fair share first, then the shortest), so that small systems keep
 * iterating while a large product is spread over several rounds.  Results and
 * state as after ommp_gpu_set_external_field on each system; energies [nsys]
 * the polarization energies.  stats5 (may be NULL): rounds, product
 * launches, launches that served two or more systems, most systems in one
 * launch, products spread over several launches. */
int32_t ommp_gpu_solve_multi(int32_t nsys, OMMP_SYSTEM_PRT *systems, const double *const *fields, double *energies,
                             int64_t *stats5);

/* ---- request server (no counterpart in the reference) -------------------
 * Continuous admission of solves on one GPU: `slots` worker threads each carry
 * one request at a time (host setup, upload and E_M2D on its system's own
 * CUDA stream; in the mixed modes the solve then joins the multi-system
 * engine of ommp_gpu_solve_multi, in FP64 it runs on the system's stream);
 * a request starts as soon as a slot is free
 * and its device memory fits `hbm_budget_bytes`, idle systems being evicted
 * least-recently-used first.  ommp_gpu_server_submit reads a new system from
 * a .mmp file (host setup, upload, E_M2D, solve); _submit_followup solves a
 * new field on a resident instance warm-started from its last dipoles
 * (follow-ups on one instance run in submission order).  _wait blocks until
 * the request is done and returns its dipoles [n_ipd][pol_atoms][3], its
 * polarization energy, the instance id (for follow-ups) and the latency from
 * submission to completion.  _stats fills 7 numbers: device bytes in use,
 * peak bytes, resident instances, evictions, peak concurrent requests,
 * completed requests, budget.  _cancel removes a request that is still
 * queued (its _wait then returns OMMP_GPU_ERR_CANCELLED) and returns
 * OMMP_GPU_ERR_BAD_ARG for one that is running, done or unknown.  Destroy
 * the server after waiting for every submitted request. */
int32_t ommp_gpu_server_create(int64_t hbm_budget_bytes, int32_t slots, int32_t precision, double tol,
                               void **server);
void ommp_gpu_server_destroy(void *server);
int32_t ommp_gpu_server_submit(void *server, const char *mmp_path, const double *field, int32_t pol_atoms,
                               int64_t *request_id);
int32_t ommp_gpu_server_submit_followup(void *server, int64_t instance, const double *field,
                                        int32_t pol_atoms, int64_t *request_id);
int32_t ommp_gpu_server_wait(void *server, int64_t request_id, double *ipd_out, double *energy,
                             int64_t *instance, double *latency_ms);
void ommp_gpu_server_release(void *server, int64_t instance);
int32_t ommp_gpu_server_cancel(void *server, int64_t request_id);
void ommp_gpu_server_stats(void *server, double *out7);
/* the multi-system engine of the mixed modes: rounds, product launches,
 * launches that served two or more systems, most systems in one launch,
 * products spread over several rounds (zeros in FP64) */
void ommp_gpu_server_engine_stats(void *server, int64_t *out5);
/* where the engine's rounds spent their time, in milliseconds summed over
 * rounds: [0] GPU time of the product launches, [1] GPU time of the
 * per-system bookkeeping after them, [2] host wall time of the rounds */
void ommp_gpu_server_engine_times(void *server, double *out3);
/* where the new systems' latency went, summed over those that completed
 * without error: [0] their count, then milliseconds [1] waiting for a
 * worker slot, [2] in host setup (file, topology, lists, rotation), [3]
 * waiting for device memory, [4] uploading, [5] forming the permanent field
 * and right-hand side (mixed modes; 0 in FP64, where it is part of [6]),
 * [6] solving */
void ommp_gpu_server_phase_stats(void *server, double *out7);
/* work per product kind in one round of the engine, in milliseconds of GPU
 * time (default 1.5): shorter rounds let small systems iterate faster beside
 * large ones, longer ones spend less on the per-round bookkeeping */
int32_t ommp_gpu_server_set_round_ms(void *server, double ms);

/* No counterpart in the reference.  y = T x (dodiag = 1) or y = -E_dd(x)
 * (dodiag = 0) for nrhs (1|2) columns [nrhs][pol_atoms][3], with x and y in
 * caller-owned DEVICE memory, and no memory allocation inside the call: for
 * hosts that manage all GPU memory themselves (a QM code's SCF loop with its
 * own memory pool, an MD step that must not stall on cudaMalloc).  The
 * product is always the direct FP64 sum over all pairs, whatever the
 * system's FMM, matrix-vector or FP64-kernel settings.  Scratch is a 16 MiB
 * static device array, so pol_atoms * nrhs <= 699050; larger sizes are
 * rejected with OMMP_GPU_ERR_BAD_ARG, and so are overlapping x and y (no
 * in-place product).  The array is placed on a device when a system is
 * created there; a call on a device without a system created first places
 * it itself (make such a first call before any stream capture).  The kernels
 * run on the system's own stream, which is not ordered against the caller's
 * streams: whatever wrote x (a copy or a kernel) must have completed before
 * the call.  Calls share the array: calls that overlap on the GPU race.  The
 * call returns after its kernels have finished. */
int32_t ommp_gpu_tmatvec_noalloc(OMMP_SYSTEM_PRT s, const double *x_dev, double *y_dev, int32_t nrhs,
                                 int32_t dodiag);

#ifdef __cplusplus
}
#endif
#endif
