/*
 * ommp_oracle.h -- CPU restatement of OpenMMPol's induced-point-dipole path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * implementation in openmmpol_gb300/; only tests/, __graft_entry__.smoke()
 * and the CPU-baseline leg of bench.py may load it.  The product library never
 * links it and never falls back to it.
 *
 * It restates, loop for loop, the reference algorithms (file:line are in the
 * reference project's source tree):
 *   .mmp loader             src/mod_inputloader.F90:15-295
 *   mmpol_prepare           src/mod_mmpol.F90:139-237, 272-323
 *   connectivity C_n        src/mod_adjacency_mat.F90:367-422
 *   thole_init              src/mod_electrostatics.F90:866-897
 *   rotate_multipoles       src/rotate_multipoles.F90:232-643
 *   make_screening_lists    src/mod_electrostatics.F90:538-864
 *   screening_rules         src/mod_electrostatics.F90:3338-3487
 *   damped_coulomb_kernel   src/mod_electrostatics.F90:978-1095
 *   q/mu/quad_elec_prop     src/mod_electrostatics.F90:1097-1405 (field only)
 *   elec_prop_M2D (direct)  src/mod_electrostatics.F90:2579-2731
 *   field_extD2D (direct)   src/mod_electrostatics.F90:2068-2109
 *   TMatVec_*, PolVec       src/mod_polarization.F90:327-557
 *   polarization            src/mod_polarization.F90:49-313
 *   CG / Jacobi-DIIS / inv  src/mod_solvers.F90:30-494
 *   set_external_field      src/mod_interface.F90:184-233
 *   get_polelec_energy      src/mod_interface.F90:343-370, energy_MM_pol
 *                           src/mod_electrostatics.F90:943-976
 *   polelec_geomgrad        src/mod_geomgrad.F90:113-277, rotation_geomgrad
 *                           src/rotate_multipoles.F90:3-230, 298-643
 *   potential/field at external points (QM coupling)
 *                           src/mod_electrostatics.F90:3067-3336,
 *                           src/mod_interface.F90:250-330
 *
 * Parity of this restatement is pinned against the reference's own golden
 * files (tests/N-methylacetamide, tests/1crn, tests/1ao6, tests/1ubq IPD_* and
 * ENE_*) by tests/test_oracle_golden.py.
 *
 * Errors never exit the process: every entry returns a status (0 = success)
 * and the message is available from orc_last_error().
 */
#ifndef OMMP_ORACLE_H
#define OMMP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sys orc_sys;

/* status codes */
#define ORC_OK 0
#define ORC_ERR_INPUT 1
#define ORC_ERR_NOT_CONVERGED 2
#define ORC_ERR_BAD_ARG 3
#define ORC_ERR_NUMERIC 4

const char *orc_last_error(void);

orc_sys *orc_init_mmp(const char *path);
void orc_free(orc_sys *s);

int32_t orc_mm_atoms(const orc_sys *s);
int32_t orc_pol_atoms(const orc_sys *s);
int32_t orc_n_ipd(const orc_sys *s);
int32_t orc_is_amoeba(const orc_sys *s);
int32_t orc_ld_cart(const orc_sys *s);

/* solver controls (reference defaults: tol 1e-8, 200 iterations, DIIS 20) */
void orc_set_tol(orc_sys *s, double tol);
void orc_set_maxiter(orc_sys *s, int32_t n);
void orc_set_default_solver(orc_sys *s, int32_t solver);
void orc_set_default_matv(orc_sys *s, int32_t matv);
void orc_set_num_threads(int32_t n);

/* copies out; shapes are C-order */
void orc_get_cmm(const orc_sys *s, double *out);        /* [mm][3] bohr */
void orc_get_q(const orc_sys *s, double *out);          /* [mm][ld_cart] lab frame */
void orc_get_pol(const orc_sys *s, double *out);        /* [npol] */
void orc_get_polar_mm(const orc_sys *s, int32_t *out);  /* [npol], 0-based */
void orc_get_thole(const orc_sys *s, double *out);      /* [mm] */
int orc_get_e_m2d(orc_sys *s, double *out);             /* [n_ipd][npol][3] */
void orc_get_ipd(const orc_sys *s, double *out);        /* [n_ipd][npol][3] */
int32_t orc_screening_nnz(const orc_sys *s, int32_t which); /* 0 S_P_P, 1 S_P_D, 2 P_P */
void orc_get_screening(const orc_sys *s, int32_t which, int32_t *ri, int32_t *ci, double *scale);

/* y = T x (dodiag=1) or y = -E_dd(x) (dodiag=0); x,y [npol][3] */
int orc_tmatvec(orc_sys *s, const double *x, double *y, int32_t dodiag, int32_t matv);
/* rows of T x with the diagonal, for sampled residual checks; y [nrows][3] */
int orc_tmatvec_rows(orc_sys *s, const double *x, const int32_t *rows, int32_t nrows, double *y);

/* ommp_set_external_field[_nomm]: ext [npol][3]; returns status */
int orc_set_external_field(orc_sys *s, const double *ext, int32_t solver, int32_t matv,
                           int32_t add_mm);
/* ommp_get_polelec_energy; status via *status if non-NULL */
double orc_get_polelec_energy(orc_sys *s, int32_t *status);
/* per-set iteration count and residual history of the last solve */
int32_t orc_last_iterations(const orc_sys *s, int32_t set);
/* T.mu products evaluated by the last polarization solve */
int64_t orc_matvec_count(const orc_sys *s);
int32_t orc_residual_history(const orc_sys *s, int32_t set, double *out, int32_t maxn);
/* ommp_update_coordinates: c [mm][3] bohr */
int orc_update_coordinates(orc_sys *s, const double *c);
/* drop the warm-start guess (ipd_use_guess = false) */
void orc_clear_guess(orc_sys *s);
/* potential [n] / field [n][3] at points cext [n][3] (bohr), ADDED into the
   output like the reference's ommp_{potential,field}_*2ext; which: 0 static
   multipoles + induced dipoles, 1 static multipoles, 2 induced dipoles */
int orc_potential_ext(orc_sys *s, int32_t which, int32_t n, const double *cext, double *v);
int orc_field_ext(orc_sys *s, int32_t which, int32_t n, const double *cext, double *e);
/* polelec_geomgrad: gradient of the polarization energy with respect to the
   static-site coordinates, ADDED into grad [mm][3] (solves with the
   permanent field alone first if no dipoles are available) */
int orc_polelec_geomgrad(orc_sys *s, double *grad);
/* the same gradient on the listed atoms only, out [na][3] (overwritten);
   fields are evaluated only where those atoms need them */
int orc_polelec_geomgrad_atoms(orc_sys *s, int32_t na, const int32_t *atoms, double *out);
/* install induced dipoles ipd [n_ipd][npol][3] as the solved state (so that
   the gradient can be evaluated on dipoles solved elsewhere) */
int orc_set_ipd(orc_sys *s, const double *ipd);
/* fields of QM nuclei (charges qqm at cqm [nq][3]) at the MM sites, the QM
   helper's E_n2p (which 0: E [npol][3]) or E_n2m / G_n2m / H_n2m (which 1:
   E [mm][3], G [mm][6], H [mm][10]); outputs overwritten */
/* ommp_get_fixedelec_energy: interaction energy of the static multipoles
   (m-scaled pairs, undamped) */
int orc_get_fixedelec_energy(orc_sys *s, double *energy);
/* ommp_rotation_geomgrad: frame forces of the static multipoles in E [mm][3]
   and field gradient G [mm][6]; grad [mm][3] overwritten */
int orc_rotation_geomgrad(orc_sys *s, const double *E, const double *G, double *grad);
/* ommp_fixedelec_geomgrad: gradient of the static multipole energy,
   grad [mm][3] overwritten */
int orc_fixedelec_geomgrad(orc_sys *s, double *grad);
int orc_nuclei_fields(orc_sys *s, int32_t which, int32_t nq, const double *cqm, const double *qqm, double *E,
                      double *G, double *H);

#ifdef __cplusplus
}
#endif
#endif
