/*
 * ommp_oracle.c -- CPU restatement (C99 + OpenMP) of OpenMMPol's induced
 * point dipole path.  TEST INFRASTRUCTURE ONLY: the checker for the GPU
 * library, never linked by it.  See ommp_oracle.h for the list of reference
 * routines restated here; each function below cites its reference lines.
 *
 * Loop structure follows the reference on purpose (target-outer pair loops,
 * linear scan of the screening-list row for every pair, skip when the scale
 * factor is zero, multiply when it differs from one) so that the oracle is a
 * literal restatement, not a second optimised implementation.
 */
#include "ommp_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ANG2AU 1.8897261245650            /* config/openmmpol_const.h.in:40 */
#define EPS_RP (2.220446049250313e-16 * 100) /* mod_constants.F90:62 */
#define SOLVER_NONE 0
#define SOLVER_CG 1
#define SOLVER_DIIS 2
#define SOLVER_INVERSION 3
#define MATV_NONE 0
#define MATV_INCORE 1
#define MATV_DIRECT 2
#define MAXN12 8   /* mod_inputloader.F90:65 */
#define MAXPGP 120 /* mod_inputloader.F90:67 */
#define MAX_HIST 1024

static char g_err[512];
const char *orc_last_error(void) { return g_err; }
static void set_err(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

void orc_set_num_threads(int32_t n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* boolean CSR ("yale_sparse", mod_adjacency_mat.F90:28-38), 0-based */
typedef struct {
    int n;
    int *ri; /* n+1 */
    int *ci;
} csr_t;

typedef struct {
    csr_t m;
    double *scale; /* per entry */
    unsigned char *todo;
} slist_t;

struct orc_sys {
    int amoeba, mm, npol, ld_cart, n_ipd;
    double *cmm;      /* [mm][3] */
    double *q0, *q;   /* [mm][ld_cart] */
    double *pol;      /* [npol] */
    int *polar_mm;    /* [npol] */
    int *mm_polar;    /* [mm], -1 = not polarizable */
    double *thole;    /* [mm] */
    double *thole_damping; /* [npol] */
    double thole_scale;
    int *grp;         /* [mm] polarization group, 0-based (AMOEBA) */
    int ngrp;
    int *frame, *iz, *ix, *iy; /* [mm], -1 = none */
    csr_t conn[4];    /* 1-2 .. 1-5 */
    csr_t grp_atoms;  /* group -> atoms */
    csr_t pg_conn[4]; /* identity, 1-2, 1-3, 1-4 between groups */
    double mscale[4], pscale[4], dscale[4], uscale[4], pscale_intra[4];
    slist_t sPP, sPD, PP;
    double *e_m2d; /* [n_ipd][npol][3] */
    int m2d_done;
    double *ipd;   /* [n_ipd][npol][3] */
    int ipd_done, ipd_use_guess;
    int def_solver, def_matv;
    double tol;
    int maxiter, diis_max;
    double *tmat;  /* [3n][3n] column-major like the reference */
    int last_iters[2];
    long matvecs; /* T.mu products since the last polarization() call */
    int hist_n[2];
    double hist[2][MAX_HIST];
};

/* ------------------------------------------------------------------ */
/* small helpers                                                       */
/* ------------------------------------------------------------------ */
static void *xcalloc(size_t n, size_t sz) {
    void *p = calloc(n ? n : 1, sz);
    if (!p) {
        fprintf(stderr, "oracle: out of memory\n");
        abort();
    }
    return p;
}

static void csr_free(csr_t *m) {
    free(m->ri);
    free(m->ci);
    m->ri = m->ci = NULL;
    m->n = 0;
}

static int csr_has(const csr_t *m, int row, int col) {
    for (int k = m->ri[row]; k < m->ri[row + 1]; k++)
        if (m->ci[k] == col) return 1;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Fortran list-directed reader for the .mmp format                    */
/* ------------------------------------------------------------------ */
typedef struct {
    FILE *f;
    char *line;
    size_t cap;
    int eof;
} rdr_t;

static int rd_line(rdr_t *r) {
    ssize_t n = getline(&r->line, &r->cap, r->f);
    if (n < 0) {
        r->eof = 1;
        return 0;
    }
    return 1;
}

/* skip_lines (mod_utils.F90:302-318): one record per skipped line */
static int rd_skip(rdr_t *r, long n) {
    for (long i = 0; i < n; i++)
        if (!rd_line(r)) return 0;
    return 1;
}

/* list-directed read of `want` numbers: continues over records until
 * satisfied, the rest of the last record is discarded.  Fortran 'D'
 * exponents and r*c repeat counts are accepted. */
static int rd_values(rdr_t *r, double *out, int want) {
    int got = 0;
    while (got < want) {
        if (!rd_line(r)) return 0;
        char *p = r->line;
        while (*p && got < want) {
            while (*p && (isspace((unsigned char)*p) || *p == ',')) p++;
            if (!*p) break;
            char tok[128];
            int k = 0;
            while (*p && !isspace((unsigned char)*p) && *p != ',' && k < 127) {
                char c = *p++;
                if (c == 'D' || c == 'd') c = 'e';
                tok[k++] = c;
            }
            tok[k] = 0;
            long rep = 1;
            char *num = tok;
            char *star = strchr(tok, '*');
            if (star) {
                *star = 0;
                rep = strtol(tok, NULL, 10);
                num = star + 1;
                if (rep <= 0) return 0;
            }
            char *end;
            double v = strtod(num, &end);
            if (end == num) return 0;
            for (long t = 0; t < rep && got < want; t++) out[got++] = v;
        }
    }
    return 1;
}

static int rd_ints(rdr_t *r, int *out, int want) {
    double tmp[MAXPGP];
    if (want > MAXPGP) return 0;
    if (!rd_values(r, tmp, want)) return 0;
    for (int i = 0; i < want; i++) out[i] = (int)tmp[i];
    return 1;
}

/* ------------------------------------------------------------------ */
/* connectivity: C_n = C_{n-1} C_1 - (C_{n-1} + C_{n-2}), C_0 = 1      */
/* mod_adjacency_mat.F90:367-422 (mat_mult :222, mat_andnot :269)      */
/* ------------------------------------------------------------------ */
static void csr_mult_andnot(const csr_t *a, const csr_t *adj, const csr_t *m1,
                            const csr_t *m2, int m2_is_identity, csr_t *res) {
    int n = a->n;
    int cap = 16;
    res->n = n;
    res->ri = xcalloc(n + 1, sizeof(int));
    res->ci = xcalloc(cap, sizeof(int));
    int nnz = 0;
    for (int i = 0; i < n; i++) {
        res->ri[i] = nnz;
        for (int k = a->ri[i]; k < a->ri[i + 1]; k++) {
            int mid = a->ci[k];
            for (int l = adj->ri[mid]; l < adj->ri[mid + 1]; l++) {
                int c = adj->ci[l];
                /* not already present in the product row */
                int dup = 0;
                for (int t = res->ri[i]; t < nnz; t++)
                    if (res->ci[t] == c) {
                        dup = 1;
                        break;
                    }
                if (dup) continue;
                if (csr_has(m1, i, c)) continue;
                if (m2_is_identity ? (c == i) : csr_has(m2, i, c)) continue;
                if (nnz == cap) {
                    cap *= 2;
                    res->ci = realloc(res->ci, cap * sizeof(int));
                }
                res->ci[nnz++] = c;
            }
        }
    }
    res->ri[n] = nnz;
}

static void csr_copy(const csr_t *f, csr_t *t) {
    t->n = f->n;
    t->ri = xcalloc(f->n + 1, sizeof(int));
    memcpy(t->ri, f->ri, (f->n + 1) * sizeof(int));
    int nnz = f->ri[f->n];
    t->ci = xcalloc(nnz, sizeof(int));
    memcpy(t->ci, f->ci, nnz * sizeof(int));
}

static void csr_identity(int n, csr_t *t) {
    t->n = n;
    t->ri = xcalloc(n + 1, sizeof(int));
    t->ci = xcalloc(n, sizeof(int));
    for (int i = 0; i < n; i++) {
        t->ri[i] = i;
        t->ci[i] = i;
    }
    t->ri[n] = n;
}

/* build_conn_upto_n: res[0..] ; with start_id res[0]=identity, res[1]=adj */
static void build_conn(const csr_t *adj, int nlev, csr_t *res, int start_id) {
    int a = start_id ? 1 : 0;
    if (start_id) csr_identity(adj->n, &res[0]);
    csr_copy(adj, &res[a]);
    csr_t id;
    csr_identity(adj->n, &id);
    for (int i = a + 1; i < a + nlev; i++) {
        const csr_t *m2 = (i == a + 1) ? &id : &res[i - 2];
        csr_mult_andnot(&res[i - 1], &res[a], &res[i - 1], m2, i == a + 1, &res[i]);
    }
    csr_free(&id);
}

/* ------------------------------------------------------------------ */
/* rotate_multipoles / rotation_matrix, rotate_multipoles.F90:232-464  */
/* ------------------------------------------------------------------ */
static int rotation_matrix(const double *c, const double *cx, const double *cy,
                           const double *cz, int frame, double r[3][3]) {
    double xi[3], eta[3], zeta[3], u[3] = {0, 0, 0}, v[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++) {
        xi[k] = cz[k] - c[k];
        eta[k] = cx[k] - c[k];
        zeta[k] = cy[k] - c[k];
    }
    double xin = sqrt(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]);
    double etan = sqrt(eta[0] * eta[0] + eta[1] * eta[1] + eta[2] * eta[2]);
    double zetan = sqrt(zeta[0] * zeta[0] + zeta[1] * zeta[1] + zeta[2] * zeta[2]);
    memset(r, 0, 9 * sizeof(double));
    if (frame == 0) {
        r[0][0] = r[1][1] = r[2][2] = 1.0;
        return 0;
    } else if (frame == 1) { /* z-then-x */
        for (int k = 0; k < 3; k++) {
            u[k] = xi[k];
            v[k] = eta[k];
        }
    } else if (frame == 2) { /* bisector */
        for (int k = 0; k < 3; k++) {
            u[k] = etan * xi[k] + xin * eta[k];
            v[k] = eta[k];
        }
    } else if (frame == 3) { /* z-only */
        for (int k = 0; k < 3; k++) u[k] = xi[k];
        double dot = u[2] / xin;
        if (dot <= 0.866 && fabs(u[1]) > EPS_RP)
            v[0] = 1.0;
        else
            v[1] = 1.0;
    } else if (frame == 4) { /* z-bisector */
        for (int k = 0; k < 3; k++) {
            u[k] = xi[k];
            v[k] = zetan * eta[k] + etan * zeta[k];
        }
    } else if (frame == 5) { /* 3-fold */
        for (int k = 0; k < 3; k++) {
            u[k] = etan * zetan * xi[k] + xin * zetan * eta[k] + xin * etan * zeta[k];
            v[k] = eta[k];
        }
    }
    double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    double vn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (un < EPS_RP || vn < EPS_RP) {
        set_err("Ill defined rotation axis (either u or v vectors have 0 norm.");
        return ORC_ERR_INPUT;
    }
    double ez[3], ex[3], ey[3];
    for (int k = 0; k < 3; k++) ez[k] = u[k] / un;
    double vez = v[0] * ez[0] + v[1] * ez[1] + v[2] * ez[2];
    for (int k = 0; k < 3; k++) ex[k] = v[k] - vez * ez[k];
    double exn = sqrt(ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2]);
    for (int k = 0; k < 3; k++) ex[k] /= exn;
    ey[0] = ez[1] * ex[2] - ez[2] * ex[1];
    ey[1] = ez[2] * ex[0] - ez[0] * ex[2];
    ey[2] = ez[0] * ex[1] - ez[1] * ex[0];
    for (int k = 0; k < 3; k++) {
        r[k][0] = ex[k];
        r[k][1] = ey[k];
        r[k][2] = ez[k];
    }
    return 0;
}

static int rotate_multipoles(orc_sys *s) {
    for (int j = 0; j < s->mm; j++) {
        int jz = s->iz[j] >= 0 ? s->iz[j] : j;
        int jx = s->ix[j] >= 0 ? s->ix[j] : j;
        int jy = s->iy[j] >= 0 ? s->iy[j] : j;
        double r[3][3];
        int st = rotation_matrix(&s->cmm[3 * j], &s->cmm[3 * jx], &s->cmm[3 * jy],
                                 &s->cmm[3 * jz], s->frame[j], r);
        if (st) return st;
        const double *q0 = &s->q0[10 * j];
        double *q = &s->q[10 * j];
        q[0] = q0[0];
        for (int a = 0; a < 3; a++)
            q[1 + a] = r[a][0] * q0[1] + r[a][1] * q0[2] + r[a][2] * q0[3];
        /* quadrupole storage xx,xy,yy,xz,yz,zz (f_cart_components.h) */
        double Q[3][3] = {{q0[4], q0[5], q0[7]}, {q0[5], q0[6], q0[8]}, {q0[7], q0[8], q0[9]}};
        double t[3][3], R[3][3];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                t[a][b] = 0;
                for (int c = 0; c < 3; c++) t[a][b] += r[a][c] * Q[c][b];
            }
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                R[a][b] = 0;
                for (int c = 0; c < 3; c++) R[a][b] += t[a][c] * r[b][c];
            }
        q[4] = R[0][0];
        q[5] = R[0][1];
        q[6] = R[1][1];
        q[7] = R[0][2];
        q[8] = R[1][2];
        q[9] = R[2][2];
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* screening_rules, mod_electrostatics.F90:3338-3487                    */
/* kind: 'S' static (mm index) / 'P' polarizable (pol index)           */
/* ------------------------------------------------------------------ */
static double screening_rules(const orc_sys *s, int i, char kind_i, int j, char kind_j,
                              char in_field) {
    int i_mm = (kind_i == 'P') ? s->polar_mm[i] : i;
    int j_mm = (kind_j == 'P') ? s->polar_mm[j] : j;
    const double *myscale;
    const double *myintra = NULL;
    char interaction, field = '-';
    if (kind_i == 'P' && kind_j == 'P') {
        myscale = s->uscale;
        interaction = 'P';
    } else if (kind_i == 'S' && kind_j == 'S') {
        myscale = s->mscale;
        interaction = 'S';
    } else {
        if (in_field == 'P' && s->amoeba) {
            myscale = s->pscale;
            myintra = s->pscale_intra;
            field = 'P';
        } else if (in_field == 'D' && s->amoeba) {
            myscale = s->dscale;
            field = 'D';
        } else {
            myscale = s->pscale;
            field = 'P';
        }
        interaction = 'M';
    }
    double scalf = 1.0;
    if (!s->amoeba || (interaction == 'M' && field == 'P') || interaction == 'S') {
        for (int ineigh = 0; ineigh < 4; ineigh++) {
            if (csr_has(&s->conn[ineigh], i_mm, j_mm)) {
                if (interaction == 'M' && s->amoeba) {
                    scalf = (s->grp[i_mm] == s->grp[j_mm]) ? myintra[ineigh] : myscale[ineigh];
                } else {
                    scalf = myscale[ineigh];
                }
                break;
            }
        }
    } else {
        int pg_i = s->grp[i_mm];
        for (int ineigh = 0; ineigh < 4; ineigh++) {
            const csr_t *pc = &s->pg_conn[ineigh];
            for (int ig = pc->ri[pg_i]; ig < pc->ri[pg_i + 1]; ig++) {
                int g = pc->ci[ig];
                if (csr_has(&s->grp_atoms, g, j_mm)) {
                    return myscale[ineigh];
                }
            }
        }
    }
    return scalf;
}

/* list builder (compress_list + compress_data + todo), one row at a time */
typedef struct {
    int n, cap, nnz;
    int *ri, *ci;
    double *sc;
} lbuild_t;

static void lb_init(lbuild_t *b, int n) {
    b->n = n;
    b->cap = 64;
    b->nnz = 0;
    b->ri = xcalloc(n + 1, sizeof(int));
    b->ci = xcalloc(b->cap, sizeof(int));
    b->sc = xcalloc(b->cap, sizeof(double));
}
static void lb_push(lbuild_t *b, int c, double v) {
    if (b->nnz == b->cap) {
        b->cap *= 2;
        b->ci = realloc(b->ci, b->cap * sizeof(int));
        b->sc = realloc(b->sc, b->cap * sizeof(double));
    }
    b->ci[b->nnz] = c;
    b->sc[b->nnz] = v;
    b->nnz++;
}
static void lb_finish(lbuild_t *b, slist_t *out) {
    b->ri[b->n] = b->nnz;
    out->m.n = b->n;
    out->m.ri = b->ri;
    out->m.ci = b->ci;
    out->scale = b->sc;
    out->todo = xcalloc(b->nnz, 1);
    for (int k = 0; k < b->nnz; k++) out->todo[k] = fabs(b->sc[k]) > EPS_RP;
}

/* make_screening_lists, mod_electrostatics.F90:538-864 (no FMM split) */
static void make_screening_lists(orc_sys *s) {
    lbuild_t b;
    /* P-P list, rows over polarizable sites (:655-710) */
    lb_init(&b, s->npol);
    for (int ip = 0; ip < s->npol; ip++) {
        b.ri[ip] = b.nnz;
        int i = s->polar_mm[ip];
        for (int ineigh = 0; ineigh < 4; ineigh++) {
            const csr_t *c = &s->conn[ineigh];
            for (int k = c->ri[i]; k < c->ri[i + 1]; k++) {
                int jp = s->mm_polar[c->ci[k]];
                if (jp >= 0) {
                    double sc = screening_rules(s, ip, 'P', jp, 'P', '-');
                    if (fabs(sc - 1.0) > EPS_RP) lb_push(&b, jp, sc);
                }
            }
        }
    }
    lb_finish(&b, &s->PP);
    /* S-P list for the P field (:712-766) */
    lb_init(&b, s->mm);
    for (int i = 0; i < s->mm; i++) {
        b.ri[i] = b.nnz;
        for (int ineigh = 0; ineigh < 4; ineigh++) {
            const csr_t *c = &s->conn[ineigh];
            for (int k = c->ri[i]; k < c->ri[i + 1]; k++) {
                int jp = s->mm_polar[c->ci[k]];
                if (jp >= 0) {
                    double sc = screening_rules(s, i, 'S', jp, 'P', 'P');
                    if (fabs(sc - 1.0) > EPS_RP) lb_push(&b, jp, sc);
                }
            }
        }
    }
    lb_finish(&b, &s->sPP);
    /* S-P list for the D field (AMOEBA only, :768-857) */
    if (s->amoeba) {
        lb_init(&b, s->mm);
        for (int i = 0; i < s->mm; i++) {
            b.ri[i] = b.nnz;
            int pg_i = s->grp[i];
            for (int ineigh = 0; ineigh < 4; ineigh++) {
                const csr_t *pc = &s->pg_conn[ineigh];
                for (int ig = pc->ri[pg_i]; ig < pc->ri[pg_i + 1]; ig++) {
                    int g = pc->ci[ig];
                    for (int a = s->grp_atoms.ri[g]; a < s->grp_atoms.ri[g + 1]; a++) {
                        int jp = s->mm_polar[s->grp_atoms.ci[a]];
                        if (jp >= 0) {
                            double sc = screening_rules(s, i, 'S', jp, 'P', 'D');
                            if (fabs(sc - 1.0) > EPS_RP) lb_push(&b, jp, sc);
                        }
                    }
                }
            }
        }
        lb_finish(&b, &s->sPD);
    }
}

/* ------------------------------------------------------------------ */
/* .mmp loader + mmpol_prepare                                         */
/* ------------------------------------------------------------------ */
static void sort_ints(int *a, int n) {
    for (int i = 1; i < n; i++) {
        int v = a[i], j = i - 1;
        while (j >= 0 && a[j] > v) {
            a[j + 1] = a[j];
            j--;
        }
        a[j + 1] = v;
    }
}

static int prepare(orc_sys *s, const int *i12);

orc_sys *orc_init_mmp(const char *path) {
    g_err[0] = 0;
    FILE *f = fopen(path, "r");
    if (!f) {
        set_err("Input file '%s' does not exist.", path);
        return NULL;
    }
    rdr_t r = {f, NULL, 0, 0};
    double v[MAXPGP];
    orc_sys *s = NULL;
    int *i12 = NULL;
    int ok = 0;
    int rev, fft, rules, mm;
    if (!rd_values(&r, v, 1)) goto done;
    rev = (int)v[0];
    if (rev != 2 && rev != 3) {
        set_err("MMP file is only supported with version 2 or 3.");
        goto done;
    }
    if (!rd_skip(&r, 2) || !rd_values(&r, v, 1)) goto done;
    fft = (int)v[0];
    if (!rd_values(&r, v, 1)) goto done;
    rules = (int)v[0];
    if (!rd_skip(&r, rev == 3 ? 17 : 15) || !rd_values(&r, v, 1)) goto done;
    mm = (int)v[0];
    if (mm <= 0) {
        set_err("invalid number of MM atoms");
        goto done;
    }
    s = xcalloc(1, sizeof(orc_sys));
    s->amoeba = (fft == 1);
    s->mm = mm;
    s->ld_cart = s->amoeba ? 10 : 1;
    s->n_ipd = s->amoeba ? 2 : 1;
    s->cmm = xcalloc(3 * mm, sizeof(double));
    s->q = xcalloc((size_t)s->ld_cart * mm, sizeof(double));
    s->q0 = xcalloc((size_t)s->ld_cart * mm, sizeof(double));
    double *polin = xcalloc(mm, sizeof(double));
    if (!rd_skip(&r, mm + 1)) goto done;
    for (int i = 0; i < mm; i++)
        if (!rd_values(&r, &s->cmm[3 * i], 3)) goto done;
    if (!rd_skip(&r, mm)) goto done;
    for (int i = 0; i < mm; i++)
        if (!rd_values(&r, &s->q[(size_t)s->ld_cart * i], s->ld_cart)) goto done;
    for (int i = 0; i < mm; i++)
        if (!rd_values(&r, &polin[i], 1)) goto done;
    /* polarizable atoms: pol > 1e-8 (mod_inputloader.F90:155-163) */
    int npol = 0;
    int *plist = xcalloc(mm, sizeof(int));
    for (int i = 0; i < mm; i++)
        if (polin[i] > 1e-8) plist[npol++] = i;
    s->npol = npol;
    s->pol = xcalloc(npol, sizeof(double));
    s->polar_mm = plist;
    for (int k = 0; k < npol; k++) {
        s->pol[k] = polin[plist[k]];
        if (s->amoeba) s->pol[k] *= ANG2AU * ANG2AU * ANG2AU;
    }
    free(polin);
    for (int i = 0; i < 3 * mm; i++) s->cmm[i] *= ANG2AU;
    /* screening parameters (mod_constants.F90:37-52, mod_inputloader.F90:175-200) */
    if (s->amoeba) {
        double m[4] = {0, 0, 0.4, 0.8}, p[4] = {0, 0, 1, 1}, d[4] = {0, 1, 1, 1},
               u[4] = {1, 1, 1, 1}, pi[4] = {0, 0, 0.5, 1};
        memcpy(s->mscale, m, sizeof m);
        memcpy(s->pscale, p, sizeof p);
        memcpy(s->dscale, d, sizeof d);
        memcpy(s->uscale, u, sizeof u);
        memcpy(s->pscale_intra, pi, sizeof pi);
        s->thole_scale = 0.0;
    } else if (rules == 1) {
        for (int k = 0; k < 4; k++) s->mscale[k] = s->pscale[k] = s->dscale[k] = s->uscale[k] = 1.0;
        s->thole_scale = 2.0580;
    } else {
        double a[4] = {0, 0, 1, 1};
        memcpy(s->mscale, a, sizeof a);
        memcpy(s->pscale, a, sizeof a);
        memcpy(s->dscale, a, sizeof a);
        memcpy(s->uscale, a, sizeof a);
        s->thole_scale = 2.5874;
    }
    /* 1-2 connectivity (adj_mat_from_conn, mod_adjacency_mat.F90:126-166) */
    i12 = xcalloc((size_t)MAXN12 * mm, sizeof(int));
    for (int i = 0; i < mm; i++) {
        int tmp[MAXN12];
        if (!rd_ints(&r, tmp, MAXN12)) goto done;
        for (int k = 0; k < MAXN12; k++) i12[MAXN12 * i + k] = tmp[k];
    }
    s->grp = xcalloc(mm, sizeof(int));
    s->frame = xcalloc(mm, sizeof(int));
    s->iz = xcalloc(mm, sizeof(int));
    s->ix = xcalloc(mm, sizeof(int));
    s->iy = xcalloc(mm, sizeof(int));
    if (s->amoeba) {
        /* polgroup11_to_mm2pg, mod_inputloader.F90:259-295 */
        for (int i = 0; i < mm; i++) s->grp[i] = -1;
        int ipg = 0;
        int *row = xcalloc(MAXPGP, sizeof(int));
        int *rows = xcalloc((size_t)MAXPGP * mm, sizeof(int));
        for (int i = 0; i < mm; i++) {
            if (!rd_ints(&r, row, MAXPGP)) {
                free(row);
                free(rows);
                goto done;
            }
            memcpy(&rows[(size_t)MAXPGP * i], row, MAXPGP * sizeof(int));
        }
        for (int i = 0; i < mm; i++) {
            if (s->grp[i] == -1) {
                for (int k = 0; k < MAXPGP; k++) {
                    int a = rows[(size_t)MAXPGP * i + k];
                    if (a == 0) break;
                    if (a < 1 || a > mm || s->grp[a - 1] != -1) {
                        free(row);
                        free(rows);
                        set_err("Unexpected error in polgroup11_to_mm2pg");
                        goto done;
                    }
                    s->grp[a - 1] = ipg;
                }
                ipg++;
            }
        }
        free(row);
        free(rows);
        for (int i = 0; i < mm; i++)
            if (s->grp[i] < 0) {
                set_err("Unexpected error in polgroup11_to_mm2pg");
                goto done;
            }
        s->ngrp = ipg;
        for (int i = 0; i < mm; i++) {
            int t[4];
            if (!rd_ints(&r, t, 4)) goto done;
            s->frame[i] = t[0];
            s->iz[i] = t[1] - 1;
            s->ix[i] = t[2] - 1;
            s->iy[i] = t[3] - 1;
        }
    }
    ok = 1;
done:
    if (r.line) free(r.line);
    fclose(f);
    if (!ok) {
        if (!g_err[0]) set_err("error while reading MMP file '%s'", path);
        if (s) orc_free(s);
        free(i12);
        return NULL;
    }
    if (prepare(s, i12)) {
        free(i12);
        orc_free(s);
        return NULL;
    }
    free(i12);
    return s;
}

/* mmpol_prepare, mod_mmpol.F90:139-237 */
static int prepare(orc_sys *s, const int *i12) {
    int mm = s->mm;
    csr_t adj;
    adj.n = mm;
    adj.ri = xcalloc(mm + 1, sizeof(int));
    adj.ci = xcalloc((size_t)MAXN12 * mm, sizeof(int));
    int nnz = 0;
    for (int i = 0; i < mm; i++) {
        adj.ri[i] = nnz;
        int row[MAXN12], nr = 0;
        for (int k = 0; k < MAXN12; k++) {
            int a = i12[MAXN12 * i + k];
            if (a != 0) {
                if (a < 1 || a > mm) {
                    set_err("connectivity index out of range");
                    csr_free(&adj);
                    return ORC_ERR_INPUT;
                }
                row[nr++] = a - 1;
            }
        }
        sort_ints(row, nr);
        for (int k = 0; k < nr; k++) adj.ci[nnz++] = row[k];
    }
    adj.ri[mm] = nnz;
    build_conn(&adj, 4, s->conn, 0);
    csr_free(&adj);
    /* remove_null_pol (mod_electrostatics.F90:469-536) */
    {
        int k2 = 0;
        for (int k = 0; k < s->npol; k++)
            if (fabs(s->pol[k]) > EPS_RP) {
                s->pol[k2] = s->pol[k];
                s->polar_mm[k2] = s->polar_mm[k];
                k2++;
            }
        s->npol = k2;
    }
    s->mm_polar = xcalloc(mm, sizeof(int));
    for (int i = 0; i < mm; i++) s->mm_polar[i] = -1;
    for (int k = 0; k < s->npol; k++) s->mm_polar[s->polar_mm[k]] = k;
    /* thole_init (mod_electrostatics.F90:866-897) */
    s->thole = xcalloc(mm, sizeof(double));
    for (int k = 0; k < s->npol; k++) s->thole[s->polar_mm[k]] = pow(s->pol[k], 1.0 / 6.0);
    if (!s->amoeba) {
        if (s->thole_scale > EPS_RP) {
            double sq = sqrt(s->thole_scale);
            for (int i = 0; i < mm; i++) s->thole[i] *= sq;
        } else {
            set_err("Scale factor for Thole damping should be greater than 0.0");
            return ORC_ERR_INPUT;
        }
    }
    s->thole_damping = xcalloc(s->npol, sizeof(double));
    for (int k = 0; k < s->npol; k++) s->thole_damping[k] = s->amoeba ? 0.39 : 0.0;
    if (s->amoeba) {
        memcpy(s->q0, s->q, sizeof(double) * 10 * mm);
        for (int i = 0; i < mm; i++)
            for (int k = 4; k < 10; k++) s->q0[10 * i + k] /= 3.0;
        /* reverse_grp_tab (mod_adjacency_mat.F90:424-493) */
        int ng = s->ngrp;
        s->grp_atoms.n = ng;
        s->grp_atoms.ri = xcalloc(ng + 1, sizeof(int));
        s->grp_atoms.ci = xcalloc(mm, sizeof(int));
        int *cnt = xcalloc(ng, sizeof(int));
        for (int i = 0; i < mm; i++) cnt[s->grp[i]]++;
        for (int g = 0; g < ng; g++) s->grp_atoms.ri[g + 1] = s->grp_atoms.ri[g] + cnt[g];
        memset(cnt, 0, ng * sizeof(int));
        for (int i = 0; i < mm; i++) {
            int g = s->grp[i];
            s->grp_atoms.ci[s->grp_atoms.ri[g] + cnt[g]++] = i;
        }
        free(cnt);
        /* build_pg_adjacency_matrix (mod_mmpol.F90:272-323) */
        csr_t pga;
        pga.n = ng;
        pga.ri = xcalloc(ng + 1, sizeof(int));
        int cap = 2 * ng + 16;
        pga.ci = xcalloc(cap, sizeof(int));
        int pn = 0;
        for (int g = 0; g < ng; g++) {
            pga.ri[g] = pn;
            for (int a = s->grp_atoms.ri[g]; a < s->grp_atoms.ri[g + 1]; a++) {
                int a1 = s->grp_atoms.ci[a];
                const csr_t *c1 = &s->conn[0];
                for (int l = c1->ri[a1]; l < c1->ri[a1 + 1]; l++) {
                    int a2 = c1->ci[l];
                    int g2 = s->grp[a2];
                    if (g2 == s->grp[a1]) continue;
                    int dup = 0;
                    for (int t = pga.ri[g]; t < pn; t++)
                        if (pga.ci[t] == g2) dup = 1;
                    if (dup) continue;
                    if (pn == cap) {
                        cap *= 2;
                        pga.ci = realloc(pga.ci, cap * sizeof(int));
                    }
                    pga.ci[pn++] = g2;
                }
            }
        }
        pga.ri[ng] = pn;
        build_conn(&pga, 3, s->pg_conn, 1);
        csr_free(&pga);
        int st = rotate_multipoles(s);
        if (st) return st;
    } else {
        memcpy(s->q0, s->q, sizeof(double) * mm);
    }
    make_screening_lists(s);
    s->e_m2d = xcalloc((size_t)3 * s->npol * s->n_ipd, sizeof(double));
    s->ipd = xcalloc((size_t)3 * s->npol * s->n_ipd, sizeof(double));
    s->def_solver = SOLVER_CG;
    s->def_matv = MATV_DIRECT;
    s->tol = 1e-8;
    s->maxiter = 200;
    s->diis_max = 20;
    return 0;
}

void orc_free(orc_sys *s) {
    if (!s) return;
    free(s->cmm);
    free(s->q0);
    free(s->q);
    free(s->pol);
    free(s->polar_mm);
    free(s->mm_polar);
    free(s->thole);
    free(s->thole_damping);
    free(s->grp);
    free(s->frame);
    free(s->iz);
    free(s->ix);
    free(s->iy);
    for (int k = 0; k < 4; k++) {
        csr_free(&s->conn[k]);
        csr_free(&s->pg_conn[k]);
    }
    csr_free(&s->grp_atoms);
    slist_t *ls[3] = {&s->sPP, &s->sPD, &s->PP};
    for (int k = 0; k < 3; k++) {
        csr_free(&ls[k]->m);
        free(ls[k]->scale);
        free(ls[k]->todo);
    }
    free(s->e_m2d);
    free(s->ipd);
    free(s->tmat);
    free(s);
}

int32_t orc_mm_atoms(const orc_sys *s) { return s->mm; }
int32_t orc_pol_atoms(const orc_sys *s) { return s->npol; }
int32_t orc_n_ipd(const orc_sys *s) { return s->n_ipd; }
int32_t orc_is_amoeba(const orc_sys *s) { return s->amoeba; }
int32_t orc_ld_cart(const orc_sys *s) { return s->ld_cart; }
void orc_set_tol(orc_sys *s, double tol) { s->tol = tol; }
void orc_set_maxiter(orc_sys *s, int32_t n) { s->maxiter = n; }
void orc_set_default_solver(orc_sys *s, int32_t v) { s->def_solver = v; }
void orc_set_default_matv(orc_sys *s, int32_t v) { s->def_matv = v; }
void orc_get_cmm(const orc_sys *s, double *o) { memcpy(o, s->cmm, sizeof(double) * 3 * s->mm); }
void orc_get_q(const orc_sys *s, double *o) {
    memcpy(o, s->q, sizeof(double) * s->ld_cart * s->mm);
}
void orc_get_pol(const orc_sys *s, double *o) { memcpy(o, s->pol, sizeof(double) * s->npol); }
void orc_get_polar_mm(const orc_sys *s, int32_t *o) {
    for (int k = 0; k < s->npol; k++) o[k] = s->polar_mm[k];
}
void orc_get_thole(const orc_sys *s, double *o) { memcpy(o, s->thole, sizeof(double) * s->mm); }
void orc_get_ipd(const orc_sys *s, double *o) {
    memcpy(o, s->ipd, sizeof(double) * 3 * s->npol * s->n_ipd);
}
int32_t orc_screening_nnz(const orc_sys *s, int32_t which) {
    const slist_t *l = which == 0 ? &s->sPP : which == 1 ? &s->sPD : &s->PP;
    if (!l->m.ri) return 0;
    return l->m.ri[l->m.n];
}
void orc_get_screening(const orc_sys *s, int32_t which, int32_t *ri, int32_t *ci, double *sc) {
    const slist_t *l = which == 0 ? &s->sPP : which == 1 ? &s->sPD : &s->PP;
    if (!l->m.ri) return;
    int nnz = l->m.ri[l->m.n];
    for (int i = 0; i <= l->m.n; i++) ri[i] = l->m.ri[i];
    for (int k = 0; k < nnz; k++) {
        ci[k] = l->m.ci[k];
        sc[k] = l->scale[k];
    }
}
void orc_clear_guess(orc_sys *s) { s->ipd_use_guess = 0; }

/* ------------------------------------------------------------------ */
/* kernels                                                             */
/* ------------------------------------------------------------------ */
/* damped_coulomb_kernel(eel, i, j, maxder, res, dr), mm indices;
 * dr = c_j - c_i; res[k] = damped r^-(2k+1).  :1018-1095 */
static int damped_kernel(const orc_sys *s, int i, int j, int maxder, double *res, double *dr) {
    double sij = s->thole[i] * s->thole[j];
    int pi = s->mm_polar[i], pj = s->mm_polar[j];
    double a;
    if (pi >= 0 && pj >= 0) {
        a = fmin(s->thole_damping[pi], s->thole_damping[pj]);
    } else if (pi >= 0) {
        a = s->thole_damping[pi];
    } else if (pj >= 0) {
        a = s->thole_damping[pj];
    } else {
        return ORC_ERR_NUMERIC;
    }
    for (int k = 0; k < 3; k++) dr[k] = s->cmm[3 * j + k] - s->cmm[3 * i + k];
    double nr = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
    if (nr < EPS_RP) return ORC_ERR_NUMERIC;
    res[0] = 1.0 / nr;
    double inv2 = res[0] * res[0];
    for (int k = 1; k <= maxder; k++) res[k] = res[k - 1] * inv2;
    if (fabs(sij) < EPS_RP) return 0;
    double u = 1.0 / (res[0] * sij);
    double u3 = u * u * u;
    if (s->amoeba && u3 * a < 50.0) {
        double fexp = -a * u3;
        double eexp = exp(fexp);
        if (maxder >= 1) res[1] *= 1.0 - eexp;
        if (maxder >= 2) res[2] *= 1.0 - (1.0 - fexp) * eexp;
        if (maxder >= 3) res[3] *= 1.0 - (1.0 - fexp + 0.6 * fexp * fexp) * eexp;
        if (maxder >= 4)
            res[4] *= 1.0 - (1.0 - fexp + 18.0 / 35.0 * fexp * fexp - 9.0 / 35.0 * fexp * fexp * fexp) * eexp;
    } else if (!s->amoeba && res[0] > 1.0 / sij) {
        double u4 = u3 * u;
        if (maxder >= 1) res[1] *= 4.0 * u3 - 3.0 * u4;
        if (maxder >= 2) res[2] *= u4;
        if (maxder >= 3) res[3] *= 0.2 * u4;
    }
    return 0;
}

static inline int list_find(const slist_t *l, int row, int col) {
    for (int k = l->m.ri[row]; k < l->m.ri[row + 1]; k++)
        if (l->m.ci[k] == col) return k;
    return -1;
}

/* elec_prop_M2D, direct path, E only (mod_electrostatics.F90:2579-2731) */
static int elec_prop_m2d(orc_sys *s) {
    int npol = s->npol, mm = s->mm;
    int bad = 0;
    memset(s->e_m2d, 0, sizeof(double) * 3 * npol * s->n_ipd);
    double *eD = s->e_m2d;                    /* set 1 = D (or the only set) */
    double *eP = s->amoeba ? s->e_m2d + 3 * npol : s->e_m2d;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : bad)
    for (int j = 0; j < npol; j++) {
        int jm = s->polar_mm[j];
        for (int i = 0; i < mm; i++) {
            if (i == jm) continue;
            if (s->amoeba) {
                int kp = list_find(&s->sPP, i, j);
                int todo_p = 1, todo_d = 1;
                double sp = 1.0, sd = 1.0;
                if (kp >= 0) {
                    todo_p = s->sPP.todo[kp];
                    sp = s->sPP.scale[kp];
                }
                int kd = list_find(&s->sPD, i, j);
                if (kd >= 0) {
                    todo_d = s->sPD.todo[kd];
                    sd = s->sPD.scale[kd];
                }
                if (!(todo_p || todo_d)) continue;
                double k[4], dr[3];
                if (damped_kernel(s, i, jm, 3, k, dr)) {
                    bad = 1;
                    continue;
                }
                const double *q = &s->q[10 * i];
                double e[3];
                /* q_elec_prop */
                for (int c = 0; c < 3; c++) e[c] = q[0] * k[1] * dr[c];
                /* mu_elec_prop */
                double mdr = q[1] * dr[0] + q[2] * dr[1] + q[3] * dr[2];
                for (int c = 0; c < 3; c++) e[c] += 3.0 * mdr * dr[c] * k[2] - q[1 + c] * k[1];
                /* quad_elec_prop */
                double qx[3];
                qx[0] = q[4] * dr[0] + q[5] * dr[1] + q[7] * dr[2];
                qx[1] = q[5] * dr[0] + q[6] * dr[1] + q[8] * dr[2];
                qx[2] = q[7] * dr[0] + q[8] * dr[1] + q[9] * dr[2];
                double qxr = qx[0] * dr[0] + qx[1] * dr[1] + qx[2] * dr[2];
                for (int c = 0; c < 3; c++) e[c] += 15.0 * qxr * dr[c] * k[3] - 6.0 * qx[c] * k[2];
                if (todo_p) {
                    if (kp >= 0)
                        for (int c = 0; c < 3; c++) eP[3 * j + c] += e[c] * sp;
                    else
                        for (int c = 0; c < 3; c++) eP[3 * j + c] += e[c];
                }
                if (todo_d) {
                    if (kd >= 0)
                        for (int c = 0; c < 3; c++) eD[3 * j + c] += e[c] * sd;
                    else
                        for (int c = 0; c < 3; c++) eD[3 * j + c] += e[c];
                }
            } else {
                int kp = list_find(&s->sPP, i, j);
                int todo = 1;
                double sc = 1.0;
                if (kp >= 0) {
                    todo = s->sPP.todo[kp];
                    sc = s->sPP.scale[kp];
                }
                if (!todo) continue;
                double k[2], dr[3];
                if (damped_kernel(s, i, jm, 1, k, dr)) {
                    bad = 1;
                    continue;
                }
                double qq = s->q[i];
                for (int c = 0; c < 3; c++) {
                    double e = qq * k[1] * dr[c];
                    eD[3 * j + c] += (kp >= 0) ? e * sc : e;
                }
            }
        }
    }
    if (bad) {
        set_err("Requesting Coulomb kernel for two atoms placed in the same point");
        return ORC_ERR_NUMERIC;
    }
    return 0;
}

/* prepare_polelec (E only), mod_electrostatics.F90:1487-1596 */
static int prepare_polelec(orc_sys *s) {
    if (s->m2d_done) return 0;
    int st = elec_prop_m2d(s);
    if (st) return st;
    s->m2d_done = 1;
    return 0;
}

int orc_get_e_m2d(orc_sys *s, double *out) {
    int st = prepare_polelec(s);
    if (st) return st;
    memcpy(out, s->e_m2d, sizeof(double) * 3 * s->npol * s->n_ipd);
    return 0;
}

/* field of dipole i at target j, for the D2D field: returns 1 if computed */
static inline int d2d_pair(const orc_sys *s, const double *x, int i, int j, double *e, int *bad) {
    int to_do = 1;
    double scalf = 1.0;
    int k = list_find(&s->PP, i, j);
    if (k >= 0) {
        to_do = s->PP.todo[k];
        scalf = s->PP.scale[k];
    }
    if (!to_do) return 0;
    double ker[3], dr[3];
    if (damped_kernel(s, s->polar_mm[i], s->polar_mm[j], 2, ker, dr)) {
        *bad = 1;
        return 0;
    }
    const double *mu = &x[3 * i];
    double mdr = mu[0] * dr[0] + mu[1] * dr[1] + mu[2] * dr[2];
    for (int c = 0; c < 3; c++) {
        double t = 3.0 * mdr * dr[c] * ker[2] - mu[c] * ker[1];
        e[c] += (k >= 0) ? t * scalf : t;
    }
    return 1;
}

/* field_extD2D direct (mod_electrostatics.F90:2068-2109), E += */
static int field_extd2d(const orc_sys *s, const double *x, double *E) {
    int n = s->npol, bad = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : bad)
    for (int j = 0; j < n; j++) {
        double e[3] = {0, 0, 0};
        for (int i = 0; i < n; i++) {
            if (i == j) continue;
            d2d_pair(s, x, i, j, e, &bad);
        }
        for (int c = 0; c < 3; c++) E[3 * j + c] += e[c];
    }
    if (bad) {
        set_err("Requesting Coulomb kernel for two atoms placed in the same point");
        return ORC_ERR_NUMERIC;
    }
    return 0;
}

/* dipole_T (mod_polarization.F90:327-387), 3x3 block (row=target comp) */
static int dipole_t(const orc_sys *s, int i, int j, double t[3][3]) {
    memset(t, 0, 9 * sizeof(double));
    if (i == j) {
        for (int a = 0; a < 3; a++) t[a][a] = 1.0 / s->pol[i];
        return 0;
    }
    double scalf = screening_rules(s, i, 'P', j, 'P', '-');
    if (fabs(scalf) > EPS_RP) {
        double ker[3], dr[3];
        if (damped_kernel(s, s->polar_mm[i], s->polar_mm[j], 2, ker, dr)) return ORC_ERR_NUMERIC;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                if (a == b)
                    t[a][a] = ker[1] - 3.0 * ker[2] * dr[a] * dr[a];
                else
                    t[b][a] = -3.0 * ker[2] * dr[a] * dr[b];
            }
        if (fabs(scalf - 1.0) > EPS_RP)
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) t[a][b] *= scalf;
    }
    return 0;
}

/* create_tmat (mod_polarization.F90:389-435); column-major n x n */
static int create_tmat(orc_sys *s) {
    if (s->tmat) return 0;
    int np = s->npol, n = 3 * np, bad = 0;
    s->tmat = xcalloc((size_t)n * n, sizeof(double));
#pragma omp parallel for schedule(dynamic) reduction(| : bad)
    for (int i = 0; i < np; i++) {
        for (int j = 0; j <= i; j++) {
            double t[3][3];
            if (dipole_t(s, i, j, t)) {
                bad = 1;
                continue;
            }
            for (int ii = 0; ii < 3; ii++)
                for (int jj = 0; jj < 3; jj++) {
                    /* tmat((j-1)*3+jj, (i-1)*3+ii) = tensor(jj, ii) and its transpose */
                    s->tmat[(size_t)(3 * i + ii) * n + (3 * j + jj)] = t[jj][ii];
                    s->tmat[(size_t)(3 * j + jj) * n + (3 * i + ii)] = t[jj][ii];
                }
        }
    }
    if (bad) {
        free(s->tmat);
        s->tmat = NULL;
        set_err("Requesting Coulomb kernel for two atoms placed in the same point");
        return ORC_ERR_NUMERIC;
    }
    return 0;
}

/* TMatVec_otf / TMatVec_incore + TMatVec_diag (mod_polarization.F90:437-504) */
static int matvec(orc_sys *s, int matv, const double *x, double *y, int dodiag) {
    int np = s->npol, n = 3 * np;
    s->matvecs++;
    if (matv == MATV_INCORE) {
        int st = create_tmat(s);
        if (st) return st;
#pragma omp parallel for schedule(static)
        for (int r = 0; r < n; r++) {
            double acc = 0.0;
            for (int c = 0; c < n; c++) acc += s->tmat[(size_t)c * n + r] * x[c];
            y[r] = acc - s->tmat[(size_t)r * n + r] * x[r];
        }
    } else {
        memset(y, 0, sizeof(double) * n);
        int st = field_extd2d(s, x, y);
        if (st) return st;
        for (int k = 0; k < n; k++) y[k] = -y[k];
    }
    if (dodiag)
        for (int k = 0; k < n; k++) y[k] += x[k] / s->pol[k / 3];
    return 0;
}

int orc_tmatvec(orc_sys *s, const double *x, double *y, int32_t dodiag, int32_t matv) {
    if (matv == MATV_NONE) matv = s->def_matv;
    return matvec(s, matv, x, y, dodiag);
}

int orc_tmatvec_rows(orc_sys *s, const double *x, const int32_t *rows, int32_t nrows, double *y) {
    int bad = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : bad)
    for (int r = 0; r < nrows; r++) {
        int j = rows[r];
        double e[3] = {0, 0, 0};
        for (int i = 0; i < s->npol; i++) {
            if (i == j) continue;
            d2d_pair(s, x, i, j, e, &bad);
        }
        for (int c = 0; c < 3; c++) y[3 * r + c] = -e[c] + x[3 * j + c] / s->pol[j];
    }
    return bad ? ORC_ERR_NUMERIC : 0;
}

static double dot(const double *a, const double *b, int n) {
    double acc = 0.0;
    for (int k = 0; k < n; k++) acc += a[k] * b[k];
    return acc;
}

/* conjugate_gradient_solver (mod_solvers.F90:86-216) */
static int cg_solve(orc_sys *s, int matv, int set, const double *rhs, double *x) {
    int np = s->npol, n = 3 * np;
    double *r = xcalloc(n, sizeof(double)), *p = xcalloc(n, sizeof(double));
    double *h = xcalloc(n, sizeof(double)), *z = xcalloc(n, sizeof(double));
    double tol = s->tol;
    int st = 0;
    s->hist_n[set] = 0;
    s->last_iters[set] = 0;
    double rms = dot(x, x, n);
    if (rms < EPS_RP) {
        /* precnd(eel, x, x): alpha * x */
        for (int k = 0; k < n; k++) x[k] = s->pol[k / 3] * x[k];
    }
    if ((st = matvec(s, matv, x, z, 1))) goto out;
    for (int k = 0; k < n; k++) r[k] = rhs[k] - z[k];
    for (int k = 0; k < n; k++) z[k] = s->pol[k / 3] * r[k];
    memcpy(p, z, sizeof(double) * n);
    double gold = dot(r, z, n), gama = 0.0, gnew;
    for (int it = 1; it <= s->maxiter; it++) {
        if ((st = matvec(s, matv, p, h, 1))) goto out;
        gama = dot(h, p, n);
        if (fabs(gama) < EPS_RP) break;
        double alpha = gold / gama;
        for (int k = 0; k < n; k++) {
            x[k] += alpha * p[k];
            r[k] -= alpha * h[k];
        }
        for (int k = 0; k < n; k++) z[k] = s->pol[k / 3] * r[k];
        gnew = dot(r, z, n);
        rms = sqrt(gnew / (double)n);
        if (s->hist_n[set] < MAX_HIST) s->hist[set][s->hist_n[set]++] = rms;
        s->last_iters[set] = it;
        if (rms < tol) break;
        gama = gnew / gold;
        for (int k = 0; k < n; k++) p[k] = gama * p[k] + z[k];
        gold = gnew;
    }
    if (rms > tol && fabs(gama) > EPS_RP) {
        set_err("Iterative solver did not converged");
        st = ORC_ERR_NOT_CONVERGED;
    }
out:
    free(r);
    free(p);
    free(h);
    free(z);
    return st;
}

/* LU with partial pivoting (dgesv semantics: info != 0 on a zero pivot);
 * a is column-major n x n, solves in place for one rhs */
static int lu_solve(int n, double *a, double *b) {
    int *piv = xcalloc(n, sizeof(int));
    int info = 0;
    for (int k = 0; k < n; k++) {
        int pr = k;
        double mx = fabs(a[(size_t)k * n + k]);
        for (int r = k + 1; r < n; r++) {
            double v = fabs(a[(size_t)k * n + r]);
            if (v > mx) {
                mx = v;
                pr = r;
            }
        }
        piv[k] = pr;
        if (a[(size_t)k * n + pr] == 0.0) {
            info = k + 1;
            break;
        }
        if (pr != k) {
            for (int c = 0; c < n; c++) {
                double t = a[(size_t)c * n + k];
                a[(size_t)c * n + k] = a[(size_t)c * n + pr];
                a[(size_t)c * n + pr] = t;
            }
            double t = b[k];
            b[k] = b[pr];
            b[pr] = t;
        }
        double d = a[(size_t)k * n + k];
        for (int r = k + 1; r < n; r++) a[(size_t)k * n + r] /= d;
        for (int c = k + 1; c < n; c++) {
            double f = a[(size_t)c * n + k];
            if (f != 0.0)
                for (int r = k + 1; r < n; r++) a[(size_t)c * n + r] -= a[(size_t)k * n + r] * f;
        }
    }
    if (!info) {
        for (int k = 0; k < n; k++)
            for (int r = k + 1; r < n; r++) b[r] -= a[(size_t)k * n + r] * b[k];
        for (int k = n - 1; k >= 0; k--) {
            b[k] /= a[(size_t)k * n + k];
            for (int r = 0; r < k; r++) b[r] -= a[(size_t)k * n + r] * b[k];
        }
    }
    free(piv);
    return info;
}

/* diis + makeb (mod_solvers.F90:367-469); b is (ndiis+1)^2 column-major */
static void diis_step(int n, int *nmat, int ndiis, double *xd, double *ed, double *b,
                      double *xnew) {
    int ld = ndiis + 1;
#define B(r, c) b[(size_t)(c) * ld + (r)]
    if (*nmat >= ndiis) {
        for (int j = 2; j <= *nmat - 10; j++)
            for (int k = 2; k <= *nmat - 10; k++) B(j - 1, k - 1) = B(j + 10 - 1, k + 10 - 1);
        for (int j = 1; j <= *nmat - 10; j++) {
            memcpy(&xd[(size_t)(j - 1) * n], &xd[(size_t)(j + 10 - 1) * n], sizeof(double) * n);
            memcpy(&ed[(size_t)(j - 1) * n], &ed[(size_t)(j + 10 - 1) * n], sizeof(double) * n);
        }
        *nmat -= 10;
    }
    int nm = *nmat, nm1 = nm + 1;
    /* makeb */
    if (nm == 1) {
        B(0, 0) = 0.0;
        B(0, 1) = 1.0;
        B(1, 0) = 1.0;
        B(1, 1) = dot(&ed[0], &ed[0], n);
    } else {
        B(nm, 0) = 1.0;
        B(0, nm) = 1.0;
        for (int i = 1; i <= nm - 1; i++) {
            double bij = dot(&ed[(size_t)(i - 1) * n], &ed[(size_t)(nm - 1) * n], n);
            B(nm, i) = bij;
            B(i, nm) = bij;
        }
        B(nm, nm) = dot(&ed[(size_t)(nm - 1) * n], &ed[(size_t)(nm - 1) * n], n);
    }
    double *bloc = xcalloc((size_t)nm1 * nm1, sizeof(double));
    double *cex = xcalloc(nm1, sizeof(double));
    for (int c = 0; c < nm1; c++)
        for (int r = 0; r < nm1; r++) bloc[(size_t)c * nm1 + r] = B(r, c);
    cex[0] = 1.0;
    int info = lu_solve(nm1, bloc, cex);
    if (info != 0) {
        *nmat = 1;
    } else {
        memset(xnew, 0, sizeof(double) * n);
        for (int i = 1; i <= nm; i++)
            for (int k = 0; k < n; k++) xnew[k] += cex[i] * xd[(size_t)(i - 1) * n + k];
        *nmat = nm + 1;
    }
    free(bloc);
    free(cex);
#undef B
}

/* jacobi_diis_solver (mod_solvers.F90:218-365) */
static int diis_solve(orc_sys *s, int matv, int set, const double *rhs, double *x) {
    int np = s->npol, n = 3 * np, ndiis = s->diis_max;
    double *xnew = xcalloc(n, sizeof(double)), *y = xcalloc(n, sizeof(double));
    double *xd = xcalloc((size_t)n * ndiis, sizeof(double));
    double *ed = xcalloc((size_t)n * ndiis, sizeof(double));
    double *b = xcalloc((size_t)(ndiis + 1) * (ndiis + 1), sizeof(double));
    int nmat = 1, st = 0;
    double rms, mx = 0.0;
    s->hist_n[set] = 0;
    s->last_iters[set] = 0;
    rms = dot(x, x, n);
    if (rms < EPS_RP)
        for (int k = 0; k < n; k++) x[k] = s->pol[k / 3] * rhs[k];
    for (int it = 1; it <= s->maxiter; it++) {
        if ((st = matvec(s, matv, x, y, 0))) goto out;
        for (int k = 0; k < n; k++) y[k] = rhs[k] - y[k];
        for (int k = 0; k < n; k++) xnew[k] = s->pol[k / 3] * y[k];
        if (ndiis > 0) {
            memcpy(&xd[(size_t)(nmat - 1) * n], xnew, sizeof(double) * n);
            for (int k = 0; k < n; k++) ed[(size_t)(nmat - 1) * n + k] = xnew[k] - x[k];
            diis_step(n, &nmat, ndiis, xd, ed, b, xnew);
        }
        double acc = 0.0;
        mx = 0.0;
        for (int k = 0; k < n; k++) {
            double d = xnew[k] - x[k];
            if (fabs(d) > mx) mx = fabs(d);
            acc += d * d;
        }
        rms = sqrt(acc / (double)n);
        memcpy(x, xnew, sizeof(double) * n);
        if (s->hist_n[set] < MAX_HIST) s->hist[set][s->hist_n[set]++] = mx;
        s->last_iters[set] = it;
        if (mx < s->tol) break;
    }
    if (mx > s->tol) {
        set_err("Iterative solver did not converged");
        st = ORC_ERR_NOT_CONVERGED;
    }
out:
    free(xnew);
    free(y);
    free(xd);
    free(ed);
    free(b);
    return st;
}

/* inversion_solver (mod_solvers.F90:41-84): x = T^-1 rhs */
static int inversion_solve(orc_sys *s, const double *rhs, double *x) {
    int n = 3 * s->npol;
    double *a = xcalloc((size_t)n * n, sizeof(double));
    memcpy(a, s->tmat, sizeof(double) * (size_t)n * n);
    memcpy(x, rhs, sizeof(double) * n);
    int info = lu_solve(n, a, x);
    free(a);
    if (info) {
        set_err("inversion solver: singular matrix");
        return ORC_ERR_NUMERIC;
    }
    return 0;
}

/* polarization (mod_polarization.F90:49-313); e: [n_ipd][npol][3] */
static int polarization(orc_sys *s, const double *e, int solver, int mv, const int *mask_in) {
    int np = s->npol, n = 3 * np;
    s->matvecs = 0;
    if (np == 0) return 0;
    if (solver == SOLVER_NONE) solver = s->def_solver;
    if (mv == MATV_NONE) mv = s->def_matv;
    int mask[2] = {1, 1};
    if (mask_in && s->n_ipd > 1) {
        mask[0] = mask_in[0];
        mask[1] = mask_in[1];
    }
    if (mv == MATV_INCORE || solver == SOLVER_INVERSION) {
        int st = create_tmat(s);
        if (st) return st;
    }
    double *x = xcalloc((size_t)n * s->n_ipd, sizeof(double));
    int st = 0;
    if (solver != SOLVER_INVERSION) {
        if (s->ipd_use_guess) {
            for (int k = 0; k < s->n_ipd; k++)
                if (mask[k]) memcpy(&x[(size_t)k * n], &s->ipd[(size_t)k * n], sizeof(double) * n);
        }
        if (mv != MATV_INCORE && mv != MATV_DIRECT) {
            set_err("Unknown matrix-vector method requested");
            free(x);
            return ORC_ERR_BAD_ARG;
        }
    }
    if (solver == SOLVER_CG || solver == SOLVER_DIIS) {
        int (*fn)(orc_sys *, int, int, const double *, double *) =
            solver == SOLVER_CG ? cg_solve : diis_solve;
        s->last_iters[0] = s->last_iters[1] = 0;
        if (s->amoeba) {
            if (mask[0]) st = fn(s, mv, 0, &e[0], &x[0]);
            if (!st && mask[0] && mask[1] && !s->ipd_use_guess) memcpy(&x[n], &x[0], sizeof(double) * n);
            if (!st && mask[1]) st = fn(s, mv, 1, &e[n], &x[n]);
        } else {
            st = fn(s, mv, 0, e, x);
        }
    } else if (solver == SOLVER_INVERSION) {
        for (int k = 0; k < s->n_ipd && !st; k++)
            if (mask[k]) st = inversion_solve(s, &e[(size_t)k * n], &x[(size_t)k * n]);
    } else {
        set_err("Unknown solver for calculation of the induced point dipoles");
        st = ORC_ERR_BAD_ARG;
    }
    if (!st) {
        memcpy(s->ipd, x, sizeof(double) * n * s->n_ipd);
        s->ipd_done = 1;
        s->ipd_use_guess = 1;
    }
    free(x);
    return st;
}

/* ommp_set_external_field (mod_interface.F90:184-233) */
int orc_set_external_field(orc_sys *s, const double *ext, int32_t solver, int32_t matv,
                           int32_t add_mm) {
    int np = s->npol, n = 3 * np;
    s->ipd_done = 0;
    double *ef = xcalloc((size_t)n * s->n_ipd, sizeof(double));
    int st;
    if (add_mm) {
        st = prepare_polelec(s);
        if (!st) {
            for (int k = 0; k < s->n_ipd; k++)
                for (int c = 0; c < n; c++) ef[(size_t)k * n + c] = s->e_m2d[(size_t)k * n + c] + ext[c];
            /* matv is not forwarded on this path (:222) */
            st = polarization(s, ef, solver, MATV_NONE, NULL);
        }
    } else {
        memcpy(ef, ext, sizeof(double) * n);
        int mask[2] = {1, 0};
        st = polarization(s, ef, solver, matv, mask);
    }
    free(ef);
    return st;
}

/* ommp_get_polelec_energy (mod_interface.F90:343-370) + energy_MM_pol */
double orc_get_polelec_energy(orc_sys *s, int32_t *status) {
    int st = 0;
    double ene = 0.0;
    if (s->npol > 0) {
        if (!s->ipd_done) {
            st = prepare_polelec(s);
            if (!st) st = polarization(s, s->e_m2d, SOLVER_NONE, MATV_NONE, NULL);
        }
        if (!st) {
            int n = 3 * s->npol;
            double e = 0.0;
            if (s->amoeba) {
                /* -1/2 sum ipd(:,:,D) . E_M2D(:,:,P) */
                for (int c = 0; c < 3; c++) {
                    double acc = 0.0;
                    for (int j = 0; j < s->npol; j++) acc += s->ipd[3 * j + c] * s->e_m2d[n + 3 * j + c];
                    e -= acc;
                }
            } else {
                for (int c = 0; c < 3; c++) {
                    double acc = 0.0;
                    for (int j = 0; j < s->npol; j++) acc += s->ipd[3 * j + c] * s->e_m2d[3 * j + c];
                    e -= acc;
                }
            }
            ene = 0.5 * e;
        }
    }
    if (status) *status = st;
    return ene;
}

int32_t orc_last_iterations(const orc_sys *s, int32_t set) { return s->last_iters[set & 1]; }
int64_t orc_matvec_count(const orc_sys *s) { return s->matvecs; }
int32_t orc_residual_history(const orc_sys *s, int32_t set, double *out, int32_t maxn) {
    int k = s->hist_n[set & 1];
    if (k > maxn) k = maxn;
    memcpy(out, s->hist[set & 1], sizeof(double) * k);
    return s->hist_n[set & 1];
}

/* update_coordinates (mod_mmpol.F90:325-371) */
int orc_update_coordinates(orc_sys *s, const double *c) {
    memcpy(s->cmm, c, sizeof(double) * 3 * s->mm);
    s->m2d_done = 0;
    s->ipd_done = 0;
    s->ipd_use_guess = 0;
    free(s->tmat);
    s->tmat = NULL;
    if (s->amoeba) return rotate_multipoles(s);
    return 0;
}

/* ------------------------------------------------------------------ */
/* potential and field at arbitrary points (QM coupling)               */
/* potential_M2E / potential_D2E / field_M2E / field_D2E,              */
/* src/mod_electrostatics.F90:3067-3336, with the undamped             */
/* coulomb_kernel :978-1016 and q/mu/quad_elec_prop :1097-1405; the    */
/* ABI wrappers ommp_{potential,field}_{mmpol,mm,pol}2ext              */
/* (src/mod_interface.F90:250-330) add into the caller's array.         */
/* ------------------------------------------------------------------ */
static int coulomb_kernel(const double *dr, int maxder, double *res) {
    double nr = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
    if (nr < EPS_RP) {
        set_err("Requesting Coulomb kernel for two atoms placed in the same point, this could be an internal "
                "bug or a problem in your input file, please check.");
        return 1;
    }
    res[0] = 1.0 / nr;
    double inv2 = res[0] * res[0];
    for (int k = 1; k <= maxder; k++) res[k] = res[k - 1] * inv2;
    return 0;
}

/* which: 0 = static multipoles + induced dipoles, 1 = static only,
   2 = induced dipoles only; field != 0 selects the field (3 per point) */
static int ext_props(orc_sys *s, int32_t which, int32_t n, const double *cext, double *out, int field) {
    const int do_mm = which == 0 || which == 1, do_pol = which == 0 || which == 2;
    if (do_pol && s->npol > 0 && !s->ipd_done) {
        set_err(field ? "IPD should be computed before computing D2E field."
                      : "IPD should be computed before D2E potential.");
        return ORC_ERR_INPUT;
    }
    const int C = field ? 3 : 1;
    int bad = 0;
    /* the dipoles seen from outside: D (potential) or (P + D) / 2 (field)
       for AMOEBA, the single set otherwise (:3100-3120, :3240-3250) */
    double *mu = NULL;
    if (do_pol && s->npol > 0) {
        mu = xcalloc(3 * (size_t)s->npol, sizeof(double));
        for (int k = 0; k < 3 * s->npol; k++)
            mu[k] = (s->amoeba && field) ? 0.5 * (s->ipd[3 * (size_t)s->npol + k] + s->ipd[k]) : s->ipd[k];
    }
#pragma omp parallel for schedule(dynamic) reduction(| : bad)
    for (int j = 0; j < n; j++) {
        double acc[3] = {0, 0, 0};
        const double *p = &cext[3 * (size_t)j];
        if (do_mm) {
            for (int i = 0; i < s->mm; i++) {
                double dr[3] = {p[0] - s->cmm[3 * i], p[1] - s->cmm[3 * i + 1], p[2] - s->cmm[3 * i + 2]};
                double k[5];
                if (coulomb_kernel(dr, s->amoeba ? (field ? 4 : 2) : (field ? 2 : 1), k)) {
                    bad = 1;
                    continue;
                }
                const double *q = &s->q[(size_t)i * s->ld_cart];
                if (!field) {
                    double v = k[0] * q[0];
                    if (s->amoeba) {
                        double mdr = q[1] * dr[0] + q[2] * dr[1] + q[3] * dr[2];
                        double qx = q[4] * dr[0] + q[5] * dr[1] + q[7] * dr[2];
                        double qy = q[5] * dr[0] + q[6] * dr[1] + q[8] * dr[2];
                        double qz = q[7] * dr[0] + q[8] * dr[1] + q[9] * dr[2];
                        v += mdr * k[1] + 3.0 * (qx * dr[0] + qy * dr[1] + qz * dr[2]) * k[2];
                    }
                    acc[0] += v;
                } else {
                    for (int c = 0; c < 3; c++) acc[c] += q[0] * k[1] * dr[c];
                    if (s->amoeba) {
                        double mdr = q[1] * dr[0] + q[2] * dr[1] + q[3] * dr[2];
                        double qv[3] = {q[4] * dr[0] + q[5] * dr[1] + q[7] * dr[2],
                                        q[5] * dr[0] + q[6] * dr[1] + q[8] * dr[2],
                                        q[7] * dr[0] + q[8] * dr[1] + q[9] * dr[2]};
                        double qxr = qv[0] * dr[0] + qv[1] * dr[1] + qv[2] * dr[2];
                        for (int c = 0; c < 3; c++) {
                            acc[c] += 3.0 * mdr * dr[c] * k[2] - q[1 + c] * k[1];
                            acc[c] += 15.0 * qxr * dr[c] * k[3] - 6.0 * qv[c] * k[2];
                        }
                    }
                }
            }
        }
        if (do_pol) {
            for (int i = 0; i < s->npol; i++) {
                const double *c0 = &s->cmm[3 * (size_t)s->polar_mm[i]];
                double dr[3] = {p[0] - c0[0], p[1] - c0[1], p[2] - c0[2]};
                double k[4];
                if (coulomb_kernel(dr, field ? 2 : 1, k)) {
                    bad = 1;
                    continue;
                }
                const double *m = &mu[3 * (size_t)i];
                double mdr = m[0] * dr[0] + m[1] * dr[1] + m[2] * dr[2];
                if (!field)
                    acc[0] += mdr * k[1];
                else
                    for (int c = 0; c < 3; c++) acc[c] += 3.0 * mdr * dr[c] * k[2] - m[c] * k[1];
            }
        }
        for (int c = 0; c < C; c++) out[(size_t)j * C + c] += acc[c];
    }
    free(mu);
    return bad ? ORC_ERR_NUMERIC : ORC_OK;
}

int orc_potential_ext(orc_sys *s, int32_t which, int32_t n, const double *cext, double *v) {
    return ext_props(s, which, n, cext, v, 0);
}

int orc_field_ext(orc_sys *s, int32_t which, int32_t n, const double *cext, double *e) {
    return ext_props(s, which, n, cext, e, 1);
}

/* ------------------------------------------------------------------ */
/* geometric gradients of the polarization energy                       */
/* polelec_geomgrad, src/mod_geomgrad.F90:113-277; prepare_polelec with  */
/* gradients, src/mod_electrostatics.F90:1487-1596; elec_prop_M2D /     */
/* D2D / D2M with field gradients and Hessians :2113-3065; the          */
/* q/mu/quad_elec_prop derivative formulas :1097-1405; rotation_geomgrad */
/* and rotation_matrix(doder), src/rotate_multipoles.F90:3-230,298-643.  */
/* Component orders: gradient xx,xy,yy,xz,yz,zz; Hessian xxx,xxy,xxz,    */
/* xyy,xyz,xzz,yyy,yyz,yzz,zzz (include/f_cart_components.h).           */
/* ------------------------------------------------------------------ */
static const int G6[3][3] = {{0, 1, 3}, {1, 2, 4}, {3, 4, 5}};
static const int H10[3][3][3] = {{{0, 1, 2}, {1, 3, 4}, {2, 4, 5}},
                                 {{1, 3, 4}, {3, 6, 7}, {4, 7, 8}},
                                 {{2, 4, 5}, {4, 7, 8}, {5, 8, 9}}};
static const int G6A[6] = {0, 0, 1, 0, 1, 2}, G6B[6] = {0, 1, 1, 2, 2, 2};
static const int H10A[10] = {0, 0, 0, 0, 0, 0, 1, 1, 1, 2}, H10B[10] = {0, 0, 0, 1, 1, 2, 1, 1, 2, 2},
                 H10C[10] = {0, 1, 2, 1, 2, 2, 1, 2, 2, 2};
static inline double kd(int a, int b) { return a == b ? 1.0 : 0.0; }

/* field gradient of a charge q (kernel k: 1/r, r^-3, r^-5, ...) */
static void q_grad(double q, const double *d, const double *k, double *g) {
    for (int c = 0; c < 6; c++) {
        int a = G6A[c], b = G6B[c];
        g[c] += q * (3.0 * k[2] * d[a] * d[b] - k[1] * kd(a, b));
    }
}
/* field gradient and Hessian of a point dipole */
static void mu_grad(const double *mu, const double *d, const double *k, double *g, double *h) {
    double md = mu[0] * d[0] + mu[1] * d[1] + mu[2] * d[2];
    if (g)
        for (int c = 0; c < 6; c++) {
            int a = G6A[c], b = G6B[c];
            g[c] += md * k[3] * 15.0 * d[a] * d[b] - (md * kd(a, b) + mu[a] * d[b] + mu[b] * d[a]) * 3.0 * k[2];
        }
    if (h)
        for (int c = 0; c < 10; c++) {
            int a = H10A[c], b = H10B[c], e = H10C[c];
            h[c] += 105.0 * md * k[4] * d[a] * d[b] * d[e] -
                    15.0 * k[3] * (mu[a] * d[b] * d[e] + mu[b] * d[a] * d[e] + mu[e] * d[a] * d[b] +
                                   md * (kd(a, b) * d[e] + kd(a, e) * d[b] + kd(b, e) * d[a])) +
                    3.0 * k[2] * (mu[a] * kd(b, e) + mu[b] * kd(a, e) + mu[e] * kd(a, b));
        }
}
/* field gradient of a point quadrupole stored xx,xy,yy,xz,yz,zz */
static void quad_grad(const double *q6, const double *d, const double *k, double *g) {
    double Q[3][3] = {{q6[0], q6[1], q6[3]}, {q6[1], q6[2], q6[4]}, {q6[3], q6[4], q6[5]}};
    double t[3];
    for (int a = 0; a < 3; a++) t[a] = Q[a][0] * d[0] + Q[a][1] * d[1] + Q[a][2] * d[2];
    double sdr = t[0] * d[0] + t[1] * d[1] + t[2] * d[2];
    for (int c = 0; c < 6; c++) {
        int a = G6A[c], b = G6B[c];
        g[c] += 105.0 * k[4] * sdr * d[a] * d[b] + 6.0 * k[2] * Q[a][b] -
                15.0 * k[3] * (sdr * kd(a, b) + 2.0 * (t[a] * d[b] + t[b] * d[a]));
    }
}
/* field of a point dipole */
static void mu_field(const double *mu, const double *d, const double *k, double *e) {
    double md = mu[0] * d[0] + mu[1] * d[1] + mu[2] * d[2];
    for (int c = 0; c < 3; c++) e[c] += 3.0 * md * d[c] * k[2] - mu[c] * k[1];
}

/* rotation_matrix with derivatives: dr*[a][b][c] = d R[b][c] / d (coordinate a
   of the atom); R columns are ex, ey, ez */
static void m3mul(double a[3][3], double b[3][3], double o[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            o[i][j] = 0.0;
            for (int k = 0; k < 3; k++) o[i][j] += a[i][k] * b[k][j];
        }
}
static int rotation_derivatives(const double *c, const double *cx, const double *cy, const double *cz, int frame,
                                double r[3][3], double dri[3][3][3], double driz[3][3][3], double drix[3][3][3],
                                double driy[3][3][3]) {
    memset(dri, 0, 27 * sizeof(double));
    memset(driz, 0, 27 * sizeof(double));
    memset(drix, 0, 27 * sizeof(double));
    memset(driy, 0, 27 * sizeof(double));
    int st = rotation_matrix(c, cx, cy, cz, frame, r);
    if (st || frame == 0) return st;
    double xi[3], eta[3], zeta[3], u[3] = {0, 0, 0}, v[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++) {
        xi[k] = cz[k] - c[k];
        eta[k] = cx[k] - c[k];
        zeta[k] = cy[k] - c[k];
    }
    double xin = sqrt(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]);
    double etan = sqrt(eta[0] * eta[0] + eta[1] * eta[1] + eta[2] * eta[2]);
    double zetan = sqrt(zeta[0] * zeta[0] + zeta[1] * zeta[1] + zeta[2] * zeta[2]);
    if (frame == 1) {
        for (int k = 0; k < 3; k++) u[k] = xi[k], v[k] = eta[k];
    } else if (frame == 2) {
        for (int k = 0; k < 3; k++) u[k] = etan * xi[k] + xin * eta[k], v[k] = eta[k];
    } else if (frame == 3) {
        for (int k = 0; k < 3; k++) u[k] = xi[k];
        if (u[2] / xin <= 0.866 && fabs(u[1]) > EPS_RP)
            v[0] = 1.0;
        else
            v[1] = 1.0;
    } else if (frame == 4) {
        for (int k = 0; k < 3; k++) u[k] = xi[k], v[k] = zetan * eta[k] + etan * zeta[k];
    } else if (frame == 5) {
        for (int k = 0; k < 3; k++)
            u[k] = etan * zetan * xi[k] + xin * zetan * eta[k] + xin * etan * zeta[k], v[k] = eta[k];
    }
    double ex[3], ey[3], ez[3];
    for (int k = 0; k < 3; k++) ex[k] = r[k][0], ey[k] = r[k][1], ez[k] = r[k][2];
    (void)ey;
    double usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2], un = sqrt(usq), ucube = usq * un;
    double vez = v[0] * ez[0] + v[1] * ez[1] + v[2] * ez[2];
    double exr[3];
    for (int k = 0; k < 3; k++) exr[k] = v[k] - vez * ez[k];
    double exsq = exr[0] * exr[0] + exr[1] * exr[1] + exr[2] * exr[2], exn = sqrt(exsq);
    double ez_u[3][3] = {{0}}, ex_v[3][3] = {{0}}, ex_ez[3][3] = {{0}}, ey_ez[3][3], ey_ex[3][3];
    double u_ri[3][3] = {{0}}, u_riz[3][3] = {{0}}, u_rix[3][3] = {{0}}, u_riy[3][3] = {{0}};
    double v_ri[3][3] = {{0}}, v_rix[3][3] = {{0}}, v_riy[3][3] = {{0}};
    for (int k = 0; k < 3; k++) {
        ez_u[k][k] = 1.0 / un;
        ex_v[k][k] = 1.0 / exn;
        ex_ez[k][k] = -vez / exn;
    }
    for (int k = 0; k < 3; k++)
        for (int a = 0; a < 3; a++) {
            ez_u[a][k] -= u[a] * u[k] / ucube;
            ex_v[a][k] -= ez[a] * ez[k] / exn + ex[a] * ex[k] / exn;
            ex_ez[a][k] += ex[a] * vez * v[k] / exsq - ez[a] * v[k] / exn;
        }
    double ey_ez_[3][3] = {{0, ex[2], -ex[1]}, {-ex[2], 0, ex[0]}, {ex[1], -ex[0], 0}};
    double ey_ex_[3][3] = {{0, -ez[2], ez[1]}, {ez[2], 0, -ez[0]}, {-ez[1], ez[0], 0}};
    memcpy(ey_ez, ey_ez_, sizeof(ey_ez));
    memcpy(ey_ex, ey_ex_, sizeof(ey_ex));
    if (frame == 1) {
        for (int k = 0; k < 3; k++) u_ri[k][k] = -1.0, u_riz[k][k] = 1.0, v_ri[k][k] = -1.0, v_rix[k][k] = 1.0;
    } else if (frame == 2) {
        for (int k = 0; k < 3; k++)
            u_ri[k][k] = -xin - etan, u_riz[k][k] = etan, u_rix[k][k] = xin, v_ri[k][k] = -1.0, v_rix[k][k] = 1.0;
        for (int k = 0; k < 3; k++)
            for (int a = 0; a < 3; a++) {
                u_ri[a][k] += -eta[a] * xi[k] / xin - xi[a] * eta[k] / etan;
                u_riz[a][k] += eta[a] * xi[k] / xin;
                u_rix[a][k] += xi[a] * eta[k] / etan;
            }
    } else if (frame == 3) {
        for (int k = 0; k < 3; k++) u_ri[k][k] = -1.0, u_riz[k][k] = 1.0;
    } else if (frame == 4) {
        for (int k = 0; k < 3; k++)
            u_ri[k][k] = -1.0, u_riz[k][k] = 1.0, v_ri[k][k] = -etan - zetan, v_rix[k][k] = zetan,
            u_riy[k][k] = etan;
        for (int k = 0; k < 3; k++)
            for (int a = 0; a < 3; a++) {
                v_ri[a][k] += -eta[a] * zeta[k] / zetan - zeta[a] * eta[k] / etan;
                v_rix[a][k] += zeta[a] * eta[k] / etan;
                v_riy[a][k] += eta[a] * zeta[k] / zetan;
            }
    } else if (frame == 5) {
        for (int k = 0; k < 3; k++)
            u_ri[k][k] = -xin * etan - xin * zetan - etan * zetan, u_riz[k][k] = etan * zetan,
            u_rix[k][k] = xin * zetan, u_riy[k][k] = xin * etan, v_ri[k][k] = -1.0, v_rix[k][k] = 1.0;
        for (int k = 0; k < 3; k++)
            for (int a = 0; a < 3; a++) {
                double A = eta[a] * zetan + zeta[a] * etan, B = xi[a] * zetan + zeta[a] * xin,
                       Cc = xi[a] * etan + eta[a] * xin;
                u_ri[a][k] += -A * xi[k] / xin - B * eta[k] / etan - Cc * zeta[k] / zetan;
                u_riz[a][k] += A * xi[k] / xin;
                u_rix[a][k] += B * eta[k] / etan;
                u_riy[a][k] += Cc * zeta[k] / zetan;
            }
    }
    double ez_ri[3][3], ez_riz[3][3], ez_rix[3][3], ez_riy[3][3];
    m3mul(ez_u, u_ri, ez_ri);
    m3mul(ez_u, u_riz, ez_riz);
    m3mul(ez_u, u_rix, ez_rix);
    m3mul(ez_u, u_riy, ez_riy);
    double t1[3][3], t2[3][3], ex_ri[3][3], ex_riz[3][3], ex_rix[3][3], ex_riy[3][3];
    m3mul(ex_v, v_ri, t1);
    m3mul(ex_ez, ez_ri, t2);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) ex_ri[a][b] = t1[a][b] + t2[a][b];
    m3mul(ex_ez, ez_riz, ex_riz);
    m3mul(ex_v, v_rix, t1);
    m3mul(ex_ez, ez_rix, t2);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) ex_rix[a][b] = t1[a][b] + t2[a][b];
    m3mul(ex_v, v_riy, t1);
    m3mul(ex_ez, ez_riy, t2);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) ex_riy[a][b] = t1[a][b] + t2[a][b];
    double ey_ri[3][3], ey_riz[3][3], ey_rix[3][3], ey_riy[3][3];
    double (*exs[4])[3] = {ex_ri, ex_riz, ex_rix, ex_riy};
    double (*ezs[4])[3] = {ez_ri, ez_riz, ez_rix, ez_riy};
    double (*eys[4])[3] = {ey_ri, ey_riz, ey_rix, ey_riy};
    for (int w = 0; w < 4; w++) {
        m3mul(ey_ex, exs[w], t1);
        m3mul(ey_ez, ezs[w], t2);
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) eys[w][a][b] = t1[a][b] + t2[a][b];
    }
    /* d[a][b][col] = d e_col(b) / d r_a  (the transposes of the reference) */
    double (*outs[4])[3][3] = {dri, driz, drix, driy};
    for (int w = 0; w < 4; w++)
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                outs[w][a][b][0] = exs[w][b][a];
                outs[w][a][b][1] = eys[w][b][a];
                outs[w][a][b][2] = ezs[w][b][a];
            }
    return 0;
}

/* rotation_geomgrad: forces from the frame dependence of the rotated dipoles
   and quadrupoles in the field E / field gradient G at each static site */
static int rotation_geomgrad(orc_sys *s, const double *E, const double *G, double *grad,
                             const unsigned char *fmask) {
    for (int j = 0; j < s->mm; j++) {
        if (fmask && !fmask[j]) continue;
        int jz = s->iz[j] >= 0 ? s->iz[j] : j;
        int jx = s->ix[j] >= 0 ? s->ix[j] : j;
        int jy = s->iy[j] >= 0 ? s->iy[j] : j;
        double r[3][3], d[4][3][3][3];
        int st = rotation_derivatives(&s->cmm[3 * j], &s->cmm[3 * jx], &s->cmm[3 * jy], &s->cmm[3 * jz],
                                      s->frame[j], r, d[0], d[1], d[2], d[3]);
        if (st) return st;
        const double *q0 = &s->q0[10 * j], *q = &s->q[10 * j];
        double dip[3] = {q0[1], q0[2], q0[3]};
        double qua[3][3] = {{q0[4], q0[5], q0[7]}, {q0[5], q0[6], q0[8]}, {q0[7], q0[8], q0[9]}};
        double rqua[3][3] = {{q[4], q[5], q[7]}, {q[5], q[6], q[8]}, {q[7], q[8], q[9]}};
        const int atoms[4] = {j, jz, jx, jy};
        const double *Ej = &E[3 * j], *Gj = &G[6 * j];
        for (int w = 0; w < 4; w++) {
            double ddip[3][3] = {{0}}, dqua[3][3][3] = {{{0}}};
            for (int a = 0; a < 3; a++)
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++) ddip[a][k] += d[w][a][k][l] * dip[l];
            for (int a = 0; a < 3; a++)
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++)
                        for (int m = 0; m < 3; m++)
                            for (int n = 0; n < 3; n++)
                                dqua[a][k][l] += (d[w][a][k][m] * qua[m][n] - rqua[k][m] * d[w][a][m][n]) * r[l][n];
            double *g = &grad[3 * atoms[w]];
            for (int a = 0; a < 3; a++) {
                g[a] -= ddip[a][0] * Ej[0] + ddip[a][1] * Ej[1] + ddip[a][2] * Ej[2];
                g[a] += dqua[a][0][0] * Gj[0] + dqua[a][1][1] * Gj[2] + dqua[a][2][2] * Gj[5] +
                        2.0 * (dqua[a][0][1] * Gj[1] + dqua[a][0][2] * Gj[3] + dqua[a][1][2] * Gj[4]);
            }
        }
    }
    return 0;
}

/* the scale of the (static site i, polarizable site j) pair in one list */
static inline void pair_scale(const slist_t *l, int i, int j, int *todo, double *sc) {
    int k = list_find(l, i, j);
    *todo = 1;
    *sc = 1.0;
    if (k >= 0) {
        *todo = l->todo[k];
        *sc = l->scale[k];
    }
}

/* fmask [mm]: static sites whose field, field gradient and Hessian are
   needed; pmask [npol]: polarizable sites whose field gradients are needed
   (NULL: all).  The gradient is exact on every atom whose own site is in
   both masks (when polarizable) and whose frame dependents are in fmask. */
static int geomgrad_impl(orc_sys *s, double *grad, const unsigned char *fmask, const unsigned char *pmask) {
    const int np = s->npol, mm = s->mm, amoeba = s->amoeba, nset = s->n_ipd;
    if (np == 0) return 0;
    int st = 0;
    if (!s->ipd_done) {
        st = prepare_polelec(s);
        if (!st) st = polarization(s, s->e_m2d, SOLVER_NONE, MATV_NONE, NULL);
        if (st) return st;
    }
    double *gm2d = xcalloc(6 * (size_t)np * nset, sizeof(double));
    double *gd2d = xcalloc(6 * (size_t)np * nset, sizeof(double));
    double *ed2m = xcalloc(3 * (size_t)mm, sizeof(double));
    double *gd2m = xcalloc(6 * (size_t)mm, sizeof(double));
    double *hd2m = xcalloc(10 * (size_t)mm, sizeof(double));
    int bad = 0;
    /* Egrd_M2D: set 0 (D, S_P_D scales) and set 1 (P, S_P_P scales) for AMOEBA */
#pragma omp parallel for schedule(dynamic, 4) reduction(| : bad)
    for (int j = 0; j < np; j++) {
        int jm = s->polar_mm[j];
        if (pmask && !pmask[j]) continue;
        for (int i = 0; i < mm; i++) {
            if (i == jm) continue;
            int tp, td = 0;
            double sp, sd = 1.0;
            pair_scale(&s->sPP, i, j, &tp, &sp);
            if (amoeba) pair_scale(&s->sPD, i, j, &td, &sd);
            if (!tp && !td) continue;
            double k[5], dr[3], g[6] = {0, 0, 0, 0, 0, 0};
            if (damped_kernel(s, i, jm, amoeba ? 4 : 2, k, dr)) {
                bad = 1;
                continue;
            }
            const double *q = &s->q[(size_t)s->ld_cart * i];
            q_grad(q[0], dr, k, g);
            if (amoeba) {
                mu_grad(&q[1], dr, k, g, NULL);
                quad_grad(&q[4], dr, k, g);
            }
            if (amoeba) {
                for (int c = 0; c < 6; c++) {
                    if (tp) gm2d[6 * ((size_t)np + j) + c] += g[c] * sp;
                    if (td) gm2d[6 * (size_t)j + c] += g[c] * sd;
                }
            } else if (tp) {
                for (int c = 0; c < 6; c++) gm2d[6 * (size_t)j + c] += g[c] * sp;
            }
        }
    }
    /* Egrd_D2D per set, list_P_P scales */
#pragma omp parallel for schedule(dynamic, 4) reduction(| : bad)
    for (int j = 0; j < np; j++) {
        if (pmask && !pmask[j]) continue;
        for (int i = 0; i < np; i++) {
            if (i == j) continue;
            int todo = 1;
            double sc = 1.0;
            int kk = list_find(&s->PP, i, j);
            if (kk >= 0) {
                todo = s->PP.todo[kk];
                sc = s->PP.scale[kk];
            }
            if (!todo) continue;
            double k[4], dr[3];
            if (damped_kernel(s, s->polar_mm[i], s->polar_mm[j], 3, k, dr)) {
                bad = 1;
                continue;
            }
            for (int set = 0; set < nset; set++) {
                double g[6] = {0, 0, 0, 0, 0, 0};
                mu_grad(&s->ipd[3 * ((size_t)set * np + i)], dr, k, g, NULL);
                for (int c = 0; c < 6; c++) gd2d[6 * ((size_t)set * np + j) + c] += g[c] * sc;
            }
        }
    }
    /* E / Egrd / EHes of the induced dipoles at the static sites: AMOEBA
       averages the P dipoles with S_P_D scales and the D dipoles with S_P_P
       scales; Wang-AL uses its one set with S_P_P */
#pragma omp parallel for schedule(dynamic, 4) reduction(| : bad)
    for (int j = 0; j < mm; j++) {
        if (fmask && !fmask[j]) continue;
        for (int i = 0; i < np; i++) {
            if (s->polar_mm[i] == j) continue;
            double k[5], dr[3];
            int have = 0;
            for (int kind = 0; kind < (amoeba ? 2 : 1); kind++) {
                /* kind 0: D dipoles (S_P_P); kind 1: P dipoles (S_P_D) */
                int todo;
                double sc;
                pair_scale(kind == 0 ? &s->sPP : &s->sPD, j, i, &todo, &sc);
                if (!todo) continue;
                if (!have) {
                    if (damped_kernel(s, s->polar_mm[i], j, amoeba ? 4 : 2, k, dr)) {
                        bad = 1;
                        break;
                    }
                    have = 1;
                }
                const double *mu = &s->ipd[3 * ((size_t)(kind == 0 ? 0 : 1) * np + i)];
                double e[3] = {0, 0, 0}, g[6] = {0, 0, 0, 0, 0, 0}, h[10] = {0};
                mu_field(mu, dr, k, e);
                if (amoeba) mu_grad(mu, dr, k, g, h);
                const double w = (amoeba ? 0.5 : 1.0) * sc;
                for (int c = 0; c < 3; c++) ed2m[3 * (size_t)j + c] += e[c] * w;
                if (amoeba) {
                    for (int c = 0; c < 6; c++) gd2m[6 * (size_t)j + c] += g[c] * w;
                    for (int c = 0; c < 10; c++) hd2m[10 * (size_t)j + c] += h[c] * w;
                }
            }
        }
    }
    if (bad) {
        set_err("Requesting Coulomb kernel for two atoms placed in the same point");
        free(gm2d), free(gd2d), free(ed2m), free(gd2m), free(hd2m);
        return ORC_ERR_NUMERIC;
    }
    /* assembly (mod_geomgrad.F90:132-271) */
    for (int i = 0; i < mm; i++) {
        const double *q = &s->q[(size_t)s->ld_cart * i];
        for (int a = 0; a < 3; a++) grad[3 * i + a] -= q[0] * ed2m[3 * i + a];
        if (!amoeba) continue;
        const double *G = &gd2m[6 * (size_t)i], *H = &hd2m[10 * (size_t)i];
        for (int a = 0; a < 3; a++) {
            grad[3 * i + a] += q[1] * G[G6[a][0]] + q[2] * G[G6[a][1]] + q[3] * G[G6[a][2]];
            double Q[3][3] = {{q[4], q[5], q[7]}, {q[5], q[6], q[8]}, {q[7], q[8], q[9]}};
            double acc = 0.0;
            for (int b = 0; b < 3; b++)
                for (int c = 0; c < 3; c++) acc += Q[b][c] * H[H10[b][c][a]];
            grad[3 * i + a] -= acc;
        }
    }
    for (int j = 0; j < np; j++) {
        double *g = &grad[3 * (size_t)s->polar_mm[j]];
        if (amoeba) {
            const double *mD = &s->ipd[3 * (size_t)j], *mP = &s->ipd[3 * ((size_t)np + j)];
            const double *GP = &gm2d[6 * ((size_t)np + j)], *GD = &gm2d[6 * (size_t)j];
            const double *HP = &gd2d[6 * ((size_t)np + j)], *HD = &gd2d[6 * (size_t)j];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    int c = G6[a][b];
                    g[a] += 0.5 * mD[b] * (GP[c] + HP[c]) + 0.5 * mP[b] * (GD[c] + HD[c]);
                }
        } else {
            const double *m = &s->ipd[3 * (size_t)j];
            const double *GM = &gm2d[6 * (size_t)j], *HM = &gd2d[6 * (size_t)j];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) g[a] += m[b] * (GM[G6[a][b]] + HM[G6[a][b]]);
        }
    }
    if (amoeba) st = rotation_geomgrad(s, ed2m, gd2m, grad, fmask);
    free(gm2d), free(gd2d), free(ed2m), free(gd2m), free(hd2m);
    return st;
}

int orc_polelec_geomgrad(orc_sys *s, double *grad) { return geomgrad_impl(s, grad, NULL, NULL); }

int orc_polelec_geomgrad_atoms(orc_sys *s, int32_t na, const int32_t *atoms, double *out) {
    const int mm = s->mm;
    unsigned char *want = xcalloc(mm, 1), *fmask = xcalloc(mm, 1), *pmask = xcalloc(s->npol > 0 ? s->npol : 1, 1);
    for (int k = 0; k < na; k++) {
        if (atoms[k] < 0 || atoms[k] >= mm) {
            free(want), free(fmask), free(pmask);
            set_err("atom index out of range");
            return ORC_ERR_BAD_ARG;
        }
        want[atoms[k]] = 1;
    }
    for (int j = 0; j < mm; j++) {
        int jz = s->iz[j] >= 0 ? s->iz[j] : j, jx = s->ix[j] >= 0 ? s->ix[j] : j;
        int jy = s->iy[j] >= 0 ? s->iy[j] : j;
        if (want[j] || (s->amoeba && s->frame[j] != 0 && (want[jz] || want[jx] || want[jy]))) fmask[j] = 1;
        if (want[j] && s->mm_polar[j] >= 0) pmask[s->mm_polar[j]] = 1;
    }
    double *g = xcalloc(3 * (size_t)mm, sizeof(double));
    int st = geomgrad_impl(s, g, fmask, pmask);
    for (int k = 0; k < na; k++)
        for (int c = 0; c < 3; c++) out[3 * k + c] = g[3 * (size_t)atoms[k] + c];
    free(g), free(want), free(fmask), free(pmask);
    return st;
}

int orc_set_ipd(orc_sys *s, const double *ipd) {
    if (s->npol == 0) return 0;
    memcpy(s->ipd, ipd, sizeof(double) * 3 * (size_t)s->npol * s->n_ipd);
    s->ipd_done = 1;
    return 0;
}

/* ------------------------------------------------------------------ */
/* QM helper electrostatics: fields of the QM nuclei (point charges,   */
/* undamped coulomb_kernel) at the MM sites, electrostatic_for_ene /   */
/* electrostatic_for_grad (src/mod_qm_helper.F90:356-520) with         */
/* q_elec_prop (src/mod_electrostatics.F90:1097-1176).  The MM side    */
/* (V_m2n, V_p2n, E_m2n, E_p2n) is orc_potential_ext / orc_field_ext.  */
/* which 0: E_n2p [npol][3] only; 1: E_n2m [mm][3], G_n2m [mm][6],     */
/* H_n2m [mm][10] (outputs overwritten).                               */
/* ------------------------------------------------------------------ */
int orc_nuclei_fields(orc_sys *s, int32_t which, int32_t nq, const double *cqm, const double *qqm, double *E,
                      double *G, double *H) {
    const int nt = which == 0 ? s->npol : s->mm;
    int bad = 0;
    memset(E, 0, sizeof(double) * 3 * (size_t)nt);
    if (which) {
        memset(G, 0, sizeof(double) * 6 * (size_t)nt);
        memset(H, 0, sizeof(double) * 10 * (size_t)nt);
    }
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int j = 0; j < nt; j++) {
        const double *c = &s->cmm[3 * (size_t)(which == 0 ? s->polar_mm[j] : j)];
        for (int i = 0; i < nq; i++) {
            double d[3] = {c[0] - cqm[3 * i], c[1] - cqm[3 * i + 1], c[2] - cqm[3 * i + 2]};
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (r < EPS_RP) {
                bad = 1;
                continue;
            }
            double k[4];
            k[0] = 1.0 / r;
            for (int l = 1; l < 4; l++) k[l] = k[l - 1] / (r * r);
            const double q = qqm[i];
            for (int a = 0; a < 3; a++) E[3 * (size_t)j + a] += q * k[1] * d[a];
            if (!which) continue;
            for (int c6 = 0; c6 < 6; c6++) {
                int a = G6A[c6], b = G6B[c6];
                G[6 * (size_t)j + c6] += q * (3.0 * k[2] * d[a] * d[b] - k[1] * kd(a, b));
            }
            for (int c10 = 0; c10 < 10; c10++) {
                int a = H10A[c10], b = H10B[c10], e = H10C[c10];
                H[10 * (size_t)j + c10] +=
                    q * (15.0 * k[3] * d[a] * d[b] * d[e] - 3.0 * k[2] * (kd(a, b) * d[e] + kd(a, e) * d[b] + kd(b, e) * d[a]));
            }
        }
    }
    if (bad) {
        set_err("Requesting Coulomb kernel for two atoms placed in the same point, this could be an internal bug or "
                "a problem in your input file, please check.");
        return ORC_ERR_NUMERIC;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Electrostatic properties of the static multipoles at the static     */
/* sites, elec_prop_M2M direct path (src/mod_electrostatics.F90:       */
/* 1678-1952): undamped coulomb_kernel, list_S_S of m-scaled pairs     */
/* (:597-648, screening_rules 'S','S'); potential V [mm], field E      */
/* [mm][3], and for AMOEBA field gradient G [mm][6] and (H not NULL)   */
/* field Hessian H [mm][10], from q_elec_prop / mu_elec_prop /         */
/* quad_elec_prop (:1097-1405).                                        */
/* ------------------------------------------------------------------ */
/* field Hessian of a point charge (q_elec_prop, do_HE) */
static void q_hess(double q, const double *d, const double *k, double *h) {
    for (int c = 0; c < 10; c++) {
        int a = H10A[c], b = H10B[c], e = H10C[c];
        h[c] += q * (15.0 * k[3] * d[a] * d[b] * d[e] - 3.0 * k[2] * (kd(a, b) * d[e] + kd(a, e) * d[b] + kd(b, e) * d[a]));
    }
}
/* field Hessian of a point quadrupole stored xx,xy,yy,xz,yz,zz (quad_elec_prop, do_HE) */
static void quad_hess(const double *q6, const double *d, const double *k, double *h) {
    double Q[3][3] = {{q6[0], q6[1], q6[3]}, {q6[1], q6[2], q6[4]}, {q6[3], q6[4], q6[5]}};
    double t[3];
    for (int a = 0; a < 3; a++) t[a] = Q[a][0] * d[0] + Q[a][1] * d[1] + Q[a][2] * d[2];
    double sdr = t[0] * d[0] + t[1] * d[1] + t[2] * d[2];
    for (int c = 0; c < 10; c++) {
        int a = H10A[c], b = H10B[c], e = H10C[c];
        h[c] += 945.0 * k[5] * sdr * d[a] * d[b] * d[e] -
                105.0 * k[4] * (sdr * (kd(a, b) * d[e] + kd(a, e) * d[b] + kd(b, e) * d[a]) +
                                2.0 * (t[a] * d[b] * d[e] + t[b] * d[a] * d[e] + t[e] * d[a] * d[b])) +
                30.0 * k[3] * (Q[a][b] * d[e] + Q[a][e] * d[b] + Q[b][e] * d[a] + kd(a, b) * t[e] + kd(a, e) * t[b] +
                               kd(b, e) * t[a]);
    }
}

static int m2m_props(orc_sys *s, double *V, double *E, double *G, double *H) {
    const int mm = s->mm, amoeba = s->amoeba, ld = s->ld_cart;
    /* list_S_S: row i, pairs within four bonds whose scale is not 1 */
    lbuild_t b;
    lb_init(&b, mm);
    for (int i = 0; i < mm; i++) {
        for (int ineigh = 0; ineigh < 4; ineigh++)
            for (int k = s->conn[ineigh].ri[i]; k < s->conn[ineigh].ri[i + 1]; k++) {
                int j = s->conn[ineigh].ci[k];
                double sc = screening_rules(s, i, 'S', j, 'S', '-');
                if (fabs(sc - 1.0) > EPS_RP) lb_push(&b, j, sc);
            }
        b.ri[i + 1] = b.nnz;
    }
    slist_t ss;
    lb_finish(&b, &ss);
    memset(V, 0, mm * sizeof(double));
    memset(E, 0, 3 * (size_t)mm * sizeof(double));
    if (amoeba) memset(G, 0, 6 * (size_t)mm * sizeof(double));
    if (amoeba && H) memset(H, 0, 10 * (size_t)mm * sizeof(double));
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : bad)
    for (int j = 0; j < mm; j++) {
        for (int i = 0; i < mm; i++) {
            if (i == j) continue;
            int todo = 1;
            double sc = 1.0;
            int kk = list_find(&ss, i, j);
            if (kk >= 0) {
                todo = ss.todo[kk];
                sc = ss.scale[kk];
            }
            if (!todo) continue;
            double d[3];
            for (int c = 0; c < 3; c++) d[c] = s->cmm[3 * (size_t)j + c] - s->cmm[3 * (size_t)i + c];
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (r < EPS_RP) {
                bad = 1;
                continue;
            }
            double k[6];
            k[0] = 1.0 / r;
            for (int l = 1; l < 6; l++) k[l] = k[l - 1] / (r * r);
            const double *q = &s->q[(size_t)ld * i];
            double v = q[0] * k[0], e[3], g[6] = {0, 0, 0, 0, 0, 0}, h[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int c = 0; c < 3; c++) e[c] = q[0] * k[1] * d[c];
            if (amoeba) {
                double md = q[1] * d[0] + q[2] * d[1] + q[3] * d[2];
                double Q[3][3] = {{q[4], q[5], q[7]}, {q[5], q[6], q[8]}, {q[7], q[8], q[9]}};
                double t[3];
                for (int a = 0; a < 3; a++) t[a] = Q[a][0] * d[0] + Q[a][1] * d[1] + Q[a][2] * d[2];
                double dqd = t[0] * d[0] + t[1] * d[1] + t[2] * d[2];
                v += md * k[1] + 3.0 * dqd * k[2];
                for (int c = 0; c < 3; c++)
                    e[c] += 3.0 * md * d[c] * k[2] - q[1 + c] * k[1] + 15.0 * dqd * d[c] * k[3] - 6.0 * t[c] * k[2];
                q_grad(q[0], d, k, g);
                mu_grad(&q[1], d, k, g, H ? h : NULL);
                quad_grad(&q[4], d, k, g);
                if (H) {
                    q_hess(q[0], d, k, h);
                    quad_hess(&q[4], d, k, h);
                }
            }
            const double w = (kk >= 0) ? sc : 1.0;
            V[j] += v * w;
            for (int c = 0; c < 3; c++) E[3 * (size_t)j + c] += e[c] * w;
            if (amoeba)
                for (int c = 0; c < 6; c++) G[6 * (size_t)j + c] += g[c] * w;
            if (amoeba && H)
                for (int c = 0; c < 10; c++) H[10 * (size_t)j + c] += h[c] * w;
        }
    }
    free(ss.m.ri), free(ss.m.ci), free(ss.scale), free(ss.todo);
    if (bad) {
        set_err("Requesting Coulomb kernel for two atoms placed in the same point, this could be an internal bug or "
                "a problem in your input file, please check.");
        return ORC_ERR_NUMERIC;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Static multipole energy (fixed electrostatics): energy_MM_MM        */
/* (src/mod_electrostatics.F90:899-941) on m2m_props.                  */
/* ------------------------------------------------------------------ */
int orc_get_fixedelec_energy(orc_sys *s, double *energy) {
    const int mm = s->mm, amoeba = s->amoeba, ld = s->ld_cart;
    double *V = xcalloc(mm, sizeof(double)), *E = xcalloc(3 * (size_t)mm, sizeof(double));
    double *G = xcalloc(6 * (size_t)mm, sizeof(double));
    int st = m2m_props(s, V, E, G, NULL);
    double em = 0.0;
    if (!st)
        for (int j = 0; j < mm; j++) {
            const double *q = &s->q[(size_t)ld * j];
            em += q[0] * V[j];
            if (amoeba) {
                for (int c = 0; c < 3; c++) em -= q[1 + c] * E[3 * (size_t)j + c];
                const double *g = &G[6 * (size_t)j];
                em += q[4] * g[0] + q[6] * g[2] + q[9] * g[5] + 2.0 * (q[5] * g[1] + q[7] * g[3] + q[8] * g[4]);
            }
        }
    free(V), free(E), free(G);
    if (st) return st;
    *energy = 0.5 * em;
    return 0;
}

/* ------------------------------------------------------------------ */
/* ommp_fixedelec_geomgrad (src/mod_interface.F90:657-668): the output */
/* zeroed, then fixedelec_geomgrad (src/mod_geomgrad.F90:17-111):      */
/* per static site -q E + mu.Egrd - Q:EHes (off-diagonal quadrupole    */
/* components twice) and, for AMOEBA, rotation_geomgrad with E, Egrd.  */
/* ------------------------------------------------------------------ */
int orc_fixedelec_geomgrad(orc_sys *s, double *grad) {
    const int mm = s->mm, amoeba = s->amoeba, ld = s->ld_cart;
    memset(grad, 0, 3 * (size_t)mm * sizeof(double));
    double *V = xcalloc(mm, sizeof(double)), *E = xcalloc(3 * (size_t)mm, sizeof(double));
    double *G = xcalloc(6 * (size_t)mm, sizeof(double)), *H = xcalloc(10 * (size_t)mm, sizeof(double));
    int st = m2m_props(s, V, E, G, H);
    if (!st) {
        for (int i = 0; i < mm; i++) {
            const double *q = &s->q[(size_t)ld * i], *e = &E[3 * (size_t)i];
            double *g = &grad[3 * (size_t)i];
            for (int a = 0; a < 3; a++) g[a] -= q[0] * e[a];
            if (!amoeba) continue;
            const double *eg = &G[6 * (size_t)i], *h = &H[10 * (size_t)i];
            double Q[3][3] = {{q[4], q[5], q[7]}, {q[5], q[6], q[8]}, {q[7], q[8], q[9]}};
            for (int a = 0; a < 3; a++) {
                for (int b = 0; b < 3; b++) g[a] += q[1 + b] * eg[G6[a][b]];
                for (int b = 0; b < 3; b++)
                    for (int c = 0; c < 3; c++) g[a] -= Q[b][c] * h[H10[b][c][a]];
            }
        }
        if (amoeba) st = rotation_geomgrad(s, E, G, grad, NULL);
    }
    free(V), free(E), free(G), free(H);
    return st;
}

/* ------------------------------------------------------------------ */
/* ommp_rotation_geomgrad (src/mod_interface.F90:699-710): the output  */
/* zeroed, then the frame forces of the rotated static dipoles and     */
/* quadrupoles in a given E [mm][3] and field gradient G [mm][6]       */
/* (src/rotate_multipoles.F90:3-230).  Point charges have no frame.    */
/* ------------------------------------------------------------------ */
int orc_rotation_geomgrad(orc_sys *s, const double *E, const double *G, double *grad) {
    memset(grad, 0, 3 * (size_t)s->mm * sizeof(double));
    if (!s->amoeba) return 0;
    return rotation_geomgrad(s, E, G, grad, NULL);
}
