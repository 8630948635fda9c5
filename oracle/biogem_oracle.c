/*
 * ORACLE -- test infrastructure only.  Nothing in the product links, loads or
 * calls this file; only the tests, the smoke check and bench.py's CPU-baseline
 * leg do, and only as the checker or the timed CPU reference.
 *
 * C restatement of the reference BIOGEM tracer coupling:
 *   biogem_tracercoupling   src/biogem/biogem.f90:1885-2077
 *   fun_lib_init_vocn       src/biogem/biogem_lib.f90:1056-1081  (column order: i outer, j inner)
 *   fun_lib_conv_tsTOvocn   src/biogem/biogem_lib.f90:1335-1373
 *   fun_lib_conv_vocnTOts   src/biogem/biogem_lib.f90:1379-1410
 * BIOGEM's vector fields arrive packed as in include/gb_biogem.h: vocn(n)%mk(l,k)
 * as (n_l_ocn, n_k, n_vocn), vphys_ocn(n)%mk(ipo,k) as (n_k, n_vocn).  The GOLDSTEIN
 * tracers are go_ts / go_ts1, (n_l_ocn, n_i, n_j, n_k) without halos.
 *
 * Fortran's SUM over an array section (no -ffast-math) adds left to right from 0;
 * the per-column partial sums and the sums over columns below do the same, in the
 * reference's column order.  Expressions keep gfortran's left-to-right evaluation;
 * compile with -ffp-contract=off.
 *
 * Parity pin: as for goldstein_oracle.c, no Fortran compiler exists here and the
 * reference ships no fixtures for this routine: the restatement is cross-checked
 * against the independent NumPy restatement (oracle/biogem_np.py) and by the
 * inventory-conservation known-answer test ("parity unpinned").
 */
#include "../include/gb_biogem.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* const_real_nullsmall (src/common/gem_cmn.f90:719) */
#define BG_NULLSMALL 0.999999e-19

typedef struct {
    int i, j, k1;
} bg_col;

/* the wet columns in vector order (biogem_lib.f90:1069-1079) */
static int bg_columns(const gb_bg_dims *d, const int32_t *k1, bg_col *out)
{
    int n = 0;
    for (int i = 1; i <= d->n_i; ++i)
        for (int j = 1; j <= d->n_j; ++j) {
            const int kk = k1[(i - 1) + (size_t)d->n_i * (j - 1)];
            if (d->n_k >= kk) {
                if (out) {
                    out[n].i = i;
                    out[n].j = j;
                    out[n].k1 = kk;
                }
                ++n;
            }
        }
    return n;
}

int gbo_bg_columns(const gb_bg_dims *d, const int32_t *k1) { return bg_columns(d, k1, NULL); }

/* go_ts(l,i,j,k), 1-based, no halos */
#define TS(a, l, i, j, k) (a)[((l) - 1) + (size_t)L * (((i) - 1) + (size_t)d->n_i * (((j) - 1) + (size_t)d->n_j * ((k) - 1)))]
/* vocn(n)%mk(l,k), 1-based l, k; 0-based n */
#define VO(a, n, l, k) (a)[((l) - 1) + (size_t)L * (((k) - 1) + (size_t)nk * (size_t)(n))]
#define VP(a, n, k) (a)[((k) - 1) + (size_t)nk * (size_t)(n)]
#define VS(a, n, l, k) (a)[((l) - 1) + (size_t)Ls * (((k) - 1) + (size_t)nk * (size_t)(n))]

int gbo_bg_tracercoupling(const gb_bg_dims *d, const gb_bg_params *p, const int32_t *k1, double *go_ts,
                          double *go_ts1, double *vocn, double *mass, const double *volume, double *rmass,
                          const double *vdocn, double *vbio_part, const double *vdbio_part)
{
    const int L = d->n_l_ocn, Ls = d->n_l_sed, nk = d->n_k;
    if (L < 2 || nk < 1 || d->n_i < 1 || d->n_j < 1 || Ls < 0) return -1;
    const int nv = bg_columns(d, k1, NULL);
    bg_col *col = (bg_col *)malloc(sizeof(bg_col) * (size_t)(nv > 0 ? nv : 1));
    const size_t nf = (size_t)L * nk * (size_t)nv;
    double *loc_vocn = (double *)calloc(nf ? nf : 1, sizeof(double));
    double *loc_vts = (double *)calloc(nf ? nf : 1, sizeof(double));
    double *part = (double *)malloc(sizeof(double) * (size_t)(nv > 0 ? nv : 1));
    double *tot_old = (double *)calloc((size_t)L + 1, sizeof(double));
    double *tot_new = (double *)calloc((size_t)L + 1, sizeof(double));
    double *rtot_new = (double *)calloc((size_t)L + 1, sizeof(double));
    if (!col || !loc_vocn || !loc_vts || !part || !tot_old || !tot_new || !rtot_new) {
        free(col); free(loc_vocn); free(loc_vts); free(part); free(tot_old); free(tot_new); free(rtot_new);
        return -2;
    }
    bg_columns(d, k1, col);
    /* loc_vts = fun_lib_conv_tsTOvocn(dum_ts): levels k1..n_k, 0 elsewhere */
    for (int n = 0; n < nv; ++n)
        for (int k = col[n].k1; k <= nk; ++k)
            for (int l = 1; l <= L; ++l) VO(loc_vts, n, l, k) = TS(go_ts, l, col[n].i, col[n].j, k);

    /* total ocean volume and its reciprocal (:1928-1936); the mass total (:1919-1927)
       is computed by the reference but not used in this routine */
    for (int n = 0; n < nv; ++n) {
        double s = 0.0;
        for (int k = col[n].k1; k <= nk; ++k) s += VP(volume, n, k);
        part[n] = s;
    }
    double tot_v = 0.0;
    for (int n = 0; n < nv; ++n) tot_v += part[n];
    const double rtot_v = 1.0 / tot_v;

    /* (0) old mean salinity (:1946-1953) */
    for (int n = 0; n < nv; ++n) {
        double s = 0.0;
        for (int k = col[n].k1; k <= nk; ++k) s += VO(vocn, n, 2, k) * VP(volume, n, k);
        part[n] = s * rtot_v;
    }
    double mean_s_old = 0.0;
    for (int n = 0; n < nv; ++n) mean_s_old += part[n];
    const double rmean_s_old = 1.0 / mean_s_old;
    /* old biogeochemical inventories (:1955-1963) */
    for (int l = 3; l <= L; ++l) {
        for (int n = 0; n < nv; ++n) {
            double s = 0.0;
            for (int k = col[n].k1; k <= nk; ++k) s += VO(vocn, n, l, k) * VP(mass, n, k);
            part[n] = s;
        }
        double t = 0.0;
        for (int n = 0; n < nv; ++n) t += part[n];
        tot_old[l] = t;
    }
    /* (1) salinity-adjusted GOLDSTEIN tracers (:1970-1980) */
    for (int n = 0; n < nv; ++n)
        for (int k = nk; k >= col[n].k1; --k) {
            VO(loc_vocn, n, 1, k) = VO(loc_vts, n, 1, k) + p->ts_offset[0];
            VO(loc_vocn, n, 2, k) = VO(loc_vts, n, 2, k) + p->ts_offset[1];
            for (int l = 3; l <= L; ++l)
                VO(loc_vocn, n, l, k) = VO(loc_vts, n, l, k) * VO(vocn, n, 2, k) * rmean_s_old;
        }
    /* new inventories and their reciprocals, 0 when below const_real_nullsmall (:1983-1996) */
    for (int l = 3; l <= L; ++l) {
        for (int n = 0; n < nv; ++n) {
            double s = 0.0;
            for (int k = col[n].k1; k <= nk; ++k) s += VO(loc_vocn, n, l, k) * VP(mass, n, k);
            part[n] = s;
        }
        double t = 0.0;
        for (int n = 0; n < nv; ++n) t += part[n];
        tot_new[l] = t;
        rtot_new[l] = fabs(t) < BG_NULLSMALL ? 0.0 : 1.0 / t;
    }
    /* (2) T and S (:2000-2013) */
    for (int n = 0; n < nv; ++n)
        for (int k = nk; k >= col[n].k1; --k)
            for (int l = 1; l <= 2; ++l) {
                if (p->force_ts) {
                    VO(loc_vocn, n, l, k) = VO(loc_vts, n, l, k) + p->ts_offset[l - 1] + VO(vdocn, n, l, k);
                    VO(vocn, n, l, k) = VO(loc_vocn, n, l, k);
                } else {
                    VO(vocn, n, l, k) = VO(loc_vocn, n, l, k) + VO(vdocn, n, l, k);
                }
            }
    /* new mean salinity, with the volume taken as invariant (:2016-2023) */
    for (int n = 0; n < nv; ++n) {
        double s = 0.0;
        for (int k = col[n].k1; k <= nk; ++k) s += VO(vocn, n, 2, k) * VP(volume, n, k);
        part[n] = s * rtot_v;
    }
    double mean_s_new = 0.0;
    for (int n = 0; n < nv; ++n) mean_s_new += part[n];
    const double s_ratio = mean_s_new / mean_s_old;
    const double rs_ratio = 1.0 / s_ratio;
    /* (3) biogeochemical fields, particulates, GOLDSTEIN tracers (:2033-2047) */
    for (int n = 0; n < nv; ++n)
        for (int k = nk; k >= col[n].k1; --k) {
            for (int l = 3; l <= L; ++l) {
                VO(vocn, n, l, k) = (tot_old[l] * rtot_new[l]) * VO(loc_vocn, n, l, k) + VO(vdocn, n, l, k);
                VO(vocn, n, l, k) = s_ratio * VO(vocn, n, l, k);
            }
            for (int l = 1; l <= Ls; ++l) {
                VS(vbio_part, n, l, k) = VS(vbio_part, n, l, k) + VS(vdbio_part, n, l, k);
                VS(vbio_part, n, l, k) = s_ratio * VS(vbio_part, n, l, k);
            }
            VO(loc_vts, n, 1, k) = VO(loc_vocn, n, 1, k) - p->ts_offset[0];
            VO(loc_vts, n, 2, k) = VO(loc_vocn, n, 2, k) - p->ts_offset[1];
            for (int l = 3; l <= L; ++l)
                VO(loc_vts, n, l, k) = (mean_s_new / VO(vocn, n, 2, k)) * VO(vocn, n, l, k);
        }
    /* cell masses (:2049-2053) */
    for (int n = 0; n < nv; ++n)
        for (int k = col[n].k1; k <= nk; ++k) {
            VP(mass, n, k) = rs_ratio * VP(mass, n, k);
            VP(rmass, n, k) = s_ratio * VP(rmass, n, k);
        }
    /* dum_ts = fun_lib_conv_vocnTOts(loc_vts): 0 outside the wet levels; dum_ts1 = dum_ts (:2055-2056) */
    const size_t nts = (size_t)L * d->n_i * d->n_j * nk;
    memset(go_ts, 0, nts * sizeof(double));
    for (int n = 0; n < nv; ++n)
        for (int l = 1; l <= L; ++l)
            for (int k = col[n].k1; k <= nk; ++k) TS(go_ts, l, col[n].i, col[n].j, k) = VO(loc_vts, n, l, k);
    memcpy(go_ts1, go_ts, nts * sizeof(double));
    free(col); free(loc_vocn); free(loc_vts); free(part); free(tot_old); free(tot_new); free(rtot_new);
    return 0;
}
