/*
 * ORACLE -- test infrastructure only.  Nothing in the product links, loads or
 * calls this file; only the tests and bench.py's CPU legs do, and only as the
 * checker or the timed CPU reference.
 *
 * C restatement of the reference's 2-D iterative implicit surface steppers:
 *   tstipa    src/embm/embm.f90:2039-2138                   (EMBM air temperature, humidity)
 *   tstipsic  src/goldsteinseaice/gold_seaice.f90:937-1058  (sea-ice height, area; the
 *             diagnostic variceth/varicedy of :1047-1055 are not restated)
 *   tstepsic  src/goldsteinseaice/gold_seaice.f90:844-929   (the explicit sea-ice step)
 * Arrays as in include/gb_embm.h.  Every expression keeps gfortran's left-to-right
 * evaluation in IEEE double; compile with -ffp-contract=off.
 *
 * Parity pin: no Fortran compiler exists here and the reference ships no fixtures for
 * these routines ("parity unpinned"); the restatement is cross-checked against the
 * independent NumPy restatement in oracle/surface_np.py.
 */
#include "../include/gb_embm.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* 0-based local arrays with the reference's bounds */
#define C2(a, i, j) (a)[(size_t)(i) + (size_t)(maxi + 1) * (size_t)(j)]          /* (0:maxi, 0:maxj) */
#define V2(a, i, j) (a)[(size_t)(i) + (size_t)(maxi + 2) * (size_t)(j)]          /* (0:maxi+1, 0:maxj+1) */
#define TQ(a, l, i, j) (a)[((l) - 1) + 2 * (((size_t)(i) - 1) + (size_t)maxi * ((size_t)(j) - 1))]
#define K1(i, j) g->k1[(size_t)(i) + (size_t)(maxi + 2) * (size_t)(j)]

static double dmax(double a, double b) { return a > b ? a : b; }   /* MAX(0.0, x): x unless x < 0 */
static double dmin(double a, double b) { return a < b ? a : b; }

static void coefficients(const gb_ea_dims *d, const gb_ea_params *p, const gb_ea_grid *g, int l, const double *vel,
                         const double *pptn, double *cie, double *ciw, double *cin, double *cis)
{
    const int maxi = d->maxi, maxj = d->maxj;
    for (int j = 1; j <= maxj; ++j)
        for (int i = 1; i <= maxi; ++i) {
            double tv, ups, pec, diffpp;
            const double u1 = TQ(vel, 1, i, j), u2 = TQ(vel, 2, i, j);
            if (p->kind == GB_EA_EMBM) {
                /* embm.f90:2061-2088 */
                const double clampp = dmax(0.0, dmin(1.0, (pptn[(i - 1) + (size_t)maxi * (j - 1)] - p->ppmin) /
                                                              (p->ppmax - p->ppmin)));
                C2(cie, i, j) = p->betaz[l - 1] * u1 * g->rc[j] * 0.5 * p->rdphi;
                diffpp = g->diffa[(l - 1) + 2 * (0 + 2 * (size_t)(j - 1))] + (double)(2 - l) * p->diffmod0 * clampp;
                tv = g->rc[j] * g->rc[j] * p->rdphi * diffpp * p->rdphi;
                pec = p->betaz[l - 1] * u1 * p->dphi / diffpp;
                ups = pec / (2.0 + fabs(pec));
                C2(ciw, i, j) = C2(cie, i, j) * (1 + ups) + tv;
                C2(cie, i, j) = C2(cie, i, j) * (1 - ups) - tv;
                C2(cin, i, j) = g->cv[j] * p->betam[l - 1] * u2 * 0.5;
                diffpp = g->diffa[(l - 1) + 2 * (1 + 2 * (size_t)(j - 1))] + (double)(2 - l) * p->diffmod0 * clampp;
                if (j < maxj) {
                    tv = g->cv[j] * g->cv[j] * g->rdsv[j - 1] * g->diffa[(l - 1) + 2 * (1 + 2 * (size_t)(j - 1))];
                    pec = p->betam[l - 1] * u2 * g->dsv[j - 1] / diffpp;
                    ups = pec / (2.0 + fabs(pec));
                } else {
                    tv = 0.0;
                    ups = 0.0;
                }
                C2(cis, i, j) = C2(cin, i, j) * (1 + ups) + tv;
                C2(cin, i, j) = C2(cin, i, j) * (1 - ups) - tv;
            } else {
                /* gold_seaice.f90:966-992 */
                const int maxk = p->maxk;
                int kk = K1(i, j) > K1(i + 1, j) ? K1(i, j) : K1(i + 1, j);
                if (maxk < kk) {
                    C2(cie, i, j) = 0;
                    C2(ciw, i, j) = 0;
                } else {
                    C2(cie, i, j) = u1 * g->rc[j] * 0.5 * p->rdphi;
                    tv = g->rc[j] * g->rc[j] * p->rdphi * p->diffsic * p->rdphi;
                    pec = u1 * p->dphi / p->diffsic;
                    ups = pec / (2.0 + fabs(pec));
                    C2(ciw, i, j) = C2(cie, i, j) * (1 + ups) + tv;
                    C2(cie, i, j) = C2(cie, i, j) * (1 - ups) - tv;
                }
                kk = K1(i, j) > K1(i, j + 1) ? K1(i, j) : K1(i, j + 1);
                if (maxk < kk) {
                    C2(cin, i, j) = 0;
                    C2(cis, i, j) = 0;
                } else {
                    C2(cin, i, j) = g->cv[j] * u2 * 0.5;
                    tv = g->cv[j] * g->cv[j] * g->rdsv[j - 1] * p->diffsic;
                    pec = u2 * g->dsv[j - 1] / p->diffsic;
                    ups = pec / (2.0 + fabs(pec));
                    C2(cis, i, j) = C2(cin, i, j) * (1 + ups) + tv;
                    C2(cin, i, j) = C2(cin, i, j) * (1 - ups) - tv;
                }
            }
        }
    for (int j = 1; j <= maxj; ++j) {
        C2(cie, 0, j) = C2(cie, maxi, j);
        C2(ciw, 0, j) = C2(ciw, maxi, j);
    }
}

/* tstepsic, with the reference's west/south flux carries (gold_seaice.f90:844-929);
   tq = varice (written on wet cells), tq1 = varice1 */
static int tstepsic(const gb_ea_dims *d, const gb_ea_params *p, const gb_ea_grid *g, double *tq, const double *tq1,
                    const double *dtha, const double *u)
{
    const int maxi = d->maxi, maxj = d->maxj, maxk = p->maxk;
    double fe[2], fw[2], fn[2], fwsave[2];
    double *fs = calloc(2 * (size_t)maxi, sizeof(double));   /* fs(2, maxi) = 0 */
    if (!fs) return -2;
#define FS(l, i) fs[((l) - 1) + 2 * ((size_t)(i) - 1)]
    for (int j = 1; j <= maxj; ++j) {
        for (int l = 1; l <= 2; ++l) {
            const int kk = K1(maxi, j) > K1(1, j) ? K1(maxi, j) : K1(1, j);
            if (maxk >= kk) {
                fw[l - 1] = TQ(u, 1, maxi, j) * g->rc[j] * (TQ(tq1, l, 1, j) + TQ(tq1, l, maxi, j)) * 0.5;
                if (TQ(u, 1, maxi, j) >= 0.0) {
                    if (TQ(tq1, 2, 1, j) > p->sica_thresh) fw[l - 1] = 0;
                    if (TQ(tq1, 1, 1, j) > p->sich_thresh) fw[l - 1] = 0;
                } else {
                    if (TQ(tq1, 2, maxi, j) > p->sica_thresh) fw[l - 1] = 0;
                    if (TQ(tq1, 1, maxi, j) > p->sich_thresh) fw[l - 1] = 0;
                }
                fw[l - 1] = fw[l - 1] - (TQ(tq1, l, 1, j) - TQ(tq1, l, maxi, j)) * g->rc[j] * g->rc[j] * p->rdphi * p->diffsic;
            } else {
                fw[l - 1] = 0;
            }
            fwsave[l - 1] = fw[l - 1];
        }
        for (int i = 1; i <= maxi; ++i)
            for (int l = 1; l <= 2; ++l) {
                const int ke = K1(i, j) > K1(i + 1, j) ? K1(i, j) : K1(i + 1, j);
                if (i == maxi) {
                    fe[l - 1] = fwsave[l - 1];
                } else if (maxk < ke) {
                    fe[l - 1] = 0;
                } else {
                    fe[l - 1] = TQ(u, 1, i, j) * g->rc[j] * (TQ(tq1, l, i + 1, j) + TQ(tq1, l, i, j)) * 0.5;
                    if (TQ(u, 1, i, j) >= 0.0) {
                        if (TQ(tq1, 2, i + 1, j) > p->sica_thresh) fe[l - 1] = 0;
                        if (TQ(tq1, 1, i + 1, j) > p->sich_thresh) fe[l - 1] = 0;
                    } else {
                        if (TQ(tq1, 2, i, j) > p->sica_thresh) fe[l - 1] = 0;
                        if (TQ(tq1, 1, i, j) > p->sich_thresh) fe[l - 1] = 0;
                    }
                    fe[l - 1] = fe[l - 1] - (TQ(tq1, l, i + 1, j) - TQ(tq1, l, i, j)) * g->rc[j] * g->rc[j] * p->rdphi * p->diffsic;
                }
                const int kn = K1(i, j) > K1(i, j + 1) ? K1(i, j) : K1(i, j + 1);
                if (maxk < kn) {
                    fn[l - 1] = 0;
                } else {
                    /* j + 1 <= maxj here: row maxj + 1 is land */
                    fn[l - 1] = g->cv[j] * TQ(u, 2, i, j) * (TQ(tq1, l, i, j + 1) + TQ(tq1, l, i, j)) * 0.5;
                    if (TQ(u, 2, i, j) >= 0.0) {
                        if (TQ(tq1, 2, i, j + 1) > p->sica_thresh) fn[l - 1] = 0;
                        if (TQ(tq1, 1, i, j + 1) > p->sich_thresh) fn[l - 1] = 0;
                    } else {
                        if (TQ(tq1, 2, i, j) > p->sica_thresh) fn[l - 1] = 0;
                        if (TQ(tq1, 1, i, j) > p->sich_thresh) fn[l - 1] = 0;
                    }
                    fn[l - 1] = fn[l - 1] - g->cv[j] * g->cv[j] * (TQ(tq1, l, i, j + 1) - TQ(tq1, l, i, j)) * g->rdsv[j - 1] * p->diffsic;
                }
                if (maxk >= K1(i, j))
                    TQ(tq, l, i, j) = TQ(tq1, l, i, j) - p->dt * ((fe[l - 1] - fw[l - 1]) * p->rdphi + (fn[l - 1] - FS(l, i)) * g->rds[j - 1]) +
                                      p->tsc * p->dt * TQ(dtha, l, i, j);
                fw[l - 1] = fe[l - 1];
                FS(l, i) = fn[l - 1];
            }
    }
#undef FS
    free(fs);
    return 0;
}

int gbo_ea_step(const gb_ea_dims *d, const gb_ea_params *p, const gb_ea_grid *g, double *tq, double *tq1,
                const double *source, const double *vel, const double *pptn, int nsteps)
{
    const int maxi = d->maxi, maxj = d->maxj;
    if (maxi < 1 || maxj < 2 || nsteps < 0) return -1;
    if (p->kind == GB_EA_SEAICE_EXPLICIT) {
        if (nsteps > 1) return -1;
        return nsteps ? tstepsic(d, p, g, tq, tq1, source, vel) : 0;
    }
    if (p->kind == GB_EA_SEAICE && nsteps > 1) return -1;
    const size_t nc = (size_t)(maxi + 1) * (maxj + 1), nv = (size_t)(maxi + 2) * (maxj + 2);
    double *cie = calloc(nc, sizeof(double)), *ciw = calloc(nc, sizeof(double));
    double *cin = calloc(nc, sizeof(double)), *cis = calloc(nc, sizeof(double));
    double *v2 = calloc(nv, sizeof(double));
    if (!cie || !ciw || !cin || !cis || !v2) {
        free(cie); free(ciw); free(cin); free(cis); free(v2);
        return -2;
    }
    const double cimp = 0.5;
    const int nii = 4;
    const int ice = p->kind == GB_EA_SEAICE;
    const double dt = p->dt;
    for (int step = 0; step < nsteps; ++step) {
        for (int l = 1; l <= 2; ++l) {
            /* b.c. of the local arrays (embm.f90:2054-2059, gold_seaice.f90:952-957) */
            for (int i = 0; i <= maxi; ++i) {
                C2(cin, i, 0) = 0.0; C2(cis, i, 0) = 0.0;
                C2(cin, i, maxj) = 0.0; C2(cis, i, maxj) = 0.0;
            }
            for (int i = 0; i <= maxi + 1; ++i) {
                V2(v2, i, 0) = 0.0;
                V2(v2, i, maxj + 1) = 0.0;
            }
            coefficients(d, p, g, l, vel, pptn, cie, ciw, cin, cis);
            for (int it = 1; it <= nii + 1; ++it) {
                const int corr = it == nii + 1;
                for (int j = 1; j <= maxj; ++j)
                    for (int i = 1; i <= maxi; ++i) {
                        if (!corr)
                            V2(v2, i, j) = cimp * TQ(tq, l, i, j) + (1.0 - cimp) * TQ(tq1, l, i, j);
                        else
                            V2(v2, i, j) = 0.5 * (V2(v2, i, j) + cimp * TQ(tq, l, i, j) + (1.0 - cimp) * TQ(tq1, l, i, j));
                    }
                for (int j = 1; j <= maxj; ++j) {
                    V2(v2, 0, j) = V2(v2, maxi, j);
                    V2(v2, maxi + 1, j) = V2(v2, 1, j);
                }
                for (int j = 1; j <= maxj; ++j)
                    for (int i = 1; i <= maxi; ++i) {
                        if (ice && p->maxk < K1(i, j)) continue;
                        /* tstipa: -tqa(l,i,j); tstipsic: -dtha(l,i,j) * tsc */
                        const double src = ice ? -TQ(source, l, i, j) * p->tsc : -TQ(source, l, i, j);
                        const double flux = src + C2(cie, i, j) * V2(v2, i + 1, j) - C2(ciw, i - 1, j) * V2(v2, i - 1, j) +
                                            (C2(cin, i, j) * V2(v2, i, j + 1) - C2(cis, i, j - 1) * V2(v2, i, j - 1)) * g->rds[j - 1];
                        if (!corr) {
                            const double centre = dt * (C2(ciw, i, j) - C2(cie, i - 1, j) +
                                                        (C2(cis, i, j) - C2(cin, i, j - 1)) * g->rds[j - 1]);
                            TQ(tq, l, i, j) = (TQ(tq1, l, i, j) * (1.0 - (1.0 - cimp) * centre) - dt * flux) / (1 + cimp * centre);
                        } else {
                            TQ(tq, l, i, j) = TQ(tq1, l, i, j) - dt * flux -
                                              dt * V2(v2, i, j) * (C2(ciw, i, j) - C2(cie, i - 1, j) +
                                                                   (C2(cis, i, j) - C2(cin, i, j - 1)) * g->rds[j - 1]);
                        }
                    }
            }
        }
        if (!ice) memcpy(tq1, tq, sizeof(double) * 2 * (size_t)maxi * maxj);   /* tq1 = tq */
    }
    free(cie); free(ciw); free(cin); free(cis); free(v2);
    return 0;
}
