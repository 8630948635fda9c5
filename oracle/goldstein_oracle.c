/*
 * ORACLE -- test infrastructure only.  Nothing in the product links, loads or
 * calls this file; only the tests, the smoke check and bench.py's CPU-baseline
 * leg do, and only as the checker or the timed CPU reference.
 *
 * Line-for-line C restatement of the reference GOLDSTEIN tracer timestep:
 *   tstepo       src/goldstein/goldstein.f90:2280-2432   (imld = 0 and imld = 1)
 *   tstepo_flux  src/goldstein/goldstein.f90:2436-2642   (incl. diso branch :2561-2624)
 *   co           src/goldstein/goldstein.f90:2657-2777
 *   coshuffle    src/goldstein/goldstein.f90:2781-2841
 *   eos / eosd   src/goldstein/goldstein.f90:3048-3082
 *   krausturner  src/goldstein/goldstein.f90:3337-3442   (imld = 1)
 * The module state of src/goldstein/goldstein_lib.f90:6-180 is passed in through
 * the structs of include/gb_goldstein.h.  The reference is Fortran compiled with
 * -fdefault-real-8 and no FMA-capable -march (platforms/LINUX), so every
 * expression below is evaluated in IEEE double, left to right as gfortran
 * evaluates it, and this file must be compiled with -ffp-contract=off.
 *
 * Parity pin: no Fortran compiler exists on either build machine and the
 * reference ships no golden vectors for this routine, so this restatement is
 * pinned only by an independent NumPy restatement (oracle/goldstein_np.py) and
 * by conservation / invariance known-answer tests ("parity unpinned" against a
 * run of the reference itself).
 */
#include "../include/gb_goldstein.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int maxi, maxj, maxk, maxl;
    size_t NI, NJ;
    const gb_go_params *p;
    const gb_go_grid *g;
    double *ts, *ts1, *rho;
    const double *u;
    double *cost;
    int32_t *icosd;
    int32_t *mldpk;        /* (2, maxi, maxj): local of tstepo, kept for fidelity */
    /* imld = 1: diagnostics mld, mldk (maxi, maxj); scratch of tstepo: mldpelayer1 (maxi, maxj),
     * T and S before co (2, maxi, maxj, maxk), qmix of krausturner (maxl + 1) */
    double *mld;
    int32_t *mldk;
    double *pe1, *tsold, *qmix;
    double dmax;
    int32_t limps;
    /* scratch of tstepo_flux */
    double *fe, *fw, *fn, *fa, *fwsave, *fs, *fb, *dxts, *dyts, *dzts, *sum;
} ctx;

/* Fortran-bound accessors */
#define TSA(A, l, i, j, k) (A)[((size_t)(l) - 1) + (size_t)c->maxl * ((size_t)(i) + c->NI * ((size_t)(j) + c->NJ * (size_t)(k)))]
#define TS(l, i, j, k)  TSA(c->ts, l, i, j, k)
#define TS1(l, i, j, k) TSA(c->ts1, l, i, j, k)
#define U(cc, i, j, k) c->u[((size_t)(cc) - 1) + 3 * ((size_t)(i) + (size_t)(c->maxi + 1) * ((size_t)(j) + (size_t)(c->maxj + 1) * ((size_t)(k) - 1)))]
#define K1(i, j) c->g->k1[(size_t)(i) + c->NI * (size_t)(j)]
#define RHO(i, j, k) c->rho[(size_t)(i) + c->NI * ((size_t)(j) + c->NJ * (size_t)(k))]
#define COST(i, j) c->cost[((size_t)(i) - 1) + (size_t)c->maxi * ((size_t)(j) - 1)]
#define ICOSD(i, j) c->icosd[((size_t)(i) - 1) + (size_t)c->maxi * ((size_t)(j) - 1)]
#define MLDPK(n, i, j) c->mldpk[((size_t)(n) - 1) + 2 * (((size_t)(i) - 1) + (size_t)c->maxi * ((size_t)(j) - 1))]
#define RC(j)   c->g->rc[(j)]
#define RC2(j)  c->g->rc2[(j)]
#define CV(j)   c->g->cv[(j)]
#define CV2(j)  c->g->cv2[(j) - 1]
#define DSV(j)  c->g->dsv[(j) - 1]
#define RDSV(j) c->g->rdsv[(j) - 1]
#define RDS(j)  c->g->rds[(j) - 1]
#define DZ(k)   c->g->dz[(k) - 1]
#define DZA(k)  c->g->dza[(k) - 1]
#define RDZ(k)  c->g->rdz[(k) - 1]
#define RDZA(k) c->g->rdza[(k) - 1]
#define ZRO(k)  c->g->zro[(k) - 1]
#define DT(k)   c->g->dt[(k) - 1]
#define ZW(k)   c->g->zw[(k)]
#define SSMAX(k) c->g->ssmax[(k) - 1]
#define MLDDEC(k)  c->g->mlddec[(k) - 1]
#define MLDDECD(k) c->g->mlddecd[(k) - 1]
#define MLDKETAU(i, j) c->g->mldketau[((size_t)(i) - 1) + (size_t)c->maxi * ((size_t)(j) - 1)]
#define MLD(i, j)  c->mld[((size_t)(i) - 1) + (size_t)c->maxi * ((size_t)(j) - 1)]
#define MLDK(i, j) c->mldk[((size_t)(i) - 1) + (size_t)c->maxi * ((size_t)(j) - 1)]
#define PE1(i, j)  c->pe1[((size_t)(i) - 1) + (size_t)c->maxi * ((size_t)(j) - 1)]
#define TSOLD(l, i, j, k) c->tsold[((size_t)(l) - 1) + 2 * (((size_t)(i) - 1) + (size_t)c->maxi * (((size_t)(j) - 1) + (size_t)c->maxj * ((size_t)(k) - 1)))]
#define DIFFMAX(k) c->g->diffmax[(k) - 1]
#define EDIFF1(i, j, k) c->g->ediff1[((size_t)(i) - 1) + (size_t)c->maxi * (((size_t)(j) - 1) + (size_t)c->maxj * ((size_t)(k) - 1))]
/* tstepo_flux scratch: fs(maxl,maxi), fb(maxl,maxi,maxj), dxts(maxl,4), dyts(maxl,4) */
#define FS(l, i) c->fs[((l) - 1) + (size_t)c->maxl * ((i) - 1)]
#define FB(l, i, j) c->fb[((l) - 1) + (size_t)c->maxl * (((i) - 1) + (size_t)c->maxi * ((j) - 1))]
#define DXTS(l, n) c->dxts[((l) - 1) + (size_t)c->maxl * ((n) - 1)]
#define DYTS(l, n) c->dyts[((l) - 1) + (size_t)c->maxl * ((n) - 1)]

static int imax2(int a, int b) { return a > b ? a : b; }

/* eos, goldstein.f90:3048-3061.  gfortran expands t**2 as t*t and t**3 as
 * (t*t)*t; sums are evaluated left to right. */
static double eos(const double *ec, double t, double s, double z, int ieos)
{
    double rho;
    if (ieos == 0) {
        rho = ec[0] * t + ec[1] * s + ec[2] * (t * t) + ec[3] * ((t * t) * t);
    } else {
        rho = ec[0] * t + ec[1] * s + ec[2] * (t * t) + ec[3] * ((t * t) * t) + ec[4] * t * z;
    }
    return rho;
}

/* eosd, goldstein.f90:3064-3082 */
static void eosd(const double *ec, double t1, double t2, double s1, double s2,
                 double z, double rdz, int ieos, double *dzrho, double *tec)
{
    double tatw = 0.5 * (t1 + t2);
    if (ieos == 0) {
        *tec = -ec[0] - ec[2] * tatw * 2 - ec[3] * tatw * tatw * 3;
    } else {
        *tec = -ec[0] - ec[2] * tatw * 2 - ec[3] * tatw * tatw * 3 - ec[4] * z;
    }
    *dzrho = (ec[1] * (s2 - s1) - *tec * (t2 - t1)) * rdz;
}

/* tstepo_flux, goldstein.f90:2436-2642 */
static void tstepo_flux(ctx *c)
{
    const gb_go_params *p = c->p;
    const gb_go_grid *g = c->g;
    const int maxi = c->maxi, maxj = c->maxj, maxk = c->maxk, maxl = c->maxl;
    const double *ec = p->ec;
    double tv, ups[3], pec[3];
    double *fe = c->fe, *fw = c->fw, *fn = c->fn, *fa = c->fa, *fwsave = c->fwsave, *dzts = c->dzts;
    double diffv;
    double tec = 0.0, scc, dzrho = 0.0, rdzrho, slim, tv1;
    double dxrho[5], dyrho[5];
    int i, j, k, l, ina, nnp, knp;

    scc = 0.0;
    rdzrho = 0.0;
    if (p->diso) {
        scc = ec[1];
        c->limps = 0;
    }
    diffv = p->diff[1];
    c->dmax = 0;

    memset(c->fb, 0, sizeof(double) * (size_t)maxl * maxi * maxj);

    for (k = 1; k <= maxk; ++k) {
        memset(c->fs, 0, sizeof(double) * (size_t)maxl * maxi);
        for (j = 1; j <= maxj; ++j) {
            /* western boundary fluxes */
            pec[0] = U(1, maxi, j, k) * g->dphi / p->diff[0];
            ups[0] = pec[0] / (2.0 + fabs(pec[0]));
            for (l = 1; l <= maxl; ++l) {
                if (k >= imax2(K1(maxi, j), K1(1, j))) {
                    fw[l] = U(1, maxi, j, k) * RC(j) *
                            ((1.0 - ups[0]) * TS1(l, 1, j, k) + (1.0 + ups[0]) * TS1(l, maxi, j, k)) * 0.5;
                    fw[l] = fw[l] - (TS1(l, 1, j, k) - TS1(l, maxi, j, k)) * RC2(j) * p->diff[0];
                } else {
                    fw[l] = 0;
                }
                fwsave[l] = fw[l];
            }
            for (i = 1; i <= maxi; ++i) {
                /* local vertical diffusivity */
                if (k >= K1(i, j) && k < maxk) {
                    eosd(ec, TS1(1, i, j, k), TS1(1, i, j, k + 1), TS1(2, i, j, k), TS1(2, i, j, k + 1),
                         ZW(k), RDZA(k), p->ieos, &dzrho, &tec);
                    if (dzrho < -1.0e-12) {
                        rdzrho = 1.0 / dzrho;
                    } else {
                        rdzrho = -1.0e12;
                    }
                    if (p->iediff > 0 && p->iediff < 3) {
                        if (p->ediffpow2i == 0) {
                            diffv = p->ediff0 + EDIFF1(i, j, k);
                        } else if (p->ediffpow2i == 1) {
                            diffv = p->ediff0 + EDIFF1(i, j, k) * (-rdzrho);
                        } else if (p->ediffpow2i == 2) {
                            diffv = p->ediff0 + EDIFF1(i, j, k) * sqrt(-rdzrho);
                        } else {
                            diffv = p->ediff0 + EDIFF1(i, j, k) * pow(-rdzrho, p->ediffpow2);
                        }
                        if (diffv > DIFFMAX(k + 1)) diffv = DIFFMAX(k + 1);
                    }
                }
                pec[0] = U(1, i, j, k) * g->dphi / p->diff[0];
                ups[0] = pec[0] / (2.0 + fabs(pec[0]));
                pec[1] = U(2, i, j, k) * DSV(j < maxj - 1 ? j : maxj - 1) / p->diff[0];
                ups[1] = pec[1] / (2.0 + fabs(pec[1]));
                pec[2] = U(3, i, j, k) * DZA(k) / diffv;
                ups[2] = pec[2] / (2.0 + fabs(pec[2]));
                for (l = 1; l <= maxl; ++l) {
                    /* flux to east */
                    if (i == maxi) {
                        fe[l] = fwsave[l];
                    } else if (k < imax2(K1(i, j), K1(i + 1, j))) {
                        fe[l] = 0;
                    } else {
                        fe[l] = U(1, i, j, k) * RC(j) *
                                ((1.0 - ups[0]) * TS1(l, i + 1, j, k) + (1.0 + ups[0]) * TS1(l, i, j, k)) * 0.5;
                        fe[l] = fe[l] - (TS1(l, i + 1, j, k) - TS1(l, i, j, k)) * RC2(j) * p->diff[0];
                    }
                    /* flux to north */
                    if (k < imax2(K1(i, j), K1(i, j + 1))) {
                        fn[l] = 0;
                    } else {
                        fn[l] = CV(j) * U(2, i, j, k) *
                                ((1.0 - ups[1]) * TS1(l, i, j + 1, k) + (1.0 + ups[1]) * TS1(l, i, j, k)) * 0.5;
                        fn[l] = fn[l] - CV2(j) * (TS1(l, i, j + 1, k) - TS1(l, i, j, k)) * p->diff[0];
                    }
                    /* flux above */
                    if (k < K1(i, j)) {
                        fa[l] = 0;
                    } else if (k == maxk) {
                        fa[l] = TS(l, i, j, maxk + 1);
                    } else {
                        fa[l] = U(3, i, j, k) *
                                ((1.0 - ups[2]) * TS1(l, i, j, k + 1) + (1.0 + ups[2]) * TS1(l, i, j, k)) * 0.5;
                        fa[l] = fa[l] - (TS1(l, i, j, k + 1) - TS1(l, i, j, k)) * RDZA(k) * diffv;
                    }
                }
                if (p->diso) {
                    /* isoneutral diffusion */
                    if (k >= K1(i, j) && k < maxk) {
                        if (dzrho < -1.0e-12) {
                            tv1 = 0.0;
                            for (knp = 0; knp <= 1; ++knp) {
                                for (nnp = 0; nnp <= 1; ++nnp) {
                                    ina = 1 + nnp + 2 * knp;
                                    for (l = 1; l <= maxl; ++l) {
                                        if (k + knp >= K1(i - 1 + 2 * nnp, j)) {
                                            DXTS(l, ina) = (TS1(l, i + nnp, j, k + knp) - TS1(l, i + nnp - 1, j, k + knp)) *
                                                           RC(j) * g->rdphi;
                                        } else {
                                            DXTS(l, ina) = 0.0;
                                        }
                                        if (k + knp >= K1(i, j - 1 + 2 * nnp)) {
                                            DYTS(l, ina) = (TS1(l, i, j + nnp, k + knp) - TS1(l, i, j + nnp - 1, k + knp)) *
                                                           CV(j - 1 + nnp) * RDSV(j + nnp - 1);
                                        } else {
                                            DYTS(l, ina) = 0.0;
                                        }
                                    }
                                    dxrho[ina] = scc * DXTS(2, ina) - tec * DXTS(1, ina);
                                    dyrho[ina] = scc * DYTS(2, ina) - tec * DYTS(1, ina);
                                    tv1 = tv1 + dxrho[ina] * dxrho[ina] + dyrho[ina] * dyrho[ina];
                                }
                            }
                            tv1 = 0.25 * tv1 * rdzrho * rdzrho;
                            if (tv1 > SSMAX(k)) {
                                slim = SSMAX(k) * SSMAX(k) / (tv1 * tv1);
                                c->limps = c->limps + 1;
                            } else {
                                slim = 1.0;
                            }
                            tv1 = tv1 * slim * p->diff[0] * RDZA(k);
                            tv = tv1 * DT(k) * RDZA(k);
                            if (tv > c->dmax) c->dmax = tv;
                            for (l = 1; l <= maxl; ++l) {
                                dzts[l] = (TS1(l, i, j, k + 1) - TS1(l, i, j, k)) * RDZA(k);
                                tv = 0;
                                for (ina = 1; ina <= 4; ++ina) {
                                    tv = tv + (2 * dzrho * DXTS(l, ina) - dxrho[ina] * dzts[l]) * dxrho[ina] +
                                         (2 * dzrho * DYTS(l, ina) - dyrho[ina] * dzts[l]) * dyrho[ina];
                                }
                                tv = 0.25 * slim * p->diff[0] * tv / (dzrho * dzrho);
                                fa[l] = fa[l] + tv;
                            }
                        }
                    }
                }
                for (l = 1; l <= maxl; ++l) {
                    tv = 0;
                    if (k >= K1(i, j)) {
                        TS(l, i, j, k) = TS1(l, i, j, k) -
                                         DT(k) * (-tv + (fe[l] - fw[l]) * g->rdphi + (fn[l] - FS(l, i)) * RDS(j) +
                                                  (fa[l] - FB(l, i, j)) * RDZ(k));
                    }
                    fw[l] = fe[l];
                    FS(l, i) = fn[l];
                    FB(l, i, j) = fa[l];
                }
                RHO(i, j, k) = eos(ec, TS(1, i, j, k), TS(2, i, j, k), ZRO(k), p->ieos);
            }
        }
    }
}

/* coshuffle, goldstein.f90:2781-2841 (tv is ts) */
static void coshuffle(ctx *c)
{
    const gb_go_params *p = c->p;
    const int maxi = c->maxi, maxj = c->maxj, maxk = c->maxk, maxl = c->maxl;
    const double *ec = p->ec;
    double tv_temp;
    int i, j, k, k0, l, ipass, maxpass;

    maxpass = maxk;
    for (j = 1; j <= maxj; ++j) {
        for (i = 1; i <= maxi; ++i) {
            if (K1(i, j) <= maxk) {
                ICOSD(i, j) = 0;
                k0 = 0;
                ipass = 0;
                while (k0 < maxk && ipass < maxpass) {
                    ipass = ipass + 1;
                    k = maxk - 1;
                    if (p->ieos != 0) {
                        RHO(i, j, maxk) = eos(ec, TS(1, i, j, maxk), TS(2, i, j, maxk), ZW(k), p->ieos);
                        RHO(i, j, k) = eos(ec, TS(1, i, j, k), TS(2, i, j, k), ZW(k), p->ieos);
                    }
                    while ((RHO(i, j, maxk) > RHO(i, j, k)) && (k >= K1(i, j))) {
                        k = k - 1;
                        if (p->ieos != 0) {
                            RHO(i, j, maxk) = eos(ec, TS(1, i, j, maxk), TS(2, i, j, maxk), ZW(k), p->ieos);
                            RHO(i, j, k) = eos(ec, TS(1, i, j, k), TS(2, i, j, k), ZW(k), p->ieos);
                        }
                    }
                    MLDPK(2, i, j) = k0;
                    k0 = k + 1;
                    if (k0 < maxk) {
                        for (l = 1; l <= maxl; ++l) {
                            tv_temp = TS(l, i, j, maxk);
                            for (k = maxk; k >= k0 + 1; --k) {
                                TS(l, i, j, k) = ((DZ(k) - DZ(maxk)) * TS(l, i, j, k) + DZ(maxk) * TS(l, i, j, k - 1)) * RDZ(k);
                            }
                            TS(l, i, j, k0) = ((DZ(k0) - DZ(maxk)) * TS(l, i, j, k0) + DZ(maxk) * tv_temp) * RDZ(k0);
                        }
                        for (k = k0; k <= maxk; ++k) {
                            RHO(i, j, k) = eos(ec, TS(1, i, j, k), TS(2, i, j, k), ZW(maxk - 1), p->ieos);
                        }
                        if (maxk - k0 > ICOSD(i, j)) ICOSD(i, j) = maxk - k0;
                    }
                }
            }
        }
    }
}

/* co, goldstein.f90:2657-2777 (tv is ts) */
static void co(ctx *c)
{
    const gb_go_params *p = c->p;
    const int maxi = c->maxi, maxj = c->maxj, maxk = c->maxk, maxl = c->maxl;
    const double *ec = p->ec;
    const int ieos = p->ieos;
    double dzm[GB_GO_MAX_K + 1];
    double *sum = c->sum;
    int kk[GB_GO_MAX_K + 1];
    int i, j, l, lastmix, m, n, ni, icond;

    icond = 0;
    if (p->iconv == 1) coshuffle(c);

    for (j = 1; j <= maxj; ++j) {
        for (i = 1; i <= maxi; ++i) {
            if (K1(i, j) <= maxk) {
                if (p->iconv == 1) icond = 0;
                kk[K1(i, j) - 1] = 0;
                for (m = K1(i, j); m <= maxk; ++m) {
                    kk[m] = m;
                    dzm[m] = DZ(m);
                }
                m = maxk;
                lastmix = 0;
                while (kk[m - 1] > 0 || (lastmix != 0 && kk[m] != maxk)) {
                    if (ieos != 0) {
                        RHO(i, j, kk[m]) = eos(ec, TS(1, i, j, kk[m]), TS(2, i, j, kk[m]), ZW(kk[m - 1]), ieos);
                        RHO(i, j, kk[m - 1]) = eos(ec, TS(1, i, j, kk[m - 1]), TS(2, i, j, kk[m - 1]), ZW(kk[m - 1]), ieos);
                    }
                    if (RHO(i, j, kk[m]) < RHO(i, j, kk[m - 1]) || kk[m - 1] == 0) {
                        if (lastmix == 0 || kk[m] == maxk) {
                            m = m - 1;
                        } else {
                            m = m + 1;
                        }
                        lastmix = 0;
                    } else {
                        lastmix = 1;
                        n = m - 1;
                        if (ieos != 0) {
                            RHO(i, j, kk[n]) = eos(ec, TS(1, i, j, kk[n]), TS(2, i, j, kk[n]), ZW(kk[n - 1]), ieos);
                            RHO(i, j, kk[n - 1]) = eos(ec, TS(1, i, j, kk[n - 1]), TS(2, i, j, kk[n - 1]), ZW(kk[n - 1]), ieos);
                        }
                        while (kk[n - 1] > 0 && RHO(i, j, kk[n]) >= RHO(i, j, kk[n - 1])) {
                            n = n - 1;
                            if (ieos != 0) {
                                RHO(i, j, kk[n]) = eos(ec, TS(1, i, j, kk[n]), TS(2, i, j, kk[n]), ZW(kk[n - 1]), ieos);
                                RHO(i, j, kk[n - 1]) = eos(ec, TS(1, i, j, kk[n - 1]), TS(2, i, j, kk[n - 1]), ZW(kk[n - 1]), ieos);
                            }
                        }
                        for (l = 1; l <= maxl; ++l) sum[l] = TS(l, i, j, kk[m]) * dzm[kk[m]];
                        for (ni = 1; ni <= m - n; ++ni) {
                            for (l = 1; l <= maxl; ++l) sum[l] = sum[l] + TS(l, i, j, kk[m - ni]) * dzm[kk[m - ni]];
                            dzm[kk[m]] = dzm[kk[m]] + dzm[kk[m - ni]];
                        }
                        for (l = 1; l <= maxl; ++l) TS(l, i, j, kk[m]) = sum[l] / dzm[kk[m]];
                        RHO(i, j, kk[m]) = eos(ec, TS(1, i, j, kk[m]), TS(2, i, j, kk[m]), ZW(kk[m - 1]), ieos);
                        /* reindex k(m) */
                        ni = m - 1;
                        while (kk[ni + 1] > 0) {
                            kk[ni] = kk[ni - m + n];
                            ni = ni - 1;
                        }
                    }
                }
                /* fill in T,S values in mixed regions */
                m = maxk - 1;
                for (n = maxk - 1; n >= K1(i, j); --n) {
                    if (n > kk[m]) {
                        for (l = 1; l <= maxl; ++l) TS(l, i, j, n) = TS(l, i, j, kk[m + 1]);
                        RHO(i, j, n) = eos(ec, TS(1, i, j, n), TS(2, i, j, n), ZW(kk[n - 1]), ieos);
                        if (p->iconv == 1) {
                            icond = icond + 1;
                        } else {
                            COST(i, j) = COST(i, j) + 1.0;
                        }
                    } else {
                        m = m - 1;
                    }
                }
                if (p->iconv == 1) {
                    if (icond > ICOSD(i, j)) ICOSD(i, j) = icond;
                    COST(i, j) = p->dsc * ZW(maxk - 1 - ICOSD(i, j));
                }
                MLDPK(1, i, j) = kk[m + 1];
            }
        }
    }
}

/* Level-pair depth grids of the mixed-layer scheme, goldstein.f90:1013-1025:
 * dzg(k,kk) = zw(k) - zw(kk-1), z2dzg(k,kk) = -zw(k)^2 + zw(kk-1)^2,
 * rdzg(k,kk) = 1/dzg(k,kk), or 1e10 where k = kk-1. */
static double dzg(const ctx *c, int k, int kk) { return ZW(k) - ZW(kk - 1); }
static double z2dzg(const ctx *c, int k, int kk) { return -ZW(k) * ZW(k) + ZW(kk - 1) * ZW(kk - 1); }
static double rdzg(const ctx *c, int k, int kk) { return k != kk - 1 ? 1.0 / dzg(c, k, kk) : 1.0E10; }

/* Energy of mixing the surface forcing over the top layer, goldstein.f90:2294-2309
 * (before the flux step: rho is still the previous step's). */
static void mld_layer1(ctx *c)
{
    const int maxi = c->maxi, maxj = c->maxj, maxk = c->maxk;
    const gb_go_params *p = c->p;
    for (int j = 1; j <= maxj; ++j)
        for (int i = 1; i <= maxi; ++i) {
            const double t = TS(1, i, j, maxk) - TS(1, i, j, maxk + 1);
            const double s = TS(2, i, j, maxk) - TS(2, i, j, maxk + 1);
            const double r = eos(p->ec, t, s, ZRO(maxk), p->ieos);
            PE1(i, j) = (r - RHO(i, j, maxk)) * z2dzg(c, maxk, maxk);
        }
}

/* krausturner, goldstein.f90:3337-3442, on column (i, j) */
static void krausturner(ctx *c, int i, int j, double pebuoy, double ketau)
{
    const int maxk = c->maxk, maxl = c->maxl, tvkl = K1(i, j);
    const gb_go_params *p = c->p;
    const double *ec = p->ec;
    double *qmix = c->qmix;
    const int mldpk = maxk;   /* the routine's first statement (goldstein.f90:3350) */
    int k = mldpk, l, n, partmix = 1;
    double empe = pebuoy;
    double emke = ketau * MLDDEC(k);
    double em = empe + emke;
    double eneed = 0.0;
    double tmix = TS(1, i, j, k), smix = TS(2, i, j, k);
    double rhomix, rhou = 0.0, rhol = 0.0, emr;
    for (l = 1; l <= maxl; ++l) qmix[l] = TS(l, i, j, k);
    rhomix = eos(ec, tmix, smix, ZW(k), p->ieos);
    while (eneed < em && em > 0) {
        if (k < mldpk) {
            qmix[1] = tmix;
            qmix[2] = smix;
            for (l = 3; l <= maxl; ++l)
                qmix[l] = rdzg(c, maxk, k) * (qmix[l] * dzg(c, maxk, k + 1) + TS(l, i, j, k) * DZ(k));
        }
        if (k == tvkl) {
            MLDK(i, j) = k;
            MLD(i, j) = ZW(k - 1);
            partmix = 0;
            em = -1.0E-8;
            if (k < maxk)
                for (l = 1; l <= maxl; ++l)
                    for (n = k; n <= maxk; ++n) TS(l, i, j, n) = qmix[l];
        } else {
            k = k - 1;
            emr = (em - eneed) / em;
            empe = empe * emr;
            emke = emke * emr * MLDDECD(k);
            em = empe + emke;
            rhou = p->ieos != 0 ? eos(ec, tmix, smix, ZW(k), p->ieos) : rhomix;
            tmix = rdzg(c, maxk, k) * (tmix * dzg(c, maxk, k + 1) + TS(1, i, j, k) * DZ(k));
            smix = rdzg(c, maxk, k) * (smix * dzg(c, maxk, k + 1) + TS(2, i, j, k) * DZ(k));
            rhol = eos(ec, TS(1, i, j, k), TS(2, i, j, k), ZW(k), p->ieos);
            rhomix = eos(ec, tmix, smix, ZW(k), p->ieos);
            eneed = z2dzg(c, maxk, k + 1) * rhou + z2dzg(c, k, k) * rhol - z2dzg(c, maxk, k) * rhomix;
        }
    }
    if (partmix == 1 && em > 0) {
        double mlda, mldb;
        MLDK(i, j) = k;
        mlda = dzg(c, maxk, k + 1) * rdzg(c, maxk, k) * em / eneed;
        mldb = (dzg(c, maxk, k) * rdzg(c, maxk, k + 1) - 1) * mlda;
        for (l = 1; l <= maxl; ++l) {
            TS(l, i, j, maxk) = (1 - mldb) * qmix[l] + mldb * TS(l, i, j, k);
            for (n = k + 1; n <= maxk - 1; ++n) TS(l, i, j, n) = TS(l, i, j, maxk);
            TS(l, i, j, k) = mlda * qmix[l] + (1 - mlda) * TS(l, i, j, k);
        }
        if (k < maxk) MLD(i, j) = ZW(k) + em / (ZW(k) * (rhol - rhou));
        else MLD(i, j) = 0.0;
    } else if (partmix == 1 && k < maxk) {
        MLDK(i, j) = k + 1;
        MLD(i, j) = ZW(k);
    }
}

/* co with the mixed-layer scheme around it, goldstein.f90:2318-2389 */
static void co_mld(ctx *c)
{
    const int maxi = c->maxi, maxj = c->maxj, maxk = c->maxk;
    const gb_go_params *p = c->p;
    int i, j, k;
    /* T and S before co, every level of the wet columns (the PE change uses only these two) */
    for (i = 1; i <= maxi; ++i)
        for (j = 1; j <= maxj; ++j)
            if (K1(i, j) <= maxk)
                for (k = 1; k <= maxk; ++k) {
                    TSOLD(1, i, j, k) = TS(1, i, j, k);
                    TSOLD(2, i, j, k) = TS(2, i, j, k);
                }
    co(c);
    for (i = 1; i <= maxi; ++i)
        for (j = 1; j <= maxj; ++j) {
            if (K1(i, j) > maxk) continue;
            double peconv = 0.0, pebuoy, emix;
            for (k = maxk; k > 0; --k) {
                const double rold = eos(p->ec, TSOLD(1, i, j, k), TSOLD(2, i, j, k), ZRO(k), p->ieos);
                const double rnew = eos(p->ec, TS(1, i, j, k), TS(2, i, j, k), ZRO(k), p->ieos);
                peconv = peconv + (rnew - rold) * z2dzg(c, k, k);
            }
            pebuoy = peconv + PE1(i, j);
            if (pebuoy > 0.0) pebuoy = pebuoy * p->mldpebuoycoeff;
            emix = pebuoy + MLDKETAU(i, j) * MLDDEC(maxk);
            if (emix > 0.0) {
                krausturner(c, i, j, pebuoy, MLDKETAU(i, j));
            } else {
                MLDK(i, j) = maxk;
                if (PE1(i, j) < 0) MLD(i, j) = ZW(maxk - 1) * (1 - emix / PE1(i, j));
                else MLD(i, j) = ZW(maxk - 1);
            }
        }
}

/* dead copies of tstepo (goldstein.f90:2311-2316): kept in faithful mode so the
 * timed CPU baseline moves the same bytes as the reference */
typedef struct {
    double *ts_t1, *ts1_t1, *ts_t2, *ts1_t2, *rho_t1, *rho_t2;
} dead_copies;

static void do_dead_copies(ctx *c, dead_copies *d)
{
    const int maxi = c->maxi, maxj = c->maxj, maxk = c->maxk, maxl = c->maxl;
    size_t n = 0, m = 0;
    for (int k = 1; k <= maxk; ++k)
        for (int j = 1; j <= maxj; ++j)
            for (int i = 1; i <= maxi; ++i) {
                for (int l = 1; l <= maxl; ++l) {
                    d->ts_t1[n] = TS(l, i, j, k);
                    d->ts1_t1[n] = TS1(l, i, j, k);
                    d->ts_t2[n] = TS(l, i, j, k);
                    d->ts1_t2[n] = TS1(l, i, j, k);
                    ++n;
                }
                d->rho_t1[m] = RHO(i, j, k);
                d->rho_t2[m] = RHO(i, j, k);
                ++m;
            }
}

/* tstepo, goldstein.f90:2280-2432 */
static void tstepo(ctx *c, dead_copies *d)
{
    const int maxi = c->maxi, maxj = c->maxj, maxk = c->maxk, maxl = c->maxl;
    const gb_go_params *p = c->p;
    int i, j, k, l;

    if (p->imld == 1) mld_layer1(c);
    if (d) do_dead_copies(c, d);
    tstepo_flux(c);
    if (p->imld == 1) co_mld(c);
    else co(c);

    if (p->ieos != 0) {
        for (i = 1; i <= maxi; ++i)
            for (j = 1; j <= maxj; ++j)
                if (K1(i, j) <= maxk)
                    for (k = 1; k <= maxk; ++k)
                        RHO(i, j, k) = eos(p->ec, TS(1, i, j, k), TS(2, i, j, k), ZRO(k), p->ieos);
    }

    /* periodic b.c. for rho and ts1 */
    for (j = 1; j <= maxj; ++j) {
        for (k = K1(0, j); k <= maxk; ++k) {
            RHO(0, j, k) = RHO(maxi, j, k);
            for (l = 1; l <= maxl; ++l) TS1(l, 0, j, k) = TS(l, maxi, j, k);
        }
        for (k = K1(maxi + 1, j); k <= maxk; ++k) {
            RHO(maxi + 1, j, k) = RHO(1, j, k);
            for (l = 1; l <= maxl; ++l) TS1(l, maxi + 1, j, k) = TS(l, 1, j, k);
        }
    }

    for (k = 1; k <= maxk; ++k)
        for (j = 1; j <= maxj; ++j)
            for (i = 1; i <= maxi; ++i)
                for (l = 1; l <= maxl; ++l)
                    if (k >= K1(i, j)) TS1(l, i, j, k) = TS(l, i, j, k);
}

static int check_args(const gb_go_dims *dims, const gb_go_params *p, const gb_go_grid *g)
{
    if (!dims || !p || !g) return GB_GO_EINVAL;
    if (dims->maxi < 2 || dims->maxj < 3 || dims->maxk < 2 || dims->maxl < 2) return GB_GO_EINVAL;
    if (dims->maxk > GB_GO_MAX_K || dims->maxl > GB_GO_MAX_L) return GB_GO_ERANGE;
    if (p->imld != 0 && p->imld != 1) return GB_GO_EINVAL;
    if (p->imld == 1 && (!g->mlddec || !g->mlddecd || !g->mldketau)) return GB_GO_EINVAL;
    if (p->ieos != 0 && p->ieos != 1) return GB_GO_EINVAL;
    if (p->iconv != 0 && p->iconv != 1) return GB_GO_EINVAL;
    if (!g->k1 || !g->rc || !g->rc2 || !g->cv || !g->cv2 || !g->dsv || !g->rdsv || !g->rds ||
        !g->dz || !g->dza || !g->rdz || !g->rdza || !g->zro || !g->dt || !g->zw)
        return GB_GO_EINVAL;
    if (p->diso && !g->ssmax) return GB_GO_EINVAL;
    if (p->iediff > 0 && p->iediff < 3 && (!g->ediff1 || !g->diffmax)) return GB_GO_EINVAL;
    return GB_GO_OK;
}

static int ctx_init(ctx *c, const gb_go_dims *dims, const gb_go_params *p, const gb_go_grid *g)
{
    memset(c, 0, sizeof(*c));
    c->maxi = dims->maxi; c->maxj = dims->maxj; c->maxk = dims->maxk; c->maxl = dims->maxl;
    c->NI = (size_t)dims->maxi + 2; c->NJ = (size_t)dims->maxj + 2;
    c->p = p; c->g = g;
    size_t L = (size_t)dims->maxl + 1;
    c->fe = calloc(L, sizeof(double)); c->fw = calloc(L, sizeof(double));
    c->fn = calloc(L, sizeof(double)); c->fa = calloc(L, sizeof(double));
    c->fwsave = calloc(L, sizeof(double)); c->dzts = calloc(L, sizeof(double));
    c->sum = calloc(L, sizeof(double));
    c->fs = calloc((size_t)dims->maxl * dims->maxi, sizeof(double));
    c->fb = calloc((size_t)dims->maxl * dims->maxi * dims->maxj, sizeof(double));
    c->dxts = calloc((size_t)dims->maxl * 4, sizeof(double));
    c->dyts = calloc((size_t)dims->maxl * 4, sizeof(double));
    c->mldpk = calloc((size_t)2 * dims->maxi * dims->maxj, sizeof(int32_t));
    if (!c->fe || !c->fw || !c->fn || !c->fa || !c->fwsave || !c->dzts || !c->sum || !c->fs || !c->fb ||
        !c->dxts || !c->dyts || !c->mldpk)
        return GB_GO_ENOMEM;
    if (p->imld == 1) {
        const size_t ncol = (size_t)dims->maxi * dims->maxj;
        c->pe1 = calloc(ncol, sizeof(double));
        c->tsold = calloc(2 * ncol * (size_t)dims->maxk, sizeof(double));
        c->qmix = calloc(L, sizeof(double));
        if (!c->pe1 || !c->tsold || !c->qmix) return GB_GO_ENOMEM;
    }
    return GB_GO_OK;
}

static void ctx_free(ctx *c)
{
    free(c->fe); free(c->fw); free(c->fn); free(c->fa); free(c->fwsave); free(c->dzts);
    free(c->sum); free(c->fs); free(c->fb); free(c->dxts); free(c->dyts); free(c->mldpk);
    free(c->pe1); free(c->tsold); free(c->qmix);
}

/*
 * Advance `nsteps` tracer steps in place on Fortran-layout arrays (the index
 * maps of include/gb_goldstein.h).  cost/icosd (and, for imld = 1, the mixed-layer
 * diagnostics mld/mldk, (maxi, maxj)) may be NULL (then a zeroed internal array is
 * used).  faithful != 0 performs the reference's dead array copies each step.
 * Returns 0 or a GB_GO_E* code.
 */
int gbo_tstepo_mld(const gb_go_dims *dims, const gb_go_params *p, const gb_go_grid *g,
                   double *ts, double *ts1, double *rho, const double *u,
                   double *cost, int32_t *icosd, double *dmax, int32_t *limps,
                   int32_t nsteps, int32_t faithful, double *mld, int32_t *mldk)
{
    int rc = check_args(dims, p, g);
    if (rc) return rc;
    if (!ts || !ts1 || !rho || !u || nsteps < 0) return GB_GO_EINVAL;
    ctx c;
    rc = ctx_init(&c, dims, p, g);
    double *own_cost = NULL;
    int32_t *own_icosd = NULL;
    dead_copies d = {0};
    size_t ncol = (size_t)dims->maxi * dims->maxj;
    size_t nts = (size_t)dims->maxl * ncol * dims->maxk;
    if (rc == GB_GO_OK && !cost) { own_cost = calloc(ncol, sizeof(double)); if (!own_cost) rc = GB_GO_ENOMEM; }
    if (rc == GB_GO_OK && !icosd) { own_icosd = calloc(ncol, sizeof(int32_t)); if (!own_icosd) rc = GB_GO_ENOMEM; }
    double *own_mld = NULL;
    int32_t *own_mldk = NULL;
    if (rc == GB_GO_OK && !mld) { own_mld = calloc(ncol, sizeof(double)); if (!own_mld) rc = GB_GO_ENOMEM; }
    if (rc == GB_GO_OK && !mldk) { own_mldk = calloc(ncol, sizeof(int32_t)); if (!own_mldk) rc = GB_GO_ENOMEM; }
    if (rc == GB_GO_OK && faithful) {
        d.ts_t1 = malloc(nts * sizeof(double)); d.ts1_t1 = malloc(nts * sizeof(double));
        d.ts_t2 = malloc(nts * sizeof(double)); d.ts1_t2 = malloc(nts * sizeof(double));
        d.rho_t1 = malloc(ncol * dims->maxk * sizeof(double)); d.rho_t2 = malloc(ncol * dims->maxk * sizeof(double));
        if (!d.ts_t1 || !d.ts1_t1 || !d.ts_t2 || !d.ts1_t2 || !d.rho_t1 || !d.rho_t2) rc = GB_GO_ENOMEM;
    }
    if (rc == GB_GO_OK) {
        c.ts = ts; c.ts1 = ts1; c.rho = rho; c.u = u;
        c.cost = cost ? cost : own_cost;
        c.icosd = icosd ? icosd : own_icosd;
        c.mld = mld ? mld : own_mld;
        c.mldk = mldk ? mldk : own_mldk;
        c.dmax = 0; c.limps = 0;
        for (int s = 0; s < nsteps; ++s) tstepo(&c, faithful ? &d : NULL);
        if (dmax) *dmax = c.dmax;
        if (limps) *limps = c.limps;
    }
    free(own_cost); free(own_icosd); free(own_mld); free(own_mldk);
    free(d.ts_t1); free(d.ts1_t1); free(d.ts_t2); free(d.ts1_t2); free(d.rho_t1); free(d.rho_t2);
    ctx_free(&c);
    return rc;
}

int gbo_tstepo(const gb_go_dims *dims, const gb_go_params *p, const gb_go_grid *g,
               double *ts, double *ts1, double *rho, const double *u,
               double *cost, int32_t *icosd, double *dmax, int32_t *limps,
               int32_t nsteps, int32_t faithful)
{
    return gbo_tstepo_mld(dims, p, g, ts, ts1, rho, u, cost, icosd, dmax, limps, nsteps, faithful, NULL, NULL);
}

/* The flux part alone (tstepo_flux), for unit tests of the pieces. */
int gbo_tstepo_flux(const gb_go_dims *dims, const gb_go_params *p, const gb_go_grid *g,
                    double *ts, const double *ts1, double *rho, const double *u,
                    double *dmax, int32_t *limps)
{
    int rc = check_args(dims, p, g);
    if (rc) return rc;
    ctx c;
    rc = ctx_init(&c, dims, p, g);
    if (rc == GB_GO_OK) {
        c.ts = ts; c.ts1 = (double *)ts1; c.rho = rho; c.u = u;
        tstepo_flux(&c);
        if (dmax) *dmax = c.dmax;
        if (limps) *limps = c.limps;
    }
    ctx_free(&c);
    return rc;
}

/* Convective adjustment alone (co, with coshuffle first when iconv=1). */
int gbo_co(const gb_go_dims *dims, const gb_go_params *p, const gb_go_grid *g,
           double *ts, double *rho, double *cost, int32_t *icosd)
{
    int rc = check_args(dims, p, g);
    if (rc) return rc;
    if (!ts || !rho || !cost || !icosd) return GB_GO_EINVAL;
    ctx c;
    rc = ctx_init(&c, dims, p, g);
    if (rc == GB_GO_OK) {
        c.ts = ts; c.rho = rho; c.cost = cost; c.icosd = icosd;
        co(&c);
    }
    ctx_free(&c);
    return rc;
}

/* Scalar eos / eosd, for unit tests. */
double gbo_eos(const double *ec, double t, double s, double z, int32_t ieos) { return eos(ec, t, s, z, ieos); }
void gbo_eosd(const double *ec, double t1, double t2, double s1, double s2, double z, double rdz,
              int32_t ieos, double *dzrho, double *tec)
{
    eosd(ec, t1, t2, s1, s2, z, rdz, ieos, dzrho, tec);
}

/* Per-tracer inventory over wet interior cells of ts*ds(j)*dz(k), Neumaier
 * compensated, in the k, j, i order of the reference's diagnostic loop
 * (goldstein.f90:466-471). */
int gbo_inventory(const gb_go_dims *dims, const gb_go_grid *g, const double *ts, double *out)
{
    if (!dims || !g || !ts || !out) return GB_GO_EINVAL;
    ctx cc, *c = &cc;
    memset(c, 0, sizeof(*c));
    c->maxi = dims->maxi; c->maxj = dims->maxj; c->maxk = dims->maxk; c->maxl = dims->maxl;
    c->NI = (size_t)dims->maxi + 2; c->NJ = (size_t)dims->maxj + 2; c->g = g; c->ts = (double *)ts;
    for (int l = 1; l <= dims->maxl; ++l) {
        double s = 0.0, comp = 0.0;
        for (int k = 1; k <= dims->maxk; ++k)
            for (int j = 1; j <= dims->maxj; ++j)
                for (int i = 1; i <= dims->maxi; ++i) {
                    if (k < K1(i, j)) continue;
                    double x = TS(l, i, j, k) * g->ds[j - 1] * DZ(k);
                    double t = s + x;
                    if (fabs(s) >= fabs(x)) comp += (s - t) + x; else comp += (x - t) + s;
                    s = t;
                }
        out[l - 1] = s + comp;
    }
    return GB_GO_OK;
}

int gbo_abi_version(void) { return GB_GO_ABI_VERSION; }
