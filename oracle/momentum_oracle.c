/*
 * ORACLE -- test infrastructure only.  Nothing in the product links, loads or
 * calls this file; only the tests and bench.py's CPU legs do, and only as the
 * checker or the timed CPU reference.
 *
 * C restatement of the reference GOLDSTEIN momentum step and its initialisation:
 *   invert       src/goldstein/goldstein.f90:3138-3204
 *   jbar         src/goldstein/goldstein.f90:3217-3315
 *   matinv_gold  src/goldstein/goldstein.f90:3452-3467
 *   matmult      src/goldstein/goldstein.f90:3470-3492
 *   ubarsolv     src/goldstein/goldstein.f90:3500-3565
 *   velc         src/goldstein/goldstein.f90:3568-3679
 *   wind         src/goldstein/goldstein.f90:3685-3714
 *   island       src/goldstein/goldstein_lib.f90:186-241
 *   init order   src/goldstein/goldstein.f90:1788-1814 (invert, unit-source solves, island
 *                integrals, matinv_gold); step order :198-233
 * Arrays as in include/gb_momentum.h.  Expressions keep gfortran's left-to-right evaluation
 * in IEEE double; compile with -ffp-contract=off.  This is the reference's banded LU solve,
 * operation for operation: the device path's streamfunction differs from it by rounding.
 *
 * Parity pin: no Fortran compiler exists here and the reference ships no fixtures for these
 * routines ("parity unpinned"); the restatement is checked by the residual of the solved
 * streamfunction against the assembled matrix and by the island and boundary conditions
 * (tests/test_momentum_cpu.py).
 */
#include "../include/gb_momentum.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    gb_mo_dims d;
    gb_mo_params p;
    const gb_mo_grid *g;
    int n, m, nm;
    double *gap, *ratm, *gb, *gbold;
    double *bp, *sbp, *ub, *psi, *ubisl, *psisl, *erisl, *psibc;
    double *u, *u1;
} mo_state;

#define MAXI (S->d.maxi)
#define MAXJ (S->d.maxj)
#define MAXK (S->d.maxk)
#define K1(i, j) S->g->k1[(size_t)(i) + (size_t)(MAXI + 2) * (size_t)(j)]
#define RH(l, i, j) S->g->rh[((l) - 1) + 3 * ((size_t)(i) + (size_t)(MAXI + 2) * (size_t)(j))]
#define DRAG(l, i, j) S->g->drag[((l) - 1) + 2 * (((size_t)(i) - 1) + (size_t)(MAXI + 1) * ((size_t)(j) - 1))]
#define KU(l, i, j) S->g->ku[((l) - 1) + 2 * (((size_t)(i) - 1) + (size_t)MAXI * ((size_t)(j) - 1))]
#define MK(i, j) S->g->mk[((size_t)(i) - 1) + (size_t)(MAXI + 1) * ((size_t)(j) - 1)]
#define GETJ(i, j) S->g->getj[((size_t)(i) - 1) + (size_t)MAXI * ((size_t)(j) - 1)]
#define RTV(i, j) S->g->rtv[((size_t)(i) - 1) + (size_t)MAXI * ((size_t)(j) - 1)]
#define RTV3(i, j) S->g->rtv3[((size_t)(i) - 1) + (size_t)MAXI * ((size_t)(j) - 1)]
#define RCV(j) S->g->rcv[(j) - 1]
#define DSV(j) S->g->dsv[(j) - 1]
#define RDSV(j) S->g->rdsv[(j) - 1]
#define DS(j) S->g->ds[(j) - 1]
#define RDS(j) S->g->rds[(j) - 1]
#define RDS2(j) S->g->rds2[(j) - 2]
#define DZ(k) S->g->dz[(k) - 1]
#define DZA(k) S->g->dza[(k) - 1]
#define GAP(r, c) S->gap[((size_t)(r) - 1) + (size_t)S->nm * ((size_t)(c) - 1)]
#define RATM(r, c) S->ratm[((size_t)(r) - 1) + (size_t)S->nm * ((size_t)(c) - 1)]
#define BP(i, j, k) S->bp[((size_t)(i) - 1) + (size_t)(MAXI + 1) * (((size_t)(j) - 1) + (size_t)MAXJ * ((size_t)(k) - 1))]
#define SBP(i, j) S->sbp[((size_t)(i) - 1) + (size_t)(MAXI + 1) * ((size_t)(j) - 1)]
#define UB(a, l, i, j) (a)[((l) - 1) + 2 * ((size_t)(i) + (size_t)(MAXI + 2) * (size_t)(j))]
#define PSI(a, i, j) (a)[(size_t)(i) + (size_t)(MAXI + 1) * (size_t)(j)]
#define ERISL(r, c) S->erisl[((size_t)(r) - 1) + (size_t)S->d.isles * ((size_t)(c) - 1)]
#define U(a, l, i, j, k) (a)[((l) - 1) + 3 * ((size_t)(i) + (size_t)(MAXI + 1) * ((size_t)(j) + (size_t)(MAXJ + 1) * ((size_t)(k) - 1)))]
#define RHO(i, j, k) rho[(size_t)(i) + (size_t)(MAXI + 2) * ((size_t)(j) + (size_t)(MAXJ + 2) * (size_t)(k))]
#define TAU(a, l, i, j) (a)[((l) - 1) + 2 * (((size_t)(i) - 1) + (size_t)MAXI * ((size_t)(j) - 1))]
#define PATH(a, p, isl) S->g->a[((size_t)(p) - 1) + (size_t)S->d.mpi * ((size_t)(isl) - 1)]

static int imax2(int a, int b) { return a > b ? a : b; }
static int imax4(int a, int b, int c, int d) { return imax2(imax2(a, b), imax2(c, d)); }
static double dsign1(int l) { return l >= 0 ? 1.0 : -1.0; }   /* SIGN(1, l) as a REAL factor */

/* the band matrix of invert before the elimination (goldstein.f90:3149-3188) */
static void assemble(mo_state *S)
{
    const int n = S->n, nm = S->nm;
    const double dphi = S->p.dphi, rdphi = S->p.rdphi;
    const gb_mo_grid *g = S->g;
    memset(S->gap, 0, sizeof(double) * (size_t)nm * (2 * n + 3));
    for (int i = 1; i <= MAXI; ++i)
        for (int j = 0; j <= MAXJ; ++j) {
            const int k = i + j * n;
            if (imax4(K1(i, j), K1(i + 1, j), K1(i, j + 1), K1(i + 1, j + 1)) <= MAXK) {
                const double tv = (g->s[j + 1] * RH(1, i, j + 1) - g->s[j] * RH(1, i, j)) / (2.0 * DSV(j) * dphi);
                const double tv1 = (g->sv[j] * RH(2, i + 1, j) - g->sv[j] * RH(2, i, j)) / (2.0 * dphi * DSV(j));
                GAP(k, 2) = DRAG(1, i, j) * g->c[j] * g->c[j] * RH(1, i, j) / (DS(j) * DSV(j)) + tv1;
                int l = n + 1;
                if (i == 1) l = 2 * n + 1;
                GAP(k, l) = DRAG(2, i, j) * RCV(j) * RCV(j) * rdphi * rdphi * RH(2, i, j) - tv;
                GAP(k, n + 2) = -((DRAG(2, i, j) * RH(2, i, j) + DRAG(2, i + 1, j) * RH(2, i + 1, j)) /
                                  (g->cv[j] * g->cv[j] * dphi * dphi)) -
                                (DRAG(1, i, j) * g->c[j] * g->c[j] * RH(1, i, j) / DS(j) +
                                 DRAG(1, i, j + 1) * g->c[j + 1] * g->c[j + 1] * RH(1, i, j + 1) / DS(j + 1)) / DSV(j);
                l = n + 3;
                if (i == MAXI) l = 3;
                GAP(k, l) = DRAG(2, i + 1, j) * RH(2, i + 1, j) / (g->cv[j] * g->cv[j] * dphi * dphi) + tv;
                GAP(k, 2 * n + 2) = DRAG(1, i, j + 1) * g->c[j + 1] * g->c[j + 1] * RH(1, i, j + 1) / (DS(j + 1) * DSV(j)) - tv1;
            } else {
                GAP(k, n + 2) = 1;
            }
        }
}

static void invert(mo_state *S)
{
    const int n = S->n, nm = S->nm;
    assemble(S);
    for (int i = 1; i <= nm - 1; ++i) {
        const int im = i + n + 1 < nm ? i + n + 1 : nm;
        for (int j = i + 1; j <= im; ++j) {
            const double rat = GAP(j, n + 2 - j + i) / GAP(i, n + 2);
            RATM(j, j - i) = rat;
            if (rat != 0)
                for (int k = n + 2 - j + i; k <= 2 * n + 3 - j + i; ++k) GAP(j, k) = GAP(j, k) - rat * GAP(i, k + j - i);
        }
    }
}

static void ubarsolv(mo_state *S, double *ubloc, double *psiloc)
{
    const int n = S->n, nm = S->nm;
    const gb_mo_grid *g = S->g;
    double *gb = S->gb;
    for (int i = 1; i <= nm - 1; ++i) {
        const int im = i + n + 1 < nm ? i + n + 1 : nm;
        for (int j = i + 1; j <= im; ++j) gb[j - 1] = gb[j - 1] - RATM(j, j - i) * gb[i - 1];
    }
    gb[nm - 1] = gb[nm - 1] / GAP(nm, n + 2);
    for (int i = nm - 1; i >= 1; --i) {
        const int km = n + 1 < nm - i ? n + 1 : nm - i;
        for (int k = 1; k <= km; ++k) gb[i - 1] = gb[i - 1] - GAP(i, n + 2 + k) * gb[i + k - 1];
        gb[i - 1] = gb[i - 1] / GAP(i, n + 2);
    }
    for (int j = 0; j <= MAXJ; ++j) {
        for (int i = 1; i <= MAXI; ++i) PSI(psiloc, i, j) = gb[i + j * n - 1];
        PSI(psiloc, 0, j) = PSI(psiloc, MAXI, j);
    }
    for (int j = 1; j <= MAXJ; ++j)
        for (int i = 1; i <= MAXI; ++i)
            UB(ubloc, 1, i, j) = -RH(1, i, j) * g->c[j] * (PSI(psiloc, i, j) - PSI(psiloc, i, j - 1)) * RDS(j);
    for (int j = 1; j <= MAXJ - 1; ++j)
        for (int i = 1; i <= MAXI; ++i)
            UB(ubloc, 2, i, j) = RH(2, i, j) * (PSI(psiloc, i, j) - PSI(psiloc, i - 1, j)) * RCV(j) * S->p.rdphi;
    for (int i = 1; i <= MAXI; ++i) {
        UB(ubloc, 2, i, MAXJ) = 0.0;
        UB(ubloc, 2, i, 0) = 0.0;
    }
    for (int j = 1; j <= MAXJ; ++j) {
        UB(ubloc, 2, MAXI + 1, j) = UB(ubloc, 2, 1, j);
        UB(ubloc, 1, 0, j) = UB(ubloc, 1, MAXI, j);
        UB(ubloc, 1, MAXI + 1, j) = UB(ubloc, 1, 1, j);
        UB(ubloc, 2, 0, j) = UB(ubloc, 2, MAXI, j);
    }
    UB(ubloc, 2, MAXI + 1, 0) = UB(ubloc, 2, 1, 0);
    UB(ubloc, 2, 0, 0) = UB(ubloc, 2, MAXI, 0);
}

static double island(mo_state *S, const double *ubloc, int isl, int indj, const double *tau)
{
    const gb_mo_grid *g = S->g;
    double erisl1 = 0.0;
    for (int p = 1; p <= g->npi[isl - 1]; ++p) {
        const int lpi = PATH(lpisl, p, isl), ipi = PATH(ipisl, p, isl), jpi = PATH(jpisl, p, isl);
        const int al = abs(lpi);
        double cor;
        if (al == 1)
            cor = -g->s[jpi] * 0.25 * (UB(ubloc, 2, ipi, jpi) + UB(ubloc, 2, ipi + 1, jpi) + UB(ubloc, 2, ipi, jpi - 1) +
                                       UB(ubloc, 2, ipi + 1, jpi - 1));
        else
            cor = g->sv[jpi] * 0.25 * (UB(ubloc, 1, ipi - 1, jpi) + UB(ubloc, 1, ipi, jpi) + UB(ubloc, 1, ipi - 1, jpi + 1) +
                                       UB(ubloc, 1, ipi, jpi + 1));
        const double tauterm = indj ? (double)indj * TAU(tau, al, ipi, jpi) * RH(al, ipi, jpi) : 0.0 * RH(al, ipi, jpi);
        erisl1 = erisl1 + dsign1(lpi) * (DRAG(al, ipi, jpi) * UB(ubloc, al, ipi, jpi) + cor - tauterm) *
                              (g->c[jpi] * S->p.dphi * (2.0 - al) + RCV(jpi) * DSV(jpi) * (al - 1.0));
        if (indj == 1) {
            if (al == 1) {
                double tv1 = 0.0;
                for (int k = KU(1, ipi, jpi); k <= MK(ipi + 1, jpi); ++k) tv1 = tv1 + BP(ipi + 1, jpi, k) * DZ(k);
                for (int k = KU(1, ipi, jpi); k <= MK(ipi, jpi); ++k) tv1 = tv1 - BP(ipi, jpi, k) * DZ(k);
                erisl1 = erisl1 + (SBP(ipi + 1, jpi) - SBP(ipi, jpi) + tv1) * dsign1(lpi) * RH(1, ipi, jpi);
            } else {
                double tv2 = 0.0;
                for (int k = KU(2, ipi, jpi); k <= MK(ipi, jpi + 1); ++k) tv2 = tv2 + BP(ipi, jpi + 1, k) * DZ(k);
                for (int k = KU(2, ipi, jpi); k <= MK(ipi, jpi); ++k) tv2 = tv2 - BP(ipi, jpi, k) * DZ(k);
                erisl1 = erisl1 + (SBP(ipi, jpi + 1) - SBP(ipi, jpi) + tv2) * dsign1(lpi) * RH(2, ipi, jpi);
            }
        }
    }
    return erisl1;
}

static void wind(mo_state *S, const double *tau)
{
    const int n = S->n;
    const gb_mo_grid *g = S->g;
    for (int i = 1; i <= MAXI; ++i)
        for (int j = 0; j <= MAXJ; ++j) {
            const int ip1 = i % MAXI + 1, k = i + j * n;
            if (imax4(K1(i, j), K1(i + 1, j), K1(i, j + 1), K1(i + 1, j + 1)) <= MAXK) {
                S->gb[k - 1] = (TAU(tau, 2, ip1, j) * RH(2, i + 1, j) - TAU(tau, 2, i, j) * RH(2, i, j)) * S->p.rdphi * RCV(j) -
                               (TAU(tau, 1, i, j + 1) * g->c[j + 1] * RH(1, i, j + 1) - TAU(tau, 1, i, j) * g->c[j] * RH(1, i, j)) *
                                   RDSV(j);
            } else {
                S->gb[k - 1] = 0;
            }
            S->gbold[k - 1] = S->gb[k - 1];
        }
}

static void jbar(mo_state *S, const double *rho)
{
    const int n = S->n;
    for (int j = 1; j <= MAXJ; ++j)
        for (int i = 1; i <= MAXI; ++i)
            if (K1(i, j) <= MAXK)
                for (int k = K1(i, j) + 1; k <= MAXK; ++k)
                    BP(i, j, k) = BP(i, j, k - 1) - (RHO(i, j, k) + RHO(i, j, k - 1)) * DZA(k - 1) * 0.5;
    for (int j = 1; j <= MAXJ; ++j)
        for (int i = 1; i <= MAXI; ++i)
            if (MK(i, j) > 0) {
                SBP(i, j) = 0;
                for (int k = MK(i, j) + 1; k <= MAXK; ++k) SBP(i, j) = SBP(i, j) + BP(i, j, k) * DZ(k);
            }
    for (int j = 1; j <= MAXJ; ++j) {
        if (K1(1, j) < MAXK)
            for (int k = K1(1, j); k <= MAXK; ++k) BP(MAXI + 1, j, k) = BP(1, j, k);
        if (K1(1, j) <= MAXK) SBP(MAXI + 1, j) = SBP(1, j);
    }
    const double rdphi = S->p.rdphi;
    for (int j = 1; j <= MAXJ - 1; ++j)
        for (int i = 1; i <= MAXI; ++i) {
            const int ip1 = i % MAXI + 1, l = i + j * n;
            if (GETJ(i, j)) {
                double tv1 = 0, tv2 = 0, tv3 = 0, tv4 = 0;
                for (int k = KU(2, ip1, j); k <= MK(ip1, j + 1); ++k) tv1 = tv1 + BP(ip1, j + 1, k) * DZ(k);
                for (int k = KU(2, ip1, j); k <= MK(ip1, j); ++k) tv2 = tv2 + BP(ip1, j, k) * DZ(k);
                for (int k = KU(2, i, j); k <= MK(i, j + 1); ++k) tv3 = tv3 + BP(i, j + 1, k) * DZ(k);
                for (int k = KU(2, i, j); k <= MK(i, j); ++k) tv4 = tv4 + BP(i, j, k) * DZ(k);
                S->gb[l - 1] = S->gbold[l - 1] + ((tv3 + SBP(i, j + 1) - tv4 - SBP(i, j)) * RH(2, i, j) -
                                                  (tv1 + SBP(ip1, j + 1) - tv2 - SBP(ip1, j)) * RH(2, ip1, j)) *
                                                     rdphi * RDSV(j);
                tv1 = tv2 = tv3 = tv4 = 0;
                for (int k = KU(1, i, j + 1); k <= MK(ip1, j + 1); ++k) tv1 = tv1 + BP(ip1, j + 1, k) * DZ(k);
                for (int k = KU(1, i, j); k <= MK(ip1, j); ++k) tv2 = tv2 + BP(ip1, j, k) * DZ(k);
                for (int k = KU(1, i, j + 1); k <= MK(i, j + 1); ++k) tv3 = tv3 + BP(i, j + 1, k) * DZ(k);
                for (int k = KU(1, i, j); k <= MK(i, j); ++k) tv4 = tv4 + BP(i, j, k) * DZ(k);
                S->gb[l - 1] = S->gb[l - 1] + ((tv1 + SBP(ip1, j + 1) - tv3 - SBP(i, j + 1)) * RH(1, i, j + 1) -
                                               (tv2 + SBP(ip1, j) - tv4 - SBP(i, j)) * RH(1, i, j)) *
                                                  rdphi * RDSV(j);
            } else {
                S->gb[l - 1] = S->gbold[l - 1];
            }
        }
}

static void velc(mo_state *S, const double *rho, const double *dztau, const double *dztav)
{
    const gb_mo_grid *g = S->g;
    const double rdphi = S->p.rdphi, rel = S->p.rel;
    double *u = S->u, *u1 = S->u1;
    double *dzu = calloc(2 * (size_t)MAXK, sizeof(double));
#define DZU(l, k) dzu[((l) - 1) + 2 * ((size_t)(k) - 1)]
    for (int j = 1; j <= MAXJ; ++j)
        for (int i = 1; i <= MAXI; ++i) {
            double sum[2] = {0.0, 0.0};
            for (int k = K1(i, j); k <= MAXK; ++k) {
                double tv1, tv2, tv4, tv5;
                if (K1(i + 1, j) > k) {
                    tv1 = 0;
                    tv2 = 0;
                } else {
                    tv2 = -(RHO(i + 1, j, k) - RHO(i, j, k)) * rdphi * g->rc[j];
                    if (imax4(K1(i, j - 1), K1(i, j + 1), K1(i + 1, j - 1), K1(i + 1, j + 1)) <= k)
                        tv1 = -g->c[j] * (RHO(i + 1, j + 1, k) - RHO(i + 1, j - 1, k) + RHO(i, j + 1, k) - RHO(i, j - 1, k)) * RDS2(j) * 0.25;
                    else if (imax2(K1(i, j - 1), K1(i + 1, j - 1)) <= k)
                        tv1 = -g->c[j] * (RHO(i + 1, j, k) - RHO(i + 1, j - 1, k) + RHO(i, j, k) - RHO(i, j - 1, k)) * RDSV(j - 1) * 0.5;
                    else if (imax2(K1(i, j + 1), K1(i + 1, j + 1)) <= k)
                        tv1 = -g->c[j] * (RHO(i + 1, j + 1, k) - RHO(i + 1, j, k) + RHO(i, j + 1, k) - RHO(i, j, k)) * RDSV(j) * 0.5;
                    else
                        tv1 = 0;
                }
                if (K1(i, j + 1) > k) {
                    tv4 = 0;
                    tv5 = 0;
                } else {
                    tv4 = -g->cv[j] * (RHO(i, j + 1, k) - RHO(i, j, k)) * RDSV(j);
                    if (imax4(K1(i - 1, j), K1(i - 1, j + 1), K1(i + 1, j), K1(i + 1, j + 1)) <= k)
                        tv5 = -(RHO(i + 1, j + 1, k) - RHO(i - 1, j + 1, k) + RHO(i + 1, j, k) - RHO(i - 1, j, k)) * rdphi * 0.25 * RCV(j);
                    else if (imax2(K1(i - 1, j), K1(i - 1, j + 1)) <= k)
                        tv5 = -(RHO(i, j + 1, k) - RHO(i - 1, j + 1, k) + RHO(i, j, k) - RHO(i - 1, j, k)) * rdphi * 0.5 * RCV(j);
                    else if (imax2(K1(i + 1, j), K1(i + 1, j + 1)) <= k)
                        tv5 = -(RHO(i + 1, j + 1, k) - RHO(i, j + 1, k) + RHO(i + 1, j, k) - RHO(i, j, k)) * rdphi * 0.5 * RCV(j);
                    else
                        tv5 = 0;
                }
                if (k == MAXK) {
                    if (K1(i + 1, j) <= k) {
                        tv1 = tv1 - TAU(dztau, 2, i, j);
                        tv2 = tv2 - TAU(dztau, 1, i, j);
                    }
                    if (K1(i, j + 1) <= k) {
                        tv4 = tv4 - TAU(dztav, 2, i, j);
                        tv5 = tv5 - TAU(dztav, 1, i, j);
                    }
                }
                DZU(1, k) = -(g->s[j] * tv1 + DRAG(1, i, j) * tv2) * RTV(i, j);
                DZU(2, k) = -(DRAG(2, i, j) * tv4 - g->sv[j] * tv5) * RTV3(i, j);
                for (int l = 1; l <= 2; ++l) {
                    if (k == K1(i, j)) {
                        U(u, l, i, j, k) = 0;
                    } else {
                        U(u, l, i, j, k) = U(u, l, i, j, k - 1) + DZA(k - 1) * (DZU(l, k) + DZU(l, k - 1)) * 0.5;
                        sum[l - 1] = sum[l - 1] + DZ(k) * U(u, l, i, j, k);
                    }
                }
            }
            for (int k = K1(i, j); k <= MAXK; ++k) {
                if (K1(i + 1, j) <= k) {
                    U(u, 1, i, j, k) = U(u, 1, i, j, k) - sum[0] * RH(1, i, j) + UB(S->ub, 1, i, j);
                    U(u, 1, i, j, k) = rel * U(u1, 1, i, j, k) + (1.0 - rel) * U(u, 1, i, j, k);
                    U(u1, 1, i, j, k) = U(u, 1, i, j, k);
                }
                if (K1(i, j + 1) <= k) {
                    U(u, 2, i, j, k) = U(u, 2, i, j, k) - sum[1] * RH(2, i, j) + UB(S->ub, 2, i, j);
                    U(u, 2, i, j, k) = rel * U(u1, 2, i, j, k) + (1.0 - rel) * U(u, 2, i, j, k);
                    U(u1, 2, i, j, k) = U(u, 2, i, j, k);
                }
            }
        }
#undef DZU
    free(dzu);
    for (int j = 1; j <= MAXJ; ++j)
        for (int k = K1(1, j); k <= MAXK; ++k) U(u, 1, 0, j, k) = U(u, 1, MAXI, j, k);
    for (int j = 1; j <= MAXJ; ++j)
        for (int i = 1; i <= MAXI; ++i) {
            double tv = 0;
            for (int k = K1(i, j); k <= MAXK - 1; ++k) {
                const double tv1 = (U(u, 1, i, j, k) - U(u, 1, i - 1, j, k)) * rdphi * g->rc[j];
                const double tv2 = (U(u, 2, i, j, k) * g->cv[j] - U(u, 2, i, j - 1, k) * g->cv[j - 1]) * RDS(j);
                U(u, 3, i, j, k) = tv - DZ(k) * (tv1 + tv2);
                tv = U(u, 3, i, j, k);
            }
        }
}

static void matinv_gold(mo_state *S)
{
    const int nvar = S->d.isles;
    for (int i = 1; i <= nvar - 1; ++i)
        for (int j = i + 1; j <= nvar; ++j)
            for (int k = i + 1; k <= nvar; ++k) ERISL(j, k) = ERISL(i, i) * ERISL(j, k) - ERISL(j, i) * ERISL(i, k);
}

static void matmult(mo_state *S)
{
    const int nvar = S->d.isles, c = nvar + 1;
    for (int i = 1; i <= nvar - 1; ++i)
        for (int j = i + 1; j <= nvar; ++j) ERISL(j, c) = ERISL(i, i) * ERISL(j, c) - ERISL(j, i) * ERISL(i, c);
    ERISL(nvar, c) = ERISL(nvar, c) / ERISL(nvar, nvar);
    for (int i = nvar - 1; i >= 1; --i) {
        for (int j = i + 1; j <= nvar; ++j) ERISL(i, c) = ERISL(i, c) - ERISL(i, j) * ERISL(j, c);
        ERISL(i, c) = ERISL(i, c) / ERISL(i, i);
    }
}

void gbo_mo_free(void *state)
{
    mo_state *S = (mo_state *)state;
    if (!S) return;
    free(S->gap); free(S->ratm); free(S->gb); free(S->gbold); free(S->bp); free(S->sbp); free(S->ub);
    free(S->psi); free(S->ubisl); free(S->psisl); free(S->erisl); free(S->psibc); free(S->u); free(S->u1);
    free(S);
}

/* The reference's initialisation (goldstein.f90:1788-1814 with u = u1 = ub = psi = bp = sbp = 0).
   The grid struct and its arrays must outlive the state. */
void *gbo_mo_init(const gb_mo_dims *d, const gb_mo_params *p, const gb_mo_grid *g)
{
    if (d->maxi < 1 || d->maxj < 2 || d->maxk < 1 || d->isles < 1) return NULL;
    mo_state *S = (mo_state *)calloc(1, sizeof(mo_state));
    if (!S) return NULL;
    S->d = *d;
    S->p = *p;
    S->g = g;
    S->n = d->maxi;
    S->m = d->maxj + 1;
    S->nm = S->n * S->m;
    const size_t nm = (size_t)S->nm, nu = 3 * (size_t)(d->maxi + 1) * (d->maxj + 1) * d->maxk;
    const size_t nub = 2 * (size_t)(d->maxi + 2) * (d->maxj + 1), npsi = (size_t)(d->maxi + 1) * (d->maxj + 1);
    S->gap = calloc(nm * (2 * (size_t)S->n + 3), sizeof(double));
    S->ratm = calloc(nm * ((size_t)S->n + 1), sizeof(double));
    S->gb = calloc(nm, sizeof(double));
    S->gbold = calloc(nm, sizeof(double));
    S->bp = calloc((size_t)(d->maxi + 1) * d->maxj * d->maxk, sizeof(double));
    S->sbp = calloc((size_t)(d->maxi + 1) * d->maxj, sizeof(double));
    S->ub = calloc(nub, sizeof(double));
    S->psi = calloc(npsi, sizeof(double));
    S->ubisl = calloc(nub * d->isles, sizeof(double));
    S->psisl = calloc(npsi * d->isles, sizeof(double));
    S->erisl = calloc((size_t)d->isles * (d->isles + 1), sizeof(double));
    S->psibc = calloc((size_t)d->isles, sizeof(double));
    S->u = calloc(nu, sizeof(double));
    S->u1 = calloc(nu, sizeof(double));
    if (!S->gap || !S->ratm || !S->gb || !S->gbold || !S->bp || !S->sbp || !S->ub || !S->psi || !S->ubisl ||
        !S->psisl || !S->erisl || !S->psibc || !S->u || !S->u1) {
        gbo_mo_free(S);
        return NULL;
    }
    memcpy(S->gbold, g->psiles, nm * sizeof(double));
    invert(S);
    for (int isol = 1; isol <= d->isles; ++isol) {
        for (int j = 0; j <= d->maxj; ++j)
            for (int i = 1; i <= d->maxi; ++i) {
                const int k = i + j * d->maxi;
                S->gb[k - 1] = ((int)S->gbold[k - 1] == isol + 1) ? 1.0 : 0.0;
            }
        ubarsolv(S, S->ubisl + nub * (isol - 1), S->psisl + npsi * (isol - 1));
        for (int isl = 1; isl <= d->isles; ++isl) ERISL(isl, isol) = island(S, S->ubisl + nub * (isol - 1), isl, 0, NULL);
    }
    matinv_gold(S);
    return S;
}

/* One momentum step (goldstein.f90:198-233) on rho (0:maxi+1, 0:maxj+1, 0:maxk). */
int gbo_mo_step(void *state, const double *tau, const double *dztau, const double *dztav, const double *rho)
{
    mo_state *S = (mo_state *)state;
    const int isles = S->d.isles;
    const size_t nub = 2 * (size_t)(MAXI + 2) * (MAXJ + 1), npsi = (size_t)(MAXI + 1) * (MAXJ + 1);
    wind(S, tau);
    jbar(S, rho);
    ubarsolv(S, S->ub, S->psi);
    for (int isl = 1; isl <= isles; ++isl) ERISL(isl, isles + 1) = island(S, S->ub, isl, 1, tau);
    if (isles > 1) {
        matmult(S);
        for (int isl = 1; isl <= isles; ++isl) S->psibc[isl - 1] = -ERISL(isl, isles + 1);
    } else {
        S->psibc[0] = -ERISL(1, 2) / ERISL(1, 1);
    }
    for (int j = 1; j <= MAXJ; ++j)
        for (int i = 0; i <= MAXI + 1; ++i)
            for (int l = 1; l <= 2; ++l) {
                double s = 0.0;
                for (int isl = 1; isl <= isles; ++isl) s = s + UB(S->ubisl + nub * (isl - 1), l, i, j) * S->psibc[isl - 1];
                UB(S->ub, l, i, j) = UB(S->ub, l, i, j) + s;
            }
    for (int j = 0; j <= MAXJ; ++j)
        for (int i = 0; i <= MAXI; ++i) {
            double s = 0.0;
            for (int isl = 1; isl <= isles; ++isl) s = s + PSI(S->psisl + npsi * (isl - 1), i, j) * S->psibc[isl - 1];
            PSI(S->psi, i, j) = PSI(S->psi, i, j) + s;
        }
    velc(S, rho, dztau, dztav);
    return 0;
}

/* copies of the state (any pointer may be NULL) */
void gbo_mo_get(void *state, double *u, double *u1, double *ub, double *psi, double *gap, double *gbrhs)
{
    mo_state *S = (mo_state *)state;
    const size_t nu = 3 * (size_t)(MAXI + 1) * (MAXJ + 1) * MAXK;
    if (u) memcpy(u, S->u, nu * sizeof(double));
    if (u1) memcpy(u1, S->u1, nu * sizeof(double));
    if (ub) memcpy(ub, S->ub, 2 * (size_t)(MAXI + 2) * (MAXJ + 1) * sizeof(double));
    if (psi) memcpy(psi, S->psi, (size_t)(MAXI + 1) * (MAXJ + 1) * sizeof(double));
    if (gap) memcpy(gap, S->gap, (size_t)S->nm * (2 * (size_t)S->n + 3) * sizeof(double));
    if (gbrhs) memcpy(gbrhs, S->gbold, (size_t)S->nm * sizeof(double));
}

void gbo_mo_set_velocity(void *state, const double *u, const double *u1)
{
    mo_state *S = (mo_state *)state;
    const size_t nu = 3 * (size_t)(MAXI + 1) * (MAXJ + 1) * MAXK;
    memcpy(S->u, u, nu * sizeof(double));
    memcpy(S->u1, u1, nu * sizeof(double));
}

/* the dense matrix (nm x nm, row-major) of the streamfunction equations: band column c of
   row k is matrix column k + c - (n+2) */
void gbo_mo_matrix(void *state, double *A)
{
    mo_state *S = (mo_state *)state;
    const int n = S->n, nm = S->nm;
    double *save = malloc((size_t)nm * (2 * n + 3) * sizeof(double));
    memcpy(save, S->gap, (size_t)nm * (2 * n + 3) * sizeof(double));
    assemble(S);
    memset(A, 0, (size_t)nm * nm * sizeof(double));
    for (int k = 1; k <= nm; ++k)
        for (int c = 1; c <= 2 * n + 3; ++c) {
            const int col = k + c - (n + 2);
            if (GAP(k, c) != 0.0 && col >= 1 && col <= nm) A[(size_t)(k - 1) * nm + (col - 1)] = GAP(k, c);
        }
    memcpy(S->gap, save, (size_t)nm * (2 * n + 3) * sizeof(double));
    free(save);
}

/* the unit-source solutions and the island matrix after matinv_gold */
void gbo_mo_get_islands(void *state, double *psisl, double *ubisl, double *erisl)
{
    mo_state *S = (mo_state *)state;
    const size_t nub = 2 * (size_t)(MAXI + 2) * (MAXJ + 1), npsi = (size_t)(MAXI + 1) * (MAXJ + 1);
    if (psisl) memcpy(psisl, S->psisl, npsi * S->d.isles * sizeof(double));
    if (ubisl) memcpy(ubisl, S->ubisl, nub * S->d.isles * sizeof(double));
    if (erisl) memcpy(erisl, S->erisl, (size_t)S->d.isles * (S->d.isles + 1) * sizeof(double));
}
