/* ORACLE -- test infrastructure only.
 *
 * C restatement of the GOLDSTEIN time-series diagnostics, in the reference's loop and
 * operation order:
 *   diag2     src/goldstein/goldstein_diag.f90:10-71
 *   diagopsi  src/goldstein/goldstein_diag.f90:350-411
 * Arrays in the layouts of include/gb_goldstein.h (ts(l,i,j,k), rho(i,j,k), u(c,i,j,k),
 * k1(i,j)); basin rows as include/gb_timeseries.h.  Compiled with -ffp-contract=off.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "../include/gb_timeseries.h"

#define TS(l, i, j, k) ts[(size_t)((l) - 1) + (size_t)L * ((size_t)(i) + (size_t)NI * ((size_t)(j) + (size_t)NJ * (size_t)(k)))]
#define RHO(i, j, k) rho[(size_t)(i) + (size_t)NI * ((size_t)(j) + (size_t)NJ * (size_t)(k))]
#define U(c, i, j, k) u[(size_t)((c) - 1) + 3 * ((size_t)(i) + (size_t)(maxi + 1) * ((size_t)(j) + (size_t)(maxj + 1) * (size_t)((k) - 1)))]
#define K1(i, j) g->k1[(size_t)(i) + (size_t)NI * (size_t)(j)]

/* diag2(sum, avn, avs) on the first call (vol computed in the same loop). */
int gbo_diag2(const gb_go_dims *d, const gb_go_grid *g, const gb_ts_basins *b, const double *ts, const double *rho,
              const double *u, double *sum, double *avn_out, double *avs_out)
{
    const int maxi = d->maxi, maxj = d->maxj, maxk = d->maxk, L = d->maxl, NI = maxi + 2, NJ = maxj + 2;
    double vol[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double avn = 0.0, avs = 0.0;
    long long ntot = 0, intot = 0;
    for (int n = 0; n < 8 * L; ++n) sum[n] = 0.0;
    for (int j = 1; j <= maxj; ++j)
        for (int i = 1; i <= maxi; ++i)
            if (K1(i, j) <= maxk) {
                ntot += maxk - K1(i, j) + 1;
                intot += maxk - K1(i, j);
            }
    for (int k = 1; k <= maxk; ++k)
        for (int j = 1; j <= maxj; ++j)
            for (int i = 1; i <= maxi; ++i) {
                if (k < K1(i, j)) continue;
                const int ndep = (2 * k - 1) / maxk;
                const int ips = b->ips[j - 1], ipf = b->ipf[j - 1], ias = b->ias[j - 1], iaf = b->iaf[j - 1];
                int mo;
                if (j <= b->jsf) mo = 4;
                else if (i >= ips && i <= ipf) mo = 1;
                else if ((i >= ias && i <= iaf) || (iaf <= ias && (i <= iaf || ias <= i))) mo = 2;
                else mo = 3;
                for (int l = 1; l <= L; ++l)
                    sum[mo + 4 * ndep + 8 * (l - 1) - 1] =
                        sum[mo + 4 * ndep + 8 * (l - 1) - 1] + TS(l, i, j, k) * g->dphi * g->ds[j - 1] * g->dz[k - 1];
                vol[mo + 4 * ndep] = vol[mo + 4 * ndep] + g->dphi * g->ds[j - 1] * g->dz[k - 1];
                if (k < maxk) avn = avn + fabs(RHO(i, j, k) - RHO(i, j, k + 1)) / g->dza[k - 1];
                avs = avs + U(1, i, j, k) * U(1, i, j, k) + U(2, i, j, k) * U(2, i, j, k);
            }
    for (int i = 1; i <= 8; ++i)
        for (int l = 1; l <= L; ++l)
            if (vol[i] != 0.0) sum[i + 8 * (l - 1) - 1] = sum[i + 8 * (l - 1) - 1] / vol[i];
    *avs_out = sqrt(avs / (double)ntot);
    *avn_out = avn / (double)intot;
    return 0;
}

/* diagopsi(ominp, omaxp, omina, omaxa, opsi, opsia, opsip, iposa); opsi arrays (0:maxj, 0:maxk). */
int gbo_diagopsi(const gb_go_dims *d, const gb_go_grid *g, const gb_ts_basins *b, const double *u, double *opsi,
                 double *opsip, double *opsia, double *ext, int32_t *iposa)
{
    const int maxi = d->maxi, maxj = d->maxj, maxk = d->maxk, nj = maxj + 1;
#define OP(a, j, k) a[(size_t)(j) + (size_t)nj * (size_t)(k)]
    const size_t plane = (size_t)nj * (maxk + 1);
    memset(opsi, 0, plane * sizeof(double));
    memset(opsip, 0, plane * sizeof(double));
    memset(opsia, 0, plane * sizeof(double));
    for (int j = 1; j <= maxj - 1; ++j)
        for (int k = 1; k <= maxk - 1; ++k) {
            double ou = 0.0;
            for (int i = 1; i <= maxi; ++i) ou = ou + g->cv[j] * U(2, i, j, k) * g->dphi;
            OP(opsi, j, k) = OP(opsi, j, k - 1) - g->dz[k - 1] * ou;
        }
    double ominp = 0.0, omaxp = 0.0;
    for (int j = b->jsf + 1; j <= maxj - 1; ++j)
        for (int k = 1; k <= maxk - 1; ++k) {
            double ou = 0.0;
            for (int i = b->ips[j - 1]; i <= b->ipf[j - 1]; ++i) ou = ou + g->cv[j] * U(2, i, j, k) * g->dphi;
            OP(opsip, j, k) = OP(opsip, j, k - 1) - g->dz[k - 1] * ou;
            if (OP(opsip, j, k) < ominp && k <= b->overdep) ominp = OP(opsip, j, k);
            if (OP(opsip, j, k) > omaxp && k <= b->overdep) omaxp = OP(opsip, j, k);
        }
    double omina = 0.0, omaxa = 0.0;
    iposa[0] = iposa[1] = 0;
    for (int j = b->jsf + 1; j <= maxj - 1; ++j)
        for (int k = 1; k <= maxk - 1; ++k) {
            double ou = 0.0;
            const int ias = b->ias[j - 1], iaf = b->iaf[j - 1];
            if (ias > iaf) {
                for (int i = ias; i <= maxi; ++i) ou = ou + g->cv[j] * U(2, i, j, k) * g->dphi;
                for (int i = 1; i <= iaf; ++i) ou = ou + g->cv[j] * U(2, i, j, k) * g->dphi;
            } else {
                for (int i = ias; i <= iaf; ++i) ou = ou + g->cv[j] * U(2, i, j, k) * g->dphi;
            }
            OP(opsia, j, k) = OP(opsia, j, k - 1) - g->dz[k - 1] * ou;
            if (OP(opsia, j, k) < omina && k <= b->overdep) omina = OP(opsia, j, k);
            if (OP(opsia, j, k) > omaxa && k <= b->overdep) {
                omaxa = OP(opsia, j, k);
                iposa[0] = j;
                iposa[1] = k;
            }
        }
    ext[0] = ominp;
    ext[1] = omaxp;
    ext[2] = omina;
    ext[3] = omaxa;
#undef OP
    return 0;
}
