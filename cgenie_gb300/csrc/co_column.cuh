// Convective adjustment of one water column in IEEE double with explicit
// round-to-nearest intrinsics (no contraction whatever the compile flags), so
// the FP32-flux form applies the reference's exact co/coshuffle arithmetic to
// its FP64 state.
//   co         src/goldstein/goldstein.f90:2657-2777
//   coshuffle  src/goldstein/goldstein.f90:2781-2841
//   eos        src/goldstein/goldstein.f90:3048-3061
//
// `Col` provides:  double T(int l, int lev) const;  void setT(int l, int lev, double v);
//                  double &R(int lev);   (rho of this column, levels 0..maxk)
#pragma once

#include "gb_internal.h"

namespace gbgo {

struct EosCoef {
    double ec[5];
    int ieos;
};

__device__ __forceinline__ double eos_rn(const EosCoef &c, double t, double s, double z)
{
    const double tt = __dmul_rn(t, t);
    double r = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(c.ec[0], t), __dmul_rn(c.ec[1], s)), __dmul_rn(c.ec[2], tt)),
                         __dmul_rn(c.ec[3], __dmul_rn(tt, t)));
    if (c.ieos != 0) r = __dadd_rn(r, __dmul_rn(__dmul_rn(c.ec[4], t), z));
    return r;
}

// coshuffle for one wet column; returns icosd of the column
template <class Col>
__device__ int coshuffle_rn(Col &col, const EosCoef &ec, int maxk, int L, int k1, const double *dz, const double *rdz,
                            const double *zw)
{
    int icos = 0;
    int k0 = 0, ipass = 0;
    while (k0 < maxk && ipass < maxk) {
        ipass = ipass + 1;
        int k = maxk - 1;
        if (ec.ieos != 0) {
            col.R(maxk) = eos_rn(ec, col.T(0, maxk), col.T(1, maxk), zw[k]);
            col.R(k) = eos_rn(ec, col.T(0, k), col.T(1, k), zw[k]);
        }
        while ((col.R(maxk) > col.R(k)) && (k >= k1)) {
            k = k - 1;
            if (ec.ieos != 0) {
                col.R(maxk) = eos_rn(ec, col.T(0, maxk), col.T(1, maxk), zw[k]);
                col.R(k) = eos_rn(ec, col.T(0, k), col.T(1, k), zw[k]);
            }
        }
        k0 = k + 1;
        if (k0 < maxk) {
            const double dzt = dz[maxk];
            for (int l = 0; l < L; ++l) {
                const double tv_temp = col.T(l, maxk);
                for (int kk = maxk; kk >= k0 + 1; --kk) {
                    const double v = __dmul_rn(
                        __dadd_rn(__dmul_rn(__dadd_rn(dz[kk], -dzt), col.T(l, kk)), __dmul_rn(dzt, col.T(l, kk - 1))),
                        rdz[kk]);
                    col.setT(l, kk, v);
                }
                const double v0 = __dmul_rn(
                    __dadd_rn(__dmul_rn(__dadd_rn(dz[k0], -dzt), col.T(l, k0)), __dmul_rn(dzt, tv_temp)), rdz[k0]);
                col.setT(l, k0, v0);
            }
            for (int kk = k0; kk <= maxk; ++kk) col.R(kk) = eos_rn(ec, col.T(0, kk), col.T(1, kk), zw[maxk - 1]);
            if (maxk - k0 > icos) icos = maxk - k0;
        }
    }
    return icos;
}

// co main loop + fill for one wet column; returns the number of filled levels
template <class Col>
__device__ int co_rn(Col &col, const EosCoef &ec, int maxk, int L, int k1, const double *dz, const double *zw)
{
    int kk[kMaxK + 1];
    double dzm[kMaxK + 1];
    kk[k1 - 1] = 0;
    for (int m = k1; m <= maxk; ++m) {
        kk[m] = m;
        dzm[m] = dz[m];
    }
    auto refresh = [&](int x, int y) {
        if (ec.ieos != 0) {
            col.R(kk[x]) = eos_rn(ec, col.T(0, kk[x]), col.T(1, kk[x]), zw[kk[y]]);
            col.R(kk[y]) = eos_rn(ec, col.T(0, kk[y]), col.T(1, kk[y]), zw[kk[y]]);
        }
    };
    int m = maxk, lastmix = 0;
    while (kk[m - 1] > 0 || (lastmix != 0 && kk[m] != maxk)) {
        refresh(m, m - 1);
        if (col.R(kk[m]) < col.R(kk[m - 1]) || kk[m - 1] == 0) {
            if (lastmix == 0 || kk[m] == maxk) m = m - 1;
            else m = m + 1;
            lastmix = 0;
        } else {
            lastmix = 1;
            int n = m - 1;
            refresh(n, n - 1);
            while (kk[n - 1] > 0 && col.R(kk[n]) >= col.R(kk[n - 1])) {
                n = n - 1;
                refresh(n, n - 1);
            }
            const int km = kk[m];
            const double d0 = dzm[km];
            double dtot = d0;
            for (int ni = 1; ni <= m - n; ++ni) dtot = __dadd_rn(dtot, dzm[kk[m - ni]]);
            for (int l = 0; l < L; ++l) {
                double s = __dmul_rn(col.T(l, km), d0);
                for (int ni = 1; ni <= m - n; ++ni) s = __dadd_rn(s, __dmul_rn(col.T(l, kk[m - ni]), dzm[kk[m - ni]]));
                col.setT(l, km, __ddiv_rn(s, dtot));
            }
            dzm[km] = dtot;
            col.R(km) = eos_rn(ec, col.T(0, km), col.T(1, km), zw[kk[m - 1]]);
            int ni = m - 1;
            while (kk[ni + 1] > 0) {
                kk[ni] = kk[ni - m + n];
                ni = ni - 1;
            }
        }
    }
    int filled = 0;
    m = maxk - 1;
    for (int n = maxk - 1; n >= k1; --n) {
        if (n > kk[m]) {
            const int src = kk[m + 1];
            for (int l = 0; l < L; ++l) col.setT(l, n, col.T(l, src));
            col.R(n) = eos_rn(ec, col.T(0, n), col.T(1, n), zw[kk[n - 1]]);
            filled = filled + 1;
        } else {
            m = m - 1;
        }
    }
    return filled;
}

// Integer key that orders doubles as < does (no NaN; -0 and +0 both map to 0).
__device__ __forceinline__ long long order_key(double x)
{
    const long long b = __double_as_longlong(x);
    if ((b & 0x7fffffffffffffffLL) == 0) return 0;
    return b < 0 ? (b ^ 0x7fffffffffffffffLL) : b;
}

// Working arrays of co_warp (one per warp, shared memory).  Densities are kept as
// order_key values: every lane runs the same merge decisions, on the integer pipe.
struct CoWarpState {
    int kk[kMaxK + 2];
    double dzm[kMaxK + 1];
    long long rho[kMaxK + 1];
};

// co_rn with one warp per column: the tracers of the column are in shared memory,
// tv[lev * 32 + l] for the wet levels, and lane l mixes and fills tracer l.  The levels
// to merge (kk, dzm, rho in cs) are kept by lane 0 (densities of the first pass one lane
// per level); every value is the one co_rn computes.  Returns the number of filled levels
// (in every lane).
// rho0: the column's densities eos(T, S) of the wet levels (rho0[lev * rstride]) when
// given (ieos = 0), else computed here.
__device__ inline int co_warp(double *tv, CoWarpState *cs, const EosCoef &ec, int maxk, int L, int k1,
                              const double *dz, const double *zro, const double *zw, int lane, const double *rho0,
                              size_t rstride)
{
    int *kk = cs->kk;
    double *dzm = cs->dzm;
    long long *rho = cs->rho;
    auto T = [&](int l, int lev) { return tv[lev * 32 + l]; };
    for (int lev = k1 + lane; lev <= maxk; lev += 32) {
        rho[lev] = order_key(rho0 ? rho0[(size_t)lev * rstride] : eos_rn(ec, T(0, lev), T(1, lev), zro[lev]));
        kk[lev] = lev;
        dzm[lev] = dz[lev];
    }
    if (lane == 0) {
        rho[0] = 0;
        kk[k1 - 1] = 0;
    }
    __syncwarp();
    auto refresh = [&](int x, int y) {
        if (ec.ieos != 0) {
            if (lane == 0) {
                rho[kk[x]] = order_key(eos_rn(ec, T(0, kk[x]), T(1, kk[x]), zw[kk[y]]));
                rho[kk[y]] = order_key(eos_rn(ec, T(0, kk[y]), T(1, kk[y]), zw[kk[y]]));
            }
            __syncwarp();
        }
    };
    // m, n, lastmix follow from the shared arrays, so they are the same in every lane
    int m = maxk, lastmix = 0;
    while (kk[m - 1] > 0 || (lastmix != 0 && kk[m] != maxk)) {
        refresh(m, m - 1);
        if (rho[kk[m]] < rho[kk[m - 1]] || kk[m - 1] == 0) {
            if (lastmix == 0 || kk[m] == maxk) m = m - 1;
            else m = m + 1;
            lastmix = 0;
        } else {
            lastmix = 1;
            int n = m - 1;
            refresh(n, n - 1);
            while (kk[n - 1] > 0 && rho[kk[n]] >= rho[kk[n - 1]]) {
                n = n - 1;
                refresh(n, n - 1);
            }
            const int km = kk[m];
            const double d0 = dzm[km];
            double dtot = d0;
            if (lane == 0)
                for (int ni = 1; ni <= m - n; ++ni) dtot = __dadd_rn(dtot, dzm[kk[m - ni]]);
            dtot = __shfl_sync(0xffffffffu, dtot, 0);
            if (lane < L) {
                double s = __dmul_rn(T(lane, km), d0);
                for (int ni = 1; ni <= m - n; ++ni) s = __dadd_rn(s, __dmul_rn(T(lane, kk[m - ni]), dzm[kk[m - ni]]));
                tv[km * 32 + lane] = __ddiv_rn(s, dtot);
            }
            __syncwarp();
            if (lane == 0) {
                dzm[km] = dtot;
                rho[km] = order_key(eos_rn(ec, T(0, km), T(1, km), zw[kk[m - 1]]));
                int ni = m - 1;
                while (kk[ni + 1] > 0) {
                    kk[ni] = kk[ni - m + n];
                    ni = ni - 1;
                }
            }
            __syncwarp();
        }
    }
    // fill the merged levels (the densities of filled levels, which co also recomputes,
    // are not read again: the step recomputes every density from the state)
    int filled = 0;
    m = maxk - 1;
    for (int n = maxk - 1; n >= k1; --n) {
        if (n > kk[m]) {
            const int src = kk[m + 1];
            if (lane < L) tv[n * 32 + lane] = T(lane, src);
            filled = filled + 1;
        } else {
            m = m - 1;
        }
    }
    __syncwarp();
    return filled;
}

}  // namespace gbgo
