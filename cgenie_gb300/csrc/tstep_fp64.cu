// Plain (FP64) GOLDSTEIN tracer timestep for sm_103a: one launch per step.
//
// Restates src/goldstein/goldstein.f90:2280-2432 (tstepo, imld=0 and 1), :2436-2642
// (tstepo_flux incl. the diso branch), :2657-2777 (co), :2781-2841 (coshuffle)
// and :3048-3082 (eos/eosd).  Every expression keeps the reference's operation
// order and this translation unit is compiled with -fmad=false, so each double
// result is the one the reference's non-FMA IEEE arithmetic produces.
//
// Mapping: a CTA owns a tile of TX x TY water columns over all maxk levels, one
// thread per cell (i, j, k).  Each thread computes the three faces it owns
// (east, north, top) once per tracer and publishes them in shared memory; the
// tile's west/south edge threads also compute the faces they share with the
// neighbouring tile.  Because the tile spans the whole column, the convective
// adjustment `co` of every column and the periodic halo columns are finished in
// the same launch, after a barrier, by one thread per column.
#include "gb_internal.h"
#include "../../include/gb_goldstein.h"

#include <cuda_runtime.h>

namespace gbgo {

__device__ __forceinline__ double eos_d(const PhysParams &p, double t, double s, double z)
{
    // goldstein.f90:3048-3061; t**2 -> t*t, t**3 -> (t*t)*t
    double rho = p.ec[0] * t + p.ec[1] * s + p.ec[2] * (t * t) + p.ec[3] * ((t * t) * t);
    if (p.ieos != 0) rho = rho + p.ec[4] * t * z;
    return rho;
}

__device__ __forceinline__ void eosd_d(const PhysParams &p, double t1, double t2, double s1, double s2,
                                       double z, double rdz, double &dzrho, double &tec)
{
    // goldstein.f90:3064-3082
    double tatw = 0.5 * (t1 + t2);
    tec = -p.ec[0] - p.ec[2] * tatw * 2 - p.ec[3] * tatw * tatw * 3;
    if (p.ieos != 0) tec = tec - p.ec[4] * z;
    dzrho = (p.ec[1] * (s2 - s1) - tec * (t2 - t1)) * rdz;
}

__device__ __forceinline__ double upstream(double pec) { return pec / (2.0 + fabs(pec)); }

// Advective-diffusive face flux with upstream weighting, east/north form:
// a * ((1-ups)*tp + (1+ups)*tc) * 0.5 - (tp - tc) * b * c
__device__ __forceinline__ double face_flux(double a, double ups, double tp, double tc, double b, double c)
{
    double f = a * ((1.0 - ups) * tp + (1.0 + ups) * tc) * 0.5;
    return f - (tp - tc) * b * c;
}

struct ColumnView {
    double *tsw;               // write buffer
    const double *tss;         // ts_static (for levels below k1)
    const Dims *d;
    int i, j, k1;
    __device__ double get(int l, int lev) const
    {
        size_t o = ts_index(*d, l, i, j, lev);
        return lev >= k1 ? tsw[o] : tss[o];
    }
    __device__ void set(int l, int lev, double v) const { tsw[ts_index(*d, l, i, j, lev)] = v; }
};

// coshuffle, goldstein.f90:2781-2841 (one column)
__device__ void coshuffle_column(const StepArgs &a, const ColumnView &cv, int32_t &icos)
{
    const Dims &d = a.d;
    const PhysParams &p = a.p;
    const int maxk = d.maxk;
    const int k1 = cv.k1;
    double *rho = a.rho;
    auto R = [&](int lev) -> double & { return rho[rho_index(d, cv.i, cv.j, lev)]; };
    icos = 0;
    int k0 = 0, ipass = 0;
    while (k0 < maxk && ipass < maxk) {
        ipass = ipass + 1;
        int k = maxk - 1;
        if (p.ieos != 0) {
            R(maxk) = eos_d(p, cv.get(0, maxk), cv.get(1, maxk), a.m.zw[k]);
            R(k) = eos_d(p, cv.get(0, k), cv.get(1, k), a.m.zw[k]);
        }
        while ((R(maxk) > R(k)) && (k >= k1)) {
            k = k - 1;
            if (p.ieos != 0) {
                R(maxk) = eos_d(p, cv.get(0, maxk), cv.get(1, maxk), a.m.zw[k]);
                R(k) = eos_d(p, cv.get(0, k), cv.get(1, k), a.m.zw[k]);
            }
        }
        k0 = k + 1;
        if (k0 < maxk) {
            const double dzt = a.m.dz[maxk];
            for (int l = 0; l < d.L; ++l) {
                double tv_temp = cv.get(l, maxk);
                for (int kk = maxk; kk >= k0 + 1; --kk) {
                    cv.set(l, kk, ((a.m.dz[kk] - dzt) * cv.get(l, kk) + dzt * cv.get(l, kk - 1)) * a.m.rdz[kk]);
                }
                cv.set(l, k0, ((a.m.dz[k0] - dzt) * cv.get(l, k0) + dzt * tv_temp) * a.m.rdz[k0]);
            }
            for (int kk = k0; kk <= maxk; ++kk) R(kk) = eos_d(p, cv.get(0, kk), cv.get(1, kk), a.m.zw[maxk - 1]);
            if (maxk - k0 > icos) icos = maxk - k0;
        }
    }
}

// co main loop and fill, goldstein.f90:2674-2772 (one wet column).  Returns the
// number of filled levels.
__device__ int co_column(const StepArgs &a, const ColumnView &cv)
{
    const Dims &d = a.d;
    const PhysParams &p = a.p;
    const int maxk = d.maxk;
    const int k1 = cv.k1;
    const int ieos = p.ieos;
    double *rho = a.rho;
    auto R = [&](int lev) -> double & { return rho[rho_index(d, cv.i, cv.j, lev)]; };
    int kk[kMaxK + 1];
    double dzm[kMaxK + 1];
    kk[k1 - 1] = 0;
    for (int m = k1; m <= maxk; ++m) {
        kk[m] = m;
        dzm[m] = a.m.dz[m];
    }
    auto refresh = [&](int x, int y) {
        if (ieos != 0) {
            R(kk[x]) = eos_d(p, cv.get(0, kk[x]), cv.get(1, kk[x]), a.m.zw[kk[y]]);
            R(kk[y]) = eos_d(p, cv.get(0, kk[y]), cv.get(1, kk[y]), a.m.zw[kk[y]]);
        }
    };
    int m = maxk, lastmix = 0;
    while (kk[m - 1] > 0 || (lastmix != 0 && kk[m] != maxk)) {
        refresh(m, m - 1);
        if (R(kk[m]) < R(kk[m - 1]) || kk[m - 1] == 0) {
            if (lastmix == 0 || kk[m] == maxk) m = m - 1;
            else m = m + 1;
            lastmix = 0;
        } else {
            lastmix = 1;
            int n = m - 1;
            refresh(n, n - 1);
            while (kk[n - 1] > 0 && R(kk[n]) >= R(kk[n - 1])) {
                n = n - 1;
                refresh(n, n - 1);
            }
            // volume-weighted mean of levels k(n..m) into k(m); loop order
            // interchanged (tracer outer) with identical per-tracer arithmetic
            const int km = kk[m];
            const double d0 = dzm[km];
            double dtot = d0;
            for (int ni = 1; ni <= m - n; ++ni) dtot = dtot + dzm[kk[m - ni]];
            for (int l = 0; l < d.L; ++l) {
                double s = cv.get(l, km) * d0;
                for (int ni = 1; ni <= m - n; ++ni) s = s + cv.get(l, kk[m - ni]) * dzm[kk[m - ni]];
                cv.set(l, km, s / dtot);
            }
            dzm[km] = dtot;
            R(km) = eos_d(p, cv.get(0, km), cv.get(1, km), a.m.zw[kk[m - 1]]);
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
            for (int l = 0; l < d.L; ++l) cv.set(l, n, cv.get(l, src));
            R(n) = eos_d(p, cv.get(0, n), cv.get(1, n), a.m.zw[kk[n - 1]]);
            filled = filled + 1;
        } else {
            m = m - 1;
        }
    }
    return filled;
}

// ---- Kraus-Turner mixed layer (imld = 1) ----
// Level-pair depth grids of goldstein.f90:1013-1025: dzg(k,kk) = zw(k) - zw(kk-1),
// z2dzg(k,kk) = -zw(k)^2 + zw(kk-1)^2, rdzg(k,kk) = 1/dzg(k,kk) (1e10 where k = kk-1).
__device__ __forceinline__ double dzg_d(const Metrics &M, int k, int kk) { return M.zw[k] - M.zw[kk - 1]; }
__device__ __forceinline__ double z2dzg_d(const Metrics &M, int k, int kk)
{
    return -M.zw[k] * M.zw[k] + M.zw[kk - 1] * M.zw[kk - 1];
}
__device__ __forceinline__ double rdzg_d(const Metrics &M, int k, int kk)
{
    return k != kk - 1 ? 1.0 / dzg_d(M, k, kk) : 1.0E10;
}

// krausturner, goldstein.f90:3337-3442, on one column (every level it touches is wet)
__device__ void kraus_turner_column(const StepArgs &a, const ColumnView &cv, size_t c2, double pebuoy, double ketau)
{
    const Dims &d = a.d;
    const PhysParams &p = a.p;
    const Metrics &M = a.m;
    const int maxk = d.maxk, L = d.L, tvkl = cv.k1;
    double qmix[GB_GO_MAX_L + 1];
    const int mldpk = maxk;   // the routine's first statement (goldstein.f90:3350)
    int k = mldpk, partmix = 1;
    double empe = pebuoy;
    double emke = ketau * M.mlddec[k];
    double em = empe + emke;
    double eneed = 0.0;
    double tmix = cv.get(0, k), smix = cv.get(1, k);
    double rhou = 0.0, rhol = 0.0;
    for (int l = 0; l < L; ++l) qmix[l] = cv.get(l, k);
    double rhomix = eos_d(p, tmix, smix, M.zw[k]);
    while (eneed < em && em > 0) {
        if (k < mldpk) {
            qmix[0] = tmix;
            qmix[1] = smix;
            for (int l = 2; l < L; ++l) qmix[l] = rdzg_d(M, maxk, k) * (qmix[l] * dzg_d(M, maxk, k + 1) + cv.get(l, k) * M.dz[k]);
        }
        if (k == tvkl) {
            a.mldk[c2] = k;
            a.mld[c2] = M.zw[k - 1];
            partmix = 0;
            em = -1.0E-8;
            if (k < maxk)
                for (int l = 0; l < L; ++l)
                    for (int n = k; n <= maxk; ++n) cv.set(l, n, qmix[l]);
        } else {
            k = k - 1;
            const double emr = (em - eneed) / em;
            empe = empe * emr;
            emke = emke * emr * M.mlddecd[k];
            em = empe + emke;
            rhou = p.ieos != 0 ? eos_d(p, tmix, smix, M.zw[k]) : rhomix;
            tmix = rdzg_d(M, maxk, k) * (tmix * dzg_d(M, maxk, k + 1) + cv.get(0, k) * M.dz[k]);
            smix = rdzg_d(M, maxk, k) * (smix * dzg_d(M, maxk, k + 1) + cv.get(1, k) * M.dz[k]);
            rhol = eos_d(p, cv.get(0, k), cv.get(1, k), M.zw[k]);
            rhomix = eos_d(p, tmix, smix, M.zw[k]);
            eneed = z2dzg_d(M, maxk, k + 1) * rhou + z2dzg_d(M, k, k) * rhol - z2dzg_d(M, maxk, k) * rhomix;
        }
    }
    if (partmix == 1 && em > 0) {
        a.mldk[c2] = k;
        const double mlda = dzg_d(M, maxk, k + 1) * rdzg_d(M, maxk, k) * em / eneed;
        const double mldb = (dzg_d(M, maxk, k) * rdzg_d(M, maxk, k + 1) - 1) * mlda;
        for (int l = 0; l < L; ++l) {
            const double below = cv.get(l, k);
            const double surf = (1 - mldb) * qmix[l] + mldb * below;
            cv.set(l, maxk, surf);
            for (int n = k + 1; n <= maxk - 1; ++n) cv.set(l, n, surf);
            cv.set(l, k, mlda * qmix[l] + (1 - mlda) * below);
        }
        a.mld[c2] = k < maxk ? M.zw[k] + em / (M.zw[k] * (rhol - rhou)) : 0.0;
    } else if (partmix == 1 && k < maxk) {
        a.mldk[c2] = k + 1;
        a.mld[c2] = M.zw[k];
    }
}

// The mixed-layer part of tstepo after co, goldstein.f90:2336-2389, on one wet column:
// potential energy released by co (rold: densities before co), wind energy, then
// krausturner or the shallow-layer diagnostic.
__device__ void mixed_layer_column(const StepArgs &a, const ColumnView &cv, size_t c2, const double *rold)
{
    const PhysParams &p = a.p;
    const Metrics &M = a.m;
    const int maxk = a.d.maxk;
    double peconv = 0.0;
    for (int k = maxk; k > 0; --k) {
        const double rnew = eos_d(p, cv.get(0, k), cv.get(1, k), M.zro[k]);
        peconv = peconv + (rnew - rold[k]) * z2dzg_d(M, k, k);
    }
    double pebuoy = peconv + a.mldpe1[c2];
    if (pebuoy > 0.0) pebuoy = pebuoy * p.mldpebuoycoeff;
    const double ketau = a.mldketau[c2];
    const double emix = pebuoy + ketau * M.mlddec[maxk];
    if (emix > 0.0) {
        kraus_turner_column(a, cv, c2, pebuoy, ketau);
    } else {
        a.mldk[c2] = maxk;
        const double pe1 = a.mldpe1[c2];
        a.mld[c2] = pe1 < 0 ? M.zw[maxk - 1] * (1 - emix / pe1) : M.zw[maxk - 1];
    }
}

__global__ void __launch_bounds__(256) k_step_fp64(const StepArgs a)
{
    extern __shared__ double smem[];
    const Dims &d = a.d;
    const PhysParams &p = a.p;
    const Metrics &M = a.m;
    const int TX = a.tile_i, TY = a.tile_j, K = d.maxk;
    const int t = threadIdx.x;
    const int ti = t % TX;
    const int tj = (t / TX) % TY;
    const int kz = t / (TX * TY);
    const int k = kz + 1;
    const int bi = blockIdx.x % a.tiles_i, bj = blockIdx.x / a.tiles_i;
    const int i = bi * TX + ti + 1, j = bj * TY + tj + 1;
    // the block is padded to whole warps; threads past the last level idle
    const bool inside = (i <= d.maxi) && (j <= d.maxj) && (kz < K);
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk;

    double *FE = smem;                         // [K][TY][TX+1]  west face of slot x at x
    double *FN = FE + K * TY * (TX + 1);       // [K][TY+1][TX]  south face of slot y at y
    double *FA = FN + K * (TY + 1) * TX;       // [K+1][TY][TX]  bottom face of level kz at kz
    auto fe_at = [&](int x, int y, int z) -> double & { return FE[(z * TY + y) * (TX + 1) + x]; };
    auto fn_at = [&](int x, int y, int z) -> double & { return FN[(z * (TY + 1) + y) * TX + x]; };
    auto fa_at = [&](int x, int y, int z) -> double & { return FA[(z * TY + y) * TX + x]; };

    if (blockIdx.x == 0 && t == 0) {
        a.diag_next[0] = 0ull;
        a.diag_next[1] = 0ull;
    }

    // ---- per-cell coefficients (goldstein.f90:2488-2523) ----
    int k1c = 0, k1e = 0, k1n = 0, ie = 0;
    bool wet = false, vwet = false;
    double dzrho = 0.0, tec = 0.0, rdzrho = 0.0, diffv = p.diff2;
    double ups1 = 0.0, ups2 = 0.0, ups3 = 0.0, u1 = 0.0, u2 = 0.0, u3 = 0.0;
    // west / south edge faces shared with the neighbouring tile
    int iw = 0, k1w = 0, k1s = 0;
    double uw = 0.0, upsw = 0.0, us = 0.0, upss = 0.0;
    bool edge_w = (ti == 0), edge_s = (tj == 0);
    // isoneutral per-cell state
    bool iso = false;
    double dxrho[4] = {0, 0, 0, 0}, dyrho[4] = {0, 0, 0, 0}, slim = 1.0, isofac = 0.0, dz2 = 0.0, dzrho2 = 0.0;
    double dmax_local = 0.0;
    unsigned int limps_local = 0;

    if (inside) {
        k1c = M.k1[i + d.NI * j];
        ie = (i == maxi) ? 1 : i + 1;   // the i=maxi east face is the western doorway (goldstein.f90:2473-2487)
        k1e = M.k1[ie + d.NI * j];
        k1n = M.k1[i + d.NI * (j + 1)];
        wet = k >= k1c;
        vwet = wet && (k < maxk);
        if (vwet) {
            eosd_d(p, a.ts1[ts_index(d, 0, i, j, k)], a.ts1[ts_index(d, 0, i, j, k + 1)],
                   a.ts1[ts_index(d, 1, i, j, k)], a.ts1[ts_index(d, 1, i, j, k + 1)], M.zw[k], M.rdza[k], dzrho, tec);
            rdzrho = (dzrho < -1.0e-12) ? 1.0 / dzrho : -1.0e12;
            if (p.iediff > 0 && p.iediff < 3) {
                const double e1 = M.ediff1[(size_t)(i - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (size_t)(k - 1))];
                if (p.ediffpow2i == 0) diffv = p.ediff0 + e1;
                else if (p.ediffpow2i == 1) diffv = p.ediff0 + e1 * (-rdzrho);
                else if (p.ediffpow2i == 2) diffv = p.ediff0 + e1 * sqrt(-rdzrho);
                else diffv = p.ediff0 + e1 * pow(-rdzrho, p.ediffpow2);
                if (diffv > M.diffmax[k + 1]) diffv = M.diffmax[k + 1];
            }
        }
        u1 = a.u[u_index(d, 0, i, j, k)];
        u2 = a.u[u_index(d, 1, i, j, k)];
        u3 = a.u[u_index(d, 2, i, j, k)];
        ups1 = upstream(u1 * p.dphi / p.diff1);
        ups2 = upstream(u2 * M.dsv[j < maxj - 1 ? j : maxj - 1] / p.diff1);
        ups3 = upstream(u3 * M.dza[k] / diffv);
        if (edge_w) {
            iw = (i == 1) ? maxi : i - 1;
            k1w = M.k1[iw + d.NI * j];
            uw = a.u[u_index(d, 0, iw, j, k)];
            upsw = upstream(uw * p.dphi / p.diff1);
        }
        if (edge_s && j > 1) {
            k1s = M.k1[i + d.NI * (j - 1)];
            us = a.u[u_index(d, 1, i, j - 1, k)];
            upss = upstream(us * M.dsv[(j - 1) < maxj - 1 ? (j - 1) : maxj - 1] / p.diff1);
        }
        // isoneutral slope and taper (goldstein.f90:2561-2608)
        if (p.diso && vwet && dzrho < -1.0e-12) {
            iso = true;
            const double scc = p.ec[1];
            double tv1 = 0.0;
            for (int knp = 0; knp <= 1; ++knp) {
                for (int nnp = 0; nnp <= 1; ++nnp) {
                    const int ina = nnp + 2 * knp;
                    const int kk = k + knp;
                    double dxt[2] = {0.0, 0.0}, dyt[2] = {0.0, 0.0};
                    const bool mx = kk >= M.k1[(i - 1 + 2 * nnp) + d.NI * j];
                    const bool my = kk >= M.k1[i + d.NI * (j - 1 + 2 * nnp)];
                    for (int l = 0; l < 2; ++l) {
                        if (mx) dxt[l] = (a.ts1[ts_index(d, l, i + nnp, j, kk)] - a.ts1[ts_index(d, l, i + nnp - 1, j, kk)]) * M.rc[j] * p.rdphi;
                        if (my) dyt[l] = (a.ts1[ts_index(d, l, i, j + nnp, kk)] - a.ts1[ts_index(d, l, i, j + nnp - 1, kk)]) * M.cv[j - 1 + nnp] * M.rdsv[j + nnp - 1];
                    }
                    dxrho[ina] = scc * dxt[1] - tec * dxt[0];
                    dyrho[ina] = scc * dyt[1] - tec * dyt[0];
                    tv1 = tv1 + dxrho[ina] * dxrho[ina] + dyrho[ina] * dyrho[ina];
                }
            }
            tv1 = 0.25 * tv1 * rdzrho * rdzrho;
            const double ss = M.ssmax[k];
            if (tv1 > ss) {
                slim = ss * ss / (tv1 * tv1);
                limps_local = 1;
            } else {
                slim = 1.0;
            }
            tv1 = tv1 * slim * p.diff1 * M.rdza[k];
            const double tvd = tv1 * M.dt[k] * M.rdza[k];
            if (tvd > dmax_local) dmax_local = tvd;
            isofac = 0.25 * slim * p.diff1;
            dz2 = 2 * dzrho;
            dzrho2 = dzrho * dzrho;
        }
    }

    // ---- per tracer: faces, exchange, update (goldstein.f90:2524-2636) ----
    double tnew0 = 0.0, tnew1 = 0.0;
    const double rcj = inside ? M.rc[j] : 0.0, rc2j = inside ? M.rc2[j] : 0.0;
    const double cvj = inside ? M.cv[j] : 0.0, cv2j = (inside && j < maxj) ? M.cv2[j] : 0.0;
    const double a_e = u1 * rcj;          // u(1)*rc(j)
    const double a_n = cvj * u2;          // cv(j)*u(2)
    for (int l = 0; l < d.L; ++l) {
        double fe = 0.0, fn = 0.0, fa = 0.0, tc = 0.0;
        if (inside) {
            tc = a.ts1[ts_index(d, l, i, j, k)];
            if (k >= max(k1c, k1e)) {
                fe = face_flux(a_e, ups1, a.ts1[ts_index(d, l, ie, j, k)], tc, rc2j, p.diff1);
            }
            if (k >= max(k1c, k1n)) {
                const double tp = a.ts1[ts_index(d, l, i, j + 1, k)];
                fn = a_n * ((1.0 - ups2) * tp + (1.0 + ups2) * tc) * 0.5;
                fn = fn - cv2j * (tp - tc) * p.diff1;
            }
            if (k < k1c) {
                fa = 0.0;
            } else if (k == maxk) {
                fa = a.top[(size_t)l + (size_t)d.L * ((size_t)i + (size_t)d.NI * (size_t)j)];
            } else {
                const double ta = a.ts1[ts_index(d, l, i, j, k + 1)];
                fa = u3 * ((1.0 - ups3) * ta + (1.0 + ups3) * tc) * 0.5;
                fa = fa - (ta - tc) * M.rdza[k] * diffv;
                if (iso) {
                    // isoneutral vertical flux (goldstein.f90:2609-2621)
                    const double dzts = (ta - tc) * M.rdza[k];
                    double tv = 0.0;
                    for (int knp = 0; knp <= 1; ++knp) {
                        for (int nnp = 0; nnp <= 1; ++nnp) {
                            const int ina = nnp + 2 * knp;
                            const int kk = k + knp;
                            double dxt = 0.0, dyt = 0.0;
                            if (kk >= M.k1[(i - 1 + 2 * nnp) + d.NI * j])
                                dxt = (a.ts1[ts_index(d, l, i + nnp, j, kk)] - a.ts1[ts_index(d, l, i + nnp - 1, j, kk)]) * rcj * p.rdphi;
                            if (kk >= M.k1[i + d.NI * (j - 1 + 2 * nnp)])
                                dyt = (a.ts1[ts_index(d, l, i, j + nnp, kk)] - a.ts1[ts_index(d, l, i, j + nnp - 1, kk)]) * M.cv[j - 1 + nnp] * M.rdsv[j + nnp - 1];
                            tv = tv + (dz2 * dxt - dxrho[ina] * dzts) * dxrho[ina] + (dz2 * dyt - dyrho[ina] * dzts) * dyrho[ina];
                        }
                    }
                    tv = isofac * tv / dzrho2;
                    fa = fa + tv;
                }
            }
            fe_at(ti + 1, tj, kz) = fe;
            fn_at(ti, tj + 1, kz) = fn;
            fa_at(ti, tj, kz + 1) = fa;
            if (kz == 0) fa_at(ti, tj, 0) = 0.0;
            if (edge_w) {
                double fw = 0.0;
                if (k >= max(k1w, k1c)) {
                    // east face of column iw, whose east neighbour is column i
                    fw = face_flux(uw * rcj, upsw, tc, a.ts1[ts_index(d, l, iw, j, k)], rc2j, p.diff1);
                }
                fe_at(0, tj, kz) = fw;
            }
            if (edge_s) {
                double fs = 0.0;
                if (j > 1 && k >= max(k1s, k1c)) {
                    const double tsouth = a.ts1[ts_index(d, l, i, j - 1, k)];
                    fs = M.cv[j - 1] * us * ((1.0 - upss) * tc + (1.0 + upss) * tsouth) * 0.5;
                    fs = fs - M.cv2[j - 1] * (tc - tsouth) * p.diff1;
                }
                fn_at(ti, 0, kz) = fs;
            }
        }
        __syncthreads();
        if (inside && wet) {
            const double fw = fe_at(ti, tj, kz), fs = fn_at(ti, tj, kz), fb = fa_at(ti, tj, kz);
            const double tv = 0.0;
            const double nv = tc - M.dt[k] * (-tv + (fe - fw) * p.rdphi + (fn - fs) * M.rds[j] + (fa - fb) * M.rdz[k]);
            a.ts[ts_index(d, l, i, j, k)] = nv;
            if (l == 0) tnew0 = nv;
            if (l == 1) tnew1 = nv;
        }
        __syncthreads();
    }

    // ---- rho for every interior cell (goldstein.f90:2638) ----
    if (inside) {
        double t0, t1;
        if (wet) {
            t0 = tnew0;
            t1 = tnew1;
        } else {
            t0 = a.ts_static[ts_index(d, 0, i, j, k)];
            t1 = a.ts_static[ts_index(d, 1, i, j, k)];
        }
        if (p.imld == 1 && k == maxk) {
            // imld = 1: energy of mixing the surface forcing over the top layer, from ts at
            // the start of the step and the previous step's rho (goldstein.f90:2294-2309)
            const size_t o = (size_t)d.L * ((size_t)i + (size_t)d.NI * (size_t)j);
            const double tt = a.ts_start[ts_index(d, 0, i, j, maxk)] - a.top[o];
            const double st = a.ts_start[ts_index(d, 1, i, j, maxk)] - a.top[o + 1];
            const double r = eos_d(p, tt, st, M.zro[maxk]);
            a.mldpe1[(size_t)(i - 1) + (size_t)maxi * (size_t)(j - 1)] =
                (r - a.rho[rho_index(d, i, j, maxk)]) * z2dzg_d(M, maxk, maxk);
        }
        a.rho[rho_index(d, i, j, k)] = eos_d(p, t0, t1, M.zro[k]);
    }

    // ---- diagnostics dmax / limps ----
    if (p.diso) {
        unsigned long long dbits = __double_as_longlong(dmax_local);
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long ob = __shfl_xor_sync(0xffffffffu, dbits, o);
            dbits = ob > dbits ? ob : dbits;
            limps_local += __shfl_xor_sync(0xffffffffu, limps_local, o);
        }
        if ((t & 31) == 0) {
            if (dbits) atomicMax(&a.diag[0], dbits);
            if (limps_local) atomicAdd(&a.diag[1], (unsigned long long)limps_local);
        }
    }
    __syncthreads();

    // ---- convective adjustment + periodic halos, one thread per column ----
    if (inside && kz == 0 && k1c <= maxk) {
        ColumnView cv{a.ts, a.ts_static, &a.d, i, j, k1c};
        const size_t c2 = (size_t)(i - 1) + (size_t)maxi * (size_t)(j - 1);
        // imld = 1: densities before co (the flux step's, every level) for its energy release
        double rold[GB_GO_MAX_K + 1];
        if (p.imld == 1)
            for (int kk = 1; kk <= maxk; ++kk) rold[kk] = a.rho[rho_index(d, i, j, kk)];
        int32_t icos = 0;
        if (p.iconv == 1) coshuffle_column(a, cv, icos);
        const int filled = co_column(a, cv);
        if (p.iconv == 1) {
            if (filled > icos) icos = filled;
            a.icosd[c2] = icos;
            a.cost[c2] = p.dsc * M.zw[maxk - 1 - icos];
        } else if (filled > 0) {
            a.cost[c2] = add_count_rn(a.cost[c2], filled);
        }
        if (p.imld == 1) mixed_layer_column(a, cv, c2, rold);
        if (p.ieos != 0) {
            for (int kk = 1; kk <= maxk; ++kk) {
                const double t0 = kk >= k1c ? a.ts[ts_index(d, 0, i, j, kk)] : a.ts_static[ts_index(d, 0, i, j, kk)];
                const double t1 = kk >= k1c ? a.ts[ts_index(d, 1, i, j, kk)] : a.ts_static[ts_index(d, 1, i, j, kk)];
                a.rho[rho_index(d, i, j, kk)] = eos_d(p, t0, t1, M.zro[kk]);
            }
        }
    }
    // halo columns need this column's final values: i = maxi feeds i = 0,
    // i = 1 feeds i = maxi+1 (goldstein.f90:2412-2421)
    if (inside && kz == 0 && (i == maxi || i == 1)) {
        for (int side = 0; side < 2; ++side) {
            int src, dst;
            if (side == 0) { if (i != maxi) continue; src = maxi; dst = 0; }
            else { if (i != 1) continue; src = 1; dst = maxi + 1; }
            const int kh = M.k1[dst + d.NI * j];
            for (int kk = kh; kk <= maxk; ++kk) {
                a.rho[rho_index(d, dst, j, kk)] = a.rho[rho_index(d, src, j, kk)];
                for (int l = 0; l < d.L; ++l) a.ts[ts_index(d, l, dst, j, kk)] = a.ts[ts_index(d, l, src, j, kk)];
            }
        }
    }
}

void step_fp64_tile(int maxi, int maxj, int maxk, int nsm, int *tile_i, int *tile_j)
{
    // Column tiles from large to small (one thread per cell, at most 256): the largest that
    // still gives every SM kFp64TilesPerSm CTAs.  Larger tiles compute fewer edge faces
    // twice; a small grid needs small tiles to occupy the GPU (one 36x36 grid of 4x4 tiles
    // fills 81 of 152 SMs).
    static const int cand[][2] = {{8, 4}, {4, 4}, {4, 2}, {2, 2}, {2, 1}, {1, 1}};
    int bi = 1, bj = 1;
    for (const auto &c : cand) {
        if (c[0] * c[1] * maxk > 256) continue;
        bi = c[0];
        bj = c[1];
        const long long tiles = (long long)((maxi + c[0] - 1) / c[0]) * ((maxj + c[1] - 1) / c[1]);
        if (tiles >= (long long)kFp64TilesPerSm * nsm) break;
    }
    *tile_i = bi;
    *tile_j = bj;
}

int launch_step_fp64(const StepArgs &a, void *stream)
{
    const int TX = a.tile_i, TY = a.tile_j, K = a.d.maxk;
    const int tiles_i = (a.d.maxi + TX - 1) / TX, tiles_j = (a.d.maxj + TY - 1) / TY;
    const size_t shmem = sizeof(double) * ((size_t)K * TY * (TX + 1) + (size_t)K * (TY + 1) * TX + (size_t)(K + 1) * TY * TX);
    const int threads = (TX * TY * K + 31) / 32 * 32;   // <= 256 for every tile choice above
    k_step_fp64<<<tiles_i * tiles_j, threads, shmem, (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace gbgo
