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

#include "gb_fp32.h"
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

// ---------------------------------------------------------------------------
// Double-float densities for the order decisions of the adjustment (ieos = 0).
// An FP32 pair (hi, lo) carries ~47 bits, so the density difference of two levels is
// known to ~1e-13 of the size of the terms; only closer pairs need the FP64 density.

struct CoDf {
    float hi, lo;
};

// x as an FP32 pair by integer operations: hi = x with its mantissa truncated to 24 bits,
// lo = the remaining 29 bits rounded to FP32, so |x - hi - lo| <= 2^-47 |x|.  A nonzero |x|
// outside [2^-74, 2^60] gives a NaN pair: every decision that uses it takes the FP64 path.
__device__ __forceinline__ CoDf co_split(double x)
{
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const unsigned a = hw & 0x7fffffffu, sgn = hw & 0x80000000u;
    const int E = (int)(a >> 20);
    if ((a | lw) == 0u) return {0.0f, 0.0f};
    if (E < 949 || E > 1082) return {__int_as_float(0x7fc00000), 0.0f};
    const float hi = __uint_as_float(sgn | ((unsigned)(E - 896) << 23) | ((a & 0xfffffu) << 3) | (lw >> 29));
    const float lo = __fmul_rn(__uint2float_rn(lw & 0x1fffffffu), __uint_as_float((unsigned)(E - 948) << 23));
    return {hi, __uint_as_float(__float_as_uint(lo) | sgn)};
}

// a + b, |a| >= |b| (or a = 0): exact pair
__device__ __forceinline__ CoDf co_fast2sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// pair sum (Knuth's TwoSum of the hi parts, lo parts added): error <= ~3u^2 (|a| + |b|),
// u = 2^-24
__device__ __forceinline__ CoDf co_dfadd(CoDf a, CoDf b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    return co_fast2sum(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}

// pair product (exact FMA product of the hi parts, cross terms; lo*lo dropped):
// relative error <= ~7u^2
__device__ __forceinline__ CoDf co_dfmul(CoDf a, CoDf b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return co_fast2sum(p, e);
}

// eos (goldstein.f90:3048-3061, ieos = 0) as a pair, and M = the sum of the magnitudes of
// its four terms.  Split errors (2^-47 per input, three-fold in t^3), the products and the
// three sums keep |result - eos_rn| below ~45u^2 M < 2^-42 M.
__device__ __forceinline__ CoDf eos_df(const CoDf ecd[4], double t, double s, float &mag)
{
    const CoDf td = co_split(t), sd = co_split(s);
    const CoDf tt = co_dfmul(td, td);
    const CoDf ttt = co_dfmul(tt, td);
    const CoDf p0 = co_dfmul(ecd[0], td), p1 = co_dfmul(ecd[1], sd);
    const CoDf p2 = co_dfmul(ecd[2], tt), p3 = co_dfmul(ecd[3], ttt);
    mag = __fadd_rn(__fadd_rn(fabsf(p0.hi), fabsf(p1.hi)), __fadd_rn(fabsf(p2.hi), fabsf(p3.hi)));
    return co_dfadd(co_dfadd(co_dfadd(p0, p1), p2), p3);
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
    long long rho[kMaxK + 1];   // exact keys; with ieos = 0 computed when first needed (kNoKey before)
    float2 rd[kMaxK + 1];       // ieos = 0: double-float density of the level
    float rm[kMaxK + 1];        // ieos = 0: the magnitude M of its terms (error scale)
};

constexpr long long kNoKey = (long long)0x8000000000000000ULL;

// co_rn with one warp per column: the tracers of the column are in shared memory,
// tv[lev * 32 + l] for the wet levels, and lane l mixes and fills tracer l.  The levels
// to merge (kk, dzm, densities in cs) live in shared memory and are updated by lane 0;
// every lane runs the same decisions from them.  Every value and decision is the one co_rn
// makes.  Returns the number of filled levels (in every lane).
// With ieos = 0 a density depends on (T, S) only, and a decision rho(a) < rho(b) is taken
// from the double-float densities when their difference exceeds 2^-40 (M_a + M_b) (more
// than 4x their error bound); otherwise (and for bit-equal T and S, which give equal
// densities) from the exact FP64 densities, computed once per level value.  With
// ieos != 0 the FP64 densities are recomputed as co does.
__device__ inline int co_warp(double *tv, CoWarpState *cs, const EosCoef &ec, int maxk, int L, int k1,
                              const double *dz, const double *zro, const double *zw, int lane)
{
    int *kk = cs->kk;
    double *dzm = cs->dzm;
    long long *rho = cs->rho;
    float2 *rd = cs->rd;
    float *rm = cs->rm;
    const bool lazy = ec.ieos == 0;
    auto T = [&](int l, int lev) { return tv[lev * 32 + l]; };
    CoDf ecd[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) ecd[n] = co_split(ec.ec[n]);
    auto set_df = [&](int lev) {
        float mg;
        const CoDf r = eos_df(ecd, T(0, lev), T(1, lev), mg);
        rd[lev] = make_float2(r.hi, r.lo);
        rm[lev] = mg;
        rho[lev] = kNoKey;
    };
    for (int lev = k1 + lane; lev <= maxk; lev += 32) {
        if (lazy) set_df(lev);
        else rho[lev] = order_key(eos_rn(ec, T(0, lev), T(1, lev), zro[lev]));
        kk[lev] = lev;
        dzm[lev] = dz[lev];
    }
    if (lane == 0) {
        rho[0] = 0;
        kk[k1 - 1] = 0;
    }
    __syncwarp();
    auto refresh = [&](int x, int y) {
        if (!lazy) {
            if (lane == 0) {
                rho[kk[x]] = order_key(eos_rn(ec, T(0, kk[x]), T(1, kk[x]), zw[kk[y]]));
                rho[kk[y]] = order_key(eos_rn(ec, T(0, kk[y]), T(1, kk[y]), zw[kk[y]]));
            }
            __syncwarp();
        }
    };
    // rho(a) < rho(b) for wet levels a, b (uniform over the warp)
    auto lt = [&](int a, int b) -> bool {
        if (lazy) {
            const float2 ra = rd[a], rb = rd[b];
            const float d = __fadd_rn(__fsub_rn(ra.x, rb.x), __fsub_rn(ra.y, rb.y));
            const float tol = __fmul_rn(0x1p-40f, __fadd_rn(rm[a], rm[b]));
            if (d < -tol) return true;
            if (d > tol) return false;
            if (__double_as_longlong(T(0, a)) == __double_as_longlong(T(0, b)) &&
                __double_as_longlong(T(1, a)) == __double_as_longlong(T(1, b)))
                return false;
            if (lane == 0) {
                if (rho[a] == kNoKey) rho[a] = order_key(eos_rn(ec, T(0, a), T(1, a), zro[a]));
                if (rho[b] == kNoKey) rho[b] = order_key(eos_rn(ec, T(0, b), T(1, b), zro[b]));
            }
            __syncwarp();
        }
        return rho[a] < rho[b];
    };
    // m, n, lastmix follow from the shared arrays, so they are the same in every lane
    int m = maxk, lastmix = 0;
    while (kk[m - 1] > 0 || (lastmix != 0 && kk[m] != maxk)) {
        refresh(m, m - 1);
        if (kk[m - 1] == 0 || lt(kk[m], kk[m - 1])) {
            if (lastmix == 0 || kk[m] == maxk) m = m - 1;
            else m = m + 1;
            lastmix = 0;
        } else {
            lastmix = 1;
            int n = m - 1;
            refresh(n, n - 1);
            while (kk[n - 1] > 0 && !lt(kk[n], kk[n - 1])) {
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
                if (lazy) set_df(km);
                else rho[km] = order_key(eos_rn(ec, T(0, km), T(1, km), zw[kk[m - 1]]));
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


// ---------------------------------------------------------------------------
// Convective adjustment of the columns with maxk <= 32 and ieos = 0 in two phases.
//
// Decisions (k_co_decide): one lane per column runs co (goldstein.f90:2657-2777) on T and S,
// with the list kk held as a bit mask of the active levels (a merge of positions n..m clears
// the levels it absorbs), so the walk down a stable stretch (2715-2719), the scan for the
// bottom of an unstable stretch (2727-2731) and the step back up after a merge are bit
// operations.  The lanes advance in rounds: each lane walks to its next merge, then every
// lane that has one mixes T and S (2732-2746) at once, so a round's FP64 instructions serve
// all the merging columns of the warp (GB300's FP64 pipe costs per warp instruction, not per
// active lane).  Each merge is logged: the top level, the absorbed levels in co's order with
// the thicknesses co used, and the summed thickness.
// Tracers (k_co_mix): one lane per (column, tracer l >= 2) replays its column's log in co's
// order and arithmetic, then the fill (2748-2765) from the final list.
// Density decisions as in the one-warp-per-column form below (double-float densities, exact
// FP64 eos where they are closer than their error bound, equal T and S as equal densities).
// Each merge divides by its summed thickness through co_div with the reciprocal computed once
// per merge.  The two-phase form pays a fixed latency per batch of 32 columns, so it serves
// large batches; the one-warp-per-column form below serves small ones.

// bits of levels lo..hi (level l = bit l-1)
__device__ __forceinline__ unsigned co_bits(int lo, int hi)
{
    if (hi < lo) return 0u;
    const unsigned up = hi >= 32 ? 0xffffffffu : ((1u << hi) - 1u);
    return up & ~((1u << (lo - 1)) - 1u);
}

// ---------------------------------------------------------------------------
// The one-warp-per-column form (small batches) of the columns with maxk <= 32 and ieos = 0.
//
// co's working list kk (position -> level, the sentinel 0 below the lowest active
// position) is held one position per lane (position p = lane + 1), each position
// carrying the record of its level: thickness dzm, T, S, double-float density and the
// exact FP64 key once computed.  A round evaluates every pair (p, p-1) at once
// (ballot), so co's walk down a stable stretch (goldstein.f90:2715-2719), and the scan
// for the bottom of an unstable stretch (2727-2731), each take one round; a merge
// (2732-2746) shifts the records below it with one shuffle.  Decisions, merge order and
// arithmetic are co's; the fill (2748-2765) is computed from the final list.

struct CoRec {
    int kk;            // level at this position
    double dzm, t, s;  // thickness, T and S of that level
    float rdh, rdl, rm;
    long long key;     // exact order key of its FP64 density, kNoKey until needed
};

__device__ __forceinline__ CoRec co_rec_up(const CoRec &r, int d)
{
    const unsigned F = 0xffffffffu;
    CoRec o;
    o.kk = __shfl_up_sync(F, r.kk, d);
    o.dzm = __shfl_up_sync(F, r.dzm, d);
    o.t = __shfl_up_sync(F, r.t, d);
    o.s = __shfl_up_sync(F, r.s, d);
    o.rdh = __shfl_up_sync(F, r.rdh, d);
    o.rdl = __shfl_up_sync(F, r.rdl, d);
    o.rm = __shfl_up_sync(F, r.rm, d);
    o.key = __shfl_up_sync(F, r.key, d);
    return o;
}


// tv: shared memory, tv[lev * 32 + l]; ts0: T of the column at level 0 (S follows), level
// stride s0; wc (lanes < L): this lane's tracer at level 0, level stride lstride.  Loads
// the column, adjusts it, writes back the levels that changed; returns the number of
// filled levels.
__device__ inline int co_warp32(double *tv, const EosCoef &ec, int maxk, int L, int k1, const double *dz,
                                int lane, const double *ts0, size_t s0, double *wc, size_t lstride)
{
    const unsigned F = 0xffffffffu;
    const int p = lane + 1;
    CoDf ecd[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) ecd[n] = co_split(ec.ec[n]);
    CoRec rec;
    rec.kk = p;
    rec.dzm = 0.0;
    rec.t = 0.0;
    rec.s = 0.0;
    rec.rdh = rec.rdl = rec.rm = 0.0f;
    rec.key = kNoKey;
    if (p >= k1 && p <= maxk) {
        const double2 v = *reinterpret_cast<const double2 *>(ts0 + (size_t)p * s0);
        rec.t = v.x;
        rec.s = v.y;
        rec.dzm = dz[p];
        float mg;
        const CoDf r = eos_df(ecd, v.x, v.y, mg);
        rec.rdh = r.hi;
        rec.rdl = r.lo;
        rec.rm = mg;
    }
    int sp = k1 - 1;   // sentinel position
    // bit p-1 set iff rho(kk[p]) < rho(kk[p-1]) or p-1 is the sentinel, for p in [sp+2, lim];
    // positions outside that range read as stable
    auto stable_mask = [&](int lim) -> unsigned {
        const float bh = __shfl_up_sync(F, rec.rdh, 1), bl = __shfl_up_sync(F, rec.rdl, 1);
        const float bm = __shfl_up_sync(F, rec.rm, 1);
        int st = 1;
        if (p >= sp + 2 && p <= lim) {
            const float d = __fadd_rn(__fsub_rn(rec.rdh, bh), __fsub_rn(rec.rdl, bl));
            const float tol = __fmul_rn(0x1p-40f, __fadd_rn(rec.rm, bm));
            st = d < -tol ? 1 : (d > tol ? 0 : 2);
        }
        if (__any_sync(F, st == 2)) {
            const double bt = __shfl_up_sync(F, rec.t, 1), bs = __shfl_up_sync(F, rec.s, 1);
            // equal T and S: equal densities, not stable
            if (st == 2 && __double_as_longlong(rec.t) == __double_as_longlong(bt) &&
                __double_as_longlong(rec.s) == __double_as_longlong(bs))
                st = 0;
            const int above = __shfl_down_sync(F, st, 1);
            if ((st == 2 || (lane < 31 && above == 2)) && rec.key == kNoKey)
                rec.key = order_key(eos_rn(ec, rec.t, rec.s, 0.0));
            const long long bk = __shfl_up_sync(F, rec.key, 1);
            if (st == 2) st = rec.key < bk ? 1 : 0;
        }
        return __ballot_sync(F, st == 1);
    };
    unsigned stab = stable_mask(maxk);
    // no unstable pair: co changes nothing
    if ((~stab & co_bits(k1 + 1, maxk)) == 0u) return 0;
    if (lane < L)
        for (int lev = k1; lev <= maxk; lev += 8) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (lev + u <= maxk) v[u] = wc[(size_t)(lev + u) * lstride];
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (lev + u <= maxk) tv[(lev + u) * 32 + lane] = v[u];
        }
    __syncwarp();
    unsigned modified = 0u;
    int m = maxk, lastmix = 0;
    bool fresh = true;   // stab holds the pairs of the current list up to m
    while (m > sp + 1 || (lastmix != 0 && m != maxk)) {
        if (!fresh) stab = stable_mask(m);
        fresh = false;
        if (lastmix == 0) {
            // walk down the stable pairs to the highest unstable one
            const unsigned un = ~stab & co_bits(sp + 2, m);
            if (un == 0u) break;
            m = 32 - __clz(un);
        } else if ((stab >> (m - 1)) & 1u) {
            m = (m == maxk) ? m - 1 : m + 1;
            lastmix = 0;
            continue;
        }
        // merge positions n..m: n = the highest stable position below m (sp+1 always is)
        const int n = 32 - __clz(stab & co_bits(sp + 1, m - 1));
        const int d = m - n, lm = m - 1;
        const int km = __shfl_sync(F, rec.kk, lm);
        const double d0 = __shfl_sync(F, rec.dzm, lm);
        double dtot = d0, acc = 0.0;
        if (lane < L) acc = __dmul_rn(tv[km * 32 + lane], d0);
        for (int ni = 1; ni <= d; ++ni) {
            const int lv = __shfl_sync(F, rec.kk, lm - ni);
            const double dzv = __shfl_sync(F, rec.dzm, lm - ni);
            dtot = __dadd_rn(dtot, dzv);
            if (lane < L) acc = __dadd_rn(acc, __dmul_rn(tv[lv * 32 + lane], dzv));
        }
        if (lane < L) tv[km * 32 + lane] = __ddiv_rn(acc, dtot);
        __syncwarp();
        modified |= 1u << (km - 1);
        if (lane == lm) {
            rec.dzm = dtot;
            rec.t = tv[km * 32];
            rec.s = tv[km * 32 + 1];
            float mg;
            const CoDf r = eos_df(ecd, rec.t, rec.s, mg);
            rec.rdh = r.hi;
            rec.rdl = r.lo;
            rec.rm = mg;
            rec.key = kNoKey;
        }
        // positions sp+d .. m-1 take the records d below (sp+d becomes the sentinel)
        const CoRec sh = co_rec_up(rec, d);
        if (p >= sp + d && p <= m - 1) rec = sh;
        sp += d;
        lastmix = 1;
    }
    // fill: every level of [k1, maxk-1] no longer in the list takes the values of the
    // lowest listed level above it
    const unsigned act = __reduce_or_sync(F, (p >= sp + 1 && p <= maxk) ? (1u << (rec.kk - 1)) : 0u);
    const unsigned fillm = ~act & co_bits(k1, maxk - 1);
    for (unsigned f = fillm; f; f &= f - 1u) {
        const int lev = __ffs(f);
        const int src = __ffs(act & ~((1u << lev) - 1u));
        if (lane < L) tv[lev * 32 + lane] = tv[src * 32 + lane];
    }
    modified |= fillm;
    __syncwarp();
    if (lane < L)
        for (unsigned f = modified; f; f &= f - 1u) {
            const int lev = __ffs(f);
            wc[(size_t)lev * lstride] = tv[lev * 32 + lane];
        }
    return __popc(fillm);
}

// Merge log of a column (one slot of kCoLogBytes per list entry): header {int nm, unsigned
// final mask}; per merge k: dtot[k] (summed thickness), y[k] = RN(1 / dtot[k]), dtop[k] (the
// top level's thickness before it), x[k] (top level), cnt[k] (levels absorbed); per absorbed
// level in co's order: its thickness and level.  maxk <= 32: at most 31 merges and 31
// absorbed levels.
constexpr int kCoLogBytes = (int)kCoLogSlotBytes;
constexpr int kCoLogDtot = 16, kCoLogY = 264, kCoLogDtop = 512, kCoLogEdz = 760, kCoLogX = 1008, kCoLogCnt = 1039,
              kCoLogElev = 1070;
static_assert(kCoLogElev + 31 <= kCoLogBytes, "merge log layout");

// RN(a / b) given y = RN(1 / b): q0 = a y, then two residual corrections q <- q + (a - b q) y
// (fma).  The first makes q faithful, the second correctly rounded (Markstein's theorem:
// P. Markstein, IBM J. Res. Dev. 34 (1990) 111-119; the remainder a - b q of a faithful q is
// exact).  Five FP64 operations instead of a division; operands outside the range where every
// intermediate stays normal (and a = 0, whose sign the corrections would lose) divide.
__device__ __forceinline__ double co_div(double a, double b, double y)
{
    const int ea = (__double2hiint(a) >> 20) & 0x7ff, eb = (__double2hiint(b) >> 20) & 0x7ff;
    if (ea < 512 || ea > 1535 || eb < 768 || eb > 1279) return __ddiv_rn(a, b);
    const double q0 = __dmul_rn(a, y);
    const double q1 = __fma_rn(__fma_rn(-b, q0, a), y, q0);
    return __fma_rn(__fma_rn(-b, q1, a), y, q1);
}

// Tracer l of a member's column: its value at level 0 and the level stride (group-planar
// layout: tracer groups in planes of NI*NJ*(maxk+2) cells of gp values).
__device__ __forceinline__ double *co_tracer(double *W, int L, size_t plane, size_t cell, size_t NIJ, int l, size_t &lstride)
{
    int g0 = 0, gl = 2, gp = 2, pl = 0;
    for (int g = 0; g < fp32_ngroups(L); ++g) {
        fp32_plane(L, g, &g0, &gl, &gp, &pl);
        if (l < g0 + gl) break;
    }
    lstride = NIJ * (size_t)gp;
    return W + (size_t)pl * plane + (size_t)(l - g0) + cell * (size_t)gp;
}

// ---------------------------------------------------------------------------
// Kraus-Turner mixed layer (imld = 1) of one wet column, with explicit round-to-nearest
// intrinsics like co above, so that the FP32-flux form applies the reference's arithmetic
// (and the same operation order as the FP64 drop-in kernel) to its FP64 state.
//   energy of the surface forcing    goldstein.f90:2294-2309
//   energy released by co, decision  goldstein.f90:2336-2389
//   krausturner                      goldstein.f90:3337-3442
// Level-pair depth grids of goldstein.f90:1013-1025: dzg(k,kk) = zw(k) - zw(kk-1),
// z2dzg(k,kk) = -zw(k)^2 + zw(kk-1)^2, rdzg(k,kk) = 1/dzg(k,kk) (1e10 where k = kk-1).

struct MixedLayerArgs {
    const double *zw, *zro, *dz;        // Fortran-indexed k metrics
    const double *mlddec, *mlddecd;     // [1..maxk]
    double mldpebuoycoeff;
    double ketau;                       // the column's wind mixing energy
    double pe1;                         // the column's mldpe1 (forcing energy over the top layer)
};

__device__ __forceinline__ double ml_dzg(const double *zw, int k, int kk) { return __dadd_rn(zw[k], -zw[kk - 1]); }
__device__ __forceinline__ double ml_z2dzg(const double *zw, int k, int kk)
{
    return __dadd_rn(__dmul_rn(-zw[k], zw[k]), __dmul_rn(zw[kk - 1], zw[kk - 1]));
}
__device__ __forceinline__ double ml_rdzg(const double *zw, int k, int kk)
{
    return k != kk - 1 ? __ddiv_rn(1.0, ml_dzg(zw, k, kk)) : 1.0E10;
}

// mldpe1 of goldstein.f90:2294-2309: the density change of the top layer when the step's
// surface forcing is taken out of its start-of-step T and S (tt, st), against the density
// the previous step left there (rho_prev), times z2dzg(maxk, maxk)
__device__ __forceinline__ double ml_pe1(const EosCoef &ec, double tt, double st, double rho_prev, const double *zw,
                                         const double *zro, int maxk)
{
    const double r = eos_rn(ec, tt, st, zro[maxk]);
    return __dmul_rn(__dadd_rn(r, -rho_prev), ml_z2dzg(zw, maxk, maxk));
}

// krausturner on one column (tvkl = k1, every level it touches is wet)
template <class Col>
__device__ void kraus_turner_rn(Col &col, const EosCoef &ec, int maxk, int L, int tvkl, const MixedLayerArgs &a,
                                double pebuoy, double *mld, int32_t *mldk)
{
    const double *zw = a.zw, *dz = a.dz;
    double qmix[kFp32MaxL];
    const int mldpk = maxk;   // the routine's first statement (goldstein.f90:3350)
    int k = mldpk, partmix = 1;
    double empe = pebuoy;
    double emke = __dmul_rn(a.ketau, a.mlddec[k]);
    double em = __dadd_rn(empe, emke);
    double eneed = 0.0;
    double tmix = col.T(0, k), smix = col.T(1, k);
    double rhou = 0.0, rhol = 0.0;
    for (int l = 0; l < L; ++l) qmix[l] = col.T(l, k);
    double rhomix = eos_rn(ec, tmix, smix, zw[k]);
    while (eneed < em && em > 0) {
        if (k < mldpk) {
            qmix[0] = tmix;
            qmix[1] = smix;
            const double r = ml_rdzg(zw, maxk, k), g = ml_dzg(zw, maxk, k + 1);
            for (int l = 2; l < L; ++l) qmix[l] = __dmul_rn(r, __dadd_rn(__dmul_rn(qmix[l], g), __dmul_rn(col.T(l, k), dz[k])));
        }
        if (k == tvkl) {
            *mldk = k;
            *mld = zw[k - 1];
            partmix = 0;
            em = -1.0E-8;
            if (k < maxk)
                for (int l = 0; l < L; ++l)
                    for (int n = k; n <= maxk; ++n) col.setT(l, n, qmix[l]);
        } else {
            k = k - 1;
            const double emr = __ddiv_rn(__dadd_rn(em, -eneed), em);
            empe = __dmul_rn(empe, emr);
            emke = __dmul_rn(__dmul_rn(emke, emr), a.mlddecd[k]);
            em = __dadd_rn(empe, emke);
            rhou = ec.ieos != 0 ? eos_rn(ec, tmix, smix, zw[k]) : rhomix;
            const double r = ml_rdzg(zw, maxk, k), g = ml_dzg(zw, maxk, k + 1);
            tmix = __dmul_rn(r, __dadd_rn(__dmul_rn(tmix, g), __dmul_rn(col.T(0, k), dz[k])));
            smix = __dmul_rn(r, __dadd_rn(__dmul_rn(smix, g), __dmul_rn(col.T(1, k), dz[k])));
            rhol = eos_rn(ec, col.T(0, k), col.T(1, k), zw[k]);
            rhomix = eos_rn(ec, tmix, smix, zw[k]);
            eneed = __dadd_rn(__dadd_rn(__dmul_rn(ml_z2dzg(zw, maxk, k + 1), rhou), __dmul_rn(ml_z2dzg(zw, k, k), rhol)),
                              -__dmul_rn(ml_z2dzg(zw, maxk, k), rhomix));
        }
    }
    if (partmix == 1 && em > 0) {
        *mldk = k;
        const double mlda = __ddiv_rn(__dmul_rn(__dmul_rn(ml_dzg(zw, maxk, k + 1), ml_rdzg(zw, maxk, k)), em), eneed);
        const double mldb = __dmul_rn(__dadd_rn(__dmul_rn(ml_dzg(zw, maxk, k), ml_rdzg(zw, maxk, k + 1)), -1.0), mlda);
        for (int l = 0; l < L; ++l) {
            const double below = col.T(l, k);
            const double surf = __dadd_rn(__dmul_rn(__dadd_rn(1.0, -mldb), qmix[l]), __dmul_rn(mldb, below));
            col.setT(l, maxk, surf);
            for (int n = k + 1; n <= maxk - 1; ++n) col.setT(l, n, surf);
            col.setT(l, k, __dadd_rn(__dmul_rn(mlda, qmix[l]), __dmul_rn(__dadd_rn(1.0, -mlda), below)));
        }
        *mld = k < maxk ? __dadd_rn(zw[k], __ddiv_rn(em, __dmul_rn(zw[k], __dadd_rn(rhol, -rhou)))) : 0.0;
    } else if (partmix == 1 && k < maxk) {
        *mldk = k + 1;
        *mld = zw[k];
    }
}

// The mixed-layer part of tstepo after co (goldstein.f90:2336-2389) on one wet column: the
// potential energy co released (rold: the densities before co, levels 1..maxk), the wind
// energy, then krausturner or the shallow-layer diagnostic.
template <class Col>
__device__ void mixed_layer_rn(Col &col, const EosCoef &ec, int maxk, int L, int k1, const MixedLayerArgs &a,
                               const double *rold, double *mld, int32_t *mldk)
{
    double peconv = 0.0;
    for (int k = maxk; k > 0; --k) {
        const double rnew = eos_rn(ec, col.T(0, k), col.T(1, k), a.zro[k]);
        peconv = __dadd_rn(peconv, __dmul_rn(__dadd_rn(rnew, -rold[k]), ml_z2dzg(a.zw, k, k)));
    }
    double pebuoy = __dadd_rn(peconv, a.pe1);
    if (pebuoy > 0.0) pebuoy = __dmul_rn(pebuoy, a.mldpebuoycoeff);
    const double emix = __dadd_rn(pebuoy, __dmul_rn(a.ketau, a.mlddec[maxk]));
    if (emix > 0.0) {
        kraus_turner_rn(col, ec, maxk, L, k1, a, pebuoy, mld, mldk);
    } else {
        *mldk = maxk;
        *mld = a.pe1 < 0 ? __dmul_rn(a.zw[maxk - 1], __dadd_rn(1.0, -__ddiv_rn(emix, a.pe1))) : a.zw[maxk - 1];
    }
}

}  // namespace gbgo
