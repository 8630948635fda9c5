// FP32-flux / FP64-state GOLDSTEIN tracer step for sm_103a (batched).
//
// The arithmetic of src/goldstein/goldstein.f90:2436-2642 (tstepo_flux) is
// rewritten per face as a linear transfer G = A*T_neighbour + B*T_centre with
// tracer-independent coefficients (upstream weights, masks and the metric
// factors dt*area folded in, built once per velocity field in FP64 and kept as
// an FP32 pair hi+lo); the isoneutral term of the vertical face
// (goldstein.f90:2561-2624) becomes a 10-point stencil whose coefficients are
// built per cell and step in FP64 from the FP64 state.
//
// Two precision classes share the launch:
//  * T and S (l = 1, 2), the tracers that decide convection through the
//    equation of state, use double-float (FP32 pair) transfers on the FP32
//    pipe, ~1e-14 relative, so convective decisions follow the FP64 reference;
//  * every other tracer uses FP32 transfers on values scaled by a per-tracer
//    power of two, rounded once to int32 (F2I).  The SAME integer is taken from
//    one cell and given to the other, so the budget telescopes exactly.
// The FP64 state is then updated with one FMA per tracer-cell.  FP64 <-> FP32
// and int -> FP64 conversions use integer bit operations: GB300's FP64 pipe
// (and its hardware conversions) run at ~2 ops/clk/SM.
//
// Convective adjustment (goldstein.f90:2657-2841) runs in exact FP64 on columns
// that an FP32 density prescreen cannot prove statically stable.
//
// Mapping: persistent CTAs of 128 threads take work items (member, patch) from
// a counter.  A patch is a rectangle of water columns with the ring of wet
// neighbour columns around it, its columns sorted by k1 so that the wet cells
// of each level form a prefix (land and the cells below the sea floor are never
// loaded).  Per level, a memory phase with tracers innermost (coalesced FP64
// loads and stores) converts and updates, and a compute phase with one thread
// per column forms the transfers.
#include "gb_fp32.h"
#include "co_column.cuh"
#include "../../include/gb_goldstein.h"

#include <cuda_runtime.h>
#include <mutex>
#include <vector>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

namespace gbgo {

// The last CUDA error this file's checks saw in this thread (for the callers' messages).
static thread_local cudaError_t tl_cuda_error = cudaSuccess;

static int launch_status()
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) tl_cuda_error = e;
    return e == cudaSuccess ? 0 : GB_GO_ECUDA;
}

const char *fp32_cuda_error_string() { return cudaGetErrorString(tl_cuda_error); }

// ---------------------------------------------------------------------------
// bit-level conversions (exact, integer pipe)

// x * 2^s truncated to FP32; |x*2^s| below the FP32 normal range gives 0.
__device__ __forceinline__ float d2f_scaled(double x, int s)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned a = hi & 0x7fffffffu;
    unsigned f = __funnelshift_l(lo, a, 3) - ((unsigned)(896 - s) << 23);
    f = (a < ((unsigned)(897 - s) << 20)) ? 0u : f;
    return __uint_as_float(f | (hi & 0x80000000u));
}

// d2f_scaled(x - f2d_scaled(d2f_scaled(x, s), s), s) by integer operations: the FP32
// truncation of the 29 mantissa bits that d2f_scaled drops, scaled by 2^s (0 below the
// FP32 normal range, like d2f_scaled).  No FP64 instruction.
__device__ __forceinline__ float d2f_lo_scaled(double x, int s)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned r = lo & 0x1fffffffu;
    const unsigned fb = __float_as_uint(__uint2float_rz(r));   // the top 24 bits of r, exactly
    const int k = (int)((hi & 0x7fffffffu) >> 20) - 1075 + s;  // r counts units of 2^(E-1075)
    const bool zero = r == 0u || (int)(fb >> 23) + k < 1;
    return __uint_as_float(zero ? 0u : ((fb + ((unsigned)k << 23)) | (hi & 0x80000000u)));
}

// (double)f * 2^-s exactly (FP32 zero and subnormals give 0)
__device__ __forceinline__ double f2d_scaled(float f, int s)
{
    const unsigned b = __float_as_uint(f);
    const unsigned a = b & 0x7fffffffu;
    const unsigned hi = (b & 0x80000000u) | ((a >> 3) + ((unsigned)(896 - s) << 20));
    const unsigned lo = a << 29;
    const double r = __hiloint2double((int)hi, (int)lo);
    return a < 0x00800000u ? 0.0 : r;
}

// (double)q * 2^-s exactly
__device__ __forceinline__ double i2d_scaled(int q, int s)
{
    const unsigned a = q < 0 ? 0u - (unsigned)q : (unsigned)q;
    const int lz = __clz(a);
    const unsigned m = (a << lz) << 1;
    const unsigned hi = ((unsigned)q & 0x80000000u) | ((unsigned)(1023 + 31 - lz - s) << 20) | (m >> 12);
    const unsigned lo = m << 20;
    const double r = __hiloint2double((int)hi, (int)lo);
    return q == 0 ? 0.0 : r;
}

// ---------------------------------------------------------------------------
// double-float (unevaluated FP32 pair) arithmetic

struct dflt {
    float hi, lo;
};

__device__ __forceinline__ dflt df_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ dflt df_fast(float a, float b)
{
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ dflt df_add(dflt a, dflt b)
{
    const dflt s = df_two_sum(a.hi, b.hi);
    return df_fast(s.hi, (a.lo + b.lo) + s.lo);
}

__device__ __forceinline__ dflt df_sub(dflt a, dflt b) { return df_add(a, dflt{-b.hi, -b.lo}); }

// A*X + B*Y
__device__ __forceinline__ dflt df_dot2(dflt A, dflt X, dflt B, dflt Y)
{
    const float p1 = A.hi * X.hi, p2 = B.hi * Y.hi;
    const float e1 = fmaf(A.hi, X.hi, -p1), e2 = fmaf(B.hi, Y.hi, -p2);
    const dflt s = df_two_sum(p1, p2);
    const float t = fmaf(A.hi, X.lo, fmaf(A.lo, X.hi, fmaf(B.hi, Y.lo, B.lo * Y.hi)));
    return df_fast(s.hi, ((e1 + e2) + t) + s.lo);
}

// rint(tr * (dh + dl)) for an FP32 offset tr and an FP32 pair (dh, dl): the product's hi part
// and its exact remainder (FMA), rounded to an integer in two parts, within 1 of the exact value
__device__ __forceinline__ int offset_transfer(float tr, float dh, float dl)
{
    const float p = __fmul_rn(tr, dh);
    const float e = __fmaf_rn(tr, dh, -p);
    const int qi = __float2int_rn(p);
    const float r = __fadd_rn(__fsub_rn(p, __int2float_rn(qi)), __fadd_rn(e, __fmul_rn(tr, dl)));
    return qi + __float2int_rn(r);
}

// FP64 value as a double-float (hi truncated, lo the rest)
__device__ __forceinline__ dflt df_split(double x)
{
    const float h = d2f_scaled(x, 0);
    return {h, d2f_lo_scaled(x, 0)};
}


// column view used by the exact co: the group-planar FP64 state at and above k1,
// the uploaded (Fortran-layout) state below
struct Fp32Col {
    double *w;
    const double *stat;
    int L, NI, NJ, nk, i, j, k1;
    int pofs[kFp32MaxL];   // per tracer: plane * NIJK + q (l = g0 + q)
    int gpl[kFp32MaxL];    // per tracer: gp of its group
    double rho[kMaxK + 1];
    __device__ void init_planes()
    {
        NIJK = (size_t)NI * NJ * (size_t)(nk);
        const int ng = fp32_ngroups(L);
        for (int g = 0; g < ng; ++g) {
            int g0, gl, gp, pl;
            fp32_plane(L, g, &g0, &gl, &gp, &pl);
            for (int q = 0; q < gl; ++q) {
                pofs[g0 + q] = pl;
                gpl[g0 + q] = gp * 64 + q;
            }
        }
    }
    __device__ size_t widx(int l, int lev, size_t NIJK) const
    {
        const size_t cell = (size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * (size_t)lev);
        return (size_t)pofs[l] * NIJK + cell * (size_t)(gpl[l] >> 6) + (size_t)(gpl[l] & 63);
    }
    size_t NIJK;
    __device__ size_t sidx(int l, int lev) const
    {
        return (size_t)l + (size_t)L * ((size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * (size_t)lev));
    }
    __device__ double T(int l, int lev) const { return lev >= k1 ? w[widx(l, lev, NIJK)] : stat[sidx(l, lev)]; }
    __device__ void setT(int l, int lev, double v) { w[widx(l, lev, NIJK)] = v; }
    __device__ double &R(int lev) { return rho[lev]; }
};

// ---------------------------------------------------------------------------
// the step kernel
//
// A work item is one patch of one member: a rectangle of water columns (periodic
// in i) plus the ring of wet neighbour columns outside it.  Each column of the
// patch (a "slot") belongs to one thread for the whole step: interior slots
// first, then ring slots, each part sorted by k1, so the wet cells of a level are
// two prefixes of the threads (land and cells below the sea floor are never
// touched).  A work item is one tracer group of one patch, marched up in k.  At level k every slot's thread converts its FP64 values
// of level k+1 (loaded one level earlier) into the scaled FP32 slab, starts the
// loads of level k+2, and, after one barrier, each interior thread forms the
// face transfers of level k from the slabs of k and k+1 (the bottom face carried
// in registers) and writes its column's FP64 update.  Three slab buffers make one
// barrier per level enough.  The group of T and S also flags the columns whose FP32
// density profile may be unstable; the adjustment kernels (k_co_warp or k_co_decide and
// k_co_mix, and k_co_serial) then adjust those columns exactly.

// FP32 slab pitch per slot (kGroup tracers + 1: consecutive slots hit distinct banks)
constexpr int kGP = 9;
constexpr int kPatchHdr = 8;
constexpr int kIcolWords = 8;

// Dynamic shared memory for patches of up to P - 1 slots (slot P - 1 stays zero: the
// neighbour of a column next to land).  Byte offsets, 16-byte aligned.
struct Fp32Smem {
    int slab;    // float[3][P][kGP]  scaled FP32 values of three levels
    int slo;     // float[3][P][3]    lo parts of T and S for the same levels
    int total;
};

__host__ __device__ inline Fp32Smem fp32_smem_layout(int P)
{
    Fp32Smem s;
    int o = 0;
    s.slab = o; o += (3 * P * kGP * 4 + 15) & ~15;
    s.slo = o; o += (3 * P * 3 * 4 + 15) & ~15;
    s.total = o;
    return s;
}

__device__ __forceinline__ double ldg_d(const double *p) { return __ldg(p); }

// ISO: the isoneutral branch is compiled in (members with diso); without it the kernel
// needs fewer registers.  TS: the instance for group 0 (T and S); the other instance takes
// the other groups.  A work item is (member, patch table offset, tracer group).
template <bool ISO, bool TS>
__global__ void __launch_bounds__(kFp32Threads, TS ? 4 : 5)
k_step_fp32(const MemberDesc *__restrict__ mds, const int4 *__restrict__ items, int nitems,
            const long long *__restrict__ step_ctr, int rel, int *__restrict__ work, int P,
            int2 *__restrict__ colist, int *__restrict__ cocount, int cocap)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ int s_nki[kMaxK + 2], s_nkr[kMaxK + 2];
    __shared__ int s_scale[kFp32MaxL];
    __shared__ float s_trs[kFp32MaxL];      // tref * 2^scale per tracer (0: no offset)
    __shared__ unsigned int s_gmax[kFp32MaxL];
    __shared__ int s_it;
    const int t = threadIdx.x;
    const int lane = t & 31;
    const long long step = *step_ctr + rel;
    // the counter of the next step is free: this launch runs after the previous one ended
    if (blockIdx.x == 0 && t == 0) work[(step + 1) & 1] = 0;

    const Fp32Smem lay = fp32_smem_layout(P);
    float *slab = reinterpret_cast<float *>(smraw + lay.slab);
    float *slo = reinterpret_cast<float *>(smraw + lay.slo);
    const int zs = P - 1;
    // Slab entries of slots not yet wet, and the zero slot, meet only zero coefficients; they
    // must be finite, so the slabs start at zero (afterwards they only hold converted values).
    for (int e = t; e < 3 * P * kGP; e += blockDim.x) slab[e] = 0.0f;
    for (int e = t; e < 3 * P * 3; e += blockDim.x) slo[e] = 0.0f;

    for (;;) {
        if (t == 0) s_it = atomicAdd(&work[step & 1], 1);
        __syncthreads();
        const int it = s_it;
        __syncthreads();
        if (it >= nitems) break;
        const int4 item = items[it];
        const MemberDesc &md = mds[item.x];
        if (step >= md.stop_step) continue;   // uniform over the CTA
        const int32_t *__restrict__ tab = md.ptab + item.y;
        const int ns = tab[0], ni = tab[1], kstart = tab[2], pidx = tab[3];
        const int maxi = md.maxi, maxj = md.maxj, maxk = md.maxk, L = md.L, NI = md.NI, NJ = md.NJ;
        const int32_t *__restrict__ tgoff = tab + kPatchHdr + 2 * (maxk + 2);
        const int32_t *__restrict__ ticol = tab + ((kPatchHdr + 2 * (maxk + 2) + ns + 3) & ~3);
        // every 4th step of the member's own the per-tracer transfer maxima are gathered
        // to re-target the scales (a member's result does not depend on when it was admitted)
        const bool track = ((step - md.origin) & 3) == 0;
        // the member's first patch clears the diagnostics slot of the next step
        if (pidx == 0 && t == 0) {
            unsigned long long *dn = md.diag + 2 * ((step + 1) & 1);
            dn[0] = 0ull;
            dn[1] = 0ull;
        }
        const int par = (int)((step + md.parity) & 1);
        const double *__restrict__ R = md.buf[par];
        double *__restrict__ W = md.buf[par ^ 1];
        const size_t nij = (size_t)maxi * maxj;
        const double *mk = md.mk;
        const double *mj = md.mj;
        const int mkn = maxk + 2, mjn = maxj + 2;
        for (int l = t; l < L; l += blockDim.x) {
            const int sc = md.scale[l];
            s_scale[l] = sc;
            s_trs[l] = md.tref ? md.tref[l] * __int_as_float((127 + sc) << 23) : 0.0f;
            s_gmax[l] = 0u;
        }
        for (int e = t; e < maxk + 2; e += blockDim.x) {
            s_nki[e] = tab[kPatchHdr + e];
            s_nkr[e] = tab[kPatchHdr + maxk + 2 + e];
        }

        // this thread's slot (t < ns): interior column (t < ni) or ring column
        const bool own = t < ns;
        const bool interior = t < ni;
        const int goffs = own ? __ldg(tgoff + t) : 0;
        int sE = zs, sW = zs, sN = zs, sS = zs, k1c = maxk + 1, i = 1, j = 1;
        int cl0 = 0, cw0 = 0, k1nb = 0;
        if (interior) {
            const int4 w0 = __ldg(reinterpret_cast<const int4 *>(ticol + kIcolWords * t));
            const int4 w1 = __ldg(reinterpret_cast<const int4 *>(ticol + kIcolWords * t + 4));
            auto sl16 = [&](int v) { v &= 0xffff; return v == 0xffff ? zs : v; };
            sE = sl16(w0.x >> 16);
            sW = sl16(w0.y);
            sN = sl16(w0.y >> 16);
            sS = sl16(w0.z);
            k1c = (w0.z >> 16) & 0xffff;
            cl0 = w0.w;
            i = w1.x & 0xffff;
            j = (w1.x >> 16) & 0xffff;
            k1nb = w1.y;
            cw0 = w1.z;
        }
        // first level at which this slot is wet (ring slots: their k1, from the prefix tables)
        __syncthreads();
        int kown = maxk + 1;
        if (own) {
            if (interior) kown = k1c;
            else
                for (int k = kstart; k <= maxk; ++k)
                    if (t - ni < s_nkr[k]) {
                        kown = k;
                        break;
                    }
        }

        float rho_prev = 0.0f, mag_prev = 0.0f;
        float ecf[4];
        for (int n = 0; n < 4; ++n) ecf[n] = (float)md.ec[n];
        bool unstable = false;
        float gmax = 0.0f;
        unsigned hmax = 0u;

        {
            int g0, gl, gp, plane;
            fp32_plane(L, item.z, &g0, &gl, &gp, &plane);
            constexpr bool ts_group = TS;
            const long long NIJK = (long long)NI * NJ * (maxk + 2), NIJ = (long long)NI * NJ;
            const double *__restrict__ Rg = R + NIJK * plane;
            double *__restrict__ Wg = W + NIJK * plane;
            int scl[kGroup];
#pragma unroll
            for (int q = 0; q < kGroup; ++q) scl[q] = q < gl ? s_scale[g0 + q] : 0;

            double xr[kGroup];
            // this slot's FP64 values of level lev (if wet there) into xr
            auto load_level = [&](int lev) {
                if (lev >= kown) {
                    const double2 *p = reinterpret_cast<const double2 *>(Rg + ((long long)goffs + NIJ * lev) * gp);
#pragma unroll
                    for (int m = 0; m < kGroup / 2; ++m)
                        if (2 * m < gl) {
                            const double2 v = __ldg(p + m);
                            xr[2 * m] = v.x;
                            xr[2 * m + 1] = v.y;
                        }
                }
            };
            // xr (level lev) -> this slot's scaled FP32 slab entries of lev (and lo of T and S)
            auto convert_level = [&](int lev, int buf) {
                if (lev >= kown) {
                    float *F = slab + (buf * P + t) * kGP;
#pragma unroll
                    for (int q = 0; q < kGroup; ++q) {
                        if (q >= gl) continue;
                        float h = d2f_scaled(xr[q], scl[q]);
                        if (!ts_group) {
                            // offset tracers: T - tref to FP32 from the leading 24 and the next 24 bits
                            const float tr = s_trs[g0 + q];
                            if (tr != 0.0f) h = __fadd_rn(__fsub_rn(h, tr), d2f_lo_scaled(xr[q], scl[q]));
                        }
                        F[q] = h;
                        if (ts_group && q < 2) slo[(buf * P + t) * 3 + q] = d2f_lo_scaled(xr[q], scl[q]);
                    }
                }
            };

            int carry[kGroup];
#pragma unroll
            for (int q = 0; q < kGroup; ++q) carry[q] = 0;
            dflt carryT[2] = {{0.f, 0.f}, {0.f, 0.f}};

            // prologue: level kstart in the slab, kstart+1 in registers
            int bk = kstart % 3;
            load_level(kstart);
            convert_level(kstart, bk);
            if (kstart + 1 <= maxk) load_level(kstart + 1);

            for (int k = kstart; k <= maxk; ++k) {
                const int bk1 = bk == 2 ? 0 : bk + 1;
                // ---- this slot: convert level k+1, start the loads of k+2
                if (k + 1 <= maxk) {
                    convert_level(k + 1, bk1);
                    if (k + 2 <= maxk) load_level(k + 2);
                }
                const bool act = interior && k >= k1c;
                // coefficients of level k, loaded before the barrier (used after it)
                const size_t cl = (size_t)cl0 + nij * (size_t)(k - 1);
                const float *cf = md.coef + 8 * cl;
                const float *cfl = md.coefl + 8 * cl;
                const size_t cwi = 8 * ((size_t)cw0 + nij * (size_t)(k - 1));
                float4 a4 = make_float4(0.f, 0.f, 0.f, 0.f), l4 = a4, a2 = a4;
                float2 w2 = make_float2(0.f, 0.f), s2 = w2, l2 = w2, lw = w2, ls = w2;
                double rv = 0.0;
                auto load_coef = [&]() {
                    a4 = __ldg(reinterpret_cast<const float4 *>(cf));        // Ae Be An Bn
                    a2 = __ldg(reinterpret_cast<const float4 *>(cf + 4));    // Aa Ba Dh Dl
                    w2 = __ldg(reinterpret_cast<const float2 *>(md.coef + cwi));   // Ae Be of the west cell
                    if (j > 1) s2 = __ldg(reinterpret_cast<const float2 *>(cf - 8 * (size_t)maxi + 2));  // An Bn south
                    rv = __ldg(md.rvol + (size_t)(j - 1) + (size_t)maxj * (size_t)(k - 1));
                    if (ts_group) {
                        // lo parts of the coefficients (T and S use the FP32 pairs)
                        l4 = __ldg(reinterpret_cast<const float4 *>(cfl));      // lo Ae Be An Bn
                        l2 = __ldg(reinterpret_cast<const float2 *>(cfl + 4));  // lo Aa Ba
                        lw = __ldg(reinterpret_cast<const float2 *>(md.coefl + cwi));
                        if (j > 1) ls = __ldg(reinterpret_cast<const float2 *>(cfl - 8 * (size_t)maxi + 2));
                    }
                };
                if (act) load_coef();
                __syncthreads();
                // ---- interior column wet at k: transfers of level k and the FP64 update
                if (act) {
                    const double2 *Rk = reinterpret_cast<const double2 *>(Rg + ((long long)goffs + NIJ * k) * gp);
                    double2 *Wk = reinterpret_cast<double2 *>(Wg + ((long long)goffs + NIJ * k) * gp);
                    const bool top = (k == maxk);
                    const float *gt = md.gtop + (size_t)(L + 2) * (size_t)cl0;
                    const float *Fk = slab + bk * P * kGP;
                    const float *Fu = slab + bk1 * P * kGP;
                    const float *pC = Fk + t * kGP, *pE = Fk + sE * kGP, *pW = Fk + sW * kGP;
                    const float *pN = Fk + sN * kGP, *pS = Fk + sS * kGP, *pU = Fu + t * kGP;
                    const int sC = t;

                    // top-face stencil: C1*T(k+1) + C0*T(k) (+ isoneutral terms)
                    bool iso = false;
                    dflt C1X = {a2.x, 0.f}, C0X = {a2.y, 0.f};
                    dflt W0X = {0.f, 0.f}, E0X = {0.f, 0.f}, S0X = {0.f, 0.f}, N0X = {0.f, 0.f};
                    dflt W1X = {0.f, 0.f}, E1X = {0.f, 0.f}, S1X = {0.f, 0.f}, N1X = {0.f, 0.f};
                    dflt AeX = {a4.x, 0.f}, BeX = {a4.y, 0.f}, AnX = {a4.z, 0.f}, BnX = {a4.w, 0.f};
                    dflt AwX = {w2.x, 0.f}, BwX = {w2.y, 0.f}, AsX = {s2.x, 0.f}, BsX = {s2.y, 0.f};
                    if (ts_group) {
                        C1X.lo = l2.x; C0X.lo = l2.y;
                        AeX.lo = l4.x; BeX.lo = l4.y; AnX.lo = l4.z; BnX.lo = l4.w;
                        AwX.lo = lw.x; BwX.lo = lw.y; AsX.lo = ls.x; BsX.lo = ls.y;
                    }
                    if (ISO && md.stencil && !top) {
                        // the cell's top-face stencil from this step's prepass (k_stencil_fp32):
                        // C1 C0 W0 E0 S0 N0 W1 E1 S1 N1 as FP32 pairs and the isoneutral flag
                        const float4 *sp = reinterpret_cast<const float4 *>(md.stencil + (size_t)kStencilWords * cl);
                        const float4 h0 = __ldg(sp), h1 = __ldg(sp + 1), h2 = __ldg(sp + 2);
                        C1X = {h0.x, 0.f}; C0X = {h0.y, 0.f}; W0X = {h0.z, 0.f}; E0X = {h0.w, 0.f};
                        S0X = {h1.x, 0.f}; N0X = {h1.y, 0.f}; W1X = {h1.z, 0.f}; E1X = {h1.w, 0.f};
                        S1X = {h2.x, 0.f}; N1X = {h2.y, 0.f};
                        iso = h2.z != 0.f;
                        if (ts_group) {
                            const float4 l0 = __ldg(sp + 3), l1 = __ldg(sp + 4), l2 = __ldg(sp + 5);
                            C1X.lo = l0.x; C0X.lo = l0.y; W0X.lo = l0.z; E0X.lo = l0.w;
                            S0X.lo = l1.x; N0X.lo = l1.y; W1X.lo = l1.z; E1X.lo = l1.w;
                            S1X.lo = l2.x; N1X.lo = l2.y;
                        }
                    }
                    const float *pUE = Fu + sE * kGP, *pUW = Fu + sW * kGP, *pUN = Fu + sN * kGP, *pUS = Fu + sS * kGP;
                    const unsigned amask = __activemask();
                    if (ts_group) {
                        // T and S: double-float transfers, FP64 update
                        const float *Lk = slo + bk * P * 3, *Lu = slo + bk1 * P * 3;
                        double tn[2];
                        const double2 ts_old = __ldg(Rk);
#pragma unroll
                        for (int l = 0; l < 2; ++l) {
                            const double told = l ? ts_old.y : ts_old.x;
                            const dflt Tc = {pC[l], Lk[sC * 3 + l]};
                            const int sl = scl[l];
                            // sum = (Gw - Ge) + (Gs - Gn) + (Gb - Ga), faces formed as needed
                            dflt sum;
                            {
                                const dflt TE = {pE[l], Lk[sE * 3 + l]}, TW = {pW[l], Lk[sW * 3 + l]};
                                sum = df_sub(df_dot2(AwX, Tc, BwX, TW), df_dot2(AeX, TE, BeX, Tc));
                            }
                            {
                                const dflt TN = {pN[l], Lk[sN * 3 + l]}, TS = {pS[l], Lk[sS * 3 + l]};
                                sum = df_add(sum, df_sub(df_dot2(AsX, Tc, BsX, TS), df_dot2(AnX, TN, BnX, Tc)));
                            }
                            dflt Ga;
                            if (top) {
                                const float sc = __int_as_float((127 + sl) << 23);
                                Ga = {__ldg(gt + l) * sc, __ldg(gt + L + l) * sc};
                            } else {
                                Ga = df_dot2(C1X, dflt{pU[l], Lu[sC * 3 + l]}, C0X, Tc);
                                if (ISO && iso) {
                                    const dflt TE = {pE[l], Lk[sE * 3 + l]}, TW = {pW[l], Lk[sW * 3 + l]};
                                    const dflt TN = {pN[l], Lk[sN * 3 + l]}, TS = {pS[l], Lk[sS * 3 + l]};
                                    Ga = df_add(Ga, df_dot2(W0X, TW, E0X, TE));
                                    Ga = df_add(Ga, df_dot2(S0X, TS, N0X, TN));
                                    Ga = df_add(Ga, df_dot2(W1X, dflt{pUW[l], Lu[sW * 3 + l]}, E1X, dflt{pUE[l], Lu[sE * 3 + l]}));
                                    Ga = df_add(Ga, df_dot2(S1X, dflt{pUS[l], Lu[sS * 3 + l]}, N1X, dflt{pUN[l], Lu[sN * 3 + l]}));
                                }
                            }
                            sum = df_add(sum, df_sub(carryT[l], Ga));
                            carryT[l] = Ga;
                            const double dlt = f2d_scaled(sum.hi, sl) + f2d_scaled(sum.lo, sl);
                            tn[l] = fma(dlt, rv, told);
                            hmax = max(hmax, (unsigned)__double2hiint(tn[l]) & 0x7fffffffu);
                        }
                        *Wk = make_double2(tn[0], tn[1]);
                        // FP32 density prescreen: a column joins the adjustment unless its densities
                        // decrease upwards by clearly more than their FP32 error at every level
                        // (the test of co, goldstein.f90:2715-2716, is then certainly passed); levels
                        // that co mixed are equal and always join (with ieos != 0 or iconv = 1 every
                        // column joins)
                        const float tf = d2f_scaled(tn[0], 0), sf = d2f_scaled(tn[1], 0);
                        const float e0 = ecf[0] * tf, e1 = ecf[1] * sf, e2 = ecf[2] * (tf * tf), e3 = ecf[3] * (tf * tf * tf);
                        const float rf = ((e0 + e1) + e2) + e3;
                        const float mag = fabsf(e0) + fabsf(e1) + fabsf(e2) + fabsf(e3);
                        if (k > k1c && !(rho_prev - rf > 2.0e-6f * (mag + mag_prev) + 1.0e-30f)) unstable = true;
                        rho_prev = rf;
                        mag_prev = mag;
                    }
                    // other tracers: FP32 transfers rounded once to int32, FP64 update
                    const float Ae = AeX.hi, Be = BeX.hi, An = AnX.hi, Bn = BnX.hi, Aw = AwX.hi, Bw = BwX.hi;
                    const float As = AsX.hi, Bs = BsX.hi;
                    const float cC0 = C0X.hi, cC1 = C1X.hi, cW0 = W0X.hi, cE0 = E0X.hi, cS0 = S0X.hi, cN0 = N0X.hi;
                    const float cW1 = W1X.hi, cE1 = E1X.hi, cS1 = S1X.hi, cN1 = N1X.hi;
                    double2 told2 = make_double2(0.0, 0.0);
                    double tlast = 0.0;
#pragma unroll
                    for (int q = 0; q < kGroup; ++q) {
                        if (ts_group || q >= gl) continue;
                        if ((q & 1) == 0) told2 = __ldg(Rk + q / 2);
                        const double told = (q & 1) ? told2.y : told2.x;
                        const float Tc = pC[q], TE = pE[q], TW = pW[q], TN = pN[q], TS = pS[q];
                        const float ge = fmaf(Ae, TE, Be * Tc);
                        const float gw = fmaf(Aw, Tc, Bw * TW);
                        const float gn = fmaf(An, TN, Bn * Tc);
                        const float gs = fmaf(As, Tc, Bs * TS);
                        float ga;
                        if (top) {
                            ga = __ldg(gt + g0 + q) * __int_as_float((127 + scl[q]) << 23);
                        } else {
                            ga = fmaf(cC1, pU[q], cC0 * Tc);
                            if (ISO && iso) {
                                ga = fmaf(cW0, TW, ga);
                                ga = fmaf(cE0, TE, ga);
                                ga = fmaf(cS0, TS, ga);
                                ga = fmaf(cN0, TN, ga);
                                ga = fmaf(cW1, pUW[q], ga);
                                ga = fmaf(cE1, pUE[q], ga);
                                ga = fmaf(cS1, pUS[q], ga);
                                ga = fmaf(cN1, pUN[q], ga);
                            }
                        }
                        if (track) {
                            // per-tracer maximum for the scale of later steps (the faces and the
                            // offset's share tref * D): one shared atomic per warp; also the int32
                            // range check
                            const float gm = fmaxf(fmaxf(fmaxf(fabsf(ge), fabsf(gw)), fmaxf(fmaxf(fabsf(gn), fabsf(gs)), fabsf(ga))),
                                                   a2.z != 0.0f ? fabsf(__fmul_rn(s_trs[g0 + q], a2.z)) : 0.0f);
                            gmax = fmaxf(gmax, gm);
                            const unsigned wmax = __reduce_max_sync(amask, __float_as_uint(gm));
                            if (lane == __ffs(amask) - 1) atomicMax(&s_gmax[g0 + q], wmax);
                        }
                        const int qe = __float2int_rn(ge), qw = __float2int_rn(gw);
                        const int qn = __float2int_rn(gn), qs = __float2int_rn(gs);
                        const int qa = __float2int_rn(ga);
                        int sum = (qw - qe) + (qs - qn) + (carry[q] - qa);
                        if (a2.z != 0.0f) {
                            // the offset's share tref * D of a cell whose faces do not cancel
                            const float tr = s_trs[g0 + q];
                            if (tr != 0.0f) sum += offset_transfer(tr, a2.z, a2.w);
                        }
                        carry[q] = qa;
                        const double tnew = fma(i2d_scaled(sum, scl[q]), rv, told);
                        hmax = max(hmax, (unsigned)__double2hiint(tnew) & 0x7fffffffu);
                        // 16-byte stores of pairs (the pad of an odd group is written as zero)
                        if (q & 1) Wk[q / 2] = make_double2(tlast, tnew);
                        else if (q + 1 >= gl) Wk[q / 2] = make_double2(tnew, 0.0);
                        tlast = tnew;
                    }
                }
                bk = bk1;
            }
            // the next item's prologue writes slab buffers the last levels read
            __syncthreads();
        }

        // columns that need the exact convective adjustment (every column with iconv = 1,
        // ieos != 0 or imld = 1) join the step's list: (member, word offset of the column's record)
        if (item.z == 0 && interior && (unstable || md.iconv == 1 || md.ieos != 0 || md.imld != 0)) {
            const int at = atomicAdd(&cocount[step & 1], 1);
            if (at < cocap) colist[at] = make_int2(item.x, (int)(ticol - md.ptab) + kIcolWords * t);
            else atomicOr(md.status, 4u);
        }
        // a scaled transfer above 3.5e8 could overflow the int32 sum of six faces
        const bool nonfinite = hmax >= 0x7ff00000u;
        if (nonfinite || gmax > 3.5e8f) atomicOr(md.status, (nonfinite ? 1u : 0u) | (gmax > 3.5e8f ? 2u : 0u));
        __syncthreads();
        if (track)
            for (int l = 2 + t; l < L; l += blockDim.x)
                if (s_gmax[l]) atomicMax(&md.gmax[l], s_gmax[l]);
    }
}

// After a tracking step: move each tracer's scale so that the step's largest transfer
// would have landed in [2^25, 2^26); clear the maxima.  T and S (double-float) keep theirs.
__global__ void k_rescale(const MemberDesc *__restrict__ mds, int n)
{
    for (int m = blockIdx.x; m < n; m += gridDim.x) {
        const MemberDesc &md = mds[m];
        for (int l = 2 + threadIdx.x; l < md.L; l += blockDim.x) {
            const unsigned gb = md.gmax[l];
            if (gb == 0u) continue;
            const int e = (int)((gb >> 23) & 0xff) - 127;      // floor(log2(max |scaled transfer|))
            int s = md.scale[l] + (25 - e);
            s = s < -120 ? -120 : (s > 120 ? 120 : s);
            md.scale[l] = s;
            md.gmax[l] = 0u;
        }
    }
}

// Top-face stencil of every wet cell below the surface, for the members with the isoneutral
// branch or the local vertical diffusivity, built once per step (both transfer instances read
// it) in FP64 from the step's T and S:
//  * C1, C0: the weights of T(k+1) and T(k) -- the static coefficients, or with iediff 1/2
//    those of the local diffusivity diffv (goldstein.f90:2490-2516, eosd :3064-3082);
//  * with the isoneutral branch (goldstein.f90:2561-2624) the slope-tapered terms, which add
//    to C1, C0 and give the weights of T at the W, E, S, N neighbours of levels k and k+1.
// The density differences scc*dS - tec*dT cancel strongly in weakly stratified water, so they
// are taken as differences of D = ec(2)*S - tec*T with the cell's tec (goldstein.f90:2587-2588).
// One block row per listed member (blockIdx.y); also the diagnostics dmax and limps.
__global__ void __launch_bounds__(256) k_stencil_fp32(const MemberDesc *__restrict__ mds, const int *__restrict__ list,
                                                      const long long *__restrict__ step_ctr, int rel)
{
    const long long step = *step_ctr + rel;
    const MemberDesc &md = mds[list[blockIdx.y]];
    if (step >= md.stop_step) return;
    const int maxi = md.maxi, maxj = md.maxj, maxk = md.maxk, NI = md.NI, NJ = md.NJ;
    const int mkn = maxk + 2, mjn = maxj + 2;
    const double *mk = md.mk, *mj = md.mj;
    const double *R = md.buf[(int)((step + md.parity) & 1)];
    auto ld = [&](int ii, int jj, int kk, int l) {
        return ldg_d(R + 2 * ((size_t)ii + (size_t)NI * ((size_t)jj + (size_t)NJ * (size_t)kk)) + l);
    };
    double dmax_l = 0.0;
    unsigned limps_l = 0;
    const size_t nij = (size_t)maxi * maxj, ncell = nij * (size_t)(maxk - 1);
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % maxi) + 1, j = (int)((c / maxi) % maxj) + 1, k = (int)(c / nij) + 1;
        if (k < md.k1[i + NI * j]) continue;
        double c1 = (double)__ldg(md.coef + 8 * c + 4) + (double)__ldg(md.coefl + 8 * c + 4);
        double c0 = (double)__ldg(md.coef + 8 * c + 5) + (double)__ldg(md.coefl + 8 * c + 5);
        double w[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // W0 E0 S0 N0 W1 E1 S1 N1
        bool iso = false;
        const double t1 = ld(i, j, k, 0), t2 = ld(i, j, k + 1, 0);
        const double s1 = ld(i, j, k, 1), s2 = ld(i, j, k + 1, 1);
        const double tatw = 0.5 * (t1 + t2);
        double tec = -md.ec[0] - md.ec[2] * tatw * 2.0 - md.ec[3] * tatw * tatw * 3.0;
        if (md.ieos) tec = tec - md.ec[4] * mk[2 * mkn + k];
        const double rdza = mk[4 * mkn + k];
        if (md.iediff) {
            const double dzrho = (md.ec[1] * (s2 - s1) - tec * (t2 - t1)) * rdza;
            const double rdzrho = dzrho < -1.0e-12 ? 1.0 / dzrho : -1.0e12;
            const double e1 = md.ediff1[(size_t)(i - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (size_t)(k - 1))];
            double diffv;
            if (md.ediffpow2i == 0) diffv = md.ediff0 + e1;
            else if (md.ediffpow2i == 1) diffv = md.ediff0 + e1 * (-rdzrho);
            else if (md.ediffpow2i == 2) diffv = md.ediff0 + e1 * sqrt(-rdzrho);
            else diffv = md.ediff0 + e1 * pow(-rdzrho, md.ediffpow2);
            if (diffv > md.diffmax[k + 1]) diffv = md.diffmax[k + 1];
            const double u3 = md.u[2 + 3 * ((size_t)i + (size_t)(maxi + 1) * ((size_t)j + (size_t)(maxj + 1) * (size_t)(k - 1)))];
            const double pec = u3 * md.dza[k] / diffv, ups = pec / (2.0 + fabs(pec));
            const double g = mj[2 * mjn + j];   // dt*dphi*ds(j)
            c1 = g * (u3 * (1.0 - ups) * 0.5 - rdza * diffv);
            c0 = g * (u3 * (1.0 + ups) * 0.5 + rdza * diffv);
        }
        if (md.diso) {
            const double scc = md.ec[1];
            const double Dc0 = scc * s1 - tec * t1, Dc1 = scc * s2 - tec * t2;
            const double dzrho = (Dc1 - Dc0) * rdza;
            if (dzrho < -1.0e-12) {
                iso = true;
                const double rdzrho = 1.0 / dzrho;
                const double rcr = mj[j];                                 // rc(j)*rdphi
                const double cvs = mj[mjn + j - 1], cvn = mj[mjn + j];   // cv*rdsv at j-1, j
                const int im = (i == 1) ? maxi : i - 1, ip = (i == maxi) ? 1 : i + 1;
                const int k1E = md.k1[ip + NI * j], k1W = md.k1[im + NI * j];
                const int k1N = md.k1[i + NI * (j + 1)], k1S = md.k1[i + NI * (j - 1)];
                double dxr[4], dyr[4], mx[4], my[4];
                double tv1 = 0.0;
#pragma unroll
                for (int knp = 0; knp <= 1; ++knp) {
                    const double Dck = knp ? Dc1 : Dc0;
#pragma unroll
                    for (int nnp = 0; nnp <= 1; ++nnp) {
                        const int ina = nnp + 2 * knp;
                        const int kk = k + knp;
                        const bool okx = kk >= (nnp ? k1E : k1W);
                        const bool oky = kk >= (nnp ? k1N : k1S);
                        mx[ina] = okx ? rcr : 0.0;
                        my[ina] = oky ? (nnp ? cvn : cvs) : 0.0;
                        dxr[ina] = 0.0;
                        dyr[ina] = 0.0;
                        if (okx) {
                            const int ii = nnp ? ip : im;
                            const double Dn = scc * ld(ii, j, kk, 1) - tec * ld(ii, j, kk, 0);
                            dxr[ina] = (nnp ? Dn - Dck : Dck - Dn) * rcr;
                        }
                        if (oky) {
                            const int jj = nnp ? j + 1 : j - 1;
                            const double Dn = scc * ld(i, jj, kk, 1) - tec * ld(i, jj, kk, 0);
                            dyr[ina] = (nnp ? Dn - Dck : Dck - Dn) * my[ina];
                        }
                        tv1 += dxr[ina] * dxr[ina] + dyr[ina] * dyr[ina];
                    }
                }
                const double sum2 = tv1;
                tv1 = 0.25 * tv1 * rdzrho * rdzrho;
                const double ss = mk[5 * mkn + k];
                double slim = 1.0;
                if (tv1 > ss) {
                    slim = ss * ss / (tv1 * tv1);
                    limps_l += 1;
                }
                dmax_l = fmax(dmax_l, tv1 * slim * md.diff1 * rdza * md.dt * rdza);
                // G_iso = dt*dphi*ds * 0.25*slim*diff1/dzrho^2 * sum_ina[...]
                const double cc = mj[2 * mjn + j] * 0.25 * slim * md.diff1 * rdzrho * rdzrho;
                const double two_dz = 2.0 * dzrho * cc;
                double wx[4], wy[4];
#pragma unroll
                for (int n = 0; n < 4; ++n) {
                    wx[n] = two_dz * dxr[n] * mx[n];
                    wy[n] = two_dz * dyr[n] * my[n];
                }
                const double wz = -cc * sum2 * rdza;      // dzts = (T(k+1)-T(k))*rdza
                c0 = c0 + ((wx[0] - wx[1]) + (wy[0] - wy[1]) - wz);
                c1 = c1 + ((wx[2] - wx[3]) + (wy[2] - wy[3]) + wz);
                w[0] = -wx[0]; w[1] = wx[1]; w[2] = -wy[0]; w[3] = wy[1];
                w[4] = -wx[2]; w[5] = wx[3]; w[6] = -wy[2]; w[7] = wy[3];
            }
        }
        const double v[10] = {c1, c0, w[0], w[1], w[2], w[3], w[4], w[5], w[6], w[7]};
        float hi[12], lo[12];
#pragma unroll
        for (int n = 0; n < 10; ++n) {
            const dflt x = df_split(v[n]);
            hi[n] = x.hi;
            lo[n] = x.lo;
        }
        hi[10] = iso ? 1.f : 0.f;
        hi[11] = lo[10] = lo[11] = 0.f;
        float4 *dst = reinterpret_cast<float4 *>(md.stencil + (size_t)kStencilWords * c);
        dst[0] = make_float4(hi[0], hi[1], hi[2], hi[3]);
        dst[1] = make_float4(hi[4], hi[5], hi[6], hi[7]);
        dst[2] = make_float4(hi[8], hi[9], hi[10], hi[11]);
        dst[3] = make_float4(lo[0], lo[1], lo[2], lo[3]);
        dst[4] = make_float4(lo[4], lo[5], lo[6], lo[7]);
        dst[5] = make_float4(lo[8], lo[9], lo[10], lo[11]);
    }
    if (md.diso) {
        // diagnostics dmax, limps of the step (goldstein.f90:2459, 2598-2608): one atomic per warp
        unsigned long long db = __double_as_longlong(dmax_l);
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ob = __shfl_xor_sync(0xffffffffu, db, o);
            db = ob > db ? ob : db;
            limps_l += __shfl_xor_sync(0xffffffffu, limps_l, o);
        }
        if ((threadIdx.x & 31) == 0) {
            unsigned long long *dg = md.diag + 2 * (step & 1);
            if (db) atomicMax(&dg[0], db);
            if (limps_l) atomicAdd(&dg[1], (unsigned long long)limps_l);
        }
    }
}

int fp32_rescale(const MemberDesc *descs, int n, cudaStream_t s)
{
    if (n <= 0) return 0;
    k_rescale<<<std::min(n, 1024), 32, 0, s>>>(descs, n);
    return launch_status();
}

// Exact convective adjustment (goldstein.f90:2657-2841) of the columns the step listed (those
// its FP32 prescreen cannot prove stable, and every column of members with iconv = 1,
// ieos != 0 or imld = 1), on the FP64 state the step wrote.  A list
// entry is (member, word offset of the column's record).  Columns of members with iconv = 0,
// ieos = 0, imld = 0 and maxk <= 32 take k_co_warp (one warp per column; small batches) or the
// two phases k_co_decide and k_co_mix (large batches; fp32_co_two_phase); the others take
// k_co_serial, one entry per warp, by co_warp (the column staged in shared memory, one lane per
// tracer), with coshuffle (iconv = 1) and the mixed layer on one lane.

// A list entry's column as the adjustment kernels see it.
struct CoCol {
    double *W;             // group-planar FP64 state the step wrote
    const double *dz;      // dz[lev]
    double *cost;          // the column's cost entry
    size_t cell, NIJ, plane;
    int maxk, L, k1;
};

__device__ __forceinline__ CoCol co_col(const MemberDesc &md, int2 ent, long long step)
{
    const int32_t *ticol = md.ptab + ent.y;
    const int i = ticol[4] & 0xffff, j = (ticol[4] >> 16) & 0xffff;
    CoCol c;
    c.W = md.buf[(int)((step + md.parity) & 1) ^ 1];
    c.dz = md.mk;
    c.cost = md.cost + ticol[3];
    c.NIJ = (size_t)md.NI * md.NJ;
    c.cell = (size_t)i + (size_t)md.NI * j;
    c.plane = c.NIJ * (size_t)(md.maxk + 2);
    c.maxk = md.maxk;
    c.L = md.L;
    c.k1 = (ticol[2] >> 16) & 0xffff;
    return c;
}

constexpr int kCoDecideThreads = 32;
constexpr int kCoDecideWarpBytes = 33 * 32 * (8 + 1);   // per warp: double-float density, merge index

// Decisions of co for the columns with maxk <= 32, ieos = 0, iconv = 0, imld = 0: one lane
// per list entry (co_column.cuh).  T and S are adjusted in place and the merges logged in
// colog; a column with merges and L > 2 reserves L - 2 slots of comap (entry, tracer) for
// k_co_mix: from the front (count cocount[2 + (step & 1)]) with at most two merges, else from
// the back (count cocount[4 + (step & 1)]).  Shared memory per warp, [level][lane] for
// levels 0..32: a level's double-float density (on the FP32 pipes: GB300's FP64 pipe takes
// ~15 SM cycles per warp instruction) and the index of the last merge it headed, whose logged
// sum is its thickness (dz otherwise); 9.5 KB per warp, so a step's batches are resident at
// once.  A pair is
// decided by the pair densities when their difference exceeds 2^-39 M, M the largest
// magnitude of the column's eos terms (M is convex in (T, S), so no mixed level exceeds
// it); otherwise equal T and S are equal densities and the rest compare exact FP64 eos
// values (goldstein.f90:3048-3061).  T and S are read and written in place.
__global__ void __launch_bounds__(kCoDecideThreads)
k_co_decide(const MemberDesc *__restrict__ mds, const int2 *__restrict__ colist, int *__restrict__ cocount, int cocap,
            const long long *__restrict__ step_ctr, int rel, unsigned char *__restrict__ colog, int2 *__restrict__ comap,
            int mapcap)
{
    extern __shared__ double cosm[];
    const unsigned F = 0xffffffffu;
    const long long step = *step_ctr + rel;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarp = blockDim.x >> 5;
    const int ncol = min(cocount[step & 1], cocap);
    // slots of columns with at most two merges from the front of comap, the others from the
    // back, so that a warp of k_co_mix replays logs of similar length
    int *nslot = cocount + 2 + (int)(step & 1), *nslotb = cocount + 4 + (int)(step & 1);
    // the lists of the next step start empty (that step's kernels run after this one)
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        cocount[(step + 1) & 1] = 0;
        cocount[2 + ((step + 1) & 1)] = 0;
        cocount[4 + ((step + 1) & 1)] = 0;
    }
    unsigned char *wsm = reinterpret_cast<unsigned char *>(cosm) + (size_t)warp * kCoDecideWarpBytes;
    float2 *dd = reinterpret_cast<float2 *>(wsm) + lane;
    unsigned char *tix = wsm + 33 * 32 * 8 + lane;   // the last merge a level headed, 0xff: none
    for (int base = (blockIdx.x * nwarp + warp) * 32; base < ncol; base += gridDim.x * nwarp * 32) {
        const int e = base + lane;
        bool valid = false;
        const MemberDesc *mdp = nullptr;
        CoCol c{};
        if (e < ncol) {
            const int2 ent = colist[e];
            mdp = mds + ent.x;
            if (fp32_co_fast(mdp->iconv, mdp->ieos, mdp->imld, mdp->maxk)) {
                valid = true;
                c = co_col(*mdp, ent, step);
            }
        }
        // T and S of level l in the state (plane 0: two values per cell)
        double *TS = valid ? c.W + 2 * c.cell : nullptr;
        const size_t tstr = 2 * c.NIJ;
        auto ts_at = [&](int l) -> double2 { return *reinterpret_cast<const double2 *>(TS + (size_t)l * tstr); };
        auto ts_set = [&](int l, double2 v) { *reinterpret_cast<double2 *>(TS + (size_t)l * tstr) = v; };
        CoDf ecd[4];
#pragma unroll
        for (int n = 0; n < 4; ++n) ecd[n] = co_split(valid ? mdp->ec[n] : 0.0);
        const int k1 = valid ? c.k1 : 1, maxk = valid ? c.maxk : 1;
        float mmax = 0.0f;
        if (valid) {
            // levels in blocks of 8, the next block's loads issued before this block's densities
            double2 v[8], vn[8];
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (k1 + u <= maxk) vn[u] = ts_at(k1 + u);
            for (int l0 = k1; l0 <= maxk; l0 += 8) {
#pragma unroll
                for (int u = 0; u < 8; ++u) v[u] = vn[u];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (l0 + 8 + u <= maxk) vn[u] = ts_at(l0 + 8 + u);
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (l0 + u <= maxk) {
                        float mg;
                        const CoDf r = eos_df(ecd, v[u].x, v[u].y, mg);
                        dd[(l0 + u) * 32] = make_float2(r.hi, r.lo);
                        tix[(l0 + u) * 32] = 0xff;
                        mmax = fmaxf(mmax, mg);
                    }
            }
        }
        const float tol = __fmul_rn(0x1p-39f, mmax);   // >= 2^-40 (M_a + M_b)
        // rho(a) < rho(b) for active levels a above b: co's stable pair
        auto stable = [&](int a, int b) -> bool {
            const float2 da = dd[a * 32], db = dd[b * 32];
            const float d = __fadd_rn(__fsub_rn(da.x, db.x), __fsub_rn(da.y, db.y));
            if (d < -tol) return true;
            if (d > tol) return false;
            const double2 va = ts_at(a), vb = ts_at(b);
            // equal T and S: equal densities, not stable
            if (__double_as_longlong(va.x) == __double_as_longlong(vb.x) && __double_as_longlong(va.y) == __double_as_longlong(vb.y))
                return false;
            EosCoef ec;
            for (int n = 0; n < 4; ++n) ec.ec[n] = mdp->ec[n];
            ec.ec[4] = 0.0;
            ec.ieos = 0;
            return order_key(eos_rn(ec, va.x, va.y, 0.0)) < order_key(eos_rn(ec, vb.x, vb.y, 0.0));
        };
        unsigned mask = valid ? co_bits(k1, maxk) : 0u;   // active levels (co's list)
        auto below = [&](int x) -> int {
            const unsigned m = mask & ((1u << (x - 1)) - 1u);
            return m ? 32 - __clz(m) : 0;
        };
        auto above = [&](int x) -> int { return __ffs(mask & ~((1u << x) - 1u)); };
        unsigned char *log = valid ? colog + (size_t)e * kCoLogBytes : nullptr;
        double *ldt = reinterpret_cast<double *>(log + kCoLogDtot), *ly = reinterpret_cast<double *>(log + kCoLogY);
        double *ldp = reinterpret_cast<double *>(log + kCoLogDtop), *ledz = reinterpret_cast<double *>(log + kCoLogEdz);
        int x = maxk, lastmix = 0, nm = 0, ne = 0, guard = 0;
        int xlast = 0;               // level of the last merge, its new T and S and thickness
        double2 tslast = make_double2(0.0, 0.0);
        double dtlast = 0.0;
        // thickness of the stretch level l heads: dz, or the summed thickness of the last merge
        // it headed (the log's, or registers for the latest merge)
        auto dzm_of = [&](int l) -> double {
            if (l == xlast) return dtlast;
            const int k = tix[l * 32];
            return k == 0xff ? c.dz[l] : ldt[k];
        };
        bool done = !valid;
        for (;;) {
            // walk to this column's next merge (levels nl..x), or to the end of co's loop
            bool ready = false;
            int nl = 0;
            while (!done && !ready) {
                if (++guard > 2048) {   // co ends within maxk^2 steps; a longer walk is a fault
                    atomicOr(mdp->status, 4u);
                    done = true;
                    break;
                }
                const int b = below(x);
                if (!(b > 0 || (lastmix != 0 && x != maxk))) {
                    done = true;
                    break;
                }
                if (b <= 0 || stable(x, b)) {
                    x = (lastmix == 0 || x == maxk) ? b : above(x);
                    lastmix = 0;
                    continue;
                }
                nl = b;
                for (;;) {
                    const int bb = below(nl);
                    if (bb <= 0 || stable(nl, bb)) break;
                    nl = bb;
                }
                ready = true;
            }
            if (!__any_sync(F, ready)) break;
            if (ready) {
                // mix T and S of level x, then of the active levels below it down to nl
                const unsigned sm = mask & co_bits(nl, x - 1);
                const double dtop = dzm_of(x);
                // the last merge's level (the next merge's top, usually) is held in registers; the
                // absorbed levels' loads go out before the FP64 chain, one ahead
                const double2 vx = x == xlast ? tslast : ts_at(x);
                int l = sm ? 32 - __clz(sm) : 0;
                double2 vn = l ? ts_at(l) : make_double2(0.0, 0.0);
                double at = __dmul_rn(vx.x, dtop), as = __dmul_rn(vx.y, dtop), dtot = dtop;
                int cnt = 0;
                for (unsigned f = sm; f;) {
                    f &= ~(1u << (l - 1));
                    const double2 vl = vn;
                    const int ln = f ? 32 - __clz(f) : 0;
                    if (ln) vn = ts_at(ln);
                    const double dzl = dzm_of(l);
                    dtot = __dadd_rn(dtot, dzl);
                    at = __dadd_rn(at, __dmul_rn(vl.x, dzl));
                    as = __dadd_rn(as, __dmul_rn(vl.y, dzl));
                    ledz[ne] = dzl;
                    log[kCoLogElev + ne] = (unsigned char)l;
                    ++ne;
                    ++cnt;
                    l = ln;
                }
                const double y = __drcp_rn(dtot);
                const double nt = co_div(at, dtot, y), ns = co_div(as, dtot, y);
                ts_set(x, make_double2(nt, ns));
                xlast = x;
                tslast = make_double2(nt, ns);
                dtlast = dtot;
                tix[x * 32] = (unsigned char)nm;
                float mg;
                const CoDf r = eos_df(ecd, nt, ns, mg);
                dd[x * 32] = make_float2(r.hi, r.lo);
                mask &= ~sm;
                ldt[nm] = dtot;
                ly[nm] = y;
                ldp[nm] = dtop;
                log[kCoLogX + nm] = (unsigned char)x;
                log[kCoLogCnt + nm] = (unsigned char)cnt;
                ++nm;
                lastmix = 1;
            }
        }
        int need = 0;
        if (valid) {
            // fill: every level of [k1, maxk-1] no longer active takes T and S of the lowest
            // active level above it
            const unsigned fillm = ~mask & co_bits(k1, maxk - 1);
            for (unsigned f = fillm; f;) {
                // the filled levels below one active level take its values: one load per group
                const int src = __ffs(mask & ~((1u << __ffs(f)) - 1u));
                const double2 v = src == xlast ? tslast : ts_at(src);
                const unsigned grp = f & ((1u << (src - 1)) - 1u);
                for (unsigned g = grp; g; g &= g - 1u) ts_set(__ffs(g), v);
                f &= ~grp;
            }
            const int filled = __popc(fillm);
            if (filled > 0) *c.cost = add_count_rn(*c.cost, filled);
            *reinterpret_cast<int *>(log) = nm;
            *reinterpret_cast<unsigned *>(log + 4) = mask;
            if (nm > 0) need = c.L - 2;
        }
        // slots of the other tracers: one reservation per warp and class
        const bool back = nm > 2;
#pragma unroll
        for (int cls = 0; cls < 2; ++cls) {
            const int nd = (cls == 1) == back ? need : 0;
            int incl = nd;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(F, incl, o);
                if (lane >= o) incl += v;
            }
            const int tot = __shfl_sync(F, incl, 31);
            int wb = 0;
            if (lane == 31 && tot > 0) wb = atomicAdd(cls ? nslotb : nslot, tot);
            wb = __shfl_sync(F, wb, 31);
            for (int l = 0; l < nd; ++l) {
                const int at = wb + incl - nd + l;
                if (at < mapcap) comap[cls ? mapcap - 1 - at : at] = make_int2(e, l + 2);
                else atomicOr(mdp->status, 4u);
            }
        }
        __syncwarp();
    }
}

constexpr int kCoMixThreads = 256;

// The other tracers of the columns k_co_decide adjusted: one thread per (list entry, tracer)
// slot replays the entry's merge log in place, in co's order and arithmetic
// (goldstein.f90:2732-2746), then the fill (2748-2765).
__global__ void __launch_bounds__(kCoMixThreads)
k_co_mix(const MemberDesc *__restrict__ mds, const int2 *__restrict__ colist, const int *__restrict__ cocount,
         const long long *__restrict__ step_ctr, int rel, const unsigned char *__restrict__ colog,
         const int2 *__restrict__ comap, int mapcap)
{
    const long long step = *step_ctr + rel;
    const int nf = min(cocount[2 + (int)(step & 1)], mapcap), nb = min(cocount[4 + (int)(step & 1)], mapcap - nf);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nf + nb; t += gridDim.x * blockDim.x) {
        const int2 sl = comap[t < nf ? t : mapcap - 1 - (t - nf)];
        const int2 ent = colist[sl.x];
        const CoCol c = co_col(mds[ent.x], ent, step);
        size_t ls;
        double *w = co_tracer(c.W, c.L, c.plane, c.cell, c.NIJ, sl.y, ls);
        const unsigned char *log = colog + (size_t)sl.x * kCoLogBytes;
        const int nm = *reinterpret_cast<const int *>(log);
        const unsigned mask = *reinterpret_cast<const unsigned *>(log + 4);
        const double *ldt = reinterpret_cast<const double *>(log + kCoLogDtot);
        const double *ly = reinterpret_cast<const double *>(log + kCoLogY);
        const double *ldp = reinterpret_cast<const double *>(log + kCoLogDtop);
        const double *ledz = reinterpret_cast<const double *>(log + kCoLogEdz);
        // the next merge's and the next absorbed level's log entries are read one ahead (every
        // index stays inside the slot), so their loads overlap the FP64 chain
        int ei = 0, lv = log[kCoLogElev];
        double dzv = ledz[0];
        int x = log[kCoLogX], cnt = log[kCoLogCnt];
        double dtop = ldp[0], dtot = ldt[0], y = ly[0];
        for (int k = 0; k < nm; ++k) {
            const int xn = log[kCoLogX + k + 1], cntn = log[kCoLogCnt + k + 1];
            const double dtopn = ldp[k + 1], dtotn = ldt[k + 1], yn = ly[k + 1];
            double acc = __dmul_rn(w[(size_t)x * ls], dtop);
            for (int q = 0; q < cnt; ++q) {
                const int l = lv;
                const double dz = dzv;
                ++ei;
                lv = log[kCoLogElev + ei];
                dzv = ledz[ei];
                acc = __dadd_rn(acc, __dmul_rn(w[(size_t)l * ls], dz));
            }
            w[(size_t)x * ls] = co_div(acc, dtot, y);
            x = xn;
            cnt = cntn;
            dtop = dtopn;
            dtot = dtotn;
            y = yn;
        }
        const unsigned fillm = ~mask & co_bits(c.k1, c.maxk - 1);
        for (unsigned f = fillm; f; f &= f - 1u) {
            const int lev = __ffs(f);
            w[(size_t)lev * ls] = w[(size_t)__ffs(mask & ~((1u << lev) - 1u)) * ls];
        }
    }
}

// The one-warp-per-column form (small batches) of the columns with maxk <= 32, ieos = 0,
// iconv = 0, imld = 0: warps take list entries in turn; co_warp32 (co_column.cuh) holds one
// list position per lane and mixes the column's tracers one lane each.  kmax: the largest maxk
// of the batch (shared memory: (kmax+1) x 32 tracer values per warp).
__global__ void __launch_bounds__(kFp32Threads)
k_co_warp(const MemberDesc *__restrict__ mds, const int2 *__restrict__ colist, int *__restrict__ cocount, int cocap,
          const long long *__restrict__ step_ctr, int rel, int kmax)
{
    extern __shared__ double cosm[];
    const long long step = *step_ctr + rel;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int ncol = min(cocount[step & 1], cocap);
    // the list of the next step starts empty (that step's kernels run after this one)
    if (blockIdx.x == 0 && threadIdx.x == 0) cocount[(step + 1) & 1] = 0;
    double *tv = cosm + (size_t)warp * (kmax + 1) * 32;
    for (int e = blockIdx.x * nwarp + warp; e < ncol; e += gridDim.x * nwarp) {
        const int2 ent = colist[e];
        const MemberDesc &md = mds[ent.x];
        if (!fp32_co_fast(md.iconv, md.ieos, md.imld, md.maxk)) continue;
        const CoCol c = co_col(md, ent, step);
        EosCoef ec;
        for (int n = 0; n < 5; ++n) ec.ec[n] = md.ec[n];
        ec.ieos = 0;
        // this lane's tracer (lanes < L) at level 0 and its level stride
        size_t lstride = 0;
        double *wc = lane < c.L ? co_tracer(c.W, c.L, c.plane, c.cell, c.NIJ, lane, lstride) : nullptr;
        // T and S are plane 0, two values per cell
        const int filled = co_warp32(tv, ec, c.maxk, c.L, c.k1, c.dz, lane, c.W + 2 * c.cell, 2 * c.NIJ, wc, lstride);
        if (lane == 0 && filled > 0) *c.cost = add_count_rn(*c.cost, filled);
        __syncwarp();
    }
}

// The serial form for the other listed columns.  kmax: the largest maxk of the batch (shared
// memory layout).
__global__ void __launch_bounds__(kFp32Threads)
k_co_serial(const MemberDesc *__restrict__ mds, const int2 *__restrict__ colist, int *__restrict__ cocount, int cocap,
            const long long *__restrict__ step_ctr, int rel, int kmax)
{
    extern __shared__ double cosm[];
    const long long step = *step_ctr + rel;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int ncol = min(cocount[step & 1], cocap);
    double *tv = cosm + (size_t)warp * (kmax + 1) * 32;
    CoWarpState *cs = reinterpret_cast<CoWarpState *>(cosm + (size_t)nwarp * (kmax + 1) * 32) + warp;
    for (int e = blockIdx.x * nwarp + warp; e < ncol; e += gridDim.x * nwarp) {
        const int2 ent = colist[e];
        const MemberDesc &md = mds[ent.x];
        const int32_t *ticol = md.ptab + ent.y;
        const int maxk = md.maxk, L = md.L, NI = md.NI, NJ = md.NJ, mkn = maxk + 2;
        // the two-phase form takes the others
        if (fp32_co_fast(md.iconv, md.ieos, md.imld, maxk)) continue;
        const int k1c = (ticol[2] >> 16) & 0xffff, cl0 = ticol[3];
        const int i = ticol[4] & 0xffff, j = (ticol[4] >> 16) & 0xffff;
        const int par = (int)((step + md.parity) & 1);
        double *W = md.buf[par ^ 1];
        const double *mk = md.mk;
        const double *dz = mk, *rdz = mk + mkn, *zw = mk + 2 * mkn, *zro = mk + 3 * mkn;
        EosCoef ec;
        for (int n = 0; n < 5; ++n) ec.ec[n] = md.ec[n];
        ec.ieos = md.ieos;
        if (md.iconv == 1 || md.imld != 0) {
            // coshuffle (iconv = 1), co and the mixed layer (imld = 1) on one lane, in the
            // order of tstepo (goldstein.f90:2311-2389)
            if (lane == 0) {
                Fp32Col col;
                col.w = W;
                col.stat = md.ts_static;
                col.L = L;
                col.NI = NI;
                col.NJ = NJ;
                col.nk = maxk + 2;
                col.init_planes();
                col.i = i;
                col.j = j;
                col.k1 = k1c;
                col.rho[0] = 0.0;
                for (int kk = 1; kk <= maxk; ++kk) col.rho[kk] = eos_rn(ec, col.T(0, kk), col.T(1, kk), zro[kk]);
                double rold[kMaxK + 1];
                MixedLayerArgs ml{};
                if (md.imld != 0) {
                    // the densities before co, and mldpe1 from the start-of-step T and S of the top
                    // layer (the other buffer) less the forcing slot ts(:,i,j,maxk+1)
                    for (int kk = 1; kk <= maxk; ++kk) rold[kk] = col.rho[kk];
                    Fp32Col c0 = col;
                    c0.w = md.buf[par];
                    // the first step after an upload reads the uploaded ts (the step itself starts
                    // from ts1), as the reference's first tstepo does
                    if (step == md.origin) c0.k1 = maxk + 1;
                    const double *top = md.ts_static + (size_t)L * ((size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * (maxk + 1)));
                    ml.zw = zw;
                    ml.zro = zro;
                    ml.dz = dz;
                    ml.mlddec = md.mlddec;
                    ml.mlddecd = md.mlddecd;
                    ml.mldpebuoycoeff = md.mldpebuoycoeff;
                    ml.ketau = md.mldketau[cl0];
                    ml.pe1 = ml_pe1(ec, __dadd_rn(c0.T(0, maxk), -top[0]), __dadd_rn(c0.T(1, maxk), -top[1]), md.rhos[cl0],
                                    zw, zro, maxk);
                }
                if (md.iconv == 1) {
                    int icos = coshuffle_rn(col, ec, maxk, L, k1c, dz, rdz, zw);
                    const int filled = co_rn(col, ec, maxk, L, k1c, dz, zw);
                    if (filled > icos) icos = filled;
                    md.icosd[cl0] = icos;
                    md.cost[cl0] = __dmul_rn(md.dsc, zw[maxk - 1 - icos]);
                } else {
                    const int filled = co_rn(col, ec, maxk, L, k1c, dz, zw);
                    if (filled > 0) md.cost[cl0] = add_count_rn(md.cost[cl0], filled);
                }
                if (md.imld != 0) {
                    mixed_layer_rn(col, ec, maxk, L, k1c, ml, rold, &md.mld[cl0], &md.mldk[cl0]);
                    // rho(maxk) for the next step's mldpe1: co's value, or with ieos != 0 the
                    // density of the final state (goldstein.f90:2391-2398)
                    md.rhos[cl0] = ec.ieos != 0 ? eos_rn(ec, col.T(0, maxk), col.T(1, maxk), zro[maxk]) : col.rho[maxk];
                }
            }
            __syncwarp();
            continue;
        }
        // the column's wet levels into shared memory, lane l holding tracer l
        size_t wofs = 0;
        int gpw = 2;
        if (lane < L) {
            int g0 = 0, gl = 2, gp = 2, pl = 0;
            for (int h = 0; h < fp32_ngroups(L); ++h) {
                fp32_plane(L, h, &g0, &gl, &gp, &pl);
                if (lane < g0 + gl) break;
            }
            wofs = (size_t)pl * NI * NJ * (maxk + 2) + (lane - g0);
            gpw = gp;
        }
        const size_t NIJ = (size_t)NI * NJ;
        const double *wc = W + wofs + ((size_t)i + (size_t)NI * j) * gpw;
        const size_t lstride = NIJ * gpw;
        if (lane < L)
            for (int lev = k1c; lev <= maxk; lev += 8) {
                double v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (lev + u <= maxk) v[u] = wc[(size_t)(lev + u) * lstride];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (lev + u <= maxk) tv[(lev + u) * 32 + lane] = v[u];
            }
        __syncwarp();
        const int filled = co_warp(tv, cs, ec, maxk, L, k1c, dz, zro, zw, lane);
        if (lane < L)
            for (int lev = k1c; lev <= maxk; ++lev) const_cast<double *>(wc)[(size_t)lev * lstride] = tv[lev * 32 + lane];
        if (lane == 0 && filled > 0) md.cost[cl0] = add_count_rn(md.cost[cl0], filled);
        __syncwarp();
    }
}

int fp32_smem_bytes(int max_slots) { return fp32_smem_layout(max_slots + 1).total; }

// Resident CTAs per SM of a kernel at a block size and dynamic shared memory size, with the
// kernel's shared-memory limit raised to at least that size first.  Both are runtime calls
// costing microseconds on every launch of a step that is not replayed from a CUDA graph, so the
// process remembers, per device and kernel, the largest limit it has set (it is only ever
// raised: a launch with less shared memory stays valid) and the occupancy of every size asked.
static int resident_ctas(const void *fn, int threads, int smem)
{
    struct Limit {
        int dev;
        const void *fn;
        int smem;
    };
    struct Occ {
        int dev;
        const void *fn;
        int threads, smem, per_sm;
    };
    static std::mutex mu;
    static std::vector<Limit> limits;
    static std::vector<Occ> occ;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    if (smem > 0) {
        Limit *lim = nullptr;
        for (Limit &x : limits)
            if (x.dev == dev && x.fn == fn) lim = &x;
        if (!lim) {
            limits.push_back({dev, fn, 0});
            lim = &limits.back();
        }
        if (smem > lim->smem && cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess)
            lim->smem = smem;
    }
    for (const Occ &x : occ)
        if (x.dev == dev && x.fn == fn && x.threads == threads && x.smem == smem) return x.per_sm;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
    occ.push_back({dev, fn, threads, smem, per_sm});
    return per_sm;
}

template <bool ISO, bool TS>
static void launch_step_instance(const MemberDesc *descs, const int4 *items, int nitems, int P,
                                 const long long *step_ctr, int rel, int *work, int2 *colist, int *cocount, int cocap,
                                 int nsm, int ctas_cap, cudaStream_t s)
{
    if (nitems <= 0) return;
    const int smem_bytes = fp32_smem_layout(P).total;
    auto kern = k_step_fp32<ISO, TS>;
    int per_sm = resident_ctas((const void *)kern, kFp32Threads, smem_bytes);
    if (ctas_cap > 0) per_sm = std::min(per_sm, ctas_cap);
    if (per_sm < 1) per_sm = 1;
    const int grid = std::max(1, std::min(nitems, nsm * per_sm));
    kern<<<grid, kFp32Threads, smem_bytes, s>>>(descs, items, nitems, step_ctr, rel, work, P, colist, cocount, cocap);
}

int fp32_launch(const Fp32Batch &b, const long long *step_ctr, int rel, cudaStream_t s, cudaStream_t s2,
                cudaEvent_t fork, cudaEvent_t join)
{
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    }
    const int P = b.max_slots + 1;
    // the top-face stencils of the members that rebuild them every step
    if (b.n_stencil > 0)
        k_stencil_fp32<<<dim3(b.stencil_blocks, b.n_stencil), 256, 0, s>>>(b.descs, b.stencil_list, step_ctr, rel);
    // the T-S items and the other items run side by side (two streams), then the adjustment
    const bool two = b.n_ts > 0 && b.n_bgc > 0 && s2 != nullptr;
    if (two) {
        cudaEventRecord(fork, s);
        cudaStreamWaitEvent(s2, fork, 0);
    }
    cudaStream_t sb = two ? s2 : s;
    if (b.iso) {
        launch_step_instance<true, true>(b.descs, b.items, b.n_ts, P, step_ctr, rel, b.work, b.colist,
                                         b.cocount, b.cocap, nsm, b.ctas_per_sm, s);
        launch_step_instance<true, false>(b.descs, b.items + b.n_ts, b.n_bgc, P, step_ctr, rel, b.work + 2,
                                          b.colist, b.cocount, b.cocap, nsm, b.ctas_per_sm, sb);
    } else {
        launch_step_instance<false, true>(b.descs, b.items, b.n_ts, P, step_ctr, rel, b.work, b.colist,
                                          b.cocount, b.cocap, nsm, b.ctas_per_sm, s);
        launch_step_instance<false, false>(b.descs, b.items + b.n_ts, b.n_bgc, P, step_ctr, rel,
                                           b.work + 2, b.colist, b.cocount, b.cocap, nsm, b.ctas_per_sm, sb);
    }
    // the adjustment's form: two phases for large batches, one warp per column for small ones
    const bool two_phase = fp32_co_two_phase(b);
    // the two-phase decisions need only T, S and the column list, which the T-S items complete:
    // they run while the other tracer groups are still stepping (k_co_decide writes T and S in
    // place, plane 0 of the new state, which the group items neither read nor write)
    if (two_phase) {
        const int smem = (kCoDecideThreads / 32) * kCoDecideWarpBytes;
        resident_ctas((const void *)k_co_decide, kCoDecideThreads, smem);
        // one one-warp block per 32 list entries of the capacity: blocks past the step's count
        // exit, and the others are scheduled as SMs free up (a deep column's warp delays only itself)
        const int grid = std::max(1, (b.cocap + kCoDecideThreads - 1) / kCoDecideThreads);
        k_co_decide<<<grid, kCoDecideThreads, smem, s>>>(b.descs, b.colist, b.cocount, b.cocap, step_ctr,
                                                                            rel, b.colog, b.comap, b.mapcap);
    }
    if (two) {
        cudaEventRecord(join, s2);
        cudaStreamWaitEvent(s, join, 0);
    }
    // then the other tracers of the two-phase columns (or the one-warp-per-column form), and (if
    // the batch has any) the serial columns
    if (!two_phase) {
        const int kst = std::min(b.kmax, 32) + 1;
        const int wsmem = (kFp32Threads / 32) * kst * 32 * (int)sizeof(double);
        const int wper_sm = resident_ctas((const void *)k_co_warp, kFp32Threads, wsmem);
        k_co_warp<<<nsm * std::max(1, wper_sm), kFp32Threads, wsmem, s>>>(b.descs, b.colist, b.cocount, b.cocap, step_ctr,
                                                                        rel, std::min(b.kmax, 32));
    } else {
        const int mper_sm = resident_ctas((const void *)k_co_mix, kCoMixThreads, 0);
        k_co_mix<<<nsm * std::max(1, mper_sm), kCoMixThreads, 0, s>>>(b.descs, b.colist, b.cocount, step_ctr, rel, b.colog,
                                                                     b.comap, b.mapcap);
    }
    if (b.co_general) {
        const int co_smem = (kFp32Threads / 32) * ((b.kmax + 1) * 32 * (int)sizeof(double) + (int)sizeof(CoWarpState));
        const int co_per_sm = resident_ctas((const void *)k_co_serial, kFp32Threads, co_smem);
        k_co_serial<<<nsm * std::max(1, co_per_sm), kFp32Threads, co_smem, s>>>(b.descs, b.colist, b.cocount, b.cocap,
                                                                               step_ctr, rel, b.kmax);
    }
    return launch_status();
}

int fp32_launches_per_step(const Fp32Batch &b)
{
    return (b.n_stencil > 0) + (b.n_ts > 0) + (b.n_bgc > 0) + (fp32_co_two_phase(b) ? 2 : 1) + (b.co_general ? 1 : 0);
}

// ---------------------------------------------------------------------------
// patch plan (host): rectangles of water columns, periodic in i, with the ring of
// wet neighbour columns; slots sorted by k1 so the wet cells of a level are a prefix

int fp32_group_count(int L) { return fp32_ngroups(L); }

// one thread per slot; slot indices are 16-bit in the tables
static int plan_cap_slots(int) { return kFp32Threads; }

namespace {
struct PatchShape {
    std::vector<std::pair<int, int>> inner;   // (i, j) wet columns of the rectangle
    std::vector<std::pair<int, int>> ring;    // wet neighbours outside it
    std::vector<int> seen;                    // scratch: stamp of the last patch that took a column
    int stamp = 0;
};
}

// Columns of rectangle [i0, i1] x [j0, j1] and its ring; false if over the kernel limits.
static bool patch_shape(const Dims &d, const int32_t *k1, int i0, int i1, int j0, int j1, int cap, PatchShape &ps)
{
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk, NI = d.NI;
    auto wet = [&](int i, int j) { return j >= 0 && j <= maxj + 1 && k1[i + (size_t)NI * j] <= maxk; };
    auto inside = [&](int i, int j) { return i >= i0 && i <= i1 && j >= j0 && j <= j1; };
    ps.inner.clear();
    ps.ring.clear();
    for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i)
            if (wet(i, j)) ps.inner.push_back({i, j});
    if ((int)ps.inner.size() > kFp32Threads) return false;
    if (ps.seen.size() != (size_t)NI * (maxj + 2)) {
        ps.seen.assign((size_t)NI * (maxj + 2), 0);
        ps.stamp = 0;
    }
    const int stamp = ++ps.stamp;
    for (auto &c : ps.inner) {
        const int i = c.first, j = c.second;
        const int nb[4][2] = {{i == maxi ? 1 : i + 1, j}, {i == 1 ? maxi : i - 1, j}, {i, j + 1}, {i, j - 1}};
        for (auto &n : nb) {
            if (n[1] < 0 || n[1] > maxj + 1 || inside(n[0], n[1]) || !wet(n[0], n[1])) continue;
            int &s = ps.seen[n[0] + (size_t)NI * n[1]];
            if (s != stamp) {
                s = stamp;
                ps.ring.push_back({n[0], n[1]});
            }
        }
    }
    return (int)(ps.inner.size() + ps.ring.size()) <= cap;
}

// Estimated issue cost of a tiling: per patch, level and tracer group, the warps that hold
// wet interior slots (load, convert, transfers, update: ~60 instructions per tracer) and
// wet ring slots (load and convert: ~10), plus a per-level overhead of the CTA.
static double plan_cost(const Dims &d, const int32_t *k1, int tx, int ty, int cap, bool *ok)
{
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk, NI = d.NI;
    const int ng = (d.L + kGroup - 1) / kGroup;
    const double per_t = (double)d.L / ng;
    double cost = 0.0;
    PatchShape ps;
    std::vector<int> hi(maxk + 2), hr(maxk + 2);
    *ok = true;
    for (int j0 = 1; j0 <= maxj; j0 += ty)
        for (int i0 = 1; i0 <= maxi; i0 += tx) {
            if (!patch_shape(d, k1, i0, std::min(maxi, i0 + tx - 1), j0, std::min(maxj, j0 + ty - 1), cap, ps)) {
                *ok = false;
                return 0.0;
            }
            if (ps.inner.empty()) continue;
            std::fill(hi.begin(), hi.end(), 0);
            std::fill(hr.begin(), hr.end(), 0);
            int kst = maxk + 1;
            for (auto &c : ps.inner) {
                const int kk = k1[c.first + (size_t)NI * c.second];
                hi[kk] += 1;
                kst = std::min(kst, kk);
            }
            for (auto &c : ps.ring) hr[std::max(kst, (int)k1[c.first + (size_t)NI * c.second])] += 1;
            int ni = 0, nr = 0;
            for (int k = 1; k <= maxk; ++k) {
                ni += hi[k];
                nr += hr[k];
                if (k < kst) continue;
                cost += ng * (std::ceil(ni / 32.0) * 32 * 60 * per_t + std::ceil(nr / 32.0) * 32 * 10 * per_t + 256 * 20);
            }
        }
    return cost;
}

int fp32_plan_patches(const Dims &d, const int32_t *k1, int tile_i, int tile_j, PatchPlan &plan)
{
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk, NI = d.NI;
    const int cap = plan_cap_slots(d.L);
    int best_tx = 0, best_ty = 0;
    if (tile_i > 0 && tile_j > 0) {
        bool ok = false;
        plan_cost(d, k1, std::min(tile_i, maxi), std::min(tile_j, maxj), cap, &ok);
        if (ok) {
            best_tx = std::min(tile_i, maxi);
            best_ty = std::min(tile_j, maxj);
        }
    }
    // Rectangles that split the rows and columns evenly (or nearly).  The first pass keeps
    // to 48..256 cells: a patch holds at most 128 slots, so larger rectangles fit only on
    // land-heavy grids, and below 48 cells the ring outweighs the interior.  A grid on
    // which no such rectangle fits gets the full search.
    for (int pass = 0; pass < 2 && !best_tx; ++pass) {
        double best = 1e300;
        for (int tx = maxi; tx >= 1; --tx) {
            const int nti = (maxi + tx - 1) / tx;
            if (tx != (maxi + nti - 1) / nti) continue;
            for (int ty = 1; ty <= maxj; ++ty) {
                const int ntj = (maxj + ty - 1) / ty;
                if (ty != (maxj + ntj - 1) / ntj) continue;
                if (tx * ty > (pass ? 4 : 2) * kFp32Threads) break;
                if (pass == 0 && tx * ty < 48 && tx * ty < maxi * maxj) continue;
                bool ok = false;
                const double c = plan_cost(d, k1, tx, ty, cap, &ok);
                if (ok && c < best) {
                    best = c;
                    best_tx = tx;
                    best_ty = ty;
                }
            }
        }
    }
    if (!best_tx) return GB_GO_ERANGE;
    plan.words.clear();
    plan.offset.clear();
    plan.cost.clear();
    plan.max_slots = 1;
    plan.tile_i = best_tx;
    plan.tile_j = best_ty;
    PatchShape ps;
    int pidx = 0;
    for (int j0 = 1; j0 <= maxj; j0 += best_ty)
        for (int i0 = 1; i0 <= maxi; i0 += best_tx) {
            patch_shape(d, k1, i0, std::min(maxi, i0 + best_tx - 1), j0, std::min(maxj, j0 + best_ty - 1), cap, ps);
            if (ps.inner.empty()) continue;
            struct Slot { int k1, j, i, inner; };
            std::vector<Slot> sl;
            for (auto &c : ps.inner) sl.push_back({k1[c.first + (size_t)NI * c.second], c.second, c.first, 1});
            for (auto &c : ps.ring) sl.push_back({k1[c.first + (size_t)NI * c.second], c.second, c.first, 0});
            // interior slots first, then the ring; each part by k1 (then row, column)
            std::stable_sort(sl.begin(), sl.end(), [](const Slot &a, const Slot &b) {
                if (a.inner != b.inner) return a.inner > b.inner;
                if (a.k1 != b.k1) return a.k1 < b.k1;
                if (a.j != b.j) return a.j < b.j;
                return a.i < b.i;
            });
            const int ns = (int)sl.size(), ni = (int)ps.inner.size();
            std::vector<int> slot_of((size_t)NI * (maxj + 2), -1);
            for (int s = 0; s < ns; ++s) slot_of[sl[s].i + (size_t)NI * sl[s].j] = s;
            int kst = maxk + 1;
            for (auto &s : sl)
                if (s.inner) kst = std::min(kst, s.k1);
            const size_t off = plan.words.size();
            plan.offset.push_back((int32_t)off);
            std::vector<int32_t> w(kPatchHdr + 2 * (maxk + 2) + ns, 0);
            w[0] = ns;
            w[1] = ni;
            w[2] = kst;
            w[3] = pidx++;
            for (int k = 0; k <= maxk + 1; ++k) {
                int a = 0, r = 0;
                for (auto &x : sl)
                    if (x.k1 <= k) (x.inner ? a : r) += 1;
                w[kPatchHdr + k] = a;
                w[kPatchHdr + maxk + 2 + k] = r;
            }
            for (int s = 0; s < ns; ++s) w[kPatchHdr + 2 * (maxk + 2) + s] = sl[s].i + NI * sl[s].j;
            while (w.size() & 3) w.push_back(0);
            auto nbslot = [&](int i, int j) -> int {
                if (j < 0 || j > maxj + 1) return 0xffff;
                const int s = slot_of[i + (size_t)NI * j];
                return s < 0 ? 0xffff : s;
            };
            auto k1c8 = [&](int i, int j) -> int {
                if (j < 0 || j > maxj + 1) return 255;
                return std::min(255, (int)k1[i + (size_t)NI * j]);
            };
            double cost = 0.0;
            for (int s = 0; s < ns; ++s) {
                if (!sl[s].inner) continue;
                const int i = sl[s].i, j = sl[s].j;
                const int ie = i == maxi ? 1 : i + 1, iw = i == 1 ? maxi : i - 1;
                w.push_back(s | (nbslot(ie, j) << 16));
                w.push_back(nbslot(iw, j) | (nbslot(i, j + 1) << 16));
                w.push_back(nbslot(i, j - 1) | (sl[s].k1 << 16));
                w.push_back((i - 1) + maxi * (j - 1));
                w.push_back(i | (j << 16));
                w.push_back(k1c8(ie, j) | (k1c8(iw, j) << 8) | (k1c8(i, j + 1) << 16) | (k1c8(i, j - 1) << 24));
                w.push_back((iw - 1) + maxi * (j - 1));
                w.push_back(0);
                cost += (double)(maxk - sl[s].k1 + 1) * d.L;
            }
            plan.words.insert(plan.words.end(), w.begin(), w.end());
            plan.cost.push_back(cost);
            plan.max_slots = std::max(plan.max_slots, ns);
        }
    return GB_GO_OK;
}

// ---------------------------------------------------------------------------
// host-side static data

// The cell's sum of signed face transfer sums D = (Cw - Ce) + (Cs - Cn) + (Cb - Ca), C = A + B of a
// face, in FP64 from the FP32 pairs (coefficient + remainder) of the cell and of its west, south
// and lower neighbours, as an FP32 pair (dh, dl); zero where |D| is within 2^-40 of the faces'
// magnitudes (a divergence-free velocity field leaves only FP64 rounding there).  A uniform
// offset tref then gains tref * D per step, the share of the offset the transfers of T - tref
// leave out.  Host and device evaluate the same expressions (additions only).
__host__ __device__ inline void fp32_div_pair(const float *ch, const float *cl, int maxi, size_t nij, size_t c,
                                              size_t cw, bool south, bool below, float *dh, float *dl)
{
    auto C = [&](size_t cell, int f) {
        return ((double)ch[8 * cell + 2 * f] + (double)cl[8 * cell + 2 * f]) +
               ((double)ch[8 * cell + 2 * f + 1] + (double)cl[8 * cell + 2 * f + 1]);
    };
    const double ce = C(c, 0), cn = C(c, 1), ca = C(c, 2), cwe = C(cw, 0);
    const double cs = south ? C(c - (size_t)maxi, 1) : 0.0;
    const double cb = below ? C(c - nij, 2) : 0.0;
    const double D = ((cwe - ce) + (cs - cn)) + (cb - ca);
    const double S = ((fabs(cwe) + fabs(ce)) + (fabs(cs) + fabs(cn))) + (fabs(cb) + fabs(ca));
    if (!(fabs(D) > 0x1p-40 * S)) {
        *dh = 0.0f;
        *dl = 0.0f;
        return;
    }
    const float h = (float)D;
    *dh = h;
    *dl = (float)(D - (double)h);
}

void fp32_build_static(const Dims &d, const PhysParams &p, const std::vector<double> &blob, const int32_t *k1,
                       const double *u, Fp32Static &out)
{
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk, NI = d.NI;
    const int nj = maxj + 2, nk = maxk + 2;
    const double *b = blob.data();
    const double *rc = b, *rc2 = b + nj, *cv = b + 2 * nj, *cv2 = b + 3 * nj, *dsv = b + 4 * nj, *rdsv = b + 5 * nj,
                 *ds = b + 6 * nj;
    const double *kb = b + 8 * nj;
    const double *dz = kb, *dza = kb + nk, *rdz = kb + 2 * nk, *rdza = kb + 3 * nk, *zro = kb + 4 * nk,
                 *dt = kb + 5 * nk, *zw = kb + 6 * nk, *ssmax = kb + 7 * nk, *diffmax = kb + 8 * nk;
    const size_t ncell = (size_t)maxi * maxj * maxk;
    out.coef.assign(8 * ncell, 0.0f);
    out.coefl.assign(8 * ncell, 0.0f);
    out.cmax = 0.0;
    out.dmax = 0.0;
    auto U = [&](int c, int i, int j, int k) -> double {
        return u[(size_t)c + 3 * ((size_t)i + (size_t)(maxi + 1) * ((size_t)j + (size_t)(maxj + 1) * (size_t)(k - 1)))];
    };
    auto K1 = [&](int i, int j) { return k1[i + (size_t)NI * j]; };
    for (int k = 1; k <= maxk; ++k) {
        for (int j = 1; j <= maxj; ++j) {
            for (int i = 1; i <= maxi; ++i) {
                const size_t cell = (size_t)(i - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (k - 1));
                float *c = &out.coef[8 * cell];
                float *cl = &out.coefl[8 * cell];
                double cd[6] = {0, 0, 0, 0, 0, 0};
                const int k1c = K1(i, j);
                const int ie = (i == maxi) ? 1 : i + 1;
                if (k >= std::max(k1c, K1(ie, j))) {
                    const double u1 = U(0, i, j, k);
                    const double pec = u1 * p.dphi / p.diff1, ups = pec / (2.0 + std::fabs(pec));
                    const double g = dt[k] * ds[j] * dz[k], a = u1 * rc[j];
                    cd[0] = g * (a * (1.0 - ups) * 0.5 - rc2[j] * p.diff1);
                    cd[1] = g * (a * (1.0 + ups) * 0.5 + rc2[j] * p.diff1);
                }
                if (k >= std::max(k1c, K1(i, j + 1))) {
                    const double u2 = U(1, i, j, k);
                    const double pec = u2 * dsv[std::min(j, maxj - 1)] / p.diff1, ups = pec / (2.0 + std::fabs(pec));
                    const double g = dt[k] * p.dphi * dz[k], a = cv[j] * u2;
                    cd[2] = g * (a * (1.0 - ups) * 0.5 - cv2[j] * p.diff1);
                    cd[3] = g * (a * (1.0 + ups) * 0.5 + cv2[j] * p.diff1);
                }
                if (k >= k1c && k < maxk) {
                    const double u3 = U(2, i, j, k);
                    const double pec = u3 * dza[k] / p.diff2, ups = pec / (2.0 + std::fabs(pec));
                    const double g = dt[k] * p.dphi * ds[j];
                    cd[4] = g * (u3 * (1.0 - ups) * 0.5 - rdza[k] * p.diff2);
                    cd[5] = g * (u3 * (1.0 + ups) * 0.5 + rdza[k] * p.diff2);
                    if (p.iediff > 0 && p.iediff < 3) {
                        // the step rebuilds these with diffv <= diffmax(k+1): bound the initial
                        // fixed-point scales with the larger diffusivity
                        const double dv = std::max(p.diff2, diffmax[k + 1]);
                        out.cmax = std::max(out.cmax, g * (std::fabs(u3) + 2.0 * rdza[k] * dv));
                    }
                }
                // Ae Be An Bn Aa Ba 0 0 as FP32, and their FP64 remainders in the same order
                for (int n = 0; n < 6; ++n) {
                    c[n] = (float)cd[n];
                    cl[n] = (float)(cd[n] - (double)c[n]);
                }
                for (int f = 0; f < 3; ++f)
                    out.cmax = std::max(out.cmax, (double)std::fabs(c[2 * f]) + (double)std::fabs(c[2 * f + 1]));
            }
        }
    }
    // words 6, 7: the cell's divergence pair (fp32_div_pair)
    const size_t nij = (size_t)maxi * maxj;
    for (int k = 1; k <= maxk; ++k)
        for (int j = 1; j <= maxj; ++j)
            for (int i = 1; i <= maxi; ++i) {
                const size_t c = (size_t)(i - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (k - 1));
                const int iw = i == 1 ? maxi : i - 1;
                const size_t cw = (size_t)(iw - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (k - 1));
                fp32_div_pair(out.coef.data(), out.coefl.data(), maxi, nij, c, cw, j > 1, k > 1, &out.coef[8 * c + 6],
                              &out.coef[8 * c + 7]);
                out.dmax = std::max(out.dmax, std::fabs((double)out.coef[8 * c + 6]) + std::fabs((double)out.coef[8 * c + 7]));
            }
    fp32_build_small(d, p, blob, out);
}

void fp32_build_small(const Dims &d, const PhysParams &p, const std::vector<double> &blob, Fp32Static &out)
{
    const int maxj = d.maxj, maxk = d.maxk;
    const int nj = maxj + 2, nk = maxk + 2;
    const double *b = blob.data();
    const double *rc = b, *cv = b + 2 * nj, *rdsv = b + 5 * nj, *ds = b + 6 * nj;
    const double *kb = b + 8 * nj;
    const double *dz = kb, *rdz = kb + 2 * nk, *rdza = kb + 3 * nk, *zro = kb + 4 * nk, *dt = kb + 5 * nk,
                 *zw = kb + 6 * nk, *ssmax = kb + 7 * nk;
    out.rvol.assign((size_t)maxj * maxk, 0.0);
    for (int k = 1; k <= maxk; ++k)
        for (int j = 1; j <= maxj; ++j) out.rvol[(size_t)(j - 1) + (size_t)maxj * (k - 1)] = 1.0 / (p.dphi * ds[j] * dz[k]);
    out.mk.assign(6 * (size_t)nk, 0.0);
    for (int k = 0; k <= maxk + 1; ++k) {
        out.mk[k] = dz[k];
        out.mk[nk + k] = rdz[k];
        out.mk[2 * nk + k] = zw[k];
        out.mk[3 * nk + k] = zro[k];
        out.mk[4 * nk + k] = rdza[k];
        out.mk[5 * nk + k] = ssmax[k];
    }
    out.mj.assign(3 * (size_t)nj, 0.0);
    for (int j = 0; j <= maxj; ++j) {
        out.mj[j] = rc[j] * p.rdphi;
        out.mj[nj + j] = cv[j] * rdsv[j];
        if (j >= 1) out.mj[2 * nj + j] = dt[1] * p.dphi * ds[j];
    }
}

// The transfer coefficients of fp32_build_static from device-resident velocities (the
// velocity field of every ocean step in a coupled run): the same FP64 expressions in the
// same order, with round-to-nearest intrinsics (no contraction), so the coefficients are
// those the host builds.  One thread per interior cell.
__device__ __forceinline__ void build_coef_cells(const double *__restrict__ u, const Metrics &m, const Dims &d,
                                                 const PhysParams &p, float *coef, float *coefl, size_t c0, size_t cs)
{
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk, NI = d.NI;
    const size_t ncell = (size_t)maxi * maxj * maxk;
    for (size_t c = c0; c < ncell; c += cs) {
        const int i = (int)(c % maxi) + 1;
        const int j = (int)((c / maxi) % maxj) + 1;
        const int k = (int)(c / ((size_t)maxi * maxj)) + 1;
        auto U = [&](int cc, int ii, int jj, int kk) {
            return u[(size_t)cc + 3 * ((size_t)ii + (size_t)(maxi + 1) * ((size_t)jj + (size_t)(maxj + 1) * (size_t)(kk - 1)))];
        };
        auto K1 = [&](int ii, int jj) { return m.k1[ii + (size_t)NI * jj]; };
        double cd[6] = {0, 0, 0, 0, 0, 0};
        const int k1c = K1(i, j);
        const int ie = (i == maxi) ? 1 : i + 1;
        const int ke = K1(ie, j) > k1c ? K1(ie, j) : k1c;
        if (k >= ke) {
            const double u1 = U(0, i, j, k);
            const double pec = __ddiv_rn(__dmul_rn(u1, p.dphi), p.diff1);
            const double ups = __ddiv_rn(pec, __dadd_rn(2.0, fabs(pec)));
            const double g = __dmul_rn(__dmul_rn(m.dt[k], m.ds[j]), m.dz[k]), a = __dmul_rn(u1, m.rc[j]);
            const double dd = __dmul_rn(m.rc2[j], p.diff1);
            cd[0] = __dmul_rn(g, __dsub_rn(__dmul_rn(__dmul_rn(a, __dsub_rn(1.0, ups)), 0.5), dd));
            cd[1] = __dmul_rn(g, __dadd_rn(__dmul_rn(__dmul_rn(a, __dadd_rn(1.0, ups)), 0.5), dd));
        }
        const int kn = K1(i, j + 1) > k1c ? K1(i, j + 1) : k1c;
        if (k >= kn) {
            const double u2 = U(1, i, j, k);
            const double pec = __ddiv_rn(__dmul_rn(u2, m.dsv[j < maxj - 1 ? j : maxj - 1]), p.diff1);
            const double ups = __ddiv_rn(pec, __dadd_rn(2.0, fabs(pec)));
            const double g = __dmul_rn(__dmul_rn(m.dt[k], p.dphi), m.dz[k]), a = __dmul_rn(m.cv[j], u2);
            const double dd = __dmul_rn(m.cv2[j], p.diff1);
            cd[2] = __dmul_rn(g, __dsub_rn(__dmul_rn(__dmul_rn(a, __dsub_rn(1.0, ups)), 0.5), dd));
            cd[3] = __dmul_rn(g, __dadd_rn(__dmul_rn(__dmul_rn(a, __dadd_rn(1.0, ups)), 0.5), dd));
        }
        if (k >= k1c && k < maxk) {
            const double u3 = U(2, i, j, k);
            const double pec = __ddiv_rn(__dmul_rn(u3, m.dza[k]), p.diff2);
            const double ups = __ddiv_rn(pec, __dadd_rn(2.0, fabs(pec)));
            const double g = __dmul_rn(__dmul_rn(m.dt[k], p.dphi), m.ds[j]);
            const double dd = __dmul_rn(m.rdza[k], p.diff2);
            cd[4] = __dmul_rn(g, __dsub_rn(__dmul_rn(__dmul_rn(u3, __dsub_rn(1.0, ups)), 0.5), dd));
            cd[5] = __dmul_rn(g, __dadd_rn(__dmul_rn(__dmul_rn(u3, __dadd_rn(1.0, ups)), 0.5), dd));
        }
        float *co = coef + 8 * c, *cl = coefl + 8 * c;
        for (int n = 0; n < 6; ++n) {
            const float h = __double2float_rn(cd[n]);
            co[n] = h;
            cl[n] = __double2float_rn(__dsub_rn(cd[n], (double)h));
        }
        co[6] = co[7] = cl[6] = cl[7] = 0.0f;
    }
}

__global__ void k_build_coef(const double *__restrict__ u, Metrics m, Dims d, PhysParams p, float *coef, float *coefl)
{
    build_coef_cells(u, m, d, p, coef, coefl, blockIdx.x * (size_t)blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
}

// Words 6, 7 of the coefficients (the divergence pair) after k_build_coef, as the host builds them.
__device__ __forceinline__ void build_div_cells(const Dims &d, float *coef, const float *coefl, size_t c0, size_t cs)
{
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk;
    const size_t nij = (size_t)maxi * maxj, ncell = nij * maxk;
    for (size_t c = c0; c < ncell; c += cs) {
        const int i = (int)(c % maxi) + 1;
        const int j = (int)((c / maxi) % maxj) + 1;
        const int k = (int)(c / nij) + 1;
        const int iw = i == 1 ? maxi : i - 1;
        const size_t cw = (size_t)(iw - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (k - 1));
        float dh, dl;
        fp32_div_pair(coef, coefl, maxi, nij, c, cw, j > 1, k > 1, &dh, &dl);
        coef[8 * c + 6] = dh;
        coef[8 * c + 7] = dl;
    }
}

__global__ void k_build_div(Dims d, float *coef, const float *coefl)
{
    build_div_cells(d, coef, coefl, blockIdx.x * (size_t)blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
}

// The coefficient maxima fp32_build_static keeps, from the coefficients on the device: cd[0]
// = max over faces of |A| + |B| (and, with iediff 1/2, the bound of the rebuilt top faces),
// cd[1] = max over cells of |Dh| + |Dl|; as double bits (non-negative doubles order as their
// bits).  Same expressions and order as the host, round-to-nearest intrinsics.
__device__ __forceinline__ void coef_stats_cells(const Dims &d, const PhysParams &p, const Metrics &m,
                                                 const double *__restrict__ u, const float *__restrict__ coef,
                                                 unsigned long long *cd, size_t c0, size_t cs)
{
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk, NI = d.NI;
    const size_t nij = (size_t)maxi * maxj, ncell = nij * maxk;
    double cm = 0.0, dm = 0.0;
    for (size_t c = c0; c < ncell; c += cs) {
        const float *cf = coef + 8 * c;
        for (int f = 0; f < 3; ++f) cm = fmax(cm, __dadd_rn((double)fabsf(cf[2 * f]), (double)fabsf(cf[2 * f + 1])));
        dm = fmax(dm, __dadd_rn((double)fabsf(cf[6]), (double)fabsf(cf[7])));
        if (p.iediff > 0 && p.iediff < 3) {
            const int i = (int)(c % maxi) + 1, j = (int)((c / maxi) % maxj) + 1, k = (int)(c / nij) + 1;
            if (k >= m.k1[i + (size_t)NI * j] && k < maxk) {
                const double u3 = u[2 + 3 * ((size_t)i + (size_t)(maxi + 1) * ((size_t)j + (size_t)(maxj + 1) * (size_t)(k - 1)))];
                const double g = __dmul_rn(__dmul_rn(m.dt[k], p.dphi), m.ds[j]);
                const double dv = fmax(p.diff2, m.diffmax[k + 1]);
                cm = fmax(cm, __dmul_rn(g, __dadd_rn(fabs(u3), __dmul_rn(__dmul_rn(2.0, m.rdza[k]), dv))));
            }
        }
    }
    unsigned long long a = (unsigned long long)__double_as_longlong(cm), b = (unsigned long long)__double_as_longlong(dm);
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long x = __shfl_xor_sync(0xffffffffu, a, o), y = __shfl_xor_sync(0xffffffffu, b, o);
        a = x > a ? x : a;
        b = y > b ? y : b;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(cd, a);
        atomicMax(cd + 1, b);
    }
}

// Per-tracer fixed-point scales from the device coefficient maxima (fp32_transfer_bound, fp32_scale_of).
__device__ __forceinline__ void member_scales(const unsigned long long *cd, const double *tmax, const double *gmax,
                                              const float *tref, int L, int32_t *scale)
{
    const double cmax = __longlong_as_double((long long)cd[0]), dmax = __longlong_as_double((long long)cd[1]);
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
        const double g = fmax(fmax(__dmul_rn(__dmul_rn(2.0, cmax), tmax[l]), gmax[l]), __dmul_rn(fabs((double)tref[l]), dmax));
        scale[l] = fp32_scale_of(g);
    }
}

void fp32_gtop(const Dims &d, const PhysParams &p, const std::vector<double> &blob, const double *top,
               std::vector<float> &gtop)
{
    // transfer through the surface face: dt*dphi*ds(j)*ts(l,i,j,maxk+1); per column the FP32
    // value of every tracer, then the FP64 remainders of T and S
    const int maxi = d.maxi, maxj = d.maxj, L = d.L, NI = d.NI;
    const int nj = maxj + 2, nk = d.maxk + 2;
    const double *ds = blob.data() + 6 * nj;
    const double dt = blob.data()[8 * nj + 5 * nk + 1];
    gtop.assign((size_t)(L + 2) * maxi * maxj, 0.0f);
    for (int j = 1; j <= maxj; ++j)
        for (int i = 1; i <= maxi; ++i) {
            float *g = &gtop[(size_t)(L + 2) * ((size_t)(i - 1) + (size_t)maxi * (j - 1))];
            for (int l = 0; l < L; ++l) {
                const double v = dt * p.dphi * ds[j] * top[(size_t)l + (size_t)L * ((size_t)i + (size_t)NI * j)];
                g[l] = (float)v;
                if (l < 2) g[L + l] = (float)(v - (double)g[l]);
            }
        }
}

void fp32_tracer_maxima(const Dims &d, const int32_t *k1, const double *ts, const float *gtop, std::vector<float> &tref,
                        std::vector<double> &tmax, std::vector<double> &gmax)
{
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk, L = d.L, NI = d.NI, NJ = d.NJ;
    std::vector<double> vlo(L, HUGE_VAL), vhi(L, -HUGE_VAL);
    for (int k = 1; k <= maxk; ++k)
        for (int j = 1; j <= maxj; ++j)
            for (int i = 1; i <= maxi; ++i) {
                if (k < k1[i + (size_t)NI * j]) continue;
                const double *p = ts + (size_t)L * ((size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * k));
                for (int l = 0; l < L; ++l) {
                    vlo[l] = std::min(vlo[l], p[l]);
                    vhi[l] = std::max(vhi[l], p[l]);
                }
            }
    // offset: the mid-range, rounded to 8 significant bits, for tracers (other than T and S)
    // whose wet values stay within a factor of two of each other; the transfers then carry
    // T - tref, whose FP32 rounding is smaller than T's by about max|T| / max|T - tref|
    tref.assign(L, 0.0f);
    for (int l = 2; l < L; ++l) {
        const double lo = vlo[l], hi = vhi[l];
        if (!((lo > 0.0 && lo > 0.5 * hi) || (hi < 0.0 && hi < 0.5 * lo))) continue;
        int ex = 0;
        const double f = std::frexp(0.5 * (lo + hi), &ex);
        tref[l] = (float)std::ldexp(std::nearbyint(f * 256.0), ex - 8);
    }
    // max over wet cells of |T - tref|: T - tref rounds monotonically, so the extremes decide
    tmax.assign(L, 0.0);
    for (int l = 0; l < L; ++l)
        if (vlo[l] <= vhi[l])
            tmax[l] = std::max(std::fabs(vlo[l] - (double)tref[l]), std::fabs(vhi[l] - (double)tref[l]));
    gmax.assign(L, 0.0);
    if (gtop)
        for (size_t n = 0; n < (size_t)maxi * maxj; ++n)
            for (int l = 0; l < L; ++l) gmax[l] = std::max(gmax[l], (double)std::fabs(gtop[n * (L + 2) + l]));
}

double fp32_transfer_bound(double cmax, double dmax, double tmax, double gmax, float tref)
{
    // largest transfer the step can produce: (|A|+|B|)*max|T - tref| per face, the forcing, the
    // offset's share; the isoneutral stencil and growth of max|T| are covered by 2^4 headroom
    // below the int32 range (2^26 target); a transfer above 3.5e8 (the sum of six stays inside
    // int32) sets the member's range flag
    return std::max(std::max(2.0 * cmax * tmax, gmax), std::fabs((double)tref) * dmax);
}

void fp32_scales(const Dims &d, const int32_t *k1, const double *ts, double cmax, double dmax, const float *gtop,
                 std::vector<int32_t> &scale, std::vector<float> &tref)
{
    std::vector<double> tmax, gmax;
    fp32_tracer_maxima(d, k1, ts, gtop, tref, tmax, gmax);
    scale.assign(d.L, 0);
    for (int l = 0; l < d.L; ++l) scale[l] = fp32_scale_of(fp32_transfer_bound(cmax, dmax, tmax[l], gmax[l], tref[l]));
}

// ---------------------------------------------------------------------------
// export: fill halo columns and rho of the current state (download)

__global__ void k_export_fp32(const MemberDesc md, double *cur, double *rho)
{
    const int maxi = md.maxi, maxj = md.maxj, maxk = md.maxk, L = md.L, NI = md.NI, NJ = md.NJ;
    const size_t ncell = (size_t)maxj * maxk * (maxi + 2);
    const double *zro = md.mk + 3 * (maxk + 2);
    EosCoef ec;
    for (int n = 0; n < 5; ++n) ec.ec[n] = md.ec[n];
    ec.ieos = md.ieos;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % (maxi + 2));
        const int j = (int)((c / (maxi + 2)) % maxj) + 1;
        const int k = (int)(c / ((size_t)(maxi + 2) * maxj)) + 1;
        const size_t o = (size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * k);
        const int kk = md.k1[i + NI * j];
        if (i >= 1 && i <= maxi) {
            if (k >= kk) rho[o] = eos_rn(ec, cur[o * L], cur[o * L + 1], zro[k]);
            else rho[o] = eos_rn(ec, md.ts_static[o * L], md.ts_static[o * L + 1], zro[k]);
        }
    }
}

__global__ void k_export_halo(const MemberDesc md, double *cur, double *rho)
{
    const int maxi = md.maxi, maxj = md.maxj, maxk = md.maxk, L = md.L, NI = md.NI, NJ = md.NJ;
    const size_t n = (size_t)2 * maxj * maxk;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const int side = (int)(c & 1);
        const int j = (int)((c >> 1) % maxj) + 1;
        const int k = (int)((c >> 1) / maxj) + 1;
        const int dst = side ? maxi + 1 : 0, src = side ? 1 : maxi;
        if (k < md.k1[dst + NI * j]) continue;
        const size_t od = (size_t)dst + (size_t)NI * ((size_t)j + (size_t)NJ * k);
        const size_t os = (size_t)src + (size_t)NI * ((size_t)j + (size_t)NJ * k);
        rho[od] = rho[os];
        for (int l = 0; l < L; ++l) cur[od * L + l] = cur[os * L + l];
    }
}

// Fortran layout <-> group-planar layout, every cell of the arrays
__device__ __forceinline__ void to_planar_range(double *planar, double *fortran, const Dims &d, int to, double *planar2,
                                                size_t e0, size_t es)
{
    const size_t ncell = (size_t)d.NI * d.NJ * (d.maxk + 2);
    const size_t n = ncell * d.L;
    const int ng = fp32_ngroups(d.L);
    for (size_t e = e0; e < n; e += es) {
        const int l = (int)(e % d.L);
        const size_t c = e / d.L;
        int g0 = 0, gl = 2, gp = 2, pl = 0;
        for (int h = 0; h < ng; ++h) {
            fp32_plane(d.L, h, &g0, &gl, &gp, &pl);
            if (l < g0 + gl) break;
        }
        const size_t pi = (size_t)pl * ncell + c * gp + (l - g0);
        if (to) {
            const double v = fortran[e];
            planar[pi] = v;
            if (planar2) planar2[pi] = v;
        } else {
            fortran[e] = planar[pi];
        }
    }
}

__global__ void k_to_planar(double *planar, double *fortran, Dims d, int to)
{
    to_planar_range(planar, fortran, d, to, nullptr, blockIdx.x * (size_t)blockDim.x + threadIdx.x,
                    (size_t)gridDim.x * blockDim.x);
}

// Batched device set-up of ensemble members (blockIdx.y: the member's item).
__global__ void k_setup_planar_many(const SetupItem *it)
{
    const SetupItem &I = it[blockIdx.y];
    to_planar_range(I.buf0, const_cast<double *>(I.ts_static), I.d, 1, I.buf1, blockIdx.x * (size_t)blockDim.x + threadIdx.x,
                    (size_t)gridDim.x * blockDim.x);
}
__global__ void k_setup_coef_many(const SetupItem *it)
{
    const SetupItem &I = it[blockIdx.y];
    build_coef_cells(I.u, I.m, I.d, I.p, I.coef, I.coefl, blockIdx.x * (size_t)blockDim.x + threadIdx.x,
                     (size_t)gridDim.x * blockDim.x);
}
__global__ void k_setup_div_many(const SetupItem *it)
{
    const SetupItem &I = it[blockIdx.y];
    build_div_cells(I.d, I.coef, I.coefl, blockIdx.x * (size_t)blockDim.x + threadIdx.x, (size_t)gridDim.x * blockDim.x);
}
__global__ void k_setup_stats_many(const SetupItem *it)
{
    const SetupItem &I = it[blockIdx.y];
    coef_stats_cells(I.d, I.p, I.m, I.u, I.coef, I.cd, blockIdx.x * (size_t)blockDim.x + threadIdx.x,
                     (size_t)gridDim.x * blockDim.x);
}
// order key of a double: unsigned comparison of keys is the comparison of the values
__device__ __forceinline__ unsigned long long order_key_u(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_value(unsigned long long k)
{
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

// the extremes of every tracer over the member's wet interior cells: ext[2l] the largest key,
// ext[2l+1] the largest inverted key (the smallest value); shared-memory maxima per block
__global__ void __launch_bounds__(256) k_setup_extrema_many(const SetupItem *it)
{
    __shared__ unsigned long long sh[2 * kFp32MaxL];
    const SetupItem &I = it[blockIdx.y];
    const int L = I.d.L, maxi = I.d.maxi, maxj = I.d.maxj, NI = I.d.NI, NJ = I.d.NJ;
    for (int e = threadIdx.x; e < 2 * L; e += blockDim.x) sh[e] = 0ull;
    __syncthreads();
    const size_t nij = (size_t)maxi * maxj, n = nij * I.d.maxk * L;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(e % L);
        const size_t c = e / L;
        const int i = (int)(c % maxi) + 1, j = (int)((c / maxi) % maxj) + 1, k = (int)(c / nij) + 1;
        if (k < I.m.k1[i + (size_t)NI * j]) continue;
        const double v = I.ts_static[(size_t)l + (size_t)L * ((size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * k))];
        const unsigned long long key = order_key_u(v);
        atomicMax(&sh[2 * l], key);
        atomicMax(&sh[2 * l + 1], ~key);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * L; e += blockDim.x)
        if (sh[e]) atomicMax(&I.ext[e], sh[e]);
}

// the offsets and maxima of fp32_tracer_maxima from the extremes, then the scales
__global__ void k_setup_scales_many(const SetupItem *it)
{
    const SetupItem &I = it[blockIdx.x];
    const int L = I.d.L;
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
        const unsigned long long kh = I.ext[2 * l], kl = I.ext[2 * l + 1];
        float tr = 0.0f;
        double tm = 0.0;
        if (kh != 0ull) {   // the tracer has wet cells
            const double hi = key_value(kh), lo = key_value(~kl);
            if (l >= 2 && ((lo > 0.0 && lo > __dmul_rn(0.5, hi)) || (hi < 0.0 && hi < __dmul_rn(0.5, lo)))) {
                int ex = 0;
                const double f = frexp(__dmul_rn(0.5, __dadd_rn(lo, hi)), &ex);
                tr = (float)ldexp(rint(__dmul_rn(f, 256.0)), ex - 8);
            }
            tm = fmax(fabs(__dadd_rn(lo, -(double)tr)), fabs(__dadd_rn(hi, -(double)tr)));
        }
        I.tref[l] = tr;
        I.tmax[l] = tm;
    }
    __syncthreads();
    member_scales(I.cd, I.tmax, I.gmax, I.tref, L, I.scale);
}

int fp32_setup_many(const SetupItem *items_dev, int n, size_t max_elems, size_t max_cells, cudaStream_t s)
{
    for (int q0 = 0; q0 < n; q0 += 65535) {
        const int nq = std::min(n - q0, 65535);
        const SetupItem *it = items_dev + q0;
        const int pb = (int)std::max<size_t>(1, std::min<size_t>((max_elems + 255) / 256, 128));
        const int cb = (int)std::max<size_t>(1, std::min<size_t>((max_cells + 255) / 256, 64));
        k_setup_planar_many<<<dim3(pb, nq), 256, 0, s>>>(it);
        k_setup_coef_many<<<dim3(cb, nq), 256, 0, s>>>(it);
        k_setup_div_many<<<dim3(cb, nq), 256, 0, s>>>(it);
        k_setup_stats_many<<<dim3(cb, nq), 256, 0, s>>>(it);
        k_setup_extrema_many<<<dim3(pb, nq), 256, 0, s>>>(it);
        k_setup_scales_many<<<nq, 64, 0, s>>>(it);
        count_launches(6);
    }
    return launch_status();
}

static int planar_copy(double *planar, double *fortran, const Dims &d, int to, cudaStream_t s)
{
    const size_t n = (size_t)d.NI * d.NJ * (d.maxk + 2) * d.L;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 8192);
    k_to_planar<<<std::max(1, blocks), 256, 0, s>>>(planar, fortran, d, to);
    count_launches(1);
    return launch_status();
}

int fp32_to_planar(double *planar, const double *fortran, const Dims &d, cudaStream_t s)
{
    return planar_copy(planar, const_cast<double *>(fortran), d, 1, s);
}

int fp32_from_planar(double *fortran, const double *planar, const Dims &d, cudaStream_t s)
{
    return planar_copy(const_cast<double *>(planar), fortran, d, 0, s);
}

// The current state in Fortran layout (halo columns filled) and rho of it.
int fp32_export(const MemberDesc &md, const double *planar, double *cur, double *rho, cudaStream_t s)
{
    Dims d{md.maxi, md.maxj, md.maxk, md.L, md.NI, md.NJ};
    if (fp32_from_planar(cur, planar, d, s)) return GB_GO_ECUDA;
    const size_t ncell = (size_t)md.maxj * md.maxk * (md.maxi + 2);
    const int blocks = (int)std::min<size_t>((ncell + 255) / 256, 4096);
    k_export_fp32<<<blocks, 256, 0, s>>>(md, const_cast<double *>(cur), rho);
    k_export_halo<<<std::max(1, (int)std::min<size_t>((2 * (size_t)md.maxj * md.maxk + 255) / 256, 1024)), 256, 0, s>>>(
        md, const_cast<double *>(cur), rho);
    count_launches(2);
    return launch_status();
}

}  // namespace gbgo

// ---------------------------------------------------------------------------
// single grid = a batch of one member

namespace gbgo {

static int cuda_ok(cudaError_t e) { return e == cudaSuccess ? 0 : (e == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA); }

struct Fp32Host {
    Fp32Data data;
    Dims d{};
    PhysParams p{};
    std::vector<double> blob;
    std::vector<int32_t> k1;
    std::vector<double> ts1_host;     // state used to pick the transfer scales
    const int32_t *k1_dev = nullptr;
    Metrics m{};                      // the handle's device metrics (iediff reads dza, diffmax, ediff1)
    const double *u_dev = nullptr;    // the handle's device velocities (iediff)
    bool have_state = false, have_vel = false;
    double dt = 0.0;
};

int fp32_member_init(Fp32Member *f, const Dims &d, const PhysParams &p, const Metrics &m, const std::vector<double> &blob,
                     const int32_t *k1_host, cudaStream_t s, std::string &msg)
{
    if (d.L > kFp32MaxL) {
        msg = "GB_GO_FP32FLUX supports at most 32 tracers per grid";
        return GB_GO_ERANGE;
    }
    const int nj = d.maxj + 2, nk = d.maxk + 2;
    const double *dtp = blob.data() + 8 * nj + 5 * nk;
    for (int k = 2; k <= d.maxk; ++k)
        if (dtp[k] != dtp[1]) {
            msg = "GB_GO_FP32FLUX needs the same dt on every level (the transfers are shared between levels)";
            return GB_GO_EUNSUPPORTED;
        }
    if (d.maxk > kMaxK) {
        msg = "GB_GO_FP32FLUX supports at most 64 levels";
        return GB_GO_ERANGE;
    }
    PatchPlan plan;
    if (fp32_plan_patches(d, k1_host, 0, 0, plan) != GB_GO_OK) {
        msg = "no patch shape fits the FP32-flux kernel limits";
        return GB_GO_ERANGE;
    }
    Fp32Host *h = new Fp32Host();
    h->d = d;
    h->p = p;
    h->blob = blob;
    h->k1.assign(k1_host, k1_host + (size_t)d.NI * d.NJ);
    h->k1_dev = m.k1;
    h->m = m;
    h->dt = dtp[1];
    Fp32Data &D = h->data;
    D.max_slots = plan.max_slots;
    const size_t ncell = (size_t)d.maxi * d.maxj * d.maxk;
    cudaError_t e = cudaMalloc(&D.coef, 8 * ncell * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&D.coefl, 8 * ncell * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&D.plan_buf[0], fp32_planar_size(d) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.plan_buf[1], fp32_planar_size(d) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.rvol, (size_t)d.maxj * d.maxk * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.gtop, (size_t)(d.L + 2) * d.maxi * d.maxj * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&D.scale, (size_t)d.L * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&D.tref, (size_t)d.L * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(D.tref, 0, (size_t)d.L * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&D.gmax, (size_t)d.L * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(D.gmax, 0, (size_t)d.L * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&D.mk, 6 * (size_t)nk * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.mj, 3 * (size_t)nj * sizeof(double));
    if (e == cudaSuccess && p.imld == 1) e = cudaMalloc(&D.rhos, (size_t)d.maxi * d.maxj * sizeof(double));
    if (e == cudaSuccess && p.imld == 1) e = cudaMemset(D.rhos, 0, (size_t)d.maxi * d.maxj * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.status, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&D.dev, sizeof(MemberDesc));
    if (e == cudaSuccess) e = cudaMalloc(&D.step_ctr, sizeof(long long));
    const int ng = fp32_ngroups(d.L);
    D.nitems = (int)plan.offset.size() * ng;
    D.cocap = 0;
    for (int j = 1; j <= d.maxj; ++j)
        for (int i = 1; i <= d.maxi; ++i) D.cocap += k1_host[i + (size_t)d.NI * j] <= d.maxk;
    if (e == cudaSuccess) e = cudaMalloc(&D.work, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(D.work, 0, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&D.s2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&D.fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&D.join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&D.ptab, std::max<size_t>(1, plan.words.size()) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&D.colist, std::max(1, D.cocap) * sizeof(int2));
    if (e == cudaSuccess) e = cudaMalloc(&D.cocount, 6 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(D.cocount, 0, 6 * sizeof(int));
    D.mapcap = std::max(1, D.cocap) * fp32_co_slots(d.L);
    if (e == cudaSuccess) e = cudaMalloc(&D.colog, std::max(1, D.cocap) * kCoLogSlotBytes);
    if (e == cudaSuccess) e = cudaMalloc(&D.comap, (size_t)D.mapcap * sizeof(int2));
    if (e == cudaSuccess) e = cudaMalloc(&D.items, std::max(1, D.nitems) * sizeof(int4));
    if ((p.diso || p.iediff) && e == cudaSuccess) {
        e = cudaMalloc(&D.stencil, (size_t)kStencilWords * ncell * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc(&D.stencil_list, sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(D.stencil_list, 0, sizeof(int));
    }
    if (e == cudaSuccess) {
        // the T-S items of the patches, then the other (patch, group) items
        std::vector<int4> it;
        for (size_t n = 0; n < plan.offset.size(); ++n) it.push_back(make_int4(0, plan.offset[n], 0, 0));
        for (size_t n = 0; n < plan.offset.size(); ++n)
            for (int g = 1; g < ng; ++g) it.push_back(make_int4(0, plan.offset[n], g, 0));
        D.n_ts = (int)plan.offset.size();
        if (!plan.words.empty())
            e = cudaMemcpyAsync(D.ptab, plan.words.data(), plan.words.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && !it.empty())
            e = cudaMemcpyAsync(D.items, it.data(), it.size() * sizeof(int4), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(D.status, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(D.gtop, 0, (size_t)(d.L + 2) * d.maxi * d.maxj * sizeof(float), s);
    f->impl = h;
    f->ready = true;
    if (e != cudaSuccess) {
        msg = cudaGetErrorString(e);
        return cuda_ok(e);
    }
    return 0;
}

static Fp32Host *host_of(Fp32Member *f) { return static_cast<Fp32Host *>(f->impl); }

void fp32_member_free(Fp32Member *f)
{
    if (!f || !f->impl) return;
    Fp32Host *h = host_of(f);
    Fp32Data &D = h->data;
    cudaFree(D.coef); cudaFree(D.coefl); cudaFree(D.plan_buf[0]); cudaFree(D.plan_buf[1]); cudaFree(D.rvol); cudaFree(D.gtop); cudaFree(D.scale); cudaFree(D.tref); cudaFree(D.gmax); cudaFree(D.mk); cudaFree(D.mj);
    cudaFree(D.status); cudaFree(D.dev); cudaFree(D.items); cudaFree(D.step_ctr); cudaFree(D.ptab); cudaFree(D.work);
    cudaFree(D.colist); cudaFree(D.cocount); cudaFree(D.colog); cudaFree(D.comap); cudaFree(D.stencil); cudaFree(D.stencil_list); cudaFree(D.rhos);
    if (D.s2) cudaStreamDestroy(D.s2);
    if (D.fork) cudaEventDestroy(D.fork);
    if (D.join) cudaEventDestroy(D.join);
    delete h;
    f->impl = nullptr;
    f->ready = false;
}

static int upload_scales(Fp32Host *h, cudaStream_t s)
{
    if (!h->have_state || !h->have_vel) return 0;
    std::vector<int32_t> sc;
    std::vector<float> tr;
    fp32_scales(h->d, h->k1.data(), h->ts1_host.data(), h->data.cmax, h->data.dmax, h->data.gtop_host_unscaled.data(),
                sc, tr);
    h->data.scale_host = sc;
    h->data.tref_host = tr;
    return cuda_ok(cudaMemcpyAsync(h->data.scale, h->data.scale_host.data(), sc.size() * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, s)) ||
           cuda_ok(cudaMemcpyAsync(h->data.tref, h->data.tref_host.data(), tr.size() * sizeof(float),
                                   cudaMemcpyHostToDevice, s)) ||
           cuda_ok(cudaStreamSynchronize(s));
}

int fp32_member_upload(Fp32Member *f, const double *ts1_host, const double *ts_host, const double *ts1_dev, cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    if (fp32_to_planar(h->data.plan_buf[0], ts1_dev, h->d, s) || fp32_to_planar(h->data.plan_buf[1], ts1_dev, h->d, s))
        return GB_GO_ECUDA;
    const size_t nts = (size_t)h->d.L * h->d.NI * h->d.NJ * (h->d.maxk + 2);
    h->ts1_host.assign(ts1_host, ts1_host + nts);
    h->have_state = true;
    h->data.steps = 0;
    const size_t ntop = (size_t)h->d.L * h->d.NI * h->d.NJ;
    int r = fp32_member_set_top(f, ts_host + ntop * (h->d.maxk + 1), s);
    if (r) return r;
    return upload_scales(h, s);
}

int fp32_member_reload(Fp32Member *f, const double *ts1_dev, cudaStream_t s)
{
    // the state rewritten on the device (the BIOGEM coupling): both step buffers from ts1, the
    // step parity restarts; the forcing transfers and the fixed-point scales are kept (the
    // scales follow the state through the rescaling of the steps)
    Fp32Host *h = host_of(f);
    if (fp32_to_planar(h->data.plan_buf[0], ts1_dev, h->d, s) || fp32_to_planar(h->data.plan_buf[1], ts1_dev, h->d, s))
        return GB_GO_ECUDA;
    h->data.steps = 0;
    return cuda_ok(cudaStreamSynchronize(s));
}

__global__ void k_surface_rho(const double *rho, double *rhos, int maxi, int maxj, int maxk, int NI, int NJ)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= maxi * maxj) return;
    const int i = c % maxi + 1, j = c / maxi + 1;
    rhos[c] = rho[(size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * maxk)];
}

int fp32_member_set_mixed_layer(Fp32Member *f, const double *mldketau, double *mld, int32_t *mldk, const double *mlddec,
                                const double *mlddecd, const double *rho, cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    Fp32Data &D = h->data;
    if (h->p.imld != 1 || !D.rhos) return GB_GO_EINVAL;
    MemberDesc &md = D.host;
    md.imld = 1;
    md.mldpebuoycoeff = h->p.mldpebuoycoeff;
    md.mlddec = mlddec;
    md.mlddecd = mlddecd;
    md.mldketau = mldketau;
    md.mld = mld;
    md.mldk = mldk;
    md.rhos = D.rhos;
    D.desc_valid = false;
    const int ncol = h->d.maxi * h->d.maxj;
    k_surface_rho<<<(ncol + 127) / 128, 128, 0, s>>>(rho, D.rhos, h->d.maxi, h->d.maxj, h->d.maxk, h->d.NI, h->d.NJ);
    count_launches(1);
    if (launch_status()) return GB_GO_ECUDA;
    return cuda_ok(cudaStreamSynchronize(s));
}

int fp32_member_set_top(Fp32Member *f, const double *top_host, cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    fp32_gtop(h->d, h->p, h->blob, top_host, h->data.gtop_host_unscaled);
    int r = cuda_ok(cudaMemcpyAsync(h->data.gtop, h->data.gtop_host_unscaled.data(),
                                    h->data.gtop_host_unscaled.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    if (r) return r;
    return cuda_ok(cudaStreamSynchronize(s));
}

int fp32_member_set_velocity(Fp32Member *f, const double *u_host, const double *u_dev, const Metrics &m,
                              cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    if (u_dev) h->u_dev = u_dev;
    if (h->have_vel && u_dev) {
        // later velocity fields: coefficients on the device; the fixed-point scales follow
        // through the rescaling of the steps
        Fp32Data &D = h->data;
        const size_t ncell = (size_t)h->d.maxi * h->d.maxj * h->d.maxk;
        const int blocks = (int)std::min<size_t>((ncell + 255) / 256, 8192);
        k_build_coef<<<std::max(1, blocks), 256, 0, s>>>(u_dev, m, h->d, h->p, D.coef, D.coefl);
        k_build_div<<<std::max(1, blocks), 256, 0, s>>>(h->d, D.coef, D.coefl);
        count_launches(2);
        return launch_status();
    }
    Fp32Static st;
    fp32_build_static(h->d, h->p, h->blob, h->k1.data(), u_host, st);
    Fp32Data &D = h->data;
    D.cmax = st.cmax;
    D.dmax = st.dmax;
    cudaError_t e = cudaMemcpyAsync(D.coef, st.coef.data(), st.coef.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(D.coefl, st.coefl.data(), st.coefl.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(D.rvol, st.rvol.data(), st.rvol.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(D.mk, st.mk.data(), st.mk.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(D.mj, st.mj.data(), st.mj.size() * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_ok(e);
    h->have_vel = true;
    return upload_scales(h, s);
}

int fp32_member_step(Fp32Member *f, double *ts_buf[2], int *cur, double *rho, const double *ts_static, double *cost,
                     int32_t *icosd, unsigned long long *diag, int *slot, int nsteps, cudaStream_t s)
{
    (void)ts_buf;   // the FP32-flux state lives in its own group-planar buffers
    (void)rho;      // rho is computed on export
    Fp32Host *h = host_of(f);
    Fp32Data &D = h->data;
    if (!h->have_state || !h->have_vel) return GB_GO_ENOTREADY;
    if (!D.desc_valid) {
        MemberDesc &md = D.host;
        md.maxi = h->d.maxi; md.maxj = h->d.maxj; md.maxk = h->d.maxk; md.L = h->d.L; md.NI = h->d.NI; md.NJ = h->d.NJ;
        md.diso = h->p.diso; md.ieos = h->p.ieos; md.iconv = h->p.iconv;
        md.iediff = h->p.iediff; md.ediffpow2i = h->p.ediffpow2i;
        md.diff2 = h->p.diff2; md.ediff0 = h->p.ediff0; md.ediffpow2 = h->p.ediffpow2;
        md.u = h->u_dev; md.ediff1 = h->m.ediff1; md.dza = h->m.dza; md.diffmax = h->m.diffmax;
        md.parity = 0;
        md.stop_step = (long long)1 << 62;
        md.origin = 0;
        md.dt = h->dt; md.dphi = h->p.dphi; md.rdphi = h->p.rdphi; md.diff1 = h->p.diff1;
        for (int n = 0; n < 5; ++n) md.ec[n] = h->p.ec[n];
        md.dsc = h->p.dsc;
        md.buf[0] = D.plan_buf[0];
        md.buf[1] = D.plan_buf[1];
        md.ts_static = ts_static;
        md.coef = D.coef; md.coefl = D.coefl; md.rvol = D.rvol; md.gtop = D.gtop; md.k1 = h->k1_dev; md.scale = D.scale; md.tref = D.tref; md.gmax = D.gmax;
        md.mk = D.mk; md.mj = D.mj; md.cost = cost; md.icosd = icosd;
        md.ptab = D.ptab;
        md.status = D.status;
        md.diag = diag;
        md.stencil = D.stencil;
        if (h->p.imld == 1 && !md.rhos) return GB_GO_ENOTREADY;   // fp32_member_set_mixed_layer first
        if (cudaMemcpyAsync(D.dev, &md, sizeof(md), cudaMemcpyHostToDevice, s) != cudaSuccess) return GB_GO_ECUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return GB_GO_ECUDA;
        D.desc_valid = true;
    }
    // buffer and diag slot of step n are (n & 1): the ping-pong starts at buffer 0 on upload
    D.step_host = D.steps;
    if (cudaMemcpyAsync(D.step_ctr, &D.step_host, sizeof(long long), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return GB_GO_ECUDA;
    for (int n = 0; n < nsteps; ++n) {
        const long long step = D.steps + n;
        if (cudaMemsetAsync(diag + 2 * (step & 1), 0, 2 * sizeof(unsigned long long), s) != cudaSuccess)
            return GB_GO_ECUDA;
        Fp32Batch bt;
        bt.descs = D.dev;
        bt.items = D.items;
        bt.n_ts = D.n_ts;
        bt.n_bgc = D.nitems - D.n_ts;
        bt.max_slots = D.max_slots;
        bt.kmax = h->d.maxk;
        bt.lmax = h->d.L;
        bt.work = D.work;
        bt.colist = D.colist;
        bt.cocount = D.cocount;
        bt.cocap = D.cocap;
        bt.colog = D.colog;
        bt.comap = D.comap;
        bt.mapcap = D.mapcap;
        bt.iso = D.stencil != nullptr;
        bt.co_general = !fp32_co_fast(h->p.iconv, h->p.ieos, h->p.imld, h->d.maxk);
        if (D.stencil) {
            bt.stencil_list = D.stencil_list;
            bt.n_stencil = 1;
            bt.stencil_blocks = fp32_stencil_blocks((size_t)h->d.maxi * h->d.maxj * h->d.maxk);
        }
        int r = D.nitems ? fp32_launch(bt, D.step_ctr, n, s, D.s2, D.fork, D.join) : 0;
        if (!r) r = fp32_rescale(D.dev, 1, s);
        if (r) return r;
        count_launches((D.nitems ? fp32_launches_per_step(bt) : 0) + 1);
    }
    D.steps += nsteps;
    *cur = (int)(D.steps & 1);
    *slot = (int)(D.steps & 1);
    return 0;
}

int fp32_member_fortran(Fp32Member *f, double *dst, cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    return fp32_from_planar(dst, h->data.plan_buf[h->data.steps & 1], h->d, s);
}

// rho of the current state without the Fortran-layout export of the tracers: interior cells
// from T and S of the group-planar state (wet) or of the uploaded state (dry), wet halo cells
// from their periodic source column -- the values k_export_fp32 and k_export_halo give
__global__ void k_rho_fp32(const MemberDesc md, const double *planar, double *rho)
{
    const int maxi = md.maxi, maxj = md.maxj, maxk = md.maxk, L = md.L, NI = md.NI, NJ = md.NJ;
    const size_t ncell = (size_t)maxj * maxk * (maxi + 2);
    const double *zro = md.mk + 3 * (maxk + 2);
    EosCoef ec;
    for (int n = 0; n < 5; ++n) ec.ec[n] = md.ec[n];
    ec.ieos = md.ieos;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % (maxi + 2));
        const int j = (int)((c / (maxi + 2)) % maxj) + 1;
        const int k = (int)(c / ((size_t)(maxi + 2) * maxj)) + 1;
        const size_t o = (size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * k);
        const int kk = md.k1[i + NI * j];
        if (i >= 1 && i <= maxi) {
            if (k >= kk) rho[o] = eos_rn(ec, planar[o * 2], planar[o * 2 + 1], zro[k]);
            else rho[o] = eos_rn(ec, md.ts_static[o * L], md.ts_static[o * L + 1], zro[k]);
        } else if (k >= kk) {
            const int src = i == 0 ? maxi : 1;
            const size_t os = (size_t)src + (size_t)NI * ((size_t)j + (size_t)NJ * k);
            rho[o] = eos_rn(ec, planar[os * 2], planar[os * 2 + 1], zro[k]);
        }
    }
}

static MemberDesc export_desc(Fp32Host *h, const double *ts_static)
{
    MemberDesc md{};
    md.maxi = h->d.maxi; md.maxj = h->d.maxj; md.maxk = h->d.maxk; md.L = h->d.L; md.NI = h->d.NI; md.NJ = h->d.NJ;
    md.ieos = h->p.ieos;
    for (int n = 0; n < 5; ++n) md.ec[n] = h->p.ec[n];
    md.ts_static = ts_static;
    md.mk = h->data.mk;
    md.k1 = h->k1_dev;
    return md;
}

static int member_status(Fp32Data &D, cudaStream_t s)
{
    unsigned int st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, D.status, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        tl_cuda_error = e;
        return GB_GO_ECUDA;
    }
    if (st & 1u) return GB_GO_ENONFINITE;
    if (st & 6u) return GB_GO_ERANGE;
    return 0;
}

int fp32_member_rho(Fp32Member *f, double *rho, const double *ts_static, cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    Fp32Data &D = h->data;
    const MemberDesc md = export_desc(h, ts_static);
    const size_t ncell = (size_t)md.maxj * md.maxk * (md.maxi + 2);
    k_rho_fp32<<<(int)std::min<size_t>((ncell + 255) / 256, 4096), 256, 0, s>>>(md, D.plan_buf[D.steps & 1], rho);
    count_launches(1);
    if (launch_status()) return GB_GO_ECUDA;
    return member_status(D, s);
}

int fp32_member_export(Fp32Member *f, double *ts_cur, double *rho, const double *ts_static, cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    Fp32Data &D = h->data;
    const MemberDesc md = export_desc(h, ts_static);
    int r = fp32_export(md, D.plan_buf[D.steps & 1], ts_cur, rho, s);
    if (r) return r;
    return member_status(D, s);
}

}  // namespace gbgo
