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
// Mapping: a CTA of 128 threads takes work items (member, TX x TY column tile)
// from a host-built list.  Each level k of a tile: cp.async brings the FP64 slab
// of level k+2 (with a one-cell halo) into shared memory while threads (one per
// column) compute the integer / double-float transfers of level k from scaled
// FP32 slabs of levels k and k+1; then the tile's FP64 state of level k is
// updated row by row with coalesced loads and stores.
#include "gb_fp32.h"
#include "co_column.cuh"
#include "../../include/gb_goldstein.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

namespace gbgo {

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

// FP64 value as a double-float (hi truncated, lo the rest)
__device__ __forceinline__ dflt df_split(double x)
{
    const float h = d2f_scaled(x, 0);
    return {h, d2f_scaled(x - f2d_scaled(h, 0), 0)};
}

__device__ __forceinline__ float eos_f(const float ec[5], float t, float s)
{
    return ec[0] * t + ec[1] * s + ec[2] * (t * t) + ec[3] * (t * t * t);
}

// column view used by the exact co on the FP64 state
struct Fp32Col {
    double *w;
    const double *stat;
    int L, NI, NJ, i, j, k1;
    double rho[kMaxK + 1];
    __device__ size_t idx(int l, int lev) const
    {
        return (size_t)l + (size_t)L * ((size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * (size_t)lev));
    }
    __device__ double T(int l, int lev) const { return lev >= k1 ? w[idx(l, lev)] : stat[idx(l, lev)]; }
    __device__ void setT(int l, int lev, double v) { w[idx(l, lev)] = v; }
    __device__ double &R(int lev) { return rho[lev]; }
};

// ---------------------------------------------------------------------------
// the step kernel

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Tracers per march of a tile: shared memory (and so CTAs per SM) scales with it.
constexpr int kGroup = 8;

// Dynamic shared memory of one work item, for tracer groups of up to kGroup
// (byte offsets, 16-byte aligned).  ncp = nc | 1 (odd pitch: conflict-free).
struct Fp32Smem {
    int stage;   // double[nc*G]      FP64 slab of one tracer group in flight (cp.async)
    int f;       // float[3][G][ncp]  scaled FP32 slabs of levels k, k+1, k+2 (tracer-major)
    int fl;      // float[3][2][ncp]  lo parts of T and S for the three slabs
    int qb;      // int[G][nin]       bottom-face carry of the group's tracers
    int qbd;     // float[2][2][nin]  the same for T and S as double-floats
    int k1t;     // int[nc]           k1 with a one-cell halo
    int total;
};

__host__ __device__ inline Fp32Smem fp32_smem_layout(int TX, int TY, int L)
{
    const int nc = (TX + 2) * (TY + 2), ncp = nc | 1, nin = TX * TY;
    const int G = L < kGroup ? L : kGroup;
    Fp32Smem s;
    int o = 0;
    s.stage = o; o += (nc * G * 8 + 15) & ~15;
    s.f = o; o += (3 * G * ncp * 4 + 15) & ~15;
    s.fl = o; o += (3 * 2 * ncp * 4 + 15) & ~15;
    s.qb = o; o += (G * nin * 4 + 15) & ~15;
    s.qbd = o; o += (4 * nin * 4 + 15) & ~15;
    s.k1t = o; o += (nc * 4 + 15) & ~15;
    s.total = o;
    return s;
}

__global__ void __launch_bounds__(kFp32Threads, 5)
k_step_fp32(const MemberDesc *__restrict__ mds, const int4 *__restrict__ items, int nitems,
            const long long *__restrict__ step_ctr, int rel)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ int s_kstart;
    __shared__ int s_scale[kFp32MaxL];
    __shared__ unsigned int s_gmax[kFp32MaxL];
    const int t = threadIdx.x;
    const int warp = t >> 5, lane = t & 31, nwarp = blockDim.x >> 5;
    const long long step = *step_ctr + rel;
    // every 4th step the per-tracer transfer maxima are gathered to re-target the scales
    const bool track = (step & 3) == 0;

    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int4 item = items[it];
        const MemberDesc &md = mds[item.x];
        if (step >= md.stop_step) continue;   // uniform over the CTA
        const int TX = item.w & 0xff, TY = (item.w >> 8) & 0xff;
        const int i0 = item.y, j0 = item.z;
        // the member's first tile clears the diagnostics slot of the next step
        if (i0 == 1 && j0 == 1 && t == 0) {
            unsigned long long *dn = md.diag + 2 * ((step + 1) & 1);
            dn[0] = 0ull;
            dn[1] = 0ull;
        }
        const int maxi = md.maxi, maxj = md.maxj, maxk = md.maxk, L = md.L, NI = md.NI, NJ = md.NJ;
        const int nx = TX + 2, ny = TY + 2, nc = nx * ny, ncp = nc | 1, nin = TX * TY;
        const Fp32Smem lay = fp32_smem_layout(TX, TY, L);
        double *stage = reinterpret_cast<double *>(smraw + lay.stage);
        float *Fb = reinterpret_cast<float *>(smraw + lay.f);
        float *FLb = reinterpret_cast<float *>(smraw + lay.fl);
        int *QB = reinterpret_cast<int *>(smraw + lay.qb);
        float *QBD = reinterpret_cast<float *>(smraw + lay.qbd);
        int *k1t = reinterpret_cast<int *>(smraw + lay.k1t);
        const int par = (int)((step + md.parity) & 1);
        const double *__restrict__ R = md.buf[par];
        double *__restrict__ W = md.buf[par ^ 1];
        const double *mk = md.mk;
        const double *mj = md.mj;
        const int mkn = maxk + 2, mjn = maxj + 2;
        const int Gmax = L < kGroup ? L : kGroup;

        // k1 tile with a one-column halo (periodic in i), land outside the grid
        if (t == 0) s_kstart = 1 << 20;
        for (int e = t; e < nc; e += blockDim.x) {
            const int c = e % nx, r = e / nx;
            int gi = i0 - 1 + c, gj = j0 - 1 + r;
            int v = maxk + 1;
            if (gj <= maxj + 1 && gi <= maxi + 1) {
                if (gi == 0) gi = maxi;
                else if (gi == maxi + 1) gi = 1;
                v = md.k1[gi + NI * gj];
            }
            k1t[e] = v;
        }
        for (int l = t; l < L; l += blockDim.x) {
            s_scale[l] = md.scale[l];
            s_gmax[l] = 0u;
        }
        __syncthreads();
        const int ti = t % TX, tj = t / TX;
        const int i = i0 + ti, j = j0 + tj;
        const bool inside = (t < nin) && (i <= maxi) && (j <= maxj);
        const int cidx = (tj + 1) * nx + (ti + 1);
        const int cell = tj * TX + ti;
        const int k1c = inside ? k1t[cidx] : maxk + 1;
        if (inside && k1c <= maxk) atomicMin(&s_kstart, k1c);
        __syncthreads();
        const int kstart = s_kstart;
        if (kstart > maxk) {
            __syncthreads();
            continue;
        }

        float ecf[5];
        for (int n = 0; n < 5; ++n) ecf[n] = (float)md.ec[n];
        float rho_prev = 0.0f;
        bool unstable = false;
        float gmax = 0.0f;
        bool nonfinite = false;
        double dmax_l = 0.0;
        unsigned limps_l = 0;

        for (int g0 = 0; g0 < L; g0 += Gmax) {
            const int gl = (L - g0) < Gmax ? (L - g0) : Gmax;
            const bool ts_group = (g0 == 0);

            // Each thread owns a fixed set of slab elements (rows by warp, elements of the
            // row by lane).  pump(cv, nx_lev): convert the thread's own staged elements of
            // level cv into FP32 slot cv % 3 (its own cp.async copies are complete after
            // cp.async.wait_all, so no block barrier guards the stage), then cp.async its
            // elements of level nx_lev into the stage.  Land cells are zero-filled instead
            // of copied: their values only ever meet zero coefficients.
            auto pump = [&](int cv, int nx_lev) {
                float *F = Fb + (size_t)(cv % 3) * gl * ncp;
                float *FL = FLb + (size_t)(cv % 3) * 2 * ncp;
                const int rowlen = nx * gl;
                const int dc = 32 / gl, dl = 32 % gl;
                for (int r = warp; r < ny; r += nwarp) {
                    const int gj = j0 - 1 + r;
                    double *Srow = stage + (size_t)r * rowlen;
                    const int *krow = k1t + r * nx;
                    const bool rowok = gj <= maxj + 1;
                    const size_t rowbase = (size_t)NI * ((size_t)gj + (size_t)NJ * (size_t)nx_lev);
                    int c = lane / gl, q = lane % gl;
                    for (int e = lane; e < rowlen; e += 32) {
                        if (cv >= 0) {
                            const double x = Srow[e];
                            const int sl = s_scale[g0 + q];
                            const float h = d2f_scaled(x, sl);
                            const int cc = r * nx + c;
                            F[q * ncp + cc] = h;
                            if (ts_group && q < 2) FL[q * ncp + cc] = d2f_scaled(x - f2d_scaled(h, sl), sl);
                        }
                        if (nx_lev >= 0) {
                            int gi = i0 - 1 + c;
                            if (rowok && gi <= maxi + 1 && nx_lev >= krow[c]) {
                                if (gi == 0) gi = maxi;
                                else if (gi == maxi + 1) gi = 1;
                                cp_async8(Srow + e, R + ((size_t)gi + rowbase) * L + g0 + q);
                            } else {
                                Srow[e] = 0.0;
                            }
                        }
                        c += dc;
                        q += dl;
                        if (q >= gl) {
                            q -= gl;
                            c += 1;
                        }
                    }
                }
                cp_async_commit();
            };

            for (int e = t; e < gl * nin; e += blockDim.x) QB[e] = 0;
            if (ts_group)
                for (int e = t; e < 4 * nin; e += blockDim.x) QBD[e] = 0.0f;
            // prologue: slabs kstart and kstart+1 converted, kstart+2 in flight
            pump(-1, kstart);
            cp_async_wait_all();
            pump(kstart, kstart + 1 <= maxk ? kstart + 1 : -1);
            if (kstart + 1 <= maxk) {
                cp_async_wait_all();
                pump(kstart + 1, kstart + 2 <= maxk ? kstart + 2 : -1);
            }
            __syncthreads();

            for (int k = kstart; k <= maxk; ++k) {
                const float *Sk = Fb + (size_t)(k % 3) * gl * ncp;
                const float *Su = Fb + (size_t)((k + 1) % 3) * gl * ncp;
                const float *SkL = FLb + (size_t)(k % 3) * 2 * ncp;
                const float *SuL = FLb + (size_t)((k + 1) % 3) * 2 * ncp;
                if (inside && k >= k1c) {
                    const size_t cl = (size_t)(i - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (size_t)(k - 1));
                    const float *cf = md.coef + 12 * cl;
                    const int iw = (i == 1) ? maxi : i - 1;
                    const float *cw = md.coef + 12 * ((size_t)(iw - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (size_t)(k - 1)));
                    const dflt AeX = {__ldg(cf + 0), __ldg(cf + 6)}, BeX = {__ldg(cf + 1), __ldg(cf + 7)};
                    const dflt AnX = {__ldg(cf + 2), __ldg(cf + 8)}, BnX = {__ldg(cf + 3), __ldg(cf + 9)};
                    const dflt AaX = {__ldg(cf + 4), __ldg(cf + 10)}, BaX = {__ldg(cf + 5), __ldg(cf + 11)};
                    const dflt AwX = {__ldg(cw + 0), __ldg(cw + 6)}, BwX = {__ldg(cw + 1), __ldg(cw + 7)};
                    dflt AsX = {0.0f, 0.0f}, BsX = {0.0f, 0.0f};
                    if (j > 1) {
                        const float *cs = md.coef + 12 * (cl - (size_t)maxi);
                        AsX = {__ldg(cs + 2), __ldg(cs + 8)};
                        BsX = {__ldg(cs + 3), __ldg(cs + 9)};
                    }
                    const bool top = (k == maxk);
                    const double rv = __ldg(md.rvol + (size_t)(j - 1) + (size_t)maxj * (size_t)(k - 1));
                    const size_t base = (size_t)L * ((size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * (size_t)k));
                    const float *gt = md.gtop + (size_t)(L + 2) * ((size_t)(i - 1) + (size_t)maxi * (size_t)(j - 1));
                    bool iso = false;
                    // top-face stencil: C1*T(k+1) + C0*T(k) (+ isoneutral corners)
                    dflt C1X = AaX, C0X = BaX;
                    dflt W0X = {0.f, 0.f}, E0X = {0.f, 0.f}, S0X = {0.f, 0.f}, N0X = {0.f, 0.f};
                    dflt W1X = {0.f, 0.f}, E1X = {0.f, 0.f}, S1X = {0.f, 0.f}, N1X = {0.f, 0.f};
                    if (md.diso && !top) {
                        // isoneutral coefficients (goldstein.f90:2561-2624) in FP64 from the FP64
                        // state: the density differences scc*dS - tec*dT cancel strongly in weakly
                        // stratified water; they are differences of D = ec(2)*S - tec*T with the
                        // cell's tec (goldstein.f90:2587-2588)
                        auto ld = [&](int ii, int jj, int kk, int l) {
                            return __ldg(R + (size_t)L * ((size_t)ii + (size_t)NI * ((size_t)jj + (size_t)NJ * (size_t)kk)) + l);
                        };
                        const double t1 = ld(i, j, k, 0), t2 = ld(i, j, k + 1, 0);
                        const double s1 = ld(i, j, k, 1), s2 = ld(i, j, k + 1, 1);
                        const double tatw = 0.5 * (t1 + t2);
                        double tec = -md.ec[0] - md.ec[2] * tatw * 2.0 - md.ec[3] * tatw * tatw * 3.0;
                        if (md.ieos) tec = tec - md.ec[4] * mk[2 * mkn + k];
                        const double scc = md.ec[1];
                        const double Dc0 = scc * s1 - tec * t1, Dc1 = scc * s2 - tec * t2;
                        const double rdza = mk[4 * mkn + k];
                        const double dzrho = (Dc1 - Dc0) * rdza;
                        if (dzrho < -1.0e-12) {
                            iso = true;
                            const double rdzrho = 1.0 / dzrho;
                            const double rcr = mj[j];                          // rc(j)*rdphi
                            const double cvs = mj[mjn + j - 1], cvn = mj[mjn + j];   // cv*rdsv at j-1, j
                            const int im = (i == 1) ? maxi : i - 1, ip = (i == maxi) ? 1 : i + 1;
                            double dxr[4], dyr[4], mx[4], my[4];
                            double tv1 = 0.0;
#pragma unroll
                            for (int knp = 0; knp <= 1; ++knp) {
                                const double Dck = knp ? Dc1 : Dc0;
#pragma unroll
                                for (int nnp = 0; nnp <= 1; ++nnp) {
                                    const int ina = nnp + 2 * knp;
                                    const int kk = k + knp;
                                    const bool okx = kk >= k1t[cidx + (nnp ? 1 : -1)];
                                    const bool oky = kk >= k1t[cidx + (nnp ? nx : -nx)];
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
                                if (ts_group) limps_l += 1;
                            }
                            if (ts_group) dmax_l = fmax(dmax_l, tv1 * slim * md.diff1 * rdza * md.dt * rdza);
                            // G_iso = dt*dphi*ds * 0.25*slim*diff1/dzrho^2 * sum_ina[...]
                            const double c0 = mj[2 * mjn + j] * 0.25 * slim * md.diff1 * rdzrho * rdzrho;
                            const double two_dz = 2.0 * dzrho * c0;
                            double wx[4], wy[4];
#pragma unroll
                            for (int n = 0; n < 4; ++n) {
                                wx[n] = two_dz * dxr[n] * mx[n];
                                wy[n] = two_dz * dyr[n] * my[n];
                            }
                            const double wz = -c0 * sum2 * rdza;      // dzts = (T(k+1)-T(k))*rdza
                            const double c0d = f2d_scaled(BaX.hi, 0) + f2d_scaled(BaX.lo, 0) + ((wx[0] - wx[1]) + (wy[0] - wy[1]) - wz);
                            const double c1d = f2d_scaled(AaX.hi, 0) + f2d_scaled(AaX.lo, 0) + ((wx[2] - wx[3]) + (wy[2] - wy[3]) + wz);
                            C0X = df_split(c0d);
                            C1X = df_split(c1d);
                            W0X = df_split(-wx[0]); E0X = df_split(wx[1]); W1X = df_split(-wx[2]); E1X = df_split(wx[3]);
                            S0X = df_split(-wy[0]); N0X = df_split(wy[1]); S1X = df_split(-wy[2]); N1X = df_split(wy[3]);
                        }
                    }
                    const int cE = cidx + 1, cW = cidx - 1, cN = cidx + nx, cS = cidx - nx;
                    int q0 = 0;
                    if (ts_group) {
                        // T and S: double-float transfers, FP64 update
                        double tn[2];
#pragma unroll
                        for (int l = 0; l < 2; ++l) {
                            const float *F = Sk + l * ncp, *FL = SkL + l * ncp;
                            const float *U = Su + l * ncp, *UL = SuL + l * ncp;
                            const dflt Tc = {F[cidx], FL[cidx]}, TE = {F[cE], FL[cE]}, TW = {F[cW], FL[cW]};
                            const dflt TN = {F[cN], FL[cN]}, TS = {F[cS], FL[cS]};
                            const dflt Ge = df_dot2(AeX, TE, BeX, Tc);
                            const dflt Gw = df_dot2(AwX, Tc, BwX, TW);
                            const dflt Gn = df_dot2(AnX, TN, BnX, Tc);
                            const dflt Gs = df_dot2(AsX, Tc, BsX, TS);
                            const int sl = s_scale[l];
                            dflt Ga;
                            if (top) {
                                const float sc = __int_as_float((127 + sl) << 23);
                                Ga = {__ldg(gt + l) * sc, __ldg(gt + L + l) * sc};
                            } else {
                                Ga = df_dot2(C1X, dflt{U[cidx], UL[cidx]}, C0X, Tc);
                                if (iso) {
                                    Ga = df_add(Ga, df_dot2(W0X, TW, E0X, TE));
                                    Ga = df_add(Ga, df_dot2(S0X, TS, N0X, TN));
                                    Ga = df_add(Ga, df_dot2(W1X, dflt{U[cW], UL[cW]}, E1X, dflt{U[cE], UL[cE]}));
                                    Ga = df_add(Ga, df_dot2(S1X, dflt{U[cS], UL[cS]}, N1X, dflt{U[cN], UL[cN]}));
                                }
                            }
                            float *qb = QBD + (2 * l) * nin + cell;
                            const dflt Gb = {qb[0], qb[nin]};
                            const dflt sum = df_add(df_add(df_sub(Gw, Ge), df_sub(Gs, Gn)), df_sub(Gb, Ga));
                            qb[0] = Ga.hi;
                            qb[nin] = Ga.lo;
                            const double dlt = f2d_scaled(sum.hi, sl) + f2d_scaled(sum.lo, sl);
                            const double told = R[base + l];
                            tn[l] = fma(dlt, rv, told);
                            W[base + l] = tn[l];
                            if (((unsigned)__double2hiint(tn[l]) & 0x7ff00000u) == 0x7ff00000u) nonfinite = true;
                        }
                        // FP32 density prescreen for the exact convective adjustment
                        const float tf = d2f_scaled(tn[0], 0), sf = d2f_scaled(tn[1], 0);
                        const float rf = eos_f(ecf, tf, sf);
                        if (k > k1c) {
                            const float margin = 2.0e-6f * (fabsf(rf) + fabsf(rho_prev) + fabsf(ecf[0] * tf) +
                                                            fabsf(ecf[1] * sf) + fabsf(ecf[2] * tf * tf) +
                                                            fabsf(ecf[3] * tf * tf * tf)) + 1.0e-30f;
                            if (!(rho_prev - rf > margin)) unstable = true;
                        }
                        rho_prev = rf;
                        q0 = 2;
                    }
                    // other tracers: FP32 transfers rounded once to int32
                    const float Ae = AeX.hi, Be = BeX.hi, An = AnX.hi, Bn = BnX.hi, Aw = AwX.hi, Bw = BwX.hi;
                    const float As = AsX.hi, Bs = BsX.hi;
                    const float cC0 = C0X.hi, cC1 = C1X.hi, cW0 = W0X.hi, cE0 = E0X.hi, cS0 = S0X.hi, cN0 = N0X.hi;
                    const float cW1 = W1X.hi, cE1 = E1X.hi, cS1 = S1X.hi, cN1 = N1X.hi;
                    const unsigned amask = __activemask();
                    for (int q = q0; q < gl; ++q) {
                        const int l = g0 + q;
                        const float *F = Sk + q * ncp;
                        const float Tc = F[cidx], TE = F[cE], TW = F[cW], TN = F[cN], TS = F[cS];
                        const float ge = fmaf(Ae, TE, Be * Tc);
                        const float gw = fmaf(Aw, Tc, Bw * TW);
                        const float gn = fmaf(An, TN, Bn * Tc);
                        const float gs = fmaf(As, Tc, Bs * TS);
                        const int sl = s_scale[l];
                        float ga;
                        if (top) {
                            ga = __ldg(gt + l) * __int_as_float((127 + sl) << 23);
                        } else {
                            const float *U = Su + q * ncp;
                            ga = fmaf(cC1, U[cidx], cC0 * Tc);
                            if (iso) {
                                ga = fmaf(cW0, TW, ga);
                                ga = fmaf(cE0, TE, ga);
                                ga = fmaf(cS0, TS, ga);
                                ga = fmaf(cN0, TN, ga);
                                ga = fmaf(cW1, U[cW], ga);
                                ga = fmaf(cE1, U[cE], ga);
                                ga = fmaf(cS1, U[cS], ga);
                                ga = fmaf(cN1, U[cN], ga);
                            }
                        }
                        if (track) {
                            // per-tracer maximum for the scale of later steps: one shared atomic
                            // per warp; also the int32 range check
                            const float gm = fmaxf(fmaxf(fabsf(ge), fabsf(gw)), fmaxf(fmaxf(fabsf(gn), fabsf(gs)), fabsf(ga)));
                            gmax = fmaxf(gmax, gm);
                            const unsigned wmax = __reduce_max_sync(amask, __float_as_uint(gm));
                            if (lane == __ffs(amask) - 1) atomicMax(&s_gmax[l], wmax);
                        }
                        const int qe = __float2int_rn(ge), qw = __float2int_rn(gw);
                        const int qn = __float2int_rn(gn), qs = __float2int_rn(gs);
                        const int qa = __float2int_rn(ga);
                        int *qbp = QB + q * nin + cell;
                        const int sum = (qw - qe) + (qs - qn) + (*qbp - qa);
                        *qbp = qa;
                        const double told = R[base + l];
                        const double tnew = fma(i2d_scaled(sum, sl), rv, told);
                        W[base + l] = tnew;
                        if (((unsigned)__double2hiint(tnew) & 0x7ff00000u) == 0x7ff00000u) nonfinite = true;
                    }
                }
                // the thread's own copies of level k+2 -> FP32 slot of k+2; start level k+3
                if (k + 2 <= maxk) {
                    cp_async_wait_all();
                    pump(k + 2, k + 3 <= maxk ? k + 3 : -1);
                }
                __syncthreads();
            }
        }

        // exact convective adjustment of columns that may be unstable
        if (inside && k1c <= maxk) {
            const size_t c2 = (size_t)(i - 1) + (size_t)maxi * (size_t)(j - 1);
            if (unstable || md.iconv == 1 || md.ieos != 0) {
                Fp32Col col;
                col.w = W;
                col.stat = md.ts_static;
                col.L = L;
                col.NI = NI;
                col.NJ = NJ;
                col.i = i;
                col.j = j;
                col.k1 = k1c;
                EosCoef ec;
                for (int n = 0; n < 5; ++n) ec.ec[n] = md.ec[n];
                ec.ieos = md.ieos;
                const double *dz = mk, *rdz = mk + mkn, *zw = mk + 2 * mkn, *zro = mk + 3 * mkn;
                col.rho[0] = 0.0;
                for (int kk = 1; kk <= maxk; ++kk) col.rho[kk] = eos_rn(ec, col.T(0, kk), col.T(1, kk), zro[kk]);
                int icos = 0;
                if (md.iconv == 1) icos = coshuffle_rn(col, ec, maxk, L, k1c, dz, rdz, zw);
                const int filled = co_rn(col, ec, maxk, L, k1c, dz, zw);
                if (md.iconv == 1) {
                    if (filled > icos) icos = filled;
                    md.icosd[c2] = icos;
                    md.cost[c2] = __dmul_rn(md.dsc, zw[maxk - 1 - icos]);
                } else if (filled > 0) {
                    double cst = md.cost[c2];
                    for (int f = 0; f < filled; ++f) cst = __dadd_rn(cst, 1.0);
                    md.cost[c2] = cst;
                }
            }
        }
        if (md.diso) {
            unsigned long long *dg = md.diag + 2 * (step & 1);
            unsigned long long db = __double_as_longlong(dmax_l);
            if (db) atomicMax(&dg[0], db);
            if (limps_l) atomicAdd(&dg[1], (unsigned long long)limps_l);
        }
        // a scaled transfer above 3.5e8 could overflow the int32 sum of six faces
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

int fp32_rescale(const MemberDesc *descs, int n, cudaStream_t s)
{
    if (n <= 0) return 0;
    k_rescale<<<std::min(n, 1024), 32, 0, s>>>(descs, n);
    return cudaGetLastError() == cudaSuccess ? 0 : GB_GO_ECUDA;
}

int fp32_smem_bytes(int tile_i, int tile_j, int L) { return fp32_smem_layout(tile_i, tile_j, L).total; }

int fp32_launch(const MemberDesc *descs, const int4 *items, int nitems, int lmax, int smem_bytes,
                const long long *step_ctr, int rel, cudaStream_t s)
{
    (void)lmax;
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    }
    cudaFuncSetAttribute(k_step_fp32, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_fp32, kFp32Threads, smem_bytes);
    if (per_sm < 1) per_sm = 1;
    int grid = std::min(nitems, nsm * per_sm);
    if (grid < 1) grid = 1;
    k_step_fp32<<<grid, kFp32Threads, smem_bytes, s>>>(descs, items, nitems, step_ctr, rel);
    return cudaGetLastError() == cudaSuccess ? 0 : GB_GO_ECUDA;
}

void fp32_default_tile(int maxi, int maxj, int *ti, int *tj)
{
    // whole rows when the grid is narrow, else 32 x 4 (<= 128 threads, <= 64 wide)
    int best_i = 16, best_j = 8;
    double best = 1e30;
    for (int tx = 4; tx <= 64; ++tx) {
        for (int ty = 1; ty <= 32 && tx * ty <= kFp32Threads; ++ty) {
            if (tx * ty < 64) continue;
            const int nti = (maxi + tx - 1) / tx, ntj = (maxj + ty - 1) / ty;
            // cost: halo'd slab cells loaded + idle threads
            const double load = (double)nti * ntj * (tx + 2) * (ty + 2);
            const double idle = (double)nti * ntj * tx * ty - (double)maxi * maxj;
            const double c = load + 0.5 * idle;
            if (c < best) {
                best = c;
                best_i = tx;
                best_j = ty;
            }
        }
    }
    *ti = best_i;
    *tj = best_j;
}

// ---------------------------------------------------------------------------
// host-side static data

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
                 *dt = kb + 5 * nk, *zw = kb + 6 * nk, *ssmax = kb + 7 * nk;
    const size_t ncell = (size_t)maxi * maxj * maxk;
    out.coef.assign(12 * ncell, 0.0f);
    out.rvol.assign((size_t)maxj * maxk, 0.0);
    out.cmax = 0.0;
    auto U = [&](int c, int i, int j, int k) -> double {
        return u[(size_t)c + 3 * ((size_t)i + (size_t)(maxi + 1) * ((size_t)j + (size_t)(maxj + 1) * (size_t)(k - 1)))];
    };
    auto K1 = [&](int i, int j) { return k1[i + (size_t)NI * j]; };
    for (int k = 1; k <= maxk; ++k) {
        for (int j = 1; j <= maxj; ++j) {
            out.rvol[(size_t)(j - 1) + (size_t)maxj * (k - 1)] = 1.0 / (p.dphi * ds[j] * dz[k]);
            for (int i = 1; i <= maxi; ++i) {
                float *c = &out.coef[12 * ((size_t)(i - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (k - 1)))];
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
                }
                for (int n = 0; n < 6; ++n) {
                    c[n] = (float)cd[n];
                    c[6 + n] = (float)(cd[n] - (double)c[n]);
                }
                for (int f = 0; f < 3; ++f)
                    out.cmax = std::max(out.cmax, (double)std::fabs(c[2 * f]) + (double)std::fabs(c[2 * f + 1]));
            }
        }
    }
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

void fp32_scales(const Dims &d, const int32_t *k1, const double *ts, double cmax, const float *gtop,
                 std::vector<int32_t> &scale)
{
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk, L = d.L, NI = d.NI, NJ = d.NJ;
    std::vector<double> tmax(L, 0.0), gmax(L, 0.0);
    for (int k = 1; k <= maxk; ++k)
        for (int j = 1; j <= maxj; ++j)
            for (int i = 1; i <= maxi; ++i) {
                if (k < k1[i + (size_t)NI * j]) continue;
                const double *p = ts + (size_t)L * ((size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * k));
                for (int l = 0; l < L; ++l) tmax[l] = std::max(tmax[l], std::fabs(p[l]));
            }
    if (gtop)
        for (size_t n = 0; n < (size_t)maxi * maxj; ++n)
            for (int l = 0; l < L; ++l) gmax[l] = std::max(gmax[l], (double)std::fabs(gtop[n * (L + 2) + l]));
    scale.assign(L, 0);
    for (int l = 0; l < L; ++l) {
        // largest transfer the step can produce: (|A|+|B|)*max|T| per face; the
        // isoneutral stencil and growth of max|T| are covered by 2^4 headroom
        // below the int32 range (2^26 target); a transfer above 3e8 (the sum of six
        // stays inside int32) sets the member's range flag
        const double g = std::max(2.0 * cmax * tmax[l], gmax[l]);
        int s = 0;
        if (g > 0.0 && std::isfinite(g)) s = (int)std::floor(std::log2(67108864.0 / g));
        scale[l] = std::max(-120, std::min(120, s));
    }
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

int fp32_export(const MemberDesc &md, const double *cur, double *rho, cudaStream_t s)
{
    const size_t ncell = (size_t)md.maxj * md.maxk * (md.maxi + 2);
    const int blocks = (int)std::min<size_t>((ncell + 255) / 256, 4096);
    k_export_fp32<<<blocks, 256, 0, s>>>(md, const_cast<double *>(cur), rho);
    k_export_halo<<<std::max(1, (int)std::min<size_t>((2 * (size_t)md.maxj * md.maxk + 255) / 256, 1024)), 256, 0, s>>>(
        md, const_cast<double *>(cur), rho);
    count_launches(2);
    return cudaGetLastError() == cudaSuccess ? 0 : GB_GO_ECUDA;
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
    if (p.iediff != 0) {
        msg = "GB_GO_FP32FLUX does not provide iediff 1/2 (use GB_GO_FP64)";
        return GB_GO_EUNSUPPORTED;
    }
    const int nj = d.maxj + 2, nk = d.maxk + 2;
    const double *dtp = blob.data() + 8 * nj + 5 * nk;
    for (int k = 2; k <= d.maxk; ++k)
        if (dtp[k] != dtp[1]) {
            msg = "GB_GO_FP32FLUX needs the same dt on every level (the transfers are shared between levels)";
            return GB_GO_EUNSUPPORTED;
        }
    int ti = 16, tj = 8;
    fp32_default_tile(d.maxi, d.maxj, &ti, &tj);
    if (fp32_smem_bytes(ti, tj, d.L) > 200 * 1024) {
        msg = "tile does not fit in shared memory";
        return GB_GO_ERANGE;
    }
    Fp32Host *h = new Fp32Host();
    h->d = d;
    h->p = p;
    h->blob = blob;
    h->k1.assign(k1_host, k1_host + (size_t)d.NI * d.NJ);
    h->k1_dev = m.k1;
    h->dt = dtp[1];
    Fp32Data &D = h->data;
    D.tile_i = ti;
    D.tile_j = tj;
    const size_t ncell = (size_t)d.maxi * d.maxj * d.maxk;
    cudaError_t e = cudaMalloc(&D.coef, 12 * ncell * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&D.rvol, (size_t)d.maxj * d.maxk * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.gtop, (size_t)(d.L + 2) * d.maxi * d.maxj * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&D.scale, (size_t)d.L * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&D.gmax, (size_t)d.L * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(D.gmax, 0, (size_t)d.L * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&D.mk, 6 * (size_t)nk * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.mj, 3 * (size_t)nj * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.status, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&D.dev, sizeof(MemberDesc));
    if (e == cudaSuccess) e = cudaMalloc(&D.step_ctr, sizeof(long long));
    const int nti = (d.maxi + ti - 1) / ti, ntj = (d.maxj + tj - 1) / tj;
    D.nitems = nti * ntj;
    if (e == cudaSuccess) e = cudaMalloc(&D.items, (size_t)D.nitems * sizeof(int4));
    if (e == cudaSuccess) {
        std::vector<int4> it;
        for (int b = 0; b < ntj; ++b)
            for (int a = 0; a < nti; ++a) it.push_back(make_int4(0, 1 + a * ti, 1 + b * tj, ti | (tj << 8)));
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
    cudaFree(D.coef); cudaFree(D.rvol); cudaFree(D.gtop); cudaFree(D.scale); cudaFree(D.gmax); cudaFree(D.mk); cudaFree(D.mj);
    cudaFree(D.status); cudaFree(D.dev); cudaFree(D.items); cudaFree(D.step_ctr);
    delete h;
    f->impl = nullptr;
    f->ready = false;
}

static int upload_scales(Fp32Host *h, cudaStream_t s)
{
    if (!h->have_state || !h->have_vel) return 0;
    std::vector<int32_t> sc;
    fp32_scales(h->d, h->k1.data(), h->ts1_host.data(), h->data.cmax, h->data.gtop_host_unscaled.data(), sc);
    h->data.scale_host = sc;
    return cuda_ok(cudaMemcpyAsync(h->data.scale, h->data.scale_host.data(), sc.size() * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, s)) ||
           cuda_ok(cudaStreamSynchronize(s));
}

int fp32_member_upload(Fp32Member *f, const double *ts1_host, const double *ts_host, cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    const size_t nts = (size_t)h->d.L * h->d.NI * h->d.NJ * (h->d.maxk + 2);
    h->ts1_host.assign(ts1_host, ts1_host + nts);
    h->have_state = true;
    h->data.steps = 0;
    const size_t ntop = (size_t)h->d.L * h->d.NI * h->d.NJ;
    int r = fp32_member_set_top(f, ts_host + ntop * (h->d.maxk + 1), s);
    if (r) return r;
    return upload_scales(h, s);
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

int fp32_member_set_velocity(Fp32Member *f, const double *u_host, cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    Fp32Static st;
    fp32_build_static(h->d, h->p, h->blob, h->k1.data(), u_host, st);
    Fp32Data &D = h->data;
    D.cmax = st.cmax;
    cudaError_t e = cudaMemcpyAsync(D.coef, st.coef.data(), st.coef.size() * sizeof(float), cudaMemcpyHostToDevice, s);
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
    (void)rho;
    Fp32Host *h = host_of(f);
    Fp32Data &D = h->data;
    if (!h->have_state || !h->have_vel) return GB_GO_ENOTREADY;
    if (!D.desc_valid) {
        MemberDesc &md = D.host;
        md.maxi = h->d.maxi; md.maxj = h->d.maxj; md.maxk = h->d.maxk; md.L = h->d.L; md.NI = h->d.NI; md.NJ = h->d.NJ;
        md.diso = h->p.diso; md.ieos = h->p.ieos; md.iconv = h->p.iconv;
        md.parity = 0;
        md.stop_step = (long long)1 << 62;
        md.dt = h->dt; md.dphi = h->p.dphi; md.rdphi = h->p.rdphi; md.diff1 = h->p.diff1;
        for (int n = 0; n < 5; ++n) md.ec[n] = h->p.ec[n];
        md.dsc = h->p.dsc;
        md.buf[0] = ts_buf[0];
        md.buf[1] = ts_buf[1];
        md.ts_static = ts_static;
        md.coef = D.coef; md.rvol = D.rvol; md.gtop = D.gtop; md.k1 = h->k1_dev; md.scale = D.scale; md.gmax = D.gmax;
        md.mk = D.mk; md.mj = D.mj; md.cost = cost; md.icosd = icosd;
        md.status = D.status;
        md.diag = diag;
        if (cudaMemcpyAsync(D.dev, &md, sizeof(md), cudaMemcpyHostToDevice, s) != cudaSuccess) return GB_GO_ECUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return GB_GO_ECUDA;
        D.desc_valid = true;
    }
    // buffer and diag slot of step n are (n & 1): the ping-pong starts at buffer 0 on upload
    D.step_host = D.steps;
    if (cudaMemcpyAsync(D.step_ctr, &D.step_host, sizeof(long long), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return GB_GO_ECUDA;
    const int smem = fp32_smem_bytes(D.tile_i, D.tile_j, h->d.L);
    for (int n = 0; n < nsteps; ++n) {
        const long long step = D.steps + n;
        if (cudaMemsetAsync(diag + 2 * (step & 1), 0, 2 * sizeof(unsigned long long), s) != cudaSuccess)
            return GB_GO_ECUDA;
        int r = fp32_launch(D.dev, D.items, D.nitems, h->d.L, smem, D.step_ctr, n, s);
        if (!r) r = fp32_rescale(D.dev, 1, s);
        if (r) return r;
        count_launches(2);
    }
    D.steps += nsteps;
    *cur = (int)(D.steps & 1);
    *slot = (int)(D.steps & 1);
    return 0;
}

int fp32_member_export(Fp32Member *f, const double *ts_cur, double *rho, const double *ts_static, cudaStream_t s)
{
    Fp32Host *h = host_of(f);
    Fp32Data &D = h->data;
    MemberDesc md{};
    md.maxi = h->d.maxi; md.maxj = h->d.maxj; md.maxk = h->d.maxk; md.L = h->d.L; md.NI = h->d.NI; md.NJ = h->d.NJ;
    md.ieos = h->p.ieos;
    for (int n = 0; n < 5; ++n) md.ec[n] = h->p.ec[n];
    md.ts_static = ts_static;
    md.mk = D.mk;
    md.k1 = h->k1_dev;
    int r = fp32_export(md, ts_cur, rho, s);
    if (r) return r;
    unsigned int st = 0;
    if (cudaMemcpyAsync(&st, D.status, sizeof(st), cudaMemcpyDeviceToHost, s) != cudaSuccess) return GB_GO_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return GB_GO_ECUDA;
    if (st & 1u) return GB_GO_ENONFINITE;
    if (st & 2u) return GB_GO_ERANGE;
    return 0;
}

}  // namespace gbgo
