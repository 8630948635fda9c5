// FP32-flux / FP64-state GOLDSTEIN tracer step for sm_103a (batched).
//
// The arithmetic of src/goldstein/goldstein.f90:2436-2642 (tstepo_flux) is
// rewritten per face as a linear transfer G = A*T_neighbour + B*T_centre with
// tracer-independent coefficients (upstream weights, masks and the metric
// factors dt*area folded in, built once per velocity field); the isoneutral
// term of the vertical face (goldstein.f90:2561-2624) becomes a 10-point
// stencil whose coefficients are built per cell and step from T and S.
//
// Split precision with exact conservation: face transfers are evaluated in FP32
// on tracer values scaled by a per-tracer power of two, rounded once to int32
// (F2I), and the SAME integer is subtracted from one cell and added to the
// other, so the integer budget of every step telescopes exactly.  The FP64
// state is then updated with one FMA: T += (sum of integer transfers)*2^-s / V.
// The FP64 <-> FP32/int conversions are done with integer bit operations, so a
// tracer-cell update costs one instruction of GB300's slow FP64 pipe.
//
// Convective adjustment (goldstein.f90:2657-2841) runs in exact FP64 on columns
// that an FP32 density prescreen cannot prove statically stable.
//
// Mapping: a CTA of 128 threads takes work items (member, TX x TY column tile)
// from a host-built list; each thread owns one column and marches k upward,
// with FP32 slabs of levels k and k+1 (plus the k+2 prefetch) in shared memory.
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

struct SmemLayout {
    int nx, ny, LP;      // slab extents (TX+2, TY+2) and padded tracer stride
    int slab;            // floats per slab
};

template <int LMAX>
__global__ void __launch_bounds__(kFp32Threads, 3)
k_step_fp32(const MemberDesc *__restrict__ mds, const int4 *__restrict__ items, int nitems,
            const long long *__restrict__ step_ctr, int rel)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ int s_kstart;
    __shared__ int s_scale[LMAX];
    const int t = threadIdx.x;
    const long long step = *step_ctr + rel;

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
        const int nx = TX + 2, ny = TY + 2;
        const int LP = L | 1;
        const int slabf = nx * ny * LP;
        int *k1t = reinterpret_cast<int *>(smraw);
        float *slab0 = reinterpret_cast<float *>(smraw + ((nx * ny * 4 + 15) & ~15));
        const int par = (int)((step + md.parity) & 1);
        const double *__restrict__ R = md.buf[par];
        double *__restrict__ W = md.buf[par ^ 1];

        // k1 tile with a one-column halo (periodic in i), land outside
        if (t == 0) s_kstart = 1 << 20;
        for (int e = t; e < nx * ny; e += blockDim.x) {
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
        for (int l = t; l < L; l += blockDim.x) s_scale[l] = md.scale[l];
        __syncthreads();
        const int ti = t % TX, tj = t / TX;
        const int i = i0 + ti, j = j0 + tj;
        const bool inside = (t < TX * TY) && (i <= maxi) && (j <= maxj);
        const int cidx = (tj + 1) * nx + (ti + 1);
        const int k1c = inside ? k1t[cidx] : maxk + 1;
        if (inside && k1c <= maxk) atomicMin(&s_kstart, k1c);
        __syncthreads();
        const int kstart = s_kstart;
        if (kstart > maxk) {
            __syncthreads();
            continue;
        }

        // slab loader: level `lev` into ring slot `slot`
        auto load_slab = [&](int lev, int slot) {
            float *S = slab0 + (size_t)slot * slabf;
            const int warp = t >> 5, lane = t & 31, nwarp = blockDim.x >> 5;
            const int rowlen = nx * L;
            const int dc = 32 / L, dl = 32 % L;
            for (int r = warp; r < ny; r += nwarp) {
                const int gj = j0 - 1 + r;
                float *Srow = S + r * nx * LP;
                if (gj > maxj + 1) {
                    for (int e = lane; e < nx * LP; e += 32) Srow[e] = 0.0f;
                    continue;
                }
                const size_t rowbase = (size_t)NI * ((size_t)gj + (size_t)NJ * (size_t)lev);
                int c = lane / L, l = lane % L;
                for (int e = lane; e < rowlen; e += 32) {
                    int gi = i0 - 1 + c;
                    float v = 0.0f;
                    if (gi <= maxi + 1) {
                        if (gi == 0) gi = maxi;
                        else if (gi == maxi + 1) gi = 1;
                        v = d2f_scaled(__ldg(R + ((size_t)gi + rowbase) * L + l), s_scale[l]);
                    }
                    Srow[c * LP + l] = v;
                    c += dc;
                    l += dl;
                    if (l >= L) {
                        l -= L;
                        c += 1;
                    }
                }
            }
        };

        // per-tracer carry of the bottom-face transfer (the top face of the level below)
        int qb[LMAX];
#pragma unroll
        for (int l = 0; l < LMAX; ++l) qb[l] = 0;

        float ecf[5];
        for (int n = 0; n < 5; ++n) ecf[n] = (float)md.ec[n];
        float rho_prev = 0.0f;
        bool unstable = false;
        float gmax = 0.0f;
        bool nonfinite = false;
        float dmax_l = 0.0f;
        unsigned limps_l = 0;
        const float *fj = md.fj;
        const float *fk = md.fk;
        const int fjn = maxj + 2, fkn = maxk + 2;

        load_slab(kstart, kstart % 3);
        if (kstart + 1 <= maxk) load_slab(kstart + 1, (kstart + 1) % 3);
        __syncthreads();

        for (int k = kstart; k <= maxk; ++k) {
            if (k + 2 <= maxk) load_slab(k + 2, (k + 2) % 3);
            const float *Sk = slab0 + (size_t)(k % 3) * slabf;
            const float *Su = slab0 + (size_t)((k + 1) % 3) * slabf;
            if (inside && k >= k1c) {
                const size_t cell = (size_t)(i - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (size_t)(k - 1));
                const float *cf = md.coef + 6 * cell;
                const float Ae = __ldg(cf + 0), Be = __ldg(cf + 1), An = __ldg(cf + 2), Bn = __ldg(cf + 3);
                float Aa = __ldg(cf + 4), Ba = __ldg(cf + 5);
                const int iw = (i == 1) ? maxi : i - 1;
                const float *cw = md.coef + 6 * ((size_t)(iw - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (size_t)(k - 1)));
                const float Aw = __ldg(cw + 0), Bw = __ldg(cw + 1);
                float As = 0.0f, Bs = 0.0f;
                if (j > 1) {
                    const float *cs = md.coef + 6 * (cell - (size_t)maxi);
                    As = __ldg(cs + 2);
                    Bs = __ldg(cs + 3);
                }
                const double rv = __ldg(md.rvol + (size_t)(j - 1) + (size_t)maxj * (size_t)(k - 1));
                const bool top = (k == maxk);
                // isoneutral stencil of the top face (goldstein.f90:2561-2624), FP32
                bool iso = false;
                float cC0 = Ba, cC1 = Aa, cW0 = 0.f, cE0 = 0.f, cS0 = 0.f, cN0 = 0.f, cW1 = 0.f, cE1 = 0.f, cS1 = 0.f,
                      cN1 = 0.f;
                if (md.diso && !top) {
                    // Slopes need the density differences scc*dS - tec*dT, which cancel
                    // strongly in weakly stratified water: they are formed in FP64 from
                    // the FP64 state as differences of D = ec(2)*S - tec*T (tec of this
                    // cell, as in goldstein.f90:2587-2588); the rest is FP32.
                    const double *mk = md.mk;
                    const int mkn = maxk + 2;
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
                    const double dzrho = (Dc1 - Dc0) * mk[4 * mkn + k];
                    if (dzrho < -1.0e-12) {
                        iso = true;
                        const float rdza = fk[k];
                        const float dzf = (float)dzrho;
                        const float rdzrho = 1.0f / dzf;
                        const float rcr = fj[j];                 // rc(j)*rdphi
                        const int im = (i == 1) ? maxi : i - 1, ip = (i == maxi) ? 1 : i + 1;
                        float dxr[4], dyr[4];
                        float tv1 = 0.0f;
#pragma unroll
                        for (int knp = 0; knp <= 1; ++knp) {
                            const double Dck = knp ? Dc1 : Dc0;
#pragma unroll
                            for (int nnp = 0; nnp <= 1; ++nnp) {
                                const int ina = nnp + 2 * knp;
                                const int kk = k + knp;
                                const int cx = cidx + (nnp ? 1 : -1);
                                const int cy = cidx + (nnp ? nx : -nx);
                                dxr[ina] = 0.0f;
                                dyr[ina] = 0.0f;
                                if (kk >= k1t[cx]) {
                                    const int ii = nnp ? ip : im;
                                    const double Dn = scc * ld(ii, j, kk, 1) - tec * ld(ii, j, kk, 0);
                                    dxr[ina] = (float)(nnp ? Dn - Dck : Dck - Dn) * rcr;
                                }
                                if (kk >= k1t[cy]) {
                                    const int jj = nnp ? j + 1 : j - 1;
                                    const double Dn = scc * ld(i, jj, kk, 1) - tec * ld(i, jj, kk, 0);
                                    dyr[ina] = (float)(nnp ? Dn - Dck : Dck - Dn) * fj[fjn + j - 1 + nnp];
                                }
                                tv1 += dxr[ina] * dxr[ina] + dyr[ina] * dyr[ina];
                            }
                        }
                        const float sum2 = tv1;
                        tv1 = 0.25f * tv1 * rdzrho * rdzrho;
                        const float ss = fk[2 * fkn + k];
                        float slim = 1.0f;
                        if (tv1 > ss) {
                            slim = ss * ss / (tv1 * tv1);
                            limps_l += 1;
                        }
                        const float tvd = tv1 * slim * (float)md.diff1 * rdza * (float)md.dt * rdza;
                        dmax_l = fmaxf(dmax_l, tvd);
                        // G_iso = dt*dphi*ds * 0.25*slim*diff1/dzrho^2 * sum_ina[...]; dxr/dyr already
                        // carry the metric factors, masked corners are zero
                        const float c0 = fj[2 * fjn + j] * 0.25f * slim * (float)md.diff1 * rdzrho * rdzrho;
                        const float two_dz = 2.0f * dzf * c0;
                        const float mx0 = (k >= k1t[cidx - 1]) ? rcr : 0.0f, mx1 = (k >= k1t[cidx + 1]) ? rcr : 0.0f;
                        const float mx2 = (k + 1 >= k1t[cidx - 1]) ? rcr : 0.0f, mx3 = (k + 1 >= k1t[cidx + 1]) ? rcr : 0.0f;
                        const float cvs = fj[fjn + j - 1], cvn = fj[fjn + j];
                        const float my0 = (k >= k1t[cidx - nx]) ? cvs : 0.0f, my1 = (k >= k1t[cidx + nx]) ? cvn : 0.0f;
                        const float my2 = (k + 1 >= k1t[cidx - nx]) ? cvs : 0.0f, my3 = (k + 1 >= k1t[cidx + nx]) ? cvn : 0.0f;
                        const float wx0 = two_dz * dxr[0] * mx0, wx1 = two_dz * dxr[1] * mx1;
                        const float wx2 = two_dz * dxr[2] * mx2, wx3 = two_dz * dxr[3] * mx3;
                        const float wy0 = two_dz * dyr[0] * my0, wy1 = two_dz * dyr[1] * my1;
                        const float wy2 = two_dz * dyr[2] * my2, wy3 = two_dz * dyr[3] * my3;
                        const float wz = -c0 * sum2 * rdza;      // dzts = (T(k+1)-T(k))*rdza
                        cW0 = -wx0; cE0 = wx1; cW1 = -wx2; cE1 = wx3;
                        cS0 = -wy0; cN0 = wy1; cS1 = -wy2; cN1 = wy3;
                        cC0 += (wx0 - wx1) + (wy0 - wy1) - wz;
                        cC1 += (wx2 - wx3) + (wy2 - wy3) + wz;
                    }
                }
                const size_t base = (size_t)L * ((size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * (size_t)k));
                const float *gt = md.gtop + (size_t)L * ((size_t)(i - 1) + (size_t)maxi * (size_t)(j - 1));
                double tn0 = 0.0, tn1 = 0.0;
#pragma unroll
                for (int l = 0; l < LMAX; ++l) {
                    if (l < L) {
                        const int sl = s_scale[l];
                        const float Tc = Sk[cidx * LP + l];
                        const float TE = Sk[(cidx + 1) * LP + l];
                        const float TW = Sk[(cidx - 1) * LP + l];
                        const float TN = Sk[(cidx + nx) * LP + l];
                        const float TS = Sk[(cidx - nx) * LP + l];
                        const float ge = fmaf(Ae, TE, Be * Tc);
                        const float gw = fmaf(Aw, Tc, Bw * TW);
                        const float gn = fmaf(An, TN, Bn * Tc);
                        const float gs = fmaf(As, Tc, Bs * TS);
                        float ga;
                        if (top) {
                            ga = __ldg(gt + l) * __int_as_float((127 + sl) << 23);
                        } else {
                            const float TU = Su[cidx * LP + l];
                            ga = fmaf(cC1, TU, cC0 * Tc);
                            if (iso) {
                                ga = fmaf(cW0, TW, ga);
                                ga = fmaf(cE0, TE, ga);
                                ga = fmaf(cS0, TS, ga);
                                ga = fmaf(cN0, TN, ga);
                                ga = fmaf(cW1, Su[(cidx - 1) * LP + l], ga);
                                ga = fmaf(cE1, Su[(cidx + 1) * LP + l], ga);
                                ga = fmaf(cS1, Su[(cidx - nx) * LP + l], ga);
                                ga = fmaf(cN1, Su[(cidx + nx) * LP + l], ga);
                            }
                        }
                        gmax = fmaxf(gmax, fmaxf(fmaxf(fabsf(ge), fabsf(gw)), fmaxf(fmaxf(fabsf(gn), fabsf(gs)), fabsf(ga))));
                        const int qe = __float2int_rn(ge), qw = __float2int_rn(gw);
                        const int qn = __float2int_rn(gn), qs = __float2int_rn(gs);
                        const int qa = __float2int_rn(ga);
                        const int sum = (qw - qe) + (qs - qn) + (qb[l] - qa);
                        qb[l] = qa;
                        const double told = __ldg(R + base + l);
                        const double tnew = fma(i2d_scaled(sum, sl), rv, told);
                        W[base + l] = tnew;
                        if (((unsigned)__double2hiint(tnew) & 0x7ff00000u) == 0x7ff00000u) nonfinite = true;
                        if (l == 0) tn0 = tnew;
                        if (l == 1) tn1 = tnew;
                    }
                }
                // FP32 density prescreen for the exact convective adjustment
                const float tf = d2f_scaled(tn0, 0), sf = d2f_scaled(tn1, 0);
                const float rf = eos_f(ecf, tf, sf);
                if (k > k1c) {
                    const float margin = 2.0e-6f * (fabsf(rf) + fabsf(rho_prev) + fabsf(ecf[0] * tf) +
                                                    fabsf(ecf[1] * sf) + fabsf(ecf[2] * tf * tf) +
                                                    fabsf(ecf[3] * tf * tf * tf)) + 1.0e-30f;
                    if (!(rho_prev - rf > margin)) unstable = true;
                }
                rho_prev = rf;
            }
            __syncthreads();
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
                const double *dz = md.mk, *rdz = md.mk + (maxk + 2), *zw = md.mk + 2 * (maxk + 2),
                             *zro = md.mk + 3 * (maxk + 2);
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
            unsigned long long db = __double_as_longlong((double)dmax_l);
            if (db) atomicMax(&dg[0], db);
            if (limps_l) atomicAdd(&dg[1], (unsigned long long)limps_l);
        }
        if (nonfinite || gmax > 3.0e8f) atomicOr(md.status, (nonfinite ? 1u : 0u) | (gmax > 3.0e8f ? 2u : 0u));
        __syncthreads();
    }
}

int fp32_smem_bytes(int tile_i, int tile_j, int L)
{
    const int nx = tile_i + 2, ny = tile_j + 2;
    const int LP = L | 1;
    return ((nx * ny * 4 + 15) & ~15) + 3 * nx * ny * LP * 4;
}

int fp32_launch(const MemberDesc *descs, const int4 *items, int nitems, int lmax, int smem_bytes,
                const long long *step_ctr, int rel, cudaStream_t s)
{
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    }
    auto go = [&](auto kern) -> int {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFp32Threads, smem_bytes);
        if (per_sm < 1) per_sm = 1;
        int grid = std::min(nitems, nsm * per_sm);
        if (grid < 1) grid = 1;
        kern<<<grid, kFp32Threads, smem_bytes, s>>>(descs, items, nitems, step_ctr, rel);
        return cudaGetLastError() == cudaSuccess ? 0 : GB_GO_ECUDA;
    };
    if (lmax <= 8) return go(k_step_fp32<8>);
    if (lmax <= 16) return go(k_step_fp32<16>);
    return go(k_step_fp32<32>);
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
    out.coef.assign(6 * ncell, 0.0f);
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
                float *c = &out.coef[6 * ((size_t)(i - 1) + (size_t)maxi * ((size_t)(j - 1) + (size_t)maxj * (k - 1)))];
                const int k1c = K1(i, j);
                const int ie = (i == maxi) ? 1 : i + 1;
                if (k >= std::max(k1c, K1(ie, j))) {
                    const double u1 = U(0, i, j, k);
                    const double pec = u1 * p.dphi / p.diff1, ups = pec / (2.0 + std::fabs(pec));
                    const double g = dt[k] * ds[j] * dz[k], a = u1 * rc[j];
                    c[0] = (float)(g * (a * (1.0 - ups) * 0.5 - rc2[j] * p.diff1));
                    c[1] = (float)(g * (a * (1.0 + ups) * 0.5 + rc2[j] * p.diff1));
                }
                if (k >= std::max(k1c, K1(i, j + 1))) {
                    const double u2 = U(1, i, j, k);
                    const double pec = u2 * dsv[std::min(j, maxj - 1)] / p.diff1, ups = pec / (2.0 + std::fabs(pec));
                    const double g = dt[k] * p.dphi * dz[k], a = cv[j] * u2;
                    c[2] = (float)(g * (a * (1.0 - ups) * 0.5 - cv2[j] * p.diff1));
                    c[3] = (float)(g * (a * (1.0 + ups) * 0.5 + cv2[j] * p.diff1));
                }
                if (k >= k1c && k < maxk) {
                    const double u3 = U(2, i, j, k);
                    const double pec = u3 * dza[k] / p.diff2, ups = pec / (2.0 + std::fabs(pec));
                    const double g = dt[k] * p.dphi * ds[j];
                    c[4] = (float)(g * (u3 * (1.0 - ups) * 0.5 - rdza[k] * p.diff2));
                    c[5] = (float)(g * (u3 * (1.0 + ups) * 0.5 + rdza[k] * p.diff2));
                }
                for (int f = 0; f < 3; ++f)
                    out.cmax = std::max(out.cmax, (double)std::fabs(c[2 * f]) + (double)std::fabs(c[2 * f + 1]));
            }
        }
    }
    out.mk.assign(5 * (size_t)nk, 0.0);
    for (int k = 0; k <= maxk + 1; ++k) {
        out.mk[k] = dz[k];
        out.mk[nk + k] = rdz[k];
        out.mk[2 * nk + k] = zw[k];
        out.mk[3 * nk + k] = zro[k];
        out.mk[4 * nk + k] = rdza[k];
    }
    out.fj.assign(4 * (size_t)nj, 0.0f);
    for (int j = 0; j <= maxj + 1; ++j) {
        if (j <= maxj) out.fj[j] = (float)(rc[j] * p.rdphi);
        if (j <= maxj) out.fj[nj + j] = (float)(cv[j] * rdsv[j]);
        if (j >= 1 && j <= maxj) out.fj[2 * nj + j] = (float)(dt[1] * p.dphi * ds[j]);
    }
    out.fk.assign(3 * (size_t)nk, 0.0f);
    for (int k = 0; k <= maxk + 1; ++k) {
        out.fk[k] = (float)rdza[k];
        out.fk[nk + k] = (float)zw[k];
        out.fk[2 * nk + k] = (float)ssmax[k];
    }
}

void fp32_gtop(const Dims &d, const PhysParams &p, const std::vector<double> &blob, const double *top,
               std::vector<float> &gtop)
{
    // transfer through the surface face: dt*dphi*ds(j)*ts(l,i,j,maxk+1)
    const int maxi = d.maxi, maxj = d.maxj, L = d.L, NI = d.NI;
    const int nj = maxj + 2, nk = d.maxk + 2;
    const double *ds = blob.data() + 6 * nj;
    const double dt = blob.data()[8 * nj + 5 * nk + 1];
    gtop.assign((size_t)L * maxi * maxj, 0.0f);
    for (int j = 1; j <= maxj; ++j)
        for (int i = 1; i <= maxi; ++i)
            for (int l = 0; l < L; ++l)
                gtop[(size_t)l + (size_t)L * ((size_t)(i - 1) + (size_t)maxi * (j - 1))] =
                    (float)(dt * p.dphi * ds[j] * top[(size_t)l + (size_t)L * ((size_t)i + (size_t)NI * j)]);
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
            for (int l = 0; l < L; ++l) gmax[l] = std::max(gmax[l], (double)std::fabs(gtop[n * L + l]));
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
    cudaError_t e = cudaMalloc(&D.coef, 6 * ncell * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&D.rvol, (size_t)d.maxj * d.maxk * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.gtop, (size_t)d.L * d.maxi * d.maxj * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&D.scale, (size_t)d.L * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&D.mk, 5 * (size_t)nk * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&D.fj, 4 * (size_t)nj * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&D.fk, 3 * (size_t)nk * sizeof(float));
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
    if (e == cudaSuccess) e = cudaMemsetAsync(D.gtop, 0, (size_t)d.L * d.maxi * d.maxj * sizeof(float), s);
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
    cudaFree(D.coef); cudaFree(D.rvol); cudaFree(D.gtop); cudaFree(D.scale); cudaFree(D.mk); cudaFree(D.fj);
    cudaFree(D.fk); cudaFree(D.status); cudaFree(D.dev); cudaFree(D.items); cudaFree(D.step_ctr);
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
    if (e == cudaSuccess) e = cudaMemcpyAsync(D.fj, st.fj.data(), st.fj.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(D.fk, st.fk.data(), st.fk.size() * sizeof(float), cudaMemcpyHostToDevice, s);
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
        md.coef = D.coef; md.rvol = D.rvol; md.gtop = D.gtop; md.k1 = h->k1_dev; md.scale = D.scale;
        md.mk = D.mk; md.fj = D.fj; md.fk = D.fk; md.cost = cost; md.icosd = icosd;
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
        if (r) return r;
        count_launches(1);
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
