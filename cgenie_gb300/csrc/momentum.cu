// GOLDSTEIN momentum step on the device (include/gb_momentum.h): wind, jbar, the barotropic
// streamfunction, the island corrections and velc of step_goldstein
// (src/goldstein/goldstein.f90:198-233), reading an FP64 gb_go handle's density and writing its
// velocities.
//
// Host, once (gb_mo_create): the reference's initialisation -- the band matrix and its LU
// elimination (invert, :3138-3204), the unit-source solves, the island integrals and
// matinv_gold (:1788-1814) -- in the reference's operation order; then the explicit inverse of
// the matrix, column by column from the same LU factors (host threads).
// Device, per step (-fmad=false; the reference's operation order except in k_psi):
//   k_bp       one thread per column: bp, sbp and their periodic copies (jbar :3226-3262)
//   k_rhs      one thread per psi point: the wind forcing and the J term (wind, jbar :3266-3314)
//   k_psi      one warp per psi point: the streamfunction, inverse x right-hand side (the
//              reference's back substitution is a serial chain of dependent FP64 adds)
//   k_ub       one thread per velocity point: ub from psi (ubarsolv :3530-3564)
//   k_island   one block: the island path integrals (a thread per path point, summed in path
//              order per island), matmult, psibc (:203-215, island)
//   k_corr     ub and psi island corrections (:217-229)
//   k_dzu      one thread per cell: the thermal-wind shear dzu (velc :3580-3640)
//   k_velc     one thread per column: the vertical integration, relaxation (velc :3641-3662)
//   k_w        one thread per column: w from continuity (velc :3666-3678)
#include "../../include/gb_momentum.h"
#include "gb_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

using namespace gbgo;

namespace {

struct MoDev {
    int maxi, maxj, maxk, isles, mpi, n, nm;
    double dphi, rdphi, rel;
    const double *s, *c, *sv, *cv, *rc, *rcv, *dsv, *rdsv, *ds, *rds, *rds2, *dz, *dza;
    const int32_t *k1, *ku, *mk, *getj;
    const double *rh, *drag, *rtv, *rtv3;
    const int32_t *npi, *lpisl, *ipisl, *jpisl;
    const double *tau, *dztau, *dztav;
    const double *minv, *ubisl, *psisl, *erisl;   // erisl: (isles, isles+1) after matinv_gold
    // grids above GB_MO_MAX_PSI points: the block-tridiagonal form of the same matrix, one block
    // per row j of psi points (n = maxi unknowns): the inverse Schur complements T_j (row-major,
    // n*n each), the couplings l_j (to row j-1) and u_j (to row j+1), and the forward vectors z
    const double *btT, *btl, *btu;
    double *btz;
    int bt;
    double *psibc, *gb, *gbold, *bp, *sbp, *ub, *psi, *scr, *dzu, *u, *u1;
    const double *rho;
};

// Fortran-bound index helpers (the reference's arrays, column-major)
__device__ __forceinline__ int K1(const MoDev &a, int i, int j) { return a.k1[i + (size_t)(a.maxi + 2) * j]; }
__device__ __forceinline__ double RH(const MoDev &a, int l, int i, int j)
{
    return a.rh[(l - 1) + 3 * ((size_t)i + (size_t)(a.maxi + 2) * j)];
}
__device__ __forceinline__ double DRAG(const MoDev &a, int l, int i, int j)
{
    return a.drag[(l - 1) + 2 * ((size_t)(i - 1) + (size_t)(a.maxi + 1) * (j - 1))];
}
__device__ __forceinline__ int KU(const MoDev &a, int l, int i, int j)
{
    return a.ku[(l - 1) + 2 * ((size_t)(i - 1) + (size_t)a.maxi * (j - 1))];
}
__device__ __forceinline__ int MK(const MoDev &a, int i, int j) { return a.mk[(i - 1) + (size_t)(a.maxi + 1) * (j - 1)]; }
__device__ __forceinline__ size_t BPi(const MoDev &a, int i, int j, int k)
{
    return (size_t)(i - 1) + (size_t)(a.maxi + 1) * ((size_t)(j - 1) + (size_t)a.maxj * (k - 1));
}
__device__ __forceinline__ size_t SBPi(const MoDev &a, int i, int j) { return (size_t)(i - 1) + (size_t)(a.maxi + 1) * (j - 1); }
__device__ __forceinline__ size_t UBi(const MoDev &a, int l, int i, int j) { return (l - 1) + 2 * ((size_t)i + (size_t)(a.maxi + 2) * j); }
__device__ __forceinline__ size_t PSIi(const MoDev &a, int i, int j) { return (size_t)i + (size_t)(a.maxi + 1) * j; }
__device__ __forceinline__ size_t Ui(const MoDev &a, int l, int i, int j, int k)
{
    return (l - 1) + 3 * ((size_t)i + (size_t)(a.maxi + 1) * ((size_t)j + (size_t)(a.maxj + 1) * (k - 1)));
}
__device__ __forceinline__ double RHO(const MoDev &a, int i, int j, int k)
{
    return a.rho[(size_t)i + (size_t)(a.maxi + 2) * ((size_t)j + (size_t)(a.maxj + 2) * k)];
}
__device__ __forceinline__ double TAU(const double *t, const MoDev &a, int l, int i, int j)
{
    return t[(l - 1) + 2 * ((size_t)(i - 1) + (size_t)a.maxi * (j - 1))];
}
__device__ __forceinline__ int imax2(int x, int y) { return x > y ? x : y; }
__device__ __forceinline__ int imax4(int w, int x, int y, int z) { return imax2(imax2(w, x), imax2(y, z)); }

// jbar :3226-3262: bp, sbp, and the periodic copies at i = maxi+1 (by the i = 1 thread)
__global__ void __launch_bounds__(32) k_bp(MoDev a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.maxi * a.maxj) return;
    const int i = t % a.maxi + 1, j = t / a.maxi + 1;
    const int k1 = K1(a, i, j);
    if (k1 <= a.maxk)
        for (int k = k1 + 1; k <= a.maxk; ++k)
            a.bp[BPi(a, i, j, k)] = a.bp[BPi(a, i, j, k - 1)] - (RHO(a, i, j, k) + RHO(a, i, j, k - 1)) * a.dza[k - 2] * 0.5;
    const int mk = MK(a, i, j);
    if (mk > 0) {
        double s = 0;
        for (int k = mk + 1; k <= a.maxk; ++k) s = s + a.bp[BPi(a, i, j, k)] * a.dz[k - 1];
        a.sbp[SBPi(a, i, j)] = s;
    }
    if (i == 1) {
        if (k1 < a.maxk)
            for (int k = k1; k <= a.maxk; ++k) a.bp[BPi(a, a.maxi + 1, j, k)] = a.bp[BPi(a, 1, j, k)];
        if (k1 <= a.maxk) a.sbp[SBPi(a, a.maxi + 1, j)] = a.sbp[SBPi(a, 1, j)];
    }
}

__device__ double ksum(const MoDev &a, int i, int j, int ka, int kb)
{
    double s = 0;
    for (int k = ka; k <= kb; ++k) s = s + a.bp[BPi(a, i, j, k)] * a.dz[k - 1];
    return s;
}

// wind :3696-3712 and the J term of jbar :3266-3314, one psi point each
__global__ void __launch_bounds__(32) k_rhs(MoDev a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.nm) return;
    const int i = t % a.maxi + 1, j = t / a.maxi;   // gb(i + j*n)
    const int ip1 = i % a.maxi + 1;
    double g;
    if (imax4(K1(a, i, j), K1(a, i + 1, j), K1(a, i, j + 1), K1(a, i + 1, j + 1)) <= a.maxk) {
        g = (TAU(a.tau, a, 2, ip1, j) * RH(a, 2, i + 1, j) - TAU(a.tau, a, 2, i, j) * RH(a, 2, i, j)) * a.rdphi * a.rcv[j - 1] -
            (TAU(a.tau, a, 1, i, j + 1) * a.c[j + 1] * RH(a, 1, i, j + 1) - TAU(a.tau, a, 1, i, j) * a.c[j] * RH(a, 1, i, j)) *
                a.rdsv[j - 1];
    } else {
        g = 0;
    }
    a.gbold[t] = g;
    if (j >= 1 && j <= a.maxj - 1 && a.getj[(i - 1) + (size_t)a.maxi * (j - 1)]) {
        double tv1 = ksum(a, ip1, j + 1, KU(a, 2, ip1, j), MK(a, ip1, j + 1));
        double tv2 = ksum(a, ip1, j, KU(a, 2, ip1, j), MK(a, ip1, j));
        double tv3 = ksum(a, i, j + 1, KU(a, 2, i, j), MK(a, i, j + 1));
        double tv4 = ksum(a, i, j, KU(a, 2, i, j), MK(a, i, j));
        const double *sbp = a.sbp;
        g = g + ((tv3 + sbp[SBPi(a, i, j + 1)] - tv4 - sbp[SBPi(a, i, j)]) * RH(a, 2, i, j) -
                 (tv1 + sbp[SBPi(a, ip1, j + 1)] - tv2 - sbp[SBPi(a, ip1, j)]) * RH(a, 2, ip1, j)) *
                    a.rdphi * a.rdsv[j - 1];
        tv1 = ksum(a, ip1, j + 1, KU(a, 1, i, j + 1), MK(a, ip1, j + 1));
        tv2 = ksum(a, ip1, j, KU(a, 1, i, j), MK(a, ip1, j));
        tv3 = ksum(a, i, j + 1, KU(a, 1, i, j + 1), MK(a, i, j + 1));
        tv4 = ksum(a, i, j, KU(a, 1, i, j), MK(a, i, j));
        g = g + ((tv1 + sbp[SBPi(a, ip1, j + 1)] - tv3 - sbp[SBPi(a, i, j + 1)]) * RH(a, 1, i, j + 1) -
                 (tv2 + sbp[SBPi(a, ip1, j)] - tv4 - sbp[SBPi(a, i, j)]) * RH(a, 1, i, j)) *
                    a.rdphi * a.rdsv[j - 1];
    }
    a.gb[t] = g;
}

// psi = inverse x gb: one warp per row (the row of the inverse is contiguous)
__global__ void __launch_bounds__(256) k_psi(MoDev a)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= a.nm) return;
    const double *row = a.minv + (size_t)w * a.nm;
    double s = 0.0;
    for (int c = lane; c < a.nm; c += 32) s = s + row[c] * a.gb[c];
    for (int o = 16; o > 0; o >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        const int i = w % a.maxi + 1, j = w / a.maxi;
        a.psi[PSIi(a, i, j)] = s;
        if (i == a.maxi) a.psi[PSIi(a, 0, j)] = s;   // psi(0,j) = psi(maxi,j)
    }
}

// Block-tridiagonal streamfunction solve (grids above GB_MO_MAX_PSI points).  The matrix of
// invert couples psi point (i, j) to (i+-1, j) (periodic in i) and to (i, j+-1), so with one
// block per row j it is block tridiagonal with diagonal off-diagonal blocks: block LU with the
// Schur complements S_0 = D_0, S_j = D_j - diag(l_j) S_{j-1}^-1 diag(u_{j-1}), factored once on
// the host; per step
//   forward   z_j = T_j (g_j - l_j o z_{j-1})       (T_j = S_j^-1, z_{-1} = 0)
//   backward  x_J = z_J,  x_j = z_j - T_j (u_j o x_{j+1})
// one launch per block row, one warp per row of T_j (contiguous), x overwriting z in place.
// One row of T_j per 64 threads (two warps: each thread's products issued together, then a
// shuffle sum per warp and one shared add), four rows per 256-thread block.
constexpr int kBtRowThreads = 64, kBtRowsPerBlock = 4;

__device__ __forceinline__ double bt_row_sum(double s, double *part)
{
    for (int o = 16; o > 0; o >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, o);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) part[w] = s;
    __syncthreads();
    return part[w & ~1] + part[w | 1];   // the row's two warps, in one order
}

__global__ void __launch_bounds__(kBtRowThreads * kBtRowsPerBlock) k_bt_forward(MoDev a, int j)
{
    __shared__ double part[kBtRowsPerBlock * 2];
    const int n = a.maxi;
    const int r = blockIdx.x * kBtRowsPerBlock + threadIdx.x / kBtRowThreads, c0 = threadIdx.x % kBtRowThreads;
    double s = 0.0;
    if (r < n) {
        const double *row = a.btT + ((size_t)j * n + r) * n;
        const double *g = a.gb + (size_t)j * n;
        const double *l = a.btl + (size_t)j * n;
        const double *zp = a.btz + (size_t)(j > 0 ? j - 1 : 0) * n;
        for (int c = c0; c < n; c += kBtRowThreads) {
            const double y = j > 0 ? g[c] - l[c] * zp[c] : g[c];
            s = s + row[c] * y;
        }
    }
    s = bt_row_sum(s, part);
    if (r < n && c0 == 0) a.btz[(size_t)j * n + r] = s;
}

__global__ void __launch_bounds__(kBtRowThreads * kBtRowsPerBlock) k_bt_backward(MoDev a, int j)
{
    __shared__ double part[kBtRowsPerBlock * 2];
    const int n = a.maxi;
    const int r = blockIdx.x * kBtRowsPerBlock + threadIdx.x / kBtRowThreads, c0 = threadIdx.x % kBtRowThreads;
    double s = 0.0;
    if (r < n) {
        const double *row = a.btT + ((size_t)j * n + r) * n;
        const double *u = a.btu + (size_t)j * n;
        const double *xn = a.btz + (size_t)(j + 1) * n;
        for (int c = c0; c < n; c += kBtRowThreads) s = s + row[c] * (u[c] * xn[c]);
    }
    s = bt_row_sum(s, part);
    if (r < n && c0 == 0) a.btz[(size_t)j * n + r] = a.btz[(size_t)j * n + r] - s;
}

// psi from the solution (psi(i, j) = x(i + j*maxi), psi(0, j) = psi(maxi, j))
__global__ void __launch_bounds__(128) k_bt_psi(MoDev a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.nm) return;
    const int i = t % a.maxi + 1, j = t / a.maxi;
    const double v = a.btz[t];
    a.psi[PSIi(a, i, j)] = v;
    if (i == a.maxi) a.psi[PSIi(a, 0, j)] = v;
}

// ub from psi (ubarsolv :3538-3564); the periodic columns i = 0, maxi+1 evaluate the formula
// at the column they copy
__global__ void __launch_bounds__(128) k_ub(MoDev a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ni = a.maxi + 2;
    if (t >= ni * (a.maxj + 1)) return;
    const int ib = t % ni, j = t / ni;
    const int i = ib == 0 ? a.maxi : (ib == a.maxi + 1 ? 1 : ib);
    if (j >= 1) {
        a.ub[UBi(a, 1, ib, j)] = -RH(a, 1, i, j) * a.c[j] * (a.psi[PSIi(a, i, j)] - a.psi[PSIi(a, i, j - 1)]) * a.rds[j - 1];
    }
    double v2 = 0.0;
    if (j >= 1 && j <= a.maxj - 1)
        v2 = RH(a, 2, i, j) * (a.psi[PSIi(a, i, j)] - a.psi[PSIi(a, i - 1, j)]) * a.rcv[j - 1] * a.rdphi;
    a.ub[UBi(a, 2, ib, j)] = v2;
}

// island path integral (goldstein_lib.f90:186-241, indj = 1), then matmult and psibc (:203-215).
// Each path point's two contributions (the velocity and wind term, the J term) are computed by
// its own thread; one thread per island then adds them in path order, as the reference does.
__global__ void __launch_bounds__(256) k_island(MoDev a, double *scr)
{
    __shared__ double rhs[33];
    const int npt = a.isles * a.mpi;
    for (int q = threadIdx.x; q < npt; q += blockDim.x) {
        const int isl = q / a.mpi + 1, p = q % a.mpi + 1;
        if (p > a.npi[isl - 1]) continue;
        const int lpi = a.lpisl[q], ipi = a.ipisl[q], jpi = a.jpisl[q];
        const int al = lpi < 0 ? -lpi : lpi;
        const double sg = lpi >= 0 ? 1.0 : -1.0;
        double cor;
        if (al == 1)
            cor = -a.s[jpi] * 0.25 * (a.ub[UBi(a, 2, ipi, jpi)] + a.ub[UBi(a, 2, ipi + 1, jpi)] + a.ub[UBi(a, 2, ipi, jpi - 1)] +
                                      a.ub[UBi(a, 2, ipi + 1, jpi - 1)]);
        else
            cor = a.sv[jpi] * 0.25 * (a.ub[UBi(a, 1, ipi - 1, jpi)] + a.ub[UBi(a, 1, ipi, jpi)] + a.ub[UBi(a, 1, ipi - 1, jpi + 1)] +
                                      a.ub[UBi(a, 1, ipi, jpi + 1)]);
        scr[2 * q] = sg * (DRAG(a, al, ipi, jpi) * a.ub[UBi(a, al, ipi, jpi)] + cor - 1.0 * TAU(a.tau, a, al, ipi, jpi) * RH(a, al, ipi, jpi)) *
                     (a.c[jpi] * a.dphi * (2.0 - al) + a.rcv[jpi - 1] * a.dsv[jpi - 1] * (al - 1.0));
        if (al == 1) {
            double tv1 = 0.0;
            for (int k = KU(a, 1, ipi, jpi); k <= MK(a, ipi + 1, jpi); ++k) tv1 = tv1 + a.bp[BPi(a, ipi + 1, jpi, k)] * a.dz[k - 1];
            for (int k = KU(a, 1, ipi, jpi); k <= MK(a, ipi, jpi); ++k) tv1 = tv1 - a.bp[BPi(a, ipi, jpi, k)] * a.dz[k - 1];
            scr[2 * q + 1] = (a.sbp[SBPi(a, ipi + 1, jpi)] - a.sbp[SBPi(a, ipi, jpi)] + tv1) * sg * RH(a, 1, ipi, jpi);
        } else {
            double tv2 = 0.0;
            for (int k = KU(a, 2, ipi, jpi); k <= MK(a, ipi, jpi + 1); ++k) tv2 = tv2 + a.bp[BPi(a, ipi, jpi + 1, k)] * a.dz[k - 1];
            for (int k = KU(a, 2, ipi, jpi); k <= MK(a, ipi, jpi); ++k) tv2 = tv2 - a.bp[BPi(a, ipi, jpi, k)] * a.dz[k - 1];
            scr[2 * q + 1] = (a.sbp[SBPi(a, ipi, jpi + 1)] - a.sbp[SBPi(a, ipi, jpi)] + tv2) * sg * RH(a, 2, ipi, jpi);
        }
    }
    __syncthreads();
    const int isl = threadIdx.x + 1;
    if (isl <= a.isles) {
        double e = 0.0;
        for (int p = 0; p < a.npi[isl - 1]; ++p) {
            const size_t q = (size_t)p + (size_t)a.mpi * (isl - 1);
            e = e + scr[2 * q];
            e = e + scr[2 * q + 1];
        }
        rhs[isl] = e;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const int nv = a.isles;
    auto A = [&](int r, int cc) { return a.erisl[(size_t)(r - 1) + (size_t)nv * (cc - 1)]; };
    if (nv > 1) {
        // matmult (:3470-3492) on the matrix reduced by matinv_gold at initialisation
        for (int i = 1; i <= nv - 1; ++i)
            for (int j = i + 1; j <= nv; ++j) rhs[j] = A(i, i) * rhs[j] - A(j, i) * rhs[i];
        rhs[nv] = rhs[nv] / A(nv, nv);
        for (int i = nv - 1; i >= 1; --i) {
            for (int j = i + 1; j <= nv; ++j) rhs[i] = rhs[i] - A(i, j) * rhs[j];
            rhs[i] = rhs[i] / A(i, i);
        }
        for (int isl2 = 1; isl2 <= nv; ++isl2) a.psibc[isl2 - 1] = -rhs[isl2];
    } else {
        a.psibc[0] = -rhs[1] / A(1, 1);
    }
}

// ub(l,i,j) += SUM(ubisl(l,i,j,:)*psibc(:)) for j >= 1; psi(i,j) += SUM(psisl(i,j,:)*psibc(:))
__global__ void __launch_bounds__(128) k_corr(MoDev a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nub = 2 * (size_t)(a.maxi + 2) * (a.maxj + 1), npsi = (size_t)(a.maxi + 1) * (a.maxj + 1);
    if ((size_t)t < nub) {
        const int j = (int)(t / (2 * (a.maxi + 2)));
        if (j >= 1) {
            double s = 0.0;
            for (int isl = 0; isl < a.isles; ++isl) s = s + a.ubisl[(size_t)isl * nub + t] * a.psibc[isl];
            a.ub[t] = a.ub[t] + s;
        }
    } else if ((size_t)t < nub + npsi) {
        const size_t x = t - nub;
        double s = 0.0;
        for (int isl = 0; isl < a.isles; ++isl) s = s + a.psisl[(size_t)isl * npsi + x] * a.psibc[isl];
        a.psi[x] = a.psi[x] + s;
    }
}

// velc :3580-3640: dzu(1:2,k) of every wet cell at once (they depend on the density of level k
// only), one thread per (column, level)
__global__ void __launch_bounds__(128) k_dzu(MoDev a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ncol = a.maxi * a.maxj;
    if (t >= ncol * a.maxk) return;
    const int col = t % ncol, k = t / ncol + 1;
    const int i = col % a.maxi + 1, j = col / a.maxi + 1;
    if (k < K1(a, i, j)) return;
    const double rdphi = a.rdphi;
    double tv1, tv2, tv4, tv5;
    if (K1(a, i + 1, j) > k) {
        tv1 = 0;
        tv2 = 0;
    } else {
        tv2 = -(RHO(a, i + 1, j, k) - RHO(a, i, j, k)) * rdphi * a.rc[j];
        if (imax4(K1(a, i, j - 1), K1(a, i, j + 1), K1(a, i + 1, j - 1), K1(a, i + 1, j + 1)) <= k)
            tv1 = -a.c[j] * (RHO(a, i + 1, j + 1, k) - RHO(a, i + 1, j - 1, k) + RHO(a, i, j + 1, k) - RHO(a, i, j - 1, k)) *
                  a.rds2[j - 2] * 0.25;
        else if (imax2(K1(a, i, j - 1), K1(a, i + 1, j - 1)) <= k)
            tv1 = -a.c[j] * (RHO(a, i + 1, j, k) - RHO(a, i + 1, j - 1, k) + RHO(a, i, j, k) - RHO(a, i, j - 1, k)) *
                  a.rdsv[j - 2] * 0.5;
        else if (imax2(K1(a, i, j + 1), K1(a, i + 1, j + 1)) <= k)
            tv1 = -a.c[j] * (RHO(a, i + 1, j + 1, k) - RHO(a, i + 1, j, k) + RHO(a, i, j + 1, k) - RHO(a, i, j, k)) *
                  a.rdsv[j - 1] * 0.5;
        else
            tv1 = 0;
    }
    if (K1(a, i, j + 1) > k) {
        tv4 = 0;
        tv5 = 0;
    } else {
        tv4 = -a.cv[j] * (RHO(a, i, j + 1, k) - RHO(a, i, j, k)) * a.rdsv[j - 1];
        if (imax4(K1(a, i - 1, j), K1(a, i - 1, j + 1), K1(a, i + 1, j), K1(a, i + 1, j + 1)) <= k)
            tv5 = -(RHO(a, i + 1, j + 1, k) - RHO(a, i - 1, j + 1, k) + RHO(a, i + 1, j, k) - RHO(a, i - 1, j, k)) * rdphi * 0.25 *
                  a.rcv[j - 1];
        else if (imax2(K1(a, i - 1, j), K1(a, i - 1, j + 1)) <= k)
            tv5 = -(RHO(a, i, j + 1, k) - RHO(a, i - 1, j + 1, k) + RHO(a, i, j, k) - RHO(a, i - 1, j, k)) * rdphi * 0.5 * a.rcv[j - 1];
        else if (imax2(K1(a, i + 1, j), K1(a, i + 1, j + 1)) <= k)
            tv5 = -(RHO(a, i + 1, j + 1, k) - RHO(a, i, j + 1, k) + RHO(a, i + 1, j, k) - RHO(a, i, j, k)) * rdphi * 0.5 * a.rcv[j - 1];
        else
            tv5 = 0;
    }
    if (k == a.maxk) {
        if (K1(a, i + 1, j) <= k) {
            tv1 = tv1 - TAU(a.dztau, a, 2, i, j);
            tv2 = tv2 - TAU(a.dztau, a, 1, i, j);
        }
        if (K1(a, i, j + 1) <= k) {
            tv4 = tv4 - TAU(a.dztav, a, 2, i, j);
            tv5 = tv5 - TAU(a.dztav, a, 1, i, j);
        }
    }
    const size_t ij = (size_t)(i - 1) + (size_t)a.maxi * (j - 1);
    a.dzu[(size_t)t] = -(a.s[j] * tv1 + DRAG(a, 1, i, j) * tv2) * a.rtv[ij];
    a.dzu[(size_t)t + (size_t)ncol * a.maxk] = -(DRAG(a, 2, i, j) * tv4 - a.sv[j] * tv5) * a.rtv3[ij];
}

// velc :3641-3662: the vertical integration of dzu, the barotropic part and the relaxation,
// one column per thread, 32 columns per block; the i = maxi thread also makes u(1,0,j,:).
// The column's dzu and u1 are first loaded into shared memory for every level at once, so
// that only the FP64 additions remain on the per-level chain.
__global__ void __launch_bounds__(32) k_velc(MoDev a)
{
    extern __shared__ double vsm[];   // [6][maxk][32]: dzu(1), dzu(2), u1(1), u1(2), u(1), u(2)
    const int lane = threadIdx.x;
    const int t = blockIdx.x * blockDim.x + lane;
    const int ncol = a.maxi * a.maxj, maxk = a.maxk;
    const bool on = t < ncol;
    const int i = on ? t % a.maxi + 1 : 1, j = on ? t / a.maxi + 1 : 1;
    const int k1 = on ? K1(a, i, j) : maxk + 1;
    auto S = [&](int q, int k) -> double & { return vsm[((size_t)q * maxk + (k - 1)) * 32 + lane]; };
    for (int k = k1; k <= maxk; ++k) {
        S(0, k) = a.dzu[(size_t)t + (size_t)ncol * (k - 1)];
        S(1, k) = a.dzu[(size_t)t + (size_t)ncol * (k - 1) + (size_t)ncol * maxk];
        S(2, k) = a.u1[Ui(a, 1, i, j, k)];
        S(3, k) = a.u1[Ui(a, 2, i, j, k)];
    }
    if (!on) return;
    const double rel = a.rel;
    double sum[2] = {0.0, 0.0};
    for (int l = 0; l < 2; ++l) {
        double prev = 0.0, uprev = 0.0;
        for (int k = k1; k <= maxk; ++k) {
            const double d = S(l, k);
            if (k == k1) {
                uprev = 0;
            } else {
                uprev = uprev + a.dza[k - 2] * (d + prev) * 0.5;
                sum[l] = sum[l] + a.dz[k - 1] * uprev;
            }
            S(4 + l, k) = uprev;
            prev = d;
        }
    }
    const int k1e = K1(a, i + 1, j), k1n = K1(a, i, j + 1);
    const double rh1 = RH(a, 1, i, j), rh2 = RH(a, 2, i, j);
    const double ub1 = a.ub[UBi(a, 1, i, j)], ub2 = a.ub[UBi(a, 2, i, j)];
    for (int k = k1; k <= maxk; ++k) {
        double v1 = S(4, k), v2 = S(5, k);
        if (k1e <= k) {
            v1 = v1 - sum[0] * rh1 + ub1;
            v1 = rel * S(2, k) + (1.0 - rel) * v1;
            a.u1[Ui(a, 1, i, j, k)] = v1;
        }
        if (k1n <= k) {
            v2 = v2 - sum[1] * rh2 + ub2;
            v2 = rel * S(3, k) + (1.0 - rel) * v2;
            a.u1[Ui(a, 2, i, j, k)] = v2;
        }
        a.u[Ui(a, 1, i, j, k)] = v1;
        a.u[Ui(a, 2, i, j, k)] = v2;
    }
    if (i == a.maxi) {
        const int k1w = K1(a, 1, j);
        for (int k = k1w; k <= maxk; ++k) a.u[Ui(a, 1, 0, j, k)] = a.u[Ui(a, 1, a.maxi, j, k)];
    }
}

// w from continuity (velc :3666-3678)
__global__ void __launch_bounds__(32) k_w(MoDev a)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.maxi * a.maxj) return;
    const int i = t % a.maxi + 1, j = t / a.maxi + 1;
    double tv = 0;
    for (int k = K1(a, i, j); k <= a.maxk - 1; ++k) {
        const double tv1 = (a.u[Ui(a, 1, i, j, k)] - a.u[Ui(a, 1, i - 1, j, k)]) * a.rdphi * a.rc[j];
        const double tv2 = (a.u[Ui(a, 2, i, j, k)] * a.cv[j] - a.u[Ui(a, 2, i, j - 1, k)] * a.cv[j - 1]) * a.rds[j - 1];
        const double w = tv - a.dz[k - 1] * (tv1 + tv2);
        a.u[Ui(a, 3, i, j, k)] = w;
        tv = w;
    }
}

// ---------------------------------------------------------------------------
// host: the reference's initialisation
struct HostGrid {
    gb_mo_dims d;
    gb_mo_params p;
    std::vector<double> s, c, sv, cv, rc, rcv, dsv, rdsv, ds, rds, rds2, dz, dza, rh, drag, rtv, rtv3, psiles;
    std::vector<int32_t> k1, ku, mk, getj, npi, lpisl, ipisl, jpisl;
};

struct HostInit {
    int n = 0, nm = 0;
    std::vector<double> gap, ratm;   // (nm, 2n+3), (nm, n+1)
    std::vector<double> ubisl, psisl, erisl;
};

// band matrix of invert (goldstein.f90:3138-3188), before the elimination
void host_band(const HostGrid &G, HostInit &I)
{
    const int maxi = G.d.maxi, maxj = G.d.maxj, maxk = G.d.maxk, n = maxi, nm = I.nm;
    const double dphi = G.p.dphi, rdphi = G.p.rdphi;
    auto K1 = [&](int i, int j) { return G.k1[i + (size_t)(maxi + 2) * j]; };
    auto RH = [&](int l, int i, int j) { return G.rh[(l - 1) + 3 * ((size_t)i + (size_t)(maxi + 2) * j)]; };
    auto DRAG = [&](int l, int i, int j) { return G.drag[(l - 1) + 2 * ((size_t)(i - 1) + (size_t)(maxi + 1) * (j - 1))]; };
    auto GAP = [&](int r, int cc) -> double & { return I.gap[(size_t)(r - 1) + (size_t)nm * (cc - 1)]; };
    I.gap.assign((size_t)nm * (2 * n + 3), 0.0);
    for (int i = 1; i <= maxi; ++i)
        for (int j = 0; j <= maxj; ++j) {
            const int k = i + j * n;
            if (std::max(std::max(K1(i, j), K1(i + 1, j)), std::max(K1(i, j + 1), K1(i + 1, j + 1))) <= maxk) {
                const double dsvj = G.dsv[j - 1], rcvj = G.rcv[j - 1];
                const double tv = (G.s[j + 1] * RH(1, i, j + 1) - G.s[j] * RH(1, i, j)) / (2.0 * dsvj * dphi);
                const double tv1 = (G.sv[j] * RH(2, i + 1, j) - G.sv[j] * RH(2, i, j)) / (2.0 * dphi * dsvj);
                GAP(k, 2) = DRAG(1, i, j) * G.c[j] * G.c[j] * RH(1, i, j) / (G.ds[j - 1] * dsvj) + tv1;
                GAP(k, i == 1 ? 2 * n + 1 : n + 1) = DRAG(2, i, j) * rcvj * rcvj * rdphi * rdphi * RH(2, i, j) - tv;
                GAP(k, n + 2) = -((DRAG(2, i, j) * RH(2, i, j) + DRAG(2, i + 1, j) * RH(2, i + 1, j)) / (G.cv[j] * G.cv[j] * dphi * dphi)) -
                                (DRAG(1, i, j) * G.c[j] * G.c[j] * RH(1, i, j) / G.ds[j - 1] +
                                 DRAG(1, i, j + 1) * G.c[j + 1] * G.c[j + 1] * RH(1, i, j + 1) / G.ds[j]) /
                                    dsvj;
                GAP(k, i == maxi ? 3 : n + 3) = DRAG(2, i + 1, j) * RH(2, i + 1, j) / (G.cv[j] * G.cv[j] * dphi * dphi) + tv;
                GAP(k, 2 * n + 2) = DRAG(1, i, j + 1) * G.c[j + 1] * G.c[j + 1] * RH(1, i, j + 1) / (G.ds[j] * dsvj) - tv1;
            } else {
                GAP(k, n + 2) = 1;
            }
        }
}

// the elimination of invert (goldstein.f90:3189-3204) on the band matrix
void host_eliminate(HostInit &I)
{
    const int n = I.n, nm = I.nm;
    auto GAP = [&](int r, int cc) -> double & { return I.gap[(size_t)(r - 1) + (size_t)nm * (cc - 1)]; };
    I.ratm.assign((size_t)nm * (n + 1), 0.0);
    for (int i = 1; i <= nm - 1; ++i) {
        const int im = std::min(i + n + 1, nm);
        for (int j = i + 1; j <= im; ++j) {
            const double rat = GAP(j, n + 2 - j + i) / GAP(i, n + 2);
            I.ratm[(size_t)(j - 1) + (size_t)nm * (j - i - 1)] = rat;
            if (rat != 0)
                for (int k = n + 2 - j + i; k <= 2 * n + 3 - j + i; ++k) GAP(j, k) = GAP(j, k) - rat * GAP(i, k + j - i);
        }
    }
}

// the banded substitution of ubarsolv (:3511-3524) on gb (nm)
void host_solve(const HostInit &I, double *gb)
{
    const int n = I.n, nm = I.nm;
    auto GAP = [&](int r, int cc) { return I.gap[(size_t)(r - 1) + (size_t)nm * (cc - 1)]; };
    for (int i = 1; i <= nm - 1; ++i) {
        const int im = std::min(i + n + 1, nm);
        for (int j = i + 1; j <= im; ++j) gb[j - 1] = gb[j - 1] - I.ratm[(size_t)(j - 1) + (size_t)nm * (j - i - 1)] * gb[i - 1];
    }
    gb[nm - 1] = gb[nm - 1] / GAP(nm, n + 2);
    for (int i = nm - 1; i >= 1; --i) {
        const int km = std::min(n + 1, nm - i);
        for (int k = 1; k <= km; ++k) gb[i - 1] = gb[i - 1] - GAP(i, n + 2 + k) * gb[i + k - 1];
        gb[i - 1] = gb[i - 1] / GAP(i, n + 2);
    }
}

// Block-tridiagonal factors of the band matrix (before elimination): blocks of n = maxi rows,
// block j = psi row j.  T_j = S_j^-1 (row-major) with S_j = D_j - diag(l_j) T_{j-1} diag(u_{j-1}),
// each S_j factored by LU without pivoting (the reference's band elimination pivots on the
// diagonal too, so the leading minors it divides by are those of the S_j) and inverted column
// by column on host threads.
struct HostBT {
    int n = 0, J = 0;
    std::vector<double> T, l, u;   // (J+1)*n*n, (J+1)*n, (J+1)*n
};

int host_bt_factor(const HostInit &I, HostBT &B)
{
    const int n = I.n, nm = I.nm, J = nm / n - 1;
    auto GAP = [&](int r, int cc) { return I.gap[(size_t)(r - 1) + (size_t)nm * (cc - 1)]; };
    B.n = n;
    B.J = J;
    B.T.assign((size_t)(J + 1) * n * n, 0.0);
    B.l.assign((size_t)(J + 1) * n, 0.0);
    B.u.assign((size_t)(J + 1) * n, 0.0);
    std::vector<double> S((size_t)n * n);
    const int nt = std::max(1, std::min<int>(16, (int)std::thread::hardware_concurrency()));
    for (int j = 0; j <= J; ++j) {
        // D_j and the couplings from the band rows of block j
        std::fill(S.begin(), S.end(), 0.0);
        for (int a = 0; a < n; ++a) {
            const int k = a + 1 + j * n;
            for (int c = 1; c <= 2 * n + 3; ++c) {
                const double v = GAP(k, c);
                if (v == 0.0) continue;
                const int kk = k + c - (n + 2);
                if (kk < 1 || kk > nm) return GB_GO_EINVAL;
                const int jj = (kk - 1) / n, b = (kk - 1) % n;
                if (jj == j) S[(size_t)a * n + b] += v;
                else if (jj == j - 1 && b == a) B.l[(size_t)j * n + a] = v;
                else if (jj == j + 1 && b == a) B.u[(size_t)j * n + a] = v;
                else return GB_GO_EINVAL;
            }
        }
        if (j > 0) {
            const double *Tp = B.T.data() + (size_t)(j - 1) * n * n;
            const double *l = B.l.data() + (size_t)j * n, *up = B.u.data() + (size_t)(j - 1) * n;
            for (int a = 0; a < n; ++a)
                if (l[a] != 0.0)
                    for (int b = 0; b < n; ++b) S[(size_t)a * n + b] -= l[a] * Tp[(size_t)a * n + b] * up[b];
        }
        // LU without pivoting, in place (unit lower L below the diagonal)
        for (int p = 0; p < n; ++p) {
            const double d = S[(size_t)p * n + p];
            if (d == 0.0 || !std::isfinite(d)) return GB_GO_ERANGE;
            for (int r = p + 1; r < n; ++r) {
                const double f = S[(size_t)r * n + p] / d;
                S[(size_t)r * n + p] = f;
                if (f != 0.0) {
                    double *Sr = S.data() + (size_t)r * n;
                    const double *Sp = S.data() + (size_t)p * n;
                    for (int c = p + 1; c < n; ++c) Sr[c] -= f * Sp[c];
                }
            }
        }
        // T_j = S_j^-1, column c from L U x = e_c (threads over columns)
        double *T = B.T.data() + (size_t)j * n * n;
        std::vector<std::thread> th;
        for (int w = 0; w < nt; ++w)
            th.emplace_back([&, w]() {
                std::vector<double> x((size_t)n);
                for (int c = w; c < n; c += nt) {
                    std::fill(x.begin(), x.end(), 0.0);
                    x[c] = 1.0;
                    for (int r = c + 1; r < n; ++r) {
                        double v = x[r];
                        const double *Lr = S.data() + (size_t)r * n;
                        for (int p = c; p < r; ++p) v -= Lr[p] * x[p];
                        x[r] = v;
                    }
                    for (int r = n - 1; r >= 0; --r) {
                        double v = x[r];
                        const double *Ur = S.data() + (size_t)r * n;
                        for (int p = r + 1; p < n; ++p) v -= Ur[p] * x[p];
                        x[r] = v / Ur[r];
                    }
                    for (int r = 0; r < n; ++r) T[(size_t)r * n + c] = x[r];
                }
            });
        for (auto &t : th) t.join();
    }
    return GB_GO_OK;
}

// The block-tridiagonal solve on the host (unit-source solves of the initialisation)
void host_bt_solve(const HostBT &B, double *gb)
{
    const int n = B.n, J = B.J;
    std::vector<double> z((size_t)(J + 1) * n), y((size_t)n);
    for (int j = 0; j <= J; ++j) {
        for (int b = 0; b < n; ++b) y[b] = j > 0 ? gb[(size_t)j * n + b] - B.l[(size_t)j * n + b] * z[(size_t)(j - 1) * n + b]
                                                 : gb[b];
        const double *T = B.T.data() + (size_t)j * n * n;
        for (int a = 0; a < n; ++a) {
            double s = 0.0;
            for (int b = 0; b < n; ++b) s += T[(size_t)a * n + b] * y[b];
            z[(size_t)j * n + a] = s;
        }
    }
    for (int j = J - 1; j >= 0; --j) {
        const double *T = B.T.data() + (size_t)j * n * n;
        for (int b = 0; b < n; ++b) y[b] = B.u[(size_t)j * n + b] * z[(size_t)(j + 1) * n + b];
        for (int a = 0; a < n; ++a) {
            double s = 0.0;
            for (int b = 0; b < n; ++b) s += T[(size_t)a * n + b] * y[b];
            z[(size_t)j * n + a] -= s;
        }
    }
    std::copy(z.begin(), z.end(), gb);
}

// ubarsolv's psi and ub from a solved gb (:3527-3564), into zero-initialised psi, ub
void host_psi_ub(const HostGrid &G, const double *gb, double *psi, double *ub)
{
    const int maxi = G.d.maxi, maxj = G.d.maxj, n = maxi;
    auto PSI = [&](int i, int j) -> double & { return psi[(size_t)i + (size_t)(maxi + 1) * j]; };
    auto UB = [&](int l, int i, int j) -> double & { return ub[(l - 1) + 2 * ((size_t)i + (size_t)(maxi + 2) * j)]; };
    auto RH = [&](int l, int i, int j) { return G.rh[(l - 1) + 3 * ((size_t)i + (size_t)(maxi + 2) * j)]; };
    for (int j = 0; j <= maxj; ++j) {
        for (int i = 1; i <= maxi; ++i) PSI(i, j) = gb[i + j * n - 1];
        PSI(0, j) = PSI(maxi, j);
    }
    for (int j = 1; j <= maxj; ++j)
        for (int i = 1; i <= maxi; ++i) UB(1, i, j) = -RH(1, i, j) * G.c[j] * (PSI(i, j) - PSI(i, j - 1)) * G.rds[j - 1];
    for (int j = 1; j <= maxj - 1; ++j)
        for (int i = 1; i <= maxi; ++i) UB(2, i, j) = RH(2, i, j) * (PSI(i, j) - PSI(i - 1, j)) * G.rcv[j - 1] * G.p.rdphi;
    for (int i = 1; i <= maxi; ++i) {
        UB(2, i, maxj) = 0.0;
        UB(2, i, 0) = 0.0;
    }
    for (int j = 1; j <= maxj; ++j) {
        UB(2, maxi + 1, j) = UB(2, 1, j);
        UB(1, 0, j) = UB(1, maxi, j);
        UB(1, maxi + 1, j) = UB(1, 1, j);
        UB(2, 0, j) = UB(2, maxi, j);
    }
    UB(2, maxi + 1, 0) = UB(2, 1, 0);
    UB(2, 0, 0) = UB(2, maxi, 0);
}

// the island integral without the J term and the wind (island, indj = 0)
double host_island0(const HostGrid &G, const double *ub, int isl)
{
    const int maxi = G.d.maxi;
    auto UB = [&](int l, int i, int j) { return ub[(l - 1) + 2 * ((size_t)i + (size_t)(maxi + 2) * j)]; };
    auto RH = [&](int l, int i, int j) { return G.rh[(l - 1) + 3 * ((size_t)i + (size_t)(maxi + 2) * j)]; };
    auto DRAG = [&](int l, int i, int j) { return G.drag[(l - 1) + 2 * ((size_t)(i - 1) + (size_t)(maxi + 1) * (j - 1))]; };
    double e = 0.0;
    for (int p = 1; p <= G.npi[isl - 1]; ++p) {
        const size_t q = (size_t)(p - 1) + (size_t)G.d.mpi * (isl - 1);
        const int lpi = G.lpisl[q], ipi = G.ipisl[q], jpi = G.jpisl[q];
        const int al = std::abs(lpi);
        const double sg = lpi >= 0 ? 1.0 : -1.0;
        double cor;
        if (al == 1)
            cor = -G.s[jpi] * 0.25 * (UB(2, ipi, jpi) + UB(2, ipi + 1, jpi) + UB(2, ipi, jpi - 1) + UB(2, ipi + 1, jpi - 1));
        else
            cor = G.sv[jpi] * 0.25 * (UB(1, ipi - 1, jpi) + UB(1, ipi, jpi) + UB(1, ipi - 1, jpi + 1) + UB(1, ipi, jpi + 1));
        e = e + sg * (DRAG(al, ipi, jpi) * UB(al, ipi, jpi) + cor - 0.0 * RH(al, ipi, jpi)) *
                    (G.c[jpi] * G.p.dphi * (2.0 - al) + G.rcv[jpi - 1] * G.dsv[jpi - 1] * (al - 1.0));
    }
    return e;
}

template <class T>
void copy_in(std::vector<T> &v, const T *p, size_t n)
{
    v.assign(p, p + n);
}

}  // namespace

struct gb_mo {
    int device = 0;
    cudaStream_t stream = nullptr;
    MoDev dev{};
    // the step's launches as a CUDA graph, captured for one ocean handle's density, velocity
    // buffer and stream (re-captured when those change)
    cudaGraphExec_t graph = nullptr;
    const double *graph_rho = nullptr;
    double *graph_u = nullptr;
    cudaStream_t graph_stream = nullptr;
    std::vector<void *> allocs;
    bool have_wind = false;
    std::string last_error;
};

static int mfail(gb_mo *h, int code, const std::string &msg)
{
    if (h) h->last_error = msg;
    return code;
}

#define MO_TRY(h, call)                                                                                   \
    do {                                                                                                  \
        cudaError_t _e = (call);                                                                          \
        if (_e != cudaSuccess)                                                                            \
            return mfail(h, _e == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA,                 \
                         std::string(#call) + ": " + cudaGetErrorString(_e));                             \
    } while (0)

template <class T>
static cudaError_t dev_copy(gb_mo *h, const T **dst, const std::vector<T> &v)
{
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(1, v.size()) * sizeof(T));
    if (e != cudaSuccess) return e;
    h->allocs.push_back(p);
    *dst = static_cast<const T *>(p);
    if (!v.empty()) e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

template <class T>
static cudaError_t dev_zero(gb_mo *h, T **dst, size_t n)
{
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T));
    if (e != cudaSuccess) return e;
    h->allocs.push_back(p);
    *dst = static_cast<T *>(p);
    return cudaMemset(p, 0, std::max<size_t>(1, n) * sizeof(T));
}

extern "C" int gb_mo_create(const gb_mo_dims *dims, const gb_mo_params *params, const gb_mo_grid *grid, int device, gb_mo **out)
{
    if (!out) return GB_GO_EINVAL;
    *out = nullptr;
    if (!dims || !params || !grid) return GB_GO_EINVAL;
    const gb_mo_dims d = *dims;
    if (d.maxi < 3 || d.maxj < 3 || d.maxk < 1 || d.maxk > GB_GO_MAX_K || d.isles < 1 || d.isles > 32 || d.mpi < 1)
        return GB_GO_EINVAL;
    const long long nm = (long long)d.maxi * (d.maxj + 1);
    if (d.maxi > GB_MO_MAX_ROW || nm > GB_MO_MAX_PSI_BT) return GB_GO_ERANGE;
    if (d.solver != 0 && d.solver != 1) return GB_GO_EINVAL;
    const bool bt = nm > GB_MO_MAX_PSI || d.solver == 1;   // the block-tridiagonal solve instead of the inverse
    const gb_mo_grid &g = *grid;
    const void *need[] = {g.s, g.c, g.sv, g.cv, g.rc, g.rcv, g.dsv, g.rdsv, g.ds, g.rds, g.rds2, g.dz, g.dza, g.k1, g.ku,
                          g.mk, g.getj, g.rh, g.drag, g.rtv, g.rtv3, g.psiles, g.npi, g.lpisl, g.ipisl, g.jpisl};
    for (const void *q : need)
        if (!q) return GB_GO_EINVAL;
    const int maxi = d.maxi, maxj = d.maxj, maxk = d.maxk;
    // the island paths stay on interior velocity points (the integral reads ub at ipi+-1, jpi+-1)
    for (int isl = 0; isl < d.isles; ++isl) {
        if (g.npi[isl] < 1 || g.npi[isl] > d.mpi) return GB_GO_EINVAL;
        for (int p = 0; p < g.npi[isl]; ++p) {
            const size_t q = (size_t)p + (size_t)d.mpi * isl;
            const int l = std::abs(g.lpisl[q]), ip = g.ipisl[q], jp = g.jpisl[q];
            if ((l != 1 && l != 2) || ip < 1 || ip > maxi || jp < 1 || jp > maxj - 1) return GB_GO_EINVAL;
        }
    }
    for (int i = 0; i <= maxi + 1; ++i)
        if (g.k1[i] <= maxk || g.k1[i + (size_t)(maxi + 2) * (maxj + 1)] <= maxk) return GB_GO_EINVAL;   // land rows 0, maxj+1
    HostGrid G;
    G.d = d;
    G.p = *params;
    const size_t nj1 = (size_t)maxj + 1, nj_1 = (size_t)std::max(1, maxj - 1);
    copy_in(G.s, g.s, nj1); copy_in(G.c, g.c, nj1); copy_in(G.sv, g.sv, nj1); copy_in(G.cv, g.cv, nj1); copy_in(G.rc, g.rc, nj1);
    copy_in(G.rcv, g.rcv, nj_1); copy_in(G.dsv, g.dsv, nj_1); copy_in(G.rdsv, g.rdsv, nj_1);
    copy_in(G.ds, g.ds, (size_t)maxj); copy_in(G.rds, g.rds, (size_t)maxj);
    copy_in(G.rds2, g.rds2, (size_t)std::max(1, maxj - 2));
    copy_in(G.dz, g.dz, (size_t)maxk); copy_in(G.dza, g.dza, (size_t)maxk);
    copy_in(G.k1, g.k1, (size_t)(maxi + 2) * (maxj + 2));
    copy_in(G.ku, g.ku, 2 * (size_t)maxi * maxj);
    copy_in(G.mk, g.mk, (size_t)(maxi + 1) * maxj);
    copy_in(G.getj, g.getj, (size_t)maxi * maxj);
    copy_in(G.rh, g.rh, 3 * (size_t)(maxi + 2) * (maxj + 2));
    copy_in(G.drag, g.drag, 2 * (size_t)(maxi + 1) * maxj);
    copy_in(G.rtv, g.rtv, (size_t)maxi * maxj); copy_in(G.rtv3, g.rtv3, (size_t)maxi * maxj);
    copy_in(G.psiles, g.psiles, (size_t)nm);
    copy_in(G.npi, g.npi, (size_t)d.isles);
    copy_in(G.lpisl, g.lpisl, (size_t)d.mpi * d.isles);
    copy_in(G.ipisl, g.ipisl, (size_t)d.mpi * d.isles);
    copy_in(G.jpisl, g.jpisl, (size_t)d.mpi * d.isles);

    // initialisation (goldstein.f90:1788-1814)
    HostInit I;
    I.n = maxi;
    I.nm = (int)nm;
    host_band(G, I);
    HostBT B;
    if (bt) {
        const int r = host_bt_factor(I, B);
        if (r) return r;
    } else {
        host_eliminate(I);
    }
    const size_t nub = 2 * (size_t)(maxi + 2) * (maxj + 1), npsi = (size_t)(maxi + 1) * (maxj + 1);
    I.ubisl.assign(nub * d.isles, 0.0);
    I.psisl.assign(npsi * d.isles, 0.0);
    I.erisl.assign((size_t)d.isles * (d.isles + 1), 0.0);
    std::vector<double> gbv((size_t)nm);
    for (int isol = 1; isol <= d.isles; ++isol) {
        for (long long k = 0; k < nm; ++k) gbv[k] = ((int)G.psiles[k] == isol + 1) ? 1.0 : 0.0;
        if (bt) host_bt_solve(B, gbv.data());
        else host_solve(I, gbv.data());
        host_psi_ub(G, gbv.data(), I.psisl.data() + npsi * (isol - 1), I.ubisl.data() + nub * (isol - 1));
        for (int isl = 1; isl <= d.isles; ++isl)
            I.erisl[(size_t)(isl - 1) + (size_t)d.isles * (isol - 1)] = host_island0(G, I.ubisl.data() + nub * (isol - 1), isl);
    }
    {   // matinv_gold (:3452-3467)
        const int nv = d.isles;
        auto A = [&](int r, int cc) -> double & { return I.erisl[(size_t)(r - 1) + (size_t)nv * (cc - 1)]; };
        for (int i = 1; i <= nv - 1; ++i)
            for (int j = i + 1; j <= nv; ++j)
                for (int k = i + 1; k <= nv; ++k) A(j, k) = A(i, i) * A(j, k) - A(j, i) * A(i, k);
    }
    // the explicit inverse, row-major (row r of the inverse is the response of psi(r) to every
    // right-hand side entry): column c = the solve of unit vector c
    std::vector<double> minv(bt ? 0 : (size_t)nm * nm);
    if (!bt) {
        const int nt = std::max(1, std::min<int>(16, (int)std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        for (int w = 0; w < nt; ++w)
            th.emplace_back([&, w]() {
                std::vector<double> x((size_t)nm);
                for (long long col = w; col < nm; col += nt) {
                    std::fill(x.begin(), x.end(), 0.0);
                    x[col] = 1.0;
                    host_solve(I, x.data());
                    for (long long r = 0; r < nm; ++r) minv[(size_t)r * nm + col] = x[r];
                }
            });
        for (auto &t : th) t.join();
    }

    gb_mo *h = new gb_mo();
    if (device < 0) cudaGetDevice(&device);
    h->device = device;
    MoDev &a = h->dev;
    a.maxi = maxi; a.maxj = maxj; a.maxk = maxk; a.isles = d.isles; a.mpi = d.mpi; a.n = maxi; a.nm = (int)nm;
    a.dphi = G.p.dphi; a.rdphi = G.p.rdphi; a.rel = G.p.rel;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
#define UP(field, vec) if (e == cudaSuccess) e = dev_copy(h, &a.field, G.vec)
    UP(s, s); UP(c, c); UP(sv, sv); UP(cv, cv); UP(rc, rc); UP(rcv, rcv); UP(dsv, dsv); UP(rdsv, rdsv); UP(ds, ds);
    UP(rds, rds); UP(rds2, rds2); UP(dz, dz); UP(dza, dza); UP(k1, k1); UP(ku, ku); UP(mk, mk); UP(getj, getj); UP(rh, rh);
    UP(drag, drag); UP(rtv, rtv); UP(rtv3, rtv3); UP(npi, npi); UP(lpisl, lpisl); UP(ipisl, ipisl); UP(jpisl, jpisl);
#undef UP
    a.bt = bt ? 1 : 0;
    if (e == cudaSuccess && !bt) e = dev_copy(h, &a.minv, minv);
    if (e == cudaSuccess && bt) e = dev_copy(h, &a.btT, B.T);
    if (e == cudaSuccess && bt) e = dev_copy(h, &a.btl, B.l);
    if (e == cudaSuccess && bt) e = dev_copy(h, &a.btu, B.u);
    if (e == cudaSuccess && bt) e = dev_zero(h, &a.btz, (size_t)nm);
    if (e == cudaSuccess) e = dev_copy(h, &a.ubisl, I.ubisl);
    if (e == cudaSuccess) e = dev_copy(h, &a.psisl, I.psisl);
    if (e == cudaSuccess) e = dev_copy(h, &a.erisl, I.erisl);
    const size_t nt2 = 2 * (size_t)maxi * maxj, nu = 3 * (size_t)(maxi + 1) * (maxj + 1) * maxk;
    double *tau = nullptr, *dztau = nullptr, *dztav = nullptr;
    if (e == cudaSuccess) e = dev_zero(h, &tau, nt2);
    if (e == cudaSuccess) e = dev_zero(h, &dztau, nt2);
    if (e == cudaSuccess) e = dev_zero(h, &dztav, nt2);
    a.tau = tau; a.dztau = dztau; a.dztav = dztav;
    if (e == cudaSuccess) e = dev_zero(h, &a.psibc, (size_t)d.isles);
    if (e == cudaSuccess) e = dev_zero(h, &a.gb, (size_t)nm);
    if (e == cudaSuccess) e = dev_zero(h, &a.gbold, (size_t)nm);
    if (e == cudaSuccess) e = dev_zero(h, &a.bp, (size_t)(maxi + 1) * maxj * maxk);
    if (e == cudaSuccess) e = dev_zero(h, &a.sbp, (size_t)(maxi + 1) * maxj);
    if (e == cudaSuccess) e = dev_zero(h, &a.ub, nub);
    if (e == cudaSuccess) e = dev_zero(h, &a.psi, npsi);
    if (e == cudaSuccess) e = dev_zero(h, &a.scr, 2 * (size_t)d.isles * d.mpi);   // island path terms
    if (e == cudaSuccess) e = dev_zero(h, &a.dzu, 2 * (size_t)maxi * maxj * maxk);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_velc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(6 * (size_t)maxk * 32 * sizeof(double)));
    if (e == cudaSuccess) e = dev_zero(h, &a.u, nu);
    if (e == cudaSuccess) e = dev_zero(h, &a.u1, nu);
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA;
        gb_mo_destroy(h);
        return code;
    }
    *out = h;
    return GB_GO_OK;
}

extern "C" void gb_mo_destroy(gb_mo *h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (void *p : h->allocs) cudaFree(p);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

extern "C" const char *gb_mo_last_error(const gb_mo *h) { return h ? h->last_error.c_str() : ""; }

extern "C" int gb_mo_set_wind(gb_mo *h, const double *tau, const double *dztau, const double *dztav)
{
    if (!h || !tau || !dztau || !dztav) return mfail(h, GB_GO_EINVAL, "set_wind: NULL array");
    MO_TRY(h, cudaSetDevice(h->device));
    const size_t n = 2 * (size_t)h->dev.maxi * h->dev.maxj * sizeof(double);
    MO_TRY(h, cudaMemcpyAsync(const_cast<double *>(h->dev.tau), tau, n, cudaMemcpyHostToDevice, h->stream));
    MO_TRY(h, cudaMemcpyAsync(const_cast<double *>(h->dev.dztau), dztau, n, cudaMemcpyHostToDevice, h->stream));
    MO_TRY(h, cudaMemcpyAsync(const_cast<double *>(h->dev.dztav), dztav, n, cudaMemcpyHostToDevice, h->stream));
    MO_TRY(h, cudaStreamSynchronize(h->stream));
    h->have_wind = true;
    return GB_GO_OK;
}

extern "C" int gb_mo_upload_velocity(gb_mo *h, const double *u, const double *u1)
{
    if (!h || !u || !u1) return mfail(h, GB_GO_EINVAL, "upload_velocity: NULL array");
    MO_TRY(h, cudaSetDevice(h->device));
    const size_t n = 3 * (size_t)(h->dev.maxi + 1) * (h->dev.maxj + 1) * h->dev.maxk * sizeof(double);
    MO_TRY(h, cudaMemcpyAsync(h->dev.u, u, n, cudaMemcpyHostToDevice, h->stream));
    MO_TRY(h, cudaMemcpyAsync(h->dev.u1, u1, n, cudaMemcpyHostToDevice, h->stream));
    MO_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}

static int launch_step(const MoDev &a, cudaStream_t s, double *ocean_u);

extern "C" int gb_mo_step(gb_mo *h, gb_go_handle *ocean)
{
    gbgo::TraceRange tr_("mo_step");
    if (!h || !ocean) return mfail(h, GB_GO_EINVAL, "step: NULL handle");
    if (!h->have_wind) return mfail(h, GB_GO_ENOTREADY, "step before set_wind");
    OceanState o{};
    if (ocean_state(ocean, &o) != GB_GO_OK) return mfail(h, GB_GO_EINVAL, "step: bad ocean handle");
    if (!o.state_ready) return mfail(h, GB_GO_ENOTREADY, "step: ocean state not uploaded");
    MoDev a = h->dev;
    if (o.d.maxi != a.maxi || o.d.maxj != a.maxj || o.d.maxk != a.maxk)
        return mfail(h, GB_GO_EINVAL, "step: ocean grid differs from the momentum grid");
    if (o.device != h->device) return mfail(h, GB_GO_EINVAL, "step: handles on different devices");
    MO_TRY(h, cudaSetDevice(h->device));
    // the split-precision form's density is formed from its current state first
    if (const int rr = ocean_refresh_rho_only(ocean)) return mfail(h, rr, std::string("step: ") + gb_go_last_error(ocean));
    cudaStream_t s = static_cast<cudaStream_t>(o.stream);
    a.rho = o.rho;
    if (h->graph && (h->graph_rho != o.rho || h->graph_u != o.u || h->graph_stream != s)) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    if (!h->graph) {
        cudaGraph_t gr = nullptr;
        MO_TRY(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int r = launch_step(a, s, o.u);
        cudaError_t e = cudaStreamEndCapture(s, &gr);
        if (r || e != cudaSuccess) {
            if (gr) cudaGraphDestroy(gr);
            return mfail(h, GB_GO_ECUDA, std::string("step: graph capture failed: ") + cudaGetErrorString(e));
        }
        e = cudaGraphInstantiate(&h->graph, gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) {
            h->graph = nullptr;
            return mfail(h, GB_GO_ECUDA, std::string("step: graph instantiation failed: ") + cudaGetErrorString(e));
        }
        h->graph_rho = o.rho;
        h->graph_u = o.u;
        h->graph_stream = s;
    }
    MO_TRY(h, cudaGraphLaunch(h->graph, s));
    count_launches(a.bt ? 8 + 2 * (a.nm / a.maxi) : 9);
    // the split-precision form rebuilds its transfer coefficients from the new velocities
    const int r = ocean_velocity_changed(ocean);
    if (r != GB_GO_OK) return mfail(h, r, std::string("step: ") + gb_go_last_error(ocean));
    MO_TRY(h, cudaStreamSynchronize(s));
    return GB_GO_OK;
}

// the step's kernels and the copy of the new velocities into the ocean handle's buffer
static int launch_step(const MoDev &a, cudaStream_t s, double *ocean_u)
{
    const int ncol = a.maxi * a.maxj;
    const size_t nub = 2 * (size_t)(a.maxi + 2) * (a.maxj + 1), npsi = (size_t)(a.maxi + 1) * (a.maxj + 1);
    // blocks of one warp for the per-column kernels: their FP64 chains then spread over many
    // SMs (GB300's FP64 pipe is ~2 lanes per clock per SM)
    k_bp<<<(ncol + 31) / 32, 32, 0, s>>>(a);
    k_rhs<<<(a.nm + 31) / 32, 32, 0, s>>>(a);
    if (a.bt) {
        const int nb = (a.maxi + kBtRowsPerBlock - 1) / kBtRowsPerBlock, J = a.nm / a.maxi - 1;
        const int nt = kBtRowThreads * kBtRowsPerBlock;
        for (int j = 0; j <= J; ++j) k_bt_forward<<<nb, nt, 0, s>>>(a, j);
        for (int j = J - 1; j >= 0; --j) k_bt_backward<<<nb, nt, 0, s>>>(a, j);
        k_bt_psi<<<(a.nm + 127) / 128, 128, 0, s>>>(a);
    } else {
        k_psi<<<(a.nm * 32 + 255) / 256, 256, 0, s>>>(a);
    }
    k_ub<<<((a.maxi + 2) * (a.maxj + 1) + 127) / 128, 128, 0, s>>>(a);
    k_island<<<1, 256, 0, s>>>(a, a.scr);
    k_corr<<<(unsigned)((nub + npsi + 127) / 128), 128, 0, s>>>(a);
    k_dzu<<<(unsigned)(((size_t)ncol * a.maxk + 127) / 128), 128, 0, s>>>(a);
    k_velc<<<(ncol + 31) / 32, 32, 6 * (size_t)a.maxk * 32 * sizeof(double), s>>>(a);
    k_w<<<(ncol + 31) / 32, 32, 0, s>>>(a);
    if (cudaGetLastError() != cudaSuccess) return GB_GO_ECUDA;
    // the new velocities are the ocean handle's for its next tstepo
    const size_t nu = 3 * (size_t)(a.maxi + 1) * (a.maxj + 1) * a.maxk;
    return cudaMemcpyAsync(ocean_u, a.u, nu * sizeof(double), cudaMemcpyDeviceToDevice, s) == cudaSuccess ? 0 : GB_GO_ECUDA;
}

extern "C" int gb_mo_download(gb_mo *h, double *u, double *u1, double *ub, double *psi)
{
    if (!h) return GB_GO_EINVAL;
    MO_TRY(h, cudaSetDevice(h->device));
    const MoDev &a = h->dev;
    const size_t nu = 3 * (size_t)(a.maxi + 1) * (a.maxj + 1) * a.maxk;
    if (u) MO_TRY(h, cudaMemcpyAsync(u, a.u, nu * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (u1) MO_TRY(h, cudaMemcpyAsync(u1, a.u1, nu * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (ub) MO_TRY(h, cudaMemcpyAsync(ub, a.ub, 2 * (size_t)(a.maxi + 2) * (a.maxj + 1) * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (psi) MO_TRY(h, cudaMemcpyAsync(psi, a.psi, (size_t)(a.maxi + 1) * (a.maxj + 1) * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    MO_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}
