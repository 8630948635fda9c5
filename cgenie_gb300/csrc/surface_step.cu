// 2-D surface steppers on the device: the EMBM atmosphere step tstipa
// (src/embm/embm.f90:2039-2138) and the sea-ice transport steps tstipsic
// (src/goldsteinseaice/gold_seaice.f90:937-1058, iterative implicit) and tstepsic (:844-929,
// explicit), behind include/gb_embm.h.
//
// One thread-block cluster per tracer (the two tracers never interact), its blocks splitting the
// rows: GB300's FP64 pipe is ~2 lanes per clock per SM, so the grid's FP64 work is spread over
// up to 8 SMs per tracer.  Each block keeps its rows' face coefficients and Jacobi iterate in
// shared memory and its cells' tq, tq1 and source in registers; the four iterations and the
// corrector are separated by cluster barriers, with the halo rows of the iterate read from the
// neighbouring blocks' shared memory, instead of kernel launches.  A launch runs nsteps steps
// (the coefficients depend only on the forcing, fixed within a launch).  Compiled with
// -fmad=false: every expression rounds as the reference's.
#include "../../include/gb_embm.h"
#include "gb_internal.h"

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

using namespace gbgo;

namespace {

constexpr int kThreads = 1024;
constexpr int kClusterMax = 16;        // blocks per tracer (GB300 runs clusters of 16 when opted in)
constexpr int kCellsPerThread = 4;     // cells of one block: at most kThreads * kCellsPerThread

struct EaArgs {
    int maxi, maxj, maxk, kind, nsteps;
    double dt, dphi, rdphi, betaz[2], betam[2], diffmod0, ppmin, ppmax, diffsic, tsc;
    double sica, sich;
    const double *rc, *cv, *dsv, *rdsv, *rds, *diffa;
    const int32_t *k1;
    double *tq, *tq1;
    const double *src, *vel, *pptn;
    double *dth, *ddy;   // sea ice: variceth, varicedy (2, maxi, maxj)
    double rhoio, rhoice, hlf, hmin, rdtdim, m2mm;   // sea ice: step_seaice's post-processing
    double *fx, *fw;     // sea ice: fx_delta, fw_delta (maxi, maxj)
};

__device__ __forceinline__ double clamp01(double x)
{
    // MAX(0.0, MIN(1.0, x)) (embm.f90:2065-2066)
    const double m = 1.0 < x ? 1.0 : x;
    return 0.0 > m ? 0.0 : m;
}

// Face coefficients of cell (i, j) for tracer l: east (cie, ciw) and north (cin, cis) faces.
__device__ __forceinline__ void face_coefs(const EaArgs &a, int l, int i, int j, double *e_, double *w_, double *n_,
                                           double *s_)
{
    const int maxi = a.maxi, maxj = a.maxj;
    const size_t c = (size_t)(i - 1) + (size_t)maxi * (j - 1);
    const double u1 = a.vel[2 * c], u2 = a.vel[2 * c + 1];
    const double rcj = a.rc[j], cvj = a.cv[j];
    double e, w, n, s;
    if (a.kind == GB_EA_EMBM) {
        // embm.f90:2061-2088
        const double clampp = clamp01((a.pptn[c] - a.ppmin) / (a.ppmax - a.ppmin));
        const double bz = a.betaz[l - 1], bm = a.betam[l - 1];
        const double fac = (double)(2 - l) * a.diffmod0;
        e = bz * u1 * rcj * 0.5 * a.rdphi;
        double diffpp = a.diffa[(l - 1) + 2 * (0 + 2 * (size_t)(j - 1))] + fac * clampp;
        double tv = rcj * rcj * a.rdphi * diffpp * a.rdphi;
        double pec = bz * u1 * a.dphi / diffpp;
        double ups = pec / (2.0 + fabs(pec));
        w = e * (1 + ups) + tv;
        e = e * (1 - ups) - tv;
        n = cvj * bm * u2 * 0.5;
        const double da2 = a.diffa[(l - 1) + 2 * (1 + 2 * (size_t)(j - 1))];
        diffpp = da2 + fac * clampp;
        if (j < maxj) {
            tv = cvj * cvj * a.rdsv[j - 1] * da2;
            pec = bm * u2 * a.dsv[j - 1] / diffpp;
            ups = pec / (2.0 + fabs(pec));
        } else {
            tv = 0.0;
            ups = 0.0;
        }
        s = n * (1 + ups) + tv;
        n = n * (1 - ups) - tv;
    } else {
        // gold_seaice.f90:966-992
        const int NK = maxi + 2;
        const int k1c = a.k1[i + (size_t)NK * j];
        const int k1e = a.k1[i + 1 + (size_t)NK * j], k1n = a.k1[i + (size_t)NK * (j + 1)];
        if (a.maxk < (k1c > k1e ? k1c : k1e)) {
            e = 0;
            w = 0;
        } else {
            e = u1 * rcj * 0.5 * a.rdphi;
            const double tv = rcj * rcj * a.rdphi * a.diffsic * a.rdphi;
            const double pec = u1 * a.dphi / a.diffsic;
            const double ups = pec / (2.0 + fabs(pec));
            w = e * (1 + ups) + tv;
            e = e * (1 - ups) - tv;
        }
        if (a.maxk < (k1c > k1n ? k1c : k1n)) {
            n = 0;
            s = 0;
        } else {
            n = cvj * u2 * 0.5;
            const double tv = cvj * cvj * a.rdsv[j - 1] * a.diffsic;
            const double pec = u2 * a.dsv[j - 1] / a.diffsic;
            const double ups = pec / (2.0 + fabs(pec));
            s = n * (1 + ups) + tv;
            n = n * (1 - ups) - tv;
        }
    }
    *e_ = e;
    *w_ = w;
    *n_ = n;
    *s_ = s;
}

// One cluster per tracer; cluster rank r holds rows [1 + r*R, min(maxj, (r+1)*R)] (R = rows_per)
// with the face coefficients of those rows (and the north faces of the row below, recomputed
// locally), and the iterate tq2 of those rows plus one halo row on each side, which it copies
// from its neighbours' shared memory (distributed shared memory) after every iterate update.
// Shared-memory layout of every block: cie, ciw (maxi+1) x R; cin, cis (maxi+1) x (R+1) from
// row j0-1; v2 (maxi+2) x (R+2) from row j0-1.
__global__ void __launch_bounds__(kThreads) k_surface_step(const EaArgs *__restrict__ args, int R)
{
    const EaArgs a = args[blockIdx.y];   // one grid per blockIdx.y (gb_ea_step_many)
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ double sm[];
    const int maxi = a.maxi, maxj = a.maxj;
    const int C = (int)cluster.num_blocks(), rank = (int)cluster.block_rank();
    const int l = (int)(blockIdx.x / C) + 1;   // tracer, 1-based
    const int j0 = 1 + rank * R, j1 = min(maxj + 1, j0 + R), nrow = j1 - j0;
    const int NC = maxi + 1, NV = maxi + 2;
    double *cie = sm, *ciw = cie + (size_t)NC * R, *cin = ciw + (size_t)NC * R;
    double *cis = cin + (size_t)NC * (R + 1), *v2 = cis + (size_t)NC * (R + 1);
    const int t = threadIdx.x;
    const int ncell = maxi * nrow;
    const bool ice = a.kind == GB_EA_SEAICE;
    const double cimp = 0.5, dt = a.dt;

    // coefficients of the block's rows; north faces of the row below (0 below j = 1: the
    // boundary rows of embm.f90:2054-2059, gold_seaice.f90:952-957)
    for (int c = t; c < ncell; c += blockDim.x) {
        const int i = c % maxi + 1, j = j0 + c / maxi;
        double e, w, n, s;
        face_coefs(a, l, i, j, &e, &w, &n, &s);
        const int lr = j - j0;
        cie[i + (size_t)NC * lr] = e;
        ciw[i + (size_t)NC * lr] = w;
        cin[i + (size_t)NC * (lr + 1)] = n;
        cis[i + (size_t)NC * (lr + 1)] = s;
    }
    for (int i = 1 + t; i <= maxi; i += blockDim.x) {
        double e, w, n = 0.0, s = 0.0;
        if (j0 > 1) face_coefs(a, l, i, j0 - 1, &e, &w, &n, &s);
        cin[i] = n;
        cis[i] = s;
    }
    __syncthreads();
    for (int lr = t; lr < nrow; lr += blockDim.x) {   // periodic in i: cie(0,j) = cie(maxi,j)
        cie[(size_t)NC * lr] = cie[maxi + (size_t)NC * lr];
        ciw[(size_t)NC * lr] = ciw[maxi + (size_t)NC * lr];
    }
    __syncthreads();

    // the thread's cells: state, source, and the iteration-invariant centre terms
    double tq[kCellsPerThread], tq1[kCellsPerThread], src[kCellsPerThread], cen[kCellsPerThread];
    bool upd[kCellsPerThread];
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r) {
        const int c = t + r * blockDim.x;
        upd[r] = false;
        tq[r] = tq1[r] = src[r] = cen[r] = 0.0;
        if (c >= ncell) continue;
        const int i = c % maxi + 1, j = j0 + c / maxi, lr = j - j0;
        const size_t x = (size_t)(l - 1) + 2 * ((size_t)(i - 1) + (size_t)maxi * (j - 1));
        tq[r] = a.tq[x];
        tq1[r] = a.tq1[x];
        // tstipa: -tqa(l,i,j); tstipsic: -dtha(l,i,j) * tsc
        src[r] = ice ? -a.src[x] * a.tsc : -a.src[x];
        cen[r] = ciw[i + (size_t)NC * lr] - cie[i - 1 + (size_t)NC * lr] +
                 (cis[i + (size_t)NC * (lr + 1)] - cin[i + (size_t)NC * lr]) * a.rds[j - 1];
        upd[r] = !ice || !(a.maxk < a.k1[i + (size_t)(maxi + 2) * j]);
    }
    const double *v2_lo = rank > 0 ? cluster.map_shared_rank(v2, rank - 1) : nullptr;
    const double *v2_hi = j1 <= maxj ? cluster.map_shared_rank(v2, rank + 1) : nullptr;

    for (int step = 0; step < a.nsteps; ++step) {
        for (int it = 0; it < 5; ++it) {
            const bool corr = it == 4;
            // own rows of the iterate: tq2 = cimp*tq + (1-cimp)*tq1; the corrector's average with the last one
#pragma unroll
            for (int r = 0; r < kCellsPerThread; ++r) {
                const int c = t + r * blockDim.x;
                if (c >= ncell) continue;
                const int i = c % maxi + 1, lr = c / maxi + 1;
                const size_t v = (size_t)i + (size_t)NV * lr;
                const double nv = corr ? 0.5 * (v2[v] + cimp * tq[r] + (1.0 - cimp) * tq1[r])
                                       : cimp * tq[r] + (1.0 - cimp) * tq1[r];
                v2[v] = nv;
                if (i == maxi) v2[(size_t)NV * lr] = nv;          // tq2(0,j) = tq2(maxi,j)
                if (i == 1) v2[maxi + 1 + (size_t)NV * lr] = nv;  // tq2(maxi+1,j) = tq2(1,j)
            }
            cluster.sync();
            // halo rows j0-1 and j1 from the neighbours (0 outside the grid)
            for (int i = t; i <= maxi + 1; i += blockDim.x) {
                v2[i] = v2_lo ? v2_lo[i + (size_t)NV * R] : 0.0;
                v2[i + (size_t)NV * (nrow + 1)] = v2_hi ? v2_hi[i + (size_t)NV * 1] : 0.0;
            }
            cluster.sync();   // the neighbours have their copies: own rows may change again
#pragma unroll
            for (int r = 0; r < kCellsPerThread; ++r) {
                const int c = t + r * blockDim.x;
                if (c >= ncell || !upd[r]) continue;
                const int i = c % maxi + 1, lr = c / maxi, j = j0 + lr;
                const size_t v = (size_t)i + (size_t)NV * (lr + 1);
                const size_t fe = (size_t)i + (size_t)NC * lr, fn = (size_t)i + (size_t)NC * (lr + 1);
                const double rdsj = a.rds[j - 1];
                const double flux = src[r] + cie[fe] * v2[v + 1] - ciw[fe - 1] * v2[v - 1] +
                                    (cin[fn] * v2[v + NV] - cis[fn - NC] * v2[v - NV]) * rdsj;
                if (!corr) {
                    const double centre = dt * cen[r];
                    tq[r] = (tq1[r] * (1.0 - (1.0 - cimp) * centre) - dt * flux) / (1 + cimp * centre);
                } else {
                    tq[r] = tq1[r] - dt * flux - dt * v2[v] * cen[r];
                }
            }
            __syncthreads();
        }
        if (!ice) {
#pragma unroll
            for (int r = 0; r < kCellsPerThread; ++r) tq1[r] = tq[r];   // tq1 = tq (embm.f90:2137)
        }
    }
#pragma unroll
    for (int r = 0; r < kCellsPerThread; ++r) {
        const int c = t + r * blockDim.x;
        if (c >= ncell) continue;
        const int i = c % maxi + 1, j = j0 + c / maxi;
        const size_t x = (size_t)(l - 1) + 2 * ((size_t)(i - 1) + (size_t)maxi * (j - 1));
        a.tq[x] = tq[r];
        a.tq1[x] = tq1[r];
        if (ice && upd[r]) {
            // the thermal and dynamical parts of the step's ice change, purely diagnostic
            // (gold_seaice.f90:1046-1056)
            const double th = a.tsc * dt * a.src[x];
            a.dth[x] = th;
            a.ddy[x] = tq[r] - tq1[r] - th;
        }
    }
}

// tstepsic (gold_seaice.f90:844-929): the ice flux through the east face of (i, j) for tracer
// l (the west "doorway" flux of cell 1 is the east flux of cell maxi), and through the north
// face.  Advection stops when the receiving cell already holds more ice than the thresholds.
__device__ __forceinline__ double ice_east(const EaArgs &a, int l, int i, int j)
{
    const int maxi = a.maxi, NK = maxi + 2;
    const int ip = i == maxi ? 1 : i + 1;
    const int k1c = a.k1[i + (size_t)NK * j], k1e = a.k1[ip + (size_t)NK * j];
    if (a.maxk < (k1c > k1e ? k1c : k1e)) return 0;
    auto v = [&](int ll, int ii) { return a.tq1[(size_t)(ll - 1) + 2 * ((size_t)(ii - 1) + (size_t)maxi * (j - 1))]; };
    const double u1 = a.vel[2 * ((size_t)(i - 1) + (size_t)maxi * (j - 1))];
    const double rcj = a.rc[j];
    double f = u1 * rcj * (v(l, ip) + v(l, i)) * 0.5;
    const int down = u1 >= 0.0 ? ip : i;
    if (v(2, down) > a.sica) f = 0;
    if (v(1, down) > a.sich) f = 0;
    return f - (v(l, ip) - v(l, i)) * rcj * rcj * a.rdphi * a.diffsic;
}

__device__ __forceinline__ double ice_north(const EaArgs &a, int l, int i, int j)
{
    const int maxi = a.maxi, NK = maxi + 2;
    const int k1c = a.k1[i + (size_t)NK * j], k1n = a.k1[i + (size_t)NK * (j + 1)];
    if (a.maxk < (k1c > k1n ? k1c : k1n)) return 0;   // always for j = maxj: row maxj+1 is land
    auto v = [&](int ll, int jj) { return a.tq1[(size_t)(ll - 1) + 2 * ((size_t)(i - 1) + (size_t)maxi * (jj - 1))]; };
    const double u2 = a.vel[2 * ((size_t)(i - 1) + (size_t)maxi * (j - 1)) + 1];
    const double cvj = a.cv[j];
    double f = cvj * u2 * (v(l, j + 1) + v(l, j)) * 0.5;
    const int down = u2 >= 0.0 ? j + 1 : j;
    if (v(2, down) > a.sica) f = 0;
    if (v(1, down) > a.sich) f = 0;
    return f - cvj * cvj * (v(l, j + 1) - v(l, j)) * a.rdsv[j - 1] * a.diffsic;
}

// One thread per cell: the reference's west and south carries are the east and north fluxes of
// the neighbours, recomputed here with the same expressions.
__global__ void __launch_bounds__(256) k_seaice_explicit(const EaArgs *__restrict__ args)
{
    const EaArgs a = args[blockIdx.y];
    const int maxi = a.maxi, maxj = a.maxj;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= maxi * maxj) return;
    const int i = c % maxi + 1, j = c / maxi + 1;
    if (a.maxk < a.k1[i + (size_t)(maxi + 2) * j]) return;
    for (int l = 1; l <= 2; ++l) {
        const double fe = ice_east(a, l, i, j);
        const double fw = ice_east(a, l, i == 1 ? maxi : i - 1, j);
        const double fn = ice_north(a, l, i, j);
        const double fs = j > 1 ? ice_north(a, l, i, j - 1) : 0.0;
        const size_t x = (size_t)(l - 1) + 2 * (size_t)c;
        a.tq[x] = a.tq1[x] - a.dt * ((fe - fw) * a.rdphi + (fn - fs) * a.rds[j - 1]) + a.tsc * a.dt * a.src[x];
    }
}

// step_seaice's post-processing of a sea-ice step (gold_seaice.f90:599-619), one thread per
// cell: the area is held in [0, 1]; ice thinner than hmin is removed, its latent heat and
// water returned to the ocean as fluxes; varice1 = varice.  Land cells keep fx = fw = 0
// (gold_seaice.f90:578-579).
__global__ void __launch_bounds__(256) k_seaice_post(const EaArgs *__restrict__ args)
{
    const EaArgs a = args[blockIdx.y];
    const int maxi = a.maxi;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= maxi * a.maxj) return;
    const int i = c % maxi + 1, j = c / maxi + 1;
    if (a.maxk < a.k1[i + (size_t)(maxi + 2) * j]) return;
    const size_t x = 2 * (size_t)c;
    double fw = -(a.rhoio * a.src[x]);
    double fx = 0.0;
    double h = a.tq[x];
    double ar = clamp01(a.tq[x + 1]);
    if (h < a.hmin) {
        fx = -(((h * a.rhoice) * a.hlf) * a.rdtdim);
        fw = fw + (h * a.rhoio) * a.rdtdim;
        h = 0.0;
        ar = 0.0;
    }
    a.tq[x] = a.tq1[x] = h;
    a.tq[x + 1] = a.tq1[x + 1] = ar;
    a.fx[c] = fx;
    a.fw[c] = fw * a.m2mm;   // m/s to mm/s
}

// rows per block and blocks per tracer (the cluster size, at most kClusterMax)
void split_rows(int maxj, int *R, int *C, int cmax = kClusterMax)
{
    *R = (maxj + cmax - 1) / cmax;
    *C = (maxj + *R - 1) / *R;
}

size_t smem_bytes(int maxi, int R)
{
    return (2 * (size_t)(maxi + 1) * R + 2 * (size_t)(maxi + 1) * (R + 1) + (size_t)(maxi + 2) * (R + 2)) * sizeof(double);
}

}  // namespace

struct gb_ea {
    int device = 0;
    gb_ea_dims d{};
    gb_ea_params p{};
    cudaStream_t stream = nullptr;
    double *rc = nullptr, *cv = nullptr, *dsv = nullptr, *rdsv = nullptr, *rds = nullptr, *diffa = nullptr;
    int32_t *k1 = nullptr;
    double *tq = nullptr, *tq1 = nullptr, *src = nullptr, *vel = nullptr, *pptn = nullptr;
    double *dth = nullptr, *ddy = nullptr;   // sea ice: variceth, varicedy
    double *fx = nullptr, *fw = nullptr;     // sea ice: fx_delta, fw_delta
    bool post = false;                        // sea ice: post-process each step
    gb_ea_seaice_post pp{};
    bool have_state = false, have_forcing = false;
    int cluster_max = 8;   // 16 where the device schedules clusters of 16 (gb_ea_create)
    EaArgs *dargs = nullptr;   // kernel arguments in device memory (capacity cap_args grids)
    int cap_args = 0;
    std::string last_error;
};

static int efail(gb_ea *h, int code, const std::string &msg)
{
    if (h) h->last_error = msg;
    return code;
}

#define EA_TRY(h, call)                                                                                   \
    do {                                                                                                  \
        cudaError_t _e = (call);                                                                          \
        if (_e != cudaSuccess)                                                                            \
            return efail(h, _e == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA,                 \
                         std::string(#call) + ": " + cudaGetErrorString(_e));                             \
    } while (0)

extern "C" int gb_ea_create(const gb_ea_dims *dims, const gb_ea_params *params, const gb_ea_grid *grid, int device,
                            gb_ea **out)
{
    if (!out) return GB_GO_EINVAL;
    *out = nullptr;
    if (!dims || !params || !grid) return GB_GO_EINVAL;
    const int maxi = dims->maxi, maxj = dims->maxj;
    if (maxi < 1 || maxj < 2) return GB_GO_EINVAL;
    if ((long long)maxi * maxj > GB_EA_MAX_CELLS) return GB_GO_ERANGE;
    // limits for the portable cluster size (the larger rows per block)
    int R = 0, C = 0;
    split_rows(maxj, &R, &C, 8);
    if ((long long)maxi * R > (long long)kThreads * kCellsPerThread) return GB_GO_ERANGE;   // one block's cells
    const gb_ea_params p = *params;
    if (p.kind != GB_EA_EMBM && p.kind != GB_EA_SEAICE && p.kind != GB_EA_SEAICE_EXPLICIT) return GB_GO_EINVAL;
    if (!grid->rc || !grid->cv || !grid->dsv || !grid->rdsv || !grid->rds) return GB_GO_EINVAL;
    if (p.kind == GB_EA_EMBM && !grid->diffa) return GB_GO_EINVAL;
    if (p.kind != GB_EA_EMBM) {
        if (!grid->k1 || p.maxk < 1) return GB_GO_EINVAL;
        // rows 0 and maxj+1 are land (the reference's grid convention): no north face of row maxj
        // is wet, so nothing reads beyond row maxj
        for (int i = 0; i <= maxi + 1; ++i)
            if (grid->k1[i] <= p.maxk || grid->k1[i + (size_t)(maxi + 2) * (maxj + 1)] <= p.maxk) return GB_GO_EINVAL;
    }
    if (device < 0) cudaGetDevice(&device);
    int smem_max = 0;
    if (cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess)
        return GB_GO_ECUDA;
    if (smem_bytes(maxi, R) > (size_t)smem_max) return GB_GO_ERANGE;   // a block's rows must fit its shared memory
    gb_ea *h = new gb_ea();
    h->d = *dims;
    h->p = p;
    h->device = device;
    const size_t n2 = 2 * (size_t)maxi * maxj;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    auto up = [&](double **dst, const double *srcp, size_t n) {
        if (e != cudaSuccess) return;
        e = cudaMalloc(dst, std::max<size_t>(1, n) * sizeof(double));
        if (e == cudaSuccess && srcp && n) e = cudaMemcpy(*dst, srcp, n * sizeof(double), cudaMemcpyHostToDevice);
    };
    up(&h->rc, grid->rc, (size_t)maxj + 1);
    up(&h->cv, grid->cv, (size_t)maxj + 1);
    up(&h->dsv, grid->dsv, (size_t)maxj - 1);
    up(&h->rdsv, grid->rdsv, (size_t)maxj - 1);
    up(&h->rds, grid->rds, (size_t)maxj);
    up(&h->diffa, p.kind == GB_EA_EMBM ? grid->diffa : nullptr, p.kind == GB_EA_EMBM ? 4 * (size_t)maxj : 1);
    up(&h->tq, nullptr, n2);
    up(&h->tq1, nullptr, n2);
    up(&h->src, nullptr, n2);
    up(&h->vel, nullptr, n2);
    up(&h->pptn, nullptr, (size_t)maxi * maxj);
    up(&h->dth, nullptr, n2);
    up(&h->ddy, nullptr, n2);
    if (e == cudaSuccess) e = cudaMemset(h->dth, 0, n2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(h->ddy, 0, n2 * sizeof(double));
    up(&h->fx, nullptr, n2 / 2);
    up(&h->fw, nullptr, n2 / 2);
    if (e == cudaSuccess) e = cudaMemset(h->fx, 0, n2 / 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(h->fw, 0, n2 / 2 * sizeof(double));
    const size_t nk = (size_t)(maxi + 2) * (maxj + 2);
    if (e == cudaSuccess) e = cudaMalloc(&h->k1, nk * sizeof(int32_t));
    if (e == cudaSuccess && p.kind != GB_EA_EMBM)
        e = cudaMemcpy(h->k1, grid->k1, nk * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && p.kind == GB_EA_EMBM) e = cudaMemset(h->k1, 0, nk * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemset(h->pptn, 0, (size_t)maxi * maxj * sizeof(double));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_surface_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes(maxi, R));
    // clusters of up to 16 blocks where the device schedules them, else the portable 8
    h->cluster_max = 8;
    int R16 = 0, C16 = 0;
    split_rows(maxj, &R16, &C16, 16);
    if (e == cudaSuccess && C16 > 8 &&
        cudaFuncSetAttribute(k_surface_step, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(2 * C16);
        cfg.blockDim = dim3(std::min(kThreads, (maxi * R16 + 31) / 32 * 32));
        cfg.dynamicSmemBytes = smem_bytes(maxi, R16);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = C16;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, k_surface_step, &cfg) == cudaSuccess && nclusters >= 1)
            h->cluster_max = 16;
    }
    cudaGetLastError();   // a refused query leaves no sticky error: clear the last one
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA;
        gb_ea_destroy(h);
        return code;
    }
    *out = h;
    return GB_GO_OK;
}

extern "C" void gb_ea_destroy(gb_ea *h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    void *ptrs[] = {h->rc, h->cv, h->dsv, h->rdsv, h->rds, h->diffa, h->k1, h->tq, h->tq1, h->src, h->vel, h->pptn, h->dth, h->ddy, h->fx, h->fw, h->dargs};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

extern "C" const char *gb_ea_last_error(const gb_ea *h) { return h ? h->last_error.c_str() : ""; }

extern "C" int gb_ea_upload_state(gb_ea *h, const double *tq, const double *tq1)
{
    if (!h || !tq || !tq1) return efail(h, GB_GO_EINVAL, "upload_state: NULL array");
    EA_TRY(h, cudaSetDevice(h->device));
    const size_t n2 = 2 * (size_t)h->d.maxi * h->d.maxj;
    EA_TRY(h, cudaMemcpyAsync(h->tq, tq, n2 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    EA_TRY(h, cudaMemcpyAsync(h->tq1, tq1, n2 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    EA_TRY(h, cudaStreamSynchronize(h->stream));
    h->have_state = true;
    return GB_GO_OK;
}

extern "C" int gb_ea_set_forcing(gb_ea *h, const double *source, const double *vel, const double *pptn)
{
    if (!h || !source || !vel) return efail(h, GB_GO_EINVAL, "set_forcing: NULL array");
    if (h->p.kind == GB_EA_EMBM && !pptn) return efail(h, GB_GO_EINVAL, "set_forcing: EMBM needs pptn");
    EA_TRY(h, cudaSetDevice(h->device));
    const size_t n1 = (size_t)h->d.maxi * h->d.maxj, n2 = 2 * n1;
    EA_TRY(h, cudaMemcpyAsync(h->src, source, n2 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    EA_TRY(h, cudaMemcpyAsync(h->vel, vel, n2 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (pptn) EA_TRY(h, cudaMemcpyAsync(h->pptn, pptn, n1 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    EA_TRY(h, cudaStreamSynchronize(h->stream));
    h->have_forcing = true;
    return GB_GO_OK;
}

static EaArgs args_of(const gb_ea *h, int nsteps)
{
    EaArgs a{};
    a.maxi = h->d.maxi;
    a.maxj = h->d.maxj;
    a.maxk = h->p.maxk;
    a.kind = h->p.kind;
    a.nsteps = nsteps;
    a.dt = h->p.dt;
    a.dphi = h->p.dphi;
    a.rdphi = h->p.rdphi;
    for (int l = 0; l < 2; ++l) {
        a.betaz[l] = h->p.betaz[l];
        a.betam[l] = h->p.betam[l];
    }
    a.diffmod0 = h->p.diffmod0;
    a.ppmin = h->p.ppmin;
    a.ppmax = h->p.ppmax;
    a.diffsic = h->p.diffsic;
    a.tsc = h->p.tsc;
    a.sica = h->p.sica_thresh;
    a.sich = h->p.sich_thresh;
    a.rc = h->rc;
    a.cv = h->cv;
    a.dsv = h->dsv;
    a.rdsv = h->rdsv;
    a.rds = h->rds;
    a.diffa = h->diffa;
    a.k1 = h->k1;
    a.tq = h->tq;
    a.tq1 = h->tq1;
    a.src = h->src;
    a.vel = h->vel;
    a.pptn = h->pptn;
    a.dth = h->dth;
    a.ddy = h->ddy;
    a.rhoio = h->pp.rhoio;
    a.rhoice = h->pp.rhoice;
    a.hlf = h->pp.hlf;
    a.hmin = h->pp.hmin;
    a.rdtdim = h->pp.rdtdim;
    a.m2mm = h->pp.m2mm;
    a.fx = h->fx;
    a.fw = h->fw;
    return a;
}

// nsteps steps of n grids of the same kind and shape, one launch (blockIdx.y = grid)
static int step_grids(gb_ea *const *hs, int n, int nsteps)
{
    gb_ea *h = hs[0];
    if (nsteps < 0) return efail(h, GB_GO_EINVAL, "step: nsteps < 0");
    for (int m = 0; m < n; ++m) {
        const gb_ea *g = hs[m];
        if (!g) return efail(h, GB_GO_EINVAL, "step: NULL handle");
        if (g->device != h->device || g->p.kind != h->p.kind || g->d.maxi != h->d.maxi || g->d.maxj != h->d.maxj ||
            g->cluster_max != h->cluster_max || g->post != h->post)
            return efail(h, GB_GO_EINVAL, "step_many: grids differ in device, kind, shape or post-processing");
        if (!g->have_state || !g->have_forcing) return efail(h, GB_GO_ENOTREADY, "step before upload_state/set_forcing");
    }
    if (h->p.kind != GB_EA_EMBM && nsteps > 1 && !h->post)
        return efail(h, GB_GO_EINVAL,
                     "step: sea ice takes one step per call unless its post-processing is on (gb_ea_set_seaice_post)");
    if (nsteps == 0 || n == 0) return GB_GO_OK;
    EA_TRY(h, cudaSetDevice(h->device));
    if (n > h->cap_args) {
        if (h->dargs) cudaFree(h->dargs);
        h->dargs = nullptr;
        h->cap_args = 0;
        EA_TRY(h, cudaMalloc(&h->dargs, (size_t)n * sizeof(EaArgs)));
        h->cap_args = n;
    }
    std::vector<EaArgs> args((size_t)n);
    // with the sea-ice post-processing on, every step is a step launch and a post launch
    const bool post = h->post && h->p.kind != GB_EA_EMBM;
    for (int m = 0; m < n; ++m) args[m] = args_of(hs[m], post ? 1 : nsteps);
    EA_TRY(h, cudaMemcpyAsync(h->dargs, args.data(), (size_t)n * sizeof(EaArgs), cudaMemcpyHostToDevice, h->stream));
    const int ncell = h->d.maxi * h->d.maxj;
    for (int s = 0; s < (post ? nsteps : 1); ++s) {
        if (h->p.kind == GB_EA_SEAICE_EXPLICIT) {
            k_seaice_explicit<<<dim3((ncell + 255) / 256, n), 256, 0, h->stream>>>(h->dargs);
        } else {
            int R = 0, C = 0;
            split_rows(h->d.maxj, &R, &C, h->cluster_max);
            const int cells = h->d.maxi * R;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(2 * C, n);
            cfg.blockDim = dim3(std::min(kThreads, (cells + 31) / 32 * 32));
            cfg.dynamicSmemBytes = smem_bytes(h->d.maxi, R);
            cfg.stream = h->stream;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = C;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            EA_TRY(h, cudaLaunchKernelEx(&cfg, k_surface_step, (const EaArgs *)h->dargs, R));
        }
        count_launches(1);
        if (post) {
            k_seaice_post<<<dim3((ncell + 255) / 256, n), 256, 0, h->stream>>>(h->dargs);
            count_launches(1);
        }
    }
    EA_TRY(h, cudaGetLastError());
    EA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}

extern "C" int gb_ea_step(gb_ea *h, int32_t nsteps)
{
    gbgo::TraceRange tr_("ea_step");
    if (!h) return GB_GO_EINVAL;
    return step_grids(&h, 1, nsteps);
}

extern "C" int gb_ea_step_many(gb_ea *const *handles, int32_t n, int32_t nsteps)
{
    gbgo::TraceRange tr_("ea_step_many");
    if (!handles || n < 1 || !handles[0]) return GB_GO_EINVAL;
    return step_grids(handles, n, nsteps);
}

extern "C" int gb_ea_download(gb_ea *h, double *tq, double *tq1)
{
    if (!h) return GB_GO_EINVAL;
    if (!h->have_state) return efail(h, GB_GO_ENOTREADY, "download before upload_state");
    EA_TRY(h, cudaSetDevice(h->device));
    const size_t n2 = 2 * (size_t)h->d.maxi * h->d.maxj;
    if (tq) EA_TRY(h, cudaMemcpyAsync(tq, h->tq, n2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (tq1) EA_TRY(h, cudaMemcpyAsync(tq1, h->tq1, n2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}

extern "C" int gb_ea_download_seaice_diag(gb_ea *h, double *variceth, double *varicedy)
{
    if (!h) return GB_GO_EINVAL;
    if (h->p.kind == GB_EA_EMBM) return efail(h, GB_GO_EINVAL, "download_seaice_diag: an EMBM handle has no ice");
    EA_TRY(h, cudaSetDevice(h->device));
    const size_t n2 = 2 * (size_t)h->d.maxi * h->d.maxj;
    if (variceth) EA_TRY(h, cudaMemcpyAsync(variceth, h->dth, n2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (varicedy) EA_TRY(h, cudaMemcpyAsync(varicedy, h->ddy, n2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}

extern "C" int gb_ea_set_seaice_post(gb_ea *h, const gb_ea_seaice_post *post)
{
    if (!h) return GB_GO_EINVAL;
    if (h->p.kind == GB_EA_EMBM) return efail(h, GB_GO_EINVAL, "set_seaice_post: an EMBM handle has no ice");
    h->post = post != nullptr;
    if (post) h->pp = *post;
    return GB_GO_OK;
}

extern "C" int gb_ea_download_seaice_fluxes(gb_ea *h, double *fx_delta, double *fw_delta)
{
    if (!h) return GB_GO_EINVAL;
    if (h->p.kind == GB_EA_EMBM) return efail(h, GB_GO_EINVAL, "download_seaice_fluxes: an EMBM handle has no ice");
    EA_TRY(h, cudaSetDevice(h->device));
    const size_t n1 = (size_t)h->d.maxi * h->d.maxj;
    if (fx_delta) EA_TRY(h, cudaMemcpyAsync(fx_delta, h->fx, n1 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (fw_delta) EA_TRY(h, cudaMemcpyAsync(fw_delta, h->fw, n1 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    EA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}
