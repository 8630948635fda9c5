// BIOGEM tracer coupling on the device: biogem_tracercoupling (src/biogem/biogem.f90:1885-2077)
// applied to the tracer state of a single-grid GOLDSTEIN handle, with BIOGEM's vector fields
// resident on the same device.
//
// Structure of one coupling (all on the ocean handle's stream, -fmad=false: every expression
// rounds as the reference's left-to-right double arithmetic):
//   k_bg_partials<0>  one thread per (quantity q, column n): the per-column sums over k = k1..n_k
//                     of vocn(S)*V (q = 1) and vocn(l)*M (q = l >= 2) -- the SUMs of :1946-1963
//   k_bg_seqsum<0>    one block: the sums over the columns, each quantity left to right in the
//                     reference's column order (Fortran SUM), staged through shared memory;
//                     then the old mean salinity and inventories
//   k_bg_partials<1>  the same for vocn_new(S)*V and loc_vocn(l)*M (:1983-1996, :2016-2023)
//   k_bg_seqsum<1>    the new mean salinity, the salinity ratio, the new inventories
//   k_bg_zero         interior cells that are land or below k1: 0 in ts and ts1 (conv_vocnTOts);
//                     once per upload of the ocean state, as nothing else writes those cells
//   k_bg_apply        one thread per wet cell: T and S, the biogeochemical tracers, particulates,
//                     masses, and the GOLDSTEIN tracers written back into ts and ts1 (:2000-2056)
//   k_bg_halo         ts1's periodic i-halo from the new ts (goldstein.f90:180-186)
// then the handle reloads its step buffers from ts/ts1, as after an upload.
//
// The column sums are sequential by definition (each partial sum rounds), so they run as
// dependent FP64 additions, one chain per quantity; everything else is one pass over the cells.
#include "../../include/gb_biogem.h"
#include "gb_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

using namespace gbgo;

namespace {

constexpr double kNullSmall = 0.999999e-19;   // const_real_nullsmall, src/common/gem_cmn.f90:719
constexpr int kSumThreads = 256;

// Device scalars of one coupling.  tot_v is the total volume (the reference recomputes it each
// call from the volumes, which only change on upload, so it is summed at upload).
struct BgScalars {
    double tot_v, rtot_v;
    double mean_s_old, rmean_s_old;
    double mean_s_new, s_ratio, rs_ratio;
    double pad;
    // then tot_old[L], rtot_new[L]
};

struct BgArgs {
    int L, Ls, nk, nv;
    int NI, NJ;              // ocean halo'd extents
    int force_ts;
    double off0, off1;
    const int32_t *ci, *cj, *ck1;   // per column: i, j (1-based), k1
    double *vocn, *mass, *rmass, *vbio;
    const double *volume, *vdocn, *vdbio;
    double *part;            // (L, nv): q-major partial sums
    BgScalars *sc;
    double *tot_old, *rtot_new;   // (L)
    const double *tsrc;      // current GOLDSTEIN ts (halo'd Fortran layout)
    double *ts_out, *ts1_out;
};

__device__ __forceinline__ size_t ts_index(const BgArgs &a, int l, int i, int j, int k)
{
    return (size_t)l + (size_t)a.L * ((size_t)i + (size_t)a.NI * ((size_t)j + (size_t)a.NJ * (size_t)k));
}

// PHASE 0: q = 0: V (the volume total, at upload); q = 1: S*V times rtot_V; q >= 2: vocn(q)*M.
// PHASE 1: q = 1: S_new*V times rtot_V with S_new = (vts(S) + offset) + vdocn(S); q >= 2:
//          loc_vocn(q)*M with loc_vocn = vts(q)*S_old*rmean_s_old.
template <int PHASE>
__global__ void __launch_bounds__(256) k_bg_partials(BgArgs a)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)a.L * a.nv) return;
    const int n = (int)(t / a.L), q = (int)(t % a.L);
    const int k1 = a.ck1[n], i = a.ci[n], j = a.cj[n];
    const double *vo = a.vocn + (size_t)a.L * a.nk * n;
    const double *M = a.mass + (size_t)a.nk * n;
    const double *V = a.volume + (size_t)a.nk * n;
    double s = 0.0;
    if (PHASE == 0) {
        if (q == 0) {
            for (int k = k1; k <= a.nk; ++k) s = s + V[k - 1];
        } else if (q == 1) {
            for (int k = k1; k <= a.nk; ++k) s = s + vo[1 + (size_t)a.L * (k - 1)] * V[k - 1];
            s = s * a.sc->rtot_v;   // loc_partialtot(n) = SUM(...)*loc_ocn_rtot_V (biogem.f90:1951)
        } else {
            for (int k = k1; k <= a.nk; ++k) s = s + vo[q + (size_t)a.L * (k - 1)] * M[k - 1];
        }
    } else {
        const double *vd = a.vdocn + (size_t)a.L * a.nk * n;
        if (q == 0) return;
        if (q == 1) {
            for (int k = k1; k <= a.nk; ++k) {
                const double snew = (a.tsrc[ts_index(a, 1, i, j, k)] + a.off1) + vd[1 + (size_t)a.L * (k - 1)];
                s = s + snew * V[k - 1];
            }
            s = s * a.sc->rtot_v;   // biogem.f90:2021
        } else {
            const double rm = a.sc->rmean_s_old;
            for (int k = k1; k <= a.nk; ++k) {
                const double loc = a.tsrc[ts_index(a, q, i, j, k)] * vo[1 + (size_t)a.L * (k - 1)] * rm;
                s = s + loc * M[k - 1];
            }
        }
    }
    a.part[(size_t)q * a.nv + n] = s;
}

// One block.  Thread q < L owns quantity q and adds its nv partials left to right; the block
// stages tiles of partials through shared memory with cp.async so that the loads of the next
// tile overlap the additions of this one.  MODE 0: volume total (upload).  MODE 1: old mean
// salinity and inventories.  MODE 2: new mean salinity, salinity ratio, new inventories.
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <int MODE>
__global__ void __launch_bounds__(kSumThreads) k_bg_seqsum(BgArgs a, int tile)
{
    extern __shared__ double sm[];
    const int q0 = MODE == 0 ? 0 : 1, q1 = MODE == 0 ? 1 : a.L;   // quantities [q0, q1)
    const int nq = q1 - q0;
    const int stride = tile + 1;   // padded rows: the summing threads read distinct banks
    double *buf[2] = {sm, sm + (size_t)nq * stride};
    const int t = threadIdx.x;
    auto load = [&](int b, int n0) {
        const int cnt = min(tile, a.nv - n0);
        for (int e = t; e < nq * cnt; e += blockDim.x) {
            const int r = e / cnt, c = e % cnt;
            cp_async8(buf[b] + (size_t)r * stride + c, a.part + (size_t)(q0 + r) * a.nv + n0 + c);
        }
        cp_async_commit();
    };
    double s = 0.0;
    int b = 0;
    if (a.nv > 0) load(0, 0);
    for (int n0 = 0; n0 < a.nv; n0 += tile) {
        cp_async_wait_all();
        __syncthreads();
        if (n0 + tile < a.nv) load(b ^ 1, n0 + tile);
        if (t < nq) {
            const int cnt = min(tile, a.nv - n0);
            const double *row = buf[b] + (size_t)t * stride;
            // only the additions chain (an FP64 add takes ~63 cycles on GB300): the shared-memory
            // loads of the next 8 columns are issued before the additions of these 8
            int c = 0;
            double nxt[8];
            if (cnt >= 8) {
#pragma unroll
                for (int u = 0; u < 8; ++u) nxt[u] = row[u];
            }
            for (; c + 8 <= cnt; c += 8) {
                double cur[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) cur[u] = nxt[u];
                if (c + 16 <= cnt) {
#pragma unroll
                    for (int u = 0; u < 8; ++u) nxt[u] = row[c + 8 + u];
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) s = s + cur[u];
            }
            for (; c < cnt; ++c) s = s + row[c];
        }
        __syncthreads();   // buffer b is reloaded two tiles later
        b ^= 1;
    }
    if (t >= nq) return;
    const int q = q0 + t;
    BgScalars *sc = a.sc;
    if (MODE == 0) {
        sc->tot_v = s;
        sc->rtot_v = 1.0 / s;
    } else if (MODE == 1) {
        if (q == 1) {
            sc->mean_s_old = s;
            sc->rmean_s_old = 1.0 / s;
        } else {
            a.tot_old[q] = s;
        }
    } else {
        if (q == 1) {
            sc->mean_s_new = s;
            const double r = s / sc->mean_s_old;
            sc->s_ratio = r;
            sc->rs_ratio = 1.0 / r;
        } else {
            a.rtot_new[q] = fabs(s) < kNullSmall ? 0.0 : 1.0 / s;
        }
    }
}

// Interior cells of land columns and below k1: 0 in ts and ts1 (fun_lib_conv_vocnTOts fills
// only the wet levels; step_goldstein copies go_ts / go_ts1 over the whole interior).
__global__ void __launch_bounds__(256) k_bg_zero(BgArgs a, int maxi, int maxj, const int32_t *k1h)
{
    const long long ncell = (long long)maxi * maxj * a.nk;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % maxi) + 1, j = (int)((c / maxi) % maxj) + 1, k = (int)(c / ((long long)maxi * maxj)) + 1;
        if (k >= k1h[i + (size_t)a.NI * j]) continue;
        for (int l = 0; l < a.L; ++l) {
            const size_t x = ts_index(a, l, i, j, k);
            a.ts_out[x] = 0.0;
            a.ts1_out[x] = 0.0;
        }
    }
}

// One thread per (column, level): the cell's T and S, biogeochemical tracers, particulates and
// masses, and its GOLDSTEIN tracers in ts and ts1 (biogem.f90:2000-2013, 2033-2056).  The
// thread reads its own cell only, so ts may be both the source and a destination.
__global__ void __launch_bounds__(256) k_bg_apply(BgArgs a)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)a.nk * a.nv) return;
    const int n = (int)(t / a.nk), k = (int)(t % a.nk) + 1;
    if (k < a.ck1[n]) return;
    const int i = a.ci[n], j = a.cj[n];
    double *vo = a.vocn + (size_t)a.L * ((size_t)(k - 1) + (size_t)a.nk * n);
    const double *vd = a.vdocn + (size_t)a.L * ((size_t)(k - 1) + (size_t)a.nk * n);
    const BgScalars sc = *a.sc;
    const double s_old = vo[1];
    // T and S: (vts + offset) + vdocn in both modes; loc_vocn keeps vts + offset unless forced
    double tsn[2];
    const double off[2] = {a.off0, a.off1};
    double vnew[2];
    for (int l = 0; l < 2; ++l) {
        const double v = a.tsrc[ts_index(a, l, i, j, k)];
        const double loc = v + off[l];
        vnew[l] = loc + vd[l];
        tsn[l] = (a.force_ts ? vnew[l] : loc) - off[l];
    }
    for (int l = 0; l < 2; ++l) {
        vo[l] = vnew[l];
        const size_t x = ts_index(a, l, i, j, k);
        a.ts_out[x] = tsn[l];
        a.ts1_out[x] = tsn[l];
    }
    const double s_new = vnew[1];
    const double q_s = sc.mean_s_new / s_new;
    for (int l = 2; l < a.L; ++l) {
        const size_t x = ts_index(a, l, i, j, k);
        const double loc = a.tsrc[x] * s_old * sc.rmean_s_old;
        double v = (a.tot_old[l] * a.rtot_new[l]) * loc + vd[l];
        v = sc.s_ratio * v;
        vo[l] = v;
        const double out = q_s * v;
        a.ts_out[x] = out;
        a.ts1_out[x] = out;
    }
    if (a.Ls > 0) {
        double *vb = a.vbio + (size_t)a.Ls * ((size_t)(k - 1) + (size_t)a.nk * n);
        const double *vdb = a.vdbio + (size_t)a.Ls * ((size_t)(k - 1) + (size_t)a.nk * n);
        for (int l = 0; l < a.Ls; ++l) {
            const double v = vb[l] + vdb[l];
            vb[l] = sc.s_ratio * v;
        }
    }
    const size_t m = (size_t)(k - 1) + (size_t)a.nk * n;
    a.mass[m] = sc.rs_ratio * a.mass[m];
    a.rmass[m] = sc.s_ratio * a.rmass[m];
}

// ts1's periodic i-halo from ts, as step_goldstein sets it after the copy-in
// (goldstein.f90:180-186): ts1(:,0,j,k) = ts(:,maxi,j,k) for k >= k1(0,j),
// ts1(:,maxi+1,j,k) = ts(:,1,j,k) for k >= k1(maxi+1,j).
__global__ void __launch_bounds__(256) k_bg_halo(BgArgs a, int maxi, int maxj, const int32_t *k1h)
{
    const long long nwork = 2LL * maxj * a.nk * a.L;
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nwork; w += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(w % a.L);
        const long long r = w / a.L;
        const int k = (int)(r % a.nk) + 1;
        const int j = (int)((r / a.nk) % maxj) + 1;
        const int side = (int)(r / ((long long)a.nk * maxj));
        const int ih = side ? maxi + 1 : 0, isrc = side ? 1 : maxi;
        if (k < k1h[ih + (size_t)a.NI * j]) continue;
        a.ts1_out[ts_index(a, l, ih, j, k)] = a.ts_out[ts_index(a, l, isrc, j, k)];
    }
}

}  // namespace

struct gb_bg {
    int device = 0;
    gb_bg_dims d{};
    gb_bg_params p{};
    int nv = 0;
    cudaStream_t stream = nullptr;
    int32_t *ci = nullptr, *cj = nullptr, *ck1 = nullptr;
    double *vocn = nullptr, *mass = nullptr, *volume = nullptr, *rmass = nullptr;
    double *vdocn = nullptr, *vbio = nullptr, *vdbio = nullptr;
    double *part = nullptr;
    double *scal = nullptr;   // BgScalars, then tot_old[L], rtot_new[L]
    bool have_state = false, have_inc = false;
    std::string last_error;
};

static int bfail(gb_bg *h, int code, const std::string &msg)
{
    if (h) h->last_error = msg;
    return code;
}

#define BG_TRY(h, call)                                                                                   \
    do {                                                                                                  \
        cudaError_t _e = (call);                                                                          \
        if (_e != cudaSuccess)                                                                            \
            return bfail(h, _e == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA,                 \
                         std::string(#call) + ": " + cudaGetErrorString(_e));                             \
    } while (0)

static BgArgs args_of(gb_bg *h)
{
    BgArgs a{};
    a.L = h->d.n_l_ocn;
    a.Ls = h->d.n_l_sed;
    a.nk = h->d.n_k;
    a.nv = h->nv;
    a.NI = h->d.n_i + 2;
    a.NJ = h->d.n_j + 2;
    a.force_ts = h->p.force_ts;
    a.off0 = h->p.ts_offset[0];
    a.off1 = h->p.ts_offset[1];
    a.ci = h->ci;
    a.cj = h->cj;
    a.ck1 = h->ck1;
    a.vocn = h->vocn;
    a.mass = h->mass;
    a.rmass = h->rmass;
    a.vbio = h->vbio;
    a.volume = h->volume;
    a.vdocn = h->vdocn;
    a.vdbio = h->vdbio;
    a.part = h->part;
    a.sc = reinterpret_cast<BgScalars *>(h->scal);
    a.tot_old = h->scal + sizeof(BgScalars) / sizeof(double);
    a.rtot_new = a.tot_old + h->d.n_l_ocn;
    return a;
}

// shared memory tile of the column sums: two buffers of nq rows of (tile + 1) doubles
static int sum_tile(int nq)
{
    // even, so that the padded row stride (tile + 1 doubles) is odd and the rows fall in distinct banks
    return std::max(32, std::min(256, (6 * 1024) / std::max(1, nq) - 1)) & ~1;
}
static size_t sum_smem(int nq, int tile) { return 2 * (size_t)nq * (tile + 1) * sizeof(double); }

template <int MODE>
static cudaError_t launch_seqsum(const BgArgs &a, cudaStream_t s)
{
    const int nq = MODE == 0 ? 1 : a.L - 1;
    const int tile = sum_tile(nq);
    const size_t smem = sum_smem(nq, tile);
    cudaError_t e = cudaFuncSetAttribute(k_bg_seqsum<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_bg_seqsum<MODE><<<1, kSumThreads, smem, s>>>(a, tile);
    count_launches(1);
    return cudaGetLastError();
}

extern "C" int gb_bg_create(const gb_bg_dims *dims, const gb_bg_params *params, const int32_t *k1, int device, gb_bg **out)
{
    if (!out) return GB_GO_EINVAL;
    *out = nullptr;
    if (!dims || !params || !k1) return GB_GO_EINVAL;
    const gb_bg_dims d = *dims;
    if (d.n_i < 1 || d.n_j < 1 || d.n_k < 1 || d.n_k > GB_GO_MAX_K || d.n_l_ocn < 2 || d.n_l_ocn > GB_GO_MAX_L ||
        d.n_l_sed < 0 || d.n_l_sed > 1024)
        return GB_GO_EINVAL;
    if (params->force_ts != 0 && params->force_ts != 1) return GB_GO_EINVAL;
    gb_bg *h = new gb_bg();
    h->d = d;
    h->p = *params;
    if (device < 0) cudaGetDevice(&device);
    h->device = device;
    std::vector<int32_t> ci, cj, ck1;
    for (int i = 1; i <= d.n_i; ++i)
        for (int j = 1; j <= d.n_j; ++j) {
            const int kk = k1[(i - 1) + (size_t)d.n_i * (j - 1)];
            if (d.n_k >= kk) {
                if (kk < 1) {
                    delete h;
                    return GB_GO_EINVAL;
                }
                ci.push_back(i);
                cj.push_back(j);
                ck1.push_back(kk);
            }
        }
    h->nv = (int)ci.size();
    const size_t nv = std::max<size_t>(1, ci.size());
    const size_t nf = (size_t)d.n_l_ocn * d.n_k * nv, np = (size_t)d.n_k * nv, ns = (size_t)d.n_l_sed * d.n_k * nv;
    auto cleanup = [&](int code, const char *what) {
        gb_bg_destroy(h);
        (void)what;
        return code;
    };
    if (cudaSetDevice(device) != cudaSuccess) return cleanup(GB_GO_ECUDA, "device");
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&h->ci, nv * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->cj, nv * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->ck1, nv * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->vocn, nf * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->vdocn, nf * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->mass, np * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->volume, np * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->rmass, np * sizeof(double));
    if (e == cudaSuccess && ns) e = cudaMalloc(&h->vbio, ns * sizeof(double));
    if (e == cudaSuccess && ns) e = cudaMalloc(&h->vdbio, ns * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->part, (size_t)d.n_l_ocn * nv * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->scal, sizeof(BgScalars) + 2 * (size_t)d.n_l_ocn * sizeof(double));
    if (e == cudaSuccess && !ci.empty()) {
        e = cudaMemcpy(h->ci, ci.data(), ci.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(h->cj, cj.data(), cj.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(h->ck1, ck1.data(), ck1.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemset(h->scal, 0, sizeof(BgScalars) + 2 * (size_t)d.n_l_ocn * sizeof(double));
    if (e != cudaSuccess) return cleanup(e == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA, "alloc");
    *out = h;
    return GB_GO_OK;
}

extern "C" void gb_bg_destroy(gb_bg *h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    void *ptrs[] = {h->ci, h->cj, h->ck1, h->vocn, h->vdocn, h->mass, h->volume, h->rmass, h->vbio, h->vdbio, h->part, h->scal};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

extern "C" int32_t gb_bg_columns(const gb_bg *h) { return h ? h->nv : 0; }

extern "C" const char *gb_bg_last_error(const gb_bg *h) { return h ? h->last_error.c_str() : ""; }

extern "C" int gb_bg_upload(gb_bg *h, const double *vocn, const double *mass, const double *volume, const double *rmass,
                            const double *vbio_part)
{
    gbgo::TraceRange tr_("bg_upload");
    if (!h || !vocn || !mass || !volume || !rmass || (h->d.n_l_sed > 0 && !vbio_part))
        return bfail(h, GB_GO_EINVAL, "upload: NULL array");
    BG_TRY(h, cudaSetDevice(h->device));
    const size_t nv = (size_t)h->nv;
    const size_t nf = (size_t)h->d.n_l_ocn * h->d.n_k * nv, np = (size_t)h->d.n_k * nv,
                 ns = (size_t)h->d.n_l_sed * h->d.n_k * nv;
    cudaStream_t s = h->stream;
    if (nv) {
        BG_TRY(h, cudaMemcpyAsync(h->vocn, vocn, nf * sizeof(double), cudaMemcpyHostToDevice, s));
        BG_TRY(h, cudaMemcpyAsync(h->mass, mass, np * sizeof(double), cudaMemcpyHostToDevice, s));
        BG_TRY(h, cudaMemcpyAsync(h->volume, volume, np * sizeof(double), cudaMemcpyHostToDevice, s));
        BG_TRY(h, cudaMemcpyAsync(h->rmass, rmass, np * sizeof(double), cudaMemcpyHostToDevice, s));
        if (ns) BG_TRY(h, cudaMemcpyAsync(h->vbio, vbio_part, ns * sizeof(double), cudaMemcpyHostToDevice, s));
        // the volume total (biogem.f90:1928-1936), fixed until the next upload
        BgArgs a = args_of(h);
        const long long nt = (long long)a.L * a.nv;
        k_bg_partials<0><<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(a);
        count_launches(1);
        BG_TRY(h, cudaGetLastError());
        BG_TRY(h, launch_seqsum<0>(a, s));
    }
    BG_TRY(h, cudaStreamSynchronize(s));
    h->have_state = true;
    return GB_GO_OK;
}

extern "C" int gb_bg_set_increments(gb_bg *h, const double *vdocn, const double *vdbio_part)
{
    if (!h || !vdocn || (h->d.n_l_sed > 0 && !vdbio_part)) return bfail(h, GB_GO_EINVAL, "set_increments: NULL array");
    BG_TRY(h, cudaSetDevice(h->device));
    const size_t nv = (size_t)h->nv;
    const size_t nf = (size_t)h->d.n_l_ocn * h->d.n_k * nv, ns = (size_t)h->d.n_l_sed * h->d.n_k * nv;
    if (nv) {
        BG_TRY(h, cudaMemcpyAsync(h->vdocn, vdocn, nf * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        if (ns) BG_TRY(h, cudaMemcpyAsync(h->vdbio, vdbio_part, ns * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    }
    BG_TRY(h, cudaStreamSynchronize(h->stream));
    h->have_inc = true;
    return GB_GO_OK;
}

extern "C" int gb_bg_tracercoupling(gb_bg *h, gb_go_handle *ocean)
{
    gbgo::TraceRange tr_("bg_tracercoupling");
    if (!h || !ocean) return bfail(h, GB_GO_EINVAL, "tracercoupling: NULL handle");
    if (!h->have_state || !h->have_inc) return bfail(h, GB_GO_ENOTREADY, "tracercoupling before upload/set_increments");
    OceanState o{};
    if (ocean_state(ocean, &o) != GB_GO_OK) return bfail(h, GB_GO_EINVAL, "tracercoupling: bad ocean handle");
    if (!o.state_ready) return bfail(h, GB_GO_ENOTREADY, "tracercoupling: ocean state not uploaded");
    if (o.d.maxi != h->d.n_i || o.d.maxj != h->d.n_j || o.d.maxk != h->d.n_k || o.d.L != h->d.n_l_ocn)
        return bfail(h, GB_GO_EINVAL, "tracercoupling: ocean grid differs from the BIOGEM grid");
    if (o.device != h->device) return bfail(h, GB_GO_EINVAL, "tracercoupling: handles on different devices");
    BG_TRY(h, cudaSetDevice(h->device));
    // the split-precision form: its current state in Fortran layout first (into ts_buf[cur])
    if (const int rr = ocean_refresh_rho(ocean))
        return bfail(h, rr, std::string("tracercoupling: ") + gb_go_last_error(ocean));
    cudaStream_t s = static_cast<cudaStream_t>(o.stream);
    BgArgs a = args_of(h);
    // go_ts: the wet cells of the current step buffer once the handle has stepped
    a.tsrc = o.steps_since_upload > 0 ? o.ts_buf[o.cur] : o.ts_static;
    a.ts_out = o.ts_static;
    a.ts1_out = o.ts1_static;
    const int maxi = o.d.maxi, maxj = o.d.maxj;
    if (a.nv > 0) {
        const long long nt = (long long)a.L * a.nv;
        const unsigned gq = (unsigned)((nt + 255) / 256);
        k_bg_partials<0><<<gq, 256, 0, s>>>(a);
        count_launches(1);
        BG_TRY(h, cudaGetLastError());
        BG_TRY(h, launch_seqsum<1>(a, s));
        k_bg_partials<1><<<gq, 256, 0, s>>>(a);
        count_launches(1);
        BG_TRY(h, cudaGetLastError());
        BG_TRY(h, launch_seqsum<2>(a, s));
        // the source (ts_static before any step) is read cell by cell by the thread that
        // rewrites the cell, so the wet cells are updated in place
        const long long nc = (long long)a.nk * a.nv;
        k_bg_apply<<<(unsigned)((nc + 255) / 256), 256, 0, s>>>(a);
        count_launches(1);
        BG_TRY(h, cudaGetLastError());
    }
    if (!*o.dry_zeroed) {
        // once per upload: nothing else writes the dry interior cells of ts_static / ts1_static
        const long long ncell = (long long)maxi * maxj * a.nk;
        const unsigned gz = (unsigned)std::min<long long>((ncell + 255) / 256, 8192);
        k_bg_zero<<<gz, 256, 0, s>>>(a, maxi, maxj, o.k1);
        count_launches(1);
        *o.dry_zeroed = true;
    }
    const long long nh = 2LL * maxj * a.nk * a.L;
    k_bg_halo<<<(unsigned)std::min<long long>((nh + 255) / 256, 4096), 256, 0, s>>>(a, maxi, maxj, o.k1);
    count_launches(1);
    BG_TRY(h, cudaGetLastError());
    const int r = ocean_state_reloaded(ocean);
    if (r) return bfail(h, r, "tracercoupling: reloading the ocean step buffers failed");
    BG_TRY(h, cudaStreamSynchronize(s));
    return GB_GO_OK;
}

extern "C" int gb_bg_download(gb_bg *h, double *vocn, double *mass, double *rmass, double *vbio_part)
{
    gbgo::TraceRange tr_("bg_download");
    if (!h) return GB_GO_EINVAL;
    if (!h->have_state) return bfail(h, GB_GO_ENOTREADY, "download before upload");
    BG_TRY(h, cudaSetDevice(h->device));
    const size_t nv = (size_t)h->nv;
    const size_t nf = (size_t)h->d.n_l_ocn * h->d.n_k * nv, np = (size_t)h->d.n_k * nv,
                 ns = (size_t)h->d.n_l_sed * h->d.n_k * nv;
    cudaStream_t s = h->stream;
    if (nv) {
        if (vocn) BG_TRY(h, cudaMemcpyAsync(vocn, h->vocn, nf * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (mass) BG_TRY(h, cudaMemcpyAsync(mass, h->mass, np * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (rmass) BG_TRY(h, cudaMemcpyAsync(rmass, h->rmass, np * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (vbio_part && ns) BG_TRY(h, cudaMemcpyAsync(vbio_part, h->vbio, ns * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    BG_TRY(h, cudaStreamSynchronize(s));
    return GB_GO_OK;
}
