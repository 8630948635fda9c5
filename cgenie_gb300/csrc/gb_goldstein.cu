// C-ABI of the GB300 GOLDSTEIN tracer step (include/gb_goldstein.h): one grid,
// device-resident state, drop-in for `CALL tstepo` (goldstein.f90:235).
#include "gb_internal.h"
#include "gb_fp32.h"
#include "../../include/gb_goldstein.h"

#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <map>
#include <mutex>
#include <string>
#include <vector>

using namespace gbgo;

static std::atomic<uint64_t> g_launches{0};

namespace gbgo {
void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
}

struct gb_go_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    Dims d{};
    PhysParams p{};
    int precision = GB_GO_FP64;
    int tile_i = 4, tile_j = 4;
    double *ts_buf[2] = {nullptr, nullptr};
    int cur = 0;
    double *ts_static = nullptr, *ts1_static = nullptr, *top = nullptr, *rho = nullptr, *u = nullptr;
    double *cost = nullptr;
    int32_t *icosd = nullptr;
    unsigned long long *diag = nullptr;  // two slots of {dmax bits, limps}
    int slot = 0;
    double *metrics = nullptr;
    int32_t *k1 = nullptr;
    double *ediff1 = nullptr;
    double *stage = nullptr;
    double *mldketau = nullptr, *mld = nullptr, *mldpe1 = nullptr;   // imld = 1, (maxi, maxj)
    int32_t *mldk = nullptr;
    double *inv_part = nullptr;
    int inv_blocks = 0;
    double *inv_noalloc = nullptr;        // static scratch of gb_go_inventory_noalloc on this device
    std::string inv_noalloc_err;
    Metrics m{};
    std::vector<int32_t> k1_host;
    bool state_ready = false, vel_ready = false;
    bool dry_zeroed = false;   // interior dry cells of ts_static/ts1_static are 0 (after a coupling)
    long long steps_since_upload = 0;
    std::string last_error;
    Fp32Member f32{};   // FP32-flux path data
};

static const char *kErrText[] = {
    "ok", "invalid argument", "unsupported option", "CUDA error", "out of memory",
    "state or velocity not uploaded", "device-side error", "size beyond compiled-in limit",
    "non-finite tracer value",
};

extern "C" const char *gb_go_errstr(int code)
{
    int c = -code;
    if (c < 0 || c > 8) return "unknown error";
    return kErrText[c];
}

extern "C" const char *gb_go_last_error(const gb_go_handle *h) { return h ? h->last_error.c_str() : ""; }

extern "C" uint64_t gb_go_kernel_launch_count(void) { return g_launches.load(); }

static int fail(gb_go_handle *h, int code, const std::string &msg)
{
    if (h) h->last_error = msg;
    return code;
}

static int cuda_fail(gb_go_handle *h, cudaError_t e, const char *what)
{
    return fail(h, GB_GO_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CUDA_TRY(h, call)                                  \
    do {                                                   \
        cudaError_t _e = (call);                           \
        if (_e != cudaSuccess) return cuda_fail(h, _e, #call); \
    } while (0)

namespace gbgo {

int validate_config(const gb_go_dims *dims, const gb_go_params *params, const gb_go_grid *grid, std::string &msg)
{
    if (!dims || !params || !grid) { msg = "NULL dims/params/grid"; return GB_GO_EINVAL; }
    if (dims->maxi < 2 || dims->maxj < 2 || dims->maxk < 2 || dims->maxl < 2) {
        msg = "dimensions must be >= 2 (maxl >= 2: T and S are read by the equation of state)";
        return GB_GO_EINVAL;
    }
    if (dims->maxk > GB_GO_MAX_K || dims->maxl > GB_GO_MAX_L) {
        msg = "maxk > GB_GO_MAX_K or maxl > GB_GO_MAX_L";
        return GB_GO_ERANGE;
    }
    if ((long long)dims->maxi * dims->maxj > (1LL << 28)) { msg = "grid too large"; return GB_GO_ERANGE; }
    if (params->imld != 0 && params->imld != 1) { msg = "imld must be 0 or 1"; return GB_GO_EINVAL; }
    if (params->imld == 1 && (!grid->mlddec || !grid->mlddecd || !grid->mldketau)) {
        msg = "imld=1 needs mlddec, mlddecd and mldketau";
        return GB_GO_EINVAL;
    }
    if (params->ieos != 0 && params->ieos != 1) { msg = "ieos must be 0 or 1"; return GB_GO_EINVAL; }
    if (params->iconv != 0 && params->iconv != 1) { msg = "iconv must be 0 or 1"; return GB_GO_EINVAL; }
    if (params->iediff < 0) { msg = "iediff must be >= 0"; return GB_GO_EINVAL; }
    if (params->precision != GB_GO_FP64 && params->precision != GB_GO_FP32FLUX) {
        msg = "precision must be GB_GO_FP64 or GB_GO_FP32FLUX";
        return GB_GO_EINVAL;
    }
    if (params->reserved != 0) { msg = "reserved must be 0"; return GB_GO_EINVAL; }
    if (!(params->diff[0] != 0.0)) { msg = "diff(1) must be non-zero"; return GB_GO_EINVAL; }
    const gb_go_grid *g = grid;
    if (!g->k1 || !g->rc || !g->rc2 || !g->cv || !g->cv2 || !g->dsv || !g->rdsv || !g->ds || !g->rds || !g->dz ||
        !g->dza || !g->rdz || !g->rdza || !g->zro || !g->dt || !g->zw) {
        msg = "NULL grid metric";
        return GB_GO_EINVAL;
    }
    if (params->diso && !g->ssmax) { msg = "diso needs ssmax"; return GB_GO_EINVAL; }
    if (params->iediff > 0 && params->iediff < 3 && (!g->ediff1 || !g->diffmax)) {
        msg = "iediff 1/2 needs ediff1 and diffmax";
        return GB_GO_EINVAL;
    }
    const int NI = dims->maxi + 2, NJ = dims->maxj + 2;
    for (int i = 0; i < NI; ++i) {
        if (g->k1[i] <= dims->maxk || g->k1[i + (size_t)NI * (NJ - 1)] <= dims->maxk) {
            msg = "k1 rows j=0 and j=maxj+1 must be land (k1 > maxk)";
            return GB_GO_EINVAL;
        }
    }
    for (int j = 0; j < NJ; ++j) {
        const int32_t *row = g->k1 + (size_t)NI * j;
        if (row[0] != row[dims->maxi] || row[NI - 1] != row[1]) {
            msg = "k1 must be periodic in i: k1(0,j)=k1(maxi,j), k1(maxi+1,j)=k1(1,j)";
            return GB_GO_EINVAL;
        }
        for (int i = 0; i < NI; ++i) {
            if (row[i] < 1) { msg = "k1 must be >= 1"; return GB_GO_EINVAL; }
        }
    }
    return GB_GO_OK;
}

// Fortran-indexed metric blob: 8 j-arrays of maxj+2 entries then 11 k-arrays of maxk+2.
void build_metric_blob(const gb_go_dims *dims, const gb_go_params *params, const gb_go_grid *g, std::vector<double> &blob)
{
    const int nj = dims->maxj + 2, nk = dims->maxk + 2, maxj = dims->maxj, maxk = dims->maxk;
    blob.assign((size_t)8 * nj + (size_t)11 * nk, 0.0);
    double *b = blob.data();
    double *rc = b, *rc2 = b + nj, *cv = b + 2 * nj, *cv2 = b + 3 * nj, *dsv = b + 4 * nj, *rdsv = b + 5 * nj,
           *ds = b + 6 * nj, *rds = b + 7 * nj;
    double *kb = b + 8 * nj;
    double *dz = kb, *dza = kb + nk, *rdz = kb + 2 * nk, *rdza = kb + 3 * nk, *zro = kb + 4 * nk, *dt = kb + 5 * nk,
           *zw = kb + 6 * nk, *ssmax = kb + 7 * nk, *diffmax = kb + 8 * nk;
    double *mlddec = kb + 9 * nk, *mlddecd = kb + 10 * nk;
    if (params->imld == 1)
        for (int k = 1; k <= maxk; ++k) { mlddec[k] = g->mlddec[k - 1]; mlddecd[k] = g->mlddecd[k - 1]; }
    for (int j = 0; j <= maxj; ++j) { rc[j] = g->rc[j]; rc2[j] = g->rc2[j]; cv[j] = g->cv[j]; }
    for (int j = 1; j <= maxj - 1; ++j) { cv2[j] = g->cv2[j - 1]; dsv[j] = g->dsv[j - 1]; rdsv[j] = g->rdsv[j - 1]; }
    for (int j = 1; j <= maxj; ++j) { ds[j] = g->ds[j - 1]; rds[j] = g->rds[j - 1]; }
    for (int k = 1; k <= maxk; ++k) {
        dz[k] = g->dz[k - 1]; dza[k] = g->dza[k - 1]; rdz[k] = g->rdz[k - 1]; rdza[k] = g->rdza[k - 1];
        zro[k] = g->zro[k - 1]; dt[k] = g->dt[k - 1];
    }
    for (int k = 0; k <= maxk; ++k) zw[k] = g->zw[k];
    if (params->diso && g->ssmax)
        for (int k = 1; k <= maxk - 1; ++k) ssmax[k] = g->ssmax[k - 1];
    if (params->iediff > 0 && params->iediff < 3 && g->diffmax)
        for (int k = 1; k <= maxk; ++k) diffmax[k] = g->diffmax[k - 1];
}

Metrics metrics_from_blob(const double *b, const int32_t *k1, const double *ediff1, int maxj, int maxk)
{
    const int nj = maxj + 2, nk = maxk + 2;
    Metrics m{};
    m.rc = b; m.rc2 = b + nj; m.cv = b + 2 * nj; m.cv2 = b + 3 * nj; m.dsv = b + 4 * nj; m.rdsv = b + 5 * nj;
    m.ds = b + 6 * nj; m.rds = b + 7 * nj;
    const double *kb = b + 8 * nj;
    m.dz = kb; m.dza = kb + nk; m.rdz = kb + 2 * nk; m.rdza = kb + 3 * nk; m.zro = kb + 4 * nk; m.dt = kb + 5 * nk;
    m.zw = kb + 6 * nk; m.ssmax = kb + 7 * nk; m.diffmax = kb + 8 * nk;
    m.mlddec = kb + 9 * nk; m.mlddecd = kb + 10 * nk;
    m.ediff1 = ediff1;
    m.k1 = k1;
    return m;
}

PhysParams phys_from(const gb_go_params *pp, const gb_go_grid *g)
{
    PhysParams p{};
    p.diff1 = pp->diff[0];
    p.diff2 = pp->diff[1];
    for (int n = 0; n < 5; ++n) p.ec[n] = pp->ec[n];
    p.ediff0 = pp->ediff0;
    p.ediffpow2 = pp->ediffpow2;
    p.dsc = pp->dsc;
    p.dphi = g->dphi;
    p.rdphi = g->rdphi;
    p.ieos = pp->ieos;
    p.iediff = (pp->iediff > 0 && pp->iediff < 3) ? pp->iediff : 0;
    p.ediffpow2i = pp->ediffpow2i;
    p.iconv = pp->iconv;
    p.diso = pp->diso ? 1 : 0;
    p.imld = pp->imld;
    p.mldpebuoycoeff = pp->mldpebuoycoeff;
    return p;
}

}  // namespace gbgo

// ---------------------------------------------------------------------------
// auxiliary kernels

// out = stat; wet interior cells (and, for ts1, wet halo columns) from cur.
__global__ void k_merge_download(double *out, const double *stat, const double *cur, Dims d, const int32_t *k1,
                                 int with_halo, int use_cur)
{
    const size_t ncell = (size_t)d.NI * d.NJ * (d.maxk + 2);
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % d.NI);
        const int j = (int)((c / d.NI) % d.NJ);
        const int k = (int)(c / ((size_t)d.NI * d.NJ));
        bool take = false;
        if (use_cur && k >= 1 && k <= d.maxk && j >= 1 && j <= d.maxj) {
            const int kk = k1[i + d.NI * j];
            if (i >= 1 && i <= d.maxi) take = k >= kk;
            else if (with_halo) take = k >= kk;
        }
        const double *src = take ? cur : stat;
        for (int l = 0; l < d.L; ++l) out[c * d.L + l] = src[c * d.L + l];
    }
}

// Per-tracer Neumaier partial sums of ts*ds(j)*dz(k) over wet interior cells.
__global__ void k_inventory_partial(const double *ts, Dims d, Metrics m, double *part)
{
    const int l = blockIdx.y;
    const size_t ncol = (size_t)d.maxi * d.maxj;
    const size_t ncell = ncol * d.maxk;
    double s = 0.0, comp = 0.0;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % d.maxi) + 1;
        const int j = (int)((c / d.maxi) % d.maxj) + 1;
        const int k = (int)(c / ncol) + 1;
        if (k < m.k1[i + d.NI * j]) continue;
        const double x = __dmul_rn(__dmul_rn(ts[ts_index(d, l, i, j, k)], m.ds[j]), m.dz[k]);
        const double t = __dadd_rn(s, x);
        if (fabs(s) >= fabs(x)) comp = __dadd_rn(comp, __dadd_rn(__dadd_rn(s, -t), x));
        else comp = __dadd_rn(comp, __dadd_rn(__dadd_rn(x, -t), s));
        s = t;
    }
    __shared__ double ss[256], sc[256];
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = comp;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, Cc = 0.0;
        for (int n = 0; n < blockDim.x; ++n) {
            const double x = ss[n];
            const double t = __dadd_rn(S, x);
            if (fabs(S) >= fabs(x)) Cc = __dadd_rn(Cc, __dadd_rn(__dadd_rn(S, -t), x));
            else Cc = __dadd_rn(Cc, __dadd_rn(__dadd_rn(x, -t), S));
            S = t;
            Cc = __dadd_rn(Cc, sc[n]);
        }
        part[2 * ((size_t)l * gridDim.x + blockIdx.x)] = S;
        part[2 * ((size_t)l * gridDim.x + blockIdx.x) + 1] = Cc;
    }
}

__global__ void k_inventory_final(const double *part, int nblk, int L, double *out)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= L) return;
    double S = 0.0, Cc = 0.0;
    for (int n = 0; n < nblk; ++n) {
        const double x = part[2 * ((size_t)l * nblk + n)];
        const double t = __dadd_rn(S, x);
        if (fabs(S) >= fabs(x)) Cc = __dadd_rn(Cc, __dadd_rn(__dadd_rn(S, -t), x));
        else Cc = __dadd_rn(Cc, __dadd_rn(__dadd_rn(x, -t), S));
        S = t;
        Cc = __dadd_rn(Cc, part[2 * ((size_t)l * nblk + n) + 1]);
    }
    out[l] = __dadd_rn(S, Cc);
}

// ---------------------------------------------------------------------------

static void free_handle(gb_go_handle *h)
{
    if (!h) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->ts_buf[0]); cudaFree(h->ts_buf[1]);
    cudaFree(h->ts_static); cudaFree(h->ts1_static); cudaFree(h->top); cudaFree(h->rho); cudaFree(h->u);
    cudaFree(h->cost); cudaFree(h->icosd); cudaFree(h->diag); cudaFree(h->metrics); cudaFree(h->k1);
    cudaFree(h->ediff1); cudaFree(h->stage); cudaFree(h->inv_part);
    cudaFree(h->mldketau); cudaFree(h->mld); cudaFree(h->mldpe1); cudaFree(h->mldk);
    fp32_member_free(&h->f32);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    if (prev >= 0) cudaSetDevice(prev);
    delete h;
}

// Scratch of gb_go_inventory_noalloc, a file-scope device array: for up to
// kInvNoallocMaxL tracers, 64 (sum, compensation) pairs per tracer from the partial
// kernel, then the per-tracer results.  Every entry is written before it is read, so
// nothing has to start at zero.
constexpr int kInvNoallocBlocks = 64;
constexpr int kInvNoallocMaxL = 64;
constexpr int kInvNoallocDoubles = 2 * kInvNoallocBlocks * kInvNoallocMaxL + kInvNoallocMaxL;
static __device__ __align__(256) double g_inv_noalloc[kInvNoallocDoubles];

// Device address of g_inv_noalloc, looked up once per device at handle set-up, with that
// device current.  In host code the name g_inv_noalloc is a host-side stand-in, not a
// device address: kernels get this pointer.
static cudaError_t inv_noalloc_scratch(int device, double **out)
{
    static std::mutex mu;
    static std::map<int, double *> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(device);
    if (it != cache.end()) {
        *out = it->second;
        return cudaSuccess;
    }
    double *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_inv_noalloc);
    if (e != cudaSuccess) return e;
    cache[device] = p;
    *out = p;
    return cudaSuccess;
}

extern "C" int gb_go_create(const gb_go_dims *dims, const gb_go_params *params, const gb_go_grid *grid, int device,
                            gb_go_handle **out)
{
    if (!out) return GB_GO_EINVAL;
    *out = nullptr;
    std::string msg;
    int rc = validate_config(dims, params, grid, msg);
    if (rc) {
        fprintf(stderr, "gb_go_create: %s\n", msg.c_str());
        return rc;
    }
    gb_go_handle *h = new (std::nothrow) gb_go_handle();
    if (!h) return GB_GO_ENOMEM;
    if (device < 0) {
        if (cudaGetDevice(&h->device) != cudaSuccess) { delete h; return GB_GO_ECUDA; }
    } else {
        h->device = device;
    }
    if (cudaSetDevice(h->device) != cudaSuccess) { delete h; return GB_GO_ECUDA; }
    h->d.maxi = dims->maxi; h->d.maxj = dims->maxj; h->d.maxk = dims->maxk; h->d.L = dims->maxl;
    h->d.NI = dims->maxi + 2; h->d.NJ = dims->maxj + 2;
    h->p = phys_from(params, grid);
    h->precision = params->precision;
    {
        int nsm = 0;
        if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess || nsm < 1) nsm = 1;
        step_fp64_tile(dims->maxi, dims->maxj, dims->maxk, nsm, &h->tile_i, &h->tile_j);
    }

    const size_t nts = (size_t)h->d.L * h->d.NI * h->d.NJ * (h->d.maxk + 2);
    const size_t ntop = (size_t)h->d.L * h->d.NI * h->d.NJ;
    const size_t nrho = (size_t)h->d.NI * h->d.NJ * (h->d.maxk + 1);
    const size_t nu = (size_t)3 * (h->d.maxi + 1) * (h->d.maxj + 1) * h->d.maxk;
    const size_t ncol = (size_t)h->d.maxi * h->d.maxj;
    std::vector<double> blob;
    build_metric_blob(dims, params, grid, blob);
    h->inv_blocks = 64;
    {
        const cudaError_t se = inv_noalloc_scratch(h->device, &h->inv_noalloc);
        if (se != cudaSuccess) {
            h->inv_noalloc = nullptr;
            h->inv_noalloc_err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(se);
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        h->stream = h->own_stream;
        e = cudaMalloc(&h->ts_buf[0], nts * sizeof(double));
    }
    if (e == cudaSuccess) e = cudaMalloc(&h->ts_buf[1], nts * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->ts_static, nts * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->ts1_static, nts * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->stage, nts * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->top, ntop * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->rho, nrho * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->u, nu * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->cost, ncol * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->icosd, ncol * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->diag, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&h->metrics, blob.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->k1, (size_t)h->d.NI * h->d.NJ * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&h->inv_part, (size_t)2 * h->inv_blocks * h->d.L * sizeof(double));
    const bool need_ediff = params->iediff > 0 && params->iediff < 3;
    const size_t ned = (size_t)h->d.maxi * h->d.maxj * (h->d.maxk - 1);
    if (e == cudaSuccess && need_ediff) e = cudaMalloc(&h->ediff1, ned * sizeof(double));
    const bool need_mld = params->imld == 1;
    if (e == cudaSuccess && need_mld) e = cudaMalloc(&h->mldketau, ncol * sizeof(double));
    if (e == cudaSuccess && need_mld) e = cudaMalloc(&h->mld, ncol * sizeof(double));
    if (e == cudaSuccess && need_mld) e = cudaMalloc(&h->mldpe1, ncol * sizeof(double));
    if (e == cudaSuccess && need_mld) e = cudaMalloc(&h->mldk, ncol * sizeof(int32_t));
    if (e == cudaSuccess && need_mld)
        e = cudaMemcpyAsync(h->mldketau, grid->mldketau, ncol * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && need_mld) e = cudaMemsetAsync(h->mld, 0, ncol * sizeof(double), h->stream);
    if (e == cudaSuccess && need_mld) e = cudaMemsetAsync(h->mldk, 0, ncol * sizeof(int32_t), h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->metrics, blob.data(), blob.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h->k1, grid->k1, (size_t)h->d.NI * h->d.NJ * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && need_ediff) e = cudaMemcpyAsync(h->ediff1, grid->ediff1, ned * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->diag, 0, 4 * sizeof(unsigned long long), h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->cost, 0, ncol * sizeof(double), h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->icosd, 0, ncol * sizeof(int32_t), h->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->u, 0, nu * sizeof(double), h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        fprintf(stderr, "gb_go_create: %s\n", cudaGetErrorString(e));
        int code = (e == cudaErrorMemoryAllocation) ? GB_GO_ENOMEM : GB_GO_ECUDA;
        free_handle(h);
        return code;
    }
    h->k1_host.assign(grid->k1, grid->k1 + (size_t)h->d.NI * h->d.NJ);
    h->m = metrics_from_blob(h->metrics, h->k1, h->ediff1, h->d.maxj, h->d.maxk);
    if (h->precision == GB_GO_FP32FLUX) {
        int r = fp32_member_init(&h->f32, h->d, h->p, h->m, blob, h->k1_host.data(), h->stream, msg);
        if (r) {
            fprintf(stderr, "gb_go_create: %s\n", msg.c_str());
            free_handle(h);
            return r;
        }
    }
    *out = h;
    return GB_GO_OK;
}

extern "C" void gb_go_destroy(gb_go_handle *h) { free_handle(h); }

extern "C" int gb_go_set_stream(gb_go_handle *h, void *cuda_stream)
{
    if (!h) return GB_GO_EINVAL;
    h->stream = cuda_stream ? (cudaStream_t)cuda_stream : h->own_stream;
    return GB_GO_OK;
}

namespace gbgo {
int ocean_state(gb_go_handle *h, OceanState *o)
{
    if (!h || !o) return GB_GO_EINVAL;
    o->d = h->d;
    o->precision = h->precision;
    o->device = h->device;
    o->stream = h->stream;
    o->ts_static = h->ts_static;
    o->ts1_static = h->ts1_static;
    o->ts_buf[0] = h->ts_buf[0];
    o->ts_buf[1] = h->ts_buf[1];
    o->cur = h->cur;
    o->steps_since_upload = h->steps_since_upload;
    o->k1 = h->k1;
    o->state_ready = h->state_ready;
    o->dry_zeroed = &h->dry_zeroed;
    o->rho = h->rho;
    o->u = h->u;
    o->vel_ready = &h->vel_ready;
    return GB_GO_OK;
}

int ocean_refresh_rho(gb_go_handle *h)
{
    if (h->precision != GB_GO_FP32FLUX || h->steps_since_upload == 0) return GB_GO_OK;
    const int r = fp32_member_export(&h->f32, h->ts_buf[h->cur], h->rho, h->ts_static, h->stream);
    return r ? fail(h, r, std::string("fp32 export failed: ") + fp32_cuda_error_string()) : GB_GO_OK;
}

int ocean_refresh_rho_only(gb_go_handle *h)
{
    if (h->precision != GB_GO_FP32FLUX || h->steps_since_upload == 0) return GB_GO_OK;
    const int r = fp32_member_rho(&h->f32, h->rho, h->ts_static, h->stream);
    return r ? fail(h, r, std::string("fp32 density failed: ") + fp32_cuda_error_string()) : GB_GO_OK;
}

int ocean_velocity_changed(gb_go_handle *h)
{
    if (h->precision != GB_GO_FP32FLUX) {
        h->vel_ready = true;
        return GB_GO_OK;
    }
    if (!h->vel_ready) return fail(h, GB_GO_ENOTREADY, "split-precision form: the first velocity field comes from gb_go_set_velocity");
    const int r = fp32_member_set_velocity(&h->f32, nullptr, h->u, h->m, h->stream);
    return r ? fail(h, r, "fp32 set_velocity (device) failed") : GB_GO_OK;
}

int ocean_state_reloaded(gb_go_handle *h)
{
    const size_t nts = (size_t)h->d.L * h->d.NI * h->d.NJ * (h->d.maxk + 2);
    CUDA_TRY(h, cudaMemcpyAsync(h->ts_buf[0], h->ts1_static, nts * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->ts_buf[1], h->ts_static, nts * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    h->cur = 0;
    h->slot = 0;
    h->steps_since_upload = 0;
    if (h->precision == GB_GO_FP32FLUX) {
        const int r = fp32_member_reload(&h->f32, h->ts1_static, h->stream);
        if (r) return fail(h, r, "fp32 reload failed");
    }
    return GB_GO_OK;
}
}  // namespace gbgo

extern "C" int gb_go_upload_state(gb_go_handle *h, const double *ts, const double *ts1, const double *rho)
{
    gbgo::TraceRange tr_("go_upload_state");
    if (!h || !ts || !ts1 || !rho) return fail(h, GB_GO_EINVAL, "upload_state: NULL array");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t nts = (size_t)h->d.L * h->d.NI * h->d.NJ * (h->d.maxk + 2);
    const size_t ntop = (size_t)h->d.L * h->d.NI * h->d.NJ;
    const size_t nrho = (size_t)h->d.NI * h->d.NJ * (h->d.maxk + 1);
    CUDA_TRY(h, cudaMemcpyAsync(h->ts_static, ts, nts * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->ts1_static, ts1, nts * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->ts_buf[0], h->ts1_static, nts * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->ts_buf[1], h->ts_static, nts * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->top, h->ts_static + ntop * (h->d.maxk + 1), ntop * sizeof(double),
                                cudaMemcpyDeviceToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->rho, rho, nrho * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    h->cur = 0;
    h->slot = 0;
    h->state_ready = true;
    h->dry_zeroed = false;
    h->steps_since_upload = 0;
    if (h->precision == GB_GO_FP32FLUX) {
        int r = fp32_member_upload(&h->f32, ts1, ts, h->ts_buf[0], h->stream);
        if (r) return fail(h, r, "fp32 upload failed");
        if (h->p.imld == 1) {
            // the mixed layer's arrays, and rho(maxk) of the uploaded rho as the previous step's
            r = fp32_member_set_mixed_layer(&h->f32, h->mldketau, h->mld, h->mldk, h->m.mlddec, h->m.mlddecd, h->rho,
                                            h->stream);
            if (r) return fail(h, r, "fp32 mixed-layer set-up failed");
        }
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}

extern "C" int gb_go_set_forcing(gb_go_handle *h, const double *ts_top)
{
    if (!h || !ts_top) return fail(h, GB_GO_EINVAL, "set_forcing: NULL array");
    if (!h->state_ready) return fail(h, GB_GO_ENOTREADY, "set_forcing before upload_state");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t ntop = (size_t)h->d.L * h->d.NI * h->d.NJ;
    CUDA_TRY(h, cudaMemcpyAsync(h->top, ts_top, ntop * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(h->ts_static + ntop * (h->d.maxk + 1), h->top, ntop * sizeof(double),
                                cudaMemcpyDeviceToDevice, h->stream));
    if (h->precision == GB_GO_FP32FLUX) {
        int r = fp32_member_set_top(&h->f32, ts_top, h->stream);
        if (r) return fail(h, r, "fp32 set_forcing failed");
    }
    return GB_GO_OK;
}

extern "C" int gb_go_set_velocity(gb_go_handle *h, const double *u)
{
    if (!h || !u) return fail(h, GB_GO_EINVAL, "set_velocity: NULL array");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t nu = (size_t)3 * (h->d.maxi + 1) * (h->d.maxj + 1) * h->d.maxk;
    CUDA_TRY(h, cudaMemcpyAsync(h->u, u, nu * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (h->precision == GB_GO_FP32FLUX) {
        int r = fp32_member_set_velocity(&h->f32, u, h->u, h->m, h->stream);
        if (r) return fail(h, r, "fp32 set_velocity failed");
    }
    h->vel_ready = true;
    return GB_GO_OK;
}

extern "C" int gb_go_set_diag(gb_go_handle *h, const double *cost, const int32_t *icosd)
{
    if (!h) return GB_GO_EINVAL;
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t ncol = (size_t)h->d.maxi * h->d.maxj;
    if (cost) CUDA_TRY(h, cudaMemcpyAsync(h->cost, cost, ncol * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (icosd) CUDA_TRY(h, cudaMemcpyAsync(h->icosd, icosd, ncol * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    return GB_GO_OK;
}

extern "C" int gb_go_tstepo(gb_go_handle *h, int32_t nsteps)
{
    gbgo::TraceRange tr_("go_tstepo");
    if (!h || nsteps < 0) return fail(h, GB_GO_EINVAL, "tstepo: bad arguments");
    if (!h->state_ready || !h->vel_ready) return fail(h, GB_GO_ENOTREADY, "tstepo before upload_state/set_velocity");
    CUDA_TRY(h, cudaSetDevice(h->device));
    if (h->precision == GB_GO_FP32FLUX) {
        int r = fp32_member_step(&h->f32, h->ts_buf, &h->cur, h->rho, h->ts_static, h->cost, h->icosd,
                                 h->diag, &h->slot, nsteps, h->stream);
        if (r) return fail(h, r, "fp32 step launch failed");
        h->steps_since_upload += nsteps;
        return GB_GO_OK;
    }
    StepArgs a{};
    a.d = h->d;
    a.p = h->p;
    a.m = h->m;
    a.ts_static = h->ts_static;
    a.top = h->top;
    a.rho = h->rho;
    a.u = h->u;
    a.cost = h->cost;
    a.icosd = h->icosd;
    a.tile_i = h->tile_i;
    a.tile_j = h->tile_j;
    a.tiles_i = (h->d.maxi + h->tile_i - 1) / h->tile_i;
    a.mldketau = h->mldketau;
    a.mld = h->mld;
    a.mldk = h->mldk;
    a.mldpe1 = h->mldpe1;
    for (int s = 0; s < nsteps; ++s) {
        a.ts1 = h->ts_buf[h->cur];
        a.ts = h->ts_buf[1 - h->cur];
        // ts at the start of the step: the uploaded ts before the first step, then the last
        // step's result (equal to ts1 on wet cells)
        a.ts_start = h->steps_since_upload == 0 ? h->ts_static : a.ts1;
        a.diag = h->diag + 2 * h->slot;
        a.diag_next = h->diag + 2 * (1 - h->slot);
        if (launch_step_fp64(a, h->stream)) return cuda_fail(h, cudaGetLastError(), "step_fp64 launch");
        count_launches(1);
        h->cur = 1 - h->cur;
        h->slot = 1 - h->slot;
        ++h->steps_since_upload;
    }
    return GB_GO_OK;
}

extern "C" int gb_go_set_mld_wind(gb_go_handle *h, const double *mldketau)
{
    if (!h || !mldketau) return fail(h, GB_GO_EINVAL, "set_mld_wind: NULL array");
    if (h->p.imld != 1) return fail(h, GB_GO_EINVAL, "set_mld_wind: the handle was created with imld = 0");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t ncol = (size_t)h->d.maxi * h->d.maxj;
    CUDA_TRY(h, cudaMemcpyAsync(h->mldketau, mldketau, ncol * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}

extern "C" int gb_go_download_mld(gb_go_handle *h, double *mld, int32_t *mldk)
{
    if (!h) return GB_GO_EINVAL;
    if (h->p.imld != 1) return fail(h, GB_GO_EINVAL, "download_mld: the handle was created with imld = 0");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t ncol = (size_t)h->d.maxi * h->d.maxj;
    if (mld) CUDA_TRY(h, cudaMemcpyAsync(mld, h->mld, ncol * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (mldk) CUDA_TRY(h, cudaMemcpyAsync(mldk, h->mldk, ncol * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}

extern "C" int gb_go_download(gb_go_handle *h, double *ts, double *ts1, double *rho, double *cost, int32_t *icosd,
                              double *dmax, int32_t *limps)
{
    gbgo::TraceRange tr_("go_download");
    if (!h) return GB_GO_EINVAL;
    if (!h->state_ready) return fail(h, GB_GO_ENOTREADY, "download before upload_state");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const size_t nts = (size_t)h->d.L * h->d.NI * h->d.NJ * (h->d.maxk + 2);
    const size_t nrho = (size_t)h->d.NI * h->d.NJ * (h->d.maxk + 1);
    const size_t ncol = (size_t)h->d.maxi * h->d.maxj;
    const int use_cur = h->steps_since_upload > 0 ? 1 : 0;
    const double *curbuf = h->ts_buf[h->cur];
    if (h->precision == GB_GO_FP32FLUX && use_cur) {
        int r = fp32_member_export(&h->f32, h->ts_buf[h->cur], h->rho, h->ts_static, h->stream);
        if (r) return fail(h, r, "fp32 export failed");
    }
    const size_t ncell = (size_t)h->d.NI * h->d.NJ * (h->d.maxk + 2);
    const int blocks = (int)std::min<size_t>((ncell + 255) / 256, 4096);
    if (ts) {
        k_merge_download<<<blocks, 256, 0, h->stream>>>(h->stage, h->ts_static, curbuf, h->d, h->k1, 0, use_cur);
        count_launches(1);
        CUDA_TRY(h, cudaGetLastError());
        CUDA_TRY(h, cudaMemcpyAsync(ts, h->stage, nts * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    }
    if (ts1) {
        k_merge_download<<<blocks, 256, 0, h->stream>>>(h->stage, h->ts1_static, curbuf, h->d, h->k1, 1, use_cur);
        count_launches(1);
        CUDA_TRY(h, cudaGetLastError());
        CUDA_TRY(h, cudaMemcpyAsync(ts1, h->stage, nts * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    if (rho) CUDA_TRY(h, cudaMemcpyAsync(rho, h->rho, nrho * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (cost) CUDA_TRY(h, cudaMemcpyAsync(cost, h->cost, ncol * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (icosd) CUDA_TRY(h, cudaMemcpyAsync(icosd, h->icosd, ncol * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    unsigned long long dg[2] = {0, 0};
    if ((dmax || limps) && h->steps_since_upload > 0)
        CUDA_TRY(h, cudaMemcpyAsync(dg, h->diag + 2 * (1 - h->slot), sizeof(dg), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (dmax) {
        double v;
        std::memcpy(&v, &dg[0], sizeof(v));
        *dmax = v;
    }
    if (limps) *limps = h->p.diso ? (int32_t)dg[1] : 0;
    return GB_GO_OK;
}

extern "C" int gb_go_inventory(gb_go_handle *h, double *out)
{
    gbgo::TraceRange tr_("go_inventory");
    if (!h || !out) return GB_GO_EINVAL;
    if (!h->state_ready) return fail(h, GB_GO_ENOTREADY, "inventory before upload_state");
    CUDA_TRY(h, cudaSetDevice(h->device));
    const double *src = h->ts_buf[h->cur];
    if (h->steps_since_upload == 0) src = h->ts_static;
    else if (h->precision == GB_GO_FP32FLUX) {
        int r = fp32_member_fortran(&h->f32, h->ts_buf[h->cur], h->stream);
        if (r) return fail(h, r, "fp32 export failed");
    }
    dim3 grid(h->inv_blocks, h->d.L);
    k_inventory_partial<<<grid, 256, 0, h->stream>>>(src, h->d, h->m, h->inv_part);
    k_inventory_final<<<(h->d.L + 63) / 64, 64, 0, h->stream>>>(h->inv_part, h->inv_blocks, h->d.L, h->stage);
    count_launches(2);
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaMemcpyAsync(out, h->stage, h->d.L * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}

extern "C" int gb_go_inventory_noalloc(gb_go_handle *h, double *out)
{
    if (!h || !out) return GB_GO_EINVAL;
    if (!h->state_ready) return fail(h, GB_GO_ENOTREADY, "inventory before upload_state");
    if (h->d.L > kInvNoallocMaxL)
        return fail(h, GB_GO_ERANGE, "gb_go_inventory_noalloc takes at most 64 tracers (static scratch of 8256 doubles)");
    if (!h->inv_noalloc) return fail(h, GB_GO_ECUDA, "gb_go_inventory_noalloc scratch unavailable: " + h->inv_noalloc_err);
    CUDA_TRY(h, cudaSetDevice(h->device));
    const double *src = h->ts_buf[h->cur];
    if (h->steps_since_upload == 0) src = h->ts_static;
    else if (h->precision == GB_GO_FP32FLUX) {
        int r = fp32_member_fortran(&h->f32, h->ts_buf[h->cur], h->stream);
        if (r) return fail(h, r, "fp32 export failed");
    }
    // the same kernels and partition as gb_go_inventory, on the static scratch
    double *part = h->inv_noalloc;
    double *res = part + 2 * (size_t)kInvNoallocBlocks * h->d.L;
    dim3 grid(kInvNoallocBlocks, h->d.L);
    k_inventory_partial<<<grid, 256, 0, h->stream>>>(src, h->d, h->m, part);
    k_inventory_final<<<(h->d.L + 63) / 64, 64, 0, h->stream>>>(part, kInvNoallocBlocks, h->d.L, res);
    count_launches(2);
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaMemcpyAsync(out, res, h->d.L * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}

extern "C" int gb_go_sync(gb_go_handle *h)
{
    if (!h) return GB_GO_EINVAL;
    CUDA_TRY(h, cudaSetDevice(h->device));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return GB_GO_OK;
}
