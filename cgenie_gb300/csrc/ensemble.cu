// Batched ensemble runtime: many independent GOLDSTEIN grids advanced together
// by one persistent launch of the FP32-flux kernel per step (no counterpart in
// the reference, which runs one grid serially).
//
// Members are admitted and retired between steps (continuous batching).  Each
// member owns its state ping-pong, uploaded copy and static transfer
// coefficients, allocated from a stream-ordered memory pool so admission does
// not synchronise the device.  A member advances at step s while
// s < stop_step; its current state is in buf[(s + parity) & 1].  The work list
// holds (member, column tile) items ordered by decreasing cost (longest
// processing time first); persistent CTAs take items round-robin.
#include "gb_fp32.h"
#include "co_column.cuh"
#include "gb_internal.h"
#include "../../include/gb_goldstein.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>
#include <thread>
#include <atomic>
#include <unordered_map>

namespace gbgo {
int validate_config(const gb_go_dims *dims, const gb_go_params *params, const gb_go_grid *grid, std::string &msg);
void build_metric_blob(const gb_go_dims *dims, const gb_go_params *params, const gb_go_grid *g, std::vector<double> &blob);
PhysParams phys_from(const gb_go_params *pp, const gb_go_grid *g);
Metrics metrics_from_blob(const double *b, const int32_t *k1, const double *ediff1, int maxj, int maxk);
}  // namespace gbgo

using namespace gbgo;

namespace {

__global__ void k_add_step(long long *ctr, long long n) { *ctr += n; }

// ---------------------------------------------------------------------------
// mapped host memory
//
// gb_ens_host_alloc's allocations (page-locked, mapped) are registered by address range, so a
// call can tell whether a caller's array lies inside one and then let its batched kernel read or
// write it through the device address (over NVLink-C2C on Grace) instead of issuing one copy
// call per array.  The staging arena of admission is such an allocation too: the members' host
// segments are gathered there and the scatter kernel copies them into the member blocks.

struct HostRange {
    size_t bytes;
    uintptr_t dev;
};

std::mutex &host_mu()
{
    static std::mutex m;
    return m;
}

std::map<uintptr_t, HostRange> &host_ranges()
{
    static std::map<uintptr_t, HostRange> r;
    return r;
}

// The device address of [p, p + bytes) when the range lies inside one registered allocation.
void *host_mapped(const void *p, size_t bytes)
{
    if (!p) return nullptr;
    std::lock_guard<std::mutex> lk(host_mu());
    auto &r = host_ranges();
    auto it = r.upper_bound((uintptr_t)p);
    if (it == r.begin()) return nullptr;
    --it;
    const uintptr_t a = (uintptr_t)p;
    if (a < it->first || a + bytes > it->first + it->second.bytes) return nullptr;
    return (void *)(it->second.dev + (a - it->first));
}

int host_alloc(size_t bytes, void **out, void **dev)
{
    void *p = nullptr, *d = nullptr;
    cudaError_t x = cudaHostAlloc(&p, bytes, cudaHostAllocMapped | cudaHostAllocPortable);
    if (x != cudaSuccess) return x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA;
    x = cudaHostGetDevicePointer(&d, p, 0);
    if (x != cudaSuccess) {
        cudaFreeHost(p);
        return GB_GO_ECUDA;
    }
    {
        std::lock_guard<std::mutex> lk(host_mu());
        host_ranges()[(uintptr_t)p] = HostRange{bytes, (uintptr_t)d};
    }
    *out = p;
    if (dev) *dev = d;
    return GB_GO_OK;
}

int host_free(void *p)
{
    {
        std::lock_guard<std::mutex> lk(host_mu());
        auto it = host_ranges().find((uintptr_t)p);
        if (it == host_ranges().end()) return GB_GO_EINVAL;
        host_ranges().erase(it);
    }
    return cudaFreeHost(p) == cudaSuccess ? GB_GO_OK : GB_GO_ECUDA;
}

// The process's admission staging arena (grown on demand, kept): one admission call at a time
// holds `mu` from the gathering of its segments until its synchronisation.
struct StagingArena {
    std::mutex mu;
    char *host = nullptr;
    char *dev = nullptr;
    size_t bytes = 0;
};

StagingArena &staging_arena()
{
    static StagingArena a;
    return a;
}

// At least `bytes` of arena (caller holds its mutex); false when page-locked memory is short.
bool arena_reserve(StagingArena &a, size_t bytes)
{
    if (a.bytes >= bytes) return true;
    if (a.host) host_free(a.host);
    a.host = a.dev = nullptr;
    a.bytes = 0;
    const size_t want = std::max(bytes, (size_t)1 << 24);
    void *h = nullptr, *d = nullptr;
    if (host_alloc(want, &h, &d) != GB_GO_OK) return false;
    a.host = (char *)h;
    a.dev = (char *)d;
    a.bytes = want;
    return true;
}

// One copy of the batched admission: `bytes` from src (device or mapped host address) to dst;
// src NULL: zero fill.
struct CopySeg {
    const void *src;
    void *dst;
    unsigned long long bytes;
};

// Segment blockIdx.y, grid-stride over 16-byte words when the addresses and size allow,
// else over 8-byte words (the segments are arrays of doubles or 256-byte aligned blocks).
__global__ void __launch_bounds__(256) k_scatter(const CopySeg *segs)
{
    const CopySeg g = segs[blockIdx.y];
    const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x, ts = (size_t)gridDim.x * blockDim.x;
    if ((((uintptr_t)g.src | (uintptr_t)g.dst | g.bytes) & 15) == 0) {
        const size_t n = g.bytes / 16;
        const uint4 *s = (const uint4 *)g.src;
        uint4 *d = (uint4 *)g.dst;
        for (size_t w = t0; w < n; w += ts) d[w] = s ? s[w] : make_uint4(0u, 0u, 0u, 0u);
    } else {
        const size_t n = g.bytes / 8;
        const unsigned long long *s = (const unsigned long long *)g.src;
        unsigned long long *d = (unsigned long long *)g.dst;
        for (size_t w = t0; w < n; w += ts) d[w] = s ? s[w] : 0ull;
    }
}

struct Member {
    int id = -1;
    Dims d{};
    PhysParams p{};
    double dt = 0.0;
    size_t bytes = 0;
    // device
    double *buf0 = nullptr, *buf1 = nullptr, *ts_static = nullptr, *rho = nullptr, *stage = nullptr;
    float *coef = nullptr, *coefl = nullptr, *gtop = nullptr;
    double *rvol = nullptr, *mk = nullptr, *mj = nullptr, *cost = nullptr, *dsj = nullptr;
    int32_t *k1 = nullptr, *scale = nullptr, *icosd = nullptr;
    float *tref = nullptr;                // per tracer offset of the FP32 transfers
    unsigned int *gmax = nullptr;         // per tracer, scale re-targeting
    unsigned long long *diag = nullptr;   // two slots {dmax bits, limps}
    unsigned int *status = nullptr;
    int32_t *ptab = nullptr;              // patch tables
    double *vel = nullptr, *ediff1 = nullptr, *mkd = nullptr;   // iediff: u, ediff1, dza and diffmax
    float *stencil = nullptr;             // diso or iediff: the per-step top-face stencil
    double *mld = nullptr;                // imld = 1: mixed-layer depth and level per column
    int32_t *mldk = nullptr;
    double *mldketau = nullptr;           // imld = 1: wind mixing energy per column
    char *block = nullptr;                // the one device allocation every array above lies in
    double *blob = nullptr;               // metrics (build_metric_blob layout) on the device
    double *tmaxd = nullptr, *gmaxd = nullptr;   // per tracer max |T - tref| and largest forcing transfer
    unsigned long long *cd = nullptr;     // coefficient maxima (k_setup_stats_many)
    int wet_cols = 0;                     // wet columns (entries it may add to the co list)
    std::vector<int32_t> poff;            // per patch: word offset in ptab
    std::vector<double> pcost;            // per patch: cell-updates per step
    int max_slots = 1;
    MemberDesc desc{};
    long long start_step = 0;    // step index at admission (state in buf0)
    long long stop_step = 0;
    double cost_est = 0.0;
    int slot = -1;               // index in the descriptor array
};

}  // namespace

struct gb_ens {
    // gb_ens_add may run in several host threads at once: the host preparation of a member
    // runs unlocked, its allocation and registration under `mu`; `err_mu` guards last_error
    std::mutex mu, err_mu;
    int device = 0;
    cudaStream_t stream = nullptr, own_stream = nullptr;
    cudaMemPool_t pool = nullptr;
    size_t budget = 0, in_use = 0;
    std::map<int, std::unique_ptr<Member>> members;
    int next_id = 0;
    long long step = 0;                 // host mirror of the device step counter
    long long *step_ctr = nullptr;      // device
    MemberDesc *descs = nullptr;        // device, capacity cap_desc
    int cap_desc = 0;
    int4 *items = nullptr;              // device, capacity cap_items
    int cap_items = 0, nitems = 0, n_ts = 0;
    cudaStream_t s2 = nullptr;          // second stream: T-S items and the others side by side
    cudaEvent_t fork = nullptr, join = nullptr;
    int max_slots = 1;
    bool any_iso = false;               // some member has the isoneutral branch
    bool co_general = false;            // some member needs the serial adjustment
    int *stencil_list = nullptr;        // device: descriptor slots of the members with a stencil
    int cap_stencil = 0, n_stencil = 0, stencil_blocks = 1;
    int kmax = 1;                       // largest maxk of the members
    int lmax = 2;                       // largest L of the members
    int2 *colist = nullptr;             // columns listed for the exact convective adjustment
    int *cocount = nullptr;             // list and (front, back) slot counters, two each by step parity
    int cocap = 0;
    unsigned char *colog = nullptr;     // merge logs of the two-phase adjustment (cocap slots)
    int2 *comap = nullptr;              // its second-phase slots
    int mapcap = 0;
    int *work = nullptr;                // device work counters (two, by step parity)
    bool dirty = true;
    gb_ens_tuning tuning{0, 0, 0, 0, GB_ENS_PACK_MEMBERS, 0};
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    std::string last_error;
    // patch plans by (dims, tracers, tile, k1): members admitted again with a mask the ensemble
    // has seen (a serving loop's request types) skip the planner; bounded, cleared when full
    std::mutex plan_mu;
    std::unordered_map<std::string, std::shared_ptr<const PatchPlan>> plans;
};

static int efail(gb_ens *e, int code, const std::string &msg)
{
    if (e) {
        std::lock_guard<std::mutex> lk(e->err_mu);
        e->last_error = msg;
    }
    return code;
}

#define ETRY(e, call)                                                                                   \
    do {                                                                                                \
        cudaError_t _x = (call);                                                                        \
        if (_x != cudaSuccess)                                                                          \
            return efail(e, _x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA,                \
                         std::string(#call) + ": " + cudaGetErrorString(_x));                          \
    } while (0)

static bool has_stencil(const gb_go_params *p) { return p && (p->diso || (p->iediff > 0 && p->iediff < 3)); }

static size_t member_bytes(const gb_go_dims *d, const gb_go_params *p)
{
    // iediff 1/2: velocities, ediff1, dza and diffmax stay on the device
    const size_t ned = (p && p->iediff > 0 && p->iediff < 3)
                           ? (size_t)3 * (d->maxi + 1) * (d->maxj + 1) * d->maxk + (size_t)d->maxi * d->maxj * d->maxk +
                                 2 * ((size_t)d->maxk + 2)
                           : 0;
    // diso or iediff: the per-step top-face stencil
    const size_t nst = has_stencil(p) ? (size_t)kStencilWords * d->maxi * d->maxj * d->maxk : 0;
    const size_t nts = (size_t)d->maxl * (d->maxi + 2) * (d->maxj + 2) * (d->maxk + 2);
    const size_t nrho = (size_t)(d->maxi + 2) * (d->maxj + 2) * (d->maxk + 1);
    const size_t ncell = (size_t)d->maxi * d->maxj * d->maxk;
    const size_t ncol = (size_t)d->maxi * d->maxj;
    // two group-planar state buffers, uploaded copy, download stage, rho, coefficients (FP32
    // and remainders), forcing, small arrays; patch tables: at most (31 + maxk) words per column
    const size_t nplan = (size_t)fp32_planar_width(d->maxl) * (d->maxi + 2) * (d->maxj + 2) * (d->maxk + 2);
    return 2 * nplan * 8 + 2 * nts * 8 + nrho * 8 + 16 * ncell * 4 + ncol * (d->maxl + 2) * 4 + (size_t)d->maxj * d->maxk * 8 +
           ncol * 12 + (size_t)(d->maxi + 2) * (d->maxj + 2) * 4 + ncol * (31 + (size_t)d->maxk) * 4 + ned * 8 + nst * 4 + (size_t)d->maxl * 4 +
           (p && p->imld == 1 ? ncol * 28 + ((size_t)d->maxk + 1) * 16 + 1024 : 0) +
           ncol * (kCoLogSlotBytes + 8 * (size_t)fp32_co_slots(d->maxl)) + 4096;
}

extern "C" size_t gb_ens_member_bytes(const gb_go_dims *dims, const gb_go_params *params)
{
    return dims ? member_bytes(dims, params) : 0;
}

extern "C" int gb_ens_create(int device, size_t hbm_budget_bytes, gb_ens **out)
{
    if (!out) return GB_GO_EINVAL;
    *out = nullptr;
    gb_ens *e = new gb_ens();
    if (device < 0) cudaGetDevice(&e->device);
    else e->device = device;
    if (cudaSetDevice(e->device) != cudaSuccess) {
        delete e;
        return GB_GO_ECUDA;
    }
    size_t freeb = 0, total = 0;
    cudaMemGetInfo(&freeb, &total);
    e->budget = hbm_budget_bytes ? std::min(hbm_budget_bytes, freeb) : (size_t)(0.9 * freeb);
    cudaError_t x = cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking);
    e->stream = e->own_stream;
    if (x == cudaSuccess) x = cudaDeviceGetDefaultMemPool(&e->pool, e->device);
    if (x == cudaSuccess) {
        uint64_t thr = UINT64_MAX;   // keep freed blocks in the pool between admissions
        x = cudaMemPoolSetAttribute(e->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if (x == cudaSuccess) x = cudaMalloc(&e->step_ctr, sizeof(long long));
    if (x == cudaSuccess) x = cudaMemset(e->step_ctr, 0, sizeof(long long));
    if (x == cudaSuccess) x = cudaMalloc(&e->work, 4 * sizeof(int));
    if (x == cudaSuccess) x = cudaMemset(e->work, 0, 4 * sizeof(int));
    if (x == cudaSuccess) x = cudaStreamCreateWithFlags(&e->s2, cudaStreamNonBlocking);
    if (x == cudaSuccess) x = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
    if (x == cudaSuccess) x = cudaEventCreateWithFlags(&e->join, cudaEventDisableTiming);
    if (x == cudaSuccess) x = cudaMalloc(&e->cocount, 6 * sizeof(int));
    if (x == cudaSuccess) x = cudaMemset(e->cocount, 0, 6 * sizeof(int));
    if (x != cudaSuccess) {
        gb_ens_destroy(e);
        return x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA;
    }
    *out = e;
    return GB_GO_OK;
}

static void free_member(gb_ens *e, Member *m)
{
    if (m->block) cudaFreeAsync(m->block, e->stream);
    m->block = nullptr;
}

extern "C" void gb_ens_destroy(gb_ens *e)
{
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (auto &kv : e->members) free_member(e, kv.second.get());
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->graph) cudaGraphExecDestroy(e->graph);
    cudaFree(e->step_ctr);
    cudaFree(e->work);
    if (e->s2) cudaStreamDestroy(e->s2);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->join) cudaEventDestroy(e->join);
    cudaFree(e->cocount);
    cudaFree(e->colog);
    cudaFree(e->comap);
    cudaFree(e->colist);
    cudaFree(e->stencil_list);
    cudaFree(e->descs);
    cudaFree(e->items);
    if (e->own_stream) cudaStreamDestroy(e->own_stream);
    delete e;
}

extern "C" int gb_ens_set_tuning(gb_ens *e, const gb_ens_tuning *t)
{
    if (!e || !t) return GB_GO_EINVAL;
    // tile_i x tile_j: the patch rectangle asked for (0, 0: chosen per member); a rectangle
    // over the kernel limits for a member falls back to the chosen one
    if (t->tile_i < 0 || t->tile_j < 0 || t->tile_i > 4096 || t->tile_j > 4096)
        return efail(e, GB_GO_EINVAL, "tile sizes must be in 0..4096");
    if (t->ctas_per_sm < 0 || t->ctas_per_sm > 32) return efail(e, GB_GO_EINVAL, "ctas_per_sm must be in 0..32");
    if (t->packing < GB_ENS_PACK_MEMBERS || t->packing > GB_ENS_PACK_ROUND_ROBIN)
        return efail(e, GB_GO_EINVAL, "unknown packing");
    if (t->co_form < GB_ENS_CO_AUTO || t->co_form > GB_ENS_CO_TWO_PHASE) return efail(e, GB_GO_EINVAL, "unknown co_form");
    e->tuning = *t;
    e->dirty = true;
    return GB_GO_OK;
}

extern "C" int gb_ens_set_stream(gb_ens *e, void *s)
{
    if (!e) return GB_GO_EINVAL;
    e->stream = s ? (cudaStream_t)s : e->own_stream;
    if (e->graph) {
        cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
    }
    return GB_GO_OK;
}


namespace {
// Host part of a member's admission (no CUDA call): checks, patch plan, metrics, forcing
// transfers, per-tracer offsets and maxima, and the block of small arrays copied to the device
// in one piece.  Several host threads may prepare members at once.
struct Prepared {
    const gb_go_dims *dims = nullptr;
    const gb_go_params *params = nullptr;
    const gb_go_grid *grid = nullptr;
    const double *ts = nullptr, *u = nullptr;
    Dims d{};
    PhysParams p{};
    double dt = 0.0;
    size_t bytes = 0;              // budget charge (member_bytes)
    PatchPlan plan;
    std::vector<double> blob;
    Fp32Static small;              // rvol, mk, mj
    std::vector<float> gtop, tref;
    std::vector<double> tmax, gmax;
    long long wet = 0;
    int wet_cols = 0;
    // device block layout (byte offsets): the copied segment [0, copied), the zeroed segment
    // [copied, zeroed), then the arrays the device fills
    size_t o_blob, o_mj, o_rvol, o_mk, o_dsj, o_tmax, o_gmax, o_k1, o_tref, o_gtop, o_ptab, o_ediff1;
    size_t o_mlddec, o_mldketau, o_rhos, copied;
    size_t o_rho, o_cost, o_icosd, o_gmaxu, o_diag, o_status, o_cd, o_scale, o_ext, o_mld, o_mldk, zeroed;
    size_t o_buf0, o_buf1, o_static, o_stage, o_vel, o_coef, o_coefl, o_stencil, total;
    std::vector<char> host;        // the copied segment
    int rc = GB_GO_OK;
    std::string msg;
};

// eos (goldstein.f90:3048-3061) in the operation order of the device's eos_rn (the host code is
// compiled without contraction)
static double eos_host(const PhysParams &p, double t, double s, double z)
{
    const double tt = t * t;
    double r = ((p.ec[0] * t + p.ec[1] * s) + p.ec[2] * tt) + p.ec[3] * (tt * t);
    if (p.ieos != 0) r = r + (p.ec[4] * t) * z;
    return r;
}

// The patch plan of a member from the ensemble's cache, or the planner's (then cached).
int cached_plan(gb_ens *e, const Dims &d, const int32_t *k1, const gb_ens_tuning &tuning, PatchPlan &out)
{
    std::string key(sizeof(int) * 6 + sizeof(int32_t) * (size_t)d.NI * d.NJ, '\0');
    const int hdr[6] = {d.maxi, d.maxj, d.maxk, d.L, tuning.tile_i, tuning.tile_j};
    std::memcpy(&key[0], hdr, sizeof(hdr));
    std::memcpy(&key[sizeof(hdr)], k1, sizeof(int32_t) * (size_t)d.NI * d.NJ);
    {
        std::lock_guard<std::mutex> lk(e->plan_mu);
        auto it = e->plans.find(key);
        if (it != e->plans.end()) {
            out = *it->second;
            return GB_GO_OK;
        }
    }
    int rc = fp32_plan_patches(d, k1, tuning.tile_i, tuning.tile_j, out);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(e->plan_mu);
    if (e->plans.size() >= 1024) e->plans.clear();
    e->plans.emplace(std::move(key), std::make_shared<const PatchPlan>(out));
    return GB_GO_OK;
}

int prepare_member(gb_ens *e, const gb_ens_tuning &tuning, const gb_go_dims *dims, const gb_go_params *params,
                   const gb_go_grid *grid, const double *ts, const double *u, Prepared &pm)
{
    pm.dims = dims;
    pm.params = params;
    pm.grid = grid;
    pm.ts = ts;
    pm.u = u;
    if (!dims || !params || !grid || !ts || !u) {
        pm.msg = "NULL argument";
        return pm.rc = GB_GO_EINVAL;
    }
    int rc = validate_config(dims, params, grid, pm.msg);
    if (rc) return pm.rc = rc;
    if (dims->maxl > kFp32MaxL) {
        pm.msg = "ensemble members carry at most 32 tracers";
        return pm.rc = GB_GO_ERANGE;
    }
    for (int k = 1; k < dims->maxk; ++k)
        if (grid->dt[k] != grid->dt[0]) {
            pm.msg = "ensemble members need one dt for all levels";
            return pm.rc = GB_GO_EUNSUPPORTED;
        }
    if (dims->maxk > kMaxK) {
        pm.msg = "ensemble members have at most 64 levels";
        return pm.rc = GB_GO_ERANGE;
    }
    pm.d = Dims{dims->maxi, dims->maxj, dims->maxk, dims->maxl, dims->maxi + 2, dims->maxj + 2};
    pm.p = phys_from(params, grid);
    pm.dt = grid->dt[0];
    pm.bytes = member_bytes(dims, params);
    if (cached_plan(e, pm.d, grid->k1, tuning, pm.plan) != GB_GO_OK) {
        pm.msg = "no patch shape fits the FP32-flux kernel limits";
        return pm.rc = GB_GO_ERANGE;
    }
    build_metric_blob(dims, params, grid, pm.blob);
    fp32_build_small(pm.d, pm.p, pm.blob, pm.small);
    const int L = dims->maxl, NI = pm.d.NI, NJ = pm.d.NJ, maxi = dims->maxi, maxj = dims->maxj, maxk = dims->maxk;
    const size_t ntop = (size_t)L * NI * NJ;
    fp32_gtop(pm.d, pm.p, pm.blob, ts + ntop * (maxk + 1), pm.gtop);
    // the offsets and maxima of the tracers are found on the device (the set-up's extrema
    // kernel reads the uploaded state); the forcing's maxima here
    pm.tref.assign(L, 0.0f);
    pm.tmax.assign(L, 0.0);
    pm.gmax.assign(L, 0.0);
    for (size_t c = 0; c < (size_t)dims->maxi * dims->maxj; ++c)
        for (int l = 0; l < L; ++l) pm.gmax[l] = std::max(pm.gmax[l], (double)std::fabs(pm.gtop[c * (L + 2) + l]));
    for (int j = 1; j <= maxj; ++j)
        for (int i = 1; i <= maxi; ++i) {
            const int k1 = grid->k1[i + (size_t)NI * j];
            if (k1 <= maxk) {
                pm.wet += maxk - k1 + 1;
                pm.wet_cols += 1;
            }
        }
    // layout of the member's device block (256-byte aligned arrays)
    const bool ediff = params->iediff > 0 && params->iediff < 3;
    const size_t nts = ntop * (maxk + 2), nrho = (size_t)NI * NJ * (maxk + 1), ncol = (size_t)maxi * maxj;
    const size_t ncell = ncol * maxk, nplan = fp32_planar_size(pm.d);
    const size_t nu = (size_t)3 * (maxi + 1) * (maxj + 1) * maxk;
    const size_t ned = ediff ? (size_t)maxi * maxj * (maxk - 1) : 0;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = (off + bytes + 255) & ~(size_t)255;
        return o;
    };
    pm.o_blob = take(pm.blob.size() * 8);
    pm.o_mj = take(pm.small.mj.size() * 8);
    pm.o_rvol = take(pm.small.rvol.size() * 8);
    pm.o_mk = take(pm.small.mk.size() * 8);
    pm.o_dsj = take((size_t)(maxj + 2) * 8);
    pm.o_tmax = take((size_t)L * 8);
    pm.o_gmax = take((size_t)L * 8);
    pm.o_k1 = take((size_t)NI * NJ * 4);
    pm.o_tref = take((size_t)L * 4);
    pm.o_gtop = take(pm.gtop.size() * 4);
    pm.o_ptab = take(std::max<size_t>(4, pm.plan.words.size()) * 4);
    pm.o_ediff1 = take(std::max<size_t>(1, ned) * 8);
    const bool mldon = params->imld == 1;
    pm.o_mlddec = take(mldon ? (size_t)2 * (maxk + 1) * 8 : 0);
    pm.o_mldketau = take(mldon ? ncol * 8 : 0);
    pm.o_rhos = take(mldon ? ncol * 8 : 0);
    pm.copied = off;
    pm.o_rho = take(nrho * 8);
    pm.o_cost = take(ncol * 8);
    pm.o_icosd = take(ncol * 4);
    pm.o_gmaxu = take((size_t)L * 4);
    pm.o_diag = take(4 * 8);
    pm.o_status = take(4);
    pm.o_cd = take(2 * 8);
    pm.o_scale = take((size_t)L * 4);
    pm.o_ext = take((size_t)2 * L * 8);
    pm.o_mld = take(mldon ? ncol * 8 : 0);
    pm.o_mldk = take(mldon ? ncol * 4 : 0);
    pm.zeroed = off;
    pm.o_buf0 = take(nplan * 8);
    pm.o_buf1 = take(nplan * 8);
    pm.o_static = take(nts * 8);
    pm.o_stage = take(nts * 8);
    pm.o_vel = take(nu * 8);
    pm.o_coef = take(8 * ncell * 4);
    pm.o_coefl = take(8 * ncell * 4);
    pm.o_stencil = take(has_stencil(params) ? (size_t)kStencilWords * ncell * 4 : 0);
    pm.total = off;
    pm.host.assign(pm.copied, 0);
    char *h = pm.host.data();
    auto put = [&](size_t o, const void *src, size_t bytes) {
        if (bytes) std::memcpy(h + o, src, bytes);
    };
    put(pm.o_blob, pm.blob.data(), pm.blob.size() * 8);
    put(pm.o_mj, pm.small.mj.data(), pm.small.mj.size() * 8);
    put(pm.o_rvol, pm.small.rvol.data(), pm.small.rvol.size() * 8);
    put(pm.o_mk, pm.small.mk.data(), pm.small.mk.size() * 8);
    put(pm.o_dsj, pm.blob.data() + 6 * (maxj + 2), (size_t)(maxj + 2) * 8);   // ds(0:maxj+1)
    put(pm.o_tmax, pm.tmax.data(), (size_t)L * 8);
    put(pm.o_gmax, pm.gmax.data(), (size_t)L * 8);
    put(pm.o_k1, grid->k1, (size_t)NI * NJ * 4);
    put(pm.o_tref, pm.tref.data(), (size_t)L * 4);
    put(pm.o_gtop, pm.gtop.data(), pm.gtop.size() * 4);
    put(pm.o_ptab, pm.plan.words.data(), pm.plan.words.size() * 4);
    if (ned) put(pm.o_ediff1, grid->ediff1, ned * 8);
    if (mldon) {
        // mlddec, mlddecd Fortran-indexed [1..maxk]; the wind energy; rho(maxk) of the initial state
        double *dec = reinterpret_cast<double *>(h + pm.o_mlddec);
        for (int k = 1; k <= maxk; ++k) {
            dec[k] = grid->mlddec[k - 1];
            dec[maxk + 1 + k] = grid->mlddecd[k - 1];
        }
        put(pm.o_mldketau, grid->mldketau, ncol * 8);
        double *rhos = reinterpret_cast<double *>(h + pm.o_rhos);
        const double zro = pm.small.mk[3 * (size_t)(maxk + 2) + maxk];
        for (int j = 1; j <= maxj; ++j)
            for (int i = 1; i <= maxi; ++i) {
                const size_t c = (size_t)L * ((size_t)i + (size_t)NI * ((size_t)j + (size_t)NJ * maxk));
                rhos[(i - 1) + (size_t)maxi * (j - 1)] =
                    grid->k1[i + (size_t)NI * j] <= maxk ? eos_host(pm.p, ts[c], ts[c + 1], zro) : 0.0;
            }
    }
    return GB_GO_OK;
}
}  // namespace

// Device part of a member's admission (caller holds e->mu): one pool allocation, the copied
// segment, the zeroed segment, ts and u from the caller's arrays; the member's item of the
// batched device set-up; then its descriptor and registration.  Queued on the ensemble's
// stream: the caller synchronises before the caller's arrays or pm.host may go.  With `staged`
// (the device address of the member's copied segment in the staging arena) the segment copy,
// the zero fill and the copies of mapped ts and u become entries of `segs` for the batched
// scatter kernel; the rest are copy calls.
static int commit_member(gb_ens *e, Prepared &pm, int32_t *member_id, SetupItem *item, const char *staged,
                         const char *ts_dev, const char *u_dev, std::vector<CopySeg> &segs)
{
    if (e->in_use + pm.bytes > e->budget) return efail(e, GB_GO_ENOMEM, "member does not fit in the HBM budget");
    cudaStream_t s = e->stream;
    const gb_go_dims *dims = pm.dims;
    const gb_go_params *params = pm.params;
    const int L = dims->maxl, maxk = dims->maxk;
    const size_t nts = (size_t)L * pm.d.NI * pm.d.NJ * (maxk + 2);
    const size_t nu = (size_t)3 * (dims->maxi + 1) * (dims->maxj + 1) * maxk;
    auto m = std::make_unique<Member>();
    m->d = pm.d;
    m->p = pm.p;
    m->dt = pm.dt;
    m->bytes = pm.bytes;
    m->poff = pm.plan.offset;
    m->pcost = pm.plan.cost;
    m->max_slots = pm.plan.max_slots;
    m->wet_cols = pm.wet_cols;
    cudaError_t x = cudaMallocFromPoolAsync((void **)&m->block, pm.total, e->pool, s);
    if (x != cudaSuccess) return efail(e, x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA, cudaGetErrorString(x));
    char *b = m->block;
    m->blob = (double *)(b + pm.o_blob);
    m->mj = (double *)(b + pm.o_mj);
    m->rvol = (double *)(b + pm.o_rvol);
    m->mk = (double *)(b + pm.o_mk);
    m->dsj = (double *)(b + pm.o_dsj);
    m->tmaxd = (double *)(b + pm.o_tmax);
    m->gmaxd = (double *)(b + pm.o_gmax);
    m->k1 = (int32_t *)(b + pm.o_k1);
    m->tref = (float *)(b + pm.o_tref);
    m->gtop = (float *)(b + pm.o_gtop);
    m->ptab = (int32_t *)(b + pm.o_ptab);
    const bool ediff = params->iediff > 0 && params->iediff < 3;
    m->ediff1 = ediff ? (double *)(b + pm.o_ediff1) : nullptr;
    m->rho = (double *)(b + pm.o_rho);
    m->cost = (double *)(b + pm.o_cost);
    m->icosd = (int32_t *)(b + pm.o_icosd);
    m->gmax = (unsigned int *)(b + pm.o_gmaxu);
    m->diag = (unsigned long long *)(b + pm.o_diag);
    m->status = (unsigned int *)(b + pm.o_status);
    m->cd = (unsigned long long *)(b + pm.o_cd);
    m->scale = (int32_t *)(b + pm.o_scale);
    m->buf0 = (double *)(b + pm.o_buf0);
    m->buf1 = (double *)(b + pm.o_buf1);
    m->ts_static = (double *)(b + pm.o_static);
    m->stage = (double *)(b + pm.o_stage);
    m->vel = (double *)(b + pm.o_vel);
    m->coef = (float *)(b + pm.o_coef);
    m->coefl = (float *)(b + pm.o_coefl);
    m->stencil = has_stencil(params) ? (float *)(b + pm.o_stencil) : nullptr;
    const bool mldon = params->imld == 1;
    m->mld = mldon ? (double *)(b + pm.o_mld) : nullptr;
    m->mldk = mldon ? (int32_t *)(b + pm.o_mldk) : nullptr;
    m->mldketau = mldon ? (double *)(b + pm.o_mldketau) : nullptr;
    const int nj = dims->maxj + 2, nk = maxk + 2;
    m->mkd = ediff ? m->blob + 8 * nj + nk : nullptr;   // dza, then (7 k-arrays on) diffmax
    if (staged) {
        segs.push_back(CopySeg{staged, b, pm.copied});
        segs.push_back(CopySeg{nullptr, b + pm.copied, pm.zeroed - pm.copied});
    } else {
        x = cudaMemcpyAsync(b, pm.host.data(), pm.copied, cudaMemcpyHostToDevice, s);
        if (x == cudaSuccess) x = cudaMemsetAsync(b + pm.copied, 0, pm.zeroed - pm.copied, s);
    }
    // ts and u already on the device (ts_dev, u_dev: staged at the start of the call) or in
    // mapped host memory (8-byte aligned) are copied by the scatter kernel
    // (the segment list lives in the staging arena: without it, copy calls)
    const void *tsd = !staged ? nullptr : ts_dev ? (const void *)ts_dev
                                                 : (((uintptr_t)pm.ts & 7) == 0 ? host_mapped(pm.ts, nts * 8) : nullptr);
    const void *ud = !staged ? nullptr : u_dev ? (const void *)u_dev
                                               : (((uintptr_t)pm.u & 7) == 0 ? host_mapped(pm.u, nu * 8) : nullptr);
    if (tsd) segs.push_back(CopySeg{tsd, m->ts_static, nts * 8});
    else if (x == cudaSuccess) x = cudaMemcpyAsync(m->ts_static, pm.ts, nts * 8, cudaMemcpyHostToDevice, s);
    if (ud) segs.push_back(CopySeg{ud, m->vel, nu * 8});
    else if (x == cudaSuccess) x = cudaMemcpyAsync(m->vel, pm.u, nu * 8, cudaMemcpyHostToDevice, s);
    if (x != cudaSuccess) {
        free_member(e, m.get());
        return efail(e, x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA, cudaGetErrorString(x));
    }
    // the device set-up (state buffers, coefficients, scales) runs batched after the copies
    item->d = m->d;
    item->p = m->p;
    item->m = metrics_from_blob(m->blob, m->k1, m->ediff1, dims->maxj, maxk);
    item->u = m->vel;
    item->ts_static = m->ts_static;
    item->buf0 = m->buf0;
    item->buf1 = m->buf1;
    item->coef = m->coef;
    item->coefl = m->coefl;
    item->cd = m->cd;
    item->tmax = m->tmaxd;
    item->gmax = m->gmaxd;
    item->tref = m->tref;
    item->ext = (unsigned long long *)(b + pm.o_ext);
    item->scale = m->scale;
    MemberDesc &md = m->desc;
    md.maxi = dims->maxi; md.maxj = dims->maxj; md.maxk = maxk; md.L = L;
    md.NI = m->d.NI; md.NJ = m->d.NJ; md.diso = m->p.diso; md.ieos = m->p.ieos; md.iconv = m->p.iconv;
    md.iediff = m->p.iediff; md.ediffpow2i = m->p.ediffpow2i;
    md.diff2 = m->p.diff2; md.ediff0 = m->p.ediff0; md.ediffpow2 = m->p.ediffpow2;
    md.u = m->vel; md.ediff1 = m->ediff1;
    md.dza = m->mkd; md.diffmax = m->mkd ? m->blob + 8 * nj + 8 * nk : nullptr;
    md.stencil = m->stencil;
    md.dt = m->dt; md.dphi = m->p.dphi; md.rdphi = m->p.rdphi; md.diff1 = m->p.diff1;
    for (int n = 0; n < 5; ++n) md.ec[n] = m->p.ec[n];
    md.dsc = m->p.dsc;
    md.buf[0] = m->buf0; md.buf[1] = m->buf1;
    md.ts_static = m->ts_static; md.coef = m->coef; md.coefl = m->coefl; md.rvol = m->rvol; md.gtop = m->gtop; md.k1 = m->k1;
    md.scale = m->scale; md.tref = m->tref; md.mk = m->mk; md.mj = m->mj; md.cost = m->cost; md.icosd = m->icosd;
    md.diag = m->diag; md.status = m->status; md.gmax = m->gmax; md.ptab = m->ptab;
    md.imld = mldon ? 1 : 0;
    md.mldpebuoycoeff = m->p.mldpebuoycoeff;
    md.mlddec = mldon ? (const double *)(b + pm.o_mlddec) : nullptr;
    md.mlddecd = mldon ? (const double *)(b + pm.o_mlddec) + (maxk + 1) : nullptr;
    md.mldketau = m->mldketau;
    md.mld = m->mld;
    md.mldk = m->mldk;
    md.rhos = mldon ? (double *)(b + pm.o_rhos) : nullptr;
    m->start_step = e->step;
    m->stop_step = (long long)1 << 62;
    md.parity = (int)(e->step & 1);     // (step + parity) & 1 == 0 at admission
    md.stop_step = m->stop_step;
    md.origin = e->step;
    m->cost_est = (double)pm.wet * (L + 4) * (params->diso ? 2.0 : 1.0);
    m->id = e->next_id++;
    *member_id = m->id;
    e->in_use += pm.bytes;
    e->members[m->id] = std::move(m);
    e->dirty = true;
    return GB_GO_OK;
}

extern "C" int gb_ens_add(gb_ens *e, const gb_go_dims *dims, const gb_go_params *params, const gb_go_grid *grid,
                          const double *ts, const double *u, int32_t *member_id)
{
    if (!e || !ts || !u || !member_id) return GB_GO_EINVAL;
    return gb_ens_add_many(e, 1, dims, params, grid, &ts, &u, member_id);
}

extern "C" int gb_ens_add_many(gb_ens *e, int32_t n, const gb_go_dims *dims, const gb_go_params *params,
                               const gb_go_grid *grids, const double *const *ts, const double *const *u, int32_t *ids)
{
    gbgo::TraceRange tr_("ens_add_many");
    if (!e || n < 0 || (n > 0 && (!dims || !params || !grids || !ts || !u || !ids))) return GB_GO_EINVAL;
    if (n == 0) return GB_GO_OK;
    ETRY(e, cudaSetDevice(e->device));
    // ts and u in mapped host memory start their transfer now, into one device staging block,
    // so that it overlaps the host preparation; the members then take them with device copies
    std::vector<const char *> ts_pre(n, nullptr), u_pre(n, nullptr);
    char *dstage = nullptr;
    {
        std::vector<CopySeg> pre;
        std::vector<size_t> tso(n, SIZE_MAX), uo(n, SIZE_MAX);
        size_t db = 0;
        for (int q = 0; q < n; ++q) {
            const gb_go_dims &d = dims[q];
            // sizes of plausible dimensions only (the preparation validates them)
            if (d.maxi < 1 || d.maxj < 1 || d.maxk < 1 || d.maxl < 1 || d.maxi > 65536 || d.maxj > 65536 ||
                d.maxk > GB_GO_MAX_K || d.maxl > GB_GO_MAX_L)
                continue;
            const size_t nts = (size_t)d.maxl * (d.maxi + 2) * (d.maxj + 2) * (d.maxk + 2);
            const size_t nu = (size_t)3 * (d.maxi + 1) * (d.maxj + 1) * d.maxk;
            const void *th = ((uintptr_t)ts[q] & 7) == 0 ? host_mapped(ts[q], nts * 8) : nullptr;
            const void *uh = ((uintptr_t)u[q] & 7) == 0 ? host_mapped(u[q], nu * 8) : nullptr;
            if (th) {
                tso[q] = db;
                pre.push_back(CopySeg{th, (void *)(uintptr_t)db, nts * 8});
                db += (nts * 8 + 255) & ~(size_t)255;
            }
            if (uh) {
                uo[q] = db;
                pre.push_back(CopySeg{uh, (void *)(uintptr_t)db, nu * 8});
                db += (nu * 8 + 255) & ~(size_t)255;
            }
        }
        CopySeg *dl = nullptr;
        if (!pre.empty() && cudaMallocFromPoolAsync((void **)&dstage, db, e->pool, e->stream) == cudaSuccess &&
            cudaMallocAsync((void **)&dl, sizeof(CopySeg) * pre.size(), e->stream) == cudaSuccess) {
            size_t longest = 16;
            for (CopySeg &g : pre) {
                g.dst = dstage + (uintptr_t)g.dst;
                longest = std::max<size_t>(longest, g.bytes);
            }
            cudaError_t x = cudaMemcpyAsync(dl, pre.data(), sizeof(CopySeg) * pre.size(), cudaMemcpyHostToDevice, e->stream);
            const int bx = (int)std::min<size_t>((longest / 16 + 255) / 256, 64);
            for (size_t g0 = 0; x == cudaSuccess && g0 < pre.size(); g0 += 65535) {
                const int ng = (int)std::min<size_t>(pre.size() - g0, 65535);
                k_scatter<<<dim3(bx, ng), 256, 0, e->stream>>>(dl + g0);
                count_launches(1);
                x = cudaGetLastError();
            }
            if (x == cudaSuccess)
                for (int q = 0; q < n; ++q) {
                    if (tso[q] != SIZE_MAX) ts_pre[q] = dstage + tso[q];
                    if (uo[q] != SIZE_MAX) u_pre[q] = dstage + uo[q];
                }
        }
        if (dl) cudaFreeAsync(dl, e->stream);
        cudaGetLastError();
    }
    // the staging block goes after the member copies; an early return waits for the transfer
    // (it reads the caller's arrays)
    auto drop_stage = [&](bool wait) {
        if (dstage) cudaFreeAsync(dstage, e->stream);
        dstage = nullptr;
        if (wait) cudaStreamSynchronize(e->stream);
    };
    // host preparation on up to 16 threads
    std::vector<Prepared> pm(n);
    const gb_ens_tuning tuning = e->tuning;
    std::atomic<int> next{0};
    auto work = [&]() {
        for (int q = next++; q < n; q = next++) prepare_member(e, tuning, dims + q, params + q, grids + q, ts[q], u[q], pm[q]);
    };
    const int nt = std::max(1, std::min<int>(std::min<int>(n, 16), (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(work);
    work();
    for (auto &t : th) t.join();
    for (int q = 0; q < n; ++q)
        if (pm[q].rc) {
            drop_stage(true);
            return efail(e, pm[q].rc, pm[q].msg);
        }
    // the members' copied segments gathered in the staging arena (threads), then one scatter
    // kernel; without arena memory, one copy call per segment
    std::vector<size_t> soff(n);
    size_t sbytes = 0;
    for (int q = 0; q < n; ++q) {
        soff[q] = sbytes;
        sbytes += (pm[q].copied + 255) & ~(size_t)255;
    }
    const size_t seg_at = sbytes;
    sbytes += sizeof(CopySeg) * 4 * (size_t)n;
    StagingArena &arena = staging_arena();
    std::unique_lock<std::mutex> alk(arena.mu);
    const bool staged = arena_reserve(arena, sbytes);
    if (staged) {
        next = 0;
        auto gather = [&]() {
            for (int q = next++; q < n; q = next++) std::memcpy(arena.host + soff[q], pm[q].host.data(), pm[q].copied);
        };
        th.clear();
        for (int t = 1; t < nt; ++t) th.emplace_back(gather);
        gather();
        for (auto &t : th) t.join();
    }
    // the device part, one member at a time, the batched set-up, then one synchronisation
    std::lock_guard<std::mutex> lk(e->mu);
    int q = 0, rc = GB_GO_OK;
    std::vector<SetupItem> items(n);
    std::vector<CopySeg> segs;
    size_t max_elems = 1, max_cells = 1;
    for (; q < n; ++q) {
        if ((rc = commit_member(e, pm[q], ids + q, &items[q], staged ? arena.dev + soff[q] : nullptr, ts_pre[q], u_pre[q],
                                segs)))
            break;
        const Dims &d = items[q].d;
        max_elems = std::max(max_elems, (size_t)d.NI * d.NJ * (d.maxk + 2) * d.L);
        max_cells = std::max(max_cells, (size_t)d.maxi * d.maxj * d.maxk);
    }
    if (!rc && !segs.empty()) {
        // the segment list in the arena, read by the kernel through its device address
        std::memcpy(arena.host + seg_at, segs.data(), segs.size() * sizeof(CopySeg));
        size_t longest = 16;
        for (const CopySeg &g : segs) longest = std::max<size_t>(longest, g.bytes);
        const int bx = (int)std::min<size_t>((longest / 16 + 255) / 256, 64);
        const CopySeg *dsegs = (const CopySeg *)(arena.dev + seg_at);
        for (size_t g0 = 0; g0 < segs.size(); g0 += 65535) {
            const int ng = (int)std::min<size_t>(segs.size() - g0, 65535);
            k_scatter<<<dim3(bx, ng), 256, 0, e->stream>>>(dsegs + g0);
            count_launches(1);
        }
        const cudaError_t x = cudaGetLastError();
        if (x != cudaSuccess) {
            rc = efail(e, GB_GO_ECUDA, cudaGetErrorString(x));
            q = n;
        }
    }
    if (!rc) {
        SetupItem *dit = nullptr;
        cudaError_t x = cudaMallocAsync((void **)&dit, sizeof(SetupItem) * n, e->stream);
        if (x == cudaSuccess) x = cudaMemcpyAsync(dit, items.data(), sizeof(SetupItem) * n, cudaMemcpyHostToDevice, e->stream);
        if (x == cudaSuccess && fp32_setup_many(dit, n, max_elems, max_cells, e->stream)) x = cudaErrorLaunchFailure;
        if (dit) cudaFreeAsync(dit, e->stream);
        if (x != cudaSuccess) {
            rc = efail(e, x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA, cudaGetErrorString(x));
            q = n;
        }
    }
    drop_stage(false);
    if (rc) {
        // all or nothing: the members of this call that were committed leave again
        for (int r = 0; r < q; ++r) {
            auto it = e->members.find(ids[r]);
            if (it == e->members.end()) continue;
            free_member(e, it->second.get());
            e->in_use -= it->second->bytes;
            e->members.erase(it);
        }
        const std::string msg = e->last_error;
        cudaStreamSynchronize(e->stream);
        return efail(e, rc, msg);
    }
    ETRY(e, cudaStreamSynchronize(e->stream));
    return GB_GO_OK;
}

extern "C" int gb_ens_host_alloc(size_t bytes, void **out)
{
    if (!out || bytes == 0) return GB_GO_EINVAL;
    *out = nullptr;
    return host_alloc(bytes, out, nullptr);
}

extern "C" int gb_ens_host_free(void *p)
{
    if (!p) return GB_GO_EINVAL;
    return host_free(p);
}

extern "C" int gb_ens_remove(gb_ens *e, int32_t id)
{
    if (!e) return GB_GO_EINVAL;
    auto it = e->members.find(id);
    if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
    ETRY(e, cudaSetDevice(e->device));
    free_member(e, it->second.get());
    e->in_use -= it->second->bytes;
    e->members.erase(it);
    e->dirty = true;
    return GB_GO_OK;
}

// Rebuild the descriptor array and the work list after membership changes.
static int rebuild(gb_ens *e)
{
    cudaStream_t s = e->stream;
    const int nm = (int)e->members.size();
    if (nm > e->cap_desc) {
        int cap = std::max(16, 2 * nm);
        if (e->descs) cudaFreeAsync(e->descs, s);
        ETRY(e, cudaMallocAsync(&e->descs, (size_t)cap * sizeof(MemberDesc), s));
        e->cap_desc = cap;
    }
    std::vector<MemberDesc> descs;
    // members in decreasing order of work (longest first); a member's patches stay
    // together so the ring columns one patch reads are in L2 from its neighbours
    std::vector<std::pair<double, Member *>> order;
    int max_slots = 1;
    bool any_iso = false, co_general = false;
    int kmax = 1, lmax = 2;
    int slot = 0;
    std::vector<int> slist;   // members with a stencil
    int sblocks = 1;
    for (auto &kv : e->members) {
        Member *m = kv.second.get();
        // keep each member's status word and diag slots across rebuilds by
        // assigning slots in id order (stable while members only leave)
        m->slot = slot;
        MemberDesc md = m->desc;
        md.stop_step = m->stop_step;
        md.status_idx = slot;
        descs.push_back(md);
        double c = 0.0;
        for (double v : m->pcost) c += v;
        order.push_back({c, m});
        max_slots = std::max(max_slots, m->max_slots);
        any_iso = any_iso || m->desc.diso || m->desc.iediff;
        if (m->stencil) {
            slist.push_back(slot);
            sblocks = std::max(sblocks, fp32_stencil_blocks((size_t)m->d.maxi * m->d.maxj * m->d.maxk));
        }
        co_general = co_general || !fp32_co_fast(m->desc.iconv, m->desc.ieos, m->desc.imld, m->d.maxk);
        kmax = std::max(kmax, m->d.maxk);
        lmax = std::max(lmax, m->d.L);
        ++slot;
    }
    std::stable_sort(order.begin(), order.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
    // transfer items (member, patch, group), T-S items first, in the tuning's packing order.
    // GB_ENS_PACK_MEMBERS: a patch's groups and a member's patches next to each other (items
    // taken together share the coefficients and ring columns in L2).  The co column list holds
    // at most every wet column of the batch.
    std::vector<int4> it;
    auto add_items = [&](bool ts) {
        struct Cand {
            double cost;
            size_t rank;
            int4 item;
        };
        std::vector<Cand> c;
        size_t rank = 0;
        for (auto &o : order) {
            const Member *m = o.second;
            const int ng = fp32_group_count(m->d.L);
            for (size_t n = 0; n < m->poff.size(); ++n)
                for (int g = ts ? 0 : 1; g < (ts ? 1 : ng); ++g) {
                    int g0, gl;
                    fp32_group(m->d.L, g, &g0, &gl);
                    // cost: the patch's estimate times the group's share of the tracers
                    const double w = m->pcost[n] * (double)gl / (double)m->d.L;
                    // round robin: patch index first, then the member order
                    const size_t rr = (n << 20) + (rank << 5) + (size_t)g;
                    c.push_back(Cand{w, e->tuning.packing == GB_ENS_PACK_ROUND_ROBIN ? rr : c.size(),
                                     make_int4(m->slot, m->poff[n], g, 0)});
                }
            ++rank;
        }
        if (e->tuning.packing == GB_ENS_PACK_ITEMS)
            std::stable_sort(c.begin(), c.end(), [](const Cand &a, const Cand &b) { return a.cost > b.cost; });
        else if (e->tuning.packing == GB_ENS_PACK_ROUND_ROBIN)
            std::stable_sort(c.begin(), c.end(), [](const Cand &a, const Cand &b) { return a.rank < b.rank; });
        for (const Cand &x : c) it.push_back(x.item);
    };
    add_items(true);
    const int n_ts = (int)it.size();
    add_items(false);
    int cocap = 0;
    for (auto &o : order) cocap += o.second->wet_cols;
    if ((int)it.size() > e->cap_items) {
        int cap = std::max(256, (int)(2 * it.size()));
        if (e->items) cudaFreeAsync(e->items, s);
        ETRY(e, cudaMallocAsync(&e->items, (size_t)cap * sizeof(int4), s));
        e->cap_items = cap;
    }
    if ((int)slist.size() > e->cap_stencil) {
        int cap = std::max(64, (int)(2 * slist.size()));
        if (e->stencil_list) cudaFreeAsync(e->stencil_list, s);
        e->stencil_list = nullptr;
        ETRY(e, cudaMallocAsync(&e->stencil_list, (size_t)cap * sizeof(int), s));
        e->cap_stencil = cap;
    }
    if (!slist.empty())
        ETRY(e, cudaMemcpyAsync(e->stencil_list, slist.data(), slist.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    if (!descs.empty()) ETRY(e, cudaMemcpyAsync(e->descs, descs.data(), descs.size() * sizeof(MemberDesc), cudaMemcpyHostToDevice, s));
    if (!it.empty()) ETRY(e, cudaMemcpyAsync(e->items, it.data(), it.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
    ETRY(e, cudaStreamSynchronize(s));
    e->nitems = (int)it.size();
    e->n_ts = n_ts;
    if (cocap > e->cocap) {
        if (e->colist) cudaFreeAsync(e->colist, s);
        if (e->colog) cudaFreeAsync(e->colog, s);
        e->colist = nullptr;
        e->colog = nullptr;
        ETRY(e, cudaMallocAsync(&e->colist, (size_t)cocap * sizeof(int2), s));
        ETRY(e, cudaMallocAsync(&e->colog, (size_t)cocap * kCoLogSlotBytes, s));
        e->cocap = cocap;
    }
    // second-phase slots: at most L - 2 per listed column
    if ((size_t)e->cocap * fp32_co_slots(lmax) > (size_t)e->mapcap) {
        if (e->comap) cudaFreeAsync(e->comap, s);
        e->comap = nullptr;
        const int mapcap = e->cocap * fp32_co_slots(lmax);
        ETRY(e, cudaMallocAsync(&e->comap, (size_t)mapcap * sizeof(int2), s));
        e->mapcap = mapcap;
    }
    e->max_slots = max_slots;
    e->any_iso = any_iso;
    e->co_general = co_general;
    e->n_stencil = (int)slist.size();
    e->stencil_blocks = sblocks;
    e->kmax = kmax;
    e->lmax = lmax;
    e->dirty = false;
    if (e->graph) {
        cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
    }
    return GB_GO_OK;
}

static Fp32Batch batch_of(gb_ens *e)
{
    Fp32Batch b;
    b.descs = e->descs;
    b.items = e->items;
    b.n_ts = e->n_ts;
    b.n_bgc = e->nitems - e->n_ts;
    b.max_slots = e->max_slots;
    b.kmax = e->kmax;
    b.lmax = e->lmax;
    b.work = e->work;
    b.colist = e->colist;
    b.cocount = e->cocount;
    b.cocap = e->cocap;
    b.colog = e->colog;
    b.comap = e->comap;
    b.mapcap = e->mapcap;
    b.iso = e->any_iso;
    b.co_general = e->co_general;
    b.stencil_list = e->stencil_list;
    b.n_stencil = e->n_stencil;
    b.stencil_blocks = e->stencil_blocks;
    b.ctas_per_sm = e->tuning.ctas_per_sm;
    b.co_form = e->tuning.co_form;
    return b;
}

// kernels started by launch_steps(e, nsteps)
static uint64_t launches_of(gb_ens *e, int nsteps)
{
    return (uint64_t)nsteps * (fp32_launches_per_step(batch_of(e)) + 1) + 1;
}

static int launch_steps(gb_ens *e, int nsteps)
{
    cudaStream_t s = e->stream;
    const Fp32Batch b = batch_of(e);
    for (int n = 0; n < nsteps; ++n) {
        int r = fp32_launch(b, e->step_ctr, n, s, e->s2, e->fork, e->join);
        if (!r) r = fp32_rescale(e->descs, (int)e->members.size(), s);
        if (r) return efail(e, r, "fp32 batched launch failed");
    }
    k_add_step<<<1, 1, 0, s>>>(e->step_ctr, nsteps);
    return cudaGetLastError() == cudaSuccess ? GB_GO_OK : efail(e, GB_GO_ECUDA, "launch failed");
}

extern "C" int gb_ens_step(gb_ens *e, int32_t nsteps)
{
    gbgo::TraceRange tr_("ens_step");
    if (!e || nsteps < 0) return GB_GO_EINVAL;
    ETRY(e, cudaSetDevice(e->device));
    if (e->dirty) {
        int r = rebuild(e);
        if (r) return r;
    }
    if (nsteps == 0 || e->members.empty() || e->nitems == 0) {
        e->step += nsteps;
        if (nsteps) {
            k_add_step<<<1, 1, 0, e->stream>>>(e->step_ctr, nsteps);
            count_launches(1);
        }
        return GB_GO_OK;
    }
    if (e->tuning.use_graph) {
        if (!e->graph || e->graph_steps != nsteps) {
            if (e->graph) cudaGraphExecDestroy(e->graph);
            e->graph = nullptr;
            cudaGraph_t g;
            ETRY(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
            int r = launch_steps(e, nsteps);
            cudaError_t x = cudaStreamEndCapture(e->stream, &g);
            if (r) return r;
            if (x != cudaSuccess) return efail(e, GB_GO_ECUDA, "graph capture failed");
            x = cudaGraphInstantiate(&e->graph, g, 0);
            cudaGraphDestroy(g);
            if (x != cudaSuccess) return efail(e, GB_GO_ECUDA, "graph instantiate failed");
            e->graph_steps = nsteps;
        }
        ETRY(e, cudaGraphLaunch(e->graph, e->stream));
    } else {
        int r = launch_steps(e, nsteps);
        if (r) return r;
    }
    count_launches(launches_of(e, nsteps));
    e->step += nsteps;
    return GB_GO_OK;
}

extern "C" int gb_ens_set_remaining(gb_ens *e, int32_t id, int64_t steps)
{
    if (!e || steps < 0) return GB_GO_EINVAL;
    auto it = e->members.find(id);
    if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
    Member *m = it->second.get();
    // buffer holding the current state: after its last step
    const long long done_at = std::min(e->step, m->stop_step);
    const int curbuf = (int)((done_at + m->desc.parity) & 1);
    m->desc.parity = (int)((curbuf - (e->step & 1) + 2) & 1);
    // keep the member's own step count running across a pause
    m->desc.origin = e->step - (done_at - m->desc.origin);
    m->stop_step = e->step + steps;
    e->dirty = true;
    return GB_GO_OK;
}

extern "C" int gb_ens_step_remaining(gb_ens *e, int32_t nsteps) { return gb_ens_step(e, nsteps); }

extern "C" int gb_ens_remaining(gb_ens *e, int32_t id, int64_t *steps)
{
    if (!e || !steps) return GB_GO_EINVAL;
    auto it = e->members.find(id);
    if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
    *steps = std::max<long long>(0, it->second->stop_step - e->step);
    return GB_GO_OK;
}

static double *current_buffer(gb_ens *e, Member *m)
{
    const long long done_at = std::min(e->step, m->stop_step);
    return ((done_at + m->desc.parity) & 1) ? m->buf1 : m->buf0;
}

// The other ping-pong buffer: the next step overwrites every cell of it that anything reads,
// so downloads use it as scratch for the Fortran-layout copy of the current state.
static double *scratch_buffer(gb_ens *e, Member *m) { return current_buffer(e, m) == m->buf0 ? m->buf1 : m->buf0; }

__global__ void k_merge_member(double *out, const double *stat, const double *cur, Dims d, const int32_t *k1)
{
    const size_t ncell = (size_t)d.NI * d.NJ * (d.maxk + 2);
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < ncell; c += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % d.NI);
        const int j = (int)((c / d.NI) % d.NJ);
        const int k = (int)(c / ((size_t)d.NI * d.NJ));
        bool take = false;
        if (k >= 1 && k <= d.maxk && j >= 1 && j <= d.maxj && i >= 1 && i <= d.maxi) take = k >= k1[i + d.NI * j];
        const double *src = take ? cur : stat;
        for (int l = 0; l < d.L; ++l) out[c * d.L + l] = src[c * d.L + l];
    }
}

static int download_on(gb_ens *e, Member *m, cudaStream_t s, double *ts, double *rho, double *cost)
{
    double *cur = scratch_buffer(e, m);
    MemberDesc md = m->desc;
    int r = fp32_export(md, current_buffer(e, m), cur, m->rho, s);
    if (r) return efail(e, r, "export failed");
    const size_t nts = (size_t)m->d.L * m->d.NI * m->d.NJ * (m->d.maxk + 2);
    if (ts) {
        const size_t ncell = (size_t)m->d.NI * m->d.NJ * (m->d.maxk + 2);
        k_merge_member<<<(int)std::min<size_t>((ncell + 255) / 256, 4096), 256, 0, s>>>(m->stage, m->ts_static, cur, m->d, m->k1);
        count_launches(1);
        ETRY(e, cudaMemcpyAsync(ts, m->stage, nts * 8, cudaMemcpyDeviceToHost, s));
    }
    if (rho) ETRY(e, cudaMemcpyAsync(rho, m->rho, (size_t)m->d.NI * m->d.NJ * (m->d.maxk + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (cost) ETRY(e, cudaMemcpyAsync(cost, m->cost, (size_t)m->d.maxi * m->d.maxj * 8, cudaMemcpyDeviceToHost, s));
    ETRY(e, cudaStreamSynchronize(s));
    return GB_GO_OK;
}

// One member's download in one kernel: the Fortran-layout ts (the current group-planar state on
// wet interior cells, the uploaded values elsewhere -- halo columns included, which the steps
// leave as uploaded) into `stage`, and rho (eos of that state on interior cells at zro(k), the
// periodic copies on wet halo cells; other entries keep their value, zero from admission).
// The same values as fp32_export followed by k_merge_member, without the intermediate Fortran
// copy.  A grid-stride range over the cells of the (NI, NJ, maxk+2) box.
struct DownloadItem {
    MemberDesc md;
    const double *planar;
    double *stage, *rho;
};

__device__ __forceinline__ void member_download_cells(const MemberDesc &md, const double *planar, double *stage, double *rho,
                                                      size_t c0, size_t cs)
{
    const int maxi = md.maxi, maxj = md.maxj, maxk = md.maxk, L = md.L, NI = md.NI, NJ = md.NJ;
    const size_t NIJ = (size_t)NI * NJ, ncell = NIJ * (maxk + 2), NIJK = ncell;
    const double *zro = md.mk + 3 * (maxk + 2);
    EosCoef ec;
    for (int n = 0; n < 5; ++n) ec.ec[n] = md.ec[n];
    ec.ieos = md.ieos;
    const int ng = fp32_ngroups(L);
    for (size_t c = c0; c < ncell; c += cs) {
        const int i = (int)(c % NI);
        const int j = (int)((c / NI) % NJ);
        const int k = (int)(c / NIJ);
        const bool inner = k >= 1 && k <= maxk && j >= 1 && j <= maxj;
        const bool wet = inner && i >= 1 && i <= maxi && k >= md.k1[i + NI * j];
        double t = 0.0, sv = 0.0;
        for (int g = 0, l = 0; g < ng; ++g) {
            int g0, gl, gp, pl;
            fp32_plane(L, g, &g0, &gl, &gp, &pl);
            for (int q = 0; q < gl; ++q, ++l) {
                const double v = wet ? planar[(size_t)pl * NIJK + c * gp + q] : md.ts_static[c * L + l];
                stage[c * L + l] = v;
                if (l == 0) t = v;
                if (l == 1) sv = v;
            }
        }
        if (!inner) continue;
        if (i >= 1 && i <= maxi) {
            rho[i + NI * (j + NJ * (size_t)k)] = eos_rn(ec, t, sv, zro[k]);
        } else {
            // wet halo cells: the density of the periodic source column (k1 is periodic, so the
            // source is wet there too)
            if (k < md.k1[i + NI * j]) continue;
            const int src = i == 0 ? maxi : 1;
            const size_t cs2 = (size_t)src + NI * (j + NJ * (size_t)k);
            rho[i + NI * (j + NJ * (size_t)k)] = eos_rn(ec, planar[cs2 * 2], planar[cs2 * 2 + 1], zro[k]);
        }
    }
}

// The downloads of several members in one launch (blockIdx.y: the member's item).
__global__ void k_member_download_many(const DownloadItem *it)
{
    const DownloadItem &I = it[blockIdx.y];
    member_download_cells(I.md, I.planar, I.stage, I.rho, blockIdx.x * (size_t)blockDim.x + threadIdx.x,
                          (size_t)gridDim.x * blockDim.x);
}

extern "C" int gb_ens_download_many(gb_ens *e, int32_t n, const int32_t *ids, double *const *ts, double *const *rho,
                                    double *const *cost)
{
    gbgo::TraceRange tr_("ens_download_many");
    if (!e || n < 0 || (n > 0 && !ids)) return GB_GO_EINVAL;
    std::vector<Member *> ms;
    for (int32_t q = 0; q < n; ++q) {
        auto it = e->members.find(ids[q]);
        if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
        ms.push_back(it->second.get());
    }
    ETRY(e, cudaSetDevice(e->device));
    if (n == 0) return GB_GO_OK;
    // one kernel forms every member's Fortran-layout ts and rho on the device; destinations in
    // mapped host memory (8-byte aligned) then take their arrays in one scatter kernel with
    // coalesced 16-byte stores, the others in one copy call each
    std::vector<DownloadItem> items(n);
    std::vector<CopySeg> segs;
    std::vector<unsigned char> direct(n, 0);   // bit 0 ts, bit 1 rho, bit 2 cost by the scatter kernel
    size_t max_cells = 1;
    auto mapped = [](double *p, size_t count) -> void * {
        return p && ((uintptr_t)p & 7) == 0 ? host_mapped(p, count * 8) : nullptr;
    };
    for (int32_t q = 0; q < n; ++q) {
        Member *m = ms[q];
        const size_t ncell = (size_t)m->d.NI * m->d.NJ * (m->d.maxk + 2);
        const size_t nrho = (size_t)m->d.NI * m->d.NJ * (m->d.maxk + 1), ncol = (size_t)m->d.maxi * m->d.maxj;
        items[q].md = m->desc;
        items[q].planar = current_buffer(e, m);
        items[q].stage = m->stage;
        items[q].rho = m->rho;
        if (void *d = mapped(ts ? ts[q] : nullptr, ncell * m->d.L)) {
            segs.push_back(CopySeg{m->stage, d, ncell * m->d.L * 8});
            direct[q] |= 1;
        }
        if (void *d = mapped(rho ? rho[q] : nullptr, nrho)) {
            segs.push_back(CopySeg{m->rho, d, nrho * 8});
            direct[q] |= 2;
        }
        if (void *d = mapped(cost ? cost[q] : nullptr, ncol)) {
            segs.push_back(CopySeg{m->cost, d, ncol * 8});
            direct[q] |= 4;
        }
        max_cells = std::max(max_cells, ncell);
    }
    cudaStream_t s = e->stream;
    for (int32_t q0 = 0; q0 < n; q0 += 65535) {
        const int nq = std::min<int>(n - q0, 65535);
        DownloadItem *dit = nullptr;
        ETRY(e, cudaMallocAsync((void **)&dit, sizeof(DownloadItem) * nq, s));
        cudaError_t x = cudaMemcpyAsync(dit, items.data() + q0, sizeof(DownloadItem) * nq, cudaMemcpyHostToDevice, s);
        if (x == cudaSuccess) {
            const int bx = (int)std::max<size_t>(1, std::min<size_t>((max_cells + 255) / 256, 128));
            k_member_download_many<<<dim3(bx, nq), 256, 0, s>>>(dit);
            count_launches(1);
            x = cudaGetLastError();
        }
        cudaFreeAsync(dit, s);
        if (x != cudaSuccess) return efail(e, GB_GO_ECUDA, cudaGetErrorString(x));
    }
    if (!segs.empty()) {
        CopySeg *dsg = nullptr;
        ETRY(e, cudaMallocAsync((void **)&dsg, sizeof(CopySeg) * segs.size(), s));
        cudaError_t x = cudaMemcpyAsync(dsg, segs.data(), sizeof(CopySeg) * segs.size(), cudaMemcpyHostToDevice, s);
        size_t longest = 16;
        for (const CopySeg &g : segs) longest = std::max<size_t>(longest, g.bytes);
        const int bx = (int)std::min<size_t>((longest / 16 + 255) / 256, 64);
        for (size_t g0 = 0; x == cudaSuccess && g0 < segs.size(); g0 += 65535) {
            const int ng = (int)std::min<size_t>(segs.size() - g0, 65535);
            k_scatter<<<dim3(bx, ng), 256, 0, s>>>(dsg + g0);
            count_launches(1);
            x = cudaGetLastError();
        }
        cudaFreeAsync(dsg, s);
        if (x != cudaSuccess) return efail(e, GB_GO_ECUDA, cudaGetErrorString(x));
    }
    for (int32_t q = 0; q < n; ++q) {
        Member *m = ms[q];
        const size_t nts = (size_t)m->d.NI * m->d.NJ * (m->d.maxk + 2) * m->d.L;
        if (ts && ts[q] && !(direct[q] & 1)) ETRY(e, cudaMemcpyAsync(ts[q], m->stage, nts * 8, cudaMemcpyDeviceToHost, s));
        if (rho && rho[q] && !(direct[q] & 2))
            ETRY(e, cudaMemcpyAsync(rho[q], m->rho, (size_t)m->d.NI * m->d.NJ * (m->d.maxk + 1) * 8, cudaMemcpyDeviceToHost, s));
        if (cost && cost[q] && !(direct[q] & 4))
            ETRY(e, cudaMemcpyAsync(cost[q], m->cost, (size_t)m->d.maxi * m->d.maxj * 8, cudaMemcpyDeviceToHost, s));
    }
    ETRY(e, cudaStreamSynchronize(s));
    return GB_GO_OK;
}

extern "C" int gb_ens_download(gb_ens *e, int32_t id, double *ts, double *rho, double *cost)
{
    return gb_ens_download_many(e, 1, &id, ts ? &ts : nullptr, rho ? &rho : nullptr, cost ? &cost : nullptr);
}

extern "C" int gb_ens_download_stream(gb_ens *e, int32_t id, void *cuda_stream, double *ts, double *rho, double *cost)
{
    if (!e) return GB_GO_EINVAL;
    auto it = e->members.find(id);
    if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
    ETRY(e, cudaSetDevice(e->device));
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : e->stream;
    if (s != e->stream) {
        // after everything queued on the ensemble's stream (the steps)
        cudaEvent_t ev;
        ETRY(e, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        cudaError_t x = cudaEventRecord(ev, e->stream);
        if (x == cudaSuccess) x = cudaStreamWaitEvent(s, ev, 0);
        cudaEventDestroy(ev);
        if (x != cudaSuccess) return efail(e, GB_GO_ECUDA, cudaGetErrorString(x));
    }
    return download_on(e, it->second.get(), s, ts, rho, cost);
}

__global__ void k_member_inventory(const double *ts, Dims d, const int32_t *k1, const double *mk, const double *rvol_unused,
                                   const double *dsj, double *out)
{
    // one block per tracer; Neumaier-compensated sum of ts*ds(j)*dz(k) over wet cells
    const int l = blockIdx.x;
    const size_t ncol = (size_t)d.maxi * d.maxj, ncell = ncol * d.maxk;
    double s = 0.0, c = 0.0;
    for (size_t n = threadIdx.x; n < ncell; n += blockDim.x) {
        const int i = (int)(n % d.maxi) + 1, j = (int)((n / d.maxi) % d.maxj) + 1, k = (int)(n / ncol) + 1;
        if (k < k1[i + d.NI * j]) continue;
        const double x = __dmul_rn(__dmul_rn(ts[ts_index(d, l, i, j, k)], dsj[j]), mk[k]);
        const double t = __dadd_rn(s, x);
        if (fabs(s) >= fabs(x)) c = __dadd_rn(c, __dadd_rn(__dadd_rn(s, -t), x));
        else c = __dadd_rn(c, __dadd_rn(__dadd_rn(x, -t), s));
        s = t;
    }
    __shared__ double ss[256], sc[256];
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, C = 0.0;
        for (int n = 0; n < blockDim.x; ++n) {
            const double x = ss[n];
            const double t = __dadd_rn(S, x);
            if (fabs(S) >= fabs(x)) C = __dadd_rn(C, __dadd_rn(__dadd_rn(S, -t), x));
            else C = __dadd_rn(C, __dadd_rn(__dadd_rn(x, -t), S));
            S = t;
            C = __dadd_rn(C, sc[n]);
        }
        out[l] = __dadd_rn(S, C);
    }
}

extern "C" int gb_ens_inventory(gb_ens *e, int32_t id, double *out)
{
    if (!e || !out) return GB_GO_EINVAL;
    auto it = e->members.find(id);
    if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
    Member *m = it->second.get();
    ETRY(e, cudaSetDevice(e->device));
    cudaStream_t s = e->stream;
    double *dout = nullptr;
    ETRY(e, cudaMallocAsync(&dout, m->d.L * sizeof(double), s));
    double *fort = scratch_buffer(e, m);
    if (fp32_from_planar(fort, current_buffer(e, m), m->d, s)) return efail(e, GB_GO_ECUDA, "export failed");
    k_member_inventory<<<m->d.L, 256, 0, s>>>(fort, m->d, m->k1, m->mk, nullptr, m->dsj, dout);
    count_launches(1);
    ETRY(e, cudaMemcpyAsync(out, dout, m->d.L * sizeof(double), cudaMemcpyDeviceToHost, s));
    cudaFreeAsync(dout, s);
    ETRY(e, cudaStreamSynchronize(s));
    return GB_GO_OK;
}

extern "C" int gb_ens_set_mld_wind(gb_ens *e, int32_t id, const double *mldketau)
{
    if (!e || !mldketau) return GB_GO_EINVAL;
    auto it = e->members.find(id);
    if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
    Member *m = it->second.get();
    if (!m->mldketau) return efail(e, GB_GO_EINVAL, "set_mld_wind: the member has imld = 0");
    ETRY(e, cudaSetDevice(e->device));
    // queued behind the steps already launched: it applies from the next step on
    ETRY(e, cudaMemcpyAsync(m->mldketau, mldketau, (size_t)m->d.maxi * m->d.maxj * 8, cudaMemcpyHostToDevice, e->stream));
    ETRY(e, cudaStreamSynchronize(e->stream));
    return GB_GO_OK;
}

extern "C" int gb_ens_download_mld(gb_ens *e, int32_t id, double *mld, int32_t *mldk)
{
    if (!e) return GB_GO_EINVAL;
    auto it = e->members.find(id);
    if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
    Member *m = it->second.get();
    if (!m->mld) return efail(e, GB_GO_EINVAL, "download_mld: the member has imld = 0");
    ETRY(e, cudaSetDevice(e->device));
    const size_t ncol = (size_t)m->d.maxi * m->d.maxj;
    if (mld) ETRY(e, cudaMemcpyAsync(mld, m->mld, ncol * 8, cudaMemcpyDeviceToHost, e->stream));
    if (mldk) ETRY(e, cudaMemcpyAsync(mldk, m->mldk, ncol * 4, cudaMemcpyDeviceToHost, e->stream));
    ETRY(e, cudaStreamSynchronize(e->stream));
    return GB_GO_OK;
}

extern "C" int gb_ens_status(gb_ens *e, int32_t id, int32_t *status)
{
    if (!e || !status) return GB_GO_EINVAL;
    auto it = e->members.find(id);
    if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
    unsigned int st = 0;
    ETRY(e, cudaMemcpyAsync(&st, it->second->status, sizeof(st), cudaMemcpyDeviceToHost, e->stream));
    ETRY(e, cudaStreamSynchronize(e->stream));
    *status = (int32_t)st;
    return GB_GO_OK;
}

extern "C" int gb_ens_sync(gb_ens *e)
{
    if (!e) return GB_GO_EINVAL;
    ETRY(e, cudaSetDevice(e->device));
    ETRY(e, cudaStreamSynchronize(e->stream));
    return GB_GO_OK;
}

extern "C" int gb_ens_count(gb_ens *e, int32_t *active, size_t *bytes_in_use)
{
    if (!e) return GB_GO_EINVAL;
    if (active) {
        int n = 0;
        for (auto &kv : e->members)
            if (kv.second->stop_step > e->step) ++n;
        *active = n;
    }
    if (bytes_in_use) *bytes_in_use = e->in_use;
    return GB_GO_OK;
}

extern "C" const char *gb_ens_last_error(const gb_ens *e) { return e ? e->last_error.c_str() : ""; }
