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

namespace gbgo {
int validate_config(const gb_go_dims *dims, const gb_go_params *params, const gb_go_grid *grid, std::string &msg);
void build_metric_blob(const gb_go_dims *dims, const gb_go_params *params, const gb_go_grid *g, std::vector<double> &blob);
PhysParams phys_from(const gb_go_params *pp, const gb_go_grid *g);
}  // namespace gbgo

using namespace gbgo;

namespace {

__global__ void k_add_step(long long *ctr, long long n) { *ctr += n; }

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
    int wet_cols = 0;                     // wet columns (entries it may add to the co list)
    std::vector<int32_t> poff;            // per patch: word offset in ptab
    std::vector<double> pcost;            // per patch: cell-updates per step
    int max_slots = 1;
    std::vector<double> ds_host;          // ds(0:maxj+1), for the inventory
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
    int2 *colist = nullptr;             // columns listed for the exact convective adjustment
    int *cocount = nullptr;             // two counters, by step parity
    int cocap = 0;
    int *work = nullptr;                // device work counters (two, by step parity)
    bool dirty = true;
    gb_ens_tuning tuning{0, 0, 0, 0};
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    std::string last_error;
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
           ncol * 12 + (size_t)(d->maxi + 2) * (d->maxj + 2) * 4 + ncol * (31 + (size_t)d->maxk) * 4 + ned * 8 + nst * 4 + (size_t)d->maxl * 4 + 4096;
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
    if (x == cudaSuccess) x = cudaMalloc(&e->cocount, 2 * sizeof(int));
    if (x == cudaSuccess) x = cudaMemset(e->cocount, 0, 2 * sizeof(int));
    if (x != cudaSuccess) {
        gb_ens_destroy(e);
        return x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA;
    }
    *out = e;
    return GB_GO_OK;
}

static void free_member(gb_ens *e, Member *m)
{
    cudaStream_t s = e->stream;
    void *ptrs[] = {m->buf0, m->buf1, m->ts_static, m->rho, m->stage, m->coef, m->coefl, m->gtop, m->mj,
                    m->rvol, m->mk, m->cost, m->k1, m->scale, m->tref, m->icosd, m->dsj, m->diag, m->status, m->gmax,
                    m->ptab, m->vel, m->ediff1, m->mkd, m->stencil};
    for (void *p : ptrs)
        if (p) cudaFreeAsync(p, s);
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

template <class T>
static cudaError_t dalloc(gb_ens *e, T **p, size_t n)
{
    return cudaMallocFromPoolAsync((void **)p, n * sizeof(T), e->pool, e->stream);
}

extern "C" int gb_ens_add(gb_ens *e, const gb_go_dims *dims, const gb_go_params *params, const gb_go_grid *grid,
                          const double *ts, const double *u, int32_t *member_id)
{
    if (!e || !ts || !u || !member_id) return GB_GO_EINVAL;
    std::string msg;
    int rc = validate_config(dims, params, grid, msg);
    if (rc) return efail(e, rc, msg);
    if (dims->maxl > kFp32MaxL) return efail(e, GB_GO_ERANGE, "ensemble members carry at most 32 tracers");
    if (params->imld != 0) return efail(e, GB_GO_EUNSUPPORTED, "imld=1 not provided in ensembles");
    for (int k = 1; k < dims->maxk; ++k)
        if (grid->dt[k] != grid->dt[0]) return efail(e, GB_GO_EUNSUPPORTED, "ensemble members need one dt for all levels");
    const size_t bytes = member_bytes(dims, params);
    ETRY(e, cudaSetDevice(e->device));

    auto m = std::make_unique<Member>();
    m->d = Dims{dims->maxi, dims->maxj, dims->maxk, dims->maxl, dims->maxi + 2, dims->maxj + 2};
    m->p = phys_from(params, grid);
    m->dt = grid->dt[0];
    m->bytes = bytes;
    if (dims->maxk > kMaxK) return efail(e, GB_GO_ERANGE, "ensemble members have at most 64 levels");
    PatchPlan plan;
    if (fp32_plan_patches(m->d, grid->k1, e->tuning.tile_i, e->tuning.tile_j, plan) != GB_GO_OK)
        return efail(e, GB_GO_ERANGE, "no patch shape fits the FP32-flux kernel limits");
    m->poff = plan.offset;
    m->pcost = plan.cost;
    m->max_slots = plan.max_slots;
    std::vector<double> blob;
    build_metric_blob(dims, params, grid, blob);
    Fp32Static st;
    fp32_build_static(m->d, m->p, blob, grid->k1, u, st);
    std::vector<float> gtop;
    const size_t ntop = (size_t)dims->maxl * m->d.NI * m->d.NJ;
    fp32_gtop(m->d, m->p, blob, ts + ntop * (dims->maxk + 1), gtop);
    std::vector<int32_t> scale;
    std::vector<float> tref;
    fp32_scales(m->d, grid->k1, ts, st.cmax, st.dmax, gtop.data(), scale, tref);

    // device allocation, copies and registration: one member at a time
    std::lock_guard<std::mutex> lk(e->mu);
    if (e->in_use + bytes > e->budget) return efail(e, GB_GO_ENOMEM, "member does not fit in the HBM budget");
    const size_t nts = ntop * (dims->maxk + 2);
    const size_t nrho = (size_t)m->d.NI * m->d.NJ * (dims->maxk + 1);
    const size_t ncol = (size_t)dims->maxi * dims->maxj;
    cudaStream_t s = e->stream;
    const size_t nplan = fp32_planar_size(m->d);
    cudaError_t x = dalloc(e, &m->buf0, nplan);
    if (x == cudaSuccess) x = dalloc(e, &m->buf1, nplan);
    if (x == cudaSuccess) x = dalloc(e, &m->ts_static, nts);
    if (x == cudaSuccess) x = dalloc(e, &m->stage, nts);
    if (x == cudaSuccess) x = dalloc(e, &m->rho, nrho);
    if (x == cudaSuccess) x = dalloc(e, &m->coef, st.coef.size());
    if (x == cudaSuccess) x = dalloc(e, &m->coefl, st.coefl.size());
    if (x == cudaSuccess) x = dalloc(e, &m->gtop, gtop.size());
    if (x == cudaSuccess) x = dalloc(e, &m->mj, st.mj.size());
    if (x == cudaSuccess) x = dalloc(e, &m->rvol, st.rvol.size());
    if (x == cudaSuccess) x = dalloc(e, &m->mk, st.mk.size());
    if (x == cudaSuccess) x = dalloc(e, &m->cost, ncol);
    if (x == cudaSuccess) x = dalloc(e, &m->icosd, ncol);
    if (x == cudaSuccess) x = dalloc(e, &m->k1, (size_t)m->d.NI * m->d.NJ);
    if (x == cudaSuccess) x = dalloc(e, &m->scale, scale.size());
    if (x == cudaSuccess) x = dalloc(e, &m->tref, tref.size());
    if (x == cudaSuccess) x = dalloc(e, &m->dsj, (size_t)dims->maxj + 2);
    if (x == cudaSuccess) x = dalloc(e, &m->gmax, (size_t)dims->maxl);
    if (x == cudaSuccess) x = cudaMemsetAsync(m->gmax, 0, (size_t)dims->maxl * sizeof(unsigned int), s);
    if (x == cudaSuccess) x = dalloc(e, &m->diag, 4);
    if (x == cudaSuccess) x = dalloc(e, &m->status, 1);
    if (x == cudaSuccess) x = dalloc(e, &m->ptab, std::max<size_t>(4, plan.words.size()));
    if (x == cudaSuccess && !plan.words.empty())
        x = cudaMemcpyAsync(m->ptab, plan.words.data(), plan.words.size() * 4, cudaMemcpyHostToDevice, s);
    m->ds_host.assign(blob.begin() + 6 * (dims->maxj + 2), blob.begin() + 7 * (dims->maxj + 2));
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->dsj, m->ds_host.data(), m->ds_host.size() * 8, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess) x = cudaMemsetAsync(m->diag, 0, 4 * sizeof(unsigned long long), s);
    if (x == cudaSuccess) x = cudaMemsetAsync(m->status, 0, sizeof(unsigned int), s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->ts_static, ts, nts * 8, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess && (fp32_to_planar(m->buf0, m->ts_static, m->d, s) || fp32_to_planar(m->buf1, m->ts_static, m->d, s))) {
        const cudaError_t le = cudaGetLastError();
        x = le != cudaSuccess ? le : cudaErrorLaunchFailure;
    }
    if (x == cudaSuccess) x = cudaMemsetAsync(m->rho, 0, nrho * 8, s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->coef, st.coef.data(), st.coef.size() * 4, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->coefl, st.coefl.data(), st.coefl.size() * 4, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->gtop, gtop.data(), gtop.size() * 4, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->mj, st.mj.data(), st.mj.size() * 8, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->rvol, st.rvol.data(), st.rvol.size() * 8, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->mk, st.mk.data(), st.mk.size() * 8, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess) x = cudaMemsetAsync(m->cost, 0, ncol * 8, s);
    if (x == cudaSuccess) x = cudaMemsetAsync(m->icosd, 0, ncol * 4, s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->k1, grid->k1, (size_t)m->d.NI * m->d.NJ * 4, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->scale, scale.data(), scale.size() * 4, cudaMemcpyHostToDevice, s);
    if (x == cudaSuccess) x = cudaMemcpyAsync(m->tref, tref.data(), tref.size() * 4, cudaMemcpyHostToDevice, s);
    const bool need_ediff = params->iediff > 0 && params->iediff < 3;
    if (need_ediff) {
        // the step rebuilds the top-face coefficients from u, ediff1, dza and diffmax
        const size_t nu = (size_t)3 * (dims->maxi + 1) * (dims->maxj + 1) * dims->maxk;
        const size_t ned = (size_t)dims->maxi * dims->maxj * (dims->maxk - 1);
        const size_t nk = (size_t)dims->maxk + 2, nj = (size_t)dims->maxj + 2;
        if (x == cudaSuccess) x = dalloc(e, &m->vel, nu);
        if (x == cudaSuccess) x = dalloc(e, &m->ediff1, std::max<size_t>(1, ned));
        if (x == cudaSuccess) x = dalloc(e, &m->mkd, 2 * nk);
        if (x == cudaSuccess) x = cudaMemcpyAsync(m->vel, u, nu * 8, cudaMemcpyHostToDevice, s);
        if (x == cudaSuccess && ned) x = cudaMemcpyAsync(m->ediff1, grid->ediff1, ned * 8, cudaMemcpyHostToDevice, s);
        // Fortran-indexed dza, then diffmax, from the metric blob (8 j-arrays, then k-arrays)
        if (x == cudaSuccess) x = cudaMemcpyAsync(m->mkd, blob.data() + 8 * nj + nk, nk * 8, cudaMemcpyHostToDevice, s);
        if (x == cudaSuccess) x = cudaMemcpyAsync(m->mkd + nk, blob.data() + 8 * nj + 8 * nk, nk * 8, cudaMemcpyHostToDevice, s);
    }
    if (x == cudaSuccess && has_stencil(params)) x = dalloc(e, &m->stencil, (size_t)kStencilWords * dims->maxi * dims->maxj * dims->maxk);
    // host staging vectors must outlive the copies
    if (x == cudaSuccess) x = cudaStreamSynchronize(s);
    if (x != cudaSuccess) {
        free_member(e, m.get());
        cudaStreamSynchronize(s);
        return efail(e, x == cudaErrorMemoryAllocation ? GB_GO_ENOMEM : GB_GO_ECUDA, cudaGetErrorString(x));
    }
    MemberDesc &md = m->desc;
    md.maxi = dims->maxi; md.maxj = dims->maxj; md.maxk = dims->maxk; md.L = dims->maxl;
    md.NI = m->d.NI; md.NJ = m->d.NJ; md.diso = m->p.diso; md.ieos = m->p.ieos; md.iconv = m->p.iconv;
    md.iediff = m->p.iediff; md.ediffpow2i = m->p.ediffpow2i;
    md.diff2 = m->p.diff2; md.ediff0 = m->p.ediff0; md.ediffpow2 = m->p.ediffpow2;
    md.u = m->vel; md.ediff1 = m->ediff1;
    md.dza = m->mkd; md.diffmax = m->mkd ? m->mkd + (dims->maxk + 2) : nullptr;
    md.stencil = m->stencil;
    md.dt = m->dt; md.dphi = m->p.dphi; md.rdphi = m->p.rdphi; md.diff1 = m->p.diff1;
    for (int n = 0; n < 5; ++n) md.ec[n] = m->p.ec[n];
    md.dsc = m->p.dsc;
    md.buf[0] = m->buf0; md.buf[1] = m->buf1;
    md.ts_static = m->ts_static; md.coef = m->coef; md.coefl = m->coefl; md.rvol = m->rvol; md.gtop = m->gtop; md.k1 = m->k1;
    md.scale = m->scale; md.tref = m->tref; md.mk = m->mk; md.mj = m->mj; md.cost = m->cost; md.icosd = m->icosd;
    md.diag = m->diag; md.status = m->status; md.gmax = m->gmax; md.ptab = m->ptab;
    m->start_step = e->step;
    m->stop_step = (long long)1 << 62;
    md.parity = (int)(e->step & 1);     // (step + parity) & 1 == 0 at admission
    md.stop_step = m->stop_step;
    md.origin = e->step;
    long long wet = 0;
    for (int j = 1; j <= dims->maxj; ++j)
        for (int i = 1; i <= dims->maxi; ++i) {
            const int k1 = grid->k1[i + (size_t)m->d.NI * j];
            if (k1 <= dims->maxk) {
                wet += dims->maxk - k1 + 1;
                m->wet_cols += 1;
            }
        }
    m->cost_est = (double)wet * (dims->maxl + 4) * (params->diso ? 2.0 : 1.0);
    m->id = e->next_id++;
    *member_id = m->id;
    e->in_use += bytes;
    e->members[m->id] = std::move(m);
    e->dirty = true;
    return GB_GO_OK;
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
    int kmax = 1;
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
        co_general = co_general || !fp32_co_fast(m->desc.iconv, m->desc.ieos, m->d.maxk);
        kmax = std::max(kmax, m->d.maxk);
        ++slot;
    }
    std::stable_sort(order.begin(), order.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
    // transfer items (member, patch, group) with a patch's groups and a member's patches next to
    // each other: items taken together share the coefficients and ring columns in L2.  The co
    // column list holds at most every wet column of the batch.
    std::vector<int4> it;
    for (auto &o : order)
        for (size_t n = 0; n < o.second->poff.size(); ++n) it.push_back(make_int4(o.second->slot, o.second->poff[n], 0, 0));
    const int n_ts = (int)it.size();
    for (auto &o : order)
        for (size_t n = 0; n < o.second->poff.size(); ++n)
            for (int g = 1; g < fp32_group_count(o.second->d.L); ++g)
                it.push_back(make_int4(o.second->slot, o.second->poff[n], g, 0));
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
        e->colist = nullptr;
        ETRY(e, cudaMallocAsync(&e->colist, (size_t)cocap * sizeof(int2), s));
        e->cocap = cocap;
    }
    e->max_slots = max_slots;
    e->any_iso = any_iso;
    e->co_general = co_general;
    e->n_stencil = (int)slist.size();
    e->stencil_blocks = sblocks;
    e->kmax = kmax;
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
    b.work = e->work;
    b.colist = e->colist;
    b.cocount = e->cocount;
    b.cocap = e->cocap;
    b.iso = e->any_iso;
    b.co_general = e->co_general;
    b.stencil_list = e->stencil_list;
    b.n_stencil = e->n_stencil;
    b.stencil_blocks = e->stencil_blocks;
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

extern "C" int gb_ens_download(gb_ens *e, int32_t id, double *ts, double *rho, double *cost)
{
    if (!e) return GB_GO_EINVAL;
    auto it = e->members.find(id);
    if (it == e->members.end()) return efail(e, GB_GO_EINVAL, "no such member");
    ETRY(e, cudaSetDevice(e->device));
    return download_on(e, it->second.get(), e->stream, ts, rho, cost);
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
