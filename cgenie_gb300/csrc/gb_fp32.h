// FP32-flux / FP64-state form of the tracer step, for one grid and for the
// batched ensemble (a single grid is a batch of one member).
#pragma once

#include "gb_goldstein.h"
#include "gb_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

namespace gbgo {

constexpr int kFp32MaxL = 32;   // tracers per member supported by the FP32-flux kernel
constexpr int kFp32Threads = 128;   // CTA of the FP32-flux kernel: one thread per patch column

// Tracer groups: group 0 is T and S (double-float transfers, convection flag); the other
// tracers form groups of at most kGroup.  A work item of the step kernel is one group of
// one patch.
constexpr int kGroup = 8;

__host__ __device__ inline int fp32_ngroups(int L)
{
    return L <= 2 ? 1 : 1 + (L - 2 + kGroup - 1) / kGroup;
}

// First tracer g0 and size gl of group g.
__host__ __device__ inline void fp32_group(int L, int g, int *g0, int *gl)
{
    if (g == 0) {
        *g0 = 0;
        *gl = 2;
        return;
    }
    const int nb = L - 2, ngb = (nb + kGroup - 1) / kGroup;
    const int base = nb / ngb, rem = nb % ngb, h = g - 1;
    *gl = base + (h < rem ? 1 : 0);
    *g0 = 2 + h * base + (h < rem ? h : rem);
}

// Device-resident state of the FP32-flux path ("group-planar"): group g is a plane of
// NI*NJ*(maxk+2) cells with gp = gl rounded up to even doubles per cell, so that a
// group's values of one cell are contiguous and 16-byte aligned pairs:
//   (l, i, j, k), l = g0 + q  ->  plane(g) * NIJK + (i + NI*(j + NJ*k)) * gp + q
// plane(g) = sum of gp over the groups before g.  Fortran-layout arrays are converted
// on upload and export only.
__host__ __device__ inline void fp32_plane(int L, int g, int *g0, int *gl, int *gp, int *plane)
{
    fp32_group(L, g, g0, gl);
    *gp = *gl + (*gl & 1);
    int pl = 0;
    for (int h = 0; h < g; ++h) {
        int a, b;
        fp32_group(L, h, &a, &b);
        pl += b + (b & 1);
    }
    *plane = pl;
}

__host__ __device__ inline int fp32_planar_width(int L)
{
    int g0, gl, gp, pl;
    const int ng = fp32_ngroups(L);
    fp32_plane(L, ng - 1, &g0, &gl, &gp, &pl);
    return pl + gp;
}

// Top-face stencil words per cell: the hi parts of C1 C0 W0 E0 S0 N0 W1 E1 S1 N1 (the weights of
// T(k+1), T(k) and of T at the W, E, S, N neighbours of levels k and k+1), the isoneutral flag, 0,
// then the lo parts in the same order, 0, 0.
constexpr int kStencilWords = 24;

// Per-member descriptor read by the batched kernel (device memory).
struct MemberDesc {
    int maxi, maxj, maxk, L;
    int NI, NJ, diso, ieos;
    int iconv, status_idx, parity, iediff;
    long long stop_step;        // the member advances while step < stop_step
    long long origin;           // step - origin = the member's own count of steps taken (while active);
                                // its own steps 0, 4, 8, ... gather the transfer maxima for rescaling
    double dt, dphi, rdphi, diff1;
    double ec[5];
    double dsc;
    // iediff 1/2 (local vertical diffusivity, goldstein.f90:2490-2516): the top-face
    // coefficients of every cell are rebuilt each step from the FP64 T and S
    double diff2, ediff0, ediffpow2;
    int ediffpow2i, pad1;
    const double *u;            // velocities u(3,0:maxi,0:maxj,1:maxk) (iediff)
    const double *ediff1;       // (maxi, maxj, maxk-1) (iediff)
    const double *dza, *diffmax;   // Fortran-indexed [0..maxk+1] (iediff)
    float *stencil;             // diso or iediff: kStencilWords floats per interior cell (index as coef),
                                // the top-face stencil rebuilt every step by k_stencil_fp32
    double *buf[2];             // state ping-pong, group-planar layout (fp32_plane)
    const double *ts_static;    // uploaded ts (values below k1 for co with ieos=1)
    const float *coef;          // 8 floats per interior cell: Ae Be An Bn Aa Ba as FP32, then Dh Dl: the
                                // cell's sum of signed face transfer sums (A + B) as an FP32 pair, 0 where
                                // it is at the rounding level of FP64 (a divergence-free velocity field)
    const float *coefl;         // 8 floats per interior cell: the FP64 remainders of the same (hi+lo
                                // carries the FP64 coefficient; read by the T-S group only)
    const double *rvol;         // 1/(dphi*ds(j)*dz(k)), index (j-1) + maxj*(k-1)
    const float *gtop;          // forcing transfer dt*dphi*ds(j)*ts(l,i,j,maxk+1): L+2 floats per column
                                // ((i-1)+maxi*(j-1)): FP32 value of every tracer, then the lo parts of T, S
    const int32_t *k1;          // (maxi+2, maxj+2)
    const int32_t *ptab;        // patch tables (fp32_plan_patches); a work item gives a word offset
    int32_t *scale;             // per tracer power-of-two exponent of the fixed-point transfers; re-targeted
                                // between steps from gmax so the largest transfer sits near 2^26
    const float *tref;          // per tracer offset (FP32, 8 significant bits, 0 = none): the FP32 transfers
                                // carry T - tref, the offset's share enters through Dh Dl
    unsigned int *gmax;         // per tracer: largest |scaled transfer| of the step (FP32 bits)
    const double *mk;           // FP64 k metrics, Fortran-indexed, 6 arrays of maxk+2: dz, rdz, zw, zro, rdza, ssmax
    const double *mj;           // FP64 j metrics, 3 arrays of maxj+2: rc*rdphi, cv(j)*rdsv(j), dt*dphi*ds(j)
    double *cost;
    int32_t *icosd;
    unsigned long long *diag;   // two slots {dmax bits, limps}; step n uses slot n & 1 and clears
                                // slot (n+1) & 1 for the next step
    unsigned int *status;       // bit0 non-finite, bit1 transfer range exceeded, bit2 column list full
    // imld = 1, the Kraus-Turner mixed layer (goldstein.f90:2294-2390): every wet column joins the
    // column pass, which runs co and then the mixed layer in FP64 on the FP64 state
    int imld, pad2;
    double mldpebuoycoeff;
    const double *mlddec, *mlddecd;   // Fortran-indexed [1..maxk] (entry 0 unused)
    const double *mldketau;           // per column (i-1)+maxi*(j-1): wind mixing energy
    double *mld;                      // per column: mixed-layer depth
    int32_t *mldk;                    // per column: the level the mixed layer reaches
    double *rhos;                     // per column: rho(i,j,maxk) as the previous step left it
};

// Host-side owner of one member's FP32-path device data.
struct Fp32Data {
    MemberDesc host{};          // descriptor contents (device pointers)
    MemberDesc *dev = nullptr;  // device copy when used alone
    float *coef = nullptr, *coefl = nullptr;
    double *plan_buf[2] = {nullptr, nullptr};   // group-planar state ping-pong
    double *rvol = nullptr;
    float *gtop = nullptr;
    int32_t *scale = nullptr;
    float *tref = nullptr;
    unsigned int *gmax = nullptr;
    double *mk = nullptr, *mj = nullptr;
    unsigned int *status = nullptr;
    unsigned long long *diag = nullptr;
    float *stencil = nullptr;   // diso or iediff: the per-step top-face stencil (kStencilWords per cell)
    double *rhos = nullptr;     // imld = 1: rho(maxk) per column as the previous step left it
    int *stencil_list = nullptr;   // {0}: the member's descriptor index for the prepass when stepped alone
    int4 *items = nullptr;      // work items when stepped alone: (0, patch, group)
    int nitems = 0;
    int2 *colist = nullptr;     // columns for the exact convective adjustment (capacity cocap)
    int *cocount = nullptr;     // their count and the second phase's two slot counts, two each by step parity
    int cocap = 0;
    unsigned char *colog = nullptr;   // merge logs (cocap slots)
    int2 *comap = nullptr;      // second-phase slots (capacity mapcap)
    int mapcap = 0;
    int n_ts = 0;               // items[0, n_ts): T-S groups
    cudaStream_t s2 = nullptr;  // second stream and events: the two kinds of items side by side
    cudaEvent_t fork = nullptr, join = nullptr;
    int32_t *ptab = nullptr;    // patch tables
    int *work = nullptr;        // work counters (two, by step parity)
    int max_slots = 1;
    long long *step_ctr = nullptr;
    std::vector<int32_t> scale_host;
    std::vector<float> tref_host;
    std::vector<float> gtop_host_unscaled;
    double cmax = 0.0;          // max over faces of |A|+|B|
    double dmax = 0.0;          // max over cells of |D| (the divergence pair)
    long long steps = 0;
    long long step_host = 0;
    bool desc_valid = false;
};

struct Fp32Member {
    bool ready = false;
    void *impl = nullptr;   // owner of the member's FP32-path data (tstep_fp32.cu)
};

int fp32_member_init(Fp32Member *f, const Dims &d, const PhysParams &p, const Metrics &m,
                     const std::vector<double> &blob, const int32_t *k1_host, cudaStream_t s, std::string &msg);
void fp32_member_free(Fp32Member *f);
// host pointers: the transfer scales and coefficients are built on the host; ts1_dev is the
// uploaded ts1 on the device (Fortran layout), converted to the group-planar state
int fp32_member_upload(Fp32Member *f, const double *ts1_host, const double *ts_host, const double *ts1_dev, cudaStream_t s);
int fp32_member_set_top(Fp32Member *f, const double *top_host, cudaStream_t s);
// both step buffers from a Fortran-layout ts1 on the device (state rewritten between steps)
int fp32_member_reload(Fp32Member *f, const double *ts1_dev, cudaStream_t s);
// The first velocity field is taken from the host (coefficients and fixed-point scales);
// later ones from u_dev (device copy, coefficients rebuilt on the device).
int fp32_member_set_velocity(Fp32Member *f, const double *u_host, const double *u_dev, const Metrics &m,
                              cudaStream_t s);
int fp32_member_step(Fp32Member *f, double *ts_buf[2], int *cur, double *rho, const double *ts_static, double *cost,
                     int32_t *icosd, unsigned long long *diag, int *slot, int nsteps, cudaStream_t s);
// current state -> ts_cur (Fortran layout, halo columns) and rho
int fp32_member_export(Fp32Member *f, double *ts_cur, double *rho, const double *ts_static, cudaStream_t s);
// rho of the current state only (no Fortran-layout export of the tracers)
int fp32_member_rho(Fp32Member *f, double *rho, const double *ts_static, cudaStream_t s);
// the last CUDA error the FP32-path checks saw in this thread
const char *fp32_cuda_error_string();
// imld = 1: the handle's mixed-layer arrays (wind energy, outputs; mlddec, mlddecd Fortran-indexed
// [1..maxk]) and rho(maxk) of the uploaded density rho (NI, NJ, maxk+1) as the previous step's
int fp32_member_set_mixed_layer(Fp32Member *f, const double *mldketau, double *mld, int32_t *mldk, const double *mlddec,
                                const double *mlddecd, const double *rho, cudaStream_t s);
// current state -> dst (Fortran layout)
int fp32_member_fortran(Fp32Member *f, double *dst, cudaStream_t s);

// shared by the single-grid path and the ensemble
struct Fp32Static {
    std::vector<float> coef;       // 8 per interior cell (FP32 parts)
    std::vector<float> coefl;      // 8 per interior cell (remainders)
    std::vector<double> rvol;
    std::vector<double> mk, mj;
    double cmax = 0.0;
    double dmax = 0.0;             // max over cells of |D| (coefficient words 6, 7)
};
void fp32_build_static(const Dims &d, const PhysParams &p, const std::vector<double> &blob, const int32_t *k1,
                       const double *u_host, Fp32Static &out);
// rvol, mk, mj of fp32_build_static only (no coefficients)
void fp32_build_small(const Dims &d, const PhysParams &p, const std::vector<double> &blob, Fp32Static &out);

// Exponent s of the fixed-point transfers of a tracer whose largest transfer is g: the largest
// s with g * 2^s <= 2^26, i.e. floor(log2(2^26 / g)), from the exact binary exponent of g;
// clamped to [-120, 120]; 0 for g = 0 or non-finite g.  Host and device give the same value.
__host__ __device__ inline int fp32_scale_of(double g)
{
    if (!(g > 0.0) || !(g <= 1.7976931348623157e308)) return 0;
    int e = 0;
    const double f = frexp(g, &e);   // g = f 2^e, f in [0.5, 1)
    const int s = 26 - e + (f == 0.5 ? 1 : 0);
    return s < -120 ? -120 : (s > 120 ? 120 : s);
}
// Per tracer: the offset tref (tracers whose wet values lie within a factor of two of each
// other: DIC, alkalinity; 0 for the others and for T and S) and the fixed-point scale from
// the largest transfer: 2 cmax max |T - tref|, the forcing, and |tref| dmax.
void fp32_scales(const Dims &d, const int32_t *k1, const double *ts_host, double cmax, double dmax,
                 const float *gtop_unscaled, std::vector<int32_t> &scale, std::vector<float> &tref);
// The per-tracer inputs of fp32_scales that come from the state: tref, max |T - tref| over wet
// cells, and the largest forcing transfer.
void fp32_tracer_maxima(const Dims &d, const int32_t *k1, const double *ts, const float *gtop, std::vector<float> &tref,
                        std::vector<double> &tmax, std::vector<double> &gmax);
// the largest transfer bound whose exponent fp32_scale_of gives (host; k_member_scales on the device)
double fp32_transfer_bound(double cmax, double dmax, double tmax, double gmax, float tref);

// One member of a batched device set-up (device pointers; Metrics into the member's uploaded
// metric blob).
struct SetupItem {
    Dims d;
    PhysParams p;
    Metrics m;
    const double *u, *ts_static;
    double *buf0, *buf1;
    float *coef, *coefl;
    unsigned long long *cd;
    double *tmax;               // written by the set-up: max over wet cells of |T - tref|
    const double *gmax;
    float *tref;                // written by the set-up: the per-tracer offsets
    unsigned long long *ext;    // 2 L words, zeroed: order keys of the wet maxima and (inverted) minima
    int32_t *scale;
};
// Device part of the set-up of n ensemble members (items in device memory; stream order, no
// synchronisation), six launches in all: both state buffers from the uploaded ts; the transfer
// coefficients from u as fp32_build_static builds them (words 0-5, then the divergence pair);
// their largest face sums and divergence into cd[0], cd[1] (double bits, cd zeroed beforehand);
// the extremes of every tracer over the wet cells (ext); then the offsets and maxima of
// fp32_tracer_maxima from them and the fixed-point scales from cd (fp32_transfer_bound,
// fp32_scale_of).  max_elems / max_cells: the largest state (L x cells) and interior cell count
// of the items.
int fp32_setup_many(const SetupItem *items_dev, int n, size_t max_elems, size_t max_cells, cudaStream_t s);
void fp32_gtop(const Dims &d, const PhysParams &p, const std::vector<double> &blob, const double *top_host,
               std::vector<float> &gtop);
// Patch plan of one member: the kernel's work items.  Word layout of one patch table:
//   [ns, ni, kstart, patch index, 0, 0, 0, 0], nki[0..maxk+1] (interior slots with k1 <= k),
//   nkr[0..maxk+1] (ring slots with k1 <= k), goff[ns] (i + NI*j of each slot; interior
//   slots 0..ni-1, then the ring), padding to 4 words,
//   then 8 words per interior column (in slot order): slot | E << 16, W | N << 16,
//   S | k1 << 16, (i-1) + maxi*(j-1), i | j << 16, neighbour k1 (E, W, N, S bytes),
//   west cell index, 0.  A neighbour slot 0xffff is land.
struct PatchPlan {
    std::vector<int32_t> words;
    std::vector<int32_t> offset;   // per patch: word offset of its table
    std::vector<double> cost;      // per patch: cell-updates per step
    int max_slots = 1;
    int tile_i = 0, tile_j = 0;    // rectangle chosen
};
// tile_i/tile_j > 0 ask for that rectangle (if within the kernel limits), else the cheapest one
int fp32_plan_patches(const Dims &d, const int32_t *k1, int tile_i, int tile_j, PatchPlan &plan);
int fp32_group_count(int L);   // tracer groups (work items per patch): T and S, then groups of <= 8
// blocks per member of the stencil prepass for a grid of `ncell` interior cells
inline int fp32_stencil_blocks(size_t ncell) { return (int)std::min<size_t>(16384, (ncell + 255) / 256); }
// Fortran layout (L, NI, NJ, maxk+2) <-> group-planar layout of the FP32-flux state
int fp32_to_planar(double *planar, const double *fortran, const Dims &d, cudaStream_t s);
int fp32_from_planar(double *fortran, const double *planar, const Dims &d, cudaStream_t s);
inline size_t fp32_planar_size(const Dims &d) { return (size_t)fp32_planar_width(d.L) * d.NI * d.NJ * (d.maxk + 2); }
// One step of a batch: the transfer kernels over (member, patch, group) items (items[0, n_ts)
// are the T-S groups, items[n_ts, n_ts + n_bgc) the others), which list the columns that
// need the exact convective adjustment (colist, count in cocount[step & 1], capacity cocap:
// the wet columns of the batch), then the adjustment of those columns.  kmax: the largest
// maxk of the batch; iso: some member has the isoneutral branch (selects the kernel
// instances that have it); work: four counters.
struct Fp32Batch {
    const MemberDesc *descs = nullptr;
    const int4 *items = nullptr;
    int n_ts = 0, n_bgc = 0;
    int max_slots = 1, kmax = 1;
    int lmax = kFp32MaxL;       // the largest L of the members (shared memory of the adjustment)
    int *work = nullptr;
    int2 *colist = nullptr;
    int *cocount = nullptr;     // list counts, then front and back slot counts, two each by step parity
    int cocap = 0;
    unsigned char *colog = nullptr;   // merge logs of the two-phase adjustment (cocap slots)
    int2 *comap = nullptr;      // (list entry, tracer) slots of its second phase
    int mapcap = 0;
    bool iso = false;
    bool co_general = false;   // some member has iconv = 1, ieos != 0, imld = 1 or maxk > 32
    const int *stencil_list = nullptr;   // descriptor indices of the members with a stencil
    int n_stencil = 0, stencil_blocks = 1;   // their count; blocks per member of the prepass
    int ctas_per_sm = 0;        // cap on resident CTAs per SM of the transfer kernels (0: none)
    int co_form = 0;            // GB_ENS_CO_*: the adjustment's form (0: by the list capacity)
};
// s2/fork/join: a second stream and two events to run the two item kinds side by side
// (s2 null: one stream).
int fp32_launch(const Fp32Batch &b, const long long *step_ctr, int rel, cudaStream_t s, cudaStream_t s2,
                cudaEvent_t fork, cudaEvent_t join);
int fp32_launches_per_step(const Fp32Batch &b);   // kernels fp32_launch starts
// the adjustment runs in two phases (else one warp per column): by the batch's form, or for
// GB_ENS_CO_AUTO from GB_ENS_CO_TWO_PHASE_MIN listable columns
inline bool fp32_co_two_phase(const Fp32Batch &b)
{
    return b.co_form == GB_ENS_CO_TWO_PHASE || (b.co_form == GB_ENS_CO_AUTO && b.cocap >= GB_ENS_CO_TWO_PHASE_MIN);
}
// scratch of the two-phase adjustment: merge-log bytes per listed column, and slots per column
constexpr size_t kCoLogSlotBytes = 1152;
inline int fp32_co_slots(int L) { return L > 2 ? L - 2 : 1; }
// columns the warp-parallel adjustment takes (the others run co's serial form)
__host__ __device__ inline bool fp32_co_fast(int iconv, int ieos, int imld, int maxk)
{
    return iconv == 0 && ieos == 0 && imld == 0 && maxk <= 32;
}
int fp32_smem_bytes(int max_slots);
// current state (group-planar) -> Fortran layout with halo columns, and rho
int fp32_export(const MemberDesc &md, const double *planar, double *cur, double *rho, cudaStream_t s);
// re-target the fixed-point scales of `n` members after a step (stream order)
int fp32_rescale(const MemberDesc *descs, int n, cudaStream_t s);

void count_launches(uint64_t n);

}  // namespace gbgo
