// FP32-flux / FP64-state form of the tracer step, for one grid and for the
// batched ensemble (a single grid is a batch of one member).
#pragma once

#include "gb_internal.h"

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace gbgo {

constexpr int kFp32MaxL = 32;   // tracers per member supported by the FP32-flux kernel
constexpr int kFp32Threads = 128;   // CTA of the FP32-flux kernel: one thread per patch column

// Per-member descriptor read by the batched kernel (device memory).
struct MemberDesc {
    int maxi, maxj, maxk, L;
    int NI, NJ, diso, ieos;
    int iconv, status_idx, parity, pad0;
    long long stop_step;        // the member advances while step < stop_step
    long long origin;           // step - origin = the member's own count of steps taken (while active);
                                // its own steps 0, 4, 8, ... gather the transfer maxima for rescaling
    double dt, dphi, rdphi, diff1;
    double ec[5];
    double dsc;
    double *buf[2];             // state ping-pong, Fortran layout with halos
    const double *ts_static;    // uploaded ts (values below k1 for co with ieos=1)
    const float *coef;          // 12 floats per interior cell: Ae Be An Bn Aa Ba as FP32, then their
                                // FP64 remainders (the pair hi+lo carries the FP64 coefficient)
    const double *rvol;         // 1/(dphi*ds(j)*dz(k)), index (j-1) + maxj*(k-1)
    const float *gtop;          // forcing transfer dt*dphi*ds(j)*ts(l,i,j,maxk+1): L+2 floats per column
                                // ((i-1)+maxi*(j-1)): FP32 value of every tracer, then the lo parts of T, S
    const int32_t *k1;          // (maxi+2, maxj+2)
    const int32_t *ptab;        // patch tables (fp32_plan_patches); a work item gives a word offset
    int32_t *scale;             // per tracer power-of-two exponent of the fixed-point transfers; re-targeted
                                // between steps from gmax so the largest transfer sits near 2^26
    unsigned int *gmax;         // per tracer: largest |scaled transfer| of the step (FP32 bits)
    const double *mk;           // FP64 k metrics, Fortran-indexed, 6 arrays of maxk+2: dz, rdz, zw, zro, rdza, ssmax
    const double *mj;           // FP64 j metrics, 3 arrays of maxj+2: rc*rdphi, cv(j)*rdsv(j), dt*dphi*ds(j)
    double *cost;
    int32_t *icosd;
    unsigned long long *diag;   // two slots {dmax bits, limps}; step n uses slot n & 1 and clears
                                // slot (n+1) & 1 for the next step
    unsigned int *status;       // bit0 non-finite, bit1 transfer range exceeded
    uint8_t *coflag;            // per column ((i-1) + maxi*(j-1)): density profile may be unstable
};

// Host-side owner of one member's FP32-path device data.
struct Fp32Data {
    MemberDesc host{};          // descriptor contents (device pointers)
    MemberDesc *dev = nullptr;  // device copy when used alone
    float *coef = nullptr;
    double *rvol = nullptr;
    float *gtop = nullptr;
    int32_t *scale = nullptr;
    unsigned int *gmax = nullptr;
    double *mk = nullptr, *mj = nullptr;
    unsigned int *status = nullptr;
    unsigned long long *diag = nullptr;
    int4 *items = nullptr;      // work items when stepped alone: (0, patch, group), then (0, patch) for co
    int nitems = 0, nco = 0;
    uint8_t *coflag = nullptr;
    int32_t *ptab = nullptr;    // patch tables
    int *work = nullptr;        // work counters (two, by step parity)
    int max_slots = 1;
    long long *step_ctr = nullptr;
    std::vector<int32_t> scale_host;
    std::vector<float> gtop_host_unscaled;
    double cmax = 0.0;          // max over faces of |A|+|B|
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
// host pointers: the transfer scales and coefficients are built on the host
int fp32_member_upload(Fp32Member *f, const double *ts1_host, const double *ts_host, cudaStream_t s);
int fp32_member_set_top(Fp32Member *f, const double *top_host, cudaStream_t s);
int fp32_member_set_velocity(Fp32Member *f, const double *u_host, cudaStream_t s);
int fp32_member_step(Fp32Member *f, double *ts_buf[2], int *cur, double *rho, const double *ts_static, double *cost,
                     int32_t *icosd, unsigned long long *diag, int *slot, int nsteps, cudaStream_t s);
int fp32_member_export(Fp32Member *f, const double *ts_cur, double *rho, const double *ts_static, cudaStream_t s);

// shared by the single-grid path and the ensemble
struct Fp32Static {
    std::vector<float> coef;       // 12 per interior cell
    std::vector<double> rvol;
    std::vector<double> mk, mj;
    double cmax = 0.0;
};
void fp32_build_static(const Dims &d, const PhysParams &p, const std::vector<double> &blob, const int32_t *k1,
                       const double *u_host, Fp32Static &out);
void fp32_scales(const Dims &d, const int32_t *k1, const double *ts_host, double cmax, const float *gtop_unscaled,
                 std::vector<int32_t> &scale);
void fp32_gtop(const Dims &d, const PhysParams &p, const std::vector<double> &blob, const double *top_host,
               std::vector<float> &gtop);
// Patch plan of one member: the kernel's work items.  Word layout of one patch table:
//   [ns, ni, kstart, patch index, 0, 0, 0, 0], nki[0..maxk+1] (interior slots with k1 <= k),
//   nkr[0..maxk+1] (ring slots with k1 <= k), goff[ns] (L*(i + NI*j) of each slot; interior
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
// One step of a batch: the transfer kernel over (member, patch, group) items, then the exact
// convective adjustment over (member, patch) items.  iso: some member has the isoneutral
// branch (selects the kernel instance that has it).
int fp32_launch(const MemberDesc *descs, const int4 *items, int nitems, const int4 *co_items, int nco,
                int max_slots, const long long *step_ctr, int rel, int *work, bool iso, cudaStream_t s);
int fp32_smem_bytes(int max_slots);
int fp32_export(const MemberDesc &md, const double *cur, double *rho, cudaStream_t s);
// re-target the fixed-point scales of `n` members after a step (stream order)
int fp32_rescale(const MemberDesc *descs, int n, cudaStream_t s);

void count_launches(uint64_t n);

}  // namespace gbgo
