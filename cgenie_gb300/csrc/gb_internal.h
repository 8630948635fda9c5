// Internal definitions shared by the GOLDSTEIN GB300 kernels and the C-ABI.
//
// Device layout (one grid):
//   state buffers  ts[2]      (maxl, 0:maxi+1, 0:maxj+1, 0:maxk+1) FP64, the
//                             Fortran layout of ts/ts1, ping-ponged: a step reads
//                             buffer `cur` (the reference's ts1) and writes the other
//                             one (the reference's ts), so the reference's closing
//                             ts1 = ts copy (goldstein.f90:2423-2431) disappears.
//   ts_static/ts1_static      the uploaded ts/ts1: land cells, halo rows, level 0 and
//                             the forcing level keep their uploaded values exactly as
//                             the reference leaves them untouched.
//   top                       forcing level ts(:, :, :, maxk+1)
//   rho                       (0:maxi+1, 0:maxj+1, 0:maxk)
//   u                         (3, 0:maxi, 0:maxj, 1:maxk)
//   k1                        (0:maxi+1, 0:maxj+1) int32
//   metrics                   one blob; j-arrays hold maxj+2 entries and k-arrays maxk+2
//                             entries, both indexed by the Fortran index.
#pragma once

#include <cstddef>
#include <cstdint>

namespace gbgo {

// An NVTX range of the library's domain ("cgenie_gb300") for the lifetime of the object: the
// public calls open one named after the call (no-op unless a profiler is attached).
struct TraceRange {
    explicit TraceRange(const char *name);
    ~TraceRange();
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace gbgo

namespace gbgo {

constexpr int kMaxK = 64;

// Fortran-indexed metric pointers (device).
struct Metrics {
    const double *rc, *rc2, *cv, *cv2, *dsv, *rdsv, *ds, *rds;      // [0 .. maxj+1]
    const double *dz, *dza, *rdz, *rdza, *zro, *dt, *zw, *ssmax, *diffmax;  // [0 .. maxk+1]
    const double *mlddec, *mlddecd;                                 // [0 .. maxk+1] (imld = 1)
    const double *ediff1;                                           // (maxi, maxj, maxk-1)
    const int32_t *k1;                                              // (maxi+2, maxj+2)
};

struct Dims {
    int maxi, maxj, maxk, L;
    int NI, NJ;          // maxi+2, maxj+2
};

struct PhysParams {
    double diff1, diff2;
    double ec[5];
    double ediff0, ediffpow2, dsc;
    double dphi, rdphi;
    int ieos, iediff, ediffpow2i, iconv, diso;
    int imld;
    double mldpebuoycoeff;
};

// Arguments of one FP64 step launch.
struct StepArgs {
    Dims d;
    PhysParams p;
    Metrics m;
    const double *ts1;        // read buffer (old state)
    double *ts;               // write buffer (new state)
    const double *ts_static;  // uploaded ts: land / level-0 values
    const double *top;        // forcing level (L, NI, NJ)
    double *rho;
    const double *u;
    double *cost;
    int32_t *icosd;
    unsigned long long *diag;       // [0] dmax bits, [1] limps  (this step)
    unsigned long long *diag_next;  // zeroed by block 0 for the next step
    int tile_i, tile_j, tiles_i;
    // imld = 1 (mixed layer): ts at the start of the step (its surface level), wind mixing
    // energy, diagnostics mld/mldk and the per-column surface-layer energy (maxi, maxj)
    const double *ts_start;
    const double *mldketau;
    double *mld;
    int32_t *mldk;
    double *mldpe1;
};

__host__ __device__ inline size_t ts_index(const Dims &d, int l, int i, int j, int k)
{
    return (size_t)l + (size_t)d.L * ((size_t)i + (size_t)d.NI * ((size_t)j + (size_t)d.NJ * (size_t)k));
}
__host__ __device__ inline size_t u_index(const Dims &d, int c, int i, int j, int k)
{
    return (size_t)c + 3 * ((size_t)i + (size_t)(d.maxi + 1) * ((size_t)j + (size_t)(d.maxj + 1) * (size_t)(k - 1)));
}
__host__ __device__ inline size_t rho_index(const Dims &d, int i, int j, int k)
{
    return (size_t)i + (size_t)d.NI * ((size_t)j + (size_t)d.NJ * (size_t)k);
}

// Launchers (tstep_fp64.cu)
int launch_step_fp64(const StepArgs &a, void *stream);
void step_fp64_tile(int maxi, int maxj, int maxk, int nsm, int *tile_i, int *tile_j);
constexpr int kFp64TilesPerSm = 4;

// The device tracer state of a single-grid handle, for the routines that act on it between
// steps (the BIOGEM tracer coupling).  ts_static / ts1_static: the uploaded Fortran-layout
// arrays; ts_buf: the step's ping-pong buffers; `cur`: the current one, valid on the wet cells
// once steps_since_upload > 0 (before that the current ts is ts_static).
struct OceanState {
    Dims d;
    int precision;
    int device;
    void *stream;   // cudaStream_t
    double *ts_static, *ts1_static, *ts_buf[2];
    int cur;
    long long steps_since_upload;
    const int32_t *k1;   // device, (maxi+2, maxj+2)
    bool state_ready;
    bool *dry_zeroed;    // the interior cells that are land or below k1 hold 0 in ts_static and
                         // ts1_static (set by the coupling, cleared by an upload)
    const double *rho;   // (0:maxi+1, 0:maxj+1, 0:maxk), the last step's density
    double *u;           // (3, 0:maxi, 0:maxj, 1:maxk), the velocities the next step reads
    bool *vel_ready;
};
}  // namespace gbgo
struct gb_go_handle;
namespace gbgo {
int ocean_state(gb_go_handle *h, OceanState *out);
// the split-precision form keeps its state group-planar and forms rho on export: bring rho up to
// date with the current state (a no-op for the FP64 form)
int ocean_refresh_rho(gb_go_handle *h);
// the split-precision form's rho only (callers that read rho and not the tracers)
int ocean_refresh_rho_only(gb_go_handle *h);
// velocities written on the device: the split-precision form rebuilds its transfer
// coefficients from them (on the device; the first velocity field must come from the host)
int ocean_velocity_changed(gb_go_handle *h);
void count_launches(uint64_t n);   // kernels this library started (gb_go_kernel_launch_count)
// after the state arrays were rewritten on the device: the handle continues as after an upload
// (ts_buf[0] = ts1_static, ts_buf[1] = ts_static, step counters reset)
int ocean_state_reloaded(gb_go_handle *h);

#ifdef __CUDACC__
// c + n computed as n additions of 1.0 in round-to-nearest (co adds 1 to cost(i,j) per
// filled level, goldstein.f90:2759).  When c is integer-valued with |c| < 2^52 every partial
// sum is exact, so one addition gives the same double; otherwise they run one by one.
__device__ __forceinline__ double add_count_rn(double c, int n)
{
    if (n <= 0) return c;
    const long long b = __double_as_longlong(c);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    const long long frac = b & 0xfffffffffffffLL;
    const bool integral = ((unsigned long long)b << 1) == 0ull || (e >= 0 && e < 52 && (frac & ((1LL << (52 - e)) - 1)) == 0);
    if (integral) return __dadd_rn(c, (double)n);
    for (int f = 0; f < n; ++f) c = __dadd_rn(c, 1.0);
    return c;
}
#endif

}  // namespace gbgo
