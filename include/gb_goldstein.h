/*
 * gb_goldstein.h -- C-ABI of the GB300 GOLDSTEIN ocean tracer timestep.
 *
 * This library replaces the body of the reference's `SUBROUTINE tstepo`
 * (src/goldstein/goldstein.f90:2280-2432) together with the routines it calls:
 * `tstepo_flux` (:2436-2642, including the `diso` isoneutral branch :2561-2624),
 * `co` (:2657-2777), `coshuffle` (:2781-2841), `eos` (:3048-3061) and `eosd`
 * (:3064-3082).  The reference routine takes no arguments and works on SAVE'd
 * module state declared in src/goldstein/goldstein_lib.f90:6-180; here that state
 * is passed once through plain C structs and pointers, and kept resident on the
 * GPU between calls.  A Fortran caller binds these symbols with ISO_C_BINDING
 * (`BIND(C, NAME=...)`, `TYPE(c_ptr), VALUE`), the same pattern the reference
 * already uses for its ITT shim (src/utils/itt_fortran.f90:1-44).
 *
 * Conventions
 * -----------
 *  - Every array argument is a pointer to the FIRST element of the Fortran array
 *    (its declared lower bound), column-major, REAL(8) = double, INTEGER = int32_t.
 *  - Index maps (i, j, k counted from the Fortran lower bound, halos included):
 *      ts(l,i,j,k), ts1(l,i,j,k): (maxl, 0:maxi+1, 0:maxj+1, 0:maxk+1)
 *          offset = (l-1) + maxl*(i + (maxi+2)*(j + (maxj+2)*k))
 *      u(c,i,j,k):   (3, 0:maxi, 0:maxj, 1:maxk)
 *          offset = (c-1) + 3*(i + (maxi+1)*(j + (maxj+1)*(k-1)))
 *      rho(i,j,k):   (0:maxi+1, 0:maxj+1, 0:maxk)
 *          offset = i + (maxi+2)*(j + (maxj+2)*k)
 *      k1(i,j):      (0:maxi+1, 0:maxj+1)      offset = i + (maxi+2)*j
 *      cost(i,j), icosd(i,j): (1:maxi, 1:maxj) offset = (i-1) + maxi*(j-1)
 *  - A column (i,j) is wet iff k1(i,j) <= maxk; level k=1 is the deepest and
 *    k=maxk the surface.  Rows j=0 and j=maxj+1 must be land, and k1 must be
 *    periodic in i (k1(0,j)=k1(maxi,j), k1(maxi+1,j)=k1(1,j)), as the reference
 *    enforces when it reads the .k1 file (goldstein.f90:1111-1118).
 *  - Return value: 0 on success, a negative GB_GO_E* code on failure;
 *    gb_go_errstr() turns it into text.  The reference aborts through
 *    `die` -> write_status('ERRORED') -> STOP (src/wrappers/genie_util.f90:14-30);
 *    the Fortran shim is expected to do that on a non-zero return.
 *  - Ownership: the caller owns every host array; the library copies what it
 *    needs during the call and never keeps or frees a caller pointer.
 *  - A handle is not thread-safe; use one handle per host thread.
 */
#ifndef GB_GOLDSTEIN_H
#define GB_GOLDSTEIN_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_GO_ABI_VERSION 2

/* Error codes. */
#define GB_GO_OK            0
#define GB_GO_EINVAL       -1   /* bad argument (NULL pointer, size, flag value) */
#define GB_GO_EUNSUPPORTED -2   /* option combination not implemented (e.g. GB_GO_FP32FLUX with per-level dt) */
#define GB_GO_ECUDA        -3   /* a CUDA runtime call failed */
#define GB_GO_ENOMEM       -4   /* device allocation failed or over the memory budget */
#define GB_GO_ENOTREADY    -5   /* state/velocity not uploaded yet */
#define GB_GO_EDEVICE      -6   /* a kernel reported an error status (see detail) */
#define GB_GO_ERANGE       -7   /* a size exceeds a compiled-in limit */
#define GB_GO_ENONFINITE   -8   /* non-finite tracer value detected (blow-up guard) */

/* Precision of the flux arithmetic. */
#define GB_GO_FP64         0    /* plain form: every operation in IEEE double, no FMA
                                   contraction, in the reference order; bit-identical to
                                   the reference arithmetic */
#define GB_GO_FP32FLUX     1    /* face fluxes in FP32, tracer state and its update in
                                   FP64; inventories in compensated FP64 */

/* Largest supported vertical level count and tracer count. */
#define GB_GO_MAX_K        64
#define GB_GO_MAX_L        128

typedef struct gb_go_dims {
    int32_t maxi;   /* longitudes (dim_GOLDSTEINNLONS) */
    int32_t maxj;   /* latitudes  (dim_GOLDSTEINNLATS) */
    int32_t maxk;   /* levels     (dim_GOLDSTEINNLEVS), 2..GB_GO_MAX_K */
    int32_t maxl;   /* tracers    (dim_GOLDSTEINNTRACS), 2..GB_GO_MAX_L; l=1 is T, l=2 is S */
} gb_go_dims;

/* Namelist-derived switches and coefficients read by tstepo
 * (ini_gold_nml, goldstein.f90:596-622; defaults goldstein-defaults.nml). */
typedef struct gb_go_params {
    double  diff[2];      /* nondimensional diffusivities after goldstein.f90:1406-1407 */
    double  ec[5];        /* equation-of-state coefficients, goldstein.f90:1063-1075 */
    double  ediff0;       /* nondimensional, after ediff (goldstein.f90:2946) */
    double  ediffpow2;    /* exponent used when ediffpow2i is neither 0, 1 nor 2 */
    double  dsc;          /* depth scale (goldstein_lib.f90:51), used by co when iconv=1 */
    int32_t ieos;         /* 0: no thermobaricity; 1: ec(5)*t*z term */
    int32_t iediff;       /* 0: uniform diff(2); 1 or 2: ediff1/diffmax profile */
    int32_t ediffpow2i;   /* 0, 1, 2 or any other value for the general power */
    int32_t iconv;        /* 0: co only; 1: coshuffle before co */
    int32_t imld;         /* 0, or 1: Kraus-Turner mixed layer after co (goldstein.f90:2294-2390,
                             3337-3442); both precision forms, single grids and ensembles */
    int32_t diso;         /* non-zero: isoneutral (Redi) branch on */
    int32_t precision;    /* GB_GO_FP64 or GB_GO_FP32FLUX */
    int32_t reserved;     /* must be 0 */
    double  mldpebuoycoeff;  /* imld = 1: efficiency of convective energy release (ini_gold_nml,
                                default 0.15, goldstein.f90:2354-2356) */
} gb_go_params;

/* Grid metrics (goldstein.f90:908-1076, 2057-2070).  Lower bounds in brackets. */
typedef struct gb_go_grid {
    const double  *rc, *rc2, *cv;        /* [0:maxj]   */
    const double  *cv2, *dsv, *rdsv;     /* [1:maxj-1] */
    const double  *ds, *rds;             /* [1:maxj]   */
    const double  *dz, *dza, *rdz, *rdza, *zro, *dt;  /* [1:maxk] */
    const double  *zw;                   /* [0:maxk]   */
    const double  *ssmax;                /* [1:maxk-1], read when diso != 0 */
    const double  *ediff1;               /* (1:maxi,1:maxj,1:maxk-1), read when iediff is 1 or 2 */
    const double  *diffmax;              /* [1:maxk], read when iediff is 1 or 2 */
    const int32_t *k1;                   /* (0:maxi+1, 0:maxj+1) */
    double dphi, rdphi;
    const double  *mlddec, *mlddecd;     /* [1:maxk], read when imld = 1 (goldstein.f90:1678-1685) */
    const double  *mldketau;             /* (1:maxi,1:maxj) wind mixing energy, read when imld = 1
                                            (goldstein.f90:120-140); gb_go_set_mld_wind updates it */
} gb_go_grid;

typedef struct gb_go_handle gb_go_handle;

/* ---- single grid: drop-in for `CALL tstepo` (goldstein.f90:235) ------------- */

/* Validate the configuration, copy grid/params to the device, allocate resident
 * state.  `device` selects the CUDA device (-1 = current). */
int  gb_go_create(const gb_go_dims *dims, const gb_go_params *params,
                  const gb_go_grid *grid, int device, gb_go_handle **out);
void gb_go_destroy(gb_go_handle *h);

/* Use this CUDA stream (a cudaStream_t; NULL = the handle's own stream) for
 * every later call on the handle. */
int  gb_go_set_stream(gb_go_handle *h, void *cuda_stream);

/* Upload ts, ts1 (full halo'd arrays, including the surface-forcing slot
 * ts(:,:,:,maxk+1)) and rho.  Replaces the per-step copy-in at
 * goldstein.f90:176-187; call it at coupling intervals only. */
int  gb_go_upload_state(gb_go_handle *h, const double *ts, const double *ts1,
                        const double *rho);

/* Surface forcing slot ts(1:maxl, 0:maxi+1, 0:maxj+1, maxk+1) (one contiguous
 * level of ts), written by step_goldstein at goldstein.f90:167-170. */
int  gb_go_set_forcing(gb_go_handle *h, const double *ts_top);

/* Velocities u(3, 0:maxi, 0:maxj, 1:maxk) from velc (goldstein.f90:3668-3678). */
int  gb_go_set_velocity(gb_go_handle *h, const double *u);

/* Convection diagnostics cost(maxi,maxj) (passed back in from BIOGEM at
 * goldstein.f90:99) and icosd(maxi,maxj).  Either may be NULL. */
int  gb_go_set_diag(gb_go_handle *h, const double *cost, const int32_t *icosd);

/* Advance `nsteps` tracer timesteps on the device (tstepo repeated). */
int  gb_go_tstepo(gb_go_handle *h, int32_t nsteps);

/* Copy the state back (the copy-out at goldstein.f90:443-450), at coupling
 * intervals.  Any pointer may be NULL to skip that array.  dmax and limps
 * are the diagnostics of the last step (goldstein.f90:2459, 2598-2608). */
int  gb_go_download(gb_go_handle *h, double *ts, double *ts1, double *rho,
                    double *cost, int32_t *icosd, double *dmax, int32_t *limps);

/* imld = 1: replace the wind mixing energy mldketau(1:maxi,1:maxj), which the reference
 * recomputes from the wind stress at goldstein.f90:120-140. */
int  gb_go_set_mld_wind(gb_go_handle *h, const double *mldketau);

/* imld = 1: the mixed-layer diagnostics of the last step, mld(maxi,maxj) (depth, <= 0) and
 * mldk(maxi,maxj) (index of the level holding it), written by tstepo for wet columns
 * (goldstein.f90:2371-2386, 3337-3442); 0 where never written.  Either may be NULL. */
int  gb_go_download_mld(gb_go_handle *h, double *mld, int32_t *mldk);

/* Per-tracer inventory sum over wet cells of ts(l,i,j,k)*ds(j)*dz(k)
 * (the weighting of the reference's conservation diagnostic,
 * goldstein.f90:458-478), computed on the device in FP64 with compensated
 * (Neumaier) summation.  `out` has maxl entries. */
int  gb_go_inventory(gb_go_handle *h, double *out);

/* gb_go_inventory without any device allocation: the same kernels and result, with their
 * scratch in a static device array of the library (64 x 2 partial sums per tracer and the
 * results, 8256 doubles, held by every device that loads the library until the process
 * exits).  No counterpart in the reference.  It serves callers that cannot allocate device
 * memory at this point of their time loop: a host model whose device memory is reserved
 * up front by a pool it does not control, or one that runs other work on other streams
 * and cannot afford cudaMalloc/cudaFree, which may synchronise the whole device.
 * - at most 64 tracers: a handle with more returns GB_GO_ERANGE;
 * - the scratch address is looked up once per device when a handle is created
 *   (cudaGetSymbolAddress);
 * - the call is synchronous: it copies the sums into `out` and waits for the handle's
 *   stream before it returns;
 * - every scratch entry is written before it is read (nothing needs to start at zero);
 * - the scratch is shared by all handles of a device: calls that overlap in time (other
 *   threads, or handles on different streams) race and must be serialised by the caller. */
int  gb_go_inventory_noalloc(gb_go_handle *h, double *out);

/* Wait for all work queued on the handle's stream. */
int  gb_go_sync(gb_go_handle *h);

/* Text for an error code; the handle's last detailed message. */
const char *gb_go_errstr(int code);
const char *gb_go_last_error(const gb_go_handle *h);

/* Number of CUDA kernels this library launched in this process (all handles). */
uint64_t gb_go_kernel_launch_count(void);

/* ---- ensembles: many independent grids advanced by one batched launch -------
 * No counterpart in the reference (a single serial run).  Members may differ in
 * every dimension and parameter; they are packed into one work list and stepped
 * together by a persistent kernel.  Members can be added and removed between
 * steps (continuous batching). */

typedef struct gb_ens gb_ens;

typedef struct gb_ens_tuning {
    int32_t tile_i, tile_j;   /* columns per work item (0 = autotuned default) */
    int32_t ctas_per_sm;      /* at most this many persistent CTAs per SM for the transfer
                                 kernels (0 = as many as fit) */
    int32_t use_graph;        /* capture a multi-step launch in a CUDA graph */
    int32_t packing;          /* order of the work items in the launch (member packing):
                                 GB_ENS_PACK_MEMBERS, GB_ENS_PACK_ITEMS or GB_ENS_PACK_ROUND_ROBIN */
    int32_t co_form;          /* convective adjustment of the maxk <= 32, ieos = 0 columns:
                                 GB_ENS_CO_AUTO, GB_ENS_CO_WARP or GB_ENS_CO_TWO_PHASE */
} gb_ens_tuning;

/* Member packing: members by decreasing work, each member's patches together and a patch's
 * tracer groups together (neighbouring items share coefficients and ring columns in L2) */
#define GB_ENS_PACK_MEMBERS     0
/* work items by decreasing cost over the whole batch (longest first, the shortest tail) */
#define GB_ENS_PACK_ITEMS       1
/* the n-th patch of every member, then the (n+1)-th (DRAM traffic spread over members) */
#define GB_ENS_PACK_ROUND_ROBIN 2

/* The adjustment's form: one warp per listed column (small batches), or two phases (a lane per
 * column for the decisions on T and S, a lane per column and tracer replaying the logged merges;
 * large batches).  AUTO: two phases from GB_ENS_CO_TWO_PHASE_MIN listable (wet) columns in the
 * batch.  Every form gives the same results bit for bit. */
#define GB_ENS_CO_AUTO          0
#define GB_ENS_CO_WARP          1
#define GB_ENS_CO_TWO_PHASE     2
#define GB_ENS_CO_TWO_PHASE_MIN 100000

int  gb_ens_create(int device, size_t hbm_budget_bytes, gb_ens **out);
void gb_ens_destroy(gb_ens *e);
int  gb_ens_set_tuning(gb_ens *e, const gb_ens_tuning *t);
int  gb_ens_set_stream(gb_ens *e, void *cuda_stream);

/* Bytes of device memory one member of this shape needs. */
size_t gb_ens_member_bytes(const gb_go_dims *dims, const gb_go_params *params);

/* Add a member: copies grid/params and the initial ts (full halo'd array,
 * also used as ts1), u and forcing slot; returns its id in *member_id.
 * GB_GO_ENOMEM when it does not fit in the budget.  Several host threads may call
 * it at once (each member's host preparation runs in parallel, its device part one
 * member at a time); no other gb_ens_* call on the ensemble may overlap them. */
int  gb_ens_add(gb_ens *e, const gb_go_dims *dims, const gb_go_params *params,
                const gb_go_grid *grid, const double *ts, const double *u,
                int32_t *member_id);
/* gb_ens_add for n members in one call: dims[q], params[q], grids[q], ts[q], u[q] describe
 * member q, whose id goes to ids[q].  The host preparation of the members runs on up to 16
 * threads, their device set-up (one allocation each, the coefficients and fixed-point scales
 * built on the device) is queued on the ensemble's stream, and the call returns after one
 * synchronisation (the caller's arrays are then no longer needed).  ts and u in memory from
 * gb_ens_host_alloc are read by the device directly, from the start of the call (the transfer
 * overlaps the host preparation); other arrays take one copy call each.  All or nothing: on
 * an error no member of the call is admitted. */
int  gb_ens_add_many(gb_ens *e, int32_t n, const gb_go_dims *dims, const gb_go_params *params,
                     const gb_go_grid *grids, const double *const *ts, const double *const *u,
                     int32_t *ids);
int  gb_ens_remove(gb_ens *e, int32_t member_id);

/* Host memory for the arrays of the ensemble calls: page-locked and mapped into the devices'
 * address space (cudaHostAlloc, mapped and portable).  Arrays that lie inside one such
 * allocation are read (ts and u of gb_ens_add_many) and written (ts, rho and cost of
 * gb_ens_download_many) by the device directly, in one batched kernel per call, instead of
 * one copy call per array.  Other host memory is copied as before.  gb_ens_host_free takes
 * the pointer gb_ens_host_alloc returned (GB_GO_EINVAL otherwise); the caller frees only
 * memory that no call in progress uses. */
int  gb_ens_host_alloc(size_t bytes, void **out);
int  gb_ens_host_free(void *p);

/* Advance every active member by `nsteps` steps. */
int  gb_ens_step(gb_ens *e, int32_t nsteps);

/* Advance only members whose remaining-step counter is positive, decrementing
 * it; members reaching zero stop advancing.  Used by the serving loop. */
int  gb_ens_set_remaining(gb_ens *e, int32_t member_id, int64_t steps);
int  gb_ens_step_remaining(gb_ens *e, int32_t nsteps);
int  gb_ens_remaining(gb_ens *e, int32_t member_id, int64_t *steps);

int  gb_ens_download(gb_ens *e, int32_t member_id, double *ts, double *rho,
                     double *cost);
/* gb_ens_download on the CUDA stream `cuda_stream` (NULL = the ensemble's), ordered
 * after the work queued on the ensemble's stream.  Several host threads may call it at
 * once for different members, each with its own stream, so that the copies overlap; no
 * other gb_ens_* call on the ensemble may overlap them. */
int  gb_ens_download_stream(gb_ens *e, int32_t member_id, void *cuda_stream, double *ts,
                            double *rho, double *cost);
/* gb_ens_download for n members at once: one kernel forms every member's arrays, their copies
 * are queued on the ensemble's stream behind the steps, and the call returns after one
 * synchronisation.  ts[q], rho[q], cost[q] receive member ids[q] (any of the three pointer
 * arrays, or entries of them, may be NULL).  Destinations in memory from gb_ens_host_alloc are
 * written by one scatter kernel for the whole call; other destinations take one copy call each. */
int  gb_ens_download_many(gb_ens *e, int32_t n, const int32_t *ids, double *const *ts, double *const *rho,
                          double *const *cost);
/* Members with imld = 1 (the Kraus-Turner mixed layer, run in FP64 after the convective
 * adjustment of every wet column): the wind mixing energy mldketau (maxi*maxj, Fortran
 * (1:maxi, 1:maxj)) used from the next step on, as gb_go_set_mld_wind; and the mixed-layer depth
 * and level of every column, as gb_go_download_mld.  GB_GO_EINVAL for a member with imld = 0. */
int  gb_ens_set_mld_wind(gb_ens *e, int32_t member_id, const double *mldketau);
int  gb_ens_download_mld(gb_ens *e, int32_t member_id, double *mld, int32_t *mldk);
int  gb_ens_inventory(gb_ens *e, int32_t member_id, double *out);
/* The member's status word: bit 0 (1) a non-finite tracer value; bit 1 (2) a scaled transfer
 * beyond the fixed-point range; bit 2 (4) the convective adjustment did not complete (a full
 * column list or slot map, or a decision walk past its bound: none can happen with the sizes
 * the library allocates, so it marks a fault).  0: healthy.  Bits are sticky; the other members
 * of the batch are unaffected. */
int  gb_ens_status(gb_ens *e, int32_t member_id, int32_t *status);
int  gb_ens_sync(gb_ens *e);
int  gb_ens_count(gb_ens *e, int32_t *active, size_t *bytes_in_use);
const char *gb_ens_last_error(const gb_ens *e);

#ifdef __cplusplus
}
#endif
#endif /* GB_GOLDSTEIN_H */
