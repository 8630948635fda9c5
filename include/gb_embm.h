/*
 * gb_embm.h -- C-ABI of the device-resident 2-D iterative implicit steppers: the EMBM
 * atmosphere step tstipa (src/embm/embm.f90:2039-2138) and the sea-ice transport step
 * tstipsic (src/goldsteinseaice/gold_seaice.f90:937-1058).
 *
 * Both advance two tracers on the (maxi, maxj) surface grid (air temperature and humidity;
 * ice height and area) by four Jacobi iterations of a Crank-Nicolson (cimp = 0.5) upwind
 * advection-diffusion step and an explicit conservative corrector, periodic in i.  Here the
 * tracers stay on the device between steps; a step is one kernel launch.  The arithmetic is
 * the reference's, operation for operation (no FMA contraction): results are bit-identical.
 *
 * Layouts are the reference's, column-major: tq(2, maxi, maxj) (tq(l,i,j) at
 * (l-1) + 2*((i-1) + maxi*(j-1))), uatm(2, maxi, maxj), pptn(maxi, maxj); the j-metric arrays
 * keep their Fortran bounds (rc(0:maxj) has maxj+1 entries starting at j = 0, dsv and rdsv
 * (1:maxj-1), rds(1:maxj)); diffa(2, 2, maxj).
 *
 * Return codes are those of gb_goldstein.h.  A handle is not thread-safe; every call returns
 * after its work has finished.
 */
#ifndef GB_EMBM_H
#define GB_EMBM_H

#include "gb_goldstein.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_ea gb_ea;

/* grids up to GB_EA_MAX_CELLS surface cells (a cluster of up to 8 thread blocks holds a
   tracer's grid; each block at most 4096 cells of ceil(maxj/8) rows, in shared memory) */
#define GB_EA_MAX_CELLS 32768

typedef struct {
    int32_t maxi, maxj;
} gb_ea_dims;

/* kind = GB_EA_SEAICE_EXPLICIT: tstepsic: as GB_EA_SEAICE, plus the area and height thresholds
   above which advection into a cell stops.
   kind = GB_EA_EMBM: tstipa.  dt = dtatm, betaz/betam (embm_lib.f90:98), diffmod0, ppmin,
   ppmax (embm_lib.f90:83, 112).
   kind = GB_EA_SEAICE: tstipsic.  dt = dtsic, diffsic, tsc (the source term is
   dtha(l,i,j)*tsc); betaz, betam, diffmod0, ppmin, ppmax unused. */
#define GB_EA_EMBM 0
#define GB_EA_SEAICE 1
#define GB_EA_SEAICE_EXPLICIT 2   /* tstepsic (gold_seaice.f90:844-929), the impsic = .FALSE. step */
typedef struct {
    int32_t kind;
    int32_t maxk;        /* sea ice: land iff k1(i,j) > maxk */
    double dt, dphi, rdphi;
    double betaz[2], betam[2];
    double diffmod0, ppmin, ppmax;
    double diffsic, tsc;
    double sica_thresh, sich_thresh;   /* tstepsic: par_sica_thresh, par_sich_thresh */
} gb_ea_params;

typedef struct {
    const double *rc;    /* rc(0:maxj) */
    const double *cv;    /* cv(0:maxj) */
    const double *dsv;   /* dsv(1:maxj-1) */
    const double *rdsv;  /* rdsv(1:maxj-1) */
    const double *rds;   /* rds(1:maxj) */
    const double *diffa; /* EMBM: diffa(2, 2, maxj); NULL for sea ice */
    const int32_t *k1;   /* sea ice: k1(0:maxi+1, 0:maxj+1) of the ocean; NULL for EMBM */
} gb_ea_grid;

int gb_ea_create(const gb_ea_dims *dims, const gb_ea_params *params, const gb_ea_grid *grid, int device, gb_ea **out);
void gb_ea_destroy(gb_ea *h);
/* tq (the new iterate's starting value) and tq1 (the previous step), (2, maxi, maxj) each */
int gb_ea_upload_state(gb_ea *h, const double *tq, const double *tq1);
/* EMBM: tqa (2, maxi, maxj), uatm (2, maxi, maxj), pptn (maxi, maxj).
   Sea ice: dtha (2, maxi, maxj) as `source`, the surface ocean velocities u(1:2, i, j) as
   `vel` (2, maxi, maxj) -- u(1,i,j) on the east face, u(2,i,j) on the north face; pptn NULL. */
int gb_ea_set_forcing(gb_ea *h, const double *source, const double *vel, const double *pptn);
/* EMBM: nsteps tstipa steps with the same forcing, each ending with tq1 = tq
   (embm.f90:2137).  Sea ice without post-processing: nsteps = 1, one tstipsic (or tstepsic);
   tq1 is left as it was, for the caller's step_seaice to post-process the ice and copy it
   (gold_seaice.f90:599-619).  Sea ice with post-processing (gb_ea_set_seaice_post): nsteps
   step_seaice steps with the same forcing, each the transport step followed by that
   post-processing on the device. */
int gb_ea_step(gb_ea *h, int32_t nsteps);

/* step_seaice's post-processing of each sea-ice step (gold_seaice.f90:599-619) on the ocean
   cells: varice(2) held in [0, 1]; where varice(1) < hmin the ice is removed with
   fx_delta = -varice(1)*rhoice*hlf*rdtdim and fw_delta += varice(1)*rhoio*rdtdim, after
   fw_delta = -rhoio*dtha(1); fw_delta is then converted by m2mm; varice1 = varice.  The
   constants are the reference's (gold_seaice.f90:262, 304; gold_seaice_lib.f90:33-34, 38). */
typedef struct {
    double rhoio, rhoice, hlf, hmin, rdtdim, m2mm;
} gb_ea_seaice_post;
/* Turn the post-processing on for the handle's following steps (post copied), or off (NULL).
   GB_GO_EINVAL for an EMBM handle.  Grids stepped together must agree on it. */
int gb_ea_set_seaice_post(gb_ea *h, const gb_ea_seaice_post *post);
/* fx_delta, fw_delta (maxi, maxj) of the last post-processed step: 0 on land and before the
   first post-processed step.  Either pointer may be NULL. */
int gb_ea_download_seaice_fluxes(gb_ea *h, double *fx_delta, double *fw_delta);
/* The same for n grids of one kind and shape on one device (an ensemble), in one launch:
   errors are reported on handles[0]. */
int gb_ea_step_many(gb_ea *const *handles, int32_t n, int32_t nsteps);
int gb_ea_download(gb_ea *h, double *tq, double *tq1);
/* Sea ice: the diagnostic split of the last tstipsic's ice change, variceth = tsc*dtsic*dtha
   (thermal) and varicedy = varice - varice1 - variceth (dynamical), (2, maxi, maxj) each, as
   gold_seaice.f90:1046-1056 sets them on the ocean cells; other cells keep their previous
   values (0 from creation, as initialise_seaice, gold_seaice.f90:329-330).  tstepsic (kind
   GB_EA_SEAICE_EXPLICIT) does not set them: they stay 0.  Either pointer may be NULL.
   GB_GO_EINVAL for an EMBM handle. */
int gb_ea_download_seaice_diag(gb_ea *h, double *variceth, double *varicedy);
const char *gb_ea_last_error(const gb_ea *h);

#ifdef __cplusplus
}
#endif

#endif
