/*
 * gb_biogem.h -- C-ABI of the device-resident BIOGEM tracer coupling.
 *
 * Replaces SUBROUTINE biogem_tracercoupling(dum_ts, dum_ts1) (src/biogem/biogem.f90:1885-2077),
 * called as biogem_tracercoupling(go_ts, go_ts1) from biogem_tracercoupling_wrapper
 * (src/wrappers/genie_loop_wrappers.f90:318-322) once per BIOGEM interval (src/genie.f90:360-381).
 * The routine salinity-normalises the circulation-updated GOLDSTEIN tracers into BIOGEM's ocean
 * tracer field, adds BIOGEM's increments (vdocn, vdbio_part), rescales the biogeochemical
 * inventories and the cell masses with the change of mean salinity, and writes the result back
 * into go_ts and go_ts1.  Here the GOLDSTEIN tracers are the device state of a gb_go handle
 * (either form) and BIOGEM's vector fields stay on the same device, so no tracer array crosses
 * the host boundary at a coupling.
 *
 * Vector form (src/biogem/biogem_lib.f90:1056-1081, 1335-1410): the wet columns of
 * goldstein_k1 (k1(i,j) <= n_k) numbered n = 1..n_vocn with i outer and j inner.  A field
 * vocn(n)%mk(l,k) crosses this boundary packed column-major as (n_l_ocn, n_k, n_vocn), a cell
 * property vphys_ocn(n)%mk(ipo,k) as (n_k, n_vocn).  Levels below k1 are ignored on input and
 * written as 0 on output.
 *
 * Return codes are those of gb_goldstein.h (0 = ok, negative = error).  A handle is not
 * thread-safe; its calls run on the stream of the gb_go handle they are given (coupling) or
 * on their own stream (upload, download), and each returns after its work has finished.
 */
#ifndef GB_BIOGEM_H
#define GB_BIOGEM_H

#include "gb_goldstein.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_bg gb_bg;

/* Sizes: n_i, n_j, n_k (biogem_lib.f90 n_i, n_j, n_k = GOLDSTEIN maxi, maxj, maxk),
   n_l_ocn ocean tracers (T, S, then the biogeochemical tracers; = GOLDSTEIN maxl),
   n_l_sed particulate tracers of vbio_part (may be 0). */
typedef struct {
    int32_t n_i, n_j, n_k;
    int32_t n_l_ocn, n_l_sed;
    int32_t pad;
} gb_bg_dims;

/* ts_offset = tstoocn_offset(1:2) (biogem.f90:283-285: const_zeroC and goldstein_saln0);
   force_ts = ctrl_force_GOLDSTEInTS (biogem_lib.f90:57, used at biogem.f90:2005). */
typedef struct {
    double ts_offset[2];
    int32_t force_ts;
    int32_t pad;
} gb_bg_params;

/* k1: goldstein_k1(1:n_i, 1:n_j), column-major (i fastest).  device: CUDA ordinal. */
int gb_bg_create(const gb_bg_dims *dims, const gb_bg_params *params, const int32_t *k1, int device, gb_bg **out);
void gb_bg_destroy(gb_bg *h);
/* n_vocn: the number of wet columns (the vector length) */
int32_t gb_bg_columns(const gb_bg *h);

/* BIOGEM's state: vocn (n_l_ocn, n_k, n_vocn); the cell masses vphys_ocn(:)%mk(ipo_M,:),
   volumes (ipo_V) and reciprocal masses (ipo_rM), each (n_k, n_vocn); vbio_part
   (n_l_sed, n_k, n_vocn; NULL when n_l_sed = 0). */
int gb_bg_upload(gb_bg *h, const double *vocn, const double *mass, const double *volume, const double *rmass,
                 const double *vbio_part);
/* The increments of the interval: vdocn (n_l_ocn, n_k, n_vocn) and vdbio_part
   (n_l_sed, n_k, n_vocn; NULL when n_l_sed = 0). */
int gb_bg_set_increments(gb_bg *h, const double *vdocn, const double *vdbio_part);
/* biogem_tracercoupling(go_ts, go_ts1) on the current state of `ocean` (a gb_go handle of the
   same n_i, n_j, n_k and maxl = n_l_ocn, with its state uploaded).  The split-precision form's
   state is exported to Fortran layout first and re-imported afterwards (its fixed-point scales
   are kept and follow the state through the steps' rescaling).
   Afterwards the handle's ts and ts1 hold the coupled tracers on every interior cell (0 on
   land and below k1) and ts1 its periodic i-halo, as step_goldstein's copy-in and boundary
   conditions (src/goldstein/goldstein.f90:176-187) leave them before the next tstepo. */
int gb_bg_tracercoupling(gb_bg *h, gb_go_handle *ocean);
/* BIOGEM's state after the coupling (any pointer may be NULL). */
int gb_bg_download(gb_bg *h, double *vocn, double *mass, double *rmass, double *vbio_part);
const char *gb_bg_last_error(const gb_bg *h);

#ifdef __cplusplus
}
#endif

#endif
