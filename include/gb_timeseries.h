/*
 * gb_timeseries.h -- GOLDSTEIN time-series diagnostics of the device-resident ocean.
 *
 * Every itstp steps step_goldstein (src/goldstein/goldstein.f90:284-310) calls
 *   diag2(sums, avn, avs)   goldstein_diag.f90:10-71: the regional volume means of every
 *                           tracer (4 basins x 2 depth halves), the mean |d rho / dz| and the
 *                           RMS horizontal velocity, with the crash barrier avs >= 1e20;
 *   diagopsi(...)           goldstein_diag.f90:350-411: the meridional overturning
 *                           streamfunctions (global, Pacific, Atlantic) and the Pacific and
 *                           Atlantic extrema above level overdep;
 * and appends the .t, .s and .opsit records (formats 110 and 100).  Here both diagnostics
 * run on a gb_go handle's device state (either precision form), so no tracer array crosses
 * the host boundary for a time-series record: the host receives 8*maxl + 8 numbers.
 * Every sum is formed in the reference's loop order (one thread per sum), so the numbers are
 * the reference's bit for bit.
 */
#ifndef GB_TIMESERIES_H
#define GB_TIMESERIES_H

#include <stdint.h>
#include <stddef.h>

#include "gb_goldstein.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The basin definition of the diagnostics (goldstein_lib.f90:11-12, set by
 * initialise_goldstein at goldstein.f90:1139-1200 from the .bmask file or the land mask). */
typedef struct gb_ts_basins {
    const int32_t *ips, *ipf;   /* (1:maxj) first and last longitude of the Pacific per row */
    const int32_t *ias, *iaf;   /* (1:maxj) Atlantic; iaf < ias: the Atlantic wraps through i = maxi */
    int32_t jsf;                /* rows 1..jsf: the Southern Ocean region */
    int32_t overdep;            /* levels k <= overdep enter the overturning extrema */
} gb_ts_basins;

typedef struct gb_ts_handle gb_ts_handle;

/* Set up the diagnostics of a grid: the ordered cell list of each region, the region volumes
 * (computed once, as diag2's first call does), the wet-cell counts ntot and intot, and the
 * metrics and basin rows on `device`.  grid: the same struct gb_go_create takes (ds, dz, dza,
 * cv, dphi and k1 are read).  Errors: GB_GO_EINVAL for bad basin rows. */
int  gb_ts_create(const gb_go_dims *dims, const gb_go_grid *grid, const gb_ts_basins *basins,
                  int device, gb_ts_handle **out);
void gb_ts_destroy(gb_ts_handle *h);

/* diag2 and diagopsi of the ocean handle's current state, on the handle's stream; returns
 * after the copies.  sums[mo + 4*ndep + 8*(l-1) - 1] as diag2's sum (mo: 1 Pacific, 2
 * Atlantic, 3 other, 4 Southern Ocean; ndep 0 for the lower, 1 for the upper half of the
 * levels); ext = {ominp, omaxp, omina, omaxa}; iposa = the row and level of omaxa.  Any
 * pointer may be NULL.  opsi, opsip, opsia (each (0:maxj, 0:maxk), column-major) receive the
 * three streamfunctions when not NULL.  avs >= 1e20 is the reference's crash barrier
 * (write_status('ERRORED')): the caller decides. */
int  gb_ts_diagnose(gb_ts_handle *h, gb_go_handle *ocean, double *sums, double *avn, double *avs,
                    double *ext, int32_t *iposa, double *opsi, double *opsip, double *opsia);

/* The three records of one time-series line, as step_goldstein writes them: .t = FORMAT 110
 * (11e14.6) of time, sums(1:8), avn, avs; .s of time, sums(9:16), avn, avs; .opsit = FORMAT
 * 100 (5e14.6,2i5) of time, ext * opsisc, iposa.  Each line ends in a newline; len is the size
 * of each buffer (at least 160).  Returns GB_GO_EINVAL for short buffers or maxl < 2. */
int  gb_ts_format(double time, int32_t maxl, const double *sums, double avn, double avs, const double *ext,
                  const int32_t *iposa, double opsisc, char *t_line, char *s_line, char *opsit_line, int32_t len);

const char *gb_ts_last_error(const gb_ts_handle *h);

#ifdef __cplusplus
}
#endif
#endif /* GB_TIMESERIES_H */
