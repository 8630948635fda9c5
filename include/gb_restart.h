/*
 * gb_restart.h -- C-ABI of the GOLDSTEIN restart files of a device-resident ocean.
 *
 * Replaces outm_netcdf(istep) (src/goldstein/goldstein_data.f90:153-354) and the file part of
 * inm_netcdf(lrestart_genie) (:10-149).  The reference writes the restart through the netCDF
 * library; here the file is encoded directly in the netCDF classic format (the published
 * format of Unidata's netCDF: big-endian header of dimensions, attributes and variables,
 * then each variable's data), variable for variable as outm_netcdf defines it:
 *
 *   dimensions nrecs = 1, longitude = maxi, latitude = maxj, depth = maxk
 *   float  longitude(longitude)   units "degrees_east",  long_name "longitude"  (nclon1)
 *   float  latitude(latitude)     units "degrees_north", long_name "latitude"   (nclat1)
 *   float  depth(depth)           ncdepth(maxk-k+1)
 *   int    ioffset, iyear, imonth, iday (nrecs) [, istep_ocn (nrecs) in a GUI restart]
 *   double temp, salinity, uvel, vvel (depth, latitude, longitude)
 *   double evap, late, sens (latitude, longitude)
 *
 * temp/salinity are ts(1:2, 1:maxi, 1:maxj, 1:maxk) times the reference's landmask (1 on every
 * level of a column with k1 <= maxk, else 0, :200-206); uvel/vvel are u(1:2, ...).  The writer
 * forms these four fields on the device from the ocean handle's current state, already in the
 * file's byte order, so a restart moves 32 bytes per cell to the host and nothing else of the
 * tracer state.  The file is CDF-1 (32-bit offsets), as NF90_CREATE(NF90_CLOBBER) makes it, or
 * CDF-2 when it does not fit in 2 GiB.  The reader accepts CDF-1 and CDF-2 files of any
 * numeric variable types (converted to double as nf90_get_var converts them); netCDF-4 (HDF5)
 * files need the netCDF library and are refused with GB_GO_EUNSUPPORTED.
 *
 * Arrays are column-major (i fastest): 3-D fields (maxi, maxj, maxk), 2-D fields (maxi, maxj).
 * Return codes are those of gb_goldstein.h; gb_rs_last_error() describes the last failure of
 * the calling thread.
 */
#ifndef GB_RESTART_H
#define GB_RESTART_H

#include "gb_goldstein.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The restart calendar of goldstein_data.f90: iyear_rest, imonth_rest, ioffset_rest, day_rest,
   and istep_ocn (written and read only in a GUI restart). */
typedef struct {
    int32_t iyear, imonth, ioffset, istep;
    double day;
} gb_rs_calendar;

/* outm_netcdf's write: the restart file of `ocean`'s current state at `path`.  nclon1 (maxi),
   nclat1 (maxj) and ncdepth (maxk) are the grid coordinates (goldstein.f90:1862-1926);
   evap, late, sens (maxi, maxj) the saved surface fluxes (NULL writes zeros).  iday is
   NINT(cal->day); gui != 0 adds istep_ocn = cal->istep, as a GUI restart does.  The calendar
   is not advanced: gb_rs_calendar_step follows, as in outm_netcdf. */
int gb_rs_write_goldstein(gb_go_handle *ocean, const char *path, const gb_rs_calendar *cal, int32_t gui,
                          const double *nclon1, const double *nclat1, const double *ncdepth,
                          const double *evap, const double *late, const double *sens);

/* The device part of gb_rs_write_goldstein alone: temp, salinity, uvel, vvel of `ocean`'s current
   state, each maxi*maxj*maxk big-endian doubles (the file's data of the four variables, back to
   back), written to the device buffer dev_out (4*maxi*maxj*maxk*8 bytes, 8-byte aligned).  The
   work is enqueued on the ocean handle's stream and the call returns without waiting, for
   callers that move the restart data themselves. */
int gb_rs_pack_goldstein(gb_go_handle *ocean, void *dev_out);

/* The same file from host fields already in file form: temp and salinity masked, the depth
   axis as written (depths1, bottom level first).  No device is used. */
int gb_rs_write_fields(const char *path, int32_t maxi, int32_t maxj, int32_t maxk, const gb_rs_calendar *cal,
                       int32_t gui, const double *lon, const double *lat, const double *depths1,
                       const double *temp, const double *salinity, const double *uvel, const double *vvel,
                       const double *evap, const double *late, const double *sens);

/* inm_netcdf's read: the fields of a restart file of this grid (any output pointer may be NULL).
   cal receives iyear, imonth, ioffset (as stored), istep (gui != 0) and day = iday; apply
   gb_rs_calendar_after_read for inm_netcdf's calendar update.  The caller places temp and
   salinity into ts(1:2, ...) and uvel/vvel into u and u1 (gb_go_upload_state,
   gb_go_set_velocity, gb_mo_upload_velocity), as inm_netcdf's assignments do. */
int gb_rs_read_goldstein(const char *path, int32_t maxi, int32_t maxj, int32_t maxk, int32_t gui,
                         gb_rs_calendar *cal, double *temp, double *salinity, double *uvel, double *vvel,
                         double *evap, double *late, double *sens);

/* The restart file name outm_netcdf forms: <dir>/goldstein_restart_<iyear>_<mm>_<dd>.nc with
   dd = NINT(day).  Returns the length written (without the NUL) or a negative code. */
int gb_rs_goldstein_name(const char *dir, const gb_rs_calendar *cal, char *out, int32_t out_len);

/* outm_netcdf's calendar update after its (optional) write (:188, :320-338): with
   iday = NINT(day) taken before the advance, day advances by yearlen / nyear days, returns to
   iday when within 1e-3 of it, and after day 31 rolls 30 days over into the next month (and
   after month 12 into the next year).  Call once per ocean step. */
void gb_rs_calendar_step(gb_rs_calendar *cal, double yearlen, int32_t nyear);

/* inm_netcdf's calendar update after its read (:70-85), on cal->day = iday as read:
   ioffset = MOD(ioffset, NINT(yearlen)), then day advances by one step of
   (86400 * yearlen / nyear) / 86400 days with the same re-anchoring and roll-over. */
void gb_rs_calendar_after_read(gb_rs_calendar *cal, double yearlen, int32_t nyear);

const char *gb_rs_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
