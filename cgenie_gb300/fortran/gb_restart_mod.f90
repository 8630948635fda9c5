! ISO_C_BINDING interfaces to the GOLDSTEIN restart files (include/gb_restart.h) of
! libgb_goldstein.so, in the binding style of gb_goldstein_mod.f90.
!
! Drop-in use (sketch):
!   - outm_netcdf(istep) (src/goldstein/goldstein_data.f90:153-354): when MOD(istep, iwstp) == 0
!     (or a GUI restart is due) form the name with gb_rs_goldstein_name(dirnetout, cal, ...) and
!     CALL gb_rs_write_goldstein(goh, name, cal, gui, nclon1, nclat1, ncdepth, evap_save2,
!     late_save2, sens_save2); then, every call, gb_rs_calendar_step(cal, yearlen, nyear).
!     The tracers stay on the device in the gb_go handle.
!   - inm_netcdf (:10-149): gb_rs_read_goldstein(filenetin, maxi, maxj, maxk, gui, cal, temp,
!     salinity, uvel, vvel, evap, late, sens), gb_rs_calendar_after_read(cal, yearlen, nyear),
!     then the assignments of :89-93 and the uploads of gb_goldstein_mod.
!   Strings cross as NUL-terminated character arrays (TRIM(name)//C_NULL_CHAR).
!
! Not compiled in this repository (no Fortran compiler on the build machines); the same
! entry points are exercised from C via ctypes in tests/.
MODULE gb_restart_c
  USE, INTRINSIC :: ISO_C_BINDING
  IMPLICIT NONE

  TYPE, BIND(C) :: gb_rs_calendar
     INTEGER(C_INT32_T) :: iyear, imonth, ioffset, istep   ! iyear_rest, imonth_rest, ioffset_rest, istep_ocn
     REAL(C_DOUBLE) :: day                                 ! day_rest
  END TYPE gb_rs_calendar

  INTERFACE
     FUNCTION gb_rs_write_goldstein(ocean, path, cal, gui, nclon1, nclat1, ncdepth, evap, late, sens) &
          BIND(C, NAME='gb_rs_write_goldstein')
       IMPORT :: C_INT, C_INT32_T, C_PTR, C_CHAR, gb_rs_calendar
       TYPE(C_PTR), VALUE :: ocean
       CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*)
       TYPE(gb_rs_calendar), INTENT(IN) :: cal
       INTEGER(C_INT32_T), VALUE :: gui
       TYPE(C_PTR), VALUE :: nclon1, nclat1, ncdepth, evap, late, sens
       INTEGER(C_INT) :: gb_rs_write_goldstein
     END FUNCTION gb_rs_write_goldstein

     FUNCTION gb_rs_read_goldstein(path, maxi, maxj, maxk, gui, cal, temp, salinity, uvel, vvel, evap, late, sens) &
          BIND(C, NAME='gb_rs_read_goldstein')
       IMPORT :: C_INT, C_INT32_T, C_PTR, C_CHAR, gb_rs_calendar
       CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*)
       INTEGER(C_INT32_T), VALUE :: maxi, maxj, maxk, gui
       TYPE(gb_rs_calendar), INTENT(INOUT) :: cal
       TYPE(C_PTR), VALUE :: temp, salinity, uvel, vvel, evap, late, sens
       INTEGER(C_INT) :: gb_rs_read_goldstein
     END FUNCTION gb_rs_read_goldstein

     FUNCTION gb_rs_goldstein_name(dir, cal, out, out_len) BIND(C, NAME='gb_rs_goldstein_name')
       IMPORT :: C_INT, C_INT32_T, C_CHAR, gb_rs_calendar
       CHARACTER(KIND=C_CHAR), INTENT(IN) :: dir(*)
       TYPE(gb_rs_calendar), INTENT(IN) :: cal
       CHARACTER(KIND=C_CHAR), INTENT(OUT) :: out(*)
       INTEGER(C_INT32_T), VALUE :: out_len
       INTEGER(C_INT) :: gb_rs_goldstein_name
     END FUNCTION gb_rs_goldstein_name

     SUBROUTINE gb_rs_calendar_step(cal, yearlen, nyear) BIND(C, NAME='gb_rs_calendar_step')
       IMPORT :: C_INT32_T, C_DOUBLE, gb_rs_calendar
       TYPE(gb_rs_calendar), INTENT(INOUT) :: cal
       REAL(C_DOUBLE), VALUE :: yearlen
       INTEGER(C_INT32_T), VALUE :: nyear
     END SUBROUTINE gb_rs_calendar_step

     SUBROUTINE gb_rs_calendar_after_read(cal, yearlen, nyear) BIND(C, NAME='gb_rs_calendar_after_read')
       IMPORT :: C_INT32_T, C_DOUBLE, gb_rs_calendar
       TYPE(gb_rs_calendar), INTENT(INOUT) :: cal
       REAL(C_DOUBLE), VALUE :: yearlen
       INTEGER(C_INT32_T), VALUE :: nyear
     END SUBROUTINE gb_rs_calendar_after_read
  END INTERFACE
END MODULE gb_restart_c
