! ISO_C_BINDING interface to libgb_goldstein.so (include/gb_goldstein.h) and a
! drop-in body for the reference's `SUBROUTINE tstepo`
! (src/goldstein/goldstein.f90:2280-2432), written in the binding style the
! reference already uses for its ITT shim (src/utils/itt_fortran.f90:1-44).
!
! Usage in goldstein.f90 (sketch):
!   - at the end of initialise_goldstein: CALL gb_tstepo_init()
!   - replace the body of tstepo with:     CALL gb_tstepo_step()
!   - at coupling intervals (before go_ts is exported):  CALL gb_tstepo_sync_out()
!   - after BIOGEM rewrites go_ts/go_ts1:                 CALL gb_tstepo_sync_in()
!
! Not compiled in this repository (no Fortran compiler on the build machines);
! the same entry points are exercised from C via ctypes in tests/.
MODULE gb_goldstein_c
  USE, INTRINSIC :: ISO_C_BINDING
  IMPLICIT NONE

  TYPE, BIND(C) :: gb_go_dims
     INTEGER(C_INT32_T) :: maxi, maxj, maxk, maxl
  END TYPE gb_go_dims

  TYPE, BIND(C) :: gb_go_params
     REAL(C_DOUBLE) :: diff(2)
     REAL(C_DOUBLE) :: ec(5)
     REAL(C_DOUBLE) :: ediff0, ediffpow2, dsc
     INTEGER(C_INT32_T) :: ieos, iediff, ediffpow2i, iconv, imld, diso, precision, reserved
     REAL(C_DOUBLE) :: mldpebuoycoeff
  END TYPE gb_go_params

  TYPE, BIND(C) :: gb_go_grid
     TYPE(C_PTR) :: rc, rc2, cv, cv2, dsv, rdsv, ds, rds
     TYPE(C_PTR) :: dz, dza, rdz, rdza, zro, dt, zw, ssmax, ediff1, diffmax
     TYPE(C_PTR) :: k1
     REAL(C_DOUBLE) :: dphi, rdphi
     TYPE(C_PTR) :: mlddec, mlddecd, mldketau
  END TYPE gb_go_grid

  INTEGER(C_INT32_T), PARAMETER :: GB_GO_FP64 = 0, GB_GO_FP32FLUX = 1

  INTERFACE
     FUNCTION gb_go_create(dims, params, grid, device, handle) BIND(C, NAME='gb_go_create')
       IMPORT :: C_INT, C_PTR, gb_go_dims, gb_go_params, gb_go_grid
       TYPE(gb_go_dims), INTENT(IN) :: dims
       TYPE(gb_go_params), INTENT(IN) :: params
       TYPE(gb_go_grid), INTENT(IN) :: grid
       INTEGER(C_INT), VALUE :: device
       TYPE(C_PTR), INTENT(OUT) :: handle
       INTEGER(C_INT) :: gb_go_create
     END FUNCTION gb_go_create

     SUBROUTINE gb_go_destroy(handle) BIND(C, NAME='gb_go_destroy')
       IMPORT :: C_PTR
       TYPE(C_PTR), VALUE :: handle
     END SUBROUTINE gb_go_destroy

     FUNCTION gb_go_upload_state(handle, ts, ts1, rho) BIND(C, NAME='gb_go_upload_state')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, ts, ts1, rho
       INTEGER(C_INT) :: gb_go_upload_state
     END FUNCTION gb_go_upload_state

     FUNCTION gb_go_set_forcing(handle, ts_top) BIND(C, NAME='gb_go_set_forcing')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, ts_top
       INTEGER(C_INT) :: gb_go_set_forcing
     END FUNCTION gb_go_set_forcing

     FUNCTION gb_go_set_velocity(handle, u) BIND(C, NAME='gb_go_set_velocity')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, u
       INTEGER(C_INT) :: gb_go_set_velocity
     END FUNCTION gb_go_set_velocity

     FUNCTION gb_go_set_diag(handle, cost, icosd) BIND(C, NAME='gb_go_set_diag')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, cost, icosd
       INTEGER(C_INT) :: gb_go_set_diag
     END FUNCTION gb_go_set_diag

     FUNCTION gb_go_tstepo(handle, nsteps) BIND(C, NAME='gb_go_tstepo')
       IMPORT :: C_INT, C_INT32_T, C_PTR
       TYPE(C_PTR), VALUE :: handle
       INTEGER(C_INT32_T), VALUE :: nsteps
       INTEGER(C_INT) :: gb_go_tstepo
     END FUNCTION gb_go_tstepo

     FUNCTION gb_go_download(handle, ts, ts1, rho, cost, icosd, dmax, limps) BIND(C, NAME='gb_go_download')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, ts, ts1, rho, cost, icosd, dmax, limps
       INTEGER(C_INT) :: gb_go_download
     END FUNCTION gb_go_download

     FUNCTION gb_go_inventory(handle, out) BIND(C, NAME='gb_go_inventory')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, out
       INTEGER(C_INT) :: gb_go_inventory
     END FUNCTION gb_go_inventory

     FUNCTION gb_go_inventory_noalloc(handle, out) BIND(C, NAME='gb_go_inventory_noalloc')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, out
       INTEGER(C_INT) :: gb_go_inventory_noalloc
     END FUNCTION gb_go_inventory_noalloc

     FUNCTION gb_go_set_mld_wind(handle, mldketau) BIND(C, NAME='gb_go_set_mld_wind')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, mldketau
       INTEGER(C_INT) :: gb_go_set_mld_wind
     END FUNCTION gb_go_set_mld_wind

     FUNCTION gb_go_download_mld(handle, mld, mldk) BIND(C, NAME='gb_go_download_mld')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, mld, mldk
       INTEGER(C_INT) :: gb_go_download_mld
     END FUNCTION gb_go_download_mld

     FUNCTION gb_go_errstr(code) BIND(C, NAME='gb_go_errstr')
       IMPORT :: C_INT, C_PTR
       INTEGER(C_INT), VALUE :: code
       TYPE(C_PTR) :: gb_go_errstr
     END FUNCTION gb_go_errstr
  END INTERFACE

CONTAINS

  ! Turn a non-zero return code into the reference's fatal-error path
  ! (die -> write_status('ERRORED') -> STOP, src/wrappers/genie_util.f90:14-30).
  SUBROUTINE gb_check(rc, what)
    USE genie_util, ONLY: die
    INTEGER(C_INT), INTENT(IN) :: rc
    CHARACTER(LEN=*), INTENT(IN) :: what
    CHARACTER(KIND=C_CHAR), POINTER :: msg(:)
    CHARACTER(LEN=128) :: text
    INTEGER :: n
    IF (rc /= 0) THEN
       CALL C_F_POINTER(gb_go_errstr(rc), msg, [128])
       text = ' '
       DO n = 1, 128
          IF (msg(n) == C_NULL_CHAR) EXIT
          text(n:n) = msg(n)
       END DO
       CALL die('libgb_goldstein: '//what//': '//TRIM(text), __LINE__, __FILE__)
    END IF
  END SUBROUTINE gb_check

END MODULE gb_goldstein_c
