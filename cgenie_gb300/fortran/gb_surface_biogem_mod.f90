! ISO_C_BINDING interfaces to the BIOGEM tracer coupling (include/gb_biogem.h) and the
! 2-D surface steppers (include/gb_embm.h) of libgb_goldstein.so, in the binding style of
! gb_goldstein_mod.f90.
!
! Drop-in use (sketch):
!   - biogem_tracercoupling (src/biogem/biogem.f90:1885-2077): pack vocn(n)%mk, the masses,
!     volumes, reciprocal masses and vbio_part once (gb_bg_upload), the interval's vdocn and
!     vdbio_part every call (gb_bg_set_increments), then CALL gb_bg_tracercoupling(bgh, goh)
!     in place of the routine; go_ts/go_ts1 stay on the device in the gb_go handle.
!   - tstipa (src/embm/embm.f90:2039-2138): gb_ea_set_forcing(tqa, uatm, pptn) then
!     gb_ea_step(eah, 1) in place of CALL tstipa.
!   - tstipsic (src/goldsteinseaice/gold_seaice.f90:937-1058) or tstepsic (:844-929):
!     gb_ea_set_forcing(dtha, u, NULL) then gb_ea_step(sih, 1).
!
! Not compiled in this repository (no Fortran compiler on the build machines); the same
! entry points are exercised from C via ctypes in tests/.
MODULE gb_surface_biogem_c
  USE, INTRINSIC :: ISO_C_BINDING
  IMPLICIT NONE

  TYPE, BIND(C) :: gb_bg_dims
     INTEGER(C_INT32_T) :: n_i, n_j, n_k, n_l_ocn, n_l_sed, pad
  END TYPE gb_bg_dims

  TYPE, BIND(C) :: gb_bg_params
     REAL(C_DOUBLE) :: ts_offset(2)          ! tstoocn_offset(1:2)
     INTEGER(C_INT32_T) :: force_ts, pad     ! ctrl_force_GOLDSTEInTS
  END TYPE gb_bg_params

  TYPE, BIND(C) :: gb_ea_dims
     INTEGER(C_INT32_T) :: maxi, maxj
  END TYPE gb_ea_dims

  TYPE, BIND(C) :: gb_ea_params
     INTEGER(C_INT32_T) :: kind, maxk        ! 0: tstipa, 1: tstipsic, 2: tstepsic
     REAL(C_DOUBLE) :: dt, dphi, rdphi
     REAL(C_DOUBLE) :: betaz(2), betam(2)
     REAL(C_DOUBLE) :: diffmod0, ppmin, ppmax
     REAL(C_DOUBLE) :: diffsic, tsc
     REAL(C_DOUBLE) :: sica_thresh, sich_thresh   ! par_sica_thresh, par_sich_thresh (tstepsic)
  END TYPE gb_ea_params

  TYPE, BIND(C) :: gb_ea_grid
     TYPE(C_PTR) :: rc, cv, dsv, rdsv, rds, diffa, k1
  END TYPE gb_ea_grid

  INTERFACE
     FUNCTION gb_bg_create(dims, params, k1, device, handle) BIND(C, NAME='gb_bg_create')
       IMPORT :: C_INT, C_PTR, gb_bg_dims, gb_bg_params
       TYPE(gb_bg_dims), INTENT(IN) :: dims
       TYPE(gb_bg_params), INTENT(IN) :: params
       TYPE(C_PTR), VALUE :: k1
       INTEGER(C_INT), VALUE :: device
       TYPE(C_PTR), INTENT(OUT) :: handle
       INTEGER(C_INT) :: gb_bg_create
     END FUNCTION gb_bg_create

     FUNCTION gb_bg_upload(handle, vocn, mass, volume, rmass, vbio_part) BIND(C, NAME='gb_bg_upload')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, vocn, mass, volume, rmass, vbio_part
       INTEGER(C_INT) :: gb_bg_upload
     END FUNCTION gb_bg_upload

     FUNCTION gb_bg_set_increments(handle, vdocn, vdbio_part) BIND(C, NAME='gb_bg_set_increments')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, vdocn, vdbio_part
       INTEGER(C_INT) :: gb_bg_set_increments
     END FUNCTION gb_bg_set_increments

     FUNCTION gb_bg_tracercoupling(handle, ocean) BIND(C, NAME='gb_bg_tracercoupling')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, ocean
       INTEGER(C_INT) :: gb_bg_tracercoupling
     END FUNCTION gb_bg_tracercoupling

     FUNCTION gb_bg_download(handle, vocn, mass, rmass, vbio_part) BIND(C, NAME='gb_bg_download')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, vocn, mass, rmass, vbio_part
       INTEGER(C_INT) :: gb_bg_download
     END FUNCTION gb_bg_download

     SUBROUTINE gb_bg_destroy(handle) BIND(C, NAME='gb_bg_destroy')
       IMPORT :: C_PTR
       TYPE(C_PTR), VALUE :: handle
     END SUBROUTINE gb_bg_destroy

     FUNCTION gb_ea_create(dims, params, grid, device, handle) BIND(C, NAME='gb_ea_create')
       IMPORT :: C_INT, C_PTR, gb_ea_dims, gb_ea_params, gb_ea_grid
       TYPE(gb_ea_dims), INTENT(IN) :: dims
       TYPE(gb_ea_params), INTENT(IN) :: params
       TYPE(gb_ea_grid), INTENT(IN) :: grid
       INTEGER(C_INT), VALUE :: device
       TYPE(C_PTR), INTENT(OUT) :: handle
       INTEGER(C_INT) :: gb_ea_create
     END FUNCTION gb_ea_create

     FUNCTION gb_ea_upload_state(handle, tq, tq1) BIND(C, NAME='gb_ea_upload_state')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, tq, tq1
       INTEGER(C_INT) :: gb_ea_upload_state
     END FUNCTION gb_ea_upload_state

     FUNCTION gb_ea_set_forcing(handle, source, vel, pptn) BIND(C, NAME='gb_ea_set_forcing')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, source, vel, pptn
       INTEGER(C_INT) :: gb_ea_set_forcing
     END FUNCTION gb_ea_set_forcing

     FUNCTION gb_ea_step(handle, nsteps) BIND(C, NAME='gb_ea_step')
       IMPORT :: C_INT, C_PTR, C_INT32_T
       TYPE(C_PTR), VALUE :: handle
       INTEGER(C_INT32_T), VALUE :: nsteps
       INTEGER(C_INT) :: gb_ea_step
     END FUNCTION gb_ea_step

     FUNCTION gb_ea_download(handle, tq, tq1) BIND(C, NAME='gb_ea_download')
       IMPORT :: C_INT, C_PTR
       TYPE(C_PTR), VALUE :: handle, tq, tq1
       INTEGER(C_INT) :: gb_ea_download
     END FUNCTION gb_ea_download

     SUBROUTINE gb_ea_destroy(handle) BIND(C, NAME='gb_ea_destroy')
       IMPORT :: C_PTR
       TYPE(C_PTR), VALUE :: handle
     END SUBROUTINE gb_ea_destroy
  END INTERFACE
END MODULE gb_surface_biogem_c
