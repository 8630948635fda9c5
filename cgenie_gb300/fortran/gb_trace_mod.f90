! ISO_C_BINDING interface to the tracing calls of libgb_goldstein.so (include/gb_trace.h):
! the six operations of the reference's ITT interface module (src/utils/itt_fortran.f90:1-44,
! onto src/profile_api/api_fortran_itt.c), backed by NVTX ranges and the CUDA profiler's
! collection window instead of Intel ITT.  The reference's itt_profile.f90 routines keep their
! calls; only their USE ITT_FORTRAN and the FITT_* names change to this module's GB_TR_*:
!
!   FITT_RESUME / FITT_PAUSE            -> GB_TR_RESUME / GB_TR_PAUSE (return 0 or GB_GO_ECUDA)
!   FITT_DOMAIN_CREATE(name)            -> GB_TR_DOMAIN_CREATE(name)
!   FITT_STRING_HANDLE_CREATE(name)     -> GB_TR_STRING_HANDLE_CREATE(name)
!   FITT_TASK_BEGIN(domain, handle)     -> GB_TR_TASK_BEGIN(domain, handle)
!   FITT_TASK_END(domain)               -> GB_TR_TASK_END(domain)
!
! Names are NUL-terminated C strings (pass TRIM(name)//C_NULL_CHAR).
! Not compiled in this repository (no Fortran compiler on the build machines); the same entry
! points are exercised from C via ctypes in tests/.
MODULE gb_trace_c
  USE, INTRINSIC :: ISO_C_BINDING
  IMPLICIT NONE

  INTERFACE

     FUNCTION GB_TR_RESUME() BIND(C, NAME='gb_tr_resume')
       IMPORT :: C_INT
       INTEGER(C_INT) :: GB_TR_RESUME
     END FUNCTION GB_TR_RESUME

     FUNCTION GB_TR_PAUSE() BIND(C, NAME='gb_tr_pause')
       IMPORT :: C_INT
       INTEGER(C_INT) :: GB_TR_PAUSE
     END FUNCTION GB_TR_PAUSE

     FUNCTION GB_TR_DOMAIN_CREATE(name) BIND(C, NAME='gb_tr_domain_create')
       IMPORT :: C_CHAR, C_PTR
       CHARACTER(KIND=C_CHAR) :: name(*)
       TYPE(C_PTR) :: GB_TR_DOMAIN_CREATE
     END FUNCTION GB_TR_DOMAIN_CREATE

     FUNCTION GB_TR_STRING_HANDLE_CREATE(name) BIND(C, NAME='gb_tr_string_handle_create')
       IMPORT :: C_CHAR, C_PTR
       CHARACTER(KIND=C_CHAR) :: name(*)
       TYPE(C_PTR) :: GB_TR_STRING_HANDLE_CREATE
     END FUNCTION GB_TR_STRING_HANDLE_CREATE

     SUBROUTINE GB_TR_TASK_BEGIN(domain, handle) BIND(C, NAME='gb_tr_task_begin')
       IMPORT :: C_PTR
       TYPE(C_PTR), VALUE, INTENT(IN) :: domain
       TYPE(C_PTR), VALUE, INTENT(IN) :: handle
     END SUBROUTINE GB_TR_TASK_BEGIN

     SUBROUTINE GB_TR_TASK_END(domain) BIND(C, NAME='gb_tr_task_end')
       IMPORT :: C_PTR
       TYPE(C_PTR), VALUE, INTENT(IN) :: domain
     END SUBROUTINE GB_TR_TASK_END

  END INTERFACE

END MODULE gb_trace_c
