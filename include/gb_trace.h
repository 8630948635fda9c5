/*
 * gb_trace.h -- tracing of the boundary calls with NVTX ranges.
 *
 * The reference marks its module calls as Intel ITT tasks for VTune (genie.f90:118-166 under
 * INTEL_PROFILE, through utils/itt_profile.f90 and the ISO_C_BINDING interfaces of
 * utils/itt_fortran.f90:1-44 onto the C shim src/profile_api/api_fortran_itt.c:1-41).  These
 * entry points have that shim's six operations, backed by NVTX (header-only NVTX 3: every call
 * is a no-op unless a tool such as Nsight Systems or Nsight Compute is attached), so the
 * reference's profiling calls can be pointed at them unchanged in meaning:
 *
 *   fortran_itt_resume               -> gb_tr_resume            (cudaProfilerStart)
 *   fortran_itt_pause                -> gb_tr_pause             (cudaProfilerStop)
 *   fortran_itt_domain_create        -> gb_tr_domain_create     (nvtxDomainCreateA)
 *   fortran_itt_string_handle_create -> gb_tr_string_handle_create
 *   fortran_itt_task_begin           -> gb_tr_task_begin        (nvtxDomainRangePushEx)
 *   fortran_itt_task_end             -> gb_tr_task_end          (nvtxDomainRangePop)
 *
 * The library itself opens ranges in the domain "cgenie_gb300" around its public calls
 * (gb_go_tstepo, gb_go_upload_state, gb_go_download, gb_ens_step, gb_ens_add_many,
 * gb_ens_download_many, gb_mo_step, gb_rs_write, gb_ts_diagnose, ...), named after the call
 * without its "gb_" prefix; a profiler can select the kernels inside one of them (ncu --nvtx
 * --nvtx-include "cgenie_gb300@go_tstepo/").
 */
#ifndef GB_TRACE_H
#define GB_TRACE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_tr_domain gb_tr_domain;
typedef struct gb_tr_string gb_tr_string;

/* Start / stop the profiler's collection window (a tool started with a cudaProfilerApi
 * capture range collects between them).  0, or GB_GO_ECUDA when the CUDA runtime refuses
 * (no device). */
int gb_tr_resume(void);
int gb_tr_pause(void);

/* A named domain (one per name; the handle lives until the process ends), or NULL for a NULL
 * or empty name. */
gb_tr_domain *gb_tr_domain_create(const char *name);
/* A task name (the string is copied; the handle lives until the process ends), or NULL for a
 * NULL name. */
gb_tr_string *gb_tr_string_handle_create(const char *name);

/* Open / close a task of the domain on the calling thread (ranges nest).  A NULL domain is
 * the library's own; a NULL name opens an unnamed range. */
void gb_tr_task_begin(gb_tr_domain *domain, gb_tr_string *name);
void gb_tr_task_end(gb_tr_domain *domain);

#ifdef __cplusplus
}
#endif
#endif /* GB_TRACE_H */
