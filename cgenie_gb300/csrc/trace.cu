// Tracing of the boundary calls (include/gb_trace.h): the operations of the reference's ITT
// task shim (src/profile_api/api_fortran_itt.c:1-41) on NVTX 3 ranges, and the library's own
// ranges around its public calls (TraceRange, gb_internal.h).
#include <cuda_profiler_api.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <mutex>
#include <string>
#include <unordered_map>

#include "gb_goldstein.h"
#include "gb_internal.h"
#include "gb_trace.h"

// A domain is its NVTX handle; a task name keeps its string (NVTX copies ASCII messages at
// every push, so a name needs no registration per domain).
struct gb_tr_domain {
    nvtxDomainHandle_t h;
};
struct gb_tr_string {
    std::string name;
};

namespace {

std::mutex g_mu;

std::unordered_map<std::string, gb_tr_domain *> &domains()
{
    static auto *m = new std::unordered_map<std::string, gb_tr_domain *>();
    return *m;
}

gb_tr_domain *library_domain()
{
    static gb_tr_domain *d = gb_tr_domain_create("cgenie_gb300");
    return d;
}

void push(gb_tr_domain *d, const char *name)
{
    nvtxEventAttributes_t a = {};
    a.version = NVTX_VERSION;
    a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
    if (name) {
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
    }
    nvtxDomainRangePushEx(d ? d->h : library_domain()->h, &a);
}

}  // namespace

namespace gbgo {

TraceRange::TraceRange(const char *name) { push(nullptr, name); }
TraceRange::~TraceRange() { nvtxDomainRangePop(library_domain()->h); }

}  // namespace gbgo

extern "C" int gb_tr_resume(void) { return cudaProfilerStart() == cudaSuccess ? GB_GO_OK : GB_GO_ECUDA; }

extern "C" int gb_tr_pause(void) { return cudaProfilerStop() == cudaSuccess ? GB_GO_OK : GB_GO_ECUDA; }

extern "C" gb_tr_domain *gb_tr_domain_create(const char *name)
{
    if (!name || !*name) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    auto &m = domains();
    auto it = m.find(name);
    if (it != m.end()) return it->second;
    auto *d = new gb_tr_domain{nvtxDomainCreateA(name)};
    m.emplace(name, d);
    return d;
}

extern "C" gb_tr_string *gb_tr_string_handle_create(const char *name)
{
    if (!name) return nullptr;
    return new gb_tr_string{name};
}

extern "C" void gb_tr_task_begin(gb_tr_domain *domain, gb_tr_string *name) { push(domain, name ? name->name.c_str() : nullptr); }

extern "C" void gb_tr_task_end(gb_tr_domain *domain) { nvtxDomainRangePop(domain ? domain->h : library_domain()->h); }
