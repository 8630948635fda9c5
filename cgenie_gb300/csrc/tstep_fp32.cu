// FP32-flux / FP64-state tracer step (placeholder until the kernel lands).
#include "gb_fp32.h"
#include "../../include/gb_goldstein.h"

namespace gbgo {

int fp32_member_init(Fp32Member *f, const Dims &, const PhysParams &, const Metrics &, const std::vector<double> &,
                     const int32_t *, cudaStream_t, std::string &msg)
{
    f->ready = false;
    msg = "GB_GO_FP32FLUX is not available in this build";
    return GB_GO_EUNSUPPORTED;
}
void fp32_member_free(Fp32Member *) {}
int fp32_member_upload(Fp32Member *, const double *, const double *, cudaStream_t) { return GB_GO_EUNSUPPORTED; }
int fp32_member_set_top(Fp32Member *, const double *, cudaStream_t) { return GB_GO_EUNSUPPORTED; }
int fp32_member_set_velocity(Fp32Member *, const double *, cudaStream_t) { return GB_GO_EUNSUPPORTED; }
int fp32_member_step(Fp32Member *, double **, int *, double *, const double *, double *, int32_t *,
                     unsigned long long *, int *, int, cudaStream_t)
{
    return GB_GO_EUNSUPPORTED;
}
int fp32_member_export(Fp32Member *, const double *, double *, const double *, cudaStream_t) { return GB_GO_EUNSUPPORTED; }

}  // namespace gbgo
