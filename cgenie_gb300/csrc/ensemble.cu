// Batched ensemble C-ABI (placeholder until the batched kernel lands).
#include "../../include/gb_goldstein.h"

extern "C" {
int gb_ens_create(int, size_t, gb_ens **out) { if (out) *out = nullptr; return GB_GO_EUNSUPPORTED; }
void gb_ens_destroy(gb_ens *) {}
int gb_ens_set_tuning(gb_ens *, const gb_ens_tuning *) { return GB_GO_EUNSUPPORTED; }
int gb_ens_set_stream(gb_ens *, void *) { return GB_GO_EUNSUPPORTED; }
size_t gb_ens_member_bytes(const gb_go_dims *, const gb_go_params *) { return 0; }
int gb_ens_add(gb_ens *, const gb_go_dims *, const gb_go_params *, const gb_go_grid *, const double *, const double *, int32_t *) { return GB_GO_EUNSUPPORTED; }
int gb_ens_remove(gb_ens *, int32_t) { return GB_GO_EUNSUPPORTED; }
int gb_ens_step(gb_ens *, int32_t) { return GB_GO_EUNSUPPORTED; }
int gb_ens_set_remaining(gb_ens *, int32_t, int64_t) { return GB_GO_EUNSUPPORTED; }
int gb_ens_step_remaining(gb_ens *, int32_t) { return GB_GO_EUNSUPPORTED; }
int gb_ens_remaining(gb_ens *, int32_t, int64_t *) { return GB_GO_EUNSUPPORTED; }
int gb_ens_download(gb_ens *, int32_t, double *, double *, double *) { return GB_GO_EUNSUPPORTED; }
int gb_ens_inventory(gb_ens *, int32_t, double *) { return GB_GO_EUNSUPPORTED; }
int gb_ens_status(gb_ens *, int32_t, int32_t *) { return GB_GO_EUNSUPPORTED; }
int gb_ens_sync(gb_ens *) { return GB_GO_EUNSUPPORTED; }
int gb_ens_count(gb_ens *, int32_t *, size_t *) { return GB_GO_EUNSUPPORTED; }
const char *gb_ens_last_error(const gb_ens *) { return "ensemble not available"; }
}
