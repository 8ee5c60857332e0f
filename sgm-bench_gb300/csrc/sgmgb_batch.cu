// sgmgb_batch.cu -- placeholder until the persistent batch launch lands.
#include "sgmgb_internal.h"
extern "C" {
int sgmgb_batch_create(sgmgb_ctx *, const sgmgb_frame_desc *, int, sgmgb_batch **out) { if (out) *out = nullptr; return SGMGB_ERR_STATE; }
int sgmgb_batch_run(sgmgb_batch *, const uint8_t *const *, const uint8_t *const *, uint8_t *const *, void *) { return SGMGB_ERR_STATE; }
int sgmgb_batch_tile_shape(const sgmgb_batch *, int, int *, int *) { return SGMGB_ERR_STATE; }
void sgmgb_batch_destroy(sgmgb_batch *) {}
}
