// sgmgb_server.cu -- placeholder until the serving loop lands.
#include "sgmgb_internal.h"
extern "C" {
int sgmgb_server_create(sgmgb_ctx *, const sgmgb_server_config *, sgmgb_server **out) { if (out) *out = nullptr; return SGMGB_ERR_STATE; }
int sgmgb_server_add_camera(sgmgb_server *, int, const sgmgb_frame_desc *) { return SGMGB_ERR_STATE; }
int sgmgb_server_submit(sgmgb_server *, int, const uint8_t *, const uint8_t *, uint64_t *) { return SGMGB_ERR_STATE; }
int sgmgb_server_poll(sgmgb_server *, uint64_t, uint8_t *, double *) { return SGMGB_ERR_STATE; }
int sgmgb_server_wait(sgmgb_server *, uint64_t, uint8_t *, double *, int) { return SGMGB_ERR_STATE; }
int sgmgb_server_stats_get(sgmgb_server *, sgmgb_server_stats *) { return SGMGB_ERR_STATE; }
void sgmgb_server_destroy(sgmgb_server *) {}
}
