/* sgm_gb300.c -- the engine behind sgm-bench's single-frame plugin interface.
 *
 * Exports `const sgm_impl SGM_IMPL = { "gb300", gb300_run }` exactly as the
 * reference's implementations do (common/sgm.h:33-40, e.g. cuda/sgm_cuda_opt.cu:
 * 368), so common/harness.c links against this object unchanged. D and the
 * path count are compile-time, as in the reference (common/sgm_params.h:13-18):
 * build with -DSGM_D=<D> -DSGM_PATHS=<4|8>; defaults 64 and 4.
 *
 * Behaviour kept from the reference plugin: host buffers in and out,
 * synchronous, `threads` ignored (a GPU implementation), static device state
 * reused across calls and re-planned on a size change, non-zero return on any
 * failure with the reason on stderr. Stage times: census, aggregate (all path
 * passes with the cost and the argmin fused in; cost_ms = argmin_ms = -1 so the
 * cost gate folds their ops into aggregate), transfer (host<->device copies).
 */
#include <stdio.h>
#include "../../include/sgm_plugin.h"
#include "../../include/sgmgb.h"

#ifndef SGM_D
#define SGM_D 64
#endif
#ifndef SGM_PATHS
#define SGM_PATHS 4
#endif

static sgmgb_ctx *g_ctx;

static int gb300_run(const uint8_t *left, const uint8_t *right, int W, int H, uint8_t *disp,
                     int threads, sgm_stage_times *t)
{
    (void)threads;
    int rc;
    if (!g_ctx && (rc = sgmgb_create(0, &g_ctx)) != SGMGB_OK) {
        fprintf(stderr, "gb300: %s\n", sgmgb_strerror(rc));
        return -1;
    }
    const sgmgb_frame_desc fd = { W, H, SGM_D, SGM_PATHS, SGMGB_PLAIN };
    if ((rc = sgmgb_plan(g_ctx, &fd)) != SGMGB_OK) {
        fprintf(stderr, "gb300: plan %dx%d D=%d paths=%d: %s (%s)\n", W, H, SGM_D, SGM_PATHS,
                sgmgb_strerror(rc), sgmgb_last_error(g_ctx));
        return -1;
    }
    sgmgb_stage_times st;
    if ((rc = sgmgb_run_frame(g_ctx, left, right, disp, &st)) != SGMGB_OK) {
        fprintf(stderr, "gb300: %s (%s)\n", sgmgb_strerror(rc), sgmgb_last_error(g_ctx));
        return -1;
    }
    if (t) {
        t->census_ms = st.census_ms;
        t->cost_ms = st.cost_ms;
        t->aggregate_ms = st.aggregate_ms;
        t->argmin_ms = st.argmin_ms;
        t->transfer_ms = st.transfer_ms;
        t->threads_used = st.threads_used;
    }
    return 0;
}

const sgm_impl SGM_IMPL = { "gb300", gb300_run };
