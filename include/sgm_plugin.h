/* sgm_plugin.h -- the single-frame plugin interface of sgm-bench, declared
 * with the same layout so a binary built against the reference's harness can
 * link this engine unchanged.
 *
 * The reference declares these types in common/sgm.h:9-40 (sgm_stage_times,
 * sgm_run_fn, sgm_impl, `extern const sgm_impl SGM_IMPL`). The layout and
 * meaning are kept exactly: milliseconds per phase, -1 where a phase is fused
 * or not applicable, `threads_used` = 0 when not applicable; `run` returns 0
 * on success and non-zero on failure.
 *
 * This engine's implementation of the interface lives in
 * sgm-bench_gb300/csrc/sgm_gb300.c and exports SGM_IMPL = { "gb300", ... }.
 */
#ifndef SGM_PLUGIN_H
#define SGM_PLUGIN_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same fields, order and types as common/sgm.h:9-25. */
typedef struct {
    double census_ms;     /* -1: the census runs inside the frame's one graph (aggregate_ms) */
    double cost_ms;       /* -1: likewise */
    double aggregate_ms;  /* the whole frame on the device: census, cost, paths, argmin */
    double argmin_ms;     /* -1: the argmin is fused into the last path pass */
    double transfer_ms;   /* host<->device copies, kept apart from the phases */
    int    threads_used;  /* 0: not applicable on the GPU */
} sgm_stage_times;

/* common/sgm.h:29-31 */
typedef int (*sgm_run_fn)(const uint8_t *left, const uint8_t *right, int W, int H,
                          uint8_t *disp, int threads, sgm_stage_times *t);

/* common/sgm.h:33-36 */
typedef struct {
    const char *name;
    sgm_run_fn  run;
} sgm_impl;

/* common/sgm.h:40: one implementation per binary. */
extern const sgm_impl SGM_IMPL;

#ifdef __cplusplus
}
#endif
#endif
