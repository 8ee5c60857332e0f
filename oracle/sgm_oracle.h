/* sgm_oracle.h -- CPU restatement of the reference SGM algorithms.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it. The
 * engine never links it and never falls back to it.
 *
 * Every function restates one reference function (kylefoxaustin/sgm-bench):
 *   sgmo_census          common/sgm_ref.c:23-41        (9x7, edge-replicated)
 *   sgmo_plain           common/sgm_ref.c:44-144       (cost, 4/8 paths, argmin)
 *   sgmo_sobelx          multiscale/sgm_ms_ref.c:47-54
 *   sgmo_half            multiscale/sgm_ms_ref.c:145-150
 *   sgmo_multiscale      multiscale/sgm_ms_ref.c:151-200
 *   sgmo_gen_reference   common/gen_synthetic.c:21-112 (the reference's scene
 *                        generator, so its committed scenes can be rebuilt)
 *   sgmo_fnv1a64         common/util.c:54-59
 *   sgmo_post            no reference counterpart (optional post-steps; see below)
 * D and the path count are runtime arguments here; the reference fixes them
 * at compile time (common/sgm_params.h:13-18), and the restatement is
 * checked against the reference's committed goldens at D = 64, 128, 256.
 */
#ifndef SGM_ORACLE_H
#define SGM_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 0 on success, -1 on bad arguments or allocation failure. */
int sgmo_census(const uint8_t *im, uint64_t *out, int W, int H);

/* Plain SGM: census 9x7, Hamming cost (invalid = 62), `paths` (4 or 8)
 * directions with P1 = 20 / P2 = 192, argmin with the lowest d winning ties.
 * disp is W*H. If S != NULL it receives the W*H*D uint16 summed volume. */
int sgmo_plain(const uint8_t *left, const uint8_t *right, int W, int H, int D, int paths,
               uint8_t *disp, uint16_t *S);

/* Multi-scale 8-path variant: SobelX prefilter, two scales with averaged
 * costs (invalid = 63), P1 = 40/20/10 by direction, P2 = 200 saturating,
 * argmin of the full-resolution sum at (2x,2y). D is fixed at 64 by the
 * reference. disp is (W/2)*(H/2). W and H must be even (the reference reads
 * past its half-resolution cost volume otherwise). */
int sgmo_multiscale(const uint8_t *left, const uint8_t *right, int W, int H, uint8_t *disp);

/* Optional post-steps on the plain variant's summed volume (no reference
 * counterpart: the reference has none, common/sgm_params.h:58); defined in
 * sgm_oracle.c. flags: SGMO_POST_LR (left-right check, invalid = 255; D <=
 * 240), SGMO_POST_MEDIAN (3x3 median after the check), SGMO_POST_SUBPIXEL
 * (disp16 = 16 * d + parabola offset; 0xFFFF where the check failed). */
#define SGMO_POST_LR       1
#define SGMO_POST_MEDIAN   2
#define SGMO_POST_SUBPIXEL 4
int sgmo_post(const uint8_t *left, const uint8_t *right, int W, int H, int D, int paths, int flags,
              uint8_t *disp, uint16_t *disp16);

int sgmo_sobelx(const uint8_t *im, uint8_t *out, int W, int H);
int sgmo_half(const uint8_t *im, uint8_t *out, int W, int H);

/* The reference's deterministic scene generator (gen_synthetic), with its
 * compile-time D as an argument. Writes W*H left, right and ground truth. */
int sgmo_gen_reference(int W, int H, int D, uint32_t seed,
                       uint8_t *left, uint8_t *right, uint8_t *gt);

uint64_t sgmo_fnv1a64(const void *data, size_t n);

#ifdef __cplusplus
}
#endif
#endif
