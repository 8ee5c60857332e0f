/* tune.c -- the autotuner's result cache: one text line per decision,
 *   W H D paths variant warps_per_block lines_per_tile microseconds
 * The last line that matches a frame shape wins, so re-tuning appends. */
#include <stdio.h>
#include <string.h>
#include "sgmgb.h"

int sgmgb_tune_lookup(const char *cache_path, const sgmgb_frame_desc *fd, int *warps_per_block,
                      int *lines_per_tile)
{
    if (!cache_path || !fd || sgmgb_check_desc(fd) != SGMGB_OK) return SGMGB_ERR_ARG;
    FILE *f = fopen(cache_path, "r");
    if (!f) return SGMGB_ERR_STATE;
    char line[256];
    int found = 0, bw = 0, bl = 0;
    while (fgets(line, sizeof line, f)) {
        int W, H, D, P, V, w, l;
        double us;
        if (line[0] == '#') continue;
        if (sscanf(line, "%d %d %d %d %d %d %d %lf", &W, &H, &D, &P, &V, &w, &l, &us) != 8) continue;
        if (W == fd->W && H == fd->H && D == fd->D && P == fd->paths && V == fd->variant &&
            w >= 1 && w <= 8 && l >= 1) {
            found = 1; bw = w; bl = l;
        }
    }
    fclose(f);
    if (!found) return SGMGB_ERR_STATE;
    if (warps_per_block) *warps_per_block = bw;
    if (lines_per_tile) *lines_per_tile = bl;
    return SGMGB_OK;
}

int sgmgb_tune_record(const char *cache_path, const sgmgb_frame_desc *fd, int warps_per_block,
                      int lines_per_tile, double us)
{
    if (!cache_path || !fd || sgmgb_check_desc(fd) != SGMGB_OK) return SGMGB_ERR_ARG;
    if (warps_per_block < 1 || warps_per_block > 8 || lines_per_tile < 1) return SGMGB_ERR_ARG;
    FILE *f = fopen(cache_path, "a");
    if (!f) return SGMGB_ERR_STATE;
    fprintf(f, "%d %d %d %d %d %d %d %.3f\n", fd->W, fd->H, fd->D, fd->paths, fd->variant,
            warps_per_block, lines_per_tile, us);
    fclose(f);
    return SGMGB_OK;
}
