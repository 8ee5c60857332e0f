/* tune.c -- the autotuner's result cache: one text line per decision,
 *   W H D paths variant warps_per_block disp_per_lane microseconds
 * (disp_per_lane 0: two lines per warp in register halves where that layout applies)
 * The last line that matches a frame shape wins, so re-tuning appends. */
#include <stdio.h>
#include <string.h>
#include "sgmgb.h"

int sgmgb_tune_lookup(const char *cache_path, const sgmgb_frame_desc *fd, int *warps_per_block,
                      int *disp_per_lane)
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
            w >= 1 && w <= 4 && (l == 0 || l == 2 || l == 4 || l == 8)) {
            found = 1; bw = w; bl = l;
        }
    }
    fclose(f);
    if (!found) return SGMGB_ERR_STATE;
    if (warps_per_block) *warps_per_block = bw;
    if (disp_per_lane) *disp_per_lane = bl;
    return SGMGB_OK;
}

int sgmgb_tune_record(const char *cache_path, const sgmgb_frame_desc *fd, int warps_per_block,
                      int disp_per_lane, double us)
{
    if (!cache_path || !fd || sgmgb_check_desc(fd) != SGMGB_OK) return SGMGB_ERR_ARG;
    if (warps_per_block < 1 || warps_per_block > 4) return SGMGB_ERR_ARG;
    if (disp_per_lane != 0 && disp_per_lane != 2 && disp_per_lane != 4 && disp_per_lane != 8) return SGMGB_ERR_ARG;
    FILE *f = fopen(cache_path, "a");
    if (!f) return SGMGB_ERR_STATE;
    fprintf(f, "%d %d %d %d %d %d %d %.3f\n", fd->W, fd->H, fd->D, fd->paths, fd->variant,
            warps_per_block, disp_per_lane, us);
    fclose(f);
    return SGMGB_OK;
}
