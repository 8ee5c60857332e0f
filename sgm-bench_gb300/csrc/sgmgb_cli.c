/* sgmgb_cli.c -- command-line front end of the GB300 SGM engine.
 *
 *   sgmgb_cli ms    L.pgm R.pgm [-o out.pgm] [-g golden.pgm] [-n N] [-j results.jsonl]
 *   sgmgb_cli plain L.pgm R.pgm [-D 64] [-p 4] [-o out.pgm] [-g golden.pgm] [-n N] [-w W] [-j results.jsonl]
 *   sgmgb_cli gen   W H D seed OUTDIR
 *
 * `ms` keeps the contract of the reference's multi-scale program
 * (multiscale/sgm_ms_ref.c:151-217): the same arguments, one result line
 *   ms_gb300  in WxH out wxh D=64 paths=8  median X ms  fps F  MDE/s(work) M  hash H[  GOLDEN OK|FAIL]
 * (MDE/s under the work convention: (half-resolution + full-resolution
 * pixels) x D per second), an optional JSON line appended to -j, and exit
 * status 2 when a golden was given and differs (1 on bad input or a failed
 * frame, 0 otherwise). `plain` prints the same kind of line for the plain
 * variant ("gb300  in WxH D=.. paths=..  median ..", MDE/s = W*H*D per
 * second). Times are wall-clock medians of the host-buffer call
 * sgmgb_run_frame (copies in and out included) after W warm-up frames.
 * `gen` writes OUTDIR/left.pgm, right.pgm and gt.pgm from sgmgb_synth_pair. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "sgmgb.h"

static uint8_t *pgm_load(const char *path, int *W, int *H)
{
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); return NULL; }
    int v[3], n = 0, c;
    char magic[3] = {0};
    if (fread(magic, 1, 2, f) != 2 || magic[0] != 'P' || magic[1] != '5') {
        fprintf(stderr, "%s: not a binary PGM (P5)\n", path);
        fclose(f);
        return NULL;
    }
    while (n < 3) {
        c = fgetc(f);
        if (c == EOF) break;
        if (c == '#') { while (c != '\n' && c != EOF) c = fgetc(f); continue; }
        if (c >= '0' && c <= '9') {
            int x = 0;
            while (c >= '0' && c <= '9') { x = x * 10 + (c - '0'); c = fgetc(f); }
            v[n++] = x;
        }
    }
    if (n < 3 || v[0] < 1 || v[1] < 1 || v[2] != 255) {
        fprintf(stderr, "%s: bad PGM header (need maxval 255)\n", path);
        fclose(f);
        return NULL;
    }
    const size_t sz = (size_t)v[0] * v[1];
    uint8_t *img = (uint8_t *)malloc(sz);
    if (!img || fread(img, 1, sz, f) != sz) {
        fprintf(stderr, "%s: short read\n", path);
        free(img);
        fclose(f);
        return NULL;
    }
    fclose(f);
    *W = v[0];
    *H = v[1];
    return img;
}

static int pgm_save(const char *path, const uint8_t *img, int W, int H)
{
    FILE *f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path); return -1; }
    fprintf(f, "P5\n%d %d\n255\n", W, H);
    const size_t sz = (size_t)W * H;
    const int ok = fwrite(img, 1, sz, f) == sz;
    fclose(f);
    return ok ? 0 : -1;
}

/* FNV-1a 64 over the map bytes: the reference's golden hash (common/util.c:54-59). */
static uint64_t fnv1a64(const uint8_t *p, size_t n)
{
    uint64_t h = 0xcbf29ce484222325ull;
    for (size_t i = 0; i < n; i++) { h ^= p[i]; h *= 0x100000001b3ull; }
    return h;
}

static double now_ms(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static int cmp_double(const void *a, const void *b)
{
    const double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : x > y;
}

static int run_gen(int argc, char **argv)
{
    if (argc < 7) { fprintf(stderr, "usage: %s gen W H D seed OUTDIR\n", argv[0]); return 1; }
    const int W = atoi(argv[2]), H = atoi(argv[3]), D = atoi(argv[4]);
    const uint64_t seed = strtoull(argv[5], NULL, 10);
    const size_t n = (size_t)(W > 0 ? W : 0) * (H > 0 ? H : 0);
    uint8_t *l = malloc(n ? n : 1), *r = malloc(n ? n : 1), *g = malloc(n ? n : 1);
    int rc = sgmgb_synth_pair(W, H, D, seed, l, r, g);
    if (rc) fprintf(stderr, "gen: %s\n", sgmgb_strerror(rc));
    char path[4096];
    const char *names[3] = {"left.pgm", "right.pgm", "gt.pgm"};
    const uint8_t *imgs[3] = {l, r, g};
    for (int i = 0; i < 3 && !rc; i++) {
        snprintf(path, sizeof path, "%s/%s", argv[6], names[i]);
        if (pgm_save(path, imgs[i], W, H)) rc = -1;
    }
    free(l); free(r); free(g);
    return rc ? 1 : 0;
}

static int run_frames(int argc, char **argv, int variant)
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s %s L.pgm R.pgm [-D d] [-p paths] [-o out] [-g golden] [-n N] [-w W] [-j json]\n",
                argv[0], argv[1]);
        return 1;
    }
    const char *op = NULL, *gp = NULL, *jp = NULL;
    int reps = 1, warm = variant == SGMGB_MULTISCALE ? 0 : 1, D = 64, paths = variant == SGMGB_MULTISCALE ? 8 : 4;
    for (int i = 4; i < argc; i++) {
        if (!strcmp(argv[i], "-o") && i + 1 < argc) op = argv[++i];
        else if (!strcmp(argv[i], "-g") && i + 1 < argc) gp = argv[++i];
        else if (!strcmp(argv[i], "-n") && i + 1 < argc) reps = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-w") && i + 1 < argc) warm = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-j") && i + 1 < argc) jp = argv[++i];
        else if (!strcmp(argv[i], "-D") && i + 1 < argc && variant == SGMGB_PLAIN) D = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-p") && i + 1 < argc && variant == SGMGB_PLAIN) paths = atoi(argv[++i]);
        else { fprintf(stderr, "unknown argument %s\n", argv[i]); return 1; }
    }
    if (reps < 1) reps = 1;
    if (warm < 0) warm = 0;
    int W, H, W2, H2;
    uint8_t *L = pgm_load(argv[2], &W, &H), *R = pgm_load(argv[3], &W2, &H2);
    if (!L || !R || W != W2 || H != H2) { fprintf(stderr, "bad input\n"); free(L); free(R); return 1; }
    sgmgb_frame_desc fd = {W, H, D, paths, variant};
    int ow = 0, oh = 0, rc = sgmgb_check_desc(&fd);
    if (!rc) rc = sgmgb_out_size(&fd, &ow, &oh);
    if (rc) { fprintf(stderr, "unsupported frame %dx%d D=%d paths=%d\n", W, H, D, paths); free(L); free(R); return 1; }
    sgmgb_ctx *ctx = NULL;
    rc = sgmgb_create(0, &ctx);
    if (rc) { fprintf(stderr, "gb300: %s\n", sgmgb_strerror(rc)); free(L); free(R); return 1; }
    uint8_t *disp = (uint8_t *)calloc((size_t)ow * oh, 1);
    double *ms = (double *)malloc(sizeof(double) * reps);
    rc = sgmgb_plan(ctx, &fd);
    for (int i = 0; i < warm && !rc; i++) rc = sgmgb_run_frame(ctx, L, R, disp, NULL);
    for (int i = 0; i < reps && !rc; i++) {
        const double t0 = now_ms();
        rc = sgmgb_run_frame(ctx, L, R, disp, NULL);
        ms[i] = now_ms() - t0;
    }
    if (rc) {
        fprintf(stderr, "gb300: frame failed: %s: %s\n", sgmgb_strerror(rc), sgmgb_last_error(ctx));
        sgmgb_destroy(ctx); free(L); free(R); free(disp); free(ms);
        return 1;
    }
    qsort(ms, reps, sizeof(double), cmp_double);
    const double med = ms[reps / 2];
    const uint64_t h = fnv1a64(disp, (size_t)ow * oh);
    int gm = -1;
    if (gp) {
        int gw, gh;
        uint8_t *G = pgm_load(gp, &gw, &gh);
        gm = G && gw == ow && gh == oh && !memcmp(G, disp, (size_t)ow * oh);
        free(G);
    }
    const char *tag = gm == 1 ? "  GOLDEN OK" : gm == 0 ? "  GOLDEN FAIL" : "";
    if (variant == SGMGB_MULTISCALE) {
        const double work = ((double)(W / 2) * (H / 2) + (double)W * H) * D;
        printf("ms_gb300  in %dx%d out %dx%d D=%d paths=8  median %.2f ms  fps %.2f  MDE/s(work) %.0f  hash %016llx%s\n",
               W, H, ow, oh, D, med, 1000.0 / med, work / med / 1000.0, (unsigned long long)h, tag);
    } else {
        printf("gb300  in %dx%d D=%d paths=%d  median %.3f ms  fps %.2f  MDE/s %.0f  hash %016llx%s\n", W, H, D,
               paths, med, 1000.0 / med, (double)W * H * D / med / 1000.0, (unsigned long long)h, tag);
    }
    if (op && pgm_save(op, disp, ow, oh)) rc = 1;
    if (jp) {
        FILE *f = fopen(jp, "a");
        if (f) {
            fprintf(f, "{\"impl\":\"%s\",\"W\":%d,\"H\":%d,\"outW\":%d,\"outH\":%d,\"D\":%d,\"paths\":%d,"
                       "\"median_ms\":%.3f,\"hash\":\"%016llx\",\"golden_match\":%d}\n",
                    variant == SGMGB_MULTISCALE ? "ms_gb300" : "gb300", W, H, ow, oh, D, paths, med,
                    (unsigned long long)h, gm);
            fclose(f);
        }
    }
    sgmgb_destroy(ctx);
    free(L); free(R); free(disp); free(ms);
    if (gm == 0) return 2;
    return rc ? 1 : 0;
}

int main(int argc, char **argv)
{
    if (argc >= 2 && !strcmp(argv[1], "gen")) return run_gen(argc, argv);
    if (argc >= 2 && !strcmp(argv[1], "ms")) return run_frames(argc, argv, SGMGB_MULTISCALE);
    if (argc >= 2 && !strcmp(argv[1], "plain")) return run_frames(argc, argv, SGMGB_PLAIN);
    fprintf(stderr,
            "usage: %s ms    L.pgm R.pgm [-o out] [-g golden] [-n N] [-j json]\n"
            "       %s plain L.pgm R.pgm [-D d] [-p paths] [-o out] [-g golden] [-n N] [-w W] [-j json]\n"
            "       %s gen   W H D seed OUTDIR\n",
            argv[0], argv[0], argv[0]);
    return 1;
}
