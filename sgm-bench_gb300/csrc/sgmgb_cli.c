/* sgmgb_cli.c -- command-line front end of the GB300 SGM engine.
 *
 *   sgmgb_cli ms    L.pgm R.pgm [-o out.pgm] [-g golden.pgm] [-n N] [-j results.jsonl]
 *   sgmgb_cli plain L.pgm R.pgm [-D 64] [-p 4] [-w W] [-n N] [-t T] [-o out.pgm] [-g golden.pgm]
 *                   [-j results.jsonl] [--board B] [--no-roofline] [--roofline-max X]
 *                   [--roofline-cal FILE] [--roofline-calibrate] [--max-spread X]
 *   sgmgb_cli gen   W H D seed OUTDIR
 *
 * `ms` keeps the contract of the reference's multi-scale program
 * (multiscale/sgm_ms_ref.c:151-217): the same arguments, one result line
 *   ms_gb300  in WxH out wxh D=64 paths=8  median X ms  fps F  MDE/s(work) M  hash H[  GOLDEN OK|FAIL]
 * (MDE/s under the work convention: (half-resolution + full-resolution
 * pixels) x D per second), an optional JSON line appended to -j, and exit
 * status 2 when a golden was given and differs (1 on bad input or a failed
 * frame, 0 otherwise).
 *
 * `plain` keeps the contract of the reference harness (common/harness.c:
 * 161-231) with this engine as the implementation: the same result line
 *   gb300        WxH D=.. paths=.. th=0  median .. ms  p95 ..  min ..  sd ..  spread hi/lo[ UNSTABLE]  fps ..  Mpix/s ..  hash H[  GOLDEN OK|FAIL]
 * (p95 at rank ceil(0.95 n) - 1, sd the RMS deviation about the median,
 * spread = p95/median and min/median, UNSTABLE above --max-spread), the same
 * JSON record appended to -j, and the same per-phase cost gate
 * (common/roofline.h:67-179): the stage times of the last frame divided by
 * the phase's scalar-equivalent op count (census 2*W*H*62, cost W*H*D,
 * aggregate paths*W*H*D*4, argmin W*H*D; a fused phase, reported as -1,
 * folds into aggregate) give ns per op, checked against the calibration rows
 * "impl board WxH D<d> phase ns_per_op" of --roofline-cal (default: the
 * gb300 rows committed beside this file) or written there with
 * --roofline-calibrate. Exit status 2 on a golden mismatch, 3 when the gate
 * fails, 1 on bad input or a failed frame. -t is accepted and reported as
 * requested; the GPU ignores it (threads_used 0). Times are wall-clock
 * medians of the host-buffer call sgmgb_run_frame (copies in and out
 * included) after W warm-up frames.
 * `gen` writes OUTDIR/left.pgm, right.pgm and gt.pgm from sgmgb_synth_pair. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>
#include <unistd.h>
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

/* ---- the plain harness contract (common/harness.c:161-231, common/roofline.h) ---- */
#define RL_PHASES 4
static const char *rl_names[RL_PHASES] = {"census", "cost", "aggregate", "argmin"};

/* Scalar-equivalent op count of each phase; a phase reported as -1 (fused)
 * folds its ops into aggregate (common/roofline.h:67-77). */
static void rl_ops(int W, int H, int D, int paths, const sgmgb_stage_times *t, double *ops)
{
    const double px = (double)W * H;
    ops[0] = 2.0 * px * 62;
    ops[1] = px * D;
    ops[2] = (double)paths * px * D * 4.0;
    ops[3] = px * D;
    const double ms[RL_PHASES] = {t->census_ms, t->cost_ms, t->aggregate_ms, t->argmin_ms};
    for (int i = 0; i < RL_PHASES; i++)
        if (i != 2 && ms[i] < 0) { ops[2] += ops[i]; ops[i] = 0; }
}

/* The calibration file shipped beside the package: <dir of the executable>/../roofline_gb300.cal. */
static void default_cal(char *out, size_t n)
{
    char exe[4096];
    const ssize_t k = readlink("/proc/self/exe", exe, sizeof exe - 1);
    out[0] = 0;
    if (k <= 0) return;
    exe[k] = 0;
    char *slash = strrchr(exe, '/');
    if (!slash) return;
    *slash = 0;
    snprintf(out, n, "%s/../roofline_gb300.cal", exe);
}

/* 0 = pass or not armed, 1 = fail; *armed says whether it ran. */
static int rl_check(const char *path, const char *board, int W, int H, int D, int paths,
                    const sgmgb_stage_times *t, double max_ratio, int *armed)
{
    double ops[RL_PHASES];
    rl_ops(W, H, D, paths, t, ops);
    const double ms[RL_PHASES] = {t->census_ms, t->cost_ms, t->aggregate_ms, t->argmin_ms};
    *armed = 0;
    if (t->aggregate_ms < 0) {
        fprintf(stderr, "ROOFLINE FAIL: aggregate_ms unreported\n");
        return 1;
    }
    FILE *f = fopen(path, "r");
    if (!f) {
        fprintf(stderr, "ROOFLINE NOT ARMED: no calibration file at %s\n", path);
        return 0;
    }
    char want[96];
    snprintf(want, sizeof want, "%dx%d D%d", W, H, D);
    double cal[RL_PHASES] = {-1, -1, -1, -1};
    char li[64], lb[64], lr[64], ld[64], lp[64];
    double v;
    while (fscanf(f, "%63s %63s %63s %63s %63s %lf", li, lb, lr, ld, lp, &v) == 6) {
        char got[160];
        snprintf(got, sizeof got, "%s %s", lr, ld);
        for (int i = 0; i < RL_PHASES; i++)
            if (!strcmp(li, "gb300") && !strcmp(lb, board) && !strcmp(got, want) && !strcmp(lp, rl_names[i]))
                cal[i] = v;
    }
    fclose(f);
    int have = 0;
    for (int i = 0; i < RL_PHASES; i++) have |= cal[i] > 0;
    if (!have) {
        fprintf(stderr, "ROOFLINE NOT ARMED: no calibration for gb300/%s at %dx%d D=%d\n", board, W, H, D);
        return 0;
    }
    *armed = 1;
    int fail = 0;
    printf("  roofline:");
    for (int i = 0; i < RL_PHASES; i++) {
        if (ms[i] < 0 || ops[i] == 0) continue;
        const double nspo = ms[i] * 1e6 / ops[i];
        if (cal[i] <= 0) { printf("  %s %.6f (uncal)", rl_names[i], nspo); continue; }
        const double r = nspo / cal[i];
        printf("  %s %.6f/%.6f %.2fx", rl_names[i], nspo, cal[i], r);
        if (r > max_ratio) {
            fprintf(stderr, "\nROOFLINE FAIL: phase '%s' costs %.6f ns/op against a calibrated %.6f "
                            "(%.2fx, limit %.2fx)\n", rl_names[i], nspo, cal[i], r, max_ratio);
            fail = 1;
        }
    }
    printf("\n");
    return fail;
}

static int rl_calibrate(const char *path, const char *board, int W, int H, int D, int paths,
                        const sgmgb_stage_times *t)
{
    double ops[RL_PHASES];
    rl_ops(W, H, D, paths, t, ops);
    const double ms[RL_PHASES] = {t->census_ms, t->cost_ms, t->aggregate_ms, t->argmin_ms};
    FILE *f = fopen(path, "a");
    if (!f) { fprintf(stderr, "cannot write calibration %s\n", path); return 1; }
    for (int i = 0; i < RL_PHASES; i++) {
        if (ms[i] < 0 || ops[i] == 0) continue;
        fprintf(f, "gb300 %s %dx%d D%d %s %.6f\n", board, W, H, D, rl_names[i], ms[i] * 1e6 / ops[i]);
    }
    fclose(f);
    fprintf(stderr, "roofline: calibration written to %s for gb300/%s\n", path, board);
    return 0;
}

static int run_plain(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s plain L.pgm R.pgm [-D d] [-p paths] [-w W] [-n N] [-t T] [-o out] [-g golden] "
                        "[-j json] [--board B] [--no-roofline] [--roofline-max X] [--roofline-cal F] "
                        "[--roofline-calibrate] [--max-spread X]\n", argv[0]);
        return 1;
    }
    const char *op = NULL, *gp = NULL, *jp = NULL, *board = "gb300", *cal = NULL;
    int warm = 3, timed = 20, threads = 0, D = 64, paths = 4, roofline = 1, cal_write = 0;
    double rl_max = 1.15, max_spread = 1.5;
    for (int i = 4; i < argc; i++) {
        if (!strcmp(argv[i], "-o") && i + 1 < argc) op = argv[++i];
        else if (!strcmp(argv[i], "-g") && i + 1 < argc) gp = argv[++i];
        else if (!strcmp(argv[i], "-n") && i + 1 < argc) timed = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-w") && i + 1 < argc) warm = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-t") && i + 1 < argc) threads = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-j") && i + 1 < argc) jp = argv[++i];
        else if (!strcmp(argv[i], "-D") && i + 1 < argc) D = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-p") && i + 1 < argc) paths = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--board") && i + 1 < argc) board = argv[++i];
        else if (!strcmp(argv[i], "--no-roofline")) roofline = 0;
        else if (!strcmp(argv[i], "--roofline-max") && i + 1 < argc) rl_max = atof(argv[++i]);
        else if (!strcmp(argv[i], "--roofline-cal") && i + 1 < argc) cal = argv[++i];
        else if (!strcmp(argv[i], "--roofline-calibrate")) cal_write = 1;
        else if (!strcmp(argv[i], "--max-spread") && i + 1 < argc) max_spread = atof(argv[++i]);
        else { fprintf(stderr, "unknown argument %s\n", argv[i]); return 1; }
    }
    if (warm < 0) warm = 0;
    char calbuf[4200];
    if (!cal) { default_cal(calbuf, sizeof calbuf); cal = calbuf; }
    int W, H, W2, H2;
    uint8_t *L = pgm_load(argv[2], &W, &H), *R = pgm_load(argv[3], &W2, &H2);
    if (!L || !R || W != W2 || H != H2) { fprintf(stderr, "bad input\n"); free(L); free(R); return 1; }
    sgmgb_frame_desc fd = {W, H, D, paths, SGMGB_PLAIN};
    if (sgmgb_check_desc(&fd)) {
        fprintf(stderr, "unsupported frame %dx%d D=%d paths=%d\n", W, H, D, paths);
        free(L); free(R);
        return 1;
    }
    sgmgb_ctx *ctx = NULL;
    int rc = sgmgb_create(0, &ctx);
    if (rc) { fprintf(stderr, "gb300: %s\n", sgmgb_strerror(rc)); free(L); free(R); return 1; }
    const int n = timed > 0 ? timed : 1;
    uint8_t *disp = (uint8_t *)calloc((size_t)W * H, 1);
    double *ms = (double *)malloc(sizeof(double) * n);
    sgmgb_stage_times st = {-1, -1, -1, -1, -1, 0};
    rc = sgmgb_plan(ctx, &fd);
    for (int i = 0; i < warm && !rc; i++) rc = sgmgb_run_frame(ctx, L, R, disp, &st);
    for (int i = 0; i < n && !rc; i++) {
        const double t0 = now_ms();
        rc = sgmgb_run_frame(ctx, L, R, disp, &st);
        ms[i] = now_ms() - t0;
    }
    if (rc) {
        fprintf(stderr, "gb300: frame failed: %s: %s\n", sgmgb_strerror(rc), sgmgb_last_error(ctx));
        sgmgb_destroy(ctx); free(L); free(R); free(disp); free(ms);
        return 1;
    }
    qsort(ms, n, sizeof(double), cmp_double);
    const double med = ms[n / 2], mn = ms[0];
    int p95i = (n * 95 + 99) / 100 - 1;
    if (p95i < 0) p95i = 0;
    if (p95i >= n) p95i = n - 1;
    const double p95 = ms[p95i];
    double sd = 0;
    for (int i = 0; i < n; i++) sd += (ms[i] - med) * (ms[i] - med);
    sd = n > 1 ? sqrt(sd / (n - 1)) : 0;
    const double spread_hi = med > 0 ? p95 / med : 0, spread_lo = med > 0 ? mn / med : 0;
    const int unstable = spread_hi > max_spread;
    const double fps = 1000.0 / med, mpix = (double)W * H / 1e6 * fps;
    const uint64_t h = fnv1a64(disp, (size_t)W * H);
    int gm = -1;
    if (gp) {
        int gw, gh;
        uint8_t *G = pgm_load(gp, &gw, &gh);
        if (!G) { sgmgb_destroy(ctx); free(L); free(R); free(disp); free(ms); return 1; }
        gm = gw == W && gh == H && !memcmp(G, disp, (size_t)W * H);
        free(G);
    }
    if (op && pgm_save(op, disp, W, H)) rc = 1;
    printf("%-12s %dx%d D=%d paths=%d th=%d  median %8.2f ms  p95 %8.2f  min %8.2f  sd %6.3f  spread %.2f/%.2f%s"
           "  fps %7.2f  Mpix/s %7.2f  hash %016llx%s\n",
           "gb300", W, H, D, paths, st.threads_used, med, p95, mn, sd, spread_hi, spread_lo,
           unstable ? " UNSTABLE" : "", fps, mpix, (unsigned long long)h,
           gm == 1 ? "  GOLDEN OK" : gm == 0 ? "  GOLDEN FAIL" : "");
    int rl_fail = 0, rl_armed = 0;
    if (cal_write) rl_calibrate(cal, board, W, H, D, paths, &st);
    else if (roofline) rl_fail = rl_check(cal, board, W, H, D, paths, &st, rl_max, &rl_armed);
    if (jp) {
        FILE *f = fopen(jp, "a");
        if (!f) { fprintf(stderr, "cannot open %s\n", jp); rc = 1; }
        else {
            char ts[64];
            const time_t now = time(NULL);
            strftime(ts, sizeof ts, "%Y-%m-%dT%H:%M:%SZ", gmtime(&now));
            fprintf(f, "{\"impl\":\"gb300\",\"board\":\"%s\",\"W\":%d,\"H\":%d,\"D\":%d,\"paths\":%d,\"census\":\"9x7\","
                       "\"P1\":20,\"P2\":192,\"threads\":%d,\"threads_requested\":%d,\"cpu_mask\":\"\",\"warm\":%d,"
                       "\"timed\":%d,\"median_ms\":%.3f,\"p95_ms\":%.3f,\"min_ms\":%.3f,\"rmsd_ms\":%.4f,"
                       "\"spread_hi\":%.3f,\"spread_lo\":%.3f,\"unstable\":%d,\"transfer_ms\":%.3f,\"threads_used\":%d,"
                       "\"fps\":%.3f,\"mpix_s\":%.3f,\"census_ms\":%.3f,\"cost_ms\":%.3f,\"aggregate_ms\":%.3f,"
                       "\"argmin_ms\":%.3f,\"hash\":\"%016llx\",\"golden_match\":%d,\"roofline_ok\":%d,"
                       "\"cflags\":\"sm_103a\",\"git\":\"\",\"ts\":\"%s\"}\n",
                    board, W, H, D, paths, st.threads_used, threads, warm, n, med, p95, mn, sd, spread_hi,
                    spread_lo, unstable, st.transfer_ms, st.threads_used, fps, mpix, st.census_ms, st.cost_ms,
                    st.aggregate_ms, st.argmin_ms, (unsigned long long)h, gm, rl_armed ? !rl_fail : -1, ts);
            fclose(f);
        }
    }
    sgmgb_destroy(ctx);
    free(L); free(R); free(disp); free(ms);
    if (gm == 0) return 2;
    if (rc) return 1;
    return rl_fail ? 3 : 0;
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
    if (argc >= 2 && !strcmp(argv[1], "plain")) return run_plain(argc, argv);
    fprintf(stderr,
            "usage: %s ms    L.pgm R.pgm [-o out] [-g golden] [-n N] [-j json]\n"
            "       %s plain L.pgm R.pgm [-D d] [-p paths] [-w W] [-n N] [-t T] [-o out] [-g golden] [-j json]\n"
            "                [--board B] [--no-roofline] [--roofline-max X] [--roofline-cal F] [--roofline-calibrate]\n"
            "                [--max-spread X]\n"
            "       %s gen   W H D seed OUTDIR\n",
            argv[0], argv[0], argv[0]);
    return 1;
}
