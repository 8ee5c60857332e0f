/* synth.c -- seeded synthetic rectified stereo pairs (sgmgb_synth_pair).
 *
 * The scene every benchmark configuration is quoted on:
 *   left   band-limited noise: three octaves of blurred uniform noise with
 *          sigma 1, 4 and 16 px, each scaled to unit variance, summed and
 *          rescaled to 0..255;
 *   gt     piecewise-planar disparity over 40 Voronoi cells, each with an
 *          offset uniform in [0, D-1] and slopes uniform in +-0.02 px/px,
 *          clamped to [0, D-1];
 *   right  the left image warped by gt (left(x) = right(x - d), nearer
 *          surface wins, target rounded to the nearest pixel); right pixels
 *          nothing lands on (occlusions) take fresh noise from an independent
 *          texture; then Gaussian noise with sigma 2; clamped to 0..255.
 * Choices the description leaves open, fixed here so every machine produces
 * the same bytes: the RNG is splitmix64; each Gaussian blur is three
 * successive box filters of the widths that match sigma (Kovesi's method),
 * with edge-replicated borders, computed in exact integers; the sigma-2 noise
 * is the sum of 12 uniform 16-bit draws (Irwin-Hall), rounded to integers;
 * floating point uses only + - * / sqrt (IEEE, no contraction).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "sgmgb.h"

static uint64_t sm64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double unif(uint64_t *s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }

/* Box widths (odd) of a 3-pass box blur matching sigma. */
static void box_widths(double sigma, int w[3])
{
    const double ideal = sqrt(12.0 * sigma * sigma / 3.0 + 1.0);
    int wl = (int)ideal;
    if (wl % 2 == 0) wl--;
    const int wu = wl + 2;
    const double mi = (12.0 * sigma * sigma - 3.0 * wl * wl - 12.0 * wl - 9.0) / (-4.0 * wl - 4.0);
    const int m = (int)(mi + 0.5);
    for (int i = 0; i < 3; i++) w[i] = i < m ? wl : wu;
}

/* One box pass of odd width w along rows (stride 1) or columns (stride W),
 * unnormalised running sum, edge-replicated. */
static void box_pass(const int64_t *in, int64_t *out, int W, int H, int w, int along_rows)
{
    const int r = w / 2;
    const int n = along_rows ? W : H, lines = along_rows ? H : W;
    const size_t step = along_rows ? 1 : (size_t)W, lstep = along_rows ? (size_t)W : 1;
    for (int l = 0; l < lines; l++) {
        const int64_t *src = in + l * lstep;
        int64_t *dst = out + l * lstep;
        int64_t acc = 0;
        for (int i = -r; i <= r; i++) {
            int k = i < 0 ? 0 : (i >= n ? n - 1 : i);
            acc += src[(size_t)k * step];
        }
        for (int i = 0; i < n; i++) {
            dst[(size_t)i * step] = acc;
            int ko = i - r, ki = i + r + 1;
            ko = ko < 0 ? 0 : (ko >= n ? n - 1 : ko);
            ki = ki < 0 ? 0 : (ki >= n ? n - 1 : ki);
            acc += src[(size_t)ki * step] - src[(size_t)ko * step];
        }
    }
}

/* Sum of three unit-variance blurred-noise octaves into acc (W*H doubles). */
static int octave_texture(double *acc, int W, int H, uint64_t *rng)
{
    const size_t N = (size_t)W * H;
    int64_t *a = malloc(N * sizeof *a), *b = malloc(N * sizeof *b);
    if (!a || !b) { free(a); free(b); return -1; }
    static const double sig[3] = { 1.0, 4.0, 16.0 };
    memset(acc, 0, N * sizeof *acc);
    for (int o = 0; o < 3; o++) {
        for (size_t i = 0; i < N; i++) a[i] = (int64_t)(sm64(rng) >> 48);
        int w[3];
        box_widths(sig[o], w);
        for (int p = 0; p < 3; p++) { box_pass(a, b, W, H, w[p], 1); int64_t *t = a; a = b; b = t; }
        for (int p = 0; p < 3; p++) { box_pass(a, b, W, H, w[p], 0); int64_t *t = a; a = b; b = t; }
        double mean = 0, var = 0;
        for (size_t i = 0; i < N; i++) mean += (double)a[i];
        mean /= (double)N;
        for (size_t i = 0; i < N; i++) { const double d = (double)a[i] - mean; var += d * d; }
        const double sd = sqrt(var / (double)N);
        const double inv = sd > 0 ? 1.0 / sd : 0.0;
        for (size_t i = 0; i < N; i++) acc[i] += ((double)a[i] - mean) * inv;
    }
    free(a); free(b);
    return 0;
}

static void rescale_u8(const double *acc, uint8_t *out, size_t N)
{
    double lo = acc[0], hi = acc[0];
    for (size_t i = 1; i < N; i++) { if (acc[i] < lo) lo = acc[i]; if (acc[i] > hi) hi = acc[i]; }
    const double k = hi > lo ? 255.0 / (hi - lo) : 0.0;
    for (size_t i = 0; i < N; i++) {
        const double v = (acc[i] - lo) * k + 0.5;
        out[i] = (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : (int)v));
    }
}

int sgmgb_synth_pair(int W, int H, int D, uint64_t seed, uint8_t *left, uint8_t *right, uint8_t *gt)
{
    if (W < 1 || H < 1 || D < 1 || D > 256) return SGMGB_ERR_ARG;
    const size_t N = (size_t)W * H;
    double *acc = malloc(N * sizeof *acc);
    float *dgt = malloc(N * sizeof *dgt), *zb = malloc((size_t)W * sizeof *zb);
    uint8_t *L = malloc(N), *R = malloc(N), *fresh = malloc(N), *G = malloc(N);
    int rc = SGMGB_ERR_NOMEM;
    if (!acc || !dgt || !zb || !L || !R || !fresh || !G) goto out;
    uint64_t rng = seed * 0x9E3779B97F4A7C15ull + 0x5851F42D4C957F2Dull;

    /* left texture and the independent occlusion-fill texture */
    if (octave_texture(acc, W, H, &rng)) goto out;
    rescale_u8(acc, L, N);
    if (octave_texture(acc, W, H, &rng)) goto out;
    rescale_u8(acc, fresh, N);

    /* piecewise-planar ground truth over 40 Voronoi cells */
    enum { NC = 40 };
    double cx[NC], cy[NC], d0[NC], gx[NC], gy[NC];
    for (int k = 0; k < NC; k++) {
        cx[k] = unif(&rng) * W; cy[k] = unif(&rng) * H;
        d0[k] = unif(&rng) * (D - 1);
        gx[k] = (unif(&rng) * 2.0 - 1.0) * 0.02;
        gy[k] = (unif(&rng) * 2.0 - 1.0) * 0.02;
    }
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            int best = 0; double bd = 0;
            for (int k = 0; k < NC; k++) {
                const double ex = x - cx[k], ey = y - cy[k], dd = ex * ex + ey * ey;
                if (k == 0 || dd < bd) { bd = dd; best = k; }
            }
            double d = d0[best] + gx[best] * (x - cx[best]) + gy[best] * (y - cy[best]);
            if (d < 0) d = 0;
            if (d > D - 1) d = D - 1;
            dgt[(size_t)y * W + x] = (float)d;
            G[(size_t)y * W + x] = (uint8_t)(d + 0.5);
        }

    /* forward warp left -> right with a z-buffer (larger disparity = nearer wins) */
    for (int y = 0; y < H; y++) {
        uint8_t *rr = R + (size_t)y * W;
        const uint8_t *lr = L + (size_t)y * W, *fr = fresh + (size_t)y * W;
        for (int x = 0; x < W; x++) zb[x] = -1.0f;
        for (int x = 0; x < W; x++) {
            const float d = dgt[(size_t)y * W + x];
            const double t = (double)x - (double)d + 0.5;
            const int xi = (int)floor(t);
            if (xi < 0 || xi >= W) continue;
            if (d > zb[xi]) { zb[xi] = d; rr[xi] = lr[x]; }
        }
        for (int x = 0; x < W; x++) if (zb[x] < 0) rr[x] = fr[x];
    }

    /* sensor noise, sigma 2: Irwin-Hall sum of 12 uniform 16-bit draws */
    for (size_t i = 0; i < N; i++) {
        int64_t s = 0;
        for (int k = 0; k < 12; k++) s += (int64_t)(sm64(&rng) >> 48);
        s -= 393210;   /* 12 * 32767.5, rounded down; the half is absorbed by rounding */
        const int64_t twice = 2 * s;
        const int64_t n = (twice + (twice >= 0 ? 32768 : -32768)) / 65536;
        const int64_t v = (int64_t)R[i] + n;
        R[i] = (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
    }
    if (left) memcpy(left, L, N);
    if (right) memcpy(right, R, N);
    if (gt) memcpy(gt, G, N);
    rc = SGMGB_OK;
out:
    free(acc); free(dgt); free(zb); free(L); free(R); free(fresh); free(G);
    return rc;
}
