/* sgm_oracle.c -- CPU restatement of the reference SGM algorithms.
 *
 * TEST INFRASTRUCTURE ONLY: the checker that the GPU engine is compared
 * against. Nothing in the engine calls it. Plain scalar C on purpose; each
 * function names the reference lines it restates (kylefoxaustin/sgm-bench).
 * Build with -ffp-contract=off so the float generator rounds identically on
 * x86-64 and aarch64.
 */
#include "sgm_oracle.h"
#include <stdlib.h>
#include <string.h>

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline int sat255(int v) { return v > 255 ? 255 : v; }

/* common/sgm_ref.c:23-41 and multiscale/sgm_ms_ref.c:55-65: bit n is set iff
 * the neighbour is darker than the centre; n runs over dy = -3..3 (outer) and
 * dx = -4..4 (inner), skipping the centre; coordinates are clamped. */
int sgmo_census(const uint8_t *im, uint64_t *out, int W, int H)
{
    if (!im || !out || W < 1 || H < 1) return -1;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const uint8_t c = im[(size_t)y * W + x];
            uint64_t bits = 0;
            int n = 0;
            for (int dy = -3; dy <= 3; dy++) {
                const uint8_t *row = im + (size_t)clampi(y + dy, 0, H - 1) * W;
                for (int dx = -4; dx <= 4; dx++) {
                    if (dx == 0 && dy == 0) continue;
                    if (row[clampi(x + dx, 0, W - 1)] < c) bits |= 1ull << n;
                    n++;
                }
            }
            out[(size_t)y * W + x] = bits;
        }
    return 0;
}

/* common/sgm_ref.c:44-56 (invalid 62) and multiscale/sgm_ms_ref.c:66-72
 * (invalid 63): C[(y*W+x)*D + d] = popcount(cl[x] ^ cr[x-d]). */
static void cost_volume(const uint64_t *cl, const uint64_t *cr, uint8_t *C, int W, int H, int D,
                        int invalid)
{
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const uint64_t a = cl[(size_t)y * W + x];
            uint8_t *c = C + ((size_t)y * W + x) * D;
            for (int d = 0; d < D; d++)
                c[d] = (x - d < 0) ? (uint8_t)invalid
                                   : (uint8_t)__builtin_popcountll(a ^ cr[(size_t)y * W + x - d]);
        }
}

/* One recurrence step (common/sgm_ref.c:61-72; with the final clamp of
 * multiscale/sgm_ms_ref.c:74-84 when `saturate`):
 *   mn = min_k prev[k];  e = sat(mn + P2)
 *   m  = min(prev[d], sat(prev[d-1] + P1), sat(prev[d+1] + P1), e), 255 off the ends
 *   cur[d] = c[d] + m - mn   (clamped to 255 when saturate) */
static void step(const uint8_t *prev, const uint8_t *c, uint8_t *cur, int D, int p1, int p2,
                 int saturate)
{
    int mn = 255;
    for (int d = 0; d < D; d++) if (prev[d] < mn) mn = prev[d];
    const int e = sat255(mn + p2);
    for (int d = 0; d < D; d++) {
        int m = prev[d];
        const int lo = d > 0 ? sat255(prev[d - 1] + p1) : 255;
        const int hi = d < D - 1 ? sat255(prev[d + 1] + p1) : 255;
        if (lo < m) m = lo;
        if (hi < m) m = hi;
        if (e < m) m = e;
        const int v = c[d] + m - mn;
        cur[d] = (uint8_t)(saturate ? sat255(v) : v);
    }
}

/* One direction (dx,dy) accumulated into S (common/sgm_ref.c:75-94,
 * multiscale/sgm_ms_ref.c:93-133). The first pixel of every line takes
 * L = C; later pixels step from the pixel (x-dx, y-dy). Rows are visited in
 * the direction of dy, pixels within a row in the direction of dx, which
 * gives every step its predecessor (the previous row for dy != 0). */
static void aggregate_dir(const uint8_t *C, uint16_t *S, int W, int H, int D, int dx, int dy,
                          int p1, int p2, int saturate, uint8_t *Lprev, uint8_t *Lcur)
{
    const int y0 = dy < 0 ? H - 1 : 0, ys = dy < 0 ? -1 : 1;
    const int x0 = dx < 0 ? W - 1 : 0, xs = dx < 0 ? -1 : 1;
    for (int yi = 0, y = y0; yi < H; yi++, y += ys) {
        for (int xi = 0, x = x0; xi < W; xi++, x += xs) {
            const uint8_t *c = C + ((size_t)y * W + x) * D;
            uint8_t *cur = Lcur + (size_t)x * D;
            const int px = x - dx, py = y - dy;
            if (px >= 0 && px < W && py >= 0 && py < H) {
                const uint8_t *prev = (dy == 0 ? Lcur : Lprev) + (size_t)px * D;
                step(prev, c, cur, D, p1, p2, saturate);
            } else {
                memcpy(cur, c, (size_t)D);
            }
            uint16_t *s = S + ((size_t)y * W + x) * D;
            for (int d = 0; d < D; d++) s[d] = (uint16_t)(s[d] + cur[d]);
        }
        uint8_t *t = Lprev; Lprev = Lcur; Lcur = t;
    }
}

/* argmin_d with a strict '<' scan: the lowest d wins ties (common/sgm_ref.c:120-124). */
static inline uint8_t argmin_lowest(const uint16_t *s, int D)
{
    int best = 0;
    uint16_t bv = s[0];
    for (int d = 1; d < D; d++) if (s[d] < bv) { bv = s[d]; best = d; }
    return (uint8_t)best;
}

/* Direction order of common/sgm_ref.c:96-99: L->R, R->L, T->B, B->T, then the
 * four diagonals (1,1), (-1,1), (1,-1), (-1,-1). The order does not change the
 * integer sum; it is kept for readability. */
static const int kPlainDirs[8][2] = { {1, 0}, {-1, 0}, {0, 1}, {0, -1},
                                      {1, 1}, {-1, 1}, {1, -1}, {-1, -1} };

int sgmo_plain(const uint8_t *left, const uint8_t *right, int W, int H, int D, int paths,
               uint8_t *disp, uint16_t *S_out)
{
    if (!left || !right || !disp || W < 1 || H < 1) return -1;
    if (D < 16 || D > 256 || D % 16 != 0) return -1;
    if (paths != 4 && paths != 8) return -1;
    const size_t N = (size_t)W * H;
    uint64_t *cl = malloc(N * 8), *cr = malloc(N * 8);
    uint8_t *C = malloc(N * (size_t)D);
    uint16_t *S = S_out ? S_out : malloc(N * (size_t)D * 2);
    uint8_t *La = malloc((size_t)W * D), *Lb = malloc((size_t)W * D);
    int rc = -1;
    if (!cl || !cr || !C || !S || !La || !Lb) goto out;
    memset(S, 0, N * (size_t)D * 2);
    sgmo_census(left, cl, W, H);
    sgmo_census(right, cr, W, H);
    cost_volume(cl, cr, C, W, H, D, 62);
    for (int p = 0; p < paths; p++)
        aggregate_dir(C, S, W, H, D, kPlainDirs[p][0], kPlainDirs[p][1], 20, 192, 0, La, Lb);
    for (size_t i = 0; i < N; i++) disp[i] = argmin_lowest(S + i * D, D);
    rc = 0;
out:
    free(cl); free(cr); free(C); free(La); free(Lb);
    if (!S_out) free(S);
    return rc;
}

/* multiscale/sgm_ms_ref.c:47-54: 3x3 horizontal Sobel, clamped coordinates,
 * mapped to clamp(128 + (gx >> 3)) with an arithmetic shift. */
int sgmo_sobelx(const uint8_t *im, uint8_t *out, int W, int H)
{
    if (!im || !out || W < 1 || H < 1) return -1;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const int xm = clampi(x - 1, 0, W - 1), xp = clampi(x + 1, 0, W - 1);
            const uint8_t *rm = im + (size_t)clampi(y - 1, 0, H - 1) * W;
            const uint8_t *r0 = im + (size_t)y * W;
            const uint8_t *rp = im + (size_t)clampi(y + 1, 0, H - 1) * W;
            const int gx = (rm[xp] - rm[xm]) + 2 * (r0[xp] - r0[xm]) + (rp[xp] - rp[xm]);
            out[(size_t)y * W + x] = (uint8_t)clampi(128 + (gx >> 3), 0, 255);
        }
    return 0;
}

/* multiscale/sgm_ms_ref.c:145-150: 2x2 box mean with rounding, floored size. */
int sgmo_half(const uint8_t *im, uint8_t *out, int W, int H)
{
    if (!im || !out || W < 2 || H < 2) return -1;
    const int w = W / 2, h = H / 2;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const uint8_t *a = im + (size_t)(2 * y) * W + 2 * x, *b = a + W;
            out[(size_t)y * w + x] = (uint8_t)((a[0] + a[1] + b[0] + b[1] + 2) >> 2);
        }
    return 0;
}

/* multiscale/sgm_ms_ref.c:135-144: SobelX -> census -> cost (invalid 63). */
static uint8_t *ms_stage_cost(const uint8_t *L, const uint8_t *R, int W, int H, int D)
{
    const size_t N = (size_t)W * H;
    uint8_t *sl = malloc(N), *sr = malloc(N), *C = malloc(N * D);
    uint64_t *cl = malloc(N * 8), *cr = malloc(N * 8);
    if (sl && sr && C && cl && cr) {
        sgmo_sobelx(L, sl, W, H); sgmo_sobelx(R, sr, W, H);
        sgmo_census(sl, cl, W, H); sgmo_census(sr, cr, W, H);
        cost_volume(cl, cr, C, W, H, D, 63);
    } else {
        free(C); C = NULL;
    }
    free(sl); free(sr); free(cl); free(cr);
    return C;
}

/* Direction table of multiscale/sgm_ms_ref.c:85-87: dx, dy, P1. */
static const int kMsDirs[8][3] = { {1, 0, 40}, {-1, 0, 40}, {0, 1, 20}, {0, -1, 20},
                                   {1, 1, 10}, {-1, -1, 10}, {1, -1, 10}, {-1, 1, 10} };

static int ms_aggregate(const uint8_t *C, uint16_t *S, int W, int H, int D)
{
    uint8_t *La = malloc((size_t)W * D), *Lb = malloc((size_t)W * D);
    if (!La || !Lb) { free(La); free(Lb); return -1; }
    for (int p = 0; p < 8; p++)
        aggregate_dir(C, S, W, H, D, kMsDirs[p][0], kMsDirs[p][1], kMsDirs[p][2], 200, 1, La, Lb);
    free(La); free(Lb);
    return 0;
}

int sgmo_multiscale(const uint8_t *left, const uint8_t *right, int W, int H, uint8_t *disp)
{
    const int D = 64;
    if (!left || !right || !disp || W < 2 || H < 2 || (W & 1) || (H & 1)) return -1;
    const int hw = W / 2, hh = H / 2;
    const size_t N = (size_t)W * H, Nh = (size_t)hw * hh;
    uint8_t *Lh = malloc(Nh), *Rh = malloc(Nh), *C1 = NULL, *C2 = NULL;
    uint16_t *S1 = NULL, *S2 = NULL;
    int rc = -1;
    if (!Lh || !Rh) goto out;
    /* stage 1: full SGM at half resolution (multiscale/sgm_ms_ref.c:168-181);
     * its argmin is defined work whose result is unused. */
    sgmo_half(left, Lh, W, H);
    sgmo_half(right, Rh, W, H);
    if (!(C1 = ms_stage_cost(Lh, Rh, hw, hh, D))) goto out;
    if (!(S1 = calloc(Nh * D, 2))) goto out;
    if (ms_aggregate(C1, S1, hw, hh, D)) goto out;
    {
        volatile uint8_t sink = 0;
        for (size_t i = 0; i < Nh; i++) sink ^= argmin_lowest(S1 + i * D, D);
        (void)sink;
    }
    /* stage 2: full resolution, cost averaged with the half-resolution cost at
     * (x/2, y/2, d/2) (multiscale/sgm_ms_ref.c:183-188). */
    if (!(C2 = ms_stage_cost(left, right, W, H, D))) goto out;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            uint8_t *c2 = C2 + ((size_t)y * W + x) * D;
            const uint8_t *c1 = C1 + ((size_t)(y / 2) * hw + x / 2) * D;
            for (int d = 0; d < D; d++) c2[d] = (uint8_t)((c2[d] + c1[d / 2] + 1) >> 1);
        }
    if (!(S2 = calloc(N * D, 2))) goto out;
    if (ms_aggregate(C2, S2, W, H, D)) goto out;
    /* argmin at (2x, 2y) -> half-resolution map (multiscale/sgm_ms_ref.c:194-199) */
    for (int y = 0; y < hh; y++)
        for (int x = 0; x < hw; x++)
            disp[(size_t)y * hw + x] = argmin_lowest(S2 + ((size_t)(2 * y) * W + 2 * x) * D, D);
    rc = 0;
out:
    free(Lh); free(Rh); free(C1); free(C2); free(S1); free(S2);
    return rc;
}

/* ---- the reference's scene generator (common/gen_synthetic.c) ---- */

/* xorshift32 of common/gen_synthetic.c:21-22 */
static inline uint32_t xs32(uint32_t *s)
{
    uint32_t v = *s;
    v ^= v << 13; v ^= v >> 17; v ^= v << 5;
    *s = v;
    return v;
}

/* common/gen_synthetic.c:24-44: three octaves (cell 2, 8, 32) of bilinearly
 * interpolated uniform lattice noise with amplitudes 1, 1/2, 1/4. */
static int gen_texture(uint8_t *im, int W, int H, uint32_t seed, uint32_t *rng)
{
    *rng = seed ? seed : 1;
    float *acc = calloc((size_t)W * H, sizeof(float));
    if (!acc) return -1;
    int cell = 2;
    for (int oct = 0; oct < 3; oct++, cell *= 4) {
        const int gw = W / cell + 2, gh = H / cell + 2;
        float *g = malloc(sizeof(float) * (size_t)gw * gh);
        if (!g) { free(acc); return -1; }
        for (int i = 0; i < gw * gh; i++) g[i] = (float)(xs32(rng) & 0xffff) / 65535.0f;
        const float amp = 1.0f / (float)(1 << oct);
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                const float fx = (float)x / (float)cell, fy = (float)y / (float)cell;
                const int ix = (int)fx, iy = (int)fy;
                const float tx = fx - (float)ix, ty = fy - (float)iy;
                const float *g0 = g + (size_t)iy * gw + ix, *g1 = g0 + gw;
                float v = g0[0] * (1 - tx) * (1 - ty);
                v = v + g0[1] * tx * (1 - ty);
                v = v + g1[0] * (1 - tx) * ty;
                v = v + g1[1] * tx * ty;
                acc[(size_t)y * W + x] += v * amp;
            }
        free(g);
    }
    for (size_t i = 0; i < (size_t)W * H; i++) {
        const float v = acc[i] / 1.75f * 255.0f;
        im[i] = v < 0 ? 0 : v > 255 ? 255 : (uint8_t)v;
    }
    free(acc);
    return 0;
}

/* common/gen_synthetic.c:46-112: background plane at d = D/8 plus 12 slabs
 * whose disparities are stratified over (D/8, D-1], the last pinned at D-1;
 * left(x + d) = right(x) with the nearer surface winning, holes filled from
 * the background. */
int sgmo_gen_reference(int W, int H, int D, uint32_t seed, uint8_t *left, uint8_t *right,
                       uint8_t *gt)
{
    if (!left || !right || !gt || W < 24 || H < 24 || D < 16 || D > 256) return -1;
    const size_t N = (size_t)W * H;
    uint8_t *slab = malloc(N), *gtr = malloc(N);
    uint32_t rng = 1;
    int rc = -1;
    if (!slab || !gtr) goto out;
    if (gen_texture(right, W, H, seed, &rng)) goto out;
    if (gen_texture(slab, W, H, seed * 7919u + 17u, &rng)) goto out;
    const int bgd = D / 8;
    memset(gtr, bgd, N);
    rng = seed * 31u + 5u;
    const int nslab = 12;
    for (int s = 0; s < nslab; s++) {
        const int sw = W / 6 + (int)(xs32(&rng) % (uint32_t)(W / 4));
        const int sh = H / 6 + (int)(xs32(&rng) % (uint32_t)(H / 4));
        const int sx = (int)(xs32(&rng) % (uint32_t)(W - sw));
        const int sy = (int)(xs32(&rng) % (uint32_t)(H - sh));
        const int dlo = bgd + 1, dhi = D - 1;
        const int blo = dlo + (dhi - dlo) * s / nslab;
        int bhi = dlo + (dhi - dlo) * (s + 1) / nslab;
        if (bhi <= blo) bhi = blo + 1;
        const int d = (s == nslab - 1) ? dhi : blo + (int)(xs32(&rng) % (uint32_t)(bhi - blo));
        for (int y = sy; y < sy + sh; y++)
            for (int x = sx; x < sx + sw; x++) {
                const size_t i = (size_t)y * W + x;
                if (d > gtr[i]) { gtr[i] = (uint8_t)d; right[i] = slab[i]; }
            }
    }
    memset(gt, 0, N);
    for (int y = 0; y < H; y++) {
        uint8_t *lrow = left + (size_t)y * W, *grow = gt + (size_t)y * W;
        const uint8_t *rrow = right + (size_t)y * W, *drow = gtr + (size_t)y * W;
        memset(lrow, 0, (size_t)W);
        for (int x = 0; x < W; x++) {
            const int d = drow[x], xl = x + d;
            if (xl < W && d >= grow[xl]) { lrow[xl] = rrow[x]; grow[xl] = (uint8_t)d; }
        }
        for (int x = 0; x < W; x++)
            if (grow[x] == 0) {
                const int xr = x - bgd < 0 ? 0 : x - bgd;
                lrow[x] = rrow[xr];
                grow[x] = (uint8_t)bgd;
            }
    }
    rc = 0;
out:
    free(slab); free(gtr);
    return rc;
}

/* Optional post-steps on the plain summed volume. The reference has none
 * (common/sgm_params.h:58: "No LR check, no subpixel, no median"); these are
 * this oracle's definitions, which the engine's post mode matches bit for bit:
 *   d_L(p)   = argmin_d S(p, d), lowest d on ties (the plain map);
 *   disp16   = 16*d_L + (16*(c0 - c2)) / (2*(c0 + c2 - 2*c1)) with c0, c1, c2 =
 *              S(d_L - 1), S(d_L), S(d_L + 1), C integer division (toward zero),
 *              when 0 < d_L < D-1 and the denominator is > 0; else 16*d_L;
 *   LR:      d_R(x, y) = argmin over d with x + d < W of S((x + d, y), d),
 *              lowest d on ties; p = (x, y) is invalid (255; disp16 0xFFFF)
 *              when x - d_L < 0 or |d_L - d_R(x - d_L, y)| > 1;
 *   median:  the 3x3 median of the (checked) map, edge-replicated. */
static uint8_t median9(uint8_t *v)
{
    for (int i = 1; i < 9; i++)
        for (int j = i; j > 0 && v[j - 1] > v[j]; j--) { uint8_t t = v[j]; v[j] = v[j - 1]; v[j - 1] = t; }
    return v[4];
}

int sgmo_post(const uint8_t *left, const uint8_t *right, int W, int H, int D, int paths, int flags,
              uint8_t *disp, uint16_t *disp16)
{
    if (!left || !right || !disp || W < 1 || H < 1 || (flags & ~7)) return -1;
    if ((flags & SGMO_POST_LR) && D > 240) return -1;
    if ((flags & SGMO_POST_SUBPIXEL) && !disp16) return -1;
    const size_t N = (size_t)W * H;
    uint16_t *S = malloc(N * (size_t)D * 2);
    uint8_t *dL = malloc(N), *dR = malloc(N);
    int rc = -1;
    if (!S || !dL || !dR) goto out;
    if (sgmo_plain(left, right, W, H, D, paths, dL, S)) goto out;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            int best = 0, bv = 1 << 30;
            for (int d = 0; d < D && x + d < W; d++) {
                const int v = S[((size_t)y * W + x + d) * D + d];
                if (v < bv) { bv = v; best = d; }
            }
            dR[(size_t)y * W + x] = (uint8_t)best;
        }
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const size_t i = (size_t)y * W + x;
            const int d = dL[i];
            const uint16_t *s = S + i * D;
            int v16 = 16 * d;
            if (d > 0 && d < D - 1) {
                const int c0 = s[d - 1], c1 = s[d], c2 = s[d + 1], den = c0 + c2 - 2 * c1;
                if (den > 0) v16 += (16 * (c0 - c2)) / (2 * den);
            }
            int out = d;
            if (flags & SGMO_POST_LR) {
                const int xr = x - d;
                if (xr < 0 || abs(d - (int)dR[(size_t)y * W + xr]) > 1) { out = 255; v16 = 0xFFFF; }
            }
            disp[i] = (uint8_t)out;
            if (flags & SGMO_POST_SUBPIXEL) disp16[i] = (uint16_t)v16;
        }
    if (flags & SGMO_POST_MEDIAN) {
        memcpy(dL, disp, N);
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                uint8_t v[9];
                int k = 0;
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++)
                        v[k++] = dL[(size_t)clampi(y + dy, 0, H - 1) * W + clampi(x + dx, 0, W - 1)];
                disp[(size_t)y * W + x] = median9(v);
            }
    }
    rc = 0;
out:
    free(S); free(dL); free(dR);
    return rc;
}

/* common/util.c:54-59 */
uint64_t sgmo_fnv1a64(const void *data, size_t n)
{
    const uint8_t *p = (const uint8_t *)data;
    uint64_t h = 0xcbf29ce484222325ull;
    for (size_t i = 0; i < n; i++) { h ^= p[i]; h *= 0x100000001b3ull; }
    return h;
}
