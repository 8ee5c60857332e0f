"""The oracle is pinned before it is trusted (CPU only, no GPU).

1. The scene generator (the reference's common/gen_synthetic.c restated in
   oracle/sgm_oracle.c) reproduces the reference's committed scenes: sha256 of
   left, right and ground truth (tests/golden/reference_scenes.json).
2. The oracle reproduces all six committed golden disparity maps, FNV-1a-64
   (common/util.c:54-59) and sha256: data/golden/synthetic.pgm,
   data/shared/golden_d{64,128,256}.pgm, data/multiscale/golden_ms{,_1080}.pgm.
3. An independent pure-Python restatement of the reference's definitions
   (common/sgm_ref.c:23-144, multiscale/sgm_ms_ref.c:47-202) agrees with the
   oracle on small images, including 1-pixel and 1-row edge cases.
"""
import concurrent.futures as cf
import hashlib

import numpy as np
import pytest

import oracle


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def scenes(ref_fixtures):
    out = {}
    for name, s in ref_fixtures["scenes"].items():
        out[name] = oracle.gen_reference(s["W"], s["H"], s["gen_D"], s["seed"])
    return out


def test_generator_reproduces_reference_scenes(ref_fixtures, scenes):
    for name, s in ref_fixtures["scenes"].items():
        l, r, g = scenes[name]
        assert _sha(l) == s["sha256_left"], name
        assert _sha(r) == s["sha256_right"], name
        assert _sha(g) == s["sha256_gt"], name


def test_oracle_reproduces_reference_goldens(ref_fixtures, scenes):
    def run(item):
        name, g = item
        l, r, _ = scenes[g["scene"]]
        if g["variant"] == "plain":
            out = oracle.plain(l, r, g["D"], g["paths"])
        else:
            out = oracle.multiscale(l, r)
        return name, g, out

    with cf.ThreadPoolExecutor(max_workers=6) as ex:       # ctypes calls release the GIL
        results = list(ex.map(run, ref_fixtures["goldens"].items()))
    for name, g, out in results:
        assert out.shape == (g["H"], g["W"]), name
        assert oracle.fnv1a64(out) == g["fnv1a64"], name
        assert _sha(out) == g["sha256"], name
        assert int(out.max()) == g["max_disparity"], name
        assert len(np.unique(out)) == g["distinct"], name


# ---- independent restatement, pure Python, small images only ----
def py_census(img):
    H, W = img.shape
    out = np.zeros((H, W), np.uint64)
    for y in range(H):
        for x in range(W):
            c = int(img[y, x])
            bits, n = 0, 0
            for dy in range(-3, 4):
                for dx in range(-4, 5):
                    if dx == 0 and dy == 0:
                        continue
                    v = int(img[min(max(y + dy, 0), H - 1), min(max(x + dx, 0), W - 1)])
                    if v < c:
                        bits |= 1 << n
                    n += 1
            out[y, x] = bits
    return out


def py_cost(cl, cr, D, invalid):
    H, W = cl.shape
    C = np.zeros((H, W, D), np.int64)
    for y in range(H):
        for x in range(W):
            for d in range(D):
                C[y, x, d] = invalid if x - d < 0 else bin(int(cl[y, x]) ^ int(cr[y, x - d])).count("1")
    return C


def py_aggregate(C, dirs, p2, saturate):
    """dirs: (dx, dy, p1). L(p) depends on L(p - (dx, dy)); the first pixel of a line takes L = C."""
    H, W, D = C.shape
    S = np.zeros((H, W, D), np.int64)
    for dx, dy, p1 in dirs:
        L = np.zeros((H, W, D), np.int64)
        ys = range(H) if dy >= 0 else range(H - 1, -1, -1)
        xs = list(range(W)) if dx >= 0 else list(range(W - 1, -1, -1))
        for y in ys:
            for x in xs:
                px, py = x - dx, y - dy
                c = C[y, x]
                if not (0 <= px < W and 0 <= py < H):
                    L[y, x] = c
                    continue
                prev = L[py, px]
                mn = int(prev.min())
                e = min(255, mn + p2)
                for d in range(D):
                    lo = min(255, int(prev[d - 1]) + p1) if d > 0 else 255
                    hi = min(255, int(prev[d + 1]) + p1) if d < D - 1 else 255
                    v = int(c[d]) + min(int(prev[d]), lo, hi, e) - mn
                    L[y, x, d] = min(255, v) if saturate else v
        S += L
    return S


def py_argmin(S):
    return S.argmin(axis=2).astype(np.uint8)      # numpy argmin returns the first (lowest) index


DIRS4 = [(1, 0), (-1, 0), (0, 1), (0, -1)]
DIRS8 = DIRS4 + [(1, 1), (-1, 1), (1, -1), (-1, -1)]


def py_plain(left, right, D, paths):
    C = py_cost(py_census(left), py_census(right), D, 62)
    dirs = [(dx, dy, 20) for dx, dy in (DIRS4 if paths == 4 else DIRS8)]
    return py_argmin(py_aggregate(C, dirs, 192, False))


def py_sobelx(img):
    H, W = img.shape
    out = np.zeros((H, W), np.uint8)
    for y in range(H):
        for x in range(W):
            def p(yy, xx):
                return int(img[min(max(yy, 0), H - 1), min(max(xx, 0), W - 1)])
            gx = (p(y - 1, x + 1) - p(y - 1, x - 1)) + 2 * (p(y, x + 1) - p(y, x - 1)) + (p(y + 1, x + 1) - p(y + 1, x - 1))
            out[y, x] = min(255, max(0, 128 + (gx >> 3)))
    return out


def py_half(img):
    H, W = img.shape
    h, w = H // 2, W // 2
    a = img[:2 * h, :2 * w].astype(np.int64)
    return ((a[0::2, 0::2] + a[0::2, 1::2] + a[1::2, 0::2] + a[1::2, 1::2] + 2) >> 2).astype(np.uint8)


def py_multiscale(left, right):
    D = 64
    dirs = [(dx, dy, 40 if dy == 0 else (20 if dx == 0 else 10)) for dx, dy in DIRS8]
    hl, hr = py_half(left), py_half(right)
    C1 = py_cost(py_census(py_sobelx(hl)), py_census(py_sobelx(hr)), D, 63)
    C2 = py_cost(py_census(py_sobelx(left)), py_census(py_sobelx(right)), D, 63)
    H, W = left.shape
    for y in range(H):
        for x in range(W):
            for d in range(D):
                C2[y, x, d] = (C2[y, x, d] + C1[y // 2, x // 2, d // 2] + 1) >> 1
    S2 = py_aggregate(C2, dirs, 200, True)
    return py_argmin(S2)[0::2, 0::2][:H // 2, :W // 2]


def _rand(H, W, seed):
    return np.random.default_rng(seed).integers(0, 256, size=(H, W), dtype=np.uint8)


@pytest.mark.parametrize("W,H", [(1, 1), (9, 7), (13, 5), (3, 11)])
def test_census_restatement(W, H):
    img = _rand(H, W, W * 31 + H)
    assert np.array_equal(oracle.census(img), py_census(img))


@pytest.mark.parametrize("W,H,D,paths", [(1, 1, 16, 4), (17, 1, 16, 4), (1, 9, 16, 8), (14, 6, 16, 4),
                                         (14, 6, 16, 8), (21, 4, 32, 8)])
def test_plain_restatement(W, H, D, paths):
    left, right = _rand(H, W, 1 + W), _rand(H, W, 2 + H)
    assert np.array_equal(oracle.plain(left, right, D, paths), py_plain(left, right, D, paths))


def test_plain_restatement_ties():
    """Flat images: all costs tie, so argmin must take the lowest d (0)."""
    flat = np.full((5, 12), 77, np.uint8)
    got = oracle.plain(flat, flat, 16, 8)
    assert np.array_equal(got, py_plain(flat, flat, 16, 8))
    assert not got.any()


def test_multiscale_restatement():
    left, right = _rand(6, 20, 5), _rand(6, 20, 6)
    assert np.array_equal(oracle.multiscale(left, right), py_multiscale(left, right))


def test_oracle_rejects_invalid_shapes():
    img = np.zeros((4, 4), np.uint8)
    with pytest.raises(ValueError):
        oracle.plain(img, img, 65, 4)
    with pytest.raises(ValueError):
        oracle.plain(img, img, 64, 6)
