"""Regenerates tests/golden/reference_scenes.json from the reference checkout.

The reference commits its scenes and golden disparity maps as PGM files
(data/golden, data/shared, data/multiscale). They are several MB, and the
reference tree is not available where the GPU tests run, so this script
records what the tests need to rebuild and check them anywhere:
  - the generator call that reproduces each scene (the reference's
    gen_synthetic, restated in oracle/sgm_oracle.c), with the sha256 of the
    committed left/right/gt files it must reproduce;
  - the FNV-1a-64 (common/util.c:54-59) and sha256 of each committed golden,
    and the configuration it was made with.
It also runs the oracle on each scene and refuses to write the file unless
the oracle reproduces every golden.

Usage: python tests/golden/make_fixtures.py [/path/to/reference]
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402


def read_pgm(path):
    d = open(path, "rb").read()
    i, tok = 2, []
    while len(tok) < 3:
        while d[i:i + 1].isspace():
            i += 1
        if d[i:i + 1] == b"#":
            while d[i:i + 1] != b"\n":
                i += 1
            continue
        j = i
        while not d[j:j + 1].isspace():
            j += 1
        tok.append(int(d[i:j]))
        i = j
    i += 1
    w, h, _ = tok
    return np.frombuffer(d[i:i + w * h], np.uint8).reshape(h, w).copy()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# scene name -> generator call (common/gen_synthetic.c built with -DSGM_D=gen_D, run W H dir seed)
SCENES = {
    "synthetic": dict(W=1920, H=1080, gen_D=64, seed=1, files=None),   # Makefile:59-63 (not committed)
    "shared": dict(W=1920, H=1080, gen_D=256, seed=3, files="data/shared"),
    "multiscale": dict(W=1920, H=800, gen_D=64, seed=1, files="data/multiscale"),
}
# golden file -> (scene, variant, D, paths)
GOLDENS = {
    "data/golden/synthetic.pgm": ("synthetic", "plain", 64, 4),
    "data/shared/golden_d64.pgm": ("shared", "plain", 64, 4),
    "data/shared/golden_d128.pgm": ("shared", "plain", 128, 4),
    "data/shared/golden_d256.pgm": ("shared", "plain", 256, 4),
    "data/multiscale/golden_ms.pgm": ("multiscale", "multiscale", 64, 8),
    "data/multiscale/golden_ms_1080.pgm": ("synthetic", "multiscale", 64, 8),
}


def main(ref):
    out = {"scenes": {}, "goldens": {}}
    scenes = {}
    for name, s in SCENES.items():
        l, r, g = oracle.gen_reference(s["W"], s["H"], s["gen_D"], s["seed"])
        scenes[name] = (l, r)
        rec = dict(W=s["W"], H=s["H"], gen_D=s["gen_D"], seed=s["seed"],
                   sha256_left=sha(l), sha256_right=sha(r), sha256_gt=sha(g))
        if s["files"]:
            for part, arr in (("left", l), ("right", r), ("gt", g)):
                committed = read_pgm(os.path.join(ref, s["files"], part + ".pgm"))
                if not np.array_equal(committed, arr):
                    raise SystemExit("generator restatement does not reproduce %s/%s.pgm" % (s["files"], part))
            rec["committed_files"] = s["files"]
        out["scenes"][name] = rec
    for path, (scene, variant, D, paths) in GOLDENS.items():
        gold = read_pgm(os.path.join(ref, path))
        l, r = scenes[scene]
        got = oracle.plain(l, r, D, paths) if variant == "plain" else oracle.multiscale(l, r)
        if not np.array_equal(got, gold):
            raise SystemExit("oracle does not reproduce %s" % path)
        out["goldens"][path] = dict(scene=scene, variant=variant, D=D, paths=paths,
                                    W=int(gold.shape[1]), H=int(gold.shape[0]),
                                    fnv1a64=oracle.fnv1a64(gold), sha256=sha(gold),
                                    max_disparity=int(gold.max()), distinct=int(len(np.unique(gold))))
        print("ok", path, out["goldens"][path]["fnv1a64"])
    with open(os.path.join(HERE, "reference_scenes.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
