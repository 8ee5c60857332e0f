"""sgmgb_run_frame_noalloc: a plain frame whose workspace is a static device
array (no allocation), checked through the C ABI against the allocating
entry point sgmgb_run_frame_async on two calls in a row, and both against the
oracle. The cases cover 4 and 8 paths at D = 16, 32, 64 and 128: the 8-path
chain's first pass of each pair runs in the two-lines-per-warp layout at
D = 32, 64 and 128 and the one-line layout at D = 16, its sum passes
(S = sc + L, S += sc + L, argmin of S + sc + L) in the one-line layout. The
file name sorts last so that it runs after every other test, and it needs no
fixture from them, so it also runs alone."""
import numpy as np
import pytest

import oracle
import sgmgb

pytestmark = pytest.mark.gpu

CASES = [(320, 240, 64, 4), (200, 120, 64, 8), (200, 200, 128, 4), (97, 45, 16, 8), (1, 1, 64, 4),
         (160, 90, 32, 8), (200, 200, 128, 8)]


def _noalloc(dl, dr, out, W, H, D, paths):
    return sgmgb.lib.sgmgb_run_frame_noalloc(dl.data_ptr(), dr.data_ptr(), out.data_ptr(), W, H, D, paths, None)


def test_noalloc_equals_run_frame_async_twice():
    import torch
    eng = sgmgb.Engine(0)
    for W, H, D, paths in CASES:
        left, right, _ = sgmgb.synth_pair(max(W, 2), max(H, 2), min(D, 128), seed=W + D + paths)
        left, right = np.ascontiguousarray(left[:H, :W]), np.ascontiguousarray(right[:H, :W])
        dl, dr = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
        ref = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
        eng.plan(W, H, D, paths)
        eng.run_frame_async(dl, dr, ref)
        eng.sync()
        torch.cuda.synchronize()
        for call in range(2):
            out = torch.full((H, W), 255, dtype=torch.uint8, device="cuda")
            assert _noalloc(dl, dr, out, W, H, D, paths) == sgmgb.OK
            torch.cuda.synchronize()
            assert torch.equal(out, ref), "%dx%d D=%d paths=%d call %d" % (W, H, D, paths, call)
        # and both against the oracle directly
        assert np.array_equal(ref.cpu().numpy(), oracle.plain(left, right, D, paths)), (W, H, D, paths)
    eng.close()


def test_noalloc_rejects_what_does_not_fit():
    import torch
    a = torch.zeros((1080, 1920), dtype=torch.uint8, device="cuda")
    assert _noalloc(a, a, a, 1920, 1080, 64, 4) == sgmgb.ERR_BUDGET        # 564 MB > 24 MiB
    assert _noalloc(a, a, a, 400, 300, 64, 4) == sgmgb.ERR_BUDGET
    assert _noalloc(a, a, a, 64, 48, 65, 4) == sgmgb.ERR_ARG
    assert _noalloc(a, a, a, 64, 48, 64, 6) == sgmgb.ERR_ARG
    assert sgmgb.lib.sgmgb_run_frame_noalloc(None, a.data_ptr(), a.data_ptr(), 64, 48, 64, 4, None) == sgmgb.ERR_ARG
