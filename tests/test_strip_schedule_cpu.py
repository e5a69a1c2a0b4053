"""The strip wavefront's schedule (csrc/lssw.cuh), checked on the CPU: a
lane-by-lane model with the kernel's step, ring and copy formulas
(tests/strip_model.py) must reproduce the oracle's lin_solve bit for bit,
every read must see a value written at least one barrier earlier into a slot
not yet reused, and the fast path must give the general rules' bits."""
import numpy as np
import pytest

import oracle
from tests import strip_model as M
from tests.util import random_rects


def _case(S, K, mode, seed, G):
    rng = np.random.default_rng(seed)
    cells = np.zeros((S, S), np.uint8)
    cells[0, :] = cells[-1, :] = cells[:, 0] = cells[:, -1] = 1
    for x0, y0, x1, y1 in random_rects(rng, S, 4):
        cells[y0:y1, x0:x1] = 1
    cells = cells.reshape(-1)
    x = rng.uniform(-1, 1, S * S).astype(np.float32)
    x0 = rng.uniform(-1, 1, S * S).astype(np.float32)
    a = float(rng.uniform(0.05, 2.0))
    c = float(np.float32(1.0) + np.float32(4.0) * np.float32(a))
    if mode == M.PAS and seed % 2 == 0:
        a, c = 1.0, 4.0
    P = ((S + 31) // 32) * 32
    want = x.copy()
    oracle.lin_solve(mode, want, x0, a, c, S, K, cells)
    got, steps, fast = M.run(mode, x, x0, cells, S, P, K, a, c, G=G)
    oracle.set_boundaries(mode, got, S, cells)
    return int((got.view(np.uint32) != want.view(np.uint32)).sum()), steps, fast


# sizes from the smallest grid to several strips, sweep counts that leave the
# last group short, groups from one to ten sweeps each (ten: the widest spread
# of a row's readers over the x0 / code rings)
@pytest.mark.parametrize("S,K,G", [(20, 1, 1), (20, 3, 2), (37, 5, 3), (40, 4, 4),
                                   (66, 6, 2), (45, 9, 3), (70, 20, 5), (70, 20, 2),
                                   (150, 10, 1)])
@pytest.mark.parametrize("mode", [M.ROW, M.COL, M.PAS])
def test_strip_model_matches_oracle(S, K, G, mode):
    diff, steps, fast = _case(S, K, mode, S + K + mode, G)
    assert diff == 0
    assert steps > 0


def test_strip_model_catches_a_small_ring():
    """The model's slot keys catch a ring too narrow for the chunk schedule:
    a 16-column initial-x ring is overwritten by the chunks issued kSwAH
    periods ahead before its last read."""
    class Narrow(M.Cfg):
        PX = 16
    rng = np.random.default_rng(0)
    S, K = 70, 6
    cells = np.zeros((S, S), np.uint8)
    cells[0, :] = cells[-1, :] = cells[:, 0] = cells[:, -1] = 1
    x = rng.uniform(-1, 1, S * S).astype(np.float32)
    with pytest.raises(AssertionError, match="XR"):
        M.run(M.ROW, x, x.copy(), cells.reshape(-1), S, 96, K, 0.5, 3.0, G=1, cfg=Narrow)


def test_strip_model_catches_a_missing_frame_column():
    """The relaxed edge step must still give every value a later read needs:
    without its right frame column rule (column S-1 of an interior row left
    to the arithmetic) the model's needed-value check fails."""
    class NoRight(M.Cfg):
        EDGE_RIGHT_FRAME = False
    rng = np.random.default_rng(1)
    S, K = 40, 3
    cells = np.zeros((S, S), np.uint8)
    cells[0, :] = cells[-1, :] = cells[:, 0] = cells[:, -1] = 1
    x = rng.uniform(-1, 1, S * S).astype(np.float32)
    with pytest.raises(AssertionError):
        M.run(M.ROW, x, x.copy(), cells.reshape(-1), S, 64, K, 0.5, 3.0, G=1, cfg=NoRight)
