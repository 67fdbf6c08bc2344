"""CPU checks of the broad-phase oracle: its pair set equals brute force, and
its update follows DBVTBroadPhase's stored-box rule (dbvt_broad_phase.rs:322-347):
a proxy that stays inside its loosened box keeps it; one that leaves it is
re-stored loosened, and the events are the pair-set differences."""
import numpy as np

from oracle import oracle as O


def brute(boxes):
    out = []
    n = len(boxes)
    for i in range(n):
        a = boxes[i]
        ok = (a[None, :3] <= boxes[:, 3:]).all(1) & (a[None, 3:] >= boxes[:, :3]).all(1)
        out += [(i << 32) | int(j) for j in np.nonzero(ok)[0] if j > i]
    return np.array(sorted(out), np.uint64)


def test_pairs_equal_brute_force():
    rng = np.random.default_rng(0)
    c = rng.uniform(-5, 5, (1500, 3)).astype(np.float32)
    h = rng.uniform(0.05, 0.6, (1500, 3)).astype(np.float32)
    boxes = np.concatenate([c - h, c + h], 1)
    boxes[10] = boxes[11]                      # identical boxes
    boxes[12, :3] = boxes[13, 3:]              # touching corner (closed intervals)
    boxes[14, 0] = np.nan                      # a removed proxy
    with np.errstate(invalid="ignore"):
        assert np.array_equal(O.intersecting_pairs(boxes), brute(boxes))


def test_stored_box_rule_and_events():
    bp = O.BroadPhase(0.5)
    a = np.array([[0, 0, 0, 1, 1, 1], [3, 0, 0, 4, 1, 1]], np.float32)
    p, s, t = bp.update(a)
    assert p.size == 0 and s.size == 0 and t.size == 0
    # proxy 1 moves 0.4 towards 0: inside its loosened box [2.5, 4.5], the stored box is kept
    b = a.copy()
    b[1, [0, 3]] -= 0.4
    p, s, t = bp.update(b)
    assert p.size == 0 and np.array_equal(bp.stored[1], a[1] + np.float32([-0.5] * 3 + [0.5] * 3))
    # it leaves the loosened box: re-stored as [1.4, 3.1] loosened -> meets proxy 0's [-0.5, 1.5]
    b[1, [0, 3]] -= 1.2
    p, s, t = bp.update(b)
    assert list(p) == [1] and list(s) == [1] and t.size == 0
    # proxy 1 removed (NaN box): the pair stops
    b[1, 0] = np.nan
    p, s, t = bp.update(b)
    assert p.size == 0 and list(t) == [1]
