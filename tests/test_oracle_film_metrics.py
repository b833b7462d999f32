"""The oracle's restatement of the outlier replay cache (OutlierReplayCache.cs:9-35 over .NET's
4-ary PriorityQueue) and of the outlier-rejecting RelMSE, pinned by hand-worked cases and by the
properties the reference's code implies."""
import numpy as np
import pytest

from oracle import film_metrics as F
from seesharp_gb300 import OutlierReplayCache, Pixel, rel_mse_outlier_rejection


def run(values, n):
    w, it = [], []
    for s, v in enumerate(values):
        if np.isfinite(v):
            F.heap_notify(w, it, n, float(v), s)
    return w, it


@pytest.mark.parametrize("values,n,want_w,want_it", [
    # Enqueue 1..4 (no sift: every parent is smaller), then 5 replaces the root and sifts past 2
    ([1, 2, 3, 4, 5], 4, [2, 5, 3, 4], [1, 4, 2, 3]),
    # decreasing: every Enqueue sifts to the root; 1 does not exceed the root 2 and is dropped
    ([5, 4, 3, 2, 1], 4, [2, 5, 4, 3], [3, 0, 1, 2]),
    # ties: a sample equal to the smallest kept one is dropped; 7 evicts the root (iteration 0) and
    # the sift stops at the first of the equal children
    ([0, 0, 0, 0, 0, 7], 4, [0, 7, 0, 0], [1, 5, 2, 3]),
    # two levels of the 4-ary heap (children of node 1 are nodes 5..8)
    ([1, 2, 3, 4, 5, 6, 7, 8, 9], 8, [2, 6, 3, 4, 5, 9, 7, 8], [1, 5, 2, 3, 4, 8, 6, 7]),
    # fewer samples than slots, and non-finite samples skipped
    ([3, np.nan, 1, np.inf], 4, [1, 3], [2, 0]),
    ([4, 2, 9], 0, [], []),
])
def test_heap_hand_worked(values, n, want_w, want_it):
    w, it = run(values, n)
    assert w == want_w and it == want_it


def test_heap_keeps_the_largest_and_drops_ties_with_the_minimum():
    """Whatever the array order: the kept priorities are the n largest, a heap property holds
    (every node is at least its parent), and a sample equal to the current minimum never enters."""
    rng = np.random.default_rng(5)
    for trial in range(300):
        n = int(rng.integers(1, 9))
        vals = rng.integers(0, 6, size=int(rng.integers(0, 40))).astype(np.float32)
        w, it = run(vals, n)
        assert sorted(w, reverse=True) == sorted(vals.tolist(), reverse=True)[:n]
        for k in range(1, len(w)):
            assert w[(k - 1) // 4] <= w[k]
        # every kept entry names an iteration with that value, each iteration at most once
        assert len(set(it)) == len(it) and all(vals[i] == x for x, i in zip(w, it))
        # the first n samples of the largest value class beyond the kept minimum are all present
        if len(w) == n and len(vals) > n:
            m = min(w)
            above = [i for i, v in enumerate(vals) if v > m]
            assert set(above) <= set(it)


def test_outlier_cache_over_an_image_matches_per_pixel_heaps():
    rng = np.random.default_rng(1)
    vals = rng.exponential(size=(7, 3, 5, 3)).astype(np.float32)
    vals[2, 1, 1] = np.nan
    ow, oi = F.outlier_cache(vals, 4)
    avg = (vals[..., 0] + vals[..., 1] + vals[..., 2]) / np.float32(3)
    for y in range(3):
        for x in range(5):
            w, it = run(avg[:, y, x], 4)
            assert list(ow[y, x]) == pytest.approx(w) and list(oi[y, x]) == it


def test_outlier_replay_cache_views():
    """GetPixelOutlier lists the heap in array order (UnorderedItems); the "outlier-i" file layers
    list the iterations by descending priority, 0 where a pixel has fewer entries."""
    oc = OutlierReplayCache(2, 1, 4)
    oc.weight[0, 0] = [2, 5, 3, 4]
    oc.iteration[0, 0] = [1, 4, 2, 3]
    oc.weight[0, 1, :2] = [1, 3]
    oc.iteration[0, 1, :2] = [2, 0]
    q = oc.GetPixelOutlier(Pixel(0, 0))
    assert q.Count == 4 and [i.Element.Iteration for i in q.UnorderedItems] == [1, 4, 2, 3]
    assert [i.Priority for i in q.UnorderedItems] == [2, 5, 3, 4]
    best = max(q.UnorderedItems, key=lambda i: i.Priority)
    assert best.Element.Iteration == 4
    assert oc.GetPixelOutlier(Pixel(1, 0)).Count == 2
    layers = oc.outlier_layers()
    assert [float(l[0, 0]) for l in layers] == [4, 3, 2, 1]
    assert [float(l[0, 1]) for l in layers] == [0, 2, 0, 0]


def test_relmse_outlier_rejection_definition():
    rng = np.random.default_rng(3)
    ref = rng.uniform(0, 2, size=(40, 50, 3)).astype(np.float32)
    img = (ref + rng.normal(0, 0.1, size=ref.shape)).astype(np.float32)
    img[3, 4] = 1e4  # one firefly: 2000 pixels drop 2
    img[7, 8] = 1e3
    e = ((img.astype(np.float64) - ref) ** 2 / (ref.astype(np.float64) ** 2 + 0.01)).mean(axis=2)
    want = np.sort(e.ravel())[:-2].mean()
    assert F.relmse_outlier_rejection(img, ref) == pytest.approx(want, rel=1e-6)
    assert rel_mse_outlier_rejection(img, ref) == pytest.approx(F.relmse_outlier_rejection(img, ref), rel=1e-12)
    # fewer than 1000 pixels: nothing is dropped, the plain RelMSE
    small = (slice(0, 20), slice(0, 30))
    assert F.relmse_outlier_rejection(img[small], ref[small]) == pytest.approx(e[small].mean(), rel=1e-6)
