"""ORACLE frame-buffer bookkeeping -- test infrastructure only.

CPU restatements, in plain Python / numpy, of two pieces of SeeSharp's frame buffer that the GPU
film fold also computes.  Imported by tests/ only; never by the product package.

* The outlier replay cache (SeeSharp/Integrators/Util/OutlierReplayCache.cs:9-35, notified from
  FrameBuffer.Splat, SeeSharp/Images/FrameBuffer.cs:187-190).  Per pixel it keeps the n samples
  of largest channel average in a .NET `System.Collections.Generic.PriorityQueue<TElement,
  TPriority>` (the .NET 9 base class library; not part of the reference's sources).  Its
  published implementation is a 4-ary min-heap stored in an array: `Enqueue` appends and sifts
  up while the node's priority is strictly below its parent's; `EnqueueDequeue` replaces the root
  only when the new priority is strictly above the root's, then sifts down, each step to the first
  child of least priority, while that child's priority is strictly below the node's.
  `UnorderedItems` lists the array.  Parity of the array order is unpinned (no .NET runtime
  here); the kept set (the n largest; a sample that only ties the smallest kept one does not
  enter) follows from the reference's own code and is pinned by the tests' hand-worked cases.

* RelMSE with outlier rejection (FrameBuffer.ComputeErrorMetric, FrameBuffer.cs:378-383), which
  SimpleImageIO 1.8.3 (`Metrics.RelMSE_OutlierRejection`, not vendored) computes.  The definition
  restated here and used by the GPU: per pixel the mean over the channels of (x - r)^2 / (r^2 +
  0.01), the largest floor(pixels * 0.1 / 100) dropped, the rest averaged.  Parity unpinned.
"""
from __future__ import annotations

import numpy as np

ARITY = 4


def heap_notify(w, it, n, priority, iteration):
    """One OutlierReplayCache.Notify on one pixel's heap (lists w, it of the occupied slots)."""
    if len(w) < n:
        # PriorityQueue.Enqueue: append, sift up
        k = len(w)
        w.append(priority)
        it.append(iteration)
        while k > 0:
            parent = (k - 1) // ARITY
            if not priority < w[parent]:
                break
            w[k], it[k] = w[parent], it[parent]
            k = parent
        w[k], it[k] = priority, iteration
        return
    if len(w) == 0 or not priority > w[0]:
        return  # PriorityQueue.EnqueueDequeue hands the new element straight back
    k = 0
    while True:
        c = ARITY * k + 1
        if c >= len(w):
            break
        m = c
        for j in range(c + 1, min(c + ARITY, len(w))):
            if w[j] < w[m]:
                m = j
        if priority <= w[m]:
            break
        w[k], it[k] = w[m], it[m]
        k = m
    w[k], it[k] = priority, iteration


def outlier_cache(values, n):
    """values: (iterations, H, W, 3) float32 per-iteration sample values of every pixel (the splatted
    estimate).  Returns (weights (H, W, n) float32, iterations (H, W, n) int32, -1 for empty)."""
    values = np.asarray(values, np.float32)
    S, H, W, _ = values.shape
    avg = (values[..., 0] + values[..., 1] + values[..., 2]) / np.float32(3)
    ow = np.zeros((H, W, n), np.float32)
    oi = np.full((H, W, n), -1, np.int32)
    for y in range(H):
        for x in range(W):
            w, it = [], []
            for s in range(S):
                a = avg[s, y, x]
                if np.isfinite(a):
                    heap_notify(w, it, n, float(a), s)
            ow[y, x, :len(w)] = w
            oi[y, x, :len(it)] = it
    return ow, oi


def relmse_outlier_rejection(image, reference, percentage=0.1):
    """Per-pixel relative squared errors (float32, channel mean computed in double), the largest
    floor(pixels * percentage / 100) dropped, the mean of the rest in double."""
    x = np.asarray(image, np.float32)
    r = np.asarray(reference, np.float32)
    d = (x - r).astype(np.float64)
    r2 = r.astype(np.float64) ** 2 + 0.01
    e = ((d[..., 0] ** 2 / r2[..., 0] + d[..., 1] ** 2 / r2[..., 1]) + d[..., 2] ** 2 / r2[..., 2]) / 3.0
    e = np.sort(e.astype(np.float32).ravel())
    k = int(e.size * percentage / 100)
    kept = e[:e.size - k].astype(np.float64)
    return float(kept.sum() / kept.size)
