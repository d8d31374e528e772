"""Shared test helpers: the reference's test clouds, its query generator and
its result checks, restated (tests/helpers.h, tests/knnvalidate.cpp)."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# tests/CMakeLists.txt:9-14 -- (cloud, K, dim, method, maxRadius)
KNNVALIDATE_CASES = [
    ("scan_2d", 10, 2, -1, np.inf),
    ("scan_2d", 10, 2, 10000, np.inf),
    ("scan_3d", 10, 3, -1, np.inf),
    ("scan_3d", 10, 3, 10000, np.inf),
    ("scan_3d_large", 10, 3, 1000, np.inf),
    ("scan_3d_large", 10, 3, 1000, 0.5),
]

ALLOW_SELF_MATCH = 1
SORT_RESULTS = 2
TOUCH_STATISTICS = 1


def reference_scans() -> dict:
    with np.load(os.path.join(GOLDEN, "reference_scans.npz")) as z:
        return {k: z[k] for k in z.files}


def create_query(cloud: np.ndarray, it_count: int, method: int, seed: int = 0) -> np.ndarray:
    """tests/helpers.h:82-126 with the brute-force (true) bounds.

    method < 0: 2N queries, point i % N shifted by +-(sum of box extents)/(-method);
    method > 0: `method` queries uniform in the bounding box (seeded numpy
    instead of the unseeded rand()).
    """
    T = cloud.dtype.type
    lo = cloud.min(axis=0)
    hi = cloud.max(axis=0)
    n = cloud.shape[0]
    if method < 0:
        absb = T(np.sum((hi - lo).astype(T), dtype=T)) / T(-method)
        i = np.arange(it_count)
        q = cloud[i % n].copy()
        q[i < n] += absb
        q[i >= n] -= absb
        return q.astype(cloud.dtype)
    rng = np.random.default_rng(seed)
    u = rng.random((it_count, cloud.shape[1])).astype(cloud.dtype)
    return (lo + u * (hi - lo)).astype(cloud.dtype)


def knnvalidate_check(cloud, q, idx_bf, d2_bf, idx_other, label=""):
    """tests/knnvalidate.cpp:177-213: for each rank whose brute-force distance is
    finite, the other method's point must be valid and at the same squared
    distance to within numeric_limits<T>::epsilon()."""
    T = cloud.dtype.type
    eps = np.finfo(cloud.dtype).eps
    valid = np.isfinite(d2_bf)
    assert (idx_other[valid] >= 0).all() and (idx_other[valid] < cloud.shape[0]).all(), f"{label}: invalid index"
    qi = np.nonzero(valid)[0]
    pbf = cloud[idx_bf[valid]]
    pot = cloud[idx_other[valid]]
    pq = q[qi]
    dbf = np.sum(((pbf - pq) ** 2).astype(T), axis=1, dtype=T)
    dot = np.sum(((pot - pq) ** 2).astype(T), axis=1, dtype=T)
    diff = np.abs(dbf - dot)
    bad = np.nonzero(diff > eps)[0]
    assert bad.size == 0, f"{label}: {bad.size} ranks differ (first at query {qi[bad[0]]}, dist2 diff {diff[bad[0]]})"
    return int(valid.sum())


def assert_identical(idx_a, d2_a, idx_b, d2_b, label=""):
    """Bit-exact equality of indices and squared distances (inf included)."""
    assert idx_a.shape == idx_b.shape, f"{label}: shapes {idx_a.shape} vs {idx_b.shape}"
    bad = np.nonzero((idx_a != idx_b).any(axis=1))[0]
    assert bad.size == 0, (f"{label}: {bad.size} queries differ in indices; first q={bad[0]}: "
                           f"{idx_a[bad[0]]} vs {idx_b[bad[0]]} / {d2_a[bad[0]]} vs {d2_b[bad[0]]}")
    same = (d2_a == d2_b) | (np.isinf(d2_a) & np.isinf(d2_b))
    bad = np.nonzero(~same.all(axis=1))[0]
    assert bad.size == 0, f"{label}: {bad.size} queries differ in dists2; first q={bad[0]}: {d2_a[bad[0]]} vs {d2_b[bad[0]]}"


def assert_equal_up_to_ties(idx_a, d2_a, idx_b, d2_b, label=""):
    """Same squared distances per query; the same indices for every distance
    value except exact ties at the k-th place, where only counts must match
    (the reference keeps the first visited of tied points)."""
    da = np.sort(d2_a, axis=1)
    db = np.sort(d2_b, axis=1)
    same = (da == db) | (np.isinf(da) & np.isinf(db))
    bad = np.nonzero(~same.all(axis=1))[0]
    assert bad.size == 0, f"{label}: {bad.size} queries differ in dists2; first q={bad[0]}: {da[bad[0]]} vs {db[bad[0]]}"
    diff = np.nonzero((np.sort(idx_a, axis=1) != np.sort(idx_b, axis=1)).any(axis=1))[0]
    for i in diff:
        last = da[i][-1]
        for v in np.unique(da[i]):
            sa = set(idx_a[i][d2_a[i] == v].tolist())
            sb = set(idx_b[i][d2_b[i] == v].tolist())
            if v == last:
                assert len(sa) == len(sb), f"{label}: query {i} boundary tie counts differ"
            else:
                assert sa == sb, f"{label}: query {i} neighbours at dist2 {v} differ: {sa} vs {sb}"
    return len(diff)


def check_sorted_and_consistent(cloud, q, idx, d2, k):
    """Size-independent properties of a result: ascending (dist2, index) order,
    -1/+inf padding only at the end, and every returned dist2 equal to the
    sequentially summed squared distance of the returned point."""
    T = cloud.dtype.type
    valid = idx >= 0
    assert ((~valid) <= np.isinf(d2)).all(), "unfound slots must hold +inf"
    # padding only after valid entries
    assert (np.diff(valid.astype(np.int8), axis=1) <= 0).all(), "unfound slots must be last"
    dd = np.where(valid, d2, np.inf)
    ii = np.where(valid, idx, np.iinfo(np.int32).max).astype(np.int64)
    step_ok = (dd[:, 1:] > dd[:, :-1]) | ((dd[:, 1:] == dd[:, :-1]) & (ii[:, 1:] >= ii[:, :-1]))
    assert step_ok.all(), "results must ascend by (dist2, index)"
    rows, cols = np.nonzero(valid)
    p = cloud[idx[rows, cols]].astype(T)
    qq = q[rows].astype(T)
    acc = np.zeros(rows.shape[0], dtype=T)
    for d in range(cloud.shape[1]):
        diff = (qq[:, d] - p[:, d]).astype(T)
        acc = (acc + (diff * diff).astype(T)).astype(T)
    assert (acc == d2[rows, cols]).all(), "returned dists2 must equal the recomputed squared distances"
