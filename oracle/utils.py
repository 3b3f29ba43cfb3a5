"""CPU restatement of the reference's utilities -- TEST INFRASTRUCTURE.

* aggregrate (cpp/Kun/Aggregration.cpp:12-106): per stock, over runs of equal
  consecutive labels: Kahan sum (cpp/Kun/Ops.hpp:469-477), NaN-sticky min/max
  (Ops.hpp:488-505), first, last, count and mean = sum / count, every step in
  the buffer dtype.
* corr_with (cpp/Kun/CorrWith.hpp:12-121): the cross-sectional correlation of
  each row, (XY - X*Y) / (sqrt(X2 - X*X) * sqrt(Y2 - Y*Y)) of the row means,
  here in float64 (the reference sums in fp32 in stock order).
  rank_inputs ranks each input row as Rank does (Rank.hpp:13-57).
Only tests use this module.
"""
import numpy as np

KINDS = ["sum", "min", "max", "first", "last", "count", "mean"]


def aggregrate(x: np.ndarray, labels: np.ndarray):
    """{kind: [groups][S]} of input x [T][S] (float32 or float64)."""
    dt = x.dtype.type
    T, S = x.shape
    groups = []
    start = 0
    for t in range(1, T + 1):
        if t == T or labels[t] != labels[t - 1]:
            groups.append((start, t))
            start = t
    out = {k: np.empty((len(groups), S), x.dtype) for k in KINDS}
    for g, (a, b) in enumerate(groups):
        v = np.zeros(S, x.dtype)
        c = np.zeros(S, x.dtype)
        mn = np.full(S, np.inf, x.dtype)
        mx = np.full(S, -np.inf, x.dtype)
        for t in range(a, b):
            cur = x[t]
            y = (cur - c).astype(x.dtype)
            tt = (v + y).astype(x.dtype)
            c = ((tt - v).astype(x.dtype) - y).astype(x.dtype)
            v = tt
            nan = np.isnan(mn) | np.isnan(cur)
            mn = np.where(nan, np.nan, np.where(mn < cur, mn, cur)).astype(x.dtype)
            nan = np.isnan(mx) | np.isnan(cur)
            mx = np.where(nan, np.nan, np.where(mx > cur, mx, cur)).astype(x.dtype)
        cnt = np.full(S, dt(b - a), x.dtype)
        out["sum"][g] = v
        out["min"][g] = mn
        out["max"][g] = mx
        out["first"][g] = x[a]
        out["last"][g] = x[b - 1]
        out["count"][g] = cnt
        out["mean"][g] = (v / cnt).astype(x.dtype)
    return out


def _rank_row(row: np.ndarray) -> np.ndarray:
    ok = ~np.isnan(row)
    vals = np.sort(row[ok])
    n = len(vals)
    out = np.full(row.shape, np.nan, row.dtype)
    lo = np.searchsorted(vals, row[ok], "left")
    hi = np.searchsorted(vals, row[ok], "right")
    s = (lo + hi + 1) * (hi - lo) // 2
    out[ok] = ((s.astype(row.dtype) / (hi - lo).astype(row.dtype)) / row.dtype.type(n)).astype(row.dtype)
    return out


def corr_with(x: np.ndarray, y: np.ndarray, rank_inputs: bool = False) -> np.ndarray:
    """Per-row correlation of x and y ([T][S]); float64 moments."""
    if rank_inputs:
        x = np.stack([_rank_row(r) for r in x])
    a = x.astype(np.float64)
    b = y.astype(np.float64)
    S = a.shape[1]
    X, Y = a.sum(1) / S, b.sum(1) / S
    X2, Y2, XY = (a * a).sum(1) / S, (b * b).sum(1) / S, (a * b).sum(1) / S
    with np.errstate(invalid="ignore", divide="ignore"):
        return (XY - X * Y) / (np.sqrt(X2 - X * X) * np.sqrt(Y2 - Y * Y))
