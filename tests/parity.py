"""Comparison helpers shared by the parity tests."""
import numpy as np


def bits_equal(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Element-wise: identical bits, or both NaN (NaN payloads may differ
    between CPU and GPU)."""
    u = np.uint32 if a.dtype == np.float32 else np.uint64
    return (a.view(u) == b.view(u)) | (np.isnan(a) & np.isnan(b))


def compare_exact(got: dict, want: dict, names=None):
    """Returns {name: (mismatches, first index, got, want)} for outputs that
    are not bit-identical."""
    bad = {}
    for k in (names or want.keys()):
        g, w = np.asarray(got[k]), np.asarray(want[k])
        assert g.shape == w.shape, (k, g.shape, w.shape)
        eq = bits_equal(g, w)
        if not eq.all():
            idx = tuple(np.argwhere(~eq)[0])
            bad[k] = (int((~eq).sum()), idx, g[idx], w[idx])
    return bad


def compare_close(got: dict, want: dict, rtol: float, atol: float, names=None):
    """NaN positions identical and |got - want| <= atol + rtol * |want|."""
    bad = {}
    for k in (names or want.keys()):
        g, w = np.asarray(got[k]).astype(np.float64), np.asarray(want[k]).astype(np.float64)
        nan_g, nan_w = np.isnan(g), np.isnan(w)
        ok = (nan_g == nan_w)
        m = ~nan_g & ~nan_w
        ok[m] = np.abs(g[m] - w[m]) <= atol + rtol * np.abs(w[m])
        inf = np.isinf(w) & m
        ok[inf] = g[inf] == w[inf]
        if not ok.all():
            idx = tuple(np.argwhere(~ok)[0])
            bad[k] = (int((~ok).sum()), idx, g[idx], w[idx])
    return bad
