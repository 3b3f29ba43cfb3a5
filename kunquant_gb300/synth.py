"""Seeded synthetic OHLCV market data in the [T][S] ("TS") layout.

Distribution (per stock):
  close_0 ~ U(10, 100)             (or log-uniform in [lo, hi] via ``price_range``)
  daily log-returns ~ N(0, 0.02),  close_t = close_0 * exp(cumsum(r))
  open_t  = close_{t-1} * exp(N(0, 0.005))       (close_{-1} = close_0)
  high_t  = max(open_t, close_t) * (1 + |N(0, 0.01)|)
  low_t   = min(open_t, close_t) * (1 - |N(0, 0.01)|)
  volume  ~ LogNormal(13, 1),     amount = volume * (open + close) / 2
Optionally a fraction of cells of every field is set to NaN uniformly at random.
No public data set is involved; this stands in for daily market bars.
"""
import numpy as np

FIELDS = ("open", "high", "low", "close", "volume", "amount")


def ohlcv(num_stocks: int, num_time: int, seed: int = 0, nan_frac: float = 0.0,
          price_range=None, dtype=np.float32) -> dict:
    rng = np.random.default_rng(seed)
    S, T = num_stocks, num_time
    if price_range is None:
        c0 = rng.uniform(10.0, 100.0, size=S)
    else:
        lo, hi = price_range
        c0 = np.exp(rng.uniform(np.log(lo), np.log(hi), size=S))
    r = rng.normal(0.0, 0.02, size=(T, S))
    close = c0[None, :] * np.exp(np.cumsum(r, axis=0))
    prev = np.vstack([c0[None, :], close[:-1]])
    open_ = prev * np.exp(rng.normal(0.0, 0.005, size=(T, S)))
    high = np.maximum(open_, close) * (1.0 + np.abs(rng.normal(0.0, 0.01, size=(T, S))))
    low = np.minimum(open_, close) * (1.0 - np.abs(rng.normal(0.0, 0.01, size=(T, S))))
    volume = rng.lognormal(13.0, 1.0, size=(T, S))
    amount = volume * (open_ + close) / 2.0
    out = {"open": open_, "high": high, "low": low, "close": close, "volume": volume,
           "amount": amount}
    for k in FIELDS:
        a = out[k].astype(dtype)
        if nan_frac > 0:
            m = rng.random(size=(T, S)) < nan_frac
            a[m] = np.nan
        out[k] = np.ascontiguousarray(a)
    return out
