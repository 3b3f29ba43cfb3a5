"""Precision of the fp32 Alpha158 forms against the reference's FP64 TS build.

Five fp32 forms run on the GPU over the same seeded inputs:
  * ``alpha158``       -- the reference's default fp32 build: two-pass window
                          moments, Kahan window sums, fp32 regression sums;
  * ``alpha158_fast``  -- the fast-stat build: rolling moments in
                          Kahan-compensated fp32 accumulators;
  * ``alpha158_mixed`` -- the default build with its rolling states (Kahan
                          window sums, regression sums) in two-float
                          compensated fp32, window loops unchanged;
  * ``alpha158_comp``  -- fp32 factor arithmetic with every running sum
                          (Kahan window sums, window reductions, regression
                          sums) in two-float compensated fp32;
  * ``alpha158_acc64`` -- the same running sums in fp64 on the GPU;
  * ``alpha158_slide`` -- window moments expanded into two-float sliding
                          window sums, scans in time chunks (slide.py).
The FP64 oracle (the reference's fp64 TS build restated) is the truth.  For
each factor the relative error is |got - want| / max(|want|, 1e-3 * m), m the
factor's median |want| (a floor so that values crossing zero do not divide by
~0), over the cells where both are numbers; NaN cells that differ are
counted apart.  ``KUN_PRECISION_REPORT=<path>`` writes the per-factor table.
"""
import os

import numpy as np
import pytest

from kunquant_gb300 import runner as kr
from kunquant_gb300 import synth
from kunquant_gb300.graph import predefined_spec
from oracle.oracle import OracleProgram

FORMS = [("alpha158_f32", "alpha158"), ("alpha158_fast_f32", "alpha158_fast"),
         ("alpha158_mixed_f32", "alpha158_mixed"), ("alpha158_comp_f32", "alpha158_comp"),
         ("alpha158_acc64_f32", "alpha158_acc64"), ("alpha158_slide_f32", "alpha158_slide")]


def _errors(got, want):
    out = {}
    for k, w in want.items():
        g = np.asarray(got[k], np.float64)
        both = ~np.isnan(w) & ~np.isnan(g)
        nanmis = int((np.isnan(w) != np.isnan(g)).sum())
        if both.any():
            m = np.median(np.abs(w[both]))
            rel = np.abs(g[both] - w[both]) / np.maximum(np.abs(w[both]), 1e-3 * m + 1e-30)
            out[k] = (float(rel.max()), float(np.median(rel)), nanmis)
        else:
            out[k] = (0.0, 0.0, nanmis)
    return out


@pytest.mark.gpu
def test_alpha158_precision_vs_fp64():
    S, T = 256, 600
    d32 = synth.ohlcv(S, T, seed=21, nan_frac=0.005)
    want = OracleProgram(predefined_spec("alpha158_f64")).run({k: v.astype(np.float64) for k, v in d32.items()})
    ex = kr.createSingleThreadExecutor()
    stats = {}
    for key, name in FORMS:
        mod = kr.Library.predefined(key).getModule(name)
        stats[name] = _errors(kr.runGraph(ex, mod, d32, 0, T), want)
    names = sorted(want)
    lines = ["| factor | " + " | ".join(f"{n} max | {n} median | {n} NaN diff" for _, n in FORMS) + " |",
             "|---|" + "---|---|---|" * len(FORMS)]
    for f in names:
        cells = []
        for _, n in FORMS:
            mx, md, nm = stats[n][f]
            cells += [f"{mx:.1e}", f"{md:.1e}", str(nm)]
        lines.append(f"| {f} | " + " | ".join(cells) + " |")
    summary = []
    for _, n in FORMS:
        mx = np.array([stats[n][f][0] for f in names])
        md = np.array([stats[n][f][1] for f in names])
        nm = sum(stats[n][f][2] for f in names)
        summary.append(f"{n}: factors with max <= 1e-5: {(mx <= 1e-5).sum()}/{len(names)}, "
                       f"median <= 1e-5: {(md <= 1e-5).sum()}/{len(names)}, worst median {md.max():.1e}, "
                       f"NaN cells differing {nm}")
    report = "\n".join(summary + [""] + lines) + "\n"
    print(report)
    path = os.environ.get("KUN_PRECISION_REPORT")
    if path:
        with open(path, "w") as f:
            f.write(report)
    # fp64 running sums: every factor's median error within 1e-5, the same
    # NaN cells as fp64, and more factors within 1e-5 everywhere than the
    # reference's own fp32 build
    acc = stats["alpha158_acc64"]
    base = stats["alpha158"]
    assert all(acc[f][1] <= 1e-5 for f in names), [f for f in names if acc[f][1] > 1e-5]
    assert sum(acc[f][2] for f in names) == 0
    assert sum(acc[f][0] <= 1e-5 for f in names) > sum(base[f][0] <= 1e-5 for f in names)
    # the compensated fp32 sums hold the same bound
    comp = stats["alpha158_comp"]
    assert all(comp[f][1] <= 1e-5 for f in names), [f for f in names if comp[f][1] > 1e-5]
    assert sum(comp[f][2] for f in names) == 0
    # maximum error: with fp64 or two-float running sums every factor is
    # within 1e-5 of fp64 everywhere, except those whose loss is in the fp32
    # factor arithmetic around the sums (the deviations from a window mean
    # in CORR/CORD, the difference of two sums in VSUMD, the ratio in WVMA
    # at short windows); for them the two forms agree with each other
    ill = [f for f in names if f.startswith(("CORR", "CORD", "VSUMD")) or f in ("WVMA5", "WVMA10")]
    for form in ("alpha158_acc64", "alpha158_comp"):
        over = [f for f in names if stats[form][f][0] > 1e-5]
        assert set(over) <= set(ill), (form, sorted(set(over) - set(ill)))
    for f in ill:
        a, c = acc[f][0], comp[f][0]
        assert c <= 2 * a + 1e-5, (f, c, a)
    # compensating only the rolling states already holds every median
    mixed = stats["alpha158_mixed"]
    assert all(mixed[f][1] <= 1e-5 for f in names), [f for f in names if mixed[f][1] > 1e-5]
    assert sum(mixed[f][2] for f in names) == 0
