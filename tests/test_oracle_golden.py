"""The oracle (CPU restatement) against outputs of the reference itself.

Fixtures were produced by the reference CPU executor built from its own
sources (tests/golden/make_golden.py).  Every output must be bit-identical,
except a few window-10 statistics where the reference's GCC build contracts
multiply-adds after jump threading at the start of the window; those must
agree to 1e-5 relative (1e-6 absolute) with identical NaN positions.
"""
import numpy as np
import pytest

from oracle.oracle import OracleProgram
from tests import golden_util as G
from tests.parity import compare_close, compare_exact

KNOWN_INEXACT = {
    "alpha101": {"alpha006", "alpha014", "alpha040"},
    "alpha158": {"STD10", "CORR10", "VSTD10"},
}


def known_inexact(name):
    for prefix, outs in KNOWN_INEXACT.items():
        if name.startswith(prefix):
            return outs
    return set()


BATCH = [n for n in G.names() if not G.is_stream(n)]


@pytest.mark.parametrize("name", BATCH)
def test_oracle_matches_reference(name):
    spec, inp, ref, meta = G.load(name)
    start = meta.get("cur_time", 0)
    T = next(iter(inp.values())).shape[0]
    out = OracleProgram(spec).run(inp, cur_time=start, length=T - start)
    assert set(out) == set(ref)
    bad = compare_exact(out, ref)
    allowed = known_inexact(name)
    assert set(bad) <= allowed, f"outputs differing from the reference: {sorted(set(bad) - allowed)}"
    close = compare_close(out, ref, 1e-5, 1e-6)
    assert not close, f"outputs outside 1e-5: {close}"


def test_issue19_known_answer():
    """ArgMin with ties picks the oldest minimum (reference issue #19)."""
    spec, inp, ref, _ = G.load("argmin_issue19")
    out = OracleProgram(spec).run(inp)
    # window [.6898 .6992 .6992 .6968 .6968]: the minimum is the oldest value;
    # window [.6992 .6992 .6968 .6968 .6968]: the oldest of the tied minima
    np.testing.assert_array_equal(out["ou2"][4], np.full(8, 1.0, np.float32))
    np.testing.assert_array_equal(out["ou2"][5], np.full(8, 3.0, np.float32))
    np.testing.assert_array_equal(out["ou2"], ref["ou2"])
