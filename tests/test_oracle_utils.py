"""The utilities' CPU restatement (oracle/utils.py) against the reference's
own aggregrate and corrWith outputs (tests/golden/util_*)."""
import numpy as np
import pytest

from oracle import utils as U
from tests import golden_util as G
from tests.parity import compare_exact


@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_aggregrate_oracle_matches_reference(tag):
    _, inp, ref, _ = G.load("util_aggregrate_" + tag)
    for name in ("a", "b"):
        got = U.aggregrate(inp[name], inp["labels"])
        want = {k: ref[f"{name}_{k}"] for k in U.KINDS}
        assert not compare_exact(got, want), name


def test_corrwith_oracle_matches_reference():
    _, inp, ref, _ = G.load("util_corrwith")
    for name in ("a", "b"):
        np.testing.assert_allclose(U.corr_with(inp[name], inp["ret"]), ref[name], rtol=1e-4, atol=1e-6)
        np.testing.assert_allclose(U.corr_with(inp[name], inp["ret"], rank_inputs=True), ref["rank_" + name],
                                   rtol=1e-4, atol=1e-6)
