"""Loading of the golden fixtures written by tests/golden/make_golden.py."""
import gzip
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load(name):
    """(spec, inputs, reference outputs, meta) of one fixture."""
    with gzip.open(os.path.join(GOLDEN, name + ".json.gz"), "rb") as f:
        meta = json.loads(f.read())
    spec = meta["spec"]
    if "predefined" in spec:
        from kunquant_gb300.graph import predefined_spec
        spec = predefined_spec(spec["predefined"])
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    inputs = {k[4:]: z[k] for k in z.files if k.startswith("in__")}
    outputs = {k[5:]: z[k] for k in z.files if k.startswith("out__")}
    return spec, inputs, outputs, meta


def digest(a) -> str:
    """SHA-256 of an output's bytes with every NaN written as the one quiet
    NaN; large fixtures store reference outputs this way (meta["digests"])."""
    import hashlib
    a = np.array(a, copy=True)
    a[np.isnan(a)] = np.nan
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def is_stream(name):
    """Stream-mode fixtures hold the reference StreamContext's outputs."""
    with gzip.open(os.path.join(GOLDEN, name + ".json.gz"), "rb") as f:
        return bool(json.loads(f.read()).get("stream"))


def is_utility(name):
    """Fixtures of the reference's aggregrate / corrWith utilities."""
    with gzip.open(os.path.join(GOLDEN, name + ".json.gz"), "rb") as f:
        return "utility" in json.loads(f.read())["spec"]


def is_generic(name):
    """Fixtures of GenericCrossSectionalOp subclasses with their own C++
    bodies: pinned on the reference's outputs; the oracle does not run them."""
    with gzip.open(os.path.join(GOLDEN, name + ".json.gz"), "rb") as f:
        return bool(json.loads(f.read()).get("generic_cs"))


def num_time(inputs):
    """Rows of a fixture's inputs: [T][S] or STs [S/L][T][L]."""
    a = next(iter(inputs.values()))
    return a.shape[1] if a.ndim == 3 else a.shape[0]
