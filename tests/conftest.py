import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLDEN)
# The reference tree (its src/ and examples/), when a test may read it in
# place; tests that need it skip where the variable is unset.
REF_ROOT = os.environ.get("MAPPG_REFERENCE_ROOT") or None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmappg.so")


@pytest.fixture(scope="session")
def potentials(tmp_path_factory):
    """Analytic setfl files (A and A/B) written afresh, with their digests."""
    import hashlib

    from mapp4py_gb300 import synth

    d = tmp_path_factory.mktemp("pot")
    out = {}
    for elems in (("A",), ("A", "B")):
        p = str(d / ("%s.setfl" % "".join(elems)))
        synth.write_setfl(p, elems)
        with open(p, "rb") as fh:
            out[elems] = (p, hashlib.sha256(fh.read()).hexdigest())
    return out


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_potential(potentials, g):
    elems = tuple(str(e) for e in g["elems"]) if "elems" in g else ("A",) if g["masses"].shape[0] == 1 else ("A", "B")
    path, digest = potentials[elems]
    assert str(g["sha256"]) == digest, "regenerated potential differs from the one behind the fixture"
    return path
