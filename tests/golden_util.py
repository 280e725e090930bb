"""Loading the golden fixtures of tests/golden/ and rebuilding their inputs."""
import os

import numpy as np

from tests.golden.cases import CASES, input_digest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(HERE, f"{name}.npz")) as f:
        return {k: f[k] for k in f.files}


def build_inputs(name):
    """(case, workload, fixture): the workload rebuilt from its seeds, with the fixture's stored
    per-cell fields; asserts that the other inputs hash to the fixture's digest."""
    case = CASES[name]
    fx = load(name)
    w = case.build()
    assert input_digest(w, case) == str(fx["input_sha"]), f"{name}: inputs differ from the fixture's"
    if "Ks" in fx:
        w.Ks = fx["Ks"]
    if "alpha" in fx:
        w.alpha = fx["alpha"]
    return case, w, fx
