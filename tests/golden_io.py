"""Loading of the reference golden fixtures (tests/golden/*.npz)."""
import hashlib
import json
import os

import numpy as np

from doublyperiodicstokes_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def workload(name):
    d = load(name)["meta"]["workload"]
    return W.Workload(**d)


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    out = {k: z[k] for k in z.files if k != "meta"}
    out["meta"] = json.loads(str(z["meta"]))
    return out


def inputs(name):
    """Regenerated inputs, checked against the digest stored with the fixture."""
    g = load(name)
    w = W.Workload(**g["meta"]["workload"])
    X, F, T = W.make_inputs(w)
    h = hashlib.sha256()
    for a in (X, F, T):
        if a is not None:
            h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    if h.hexdigest() != g["meta"]["input_sha256"]:
        raise AssertionError("regenerated inputs differ from the ones the fixture was made with")
    return w, X, F, T, g


def restrict(g, A):
    """A [N][3] (or flat 3N) output restricted to the particles the fixture
    stores: all of them, or the subset g['idx'] of a full-size run."""
    A = np.asarray(A).reshape(-1, 3)
    if "idx" in g:
        A = A[g["idx"]]
    return A.ravel()
