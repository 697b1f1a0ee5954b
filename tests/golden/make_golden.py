"""Generates the golden fixtures in this directory by running the reference
CPU path itself (source/cpu of stochasticHydroTools/DoublyPeriodicStokes,
compiled unmodified by oracle/Makefile.ref and driven through its own FCM.py
by oracle/ref_harness.py).

    make -f oracle/Makefile.ref REF=$DPST_REFERENCE_ROOT/source/cpu
    python tests/golden/make_golden.py [--full]

Inputs are not stored: they are regenerated from each workload's seed
(doublyperiodicstokes_gb300.workloads.make_inputs); a SHA-256 of the input
bytes is stored with the outputs so a test can detect a generator change.
Each fixture holds V (and W with torques) from one Mdot, plus V from a second
Mdot on the same positions (the reference keeps state between calls).
"""
import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from doublyperiodicstokes_gb300 import workloads as W  # noqa: E402
import ref_harness  # noqa: E402


def input_digest(X, F, T):
    h = hashlib.sha256()
    for a in (X, F, T):
        if a is not None:
            h.update(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    return h.hexdigest()


def make(w, threads=8, subset=None):
    """One fixture.  subset = n: one Mdot only, and V (W) stored for n
    particles drawn without replacement (seed 0) from the full run, with
    their indices in `idx` (the full-size open-domain configuration, whose
    complete output would make a large fixture)."""
    X, F, T = W.make_inputs(w)
    t0 = time.time()
    r = ref_harness.run_reference(w.oracle_params(), X.ravel(), F.ravel(),
                                  None if T is None else T.ravel(), repeat=1 if subset else 2,
                                  threads=threads, timeout=6 * 3600)
    dt = time.time() - t0
    if subset:
        idx = np.sort(np.random.default_rng(0).choice(w.N, size=subset, replace=False))
        sel = (3 * idx[:, None] + np.arange(3)).ravel()
        out = dict(idx=idx, V=np.asarray(r["V"]).ravel()[sel])
        if w.has_torque:
            out["W"] = np.asarray(r["W"]).ravel()[sel]
    else:
        out = dict(V=r["V"], V_repeat=r["V_repeat"])
        if w.has_torque:
            out["W"] = r["W"]
    meta = dict(workload=w.to_dict(), input_sha256=input_digest(X, F, T), ref_seconds=dt,
                generator="tests/golden/make_golden.py via oracle/ref_harness.py")
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, w.name + ".npz"), **out)
    print("%-18s %7.1fs |V|=%.3e" % (w.name, dt, np.linalg.norm(r["V"])), flush=True)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--full", action="store_true", help="also the full-size c0, c3, c1, t0 cases")
    ap.add_argument("--only", default=None)
    ap.add_argument("--c2", action="store_true",
                    help="the full-size open-domain case (65,536 particles, 512 x 512 x 128): "
                         "one Mdot, 8,192 particles stored")
    a = ap.parse_args()
    if a.c2:
        make(W.C2, subset=8192)
        sys.exit(0)
    todo = list(W.SMALL) + list(W.SMALL_TP) + list(W.SMALL_REG) + list(W.SMALL_EDGE) + list(W.SMALL_KT)
    if a.full:
        todo += [W.C0, W.C3, W.C1, W.T0]
    for w in todo:
        if a.only and w.name != a.only:
            continue
        make(w)
