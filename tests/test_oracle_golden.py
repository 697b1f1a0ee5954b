"""The oracle (numpy restatement) against outputs of the reference CPU path
itself (tests/golden, made by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

import dpstokes_oracle as O
import golden_io
from conftest import rel_err

SMALL = [n for n in golden_io.names() if n.startswith(("s_", "e_"))]
FULL = [n for n in golden_io.names() if not n.startswith(("s_", "e_"))]


def _check(name, tol):
    w, X, F, T, g = golden_io.inputs(name)
    V, Wv = O.mdot(O.Params(**w.oracle_params()), X, F, T)
    assert rel_err(golden_io.restrict(g, V), g["V"]) < tol
    if "V_repeat" in g:
        assert rel_err(g["V_repeat"], g["V"]) == 0.0
    if w.has_torque:
        assert rel_err(golden_io.restrict(g, Wv), g["W"]) < tol


@pytest.mark.parametrize("name", SMALL)
def test_oracle_matches_reference_small(name):
    _check(name, 1e-13)


@pytest.mark.parametrize("name", [n for n in FULL if n.startswith(("c0", "t0"))])
def test_oracle_matches_reference_c0_t0(name):
    _check(name, 1e-13)


@pytest.mark.slow
@pytest.mark.parametrize("name", [n for n in FULL if not n.startswith(("c0", "t0", "c2"))])
def test_oracle_matches_reference_full(name):
    _check(name, 1e-13)


@pytest.mark.slow
@pytest.mark.skipif(os.environ.get("DPST_FULL_SIZE_ORACLE") != "1",
                    reason="the 65,536-particle 512 x 512 x 128 oracle run takes minutes and ~15 GB; "
                           "set DPST_FULL_SIZE_ORACLE=1")
def test_oracle_matches_reference_c2():
    _check("c2_dp_n65536", 1e-13)


def test_oracle_rejects_asymmetric_ghost_extension():
    # Nz=19, Lz=12: node 6 sits exactly at distance thr = 3 from the top but
    # not from the bottom; the reference overruns its interior grid here.
    p = O.Params("DP", 16, 16, 19, 16.0, 16.0, 12.0, has_torque=False)
    o = O.Oracle(p)
    with pytest.raises(ValueError):
        o.set_positions(np.array([[8.0, 8.0, 6.0]]))


def test_oracle_linearity_and_translation():
    """Mdot is linear in (F, T) and invariant to periodic shifts by whole cells."""
    from doublyperiodicstokes_gb300 import workloads as W
    # slit channel: no open ends, so no reuse of ghost-layer spread data, which
    # the reference folds only partially in x and y (not shift invariant)
    w = W.SMALL_BY_NAME["s_dpsc_t"]
    X, F, T = W.make_inputs(w)
    p = O.Params(**w.oracle_params())
    o = O.Oracle(p)
    o.set_positions(X)
    V1, W1 = o.mdot(F, T)
    V2, W2 = o.mdot(2.0 * F, 2.0 * T)
    Vs, Ws = o.mdot(3.0 * F, 3.0 * T)
    assert rel_err(Vs, V1 + V2) < 1e-13
    assert rel_err(Ws, W1 + W2) < 1e-13
    Xs = X.copy()
    Xs[:, 0] = np.mod(Xs[:, 0] + 3 * p.hx, p.Lx)
    o2 = O.Oracle(p)
    o2.set_positions(Xs)
    V3, W3 = o2.mdot(F, T)
    assert rel_err(V3, V1) < 1e-12
    assert rel_err(W3, W1) < 1e-12


def test_oracle_tp_shift_invariance():
    """Triply periodic: shifting every particle by whole cells along any axis
    (wrapping into the box) leaves Mdot unchanged up to rounding."""
    from doublyperiodicstokes_gb300 import workloads as W
    w = W.SMALL_BY_NAME["s_tp_t_hz"]
    X, F, T = W.make_inputs(w)
    p = O.Params(**w.oracle_params())
    V1, W1 = O.mdot(p, X, F, T)
    Xs = X.copy()
    Xs[:, 0] = np.mod(Xs[:, 0] + 2 * p.hx, p.Lx)
    Xs[:, 2] = np.mod(Xs[:, 2] + 7 * p.hz, p.Lz)
    V2, W2 = O.mdot(p, Xs, F, T)
    assert rel_err(V2, V1) < 1e-12
    assert rel_err(W2, W1) < 1e-12


def test_edge_positions_inside_the_cell():
    """Edge layouts keep x < Lx, y < Ly (and z < zmax in the triply periodic
    box), and hit the z ends exactly where the reference allows it."""
    from doublyperiodicstokes_gb300 import workloads as W
    for w in W.SMALL_EDGE:
        X, _, _ = W.make_inputs(w)
        assert X.shape == (w.N, 3)
        assert (X[:, 0] >= 0).all() and (X[:, 0] < w.Lx).all()
        assert (X[:, 1] >= 0).all() and (X[:, 1] < w.Ly).all()
        assert (X[:, 2] >= w.z0).all() and (X[:, 2] <= w.z0 + w.Lz).all()
        assert (X[:, 2] == w.z0).any()
        if w.domType == "TP":
            assert (X[:, 2] < w.z0 + w.Lz).all()
        else:
            assert (X[:, 2] == w.z0 + w.Lz).any()
