"""The uammd-compatible module driven exactly as the reference's
FCMJoint(device='gpu') drives the real one
(python_interface/common_interface_wrapper.py:76-101, 112-132), checked
against the oracle (the reference CPU path restated)."""
import numpy as np
import pytest

import dpstokes_oracle as O
from conftest import rel_err
from doublyperiodicstokes_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["s_dpbw_t", "s_dpsc_t", "s_dpbw_f_top"])
def test_fcmjoint_gpu_sequence_matches_oracle(name, monkeypatch):
    monkeypatch.setenv("DPSTOKES_GB300_PRECISION", "double")
    from doublyperiodicstokes_gb300 import uammd
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    R = w.radius
    hx = w.Lx / w.nx
    cbeta, cbeta_d = R / (w.wm * hx), R / (w.wd * hx)  # GridAndKernelConfig.py:328-329
    mode = {"DP": "nowall", "DPBW": "bottom", "DPSC": "slit"}[w.domType]
    par = uammd.StokesParameters(viscosity=w.eta, Lx=w.Lx, Ly=w.Ly, zmin=0, zmax=w.Lz,
                                 w=w.wm, w_d=w.wd if w.has_torque else 0,
                                 beta=w.betam_hat * w.wm,
                                 beta_d=(w.betad_hat * w.wd) if w.has_torque else 0,
                                 alpha=R / (2 * cbeta * hx),
                                 alpha_d=R / (2 * cbeta_d * hx) if w.has_torque else 0,
                                 nx=w.nx, ny=w.ny, nz=w.nz, mode=mode)
    assert uammd.getPrecision() == "double"
    s = uammd.DPStokes()
    s.initialize(par, w.N)
    s.setPositions(np.float64(X.ravel()))
    MF = np.zeros(3 * w.N)
    MT = np.zeros(3 * w.N if w.has_torque else 0)
    s.Mdot(forces=np.float64(F.ravel()), torques=np.float64(T.ravel()) if T is not None else np.empty(0),
           velocities=MF, angularVelocities=MT)
    Vo, Wo = O.mdot(O.Params(**w.oracle_params()), X, F, T)
    assert rel_err(MF, Vo) < 1e-10
    if w.has_torque:
        assert rel_err(MT, Wo) < 1e-10
    s.clear()
    with pytest.raises(RuntimeError):
        s.setPositions(np.float64(X.ravel()))
