"""Golden vectors of the reference's grid and kernel configuration
(source/cpu/python/GridAndKernelConfig.py), generated by importing the
reference module itself: python tests/golden/make_gridconfig_golden.py
(DPST_REFERENCE_ROOT names the reference checkout).  Writes
tests/golden/gridconfig.json, which tests/test_gridconfig.py compares
doublyperiodicstokes_gb300.gridconfig against."""
import contextlib
import io
import json
import os
import sys

import numpy as np

REF = os.environ["DPST_REFERENCE_ROOT"]
HERE = os.path.dirname(os.path.abspath(__file__))

XY = [  # Lx, Ly, radii, kernel types, optInd, has_torque, ref
    (128.0, 128.0, [1.0], [0], -1, False, False),
    (128.0, 128.0, [1.0], [0], 0, False, False),
    (128.0, 128.0, [1.0], [0], 3, False, False),
    (256.0, 256.0, [1.0], [1], 0, False, False),
    (100.0, 80.0, [1.3], [2], 1, False, False),
    (64.0, 64.0, [0.5], [0], 0, False, True),
    (90.0, 90.0, [1.0, 1.5], [0, 0], 0, False, False),
    (512.0, 512.0, [1.0], [0], -1, True, False),
    (512.0, 512.0, [1.0], [0], 0, True, False),
    (200.0, 200.0, [1.2], [1], 2, True, False),
    (150.0, 150.0, [1.0], [3], 0, True, False),
    (150.0, 150.0, [1.0], [4], 1, True, False),
    (150.0, 150.0, [1.0], [5], 0, True, True),
    (60.0, 60.0, [1.0], [2], 0, True, False),   # unsupported with torques
    (60.0, 60.0, [1.0], [9], 0, False, False),  # unsupported type
]
Z = [  # minZ, maxZ, h, wm, wd, domType, ref
    (0.0, 20.0, 1.0, [6], [0], "DPBW", False),
    (-16.0, 16.0, 1.0, [6], [6], "DP", False),
    (0.0, 32.0, 1.0, [6], [6], "DPSC", False),
    (0.0, 10.0, 0.5, [5], [5], "TP", False),
    (0.0, 10.3, 0.5, [5], [5], "TP", False),
    (0.0, 24.0, 0.8, [6], [0], "DPBW", True),
    (1.5, 18.5, 0.7342, [5], [4], "DP", False),
]


def _plain(v):
    if isinstance(v, np.ndarray):
        return [_plain(x) for x in v.tolist()]
    if isinstance(v, (list, tuple)):
        return [_plain(x) for x in v]
    if isinstance(v, (np.integer,)):
        return int(v)
    if isinstance(v, (np.floating,)):
        return float(v)
    return v


def main():
    if not hasattr(np, "int"):
        np.int = int  # the module predates numpy 2
    sys.path.insert(0, os.path.join(REF, "source", "cpu", "python"))
    import GridAndKernelConfig as G
    out = {"xy": [], "z": []}
    for Lx, Ly, radii, kts, opt, tq, ref in XY:
        case = {"args": [Lx, Ly, radii, kts, opt, tq, ref]}
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                r = G.configure_grid_and_kernels_xy(Lx, Ly, np.array(radii), np.array(kts), opt, tq, ref)
            case["out"] = _plain(list(r))
        except ValueError as e:
            case["error"] = str(e)
        out["xy"].append(case)
    for a in Z:
        minZ, maxZ, h, wm, wd, dom, ref = a
        case = {"args": list(a)}
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                r = G.configure_grid_and_kernels_z(minZ, maxZ, h, np.array(wm, dtype=np.ushort),
                                                   np.array(wd, dtype=np.ushort), dom, 1.5, ref)
            case["out"] = _plain(list(r))
        except Exception as e:  # the reference's own failures are recorded, by type
            case["error"] = "%s: %s" % (type(e).__name__, e)
        out["z"].append(case)
    with open(os.path.join(HERE, "gridconfig.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote %d xy and %d z cases" % (len(out["xy"]), len(out["z"])))


if __name__ == "__main__":
    main()
