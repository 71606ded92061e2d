import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "cugwas-proto_gb300"))
sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    """Returns (Problem, variant, x_b, B_ref (t,m,p), V_ref (t,m,p,p) [row, col])."""
    from fgls_gb300.datagen import Problem
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    n, m, t, wXL, wXR, xb, yb, th = (int(v) for v in z["dims"])
    p = wXL + wXR
    pb = Problem(n=n, m=m, t=t, wXL=wXL, wXR=wXR, Phi=z["Phi"], h=z["h"], sigma=z["sigma"], XL=z["XL"],
                 XR=z["XR"].astype(np.float64), Y=z["Y"])
    B = z["B_ref"].reshape(t, m, p)
    V = z["V_ref"].reshape(t, m, p, p).transpose(0, 1, 3, 2)
    return pb, str(z["variant"]), xb, B, V


def report(case, **values):
    """Appends one JSON line {case, values} to the file named by
    FGLS_TEST_REPORT (when set), so that a run can keep the measured errors
    behind each tolerance; does nothing otherwise."""
    path = os.environ.get("FGLS_TEST_REPORT")
    if not path:
        return
    import json
    with open(path, "a") as f:
        f.write(json.dumps({"case": case, **values}, default=float) + "\n")


@pytest.fixture(scope="session")
def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
