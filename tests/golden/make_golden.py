"""Regenerates the golden fixtures in this directory.

Each fixture is a compressed .npz holding seeded synthetic inputs in the
reference's on-disk layout and the B/V that the REFERENCE ITSELF wrote for
them: its driver (src/driver.c) linked with its fgls_chol (variant 'c') or
fgls_eigen (variant 'e'), built from the unmodified reference sources by
oracle/build_ref.sh against OpenBLAS.  These pin the oracle and, through it,
the CUDA library.  Run here (where the reference sources are):

    bash oracle/build_ref.sh && python tests/golden/make_golden.py
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "cugwas-proto_gb300"))
sys.path.insert(0, ROOT)
from fgls_gb300 import datagen  # noqa: E402
from oracle import run_ref  # noqa: E402

# name, variant, n, m, t, wXL, wXR, x_b, y_b, threads, seed, h/sigma mode
CASES = [
    ("chol_n128_m200_t2", "c", 128, 200, 2, 3, 1, 64, 1, 2, 11, "uniform"),
    ("chol_n96_m50_t2_wxr2", "c", 96, 50, 2, 2, 2, 16, 1, 1, 12, "uniform"),
    ("chol_n200_m37_t1_xb37", "c", 200, 37, 1, 3, 1, 37, 1, 1, 13, "fixed"),
    ("eigen_n128_m200_t3", "e", 128, 200, 3, 3, 1, 64, 1, 1, 21, "uniform"),
    ("eigen_n100_m30_t3_wxr2", "e", 100, 30, 3, 2, 2, 8, 2, 2, 22, "uniform"),
]


def main():
    assert run_ref.available(), "build the reference first: bash oracle/build_ref.sh"
    here = os.path.dirname(os.path.abspath(__file__))
    for name, var, n, m, t, wXL, wXR, xb, yb, th, seed, mode in CASES:
        pb = datagen.make_problem(n, m, t, wXL=wXL, wXR=wXR, seed=seed,
                                  hsig_uniform=(mode == "uniform"), h=0.4, sigma=1.0)
        d = tempfile.mkdtemp()
        datagen.write_problem(pb, d)
        p = wXL + wXR
        run_ref.run(var, d, n, p, m, t, wXL, xb, y_b=yb, threads=th)
        B = np.fromfile(os.path.join(d, "B.out"), dtype="<f8")
        V = np.fromfile(os.path.join(d, "V.out"), dtype="<f8")
        np.savez_compressed(
            os.path.join(here, name + ".npz"),
            dims=np.array([n, m, t, wXL, wXR, xb, yb, th], dtype=np.int64),
            variant=np.array(var), Phi=pb.Phi, h=pb.h, sigma=pb.sigma, XL=pb.XL,
            XR=pb.XR.astype(np.uint8), Y=pb.Y, B_ref=B, V_ref=V)
        print("wrote", name, B.size, V.size)


if __name__ == "__main__":
    main()
