"""Parity at the measured problem size, n = 10,000 individuals, against the
FP64 oracle (src/fgls_eigen.c:428-565 and :998-1160; src/fgls_chol.c:251-438).

The kinship has a known eigendecomposition (datagen.known_spectrum_kinship:
half of the spectrum a degenerate cluster at 1e-3 as in a rank-5000 kinship,
dense delocalised eigenvectors), so the oracle runs with the exact (W, Z) and
shares nothing with the device: the device eigensolver, operand slicing,
split GEMM, quadratic Gram and batched solves are all checked at once.

Tolerances:
* split precision (9 five-bit FP8 digit slices): beta <= 1e-10 normwise per
  (trait, SNP) and on the (|beta| + SE) scale, SE <= 1e-10 relative;
* all-FP64 device path: chol as the reference gate (beta normwise and SE
  <= 1e-12); eigen on the (|beta| + SE) scale and SE <= 1e-12 (the
  eigenvector route amplifies rounding on near-zero coefficients, where a
  normwise gate is ill-posed);
* device eigenvalues within 1e-13 of max |W|, |Phi z - w z| <= 1e-12 |Phi|
  and |Z^T z - e| <= 1e-12 on sampled eigenvectors.
"""
import numpy as np
import pytest

from conftest import report
from oracle import fgls_oracle as O

pytestmark = pytest.mark.gpu

N, M, T, XB = 10000, 520, 100, 512


@pytest.fixture(scope="module")
def big():
    from fgls_gb300 import datagen
    return datagen.make_problem_known_spectrum(N, M, T, seed=2024)


def _pvals(B, V, wXL):
    from scipy.special import erfc
    p = B.shape[-1]
    se = np.stack([V[..., k, k] for k in range(wXL, p)], axis=-1)
    return erfc(np.abs(B[..., wXL:] / se) / np.sqrt(2.0))


def test_eigen_n10k_vs_oracle(big):
    from fgls_gb300 import Engine
    pb, W, Z = big
    with Engine(N, 3, 1, T, XB, variant="eigen", precision="split", slices=9) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        Wd, Zd = e.eigen()
        Bs, Vs = e.run_snps(pb.XR)
        e.set_precision("fp64")
        B64, V64 = e.run_snps(pb.XR)
    # the device eigensolver at n = 10k
    nrm = float(np.abs(W).max())
    ew = float(np.abs(Wd - W).max() / nrm)
    cols = np.random.default_rng(0).choice(N, 128, replace=False)
    cols[:2] = (0, N - 1)
    res = float(np.abs(pb.Phi @ Zd[:, cols] - Zd[:, cols] * Wd[cols]).max() / nrm)
    orth = float(np.abs(Zd.T @ Zd[:, cols] - np.eye(N)[:, cols]).max())
    Br, Vr = O.fgls_eigen(pb, W, Z)
    ds = O.compare(Bs, Vs, Br, Vr)
    d64 = O.compare(B64, V64, Br, Vr)
    pr = _pvals(Br, Vr, 3)
    pv_s = float(np.max(np.abs(_pvals(Bs, Vs, 3) - pr) / np.maximum(pr, 1e-300)))
    pv_64 = float(np.max(np.abs(_pvals(B64, V64, 3) - pr) / np.maximum(pr, 1e-300)))
    report("eigen_n10k", eig_rel=ew, residual=res, orthogonality=orth, split=ds, fp64=d64,
           pvalue_rel_split=pv_s, pvalue_rel_fp64=pv_64)
    assert ew <= 1e-13 and res <= 1e-12 and orth <= 1e-12, (ew, res, orth)
    assert ds["finite"] and ds["upper_abs_max"] == 0.0
    assert ds["beta_normwise"] <= 1e-10 and ds["beta_se_scaled"] <= 1e-10 and ds["se_rel"] <= 1e-10, ds
    assert d64["finite"] and d64["upper_abs_max"] == 0.0
    assert d64["beta_se_scaled"] <= 1e-12 and d64["se_rel"] <= 1e-12, d64


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_chol_n10k_vs_oracle(big, precision):
    """The plain drop-in workload's parameters: t = 1, h = 0.5, sigma = 2."""
    from fgls_gb300 import Engine
    pb0, _, _ = big
    from fgls_gb300.datagen import Problem
    pb = Problem(n=N, m=M, t=1, wXL=3, wXR=1, Phi=pb0.Phi, h=np.array([0.5]), sigma=np.array([2.0]), XL=pb0.XL,
                 XR=pb0.XR, Y=pb0.Y[:, :1].copy())
    with Engine(N, 3, 1, 1, XB, variant="chol", precision=precision, slices=9) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        e.select_trait(0)
        B, V = e.run_snps(pb.XR)
    Br, Vr = O.fgls_chol(pb, XB)
    d = O.compare(B, V, Br, Vr)
    report(f"chol_n10k_{precision}", **d)
    assert d["finite"] and d["upper_abs_max"] == 0.0
    if precision == "fp64":
        assert d["beta_normwise"] <= 1e-12 and d["se_rel"] <= 1e-12 and d["v_offdiag_normwise"] <= 1e-12, d
    else:
        assert d["beta_normwise"] <= 1e-10 and d["beta_se_scaled"] <= 1e-10 and d["se_rel"] <= 1e-10, d
