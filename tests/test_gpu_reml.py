"""Variance-component estimation on the device (fglsgpu_reml_fit) and the
refit path (fglsgpu_set_hsigma), through the C ABI.

The fit is checked against the CPU oracle fit (oracle.reml_fit: the same
profiled REML, maximised with Brent's method on numpy eigenvectors of Phi).
Tolerances: h within 1e-8 absolute, sigma within 1e-8 relative, the profiled
log-likelihood within 1e-10 relative (the optimum is flat, so the value agrees
to second order in the h difference; the device eigenbasis differs from
numpy's by rounding only).
"""
import numpy as np
import pytest

from oracle import fgls_oracle as O

pytestmark = pytest.mark.gpu

H_TRUE = np.array([0.0, 0.25, 0.5, 0.8, 0.95])
SIG_TRUE = np.array([1.0, 2.0, 0.5, 1.5, 1.0])


def problem(n, wXL, seed=11, m=64):
    from fgls_gb300 import datagen
    return datagen.make_problem(n, m, len(H_TRUE), wXL=wXL, seed=seed, h=H_TRUE, sigma=SIG_TRUE)


def oracle_fit(pb, lo, hi, grid):
    W, Z = np.linalg.eigh(pb.Phi)
    return O.reml_fit(W, Z.T @ pb.XL, Z.T @ pb.Y, lo, hi, grid)


@pytest.mark.parametrize("n,wXL", [(400, 3), (257, 1), (300, 5)])
def test_reml_fit_matches_oracle(n, wXL):
    from fgls_gb300 import Engine
    pb = problem(n, wXL)
    lo, hi, grid = 0.0, 1.0 - 1e-5, 64
    with Engine(pb.n, pb.wXL, 1, pb.t, 64, variant="eigen") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        h, s, ll, dll = e.reml_fit(lo, hi, grid)
    ho, so, llo, dllo = oracle_fit(pb, lo, hi, grid)
    np.testing.assert_allclose(h, ho, rtol=0, atol=1e-8)
    np.testing.assert_allclose(s, so, rtol=1e-8)
    np.testing.assert_allclose(ll, llo, rtol=1e-10)
    assert np.all((h >= lo) & (h <= hi))
    interior = (h > lo) & (h < hi)
    # a stationary point inside, an outward-pointing gradient on an endpoint
    assert np.all(np.abs(dll[interior]) <= 1e-6 * np.abs(ll[interior]))
    assert np.all(dll[h == lo] <= 0) and np.all(dll[h == hi] >= 0)


def test_reml_fit_value_is_the_adjoint_reml_at_the_estimate():
    """At (h_hat, sigma_hat) the adjoint's null-model REML equals the profiled
    value and its h-gradient is the profiled gradient."""
    from fgls_gb300 import Engine
    pb = problem(400, 3, seed=5)
    with Engine(pb.n, pb.wXL, 1, pb.t, 64, variant="eigen") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        h, s, ll, dll = e.reml_fit()
        e.set_hsigma(h, s)
        e.adjoint_reset()
        ll2, dll2 = e.reml()
    np.testing.assert_allclose(ll2, ll, rtol=1e-11)
    np.testing.assert_allclose(dll2, dll, rtol=0, atol=1e-7 * np.max(np.abs(ll)))


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_set_hsigma_equals_set_problem(precision):
    """Refitting h and sigma on a live engine gives bit-identical B and V to a
    fresh set_problem with those values (the eigendecomposition is reused)."""
    from fgls_gb300 import Engine
    pb = problem(300, 3, seed=9, m=200)
    h2 = np.clip(pb.h + 0.07, 0.0, 1.0)
    s2 = pb.sigma * 1.3
    with Engine(pb.n, pb.wXL, 1, pb.t, 128, variant="eigen", precision=precision) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        e.run_snps(pb.XR)
        e.set_hsigma(h2, s2)
        B1, V1 = e.run_snps(pb.XR)
        rs1 = e.res_sigma()
    with Engine(pb.n, pb.wXL, 1, pb.t, 128, variant="eigen", precision=precision) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, h2, s2)
        B2, V2 = e.run_snps(pb.XR)
        rs2 = e.res_sigma()
    assert np.array_equal(B1, B2) and np.array_equal(V1, V2) and np.array_equal(rs1, rs2)


def test_set_hsigma_chol_reselects():
    from fgls_gb300 import Engine
    pb = problem(200, 3, seed=4, m=50)
    h2, s2 = np.full(pb.t, 0.3), np.full(pb.t, 0.7)
    with Engine(pb.n, pb.wXL, 1, pb.t, 50, variant="chol") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        e.set_hsigma(h2, s2)
        e.select_trait(2)
        B1, V1 = e.run_block(pb.XR)
    with Engine(pb.n, pb.wXL, 1, pb.t, 50, variant="chol") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, h2, s2)
        e.select_trait(2)
        B2, V2 = e.run_block(pb.XR)
    assert np.array_equal(B1, B2) and np.array_equal(V1, V2)


def test_reml_fit_argument_errors():
    from fgls_gb300 import Engine
    from fgls_gb300.engine import FGLSError
    pb = problem(200, 3, seed=2, m=16)
    with Engine(pb.n, pb.wXL, 1, pb.t, 16, variant="eigen") as e:
        with pytest.raises(FGLSError):
            e.reml_fit()                      # before set_problem
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        for lo, hi, grid in ((0.5, 0.5, 64), (-0.1, 0.5, 64), (0.0, 1.5, 64), (0.0, 0.9, 1), (0.0, 0.9, 1000)):
            with pytest.raises(FGLSError) as ei:
                e.reml_fit(lo, hi, grid)
            assert ei.value.code == 1
        with pytest.raises(FGLSError):
            e.set_hsigma(np.full(pb.t, 1.2), pb.sigma)
        h, s, _, _ = e.reml_fit(0.2, 0.6, 8)  # a sub-interval with a coarse grid still works
        assert np.all((h >= 0.2) & (h <= 0.6)) and np.all(s > 0)
    with Engine(pb.n, pb.wXL, 1, pb.t, 16, variant="chol") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        with pytest.raises(FGLSError):
            e.reml_fit()
