"""Split-precision (FP8 E4M3 digit-slice tcgen05) path.

* The raw split GEMM is bit-exact when A is representable in the chosen
  number of 5-bit digit slices (this pins the exactness of FP32 accumulation
  of integer slice products in TMEM, including sums near 2^19).
* For general FP64 A, 9 slices give |error| <= 2^-44 * sum_k |A_rk| |X_kc|.
* The split eigen path matches the FP64 oracle: beta relative error <= 1e-10
  (normwise per trait and SNP, and on the SE scale), SE <= 1e-10.
"""
import numpy as np
import pytest

from conftest import report
from oracle import fgls_oracle as O

pytestmark = pytest.mark.gpu


def _exact_product(Aint, shift, X):
    # A = Aint * 2^-shift exactly; product exact in int64 then scaled
    P = Aint.astype(np.int64) @ X.astype(np.int64)
    return np.ldexp(P.astype(np.float64), -shift)


# S five-bit digit slices represent bits-bit integers exactly when 4 + 5 (S - 1) >= bits
@pytest.mark.parametrize("M,K,N,S,bits", [(259, 1000, 300, 4, 15), (128, 64, 256, 2, 7), (300, 4097, 513, 5, 23)])
def test_split_gemm_exact_when_representable(M, K, N, S, bits):
    from fgls_gb300.engine import split_gemm_selftest
    rng = np.random.default_rng(M + K)
    Aint = rng.integers(-(2 ** bits) + 1, 2 ** bits, size=(M, K))
    Aint[:, 0] = 2 ** bits - 1  # every row uses its full exponent range
    X = rng.integers(0, 3, size=(K, N))
    A = np.ldexp(Aint.astype(np.float64), -bits)
    C = split_gemm_selftest(A, X, S)
    assert np.array_equal(C, _exact_product(Aint, bits, X))


def test_split_gemm_exact_at_accumulator_limit():
    """Slice products near 2^19 (K = 16000, digits of magnitude 16,
    genotypes 2) must still be exact."""
    from fgls_gb300.engine import split_gemm_selftest
    K, M, N = 16000, 128, 256
    rng = np.random.default_rng(1)
    Aint = np.where(rng.random((M, K)) < 0.5, -32767, 32767).astype(np.int64)
    Aint[:64] = 32767    # same-sign rows: |slice product| = 16 * 2 * 16000 ~ 2^19
    Aint[64:96] = -32767
    Aint[:, 0] = 32767
    X = np.full((K, N), 2)
    X[:, 1::2] = rng.integers(0, 3, size=(K, N // 2))
    C = split_gemm_selftest(np.ldexp(Aint.astype(np.float64), -15), X, 4)
    assert np.array_equal(C, _exact_product(Aint, 15, X))


def test_split_gemm_exact_fused_pair_limit():
    """A pass accumulates slices 2p and 2p+1 in one FP32 accumulator as
    P_2p + P_2p+1 / 32.  Digits (15, 15, 15, 15) at K = 16000 with genotypes
    mostly 2 put that sum near 2^19 with a fractional part in units of 2^-5:
    all 24 bits of the FP32 significand are used, and the result must still
    be exact.  Rows mix signs and digit patterns; half the columns take
    random genotypes so that the fractional parts vary."""
    from fgls_gb300.engine import split_gemm_selftest
    K, M, N = 16000, 256, 512
    rng = np.random.default_rng(3)
    top = 15 * 2 ** 15 + 15 * 2 ** 10 + 15 * 2 ** 5 + 15      # digits 15, 15, 15, 15 (20 bits)
    alt = 16 * 2 ** 15 - 1 * 2 ** 10 + 15 * 2 ** 5 - 13       # digits 16, -1, 15, -13
    Aint = np.where(rng.random((M, K)) < 0.5, -top, top).astype(np.int64)
    Aint[:64] = top
    Aint[64:96] = -top
    Aint[96:128] = alt
    Aint[128:160] = -alt
    Aint[:, 0] = np.where(Aint[:, 0] < 0, -alt, alt)  # every row's largest element starts with digit 16
    X = np.full((K, N), 2)
    X[:, 1::2] = rng.integers(0, 3, size=(K, N // 2))
    X[: K // 3, 3::4] = 1
    C = split_gemm_selftest(np.ldexp(Aint.astype(np.float64), -19), X, 4)
    assert np.array_equal(C, _exact_product(Aint, 19, X))


def test_split_gemm_fp64_accuracy():
    from fgls_gb300.engine import split_gemm_selftest
    rng = np.random.default_rng(7)
    M, K, N = 300, 2000, 700
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-5, 5, size=(M, 1)))
    X = rng.integers(0, 3, size=(K, N)).astype(np.float64)
    C = split_gemm_selftest(A, X, 9)
    ref = A @ X
    bound = np.abs(A) @ np.abs(X)
    assert np.all(np.abs(C - ref) <= 2.0 ** -44 * bound + 1e-300)


@pytest.mark.parametrize("n,m,t,xb", [(300, 700, 5, 256), (1000, 1100, 16, 512), (200, 300, 1, 256),
                                      (260, 400, 40, 256), (300, 257, 100, 512), (150, 300, 130, 256),
                                      (300, 200, 1000, 256), (500, 300, 113, 256)])
def test_split_eigen_vs_oracle(n, m, t, xb):
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(n, m, t, seed=n + t, hsig_uniform=True)
    with Engine(n, 3, 1, t, xb, variant="eigen", precision="split", slices=9) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        B, V = e.run_snps(pb.XR)
    Br, Vr = O.fgls_eigen(pb)
    d = O.compare(B, V, Br, Vr)
    report(f"split_eigen_n{n}_t{t}", **d)
    assert d["finite"] and d["upper_abs_max"] == 0.0
    assert d["beta_se_scaled"] <= 1e-10 and d["beta_normwise"] <= 1e-10, d
    assert d["se_rel"] <= 1e-10, d


@pytest.mark.parametrize("n,m,t,xb", [(300, 500, 2, 256), (700, 300, 1, 300)])
def test_split_chol_vs_oracle(n, m, t, xb):
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(n, m, t, seed=n + 3, hsig_uniform=True)
    Bs, Vs = [], []
    with Engine(n, 3, 1, t, xb, variant="chol", precision="split", slices=9) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        for j in range(t):
            e.select_trait(j)
            B, V = e.run_snps(pb.XR)
            Bs.append(B[0])
            Vs.append(V[0])
    Br, Vr = O.fgls_chol(pb, xb)
    d = O.compare(np.stack(Bs), np.stack(Vs), Br, Vr)
    report(f"split_chol_n{n}_t{t}", **d)
    assert d["finite"] and d["upper_abs_max"] == 0.0
    assert d["beta_se_scaled"] <= 1e-10 and d["beta_normwise"] <= 1e-10, d
    assert d["se_rel"] <= 1e-10, d


def test_precision_switch_keeps_eigendecomposition():
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(400, 300, 4, seed=5, hsig_uniform=True)
    with Engine(400, 3, 1, 4, 128, variant="eigen", precision="split") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        B1, V1 = e.run_snps(pb.XR)
        e.set_precision("fp64")
        B2, V2 = e.run_snps(pb.XR)
        e.set_precision("split")
        B3, V3 = e.run_snps(pb.XR)
    assert np.array_equal(B1, B3) and np.array_equal(V1, V3)  # deterministic
    d = O.compare(B1, V1, B2, V2)
    assert d["beta_se_scaled"] <= 1e-10 and d["se_rel"] <= 1e-10, d


@pytest.mark.parametrize("variant,t", [("eigen", 40), ("chol", 1)])
def test_split_run_snps_pipeline_matches_single_blocks(variant, t):
    """run_snps (uploads, compute and downloads of consecutive blocks on
    three streams) must equal, bit for bit, the same blocks run one at a
    time through the host API.  At x_b = 256 both cut the SNPs into the same
    blocks; the tensor-core quadratic Gram's fixed-order combine depends on
    how a block's tiles are dealt to CTAs, so other cuts agree to rounding
    only."""
    from fgls_gb300 import Engine, datagen
    xb, n = 256, 1500
    pb = datagen.make_problem(n, 6 * xb + 100, t, seed=11, hsig_uniform=True)
    with Engine(n, 3, 1, t, xb, variant=variant, precision="split", slices=9) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        if variant == "chol":
            e.select_trait(0)
        B, V = e.run_snps(pb.XR)
        for i0 in range(0, pb.XR.shape[1], xb):
            B2, V2 = e.run_block(pb.XR[:, i0:i0 + xb])
            assert np.array_equal(B[:, i0:i0 + xb], B2) and np.array_equal(V[:, i0:i0 + xb], V2), i0


def test_split_u8_matches_fp64_genotype_input():
    import torch
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(256, 200, 3, seed=6, hsig_uniform=True)
    with Engine(256, 3, 1, 3, 200, variant="eigen", precision="split") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        B, V = e.run_snps(pb.XR)
        xu8 = torch.from_numpy(np.asfortranarray(pb.XR).T.astype(np.uint8).copy()).cuda()
        dB = torch.empty(3 * 200 * 4, dtype=torch.float64, device="cuda")
        dV = torch.empty(3 * 200 * 16, dtype=torch.float64, device="cuda")
        e.run_block_device(xu8.data_ptr(), 200, dB.data_ptr(), dV.data_ptr(), 800, 3200, u8=True)
        e.sync()
    assert np.array_equal(B, dB.cpu().numpy().reshape(3, 200, 4))


@pytest.mark.parametrize("n,t", [(700, 40), (700, 100), (2000, 100), (900, 250)])
def test_tensor_core_quad_gram_vs_fp64_path(n, t, monkeypatch):
    """The quadratic Gram on the tensor cores (base-32 E4M3 digits of both
    operands, used for t >= 33, in groups of 112 traits) and the double-FP32 CUDA-core kernel, each
    against the all-FP64 device path on the same eigendecomposition: the
    tensor-core path is within 2e-12 on the SE scale (measured ~3e-13), the
    double-FP32 one within 1e-10 (measured ~1e-11)."""
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(n, 300, t, seed=t + 1, hsig_uniform=True)
    with Engine(pb.n, 3, 1, t, 256, variant="eigen", precision="fp64") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        B64, V64 = e.run_snps(pb.XR)
    for flag, tol in (("1", 2e-12), ("0", 1e-10)):
        monkeypatch.setenv("FGLS_QUAD_TC", flag)
        with Engine(pb.n, 3, 1, t, 256, variant="eigen", precision="split", slices=9) as e:
            e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
            B, V = e.run_snps(pb.XR)
        d = O.compare(B, V, B64, V64)
        assert d["finite"] and d["beta_se_scaled"] <= tol and d["se_rel"] <= tol, (flag, d)


def test_expired_wait_is_reported_and_the_engine_recovers():
    """Failure detection of the tcgen05 kernels on the device: with a wait
    limit of 1 ns every CTA of the split GEMM and of the tensor-core
    quadratic Gram (t = 40) gives up on its first pipeline wait that does not
    complete at once, lets its own copies and MMAs finish (those drain waits
    keep the 2 s limit), frees its TMEM and returns; the host reports
    FGLSGPU_ETIMEOUT.  With the default limit restored, the same engine gives
    results bit-identical to a run before the failure."""
    from fgls_gb300 import Engine, FGLSError, datagen
    from fgls_gb300.engine import ETIMEOUT
    pb = datagen.make_problem(300, 600, 40, seed=17, hsig_uniform=True)
    with Engine(pb.n, 3, 1, pb.t, 256, variant="eigen", precision="split", slices=9) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        B1, V1 = e.run_snps(pb.XR)
        e.set_wait_limit(1)
        with pytest.raises(FGLSError) as ei:
            e.run_snps(pb.XR)
        assert ei.value.code == ETIMEOUT and "wait expired" in str(ei.value), ei.value
        e.set_wait_limit(0)
        B2, V2 = e.run_snps(pb.XR)
        B3, V3 = e.run_block(pb.XR[:, :256])
    assert np.array_equal(B1, B2) and np.array_equal(V1, V2)
    assert np.array_equal(B1[:, :256], B3) and np.array_equal(V1[:, :256], V3)


@pytest.mark.parametrize("variant,t", [("eigen", 40), ("chol", 1)])
def test_slice_autotune(variant, t):
    """slices = 0: the operand is cut into 9 slices and a 256-SNP probe block
    keeps the smallest count in 6..9 whose beta is within 1e-10 / 8 of the
    FP64 path; the results at that count stay within 1e-10 of the oracle.
    Given slices are used as they are (no probe)."""
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(400, 300, t, seed=41, hsig_uniform=True)
    with Engine(pb.n, 3, 1, t, 256, variant=variant, precision="split", slices=0) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        e.select_trait(0)
        S, err = e.split_params()
        B, V = e.run_snps(pb.XR)
    report(f"slice_autotune_{variant}", slices=S, probe_err=err)
    assert 6 <= S <= 9 and 0.0 <= err and (err <= 1e-10 / 8 or S == 9), (S, err)
    if variant == "eigen":
        Br, Vr = O.fgls_eigen(pb)
    else:
        pb1 = datagen.Problem(n=pb.n, m=pb.m, t=1, wXL=3, wXR=1, Phi=pb.Phi, h=pb.h[:1], sigma=pb.sigma[:1],
                              XL=pb.XL, XR=pb.XR, Y=pb.Y[:, :1])
        Br, Vr = O.fgls_chol(pb1, 256)
    d = O.compare(B, V, Br, Vr)
    assert d["beta_normwise"] <= 1e-10 and d["beta_se_scaled"] <= 1e-10 and d["se_rel"] <= 1e-10, (S, d)
    with Engine(pb.n, 3, 1, t, 256, variant=variant, precision="split", slices=9) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        e.select_trait(0)
        assert e.split_params() == (9, -1.0)
