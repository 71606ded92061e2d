"""The oracle (numpy FP64 restatement) against the reference's own outputs:
tests/golden/*.npz hold B/V written by the reference driver built from its
sources (see tests/golden/make_golden.py)."""
import os
import tempfile

import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import fgls_oracle as O


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_golden(name):
    pb, var, xb, Bref, Vref = load_golden(name)
    B, V = O.fgls_chol(pb, xb) if var == "c" else O.fgls_eigen(pb)
    d = O.compare(B, V, Bref, Vref)
    assert d["finite"]
    assert d["upper_abs_max"] == 0.0
    assert float(np.abs(np.triu(Vref, 1)).max()) == 0.0  # the reference leaves the strict upper triangle 0
    if var == "c":
        assert d["beta_normwise"] < 1e-12, d
        assert d["se_rel"] < 1e-12, d
        assert d["v_offdiag_normwise"] < 1e-12, d
    else:
        # eigen: eigenvector-route rounding; the reference's own chol and
        # eigen variants differ by ~2e-12 normwise on small coefficients
        assert d["beta_se_scaled"] < 1e-11, d
        assert d["beta_normwise"] < 2e-10, d
        assert d["se_rel"] < 1e-12, d


def test_goldens_present():
    assert len(golden_cases()) >= 5


def test_oracle_detects_a_planted_error():
    """A mistake planted in the oracle's output must be caught by compare()."""
    pb, var, xb, Bref, Vref = load_golden("chol_n128_m200_t2")
    B, V = O.fgls_chol(pb, xb)
    B = B.copy()
    B[1, 17, 3] *= 1 + 1e-9
    assert O.compare(B, V, Bref, Vref)["beta_normwise"] > 1e-10


def test_chol_and_eigen_oracles_agree():
    pb, var, xb, Bref, Vref = load_golden("chol_n128_m200_t2")
    B1, V1 = O.fgls_chol(pb, 64)
    B2, V2 = O.fgls_eigen(pb)
    d = O.compare(B2, V2, B1, V1)
    assert d["beta_se_scaled"] < 1e-11 and d["se_rel"] < 1e-11, d


def test_known_spectrum_kinship_is_exact():
    """The generator's (W, Z) is an eigendecomposition of its Phi to rounding,
    its spectrum has the degenerate 1e-3 cluster of a rank-n/2 kinship, and
    the oracle gives the same results from it as from scipy's dsyevr."""
    from fgls_gb300 import datagen
    pb, W, Z = datagen.make_problem_known_spectrum(240, 40, 3, seed=8)
    nrm = np.abs(W).max()
    assert np.all(np.diff(W) >= 0) and np.sum(W == 1e-3) == 120
    assert np.abs(pb.Phi @ Z - Z * W).max() <= 1e-14 * nrm
    assert np.abs(Z.T @ Z - np.eye(pb.n)).max() <= 1e-14
    assert np.abs(pb.Phi - pb.Phi.T).max() == 0.0
    assert np.abs(Z).max() < 0.5  # delocalised eigenvectors
    B1, V1 = O.fgls_eigen(pb, W, Z)
    B2, V2 = O.fgls_eigen(pb)
    d = O.compare(B1, V1, B2, V2)
    assert d["beta_se_scaled"] < 1e-12 and d["se_rel"] < 1e-12, d


def _reference_fixture():
    from oracle import run_ref
    return os.path.join(run_ref.reference_root(), "test_cases", "test_XL")


@pytest.mark.skipif(not os.path.isdir(_reference_fixture()), reason="reference fixture absent")
def test_oracle_on_reference_fixture_inputs():
    """The reference's own fixture inputs (test_cases/test_XL: n=500, t=20,
    wXL=3; its XR.in is missing) with a synthetic XR, run through the
    reference driver and the oracle."""
    from oracle import run_ref
    from fgls_gb300 import datagen
    if not run_ref.available():
        pytest.skip("reference driver not built")
    src = _reference_fixture()
    n, t, wXL, m = 500, 4, 3, 64
    d = tempfile.mkdtemp()
    for f in ("Phi.in", "H.in", "Sig.in", "XL.in", "Y.in"):
        os.symlink(os.path.join(src, f), os.path.join(d, f))
    rng = np.random.default_rng(3)
    XR = datagen.hardcall_genotypes(rng, n, m)
    np.asfortranarray(XR).T.astype("<f8").tofile(os.path.join(d, "XR.in"))
    run_ref.run("c", d, n, 4, m, t, wXL, 32, threads=1)
    Bref, Vref = datagen.read_outputs(d, m, t, 4)
    pb = datagen.read_problem(d, n, m, t, wXL)
    B, V = O.fgls_chol(pb, 32)
    r = O.compare(B, V, Bref, Vref)
    assert r["beta_normwise"] < 1e-12 and r["se_rel"] < 1e-12, r


def _reml_problem(n=240, seed=21):
    from fgls_gb300 import datagen
    pb = datagen.make_problem(n, 4, 4, seed=seed, h=[0.0, 0.3, 0.7, 0.95], sigma=[1.0, 2.0, 0.5, 1.5])
    W, Z = np.linalg.eigh(pb.Phi)
    return pb, W, Z


def test_profiled_reml_is_the_null_model_reml_at_sigma_hat():
    """The profiled value/gradient equal oracle.reml at (h, sigma_hat(h)) and
    the gradient matches central differences of the profiled value."""
    pb, W, Z = _reml_problem()
    ZtXL, ZtY = Z.T @ pb.XL, Z.T @ pb.Y
    for j in range(pb.t):
        for h in (0.05, 0.4, 0.9):
            ll, dll, sig = O.reml_profiled(W, ZtXL, ZtY[:, j], h)
            a, da = O.reml(Z, W, pb.XL, pb.Y[:, [j]], [h], [sig])
            assert abs(a[0] - ll) <= 1e-12 * abs(ll)
            assert abs(da[0] - dll) <= 1e-10 * abs(ll)
            e = 1e-6
            fd = (O.reml_profiled(W, ZtXL, ZtY[:, j], h + e)[0] - O.reml_profiled(W, ZtXL, ZtY[:, j], h - e)[0]) / (2 * e)
            assert abs(fd - dll) <= 1e-6 * abs(ll)


def test_oracle_reml_fit_is_a_maximum():
    pb, W, Z = _reml_problem()
    ZtXL, ZtY = Z.T @ pb.XL, Z.T @ pb.Y
    lo, hi = 0.0, 1.0 - 1e-5
    h, s, ll, dll = O.reml_fit(W, ZtXL, ZtY, lo, hi, 32)
    dense = np.linspace(lo, hi, 2001)
    for j in range(pb.t):
        prof = [O.reml_profiled(W, ZtXL, ZtY[:, j], x)[0] for x in dense]
        assert ll[j] >= max(prof) - 1e-9 * abs(ll[j])
        if lo < h[j] < hi:
            assert abs(dll[j]) <= 1e-8 * abs(ll[j])
        assert abs(O.reml_profiled(W, ZtXL, ZtY[:, j], h[j])[2] - s[j]) <= 1e-14 * s[j]


def test_bed_writer_follows_the_plink_bit_layout():
    """datagen.write_xr(..., 'bed'): magic 6c 1b 01, then per SNP ceil(n/4)
    bytes, individual k in bits 2(k%4).. of byte k/4, codes 00 = 2, 10 = 1,
    11 = 0 copies of the first allele (01 = missing), padding codes 11."""
    from fgls_gb300 import datagen
    pb = datagen.make_problem(10, 4, 1, seed=3)
    d = tempfile.mkdtemp()
    raw = open(datagen.write_xr(pb, os.path.join(d, "x.bed"), "bed"), "rb").read()
    assert raw[:3] == bytes((0x6C, 0x1B, 0x01)) and len(raw) == 3 + 4 * 3
    body = np.frombuffer(raw[3:], np.uint8).reshape(4, 3)
    for i in range(4):
        for k in range(12):
            code = (body[i, k // 4] >> (2 * (k % 4))) & 3
            want = 3 if k >= 10 else {2: 0, 1: 2, 0: 3}[int(pb.XR[k, i])]
            assert code == want, (i, k, code, want)


def test_device_packer_matches_the_host_packer():
    """bench.pack_2bit_device (torch) writes the same .bed body bytes as
    datagen.pack_2bit."""
    import torch
    import bench
    from fgls_gb300 import datagen
    rng = np.random.default_rng(2)
    for n in (12, 13, 15):
        G = rng.integers(0, 3, size=(7, n)).astype(np.uint8)
        got = bench.pack_2bit_device(torch.from_numpy(G)).numpy()
        assert np.array_equal(got, datagen.pack_2bit(G)), n


def test_bench_traffic_comes_from_the_committed_profiles():
    """bench.gemm_traffic finds the DRAM bytes per launch of the default eigen
    workload's split GEMM and of the 64-cohort grouped GEMM in the committed
    ncu summaries, and they are the read + write sums those summaries list."""
    import bench
    eig = bench.gemm_traffic("ozaki_gemm_n10000_t100_xb16384")
    coh = bench.gemm_traffic("grouped_gemm_cohorts64_xb2048")
    assert eig is not None and abs(eig - (16.72 + 5.105) * 1e9) < 0.05e9
    assert coh is not None and abs(coh - (35.345 + 19.33) * 1e9) < 0.05e9
    assert bench.gemm_traffic("no_such_profile") is None
