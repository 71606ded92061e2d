"""CUDA path vs the reference's own outputs (golden fixtures) and vs the FP64
oracle, through the C ABI (engine API and the file-based drop-in entry
points).

Tolerances (FP64 path):
* chol: beta normwise per (trait, SNP) <= 1e-12, standard errors element-wise
  <= 1e-12, off-diagonal covariances normwise <= 1e-12, strict upper == 0.
* eigen: |dbeta_k| / (|beta_k| + SE_k) <= 1e-12, SE and off-diagonal
  covariances <= 1e-12 (measured at most 2e-13, 2e-14 and 5e-15 over these
  cases and at n = 10000).  Beta is not gated normwise: the eigenvector route
  amplifies rounding on near-zero coefficients (measured up to 1.8e-12
  normwise; the reference's own chol and eigen outputs differ by ~6e-13 there).
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import golden_cases, load_golden, report
from oracle import fgls_oracle as O

pytestmark = pytest.mark.gpu

CHOL_TOL = dict(beta_normwise=1e-12, se_rel=1e-12, v_offdiag_normwise=1e-12)
EIGEN_TOL = dict(beta_se_scaled=1e-12, se_rel=1e-12, v_offdiag_normwise=1e-12)


def check(d, tol, case=None):
    if case:
        report(case, **d)
    assert d["finite"], d
    assert d["upper_abs_max"] == 0.0, d
    for k, v in tol.items():
        assert d[k] <= v, (k, d)


def run_engine(pb, variant, x_b, precision="fp64"):
    from fgls_gb300 import Engine
    with Engine(pb.n, pb.wXL, pb.wXR, pb.t, x_b, variant=variant, precision=precision) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        if variant == "eigen":
            return e.run_snps(pb.XR)
        Bs, Vs = [], []
        for j in range(pb.t):
            e.select_trait(j)
            B, V = e.run_snps(pb.XR)
            Bs.append(B[0])
            Vs.append(V[0])
        return np.stack(Bs), np.stack(Vs)


@pytest.mark.parametrize("name", golden_cases())
def test_engine_vs_reference_golden(name):
    pb, var, xb, Bref, Vref = load_golden(name)
    variant = "chol" if var == "c" else "eigen"
    B, V = run_engine(pb, variant, xb)
    check(O.compare(B, V, Bref, Vref), CHOL_TOL if var == "c" else EIGEN_TOL, f"golden_engine_{name}")


@pytest.mark.parametrize("name", golden_cases())
def test_dropin_files_vs_reference_golden(name):
    """fgls_chol / fgls_eigen with the reference's 17 arguments, reading and
    writing the reference's file layout."""
    from fgls_gb300 import datagen, fgls_chol, fgls_eigen
    pb, var, xb, Bref, Vref = load_golden(name)
    d = tempfile.mkdtemp()
    paths = datagen.write_problem(pb, d)
    args = (pb.n, pb.p, pb.m, pb.t, pb.wXL, pb.wXR, xb, 1, 2, paths["Phi.in"], paths["H.in"], paths["Sig.in"],
            paths["XL.in"], paths["XR.in"], paths["Y.in"], os.path.join(d, "B.out"), os.path.join(d, "V.out"))
    (fgls_chol if var == "c" else fgls_eigen)(*args)
    raw_v = np.fromfile(os.path.join(d, "V.out"))
    assert raw_v.size == pb.t * pb.m * pb.p * pb.p
    B, V = datagen.read_outputs(d, pb.m, pb.t, pb.p)
    check(O.compare(B, V, Bref, Vref), CHOL_TOL if var == "c" else EIGEN_TOL)


@pytest.mark.parametrize("n,m,t,wXL,wXR,xb", [
    (300, 1000, 3, 3, 1, 256),   # ragged last block
    (257, 97, 2, 1, 1, 97),      # p = 2, single block, odd n
    (130, 33, 1, 6, 2, 7),       # p = 8 (maximum), tiny blocks
    (200, 1, 2, 3, 1, 64),       # m = 1 < x_b
    (129, 50, 2, 2, 3, 16),      # wXR = 3
])
@pytest.mark.parametrize("variant", ["chol", "eigen"])
def test_engine_vs_oracle_shapes(n, m, t, wXL, wXR, xb, variant):
    from fgls_gb300 import datagen
    pb = datagen.make_problem(n, m, t, wXL=wXL, wXR=wXR, seed=n + m, hsig_uniform=True)
    B, V = run_engine(pb, variant, xb)
    Br, Vr = O.fgls_chol(pb, xb) if variant == "chol" else O.fgls_eigen(pb)
    check(O.compare(B, V, Br, Vr), CHOL_TOL if variant == "chol" else EIGEN_TOL,
          f"shapes_{variant}_n{n}_m{m}_t{t}_wxl{wXL}_wxr{wXR}")


def test_chol_larger_n_vs_oracle():
    """n spans several 128-row potrf/TRSM blocks plus a ragged one."""
    from fgls_gb300 import datagen
    pb = datagen.make_problem(1000, 600, 2, seed=9, hsig_uniform=True)
    B, V = run_engine(pb, "chol", 256)
    Br, Vr = O.fgls_chol(pb, 256)
    check(O.compare(B, V, Br, Vr), CHOL_TOL)


def test_eigensolver_properties():
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(700, 4, 1, seed=4)
    with Engine(pb.n, 3, 1, 1, 4, variant="eigen") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        W, Z = e.eigen()
    Wr = np.linalg.eigvalsh(pb.Phi)
    nrm = np.abs(Wr).max()
    assert np.all(np.diff(W) >= 0)
    assert np.abs(W - Wr).max() < 1e-13 * nrm * 10
    assert np.abs(Z.T @ Z - np.eye(pb.n)).max() < 1e-12
    assert np.abs(pb.Phi @ Z - Z * W).max() < 1e-12 * nrm


def test_run_block_host_api_matches_run_snps():
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(150, 70, 3, seed=2, hsig_uniform=True)
    with Engine(pb.n, 3, 1, 3, 32, variant="eigen") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        B, V = e.run_snps(pb.XR)
        B2, V2 = e.run_block(pb.XR[:, 32:64])
    assert np.array_equal(B[:, 32:64], B2) and np.array_equal(V[:, 32:64], V2)


def test_not_spd_phi_is_reported():
    """A non-positive-definite M must fail like the reference's dpotrf(M)
    check (src/fgls_chol.c:266-271), through the status word, not a fault."""
    from fgls_gb300 import Engine, FGLSError, datagen
    pb = datagen.make_problem(64, 8, 1, seed=1)
    Phi = -np.eye(pb.n) * 5.0
    with Engine(pb.n, 3, 1, 1, 8, variant="chol") as e:
        e.set_problem(Phi, pb.XL, pb.Y, np.array([0.9]), np.array([1.0]))
        with pytest.raises(FGLSError, match="dpotrf\\(M\\) failed"):
            e.select_trait(0)


def test_truncated_xr_file_is_an_error():
    from fgls_gb300 import FGLSError, datagen, fgls_chol
    pb = datagen.make_problem(64, 20, 1, seed=1)
    d = tempfile.mkdtemp()
    paths = datagen.write_problem(pb, d)
    with open(paths["XR.in"], "r+b") as f:
        f.truncate(64 * 8 * 15)
    with pytest.raises(FGLSError, match="short read of XR"):
        fgls_chol(64, 4, 20, 1, 3, 1, 8, 1, 1, paths["Phi.in"], paths["H.in"], paths["Sig.in"],
                  paths["XL.in"], paths["XR.in"], paths["Y.in"], os.path.join(d, "B.out"), os.path.join(d, "V.out"))


def test_u8_genotypes_match_fp64():
    import torch
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(160, 48, 2, seed=8, hsig_uniform=True)
    with Engine(pb.n, 3, 1, 2, 48, variant="eigen") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        B, V = e.run_snps(pb.XR)
        xu8 = torch.from_numpy(np.asfortranarray(pb.XR).T.astype(np.uint8).copy()).cuda()
        dB = torch.empty(2 * 48 * 4, dtype=torch.float64, device="cuda")
        dV = torch.empty(2 * 48 * 16, dtype=torch.float64, device="cuda")
        e.run_block_device(xu8.data_ptr(), 48, dB.data_ptr(), dV.data_ptr(), 48 * 4, 48 * 16, u8=True)
        e.sync()
    B2 = dB.cpu().numpy().reshape(2, 48, 4)
    assert np.array_equal(B, B2)


def test_cli_driver_reference_interface():
    """fgls-driver <variant> <dir> <nrep> with 'n p m t wXL x_b y_b threads' on
    stdin (the reference's src/driver.c interface) writes dir/B.out, V.out."""
    import subprocess
    from fgls_gb300 import DRIVER_PATH, datagen
    name = "chol_n128_m200_t2"
    pb, var, xb, Bref, Vref = load_golden(name)
    d = tempfile.mkdtemp()
    datagen.write_problem(pb, d)
    stdin = f"{pb.n}\n{pb.p}\n{pb.m}\n{pb.t}\n{pb.wXL}\n{xb}\n1\n2\n"
    r = subprocess.run([DRIVER_PATH, "c", d, "2"], input=stdin, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().isdigit()  # mean ms per repetition
    B, V = datagen.read_outputs(d, pb.m, pb.t, pb.p)
    check(O.compare(B, V, Bref, Vref), CHOL_TOL)


def test_pvalues_match_normal_tail():
    import torch
    from scipy.stats import norm
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(200, 64, 2, wXL=2, wXR=2, seed=4, hsig_uniform=True)
    p, x = pb.p, pb.m
    with Engine(pb.n, 2, 2, 2, x, variant="eigen") as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        dX = torch.from_numpy(np.asfortranarray(pb.XR).T.copy()).cuda()
        dB = torch.empty(2 * x * p, dtype=torch.float64, device="cuda")
        dV = torch.empty(2 * x * p * p, dtype=torch.float64, device="cuda")
        dP = torch.empty(2 * x * 2, dtype=torch.float64, device="cuda")
        e.run_block_device(dX.data_ptr(), x, dB.data_ptr(), dV.data_ptr(), x * p, x * p * p)
        e.pvalues_device(dB.data_ptr(), dV.data_ptr(), x, x * p, x * p * p, dP.data_ptr(), x * 2)
        e.sync()
    B = dB.cpu().numpy().reshape(2, x, p)
    V = dV.cpu().numpy().reshape(2, x, p, p).transpose(0, 1, 3, 2)
    P = dP.cpu().numpy().reshape(2, x, 2)
    z = B[..., 2:] / np.stack([V[..., 2, 2], V[..., 3, 3]], axis=-1)
    assert np.allclose(P, 2 * norm.sf(np.abs(z)), rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_packed_2bit_genotypes_match_byte_input(precision):
    import torch
    from fgls_gb300 import Engine, FGLSError, datagen
    pb = datagen.make_problem(301, 150, 3, seed=12, hsig_uniform=True)
    p, x = pb.p, pb.m
    G = np.ascontiguousarray(pb.XR.T.astype(np.uint8))           # (m, n)
    packed = torch.from_numpy(datagen.pack_2bit(G)).cuda()
    u8 = torch.from_numpy(G).cuda()
    outs = []
    with Engine(pb.n, 3, 1, 3, x, variant="eigen", precision=precision) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        for src, kw in ((u8, {"u8": True}), (packed, {"packed": True})):
            dB = torch.empty(3 * x * p, dtype=torch.float64, device="cuda")
            dV = torch.empty(3 * x * p * p, dtype=torch.float64, device="cuda")
            e.run_block_device(src.data_ptr(), x, dB.data_ptr(), dV.data_ptr(), x * p, x * p * p, **kw)
            e.sync()
            outs.append((dB.cpu().numpy(), dV.cpu().numpy()))
        assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
        # a missing call is reported, not silently imputed
        Gm = G.copy().astype(np.int16)
        Gm[7, 5] = -1
        bad = torch.from_numpy(datagen.pack_2bit(Gm)).cuda()
        dB = torch.empty(3 * x * p, dtype=torch.float64, device="cuda")
        dV = torch.empty(3 * x * p * p, dtype=torch.float64, device="cuda")
        e.run_block_device(bad.data_ptr(), x, dB.data_ptr(), dV.data_ptr(), x * p, x * p * p, packed=True)
        with pytest.raises(FGLSError, match="missing genotype .* SNP 7, individual 5"):
            e.sync()


@pytest.mark.parametrize("variant,t", [("chol", 2), ("eigen", 3)])
def test_dropin_block_resume_after_interruption(variant, t):
    """FGLS_RESUME=1: a run stopped on the host after 2 blocks (FGLS_STOP_AFTER)
    and resumed computes only the missing blocks; B.out/V.out are identical to
    an uninterrupted run."""
    from fgls_gb300 import FGLSError, datagen, fgls_chol, fgls_eigen
    pb = datagen.make_problem(200, 700, t, seed=31, hsig_uniform=True)
    d = tempfile.mkdtemp()
    paths = datagen.write_problem(pb, d)
    fn = fgls_chol if variant == "chol" else fgls_eigen

    def run(bname, env):
        args = (pb.n, pb.p, pb.m, pb.t, pb.wXL, pb.wXR, 128, 1, 2, paths["Phi.in"], paths["H.in"], paths["Sig.in"],
                paths["XL.in"], paths["XR.in"], paths["Y.in"], os.path.join(d, bname + ".B"),
                os.path.join(d, bname + ".V"))
        fn(*args, env=env)

    run("full", {})
    with pytest.raises(FGLSError) as ei:
        run("part", {"FGLS_RESUME": "1", "FGLS_STOP_AFTER": "2"})
    assert ei.value.code == 3
    with open(os.path.join(d, "part.B.done")) as f:
        assert len(f.read().splitlines()) == 1 + 2
    run("part", {"FGLS_RESUME": "1"})
    for ext in ("B", "V"):
        a = np.fromfile(os.path.join(d, "full." + ext))
        b = np.fromfile(os.path.join(d, "part." + ext))
        assert a.size == b.size and np.array_equal(a, b)
    # a journal from other arguments is refused
    args = (pb.n, pb.p, pb.m, pb.t, pb.wXL, pb.wXR, 64, 1, 2, paths["Phi.in"], paths["H.in"], paths["Sig.in"],
            paths["XL.in"], paths["XR.in"], paths["Y.in"], os.path.join(d, "part.B"), os.path.join(d, "part.V"))
    with pytest.raises(FGLSError, match="different arguments"):
        fn(*args, env={"FGLS_RESUME": "1"})


@pytest.mark.parametrize("variant", ["chol", "eigen"])
def test_run_snps_compact_matches_full_output(variant):
    from scipy.special import erfc
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(180, 300, 2, seed=44, hsig_uniform=True)
    with Engine(pb.n, 3, 1, 2, 128, variant=variant) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        e.select_trait(1)
        B, V = e.run_snps(pb.XR)
        Bc, SE, P = e.run_snps_compact(pb.XR)
    idx = np.arange(pb.p)
    assert np.array_equal(B, Bc)
    assert np.array_equal(SE, V[..., idx, idx])
    assert np.allclose(P, erfc(np.abs(B / SE) / np.sqrt(2.0)), rtol=1e-13, atol=1e-300)


@pytest.mark.parametrize("variant,precision", [("eigen", "split"), ("eigen", "fp64"), ("chol", "split"),
                                               ("chol", "fp64")])
def test_run_snps_from_bytes_and_packed_matches_fp64(variant, precision):
    """fglsgpu_run_snps_u8 / _packed (host genotypes as bytes or 2-bit .bed
    body through the pinned pipeline, widened on the device) give results
    bit-identical to fglsgpu_run_snps on the same calls as FP64."""
    from fgls_gb300 import Engine, datagen
    pb = datagen.make_problem(301, 700, 40 if variant == "eigen" else 2, seed=23, hsig_uniform=True)
    G = np.ascontiguousarray(pb.XR.T.astype(np.uint8))
    with Engine(pb.n, 3, 1, pb.t, 256, variant=variant, precision=precision) as e:
        e.set_problem(pb.Phi, pb.XL, pb.Y, pb.h, pb.sigma)
        e.select_trait(1)
        B, V = e.run_snps(pb.XR)
        B1, V1 = e.run_snps_genotypes(G)
        B2, V2 = e.run_snps_genotypes(datagen.pack_2bit(G), packed=True)
    assert np.array_equal(B, B1) and np.array_equal(V, V1)
    assert np.array_equal(B, B2) and np.array_equal(V, V2)


@pytest.mark.parametrize("variant", ["chol", "eigen"])
def test_dropin_reads_bed_and_byte_genotype_files(variant):
    """FGLS_XR_FORMAT=bed (SNP-major PLINK .bed) and =u8 give the same
    B.out/V.out bytes as the reference's FP64 XR.in; a missing call is an
    error naming the SNP and the individual; a file without the .bed magic is
    refused."""
    from fgls_gb300 import FGLSError, datagen, fgls_chol, fgls_eigen
    pb = datagen.make_problem(203, 300, 3, seed=29, hsig_uniform=True)
    d = tempfile.mkdtemp()
    paths = datagen.write_problem(pb, d)
    fn = fgls_chol if variant == "chol" else fgls_eigen
    env = {"FGLS_PRECISION": "split"} if variant == "eigen" else {}

    def run(xr, tag, fmt):
        fn(pb.n, pb.p, pb.m, pb.t, pb.wXL, pb.wXR, 128, 1, 2, paths["Phi.in"], paths["H.in"], paths["Sig.in"],
           paths["XL.in"], xr, paths["Y.in"], os.path.join(d, tag + ".B"), os.path.join(d, tag + ".V"),
           env={**env, "FGLS_XR_FORMAT": fmt})
        return [np.fromfile(os.path.join(d, tag + ext)) for ext in (".B", ".V")]

    ref = run(paths["XR.in"], "f64", "f64")
    for fmt in ("u8", "bed"):
        out = run(datagen.write_xr(pb, os.path.join(d, "XR." + fmt), fmt), fmt, fmt)
        assert all(np.array_equal(a, b) for a, b in zip(ref, out)), fmt
    Gm = np.ascontiguousarray(pb.XR.T).astype(np.int16)
    Gm[211, 17] = -1
    with open(os.path.join(d, "miss.bed"), "wb") as f:
        f.write(datagen.BED_MAGIC + datagen.pack_2bit(Gm).tobytes())
    with pytest.raises(FGLSError, match="missing genotype .* SNP 211, individual 17"):
        run(os.path.join(d, "miss.bed"), "miss", "bed")
    with pytest.raises(FGLSError, match="not a SNP-major PLINK .bed"):
        run(os.path.join(d, "XR.u8"), "bad", "bed")
