#!/usr/bin/env python3
"""Headline benchmark: SNP x trait tests/s of the FGLS eigen association on
one GB300 with the split-precision tensor-core path, beside the all-FP64
device path and the CPU restatement of the reference.

Workload (synthetic, seeded): n = 10,000 individuals, p = 4 (intercept + 2
N(0,1) covariates + 1 SNP), t = 100 traits with h ~ U(0.1, 0.9),
sigma ~ U(0.5, 2), kinship Phi = G G^T / 5000 + 1e-3 I, hard-call genotypes
Binomial(2, f), f ~ U(0.05, 0.5).  The job is m = 1,000,000 SNPs; a step is
one block of x_b SNPs x t traits through the hot path (genotype operand
build, split GEMM, quadratic Gram, batched p x p solves, B/V emission).
The one-off setup (device eigendecomposition of Phi, Z^T XL, Z^T Y, null
models, slicing of [Z^T ; U^T]) is outside the timed region and reported as
setup_s.  Every step reads a different resident genotype block of 1.3 GB
(FP64, the reference's XR layout): inputs larger than L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cugwas-proto_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "SNP×trait tests/s on 1 GB300, split-prec vs FP64 path, β rel-err ≤1e-10"
UNIT = "tests/s"
N_IND, T_TRAITS, WXL, WXR, M_JOB = 10000, 100, 3, 1, 1_000_000
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        if all(k in d for k in FALLBACK_PEAKS):
            return d, "measured"
        return {**FALLBACK_PEAKS, **d}, "measured where present, else fallback"
    return dict(FALLBACK_PEAKS), "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the
    timed region (our own child process, stopped by PID)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu_id, f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
                pw.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None, "samples": len(sm), "reasons": sorted(reasons)}


def make_problem_gpu(n, t, seed, dev, h=None, sigma=None):
    """Phi, XL, Y, h, sigma (host numpy) drawn on the device (torch is the
    data generator only); h, sigma fixed when given, else h ~ U(0.1, 0.9),
    sigma ~ U(0.5, 2)."""
    import torch
    g = torch.Generator(device=dev).manual_seed(seed)
    k = 5000
    f = torch.rand(k, generator=g, device=dev, dtype=torch.float64) * 0.45 + 0.05
    G = ((torch.rand(n, k, generator=g, device=dev, dtype=torch.float64) < f).double()
         + (torch.rand(n, k, generator=g, device=dev, dtype=torch.float64) < f).double())
    G = (G - G.mean(0)) / G.std(0, unbiased=False).clamp_min(1e-12)
    Phi = G @ G.T / k
    Phi.diagonal().add_(1e-3)
    hr = torch.rand(t, generator=g, device=dev, dtype=torch.float64) * 0.8 + 0.1
    sr = torch.rand(t, generator=g, device=dev, dtype=torch.float64) * 1.5 + 0.5
    h = hr if h is None else torch.full((t,), float(h), device=dev, dtype=torch.float64)
    s = sr if sigma is None else torch.full((t,), float(sigma), device=dev, dtype=torch.float64)
    XL = torch.ones(n, WXL, device=dev, dtype=torch.float64)
    XL[:, 1:] = torch.randn(n, WXL - 1, generator=g, device=dev, dtype=torch.float64)
    u = torch.randn(k, t, generator=g, device=dev, dtype=torch.float64)
    v = torch.randn(n, t, generator=g, device=dev, dtype=torch.float64)
    Y = (G @ u) / k ** 0.5 * torch.sqrt(h * s) + v * torch.sqrt(h * s * 1e-3 + (1 - h) * s)
    out = [x.cpu().numpy() for x in (Phi, XL, Y, h, s)]
    del G, Phi
    torch.cuda.empty_cache()
    return out


def genotype_block(x, n, seed, dev):
    """x SNPs of hard calls 0/1/2 as a (x, n) FP64 tensor = column-major n x x."""
    import torch
    g = torch.Generator(device=dev).manual_seed(seed)
    f = torch.rand(x, 1, generator=g, device=dev) * 0.45 + 0.05
    X = (torch.rand(x, n, generator=g, device=dev) < f).to(torch.uint8)
    X += (torch.rand(x, n, generator=g, device=dev) < f).to(torch.uint8)
    return X.double()


def pack_2bit_device(X):
    """(cols, n) hard calls on the device -> (cols, ceil(n/4)) bytes, the
    SNP-major PLINK .bed body (codes 2 -> 00, 1 -> 10, 0 -> 11, padding 11),
    as datagen.pack_2bit does on the host."""
    import torch
    cols, n = X.shape
    code = torch.where(X == 2, 0, torch.where(X == 1, 2, 3)).to(torch.uint8)
    pad = (-n) % 4
    if pad:
        code = torch.cat([code, torch.full((cols, pad), 3, dtype=torch.uint8, device=X.device)], 1)
    code = code.view(cols, -1, 4)
    return code[..., 0] | (code[..., 1] << 2) | (code[..., 2] << 4) | (code[..., 3] << 6)


def rank_block_seeds(rank, pool):
    """Genotype-block seeds of one rank: ranks shard the SNP blocks (weak
    scaling), so no two ranks process the same block."""
    return [100 + rank * 1000 + i for i in range(pool)]


def max_over_ranks(value, dist, device):
    """The job is as slow as its slowest rank: max of a per-rank time."""
    if dist is None:
        return value
    import torch
    tt = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def aggregate_throughput(world, blocks_per_rank, snps_per_block, traits, seconds):
    """Whole-job tests/s: all ranks' SNP x trait tests over the slowest rank's time."""
    return world * blocks_per_rank * snps_per_block * traits / seconds


# GB300's nominal dense FP8 tensor rate, for context beside the measured-peak
# fraction (the measured denominator is twice a cuBLAS BF16 GEMM's rate).
NOMINAL_FP8_TFLOPS = 4500.0
# whole end-to-end calls per measurement (the median is reported)
E2E_CALLS = 5


def gemm_traffic(name):
    """DRAM bytes (read + write) of one split-GEMM launch of a workload, from the
    committed ncu summary profiles/<name>.txt (its line
    'dram_bytes_per_launch: <bytes>'); None when no capture exists."""
    f = os.path.join(ROOT, "profiles", f"{name}.txt")
    if not os.path.exists(f):
        return None
    for line in open(f):
        if line.startswith("dram_bytes_per_launch:"):
            return float(line.split(":", 1)[1])
    return None


def rel_errors(B, V, Br, Vr):
    """beta error normwise per (trait, SNP) and on the SE scale; SE element-wise."""
    p = B.shape[-1]
    idx = np.arange(p)
    se_r = Vr[..., idx, idx]
    nb = np.linalg.norm(B - Br, axis=-1) / np.linalg.norm(Br, axis=-1)
    bs = np.abs(B - Br) / (np.abs(Br) + se_r)
    se = np.abs(V[..., idx, idx] - se_r) / se_r
    return float(nb.max()), float(bs.max()), float(se.max())


GATE = 1e-10  # beta (normwise and on the SE scale) and SE against the FP64 oracle


def eigen_residuals(Phi, W, Z, cols=128, seed=0):
    """|Phi z - w z| / max|W| and |Z^T z - e| over sampled eigenvectors z of
    the device eigendecomposition (always including the extreme ones)."""
    n = Z.shape[0]
    S = np.random.default_rng(seed).choice(n, min(cols, n), replace=False)
    S[:2] = (0, n - 1)
    nrm = float(np.abs(W).max())
    res = float(np.abs(Phi @ Z[:, S] - Z[:, S] * W[S]).max() / nrm)
    orth = float(np.abs(Z.T @ Z[:, S] - np.eye(n)[:, S]).max())
    return {"residual": res, "orthogonality": orth, "columns": int(len(S))}


def pvalues_np(B, V, wXL):
    from scipy.special import erfc
    p = B.shape[-1]
    se = np.stack([V[..., k, k] for k in range(wXL, p)], axis=-1)
    return erfc(np.abs(B[..., wXL:] / se) / np.sqrt(2.0))


def oracle_errors(B, V, Br, Vr, wXL):
    """beta normwise and on the SE scale, SE, p-value of the SNP coefficient,
    each the maximum over the (trait, SNP) sample."""
    nb, bs, se = rel_errors(B, V, Br, Vr)
    pr = pvalues_np(Br, Vr, wXL)
    pv = float(np.max(np.abs(pvalues_np(B, V, wXL) - pr) / np.maximum(pr, 1e-300)))
    return {"beta_normwise": nb, "beta_se_scaled": bs, "se_rel": se, "pvalue_rel": pv}


def cpu_port_throughput(Z, W, XL, Y, h, s, X_host, budget_s, min_reps=1, steps=None):
    """The oracle's restatement of the reference's per-block eigen loop on the
    host cores: tests/s over a bounded SNP sample.  Only this leg imports
    oracle/ (the checker), and only to time it."""
    from oracle import fgls_oracle as O
    st = O.eigen_setup(Z, W, XL, Y, h, s, WXL)
    x = X_host.shape[1]
    times = []
    if steps is None:
        t0 = time.perf_counter()
        while True:
            a = time.perf_counter()
            O.eigen_block(st, X_host, WXR)
            times.append(time.perf_counter() - a)
            if len(times) >= min_reps and time.perf_counter() - t0 > budget_s:
                break
    else:
        w, k = steps
        for _ in range(w):
            O.eigen_block(st, X_host, WXR)
        for _ in range(k):
            a = time.perf_counter()
            O.eigen_block(st, X_host, WXR)
            times.append(time.perf_counter() - a)
    tot = sum(times)
    return len(times) * x * Y.shape[1] / tot, tot / len(times), len(times)


def cpu_chol_throughput(Phi, XL, y, h, sigma, X_host, budget_s, wXR=1):
    """The oracle's restatement of fgls_chol's per-block loop
    (src/fgls_chol.c:365-438: TRSM, per-SNP Gram and solve) on the host cores
    for one trait, repeated over the SNP sample for about budget_s seconds;
    the per-trait factorization and null model (src/fgls_chol.c:251-325) are
    set up once, outside the timing.  Returns (tests/s, seconds, reps)."""
    import scipy.linalg as sla
    from oracle import fgls_oracle as O
    n = Phi.shape[0]
    M = h * sigma * Phi
    M[np.diag_indices(n)] += (1.0 - h) * sigma
    L = np.linalg.cholesky(M)
    wXL = XL.shape[1]
    XLt, yt, B_t, V_tl, rs = O.null_model_chol(L, XL, y, wXL)
    times = []
    t0 = time.perf_counter()
    while not times or time.perf_counter() - t0 < budget_s:
        a = time.perf_counter()
        Xt = sla.solve_triangular(L, X_host, lower=True)
        O.snp_solve(B_t, V_tl, XLt, yt, Xt, wXL, wXR, rs)
        times.append(time.perf_counter() - a)
    tot = sum(times)
    return len(times) * X_host.shape[1] // wXR / tot, tot, len(times)


def orthogonal_basis(n, seed):
    """Dense orthogonal n x n matrix (three Householder reflectors), used by
    the reference arm where no device eigensolver may run."""
    rng = np.random.default_rng(seed)
    Z = np.eye(n)
    for _ in range(3):
        v = rng.standard_normal(n)
        v /= np.linalg.norm(v)
        Z -= 2.0 * np.outer(v, v @ Z)
    return Z


def run_chol(args):
    """The plain chol drop-in workload: n = 10000, p = 4, t = 1, h = 0.5,
    sigma = 2, blocks of 4096 SNPs.  Device throughput of the all-FP64 path
    (blocked TRSM, skinny Gram, solve) and of the split path, and end to end
    through the fgls_chol file entry point (XR streamed from a local file
    through the pinned ring) for a 16384-SNP file."""
    import tempfile

    import torch
    from fgls_gb300 import Engine, fgls_chol, launch_count
    from fgls_gb300.datagen import read_outputs
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    n, xb, t = args.n, 4096, 1
    Phi, XL, Y, h, s = make_problem_gpu(n, t, 4321, dev, h=0.5, sigma=2.0)
    pool = [genotype_block(xb, n, 500 + i, dev) for i in range(2)]
    torch.cuda.synchronize()  # the engine's streams do not wait for torch's
    p = WXL + WXR
    dB = torch.empty(xb * p, dtype=torch.float64, device=dev)
    dV = torch.empty(xb * p * p, dtype=torch.float64, device=dev)
    out = {}
    for prec, steps in (("fp64", max(2, args.steps // 6)), ("split", args.steps)):
        eng = Engine(n, WXL, WXR, t, xb, variant="chol", precision=prec, slices=args.slices)
        eng.set_problem(Phi, XL, Y, h, s)
        a = time.perf_counter()
        eng.select_trait(0)
        setup = time.perf_counter() - a
        stream = torch.cuda.ExternalStream(eng.stream(), device=dev)

        def step(k):
            eng.run_block_device(pool[k % 2].data_ptr(), xb, dB.data_ptr(), dV.data_ptr(), xb * p, xb * p * p)

        for k in range(max(1, min(args.warmup, 3))):
            step(k)
        eng.sync()
        eng.profile(True)
        l0 = launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(steps):
            step(k)
        e1.record(stream)
        e1.synchronize()
        eng.sync()
        prof = eng.profile_read()
        eng.profile(False)
        ms = e0.elapsed_time(e1)
        step0 = pool[0]
        eng.run_block_device(step0.data_ptr(), xb, dB.data_ptr(), dV.data_ptr(), xb * p, xb * p * p)
        eng.sync()
        out[prec] = {"value": steps * xb * t / (ms / 1e3), "ms_per_step": ms / steps, "steps": steps,
                     "setup_s": setup, "launches": launch_count() - l0,
                     "kernel_ms_per_step": {k: v[0] / steps for k, v in prof.items() if v[1]},
                     "B": dB.cpu().numpy().reshape(1, xb, p),
                     "V": dV.cpu().numpy().reshape(1, xb, p, p).transpose(0, 1, 3, 2)}
        eng.close()
    nb, bs, se = rel_errors(out["split"]["B"], out["split"]["V"], out["fp64"]["B"], out["fp64"]["V"])
    for v in out.values():
        v.pop("B")
        v.pop("V")
    # end to end through the file entry point (reference layout files on local disk)
    m_e2e = 4 * xb
    e2e = {}
    with tempfile.TemporaryDirectory() as d:
        paths = {k: os.path.join(d, k) for k in ("Phi.in", "H.in", "Sig.in", "XL.in", "XR.in", "Y.in")}
        Phi.T.astype("<f8").tofile(paths["Phi.in"])
        h.astype("<f8").tofile(paths["H.in"])
        s.astype("<f8").tofile(paths["Sig.in"])
        np.asfortranarray(XL).T.astype("<f8").tofile(paths["XL.in"])
        np.asfortranarray(Y).T.astype("<f8").tofile(paths["Y.in"])
        with open(paths["XR.in"], "wb") as f:
            for i in range(m_e2e // xb):
                pool[i % 2].cpu().numpy().astype("<f8").tofile(f)
        for prec in ("fp64", "split"):
            a = time.perf_counter()
            fgls_chol(n, p, m_e2e, t, WXL, WXR, xb, 1, 4, paths["Phi.in"], paths["H.in"], paths["Sig.in"],
                      paths["XL.in"], paths["XR.in"], paths["Y.in"], os.path.join(d, "B.out"),
                      os.path.join(d, "V.out"), env={"FGLS_PRECISION": prec})
            wall = time.perf_counter() - a
            B, _ = read_outputs(d, m_e2e, t, p)
            e2e[prec] = {"value": m_e2e * t / wall, "unit": UNIT, "wall_s": wall, "snps": m_e2e,
                         "finite": bool(np.isfinite(B).all())}
    cpu = None
    if not args.no_cpu:
        xs = 256
        Xc = pool[0][:xs].cpu().numpy().T.copy()
        cv, csec, creps = cpu_chol_throughput(Phi, XL, Y[:, 0], float(h[0]), float(s[0]), Xc, args.cpu_seconds)
        cpu = {"value": cv, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{creps} x {xs} SNPs at n={n}, t=1: oracle restatement of fgls_chol's per-block loop "
                         f"(TRSM + per-SNP Gram and solve, numpy/OpenBLAS, all host threads; the per-trait "
                         f"Cholesky outside the timing), {csec:.1f} s"}
    flops_trsm = float(n) * n * xb
    trsm_ms = out["fp64"]["kernel_ms_per_step"].get("trsm")
    line = {
        "metric": "SNP tests/s, fgls_chol drop-in on 1 GB300 (n=10000, p=4, t=1)",
        "value": out["fp64"]["value"], "unit": UNIT, "n_gpus": 1, "steps": out["fp64"]["steps"],
        "warmup": args.warmup, "ms_per_step": out["fp64"]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"fgls_chol, n={n} p={p} t=1 h=0.5 sigma=2, blocks of {xb} SNPs resident in HBM",
                   "fp64_path": out["fp64"], "split_path": out["split"],
                   "split_vs_fp64_error": {"beta_normwise": nb, "beta_se_scaled": bs, "se_rel": se},
                   "l2": "inputs larger than L2: 2 distinct 0.33 GB blocks cycled"},
        "roofline": {"bound": "fp64", "achieved": flops_trsm / (trsm_ms / 1e3) / 1e12 if trsm_ms else None,
                     "peak": 1.25, "unit": "TFLOP/s", "peak_source": "nominal GB300 FP64 (no measured FP64 peak)",
                     "frac": flops_trsm / (trsm_ms / 1e3) / 1e12 / 1.25 if trsm_ms else None,
                     "kernel": "dtrsm_llnn (dgemm_kernel + diag_solve_kernel)", "traffic": None},
        "e2e": {"value": e2e["fp64"]["value"], "unit": UNIT, "h2d_bytes_per_step": xb * n * 8,
                "d2h_bytes_per_step": xb * (p + p * p) * 8,
                "api": "fgls_chol file entry point, XR read from a local file through the pinned ring, "
                       "setup included", "split": e2e["split"], "fp64": e2e["fp64"]},
        "gpu_launches": out["fp64"]["launches"], "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """Adjoint workload: n = 5000, p = 4, t = 16, FP64 forward and adjoint of
    the eigen variant per block of 4096 SNPs (Gram blocks recomputed in the
    backward pass), cotangent ~ N(0, 1)."""
    import torch
    from fgls_gb300 import Engine, launch_count
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    n, t, xb = 5000, 16, 4096
    p = WXL + WXR
    Phi, XL, Y, h, s = make_problem_gpu(n, t, 99, dev)
    eng = Engine(n, WXL, WXR, t, xb, variant="eigen", precision="fp64")
    a = time.perf_counter()
    eng.set_problem(Phi, XL, Y, h, s)
    setup = time.perf_counter() - a
    eng.adjoint_reset()
    pool = [genotype_block(xb, n, 700 + i, dev) for i in range(2)]
    g = torch.Generator(device=dev).manual_seed(5)
    bbar = torch.randn(t * xb * p, generator=g, device=dev, dtype=torch.float64)
    torch.cuda.synchronize()  # the engine's streams do not wait for torch's
    dB = torch.empty(t * xb * p, dtype=torch.float64, device=dev)
    dV = torch.empty(t * xb * p * p, dtype=torch.float64, device=dev)
    stream = torch.cuda.ExternalStream(eng.stream(), device=dev)
    res = {}
    for name in ("forward", "adjoint"):
        def step(k):
            X = pool[k % 2].data_ptr()
            if name == "forward":
                eng.run_block_device(X, xb, dB.data_ptr(), dV.data_ptr(), xb * p, xb * p * p)
            else:
                eng.adjoint_block_device(X, xb, bbar.data_ptr(), xb * p)
        for k in range(2):
            step(k)
        eng.sync()
        l0 = launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            step(k)
        e1.record(stream)
        e1.synchronize()
        eng.sync()
        ms = e0.elapsed_time(e1)
        res[name] = {"tests_per_s": args.steps * xb * t / (ms / 1e3), "ms_per_block": ms / args.steps,
                     "launches": launch_count() - l0}
    # end to end through the C ABI: pinned host genotypes and cotangent in,
    # forward B and the accumulated gradients out, copies inside the timing
    Xh = pool[0].cpu().pin_memory()
    Bbh = bbar.cpu().pin_memory()
    Bh = torch.empty(t * xb * p, dtype=torch.float64, pin_memory=True)
    Xd = torch.empty_like(pool[1])
    Bbd = torch.empty_like(bbar)
    E = 3
    eng.sync()
    a = time.perf_counter()
    with torch.cuda.stream(stream):
        for _ in range(E):
            Xd.copy_(Xh, non_blocking=True)
            Bbd.copy_(Bbh, non_blocking=True)
            eng.run_block_device(Xd.data_ptr(), xb, dB.data_ptr(), dV.data_ptr(), xb * p, xb * p * p)
            eng.adjoint_block_device(Xd.data_ptr(), xb, Bbd.data_ptr(), xb * p)
            Bh.copy_(dB, non_blocking=True)
    stream.synchronize()
    dh_e, ds_e, dY_e = eng.adjoint_read()
    e2e_s = time.perf_counter() - a
    e2e = {"value": E * xb * t / e2e_s, "unit": UNIT, "h2d_bytes_per_step": xb * n * 8 + t * xb * p * 8,
           "d2h_bytes_per_step": t * xb * p * 8 + 2 * t * 8, "blocks": E,
           "api": "fglsgpu_run_block_device + fglsgpu_adjoint_block_device from pinned host buffers, "
                  "fglsgpu_adjoint_read"}
    del Xh, Bbh, Bh, Xd, Bbd
    dh, ds, dY = eng.adjoint_read()
    ll, dll = eng.reml()
    cpu = None
    if not args.no_cpu:
        # the oracle's FP64 forward (beta) and adjoint on the device's
        # eigendecomposition, over a sample of SNPs
        from oracle import fgls_oracle as O
        W, Z = eng.eigen()
        xs = 64
        Xc = pool[0][:xs].cpu().numpy().T.copy()
        Bb = bbar.view(t, xb, p)[:, :xs].cpu().numpy()
        reps, tot = 0, 0.0
        while reps == 0 or tot < args.cpu_seconds:
            a = time.perf_counter()
            O.eigen_betas(Z, W, XL, Y, h, s, Xc)
            O.eigen_adjoint(Z, W, XL, Y, h, s, Xc, Bb)
            tot += time.perf_counter() - a
            reps += 1
        cpu = {"value": reps * xs * t / tot, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{reps} x ({xs} SNPs x {t} traits) at n={n}: oracle FP64 forward (beta) + adjoint "
                         f"(numpy/OpenBLAS, all host threads), {tot:.1f} s"}
        del Z
    eng.close()
    both = 1.0 / (1.0 / res["forward"]["tests_per_s"] + 1.0 / res["adjoint"]["tests_per_s"])
    # FP64 work per block (GEMM-shaped terms; nq = t (1 + wXL)): forward Z^T X
    # 2 n^2 x, Gram terms 2 n x (nq + t); adjoint recomputes Z^T X and three
    # weightings of the Gram terms, and accumulates R g (2 n t x)
    nq = t * (1 + WXL)
    fwd_flops = 2.0 * n * n * xb + 2.0 * n * xb * (nq + t)
    adj_flops = 2.0 * n * n * xb + 6.0 * n * xb * (nq + t) + 2.0 * n * t * xb
    step_s = (res["forward"]["ms_per_block"] + res["adjoint"]["ms_per_block"]) / 1e3
    achieved = (fwd_flops + adj_flops) / step_s / 1e12
    line = {
        "metric": "SNP×trait tests/s, fgls_eigen FP64 forward + adjoint on 1 GB300 (n=5000, t=16)",
        "value": both, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": 2,
        "ms_per_step": res["forward"]["ms_per_block"] + res["adjoint"]["ms_per_block"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"eigen forward + adjoint, n={n} p={p} t={t}, blocks of {xb} SNPs, m=100000 job",
                   "setup_s": setup, "forward": res["forward"], "adjoint": res["adjoint"],
                   "job_s_estimate": 100000 * t / both + setup,
                   "grad_finite": bool(np.isfinite(dh).all() and np.isfinite(dY).all()),
                   "reml_dll_dh": [float(v) for v in dll[:4]]},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": 1.25, "unit": "TFLOP/s",
                     "frac": achieved / 1.25, "traffic": None,
                     "kernel": "dgemm_kernel (Z^T X and the Gram GEMMs of forward and adjoint)",
                     "peak_source": "nominal GB300 FP64 (no measured FP64 peak)",
                     "work": f"{(fwd_flops + adj_flops) / 1e12:.3f} TFLOP of FP64 GEMM work per block of {xb} SNPs"},
        "e2e": e2e,
        "gpu_launches": res["forward"]["launches"] + res["adjoint"]["launches"], "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def run_kernels(args):
    """The HBM-bound kernels around the split GEMM at the headline size
    (n = 10000, t = 100, one 16384-SNP block), each timed with CUDA events on
    the engine stream; achieved GB/s from the algorithmic bytes of each:
    genotype operand build (FP64 and 2-bit packed input), batched p x p
    solves with B/V emission, p-values, the compact beta/SE/p output, the
    FP64 path's 2-bit unpack + widening, and the REML fit of all traits."""
    import torch
    from fgls_gb300 import Engine
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    n, t, xb, p = args.n, args.t, args.xb, WXL + WXR
    pk, pk_kind = peaks()
    hbm = float(pk.get("hbm_gbs", FALLBACK_PEAKS["hbm_gbs"]))
    Phi, XL, Y, h, s = make_problem_gpu(n, t, 1234, dev)
    eng = Engine(n, WXL, WXR, t, xb, variant="eigen", precision="split", slices=args.slices)
    eng.set_problem(Phi, XL, Y, h, s)
    X = genotype_block(xb, n, 100, dev)
    Xpk = pack_2bit_device(X)
    torch.cuda.synchronize()  # the engine's streams do not wait for torch's
    dB = torch.empty(t * xb * p, dtype=torch.float64, device=dev)
    dV = torch.empty(t * xb * p * p, dtype=torch.float64, device=dev)
    stream = torch.cuda.ExternalStream(eng.stream(), device=dev)
    reps = max(3, args.steps // 4)
    out = {}

    def timed(fn, reps=reps):
        fn()
        eng.sync()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        b.synchronize()
        eng.sync()
        return a.elapsed_time(b) / reps

    def classes(fn, reps=reps):
        fn()
        eng.sync()
        eng.profile(True)
        for _ in range(reps):
            fn()
        eng.sync()
        pr = eng.profile_read()
        eng.profile(False)
        return {k: v[0] / max(v[1], 1) for k, v in pr.items() if v[1]}

    def gbs(nbytes, ms):
        return {"ms": ms, "bytes": nbytes, "GB_s": nbytes / (ms / 1e3) / 1e9, "frac_of_hbm": nbytes / (ms / 1e3) / 1e9 / hbm}

    Kpad = -(-n // 128) * 128
    blk = lambda packed=False: eng.run_block_device(  # noqa: E731
        (Xpk if packed else X).data_ptr(), xb, dB.data_ptr(), dV.data_ptr(), xb * p, xb * p * p, packed=packed)
    c64 = classes(lambda: blk())
    cpk = classes(lambda: blk(packed=True))
    out["genotypes_f8_kernel (FP64 input)"] = gbs(xb * n * 8 + xb * Kpad, c64["genotypes"])
    out["genotypes_packed_f8_kernel"] = gbs(xb * ((n + 3) // 4) + xb * Kpad, cpk["genotypes"])
    # solves: per test the Gram terms in (1 + wXL + 1 doubles: x~'y~, x~'XL~, x~'x~) and B, V out
    out["snp_solve_kernel"] = gbs(t * xb * ((1 + WXL + 1) + p + p * p) * 8, c64["solve"])
    dP = torch.empty(t * xb * WXR, dtype=torch.float64, device=dev)
    ms = timed(lambda: eng.pvalues_device(dB.data_ptr(), dV.data_ptr(), xb, xb * p, xb * p * p, dP.data_ptr(),
                                          xb * WXR))
    out["pvalues_kernel"] = gbs(t * xb * WXR * 3 * 8, ms)  # beta_k and SE_k in, p out
    # FP64 path with packed input: 2-bit unpack + widening to FP64 (a smaller block: the FP64 GEMM is slow)
    eng.set_precision("fp64")
    x64 = 1024
    c = classes(lambda: eng.run_block_device(Xpk.data_ptr(), x64, dB.data_ptr(), dV.data_ptr(), x64 * p,
                                             x64 * p * p, packed=True), reps=2)
    out["unpack_2bit_kernel + u8_to_f64_kernel (FP64 path)"] = gbs(x64 * ((n + 3) // 4) + x64 * n * (1 + 1 + 8),
                                                                    c["genotypes"])
    eng.set_precision("split")
    # compact beta/SE/p output through the host API (pinned host genotypes, 2
    # blocks); the snp_compact kernel's own time is in the launch list
    Xh = torch.empty((2 * xb, n), dtype=torch.float64, pin_memory=True)
    Xh[:xb].copy_(X)
    Xh[xb:].copy_(X)
    a = time.perf_counter()
    eng.run_snps_compact(Xh.numpy().T)
    out["run_snps_compact (host API, 2 blocks)"] = {"ms": (time.perf_counter() - a) * 1e3,
                                                    "tests": 2 * xb * t, "note": "host-timed, copies included"}
    eng.reml_fit()
    a = time.perf_counter()
    eng.reml_fit()
    out["reml_fit_kernel"] = {"ms": (time.perf_counter() - a) * 1e3, "traits": t,
                              "bytes_per_evaluation": (WXL + 2) * n * 8, "note": "host-timed, one launch"}
    eng.close()
    del Xh
    line = {"metric": "HBM-bound kernels of the split eigen path (achieved GB/s)", "value": None, "unit": "GB/s",
            "n_gpus": 1, "steps": reps, "warmup": 1, "higher_is_better": True, "data": "synthetic",
            "config": {"workload": f"n={n} t={t} block of {xb} SNPs", "kernels": out,
                       "hbm_peak_gbs": hbm, "peak_source": f"{pk_kind} hbm_gbs"}}
    print(json.dumps(line), flush=True)


COHORT_BUCKETS = ((500, 1000), (1000, 2000), (2000, 4000), (4000, 8001))


def make_cohorts(count, m, t, seed, dev):
    """Uneven cohorts: n log-uniform in [500, 8000], p uniform in 3..8
    (intercept + p-2 N(0,1) covariates + 1 SNP), t traits with h ~ U(0.1, 0.9),
    sigma ~ U(0.5, 2); kinship G G^T / 5000 + 1e-3 I from standardised
    genotypes G (n x 5000, FP32 product, symmetrised in FP64); seeds derived
    from one master seed."""
    import torch
    rng = np.random.default_rng(seed)
    out = []
    for c in range(count):
        n = int(round(np.exp(rng.uniform(np.log(500), np.log(8000)))))
        p = int(rng.integers(3, 9))
        g = torch.Generator(device=dev).manual_seed(int(rng.integers(1 << 31)))
        k = 5000
        f = torch.rand(k, generator=g, device=dev) * 0.45 + 0.05
        G = (torch.rand(n, k, generator=g, device=dev) < f).float() + (torch.rand(n, k, generator=g, device=dev) < f).float()
        G = (G - G.mean(0)) / G.std(0, unbiased=False).clamp_min(1e-6)
        P = (G @ G.T / k).double()
        Phi = 0.5 * (P + P.T)
        Phi.diagonal().add_(1e-3)
        h = torch.rand(t, generator=g, device=dev, dtype=torch.float64) * 0.8 + 0.1
        sg = torch.rand(t, generator=g, device=dev, dtype=torch.float64) * 1.5 + 0.5
        XL = torch.ones(n, p - 1, device=dev, dtype=torch.float64)
        XL[:, 1:] = torch.randn(n, p - 2, generator=g, device=dev, dtype=torch.float64)
        u = torch.randn(k, t, generator=g, device=dev, dtype=torch.float64)
        v = torch.randn(n, t, generator=g, device=dev, dtype=torch.float64)
        Y = (G.double() @ u) / k ** 0.5 * torch.sqrt(h * sg) + v * torch.sqrt(h * sg * 1e-3 + (1 - h) * sg)
        out.append({"Phi": Phi.cpu().numpy(), "XL": XL.cpu().numpy(), "Y": Y.cpu().numpy(),
                    "h": h.cpu().numpy(), "sigma": sg.cpu().numpy(), "n": n, "p": p, "t": t, "m": m,
                    "seed": int(rng.integers(1 << 31))})
        del G, P, Phi
    torch.cuda.empty_cache()
    return out


def run_cohorts(args):
    """Batched uneven cohorts: 64 problems, m = 200000 SNPs and t = 4 traits
    each, split precision, one grouped launch per stage, CUDA-graph steps,
    x_b and slices from the autotuner unless given."""
    import torch
    from fgls_gb300 import Batch, launch_count
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    C, M, T = args.cohorts, 200_000, 4
    t0 = time.perf_counter()
    co = make_cohorts(C, M, T, 7, dev)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = Batch(co, x_b=args.xb if args.xb_set else 0, slices=args.slices if args.slices_set else 0,
              use_graph=True, genotypes_u8=True, tol=1e-10)
    setup_s = time.perf_counter() - t0
    xb, S, perr = b.params()
    tile = b.tile()
    log(f"[bench] cohorts: data {gen_s:.1f}s, setup {setup_s:.1f}s, x_b={xb}, slices={S}, probe err {perr:.2e}")
    pool = 2
    X = [[genotype_block(xb, c["n"], c["seed"] + i, dev).to(torch.uint8) for i in range(pool)] for c in co]
    torch.cuda.synchronize()  # the batch's stream does not wait for torch's
    dB = [torch.empty(T * xb * c["p"], dtype=torch.float64, device=dev) for c in co]
    dV = [torch.empty(T * xb * c["p"] ** 2, dtype=torch.float64, device=dev) for c in co]
    stream = torch.cuda.ExternalStream(b.stream(), device=dev)
    bp, vp = [d.data_ptr() for d in dB], [d.data_ptr() for d in dV]

    def step(k, active=None):
        xs = [xb if active is None or active(c) else 0 for c in co]
        b.step([X[i][k % pool].data_ptr() for i in range(C)], xs, bp, vp)
        return sum(x * c["t"] for x, c in zip(xs, co))

    for k in range(args.warmup):
        step(k)
    b.sync()
    uuid = "GPU-" + str(torch.cuda.get_device_properties(0).uuid)
    sampler = ClockSampler(uuid)
    l0 = launch_count()
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    tests = 0
    for k in range(args.steps):
        tests += step(args.warmup + k)
    e1.record(stream)
    e1.synchronize()
    clocks = sampler.stop()
    launches = launch_count() - l0
    b.sync()
    ms = e0.elapsed_time(e1)
    value = tests / (ms / 1e3)
    # per size bucket: the other cohorts idle (x = 0) within the same batch
    buckets = {}
    for lo, hi in COHORT_BUCKETS:
        act = (lambda c, lo=lo, hi=hi: lo <= c["n"] < hi)
        if not any(act(c) for c in co):
            continue
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        tb = sum(step(k, act) for k in range(2))
        f1.record(stream)
        f1.synchronize()
        buckets[f"n_{lo}_{hi - 1 if hi == 8001 else hi}"] = {
            "cohorts": sum(1 for c in co if act(c)), "tests_per_s": tb / (f0.elapsed_time(f1) / 1e3)}
    b.sync()
    # stage times (profiled steps run without the graph)
    b.profile(True)
    for k in range(2):
        step(k)
    b.sync()
    prof, nprof = b.profile_read()
    b.profile(False)
    # tensor-core work of the grouped split GEMM per step: 2 S (nU n + n^2/2) per SNP and trait
    flops = sum(2.0 * S * ((c["p"]) * c["n"] + 0.5 * c["n"] ** 2) * xb * c["t"] for c in co)
    gemm_ms = prof["split_gemm"] / max(nprof, 1)
    pk, pk_kind = peaks()
    # FP8 (E4M3) MMAs: twice the measured BF16 rate, burst or sustained by the
    # length of the timed region (as for the eigen workload)
    timed_s = ms / 1e3
    pk_key = "bf16_tflops" if timed_s < 3.0 else "bf16_tflops_sustained"
    peak = 2.0 * float(pk.get(pk_key, FALLBACK_PEAKS[pk_key]))
    # algorithmic bytes of one grouped launch: every problem's S digit slices
    # (triangular L^-1 plus the U rows) and every cohort's E4M3 genotypes read
    # once; per problem the U-row outputs (FP64) and the 32-row group sums of
    # R^2 (float pairs) written once
    algo_bytes = sum(c["t"] * (S * (c["n"] * (c["n"] + 1) / 2 + c["p"] * c["n"])
                               + 8 * xb * (c["p"] + (c["n"] + 31) // 32)) + xb * c["n"] for c in co)
    traffic = gemm_traffic(f"grouped_gemm_cohorts{C}_xb{xb}") if S == 9 else None
    # end to end: host pinned genotypes -> device, step, results -> host
    Xh = [X[i][0].cpu().pin_memory() for i in range(C)]
    Bh = [torch.empty_like(d, device="cpu").pin_memory() for d in dB]
    Vh = [torch.empty_like(d, device="cpu").pin_memory() for d in dV]
    Xd = [X[i][1] for i in range(C)]
    E = 3
    torch.cuda.synchronize()
    a = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(E):
            for i in range(C):
                Xd[i].copy_(Xh[i], non_blocking=True)
            b.step([Xd[i].data_ptr() for i in range(C)], [xb] * C, bp, vp)
            for i in range(C):
                Bh[i].copy_(dB[i], non_blocking=True)
                Vh[i].copy_(dV[i], non_blocking=True)
    stream.synchronize()
    e2e_s = time.perf_counter() - a
    b.sync()
    e2e_tests = E * sum(xb * c["t"] for c in co)
    cpu = None
    if not args.no_cpu:
        # the oracle's fgls_chol block loop (TRSM + per-SNP Gram and solve) on
        # every 4th cohort in order of size, one trait, 64 SNPs each
        order = sorted(range(C), key=lambda i: co[i]["n"])[::4]
        xs, tests, tot = 64, 0, 0.0
        for i in order:
            c = co[i]
            Xc = X[i][0][:xs].cpu().numpy().T.astype(np.float64)
            _, sec, reps = cpu_chol_throughput(c["Phi"], c["XL"], c["Y"][:, 0], float(c["h"][0]),
                                               float(c["sigma"][0]), Xc, 0.0)
            tests += reps * xs
            tot += sec
        cpu = {"value": tests / tot, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{len(order)} cohorts (every 4th by n) x {xs} SNPs x 1 trait: oracle restatement of "
                         f"fgls_chol's per-block loop (numpy/OpenBLAS, all host threads; per-trait Cholesky "
                         f"outside the timing), {tot:.1f} s"}
    # release every tensor that touched the batch's stream before the stream goes
    del Xh, Bh, Vh, Xd, X, dB, dV, stream
    import gc
    gc.collect()
    torch.cuda.synchronize()
    b.close()
    line = {
        "metric": "SNP×trait tests/s, batched uneven cohorts (64 problems), split precision",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp8-e4m3", "data": "synthetic",
        "config": {"workload": f"{C} cohorts, n log-uniform [500, 8000], p in 3..8, t={T}, m={M} each; "
                               f"steps of x_b={xb} SNPs of every cohort",
                   "cohorts": C, "n": [c["n"] for c in co], "p": [c["p"] for c in co], "t": T, "m": M,
                   "x_b": xb, "slices": S, "probe_beta_err": perr, "setup_s": setup_s,
                   "gemm_tile": f"{tile[0]}x{tile[1]}" + (" (autotuned: 256x256 on CTA pairs vs 128x256 on one SM)"
                                                          if not args.xb_set else ""),
                   "job_s_estimate": C * M * T / value + setup_s, "buckets": buckets,
                   "stage_ms_per_step": {k: v / max(nprof, 1) for k, v in prof.items()},
                   "l2": f"inputs larger than L2: {pool} blocks per cohort, "
                         f"{pool * xb * sum(c['n'] for c in co) / 1e9:.2f} GB of genotypes cycled"},
        "roofline": {"bound": "tensor", "achieved": flops / (gemm_ms / 1e3) / 1e12, "peak": peak,
                     "unit": "TFLOP/s", "frac": flops / (gemm_ms / 1e3) / 1e12 / peak, "traffic": traffic,
                     "algorithmic_bytes": algo_bytes,
                     "kernel": ("ozaki_grouped_gemm2_kernel (2-SM CTA pairs, 256 x 256 tiles)" if tile[0] == 256 else
                                "ozaki_grouped_gemm_kernel (one SM, 128 x 256 tiles)")
                               + ", FP8 five-bit digit slices, one accumulator per slice pair",
                     "peak_source": f"2 x {pk_kind} {pk_key} (FP8 dense rate = 2 x BF16; timed region {timed_s:.2f} s)",
                     "nominal_fp8_tflops": NOMINAL_FP8_TFLOPS,
                     "frac_of_nominal": flops / (gemm_ms / 1e3) / 1e12 / NOMINAL_FP8_TFLOPS},
        "e2e": {"value": e2e_tests / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": xb * sum(c["n"] for c in co),
                "d2h_bytes_per_step": sum(T * xb * (c["p"] + c["p"] ** 2) * 8 for c in co),
                "api": "fglsgpu_batch_step (host pinned u8 genotypes -> host B/V)", "steps": E},
        "gpu_launches": launches, "clocks": clocks, "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    """The reference's CPU algorithm (oracle restatement of fgls_eigen's
    per-block loop, src/fgls_eigen.c:471-565) on the host cores."""
    if rank != 0:
        return
    from oracle import fgls_oracle  # noqa: F401  (checker; timed here as the reference arm)
    n, t = args.n, args.t
    rng = np.random.default_rng(7)
    xs = args.ref_snps
    W = np.sort(rng.uniform(1e-3, 6.0, size=n))
    Z = orthogonal_basis(n, 7)
    XL = np.ones((n, WXL))
    XL[:, 1:] = rng.standard_normal((n, WXL - 1))
    Y = rng.standard_normal((n, t))
    h = rng.uniform(0.1, 0.9, t)
    s = rng.uniform(0.5, 2.0, t)
    f = rng.uniform(0.05, 0.5, xs)
    X = rng.binomial(2, f, size=(n, xs)).astype(np.float64)
    val, sec, reps = cpu_port_throughput(Z, W, XL, Y, h, s, X, 0, steps=(args.warmup, args.steps))
    cores = os.cpu_count()
    sample = f"{xs} SNPs x {t} traits per step at n={n}: Z^T XR block + per-trait rescale + per-SNP solves"
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"fgls_eigen per-block loop, n={n} p=4 t={t}, CPU restatement", "n": n, "t": t,
                   "p": 4, "snps_per_step": xs},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_IND)
    ap.add_argument("--t", type=int, default=T_TRAITS)
    ap.add_argument("--xb", type=int, default=16384)
    ap.add_argument("--slices", type=int, default=0)  # 0: the engine's probe autotuner picks 6..9
    ap.add_argument("--pool", type=int, default=4)
    ap.add_argument("--e2e-blocks", type=int, default=8)
    ap.add_argument("--fp64-snps", type=int, default=2048)
    ap.add_argument("--oracle-snps", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-snps", type=int, default=128)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="eigen", choices=["eigen", "cohorts", "chol", "adjoint", "kernels"])
    ap.add_argument("--cohorts", type=int, default=64)
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "cohorts":
        args.xb_set = any(a.startswith("--xb") for a in sys.argv[1:])
        args.slices_set = any(a.startswith("--slices") for a in sys.argv[1:])
        return run_cohorts(args)
    if args.workload == "chol":
        return run_chol(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "kernels":
        return run_kernels(args)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    try:
        line = run_eigen(args, rank, world, local, dist)
        if rank == 0:
            print(json.dumps(line), flush=True)
    finally:
        if dist:
            dist.destroy_process_group()


def run_eigen(args, rank, world, local, dist):
    """The headline workload (split-precision fgls_eigen, n = 10000, t = 100);
    returns rank 0's JSON record."""
    import torch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from fgls_gb300 import Engine, launch_count

    n, t, xb, p = args.n, args.t, args.xb, WXL + WXR
    pk, pk_kind = peaks()
    t0 = time.perf_counter()
    Phi, XL, Y, h, s = make_problem_gpu(n, t, 1234, dev)
    gen_s = time.perf_counter() - t0
    eng = Engine(n, WXL, WXR, t, xb, variant="eigen", precision="split", slices=args.slices, device=local)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.set_problem(Phi, XL, Y, h, s)
    setup_s = time.perf_counter() - t0
    S_used, S_err = eng.split_params()
    QD_used = eng.quad_digits()
    log(f"[bench] rank {rank}: data {gen_s:.1f}s, setup (eigendecomposition + operands) {setup_s:.1f}s, "
        f"slices {S_used}, quadratic-Gram digits {QD_used} (probe err {S_err:.2e})")

    pool = [genotype_block(xb, n, sd, dev) for sd in rank_block_seeds(rank, args.pool)]
    torch.cuda.synchronize()  # the engine's streams do not wait for torch's
    dB = torch.empty(t * xb * p, dtype=torch.float64, device=dev)
    dV = torch.empty(t * xb * p * p, dtype=torch.float64, device=dev)
    stream = torch.cuda.ExternalStream(eng.stream(), device=dev)

    def step(k):
        eng.run_block_device(pool[k % len(pool)].data_ptr(), xb, dB.data_ptr(), dV.data_ptr(), xb * p, xb * p * p)

    for k in range(args.warmup):
        step(k)
    eng.sync()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    uuid = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
    sampler = ClockSampler(uuid)
    eng.profile(True)
    l0 = launch_count()
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for k in range(args.steps):
        step(args.warmup + k)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    launches = launch_count() - l0
    ms = e0.elapsed_time(e1)
    eng.sync()
    prof = eng.profile_read()
    eng.profile(False)
    ms = max_over_ranks(ms, dist, dev)
    value = aggregate_throughput(world, args.steps, xb, t, ms / 1e3)

    # roofline of the dominant kernel, the tcgen05 split GEMM: sliced FP8 MMA
    # operations per launch = 2 S M_A n per SNP column, M_A = n + t (1 + wXL)
    M_A = n + t * (1 + WXL)
    flops_snp = 2.0 * S_used * M_A * n
    gemm_ms, gemm_n = prof["split_gemm"]
    gemm_s = gemm_ms / 1e3
    achieved = flops_snp * xb * args.steps / gemm_s / 1e12
    # FP8 (E4M3) MMAs run at twice the BF16 rate on GB300; no FP8 figure is
    # measured, so the peak is twice the measured BF16 rate: the burst figure
    # for a timed region under 3 s, the sustained one above
    timed_s = ms / 1e3
    pk_key = "bf16_tflops" if timed_s < 3.0 else "bf16_tflops_sustained"
    peak = 2.0 * float(pk.get(pk_key, FALLBACK_PEAKS[pk_key]))
    traffic = gemm_traffic(f"ozaki_gemm_n{n}_t{t}_xb{xb}")
    Mpad, Kpad = -(-M_A // 128) * 128, -(-n // 128) * 128
    algo_bytes = S_used * Mpad * Kpad + xb * Kpad + 8 * Mpad * xb  # A slices + genotypes read, C written once

    # all-FP64 device path on the same problem (same eigendecomposition)
    eng.set_precision("fp64")
    x64 = min(args.fp64_snps, xb)
    Xp = pool[0][:x64].contiguous()
    torch.cuda.synchronize()
    dB64 = torch.empty(t * x64 * p, dtype=torch.float64, device=dev)
    dV64 = torch.empty(t * x64 * p * p, dtype=torch.float64, device=dev)
    eng.run_block_device(Xp.data_ptr(), x64, dB64.data_ptr(), dV64.data_ptr(), x64 * p, x64 * p * p)
    eng.sync()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    reps64 = 2
    for _ in range(reps64):
        eng.run_block_device(Xp.data_ptr(), x64, dB64.data_ptr(), dV64.data_ptr(), x64 * p, x64 * p * p)
    f1.record(stream)
    f1.synchronize()
    eng.sync()
    fp64_value = reps64 * x64 * t / (f0.elapsed_time(f1) / 1e3)
    B64 = dB64.cpu().numpy().reshape(t, x64, p)
    V64 = dV64.cpu().numpy().reshape(t, x64, p, p).transpose(0, 1, 3, 2)
    eng.set_precision("split")
    dBs = torch.empty_like(dB64)
    dVs = torch.empty_like(dV64)
    eng.run_block_device(Xp.data_ptr(), x64, dBs.data_ptr(), dVs.data_ptr(), x64 * p, x64 * p * p)
    eng.sync()
    Bs = dBs.cpu().numpy().reshape(t, x64, p)
    Vs = dVs.cpu().numpy().reshape(t, x64, p, p).transpose(0, 1, 3, 2)
    nb, bs, se = rel_errors(Bs, Vs, B64, V64)
    # p-values of the SNP coefficient from both paths (device kernel)
    dP64 = torch.empty(t * x64 * WXR, dtype=torch.float64, device=dev)
    dPs = torch.empty_like(dP64)
    eng.pvalues_device(dB64.data_ptr(), dV64.data_ptr(), x64, x64 * p, x64 * p * p, dP64.data_ptr(), x64 * WXR)
    eng.pvalues_device(dBs.data_ptr(), dVs.data_ptr(), x64, x64 * p, x64 * p * p, dPs.data_ptr(), x64 * WXR)
    eng.sync()
    P64, Ps = dP64.cpu().numpy(), dPs.cpu().numpy()
    pv_rel = float(np.max(np.abs(Ps - P64) / np.maximum(P64, 1e-300)))

    # end to end through the public host API: pinned host genotypes in the
    # reference XR layout, results back in the B.out / V.out layout
    E = args.e2e_blocks
    Xh = torch.empty((E * xb, n), dtype=torch.float64, pin_memory=True)
    for i in range(E):
        Xh[i * xb:(i + 1) * xb].copy_(pool[i % len(pool)])
    Bh = torch.empty(t * E * xb * p, dtype=torch.float64, pin_memory=True)
    Vh = torch.empty(t * E * xb * p * p, dtype=torch.float64, pin_memory=True)
    eng.run_snps_ptr(Xh.data_ptr(), xb, Bh.data_ptr(), Vh.data_ptr())  # warm
    if dist:
        dist.barrier()
    # five whole calls; the median is reported (the host memory and link are
    # shared on these machines: single FP64-input calls, which move 134 GB/s
    # of genotypes, have run up to 3x slower than the others of a run)
    e2e_runs = []
    for _ in range(E2E_CALLS):
        a = time.perf_counter()
        eng.run_snps_ptr(Xh.data_ptr(), E * xb, Bh.data_ptr(), Vh.data_ptr())
        e2e_runs.append(max_over_ranks(time.perf_counter() - a, dist, dev))
    e2e_s = statistics.median(e2e_runs)
    e2e_value = aggregate_throughput(world, E, xb, t, e2e_s)
    # the same blocks as hard calls packed 2 bits per individual (SNP-major
    # PLINK .bed body) through fglsgpu_run_snps_packed: 32x fewer input bytes
    B_f64 = Bh.clone()
    Xpk = torch.empty((E * xb, (n + 3) // 4), dtype=torch.uint8, pin_memory=True)
    for i in range(E):
        Xpk[i * xb:(i + 1) * xb].copy_(pack_2bit_device(pool[i % len(pool)]))
    eng.run_snps_genotypes_ptr(Xpk.data_ptr(), xb, Bh.data_ptr(), Vh.data_ptr(), packed=True)  # warm
    pk_runs = []
    for _ in range(E2E_CALLS):
        a = time.perf_counter()
        eng.run_snps_genotypes_ptr(Xpk.data_ptr(), E * xb, Bh.data_ptr(), Vh.data_ptr(), packed=True)
        pk_runs.append(max_over_ranks(time.perf_counter() - a, dist, dev))
    e2e_packed = {"value": aggregate_throughput(world, E, xb, t, statistics.median(pk_runs)), "unit": UNIT,
                  "h2d_bytes_per_step": xb * ((n + 3) // 4), "d2h_bytes_per_step": t * xb * (p + p * p) * 8,
                  "api": "fglsgpu_run_snps_packed (host pinned 2-bit SNP-major .bed body -> host B/V)",
                  "calls": [aggregate_throughput(world, E, xb, t, x) for x in pk_runs],
                  "stat": f"median of {E2E_CALLS} calls",
                  "beta_identical_to_fp64_input": bool(torch.equal(Bh, B_f64))}
    del Xh, Bh, Vh, Xpk, B_f64

    # variance components of every trait re-estimated on the device (REML,
    # sigma profiled out, h on a 64-point grid refined to the gradient root)
    eng.reml_fit()
    a = time.perf_counter()
    h_fit, s_fit, _, _ = eng.reml_fit()
    reml = {"device_ms": (time.perf_counter() - a) * 1e3, "traits": t, "grid": 64,
            "h_mean_abs_dev_from_truth": float(np.mean(np.abs(h_fit - np.asarray(h)))),
            "api": "fglsgpu_reml_fit"}

    # the split path against the FP64 oracle at the full problem size: the
    # oracle's restatement of the reference's per-block eigen loop
    # (src/fgls_eigen.c:428-565, res_sigma :998-1160) on the device's
    # eigendecomposition, itself pinned by its residuals on sampled vectors
    cpu = None
    pin = None
    if rank == 0:
        from oracle import fgls_oracle as O
        W, Z = eng.eigen()
        pin = eigen_residuals(Phi, W, Z)
        xs = min(args.oracle_snps, x64)
        Xc = pool[0][:xs].cpu().numpy().T.copy()
        st = O.eigen_setup(Z, W, XL, Y, h, s, WXL)
        Br, Vr = O.eigen_block(st, Xc, WXR)
        pin.update(oracle_errors(Bs[:, :xs], Vs[:, :xs], Br, Vr, WXL))
        pin["fp64_path"] = oracle_errors(B64[:, :xs], V64[:, :xs], Br, Vr, WXL)
        pin.update({"snps": xs, "traits": t, "gate": GATE})
        if world == 1 and not args.no_cpu:
            a = time.perf_counter()
            O.reml_fit(W, Z.T @ np.asarray(XL), Z.T @ np.asarray(Y)[:, :1], 0.0, 1.0 - 1e-5, 64)
            reml["cpu_oracle_ms_per_trait"] = (time.perf_counter() - a) * 1e3
            cv, csec, creps = cpu_port_throughput(Z, W, XL, Y, h, s, Xc, args.cpu_seconds)
            cpu = {"value": cv, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                   "sample": f"{creps} x ({xs} SNPs x {t} traits) at n={n}, oracle restatement of the reference's "
                             f"per-block eigen loop (numpy/OpenBLAS, all host threads), {creps * csec:.1f} s"}
        del Z
    eng.close()
    if rank != 0:
        return None
    gate_ok = all(pin[k] <= GATE for k in ("beta_normwise", "beta_se_scaled", "se_rel"))
    line = {
        "metric": METRIC, "value": value if gate_ok else None, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp8-e4m3", "data": "synthetic",
        "config": {
            "workload": f"fgls_eigen split-precision, n={n} p=4 t={t}, job m={M_JOB} SNPs, "
                        f"steps of x_b={xb} SNPs x {t} traits",
            "n": n, "t": t, "p": 4, "m_job": M_JOB, "x_b": xb, "slices": S_used, "quad_digits": QD_used,
            "slices_choice": ("autotuned: smallest of 6..9 slices, then of 8..11 quadratic-Gram digits, within "
                              f"1e-10/8 of the FP64 path on a 256-SNP probe block (probe beta error {S_err:.2e})"
                              if args.slices == 0 else "given"),
            "genotype_input": "FP64 reference layout, resident in HBM",
            "l2": f"inputs larger than L2: {len(pool)} distinct {xb * n * 8 / 1e9:.2f} GB blocks cycled",
            "setup_s": setup_s, "job_s_estimate": M_JOB * t / value + setup_s,
            "fp64_path": {"value": fp64_value, "unit": UNIT, "snps": x64,
                          "speedup_split_vs_fp64": value / fp64_value},
            "split_vs_oracle_error": pin,
            "split_vs_fp64_error": {"beta_normwise": nb, "beta_se_scaled": bs, "se_rel": se,
                                    "pvalue_rel": pv_rel, "snps": x64, "traits": t},
            "kernel_ms": {k: v[0] for k, v in prof.items() if v[1]},
            "reml_fit": reml,
        },
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic, "algorithmic_bytes": algo_bytes,
                     "kernel": "ozaki_gemm2_kernel (2-SM CTA pairs, tcgen05.mma.cta_group::2)",
                     "peak_source": f"2 x {pk_kind} {pk_key} (FP8 dense rate = 2 x BF16; "
                                    f"timed region {timed_s:.2f} s)",
                     "nominal_fp8_tflops": NOMINAL_FP8_TFLOPS,
                     "frac_of_nominal": achieved / NOMINAL_FP8_TFLOPS,
                     "fp64_equivalent_tflops": 2.0 * M_A * n * xb * args.steps / gemm_s / 1e12,
                     "work": f"2*{S_used} slices*{M_A} rows*{n} K per SNP; {gemm_n} launches, "
                             f"{gemm_ms / max(gemm_n, 1):.3f} ms each"},
        "e2e": {"value": e2e_value if gate_ok else None, "unit": UNIT, "h2d_bytes_per_step": xb * n * 8,
                "d2h_bytes_per_step": t * xb * (p + p * p) * 8,
                "api": "fglsgpu_run_snps (host pinned FP64 XR -> host B/V)", "blocks": E,
                "calls": [aggregate_throughput(world, E, xb, t, x) for x in e2e_runs],
                "stat": f"median of {E2E_CALLS} calls",
                "packed_genotypes": e2e_packed},
        "gpu_launches": launches,
        "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if not gate_ok:
        line["gate_failed"] = {k: pin[k] for k in ("beta_normwise", "beta_se_scaled", "se_rel")}
        line["value_if_passed"] = value
    return line


if __name__ == "__main__":
    main()
