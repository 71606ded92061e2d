"""Batched uneven cohorts (fglsgpu_batch_*): every cohort's results against
the oracle's chol restatement (src/fgls_chol.c:251-438), through ragged
steps, graph replay, idle cohorts and the autotuner.

Tolerances are those of the single-problem split chol path: beta within
1e-10 of the FP64 oracle on the (|beta| + SE) scale and normwise, SE
within 1e-10 relative.
"""
import numpy as np
import pytest

from conftest import report
from oracle import fgls_oracle as O

pytestmark = pytest.mark.gpu

# (n, wXL, t, m): p = wXL + 1 covers 3..8; n crosses tile boundaries
COHORTS = [(100, 2, 2, 300), (257, 3, 1, 257), (300, 7, 3, 500), (513, 4, 2, 200), (700, 5, 1, 333)]


def cohorts(spec=COHORTS, seed=20):
    from fgls_gb300 import datagen
    pbs = [datagen.make_problem(n, m, t, wXL=w, seed=seed + k, hsig_uniform=True)
           for k, (n, w, t, m) in enumerate(spec)]
    desc = [{"Phi": pb.Phi, "XL": pb.XL, "Y": pb.Y, "h": pb.h, "sigma": pb.sigma} for pb in pbs]
    return pbs, desc


def run_batch(batch, pbs, x_b, u8=True, idle=None):
    """All SNPs of every cohort in steps of up to x_b; at step `idle` the
    even cohorts sit out.  Returns per-cohort B (t, m, p), V (t, m, p, p)."""
    import torch
    X = [torch.from_numpy(np.ascontiguousarray(pb.XR.T.astype(np.uint8 if u8 else np.float64))).cuda()
         for pb in pbs]
    out = [(np.zeros((pb.t, pb.m, pb.p)), np.zeros((pb.t, pb.m, pb.p, pb.p))) for pb in pbs]
    pos = [0] * len(pbs)
    s = 0
    while any(q < pb.m for q, pb in zip(pos, pbs)):
        xs, xp, bp, vp, bufs = [], [], [], [], []
        for k, pb in enumerate(pbs):
            x = min(x_b, pb.m - pos[k])
            if s == idle and k % 2 == 0:
                x = 0
            dB = torch.empty(max(1, pb.t * x * pb.p), dtype=torch.float64, device="cuda")
            dV = torch.empty(max(1, pb.t * x * pb.p * pb.p), dtype=torch.float64, device="cuda")
            bufs.append((k, pos[k], x, dB, dV))
            xs.append(x)
            xp.append(X[k][min(pos[k], pb.m - 1)].data_ptr())
            bp.append(dB.data_ptr())
            vp.append(dV.data_ptr())
        batch.step(xp, xs, bp, vp, list(pos))
        batch.sync()
        for k, i0, x, dB, dV in bufs:
            pos[k] += x
            if x == 0:
                continue
            pb = pbs[k]
            out[k][0][:, i0:i0 + x] = dB.cpu().numpy()[:pb.t * x * pb.p].reshape(pb.t, x, pb.p)
            out[k][1][:, i0:i0 + x] = dV.cpu().numpy()[:pb.t * x * pb.p * pb.p].reshape(
                pb.t, x, pb.p, pb.p).transpose(0, 1, 3, 2)
        s += 1
    return out


def check(pbs, out):
    for pb, (B, V) in zip(pbs, out):
        Br, Vr = O.fgls_chol(pb)
        d = O.compare(B, V, Br, Vr)
        assert d["finite"] and d["upper_abs_max"] == 0.0, (pb.n, d)
        report(f"batch_n{pb.n}_p{pb.p}", **d)
        assert d["beta_se_scaled"] <= 1e-10 and d["beta_normwise"] <= 1e-10, (pb.n, pb.p, d)
        assert d["se_rel"] <= 1e-10, (pb.n, pb.p, d)


def test_batch_matches_oracle_per_cohort_with_graph():
    from fgls_gb300 import Batch
    pbs, desc = cohorts()
    with Batch(desc, x_b=256, slices=9, use_graph=True) as b:
        assert b.params()[:2] == (256, 9)
        out = run_batch(b, pbs, 256)
    check(pbs, out)


def test_batch_graph_replay_is_bit_identical_and_idle_cohorts():
    from fgls_gb300 import Batch
    pbs, desc = cohorts(COHORTS[:3], seed=40)
    with Batch(desc, x_b=128, slices=9, use_graph=False) as b:
        ref = run_batch(b, pbs, 128)
    with Batch(desc, x_b=128, slices=9, use_graph=True) as b:
        got = run_batch(b, pbs, 128, idle=1)
    for (B1, V1), (B2, V2) in zip(ref, got):
        assert np.array_equal(B1, B2) and np.array_equal(V1, V2)


def test_batch_tile_shapes_are_bit_identical():
    """The grouped split GEMM on 256 x 256 tiles over CTA pairs (2-SM MMAs,
    row-tile pairs from the launch-wide counter, odd row-tile counts leaving a
    phantom second tile) and on 128 x 256 tiles on one SM: every partial sum
    is an exact integer, so the results agree to the bit, and both match the
    oracle."""
    from fgls_gb300 import Batch
    pbs, desc = cohorts(seed=70)
    outs = []
    for rows in (256, 128):
        with Batch(desc, x_b=256, slices=9, use_graph=True, tile_rows=rows) as b:
            assert b.tile() == (rows, 256)
            outs.append(run_batch(b, pbs, 256))
    for (B1, V1), (B2, V2) in zip(*outs):
        assert np.array_equal(B1, B2) and np.array_equal(V1, V2)
    check(pbs, outs[0])


def test_batch_fp64_genotype_input():
    from fgls_gb300 import Batch
    pbs, desc = cohorts(COHORTS[1:3], seed=60)
    with Batch(desc, x_b=256, slices=9, use_graph=True, genotypes_u8=False) as b:
        out = run_batch(b, pbs, 256, u8=False)
    check(pbs, out)


def test_batch_autotuner_meets_tolerance():
    from fgls_gb300 import Batch
    pbs, desc = cohorts(COHORTS[:4], seed=80)
    with Batch(desc, x_b=0, slices=0, use_graph=True, tol=1e-10) as b:
        x_b, S, perr = b.params()
        assert x_b in (1024, 2048, 4096, 8192) and 5 <= S <= 9
        assert 0.0 <= perr <= 1e-10 / 8
        assert b.tile() in ((256, 256), (128, 256))  # the faster grouped GEMM tile at x_b
        out = run_batch(b, pbs, x_b)
    check(pbs, out)
