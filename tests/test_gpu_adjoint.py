"""Adjoint of the eigen variant (FP64) and the null-model REML gradient,
through the C ABI, wrapped in a test-only torch.autograd.Function.

Checked against the FP64 CPU reference gradient (oracle.eigen_adjoint /
oracle.reml) and central finite differences of the device forward pass
(step 1e-6).  Tolerances: adjoint vs CPU reference 1e-9 relative (both FP64,
different summation orders, eigenvectors from different solvers); vs finite
differences 1e-5 relative (FD truncation and cancellation error at h = 1e-6).
"""
import numpy as np
import pytest

from oracle import fgls_oracle as O

pytestmark = pytest.mark.gpu

N, M, T, XB = 160, 96, 3, 48


def problem(seed=3):
    from fgls_gb300 import datagen
    return datagen.make_problem(N, M, T, seed=seed, hsig_uniform=True)


def forward(pb, h, sigma, Y):
    """beta (t, m, p) from the device eigen path (FP64)."""
    from fgls_gb300 import Engine
    with Engine(pb.n, pb.wXL, 1, pb.t, XB, variant="eigen") as e:
        e.set_problem(pb.Phi, pb.XL, Y, h, sigma)
        B, _ = e.run_snps(pb.XR)
    return B


class FGLSEigenBeta:
    """torch.autograd.Function: (h, sigma, Y) -> beta, backward through the
    device adjoint (fglsgpu_adjoint_*)."""

    @staticmethod
    def make(pb):
        import torch

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, h, sigma, Y):
                ctx.save_for_backward(h, sigma, Y)
                B = forward(pb, h.detach().numpy(), sigma.detach().numpy(), Y.detach().numpy())
                return torch.from_numpy(B)

            @staticmethod
            def backward(ctx, Bbar):
                h, sigma, Y = ctx.saved_tensors
                dh, ds, dY = device_adjoint(pb, h.numpy(), sigma.numpy(), Y.numpy(), Bbar.contiguous().numpy())
                return torch.from_numpy(dh), torch.from_numpy(ds), torch.from_numpy(np.ascontiguousarray(dY))

        return Fn


def device_adjoint(pb, h, sigma, Y, Bbar):
    import torch
    from fgls_gb300 import Engine
    p = pb.p
    with Engine(pb.n, pb.wXL, 1, pb.t, XB, variant="eigen") as e:
        e.set_problem(pb.Phi, pb.XL, Y, h, sigma)
        e.adjoint_reset()
        dX = torch.from_numpy(np.asfortranarray(pb.XR).T.copy()).cuda()     # (m, n) = column-major n x m
        dBbar = torch.from_numpy(np.ascontiguousarray(Bbar)).cuda()          # (t, m, p)
        for ib in range(0, pb.m, XB):
            x = min(XB, pb.m - ib)
            e.adjoint_block_device(dX[ib].data_ptr(), x, dBbar[0, ib].data_ptr(), pb.m * p)
        dh, ds, dY = e.adjoint_read()
        ll, dll = e.reml()
        W, Z = e.eigen()
    device_adjoint.last = (ll, dll, W, Z)
    return dh, ds, dY


def test_adjoint_matches_cpu_reference_gradient():
    pb = problem()
    rng = np.random.default_rng(7)
    Bbar = rng.standard_normal((T, M, pb.p))
    dh, ds, dY = device_adjoint(pb, pb.h, pb.sigma, pb.Y, Bbar)
    ll, dll, W, Z = device_adjoint.last
    rh, rs, rY = O.eigen_adjoint(Z, W, pb.XL, pb.Y, pb.h, pb.sigma, pb.XR, Bbar)
    assert np.allclose(dh, rh, rtol=1e-9, atol=1e-12 * np.abs(rh).max())
    assert np.abs(ds).max() < 1e-9 * np.abs(dh).max()   # beta is scale-invariant in sigma
    assert np.allclose(dY, rY, rtol=1e-9, atol=1e-9 * np.abs(rY).max())
    rll, rdll = O.reml(Z, W, pb.XL, pb.Y, pb.h, pb.sigma)
    assert np.allclose(ll, rll, rtol=1e-10)
    assert np.allclose(dll, rdll, rtol=1e-9, atol=1e-12)


def test_adjoint_autograd_function_vs_finite_differences():
    import torch
    pb = problem(5)
    Fn = FGLSEigenBeta.make(pb)
    h = torch.tensor(pb.h, dtype=torch.float64, requires_grad=True)
    s = torch.tensor(pb.sigma, dtype=torch.float64, requires_grad=True)
    Y = torch.tensor(pb.Y, dtype=torch.float64, requires_grad=True)
    rng = np.random.default_rng(11)
    Bbar = torch.from_numpy(rng.standard_normal((T, M, pb.p)))
    L = (Fn.apply(h, s, Y) * Bbar).sum()
    L.backward()
    eps = 1e-6
    Lf = lambda hh, ss, YY: float(np.sum(Bbar.numpy() * forward(pb, hh, ss, YY)))
    for j in range(T):
        hp, hm = pb.h.copy(), pb.h.copy()
        hp[j] += eps
        hm[j] -= eps
        fd = (Lf(hp, pb.sigma, pb.Y) - Lf(hm, pb.sigma, pb.Y)) / (2 * eps)
        assert abs(h.grad[j].item() - fd) <= 1e-5 * max(1.0, abs(fd)), (j, h.grad[j].item(), fd)
        sp, sm = pb.sigma.copy(), pb.sigma.copy()
        sp[j] += eps
        sm[j] -= eps
        fds = (Lf(pb.h, sp, pb.Y) - Lf(pb.h, sm, pb.Y)) / (2 * eps)
        assert abs(s.grad[j].item() - fds) <= 1e-6, (j, s.grad[j].item(), fds)
    for (l, j) in [(0, 0), (17, 1), (N - 1, 2)]:
        Yp, Ym = pb.Y.copy(), pb.Y.copy()
        Yp[l, j] += eps
        Ym[l, j] -= eps
        fd = (Lf(pb.h, pb.sigma, Yp) - Lf(pb.h, pb.sigma, Ym)) / (2 * eps)
        assert abs(Y.grad[l, j].item() - fd) <= 1e-5 * max(1.0, abs(fd)), (l, j, Y.grad[l, j].item(), fd)


def test_reml_gradient_vs_finite_differences():
    from fgls_gb300 import Engine
    pb = problem(9)

    def reml_at(h):
        with Engine(pb.n, pb.wXL, 1, pb.t, XB, variant="eigen") as e:
            e.set_problem(pb.Phi, pb.XL, pb.Y, h, pb.sigma)
            e.adjoint_reset()
            return e.reml()

    ll, dll = reml_at(pb.h)
    eps = 1e-6
    for j in range(T):
        hp, hm = pb.h.copy(), pb.h.copy()
        hp[j] += eps
        hm[j] -= eps
        fd = (reml_at(hp)[0][j] - reml_at(hm)[0][j]) / (2 * eps)
        assert abs(dll[j] - fd) <= 1e-5 * max(1.0, abs(fd)), (j, dll[j], fd)
