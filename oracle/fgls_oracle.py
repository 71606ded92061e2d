"""CPU FP64 restatement of the reference FGLS association path.

TEST INFRASTRUCTURE ONLY.  This module is the checker for the CUDA library:
only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import it, and never as the thing measured or shipped.

It restates, with numpy/scipy LAPACK, the arithmetic of:

* ``fgls_chol``  src/fgls_chol.c:223-439 (per trait: M, potrf, whitening,
  null-model residual variance; per SNP: Gram, potrf, two trsv, potri,
  res_sigma scaling, square-root diagonal);
* ``fgls_eigen`` src/fgls_eigen.c:428-565 (per trait Winv rescale, per SNP
  Gram and solve), src/fgls_eigen.c:998-1160 (residual_sigma) and
  src/fgls_eigen.c:861-893 (dsyevr of Phi, lower triangle).

Pinned against the reference itself: tests/golden/ holds B/V produced by the
reference's own driver (built from its sources by oracle/build_ref.sh) on
seeded synthetic inputs, and tests/test_oracle.py checks this module against
those files.

Output conventions follow the reference exactly:
B[j, i] = beta (p values, order [XL coefs, XR coefs]);
V[j, i] = res_sigma * S^-1 lower triangle (row r >= column c), the diagonal
replaced by its square root (the standard errors), strict upper = 0
(src/fgls_chol.c:427-438).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla


def _lower(A):
    return np.tril(A)


def _sym_from_lower(A):
    L = np.tril(A)
    return L + np.tril(L, -1).T


def null_model_chol(L, XL, y, wXL):
    """src/fgls_chol.c:273-325: whitened covariates, trait, top blocks and the
    null-model residual variance res_sigma = r^T r / (n - wXL)."""
    n = XL.shape[0]
    XLt = sla.solve_triangular(L, XL, lower=True)          # :275 dtrsm
    yt = sla.solve_triangular(L, y, lower=True)            # :291 dtrsv
    B_t = XLt.T @ yt                                       # :294 dgemv
    V_tl = XLt.T @ XLt                                     # :297 dsyrk (lower used)
    cL = np.linalg.cholesky(_sym_from_lower(V_tl))         # :308 dpotrf
    bL = sla.cho_solve((cL, True), B_t)                    # :315-316 two dtrsv
    r = sla.solve_triangular(L, y - XL @ bL, lower=True)   # :318-324
    res_sigma = float(r @ r) / (n - wXL)                   # :325
    return XLt, yt, B_t, V_tl, res_sigma


def snp_solve(B_t, V_tl, XLt, yt, Xt, wXL, wXR, res_sigma):
    """src/fgls_chol.c:386-439 for a block.  Xt: n x (x*wXR) whitened SNP
    columns.  Returns B (x, p) and V (x, p, p) [row, col]."""
    x = Xt.shape[1] // wXR
    p = wXL + wXR
    XtR = Xt.reshape(Xt.shape[0], x, wXR)
    bB = np.einsum("nxc,n->xc", XtR, yt)                   # :396-399 dgemv
    SBL = np.einsum("nxc,nk->xck", XtR, XLt)               # :406-409 dgemm
    SBR = np.einsum("nxc,nxd->xcd", XtR, XtR)              # :411-414 dsyrk
    S = np.zeros((x, p, p))
    S[:, :wXL, :wXL] = _sym_from_lower(V_tl)
    S[:, wXL:, :wXL] = SBL
    S[:, :wXL, wXL:] = SBL.transpose(0, 2, 1)
    S[:, wXL:, wXL:] = SBR
    b = np.concatenate([np.broadcast_to(B_t, (x, wXL)), bB], axis=1)
    C = np.linalg.cholesky(S)                              # :417 dpotrf
    beta = np.linalg.solve(S, b[..., None])[..., 0]        # :424-425 (same solution)
    Ci = np.linalg.inv(C)
    Sinv = np.einsum("xki,xkj->xij", Ci, Ci)               # :428 dpotri = C^-T C^-1
    V = np.tril(Sinv) * res_sigma                          # :435-436 dscal on the lower part
    idx = np.arange(p)
    V[:, idx, idx] = np.sqrt(V[:, idx, idx])               # :437-438 SE on the diagonal
    return beta, V


def fgls_chol(pb, x_b=None):
    """Whole-job restatement of fgls_chol on a datagen.Problem."""
    n, m, t, wXL, wXR = pb.n, pb.m, pb.t, pb.wXL, pb.wXR
    p = wXL + wXR
    x_b = x_b or m
    B = np.zeros((t, m, p))
    V = np.zeros((t, m, p, p))
    Phil = np.tril(pb.Phi)
    for j in range(t):
        alpha = pb.h[j] * pb.sigma[j]                      # :253
        beta = (1.0 - pb.h[j]) * pb.sigma[j]               # :254
        M = alpha * _sym_from_lower(Phil)                  # :252-255
        M[np.diag_indices(n)] += beta                      # :256-257
        L = np.linalg.cholesky(M)                          # :263
        XLt, yt, B_t, V_tl, rs = null_model_chol(L, pb.XL, pb.Y[:, j], wXL)
        for ib in range(0, m, x_b):
            xi = min(x_b, m - ib)
            Xt = sla.solve_triangular(L, pb.XR[:, ib * wXR:(ib + xi) * wXR], lower=True)  # :368
            bb, vv = snp_solve(B_t, V_tl, XLt, yt, Xt, wXL, wXR, rs)
            B[j, ib:ib + xi] = bb
            V[j, ib:ib + xi] = vv
    return B, V


def eigen_decomp(Phi):
    """src/fgls_eigen.c:861-893: dsyevr('V','A','L') -> W ascending, Z."""
    W, Z = sla.eigh(np.tril(Phi), lower=True, driver="evr")
    return W, Z


def residual_sigma_eigen(Z, W, XL, ZtXL, Y, ZtY, h, sigma, wXL):
    """src/fgls_eigen.c:1085-1160."""
    n = XL.shape[0]
    t = Y.shape[1]
    rs = np.empty(t)
    for j in range(t):
        a = sigma[j] * h[j]
        b = sigma[j] * (1.0 - h[j])
        Winv = np.sqrt(1.0 / (a * W + b))                  # :1097
        yc = ZtY[:, j] * Winv                              # :1102
        XLc = ZtXL * Winv[:, None]                         # :1108
        Bt = XLc.T @ yc
        Vt = XLc.T @ XLc
        cL = np.linalg.cholesky(Vt)
        bL = sla.cho_solve((cL, True), Bt)                 # :1131-1139
        ymxb = Y[:, j] - XL @ bL                           # :1142-1146
        tmp = (Z.T @ ymxb) * Winv                          # :1148-1157
        rs[j] = float(tmp @ tmp) / (n - wXL)               # :1158-1159
    return rs


def fgls_eigen(pb, W=None, Z=None):
    """Whole-job restatement of fgls_eigen on a datagen.Problem."""
    n, m, t, wXL, wXR = pb.n, pb.m, pb.t, pb.wXL, pb.wXR
    p = wXL + wXR
    if W is None:
        W, Z = eigen_decomp(pb.Phi)
    ZtXL = Z.T @ pb.XL                                     # :720-744 ooc_gemm
    ZtXR = Z.T @ pb.XR                                     # :752-770
    ZtY = Z.T @ pb.Y                                       # :778-796
    rs = residual_sigma_eigen(Z, W, pb.XL, ZtXL, pb.Y, ZtY, pb.h, pb.sigma, wXL)
    B = np.zeros((t, m, p))
    V = np.zeros((t, m, p, p))
    for j in range(t):
        a = pb.sigma[j] * pb.h[j]                          # :430
        b = pb.sigma[j] * (1.0 - pb.h[j])                  # :431
        Winv = np.sqrt(1.0 / (a * W + b))                  # :441
        yc = ZtY[:, j] * Winv                              # :447
        XLc = ZtXL * Winv[:, None]                         # :453
        B_t = XLc.T @ yc                                   # :457
        V_tl = XLc.T @ XLc                                 # :462-465
        Xc = ZtXR * Winv[:, None]                          # :505-507
        bb, vv = snp_solve(B_t, V_tl, XLc, yc, Xc, wXL, wXR, rs[j])
        B[j] = bb
        V[j] = vv
    return B, V


def eigen_setup(Z, W, XL, Y, h, sigma, wXL):
    """Per-problem state of the eigen variant given the basis (Z, W):
    src/fgls_eigen.c:720-796 (Z^T XL, Z^T Y) and :998-1195 (res_sigma)."""
    ZtXL = Z.T @ XL
    ZtY = Z.T @ Y
    rs = residual_sigma_eigen(Z, W, XL, ZtXL, Y, ZtY, h, sigma, wXL)
    return {"Z": Z, "W": W, "ZtXL": ZtXL, "ZtY": ZtY, "rs": rs, "h": h, "sigma": sigma, "wXL": wXL}


def eigen_block(st, XR_blk, wXR=1):
    """One SNP block of fgls_eigen for all traits, as the reference's
    ooc_loops does it: Z^T XR_blk (src/fgls_eigen.c:962), then per trait the
    Winv rescale of the whole block (:505-507) and the per-SNP Gram and solve
    (:512-565).  Returns B (t, x, p), V (t, x, p, p)."""
    Z, W, wXL = st["Z"], st["W"], st["wXL"]
    ZtXR = Z.T @ XR_blk
    t = st["ZtY"].shape[1]
    Bs, Vs = [], []
    for j in range(t):
        a = st["sigma"][j] * st["h"][j]
        b = st["sigma"][j] * (1.0 - st["h"][j])
        Winv = np.sqrt(1.0 / (a * W + b))
        yc = st["ZtY"][:, j] * Winv
        XLc = st["ZtXL"] * Winv[:, None]
        B_t = XLc.T @ yc
        V_tl = XLc.T @ XLc
        Xc = ZtXR * Winv[:, None]
        bb, vv = snp_solve(B_t, V_tl, XLc, yc, Xc, wXL, wXR, st["rs"][j])
        Bs.append(bb)
        Vs.append(vv)
    return np.stack(Bs), np.stack(Vs)


# ---------------------------------------------------------------------------
# Comparators.  Element-wise relative error on beta is ill-posed for
# coefficients near zero (the reference's own chol and eigen variants differ
# by ~2e-10 element-wise there while agreeing to ~6e-13 per SNP normwise), so
# beta is compared normwise per (trait, SNP); standard errors element-wise;
# the off-diagonal covariances normwise per (trait, SNP) relative to the
# block's norm; the strict upper triangle must be exactly zero.
# ---------------------------------------------------------------------------

def compare(B, V, Bref, Vref):
    p = B.shape[-1]
    dB = np.linalg.norm(B - Bref, axis=-1) / np.maximum(np.linalg.norm(Bref, axis=-1), 1e-300)
    idx = np.arange(p)
    se = V[..., idx, idx]
    se_ref = Vref[..., idx, idx]
    dSE = np.abs(se - se_ref) / np.abs(se_ref)
    low = np.tril(np.ones((p, p), bool), -1)
    offd = V[..., low]
    offd_ref = Vref[..., low]
    nV = np.linalg.norm(Vref.reshape(*Vref.shape[:-2], -1), axis=-1)
    dV = (np.linalg.norm(offd - offd_ref, axis=-1) / np.maximum(nV, 1e-300)) if low.any() else np.zeros_like(dB)
    # |dbeta_k| / (|beta_k| + SE_k): error on the statistical scale of each
    # coefficient, well-posed when beta_k is near zero.
    dBs = np.abs(B - Bref) / (np.abs(Bref) + se_ref)
    up = np.triu(np.ones((p, p), bool), 1)
    upper_max = float(np.abs(V[..., up]).max()) if up.any() else 0.0
    return {
        "beta_normwise": float(dB.max()),
        "beta_se_scaled": float(dBs.max()),
        "se_rel": float(dSE.max()),
        "v_offdiag_normwise": float(dV.max()),
        "upper_abs_max": upper_max,
        "finite": bool(np.isfinite(B).all() and np.isfinite(V).all()),
    }


# ---------------------------------------------------------------------------
# Derivatives (no counterpart in the reference): FP64 CPU reference for the
# adjoint of the eigen variant and the null-model REML log-likelihood.
# ---------------------------------------------------------------------------

def eigen_betas(Z, W, XL, Y, h, sigma, XR):
    """beta (t, m, p) of fgls_eigen for wXR = 1 in the d-weighted form
    S = sum_l d_l v_l v_l^T, b = sum_l d_l v_l ytil_l."""
    ZtXL, ZtY, R = Z.T @ XL, Z.T @ Y, Z.T @ XR
    t, m, wXL = Y.shape[1], XR.shape[1], XL.shape[1]
    out = np.zeros((t, m, wXL + 1))
    for j in range(t):
        d = 1.0 / (sigma[j] * h[j] * W + sigma[j] * (1 - h[j]))
        V = np.concatenate([np.broadcast_to(ZtXL[None], (m,) + ZtXL.shape), R.T[:, :, None]], axis=2)  # m x n x p
        S = np.einsum("mlp,l,mlq->mpq", V, d, V)
        b = np.einsum("mlp,l,l->mp", V, d, ZtY[:, j])
        out[j] = np.linalg.solve(S, b[..., None])[..., 0]
    return out


def eigen_adjoint(Z, W, XL, Y, h, sigma, XR, Bbar):
    """(dL/dh (t), dL/dsigma (t), dL/dY (n x t)) for L = sum Bbar * beta."""
    ZtXL, ZtY, R = Z.T @ XL, Z.T @ Y, Z.T @ XR
    t, m, wXL = Y.shape[1], XR.shape[1], XL.shape[1]
    dh, ds, dY = np.zeros(t), np.zeros(t), np.zeros((Z.shape[0], t))
    V = np.concatenate([np.broadcast_to(ZtXL[None], (m,) + ZtXL.shape), R.T[:, :, None]], axis=2)
    for j in range(t):
        s, hj = sigma[j], h[j]
        d = 1.0 / (s * hj * W + s * (1 - hj))
        c = -s * (W - 1.0) * d * d
        sg = -d / s
        S = np.einsum("mlp,l,mlq->mpq", V, d, V)
        b = np.einsum("mlp,l,l->mp", V, d, ZtY[:, j])
        beta = np.linalg.solve(S, b[..., None])[..., 0]
        g = np.linalg.solve(S, Bbar[j][..., None])[..., 0]
        r = ZtY[:, j][None, :] - np.einsum("mlp,mp->ml", V, beta)       # m x n
        Vg = np.einsum("mlp,mp->ml", V, g)                               # m x n
        dh[j] = np.sum(Vg * r * c[None, :])
        ds[j] = np.sum(Vg * r * sg[None, :])
        dY[:, j] = Z @ (d * Vg.sum(0))
    return dh, ds, dY


def reml(Z, W, XL, Y, h, sigma):
    """Null-model REML log-likelihood per trait (sigma given, constants
    dropped) and its h-derivative, in the eigenbasis of Phi."""
    ZtXL, ZtY = Z.T @ XL, Z.T @ Y
    t = Y.shape[1]
    ll, dll = np.zeros(t), np.zeros(t)
    for j in range(t):
        s, hj = sigma[j], h[j]
        d = 1.0 / (s * hj * W + s * (1 - hj))
        c = -s * (W - 1.0) * d * d
        Vt = (ZtXL * d[:, None]).T @ ZtXL
        bL = np.linalg.solve(Vt, (ZtXL * d[:, None]).T @ ZtY[:, j])
        r0 = ZtY[:, j] - ZtXL @ bL
        Vc = (ZtXL * c[:, None]).T @ ZtXL
        ll[j] = -0.5 * (-np.sum(np.log(d)) + np.linalg.slogdet(Vt)[1] + np.sum(d * r0 * r0))
        dll[j] = -0.5 * (-np.sum(c / d) + np.trace(np.linalg.solve(Vt, Vc)) + np.sum(c * r0 * r0))
    return ll, dll


def reml_profiled(W, ZtXL, zty, h):
    """Profiled null-model REML of one trait at h (sigma = sigma_hat(h)).

    The reference reads h and sigma from files (src/fgls_chol.c:139-145) and
    uses M = sigma (h Phi + (1 - h) I) (src/fgls_chol.c:251-256).  With
    d = 1/(h w + 1 - h), sigma_hat(h) = r^T D r / (n - wXL) for the GLS
    residual r, and the value/gradient are ``reml`` evaluated at
    (h, sigma_hat(h)) (the sigma-gradient vanishes there).
    Returns (loglik, dloglik/dh, sigma_hat)."""
    n, wXL = ZtXL.shape
    d = 1.0 / (h * W + (1.0 - h))
    c = -(W - 1.0) * d * d
    G = (ZtXL * d[:, None]).T @ ZtXL
    b = np.linalg.solve(G, (ZtXL * d[:, None]).T @ zty)
    r = zty - ZtXL @ b
    q = float(np.sum(d * r * r))
    nn = n - wXL
    sig = q / nn
    Gc = (ZtXL * c[:, None]).T @ ZtXL
    ll = -0.5 * (nn * np.log(sig) - np.sum(np.log(d)) + np.linalg.slogdet(G)[1] + nn)
    dll = -0.5 * (nn * np.sum(c * r * r) / q - np.sum(c / d) + np.trace(np.linalg.solve(G, Gc)))
    return float(ll), float(dll), sig


def reml_fit(W, ZtXL, ZtY, lo=0.0, hi=1.0 - 1e-5, grid=64):
    """REML estimate of (h, sigma) per trait: the maximiser of the profiled
    likelihood over [lo, hi] found EMMA-style (Kang et al. 2008): grid, every
    + -> - sign change of the gradient solved by Brent's method
    (scipy.optimize.brentq), endpoints whose gradient points outward, best
    value kept.  Returns (h, sigma, loglik, dloglik) arrays of t."""
    from scipy.optimize import brentq
    t = ZtY.shape[1]
    hs = np.linspace(lo, hi, grid)
    out = np.zeros((4, t))
    for j in range(t):
        y = ZtY[:, j]
        f = lambda h: reml_profiled(W, ZtXL, y, h)  # noqa: E731
        ev = [f(h) for h in hs]
        cands = []
        if not ev[0][1] > 0:
            cands.append((hs[0],) + ev[0])
        if ev[-1][1] >= 0:
            cands.append((hs[-1],) + ev[-1])
        for k in range(grid - 1):
            if ev[k][1] > 0 and not ev[k + 1][1] > 0:
                x = brentq(lambda h: f(h)[1], hs[k], hs[k + 1], xtol=1e-15, rtol=1e-15, maxiter=200)
                cands.append((x,) + f(x))
        best = max(cands, key=lambda c: c[1])
        out[:, j] = [best[0], best[3], best[1], best[2]]
    return out[0], out[1], out[2], out[3]
