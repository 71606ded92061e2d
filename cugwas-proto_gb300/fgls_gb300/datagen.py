"""Seeded synthetic FGLS problems written in the reference's on-disk layout.

Layout (all raw little-endian float64, no headers), as read and written by
the reference's ``fgls_chol`` (src/fgls_chol.c:135-157, :333-337, :464-474):

* ``Phi.in``  n x n, column-major; only the lower triangle is used.
* ``H.in``, ``Sig.in``  >= t doubles (heritability h_j and scale sigma_j).
* ``XL.in``   n x wXL column-major covariates (the intercept is a column of
  the file; the reference never adds it, src/fgls_chol.c:146-151).
* ``XR.in``   m SNPs x wXR columns x n; SNP i's columns start at i*wXR*n.
* ``Y.in``    t x n; trait j at offset j*n.

Generator (the shapes and distributions of the workloads this engine is
measured on):

* genotypes XR[:, k] ~ Binomial(2, f_k), f_k ~ U(0.05, 0.5), stored as f64;
* kinship Phi = G G^T / 5000 + 1e-3 I, G an n x 5000 matrix of standardized
  Binomial(2, f) genotypes;
* XL = [1, N(0,1), ...] (intercept plus wXL-1 normal covariates);
* y_j with covariance sigma_j (h_j Phi + (1 - h_j) I).  Drawn as
  sqrt(h s) G u / sqrt(5000) + sqrt(h s 1e-3 + (1-h) s) v with u, v standard
  normal: the same distribution as chol(h s Phi + (1-h) s I) N(0, I) without
  an O(n^3) factorization per trait.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

N_KINSHIP_MARKERS = 5000


@dataclass
class Problem:
    n: int
    m: int
    t: int
    wXL: int
    wXR: int = 1
    Phi: np.ndarray | None = None       # n x n (C-order array of the col-major file == Phi^T == Phi)
    h: np.ndarray | None = None         # t
    sigma: np.ndarray | None = None     # t
    XL: np.ndarray | None = None        # n x wXL (column k = covariate k)
    XR: np.ndarray | None = None        # n x (m*wXR): column i*wXR+c = SNP i, column c
    Y: np.ndarray | None = None         # n x t
    meta: dict = field(default_factory=dict)

    @property
    def p(self) -> int:
        return self.wXL + self.wXR


def standardized_genotypes(rng: np.random.Generator, n: int, k: int) -> np.ndarray:
    f = rng.uniform(0.05, 0.5, size=k)
    g = rng.binomial(2, f, size=(n, k)).astype(np.float64)
    mu = g.mean(axis=0)
    sd = g.std(axis=0)
    sd[sd == 0] = 1.0
    return (g - mu) / sd


def hardcall_genotypes(rng: np.random.Generator, n: int, cols: int) -> np.ndarray:
    """n x cols matrix of 0/1/2 hard calls, per-column frequency U(0.05, 0.5)."""
    f = rng.uniform(0.05, 0.5, size=cols)
    return rng.binomial(2, f, size=(n, cols)).astype(np.float64)


def kinship(rng: np.random.Generator, n: int, markers: int = N_KINSHIP_MARKERS):
    """Returns (Phi, G) with Phi = G G^T / markers + 1e-3 I."""
    G = standardized_genotypes(rng, n, markers)
    Phi = G @ G.T / markers
    Phi[np.diag_indices(n)] += 1e-3
    return Phi, G


def traits(rng: np.random.Generator, G: np.ndarray, h: np.ndarray, sigma: np.ndarray) -> np.ndarray:
    n, k = G.shape
    t = len(h)
    u = rng.standard_normal((k, t))
    v = rng.standard_normal((n, t))
    a = np.sqrt(h * sigma)
    b = np.sqrt(h * sigma * 1e-3 + (1.0 - h) * sigma)
    return (G @ u) / np.sqrt(k) * a + v * b


def make_problem(n: int, m: int, t: int, wXL: int = 3, wXR: int = 1, seed: int = 0,
                 h=None, sigma=None, markers: int = N_KINSHIP_MARKERS,
                 hsig_uniform=False) -> Problem:
    """One seeded problem.  ``h``/``sigma`` scalars or arrays; when
    ``hsig_uniform`` they are drawn h ~ U(0.1, 0.9), sigma ~ U(0.5, 2)."""
    rng = np.random.default_rng(seed)
    Phi, G = kinship(rng, n, markers)
    if hsig_uniform:
        hv = rng.uniform(0.1, 0.9, size=t)
        sv = rng.uniform(0.5, 2.0, size=t)
    else:
        hv = np.full(t, 0.4) if h is None else np.broadcast_to(np.asarray(h, float), (t,)).copy()
        sv = np.full(t, 1.0) if sigma is None else np.broadcast_to(np.asarray(sigma, float), (t,)).copy()
    XL = np.empty((n, wXL))
    XL[:, 0] = 1.0
    if wXL > 1:
        XL[:, 1:] = rng.standard_normal((n, wXL - 1))
    XR = hardcall_genotypes(rng, n, m * wXR)
    Y = traits(rng, G, hv, sv)
    return Problem(n=n, m=m, t=t, wXL=wXL, wXR=wXR, Phi=Phi, h=hv, sigma=sv,
                   XL=XL, XR=XR, Y=Y, meta={"seed": seed})


def _reflect_sym(A: np.ndarray, v: np.ndarray) -> None:
    """A <- H A H in place for symmetric A (Fortran order) and H = I - 2 v v^T,
    |v| = 1: A - 2 (v w'^T + w' v^T) with w = A v, w' = w - (v^T w) v."""
    from scipy.linalg.blas import dger
    w = A @ v
    w -= (v @ w) * v
    dger(-2.0, v, w, a=A, overwrite_a=True)
    dger(-2.0, w, v, a=A, overwrite_a=True)


def _reflect_left(Q: np.ndarray, v: np.ndarray) -> None:
    """Q <- H Q in place (Fortran order), H = I - 2 v v^T."""
    from scipy.linalg.blas import dger
    dger(-2.0, v, v @ Q, a=Q, overwrite_a=True)


def known_spectrum_kinship(rng: np.random.Generator, n: int, markers: int | None = None):
    """A kinship matrix with a known eigendecomposition, built in O(n^2 log n).

    The spectrum is that of G G^T / k + 1e-3 I for standardized genotypes G
    (n x k, k = markers, default n/2): k eigenvalues spread over the
    Marchenko-Pastur support [(sqrt(n/k) - 1)^2, (sqrt(n/k) + 1)^2] plus 1e-3,
    and n - k eigenvalues equal to 1e-3 (a degenerate cluster, as in a real
    kinship of rank k).  The eigenvectors are Q = H1 H2 F: F the orthonormal
    DCT-II matrix (dense, delocalised columns) and H1, H2 Householder
    reflectors along random directions.  Phi = Q diag(d) Q^T is formed as
    H1 H2 (F d F^T) H2 H1 with F d F^T = dct(d * idct(I)), then symmetrised.

    Returns (Phi, W, Z): W ascending, Z the matching columns of Q, so that
    (W, Z) is an exact eigendecomposition of Phi up to the rounding of its
    construction (|Phi Z - Z W| ~ 1e-15 |Phi|)."""
    import scipy.fft as sfft
    k = min(n, markers or max(1, n // 2))
    r = n / k
    lo, hi = (np.sqrt(r) - 1.0) ** 2, (np.sqrt(r) + 1.0) ** 2
    lam = np.full(n, 1e-3)
    lam[:k] += rng.uniform(lo, hi, size=k)
    d = lam[rng.permutation(n)]
    v1 = rng.standard_normal(n)
    v1 /= np.linalg.norm(v1)
    v2 = rng.standard_normal(n)
    v2 /= np.linalg.norm(v2)
    eye = np.eye(n, order="F")
    Ft = sfft.idct(eye, axis=0, norm="ortho", workers=-1)          # F^T (columns F^-1 e_j)
    Ft *= d[:, None]
    Phi = np.asfortranarray(sfft.dct(Ft, axis=0, norm="ortho", workers=-1))  # F d F^T
    del Ft
    _reflect_sym(Phi, v2)
    _reflect_sym(Phi, v1)
    Phi += Phi.T  # exactly symmetric: fl(a + b) = fl(b + a)
    Phi *= 0.5
    Q = np.asfortranarray(sfft.dct(eye, axis=0, norm="ortho", workers=-1))   # F
    del eye
    _reflect_left(Q, v2)
    _reflect_left(Q, v1)
    idx = np.argsort(d, kind="stable")
    return Phi, d[idx].copy(), np.asfortranarray(Q[:, idx])


def make_problem_known_spectrum(n: int, m: int, t: int, wXL: int = 3, wXR: int = 1, seed: int = 0,
                                markers: int | None = None):
    """As make_problem with h ~ U(0.1, 0.9), sigma ~ U(0.5, 2), but the
    kinship from known_spectrum_kinship, so that an FP64 reference can use
    the exact eigendecomposition at any n.  Traits y_j = Z (sqrt(sigma_j
    (h_j W + 1 - h_j)) * N(0, I)), i.e. covariance sigma_j (h_j Phi + (1 - h_j) I).
    Returns (Problem, W, Z)."""
    rng = np.random.default_rng(seed)
    Phi, W, Z = known_spectrum_kinship(rng, n, markers)
    hv = rng.uniform(0.1, 0.9, size=t)
    sv = rng.uniform(0.5, 2.0, size=t)
    XL = np.empty((n, wXL))
    XL[:, 0] = 1.0
    if wXL > 1:
        XL[:, 1:] = rng.standard_normal((n, wXL - 1))
    XR = hardcall_genotypes(rng, n, m * wXR)
    sd = np.sqrt(sv[None, :] * (hv[None, :] * W[:, None] + (1.0 - hv[None, :])))
    Y = Z @ (sd * rng.standard_normal((n, t)))
    pb = Problem(n=n, m=m, t=t, wXL=wXL, wXR=wXR, Phi=Phi, h=hv, sigma=sv, XL=XL, XR=XR, Y=Y,
                 meta={"seed": seed, "kinship": "known spectrum"})
    return pb, W, Z


FILES = ("Phi.in", "H.in", "Sig.in", "XL.in", "XR.in", "Y.in")


def write_problem(pb: Problem, d: str) -> dict:
    """Write the six input files; returns the path dict."""
    os.makedirs(d, exist_ok=True)
    paths = {k: os.path.join(d, k) for k in FILES}
    # column-major n x n: write Phi^T in C order (Phi symmetric, but keep exact)
    np.asfortranarray(pb.Phi).T.astype("<f8").tofile(paths["Phi.in"])
    pb.h.astype("<f8").tofile(paths["H.in"])
    pb.sigma.astype("<f8").tofile(paths["Sig.in"])
    np.asfortranarray(pb.XL).T.astype("<f8").tofile(paths["XL.in"])
    np.asfortranarray(pb.XR).T.astype("<f8").tofile(paths["XR.in"])
    np.asfortranarray(pb.Y).T.astype("<f8").tofile(paths["Y.in"])
    return paths


def read_problem(d: str, n: int, m: int, t: int, wXL: int, wXR: int = 1) -> Problem:
    f = lambda name: np.fromfile(os.path.join(d, name), dtype="<f8")
    Phi = f("Phi.in")[: n * n].reshape(n, n).T.copy()
    h = f("H.in")[:t].copy()
    s = f("Sig.in")[:t].copy()
    XL = f("XL.in")[: n * wXL].reshape(wXL, n).T.copy()
    XR = f("XR.in")[: n * m * wXR].reshape(m * wXR, n).T.copy()
    Y = f("Y.in")[: n * t].reshape(t, n).T.copy()
    return Problem(n=n, m=m, t=t, wXL=wXL, wXR=wXR, Phi=Phi, h=h, sigma=s, XL=XL, XR=XR, Y=Y)


def read_outputs(d: str, m: int, t: int, p: int, bname="B.out", vname="V.out"):
    """B as (t, m, p) and V as (t, m, p, p) with V[j, i] the column-major
    p x p block read into row-major [col][row] order transposed back, i.e.
    V[j, i, r, c] is row r, column c."""
    B = np.fromfile(os.path.join(d, bname), dtype="<f8")
    V = np.fromfile(os.path.join(d, vname), dtype="<f8")
    B = B[: t * m * p].reshape(t, m, p)
    V = V[: t * m * p * p].reshape(t, m, p, p).transpose(0, 1, 3, 2)
    return B, V


def pack_2bit(X: np.ndarray) -> np.ndarray:
    """Hard calls (columns x n, values 0/1/2, or -1 for missing) -> 2-bit
    SNP-major bytes as in a PLINK .bed body: ceil(n/4) bytes per column,
    individual k in bits 2(k%4).., codes 2 -> 00, 1 -> 10, 0 -> 11, missing -> 01."""
    X = np.asarray(X)
    cols, n = X.shape
    code = np.select([X == 2, X == 1, X == 0], [0, 2, 3], default=1).astype(np.uint8)
    pad = (-n) % 4
    code = np.concatenate([code, np.full((cols, pad), 3, np.uint8)], axis=1).reshape(cols, -1, 4)
    return (code[..., 0] | (code[..., 1] << 2) | (code[..., 2] << 4) | (code[..., 3] << 6)).astype(np.uint8)



BED_MAGIC = bytes((0x6C, 0x1B, 0x01))  # PLINK .bed, SNP-major


def write_xr(pb: Problem, path: str, fmt: str = "f64") -> str:
    """XR in one of the drop-in's genotype file formats (FGLS_XR_FORMAT):
    'f64' (the reference's XR.in), 'u8' (one byte per individual, same
    column order) or 'bed' (SNP-major PLINK .bed: magic bytes, then the
    2-bit body of pack_2bit, column i*wXR + c = SNP i, column c)."""
    G = np.asfortranarray(pb.XR).T  # (m*wXR, n)
    if fmt == "f64":
        G.astype("<f8").tofile(path)
    elif fmt == "u8":
        np.ascontiguousarray(G.astype(np.uint8)).tofile(path)
    elif fmt == "bed":
        with open(path, "wb") as f:
            f.write(BED_MAGIC)
            f.write(pack_2bit(G.astype(np.int16)).tobytes())
    else:
        raise ValueError(fmt)
    return path
