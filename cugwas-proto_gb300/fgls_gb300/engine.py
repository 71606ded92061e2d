"""Python mirror of the C ABI in include/fgls_gb300.h (ctypes, no torch types).

The drop-in functions ``fgls_chol`` / ``fgls_eigen`` / ``fgls_chol_gpu`` take
the reference's 17 arguments (src/fgls_chol.h:4-10, src/fgls_eigen.h:68-74,
src/fgls_chol_gpu.h:4-10) and raise ``FGLSError`` where the reference would
print "[Error]: ..." and exit; they run in a child process so that the
library's exit-on-error behaviour cannot end the caller.

``Engine`` wraps the fglsgpu_* engine API.  Array arguments are numpy FP64
arrays in the natural orientation of the reference's column-major files
(Phi n x n, XL n x wXL, Y n x t, XR n x (m*wXR)); results are returned as
B (traits, m, p) and V (traits, m, p, p) with V[..., r, c] = row r, column c.
There is no CPU fallback: if the CUDA library cannot be loaded, every call
raises.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libfgls_gb300.so")
DRIVER_PATH = os.path.join(PKG, "lib", "fgls-driver")

OK, EINVAL, ENOTSPD, ECUDA, EIO, ENOMEM, ETIMEOUT, ENOCONV, ENODEV, ESTATE = range(10)
VARIANT = {"chol": 0, "eigen": 1}
PRECISION = {"fp64": 0, "split": 1}

# every symbol include/fgls_gb300.h declares
EXPORTS = (
    "fgls_chol", "fgls_eigen", "fgls_chol_gpu", "fglsgpu_create", "fglsgpu_destroy",
    "fglsgpu_set_problem", "fglsgpu_select_trait", "fglsgpu_run_block", "fglsgpu_run_snps",
    "fglsgpu_run_block_device", "fglsgpu_run_block_device_u8", "fglsgpu_sync",
    "fglsgpu_get_res_sigma", "fglsgpu_get_eigen", "fglsgpu_stream", "fglsgpu_launch_count",
    "fglsgpu_last_error", "fglsgpu_version", "fglsgpu_selftest_split_gemm", "fglsgpu_set_precision",
    "fglsgpu_profile", "fglsgpu_profile_read", "fglsgpu_split_gemm_noalloc", "fglsgpu_adjoint_reset",
    "fglsgpu_adjoint_block_device", "fglsgpu_adjoint_read", "fglsgpu_reml", "fglsgpu_pvalues_device",
    "fglsgpu_batch_create", "fglsgpu_batch_destroy", "fglsgpu_batch_params", "fglsgpu_batch_step",
    "fglsgpu_batch_sync", "fglsgpu_batch_stream", "fglsgpu_batch_last_error", "fglsgpu_batch_profile",
    "fglsgpu_batch_profile_read", "fglsgpu_run_block_device_packed", "fglsgpu_run_snps_compact",
    "fglsgpu_reml_fit", "fglsgpu_set_hsigma", "fglsgpu_set_wait_limit", "fglsgpu_run_snps_u8",
    "fglsgpu_run_snps_packed", "fglsgpu_split_params", "fglsgpu_quad_digits", "fglsgpu_batch_tile",
)
PROF_CLASSES = ("genotypes", "split_gemm", "selfgram", "solve", "fp64_gemm", "trsm", "gram", "spare")


class FGLSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [(f, C.c_int) for f in
                ("n", "wXL", "wXR", "t", "x_b", "variant", "precision", "slices", "device", "reserved")]


class CohortDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("wXL", C.c_int), ("t", C.c_int)] + \
               [(f, C.c_void_p) for f in ("Phi", "XL", "Y", "h", "sigma")]


class BatchConfig(C.Structure):
    _fields_ = [(f, C.c_int) for f in ("x_b", "slices", "device", "use_graph", "genotypes_u8", "tile_rows")] + \
               [("tol", C.c_double)]


_lib = None


def lib():
    """Loads libfgls_gb300.so (built in-tree); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FGLSError(ENODEV, f"{LIB_PATH} not built: run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    P, I, LL, D = C.c_void_p, C.c_int, C.c_longlong, C.POINTER(C.c_double)
    L.fglsgpu_create.argtypes = [C.POINTER(Config), C.POINTER(P)]
    L.fglsgpu_destroy.argtypes = [P]
    L.fglsgpu_set_problem.argtypes = [P, P, P, P, P, P]
    L.fglsgpu_select_trait.argtypes = [P, I]
    L.fglsgpu_run_block.argtypes = [P, P, I, P, P, LL, LL]
    L.fglsgpu_run_snps.argtypes = [P, P, LL, P, P]
    L.fglsgpu_run_snps_compact.argtypes = [P, P, LL, P, P, P]
    L.fglsgpu_run_snps_u8.argtypes = [P, P, LL, P, P]
    L.fglsgpu_run_snps_packed.argtypes = [P, P, LL, P, P]
    L.fglsgpu_run_block_device.argtypes = [P, P, I, P, P, LL, LL]
    L.fglsgpu_run_block_device_u8.argtypes = [P, P, I, P, P, LL, LL]
    L.fglsgpu_run_block_device_packed.argtypes = [P, P, I, P, P, LL, LL]
    L.fglsgpu_sync.argtypes = [P]
    L.fglsgpu_get_res_sigma.argtypes = [P, P]
    L.fglsgpu_get_eigen.argtypes = [P, P, P]
    L.fglsgpu_stream.argtypes = [P]
    L.fglsgpu_stream.restype = P
    L.fglsgpu_launch_count.argtypes = [P]
    L.fglsgpu_launch_count.restype = LL
    L.fglsgpu_last_error.argtypes = [P]
    L.fglsgpu_last_error.restype = C.c_char_p
    L.fglsgpu_version.restype = I
    L.fglsgpu_selftest_split_gemm.argtypes = [I, I, I, I, P, P, P]
    L.fglsgpu_set_precision.argtypes = [P, I]
    L.fglsgpu_profile.argtypes = [P, I]
    L.fglsgpu_profile_read.argtypes = [P, P, P]
    L.fglsgpu_split_gemm_noalloc.argtypes = [I, I, I, I, P, P, P, P]
    L.fglsgpu_adjoint_reset.argtypes = [P]
    L.fglsgpu_adjoint_block_device.argtypes = [P, P, I, P, LL]
    L.fglsgpu_adjoint_read.argtypes = [P, P, P, P]
    L.fglsgpu_reml.argtypes = [P, P, P]
    L.fglsgpu_reml_fit.argtypes = [P, C.c_double, C.c_double, I, P, P, P, P]
    L.fglsgpu_set_hsigma.argtypes = [P, P, P]
    L.fglsgpu_set_wait_limit.argtypes = [P, LL]
    L.fglsgpu_split_params.argtypes = [P, C.POINTER(I), C.POINTER(C.c_double)]
    L.fglsgpu_quad_digits.argtypes = [P, C.POINTER(I)]
    L.fglsgpu_pvalues_device.argtypes = [P, P, P, I, LL, LL, P, LL]
    L.fglsgpu_batch_create.argtypes = [C.POINTER(CohortDesc), I, C.POINTER(BatchConfig), C.POINTER(P)]
    L.fglsgpu_batch_destroy.argtypes = [P]
    L.fglsgpu_batch_params.argtypes = [P, C.POINTER(I), C.POINTER(I), C.POINTER(C.c_double)]
    L.fglsgpu_batch_tile.argtypes = [P, C.POINTER(I), C.POINTER(I)]
    L.fglsgpu_batch_step.argtypes = [P, P, P, P, P, P]
    L.fglsgpu_batch_sync.argtypes = [P]
    L.fglsgpu_batch_stream.argtypes = [P]
    L.fglsgpu_batch_stream.restype = P
    L.fglsgpu_batch_last_error.argtypes = [P]
    L.fglsgpu_batch_last_error.restype = C.c_char_p
    L.fglsgpu_batch_profile.argtypes = [P, I]
    L.fglsgpu_batch_profile_read.argtypes = [P, P, C.POINTER(LL)]
    _lib = L
    return L


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def _f64(a, order="F"):
    return np.require(np.asarray(a, dtype=np.float64), requirements=[order, "A"])


class Engine:
    """One fglsgpu engine (one GPU)."""

    def __init__(self, n, wXL, wXR, t, x_b, variant="chol", precision="fp64", slices=0, device=0):
        self.L = lib()
        self.cfg = Config(n, wXL, wXR, t, x_b, VARIANT[variant], PRECISION[precision], slices, device, 0)
        self.n, self.wXL, self.wXR, self.t, self.x_b = n, wXL, wXR, t, x_b
        self.p = wXL + wXR
        self.variant = variant
        h = C.c_void_p()
        self._h = None
        self._check(self.L.fglsgpu_create(C.byref(self.cfg), C.byref(h)), None)
        self._h = h

    @property
    def handle(self):
        return self._h

    def _check(self, rc, h="self"):
        if rc != OK:
            hh = self._h if h == "self" else h
            msg = self.L.fglsgpu_last_error(hh).decode(errors="replace")
            raise FGLSError(rc, msg)

    @property
    def out_traits(self):
        return self.t if self.variant == "eigen" else 1

    def set_problem(self, Phi, XL, Y, h, sigma):
        self._keep = [_f64(Phi), _f64(XL), _f64(Y), _f64(h), _f64(sigma)]
        self._check(self.L.fglsgpu_set_problem(self._h, *[_ptr(a) for a in self._keep]))

    def select_trait(self, j):
        self._check(self.L.fglsgpu_select_trait(self._h, int(j)))

    def run_block(self, XR):
        XR = _f64(XR)
        x = XR.shape[1] // self.wXR
        nt, p = self.out_traits, self.p
        B = np.empty((nt, x, p))
        V = np.empty((nt, x, p, p))
        self._check(self.L.fglsgpu_run_block(self._h, _ptr(XR), x, _ptr(B), _ptr(V), x * p, x * p * p))
        return B, V.transpose(0, 1, 3, 2)

    def run_snps(self, XR, B=None, V=None):
        XR = _f64(XR)
        m = XR.shape[1] // self.wXR
        nt, p = self.out_traits, self.p
        B = np.empty((nt, m, p)) if B is None else B
        V = np.empty((nt, m, p, p)) if V is None else V
        self._check(self.L.fglsgpu_run_snps(self._h, _ptr(XR), m, _ptr(B), _ptr(V)))
        return B, V.transpose(0, 1, 3, 2)

    def run_snps_genotypes(self, G, packed=False, B=None, V=None):
        """Whole job from hard calls: G (m*wXR columns, n) uint8 in the XR
        column order (packed=False), or its 2-bit SNP-major .bed body
        (m*wXR columns, ceil(n/4) bytes; packed=True)."""
        G = np.ascontiguousarray(G, dtype=np.uint8)
        m = G.shape[0] // self.wXR
        nt, p = self.out_traits, self.p
        B = np.empty((nt, m, p)) if B is None else B
        V = np.empty((nt, m, p, p)) if V is None else V
        f = self.L.fglsgpu_run_snps_packed if packed else self.L.fglsgpu_run_snps_u8
        self._check(f(self._h, _ptr(G), m, _ptr(B), _ptr(V)))
        return B, V.transpose(0, 1, 3, 2)

    def run_snps_genotypes_ptr(self, g_ptr, m, b_ptr, v_ptr, packed=False):
        """Host pointers (e.g. pinned torch tensors): genotypes (bytes or
        2-bit packed), B, V."""
        f = self.L.fglsgpu_run_snps_packed if packed else self.L.fglsgpu_run_snps_u8
        self._check(f(self._h, C.c_void_p(g_ptr), int(m), C.c_void_p(b_ptr), C.c_void_p(v_ptr)))

    def run_snps_compact(self, XR):
        """B, SE, P each (traits, m, p)."""
        XR = _f64(XR)
        m = XR.shape[1] // self.wXR
        nt, p = self.out_traits, self.p
        B, SE, P = (np.empty((nt, m, p)) for _ in range(3))
        self._check(self.L.fglsgpu_run_snps_compact(self._h, _ptr(XR), m, _ptr(B), _ptr(SE), _ptr(P)))
        return B, SE, P

    def run_snps_ptr(self, xr_ptr, m, b_ptr, v_ptr):
        """Host pointers (e.g. pinned torch tensors): XR, B, V."""
        self._check(self.L.fglsgpu_run_snps(self._h, C.c_void_p(xr_ptr), int(m), C.c_void_p(b_ptr),
                                            C.c_void_p(v_ptr)))

    def run_block_device(self, xr_ptr, x, b_ptr, v_ptr, bstride, vstride, u8=False, packed=False):
        f = (self.L.fglsgpu_run_block_device_packed if packed else
             self.L.fglsgpu_run_block_device_u8 if u8 else self.L.fglsgpu_run_block_device)
        self._check(f(self._h, C.c_void_p(xr_ptr), int(x), C.c_void_p(b_ptr), C.c_void_p(v_ptr),
                      int(bstride), int(vstride)))

    def split_params(self):
        """(slices in use, probe beta error of the autotuned choice or -1)."""
        sl, err = C.c_int(), C.c_double()
        self._check(self.L.fglsgpu_split_params(self._h, C.byref(sl), C.byref(err)))
        return sl.value, err.value

    def quad_digits(self):
        """Base-32 digits a side of the tensor-core quadratic Gram in use (0: off)."""
        d = C.c_int()
        self._check(self.L.fglsgpu_quad_digits(self._h, C.byref(d)))
        return d.value

    def set_wait_limit(self, ns=0):
        """Limit of one tcgen05 pipeline wait in ns (0: the 2 s default)."""
        self._check(self.L.fglsgpu_set_wait_limit(self._h, int(ns)))

    def set_precision(self, precision):
        self._check(self.L.fglsgpu_set_precision(self._h, PRECISION[precision]))

    def profile(self, enable=True):
        self._check(self.L.fglsgpu_profile(self._h, 1 if enable else 0))

    def profile_read(self):
        """{class: (milliseconds, sections)} of device time since profile()."""
        ms = np.zeros(len(PROF_CLASSES))
        cnt = np.zeros(len(PROF_CLASSES), dtype=np.int64)
        self._check(self.L.fglsgpu_profile_read(self._h, _ptr(ms), _ptr(cnt)))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(PROF_CLASSES)}

    def pvalues_device(self, b_ptr, v_ptr, x, bstride, vstride, p_ptr, pstride):
        self._check(self.L.fglsgpu_pvalues_device(self._h, C.c_void_p(b_ptr), C.c_void_p(v_ptr), int(x), int(bstride),
                                                  int(vstride), C.c_void_p(p_ptr), int(pstride)))

    def adjoint_reset(self):
        self._check(self.L.fglsgpu_adjoint_reset(self._h))

    def adjoint_block_device(self, xr_ptr, x, bbar_ptr, bbar_trait_stride):
        self._check(self.L.fglsgpu_adjoint_block_device(self._h, C.c_void_p(xr_ptr), int(x), C.c_void_p(bbar_ptr),
                                                        int(bbar_trait_stride)))

    def adjoint_read(self):
        """(dL/dh (t), dL/dsigma (t), dL/dY (n x t))"""
        dh, ds = np.empty(self.t), np.empty(self.t)
        dY = np.empty((self.n, self.t), order="F")
        self._check(self.L.fglsgpu_adjoint_read(self._h, _ptr(dh), _ptr(ds), _ptr(dY)))
        return dh, ds, dY

    def reml(self):
        """(loglik (t), dloglik/dh (t)) of the null model."""
        ll, dll = np.empty(self.t), np.empty(self.t)
        self._check(self.L.fglsgpu_reml(self._h, _ptr(ll), _ptr(dll)))
        return ll, dll

    def reml_fit(self, h_lo=0.0, h_hi=1.0 - 1e-5, grid=64):
        """REML estimates per trait: (h, sigma, profiled loglik, its h-gradient), each (t,)."""
        h, sg, ll, dll = (np.empty(self.t) for _ in range(4))
        self._check(self.L.fglsgpu_reml_fit(self._h, float(h_lo), float(h_hi), int(grid), _ptr(h), _ptr(sg),
                                            _ptr(ll), _ptr(dll)))
        return h, sg, ll, dll

    def set_hsigma(self, h, sigma):
        h, sigma = _f64(h), _f64(sigma)
        self._keep_hs = [h, sigma]
        self._check(self.L.fglsgpu_set_hsigma(self._h, _ptr(h), _ptr(sigma)))

    def sync(self):
        self._check(self.L.fglsgpu_sync(self._h))

    def res_sigma(self):
        out = np.empty(self.out_traits)
        self._check(self.L.fglsgpu_get_res_sigma(self._h, _ptr(out)))
        return out

    def eigen(self):
        W = np.empty(self.n)
        Z = np.empty((self.n, self.n), order="F")
        self._check(self.L.fglsgpu_get_eigen(self._h, _ptr(W), _ptr(Z)))
        return W, Z

    def stream(self):
        return self.L.fglsgpu_stream(self._h)

    def close(self):
        if self._h is not None:
            self.L.fglsgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """Batched uneven cohorts (fglsgpu_batch_*), chol variant, wXR = 1.

    ``cohorts``: list of dicts with Phi (n x n), XL (n x wXL), Y (n x t), h, sigma
    (numpy, natural orientation).  ``step`` takes per-cohort device pointers."""

    def __init__(self, cohorts, x_b=0, slices=0, device=0, use_graph=True, genotypes_u8=True, tol=0.0, tile_rows=0):
        self.L = lib()
        self._keep = []
        descs = (CohortDesc * len(cohorts))()
        self.dims = []
        for k, c in enumerate(cohorts):
            Phi, XL = _f64(c["Phi"]), _f64(c["XL"])
            Y = _f64(c["Y"])
            h = np.ascontiguousarray(c["h"], dtype=np.float64)
            s = np.ascontiguousarray(c["sigma"], dtype=np.float64)
            self._keep += [Phi, XL, Y, h, s]
            n, wXL = XL.shape
            t = Y.shape[1]
            descs[k] = CohortDesc(n, wXL, t, Phi.ctypes.data, XL.ctypes.data, Y.ctypes.data, h.ctypes.data,
                                  s.ctypes.data)
            self.dims.append((n, wXL + 1, t))
        self.cfg = BatchConfig(int(x_b), int(slices), int(device), int(bool(use_graph)), int(bool(genotypes_u8)),
                               int(tile_rows), float(tol))
        h = C.c_void_p()
        rc = self.L.fglsgpu_batch_create(descs, len(cohorts), C.byref(self.cfg), C.byref(h))
        self._keep = None
        if rc:
            raise FGLSError(rc, self.L.fglsgpu_batch_last_error(None).decode())
        self._h = h

    def _check(self, rc):
        if rc:
            raise FGLSError(rc, self.L.fglsgpu_batch_last_error(self._h).decode())

    def params(self):
        xb, S, e = C.c_int(), C.c_int(), C.c_double()
        self._check(self.L.fglsgpu_batch_params(self._h, C.byref(xb), C.byref(S), C.byref(e)))
        return xb.value, S.value, e.value

    def tile(self):
        """(rows, cols) of the grouped split GEMM's output tile."""
        r, c = C.c_int(), C.c_int()
        self._check(self.L.fglsgpu_batch_tile(self._h, C.byref(r), C.byref(c)))
        return r.value, c.value

    def step(self, x_ptrs, xs, b_ptrs, v_ptrs, snp_base=None):
        k = len(self.dims)
        X = (C.c_void_p * k)(*x_ptrs)
        xs = (C.c_int * k)(*xs)
        B = (C.c_void_p * k)(*b_ptrs)
        V = (C.c_void_p * k)(*v_ptrs)
        base = None if snp_base is None else (C.c_longlong * k)(*snp_base)
        self._check(self.L.fglsgpu_batch_step(self._h, X, xs, B, V, base))

    def sync(self):
        self._check(self.L.fglsgpu_batch_sync(self._h))

    def stream(self):
        return self.L.fglsgpu_batch_stream(self._h)

    def profile(self, enable=True):
        self._check(self.L.fglsgpu_batch_profile(self._h, int(bool(enable))))

    def profile_read(self):
        """{stage: summed ms} over the profiled steps, and the step count."""
        ms = np.zeros(4)
        n = C.c_longlong()
        self._check(self.L.fglsgpu_batch_profile_read(self._h, _ptr(ms), C.byref(n)))
        return dict(zip(("genotypes", "split_gemm", "selfgram", "solve"), ms.tolist())), n.value

    def close(self):
        if getattr(self, "_h", None):
            self.L.fglsgpu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def split_gemm_selftest(A, X, slices):
    """C = A @ X (A M x K FP64, X K x N integer genotypes) through the
    split-precision tensor-core GEMM."""
    A = np.ascontiguousarray(A, dtype=np.float64)          # row-major M x K
    X = np.asfortranarray(X, dtype=np.float64)             # column-major K x N
    M, K = A.shape
    N = X.shape[1]
    C = np.empty((M, N), order="F")
    rc = lib().fglsgpu_selftest_split_gemm(M, K, N, slices, _ptr(A), _ptr(X), _ptr(C))
    if rc != OK:
        raise FGLSError(rc, "split GEMM self-test failed")
    return C


def launch_count() -> int:
    return int(lib().fglsgpu_launch_count(None))


def _dropin(name, n, p, m, t, wXL, wXR, x_b, y_b, num_threads, Phi_path, h2_path, sigma2_path,
            XL_path, XR_path, Y_path, B_path, V_path, env=None):
    """Calls the C entry point in a child process (it exits on error, like the
    reference); raises FGLSError with the "[Error]: ..." text on failure."""
    lib()  # fail loudly if missing
    code = (
        "import ctypes,sys\n"
        f"L=ctypes.CDLL({LIB_PATH!r})\n"
        "a=[int(x) for x in sys.argv[1:10]]+[s.encode() for s in sys.argv[10:]]\n"
        f"sys.exit(L.{name}(*[ctypes.c_int(v) if isinstance(v,int) else ctypes.c_char_p(v) for v in a]))\n"
    )
    args = [str(v) for v in (n, p, m, t, wXL, wXR, x_b, y_b, num_threads)] + [
        Phi_path, h2_path, sigma2_path, XL_path, XR_path, Y_path, B_path, V_path]
    e = dict(os.environ)
    if env:
        e.update(env)
    r = subprocess.run([sys.executable, "-c", code] + args, capture_output=True, text=True, env=e)
    if r.returncode != 0:
        msg = (r.stderr or r.stdout).strip().splitlines()
        raise FGLSError(r.returncode, msg[-1] if msg else f"{name} exited {r.returncode}")
    return 0


def fgls_chol(*args, **kw):
    return _dropin("fgls_chol", *args, **kw)


def fgls_eigen(*args, **kw):
    return _dropin("fgls_eigen", *args, **kw)


def fgls_chol_gpu(*args, **kw):
    return _dropin("fgls_chol_gpu", *args, **kw)
