"""C ABI checks that need no GPU: the library loads, exports every function
include/fgls_gb300.h declares, and rejects invalid configurations before it
touches a device."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fgls_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b((?:fgls|fglsgpu)_\w+)\s*\(", src)))


def test_header_declares_the_dropin_entry_points():
    names = declared_functions()
    for f in ("fgls_chol", "fgls_eigen", "fgls_chol_gpu"):
        assert f in names


def test_library_exports_every_declared_symbol():
    from fgls_gb300 import EXPORTS, lib
    L = lib()
    names = declared_functions()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the Python mirror binds exactly the functions the header declares
    assert set(EXPORTS) == set(names), sorted(set(EXPORTS) ^ set(names))
    assert L.fglsgpu_version() >= 10000


def test_dropin_signatures_match_reference_arity():
    """17 arguments: 9 ints then 8 paths (src/fgls_chol.h:4-10)."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    for f in ("fgls_chol", "fgls_eigen", "fgls_chol_gpu"):
        m = re.search(r"int\s+" + f + r"\s*\((.*?)\);", src, flags=re.S)
        args = [a.strip() for a in m.group(1).split(",")]
        assert len(args) == 17
        assert all(a.startswith("int ") for a in args[:9])
        assert all(a.startswith("char *") for a in args[9:])


@pytest.mark.parametrize("cfg", [
    dict(n=0, wXL=3, wXR=1, t=1, x_b=8),
    dict(n=100, wXL=3, wXR=1, t=0, x_b=8),
    dict(n=100, wXL=7, wXR=2, t=1, x_b=8),    # p = 9 > 8
    dict(n=100, wXL=2, wXR=5, t=1, x_b=8),    # wXR > 4
    dict(n=3, wXL=3, wXR=1, t=1, x_b=8),      # n <= wXL
])
def test_create_rejects_invalid_dimensions(cfg):
    from fgls_gb300.engine import Config, EINVAL, lib
    L = lib()
    c = Config(cfg["n"], cfg["wXL"], cfg["wXR"], cfg["t"], cfg["x_b"], 0, 0, 0, 0, 0)
    h = C.c_void_p()
    assert L.fglsgpu_create(C.byref(c), C.byref(h)) == EINVAL
    assert L.fglsgpu_last_error(None)


def test_null_engine_calls_fail_cleanly():
    from fgls_gb300.engine import EINVAL, lib
    L = lib()
    assert L.fglsgpu_select_trait(None, 0) == EINVAL
    assert L.fglsgpu_sync(None) == EINVAL
    assert L.fglsgpu_destroy(None) == 0


def test_engine_without_gpu_fails_loudly(has_gpu):
    if has_gpu:
        pytest.skip("a GPU is present")
    from fgls_gb300 import Engine, FGLSError
    with pytest.raises(FGLSError, match="no CUDA device"):
        Engine(100, 3, 1, 1, 16)


def test_pack_2bit_layout():
    """The packer follows the 2-bit SNP-major layout the device unpacker reads."""
    import numpy as np
    from fgls_gb300 import datagen
    rng = np.random.default_rng(3)
    X = rng.integers(-1, 3, size=(5, 13))
    P = datagen.pack_2bit(X)
    assert P.shape == (5, 4) and P.dtype == np.uint8
    dec = {0: 2, 2: 1, 3: 0, 1: -1}
    for c in range(5):
        for k in range(13):
            code = (int(P[c, k // 4]) >> (2 * (k % 4))) & 3
            assert dec[code] == X[c, k]
