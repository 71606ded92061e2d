"""Run the reference's own CPU driver (oracle/_ref/driver.x, built from the
reference sources by oracle/build_ref.sh).  TEST INFRASTRUCTURE ONLY.

The driver reads ``n p m t wXL x_b y_b threads`` on stdin and the files
``{Phi,H,Sig,XL,XR,Y}.in`` from a directory, writes ``B.out``/``V.out`` there
and prints the mean milliseconds per repetition (src/driver.c:35-100).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
DRIVER = os.path.join(HERE, "_ref", "driver.x")


def reference_root() -> str:
    """Root of the reference checkout whose sources build_ref.sh compiles:
    $FGLS_REFERENCE_ROOT, else the default that build_ref.sh names."""
    env = os.environ.get("FGLS_REFERENCE_ROOT")
    if env:
        return env
    with open(os.path.join(HERE, "build_ref.sh")) as f:
        for line in f:
            if line.startswith("DEFAULT_REF="):
                return line.split("=", 1)[1].strip().strip('"')
    return ""


def available() -> bool:
    return os.path.exists(DRIVER)


def run(variant: str, d: str, n: int, p: int, m: int, t: int, wXL: int, x_b: int,
        y_b: int = 1, threads: int = 1, nrep: int = 1, blas_threads: int | None = None,
        timeout: float = 600.0) -> float:
    """Runs ``driver.x <variant> <d> <nrep>``; returns the printed ms/rep."""
    if not available():
        raise FileNotFoundError(DRIVER)
    env = dict(os.environ)
    bt = str(blas_threads if blas_threads is not None else threads)
    env["OPENBLAS_NUM_THREADS"] = bt
    env["OMP_NUM_THREADS"] = str(threads)
    stdin = f"{n}\n{p}\n{m}\n{t}\n{wXL}\n{x_b}\n{y_b}\n{threads}\n"
    r = subprocess.run([DRIVER, variant, d, str(nrep)], input=stdin, capture_output=True,
                       text=True, env=env, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference driver failed ({r.returncode}): {r.stderr[-2000:]}")
    lines = [ln for ln in r.stdout.strip().splitlines() if ln.strip()]
    return float(lines[-1])
