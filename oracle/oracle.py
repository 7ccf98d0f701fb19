"""ctypes front end of the CPU oracle and of the reference-kernel runner.

TEST AND BASELINE INFRASTRUCTURE ONLY: imported by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline and reference arms,
always as the checker, never as the product. See ncorr_oracle.cpp for the
reference lines each function restates and for the parity status.
"""
from __future__ import annotations

import ctypes
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "_build" / "libncorr_oracle.so"
RUNNER = HERE / "_build" / "libref_runner.so"
REF_CUBIN = HERE / "_ref" / "reference_device.cubin"

# Contraction of the reference's sqrSep under nvcc (pattern numbering of
# ncorr_oracle.cpp): fma(dz, dz, fma(dx, dx, dy*dy)). Pinned against the
# reference kernel by tests/test_gpu_reference.py::test_fma_pattern and, on
# CPU, by the recorded fma_probe fixture in tests/golden/.
FMA_PATTERN = 2

_D = ctypes.POINTER(ctypes.c_double)
_lib = None
_runner = None


def build(runner: bool = False) -> None:
    targets = ["oracle"] + (["runner"] if runner else [])
    subprocess.run(["make", "-s", "-C", str(HERE), *targets], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = ctypes.CDLL(str(LIB))
        L.oracle_count_threeD.restype = ctypes.c_int
        L.oracle_count_threeD.argtypes = [_D, _D, ctypes.c_int, ctypes.c_int, _D, ctypes.c_long, _D,
                                          ctypes.c_long, _D, ctypes.c_long, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, _D]
        L.oracle_sqr_sep.restype = ctypes.c_double
        L.oracle_sqr_sep.argtypes = [_D, _D, ctypes.c_int]
        L.oracle_triangle_index.restype = ctypes.c_int
        L.oracle_triangle_index.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, _D,
                                            ctypes.c_int]
        L.oracle_n_out_threeD.restype = ctypes.c_long
        L.oracle_n_out_threeD.argtypes = [_D, ctypes.c_int]
        L.oracle_compact_threeD.restype = ctypes.c_long
        L.oracle_compact_threeD.argtypes = [_D, ctypes.c_int, _D, _D, _D]
        L.oracle_logspace.restype = None
        L.oracle_logspace.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _D]
        L.oracle_prep_cat_survey.restype = None
        L.oracle_prep_cat_survey.argtypes = [_D, ctypes.c_long, _D, ctypes.c_long, _D, _D]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _cat(p) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(p, dtype=np.float64))
    assert a.ndim == 2 and a.shape[1] == 4
    return a


def count_threeD(box, edges, p1, p2=None, p3=None, survey=False, fma_pattern=FMA_PATTERN, nthreads=0,
                 literal=False) -> np.ndarray:
    """triCountsAll_ (nb^3 doubles) of calculateD1D2D3(p1, p2, p3).

    p2/p3 default to p1; passing the same array object marks catalogues
    identical (the oracle then gathers one list). literal=True runs the
    reference's own loop nest, otherwise the equivalent neighbour-list form.
    """
    a1 = _cat(p1)
    a2 = a1 if p2 is None or p2 is p1 else _cat(p2)
    if p3 is None or p3 is p2 or (p2 is None and p3 is p1):
        a3 = a2
    elif p3 is p1:
        a3 = a1
    else:
        a3 = _cat(p3)
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    nb = len(e) - 1
    out = np.zeros(nb ** 3)
    rc = lib().oracle_count_threeD(_p(b), _p(e), len(e), int(survey), _p(a1), a1.shape[0], _p(a2),
                                   a2.shape[0], _p(a3), a3.shape[0], int(fma_pattern), int(nthreads),
                                   0 if literal else 1, _p(out))
    if rc != 0:
        raise ValueError(f"oracle_count_threeD failed with {rc}")
    return out


def compact(edges, hist_all):
    """(counts_out, bins_out) of prepTriCountsOutThreeD (source/cudaNcorr.cu:72-86)."""
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    h = np.ascontiguousarray(np.asarray(hist_all, dtype=np.float64))
    n = lib().oracle_n_out_threeD(_p(e), len(e))
    c = np.zeros(n)
    b = np.zeros((n, 3))
    lib().oracle_compact_threeD(_p(e), len(e), _p(h), _p(c), _p(b))
    return c, b


def sqr_sep(a, b, pattern=FMA_PATTERN) -> float:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(4))
    b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(4))
    return lib().oracle_sqr_sep(_p(a), _p(b), int(pattern))


def triangle_index(r1, r2, r3, edges) -> int:
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    return lib().oracle_triangle_index(float(r1), float(r2), float(r3), _p(e), len(e))


def logspace(start, end, n) -> np.ndarray:
    out = np.zeros(n)
    lib().oracle_logspace(float(start), float(end), int(n), _p(out))
    return out


def prep_cat_survey(c1: np.ndarray, c2=None):
    box = np.zeros(3)
    ori = np.zeros(3)
    lib().oracle_prep_cat_survey(_p(c1), c1.shape[0], _p(c2) if c2 is not None else None,
                                 0 if c2 is None else c2.shape[0], _p(box), _p(ori))
    return box, ori


# ---------------------------------------------------------------- reference kernel runner
def runner():
    """The reference's own threeD kernels (oracle/_ref cubin) behind a restated
    host flow (oracle/ref_runner.cu). Needs a GPU and the cubin."""
    global _runner
    if _runner is None:
        if not RUNNER.exists():
            build(runner=True)
        if not REF_CUBIN.exists():
            raise FileNotFoundError(f"{REF_CUBIN} is missing (build it where the reference sources are: make -C oracle ref)")
        R = ctypes.CDLL(str(RUNNER))
        R.ref_runner_last_error.restype = ctypes.c_char_p
        R.ref_runner_load.restype = ctypes.c_int
        R.ref_runner_load.argtypes = [ctypes.c_char_p]
        R.ref_runner_count.restype = ctypes.c_int
        R.ref_runner_count.argtypes = [_D, _D, ctypes.c_int, ctypes.c_int, _D, _D, ctypes.c_long, _D,
                                       ctypes.c_long, _D, ctypes.c_long, _D, _D, _D]
        if R.ref_runner_load(str(REF_CUBIN).encode()) != 0:
            raise RuntimeError(R.ref_runner_last_error().decode())
        _runner = R
    return _runner


def reference_count(box, edges, p1, p2=None, p3=None, survey=False, ori=(0.0, 0.0, 0.0)):
    """Runs the reference kernel; returns (hist_all, kernel_ms, total_ms)."""
    R = runner()
    a1 = _cat(p1)
    a2 = a1 if p2 is None else _cat(p2)
    a3 = a2 if p3 is None else _cat(p3)
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    o = np.ascontiguousarray(np.asarray(ori, dtype=np.float64).reshape(3))
    nb = len(e) - 1
    out = np.zeros(nb ** 3)
    kms = ctypes.c_double(0)
    tms = ctypes.c_double(0)
    rc = R.ref_runner_count(_p(b), _p(e), len(e), int(survey), _p(o), _p(a1), a1.shape[0], _p(a2),
                            a2.shape[0], _p(a3), a3.shape[0], _p(out), ctypes.byref(kms), ctypes.byref(tms))
    if rc != 0:
        raise RuntimeError(R.ref_runner_last_error().decode())
    return out, kms.value, tms.value
