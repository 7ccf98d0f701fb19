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
# Contractions of the rppi helpers under nvcc: sqrRpBox's dx*dx + dy*dy as
# fma(dx, dx, dy*dy) (RP_PATTERN numbering of ncorr_oracle.cpp) and
# dotProduct_d3 as fma(a.z, b.z, fma(a.x, b.x, a.y*b.y)) (sqrSep numbering).
# Pinned against the reference's rppi kernels by tests/test_gpu_rppi.py and,
# on CPU, by the recorded rppi fixtures in tests/golden/.
RP_PATTERN = 2
DOT_PATTERN = 2

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
        L.oracle_count_rppi.restype = ctypes.c_int
        L.oracle_count_rppi.argtypes = [_D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D, ctypes.c_long,
                                        _D, ctypes.c_long, _D, ctypes.c_long, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D]
        L.oracle_rppi_index.restype = ctypes.c_long
        L.oracle_rppi_index.argtypes = [ctypes.c_double] * 6 + [_D, ctypes.c_int, ctypes.c_int]
        L.oracle_rppi_grid.restype = ctypes.c_int
        L.oracle_rppi_grid.argtypes = [_D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D,
                                       ctypes.POINTER(ctypes.c_int)]
        L.oracle_survey_rppi_sides.restype = None
        L.oracle_survey_rppi_sides.argtypes = [_D, _D, _D, _D, ctypes.c_int, ctypes.c_int, _D]
        L.oracle_sqr_rp.restype = ctypes.c_double
        L.oracle_sqr_rp.argtypes = [_D, _D, ctypes.c_int]
        L.oracle_compact_rppi.restype = ctypes.c_long
        L.oracle_compact_rppi.argtypes = [_D, ctypes.c_int, ctypes.c_int, _D, _D, _D, _D]
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


def _roles(p1, p2, p3):
    a1 = _cat(p1)
    a2 = a1 if p2 is None or p2 is p1 else _cat(p2)
    if p3 is None or p3 is p2 or (p2 is None and p3 is p1):
        a3 = a2
    elif p3 is p1:
        a3 = a1
    else:
        a3 = _cat(p3)
    return a1, a2, a3


def count_rppi(box, edges, num_pi_bins, p1, p2=None, p3=None, survey=False, ori=(0.0, 0.0, 0.0),
               fma_pattern=FMA_PATTERN, rp_pattern=RP_PATTERN, dot_pattern=DOT_PATTERN, nthreads=0,
               literal=False):
    """(triCountsAll_, overflow) of calculateD1D2D3 for the rppi bin type.

    triCountsAll_ has nb^3 * nPi^2 doubles; overflow is the weight the
    reference writes past its end (pi bin nPi from FP32 rounding). Same
    catalogue conventions as count_threeD."""
    a1, a2, a3 = _roles(p1, p2, p3)
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    o = np.ascontiguousarray(np.asarray(ori, dtype=np.float64).reshape(3))
    nb = len(e) - 1
    out = np.zeros(nb ** 3 * int(num_pi_bins) ** 2)
    ov = ctypes.c_double(0.0)
    rc = lib().oracle_count_rppi(_p(b), _p(e), len(e), int(num_pi_bins), int(survey), _p(o), _p(a1), a1.shape[0],
                                 _p(a2), a2.shape[0], _p(a3), a3.shape[0], int(fma_pattern), int(rp_pattern),
                                 int(dot_pattern), int(nthreads), 0 if literal else 1, _p(out), ctypes.byref(ov))
    if rc != 0:
        raise ValueError(f"oracle_count_rppi failed with {rc}")
    return out, ov.value


def rppi_index(rp1, rp2, rp3, pi1, pi2, pi3, edges, num_pi_bins) -> int:
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    return lib().oracle_rppi_index(float(rp1), float(rp2), float(rp3), float(pi1), float(pi2), float(pi3),
                                   _p(e), len(e), int(num_pi_bins))


def survey_rppi_sides(a, b, c, ori, dot_pattern=DOT_PATTERN, fma_pattern=FMA_PATTERN) -> np.ndarray:
    """(rp1, rp2, rp3, pi1, pi2, pi3) of countTrianglesRppiSurvey for one triangle."""
    v = [np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(4)) for x in (a, b, c)]
    o = np.ascontiguousarray(np.asarray(ori, dtype=np.float64).reshape(3))
    out = np.zeros(6)
    lib().oracle_survey_rppi_sides(_p(v[0]), _p(v[1]), _p(v[2]), _p(o), int(fma_pattern), int(dot_pattern),
                                   _p(out))
    return out


def sqr_rp(a, b, pattern=RP_PATTERN) -> float:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(4))
    b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(4))
    return lib().oracle_sqr_rp(_p(a), _p(b), int(pattern))


def rppi_grid(box, edges, num_pi_bins, survey=False):
    """(cell[3], nc[3]) of the rppi constructor."""
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    cell = np.zeros(3)
    nc = (ctypes.c_int * 3)()
    rc = lib().oracle_rppi_grid(_p(b), _p(e), len(e), int(num_pi_bins), int(survey), _p(cell), nc)
    if rc != 0:
        raise ValueError(f"oracle_rppi_grid failed with {rc}")
    return cell, np.array(list(nc))


def compact_rppi(edges, num_pi_bins, hist_all):
    """(counts_out, bins_out, pi_out) of prepTriCountsOutRppi (source/cudaNcorr.cu:88-105)."""
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    h = np.ascontiguousarray(np.asarray(hist_all, dtype=np.float64))
    n = lib().oracle_compact_rppi(_p(e), len(e), int(num_pi_bins), _p(h), None, None, None)
    c = np.zeros(n)
    b = np.zeros((n, 3))
    pi = np.zeros((n, 2))
    lib().oracle_compact_rppi(_p(e), len(e), int(num_pi_bins), _p(h), _p(c), _p(b), _p(pi))
    return c, b, pi


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
        R.ref_runner_count_rppi.restype = ctypes.c_int
        R.ref_runner_count_rppi.argtypes = [_D, _D, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, _D, ctypes.c_long,
                                            _D, ctypes.c_long, _D, ctypes.c_long, _D, _D, _D, _D]
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


def reference_count_rppi(box, edges, num_pi_bins, p1, p2=None, p3=None, survey=False, ori=(0.0, 0.0, 0.0)):
    """Runs the reference's rppi kernel; returns (hist_all, overflow, kernel_ms, total_ms)."""
    R = runner()
    a1 = _cat(p1)
    a2 = a1 if p2 is None else _cat(p2)
    a3 = a2 if p3 is None else _cat(p3)
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    o = np.ascontiguousarray(np.asarray(ori, dtype=np.float64).reshape(3))
    nb = len(e) - 1
    out = np.zeros(nb ** 3 * int(num_pi_bins) ** 2)
    ov = ctypes.c_double(0)
    kms = ctypes.c_double(0)
    tms = ctypes.c_double(0)
    rc = R.ref_runner_count_rppi(_p(b), _p(e), len(e), int(num_pi_bins), int(survey), _p(o), _p(a1), a1.shape[0],
                                 _p(a2), a2.shape[0], _p(a3), a3.shape[0], _p(out), ctypes.byref(ov),
                                 ctypes.byref(kms), ctypes.byref(tms))
    if rc != 0:
        raise RuntimeError(R.ref_runner_last_error().decode())
    return out, ov.value, kms.value, tms.value


# ---------------------------------------------------------------- reference-kernel cost model
def reference_cells(p, box, rmax):
    """The reference's cell index of every point, int(x / r_max) with the
    == nc clamp (source/cudaNcorr.cu:50-58); returns (cells, nc)."""
    box = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
    nc = np.ceil(box / rmax).astype(np.int64)
    c = (np.asarray(p)[:, :3] / rmax).astype(np.int64)
    for d in range(3):
        c[c[:, d] == nc[d], d] = nc[d] - 1
    return c, nc


def reference_n27(anchor_cells, p, box, rmax, survey):
    """Points of catalogue p in the 27 cells around each anchor cell (wrapped
    once in a box, clipped in a survey), as the reference's loops visit them."""
    c, nc = reference_cells(p, box, rmax)
    cnt = np.zeros(tuple(nc), np.int64)
    np.add.at(cnt, (c[:, 0], c[:, 1], c[:, 2]), 1)
    s = np.zeros_like(cnt)
    if survey:
        pad = np.pad(cnt, 1)
        for dx in range(3):
            for dy in range(3):
                for dz in range(3):
                    s += pad[dx:dx + nc[0], dy:dy + nc[1], dz:dz + nc[2]]
    else:
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    s += np.roll(cnt, (dx, dy, dz), axis=(0, 1, 2))
    a = anchor_cells
    return s[a[:, 0], a[:, 1], a[:, 2]]


def reference_anchor_cost(p1, p2, p3, box, rmax, survey=False):
    """Estimated pair evaluations of the reference kernel's thread for each
    anchor of p1 (source/device.cu:270-312: for every p2 point in the 27
    cells in range, every p3 point in the 27 cells): (1 + k2) * n27(p3), with
    the in-range count k2 ~ 0.155 n27(p2) (a ball's share of 27 cells).
    Returns (cost, face) where face marks anchors in the first or last cell
    layer of the grid."""
    a, nc = reference_cells(p1, box, rmax)
    cost = (1.0 + 0.155 * reference_n27(a, p2, box, rmax, survey)) * reference_n27(a, p3, box, rmax, survey)
    face = ((a == 0) | (a == nc - 1)).any(axis=1)
    return cost, face
