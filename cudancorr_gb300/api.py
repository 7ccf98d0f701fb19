"""Python mirror of cudaNcorr's `ncorr` class over the engine's C ABI.

The reference's public surface is a C++ class (include/cudaNcorr.hpp:10-68 of
cudaNcorr); this module keeps its names and argument meaning:

    corr = ncorr(box, 0, bins, isSurvey, ori)      # ncorr::ncorr (threeD)
    corr = ncorr(box, 1, bins, numMinorBins, isSurvey, ori)   # (rppi)
    corr.calculateD1D2D3(p1, p2, p3)               # N x 4 (x, y, z, w) arrays
    corr.getTriBinsOut(); corr.getTriCountsOut(); corr.getPiBinsOut()

Errors raise NcorrError, a RuntimeError, where the reference throws
std::runtime_error. Arrays are numpy float64 (host) or CUDA tensors of
float64 (device-resident inputs, torch only as a container). There is no CPU
path: the shared library must be built (cudancorr_gb300.build) and a CUDA
device present.
"""
from __future__ import annotations

import ctypes
import pathlib
from typing import Optional, Sequence

import numpy as np

from . import build as _build

NCORR_OK = 0
NCORR_ERR_INVALID_ARGUMENT = 1
NCORR_ERR_NOT_IMPLEMENTED = 2
NCORR_ERR_CUDA = 3
NCORR_ERR_OUT_OF_GRID = 4
NCORR_ERR_CAPACITY = 5
NCORR_ERR_NO_DEVICE = 6

threeD, rppi, smu = 0, 1, 2  # ncorr::binType (include/cudaNcorr.hpp:12)

# Every symbol the C header declares (include/ncorr_gb300.h).
EXPORTS = (
    "ncorr_create", "ncorr_create_rppi", "ncorr_destroy", "ncorr_calculate_d1d2d3",
    "ncorr_calculate_d1d2d3_device", "ncorr_num_out", "ncorr_num_bins", "ncorr_num_pi_bins",
    "ncorr_get_tri_bins_out",
    "ncorr_get_pi_bins_out", "ncorr_get_tri_counts_out", "ncorr_get_tri_counts_all",
    "ncorr_get_stats", "ncorr_last_error", "survey_prep_cat", "survey_prep_cat2",
    "survey_convert_coordinates", "ncorr_logspace", "ncorr_count_noalloc",
    "ncorr_write_three_d", "ncorr_write_rppi", "ncorr_read_catalog_txt", "ncorr_random_catalog",
    "ncorr_set_schedule", "ncorr_set_tuning", "ncorr_set_record_work", "ncorr_num_cells",
    "ncorr_get_cell_work", "ncorr_sched_create", "ncorr_sched_destroy", "ncorr_sched_num_params",
    "ncorr_sched_get_params", "ncorr_sched_set_params", "ncorr_sched_predict", "ncorr_sched_gradient",
    "ncorr_sched_set_precision",
    "ncorr_sched_train", "ncorr_batch_create", "ncorr_batch_run", "ncorr_batch_get_counts_all",
    "ncorr_batch_get_stats", "ncorr_batch_destroy",
)

# Work-queue schedules (ncorr_set_schedule).
SCHED_DYNAMIC, SCHED_STATIC, SCHED_LEARNED = 0, 1, 2
MLP_FP32, MLP_BF16 = 0, 1


class NcorrError(RuntimeError):
    """Raised where the reference throws std::runtime_error."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class NcorrStats(ctypes.Structure):
    _fields_ = [
        ("ms_grid", ctypes.c_double), ("ms_count", ctypes.c_double), ("ms_fold", ctypes.c_double),
        ("ms_total", ctypes.c_double), ("n_anchors", ctypes.c_uint64),
        ("n_pair_evals", ctypes.c_uint64), ("n_pairs", ctypes.c_uint64),
        ("n_exact_pairs", ctypes.c_uint64), ("n_exact_tris", ctypes.c_uint64),
        ("triangles", ctypes.c_uint64), ("n_flagged_rows", ctypes.c_uint64), ("n_queued", ctypes.c_uint64),
        ("weighted", ctypes.c_int), ("symmetric", ctypes.c_int),
        ("grid_ctas", ctypes.c_int), ("list_capacity", ctypes.c_int), ("overflow", ctypes.c_double),
        ("tail_idle", ctypes.c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class NcorrBatchStats(ctypes.Structure):
    _fields_ = [
        ("ms_plan", ctypes.c_double), ("ms_autotune", ctypes.c_double), ("ms_run", ctypes.c_double),
        ("ms_count", ctypes.c_double), ("n_work", ctypes.c_uint64), ("n_pairs", ctypes.c_uint64),
        ("n_pair_evals", ctypes.c_uint64),
        ("triangles", ctypes.c_uint64), ("n_items", ctypes.c_int), ("n_catalogues", ctypes.c_int),
        ("sub_j", ctypes.c_int), ("hist_copies", ctypes.c_int), ("grid_ctas", ctypes.c_int),
        ("weighted", ctypes.c_int), ("graph_nodes", ctypes.c_int),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_LIB: Optional[ctypes.CDLL] = None
_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)


def library_path() -> pathlib.Path:
    """The engine library: NCORR_LIBRARY when set, else the in-tree build."""
    import os
    override = os.environ.get("NCORR_LIBRARY")
    return pathlib.Path(override) if override else _build.library_path()


def load_library() -> ctypes.CDLL:
    """Loads libcudancorr_gb300.so; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        raise NcorrError(NCORR_ERR_NO_DEVICE,
                         f"{path} is missing: build it with `python -m cudancorr_gb300.build`")
    lib = ctypes.CDLL(str(path))
    i64, i32, vp = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
    hp = ctypes.POINTER(vp)
    sig = {
        "ncorr_create": (i32, [_D, i32, _D, i32, i32, _D, hp]),
        "ncorr_create_rppi": (i32, [_D, i32, _D, i32, i32, i32, _D, hp]),
        "ncorr_destroy": (None, [vp]),
        "ncorr_calculate_d1d2d3": (i32, [vp, _D, i64, _D, i64, _D, i64]),
        "ncorr_calculate_d1d2d3_device": (i32, [vp, vp, i64, vp, i64, vp, i64, vp]),
        "ncorr_num_out": (i64, [vp]),
        "ncorr_num_bins": (i32, [vp]),
        "ncorr_num_pi_bins": (i32, [vp]),
        "ncorr_get_tri_bins_out": (i32, [vp, _D, i64]),
        "ncorr_get_pi_bins_out": (i32, [vp, _D, i64, ctypes.POINTER(i64)]),
        "ncorr_get_tri_counts_out": (i32, [vp, _D, i64]),
        "ncorr_get_tri_counts_all": (i32, [vp, _D, i64]),
        "ncorr_get_stats": (i32, [vp, ctypes.POINTER(NcorrStats)]),
        "ncorr_last_error": (ctypes.c_char_p, []),
        "survey_prep_cat": (i32, [_D, i64, _D, _D]),
        "survey_prep_cat2": (i32, [_D, i64, _D, i64, _D, _D]),
        "survey_convert_coordinates": (i32, [_D, _D, i64, _D]),
        "ncorr_logspace": (i32, [ctypes.c_double, ctypes.c_double, i32, _D]),
        "ncorr_write_three_d": (i32, [ctypes.c_char_p, _D, _D, i64]),
        "ncorr_write_rppi": (i32, [ctypes.c_char_p, _D, _D, _D, i64]),
        "ncorr_read_catalog_txt": (i32, [ctypes.c_char_p, _D, ctypes.POINTER(i32), _D, i64, ctypes.POINTER(i64)]),
        "ncorr_random_catalog": (i32, [i64, _D, ctypes.c_uint64, _D]),
        "ncorr_count_noalloc": (i32, [_D, _D, i32, i32, vp, i64, vp, i64, vp, i64, vp, vp]),
        "ncorr_set_schedule": (i32, [vp, i32, vp]),
        "ncorr_set_tuning": (i32, [vp, i32, i32]),
        "ncorr_set_record_work": (i32, [vp, i32]),
        "ncorr_num_cells": (i64, [vp]),
        "ncorr_get_cell_work": (i32, [vp, _F, _D, i64]),
        "ncorr_sched_create": (i32, [ctypes.c_uint64, hp]),
        "ncorr_sched_destroy": (None, [vp]),
        "ncorr_sched_num_params": (i32, []),
        "ncorr_sched_get_params": (i32, [vp, _F, i64]),
        "ncorr_sched_set_params": (i32, [vp, _F, i64]),
        "ncorr_sched_predict": (i32, [vp, _F, i64, _F]),
        "ncorr_sched_set_precision": (i32, [vp, i32]),
        "ncorr_sched_gradient": (i32, [vp, _F, _F, i64, _F, _F]),
        "ncorr_sched_train": (i32, [vp, _F, _F, i64, i32, i32, ctypes.c_float, ctypes.c_uint64, _F]),
        "ncorr_batch_create": (i32, [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(i64), ctypes.POINTER(vp),
                                     ctypes.POINTER(i64), ctypes.POINTER(vp), ctypes.POINTER(i64), i32, i32,
                                     hp]),
        "ncorr_batch_run": (i32, [vp, vp]),
        "ncorr_batch_get_counts_all": (i32, [vp, i32, _D, i64]),
        "ncorr_batch_get_stats": (i32, [vp, ctypes.POINTER(NcorrBatchStats)]),
        "ncorr_batch_destroy": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _check(rc: int) -> None:
    if rc != NCORR_OK:
        msg = load_library().ncorr_last_error().decode(errors="replace")
        raise NcorrError(rc, msg)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _vec3(v: Sequence[float]) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(3))
    return a


def as_catalog(p) -> np.ndarray:
    """N x 4 float64 C-contiguous view/copy of a catalogue (x, y, z, w)."""
    a = np.asarray(p, dtype=np.float64)
    if a.ndim != 2 or a.shape[1] != 4:
        raise NcorrError(NCORR_ERR_INVALID_ARGUMENT, "catalogue must be an N x 4 array (x, y, z, w)")
    return np.ascontiguousarray(a)


class ncorr:
    """Triangle counter, the reference's `ncorr` class: threeD (r1, r2, r3)
    bins with ncorr(box, 0, bins, isSurvey, ori), or rppi (rp bins of all
    three sides, unit pi bins of the two shortest) with
    ncorr(box, 1, bins, numMinorBins, isSurvey, ori) (numMinorBins may also
    be given by keyword)."""

    def __init__(self, box, bin_type, bins, *args, isSurvey=None, ori=None, numMinorBins: Optional[int] = None):
        # The reference's two constructors (include/cudaNcorr.hpp:14-15):
        #   (box, bin_type, bins, isSurvey, ori)
        #   (box, bin_type, bins, numMinorBins, isSurvey, ori)
        if len(args) == 3:
            numMinorBins, isSurvey, ori = args
        elif len(args) <= 2:
            if len(args) >= 1:
                isSurvey = args[0]
            if len(args) == 2:
                ori = args[1]
        else:
            raise TypeError("ncorr(box, bin_type, bins, [numMinorBins,] isSurvey, ori)")
        isSurvey = False if isSurvey is None else isSurvey
        ori = (0.0, 0.0, 0.0) if ori is None else ori
        lib = load_library()
        self._h = ctypes.c_void_p()
        self._box = _vec3(box)
        self._ori = _vec3(ori)
        self._bins = np.ascontiguousarray(np.asarray(bins, dtype=np.float64))
        if numMinorBins is not None:
            rc = lib.ncorr_create_rppi(_dptr(self._box), int(bin_type), _dptr(self._bins),
                                       len(self._bins), int(numMinorBins), int(bool(isSurvey)),
                                       _dptr(self._ori), ctypes.byref(self._h))
        else:
            rc = lib.ncorr_create(_dptr(self._box), int(bin_type), _dptr(self._bins), len(self._bins),
                                  int(bool(isSurvey)), _dptr(self._ori), ctypes.byref(self._h))
        _check(rc)
        self._lib = lib
        self.isSurvey = bool(isSurvey)

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.ncorr_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def num_bins(self) -> int:
        return int(self._lib.ncorr_num_bins(self._h))

    @property
    def num_pi_bins(self) -> int:
        """numPiBins_ (rppi); 0 for threeD."""
        return int(self._lib.ncorr_num_pi_bins(self._h))

    @property
    def num_counts_all(self) -> int:
        npi = self.num_pi_bins
        return self.num_bins ** 3 * (npi * npi if npi else 1)

    def calculateD1D2D3(self, p1, p2, p3) -> None:
        """Counts triangles with p1 as anchors (source/cudaNcorr.cu:220-430).

        Host arrays go through the reference-facing C call (with its host to
        device copies); CUDA tensors go through the device-resident entry.
        Passing the same object for p2 and p3 (or all three) marks the
        catalogues identical.
        """
        if _is_cuda_tensor(p1):
            return self._calculate_device(p1, p2, p3)
        arrays = {}
        out = []
        for p in (p1, p2, p3):
            key = id(p)
            if key not in arrays:
                arrays[key] = as_catalog(p)
            out.append(arrays[key])
        a1, a2, a3 = out
        _check(self._lib.ncorr_calculate_d1d2d3(self._h, _dptr(a1), a1.shape[0], _dptr(a2),
                                                 a2.shape[0], _dptr(a3), a3.shape[0]))

    def _calculate_device(self, p1, p2, p3, stream=None) -> None:
        for t in (p1, p2, p3):
            if not _is_cuda_tensor(t) or t.dim() != 2 or t.shape[1] != 4 or not t.is_contiguous():
                raise NcorrError(NCORR_ERR_INVALID_ARGUMENT,
                                 "device catalogues must be contiguous N x 4 float64 CUDA tensors")
            if str(t.dtype) != "torch.float64":
                raise NcorrError(NCORR_ERR_INVALID_ARGUMENT, "device catalogues must be float64")
        s = ctypes.c_void_p(stream) if stream is not None else None
        _check(self._lib.ncorr_calculate_d1d2d3_device(
            self._h, ctypes.c_void_p(p1.data_ptr()), p1.shape[0], ctypes.c_void_p(p2.data_ptr()),
            p2.shape[0], ctypes.c_void_p(p3.data_ptr()), p3.shape[0], s))

    def getTriBinsOut(self) -> np.ndarray:
        """(n_out, 3) bin mids (source/cudaNcorr.cu:106-108)."""
        n = int(self._lib.ncorr_num_out(self._h))
        out = np.zeros((n, 3), dtype=np.float64)
        _check(self._lib.ncorr_get_tri_bins_out(self._h, _dptr(out), out.size))
        return out

    def getPiBinsOut(self) -> np.ndarray:
        """(n_out, 2) pi bins (l, m) for rppi; empty for threeD (source/cudaNcorr.cu:110-112)."""
        n = ctypes.c_int64(0)
        buf = np.zeros(1, dtype=np.float64)
        _check(self._lib.ncorr_get_pi_bins_out(self._h, _dptr(buf), 0, ctypes.byref(n))
               if self.num_pi_bins == 0 else NCORR_OK)
        if self.num_pi_bins == 0:
            return np.zeros((n.value, 2), dtype=np.float64)
        m = int(self._lib.ncorr_num_out(self._h))
        out = np.zeros((m, 2), dtype=np.float64)
        _check(self._lib.ncorr_get_pi_bins_out(self._h, _dptr(out), out.size, ctypes.byref(n)))
        return out

    def getTriCountsOut(self) -> np.ndarray:
        """Compacted counts of the last calculation (source/cudaNcorr.cu:114-116)."""
        n = int(self._lib.ncorr_num_out(self._h))
        out = np.zeros(n, dtype=np.float64)
        _check(self._lib.ncorr_get_tri_counts_out(self._h, _dptr(out), n))
        return out

    def getTriCountsAll(self) -> np.ndarray:
        """Full histogram (the reference's private triCountsAll_): nb^3
        entries, or nb^3 * numPiBins^2 for rppi."""
        out = np.zeros(self.num_counts_all, dtype=np.float64)
        _check(self._lib.ncorr_get_tri_counts_all(self._h, _dptr(out), out.size))
        return out

    def stats(self) -> dict:
        s = NcorrStats()
        _check(self._lib.ncorr_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    # -- scheduling (no counterpart in the reference; counts never depend on it)
    def set_schedule(self, mode: int, model: Optional["WorkModel"] = None) -> None:
        """SCHED_DYNAMIC (default), SCHED_STATIC, or SCHED_LEARNED with a WorkModel."""
        self._model = model  # the handle uses the model's parameters in later calls
        _check(self._lib.ncorr_set_schedule(self._h, int(mode), model._s if model is not None else None))

    def set_tuning(self, sub_j: int = 32, hist_copies: int = 1) -> None:
        _check(self._lib.ncorr_set_tuning(self._h, int(sub_j), int(hist_copies)))

    def set_record_work(self, on: bool = True) -> None:
        _check(self._lib.ncorr_set_record_work(self._h, int(bool(on))))

    def cell_work(self):
        """(features n_cells x 28 float32, candidate pairs per cell float64) of
        the last call made with set_record_work(True)."""
        n = int(self._lib.ncorr_num_cells(self._h))
        feats = np.zeros((n, 28), dtype=np.float32)
        work = np.zeros(n, dtype=np.float64)
        _check(self._lib.ncorr_get_cell_work(self._h, feats.ctypes.data_as(_F), _dptr(work), n))
        return feats, work


class WorkModel:
    """The scheduler's per-cell work MLP (28 -> 64 -> 64 -> 1, ReLU), with its
    inference, gradient and Adam training run by the engine's kernels."""

    def __init__(self, seed: int = 0):
        self._lib = load_library()
        self._s = ctypes.c_void_p()
        _check(self._lib.ncorr_sched_create(ctypes.c_uint64(seed), ctypes.byref(self._s)))

    @staticmethod
    def num_params() -> int:
        return int(load_library().ncorr_sched_num_params())

    def close(self) -> None:
        if getattr(self, "_s", None) and self._s.value:
            self._lib.ncorr_sched_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params(), dtype=np.float32)
        _check(self._lib.ncorr_sched_get_params(self._s, out.ctypes.data_as(_F), out.size))
        return out

    def set_params(self, p) -> None:
        a = np.ascontiguousarray(np.asarray(p, dtype=np.float32))
        _check(self._lib.ncorr_sched_set_params(self._s, a.ctypes.data_as(_F), a.size))

    def set_precision(self, precision: int) -> None:
        """MLP_FP32 (default) or MLP_BF16: the arithmetic of the forward pass in
        prediction, in the learned queue and in training."""
        _check(self._lib.ncorr_sched_set_precision(self._s, int(precision)))

    def predict(self, feats) -> np.ndarray:
        x = np.ascontiguousarray(np.asarray(feats, dtype=np.float32).reshape(-1, 28))
        out = np.zeros(x.shape[0], dtype=np.float32)
        _check(self._lib.ncorr_sched_predict(self._s, x.ctypes.data_as(_F), x.shape[0], out.ctypes.data_as(_F)))
        return out

    def gradient(self, feats, target):
        """(gradient of the mean squared error, sum of squared errors)."""
        x = np.ascontiguousarray(np.asarray(feats, dtype=np.float32).reshape(-1, 28))
        t = np.ascontiguousarray(np.asarray(target, dtype=np.float32).reshape(-1))
        g = np.zeros(self.num_params(), dtype=np.float32)
        loss = ctypes.c_float(0)
        _check(self._lib.ncorr_sched_gradient(self._s, x.ctypes.data_as(_F), t.ctypes.data_as(_F), x.shape[0],
                                              g.ctypes.data_as(_F), ctypes.byref(loss)))
        return g, float(loss.value)

    def train(self, feats, target, epochs: int = 30, batch: int = 512, lr: float = 3e-3, seed: int = 0) -> float:
        """Adam on the GPU; returns the mean squared error after training."""
        x = np.ascontiguousarray(np.asarray(feats, dtype=np.float32).reshape(-1, 28))
        t = np.ascontiguousarray(np.asarray(target, dtype=np.float32).reshape(-1))
        loss = ctypes.c_float(0)
        _check(self._lib.ncorr_sched_train(self._s, x.ctypes.data_as(_F), t.ctypes.data_as(_F), x.shape[0],
                                           int(epochs), int(batch), float(lr), ctypes.c_uint64(seed),
                                           ctypes.byref(loss)))
        return float(loss.value)


class Batch:
    """Many catalogue triples counted by one persistent launch inside one CUDA
    graph (ncorr_batch_*). `items` is a sequence of (p1, p2, p3): numpy N x 4
    float64 arrays (host) or CUDA float64 tensors (device). The arrays are
    bound to the batch; run() counts their current contents."""

    def __init__(self, corr: ncorr, items, autotune: bool = True):
        lib = load_library()
        self._lib = lib
        self._corr = corr
        keep, ptr, size = {}, [], []
        on_device = None
        for trip in items:
            for p in trip:
                dev = _is_cuda_tensor(p)
                if on_device is None:
                    on_device = dev
                elif on_device != dev:
                    raise NcorrError(NCORR_ERR_INVALID_ARGUMENT, "a batch is all host or all device arrays")
                if id(p) not in keep:
                    keep[id(p)] = p if dev else as_catalog(p)
                a = keep[id(p)]
                ptr.append(a.data_ptr() if dev else a.ctypes.data)
                size.append(a.shape[0])
        self._keep = keep
        n = len(items)
        vp_arr = ctypes.c_void_p * n
        i64_arr = ctypes.c_int64 * n
        p1 = vp_arr(*ptr[0::3]); p2 = vp_arr(*ptr[1::3]); p3 = vp_arr(*ptr[2::3])
        n1 = i64_arr(*size[0::3]); n2 = i64_arr(*size[1::3]); n3 = i64_arr(*size[2::3])
        self._b = ctypes.c_void_p()
        self.n_items = n
        _check(lib.ncorr_batch_create(corr._h, n, p1, n1, p2, n2, p3, n3, int(bool(on_device)),
                                      int(bool(autotune)), ctypes.byref(self._b)))

    def run(self, stream=None) -> None:
        _check(self._lib.ncorr_batch_run(self._b, ctypes.c_void_p(stream) if stream is not None else None))

    def counts_all(self, item: int) -> np.ndarray:
        nb = self._corr.num_bins
        out = np.zeros(nb ** 3, dtype=np.float64)
        _check(self._lib.ncorr_batch_get_counts_all(self._b, int(item), _dptr(out), out.size))
        return out

    def stats(self) -> dict:
        s = NcorrBatchStats()
        _check(self._lib.ncorr_batch_get_stats(self._b, ctypes.byref(s)))
        return s.as_dict()

    def close(self) -> None:
        if getattr(self, "_b", None) and self._b.value:
            self._lib.ncorr_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _is_cuda_tensor(x) -> bool:
    return hasattr(x, "is_cuda") and hasattr(x, "data_ptr") and bool(getattr(x, "is_cuda", False))


def prep_cat_survey(cat1: np.ndarray, cat2: Optional[np.ndarray] = None):
    """survey::prep_cat_survey (source/survey.cu:94-128): shifts the N x 4
    float64 catalogue(s) in place into a positive box; returns (box, ori)."""
    lib = load_library()
    box = np.zeros(3)
    ori = np.zeros(3)
    for c in (cat1, cat2):
        if c is not None and (c.dtype != np.float64 or not c.flags.c_contiguous or c.ndim != 2
                              or c.shape[1] != 4):
            raise NcorrError(NCORR_ERR_INVALID_ARGUMENT, "catalogues must be C-contiguous N x 4 float64")
    if cat2 is None:
        _check(lib.survey_prep_cat(_dptr(cat1), cat1.shape[0], _dptr(box), _dptr(ori)))
    else:
        _check(lib.survey_prep_cat2(_dptr(cat1), cat1.shape[0], _dptr(cat2), cat2.shape[0], _dptr(box),
                                    _dptr(ori)))
    return box, ori


def convert_coordinates(catalog: np.ndarray, H0: float, OmegaM: float, OmegaLambda: float) -> np.ndarray:
    """survey::convert_coordinates (source/survey.cu:39-57): (RA, Dec, z, w)
    rows to comoving (x, y, z, w) in Mpc/h."""
    a = as_catalog(catalog)
    out = np.empty_like(a)
    c = np.array([H0, OmegaM, OmegaLambda], dtype=np.float64)
    _check(load_library().survey_convert_coordinates(_dptr(c), _dptr(a), a.shape[0], _dptr(out)))
    return out


def logspace(start: float, end: float, n: int) -> np.ndarray:
    """logspace (source/utils.cu:16-27)."""
    out = np.zeros(n)
    _check(load_library().ncorr_logspace(float(start), float(end), int(n), _dptr(out)))
    return out


def writeToFileThreeD(filename, triBins, counts) -> None:
    """writeToFileThreeD (source/utils.cu:161-181): rows "r1 r2 r3 count", 6 decimals."""
    b = np.ascontiguousarray(np.asarray(triBins, dtype=np.float64).reshape(-1, 3))
    c = np.ascontiguousarray(np.asarray(counts, dtype=np.float64).reshape(-1))
    if b.shape[0] != c.shape[0]:
        raise NcorrError(NCORR_ERR_INVALID_ARGUMENT, "Vectors have different sizes.")
    _check(load_library().ncorr_write_three_d(str(filename).encode(), _dptr(b), _dptr(c), c.shape[0]))


def writeToFileRppi(filename, triBins, piBins, counts) -> None:
    """writeToFileRppi (source/utils.cu:183-208): rows "r1 r2 r3 pi1 pi2 count"."""
    b = np.ascontiguousarray(np.asarray(triBins, dtype=np.float64).reshape(-1, 3))
    p = np.ascontiguousarray(np.asarray(piBins, dtype=np.float64).reshape(-1, 2))
    c = np.ascontiguousarray(np.asarray(counts, dtype=np.float64).reshape(-1))
    if not (b.shape[0] == p.shape[0] == c.shape[0]):
        raise NcorrError(NCORR_ERR_INVALID_ARGUMENT, "Vectors have different sizes.")
    _check(load_library().ncorr_write_rppi(str(filename).encode(), _dptr(b), _dptr(p), _dptr(c), c.shape[0]))


def readCatalogTxt(filename, box, pos_columns=(0, 1, 2, 3)) -> np.ndarray:
    """readCatalogTxt (source/utils.cu:119-159): N x 4 (x, y, z, w) from text."""
    lib = load_library()
    b = _vec3(box)
    cols = (ctypes.c_int * 4)(*[int(c) for c in pos_columns])
    n = ctypes.c_int64(0)
    _check(lib.ncorr_read_catalog_txt(str(filename).encode(), _dptr(b), cols, None, 0, ctypes.byref(n)))
    out = np.zeros((n.value, 4), dtype=np.float64)
    _check(lib.ncorr_read_catalog_txt(str(filename).encode(), _dptr(b), cols, _dptr(out), n.value, ctypes.byref(n)))
    return out


def generateRandomCatalog(Np: int, box, seed: int = 0) -> np.ndarray:
    """generateRandomCatalog (source/utils.cu:41-52): Np points uniform in
    [0, box), weight 1; seeded here (the reference seeds from the clock)."""
    b = _vec3(box)
    out = np.zeros((int(Np), 4), dtype=np.float64)
    _check(load_library().ncorr_random_catalog(int(Np), _dptr(b), ctypes.c_uint64(seed), _dptr(out)))
    return out
