"""The entry point that allocates nothing, against the regular entry point.

ncorr_count_noalloc serves callers that may not allocate device memory (a
fixed device-memory budget handed over up front, or a path where a
cudaMalloc/cudaFree would synchronise the device). It runs the same kernels
with all working memory in one array inside the library. This file is
collected last so that a run stopping at its first failure has run every
other test before it.
"""
import ctypes

import numpy as np
import pytest

from cudancorr_gb300 import api
from cudancorr_gb300 import catalogs as C
from tests import cases

pytestmark = pytest.mark.gpu



def regular(box, edges, p1, p2, p3, survey):
    with api.ncorr(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)), api.threeD, edges, survey,
                   (0.0, 0.0, 0.0)) as corr:
        corr.calculateD1D2D3(p1, p2, p3)
        return corr.getTriCountsAll()


def noalloc(box, edges, t1, t2, t3, survey, out):
    """Calls the C ABI directly; inputs and output are caller-owned CUDA tensors."""
    lib = api.load_library()
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    D = ctypes.POINTER(ctypes.c_double)
    rc = lib.ncorr_count_noalloc(b.ctypes.data_as(D), e.ctypes.data_as(D), len(e), int(survey),
                                 ctypes.c_void_p(t1.data_ptr()), t1.shape[0], ctypes.c_void_p(t2.data_ptr()),
                                 t2.shape[0], ctypes.c_void_p(t3.data_ptr()), t3.shape[0],
                                 ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0, lib.ncorr_last_error().decode()
    return out.cpu().numpy().copy()


def test_noalloc_matches_regular_entry_twice():
    """Two calls in a row on the same scratch: unweighted box counts (the
    six-fold symmetric loop, and the pairwise loop of a non-divisible box)
    and weighted survey DDR bins, all bit for bit. The weighted sums are
    exact fixed-point integers with the same scale on both paths, so they do
    not depend on the order of the additions."""
    torch = pytest.importorskip("torch")
    for make in (cases.small_box_uniform, cases.small_box_nondivisible):
        p, box, edges = make()
        ref = regular(box, edges, p, p, p, False)
        assert ref.sum() > 0
        t = torch.from_numpy(p).cuda()
        out = torch.full(((len(edges) - 1) ** 3,), -1.0, dtype=torch.float64, device="cuda")
        for _ in range(2):
            assert np.array_equal(noalloc(box, edges, t, t, t, False, out), ref)
    d, r, sbox, _, _ = cases.small_survey(nd=3000, nr=6000, weighted=True)
    sedges = api.logspace(3.0, 40.0, 9)
    ref_w = regular(sbox, sedges, d, d, r, True)
    assert (ref_w != 0).sum() > 10
    td, tr = torch.from_numpy(d).cuda(), torch.from_numpy(r).cuda()
    out_w = torch.full(((len(sedges) - 1) ** 3,), -1.0, dtype=torch.float64, device="cuda")
    for _ in range(2):
        assert np.array_equal(noalloc(sbox, sedges, td, td, tr, True, out_w), ref_w)


def test_noalloc_three_catalogues_and_survey_ddd():
    """Three distinct box catalogues (p1, p2, p3 all different), and an
    unweighted survey DDD (the six-fold loop on the clipped grid), each twice
    in a row, bit for bit against the regular entry point."""
    torch = pytest.importorskip("torch")
    p1, box, edges = cases.small_box_uniform(seed=31, n=2500)
    p2 = C.uniform_box(2800, box, 32)
    p3 = C.uniform_box(3100, box, 33)
    ref = regular(box, edges, p1, p2, p3, False)
    assert ref.sum() > 0
    t1, t2, t3 = (torch.from_numpy(a).cuda() for a in (p1, p2, p3))
    out = torch.full(((len(edges) - 1) ** 3,), -1.0, dtype=torch.float64, device="cuda")
    for _ in range(2):
        assert np.array_equal(noalloc(box, edges, t1, t2, t3, False, out), ref)
    d, _, sbox, _, _ = cases.small_survey(nd=4000, nr=10)
    sedges = api.logspace(3.0, 40.0, 9)
    ref_s = regular(sbox, sedges, d, d, d, True)
    assert ref_s.sum() > 0
    td = torch.from_numpy(d).cuda()
    out_s = torch.full(((len(sedges) - 1) ** 3,), -1.0, dtype=torch.float64, device="cuda")
    for _ in range(2):
        assert np.array_equal(noalloc(sbox, sedges, td, td, td, True, out_s), ref_s)


def test_noalloc_dense_neighbourhoods():
    """A clustered box whose neighbourhoods hold thousands of points counts
    bit for bit like the regular entry point, twice in a row; one whose lists
    cannot fit the fixed scratch even for one CTA (all 40,000 points in one
    cell, seen through 27 images) is refused with a clear error."""
    torch = pytest.importorskip("torch")
    p, box, edges = cases.small_box_clustered()
    ref = regular(box, edges, p, p, p, False)
    t = torch.from_numpy(p).cuda()
    out = torch.full(((len(edges) - 1) ** 3,), -1.0, dtype=torch.float64, device="cuda")
    for _ in range(2):
        assert np.array_equal(noalloc(box, edges, t, t, t, False, out), ref)
    q = C.uniform_box(40000, 50.0, 9)
    tq = torch.from_numpy(q).cuda()
    with pytest.raises(AssertionError, match="too dense"):
        noalloc(50.0, edges, tq, tq, tq, False, out)


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    p = C.uniform_box(65537, 1000.0, 3)
    t = torch.from_numpy(p).cuda()
    edges = C.linear_edges(20.0, 4)
    out = torch.zeros((4 ** 3,), dtype=torch.float64, device="cuda")
    lib = api.load_library()
    b = np.full(3, 1000.0)
    D = ctypes.POINTER(ctypes.c_double)
    rc = lib.ncorr_count_noalloc(b.ctypes.data_as(D), edges.ctypes.data_as(D), len(edges), 0,
                                 ctypes.c_void_p(t.data_ptr()), t.shape[0], ctypes.c_void_p(t.data_ptr()),
                                 t.shape[0], ctypes.c_void_p(t.data_ptr()), t.shape[0],
                                 ctypes.c_void_p(out.data_ptr()), None)
    assert rc == api.NCORR_ERR_CAPACITY
    assert b"65536" in lib.ncorr_last_error()


def _raw_call(box, edges, t, out):
    lib = api.load_library()
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.float64))
    D = ctypes.POINTER(ctypes.c_double)
    rc = lib.ncorr_count_noalloc(b.ctypes.data_as(D), e.ctypes.data_as(D), len(e), 0,
                                 ctypes.c_void_p(t.data_ptr()), t.shape[0], ctypes.c_void_p(t.data_ptr()),
                                 t.shape[0], ctypes.c_void_p(t.data_ptr()), t.shape[0],
                                 ctypes.c_void_p(out.data_ptr()), None)
    return rc, lib.ncorr_last_error()


def test_noalloc_rejects_cell_and_bin_limits():
    """More than 32768 cells (33^3 here) or more than 31 bins per side is
    refused with NCORR_ERR_CAPACITY / NCORR_ERR_INVALID_ARGUMENT and a message
    naming the limit."""
    torch = pytest.importorskip("torch")
    p = C.uniform_box(1000, 330.0, 5)
    t = torch.from_numpy(p).cuda()
    out = torch.zeros((4 ** 3,), dtype=torch.float64, device="cuda")
    rc, msg = _raw_call(330.0, C.linear_edges(10.0, 4), t, out)
    assert rc == api.NCORR_ERR_CAPACITY and b"32768 cells" in msg
    out32 = torch.zeros((32 ** 3,), dtype=torch.float64, device="cuda")
    rc, msg = _raw_call(330.0, C.linear_edges(64.0, 32), t, out32)
    assert rc == api.NCORR_ERR_INVALID_ARGUMENT and b"31 bins" in msg
