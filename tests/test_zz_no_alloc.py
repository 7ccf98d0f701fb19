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

WEIGHTED_RTOL = 1e-6  # the weighted-bin tolerance of the parity tests


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
    bit for bit, weighted survey DDR bins within tolerance."""
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
    nz = ref_w != 0
    assert nz.sum() > 10
    td, tr = torch.from_numpy(d).cuda(), torch.from_numpy(r).cuda()
    out_w = torch.full(((len(sedges) - 1) ** 3,), -1.0, dtype=torch.float64, device="cuda")
    for _ in range(2):
        h = noalloc(sbox, sedges, td, td, tr, True, out_w)
        assert np.array_equal(h != 0, nz)
        assert np.max(np.abs(h[nz] - ref_w[nz]) / np.abs(ref_w[nz])) < WEIGHTED_RTOL


def test_noalloc_rejects_dense_neighbourhoods():
    """A neighbourhood larger than the on-chip lists is refused with a clear
    error (the regular entry point spills such lists to global memory)."""
    torch = pytest.importorskip("torch")
    p, box, edges = cases.small_box_clustered()
    t = torch.from_numpy(p).cuda()
    out = torch.zeros(((len(edges) - 1) ** 3,), dtype=torch.float64, device="cuda")
    with pytest.raises(AssertionError, match="too dense"):
        noalloc(box, edges, t, t, t, False, out)


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
