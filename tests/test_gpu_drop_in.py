"""The drop-in C++ classes on the GPU.

tests/cpp/drop_in_main.cu is written the way the reference's example driver
(source/main.cu:20-45 of cudaNcorr) and its survey example use the
reference's headers: `ncorr corr(box, 0, bins, false, {0,0,0})`,
calculateD1D2D3, getTriBinsOut / getTriCountsOut / getPiBinsOut,
writeToFileThreeD / writeToFileRppi, `survey::prep_cat_survey(D, R, box,
ori)`. It is compiled with nvcc against include/ and linked against the
engine's library, then run; its output files must equal, byte for byte, the
same writers applied to the CPU oracle's compacted histograms.
"""
import os
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

from cudancorr_gb300 import api
from cudancorr_gb300 import catalogs as C

pytestmark = pytest.mark.gpu

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    pytest.skip("nvcc not found")


def _write_txt(path, p):
    with open(path, "w") as f:
        for row in p:
            f.write("%.17g %.17g %.17g %.17g\n" % tuple(row))


def test_drop_in_program_on_gpu(engine_lib, oracle, tmp_path):
    lib = pathlib.Path(engine_lib._name)
    exe = tmp_path / "drop_in_main"
    subprocess.run([_nvcc(), "-std=c++17", "-O1", f"-I{ROOT / 'include'}", "-Xcompiler",
                    "-Wno-deprecated-declarations", "-diag-suppress", "1444",
                    str(ROOT / "tests" / "cpp" / "drop_in_main.cu"), "-o", str(exe), f"-L{lib.parent}",
                    "-lcudancorr_gb300", "-Xlinker", f"-rpath,{lib.parent}"], check=True)

    p = C.neyman_scott(500, 8.0, 2.0, 200.0, 41)
    d = C.survey_wedge(3000, 42, False, ra_max_deg=10.0, dec_max_deg=10.0, r_mean=300.0, r_sigma=30.0,
                       r_lo=200.0, r_hi=400.0)
    r = C.survey_wedge(6000, 43, False, ra_max_deg=10.0, dec_max_deg=10.0, r_mean=300.0, r_sigma=30.0,
                       r_lo=200.0, r_hi=400.0)
    _write_txt(tmp_path / "box.txt", p)
    _write_txt(tmp_path / "data.txt", d)
    _write_txt(tmp_path / "randoms.txt", r)
    run = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr

    # Box threeD.
    bins = np.array([3.0 * i for i in range(11)])
    h = oracle.count_threeD(200.0, bins, p)
    counts, tri = oracle.compact(bins, h)
    assert counts.sum() > 0
    api.writeToFileThreeD(tmp_path / "want_box.dat", tri, counts)
    assert (tmp_path / "ddd_box.dat").read_bytes() == (tmp_path / "want_box.dat").read_bytes()

    # Survey threeD, DDR after the joint shift.
    d2, r2 = d.copy(), r.copy()
    sbox, ori = api.prep_cat_survey(d2, r2)
    geo = np.array([float(x) for x in (tmp_path / "survey_geometry.txt").read_text().split()])
    assert np.array_equal(geo, np.concatenate([sbox, ori]))
    lbins = api.logspace(2.0, 30.0, 9)
    hs = oracle.count_threeD(sbox, lbins, d2, d2, r2, survey=True)
    counts_s, tri_s = oracle.compact(lbins, hs)
    assert counts_s.sum() > 0
    api.writeToFileThreeD(tmp_path / "want_survey.dat", tri_s, counts_s)
    assert (tmp_path / "ddr_survey.dat").read_bytes() == (tmp_path / "want_survey.dat").read_bytes()

    # Box rppi.
    rp = api.logspace(1.0, 12.0, 7)
    hr, ov = oracle.count_rppi(200.0, rp, 8, p)
    counts_r, tri_r, pi_r = oracle.compact_rppi(rp, 8, hr)
    assert counts_r.sum() > 0
    api.writeToFileRppi(tmp_path / "want_rppi.dat", tri_r, pi_r, counts_r)
    assert (tmp_path / "ddd_rppi.dat").read_bytes() == (tmp_path / "want_rppi.dat").read_bytes()
