"""CPU checks of the reference's I/O helpers as this library provides them
(include/utils.hpp of the reference, source/utils.cu:16-208): the result
writers' byte format, the text catalogue reader, the random catalogue, and
a C++ program compiled against this repository's drop-in headers."""
import os
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

from cudancorr_gb300 import api

ROOT = pathlib.Path(__file__).resolve().parent.parent


def reference_rows(*cols):
    """The reference's writers: std::fixed << std::setprecision(6), values
    separated by one space, one row per entry (source/utils.cu:174-180)."""
    n = len(cols[0])
    return "".join(" ".join(f"{c[i]:.6f}" for c in cols) + "\n" for i in range(n))


def test_write_three_d_format(engine_lib, oracle, tmp_path):
    edges = oracle.logspace(0.1, 20.0, 13)
    hist = np.random.default_rng(1).integers(0, 10 ** 9, size=12 ** 3).astype(np.float64)
    counts, bins = oracle.compact(edges, hist)
    path = tmp_path / "DDD.dat"
    api.writeToFileThreeD(path, bins, counts)
    assert path.read_text() == reference_rows(bins[:, 0], bins[:, 1], bins[:, 2], counts)


def test_write_rppi_format(engine_lib, oracle, tmp_path):
    edges = [0.0, 5.0, 10.0, 20.0]
    hist = np.random.default_rng(2).random(27 * 16) * 1e3
    counts, bins, pis = oracle.compact_rppi(edges, 4, hist)
    path = tmp_path / "DDD_rppi.dat"
    api.writeToFileRppi(path, bins, pis, counts)
    assert path.read_text() == reference_rows(bins[:, 0], bins[:, 1], bins[:, 2], pis[:, 0], pis[:, 1], counts)


def test_writers_check_sizes(engine_lib, tmp_path):
    with pytest.raises(api.NcorrError):
        api.writeToFileThreeD(tmp_path / "x.dat", np.zeros((3, 3)), np.zeros(2))
    with pytest.raises(api.NcorrError):
        api.writeToFileRppi(tmp_path / "x.dat", np.zeros((3, 3)), np.zeros((2, 2)), np.zeros(3))


def test_read_catalog_txt(engine_lib, tmp_path):
    rng = np.random.default_rng(3)
    pts = rng.random((500, 4)) * [100.0, 100.0, 100.0, 2.0]
    path = tmp_path / "cat.txt"
    # extra leading column; columns named by index as in the reference's main.cu
    path.write_text("".join(f"7 {float(w)!r} {float(x)!r} {float(y)!r} {float(z)!r}\n" for x, y, z, w in pts))
    got = api.readCatalogTxt(path, (100.0, 100.0, 100.0), (2, 3, 4, 1))
    assert np.array_equal(got, pts)


def test_read_catalog_txt_errors(engine_lib, tmp_path):
    path = tmp_path / "bad.txt"
    path.write_text("1 2 3 1\n4 5 500 1\n")
    with pytest.raises(api.NcorrError) as e:
        api.readCatalogTxt(path, (100.0, 100.0, 100.0))
    assert e.value.code == api.NCORR_ERR_OUT_OF_GRID and "line 2" in str(e.value)
    path.write_text("1 2 3 1\n4 5\n")
    with pytest.raises(api.NcorrError) as e:
        api.readCatalogTxt(path, (100.0, 100.0, 100.0))
    assert "line 2" in str(e.value)
    with pytest.raises(api.NcorrError):
        api.readCatalogTxt(tmp_path / "missing.txt", (100.0, 100.0, 100.0))


def test_random_catalog(engine_lib):
    box = (100.0, 50.0, 25.0)
    a = api.generateRandomCatalog(200_000, box, seed=5)
    b = api.generateRandomCatalog(200_000, box, seed=5)
    c = api.generateRandomCatalog(200_000, box, seed=6)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert np.all(a[:, :3] >= 0) and np.all(a[:, :3] < np.array(box)) and np.all(a[:, 3] == 1.0)
    assert np.allclose(a[:, :3].mean(axis=0), np.array(box) / 2, rtol=0.01)


def test_drop_in_headers_compile_and_run(engine_lib, tmp_path):
    """A program using the reference's class and helper names compiles
    against include/ and links against the library."""
    cxx = shutil.which("g++")
    cuda_inc = pathlib.Path("/usr/local/cuda/include")
    if not cxx or not (cuda_inc / "vector_types.h").exists():
        pytest.skip("g++ or the CUDA headers are missing")
    lib = pathlib.Path(engine_lib._name)
    exe = tmp_path / "utils_roundtrip"
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{ROOT / 'include'}", f"-I{cuda_inc}",
                    str(ROOT / "tests" / "cpp" / "utils_roundtrip.cpp"), "-o", str(exe), f"-L{lib.parent}",
                    "-lcudancorr_gb300", f"-Wl,-rpath,{lib.parent}"], check=True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "three_d.dat").read_text() == "1.500000 2.500000 3.500000 6.000000\n" \
                                                     "0.250000 1.000000 1.125000 1234567.000000\n"
    assert (tmp_path / "rppi.dat").read_text() == "1.500000 2.500000 3.500000 0.000000 1.000000 6.000000\n" \
                                                  "0.250000 1.000000 1.125000 2.000000 3.000000 1234567.000000\n"
