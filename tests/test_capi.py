"""CPU checks of the C ABI: the library loads, exports every declared
symbol, and its host-only entry points behave like the reference's."""
import ctypes
import pathlib
import re

import numpy as np
import pytest

from cudancorr_gb300 import api

HEADER = pathlib.Path(__file__).resolve().parent.parent / "include" / "ncorr_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", text)
    skip = {"defined"}
    return sorted({n for n in names if n not in skip and (n.startswith("ncorr_") or n.startswith("survey_"))})


def test_header_lists_match(engine_lib):
    assert set(declared_functions()) == set(api.EXPORTS)


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(engine_lib, name):
    assert isinstance(getattr(engine_lib, name), ctypes._CFuncPtr)


def test_bad_bin_type_is_rejected(engine_lib):
    with pytest.raises(api.NcorrError) as e:
        api.ncorr((100.0, 100.0, 100.0), api.rppi, [0.0, 5.0, 10.0], False, (0, 0, 0))
    assert e.value.code in (api.NCORR_ERR_INVALID_ARGUMENT, api.NCORR_ERR_NO_DEVICE)


def test_rppi_constructor_checks_its_arguments(engine_lib):
    """The rppi constructor rejects another bin type (the reference throws)
    and a pi binning with no bins, before it looks for a device."""
    with pytest.raises(api.NcorrError) as e:
        api.ncorr((100.0, 100.0, 100.0), api.threeD, [0.0, 5.0, 10.0], 4, False, (0, 0, 0))
    assert e.value.code == api.NCORR_ERR_INVALID_ARGUMENT
    for bad in (0, -3):
        with pytest.raises(api.NcorrError) as e:
            api.ncorr((100.0, 100.0, 100.0), api.rppi, [0.0, 5.0, 10.0], bad, False, (0, 0, 0))
        assert e.value.code == api.NCORR_ERR_INVALID_ARGUMENT


def test_smu_is_rejected_by_both_constructors(engine_lib):
    """smu is declared by the reference (include/cudaNcorr.hpp:12) but both
    of its constructors throw for it."""
    for args in ((False, (0, 0, 0)), (4, False, (0, 0, 0))):
        with pytest.raises(api.NcorrError) as e:
            api.ncorr((100.0, 100.0, 100.0), api.smu, [0.0, 5.0, 10.0], *args)
        assert e.value.code == api.NCORR_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("edges", [[5.0], [0.0, 5.0, 5.0], [-1.0, 5.0], [0.0, float("nan")]])
def test_bad_edges_are_rejected(engine_lib, edges):
    with pytest.raises(api.NcorrError) as e:
        api.ncorr((100.0, 100.0, 100.0), api.threeD, edges, False, (0, 0, 0))
    assert e.value.code == api.NCORR_ERR_INVALID_ARGUMENT


def test_survey_prep_matches_oracle(engine_lib, oracle):
    rng = np.random.default_rng(7)
    c1 = rng.normal(size=(300, 4)) * 50
    c2 = rng.normal(size=(500, 4)) * 80
    a1, a2 = c1.copy(), c2.copy()
    b1, b2 = c1.copy(), c2.copy()
    box, ori = api.prep_cat_survey(a1, a2)
    box_o, ori_o = oracle.prep_cat_survey(b1, b2)
    assert np.array_equal(box, box_o) and np.array_equal(ori, ori_o)
    assert np.array_equal(a1, b1) and np.array_equal(a2, b2)
    s1 = c1.copy()
    s1o = c1.copy()
    box, ori = api.prep_cat_survey(s1)
    box_o, ori_o = oracle.prep_cat_survey(s1o)
    assert np.array_equal(box, box_o) and np.array_equal(s1, s1o)


def test_logspace_matches_oracle(engine_lib, oracle):
    assert np.array_equal(api.logspace(0.1, 20.0, 13), oracle.logspace(0.1, 20.0, 13))


def test_catalogue_shape_is_checked():
    with pytest.raises(api.NcorrError):
        api.as_catalog(np.zeros((10, 3)))
