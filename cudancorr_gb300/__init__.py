"""GB300-native three-point correlation engine.

Drop-in for the threeD counting path of cudaNcorr: the same (r1, r2, r3)
histogram of ordered triangles, computed by hand-written CUDA kernels for
sm_103a behind the C ABI of include/ncorr_gb300.h.
"""
from .api import (NcorrError, ncorr, load_library, library_path, logspace, prep_cat_survey,
                  convert_coordinates, threeD,
                  rppi, smu, EXPORTS)
from . import catalogs

__all__ = ["NcorrError", "ncorr", "load_library", "library_path", "logspace", "prep_cat_survey",
           "threeD", "rppi", "smu", "EXPORTS", "catalogs"]
