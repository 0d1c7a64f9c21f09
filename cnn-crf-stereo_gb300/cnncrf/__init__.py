"""cnncrf -- GB300-native CNN-CRF stereo (host-side mirror of the reference's
StereoNet / SlackProp / Stereo API over libcnncrf.so's C ABI).

Import note: the package directory is cnn-crf-stereo_gb300/cnncrf; put
cnn-crf-stereo_gb300/ on sys.path (the repo's conftest.py, bench.py and
__graft_entry__.py do).
"""
from ._lib import (BF16, FP32, MATCH_COLORCNN, MATCH_COLORCNN_PAIRWISE, MATCH_GRAYCNN,
                   MATCH_GRAYCNN_PAIRWISE, MATCH_LOAD, RHO_LINEAR, RHO_STEP, TOPO_ALL3X3, TOPO_REF,
                   UNARY_NEG_SOFTMAX, UNARY_ONE_MINUS_DOT, CnnCrfError, LIB_PATH, lib)

__all__ = ["lib", "LIB_PATH", "CnnCrfError", "FP32", "BF16", "TOPO_REF", "TOPO_ALL3X3",
           "UNARY_NEG_SOFTMAX", "UNARY_ONE_MINUS_DOT", "RHO_STEP", "RHO_LINEAR", "MATCH_COLORCNN",
           "MATCH_COLORCNN_PAIRWISE", "MATCH_GRAYCNN", "MATCH_GRAYCNN_PAIRWISE", "MATCH_LOAD"]


def __getattr__(name):
    # the torch-backed API is imported lazily so that the pure-C parts
    # (symbol checks, config parsing) work without touching CUDA
    if name in ("StereoNet", "SlackProp", "Stereo", "StereoBatch", "crf_solve", "correlation_forward",
                "remap_solution", "warp_image", "tv_fit", "tv_iterate", "as_device_tensor"):
        from . import api
        return getattr(api, name)
    raise AttributeError(name)
