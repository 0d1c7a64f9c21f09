"""The CRF tile table (cnncrf_crf_tuning_*): which prefetch depth and chains
per CTA the chain passes use for a problem shape.  Every tile gives the same
bits; the table only decides speed.  Filled by StereoBatch.autotune or
cnncrf_crf_autotune, or by hand; saved to and merged from a text file so a
deployment measures once.  Host-only: no GPU needed to edit the table."""
import ctypes as C

from ._lib import CrfTile, call

DEFAULT = dict(ring_h=8, chains_per_cta_h=2, ring_v=8, chains_per_cta_v=2)


def _dict(t):
    return {k: getattr(t, k) for k, _ in CrfTile._fields_}


def set_tile(width, height, depth, npairs, delta, **tile):
    t = CrfTile(**dict(DEFAULT, **tile))
    call("cnncrf_crf_tuning_set", width, height, depth, npairs, delta, C.byref(t))


def get_tile(width, height, depth, npairs, delta):
    """(tile dict, found, ms_h, ms_v); the default tile when not found."""
    t, found, mh, mv = CrfTile(), C.c_int(), C.c_float(), C.c_float()
    call("cnncrf_crf_tuning_get", width, height, depth, npairs, delta, C.byref(t), C.byref(found), C.byref(mh),
         C.byref(mv))
    return _dict(t), bool(found.value), mh.value, mv.value


def clear():
    call("cnncrf_crf_tuning_clear")


def count():
    n = C.c_int()
    call("cnncrf_crf_tuning_count", C.byref(n))
    return n.value


def save(path):
    call("cnncrf_crf_tuning_save", str(path).encode())


def load(path):
    call("cnncrf_crf_tuning_load", str(path).encode())


CONV_KEY = ("n_img", "Hin", "Win", "cp_in", "cin", "np", "cout", "kh", "kw", "mode")


def conv_forms():
    """The tensor-core convolutions' tuned launch forms (cnncrf_conv_tuning_*):
    one dict per layer shape, with pair (1: 2-CTA pairs, 0: single CTAs),
    stages and the measured ms of one launch."""
    n = C.c_int()
    call("cnncrf_conv_tuning_count", C.byref(n))
    out = []
    for i in range(n.value):
        shape, pair, stages, ms = (C.c_int * 10)(), C.c_int(), C.c_int(), C.c_float()
        call("cnncrf_conv_tuning_get", i, shape, C.byref(pair), C.byref(stages), C.byref(ms))
        d = dict(zip(CONV_KEY, shape[:]))
        d.update(pair=pair.value, stages=stages.value, ms=ms.value)
        out.append(d)
    return out


def clear_conv():
    call("cnncrf_conv_tuning_clear")
