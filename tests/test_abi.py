"""CPU tests of the C ABI: the library loads, exports every symbol the public
headers declare, and its host-side argument checks return status codes
without touching a GPU."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in ("cnncrf.h",):
        src = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"^(?:int|const char|double)\s*\*?\s*(cnncrf_[a-z0-9_]+)\s*\(", src, re.M))
    return names


@pytest.fixture(scope="module")
def lib():
    import cnncrf
    return cnncrf.lib()


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.cnncrf_abi_version() == 1


def test_net_create_rejects_bad_descriptions(lib):
    import cnncrf._lib as L
    h = C.c_void_p()
    bad = [
        L.NetDesc(0, 0, 3, 100, 0, 0, 0, 64),    # no layers
        L.NetDesc(7, 9, 3, 100, 0, 0, 0, 64),    # topology
        L.NetDesc(7, 0, 4, 100, 0, 0, 0, 64),    # in_channels
        L.NetDesc(7, 0, 3, 300, 0, 0, 0, 64),    # feat_channels
        L.NetDesc(4, 0, 3, 100, 0, 0, 0, 64),    # odd receptive-field loss
        L.NetDesc(1, 0, 3, 100, 0, 0, 1, 64),    # pairwise needs pad >= 2
    ]
    for d in bad:
        rc = lib.cnncrf_net_create(C.byref(h), C.byref(d), 1, 64, 64)
        assert rc == L.EINVAL, (rc, lib.cnncrf_last_error())
        assert lib.cnncrf_last_error()
    d = L.NetDesc(7, 0, 3, 100, 0, 0, 0, 64)
    assert lib.cnncrf_net_create(C.byref(h), C.byref(d), 0, 64, 64) == L.EINVAL
    assert lib.cnncrf_net_create(C.byref(h), C.byref(d), 1, 6, 6) == L.ESHAPE


def test_net_shapes_follow_reference_topology(lib):
    import cnncrf._lib as L
    h = C.c_void_p()
    d = L.NetDesc(7, 0, 3, 100, 0, 0, 1, 64)
    assert lib.cnncrf_net_create(C.byref(h), C.byref(d), 1, 64, 72) == L.OK
    n = C.c_int()
    lib.cnncrf_net_num_params(h, C.byref(n))
    assert n.value == 19
    pad = C.c_int()
    lib.cnncrf_net_padding(h, C.byref(pad))
    assert pad.value == 4
    s = (C.c_int64 * 4)()
    nd = C.c_int()
    lib.cnncrf_net_param_shape(h, 0, s, C.byref(nd))
    assert tuple(s[:nd.value]) == (100, 3, 3, 3)
    lib.cnncrf_net_param_shape(h, 2, s, C.byref(nd))
    assert tuple(s[:nd.value]) == (100, 100, 2, 2)
    lib.cnncrf_net_param_shape(h, 18, s, C.byref(nd))
    assert tuple(s[:nd.value]) == (2, 64, 1, 1)
    assert lib.cnncrf_net_param_shape(h, 19, s, C.byref(nd)) == L.EINVAL
    # predict before initNet is a state error, not a crash
    assert lib.cnncrf_net_predict(h, None, None, None) == L.ESTATE
    lib.cnncrf_net_destroy(h)


def test_stereo_host_checks(lib):
    import cnncrf._lib as L
    s = C.c_void_p()
    assert lib.cnncrf_stereo_create(C.byref(s), None) == L.OK
    assert lib.cnncrf_stereo_compute_volume(s, 1) == L.ESTATE
    assert lib.cnncrf_stereo_initialize(s, 0, 10, 0.0, 1.0, 10.0) == L.EINVAL
    assert lib.cnncrf_stereo_initialize(s, 10, 10, 0.0, 0.0, 10.0) == L.EINVAL
    assert lib.cnncrf_stereo_set_matching_function(s, 42) == L.EINVAL
    lib.cnncrf_stereo_destroy(s)


def test_batch_host_checks(lib):
    import cnncrf._lib as L
    b = C.c_void_p()
    assert lib.cnncrf_batch_create(C.byref(b), None) == L.OK
    assert lib.cnncrf_batch_run(b, 1.0, 5.0, 2.0, 3, 1.0) == L.ESTATE  # no pairs
    assert lib.cnncrf_batch_set_group_size(b, -1) == L.EINVAL
    assert lib.cnncrf_batch_set_group_size(b, 2) == L.OK
    i = C.c_int()
    assert lib.cnncrf_batch_add_pair(b, 0, 10, 0.0, 1.0, 7.0, C.byref(i)) == L.EINVAL
    assert lib.cnncrf_batch_add_pair(b, 20, 10, 0.0, 1.0, 7.0, C.byref(i)) == L.OK and i.value == 0
    assert lib.cnncrf_batch_add_pair(b, 20, 10, 0.0, 1.0, 7.0, C.byref(i)) == L.OK and i.value == 1
    n = C.c_int()
    lib.cnncrf_batch_num_pairs(b, C.byref(n))
    assert n.value == 2
    assert lib.cnncrf_batch_set_group_size(b, 4) == L.ESTATE  # grouping is fixed once pairs exist
    out = C.c_void_p()
    assert lib.cnncrf_batch_get_output_device(b, 5, C.byref(out)) == L.EINVAL
    lib.cnncrf_batch_destroy(b)


def test_crf_option_checks(lib):
    import cnncrf._lib as L
    o = L.CrfOptions()
    assert lib.cnncrf_crf_default_options(C.byref(o)) == L.OK
    assert (o.L1, o.L2, o.delta, o.total_it) == (1.0, 12.0, 2.0, 4)
    o.delta = 2.5
    assert lib.cnncrf_crf_solve(None, None, None, 4, 4, 4, C.byref(o), None, None, None, 0, None) == L.EUNSUPPORTED
    o.delta = 2.0
    assert lib.cnncrf_crf_solve(None, None, None, 4, 4, 4, C.byref(o), None, None, None, 0, None) == L.EINVAL
    nb = C.c_size_t()
    assert lib.cnncrf_crf_workspace_size(10, 10, 8, C.byref(nb)) == L.OK and nb.value >= 2 * 800 * 4
    sp = C.c_void_p()
    lib.cnncrf_slackprop_create(C.byref(sp))
    assert lib.cnncrf_slackprop_execute(sp) == L.ESTATE
    assert lib.cnncrf_slackprop_set_op(sp, b"nonsense", 1.0) == L.EINVAL
    lib.cnncrf_slackprop_destroy(sp)


def test_config_file_parser():
    from cnncrf import config
    txt = "matching = COLORPAIR\nnum-layers = 7\nL1 = 1.00227201\n\ncrf-iterations = 5\nwith-xy = 1\n"
    cfg = config.parse_cfg_text(txt)
    assert cfg["matching"] == "COLORPAIR" and cfg["num-layers"] == 7
    assert abs(cfg["L1"] - 1.00227201) < 1e-9 and cfg["with-xy"] is True
    full = config.resolve(["--config-file", "x.cfg", "--L1", "3"], cfg_text=txt, positional=["a", "b"])
    assert full["L1"] == 3.0          # command line wins (stereo/stereo_img.cpp:94-103)
    assert full["L2"] == 12.0         # default
    assert full["crf-iterations"] == 5


def test_conv_pairs_switch(lib):
    """The process-wide choice between the paired (cta_group::2) and the
    single-CTA tensor-core convolution is a host flag: on by default, set and
    read back without a GPU; a null output pointer is rejected."""
    import cnncrf._lib as L
    v = C.c_int(-1)
    assert lib.cnncrf_get_conv_pairs(C.byref(v)) == L.OK and v.value == 1
    try:
        assert lib.cnncrf_set_conv_pairs(0) == L.OK
        assert lib.cnncrf_get_conv_pairs(C.byref(v)) == L.OK and v.value == 0
    finally:
        assert lib.cnncrf_set_conv_pairs(1) == L.OK
    assert lib.cnncrf_get_conv_pairs(C.byref(v)) == L.OK and v.value == 1
    assert lib.cnncrf_get_conv_pairs(None) == L.EINVAL


def test_selftest_poll_limit_checked_on_host(lib):
    """The bounded-wait probe refuses a poll limit outside 1 .. 2^20 before it
    touches the device."""
    import cnncrf._lib as L
    for polls in (0, -3, (1 << 20) + 1):
        assert L.selftest_bounded_wait(polls, arrive=False) == L.EINVAL


def test_concat_net_shapes_and_checks(lib):
    """ConcatStereoNet (TOPO_CONCAT): the reference constructor's depth /
    growth-rate table, zero padding, 2 L + 1 parameters with the pairwise
    conv over the g L concatenated channels; other depths, a wrong channel
    count and BF16 are refused before anything is allocated."""
    import cnncrf._lib as L
    h = C.c_void_p()
    n, s, nd, pad = C.c_int(), (C.c_int64 * 4)(), C.c_int(), C.c_int()
    for layers, g in L.CONCAT_GROWTH.items():
        d = L.NetDesc(layers, L.TOPO_CONCAT, 3, 0, 0, 0, 1, 64)
        assert lib.cnncrf_net_create(C.byref(h), C.byref(d), 1, 40, 30) == L.OK, lib.cnncrf_last_error()
        lib.cnncrf_net_num_params(h, C.byref(n))
        assert n.value == 2 * layers + 1
        lib.cnncrf_net_padding(h, C.byref(pad))
        assert pad.value == 0
        lib.cnncrf_net_param_shape(h, 0, s, C.byref(nd))
        assert tuple(s[:nd.value]) == (g, 3, 3, 3)
        lib.cnncrf_net_param_shape(h, 1, s, C.byref(nd))
        assert tuple(s[:nd.value]) == (g,)
        if layers > 1:
            lib.cnncrf_net_param_shape(h, 2, s, C.byref(nd))
            assert tuple(s[:nd.value]) == (g, g, 3, 3)
        lib.cnncrf_net_param_shape(h, 2 * layers, s, C.byref(nd))
        assert tuple(s[:nd.value]) == (2, g * layers, 3, 3)
        lib.cnncrf_net_destroy(h)
    for d, rc in [(L.NetDesc(4, L.TOPO_CONCAT, 3, 0, 0, 0, 0, 64), L.EINVAL),   # not in the table
                  (L.NetDesc(7, L.TOPO_CONCAT, 3, 100, 0, 0, 0, 64), L.EINVAL),  # 7 x 14 = 98 channels
                  (L.NetDesc(7, L.TOPO_CONCAT, 3, 98, 0, L.BF16, 0, 64), L.EUNSUPPORTED)]:
        assert lib.cnncrf_net_create(C.byref(h), C.byref(d), 1, 40, 30) == rc
        assert lib.cnncrf_last_error()
    d = L.NetDesc(7, L.TOPO_CONCAT, 3, 98, 0, 0, 0, 64)
    assert lib.cnncrf_net_create(C.byref(h), C.byref(d), 1, 40, 30) == L.OK
    lib.cnncrf_net_destroy(h)
