"""cnncrf_crf_solve_static: the CRF solve whose scratch is a fixed array
inside the library, for callers that may not allocate device memory.  Called
through the C ABI and compared with cnncrf_crf_solve on the same inputs over
consecutive calls, so the second and later calls run on whatever the previous
one left in the shared array.  The file name sorts last so that it also runs
after every other test in the same process."""
import ctypes as C

import numpy as np
import pytest

MAX_BYTES = 64 << 20


def _lib():
    import cnncrf
    return cnncrf.lib()


def _opts(shape):
    import cnncrf._lib as L
    if shape == "linear":
        return L.CrfOptions(0.5, 1.5, 3.0, 4, L.RHO_LINEAR, 0.5)
    return L.CrfOptions(1.0, 12.0, 2.0, 4, L.RHO_STEP, 0.5)


def test_static_rejects_oversize_before_any_device_work():
    """A problem whose workspace exceeds the built-in array is refused on the
    host with EINVAL and a message naming the limit."""
    import cnncrf._lib as L
    lib = _lib()
    opt = _opts("step")
    W, H, D = 330, 200, 128
    nb = C.c_size_t()
    assert lib.cnncrf_crf_workspace_size(W, H, D, C.byref(nb)) == L.OK
    assert nb.value > MAX_BYTES
    rc = lib.cnncrf_crf_solve_static(None, None, None, W, H, D, C.byref(opt), None, None, None)
    assert rc == L.EINVAL
    msg = lib.cnncrf_last_error().decode()
    assert "64 MiB" in msg and "cnncrf_crf_solve" in msg
    assert lib.cnncrf_crf_solve_static(None, None, None, W, H, D, None, None, None, None) == L.EINVAL


def test_static_checks_options_in_the_workspace_solves_order():
    """Bad options are reported before the size limit, with the same status
    cnncrf_crf_solve gives them: a delta outside 1..4 is EUNSUPPORTED and an
    unknown shape EINVAL, even for a problem too large for the array."""
    import cnncrf._lib as L
    lib = _lib()
    W, H, D = 330, 200, 128
    bad_delta = L.CrfOptions(1.0, 12.0, 5.0, 4, L.RHO_STEP, 0.5)
    assert lib.cnncrf_crf_solve_static(None, None, None, W, H, D, C.byref(bad_delta), None, None, None) == \
        L.EUNSUPPORTED
    assert lib.cnncrf_crf_solve(None, None, None, W, H, D, C.byref(bad_delta), None, None, None, 0, None) == \
        L.EUNSUPPORTED
    bad_shape = L.CrfOptions(1.0, 12.0, 2.0, 4, 7, 0.5)
    assert lib.cnncrf_crf_solve_static(None, None, None, W, H, D, C.byref(bad_shape), None, None, None) == L.EINVAL
    assert "shape" in lib.cnncrf_last_error().decode()


def _problem(torch, W, H, D, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    cost = torch.rand((H, W, D), device="cuda", generator=g)
    wx = torch.rand((H, W), device="cuda", generator=g)
    wy = torch.rand((H, W), device="cuda", generator=g)
    return cost, wx, wy


def _solve_with_workspace(torch, lib, L, cost, wx, wy, opt):
    H, W, D = cost.shape
    nb = C.c_size_t()
    assert lib.cnncrf_crf_workspace_size(W, H, D, C.byref(nb)) == L.OK
    ws = torch.empty(nb.value, device="cuda", dtype=torch.uint8)
    labels = torch.empty((H, W), device="cuda", dtype=torch.int32)
    lb = C.c_double()
    rc = lib.cnncrf_crf_solve(C.c_void_p(cost.data_ptr()), C.c_void_p(wx.data_ptr()), C.c_void_p(wy.data_ptr()),
                              W, H, D, C.byref(opt), C.c_void_p(labels.data_ptr()), C.byref(lb),
                              C.c_void_p(ws.data_ptr()), nb.value, None)
    assert rc == L.OK, lib.cnncrf_last_error()
    return labels.cpu().numpy(), lb.value


def _solve_static(torch, lib, L, cost, wx, wy, opt, stream=None, want_lb=True):
    H, W, D = cost.shape
    labels = torch.full((H, W), -1, device="cuda", dtype=torch.int32)
    lb = C.c_double()
    st = C.c_void_p(stream.cuda_stream) if stream is not None else None
    rc = lib.cnncrf_crf_solve_static(C.c_void_p(cost.data_ptr()), C.c_void_p(wx.data_ptr()),
                                     C.c_void_p(wy.data_ptr()), W, H, D, C.byref(opt),
                                     C.c_void_p(labels.data_ptr()), C.byref(lb) if want_lb else None, st)
    assert rc == L.OK, lib.cnncrf_last_error()
    if stream is not None:
        stream.synchronize()
    return labels.cpu().numpy(), lb.value if want_lb else None


@pytest.mark.gpu
def test_static_matches_workspace_solve_on_consecutive_calls(cuda):
    """Three calls in a row: a small problem, one that fills most of the
    64 MiB array, and the small one again.  Each result equals the result of
    cnncrf_crf_solve with a fresh caller workspace: identical labels, and a
    lower bound equal to within 1e-12 relative (the same kernels run, so it is
    bit-identical in practice)."""
    torch = cuda
    import cnncrf._lib as L
    lib = _lib()
    cases = [((61, 37, 40), "linear", 1), ((320, 200, 128), "step", 2), ((61, 37, 40), "linear", 3)]
    for (W, H, D), shape, seed in cases:
        nb = C.c_size_t()
        lib.cnncrf_crf_workspace_size(W, H, D, C.byref(nb))
        assert nb.value <= MAX_BYTES
        cost, wx, wy = _problem(torch, W, H, D, seed)
        opt = _opts(shape)
        ref_lab, ref_lb = _solve_with_workspace(torch, lib, L, cost, wx, wy, opt)
        lab, lb = _solve_static(torch, lib, L, cost, wx, wy, opt)
        assert np.array_equal(lab, ref_lab), (W, H, D)
        assert lb == pytest.approx(ref_lb, rel=1e-12, abs=0.0), (W, H, D)
        assert (lab >= 0).all() and (lab < D).all()


@pytest.mark.gpu
def test_static_on_a_caller_stream_without_bound(cuda):
    """A call on a non-default stream with lower_bound = NULL: the solve runs
    on that stream (the labels are complete once it is synchronised) and
    equals the workspace solve's labels."""
    torch = cuda
    import cnncrf._lib as L
    lib = _lib()
    W, H, D = 97, 41, 33
    cost, wx, wy = _problem(torch, W, H, D, 7)
    opt = _opts("linear")
    ref_lab, _ = _solve_with_workspace(torch, lib, L, cost, wx, wy, opt)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    lab, _ = _solve_static(torch, lib, L, cost, wx, wy, opt, stream=s, want_lb=False)
    assert np.array_equal(lab, ref_lab)
