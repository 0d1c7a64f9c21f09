"""Out-of-bounds checks of the entry points that work on caller buffers, in
place of a memory sanitizer (closed on this pool).

Every input, output and workspace of a call is carved out of one device
arena.  Each sits between guard bands, and the guard bands and the outputs
start out filled with a NaN bit pattern.  This catches three kinds of fault:
- A write past a buffer changes a guard band. The test checks every guard
  word after the calls.
- A read past a buffer fetches NaN (or a huge int), so the result no longer
  equals the oracle's bit for bit.
- An output element the kernel never writes stays NaN, with the same effect.
The sizes are odd: widths that are not a multiple of any tile, depths that
leave lanes partly empty, one-pixel rows and columns.  Every access of a
faulty kernel still lands inside the arena, so a fault shows up as a failed
comparison, not as a device fault."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SENTINEL = 0x7FC0DEAD  # a quiet NaN as float32
GUARD = 1024           # words of guard band on each side of every buffer


class Arena:
    def __init__(self, torch, words):
        self.torch = torch
        self.buf = torch.full((words,), SENTINEL, dtype=torch.int32, device="cuda")
        self.off = GUARD
        self.slots = []

    def place(self, shape, dtype="f4", init=None):
        """A buffer of 4-byte elements (or bytes for 'u1'), 256-byte aligned, guarded on both sides."""
        torch = self.torch
        n = int(np.prod(shape)) if len(shape) else 1
        words = (n + 3) // 4 if dtype == "u1" else n
        start = (self.off + 63) // 64 * 64
        assert start + words + GUARD <= self.buf.numel(), "arena too small"
        view = self.buf[start:start + words]
        if dtype == "f4":
            view = view.view(torch.float32)
        elif dtype == "u1":
            view = view.view(torch.uint8)[:n]
        view = view.view(*shape) if len(shape) else view
        if init is not None:
            view.copy_(torch.from_numpy(np.ascontiguousarray(init)))
        self.slots.append((start, words))
        self.off = start + words + GUARD
        return view

    def check(self):
        self.torch.cuda.synchronize()
        a = self.buf.cpu().numpy()
        inside = np.zeros(a.size, bool)
        for s, w in self.slots:
            inside[s:s + w] = True
        bad = np.nonzero(~inside & (a != np.int32(SENTINEL)))[0]
        assert bad.size == 0, "guard words written at %s" % bad[:8]


def ptr(t):
    return C.c_void_p(t.data_ptr())


CRF_CASES = [
    # H, W, D, delta, shape
    (13, 17, 5, 2, 0),
    (7, 45, 40, 3, 1),
    (9, 31, 128, 4, 1),
    (5, 19, 200, 1, 0),
    (1, 37, 33, 2, 0),
    (29, 1, 64, 3, 1),
]


@pytest.mark.parametrize("H,W,D,delta,shape", CRF_CASES)
def test_crf_solve_stays_in_bounds(cuda, oracle, H, W, D, delta, shape):
    torch = cuda
    from cnncrf import _lib as L
    from cnncrf.api import crf_options
    rng = np.random.default_rng(H * 1000 + W * 10 + D)
    cost = rng.random((H, W, D)).astype(np.float32)
    wx = (rng.random((H, W)) * 0.5).astype(np.float32)
    wy = (rng.random((H, W)) * 0.5).astype(np.float32)
    nb = C.c_size_t()
    L.call("cnncrf_crf_workspace_size", W, H, D, C.byref(nb))
    ar = Arena(torch, 4 * (H * W * D + 2 * H * W) + nb.value // 4 + 64 * GUARD)
    c, x, y = ar.place((H, W, D), init=cost), ar.place((H, W), init=wx), ar.place((H, W), init=wy)
    lab = ar.place((H, W), "i4")
    ws = ar.place((nb.value,), "u1")
    opt = crf_options(0.3, 1.1, delta, 3, shape, 0.5)
    lb = C.c_double()
    L.call("cnncrf_crf_solve", ptr(c), ptr(x), ptr(y), W, H, D, C.byref(opt), ptr(lab), C.byref(lb), ptr(ws),
           nb.value, None)
    ar.check()
    olab, olb, _, _ = oracle.crf(cost, wx, wy, 0.3, 1.1, delta, 3, shape=shape, slack=0.5)
    assert np.array_equal(lab.cpu().numpy(), olab)
    assert lb.value == olb


@pytest.mark.parametrize("lst", [(0.0, 23.0, 1.0), (0.5, 9.5, 0.5), (-3.0, 4.0, 1.0)])
def test_correlation_stays_in_bounds(cuda, oracle, lst):
    torch = cuda
    from cnncrf import _lib as L
    rng = np.random.default_rng(7)
    Cc, H, W = 7, 9, 37
    fl = rng.standard_normal((Cc, H, W)).astype(np.float32)
    fr = rng.standard_normal((Cc, H, W)).astype(np.float32)
    d = np.ascontiguousarray(oracle.disparity_list(*lst), np.float32)
    ar = Arena(torch, 2 * Cc * H * W + H * W * len(d) + 16 * GUARD)
    a, b = ar.place((1, Cc, H, W), init=fl[None]), ar.place((1, Cc, H, W), init=fr[None])
    out = ar.place((H, W, len(d)))
    L.call("cnncrf_correlation_forward", ptr(a), ptr(b), d.ctypes.data_as(C.c_void_p), ptr(out), 1, Cc, H, W,
           len(d), None)
    ar.check()
    assert np.array_equal(out.cpu().numpy(), oracle.correlation(fl.transpose(1, 2, 0), fr.transpose(1, 2, 0), d))


@pytest.mark.parametrize("W,H,iters", [(33, 21, 9), (130, 70, 4), (1, 23, 3), (71, 1, 5)])
def test_refinement_stays_in_bounds(cuda, oracle, W, H, iters):
    """The refinement's parts on caller buffers: remap, warp, the quadratic fit
    and the fused TV iterations with their workspace."""
    torch = cuda
    from cnncrf import _lib as L
    rng = np.random.default_rng(W * 100 + H)
    lab = rng.integers(0, 40, (H, W)).astype(np.int32)
    img = rng.random((H, W, 4)).astype(np.float32)
    vol3 = rng.standard_normal((H, W, 3)).astype(np.float32)
    wx = (rng.random((H, W)) * 2).astype(np.float32)
    wy = (rng.random((H, W)) * 2).astype(np.float32)
    nb = C.c_size_t()
    L.call("cnncrf_tv_workspace_size", W, H, C.byref(nb))
    ar = Arena(torch, 40 * H * W + nb.value // 4 + 64 * GUARD)
    d_lab = ar.place((H, W), "i4", lab)
    d_disp = ar.place((H, W))
    L.call("cnncrf_remap_solution", ptr(d_disp), ptr(d_lab), W, H, 2.0, 0.5, None)
    d_img, d_warp = ar.place((H, W, 4), init=img), ar.place((H, W, 4))
    L.call("cnncrf_warp_image", ptr(d_warp), ptr(d_img), ptr(d_disp), W, H, None)
    d_vol3, d_qf = ar.place((H, W, 3), init=vol3), ar.place((H, W, 2))
    L.call("cnncrf_tv_fit", ptr(d_vol3), ptr(d_qf), W, H, C.c_float(1.0), C.c_float(1.0 / 0.7), None)
    d_u, d_u_ = ar.place((H, W)), ar.place((H, W))
    d_u.copy_(d_disp)
    d_u_.zero_()
    d_p, d_q = ar.place((H, W, 2)), ar.place((H, W, 2))
    d_p.zero_()
    d_q.zero_()
    d_wx, d_wy = ar.place((H, W), init=wx), ar.place((H, W), init=wy)
    ws = ar.place((nb.value,), "u1")
    L.call("cnncrf_tv_iterate", ptr(d_u), ptr(d_u_), ptr(d_disp), ptr(d_qf), ptr(d_p), ptr(d_q), ptr(d_wx),
           ptr(d_wy), W, H, C.c_float(5.0), C.c_float(0.1), C.c_float(0.5), iters, ptr(ws), nb.value, None)
    ar.check()
    disp = oracle.remap(lab, 2.0, 0.5)
    assert np.array_equal(d_disp.cpu().numpy(), disp)
    assert np.array_equal(d_warp.cpu().numpy(), oracle.warp(img, disp))
    qf = oracle.tv_fit(vol3, 1.0, 1.0 / 0.7)
    assert np.array_equal(d_qf.cpu().numpy(), qf)
    for name, g, o in zip(("u", "u_", "p", "q"), (d_u, d_u_, d_p, d_q),
                          oracle.tv_iterate(disp, disp, qf, wx, wy, 5.0, 0.1, 0.5, iters)):
        assert np.array_equal(g.cpu().numpy(), o), name


@pytest.mark.parametrize("W,H,fs,dmin,dstep,D", [(61, 37, 7, 0.0, 1.0, 16), (45, 29, 2, 0.5, 0.5, 20),
                                                 (1, 9, 2, 0.0, 1.0, 4), (19, 1, 3, -2.0, 1.0, 7)])
def test_census_edges_lr_quad_stay_in_bounds(cuda, oracle, W, H, fs, dmin, dstep, D):
    """Grey conversion, the census volume, the edge weights, QuadDirect and the
    left-right check on caller buffers."""
    torch = cuda
    from cnncrf import _lib as L
    rng = np.random.default_rng(W * 31 + H)
    left = rng.random((H, W, 4)).astype(np.float32)
    right = rng.random((H, W, 4)).astype(np.float32)
    ar = Arena(torch, 12 * H * W + H * W * D * 2 + 64 * GUARD)
    d_l, d_r = ar.place((H, W, 4), init=left), ar.place((H, W, 4), init=right)
    g1, g2 = ar.place((H, W)), ar.place((H, W))
    L.call("cnncrf_rgb_to_gray", ptr(d_l), ptr(g1), W, H, None)
    L.call("cnncrf_rgb_to_gray", ptr(d_r), ptr(g2), W, H, None)
    vol = ar.place((H, W, D))
    L.call("cnncrf_census_volume", ptr(g1), ptr(g2), W, H, fs, C.c_float(dmin), C.c_float(dstep), D,
           C.c_float(1.0), ptr(vol), None)
    wx, wy = ar.place((H, W)), ar.place((H, W))
    L.call("cnncrf_edge_weights", ptr(g1), W, H, C.c_float(20.0), C.c_float(0.8), C.c_float(0.4), ptr(wx), ptr(wy),
           None)
    lab = rng.integers(0, D, (H, W)).astype(np.int32)
    u0 = oracle.remap(lab, dmin, dstep)
    c1 = rng.standard_normal((H, W, D)).astype(np.float32)
    d_u, d_c1 = ar.place((H, W), init=u0), ar.place((H, W, D), init=c1)
    L.call("cnncrf_quad_fit_direct", ptr(d_u), ptr(d_c1), W, H, D, C.c_float(dmin), C.c_float(dstep), None)
    dl = (rng.random((H, W)) * 20).astype(np.float32)
    dr = -(dl + rng.standard_normal((H, W)).astype(np.float32) * 0.8)
    d_dl, d_dr, d_lr = ar.place((H, W), init=dl), ar.place((H, W), init=dr), ar.place((H, W))
    L.call("cnncrf_left_right_check", ptr(d_dl), ptr(d_dr), W, H, C.c_float(1.0), ptr(d_lr), None)
    ar.check()
    og1, og2 = oracle.gray(left), oracle.gray(right)
    assert np.array_equal(g1.cpu().numpy(), og1) and np.array_equal(g2.cpu().numpy(), og2)
    assert np.array_equal(vol.cpu().numpy(), oracle.census(og1, og2, fs, oracle.census_list(dmin, dstep, D), 1.0))
    owx, owy = oracle.edge_weights(og1, 20.0, 0.8, 0.4)
    assert np.array_equal(wx.cpu().numpy(), owx) and np.array_equal(wy.cpu().numpy(), owy)
    assert np.array_equal(d_u.cpu().numpy(), oracle.quadfit_direct(u0, c1, dmin, dstep))
    assert np.array_equal(d_lr.cpu().numpy(), oracle.lr_check(dl, dr, 1.0))
