"""The reference's own CUDA kernels as a second oracle (TEST INFRASTRUCTURE).

oracle/build_ref.py compiles the reference's kernel code for the non-CRF
stages unchanged into oracle/_ref/refkernels.fatbin; oracle/ref_host.cpp
launches it the way the reference's host code does (pitched images, texture
objects, launch shapes).  These wrappers take and return numpy arrays and run
on the current CUDA device; available() says whether the module was built
(it can only be built where the reference tree exists).  Only tests and
fixture scripts use this module.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FATBIN = os.path.join(HERE, "_ref", "refkernels.fatbin")
HOST = os.path.join(HERE, "_build", "libref_host.so")

_lib = None


def available():
    return os.path.exists(FATBIN) and os.path.exists(HOST)


def lib():
    global _lib
    if _lib is None:
        import torch
        torch.cuda.init()  # the runtime's primary context, shared with torch
        _lib = C.CDLL(HOST)
        _lib.ref_error.restype = C.c_char_p
        if _lib.ref_open(FATBIN.encode()) != 0:
            raise RuntimeError("ref_open: %s" % _lib.ref_error().decode())
    return _lib


def _call(name, *args):
    if getattr(lib(), name)(*args) != 0:
        raise RuntimeError("%s: %s" % (name, lib().ref_error().decode()))


def _dev(a, dtype=np.float32):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype)).cuda()


def _p(t):
    return C.c_void_p(t.data_ptr())


def _f(x):
    return C.c_float(x)


def correlation(fl_nchw, fr_nchw, lst, rect=0):
    """cuda::forward on an NHWC volume: fl, fr [C][H][W]; lst the disparity
    list (d values); returns [H][W][D].  The list is stored as -d and the
    interpolating kernel runs when its second entry is not an integer, as the
    reference decides (stereo/operators/stereocorrelation.cpp:83-85,
    stereo/operators/stereocorrelation.cu:364-373)."""
    import torch
    Cc, H, W = fl_nchw.shape
    lst = np.asarray(lst, np.float32)
    D = len(lst)
    stored = (-lst).astype(np.float32)
    interp = 1 if D > 1 and abs(float(stored[1]) - round(float(stored[1]))) > 0.001 else 0
    # the reference's kernels read past a row's end where w - d > W - 1 (the
    # next row's values; past the array on the last row): one zero row more
    # keeps those reads inside the allocation.  Compare only w - d <= W - 1.
    fr_padded = np.concatenate([np.ascontiguousarray(fr_nchw, np.float32).reshape(-1), np.zeros(W, np.float32)])
    a, b, d = _dev(fl_nchw), _dev(fr_padded), _dev(stored)
    out = torch.empty((H, W, D), device="cuda", dtype=torch.float32)
    _call("ref_corr", _p(out), _p(a), _p(b), _p(d), 1, Cc, H, W, D, interp, rect)
    return out.cpu().numpy()


def census(g1, g2, fs, dmin, dstep, depth, lam=1.0):
    import torch
    H, W = g1.shape
    a, b = _dev(g1), _dev(g2)
    out = torch.empty((H, W, depth), device="cuda", dtype=torch.float32)
    _call("ref_census", _p(out), _p(a), _p(b), W, H, fs, _f(dmin), _f(dstep), depth, _f(lam))
    return out.cpu().numpy()


def argmin(vol, dmin, dstep):
    import torch
    H, W, D = vol.shape
    v = _dev(vol)
    out = torch.empty((H, W), device="cuda", dtype=torch.float32)
    _call("ref_argmin", _p(out), _p(v), W, H, D, _f(dmin), _f(dstep))
    return out.cpu().numpy()


def tv_fit(vol3, step, lam, do_abs=False):
    import torch
    H, W, _ = vol3.shape
    v = _dev(vol3)
    out = torch.empty((H, W, 2), device="cuda", dtype=torch.float32)
    _call("ref_fit", _p(out), _p(v), W, H, _f(step), _f(lam), 1 if do_abs else 0)
    return out.cpu().numpy()


def tv_iterate(u, u0, qf, wx, wy, C_, step, iters):
    """One warp's TV loop with p = q = 0 at the start and the reference's
    fixed Huber parameter 0.1; returns (u, u_, p, q)."""
    import torch
    H, W = u.shape
    du, du0, dqf, dwx, dwy = _dev(u), _dev(u0), _dev(qf), _dev(wx), _dev(wy)
    du_ = torch.empty_like(du)
    dp = torch.empty((H, W, 2), device="cuda", dtype=torch.float32)
    dq = torch.empty_like(dp)
    _call("ref_tv", _p(du), _p(du_), _p(du0), _p(dqf), _p(dwx), _p(dwy), _p(dp), _p(dq), W, H, _f(C_), _f(step),
          iters)
    return du.cpu().numpy(), du_.cpu().numpy(), dp.cpu().numpy(), dq.cpu().numpy()


def lr_check(left, right, th):
    import torch
    H, W = left.shape
    a, b = _dev(left), _dev(right)
    out = torch.empty((H, W), device="cuda", dtype=torch.float32)
    _call("ref_lrcheck", _p(out), _p(a), _p(b), W, H, _f(th))
    return out.cpu().numpy()


def warp(img, u):
    import torch
    H, W, _ = img.shape
    a, d = _dev(img), _dev(u)
    out = torch.empty((H, W, 4), device="cuda", dtype=torch.float32)
    _call("ref_warp_c4", _p(out), _p(d), _p(a), W, H)
    return out.cpu().numpy()


def remap(labels, dmin, dstep):
    import torch
    H, W = labels.shape
    lab = _dev(labels, np.int32)
    out = torch.empty((H, W), device="cuda", dtype=torch.float32)
    _call("ref_remap", _p(out), _p(lab), W, H, _f(dmin), _f(dstep))
    return out.cpu().numpy()


def gray(rgba):
    import torch
    H, W, _ = rgba.shape
    a = _dev(rgba)
    out = torch.empty((H, W), device="cuda", dtype=torch.float32)
    _call("ref_rgb2gray", _p(out), _p(a), W, H)
    return out.cpu().numpy()


def pad_rgba(img, p):
    import torch
    H, W, _ = img.shape
    a = _dev(img)
    out = torch.empty((H + 2 * p, W + 2 * p, 4), device="cuda", dtype=torch.float32)
    _call("ref_pad_color", _p(out), _p(a), W, H, p)
    return out.cpu().numpy()


def quadfit_direct(u, c1, dmin, dstep):
    """fuseQuadFitDirect on the volume c1 [H][W][D].  The reference reads
    label z + 1 = D when a pixel sits on the last label (the next pixel's
    first entry in memory); the volume gets D trailing zeros so that read
    stays inside the allocation -- compare only pixels below the last label."""
    import torch
    H, W, D = c1.shape
    flat = np.concatenate([np.ascontiguousarray(c1, np.float32).reshape(-1), np.zeros(D, np.float32)])
    v = _dev(flat)
    du = _dev(u)
    _call("ref_quadfit_direct", _p(du), _p(v), W, H, D, _f(dmin), _f(dstep))
    return du.cpu().numpy()
