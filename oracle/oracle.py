"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs import this module, and only as the checker (or the timed CPU baseline).
The product library never imports it.  See cnncrf_oracle.h for what the oracle
restates and its parity status (the CRF is parity unpinned).
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None

f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class OracleCfg(C.Structure):
    _fields_ = [
        ("num_layers", C.c_int), ("topology", C.c_int), ("in_channels", C.c_int),
        ("feat_channels", C.c_int), ("unary", C.c_int), ("with_pairwise", C.c_int),
        ("pw_channels", C.c_int), ("precision", C.c_int),
        ("disp_min", C.c_float), ("disp_step", C.c_float), ("disp_max", C.c_float),
        ("lam", C.c_float), ("L1", C.c_float), ("L2", C.c_float), ("delta", C.c_float),
        ("crf_iters", C.c_int), ("crf_shape", C.c_int), ("crf_slack", C.c_float),
        ("ref_iters", C.c_int), ("warps", C.c_int), ("huber_eps", C.c_float), ("C", C.c_float),
        ("refine_interp", C.c_int), ("threads", C.c_int),
    ]


def make_cfg(**kw):
    d = dict(num_layers=7, topology=0, in_channels=3, feat_channels=100, unary=0,
             with_pairwise=1, pw_channels=64, precision=32, disp_min=0.0, disp_step=1.0,
             disp_max=127.0, lam=1.0, L1=1.0, L2=12.0, delta=2.0, crf_iters=4, crf_shape=0,
             crf_slack=0.5, ref_iters=10, warps=0, huber_eps=0.1, C=12.0, refine_interp=0,
             threads=0)
    d.update(kw)
    cfg = OracleCfg()
    for k, v in d.items():
        setattr(cfg, k, v)
    return cfg


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        cp = C.POINTER(OracleCfg)
        L.oracle_num_params.argtypes = [cp]
        L.oracle_padding.argtypes = [cp]
        L.oracle_param_shape.argtypes = [cp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int)]
        L.oracle_xavier.argtypes = [cp, C.c_int, C.c_uint64, f32p]
        L.oracle_xavier.restype = None
        L.oracle_pad_rgba.argtypes = [f32p, C.c_int, C.c_int, C.c_int, f32p]
        L.oracle_pad_rgba.restype = None
        L.oracle_normalize.argtypes = [f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.oracle_normalize.restype = None
        L.oracle_conv.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, f32p, C.c_void_p,
                                  C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
        L.oracle_conv.restype = None
        L.oracle_l2norm.argtypes = [C.c_void_p, C.c_long, C.c_int, C.c_int]
        L.oracle_l2norm.restype = None
        L.oracle_correlation.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, f32p,
                                         C.c_int, C.c_int, C.c_void_p, C.c_int]
        L.oracle_correlation.restype = None
        L.oracle_unary.argtypes = [C.c_void_p, C.c_long, C.c_int, C.c_int, C.c_int]
        L.oracle_unary.restype = None
        L.oracle_disparity_list.argtypes = [C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_int]
        L.oracle_disp_is_float.argtypes = [f32p, C.c_int]
        L.oracle_predict_backward.argtypes = [cp, C.c_void_p, f32p, f32p, C.c_int, C.c_int, f32p, C.c_int, f64p,
                                              C.c_void_p, C.c_void_p]
        L.oracle_predict.argtypes = [cp, C.c_void_p, f32p, f32p, C.c_int, C.c_int, f32p, C.c_int,
                                     C.c_void_p, C.c_void_p]
        L.oracle_crf.argtypes = [f32p, f32p, f32p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                 C.c_int, C.c_int, C.c_int, C.c_float, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_crf.restype = None
        L.oracle_energy.argtypes = [f32p, f32p, f32p, C.c_int, C.c_int, C.c_int, C.c_float,
                                    C.c_float, C.c_int, C.c_int, i32p]
        L.oracle_energy.restype = C.c_double
        L.oracle_chain_bruteforce.argtypes = [f32p, f32p, C.c_int, C.c_int, C.c_float, C.c_float,
                                              C.c_int, C.c_int, i32p]
        L.oracle_chain_bruteforce.restype = C.c_double
        L.oracle_remap.argtypes = [i32p, C.c_long, C.c_float, C.c_float, f32p]
        L.oracle_remap.restype = None
        L.oracle_argmin.argtypes = [f32p, C.c_long, C.c_int, C.c_float, C.c_float, f32p]
        L.oracle_argmin.restype = None
        L.oracle_gray.argtypes = [f32p, C.c_long, f32p]
        L.oracle_gray.restype = None
        L.oracle_census.argtypes = [f32p, f32p, C.c_int, C.c_int, C.c_int, f32p, C.c_int, C.c_float, f32p]
        L.oracle_census.restype = None
        L.oracle_edge_weights.argtypes = [f32p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, f32p, f32p]
        L.oracle_edge_weights.restype = None
        L.oracle_quadfit_direct.argtypes = [f32p, f32p, C.c_long, C.c_int, C.c_float, C.c_float]
        L.oracle_quadfit_direct.restype = None
        L.oracle_lr_check.argtypes = [f32p, f32p, C.c_int, C.c_int, C.c_float, f32p]
        L.oracle_lr_check.restype = None
        L.oracle_warp.argtypes = [f32p, f32p, C.c_int, C.c_int, f32p]
        L.oracle_warp.restype = None
        L.oracle_tv_fit.argtypes = [f32p, C.c_int, C.c_int, C.c_float, C.c_float, f32p]
        L.oracle_tv_fit.restype = None
        L.oracle_tv_iterate.argtypes = [f32p, f32p, f32p, f32p, f32p, f32p, f32p, f32p, C.c_int,
                                        C.c_int, C.c_float, C.c_float, C.c_float, C.c_int]
        L.oracle_tv_iterate.restype = None
        L.oracle_run_pair.argtypes = [cp, C.c_void_p, f32p, f32p, C.c_int, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _dt(precision):
    return np.float64 if precision == 64 else np.float32


def num_params(cfg):
    return lib().oracle_num_params(C.byref(cfg))


def padding(cfg):
    return lib().oracle_padding(C.byref(cfg))


def param_shape(cfg, i):
    s = (C.c_int64 * 4)()
    nd = C.c_int()
    if lib().oracle_param_shape(C.byref(cfg), i, s, C.byref(nd)):
        raise IndexError(i)
    return tuple(s[:nd.value])


def xavier_params(cfg, seed=0):
    out = []
    for i in range(num_params(cfg)):
        a = np.zeros(param_shape(cfg, i), np.float32)
        lib().oracle_xavier(C.byref(cfg), i, seed, a.reshape(-1))
        out.append(a)
    return out


def _param_array(params):
    arrs = [np.ascontiguousarray(p, dtype=np.float32) for p in params]
    ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
    return ptrs, arrs


def pad_rgba(img, p):
    H, W = img.shape[:2]
    out = np.empty((H + 2 * p, W + 2 * p, 4), np.float32)
    lib().oracle_pad_rgba(np.ascontiguousarray(img, np.float32).reshape(-1), W, H, p,
                          out.reshape(-1))
    return out


def normalize(rgba_padded, in_channels, precision=32):
    Hp, Wp = rgba_padded.shape[:2]
    out = np.empty((Hp, Wp, in_channels), _dt(precision))
    lib().oracle_normalize(np.ascontiguousarray(rgba_padded, np.float32).reshape(-1), Wp, Hp,
                           in_channels, precision, _ptr(out))
    return out


def conv(x, w, b, act=1, precision=32, threads=0):
    """x: H x W x Cin NHWC; w: (co, ci, kh, kw) npz layout; valid conv."""
    x = np.ascontiguousarray(x, _dt(precision))
    H, W, Cin = x.shape
    co, ci, kh, kw = w.shape
    out = np.empty((H - kh + 1, W - kw + 1, co), _dt(precision))
    bb = None if b is None else np.ascontiguousarray(b, np.float32)
    lib().oracle_conv(_ptr(x), H, W, Cin, np.ascontiguousarray(w, np.float32).reshape(-1),
                      _ptr(bb), co, kh, kw, act, precision, _ptr(out), threads)
    return out


def l2norm(f, precision=32):
    f = np.ascontiguousarray(f, _dt(precision)).copy()
    lib().oracle_l2norm(_ptr(f), f.size // f.shape[-1], f.shape[-1], precision)
    return f


def disparity_list(dmin, dmax, step):
    n = lib().oracle_disparity_list(dmin, dmax, step, None, 0)
    out = np.empty(n, np.float32)
    lib().oracle_disparity_list(dmin, dmax, step, _ptr(out), n)
    return out


def disp_is_float(lst):
    return bool(lib().oracle_disp_is_float(np.ascontiguousarray(lst, np.float32), len(lst)))


def correlation(fl, fr, lst, precision=32, threads=0):
    fl = np.ascontiguousarray(fl, _dt(precision))
    fr = np.ascontiguousarray(fr, _dt(precision))
    H, W, Cc = fl.shape
    D = len(lst)
    out = np.empty((H, W, D), _dt(precision))
    lib().oracle_correlation(_ptr(fl), _ptr(fr), H, W, Cc, np.ascontiguousarray(lst, np.float32),
                             D, precision, _ptr(out), threads)
    return out


def unary(vol, mode, precision=32):
    v = np.ascontiguousarray(vol, _dt(precision)).copy()
    lib().oracle_unary(_ptr(v), v.size // v.shape[-1], v.shape[-1], mode, precision)
    return v


def predict(cfg, params, left_pad, right_pad, lst):
    h, w = left_pad.shape[:2]
    p = padding(cfg)
    H, W = h - 2 * p, w - 2 * p
    D = len(lst)
    dt = _dt(cfg.precision)
    vol = np.empty((H, W, D), dt)
    pw = np.zeros((2, H, W), dt)
    ptrs, keep = _param_array(params)
    rc = lib().oracle_predict(C.byref(cfg), ptrs, np.ascontiguousarray(left_pad, np.float32).reshape(-1),
                              np.ascontiguousarray(right_pad, np.float32).reshape(-1), w, h,
                              np.ascontiguousarray(lst, np.float32), D, _ptr(vol), _ptr(pw))
    if rc:
        raise RuntimeError("oracle_predict failed: %d" % rc)
    return vol, pw


def predict_backward(cfg, params, left_pad, right_pad, lst, gvol, gpw=None):
    """FP64 parameter gradients (npz layouts) of sum(gvol * vol) + sum(gpw * pw)."""
    h, w = left_pad.shape[:2]
    grads = [np.zeros(np.shape(p), np.float64) for p in params]
    gptr = (C.c_void_p * len(grads))(*[g.ctypes.data for g in grads])
    ptrs, keep = _param_array(params)
    gp = None if gpw is None else np.ascontiguousarray(gpw, np.float64)
    rc = lib().oracle_predict_backward(C.byref(cfg), ptrs, np.ascontiguousarray(left_pad, np.float32).reshape(-1),
                                       np.ascontiguousarray(right_pad, np.float32).reshape(-1), w, h,
                                       np.ascontiguousarray(lst, np.float32), len(lst),
                                       np.ascontiguousarray(gvol, np.float64).reshape(-1),
                                       None if gp is None else gp.ctypes.data_as(C.c_void_p), gptr)
    if rc:
        raise RuntimeError("oracle_predict_backward failed: %d" % rc)
    return grads


def rho_table(L1, L2, delta, shape):
    """rho(|t|) of the CRF spec: 0 at 0, min(L1, L2) (step) or min(L1 t, L2)
    (linear) up to delta, L2 beyond; float32 like the solver."""
    r = np.full(257, np.float32(L2), np.float32)
    r[0] = 0.0
    for t in range(1, int(delta) + 1):
        r[t] = min(np.float32(L1), np.float32(L2)) if shape == 0 else min(np.float32(L1) * np.float32(t),
                                                                           np.float32(L2))
    return r


def hinge(vol, pw, gt, lam, L1, L2, delta, iters, shape=1, slack=0.5):
    """Structured hinge with margin 1 per mislabelled pixel for one pair.

    E(y) = sum_i vol[i, y_i] + sum_edges lam * pw * rho(|y_i - y_j|);
    y_hat = the CRF's labelling of the loss-augmented energy, whose unary is
    vol + 1 at the ground-truth label (the same minimiser as vol - [k != gt]);
    loss = E(gt) - E(y_hat) + #(y_hat != gt).  Returns loss, y_hat, dL/dvol
    (+1 at gt, -1 at y_hat) and dL/dpw = lam * (rho at gt - rho at y_hat) per
    edge (wx on x -> x+1, wy on y -> y+1)."""
    vol = np.ascontiguousarray(vol, np.float32)
    H, W, D = vol.shape
    gt = np.ascontiguousarray(gt, np.int32)
    aug = vol.copy()
    aug[np.arange(H)[:, None], np.arange(W)[None, :], gt] += np.float32(1.0)
    wx = (np.float32(lam) * pw[0]).astype(np.float32)
    wy = (np.float32(lam) * pw[1]).astype(np.float32)
    yh, _, _, _ = crf(aug, wx, wy, L1, L2, delta, iters, shape=shape, slack=slack)
    e_gt = energy(vol, wx, wy, gt, L1, L2, delta, shape)
    e_hat = energy(vol, wx, wy, yh, L1, L2, delta, shape)
    loss = e_gt - e_hat + float((yh != gt).sum())
    gvol = np.zeros((H, W, D), np.float64)
    ii, jj = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    gvol[ii, jj, gt] += 1.0
    gvol[ii, jj, yh] -= 1.0
    r = rho_table(L1, L2, delta, shape).astype(np.float64)
    gpw = np.zeros((2, H, W), np.float64)
    gpw[0, :, :-1] = lam * (r[np.abs(gt[:, 1:] - gt[:, :-1])] - r[np.abs(yh[:, 1:] - yh[:, :-1])])
    gpw[1, :-1, :] = lam * (r[np.abs(gt[1:, :] - gt[:-1, :])] - r[np.abs(yh[1:, :] - yh[:-1, :])])
    return loss, yh, gvol, gpw


def crf(cost, wx, wy, L1, L2, delta, iters, shape=0, slack=0.5, threads=0, want_c1=False):
    cost = np.ascontiguousarray(cost, np.float32)
    H, W, D = cost.shape
    labels = np.empty((H, W), np.int32)
    lb = np.zeros(1, np.float64)
    lbi = np.zeros(max(iters, 1), np.float64)
    c1 = np.empty_like(cost) if want_c1 else None
    lib().oracle_crf(cost.reshape(-1), np.ascontiguousarray(wx, np.float32).reshape(-1),
                     np.ascontiguousarray(wy, np.float32).reshape(-1), W, H, D, L1, L2, int(delta),
                     iters, shape, slack, _ptr(labels), _ptr(lb), _ptr(lbi), _ptr(c1), threads)
    return labels, float(lb[0]), lbi[:iters].copy(), c1


def energy(cost, wx, wy, labels, L1, L2, delta, shape=0):
    cost = np.ascontiguousarray(cost, np.float32)
    H, W, D = cost.shape
    return lib().oracle_energy(cost.reshape(-1), np.ascontiguousarray(wx, np.float32).reshape(-1),
                               np.ascontiguousarray(wy, np.float32).reshape(-1), W, H, D, L1, L2,
                               int(delta), shape, np.ascontiguousarray(labels, np.int32).reshape(-1))


def chain_bruteforce(cost, w, L1, L2, delta, shape=0):
    cost = np.ascontiguousarray(cost, np.float32)
    n, D = cost.shape
    lab = np.empty(n, np.int32)
    e = lib().oracle_chain_bruteforce(cost.reshape(-1), np.ascontiguousarray(w, np.float32), n, D,
                                      L1, L2, int(delta), shape, lab)
    return e, lab


def remap(labels, dmin, dstep):
    labels = np.ascontiguousarray(labels, np.int32)
    out = np.empty(labels.shape, np.float32)
    lib().oracle_remap(labels.reshape(-1), labels.size, dmin, dstep, out.reshape(-1))
    return out


def argmin(vol, dmin, dstep):
    vol = np.ascontiguousarray(vol, np.float32)
    out = np.empty(vol.shape[:-1], np.float32)
    lib().oracle_argmin(vol.reshape(-1), out.size, vol.shape[-1], dmin, dstep, out.reshape(-1))
    return out


def gray(rgba):
    rgba = np.ascontiguousarray(rgba, np.float32)
    out = np.empty(rgba.shape[:-1], np.float32)
    lib().oracle_gray(rgba.reshape(-1), out.size, out.reshape(-1))
    return out


def census(g1, g2, fs, disparities, lam=1.0):
    """H x W x D census volume; disparities[z] = the z-th (positive) disparity."""
    g1 = np.ascontiguousarray(g1, np.float32)
    H, W = g1.shape
    d = np.ascontiguousarray(disparities, np.float32)
    out = np.empty((H, W, len(d)), np.float32)
    lib().oracle_census(g1.reshape(-1), np.ascontiguousarray(g2, np.float32).reshape(-1), W, H, fs, d, len(d), lam,
                        out.reshape(-1))
    return out


def census_list(dmin, dstep, depth):
    """The census kernel's float loop: d = dmin; d += dstep."""
    out, d = [], np.float32(dmin)
    for _ in range(depth):
        out.append(d)
        d = np.float32(d + np.float32(dstep))
    return np.array(out, np.float32)


def edge_weights(g, alpha, beta, lam):
    g = np.ascontiguousarray(g, np.float32)
    H, W = g.shape
    wx, wy = np.empty_like(g), np.empty_like(g)
    lib().oracle_edge_weights(g.reshape(-1), W, H, alpha, beta, lam, wx.reshape(-1), wy.reshape(-1))
    return wx, wy


def quadfit_direct(u, c1, dmin, dstep):
    u = np.array(u, np.float32, copy=True)
    c1 = np.ascontiguousarray(c1, np.float32)
    lib().oracle_quadfit_direct(u.reshape(-1), c1.reshape(-1), u.size, c1.shape[-1], dmin, dstep)
    return u


def lr_check(left, right, th):
    left = np.ascontiguousarray(left, np.float32)
    H, W = left.shape
    out = np.empty_like(left)
    lib().oracle_lr_check(left.reshape(-1), np.ascontiguousarray(right, np.float32).reshape(-1), W, H, th,
                          out.reshape(-1))
    return out


def warp(img, u):
    img = np.ascontiguousarray(img, np.float32)
    H, W = u.shape
    out = np.empty_like(img)
    lib().oracle_warp(img.reshape(-1), np.ascontiguousarray(u, np.float32).reshape(-1), W, H,
                      out.reshape(-1))
    return out


def tv_fit(vol3, step, lam):
    vol3 = np.ascontiguousarray(vol3, np.float32)
    H, W, _ = vol3.shape
    qf = np.empty((H, W, 2), np.float32)
    lib().oracle_tv_fit(vol3.reshape(-1), W, H, step, lam, qf.reshape(-1))
    return qf


def tv_iterate(u, u0, qf, wx, wy, C_, eps, step, iters, p=None, q=None):
    H, W = u.shape
    u = np.ascontiguousarray(u, np.float32).copy()
    u_ = np.zeros_like(u)
    p = np.zeros((H, W, 2), np.float32) if p is None else np.ascontiguousarray(p, np.float32).copy()
    q = np.zeros((H, W, 2), np.float32) if q is None else np.ascontiguousarray(q, np.float32).copy()
    lib().oracle_tv_iterate(u.reshape(-1), u_.reshape(-1), np.ascontiguousarray(u0, np.float32).reshape(-1),
                            np.ascontiguousarray(qf, np.float32).reshape(-1), p.reshape(-1),
                            q.reshape(-1), np.ascontiguousarray(wx, np.float32).reshape(-1),
                            np.ascontiguousarray(wy, np.float32).reshape(-1), W, H, C_, eps, step,
                            iters)
    return u, u_, p, q


def run_pair(cfg, params, left, right):
    H, W = left.shape[:2]
    D = len(disparity_list(cfg.disp_min, cfg.disp_max, cfg.disp_step))
    disp = np.empty((H, W), np.float32)
    labels = np.empty((H, W), np.int32)
    vol = np.empty((H, W, D), np.float32)
    wx = np.empty((H, W), np.float32)
    wy = np.empty((H, W), np.float32)
    lb = np.zeros(1, np.float64)
    ptrs, keep = _param_array(params)
    rc = lib().oracle_run_pair(C.byref(cfg), ptrs, np.ascontiguousarray(left, np.float32).reshape(-1),
                               np.ascontiguousarray(right, np.float32).reshape(-1), W, H,
                               _ptr(disp), _ptr(labels), _ptr(vol), _ptr(wx), _ptr(wy), _ptr(lb))
    if rc:
        raise RuntimeError("oracle_run_pair failed: %d" % rc)
    return dict(disp=disp, labels=labels, vol=vol, wx=wx, wy=wy, lb=float(lb[0]))
