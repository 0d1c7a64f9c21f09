"""Python mirror of the reference's C++ API for the CNN-CRF stereo path, over
the C ABI of libcnncrf.so.  Device memory is torch CUDA tensors (plumbing);
every computation is a call into the library.

  StereoNet  -- StereoNet / ColorStereoNet (stereo/stereonet.h:27-72,
                stereo/colorstereonet.h:22-33)
  SlackProp  -- slack_prop_2D_alg as used at stereo/stereo.cpp:140-154 and
                stereo/operators/slackprop.cpp:96-137
  Stereo     -- Stereo (stereo/stereo.h:40-133)
  correlation_forward, crf_solve, remap_solution, warp_image, tv_fit,
  tv_iterate -- the standalone operators.

Errors surface as CnnCrfError carrying the library status (the reference
called exit(-1), stereo/error_util.h:29-52).
"""
import ctypes as C

import numpy as np
import torch

from . import _lib as L
from ._lib import CnnCrfError, CrfOptions, NetDesc, StereoOptions, call

__all__ = ["StereoNet", "SlackProp", "Stereo", "StereoBatch", "crf_solve", "correlation_forward", "remap_solution",
           "warp_image", "tv_fit", "tv_iterate", "CnnCrfError", "as_device_tensor"]


class _CudaArray:
    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 2, "strides": None}


def as_device_tensor(ptr, shape, dtype=torch.float32):
    """Wrap library-owned device memory as a torch tensor (no copy)."""
    ts = {torch.float32: "<f4", torch.int32: "<i4"}[dtype]
    return torch.as_tensor(_CudaArray(ptr, shape, ts), device="cuda")


def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return C.c_void_p(t.data_ptr())


def _stream_ptr(stream):
    if stream is None:
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return C.c_void_p(stream.cuda_stream)


class StereoNet:
    """StereoNet(numLayers, n, c, h, w) / ColorStereoNet / ConcatStereoNet
    (topology TOPO_CONCAT); h, w are the padded size.  feat_channels defaults
    to 100, or to the concatenated width (growth rate x layers) for
    TOPO_CONCAT."""

    def __init__(self, num_layers, n, c, h, w, topology=L.TOPO_REF, feat_channels=None,
                 unary=L.UNARY_NEG_SOFTMAX, precision=L.FP32, with_pairwise=False, pw_channels=64,
                 stream=None):
        if feat_channels is None:
            feat_channels = L.CONCAT_GROWTH.get(num_layers, 0) * num_layers if topology == L.TOPO_CONCAT else 100
        d = NetDesc(num_layers, topology, c, feat_channels, unary, precision,
                    1 if with_pairwise else 0, pw_channels)
        self._h = C.c_void_p()
        call("cnncrf_net_create", C.byref(self._h), C.byref(d), n, h, w)
        self.desc = d
        self.n, self.h, self.w = n, h, w
        self.pad = self.padding()
        self.H, self.W = h - 2 * self.pad, w - 2 * self.pad
        self.volume = None
        self.pairwise_out = None
        self.stream = stream
        call("cnncrf_net_set_stream", self._h, _stream_ptr(stream))

    def __del__(self):
        if getattr(self, "_h", None) and L._lib is not None:
            L.lib().cnncrf_net_destroy(self._h)
            self._h = None

    def padding(self):
        p = C.c_int()
        call("cnncrf_net_padding", self._h, C.byref(p))
        return p.value

    def init_net(self, min_disp=0.0, max_disp=0.0, step=0.0, rect_corr=0, unary_out=None,
                 pairwise_out=None):
        D = _count_disparities(min_disp, max_disp, step)
        lead = () if self.n == 1 else (self.n,)  # the library writes every pair of the batch
        self.volume = unary_out if unary_out is not None else torch.empty(
            lead + (self.H, self.W, D), device="cuda", dtype=torch.float32)
        if self.desc.with_pairwise:
            self.pairwise_out = pairwise_out if pairwise_out is not None else torch.zeros(
                lead + (2, self.H, self.W), device="cuda", dtype=torch.float32)
        need = self.n * self.H * self.W * D
        if self.volume.numel() < need or (self.desc.with_pairwise and self.pairwise_out.numel() < 2 * need // D):
            raise ValueError("init_net: output buffers smaller than %d pairs" % self.n)
        call("cnncrf_net_init", self._h, min_disp, max_disp, step, rect_corr, _ptr(self.volume),
             _ptr(self.pairwise_out))

    def set_all_params(self, npz_path):
        call("cnncrf_net_set_all_params", self._h, str(npz_path).encode())

    def set_param(self, index, array):
        a = np.ascontiguousarray(array, dtype=np.float32)
        shape = (C.c_int64 * a.ndim)(*a.shape)
        call("cnncrf_net_set_param", self._h, index, a.ctypes.data_as(C.c_void_p), shape, a.ndim)

    def init_xavier(self, seed=0):
        call("cnncrf_net_init_xavier", self._h, seed)

    def num_params(self):
        n = C.c_int()
        call("cnncrf_net_num_params", self._h, C.byref(n))
        return n.value

    def param_shape(self, i):
        s = (C.c_int64 * 4)()
        nd = C.c_int()
        call("cnncrf_net_param_shape", self._h, i, s, C.byref(nd))
        return tuple(s[:nd.value])

    def set_disparities(self, min_disp, max_disp, step, out=None):
        D = _count_disparities(min_disp, max_disp, step)
        if out is None:
            out = torch.empty((self.H, self.W, D), device="cuda", dtype=torch.float32)
        call("cnncrf_net_set_disparities", self._h, min_disp, max_disp, step, _ptr(out))
        self.volume = out

    def num_disparities(self):
        n = C.c_int()
        call("cnncrf_net_num_disparities", self._h, C.byref(n))
        return n.value

    def predict(self, left_rgba, right_rgba):
        """ColorStereoNet::predict: padded RGBA CUDA tensors (h, w, 4) -> (H, W, D) volume."""
        out = C.c_void_p()
        call("cnncrf_net_predict", self._h, _ptr(left_rgba), _ptr(right_rgba), C.byref(out))
        return self.volume

    def features(self, side):
        f = torch.empty((self.H, self.W, self.desc.feat_channels), device="cuda", dtype=torch.float32)
        call("cnncrf_net_features", self._h, side, _ptr(f))
        return f


def _count_disparities(mn, mx, step):
    """The reference's float loop (stereo/operators/stereocorrelation.cpp:83-85)."""
    mn, mx, step = np.float32(mn), np.float32(mx), np.float32(step)
    if not step > 0:
        return 1
    n, d = 0, mn
    while d <= mx:
        n += 1
        d = np.float32(d + step)
        if n > 4096:
            break
    return max(n, 1)


def correlation_forward(fl_nchw, fr_nchw, disparities, stream=None):
    """StereoCorrelation::forward (NCHW features, stored = negated disparity list) -> (H, W, D)."""
    n, c, h, w = fl_nchw.shape
    d = np.ascontiguousarray(disparities, dtype=np.float32)
    out = torch.empty((h, w, len(d)), device="cuda", dtype=torch.float32)
    call("cnncrf_correlation_forward", _ptr(fl_nchw), _ptr(fr_nchw), d.ctypes.data_as(C.c_void_p), _ptr(out),
         n, c, h, w, len(d), _stream_ptr(stream))
    return out


def crf_options(L1=1.0, L2=12.0, delta=2, total_it=4, shape=L.RHO_STEP, slack=0.5):
    return CrfOptions(L1, L2, float(delta), total_it, shape, slack)


def crf_solve(cost, wx, wy, L1=1.0, L2=12.0, delta=2, total_it=4, shape=L.RHO_STEP, slack=0.5,
              stream=None, workspace=None):
    """One-shot CRF solve: cost (H, W, D), wx / wy (H, W) -> int32 labels (H, W), FP64 bound."""
    H, W, D = cost.shape
    opt = crf_options(L1, L2, delta, total_it, shape, slack)
    nb = C.c_size_t()
    call("cnncrf_crf_workspace_size", W, H, D, C.byref(nb))
    if workspace is None:
        workspace = torch.empty(nb.value, device="cuda", dtype=torch.uint8)
    labels = torch.empty((H, W), device="cuda", dtype=torch.int32)
    lb = C.c_double()
    call("cnncrf_crf_solve", _ptr(cost), _ptr(wx), _ptr(wy), W, H, D, C.byref(opt), _ptr(labels),
         C.byref(lb), _ptr(workspace), nb.value, _stream_ptr(stream))
    return labels, lb.value


def crf_autotune(cost, wx, wy, L1=1.0, L2=12.0, delta=2, total_it=4, shape=L.RHO_STEP, slack=0.5, stream=None,
                 workspace=None):
    """Measure every CRF tile on this single-pair problem and enter the fastest
    in the tile table (cnncrf.tuning); synchronises."""
    H, W, D = cost.shape
    opt = crf_options(L1, L2, delta, total_it, shape, slack)
    nb = C.c_size_t()
    call("cnncrf_crf_workspace_size", W, H, D, C.byref(nb))
    if workspace is None:
        workspace = torch.empty(nb.value, device="cuda", dtype=torch.uint8)
    call("cnncrf_crf_autotune", _ptr(cost), _ptr(wx), _ptr(wy), W, H, D, C.byref(opt), _ptr(workspace), nb.value,
         _stream_ptr(stream))


class SlackProp:
    """slack_prop_2D_alg: init(C{K,W,H}, sols); ops[...]; update_W; execute; LB; get_C1."""

    def __init__(self, stream=None):
        self._h = C.c_void_p()
        call("cnncrf_slackprop_create", C.byref(self._h))
        call("cnncrf_slackprop_set_stream", self._h, _stream_ptr(stream))
        self.ops = _Ops(self)
        self._keep = []

    def __del__(self):
        if getattr(self, "_h", None) and L._lib is not None:
            L.lib().cnncrf_slackprop_destroy(self._h)
            self._h = None

    def init(self, cost, labels):
        H, W, D = cost.shape
        self._shape = (H, W, D)
        self._keep = [cost, labels]
        call("cnncrf_slackprop_init", self._h, _ptr(cost), W, H, D, _ptr(labels))

    def update_W(self, wx, wy):
        self._keep += [wx, wy]
        call("cnncrf_slackprop_update_w", self._h, _ptr(wx), _ptr(wy))

    def execute(self):
        call("cnncrf_slackprop_execute", self._h)

    def LB(self):
        v = C.c_double()
        call("cnncrf_slackprop_lower_bound", self._h, C.byref(v))
        return v.value

    def get_C1(self):
        p = C.c_void_p()
        call("cnncrf_slackprop_get_c1", self._h, C.byref(p))
        return as_device_tensor(p.value, self._shape)


class _Ops:
    def __init__(self, sp):
        self._sp = sp

    def __setitem__(self, k, v):
        call("cnncrf_slackprop_set_op", self._sp._h, k.encode(), float(v))


def remap_solution(labels, disp_min, disp_step, stream=None):
    H, W = labels.shape
    out = torch.empty((H, W), device="cuda", dtype=torch.float32)
    call("cnncrf_remap_solution", _ptr(out), _ptr(labels), W, H, disp_min, disp_step, _stream_ptr(stream))
    return out


def warp_image(img_rgba, u, stream=None):
    H, W = u.shape
    out = torch.empty_like(img_rgba)
    call("cnncrf_warp_image", _ptr(out), _ptr(img_rgba), _ptr(u), W, H, _stream_ptr(stream))
    return out


def tv_fit(vol3, disp_step, lambda_census, stream=None):
    H, W, _ = vol3.shape
    qf = torch.empty((H, W, 2), device="cuda", dtype=torch.float32)
    call("cnncrf_tv_fit", _ptr(vol3), _ptr(qf), W, H, disp_step, lambda_census, _stream_ptr(stream))
    return qf


def tv_iterate(u, u0, qf, wx, wy, C_, huber_eps, disp_step, iterations, stream=None):
    """Runs the primal-dual loop (fused, several iterations per launch) on a
    copy of u with p = q = 0 at the start; returns (u, u_, p, q)."""
    H, W = u.shape
    u = u.clone()
    u_ = torch.zeros_like(u)
    p = torch.zeros((H, W, 2), device="cuda", dtype=torch.float32)
    q = torch.zeros_like(p)
    nb = C.c_size_t()
    call("cnncrf_tv_workspace_size", W, H, C.byref(nb))
    ws = torch.empty(nb.value, device="cuda", dtype=torch.uint8)
    call("cnncrf_tv_iterate", _ptr(u), _ptr(u_), _ptr(u0), _ptr(qf), _ptr(p), _ptr(q), _ptr(wx), _ptr(wy), W, H,
         C_, huber_eps, disp_step, iterations, _ptr(ws), nb.value, _stream_ptr(stream))
    return u, u_, p, q


def rgb_to_gray(img_rgba, stream=None):
    """(H, W, 4) RGBA -> (H, W) grey, .2989 R + .5870 G + .1140 B."""
    H, W, _ = img_rgba.shape
    out = torch.empty((H, W), device="cuda", dtype=torch.float32)
    call("cnncrf_rgb_to_gray", _ptr(img_rgba), _ptr(out), W, H, _stream_ptr(stream))
    return out


def census_volume(gray_ref, gray_other, filter_size, disp_min, disp_step, depth, lambda_census=1.0, stream=None):
    """Census cost volume (H, W, depth) of gray_ref against gray_other shifted by -disparity."""
    H, W = gray_ref.shape
    out = torch.empty((H, W, depth), device="cuda", dtype=torch.float32)
    call("cnncrf_census_volume", _ptr(gray_ref), _ptr(gray_other), W, H, filter_size, disp_min, disp_step, depth,
         lambda_census, _ptr(out), _stream_ptr(stream))
    return out


def edge_weights(gray, alpha, beta, lambda_reg, stream=None):
    """Image-gradient pairwise weights (wx, wy), each (H, W)."""
    H, W = gray.shape
    wx = torch.empty((H, W), device="cuda", dtype=torch.float32)
    wy = torch.empty_like(wx)
    call("cnncrf_edge_weights", _ptr(gray), W, H, alpha, beta, lambda_reg, _ptr(wx), _ptr(wy), _stream_ptr(stream))
    return wx, wy


def quad_fit_direct(u, c1, disp_min, disp_step, stream=None):
    """Sub-label refinement of the disparity map u (H, W) on the costs c1 (H, W, D); returns a new map."""
    H, W, D = c1.shape
    u = u.clone()
    call("cnncrf_quad_fit_direct", _ptr(u), _ptr(c1), W, H, D, disp_min, disp_step, _stream_ptr(stream))
    return u


def left_right_check(left, right, threshold, stream=None):
    """Left disparities where the right map agrees within threshold, else -1."""
    H, W = left.shape
    out = torch.empty_like(left)
    call("cnncrf_left_right_check", _ptr(left), _ptr(right), W, H, threshold, _ptr(out), _stream_ptr(stream))
    return out


class Stereo:
    """Stereo (stereo/stereo.h:40-133) over cnncrf_stereo_*."""

    def __init__(self, precision=L.FP32, unary=L.UNARY_NEG_SOFTMAX, topology=L.TOPO_REF,
                 feat_channels=100, pw_channels=64, ref_depth_rounding=True, crf_shape=L.RHO_STEP,
                 crf_slack=0.5, huber_eps=0.1, refine_interp=False, stream=None):
        o = StereoOptions()
        call("cnncrf_stereo_default_options", C.byref(o))
        o.precision, o.unary, o.topology = precision, unary, topology
        o.feat_channels, o.pw_channels = feat_channels, pw_channels
        o.ref_depth_rounding = 1 if ref_depth_rounding else 0
        o.crf_shape, o.crf_slack, o.huber_eps = crf_shape, crf_slack, huber_eps
        o.refine_interp = 1 if refine_interp else 0
        self._h = C.c_void_p()
        call("cnncrf_stereo_create", C.byref(self._h), C.byref(o))
        self.stream = stream
        call("cnncrf_stereo_set_stream", self._h, _stream_ptr(stream))

    def __del__(self):
        if getattr(self, "_h", None) and L._lib is not None:
            L.lib().cnncrf_stereo_destroy(self._h)
            self._h = None

    def initialize(self, width, height, disp_min, disp_step, disp_max):
        call("cnncrf_stereo_initialize", self._h, width, height, disp_min, disp_step, disp_max)
        self.W, self.H = width, height

    def set_matching_function(self, m):
        call("cnncrf_stereo_set_matching_function", self._h, m)

    def set_num_layers(self, n):
        call("cnncrf_stereo_set_num_layers", self._h, n)

    def set_parameter_file(self, base):
        call("cnncrf_stereo_set_parameter_file", self._h, None if base is None else str(base).encode())

    def set_xavier_seed(self, seed):
        call("cnncrf_stereo_set_xavier_seed", self._h, seed)

    def set_with_xy(self, v):
        call("cnncrf_stereo_set_with_xy", self._h, 1 if v else 0)

    def set_filter_size(self, fs):
        call("cnncrf_stereo_set_filter_size", self._h, fs)

    def set_color_images(self, left, right):
        """Host RGBA float arrays (H, W, 4), or CUDA tensors."""
        if isinstance(left, torch.Tensor) and left.is_cuda:
            call("cnncrf_stereo_set_color_images_device", self._h, _ptr(left), _ptr(right))
            return
        if isinstance(left, torch.Tensor):
            left, right = left.contiguous(), right.contiguous()
            call("cnncrf_stereo_set_color_images", self._h, C.c_void_p(left.data_ptr()),
                 C.c_void_p(right.data_ptr()))
            return
        l = np.ascontiguousarray(left, np.float32)
        r = np.ascontiguousarray(right, np.float32)
        call("cnncrf_stereo_set_color_images", self._h, l.ctypes.data_as(C.c_void_p), r.ctypes.data_as(C.c_void_p))

    def compute_volume(self, lr=True):
        call("cnncrf_stereo_compute_volume", self._h, 1 if lr else 0)

    def compute_slack_propagation(self, C1, C2, delta, iterations, alpha, beta, lambda_reg, lr=True):
        call("cnncrf_stereo_compute_slack_propagation", self._h, C1, C2, delta, iterations, alpha, beta,
             lambda_reg, 1 if lr else 0)

    def compute_argmax(self, lr=True):
        call("cnncrf_stereo_compute_argmax", self._h, 1 if lr else 0)

    def compute_weights(self, alpha, beta, lambda_reg, lr=True):
        call("cnncrf_stereo_compute_weights", self._h, alpha, beta, lambda_reg, 1 if lr else 0)

    def fuse_thuber_quad_fit(self, lambda_reg, C_, iterations=10, warps=2):
        call("cnncrf_stereo_fuse_thuber_quad_fit", self._h, lambda_reg, C_, iterations, warps)

    def fuse_quad_fit_direct(self):
        call("cnncrf_stereo_fuse_quad_fit_direct", self._h)

    def get_output(self, out=None):
        out = np.empty((self.H, self.W), np.float32) if out is None else out
        call("cnncrf_stereo_get_output", self._h, out.ctypes.data_as(C.c_void_p))
        return out

    def get_output_into(self, host_tensor):
        call("cnncrf_stereo_get_output", self._h, C.c_void_p(host_tensor.data_ptr()))
        return host_tensor

    def output_device(self):
        p = C.c_void_p()
        call("cnncrf_stereo_get_output_device", self._h, C.byref(p))
        return as_device_tensor(p.value, (self.H, self.W))

    def labels_device(self):
        p = C.c_void_p()
        call("cnncrf_stereo_get_labels_device", self._h, C.byref(p))
        return as_device_tensor(p.value, (self.H, self.W), torch.int32)

    def get_depth(self):
        d = C.c_int()
        call("cnncrf_stereo_get_depth", self._h, C.byref(d))
        return d.value

    def volume_device(self):
        p = C.c_void_p()
        call("cnncrf_stereo_get_volume_device", self._h, C.byref(p))
        return as_device_tensor(p.value, (self.H, self.W, self.get_depth()))

    def weights_device(self):
        a, b = C.c_void_p(), C.c_void_p()
        call("cnncrf_stereo_get_weights_device", self._h, C.byref(a), C.byref(b))
        return as_device_tensor(a.value, (self.H, self.W)), as_device_tensor(b.value, (self.H, self.W))

    def lower_bound(self):
        v = C.c_double()
        call("cnncrf_stereo_lower_bound", self._h, C.byref(v))
        return v.value

    def stage_times(self):
        a, b, c, d = C.c_float(), C.c_float(), C.c_float(), C.c_float()
        call("cnncrf_stereo_stage_times", self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d))
        return dict(cnn=a.value, corr=b.value, crf=c.value, refine=d.value)


class StereoBatch:
    """Many pairs through computeSlackPropagation at once (cnncrf_batch_*)."""

    def __init__(self, precision=L.BF16, unary=L.UNARY_ONE_MINUS_DOT, topology=L.TOPO_ALL3X3,
                 feat_channels=100, pw_channels=64, ref_depth_rounding=False, crf_shape=L.RHO_LINEAR,
                 crf_slack=0.5, matching=L.MATCH_COLORCNN_PAIRWISE, num_layers=7, with_xy=False,
                 param_base=None, seed=0, graph=False, stream=None, group_size=0, keep_volume=False):
        o = StereoOptions()
        call("cnncrf_stereo_default_options", C.byref(o))
        o.precision, o.unary, o.topology = precision, unary, topology
        o.feat_channels, o.pw_channels = feat_channels, pw_channels
        o.ref_depth_rounding = 1 if ref_depth_rounding else 0
        o.crf_shape, o.crf_slack = crf_shape, crf_slack
        self._h = C.c_void_p()
        call("cnncrf_batch_create", C.byref(self._h), C.byref(o))
        call("cnncrf_batch_set_stream", self._h, _stream_ptr(stream))
        call("cnncrf_batch_set_network", self._h, matching, num_layers, 1 if with_xy else 0,
             None if param_base is None else str(param_base).encode(), seed)
        call("cnncrf_batch_use_graph", self._h, 1 if graph else 0)
        call("cnncrf_batch_set_group_size", self._h, group_size)
        # BF16: also write the FP32 volume (else only the CRF's 16-bit copy, and volume_device() fails)
        call("cnncrf_batch_keep_volume", self._h, 1 if keep_volume else 0)
        self.shapes = []

    def __del__(self):
        if getattr(self, "_h", None) and L._lib is not None:
            L.lib().cnncrf_batch_destroy(self._h)
            self._h = None

    def add_pair(self, width, height, disp_min, disp_step, disp_max):
        i = C.c_int()
        call("cnncrf_batch_add_pair", self._h, width, height, disp_min, disp_step, disp_max, C.byref(i))
        self.shapes.append((height, width))
        return i.value

    def set_images(self, pair, left, right):
        if isinstance(left, torch.Tensor) and left.is_cuda:
            call("cnncrf_batch_set_images_device", self._h, pair, _ptr(left), _ptr(right))
            return
        if isinstance(left, torch.Tensor):
            call("cnncrf_batch_set_images", self._h, pair, C.c_void_p(left.data_ptr()), C.c_void_p(right.data_ptr()))
            return
        l = np.ascontiguousarray(left, np.float32)
        r = np.ascontiguousarray(right, np.float32)
        call("cnncrf_batch_set_images", self._h, pair, l.ctypes.data_as(C.c_void_p), r.ctypes.data_as(C.c_void_p))

    def run(self, L1, L2, delta, iterations, lambda_reg=1.0):
        call("cnncrf_batch_run", self._h, L1, L2, float(delta), iterations, lambda_reg)

    def run_host(self, lefts, rights, outs, L1, L2, delta, iterations, lambda_reg=1.0):
        """One run from host images to host disparities (cnncrf_batch_run_host):
        lefts / rights / outs are per-pair CPU tensors (page-locked ones let a
        graph replay; outs may be None); the copies overlap the other groups'
        work.  The outputs are complete once the batch's stream is synchronised
        (check())."""
        n = len(lefts)
        arr = lambda ts: (C.c_void_p * n)(*[None if t is None else t.data_ptr() for t in ts])
        hl, hr = arr(lefts), arr(rights)
        ho = None if outs is None else arr(outs)
        call("cnncrf_batch_run_host", self._h, hl, hr, ho, L1, L2, float(delta), iterations, lambda_reg)

    def autotune(self, L1, L2, delta, iterations, lambda_reg=1.0):
        """Run once, tune every group's CRF tile (see cnncrf.tuning); returns
        one dict per group: shape, pairs, tile and the measured pass times."""
        from . import tuning
        call("cnncrf_batch_autotune", self._h, L1, L2, delta, iterations, lambda_reg)
        n = C.c_int()
        call("cnncrf_batch_num_groups", self._h, C.byref(n))
        out = []
        for g in range(n.value):
            W, H, D, np_ = C.c_int(), C.c_int(), C.c_int(), C.c_int()
            call("cnncrf_batch_group_shape", self._h, g, C.byref(W), C.byref(H), C.byref(D), C.byref(np_))
            tile, found, mh, mv = tuning.get_tile(W.value, H.value, D.value, np_.value, int(delta))
            out.append(dict(W=W.value, H=H.value, D=D.value, npairs=np_.value, delta=int(delta), tile=tile,
                            found=found, ms_h=mh, ms_v=mv))
        return out

    def check(self):
        call("cnncrf_batch_check", self._h)

    def get_output(self, pair, out=None):
        H, W = self.shapes[pair]
        if out is None:
            out = np.empty((H, W), np.float32)
        ptr = C.c_void_p(out.data_ptr()) if isinstance(out, torch.Tensor) else out.ctypes.data_as(C.c_void_p)
        call("cnncrf_batch_get_output", self._h, pair, ptr)
        return out

    def labels_device(self, pair):
        p = C.c_void_p()
        call("cnncrf_batch_get_labels_device", self._h, pair, C.byref(p))
        return as_device_tensor(p.value, self.shapes[pair], torch.int32)

    def output_device(self, pair):
        p = C.c_void_p()
        call("cnncrf_batch_get_output_device", self._h, pair, C.byref(p))
        return as_device_tensor(p.value, self.shapes[pair])

    def volume_device(self, pair):
        p, d = C.c_void_p(), C.c_int()
        call("cnncrf_batch_get_volume_device", self._h, pair, C.byref(p), C.byref(d))
        return as_device_tensor(p.value, self.shapes[pair] + (d.value,))

    def lower_bound(self, pair):
        v = C.c_double()
        call("cnncrf_batch_lower_bound", self._h, pair, C.byref(v))
        return v.value
