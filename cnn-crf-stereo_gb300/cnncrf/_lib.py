"""ctypes loader of libcnncrf.so (the C ABI declared in include/cnncrf.h).

The library is the product: every compute call goes through it.  There is no
fallback -- if the shared library is missing, importing a compute entry point
raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcnncrf.so")

OK, EINVAL, ESHAPE, ENOMEM, ECUDA, ETIMEOUT, EIO, ESTATE, EUNSUPPORTED = range(9)
STATUS_NAMES = ["OK", "EINVAL", "ESHAPE", "ENOMEM", "ECUDA", "ETIMEOUT", "EIO", "ESTATE", "EUNSUPPORTED"]

# enums (include/cnncrf.h)
MATCH_COLORCNN, MATCH_GRAYCNN, MATCH_CONCATCNN, MATCH_GRAYCNN_PAIRWISE, MATCH_COLORCNN_PAIRWISE, \
    MATCH_CONCATCNN_PAIRWISE, MATCH_CENSUS, MATCH_LOAD = range(8)
FP32, BF16 = 0, 1
UNARY_NEG_SOFTMAX, UNARY_ONE_MINUS_DOT = 0, 1
TOPO_REF, TOPO_ALL3X3, TOPO_CONCAT = 0, 1, 2
# ConcatStereoNet's growth rate per depth (the library's table)
CONCAT_GROWTH = {3: 33, 5: 20, 7: 14, 10: 10, 15: 7, 20: 5, 25: 4, 33: 3, 50: 2, 100: 1}
RHO_STEP, RHO_LINEAR = 0, 1


class CnnCrfError(RuntimeError):
    def __init__(self, status, msg):
        self.status = status
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__("%s: %s" % (name, msg))


class NetDesc(C.Structure):
    _fields_ = [("num_layers", C.c_int), ("topology", C.c_int), ("in_channels", C.c_int),
                ("feat_channels", C.c_int), ("unary", C.c_int), ("precision", C.c_int),
                ("with_pairwise", C.c_int), ("pw_channels", C.c_int)]


class CrfOptions(C.Structure):
    _fields_ = [("L1", C.c_float), ("L2", C.c_float), ("delta", C.c_float), ("total_it", C.c_int),
                ("shape", C.c_int), ("slack", C.c_float)]


class CrfTile(C.Structure):
    _fields_ = [("ring_h", C.c_int), ("chains_per_cta_h", C.c_int), ("ring_v", C.c_int),
                ("chains_per_cta_v", C.c_int)]


class TrainDesc(C.Structure):
    _fields_ = [("num_layers", C.c_int), ("topology", C.c_int), ("feat_channels", C.c_int), ("pw_channels", C.c_int),
                ("disp_min", C.c_float), ("disp_step", C.c_float), ("disp_max", C.c_float), ("lam", C.c_float),
                ("L1", C.c_float), ("L2", C.c_float), ("delta", C.c_int), ("crf_shape", C.c_int),
                ("crf_slack", C.c_float), ("crf_iters", C.c_int), ("mean_loss", C.c_int), ("precision", C.c_int),
                ("checkpoint_every", C.c_int), ("tc_wgrad", C.c_int), ("tc_dgrad", C.c_int)]


class StereoOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("unary", C.c_int), ("topology", C.c_int),
                ("feat_channels", C.c_int), ("pw_channels", C.c_int),
                ("ref_depth_rounding", C.c_int), ("crf_shape", C.c_int), ("crf_slack", C.c_float),
                ("huber_eps", C.c_float), ("refine_interp", C.c_int)]


vp = C.c_void_p
i32 = C.c_int
f32 = C.c_float
PROTOS = {
    "cnncrf_last_error": ([], C.c_char_p),
    "cnncrf_abi_version": ([], i32),
    "cnncrf_set_conv_pairs": ([i32], i32),
    "cnncrf_get_conv_pairs": ([C.POINTER(i32)], i32),
    "cnncrf_net_create": ([C.POINTER(vp), C.POINTER(NetDesc), i32, i32, i32], i32),
    "cnncrf_net_destroy": ([vp], i32),
    "cnncrf_net_set_stream": ([vp, vp], i32),
    "cnncrf_net_init": ([vp, f32, f32, f32, i32, vp, vp], i32),
    "cnncrf_net_set_all_params": ([vp, C.c_char_p], i32),
    "cnncrf_net_set_param": ([vp, i32, vp, C.POINTER(C.c_int64), i32], i32),
    "cnncrf_net_num_params": ([vp, C.POINTER(i32)], i32),
    "cnncrf_net_param_shape": ([vp, i32, C.POINTER(C.c_int64), C.POINTER(i32)], i32),
    "cnncrf_net_init_xavier": ([vp, C.c_uint64], i32),
    "cnncrf_net_set_disparities": ([vp, f32, f32, f32, vp], i32),
    "cnncrf_net_num_disparities": ([vp, C.POINTER(i32)], i32),
    "cnncrf_net_predict": ([vp, vp, vp, C.POINTER(vp)], i32),
    "cnncrf_net_pairwise": ([vp, C.POINTER(vp)], i32),
    "cnncrf_net_features": ([vp, i32, vp], i32),
    "cnncrf_net_padding": ([vp, C.POINTER(i32)], i32),
    "cnncrf_correlation_forward": ([vp, vp, vp, vp, i32, i32, i32, i32, i32, vp], i32),
    "cnncrf_crf_default_options": ([C.POINTER(CrfOptions)], i32),
    "cnncrf_crf_workspace_size": ([i32, i32, i32, C.POINTER(C.c_size_t)], i32),
    "cnncrf_crf_solve": ([vp, vp, vp, i32, i32, i32, C.POINTER(CrfOptions), vp, C.POINTER(C.c_double), vp,
                          C.c_size_t, vp], i32),
    "cnncrf_crf_solve_static": ([vp, vp, vp, i32, i32, i32, C.POINTER(CrfOptions), vp, C.POINTER(C.c_double),
                                 vp], i32),
    "cnncrf_crf_tuning_set": ([i32, i32, i32, i32, i32, C.POINTER(CrfTile)], i32),
    "cnncrf_crf_tuning_get": ([i32, i32, i32, i32, i32, C.POINTER(CrfTile), C.POINTER(i32), C.POINTER(f32),
                               C.POINTER(f32)], i32),
    "cnncrf_crf_tuning_clear": ([], i32),
    "cnncrf_conv_tuning_count": ([C.POINTER(i32)], i32),
    "cnncrf_conv_tuning_get": ([i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(f32)], i32),
    "cnncrf_conv_tuning_clear": ([], i32),
    "cnncrf_crf_tuning_count": ([C.POINTER(i32)], i32),
    "cnncrf_crf_tuning_save": ([C.c_char_p], i32),
    "cnncrf_crf_tuning_load": ([C.c_char_p], i32),
    "cnncrf_crf_autotune": ([vp, vp, vp, i32, i32, i32, C.POINTER(CrfOptions), vp, C.c_size_t, vp], i32),
    "cnncrf_slackprop_create": ([C.POINTER(vp)], i32),
    "cnncrf_slackprop_destroy": ([vp], i32),
    "cnncrf_slackprop_set_stream": ([vp, vp], i32),
    "cnncrf_slackprop_init": ([vp, vp, i32, i32, i32, vp], i32),
    "cnncrf_slackprop_set_op": ([vp, C.c_char_p, C.c_double], i32),
    "cnncrf_slackprop_update_w": ([vp, vp, vp], i32),
    "cnncrf_slackprop_execute": ([vp], i32),
    "cnncrf_slackprop_lower_bound": ([vp, C.POINTER(C.c_double)], i32),
    "cnncrf_slackprop_get_c1": ([vp, C.POINTER(vp)], i32),
    "cnncrf_remap_solution": ([vp, vp, i32, i32, f32, f32, vp], i32),
    "cnncrf_warp_image": ([vp, vp, vp, i32, i32, vp], i32),
    "cnncrf_tv_fit": ([vp, vp, i32, i32, f32, f32, vp], i32),
    "cnncrf_tv_workspace_size": ([i32, i32, C.POINTER(C.c_size_t)], i32),
    "cnncrf_tv_iterate": ([vp, vp, vp, vp, vp, vp, vp, vp, i32, i32, f32, f32, f32, i32, vp, C.c_size_t, vp], i32),
    "cnncrf_rgb_to_gray": ([vp, vp, i32, i32, vp], i32),
    "cnncrf_census_volume": ([vp, vp, i32, i32, i32, f32, f32, i32, f32, vp, vp], i32),
    "cnncrf_edge_weights": ([vp, i32, i32, f32, f32, f32, vp, vp, vp], i32),
    "cnncrf_quad_fit_direct": ([vp, vp, i32, i32, i32, f32, f32, vp], i32),
    "cnncrf_left_right_check": ([vp, vp, i32, i32, f32, vp, vp], i32),
    "cnncrf_stereo_default_options": ([C.POINTER(StereoOptions)], i32),
    "cnncrf_stereo_create": ([C.POINTER(vp), C.POINTER(StereoOptions)], i32),
    "cnncrf_stereo_destroy": ([vp], i32),
    "cnncrf_stereo_set_stream": ([vp, vp], i32),
    "cnncrf_stereo_initialize": ([vp, i32, i32, f32, f32, f32], i32),
    "cnncrf_stereo_set_matching_function": ([vp, i32], i32),
    "cnncrf_stereo_set_num_layers": ([vp, i32], i32),
    "cnncrf_stereo_set_parameter_file": ([vp, C.c_char_p], i32),
    "cnncrf_stereo_set_xavier_seed": ([vp, C.c_uint64], i32),
    "cnncrf_stereo_set_with_xy": ([vp, i32], i32),
    "cnncrf_stereo_set_color_images": ([vp, vp, vp], i32),
    "cnncrf_stereo_set_color_images_device": ([vp, vp, vp], i32),
    "cnncrf_stereo_compute_volume": ([vp, i32], i32),
    "cnncrf_stereo_compute_slack_propagation": ([vp, f32, f32, f32, i32, f32, f32, f32, i32], i32),
    "cnncrf_stereo_set_filter_size": ([vp, i32], i32),
    "cnncrf_stereo_compute_weights": ([vp, f32, f32, f32, i32], i32),
    "cnncrf_stereo_fuse_quad_fit_direct": ([vp], i32),
    "cnncrf_stereo_compute_argmax": ([vp, i32], i32),
    "cnncrf_stereo_fuse_thuber_quad_fit": ([vp, f32, f32, i32, i32], i32),
    "cnncrf_stereo_get_output": ([vp, vp], i32),
    "cnncrf_stereo_get_output_device": ([vp, C.POINTER(vp)], i32),
    "cnncrf_stereo_get_labels_device": ([vp, C.POINTER(vp)], i32),
    "cnncrf_stereo_get_volume_device": ([vp, C.POINTER(vp)], i32),
    "cnncrf_stereo_get_weights_device": ([vp, C.POINTER(vp), C.POINTER(vp)], i32),
    "cnncrf_stereo_get_depth": ([vp, C.POINTER(i32)], i32),
    "cnncrf_stereo_lower_bound": ([vp, C.POINTER(C.c_double)], i32),
    "cnncrf_stereo_stage_times": ([vp, C.POINTER(f32), C.POINTER(f32), C.POINTER(f32), C.POINTER(f32)], i32),
    "cnncrf_batch_create": ([C.POINTER(vp), C.POINTER(StereoOptions)], i32),
    "cnncrf_batch_destroy": ([vp], i32),
    "cnncrf_batch_set_stream": ([vp, vp], i32),
    "cnncrf_batch_set_network": ([vp, i32, i32, i32, C.c_char_p, C.c_uint64], i32),
    "cnncrf_batch_set_group_size": ([vp, i32], i32),
    "cnncrf_batch_add_pair": ([vp, i32, i32, f32, f32, f32, C.POINTER(i32)], i32),
    "cnncrf_batch_num_pairs": ([vp, C.POINTER(i32)], i32),
    "cnncrf_batch_set_images": ([vp, i32, vp, vp], i32),
    "cnncrf_batch_set_images_device": ([vp, i32, vp, vp], i32),
    "cnncrf_batch_use_graph": ([vp, i32], i32),
    "cnncrf_batch_run": ([vp, f32, f32, f32, i32, f32], i32),
    "cnncrf_batch_keep_volume": ([vp, i32], i32),
    "cnncrf_batch_run_host": ([vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), f32, f32, f32, i32, f32], i32),
    "cnncrf_batch_get_output": ([vp, i32, vp], i32),
    "cnncrf_batch_get_output_device": ([vp, i32, C.POINTER(vp)], i32),
    "cnncrf_batch_get_labels_device": ([vp, i32, C.POINTER(vp)], i32),
    "cnncrf_batch_get_volume_device": ([vp, i32, C.POINTER(vp), C.POINTER(i32)], i32),
    "cnncrf_batch_lower_bound": ([vp, i32, C.POINTER(C.c_double)], i32),
    "cnncrf_batch_check": ([vp], i32),
    "cnncrf_batch_autotune": ([vp, f32, f32, f32, i32, f32], i32),
    "cnncrf_batch_num_groups": ([vp, C.POINTER(i32)], i32),
    "cnncrf_batch_group_shape": ([vp, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)], i32),
    "cnncrf_train_default_desc": ([C.POINTER(TrainDesc)], i32),
    "cnncrf_train_create": ([C.POINTER(vp), C.POINTER(TrainDesc), i32, i32, i32], i32),
    "cnncrf_train_destroy": ([vp], i32),
    "cnncrf_train_set_stream": ([vp, vp], i32),
    "cnncrf_train_num_params": ([vp, C.POINTER(i32)], i32),
    "cnncrf_train_param_shape": ([vp, i32, C.POINTER(C.c_int64), C.POINTER(i32)], i32),
    "cnncrf_train_init_xavier": ([vp, C.c_uint64], i32),
    "cnncrf_train_set_param": ([vp, i32, vp, C.c_size_t], i32),
    "cnncrf_train_get_param": ([vp, i32, vp, C.c_size_t], i32),
    "cnncrf_train_get_grad": ([vp, i32, vp, C.c_size_t], i32),
    "cnncrf_train_forward": ([vp, vp, vp], i32),
    "cnncrf_train_outputs": ([vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(i32)], i32),
    "cnncrf_train_hinge": ([vp, vp, C.POINTER(C.c_double), vp], i32),
    "cnncrf_train_hinge_grads": ([vp, C.POINTER(vp), C.POINTER(vp)], i32),
    "cnncrf_train_autotune": ([vp], i32),
    "cnncrf_train_backward": ([vp, vp, vp], i32),
    "cnncrf_train_sgd": ([vp, f32, f32], i32),
    "cnncrf_train_step": ([vp, vp, vp, vp, f32, f32, C.POINTER(C.c_double)], i32),
    "cnncrf_train_save": ([vp, C.c_char_p], i32),
    "cnncrf_train_load": ([vp, C.c_char_p], i32),
    "cnncrf_npz_read": ([C.c_char_p, C.c_char_p, C.POINTER(C.c_int64), C.POINTER(i32), vp, C.c_size_t], i32),
    "cnncrf_npz_write": ([C.c_char_p, i32, C.POINTER(C.c_char_p), C.POINTER(vp), C.POINTER(C.c_int64),
                          C.POINTER(i32)], i32),
    "cnncrf_kernel_launches": ([C.POINTER(C.c_uint64)], i32),
    "cnncrf_profile_enable": ([i32], i32),
    "cnncrf_profile_reset": ([], i32),
    "cnncrf_profile_query": ([C.c_char_p, C.POINTER(i32), C.POINTER(C.c_double)], i32),
    "cnncrf_profile_kernels": ([C.c_char_p, C.c_size_t], i32),
    "cnncrf_selftest_bounded_wait": ([i32, i32, vp], i32),
}

_lib = None


def lib():
    """Load libcnncrf.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libcnncrf.so not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in PROTOS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(status):
    if status != OK:
        raise CnnCrfError(status, lib().cnncrf_last_error().decode())
    return status


def call(name, *args):
    return check(getattr(lib(), name)(*args))


def kernel_launches():
    n = C.c_uint64()
    call("cnncrf_kernel_launches", C.byref(n))
    return n.value


def profile_enable(on=True):
    call("cnncrf_profile_enable", 1 if on else 0)


def profile_reset():
    call("cnncrf_profile_reset")


def profile_query(kernel):
    n, t = C.c_int(), C.c_double()
    call("cnncrf_profile_query", kernel.encode(), C.byref(n), C.byref(t))
    return n.value, t.value


def profile_kernels():
    buf = C.create_string_buffer(8192)
    call("cnncrf_profile_kernels", buf, 8192)
    return [k for k in buf.value.decode().split("\n") if k]


def selftest_bounded_wait(polls, arrive, stream=None):
    """Run the bounded-wait probe; returns the raw status (OK, or ETIMEOUT when
    the wait on a barrier nothing completes gave up) without raising."""
    return lib().cnncrf_selftest_bounded_wait(int(polls), 1 if arrive else 0, stream)


def npz_read(path, key):
    """Member `key` of an npz archive as a float32 array, through the library's own reader."""
    s = (C.c_int64 * 4)()
    nd = C.c_int()
    call("cnncrf_npz_read", os.fsencode(path), key.encode(), s, C.byref(nd), None, 0)
    out = np.empty(tuple(s[k] for k in range(nd.value)), np.float32)
    call("cnncrf_npz_read", os.fsencode(path), key.encode(), s, C.byref(nd), out.ctypes.data_as(C.c_void_p),
         out.size)
    return out


def npz_write(path, arrays):
    """Write {key: array} as an uncompressed npz through the library's own writer (float32, C order)."""
    keys = list(arrays)
    data = [np.array(arrays[k], np.float32, order="C") for k in keys]  # keeps 0-d arrays 0-d
    if any(a.ndim > 4 for a in data):
        raise ValueError("npz_write: at most 4 dimensions")
    n = len(keys)
    ks = (C.c_char_p * max(n, 1))(*[k.encode() for k in keys])
    ps = (C.c_void_p * max(n, 1))(*[a.ctypes.data for a in data])
    shp = (C.c_int64 * max(4 * n, 1))()
    nds = (C.c_int * max(n, 1))()
    for i, a in enumerate(data):
        nds[i] = a.ndim
        for j, d in enumerate(a.shape):
            shp[4 * i + j] = d
    call("cnncrf_npz_write", os.fsencode(path), n, ks, ps, shp, nds)
