"""stereo_img on the GB300 library (stereo/stereo_img.cpp:44-221).

    python -m cnncrf.cli im0.png im1.png [--config-file f.cfg] [--option value ...]

Same options, defaults and precedence as the reference (command line over the
config file over the defaults), same outputs per inference mode:

  CRF     <output-file>.png (16-bit, disparity * 256), <output-file>.pfm and the
          pairwise weights <output-file>_wx.pfm / _wy.pfm (getWx / getWy)
  ARGMAX  <output-file>.png and <output-file>.pfm
  NONE    <output-file>.npy (H x W x D volume), <output-file>_wx.npy / _wy.npy

Options beyond the reference's: --precision FP32|BF16 (default FP32, the
reference's arithmetic) and --xavier-seed N (Xavier weights from a seed instead
of the parameter file).  The VTK volume dump of NONE (ITK) is not written.
Errors are reported with the library's message and exit status 1 instead of
the reference's exit(-1).
"""
import sys

import numpy as np

from . import config, imageio
from ._lib import (BF16, FP32, MATCH_CENSUS, MATCH_COLORCNN, MATCH_COLORCNN_PAIRWISE, MATCH_LOAD, CnnCrfError)

EXTRA = {"precision": (str, "FP32"), "xavier-seed": (int, -1)}


def _split_extras(argv):
    """Take the options that are not the reference's out of argv."""
    rest, extra = [], {}
    i = 0
    while i < len(argv):
        key = argv[i][2:] if argv[i].startswith("--") else None
        if key is not None and key.split("=", 1)[0] in EXTRA:
            k, _, v = key.partition("=")
            if not _:
                i += 1
                v = argv[i]
            extra[k] = EXTRA[k][0](v)
        else:
            rest.append(argv[i])
        i += 1
    full = {k: d for k, (_, d) in EXTRA.items()}
    full.update(extra)
    return rest, full


def _weights(st, alpha, beta):
    """Stereo::getWx / getWy (stereo/stereo.cpp:425-437): with alpha > 0 the
    edge weights of the left image are recomputed at lambda 1; otherwise the
    current pairwise buffers (the pairwise net's, lambda-scaled after a CRF)."""
    if alpha > 0:
        st.compute_weights(alpha, beta, 1.0, True)
    wx, wy = st.weights_device()
    return wx.cpu().numpy(), wy.cpu().numpy()


def run(argv):
    rest, extra = _split_extras(list(argv))
    o = config.resolve(rest)
    if o.get("im0") is None or o.get("im1") is None:
        sys.stderr.write("usage: python -m cnncrf.cli im0 im1 [--option value ...]\n")
        return 1
    import torch
    from .api import Stereo
    torch.cuda.set_device(o["gpu"])
    left, right = imageio.read_png(o["im0"]), imageio.read_png(o["im1"])
    H, W = left.shape[:2]
    if right.shape != left.shape:
        sys.stderr.write("im0 and im1 differ in size\n")
        return 1
    precision = {"FP32": FP32, "BF16": BF16}[extra["precision"].upper()]
    st = Stereo(precision=precision)
    st.set_with_xy(o["with-xy"])
    st.initialize(W, H, o["disp-min"], o["disp-step"], o["disp-max"])
    alpha, beta = o["alpha"], o["beta"]
    m = o["matching"]
    if m in ("COLORCNN", "COLORPAIR"):
        if m == "COLORPAIR":
            alpha = 0.0  # to ignore the edge term (stereo/stereo_img.cpp:152)
        st.set_num_layers(o["num-layers"])
        if extra["xavier-seed"] >= 0:
            st.set_xavier_seed(extra["xavier-seed"])
        else:
            st.set_parameter_file(o["parameter-file"])
        st.set_matching_function(MATCH_COLORCNN_PAIRWISE if m == "COLORPAIR" else MATCH_COLORCNN)
    elif m == "LOAD":
        st.set_matching_function(MATCH_LOAD)
        vol = np.load(o["volume"], allow_pickle=False).astype(np.float32)
        if vol.shape[:2] != (H, W) or vol.shape[2] != st.get_depth():
            sys.stderr.write("volume %s has shape %s, expected (%d, %d, %d)\n"
                             % (o["volume"], vol.shape, H, W, st.get_depth()))
            return 1
        st.volume_device().copy_(torch.from_numpy(np.ascontiguousarray(vol)).cuda())
    elif m == "CENSUS":
        st.set_matching_function(MATCH_CENSUS)
        st.set_filter_size(o["filter-size"])
    else:
        sys.stderr.write("Unknown matching function (%s)\n" % m)
        return 1
    st.set_color_images(left, right)
    out = o["output-file"]
    inf = o["inference"]
    if inf == "CRF":
        st.compute_slack_propagation(o["L1"], o["L2"], o["delta"], o["crf-iterations"], alpha, beta,
                                     o["lambda"], True)
        ref = o["refinement"]
        if ref == "THuberQuad":
            st.fuse_thuber_quad_fit(o["lambda"], o["L2"], o["ref-iterations"], o["warps"])
        elif ref == "QuadDirect":
            st.fuse_quad_fit_direct()
        elif ref != "NONE":
            sys.stderr.write("Unknown refinement method (%s)\n" % ref)
            return 1
        disp = st.get_output()
        imageio.write_png16(out + ".png", disp)
        imageio.write_pfm(out + ".pfm", disp)
        wx, wy = _weights(st, alpha, beta)
        imageio.write_pfm(out + "_wx.pfm", wx)
        imageio.write_pfm(out + "_wy.pfm", wy)
    elif inf == "ARGMAX":
        st.compute_argmax(True)
        disp = st.get_output()
        imageio.write_png16(out + ".png", disp)
        imageio.write_pfm(out + ".pfm", disp)
    elif inf == "NONE":
        st.compute_volume(True)
        wx, wy = _weights(st, alpha, beta)
        imageio.write_npy(out + "_wx.npy", wx)
        imageio.write_npy(out + "_wy.npy", wy)
        imageio.write_npy(out + ".npy", st.volume_device().cpu().numpy())
    else:
        sys.stderr.write("Unknown inference method (%s)\n" % inf)
        return 1
    return 0


def main(argv=None):
    try:
        return run(sys.argv[1:] if argv is None else argv)
    except (CnnCrfError, KeyError, ValueError, OSError) as e:
        sys.stderr.write("stereo_img: %s\n" % e)
        return 1


if __name__ == "__main__":
    sys.exit(main())
