"""Generate the golden fixtures of tests/golden/ (run once, in a checkout that
has the reference tree; the outputs are committed).

Pins the CNN part of the oracle against an INDEPENDENT float64
implementation of the operators the reference calls, built from library
ops rather than from the oracle's code:
  - mirror padding      numpy.pad(mode="symmetric")   (cudaAddressModeMirror,
                                                        stereo/stereo.cu:879-911)
  - normalisation       numpy mean / population std over the padded image
                                                       (stereo/utils.cu:169-237)
  - convolution         torch.nn.functional.conv2d with the kernel flipped
                        (CUDNN_CONVOLUTION, stereo/operators/convolution.cpp:107-108)
                        + bias + tanh
  - correlation         numpy over the disparity list (stereo/operators/
                        stereocorrelation.cu:111-142), 0 where w - d < 0
  - softmax, negate     torch.softmax over D (stereo/operators/softmax.cpp:30-38)
  - pairwise net        crop by 2, conv3x3 tanh, conv3x3 tanh, conv1x1, abs
                        (stereo/stereonet.cpp:159-167,401)

Inputs: a 64x48 crop of the reference's sample pair data/im0.png /
data/im1.png and the shipped weights
data/parameters/kitti-2015/7-layer/cnn+crf+full/params.npz (copied here as a
fixture).  The CRF solver has no reference to pin against (absent
dependency); see cnncrf_oracle.h.

usage: python tests/golden/make_golden.py REFERENCE_ROOT
(REFERENCE_ROOT: the directory of the reference checkout, which holds data/)
"""
import os
import shutil
import struct
import sys
import zlib

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
CROP = dict(x=300, y=220, w=64, h=48)
D = 16


def read_png(path):
    """Minimal PNG decoder (8-bit RGB / RGBA, non-interlaced)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, ctype, _, _, inter = hdr
    assert depth == 8 and inter == 0 and ctype in (2, 6)
    ch = 3 if ctype == 2 else 4
    raw = zlib.decompress(idat)
    stride = w * ch
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        cur = np.zeros(stride, np.int32)
        for i in range(stride):
            a = cur[i - ch] if i >= ch else 0
            b = prev[i]
            c = prev[i - ch] if i >= ch else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) // 2
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            cur[i] = (line[i] + p) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, ch)


def rgba_crop(img):
    c = img[CROP["y"]:CROP["y"] + CROP["h"], CROP["x"]:CROP["x"] + CROP["w"], :3]
    a = np.ones(c.shape[:2] + (4,), np.float32)
    a[..., :3] = c.astype(np.float32) / 255.0
    return a


def conv(x, w, b, act):
    """x: (C, H, W) float64; true convolution (flipped kernel), valid."""
    t = torch.nn.functional.conv2d(torch.tensor(x)[None], torch.tensor(w, dtype=torch.float64).flip(2, 3),
                                   None if b is None else torch.tensor(b, dtype=torch.float64))[0]
    if act == "tanh":
        t = torch.tanh(t)
    elif act == "abs":
        t = t.abs()
    return t.numpy()


def reference_semantics(left, right, params, num_layers=7, disp_min=0.0, disp_max=D - 1.0):
    pad = 4  # 7 layers: 3x3 + 6 x 2x2 (stereo/stereo.cpp:211-213)
    def prep(img):
        p = np.pad(img[..., :3].astype(np.float64), ((pad, pad), (pad, pad), (0, 0)), mode="symmetric")
        p = p.transpose(2, 0, 1)
        out = np.empty_like(p)
        for c in range(3):
            m = p[c].mean()
            z = p[c] - m
            out[c] = z / np.sqrt((z * z).mean())
        return out
    nl, nr = prep(left), prep(right)
    fl, fr = nl, nr
    for l in range(num_layers):
        fl = conv(fl, params[2 * l], params[2 * l + 1], "tanh")
        fr = conv(fr, params[2 * l], params[2 * l + 1], "tanh")
    C, H, W = fl.shape
    disps = np.arange(disp_min, disp_max + 1.0)
    vol = np.zeros((H, W, len(disps)))
    for k, d in enumerate(disps):
        d = int(d)
        if d == 0:
            vol[:, :, k] = (fl * fr).sum(0)
        else:
            vol[:, d:, k] = (fl[:, :, d:] * fr[:, :, :-d]).sum(0)
    unary = -torch.softmax(torch.tensor(vol), dim=2).numpy()
    base = 2 * num_layers
    pin = nl[:, 2:-2, 2:-2]
    t = conv(pin, params[base], params[base + 1], "tanh")
    t = conv(t, params[base + 2], params[base + 3], "tanh")
    pw = conv(t, params[base + 4], None, "abs")
    return vol, unary, pw


def main(ref_root):
    src = os.path.join(ref_root, "data/parameters/kitti-2015/7-layer/cnn+crf+full/params.npz")
    dst = os.path.join(HERE, "kitti7_full_params.npz")
    shutil.copyfile(src, dst)
    z = np.load(dst)
    params = [z["arr_%d" % i] for i in range(19)]
    left = rgba_crop(read_png(os.path.join(ref_root, "data/im0.png")))
    right = rgba_crop(read_png(os.path.join(ref_root, "data/im1.png")))
    vol, unary, pw = reference_semantics(left, right, params)
    np.save(os.path.join(HERE, "crop_left_rgba.npy"), left)
    np.save(os.path.join(HERE, "crop_right_rgba.npy"), right)
    np.save(os.path.join(HERE, "golden_corr_f64.npy"), vol.astype(np.float64))
    np.save(os.path.join(HERE, "golden_unary_f64.npy"), unary.astype(np.float64))
    np.save(os.path.join(HERE, "golden_pairwise_f64.npy"), pw.astype(np.float64))
    print("wrote fixtures:", left.shape, vol.shape, pw.shape)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_ROOT")
    main(sys.argv[1])
