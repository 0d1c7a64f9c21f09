"""Error metrics of the reference's evaluation scripts.

KITTI 2015 (eval/compute_numbers_kitti.py:6-17):
  disparity maps are 16-bit PNGs holding d * 256; the value 0 marks a pixel
  without ground truth and is read as -1.  A pixel is wrong when the ground
  truth is valid (gt > 0), |d - gt| > 3 px and |d - gt| / |gt| > 5 %; the error
  of an image is wrong pixels / valid pixels, and the score of a method is the
  mean over images, against the occluded ("disp_occ_0") and the non-occluded
  ("disp_noc_0") ground truth.

Middlebury 2014 (eval/compute_numbers_middlebury.py:31-60): the bad-x rate of
each training image comes from the MiddEval3 SDK's runevalF (threshold 4 px at
quarter resolution, 2 px at half); the score is the average weighted by the
SDK's per-image weights, 0.5 for the five images the benchmark down-weights.
runevalF is not part of the reference; middlebury_bad restates a bad-x rate
over pixels with finite ground truth (MiddEval3 marks unknown disparities as
inf), counting non-finite predictions as bad.

    python -m cnncrf.evaluation kitti PRED_DIR GT_OCC_DIR GT_NOC_DIR
"""
import os
import sys

import numpy as np

from . import imageio

KITTI_TAU = (3.0, 0.05)  # eval/compute_numbers_kitti.py:25-26
MIDDLEBURY_TRAINING_WEIGHTS = np.array([1, 1, 1, 1, 1, 1, 0.5, 1, 0.5, 0.5, 1, 1, 0.5, 1, 0.5])
MIDDLEBURY_THRESHOLD = {"Q": 4.0, "H": 2.0}


def quantize_png16(disp):
    """A disparity map as it reads back from its 16-bit PNG: floor(max(d*256, 0)) / 256, 0 -> -1."""
    d = imageio.disparity_to_png16(disp).astype(np.float64) / 256.0
    d[d == 0] = -1.0
    return d


def read_disp16(path):
    """readdisp16: the PNG's 16-bit values / 256, 0 -> -1."""
    raw = np.rint(imageio.read_png(path)[..., 0].astype(np.float64) * 65535.0)
    d = raw / 256.0
    d[d == 0] = -1.0
    return d


def kitti_error(pred, gt, tau=KITTI_TAU):
    """computeError: fraction of valid ground-truth pixels that are wrong."""
    pred = np.asarray(pred, np.float64)
    gt = np.asarray(gt, np.float64)
    valid = gt > 0
    n = int(valid.sum())
    if n == 0:
        return float("nan")
    diff = np.abs(pred - gt)
    with np.errstate(divide="ignore", invalid="ignore"):
        wrong = valid & (diff > tau[0]) & ((diff / np.abs(gt)) > tau[1])
    return float(wrong.sum()) / n


def kitti_numbers(pred_dir, gt_occ_dir, gt_noc_dir, tau=KITTI_TAU):
    """(mean error against occluded ground truth, mean against non-occluded) over the PNGs of pred_dir."""
    files = sorted(f for f in os.listdir(pred_dir) if ".png" in f)
    if not files:
        return float("nan"), float("nan")
    occ, noc = [], []
    for f in files:
        pred = read_disp16(os.path.join(pred_dir, f))
        occ.append(kitti_error(pred, read_disp16(os.path.join(gt_occ_dir, f)), tau))
        noc.append(kitti_error(pred, read_disp16(os.path.join(gt_noc_dir, f)), tau))
    return float(np.mean(occ)), float(np.mean(noc))


def middlebury_bad(pred, gt, threshold, mask=None):
    """Percentage of pixels with finite ground truth (inside mask, if given) whose error exceeds threshold."""
    pred = np.asarray(pred, np.float64)
    gt = np.asarray(gt, np.float64)
    valid = np.isfinite(gt)
    if mask is not None:
        valid &= np.asarray(mask, bool)
    n = int(valid.sum())
    if n == 0:
        return float("nan")
    with np.errstate(invalid="ignore"):
        bad = valid & ~(np.abs(pred - gt) <= threshold)
    return 100.0 * float(bad.sum()) / n


def middlebury_weighted(badx, weights=MIDDLEBURY_TRAINING_WEIGHTS):
    """(plain mean, weighted mean) of the per-image bad-x rates."""
    badx = np.asarray(badx, np.float64)
    w = np.asarray(weights, np.float64)[: len(badx)]
    return float(badx.mean()), float((w * badx).sum() / w.sum())


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 4 or argv[0] != "kitti":
        sys.stderr.write("usage: python -m cnncrf.evaluation kitti PRED_DIR GT_OCC_DIR GT_NOC_DIR\n")
        return 1
    occ, noc = kitti_numbers(*argv[1:])
    print("%-13s %10s %14s" % ("Method", "All", "Non-Occluded"))
    print("%-13s %10.4f %14.4f" % (os.path.basename(os.path.normpath(argv[1])), occ, noc))
    return 0


if __name__ == "__main__":
    sys.exit(main())
