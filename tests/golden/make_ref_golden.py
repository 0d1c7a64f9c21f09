"""Writes tests/golden/ref_kernels.npz: the outputs of the REFERENCE'S OWN CUDA
kernels (compiled unchanged by oracle/build_ref.py, launched as the
reference's host code launches them by oracle/ref_host.cpp) on small seeded
inputs, for the hot path's non-CRF stages:

  correlation  kCorrelation_NHWC / kCorrelation_NHWC_interpolation
               (stereo/operators/stereocorrelation.cu:33-142): an integer, a
               half-step, a negative and the refinement (-1/4, 0, 1/4) list
  pad          padding_color_kernel (stereo/stereo.cu:895-911), mirror texture
  gray         rgb_to_gray_kernel (stereo/stereo.cu:853-863)
  census       cost_vol_census_kernel (stereo/stereo.cu:306-346), linear texture
  argmin       arg_min_kernel (stereo/stereo.cu:348-370)
  remap        remapsolution_kernel (stereo/stereo.cu:841-850)
  warp         warp_image_kernel, RGBA, point texture (stereo/stereo.cu:830-839)
  fit          do_fitting_kernel (stereo/stereo.cu:419-442)
  tv           ttvqf_primal_kernel + thuberqf_dual_kernel, the loop of
               stereo/stereo.cu:1133-1166 (Huber parameter 0.1 as compiled)
  lrcheck      leftrightcheck_kernel (stereo/stereo.cu:803-817)
  quadfit      do_fitting_kernel_volume + do_argmin_kernel_volume
               (stereo/stereo.cu:913-942)

The inputs are stored beside the outputs.  Needs a CUDA GPU and the module
oracle/_ref/refkernels.fatbin (built from the reference tree by
oracle/build_ref.py, and by oracle/build_oracle.py's build where that tree
exists).

usage: python tests/golden/make_ref_golden.py [OUT.npz]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def inputs():
    """The seeded inputs (also used by the tests to rebuild the lists)."""
    rng = np.random.default_rng(20240)
    x = {}
    Cc, H, W = 48, 6, 50
    x["corr_fl"] = (rng.standard_normal((Cc, H, W)) * 0.2).astype(np.float32)
    x["corr_fr"] = (rng.standard_normal((Cc, H, W)) * 0.2).astype(np.float32)
    x["img"] = rng.random((17, 23, 4)).astype(np.float32)
    Hg, Wg = 24, 40
    x["g1"] = (rng.integers(0, 256, (Hg, Wg)) / 255.0).astype(np.float32)
    x["g2"] = np.roll(x["g1"], -3, axis=1) + (rng.standard_normal((Hg, Wg)) * 0.02).astype(np.float32)
    x["vol"] = rng.random((20, 30, 17)).astype(np.float32)
    x["labels"] = rng.integers(0, 40, (20, 30)).astype(np.int32)
    x["wimg"] = rng.random((20, 30, 4)).astype(np.float32)
    x["wu"] = (rng.random((20, 30)) * 40 - 5).astype(np.float32)
    x["vol3"] = rng.standard_normal((20, 30, 3)).astype(np.float32)
    Ht, Wt = 29, 37
    x["tv_u0"] = (rng.random((Ht, Wt)) * 30).astype(np.float32)
    x["tv_qf"] = np.stack([rng.standard_normal((Ht, Wt)), rng.random((Ht, Wt)) * 3], -1).astype(np.float32)
    x["tv_wx"] = (rng.random((Ht, Wt)) * 2).astype(np.float32)
    x["tv_wy"] = (rng.random((Ht, Wt)) * 2).astype(np.float32)
    x["lr_left"] = rng.integers(0, 12, (20, 30)).astype(np.float32)
    x["lr_right"] = -np.roll(x["lr_left"], 2, axis=1) + (rng.random((20, 30)) < 0.2)
    D = 12
    x["qf_c1"] = rng.random((20, 30, D)).astype(np.float32)
    x["qf_labels"] = rng.integers(0, D - 1, (20, 30)).astype(np.int32)  # never the last label, see quadfit
    return x


# the lists and parameters, one place for the script and the tests
CORR_LISTS = {"int": (0.0, 19.0, 1.0), "half": (0.0, 9.5, 0.5), "neg": (-6.0, 13.0, 1.0),
              "refine": (-0.25, 0.25, 0.25)}
PAD = (4, 7)
CENSUS = dict(fs=3, D=16, lam=1.0, lists={"pos": (0.0, 1.0), "neg": (-15.0, 1.0)})
TV = dict(C=3.0, step=1.0, iters=10)
FIT = dict(steps=(1.0, 0.5), lam=1.0 / 0.7)
QF = dict(dmin=2.0, dstep=0.5)


def disparity_list(dmin, dmax, step):
    """The reference's list loop `for (d = min; d <= max; d += step)` in float."""
    out, d = [], np.float32(dmin)
    while d <= np.float32(dmax):
        out.append(float(d))
        d = np.float32(d + np.float32(step))
    return np.array(out, np.float32)


def main(out_path):
    from oracle import refkernels as R
    if not R.available():
        sys.exit("oracle/_ref/refkernels.fatbin or oracle/_build/libref_host.so is missing")
    x = inputs()
    o = dict(x)
    for name, (a, b, s) in CORR_LISTS.items():
        o["corr_" + name] = R.correlation(x["corr_fl"], x["corr_fr"], disparity_list(a, b, s))
    for p in PAD:
        o["pad_%d" % p] = R.pad_rgba(x["img"], p)
    o["gray"] = R.gray(x["img"])
    for name, (dmin, dstep) in CENSUS["lists"].items():
        o["census_" + name] = R.census(x["g1"], x["g2"], CENSUS["fs"], dmin, dstep, CENSUS["D"], CENSUS["lam"])
    o["argmin"] = R.argmin(x["vol"], 3.0, 0.5)
    o["remap"] = R.remap(x["labels"], 2.0, 0.5)
    o["warp"] = R.warp(x["wimg"], x["wu"])
    for s in FIT["steps"]:
        o["fit_%g" % s] = R.tv_fit(x["vol3"], s, FIT["lam"])
    u, u_, p, q = R.tv_iterate(x["tv_u0"], x["tv_u0"], x["tv_qf"], x["tv_wx"], x["tv_wy"], TV["C"], TV["step"],
                               TV["iters"])
    o.update(tv_u=u, tv_u_=u_, tv_p=p, tv_q=q)
    o["lrcheck"] = R.lr_check(x["lr_left"], x["lr_right"], 1.0)
    uq = (x["qf_labels"] * np.float32(QF["dstep"]) + np.float32(QF["dmin"])).astype(np.float32)
    o["quadfit"] = R.quadfit_direct(uq, x["qf_c1"], QF["dmin"], QF["dstep"])
    np.savez_compressed(out_path, **o)
    print("wrote", out_path, sorted(o))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "ref_kernels.npz"))
