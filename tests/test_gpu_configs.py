"""The task's FP32 configurations at their full sizes, through the Stereo C ABI,
bit for bit against the CPU oracle:

  gray 256x192, D=32: 7-layer all-3x3 100-channel CNN, L2-normalised features,
  1 - <fL,fR> unary, truncated-linear CRF (L1 0.5, truncation 3 -> L2 1.5,
  delta 3), 5 iterations, pairwise CNN weights, Xavier weights from seed 0;

  RGB 720x480, D=96: the same network and CRF on a 30-cell Voronoi scene, then
  the TV/Huber refinement with 4 iterations, Huber eps 0.01, lambda 1 (one
  warp: each warp re-runs the whole CNN on the 3-label volume).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L1, L2, DELTA, ITERS, LAM = 0.5, 1.5, 3, 5, 1.0


def _run(cuda, oracle, name, gray, D, warps=0, ref_iters=4, eps=0.1):
    from cnncrf import scenes, _lib as L
    from cnncrf.api import Stereo
    s = scenes.workload(name, seed=0)
    H, W = s["disp"].shape
    st = Stereo(precision=L.FP32, unary=L.UNARY_ONE_MINUS_DOT, topology=L.TOPO_ALL3X3, ref_depth_rounding=False,
                crf_shape=L.RHO_LINEAR, huber_eps=eps)
    st.initialize(W, H, 0.0, 1.0, float(D - 1))
    st.set_matching_function(L.MATCH_GRAYCNN_PAIRWISE if gray else L.MATCH_COLORCNN_PAIRWISE)
    st.set_num_layers(7)
    st.set_xavier_seed(0)
    st.set_color_images(s["left"], s["right"])
    st.compute_slack_propagation(L1, L2, DELTA, ITERS, 0.0, 0.0, LAM)
    labels = st.labels_device().cpu().numpy()
    lb = st.lower_bound()
    if warps:
        st.fuse_thuber_quad_fit(LAM, L2, ref_iters, warps)
    disp = st.get_output()
    cfg = oracle.make_cfg(num_layers=7, topology=1, in_channels=1 if gray else 3, unary=1, disp_max=float(D - 1),
                          lam=LAM, L1=L1, L2=L2, delta=DELTA, crf_iters=ITERS, crf_shape=1, warps=warps,
                          ref_iters=ref_iters, huber_eps=eps, C=L2)
    r = oracle.run_pair(cfg, oracle.xavier_params(cfg, seed=0), s["left"], s["right"])
    return labels, lb, disp, r, s


def test_config_gray256x192_d32(cuda, oracle):
    labels, lb, disp, r, s = _run(cuda, oracle, "gray256x192_d32", True, 32)
    assert np.array_equal(labels, r["labels"])
    assert lb == r["lb"]
    assert np.array_equal(disp, r["disp"])
    assert (labels >= 0).all() and (labels < 32).all()


def test_config_mbq720x480_d96_tv(cuda, oracle):
    labels, lb, disp, r, s = _run(cuda, oracle, "mbq720x480_d96", False, 96, warps=1, ref_iters=4, eps=0.01)
    assert np.array_equal(labels, r["labels"])
    assert lb == r["lb"]
    assert np.array_equal(disp, r["disp"])
    # the refinement moves each disparity by at most half a label step around the CRF solution
    assert np.all(np.abs(disp - labels.astype(np.float32)) <= 0.5 + 1e-6)
