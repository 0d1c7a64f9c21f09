"""GPU parity of ConcatStereoNet (CNNCRF_TOPO_CONCAT, FP32): every layer a
zero-padded 3x3 conv to the growth rate, the features all layers' outputs
side by side, the correlation and the |tanh| pairwise conv over them.  The
net, the Stereo pipeline on the CONCATCNN matchings and the FP32 batch equal
the CPU oracle (or the single-pair path) bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


CASES = [
    # layers, in_channels, unary, pairwise, W, H, D
    (3, 3, 0, True, 44, 26, 12),
    (7, 5, 1, True, 150, 20, 16),   # two 128-pixel conv tiles per row, the second partial
    (10, 1, 0, False, 40, 18, 9),
    (15, 3, 1, True, 36, 22, 20),
]


@pytest.mark.parametrize("layers,ic,unary,pairwise,W,H,D", CASES)
def test_concat_net_bitexact(cuda, oracle, layers, ic, unary, pairwise, W, H, D):
    torch = cuda
    from cnncrf import scenes, _lib as L
    from cnncrf.api import StereoNet
    s = scenes.voronoi_scene(W, H, D, seed=layers + ic, cells=4, off_range=(1, D - 2), slope=0.05)
    cfg = oracle.make_cfg(num_layers=layers, topology=L.TOPO_CONCAT, in_channels=ic, unary=unary,
                          disp_max=float(D - 1), with_pairwise=1 if pairwise else 0)
    assert oracle.padding(cfg) == 0
    params = oracle.xavier_params(cfg, seed=21)
    net = StereoNet(layers, 1, ic, H, W, topology=L.TOPO_CONCAT, unary=unary, with_pairwise=pairwise)
    assert net.pad == 0 and net.desc.feat_channels == L.CONCAT_GROWTH[layers] * layers
    net.init_net(0.0, float(D - 1), 1.0)
    net.init_xavier(21)
    vol = net.predict(dev(s["left"], torch), dev(s["right"], torch))
    torch.cuda.synchronize()
    ovol, opw = oracle.predict(cfg, params, s["left"], s["right"], oracle.disparity_list(0.0, float(D - 1), 1.0))
    g = vol.cpu().numpy()
    assert g.shape == ovol.shape == (H, W, D)
    assert np.array_equal(g, ovol), np.abs(g - ovol).max()
    if pairwise:
        pw = net.pairwise_out.cpu().numpy()
        assert np.array_equal(pw, opw)
        assert pw.min() >= 0.0


@pytest.mark.parametrize("matching,warps", [("CONCATCNN_PAIRWISE", 1), ("CONCATCNN", 0)])
def test_concat_stereo_pipeline_bitexact(cuda, oracle, matching, warps):
    """Stereo::computeSlackPropagation on the CONCATCNN matchings (the
    pairwise one with one TV refinement warp): labels, disparities, bound and
    weights equal the oracle's run of the same pair."""
    from cnncrf import scenes, _lib as L
    from cnncrf.api import Stereo
    W, H, layers = 48, 28, 5
    pw = matching == "CONCATCNN_PAIRWISE"
    s = scenes.voronoi_scene(W, H, 16, seed=6, cells=5, off_range=(1, 12), slope=0.05)
    st = Stereo(precision=L.FP32, unary=L.UNARY_ONE_MINUS_DOT, ref_depth_rounding=False, crf_shape=L.RHO_LINEAR)
    st.initialize(W, H, 0.0, 1.0, 15.0)
    st.set_matching_function(getattr(L, "MATCH_" + matching))
    st.set_num_layers(layers)
    st.set_xavier_seed(4)
    st.set_color_images(s["left"], s["right"])
    if pw:
        st.compute_slack_propagation(0.5, 1.5, 3, 3, 20.0, 0.9, 0.8)
        st.fuse_thuber_quad_fit(0.8, 1.5, 4, warps)
    else:
        st.compute_argmax()
    cfg = oracle.make_cfg(num_layers=layers, topology=L.TOPO_CONCAT, unary=1, disp_max=15.0, lam=0.8, L1=0.5,
                          L2=1.5, delta=3, crf_iters=3, crf_shape=1, warps=warps, ref_iters=4, C=1.5,
                          with_pairwise=1 if pw else 0)
    params = oracle.xavier_params(cfg, seed=4)
    if pw:
        r = oracle.run_pair(cfg, params, s["left"], s["right"])
        assert np.array_equal(st.labels_device().cpu().numpy(), r["labels"])
        assert np.array_equal(st.get_output(), r["disp"])
        assert st.lower_bound() == r["lb"]
        wx, wy = st.weights_device()
        assert np.array_equal(wx.cpu().numpy(), r["wx"]) and np.array_equal(wy.cpu().numpy(), r["wy"])
    else:
        ovol, _ = oracle.predict(cfg, params, s["left"], s["right"], oracle.disparity_list(0.0, 15.0, 1.0))
        assert np.array_equal(st.volume_device().cpu().numpy(), ovol)
        assert np.array_equal(st.get_output(), oracle.argmin(ovol, 0.0, 1.0))


def test_concat_batch_equals_single(cuda):
    """The FP32 batch on CONCATCNN_PAIRWISE (two shapes, one group of two
    pairs) gives each pair the single-pair Stereo path's labels, disparities
    and bound."""
    from cnncrf import scenes, _lib as L
    from cnncrf.api import Stereo, StereoBatch
    layers, iters, crf = 7, 3, (0.5, 1.5, 3)
    shapes = [(64, 30, 16), (48, 20, 12), (64, 30, 16)]
    sc = [scenes.voronoi_scene(W, H, D, seed=40 + i, cells=4, off_range=(1, D - 2), slope=0.05)
          for i, (W, H, D) in enumerate(shapes)]
    b = StereoBatch(precision=L.FP32, num_layers=layers, seed=2, matching=L.MATCH_CONCATCNN_PAIRWISE)
    for (W, H, D) in shapes:
        b.add_pair(W, H, 0.0, 1.0, float(D - 1))
    for i, x in enumerate(sc):
        b.set_images(i, x["left"], x["right"])
    b.run(*crf, iters)
    b.check()
    for i, (W, H, D) in enumerate(shapes):
        st = Stereo(precision=L.FP32, unary=L.UNARY_ONE_MINUS_DOT, ref_depth_rounding=False, crf_shape=L.RHO_LINEAR)
        st.initialize(W, H, 0.0, 1.0, float(D - 1))
        st.set_matching_function(L.MATCH_CONCATCNN_PAIRWISE)
        st.set_num_layers(layers)
        st.set_xavier_seed(2)
        st.set_color_images(sc[i]["left"], sc[i]["right"])
        st.compute_slack_propagation(*crf, iters, 0.0, 0.0, 1.0)
        assert np.array_equal(b.labels_device(i).cpu().numpy(), st.labels_device().cpu().numpy()), i
        assert np.array_equal(b.get_output(i), st.get_output()), i
        assert b.lower_bound(i) == st.lower_bound(), i
