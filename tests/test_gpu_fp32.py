"""GPU parity of the FP32 path: every stage through the C ABI against the CPU
oracle, bit for bit (labels, costs, weights, refined disparities), plus the
shipped-weights golden case."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def pad_np(img, p):
    return np.pad(img, ((p, p), (p, p), (0, 0)), mode="symmetric")


def dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


NET_CASES = [
    # topology, layers, in_channels, unary, D
    (0, 3, 3, 0, 16),
    (0, 7, 5, 0, 20),
    (1, 3, 1, 1, 16),
    (1, 7, 3, 1, 33),
]


@pytest.mark.parametrize("topology,layers,ic,unary,D", NET_CASES)
def test_net_predict_bitexact(cuda, oracle, topology, layers, ic, unary, D):
    torch = cuda
    from cnncrf import scenes
    from cnncrf.api import StereoNet
    W, H = 44, 26
    s = scenes.voronoi_scene(W, H, D, seed=layers + ic, cells=5, off_range=(1, D - 2), slope=0.05)
    cfg = oracle.make_cfg(num_layers=layers, topology=topology, in_channels=ic, unary=unary,
                          disp_max=float(D - 1))
    p = oracle.padding(cfg)
    lp, rp = pad_np(s["left"], p), pad_np(s["right"], p)
    params = oracle.xavier_params(cfg, seed=11)
    net = StereoNet(layers, 1, ic, H + 2 * p, W + 2 * p, topology=topology, unary=unary,
                    with_pairwise=True)
    net.init_net(0.0, float(D - 1), 1.0)
    net.init_xavier(11)
    vol = net.predict(dev(lp, torch), dev(rp, torch))
    torch.cuda.synchronize()
    ovol, opw = oracle.predict(cfg, params, lp, rp, oracle.disparity_list(0.0, float(D - 1), 1.0))
    g = vol.cpu().numpy()
    assert g.shape == ovol.shape
    assert np.array_equal(g, ovol), np.abs(g - ovol).max()
    assert np.array_equal(net.pairwise_out.cpu().numpy(), opw)


def test_shipped_weights_golden(cuda, oracle):
    """kitti-2015/7-layer/cnn+crf+full weights read by the library's npz
    reader, on the reference's sample images."""
    torch = cuda
    from cnncrf.api import StereoNet
    from test_oracle import load_golden
    params, left, right = load_golden()
    cfg = oracle.make_cfg(disp_max=15.0)
    lp, rp = oracle.pad_rgba(left, 4), oracle.pad_rgba(right, 4)
    net = StereoNet(7, 1, 3, lp.shape[0], lp.shape[1], with_pairwise=True)
    net.init_net(0.0, 15.0, 1.0)
    net.set_all_params(os.path.join(GOLDEN, "kitti7_full_params.npz"))
    vol = net.predict(dev(lp, torch), dev(rp, torch)).cpu().numpy()
    pw = net.pairwise_out.cpu().numpy()
    ovol, opw = oracle.predict(cfg, params, lp, rp, oracle.disparity_list(0.0, 15.0, 1.0))
    assert np.array_equal(vol, ovol)
    assert np.array_equal(pw, opw)
    np.testing.assert_allclose(vol, np.load(os.path.join(GOLDEN, "golden_unary_f64.npy")), atol=2e-4)
    np.testing.assert_allclose(pw, np.load(os.path.join(GOLDEN, "golden_pairwise_f64.npy")), atol=2e-4,
                               rtol=2e-4)


def test_npz_errors(cuda, tmp_path):
    from cnncrf.api import StereoNet, CnnCrfError
    from cnncrf import _lib as L
    net = StereoNet(3, 1, 3, 20, 20, with_pairwise=False)
    net.init_net(0.0, 3.0, 1.0)
    with pytest.raises(CnnCrfError) as e:
        net.set_all_params(str(tmp_path / "missing.npz"))
    assert e.value.status == L.EIO
    bad = tmp_path / "bad.npz"
    np.savez(bad, np.zeros((100, 3, 2, 2), np.float32))
    with pytest.raises(CnnCrfError) as e:
        net.set_all_params(str(bad))
    assert e.value.status == L.ESHAPE
    comp = tmp_path / "comp.npz"
    rng = np.random.default_rng(0)
    arrs = [rng.standard_normal(net.param_shape(i)).astype(np.float32) for i in range(net.num_params())]
    np.savez_compressed(comp, *arrs)
    net.set_all_params(str(comp))  # DEFLATE members


@pytest.mark.parametrize("lst", [(0.0, 23.0, 1.0), (0.5, 9.5, 0.5), (-0.25, 0.25, 0.25), (-3.0, 4.0, 1.0)])
def test_correlation_forward(cuda, oracle, lst):
    torch = cuda
    from cnncrf.api import correlation_forward
    rng = np.random.default_rng(1)
    C_, H, W = 7, 9, 37
    fl = rng.standard_normal((C_, H, W)).astype(np.float32)
    fr = rng.standard_normal((C_, H, W)).astype(np.float32)
    d = oracle.disparity_list(*lst)
    out = correlation_forward(dev(fl[None], torch), dev(fr[None], torch), d).cpu().numpy()
    ref = oracle.correlation(fl.transpose(1, 2, 0), fr.transpose(1, 2, 0), d)
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("D", [1, 5, 32, 40, 96, 128, 200])
@pytest.mark.parametrize("delta,shape", [(1, 0), (2, 0), (3, 1), (4, 1)])
def test_crf_bitexact(cuda, oracle, D, delta, shape):
    torch = cuda
    from cnncrf.api import crf_solve
    rng = np.random.default_rng(D * 10 + delta)
    H, W = 13, 17
    cost = rng.random((H, W, D)).astype(np.float32)
    wx = (rng.random((H, W)) * 0.5).astype(np.float32)
    wy = (rng.random((H, W)) * 0.5).astype(np.float32)
    for iters in (1, 3):
        lab, lb = crf_solve(dev(cost, torch), dev(wx, torch), dev(wy, torch), L1=0.3, L2=1.1, delta=delta,
                            total_it=iters, shape=shape, slack=0.5)
        olab, olb, _, _ = oracle.crf(cost, wx, wy, 0.3, 1.1, delta, iters, shape=shape, slack=0.5)
        assert np.array_equal(lab.cpu().numpy(), olab)
        assert lb == olb


@pytest.mark.parametrize("H,W,D,shape,delta", [(4, 5, 16, 1, 3), (5, 4, 40, 0, 2), (3, 6, 33, 1, 4),
                                                (6, 3, 128, 1, 3)])
def test_crf_bound_reaches_the_lp_relaxation(cuda, H, W, D, shape, delta):
    """The GPU solver's bound, after 300 iterations, equals the optimum of the
    energy's local-polytope LP relaxation as scipy's HiGHS solves it: the
    solver maximises the dual of that LP (weak duality keeps every bound at or
    below it; see tests/test_oracle.py), here to within 1e-5."""
    pytest.importorskip("scipy")
    torch = cuda
    from cnncrf.api import crf_solve
    from test_oracle import _local_polytope_lp
    rng = np.random.default_rng(H * 100 + D)
    cost = (rng.random((H, W, D)) * 3).astype(np.float32)
    wx = (rng.random((H, W)) * 2).astype(np.float32)
    wy = (rng.random((H, W)) * 2).astype(np.float32)
    lp = _local_polytope_lp(cost, wx, wy, 0.6, 1.7, delta, shape)
    _, lb = crf_solve(dev(cost, torch), dev(wx, torch), dev(wy, torch), L1=0.6, L2=1.7, delta=delta,
                      total_it=300, shape=shape, slack=0.5)
    assert abs(lb - lp) <= 1e-5 * max(1.0, abs(lp)), (lb, lp)


def test_slackprop_object(cuda, oracle):
    torch = cuda
    from cnncrf.api import SlackProp
    rng = np.random.default_rng(2)
    H, W, D = 11, 19, 24
    cost = rng.random((H, W, D)).astype(np.float32)
    wx = rng.random((H, W)).astype(np.float32)
    wy = rng.random((H, W)).astype(np.float32)
    labels = torch.empty((H, W), dtype=torch.int32, device="cuda")
    sp = SlackProp()
    c = dev(cost, torch)
    sp.init(c, labels)
    sp.ops["L1"] = 0.5
    sp.ops["L2"] = 2.0
    sp.ops["delta"] = 2
    sp.ops["total_it"] = 5
    sp.update_W(dev(wx, torch), dev(wy, torch))
    sp.execute()
    olab, olb, _, oc1 = oracle.crf(cost, wx, wy, 0.5, 2.0, 2, 5, want_c1=True)
    assert np.array_equal(labels.cpu().numpy(), olab)
    assert sp.LB() == olb
    assert np.array_equal(sp.get_C1().cpu().numpy(), oc1)


def test_remap_warp_fit_tv(cuda, oracle):
    torch = cuda
    from cnncrf import api
    rng = np.random.default_rng(3)
    H, W = 21, 33
    lab = rng.integers(0, 40, (H, W)).astype(np.int32)
    out = api.remap_solution(dev(lab, torch), 2.0, 0.5).cpu().numpy()
    assert np.array_equal(out, oracle.remap(lab, 2.0, 0.5))
    img = rng.random((H, W, 4)).astype(np.float32)
    u = (rng.random((H, W)) * 40 - 5).astype(np.float32)
    wimg = api.warp_image(dev(img, torch), dev(u, torch)).cpu().numpy()
    assert np.array_equal(wimg, oracle.warp(img, u))
    vol3 = rng.standard_normal((H, W, 3)).astype(np.float32)
    qf = api.tv_fit(dev(vol3, torch), 1.0, 1.0 / 0.7).cpu().numpy()
    assert np.array_equal(qf, oracle.tv_fit(vol3, 1.0, 1.0 / 0.7))
    w = rng.random((H, W)).astype(np.float32)
    wy = rng.random((H, W)).astype(np.float32)
    u0 = out.copy()
    g = api.tv_iterate(dev(u0, torch), dev(u0, torch), dev(qf, torch), dev(w, torch), dev(wy, torch), 5.0, 0.1,
                       0.5, 7)
    o = oracle.tv_iterate(u0, u0, qf, w, wy, 5.0, 0.1, 0.5, 7)
    for a, b in zip(g, o):
        assert np.array_equal(a.cpu().numpy(), b)


@pytest.mark.parametrize("W,H", [(33, 21), (130, 70), (201, 97)])
@pytest.mark.parametrize("iters", [1, 4, 8, 9, 17])
def test_tv_fused_tiles_and_launches(cuda, oracle, W, H, iters):
    """The fused TV kernel (K iterations per launch on 64 x 32 tiles with a
    K-pixel halo, at most 8 per launch) against the oracle's per-iteration
    loop, bit for bit in u, u_, p and q: one tile and many, ragged image
    edges, one launch, two launches, three (the state then ends in the
    caller's buffers from either ping-pong parity)."""
    torch = cuda
    from cnncrf import api
    rng = np.random.default_rng(W * 1000 + H + iters)
    u0 = (rng.random((H, W)) * 30).astype(np.float32)
    qf = np.stack([rng.standard_normal((H, W)), rng.random((H, W)) * 3], -1).astype(np.float32)
    wx = (rng.random((H, W)) * 2).astype(np.float32)
    wy = (rng.random((H, W)) * 2).astype(np.float32)
    g = api.tv_iterate(dev(u0, torch), dev(u0, torch), dev(qf, torch), dev(wx, torch), dev(wy, torch), 1.5, 0.01,
                       1.0, iters)
    o = oracle.tv_iterate(u0, u0, qf, wx, wy, 1.5, 0.01, 1.0, iters)
    for name, a, b in zip(("u", "u_", "p", "q"), g, o):
        assert np.array_equal(a.cpu().numpy(), b), name


def test_refinement_two_warps_multi_tile(cuda, oracle):
    """fuseTHuberQuadFit with two warps on an image of several TV tiles: the
    second warp's TV iterations start from the first warp's p and q (the
    reference zeroes them once, stereo/stereo.cu:1133-1135), 9 iterations =
    two fused launches per warp."""
    from cnncrf import scenes, _lib as L
    from cnncrf.api import Stereo
    W, H = 150, 70
    s = scenes.voronoi_scene(W, H, 16, seed=8, cells=6, off_range=(1, 12), slope=0.05)
    st = Stereo(precision=L.FP32, unary=0, topology=0, ref_depth_rounding=False, crf_shape=0)
    st.initialize(W, H, 0.0, 1.0, 15.0)
    st.set_matching_function(L.MATCH_COLORCNN_PAIRWISE)
    st.set_num_layers(3)
    st.set_xavier_seed(2)
    st.set_color_images(s["left"], s["right"])
    st.compute_slack_propagation(1.0, 5.0, 2, 3, 0.0, 0.0, 0.8)
    st.fuse_thuber_quad_fit(0.8, 5.0, 9, 2)
    cfg = oracle.make_cfg(num_layers=3, topology=0, unary=0, disp_max=15.0, lam=0.8, L1=1.0, L2=5.0, delta=2,
                          crf_iters=3, crf_shape=0, warps=2, ref_iters=9, C=5.0)
    r = oracle.run_pair(cfg, oracle.xavier_params(cfg, seed=2), s["left"], s["right"])
    assert np.array_equal(st.get_output(), r["disp"])


PIPE_CASES = [
    # topology, layers, unary, shape, rounding, D(max+1), refine
    dict(topology=0, layers=3, unary=0, shape=0, rounding=True, dmax=11.0, warps=2, L1=1.0, L2=5.0, delta=2),
    dict(topology=1, layers=3, unary=1, shape=1, rounding=False, dmax=13.0, warps=0, L1=0.5, L2=1.5, delta=3),
    dict(topology=0, layers=7, unary=0, shape=0, rounding=True, dmax=15.0, warps=1, L1=1.0, L2=14.98, delta=2),
]


@pytest.mark.parametrize("case", PIPE_CASES)
def test_stereo_pipeline_bitexact(cuda, oracle, case):
    """Stereo::computeSlackPropagation (+ fuseTHuberQuadFit) end to end."""
    from cnncrf import scenes, _lib as L
    from cnncrf.api import Stereo
    W, H = 52, 30
    s = scenes.voronoi_scene(W, H, 16, seed=5, cells=5, off_range=(1, 12), slope=0.05)
    st = Stereo(precision=L.FP32, unary=case["unary"], topology=case["topology"],
                ref_depth_rounding=case["rounding"], crf_shape=case["shape"])
    st.initialize(W, H, 0.0, 1.0, case["dmax"])
    st.set_matching_function(L.MATCH_COLORCNN_PAIRWISE)
    st.set_num_layers(case["layers"])
    st.set_xavier_seed(3)
    st.set_color_images(s["left"], s["right"])
    st.compute_slack_propagation(case["L1"], case["L2"], case["delta"], 3, 20.0, 0.9, 0.8)
    if case["warps"]:
        st.fuse_thuber_quad_fit(0.8, case["L2"], 4, case["warps"])
    disp = st.get_output()
    D = st.get_depth()
    cfg = oracle.make_cfg(num_layers=case["layers"], topology=case["topology"], unary=case["unary"],
                          disp_max=float(D - 1), lam=0.8, L1=case["L1"], L2=case["L2"], delta=case["delta"],
                          crf_iters=3, crf_shape=case["shape"], warps=case["warps"], ref_iters=4,
                          C=case["L2"])
    params = oracle.xavier_params(cfg, seed=3)
    r = oracle.run_pair(cfg, params, s["left"], s["right"])
    assert np.array_equal(st.labels_device().cpu().numpy(), r["labels"])
    assert np.array_equal(disp, r["disp"])
    assert st.lower_bound() == r["lb"]
    wx, wy = st.weights_device()
    assert np.array_equal(wx.cpu().numpy(), r["wx"])


def test_stereo_argmax_and_errors(cuda, oracle):
    from cnncrf import scenes, _lib as L
    from cnncrf.api import Stereo, CnnCrfError
    W, H = 40, 24
    s = scenes.voronoi_scene(W, H, 8, seed=9, cells=3, off_range=(1, 6), slope=0.0)
    st = Stereo(precision=L.BF16)
    st.initialize(W, H, 0.0, 1.0, 7.0)
    st.set_matching_function(L.MATCH_CONCATCNN)  # the concatenating net runs in FP32 only
    st.set_num_layers(7)
    st.set_color_images(s["left"], s["right"])
    with pytest.raises(CnnCrfError) as e:
        st.compute_argmax()
    assert e.value.status == L.EUNSUPPORTED
    st = Stereo()
    st.initialize(W, H, 0.0, 1.0, 7.0)
    st.set_matching_function(L.MATCH_CONCATCNN)
    st.set_num_layers(4)  # not a ConcatStereoNet depth
    st.set_color_images(s["left"], s["right"])
    with pytest.raises(CnnCrfError) as e:
        st.compute_argmax()
    assert e.value.status == L.EINVAL
    st.set_matching_function(L.MATCH_COLORCNN)
    st.set_num_layers(3)
    st.set_xavier_seed(1)
    st.compute_argmax()
    vol = st.volume_device().cpu().numpy()
    assert np.array_equal(st.get_output(), oracle.argmin(vol, 0.0, 1.0))
    st.set_num_layers(4)
    with pytest.raises(CnnCrfError) as e:
        st.compute_volume()
    assert e.value.status == L.EINVAL


def test_refinement_reuses_left_features(cuda, oracle):
    """The refinement's re-match runs the CNN on (left, warped right); the left
    input is the matching's padded left image, so its features are kept, not
    recomputed: each warp launches the convolutions of the right image and the
    pairwise net only (layers + 2), and the refined disparities still equal the
    oracle's (which recomputes them).  After a new image upload the first warp
    recomputes both sides."""
    from cnncrf import scenes, _lib as L
    from cnncrf.api import Stereo
    W, H, layers, warps = 52, 30, 5, 2
    s = scenes.voronoi_scene(W, H, 16, seed=8, cells=5, off_range=(1, 12), slope=0.05)
    st = Stereo(precision=L.FP32, unary=L.UNARY_ONE_MINUS_DOT, topology=L.TOPO_ALL3X3, ref_depth_rounding=False,
                crf_shape=L.RHO_LINEAR)
    st.initialize(W, H, 0.0, 1.0, 15.0)
    st.set_matching_function(L.MATCH_COLORCNN_PAIRWISE)
    st.set_num_layers(layers)
    st.set_xavier_seed(3)

    def convs_in_refinement():
        L.profile_reset()
        L.profile_enable(True)
        try:
            st.fuse_thuber_quad_fit(0.8, 1.5, 4, warps)
            return sum(L.profile_query(k)[0] for k in ("conv_simt", "conv_first"))
        finally:
            L.profile_enable(False)

    st.set_color_images(s["left"], s["right"])
    st.compute_slack_propagation(0.5, 1.5, 3, 3, 20.0, 0.9, 0.8)
    assert convs_in_refinement() == warps * (layers + 2)
    cfg = oracle.make_cfg(num_layers=layers, topology=1, unary=1, disp_max=15.0, lam=0.8, L1=0.5, L2=1.5, delta=3,
                          crf_iters=3, crf_shape=1, warps=warps, ref_iters=4, C=1.5)
    r = oracle.run_pair(cfg, oracle.xavier_params(cfg, seed=3), s["left"], s["right"])
    assert np.array_equal(st.get_output(), r["disp"])
    # new images without a new matching: the first warp recomputes both sides, the next one keeps them
    st.set_color_images(s["right"], s["left"])
    assert convs_in_refinement() == (2 * layers + 2) + (warps - 1) * (layers + 2)
