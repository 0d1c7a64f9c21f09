"""GPU tests of the BF16 tensor-core path (tcgen05 convolution, BF16
correlation): numerics against a torch emulation of the same BF16 arithmetic
and against the FP32 / FP64 oracle, and the BF16-vs-FP32 label change."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pad_np(img, p):
    return np.pad(img, ((p, p), (p, p), (0, 0)), mode="symmetric")


def bf16(x, torch):
    return x.to(torch.bfloat16).to(torch.float32)


def emulate_features(torch, oracle, cfg, params, img_pad):
    """The BF16 path in torch: every layer with BF16 inputs and weights, FP32
    accumulation, tanh, BF16 output (layer 1 takes the normalised FP32 image
    rounded to BF16); the last layer L2-normalised (unary 1)."""
    x = torch.from_numpy(oracle.normalize(img_pad, cfg.in_channels, 32)).permute(2, 0, 1)[None].double()
    x = bf16(x.float(), torch).double()
    L = cfg.num_layers
    for l in range(L):
        w = torch.from_numpy(params[2 * l]).flip(2, 3)
        b = torch.from_numpy(params[2 * l + 1])
        w = bf16(w, torch)
        y = torch.tanh(torch.nn.functional.conv2d(x.float(), w.float(), b.float()).double())
        if l == L - 1 and cfg.unary == 1:
            y = y / y.norm(dim=1, keepdim=True)
        x = bf16(y.float(), torch).double()
    return x[0].permute(1, 2, 0).float().numpy()


@pytest.mark.parametrize("topology,layers", [(1, 2), (0, 3), (1, 3)])
def test_tc_conv_layer_matches_emulation(cuda, oracle, topology, layers):
    torch = cuda
    from cnncrf import scenes, _lib as L
    from cnncrf.api import StereoNet
    W, H = 300, 20  # three 128-pixel tiles per row, the last one partial
    s = scenes.voronoi_scene(W, H, 16, seed=4, cells=5)
    cfg = oracle.make_cfg(num_layers=layers, topology=topology, unary=1, disp_max=15.0, with_pairwise=0)
    p = oracle.padding(cfg)
    lp, rp = pad_np(s["left"], p), pad_np(s["right"], p)
    params = oracle.xavier_params(cfg, seed=7)
    net = StereoNet(layers, 1, 3, H + 2 * p, W + 2 * p, topology=topology, unary=1, precision=L.BF16)
    net.init_net(0.0, 15.0, 1.0)
    net.init_xavier(7)
    net.predict(torch.from_numpy(lp).cuda(), torch.from_numpy(rp).cuda())
    f = net.features(0).cpu().numpy()
    ref = emulate_features(torch, oracle, cfg, params, lp)
    assert f.shape == ref.shape
    err = np.abs(f - ref)
    # one BF16 rounding step of difference at most (tanh.approx vs tanh, sum order)
    assert err.max() < 1.6e-2, err.max()
    assert err.mean() < 1e-3, err.mean()


def test_bf16_features_and_weights_vs_fp32_oracle(cuda, oracle):
    torch = cuda
    from cnncrf import scenes, _lib as L
    from cnncrf.api import StereoNet
    W, H, D = 200, 40, 32
    s = scenes.kitti_scene(W, H, D, seed=2)
    cfg = oracle.make_cfg(num_layers=7, topology=1, unary=1, disp_max=float(D - 1))
    p = oracle.padding(cfg)
    lp, rp = pad_np(s["left"], p), pad_np(s["right"], p)
    params = oracle.xavier_params(cfg, seed=0)
    net = StereoNet(7, 1, 3, H + 2 * p, W + 2 * p, topology=1, unary=1, precision=L.BF16, with_pairwise=True)
    net.init_net(0.0, float(D - 1), 1.0)
    net.init_xavier(0)
    vol = net.predict(torch.from_numpy(lp).cuda(), torch.from_numpy(rp).cuda()).cpu().numpy()
    pw = net.pairwise_out.cpu().numpy()
    cfg64 = oracle.make_cfg(num_layers=7, topology=1, unary=1, disp_max=float(D - 1), precision=64)
    ovol, opw = oracle.predict(cfg64, params, lp, rp, oracle.disparity_list(0.0, float(D - 1), 1.0))
    # cost error against the FP64 oracle (costs are 1 - cosine similarity, in [0, 2])
    cerr = np.abs(vol - ovol)
    assert cerr.mean() < 1e-2, cerr.mean()
    assert np.percentile(cerr, 99.9) < 8e-2
    werr = np.abs(pw - opw) / (np.abs(opw) + 0.05)
    assert werr.mean() < 2e-2, werr.mean()


def test_bf16_pipeline_label_change(cuda, oracle):
    """BF16 vs FP32 Stereo path on one KITTI-shaped scene: fraction of pixels
    whose integer disparity changes, held to the metric's bound of 0.5 %."""
    from cnncrf import scenes, _lib as L
    from cnncrf.api import Stereo
    W, H, D = 320, 96, 64
    s = scenes.kitti_scene(W, H, D, seed=3, ground_max=55.0, box_range=(5.0, 60.0))
    labs = []
    for prec in (L.FP32, L.BF16):
        st = Stereo(precision=prec, unary=L.UNARY_ONE_MINUS_DOT, topology=L.TOPO_ALL3X3,
                    ref_depth_rounding=False, crf_shape=L.RHO_LINEAR)
        st.initialize(W, H, 0.0, 1.0, float(D - 1))
        st.set_matching_function(L.MATCH_COLORCNN_PAIRWISE)
        st.set_num_layers(7)
        st.set_xavier_seed(0)
        st.set_color_images(s["left"], s["right"])
        st.compute_slack_propagation(0.5, 1.5, 3, 8, 0.0, 0.0, 1.0)
        labs.append(st.labels_device().cpu().numpy())
    changed = float((labs[0] != labs[1]).mean())
    print("BF16 vs FP32 label change: %.4f" % changed)
    assert changed <= 0.005
