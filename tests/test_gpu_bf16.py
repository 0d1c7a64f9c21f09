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


def q16_unary(torch, vol, unary):
    """The BF16 path's 16-bit fixed-point unary as the correlation writes it
    and the CRF reads it back: q = x / scale - offset / scale in FP32 (one
    rounding: x / scale is exact), rounded to the nearest integer (ties to
    even) and saturated to 0..65535; x' = q * scale + offset (scale 2^-15,
    offset -2^-8 for 1 - <fL,fR>; 2^-16 and -1 for -softmax)."""
    scale, offset = (2.0 ** -15, -2.0 ** -8) if unary == 1 else (2.0 ** -16, -1.0)
    q = torch.clamp(torch.round(vol * (1.0 / scale) + (-offset / scale)), 0, 65535)
    return q * scale + offset


@pytest.mark.parametrize("D,unary", [(64, 1), (96, 1), (128, 1), (128, 0), (192, 1)])
def test_bf16_crf_reads_the_16bit_unary(cuda, D, unary):
    """The BF16 path's CRF reads a 16-bit fixed-point copy of the unary volume
    that the tensor-core correlation writes beside the FP32 one (half the
    bytes of the horizontal passes' two unary reads; 2^-15 resolution for the
    1 - <fL,fR> unary, 2^-16 for -softmax), where each lane's labels are an
    even count (D = 64, 128, 192: 2, 4 and 6 per lane); at D = 96 (3 per
    lane) it reads the FP32 volume.  Either way its labels and bound equal those of the
    FP32 solver (the C ABI's cnncrf_crf_solve) on the volume as the CRF read
    it -- dequantised where the copy is used -- bit for bit; the solve itself
    stays FP32 (messages) and FP64 (bound)."""
    torch = cuda
    from cnncrf import api, scenes, _lib as L
    from cnncrf.api import Stereo
    W, H = 200, 48
    s = scenes.kitti_scene(W, H, D, seed=11, ground_max=D * 0.8, box_range=(4.0, D * 0.9))
    st = Stereo(precision=L.BF16, unary=unary, topology=L.TOPO_ALL3X3, ref_depth_rounding=False,
                crf_shape=L.RHO_LINEAR)
    st.initialize(W, H, 0.0, 1.0, float(D - 1))
    st.set_matching_function(L.MATCH_COLORCNN_PAIRWISE)
    st.set_num_layers(7)
    st.set_xavier_seed(0)
    st.set_color_images(s["left"], s["right"])
    st.compute_slack_propagation(0.5, 1.5, 3, 6, 0.0, 0.0, 1.0)
    vol = st.volume_device().clone()
    wx, wy = (t.clone() for t in st.weights_device())
    if D % 64 == 0:
        unary_in = q16_unary(torch, vol, unary)
        # the copy's resolution: within half a step of the FP32 cost wherever that lies inside the range, plus
        # the FP32 rounding of x / scale - offset / scale (half an ulp of 2, in units of x)
        scale, offset = (2.0 ** -15, -2.0 ** -8) if unary == 1 else (2.0 ** -16, -1.0)
        inside = (vol >= offset) & (vol <= offset + 65535 * scale)
        assert float((unary_in - vol).abs()[inside].max()) <= scale / 2 + 2.0 ** -23
    else:
        unary_in = vol
    lab, lb = api.crf_solve(unary_in, wx, wy, 0.5, 1.5, 3, 6, L.RHO_LINEAR, 0.5)
    assert np.array_equal(lab.cpu().numpy(), st.labels_device().cpu().numpy())
    assert lb == st.lower_bound()


def test_bf16_batch_volume_kept_only_on_request(cuda):
    """The BF16 batch writes only the CRF's 16-bit copy of the volume: asking
    for the FP32 volume then fails with ESTATE, unless keep_volume was set,
    in which case it equals the single-pair Stereo path's volume bit for bit
    and the labels are the same either way."""
    torch = cuda
    from cnncrf import scenes, _lib as L
    from cnncrf.api import Stereo, StereoBatch, CnnCrfError
    W, H, D = 96, 40, 64
    s = scenes.kitti_scene(W, H, D, seed=12, ground_max=50.0, box_range=(4.0, 60.0))
    labs = []
    for keep in (False, True):
        b = StereoBatch(precision=L.BF16, num_layers=3, seed=0, keep_volume=keep)
        b.add_pair(W, H, 0.0, 1.0, float(D - 1))
        b.set_images(0, s["left"], s["right"])
        b.run(0.5, 1.5, 3, 4)
        b.check()
        labs.append(b.labels_device(0).cpu().numpy())
        if not keep:
            with pytest.raises(CnnCrfError) as e:
                b.volume_device(0)
            assert e.value.status == L.ESTATE
        else:
            st = Stereo(precision=L.BF16, unary=L.UNARY_ONE_MINUS_DOT, topology=L.TOPO_ALL3X3,
                        ref_depth_rounding=False, crf_shape=L.RHO_LINEAR)
            st.initialize(W, H, 0.0, 1.0, float(D - 1))
            st.set_matching_function(L.MATCH_COLORCNN_PAIRWISE)
            st.set_num_layers(3)
            st.set_xavier_seed(0)
            st.set_color_images(s["left"], s["right"])
            st.compute_slack_propagation(0.5, 1.5, 3, 4, 0.0, 0.0, 1.0)
            assert np.array_equal(b.volume_device(0).cpu().numpy(), st.volume_device().cpu().numpy())
            assert np.array_equal(labs[-1], st.labels_device().cpu().numpy())
    assert np.array_equal(labs[0], labs[1])
