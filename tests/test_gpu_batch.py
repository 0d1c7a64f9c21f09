"""GPU tests of the batched form: pairs grouped by shape, each group one
batch per launch, groups on their own streams, optional CUDA-graph replay.
Batching must not change a single bit of any pair's result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def single_run(L, scene, prec, dmax, layers, iters, crf):
    from cnncrf.api import Stereo
    H, W = scene["disp"].shape
    st = Stereo(precision=prec, unary=L.UNARY_ONE_MINUS_DOT, topology=L.TOPO_ALL3X3, ref_depth_rounding=False,
                crf_shape=L.RHO_LINEAR)
    st.initialize(W, H, 0.0, 1.0, dmax)
    st.set_matching_function(L.MATCH_COLORCNN_PAIRWISE)
    st.set_num_layers(layers)
    st.set_xavier_seed(0)
    st.set_color_images(scene["left"], scene["right"])
    st.compute_slack_propagation(crf[0], crf[1], crf[2], iters, 0.0, 0.0, 1.0)
    return st.labels_device().cpu().numpy(), st.get_output(), st.lower_bound()


@pytest.mark.parametrize("prec_name,group_size", [("FP32", 0), ("BF16", 0), ("BF16", 2)])
def test_batch_equals_single(cuda, prec_name, group_size):
    """group_size 2 splits the three same-shape pairs into a pipelined group of
    two and a group of one.  The batch's CRF skips the last V pass's phi
    store (no caller of the batch reads C1) while the single-pair solve keeps
    it, so the exact equality of labels and bounds here also pins that the
    skipped store changes neither."""
    from cnncrf import scenes, _lib as L
    from cnncrf.api import StereoBatch
    prec = getattr(L, prec_name)
    layers, iters, crf = 3, 3, (0.5, 1.5, 3)
    shapes = [(64, 40, 16), (64, 40, 16), (96, 24, 32), (64, 40, 16)]  # two shapes, interleaved
    sc = [scenes.voronoi_scene(W, H, D, seed=10 + i, cells=4, off_range=(1, D - 2), slope=0.05)
          for i, (W, H, D) in enumerate(shapes)]
    b = StereoBatch(precision=prec, num_layers=layers, seed=0, group_size=group_size)
    for (W, H, D) in shapes:
        b.add_pair(W, H, 0.0, 1.0, float(D - 1))
    for i, s in enumerate(sc):
        b.set_images(i, s["left"], s["right"])
    b.run(*crf, iters)
    b.check()
    for i, (W, H, D) in enumerate(shapes):
        lab, disp, lb = single_run(L, sc[i], prec, float(D - 1), layers, iters, crf)
        assert np.array_equal(b.labels_device(i).cpu().numpy(), lab), i
        assert np.array_equal(b.get_output(i), disp), i
        assert b.lower_bound(i) == lb, i


@pytest.mark.parametrize("group_size", [0, 1])
def test_batch_graph_replay(cuda, group_size):
    from cnncrf import scenes, _lib as L
    from cnncrf.api import StereoBatch
    torch = cuda
    shapes = [(80, 32, 32)] * 3 + [(48, 24, 16)]
    b = StereoBatch(precision=L.BF16, num_layers=3, seed=1, graph=True, group_size=group_size)
    eager = StereoBatch(precision=L.BF16, num_layers=3, seed=1, graph=False)
    for (W, H, D) in shapes:
        b.add_pair(W, H, 0.0, 1.0, float(D - 1))
        eager.add_pair(W, H, 0.0, 1.0, float(D - 1))
    for rnd in range(4):  # eager run, capture, two replays with new images
        sc = [scenes.voronoi_scene(W, H, D, seed=100 * rnd + i, cells=4, off_range=(1, D - 2))
              for i, (W, H, D) in enumerate(shapes)]
        for i, s in enumerate(sc):
            b.set_images(i, torch.from_numpy(s["left"]).cuda(), torch.from_numpy(s["right"]).cuda())
            eager.set_images(i, s["left"], s["right"])
        b.run(0.5, 1.5, 3, 4)
        eager.run(0.5, 1.5, 3, 4)
        torch.cuda.synchronize()
        for i in range(len(shapes)):
            assert np.array_equal(b.get_output(i), eager.get_output(i)), (rnd, i)


@pytest.mark.parametrize("pinned", [True, False])
def test_batch_run_host_equals_staged_run(cuda, pinned):
    """cnncrf_batch_run_host (host images in, host disparities out, copies
    pipelined with the groups' work) gives the same disparities as
    set_images + run + get_output.  Page-locked buffers: the first call runs
    eagerly, the second captures a graph, the third and fourth replay it with
    new contents in the same buffers.  Pageable buffers run eagerly every
    time.  A pair whose output pointer is null gets no copy."""
    from cnncrf import scenes, _lib as L
    from cnncrf.api import StereoBatch
    torch = cuda
    shapes = [(80, 32, 32)] * 3 + [(48, 24, 16)]
    b = StereoBatch(precision=L.BF16, num_layers=3, seed=1, graph=True, group_size=2)
    ref = StereoBatch(precision=L.BF16, num_layers=3, seed=1, graph=False, group_size=2)
    for (W, H, D) in shapes:
        b.add_pair(W, H, 0.0, 1.0, float(D - 1))
        ref.add_pair(W, H, 0.0, 1.0, float(D - 1))
    host = (lambda t: t.pin_memory()) if pinned else (lambda t: t)
    hl = [host(torch.zeros((H, W, 4), dtype=torch.float32)) for (W, H, D) in shapes]
    hr = [host(torch.zeros((H, W, 4), dtype=torch.float32)) for (W, H, D) in shapes]
    ho = [host(torch.full((H, W), -7.0, dtype=torch.float32)) for (W, H, D) in shapes]
    for rnd in range(4):
        sc = [scenes.voronoi_scene(W, H, D, seed=300 + 10 * rnd + i, cells=4, off_range=(1, D - 2))
              for i, (W, H, D) in enumerate(shapes)]
        for i, s in enumerate(sc):
            hl[i].copy_(torch.from_numpy(s["left"]))
            hr[i].copy_(torch.from_numpy(s["right"]))
            ref.set_images(i, s["left"], s["right"])
        outs = list(ho)
        outs[1] = None  # no copy out for pair 1
        ho[1].fill_(-7.0)
        b.run_host(hl, hr, outs, 0.5, 1.5, 3, 4)
        b.check()
        ref.run(0.5, 1.5, 3, 4)
        ref.check()
        for i in range(len(shapes)):
            want = ref.get_output(i)
            if i == 1:
                assert (ho[1].numpy() == -7.0).all()
                assert np.array_equal(b.output_device(1).cpu().numpy(), want)
            else:
                assert np.array_equal(ho[i].numpy(), want), (rnd, i)


def test_net_batch_of_two(cuda, oracle):
    """StereoNet with n = 2: each pair's volume equals the oracle's."""
    torch = cuda
    from cnncrf import scenes
    from cnncrf.api import StereoNet
    W, H, D = 40, 20, 12
    cfg = oracle.make_cfg(num_layers=3, topology=0, disp_max=float(D - 1))
    p = oracle.padding(cfg)
    params = oracle.xavier_params(cfg, seed=4)
    sc = [scenes.voronoi_scene(W, H, D, seed=s, cells=3, off_range=(1, D - 2)) for s in (1, 2)]
    lp = np.stack([np.pad(s["left"], ((p, p), (p, p), (0, 0)), mode="symmetric") for s in sc])
    rp = np.stack([np.pad(s["right"], ((p, p), (p, p), (0, 0)), mode="symmetric") for s in sc])
    net = StereoNet(3, 2, 3, H + 2 * p, W + 2 * p, with_pairwise=True)
    vol = torch.empty((2, H, W, D), device="cuda")
    pw = torch.zeros((2, 2, H, W), device="cuda")
    net.init_net(0.0, float(D - 1), 1.0, unary_out=vol, pairwise_out=pw)
    net.init_xavier(4)
    net.predict(torch.from_numpy(lp).cuda(), torch.from_numpy(rp).cuda())
    lst = oracle.disparity_list(0.0, float(D - 1), 1.0)
    for i in range(2):
        ovol, opw = oracle.predict(cfg, params, lp[i], rp[i], lst)
        assert np.array_equal(vol[i].cpu().numpy(), ovol)
        assert np.array_equal(pw[i].cpu().numpy(), opw)


def test_net_batch_output_buffers(cuda):
    """StereoNet with n = 3 sizes its own outputs for every pair, and refuses
    caller buffers that hold fewer pairs than the library would write."""
    torch = cuda
    from cnncrf.api import StereoNet
    net = StereoNet(3, 3, 3, 26, 46, with_pairwise=True)
    net.init_net(0.0, 7.0, 1.0)
    assert tuple(net.volume.shape) == (3, 22, 42, 8) and tuple(net.pairwise_out.shape) == (3, 2, 22, 42)
    with pytest.raises(ValueError):
        StereoNet(3, 3, 3, 26, 46).init_net(0.0, 7.0, 1.0, unary_out=torch.empty((22, 42, 8), device="cuda"))


def test_uneven_batch_full_size_equals_single(cuda):
    """The uneven batch's four sizes and ranges at full size (480x320/D64,
    720x480/D96, 1242x375/D128, 1440x960/D192), two pairs each, replayed as
    one CUDA graph: every pair's labels, disparities and bound equal those of
    a single-pair run."""
    from cnncrf import scenes, _lib as L
    from cnncrf.api import StereoBatch
    layers, iters, crf = 7, 8, (0.5, 1.5, 3)
    sc = scenes.uneven_scenes(2, seed0=7)
    b = StereoBatch(precision=L.BF16, num_layers=layers, seed=0, graph=True, group_size=0)
    for s in sc:
        b.add_pair(s["W"], s["H"], 0.0, 1.0, float(s["D"] - 1))
    for rnd in range(2):  # eager run, then the captured graph
        for i, s in enumerate(sc):
            b.set_images(i, s["left"], s["right"])
        b.run(*crf, iters)
    b.check()
    for i, s in enumerate(sc):
        lab, disp, lb = single_run(L, s, L.BF16, float(s["D"] - 1), layers, iters, crf)
        assert np.array_equal(b.labels_device(i).cpu().numpy(), lab), i
        assert np.array_equal(b.get_output(i), disp), i
        assert b.lower_bound(i) == lb, i


def test_batch_autotune_tunes_conv_forms_and_changes_no_bit(cuda):
    """StereoBatch.autotune times every launch form of the tensor-core
    convolutions (2-CTA pairs or single CTAs, 2-4 stages) per layer shape and
    enters the fastest in the process-wide table, beside the CRF tiles; the
    run after it (using the tuned forms and tiles) gives the same bits."""
    from cnncrf import scenes, tuning, _lib as L
    from cnncrf.api import StereoBatch
    torch = cuda
    tuning.clear_conv()
    shapes = [(300, 40, 32), (300, 40, 32), (140, 24, 16)]
    sc = [scenes.voronoi_scene(W, H, D, seed=70 + i, cells=4, off_range=(1, D - 2)) for i, (W, H, D) in
          enumerate(shapes)]
    b = StereoBatch(precision=L.BF16, num_layers=3, seed=0, graph=True)
    for (W, H, D) in shapes:
        b.add_pair(W, H, 0.0, 1.0, float(D - 1))
    for i, s in enumerate(sc):
        b.set_images(i, s["left"], s["right"])
    b.run(0.5, 1.5, 3, 4)
    b.check()
    before = [b.get_output(i).copy() for i in range(len(shapes))]
    b.autotune(0.5, 1.5, 3, 4)
    forms = tuning.conv_forms()
    # per group: feature layers 2..3 and the pairwise layer 2, each its own shape
    assert len(forms) >= 6, forms
    for f in forms:
        assert f["pair"] in (0, 1) and 2 <= f["stages"] <= 4 and f["ms"] > 0
    for rnd in range(2):  # eager with the tuned forms, then capture and replay
        for i, s in enumerate(sc):
            b.set_images(i, s["left"], s["right"])
        b.run(0.5, 1.5, 3, 4)
        b.check()
        for i in range(len(shapes)):
            assert np.array_equal(b.get_output(i), before[i]), (rnd, i)
    tuning.clear_conv()
