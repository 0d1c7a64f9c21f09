"""GPU parity of the non-CNN parts of the Stereo pipeline against the CPU
oracle, bit for bit: grey conversion, the census cost volume, the
image-gradient edge weights, QuadDirect refinement, the left-right check,
the CENSUS and COLORCNN (non-pairwise) CRF pipelines through Stereo, and the
stereo_img command line end to end on PNG files."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _images(W, H, D, seed):
    from cnncrf import scenes
    s = scenes.voronoi_scene(W, H, D, seed=seed, cells=5, off_range=(1, D - 2), slope=0.05)
    return s["left"], s["right"]


def test_gray_bitexact(cuda, oracle):
    torch = cuda
    from cnncrf import api
    rgba = np.random.default_rng(0).random((37, 61, 4)).astype(np.float32)
    assert np.array_equal(api.rgb_to_gray(dev(rgba, torch)).cpu().numpy(), oracle.gray(rgba))


CENSUS_CASES = [
    # W, H, dmin, dstep, depth, filter size
    (61, 37, 0.0, 1.0, 16, 7),
    (64, 40, 1.0, 1.0, 12, 3),
    (45, 29, 0.5, 0.5, 20, 2),   # fractional: linear reads of the other image
    (33, 17, -4.0, 1.0, 9, 1),
    (52, 30, -15.0, 1.0, 16, 5),  # the right-reference list, -dmax upwards
    (19, 11, 0.25, 0.75, 7, 16),  # the largest window
    (1, 9, 0.0, 1.0, 4, 2),       # one column: every read clamps
]


@pytest.mark.parametrize("W,H,dmin,dstep,D,fs", CENSUS_CASES)
def test_census_volume_bitexact(cuda, oracle, W, H, dmin, dstep, D, fs):
    torch = cuda
    from cnncrf import api
    left, right = _images(max(W, 8), H, 8, seed=W)
    g1, g2 = oracle.gray(left[:, :W]), oracle.gray(right[:, :W])
    vol = api.census_volume(dev(g1, torch), dev(g2, torch), fs, dmin, dstep, D, 1.0).cpu().numpy()
    ovol = oracle.census(g1, g2, fs, oracle.census_list(dmin, dstep, D), 1.0)
    assert np.array_equal(vol, ovol), np.abs(vol - ovol).max()
    # lambda scales the normalised count
    vol2 = api.census_volume(dev(g1, torch), dev(g2, torch), fs, dmin, dstep, D, 0.7).cpu().numpy()
    assert np.array_equal(vol2, oracle.census(g1, g2, fs, oracle.census_list(dmin, dstep, D), 0.7))


def test_census_errors(cuda):
    torch = cuda
    from cnncrf import api, _lib as L
    g = torch.zeros((8, 8), device="cuda")
    for fs in (0, 17):
        with pytest.raises(api.CnnCrfError) as e:
            api.census_volume(g, g, fs, 0.0, 1.0, 4)
        assert e.value.status == L.EINVAL


EDGE_CASES = [
    # H, W, alpha, beta, lambda
    (37, 61, 20.0, 0.8, 0.4),
    (30, 52, 10.0, 1.0, 1.0),
    (30, 52, 0.0, 0.8, 0.5),   # alpha 0: lambda |gradient|
    (1, 9, 20.0, 0.8, 0.4),
    (7, 1, 5.0, 2.0, 3.0),
]


@pytest.mark.parametrize("H,W,alpha,beta,lam", EDGE_CASES)
def test_edge_weights_bitexact(cuda, oracle, H, W, alpha, beta, lam):
    torch = cuda
    from cnncrf import api
    rng = np.random.default_rng(H * W)
    g = rng.random((H, W)).astype(np.float32)
    g[:, W // 2:] += 0.5  # a vertical edge
    wx, wy = api.edge_weights(dev(g, torch), alpha, beta, lam)
    owx, owy = oracle.edge_weights(g, alpha, beta, lam)
    assert np.array_equal(wx.cpu().numpy(), owx)
    assert np.array_equal(wy.cpu().numpy(), owy)
    if alpha > 0:
        assert owx.min() >= 1e-6 and owx.max() <= lam


@pytest.mark.parametrize("dmin,dstep,D", [(0.0, 1.0, 16), (1.0, 1.0, 9), (0.5, 0.5, 21), (-3.0, 0.25, 13)])
def test_quad_fit_direct_bitexact(cuda, oracle, dmin, dstep, D):
    torch = cuda
    from cnncrf import api
    rng = np.random.default_rng(D)
    H, W = 23, 41
    lab = rng.integers(0, D, (H, W)).astype(np.int32)
    lab[0, :3] = [0, D - 1, 1]  # the two ends stay, the next one moves
    u = oracle.remap(lab, dmin, dstep)
    c1 = rng.standard_normal((H, W, D)).astype(np.float32)
    got = api.quad_fit_direct(dev(u, torch), dev(c1, torch), dmin, dstep).cpu().numpy()
    want = oracle.quadfit_direct(u, c1, dmin, dstep)
    assert np.array_equal(got, want)
    assert got[0, 0] == u[0, 0] and got[0, 1] == u[0, 1]


def test_left_right_check_bitexact(cuda, oracle):
    torch = cuda
    from cnncrf import api
    rng = np.random.default_rng(4)
    H, W = 27, 70
    left = (rng.random((H, W)) * 20).astype(np.float32)
    left[:, ::3] = np.floor(left[:, ::3])  # integer and fractional reads
    right = -(left + rng.standard_normal((H, W)).astype(np.float32) * 0.8)
    for th in (0.5, 1.0, 3.0):
        got = api.left_right_check(dev(left, torch), dev(right, torch), th).cpu().numpy()
        want = oracle.lr_check(left, right, th)
        assert np.array_equal(got, want)
        assert ((got == -1.0) | (got == left)).all()


def _census_crf_oracle(oracle, left, right, fs, dmin, dstep, D, L1, L2, delta, iters, alpha, beta, lam,
                       lr, shape, quad):
    g_ref, g_other = (oracle.gray(left), oracle.gray(right)) if lr else (oracle.gray(right), oracle.gray(left))
    dmax = np.float32(dmin) + np.float32(D - 1) * np.float32(dstep)  # the range after depth rounding
    start = dmin if lr else -float(dmax)
    vol = oracle.census(g_ref, g_other, fs, oracle.census_list(start, dstep, D), 1.0)
    wx, wy = oracle.edge_weights(g_ref, alpha, beta, lam)
    labels, lb, _, c1 = oracle.crf(vol, wx, wy, L1, L2, delta, iters, shape=shape, want_c1=True)
    disp = oracle.remap(labels, start, dstep)
    if quad:
        disp = oracle.quadfit_direct(disp, c1, dmin, dstep)
    return dict(vol=vol, wx=wx, wy=wy, labels=labels, lb=lb, disp=disp)


@pytest.mark.parametrize("lr,fs,dmin,dmax", [(True, 7, 1.0, 16.0), (False, 4, 0.0, 13.0), (True, 2, 0.0, 31.0)])
def test_stereo_census_crf_bitexact(cuda, oracle, lr, fs, dmin, dmax):
    """Stereo with CENSUS matching: computeSlackPropagation (census volume,
    edge weights, CRF, remap), then fuseQuadFitDirect on the left view."""
    from cnncrf import _lib as L
    from cnncrf.api import Stereo
    W, H = 58, 34
    left, right = _images(W, H, 16, seed=fs)
    st = Stereo()
    st.initialize(W, H, dmin, 1.0, dmax)
    st.set_matching_function(L.MATCH_CENSUS)
    st.set_filter_size(fs)
    st.set_color_images(left, right)
    st.compute_slack_propagation(1.0, 12.0, 2, 4, 20.0, 0.8, 0.4, lr)
    D = st.get_depth()
    r = _census_crf_oracle(oracle, left, right, fs, dmin, 1.0, D, 1.0, 12.0, 2, 4, 20.0, 0.8, 0.4, lr,
                           L.RHO_STEP, quad=lr)
    assert np.array_equal(st.volume_device().cpu().numpy(), r["vol"])
    wx, wy = st.weights_device()
    assert np.array_equal(wx.cpu().numpy(), r["wx"]) and np.array_equal(wy.cpu().numpy(), r["wy"])
    assert np.array_equal(st.labels_device().cpu().numpy(), r["labels"])
    assert st.lower_bound() == r["lb"]
    if lr:
        st.fuse_quad_fit_direct()
    assert np.array_equal(st.get_output(), r["disp"])


def test_stereo_colorcnn_crf_edge_weights(cuda, oracle):
    """COLORCNN without the pairwise net: the CRF runs on image-gradient weights."""
    from cnncrf import _lib as L
    from cnncrf.api import Stereo
    W, H = 48, 28
    left, right = _images(W, H, 12, seed=2)
    st = Stereo()
    st.initialize(W, H, 0.0, 1.0, 11.0)
    st.set_matching_function(L.MATCH_COLORCNN)
    st.set_num_layers(3)
    st.set_xavier_seed(6)
    st.set_color_images(left, right)
    st.compute_slack_propagation(1.0, 8.0, 2, 3, 10.0, 1.0, 0.6)
    vol = st.volume_device().cpu().numpy()
    owx, owy = oracle.edge_weights(oracle.gray(left), 10.0, 1.0, 0.6)
    wx, wy = st.weights_device()
    assert np.array_equal(wx.cpu().numpy(), owx) and np.array_equal(wy.cpu().numpy(), owy)
    labels, lb, _, _ = oracle.crf(vol, owx, owy, 1.0, 8.0, 2, 3)
    assert np.array_equal(st.labels_device().cpu().numpy(), labels)
    assert st.lower_bound() == lb
    assert np.array_equal(st.get_output(), oracle.remap(labels, 0.0, 1.0))


def test_stereo_census_errors(cuda):
    from cnncrf import _lib as L
    from cnncrf.api import Stereo, CnnCrfError
    st = Stereo()
    with pytest.raises(CnnCrfError) as e:
        st.fuse_quad_fit_direct()  # no solve yet
    assert e.value.status == L.ESTATE
    for fs in (0, 17):
        with pytest.raises(CnnCrfError) as e:
            st.set_filter_size(fs)
        assert e.value.status == L.EINVAL


def _write_pair(tmp_path, W, H, seed):
    from cnncrf import imageio
    left, right = _images(W, H, 16, seed)
    paths = []
    for name, im in (("l.png", left), ("r.png", right)):
        p = str(tmp_path / name)
        imageio.write_png(p, np.rint(np.clip(im[..., :3], 0, 1) * 255).astype(np.uint8))
        paths.append(p)
    return paths


def test_cli_census_crf_quaddirect(cuda, oracle, tmp_path):
    """stereo_img im0 im1 --matching CENSUS --refinement QuadDirect: the PFM
    equals the oracle's composition, the PNG is its 16-bit encoding, and the
    _wx/_wy files are the edge weights."""
    from cnncrf import cli, imageio, _lib as L
    W, H = 56, 32
    l, r = _write_pair(tmp_path, W, H, seed=3)
    out = str(tmp_path / "res")
    rc = cli.main([l, r, "--disp-max", "15", "--filter-size", "3", "--refinement", "QuadDirect",
                   "--output-file", out, "--crf-iterations", "3"])
    assert rc == 0
    left, right = imageio.read_png(l), imageio.read_png(r)
    from cnncrf.api import Stereo
    st = Stereo()
    st.initialize(W, H, 1.0, 1.0, 15.0)
    D = st.get_depth()
    o = _census_crf_oracle(oracle, left, right, 3, 1.0, 1.0, D, 1.0, 12.0, 2, 3, 20.0, 0.8, 0.4, True,
                           L.RHO_STEP, quad=True)
    disp = imageio.read_pfm(out + ".pfm")
    assert np.array_equal(disp, o["disp"])
    png = imageio.read_png(out + ".png")[..., 0] * 65535.0
    assert np.array_equal(np.rint(png).astype(np.uint16), imageio.disparity_to_png16(disp))
    # getWx / getWy with alpha > 0 recompute the edge weights at lambda 1
    wx1, wy1 = oracle.edge_weights(oracle.gray(left), 20.0, 0.8, 1.0)
    assert np.array_equal(imageio.read_pfm(out + "_wx.pfm"), wx1)
    assert np.array_equal(imageio.read_pfm(out + "_wy.pfm"), wy1)


def test_cli_none_then_load(cuda, oracle, tmp_path):
    """--inference NONE writes the census volume as .npy; --matching LOAD reads
    it back and solves the CRF on it with edge weights."""
    from cnncrf import cli, imageio
    W, H = 40, 24
    l, r = _write_pair(tmp_path, W, H, seed=8)
    out = str(tmp_path / "vol")
    assert cli.main([l, r, "--disp-min", "0", "--disp-max", "11", "--filter-size", "2", "--inference", "NONE",
                     "--output-file", out]) == 0
    vol = np.load(out + ".npy")
    left, right = imageio.read_png(l), imageio.read_png(r)
    g1, g2 = oracle.gray(left), oracle.gray(right)
    assert np.array_equal(vol, oracle.census(g1, g2, 2, oracle.census_list(0.0, 1.0, vol.shape[2]), 1.0))
    out2 = str(tmp_path / "load")
    assert cli.main([l, r, "--disp-min", "0", "--disp-max", "11", "--matching", "LOAD", "--volume", out + ".npy",
                     "--output-file", out2, "--lambda", "0.7", "--alpha", "5"]) == 0
    wx, wy = oracle.edge_weights(g1, 5.0, 0.8, 0.7)
    labels, _, _, _ = oracle.crf(vol, wx, wy, 1.0, 12.0, 2, 4)
    assert np.array_equal(imageio.read_pfm(out2 + ".pfm"), oracle.remap(labels, 0.0, 1.0))


def test_cli_colorpair_argmax_and_errors(cuda, oracle, tmp_path):
    from cnncrf import cli, imageio
    W, H = 44, 26
    l, r = _write_pair(tmp_path, W, H, seed=5)
    out = str(tmp_path / "am")
    assert cli.main([l, r, "--matching", "COLORPAIR", "--num-layers", "3", "--xavier-seed", "4",
                     "--inference", "ARGMAX", "--disp-min", "0", "--disp-max", "9", "--output-file", out]) == 0
    disp = imageio.read_pfm(out + ".pfm")
    assert disp.shape == (H, W) and disp.min() >= 0.0 and disp.max() <= 15.0  # 10 labels round up to 16
    assert np.all(disp == np.floor(disp))  # argmax of an integer list
    # reference error exits: unknown refinement / matching, and a missing parameter file
    assert cli.main([l, r, "--refinement", "Bogus", "--filter-size", "1", "--disp-max", "4",
                     "--output-file", out]) == 1
    assert cli.main([l, r, "--matching", "COLORCNN", "--num-layers", "3", "--parameter-file",
                     str(tmp_path / "missing"), "--disp-max", "4", "--output-file", out]) == 1
