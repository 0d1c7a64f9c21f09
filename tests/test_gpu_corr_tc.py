"""GPU tests of the tensor-core correlation (tcgen05 banded GEMM with the
unary in its epilogue) on the BF16 path: the cost volume equals an FP64
correlation of the same BF16 feature maps, for integer disparity lists with
positive, negative and offset ranges, partial last tiles, both unaries,
batches of pairs and wide lists cut into disparity parts; lists the kernel
does not take go to the SIMT kernel."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pad(img, p):
    return np.pad(img, ((p, p), (p, p), (0, 0)), mode="symmetric")


def corr_f64(fl, fr, disparities):
    """C[y, x, k] = <fL(y, x), fR(y, x - d_k)>, 0 where x - d_k is outside the row."""
    H, W, _ = fl.shape
    fl = fl.astype(np.float64)
    fr = fr.astype(np.float64)
    out = np.zeros((H, W, len(disparities)))
    for k, d in enumerate(disparities):
        xs = np.arange(W) - int(d)
        ok = (xs >= 0) & (xs < W)
        out[:, ok, k] = np.einsum("hwc,hwc->hw", fl[:, ok], fr[:, xs[ok]])
    return out


def unary_f64(c, unary):
    if unary == 1:
        return 1.0 - c
    e = np.exp(c - c.max(axis=2, keepdims=True))
    return -e / e.sum(axis=2, keepdims=True)


def run_net(torch, L, scenes_list, W, H, dmin, dmax, unary, layers=3, step=1):
    from cnncrf.api import StereoNet
    n = len(scenes_list)
    p = layers  # every layer 3x3, valid: the receptive field loses one pixel per side per layer
    net = StereoNet(layers, n, 3, H + 2 * p, W + 2 * p, topology=L.TOPO_ALL3X3, unary=unary, precision=L.BF16)
    assert net.padding() == p
    D = int(round(dmax - dmin)) // step + 1
    vol = torch.empty((n, H, W, D), device="cuda")
    net.init_net(float(dmin), float(dmax), float(step), unary_out=vol)
    net.init_xavier(7)
    lp = np.stack([_pad(s["left"], p) for s in scenes_list])
    rp = np.stack([_pad(s["right"], p) for s in scenes_list])
    L.profile_reset()
    L.profile_enable(True)
    try:
        net.predict(torch.from_numpy(lp).cuda(), torch.from_numpy(rp).cuda())
        torch.cuda.synchronize()
        kernels = L.profile_kernels()
    finally:
        L.profile_enable(False)
    return net, vol, kernels


@pytest.mark.parametrize("dmin,dmax,unary", [(0, 47, 1), (0, 47, 0), (-3, 4, 1), (5, 132, 1), (0, 127, 0)])
def test_corr_tc_matches_f64_on_bf16_features(cuda, dmin, dmax, unary):
    torch = cuda
    from cnncrf import scenes, _lib as L
    W, H = 300, 6  # three tiles per row, the last one partial
    sc = scenes.voronoi_scene(W, H, 64, seed=11, cells=4, off_range=(1, 40))
    net, vol, kernels = run_net(torch, L, [sc], W, H, dmin, dmax, unary)
    assert "corr_tc" in kernels and "corr" not in kernels, kernels
    fl = net.features(0).cpu().numpy()
    fr = net.features(1).cpu().numpy()
    ref = unary_f64(corr_f64(fl, fr, np.arange(dmin, dmax + 1)), unary)
    got = vol[0].cpu().numpy()
    tol = 2e-5 if unary == 1 else 1e-4
    err = np.abs(got - ref)
    assert err.max() < tol, (err.max(), np.unravel_index(err.argmax(), err.shape))


def test_corr_tc_batch_equals_single(cuda):
    """Pairs batched through one launch give each pair's single-pair volume bit for bit."""
    torch = cuda
    from cnncrf import scenes, _lib as L
    W, H = 170, 5
    sc = [scenes.voronoi_scene(W, H, 32, seed=s, cells=3, off_range=(1, 30)) for s in (21, 22, 23)]
    _, vol3, k3 = run_net(torch, L, sc, W, H, 0, 31, 1)
    assert "corr_tc" in k3
    for i in range(3):
        _, vol1, _ = run_net(torch, L, [sc[i]], W, H, 0, 31, 1)
        assert torch.equal(vol3[i], vol1[0]), i


@pytest.mark.parametrize("dmin,dmax", [(0, 140), (0, 191), (0, 255), (-40, 260)])
def test_wide_band_in_parts(cuda, dmin, dmax):
    """Bands wider than a tile's 128 extra columns run as 2-3 disparity parts
    on the tensor cores (D = 192 is the 1440 x 960 pairs' range)."""
    torch = cuda
    from cnncrf import scenes, _lib as L
    W, H = 300, 3
    sc = scenes.voronoi_scene(W, H, 64, seed=5, cells=3, off_range=(1, 40))
    net, vol, kernels = run_net(torch, L, [sc], W, H, dmin, dmax, 1)
    assert "corr_tc" in kernels and "corr" not in kernels, kernels
    fl = net.features(0).cpu().numpy()
    fr = net.features(1).cpu().numpy()
    ref = unary_f64(corr_f64(fl, fr, np.arange(dmin, dmax + 1)), 1)
    err = np.abs(vol[0].cpu().numpy() - ref)
    assert err.max() < 2e-5, (err.max(), np.unravel_index(err.argmax(), err.shape))


def test_wide_softmax_uses_simt_kernel(cuda):
    """The softmax over a band wider than one tile needs all D taps of a pixel
    together: it goes to the SIMT kernel."""
    torch = cuda
    from cnncrf import scenes, _lib as L
    W, H = 200, 2
    sc = scenes.voronoi_scene(W, H, 64, seed=6, cells=3, off_range=(1, 40))
    net, vol, kernels = run_net(torch, L, [sc], W, H, 0, 140, 0)
    assert "corr" in kernels and "corr_tc" not in kernels, kernels
    fl = net.features(0).cpu().numpy()
    fr = net.features(1).cpu().numpy()
    ref = unary_f64(corr_f64(fl, fr, np.arange(0, 141)), 0)
    assert np.abs(vol[0].cpu().numpy() - ref).max() < 1e-4


def test_band_beyond_both_kernels_is_an_error(cuda):
    """301 disparities two pixels apart: more than four tensor-core parts, and
    a band (600 columns) past the SIMT kernel's shared memory."""
    torch = cuda
    from cnncrf import scenes, _lib as L
    from cnncrf.api import CnnCrfError
    sc = scenes.voronoi_scene(200, 2, 64, seed=6, cells=3, off_range=(1, 40))
    with pytest.raises(CnnCrfError) as e:
        run_net(torch, L, [sc], 200, 2, 0, 600, 1, step=2)
    assert e.value.status == L.EINVAL
