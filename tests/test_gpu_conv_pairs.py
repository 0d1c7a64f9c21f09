"""GPU tests of the tensor-core convolution run as 2-CTA pairs (tcgen05
cta_group::2: M = 256 MMAs spanning two SMs, each CTA staging half of every
tap's weights) against the single-CTA form on the same inputs: the inference
nets' features, cost volume and pairwise output (convolution modes 0-2), and a
training step's gradients (the input-gradient modes 3-4 too), on ragged widths
and on tile counts where the last pair's second CTA has no tile."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def set_pairs(on):
    from cnncrf import _lib as L
    L.check(L.lib().cnncrf_set_conv_pairs(1 if on else 0))


def get_pairs():
    from cnncrf import _lib as L
    v = ctypes.c_int(-1)
    L.check(L.lib().cnncrf_get_conv_pairs(ctypes.byref(v)))
    return v.value


@pytest.fixture
def restore_pairs(cuda):
    yield
    set_pairs(True)


def compare(a, b, what, tol):
    d = (a - b).abs().max().item()
    print("%s: %s" % (what, "bit-exact" if bool((a == b).all()) else "max |diff| %.3g" % d))
    assert d <= tol, (what, d)


@pytest.mark.parametrize("W,H", [(300, 21), (517, 9), (1242, 6)])
def test_paired_convolution_matches_single_cta(cuda, oracle, restore_pairs, W, H):
    """Features (BF16 after tanh), the 1 - dot volume and the pairwise output
    with pairs on and off.  Both forms sum each output over the same K order
    in FP32; the bound allows one BF16 rounding step, compounded over 7 layers."""
    torch = cuda
    from cnncrf import scenes, _lib as L
    from cnncrf.api import StereoNet
    assert get_pairs() == 1  # on by default
    s = scenes.voronoi_scene(W, H, 16, seed=4, cells=5)
    cfg = oracle.make_cfg(num_layers=7, topology=1, unary=1, disp_max=31.0)
    p = oracle.padding(cfg)
    pad = lambda im: np.pad(im, ((p, p), (p, p), (0, 0)), mode="symmetric")
    lp, rp = pad(s["left"]), pad(s["right"])
    out = {}
    for on in (True, False):
        set_pairs(on)
        net = StereoNet(7, 1, 3, H + 2 * p, W + 2 * p, topology=1, unary=1, precision=L.BF16, with_pairwise=True)
        net.init_net(0.0, 31.0, 1.0)
        net.init_xavier(0)
        vol = net.predict(torch.from_numpy(lp).cuda(), torch.from_numpy(rp).cuda()).clone()
        torch.cuda.synchronize()
        out[on] = (vol, net.features(0).clone(), net.features(1).clone(), net.pairwise_out.clone())
    for a, b, what in zip(out[True], out[False], ("volume", "left features", "right features", "pairwise")):
        compare(a, b, what, 5e-2)


def test_paired_convolution_training_gradients(cuda, oracle, restore_pairs):
    """A BF16 training step's volume, pairwise output and every gradient slot
    with pairs on and off (forward modes 0-2, recomputation, input gradients
    in modes 3-4 with the fused tanh' and bias sums), relative to each slot's
    largest value."""
    torch = cuda
    from cnncrf import scenes, _lib as L
    from cnncrf.train import Trainer
    n, W, H, D = 2, 300, 20, 24
    sc = [scenes.voronoi_scene(W, H, D, seed=3 + 10 * i, cells=4, off_range=(1, D - 2), slope=0.05)
          for i in range(n)]
    left = torch.from_numpy(np.stack([s["left"] for s in sc])).cuda()
    right = torch.from_numpy(np.stack([s["right"] for s in sc])).cuda()
    res = {}
    for on in (True, False):
        set_pairs(on)
        t = Trainer(n, W, H, num_layers=4, topology=1, feat_channels=100, pw_channels=64, disp_max=float(D - 1),
                    precision=L.BF16, checkpoint_every=2)
        t.init_xavier(3)
        vol, pw = t.forward(left, right)
        rng = np.random.default_rng(6)
        gvol = torch.from_numpy(rng.standard_normal(tuple(vol.shape)).astype(np.float32)).cuda()
        gpw = torch.from_numpy(rng.standard_normal(tuple(pw.shape)).astype(np.float32)).cuda()
        t.backward(gvol, gpw)
        torch.cuda.synchronize()
        res[on] = (vol.clone(), pw.clone(), [t.get_grad(i) for i in range(t.num_params())])
    compare(res[True][0], res[False][0], "volume", 5e-2)
    compare(res[True][1], res[False][1], "pairwise", 5e-2)
    errs = {}
    for i, (a, b) in enumerate(zip(res[True][2], res[False][2])):
        errs[i] = float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-12))
    print("paired vs single-CTA gradients:", {k: float("%.2e" % v) for k, v in errs.items()})
    assert max(errs.values()) < 2e-2, errs
