"""Our CUDA kernels against the REFERENCE'S OWN CUDA kernels, bit for bit.

1. Against the committed outputs of the reference's kernels
   (tests/golden/ref_kernels.npz, see tests/test_oracle_refkernels.py): our
   correlation (FP32 path), grey, census, remap, warp, quadratic fit, fused TV
   iterations, left-right check and QuadDirect, through the C ABI.
2. Live, where the reference-kernel module oracle/_ref/refkernels.fatbin was
   built (it can only be built where the reference tree exists): the same
   stages on fresh seeded inputs of other sizes, both run on this GPU.

Entries where the reference reads outside the row or volume it indexes are
excluded, as in tests/test_oracle_refkernels.py."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_ref_golden as G  # noqa: E402

FIX = os.path.join(HERE, "golden", "ref_kernels.npz")


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _corr_ours(torch, fl_chw, fr_chw, lst):
    from cnncrf import api
    stored = (-np.asarray(lst, np.float32)).astype(np.float32)
    return api.correlation_forward(_dev(torch, fl_chw[None]), _dev(torch, fr_chw[None]), stored).cpu().numpy()


def _inside(W, lst, shape):
    return np.broadcast_to(np.arange(W)[None, :, None] - np.asarray(lst)[None, None, :] <= W - 1, shape)


def _stages_ours(torch, x):
    """Our outputs for the fixture's stages (a dict keyed like the fixture)."""
    from cnncrf import api
    o = {}
    for name, (a, b, s) in G.CORR_LISTS.items():
        o["corr_" + name] = _corr_ours(torch, x["corr_fl"], x["corr_fr"], G.disparity_list(a, b, s))
    o["gray"] = api.rgb_to_gray(_dev(torch, x["img"])).cpu().numpy()
    for name, (dmin, dstep) in G.CENSUS["lists"].items():
        o["census_" + name] = api.census_volume(_dev(torch, x["g1"]), _dev(torch, x["g2"]), G.CENSUS["fs"], dmin,
                                                dstep, G.CENSUS["D"], G.CENSUS["lam"]).cpu().numpy()
    o["remap"] = api.remap_solution(_dev(torch, x["labels"]), 2.0, 0.5).cpu().numpy()
    o["warp"] = api.warp_image(_dev(torch, x["wimg"]), _dev(torch, x["wu"])).cpu().numpy()
    for s in G.FIT["steps"]:
        o["fit_%g" % s] = api.tv_fit(_dev(torch, x["vol3"]), s, G.FIT["lam"]).cpu().numpy()
    T = G.TV
    tv = api.tv_iterate(_dev(torch, x["tv_u0"]), _dev(torch, x["tv_u0"]), _dev(torch, x["tv_qf"]),
                        _dev(torch, x["tv_wx"]), _dev(torch, x["tv_wy"]), T["C"], 0.1, T["step"], T["iters"])
    for k, t in zip(("u", "u_", "p", "q"), tv):
        o["tv_" + k] = t.cpu().numpy()
    o["lrcheck"] = api.left_right_check(_dev(torch, x["lr_left"]), _dev(torch, x["lr_right"].astype(np.float32)),
                                        1.0).cpu().numpy()
    Q = G.QF
    uq = (x["qf_labels"] * np.float32(Q["dstep"]) + np.float32(Q["dmin"])).astype(np.float32)
    o["quadfit"] = api.quad_fit_direct(_dev(torch, uq), _dev(torch, x["qf_c1"]), Q["dmin"], Q["dstep"]).cpu().numpy()
    return o


def test_ours_equal_reference_kernel_fixture(cuda):
    torch = cuda
    f = np.load(FIX)
    x = {k: f[k] for k in f.files}
    ours = _stages_ours(torch, x)
    W = x["corr_fl"].shape[2]
    for k, got in ours.items():
        want = x[k]
        if k.startswith("corr_"):
            lst = G.disparity_list(*G.CORR_LISTS[k[5:]])
            m = _inside(W, lst, want.shape)
            assert np.array_equal(got.reshape(want.shape)[m], want[m]), k
        else:
            assert np.array_equal(got, want), k


def test_ours_equal_reference_kernels_live(cuda):
    """Fresh inputs of other sizes; skipped where the reference-kernel module
    was not built (no reference tree on the machine that built this copy)."""
    torch = cuda
    from oracle import refkernels as R
    if not R.available():
        pytest.skip("oracle/_ref/refkernels.fatbin not built here (needs the reference tree)")
    from cnncrf import api
    rng = np.random.default_rng(77)
    # correlation: 100 channels, a 64-entry integer list and a 40-entry half-step list
    Cc, H, W = 100, 9, 131
    fl = (rng.standard_normal((Cc, H, W)) * 0.1).astype(np.float32)
    fr = (rng.standard_normal((Cc, H, W)) * 0.1).astype(np.float32)
    for lst in (G.disparity_list(0.0, 63.0, 1.0), G.disparity_list(1.0, 20.5, 0.5)):
        want = R.correlation(fl, fr, lst)
        m = _inside(W, lst, want.shape)
        assert np.array_equal(_corr_ours(torch, fl, fr, lst)[m], want[m])
    # census with the CLI's default window (filter size 7), both directions
    Hg, Wg = 37, 61
    g1 = (rng.integers(0, 256, (Hg, Wg)) / 255.0).astype(np.float32)
    g2 = np.roll(g1, -5, axis=1).astype(np.float32)
    for dmin in (0.0, -23.0):
        want = R.census(g1, g2, 7, dmin, 1.0, 24, 1.0)
        got = api.census_volume(_dev(torch, g1), _dev(torch, g2), 7, dmin, 1.0, 24, 1.0).cpu().numpy()
        assert np.array_equal(got, want), dmin
    # TV: 7 iterations (one fused launch) at step 0.5 on several tiles
    Ht, Wt = 45, 83
    u0 = (rng.random((Ht, Wt)) * 20).astype(np.float32)
    qf = np.stack([rng.standard_normal((Ht, Wt)), rng.random((Ht, Wt)) * 2], -1).astype(np.float32)
    wx, wy = (rng.random((Ht, Wt)) * 3).astype(np.float32), (rng.random((Ht, Wt)) * 3).astype(np.float32)
    want = R.tv_iterate(u0, u0, qf, wx, wy, 2.0, 0.5, 7)
    got = api.tv_iterate(_dev(torch, u0), _dev(torch, u0), _dev(torch, qf), _dev(torch, wx), _dev(torch, wy), 2.0,
                         0.1, 0.5, 7)
    for k, a, b in zip(("u", "u_", "p", "q"), got, want):
        assert np.array_equal(a.cpu().numpy(), b), k
    # warp and the 3-label fit at a fractional step
    img = rng.random((Ht, Wt, 4)).astype(np.float32)
    u = (rng.random((Ht, Wt)) * 30 - 4).astype(np.float32)
    assert np.array_equal(api.warp_image(_dev(torch, img), _dev(torch, u)).cpu().numpy(), R.warp(img, u))
    vol3 = rng.standard_normal((Ht, Wt, 3)).astype(np.float32)
    assert np.array_equal(api.tv_fit(_dev(torch, vol3), 0.25, 2.0).cpu().numpy(), R.tv_fit(vol3, 0.25, 2.0))
