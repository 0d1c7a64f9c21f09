"""The FP64 oracle's training-step adjoints (oracle_predict_backward) against
FP64 central differences (h = 1e-4) of its own FP64 forward, for every
parameter slot of both nets, and the structured hinge's subgradient on cases
with a known answer.  CPU only: the oracle pins the GPU adjoints."""
import numpy as np
import pytest


def small_case(oracle, layers=3, topology=1, seed=0, W=14, H=9, D=6):
    from cnncrf import scenes
    cfg = oracle.make_cfg(num_layers=layers, topology=topology, in_channels=3, feat_channels=8, unary=1,
                          with_pairwise=1, pw_channels=6, precision=64, disp_min=0.0, disp_max=float(D - 1))
    p = oracle.padding(cfg)
    s = scenes.voronoi_scene(W, H, D, seed=seed, cells=4, off_range=(1, D - 2), slope=0.05)
    lp, rp = oracle.pad_rgba(s["left"], p), oracle.pad_rgba(s["right"], p)
    params = oracle.xavier_params(cfg, seed=seed + 1)
    lst = oracle.disparity_list(0.0, float(D - 1), 1.0)
    return cfg, params, lp, rp, lst


@pytest.mark.parametrize("layers,topology", [(3, 1), (3, 0)])
def test_predict_backward_matches_central_differences(oracle, layers, topology):
    cfg, params, lp, rp, lst = small_case(oracle, layers, topology)
    rng = np.random.default_rng(5)
    vol, pw = oracle.predict(cfg, params, lp, rp, lst)
    gvol = rng.standard_normal(vol.shape)
    gpw = rng.standard_normal(pw.shape)
    grads = oracle.predict_backward(cfg, params, lp, rp, lst, gvol, gpw)

    def S(ps):
        v, q = oracle.predict(cfg, ps, lp, rp, lst)
        return float((gvol * v).sum() + (gpw * q).sum())

    h = 1e-4
    worst = 0.0
    for slot, (prm, g) in enumerate(zip(params, grads)):
        assert g.shape == np.shape(prm)
        flat = np.asarray(prm, np.float32).reshape(-1)
        for idx in rng.choice(flat.size, size=min(4, flat.size), replace=False):
            plus = [np.array(a, np.float32, copy=True) for a in params]
            minus = [np.array(a, np.float32, copy=True) for a in params]
            plus[slot].reshape(-1)[idx] = np.float32(flat[idx] + h)
            minus[slot].reshape(-1)[idx] = np.float32(flat[idx] - h)
            step = float(plus[slot].reshape(-1)[idx]) - float(minus[slot].reshape(-1)[idx])
            fd = (S(plus) - S(minus)) / step
            an = g.reshape(-1)[idx]
            err = abs(fd - an) / max(1.0, abs(an))
            worst = max(worst, err)
            assert err < 1e-6, (slot, idx, fd, an)
    assert worst < 1e-6


def test_hinge_zero_when_the_data_term_picks_the_truth(oracle):
    rng = np.random.default_rng(1)
    H, W, D = 6, 7, 5
    gt = rng.integers(0, D, (H, W)).astype(np.int32)
    vol = np.ones((H, W, D), np.float32)
    vol[np.arange(H)[:, None], np.arange(W)[None, :], gt] = -9.0
    pw = np.zeros((2, H, W), np.float32)
    loss, yh, gvol, gpw = oracle.hinge(vol, pw, gt, 1.0, 0.5, 1.5, 3, 4)
    assert np.array_equal(yh, gt) and loss == 0.0
    assert not gvol.any() and not gpw.any()


def test_hinge_subgradient_when_the_data_term_picks_another_label(oracle):
    """vol prefers label 4 everywhere by 2 (more than the margin), no pairwise
    term: y_hat = 4, loss = sum(vol[gt] - vol[4]) + #mislabelled."""
    H, W, D = 5, 6, 6
    gt = np.full((H, W), 1, np.int32)
    gt[:, 3:] = 2
    vol = np.zeros((H, W, D), np.float32)
    vol[..., 4] = -2.0
    pw = np.zeros((2, H, W), np.float32)
    loss, yh, gvol, gpw = oracle.hinge(vol, pw, gt, 1.0, 0.5, 1.5, 3, 4)
    assert (yh == 4).all()
    assert loss == pytest.approx(H * W * 2.0 + H * W - 0.0)
    assert (gvol[..., 4] == -1).all() and (gvol[..., 1][:, :3] == 1).all() and (gvol[..., 2][:, 3:] == 1).all()
    assert gvol.sum() == 0
    # the ground truth has a 1-label jump between columns 2 and 3 (rho 0.5); y_hat is flat
    assert (gpw[0][:, 2] == 0.5).all() and gpw[0][:, [0, 1, 3, 4, 5]].sum() == 0 and not gpw[1].any()
