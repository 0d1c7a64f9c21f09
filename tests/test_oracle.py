"""CPU tests of the oracle: its math kernels, its pin against the golden
fixtures (an independent float64 restatement of the reference operators on
the reference's own sample images and shipped weights), and the solver
properties the CRF spec guarantees."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def load_golden():
    z = np.load(os.path.join(GOLDEN, "kitti7_full_params.npz"))
    params = [z["arr_%d" % i] for i in range(19)]
    left = np.load(os.path.join(GOLDEN, "crop_left_rgba.npy"))
    right = np.load(os.path.join(GOLDEN, "crop_right_rgba.npy"))
    return params, left, right


def test_tanh_exp_accuracy(oracle):
    """Own exp/tanh (cnncrf_fmath.h) stay within 3 ulp of float64 references."""
    x = np.linspace(-12, 12, 400001).astype(np.float32)
    w = np.ones((1, 1, 1, 1), np.float32)
    t = oracle.conv(x.reshape(1, -1, 1), w, None, act=1)[0, :, 0].astype(np.float64)
    ref = np.tanh(x.astype(np.float64))
    ulp = np.abs(t - ref) / np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    assert ulp.max() <= 3.0
    # exp through the softmax of two values: -softmax([0, x])[1] = -e^x / (1 + e^x)
    xs = np.linspace(-80, 0, 20001).astype(np.float32)
    vol = np.stack([np.zeros_like(xs), xs], -1).reshape(-1, 1, 2)
    u = oracle.unary(vol, 0).reshape(-1, 2)
    e = np.exp(xs.astype(np.float64))
    ref = -e / (1 + e)
    ok = np.abs(ref) > 1e-30
    rel = np.abs(u[ok, 1] - ref[ok]) / np.abs(ref[ok])
    assert rel.max() < 4e-7


def test_padding_is_symmetric(oracle):
    rng = np.random.default_rng(1)
    img = rng.random((5, 7, 4)).astype(np.float32)
    for p in (1, 2, 4, 7):
        out = oracle.pad_rgba(img, p)
        ref = np.pad(img, ((p, p), (p, p), (0, 0)), mode="symmetric")
        np.testing.assert_array_equal(out, ref)


def test_conv_is_true_convolution(oracle):
    import torch
    rng = np.random.default_rng(2)
    x = rng.standard_normal((11, 13, 5)).astype(np.float32)
    w = rng.standard_normal((7, 5, 3, 2)).astype(np.float32)
    b = rng.standard_normal(7).astype(np.float32)
    o = oracle.conv(x, w, b, act=0, precision=64)
    t = torch.nn.functional.conv2d(torch.tensor(x, dtype=torch.float64).permute(2, 0, 1)[None],
                                   torch.tensor(w, dtype=torch.float64).flip(2, 3),
                                   torch.tensor(b, dtype=torch.float64))[0].permute(1, 2, 0).numpy()
    np.testing.assert_allclose(o, t, atol=1e-12)


@pytest.mark.parametrize("precision,tol", [(64, 1e-9), (32, 2e-4)])
def test_oracle_predict_matches_golden(oracle, precision, tol):
    """Shipped weights + sample images: oracle volume and pairwise weights vs
    the independent float64 golden (tests/golden/make_golden.py)."""
    params, left, right = load_golden()
    cfg = oracle.make_cfg(precision=precision, disp_max=15.0)
    p = oracle.padding(cfg)
    lp, rp = oracle.pad_rgba(left, p), oracle.pad_rgba(right, p)
    lst = oracle.disparity_list(0.0, 15.0, 1.0)
    vol, pw = oracle.predict(cfg, params, lp, rp, lst)
    g_unary = np.load(os.path.join(GOLDEN, "golden_unary_f64.npy"))
    g_pw = np.load(os.path.join(GOLDEN, "golden_pairwise_f64.npy"))
    assert vol.shape == g_unary.shape
    np.testing.assert_allclose(vol, g_unary, atol=tol, rtol=tol)
    np.testing.assert_allclose(pw, g_pw, atol=tol, rtol=tol)


def test_oracle_raw_correlation_matches_golden(oracle):
    params, left, right = load_golden()
    cfg = oracle.make_cfg(precision=64)
    p = oracle.padding(cfg)
    nl = oracle.normalize(oracle.pad_rgba(left, p), 3, 64)
    nr = oracle.normalize(oracle.pad_rgba(right, p), 3, 64)
    for l in range(7):
        w, b = params[2 * l], params[2 * l + 1]
        nl = oracle.conv(nl, w, b, 1, 64)
        nr = oracle.conv(nr, w, b, 1, 64)
    corr = oracle.correlation(nl, nr, oracle.disparity_list(0.0, 15.0, 1.0), precision=64)
    g = np.load(os.path.join(GOLDEN, "golden_corr_f64.npy"))
    np.testing.assert_allclose(corr, g, atol=1e-9, rtol=1e-9)


def test_disparity_list_and_dispatch(oracle):
    np.testing.assert_array_equal(oracle.disparity_list(0, 3, 1), -np.arange(4, dtype=np.float32))
    # the 3-label refinement list for step 1 is judged "integer" (element 1 is -0)
    lst = oracle.disparity_list(-0.25, 0.25, 0.25)
    assert len(lst) == 3 and not oracle.disp_is_float(lst)
    assert oracle.disp_is_float(oracle.disparity_list(-1.0, 1.0, 0.5))


def test_refinement_integer_truncation(oracle):
    """With step 1 the reference truncates (int)(+-0.25) to 0: all three labels
    of the refinement volume equal the centre one except where w - 0.25 < 0."""
    rng = np.random.default_rng(3)
    f = rng.standard_normal((4, 9, 6)).astype(np.float32)
    g = rng.standard_normal((4, 9, 6)).astype(np.float32)
    c = oracle.correlation(f, g, oracle.disparity_list(-0.25, 0.25, 0.25))
    np.testing.assert_array_equal(c[:, :, 0], c[:, :, 1])
    np.testing.assert_array_equal(c[:, 1:, 2], c[:, 1:, 1])
    assert np.all(c[:, 0, 2] == 0)


def test_chain_equals_bruteforce(oracle):
    """Single-row images: the first H pass's chain minimum is the exact MAP."""
    rng = np.random.default_rng(4)
    for trial in range(40):
        n, D = int(rng.integers(2, 7)), int(rng.integers(1, 5))
        cost = (rng.random((1, n, D)) * 3).astype(np.float32)
        wx = (rng.random((1, n)) * 2).astype(np.float32)
        wy = np.zeros((1, n), np.float32)
        shape, delta = int(rng.integers(0, 2)), int(rng.integers(1, 4))
        lab, lb, lbi, _ = oracle.crf(cost, wx, wy, 0.7, 2.5, delta, 2, shape=shape)
        e_bf, _ = oracle.chain_bruteforce(cost[0], wx[0], 0.7, 2.5, delta, shape)
        assert abs(lbi[0] - e_bf) <= 1e-5 * max(1.0, abs(e_bf))
        assert lb <= e_bf + 1e-5


def test_crf_exact_on_single_chains(oracle):
    """The decomposition is exact on a tree: on an image that is one row or
    one column the dual bound reaches the minimum energy and the labels are
    the exact minimiser.  A row is one horizontal chain, optimal from the
    first pass; a column is one vertical chain whose unary the horizontal
    single-node subproblems hand over a slack fraction at a time, so its bound
    converges geometrically (30 iterations)."""
    rng = np.random.default_rng(41)
    for trial in range(30):
        n, D = int(rng.integers(2, 7)), int(rng.integers(2, 5))
        shape, delta = int(rng.integers(0, 2)), int(rng.integers(1, 4))
        c = (rng.random((n, D)) * 3).astype(np.float32)
        w = (rng.random(n) * 2).astype(np.float32)
        e_bf, lab_bf = oracle.chain_bruteforce(c, w, 0.7, 2.5, delta, shape)
        for orient in ("row", "column"):
            if orient == "row":
                cost, wx, wy = c[None], w[None], np.zeros((1, n), np.float32)
            else:
                cost, wx, wy = c[:, None, :], np.zeros((n, 1), np.float32), w[:, None]
            lab, lb, lbi, _ = oracle.crf(cost, wx, wy, 0.7, 2.5, delta, 30, shape=shape)
            assert abs(lb - e_bf) <= 1e-4 * max(1.0, abs(e_bf)), (trial, orient, lb, e_bf)
            assert np.array_equal(lab.reshape(-1), lab_bf), (trial, orient)


def test_crf_bound_monotone_and_below_energy(oracle):
    rng = np.random.default_rng(5)
    for shape in (0, 1):
        cost = rng.random((10, 13, 7)).astype(np.float32)
        wx = rng.random((10, 13)).astype(np.float32)
        wy = rng.random((10, 13)).astype(np.float32)
        lab, lb, lbi, _ = oracle.crf(cost, wx, wy, 0.4, 1.2, 2, 8, shape=shape)
        e = oracle.energy(cost, wx, wy, lab, 0.4, 1.2, 2, shape)
        assert np.all(np.diff(lbi) >= -1e-6 * np.abs(lbi[1:]))
        assert lb <= e + 1e-6 * abs(e)
        assert lab.min() >= 0 and lab.max() < 7


def _local_polytope_lp(cost, wx, wy, L1, L2, delta, shape):
    """The LP relaxation of the grid energy over the local polytope: node
    marginals mu_i(x) and edge marginals mu_ij(x, y), each node's summing to
    one and each edge's summing to its two nodes' marginals.  Its optimum is
    what the dual of a decomposition into chains that cover every edge can at
    best reach, so the solver's bound can never exceed it (weak duality)."""
    from scipy.optimize import linprog
    from scipy.sparse import coo_matrix
    H, W, D = cost.shape
    f32 = np.float32
    rho = np.zeros((D, D))
    for a in range(D):
        for b in range(D):
            t = abs(a - b)
            if t == 0:
                continue
            if t <= delta:
                rho[a, b] = min(f32(L1), f32(L2)) if shape == 0 else min(f32(L1) * f32(t), f32(L2))
            else:
                rho[a, b] = f32(L2)
    edges = [(y * W + x, y * W + x + 1, wx[y, x]) for y in range(H) for x in range(W - 1)]
    edges += [(y * W + x, (y + 1) * W + x, wy[y, x]) for y in range(H - 1) for x in range(W)]
    nn = H * W * D
    obj = [cost.reshape(-1).astype(np.float64)]
    for (_, _, w) in edges:
        obj.append((f32(w) * rho.astype(f32)).astype(np.float64).reshape(-1))
    obj = np.concatenate(obj)
    rows, cols, vals, rhs = [], [], [], []
    r = 0
    for i in range(H * W):  # sum_x mu_i(x) = 1
        rows += [r] * D
        cols += list(range(i * D, i * D + D))
        vals += [1.0] * D
        rhs.append(1.0)
        r += 1
    for e, (i, j, _) in enumerate(edges):
        base = nn + e * D * D
        for a in range(D):  # sum_b mu_ij(a, b) = mu_i(a)
            rows += [r] * (D + 1)
            cols += [base + a * D + b for b in range(D)] + [i * D + a]
            vals += [1.0] * D + [-1.0]
            rhs.append(0.0)
            r += 1
        for b in range(D):  # sum_a mu_ij(a, b) = mu_j(b)
            rows += [r] * (D + 1)
            cols += [base + a * D + b for a in range(D)] + [j * D + b]
            vals += [1.0] * D + [-1.0]
            rhs.append(0.0)
            r += 1
    A = coo_matrix((vals, (rows, cols)), shape=(r, obj.size)).tocsr()
    res = linprog(obj, A_eq=A, b_eq=np.array(rhs), bounds=(0, None), method="highs")
    assert res.status == 0, res.message
    return res.fun


def test_crf_bound_reaches_the_lp_relaxation(oracle):
    """The chain decomposition's dual is the dual of the local-polytope LP
    relaxation, so its bound can never exceed the LP optimum (weak duality),
    at any iteration, and the LP never exceeds the minimum energy.  The solver
    is a block-coordinate ascent of that dual, and on these grids it reaches
    the optimum: after 200 iterations the bound equals the LP optimum that
    scipy's HiGHS computes from the energy alone (measured: within 1e-4 by
    iteration 38 on 150 random grids up to 4 x 4 with up to 5 labels).  With
    two labels and the STEP term (w >= 0: an attractive, submodular energy)
    the relaxation is tight, which checks the LP's construction against
    brute force."""
    pytest.importorskip("scipy")
    import itertools
    rng = np.random.default_rng(17)
    for trial in range(24):
        H, W = int(rng.integers(2, 4)), int(rng.integers(2, 4))
        D = 2 if trial < 8 else int(rng.integers(2, 5))
        shape = 0 if trial < 8 else int(rng.integers(0, 2))
        delta = int(rng.integers(1, 4))
        cost = (rng.random((H, W, D)) * 3).astype(np.float32)
        wx = (rng.random((H, W)) * 2).astype(np.float32)
        wy = (rng.random((H, W)) * 2).astype(np.float32)
        L1, L2 = 0.6, 1.7
        lp = _local_polytope_lp(cost, wx, wy, L1, L2, delta, shape)
        tol = 1e-5 * max(1.0, abs(lp))
        lab, lb, lbi, _ = oracle.crf(cost, wx, wy, L1, L2, delta, 200, shape=shape)
        assert np.all(lbi <= lp + tol), (trial, lbi.max(), lp)
        assert abs(lb - lp) <= tol, (trial, lb, lp)
        assert oracle.energy(cost, wx, wy, lab, L1, L2, delta, shape) >= lp - tol
        if D ** (H * W) > 20000:
            continue
        emin = min(oracle.energy(cost, wx, wy, np.array(x, np.int32).reshape(H, W), L1, L2, delta, shape)
                   for x in itertools.product(range(D), repeat=H * W))
        assert lp <= emin + tol
        if D == 2 and shape == 0:
            assert abs(lp - emin) <= tol, (trial, lp, emin)


def test_crf_zero_weights_is_wta(oracle):
    rng = np.random.default_rng(6)
    cost = rng.random((6, 9, 5)).astype(np.float32)
    z = np.zeros((6, 9), np.float32)
    lab, lb, _, _ = oracle.crf(cost, z, z, 1.0, 3.0, 2, 3)
    np.testing.assert_array_equal(lab, np.argmin(cost, axis=2))
    np.testing.assert_allclose(lb, cost.min(axis=2).astype(np.float64).sum(), rtol=1e-6)


def test_concat_net_matches_numpy(oracle):
    """The oracle's ConcatStereoNet against an independent FP64 numpy
    restatement: each layer a true (flipped-kernel) 3x3 convolution of the
    zero-padded previous output plus bias, tanh; the features all layers'
    outputs in order; the correlation and unary of the oracle's own, pinned
    elsewhere, applied to them; the pairwise weights |tanh| of a 3x3
    convolution of the zero-padded raw left features (no bias)."""
    from cnncrf import scenes
    W, H, D, layers = 23, 17, 7, 5
    g = 20
    s = scenes.voronoi_scene(W, H, D, seed=2, cells=3, off_range=(1, D - 2))
    for unary in (0, 1):
        cfg = oracle.make_cfg(num_layers=layers, topology=2, in_channels=3, unary=unary, disp_max=float(D - 1),
                              with_pairwise=1, precision=64)
        params = oracle.xavier_params(cfg, seed=5)
        lst = oracle.disparity_list(0.0, float(D - 1), 1.0)
        vol, pw = oracle.predict(cfg, params, s["left"], s["right"], lst)

        def conv_same(x, w, b):
            xp = np.pad(x, ((1, 1), (1, 1), (0, 0)))
            win = np.lib.stride_tricks.sliding_window_view(xp, (3, 3), axis=(0, 1))  # H, W, Cin, 3, 3
            y = np.einsum("hwcij,ocij->hwo", win, w[:, :, ::-1, ::-1].astype(np.float64))
            return y if b is None else y + b.astype(np.float64)

        feats = []
        for img in (s["left"], s["right"]):
            x = oracle.normalize(img, 3, precision=64)
            outs = []
            for l in range(layers):
                x = np.tanh(conv_same(x, params[2 * l], params[2 * l + 1]))
                outs.append(x)
            feats.append(np.concatenate(outs, axis=2))
        assert feats[0].shape == (H, W, g * layers)
        opw = np.abs(np.tanh(conv_same(feats[0], params[2 * layers], None))).transpose(2, 0, 1)
        np.testing.assert_allclose(pw, opw, rtol=1e-9, atol=1e-12)
        f = [oracle.l2norm(x, precision=64) if unary == 1 else x for x in feats]
        ref = oracle.unary(oracle.correlation(f[0], f[1], lst, precision=64), unary, precision=64)
        np.testing.assert_allclose(vol, ref, rtol=1e-9, atol=1e-12)


def test_crf_ties_take_first_minimum(oracle):
    cost = np.zeros((3, 4, 6), np.float32)
    z = np.zeros((3, 4), np.float32)
    lab, _, _, _ = oracle.crf(cost, z, z, 1.0, 3.0, 2, 2)
    assert np.all(lab == 0)


def test_remap_and_argmin(oracle):
    lab = np.array([[0, 3], [7, 1]], np.int32)
    np.testing.assert_array_equal(oracle.remap(lab, 2.0, 0.5), lab * 0.5 + 2.0)
    vol = np.array([[[3, 1, 1, 2]]], np.float32)
    assert oracle.argmin(vol, 1.0, 1.0)[0, 0] == 2.0


def test_tv_box_constraint(oracle):
    rng = np.random.default_rng(7)
    H, W = 9, 11
    u0 = rng.integers(0, 20, (H, W)).astype(np.float32)
    qf = np.stack([rng.standard_normal((H, W)), rng.random((H, W))], -1).astype(np.float32)
    w = rng.random((H, W)).astype(np.float32)
    u, _, p, q = oracle.tv_iterate(u0, u0, qf, w, w, 5.0, 0.1, 1.0, 20)
    assert np.all(u >= u0 - 0.5) and np.all(u <= u0 + 0.5)
    assert np.all(np.abs(p[..., 0]) <= w) and np.all(np.abs(q[..., 1]) <= w)


def test_run_pair_small_scene(oracle):
    """End to end on a tiny synthetic scene: the CRF improves on WTA."""
    from cnncrf import scenes
    s = scenes.voronoi_scene(48, 32, 16, seed=1, cells=4, off_range=(2, 12), slope=0.05)
    cfg = oracle.make_cfg(num_layers=3, disp_max=15.0, crf_iters=4, L1=0.5, L2=1.5, delta=3,
                          crf_shape=1, topology=1, unary=1, feat_channels=16, pw_channels=8)
    params = oracle.xavier_params(cfg, seed=0)
    r = oracle.run_pair(cfg, params, s["left"], s["right"])
    assert r["disp"].shape == (32, 48)
    e = oracle.energy(r["vol"], r["wx"], r["wy"], r["labels"], 0.5, 1.5, 3, 1)
    wta = np.argmin(r["vol"], axis=2).astype(np.int32)
    e_wta = oracle.energy(r["vol"], r["wx"], r["wy"], wta, 0.5, 1.5, 3, 1)
    assert r["lb"] <= e + 1e-5 * abs(e)
    assert e <= e_wta + 1e-6
