"""GPU tests of the training step (cnncrf_train_*) against the oracle: the
forward equals the oracle's FP32 forward bit for bit; the adjoints equal the
FP64 oracle's gradient (itself pinned by central differences in
test_oracle_train.py) within FP32 accumulation error; the hinge finds the
oracle's loss-augmented labelling, loss and subgradient; SGD with momentum
follows v = mu v + g, theta -= lr v; the autograd form gives the fused step's
gradients; the full-size training step of 4 crops of 512 x 256, D = 128 runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# |g - g64| <= TOL * max|g64| per parameter slot: FP32 activations and sums against FP64
TOL = 2e-4


def setup(oracle, layers=3, topology=1, n=2, W=40, H=22, D=10, F=16, P=8, seed=3, mean_loss=False, precision=None,
          checkpoint_every=0, tc_wgrad=True, tc_dgrad=True):
    import torch
    from cnncrf import scenes
    from cnncrf import _lib as L
    from cnncrf.train import Trainer
    precision = L.FP32 if precision is None else precision
    cfg = oracle.make_cfg(num_layers=layers, topology=topology, in_channels=3, feat_channels=F, unary=1,
                          with_pairwise=1, pw_channels=P, precision=32, disp_min=0.0, disp_max=float(D - 1))
    params = oracle.xavier_params(cfg, seed=seed)
    sc = [scenes.voronoi_scene(W, H, D, seed=seed + 10 * i, cells=4, off_range=(1, D - 2), slope=0.05)
          for i in range(n)]
    t = Trainer(n, W, H, num_layers=layers, topology=topology, feat_channels=F, pw_channels=P, disp_max=float(D - 1),
                mean_loss=mean_loss, precision=precision, checkpoint_every=checkpoint_every, tc_wgrad=tc_wgrad,
                tc_dgrad=tc_dgrad)
    t.init_xavier(seed)
    left = torch.from_numpy(np.stack([s["left"] for s in sc])).cuda()
    right = torch.from_numpy(np.stack([s["right"] for s in sc])).cuda()
    p = oracle.padding(cfg)
    pads = [(oracle.pad_rgba(s["left"], p), oracle.pad_rgba(s["right"], p)) for s in sc]
    gt = np.stack([np.clip(np.rint(s["disp"]), 0, D - 1).astype(np.int32) for s in sc])
    lst = oracle.disparity_list(0.0, float(D - 1), 1.0)
    return cfg, params, t, left, right, pads, gt, lst


def close(g, g64, what):
    scale = max(np.abs(g64).max(), 1e-12)
    err = np.abs(g - g64).max() / scale
    assert err <= TOL, (what, err)


@pytest.mark.parametrize("layers,topology", [(3, 1), (3, 0)])
def test_forward_bitexact(cuda, oracle, layers, topology):
    cfg, params, t, left, right, pads, gt, lst = setup(oracle, layers, topology)
    for i, prm in enumerate(params):
        assert np.array_equal(t.get_param(i), prm), i  # the same seeded Xavier init
    vol, pw = t.forward(left, right)
    for i, (lp, rp) in enumerate(pads):
        ovol, opw = oracle.predict(cfg, params, lp, rp, lst)
        assert np.array_equal(vol[i].cpu().numpy(), ovol)
        assert np.array_equal(pw[i].cpu().numpy(), opw)


@pytest.mark.parametrize("layers,topology", [(3, 1), (3, 0)])
def test_backward_matches_fp64_oracle(cuda, oracle, layers, topology):
    torch = cuda
    cfg, params, t, left, right, pads, gt, lst = setup(oracle, layers, topology)
    vol, pw = t.forward(left, right)
    rng = np.random.default_rng(7)
    gvol = rng.standard_normal(tuple(vol.shape)).astype(np.float32)
    gpw = rng.standard_normal(tuple(pw.shape)).astype(np.float32)
    t.backward(torch.from_numpy(gvol).cuda(), torch.from_numpy(gpw).cuda())
    g64 = None
    cfg64 = oracle.make_cfg(**{k: getattr(cfg, k) for k, _ in cfg._fields_})
    cfg64.precision = 64
    for i, (lp, rp) in enumerate(pads):
        g = oracle.predict_backward(cfg64, params, lp, rp, lst, gvol[i], gpw[i])
        g64 = g if g64 is None else [a + b for a, b in zip(g64, g)]
    for i in range(len(params)):
        close(t.get_grad(i), g64[i], i)


def test_volume_only_gradient_leaves_the_pairwise_net_at_zero(cuda, oracle):
    torch = cuda
    cfg, params, t, left, right, pads, gt, lst = setup(oracle)
    vol, pw = t.forward(left, right)
    t.backward(torch.ones_like(vol), None)
    npw = 2 * cfg.num_layers
    assert all(not t.get_grad(i).any() for i in range(npw, len(params)))
    assert any(t.get_grad(i).any() for i in range(npw))


def test_hinge_matches_oracle(cuda, oracle):
    torch = cuda
    cfg, params, t, left, right, pads, gt, lst = setup(oracle)
    t.forward(left, right)
    losses, yh = t.hinge(torch.from_numpy(gt).cuda())
    gv, gp = t.hinge_grads()
    cfg64 = oracle.make_cfg(**{k: getattr(cfg, k) for k, _ in cfg._fields_})
    cfg64.precision = 64
    g64 = None
    for i, (lp, rp) in enumerate(pads):
        vol32, pw32 = oracle.predict(cfg, params, lp, rp, lst)
        loss, yho, gvo, gpo = oracle.hinge(vol32, pw32, gt[i], 1.0, 0.5, 1.5, 3, 8, shape=1)
        assert np.array_equal(yh[i].cpu().numpy(), yho), i
        assert losses[i] == pytest.approx(loss, rel=1e-12, abs=1e-9), i
        assert np.array_equal(gv[i].cpu().numpy(), gvo.astype(np.float32)), i
        assert np.array_equal(gp[i].cpu().numpy(), gpo.astype(np.float32)), i
        g = oracle.predict_backward(cfg64, params, lp, rp, lst, gvo, gpo)
        g64 = g if g64 is None else [a + b for a, b in zip(g64, g)]
    t.backward()  # from the hinge's own subgradient
    for i in range(len(params)):
        close(t.get_grad(i), g64[i], i)


def test_sgd_momentum_and_training_progress(cuda, oracle):
    torch = cuda
    cfg, params, t, left, right, pads, gt, lst = setup(oracle, n=1)
    g_t = torch.from_numpy(gt).cuda()
    th0 = [t.get_param(i) for i in range(len(params))]
    first = t.step(left, right, g_t, lr=0.01, momentum=0.9)
    g1 = [t.get_grad(i) for i in range(len(params))]
    th1 = [t.get_param(i) for i in range(len(params))]
    # the update is one fused multiply-add per element: allow an ulp of the larger operand
    for a, g, b in zip(th0, g1, th1):  # v = g after the first step
        np.testing.assert_allclose(b, a - np.float32(0.01) * g, rtol=1e-6, atol=2e-7)
    t.step(left, right, g_t, lr=0.01, momentum=0.9)
    g2 = [t.get_grad(i) for i in range(len(params))]
    th2 = [t.get_param(i) for i in range(len(params))]
    for a, ga, gb, b in zip(th1, g1, g2, th2):  # v = 0.9 g1 + g2
        np.testing.assert_allclose(b, a - np.float32(0.01) * (np.float32(0.9) * ga + gb), rtol=1e-5, atol=2e-7)
    hist = [first.sum()]
    for _ in range(25):
        hist.append(t.step(left, right, g_t, lr=0.01, momentum=0.9).sum())
    assert np.mean(hist[-3:]) < hist[0], hist


@pytest.mark.parametrize("prec", ["FP32", "BF16"])
def test_checkpoint_resume_is_exact(cuda, oracle, tmp_path, prec):
    """Two steps, a checkpoint, then a third step on the saved trainer and on a
    fresh one loaded from the file: the same loss and the same weights and
    momentum bit for bit.  The file is also a parameter file: the inference
    net loads its arr_i, and a trainer loading a plain parameter file (no
    mom_i) starts with zero momentum."""
    torch = cuda
    from cnncrf import _lib as L
    from cnncrf.api import StereoNet
    from cnncrf.train import Trainer
    P = getattr(L, prec)
    cfg, params, t, left, right, pads, gt, lst = setup(oracle, n=2, precision=P, P=16)
    g_t = torch.from_numpy(gt).cuda()
    for _ in range(2):
        t.step(left, right, g_t, lr=0.01, momentum=0.9)
    ck = tmp_path / "ck.npz"
    t.save(str(ck))
    u = Trainer(2, 40, 22, num_layers=3, topology=1, feat_channels=16, pw_channels=16, disp_max=9.0,
                mean_loss=False, precision=P, checkpoint_every=0)
    u.load(str(ck))
    la = t.step(left, right, g_t, lr=0.01, momentum=0.9)
    lb = u.step(left, right, g_t, lr=0.01, momentum=0.9)
    assert np.array_equal(la, lb)
    for i in range(t.num_params()):
        assert np.array_equal(t.get_param(i), u.get_param(i)), i
    t.save(str(tmp_path / "a.npz"))
    u.save(str(tmp_path / "b.npz"))
    with np.load(tmp_path / "a.npz") as za, np.load(tmp_path / "b.npz") as zb:
        assert sorted(za.files) == sorted(zb.files)
        for k in za.files:
            assert np.array_equal(za[k], zb[k]), k
        assert any(za["mom_%d" % i].any() for i in range(t.num_params()))
        plain = {"arr_%d" % i: za["arr_%d" % i] for i in range(t.num_params())}
    # the checkpoint as an inference parameter file
    net = StereoNet(3, 1, 3, 22 + 6, 40 + 6, feat_channels=16, pw_channels=16, topology=1,
                    unary=L.UNARY_ONE_MINUS_DOT, with_pairwise=True)
    net.set_all_params(str(ck))
    # a plain parameter file: the weights, zero momentum
    np.savez(tmp_path / "plain.npz", **plain)
    w = Trainer(2, 40, 22, num_layers=3, topology=1, feat_channels=16, pw_channels=16, disp_max=9.0,
                mean_loss=False, precision=P, checkpoint_every=0)
    w.load(str(tmp_path / "plain.npz"))
    w.save(str(tmp_path / "c.npz"))
    with np.load(tmp_path / "c.npz") as zc:
        for i in range(t.num_params()):
            assert np.array_equal(zc["arr_%d" % i], plain["arr_%d" % i]) and not zc["mom_%d" % i].any()
    bad = dict(plain)
    bad["arr_0"] = bad["arr_0"][:1]
    np.savez(tmp_path / "bad.npz", **bad)
    with pytest.raises(L.CnnCrfError) as e:
        w.load(str(tmp_path / "bad.npz"))
    assert e.value.status == L.ESHAPE


def test_autograd_equals_fused_step(cuda, oracle):
    torch = cuda
    from cnncrf.train import HingeLossFunction, StereoNetsFunction
    cfg, params, t, left, right, pads, gt, lst = setup(oracle)
    g_t = torch.from_numpy(gt).cuda()
    t.forward(left, right)
    fused_loss, _ = t.hinge(g_t)
    t.backward()
    fused = [t.get_grad(i) for i in range(len(params))]
    ps = [torch.from_numpy(np.ascontiguousarray(p, np.float32)).cuda().requires_grad_() for p in params]
    vol, pw = StereoNetsFunction.apply(t, left, right, *ps)
    loss = HingeLossFunction.apply(t, vol, pw, g_t)
    assert loss.item() == pytest.approx(fused_loss.sum(), rel=1e-12)  # mean_loss off: sums
    loss.backward()
    for i, p in enumerate(ps):
        assert np.array_equal(p.grad.cpu().numpy(), fused[i]), i
    # torch's SGD on the autograd gradients and the library's update agree
    opt = torch.optim.SGD(ps, lr=0.01, momentum=0.9)
    opt.step()
    t.sgd(0.01, 0.9)
    for i, p in enumerate(ps):
        np.testing.assert_allclose(p.detach().cpu().numpy(), t.get_param(i), rtol=1e-6, atol=2e-7)


def test_errors(cuda, oracle):
    torch = cuda
    from cnncrf import _lib as L
    from cnncrf.api import CnnCrfError
    cfg, params, t, left, right, pads, gt, lst = setup(oracle)
    with pytest.raises(CnnCrfError) as e:
        t.backward()
    assert e.value.status == L.ESTATE
    t.forward(left, right)
    bad = gt.copy()
    bad[0, 0, 0] = 10  # D = 10: labels 0..9
    with pytest.raises(CnnCrfError) as e:
        t.hinge(torch.from_numpy(bad).cuda())
    assert e.value.status == L.EINVAL
    with pytest.raises(CnnCrfError) as e:
        t.set_param(0, np.zeros(3, np.float32))
    assert e.value.status == L.ESHAPE


def test_full_size_training_step(cuda, oracle):
    """4 crops of 512 x 256 from the KITTI-shaped generator, D = 128, the
    7-layer 100-channel nets: two steps, finite losses and gradients, and the
    forward of the first equals the FP32 inference net's."""
    torch = cuda
    import time
    from cnncrf import scenes, _lib as L
    from cnncrf.api import StereoNet
    from cnncrf.train import Trainer
    n, W, H, D = 4, 512, 256, 128
    sc = [scenes.kitti_scene(W, H, D, seed=40 + i) for i in range(n)]
    left = torch.from_numpy(np.stack([s["left"] for s in sc])).cuda()
    right = torch.from_numpy(np.stack([s["right"] for s in sc])).cuda()
    gt = torch.from_numpy(np.stack([np.clip(np.rint(s["disp"]), 0, D - 1).astype(np.int32) for s in sc])).cuda()
    t = Trainer(n, W, H, precision=L.FP32, checkpoint_every=0)  # the exact mode: equals the inference net
    t.init_xavier(0)
    vol, pw = t.forward(left, right)
    net = StereoNet(7, n, 3, H + 14, W + 14, topology=L.TOPO_ALL3X3, unary=L.UNARY_ONE_MINUS_DOT,
                    with_pairwise=True)
    net.init_net(0.0, float(D - 1), 1.0)
    net.init_xavier(0)
    lp = np.stack([oracle.pad_rgba(s["left"], 7) for s in sc])
    rp = np.stack([oracle.pad_rgba(s["right"], 7) for s in sc])
    ivol = net.predict(torch.from_numpy(lp).cuda(), torch.from_numpy(rp).cuda())
    assert torch.equal(vol.reshape(ivol.shape), ivol)
    assert torch.equal(pw.reshape(net.pairwise_out.shape), net.pairwise_out)
    del net, ivol, t
    # the task's step: BF16 activations, checkpoints, mean loss, lr 1e-3, momentum 0.9
    t = Trainer(n, W, H)
    t.init_xavier(0)
    t.step(left, right, gt, lr=0.0, momentum=0.9)  # warm up, no update
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    l1 = t.step(left, right, gt, lr=1e-3, momentum=0.9)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    l2 = t.step(left, right, gt, lr=1e-3, momentum=0.9)
    assert np.isfinite(l1).all() and np.isfinite(l2).all() and (l1 > 0).all()
    assert (np.abs(l2 - l1) < 0.5 * l1).all()  # a sane step: the per-pixel loss moves, it does not explode
    for i in range(t.num_params()):
        g = t.get_grad(i)
        assert np.isfinite(g).all(), i
    assert any(t.get_grad(i).any() for i in range(t.num_params()))
    print("training step 4 x 512x256 D128: %.1f ms, losses %s -> %s" % (dt * 1e3, l1, l2))


def test_mean_loss_scaling(cuda, oracle):
    """mean_loss: every pair's loss per pixel, the subgradient and the
    gradients of their mean over the batch (sums / pixels)."""
    torch = cuda
    cfg, params, t, left, right, pads, gt, lst = setup(oracle, mean_loss=False)
    cfg2, params2, tm, left2, right2, _, _, _ = setup(oracle, mean_loss=True)
    g_t = torch.from_numpy(gt).cuda()
    t.forward(left, right)
    tm.forward(left, right)
    ls, _ = t.hinge(g_t)
    lm, _ = tm.hinge(g_t)
    npx = t.H * t.W
    np.testing.assert_allclose(lm, ls / npx, rtol=1e-12)
    t.backward()
    tm.backward()
    for i in range(len(params)):
        # the scale 1 / pixels is no power of two: the FP32 sums round differently
        ref = t.get_grad(i) / (t.n * npx)
        np.testing.assert_allclose(tm.get_grad(i), ref, rtol=2e-5, atol=2e-5 * np.abs(ref).max())


@pytest.mark.parametrize("prec,r", [("FP32", 2), ("FP32", 3), ("BF16", 2), ("BF16", 3)])
def test_checkpointing_changes_no_bit(cuda, oracle, prec, r):
    """Recomputing the layers between checkpoints during backward gives the
    keep-all step's losses and gradients exactly."""
    torch = cuda
    from cnncrf import _lib as L
    kw = dict(layers=5, F=100, P=64, precision=getattr(L, prec))
    _, params, t0, left, right, _, gt, _ = setup(oracle, checkpoint_every=0, **kw)
    _, _, tr, _, _, _, _, _ = setup(oracle, checkpoint_every=r, **kw)
    g_t = torch.from_numpy(gt).cuda()
    for t in (t0, tr):
        t.forward(left, right)
    l0, y0 = t0.hinge(g_t)
    lr_, yr = tr.hinge(g_t)
    assert np.array_equal(l0, lr_) and torch.equal(y0, yr)
    t0.backward()
    tr.backward()
    for i in range(len(params)):
        assert np.array_equal(t0.get_grad(i), tr.get_grad(i)), i


def test_bf16_mode_against_fp64_oracle(cuda, oracle):
    """The BF16 mode (tensor-core forward, BF16 activations, FP32 gradients):
    the volume and every slot's gradient against the FP64 oracle, errors
    relative to the largest value, stated per output."""
    torch = cuda
    from cnncrf import _lib as L
    cfg, params, t, left, right, pads, gt, lst = setup(oracle, layers=3, F=100, P=64, precision=L.BF16,
                                                       checkpoint_every=2)
    cfg64 = oracle.make_cfg(**{k: getattr(cfg, k) for k, _ in cfg._fields_})
    cfg64.precision = 64
    vol, pw = t.forward(left, right)
    rng = np.random.default_rng(11)
    gvol = rng.standard_normal(tuple(vol.shape)).astype(np.float32)
    gpw = rng.standard_normal(tuple(pw.shape)).astype(np.float32)
    t.backward(torch.from_numpy(gvol).cuda(), torch.from_numpy(gpw).cuda())
    errs = {}
    g64 = None
    for i, (lp, rp) in enumerate(pads):
        v64, p64 = oracle.predict(cfg64, params, lp, rp, lst)
        errs.setdefault("volume", []).append(np.abs(vol[i].cpu().numpy() - v64).max())
        errs.setdefault("pairwise", []).append(np.abs(pw[i].cpu().numpy() - p64).max() / np.abs(p64).max())
        g = oracle.predict_backward(cfg64, params, lp, rp, lst, gvol[i], gpw[i])
        g64 = g if g64 is None else [a + b for a, b in zip(g64, g)]
    for i in range(len(params)):
        errs["grad%d" % i] = [np.abs(t.get_grad(i) - g64[i]).max() / max(np.abs(g64[i]).max(), 1e-12)]
    print("BF16 mode vs FP64:", {k: float("%.2e" % max(v)) for k, v in errs.items()})
    assert max(errs["volume"]) < 2e-2  # 1 - <fL, fR> on BF16 features (measured 3e-3)
    assert max(errs["pairwise"]) < 5e-2  # measured 4e-3
    npf = 2 * cfg.num_layers
    for i in range(npf):  # feature net (measured 5e-3 .. 7e-3)
        assert errs["grad%d" % i][0] < 2e-2, (i, errs["grad%d" % i])
    # pairwise net (measured up to 8.5e-2): d|h|/dh = sign(h), and where h is
    # near 0 BF16 and FP64 can fall on opposite sides of the kink; a few such
    # pixels out of ~1800 give errors of this size
    for i in range(npf, len(params)):
        assert errs["grad%d" % i][0] < 0.15, (i, errs["grad%d" % i])



@pytest.mark.parametrize("layers,topology,n,W,H", [(3, 1, 2, 40, 22), (4, 1, 1, 150, 37), (3, 0, 3, 97, 19)])
def test_tensor_core_weight_gradient_matches_cuda_cores(cuda, oracle, layers, topology, n, W, H):
    """The BF16 mode's weight gradients of the tanh layers on the tensor
    cores (dz rounded to BF16, FP32 accumulation; the first layers read a
    BF16 copy of the normalised image) against the CUDA-core path (FP32 dz
    and input) of the same forward and output gradients.  Every other slot
    (biases, the pairwise head) comes from the same kernels and must match
    bit for bit; the tensor-core slots within 1e-2 of their largest value
    (BF16 operands: a relative rounding of 2^-9 per term).  Widths 40, 150
    and 97 leave ragged 64-pixel chunks; topology 0 has 2 x 2 kernels."""
    torch = cuda
    from cnncrf import _lib as L
    kw = dict(layers=layers, topology=topology, n=n, W=W, H=H, F=100, P=64, precision=L.BF16, checkpoint_every=2,
              tc_dgrad=False)
    _, params, t_tc, left, right, _, _, _ = setup(oracle, tc_wgrad=True, **kw)
    t_cc = setup(oracle, tc_wgrad=False, **kw)[2]
    vol, pw = t_tc.forward(left, right)
    vol2, pw2 = t_cc.forward(left, right)
    assert torch.equal(vol, vol2) and torch.equal(pw, pw2)
    rng = np.random.default_rng(5)
    gvol = torch.from_numpy(rng.standard_normal(tuple(vol.shape)).astype(np.float32)).cuda()
    gpw = torch.from_numpy(rng.standard_normal(tuple(pw.shape)).astype(np.float32)).cuda()
    t_tc.backward(gvol, gpw)
    t_cc.backward(gvol, gpw)
    tc_slots = {2 * l for l in range(layers)} | {2 * layers, 2 * layers + 2}
    errs = {}
    for i in range(len(params)):
        a, b = t_tc.get_grad(i), t_cc.get_grad(i)
        if i in tc_slots:
            errs[i] = np.abs(a - b).max() / max(np.abs(b).max(), 1e-12)
        else:
            assert np.array_equal(a, b), i
    print("tensor-core vs CUDA-core weight gradients:", {k: float("%.2e" % v) for k, v in errs.items()})
    assert max(errs.values()) < 1e-2, errs


@pytest.mark.parametrize("layers,topology,n,W,H", [(3, 1, 2, 40, 22), (4, 1, 1, 300, 37), (3, 0, 3, 97, 19)])
def test_tensor_core_input_gradient_matches_cuda_cores(cuda, oracle, layers, topology, n, W, H):
    """The BF16 mode's input gradients on the tensor cores (the padded output
    gradient rounded to BF16, the unflipped transposed kernel in BF16, FP32
    sums; the correlation adjoint with the volume gradient in BF16) against
    the CUDA-core path, weight gradients on the CUDA cores in both.  The
    pairwise net's second layer and head, above its first tensor-core input
    gradient, match bit for bit; every other slot within 2e-2 of its largest
    value (two BF16 roundings per layer, compounded over the layers below).
    Width 300 gives two 256-pixel tiles per row, the last one ragged."""
    torch = cuda
    from cnncrf import _lib as L
    kw = dict(layers=layers, topology=topology, n=n, W=W, H=H, F=100, P=64, precision=L.BF16, checkpoint_every=2,
              tc_wgrad=False)
    _, params, t_tc, left, right, _, _, _ = setup(oracle, tc_dgrad=True, **kw)
    t_cc = setup(oracle, tc_dgrad=False, **kw)[2]
    vol, pw = t_tc.forward(left, right)
    vol2, pw2 = t_cc.forward(left, right)
    assert torch.equal(vol, vol2) and torch.equal(pw, pw2)
    rng = np.random.default_rng(6)
    gvol = torch.from_numpy(rng.standard_normal(tuple(vol.shape)).astype(np.float32)).cuda()
    gpw = torch.from_numpy(rng.standard_normal(tuple(pw.shape)).astype(np.float32)).cuda()
    t_tc.backward(gvol, gpw)
    t_cc.backward(gvol, gpw)
    base = 2 * layers
    same = {base + 2, base + 3, base + 4}
    errs = {}
    for i in range(len(params)):
        a, b = t_tc.get_grad(i), t_cc.get_grad(i)
        if i in same:
            assert np.array_equal(a, b), i
        else:
            errs[i] = np.abs(a - b).max() / max(np.abs(b).max(), 1e-12)
    print("tensor-core vs CUDA-core input gradients:", {k: float("%.2e" % v) for k, v in errs.items()})
    assert max(errs.values()) < 2e-2, errs


@pytest.mark.parametrize("dmin,dstep,dmax,W", [(0.0, 1.0, 40.0, 150), (2.0, 3.0, 47.0, 97), (0.0, 1.0, 127.0, 300)])
def test_tensor_core_correlation_adjoint(cuda, oracle, dmin, dstep, dmax, W):
    """The correlation adjoint on the tensor cores (banded volume gradient in
    BF16 built in shared memory, BF16 features, FP32 sums; the right side
    through the gathered right-view gradient) against the FP32 CUDA-core
    adjoint, on a volume-only output gradient.  With two layers the top
    layer's weight and bias gradients see the correlation adjoint through the
    L2 normalisation alone: within 1e-2 of their largest value.  Lists: a
    contiguous one, one with step 3 (offsets with gaps) and the full 128."""
    torch = cuda
    from cnncrf import _lib as L
    from cnncrf.train import Trainer
    n, H = 2, 9
    ts = [Trainer(n, W, H, num_layers=2, feat_channels=100, pw_channels=64, disp_min=dmin, disp_step=dstep,
                  disp_max=dmax, precision=L.BF16, checkpoint_every=0, tc_wgrad=False, tc_dgrad=tc)
          for tc in (True, False)]
    for t in ts:
        t.init_xavier(4)
    rng = np.random.default_rng(8)
    left = torch.from_numpy(rng.random((n, H, W, 4)).astype(np.float32)).cuda()
    right = torch.from_numpy(rng.random((n, H, W, 4)).astype(np.float32)).cuda()
    vols = [t.forward(left, right)[0] for t in ts]
    assert torch.equal(vols[0], vols[1])
    gvol = torch.from_numpy(rng.standard_normal(tuple(vols[0].shape)).astype(np.float32)).cuda()
    for t in ts:
        t.backward(gvol, torch.zeros((n, 2, H, W), device="cuda"))
    errs = {}
    for i in (2, 3):
        a, b = ts[0].get_grad(i), ts[1].get_grad(i)
        errs[i] = np.abs(a - b).max() / max(np.abs(b).max(), 1e-12)
    print("tensor-core vs CUDA-core correlation adjoint:", {k: float("%.2e" % v) for k, v in errs.items()})
    assert max(errs.values()) < 1e-2, errs


def test_autotune_changes_no_bit(cuda, oracle):
    """cnncrf_train_autotune enters the hinge problem's CRF tile in the
    process-wide table; a step after it gives the same losses, labelling and
    gradients as a step of an identical trainer before it."""
    torch = cuda
    from cnncrf import _lib as L
    from cnncrf import tuning
    tuning.clear()
    kw = dict(n=2, W=150, H=37, D=24, F=16, P=16, precision=L.BF16, checkpoint_every=2)
    _, params, t0, left, right, _, gt, _ = setup(oracle, **kw)
    t1 = setup(oracle, **kw)[2]
    gt = torch.from_numpy(gt).cuda()
    t0.forward(left, right)
    l0, y0 = t0.hinge(gt)
    t0.backward()
    assert tuning.count() == 0
    t1.forward(left, right)
    t1.autotune()
    assert tuning.count() == 1
    t1.forward(left, right)
    l1, y1 = t1.hinge(gt)
    t1.backward()
    assert np.array_equal(l0, l1) and torch.equal(y0, y1)
    for i in range(len(params)):
        assert np.array_equal(t0.get_grad(i), t1.get_grad(i)), i
    tuning.clear()
