"""Benchmark of the CNN-CRF stereo hot path (one JSON line on rank 0).

Workload (the reference's metric "stereo pairs/s at 1242x375 D=128"):
KITTI-shaped RGB pairs, 1242x375, D = 128 (disparities 0..127), the 7-layer
all-3x3 100-channel feature CNN with L2-normalised features and the
1 - <fL,fR> unary, the 2-layer 3x3 (+1x1) pairwise CNN, a 4-connected CRF
with truncated-linear pairwise (L1 = 0.5, truncation 3) solved with 8
iterations, Xavier weights from seed 0, seeded synthetic scenes (ground plane
+ 15 boxes; the KITTI images are not available).  A step is one batched run
of --batch pairs (default 8) through the BF16 path.

  value   pairs/s with the input pairs already in HBM (device-to-device
          staging + CNN + correlation + CRF + remap per step), CUDA events on
          the library's stream, L2 flushed (256 MiB write) between steps
  e2e     same through the public API from pinned HOST buffers: H2D of the
          RGBA images, the whole path, D2H of the disparity maps per step
  --impl reference   the CPU restatement of the reference path (OpenMP, all
          host threads) on the same workload, one pair per step.

The default line also carries the other configurations of the benchmark spec, each with
its own value, e2e, roofline and clocks (skip them with --no-extras):
  mbq_tv   720x480, D = 96, the plain FP32 path (bit-exact against the oracle)
           with 4 TV/Huber iterations (eps 0.01, lambda 1) after the CRF, and
           the oracle's time for the same pair on the host cores beside it
  train    the training step of 4 crops of 512x256, D = 128 (BF16 with
           per-layer recomputation, structured hinge, SGD with momentum)
  uneven   the uneven batch of 32 pairs in four sizes and disparity ranges,
           replayed as one CUDA graph

Multi-GPU: pairs are independent, so N ranks run N replicas (no
collective on the data path); value = pairs of all ranks / max rank time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cnn-crf-stereo_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "stereo pairs/s at 1242x375 D=128, BF16 vs FP32 GPU (<=0.5% disparity change)"

WORKLOAD = dict(name="kitti1242x375_d128", W=1242, H=375, D=128, layers=7, topology="all3x3",
                feat=100, pw=64, unary="one_minus_dot", L1=0.5, L2=1.5, delta=3, shape="linear",
                crf_iters=8, lam=1.0, seed=0)


def workload_config(wl):
    """The workload as both arms describe it (the same dict in the line of
    the GPU arm and of --impl reference); how a step runs goes under "run"."""
    return {"workload": wl["name"], "W": wl["W"], "H": wl["H"], "D": wl["D"], "crf_iters": wl["crf_iters"],
            "net": "7x3x3 conv 100ch + L2 norm, 1-dot unary, pairwise CNN 3x3-3x3-1x1",
            "crf": "truncated linear L1=0.5 T=3"}


def conv_flops(W, H, layers=7, feat=100, ic=3, pw=64, k=3):
    """Algorithmic FLOPs of the convolutions of one pair, 2 x output pixels x
    Cout x (kh kw Cin) per layer, both sides.  Returns (tensor-core layers:
    feature layers 2..L and the pairwise 64->64 conv; SIMT layers: feature
    layer 1, pairwise 3->64 conv and the 1x1 head)."""
    p = layers  # all-3x3: padding = number of layers
    h, w = H + 2 * p, W + 2 * p
    tc = simt = 0
    cin = ic
    for l in range(layers):
        h, w = h - (k - 1), w - (k - 1)
        f = 2 * 2 * h * w * feat * k * k * cin
        if l == 0:
            simt += f
        else:
            tc += f
        cin = feat
    simt += 2 * (H + 2) * (W + 2) * pw * 9 * 3 + 2 * H * W * 2 * pw
    tc += 2 * H * W * pw * 9 * pw
    return tc, simt


def conv_forms_summary():
    """The tuned launch forms of the tensor-core convolutions (after autotune):
    per layer shape, 2-CTA pairs or single CTAs, the stages and the best launch time."""
    from cnncrf import tuning
    return [{"layer": "%d img %dx%d %d->%d k%dx%d mode %d" % (f["n_img"], f["Win"], f["Hin"], f["cin"], f["cout"],
                                                            f["kh"], f["kw"], f["mode"]),
             "pair": f["pair"], "stages": f["stages"], "ms": round(f["ms"], 4)} for f in tuning.conv_forms()]


def crf_bytes_per_pass(W, H, D):
    """Algorithmic bytes of one chain pass as counted for the roofline: three
    N*D float arrays (the subproblem's unary inputs read once, phi written)."""
    return 3 * W * H * D * 4


class ClockSampler:
    def __init__(self, index):
        self.index, self.samples, self.proc = index, [], None

    def start(self):
        cmd = ["nvidia-smi", "-i", str(self.index),
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "100"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def dist_setup():
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return rank, world, local


def replica_value(steps, pairs_per_step, world, t_ms):
    """Whole-job pairs/s: every rank runs `steps` steps of its own pairs; the
    time is the slowest rank's (max over ranks)."""
    return steps * pairs_per_step * world / (t_ms / 1000.0)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def oracle_cfg(O, wl, threads=0):
    return O.make_cfg(num_layers=wl["layers"], topology=1, unary=1, feat_channels=wl["feat"],
                      pw_channels=wl["pw"], disp_max=float(wl["D"] - 1), lam=wl["lam"], L1=wl["L1"],
                      L2=wl["L2"], delta=float(wl["delta"]), crf_iters=wl["crf_iters"], crf_shape=1,
                      threads=threads)


def cpu_pairs_per_s(wl, scene, pairs=1):
    """Time the CPU oracle (all host threads) on `pairs` full pairs."""
    from oracle import oracle as O
    cfg = oracle_cfg(O, wl)
    params = O.xavier_params(cfg, seed=wl["seed"])
    O.run_pair(cfg, params, scene["left"][:16], scene["right"][:16])  # warm the library / threads
    t = time.perf_counter()
    for _ in range(pairs):
        O.run_pair(cfg, params, scene["left"], scene["right"])
    dt = time.perf_counter() - t
    return pairs / dt, dt


def run_reference(args):
    # rank 0 alone times the CPU path; it needs no process group, so the other
    # ranks of a torchrun launch exit at once
    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    from cnncrf import scenes
    wl = WORKLOAD
    scene = scenes.kitti_scene(wl["W"], wl["H"], wl["D"], seed=0)
    cores = os.cpu_count()
    times = []
    for i in range(args.warmup + args.steps):
        v, dt = cpu_pairs_per_s(wl, scene, 1)
        if i >= args.warmup:
            times.append(dt)
    value = len(times) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded KITTI-shaped scene)",
        "config": workload_config(wl),
        "run": {"pairs_per_step": 1, "parallelism": "host OpenMP, %d threads" % cores},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": cores, "kind": "port",
                         "sample": "one full 1242x375 D=128 pair per step (CNN, correlation, CRF, remap)"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def build_stereo(cnncrf, wl, precision, stream):
    from cnncrf.api import Stereo
    st = Stereo(precision=precision, unary=cnncrf.UNARY_ONE_MINUS_DOT, topology=cnncrf.TOPO_ALL3X3,
                feat_channels=wl["feat"], pw_channels=wl["pw"], ref_depth_rounding=False,
                crf_shape=cnncrf.RHO_LINEAR, stream=stream)
    st.initialize(wl["W"], wl["H"], 0.0, 1.0, float(wl["D"] - 1))
    st.set_matching_function(cnncrf.MATCH_COLORCNN_PAIRWISE)
    st.set_num_layers(wl["layers"])
    st.set_xavier_seed(wl["seed"])
    return st


def train_setup(n=4, W=512, H=256, D=128, fp32=False, autotune=True):
    """The training step of 4 crops of 512 x 256 from the KITTI-shaped
    generator with its ground truth, D = 128, the 7-layer 100-channel nets.
    autotune: time the CRF tiles on the hinge's problem first (outside any
    timed region; tiles change no bit)."""
    import numpy as np
    import torch
    import cnncrf
    from cnncrf import scenes
    from cnncrf.train import Trainer
    sc = [scenes.kitti_scene(W, H, D, seed=40 + i) for i in range(n)]
    left = torch.from_numpy(np.stack([s["left"] for s in sc])).cuda()
    right = torch.from_numpy(np.stack([s["right"] for s in sc])).cuda()
    gt = torch.from_numpy(np.stack([np.clip(np.rint(s["disp"]), 0, D - 1).astype(np.int32) for s in sc])).cuda()
    kw = dict(precision=cnncrf.FP32, checkpoint_every=0) if fp32 else {}
    t = Trainer(n, W, H, disp_max=float(D - 1), **kw)
    t.init_xavier(0)
    if autotune:
        t.forward(left, right)
        t.autotune()
    return t, left, right, gt


def train_line(args, steps):
    """Training steps per second: forward, hinge on the loss-augmented CRF,
    the adjoints, SGD with momentum (lr 1e-3, momentum 0.9).  value: crops
    resident in HBM; e2e: the same step from pinned host crops and labels
    (H2D inside the timed region) with the per-pair losses read back."""
    import torch
    from cnncrf import _lib, tuning
    t, left, right, gt = train_setup(n=args.train_pairs, fp32=args.precision == "fp32",
                                     autotune=not args.no_autotune)
    hl, hr, hg = left.cpu().pin_memory(), right.cpu().pin_memory(), gt.cpu().pin_memory()
    dl, dr, dg = torch.empty_like(left), torch.empty_like(right), torch.empty_like(gt)
    for _ in range(max(args.warmup, 3)):
        t.step(left, right, gt, lr=1e-3, momentum=0.9)
    torch.cuda.synchronize()

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(steps):
            out = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, out

    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    l0 = _lib.kernel_launches()
    ms, losses = timed(lambda: t.step(left, right, gt, lr=1e-3, momentum=0.9))
    launches = _lib.kernel_launches() - l0
    clk = clocks.stop()

    def step_e2e():
        dl.copy_(hl, non_blocking=True)
        dr.copy_(hr, non_blocking=True)
        dg.copy_(hg, non_blocking=True)
        return t.step(dl, dr, dg, lr=1e-3, momentum=0.9)  # returns the losses on the host
    e_ms, _ = timed(step_e2e)
    _lib.profile_reset()
    _lib.profile_enable(True)
    for _ in range(3):
        t.step(left, right, gt, lr=1e-3, momentum=0.9)
    torch.cuda.synchronize()
    _lib.profile_enable(False)
    prof = {k: _lib.profile_query(k) for k in _lib.profile_kernels()}
    _lib.profile_reset()
    tot = sum(v for _, v in prof.values()) or 1.0
    peaks, peak_src = measured_peaks()
    n, W, H, D, iters = args.train_pairs, 512, 256, 128, WORKLOAD["crf_iters"]
    roof = None
    if "crf_h" in prof and "crf_v" in prof:  # the loss-augmented CRF, the largest share of the step
        tt = prof["crf_h"][1] + prof["crf_v"][1]
        nl = prof["crf_h"][0] + prof["crf_v"][0]
        gbs = crf_bytes_per_pass(W, H, D) * n * nl / (tt / 1000.0) / 1e9
        roof = {"kernel": "crf_h+crf_v", "bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": gbs / peaks["hbm_gbs"], "traffic": None, "peak_source": peak_src,
                "per_launch": "algorithmic 3 x N x D x 4 B per pass of the %d crops / the passes' summed "
                              "launch time" % n}
    conv_roof = None
    if "conv_tc" in prof:
        # forward and recomputed feature / pairwise layers and the input gradients run on k_conv_tc; its
        # FLOPs per step are counted by the launches' own shapes in the training profile summary
        conv_roof = {"kernel": "conv_tc", "share": round(prof["conv_tc"][1] / tot, 4),
                     "ms_per_step": round(prof["conv_tc"][1] / 3, 3)}
    return {"metric": "training steps/s, %d crops 512x256 D=128 (7x3x3 100ch + pairwise nets, CRF hinge, SGD)"
                      % n,
            "value": 1000.0 / ms, "unit": "steps/s", "steps": steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms, "higher_is_better": True,
            "dtype": "bf16" if args.precision == "bf16" else "f32", "data": "synthetic (KITTI-shaped crops)",
            "config": {"workload": "train%dx512x256_d128" % n,
                       "checkpoint_every": 0 if args.precision == "fp32" else 3,
                       "lr": 1e-3, "momentum": 0.9, "loss": "mean structured hinge", "crf_iters": iters,
                       "crf_tile": tuning.get_tile(W, H, D, n, 3)[0]},
            "e2e": {"value": 1000.0 / e_ms, "unit": "steps/s", "ms_per_step": e_ms,
                    "h2d_bytes_per_step": 2 * hl.numel() * 4 + hg.numel() * 4, "d2h_bytes_per_step": 8 * n},
            "gpu_launches": int(round(launches / steps)) * steps,
            "roofline": roof, "conv_tc": conv_roof,
            "loss_per_pixel": [float(x) for x in losses], "clocks": clk,
            "kernels": {k: {"launches": c // 3, "ms_per_step": round(v / 3, 3), "share": round(v / tot, 4)}
                        for k, (c, v) in sorted(prof.items(), key=lambda kv: -kv[1][1])}}


def run_train(args):
    line = train_line(args, args.steps)
    line.update({"n_gpus": 1, "scaling": "weak", "vs_baseline": None})
    print(json.dumps(line))
    return 0


MBQ = dict(name="mbq720x480_d96", W=720, H=480, D=96, L1=0.5, L2=1.5, delta=3, crf_iters=5, lam=1.0,
           tv_iters=4, tv_warps=1, huber_eps=0.01)


def tv_bytes_per_launch(W, H, first, last):
    """Algorithmic bytes of one fused TV launch: u, u0, the fit (a, b) and the
    two weights read, p and q read unless the launch starts from p = q = 0,
    u, p and q written, and u_ written by the last launch."""
    rd = 4 + 4 + 8 + 4 + 4 + (0 if first else 16)
    wr = 4 + 8 + 8 + (4 if last else 0)
    return (rd + wr) * W * H


def mbq_tv_line(args, steps):
    """The Middlebury-Q-shaped configuration: 720x480 RGB, D = 96, the plain
    FP32 path (7-layer all-3x3 100-channel net, L2-normalised features, 1-dot
    unary, pairwise CNN, truncated-linear CRF with 5 iterations), then the
    TV/Huber refinement: one warp (re-match on 3 labels through the net,
    quadratic fit) and 4 fused primal-dual iterations, Huber eps 0.01,
    lambda 1.  value: pairs/s with the images in HBM; e2e: from pinned host
    images to the refined disparities on the host.  The oracle runs the same
    pair on the host cores (cpu_baseline), and its result is compared bit for
    bit.  The TV kernel's roofline is measured at this size and, because one
    720x480 launch moves 17 MB (less than L2), also on a 4096x2160 field."""
    import numpy as np
    import torch
    import cnncrf
    from cnncrf import scenes, _lib, api
    from cnncrf.api import Stereo
    m = MBQ
    W, H, D = m["W"], m["H"], m["D"]
    sc = scenes.workload(m["name"], seed=0)
    stream = torch.cuda.Stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    with torch.cuda.stream(stream):
        st = Stereo(precision=cnncrf.FP32, unary=cnncrf.UNARY_ONE_MINUS_DOT, topology=cnncrf.TOPO_ALL3X3,
                    ref_depth_rounding=False, crf_shape=cnncrf.RHO_LINEAR, huber_eps=m["huber_eps"], stream=stream)
        st.initialize(W, H, 0.0, 1.0, float(D - 1))
        st.set_matching_function(cnncrf.MATCH_COLORCNN_PAIRWISE)
        st.set_num_layers(7)
        st.set_xavier_seed(0)
        dl, dr = torch.from_numpy(sc["left"]).cuda(), torch.from_numpy(sc["right"]).cuda()
        hl, hr = torch.from_numpy(sc["left"]).pin_memory(), torch.from_numpy(sc["right"]).pin_memory()
        hout = torch.empty((H, W), dtype=torch.float32).pin_memory()

        def run(l, r):
            st.set_color_images(l, r)
            st.compute_slack_propagation(m["L1"], m["L2"], m["delta"], m["crf_iters"], 0.0, 0.0, m["lam"])
            st.fuse_thuber_quad_fit(m["lam"], m["L2"], m["tv_iters"], m["tv_warps"])

        def timed(fn, n):
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
            torch.cuda.synchronize()
            for a, e in evs:
                flush.zero_()
                a.record(stream)
                fn()
                e.record(stream)
            torch.cuda.synchronize()
            return sum(a.elapsed_time(e) for a, e in evs)

        for _ in range(max(args.warmup, 3)):
            run(dl, dr)
        torch.cuda.synchronize()
        clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
        clocks.start()
        l0 = _lib.kernel_launches()
        t_ms = timed(lambda: run(dl, dr), steps)
        launches = _lib.kernel_launches() - l0
        clk = clocks.stop()
        e_ms = timed(lambda: (run(hl, hr), st.get_output_into(hout)), steps)
        disp = hout.numpy().copy()
        labels = st.labels_device().cpu().numpy()
        # per-kernel device time over a few steps
        _lib.profile_reset()
        _lib.profile_enable(True)
        nprof = 3
        timed(lambda: run(dl, dr), nprof)
        _lib.profile_enable(False)
        prof = {k: _lib.profile_query(k) for k in _lib.profile_kernels()}
        _lib.profile_reset()
        # the TV kernel alone on a field larger than L2 (4 iterations from p = q = 0: one launch)
        Wl, Hl = 4096, 2160
        g = torch.Generator(device="cuda").manual_seed(1)
        u0 = torch.rand((Hl, Wl), device="cuda", generator=g) * 90
        qf = torch.stack([torch.randn((Hl, Wl), device="cuda", generator=g),
                          torch.rand((Hl, Wl), device="cuda", generator=g) * 3], -1).contiguous()
        wx = torch.rand((Hl, Wl), device="cuda", generator=g) * 2
        wy = torch.rand((Hl, Wl), device="cuda", generator=g) * 2
        api.tv_iterate(u0, u0, qf, wx, wy, m["L2"], m["huber_eps"], 1.0, m["tv_iters"], stream=stream)
        _lib.profile_reset()
        _lib.profile_enable(True)
        big_n = 10
        timed(lambda: api.tv_iterate(u0, u0, qf, wx, wy, m["L2"], m["huber_eps"], 1.0, m["tv_iters"],
                                     stream=stream), big_n)
        _lib.profile_enable(False)
        big = _lib.profile_query("tv")
        _lib.profile_reset()
    peaks, peak_src = measured_peaks()
    roof = None
    if "tv" in prof:
        c, tt = prof["tv"]
        per = tv_bytes_per_launch(W, H, True, True)  # 4 iterations from p = q = 0: one launch per refinement
        gbs = per * c / (tt / 1000.0) / 1e9
        roof = {"kernel": "tv", "bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": gbs / peaks["hbm_gbs"], "traffic": None, "peak_source": peak_src,
                "us_per_launch": 1000.0 * tt / c,
                "per_launch": "algorithmic %d B per pixel (u, u0, a, b, wx, wy read; u, p, q, u_ written) x "
                              "720 x 480 / the launch's CUDA-event time" % (per // (W * H))}
        bc, bt = big
        bper = tv_bytes_per_launch(Wl, Hl, True, True)
        bgbs = bper * bc / (bt / 1000.0) / 1e9
        roof["streaming"] = {"field": "%dx%d" % (Wl, Hl), "achieved": bgbs, "frac": bgbs / peaks["hbm_gbs"],
                             "us_per_launch": 1000.0 * bt / bc, "launches": bc}
    tot = sum(v for _, v in prof.values()) or 1.0
    kernels = {k: {"launches": c // nprof, "ms_per_step": round(v / nprof, 4), "share": round(v / tot, 4)}
               for k, (c, v) in sorted(prof.items(), key=lambda kv: -kv[1][1])}
    # the oracle on the same pair: the CPU baseline, and the bit-exact check of this run's result
    from oracle import oracle as O
    cfg = O.make_cfg(num_layers=7, topology=1, unary=1, disp_max=float(D - 1), lam=m["lam"], L1=m["L1"],
                     L2=m["L2"], delta=float(m["delta"]), crf_iters=m["crf_iters"], crf_shape=1,
                     warps=m["tv_warps"], ref_iters=m["tv_iters"], huber_eps=m["huber_eps"], C=m["L2"])
    params = O.xavier_params(cfg, seed=0)
    t0 = time.perf_counter()
    r = O.run_pair(cfg, params, sc["left"], sc["right"])
    dt = time.perf_counter() - t0
    return {"metric": "stereo pairs/s at 720x480 D=96, FP32 path + 4 TV/Huber iterations",
            "value": steps / (t_ms / 1000.0), "unit": "pairs/s", "steps": steps, "warmup": max(args.warmup, 3),
            "ms_per_step": t_ms / steps, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded Voronoi plane scene, 30 cells)",
            "config": {"workload": m["name"], "W": W, "H": H, "D": D, "crf_iters": m["crf_iters"],
                       "tv_iterations": m["tv_iters"], "tv_warps": m["tv_warps"], "huber_eps": m["huber_eps"],
                       "lambda": m["lam"], "net": "7x3x3 conv 100ch + L2 norm, 1-dot unary, pairwise CNN",
                       "crf": "truncated linear L1=0.5 T=3", "l2": "flushed (256 MiB write) between steps"},
            "e2e": {"value": steps / (e_ms / 1000.0), "unit": "pairs/s", "h2d_bytes_per_step": 2 * W * H * 16,
                    "d2h_bytes_per_step": W * H * 4},
            "gpu_launches": launches,
            "roofline": roof, "kernels": kernels, "clocks": clk,
            "bitexact_vs_oracle": {"labels": bool(np.array_equal(labels, r["labels"])),
                                   "refined_disparities": bool(np.array_equal(disp, r["disp"]))},
            "cpu_baseline": {"value": 1.0 / dt, "unit": "pairs/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "one full 720x480 D=96 pair (CNN, correlation, CRF, TV refinement), "
                                       "%.1f s" % dt}}


def run_profile(args):
    """The device work alone, for ncu: eager launches, no timing, FP32
    comparison or CPU leg.  kitti: one group of --batch pairs; uneven: the
    uneven batch; train: training steps."""
    import torch
    import cnncrf
    wl = WORKLOAD
    if args.workload == "tv":
        # the fused TV kernel alone: 4 iterations from p = q = 0 (one launch) on a 4096 x 2160 field
        from cnncrf import api
        Wl, Hl = 4096, 2160
        g = torch.Generator(device="cuda").manual_seed(1)
        u0 = torch.rand((Hl, Wl), device="cuda", generator=g) * 90
        qf = torch.stack([torch.randn((Hl, Wl), device="cuda", generator=g),
                          torch.rand((Hl, Wl), device="cuda", generator=g) * 3], -1).contiguous()
        wx = torch.rand((Hl, Wl), device="cuda", generator=g) * 2
        wy = torch.rand((Hl, Wl), device="cuda", generator=g) * 2
        for _ in range(args.warmup + args.steps):
            api.tv_iterate(u0, u0, qf, wx, wy, MBQ["L2"], MBQ["huber_eps"], 1.0, MBQ["tv_iters"])
        torch.cuda.synchronize()
        print("profile run done")
        return 0
    if args.workload == "train":
        t, left, right, gt = train_setup(n=args.train_pairs, fp32=args.precision == "fp32",
                                         autotune=not args.no_autotune)
        for _ in range(args.warmup + args.steps):
            t.step(left, right, gt, lr=1e-3, momentum=0.9)
        torch.cuda.synchronize()
        print("profile run done")
        return 0
    if args.workload == "uneven":
        from cnncrf import scenes
        from cnncrf.api import StereoBatch
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            sc = scenes.uneven_scenes(args.per_shape)
            b = StereoBatch(precision=cnncrf.BF16, unary=cnncrf.UNARY_ONE_MINUS_DOT, topology=cnncrf.TOPO_ALL3X3,
                            crf_shape=cnncrf.RHO_LINEAR, num_layers=wl["layers"], seed=wl["seed"], graph=False,
                            stream=stream, group_size=max(1, args.per_shape // 2))
            for x in sc:
                b.add_pair(x["W"], x["H"], 0.0, 1.0, float(x["D"] - 1))
            dl = [torch.from_numpy(x["left"]).cuda() for x in sc]
            dr = [torch.from_numpy(x["right"]).cuda() for x in sc]
            for _ in range(args.warmup + args.steps):
                for i in range(len(sc)):
                    b.set_images(i, dl[i], dr[i])
                b.run(wl["L1"], wl["L2"], wl["delta"], wl["crf_iters"], wl["lam"])
            b.check()
            torch.cuda.synchronize()
        print("profile run done")
        return 0
    precision = cnncrf.BF16 if args.precision == "bf16" else cnncrf.FP32
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        b, sc = make_batch(cnncrf, wl, args.batch, precision, False, stream, seed0=0, group_size=0)
        dl = [torch.from_numpy(x["left"]).cuda() for x in sc]
        dr = [torch.from_numpy(x["right"]).cuda() for x in sc]
        for _ in range(args.warmup + args.steps):
            for i in range(args.batch):
                b.set_images(i, dl[i], dr[i])
            b.run(wl["L1"], wl["L2"], wl["delta"], wl["crf_iters"], wl["lam"])
        b.check()
        torch.cuda.synchronize()
    print("profile run done")
    return 0


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) measured with ncu on one-pair launches
# of this workload, scaled to a launch of the 8-pair step (traffic grows with the images / chains):
# k_conv_tc layer 3 over 2 images 449.9 MB; k_crf_chain H pass (reading the 16-bit unary) 1311.8 MB and
# V pass 1069.9 MB per pair.
CONV_TC_BYTES_PER_IMAGE = 449.9e6 / 2
CRF_H_BYTES_PER_PAIR, CRF_V_BYTES_PER_PAIR = 1311.8e6, 1069.9e6


def make_batch(cnncrf, wl, B, precision, graph, stream, seed0, group_size=0):
    from cnncrf import scenes
    from cnncrf.api import StereoBatch
    b = StereoBatch(precision=precision, unary=cnncrf.UNARY_ONE_MINUS_DOT, topology=cnncrf.TOPO_ALL3X3,
                    feat_channels=wl["feat"], pw_channels=wl["pw"], crf_shape=cnncrf.RHO_LINEAR,
                    num_layers=wl["layers"], seed=wl["seed"], graph=graph, stream=stream, group_size=group_size)
    sc = [scenes.kitti_scene(wl["W"], wl["H"], wl["D"], seed=seed0 + i) for i in range(B)]
    for _ in range(B):
        b.add_pair(wl["W"], wl["H"], 0.0, 1.0, float(wl["D"] - 1))
    return b, sc


def uneven_line(args, steps, rank=0, world=1, local=0):
    """The uneven batch: --per-shape pairs of each of 480x320/D64, 720x480/D96,
    1242x375/D128 and 1440x960/D192 (32 by default) through one StereoBatch,
    replayed as one CUDA graph per step; pairs/s of the whole batch, the CRF's
    HBM GB/s and the tensor-core convolutions' TFLOP/s."""
    import numpy as np
    import torch
    import cnncrf
    from cnncrf import scenes, _lib
    from cnncrf.api import StereoBatch

    wl = WORKLOAD
    shapes, per = scenes.UNEVEN_SHAPES, args.per_shape
    gs = args.group_size if args.group_size >= 0 else max(1, per // 2)
    crf = (wl["L1"], wl["L2"], wl["delta"], wl["crf_iters"], wl["lam"])
    stream = torch.cuda.Stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2

    def batch(scs, graph, group_size):
        b = StereoBatch(precision=cnncrf.BF16, unary=cnncrf.UNARY_ONE_MINUS_DOT, topology=cnncrf.TOPO_ALL3X3,
                        feat_channels=wl["feat"], pw_channels=wl["pw"], crf_shape=cnncrf.RHO_LINEAR,
                        num_layers=wl["layers"], seed=wl["seed"], graph=graph, stream=stream,
                        group_size=group_size)
        for x in scs:
            b.add_pair(x["W"], x["H"], 0.0, 1.0, float(x["D"] - 1))
        return b

    def timed(fn, steps):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier(world)
        torch.cuda.synchronize()
        for a, e in evs:
            flush.zero_()
            a.record(stream)
            fn()
            e.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        return allmax(sum(a.elapsed_time(e) for a, e in evs), world)

    sc = scenes.uneven_scenes(per, seed0=1000 * rank)
    B = len(sc)
    with torch.cuda.stream(stream):
        b = batch(sc, not args.no_graph, gs)
        dl = [torch.from_numpy(x["left"]).cuda() for x in sc]
        dr = [torch.from_numpy(x["right"]).cuda() for x in sc]
        hl = [torch.from_numpy(x["left"]).pin_memory() for x in sc]
        hr = [torch.from_numpy(x["right"]).pin_memory() for x in sc]
        hout = [torch.empty((x["H"], x["W"]), dtype=torch.float32).pin_memory() for x in sc]

        def step_device():
            for i in range(B):
                b.set_images(i, dl[i], dr[i])
            b.run(*crf)

        def step_e2e():
            # host images in, host disparities out, the copies pipelined with the groups' work
            b.run_host(hl, hr, hout, *crf)

        for i in range(B):
            b.set_images(i, dl[i], dr[i])
        tiles = b.autotune(*crf) if not args.no_autotune else []
        for _ in range(max(args.warmup, 3)):
            step_device()
        for _ in range(2):  # its graph: an eager run, then the capture
            step_e2e()
        b.check()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        l0 = _lib.kernel_launches()
        t_ms = timed(step_device, steps)
        launches = _lib.kernel_launches() - l0
        clk = clocks.stop()
        e_ms = timed(step_e2e, steps)
        b.check()
        bad = float(np.mean([scenes.bad_pixels(hout[i].numpy(), sc[i]["disp"]) for i in range(B)]))
        del b
        torch.cuda.synchronize()

        # per-kernel device time, one shape at a time (one group, eager), so
        # no kernel of another group overlaps the events around a launch
        nprof = 2
        prof, per_shape = {}, {}
        for j, (W, H, D) in enumerate(shapes):
            part = sc[j * per:(j + 1) * per]
            bp = batch(part, False, 0)
            for i in range(per):
                bp.set_images(i, dl[j * per + i], dr[j * per + i])
            if not args.no_autotune:
                bp.autotune(*crf)
            bp.run(*crf)
            torch.cuda.synchronize()
            _lib.profile_reset()
            _lib.profile_enable(True)
            p_ms = timed(lambda: bp.run(*crf), nprof)
            _lib.profile_enable(False)
            kp = {k: _lib.profile_query(k) for k in _lib.profile_kernels()}
            _lib.profile_reset()
            bp.check()
            del bp
            per_shape["%dx%d_d%d" % (W, H, D)] = {
                "pairs": per, "ms_per_pair_eager": p_ms / nprof / per,
                "kernels_ms_per_pair": {k: round(t / nprof / per, 4) for k, (n, t) in kp.items()}}
            for k, (n, t) in kp.items():
                a = prof.setdefault(k, [0, 0.0])
                a[0] += n
                a[1] += t
    if not args.no_graph:
        launches_per_step = sum(n for n, _ in prof.values()) / nprof
    else:
        launches_per_step = launches / steps
    if rank != 0:
        return None
    peaks, peak_src = measured_peaks()
    tc_f = sum(conv_flops(W, H, wl["layers"], wl["feat"], 3, wl["pw"])[0] for (W, H, D) in shapes) * per
    crf_b = sum(crf_bytes_per_pass(W, H, D) for (W, H, D) in shapes) * per * 2 * wl["crf_iters"]
    roof = crf_roof = None
    if "conv_tc" in prof:
        ach = tc_f * nprof / (prof["conv_tc"][1] / 1000.0) / 1e12
        roof = {"kernel": "conv_tc", "bound": "tensor", "achieved": ach, "peak": peaks["bf16_tflops"],
                "unit": "TFLOP/s", "frac": ach / peaks["bf16_tflops"], "traffic": None,
                "peak_source": peak_src + " (bf16 dense burst)",
                "per_launch": "FLOPs of the tensor-core layers of all pairs / their summed launch time"}
    if "crf_h" in prof and "crf_v" in prof:
        t = prof["crf_h"][1] + prof["crf_v"][1]
        gbs = crf_b * nprof / (t / 1000.0) / 1e9
        crf_roof = {"kernel": "crf_h+crf_v", "bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"],
                    "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"], "traffic": None, "peak_source": peak_src,
                    "per_launch": "algorithmic 3 x N x D x 4 B per pass of all pairs / summed pass time"}
    tot = sum(t for _, t in prof.values()) or 1.0
    kernels = {k: {"launches": n, "total_ms": round(t, 4), "share": round(t / tot, 4)} for k, (n, t) in prof.items()}
    value = replica_value(steps, B, world, t_ms)
    line = {
        "metric": "stereo pairs/s, uneven batch (480x320/D64, 720x480/D96, 1242x375/D128, 1440x960/D192)",
        "value": value, "unit": "pairs/s", "n_gpus": world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": t_ms / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16", "data": "synthetic (seeded Voronoi plane scenes, 30 cells, per pair seed)",
        "config": {"workload": "uneven%d" % B, "shapes": ["%dx%d_d%d" % x for x in shapes], "pairs_per_shape": per,
                   "pairs_per_group": gs, "graph": not args.no_graph, "crf_iters": wl["crf_iters"],
                   "net": "7x3x3 conv 100ch + L2 norm, 1-dot unary, pairwise CNN 3x3-3x3-1x1",
                   "crf": "truncated linear L1=0.5 T=3", "l2": "flushed (256 MiB write) between steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": replica_value(steps, B, world, e_ms), "unit": "pairs/s",
                "h2d_bytes_per_step": sum(2 * x["W"] * x["H"] * 16 for x in sc),
                "d2h_bytes_per_step": sum(x["W"] * x["H"] * 4 for x in sc)},
        "gpu_launches": int(round(launches_per_step * steps)),
        # the dominant kernel is the CRF (its two passes are most of the step); the conv beside it
        "roofline": crf_roof, "conv_roofline": roof, "kernels": kernels, "per_shape": per_shape, "clocks": clk,
        "crf_tiles": [dict(shape="%dx%d_d%d x%d" % (t["W"], t["H"], t["D"], t["npairs"]), **t["tile"])
                      for t in tiles],
        "conv_forms": conv_forms_summary(),
        "cpu_baseline": None,
        "disparity_stats": {"kitti_bad3px_5pct_mean": bad,
                            "definition": "eval/compute_numbers_kitti.py computeError on PNG16-quantised maps, "
                                          "mean over the batch, synthetic ground truth"},
    }
    return line


def run_uneven(args):
    import torch
    rank, world, local = dist_setup()
    torch.cuda.set_device(local)
    line = uneven_line(args, args.steps, rank, world, local)
    if line is not None:
        print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=8, help="KITTI pairs per step (the batched form)")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--group-size", type=int, default=-1,
                    help="pairs per pipelined group of the batch (0: one group of --batch pairs; "
                         "default: half the batch)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16", choices=["bf16", "fp32"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="kitti", choices=["kitti", "uneven", "train", "tv"],
                    help="uneven: --per-shape pairs of each of four sizes / ranges in one batch; "
                         "train: the training step of 4 crops of 512 x 256, D = 128; "
                         "tv: the fused TV kernel alone (--mode profile only)")
    ap.add_argument("--per-shape", type=int, default=8)
    ap.add_argument("--train-pairs", type=int, default=4, help="crops per training step (train workload)")
    ap.add_argument("--no-autotune", action="store_true", help="run the default CRF tile (no tile tuning)")
    ap.add_argument("--no-extras", action="store_true",
                    help="only the KITTI line: leave out the mbq_tv, train and uneven sub-benchmarks")
    ap.add_argument("--mode", default="bench", choices=["bench", "profile"],
                    help="profile: only warm-up + `steps` device steps of the path (for ncu captures)")
    args = ap.parse_args()
    if args.workload == "tv" and args.mode != "profile":
        ap.error("--workload tv runs the TV kernel alone for a profiler: add --mode profile")
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "profile":
        return run_profile(args)
    if args.workload == "uneven":
        return run_uneven(args)
    if args.workload == "train":
        return run_train(args)

    import torch
    rank, world, local = dist_setup()
    torch.cuda.set_device(local)
    line = kitti_line(args, rank, world, local)
    if line is None:
        return 0
    if world == 1 and not args.no_extras and args.precision == "bf16":
        # the task's other configurations, each with its own value / e2e / roofline / clocks
        import copy
        sub = copy.copy(args)
        sub.group_size = -1
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        line["mbq_tv"] = mbq_tv_line(sub, steps=10)
        torch.cuda.empty_cache()
        line["train"] = train_line(sub, steps=20)
        torch.cuda.empty_cache()
        line["uneven"] = uneven_line(sub, steps=5)
    print(json.dumps(line))
    return 0


def kitti_line(args, rank, world, local):
    """The metric's workload (one line; None on ranks other than 0)."""
    import numpy as np
    import torch
    import cnncrf
    from cnncrf import scenes, _lib

    wl = WORKLOAD
    W, H, D, B = wl["W"], wl["H"], wl["D"], args.batch
    if args.group_size < 0:
        args.group_size = max(1, B // 2) if B >= 4 else 0
    precision = cnncrf.BF16 if args.precision == "bf16" else cnncrf.FP32
    crf = (wl["L1"], wl["L2"], wl["delta"], wl["crf_iters"], wl["lam"])
    stream = torch.cuda.Stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    with torch.cuda.stream(stream):
        b, sc = make_batch(cnncrf, wl, B, precision, not args.no_graph, stream, seed0=1000 * rank,
                           group_size=args.group_size)
        dl = [torch.from_numpy(x["left"]).cuda() for x in sc]
        dr = [torch.from_numpy(x["right"]).cuda() for x in sc]
        hl = [torch.from_numpy(x["left"]).pin_memory() for x in sc]
        hr = [torch.from_numpy(x["right"]).pin_memory() for x in sc]
        hout = [torch.empty((H, W), dtype=torch.float32).pin_memory() for _ in range(B)]

        def step_device():
            for i in range(B):
                b.set_images(i, dl[i], dr[i])
            b.run(*crf)

        def step_e2e():
            # host images in, host disparities out, the copies pipelined with the groups' work
            b.run_host(hl, hr, hout, *crf)

        for i in range(B):
            b.set_images(i, dl[i], dr[i])
        tiles = b.autotune(*crf) if not args.no_autotune else []
        for _ in range(max(args.warmup, 3)):
            step_device()
        for _ in range(2):  # its graph: an eager run, then the capture
            step_e2e()
        b.check()
        torch.cuda.synchronize()

        def timed(fn, steps):
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(steps)]
            barrier(world)
            torch.cuda.synchronize()
            for a, e in evs:
                flush.zero_()
                a.record(stream)
                fn()
                e.record(stream)
            torch.cuda.synchronize()
            barrier(world)
            return allmax(sum(a.elapsed_time(e) for a, e in evs), world)

        # ---- timed region: device-resident inputs (graph replay of the batch step)
        clocks = ClockSampler(local)
        clocks.start()
        l0 = _lib.kernel_launches()
        t_ms = timed(step_device, args.steps)
        launches = _lib.kernel_launches() - l0
        clk = clocks.stop()
        value = replica_value(args.steps, B, world, t_ms)
        # ---- end to end through the public API from pinned host buffers
        e_ms = timed(step_e2e, args.steps)
        e2e = replica_value(args.steps, B, world, e_ms)
        b.check()
        labels_b = [b.labels_device(i).cpu().numpy() for i in range(B)]

        # ---- per-kernel device time: the same batch step run eagerly as one
        # group (no overlap between kernels) with CUDA events around every
        # launch on its stream
        bp, _ = make_batch(cnncrf, wl, B, precision, False, stream, seed0=1000 * rank)
        for i in range(B):
            bp.set_images(i, dl[i], dr[i])
        if not args.no_autotune:
            bp.autotune(*crf)
        bp.run(*crf)
        torch.cuda.synchronize()
        _lib.profile_reset()
        _lib.profile_enable(True)
        nprof = max(3, args.steps // 4)
        p_ms = timed(lambda: bp.run(*crf), nprof)
        _lib.profile_enable(False)
        prof = {k: _lib.profile_query(k) for k in _lib.profile_kernels()}
        _lib.profile_reset()
        del bp
        if args.no_graph:
            launches_per_step = launches / args.steps
        else:
            launches_per_step = sum(n for n, _ in prof.values()) / nprof

    # ---- BF16 vs FP32: label change on the same pair, single-pair FP32 pairs/s
    cmp = {}
    if precision == cnncrf.BF16:
        with torch.cuda.stream(stream):
            st32 = build_stereo(cnncrf, wl, cnncrf.FP32, stream)
            st32.set_color_images(dl[0], dr[0])
            st32.compute_slack_propagation(wl["L1"], wl["L2"], wl["delta"], wl["crf_iters"], 0.0, 0.0, wl["lam"])
            torch.cuda.synchronize()
            if not args.no_autotune:  # the single-pair shape both single-pair paths run
                from cnncrf.api import crf_autotune
                wx32, wy32 = st32.weights_device()
                crf_autotune(st32.volume_device(), wx32, wy32, wl["L1"], wl["L2"], wl["delta"], wl["crf_iters"],
                             cnncrf.RHO_LINEAR, stream=stream)
            n32 = 3

            def step32():
                st32.set_color_images(dl[0], dr[0])
                st32.compute_slack_propagation(wl["L1"], wl["L2"], wl["delta"], wl["crf_iters"], 0.0, 0.0,
                                               wl["lam"])
            t32 = timed(step32, n32)
            # every pair of the step against the FP32 path on the same images
            changes = []
            for i in range(B):
                st32.set_color_images(dl[i], dr[i])
                st32.compute_slack_propagation(wl["L1"], wl["L2"], wl["delta"], wl["crf_iters"], 0.0, 0.0,
                                               wl["lam"])
                lab32 = st32.labels_device().cpu().numpy()
                changes.append(float((lab32 != labels_b[i]).mean()))
            st1 = build_stereo(cnncrf, wl, cnncrf.BF16, stream)
            step1 = lambda: (st1.set_color_images(dl[0], dr[0]),
                             st1.compute_slack_propagation(wl["L1"], wl["L2"], wl["delta"], wl["crf_iters"],
                                                           0.0, 0.0, wl["lam"]))
            step1()
            t1 = timed(step1, n32)
            cmp = {"fp32_single_pair_pairs_per_s": n32 / (t32 / 1000.0),
                   "bf16_single_pair_pairs_per_s": n32 / (t1 / 1000.0),
                   "disparity_change_vs_fp32_per_pair": changes,
                   "disparity_change_vs_fp32_max": max(changes),
                   "disparity_change_bound": 0.005,
                   "within_bound": max(changes) <= 0.005}
            cmp["speedup_vs_fp32"] = value / world / cmp["fp32_single_pair_pairs_per_s"]

    if rank != 0:
        return None

    peaks, peak_src = measured_peaks()
    tc_f, simt_f = conv_flops(W, H, wl["layers"], wl["feat"], 3, wl["pw"])
    kernels = {k: {"launches": n, "total_ms": round(t, 4)} for k, (n, t) in prof.items()}
    tot = sum(t for _, t in prof.values()) or 1.0
    for k in kernels:
        kernels[k]["share"] = round(prof[k][1] / tot, 4)
    roof = None
    conv_name = "conv_tc" if "conv_tc" in prof else "conv_simt"
    if conv_name in prof:
        n, t = prof[conv_name]
        flops = (tc_f if conv_name == "conv_tc" else tc_f + simt_f) * B * nprof
        achieved = flops / (t / 1000.0) / 1e12
        roof = {"kernel": conv_name, "bound": "tensor", "achieved": achieved, "peak": peaks["bf16_tflops"],
                "unit": "TFLOP/s", "frac": achieved / peaks["bf16_tflops"],
                "traffic": CONV_TC_BYTES_PER_IMAGE * 2 * B if conv_name == "conv_tc" else None,
                "traffic_unit": "DRAM bytes of one feature-layer launch (%d images; ncu, 2-image launch scaled)"
                                % (2 * B),
                "peak_source": peak_src + " (bf16 dense burst)",
                "per_launch": "FLOPs of the tensor-core layers of %d pairs / their summed launch time" % B}
    crf_roof = None
    if "crf_h" in prof and "crf_v" in prof:
        n = prof["crf_h"][0] + prof["crf_v"][0]
        t = prof["crf_h"][1] + prof["crf_v"][1]
        gbs = crf_bytes_per_pass(W, H, D) * B * n / (t / 1000.0) / 1e9
        tb = (CRF_H_BYTES_PER_PAIR + CRF_V_BYTES_PER_PAIR) / 2 * B
        crf_roof = {"kernel": "crf_h+crf_v", "bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"],
                    "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"], "traffic": tb,
                    "traffic_unit": "DRAM bytes per pass launch (%d pairs, mean of H and V; ncu, 1-pair launches "
                                    "scaled); achieved counts the algorithmic 3 x N x D x 4 B per pass" % B,
                    "measured_gbs": tb * n / (t / 1000.0) / 1e9, "peak_source": peak_src}

    cpu = None
    if not args.no_cpu_baseline:
        v, dt = cpu_pairs_per_s(wl, sc[0], 1)
        cpu = {"value": v, "unit": "pairs/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "one full 1242x375 D=128 pair (CNN, correlation, CRF, remap), %.1f s" % dt}

    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16" if precision == cnncrf.BF16 else "f32",
        "data": "synthetic (seeded KITTI-shaped scenes: ground plane + 15 boxes)",
        "config": workload_config(wl),
        "run": {"pairs_per_step": B, "pairs_per_group": args.group_size or B, "graph": not args.no_graph,
                "l2": "flushed (256 MiB write) between steps",
                "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "pairs/s", "h2d_bytes_per_step": B * 2 * W * H * 4 * 4,
                "d2h_bytes_per_step": B * W * H * 4},
        "gpu_launches": int(round(launches_per_step * args.steps)),
        # the dominant kernel is the CRF (its two passes are most of the step); the conv beside it
        "roofline": crf_roof, "conv_roofline": roof,
        "crf_tiles": [dict(shape="%dx%d_d%d x%d" % (t["W"], t["H"], t["D"], t["npairs"]), **t["tile"])
                      for t in tiles],
        "conv_forms": conv_forms_summary(),
        "kernels": kernels, "kernel_profile_ms_per_step": p_ms / nprof, "clocks": clk,
        "cpu_baseline": cpu,
        "precision_check": cmp,
        "disparity_stats": {"kitti_bad3px_5pct_mean": float(np.mean([scenes.bad_pixels(hout[i].numpy(), sc[i]["disp"])
                                                                    for i in range(B)])),
                            "definition": "eval/compute_numbers_kitti.py computeError on PNG16-quantised maps, "
                                          "mean over the step's pairs, synthetic ground truth"},
    }
    return line


if __name__ == "__main__":
    sys.exit(main())
