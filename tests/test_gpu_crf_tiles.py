"""GPU tests of the CRF tiles (prefetch depth and chains per CTA of the H and
V passes): every tile gives the oracle's labels and bound bit for bit, the
autotuners enter valid tiles and change no result, and chains far longer than
any image row run at every tile."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TILES = [(8, 2, 8, 2), (4, 1, 4, 1), (4, 2, 8, 4), (8, 4, 4, 2), (4, 4, 4, 4), (8, 1, 8, 1)]


def dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def problem(D, H=19, W=23, seed=0):
    rng = np.random.default_rng(seed + D)
    cost = rng.random((H, W, D)).astype(np.float32)
    wx = (rng.random((H, W)) * 0.5).astype(np.float32)
    wy = (rng.random((H, W)) * 0.5).astype(np.float32)
    return cost, wx, wy


def set_tile(tuning, W, H, D, np_, delta, t):
    tuning.set_tile(W, H, D, np_, delta, ring_h=t[0], chains_per_cta_h=t[1], ring_v=t[2], chains_per_cta_v=t[3])


@pytest.mark.parametrize("D", [5, 40, 96, 128, 192, 256])
def test_every_tile_gives_the_oracle_bits(cuda, oracle, D):
    torch = cuda
    from cnncrf import tuning
    from cnncrf.api import crf_solve
    H, W = 19, 23  # 19 and 23 chains: partial CTAs for 2 and 4 chains per CTA
    cost, wx, wy = problem(D, H, W)
    olab, olb, _, _ = oracle.crf(cost, wx, wy, 0.4, 1.3, 3, 3, shape=1)
    try:
        for t in TILES:
            set_tile(tuning, W, H, D, 1, 3, t)
            lab, lb = crf_solve(dev(cost, torch), dev(wx, torch), dev(wy, torch), L1=0.4, L2=1.3, delta=3,
                                total_it=3, shape=1)
            assert np.array_equal(lab.cpu().numpy(), olab), t
            assert lb == olb, t
    finally:
        tuning.clear()


def test_crf_autotune_single_pair(cuda):
    torch = cuda
    from cnncrf import tuning
    from cnncrf.api import crf_autotune, crf_solve
    D, H, W = 96, 40, 120
    cost, wx, wy = (dev(a, torch) for a in problem(D, H, W, seed=3))
    tuning.clear()
    try:
        lab0, lb0 = crf_solve(cost, wx, wy, L1=0.5, L2=1.5, delta=3, total_it=4, shape=1)
        crf_autotune(cost, wx, wy, L1=0.5, L2=1.5, delta=3, total_it=4, shape=1)
        tile, found, mh, mv = tuning.get_tile(W, H, D, 1, 3)
        assert found and mh > 0 and mv > 0
        assert tile["ring_h"] in (4, 8) and tile["ring_v"] in (4, 8)
        assert tile["chains_per_cta_h"] in (1, 2, 4) and tile["chains_per_cta_v"] in (1, 2, 4)
        lab1, lb1 = crf_solve(cost, wx, wy, L1=0.5, L2=1.5, delta=3, total_it=4, shape=1)
        assert torch.equal(lab0, lab1) and lb0 == lb1
    finally:
        tuning.clear()


def test_batch_autotune_changes_no_result(cuda):
    """Two shapes, two pairs each: results before tuning, from the tuning run
    and from the graph replays after it are the same bits."""
    torch = cuda
    from cnncrf import scenes, tuning, _lib as L
    from cnncrf.api import StereoBatch
    shapes = [(96, 48, 32), (64, 40, 40)]
    sc = scenes.uneven_scenes(2, shapes=shapes, seed0=3)
    tuning.clear()
    try:
        b = StereoBatch(precision=L.BF16, num_layers=3, seed=2, graph=True, group_size=0)
        for s in sc:
            b.add_pair(s["W"], s["H"], 0.0, 1.0, float(s["D"] - 1))
        for i, s in enumerate(sc):
            b.set_images(i, s["left"], s["right"])
        b.run(0.5, 1.5, 3, 4)
        ref = [b.get_output(i).copy() for i in range(len(sc))]
        lbs = [b.lower_bound(i) for i in range(len(sc))]
        groups = b.autotune(0.5, 1.5, 3, 4)
        assert [(g["W"], g["H"], g["D"], g["npairs"]) for g in groups] == [(96, 48, 32, 2), (64, 40, 40, 2)]
        assert all(g["found"] and g["ms_h"] > 0 and g["ms_v"] > 0 for g in groups)
        for rnd in range(3):  # the tuning run's outputs, then eager + captured replays with the tuned tiles
            for i in range(len(sc)):
                assert np.array_equal(b.get_output(i), ref[i]), (rnd, i)
                assert b.lower_bound(i) == lbs[i], (rnd, i)
            b.run(0.5, 1.5, 3, 4)
        b.check()
    finally:
        tuning.clear()


def test_long_chains_at_every_tile(cuda, oracle):
    """A 60000-pixel row: the chains' edge weights stream through registers,
    so a chain's shared memory does not grow with its length and every tile
    runs it, with the oracle's labels and bound."""
    torch = cuda
    from cnncrf import tuning
    from cnncrf.api import crf_solve
    D, H, W = 64, 2, 60000
    cost, wx, wy = problem(D, H, W, seed=5)
    olab, olb, _, _ = oracle.crf(cost, wx, wy, 0.5, 1.5, 2, 2, shape=1)
    try:
        for t in TILES:
            set_tile(tuning, W, H, D, 1, 2, t)
            lab, lb = crf_solve(dev(cost, torch), dev(wx, torch), dev(wy, torch), L1=0.5, L2=1.5, delta=2,
                                total_it=2, shape=1)
            assert np.array_equal(lab.cpu().numpy(), olab), t
            assert lb == olb, t
    finally:
        tuning.clear()
