"""Failure detection on the GPU without a fault: every device wait of the
tensor-core kernels is bounded, and a wait that runs out raises the kernel's
error flag, which the host reports as CNNCRF_ETIMEOUT.  The probe below runs
that wait on a barrier nothing completes, with a small poll limit, so the
timeout path runs for real; the context must stay usable afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_completes_when_the_barrier_does(cuda):
    from cnncrf import _lib as L
    for polls in (1, 64, 4096):
        assert L.selftest_bounded_wait(polls, arrive=True) == L.OK


@pytest.mark.parametrize("polls", [1, 256, 4096])
def test_bounded_wait_times_out_and_reports(cuda, polls):
    from cnncrf import _lib as L
    st = L.selftest_bounded_wait(polls, arrive=False)
    assert st == L.ETIMEOUT
    msg = L.lib().cnncrf_last_error().decode()
    assert "bounded wait" in msg and str(polls) in msg


def test_context_usable_after_timeout(cuda, oracle):
    """After a run-out wait on the same stream, a CRF solve still matches the
    oracle bit for bit, and a BF16 batch (whose tensor-core kernels carry the
    bounded waits) runs and checks clean."""
    torch = cuda
    from cnncrf import scenes, _lib as L
    from cnncrf.api import crf_solve, StereoBatch
    assert L.selftest_bounded_wait(512, arrive=False) == L.ETIMEOUT
    rng = np.random.default_rng(5)
    H, W, D = 11, 19, 40
    cost = rng.random((H, W, D)).astype(np.float32)
    wx = (rng.random((H, W)) * 0.5).astype(np.float32)
    wy = (rng.random((H, W)) * 0.5).astype(np.float32)
    lab, lb = crf_solve(torch.from_numpy(cost).cuda(), torch.from_numpy(wx).cuda(), torch.from_numpy(wy).cuda(),
                        L1=0.3, L2=1.1, delta=2, total_it=3, shape=0, slack=0.5)
    olab, olb, _, _ = oracle.crf(cost, wx, wy, 0.3, 1.1, 2, 3, shape=0, slack=0.5)
    assert np.array_equal(lab.cpu().numpy(), olab) and lb == olb
    assert L.selftest_bounded_wait(512, arrive=False) == L.ETIMEOUT
    b = StereoBatch(precision=L.BF16, num_layers=3, seed=0)
    b.add_pair(64, 32, 0.0, 1.0, 31.0)
    s = scenes.voronoi_scene(64, 32, 32, seed=3, cells=4, off_range=(1, 30))
    b.set_images(0, s["left"], s["right"])
    b.run(0.5, 1.5, 3, 2)
    b.check()
    assert np.isfinite(b.get_output(0)).all()
    assert L.selftest_bounded_wait(64, arrive=True) == L.OK
