"""The C oracle's census, edge-weight, QuadDirect and left-right-check
functions against an independent numpy restatement of the reference kernels
(stereo/stereo.cu:306-346, 471-520, 803-817, 853-863, 913-942, 1090-1095)
on small cases.  The reference ships no test vectors for these paths, so this
is the pin: two restatements written separately must agree."""
import numpy as np

f32 = np.float32


def _lerp_row(r, u):
    """Clamp-addressed linear read at texture coordinate u, FP32 lerp."""
    W = len(r)
    t = f32(f32(u) - f32(0.5))
    i = int(np.floor(t))
    a = f32(t - f32(np.floor(t)))
    v0 = r[min(max(i, 0), W - 1)]
    if a == 0:
        return v0
    v1 = r[min(max(i + 1, 0), W - 1)]
    return f32(v0 + f32(a * f32(v1 - v0)))


def _census_np(g1, g2, fs, lst, lam):
    H, W = g1.shape
    out = np.zeros((H, W, len(lst)), np.float32)
    norm = f32(fs * fs * 4)
    for y in range(H):
        for x in range(W):
            c1 = g1[y, x]
            for z, d in enumerate(lst):
                c2 = _lerp_row(g2[y], f32(f32(x + 0.5) - d))
                cnt = 0
                for dy in range(-fs, fs + 1):
                    yy = min(max(y + dy, 0), H - 1)
                    for dx in range(-fs, fs + 1):
                        if dx == 0 and dy == 0:
                            continue
                        i1 = g1[yy, min(max(x + dx, 0), W - 1)]
                        i2 = _lerp_row(g2[yy], f32(f32(x + dx + 0.5) - d))
                        cnt += (c1 > i1) != (c2 > i2)
                out[y, x, z] = f32(f32(lam) * f32(f32(cnt) / norm))
    return out


def test_gray(oracle):
    rgba = np.random.default_rng(0).random((5, 7, 4)).astype(np.float32)
    c = rgba.astype(np.float64)  # the reference's double constants promote every term
    want = 0.2989 * c[..., 0] + 0.5870 * c[..., 1] + 0.1140 * c[..., 2]
    assert np.array_equal(oracle.gray(rgba), want.astype(np.float32))


def test_census_matches_restatement(oracle):
    rng = np.random.default_rng(1)
    g1 = np.round(rng.random((6, 11)) * 8).astype(np.float32) / 8  # ties exercise the strict comparison
    g2 = np.round(rng.random((6, 11)) * 8).astype(np.float32) / 8
    for fs, dmin, dstep, D in ((1, 0.0, 1.0, 4), (2, 0.5, 0.5, 5), (2, -3.0, 1.0, 4)):
        lst = oracle.census_list(dmin, dstep, D)
        assert np.array_equal(oracle.census(g1, g2, fs, lst, 0.9), _census_np(g1, g2, fs, lst, 0.9))


def test_census_list_is_float_accumulation(oracle):
    lst = oracle.census_list(0.1, 0.1, 30)
    d, want = f32(0.1), []
    for _ in range(30):
        want.append(d)
        d = f32(d + f32(0.1))
    assert np.array_equal(lst, np.array(want, np.float32))


def test_edge_weights_matches_restatement(oracle):
    rng = np.random.default_rng(2)
    g = rng.random((9, 13)).astype(np.float32)
    g[:, 6:] += 1.0
    sigma, R = 0.7, 3
    k = np.exp(-np.arange(-R, R + 1) ** 2 / (2 * sigma * sigma))
    k /= k.sum()
    gp = np.pad(g.astype(np.float64), R, mode="edge")
    sm = np.zeros_like(gp)
    for i in range(-R, R + 1):
        sm[:, R:-R] += k[i + R] * np.roll(gp, -i, axis=1)[:, R:-R]
    t = np.zeros_like(gp)
    for i in range(-R, R + 1):
        t[R:-R] += k[i + R] * np.roll(sm, -i, axis=0)[R:-R]
    t = t[R:-R, R:-R]
    dx = np.abs(np.diff(t, axis=1, append=t[:, -1:]))
    dy = np.abs(np.diff(t, axis=0, append=t[-1:, :]))
    for alpha, beta, lam in ((20.0, 0.8, 0.4), (0.0, 0.8, 0.5), (5.0, 2.0, 1.5)):
        wx, wy = oracle.edge_weights(g, alpha, beta, lam)
        if alpha > 0:
            ex = np.maximum(lam * np.exp(-alpha * dx ** beta), 1e-6)
            ey = np.maximum(lam * np.exp(-alpha * dy ** beta), 1e-6)
        else:
            ex, ey = lam * dx, lam * dy
        np.testing.assert_allclose(wx, ex, rtol=2e-5, atol=1e-7)
        np.testing.assert_allclose(wy, ey, rtol=2e-5, atol=1e-7)
        assert np.all(wx[:, -1] == (lam if alpha > 0 else 0.0))  # last column: zero difference


def test_quadfit_direct_matches_restatement(oracle):
    rng = np.random.default_rng(3)
    H, W, D = 4, 9, 7
    dmin, dstep = f32(0.5), f32(0.5)
    lab = rng.integers(0, D, (H, W)).astype(np.int32)
    u = oracle.remap(lab, dmin, dstep)
    c1 = rng.standard_normal((H, W, D)).astype(np.float32)
    want = u.copy()
    for y in range(H):
        for x in range(W):
            z = int(f32(f32(u[y, x] - dmin) / dstep))
            if z <= 0 or z >= D - 1:
                continue
            c = c1[y, x]
            a = f32(f32(c[z - 1] - c[z + 1]) / f32(dstep * f32(2)))
            b = max(f32(1e-3), f32(f32(f32(c[z - 1] + c[z + 1]) - f32(f32(2) * c[z])) / f32(dstep * dstep)))
            want[y, x] = f32(u[y, x] + f32(a / b))
    assert np.array_equal(oracle.quadfit_direct(u, c1, dmin, dstep), want)


def test_lr_check_matches_restatement(oracle):
    rng = np.random.default_rng(4)
    H, W = 5, 17
    left = (rng.random((H, W)) * 6).astype(np.float32)
    right = -(left + rng.standard_normal((H, W)).astype(np.float32))
    want = np.empty_like(left)
    for y in range(H):
        for x in range(W):
            d = left[y, x]
            dr = -_lerp_row(right[y], f32(f32(x + 0.5) - d))
            want[y, x] = d if abs(f32(d - dr)) <= f32(1.0) else f32(-1)
    assert np.array_equal(oracle.lr_check(left, right, 1.0), want)
