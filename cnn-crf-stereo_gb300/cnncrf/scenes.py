"""Seeded synthetic stereo scenes with ground truth (stand-ins for KITTI 2015
and Middlebury 2014, which are not available here).

Texture: uint8 band-limited noise (white noise smoothed by a separable
Gaussian, sigma 1.2 px, rescaled to 0..255) with 5% random dots (0 or 255).
The right image is the left forward-warped by the left disparity (nearest
target column, nearer surfaces win); columns nothing maps to are occlusions
and get fresh texture; then Gaussian noise of sigma 2 grey levels is added to
both views.  Images are returned as RGBA float32 in [0, 1] (alpha = 1), the
iu::imread_32f_C4 convention of the reference.

  voronoi : N seeds, each Voronoi cell a plane offset + sx (x - cx) + sy (y - cy)
  kitti   : ground plane 0 -> dmax_ground from the top row to the bottom row,
            plus fronto-parallel boxes drawn far to near
"""
import numpy as np


def _gauss_kernel(sigma):
    r = max(1, int(np.ceil(3 * sigma)))
    x = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (x / sigma) ** 2)
    return k / k.sum()


def _blur(img, sigma):
    k = _gauss_kernel(sigma)
    r = len(k) // 2
    p = np.pad(img, ((r, r), (r, r)), mode="reflect")
    t = sum(k[i] * p[:, i:i + img.shape[1]] for i in range(len(k)))
    return sum(k[i] * t[i:i + img.shape[0], :] for i in range(len(k)))


def texture(rng, H, W, channels=3):
    out = np.empty((H, W, channels), np.float64)
    for c in range(channels):
        t = _blur(rng.standard_normal((H, W)), 1.2)
        t = (t - t.min()) / max(t.max() - t.min(), 1e-12) * 255.0
        dots = rng.random((H, W)) < 0.05
        t[dots] = np.where(rng.random(dots.sum()) < 0.5, 0.0, 255.0)
        out[..., c] = t
    return np.round(out).astype(np.uint8)


def _render(rng, disp, channels, noise_sigma=2.0):
    H, W = disp.shape
    left = texture(rng, H, W, channels).astype(np.float64)
    right = texture(rng, H, W, channels).astype(np.float64)  # fresh texture for occlusions
    ys, xs = np.mgrid[0:H, 0:W]
    xr = np.rint(xs - disp).astype(np.int64)
    ok = (xr >= 0) & (xr < W)
    order = np.argsort(disp[ok], kind="stable")  # far first, near last wins
    yy, xx, tx = ys[ok][order], xs[ok][order], xr[ok][order]
    right[yy, tx] = left[yy, xx]
    left = left + rng.normal(0.0, noise_sigma, left.shape)
    right = right + rng.normal(0.0, noise_sigma, right.shape)
    left = np.clip(left, 0, 255)
    right = np.clip(right, 0, 255)

    def rgba(img):
        if channels == 1:
            img = np.repeat(img, 3, axis=2)
        a = np.ones(img.shape[:2] + (4,), np.float32)
        a[..., :3] = (img / 255.0).astype(np.float32)
        return a

    return rgba(left), rgba(right)


def voronoi_scene(W, H, D, seed, cells=12, off_range=(2.0, 28.0), slope=0.1, channels=3):
    rng = np.random.default_rng(seed)
    cx = rng.uniform(0, W, cells)
    cy = rng.uniform(0, H, cells)
    off = rng.uniform(off_range[0], off_range[1], cells)
    sx = rng.uniform(-slope, slope, cells)
    sy = rng.uniform(-slope, slope, cells)
    ys, xs = np.mgrid[0:H, 0:W].astype(np.float64)
    d2 = (xs[None] - cx[:, None, None]) ** 2 + (ys[None] - cy[:, None, None]) ** 2
    lab = np.argmin(d2, axis=0)
    disp = off[lab] + sx[lab] * (xs - cx[lab]) + sy[lab] * (ys - cy[lab])
    disp = np.clip(disp, 0.0, D - 1.0)
    left, right = _render(rng, disp, channels)
    return dict(left=left, right=right, disp=disp.astype(np.float32), W=W, H=H, D=D)


def kitti_scene(W, H, D, seed, boxes=15, ground_max=110.0, box_range=(10.0, 120.0), channels=3):
    rng = np.random.default_rng(seed)
    ys, xs = np.mgrid[0:H, 0:W].astype(np.float64)
    disp = ground_max * ys / max(H - 1, 1)
    bd = np.sort(rng.uniform(box_range[0], box_range[1], boxes))
    for d in bd:  # far to near: nearer boxes occlude
        bw = rng.integers(max(8, W // 30), max(9, W // 5))
        bh = rng.integers(max(6, H // 12), max(7, H // 2.5))
        x0 = rng.integers(0, max(1, W - bw))
        y0 = rng.integers(0, max(1, H - bh))
        disp[y0:y0 + bh, x0:x0 + bw] = d
    disp = np.clip(disp, 0.0, D - 1.0)
    left, right = _render(rng, disp, channels)
    return dict(left=left, right=right, disp=disp.astype(np.float32), W=W, H=H, D=D)


# the named workloads (sizes, disparity ranges, generators)
def workload(name, seed=0):
    if name == "gray256x192_d32":
        return voronoi_scene(256, 192, 32, seed, cells=12, off_range=(2, 28), slope=0.1, channels=1)
    if name == "mbq720x480_d96":
        return voronoi_scene(720, 480, 96, seed, cells=30, off_range=(4, 90), slope=0.2)
    if name == "kitti1242x375_d128":
        return kitti_scene(1242, 375, 128, seed)
    if name == "crop512x256_d128":
        return kitti_scene(512, 256, 128, seed)
    raise KeyError(name)


# the uneven batch: 8 pairs of each (W, H, D), each from the Middlebury-shaped
# generator (30 planar cells, offsets in [4, 90] clipped to D - 1, slopes
# +-0.2) with its own seed
UNEVEN_SHAPES = [(480, 320, 64), (720, 480, 96), (1242, 375, 128), (1440, 960, 192)]


def uneven_scenes(per_shape=8, seed0=0, shapes=None):
    out = []
    for j, (W, H, D) in enumerate(shapes or UNEVEN_SHAPES):
        for i in range(per_shape):
            out.append(voronoi_scene(W, H, D, seed0 + 100 * j + i, cells=30, off_range=(4, 90), slope=0.2))
    return out


def bad_pixels(disp, gt, thresh=3.0, rel=0.05):
    """KITTI error rate of a disparity map against a synthetic ground truth,
    both read as 16-bit PNGs would be (eval/compute_numbers_kitti.py:6-17)."""
    from .evaluation import kitti_error, quantize_png16
    return kitti_error(quantize_png16(disp), quantize_png16(gt), (thresh, rel))
