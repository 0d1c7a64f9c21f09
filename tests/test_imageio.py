"""CPU tests of stereo_img's file formats (cnncrf.imageio), option handling
(cnncrf.cli) and the evaluation metrics (cnncrf.evaluation): PNG decoding of
every row filter type at 8 and 16 bits, the KITTI 16-bit disparity encoding,
PFM row order, the command line of the CLI (reference flags, config-file
precedence, the extra options), the KITTI error and the Middlebury bad-x
weighting."""
import struct
import zlib

import numpy as np


def _png_with_filters(img, depth):
    """Encode (H, W, C) unsigned data cycling the row filters 0..4 (ISO/IEC 15948 6.3)."""
    h, w, c = img.shape
    bpp = c * depth // 8
    rows = img.astype(">u2" if depth == 16 else "u1").reshape(h, -1).view(np.uint8).astype(np.int32)
    prev = np.zeros(rows.shape[1], np.int32)
    out = b""
    for y in range(h):
        ft = y % 5
        cur = rows[y]
        left = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        upleft = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        if ft == 0:
            f = cur
        elif ft == 1:
            f = cur - left
        elif ft == 2:
            f = cur - prev
        elif ft == 3:
            f = cur - ((left + prev) >> 1)
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            f = cur - pred
        out += bytes([ft]) + (f & 255).astype(np.uint8).tobytes()
        prev = cur
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[c]

    def chunk(t, b):
        return struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xFFFFFFFF)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(out)) + chunk(b"IEND", b""))


def test_png_decoder_all_filters(tmp_path):
    from cnncrf import imageio
    rng = np.random.default_rng(0)
    for depth, c in ((8, 3), (8, 4), (8, 1), (16, 1), (16, 3)):
        img = rng.integers(0, 1 << depth, (11, 13, c))
        p = tmp_path / ("f%d_%d.png" % (depth, c))
        p.write_bytes(_png_with_filters(img, depth))
        got = imageio.read_png(str(p))
        ref = img.astype(np.float32) / float((1 << depth) - 1)
        if c == 1:
            for ch in range(3):
                assert np.array_equal(got[..., ch], ref[..., 0])
        else:
            assert np.array_equal(got[..., :3], ref[..., :3])
        if c == 4:
            assert np.array_equal(got[..., 3], ref[..., 3])
        else:
            assert np.all(got[..., 3] == 1.0)


def test_png_writer_round_trip(tmp_path):
    from cnncrf import imageio
    rng = np.random.default_rng(1)
    rgb = rng.integers(0, 256, (7, 9, 3))
    imageio.write_png(str(tmp_path / "a.png"), rgb)
    assert np.array_equal(imageio.read_png(str(tmp_path / "a.png"))[..., :3], rgb.astype(np.float32) / 255.0)


def test_png16_disparity_encoding(tmp_path):
    from cnncrf import imageio
    d = np.array([[-3.0, 0.0, 1.0 / 256 - 1e-4, 1.5], [255.99, 300.0, 12.34, 0.001]], np.float32)
    enc = imageio.disparity_to_png16(d)
    assert enc.tolist() == [[0, 0, 0, 384], [65533, 65535, 3159, 0]]  # (uint16)max(d*256, 0), saturated
    imageio.write_png16(str(tmp_path / "d.png"), d)
    back = imageio.read_png(str(tmp_path / "d.png"))[..., 0] * 65535.0
    assert np.array_equal(np.rint(back).astype(np.uint16), enc)


def test_pfm_rows_bottom_up(tmp_path):
    from cnncrf import imageio
    a = np.arange(12, dtype=np.float32).reshape(3, 4)
    p = tmp_path / "x.pfm"
    imageio.write_pfm(str(p), a)
    raw = p.read_bytes()
    head = b"Pf\n4 3\n-1.0\n"
    assert raw.startswith(head)
    first_row = np.frombuffer(raw[len(head):len(head) + 16], "<f4")
    assert np.array_equal(first_row, a[2])  # the file starts with the bottom row
    assert np.array_equal(imageio.read_pfm(str(p)), a)


def test_cli_option_split_and_precedence():
    from cnncrf import cli, config
    rest, extra = cli._split_extras(["l.png", "r.png", "--precision", "BF16", "--L1", "2", "--xavier-seed=5"])
    assert rest == ["l.png", "r.png", "--L1", "2"]
    assert extra == {"precision": "BF16", "xavier-seed": 5}
    o = config.resolve(rest, cfg_text="L1 = 7\nL2 = 9\nmatching = COLORPAIR\n")
    assert (o["im0"], o["im1"], o["L1"], o["L2"], o["matching"]) == ("l.png", "r.png", 2.0, 9.0, "COLORPAIR")
    assert o["crf-iterations"] == 4 and o["refinement"] == "NONE"  # reference defaults


def test_kitti_error_definition():
    """computeError: invalid ground truth (<= 0) is ignored, a pixel is wrong
    only past both 3 px and 5 % of the ground truth."""
    from cnncrf import evaluation as E
    gt = np.array([[-1.0, 10.0, 100.0, 50.0], [20.0, 2.0, -1.0, 80.0]])
    pred = np.array([[5.0, 13.5, 104.0, 57.0], [20.0, 9.0, 0.0, 83.9]])
    # valid: 6; wrong: 13.5 (3.5 > 3, 35 %), 57 (7, 14 %), 9 (7, 350 %); 104 is 4 % -> right; 83.9 is 3.9 px, 4.9 %
    assert E.kitti_error(pred, gt) == 3 / 6
    assert np.isnan(E.kitti_error(pred, -np.ones_like(gt)))


def test_disp16_round_trip_and_kitti_numbers(tmp_path):
    from cnncrf import evaluation as E, imageio
    rng = np.random.default_rng(7)
    for d in ("pred", "occ", "noc"):
        (tmp_path / d).mkdir()
    errs_occ, errs_noc = [], []
    for k in range(3):
        gt = (rng.random((6, 9)) * 60).astype(np.float32)
        gt[0, :4] = 0.0  # no ground truth
        pred = gt + rng.standard_normal(gt.shape).astype(np.float32) * 6
        noc = gt.copy()
        noc[1] = 0.0
        imageio.write_png16(str(tmp_path / "pred" / ("%06d_10.png" % k)), pred)
        imageio.write_png16(str(tmp_path / "occ" / ("%06d_10.png" % k)), gt)
        imageio.write_png16(str(tmp_path / "noc" / ("%06d_10.png" % k)), noc)
        assert np.array_equal(E.read_disp16(str(tmp_path / "pred" / ("%06d_10.png" % k))), E.quantize_png16(pred))
        errs_occ.append(E.kitti_error(E.quantize_png16(pred), E.quantize_png16(gt)))
        errs_noc.append(E.kitti_error(E.quantize_png16(pred), E.quantize_png16(noc)))
    occ, noc = E.kitti_numbers(str(tmp_path / "pred"), str(tmp_path / "occ"), str(tmp_path / "noc"))
    assert occ == np.mean(errs_occ) and noc == np.mean(errs_noc)
    assert E.main(["kitti", str(tmp_path / "pred"), str(tmp_path / "occ"), str(tmp_path / "noc")]) == 0


def test_middlebury_bad_and_weights():
    from cnncrf import evaluation as E
    gt = np.array([[1.0, np.inf, 10.0], [4.0, 5.0, 6.0]])
    pred = np.array([[1.5, 0.0, 15.0], [np.nan, 5.0, 8.1]])
    # finite gt: 5; bad at threshold 2: 15 vs 10, nan, 8.1 vs 6 -> 3
    assert E.middlebury_bad(pred, gt, 2.0) == 60.0
    assert E.middlebury_bad(pred, gt, 2.0, mask=[[1, 1, 0], [1, 1, 1]]) == 50.0
    badx = np.arange(15, dtype=np.float64)
    mean, weighted = E.middlebury_weighted(badx)
    w = E.MIDDLEBURY_TRAINING_WEIGHTS
    assert mean == 7.0 and weighted == (w * badx).sum() / w.sum()
