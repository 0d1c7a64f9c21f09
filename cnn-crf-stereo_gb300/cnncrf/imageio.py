"""Image and result files of stereo_img, without OpenCV / png++ / cnpy:

  read_png     8- or 16-bit grey, grey+alpha, RGB or RGBA PNG (non-interlaced)
               -> RGBA float32 in [0, 1], the iu::ImageCpu_32f_C4 stereo_img reads
  write_png16  disparity map as 16-bit grey PNG, value = (uint16)max(d * 256, 0),
               the KITTI format saveMat writes (stereo/tools.cpp:37-43); values past
               65535 saturate
  write_pfm / read_pfm   little-endian float PFM, "Pf", scale -1.0, rows bottom-up
               (stereo/tools.cpp:47-60)
  write_npy    numpy .npy (cnpy::npy_save in stereo/tools.cpp:86-93)

PNG is decoded and encoded here with zlib and the five PNG row filters
(ISO/IEC 15948), written from the specification.
"""
import struct
import zlib

import numpy as np

_SIG = b"\x89PNG\r\n\x1a\n"


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _unfilter(raw, h, stride, bpp):
    out = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(h):
        ft = raw[pos]
        line = np.frombuffer(raw, np.uint8, stride, pos + 1).astype(np.int32)
        pos += 1 + stride
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 255
        elif ft in (1, 3, 4):
            cur = np.zeros(stride, np.int32)
            for x in range(stride):  # depends on the byte bpp to the left: sequential
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                if ft == 1:
                    v = line[x] + a
                elif ft == 3:
                    v = line[x] + ((a + b) >> 1)
                else:
                    c = prev[x - bpp] if x >= bpp else 0
                    v = line[x] + int(_paeth(np.int32(a), np.int32(b), np.int32(c)))
                cur[x] = v & 255
        else:
            raise ValueError("PNG: unknown filter type %d" % ft)
        out[y] = cur
        prev = cur
    return out


def read_png(path):
    data = open(path, "rb").read()
    if data[:8] != _SIG:
        raise ValueError("%s: not a PNG file" % path)
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif typ == b"IDAT":
            idat.append(body)
        elif typ == b"IEND":
            break
        pos += 12 + n
    if hdr is None:
        raise ValueError("%s: no IHDR" % path)
    w, h, depth, ctype, _, _, interlace = hdr
    chans = {0: 1, 2: 3, 4: 2, 6: 4}.get(ctype)
    if chans is None or depth not in (8, 16) or interlace:
        raise ValueError("%s: unsupported PNG (colour type %d, depth %d, interlace %d)" % (path, ctype, depth, interlace))
    bps = depth // 8
    raw = zlib.decompress(b"".join(idat))
    rows = _unfilter(raw, h, w * chans * bps, chans * bps).astype(np.uint32)
    if bps == 2:
        rows = (rows[:, 0::2] << 8) | rows[:, 1::2]
    img = rows.reshape(h, w, chans).astype(np.float32) / float((1 << depth) - 1)
    rgba = np.ones((h, w, 4), np.float32)
    if chans in (1, 2):
        rgba[..., :3] = img[..., :1]
        if chans == 2:
            rgba[..., 3] = img[..., 1]
    else:
        rgba[..., :3] = img[..., :3]
        if chans == 4:
            rgba[..., 3] = img[..., 3]
    return rgba


def _chunk(typ, body):
    return struct.pack(">I", len(body)) + typ + body + struct.pack(">I", zlib.crc32(typ + body) & 0xFFFFFFFF)


def write_png(path, img, depth=8):
    """Grey (H, W) or RGB / RGBA (H, W, 3|4) unsigned integer image, filter 0."""
    a = np.asarray(img)
    if a.ndim == 2:
        a = a[..., None]
    h, w, c = a.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[c]
    dt = ">u2" if depth == 16 else "u1"
    rows = a.astype(dt).reshape(h, w * c)
    raw = b"".join(b"\x00" + rows[y].tobytes() for y in range(h))
    with open(path, "wb") as f:
        f.write(_SIG + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)) +
                _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b""))


def disparity_to_png16(disp):
    """(uint16)max(d * 256, 0) of saveMat (stereo/tools.cpp:40), saturated at 65535."""
    v = np.maximum(np.asarray(disp, np.float64) * 256.0, 0.0)
    return np.minimum(np.floor(v), 65535).astype(np.uint16)


def write_png16(path, disp):
    write_png(path, disparity_to_png16(disp), depth=16)


def write_pfm(path, a):
    a = np.asarray(a, np.float32)
    h, w = a.shape
    with open(path, "wb") as f:
        f.write(b"Pf\n%d %d\n-1.0\n" % (w, h))
        f.write(np.ascontiguousarray(a[::-1]).astype("<f4").tobytes())


def read_pfm(path):
    with open(path, "rb") as f:
        if f.readline().strip() != b"Pf":
            raise ValueError("%s: not a one-channel PFM" % path)
        w, h = (int(t) for t in f.readline().split())
        scale = float(f.readline())
        data = np.frombuffer(f.read(4 * w * h), "<f4" if scale < 0 else ">f4")
    return data.reshape(h, w)[::-1].astype(np.float32)


def write_npy(path, a):
    np.save(path, np.ascontiguousarray(a))
