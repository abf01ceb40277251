"""The TIFF reader (wc_tiff_info / wc_tiff_read): the reference's own test images
(uncompressed and LZW, big-endian) decode to the pixel values the reference
library reads, and small little-endian / PackBits / predictor / 8-bit files
written here round-trip.  Host code only: no GPU needed."""
import struct

import numpy as np
import pytest

from conftest import golden
import synth_loader  # noqa: F401
import wndcharm


@pytest.mark.parametrize("key", ["t1_s01_c05_ij", "010067_301x300", "binuc1", "norm1"])
def test_reference_tiffs(tmp_path, key):
    data = golden("reference_tiff.npz")[key]
    p = tmp_path / (key + ".tif")
    p.write_bytes(data.tobytes())
    pix, bits = wndcharm.read_tiff(str(p))
    assert bits == 16 and pix.dtype == np.uint16
    np.testing.assert_array_equal(pix, golden("reference_images.npz")["img_" + key])
    im = wndcharm.ImageMatrix()
    assert im.OpenImage(str(p)) == 1 and im.bits == 16
    assert im.OpenImage(str(p), bounding_rect=(3, 5, 20, 10)) == 1
    np.testing.assert_array_equal(im.pix_plane, pix[5:15, 3:23])


def _packbits(row):
    out = bytearray()
    i = 0
    while i < len(row):
        j = i
        while j + 1 < len(row) and row[j + 1] == row[i] and j - i < 127:
            j += 1
        if j > i:  # run
            out += struct.pack("b", -(j - i)) + row[i:i + 1]
            i = j + 1
        else:
            k = i
            while k < len(row) and k - i < 128 and not (k + 1 < len(row) and row[k + 1] == row[k]):
                k += 1
            k = max(k, i + 1)
            out += struct.pack("b", k - i - 1) + row[i:k]
            i = k
    return bytes(out)


def _write_tiff(path, a, compression=1, predictor=1, order="<"):
    h, w = a.shape[:2]
    spp = 1 if a.ndim == 2 else a.shape[2]
    bps = 8 * a.dtype.itemsize
    if predictor == 2:  # each sample minus the same sample of the pixel to its left
        d = a.astype(np.int64)
        d[:, 1:] = d[:, 1:] - d[:, :-1]
        a = (d % (1 << bps)).astype(a.dtype)
    rows = [a[y].astype(a.dtype.newbyteorder(order)).tobytes() for y in range(h)]
    strips = [b"".join(rows[y:y + 3]) for y in range(0, h, 3)]  # 3 rows per strip
    if compression == 32773:
        strips = [b"".join(_packbits(r) for r in rows[y:y + 3]) for y in range(0, h, 3)]
    entries = [(256, 3, 1, w), (257, 3, 1, h), (258, 3, spp, bps), (259, 3, 1, compression),
               (262, 3, 1, 1 if spp == 1 else 2), (273, 4, len(strips), None), (277, 3, 1, spp), (278, 3, 1, 3),
               (279, 4, len(strips), None), (284, 3, 1, 1), (317, 3, 1, predictor)]
    head = 8
    data = b"".join(strips)
    offs, o = [], head
    for s_ in strips:
        offs.append(o)
        o += len(s_)
    arrays = head + len(data)
    bps_at = arrays + 8 * len(strips)  # BitsPerSample per sample (6 bytes for 3 samples: stored out of line)
    ifd = bps_at + 8
    out = bytearray((b"II" if order == "<" else b"MM") + struct.pack(order + "HI", 42, ifd))
    out += data
    out += struct.pack(order + "%dI" % len(strips), *offs)
    out += struct.pack(order + "%dI" % len(strips), *[len(s_) for s_ in strips])
    out += struct.pack(order + "4H", bps, bps, bps, 0)
    out += struct.pack(order + "H", len(entries))
    for tag, typ, cnt, val in entries:
        if tag == 273:
            out += struct.pack(order + "HHII", tag, typ, cnt, arrays)
        elif tag == 279:
            out += struct.pack(order + "HHII", tag, typ, cnt, arrays + 4 * len(strips))
        elif tag == 258 and spp > 2:
            out += struct.pack(order + "HHII", tag, typ, cnt, bps_at)
        else:
            out += struct.pack(order + "HHIHH", tag, typ, cnt, val, 0)
    out += struct.pack(order + "I", 0)
    path.write_bytes(bytes(out))


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
@pytest.mark.parametrize("compression,predictor,order", [(1, 1, "<"), (1, 1, ">"), (32773, 1, "<"), (1, 2, ">")])
def test_written_tiffs(tmp_path, dtype, compression, predictor, order):
    rng = np.random.default_rng(1)
    a = rng.integers(0, np.iinfo(dtype).max, size=(11, 13)).astype(dtype)
    a[4, 2:9] = 7  # a run for PackBits
    p = tmp_path / "x.tif"
    _write_tiff(p, a, compression, predictor, order)
    pix, bits = wndcharm.read_tiff(str(p))
    assert bits == 8 * a.dtype.itemsize
    np.testing.assert_array_equal(pix, a)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
@pytest.mark.parametrize("compression,predictor,order", [(1, 1, "<"), (32773, 1, ">"), (1, 2, "<")])
def test_written_rgb_tiffs(tmp_path, dtype, compression, predictor, order):
    rng = np.random.default_rng(2)
    a = rng.integers(0, np.iinfo(dtype).max, size=(9, 14, 3)).astype(dtype)
    a[3, 1:12] = a[3, 1]  # a run of one colour
    p = tmp_path / "rgb.tif"
    _write_tiff(p, a, compression, predictor, order)
    pix, bits = wndcharm.read_tiff(str(p))
    assert bits == 8 * a.dtype.itemsize and pix.shape == (9, 14, 3)
    np.testing.assert_array_equal(pix, a)
    im = wndcharm.ImageMatrix()
    assert im.OpenImage(str(p), bounding_rect=(2, 1, 5, 6)) == 1
    np.testing.assert_array_equal(im.pix_plane, a[1:7, 2:7])


def test_tiff_errors(tmp_path):
    p = tmp_path / "bad.tif"
    p.write_bytes(b"not a tiff at all")
    with pytest.raises(wndcharm.WndcharmError):
        wndcharm.read_tiff(str(p))
    with pytest.raises(wndcharm.WndcharmError):
        wndcharm.read_tiff(str(tmp_path / "missing.tif"))
    assert wndcharm.ImageMatrix().OpenImage(str(tmp_path / "x.png")) == 0


@pytest.mark.parametrize("compression", [1, 32773])
def test_truncated_tiffs_are_io_errors(tmp_path, compression):
    """A TIFF cut short anywhere (header, directory, strips) is WC_ERR_IO, never a crash."""
    rng = np.random.default_rng(4)
    a = rng.integers(0, 4096, size=(20, 17)).astype(np.uint16)
    full = tmp_path / "full.tif"
    _write_tiff(full, a, compression, 1, "<")
    raw = full.read_bytes()
    np.testing.assert_array_equal(wndcharm.read_tiff(str(full))[0], a)
    for cut in sorted({4, 8, 12, len(raw) // 3, len(raw) // 2, len(raw) - 7, len(raw) - 1}):
        p = tmp_path / ("cut%d.tif" % cut)
        p.write_bytes(raw[:cut])
        with pytest.raises(wndcharm.WndcharmError):
            wndcharm.read_tiff(str(p))
