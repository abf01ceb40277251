"""TIFF strips decoded on the GPU (wc_tiff_read_device): every layout the
host reader takes -- uncompressed and PackBits strips, both byte orders, the
horizontal predictor, 8 and 16 bits, grayscale and RGB, and the reference's
own LZW test images -- decodes to the host reader's samples bit for bit, in
one call for all files; the features of the device-decoded images equal those
of the host-read arrays; damaged files are WC_ERR_IO."""
import struct

import numpy as np
import pytest

from conftest import golden
from test_tiff import _write_tiff
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


def _device_images(eng, paths):
    buf, descs = eng.read_tiffs_device([str(p) for p in paths])
    host = buf.cpu().numpy()
    base = buf.data_ptr()
    out = []
    for d in descs:
        es = 1 if d.dtype in (0, 4) else 2
        spp = 3 if d.dtype in (4, 5) else 1
        off = d.pixels - base
        assert off % 256 == 0 and d.on_device == 1
        a = host[off:off + d.width * d.height * spp * es].view(np.uint8 if es == 1 else np.uint16)
        out.append(a.reshape((d.height, d.width) + ((3,) if spp == 3 else ())))
    return out, descs


def _files(tmp_path):
    rng = np.random.default_rng(21)
    files = []
    k = 0
    for dtype in (np.uint8, np.uint16):
        for comp, pred, order in [(1, 1, "<"), (1, 1, ">"), (32773, 1, "<"), (32773, 1, ">"), (1, 2, ">"),
                                  (32773, 2, "<")]:
            for shape in [(37, 29), (8, 61, 3)]:
                a = rng.integers(0, np.iinfo(dtype).max, size=shape).astype(dtype)
                a[min(4, shape[0] - 1), 2:20] = a[0, 0]  # runs for PackBits
                p = tmp_path / ("f%d.tif" % k)
                _write_tiff(p, a, comp, pred, order)
                files.append((p, a))
                k += 1
    for key in ["t1_s01_c05_ij", "010067_301x300"]:  # the reference's LZW, big-endian files
        p = tmp_path / (key + ".tif")
        p.write_bytes(golden("reference_tiff.npz")[key].tobytes())
        files.append((p, golden("reference_images.npz")["img_" + key]))
    return files


def test_device_decode_equals_host_reader(tmp_path):
    import wndcharm
    files = _files(tmp_path)
    eng = wndcharm.Engine(0, "fp64")
    got, descs = _device_images(eng, [p for p, _ in files])
    for (p, a), g, d in zip(files, got, descs):
        host, bits = wndcharm.read_tiff(str(p))
        np.testing.assert_array_equal(g, host)
        np.testing.assert_array_equal(g, a)
        assert d.bits == bits


def test_features_of_device_decoded_files(tmp_path):
    import wndcharm
    files = _files(tmp_path)
    gray = [(p, a) for p, a in files if a.ndim == 2]
    eng = wndcharm.Engine(0, "mixed")
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSet()
    rows = eng.extract_tiffs(plan, [p for p, _ in gray])
    for (p, _), r in zip(gray, rows):
        host, bits = wndcharm.read_tiff(str(p))
        np.testing.assert_array_equal(r, eng.extract(plan, [host], bits=bits)[0])
    s = wndcharm.Sampling(tiles_x=2, tiles_y=2)
    big = [p for p, a in gray if a.shape[0] >= 32]
    rs = eng.extract_tiffs(plan, big, sampling=s)
    host = [wndcharm.read_tiff(str(p))[0] for p in big]
    np.testing.assert_array_equal(rs, eng.extract_samples(plan, host, s))


def test_damaged_files_are_io_errors(tmp_path):
    import wndcharm
    rng = np.random.default_rng(5)
    a = rng.integers(0, 4096, size=(20, 17)).astype(np.uint16)
    eng = wndcharm.Engine(0, "fp64")
    for comp in (1, 32773):
        full = tmp_path / ("full%d.tif" % comp)
        _write_tiff(full, a, comp, 1, "<")
        raw = full.read_bytes()
        for cut in (12, len(raw) // 2, len(raw) - 7):
            p = tmp_path / ("cut%d_%d.tif" % (comp, cut))
            p.write_bytes(raw[:cut])
            with pytest.raises(wndcharm.WndcharmError):
                eng.read_tiffs_device([str(full), str(p)])
    # a PackBits strip whose stored byte count is cut short: found short on the GPU
    p = tmp_path / "pb.tif"
    _write_tiff(p, a, 32773, 1, "<")
    b = bytearray(p.read_bytes())
    ifd = struct.unpack_from("<I", b, 4)[0]
    for k in range(struct.unpack_from("<H", b, ifd)[0]):
        tag, typ, cnt, at = struct.unpack_from("<HHII", b, ifd + 2 + 12 * k)
        if tag == 279:
            first = struct.unpack_from("<I", b, at)[0]
            struct.pack_into("<I", b, at, first - 3)
    p.write_bytes(bytes(b))
    with pytest.raises(wndcharm.WndcharmError, match="too short"):
        wndcharm.read_tiff(str(p))
    with pytest.raises(wndcharm.WndcharmError, match="too short"):
        eng.read_tiffs_device([str(p)])
    # the engine still works
    got, _ = _device_images(eng, [full])
    np.testing.assert_array_equal(got[0], a)
