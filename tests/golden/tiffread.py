"""Minimal baseline-TIFF decoder for the reference's grayscale test images.

Covers what ImageMatrix::LoadTIFF (src/cmatrix.cpp:85-203) is fed by the
reference's fixtures: one image directory, one sample per pixel, 8- or 16-bit,
uncompressed (1) or LZW (5) strips, either byte order, optional horizontal
predictor (2).  Returns a numpy array of shape (height, width).
"""
import struct

import numpy as np


def _lzw_decode(data):
    # TIFF LZW: MSB-first codes, 9..12 bits, ClearCode 256, EOI 257, "early change".
    out = bytearray()
    table = [bytes([i]) for i in range(256)] + [b"", b""]
    nbits, bitbuf, bitcnt, pos = 9, 0, 0, 0
    prev = None
    n = len(data)
    while True:
        while bitcnt < nbits and pos < n:
            bitbuf = (bitbuf << 8) | data[pos]
            pos += 1
            bitcnt += 8
        if bitcnt < nbits:
            break
        code = (bitbuf >> (bitcnt - nbits)) & ((1 << nbits) - 1)
        bitcnt -= nbits
        if code == 257:
            break
        if code == 256:
            table = table[:258]
            nbits = 9
            prev = None
            continue
        if prev is None:
            entry = table[code]
            out += entry
            prev = entry
            continue
        if code < len(table):
            entry = table[code]
            table.append(prev + entry[:1])
        else:
            entry = prev + prev[:1]
            table.append(entry)
        out += entry
        prev = entry
        if len(table) + 1 >= (1 << nbits) and nbits < 12:
            nbits += 1
    return bytes(out)


def read_tiff(path):
    with open(path, "rb") as fh:
        buf = fh.read()
    bo = {b"II": "<", b"MM": ">"}[buf[:2]]
    (ifd,) = struct.unpack(bo + "I", buf[4:8])
    (count,) = struct.unpack(bo + "H", buf[ifd:ifd + 2])
    sizes = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8}
    tags = {}
    for k in range(count):
        e = ifd + 2 + 12 * k
        tag, typ, cnt = struct.unpack(bo + "HHI", buf[e:e + 8])
        sz = sizes.get(typ, 1) * cnt
        raw = buf[e + 8:e + 12] if sz <= 4 else buf[struct.unpack(bo + "I", buf[e + 8:e + 12])[0]:][:sz]
        if typ == 3:
            vals = struct.unpack(bo + "%dH" % cnt, raw[:2 * cnt])
        elif typ == 4:
            vals = struct.unpack(bo + "%dI" % cnt, raw[:4 * cnt])
        else:
            vals = tuple(raw[:cnt])
        tags[tag] = vals
    w, h = tags[256][0], tags[257][0]
    bps = tags.get(258, (1,))[0]
    comp = tags.get(259, (1,))[0]
    spp = tags.get(277, (1,))[0]
    pred = tags.get(317, (1,))[0]
    if spp != 1 or bps not in (8, 16) or comp not in (1, 5):
        raise ValueError("unsupported TIFF: spp=%d bps=%d compression=%d" % (spp, bps, comp))
    offs, cnts = tags[273], tags[279]
    data = bytearray()
    for o, c in zip(offs, cnts):
        chunk = buf[o:o + c]
        data += _lzw_decode(chunk) if comp == 5 else chunk
    dt = np.dtype(bo + ("u1" if bps == 8 else "u2"))
    arr = np.frombuffer(bytes(data[:w * h * dt.itemsize]), dtype=dt).reshape(h, w)
    if pred == 2:
        arr = np.cumsum(arr, axis=1, dtype=dt)
    return arr.astype(np.uint16 if bps == 16 else np.uint8), bps
