"""TIFF codec and command-line front door (no GPU: the reconstruction is
replaced by a stand-in where a test needs one)."""
import struct
import zlib

import numpy as np
import pytest

from nanopyx_gb300 import cli, tiff


@pytest.mark.parametrize("shape,dtype", [((5, 7), np.float32), ((3, 6, 4), np.float32),
                                         ((2, 3, 4, 5), np.float32), ((9, 8), np.uint16),
                                         ((2, 5, 5), np.int32), ((4, 3), np.float64)])
@pytest.mark.parametrize("big", [False, True])
def test_round_trip(tmp_path, shape, dtype, big):
    rng = np.random.default_rng(1)
    a = (rng.random(shape) * 1000).astype(dtype)
    p = tmp_path / "a.tif"
    p.write_bytes(tiff._encode(a, bigtiff=big))
    b = tiff._decode(p.read_bytes())
    assert b.dtype == a.dtype and b.shape == a.shape and np.array_equal(a, b)


def _lzw_encode(data: bytes) -> bytes:
    """TIFF LZW as libtiff writes it (TIFF 6.0 section 13): clear code first,
    MSB-first codes, the width growing once the next free code passes
    2^width - 1, a clear code when the table reaches 4094 entries."""
    def fresh():
        return {bytes((i,)): i for i in range(256)}, 258, 9

    table, nxt, width = fresh()
    codes = [(256, 9)]
    w = b""
    for c in data:
        wc = w + bytes((c,))
        if wc in table:
            w = wc
            continue
        codes.append((table[w], width))
        table[wc] = nxt
        nxt += 1
        if nxt > (1 << width) - 1 and width < 12:
            width += 1
        if nxt >= 4094:
            codes.append((256, width))
            table, nxt, width = fresh()
        w = bytes((c,))
    if w:
        codes.append((table[w], width))
    codes.append((257, width))
    out, acc, nb = bytearray(), 0, 0
    for code, wd in codes:
        acc = (acc << wd) | code
        nb += wd
        while nb >= 8:
            nb -= 8
            out.append((acc >> nb) & 0xFF)
    if nb:
        out.append((acc << (8 - nb)) & 0xFF)
    return bytes(out)


def _classic_be(pages, compress=None, predictor=1):
    """A big-endian uint16 TIFF of several pages, each in 2-row strips."""
    out = bytearray(b"MM" + struct.pack(">HI", 42, 0))
    prev = 4
    for img in pages:
        H, W = img.shape
        offs, cnts = [], []
        for r in range(0, H, 2):
            rows = img[r:r + 2].astype(">u2")
            if predictor == 2:
                rows = np.concatenate([rows[:, :1], np.diff(rows, axis=1)], axis=1).astype(">u2")
            raw = rows.tobytes()
            if compress == "deflate":
                raw = zlib.compress(raw)
            elif compress == "lzw":
                raw = _lzw_encode(raw)
            offs.append(len(out))
            cnts.append(len(raw))
            out += raw
            if len(out) % 2:
                out += b"\0"
        so = len(out)
        out += struct.pack(">" + "I" * len(offs), *offs)
        sc = len(out)
        out += struct.pack(">" + "I" * len(cnts), *cnts)
        ent = [(256, 3, 1, W), (257, 3, 1, H), (258, 3, 1, 16),
               (259, 3, 1, {"deflate": 8, "lzw": 5}.get(compress, 1)), (262, 3, 1, 1),
               (273, 4, len(offs), so), (277, 3, 1, 1), (278, 3, 1, 2),
               (279, 4, len(cnts), sc), (317, 3, 1, predictor)]
        ifd = len(out)
        out += struct.pack(">H", len(ent))
        for tag, typ, cnt, val in ent:
            out += struct.pack(">HHI", tag, typ, cnt)
            out += struct.pack(">HH", val, 0) if typ == 3 and cnt == 1 else struct.pack(">I", val)
        link = len(out)
        out += struct.pack(">I", 0)
        struct.pack_into(">I", out, prev, ifd)
        prev = link
    return bytes(out)


@pytest.mark.parametrize("compress,predictor", [(None, 1), ("deflate", 1), ("deflate", 2),
                                                ("lzw", 1), ("lzw", 2)])
def test_reads_big_endian_multipage_strips(compress, predictor):
    rng = np.random.default_rng(2)
    pages = [rng.integers(0, 60000, (5, 6)).astype(np.uint16) for _ in range(3)]
    got = tiff._decode(_classic_be(pages, compress, predictor))
    assert got.shape == (3, 5, 6) and got.dtype == np.uint16
    assert np.array_equal(got, np.stack(pages))


def test_lzw_decoder_round_trips_long_strips():
    """Code widths 9..12 and the clear codes of a full table."""
    rng = np.random.default_rng(3)
    for data in (rng.integers(0, 256, 30000).astype(np.uint8).tobytes(),
                 bytes(rng.integers(0, 4, 50000).astype(np.uint8)),
                 b"abcabcabcabcabcabcabcabcabc" * 700, b"", b"x"):
        assert tiff._lzw_decode(_lzw_encode(data), len(data)) == data


def _float_strip(img, bo, compress, predictor):
    """A one-page float32 TIFF (one strip) in byte order `bo` ('<' or '>')."""
    H, W = img.shape
    if predictor == 3:
        b = img.astype(">f4").view(np.uint8).reshape(H, W, 4).transpose(0, 2, 1)
        b = b.reshape(H, 4 * W).astype(np.int16)
        raw = np.concatenate([b[:, :1], np.diff(b, axis=1) % 256], axis=1).astype(np.uint8)
        raw = raw.tobytes()
    else:
        raw = img.astype(bo + "f4").tobytes()
    raw = zlib.compress(raw) if compress == "deflate" else _lzw_encode(raw)
    out = bytearray((b"II" if bo == "<" else b"MM") + struct.pack(bo + "HI", 42, 8))
    ent = [(256, 3, W), (257, 3, H), (258, 3, 32), (259, 3, 8 if compress == "deflate" else 5),
           (262, 3, 1), (273, 4, 0), (277, 3, 1), (278, 3, H), (279, 4, len(raw)),
           (317, 3, predictor), (339, 3, 3)]
    data_off = 8 + 2 + 12 * len(ent) + 4
    out += struct.pack(bo + "H", len(ent))
    for tag, typ, val in ent:
        val = data_off if tag == 273 else val
        out += struct.pack(bo + "HHI", tag, typ, 1)
        out += struct.pack(bo + "HH", val, 0) if typ == 3 else struct.pack(bo + "I", val)
    out += struct.pack(bo + "I", 0)
    return bytes(out) + raw


@pytest.mark.parametrize("bo", ["<", ">"])
@pytest.mark.parametrize("compress", ["deflate", "lzw"])
@pytest.mark.parametrize("predictor", [1, 3])
def test_reads_float_strips_with_the_floating_point_predictor(bo, compress, predictor):
    rng = np.random.default_rng(4)
    img = (rng.standard_normal((7, 13)) * 100).astype(np.float32)
    img[0, 0], img[1, 2], img[3, 4] = 0.0, -0.0, np.float32(1e-40)
    got = tiff._decode(_float_strip(img, bo, compress, predictor))
    assert got.dtype == np.float32 and got.shape == img.shape
    assert np.array_equal(got.view(np.uint32), img.view(np.uint32))


def test_rejects_non_tiff():
    with pytest.raises(ValueError):
        tiff._decode(b"PK\x03\x04")


def test_cli_esrrf_maps_arguments_and_writes_tiff(tmp_path, monkeypatch):
    from nanopyx_gb300 import methods

    seen = {}

    def fake_esrrf(image, **kw):
        seen.update(kw, shape=image.shape)
        return np.full((1, 4, 4), 7.0, np.float32)

    monkeypatch.setattr(methods, "eSRRF", fake_esrrf)
    src, dst = tmp_path / "in.tif", tmp_path / "out.tif"
    tiff.imwrite(str(src), np.ones((6, 8, 8), np.float32))
    assert cli.main(["linkinpy-SuperResolution-eSRRF", str(src), str(dst), "--magnification",
                     "2", "--radius", "2.0", "--temporal-correlation", "VAR",
                     "--no-macro-pixel-correction", "--pad-edges"]) == 0
    assert seen["shape"] == (6, 8, 8) and seen["magnification"] == 2
    assert seen["radius"] == 2.0 and seen["temporal_correlation"] == "VAR"
    assert seen["macro_pixel_correction"] is False and seen["pad_edges"] is True
    assert seen["use_fht"] is False and seen["doIntensityWeighting"] is True
    assert np.array_equal(tiff.imread(str(dst)), np.full((1, 4, 4), 7.0, np.float32))


def test_cli_unknown_command():
    assert cli.main(["linkinpy-Restoration-NLMDenoising"]) == 2
