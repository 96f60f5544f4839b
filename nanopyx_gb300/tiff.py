"""TIFF input/output of the command-line front door.

The reference's CLI reads and writes TIFF through ``tifffile``
(src/nanopyx/cli/superresolution.py:5); that package is used when it is
installed.  Otherwise this module's own baseline-TIFF codec serves:

* read: classic and BigTIFF, either byte order, every page (IFD) of the file,
  strips or tiles, no compression / LZW / Deflate (zlib) / PackBits, with
  horizontal differencing (predictor 2) or the floating-point predictor (3),
  8/16/32/64-bit unsigned, signed and float samples, one sample per pixel; pages of one shape stack to (pages, H, W),
  and an ImageJ description or a ``{"shape": [...]}`` JSON description
  restores the array's shape.
* write: little-endian uncompressed TIFF (BigTIFF past 4 GB), one page per
  2-D plane, the array's shape in a JSON ImageDescription (the convention
  tifffile itself follows), float32/float64/integer samples.
"""
from __future__ import annotations

import json
import struct
import zlib

import numpy as np

_TYPES = {1: "B", 2: "s", 3: "H", 4: "I", 5: "II", 6: "b", 7: "B", 8: "h", 9: "i", 10: "ii",
          11: "f", 12: "d", 16: "Q", 17: "q", 18: "Q"}
_SIZES = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8, 6: 1, 7: 1, 8: 2, 9: 4, 10: 8, 11: 4, 12: 8, 16: 8,
          17: 8, 18: 8}
_SAMPLE = {1: "u", 2: "i", 3: "f"}


def _have_tifffile():
    try:
        import tifffile  # noqa: F401

        return True
    except ImportError:
        return False


def imread(path: str) -> np.ndarray:
    """The image data of a TIFF file as a NumPy array."""
    if _have_tifffile():
        import tifffile

        return tifffile.imread(path)
    with open(path, "rb") as f:
        data = f.read()
    return _decode(data)


def imwrite(path: str, array) -> None:
    """Write an array (2-D or more; leading axes become pages) as TIFF."""
    arr = np.asarray(array)
    if _have_tifffile():
        import tifffile

        tifffile.imwrite(path, arr)
        return
    with open(path, "wb") as f:
        f.write(_encode(arr))


# ---------------------------------------------------------------------------
# reading
# ---------------------------------------------------------------------------
def _decode(data: bytes) -> np.ndarray:
    if data[:2] == b"II":
        bo = "<"
    elif data[:2] == b"MM":
        bo = ">"
    else:
        raise ValueError("not a TIFF file")
    (magic,) = struct.unpack(bo + "H", data[2:4])
    if magic == 42:
        big = False
        (off,) = struct.unpack(bo + "I", data[4:8])
    elif magic == 43:
        big = True
        (off,) = struct.unpack(bo + "Q", data[8:16])
    else:
        raise ValueError("not a TIFF file")
    pages, desc = [], None
    seen = set()
    while off:
        if off in seen or off >= len(data):
            raise ValueError("corrupt TIFF: IFD chain")
        seen.add(off)
        tags, off = _read_ifd(data, off, bo, big)
        if desc is None and 270 in tags:
            desc = tags[270]
        pages.append(_read_page(data, tags, bo))
    if not pages:
        raise ValueError("TIFF file has no pages")
    shapes = {p.shape for p in pages}
    out = np.stack(pages) if len(shapes) == 1 else pages[0][None]
    return _reshape(out, desc)


def _read_ifd(data, off, bo, big):
    cnt_fmt, ent_size, hdr = ("Q", 20, 8) if big else ("H", 12, 2)
    (n,) = struct.unpack(bo + cnt_fmt, data[off:off + hdr])
    tags = {}
    for k in range(n):
        e = off + hdr + k * ent_size
        if big:
            tag, typ, count = struct.unpack(bo + "HHQ", data[e:e + 12])
            val = data[e + 12:e + 20]
            inline = 8
        else:
            tag, typ, count = struct.unpack(bo + "HHI", data[e:e + 8])
            val = data[e + 8:e + 12]
            inline = 4
        if typ not in _SIZES:
            continue
        nbytes = _SIZES[typ] * count
        if nbytes > inline:
            (p,) = struct.unpack(bo + ("Q" if big else "I"), val[:inline])
            raw = data[p:p + nbytes]
        else:
            raw = val[:nbytes]
        if typ == 2:
            tags[tag] = raw.rstrip(b"\0").decode("utf-8", "replace")
        else:
            fmt = _TYPES[typ]
            vals = struct.unpack(bo + fmt * count, raw)
            if typ in (5, 10):
                vals = tuple(vals[i] / vals[i + 1] if vals[i + 1] else 0.0
                             for i in range(0, len(vals), 2))
            tags[tag] = vals
    nxt_fmt = "Q" if big else "I"
    pos = off + hdr + n * ent_size
    (nxt,) = struct.unpack(bo + nxt_fmt, data[pos:pos + (8 if big else 4)])
    return tags, nxt


def _unpackbits(buf: bytes, expected: int) -> bytes:
    out = bytearray()
    i = 0
    while i < len(buf) and len(out) < expected:
        n = buf[i]
        i += 1
        if n < 128:
            out += buf[i:i + n + 1]
            i += n + 1
        elif n > 128:
            out += bytes([buf[i]]) * (257 - n)
            i += 1
    return bytes(out)


def _lzw_decode(buf: bytes, expected: int) -> bytes:
    """TIFF LZW (TIFF 6.0 section 13): MSB-first codes of 9 to 12 bits,
    256 = clear, 257 = end of information, the code width growing one code
    early (after table entries 510, 1022 and 2046)."""
    src = bytes(buf) + b"\0\0\0\0"
    nbits = len(buf) * 8
    out = bytearray()
    table = [bytes((i,)) for i in range(256)] + [b"", b""]
    width, pos, prev = 9, 0, None
    while pos + width <= nbits and len(out) < expected:
        i = pos >> 3
        word = (src[i] << 24) | (src[i + 1] << 16) | (src[i + 2] << 8) | src[i + 3]
        code = (word >> (32 - (pos & 7) - width)) & ((1 << width) - 1)
        pos += width
        if code == 257:
            break
        if code == 256:
            del table[258:]
            width, prev = 9, None
            continue
        if prev is None:
            if code >= 256:
                raise ValueError("corrupt TIFF LZW data")
            entry = table[code]
        else:
            if code < len(table):
                entry = table[code]
                new_entry = prev + entry[:1]
            elif code == len(table):
                entry = new_entry = prev + prev[:1]
            else:
                raise ValueError("corrupt TIFF LZW data")
            if len(table) < 4096:
                table.append(new_entry)
                if len(table) + 1 >= (1 << width) and width < 12:
                    width += 1
        out += entry
        prev = entry
    return bytes(out)


def _read_page(data, tags, bo) -> np.ndarray:
    W = tags[256][0]
    H = tags[257][0]
    bits = tags.get(258, (1,))[0]
    comp = tags.get(259, (1,))[0]
    spp = tags.get(277, (1,))[0]
    fmt = _SAMPLE.get(tags.get(339, (1,))[0])
    pred = tags.get(317, (1,))[0]
    if pred not in (1, 2, 3):
        raise NotImplementedError(f"TIFF predictor {pred} (install tifffile)")
    if spp != 1:
        raise NotImplementedError("TIFF pages with more than one sample per pixel")
    if fmt is None or bits not in (8, 16, 32, 64):
        raise NotImplementedError(f"TIFF samples of {bits} bits, format {tags.get(339)}")
    if comp not in (1, 5, 8, 32946, 32773):
        raise NotImplementedError(f"TIFF compression {comp} (install tifffile)")
    if pred == 3 and fmt != "f":
        raise ValueError("TIFF floating-point predictor on non-float samples")
    dt = np.dtype(f"{bo}{fmt}{bits // 8}")

    def chunk(offset, count, nbytes):
        raw = data[offset:offset + count]
        if comp in (8, 32946):
            raw = zlib.decompress(raw)
        elif comp == 32773:
            raw = _unpackbits(raw, nbytes)
        elif comp == 5:
            raw = _lzw_decode(raw, nbytes)
        return raw[:nbytes]

    def block(raw, rows, width):
        # one strip or tile as a (rows, width) array, the predictor undone
        if pred == 3:
            # floating-point predictor (Adobe TIFF technical note 3): each row
            # holds the samples' bytes most significant first, byte plane by
            # byte plane, horizontally differenced as bytes
            b = np.frombuffer(raw, dtype=np.uint8).reshape(rows, dt.itemsize * width)
            b = np.cumsum(b, axis=1, dtype=np.uint8).reshape(rows, dt.itemsize, width)
            b = np.ascontiguousarray(b.transpose(0, 2, 1))
            return b.view(dt.newbyteorder(">")).reshape(rows, width).astype(dt)
        a = np.frombuffer(raw, dtype=dt).reshape(rows, width)
        return np.cumsum(a, axis=1, dtype=dt) if pred == 2 else a

    if 322 in tags:  # tiled
        tw, tl = tags[322][0], tags[323][0]
        offs, cnts = tags[324], tags[325]
        img = np.zeros((H, W), dtype=dt)
        across = -(-W // tw)
        for k, (o, c) in enumerate(zip(offs, cnts)):
            t = block(chunk(o, c, tw * tl * dt.itemsize), tl, tw)
            r0, c0 = (k // across) * tl, (k % across) * tw
            h, w = min(tl, H - r0), min(tw, W - c0)
            img[r0:r0 + h, c0:c0 + w] = t[:h, :w]
    else:
        rps = tags.get(278, (H,))[0]
        offs, cnts = tags[273], tags.get(279)
        if cnts is None:
            cnts = (H * W * dt.itemsize,)
        parts = []
        for k, (o, c) in enumerate(zip(offs, cnts)):
            rows = min(rps, H - k * rps)
            parts.append(block(chunk(o, c, rows * W * dt.itemsize), rows, W))
        img = np.concatenate(parts, axis=0)
    return img.astype(dt.newbyteorder("="))


def _reshape(arr: np.ndarray, desc) -> np.ndarray:
    if not isinstance(desc, str):
        return arr if arr.shape[0] > 1 else arr[0]
    try:
        shape = json.loads(desc).get("shape")
        if shape and int(np.prod(shape)) == arr.size:
            return arr.reshape(shape)
    except (ValueError, AttributeError):
        pass
    if desc.startswith("ImageJ="):
        kv = dict(line.split("=", 1) for line in desc.splitlines() if "=" in line)
        dims = [int(kv[k]) for k in ("frames", "slices", "channels") if int(kv.get(k, 1)) > 1]
        if dims and int(np.prod(dims)) == arr.shape[0]:
            return arr.reshape(dims + list(arr.shape[1:]))
    return arr if arr.shape[0] > 1 else arr[0]


# ---------------------------------------------------------------------------
# writing
# ---------------------------------------------------------------------------
def _encode(arr: np.ndarray, bigtiff=None) -> bytes:
    if arr.ndim < 2:
        raise ValueError("TIFF images need at least two dimensions")
    if arr.dtype.kind not in "uif" or arr.dtype.itemsize not in (1, 2, 4, 8):
        raise ValueError(f"cannot write {arr.dtype} samples")
    arr = np.ascontiguousarray(arr.astype(arr.dtype.newbyteorder("<")))
    H, W = arr.shape[-2:]
    planes = arr.reshape(-1, H, W)
    n = planes.shape[0]
    plane_bytes = H * W * arr.dtype.itemsize
    desc = json.dumps({"shape": list(arr.shape)}).encode() + b"\0"
    big = (n * plane_bytes + 4096 + n * 256 > 2 ** 32 - 1) if bigtiff is None else bool(bigtiff)
    fmt_sample = {"u": 1, "i": 2, "f": 3}[arr.dtype.kind]
    bits = arr.dtype.itemsize * 8
    out = bytearray()
    if big:
        out += b"II" + struct.pack("<HHHQ", 43, 8, 0, 0)
    else:
        out += b"II" + struct.pack("<HI", 42, 0)
    desc_off = len(out)
    out += desc
    if len(out) % 2:
        out += b"\0"
    first_ifd_field = 8 if big else 4
    prev_link = first_ifd_field
    for k in range(n):
        data_off = len(out)
        out += planes[k].tobytes()
        if len(out) % 2:
            out += b"\0"
        entries = [(256, 4, 1, W), (257, 4, 1, H), (258, 3, 1, bits), (259, 3, 1, 1),
                   (262, 3, 1, 1)]
        if k == 0:
            entries.append((270, 2, len(desc), desc_off))
        entries += [(273, 16 if big else 4, 1, data_off), (277, 3, 1, 1), (278, 4, 1, H),
                    (279, 16 if big else 4, 1, plane_bytes), (339, 3, 1, fmt_sample)]
        ifd_off = len(out)
        if big:
            out += struct.pack("<Q", len(entries))
            for tag, typ, cnt, val in entries:
                out += struct.pack("<HHQ", tag, typ, cnt)
                out += struct.pack("<Q", val) if typ in (4, 16) or tag == 270 else \
                    struct.pack("<H", val) + b"\0" * 6
            link_pos = len(out)
            out += struct.pack("<Q", 0)
            struct.pack_into("<Q", out, prev_link, ifd_off)
        else:
            out += struct.pack("<H", len(entries))
            for tag, typ, cnt, val in entries:
                out += struct.pack("<HHI", tag, typ, cnt)
                out += struct.pack("<I", val) if typ == 4 or tag == 270 else \
                    struct.pack("<H", val) + b"\0\0"
            link_pos = len(out)
            out += struct.pack("<I", 0)
            struct.pack_into("<I", out, prev_link, ifd_off)
        prev_link = link_pos
    return bytes(out)
