"""A small reader of ZDF version 1 files (the record stream written by
zdf_io.c and by the reference's em2d/zdf.c), for the tests: magic "ZDF1",
then records of uint32 id/version, name string, uint64 payload length and
payload, little endian; strings are a uint32 length plus bytes padded to 4."""
import struct

import numpy as np

TYPES = {1: np.int8, 2: np.uint8, 3: np.int16, 4: np.uint16, 5: np.int32, 6: np.uint32, 7: np.int64,
         8: np.uint64, 9: np.float32, 10: np.float64}


class _Cursor:
    def __init__(self, b, pos=0):
        self.b, self.pos = b, pos

    def u32(self):
        v = struct.unpack_from("<I", self.b, self.pos)[0]
        self.pos += 4
        return v

    def i32(self):
        v = struct.unpack_from("<i", self.b, self.pos)[0]
        self.pos += 4
        return v

    def u64(self):
        v = struct.unpack_from("<Q", self.b, self.pos)[0]
        self.pos += 8
        return v

    def f64(self):
        v = struct.unpack_from("<d", self.b, self.pos)[0]
        self.pos += 8
        return v

    def string(self):
        n = self.u32()
        s = self.b[self.pos:self.pos + n].decode()
        self.pos += (n + 3) // 4 * 4
        return s


def read(path):
    """Returns the records as a list of (kind, name, value) and the raw
    bytes; datasets come as numpy arrays shaped (count[n-1], ..., count[0])."""
    b = open(path, "rb").read()
    assert b[:4] == b"ZDF1", "not a ZDF file"
    c = _Cursor(b, 4)
    recs = []
    while c.pos < len(b):
        rid = c.u32()
        name = c.string()
        length = c.u64()
        start = c.pos
        kind = rid >> 16
        if kind == 1:
            val = c.i32()
        elif kind == 2:
            val = c.f64()
        elif kind == 3:
            val = c.string()
        elif kind == 0x20:
            val = {"n": c.i32(), "t": c.f64(), "time_units": c.string()}
        elif kind == 0x21:
            nd = c.u32()
            count = [c.u64() for _ in range(nd)]
            val = {"ndims": nd, "count": count, "label": c.string(), "units": c.string()}
            if c.i32():
                val["axis"] = [{"name": c.string(), "type": c.i32(), "min": c.f64(), "max": c.f64(),
                                "label": c.string(), "units": c.string()} for _ in range(nd)]
        elif kind == 0x22:
            val = {"label": c.string(), "np": c.u64()}
            nq = c.u32()
            q = [c.string() for _ in range(nq)]
            ql = [c.string() for _ in range(nq)]
            qu = [c.string() for _ in range(nq)]
            val.update(quants=q, qlabels=ql, qunits=qu)
        elif kind in (0x10, 0x11):
            ds_id, dtype, nd = c.u32(), c.i32(), c.u32()
            count = [c.u64() for _ in range(nd)]
            val = {"id": ds_id, "type": dtype, "count": count}
            if kind == 0x10:
                n = int(np.prod(count)) if count else 0
                arr = np.frombuffer(b, dtype=np.dtype(TYPES[dtype]).newbyteorder("<"), count=n, offset=c.pos)
                val["data"] = arr.reshape(count[::-1]) if n else arr
        else:
            val = None
        c.pos = start + length
        recs.append((kind, name, val))
    return recs, b


def header_bytes(raw):
    """The file without the dataset payloads (metadata records plus the
    dataset record headers), for byte comparisons that leave the data
    values to a tolerance check."""
    c = _Cursor(raw, 4)
    out, keep = [raw[:4]], 4
    while c.pos < len(raw):
        rid = c.u32()
        c.string()
        length = c.u64()
        if rid >> 16 == 0x10:
            c.u32(), c.i32()
            nd = c.u32()
            c.pos += 8 * nd
            out.append(raw[keep:c.pos])
            c.pos = c.pos + length - (12 + 8 * nd)
            keep = c.pos
        else:
            c.pos += length
    out.append(raw[keep:])
    return b"".join(out)
