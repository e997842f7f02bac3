"""Readers for the record files that the catalog programs write, and the catalog's inputs.

A record file starts with b"NEBOCAT1" and holds, per record,
  u32 kind (0 field, 1 value, 2 error), u32 name length, name bytes, then
  field: i32 gx, gy, gz, type code, f64[gz*gy*gx] (x fastest) | value: f64 | error: u32 len, bytes
"""
from __future__ import annotations

import struct

import numpy as np

SENTINEL = -7777.25

# location type codes shared with tests/cpp (SVol=1 ... ZSurfZ=16, SingleValue=17)
TYPE_CODES = {
    "SVol": 1, "XVol": 2, "YVol": 3, "ZVol": 4,
    "SSurfX": 5, "SSurfY": 6, "SSurfZ": 7,
    "XSurfX": 8, "XSurfY": 9, "XSurfZ": 10,
    "YSurfX": 11, "YSurfY": 12, "YSurfZ": 13,
    "ZSurfX": 14, "ZSurfY": 15, "ZSurfZ": 16,
    "SingleValue": 17,
}


def read_records(path_or_bytes):
    b = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    if b[:8] != b"NEBOCAT1":
        raise ValueError("not a catalog record file")
    o = 8
    recs = {}
    while o < len(b):
        kind, n = struct.unpack_from("<II", b, o)
        o += 8
        name = b[o:o + n].decode()
        o += n
        if kind == 0:
            gx, gy, gz, tc = struct.unpack_from("<4i", b, o)
            o += 16
            a = np.frombuffer(b, "<f8", gx * gy * gz, o).reshape(gz, gy, gx).copy()
            o += 8 * gx * gy * gz
            recs[name] = ("field", tc, a)
        elif kind == 1:
            (v,) = struct.unpack_from("<d", b, o)
            o += 8
            recs[name] = ("value", v)
        elif kind == 2:
            (m,) = struct.unpack_from("<I", b, o)
            o += 4
            recs[name] = ("error", b[o:o + m].decode())
            o += m
        else:
            raise ValueError(f"bad record kind {kind}")
    return recs


def records_to_npz_dict(recs):
    out = {}
    for name, r in recs.items():
        if r[0] == "field":
            out["f:" + name] = r[2]
            out["t:" + name] = np.int32(r[1])
        elif r[0] == "value":
            out["v:" + name] = np.float64(r[1])
        else:
            out["e:" + name] = np.array(r[1])
    return out


def npz_to_records(z):
    recs = {}
    for k in z.files:
        kind, name = k.split(":", 1)
        if kind == "f":
            recs[name] = ("field", int(z["t:" + name]), z[k])
        elif kind == "v":
            recs[name] = ("value", float(z[k]))
        elif kind == "e":
            recs[name] = ("error", str(z[k]))
    return recs


# ----------------------------------------------------------------------------- inputs
M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x):
    with np.errstate(over="ignore"):
        x = (x + np.uint64(0x9E3779B97F4A7C15)) & M64
        x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & M64
        x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & M64
        return x ^ (x >> np.uint64(31))


def uniform_pm1(stream, count):
    """Same values as catalog::uniform_pm1(stream, i) for i in [0, count)."""
    s = _splitmix64(np.uint64(stream))
    with np.errstate(over="ignore"):
        h = _splitmix64((s + np.arange(count, dtype=np.uint64)) & M64)
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0) * 2.0 - 1.0


def field_stream(type_code, k, domain):
    return 1000003 * type_code + 7919 * k + 104729 * domain + 17


def mask_points(k, domain, n, ghost):
    gx, gy, gz = n[0] + 2 * ghost, n[1] + 2 * ghost, n[2] + 2 * ghost
    u = uniform_pm1(field_stream(99, k, domain), gx * gy * gz).reshape(gz, gy, gx)
    zz, yy, xx = np.nonzero(u < -0.6)
    return np.stack([xx - ghost, yy - ghost, zz - ghost], axis=1).astype(np.int32)
