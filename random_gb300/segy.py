"""SEG-Y / IBM-float helpers (numpy) for building and reading trace files.

The reference reads big-endian SEG-Y: a 3600-byte file header, then per
trace 60 big-endian 32-bit header words and ns IBM System/360 floats
(Kirchhoff.c:633-661, 1280-1290).  It writes big-endian IEEE SU traces
(Kirchhoff.c:1482-1593).  These helpers create such files for synthetic
surveys and decode them; the C library has its own decoder
(kpstm_ibm_to_ieee) for the product path.
"""
from __future__ import annotations

import numpy as np

HEADER_WORDS = 60
# 0-based 32-bit word indices in the 240-byte trace header.
W_TRACL, W_CDP, W_OFFSET, W_SX, W_SY, W_GX, W_GY = 0, 5, 9, 18, 19, 20, 21
W_NS = 28             # bytes 115-116: ns is the low half of word 28
W_DT = 29             # bytes 117-118: dt (microseconds) is the high half of word 29
W_CDPX, W_CDPY, W_ILINE, W_XLINE = 45, 46, 47, 48


def ieee_to_ibm(x: np.ndarray) -> np.ndarray:
    """IEEE float32 -> IBM single words (host-order uint32), round to nearest."""
    x = np.asarray(x, dtype=np.float64)
    out = np.zeros(x.shape, dtype=np.uint32)
    nz = x != 0
    a = np.abs(x[nz])
    sign = (x[nz] < 0).astype(np.uint64)
    # |x| = F * 16**E with F in [1/16, 1)
    e = np.floor(np.log2(a) / 4.0).astype(np.int64) + 1
    f = a / np.power(16.0, e)
    lo = f < 1.0 / 16.0
    e[lo] -= 1
    f[lo] *= 16.0
    hi = f >= 1.0
    e[hi] += 1
    f[hi] /= 16.0
    frac = np.rint(f * 2.0 ** 24).astype(np.int64)
    carry = frac >= (1 << 24)
    frac[carry] >>= 4
    e[carry] += 1
    if np.any(e + 64 > 127) or np.any(e + 64 < 0):
        raise ValueError("value outside IBM single range")
    words = (sign << 31) | ((e + 64).astype(np.uint64) << 24) | frac.astype(np.uint64)
    out[nz] = words.astype(np.uint32)
    return out


def ibm_to_ieee(words: np.ndarray) -> np.ndarray:
    """IBM words (host-order uint32) -> float32, with the arithmetic of
    Kirchhoff.c:1284-1290: sign * (float)(frac / 2^24) * (float)16^(exp-64),
    all products in float."""
    w = np.asarray(words, dtype=np.uint32).astype(np.int64)
    sign = np.where((w >> 31) & 1, -1.0, 1.0).astype(np.float32)
    frac = ((w & 0x00FFFFFF).astype(np.float32) / np.float32(0x1000000)).astype(np.float32)
    scale = np.power(16.0, ((w >> 24) & 0x7F) - 64).astype(np.float32)
    return (sign * frac * scale).astype(np.float32)


def ibm_roundtrip(x: np.ndarray) -> np.ndarray:
    """The float32 values a reader of the IBM file sees for ``x``."""
    return ibm_to_ieee(ieee_to_ibm(x))


def trace_headers(sx, sy, gx, gy, ns: int, dt_us: int, extra: dict | None = None) -> np.ndarray:
    """[ntr, 60] int32 host-order header words with the fields the
    reference reads (sx, sy, gx, gy; ns and dt of the first trace)."""
    ntr = len(sx)
    h = np.zeros((ntr, HEADER_WORDS), dtype=np.int64)
    h[:, W_TRACL] = np.arange(1, ntr + 1)
    h[:, W_SX] = sx
    h[:, W_SY] = sy
    h[:, W_GX] = gx
    h[:, W_GY] = gy
    h[:, W_NS] = int(ns) & 0xFFFF
    h[:, W_DT] = (int(dt_us) & 0xFFFF) << 16
    for k, v in (extra or {}).items():
        h[:, k] = v
    if np.any(h > np.iinfo(np.int32).max) or np.any(h < np.iinfo(np.int32).min):
        raise ValueError("header value outside int32")
    return h.astype(np.int32)


def headers_be(h: np.ndarray) -> np.ndarray:
    """Header words as the bytes of a file: big-endian int32 words,
    returned as a native-int32 view of those bytes (what fread gives)."""
    return np.ascontiguousarray(h, dtype=">i4").view(np.int32)


def write_segy(path, headers: np.ndarray, samples: np.ndarray) -> None:
    """SEG-Y file: 3200 + 400 header bytes, then per trace 240 header bytes
    and ns IBM floats, all big-endian."""
    ntr, ns = samples.shape
    rec = np.empty((ntr, HEADER_WORDS + ns), dtype=">u4")
    rec[:, :HEADER_WORDS] = headers.astype(np.int64) & 0xFFFFFFFF
    rec[:, HEADER_WORDS:] = ieee_to_ibm(samples)
    with open(path, "wb") as f:
        f.write(b"\x40" * 3200)
        binh = np.zeros(200, dtype=">u2")
        binh[8] = (int(headers[0, W_DT]) >> 16) & 0xFFFF      # dt, bytes 3217-3218
        binh[10] = int(headers[0, W_NS]) & 0xFFFF             # ns, bytes 3221-3222
        binh[12] = 1                                          # IBM float
        f.write(binh.tobytes())
        f.write(rec.tobytes())


def segy_records(headers: np.ndarray, samples: np.ndarray) -> np.ndarray:
    """The trace records of a SEG-Y file (no file header) as uint8 [ntr, 240+4ns]."""
    ntr, ns = samples.shape
    rec = np.empty((ntr, HEADER_WORDS + ns), dtype=">u4")
    rec[:, :HEADER_WORDS] = headers.astype(np.int64) & 0xFFFFFFFF
    rec[:, HEADER_WORDS:] = ieee_to_ibm(samples)
    return rec.view(np.uint8).reshape(ntr, -1)


def velocity_headers(n_il: int, n_xl: int, o_il: int, o_xl: int, d_il: int, d_xl: int,
                     nsm: int, dtm_us: int) -> np.ndarray:
    """Headers of a gridded velocity SEG-Y: iline/xline in words 47/48
    (Kirchhoff.c:537-538), grid order [il][xl]."""
    il = o_il + d_il * np.repeat(np.arange(n_il), n_xl)
    xl = o_xl + d_xl * np.tile(np.arange(n_xl), n_il)
    z = np.zeros(n_il * n_xl, dtype=np.int64)
    return trace_headers(z, z, z, z, nsm, dtm_us, {W_ILINE: il, W_XLINE: xl})
