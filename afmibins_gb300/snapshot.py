"""Reader for the solver snapshot files that ``afmib_save`` writes (layout in
``afmibins_gb300/csrc/snapshot_io.h``): a 64-byte header, then named sections
of float64 or int32 values. Needs only numpy, no GPU."""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"AFMIBSNP"
VERSION = 1
_HEADER = struct.Struct("<8sII8iqd")       # 64 bytes
_SECTION = struct.Struct("<16sIIQ")        # 32 bytes
_DTYPES = {1: np.dtype("<f8"), 2: np.dtype("<i4")}
HEADER_FIELDS = ("nx", "ny", "nz", "n", "bc", "precision", "half", "reserved")


def _header(f):
    raw = f.read(_HEADER.size)
    if len(raw) != _HEADER.size:
        raise ValueError("not a snapshot file")
    magic, version, nsec, *ints = _HEADER.unpack(raw)
    if magic != MAGIC:
        raise ValueError("not a snapshot file")
    if version != VERSION:
        raise ValueError(f"unsupported snapshot version {version}")
    head = dict(zip(HEADER_FIELDS, ints[:8]))
    head["substeps"], head["mg_rho"] = ints[8], ints[9]
    return head, nsec


def _sections(f, nsec, load):
    out = {}
    for _ in range(nsec):
        raw = f.read(_SECTION.size)
        if len(raw) != _SECTION.size:
            raise ValueError("truncated snapshot")
        name, dtype, _, count = _SECTION.unpack(raw)
        if dtype not in _DTYPES:
            raise ValueError("bad section type")
        name = name.rstrip(b"\0").decode()
        dt = _DTYPES[dtype]
        if load:
            data = np.frombuffer(f.read(count * dt.itemsize), dtype=dt)
            if data.size != count:
                raise ValueError("truncated snapshot")
            out[name] = data
        else:
            out[name] = (dt, count)
            f.seek(count * dt.itemsize, 1)
    return out


def read(path):
    """All sections as numpy arrays, plus the header as ``sec["header"]``."""
    with open(path, "rb") as f:
        head, nsec = _header(f)
        sec = _sections(f, nsec, True)
    sec["header"] = head
    return sec


def sections(path):
    """Section names -> (dtype, count), without reading the data."""
    with open(path, "rb") as f:
        _, nsec = _header(f)
        return _sections(f, nsec, False)
