"""Test helper: writes MMPLD files in the layout MegaMol's MMPLD reader expects
(plugins/moldyn/src/io/MMPLDDataSource.cpp:50-220 and :386-401): versions 1.0-1.3, frame table, per frame a
timestamp (1.2+) and lists of interleaved vertex + colour records."""
import struct

import numpy as np

VERTEX_BYTES = {0: 0, 1: 12, 2: 16, 3: 6, 4: 24}
COLOUR_BYTES = {0: 0, 1: 3, 2: 4, 3: 4, 4: 12, 5: 16, 6: 8, 7: 8}


def list_bytes(lst: dict, version: int) -> bytes:
    """lst: vt, ct, records (uint8 array of count * stride bytes), count, and radius / colour / irange /
    bbox / clusters as the types need them."""
    vt, ct = lst["vt"], lst["ct"]
    out = struct.pack("<BB", vt, ct)
    if vt in (1, 3, 4):
        out += struct.pack("<f", lst.get("radius", 0.5))
    if ct == 0:
        out += bytes(lst.get("colour", (10, 20, 30, 40)))
    elif ct in (3, 7):
        out += struct.pack("<ff", *lst.get("irange", (0.0, 1.0)))
    out += struct.pack("<Q", lst["count"])
    if version >= 103:
        out += struct.pack("<6f", *lst.get("bbox", (0, 0, 0, 1, 1, 1)))
    out += bytes(lst["records"])
    if version == 101:
        blob = bytes(lst.get("cluster_blob", b"\x01\x02\x03"))
        out += struct.pack("<IQ", lst.get("clusters", 2), len(blob)) + blob
    return out


def write(path, frames, version=103, bbox=(0, 0, 0, 10, 10, 10), clipbox=(-1, -1, -1, 11, 11, 11)):
    """frames: list of (timestamp, [list dicts])."""
    blobs = []
    for ts, lists in frames:
        b = struct.pack("<f", ts) if version >= 102 else b""
        b += struct.pack("<I", len(lists))
        for lst in lists:
            b += list_bytes(lst, version)
        blobs.append(b)
    head = b"MMPLD\0" + struct.pack("<HI", version, len(frames)) + struct.pack("<6f", *bbox) + \
        struct.pack("<6f", *clipbox)
    off = len(head) + 8 * (len(frames) + 1)
    offsets = [off]
    for b in blobs:
        off += len(b)
        offsets.append(off)
    with open(path, "wb") as f:
        f.write(head)
        f.write(struct.pack(f"<{len(offsets)}Q", *offsets))
        for b in blobs:
            f.write(b)


def records(vertex: np.ndarray, colour: np.ndarray = None) -> np.ndarray:
    """Interleave per-particle vertex and colour arrays (any dtypes) into one byte array."""
    n = vertex.shape[0]
    v = np.ascontiguousarray(vertex).view(np.uint8).reshape(n, -1)
    if colour is None:
        return v.ravel()
    c = np.ascontiguousarray(colour).view(np.uint8).reshape(n, -1)
    return np.concatenate([v, c], 1).ravel()
