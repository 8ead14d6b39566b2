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


def mixed_lists(rng):
    """Particle lists of every vertex type and every colour type of the MMPLD format
    (MMPLDDataSource.cpp:84-160), with global radius / colour / intensity ranges, in mmpld_io's form."""
    lists = []
    n = [37, 50, 11, 23, 19, 13, 29, 7]
    vt_dtype = {1: (np.float32, 3), 2: (np.float32, 4), 3: (np.uint16, 3), 4: (np.float64, 3)}
    ct_dtype = {1: (np.uint8, 3), 2: (np.uint8, 4), 3: (np.float32, 1), 4: (np.float32, 3), 5: (np.float32, 4),
                6: (np.uint16, 4), 7: (np.float64, 1)}
    combos = [(2, 2), (1, 3), (3, 0), (4, 4), (1, 5), (2, 6), (4, 7), (3, 1)]
    for k, (vt, ct) in enumerate(combos):
        dt, nc = vt_dtype[vt]
        v = (rng.integers(0, 60000, (n[k], nc)) if dt == np.uint16 else rng.uniform(-5, 15, (n[k], nc))).astype(dt)
        c = None
        if ct:
            cdt, cnc = ct_dtype[ct]
            c = (rng.integers(0, 255, (n[k], cnc)) if cdt in (np.uint8, np.uint16) else
                 rng.uniform(-1, 4, (n[k], cnc))).astype(cdt)
        lists.append(dict(vt=vt, ct=ct, count=n[k], records=records(v, c),
                          radius=float(rng.uniform(0.1, 2.0)), colour=tuple(int(x) for x in rng.integers(0, 255, 4)),
                          irange=(float(rng.uniform(-2, 0)), float(rng.uniform(1, 3))),
                          bbox=tuple(float(x) for x in rng.uniform(-3, 3, 6)), clusters=int(rng.integers(1, 9)),
                          cluster_blob=bytes(rng.integers(0, 255, int(rng.integers(0, 12))).astype(np.uint8))))
    # lists without vertex data: the raw colour byte still decides which header fields follow (:164-177)
    lists.append(dict(vt=0, ct=0, count=5, records=b"", colour=(1, 2, 3, 4)))
    lists.append(dict(vt=0, ct=3, count=4, records=b"", irange=(-7.5, 2.25)))
    lists.append(dict(vt=0, ct=5, count=3, records=b""))
    # unknown colour type: no colour data, no extra header field (:150-153); an empty list
    v = rng.uniform(0, 1, (6, 3)).astype(np.float32)
    lists.append(dict(vt=1, ct=9, count=6, records=records(v), radius=0.3))
    lists.append(dict(vt=2, ct=2, count=0, records=b""))
    return lists
