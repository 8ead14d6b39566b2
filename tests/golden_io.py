"""Loading of the committed golden fixtures (tests/golden/p2d_*.npz) and conversion of their particle
lists into the float xyzr records the reference's accessors produce (SimpleSphericalParticles.h:86-130:
Get_f() is a static_cast<float> of the stored component; lists without a radius use the global one)."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
VERT_NONE, VERT_FLOAT_XYZ, VERT_FLOAT_XYZR, VERT_SHORT_XYZ, VERT_DOUBLE_XYZ = 0, 1, 2, 3, 4
_COMP = {VERT_FLOAT_XYZ: (np.float32, 3), VERT_FLOAT_XYZR: (np.float32, 4), VERT_SHORT_XYZ: (np.uint16, 3),
         VERT_DOUBLE_XYZ: (np.float64, 3)}


def golden_names():
    return sorted(os.path.basename(p)[4:-4] for p in glob.glob(os.path.join(GOLDEN, "p2d_*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, f"p2d_{name}.npz"))
    case = {k: z[k] for k in z.files}
    lists = []
    for i in range(int(case["nlists"])):
        lists.append(dict(type=int(case[f"l{i}_type"]), data=case[f"l{i}_data"], stride=int(case[f"l{i}_stride"]),
                          radius=float(case[f"l{i}_radius"]), count=int(case[f"l{i}_count"])))
    case["lists"] = lists
    case.setdefault("surface", np.int32(0))
    return case


def grid(case):
    """(bbox, resolution) of the grid the module computes on: the stored box and slot resolution, or for a
    forSurfaceReconstruction case the box adjustment restated by the oracle (ParticlesToDensity.cpp:749-799)."""
    if int(case["surface"]):
        import oracle
        return oracle.modify_bbox_f32(case["bbox"], case["res"])
    return tuple(float(v) for v in case["bbox"]), tuple(int(v) for v in case["res"])


def list_to_xyzr(L):
    """Float xyzr records of one particle list, read as the reference's accessors read them."""
    t = L["type"]
    if t == VERT_NONE:
        return np.zeros((0, 4), np.float32)
    dt, nc = _COMP[t]
    n = int(L["count"])
    raw = np.ascontiguousarray(L["data"]).view(np.uint8).reshape(-1)
    isz = np.dtype(dt).itemsize
    stride = int(L["stride"]) or nc * isz
    out = np.empty((n, 4), np.float32)
    for c in range(nc):
        idx = np.arange(n) * stride + c * isz
        comp = np.frombuffer(raw.tobytes(), dtype=np.uint8)
        vals = np.stack([comp[idx + b] for b in range(isz)], 1).copy().view(dt).reshape(n)
        out[:, c] = vals.astype(np.float32)
    if nc == 3:
        out[:, 3] = np.float32(L["radius"])
    return out


def case_xyzr(case):
    return np.concatenate([list_to_xyzr(L) for L in case["lists"]], 0)
