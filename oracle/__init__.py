"""CPU oracle for the particle-to-volume path — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this package,
and only to check results / as the timed CPU baseline. The shipped GPU library never calls it.

Native libraries back it (all built by ``oracle/Makefile``):

* ``_build/libp2v_oracle.so`` — our restatement of the reference algorithms (``p2v_oracle.cpp``), FP32
  with the reference's operation order and FP64 for error judging.
* ``_ref/libref_p2d.so`` — MegaMol's own ``plugins/datatools/src/ParticlesToDensity.cpp``, compiled
  unmodified against ``oracle/shim`` and driven through its slots by ``ref_harness.cpp``;
  ``_ref/libref_datraw.so`` (``volume::DatRawWriter``, ``ref_datraw.cpp``) and ``_ref/libref_mmpld.so``
  (``moldyn::io::MMPLDDataSource`` with the vislib classes it reads through, ``ref_mmpld.cpp``) likewise.
  They exist only where the reference tree was available at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libp2v_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_p2d.so")
# The MegaMol source tree: P2V_REFERENCE_TREE when set, else a checkout named "reference" beside the repository.
REFERENCE_TREE = os.environ.get("P2V_REFERENCE_TREE") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                       "reference")

BUMP, GAUSS3 = 0, 1


def build(with_reference: bool | None = None) -> None:
    """Compile the restatement, and the reference module when its source tree is present."""
    subprocess.run(["make", "-s", "-C", HERE, "restatement"], check=True)
    if with_reference is None:
        with_reference = os.path.isdir(os.path.join(REFERENCE_TREE, "plugins", "datatools"))
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_TREE}"], check=True)


class _Grid(C.Structure):
    _fields_ = [("bbox", C.c_float * 6), ("res", C.c_int32 * 3), ("cyclic", C.c_int32 * 3), ("sigma", C.c_float)]


class _ConeParams(C.Structure):
    _fields_ = [
        ("bounds_min", C.c_float * 3), ("bounds_size", C.c_float * 3),
        ("offset", C.c_float), ("strength", C.c_float), ("cone_length", C.c_float),
        ("shortest_edge", C.c_float), ("max_lod", C.c_float),
        ("steps", C.c_int32), ("early_exit", C.c_int32), ("border", C.c_int32), ("sat_scale", C.c_float),
    ]


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_reference=False)
        _lib = C.CDLL(ORACLE_SO)
        f = _lib
        f.p2vo_density_f32.argtypes = [C.c_void_p, C.c_int64, C.POINTER(_Grid), C.c_int, C.c_int, C.c_void_p]
        f.p2vo_density_f64.argtypes = [C.c_void_p, C.c_int64, C.POINTER(_Grid), C.c_int, C.c_int, C.c_void_p]
        f.p2vo_normalize_minmax_f32.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.POINTER(C.c_float),
                                                C.POINTER(C.c_float)]
        f.p2vo_mip_step_f64.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.c_void_p, C.POINTER(C.c_int32)]
        f.p2vo_cone_dirs.argtypes = [C.c_int, C.c_float, C.c_void_p]
        f.p2vo_cone_steps.argtypes = [C.POINTER(_ConeParams), C.c_float, C.c_void_p, C.c_void_p, C.c_int]
        f.p2vo_cone_steps.restype = C.c_int
        f.p2vo_cone_ao_f64.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_int32), C.c_int, C.c_void_p, C.c_int,
                                       C.POINTER(_ConeParams), C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        f.p2vo_gradient_normals_f32.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                                C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_void_p, C.c_int64,
                                                C.c_int, C.c_void_p]
        f.p2vo_mip_levels_f32.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.c_float, C.c_int,
                                          C.POINTER(C.c_void_p), C.c_int]
        f.p2vo_cone_ao_f32.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_int32), C.c_int, C.c_void_p, C.c_int,
                                       C.POINTER(_ConeParams), C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p]
        f.p2vo_aosphere_volume_ex_f64.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_int32),
                                                  C.c_float, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_void_p]
        f.p2vo_aosphere_volume_f64.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_int32),
                                               C.c_float, C.c_void_p]
        f.p2vo_aosphere_ao_f64.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_float), C.c_float,
                                           C.c_float, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p]
        f.p2vo_density_weighted_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int64, C.POINTER(_Grid), C.c_int,
                                                C.c_int, C.c_void_p]
        f.p2vo_density_weighted_f64.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int64, C.POINTER(_Grid), C.c_int,
                                                C.c_int, C.c_void_p]
        f.p2vo_vector_finish_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.POINTER(C.c_float),
                                             C.POINTER(C.c_float)]
        f.p2vo_mdao_dims.argtypes = [C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_float),
                                     C.POINTER(C.c_float)]
        f.p2vo_mdao_volume_f32.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_int32),
                                           C.c_int, C.c_void_p]
        f.p2vo_mdao_mip_u8.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.c_void_p, C.POINTER(C.c_int32)]
        f.p2vo_mlp_f64.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(C.c_double),
                                   C.c_void_p]
    return _lib


def _grid(bbox, res, cyclic, sigma) -> _Grid:
    g = _Grid()
    g.bbox[:] = [float(v) for v in bbox]
    g.res[:] = [int(v) for v in res]
    g.cyclic[:] = [int(bool(v)) for v in cyclic]
    g.sigma = float(sigma)
    return g


def _xyzr(xyzr) -> np.ndarray:
    a = np.ascontiguousarray(xyzr, dtype=np.float32)
    assert a.ndim == 2 and a.shape[1] == 4
    return a


def density_f32(xyzr, bbox, res, cyclic=(1, 1, 1), sigma=1.0, kernel=BUMP, nthreads=1) -> np.ndarray:
    """FP32 restatement of createVolumeCPU (raw sums, no normalisation); shape (z, y, x)."""
    a = _xyzr(xyzr)
    out = np.zeros((res[2], res[1], res[0]), np.float32)
    g = _grid(bbox, res, cyclic, sigma)
    rc = lib().p2vo_density_f32(a.ctypes.data, a.shape[0], C.byref(g), kernel, nthreads, out.ctypes.data)
    if rc:
        raise ValueError("invalid grid")
    return out


def density_f64(xyzr, bbox, res, cyclic=(1, 1, 1), sigma=1.0, kernel=BUMP, nthreads=1) -> np.ndarray:
    """FP64 restatement (the error reference); raw sums, shape (z, y, x)."""
    a = _xyzr(xyzr)
    out = np.zeros((res[2], res[1], res[0]), np.float64)
    g = _grid(bbox, res, cyclic, sigma)
    rc = lib().p2vo_density_f64(a.ctypes.data, a.shape[0], C.byref(g), kernel, nthreads, out.ctypes.data)
    if rc:
        raise ValueError("invalid grid")
    return out


def density_weighted(xyzr, w, bbox, res, cyclic=(1, 1, 1), sigma=1.0, kernel=BUMP, nthreads=1, fp64=False):
    """Weighted createVolumeCPU sums (the intensity aggregator with w of shape (n,), one direction component
    per column of w of shape (n, nc) for the vector aggregator); returns (z, y, x) or (z, y, x, nc)."""
    a = _xyzr(xyzr)
    wa = np.ascontiguousarray(w, np.float32)
    nc = 1 if wa.ndim == 1 else wa.shape[1]
    dt = np.float64 if fp64 else np.float32
    out = np.zeros((res[2], res[1], res[0], nc), dt)
    g = _grid(bbox, res, cyclic, sigma)
    fn = lib().p2vo_density_weighted_f64 if fp64 else lib().p2vo_density_weighted_f32
    if fn(a.ctypes.data, wa.ctypes.data, nc, a.shape[0], C.byref(g), kernel, nthreads, out.ctypes.data):
        raise ValueError("invalid grid")
    return out[..., 0] if nc == 1 else out


def vector_finish_f32(vol3: np.ndarray, weights: np.ndarray, normalize: bool):
    """The vector aggregator's finish in float (ParticlesToDensity.cpp:628-682); returns (volume, min, max)."""
    v = np.ascontiguousarray(vol3, np.float32).copy()
    w = np.ascontiguousarray(weights, np.float32)
    mn, mx = C.c_float(), C.c_float()
    lib().p2vo_vector_finish_f32(v.ctypes.data, w.ctypes.data, w.size, int(bool(normalize)), C.byref(mn), C.byref(mx))
    return v, mn.value, mx.value


def normalize_minmax_f32(vol: np.ndarray, apply: bool = True):
    """ParticlesToDensity.cpp:669-682 in float; returns (volume, min, max)."""
    v = np.ascontiguousarray(vol, dtype=np.float32).copy()
    mn, mx = C.c_float(), C.c_float()
    lib().p2vo_normalize_minmax_f32(v.ctypes.data, v.size, int(apply), C.byref(mn), C.byref(mx))
    return v, mn.value, mx.value


def normalize_f64(vol: np.ndarray, mode: str, n_particles: int = 0, spacing=(1.0, 1.0, 1.0)):
    """FP64 normalisation: 'minmax' as the reference, 'mass' scales so sum(v)*dV equals n_particles."""
    v = np.asarray(vol, np.float64)
    if mode == "minmax":
        mn, mx = v.min(), v.max()
        return (v - mn) / (mx - mn), mn, mx
    if mode == "mass":
        dv = float(spacing[0]) * float(spacing[1]) * float(spacing[2])
        s = v.sum(dtype=np.float64) * dv
        out = v * (n_particles / s) if s > 0 else v.copy()
        return out, out.min(), out.max()
    return v.copy(), v.min(), v.max()


def modify_bbox_f32(bbox, res):
    """ParticlesToDensity::modifyBBox (ParticlesToDensity.cpp:749-799) in FP32 numpy scalars, one rounding
    per C++ operation: grow the box by 1.1 plus two voxels in z, make voxels cubic by rewriting sizex and
    sizey, centre the grown box on the old one. Returns (bbox (6 floats), resolution (3 ints))."""
    f = np.float32
    sz = int(res[2])
    lo = [f(bbox[a]) for a in range(3)]
    hi = [f(bbox[a + 3]) for a in range(3)]
    rng = [abs(hi[a] - lo[a]) for a in range(3)]  # vislib Cuboid::Width/Height/Depth
    scale = f(1.1)
    spacing = (rng[2] * scale) / f(sz)
    depth = (rng[2] * scale) + f(2) * spacing
    spacing = depth / f(sz)

    def cubic(r):
        size = (r * scale) + f(2) * spacing
        q = size / spacing
        n = int(q)  # float -> int truncation
        rest = q - f(n)
        size = size + (f(1) - rest) * spacing
        return size, n + 1

    width, sx = cubic(rng[0])
    height, sy = cubic(rng[1])
    grown = (width, height, depth)
    out = [lo[a] - (grown[a] - rng[a]) / f(2) for a in range(3)] + \
          [hi[a] + (grown[a] - rng[a]) / f(2) for a in range(3)]
    return tuple(float(v) for v in out), (sx, sy, sz)


def spacing_f64(bbox, res):
    """Exact grid spacing of the reference grid, (right-left)/(res-1) per axis."""
    return tuple(abs(float(bbox[a + 3]) - float(bbox[a])) / (res[a] - 1) for a in range(3))


def mip_step_f64(src: np.ndarray) -> np.ndarray:
    """One MDAO mip level (mdao_mipmap_compute_main.comp.glsl:8-26); arrays shaped (z, y, x)."""
    s = np.ascontiguousarray(src, np.float64)
    sd = (C.c_int32 * 3)(s.shape[2], s.shape[1], s.shape[0])
    dd = (C.c_int32 * 3)(*[max(1, d // 2) for d in (s.shape[2], s.shape[1], s.shape[0])])
    out = np.zeros((dd[2], dd[1], dd[0]), np.float64)
    lib().p2vo_mip_step_f64(s.ctypes.data, sd, out.ctypes.data, dd)
    return out


# ------------------------------------------------------------------------------------------------
# The reference's own module (compiled from the MegaMol tree)
# ------------------------------------------------------------------------------------------------
class _RefList(C.Structure):
    _fields_ = [("vert_type", C.c_int), ("vert", C.c_void_p), ("vert_stride", C.c_uint32),
                ("global_radius", C.c_float), ("count", C.c_uint64), ("icol", C.c_void_p), ("dir", C.c_void_p),
                ("has_col", C.c_int), ("col_type", C.c_int), ("col", C.c_void_p), ("col_stride", C.c_uint32),
                ("global_colour", C.c_uint8 * 4)]


class _RefParams(C.Structure):
    _fields_ = [("aggregator", C.c_int), ("sizex", C.c_int), ("sizey", C.c_int), ("sizez", C.c_int),
                ("cyclX", C.c_int), ("cyclY", C.c_int), ("cyclZ", C.c_int), ("normalize", C.c_int),
                ("surface", C.c_int), ("sigma", C.c_float)]


class _RefResult(C.Structure):
    _fields_ = [("resolution", C.c_uint64 * 3), ("components", C.c_uint64), ("slice_dists", C.c_float * 3),
                ("origin", C.c_float * 3), ("extents", C.c_float * 3), ("min_value", C.c_double),
                ("max_value", C.c_double), ("millis", C.c_double), ("needed_floats", C.c_uint64)]


class _RefVGrid(C.Structure):
    _fields_ = [("count", C.c_uint64), ("info_cols", C.c_uint64), ("global_radius", C.c_float),
                ("col_min", C.c_float * 7), ("col_max", C.c_float * 7)]


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        if not reference_available():
            raise FileNotFoundError("the reference ParticlesToDensity build (oracle/_ref) is not present")
        _ref = C.CDLL(REF_SO)
        _ref.ref_p2d_run.argtypes = [C.POINTER(_RefList), C.c_int, C.POINTER(C.c_float), C.POINTER(_RefParams),
                                     C.c_void_p, C.c_uint64, C.POINTER(_RefResult)]
        _ref.ref_p2d_run.restype = C.c_int
        _ref.ref_p2d_run_vector.argtypes = [C.POINTER(_RefList), C.c_int, C.POINTER(C.c_float),
                                            C.POINTER(_RefParams), C.c_void_p, C.c_uint64, C.POINTER(_RefResult),
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64,
                                            C.POINTER(_RefVGrid)]
        _ref.ref_p2d_run_vector.restype = C.c_int
    return _ref


def _ref_lists(lists):
    keep = []
    arr = (_RefList * max(1, len(lists)))()
    for i, L in enumerate(lists):
        data = np.ascontiguousarray(L["data"])
        keep.append(data)
        icol = L.get("icol")
        dr = L.get("dir")
        if icol is not None:
            icol = np.ascontiguousarray(icol, np.float32)
            keep.append(icol)
        if dr is not None:
            dr = np.ascontiguousarray(dr, np.float32)
            keep.append(dr)
        # other colour types: "col_type", "col_offset" (bytes into each vertex record, the colour interleaved
        # with the vertex data) or a separate "col" array with "col_stride", and "global_colour"
        col_ptr, has_col = None, int("col_type" in L)
        if "col_offset" in L:
            col_ptr = data.ctypes.data + int(L["col_offset"])
        elif L.get("col") is not None:
            col = np.ascontiguousarray(L["col"])
            keep.append(col)
            col_ptr = col.ctypes.data
        gcol = (C.c_uint8 * 4)(*L.get("global_colour", (255, 255, 255, 255)))
        arr[i] = _RefList(int(L["type"]), data.ctypes.data, int(L.get("stride", 0)), float(L.get("radius", 0.5)),
                          int(L["count"]), icol.ctypes.data if icol is not None else None,
                          dr.ctypes.data if dr is not None else None, has_col, int(L.get("col_type", 0)), col_ptr,
                          int(L.get("col_stride", 0)), gcol)
    return arr, keep


def reference_density(lists, bbox, res, cyclic=(1, 1, 1), normalize=False, sigma=1.0, aggregator=0,
                      surface=False):
    """Run MegaMol's ParticlesToDensity once.

    ``lists`` is a sequence of dicts with keys ``type`` (VertexDataType), ``data`` (numpy array whose
    bytes are the vertex records), ``stride`` (bytes, 0 = packed), ``radius`` (global radius), ``count``
    and optionally ``icol`` / ``dir``. Returns (volume (z,y,x) float32, metadata dict).
    """
    arr, keep = _ref_lists(lists)
    prm = _RefParams(int(aggregator), int(res[0]), int(res[1]), int(res[2]), int(bool(cyclic[0])),
                     int(bool(cyclic[1])), int(bool(cyclic[2])), int(bool(normalize)), int(bool(surface)),
                     float(sigma))
    bb = (C.c_float * 6)(*[float(v) for v in bbox])
    res_out = _RefResult()
    comps = 3 if aggregator == 2 else 1
    cap = int(res[0]) * int(res[1]) * int(res[2]) * comps
    out = np.zeros(cap, np.float32)
    rc = ref().ref_p2d_run(arr, len(lists), bb, C.byref(prm), out.ctypes.data, cap, C.byref(res_out))
    if rc == 2:
        cap = int(res_out.needed_floats)
        out = np.zeros(cap, np.float32)
        rc = ref().ref_p2d_run(arr, len(lists), bb, C.byref(prm), out.ctypes.data, cap, C.byref(res_out))
    if rc != 0:
        raise RuntimeError(f"reference ParticlesToDensity failed (rc={rc})")
    r = [int(v) for v in res_out.resolution]
    comps = int(res_out.components)
    n = r[0] * r[1] * r[2] * comps
    vol = out[:n].reshape((r[2], r[1], r[0]) if comps == 1 else (r[2], r[1], r[0], comps))
    meta = dict(resolution=r, components=comps, slice_dists=list(res_out.slice_dists), origin=list(res_out.origin),
                extents=list(res_out.extents), min_value=res_out.min_value, max_value=res_out.max_value,
                millis=res_out.millis)
    return vol, meta


REF_DATRAW_SO = os.path.join(os.path.dirname(REF_SO), "libref_datraw.so")


def reference_write_datraw(prefix, frame, volume, resolution, components, slice_dists, origin, frame_count=1):
    """Run MegaMol's own volume::DatRawWriter (oracle/_ref/libref_datraw.so) on a float volume; returns
    True when the module reported success."""
    lib_ = C.CDLL(REF_DATRAW_SO)
    lib_.ref_datraw_write.argtypes = [C.c_char_p, C.c_uint, C.c_uint, C.POINTER(C.c_uint64), C.c_uint64, C.c_int,
                                      C.c_uint64, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_void_p]
    lib_.ref_datraw_write.restype = C.c_int
    v = np.ascontiguousarray(volume, np.float32)
    res = (C.c_uint64 * 3)(*[int(x) for x in resolution])
    sd = (C.c_float * 3)(*[float(x) for x in slice_dists])
    org = (C.c_float * 3)(*[float(x) for x in origin])
    # ScalarType_t FLOATING_POINT = 3, GridType_t CARTESIAN = 1 (VolumetricDataCallTypes.h:16-19)
    return lib_.ref_datraw_write(prefix.encode(), int(frame), int(frame_count), res, int(components), 3, 4, 1, sd,
                                 org, v.ctypes.data) == 0


REF_MMPLD_SO = os.path.join(os.path.dirname(REF_SO), "libref_mmpld.so")
# record bytes of SimpleSphericalParticles' vertex and colour types (SimpleSphericalParticles.h:28-50)
VERTEX_RECORD_BYTES = {0: 0, 1: 12, 2: 16, 3: 6, 4: 24}
COLOUR_RECORD_BYTES = {0: 0, 1: 3, 2: 4, 3: 12, 4: 16, 5: 4, 6: 8, 7: 8}


class _RefMmpldList(C.Structure):
    _fields_ = [("vert_type", C.c_int32), ("col_type", C.c_int32), ("count", C.c_uint64),
                ("global_radius", C.c_float), ("global_colour", C.c_uint8 * 4), ("col_min", C.c_float),
                ("col_max", C.c_float), ("vert_stride", C.c_uint32), ("col_stride", C.c_uint32),
                ("bbox", C.c_float * 6), ("clusters", C.c_uint32), ("cluster_bytes", C.c_uint64)]


class _RefMmpldExtent(C.Structure):
    _fields_ = [("frames", C.c_uint32), ("bbox", C.c_float * 6), ("clipbox", C.c_float * 6)]


def reference_mmpld(path, max_lists: int = 256) -> dict:
    """Read an MMPLD file with MegaMol's own MMPLDDataSource (oracle/_ref/libref_mmpld.so): the extent it
    publishes (frames, bbox, clipbox) and, for every frame, the lists of the MultiParticleDataCall as dicts
    (types, count, global radius / colour, colour map range, strides, list box, cluster infos, and the packed
    vertex and colour records as uint8 arrays)."""
    lib_ = C.CDLL(REF_MMPLD_SO)
    lib_.ref_mmpld_open.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), C.POINTER(_RefMmpldExtent)]
    lib_.ref_mmpld_frame.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(_RefMmpldList), C.c_uint32,
                                     C.POINTER(C.c_uint32)]
    lib_.ref_mmpld_list_data.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]
    lib_.ref_mmpld_close.argtypes = [C.c_void_p]
    h, ext = C.c_void_p(), _RefMmpldExtent()
    if lib_.ref_mmpld_open(os.fsencode(str(path)), C.byref(h), C.byref(ext)) != 0:
        lib_.ref_mmpld_close(h)
        raise RuntimeError("reference MMPLDDataSource: GetExtent failed")
    out = dict(frames=int(ext.frames), bbox=list(ext.bbox), clipbox=list(ext.clipbox), frame_lists=[])
    try:
        arr = (_RefMmpldList * max_lists)()
        for fi in range(out["frames"]):
            n = C.c_uint32()
            if lib_.ref_mmpld_frame(h, fi, arr, max_lists, C.byref(n)) != 0:
                raise RuntimeError(f"reference MMPLDDataSource: GetData failed on frame {fi}")
            lists = []
            for i in range(min(n.value, max_lists)):
                L = arr[i]
                vb, cb = VERTEX_RECORD_BYTES.get(L.vert_type, 0), COLOUR_RECORD_BYTES.get(L.col_type, 0)
                vert = np.zeros(vb * L.count, np.uint8)
                col = np.zeros(cb * L.count, np.uint8)
                lib_.ref_mmpld_list_data(h, i, vb, vert.ctypes.data if vb else None, cb,
                                         col.ctypes.data if cb else None)
                lists.append(dict(vert_type=L.vert_type, col_type=L.col_type, count=int(L.count),
                                  global_radius=float(L.global_radius), global_colour=tuple(L.global_colour),
                                  col_min=float(L.col_min), col_max=float(L.col_max), vert_stride=int(L.vert_stride),
                                  col_stride=int(L.col_stride), bbox=list(L.bbox), clusters=int(L.clusters),
                                  cluster_bytes=int(L.cluster_bytes), vertex=vert, colour=col))
            out["frame_lists"].append(lists)
    finally:
        lib_.ref_mmpld_close(h)
    return out


def reference_vector_grid(lists, bbox, res, cyclic=(1, 1, 1), normalize=False, sigma=1.0):
    """The vector aggregator's outParticles and outInfo outputs of MegaMol's ParticlesToDensity
    (ParticlesToDensity.cpp:306-380, 628-727): dict with positions (n, 3), directions (n, 3), colours (n,),
    info (n, 7), global_radius, col_min / col_max (7 each), and the volume."""
    arr, keep = _ref_lists(lists)
    prm = _RefParams(2, int(res[0]), int(res[1]), int(res[2]), int(bool(cyclic[0])), int(bool(cyclic[1])),
                     int(bool(cyclic[2])), int(bool(normalize)), 0, float(sigma))
    bb = (C.c_float * 6)(*[float(v) for v in bbox])
    res_out, vg = _RefResult(), _RefVGrid()
    V = int(res[0]) * int(res[1]) * int(res[2])
    vol = np.zeros(3 * V, np.float32)
    pos, dr, col, info = (np.zeros(3 * V, np.float32), np.zeros(3 * V, np.float32), np.zeros(V, np.float32),
                          np.zeros(7 * V, np.float32))
    rc = ref().ref_p2d_run_vector(arr, len(lists), bb, C.byref(prm), vol.ctypes.data, vol.size, C.byref(res_out),
                                  pos.ctypes.data, dr.ctypes.data, col.ctypes.data, info.ctypes.data, V,
                                  C.byref(vg))
    if rc != 0:
        raise RuntimeError(f"reference ParticlesToDensity failed (rc={rc})")
    n = int(vg.count)
    return dict(volume=vol.reshape(int(res[2]), int(res[1]), int(res[0]), 3), count=n,
                positions=pos[:3 * n].reshape(n, 3), directions=dr[:3 * n].reshape(n, 3), colours=col[:n],
                info=info[:7 * n].reshape(n, 7), global_radius=float(vg.global_radius),
                col_min=np.array(vg.col_min[:], np.float32), col_max=np.array(vg.col_max[:], np.float32),
                min_value=res_out.min_value, max_value=res_out.max_value)


def vector_grid_f32(v3, bbox, res, normalize):
    """The vector aggregator's compacted grid (ParticlesToDensity.cpp:436-456, 628-668, 685-727) from the
    finished, not normalised direction volume v3 (z, y, x, 3) in float32: per node the position
    min + h * x, the density |v|, the unit direction v / |v| (0 where |v| = 0) and the colour
    (|v| - min) / (max - min); the nodes with |v| > 0 sorted by |v| descending, equal densities in node
    order (a stable sort); info rows (position, direction, colour if normalize else |v|). numpy float32
    arithmetic rounds every operation as the reference's float code does."""
    f = np.float32
    v = np.ascontiguousarray(v3, f).reshape(-1, 3)
    d = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
    with np.errstate(invalid="ignore", divide="ignore"):
        dirs = np.where(d[:, None] == 0, f(0), v / np.where(d == 0, f(1), d)[:, None]).astype(f)
    mx = max(f(0), d.max()) if d.size else f(0)
    mn = min(f(np.finfo(f).max), d.min()) if d.size else f(np.finfo(f).max)
    with np.errstate(invalid="ignore", divide="ignore"):
        col = ((d - mn) / (mx - mn)).astype(f)
    h = [f(abs(f(bbox[a + 3]) - f(bbox[a]))) / f(res[a] - 1) for a in range(3)]
    z, y, x = np.meshgrid(np.arange(res[2]), np.arange(res[1]), np.arange(res[0]), indexing="ij")
    pos = np.stack([f(bbox[0]) + h[0] * x.ravel().astype(f), f(bbox[1]) + h[1] * y.ravel().astype(f),
                    f(bbox[2]) + h[2] * z.ravel().astype(f)], axis=1).astype(f)
    order = np.argsort(-d, kind="stable")
    n = int(np.count_nonzero(d != 0))
    order = order[:n]
    info = np.column_stack([pos[order], dirs[order], col[order] if normalize else d[order]]).astype(f)
    return dict(count=n, positions=pos[order], directions=dirs[order], colours=col[order], info=info,
                order=order, min=mn, max=mx,
                global_radius=f(f(abs(f(bbox[3]) - f(bbox[0]))) / f(res[0])) / f(5))


# ------------------------------------------------------------------------------------------------
# AO restatements
# ------------------------------------------------------------------------------------------------
def cone_dirs(k: int, apex_rad: float) -> np.ndarray:
    out = np.zeros((k, 4), np.float32)
    lib().p2vo_cone_dirs(k, float(apex_rad), out.ctypes.data)
    return out


def _cone_params(bounds_min, bounds_size, offset=0.01, strength=1.0, cone_length=0.8, shortest_edge=128.0,
                 max_lod=6.0, steps=0, early_exit=1, border=0, sat_scale=0.0) -> _ConeParams:
    cp = _ConeParams()
    cp.bounds_min[:] = [float(v) for v in bounds_min]
    cp.bounds_size[:] = [float(v) for v in bounds_size]
    cp.offset, cp.strength, cp.cone_length = float(offset), float(strength), float(cone_length)
    cp.shortest_edge, cp.max_lod = float(shortest_edge), float(max_lod)
    cp.steps, cp.early_exit, cp.border, cp.sat_scale = int(steps), int(early_exit), int(border), float(sat_scale)
    return cp


def cone_steps(w: float, **kw):
    cp = _cone_params((0, 0, 0), (1, 1, 1), **kw)
    t = np.zeros(1024, np.float32)
    lod = np.zeros(1024, np.float32)
    n = lib().p2vo_cone_steps(C.byref(cp), float(w), t.ctypes.data, lod.ctypes.data, 1024)
    return t[:n], lod[:n]


def mip_chain_f64(l0: np.ndarray, nlevels: int, sat_scale: float = 0.0):
    """Levels 0..nlevels-1 of the MDAO pyramid. Level 0 is returned raw (cone_ao_f64 saturates it with
    the same sat_scale); level 1 is built from the saturated texels clamp(v*scale, 0, 1)."""
    raw = np.asarray(l0, np.float64)
    base = np.clip(raw * sat_scale, 0.0, 1.0) if sat_scale > 0 else raw
    levels = [raw]
    cur = base
    for _ in range(1, nlevels):
        cur = mip_step_f64(cur)
        levels.append(cur)
    return levels


def cone_ao_f64(levels, dirs, xyzr, normals, bounds_min, bounds_size, **kw) -> np.ndarray:
    """Cone-marched AO per particle (FP64). `levels` are (z, y, x) arrays; level 0 raw (the kernel applies
    sat_scale to it), the others as mip_chain_f64 builds them."""
    lv = [np.ascontiguousarray(L, np.float64) for L in levels]
    ptrs = (C.c_void_p * len(lv))(*[L.ctypes.data for L in lv])
    dims = (C.c_int32 * (3 * len(lv)))(*[d for L in lv for d in (L.shape[2], L.shape[1], L.shape[0])])
    d = np.ascontiguousarray(dirs, np.float32)
    x = _xyzr(xyzr)
    nrm = np.ascontiguousarray(normals, np.float32)
    out = np.zeros(x.shape[0], np.float64)
    cp = _cone_params(bounds_min, bounds_size, **kw)
    lib().p2vo_cone_ao_f64(ptrs, dims, len(lv), d.ctypes.data, d.shape[0], C.byref(cp), x.ctypes.data,
                           nrm.ctypes.data, x.shape[0], out.ctypes.data)
    return out


def gradient_normals_f32(grid, bbox, res, xyzr, cyclic=(1, 1, 1), nthreads: int = 1) -> np.ndarray:
    """The library's P2V_NORMALS_GRADIENT normals restated in FP32 (OpenMP): unit vectors down the density
    gradient of the node grid (z, y, x) at each particle, (n, 3) float32; zero where the gradient vanishes. The
    node origin is the box minimum and the spacing the reference's float(|max - min|) / float(res - 1)."""
    g = np.ascontiguousarray(grid, np.float32)
    x = _xyzr(xyzr)
    f = np.float32
    h = [f(abs(f(bbox[a + 3]) - f(bbox[a]))) / f(res[a] - 1) for a in range(3)]
    out = np.zeros((x.shape[0], 3), np.float32)
    lib().p2vo_gradient_normals_f32(g.ctypes.data, (C.c_int32 * 3)(*[int(r) for r in res]),
                                    (C.c_int32 * 3)(*[int(c) for c in cyclic]),
                                    (C.c_float * 3)(*[float(bbox[a]) for a in range(3)]),
                                    (C.c_float * 3)(*[float(v) for v in h]), x.ctypes.data, x.shape[0],
                                    int(nthreads), out.ctypes.data)
    return out


def mip_levels_f32(l0: np.ndarray, nlevels: int, sat_scale: float = 0.0, nthreads: int = 1):
    """Levels 0..nlevels-1 of the MDAO pyramid in FP32 with OpenMP (level 0 returned as given; level 1 built
    from clamp(v * sat_scale, 0, 1) when sat_scale > 0). Arrays (z, y, x) float32."""
    src = np.ascontiguousarray(l0, np.float32)
    d = list(src.shape[::-1])
    outs = []
    for _ in range(1, nlevels):
        d = [max(1, v // 2) for v in d]
        outs.append(np.empty(d[::-1], np.float32))
    ptrs = (C.c_void_p * max(1, len(outs)))(*[o.ctypes.data for o in outs])
    d0 = (C.c_int32 * 3)(*src.shape[::-1])
    lib().p2vo_mip_levels_f32(src.ctypes.data, d0, float(sat_scale), int(nlevels), ptrs, int(nthreads))
    return [src] + outs


def cone_ao_f32(levels, dirs, xyzr, normals, bounds_min, bounds_size, nthreads: int = 1, **kw) -> np.ndarray:
    """Cone-marched AO per particle in FP32 with OpenMP, the GPU kernel's operation order (the CPU baseline's
    timing stand-in; the error reference is cone_ao_f64). `levels` as mip_levels_f32 returns them."""
    lv = [np.ascontiguousarray(L, np.float32) for L in levels]
    ptrs = (C.c_void_p * len(lv))(*[L.ctypes.data for L in lv])
    dims = (C.c_int32 * (3 * len(lv)))(*[d for L in lv for d in (L.shape[2], L.shape[1], L.shape[0])])
    d = np.ascontiguousarray(dirs, np.float32)
    x = _xyzr(xyzr)
    nrm = np.ascontiguousarray(normals, np.float32)
    out = np.zeros(x.shape[0], np.float32)
    cp = _cone_params(bounds_min, bounds_size, **kw)
    lib().p2vo_cone_ao_f32(ptrs, dims, len(lv), d.ctypes.data, d.shape[0], C.byref(cp), x.ctypes.data,
                           nrm.ctypes.data, x.shape[0], int(nthreads), out.ctypes.data)
    return out


def aosphere_volume_f64(xyzr, clip, s, gen_fac=1.0, glsl_rule=0, clip_plane=None) -> np.ndarray:
    """AOSphere volume (FP64 sums; voxel decisions in float as the reference): the CPU rule of createVolumeCPU
    (with the clip-plane discard when clip_plane = (nx, ny, nz, d) is given) or the GLSL rule of
    createVolumeGLSL (glsl_rule=1)."""
    x = _xyzr(xyzr)
    tex = np.zeros((s[2], s[1], s[0]), np.float64)
    cl = (C.c_float * 6)(*[float(v) for v in clip])
    ss = (C.c_int32 * 3)(*[int(v) for v in s])
    pl = (C.c_float * 4)(*([float(v) for v in clip_plane] if clip_plane is not None else [0.0] * 4))
    lib().p2vo_aosphere_volume_ex_f64(x.ctypes.data, x.shape[0], cl, ss, float(gen_fac), int(glsl_rule),
                                      int(clip_plane is not None), pl, tex.ctypes.data)
    return tex


def aosphere_ao_f64(tex, clip, xyzr, normals, mode=0, step_len=0.5, eval_fac=1.0) -> np.ndarray:
    t = np.ascontiguousarray(tex, np.float64)
    x = _xyzr(xyzr)
    nrm = np.ascontiguousarray(normals, np.float32)
    out = np.zeros(x.shape[0], np.float64)
    cl = (C.c_float * 6)(*[float(v) for v in clip])
    ss = (C.c_int32 * 3)(t.shape[2], t.shape[1], t.shape[0])
    lib().p2vo_aosphere_ao_f64(t.ctypes.data, ss, cl, float(step_len), float(eval_fac), x.ctypes.data, nrm.ctypes.data,
                               x.shape[0], int(mode), out.ctypes.data)
    return out


MLP_IN, MLP_HIDDEN = 54, 64
MLP_CONES, MLP_FSTEPS = 8, 6


def mlp_feature_steps(nsteps: int, fsteps: int = MLP_FSTEPS) -> list[int]:
    """March steps the learned AO's features sample: step round(j (nsteps - 1) / (fsteps - 1)) for feature j."""
    return [int(np.floor(j * (nsteps - 1) / (fsteps - 1) + 0.5)) for j in range(fsteps)]


def _linear_border(T, q):
    """GL LINEAR sample (texel centres (i + 0.5) / N, CLAMP_TO_BORDER with 0) of texels T (z, y, x) at
    normalised points q (n, 3), FP64."""
    dz, dy, dx = T.shape
    c = q * np.array([dx, dy, dz], np.float64) - 0.5
    i0 = np.floor(c).astype(np.int64)
    f = c - i0
    out = np.zeros(q.shape[0], np.float64)
    for oz in (0, 1):
        for oy in (0, 1):
            for ox in (0, 1):
                ix, iy, iz = i0[:, 0] + ox, i0[:, 1] + oy, i0[:, 2] + oz
                ok = (ix >= 0) & (ix < dx) & (iy >= 0) & (iy < dy) & (iz >= 0) & (iz < dz)
                v = np.where(ok, T[np.clip(iz, 0, dz - 1), np.clip(iy, 0, dy - 1), np.clip(ix, 0, dx - 1)], 0.0)
                out += v * (f[:, 0] if ox else 1 - f[:, 0]) * (f[:, 1] if oy else 1 - f[:, 1]) * \
                    (f[:, 2] if oz else 1 - f[:, 2])
    return out


def cone_features_f64(levels, dirs, t, lod, xyzr, normals, bounds_min, inv_size) -> np.ndarray:
    """The learned AO's input features, FP64: for each cone (dirs, around +Y), in the MDAO cone frame of the
    surface point x = p + r n (mdao_deferred_fragment_ambocc.inc.glsl:18-21: y = n, x = cross(n, normalize(x)),
    z = cross(x, y)), the texels `levels` (z, y, x; as the sampler sees them, level 0 already saturated) at the
    feature steps of the step table (t, lod), LINEAR within and between the two levels around each lod; then
    the unit normal and x in normalised volume coordinates. Returns (n, cones * MLP_FSTEPS + 6)."""
    p = np.asarray(xyzr, np.float64).reshape(-1, 4)
    n = np.asarray(normals, np.float64).reshape(-1, 3)
    n = n / np.linalg.norm(n, axis=1, keepdims=True)
    x = p[:, :3] + p[:, 3:4] * n
    u = (x - np.asarray(bounds_min, np.float64)) * np.asarray(inv_size, np.float64)
    xn = x / np.linalg.norm(x, axis=1, keepdims=True)
    ex = np.cross(n, xn)
    ez = np.cross(ex, n)
    L = len(levels)
    cols = []
    for d in np.asarray(dirs, np.float64):
        dv = ex * d[0] + n * d[1] + ez * d[2]
        for k in mlp_feature_steps(len(t)):
            q = u + float(t[k]) * dv
            l0 = min(int(lod[k]), L - 1)
            fr = float(lod[k]) - l0
            v = _linear_border(levels[l0], q)
            if fr > 0 and l0 + 1 < L:
                v = (1 - fr) * v + fr * _linear_border(levels[l0 + 1], q)
            cols.append(v)
    return np.column_stack(cols + [n, u])
MLP_NPARAM = MLP_HIDDEN * MLP_IN + MLP_HIDDEN + MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN + MLP_HIDDEN + 1


def bin_keys(xyzr, bbox, res) -> tuple[np.ndarray, int]:
    """Bin key of every particle (numpy restatement in FP32, the reference's cell expression of
    ParticlesToDensity.cpp:561-568: cell = (p - min) / h with h = |max - min| / (res - 1) in float). The bin is
    floor(cell) clamped to [-1, res] per axis (one underflow and one overflow bin), key =
    (bz * (sy + 2) + by) * (sx + 2) + bx with b = bin + 1; particles with non-finite coordinates or radius,
    radius <= 0 or a cell beyond 2^30 get key nbins. Returns (keys, nbins)."""
    x = np.asarray(xyzr, np.float32).reshape(-1, 4)
    nb = [int(r) + 2 for r in res]
    nbins = nb[0] * nb[1] * nb[2]
    valid = np.isfinite(x).all(1) & (x[:, 3] > 0)
    b = []
    with np.errstate(invalid="ignore", over="ignore"):
        for a in range(3):
            lo, hi = np.float32(bbox[a]), np.float32(bbox[a + 3])
            h = np.float32(abs(hi - lo)) / np.float32(res[a] - 1)
            q = (x[:, a] - lo) / h
            valid &= np.abs(q) < np.float32(2.0 ** 30)
            c = np.floor(np.where(np.isfinite(q), q, 0.0)).astype(np.int64)
            b.append(np.clip(c, -1, int(res[a])) + 1)
    keys = (b[2] * nb[1] + b[1]) * nb[0] + b[0]
    keys = np.where(valid, keys, nbins).astype(np.uint32)
    return keys, nbins


def support_misses_nodes_f64(xyzr, bbox, res, sigma=1.0, kernel=0) -> np.ndarray:
    """Particles whose kernel support (radius sigma r, bump, or 3 sigma r, Gaussian) holds no grid node along
    some axis, in FP64 without margin: nodes at bbox min + k h, h = |max - min| / (res - 1). The library's
    radix binning sorts such particles after all others (it flags them with a margin, so every particle it
    flags is one of these)."""
    x = np.asarray(xyzr, np.float64).reshape(-1, 4)
    eps = (1.0 if kernel == 0 else 3.0) * sigma * x[:, 3]
    miss = np.zeros(x.shape[0], bool)
    with np.errstate(invalid="ignore"):
        for a in range(3):
            lo, hi = float(bbox[a]), float(bbox[a + 3])
            h = abs(hi - lo) / (res[a] - 1)
            q = (x[:, a] - lo) / h
            phi = q - np.floor(q)
            eh = eps / h
            miss |= (phi > eh) & (1.0 - phi > eh)
    return miss


def binning(xyzr, bbox, res):
    """Stable sort of the bin keys (np.argsort kind="stable"): (sorted keys, permutation, cell starts of the
    nbins + 1 bins)."""
    keys, nbins = bin_keys(xyzr, bbox, res)
    order = np.argsort(keys, kind="stable").astype(np.uint32)
    sk = keys[order]
    start = np.searchsorted(sk, np.arange(nbins + 1, dtype=np.int64), side="left").astype(np.uint32)
    return sk, order, start


def mdao_dims(clip, vol_size: int):
    """MDAO volume size for a clip box: (dims (x, y, z), shortest edge, max lod)."""
    c = (C.c_float * 6)(*[float(v) for v in clip])
    d = (C.c_int32 * 3)()
    sh, ml = C.c_float(), C.c_float()
    lib().p2vo_mdao_dims(c, int(vol_size), d, C.byref(sh), C.byref(ml))
    return (int(d[0]), int(d[1]), int(d[2])), float(sh.value), float(ml.value)


def mdao_volume_f32(xyzr, clip, dims, unorm8: bool = True) -> np.ndarray:
    """MDAO occupancy volume, (z, y, x) float32: k/255 per voxel (unorm8) or min(1, sum of fractions)."""
    x = _xyzr(xyzr)
    c = (C.c_float * 6)(*[float(v) for v in clip])
    d = (C.c_int32 * 3)(*[int(v) for v in dims])
    out = np.zeros((dims[2], dims[1], dims[0]), np.float32)
    lib().p2vo_mdao_volume_f32(x.ctypes.data, x.shape[0], c, d, int(bool(unorm8)), out.ctypes.data)
    return out


def mdao_mip_u8(src: np.ndarray) -> np.ndarray:
    """One R8 mip step (integer /8 rule, rounded half up) of a (z, y, x) float32 volume of k/255 values."""
    s = np.ascontiguousarray(src, np.float32)
    sd = (C.c_int32 * 3)(s.shape[2], s.shape[1], s.shape[0])
    dd = (C.c_int32 * 3)(max(1, s.shape[2] // 2), max(1, s.shape[1] // 2), max(1, s.shape[0] // 2))
    out = np.zeros((dd[2], dd[1], dd[0]), np.float32)
    lib().p2vo_mdao_mip_u8(s.ctypes.data, sd, out.ctypes.data, dd)
    return out


def mlp_f64(params, x, t=None, grads=True):
    """FP64 forward (+ backward) of the learned-AO MLP; returns (loss, y, grads)."""
    p = np.ascontiguousarray(params, np.float64)
    assert p.size == MLP_NPARAM
    xx = np.ascontiguousarray(x, np.float32)
    n = xx.shape[0]
    tt = np.ascontiguousarray(t, np.float32) if t is not None else None
    y = np.zeros(n, np.float64)
    g = np.zeros(MLP_NPARAM, np.float64) if grads else None
    loss = C.c_double()
    lib().p2vo_mlp_f64(p.ctypes.data, xx.ctypes.data, tt.ctypes.data if tt is not None else None, n,
                       g.ctypes.data if g is not None else None, C.byref(loss), y.ctypes.data)
    return loss.value, y, g
