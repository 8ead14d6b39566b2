"""Python binding of libp2v (ctypes over the C ABI in include/p2v.h) and a host-side mirror of MegaMol's
``datatools::ParticlesToDensity`` module.

``ParticlesToDensity`` keeps the reference module's parameter names and meaning
(plugins/datatools/src/ParticlesToDensity.cpp:59-152): ``aggregator``, ``sizex``/``sizey``/``sizez``,
``cyclX``/``cyclY``/``cyclZ``, ``normalize``, ``sigma``, ``forSurfaceReconstruction``; ``get_data`` plays
the role of the VolumetricDataCall GET_DATA callback (:210-304) and returns the volume together with the
VolumetricMetadata_t fields the module publishes. Errors surface as ``P2VError`` (the reference returns
false and logs; there is no silent fallback: without the compiled library or a GPU the calls raise).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Any, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libp2v.so")

# enums of include/p2v.h
OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, EDOMAIN, EUNSUPPORTED = range(7)
VERTDATA_NONE, VERTDATA_FLOAT_XYZ, VERTDATA_FLOAT_XYZR, VERTDATA_SHORT_XYZ, VERTDATA_DOUBLE_XYZ = range(5)
(COLDATA_NONE, COLDATA_UINT8_RGB, COLDATA_UINT8_RGBA, COLDATA_FLOAT_RGB, COLDATA_FLOAT_RGBA, COLDATA_FLOAT_I,
 COLDATA_USHORT_RGBA, COLDATA_DOUBLE_I) = range(8)
MEM_HOST, MEM_DEVICE = 0, 1
KERNEL_BUMP, KERNEL_GAUSS3 = 0, 1
ACCUM_EXACT, ACCUM_KAHAN = 0, 1
AO_NONE, AO_CONE, AO_AOSPHERE_AXES, AO_AOSPHERE_NORMAL, AO_LEARNED = range(5)
AOVOL_DENSITY, AOVOL_MDAO = 0, 1
AOS_DEPOSIT_CPU, AOS_DEPOSIT_GLSL = 0, 1
NORMALS_LIST, NORMALS_GRADIENT = 0, 1
AO_MARCH_THREAD, AO_MARCH_WARP = 0, 1
STATUS_NAMES = {0: "P2V_OK", 1: "P2V_EINVAL", 2: "P2V_ENOMEM", 3: "P2V_ECUDA", 4: "P2V_ETIMEOUT", 5: "P2V_EDOMAIN",
                6: "P2V_EUNSUPPORTED"}


class P2VError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Params(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("aggregator", C.c_int32), ("sizex", C.c_int32), ("sizey", C.c_int32), ("sizez", C.c_int32),
        ("cyclX", C.c_int32), ("cyclY", C.c_int32), ("cyclZ", C.c_int32), ("normalize", C.c_int32),
        ("sigma", C.c_float), ("forSurfaceReconstruction", C.c_int32),
        ("kernel", C.c_int32), ("mass_normalize", C.c_int32), ("accumulate", C.c_int32),
        ("ao_mode", C.c_int32), ("ao_volume", C.c_int32), ("ao_volume_scale", C.c_float), ("ao_cones", C.c_int32),
        ("ao_steps", C.c_int32), ("ao_levels", C.c_int32), ("ao_apex_deg", C.c_float), ("ao_offset", C.c_float),
        ("ao_strength", C.c_float), ("ao_cone_length", C.c_float), ("ao_early_exit", C.c_int32),
        ("mdao_volume_size", C.c_int32), ("mdao_unorm8", C.c_int32),
        ("aos_sizex", C.c_int32), ("aos_sizey", C.c_int32), ("aos_sizez", C.c_int32),
        ("aos_step_len", C.c_float), ("aos_gen_fac", C.c_float), ("aos_eval_fac", C.c_float),
        ("tile_x", C.c_int32), ("tile_y", C.c_int32), ("tile_z", C.c_int32),
        ("batch_lanes", C.c_int32), ("batch_graph", C.c_int32), ("vector_grid", C.c_int32),
        ("aos_deposit", C.c_int32), ("aos_clip", C.c_int32), ("aos_clip_plane", C.c_float * 4),
        ("ao_normals", C.c_int32), ("mma_wait_polls", C.c_int32), ("test_hold_mma", C.c_int32),
        ("slab_z0", C.c_int32), ("slab_z1", C.c_int32),
        ("batch_persistent", C.c_int32), ("queue_wait_polls", C.c_int32), ("test_hold_queue", C.c_int32),
        ("sort_wait_polls", C.c_int32), ("test_hold_sort", C.c_int32), ("ao_march", C.c_int32),
        ("ao_brick_order", C.c_int32),
    ]


class ParticleListC(C.Structure):
    _fields_ = [("vertex_type", C.c_int32), ("vertex_stride", C.c_uint32), ("vertex_data", C.c_void_p),
                ("count", C.c_uint64), ("global_radius", C.c_float), ("mem", C.c_int32),
                ("normals", C.c_void_p), ("normal_stride", C.c_uint32), ("ao_out", C.c_void_p),
                ("colour_type", C.c_int32), ("colour_stride", C.c_uint32), ("colour_data", C.c_void_p),
                ("global_colour", C.c_uint8 * 4)]


class MmpldInfoC(C.Structure):
    _fields_ = [("version", C.c_uint32), ("frames", C.c_uint32), ("bbox", C.c_float * 6),
                ("clipbox", C.c_float * 6)]


class MmpldListInfoC(C.Structure):
    _fields_ = [("intensity_range", C.c_float * 2), ("bbox", C.c_float * 6), ("clusters", C.c_uint32)]


class FrameC(C.Structure):
    _fields_ = [("bbox", C.c_float * 6), ("clipbox", C.c_float * 6), ("frame_id", C.c_uint32),
                ("list_count", C.c_uint32), ("lists", C.POINTER(ParticleListC))]


class VectorGridInfoC(C.Structure):
    _fields_ = [("count", C.c_uint64), ("global_radius", C.c_float), ("col_min", C.c_float * 7),
                ("col_max", C.c_float * 7)]


class BatchItemC(C.Structure):
    _fields_ = [("frame", C.c_void_p), ("volume", C.c_void_p), ("size", C.c_int32 * 3)]


TUNE_MAX = 32
NOALLOC_MAX_VOXELS = 262144  # P2V_NOALLOC_MAX_VOXELS: voxels of p2v_aosphere_ao_noalloc's static scratch


class TuneReportC(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("tile", C.c_int32 * 3), ("lanes", C.c_int32), ("ms_best", C.c_float),
                ("candidates", C.c_int32), ("cand_tile", (C.c_int32 * 3) * TUNE_MAX),
                ("cand_lanes", C.c_int32 * TUNE_MAX), ("cand_ms", C.c_float * TUNE_MAX),
                ("persistent", C.c_int32), ("cand_persistent", C.c_int32 * TUNE_MAX)]


class VolumeC(C.Structure):
    _fields_ = [("data", C.c_void_p), ("mem", C.c_int32), ("capacity", C.c_uint64),
                ("resolution", C.c_uint64 * 3), ("components", C.c_uint64), ("slice_dists", C.c_float * 3),
                ("origin", C.c_float * 3), ("extents", C.c_float * 3), ("min_value", C.c_double),
                ("max_value", C.c_double), ("bbox", C.c_float * 6), ("data_hash", C.c_uint64)]


class StatsC(C.Structure):
    _fields_ = [("particles_in", C.c_uint64), ("particles_binned", C.c_uint64), ("particles_dropped", C.c_uint64),
                ("radius_max", C.c_float), ("cell_min", C.c_int32 * 3), ("cell_max", C.c_int32 * 3),
                ("mass_sum", C.c_double), ("ms_upload", C.c_double), ("ms_binning", C.c_double),
                ("ms_density", C.c_double), ("ms_normalize", C.c_double), ("ms_ao", C.c_double),
                ("ms_download", C.c_double), ("ms_total", C.c_double), ("device_error", C.c_uint32),
                ("ao_fallback", C.c_uint32), ("cell_max_count", C.c_uint32), ("ao_fetches", C.c_uint32),
                ("ms_ao_kernel", C.c_double)]


class TrainParams(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float),
                ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float), ("lr_decay", C.c_float),
                ("val_fraction", C.c_float), ("range_margin", C.c_float), ("seed", C.c_uint64)]


class TrainReport(C.Structure):
    _fields_ = [("pairs_train", C.c_uint64), ("pairs_val", C.c_uint64), ("steps", C.c_int32),
                ("final_loss", C.c_float), ("val_rmse", C.c_float), ("val_max_err", C.c_float), ("ms", C.c_double)]


MLP_CONES, MLP_FSTEPS, MLP_INPUTS, MLP_HIDDEN, MLP_PARAMS = 8, 6, 54, 64, 7745

# Every entry point include/p2v.h declares, with its ctypes signature.
_SIGNATURES = {
    "p2v_abi_version": ([], C.c_int),
    "p2v_params_default": ([C.POINTER(Params)], None),
    "p2v_create": ([C.POINTER(C.c_void_p), C.c_int], C.c_int),
    "p2v_destroy": ([C.c_void_p], None),
    "p2v_set_params": ([C.c_void_p, C.POINTER(Params)], C.c_int),
    "p2v_get_params": ([C.c_void_p, C.POINTER(Params)], C.c_int),
    "p2v_run_frame": ([C.c_void_p, C.POINTER(FrameC), C.POINTER(VolumeC), C.c_void_p], C.c_int),
    "p2v_get_device_volume": ([C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64)], C.c_int),
    "p2v_mmpld_open": ([C.c_char_p, C.POINTER(C.c_void_p), C.POINTER(MmpldInfoC)], C.c_int),
    "p2v_mmpld_close": ([C.c_void_p], None),
    "p2v_mmpld_frame_size": ([C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64)], C.c_int),
    "p2v_mmpld_read_frame": ([C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint32,
                              C.POINTER(C.c_uint32), C.POINTER(C.c_float)], C.c_int),
    "p2v_host_alloc": ([C.c_uint64], C.c_void_p),
    "p2v_host_free": ([C.c_void_p], None),
    "p2v_run_ao_on_grid": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "p2v_run_batch": ([C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p], C.c_int),
    "p2v_autotune_batch": ([C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(TuneReportC)], C.c_int),
    "p2v_get_ao_volume": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_uint64, C.c_int32, C.POINTER(C.c_int32)],
                          C.c_int),
    "p2v_mlp_get_pairs": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
    "p2v_write_datraw": ([C.c_void_p, C.c_char_p, C.c_uint32, C.c_uint32, C.c_void_p], C.c_int),
    "p2v_get_vector_grid": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int32,
                             C.c_void_p], C.c_int),
    "p2v_get_binning": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                         C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)], C.c_int),
    "p2v_get_stats": ([C.c_void_p, C.POINTER(StatsC)], C.c_int),
    "p2v_get_last_error": ([C.c_void_p, C.c_char_p, C.c_size_t], C.c_size_t),
    "p2v_train_params_default": ([C.POINTER(TrainParams)], None),
    "p2v_mlp_collect": ([C.c_void_p, C.POINTER(FrameC), C.c_uint32, C.c_uint64, C.POINTER(C.c_uint64)], C.c_int),
    "p2v_mlp_clear": ([C.c_void_p], C.c_int),
    "p2v_mlp_train": ([C.c_void_p, C.POINTER(TrainParams), C.POINTER(TrainReport)], C.c_int),
    "p2v_mlp_save": ([C.c_void_p, C.c_char_p], C.c_int),
    "p2v_mlp_load": ([C.c_void_p, C.c_char_p], C.c_int),
    "p2v_mlp_get_weights": ([C.c_void_p, C.c_void_p, C.c_uint64], C.c_int),
    "p2v_mlp_set_weights": ([C.c_void_p, C.c_void_p, C.c_uint64], C.c_int),
    "p2v_mlp_gradients": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_float)],
                          C.c_int),
    "p2v_mlp_infer": ([C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p], C.c_int),
    "p2v_aosphere_ao_noalloc": ([C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_float), C.POINTER(C.c_int32),
                                 C.c_float, C.c_float, C.c_float, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    # include/p2v_measure.h
    "p2v_measure_texture_rate": ([C.c_int, C.POINTER(C.c_double)], C.c_int),
}

_lib: Optional[C.CDLL] = None


def library(path: str = LIB_PATH) -> C.CDLL:
    """Load libp2v.so. Raises if it has not been built: there is no fallback implementation."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is missing: build it with `python -m megamol_gb300.build` "
                                    "(the GPU path has no CPU fallback)")
        lib = C.CDLL(path)
        for name, (args, res) in _SIGNATURES.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        _lib = lib
    return _lib


def measure_texture_rate(pattern: int) -> float:
    """G texture samples/s of the current device in the learned AO's feature format: pattern 0 = coherent quads,
    1 = every lane its own random point (p2v_measure_texture_rate)."""
    v = C.c_double(0.0)
    st = library().p2v_measure_texture_rate(int(pattern), C.byref(v))
    if st != OK:
        raise P2VError(st, "p2v_measure_texture_rate failed")
    return float(v.value)


def default_params() -> Params:
    p = Params()
    library().p2v_params_default(C.byref(p))
    return p


def _ptr(x) -> tuple[int, int]:
    """(address, mem kind) of a numpy array, a CUDA torch tensor or a raw host address."""
    if x is None:
        return 0, MEM_HOST
    if isinstance(x, int):
        return x, MEM_HOST
    if isinstance(x, np.ndarray):
        return x.ctypes.data, MEM_HOST
    if hasattr(x, "data_ptr"):
        return x.data_ptr(), (MEM_DEVICE if getattr(x, "is_cuda", False) else MEM_HOST)
    raise TypeError(f"unsupported buffer type {type(x)}")


def write_datraw(prefix: str, frame: int, volume, meta: dict, frame_count: int = 0, ctx: "Context" = None) -> None:
    """Write a volume as MegaMol's DatRawWriter does (plugins/volume/src/DatRawWriter.cpp:58-186):
    <prefix><frame:04>.dat and .raw. `volume` is a host array, a CUDA tensor, or None for the context's
    device grid of the last frame; `meta` the metadata dict run_frame returned (resolution, components,
    slice_dists, origin). frame_count > 0 rejects frames past it, as the reference does."""
    v = VolumeC()
    p, mem = _ptr(volume)
    v.data = p or None
    v.mem = mem
    v.capacity = int(volume.size if isinstance(volume, np.ndarray) else (volume.numel() if volume is not None else 0))
    v.resolution[:] = [int(x) for x in meta["resolution"]]
    v.components = int(meta.get("components", 1))
    v.slice_dists[:] = [float(x) for x in meta["slice_dists"]]
    v.origin[:] = [float(x) for x in meta["origin"]]
    st = library().p2v_write_datraw(ctx.h if ctx is not None else None, prefix.encode(), int(frame),
                                    int(frame_count), C.byref(v))
    if st != OK:
        raise P2VError(st, f"dat/raw write of {prefix}{int(frame):04d} failed")


@dataclass
class ParticleList:
    """One SimpleSphericalParticles list: vertex data of `vertex_type` with `stride` bytes per record."""
    data: Any
    vertex_type: int = VERTDATA_FLOAT_XYZR
    count: Optional[int] = None
    stride: int = 0
    global_radius: float = 0.5
    normals: Any = None
    normal_stride: int = 0
    ao_out: Any = None
    colour: Any = None            # colour data of colour_type (SimpleSphericalParticles colour layouts)
    colour_type: int = 0          # COLDATA_*
    colour_stride: int = 0
    global_colour: tuple = (255, 255, 255, 255)

    def to_c(self) -> "ParticleListC":
        dp, mem = _ptr(self.data)
        npp, _ = _ptr(self.normals)
        ap, _ = _ptr(self.ao_out)
        cp, _ = _ptr(self.colour)
        return ParticleListC(int(self.vertex_type), int(self.stride), dp, self.n(), float(self.global_radius), mem,
                             npp or None, int(self.normal_stride), ap or None, int(self.colour_type),
                             int(self.colour_stride), cp or None, (C.c_uint8 * 4)(*self.global_colour))

    def n(self) -> int:
        if self.count is not None:
            return int(self.count)
        comps = {1: 3, 2: 4, 3: 3, 4: 3}.get(self.vertex_type, 1)
        if isinstance(self.data, np.ndarray) and self.stride == 0:
            return self.data.size // comps
        return int(self.data.shape[0])


class Mmpld:
    """An MMPLD file read through libp2v (p2v_mmpld_*): header info and frames as ParticleLists that point
    into a frame buffer (pinned host memory when `pinned`)."""

    def __init__(self, path: str):
        self.lib = library()
        h = C.c_void_p()
        info = MmpldInfoC()
        st = self.lib.p2v_mmpld_open(str(path).encode(), C.byref(h), C.byref(info))
        if st != OK:
            raise P2VError(st, f"cannot open MMPLD file {path}")
        self.h = h
        self.version, self.frames = info.version, info.frames
        self.bbox, self.clipbox = list(info.bbox), list(info.clipbox)

    def close(self):
        if getattr(self, "h", None):
            self.lib.p2v_mmpld_close(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def frame_size(self, frame: int) -> int:
        b = C.c_uint64()
        st = self.lib.p2v_mmpld_frame_size(self.h, int(frame), C.byref(b))
        if st != OK:
            raise P2VError(st, f"frame {frame}")
        return b.value

    def read(self, frame: int, max_lists: int = 64):
        """(lists, list infos, timestamp, buffer): the ParticleLists reference `buffer` (keep it alive)."""
        size = self.frame_size(frame)
        buf = np.empty(max(size, 1), np.uint8)
        lists = (ParticleListC * max_lists)()
        infos = (MmpldListInfoC * max_lists)()
        n = C.c_uint32()
        ts = C.c_float()
        st = self.lib.p2v_mmpld_read_frame(self.h, int(frame), buf.ctypes.data, buf.size, C.cast(lists, C.c_void_p),
                                           C.cast(infos, C.c_void_p), max_lists, C.byref(n), C.byref(ts))
        if st != OK:
            raise P2VError(st, f"cannot read frame {frame}")
        out = []
        for k in range(min(n.value, max_lists)):
            L = lists[k]
            out.append(ParticleList(data=int(L.vertex_data or 0), vertex_type=L.vertex_type, count=L.count,
                                    stride=L.vertex_stride, global_radius=L.global_radius,
                                    colour=int(L.colour_data or 0) or None, colour_type=L.colour_type,
                                    colour_stride=L.colour_stride, global_colour=tuple(L.global_colour)))
        inf = [dict(intensity_range=list(infos[k].intensity_range), bbox=list(infos[k].bbox),
                    clusters=infos[k].clusters) for k in range(min(n.value, max_lists))]
        return out, inf, ts.value, buf


class Context:
    """One libp2v context on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = library()
        h = C.c_void_p()
        st = self.lib.p2v_create(C.byref(h), int(device))
        if st != OK:
            raise P2VError(st, f"p2v_create(device={device}) failed (no CUDA device?)")
        self.h = h
        self.params = default_params()

    def close(self):
        if getattr(self, "h", None):
            self.lib.p2v_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st != OK:
            buf = C.create_string_buffer(1024)
            self.lib.p2v_get_last_error(self.h, buf, 1024)
            raise P2VError(st, buf.value.decode(errors="replace"))

    def set_params(self, **kw) -> None:
        for k, v in kw.items():
            if not hasattr(self.params, k):
                raise AttributeError(f"unknown parameter {k}")
            cur = getattr(self.params, k)
            if isinstance(cur, C.Array):
                v = type(cur)(*v)
            setattr(self.params, k, v)
        self._check(self.lib.p2v_set_params(self.h, C.byref(self.params)))

    def get_params(self) -> Params:
        p = Params()
        self._check(self.lib.p2v_get_params(self.h, C.byref(p)))
        return p

    def _frame(self, lists, bbox, clipbox=None, frame_id=0):
        arr = (ParticleListC * max(1, len(lists)))()
        for i, L in enumerate(lists):
            arr[i] = L.to_c()
        fr = FrameC()
        fr.bbox[:] = [float(v) for v in bbox]
        fr.clipbox[:] = [float(v) for v in (clipbox if clipbox is not None else bbox)]
        fr.frame_id = frame_id
        fr.list_count = len(lists)
        fr.lists = arr
        return fr, arr

    # ---- learned AO ----
    def mlp_collect(self, lists, bbox, max_pairs: int, seed: int = 0, clipbox=None) -> int:
        fr, keep = self._frame(lists, bbox, clipbox)
        total = C.c_uint64()
        self._check(self.lib.p2v_mlp_collect(self.h, C.byref(fr), int(max_pairs), int(seed), C.byref(total)))
        return int(total.value)

    def mlp_clear(self):
        self._check(self.lib.p2v_mlp_clear(self.h))

    def mlp_train(self, **kw) -> dict:
        tp = TrainParams()
        self.lib.p2v_train_params_default(C.byref(tp))
        for k, v in kw.items():
            if not hasattr(tp, k):
                raise AttributeError(f"unknown training parameter {k}")
            setattr(tp, k, v)
        rep = TrainReport()
        self._check(self.lib.p2v_mlp_train(self.h, C.byref(tp), C.byref(rep)))
        return {k: getattr(rep, k) for k, _ in rep._fields_}

    def mlp_save(self, path: str):
        self._check(self.lib.p2v_mlp_save(self.h, path.encode()))

    def mlp_load(self, path: str):
        self._check(self.lib.p2v_mlp_load(self.h, path.encode()))

    def mlp_get_weights(self) -> np.ndarray:
        w = np.zeros(MLP_PARAMS, np.float32)
        self._check(self.lib.p2v_mlp_get_weights(self.h, w.ctypes.data, w.size))
        return w

    def mlp_set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        self._check(self.lib.p2v_mlp_set_weights(self.h, w.ctypes.data, w.size))

    def mlp_gradients(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = C.c_float()
        self._check(self.lib.p2v_mlp_gradients(self.h, x.ctypes.data, t.ctypes.data, x.shape[0], g.ctypes.data,
                                               C.byref(loss)))
        return g, loss.value

    def mlp_infer(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros(x.shape[0], np.float32)
        self._check(self.lib.p2v_mlp_infer(self.h, x.ctypes.data, x.shape[0], y.ctypes.data))
        return y

    def run_frame(self, lists: Sequence[ParticleList], bbox, out=None, clipbox=None, stream: int = 0,
                  frame_id: int = 0) -> dict:
        """Run one frame. `out` is a host numpy float32 array or a CUDA float32 tensor (or None)."""
        arr = (ParticleListC * max(1, len(lists)))()
        for i, L in enumerate(lists):
            arr[i] = L.to_c()
        fr = FrameC()
        fr.bbox[:] = [float(v) for v in bbox]
        fr.clipbox[:] = [float(v) for v in (clipbox if clipbox is not None else bbox)]
        fr.frame_id = frame_id
        fr.list_count = len(lists)
        fr.lists = arr
        vol = VolumeC()
        if out is not None:
            op, omem = _ptr(out)
            vol.data = op
            vol.mem = omem
            vol.capacity = int(out.size if isinstance(out, np.ndarray) else out.numel())
        self._check(self.lib.p2v_run_frame(self.h, C.byref(fr), C.byref(vol), C.c_void_p(stream)))
        return dict(resolution=list(vol.resolution), components=int(vol.components),
                    slice_dists=list(vol.slice_dists), origin=list(vol.origin), extents=list(vol.extents),
                    min_value=vol.min_value, max_value=vol.max_value, bbox=list(vol.bbox), data_hash=vol.data_hash)

    def run_ao_on_grid(self, lists: Sequence[ParticleList], bbox, grid, clipbox=None, stream: int = 0):
        """AO of the lists' particles (written to their ao_out) against `grid` (the frame's sizex * sizey * sizez
        density, host numpy float32 or CUDA float32 tensor) instead of the grid of their own density."""
        fr, keep = self._frame(lists, bbox, clipbox)
        gp, gmem = _ptr(grid)
        self._check(self.lib.p2v_run_ao_on_grid(self.h, C.byref(fr), C.c_void_p(gp), gmem, C.c_void_p(stream)))

    # ---- batches ----
    def _batch(self, frames):
        """frames: sequence of dicts with keys lists, bbox, and optionally out, size, clipbox. Returns the
        ctypes objects (kept alive by the caller) and the item array."""
        keep, vols = [], []
        items = (BatchItemC * max(1, len(frames)))()
        for i, f in enumerate(frames):
            fr, arr = self._frame(f["lists"], f["bbox"], f.get("clipbox"), i)
            vol = VolumeC()
            out = f.get("out")
            if out is not None:
                op, omem = _ptr(out)
                vol.data = op
                vol.mem = omem
                vol.capacity = int(out.size if isinstance(out, np.ndarray) else out.numel())
            keep += [fr, arr, vol]
            vols.append(vol)
            size = f.get("size", (0, 0, 0))
            items[i] = BatchItemC(C.cast(C.pointer(fr), C.c_void_p), C.cast(C.pointer(vol), C.c_void_p),
                                  (C.c_int32 * 3)(*[int(v) for v in size]))
        return keep, vols, items

    def run_batch(self, frames, stream: int = 0):
        """Run a batch of frames (see _batch); returns per-frame metadata dicts and per-frame stats."""
        keep, vols, items = self._batch(frames)
        st = (StatsC * max(1, len(frames)))()
        self._check(self.lib.p2v_run_batch(self.h, C.cast(items, C.c_void_p), len(frames), C.cast(st, C.c_void_p),
                                           C.c_void_p(stream)))
        meta = [dict(resolution=list(v.resolution), min_value=v.min_value, max_value=v.max_value,
                     slice_dists=list(v.slice_dists), origin=list(v.origin), data_hash=v.data_hash) for v in vols]
        stats = [{k: (list(getattr(x, k)) if k in ("cell_min", "cell_max") else getattr(x, k))
                  for k, _ in x._fields_} for x in st[:len(frames)]]
        return meta, stats

    def autotune_batch(self, frames) -> dict:
        keep, vols, items = self._batch(frames)
        rep = TuneReportC()
        rep.struct_size = C.sizeof(TuneReportC)
        self._check(self.lib.p2v_autotune_batch(self.h, C.cast(items, C.c_void_p), len(frames), C.byref(rep)))
        n = rep.candidates
        return dict(tile=list(rep.tile), lanes=rep.lanes, persistent=rep.persistent, ms_best=rep.ms_best,
                    candidates=[dict(tile=list(rep.cand_tile[k]), lanes=rep.cand_lanes[k], ms=rep.cand_ms[k],
                                     persistent=rep.cand_persistent[k]) for k in range(n)])

    def stats(self) -> dict:
        s = StatsC()
        self._check(self.lib.p2v_get_stats(self.h, C.byref(s)))
        return {k: (list(getattr(s, k)) if k in ("cell_min", "cell_max") else getattr(s, k)) for k, _ in s._fields_}

    def device_volume(self):
        p = C.c_void_p()
        res = (C.c_uint64 * 3)()
        self._check(self.lib.p2v_get_device_volume(self.h, C.byref(p), res))
        return p.value, list(res)

    def binning(self):
        """(sorted keys, sort permutation, cell starts) of the last frame, as host arrays."""
        n, nb = C.c_uint32(), C.c_uint32()
        self._check(self.lib.p2v_get_binning(self.h, None, None, 0, None, 0, C.byref(n), C.byref(nb)))
        keys = np.empty(n.value, np.uint32)
        order = np.empty(n.value, np.uint32)
        start = np.empty(nb.value + 1, np.uint32)
        self._check(self.lib.p2v_get_binning(self.h, keys.ctypes.data, order.ctypes.data, keys.size,
                                             start.ctypes.data, start.size, None, None))
        return keys, order, start

    def mlp_pairs(self):
        """(features (n, MLP_INPUTS), targets (n,)) of the collected training pairs, in collection order."""
        n = C.c_uint64()
        self._check(self.lib.p2v_mlp_get_pairs(self.h, None, None, 0, C.byref(n)))
        x = np.empty((n.value, MLP_INPUTS), np.float32)
        t = np.empty(n.value, np.float32)
        self._check(self.lib.p2v_mlp_get_pairs(self.h, x.ctypes.data, t.ctypes.data, n.value, None))
        return x, t

    def vector_grid(self) -> dict:
        """The vector aggregator's outParticles / outInfo grid of the last frame (aggregator 2 with
        vector_grid): positions (n, 3), directions (n, 3), colours (n,), info (n, 7), global_radius and the
        7 columns' col_min / col_max."""
        meta = VectorGridInfoC()
        self._check(self.lib.p2v_get_vector_grid(self.h, None, None, None, None, 0, MEM_HOST, C.byref(meta)))
        n = int(meta.count)
        pos, dr = np.empty((n, 3), np.float32), np.empty((n, 3), np.float32)
        col, info = np.empty(n, np.float32), np.empty((n, 7), np.float32)
        self._check(self.lib.p2v_get_vector_grid(self.h, pos.ctypes.data, dr.ctypes.data, col.ctypes.data,
                                                 info.ctypes.data, n, MEM_HOST, C.byref(meta)))
        return dict(count=n, positions=pos, directions=dr, colours=col, info=info,
                    global_radius=float(meta.global_radius), col_min=np.array(meta.col_min[:], np.float32),
                    col_max=np.array(meta.col_max[:], np.float32))

    def ao_volume(self, level: int = 0) -> np.ndarray:
        """Level `level` of the last cone-march pyramid as a (z, y, x) float32 host array."""
        dims = (C.c_int32 * 3)()
        self._check(self.lib.p2v_get_ao_volume(self.h, int(level), None, 0, MEM_HOST, dims))
        out = np.empty((dims[2], dims[1], dims[0]), np.float32)
        self._check(self.lib.p2v_get_ao_volume(self.h, int(level), out.ctypes.data, out.size, MEM_HOST, dims))
        return out


class ParticlesToDensity:
    """Host-side mirror of datatools::ParticlesToDensity (ParticlesToDensity.h:32-145): same parameter
    slots, same outputs, computed on the GPU through libp2v."""

    SLOTS = ("aggregator", "sizex", "sizey", "sizez", "cyclX", "cyclY", "cyclZ", "normalize", "sigma",
             "forSurfaceReconstruction")

    def __init__(self, device: int = 0, **params):
        self.ctx = Context(device)
        self.ctx.set_params(**params)
        self.metadata: dict = {}

    def set(self, **params) -> None:
        self.ctx.set_params(**params)

    def param(self, name: str):
        return getattr(self.ctx.get_params(), name)

    def get_data(self, lists: Sequence[ParticleList], bbox, clipbox=None, out=None):
        """VolumetricDataCall GET_DATA: returns (volume, metadata). The volume is a (z, y, x) float32 array,
        (z, y, x, 3) for the vector aggregator (or the given `out`)."""
        p = self.ctx.get_params()
        comps = 3 if p.aggregator == 2 else 1
        if p.aggregator == 2 and not p.vector_grid:
            self.ctx.set_params(vector_grid=1)  # the outParticles / outInfo grid, as the reference always builds
        res = [p.sizex, p.sizey, p.sizez]
        host_out = out
        if out is None:
            if p.forSurfaceReconstruction:
                # the resolution is only known after the box adjustment: compute into the device buffer
                meta = self.ctx.run_frame(lists, bbox, None, clipbox)
                res = meta["resolution"]
                host_out = np.empty(res[2] * res[1] * res[0] * comps, np.float32)
                meta = self.ctx.run_frame(lists, bbox, host_out, clipbox)
                self.metadata = meta
                return self._shape(host_out, res, comps), meta
            host_out = np.empty(res[2] * res[1] * res[0] * comps, np.float32)
        meta = self.ctx.run_frame(lists, bbox, host_out, clipbox)
        self.metadata = meta
        if isinstance(host_out, np.ndarray):
            return self._shape(host_out, meta["resolution"], comps), meta
        return host_out, meta

    @staticmethod
    def _shape(a, r, comps):
        return a.reshape(r[2], r[1], r[0]) if comps == 1 else a.reshape(r[2], r[1], r[0], comps)

    def get_particles(self) -> dict:
        """The "outParticles" MultiParticleDataCall of the vector aggregator after get_data
        (ParticlesToDensity.cpp:306-323): one list of grid nodes with VERTDATA_FLOAT_XYZ positions,
        DIRDATA_FLOAT_XYZ directions, COLDATA_FLOAT_I colours and the global radius."""
        g = self.ctx.vector_grid()
        return dict(count=g["count"], vertex=g["positions"], directions=g["directions"], colours=g["colours"],
                    global_radius=g["global_radius"])

    COLUMNS = ("PositionX", "PositionY", "PositionZ", "VelocityX", "VelocityY", "VelocityZ", "VelocityMag")

    def get_info(self):
        """The "outInfo" TableDataCall of the vector aggregator after get_data (ParticlesToDensity.cpp:
        325-380): (columns as (name, minimum, maximum), rows (n, 7))."""
        g = self.ctx.vector_grid()
        cols = [(nm, float(g["col_min"][k]), float(g["col_max"][k])) for k, nm in enumerate(self.COLUMNS)]
        return cols, g["info"]
