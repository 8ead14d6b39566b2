"""CPU tests of the C ABI boundary: the library loads, exports every entry point include/p2v.h declares,
and the ctypes mirror has the header's struct layout. No compute call is made here."""
import ctypes as C
import json
import os
import re
import subprocess

import pytest

from megamol_gb300 import build as nbuild
from megamol_gb300 import p2v

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]


@pytest.fixture(scope="module")
def lib():
    nbuild.build()
    return p2v.library()


def declared_symbols():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        names |= set(re.findall(r"P2V_API\s+[\w\s\*]+?\b(p2v_\w+)\s*\(", txt))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 10
    out = subprocess.run(["nm", "-D", "--defined-only", nbuild.LIB], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (p2v_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in names:
        assert hasattr(lib, n)


def test_ctypes_signatures_cover_header():
    assert set(declared_symbols()) <= set(p2v._SIGNATURES)


def test_struct_layout_matches_header(tmp_path):
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "abi_layout.c"),
                    "-o", str(exe)], check=True)
    lay = json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    types = {"p2v_params": p2v.Params, "p2v_particle_list": p2v.ParticleListC, "p2v_frame": p2v.FrameC,
             "p2v_volume": p2v.VolumeC, "p2v_stats": p2v.StatsC, "p2v_batch_item": p2v.BatchItemC,
             "p2v_tune_report": p2v.TuneReportC, "p2v_mmpld_info": p2v.MmpldInfoC,
             "p2v_mmpld_list_info": p2v.MmpldListInfoC, "p2v_vector_grid_info": p2v.VectorGridInfoC}
    for k, v in lay.items():
        if k == "end":
            continue
        if "." in k:
            t, m = k.split(".")
            assert getattr(types[t], m).offset == v, k
        else:
            assert C.sizeof(types[k]) == v, k


def test_params_default_mirror_reference_slots(lib):
    p = p2v.default_params()
    assert p.struct_size == C.sizeof(p2v.Params)
    # ParticlesToDensity.cpp:126-147
    assert (p.sizex, p.sizey, p.sizez) == (16, 16, 16)
    assert (p.cyclX, p.cyclY, p.cyclZ, p.normalize) == (1, 1, 1, 1)
    assert p.sigma == 1.0 and p.forSurfaceReconstruction == 0 and p.aggregator == 0
    # SphereRenderer.cpp:199-212 MDAO defaults
    assert p.ao_cones == 3 and abs(p.ao_apex_deg - 50) < 1e-6 and abs(p.ao_offset - 0.01) < 1e-7
    assert abs(p.ao_cone_length - 0.8) < 1e-7 and p.mdao_volume_size == 128
    assert p.batch_lanes == 0 and p.batch_graph == 1 and p.vector_grid == 0
    assert p.batch_persistent == -1 and p.queue_wait_polls == 0 and p.test_hold_queue == 0
    assert p.sort_wait_polls == 0 and p.test_hold_sort == 0 and p.ao_march == p2v.AO_MARCH_THREAD
    assert p.ao_brick_order == 0
    assert lib.p2v_abi_version() == 10


def test_create_without_device_fails_cleanly(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    assert lib.p2v_create(C.byref(h), 0) == p2v.ECUDA
    assert not h.value


def test_megamol_adapter_compiles_against_reference_headers():
    """The drop-in module (megamol_gb300/adapter) compiles against MegaMol's own geometry_calls and
    vislib headers, with the oracle's stand-ins for the core headers. Needs the MegaMol source tree."""
    import oracle

    ref = oracle.REFERENCE_TREE
    if not os.path.isdir(os.path.join(ref, "plugins", "geometry_calls")):
        pytest.skip("MegaMol source tree not present")
    src = os.path.join(ROOT, "megamol_gb300", "adapter", "ParticlesToDensityGPU.cpp")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "oracle", "shim"), "-I",
                        os.path.join(ROOT, "include"), "-I", os.path.join(ref, "plugins", "geometry_calls", "include"),
                        "-I", os.path.join(ref, "vislib", "include"), src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_header_constants_match_binding():
    """Every #define and enum value of include/p2v.h that the ctypes binding mirrors (P2V_X -> p2v.X) has
    the same value there."""
    consts = {}
    for h in HEADERS:
        txt = open(h).read()
        consts.update({m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+P2V_(\w+)\s+(-?\d+)\b", txt)})
        consts.update({m.group(1): int(m.group(2)) for m in re.finditer(r"\bP2V_(\w+)\s*=\s*(-?\d+)", txt)})
    matched = {k: v for k, v in consts.items() if hasattr(p2v, k) and isinstance(getattr(p2v, k), int)}
    assert len(matched) >= 20, sorted(matched)
    assert {"NOALLOC_MAX_VOXELS", "MLP_INPUTS", "MLP_PARAMS", "TUNE_MAX"} <= set(matched), sorted(matched)
    wrong = {k: (v, getattr(p2v, k)) for k, v in matched.items() if getattr(p2v, k) != v}
    assert not wrong, wrong
