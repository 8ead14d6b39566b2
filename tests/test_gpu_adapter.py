"""The MegaMol module ParticlesToDensityGPU at run time on the GPU: tests/adapter/adapter_harness.cpp drives it as
a MegaMol graph would (a particle source on "inData", a clip-plane module on "getclipplane", parameters by slot
name, "outData" GetExtents / GetData and "outAO" GetData by call and function name) and compares the volume, its
metadata and the AO with p2v_run_frame called directly with the same parameters: they must be identical. The
module is compiled with the oracle's stand-ins for MegaMol's core headers and tests/adapter/standins for the
particle, volume and vislib types (the MegaMol tree itself is not needed; tests/test_abi.py compiles the same
module against MegaMol's own geometry_calls and vislib headers)."""
import os
import subprocess

import pytest

from megamol_gb300 import build as nbuild

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_module_callbacks_match_the_c_abi(tmp_path):
    lib = nbuild.build()
    exe = str(tmp_path / "adapter_harness")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "tests", "adapter", "standins"), "-I",
           os.path.join(ROOT, "oracle", "shim"), "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "megamol_gb300", "adapter"), os.path.join(ROOT, "tests", "adapter", "adapter_harness.cpp"),
           os.path.join(ROOT, "megamol_gb300", "adapter", "ParticlesToDensityGPU.cpp"), "-o", exe, "-L", libdir,
           "-lp2v", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "0 failures" in r.stdout, r.stdout[-3000:] + r.stderr[-2000:]
    assert r.stdout.count("ok  ") >= 14, r.stdout
