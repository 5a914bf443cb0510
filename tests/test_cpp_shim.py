"""The C++ classes of include/kifi_gpu.hpp (the reference's Volume /
Integrator / Mesher / ICP / Renderer signatures over the C ABI), compiled
with the reference's own util headers and DepthSensorParams from the staged
reference sources (oracle/_ref/src, made by oracle/build_ref.py)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.path.join(ROOT, "oracle", "_ref", "src")
SHIM = os.path.join(ROOT, "oracle", "shim")
FLAGS = ["-std=c++14", "-O1", "-w", "-include", os.path.join(SHIM, "kifi_ref_prelude.h"),
         "-I", SHIM, "-I", REF_SRC, "-I", os.path.join(ROOT, "include")]


def _need_sources():
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    if not os.path.isdir(os.path.join(REF_SRC, "kifi")):
        pytest.skip("staged reference sources absent (oracle/build_ref.py stage)")


def test_shim_compiles_against_reference_headers(tmp_path):
    _need_sources()
    src = tmp_path / "use.cpp"
    src.write_text('#include "kifi_gpu.hpp"\n'
                   "void use(kifi::Volume& v, kifi::util::vector2d<float> const& f,\n"
                   "         kifi::DepthSensorParams const& p, kifi::util::float4x4 const& m) {\n"
                   "  kifi::Integrator().Integrate(v, f, p, m);\n"
                   "  std::vector<kifi::util::float3> verts; std::vector<unsigned> idx;\n"
                   "  kifi::Mesher().Mesh(v, verts); kifi::Mesher().Mesh(v, verts, idx);\n"
                   "  kifi::util::vector2d<kifi::util::float3> synth(640, 480);\n"
                   "  kifi::util::float4x4 pose = kifi::ICP().Align(f, m, synth, m, p);\n"
                   "  kifi::Renderer().Bin(verts, pose, synth);\n"
                   "  (void)v.Data().size();\n"
                   "}\n")
    r = subprocess.run(["g++"] + FLAGS + ["-fsyntax-only", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_shim_runs_reference_unit_case(gpu, golden, tmp_path):
    _need_sources()
    from merge_fusion_gb300 import _lib
    lib = _lib.load()  # builds nothing; the library must exist
    del lib
    exe = tmp_path / "shim_unit"
    cmd = (["g++"] + FLAGS + [os.path.join(ROOT, "tests", "cpp", "shim_unit.cpp"),
                              os.path.join(REF_SRC, "kifi", "DepthSensorParams.cpp"),
                              "-L" + os.path.dirname(_lib.LIB_PATH), "-lkifi_gpu",
                              "-Wl,-rpath," + os.path.dirname(_lib.LIB_PATH), "-o", str(exe)])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    blob = tmp_path / "frame.bin"
    with open(blob, "wb") as f:
        f.write(np.ascontiguousarray(golden["depth"], np.float32).tobytes())
        f.write(np.ascontiguousarray(golden["view"], np.float32).reshape(16).tobytes())
    r = subprocess.run([str(exe), str(blob)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    voxels, v0, v1, ni = (int(x) for x in r.stdout.split())
    case = golden["cases"][0]
    assert (voxels, v0, v1, ni) == (case["voxels"], case["mesh_verts_only"], case["mesh_verts"],
                                    case["mesh_indices"])
