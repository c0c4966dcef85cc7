"""CPU tests of the C ABI library and the command-line driver (no compute calls: no GPU here)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import navier_stokes_fem_gb300 as nsf
from navier_stokes_fem_gb300 import mesh as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "navier_stokes_fem_gb300", "bin", "nsfem")


def _has_gpu():
    h = ctypes.c_void_p()
    st = nsf.library().nsf_create(0, ctypes.byref(h))
    if st == 0:
        nsf.library().nsf_destroy(h)
    return st == 0


def test_library_exports_every_declared_symbol():
    lib = nsf.library()
    declared = nsf.declared_symbols()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(lib, name), name


def test_header_is_plain_c():
    with open(nsf.header_path) as f:
        text = f.read()
    assert 'extern "C"' in text and "torch" not in text and "std::" not in text


@pytest.mark.skipif(_has_gpu(), reason="a GPU is present")
def test_no_device_is_a_status_not_a_crash():
    h = ctypes.c_void_p()
    assert nsf.library().nsf_create(0, ctypes.byref(h)) == 7          # NSF_ERR_NO_DEVICE
    assert nsf.library().nsf_sim_step(None, 1, None) == 5             # NSF_ERR_BAD_ARG on a null handle
    with pytest.raises(nsf.NSFemError) as e:
        nsf.GPUSimulationDevice(0)
    assert e.value.status == 7


def test_cli_help_and_argument_errors(tmp_path):
    r = subprocess.run([CLI, "-help"], capture_output=True, text=True)
    assert r.returncode == 0 and "sceneFile" in r.stdout
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 1 and "Missing required parameter: sceneFile" in r.stderr
    r = subprocess.run([CLI, "-bogus=1"], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([CLI, f"-sceneFile={tmp_path}/nope.json"], capture_output=True, text=True)
    assert r.returncode == 1 and "Cannot open JSON file" in r.stderr


def test_cli_reads_scene_and_mesh(tmp_path):
    m = M.cavity(4)
    M.write_mesh_json(m, str(tmp_path / "mesh.json"))
    M.write_scene_json(str(tmp_path / "scene.json"), "./mesh.json", total_time=1, viscosity=0.01, dt=0.01)
    r = subprocess.run([CLI, f"-sceneFile={tmp_path}/scene.json"], capture_output=True, text=True)
    assert "Elements: 32" in r.stdout and "Velocity nodes: 81" in r.stdout and "Pressure nodes: 25" in r.stdout
    assert "Total steps: 99" in r.stdout      # int(total_time/dt) - 1, as the reference loop runs
    if not _has_gpu():
        assert r.returncode == 1 and "cannot initialise CUDA device" in r.stderr


def test_cli_reports_missing_scene_keys(tmp_path):
    (tmp_path / "scene.json").write_text('{"mesh_path": "./m.json", "total_time": 1, "viscosity": 0.1}')
    r = subprocess.run([CLI, f"-sceneFile={tmp_path}/scene.json"], capture_output=True, text=True)
    assert r.returncode == 1 and "Missing required param: dt" in r.stderr


def test_python_bc_occurrences_follow_group_order():
    m = M.channel_with_obstacle(16, 4)
    un, gu, gv, pn, gp = nsf.bc_occurrences(m)
    assert len(un) == sum(len(g[0]) for g in m.u_dirichlet)
    y = m.nodes[un[: len(m.u_dirichlet[0][0])], 1].astype(np.float64)
    assert np.allclose(gu[: len(y)], 4 * y * (1 - y))
    f = nsf._bc_fast(m)
    for a, b in zip(f, (un, gu, gv, pn, gp)):
        assert np.array_equal(a, b)


def test_integration_shim_compiles_against_reference_header(tmp_path):
    """The C++ shim of INTEGRATION.md section 2 against the reference's own, unmodified
    include/gpu_simulation_device.h (g++ -fsyntax-only), with declarations standing in for the absent
    sparse_matrix_math submodule; only where the reference checkout is present."""
    import re
    import shutil
    import subprocess

    import oracle

    ref = oracle.reference_dir()
    if ref is None or shutil.which("g++") is None:
        pytest.skip("reference checkout not present here")
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        md = f.read()
    block = re.search(r"```cpp\n(// gpu_simulation_device_gb300\.cpp.*?)```", md, re.S)
    assert block, "shim block not found"
    src = tmp_path / "gpu_simulation_device_gb300.cpp"
    src.write_text(block.group(1))
    forced = []
    for h in ("vector", "string", "cstring", "cinttypes", "cassert", "cmath", "algorithm", "memory", "cstdarg",
              "cstdio", "cfloat", "cstdint"):
        forced += ["-include", h]
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", *forced, "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle", "stub_include"), "-I", os.path.join(ref, "include"),
           "-I", os.path.join(ref, "gpu_cpu_shared"), "-I", "/usr/local/cuda/include", str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
