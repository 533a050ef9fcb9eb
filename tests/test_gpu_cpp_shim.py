"""The C++ mirror of goal's host classes (goal_gb300/host/goal.hpp), compiled
with g++ against the C ABI, reproduces two of the reference's regression values
on the reference's cube mesh."""
import os
import struct
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write_mesh(mesh, path):
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", mesh.num_nodes, mesh.num_elems))
        f.write(np.ascontiguousarray(mesh.coords, "<f8").tobytes())
        f.write(np.ascontiguousarray(mesh.tets, "<i4").tobytes())
        for sets in (mesh.node_sets, mesh.side_sets):
            f.write(struct.pack("<i", len(sets)))
            for name, ids in sets.items():
                ids = np.ascontiguousarray(ids, "<i4")
                n = ids.shape[0]
                f.write(struct.pack("<i", len(name)) + name.encode() + struct.pack("<i", n))
                f.write(ids.tobytes())


def test_cpp_driver_regression(cube_kat, tmp_path):
    mesh, _ = cube_kat
    mpath = tmp_path / "cube.bin"
    write_mesh(mesh, mpath)
    exe = tmp_path / "primal_kat"
    lib_dir = os.path.join(ROOT, "goal_gb300")
    subprocess.check_call(["g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "primal_kat.cpp"),
                           "-I", os.path.join(ROOT, "include"), "-L", lib_dir, "-lgoal_gb300",
                           "-Wl,-rpath," + lib_dir, "-o", str(exe)])
    out = subprocess.run([str(exe), str(mpath)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    assert "OK" in out.stdout
    assert "J(uH) = " in out.stdout


def _cuda_home():
    return os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH") or "/usr/local/cuda"


def test_cpp_device_views(cube_kat, tmp_path):
    """goal_disc_device_graph, goal_sol_info_device_view / _device_csr and
    goal_mechanics_device_solution equal the host copies entry for entry, and
    goal_solve_device on the SolInfo's own dM/du gives the host solve's
    iterate (tests/cpp/device_views.cpp)."""
    mesh, _ = cube_kat
    mpath = tmp_path / "cube.bin"
    write_mesh(mesh, mpath)
    exe = tmp_path / "device_views"
    lib_dir = os.path.join(ROOT, "goal_gb300")
    cuda = _cuda_home()
    subprocess.check_call(["g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "device_views.cpp"),
                           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
                           "-L", lib_dir, "-lgoal_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart",
                           "-Wl,-rpath," + lib_dir, "-Wl,-rpath," + os.path.join(cuda, "lib64"), "-o", str(exe)])
    out = subprocess.run([str(exe), str(mpath)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    assert "OK" in out.stdout
