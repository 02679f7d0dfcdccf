"""The C++ facade (include/pbat_gb300.hpp) that mirrors pbat::gpu::vbd::Integrator: compiled with
the host compiler against the library, fed an object with the reference Data's member names
(tests/cpp/facade_main.cpp).  Without a device it fails loudly; on a device its trajectory equals
the Python integrator's on the same mesh."""

import pathlib
import shutil
import subprocess

import numpy as np
import pytest

from physicsbasedanimationtoolkit_gb300 import _build, meshgen, pbat

ROOT = pathlib.Path(__file__).resolve().parent.parent


def build_driver(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib = _build.build()
    exe = tmp_path / "facade_main"
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "facade_main.cpp"), f"-L{lib.parent}", "-lpbat_gb300",
                    f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    return exe


def write_mesh(path, X, T, dbc):
    with open(path, "w") as f:
        f.write(f"{X.shape[0]} {T.shape[0]} {dbc.size}\n")
        for p in X:
            f.write("%.17g %.17g %.17g\n" % tuple(p))
        for t in T:
            f.write("%d %d %d %d\n" % tuple(t))
        f.write(" ".join(map(str, dbc)) + "\n")


def mesh():
    X, T = meshgen.hex_grid(4, 3, 3, hi=(1.5, 1.0, 1.0))
    return X, T, meshgen.face_vertices(X, 0, 0.0)


def test_facade_compiles_and_fails_loudly_without_a_device(tmp_path):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is present (covered by the GPU test)")
    exe = build_driver(tmp_path)
    X, T, dbc = mesh()
    write_mesh(tmp_path / "mesh.txt", X, T, dbc)
    r = subprocess.run([str(exe), str(tmp_path / "mesh.txt"), str(tmp_path / "out.txt"), "2", "5"],
                       capture_output=True, text=True)
    assert r.returncode == 3, (r.returncode, r.stderr)
    assert "no CUDA device" in r.stderr


@pytest.mark.gpu
def test_facade_trajectory_equals_the_python_integrator(tmp_path):
    exe = build_driver(tmp_path)
    X, T, dbc = mesh()
    write_mesh(tmp_path / "mesh.txt", X, T, dbc)
    r = subprocess.run([str(exe), str(tmp_path / "mesh.txt"), str(tmp_path / "out.txt"), "4", "12"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    x_cpp = np.loadtxt(tmp_path / "out.txt", dtype=np.float32)
    nT = T.shape[0]
    mu, lam = meshgen.lame(np.full(nT, 1e6), np.full(nT, 0.45))
    d = (pbat.sim.vbd.Data().with_volume_mesh(X.T, T.T).with_material(np.full(nT, 1000.0), mu, lam)
         .with_dirichlet_vertices(dbc).with_initialization_strategy(2).construct())
    I = pbat.gpu.vbd.Integrator(d)
    I.gpu_block_size = 64
    for _ in range(4):
        I.step(1 / 60, 12, 1)
    np.testing.assert_array_equal(x_cpp, I.x.T)
