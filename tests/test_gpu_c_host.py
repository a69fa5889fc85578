"""A host written in plain C (tests/c/abi_host.c) against include/forcegpu.h alone: built with
gcc, linked to libforcegpu.so, it steps a layout through the C ABI (and checks that
fl_sync_packed reads back the same x, y, z as fl_sync); the same layout stepped through the
Python binding gives the same positions (one library, the same inputs)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from forcegpu import _lib
from forcegpu._lib import Engine, desc_from_gpu

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "abi_host")
    subprocess.check_call([cc, "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "c", "abi_host.c"), "-L", libdir,
                           "-lforcegpu", "-Wl,-rpath," + libdir, "-lm", "-o", exe])
    return exe


def python_run(n, ticks):
    """The C program's layout, through the Python binding."""
    i = np.arange(n, dtype=np.float64)
    ang, ang2 = np.pi * (3 - np.sqrt(5.0)), np.pi * 20 / (9 + np.sqrt(221.0))
    r, a, b = 10.0 * np.cbrt(0.5 + i), i * ang, i * ang2
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, 0] = (r * np.sin(b) * np.cos(a)).astype(np.float32)
    pos4[:, 1] = (r * np.cos(b)).astype(np.float32)
    pos4[:, 2] = (r * np.sin(b) * np.sin(a)).astype(np.float32)
    src = np.concatenate([np.arange(n - 1), np.arange(n)]).astype(np.int32)
    dst = np.concatenate([np.arange(1, n), (np.arange(n) + 7) % n]).astype(np.int32)
    deg = np.bincount(np.concatenate([src, dst]), minlength=n).astype(np.float32)
    strength = np.float32(1) / np.minimum(deg[src], deg[dst])
    bias = deg[src] / (deg[src] + deg[dst])
    e = Engine(0)
    e.set_nodes(pos4, 3)
    forces = [
        {"type": "link", "version": 1, "source": src, "target": dst, "iterations": 1,
         "strengths": strength, "distances": np.full(len(src), 30.0), "bias": bias},
        {"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0), "distanceMin2": 1.0,
         "distanceMax2": np.inf, "theta2": 0.81},
        {"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0},
    ]
    e.set_forces([desc_from_gpu(f, k + 1, n) for k, f in enumerate(forces)])
    e.set_seed(7)
    alphas, a = [], 1.0
    decay = 1 - 0.001 ** (1 / 300)
    for _ in range(ticks):
        a += (0.0 - a) * decay
        alphas.append(a)
    e.enqueue(np.array(alphas), 0.6)
    pos, _ = e.sync()
    e.close()
    return pos[:, :3]


@pytest.mark.parametrize("n,ticks", [(1000, 10), (20000, 5)])
def test_a_c_host_and_the_python_binding_agree(tmp_path, n, ticks):
    exe = build(tmp_path)
    out = subprocess.run([exe, str(n), str(ticks)], capture_output=True, text=True, check=True)
    got = np.array([[float(v) for v in line.split()] for line in out.stdout.splitlines()])
    assert got.shape == (n, 3) and np.isfinite(got).all()
    want = python_run(n, ticks)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-4)
