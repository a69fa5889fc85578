"""The C-ABI library loads and exports every entry point include/forcegpu.h declares; without a
GPU the facade fails loudly (no CPU path). No compute calls here."""
import asyncio
import os
import re
import subprocess

import pytest

import forcegpu
from forcegpu import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "forcegpu.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fl_[a-z_]+)\s*\(", text)))


def test_header_and_bindings_agree():
    assert declared() == sorted(_lib.EXPORTS)


def test_library_exports_every_symbol():
    L = forcegpu.load()
    for name in declared():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (fl_\w+)", out))
    assert set(declared()) <= exported


def test_simulation_keys():
    """test/gpu-simulation-test.js:25-29: forceSimulation's API plus the GPU additions."""
    sim = forceSimulationGPU_stopped()
    public = sorted(k for k in dir(sim) if not k.startswith("_") and callable(getattr(sim, k)))
    assert public == sorted(forcegpu.SIMULATION_KEYS + forcegpu.GPU_KEYS)
    sim.destroy()


def forceSimulationGPU_stopped(*a):
    return forcegpu.forceSimulationGPU(*a).stop()


def test_phyllotaxis_like_force_simulation():
    """test/gpu-simulation-test.js:38-44."""
    a, b, c = {}, {}, {}
    sim = forceSimulationGPU_stopped([a, b, c])
    for node, (x, y) in zip((a, b, c), [(7.0710678118654755, 0), (-9.03088751750192, 8.27303273571596),
                                        (1.3823220809823638, -15.750847141167634)]):
        assert abs(node["x"] - x) < 1e-6 and abs(node["y"] - y) < 1e-6
        assert node["vx"] == 0 and node["vy"] == 0
    sim.destroy()


@pytest.mark.skipif(forcegpu.isWebGPUAvailable(), reason="a GPU is present")
def test_without_a_gpu_every_compute_call_raises():
    sim = forceSimulationGPU_stopped([{}, {}])
    assert sim.isGPUEnabled() is False
    assert asyncio.run(sim.gpuReady()) is False
    assert sim.gpuBuffers() is None
    with pytest.raises(forcegpu.FlError):
        sim.tick()
    with pytest.raises(forcegpu.FlError):
        asyncio.run(sim.tickAsync(1))
    sim.destroy()


def test_forces_are_not_cpu_callables():
    with pytest.raises(RuntimeError):
        forcegpu.forceManyBody()(0.5)
