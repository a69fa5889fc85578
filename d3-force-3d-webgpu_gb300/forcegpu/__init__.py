"""GB300 force-layout engine: a drop-in for forceSimulationGPU of d3-force-3d-webgpu.

    from forcegpu import forceSimulationGPU, forceLink, forceManyBody, forceCenter
    sim = forceSimulationGPU(nodes, 3).stop()
    sim.force("link", forceLink(links)).force("charge", forceManyBody()).force("center", forceCenter())
    asyncio.run(sim.tickAsync(300))

The physics runs in libforcegpu.so (sm_103a CUDA, C ABI in include/forcegpu.h); this package is
the host side: the simulation object, the force objects and the ctypes bindings.
"""
import os as _os

# Every simulation runs on three streams and a batch on two; a server runs many of them at
# once. With the CUDA default of 8 hardware work queues, streams share queues and wait on each
# other's unrelated work; 32 (the most) lets them run side by side. The setting is read when the
# process's CUDA context is created, so it only takes effect if nothing created one before.
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from ._lib import Engine, FlError, load  # noqa: E402
from .forces import (constant, forceCenter, forceCollide, forceLink,  # noqa: E402
                     forceManyBody, forceRadial, forceX, forceY, forceZ)
from .simulation import GPU_KEYS, SIMULATION_KEYS, Simulation, forceSimulationGPU, lcg  # noqa: E402


def isWebGPUAvailable():
    """The reference's probe (src/index.js): here, whether a CUDA device and the engine load."""
    try:
        e = Engine(0)
        e.close()
        return True
    except Exception:
        return False


__all__ = ["forceSimulationGPU", "forceLink", "forceManyBody", "forceCollide", "forceCenter",
           "forceRadial", "forceX", "forceY", "forceZ", "constant", "isWebGPUAvailable", "Engine",
           "FlError", "load", "lcg", "Simulation", "SIMULATION_KEYS", "GPU_KEYS"]
