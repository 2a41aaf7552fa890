"""Failure detection on the device without a GPU fault: every device wait is
bounded. With `wait_limit` = 1 poll the first grid barrier of the colouring
kernel gives up (and every later wait then leaves through the timeout flag);
with only `neighbor_wait_limit` = 1 the grid barriers keep their default
limit and the neighbour-progress waits themselves run out: the wavefront
kernel's (schedule 1) and the colour-phase kernel's tail segment (schedule
0). Each time the kernels return, the host reports AVBD_ERR_TIMEOUT, and the
same process steps a fresh context normally."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend_mod():
    return importlib.import_module("avbd-sandbox_gb300.backend")


@pytest.mark.parametrize("schedule", [0, 1])
def test_wait_gives_up_and_reports_timeout(abi, scenes, backend_mod, schedule):
    s = scenes.pyramid(layers=8)
    gpu = backend_mod.GpuBackend(abi.default_params(**s.params, schedule=schedule, wait_limit=1))
    gpu.pack(s.world())
    gpu.step(3)
    with pytest.raises(backend_mod.AvbdError) as e:
        gpu.idle()
    assert e.value.code == abi.AVBD_ERR_TIMEOUT
    gpu.destroy()
    # the device and the library stay usable: a fresh context steps normally
    ok = backend_mod.GpuBackend(abi.default_params(**s.params, schedule=schedule))
    ok.pack(s.world())
    ok.step(5)
    ok.idle()
    assert np.all(np.isfinite(ok.read_state().pos))


@pytest.mark.parametrize("schedule", [0, 1])
def test_neighbour_wait_gives_up_and_reports_timeout(abi, scenes, backend_mod, schedule):
    """A hanging chain (links in two thin colours, which the colour-phase
    schedule with an explicit tail_div runs in its tail segment; the
    automatic rule keeps a barrier per colour for so few colours) and a spring
    chain: a body of the second colour reaches its wait while its
    first-colour neighbour is still being solved, and one poll is not
    enough."""
    s = scenes.heavy_chain(links=8, springs=10)
    gpu = backend_mod.GpuBackend(abi.default_params(**s.params, schedule=schedule, neighbor_wait_limit=1, tail_div=8))
    gpu.pack(s.world())
    gpu.step(5)
    with pytest.raises(backend_mod.AvbdError) as e:
        gpu.idle()
    assert e.value.code == abi.AVBD_ERR_TIMEOUT
    gpu.destroy()
    ok = backend_mod.GpuBackend(abi.default_params(**s.params, schedule=schedule))
    ok.pack(s.world())
    ok.step(5)
    ok.idle()
    assert np.all(np.isfinite(ok.read_state().pos))
