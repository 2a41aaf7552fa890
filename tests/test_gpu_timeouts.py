"""Failure detection on the device without a GPU fault: every device wait is
bounded (`wait_limit` polls). With a limit of one poll the grid barriers of
the colouring and colour-phase kernels, and the neighbour waits of the
wavefront kernel, give up; the kernels return, the host reports
AVBD_ERR_TIMEOUT, and the same process steps a fresh context normally."""
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
