"""The CUDA backend against the reference's headless GPU-test contracts
(test/gpu_headless.mjs:252-286, 753-775, 832-860), with the scenes of
tests/test_oracle_headless_contracts.py: a hash-twin sphere pair gives one
pair, one manifold and one contact, as in the oracle; the 45-degree box stack
keeps a manifold of 8 contacts; the cube column's warm start carries the
contact penalty above 100 x penaltyMin.
"""
import importlib

import numpy as np
import pytest

from oracle import Oracle
from test_oracle_headless_contracts import cube_column, hash_twin, octagon_stack

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend_mod():
    return importlib.import_module("avbd-sandbox_gb300.backend")


def test_hash_twin_single_pair(abi, scenes, backend_mod):
    s = hash_twin(scenes)
    params = abi.default_params(**s.params)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(s.world())
    gpu.step(1)
    a, b = gpu.read_pairs()
    assert len(a) == 1
    o = Oracle(params, s.world())
    o.step(1)
    assert gpu.read_state(manifolds=True).manifold_dict() == o.state().manifold_dict()


def test_maximum_width_manifold(abi, scenes, backend_mod):
    s = octagon_stack(scenes)
    gpu = backend_mod.GpuBackend(abi.default_params(**s.params))
    gpu.pack(s.world())
    gpu.step(30)
    widest = max(c for c, _ in gpu.read_state(manifolds=True).manifold_dict().values())
    assert widest == 8


def test_warm_start_accumulates_penalty(abi, scenes, backend_mod):
    s = cube_column(scenes)
    params = abi.default_params(**s.params)
    gpu = backend_mod.GpuBackend(params)
    gpu.pack(s.world())
    gpu.step(150)
    st = gpu.read_state(manifolds=True)
    live = np.where(st.m_num_contacts[:st.m_count] > 0)[0]
    assert len(live) > 0
    peak = max(float(np.max(st.m_penalty[m, :st.m_num_contacts[m]])) for m in live)
    assert peak > 100 * params.penalty_min
