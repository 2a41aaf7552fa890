"""avbd_overlap_pairs_static: the allocation-free overlap query.

Its pairs must equal the candidate pairs of a context's first step on the
same positions (no previous manifolds, no joints: exactly the bounding-sphere
overlaps), on two calls in a row sharing the one static scratch array, and
the second call must not change the device's free memory.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend_mod():
    return importlib.import_module("avbd-sandbox_gb300.backend")


def step_pairs(abi, backend_mod, s):
    gpu = backend_mod.GpuBackend(abi.default_params(**s.params))
    gpu.pack(s.world())
    gpu.step(1)
    gpu.idle()
    a, b = gpu.read_pairs()
    gpu.destroy()
    return (a.astype(np.uint64) << np.uint64(32)) | b.astype(np.uint64)


@pytest.mark.parametrize("name", ["pyramid", "pile"])
def test_static_pairs_equal_step_pairs(abi, scenes, backend_mod, name):
    torch = pytest.importorskip("torch")
    s = scenes.pyramid(layers=9) if name == "pyramid" else scenes.random_pile(300, seed=5)
    w = s.world()
    expect = step_pairs(abi, backend_mod, s)
    dev = torch.device("cuda", torch.cuda.current_device())
    pos = torch.tensor(np.ascontiguousarray(w.pos), dtype=torch.float64, device=dev)
    rad = torch.tensor(np.ascontiguousarray(w.radius), dtype=torch.float64, device=dev)
    dyn = torch.tensor((w.mass > 0).astype(np.int32), device=dev)
    cap = len(expect) + 64
    # cell: twice the largest radius below twice the median (the ground box is tested against all)
    r = np.asarray(w.radius)
    cell = 2.0 * float(r[r <= 2 * np.median(r)].max()) * (1 + 1e-6) + 1e-9
    stream = torch.cuda.current_stream()
    results, free = [], []
    for call in range(2):
        keys = torch.full((cap,), -1, dtype=torch.int64, device=dev)
        count = torch.full((1,), -7, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        backend_mod.overlap_pairs_static(w.n_bodies, pos.data_ptr(), rad.data_ptr(), dyn.data_ptr(), cell,
                                         keys.data_ptr(), cap, count.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        free.append((free_before, torch.cuda.mem_get_info()[0]))
        n = int(count.item())
        assert 0 <= n <= cap
        results.append(keys[:n].cpu().numpy().view(np.uint64).copy())
    for got in results:
        assert got.shape == expect.shape and np.array_equal(got, expect)
    assert free[1][0] == free[1][1], "the second call changed the device's free memory"


def test_static_pairs_reports_short_capacity(abi, scenes, backend_mod):
    torch = pytest.importorskip("torch")
    s = scenes.pyramid(layers=5)
    w = s.world()
    expect = step_pairs(abi, backend_mod, s)
    dev = torch.device("cuda", torch.cuda.current_device())
    pos = torch.tensor(np.ascontiguousarray(w.pos), dtype=torch.float64, device=dev)
    rad = torch.tensor(np.ascontiguousarray(w.radius), dtype=torch.float64, device=dev)
    keys = torch.zeros(8, dtype=torch.int64, device=dev)
    count = torch.zeros(1, dtype=torch.int32, device=dev)
    backend_mod.overlap_pairs_static(w.n_bodies, pos.data_ptr(), rad.data_ptr(), 0, 2.0, keys.data_ptr(), 8,
                                     count.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    # all bodies dynamic here (dynamic = NULL): the ground pairs count too
    assert int(count.item()) == len(expect) > 8


def test_static_pairs_at_the_documented_maximum(abi, scenes, backend_mod):
    """Exactly AVBD_STATIC_PAIRS_MAX_BODIES bodies fit the static scratch
    array: a sparse random cloud of that many boxes gives the pairs of a
    context's first step on the same positions."""
    torch = pytest.importorskip("torch")
    n = backend_mod.STATIC_PAIRS_MAX_BODIES
    rng = np.random.default_rng(7)
    s = scenes.Scene("cloud")
    side = int(np.ceil(n ** (1 / 3)))
    for k in range(n):
        x, y, z = k % side, (k // side) % side, k // (side * side)
        s.box((0.5, 0.5, 0.5), 100.0, 0.5, (1.2 * x + rng.uniform(-0.4, 0.4), 1.2 * y + rng.uniform(-0.4, 0.4),
                                            1.2 * z + rng.uniform(-0.4, 0.4)))
    s.params = dict(gravity=0.0)
    w = s.world()
    expect = step_pairs(abi, backend_mod, s)
    dev = torch.device("cuda", torch.cuda.current_device())
    pos = torch.tensor(np.ascontiguousarray(w.pos), dtype=torch.float64, device=dev)
    rad = torch.tensor(np.ascontiguousarray(w.radius), dtype=torch.float64, device=dev)
    cap = len(expect) + 64
    keys = torch.full((cap,), -1, dtype=torch.int64, device=dev)
    count = torch.zeros(1, dtype=torch.int32, device=dev)
    cell = 2.0 * float(np.max(w.radius)) * (1 + 1e-6) + 1e-9
    backend_mod.overlap_pairs_static(n, pos.data_ptr(), rad.data_ptr(), 0, cell, keys.data_ptr(), cap,
                                     count.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = keys[:int(count.item())].cpu().numpy().view(np.uint64)
    assert len(expect) > 0 and np.array_equal(got, expect)


def test_static_pairs_rejects_too_many_bodies(backend_mod):
    with pytest.raises(backend_mod.AvbdError) as e:
        backend_mod.overlap_pairs_static(backend_mod.STATIC_PAIRS_MAX_BODIES + 1, 1, 1, 0, 1.0, 1, 1, 1, 0)
    assert "at most 65000" in str(e.value)


def test_static_pairs_capture_into_a_graph(abi, scenes, backend_mod):
    """The call allocates nothing and never waits on the host, so it can be
    captured into a CUDA graph (a cudaMalloc inside a capture would fail it);
    replaying the graph gives the pairs of a direct call."""
    torch = pytest.importorskip("torch")
    s = scenes.random_pile(300, seed=11)
    w = s.world()
    expect = step_pairs(abi, backend_mod, s)
    dev = torch.device("cuda", torch.cuda.current_device())
    pos = torch.tensor(np.ascontiguousarray(w.pos), dtype=torch.float64, device=dev)
    rad = torch.tensor(np.ascontiguousarray(w.radius), dtype=torch.float64, device=dev)
    dyn = torch.tensor((w.mass > 0).astype(np.int32), device=dev)
    cap = len(expect) + 64
    r = np.asarray(w.radius)
    cell = 2.0 * float(r[r <= 2 * np.median(r)].max()) * (1 + 1e-6) + 1e-9
    keys = torch.full((cap,), -1, dtype=torch.int64, device=dev)
    count = torch.full((1,), -7, dtype=torch.int32, device=dev)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):  # one call outside the capture: the array's address
        backend_mod.overlap_pairs_static(w.n_bodies, pos.data_ptr(), rad.data_ptr(), dyn.data_ptr(), cell,
                                         keys.data_ptr(), cap, count.data_ptr(), side.cuda_stream)
    torch.cuda.synchronize()
    keys.fill_(-1)
    count.fill_(-7)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        backend_mod.overlap_pairs_static(w.n_bodies, pos.data_ptr(), rad.data_ptr(), dyn.data_ptr(), cell,
                                         keys.data_ptr(), cap, count.data_ptr(),
                                         torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(count.item()) == -7  # captured, not run
    g.replay()
    torch.cuda.synchronize()
    n = int(count.item())
    got = keys[:n].cpu().numpy().view(np.uint64)
    assert np.array_equal(got, expect)
