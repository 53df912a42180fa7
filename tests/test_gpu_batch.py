"""Batched builds and traces (rtg_batch_*): one set of build kernels for many
scenes and one persistent trace launch for many tasks give exactly the grids
and hits of the per-scene calls, also when captured in a CUDA graph."""
import numpy as np
import pytest

from gridrt import scenes

pytestmark = pytest.mark.gpu


def _items():
    return scenes.batched_workload(seed=777, nscenes=8, tri_range=(500, 40_000), ray_range=(1_000, 40_000))


def _upload(items):
    import torch
    d_rays = [torch.from_numpy(it.rays).cuda() for it in items]
    return d_rays


def test_batch_build_equals_scene_builds(gridlib, oracle):
    items = _items()
    ks = [2 + (i % 3) * 2 for i in range(len(items))]
    scs = []
    for it in items:
        s = gridlib.Scene(0)
        s.set_geometry(it.scene.verts, it.scene.idx)
        scs.append(s)
    b = gridlib.Batch(scs, ks, [])
    # change nothing, rebuild every grid in one batch, compare with the oracle
    b.build_async()
    assert b.check() == 0
    for s, it, k in zip(scs, items, ks):
        off, ids = s.download()
        g = oracle.Grid(it.scene.verts, it.scene.idx, k)
        assert np.array_equal(off, g.offsets) and np.array_equal(ids, g.ids)


@pytest.mark.parametrize("cell_records,heavy,refill",
                         [(False, 0, 0), (True, 32, 0), (False, 4, 0), (True, 32, 8), (False, 4, 16), (False, 0, 1)])
def test_batch_trace_equals_scene_traces(gridlib, cell_records, heavy, refill):
    """Also with cell-ordered records written by the batched build (every
    other scene) and read by the batched trace, with the batch's warp-per-ray
    pass (heavy > 0; heavy = 4 also overflows its queue), and with lane
    refill inside each task, against per-scene traces without them."""
    import torch
    items = _items()
    scs, tasks, outs = [], [], []
    d_rays = _upload(items)
    for i, it in enumerate(items):
        s = gridlib.Scene(0)
        s.set_geometry(it.scene.verts, it.scene.idx)
        if cell_records and i % 2 == 0:
            s.set_tuning(cell_records=True)
        s.set_tuning(heavy_cell=0)
        scs.append(s)
        n = it.rays.shape[0]
        if i % 3 == 2:       # any-hit task with tmax 0.5
            r = d_rays[i].clone()
            r[:, 7] = 0.5
            d_rays[i] = r
            out = torch.empty(n, dtype=torch.uint8, device="cuda")
            tasks.append((i, gridlib.RTG_MODE_ANY, r, n, out))
        else:
            out = torch.empty((n, 4), dtype=torch.int32, device="cuda")
            tasks.append((i, gridlib.RTG_MODE_NEAREST, d_rays[i], n, out))
        outs.append(out)
    b = gridlib.Batch(scs, [4] * len(items), tasks)
    b.set_tuning(heavy_cell=heavy, heavy_lanes=4 if heavy == 4 else 8, refill=refill)
    b.build_async()
    b.trace_async()
    assert b.check() == 0
    torch.cuda.synchronize()
    for (i, mode, r, n, out), s in zip(tasks, scs):
        if mode == gridlib.RTG_MODE_ANY:
            ref = s.trace_any(r.cpu().numpy())
            assert np.array_equal(out.cpu().numpy(), ref), i
        else:
            ref = s.trace_nearest(r.cpu().numpy()).view(np.int32)
            assert np.array_equal(out.cpu().numpy(), ref), i


def test_batch_graph_capture_replays(gridlib):
    import torch
    items = _items()[:4]
    scs, tasks = [], []
    d_rays = _upload(items)
    for i, it in enumerate(items):
        s = gridlib.Scene(0)
        s.set_geometry(it.scene.verts, it.scene.idx)
        scs.append(s)
        out = torch.empty((it.rays.shape[0], 4), dtype=torch.int32, device="cuda")
        tasks.append((i, gridlib.RTG_MODE_NEAREST, d_rays[i], it.rays.shape[0], out))
    b = gridlib.Batch(scs, [4] * len(items), tasks)
    stream = torch.cuda.Stream()
    b.build_async(stream.cuda_stream)       # uploads tables before capture
    b.trace_async(stream.cuda_stream)
    torch.cuda.synchronize()
    first = [t[4].clone() for t in tasks]
    for t in tasks:
        t[4].fill_(-7)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        b.build_async(stream.cuda_stream)
        b.trace_async(stream.cuda_stream)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert b.check() == 0
    for a, t in zip(first, tasks):
        assert torch.equal(a, t[4])
