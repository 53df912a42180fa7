"""GPU traversal vs the oracle: closest hit (id, t, u, v) under the near-tie
rules of tests/parity.py, shadow any-hit, and bit-identical camera rays."""
import numpy as np
import pytest

import parity
from gridrt import scenes

pytestmark = pytest.mark.gpu


def _scene(gridlib, sc, k):
    s = gridlib.Scene(0)
    s.set_geometry(sc.verts, sc.idx)
    s.build(k)
    return s


def _report(name, st):
    print(f"\n[{name}] " + ", ".join(f"{k}={v}" for k, v in st.items() if k != "unexplained_examples"))
    if st["unexplained_examples"]:
        print("  examples:", st["unexplained_examples"][:3])


def test_plane_and_debris_primary(gridlib, oracle):
    sc = scenes.plane_and_debris()
    s = _scene(gridlib, sc, 4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    rays = scenes.camera_rays(scenes.plane_and_debris_camera())
    gh = gridlib.split_hits(s.trace_nearest(rays))
    oh = g.trace_closest(rays)
    st = parity.compare_hits(gh, oh, sc.verts, sc.idx, rays, oracle)
    _report("plane primary", st)
    parity.assert_parity(st)


def test_camera_kernel_matches_explicit_rays(gridlib, oracle):
    import torch
    sc = scenes.plane_and_debris()
    s = _scene(gridlib, sc, 4)
    for order in ("scanline", "morton8"):
        cam = scenes.plane_and_debris_camera(256, 128)
        rays = scenes.camera_rays(cam, order)
        host = s.trace_nearest(rays).view(np.int32)
        d_hits = torch.empty((rays.shape[0], 4), dtype=torch.int32, device="cuda")
        s.trace_camera_device(cam, d_hits, order=order)
        torch.cuda.synchronize()
        dev = d_hits.cpu().numpy()
        # identical rays give identical traversal, so every word matches
        assert np.array_equal(host, dev), order


def test_shadow_any_hit(gridlib, oracle):
    import torch
    sc = scenes.plane_and_debris()
    s = _scene(gridlib, sc, 4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    cam = scenes.plane_and_debris_camera()
    n = cam.width * cam.height
    d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    d_occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    d_sr = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    s.trace_frame_device(cam, scenes.PLANE_LIGHT, d_hits, d_occ, d_sr)
    torch.cuda.synchronize()
    occ = d_occ.cpu().numpy()
    sr = d_sr.cpu().numpy()
    hits = gridlib.split_hits(d_hits.cpu().numpy())
    has = sr[:, 7] >= 0
    assert (occ[~has] == 2).all()
    assert (hits["id"][has] >= 0).all()
    srh = np.ascontiguousarray(sr[has])
    ref = g.trace_any(srh)
    parity.check_occlusion("shadow", s, g, gridlib.split_hits, srh, occ[has], ref, sc.verts, sc.idx, oracle)
    # the host any-hit entry point agrees with the fused frame call
    occ2 = s.trace_any(sr[has])
    assert np.array_equal(occ2, occ[has])


@pytest.mark.parametrize("k", [2, 4, 8])
def test_deforming_sphere_primary(gridlib, oracle, k):
    sc = scenes.deforming_sphere(5)
    s = _scene(gridlib, sc, k)
    g = oracle.Grid(sc.verts, sc.idx, k)
    rays = scenes.camera_rays(scenes.deforming_sphere_camera(512, 512))
    gh = gridlib.split_hits(s.trace_nearest(rays))
    oh = g.trace_closest(rays)
    st = parity.compare_hits(gh, oh, sc.verts, sc.idx, rays, oracle)
    _report(f"sphere k={k}", st)
    parity.assert_parity(st)


def test_random_rays_inside_box(gridlib, oracle):
    sc = scenes.plane_and_debris()
    s = _scene(gridlib, sc, 4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    rng = np.random.default_rng(7)
    rays = scenes.random_rays(rng, 200_000, (-1.0, 0.0, -1.0), (1.0, 1.0, 1.0))
    gh = gridlib.split_hits(s.trace_nearest(rays))
    oh = g.trace_closest(rays)
    st = parity.compare_hits(gh, oh, sc.verts, sc.idx, rays, oracle)
    _report("random rays", st)
    parity.assert_parity(st)
    # any-hit with a finite tmax
    rays[:, 7] = 0.3
    occ = s.trace_any(rays)
    ref = g.trace_any(rays)
    parity.check_occlusion("random rays", s, g, gridlib.split_hits, rays, occ, ref, sc.verts, sc.idx, oracle)


def test_skewed_density_subsample(gridlib, oracle):
    sc = scenes.skewed_density()
    s = _scene(gridlib, sc, 4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    rays = scenes.camera_rays(scenes.skewed_density_camera(256, 256))
    gh = gridlib.split_hits(s.trace_nearest(rays))
    oh = g.trace_closest(rays)
    st = parity.compare_hits(gh, oh, sc.verts, sc.idx, rays, oracle)
    _report("skewed", st)
    parity.assert_parity(st)


def test_counters_match_oracle(gridlib, oracle):
    sc = scenes.plane_and_debris()
    s = _scene(gridlib, sc, 4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    rays = scenes.camera_rays(scenes.plane_and_debris_camera())
    s.counters(reset=True)
    s.trace_nearest(rays, counters=True)
    c = s.counters(reset=True)
    _, oc = g.trace_closest(rays, counters=True)
    # same DDA: cells visited equal exactly unless a near-tie ended a walk in
    # a different cell
    assert c["rays"] == rays.shape[0]
    assert abs(c["cells"] - int(oc[:, 0].sum())) <= 1e-4 * oc[:, 0].sum()
    assert abs(c["tests"] - int(oc[:, 1].sum())) <= 1e-3 * oc[:, 1].sum()


def test_results_independent_of_launch_tuning(gridlib, oracle):
    """Launch shape (empty-cell run, persistent vs one-shot grid, lane refill
    threshold, threads per block, lanes per ray) never changes a result bit."""
    import torch
    sc = scenes.deforming_sphere(3)
    s = _scene(gridlib, sc, 4)
    cam = scenes.deforming_sphere_camera(256, 256)
    n = cam.width * cam.height
    ref = None
    for er, persistent, refill, block in [(e, p, 0, 128) for e in (2, 4, 8, 16) for p in (True, False)] + \
            [(e, p, r, 128) for e in (2, 8) for p in (True, False) for r in (1, 16, 32)] + \
            [(4, p, r, b) for p in (True, False) for r in (0, 16) for b in (64, 256)] + \
            [(4, True, 0, -2), (4, True, 0, -4)]:
        if True:
            # block -2 / -4: every ray walked by a group of 2 / 4 lanes
            lanes = -block if block < 0 else 1
            s.set_tuning(empty_run=er, persistent=persistent, refill=refill, block=max(block, 64), lanes=lanes)
            d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
            d_sr = torch.empty((n, 8), dtype=torch.float32, device="cuda")
            d_occ = torch.empty(n, dtype=torch.uint8, device="cuda")
            s.trace_frame_device(cam, scenes.SPHERE_LIGHT, d_hits, d_occ, d_sr, order="morton8")
            torch.cuda.synchronize()
            out = (d_hits.cpu().numpy(), d_occ.cpu().numpy(), d_sr.cpu().numpy().view(np.uint32))
            if ref is None:
                ref = out
            else:
                for a, b in zip(ref, out):
                    assert np.array_equal(a, b), (er, persistent, refill, block)


def _frame(s, cam, order="morton8"):
    import torch
    n = cam.width * cam.height
    d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    d_sr = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    d_occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    s.trace_frame_device(cam, scenes.SPHERE_LIGHT, d_hits, d_occ, d_sr, order=order)
    torch.cuda.synchronize()
    return d_hits.cpu().numpy(), d_occ.cpu().numpy(), d_sr.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("heavy", [1, 16, 64])
def test_heavy_cell_deferral_is_exact(gridlib, oracle, heavy):
    """Rays handed to the warp-per-ray pass (lists longer than `heavy`) get
    the same hit words, shadow rays and occlusion bits as the one-lane walk,
    with and without cell-ordered records; heavy=1 on a 1024^2 frame also
    overflows the per-launch queue, so the in-place fallback runs too."""
    sc = scenes.deforming_sphere(2)
    s = _scene(gridlib, sc, 8)
    cam = scenes.deforming_sphere_camera(1024, 1024) if heavy == 1 else scenes.deforming_sphere_camera(512, 512)
    s.set_tuning(heavy_cell=0, cell_records=False)
    ref = _frame(s, cam)
    for crec, lanes, refill in ((False, 8, 0), (True, 4, 16), (True, 16, 1), (False, 32, 8)):
        s.set_tuning(heavy_cell=heavy, cell_records=crec, heavy_lanes=lanes, refill=refill)
        s.build(8)
        out = _frame(s, cam)
        for a, b in zip(ref, out):
            assert np.array_equal(a, b), (heavy, crec, lanes, refill)
    # the nearest / any entry points on explicit rays agree as well
    rng = np.random.default_rng(11)
    rays = scenes.random_rays(rng, 50_000, (-1.2, -1.2, -1.2), (1.2, 1.2, 1.2))
    s.set_tuning(heavy_cell=0, cell_records=False)
    s.build(8)
    h0 = s.trace_nearest(rays)
    rays_any = rays.copy()
    rays_any[:, 7] = 0.5
    o0 = s.trace_any(rays_any)
    s.set_tuning(heavy_cell=heavy, cell_records=True, refill=0)
    s.build(8)
    assert np.array_equal(h0.view(np.int32), s.trace_nearest(rays).view(np.int32))
    assert np.array_equal(o0, s.trace_any(rays_any))
    s.set_tuning(refill=16)
    assert np.array_equal(h0.view(np.int32), s.trace_nearest(rays).view(np.int32))
    assert np.array_equal(o0, s.trace_any(rays_any))


def test_heavy_cell_counters_match_oracle(gridlib, oracle):
    """Deferred rays are counted once (by the warp-per-ray pass)."""
    sc = scenes.deforming_sphere(0)
    s = _scene(gridlib, sc, 8)
    s.set_tuning(heavy_cell=32)
    g = oracle.Grid(sc.verts, sc.idx, 8)
    rays = scenes.camera_rays(scenes.deforming_sphere_camera(512, 512), "morton8")
    s.counters(reset=True)
    s.trace_nearest(rays, counters=True)
    c = s.counters(reset=True)
    _, oc = g.trace_closest(rays, counters=True)
    assert c["rays"] == rays.shape[0]
    assert abs(c["cells"] - int(oc[:, 0].sum())) <= 1e-4 * oc[:, 0].sum()
    assert abs(c["tests"] - int(oc[:, 1].sum())) <= 1e-3 * oc[:, 1].sum()


@pytest.mark.parametrize("ntris", [1 << 16, 1 << 18])
def test_huge_list_block_pass_is_exact(gridlib, oracle, ntris):
    """Lists above 2,048 entries (59,000 / 236,000 triangles in a 0.1^3
    cluster, k = 4) go from the group pass to the block-per-ray pass -- rays
    at lists of 16,384+ entries (the larger scene) from the back of its
    queue, claimed first: hit words, frame outputs, occlusion and traversal
    counters equal the one-lane walk's (with the records read through the id
    lists and in cell order), and the hits meet the oracle's near-tie
    rules."""
    sc = scenes.skewed_density(n=ntris)
    s = _scene(gridlib, sc, 4)      # a synchronous build: the scene knows its longest list
    g = oracle.Grid(sc.verts, sc.idx, 4)
    longest = int(np.diff(np.asarray(g.offsets)).max())
    assert longest > (16384 if ntris > 1 << 16 else 2048), longest
    cam = scenes.skewed_density_camera(256, 256)
    rays = scenes.camera_rays(cam, "morton8")
    rng = np.random.default_rng(3)
    rays_any = scenes.random_rays(rng, 40_000, (-0.06, -0.06, -0.06), (0.06, 0.06, 0.06))
    rays_any[:, 7] = 0.05
    s.set_tuning(heavy_cell=0)
    s.counters(reset=True)
    h0 = s.trace_nearest(rays, counters=True)
    c0 = s.counters(reset=True)
    o0 = s.trace_any(rays_any)
    f0 = _frame(s, cam)
    for lanes, records in ((8, False), (32, False), (32, True)):
        s.set_tuning(heavy_cell=32, heavy_lanes=lanes, cell_records=records)
        if records:
            s.build(4)              # the records are written by the build
        h1 = s.trace_nearest(rays, counters=True)
        c1 = s.counters(reset=True)
        assert np.array_equal(h0.view(np.int32), h1.view(np.int32)), lanes
        assert c1 == c0, (c0, c1)
        assert np.array_equal(o0, s.trace_any(rays_any)), lanes
        for a, b in zip(f0, _frame(s, cam)):
            assert np.array_equal(a, b), lanes
    # every ray walked by a group of lanes from its start, crowded lists
    # still handed to the block-per-ray pass
    for group in (2, 4):
        s.set_tuning(lanes=group)
        assert np.array_equal(h0.view(np.int32), s.trace_nearest(rays).view(np.int32)), group
        assert np.array_equal(o0, s.trace_any(rays_any)), group
        for a, b in zip(f0, _frame(s, cam)):
            assert np.array_equal(a, b), group
    s.set_tuning(lanes=1)
    st = parity.compare_hits(gridlib.split_hits(h0), g.trace_closest(rays), sc.verts, sc.idx, rays, oracle)
    _report("huge lists", st)
    parity.assert_parity(st)


@pytest.mark.parametrize("case", ["sphere", "cluster"])
def test_frame_equals_camera_then_any(gridlib, case):
    """The frame call (each camera ray's shadow ray traced in the same lane,
    deferred passes included) gives exactly the hits, shadow-ray slots and
    occlusion of a camera launch followed by an any-hit launch over the
    slots -- with deferral, lane refill and, for the dense cluster, the
    block-per-ray pass."""
    import torch
    if case == "sphere":
        sc, k = scenes.deforming_sphere(4), 8
        cam, light = scenes.deforming_sphere_camera(512, 512), scenes.SPHERE_LIGHT
    else:
        sc, k = scenes.skewed_density(n=1 << 16), 4
        cam, light = scenes.skewed_density_camera(256, 256), (0.3, 1.5, 0.4)
    s = _scene(gridlib, sc, k)
    n = cam.width * cam.height
    for heavy, refill in ((0, 0), (32, 0), (32, 16)):
        s.set_tuning(heavy_cell=heavy, refill=refill)
        d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
        d_sr = torch.empty((n, 8), dtype=torch.float32, device="cuda")
        d_occ = torch.empty(n, dtype=torch.uint8, device="cuda")
        s.trace_camera_device(cam, d_hits, light, d_sr, order="morton8")
        s.trace_any_device(d_sr, n, d_occ)
        torch.cuda.synchronize()
        ref = (d_hits.cpu().numpy(), d_sr.cpu().numpy().view(np.uint32), d_occ.cpu().numpy())
        f_hits = torch.empty_like(d_hits)
        f_sr = torch.empty_like(d_sr)
        f_occ = torch.empty_like(d_occ)
        s.trace_frame_device(cam, light, f_hits, f_occ, f_sr, order="morton8")
        torch.cuda.synchronize()
        out = (f_hits.cpu().numpy(), f_sr.cpu().numpy().view(np.uint32), f_occ.cpu().numpy())
        for a, b in zip(ref, out):
            assert np.array_equal(a, b), (case, heavy, refill)
        assert (ref[2] != 2).sum() > 0


def test_diffuse_secondary_rays(gridlib, oracle):
    """Skewed-density workload: primary camera rays, then one cosine-weighted
    diffuse ray per hit generated on the device; both generations match the
    oracle under the near-tie rules (the GPU's own secondary rays are fed to
    the oracle)."""
    import torch
    sc = scenes.skewed_density(n=1 << 18)
    s = _scene(gridlib, sc, 4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    cam = scenes.skewed_density_camera(256, 256)
    n = cam.width * cam.height
    d_hits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    d_sec = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    s.trace_camera_diffuse_device(cam, 1234, d_hits, d_sec, order="morton8")
    torch.cuda.synchronize()
    sec = d_sec.cpu().numpy()
    prim = gridlib.split_hits(d_hits.cpu().numpy())
    has = sec[:, 7] > 0
    assert int(has.sum()) == int((prim["id"] >= 0).sum())
    d = sec[has, 4:7]
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-4)
    rays = np.ascontiguousarray(sec[has])
    gh = gridlib.split_hits(s.trace_nearest(rays))
    oh = g.trace_closest(rays)
    st = parity.compare_hits(gh, oh, sc.verts, sc.idx, rays, oracle)
    _report("skewed diffuse", st)
    parity.assert_parity(st)
    # the same seed gives the same rays
    d_sec2 = torch.empty_like(d_sec)
    s.trace_camera_diffuse_device(cam, 1234, d_hits, d_sec2, order="morton8")
    torch.cuda.synchronize()
    assert torch.equal(d_sec, d_sec2)


def test_frame_async_matches_frame(gridlib):
    """rtg_trace_frame_async: frames of changing keyframes enqueued two
    ahead of the host's wait, into alternating pinned buffers, give exactly
    the synchronous rtg_trace_frame results of their keyframes."""
    import torch
    v, idx, nrm = scenes.sphere_mesh(40, 80)
    s = gridlib.Scene(0)
    s.set_geometry(v, idx)
    cam = scenes.deforming_sphere_camera(256, 256)
    n = cam.width * cam.height
    light = scenes.SPHERE_LIGHT
    keys = [np.ascontiguousarray(scenes.deform(v, nrm, f), np.float32) for f in range(3)]
    ref = []
    for kv in keys:
        s.update_vertices(kv, kv.shape[0], False)
        s.build(4)
        h, o = np.empty((n, 4), np.int32), np.empty(n, np.uint8)
        s.trace_frame(cam, light, h, o, order="morton8")
        ref.append((h, o))
    hits = [torch.empty((n, 4), dtype=torch.int32).pin_memory() for _ in range(2)]
    occ = [torch.empty(n, dtype=torch.uint8).pin_memory() for _ in range(2)]
    tickets = []
    for i in range(7):
        s.update_vertices(keys[i % 3], keys[i % 3].shape[0], False)
        s.build_async(4)
        tickets.append(s.trace_frame_async(cam, light, hits[i % 2], occ[i % 2], order="morton8"))
        if i:
            s.trace_frame_wait(tickets[i - 1])
            h, o = ref[(i - 1) % 3]
            assert np.array_equal(hits[(i - 1) % 2].numpy(), h), i - 1
            assert np.array_equal(occ[(i - 1) % 2].numpy(), o), i - 1
    s.trace_frame_wait(tickets[-1])
    h, o = ref[6 % 3]
    assert np.array_equal(hits[0].numpy(), h) and np.array_equal(occ[0].numpy(), o)
    assert tickets == list(range(7))
    assert (ref[0][1] != 2).sum() > 0          # the frames have shadow rays
    with pytest.raises(gridlib.GridRTError):
        s.trace_frame_wait(7)


@pytest.mark.parametrize("persistent", [True, False])
def test_two_frames_in_flight_match_one_at_a_time(gridlib, persistent):
    """Two scenes of one mesh with a frame in flight on each give exactly the
    hits and occlusion of the same frames one at a time on one scene: frames
    2j and 2j + 1 deformed, rebuilt and traced on their scenes' own streams
    as two branches of one CUDA graph, and frames alternating over the two
    scenes with staged host keyframes and asynchronous read-back.  With
    persistent trace grids and with one-shot grids of 64-thread blocks (whose
    blocks from the two frames share the SMs)."""
    import torch
    v, idx, nrm = scenes.sphere_mesh()
    cam = scenes.deforming_sphere_camera(512, 512)
    n = cam.width * cam.height
    light = scenes.SPHERE_LIGHT
    dev = torch.device("cuda", 0)
    d_base = torch.from_numpy(v).to(dev)
    d_nrm = torch.from_numpy(nrm).to(dev)

    def make():
        s = gridlib.Scene(0)
        s.set_geometry(v, idx)
        if persistent:
            s.set_tuning(persistent=True)
        else:
            s.set_tuning(persistent=False, block=64, heavy_cell=48)
        return (s, torch.cuda.ExternalStream(s.stream, device=dev),
                torch.empty((n, 4), dtype=torch.int32, device=dev), torch.empty(n, dtype=torch.uint8, device=dev),
                torch.empty((n, 8), dtype=torch.float32, device=dev))

    a, b = make(), make()
    for sc in (a[0], b[0]):                    # capacities for every frame
        for f in range(4):
            sc.deform(d_base, d_nrm, 0.05, 3.0, 0.3 * f)
            sc.build(4)

    def frame(on, f):
        sc, st, hits, occ, sr = on
        with torch.cuda.stream(st):
            sc.deform(d_base, d_nrm, 0.05, 3.0, 0.3 * f)
            sc.build_async(4)
            sc.trace_frame_device(cam, light, hits, occ, sr, order="morton8")

    ref = []
    for f in range(4):
        frame(a, f)
        torch.cuda.synchronize()
        ref.append((a[2].cpu().numpy(), a[3].cpu().numpy()))
    assert (ref[0][1] != 2).sum() > 0          # the frames have shadow rays
    for j in range(2):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=a[1]):
            fork = torch.cuda.Event()
            fork.record(a[1])
            b[1].wait_event(fork)
            frame(a, 2 * j)
            frame(b, 2 * j + 1)
            join = torch.cuda.Event()
            join.record(b[1])
            a[1].wait_event(join)
        for _ in range(2):
            g.replay()
            torch.cuda.synchronize()
            for on, f in ((a, 2 * j), (b, 2 * j + 1)):
                assert np.array_equal(on[2].cpu().numpy(), ref[f][0]), f
                assert np.array_equal(on[3].cpu().numpy(), ref[f][1]), f
        del g
    assert a[0].build_check() == 0 and b[0].build_check() == 0

    # host keyframes, frames alternating over the two scenes
    nv = v.shape[0]
    keys = [torch.from_numpy(np.ascontiguousarray(scenes.deform(v, nrm, f), np.float32)).pin_memory()
            for f in range(4)]
    href = []
    for f in range(4):
        a[0].update_vertices(keys[f].numpy(), nv, False)
        a[0].build(4)
        h, o = np.empty((n, 4), np.int32), np.empty(n, np.uint8)
        a[0].trace_frame(cam, light, h, o, order="morton8")
        href.append((h, o))
    scs = (a[0], b[0])
    copies = [torch.cuda.Stream() for _ in scs]
    hits = [torch.empty((n, 4), dtype=torch.int32).pin_memory() for _ in range(2)]
    occ = [torch.empty(n, dtype=torch.uint8).pin_memory() for _ in range(2)]
    for j, sc in enumerate(scs):
        sc.stage_vertices(keys[j], nv, copies[j].cuda_stream)

    def check(f):
        assert np.array_equal(hits[f % 2].numpy(), href[f % 4][0]), f
        assert np.array_equal(occ[f % 2].numpy(), href[f % 4][1]), f

    prev = None
    for f in range(9):
        sc = scs[f % 2]
        sc.build_async(4)
        sc.stage_vertices(keys[(f + 2) % 4], nv, copies[f % 2].cuda_stream)
        t = (sc, sc.trace_frame_async(cam, light, hits[f % 2], occ[f % 2], order="morton8"), f)
        if prev is not None:
            prev[0].trace_frame_wait(prev[1])
            check(prev[2])
        prev = t
    prev[0].trace_frame_wait(prev[1])
    check(prev[2])
    assert a[0].build_check() == 0 and b[0].build_check() == 0


def test_two_dense_cluster_scenes_in_flight(gridlib):
    """Two scenes of the dense-cluster scene, each rebuilt and traced
    (camera rays writing diffuse secondaries, then the secondaries) on its
    own stream at the same time, give exactly the results of the same steps
    one at a time: cluster sorts, deferral and the staged block-per-ray pass
    included."""
    import torch
    sc, k = scenes.skewed_density(n=1 << 16), 4
    cam = scenes.skewed_density_camera(256, 256)
    n = cam.width * cam.height
    dev = torch.device("cuda", 0)

    def make():
        s = gridlib.Scene(0)
        s.set_geometry(sc.verts, sc.idx)
        s.build(k)
        s.set_tuning(heavy_cell=32, heavy_lanes=16, refill=16, cell_records=True)
        return (s, torch.cuda.ExternalStream(s.stream, device=dev), torch.empty((n, 4), dtype=torch.int32, device=dev),
                torch.empty((n, 8), dtype=torch.float32, device=dev), torch.empty((n, 4), dtype=torch.int32, device=dev))

    def step(on, seed):
        g, st, hits, sec, hits2 = on
        with torch.cuda.stream(st):
            g.build_async(k)
            g.trace_camera_diffuse_device(cam, seed, hits, sec, order="morton8")
            g.trace_nearest_device(sec, n, hits2)

    def result(on):
        return [x.cpu().numpy().view(np.uint32) for x in on[2:]]

    a, b = make(), make()
    ref = {}
    for seed in range(1, 5):
        step(a, seed)
        torch.cuda.synchronize()
        ref[seed] = result(a)
    assert (ref[1][0][:, 0].view(np.int32) >= 0).sum() > 0
    for j in range(2):
        fork, join = torch.cuda.Event(), torch.cuda.Event()
        fork.record(a[1])
        b[1].wait_event(fork)
        step(a, 1 + 2 * j)
        step(b, 2 + 2 * j)
        join.record(b[1])
        a[1].wait_event(join)
        torch.cuda.synchronize()
        for on, seed in ((a, 1 + 2 * j), (b, 2 + 2 * j)):
            for got, want in zip(result(on), ref[seed]):
                assert np.array_equal(got, want), seed
    assert a[0].build_check() == 0 and b[0].build_check() == 0
