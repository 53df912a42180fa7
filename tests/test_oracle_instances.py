"""The oracle's two-level instancing (restating Context::instantiateGeometry,
IAccStructBuilder::buildInstance and IAccStruct::traceNearestInstance):
identity and duplicate instances reduce to the one-geometry trace bit for bit,
and transformed instances agree with a float64 brute force in world space."""
import numpy as np

import instancing as ins
from gridrt import scenes


def _rays(rng, n, lo, hi):
    return scenes.random_rays(rng, n, lo, hi)


def test_identity_instance_is_the_single_trace(oracle):
    sc = scenes.plane_and_debris()
    g = oracle.Grid(sc.verts, sc.idx, 4)
    I = oracle.Instances([(g, *ins.IDENTITY)])
    rays = scenes.camera_rays(scenes.plane_and_debris_camera(128, 128))
    h1 = g.trace_closest(rays)
    h2, inst, _ = I.trace(rays)
    for k in ("id", "t", "u", "v"):
        assert np.array_equal(h1[k].view(np.uint32), h2[k].view(np.uint32)), k
    assert np.array_equal(inst, np.where(h1["id"] >= 0, 0, -1))


def test_duplicate_instances_keep_the_first(oracle):
    """A later instance wins only with a strictly closer hit: two copies of
    the same geometry give the single trace, always from instance 0."""
    sc = scenes.tiny_scene(3, 2000)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    I = oracle.Instances([(g, *ins.IDENTITY), (g, *ins.IDENTITY)])
    rng = np.random.default_rng(5)
    lo, hi = sc.verts.min(0) - 0.2, sc.verts.max(0) + 0.2
    rays = _rays(rng, 5000, lo, hi)
    h1 = g.trace_closest(rays)
    h2, inst, _ = I.trace(rays)
    assert np.array_equal(h1["id"], h2["id"])
    assert np.array_equal(h1["t"].view(np.uint32), h2["t"].view(np.uint32))
    assert ((inst == 0) | (h1["id"] < 0)).all() and (inst[h1["id"] < 0] == -1).all()


def test_transformed_instances_match_float64_brute_force(oracle):
    rng = np.random.default_rng(11)
    base = [scenes.tiny_scene(s, 1500, spread=0.8, size=0.15) for s in (1, 2)]
    items, scs, tfs = [], [], []
    for j in range(5):
        sc = base[j % len(base)]
        M, inv = ins.random_transform(rng, shift=1.5)
        items.append((oracle.Grid(sc.verts, sc.idx, 4), M, inv))
        scs.append(sc)
        tfs.append((M, inv))
    I = oracle.Instances(items)
    rays = _rays(rng, 4000, (-2.5, -2.5, -2.5), (2.5, 2.5, 2.5))
    h, inst, occ = I.trace(rays)
    # brute force: every triangle of every instance in world space, float64
    best_t = np.full(rays.shape[0], np.inf)
    best_j = np.full(rays.shape[0], -1)
    o = rays[:, 0:3].astype(np.float64)
    d = rays[:, 4:7].astype(np.float64)
    for j, (sc, (M, inv)) in enumerate(zip(scs, tfs)):
        Md = M.astype(np.float64)
        v = [sc.verts[sc.idx[:, k]].astype(np.float64) @ Md[:, :3].T + Md[:, 3] for k in range(3)]
        e1, e2 = v[1] - v[0], v[2] - v[0]
        for t0 in range(0, rays.shape[0], 500):
            oo, dd = o[t0:t0 + 500, None, :], d[t0:t0 + 500, None, :]
            p = np.cross(dd, e2[None])
            det = (e1[None] * p).sum(-1)
            tv = oo - v[0][None]
            u = (tv * p).sum(-1) / det
            q = np.cross(tv, e1[None])
            w = (dd * q).sum(-1) / det
            t = (e2[None] * q).sum(-1) / det
            ok = (u >= 0) & (w >= 0) & (u + w <= 1) & (t >= 2e-4)
            t = np.where(ok, t, np.inf)
            tm = t.min(1)
            better = tm < best_t[t0:t0 + 500]
            best_t[t0:t0 + 500] = np.where(better, tm, best_t[t0:t0 + 500])
            best_j[t0:t0 + 500] = np.where(better, j, best_j[t0:t0 + 500])
    hit = np.isfinite(best_t)
    agree = (hit == (h["id"] >= 0))
    # misses / hits agree except where the float64 hit lies on an edge or the ray grazes
    assert agree.mean() > 0.995, agree.mean()
    both = hit & (h["id"] >= 0)
    rel = np.abs(h["t"][both] - best_t[both]) / best_t[both]
    assert np.median(rel) < 1e-6 and (rel < 1e-3).mean() > 0.995
    # occlusion with tmax = FLT_MAX is "any hit"
    assert np.array_equal(occ.astype(bool), h["id"] >= 0)


def test_instance_box_follows_the_reference_expansion(oracle):
    """Identity: the grid box enlarged by 1% again; a pure translation moves it."""
    sc = scenes.plane_and_debris()
    g = oracle.Grid(sc.verts, sc.idx, 4)
    M, inv = ins.translation((10.0, 0.0, 0.0))
    I = oracle.Instances([(g, *ins.IDENTITY), (g, M, inv)])
    bmin = np.array(g.info.bmin, np.float32)
    bmax = np.array(g.info.bmax, np.float32)
    s = (np.abs(bmax - bmin) * np.float32(0.01)).astype(np.float32)
    assert np.array_equal(I.boxes[0, :3], (bmin - s).astype(np.float32))
    assert np.array_equal(I.boxes[0, 3:], (bmax + s).astype(np.float32))
    assert np.array_equal(I.box[:3], I.boxes[0, :3])
    assert I.box[3] == I.boxes[1, 3] and I.box[3] > 10.0
