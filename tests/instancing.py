"""Helpers for the two-level instancing tests: seeded instance transforms,
local-space rays computed with the library's operation order, and the
near-tie rules of tests/parity.py applied per instance."""
import numpy as np

import parity


def random_transform(rng, scale=(0.5, 2.0), shift=3.0):
    """(world_from_local, local_from_world) as float32 3x4 row-major: a
    random rotation, uniform scale and translation; the inverse is taken in
    float64 and rounded once."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    s = rng.uniform(*scale)
    t = rng.uniform(-shift, shift, size=3)
    M = np.concatenate([s * R, t[:, None]], axis=1)
    Ri = R.T / s
    inv = np.concatenate([Ri, (-Ri @ t)[:, None]], axis=1)
    return M.astype(np.float32), inv.astype(np.float32)


def translation(t):
    M = np.zeros((3, 4), np.float32)
    M[:, :3] = np.eye(3, dtype=np.float32)
    M[:, 3] = t
    inv = M.copy()
    inv[:, 3] = -np.asarray(t, np.float32)
    return M, inv


IDENTITY = translation((0.0, 0.0, 0.0))


def local_rays(rays, inv):
    """World rays taken to local space with one float32 rounding per
    operation in the order ((m0 x + m1 y) + m2 z) + m3."""
    m = np.asarray(inv, np.float32).reshape(3, 4)
    o = rays[:, 0:3].astype(np.float32)
    d = rays[:, 4:7].astype(np.float32)
    out = rays.copy()
    for i in range(3):
        a = (m[i, 0] * o[:, 0]).astype(np.float32)
        b = (m[i, 1] * o[:, 1]).astype(np.float32)
        c = (m[i, 2] * o[:, 2]).astype(np.float32)
        out[:, i] = (((a + b).astype(np.float32) + c).astype(np.float32) + m[i, 3]).astype(np.float32)
        a = (m[i, 0] * d[:, 0]).astype(np.float32)
        b = (m[i, 1] * d[:, 1]).astype(np.float32)
        c = (m[i, 2] * d[:, 2]).astype(np.float32)
        out[:, 4 + i] = ((a + b).astype(np.float32) + c).astype(np.float32)
    return out


def compare_instance_hits(gpu_hits, gpu_inst, orc_hits, orc_inst, scenes, transforms, rays, pyoracle,
                          max_tie_frac=1e-3):
    """Same (instance, id): t / u / v under parity.compare_hits on the
    instance's local rays (within 1e-5 relative of the oracle).  A different
    winner is a near-tie under the rules of parity.compare_hits (t within
    TIE_REL, or a candidate on a triangle edge), at most max_tie_frac of the
    rays."""
    n = rays.shape[0]
    gid, oid = gpu_hits["id"], orc_hits["id"]
    same = (gpu_inst == orc_inst) & (gid == oid)
    stats = {"n": n, "mismatches": int((~same).sum()), "bad_values": 0, "unexplained": 0,
             "t-tie": 0, "edge": 0, "bits_equal": 0, "values": 0}
    for j, (sc, (M, inv)) in enumerate(zip(scenes, transforms)):
        sel = np.where(same & (gpu_inst == j) & (gid >= 0))[0]
        if sel.size == 0:
            continue
        lr = local_rays(rays[sel], inv)
        sub = lambda h: {k: v[sel] for k, v in h.items()}
        st = parity.compare_hits(sub(gpu_hits), sub(orc_hits), sc.verts, sc.idx, lr, pyoracle)
        stats["bad_values"] += st["bad_values"]
        stats["bits_equal"] += st["bits_equal"]
        stats["values"] += st["values"]
    for i in np.where(~same)[0]:
        cands = []
        for inst, hid, t in ((gpu_inst[i], gid[i], gpu_hits["t"][i]), (orc_inst[i], oid[i], orc_hits["t"][i])):
            if hid < 0:
                continue
            sc = scenes[inst]
            lr = local_rays(rays[i:i + 1], transforms[inst][1])
            f64 = pyoracle.mt_f64(sc.verts, sc.idx, lr, np.array([hid], np.int32))[0]
            cands.append((float(t), f64, parity._bary_margin(f64)))
        if len(cands) == 2 and abs(cands[0][0] - cands[1][0]) <= parity.TIE_REL * max(abs(cands[1][0]), 1e-30):
            stats["t-tie"] += 1
        elif any(abs(c[2]) <= parity.EDGE_EPS for c in cands):
            stats["edge"] += 1
        else:
            stats["unexplained"] += 1
    stats["ok"] = (stats["bad_values"] == 0 and stats["unexplained"] == 0
                   and stats["mismatches"] <= max(1, int(max_tie_frac * n)))
    return stats
