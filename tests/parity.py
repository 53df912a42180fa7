"""Hit-parity rules shared by the GPU tests.

The device walk mirrors the reference's 3D-DDA (same cells, same lists, same
per-cell acceptance window) and decides hits with Moller-Trumbore, where the
reference decides them with Wald's projection test
(src/rtcore/RayTriIntersection.cpp:12-48).  The values the device reports for
the winning triangle are Wald's -- hitWald's f, lambda and mue evaluated on the
triangle's TriAccel record (src/rtcore/Triangle.cpp:11-55) in the reference's
operation order -- so per ray:

* same triangle id  -> t, u and v each within 1e-5 relative of the oracle's
                       (T_REL; expected: the same bits, and the number of
                       bit-equal values is reported beside it)
* different ids, or hit / miss: accepted only as a documented near-tie
    - "t-tie":  both hit and the two t differ by less than 1e-6 relative
    - "edge":   the FP64 Moller-Trumbore recomputation puts the triangle that
                one side picked and the other did not within 1e-5 of one of
                its edges (barycentric margin): the two float tests round
                across that edge
  anything else is a failure, and near-ties may be at most `max_tie_frac` of
  the rays.

The max and mean error of both sides' t / u / v against an FP64 recomputation
are reported, not asserted: FP32 values of a grazing or far-away small
triangle are that far from FP64 in the reference itself.

Shadow rays (any-hit) report no triangle; a disagreement on occlusion is
explained through the closest hit, on the same ray, of the side that reports
occlusion (the occluding triangle): "edge" as above, or "tmax" / "tnear" when
that triangle's FP64 t lies within 1e-5 (relative, floored at 1) of the ray's
tmax or of the window's lower bound tnear - 1e-4, where the two float tests
round across the bound.
"""
from __future__ import annotations

import numpy as np

T_REL = 1e-5
TIE_REL = 1e-6
EDGE_EPS = 1e-5
BOUND_REL = 1e-5
HIT_EPSILON = 1e-4


def _bary_margin(f64row):
    t, u, v = f64row
    return min(u, v, 1.0 - u - v)


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-30)


def compare_hits(gpu: dict, orc: dict, verts, idx, rays, pyoracle, max_unexplained: int = 0,
                 max_tie_frac: float = 1e-3) -> dict:
    gid, oid = gpu["id"], orc["id"]
    n = gid.shape[0]
    same = gid == oid
    both = same & (gid >= 0)
    errs = {}
    bad_vals = 0
    bits_equal = 0
    for q in ("t", "u", "v"):
        g = np.ascontiguousarray(gpu[q][both], np.float32)
        o = np.ascontiguousarray(orc[q][both], np.float32)
        e = _rel(g.astype(np.float64), o.astype(np.float64))
        errs[q] = float(e.max()) if e.size else 0.0
        bad_vals += int((e > T_REL).sum())
        bits_equal += int((g.view(np.uint32) == o.view(np.uint32)).sum())

    # error of both sides against an FP64 Moller-Trumbore recomputation (reported)
    err64 = {}
    bi = np.nonzero(both)[0]
    if bi.size:
        f64 = pyoracle.mt_f64(verts, idx, rays[bi], gid[bi])
        for side, h in (("gpu", gpu), ("oracle", orc)):
            et = _rel(h["t"][bi].astype(np.float64), f64[:, 0])
            eu = np.abs(h["u"][bi] - f64[:, 1])
            ev = np.abs(h["v"][bi] - f64[:, 2])
            err64[side] = dict(t_max=float(et.max()), t_mean=float(et.mean()), u_max=float(eu.max()),
                               u_mean=float(eu.mean()), v_max=float(ev.max()), v_mean=float(ev.mean()))
    mism = np.nonzero(~same)[0]
    cats = {"t-tie": 0, "edge": 0, "unexplained": 0}
    unexplained = []
    if mism.size:
        r = rays[mism]
        g64 = pyoracle.mt_f64(verts, idx, r, gid[mism])
        o64 = pyoracle.mt_f64(verts, idx, r, oid[mism])
        for j, i in enumerate(mism):
            tg, to = gpu["t"][i], orc["t"][i]
            if gid[i] >= 0 and oid[i] >= 0 and abs(tg - to) <= TIE_REL * max(abs(to), 1e-30):
                cats["t-tie"] += 1
                continue
            margins = []
            if gid[i] >= 0:
                margins.append(_bary_margin(g64[j]))
            if oid[i] >= 0:
                margins.append(_bary_margin(o64[j]))
            if any(abs(m) <= EDGE_EPS for m in margins):
                cats["edge"] += 1
                continue
            cats["unexplained"] += 1
            if len(unexplained) < 10:
                unexplained.append((int(i), int(gid[i]), float(tg), int(oid[i]), float(to),
                                    [float(x) for x in g64[j]], [float(x) for x in o64[j]]))
    stats = dict(n=n, hits=int((oid >= 0).sum()), same_id_hits=int(both.sum()), mismatches=int(mism.size),
                 bad_values=bad_vals, bits_equal=bits_equal, values=3 * int(both.sum()), **cats,
                 t_err_max=errs["t"], u_err_max=errs["u"], v_err_max=errs["v"],
                 fp64=err64, unexplained_examples=unexplained)
    return stats


def assert_parity(stats: dict, max_tie_frac: float = 1e-3):
    msg = {k: v for k, v in stats.items()}
    assert stats["bad_values"] == 0, f"t/u/v of the same triangle beyond 1e-5 relative: {msg}"
    assert stats["unexplained"] == 0, f"unexplained id mismatches: {msg}"
    assert stats["mismatches"] <= max(1, int(max_tie_frac * stats["n"])), f"too many near-ties: {msg}"


def compare_occlusion(gpu_occ, orc_occ, rays, gpu_nearest, orc_nearest, verts, idx, pyoracle) -> dict:
    """Shadow-ray occlusion (0/1 per ray; slots without a shadow ray left out
    by the caller).  gpu_nearest / orc_nearest(rays) -> hit dict: each side's
    closest hit, asked only for the rays the two sides disagree on; the side
    that reports occlusion names the occluding triangle."""
    gpu_occ = np.asarray(gpu_occ).astype(np.int32)
    orc_occ = np.asarray(orc_occ).astype(np.int32)
    mism = np.nonzero(gpu_occ != orc_occ)[0]
    cats = {"edge": 0, "tmax": 0, "tnear": 0, "unexplained": 0}
    examples = []
    if mism.size:
        sub = np.ascontiguousarray(rays[mism])
        gn, on = gpu_nearest(sub), orc_nearest(sub)
        tri = np.where(gpu_occ[mism] == 1, gn["id"], on["id"]).astype(np.int32)
        ok = tri >= 0
        f64 = np.full((mism.size, 3), np.nan)
        if ok.any():
            f64[ok] = pyoracle.mt_f64(verts, idx, np.ascontiguousarray(sub[ok]), tri[ok])
        for j, i in enumerate(mism):
            if not ok[j]:
                cats["unexplained"] += 1
                continue
            t64 = f64[j, 0]
            tmax = float(rays[i, 7])
            lo = float(rays[i, 3]) - HIT_EPSILON
            if abs(_bary_margin(f64[j])) <= EDGE_EPS:
                cats["edge"] += 1
            elif abs(t64 - tmax) <= BOUND_REL * max(abs(tmax), 1.0):
                cats["tmax"] += 1
            elif abs(t64 - lo) <= BOUND_REL * max(abs(lo), 1.0):
                cats["tnear"] += 1
            else:
                cats["unexplained"] += 1
                if len(examples) < 10:
                    examples.append((int(i), int(gpu_occ[i]), int(orc_occ[i]), int(tri[j]),
                                     [float(x) for x in f64[j]]))
    return dict(n=int(gpu_occ.shape[0]), occluded=int(orc_occ.sum()), mismatches=int(mism.size), **cats,
                unexplained_examples=examples)


def assert_occlusion(stats: dict, max_tie_frac: float = 1e-3):
    assert stats["unexplained"] == 0, f"unexplained occlusion mismatches: {stats}"
    assert stats["mismatches"] <= max(1, int(max_tie_frac * stats["n"])), f"too many near-ties: {stats}"


def check_occlusion(name, scene, grid, split_hits, rays, gpu_occ, orc_occ, verts, idx, pyoracle,
                    max_tie_frac: float = 1e-3) -> dict:
    """compare_occlusion with the device scene's and the oracle grid's closest
    hits as the two sides' explanations; prints the counts and asserts."""
    st = compare_occlusion(gpu_occ, orc_occ, rays, lambda r: split_hits(scene.trace_nearest(r)),
                           lambda r: grid.trace_closest(r), verts, idx, pyoracle)
    print(f"\n[{name} occlusion] " + ", ".join(f"{k}={v}" for k, v in st.items() if k != "unexplained_examples"))
    assert_occlusion(st, max_tie_frac)
    return st
