"""Two-level instancing on the GPU (rtg_instances_*) against the oracle's
restatement of the reference's instance loop: world boxes bit-exact, hits
under the near-tie rules, identity and duplicate instances bit-exact against
the one-scene trace."""
import numpy as np
import pytest

import instancing as ins
from gridrt import scenes

pytestmark = pytest.mark.gpu


def _scene(gridlib, sc, k):
    s = gridlib.Scene(0)
    s.set_geometry(sc.verts, sc.idx)
    s.build(k)
    return s


def test_identity_instance_is_the_single_trace(gridlib):
    sc = scenes.plane_and_debris()
    s = _scene(gridlib, sc, 4)
    I = gridlib.Instances([(s, *ins.IDENTITY)])
    rays = scenes.camera_rays(scenes.plane_and_debris_camera(256, 256))
    one = s.trace_nearest(rays).view(np.int32)
    hits, inst = I.trace_nearest(rays)
    assert np.array_equal(one, hits.view(np.int32))
    assert np.array_equal(inst, np.where(one[:, 0] >= 0, 0, -1))


def test_duplicates_keep_the_first_instance(gridlib):
    sc = scenes.deforming_sphere(1)
    s = _scene(gridlib, sc, 4)
    I = gridlib.Instances([(s, *ins.IDENTITY), (s, *ins.IDENTITY), (s, *ins.IDENTITY)])
    rays = scenes.camera_rays(scenes.deforming_sphere_camera(256, 256))
    one = s.trace_nearest(rays).view(np.int32)
    hits, inst = I.trace_nearest(rays)
    assert np.array_equal(one, hits.view(np.int32))
    assert ((inst == 0) | (one[:, 0] < 0)).all()


def _world(gridlib, oracle, seed, n_inst=6):
    rng = np.random.default_rng(seed)
    base = [scenes.plane_and_debris(), scenes.deforming_sphere(2), scenes.tiny_scene(4, 3000, spread=0.8)]
    ks = [4, 2, 6]
    dev = [_scene(gridlib, sc, k) for sc, k in zip(base, ks)]
    grids = [oracle.Grid(sc.verts, sc.idx, k) for sc, k in zip(base, ks)]
    items, oitems, scs, tfs = [], [], [], []
    for j in range(n_inst):
        b = j % len(base)
        M, inv = ins.random_transform(rng, shift=2.5)
        items.append((dev[b], M, inv))
        oitems.append((grids[b], M, inv))
        scs.append(base[b])
        tfs.append((M, inv))
    return rng, dev, items, oitems, scs, tfs


def test_boxes_match_oracle(gridlib, oracle):
    _, _, items, oitems, _, _ = _world(gridlib, oracle, 3)
    I = gridlib.Instances(items)
    O = oracle.Instances(oitems)
    box, boxes = I.boxes()
    assert np.array_equal(box.view(np.uint32), O.box.view(np.uint32))
    assert np.array_equal(boxes.view(np.uint32), O.boxes.view(np.uint32))


@pytest.mark.parametrize("seed", [1, 2])
def test_transformed_instances_match_oracle(gridlib, oracle, seed):
    rng, _, items, oitems, scs, tfs = _world(gridlib, oracle, seed)
    I = gridlib.Instances(items)
    O = oracle.Instances(oitems)
    rays = np.concatenate([scenes.random_rays(rng, 60_000, (-4, -4, -4), (4, 4, 4)),
                           scenes.camera_rays(scenes.look_at_camera((6.0, 4.0, 7.0), (0, 0, 0), (0, 1, 0), 60.0,
                                                                    256, 256))])
    hits, inst = I.trace_nearest(rays)
    gh = gridlib.split_hits(hits)
    oh, oinst, _ = O.trace(rays)
    st = ins.compare_instance_hits(gh, inst, oh, oinst, scs, tfs, rays, oracle)
    print("\n[instances]", st)
    assert st["ok"], st
    assert (inst >= 0).sum() >= 2000


def test_any_hit_instances_match_oracle(gridlib, oracle):
    import torch
    rng, _, items, oitems, scs, tfs = _world(gridlib, oracle, 7)
    I = gridlib.Instances(items)
    O = oracle.Instances(oitems)
    rays = scenes.random_rays(rng, 100_000, (-4, -4, -4), (4, 4, 4))
    rays[:, 7] = rng.uniform(0.5, 6.0, size=rays.shape[0]).astype(np.float32)
    rays[::97, 7] = -1.0          # slots without a shadow ray
    d_rays = torch.from_numpy(rays).cuda()
    d_occ = torch.empty(rays.shape[0], dtype=torch.uint8, device="cuda")
    I.trace_any_device(d_rays, rays.shape[0], d_occ)
    torch.cuda.synchronize()
    occ = d_occ.cpu().numpy()
    _, _, oocc = O.trace(rays)
    oocc = np.where(rays[:, 7] < 0, 2, oocc)
    assert (occ[rays[:, 7] < 0] == 2).all()
    assert (occ != oocc).sum() <= max(1, int(1e-3 * rays.shape[0]))


def test_update_moves_instances(gridlib, oracle):
    rng, _, items, oitems, scs, tfs = _world(gridlib, oracle, 9, n_inst=3)
    I = gridlib.Instances(items)
    rays = scenes.random_rays(rng, 40_000, (-4, -4, -4), (4, 4, 4))
    new = [ins.random_transform(rng, shift=2.5) for _ in items]
    I.update([(s, M, inv) for (s, _, _), (M, inv) in zip(items, new)])
    O = oracle.Instances([(g, M, inv) for (g, _, _), (M, inv) in zip(oitems, new)])
    hits, inst = I.trace_nearest(rays)
    oh, oinst, _ = O.trace(rays)
    st = ins.compare_instance_hits(gridlib.split_hits(hits), inst, oh, oinst, scs, new, rays, oracle)
    assert st["ok"], st
