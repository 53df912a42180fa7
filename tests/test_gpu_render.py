"""Shading wavefront (rtg_render) against the oracle's restatement of the
reference's per-pixel recursion (materials, point lights with shadows,
reflection, refraction, background)."""
import numpy as np
import pytest

from gridrt import scenes

pytestmark = pytest.mark.gpu


def _vertex_normals(sc):
    v = sc.verts.astype(np.float64)
    f = sc.idx
    fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    n = np.zeros_like(v)
    for k in range(3):
        np.add.at(n, f[:, k], fn)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    n = np.where(ln > 0, n / np.maximum(ln, 1e-30), np.array([0.0, 1.0, 0.0]))
    return n.astype(np.float32)


def _setup(gridlib, oracle):
    import torch
    sc = scenes.plane_and_debris()
    s = gridlib.Scene(0)
    s.set_geometry(sc.verts, sc.idx)
    s.build(4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    rng = np.random.default_rng(21)
    normals = _vertex_normals(sc)
    colors = rng.uniform(0.2, 1.0, size=sc.verts.shape).astype(np.float32)
    mat = (np.arange(sc.ntris) % 4).astype(np.int32)
    mat[:32768] = 0                                   # the ground plane
    L = gridlib
    mats = [L.material(L.RTG_MAT_PHONG, reflexion=0.35),
            L.material(L.RTG_MAT_PHONG_COLOR, diffuse=(0.8, 0.3, 0.2), opacity=0.6, refraction_index=1.3),
            L.material(L.RTG_MAT_HEADLIGHT, ambient=(0.1, 0.1, 0.1)),
            L.material(L.RTG_MAT_HEADLIGHT_COLOR, ambient=(0.1, 0.1, 0.1), diffuse=(0.2, 0.6, 0.9))]
    lights = [L.point_light((2.0, 4.0, 2.0), (0.8, 0.8, 0.8), True),
              L.point_light((-3.0, 2.0, 1.0), (0.3, 0.3, 0.4), False)]
    dev = dict(d_normals=torch.from_numpy(normals).cuda(), d_colors=torch.from_numpy(colors).cuda(),
               d_material=torch.from_numpy(mat).cuda())
    return sc, s, g, normals, colors, mat, mats, lights, dev


def _oracle_mats(oracle, mats):
    out = []
    for m in mats:
        o = oracle.Material()
        o.type = m.type
        for a in range(3):
            o.ambient[a], o.diffuse[a], o.specular[a] = m.ambient[a], m.diffuse[a], m.specular[a]
        o.specular_exponent, o.reflexion = m.specular_exponent, m.reflexion
        o.refraction_index, o.opacity = m.refraction_index, m.opacity
        out.append(o)
    return out


def _oracle_lights(oracle, lights):
    out = []
    for L in lights:
        o = oracle.Light()
        for a in range(3):
            o.position[a], o.intensity[a] = L.position[a], L.intensity[a]
        o.cast_shadows = L.cast_shadows
        out.append(o)
    return out


@pytest.mark.parametrize("max_depth", [0, 3])
def test_render_matches_oracle(gridlib, oracle, max_depth):
    import torch
    sc, s, g, normals, colors, mat, mats, lights, dev = _setup(gridlib, oracle)
    cam = scenes.plane_and_debris_camera(160, 120)
    n = cam.width * cam.height
    d_rgb = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    rays = s.render(cam, dev["d_normals"], mats, lights, d_rgb, d_colors=dev["d_colors"],
                    d_material=dev["d_material"], background=(0.9, 0.95, 1.0), max_depth=max_depth)
    torch.cuda.synchronize()
    rgb = d_rgb.cpu().numpy()
    prim = scenes.camera_rays(cam, "scanline")
    orgb, orays = oracle.render(g, normals, colors, mat, _oracle_mats(oracle, mats), _oracle_lights(oracle, lights),
                                (0.9, 0.95, 1.0), max_depth, 1.0, prim)
    err = np.abs(rgb - orgb).max(axis=1)
    close = err <= 1e-3
    print(f"\n[render depth={max_depth}] rays gpu={rays} oracle={orays} close={close.mean():.5f} "
          f"max={err.max():.3g} mean={err.mean():.3g}")
    assert np.isfinite(rgb).all()
    assert close.mean() >= 0.99
    assert abs(rays - orays) <= 0.01 * orays
    if max_depth == 3:
        assert rays > n * 1.2          # shadow and secondary rays were traced


def test_render_headlight_only_is_tight(gridlib, oracle):
    import torch
    sc, s, g, normals, colors, mat, mats, lights, dev = _setup(gridlib, oracle)
    cam = scenes.plane_and_debris_camera(128, 128)
    n = cam.width * cam.height
    hm = [gridlib.material(gridlib.RTG_MAT_HEADLIGHT, ambient=(0.1, 0.1, 0.1))]
    d_rgb = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    rays = s.render(cam, dev["d_normals"], hm, [], d_rgb, d_colors=dev["d_colors"], max_depth=3)
    torch.cuda.synchronize()
    orgb, orays = oracle.render(g, normals, colors, None, _oracle_mats(oracle, hm), [], (1.0, 1.0, 1.0), 3, 1.0,
                                scenes.camera_rays(cam, "scanline"))
    err = np.abs(d_rgb.cpu().numpy() - orgb).max(axis=1)
    assert rays == n and orays == n
    assert (err <= 2e-5).mean() >= 0.999
