"""The CUDA path against the golden fixtures: outputs of the reference's own
CPU code (compiled unmodified) on small seeded scenes at the reference's
k = 6, committed under tests/golden/ with the script that made them.  Grid
parameters and cell lists bit for bit; closest hits under the near-tie rules
of parity.py (the device decides hits with Moller-Trumbore, the reference with
Wald's projection test; the reported t / u / v are Wald's); shadow-ray
occlusion up to near-ties, each explained by its occluding triangle."""
import glob
import os

import numpy as np
import pytest

import parity

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.skipif(not GOLDEN, reason="no golden fixtures")
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_device_matches_reference_golden(gridlib, oracle, path):
    z = np.load(path)
    verts, idx, k = z["verts"], z["idx"], int(z["k"])
    s = gridlib.Scene(0)
    s.set_geometry(verts, idx)
    s.build(k)
    info = s.info()
    assert tuple(int(r) for r in info["res"]) == tuple(int(r) for r in z["res"])
    for key in ("bmin", "bmax", "cell", "inv_cell"):
        assert np.array_equal(_bits(info[key]), _bits(z[key])), key
    off, ids = s.download()
    assert np.array_equal(off, z["offsets"]), "offsets differ from the reference's"
    assert np.array_equal(ids, z["ids"]), "cell lists differ from the reference's"
    rays = z["rays"]
    gh = gridlib.split_hits(s.trace_nearest(rays))
    ref = dict(id=z["hit_id"], t=z["hit_t"], u=z["hit_u"], v=z["hit_v"])
    st = parity.compare_hits(gh, ref, verts, idx, rays, oracle)
    print(f"\n[{os.path.basename(path)}] " + ", ".join(f"{a}={b}" for a, b in st.items()
                                                       if a != "unexplained_examples"))
    # a fixture holds a few thousand rays: allow 2 near-ties per thousand
    parity.assert_parity(st, max_tie_frac=2e-3)
    if "shadow_rays" in z.files:
        sr = z["shadow_rays"]
        occ = s.trace_any(sr)
        # every disagreement with the reference's occlusion is explained by
        # the occluding triangle (an edge, or t at the window bounds); the
        # oracle's closest hit stands in for the reference's on those rays
        g = oracle.Grid(verts, idx, k)
        parity.check_occlusion(os.path.basename(path), s, g, gridlib.split_hits, sr, occ, z["occluded"], verts,
                               idx, oracle, max_tie_frac=2e-3)
