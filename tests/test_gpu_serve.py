"""Serving loop (rtg_serve_run): requests that arrive while others run are
admitted as pool memory frees up and packed into shared trace launches; every
request's result must be bit-identical to tracing it alone, in the batched
and in the plain (one request at a time) mode."""
import numpy as np
import pytest

from gridrt import scenes

pytestmark = pytest.mark.gpu


def _setup(gridlib, nscenes=4, seed=5):
    import torch
    rng = np.random.default_rng(seed)
    scs, geo = [], []
    for i in range(nscenes):
        sc = scenes.plane_and_debris(seed=seed * 100 + i, quads=int(rng.integers(8, 40)),
                                     debris=int(rng.integers(200, 3000)))
        s = gridlib.Scene(0)
        s.set_geometry(sc.verts, sc.idx)
        s.build(4)
        scs.append(s)
        geo.append(sc)
    reqs, expect = [], []
    t = 0.0
    for r in range(160):
        t += float(rng.exponential(1.0 / 4000.0))        # ~4000 req/s: requests overlap on the GPU
        si = int(rng.integers(0, nscenes))
        n = int(np.exp(rng.uniform(np.log(64), np.log(20000))))
        mode = gridlib.RTG_MODE_ANY if rng.uniform() < 0.3 else gridlib.RTG_MODE_NEAREST
        rays = scenes.random_rays(rng, n, (-1.2, -0.1, -1.2), (1.2, 1.1, 1.2))
        if mode == gridlib.RTG_MODE_ANY:
            rays[:, 7] = 0.4
        h_rays = torch.from_numpy(rays).pin_memory()
        out = (torch.empty(n, dtype=torch.uint8) if mode == gridlib.RTG_MODE_ANY
               else torch.empty((n, 4), dtype=torch.int32)).pin_memory()
        reqs.append((t, si, mode, h_rays, n, out))
        if mode == gridlib.RTG_MODE_ANY:
            expect.append(scs[si].trace_any(rays))
        else:
            expect.append(scs[si].trace_nearest(rays).view(np.int32))
    return scs, reqs, expect


@pytest.mark.parametrize("plain", [False, True])
def test_serve_results_equal_alone(gridlib, plain):
    scs, reqs, expect = _setup(gridlib)
    pool = 64 << 20      # small pool: admission has to wait for memory
    admit, done = gridlib.serve(scs, reqs, pool_bytes=pool, plain=plain, max_in_flight=3)
    arrivals = np.array([r[0] for r in reqs])
    assert (done >= admit).all() and (admit >= arrivals - 1e-6).all()
    for (t, si, mode, h_rays, n, out), e in zip(reqs, expect):
        got = out.numpy()
        assert np.array_equal(got, e), (si, mode, n)


def test_serve_batches_requests(gridlib):
    """At a high arrival rate several requests share one step (same admit
    time) in batched mode; in plain mode every admit time is distinct."""
    scs, reqs, _ = _setup(gridlib, seed=9)
    admit, _ = gridlib.serve(scs, reqs, pool_bytes=256 << 20, plain=False, max_in_flight=2)
    assert len(np.unique(admit)) < len(reqs)
    admit_p, _ = gridlib.serve(scs, reqs, pool_bytes=256 << 20, plain=True)
    assert len(np.unique(admit_p)) == len(reqs)
