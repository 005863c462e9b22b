"""Serving: continuous batching in one pooled session.

Each request's result is bitwise the same served alone and served in the mix
(the pool keeps every scene's arithmetic independent of its neighbours);
host-side faults (a malformed request, a pool too small for everything at
once) leave the other requests' results unchanged."""
import numpy as np
import pytest

from helpers import bits

pytestmark = pytest.mark.gpu


def small_stream(seed=9, count=6):
    from parmec_gb300 import batch
    from parmec_gb300.scenes import hopper_fill
    from parmec_gb300.serving import Request
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        side = int(rng.integers(3, 7))
        m, dt = hopper_fill(n_side=side, seed=100 + k, spacing=0.036)
        if k % 2:
            exc = batch.sinusoid((0.0, 0.0, -9.81), (rng.uniform(1, 9), 0.0, 0.0), rng.uniform(1, 20))
        else:
            exc = batch.band_noise((0.0, 0.0, -9.81), (1.0, 0.0, 0.0), 3.0, 1.0, 20.0, seed=k)
        out.append(Request(k, 0.0, m, int(rng.integers(40, 160)), exc, dt))
    return out


def serve(reqs, form, **kw):
    from parmec_gb300.serving import Server
    srv = Server(reqs[0].model, reqs[0].dt, form=form, budget_bytes=2e9, max_scenes=kw.pop("max_scenes", 4),
                 max_scene_extent=1.0, **kw)
    try:
        return srv.serve(reqs, realtime=False)
    finally:
        srv.close()


@pytest.mark.parametrize("form", [1, 0])
def test_alone_equals_in_the_mix(gpu_lib, form):
    reqs = small_stream()
    mixed, stats = serve(reqs, form, max_scenes=3, chunk=37)
    assert stats["requests"] == len(reqs)
    by = {r.rid: r for r in mixed}
    for q in reqs:
        alone, _ = serve([q], form, max_scenes=1, chunk=53)
        a, b = alone[0], by[q.rid]
        assert np.array_equal(bits(a.position), bits(b.position)), q.rid
        assert np.array_equal(bits(a.linear), bits(b.linear)), q.rid


def test_small_pool_queues_and_rejects_malformed(gpu_lib):
    """A pool that holds only one scene at a time still serves everything, in
    order; a request with springs is rejected without affecting the rest."""
    from parmec_gb300.serving import Request
    from parmec_gb300.model import Model
    reqs = small_stream(seed=11, count=4)
    bad = Model()
    bad.material(1.0, 1.0, 0.25)
    p = bad.analytical()
    bad.spring(p, (0, 0, 0), -1, (0, 0, 0), [-1.0, -1.0, 1.0, 1.0])
    reqs.append(Request(99, 0.0, bad, 10, reqs[0].excitation, reqs[0].dt))
    big = max(q.model.parnum for q in reqs[:4])
    res, stats = serve(reqs, 1, max_scenes=2, max_spheres=big, chunk=25)
    assert stats["requests"] == 4 and stats["rejected"] == 1
    ref, _ = serve(reqs[:4], 1, max_scenes=4, chunk=61)
    by = {r.rid: r for r in ref}
    for r in res:
        if r.error:
            assert r.rid == 99
            continue
        assert np.array_equal(bits(r.position), bits(by[r.rid].position))


@pytest.mark.parametrize("form", [1, 0])
def test_motion_download_equals_full_download(gpu_lib, form):
    """pg_session_download_range_motion brings back the same position and
    velocity rows as the full range download."""
    from parmec_gb300.serving import Server
    reqs = small_stream(seed=5, count=2)
    srv = Server(reqs[0].model, reqs[0].dt, form=form, budget_bytes=2e9, max_scenes=2, max_scene_extent=1.0)
    try:
        r = srv._load(reqs[1], 0)
        srv.active[0] = (reqs[1], r, 30, 0.0)
        srv._update_live()
        srv.eng.run_async(srv._tab(30), srv.dt)
        srv.eng.sync()
        e0, e1 = r[0], r[1]
        P = srv.P.P
        srv.eng.download_range_motion(r)
        got = [P.position[:, e0:e1].copy(), P.linear[:, e0:e1].copy(), P.angular[:, e0:e1].copy()]
        for a in (P.position, P.linear, P.angular):
            a[:, e0:e1] = np.nan
        srv.eng.download_range(r)
        want = [P.position[:, e0:e1], P.linear[:, e0:e1], P.angular[:, e0:e1]]
        for g, w in zip(got, want):
            assert np.array_equal(bits(g), bits(w))
        assert not np.array_equal(bits(got[0]), bits(reqs[1].model.P.position[:, :e1 - e0]))   # the scene moved
    finally:
        srv.close()
