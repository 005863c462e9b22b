"""The serving loop's host logic on the CPU, with a stand-in for the device
session: every request is admitted once, in arrival order, runs exactly its
own number of steps (chunks never run past a scene's end), and the requests
staged while a chunk runs never outnumber the scene slots free after it."""
import numpy as np
import pytest


class FakeLib:
    def pg_session_set_skin(self, sess, skin):
        return 0


class FakeEngine:
    """Records what the server asks of a session; a step moves every active
    scene's spheres by +1 in x, so the positions count the steps run."""

    def __init__(self, **kw):
        self.lib = FakeLib()
        self.sess = None
        self.active = {}                  # slot -> ranges
        self.steps = {}                   # slot -> steps run since switched on
        self.inflight = False
        self.staged_max = 0

    def attach(self, model):
        self.model = model

    def set_grid(self, cell, dims):
        pass

    def set_live(self, p, e, t):
        self.live = (p, e, t)

    def upload_range(self, r, refresh=True):
        assert not self.inflight

    def set_scene(self, slot, active=True, origin=None, excitation=None, start=-1):
        assert not self.inflight
        if active:
            assert slot not in self.active
            self.active[slot] = True
            self.steps[slot] = 0
        else:
            self.active.pop(slot)

    def run_async(self, tab, step):
        assert not self.inflight
        self.inflight = True
        P = self.model.P
        for slot in self.active:
            self.steps[slot] += tab.nsteps
            sel = self.model.pscene[:self.model.parnum] == slot
            P.position[0, :self.model.parnum][sel] += tab.nsteps

    def sync(self):
        self.inflight = False

    def download_range_motion(self, r):
        assert not self.inflight

    def release_range(self, r):
        assert not self.inflight

    def close(self):
        pass


def stream(count, seed=4):
    from parmec_gb300 import batch
    from parmec_gb300.scenes import hopper_fill
    from parmec_gb300.serving import Request
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        m, dt = hopper_fill(n_side=int(rng.integers(2, 4)), seed=200 + k, spacing=0.036)
        exc = batch.sinusoid((0.0, 0.0, -9.81), (1.0, 0.0, 0.0), 5.0)
        out.append(Request(k, 0.0, m, int(rng.integers(5, 90)), exc, dt))
    return out


@pytest.mark.parametrize("slots,chunk", [(1, 16), (2, 7), (3, 40)])
def test_every_request_runs_its_own_steps(monkeypatch, slots, chunk):
    from parmec_gb300 import serving
    monkeypatch.setattr(serving, "GpuEngine", FakeEngine)
    reqs = stream(9)
    x0 = {q.rid: q.model.P.position[0, :q.model.parnum].copy() for q in reqs}
    srv = serving.Server(reqs[0].model, reqs[0].dt, budget_bytes=1e8, max_scenes=slots, max_scene_extent=1.0,
                         chunk=chunk)
    res, stats = srv.serve(reqs, realtime=False)
    srv.close()
    assert stats["requests"] == len(reqs) and stats["rejected"] == 0
    assert sorted(r.rid for r in res) == [q.rid for q in reqs]
    by = {q.rid: q for q in reqs}
    for r in res:
        # each sphere moved by the request's steps, in whole steps
        assert np.array_equal(np.rint(r.position[0] - x0[r.rid]), np.full(r.spheres, by[r.rid].steps))
    # admission in arrival order
    adm = [r.admitted for r in sorted(res, key=lambda r: r.rid)]
    assert adm == sorted(adm)
    assert stats["pool"]["peak_scenes"] <= slots
    assert not srv.eng.active


def test_ranges_first_fit_and_merge():
    from parmec_gb300.serving import _Ranges
    r = _Ranges(100)
    a, b, c = r.take(30), r.take(30), r.take(30)
    assert (a, b, c) == (0, 30, 60)
    assert r.take(20) is None                      # 10 left
    r.give(b, 30)
    assert r.take(40) is None                      # holes of 30 and 10
    assert r.take(25) == 30                        # first fit, inside the hole
    r.give(a, 30)
    r.give(30, 25)
    r.give(c, 30)
    assert r.free == [(0, 100)]                    # everything merged back
    assert r.take(0) == 0 and r.free == [(0, 100)]
