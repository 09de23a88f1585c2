"""Host-side logic of the request loop: box sizing, memory estimates, arrival
generation, budget refusal and latency statistics (no GPU needed)."""
import numpy as np
import pytest

from surfactant_enhanced_spreading_gb300 import engine as E
from surfactant_enhanced_spreading_gb300 import serve
from surfactant_enhanced_spreading_gb300 import system as S


@pytest.mark.parametrize("nw,ns", [(300, 0), (600, 6), (2000, 20)])
def test_box_holds_droplet(nw, ns):
    r = serve.make_request(0, nw, ns, 100, seed=3)
    s = r.system
    assert all(c % 4 == 0 for c in s.cells)
    half = np.array(s.cells) * 12.0 / 3.166 / 2.0
    assert np.all(np.abs(s.pos) < half)


def test_estimate_grows_with_size():
    a = serve.make_request(0, 300, 0, 100, seed=1).system
    b = serve.make_request(0, 2000, 20, 100, seed=1).system
    assert 0 < serve.estimate_bytes(a) < serve.estimate_bytes(b)


def test_poisson_requests_seeded():
    a = serve.poisson_requests(4, 5.0, seed=11, water=(300, 600), surf=(0, 4), steps=(100, 300))
    b = serve.poisson_requests(4, 5.0, seed=11, water=(300, 600), surf=(0, 4), steps=(100, 300))
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert all(np.array_equal(x.system.pos, y.system.pos) for x, y in zip(a, b))
    assert all(r.steps % 100 == 0 and 100 <= r.steps <= 300 for r in a)
    assert np.all(np.diff([r.arrival for r in a]) > 0)


def test_request_over_budget_is_refused_before_any_device_work():
    r = serve.make_request(0, 300, 0, 100, seed=1)
    srv = serve.Server(budget_bytes=1024)
    with pytest.raises(E.SespError, match="EBUDGET"):
        srv.run([r])


def test_summary_percentiles():
    res = [serve.Result(rid=k, n_sites=10, steps=100, arrival=0.0, admitted=0.0, finished=float(k + 1))
           for k in range(100)]
    s = serve.summarize(res)
    assert s["requests"] == 100
    assert abs(s["p50_latency_s"] - 50.5) < 1e-9
    assert abs(s["p99_latency_s"] - 99.01) < 1e-9
    assert abs(s["atom_steps_per_s"] - 100 * 10 * 100 / 100.0) < 1e-9


def test_surfactant_templates_are_clash_free():
    """Exact constraint lengths; no two sites closer than the shortest bond;
    sites two bonds apart (incl. two children of a branch site) at least
    1.8 A apart; sites three or more bonds apart at least 2.6 A apart."""
    import itertools
    rng = np.random.default_rng(11)
    adj = {i: set() for i in range(1, 30)}
    for i, j in S.SURF_BONDS:
        adj[i].add(j)
        adj[j].add(i)
    two = {(a, b) for u in adj for a, b in itertools.combinations(sorted(adj[u]), 2)}
    bonded = {tuple(sorted(b)) for b in S.SURF_BONDS}
    for _ in range(60):
        t = S.surfactant_template(rng)
        for b, (i, j) in enumerate(S.SURF_BONDS):
            assert abs(np.linalg.norm(t[i - 1] - t[j - 1]) - S.SURF_BOND_LEN[b]) < 1e-9
        for a, b in itertools.combinations(range(1, 30), 2):
            r = np.linalg.norm(t[a - 1] - t[b - 1])
            if (a, b) in bonded:
                continue
            assert r > (1.8 if (a, b) in two else 2.6) - 1e-9, (a, b, r)


def test_crowded_request_starts_without_failures():
    """A served-size droplet with many surfactants (21,517 waters, 270
    surfactants) takes its first steps on the oracle without a constraint
    failure or a non-finite coordinate."""
    import oracle as O
    reqs = serve.poisson_requests(3, 2.0, 777, water=(1000, 50000), surf=(0, 500), steps=(500, 5000))
    s = reqs[2].system
    assert (s.n_water, s.n_surf) == (21517, 270)
    orc = O.Oracle(s)
    orc.force(True)
    orc.init_accel()
    orc.run(99101, 2)
    assert orc.fail_count() == 0
    assert np.isfinite(orc.get(0)).all()


def test_graphite_covers_the_floor():
    """A droplet far smaller than its box still sits on a sheet that reaches
    every wall (within one lattice step), so no molecule can leave the sheet
    and sink beside its edge."""
    s = S.droplet(1500, 10, cells=(20, 20, 12), seed=3)
    half = np.array(s.cells, dtype=np.float64) * S.RS / 2.0
    c = s.carbons.reshape(-1, 3)
    step = 2.5 / S.SIGMA
    for a in (0, 1):
        assert c[:, a].min() < -half[a] + step and c[:, a].max() > half[a] - step
    assert np.all(np.abs(c[:, :2]) < half[:2])


def test_summary_counts_steps_done_of_failed_runs():
    res = [serve.Result(rid=0, n_sites=10, steps=100, arrival=0.0, admitted=0.0, finished=1.0),
           serve.Result(rid=1, n_sites=10, steps=100, arrival=0.0, admitted=0.0, finished=1.0, steps_done=30,
                        failed=True, shake_failures=5000)]
    s = serve.summarize(res)
    assert s["failed_requests"] == [1] and s["shake_failures"] == 5000
    assert abs(s["atom_steps_per_s"] - (10 * 100 + 10 * 30) / 1.0) < 1e-9


class _FakeEngine:
    """Host stand-in for an engine: its failure counter jumps after the
    first chunk when the system has an odd number of waters."""
    def __init__(self, system, precision, device=0):
        self.system, self.chunks, self.eta = system, 0, 0.0

    def force(self, rebuild=True):
        pass

    def init_accel(self):
        pass

    def device_bytes(self):
        return 1 << 20

    def run_async(self, kb, n):
        self.chunks += 1

    def busy(self):
        return False

    def sync(self):
        pass

    def counters(self):
        bad = self.system.n_water % 2 == 1 and self.chunks >= 1
        return [10 ** 6 if bad else 0] + [0] * 7

    def state(self):
        return None, None, None

    def close(self):
        pass


def test_server_stops_a_blown_up_run(monkeypatch):
    """A run whose failure count passes the limit between chunks is stopped
    after the chunk that failed; the others run all their steps."""
    monkeypatch.setattr(serve.E, "Engine", _FakeEngine)
    reqs = [serve.Request(rid=k, system=S.System(n_water=300 + k, n_surf=0, cells=(4, 4, 4),
                                                  pos=np.zeros((3 * (300 + k), 3)), vel=np.zeros((3 * (300 + k), 3)),
                                                  carbons=np.zeros((0, 3)), graphite_on=False),
                          steps=500, arrival=0.0) for k in range(2)]
    res = serve.Server(1 << 40, chunk=100, keep_state=False).run(reqs)
    assert [r.failed for r in res] == [False, True]
    assert res[0].steps_done == -1 and res[1].steps_done == 100


class _FakeBatch:
    """Stands in for a batched engine context on the CPU: each chunk of n
    steps adds n x 1e-3 to positions, n to velocities and accelerations and
    n x 0.01 to eta, so a run's final state counts the steps it was given;
    init_accel sets accelerations to 7 (a run carried into a new context
    must keep its own).  A system with a `fail_per_step` attribute reports
    that many SHAKE failures per step."""
    formed = []

    def __init__(self, systems, precision, device=0, **kw):
        _FakeBatch.formed.append(len(systems))
        self.systems = systems
        self.offsets = np.cumsum([0] + [s.n_sites for s in systems])
        self.pos = np.concatenate([s.pos for s in systems]).copy()
        self.vel = np.concatenate([s.vel for s in systems]).copy()
        self.acc = np.zeros_like(self.pos)
        self.eta = np.zeros(len(systems))
        self.fail = np.zeros(len(systems), dtype=np.int64)

    def force(self, rebuild=True, terms=None):
        return np.zeros_like(self.pos)

    def init_accel(self):
        self.acc[:] = 7.0

    def state(self, out=None):
        return self.pos.copy(), self.vel.copy(), self.acc.copy()

    def set_state(self, pos=None, vel=None, acc=None, eta=0.0):
        if acc is not None:
            self.acc = np.array(acc, dtype=np.float64)
        self.eta[:] = eta

    def etas(self):
        return self.eta.copy()

    def set_etas(self, etas):
        self.eta = np.array(etas, dtype=np.float64)

    def failures(self):
        return self.fail.copy()

    def run_async(self, kb, n):
        assert kb % 10 == 1 and n % 10 == 0   # chunks start just after a rebuild step
        self.pos += n * 1e-3
        self.vel += n
        self.acc += n
        self.eta += 0.01 * n
        for q, s in enumerate(self.systems):
            self.fail[q] += n * getattr(s, "fail_per_step", 0)

    def sync(self):
        pass

    def close(self):
        pass


def _slot_requests():
    sizes = [(300, 0, 300, 0.0), (400, 2, 200, 0.0), (300, 0, 500, 0.02), (500, 0, 100, 0.04)]
    return [serve.make_request(k, nw, ns, st, seed=40 + k, arrival=t) for k, (nw, ns, st, t) in enumerate(sizes)]


def test_slot_server_carries_each_run_through_reformed_contexts(monkeypatch):
    monkeypatch.setattr(serve.E, "Engine", _FakeBatch)
    _FakeBatch.formed = []
    reqs = _slot_requests()
    srv = serve.SlotServer(budget_bytes=1 << 40, chunk=100)
    res = srv.run(reqs)
    assert [r.rid for r in res] == [0, 1, 2, 3]
    assert srv.reforms == len(_FakeBatch.formed) >= 3
    for r, q in zip(res, reqs):
        assert not r.failed and r.steps_done == -1
        assert np.allclose(r.pos, q.system.pos + 1e-3 * q.steps)
        assert np.allclose(r.vel, q.system.vel + q.steps)
        assert abs(r.eta - 0.01 * q.steps) < 1e-9
        assert 0 <= r.admitted and r.finished >= r.admitted
    assert srv.peak_used <= srv.budget


def test_slot_server_budget_and_failures(monkeypatch):
    monkeypatch.setattr(serve.E, "Engine", _FakeBatch)
    _FakeBatch.formed = []
    reqs = _slot_requests()
    reqs[2].system.fail_per_step = 3           # passes max_failures after its first chunk
    biggest = max(serve.estimate_bytes(r.system) for r in reqs)
    srv = serve.SlotServer(budget_bytes=int(1.5 * biggest), chunk=100, max_failures=100)
    res = srv.run(reqs)
    assert max(_FakeBatch.formed) == 1             # the budget holds one run at a time
    assert srv.peak_used <= srv.budget
    bad = res[2]
    assert bad.failed and bad.steps_done == 100 and bad.shake_failures == 300
    assert all(not r.failed for k, r in enumerate(res) if k != 2)


def test_slot_server_refuses_bad_requests(monkeypatch):
    monkeypatch.setattr(serve.E, "Engine", _FakeBatch)
    r = serve.make_request(0, 300, 0, 105, seed=1)
    with pytest.raises(ValueError, match="multiple"):
        serve.SlotServer(budget_bytes=1 << 40).run([r])
    with pytest.raises(ValueError, match="multiple of the rebuild interval"):
        serve.SlotServer(budget_bytes=1 << 40, chunk=95)
    a = serve.make_request(0, 300, 0, 100, seed=1)
    b = serve.make_request(1, 300, 0, 100, seed=2, preset=1)
    with pytest.raises(ValueError, match="preset"):
        serve.SlotServer(budget_bytes=1 << 40).run([a, b])
    with pytest.raises(E.SespError, match="EBUDGET"):
        serve.SlotServer(budget_bytes=1024).run([a])
