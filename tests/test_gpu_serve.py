"""Request loop on the GPU: every run gives the same result in the mix as
alone, the HBM budget bounds what is admitted at once, and latencies are
reported."""
import numpy as np
import pytest

from surfactant_enhanced_spreading_gb300 import engine as E
from surfactant_enhanced_spreading_gb300 import serve

pytestmark = pytest.mark.gpu


def _requests():
    sizes = [(300, 3, 300), (600, 0, 200), (500, 6, 400), (300, 0, 100), (800, 4, 300)]
    return [serve.make_request(k, nw, ns, st, seed=100 + k, arrival=0.01 * k) for k, (nw, ns, st) in enumerate(sizes)]


@pytest.mark.parametrize("precision", [E.MIXED, E.PLAIN_FP64])
def test_same_result_alone_and_in_mix(precision):
    reqs = _requests()
    srv = serve.Server(budget_bytes=1 << 34, precision=precision, chunk=100)
    mixed = srv.run(reqs)
    alone = serve.run_one_at_a_time(reqs, precision, chunk=100)
    for m, a in zip(mixed, alone):
        assert m.rid == a.rid
        assert np.array_equal(m.pos, a.pos), m.rid
        assert np.array_equal(m.vel, a.vel), m.rid
        assert m.eta == a.eta


@pytest.mark.parametrize("precision", [E.MIXED, E.PLAIN_FP64])
def test_slots_of_one_context_same_result_as_alone(precision):
    """Requests as replicas of one batched context, formed again whenever a
    run joins or leaves (at rebuild boundaries): every run bit-identical to
    the same run alone."""
    reqs = _requests()
    srv = serve.SlotServer(budget_bytes=1 << 34, precision=precision, chunk=100)
    slots = srv.run(reqs)
    assert srv.reforms >= 3
    alone = serve.run_one_at_a_time(reqs, precision, chunk=100)
    for m, a in zip(slots, alone):
        assert m.rid == a.rid and not m.failed
        assert np.array_equal(m.pos, a.pos), m.rid
        assert np.array_equal(m.vel, a.vel), m.rid
        assert m.eta == a.eta


def test_slots_configuration_preset():
    from surfactant_enhanced_spreading_gb300 import config_preset as C
    sizes = [(400, 4, 200, 0.0), (700, 0, 300, 0.0), (300, 6, 100, 0.05)]
    reqs = [serve.make_request(k, nw, ns, st, seed=300 + k, arrival=t, preset=C.PRESET_CONFIG)
            for k, (nw, ns, st, t) in enumerate(sizes)]
    slots = serve.SlotServer(budget_bytes=1 << 34, precision=E.MIXED, chunk=100).run(reqs)
    alone = serve.run_one_at_a_time(reqs, E.MIXED, chunk=100)
    for m, a in zip(slots, alone):
        assert np.array_equal(m.pos, a.pos) and np.array_equal(m.vel, a.vel) and m.eta == a.eta, m.rid


def test_budget_limits_concurrency():
    reqs = _requests()
    biggest = max(serve.estimate_bytes(r.system) for r in reqs)
    srv = serve.Server(budget_bytes=int(1.5 * biggest), precision=E.MIXED, chunk=100, keep_state=False)
    res = srv.run(reqs)
    assert len(res) == len(reqs)
    assert all(0 < r.device_bytes <= r.estimate_bytes for r in res), [(r.device_bytes, r.estimate_bytes) for r in res]
    assert srv.peak_used <= srv.budget
    s = serve.summarize(res)
    assert 0 < s["p50_latency_s"] <= s["p99_latency_s"]
    assert s["atom_steps_per_s"] > 0
