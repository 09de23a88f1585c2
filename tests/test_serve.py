"""Host-side logic of the request loop: box sizing, memory estimates, arrival
generation, budget refusal and latency statistics (no GPU needed)."""
import numpy as np
import pytest

from surfactant_enhanced_spreading_gb300 import engine as E
from surfactant_enhanced_spreading_gb300 import serve


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
