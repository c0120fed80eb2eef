"""Request server (llf_server), in both forms: the worker pool and the
continuous-batching engine (requests admitted between replays of one shared
CG graph).  Requests admitted while others run overlap on the device; every
result equals the same request solved alone (llf_pcg), bit for bit."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(llf, count, seed=5, dofs_max=2e4):
    import importlib
    wl = importlib.import_module("llfem_gb300.workloads")
    rng = np.random.default_rng(seed)
    return [wl.heat_request(rng, dofs_max=dofs_max) for _ in range(count)]


def _submit(srv, req):
    m, k, fixed, x0 = req
    return srv.submit_heat(m.dim, m.xyz, m.conn, m.family, m.order, k, x0, fixed, reltol=1e-10)


@pytest.mark.parametrize("batched", [False, True], ids=["pool", "engine"])
def test_mix_equals_alone(llf, batched):
    reqs = _requests(llf, 12)
    alone = {}
    with_one = llf._lib.Server(workers=1)
    for i, r in enumerate(reqs):
        alone[i] = with_one.wait(_submit(with_one, r))[0]
    with_one.close()
    srv = llf._lib.Server(workers=4, batched=batched, max_systems=8)
    tickets = {}
    lock = threading.Lock()

    def producer(idx):
        for i in idx:
            t = _submit(srv, reqs[i])
            with lock:
                tickets[i] = t

    th = [threading.Thread(target=producer, args=(list(range(j, len(reqs), 3)),)) for j in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i, t in tickets.items():
        x, it, rr, lat, svc = srv.wait(t)
        assert np.array_equal(x, alone[i]), i
        assert rr <= 1e-10 and lat >= svc >= 0.0
    st = srv.stats()
    assert st["served"] == len(reqs) and st["queued"] == 0
    srv.close()


@pytest.mark.parametrize("batched", [False, True], ids=["pool", "engine"])
def test_solution_is_linear_between_faces(llf, batched):
    m = llf.structured_box_mesh(n=3, order=2, simplex=True)
    fixed = np.zeros(m.non, dtype=np.uint8)
    x0 = np.zeros(m.non)
    left, right = m.group("left").nodes - 1, m.group("right").nodes - 1
    fixed[left] = 1
    fixed[right] = 1
    x0[right] = 10.0
    srv = llf._lib.Server(workers=2, batched=batched)
    x, it, rr, lat, svc = srv.wait(srv.submit_heat(3, m.xyz, m.conn, m.family, m.order, 2.0, x0, fixed,
                                                   reltol=1e-13))
    # the linear field is in the P2 space: exact up to the solver tolerance
    assert rr <= 1e-13
    assert np.abs(x - 10.0 * m.xyz[:, 0]).max() < 1e-10
    srv.close()


@pytest.mark.parametrize("batched", [False, True], ids=["pool", "engine"])
def test_memory_budget_serialises_large_requests(llf, batched):
    reqs = _requests(llf, 4, seed=9, dofs_max=5e3)
    srv = llf._lib.Server(workers=4, budget_bytes=1, batched=batched)   # every request alone on the device
    ts = [_submit(srv, r) for r in reqs]
    for t in ts:
        srv.wait(t)
    assert srv.stats()["peak_bytes"] == max(0, srv.stats()["peak_bytes"])
    srv.close()


@pytest.mark.parametrize("batched", [False, True], ids=["pool", "engine"])
def test_bad_request_reports_error(llf, batched):
    m = llf.structured_rect_mesh(n=2, simplex=True)
    conn = m.conn.copy()
    conn[0, 0] = m.non + 10
    srv = llf._lib.Server(workers=1, batched=batched)
    t = srv.submit_heat(2, m.xyz, conn, m.family, m.order, 1.0, np.zeros(m.non), np.ones(m.non, np.uint8))
    with pytest.raises(llf.LLFError, match="node tag"):
        srv.wait(t)
    srv.close()


def test_engine_many_requests_few_slots(llf):
    """More requests than engine slots, submitted at once: the engine admits
    new requests as slots free up between replays; results equal llf_pcg."""
    reqs = _requests(llf, 20, seed=11, dofs_max=8e3)
    one = llf._lib.Server(workers=1)
    alone = [one.wait(_submit(one, r)) for r in reqs]
    one.close()
    srv = llf._lib.Server(workers=3, batched=True, max_systems=3)
    ts = [_submit(srv, r) for r in reqs]
    for t, a in zip(ts, alone):
        x, it, rr, lat, svc = srv.wait(t)
        assert np.array_equal(x, a[0]) and it == a[1] and rr == a[2]
    st = srv.stats()
    assert st["served"] == len(reqs) and st["queued"] == 0 and st["bytes_in_use"] == 0
    srv.close()
