"""Request server (llf_server): requests admitted while others run overlap on
the device; every result equals the same request solved alone."""
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


def test_mix_equals_alone(llf):
    reqs = _requests(llf, 12)
    alone = {}
    with_one = llf._lib.Server(workers=1)
    for i, r in enumerate(reqs):
        alone[i] = with_one.wait(_submit(with_one, r))[0]
    with_one.close()
    srv = llf._lib.Server(workers=4)
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


def test_solution_is_linear_between_faces(llf):
    m = llf.structured_box_mesh(n=3, order=2, simplex=True)
    fixed = np.zeros(m.non, dtype=np.uint8)
    x0 = np.zeros(m.non)
    left, right = m.group("left").nodes - 1, m.group("right").nodes - 1
    fixed[left] = 1
    fixed[right] = 1
    x0[right] = 10.0
    srv = llf._lib.Server(workers=2)
    x, it, rr, lat, svc = srv.wait(srv.submit_heat(3, m.xyz, m.conn, m.family, m.order, 2.0, x0, fixed,
                                                   reltol=1e-13))
    # the linear field is in the P2 space: exact up to the solver tolerance
    assert rr <= 1e-13
    assert np.abs(x - 10.0 * m.xyz[:, 0]).max() < 1e-10
    srv.close()


def test_memory_budget_serialises_large_requests(llf):
    reqs = _requests(llf, 4, seed=9, dofs_max=5e3)
    srv = llf._lib.Server(workers=4, budget_bytes=1)   # every request alone on the device
    ts = [_submit(srv, r) for r in reqs]
    for t in ts:
        srv.wait(t)
    assert srv.stats()["peak_bytes"] == max(0, srv.stats()["peak_bytes"])
    srv.close()


def test_bad_request_reports_error(llf):
    m = llf.structured_rect_mesh(n=2, simplex=True)
    conn = m.conn.copy()
    conn[0, 0] = m.non + 10
    srv = llf._lib.Server(workers=1)
    t = srv.submit_heat(2, m.xyz, conn, m.family, m.order, 1.0, np.zeros(m.non), np.ones(m.non, np.uint8))
    with pytest.raises(llf.LLFError, match="node tag"):
        srv.wait(t)
    srv.close()
