"""Continuous batching: requests that arrive while others are on the GPU join the running eigen-solver
batch; each result must be the same as the request solved alone (bit for bit: every sector's arithmetic is
independent of the batch it shares)."""
import numpy as np
import pytest

from edlib_gb300 import models

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ed():
    from edlib_gb300 import build
    build.build()
    from edlib_gb300 import ed as _ed
    return _ed


def _specs(n):
    out = []
    for seed in range(n):
        p, d = models.random_siam(300 + seed, 5 + (seed % 4))  # 5..8 sites: uneven sectors
        p.update({"arpack.NEV": 4 + (seed % 2), "lanc.BETA": 20.0 + 10 * (seed % 2), "lanc.NOMEGA": 64,
                  "lanc.NLANC": 60})
        out.append((p, d))
    return out


def _alone(ed, specs, precision):
    res = []
    for p, d in specs:
        h = ed.Hamiltonian(ed.Params(p), d, storage="SRS", precision=precision)
        h.diag()
        G = ed.GreensFunction(ed.Params(p), h).compute()
        res.append((np.array([e.eigenvalue() for e in h.eigenpairs()]), G))
        h.close()
    return res


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_requests_joining_a_running_batch_match_solo_solves(ed, precision):
    specs = _specs(5)
    alone = _alone(ed, specs, precision)
    srv = ed.Server(precision=precision)
    hams = [ed.Hamiltonian(ed.Params(p), d, storage="SRS", precision=precision) for p, d in specs]
    tickets = [srv.submit(hams[0]), srv.submit(hams[1])]
    running, queued = srv.step()
    assert queued == 0 and running <= 2
    for h in hams[2:]:  # arrive while the first two are on the GPU
        tickets.append(srv.submit(h))
        srv.step()
    for _ in range(100000):
        if all(srv.poll(t) == srv.DONE for t in tickets):
            break
        srv.step()
    for q, t in enumerate(tickets):
        h, G, _, Z = srv.result(t)
        E = np.array([e.eigenvalue() for e in h.eigenpairs()])
        assert np.array_equal(E, alone[q][0])
        assert np.array_equal(G, alone[q][1])
    srv.close()


def test_memory_budget_admits_one_at_a_time(ed):
    specs = _specs(3)
    alone = _alone(ed, specs, "fp64")
    srv = ed.Server(precision="fp64", hbm_budget=1)  # nothing fits: one request at a time
    hams = [ed.Hamiltonian(ed.Params(p), d, storage="SRS", precision="fp64") for p, d in specs]
    tickets = [srv.submit(h) for h in hams]
    running, queued = srv.step()
    assert queued == 2 and running <= 1
    for _ in range(100000):
        if all(srv.poll(t) == srv.DONE for t in tickets):
            break
        running, queued = srv.step()
        assert running <= 1
    for q, t in enumerate(tickets):
        h, G, _, _ = srv.result(t)
        assert np.array_equal(np.array([e.eigenvalue() for e in h.eigenpairs()]), alone[q][0])
        assert np.array_equal(G, alone[q][1])
    srv.close()
