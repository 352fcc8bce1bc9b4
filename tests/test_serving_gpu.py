"""Serving: continuous batching of solve requests.  Requests that arrive while
others run are admitted into the running batch, their work overlaps on the
device, and each result is identical alone and in the mix (bitwise here, which
is within any stated tolerance)."""
import numpy as np
import pytest

from rocflupicl_gb300 import case as K
from rocflupicl_gb300 import serving as S

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_mix():
    reqs = S.poisson_requests(5, lam=200.0, seed=4, cells_min=1500, cells_max=20000)
    t_end = 2.0e-4
    srv = S.Server(t_end, hbm_budget=2 << 30, keep_state=True, prepare_workers=2)
    res = srv.run(reqs)
    assert len(res) == len(reqs)
    assert srv.max_active >= 2          # requests overlapped on the device
    for q in reqs:
        cv, dv, steps = S.solve_alone(q, t_end)
        r = res[q.rid]
        assert r.steps == steps
        assert abs(r.t_final - t_end) == 0.0
        assert np.array_equal(r.cv, cv)
        assert np.array_equal(r.dv, dv)


def test_admission_respects_hbm_budget():
    reqs = S.poisson_requests(4, lam=1000.0, seed=9, cells_min=3000, cells_max=6000)
    # budget for about one solve at a time: the rest wait and are admitted as
    # slots free up
    srv = S.Server(1.0e-4, hbm_budget=int(6000 * 800 * 1.2), prepare_workers=4)
    res = srv.run(reqs)
    assert len(res) == 4
    assert srv.max_active == 1
    queues = sorted(r.queue for r in res.values())
    assert queues[-1] > queues[0]
