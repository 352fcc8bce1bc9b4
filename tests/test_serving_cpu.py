"""Serving loop host logic without a GPU: the seeded request stream and the
latency summary."""
import numpy as np

from rocflupicl_gb300 import serving as S


def test_poisson_stream_is_seeded():
    a = S.poisson_requests(50, lam=5.0, seed=1)
    b = S.poisson_requests(50, lam=5.0, seed=1)
    assert [(x.arrival, x.n, x.Ms, x.scheme) for x in a] == [(x.arrival, x.n, x.Ms, x.scheme) for x in b]
    cells = np.array([x.cells for x in a])
    assert cells.min() >= 6 * 11 ** 3 and cells.max() <= 6 * 88 ** 3
    assert S.poisson_requests(50, lam=5.0, seed=2)[0].arrival != a[0].arrival


def test_poisson_stream_rate_and_ranges():
    """Exponential gaps of mean 1/lam, Mach numbers in [1.2, 3], the three
    schemes all drawn, arrivals increasing, distinct solve seeds."""
    lam = 4.0
    r = S.poisson_requests(4000, lam=lam, seed=7)
    t = np.array([x.arrival for x in r])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert np.all(gaps > 0) and abs(gaps.mean() * lam - 1.0) < 0.05
    ms = np.array([x.Ms for x in r])
    assert ms.min() >= 1.2 and ms.max() <= 3.0
    assert set(x.scheme for x in r) == set(S.SCHEMES)
    assert len(set(x.seed for x in r)) == len(r)


def test_summary_percentiles():
    res = {i: S.Result(rid=i, cells=6 * 8 ** 3, steps=10, face_evals=1000, latency=float(i + 1),
                       queue=0.0, t_final=1e-4) for i in range(100)}
    s = S.summarize(res, wall=50.0)
    assert s["requests"] == 100 and s["p50_s"] == 50.5 and abs(s["p99_s"] - 99.01) < 1e-9
    assert s["face_evals"] == 100_000 and s["face_evals_per_s"] == 2000.0
    assert [x["latency_s"] for x in s["slowest"]] == [100.0, 99.0, 98.0]
