"""Host logic of the serving layer on CPU: admission by HBM footprint, slot
reuse, request streams and latency statistics.  Slot creation (a library
context on the GPU) is replaced by a stub that records a fixed footprint,
so these run without a device; the GPU behaviour is in test_gpu_serving.py.
"""
import numpy as np
import pytest

from dg_nn_public_gb300 import serving


class _StubSlot:
    def __init__(self):
        self.busy = False


def _server(budget, footprint, max_slots=8):
    srv = serving.SolveServer([2, 3], hbm_budget=budget, max_slots_per_size=max_slots)

    def new_slot(n):
        slot = _StubSlot()
        srv.footprint.setdefault(n, float(footprint[n]))
        srv.used += srv.footprint[n]
        srv.slots[n].append(slot)
        return slot

    srv._new_slot = new_slot
    return srv


def test_admission_stays_within_budget():
    srv = _server(budget=10.0, footprint={2: 3.0, 3: 4.0})
    got = [srv._acquire(2) for _ in range(4)]
    # three slots of 3.0 fit in 10.0, the fourth request waits
    assert sum(s is not None for s in got) == 3 and got[3] is None
    assert srv.used == 9.0
    # no room for a size-3 slot (4.0) either, but the first slot of a size
    # is always admitted so that no mesh starves
    s3 = srv._acquire(3)
    assert s3 is not None and srv.used == 13.0
    assert srv._acquire(3) is None


def test_free_slot_is_reused_before_creating_one():
    srv = _server(budget=100.0, footprint={2: 1.0, 3: 1.0})
    a = srv._acquire(2)
    a.busy = False
    b = srv._acquire(2)
    assert b is a and len(srv.slots[2]) == 1


def test_max_slots_per_size():
    srv = _server(budget=1e9, footprint={2: 1.0, 3: 1.0}, max_slots=2)
    assert srv._acquire(2) is not None and srv._acquire(2) is not None
    assert srv._acquire(2) is None


def test_prewarm_respects_budget():
    srv = _server(budget=7.0, footprint={2: 3.0, 3: 4.0})
    srv.prewarm({2: 5})
    assert len(srv.slots[2]) == 2 and srv.used == 6.0


def test_request_stream_is_seeded_and_ordered():
    r1 = serving.make_requests([2, 3], count=6, rate=10.0, seed=3)
    r2 = serving.make_requests([2, 3], count=6, rate=10.0, seed=3)
    assert [r.n for r in r1] == [r.n for r in r2]
    assert all(np.array_equal(a.kappa, b.kappa) and np.array_equal(a.f, b.f) for a, b in zip(r1, r2))
    arr = [r.arrival for r in r1]
    assert arr == sorted(arr) and arr[0] == 0.0
    assert all(r.kappa.shape == (6 * r.n ** 3,) and r.f.shape == (6 * r.n ** 3 * 20,) for r in r1)


def test_latency_stats():
    res = [serving.Result(i, 2, np.zeros(20 * 48), 10, 0.0, 1.0, arrival=0.1 * i, start=0.1 * i,
                          end=0.1 * i + 0.2 + 0.01 * i, build_s=0.05, solve_s=0.15) for i in range(10)]
    st = serving.latency_stats(res)
    lat = np.array([0.2 + 0.01 * i for i in range(10)])
    assert st["p50_s"] == pytest.approx(np.percentile(lat, 50))
    assert st["p99_s"] == pytest.approx(np.percentile(lat, 99))
    assert st["requests"] == 10 and st["mean_wait_s"] == 0.0
    assert st["mean_build_s"] == pytest.approx(0.05) and st["mean_solve_s"] == pytest.approx(0.15)
    span = res[-1].end - res[0].arrival
    assert st["dofs_per_s"] == pytest.approx(10 * 960 / span)
