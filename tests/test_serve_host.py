"""Host-side serving logic: the job population, arrivals, footprints, admission."""
import threading

import numpy as np


def test_jobs_are_seeded_and_in_range():
    from sde_gb300 import serve
    a = serve.make_job(3, sizes=(256, 512), ants=(27, 30), ints=(1, 4), chans=(1, 3))
    b = serve.make_job(3, sizes=(256, 512), ants=(27, 30), ints=(1, 4), chans=(1, 3))
    assert np.array_equal(a["vis"], b["vis"]) and a["imsize"] == b["imsize"]
    assert a["imsize"] in (256, 512)
    nbl_min, nbl_max = 27 * 26 // 2, 30 * 29 // 2
    assert nbl_min <= a["nvis"] <= nbl_max * 4 * 3


def test_poisson_rate():
    from sde_gb300.serve import poisson_arrivals
    t = poisson_arrivals(20000, 200.0)
    assert np.all(np.diff(t) > 0)
    assert abs(len(t) / t[-1] - 200.0) < 6.0


def test_footprint_grows_with_work():
    from sde_gb300.serve import footprint_bytes
    assert footprint_bytes(2_000_000, 1024) > footprint_bytes(1_000_000, 1024)
    assert footprint_bytes(1_000_000, 4096) > footprint_bytes(1_000_000, 1024)


def test_admission_waits_for_budget_and_slots():
    """The admission rule without a GPU: a stand-in server with two slots and a budget of
    10; jobs of 6 cannot run together, a job of 20 runs alone."""
    from sde_gb300.serve import Server
    s = Server.__new__(Server)
    s.slots = [None, None]
    s.budget = 10
    s._lock = threading.Condition()
    s._reserved = s._running = s.max_reserved = s.max_running = 0
    s._admit(6)
    done = []
    t = threading.Thread(target=lambda: (s._admit(6), done.append(1)))
    t.start()
    t.join(0.2)
    assert not done          # 6 + 6 > 10: waits
    s._release(6)
    t.join(2.0)
    assert done == [1]
    s._release(6)
    s._admit(20)             # larger than the budget: admitted when nothing runs
    assert s._running == 1
    s._release(20)
