"""CPU tests of the serving host logic: the admission policy (simulated),
the device-byte bound used for admission, and the seeded job stream."""
import numpy as np
import pytest

import nwchem_gb300 as ng
from nwchem_gb300 import serve


def _check_policy(arr, nb, svc, budget, slots):
    start, end = serve.simulate(arr, nb, svc, budget, slots)
    ok = start >= 0
    assert np.array_equal(ok, nb <= budget)            # only jobs larger than the budget are refused
    assert np.all(start[ok] >= arr[ok] - 1e-12)
    assert np.allclose(end[ok] - start[ok], svc[ok])
    s = start[ok]
    assert np.all(np.diff(s) >= -1e-12)                # FIFO admission
    # at every admission: running jobs within slots and bytes within budget
    for q in np.flatnonzero(ok):
        t = start[q]
        run = ok & (start <= t + 1e-12) & (end > t + 1e-12)
        assert run.sum() <= slots
        assert nb[run].sum() <= budget
    return start, end


def test_admission_policy_random_streams():
    rng = np.random.default_rng(0)
    for trial in range(20):
        n = int(rng.integers(1, 60))
        arr = np.cumsum(rng.exponential(0.02, n))
        nb = rng.integers(1, 100, n).astype(np.int64)
        svc = rng.uniform(0.001, 0.2, n)
        budget, slots = int(rng.integers(60, 200)), int(rng.integers(1, 5))
        nb[rng.random(n) < 0.05] = budget + 1           # a few that can never fit
        _check_policy(arr, nb, svc, budget, slots)


def test_admission_waits_for_memory_then_starts_at_release():
    arr = np.array([0.0, 0.0, 0.0])
    nb = np.array([60, 60, 30], dtype=np.int64)
    svc = np.array([1.0, 1.0, 1.0])
    start, end = _check_policy(arr, nb, svc, 100, 4)
    # job 1 does not fit beside job 0; FIFO keeps job 2 behind it
    assert start.tolist() == [0.0, 1.0, 1.0] and end.tolist() == [1.0, 2.0, 2.0]


def test_admission_is_work_conserving_when_everything_fits():
    arr = np.linspace(0, 1, 11)
    nb = np.ones(11, dtype=np.int64)
    svc = np.full(11, 0.05)
    start, _ = _check_policy(arr, nb, svc, 100, 2)
    assert np.allclose(start, arr)


def test_job_bytes_bound():
    t = ng.Tiling([8, 12], [16, 24, 32]).with_evl(0)
    f64, mx = serve.job_bytes(t, ng.PREC_FP64), serve.job_bytes(t, ng.PREC_MIXED_FP16)
    o, v = t.nocc, t.nvir
    assert f64 >= 8 * 3 * v * v * o * o and mx > f64
    big = ng.Tiling([8, 12, 16], [16, 24, 32, 48]).with_evl(0)
    assert serve.job_bytes(big, ng.PREC_MIXED_FP16) > mx


def test_job_stream_is_seeded_and_sized():
    a, b = serve.job_stream(30, 50.0, 7, 8, 40), serve.job_stream(30, 50.0, 7, 8, 40)
    assert [s.arrival for s in a] == [s.arrival for s in b]
    for s in a:
        t = s.tiling
        assert 8 <= t.nocc <= 40 and 5 * t.nocc - 1 <= t.nvir <= 8 * t.nocc + 1
        assert set(t.occ[:-1]) <= set(serve.OCC_SIZES) and set(t.vir[:-1]) <= set(serve.VIR_SIZES)
    arr = np.array([s.arrival for s in a])
    assert np.all(np.diff(arr) > 0) and 0.2 < arr[-1] < 1.5   # ~30 jobs at 50/s


def _check_deferred(arr, nb, svc, chk, budget, slots):
    start, ready, done = serve.simulate_checks(arr, nb, svc, chk, budget, slots)
    ok = start >= 0
    assert np.array_equal(ok, nb <= budget)
    assert np.all(start[ok] >= arr[ok] - 1e-12)
    assert np.all(np.diff(start[ok]) >= -1e-12)                      # FIFO admission
    assert np.allclose(ready[ok] - start[ok], svc[ok])
    has = ok & (chk >= 0)
    assert np.allclose(done[ok & (chk < 0)], ready[ok & (chk < 0)])
    assert np.all(done[has] - ready[has] >= chk[has] - 1e-12)        # a check never starts before the energies
    # at every event: slots hold mixed runs and running checks; admitted bytes (until done) fit
    times = np.unique(np.concatenate([start[ok], ready[ok], done[ok]]))
    for t in times:
        mixed = ok & (start <= t + 1e-12) & (ready > t + 1e-12)
        checking = has & (done - chk <= t + 1e-12) & (done > t + 1e-12)
        assert mixed.sum() + checking.sum() <= slots
        held = ok & (start <= t + 1e-12) & (done > t + 1e-12)
        assert nb[held].sum() <= budget
    return start, ready, done


def test_deferred_checks_random_streams():
    rng = np.random.default_rng(1)
    for trial in range(25):
        n = int(rng.integers(1, 50))
        arr = np.cumsum(rng.exponential(0.02, n))
        nb = rng.integers(1, 100, n).astype(np.int64)
        svc = rng.uniform(0.001, 0.1, n)
        chk = np.where(rng.random(n) < 0.3, rng.uniform(0.05, 2.0, n), -1.0)
        budget, slots = int(rng.integers(100, 300)), int(rng.integers(1, 5))
        nb[rng.random(n) < 0.05] = budget + 1
        _check_deferred(arr, nb, svc, chk, budget, slots)


def test_without_checks_matches_admission_policy():
    rng = np.random.default_rng(2)
    n = 40
    arr = np.cumsum(rng.exponential(0.02, n))
    nb = rng.integers(1, 100, n).astype(np.int64)
    svc = rng.uniform(0.001, 0.2, n)
    s0, e0 = serve.simulate(arr, nb, svc, 150, 3)
    s1, r1, d1 = serve.simulate_checks(arr, nb, svc, np.full(n, -1.0), 150, 3)
    assert np.allclose(s0, s1) and np.allclose(e0, r1) and np.allclose(r1, d1)


def test_queued_jobs_run_before_a_pending_check():
    # job 0 has a long check; job 1 is queued when job 0's energies are ready: it runs first
    arr = np.array([0.0, 0.05, 5.0])
    nb = np.array([10, 10, 10], dtype=np.int64)
    svc = np.array([0.1, 0.1, 0.1])
    chk = np.array([10.0, -1.0, -1.0])
    start, ready, done = _check_deferred(arr, nb, svc, chk, 1000, 1)
    assert start[1] == pytest.approx(0.1) and done[0] == pytest.approx(0.2 + 10.0)
    # one slot and a running check: a later job waits for it (checks are not preempted)
    assert start[2] == pytest.approx(10.2)
    # two slots: the later job starts on arrival beside the check
    start2, _, _ = _check_deferred(arr, nb, svc, chk, 1000, 2)
    assert start2[2] == pytest.approx(5.0)


def test_held_bytes_never_deadlock_the_queue():
    # every job is checked and the budget holds two: checks run whenever the head cannot fit
    n = 12
    arr = np.zeros(n)
    nb = np.full(n, 40, dtype=np.int64)
    svc = np.full(n, 0.1)
    chk = np.full(n, 0.5)
    start, ready, done = _check_deferred(arr, nb, svc, chk, 100, 4)
    assert np.all(done > 0) and done.max() < 1e3


def test_queue_settings_are_checked_without_a_gpu():
    """sdt_server_set_queue takes a precision, a work-unit shape of 1 or 2,
    at least one reserved SM and an idle time in (0, 1] s; the statistics
    start at zero and an unknown ticket is refused."""
    import ctypes as C
    import numpy as np
    from nwchem_gb300 import _capi
    lib = _capi.lib()
    lib.sdt_set_error_mode(1)
    h = C.c_void_p()
    _capi.check(lib.sdt_server_create(1 << 30, 2, 0, C.byref(h)), "sdt_server_create")
    try:
        for args in ((3, 3, 16, 0.2), (3, 2, 0, 0.2), (3, 2, 16, 0.0), (3, 2, 16, 1.5), (7, 2, 16, 0.2)):
            assert lib.sdt_server_set_queue(h, *args) == 1, args
            _capi.last_error()
        assert lib.sdt_server_set_queue(h, 3, 1, 24, 0.5) == 0
        assert lib.sdt_server_set_queue(h, 0, 2, 16, 0.2) == 0          # FP64: the queue off
        st = np.full(4, -1, dtype=np.int64)
        assert lib.sdt_server_queue_stats(h, st.ctypes.data_as(_capi.PI64)) == 0
        assert st.tolist() == [0, 0, 0, 0]
        a, b = C.c_int(), C.c_int()
        assert lib.sdt_server_job_launches(h, 5, C.byref(a), C.byref(b)) == 1
        _capi.last_error()
    finally:
        lib.sdt_server_destroy(h)
