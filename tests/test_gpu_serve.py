"""Serving with continuous batching: each request's result is the same alone
and in the mix (bit-identical: the per-cell arithmetic does not depend on
which shots share the launches), with requests arriving while others run,
cancellations, an oversize request and a small device budget."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def request(seed, t_end=0.12):
    from ela3d_gb300 import configs

    return configs.serving_request(seed, t_end=t_end, lo=40, hi=96)


def alone(p, cp, cs, rho):
    from ela3d_gb300 import Plan

    with Plan(p, cp, cs, rho, variant=0) as plan:
        plan.run(p.nstep)
        return plan.seismograms()


def test_mix_equals_alone_with_late_arrivals(built):
    from ela3d_gb300 import Server

    reqs = [request(s) for s in range(8)]
    want = [alone(*r) for r in reqs]
    with Server(steps_per_round=37, variant=0) as srv:
        tickets = [srv.submit(*reqs[q]) for q in range(4)]
        time.sleep(0.05)                     # the first four are running
        tickets += [srv.submit(*reqs[q]) for q in range(4, 8)]
        for q, t in enumerate(tickets):
            srv.wait(t)
            assert np.array_equal(srv.read(t), want[q]), q
        st = srv.stats()
    assert st["completed"] == 8 and st["failed"] == 0
    assert st["latency_p99_s"] >= st["latency_p50_s"] > 0
    assert st["rounds"] > 1


def test_streaming_samples_arrive_before_completion(built):
    from ela3d_gb300 import Server
    from ela3d_gb300._abi import REQ_DONE, REQ_RUNNING

    p, cp, cs, rho = request(11, t_end=0.25)
    want = alone(p, cp, cs, rho)
    seen_partial = False
    with Server(steps_per_round=20, variant=0) as srv:
        t = srv.submit(p, cp, cs, rho)
        got = np.zeros_like(want)
        done = 0
        while True:
            state, ready = srv.poll(t)
            if ready > done:
                got[:, :, done:ready] = srv.read(t, done, ready - done)
                if state == REQ_RUNNING:
                    seen_partial = True
                done = ready
            if state == REQ_DONE and done == p.nsamp:
                break
            time.sleep(0.002)
    assert seen_partial
    assert np.array_equal(got, want)


def test_cancel_and_oversize_leave_others_identical(built):
    from ela3d_gb300 import Ela3dError, Server

    reqs = [request(s) for s in range(20, 26)]
    want = [alone(*r) for r in reqs]
    with Server(steps_per_round=25, variant=0, hbm_budget_bytes=256 << 20) as srv:
        big = request(99)
        big_p = big[0].with_(nx=400, ny=400, nz=200, rec=np.zeros((0, 3), np.int32), src=(5, 5, 5))
        n = big_p.cells
        m = np.ones(n, np.float32)
        t_big = srv.submit(big_p, m * 3000, m * 1700, m * 2000)
        tickets = [srv.submit(*r) for r in reqs]
        srv.cancel(tickets[2])
        with pytest.raises(Ela3dError) as e:
            srv.wait(t_big)
        assert e.value.status == 7   # ELA3D_ERR_BUSY: larger than the whole budget
        assert "budget" in str(e.value)   # the worker's reason reaches the client thread
        for q, t in enumerate(tickets):
            if q == 2:
                with pytest.raises(Ela3dError):
                    srv.wait(t)
                continue
            srv.wait(t)
            assert np.array_equal(srv.read(t), want[q]), q
        st = srv.stats()
    assert st["cancelled"] == 1 and st["failed"] == 1 and st["completed"] == 5


def test_small_budget_serialises_admission(built):
    from ela3d_gb300 import Server

    reqs = [request(s) for s in range(40, 44)]
    want = [alone(*r) for r in reqs]
    with Server(steps_per_round=30, variant=0, max_active=1) as srv:
        tickets = [srv.submit(*r) for r in reqs]
        for q, t in enumerate(tickets):
            srv.wait(t)
            assert np.array_equal(srv.read(t), want[q])


def test_concurrent_clients(built):
    from ela3d_gb300 import Server

    reqs = [request(s) for s in range(60, 66)]
    want = [alone(*r) for r in reqs]
    out = [None] * len(reqs)
    with Server(steps_per_round=40, variant=0) as srv:
        def client(q):
            t = srv.submit(*reqs[q])
            srv.wait(t)
            out[q] = srv.read(t)
            srv.release(t)
        th = [threading.Thread(target=client, args=(q,)) for q in range(len(reqs))]
        for x in th:
            x.start()
        for x in th:
            x.join()
    for q in range(len(reqs)):
        assert np.array_equal(out[q], want[q])


def test_fill_target_admits_in_order_and_keeps_results(built):
    """With a fill target below one request's cells the server runs one
    request at a time, in arrival order; results are unchanged."""
    from ela3d_gb300 import Server
    from ela3d_gb300._abi import REQ_DONE, REQ_RUNNING

    reqs = [request(s) for s in range(80, 84)]
    want = [alone(*r) for r in reqs]
    with Server(steps_per_round=15, variant=0, fill_cells=1) as srv:
        tickets = [srv.submit(*r) for r in reqs]
        most, done_order = 0, []
        while len(done_order) < len(tickets):
            states = [srv.poll(t)[0] for t in tickets]
            most = max(most, sum(s == REQ_RUNNING for s in states))
            for q, s in enumerate(states):
                if s == REQ_DONE and q not in done_order:
                    done_order.append(q)
            time.sleep(0.001)
        for q, t in enumerate(tickets):
            assert np.array_equal(srv.read(t), want[q]), q
    assert most <= 1
    assert done_order == sorted(done_order)


def test_fp64_requests_equal_alone(built):
    """An FP64 server: each request's seismograms equal the FP64 shot run alone."""
    from ela3d_gb300 import Plan, Server

    reqs = [request(s, t_end=0.08) for s in range(90, 93)]
    reqs = [(p.with_(precision=1), cp, cs, rho) for p, cp, cs, rho in reqs]
    want = []
    for p, cp, cs, rho in reqs:
        with Plan(p, cp, cs, rho) as plan:
            plan.run(p.nstep)
            want.append(plan.seismograms())
    with Server(steps_per_round=20, precision=1) as srv:
        tickets = [srv.submit(*r) for r in reqs]
        for q, t in enumerate(tickets):
            srv.wait(t)
            assert np.array_equal(srv.read(t), want[q]), q


def test_destroy_releases_waiting_clients(built):
    """Destroying the server while client threads wait on unfinished requests
    (one running, one queued behind a one-slot limit) ends those requests as
    cancelled: every waiter returns ELA3D_ERR_CANCELLED, none is left
    blocked on a server that no longer exists."""
    from ela3d_gb300 import Ela3dError, Server

    reqs = [request(s) for s in (40, 41)]
    reqs = [(r[0].with_(nstep=50_000),) + tuple(r[1:]) for r in reqs]   # seconds of work each
    srv = Server(steps_per_round=10, max_active=1)
    tickets = [srv.submit(*r) for r in reqs]
    got = {}

    def client(q, t):
        try:
            srv.wait(t)
            got[q] = 0
        except Ela3dError as e:
            got[q] = e.status

    threads = [threading.Thread(target=client, args=(q, t)) for q, t in enumerate(tickets)]
    for th in threads:
        th.start()
    time.sleep(0.3)
    srv.close()
    for th in threads:
        th.join(timeout=30)
        assert not th.is_alive()
    assert got == {0: 8, 1: 8}   # ELA3D_ERR_CANCELLED


def test_completion_callbacks_once_each_with_the_final_status(built):
    """ela3d_server_on_done: every request's callback runs exactly once with
    its final status -- done, cancelled while queued, cancelled while
    running, refused as oversize, or cancelled by the server's destruction --
    and a callback may read the results (it is called without the server's
    lock).  One slot at a time makes every outcome deterministic."""
    from ela3d_gb300 import Server

    reqs = [request(s) for s in range(60, 64)]
    want = [alone(*r) for r in reqs]
    calls, seen = [], {}

    def done(t, st):
        calls.append((t, st))
        if st == 0:
            seen[t] = srv.read(t)

    long_p = reqs[0][0].with_(nstep=50_000)                         # seconds of work
    srv = Server(steps_per_round=20, variant=0, hbm_budget_bytes=256 << 20, max_active=1)
    t_first = srv.submit(long_p, *reqs[0][1:])                      # holds the only slot
    tickets = [srv.submit(*r) for r in reqs]                        # queued behind it
    big_p = reqs[1][0].with_(nx=400, ny=400, nz=200, rec=np.zeros((0, 3), np.int32), src=(5, 5, 5))
    m = np.ones(big_p.cells, np.float32)
    t_big = srv.submit(big_p, m * 3000, m * 1700, m * 2000)         # larger than the budget
    t_last = srv.submit(long_p, *reqs[0][1:])                       # still running at close
    for t in [t_first, *tickets, t_big, t_last]:
        srv.on_done(t, done)
    srv.cancel(tickets[3])                                          # while queued
    srv.cancel(t_first)                                             # while running
    for t in tickets[:3]:
        srv.wait(t)
    late = []
    srv.on_done(tickets[0], lambda t, st: late.append((t, st)))     # already over: called at once
    assert late == [(tickets[0], 0)]
    srv.close()
    got = dict(calls)
    assert len(calls) == len(got) == 7
    assert [got[t] for t in tickets[:3]] == [0, 0, 0]
    # ELA3D_ERR_CANCELLED (queued, running, at destruction), ELA3D_ERR_BUSY
    assert (got[tickets[3]], got[t_first], got[t_last], got[t_big]) == (8, 8, 8, 7)
    for q in range(3):
        assert np.array_equal(seen[tickets[q]], want[q])


def test_randomised_clients_every_request_ends_once(built):
    """Eight client threads, each with its own seeded script: submit
    requests (some generated on the device), cancel some at random moments,
    poll and read partial samples while they run, register completion
    callbacks, wait, release.  Invariants: every request ends exactly once
    (one callback, one final state), a request that ends done has exactly its
    alone result, a cancelled one reports ELA3D_ERR_CANCELLED, and the
    server's counts add up."""
    import random

    from ela3d_gb300 import Ela3dError, Server

    pool = [request(s) for s in range(70, 76)]
    want = [alone(*r) for r in pool]
    ends, results, errors = {}, {}, []
    lock = threading.Lock()

    def on_done(t, st):
        with lock:
            ends.setdefault(t, []).append(st)

    with Server(steps_per_round=15, variant=0, max_active=5) as srv:
        def client(cid):
            rnd = random.Random(cid)
            mine = []
            try:
                for _ in range(4):
                    q = rnd.randrange(len(pool))
                    t = srv.submit(*pool[q])
                    srv.on_done(t, on_done)
                    mine.append((t, q, rnd.random() < 0.25))
                    time.sleep(rnd.uniform(0, 0.01))
                for t, q, kill in mine:
                    if kill:
                        srv.cancel(t)
                    state, ready = srv.poll(t)
                    if ready:
                        srv.read(t, 0, ready)        # a partial read while it may still run
                for t, q, kill in mine:
                    try:
                        srv.wait(t)
                        with lock:
                            results[t] = (q, srv.read(t))
                    except Ela3dError as e:
                        assert kill and e.status == 8, (t, e.status)
                    srv.release(t)
            except Exception as e:  # reported to the main thread
                errors.append(repr(e))

        th = [threading.Thread(target=client, args=(c,)) for c in range(8)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        st = srv.stats()
    assert not errors, errors
    assert len(ends) == 32 and all(len(v) == 1 for v in ends.values())
    done = [t for t, v in ends.items() if v[0] == 0]
    assert sorted(done) == sorted(results)
    assert all(v[0] in (0, 8) for v in ends.values())
    for t, (q, seis) in results.items():
        assert np.array_equal(seis, want[q]), t
    assert st["submitted"] == 32 and st["completed"] + st["cancelled"] == 32 and st["failed"] == 0
