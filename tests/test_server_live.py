"""The live serving API's host logic without a GPU (dry-run mode): requests submitted one by one,
ticks driven by the caller, tickets polled for their state and result.  Admission order, the
budget and max_worlds limits, immediate rejection, statistics, and the guard against replaying a
trace while live requests are pending."""
from __future__ import annotations

import pytest

import master_thesis_gb300 as T


def req(w, h, steps, plates=8, seed=1):
    return T.Request(width=w, height=h, plates=plates, steps=steps, velRange=1.0, genSeed=seed,
                     worldSeed=seed, arrival_s=123.0)


def dry_server(budget, max_worlds=0):
    sv = T.Server(T.baseline_settings(), budget, max_worlds=max_worlds, dry_run=True)
    sv.set_dry_cost(1e-3)
    return sv


def test_lifecycle_waiting_running_done():
    sv = dry_server(4 * T.world_bytes(256, 256))
    tickets = [sv.submit(req(256, 256, s, seed=i)) for i, s in enumerate([2, 0, 3])]
    assert tickets == [0, 1, 2]
    for t in tickets:
        state, r = sv.poll(t)
        assert state == T.REQUEST_WAITING and r.status == 0 and r.admit_s < 0
        assert r.arrival_s == 0.0  # submission time on the (simulated) server clock, not the request's
    assert sv.tick() == (2, 0)     # the zero-step request retires at admission
    assert sv.poll(1)[0] == T.REQUEST_DONE
    assert sv.poll(0)[0] == T.REQUEST_RUNNING and sv.poll(2)[0] == T.REQUEST_RUNNING
    assert sv.tick() == (1, 0)     # request 0 finished its two steps
    assert sv.poll(0)[0] == T.REQUEST_DONE
    assert sv.tick() == (0, 0)
    for t in tickets:
        state, r = sv.poll(t)
        assert state == T.REQUEST_DONE and r.status == 0
        assert r.arrival_s <= r.admit_s <= r.finish_s
    st = sv.live_stats()
    assert st.completed == 3 and st.rejected == 0 and st.ticks == 3 and st.max_active == 2
    assert st.cell_updates == 256 * 256 * 5
    sv.close()


def test_impossible_requests_are_answered_at_submission():
    sv = dry_server(T.world_bytes(512, 512))
    big = sv.submit(req(2048, 2048, 5))
    bad = sv.submit(req(0, 64, 5))
    too_many_plates = sv.submit(req(64, 64, 5, plates=300))
    ok = sv.submit(req(256, 256, 1))
    assert sv.poll(big)[0] == T.REQUEST_DONE and sv.poll(big)[1].status == -6
    assert sv.poll(bad)[1].status == -1 and sv.poll(too_many_plates)[1].status == -1
    assert sv.poll(ok)[0] == T.REQUEST_WAITING
    assert sv.drain() == 1
    st = sv.live_stats()
    assert st.completed == 1 and st.rejected == 1
    sv.close()


def test_first_come_first_served_and_budget():
    big = T.world_bytes(1024, 1024)
    budget = big + T.world_bytes(256, 256) // 2
    sv = dry_server(budget)
    a = sv.submit(req(1024, 1024, 3))
    b = sv.submit(req(1024, 1024, 2))
    c = sv.submit(req(256, 256, 1))  # would fit beside a, but may not overtake b
    assert sv.tick() == (1, 2)
    assert sv.poll(c)[0] == T.REQUEST_WAITING
    sv.tick(), sv.tick()             # a done after its third step
    assert sv.poll(a)[0] == T.REQUEST_DONE
    sv.drain()
    ra, rb, rc = (sv.poll(t)[1] for t in (a, b, c))
    assert rb.admit_s >= ra.finish_s and rc.admit_s >= rb.admit_s
    assert sv.live_stats().peak_bytes <= budget
    sv.close()


def test_max_worlds_bounds_the_batch():
    sv = dry_server(100 * T.world_bytes(128, 128), max_worlds=3)
    for i in range(7):
        sv.submit(req(128, 128, 4, seed=i))
    seen = []
    while True:
        a, w = sv.tick()
        seen.append(a)
        if a == 0 and w == 0:
            break
    st = sv.live_stats()
    assert st.max_active == 3 and st.completed == 7
    assert max(seen) <= 3


def test_requests_join_mid_flight():
    sv = dry_server(8 * T.world_bytes(256, 256))
    first = sv.submit(req(256, 256, 10))
    for _ in range(4):
        sv.tick()
    late = sv.submit(req(256, 256, 2))
    sv.tick()
    assert sv.poll(late)[0] == T.REQUEST_RUNNING and sv.poll(first)[0] == T.REQUEST_RUNNING
    sv.tick()
    assert sv.poll(late)[0] == T.REQUEST_DONE and sv.poll(first)[0] == T.REQUEST_RUNNING
    sv.drain()
    assert sv.live_stats().max_active == 2


def test_trace_replay_is_refused_while_live_requests_are_pending():
    sv = dry_server(4 * T.world_bytes(256, 256))
    sv.submit(req(256, 256, 3))
    with pytest.raises(T.TectoError) as e:
        sv.run_trace([req(256, 256, 1)])
    assert e.value.code == -1
    sv.drain()
    res, st = sv.run_trace([req(256, 256, 1)])
    assert st.completed == 1 and res[0].status == 0


def test_poll_of_an_unknown_ticket_fails():
    sv = dry_server(T.world_bytes(64, 64))
    with pytest.raises(T.TectoError):
        sv.poll(0)
    t = sv.submit(req(64, 64, 1))
    with pytest.raises(T.TectoError):
        sv.poll(t + 1)
    with pytest.raises(T.TectoError):
        sv.poll(-1)
