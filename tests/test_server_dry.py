"""The serving runtime's host logic without a GPU (dry-run mode: a tick costs a modelled time per
active cell).  Admission against the HBM budget, first-come first-served order, rejection of
requests that can never fit, latency statistics, and the one-at-a-time baseline."""
from __future__ import annotations

import numpy as np

import master_thesis_gb300 as T


def req(w, h, steps, t, plates=8, seed=1):
    return T.Request(width=w, height=h, plates=plates, steps=steps, velRange=1.0, genSeed=seed,
                     worldSeed=seed, arrival_s=t)


def test_budget_is_never_exceeded_and_everything_completes():
    rng = np.random.default_rng(0)
    sizes = [(256, 256), (512, 256), (1024, 1024)]
    reqs = [req(*sizes[rng.integers(0, 3)], int(rng.integers(5, 40)), float(rng.uniform(0, 2.0)), seed=i)
            for i in range(60)]
    budget = 3 * T.world_bytes(1024, 1024)
    sv = T.Server(T.baseline_settings(), budget, dry_run=True)
    sv.set_dry_cost(2e-3)
    res, st = sv.run_trace(reqs)
    assert st.completed == 60 and st.rejected == 0
    assert st.peak_bytes <= budget
    for r, q in zip(res, reqs):
        assert r.status == 0
        assert q.arrival_s <= r.admit_s <= r.finish_s
    assert st.latency_p50_s <= st.latency_p99_s
    assert st.cell_updates == sum(q.width * q.height * q.steps for q in reqs)


def test_oversized_requests_are_rejected_and_others_served():
    budget = T.world_bytes(512, 512)
    reqs = [req(256, 256, 5, 0.0), req(2048, 2048, 5, 0.0), req(512, 512, 3, 0.1)]
    sv = T.Server(T.baseline_settings(), budget, dry_run=True)
    res, st = sv.run_trace(reqs)
    assert [r.status for r in res] == [0, -6, 0]
    assert st.completed == 2 and st.rejected == 1


def test_admission_is_first_come_first_served():
    # the budget holds one large world: the second large request waits although a small one
    # arriving later would fit, so admissions follow arrival order
    big = T.world_bytes(1024, 1024)
    budget = big + T.world_bytes(256, 256) // 2
    reqs = [req(1024, 1024, 10, 0.0), req(1024, 1024, 10, 0.01), req(256, 256, 1, 0.02)]
    sv = T.Server(T.baseline_settings(), budget, dry_run=True)
    sv.set_dry_cost(1e-2)
    res, st = sv.run_trace(reqs)
    admits = [r.admit_s for r in res]
    assert admits[0] < admits[1] <= admits[2]
    assert res[1].admit_s >= res[0].finish_s


def test_requests_overlap_under_continuous_batching():
    rng = np.random.default_rng(1)
    # a tick of one 256x256 world costs 66 us in this model; requests arrive every 0.5 ms
    reqs = [req(256, 256, int(rng.integers(10, 50)), i * 0.0005, seed=i) for i in range(40)]
    budget = 64 * T.world_bytes(256, 256)
    sv = T.Server(T.baseline_settings(), budget, dry_run=True)
    sv.set_dry_cost(1e-3)
    res, cont = sv.run_trace(reqs)
    _, seq = sv.run_trace_sequential(reqs)
    assert cont.completed == seq.completed == 40
    assert cont.max_active > 1 and seq.max_active == 1
    # requests admitted while others are mid-flight
    spans = sorted((r.admit_s, r.finish_s) for r in res)
    assert any(b[0] < a[1] for a, b in zip(spans, spans[1:]))
    # the model charges the same per cell either way, so the total busy time agrees
    work = sum(q.width * q.height * q.steps for q in reqs) / 1e6 * 1e-3
    assert cont.wall_s >= work - 1e-9 and seq.wall_s >= work - 1e-9


def test_world_bytes_grows_with_the_grid():
    a, b = T.world_bytes(256, 256), T.world_bytes(1024, 1024)
    assert a > 256 * 256 * 90 and b > 16 * (a - 2_000_000)


def test_output_settings_are_checked_and_dry_runs_write_nothing(tmp_path):
    sv = T.Server(T.baseline_settings(), T.world_bytes(256, 256), dry_run=True)
    for bad in [(tmp_path, 8, 0.0, 1.0), (tmp_path, -1, 0.0, 1.0), (None, T.SERVER_OUT_SNAPSHOT, 0.0, 1.0),
                (tmp_path, T.SERVER_OUT_HEIGHT_PNG, 1.0, 1.0)]:
        try:
            sv.set_output(*bad)
        except T.TectoError:
            continue
        raise AssertionError(f"accepted {bad}")
    sv.set_output(tmp_path, T.SERVER_OUT_HEIGHT_PNG | T.SERVER_OUT_PLATES_PNG | T.SERVER_OUT_SNAPSHOT, -1.0, 1.0)
    res, st = sv.run_trace([req(64, 64, 3, 0.0), req(32, 32, 2, 0.01)])
    assert st.completed == 2 and all(r.status == 0 for r in res)
    assert list(tmp_path.iterdir()) == []
    sv.set_output(None, 0)  # off again


def test_heavy_requests_run_one_at_a_time_and_light_ones_ride_along():
    # two heavy requests (2^20 cells each) and a light one arriving while the second heavy waits:
    # the heavies run one after the other in arrival order, the light one joins at once
    reqs = [req(1024, 1024, 20, 0.0, seed=1), req(2048, 512, 20, 0.001, seed=2), req(256, 256, 5, 0.002, seed=3)]
    sv = T.Server(T.baseline_settings(), 10 * T.world_bytes(2048, 512), dry_run=True)
    sv.set_dry_cost(1e-3)
    res, st = sv.run_trace(reqs)
    assert st.completed == 3
    assert res[1].admit_s >= res[0].finish_s                   # one heavy at a time
    assert res[2].admit_s < res[0].finish_s                    # the light one overtakes the waiting heavy
    assert res[2].finish_s < res[1].admit_s
    # with the limit lifted both heavies overlap again
    sv.set_policy(1 << 20, 0)
    res2, st2 = sv.run_trace(reqs)
    assert st2.completed == 3 and res2[1].admit_s < res2[0].finish_s
    # two heavy slots: both heavies overlap, a third waits for a slot in arrival order
    sv.set_policy(1 << 20, 2)
    reqs3 = reqs[:2] + [req(1024, 1024, 20, 0.0015, seed=4)] + reqs[2:]
    res3, st3 = sv.run_trace(reqs3)
    assert st3.completed == 4
    assert res3[1].admit_s < res3[0].finish_s
    assert res3[2].admit_s >= min(res3[0].finish_s, res3[1].finish_s)
    # a lower threshold makes the 256^2 request heavy too: it waits for the first heavy
    sv.set_policy(256 * 256, 1)
    res4, _ = sv.run_trace(reqs)
    assert res4[2].admit_s >= res4[1].finish_s


def test_policy_arguments_are_checked():
    sv = T.Server(T.baseline_settings(), T.world_bytes(256, 256), dry_run=True)
    for bad in ((1 << 20, -1), (0, 1)):
        try:
            sv.set_policy(*bad)
        except T.TectoError:
            continue
        raise AssertionError(f"accepted {bad}")
    sv.set_policy(0, 0)
