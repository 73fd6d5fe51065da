"""The serving loop (cpvs_server): continuous batching of builds and lookups
from several client threads, residency under a byte budget, cancellation.
Each served answer must equal the plain API's answer for that request alone."""
import threading

import numpy as np
import pytest

from cpvs_gb300 import scene

pytestmark = pytest.mark.gpu


def maps_for(sizes, seed0):
    return [scene.rasterise(scene.make_scene(n, 0.9, 40, 2, seed0 + i)) for i, n in enumerate(sizes)]


def test_served_answers_equal_alone(cp):
    sizes = [256, 1024, 512, 2048, 128, 1024]
    maps = maps_for(sizes, 700)
    alone_ctx = cp.Context(0)
    alone = {k: cp.CompressedShadow.from_depth(m, ctx=alone_ctx) for k, m in enumerate(maps)}
    srv = cp.Server(cp.Context(0))
    build_tickets = [srv.submit_build(k, m) for k, m in enumerate(maps)]
    results, errors = {}, []
    lock = threading.Lock()

    def client(cid):
        rng = np.random.default_rng(cid)
        for _ in range(40):
            key = int(rng.integers(0, len(maps)))
            n = int(2 ** rng.uniform(6, 16))
            pts = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
            try:
                t = srv.submit_lookup(key, pts)
                _, bits = srv.wait(t)
                with lock:
                    results[(cid, len(results))] = (key, pts, bits)
            except Exception as e:  # noqa: BLE001
                errors.append(repr(e))

    threads = [threading.Thread(target=client, args=(c,)) for c in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for t in build_tickets:
        srv.wait(t)
    assert not errors, errors[:3]
    assert len(results) == 160
    for key, pts, bits in results.values():
        assert np.array_equal(bits, alone[key].lookup_ndc(pts))
    st = srv.stats()
    assert st["builds_done"] == len(maps) and st["lookups_done"] == 160 and st["failed"] == 0
    assert st["resident_dags"] == len(maps)
    assert st["lookup_p99_ms"] >= st["lookup_p50_ms"] > 0
    srv.close()


def test_lookup_waits_for_its_build_and_unknown_key_fails(cp):
    srv = cp.Server(cp.Context(0))
    m = maps_for([1024], 800)[0]
    pts = np.random.default_rng(1).uniform(-1, 1, (5000, 3)).astype(np.float32)
    tb = srv.submit_build(7, m)
    tl = srv.submit_lookup(7, pts)  # submitted before the build is done
    _, bits = srv.wait(tl)
    srv.wait(tb)
    assert np.array_equal(bits, cp.CompressedShadow.from_depth(m).lookup_ndc(pts))
    with pytest.raises(cp.CpvsError) as e:
        srv.wait(srv.submit_lookup(99, pts))
    assert e.value.status == 1
    srv.close()


def test_budget_evicts_least_recently_used(cp):
    maps = maps_for([512, 512, 512, 512], 900)
    sizes = [cp.CompressedShadow.from_depth(m).dag_size() * 4 for m in maps]
    budget = sizes[0] + sizes[1] + sizes[2] // 2  # room for about two DAGs
    srv = cp.Server(cp.Context(0), budget_bytes=budget)
    for k, m in enumerate(maps):
        srv.wait(srv.submit_build(k, m))
    st = srv.stats()
    assert st["evictions"] >= 2 and st["resident_bytes"] <= budget
    pts = np.zeros((64, 3), np.float32)
    srv.wait(srv.submit_lookup(3, pts))  # the newest stays resident
    with pytest.raises(cp.CpvsError):
        srv.wait(srv.submit_lookup(0, pts))  # the oldest was evicted
    srv.close()


def test_cancel_a_waiting_lookup(cp):
    srv = cp.Server(cp.Context(0))
    m = maps_for([4096], 950)[0]
    pts = np.zeros((1000, 3), np.float32)
    tb = srv.submit_build(1, m)
    tl = srv.submit_lookup(1, pts)
    try:
        srv.cancel(tl)
        cancelled = True
    except cp.CpvsError:
        cancelled = False  # it already ran: then it completes normally
    if cancelled:
        with pytest.raises(cp.CpvsError) as e:
            srv.wait(tl)
        assert e.value.status == 7
    else:
        srv.wait(tl)
    srv.wait(tb)
    srv.close()


def test_rebuild_orders_lookups_by_generation(cp):
    a, b = maps_for([1024, 1024], 1000)
    pts = np.random.default_rng(2).uniform(-1, 1, (20000, 3)).astype(np.float32)
    want_a = cp.CompressedShadow.from_depth(a).lookup_ndc(pts)
    want_b = cp.CompressedShadow.from_depth(b).lookup_ndc(pts)
    assert not np.array_equal(want_a, want_b)
    srv = cp.Server(cp.Context(0))
    srv.wait(srv.submit_build(5, a))
    t_old = srv.submit_lookup(5, pts)   # needs the first build (or a later one)
    t_build = srv.submit_build(5, b)
    t_new = srv.submit_lookup(5, pts)   # needs the second build
    _, bits_new = srv.wait(t_new)
    _, bits_old = srv.wait(t_old)
    srv.wait(t_build)
    assert np.array_equal(bits_new, want_b)
    assert np.array_equal(bits_old, want_a) or np.array_equal(bits_old, want_b)
    with pytest.raises(cp.CpvsError) as e:
        srv.wait(srv.submit_lookup(6, pts))  # never built
    assert e.value.status == 1
    srv.close()


def test_lookup_after_a_failed_build_fails(cp):
    m = maps_for([2048], 1100)[0]
    dag_bytes = cp.CompressedShadow.from_depth(m).dag_size() * 4
    srv = cp.Server(cp.Context(0), budget_bytes=dag_bytes // 2)
    tb = srv.submit_build(3, m)
    tl = srv.submit_lookup(3, np.zeros((100, 3), np.float32))
    with pytest.raises(cp.CpvsError) as e:
        srv.wait(tb)
    assert e.value.status == 6  # CPVS_ERR_BUDGET
    with pytest.raises(cp.CpvsError) as e:
        srv.wait(tl)
    assert e.value.status == 1
    srv.close()
