"""Continuous-batching server: requests admitted as slots and memory free up,
sharing launches with whatever else is resident, give the same result as
when they run alone (bit-identical: one CTA computes one request's operation
with a fixed reduction order), and admission respects the HBM budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _req_params():
    return [dict(n=12, chi=16, p=0.1, depth=14, traj=0), dict(n=9, chi=8, p=0.25, depth=6, traj=1),
            dict(n=16, chi=32, p=0.05, depth=10, traj=2), dict(n=7, chi=4, p=0.3, depth=9, traj=3),
            dict(n=14, chi=16, p=0.15, depth=5, traj=4), dict(n=10, chi=32, p=0.2, depth=12, traj=5)]


def _run(pkg, reqs, slots, hbm, stagger, light_chi=0, light_ctas=0, class_stats=False):
    s = pkg.Server(hbm, max_slots=slots, precision="mixed", max_chi=32, max_n=16, light_chi=light_chi,
                   light_ctas=light_ctas)
    ids = {}
    pending = list(reqs)
    results = {}
    ticks = 0
    while pending or len(results) < len(reqs):
        # submit one request every `stagger` ticks so lifetimes overlap unevenly
        if pending and ticks % stagger == 0:
            r = pending.pop(0)
            ids[s.submit(r["n"], pkg.Trunc.both(r["chi"], 1e-10), r["p"], r["depth"], 99, r["traj"])] = r["traj"]
        s.tick()
        for d in s.poll():
            results[ids[d["id"]]] = d
        ticks += 1
        assert ticks < 500
    st = s.stats()
    if class_stats:
        st["classes"] = [s.class_stats(0), s.class_stats(1)]
    s.close()
    return results, st


def test_results_same_alone_and_in_the_mix(pkg):
    reqs = _req_params()
    mix, st = _run(pkg, reqs, slots=4, hbm=1 << 30, stagger=2)
    assert st["completed"] == len(reqs) and st["active"] == 0 and st["arena_used"] == 0
    for r in reqs:
        alone, _ = _run(pkg, [r], slots=1, hbm=1 << 30, stagger=1)
        a, m = alone[r["traj"]], mix[r["traj"]]
        assert a["layers"] == m["layers"] == r["depth"]
        assert a["final_entropy"] == m["final_entropy"], (r, a, m)


def test_two_classes_step_independently(pkg):
    # bond capacity <= 16 -> class 0 on 8 CTAs, 32 -> class 1 on the other SMs
    reqs = _req_params()
    mix, st = _run(pkg, reqs, slots=4, hbm=1 << 30, stagger=1, light_chi=16, light_ctas=8, class_stats=True)
    assert st["completed"] == len(reqs) and st["active"] == 0 and st["arena_used"] == 0
    c0, c1 = st["classes"]
    assert (c0["cap_max"], c0["ctas"], c1["cap_max"]) == (16, 8, 32)
    light = [r for r in reqs if min(r["chi"], 1 << (r["n"] // 2)) <= 16]
    heavy = [r for r in reqs if r not in light]
    assert c0["layers"] == sum(r["depth"] for r in light) and c1["layers"] == sum(r["depth"] for r in heavy)
    # the same request gives the same bits in either class layout and alone
    one, _ = _run(pkg, reqs, slots=4, hbm=1 << 30, stagger=1)
    for r in reqs:
        assert mix[r["traj"]]["final_entropy"] == one[r["traj"]]["final_entropy"], r


def test_admission_waits_for_memory(pkg):
    # an arena that holds one of these requests at a time: the second waits
    n, chi = 12, 32
    per = n * chi * chi * 2 * 8 + 8 * chi * (n + 1) + 4 * (n + 1)
    s = pkg.Server(int(per * 1.5) + 4096, max_slots=4, precision="mixed", max_chi=32, max_n=16)
    s.submit(n, pkg.Trunc.both(chi, 1e-10), 0.1, 4, 5, 0)
    s.submit(n, pkg.Trunc.both(chi, 1e-10), 0.1, 4, 5, 1)
    a, _ = s.tick()
    assert a == 1 and s.stats()["pending"] == 1
    done = []
    for _ in range(20):
        s.tick()
        done += s.poll()
        if len(done) == 2:
            break
    assert len(done) == 2
    assert done[1]["queue_s"] > 0.0
    with pytest.raises(pkg.TnError):
        s.submit(64, pkg.Trunc.both(32, 1e-10), 0.1, 4, 5, 2)  # n beyond max_n


def test_least_work_policy_and_active_cap(pkg):
    # one resident request at a time: the cheaper request, submitted second,
    # is admitted first under the least-work policy, and its result is the
    # same as under first come, first served
    out = {}
    for policy in ("fcfs", "least-work"):
        s = pkg.Server(1 << 30, max_slots=4, precision="mixed", max_chi=32, max_n=16)
        s.set_policy(policy, (1, 0))
        big = s.submit(14, pkg.Trunc.both(32, 1e-10), 0.1, 6, 3, 0)
        small = s.submit(8, pkg.Trunc.both(8, 1e-10), 0.1, 3, 3, 1)
        order = []
        res = {}
        for _ in range(40):
            a, _ = s.tick()
            assert a <= 1
            for d in s.poll():
                order.append(d["id"])
                res[d["id"]] = d
            if len(order) == 2:
                break
        s.close()
        assert sorted(order) == sorted([big, small])
        out[policy] = (order, res[big]["final_entropy"], res[small]["final_entropy"])
    assert out["fcfs"][0][0] == 1 and out["least-work"][0][0] == 2
    assert out["fcfs"][1:] == out["least-work"][1:]


def test_cancel_queued_and_resident_requests(pkg):
    """A queued request is dropped at once; a resident one is retired when its
    layer in flight finishes, freeing its memory for the next request; the
    other requests' results are untouched (failure handling on the host, no
    GPU fault involved)."""
    n, chi = 12, 32
    per = n * chi * chi * 2 * 8 + 8 * chi * (n + 1) + 4 * (n + 1)
    s = pkg.Server(int(per * 1.5) + 4096, max_slots=4, precision="mixed", max_chi=32, max_n=16)
    tr = pkg.Trunc.both(chi, 1e-10)
    a = s.submit(n, tr, 0.1, 8, 5, 0)   # resident first
    b = s.submit(n, tr, 0.1, 4, 5, 1)   # waits for memory
    c = s.submit(n, tr, 0.1, 4, 5, 2)   # waits, then cancelled while queued
    assert s.cancel(c)
    got = {d["id"]: d for d in s.poll()}
    assert got[c]["status"] == pkg.STATUS_CANCELLED and got[c]["layers"] == 0
    s.tick()
    s.tick()
    assert s.stats()["active"] == 1 and s.stats()["pending"] == 1
    assert s.cancel(a)                  # resident: retired after its current layer
    done = {}
    for _ in range(30):
        s.tick()
        done.update({d["id"]: d for d in s.poll()})
        if b in done:
            break
    assert done[a]["status"] == pkg.STATUS_CANCELLED and 0 < done[a]["layers"] < 8
    assert done[b]["status"] == 0 and done[b]["layers"] == 4
    assert not s.cancel(a) and not s.cancel(12345)
    assert s.stats()["arena_used"] == 0
    # b's result equals the same request run alone
    s2 = pkg.Server(1 << 30, max_slots=4, precision="mixed", max_chi=32, max_n=16)
    i = s2.submit(n, tr, 0.1, 4, 5, 1)
    res = []
    while not res:
        s2.tick()
        res = s2.poll()
    assert res[0]["id"] == i and res[0]["final_entropy"] == done[b]["final_entropy"]


def test_per_layer_entropy_history_matches_a_batch(pkg):
    """A served request's per-layer half-chain entropies (tn_server_history)
    equal the same trajectory stepped in a batch and end at its final
    entropy."""
    reqs = _req_params()[:3]
    s = pkg.Server(1 << 30, max_slots=4, precision="mixed", max_chi=32, max_n=16)
    ids = {s.submit(r["n"], pkg.Trunc.both(r["chi"], 1e-10), r["p"], r["depth"], 99, r["traj"]): r for r in reqs}
    got = {}
    for _ in range(200):
        s.tick()
        for d in s.poll(history=True):
            got[d["id"]] = d
        if len(got) == len(reqs):
            break
    for i, r in ids.items():
        h = got[i]["entropies"]
        assert len(h) == r["depth"] and h[-1] == got[i]["final_entropy"]
        b = pkg.Batch([r["n"]], [pkg.Trunc.both(r["chi"], 1e-10)], "mixed")
        want = [b.step([0], [pkg.gen_layer(99, r["traj"], t, r["n"], r["p"])])[1][0] for t in range(r["depth"])]
        np.testing.assert_allclose(h, want, rtol=0, atol=1e-6)
        assert s.history(i) is None  # fetched once
