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


def _run(pkg, reqs, slots, hbm, stagger):
    s = pkg.Server(hbm, max_slots=slots, precision="mixed", max_chi=32, max_n=16)
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
