"""Host logic of bench.py, on the CPU: the reference arm's summary (layers past
the time budget counted at the last measured layer's time), the censored
latency percentiles of the serving windows, the bond-operation list of one
apply_bilayer (mps.rs:2206-2252), and that the reference arm's worker runs
the oracle without loading any library of the product."""
import importlib.util
import json
import pathlib
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b


def test_summarize_reference_counts_unmeasured_layers_at_the_last_layer_time():
    b = _bench()
    res = [{"traj": 0, "p": 0.05, "prep_s": 1.0, "layer_s": [1.0, 2.0], "mid_bond_dim": 8},
           {"traj": 1, "p": 0.1, "prep_s": 1.0, "layer_s": [0.5, 0.5, 0.5, 0.5], "mid_bond_dim": 4}]
    out = b.summarize_reference(res, t_first=9, budget=3.0, layers=4)
    # T_0 = 1 + 2 + 2 x 2 = 7 s, T_1 = 2 s: 2 cores x 4 layers / mean(7, 2)
    assert out["value"] == pytest.approx(2 * 4 / 4.5)
    assert out["cores"] == 2 and out["kind"] == "port" and out["unit"] == "traj-layers/s"
    assert [p["estimated_s_for_all_layers"] for p in out["per_process"]] == [7.0, 2.0]
    assert out["seconds_per_traj_layer_per_core"] == pytest.approx((7.0 / 4 + 2.0 / 4) / 2)


def test_censored_percentiles():
    b = _bench()
    vals = [(3.0, True), (1.0, False), (4.0, True), (2.0, False)]
    assert b._censored_pct(vals, 50) == (2.0, False)
    assert b._censored_pct(vals, 99) == (4.0, True)
    assert b._censored_pct([], 50) == (None, False)


def test_layer_ops_follow_apply_meas_prob_layer():
    b = _bench()
    n = 6
    ops = b.layer_ops(n, [0, 2, 4], [3, 1, 3])
    gates = [(0, True), (2, True), (4, True)]
    # measured sites sorted and deduplicated (1, 3): refactors between them and on
    # to n - 2, then the full backward sweep n - 3 .. 0 (mps.rs:2221-2250)
    forward = [(1, False), (2, False), (3, False), (4, False)]
    backward = [(k, False) for k in range(n - 3, -1, -1)]
    assert ops == gates + forward + backward
    assert b.layer_ops(n, [1, 3], []) == [(1, True), (3, True)]


def test_reference_worker_loads_no_product_library():
    code = "\n".join([
        "import importlib.util, json, sys",
        f"spec = importlib.util.spec_from_file_location('b', {str(ROOT / 'bench.py')!r})",
        "b = importlib.util.module_from_spec(spec); spec.loader.exec_module(b)",
        "job = b.reference_jobs(8, 8, 1e-10, 3, 2, 0.0, 2, 2)[1]",
        "r = b._ref_traj_worker(job)",
        "maps = open('/proc/self/maps').read()",
        "mods = sorted(m for m in sys.modules if 'tensor_net' in m or m.split('.')[0] in ('torch', '__graft_entry__'))",
        "print(json.dumps({'layers': len(r['layer_s']), 'traj': r['traj'], 'p': r['p'],",
        "                  'lib': 'libtnmps' in maps, 'mods': mods}))",
    ])
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=str(ROOT))
    assert out.returncode == 0, out.stderr
    d = json.loads(out.stdout.strip().splitlines()[-1])
    # trajectory 1 of the batch (p = 0.10), one whole timed layer (a zero budget
    # still runs one), with neither libtnmps nor the package nor torch loaded
    assert d == {"layers": 1, "traj": 1, "p": 0.1, "lib": False, "mods": []}
