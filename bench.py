"""Benchmark of the GB300 MPS trajectory engine: trajectory-layers per second.

Workload (one "step" = one brickwork layer of every trajectory in the batch):
N=64 qubits, chi_max=256, singular-value cutoff 1e-10, Haar-random U(4)
gates, each qubit Z-measured with probability p (p cycles over
0.05/0.10/0.15/0.20/0.30 across trajectories), half-chain entropy read after
each layer; seeded synthetic inputs (counter-based generator, identical arrays
for every implementation).  The batch first evolves `--prefill` layers
untimed from |0...0> so that the timed layers run in the entangled regime.

Lines printed (rank 0): one JSON object per run.
  value     traj-layers/s from the device time of each timed layer between
            its input copy and its output copy (CUDA events on the batch
            stream around the layer's kernels: inputs resident in HBM), max
            over ranks;
  e2e       the same timed layers (the same calls) timed on the host: each
            layer through the C ABI (tn_batch_step) with host buffers, the
            pinned H2D of its inputs and the D2H of its outcomes,
            probabilities and entropies inside the timed region;
  roofline  algorithmic flops (theta GEMM + Golub-Reinsch SVD count of every
            bond operation, counted on the device) per launch / launch time;
  cpu_baseline  the FP64 oracle (numpy + LAPACK gesvd) on the host cores on a
            bounded sample of the same layers.
`--impl reference` runs only the CPU oracle arm (the reference itself is Rust
and cannot be built on these machines) and prints its line with
"impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import math
import os
import pathlib
import statistics
import subprocess
import sys
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

P_LIST = (0.05, 0.10, 0.15, 0.20, 0.30)
METRIC = "traj-layers/s & p50/p99 latency: served vs plain GPU at entropy err ≤1e-6"
UNIT = "traj-layers/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=304, help="trajectories per GPU")
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--chi", type=int, default=256)
    ap.add_argument("--cutoff", type=float, default=1e-10)
    ap.add_argument("--prefill", type=int, default=4)
    ap.add_argument("--prec", default="df", choices=["df", "mixed", "f64"])
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--cpu-seconds", type=float, default=60.0)
    ap.add_argument("--schedule", type=int, default=1, choices=[0, 1])
    ap.add_argument("--scheme", type=int, default=None, choices=[0, 1, 2, 3],
                    help="Jacobi block scheme (default: the library's)")
    ap.add_argument("--runs", type=int, default=64, help="coev: sampled trajectories")
    ap.add_argument("--workload", default="batch", choices=["batch", "mixed", "large", "precision", "coev", "plain",
                                                                 "f64", "vsplain"],
                    help="batch: the headline line; mixed: the batching workload; large: n=128, chi_max=1024; "
                         "precision: mixed vs float64 errors per p (uses --n, --chi, --depth); vsplain: batched vs "
                         "plain on layer --prefill + 1 in --prec")
    ap.add_argument("--depth", type=int, default=64)
    ap.add_argument("--theta", default="tc", choices=["tc", "simt"],
                    help="mixed precision theta contraction: tensor cores (tcgen05) or SIMT FP32")
    ap.add_argument("--large-seconds", type=float, default=300.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--plain-layers", type=int, default=1, help="timed layers of each plain trajectory")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-policy", default="least-work", choices=["fcfs", "least-work"])
    ap.add_argument("--serve-active-per-cta", type=int, default=2,
                    help="resident requests per class = this x the class's CTAs (0 = every slot)")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-sustained-rate", type=float, default=1.0)
    ap.add_argument("--serve-sustained-seconds", type=float, default=30.0)
    ap.add_argument("--serve-hbm-gb", type=int, default=96)
    ap.add_argument("--serve-slots", type=int, default=1024)
    return ap.parse_args()


# ------------------------------------------------------------------ helpers
def p_of(traj: int) -> float:
    return P_LIST[traj % len(P_LIST)]


def saturated_dims(n: int, chi: int):
    """Bond dimensions of a saturated chain: chi_b = min(chi, 2^min(b+1, n-1-b))."""
    return [min(chi, 2 ** min(b + 1, n - 1 - b)) if min(b + 1, n - 1 - b) < 30 else chi for b in range(n - 1)]


def op_flops(cl, cm, cr, gate):
    """Algorithmic flops of one bond operation (theta GEMM + SVD count)."""
    a, b = max(2 * cl, 2 * cr), min(2 * cl, 2 * cr)
    return 8.0 * (2 * cl) * cm * (2 * cr) + (128.0 * cl * cr if gate else 0.0) + \
        4.0 * (4 * a * a * b + 8 * a * b * b + 9 * b ** 3)


def layer_ops(n, gate_ks, meas_ks):
    """The bond-operation list of one apply_bilayer (mps.rs:2206-2252)."""
    ops = [(int(k), True) for k in gate_ks]
    ms = sorted(set(int(k) for k in meas_ks))
    if ms:
        last = None
        for k in ms:
            if last is not None:
                ops += [(b, False) for b in range(last, k)]
            last = k
        ops += [(b, False) for b in range(last, n - 1)]
        ops += [(b, False) for b in range(n - 3, -1, -1)]
    return ops


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = pathlib.Path(os.environ.get("TMPDIR", "/tmp")) / f"tn_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        try:
            self.path.unlink()
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return d, "measured"
        except Exception:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def ncu_traffic(prec):
    """DRAM traffic of the executor kernel per algorithmic flop, from the
    committed ncu summary of its launches (profiles/k_run_traffic_<prec>.json)."""
    p = ROOT / "profiles" / f"k_run_traffic_{prec}.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        d.setdefault("source", f"profiles/{p.name}: DRAM bytes per algorithmic flop of the captured launches "
                               f"(ncu), times this launch's algorithmic flops")
        return d
    except Exception:
        return None


# ----------------------------------------------------------- CPU (oracle)
def _ref_traj_worker(args):
    """One trajectory of the benchmark workload with the FP64 oracle on one
    core: the untimed layers [0, t_first) from |0...0>, then the timed
    layers t_first, t_first + 1, ... (each apply_bilayer plus its half-chain
    entropy read), whole layers, until `budget` seconds have passed or
    `layers` layers are done (at least one).  Inputs come from
    oracle.gen_ref, the GPU arm's generator restated in Python, so this arm
    loads no library of the product."""
    root, n, chi, cutoff, seed, traj, p, t_first, budget, layers = args
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    if root not in sys.path:
        sys.path.insert(0, root)
    from oracle import gen_ref as G
    from oracle import mps_ref as R
    m = R.MPS(n, R.Trunc.both(chi, cutoff))
    t0 = time.perf_counter()
    for t in range(t_first):
        R.apply_bilayer(m, *G.gen_layer(seed, traj, t, n, p))
    prep = time.perf_counter() - t0
    times, t = [], t_first
    start = time.perf_counter()
    while True:
        lay = G.gen_layer(seed, traj, t, n, p)
        a0 = time.perf_counter()
        R.apply_bilayer(m, *lay)
        m.entropy_vn(n // 2 - 1)
        times.append(time.perf_counter() - a0)
        t += 1
        if time.perf_counter() - start >= budget or len(times) >= layers:
            break
    return {"traj": traj, "p": p, "prep_s": prep, "layer_s": times,
            "mid_bond_dim": int(len(m.svals[n // 2 - 1]))}


def reference_jobs(n, chi, cutoff, seed, t_first, budget, cores, layers):
    return [(str(ROOT), n, chi, cutoff, seed, i, p_of(i), t_first, budget, layers) for i in range(cores)]


def summarize_reference(res, t_first, budget, layers):
    """CPU throughput on the GPU arm's workload: every trajectory must run
    the same `layers` layers from t_first, so the job takes the mean over
    trajectories of that time per core: throughput = cores * layers / mean
    T_i.  T_i = the measured whole layers plus, for layers beyond the time
    budget, the last measured layer's time each (bond dimensions only grow
    over these layers, so this underestimates the CPU's time: the CPU
    number is an upper bound)."""
    cores = len(res)
    est = []
    for r in res:
        ls = r["layer_s"]
        est.append(sum(ls) + max(0, layers - len(ls)) * ls[-1])
    rate = cores * layers / statistics.mean(est)
    measured = sum(len(r["layer_s"]) for r in res)
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"FP64 oracle (numpy + LAPACK gesvd, 1 BLAS thread per process) on {cores} processes; "
                       f"process i runs trajectory i of the GPU batch (p cycling {list(P_LIST)}) from |0...0> "
                       f"through layers [0, {t_first}) untimed, then times whole layers of [{t_first}, "
                       f"{t_first + layers}) for up to {budget:.0f} s ({measured} traj-layers measured, at least one "
                       f"per process); the layers beyond the budget are counted at the last measured layer's "
                       f"time (an underestimate of the CPU's time); throughput = cores x {layers} / mean time "
                       f"per trajectory"),
            "seconds_per_traj_layer_per_core": statistics.mean(e / layers for e in est),
            "per_process": [{"traj": r["traj"], "p": r["p"], "layers_measured": len(r["layer_s"]),
                             "layer_s": r["layer_s"], "estimated_s_for_all_layers": e, "prep_s": r["prep_s"],
                             "mid_bond_dim": r["mid_bond_dim"]} for r, e in zip(res, est)]}


def reference_arm(n, chi, cutoff, seed, t_first, budget, cores, layers):
    """The CPU arm on the same workload as the GPU arm: `cores` spawned
    processes (one BLAS thread each, the reference's rayon-over-trajectories
    pattern), process i running batch trajectory i (p cycling) from |0...0>
    to the GPU arm's first timed layer untimed, then timing whole layers of
    the GPU arm's timed range."""
    import multiprocessing as mp
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_ref_traj_worker, reference_jobs(n, chi, cutoff, seed, t_first, budget, cores, layers))
    return summarize_reference(res, t_first, budget, layers)


# --------------------------------------------------------------- GPU arm
def max_over_ranks(x: float, device=None) -> float:
    """The largest of every rank's value (the timed interval of the slowest
    rank); the value itself on a single process."""
    import torch
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, steps: int, world: int, elapsed_max: float) -> float:
    """Whole-job throughput: every rank's units over the slowest rank's time
    (weak scaling: each rank owns its own trajectories)."""
    return world * units_per_rank * steps / elapsed_max


# per-phase SM cycles of the bond operations, counted on the device (one CTA each)
CYC_KEYS = ("cyc_theta", "cyc_gram", "cyc_rot", "cyc_update", "cyc_final")

# Measured half-chain entropy error of each precision mode against the FP64
# oracle on identical inputs (tests/test_gpu_precision.py: N=32, chi_max=64,
# cutoff 1e-10, depth 64, one trajectory per p in P_LIST).
FP64_NOMINAL_TFLOPS = 1.25

PRECISION_NOTE = {
    "df": ("max 6.7e-11 over p in {0.05..0.30} at N=32 chi_max=64 depth 64 and 3.5e-12 at N=64 chi_max=256 "
           "depth 16 (profiles/precision_*.json); tests/test_gpu_precision.py asserts < 1e-6 per p"),
    "f64": "below 1e-12 (tests/test_gpu_parity.py, tests/test_gpu_workloads.py)",
    "mixed": "1e-5 .. 2e-3 over p in {0.05..0.30} (does not meet the 1e-6 bound)",
}


def run_gpu(a, rank, world, local_rank):
    """The GPU arm.  Every layer goes through the library's public C ABI with
    host buffers (tn_batch_step: one pinned H2D of the layer's gates and
    uniforms, the layer's kernels, one D2H of outcomes, probabilities and
    entropies).  Of the same K timed layers, `value` counts the device time
    between each layer's input copy and output copy (CUDA events on the batch
    stream: every kernel of the layer with its inputs resident in HBM) and
    `e2e` the host wall time of the whole calls, copies included."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    torch.cuda.set_device(local_rank)
    lib = pkg.lib()
    import ctypes
    name = ctypes.create_string_buffer(128)
    sms = ctypes.c_uint32()
    pkg._lib.check(lib.tn_device_info(name, 128, ctypes.byref(sms)), "tn_device_info")
    B = a.batch
    n, chi = a.n, a.chi
    trunc = pkg.Trunc.both(chi, a.cutoff)
    batch = pkg.Batch([n] * B, [trunc] * B, a.prec)
    batch.set_schedule(a.schedule)
    batch.set_theta_path(a.theta == "simt")
    if a.scheme is not None:
        batch.set_tuning(a.scheme, 40)
    traj0 = rank * B

    def layer_inputs(t):
        return [pkg.gen_layer(a.seed, traj0 + i, t, n, p_of(traj0 + i)) for i in range(B)]

    trajs = list(range(B))
    t_first = a.prefill + a.warmup
    untimed_ms = []
    for t in range(t_first):  # prefill and warm-up layers (untimed)
        t0 = time.perf_counter()
        batch.step(trajs, layer_inputs(t))
        untimed_ms.append(1e3 * (time.perf_counter() - t0))
    # the plain path starts from the same states (checkpoint export / import)
    plain_states = []
    if rank == 0 and world == 1 and not a.no_plain:
        for i in range(min(len(P_LIST), B)):
            plain_states.append(batch.export_parts(i))
    packs = [batch.pack(trajs, layer_inputs(t)) for t in range(t_first, t_first + a.steps)]
    batch.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    batch.stats(reset=True)
    clocks = ClockSampler(local_rank)
    clocks.start()
    dev_ms, host_s, split = [], [], []
    t_all = time.perf_counter()
    for pk in packs:
        t0 = time.perf_counter()
        batch.step_packed(pk)  # returns with the layer's outputs in host memory
        host_s.append(time.perf_counter() - t0)
        dev_ms.append(batch.last_step_device_ms())
        split.append(batch.last_launch_ms())
    batch.synchronize()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t_all
    clk = clocks.stop()
    elapsed = sum(dev_ms) / 1e3
    st = batch.stats(reset=True)
    status = batch.device_status()
    elapsed = max_over_ranks(elapsed, torch.device("cuda", local_rank))
    e2e_s = max_over_ranks(e2e_s, torch.device("cuda", local_rank))
    h2d = statistics.mean(int(pk["gates"].nbytes + pk["us"].nbytes + 4 * (pk["gate_ks"].size + pk["meas_ks"].size +
                                                                         2 * B + 2 * (B + 1))) for pk in packs)
    d2h = statistics.mean(int(int(pk["meas_off"][-1]) * (4 + 8) + 8 * B) for pk in packs)
    dims = [batch.bond_dims(i) for i in range(min(B, 5))]
    batch.close()
    return dict(value=whole_job_rate(B, a.steps, world, elapsed), elapsed=elapsed, step_ms=dev_ms,
                host_step_s=host_s, split=split, untimed_ms=untimed_ms, stats=st, status=status, clocks=clk,
                e2e=whole_job_rate(B, a.steps, world, e2e_s), h2d=h2d, d2h=d2h, B=B, gpu=name.value.decode(),
                dims=dims, sms=int(sms.value), plain_states=plain_states)


def run_plain(a, pkg, states):
    """The plain path: one trajectory at a time through the single-state API
    (tn_mps_apply_bilayer + entropy read, host-timed), on batch trajectories
    0..4 (one per p) from the states they had at the first timed layer
    (exported from the batch and imported into single-state handles), over
    `--plain-layers` of the timed layers."""
    t_lo = a.prefill + a.warmup
    nl = min(a.plain_layers, a.steps)
    total, layers = 0.0, 0
    for i, (gammas, lams) in enumerate(states):
        m = pkg.MPS.from_parts(gammas, lams, pkg.Trunc.both(a.chi, a.cutoff), a.prec, a.chi)
        m.entropy_vn(a.n // 2 - 1)
        for t in range(t_lo, t_lo + nl):
            inp = pkg.gen_layer(a.seed, i, t, a.n, p_of(i))
            t0 = time.perf_counter()
            m.apply_bilayer(*inp)
            m.entropy_vn(a.n // 2 - 1)  # the layer's entropy read (synchronises)
            total += time.perf_counter() - t0
            layers += 1
        m.close()
    return {"value": layers / total, "unit": UNIT,
            "how": f"single-state API (one trajectory at a time), {layers} traj-layers: trajectories "
                   f"0..{len(states) - 1} (one per p) from their batch states at layer {t_lo}, layers "
                   f"[{t_lo}, {t_lo + nl}), host-timed"}


def _censored_pct(values, q):
    """q-th percentile of latencies where some are lower bounds (requests still
    queued or running when the window closed): (value, censored)."""
    if not values:
        return None, False
    v = sorted(values, key=lambda x: x[0])
    x, cens = v[min(len(v) - 1, int(math.ceil(q / 100.0 * len(v))) - 1)]
    return float(x), bool(cens)


def _serve_window(pkg, a, reqs, duration, drain, max_chi, max_n, policy_caps=True):
    srv = pkg.Server(int(a.serve_hbm_gb) << 30, max_slots=a.serve_slots, precision=a.prec, max_chi=max_chi,
                     max_n=max_n)
    c0, c1 = srv.class_stats(0), srv.class_stats(1)
    caps = (a.serve_active_per_cta * c0["ctas"], a.serve_active_per_cta * c1["ctas"]) \
        if (a.serve_active_per_cta and policy_caps) else (0, 0)
    srv.set_policy(a.serve_policy, caps)
    t0 = srv.now()
    done, submitted = pkg.run_poisson(srv, reqs, duration, a.seed, drain=drain)
    wall = srv.now() - t0
    st = srv.stats()
    cls = [srv.class_stats(c) for c in (0, 1)]
    srv.close()
    by_id = {d["id"]: d for d in done}
    lat = []  # (latency or its lower bound, censored)
    for i, r in enumerate(reqs[:submitted]):
        d = by_id.get(i + 1)  # request ids are 1 + submission index
        lat.append((d["latency_s"], False) if d else (max(0.0, wall - r["t"]), True))

    def summary(idx):
        ls = [lat[i] for i in idx]
        p50, c50 = _censored_pct(ls, 50)
        p99, c99 = _censored_pct(ls, 99)
        fin = sorted(x for x, c in ls if not c)
        return {"submitted": len(ls), "completed": len(fin),
                "p50_latency_s": p50, "p50_censored": c50, "p99_latency_s": p99, "p99_censored": c99,
                "p50_latency_completed_s": fin[len(fin) // 2] if fin else None}
    out = {"wall_s": wall, "traj_layers_per_s": st["layers"] / wall if wall > 0 else None,
           "admitted": int(st["admitted"]), "active_at_end": int(st["active"]), "pending_at_end": int(st["pending"]),
           "all": summary(range(len(lat))), "max_active_per_class": list(caps), "classes": []}
    for c, cs in enumerate(cls):
        if cs["cap_max"] == 0:
            continue
        lo = cls[c - 1]["cap_max"] if c > 0 else 0
        idx = [i for i, r in enumerate(reqs[:submitted]) if lo < min(r["chi"], 1 << (r["n"] // 2)) <= cs["cap_max"]]
        out["classes"].append(dict(summary(idx), bond_cap_max=cs["cap_max"], ctas=cs["ctas"],
                                   traj_layers_per_s=cs["layers"] / wall if wall > 0 else None,
                                   launches=int(cs["launches"])))
    return out


def run_serving(a, pkg):
    """Two serving windows through the continuous-batching server:
    1. the serving workload as specified (Poisson arrivals at --serve-rate/s,
       n log-uniform in [16, 128], chi_max in {64..512}, p in [0.02, 0.3],
       depth in [2n, 4n]) for --serve-seconds: the offered load is far above
       one GPU's capacity, so most requests are still queued or running when
       the window closes; latency percentiles are over every submitted
       request, unfinished ones counted at their time in the system so far
       (a lower bound, flagged "censored");
    2. a load the server sustains: light requests (n in [16, 32], chi_max in
       {32, 64}) at --serve-sustained-rate/s for --serve-sustained-seconds,
       then drained, so every submitted request completes and the
       percentiles are exact."""
    heavy = pkg.poisson_requests(a.serve_rate, a.serve_seconds, a.seed)
    w1 = _serve_window(pkg, a, heavy, a.serve_seconds, False, 512, 128)
    w1.update(rate_per_s=a.serve_rate, window_s=a.serve_seconds,
              mix="n log-uniform [16, 128], chi_max {64, 128, 256, 512}, p U[0.02, 0.3], depth U[2n, 4n]")
    out = {"specified_load": w1}
    if a.serve_sustained_seconds > 0:
        light = pkg.poisson_requests(a.serve_sustained_rate, a.serve_sustained_seconds, a.seed + 1,
                                     n_range=(16, 32), chis=(32, 64))
        w2 = _serve_window(pkg, a, light, a.serve_sustained_seconds, True, 64, 32, policy_caps=False)
        w2.update(rate_per_s=a.serve_sustained_rate, window_s=a.serve_sustained_seconds, drained=True,
                  mix="n log-uniform [16, 32], chi_max {32, 64}, p U[0.02, 0.3], depth U[2n, 4n]")
        out["sustained_load"] = w2
    out["precision"] = a.prec
    return out


def _dev_view(torch, ptr, n, typestr):
    class V:
        __cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 2}
    return torch.as_tensor(V(), device="cuda")


def run_mixed(a):
    """The batching workload: `--batch` trajectories with n uniform in
    {16, 32, 48, 64}, chi_max uniform in {32, 64, 128, 256}, p uniform in
    [0.05, 0.3], per-trajectory seeds (depth 4n >= 64 layers, so every
    trajectory is live in the window); one graph-captured launch per layer
    (tn_batch_step_device) with the layer inputs copied device-to-device into
    the graph's input buffers; `--prefill` untimed layers, then W + K."""
    import numpy as np
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    rng = np.random.default_rng(a.seed)
    B = a.batch
    ns = rng.choice([16, 32, 48, 64], B)
    chis = rng.choice([32, 64, 128, 256], B)
    ps = rng.uniform(0.05, 0.3, B)
    batch = pkg.Batch([int(x) for x in ns], [pkg.Trunc.both(int(c), a.cutoff) for c in chis], a.prec)
    batch.set_schedule(a.schedule)
    trajs = list(range(B))

    def layer(t):
        return [pkg.gen_layer(a.seed, i, t, int(ns[i]), float(ps[i])) for i in trajs]
    assert a.prefill + a.warmup + a.steps <= 4 * 16, "every trajectory must still be live"
    for t in range(a.prefill):
        batch.step(trajs, layer(t))
    ptr = batch.device_inputs(int(sum(ns // 2)), int(sum(ns)))
    dev = torch.device("cuda")
    staged = []
    for t in range(a.prefill, a.prefill + a.warmup + a.steps):
        pk = batch.pack(trajs, layer(t))
        staged.append([(name, ts, torch.as_tensor(np.ascontiguousarray(pk[name].astype(dt)), device=dev))
                       for name, ts, dt in (("trajs", "<i4", np.int32), ("gate_off", "<i4", np.int32),
                                            ("gate_ks", "<i4", np.int32), ("gates", "<f8", np.float64),
                                            ("meas_off", "<i4", np.int32), ("meas_ks", "<i4", np.int32),
                                            ("us", "<f8", np.float64)) if pk[name].size])
    stream = torch.cuda.ExternalStream(batch.stream(), device=dev)
    views = {}

    def run(layer_arrays):
        for name, ts, src in layer_arrays:
            key = (name, src.numel())
            if key not in views:
                views[key] = _dev_view(torch, ptr[name], src.numel(), ts)
            views[key].copy_(src, non_blocking=True)
        batch.step_device(B)
    with torch.cuda.stream(stream):
        for L_ in staged[: a.warmup]:
            run(L_)
    batch.synchronize()
    batch.stats(reset=True)
    clocks = ClockSampler(0)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for L_ in staged[a.warmup:]:
            run(L_)
        ev1.record(stream)
    batch.synchronize()
    clk = clocks.stop()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    st = batch.stats(reset=True)
    status = batch.device_status()
    return {"workload": "batching: n in {16,32,48,64}, chi_max in {32,64,128,256}, p in U[0.05,0.3], "
                        "per-trajectory seeds, one graph-captured launch per layer",
            "trajectories": B, "value": B * a.steps / elapsed, "unit": UNIT, "ms_per_step": elapsed / a.steps * 1e3,
            "layers": [a.prefill + a.warmup, a.prefill + a.warmup + a.steps],
            "tflops_algorithmic": (st["flop_theta"] + st["flop_svd"]) / elapsed / 1e12,
            "bond_ops_per_step": st["bond_ops"] / a.steps, "device_status": status, "clocks": clk,
            "precision": a.prec}


def run_large(a):
    """The large single trajectory: n=128, chi_max=1024, p=0.05, cutoff 1e-10,
    layers from |0...0> until `--large-seconds` of wall time; entropy and
    wall time per layer (one trajectory of a batch, one launch per layer)."""
    import numpy as np
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    n, chi, p = 128, 1024, 0.05
    batch = pkg.Batch([n], [pkg.Trunc.both(chi, a.cutoff)], a.prec)
    batch.set_schedule(a.schedule)
    rows = []
    t_start = time.perf_counter()
    t = 0
    while time.perf_counter() - t_start < a.large_seconds and t < 256:
        inputs = [pkg.gen_layer(a.seed, 0, t, n, p)]
        batch.stats(reset=True)
        t0 = time.perf_counter()
        _, ent = batch.step([0], inputs)
        dt = time.perf_counter() - t0
        st = batch.stats(reset=True)
        dims = batch.bond_dims(0)
        rows.append({"layer": t, "s": dt, "entropy": float(ent[0]), "max_bond": int(dims.max()),
                     "tflops_algorithmic": (st["flop_theta"] + st["flop_svd"]) / dt / 1e12,
                     "bond_ops": int(st["bond_ops"])})
        t += 1
    torch.cuda.synchronize()
    return {"workload": f"single trajectory n={n} chi_max={chi} p={p} cutoff={a.cutoff:g} from |0...0>",
            "layers_run": t, "precision": a.prec, "per_layer": rows, "device_status": batch.device_status(),
            "unit": "s per layer"}


def run_plain_small(a):
    """The plain-method workload (N=16, depth 32, p=0.1, chi_max=64, cutoff
    1e-12): one trajectory through the single-state API in float64 on the
    GPU, and the FP64 oracle on one host core, on the same inputs; traj-layers
    per second for each and the largest entropy difference."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    sys.path.insert(0, str(ROOT))
    from oracle import mps_ref as R
    n, depth, p, chi, cut = 16, 32, 0.1, 64, 1e-12
    trajs = [pkg.gen_trajectory(a.seed, i, n, depth, p) for i in range(4)]
    m = pkg.MPS.new_qubits(n, pkg.Trunc.both(chi, cut), "f64")
    for L_ in trajs[0][:2]:
        m.apply_bilayer(*L_)  # warm-up (module load, first launches)
    m.close()
    g_ents, t0 = [], time.perf_counter()
    for tr in trajs:
        m = pkg.MPS.new_qubits(n, pkg.Trunc.both(chi, cut), "f64")
        e = []
        for L_ in tr:
            m.apply_bilayer(*L_)
            e.append(m.entropy_vn(n // 2 - 1))
        g_ents.append(e)
        m.close()
    g_s = time.perf_counter() - t0
    c_ents, t0 = [], time.perf_counter()
    for tr in trajs:
        r = R.MPS(n, R.Trunc.both(chi, cut))
        e = []
        for L_ in tr:
            R.apply_bilayer(r, *L_)
            e.append(r.entropy_vn(n // 2 - 1))
        c_ents.append(e)
    c_s = time.perf_counter() - t0
    err = max(abs(x - y) for ge_, ce in zip(g_ents, c_ents) for x, y in zip(ge_, ce))
    units = len(trajs) * depth
    return {"workload": f"plain method: N={n} depth={depth} p={p} chi_max={chi} cutoff={cut:g}, "
                        f"{len(trajs)} trajectories one at a time",
            "gpu_plain_f64": {"value": units / g_s, "unit": UNIT},
            "cpu_oracle_1core": {"value": units / c_s, "unit": UNIT},
            "entropy_abs_max_vs_oracle": err}


def run_f64(a):
    """The headline workload (N=64, chi_max=256, p cycling) in float64 -- the
    mode that meets the 1e-6 entropy bound (errors ~1e-14 against the oracle)
    -- batched vs plain on one timed layer: `--batch` trajectories after
    `--prefill` layers (one warm-up layer), and one trajectory (p=0.10)
    through the single-state API on the same layer."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    n, chi, B = a.n, a.chi, a.batch
    trunc = pkg.Trunc.both(chi, a.cutoff)
    batch = pkg.Batch([n] * B, [trunc] * B, "f64")
    trajs = list(range(B))
    lay = lambda t: [pkg.gen_layer(a.seed, i, t, n, p_of(i)) for i in trajs]
    for t in range(a.prefill + 1):
        batch.step(trajs, lay(t))
    batch.synchronize()
    t_lo = a.prefill + 1
    pk = batch.pack(trajs, lay(t_lo))
    t0 = time.perf_counter()
    batch.step_packed(pk)
    b_s = time.perf_counter() - t0
    st = batch.stats(reset=True)
    batch.close()
    m = pkg.MPS.new_qubits(n, trunc, "f64")
    for t in range(t_lo):
        m.apply_bilayer(*pkg.gen_layer(a.seed, 1, t, n, p_of(1)))
    t0 = time.perf_counter()
    m.apply_bilayer(*pkg.gen_layer(a.seed, 1, t_lo, n, p_of(1)))
    m.entropy_vn(n // 2 - 1)
    p_s = time.perf_counter() - t0
    m.close()
    return {"workload": f"N={n} chi_max={chi} float64, {B} trajectories, layer {t_lo} after {a.prefill + 1}",
            "batched_f64": {"value": B / b_s, "unit": UNIT, "layer_s": b_s},
            "plain_f64_p0.10": {"value": 1.0 / p_s, "unit": UNIT, "layer_s": p_s},
            "batched_over_plain": (B / b_s) * p_s,
            "note": "host-timed, inputs through tn_batch_step (e2e); plain = one p=0.10 trajectory"}


def run_vs_plain(a):
    """Batched vs plain on one layer of the headline workload (N=64,
    chi_max=256, p cycling) in `--prec`: `--batch` trajectories step through
    layers [0, --prefill] (the last one as warm-up), then layer --prefill + 1
    is timed through tn_batch_step with host buffers.  Trajectories 0..4 (one
    per p) continue from the states they had in the batch before that layer
    (checkpoint export / import) through the single-state API, one traj-layer
    each with its entropy read, host-timed: both sides run the same layer of
    the same trajectories."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    n, chi, B = a.n, a.chi, a.batch
    trunc = pkg.Trunc.both(chi, a.cutoff)
    batch = pkg.Batch([n] * B, [trunc] * B, a.prec)
    trajs = list(range(B))

    def lay(t):
        return [pkg.gen_layer(a.seed, i, t, n, p_of(i)) for i in trajs]

    for t in range(a.prefill + 1):
        batch.step(trajs, lay(t))
    t_lo = a.prefill + 1
    states = [batch.export_parts(i) for i in range(min(len(P_LIST), B))]
    pk = batch.pack(trajs, lay(t_lo))
    batch.synchronize()
    t0 = time.perf_counter()
    batch.step_packed(pk)
    b_s = time.perf_counter() - t0
    status = batch.device_status()
    dims = [int(batch.bond_dims(i)[n // 2 - 1]) for i in range(len(states))]
    batch.close()
    plain_s = []
    for i, (gammas, lams) in enumerate(states):
        m = pkg.MPS.from_parts(gammas, lams, trunc, a.prec, chi)
        m.entropy_vn(n // 2 - 1)
        inp = pkg.gen_layer(a.seed, i, t_lo, n, p_of(i))
        t0 = time.perf_counter()
        m.apply_bilayer(*inp)
        m.entropy_vn(n // 2 - 1)  # the layer's entropy read (synchronises)
        plain_s.append(time.perf_counter() - t0)
        m.close()
    batched = B / b_s
    plain = len(plain_s) / sum(plain_s)
    return {"workload": f"N={n} chi_max={chi} cutoff={a.cutoff:g} {a.prec}, {B} trajectories (p cycling "
                        f"{list(P_LIST)}), layer {t_lo} after {t_lo} untimed layers",
            "batched": {"value": batched, "unit": UNIT, "layer_s": b_s, "device_status": status},
            "plain": {"value": plain, "unit": UNIT, "traj_layer_s": dict(zip([str(p_of(i)) for i in range(len(plain_s))],
                                                                             plain_s)),
                      "how": "trajectories 0..4 (one per p) from their batch states, single-state API"},
            "middle_bond_dims_after": dims,
            "batched_over_plain": batched / plain,
            "note": "host-timed on both sides (batched: tn_batch_step with pinned H2D and D2H)"}


def run_coev(a):
    """The multi-chi coevolution replay (the reference's production driver,
    workspace/src/haar_coev_probs.rs): `--runs` sampled trajectories of one
    circuit without truncation, each replayed at the reference's 15 chi_max
    values with post-selected outcomes; n = --n, depth = --depth, p = 0.1."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    t0 = time.perf_counter()
    out = pkg.run_coevolution(a.n, a.depth, 0.1, a.runs, a.seed, precision=a.prec)
    wall = time.perf_counter() - t0
    trajs = a.runs * len(pkg.REFERENCE_BONDS)
    return {"workload": f"coevolution replay: n={a.n} depth={a.depth} p=0.1, {a.runs} runs x "
                        f"{len(pkg.REFERENCE_BONDS)} chi_max (4..72 and untruncated), host-driven layer steps",
            "trajectories": trajs, "value": trajs * a.depth / wall, "unit": UNIT, "wall_s": wall,
            "measurements_per_run": int(out["sites"].shape[0]), "device_status": list(out["device_status"]),
            "precision": a.prec}


def run_precision(a):
    """Errors of the mixed path against the float64 GPU path (itself held to
    the FP64 oracle by the parity tests) on identical inputs: per p of the
    precision workload's set, the largest half-chain entropy difference over
    the layers, the largest probability difference, and the largest relative
    Schmidt-value difference (values above 1e-4) at the last layer; compared
    up to the first layer whose outcome records differ (|p - u| ties)."""
    import numpy as np
    import __graft_entry__ as ge
    pkg = ge.load_package()
    n, chi, depth, reps = a.n, a.chi, a.depth, 2
    specs = [(p, r) for p in P_LIST for r in range(reps)]
    trajs = [pkg.gen_trajectory(a.seed, 1000 * r + int(p * 100), n, depth, p) for p, r in specs]
    out = {}
    runs = {}
    t0 = time.perf_counter()
    for prec in ("f64", "mixed"):
        b = pkg.Batch([n] * len(trajs), [pkg.Trunc.both(chi, a.cutoff)] * len(trajs), prec)
        b.set_theta_path(a.theta == "simt")
        ents, recs = [[] for _ in trajs], [[] for _ in trajs]
        for t in range(depth):
            r, e = b.step(list(range(len(trajs))), [tl[t] for tl in trajs])
            for i in range(len(trajs)):
                ents[i].append(float(e[i]))
                recs[i].append(r[i])
        sv = [[b.svals(i, bd) for bd in range(n - 1)] for i in range(len(trajs))]
        runs[prec] = (ents, recs, sv, b.device_status())
    for i, (p, r) in enumerate(specs):
        e64, r64, s64 = runs["f64"][0][i], runs["f64"][1][i], runs["f64"][2][i]
        e32, r32, s32 = runs["mixed"][0][i], runs["mixed"][1][i], runs["mixed"][2][i]
        last = depth
        for t in range(depth):
            if [x[:2] for x in r64[t]] != [x[:2] for x in r32[t]]:
                last = t
                break
        e_ent = max([abs(e64[t] - e32[t]) for t in range(last)] or [0.0])
        e_p = max([abs(x[2] - y[2]) for t in range(last) for x, y in zip(r64[t], r32[t])] or [0.0])
        e_s = None
        if last == depth:
            e_s = 0.0
            for x, y in zip(s64, s32):
                x, y = np.asarray(x), np.asarray(y)
                k = min(len(x), len(y))
                sel = x[:k] > 1e-4
                if sel.any():
                    e_s = max(e_s, float(np.max(np.abs(x[:k][sel] - y[:k][sel]) / x[:k][sel])))
        key = f"p={p}"
        prev = out.get(key)
        cur = dict(entropy_abs=e_ent, prob_abs=e_p, schmidt_rel=e_s, layers_compared=last)
        if prev is None:
            out[key] = cur
        else:
            out[key] = dict(entropy_abs=max(prev["entropy_abs"], e_ent), prob_abs=max(prev["prob_abs"], e_p),
                            schmidt_rel=None if e_s is None or prev["schmidt_rel"] is None
                            else max(prev["schmidt_rel"], e_s),
                            layers_compared=min(prev["layers_compared"], last))
    growth = {}
    for p in P_LIST:
        idx = [i for i, (pp, r) in enumerate(specs) if pp == p]
        growth[f"p={p}"] = [max(abs(runs["f64"][0][i][t] - runs["mixed"][0][i][t]) for i in idx)
                            for t in range(0, depth, max(1, depth // 16))]
    return {"entropy_abs_every_few_layers": growth,
            "workload": f"precision: N={n} chi_max={chi} cutoff={a.cutoff:g} depth {depth}, p in {list(P_LIST)}, "
                        f"{reps} trajectories per p; mixed vs float64 GPU path on identical inputs",
            "theta_path": a.theta,
            "errors": out, "device_status": {k: v[3] for k, v in runs.items()},
            "wall_s": time.perf_counter() - t0}


def main():
    a = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    t_first = a.prefill + a.warmup
    config = {"workload": f"N={a.n} chi_max={a.chi} cutoff={a.cutoff:g} Haar brickwork from |0...0>, p cycling "
                          f"{list(P_LIST)} over the trajectories, timed layers [{t_first}, {t_first + a.steps}) "
                          f"after {a.prefill} untimed and {a.warmup} warm-up layers",
              "n_qubits": a.n, "chi_max": a.chi, "cutoff": a.cutoff, "p_cycle": list(P_LIST),
              "first_timed_layer": t_first, "timed_layers": a.steps, "seed": a.seed,
              "l2": "state larger than L2 (no flush needed)"}

    if a.impl == "reference":
        if rank != 0:
            return
        cores = len(os.sched_getaffinity(0))
        cb = reference_arm(a.n, a.chi, a.cutoff, a.seed, t_first, a.cpu_seconds, cores, a.steps)
        v = cb["value"]
        out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus,
               "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * cb["seconds_per_traj_layer_per_core"],
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
               "data": "synthetic (seeded Haar gates and measurement uniforms)", "config": config,
               "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
               "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
               "per_process": cb["per_process"],
               "note": "the reference is Rust (tensor-net) and no Rust toolchain exists on these machines, so the "
                       "reference arm is its FP64 restatement (oracle/mps_ref.py, LAPACK gesvd as the reference's "
                       "ndarray-linalg svd_into) on the host cores; ms_per_step = mean seconds per traj-layer of "
                       "one core over the timed layers"}
        print(json.dumps(out), flush=True)
        return

    if a.workload in ("mixed", "large", "precision", "coev", "plain", "f64", "vsplain"):
        if rank != 0:
            return
        import torch
        torch.cuda.set_device(0)
        out = {"mixed": run_mixed, "large": run_large, "precision": run_precision, "coev": run_coev,
               "plain": run_plain_small, "f64": run_f64, "vsplain": run_vs_plain}[a.workload](a)
        out.update({"metric": METRIC if a.workload == "mixed" else "per-layer time and entropy",
                    "n_gpus": 1, "data": "synthetic (seeded Haar gates and measurement uniforms)"})
        print(json.dumps(out), flush=True)
        return

    cpu_pool = cpu_async = None
    if rank == 0 and world == 1 and not a.no_cpu:
        # The CPU baseline runs on the host cores while the GPU works (the GPU
        # arm's host thread only issues and waits; two cores are left to it and
        # to the clock sampler): spawned processes, started before any GPU call.
        import multiprocessing as mp
        cores = max(1, len(os.sched_getaffinity(0)) - 2)
        os.environ["OPENBLAS_NUM_THREADS"] = "1"
        cpu_pool = mp.get_context("spawn").Pool(cores)
        cpu_async = cpu_pool.map_async(_ref_traj_worker,
                                       reference_jobs(a.n, a.chi, a.cutoff, a.seed, t_first, a.cpu_seconds, cores,
                                                      a.steps))

    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    r = run_gpu(a, rank, world, local_rank)
    peaks, peaks_kind = measured_peaks()
    flops = r["stats"]["flop_theta"] + r["stats"]["flop_svd"]
    launch_ms = [x[0] + x[1] for x in r["split"] if x]
    launch_s = sum(launch_ms) / 1e3 / max(1, len(launch_ms))
    per_launch = flops / a.steps
    achieved = per_launch / launch_s / 1e12
    peak = float(peaks.get("bf16_tflops_sustained") or peaks.get("bf16_tflops"))
    sm_mhz = r["clocks"].get("sm_mhz") or 2070.0
    cyc_sum = sum(r["stats"][k] for k in CYC_KEYS)
    simt_peak = r["sms"] * 128 * 2 * sm_mhz * 1e6 / 1e12
    alg_bytes = r["stats"]["bytes"] / a.steps
    tr = ncu_traffic(a.prec)
    dtype = {"mixed": "c64+f64", "f64": "c128", "df": "df64 (float32 pairs) + f64"}[a.prec]
    out = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": r["elapsed"] / a.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype,
        "data": "synthetic (seeded Haar gates and measurement uniforms)",
        "config": config,
        "precision": {"mode": a.prec, "entropy_err_vs_fp64_oracle": PRECISION_NOTE.get(a.prec)},
        "e2e": {"value": r["e2e"], "unit": UNIT, "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"],
                "how": "the same K layers as value, host wall time of tn_batch_step (pinned H2D + kernels + D2H)"},
        # per timed step: k_lpt_order, k_gate_slots, k_compile_dd, k_run (schedule 1; the launch list in
        # profiles/), or k_lpt_order, k_compile and two k_run (schedule 0)
        "gpu_launches": 4 * a.steps,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "peak_kind": f"{peaks_kind} bf16 sustained",
                     "traffic": (tr["bytes_per_flop"] * per_launch) if tr and tr.get("scalable", True) else None,
                     "traffic_source": (tr.get("source") if tr.get("scalable", True) else
                                        "not scaled: " + tr.get("note", "")) if tr else None,
                     "traffic_small_case": ({k: tr[k] for k in ("workload", "dram_bytes_read", "dram_bytes_write",
                                                                "duration_s", "algorithmic_flops_of_launch",
                                                                "algorithmic_bytes_of_launch", "l2_hit_rate_pct")
                                             if k in tr} if tr and not tr.get("scalable", True) else None),
                     "algorithmic_flops_per_launch": per_launch,
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "launch_ms_mean": launch_s * 1e3,
                     "simt_fp32": {"peak_tflops_nominal": simt_peak, "frac": achieved / simt_peak},
                     # the algorithmic flops are FP64-class work in the df and f64 modes: against the
                     # chip's nominal FP64 rate (1.25 TFLOP/s on a GB300)
                     "fp64_nominal": {"peak_tflops_nominal": FP64_NOMINAL_TFLOPS,
                                      "frac": achieved / FP64_NOMINAL_TFLOPS},
                     "kernel": "k_run (theta build + Jacobi SVD + truncation + measurement, one CTA per work item)"},
        "clocks": r["clocks"],
        "work": {"batch_per_gpu": r["B"], "gpu": r["gpu"],
                 "bond_ops_per_step": r["stats"]["bond_ops"] / a.steps,
                 "jacobi_sweeps_per_op": r["stats"]["sweeps"] / max(1.0, r["stats"]["bond_ops"]),
                 "meas_per_step": r["stats"]["meas"] / a.steps, "step_ms": r["step_ms"],
                 "host_step_s": r["host_step_s"], "untimed_layer_ms": r["untimed_ms"],
                 "schedule": ("one launch per layer, sweeps pushed as gates finish" if a.schedule == 1
                              else "two launches per layer (gates, then sweeps)"),
                 "launch_ms (gate+sweep launch | gate launch, sweep launch)": r["split"],
                 "lq_refactors_per_step": r["stats"]["lq_ops"] / a.steps,
                 "bond_op_cycle_share": {k[4:]: r["stats"][k] / cyc_sum for k in CYC_KEYS} if cyc_sum else None,
                 "ctas_busy_in_bond_ops": (cyc_sum / (r["sms"] * sm_mhz * 1e6 * r["elapsed"])) if cyc_sum else None,
                 "svd_sweep_limit_hits": [r["stats"]["nonconv"], r["stats"]["nonconv_c_lq"],
                                          r["stats"]["nonconv_c_direct"]],
                 "device_status": r["status"], "middle_bond_dims": [int(d[a.n // 2 - 1]) for d in r["dims"]]},
    }
    if rank == 0 and world == 1 and r["plain_states"]:
        import __graft_entry__ as ge
        pl = run_plain(a, ge.load_package(), r["plain_states"])
        out["plain_gpu"] = pl
        # the plain path is timed on the first timed layer, so it is compared with
        # the batch's rate on that same layer (every later layer costs more)
        first = r["B"] / (r["step_ms"][0] / 1e3) if r["step_ms"] else None
        out["batched_first_layer"] = {"value": first, "unit": UNIT, "layer": t_first}
        out["batched_over_plain"] = first / pl["value"] if first else None
        out["batched_over_plain_note"] = ("batched rate on layer {0} (the first timed layer) over the plain path on "
                                          "the same layer").format(t_first)
    if rank == 0 and world == 1 and a.serve_seconds > 0:
        import __graft_entry__ as ge
        out["serving"] = run_serving(a, ge.load_package())
    if cpu_async is not None:
        res = cpu_async.get()
        cpu_pool.close()
        cpu_pool.join()
        cb = summarize_reference(res, t_first, a.cpu_seconds, a.steps)
        out["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        out["cpu_baseline"]["seconds_per_traj_layer_per_core"] = cb["seconds_per_traj_layer_per_core"]
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
