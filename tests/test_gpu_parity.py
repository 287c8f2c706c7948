"""GPU path (through the C ABI) against the FP64 oracle on identical inputs.

Tolerances: the F64 path must match the oracle to 1e-9 on Schmidt values,
probabilities and entropies (both use float64; they differ only in the SVD
algorithm: one-sided Jacobi vs LAPACK gesvd), and so must the DF path
(double-float arithmetic, about 48 significant bits).  The MIXED path (complex64
Gamma, float32 Jacobi) is held to 1e-4 on the small cases here; its error at
the benchmark sizes is measured and reported, not asserted.  Outcomes must be
identical except where |p - u| < 1e-9 (a tie the two paths may break
differently).
"""
import numpy as np
import pytest

from gates import CX, CXREV, CZ, H, xrot

pytestmark = pytest.mark.gpu

LN2 = np.log(2.0)
TOL = {"f64": 1e-9, "mixed": 1e-4, "df": 1e-9}


def _pair(pkg, ref, n, trunc_args, prec, chi_cap=0):
    kind, a = trunc_args
    gt = getattr(pkg.Trunc, kind)(*a) if kind != "none" else None
    rt = getattr(ref.Trunc, kind)(*a) if kind != "none" else None
    return pkg.MPS.new_qubits(n, gt, prec, chi_cap), ref.MPS(n, rt)


# The MIXED path drops Schmidt values below 2*sqrt(ell)*eps32 (float32 noise
# floor, ell <= 2*chi); compare spectra above this floor.
FLOOR = {"f64": 0.0, "mixed": 1e-4, "df": 0.0}


def _assert_same_state(g, r, tol, floor=0.0):
    for b in range(r.n - 1):
        sg, sr = g.svals(b), r.svals[b]
        sg, sr = sg[sg > floor], sr[sr > floor]
        assert len(sg) == len(sr), (b, len(sg), len(sr))
        assert np.max(np.abs(sg - sr)) < tol, (b, np.max(np.abs(sg - sr)))
    for k in range(r.n):
        assert np.max(np.abs(g.probs(k) - r.probs(k))) < tol, k


@pytest.mark.parametrize("prec", ["f64", "mixed", "df"])
def test_rotation_known_answer(pkg, prec):
    """workspace/src/rotation_testing.rs:13-38 on the GPU."""
    th = 3 * np.pi / 5
    m = pkg.MPS.new_qubits(5, pkg.Trunc.const(2), prec)
    m.apply_unitary1(2, xrot(th))
    m.apply_unitary2(2, CX)
    p0, p1 = np.cos(th / 2) ** 2, np.sin(th / 2) ** 2
    tol = 1e-6 if prec == "mixed" else 1e-12
    for k in range(5):
        exp = [p0, p1] if k in (2, 3) else [1.0, 0.0]
        np.testing.assert_allclose(m.probs(k), exp, atol=tol)
    m1 = m.clone()
    assert abs(m1.measure_postsel_prob(2, 1) - p1) < tol
    np.testing.assert_allclose(m1.probs(3), [0.0, 1.0], atol=tol)
    assert m.device_status() == 0 and m1.device_status() == 0


@pytest.mark.parametrize("prec", ["f64", "mixed", "df"])
def test_bell_and_ghz(pkg, prec):
    tol = 1e-6 if prec == "mixed" else 1e-12
    m = pkg.MPS.new_qubits(4, None, prec)
    m.apply_unitary1(0, H)
    m.apply_unitary2(0, CX)
    assert abs(m.entropy_vn(0) - LN2) < tol
    out, prob = m.measure_prob(0, 0.75)
    assert out == 1 and abs(prob - 0.5) < tol
    psi = m.contract()
    assert abs(abs(psi[12]) - 1.0) < tol
    # GHZ via SWAP chains (workspace/src/testing.rs:16-50)
    g = pkg.MPS.new_qubits(5, None, prec)
    g.apply_unitary1(0, H)
    for k in range(3):
        for op in (CX, CXREV, CX):
            g.apply_unitary2(k, op)
    g.apply_unitary2(3, CX)
    for k in (2, 1, 0):
        for op in (CX, CXREV, CX):
            g.apply_unitary2(k, op)
    g.apply_unitary1(2, H)
    g.apply_unitary2(2, CX)
    np.testing.assert_allclose([g.entropy_vn(b) for b in range(4)], [LN2, LN2, 2 * LN2, LN2], atol=tol)
    a = g.measure(2, 0.9)
    b = g.measure(3, 0.1)
    assert a == b
    assert g.device_status() == 0


def test_cluster_state(pkg, ref):
    """workspace/src/state.rs:4-58 on the GPU, against the oracle."""
    n = 4
    g = pkg.MPS.new_qubits(n, None, "f64")
    r = ref.MPS(n, None)
    for czs in [[0, 2], [1], [0, 2], [1], [0, 2]]:
        for k in range(n):
            g.apply_unitary1(k, H)
            r.apply_unitary1(k, H)
        for k in czs:
            g.apply_unitary2(k, CZ)
            r.apply_unitary2(k, CZ)
        assert abs(g.entropy_vn(1) - r.entropy_vn(1)) < 1e-12
    np.testing.assert_allclose(g.contract(), r.contract(), atol=1e-12)


@pytest.mark.parametrize("prec", ["f64", "mixed", "df"])
@pytest.mark.parametrize("n,chi,p,seed", [(8, 16, 0.3, 1), (10, 8, 0.2, 2), (9, 32, 0.15, 3)])
def test_trajectory_parity(pkg, ref, prec, n, chi, p, seed):
    """Seeded Haar brickwork with measurements, layer by layer."""
    tol = TOL[prec]
    g, r = _pair(pkg, ref, n, ("both", (chi, 1e-12)), prec)
    for t, (gk, gs, mk, us) in enumerate(pkg.gen_trajectory(seed, 0, n, 10, p)):
        rg = g.apply_bilayer(gk, gs, mk, us)
        rr = ref.apply_bilayer(r, gk, gs, mk, us)
        assert len(rg) == len(rr)
        for (kg, og, pg), (kr, orr, pr), u in zip(rg, rr, us):
            assert kg == kr
            if abs(pr - u) > 1e-9 or og == orr:
                assert og == orr, (t, kg, pg, pr, u)
            assert abs(pg - pr) < tol
        b = n // 2 - 1
        assert abs(g.entropy_vn(b) - r.entropy_vn(b)) < tol, t
    _assert_same_state(g, r, tol, FLOOR[prec])
    assert g.device_status() == 0


def test_dense_contract_matches_oracle(pkg, ref):
    n = 7
    g, r = _pair(pkg, ref, n, ("none", ()), "f64")
    for (gk, gs, mk, us) in pkg.gen_trajectory(5, 0, n, 6, 0.2):
        g.apply_bilayer(gk, gs, mk, us)
        ref.apply_bilayer(r, gk, gs, mk, us)
    # Gamma is gauge dependent; the contracted state is not (up to a global phase)
    a, b = g.contract(), r.contract()
    assert abs(abs(np.vdot(a, b)) - 1.0) < 1e-10


def test_edge_cases(pkg, ref):
    # n = 1: probabilities, unitary1, no bonds
    one = pkg.MPS.new_qubits(1, None, "f64")
    np.testing.assert_allclose(one.probs(0), [1.0, 0.0])
    one.apply_unitary1(0, H)
    np.testing.assert_allclose(one.probs(0), [0.5, 0.5], atol=1e-15)
    assert one.entropy_vn(0) is None and one.bond_dim(0) is None
    out, prob = one.measure_prob(0, 0.7)
    assert out == 1 and abs(prob - 0.5) < 1e-15
    # out of range: silent no-ops and None
    m = pkg.MPS.new_qubits(3, None, "f64")
    m.apply_unitary2(2, CX)
    m.apply_unitary1(7, H)
    assert m.probs(3) is None and m.measure_prob(3, 0.5) is None and m.entropy_vn(2) is None
    # bad shape
    with pytest.raises(pkg.TnError) as e:
        m.apply_unitary2(0, np.eye(2))
    assert e.value.status == -5
    with pytest.raises(pkg.TnError):
        m.apply_unitary1(0, np.eye(4))
    # empty measurement layer and duplicates / unsorted / out-of-range targets
    g, r = _pair(pkg, ref, 6, ("none", ()), "f64")
    for x in (g, r):
        x.apply_unitary1(1, H)
        x.apply_unitary2(1, CX)
        x.apply_unitary2(2, CX)
    assert g.apply_meas_prob_layer([], []) == []
    rg = g.apply_meas_prob_layer([3, 1, 9, 3], [0.8, 0.2])
    rr = r.apply_meas_prob_layer([3, 1, 9, 3], [0.8, 0.2])
    assert [x[:2] for x in rg] == [x[:2] for x in rr]
    _assert_same_state(g, r, 1e-12)
    # post-selection through the layer API (Meas::Proj)
    g2, r2 = _pair(pkg, ref, 6, ("none", ()), "f64")
    for x in (g2, r2):
        x.apply_unitary1(0, H)
        x.apply_unitary2(0, CX)
    rg = g2.apply_meas_prob_layer([0, 4], None, posts=[1, 0])
    rr = r2.apply_meas_prob_layer([0, 4], None, posts=[1, 0])
    assert [x[:2] for x in rg] == [x[:2] for x in rr] == [(0, 1), (4, 0)]
    assert abs(rg[0][2] - 0.5) < 1e-12
    # get/set trunc, bond dims
    assert g2.get_trunc() is None
    g2.set_trunc(pkg.Trunc.const(1))
    assert g2.get_trunc() == pkg.Trunc.const(1)
    assert g2.max_bond_dim() == 1


def test_last_site_measurement_reference_behaviour(pkg, ref):
    """Bond n-2 is not refactored when site n-1 is the highest measured site
    (mps.rs:2246-2250); the GPU path keeps this for parity."""
    n = 4
    g, r = _pair(pkg, ref, n, ("none", ()), "f64")
    for x in (g, r):
        x.apply_unitary1(2, H)
        x.apply_unitary2(2, CX)
    g.apply_meas_prob_layer([n - 1], [0.3])
    r.apply_meas_prob_layer([n - 1], [0.3])
    np.testing.assert_allclose(g.svals(n - 2), r.svals[n - 2], atol=1e-15)
    assert abs(g.entropy_vn(n - 2) - LN2) < 1e-12


@pytest.mark.parametrize("prec", ["f64", "df"])
def test_batch_matches_single_and_is_mix_independent(pkg, ref, prec):
    """Each trajectory's result is the same alone and in a mixed batch
    (bit-identical: one CTA runs one trajectory with a fixed reduction order),
    and equals the single-state API."""
    specs = [(8, 16, 0.2), (11, 8, 0.3), (6, 4, 0.1), (9, 32, 0.25)]
    ns = [s[0] for s in specs]
    truncs = [pkg.Trunc.both(s[1], 1e-12) for s in specs]
    mix = pkg.Batch(ns, truncs, prec)
    alone = pkg.Batch([ns[1]], [truncs[1]], prec)
    single = pkg.MPS.new_qubits(ns[1], truncs[1], prec)
    rtraj = ref.MPS(ns[1], ref.Trunc.both(8, 1e-12))
    for t in range(8):
        layers = [pkg.gen_layer(77, i, t, s[0], s[2]) for i, s in enumerate(specs)]
        recs, ents = mix.step(list(range(4)), layers)
        recs1, ents1 = alone.step([0], [layers[1]])
        rs = single.apply_bilayer(*layers[1])
        rr = ref.apply_bilayer(rtraj, *layers[1])
        assert recs[1] == recs1[0]
        assert ents[1] == ents1[0]
        assert [x[:2] for x in rs] == [x[:2] for x in recs[1]]
        assert abs(ents[1] - single.entropy_vn(ns[1] // 2 - 1)) == 0.0
        assert abs(ents[1] - rtraj.entropy_vn(ns[1] // 2 - 1)) < 1e-9
    np.testing.assert_array_equal(mix.svals(1, 4), alone.svals(0, 4))
    assert mix.device_status() == 0


def test_batch_schedules_agree(pkg):
    """The one-launch schedule (sweep items pushed as a trajectory's gates
    finish) and the two-launch schedule give bit-identical results, including
    trajectories with no gate in a layer (n = 2 on odd layers, n = 3 rows
    where the brickwork leaves one gate) whose sweep items are pushed before
    the launch."""
    specs = [(2, 4, 0.3), (12, 16, 0.2), (3, 4, 0.5), (9, 32, 0.25), (16, 32, 0.1), (5, 8, 0.0)]
    ns = [s[0] for s in specs]
    truncs = [pkg.Trunc.both(s[1], 1e-12) for s in specs]
    one = pkg.Batch(ns, truncs, "mixed")
    two = pkg.Batch(ns, truncs, "mixed")
    one.set_schedule(1)
    two.set_schedule(0)
    order = list(range(len(specs)))
    for t in range(10):
        layers = [pkg.gen_layer(31, i, t, s[0], s[2]) for i, s in enumerate(specs)]
        r1, e1 = one.step(order, layers)
        r0, e0 = two.step(order, layers)
        assert r1 == r0
        assert list(e1) == list(e0)
        ms1, ms0 = one.last_launch_ms(), two.last_launch_ms()
        assert ms1[1] == 0.0 and ms0[1] > 0.0
    for i in range(len(specs)):
        for bnd in range(ns[i] - 1):
            np.testing.assert_array_equal(one.svals(i, bnd), two.svals(i, bnd))
    assert one.device_status() == 0 and two.device_status() == 0


class _DevView:
    """A raw device range seen by torch through __cuda_array_interface__."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 2}


def test_graph_captured_step_matches_host_step(pkg):
    """tn_batch_step_device (a CUDA graph of the layer's scan, compile and
    executor launch, captured once per trajectory count) gives the same bits
    as tn_batch_step, including when the number of listed trajectories
    changes between layers (a second capture)."""
    torch = pytest.importorskip("torch")
    specs = [(10, 16, 0.2), (7, 8, 0.3), (12, 32, 0.1), (9, 16, 0.25)]
    ns = [s[0] for s in specs]
    truncs = [pkg.Trunc.both(s[1], 1e-12) for s in specs]
    host = pkg.Batch(ns, truncs, "mixed")
    dev = pkg.Batch(ns, truncs, "mixed")
    ptr = dev.device_inputs(max_gates=sum(n // 2 for n in ns), max_meas=sum(ns))
    view = lambda name, n, ts: torch.as_tensor(_DevView(ptr[name], n, ts), device="cuda")
    for t in range(8):
        nt = 4 if t % 3 else 3  # lists of 3 and 4 trajectories
        trajs = list(range(nt))
        layers = [pkg.gen_layer(5, i, t, specs[i][0], specs[i][2]) for i in trajs]
        r_host, e_host = host.step(trajs, layers)
        pk = pkg.Batch.pack(trajs, layers)
        nm = int(pk["meas_off"][-1])
        for name, ts, arr in (("trajs", "<i4", pk["trajs"].astype(np.int32)),
                              ("gate_off", "<i4", pk["gate_off"].astype(np.int32)),
                              ("gate_ks", "<i4", pk["gate_ks"].astype(np.int32)),
                              ("gates", "<f8", pk["gates"]),
                              ("meas_off", "<i4", pk["meas_off"].astype(np.int32)),
                              ("meas_ks", "<i4", pk["meas_ks"].astype(np.int32)),
                              ("us", "<f8", pk["us"])):
            if arr.size:
                view(name, arr.size, ts).copy_(torch.from_numpy(np.ascontiguousarray(arr)))
        torch.cuda.synchronize()
        dev.step_device(nt)
        dev.synchronize()
        ent = view("entropy", nt, "<f8").cpu().numpy()
        oc = view("outcomes", max(nm, 1), "<i4").cpu().numpy()[:nm]
        pr = view("probs", max(nm, 1), "<f8").cpu().numpy()[:nm]
        assert list(ent) == list(e_host)
        flat = [rec for recs in r_host for rec in recs]
        assert [int(x[1]) for x in flat] == list(oc)
        assert [x[2] for x in flat] == list(pr)
    assert host.device_status() == 0 and dev.device_status() == 0


def test_autotuner_tries_every_candidate_and_keeps_the_best(pkg):
    """tn_batch_autotune runs each candidate configuration (schedule, Jacobi
    scheme, tensor-core / SIMT theta) for its trial steps, scores it by
    device time per algorithmic flop and keeps the best; results stay within
    the mixed-precision tolerance of an untuned batch on the same inputs."""
    specs = [(12, 32, 0.1), (14, 64, 0.05), (10, 16, 0.2), (16, 64, 0.15)]
    ns = [s[0] for s in specs]
    truncs = [pkg.Trunc.both(s[1], 1e-10) for s in specs]
    tuned = pkg.Batch(ns, truncs, "mixed")
    plain = pkg.Batch(ns, truncs, "mixed")
    order = list(range(len(specs)))
    for t in range(6):  # grow entanglement first so that every candidate does real work
        layers = [pkg.gen_layer(9, i, t, s[0], s[2]) for i, s in enumerate(specs)]
        tuned.step(order, layers)
        plain.step(order, layers)
    tuned.autotune(1)
    assert tuned.tuning()["tuning"]
    for t in range(6, 12):
        layers = [pkg.gen_layer(9, i, t, s[0], s[2]) for i, s in enumerate(specs)]
        r1, e1 = tuned.step(order, layers)
        r0, e0 = plain.step(order, layers)
        assert [[x[:2] for x in a] for a in r1] == [[x[:2] for x in a] for a in r0]
        np.testing.assert_allclose(e1, e0, atol=1e-4)
    st = tuned.tuning()
    assert not st["tuning"]
    assert all(s > 0 for s in st["scores"])
    best = int(np.argmin(st["scores"]))
    cand = [(1, 3, 0), (1, 0, 0), (0, 3, 0), (1, 3, 1)][best]
    assert (st["schedule"], st["scheme"], st["theta_simt"]) == cand
    assert tuned.device_status() == 0


@pytest.mark.parametrize("prec", ["f64", "df", "mixed"])
def test_entropy_ry_schmidt_matches_oracle(pkg, ref, prec):
    """entropy_ry_schmidt (mps.rs:1268-1282): the Renyi entropy of the Schmidt
    values of every bond for a in {0.5, 1, 2, 3} (a = 1 is entropy_vn) after
    a seeded trajectory, and None off the chain."""
    n, chi = 9, 16
    g, r = _pair(pkg, ref, n, ("both", (chi, 1e-12)), prec)
    for (gk, gs, mk, us) in pkg.gen_trajectory(5, 0, n, 6, 0.2):
        g.apply_bilayer(gk, gs, mk, us)
        ref.apply_bilayer(r, gk, gs, mk, us)
    for b in range(n - 1):
        for a in (0.5, 1.0, 2.0, 3.0):
            ea, er = g.entropy_ry_schmidt(a, b), r.entropy_ry_schmidt(a, b)
            assert abs(ea - er) < TOL[prec], (b, a, ea, er)
        assert g.entropy_ry_schmidt(1.0, b) == g.entropy_vn(b)
    assert g.entropy_ry_schmidt(2.0, n - 1) is None and r.entropy_ry_schmidt(2.0, n - 1) is None
    assert g.device_status() == 0
