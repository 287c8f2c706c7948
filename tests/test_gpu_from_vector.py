"""MPS::from_vector (mps.rs:517-550) on the GPU against the FP64 oracle's
restatement of factorize (mps.rs:448-505): Schmidt values and bond
dimensions to 1e-12, the contracted state against the normalised input to
1e-12 (float64); later operations on the factorised state match the oracle
(the Schmidt form is canonical)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand_state(rng, n):
    return rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)


def _same_lambdas(g, r, tol):
    for b in range(r.n - 1):
        sg, sr = g.svals(b), r.svals[b]
        assert len(sg) == len(sr), (b, len(sg), len(sr))
        np.testing.assert_allclose(sg, sr, atol=tol)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 11])
def test_random_states_match_oracle_and_reconstruct(pkg, ref, n):
    rng = np.random.default_rng(100 + n)
    psi = _rand_state(rng, n)
    g = pkg.MPS.from_vector(psi)
    r = ref.from_vector(psi)
    _same_lambdas(g, r, 1e-12)
    np.testing.assert_allclose(g.contract(), psi / np.linalg.norm(psi), atol=1e-12)
    for k in range(n):
        np.testing.assert_allclose(g.probs(k), r.probs(k), atol=1e-12)


def test_larger_state_and_truncation(pkg, ref):
    rng = np.random.default_rng(7)
    psi = _rand_state(rng, 14)
    g = pkg.MPS.from_vector(psi)
    r = ref.from_vector(psi)
    _same_lambdas(g, r, 1e-12)
    assert abs(abs(np.vdot(g.contract(), psi / np.linalg.norm(psi))) - 1.0) < 1e-12
    for tr, rt in ((pkg.Trunc.const(5), ref.Trunc.const(5)), (pkg.Trunc.cut(1e-2), ref.Trunc.cut(1e-2)),
                   (pkg.Trunc.both(6, 1e-3), ref.Trunc.both(6, 1e-3))):
        g = pkg.MPS.from_vector(psi[: 1 << 10], tr)
        r = ref.from_vector(psi[: 1 << 10], rt)
        _same_lambdas(g, r, 1e-12)
        assert g.get_trunc() == tr


def test_exact_low_rank_states(pkg, ref):
    n = 7
    ghz = np.zeros(1 << n, complex)
    ghz[0] = ghz[-1] = 1
    g = pkg.MPS.from_vector(ghz)
    assert [g.bond_dim(b) for b in range(n - 1)] == [2] * (n - 1)
    for b in range(n - 1):
        assert abs(g.entropy_vn(b) - np.log(2)) < 1e-13
    rng = np.random.default_rng(3)
    prod = np.ones(1)
    for _ in range(n):
        prod = np.kron(prod, rng.standard_normal(2) + 1j * rng.standard_normal(2))
    p = pkg.MPS.from_vector(prod)
    assert [p.bond_dim(b) for b in range(n - 1)] == [1] * (n - 1)
    np.testing.assert_allclose(p.contract(), prod / np.linalg.norm(prod), atol=1e-13)
    w = np.zeros(1 << n, complex)
    w[[1 << j for j in range(n)]] = 1
    wm, wr = pkg.MPS.from_vector(w), ref.from_vector(w)
    _same_lambdas(wm, wr, 1e-13)
    # a sum of three product states: Schmidt rank 3 in the middle.  LAPACK
    # leaves values of ~3e-16 above the EPS rule (the oracle keeps them); the
    # GPU path's noise floor drops them and keeps the exact ranks
    r3 = np.zeros(1 << 8, complex)
    for _ in range(3):
        p1 = np.ones(1)
        for _ in range(8):
            p1 = np.kron(p1, rng.standard_normal(2) + 1j * rng.standard_normal(2))
        r3 += p1
    g3, o3 = pkg.MPS.from_vector(r3), ref.from_vector(r3)
    assert [g3.bond_dim(b) for b in range(7)] == [2, 3, 3, 3, 3, 3, 2]
    for b in range(7):
        np.testing.assert_allclose(g3.svals(b), o3.svals[b][: g3.bond_dim(b)], atol=1e-12)
    np.testing.assert_allclose(g3.contract(), r3 / np.linalg.norm(r3), atol=1e-12)


def test_evolution_after_from_vector_matches_oracle(pkg, ref):
    n = 9
    rng = np.random.default_rng(11)
    psi = _rand_state(rng, n)
    tr = (pkg.Trunc.both(12, 1e-12), ref.Trunc.both(12, 1e-12))
    g = pkg.MPS.from_vector(psi, tr[0])
    r = ref.from_vector(psi, tr[1])
    for (gk, gs, mk, us) in pkg.gen_trajectory(4, 0, n, 6, 0.2):
        rg = g.apply_bilayer(gk, gs, mk, us)
        rr = ref.apply_bilayer(r, gk, gs, mk, us)
        assert [x[:2] for x in rg] == [x[:2] for x in rr]
        for a, b in zip(rg, rr):
            assert abs(a[2] - b[2]) < 1e-10
    for b in range(n - 1):
        assert abs(g.entropy_vn(b) - r.entropy_vn(b)) < 1e-10
    assert g.device_status() == 0


def test_mixed_precision_and_errors(pkg, ref):
    rng = np.random.default_rng(5)
    psi = _rand_state(rng, 8)
    g = pkg.MPS.from_vector(psi, None, "mixed")
    np.testing.assert_allclose(g.contract(), psi / np.linalg.norm(psi), atol=1e-6)
    with pytest.raises(pkg.TnError) as e:
        pkg.MPS.from_vector(np.zeros(16))
    assert e.value.status == -6
    with pytest.raises(pkg.TnError) as e:
        pkg.MPS.from_vector(psi, pkg.Trunc.const(64), "f64", chi_cap=4)
    assert e.value.status == -9  # a Schmidt rank above the capacity
