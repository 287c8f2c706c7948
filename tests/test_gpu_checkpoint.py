"""Checkpoint / resume (tn_mps_import, MPS.save / MPS.load): a state
written mid-trajectory and read back continues bit for bit like the
original in both precisions; a state handed over from the FP64 oracle
continues like the oracle (1e-10)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["f64", "mixed"])
def test_save_load_resumes_bit_for_bit(pkg, tmp_path, prec):
    n = 10
    tr = pkg.Trunc.both(16, 1e-12)
    a = pkg.MPS.new_qubits(n, tr, prec)
    traj = pkg.gen_trajectory(13, 0, n, 12, 0.2)
    for layer in traj[:6]:
        a.apply_bilayer(*layer)
    f = tmp_path / "state.npz"
    a.save(f)
    b = pkg.MPS.load(f)
    assert b.n == n and b.get_trunc() == tr and b.precision_name() == prec
    for bd in range(n - 1):
        np.testing.assert_array_equal(b.svals(bd), a.svals(bd))
    for layer in traj[6:]:
        assert a.apply_bilayer(*layer) == b.apply_bilayer(*layer)
        assert a.entropy_vn(n // 2 - 1) == b.entropy_vn(n // 2 - 1)
    for k in range(n):
        np.testing.assert_array_equal(a.gamma(k), b.gamma(k))
    assert a.device_status() == 0 and b.device_status() == 0


def test_state_from_the_oracle_continues_like_the_oracle(pkg, ref):
    n = 9
    r = ref.MPS(n, ref.Trunc.both(16, 1e-12))
    traj = pkg.gen_trajectory(17, 0, n, 10, 0.15)
    for layer in traj[:5]:
        ref.apply_bilayer(r, *layer)
    g = pkg.MPS.from_parts(r.data, r.svals, pkg.Trunc.both(16, 1e-12), "f64")
    for layer in traj[5:]:
        rg = g.apply_bilayer(*layer)
        rr = ref.apply_bilayer(r, *layer)
        assert [x[:2] for x in rg] == [x[:2] for x in rr]
        for x, y in zip(rg, rr):
            assert abs(x[2] - y[2]) < 1e-10
    for b in range(n - 1):
        assert abs(g.entropy_vn(b) - r.entropy_vn(b)) < 1e-10
    assert g.device_status() == 0


@pytest.mark.parametrize("prec", ["f64", "mixed"])
def test_prepared_state_enters_a_batch(pkg, prec):
    """A state factorised from a dense vector (tn_mps_from_vector) enters a
    batch slot (tn_batch_import) and evolves there exactly as on its own
    handle; exported back from the batch it continues identically."""
    n = 10
    rng = np.random.default_rng(8)
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    tr = pkg.Trunc.both(16, 1e-12)
    m = pkg.MPS.from_vector(psi, tr, prec)
    b = pkg.Batch([n, n], [tr, tr], prec)
    b.import_state(1, *m.export_parts(), tr)
    for k in range(n):
        np.testing.assert_array_equal(b.gamma(1, k), m.gamma(k))
    tol = 1e-10 if prec == "f64" else 1e-5
    traj = pkg.gen_trajectory(23, 0, n, 8, 0.2)

    def same(r1, r2):
        assert [x[:2] for x in r1] == [x[:2] for x in r2]
        for x, y in zip(r1, r2):
            assert abs(x[2] - y[2]) < tol

    for layer in traj[:4]:
        recs, ents = b.step([1], [layer])
        same(recs[0], m.apply_bilayer(*layer))
        assert abs(ents[0] - m.entropy_vn(n // 2 - 1)) < tol
    m2 = pkg.MPS.from_parts(*b.export_parts(1), tr, prec)
    for layer in traj[4:]:
        same(m2.apply_bilayer(*layer), m.apply_bilayer(*layer))
    with pytest.raises(pkg.TnError) as e:
        b.import_state(0, *pkg.MPS.from_vector(psi, None, prec).export_parts(), None)  # bond 32 > capacity 16
    assert e.value.status == -9
    assert b.device_status() == 0
