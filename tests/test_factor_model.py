"""The from_vector algorithm of tensor-net_gb300/csrc/tn_factor.cu restated
in numpy (same circle ordering, rotation, convergence tolerance, zero-row
rule, rank rule with the noise floor): on the CPU it must reproduce scipy's
factorisation (the oracle's restatement of factorize, mps.rs:448-505) on
random states, and the exact Schmidt ranks of exact low-rank states, where
LAPACK leaves rounding-noise values above the EPS rule.  This pins the
kernel's design choices; the kernel itself is tested on the GPU."""
import numpy as np
import pytest

from oracle import mps_ref as R

EPS = 2.220446049250313e-16


def _row_jacobi(q, tol, zero2=1e-30, max_sweeps=60):
    q = q.copy()
    m = q.shape[0]
    rm = np.eye(m, dtype=complex)
    mp = m + (m & 1)
    ring = mp - 1
    for sweep in range(max_sweeps):
        rotated = False
        for r in range(mp - 1):
            for w in range(mp // 2):
                a, b = (r, mp - 1) if w == 0 else ((r + w) % ring, (r - w + ring) % ring)
                if a >= m or b >= m:
                    continue
                p, s = min(a, b), max(a, b)
                x, y = q[p], q[s]
                al, be, gam = np.vdot(x, x).real, np.vdot(y, y).real, np.vdot(x, y)
                if al < zero2 or be < zero2:
                    continue
                g = abs(gam)
                if not g > tol * np.sqrt(al) * np.sqrt(be):
                    continue
                zeta = (be - al) / (2 * g)
                t = (1.0 if zeta >= 0 else -1.0) / (abs(zeta) + np.hypot(1.0, zeta))
                c = 1 / np.sqrt(1 + t * t)
                sn = c * t
                ph = np.conj(gam) / g
                q[p], q[s] = c * x - sn * ph * y, sn * x + c * ph * y
                xr, yr = rm[p].copy(), rm[s].copy()
                rm[p], rm[s] = c * xr - sn * ph * yr, sn * xr + c * ph * yr
                rotated = True
        if not rotated:
            return q, rm
    raise AssertionError("sweep limit")


def _model_from_vector(psi):
    n = int(np.log2(psi.size))
    q = psi / np.linalg.norm(psi)
    udim, lams = 1, []
    for k in range(n - 1):
        m, nq = 2 * udim, psi.size >> (k + 1)
        qr, rm = _row_jacobi(q.reshape(m, nq), 1e-14 * max(1.0, np.sqrt(nq / 1024.0)))
        sv = np.linalg.norm(qr, axis=1)
        perm = sorted(range(m), key=lambda j: (-sv[j], j))
        tot = np.sqrt(sum(sv[j] ** 2 for j in perm))
        sn = np.array([sv[j] / tot for j in perm])
        eps = max(EPS, 4.0 * np.sqrt(max(m, nq)) * EPS)
        rank = 0
        while rank < min(m, nq) and sn[rank] > eps and sn[rank] >= np.finfo(float).tiny:
            rank += 1
        rank = max(rank, 1)
        lams.append(sn[:rank] / np.sqrt(np.sum(sn[:rank] ** 2)))
        q = np.stack([qr[perm[j]] / tot for j in range(rank)]).reshape(-1)
        udim = rank
    return lams


@pytest.mark.parametrize("n", [2, 5, 8])
def test_model_matches_the_oracle_on_random_states(n):
    rng = np.random.default_rng(50 + n)
    psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    lams = _model_from_vector(psi)
    ref = R.from_vector(psi)
    for a, b in zip(lams, ref.svals):
        assert len(a) == len(b)
        np.testing.assert_allclose(a, b, atol=1e-13)


def test_model_keeps_exact_ranks_of_low_rank_states():
    rng = np.random.default_rng(3)

    def product(n):
        p = np.ones(1)
        for _ in range(n):
            p = np.kron(p, rng.standard_normal(2) + 1j * rng.standard_normal(2))
        return p

    assert [len(x) for x in _model_from_vector(product(7))] == [1] * 6
    r3 = product(8) + product(8) + product(8)
    lams = _model_from_vector(r3)
    assert [len(x) for x in lams] == [2, 3, 3, 3, 3, 3, 2]
    ref = R.from_vector(r3)
    for a, b in zip(lams, ref.svals):
        np.testing.assert_allclose(a, b[: len(a)], atol=1e-12)
        assert np.all(b[len(a):] < 1e-14)  # what LAPACK keeps beyond the exact rank is rounding noise
    ghz = np.zeros(1 << 6, complex)
    ghz[0] = ghz[-1] = 1
    assert [len(x) for x in _model_from_vector(ghz)] == [2] * 5
