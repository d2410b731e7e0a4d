"""The fPEPS oracle against its own ground truth: the literal Grassmann
contraction (every bond assignment, sign of the permutation of odd symbols)
must equal the local sign rule with the plain contraction, the exact
row-boundary contraction and the boundary contraction at large max_bond."""
import numpy as np
import pytest

from oracle import lattice, peps


@pytest.mark.parametrize("Lx,Ly,D,nup,ndn,nconf", [(4, 2, 2, 2, 2, 4), (3, 3, 2, 2, 2, 4), (4, 3, 2, 3, 3, 2),
                                                  (2, 4, 2, 3, 1, 4), (4, 2, 4, 3, 3, 1)])
def test_sign_rule_matches_grassmann(Lx, Ly, D, nup, ndn, nconf):
    T = peps.init_tensors(Lx, Ly, D, seed=Lx * 10 + Ly)
    X = lattice.random_initial_configs(nconf, Lx * Ly, nup, ndn, seed=D)
    for x in X:
        g = peps.amp_grassmann(T, x)
        assert abs(g) > 1e-6
        np.testing.assert_allclose(peps.amp_bruteforce(T, x), g, rtol=1e-12)
        if Lx % 2 == 0 and Lx >= 4:
            np.testing.assert_allclose(peps.amp_rows(T, x), g, rtol=1e-12)
            np.testing.assert_allclose(peps.amp_boundary_chi(T, x, D ** (Lx // 2)), g, rtol=1e-10)


def test_odd_particle_number_vanishes():
    T = peps.init_tensors(4, 2, 2, seed=0)
    x = lattice.random_initial_configs(1, 8, 3, 2, seed=0)[0]
    assert peps.amp_grassmann(T, x) == 0.0
    assert abs(peps.amp_rows(T, x)) < 1e-14


def test_rows_matches_bruteforce_6x4():
    T = peps.init_tensors(6, 4, 2, seed=5)
    X = lattice.random_initial_configs(3, 24, 6, 6, seed=6)
    for x in X:
        np.testing.assert_allclose(peps.amp_rows(T, x), peps.amp_bruteforce(T, x), rtol=1e-11)


def test_truncated_boundary_converges_6x6():
    """max_bond -> D^(Lx/2) recovers the exact amplitude; max_bond = 16 (the
    reference's config) is an approximation on random tensors."""
    T = peps.init_tensors(6, 6, 4, seed=3)
    x = lattice.random_initial_configs(1, 36, 16, 16, seed=4)[0]
    ex = peps.amp_rows(T, x)
    np.testing.assert_allclose(peps.amp_boundary_chi(T, x, 64), ex, rtol=1e-11)
    assert abs(peps.amp_boundary_chi(T, x, 16) / ex - 1) > 1e-3


@pytest.mark.parametrize("Lx,Ly,D,chi", [(4, 4, 4, 8), (4, 4, 4, 3), (6, 6, 4, 16), (6, 6, 4, 8), (6, 4, 4, 8),
                                         (4, 6, 4, 8), (6, 6, 2, 4)])
def test_state_truncation_equals_mps_protocol(Lx, Ly, D, chi):
    """The GPU kernels' formulation (full boundary state, best rank-chi
    truncations across the scheduled cuts) equals the boundary-MPS protocol
    (left-to-right QR, right-to-left truncated SVD after each absorbed row)."""
    T = peps.init_tensors(Lx, Ly, D, seed=3)
    N = Lx * Ly
    n = N // 2 - 1 if N > 8 else N // 2
    X = lattice.random_initial_configs(3, N, n, n, seed=1)
    for x in X:
        a = peps.amp_boundary_chi(T, x, chi)
        b = peps.amp_state_chi(T, x, chi)
        assert abs(a - b) <= 1e-11 * abs(a)


def test_chi_schedule_truncates_one_cut_at_6x6_chi16():
    """6x6, D = 4, chi = 16: each side truncates only the middle cut, after its
    third row, so the result is the unique best rank-16 approximation there
    (independent of the sweep order of the compression)."""
    assert peps.chi_schedule(6, 6, 4, 16) == [[], [], [3]]
    assert peps.chi_schedule(6, 6, 4, 64) == [[], [], []]
    assert peps.chi_schedule(6, 6, 4, 8) == [[], [4, 3, 2], [4, 3, 2]]


def test_chi_gradient_oracle_matches_finite_differences():
    """The oracle's O through the chi truncation (torch autograd through
    torch.linalg.svd, as the reference differentiates its contraction)
    against central differences (h = 1e-6) of the FP64 truncated amplitude."""
    T = peps.init_tensors(4, 4, 4, seed=4)
    x = lattice.random_initial_configs(1, 16, 4, 4, seed=3)[0]
    g = peps.logamp_grad_chi(T, x, 8)
    nz = np.argwhere(np.abs(g) > 1e-8)
    rng = np.random.default_rng(0)
    for idx in nz[rng.choice(len(nz), 8, replace=False)]:
        idx = tuple(idx)
        h = 1e-6 * max(1.0, abs(T[idx]))
        Tp, Tm = T.copy(), T.copy()
        Tp[idx] += h
        Tm[idx] -= h
        fd = (np.log(abs(peps.amp_state_chi(Tp, x, 8))) - np.log(abs(peps.amp_state_chi(Tm, x, 8)))) / (2 * h)
        assert abs(fd - g[idx]) <= 1e-5 * max(abs(fd), 1e-3)


@pytest.mark.parametrize("n,k", [(32, 8), (16, 5), (8, 3)])
def test_truncation_adjoint_formula(n, k):
    """The cotangent of the rank-k truncation (the formula of the chi
    log-derivative kernels) against central differences of <P(M), B>."""
    rng = np.random.default_rng(n + k)
    M = rng.normal(size=(n, n)) * np.exp(-0.3 * np.arange(n))[:, None]
    B = rng.normal(size=(n, n))
    Mbar = peps.trunc_adjoint(M, B, k)

    def f(Mx):
        u, s, vh = np.linalg.svd(Mx)
        return float(np.sum(((u[:, :k] * s[:k]) @ vh[:k]) * B))

    for _ in range(3):
        dM = rng.normal(size=(n, n))
        h = 1e-6
        fd = (f(M + h * dM) - f(M - h * dM)) / (2 * h)
        assert abs(np.sum(dM * Mbar) - fd) <= 1e-6 * max(1.0, abs(fd))
