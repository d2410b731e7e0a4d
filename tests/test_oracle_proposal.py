"""CPU check of the learned-proposal algorithm itself: with random network
weights, the exact Metropolis-Hastings transition matrix of the proposal
(summed over hop sets and draw orders) is row-stochastic and leaves |psi|^2
stationary on an enumerable 3x2 sector."""
import numpy as np

from oracle import lattice, models, proposal as op


def test_learned_proposal_keeps_psi_squared_stationary():
    Lx, Ly, nup, ndn = 3, 2, 2, 2
    N = Lx * Ly
    edges = lattice.square_edges(Lx, Ly)
    S = lattice.all_states(N, nup, ndn)
    rng = np.random.default_rng(0)
    M = rng.normal(0, 0.5, size=(2 * N, nup + ndn))
    amp = models.slater_amp(M, S)
    Kin = 64
    flat = np.concatenate([rng.normal(0, 0.3, PHK) for PHK in
                           (op.PH * Kin, op.PH, op.PH * op.PH, op.PH, op.PLOG * op.PH, op.PLOG)])
    P = op.transition_matrix(S, lambda X: op.logits(flat, X, N), amp, edges)
    assert np.all(P >= -1e-12)
    np.testing.assert_allclose(P.sum(1), 1.0, atol=1e-12)
    pi = amp ** 2 / (amp ** 2).sum()
    np.testing.assert_allclose(pi @ P, pi, atol=1e-12)
    # the chain moves (more than local single hops: some k >= 2 transitions)
    assert (np.diag(P) < 1).mean() > 0.5


def test_log_q_orders_sum():
    edges = lattice.square_edges(3, 2)
    x = lattice.random_initial_configs(1, 6, 2, 2, seed=3)[0]
    lg = np.random.default_rng(1).normal(size=op.PLOG)
    valid = np.nonzero(op.valid_hops(x[None], edges)[0])[0]
    # single-hop probabilities sum to p(k=1)
    tot = sum(np.exp(op.log_q(lg, x, [h], edges)) for h in valid)
    H = 2 * len(edges)
    kl = lg[H:H + 4]
    pk1 = np.exp(kl[0] - kl.max()) / np.exp(kl - kl.max()).sum()
    assert abs(tot - pk1) < 1e-12
