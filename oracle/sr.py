"""minSR step, SGD update, energy statistics and chain diagnostics
(oracle, test-only; FP64).

  * minSR (vmc_torch/GPU/optimizer.py:545-563): O~ = (O - <O>)/sqrt(Ns);
    T = O~ O~^T + lambda I; solve T x = (E - <E>)/sqrt(Ns); dp = O~^T x.
    (The CPU minSR uses pinv(T) with no shift, vmc_torch/optimizer.py:223-254.)
  * plain energy gradient when run_sr is False (optimizer.py:585-613):
    <E O> - <E><O>.
  * SGD: theta <- theta - lr * dp (vmc_torch/GPU/optimizer.py:178-186).
  * energy stats: mean and <E^2> - <E>^2 (vmc_torch/GPU/VMC.py:513-534).
  * split-chain R-hat (vmc_torch/variational_state.py:574-587).
  * integrated autocorrelation time with Sokal's automatic window (c = 5) —
    no reference counterpart (the reference has no tau_int / ESS estimator).
"""
import numpy as np


def minsr(O, E, energy_mean, diag_shift):
    return minsr_with_info(O, E, energy_mean, diag_shift)[0]


def minsr_with_info(O, E, energy_mean, diag_shift):
    """(dp, info): LU solve of T x = E~, and when T is exactly singular the
    least-squares fallback with info = 1 (vmc_torch/GPU/optimizer.py:557-561;
    numpy's lstsq gives the minimum-norm solution)."""
    O = np.asarray(O, np.float64)
    E = np.asarray(E, np.float64)
    Ns = O.shape[0]
    Oc = (O - O.mean(axis=0, keepdims=True)) / np.sqrt(Ns)
    Es = (E - energy_mean) / np.sqrt(Ns)
    T = Oc @ Oc.T + diag_shift * np.eye(Ns)
    try:
        x, info = np.linalg.solve(T, Es), 0
    except np.linalg.LinAlgError:
        x, info = np.linalg.lstsq(T, Es, rcond=None)[0], 1
    return Oc.T @ x, info


def energy_gradient(O, E, energy_mean):
    O = np.asarray(O, np.float64)
    E = np.asarray(E, np.float64)
    return (E @ O) / O.shape[0] - energy_mean * O.mean(axis=0)


def sgd(theta, dp, lr):
    return np.asarray(theta) - lr * np.asarray(dp)


def energy_stats(E):
    E = np.asarray(E, np.float64)
    m = E.mean()
    return m, (E ** 2).mean() - m * m


def split_rhat(chains):
    """chains: (n_chains, L) series.  Split each chain in halves and apply the
    variance-ratio formula of vmc_torch/variational_state.py:574-587."""
    c = np.asarray(chains, np.float64)
    L = c.shape[1] // 2
    sub = np.concatenate([c[:, :L], c[:, L:2 * L]], axis=0)
    means = sub.mean(axis=1)
    Bv = L * np.var(means, ddof=1)
    W = np.mean(np.var(sub, axis=1, ddof=1))
    V = (L - 1) / L * W + Bv / L
    return float(np.sqrt(V / W))


def tau_int(series, c=5.0):
    """Integrated autocorrelation time of a (n_chains, L) set of series,
    averaged autocorrelation over chains, Sokal window M = min{M : M >= c tau(M)}.
    tau = 1/2 + sum_{t=1}^{M} rho(t) (so an uncorrelated chain gives 1/2 ... we
    report 2*tau so that an uncorrelated chain gives 1, the ESS convention)."""
    x = np.asarray(series, np.float64)
    if x.ndim == 1:
        x = x[None]
    x = x - x.mean(axis=1, keepdims=True)
    L = x.shape[1]
    n = 1 << (2 * L - 1).bit_length()
    f = np.fft.rfft(x, n=n, axis=1)
    ac = np.fft.irfft(f * np.conj(f), n=n, axis=1)[:, :L]
    ac = ac.mean(axis=0)
    if ac[0] <= 0:
        return 1.0
    rho = ac / ac[0]
    tau = 1.0
    for M in range(1, L):
        tau = 1.0 + 2.0 * rho[1:M + 1].sum()
        if M >= c * tau:
            break
    return float(max(tau, 1e-12))
