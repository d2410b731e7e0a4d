"""Chain diagnostics on the device: integrated autocorrelation time, effective
sample size and split-chain R-hat.

* tau_int: autocorrelation of each chain's series by FFT, averaged over
  chains, summed with Sokal's automatic window (smallest M with M >= c tau(M),
  c = 5); tau = 1 + 2 sum_{t=1}^{M} rho(t), so an uncorrelated series gives 1.
  (The reference has no tau_int / ESS estimator.)
* ESS = n_chains * n_samples / tau_int.
* split R-hat follows vmc_torch/variational_state.py:574-587 (each chain split
  in two halves; V = (L-1)/L W + B/L; R = sqrt(V / W)).
"""
import torch


def tau_int(series, c=5.0):
    """series: (n_chains, L) tensor (any device)."""
    x = series.double()
    if x.dim() == 1:
        x = x[None]
    x = x - x.mean(dim=1, keepdim=True)
    L = x.shape[1]
    n = 1 << (2 * L - 1).bit_length()
    f = torch.fft.rfft(x, n=n, dim=1)
    ac = torch.fft.irfft(f * f.conj(), n=n, dim=1)[:, :L].mean(dim=0)
    if float(ac[0]) <= 0.0:
        return 1.0
    rho = (ac / ac[0]).cpu()
    tau = 1.0
    for M in range(1, L):
        tau = 1.0 + 2.0 * float(rho[1:M + 1].sum())
        if M >= c * tau:
            break
    return max(tau, 1e-12)


def ess(series, c=5.0):
    x = series if series.dim() == 2 else series[None]
    return x.shape[0] * x.shape[1] / tau_int(x, c)


def split_rhat(series):
    x = series.double()
    L = x.shape[1] // 2
    sub = torch.cat([x[:, :L], x[:, L:2 * L]], dim=0)
    means = sub.mean(dim=1)
    Bv = L * means.var(unbiased=True)
    W = sub.var(dim=1, unbiased=True).mean()
    V = (L - 1) / L * W + Bv / L
    return float(torch.sqrt(V / W))
