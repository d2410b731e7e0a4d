"""Chain diagnostics of the package (device-side torch implementation) against
the oracle's numpy estimator."""
import numpy as np
import torch

from oracle import sr
from vmc_torch_gb300 import stats


def test_tau_int_and_rhat_match_oracle():
    rng = np.random.default_rng(0)
    x = np.zeros((64, 3000))
    e = rng.standard_normal(x.shape)
    for t in range(1, x.shape[1]):
        x[:, t] = 0.7 * x[:, t - 1] + e[:, t]
    x = x[:, 100:]
    assert abs(stats.tau_int(torch.as_tensor(x)) - sr.tau_int(x)) < 1e-9
    assert abs(stats.split_rhat(torch.as_tensor(x)) - sr.split_rhat(x)) < 1e-12
    assert abs(stats.tau_int(torch.as_tensor(x)) - (1 + 0.7) / (1 - 0.7)) < 0.6
