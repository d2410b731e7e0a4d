"""Host side of the error contract (no GPU): the oracle's minSR fallback
(vmc_torch/GPU/optimizer.py:557-561) and the reference's gradient-check
message (vmc_torch/GPU/vmc_utils.py:1330-1386) as the Python layer formats it."""
import numpy as np
import pytest
import torch

from oracle import sr


def test_oracle_minsr_solve_and_lstsq_fallback():
    rng = np.random.default_rng(0)
    O = rng.standard_normal((20, 9))
    E = rng.standard_normal(20)
    dp, info = sr.minsr_with_info(O, E, E.mean(), 1e-3)
    assert info == 0
    np.testing.assert_allclose(dp, sr.minsr(O, E, E.mean(), 1e-3))
    # sample 0 equals the column means exactly: T has a zero row and column
    m = np.round(rng.standard_normal(6) * 4) / 4
    d = [np.round(rng.standard_normal(6) * 4) / 4 for _ in range(2)]
    O2 = np.stack([m] + [m + v for v in d] + [m - v for v in d])
    E2 = rng.standard_normal(5)
    dp2, info2 = sr.minsr_with_info(O2, E2, E2.mean(), 0.0)
    assert info2 == 1 and np.isfinite(dp2).all()
    Oc = (O2 - O2.mean(0)) / np.sqrt(5)
    x = np.linalg.pinv(Oc @ Oc.T) @ ((E2 - E2.mean()) / np.sqrt(5))
    np.testing.assert_allclose(dp2, Oc.T @ x, rtol=1e-10, atol=1e-12)


def test_gradient_error_message_names_the_parameters():
    from vmc_torch_gb300 import energy

    class Fake:
        params = [torch.zeros(3, 4), torch.zeros(5), torch.zeros(2, 2)]

    with pytest.raises(ValueError) as e:
        energy._raise_grads(Fake(), 2, 10, [1, 13, 18], 3, 21)
    msg = str(e.value)
    assert msg.startswith("NaN/Inf in gradients: 2/10 samples affected, 3/21 params affected.\nFirst bad params:\n")
    assert "  flat[1] -> params[0][3, 4] offset 1" in msg
    assert "  flat[13] -> params[1][5] offset 1" in msg
    assert "  flat[18] -> params[2][2, 2] offset 1" in msg
