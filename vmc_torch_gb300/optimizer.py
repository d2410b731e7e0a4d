"""Stochastic reconfiguration in sample space (minSR) and the parameter update,
with the reference's preconditioner / optimizer interfaces
(vmc_torch/GPU/optimizer.py:130-251, 471-614, 884-907).

minSR: O~ = (O - <O>)/sqrt(Ns); T = O~ O~^T + lambda I (Ns x Ns, FP64
accumulation); Cholesky T = L L^T in FP64; x = T^-1 (E - <E>)/sqrt(Ns);
dp = O~^T x.  The reference solves with torch.linalg.solve and falls back to
lstsq (info = 1) when that raises; here a non-positive Cholesky pivot triggers
one retry with the shift raised to 1e-8 * trace(T)/Ns + 10 lambda and info = 1.
"""
import math
import time

import torch

from . import _lib


def _dtype_code(t):
    if t.dtype == torch.float64:
        return 0
    if t.dtype == torch.float32:
        return 1
    raise ValueError("O must be float64 or float32")


class PreconditionerGB300:
    def solve(self, *, local_o, local_energies, energy_mean, total_samples, n_params, diag_shift, device, run_sr):
        raise NotImplementedError


class MinSRGB300(PreconditionerGB300):
    """Drop-in for MinSRGPU.solve (vmc_torch/GPU/optimizer.py:884-907)."""

    def solve(self, *, local_o, local_energies, energy_mean, total_samples, n_params, diag_shift, device=None,
              run_sr=True):
        t0 = time.time()
        dev = torch.device(device) if device is not None else torch.device("cuda")
        O = torch.as_tensor(local_o, device=dev)
        if O.dtype not in (torch.float64, torch.float32):
            O = O.to(torch.float64)
        O = O.contiguous()
        E = torch.as_tensor(local_energies, device=dev, dtype=torch.float64).contiguous()
        Ns, Np = O.shape
        if Np != n_params:
            raise ValueError("local_o has %d columns, n_params is %d" % (Np, n_params))
        s = _lib.stream_of(dev)
        code = _dtype_code(O)
        if not run_sr:
            g = torch.empty(Np, dtype=torch.float64, device=dev)
            _lib.call("vmc_energy_gradient", _lib.ptr(O), code, Ns, Np, O.stride(0), _lib.ptr(E), float(energy_mean),
                      _lib.ptr(g), s)
            return g, time.time() - t0, None
        Oc = torch.empty_like(O)
        mean = torch.empty(Np, dtype=torch.float64, device=dev)
        _lib.call("vmc_sr_center", _lib.ptr(O), code, Ns, Np, O.stride(0), _lib.ptr(Oc), Oc.stride(0),
                  _lib.ptr(mean), s)
        T = torch.empty((Ns, Ns), dtype=torch.float64, device=dev)
        info = 0
        shift = float(diag_shift)
        for attempt in range(2):
            _lib.call("vmc_sr_gram", _lib.ptr(Oc), code, Ns, Np, Oc.stride(0), _lib.ptr(T), Ns, shift, 0, s)
            flag = torch.zeros(1, dtype=torch.int32, device=dev)
            _lib.call("vmc_sr_cholesky", _lib.ptr(T), Ns, Ns, _lib.ptr(flag), s)
            if int(flag.item()) == 0:
                break
            info = 1
            _lib.call("vmc_sr_gram", _lib.ptr(Oc), code, Ns, Np, Oc.stride(0), _lib.ptr(T), Ns, 0.0, 0, s)
            tr = float(torch.diagonal(T).sum().item())
            shift = 10.0 * shift + 1e-8 * tr / Ns
        x = torch.empty(Ns, dtype=torch.float64, device=dev)
        _lib.call("vmc_sr_rhs", _lib.ptr(E), Ns, float(energy_mean), _lib.ptr(x), s)
        _lib.call("vmc_sr_cholesky_solve", _lib.ptr(T), Ns, Ns, _lib.ptr(x), s)
        dp = torch.empty(Np, dtype=torch.float64, device=dev)
        _lib.call("vmc_sr_update", _lib.ptr(Oc), code, Ns, Np, Oc.stride(0), _lib.ptr(x), _lib.ptr(dp), s)
        return dp, time.time() - t0, info


class OptimizerGB300:
    """theta <- compute_update(theta, direction), copied in place per parameter
    (vmc_torch/GPU/optimizer.py:130-176)."""

    def __init__(self, learning_rate=1e-3):
        self.lr = learning_rate

    def compute_update(self, params_vec, direction_vec, learning_rate=None):
        raise NotImplementedError

    @torch.no_grad()
    def step(self, model, direction, device=None, learning_rate=None):
        current = torch.nn.utils.parameters_to_vector(model.parameters())
        d = torch.as_tensor(direction, device=current.device if device is None else device, dtype=current.dtype)
        updated = self.compute_update(current, d, learning_rate)
        off = 0
        for p in model.parameters():
            n = p.numel()
            p.data.copy_(updated[off:off + n].view_as(p.data))
            off += n
        if hasattr(model, "invalidate"):
            model.invalidate()

    def reset(self):
        pass


class SGDGB300(OptimizerGB300):
    """theta - lr * dp (vmc_torch/GPU/optimizer.py:178-186)."""

    def compute_update(self, params_vec, direction_vec, learning_rate=None):
        lr = self.lr if learning_rate is None else learning_rate
        return params_vec - lr * direction_vec
