"""Slater and neural-backflow amplitudes, log-amplitudes and log-derivatives
(oracle, test-only; FP64).

  * Slater: psi(x) = det(M[occ]) with occ the occupied netket spin-orbitals in
    ASCENDING order (vmc_torch/model.py:7437-7457; GPU form
    vmc_torch/GPU/models/slater.py:40-61 with a stable tie order).
  * NNBF: n = [up | dn]; h = act(h @ w_k^T + b_k) per hidden layer;
    dM = (h @ out_w^T + out_b).reshape(2N, N_f); M = M_base + bf_scale*dM;
    psi = det(M[occ]) (vmc_torch/GPU/models/NNBF.py:113-162).  Parameter order
    [M_base, w_0, b_0, ..., out_w, out_b] (NNBF.py:43-48, 76-111) defines the
    column order of O.
  * log form: sign = sign(psi), log|psi| = log(max(|psi|, 1e-45))
    (vmc_torch/GPU/models/_base.py:101-109).
  * O_k(x) = d log|psi(x)| / d theta_k (vmc_torch/GPU/VMC.py:418-453;
    vmc_torch/GPU/vmc_utils.py:1389-1634).
"""
import math

import numpy as np
import torch

from .lattice import quimb_to_netket


def occupied_rows(x):
    """Ascending occupied netket indices per config: (B, N_f)."""
    nk = quimb_to_netket(np.asarray(x))
    nf = int(nk[0].sum())
    idx = np.argsort(-nk, axis=-1, kind="stable")[..., :nf]
    return np.sort(idx, axis=-1)


def slater_amp(M, x):
    """(B,) amplitudes det(M[occ]) in FP64."""
    M = np.asarray(M, dtype=np.float64)
    rows = occupied_rows(x)
    return np.linalg.det(M[rows])


def slater_logamp(M, x):
    s, l = np.linalg.slogdet(np.asarray(M, np.float64)[occupied_rows(x)])
    return s, l


def slater_O(M, x):
    """(B, 2N*N_f) O rows: dlog|psi|/dM[r, c] = (A^-1)[c, k] when r = occ[k]
    (inverse-transpose adjoint of the determinant; equals the autograd O of
    vmc_torch/GPU/vmc_utils.py:1389-1634 for the Slater model)."""
    M = np.asarray(M, dtype=np.float64)
    rows = occupied_rows(x)
    A = M[rows]
    Ainv = np.linalg.inv(A)
    B = rows.shape[0]
    O = np.zeros((B,) + M.shape)
    for b in range(B):
        O[b, rows[b], :] = Ainv[b].T
    return O.reshape(B, -1)


def gelu_np(z):
    from scipy.special import erf
    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def nnbf_M(params, x, bf_scale, act="gelu"):
    """Configuration-dependent orbitals M(x): (B, 2N, N_f), FP64."""
    M_base = np.asarray(params[0], np.float64)
    nl = (len(params) - 3) // 2
    h = quimb_to_netket(np.asarray(x)).astype(np.float64)
    f = gelu_np if act == "gelu" else np.tanh
    for k in range(nl):
        w = np.asarray(params[1 + 2 * k], np.float64)
        b = np.asarray(params[2 + 2 * k], np.float64)
        h = f(h @ w.T + b)
    out_w = np.asarray(params[-2], np.float64)
    out_b = np.asarray(params[-1], np.float64)
    dM = (h @ out_w.T + out_b).reshape(h.shape[0], *M_base.shape)
    return M_base[None] + bf_scale * dM


def nnbf_logamp(params, x, bf_scale, act="gelu"):
    """(sign, log|psi|) of the NNBF amplitude, FP64, ascending occupied rows."""
    Mx = nnbf_M(params, x, bf_scale, act)
    rows = occupied_rows(x)
    A = np.take_along_axis(Mx, rows[:, :, None], axis=1)
    return np.linalg.slogdet(A)


def nnbf_amp(params, x, bf_scale, act="gelu"):
    s, l = nnbf_logamp(params, x, bf_scale, act)
    return s * np.exp(l)


def _torch_nnbf_logabs(params, x_row, bf_scale, act):
    M_base = params[0]
    nl = (len(params) - 3) // 2
    nk = torch.as_tensor(quimb_to_netket(x_row[None])[0], dtype=torch.float64)
    h = nk
    for k in range(nl):
        z = h @ params[1 + 2 * k].T + params[2 + 2 * k]
        h = torch.nn.functional.gelu(z) if act == "gelu" else torch.tanh(z)
    dM = (h @ params[-2].T + params[-1]).reshape(M_base.shape)
    M = M_base + bf_scale * dM
    rows = torch.as_tensor(occupied_rows(x_row[None])[0])
    return torch.linalg.slogdet(M[rows])[1]


def nnbf_O(params, x, bf_scale, act="gelu", columns=None):
    """(B, Np) FP64 log-derivatives by torch autograd on the CPU (the same
    differentiation the reference performs with torch.func.grad,
    vmc_torch/GPU/vmc_utils.py:1436-1466).  ``columns`` optionally selects a
    subset of flattened parameter indices to keep memory small."""
    tp = [torch.tensor(np.asarray(p), dtype=torch.float64, requires_grad=True) for p in params]
    x = np.asarray(x)
    rows = []
    for b in range(x.shape[0]):
        for p in tp:
            p.grad = None
        la = _torch_nnbf_logabs(tp, x[b], bf_scale, act)
        la.backward()
        g = torch.cat([p.grad.reshape(-1) for p in tp]).numpy()
        rows.append(g if columns is None else g[columns])
    return np.stack(rows)


def nnbf_init(n_sites, n_f, hidden, n_layers, seed, bf_scale_std=None):
    """Seeded FP64 NNBF parameters in reference order: M_base ~ N(0, 0.1^2);
    hidden w ~ N(0, 1/fan_in); biases 0; out_w ~ N(0, 1/fan_in); out_b 0.
    (The workload's stated N(0, 1/fan_in) init; the reference defaults are
    kaiming-uniform hidden / zero output, vmc_torch/GPU/models/NNBF.py:76-111.)"""
    g = np.random.default_rng(seed)
    n_orb = 2 * n_sites
    ps = [g.normal(0.0, 0.1, size=(n_orb, n_f))]
    fan = n_orb
    for _ in range(n_layers):
        ps.append(g.normal(0.0, 1.0 / math.sqrt(fan), size=(hidden, fan)))
        ps.append(np.zeros(hidden))
        fan = hidden
    ps.append(g.normal(0.0, 1.0 / math.sqrt(fan), size=(n_orb * n_f, fan)))
    ps.append(np.zeros(n_orb * n_f))
    return ps


def nnbf_logamp_bf16(params, x, bf_scale):
    """CPU emulation of the GB300 mixed-precision NNBF path: W1, out_w, h1 and
    h2 rounded to BF16, everything else FP32, exact (FP64) determinant of the
    resulting FP32 orbital matrix.  Separates the BF16 quantisation error (a
    property of the mixed path) from kernel errors."""
    def bf16(a):
        return torch.as_tensor(np.asarray(a, np.float32)).to(torch.bfloat16).to(torch.float32).numpy()

    M_base, w0, b0, w1, b1, out_w, out_b = [np.asarray(p, np.float64) for p in params]
    f32 = np.float32
    n = quimb_to_netket(np.asarray(x)).astype(f32)
    z0 = n @ w0.T.astype(f32) + b0.astype(f32)
    h1 = bf16(gelu_np(z0.astype(np.float64)))
    h2 = bf16(gelu_np((h1 @ bf16(w1).T + b1.astype(f32)).astype(np.float64)))
    dM = (h2 @ bf16(out_w).T).astype(f32) + out_b.astype(f32)
    M = M_base.astype(f32)[None] + f32(bf_scale) * dM.reshape(-1, *M_base.shape)
    rows = occupied_rows(x)
    A = np.take_along_axis(M, rows[:, :, None], axis=1).astype(np.float64)
    return np.linalg.slogdet(A)
