"""Hand-written NNBF adjoint O = d log|psi| / d theta.

fp64: against the reference's own autograd O (golden column subset and a
full-row projection) within 1e-9 relative, and against FP64 central finite
differences (h = 1e-6) of the 8x8 backflow model on 64 random walkers within
1e-6 relative plus a roundoff floor of 2e-6 (the FP64 64 x 64 LU carries
~1e-12 of rounding in log|psi| ~ -45, divided by 2h).
mixed (FP32 adjoint): against the FP64 adjoint, per-row relative error
<= 1e-4 median (FP32 Gauss-Jordan inverse; rows near nodes are looser).
The factored output (dense block + Kronecker factors of the out_w block) is
checked against the full rows."""
import hashlib

import numpy as np
import pytest
import torch

from oracle import lattice, models as om
import vmc_torch_gb300 as vg

pytestmark = pytest.mark.gpu
DEV = "cuda"


def make(ps, n_sites, nf, precision):
    m = vg.NNBF_GB300(n_sites, nf, precision=precision).to(DEV)
    with torch.no_grad():
        for p, v in zip(m.params, ps):
            p.copy_(torch.as_tensor(v))
    m.invalidate()
    return m


def grads(m, X):
    st = m._eval_state(torch.as_tensor(X, device=DEV))
    return m.logpsi_grad(st), st


def test_fp64_adjoint_matches_reference_autograd(golden):
    g = golden("nnbf.npz")
    ps = om.nnbf_init(64, 64, 256, 2, seed=int(g["seed"]))
    h = hashlib.sha256()
    for p in ps:
        h.update(np.ascontiguousarray(p, dtype=np.float64).tobytes())
    if h.hexdigest() != str(g["params_sha256"]):
        pytest.skip("numpy normal stream differs from the one that made the fixture")
    m = make(ps, 64, 64, "fp64")
    X = g["x_final"].astype(np.int64)[:4]
    O, _ = grads(m, X)
    O = O.cpu().numpy()
    np.testing.assert_allclose(O[:, g["O_cols"]], g["O_sub"], rtol=1e-9, atol=1e-12)
    r = np.random.default_rng(int(g["proj_seed"])).standard_normal(O.shape[1])
    np.testing.assert_allclose(O @ r, g["O_proj"], rtol=1e-9)


def test_fp64_adjoint_vs_central_finite_differences():
    N, nf, B, h = 64, 64, 64, 1e-6   # 8x8, 32 + 32 electrons, 64 walkers
    ps = om.nnbf_init(N, nf, 256, 2, seed=31)
    X = lattice.random_initial_configs(B, N, nf // 2, nf // 2, seed=32)
    m = make(ps, N, nf, "fp64")
    O, _ = grads(m, X)
    O = O.cpu().numpy()
    xt = torch.as_tensor(X, device=DEV)
    rng = np.random.default_rng(33)
    sizes = [p.numel() for p in m.params]
    offs = np.concatenate([[0], np.cumsum(sizes)])
    checked = 0
    for blk in range(len(sizes)):
        for _ in range(6):
            i = int(rng.integers(sizes[blk]))
            flat = m.params[blk].data.view(-1)
            v0 = float(flat[i])
            vals = []
            for d in (+h, -h):
                flat[i] = v0 + d
                m.invalidate()
                vals.append(m.forward_log(xt)[1].cpu().numpy())
            flat[i] = v0
            m.invalidate()
            fd = (vals[0] - vals[1]) / (2 * h)
            ad = O[:, offs[blk] + i]
            err = np.abs(fd - ad)
            # FD floor: rounding of the FP64 log|psi| (~1e-12) over 2h at h = 1e-6
            assert (err <= 1e-6 * np.abs(ad) + 2e-6).all(), (blk, i, err.max())
            checked += 1
    assert checked == 6 * len(sizes)


def test_mixed_adjoint_vs_fp64_and_factored_form():
    N, nf, B = 64, 64, 48
    ps = om.nnbf_init(N, nf, 256, 2, seed=41)
    X = lattice.random_initial_configs(B, N, 32, 32, seed=42)
    O64, _ = grads(make(ps, N, nf, "fp64"), X)
    mm = make(ps, N, nf, "mixed")
    O32, st = grads(mm, X)
    O64 = O64.cpu().numpy()
    O32 = O32.double().cpu().numpy()
    rel = np.linalg.norm(O32 - O64, axis=1) / np.linalg.norm(O64, axis=1)
    print("mixed adjoint row rel err: median %.2e max %.2e" % (np.median(rel), rel.max()))
    assert np.median(rel) < 1e-4
    assert rel.max() < 1e-1
    Od, kg, kh = mm.logpsi_grad_factored(st)
    Od, kg, kh = Od.double().cpu().numpy(), kg.double().cpu().numpy(), kh.double().cpu().numpy()
    nout = 2 * N * nf
    nw = nout * 256
    ow0 = O32.shape[1] - nout - nw
    full_w = O32[:, ow0:ow0 + nw]
    np.testing.assert_allclose(full_w, (kg[:, :, None] * kh[:, None, :]).reshape(B, -1), rtol=1e-6, atol=1e-12)
    np.testing.assert_array_equal(Od, np.concatenate([O32[:, :ow0], O32[:, ow0 + nw:]], axis=1))


def test_compute_grads_api_contract():
    N, nf, B = 16, 16, 32
    ps = om.nnbf_init(N, nf, 256, 2, seed=51)
    m = make(ps, N, nf, "fp64")
    X = torch.as_tensor(lattice.random_initial_configs(B, N, 8, 8, seed=52), device=DEV)
    O, (s, la) = vg.compute_grads_gpu(X, m, use_log_amp=True)
    g, amps = vg.compute_grads_gpu(X, m)
    np.testing.assert_allclose((g / amps[:, None]).cpu().numpy(), O.cpu().numpy(), rtol=1e-9, atol=1e-12)
    so, lo = om.nnbf_logamp(ps, X.cpu().numpy(), 0.01)
    np.testing.assert_allclose(la.cpu().numpy(), lo, rtol=1e-10, atol=1e-10)
