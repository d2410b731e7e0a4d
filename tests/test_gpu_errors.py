"""Error contract on the GPU, every fault made on the host:

  * non-finite parameters: NaN amplitudes (as the reference's), the sampler
    rejects every NaN ratio, and the gradient functions raise the reference's
    ValueError (vmc_torch/GPU/vmc_utils.py:1330-1386);
  * a rank-deficient orbital matrix and zero-amplitude walkers: sign 0 and
    the reference's log(1e-45) floor, zero log-derivatives (the floor's
    gradient), counted not raised; from a zero amplitude every non-zero
    proposal is accepted, replayed bit for bit against the oracle;
  * minSR when the Cholesky fails: the reference's solve (info 0) and, for an
    exactly singular Gram matrix, its least-squares fallback (info 1)
    (vmc_torch/GPU/optimizer.py:557-561);
  * the bounded device wait: a tensor-core kernel whose operand loads are not
    issued gives up after 1 ms with VMC_ERR_TIMEOUT, and the context stays
    usable;
  * configurations outside the model (a bit at or above n_sites) set the
    device status, and the Python layer raises.
"""
import math

import numpy as np
import pytest
import torch

from oracle import hubbard, lattice, models as om, sampler as osampler, sr
import vmc_torch_gb300 as vg
from vmc_torch_gb300 import _lib, energy

pytestmark = pytest.mark.gpu
DEV = "cuda"
LOG_MIN = math.log(1e-45)


def nnbf(ps, N, nf, precision):
    m = vg.NNBF_GB300(N, nf, precision=precision).to(DEV)
    with torch.no_grad():
        for p, v in zip(m.params, ps):
            p.copy_(torch.as_tensor(v))
    m.invalidate()
    return m


@pytest.mark.parametrize("kind", ["slater", "nnbf-mixed", "nnbf-fp64"])
def test_nan_parameters(kind):
    if kind == "slater":
        N, nup = 8, 4
        M = np.random.default_rng(0).normal(0, 0.1, (16, 8))
        M[:, 5] = np.nan   # a NaN column: every orbital matrix holds NaN
        m = vg.SlaterDeterminant_GB300(16, 8).to(DEV)
        with torch.no_grad():
            m.params[0].copy_(torch.as_tensor(M))
        m.invalidate()
        g = vg.SquareLattice(4, 2)
    else:
        N, nup = 36, 16
        ps = om.nnbf_init(N, 2 * nup, 256, 2, seed=5)
        ps[4][17] = np.nan   # b1
        m = nnbf(ps, N, 2 * nup, "mixed" if kind == "nnbf-mixed" else "fp64")
        g = vg.SquareLattice(6, 6)
    B = 64
    x = vg.init_walkers(B, N, nup, nup, seed=3, device=DEV)
    s, la = m.forward_log(x)
    assert torch.isnan(s).all() and torch.isnan(la).all()
    fx = x.clone()
    fx, _ = vg.MetropolisExchangeSpinfulSamplerGB300(seed=1).step(fx, m, g, use_log_amp=True)
    assert torch.equal(fx, x)          # a NaN ratio never accepts
    with pytest.raises(ValueError, match=r"NaN/Inf in amplitudes: %d NaN, 0 Inf out of %d samples" % (B, B)):
        vg.compute_grads_gpu(fx, m, use_log_amp=True)
    with pytest.raises(ValueError, match=r"NaN/Inf in amplitudes"):
        vg.compute_grads_gpu(fx, m, use_log_amp=False)


def test_rank_deficient_slater_matrix():
    """M with a zero column: every orbital matrix is exactly singular."""
    M = np.random.default_rng(1).normal(0, 0.1, (16, 8))
    M[:, 2] = 0.0
    m = vg.SlaterDeterminant_GB300(16, 8).to(DEV)
    with torch.no_grad():
        m.params[0].copy_(torch.as_tensor(M))
    m.invalidate()
    B = 128
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(4, 2, 1.0, 8.0, 8, n_fermions_per_spin=(4, 4))
    H.precompute_hops_gpu(DEV)
    fx = vg.init_walkers(B, 8, 4, 4, seed=4, device=DEV)
    s, la = m.forward_log(fx)
    assert (s == 0).all() and (la == LOG_MIN).all()
    _, eloc = vg.evaluate_energy(fx, m, H)
    assert m.take_singular_count() >= B
    X = fx.cpu().numpy()
    doublons = (X == 3).sum(axis=1)
    np.testing.assert_allclose(eloc.cpu().numpy(), 8.0 * doublons)
    O, (sg, lg) = vg.compute_grads_gpu(fx, m, use_log_amp=True)
    assert (O == 0).all() and (lg == LOG_MIN).all()
    assert energy.last_check["zero_amplitudes"] == B
    dp, _, info = vg.MinSRGB300().solve(local_o=O, local_energies=eloc, energy_mean=float(eloc.mean()),
                                        total_samples=B, n_params=m.n_params, diag_shift=1e-4, device=DEV, run_sr=True)
    assert info == 0 and (dp == 0).all()


def _zero_orbital(ps, o, nf):
    ps = [p.copy() for p in ps]
    ps[0][o] = 0.0
    ps[-2][o * nf:(o + 1) * nf] = 0.0
    ps[-1][o * nf:(o + 1) * nf] = 0.0
    return ps


def test_zero_amplitude_walkers_fp64_replay():
    """Orbital 0 (spin up at site 0) has an all-zero row: configurations that
    occupy it have amplitude exactly 0.  A zero-amplitude walker accepts every
    proposal with a non-zero amplitude and no walker enters a zero amplitude,
    exactly as the oracle's replay of the reference sampler does; the local
    energy and O of the final walkers match the oracle."""
    Lx, Ly, nup, B, S = 6, 6, 16, 40, 2
    N, nf = Lx * Ly, 2 * nup
    ps = _zero_orbital(om.nnbf_init(N, nf, 256, 2, seed=11), 0, nf)
    m = nnbf(ps, N, nf, "fp64")
    X = lattice.random_initial_configs(B, N, nup, nup, seed=12)
    for b in range(B):   # first half: an up electron on site 0; second half: none there
        want = b < B // 2
        if (X[b, 0] >= 2) != want:
            i = next(i for i in range(1, N) if (X[b, i] >= 2) == want)
            X[b, i] += -2 if want else 2
            X[b, 0] += 2 if want else -2
    assert ((X >= 2).sum(1) == nup).all() and ((X >= 1).sum(1) >= nup).all()
    s0, _ = m.forward_log(torch.as_tensor(X, device=DEV))
    assert (s0[: B // 2] == 0).all() and (s0[B // 2:] != 0).all()
    E = lattice.sweep_edges(Lx, Ly)
    rng = np.random.default_rng(13)
    um = rng.random((S, len(E), B), dtype=np.float32)
    hb = rng.integers(0, 2, (S, len(E), B)).astype(np.uint8)
    ua = rng.random((S, len(E), B), dtype=np.float32)
    xo, (so, lo), _ = osampler.sweep(X, E, lambda y: om.nnbf_logamp(ps, y, 0.01), um, hb, ua)
    fx = torch.as_tensor(X, device=DEV).clone()
    rp = tuple(torch.as_tensor(a, device=DEV).contiguous() for a in (um, hb, ua))
    fx = vg.MetropolisExchangeSpinfulSamplerGB300().burn_in(fx, m, vg.SquareLattice(Lx, Ly), S, replay=rp)
    assert np.array_equal(fx.cpu().numpy(), xo)
    assert (so != 0).sum() >= B // 2 + 10   # most zero-amplitude walkers have moved away
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, nf, n_fermions_per_spin=(nup, nup))
    H.precompute_hops_gpu(DEV)
    _, eloc = vg.evaluate_energy(fx, m, H)
    nz = so != 0
    ref = hubbard.local_energy(xo[nz], lattice.square_edges(Lx, Ly), 1.0, 8.0, lambda y: om.nnbf_amp(ps, y, 0.01))
    np.testing.assert_allclose(eloc.cpu().numpy()[nz], ref, rtol=1e-10, atol=1e-9)
    O, (sg, lg) = vg.compute_grads_gpu(fx, m, use_log_amp=True)
    z = ~nz
    assert (O[torch.as_tensor(z, device=DEV)] == 0).all()
    assert (lg.cpu().numpy()[z] == LOG_MIN).all()


def test_minsr_cholesky_failure_follows_reference():
    rng = np.random.default_rng(21)
    # (a) a negative shift makes T indefinite: the Cholesky fails, the LU solve succeeds (info 0)
    O = rng.standard_normal((40, 30)) * 0.3
    E = rng.standard_normal(40)
    kw = dict(local_energies=torch.as_tensor(E, device=DEV), energy_mean=float(E.mean()), total_samples=40,
              n_params=30, device=DEV, run_sr=True)
    dp, _, info = vg.MinSRGB300().solve(local_o=torch.as_tensor(O, device=DEV), diag_shift=-0.05, **kw)
    ref, rinfo = sr.minsr_with_info(O, E, E.mean(), -0.05)
    assert info == 0 == rinfo
    np.testing.assert_allclose(dp.cpu().numpy(), ref, rtol=1e-8, atol=1e-10)
    # (b) sample 0 equals the mean of O exactly, so its centred row and the Gram
    # matrix's row and column 0 are exactly zero: Cholesky and LU both fail and
    # the least-squares fallback gives the minimum-norm solution (info 1)
    m = np.round(rng.standard_normal(12) * 4) / 4
    d = [np.round(rng.standard_normal(12) * 4) / 4 for _ in range(3)]
    O2 = np.stack([m] + [m + v for v in d] + [m - v for v in d])
    E2 = rng.standard_normal(7)
    kw2 = dict(local_energies=torch.as_tensor(E2, device=DEV), energy_mean=float(E2.mean()), total_samples=7,
               n_params=12, device=DEV, run_sr=True)
    dp2, _, info2 = vg.MinSRGB300().solve(local_o=torch.as_tensor(O2, device=DEV), diag_shift=0.0, **kw2)
    ref2, rinfo2 = sr.minsr_with_info(O2, E2, E2.mean(), 0.0)
    assert info2 == 1 == rinfo2
    np.testing.assert_allclose(dp2.cpu().numpy(), ref2, rtol=1e-8, atol=1e-10)


def _hidden_layer(H1, W1, b1, H2, limit_ns, skip):
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    _lib.call("vmc_nnbf_hidden_layer", _lib.ptr(H1), H1.shape[0], _lib.ptr(W1), _lib.ptr(b1), _lib.ptr(H2),
              int(limit_ns), int(skip), _lib.ptr(err), _lib.stream_of(DEV))
    torch.cuda.synchronize()
    return int(err.item())


def test_bounded_wait_gives_up_and_context_survives():
    g = torch.Generator(device="cpu").manual_seed(3)
    R = 300
    H1 = (torch.randn(R, 256, generator=g) * 0.5).to(torch.bfloat16).to(DEV)
    W1 = (torch.randn(256, 256, generator=g) / 16).to(torch.bfloat16).to(DEV)
    b1 = (torch.randn(256, generator=g) * 0.1).to(DEV)
    H2 = torch.full((R, 256), 3.0, dtype=torch.bfloat16, device=DEV)
    # no operand load is issued: the 1 ms wait runs out, nothing is in flight
    assert _hidden_layer(H1, W1, b1, H2, 1_000_000, 1) == _lib.VMC_ERR_TIMEOUT
    assert (H2 == 3.0).all()
    # the same launch with its loads: the tcgen05 layer against an FP32 torch reference
    assert _hidden_layer(H1, W1, b1, H2, 0, 0) == 0
    ref = torch.nn.functional.gelu(H1.float() @ W1.float().t() + b1)
    np.testing.assert_allclose(H2.float().cpu().numpy(), ref.cpu().numpy(), rtol=1e-2, atol=1e-2)
    # and the rest of the library still runs on this context
    ps = om.nnbf_init(36, 32, 256, 2, seed=6)
    m = nnbf(ps, 36, 32, "mixed")
    X = lattice.random_initial_configs(50, 36, 16, 16, seed=7)
    s, la = m.forward_log(torch.as_tensor(X, device=DEV))
    so, lo = om.nnbf_logamp(ps, X, 0.01)
    assert np.median(np.abs(la.cpu().numpy() - lo)) < 2e-3


def test_occupation_outside_the_lattice_is_reported():
    ps = om.nnbf_init(36, 32, 256, 2, seed=8)
    m = nnbf(ps, 36, 32, "mixed")
    X = lattice.random_initial_configs(20, 36, 16, 16, seed=9)
    occ = vg.pack(torch.as_tensor(X, device=DEV))
    occ[5, 0] |= (1 << 40)   # an up electron on site 40 of a 36-site lattice
    ts, arr = m.net(occ.device)
    R = occ.shape[0]
    z0 = torch.empty((R, 256), dtype=torch.float32, device=DEV)
    H1 = torch.empty((R, 256), dtype=torch.bfloat16, device=DEV)
    H2 = torch.empty_like(H1)
    A = torch.empty((R, 32, 32), dtype=torch.float32, device=DEV)
    sign = torch.empty(R, dtype=torch.float64, device=DEV)
    la = torch.empty_like(sign)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    _lib.call("vmc_nnbf_eval", 0, arr, 36, 32, 256, m.bf_scale, _lib.ptr(occ), R, _lib.ptr(z0), _lib.ptr(H1),
              _lib.ptr(H2), _lib.ptr(A), _lib.ptr(sign), _lib.ptr(la), _lib.ptr(err), _lib.stream_of(DEV))
    torch.cuda.synchronize()
    assert int(err.item()) == _lib.VMC_ERR_ARGS
    # the other rows are unaffected
    so, lo = om.nnbf_logamp(ps, X, 0.01)
    keep = np.arange(R) != 5
    assert np.median(np.abs(la.cpu().numpy()[keep] - lo[keep])) < 2e-3
    # through the model interface the same state raises
    st = m._new_state(R, occ.device)
    st.occ.copy_(occ)
    m._refresh(st, 0)
    with pytest.raises(ValueError, match="status 1"):
        m.check_status(st, wait=True)
