"""GPU parity of the chi-truncated fPEPS kernels (vmc_peps_chi_*) against the
oracle's boundary contraction with max_bond = chi (oracle.peps.amp_state_chi,
equal to the MPS-protocol restatement amp_boundary_chi to 1e-12 in the CPU
tests).  The reference's own contraction (quimb / symmray,
vmc_torch/GPU/models/pureTNS.py:100-111) is not installed, so parity is pinned
to the oracle; at 6x6, D = 4, chi = 16 each side truncates one cut once, so the
result is the unique best rank-16 approximation there whatever the sweep order.

Tolerances: FP64 log-amplitudes within 1e-9 absolute with equal signs, local
energies within 1e-8 relative, replayed sweeps bit-exact in configurations and
acceptance counts; FP32 amplitudes within 5e-6 * |top| |bottom| (the norm
product bounds the final overlap's cancellation; FP32 Jacobi eigenvectors
carry ~1e-7 / relative gap; measured <= 2.4e-7)."""
import numpy as np
import pytest
import torch

from oracle import hubbard, lattice, peps, sampler as osampler
import vmc_torch_gb300 as vg

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _model(Lx, Ly, D, T, chi, precision="fp64"):
    m = vg.FPEPS_GB300(Lx, Ly, D, max_bond=chi, precision=precision, tensors=torch.as_tensor(T),
                       dtype=torch.float64 if precision == "fp64" else torch.float32).to(DEV)
    assert m.truncated
    return m


# (Lx, Ly, D, chi, n_up, walkers): one truncated cut (4x4 chi 8, 6x6 chi 16, 8x6 chi 16), several per row
# (6x6 chi 8, 4x6 chi 8, 8x8 D=2 chi 4), a chi below the first row's bond (4x4 chi 3)
CASES = [(4, 4, 4, 8, 4, 48), (6, 6, 4, 16, 16, 16), (6, 6, 4, 8, 16, 16), (4, 6, 4, 8, 6, 24),
         (6, 4, 4, 8, 6, 24), (8, 8, 2, 4, 28, 16), (4, 4, 4, 3, 4, 32), (8, 6, 4, 16, 22, 8)]


@pytest.mark.parametrize("Lx,Ly,D,chi,nup,B", CASES)
def test_chi_eval_fp64_vs_oracle(Lx, Ly, D, chi, nup, B):
    T = peps.init_tensors(Lx, Ly, D, seed=Lx * 10 + Ly + chi)
    X = lattice.random_initial_configs(B, Lx * Ly, nup, nup, seed=chi)
    m = _model(Lx, Ly, D, T, chi)
    s, la = m.forward_log(torch.as_tensor(X, device=DEV))
    so, lo = peps.logamp(T, X, "chi", chi=chi)
    ob = np.array([peps.amp_boundary_chi(T, x, chi) for x in X[:4]])
    np.testing.assert_allclose(so[:4] * np.exp(lo[:4]), ob, rtol=1e-10)
    assert np.array_equal(s.cpu().numpy(), so)
    np.testing.assert_allclose(la.cpu().numpy(), lo, rtol=0, atol=1e-9)


@pytest.mark.parametrize("Lx,Ly,D,chi,nup,B", [(6, 6, 4, 16, 16, 64), (4, 4, 4, 8, 4, 64), (6, 6, 4, 8, 16, 32)])
def test_chi_eval_fp32_vs_oracle(Lx, Ly, D, chi, nup, B):
    T = peps.init_tensors(Lx, Ly, D, seed=5)
    X = lattice.random_initial_configs(B, Lx * Ly, nup, nup, seed=6)
    m = _model(Lx, Ly, D, T, chi, precision="fp32")
    s, la = m.forward_log(torch.as_tensor(X, device=DEV))
    psi = s.cpu().numpy() * np.exp(la.cpu().numpy())
    T32 = T.astype(np.float32).astype(np.float64)
    errs = []
    for k, x in enumerate(X):
        ref, scale = peps.amp_state_chi(T32, x, chi, with_norms=True)
        errs.append(abs(psi[k] - ref) / scale)
    print("%dx%d D=%d chi=%d FP32: max |dpsi| / (|top||bot|) = %.2e, median %.2e"
          % (Lx, Ly, D, chi, max(errs), np.median(errs)))
    assert max(errs) <= 5e-6


def test_chi_large_matches_exact_path():
    """max_bond >= D^(Lx/2) never truncates: the model takes the exact kernels,
    and the chi kernels with a bond that only the schedule's last row
    truncates agree with the oracle's exact contraction when chi reaches the
    full rank."""
    T = peps.init_tensors(6, 6, 4, seed=2)
    X = lattice.random_initial_configs(16, 36, 16, 16, seed=3)
    m = vg.FPEPS_GB300(6, 6, 4, max_bond=64, precision="fp64", tensors=torch.as_tensor(T),
                       dtype=torch.float64).to(DEV)
    assert not m.truncated
    s, la = m.forward_log(torch.as_tensor(X, device=DEV))
    so, lo = peps.logamp(T, X, "rows")
    assert np.array_equal(s.cpu().numpy(), so)
    np.testing.assert_allclose(la.cpu().numpy(), lo, rtol=0, atol=1e-10)


@pytest.mark.parametrize("Lx,Ly,D,chi,nup,B,S", [(4, 4, 4, 8, 4, 48, 2), (6, 6, 4, 16, 16, 8, 1),
                                                 (6, 4, 4, 8, 6, 24, 1)])
def test_chi_sweep_vs_oracle_replay(Lx, Ly, D, chi, nup, B, S):
    N = Lx * Ly
    rng = np.random.default_rng(N + chi)
    T = peps.init_tensors(Lx, Ly, D, seed=N)
    edges = lattice.sweep_edges(Lx, Ly)
    E = len(edges)
    X = lattice.random_initial_configs(B, N, nup, nup, seed=N + 1)
    um = rng.random((S, E, B), dtype=np.float32)
    hb = rng.integers(0, 2, (S, E, B)).astype(np.uint8)
    ua = rng.random((S, E, B), dtype=np.float32)
    xo, (so, lo), nacc = osampler.sweep(X, edges, lambda y: peps.logamp(T, y, "chi", chi=chi), um, hb, ua)
    m = _model(Lx, Ly, D, T, chi)
    m.chi_rows = max(B // 3, 1)   # several walker chunks
    smp = vg.MetropolisExchangeSpinfulSamplerGB300()
    fx = torch.as_tensor(X, device=DEV).clone()
    rp = tuple(torch.as_tensor(a, device=DEV).contiguous() for a in (um, hb, ua))
    fx = smp.burn_in(fx, m, vg.SquareLattice(Lx, Ly), S, replay=rp)
    assert np.array_equal(fx.cpu().numpy(), xo)
    st = m.bind_state(fx)
    assert np.array_equal(st.sign.cpu().numpy(), so)
    np.testing.assert_allclose(st.logabs.cpu().numpy(), lo, rtol=0, atol=1e-9)
    assert np.array_equal(st.n_acc.cpu().numpy(), nacc)


@pytest.mark.parametrize("Lx,Ly,D,chi,nup,B", [(4, 4, 4, 8, 4, 24), (6, 6, 4, 16, 16, 4)])
def test_chi_local_energy_vs_oracle(Lx, Ly, D, chi, nup, B):
    T = peps.init_tensors(Lx, Ly, D, seed=9)
    X = lattice.random_initial_configs(B, Lx * Ly, nup, nup, seed=10)
    m = _model(Lx, Ly, D, T, chi)
    m.chi_rows = 5   # walker chunks and hop-term blocks smaller than one walker's terms
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, 2 * nup, n_fermions_per_spin=(nup, nup))
    H.precompute_hops_gpu(DEV)
    _, eloc = vg.evaluate_energy(torch.as_tensor(X, device=DEV), m, H)
    ref = hubbard.local_energy(X, lattice.square_edges(Lx, Ly), 1.0, 8.0,
                               lambda y: np.array([peps.amp_state_chi(T, v, chi) for v in y]))
    np.testing.assert_allclose(eloc.cpu().numpy(), ref, rtol=1e-8, atol=1e-8)


def _chi_O_oracle(T, X, chi):
    Lx, Ly, _, D = T.shape[:4]
    return np.stack([peps.logamp_grad_chi(T, x, chi).reshape(-1) for x in X])


def test_chi_logpsi_grad_fp64_vs_autograd():
    """O through the truncation against torch autograd of the oracle's
    truncated contraction (torch.linalg.svd, as the reference differentiates
    its quimb contraction)."""
    Lx, Ly, D, chi = 4, 4, 4, 8
    T = peps.init_tensors(Lx, Ly, D, seed=12)
    X = lattice.random_initial_configs(12, Lx * Ly, 4, 4, seed=13)
    m = _model(Lx, Ly, D, T, chi)
    st = m.bind_state(torch.as_tensor(X, device=DEV))
    O = m.logpsi_grad(st, work_rows=5).cpu().numpy()
    ref = _chi_O_oracle(T, X, chi)
    err = np.abs(O - ref).max(axis=1) / np.abs(ref).max(axis=1)
    print("4x4 chi=8 FP64 O: max row error / max|O| = %.2e" % err.max())
    assert err.max() < 1e-8
    assert np.array_equal(O != 0, ref != 0) or np.abs(O[(O != 0) != (ref != 0)]).max() < 1e-12


def test_chi_logpsi_grad_fp32_6x6():
    Lx, Ly, D, chi = 6, 6, 4, 16
    T = peps.init_tensors(Lx, Ly, D, seed=14)
    X = lattice.random_initial_configs(6, Lx * Ly, 16, 16, seed=15)
    m = _model(Lx, Ly, D, T, chi, precision="fp32")
    st = m.bind_state(torch.as_tensor(X, device=DEV))
    O = m.logpsi_grad(st).double().cpu().numpy()
    ref = _chi_O_oracle(T.astype(np.float32).astype(np.float64), X, chi)
    rel = np.linalg.norm(O - ref, axis=1) / np.linalg.norm(ref, axis=1)
    print("6x6 chi=16 FP32 O: |dO| / |O| per walker: max %.2e median %.2e" % (rel.max(), np.median(rel)))
    assert rel.max() < 1e-3


def test_chi_logpsi_grad_euler_identity_at_scale():
    """psi is homogeneous of degree 1 in every site tensor (each row enters
    the boundary linearly and the rank-chi truncation is homogeneous), so for
    every walker and site sum_e T_e d log|psi| / d T_e = 1: a check at the
    benchmark's size (6x6, chi = 16, FP32, 2048 walkers)."""
    Lx, Ly, D, chi, B = 6, 6, 4, 16, 2048
    m = vg.FPEPS_GB300(Lx, Ly, D, max_bond=chi, generator=torch.Generator().manual_seed(5)).to(DEV)
    fx = vg.init_walkers(B, Lx * Ly, 16, 16, seed=3, device=DEV)
    st = m.bind_state(fx)
    O = m.logpsi_grad(st)
    Tf = m.params[0].detach().float().reshape(1, Lx * Ly, 4 * D ** 4)
    per_site = (O.reshape(B, Lx * Ly, 4 * D ** 4) * Tf).sum(-1).double()
    dev = (per_site - 1).abs()
    print("Euler identity, 2048 walkers x 36 sites: max |sum - 1| = %.2e, median %.2e"
          % (dev.max().item(), dev.median().item()))
    assert torch.isfinite(O).all()
    assert dev.median().item() < 1e-4 and dev.max().item() < 1e-2


def test_chi_sr_steps_run():
    """Two SR steps of the 6x6 chi = 16 model through VMC_GB300: sampling,
    local energies, O through the truncation, minSR."""
    Lx, Ly, B = 6, 6, 512
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, 32, n_fermions_per_spin=(16, 16))
    H.precompute_hops_gpu(DEV)
    m = vg.FPEPS_GB300(Lx, Ly, 4, max_bond=16, generator=torch.Generator().manual_seed(2), init_std=0.5).to(DEV)
    fx = vg.init_walkers(B, Lx * Ly, 16, 16, seed=4, device=DEV)
    cfg = vg.VMCLoopConfig(vmc_steps=2, ns_per_rank=B, grad_batch_size=256, n_params=m.n_params, nsites=Lx * Ly,
                           learning_rate=0.01, diag_shift=1e-3, burn_in_steps=2)
    drv = vg.VMC_GB300(vg.MetropolisExchangeSpinfulSamplerGB300(seed=3), vg.MinSRGB300(), vg.SGDGB300(0.01))
    hist, fx = drv.run_vmc_loop(fx, m, H, H.graph, 0, 1, cfg)
    print("6x6 chi=16 SR energies per site:", np.round(hist, 5))
    assert len(hist) == 2 and all(np.isfinite(hist))
