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
carry ~1e-6 / relative gap)."""
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
