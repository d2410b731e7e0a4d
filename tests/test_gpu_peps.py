"""GPU parity of the fPEPS kernels against the oracle (exact contraction with
the Grassmann sign rule).  Tolerances: configurations and signs bit-exact;
FP64 log-amplitudes within 1e-10 absolute and local energies within 1e-9
relative; FP32 amplitudes within 2e-6 * kappa relative, kappa = (contraction
of |T~|) / |psi| the cancellation condition number of the contraction."""
import math

import numpy as np
import pytest
import torch

from oracle import hubbard, lattice, peps, sampler as osampler
import vmc_torch_gb300 as vg

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _model(Lx, Ly, D, T, precision="fp64", env=True, env_rows=2048):
    return vg.FPEPS_GB300(Lx, Ly, D, precision=precision, tensors=torch.as_tensor(T),
                          dtype=torch.float64 if precision == "fp64" else torch.float32, env_reuse=env,
                          env_rows=env_rows).to(DEV)


def _oracle_logamp(T, X):
    return peps.logamp(T, X, "rows")


SHAPES = [(4, 2, 4, 2, 2, 64), (4, 3, 2, 3, 3, 64), (6, 4, 2, 6, 6, 48), (8, 4, 2, 8, 8, 24),
          (6, 6, 4, 16, 16, 24), (4, 4, 4, 4, 4, 32)]


@pytest.mark.parametrize("Lx,Ly,D,nup,ndn,B", SHAPES)
def test_peps_eval_fp64_vs_oracle(Lx, Ly, D, nup, ndn, B):
    T = peps.init_tensors(Lx, Ly, D, seed=Lx * 10 + Ly)
    X = lattice.random_initial_configs(B, Lx * Ly, nup, ndn, seed=D)
    m = _model(Lx, Ly, D, T)
    s, la = m.forward_log(torch.as_tensor(X, device=DEV))
    so, lo = _oracle_logamp(T, X)
    assert np.array_equal(s.cpu().numpy(), so)
    np.testing.assert_allclose(la.cpu().numpy(), lo, rtol=0, atol=1e-10)


@pytest.mark.parametrize("Lx,Ly,D,nup,ndn,B", [(6, 6, 4, 16, 16, 64), (4, 4, 4, 4, 4, 64), (6, 4, 2, 6, 6, 64)])
def test_peps_eval_fp32_vs_oracle(Lx, Ly, D, nup, ndn, B):
    T = peps.init_tensors(Lx, Ly, D, seed=7)
    X = lattice.random_initial_configs(B, Lx * Ly, nup, ndn, seed=8)
    m = _model(Lx, Ly, D, T, precision="fp32")
    s, la = m.forward_log(torch.as_tensor(X, device=DEV))
    psi = s.cpu().numpy() * np.exp(la.cpu().numpy())
    for k, x in enumerate(X):
        g, A = peps.sign_rule(T.astype(np.float32).astype(np.float64), x)
        ref = g * peps.amp_rows_signed(A)
        kappa = peps.amp_rows_signed(np.abs(A)) / abs(ref)
        assert abs(psi[k] - ref) <= 2e-6 * kappa * abs(ref), (k, psi[k], ref, kappa)


def test_peps_zero_amplitude():
    T = peps.init_tensors(4, 2, 4, seed=1)
    X = lattice.random_initial_configs(4, 8, 3, 2, seed=1)  # odd electron number: psi = 0
    s, la = _model(4, 2, 4, T).forward_log(torch.as_tensor(X, device=DEV))
    # zero amplitude: sign 0 and the reference's log(1e-45) floor (vmc_torch/GPU/models/_base.py:101-109)
    assert torch.all(s == 0) and torch.all(la == math.log(1e-45))


class _Shuffled:
    """A graph whose sweep visits the nearest-neighbour edges in a fixed random order."""

    def __init__(self, edges):
        self.edges = edges

    def device_edges(self, device, kind):
        return torch.tensor(self.edges, dtype=torch.int32, device=device).reshape(-1, 2)


@pytest.mark.parametrize("env", [True, False])
@pytest.mark.parametrize("Lx,Ly,D,nup,B,S,order", [(4, 2, 4, 2, 64, 3, "sweep"), (6, 4, 2, 6, 32, 2, "sweep"),
                                                   (6, 6, 4, 16, 6, 1, "sweep"), (6, 4, 2, 6, 24, 2, "shuffled"),
                                                   (4, 3, 4, 3, 24, 2, "shuffled")])
def test_peps_sweep_vs_oracle_replay(Lx, Ly, D, nup, B, S, order, env):
    N = Lx * Ly
    rng = np.random.default_rng(N)
    T = peps.init_tensors(Lx, Ly, D, seed=N)
    edges = lattice.sweep_edges(Lx, Ly)
    if order == "shuffled":  # arbitrary visiting order (and pair orientation) exercises the cache validity logic
        perm = rng.permutation(len(edges))
        edges = [edges[k] if k % 2 else edges[k][::-1] for k in perm]
        g = _Shuffled(edges)
    else:
        g = vg.SquareLattice(Lx, Ly)
    E = len(edges)
    X = lattice.random_initial_configs(B, N, nup, nup, seed=N + 1)
    um = rng.random((S, E, B), dtype=np.float32)
    hb = rng.integers(0, 2, (S, E, B)).astype(np.uint8)
    ua = rng.random((S, E, B), dtype=np.float32)
    xo, (so, lo), nacc = osampler.sweep(X, edges, lambda y: _oracle_logamp(T, y), um, hb, ua)
    m = _model(Lx, Ly, D, T, env=env, env_rows=max(B // 3, 1))
    smp = vg.MetropolisExchangeSpinfulSamplerGB300()
    fx = torch.as_tensor(X, device=DEV).clone()
    rp = tuple(torch.as_tensor(a, device=DEV).contiguous() for a in (um, hb, ua))
    fx = smp.burn_in(fx, m, g, S, replay=rp)
    assert np.array_equal(fx.cpu().numpy(), xo)
    st = m.bind_state(fx)
    assert np.array_equal(st.sign.cpu().numpy(), so)
    np.testing.assert_allclose(st.logabs.cpu().numpy(), lo, rtol=0, atol=1e-10)
    assert np.array_equal(st.n_acc.cpu().numpy(), nacc)
    # local energy at the final configurations
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, 2 * nup, n_fermions_per_spin=(nup, nup))
    H.precompute_hops_gpu(DEV)
    _, eloc = vg.evaluate_energy(fx, m, H)
    ref = hubbard.local_energy(xo, lattice.square_edges(Lx, Ly), 1.0, 8.0,
                               lambda y: np.array([peps.amp_rows(T, v) for v in y]))
    np.testing.assert_allclose(eloc.cpu().numpy(), ref, rtol=1e-9, atol=1e-9)


def test_peps_variational_energy_4x2():
    """Sum_x |psi|^2 E_loc(x) / Sum_x |psi|^2 over the whole sector equals
    psi^T H psi / psi^T psi with the dense Hamiltonian."""
    Lx, Ly, D = 4, 2, 4
    T = peps.init_tensors(Lx, Ly, D, seed=11)
    S, Hd = hubbard.dense_hamiltonian(8, 4, 4, lattice.square_edges(Lx, Ly), 1.0, 8.0)
    m = _model(Lx, Ly, D, T)
    x = torch.as_tensor(S, device=DEV)
    s, la = m.forward_log(x)
    psi = (s * torch.exp(la)).cpu().numpy()
    np.testing.assert_allclose(psi, [peps.amp_rows(T, v) for v in S], rtol=1e-10, atol=1e-300)
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, 8, n_fermions_per_spin=(4, 4))
    H.precompute_hops_gpu(DEV)
    _, eloc = vg.evaluate_energy(x, m, H)
    w = psi ** 2
    np.testing.assert_allclose(float(np.sum(w * eloc.cpu().numpy()) / np.sum(w)), hubbard.exact_energy(psi, Hd),
                               rtol=1e-10)


def test_peps_fp32_sweep_consistent():
    """Philox sweeps in FP32 at 6x6, D = 4: the carried log-amplitudes (from the
    cached environments) agree with a fresh evaluation of the final
    configurations, and moves are accepted."""
    m = vg.FPEPS_GB300(6, 6, 4, generator=torch.Generator().manual_seed(0)).to(DEV)
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(6, 6, 1.0, 8.0, 32, n_fermions_per_spin=(16, 16))
    H.precompute_hops_gpu(DEV)
    fx = vg.init_walkers(128, 36, 16, 16, seed=3, device=DEV)
    smp = vg.MetropolisExchangeSpinfulSamplerGB300(seed=5)
    fx, (s, la) = smp.step(fx, m, H.graph, use_log_amp=True)
    s2, la2 = m.forward_log(fx)
    assert torch.equal(s, s2)
    torch.testing.assert_close(la, la2, rtol=0, atol=2e-4)  # environment contraction vs a fresh sweep, FP32
    st = m.bind_state(fx)
    assert int(st.n_acc.sum()) > 0
    E, eloc = vg.evaluate_energy(fx, m, H)
    assert torch.isfinite(eloc).all()


@pytest.mark.parametrize("Lx,Ly,D,nup,B", [(4, 2, 4, 2, 16), (4, 3, 2, 3, 12), (6, 4, 2, 6, 6), (6, 6, 4, 16, 3)])
def test_peps_logpsi_grad_fp64_vs_oracle(Lx, Ly, D, nup, B):
    T = peps.init_tensors(Lx, Ly, D, seed=Lx + Ly)
    X = lattice.random_initial_configs(B, Lx * Ly, nup, nup, seed=3)
    m = _model(Lx, Ly, D, T)
    O, _ = vg.compute_grads_gpu(torch.as_tensor(X, device=DEV), m, use_log_amp=True)
    O = O.cpu().numpy()
    for k, x in enumerate(X):
        ref = peps.logamp_grad(T, x).reshape(-1)
        np.testing.assert_allclose(O[k], ref, rtol=1e-9, atol=1e-11 * np.abs(ref).max())


def test_peps_logpsi_grad_fp32_6x6():
    """FP32 adjoint at 6x6, D = 4 against the FP64 adjoint on the same walkers
    (row-wise relative error), with a chunked workspace."""
    T = peps.init_tensors(6, 6, 4, seed=21)
    X = torch.as_tensor(lattice.random_initial_configs(40, 36, 16, 16, seed=22), device=DEV)
    m64 = _model(6, 6, 4, T)
    m32 = _model(6, 6, 4, T.astype(np.float32).astype(np.float64), precision="fp32")
    O64 = m64.logpsi_grad(m64.bind_state(X)).cpu().numpy()
    O32 = m32.logpsi_grad(m32.bind_state(X), work_rows=16).double().cpu().numpy()
    rel = np.linalg.norm(O32 - O64, axis=1) / np.linalg.norm(O64, axis=1)
    assert np.median(rel) < 1e-4 and rel.max() < 1e-2, rel


def test_peps_vmc_4x2_energy():
    """A short fPEPS VMC run (4x2, D = 2, minSR): the energy goes down and the
    final MC estimate agrees with the exact <H> of the final tensors."""
    gen = torch.Generator().manual_seed(1)
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(4, 2, 1.0, 8.0, 8, n_fermions_per_spin=(4, 4))
    H.precompute_hops_gpu(DEV)
    model = vg.FPEPS_GB300(4, 2, 2, precision="fp64", dtype=torch.float64, init_std=0.5, generator=gen).to(DEV)
    smp = vg.MetropolisExchangeSpinfulSamplerGB300(seed=3, sweeps_per_step=2)
    fx = vg.init_walkers(1024, 8, 4, 4, seed=4)
    cfg = vg.VMCLoopConfig(vmc_steps=30, ns_per_rank=1024, grad_batch_size=1024, n_params=model.n_params, nsites=8,
                           learning_rate=0.05, diag_shift=1e-3, burn_in_steps=20, outlier_clip_factor=0.0)
    drv = vg.VMC_GB300(smp, vg.MinSRGB300(), vg.SGDGB300(0.05))
    seen = []
    hist, fx = drv.run_vmc_loop(fx, model, H, H.graph, 0, 1, cfg, on_step_end=lambda info: seen.append(info))
    assert [i["step"] for i in seen] == list(range(30)) and seen[-1]["fxs"] is fx
    assert {"energy_mean", "energy_var", "energy_per_site", "error_per_site", "total_samples"} <= set(seen[0])
    assert hist[-1] < hist[0] - 0.3 / 8
    S, Hd = hubbard.dense_hamiltonian(8, 4, 4, lattice.square_edges(4, 2), 1.0, 8.0)
    s, la = model.forward_log(torch.as_tensor(S, device=DEV))
    Eex = hubbard.exact_energy((s * torch.exp(la)).cpu().numpy(), Hd)
    for _ in range(10):
        fx, _ = smp.step(fx, model, H.graph)
    _, eloc = vg.evaluate_energy(fx, model, H)
    e = eloc.cpu().numpy()
    assert abs(e.mean() - Eex) < 5 * e.std() / np.sqrt(len(e)) + 0.05


def test_peps_fp32_env_matches_recompute():
    """FP32 at 6x6, D = 4 (the register-tiled path): sweeps with environment
    reuse follow the same chains as full recomputation (acceptance decisions
    agree except within FP32 rounding of the ratio) and give the same local
    energies to 1e-4 relative on identical configurations."""
    T = peps.init_tensors(6, 6, 4, seed=31)
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(6, 6, 1.0, 8.0, 32, n_fermions_per_spin=(16, 16))
    H.precompute_hops_gpu(DEV)
    x0 = vg.init_walkers(96, 36, 16, 16, seed=6, device=DEV)
    out = []
    for env in (True, False):
        m = _model(6, 6, 4, T.astype(np.float32).astype(np.float64), precision="fp32", env=env, env_rows=40)
        fx = x0.clone()
        fx, _ = vg.MetropolisExchangeSpinfulSamplerGB300(seed=9, sweeps_per_step=2).step(fx, m, H.graph)
        out.append((m, fx))
    same = (out[0][1] == out[1][1]).all(dim=1)
    assert same.double().mean().item() >= 0.95
    x = out[1][1]
    e_env = vg.evaluate_energy(x.clone(), out[0][0], H)[1]
    e_full = vg.evaluate_energy(x.clone(), out[1][0], H)[1]
    torch.testing.assert_close(e_env, e_full, rtol=1e-4, atol=1e-4)
