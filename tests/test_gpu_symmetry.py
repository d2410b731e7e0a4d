"""GPU parity of the symmetry-projected model (FermionSymmetryProjectedModel,
vmc_torch/GPU/models/symmetry.py) against the reference's golden vectors and
the oracle.  Images and fermionic signs bit-exact; FP64 projected
log-amplitudes within 1e-10 of the reference; replayed sweeps bit-exact in the
configurations; local energies within 1e-9 relative; projected O within 1e-9."""
import numpy as np
import pytest
import torch

from oracle import hubbard, lattice, models as om, peps, sampler as osampler, symmetry as osym
import vmc_torch_gb300 as vg

pytestmark = pytest.mark.gpu
DEV = "cuda"


def slater(M):
    m = vg.SlaterDeterminant_GB300(M.shape[0], M.shape[1]).to(DEV)
    with torch.no_grad():
        m.params[0].copy_(torch.as_tensor(M))
    m.invalidate()
    return m


@pytest.mark.parametrize("tag,Lx,Ly", [("4x2", 4, 2), ("4x4", 4, 4)])
def test_projection_matches_reference(golden, tag, Lx, Ly):
    g = golden("sym.npz")
    X = g[tag + "_x"].astype(np.int64)
    base = slater(g[tag + "_M"])
    x = torch.as_tensor(X, device=DEV)
    for irrep in ("A1", "A2", "B1", "B2"):
        pm = vg.FermionSymmetryProjectedModel_GB300(base, Lx, Ly, irrep).to(DEV)
        assert np.array_equal(pm.perms.cpu().numpy(), g[tag + "_perms"])
        if irrep == "A1":
            img, fs = pm._images(vg.pack(x))
            G = pm.n_group
            assert np.array_equal(fs.cpu().numpy().reshape(-1, G), g[tag + "_fsign"])
            assert torch.equal(vg.unpack(img, Lx * Ly).reshape(-1, G, Lx * Ly), x[:, pm.perms.long()])
        s, la = pm.forward_log(x)
        assert np.array_equal(s.cpu().numpy(), g[tag + "_" + irrep + "_sign"])
        np.testing.assert_allclose(la.cpu().numpy(), g[tag + "_" + irrep + "_logabs"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("irrep", ["A1", "B2"])
def test_projected_sweep_energy_and_O_vs_oracle(irrep):
    Lx, Ly, nup, B, S = 4, 2, 4, 48, 2
    N = Lx * Ly
    rng = np.random.default_rng(5)
    M = rng.standard_normal((2 * N, 2 * nup))
    perms, chars = osym.group(Lx, Ly)
    amp = lambda y: osym.projected_amp(lambda z: om.slater_amp(M, z), y, perms, chars[irrep])  # noqa: E731

    def logamp(y):
        a = amp(y)
        return np.sign(a), np.log(np.maximum(np.abs(a), 1e-300))

    g = vg.SquareLattice(Lx, Ly)
    E = len(g.sweep_edges())
    X = lattice.random_initial_configs(B, N, nup, nup, seed=6)
    um = rng.random((S, E, B), dtype=np.float32)
    hb = rng.integers(0, 2, (S, E, B)).astype(np.uint8)
    ua = rng.random((S, E, B), dtype=np.float32)
    xo, (so, lo), nacc = osampler.sweep(X, lattice.sweep_edges(Lx, Ly), logamp, um, hb, ua)
    pm = vg.FermionSymmetryProjectedModel_GB300(slater(M), Lx, Ly, irrep).to(DEV)
    fx = torch.as_tensor(X, device=DEV).clone()
    rp = tuple(torch.as_tensor(a, device=DEV).contiguous() for a in (um, hb, ua))
    fx = vg.MetropolisExchangeSpinfulSamplerGB300().burn_in(fx, pm, g, S, replay=rp)
    assert np.array_equal(fx.cpu().numpy(), xo)
    st = pm.bind_state(fx)
    assert np.array_equal(st.sign.cpu().numpy(), so)
    np.testing.assert_allclose(st.logabs.cpu().numpy(), lo, rtol=0, atol=1e-10)
    assert np.array_equal(st.n_acc.cpu().numpy(), nacc)
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, 2 * nup, n_fermions_per_spin=(nup, nup))
    H.precompute_hops_gpu(DEV)
    _, eloc = vg.evaluate_energy(fx, pm, H)
    ref = hubbard.local_energy(xo, lattice.square_edges(Lx, Ly), 1.0, 8.0, amp)
    np.testing.assert_allclose(eloc.cpu().numpy(), ref, rtol=1e-9, atol=1e-9)
    O, _ = vg.compute_grads_gpu(fx, pm, use_log_amp=True)
    Oref = osym.projected_O(lambda z: om.slater_amp(M, z), lambda z: om.slater_O(M, z), xo, perms, chars[irrep])
    np.testing.assert_allclose(O.cpu().numpy(), Oref, rtol=1e-9, atol=1e-10)


def test_projected_variational_energy_4x2():
    """sum |psi_r|^2 E_loc / sum |psi_r|^2 over the 4900-state sector equals
    psi_r^T H psi_r / psi_r^T psi_r."""
    M = np.random.default_rng(8).standard_normal((16, 8))
    pm = vg.FermionSymmetryProjectedModel_GB300(slater(M), 4, 2, "A1").to(DEV)
    S, Hd = hubbard.dense_hamiltonian(8, 4, 4, lattice.square_edges(4, 2), 1.0, 8.0)
    x = torch.as_tensor(S, device=DEV)
    s, la = pm.forward_log(x)
    psi = (s * torch.exp(la)).cpu().numpy()
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(4, 2, 1.0, 8.0, 8, n_fermions_per_spin=(4, 4))
    H.precompute_hops_gpu(DEV)
    _, eloc = vg.evaluate_energy(x, pm, H)
    w = psi ** 2
    np.testing.assert_allclose(float(np.sum(w * eloc.cpu().numpy()) / np.sum(w)), hubbard.exact_energy(psi, Hd),
                               rtol=1e-10)


def test_projected_fpeps_base_4x4():
    """The wrapper over the fPEPS model (C4v on 4x4, D = 2, FP64)."""
    T = peps.init_tensors(4, 4, 2, seed=9)
    base = vg.FPEPS_GB300(4, 4, 2, precision="fp64", dtype=torch.float64, tensors=torch.as_tensor(T)).to(DEV)
    pm = vg.FermionSymmetryProjectedModel_GB300(base, 4, 4, "A1").to(DEV)
    X = lattice.random_initial_configs(16, 16, 4, 4, seed=10)
    s, la = pm.forward_log(torch.as_tensor(X, device=DEV))
    perms, chars = osym.group(4, 4)
    ref = osym.projected_amp(lambda z: np.array([peps.amp_rows(T, v) for v in z]), X, perms, chars["A1"])
    np.testing.assert_allclose((s * torch.exp(la)).cpu().numpy(), ref, rtol=1e-9, atol=1e-12 * np.abs(ref).max())
