"""minSR with the Kronecker-factored NNBF output block against the dense
formulation and the FP64 oracle.  fp64: factored == dense == oracle within
1e-8 relative (norm); mixed (FP32 O, FP64 Gram accumulation / Cholesky):
within 2e-3 relative of the FP64 direction."""
import numpy as np
import pytest
import torch

from oracle import lattice, models as om, sr
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


def setup(precision, Ns=256, seed=61, N=16, nf=16):
    ps = om.nnbf_init(N, nf, 256, 2, seed=seed)
    m = make(ps, N, nf, precision)
    X = torch.as_tensor(lattice.random_initial_configs(Ns, N, nf // 2, nf // 2, seed=seed + 1), device=DEV)
    E = torch.as_tensor(np.random.default_rng(seed + 2).standard_normal(Ns) - 3.0, device=DEV)
    return m, X, E


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("run_sr", [True, False])
def test_factored_minsr_equals_dense_and_oracle_fp64(run_sr):
    m, X, E = setup("fp64")
    Ns = X.shape[0]
    O, _ = vg.compute_grads_gpu(X, m, use_log_amp=True)
    F, _ = vg.compute_grads_factored(X, m)
    np.testing.assert_allclose(F.full().cpu().numpy(), O.cpu().numpy(), rtol=1e-12, atol=1e-14)
    kw = dict(local_energies=E, energy_mean=float(E.mean()), total_samples=Ns, n_params=m.n_params,
              diag_shift=1e-3, device=DEV, run_sr=run_sr)
    solver = vg.MinSRGB300()
    dp_d, _, _ = solver.solve(local_o=O, **kw)
    dp_f, _, _ = solver.solve(local_o=F, **kw)
    On, En = O.cpu().numpy(), E.cpu().numpy()
    ref = sr.minsr(On, En, En.mean(), 1e-3) if run_sr else sr.energy_gradient(On, En, En.mean())
    assert rel(dp_f.cpu().numpy(), ref) < 1e-8
    assert rel(dp_d.cpu().numpy(), ref) < 1e-8


def test_factored_minsr_mixed_precision_vs_fp64():
    m64, X, E = setup("fp64", N=36, nf=32)   # the mixed forward path needs nf in {32, 64}
    Ns = X.shape[0]
    kw = dict(local_energies=E, energy_mean=float(E.mean()), total_samples=Ns, n_params=m64.n_params,
              diag_shift=1e-3, device=DEV, run_sr=True)
    F64, _ = vg.compute_grads_factored(X, m64)
    dp64, _, _ = vg.MinSRGB300().solve(local_o=F64, **kw)
    m32, _, _ = setup("mixed", N=36, nf=32)
    F32, _ = vg.compute_grads_factored(X, m32)
    assert F32.dense.dtype == torch.float32
    dp32, _, info = vg.MinSRGB300().solve(local_o=F32, **kw)
    r = rel(dp32.cpu().numpy(), dp64.cpu().numpy())
    print("mixed factored minSR direction rel err %.2e" % r)
    assert info == 0 and r < 2e-3


def test_tensor_core_gram_is_exact_on_digit_representable_rows():
    """Rows whose entries are 7-bit integers times 2^-6 times a power of two
    per row are represented exactly by the fixed-point split (one non-zero
    digit), and the leading products are then summed exactly in FP32 and
    FP64: the tensor-core Gram equals the FP64 Gram bit for bit."""
    from vmc_torch_gb300 import _lib
    Ns, K = 300, 5000
    g = torch.Generator().manual_seed(1)
    ints = torch.randint(-64, 65, (Ns, K), generator=g).double()
    ints[:, 0] = 64.0                               # row max exactly 1 after scaling: E_i fixed
    scale = torch.pow(2.0, torch.randint(-8, 9, (Ns, 1), generator=g).double())
    Xd = ints * 2.0 ** -6 * scale * 0.5             # max |x| = 2^(e-1): E_i = e
    X = Xd.float().to(DEV)
    T = torch.empty((Ns, Ns), dtype=torch.float64, device=DEV)
    solver = vg.MinSRGB300(gram="tensor")
    solver._tc_gram(X, T, 1.0, None, 0.0, 0, DEV)
    solver._check_tc()
    ref = (Xd @ Xd.t()).to(DEV)
    assert torch.equal(T, ref)


@pytest.mark.parametrize("Ns,K", [(700, 3000), (256, 115200 // 16), (4096, 16384)])
def test_tensor_core_gram_matches_compensated_fp32(Ns, K):
    """vmc_sr_gram_tc (fixed-point 7-bit digits under a per-row exponent, nine
    products on tcgen05, the leading one summed exactly, drained into FP64)
    against the CUDA-core Gram with double-float accumulation (FP64-level) on
    the same FP32 matrix: entries within 2e-6 of the largest diagonal entry
    (the digits round each row to 2^-20 of its largest entry), also with the
    elementwise factor D and accumulation used by the Kronecker head."""
    from vmc_torch_gb300 import _lib
    g = torch.Generator().manual_seed(Ns)
    X = (torch.randn(Ns, K, generator=g) * 0.3 + 0.05).float().to(DEV)
    s = _lib.stream_of(DEV)
    T_ref = torch.empty((Ns, Ns), dtype=torch.float64, device=DEV)
    _lib.call("vmc_sr_gram", _lib.ptr(X), 1, Ns, K, X.stride(0), _lib.ptr(T_ref), Ns, 1e-3, 0, s)
    solver = vg.MinSRGB300()
    T = torch.full((Ns, Ns), 7.0, dtype=torch.float64, device=DEV)
    solver._tc_gram(X, T, 1.0, None, 1e-3, 0, DEV)
    solver._check_tc()
    scale = T_ref.diagonal().abs().max().item()
    err = (T - T_ref).abs().max().item() / scale
    print("tensor-core Gram (%d x %d): max rel err %.2e" % (Ns, K, err))
    assert err < 2e-6
    assert torch.equal(T, T.t())
    # head form: T += alpha (X X^T) o D
    D = torch.rand((Ns, Ns), generator=g, dtype=torch.float64).to(DEV)
    D = D + D.t()
    T2 = T.clone()
    solver._tc_gram(X, T2, 0.5, D, 0.0, 1, DEV)
    ref2 = T_ref + 0.5 * (T_ref - 1e-3 * torch.eye(Ns, dtype=torch.float64, device=DEV)) * D
    err2 = (T2 - ref2).abs().max().item() / scale
    assert err2 < 4e-6


def test_minsr_tensor_gram_vs_cuda_gram_mixed():
    """The factored mixed minSR direction with the tensor-core Gram equals the
    one with the compensated CUDA-core Gram to 1e-4 and FP64 to 2e-3."""
    m64, X, E = setup("fp64", N=36, nf=32)
    Ns = X.shape[0]
    kw = dict(local_energies=E, energy_mean=float(E.mean()), total_samples=Ns, n_params=m64.n_params,
              diag_shift=1e-3, device=DEV, run_sr=True)
    F64, _ = vg.compute_grads_factored(X, m64)
    dp64, _, _ = vg.MinSRGB300().solve(local_o=F64, **kw)
    m32, _, _ = setup("mixed", N=36, nf=32)
    F32, _ = vg.compute_grads_factored(X, m32)
    dpt, _, it = vg.MinSRGB300(gram="tensor").solve(local_o=F32, **kw)
    dpc, _, ic = vg.MinSRGB300(gram="cuda").solve(local_o=F32, **kw)
    a, b, c = dpt.cpu().numpy(), dpc.cpu().numpy(), dp64.cpu().numpy()
    print("minSR tensor vs cuda Gram %.2e, tensor vs FP64 %.2e" % (rel(a, b), rel(a, c)))
    assert it == ic == 0 and rel(a, b) < 1e-4 and rel(a, c) < 2e-3
