"""GPU parity of the neural-backflow path.

fp64 mode: log-amplitudes, replayed sweeps and local energies against the
reference's golden vectors and the oracle within 1e-10 relative; configurations
and signs bit-exact.
mixed mode (BF16 tensor-core MLP, FP32 determinant): |log|psi| - oracle| <=
5e-3 + 1e-4 * cond(A) per configuration (A = the FP64 orbital matrix; BF16
rounding of the MLP, ~1e-5 relative on A, is amplified by the condition number
near nodes), identical signs where cond(A) < 1e4; local energies within 1e-2
of the FP64 oracle relative to the scale of their terms; a replayed sweep
reproduces the oracle's configurations for >= 95 % of the walkers (acceptance
decisions within the precision of the mixed path may flip).  At 8x8 the
replay runs the oracle's sweep on the CPU emulation of the BF16 path
(``nnbf_logamp_bf16``), so that only FP32 rounding separates the two chains,
and checks the carried log-amplitudes against FP64."""
import hashlib

import numpy as np
import pytest
import torch

from oracle import hubbard, lattice, models as om, sampler as osampler
import vmc_torch_gb300 as vg

pytestmark = pytest.mark.gpu
DEV = "cuda"
LOG_TOL_MIXED = 5e-3


def fixture_params(g):
    ps = om.nnbf_init(64, 64, 256, 2, seed=int(g["seed"]))
    h = hashlib.sha256()
    for p in ps:
        h.update(np.ascontiguousarray(p, dtype=np.float64).tobytes())
    return ps, h.hexdigest() == str(g["params_sha256"])


def make_model(ps, n_sites, nf, precision):
    m = vg.NNBF_GB300(n_sites, nf, precision=precision).to(DEV)
    with torch.no_grad():
        for p, v in zip(m.params, ps):
            p.copy_(torch.as_tensor(v))
    m.invalidate()
    return m


def test_fp64_logamp_matches_reference(golden):
    g = golden("nnbf.npz")
    ps, same = fixture_params(g)
    m = make_model(ps, 64, 64, "fp64")
    X = g["x"].astype(np.int64)
    s, l = m.forward_log(torch.as_tensor(X, device=DEV))
    so, lo = om.nnbf_logamp(ps, X, 0.01)
    assert np.array_equal(s.cpu().numpy(), so)
    np.testing.assert_allclose(l.cpu().numpy(), lo, rtol=1e-10, atol=1e-10)
    if same:
        assert np.array_equal(s.cpu().numpy(), g["sign"])
        np.testing.assert_allclose(l.cpu().numpy(), g["logabs"], rtol=1e-10, atol=1e-10)


def test_fp64_replayed_sweep_and_energy_match_reference(golden):
    g = golden("nnbf.npz")
    ps, same = fixture_params(g)
    if not same:
        pytest.skip("numpy normal stream differs from the one that made the fixture")
    m = make_model(ps, 64, 64, "fp64")
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(8, 8, 1.0, 8.0, 64, n_fermions_per_spin=(32, 32))
    H.precompute_hops_gpu(DEV)
    fx = torch.as_tensor(g["x0"].astype(np.int64), device=DEV).clone()
    rp = tuple(torch.as_tensor(a, device=DEV).contiguous() for a in (g["u_move"], g["hop_bit"], g["u_acc"]))
    smp = vg.MetropolisExchangeSpinfulSamplerGB300()
    fx, (s, l) = smp.step(fx, m, H.graph, use_log_amp=True, replay=rp)
    assert np.array_equal(fx.cpu().numpy(), g["x_final"].astype(np.int64))
    assert np.array_equal(s.cpu().numpy(), g["sign_final"])
    np.testing.assert_allclose(l.cpu().numpy(), g["logabs_final"], rtol=1e-10, atol=1e-10)
    _, eloc = vg.evaluate_energy(fx, m, H, (s, l), use_log_amp=True)
    np.testing.assert_allclose(eloc.cpu().numpy(), g["eloc"], rtol=1e-10, atol=1e-9)


@pytest.mark.parametrize("Lx,Ly,nup,B", [(8, 8, 32, 300), (6, 6, 16, 200)])
def test_mixed_logamp_vs_fp64_oracle(Lx, Ly, nup, B):
    N = Lx * Ly
    nf = 2 * nup
    ps = om.nnbf_init(N, nf, 256, 2, seed=N + nf)
    X = lattice.random_initial_configs(B, N, nup, nup, seed=7)
    so, lo = om.nnbf_logamp(ps, X, 0.01)
    m = make_model(ps, N, nf, "mixed")
    s, l = m.forward_log(torch.as_tensor(X, device=DEV))
    s, l = s.cpu().numpy(), l.cpu().numpy()
    err = np.abs(l - lo)
    Mx = om.nnbf_M(ps, X, 0.01)
    cond = np.linalg.cond(np.take_along_axis(Mx, om.occupied_rows(X)[:, :, None], axis=1))
    print("mixed log|psi| abs err: max %.3e median %.3e; max err at cond<1e3: %.3e"
          % (err.max(), np.median(err), err[cond < 1e3].max()))
    assert np.array_equal(s[cond < 1e4], so[cond < 1e4])
    assert np.median(err) < 2e-3
    assert (err <= LOG_TOL_MIXED + 1e-4 * cond).all()
    # against the CPU emulation of the BF16 path itself: only FP32 LU / GELU rounding differences remain
    sb, lb = om.nnbf_logamp_bf16(ps, X, 0.01)
    eb = np.abs(l - lb)
    print("mixed vs BF16-path emulation: max %.3e median %.3e" % (eb.max(), np.median(eb)))
    assert np.median(eb) < 2e-4
    assert (eb <= 2e-3 + 2e-6 * cond).all()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sweep_and_local_energy_vs_oracle(precision):
    Lx, Ly, nup, B, S = 6, 6, 16, 48, 2
    N, nf = Lx * Ly, 2 * nup
    ps = om.nnbf_init(N, nf, 256, 2, seed=123)
    rng = np.random.default_rng(4)
    E = lattice.sweep_edges(Lx, Ly)
    X = lattice.random_initial_configs(B, N, nup, nup, seed=8)
    um = rng.random((S, len(E), B), dtype=np.float32)
    hb = rng.integers(0, 2, (S, len(E), B)).astype(np.uint8)
    ua = rng.random((S, len(E), B), dtype=np.float32)
    xo, (so, lo), _ = osampler.sweep(X, E, lambda y: om.nnbf_logamp(ps, y, 0.01), um, hb, ua)
    m = make_model(ps, N, nf, precision)
    g = vg.SquareLattice(Lx, Ly)
    fx = torch.as_tensor(X, device=DEV).clone()
    rp = tuple(torch.as_tensor(a, device=DEV).contiguous() for a in (um, hb, ua))
    fx = vg.MetropolisExchangeSpinfulSamplerGB300().burn_in(fx, m, g, S, replay=rp)
    same = (fx.cpu().numpy() == xo).all(axis=1)
    if precision == "fp64":
        assert same.all()
    else:
        assert same.mean() >= 0.95
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, nf, n_fermions_per_spin=(nup, nup))
    H.precompute_hops_gpu(DEV)
    _, eloc = vg.evaluate_energy(fx, m, H)
    xg = fx.cpu().numpy()
    ref = hubbard.local_energy(xg, lattice.square_edges(Lx, Ly), 1.0, 8.0, lambda y: om.nnbf_amp(ps, y, 0.01))
    if precision == "fp64":
        np.testing.assert_allclose(eloc.cpu().numpy(), ref, rtol=1e-10, atol=1e-9)
    else:
        np.testing.assert_allclose(eloc.cpu().numpy(), ref, rtol=1e-2, atol=1e-2)


def test_mixed_chunk_pipeline_is_exact():
    """Above 4096 rows the backflow GEMM of one chunk overlaps the LU of the
    previous one on a second stream, alternating two orbital-matrix slots.
    Each row's arithmetic does not depend on its chunk, so a 9000-row
    evaluation (three chunks, pipelined) equals three single-chunk
    evaluations bit for bit.  Philox sweeps of 9000 walkers carry
    log-amplitudes that agree with a fresh evaluation of their final
    configurations (up to the incremental first-layer update's FP32 rounding
    passing through BF16) -- a slot overwritten too early would corrupt whole
    chunks."""
    N, nf = 64, 64
    m = make_model(om.nnbf_init(N, nf, 256, 2, seed=77), N, nf, "mixed")
    x = vg.init_walkers(9000, N, 32, 32, seed=5, device=DEV)
    s, la = m.forward_log(x)
    parts = [m.forward_log(x[a:b]) for a, b in ((0, 4000), (4000, 8000), (8000, 9000))]
    assert torch.equal(s, torch.cat([p[0] for p in parts]))
    assert torch.equal(la, torch.cat([p[1] for p in parts]))
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(8, 8, 1.0, 8.0, 64, n_fermions_per_spin=(32, 32))
    fx = x.clone()
    fx, (s1, la1) = vg.MetropolisExchangeSpinfulSamplerGB300(seed=3, sweeps_per_step=2).step(
        fx, m, H.graph, use_log_amp=True)
    s2, la2 = m.forward_log(fx)
    bad = (la1 - la2).abs() > 1e-2
    assert bad.double().mean().item() < 0.01
    assert torch.equal(s1[~bad], s2[~bad])
    assert not torch.equal(fx, x)


def test_mixed_walker_groups_match_single_stream():
    """From 8192 walkers the mixed sweep splits the walkers into groups that run
    their edge loops on separate streams.  Each walker's arithmetic and random
    draws are unchanged, so a replayed 9000-walker sweep equals, bit for bit,
    two 4500-walker sweeps (single stream) over the same walkers and draws."""
    N, nf = 64, 64
    m = make_model(om.nnbf_init(N, nf, 256, 2, seed=78), N, nf, "mixed")
    g = vg.SquareLattice(8, 8)
    E = len(g.sweep_edges())
    B, S = 9000, 1
    rng = np.random.default_rng(12)
    um = torch.as_tensor(rng.random((S, E, B), dtype=np.float32), device=DEV)
    hb = torch.as_tensor(rng.integers(0, 2, (S, E, B)).astype(np.uint8), device=DEV)
    ua = torch.as_tensor(rng.random((S, E, B), dtype=np.float32), device=DEV)
    x = vg.init_walkers(B, N, 32, 32, seed=13, device=DEV)
    smp = vg.MetropolisExchangeSpinfulSamplerGB300()
    full = x.clone()
    full, (s_f, l_f) = smp.step(full, m, g, use_log_amp=True, replay=(um, hb, ua))
    parts = []
    for a, b in ((0, 4500), (4500, 9000)):
        xp = x[a:b].clone()
        rp = tuple(t[:, :, a:b].contiguous() for t in (um, hb, ua))
        xp, (sp, lp) = smp.step(xp, m, g, use_log_amp=True, replay=rp)
        parts.append((xp, sp, lp))
    assert torch.equal(full, torch.cat([p[0] for p in parts]))
    assert torch.equal(s_f, torch.cat([p[1] for p in parts]))
    assert torch.equal(l_f, torch.cat([p[2] for p in parts]))
    assert not torch.equal(full, x)


def test_mixed_local_energy_groups_match_single_stream():
    """With a workspace of two or more 4096-row chunks the mixed local energy
    spreads the connected configurations over several streams; the terms are
    computed exactly as on one stream, so E_loc of 9000 walkers equals that of
    the two halves evaluated separately, bit for bit."""
    N, nf = 64, 64
    m = make_model(om.nnbf_init(N, nf, 256, 2, seed=79), N, nf, "mixed")
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(8, 8, 1.0, 8.0, 64, n_fermions_per_spin=(32, 32))
    H.precompute_hops_gpu(DEV)
    x = vg.init_walkers(9000, N, 32, 32, seed=14, device=DEV)
    _, e_full = vg.evaluate_energy(x.clone(), m, H)
    e_parts = [vg.evaluate_energy(x[a:b].clone(), m, H)[1] for a, b in ((0, 4500), (4500, 9000))]
    assert torch.equal(e_full, torch.cat(e_parts))


def _cond(ps, X):
    Mx = om.nnbf_M(ps, X, 0.01)
    return np.linalg.cond(np.take_along_axis(Mx, om.occupied_rows(X)[:, :, None], axis=1))


@pytest.mark.parametrize("B", [4096, 6000, 20480])
def test_mixed_8x8_replayed_sweep_vs_oracle(B):
    """The timed 8x8 kernels against the oracle.  B = 4096: one chunk, warp-pair
    LU (k_logdet_pair<ACCEPT>); 6000: two chunks with the backflow GEMM of the
    second overlapping the LU of the first on the second stream; 20480: four
    walker groups of 5120 on their own streams, each two chunks, two matrices
    a warp (k_logdet_dual<ACCEPT>).  One replayed 112-edge sweep; 64 walkers
    spread over every group and chunk are replayed by the oracle's sweep
    (vmc_torch/GPU/sampler.py:217-388) on the CPU emulation of the BF16 path."""
    N, nf, nup = 64, 64, 32
    ps = om.nnbf_init(N, nf, 256, 2, seed=91)
    g = vg.SquareLattice(8, 8)
    E = lattice.sweep_edges(8, 8)
    assert [tuple(e) for e in g.sweep_edges()] == [tuple(e) for e in E]
    rng = np.random.default_rng(B)
    um = rng.random((1, len(E), B), dtype=np.float32)
    hb = rng.integers(0, 2, (1, len(E), B)).astype(np.uint8)
    ua = rng.random((1, len(E), B), dtype=np.float32)
    m = make_model(ps, N, nf, "mixed")
    x0 = vg.init_walkers(B, N, nup, nup, seed=B + 1, device=DEV)
    X0 = x0.cpu().numpy()
    fx = x0.clone()
    rp = tuple(torch.as_tensor(a, device=DEV).contiguous() for a in (um, hb, ua))
    fx, (s, l) = vg.MetropolisExchangeSpinfulSamplerGB300().step(fx, m, g, use_log_amp=True, replay=rp)
    torch.cuda.synchronize()
    idx = np.unique(np.linspace(0, B - 1, 64).round().astype(np.int64))
    xo, (so, lo), nacc = osampler.sweep(X0[idx], E, lambda y: om.nnbf_logamp_bf16(ps, y, 0.01),
                                        um[:, :, idx], hb[:, :, idx], ua[:, :, idx])
    xg = fx.cpu().numpy()[idx]
    sg, lg = s.cpu().numpy()[idx], l.cpu().numpy()[idx]
    same = (xg == xo).all(axis=1)
    print("B=%d: %d/%d walkers equal to the oracle chain, mean accepted moves %.1f"
          % (B, same.sum(), len(idx), nacc.mean()))
    assert nacc.mean() > 1.0          # the chains moved
    assert same.mean() >= 0.95
    # carried log-amplitudes: against the BF16-path emulation and against FP64
    cond = _cond(ps, xg)
    eb = np.abs(lg[same] - lo[same])
    sf, lf = om.nnbf_logamp(ps, xg, 0.01)
    ef = np.abs(lg - lf)
    print("carried log|psi| vs BF16 emulation: max %.3e median %.3e; vs FP64: max %.3e median %.3e"
          % (eb.max(), np.median(eb), ef.max(), np.median(ef)))
    assert (eb <= 2e-3 + 2e-6 * cond[same]).all()
    assert (ef <= LOG_TOL_MIXED + 1e-4 * cond).all()
    assert np.array_equal(sg[same & (cond < 1e4)], so[same & (cond < 1e4)])
    assert np.array_equal(sg[cond < 1e4], sf[cond < 1e4])


def _eloc_scale(ps, X, edges, U, amp_fn):
    """Per-walker scale of the local-energy sum: U * doublons + sum |H psi'/psi|."""
    etas, coeffs, bids = hubbard.get_conn_batch(X, edges, 1.0, U)
    pe, px = amp_fn(etas), amp_fn(X)
    sc = np.zeros(X.shape[0])
    np.add.at(sc, bids, np.abs(coeffs * pe / px[bids]))
    return sc


@pytest.mark.parametrize("B", [2048, 9000])
def test_mixed_8x8_local_energy_vs_oracle(B):
    """8x8 mixed E_loc (the hop terms' LU in LD_ELOC mode) against the oracle.
    B = 2048: one stream, warp-pair LU; 9000: the connected configurations
    spread over two streams, two matrices a warp.  32 walkers are checked
    against the oracle's local energy (vmc_torch/GPU/vmc_utils.py:449-476) with
    FP64 amplitudes and with the BF16-path emulation."""
    N, nf, nup = 64, 64, 32
    ps = om.nnbf_init(N, nf, 256, 2, seed=92)
    m = make_model(ps, N, nf, "mixed")
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(8, 8, 1.0, 8.0, 64, n_fermions_per_spin=(32, 32))
    H.precompute_hops_gpu(DEV)
    x = vg.init_walkers(B, N, nup, nup, seed=B + 3, device=DEV)
    _, eloc = vg.evaluate_energy(x, m, H)
    idx = np.unique(np.linspace(0, B - 1, 32).round().astype(np.int64))
    X = x.cpu().numpy()[idx]
    eg = eloc.cpu().numpy()[idx]
    edges = lattice.square_edges(8, 8)

    def amp64(y):
        return om.nnbf_amp(ps, y, 0.01)

    def amp16(y):
        s_, l_ = om.nnbf_logamp_bf16(ps, y, 0.01)
        return s_ * np.exp(l_)

    e64 = hubbard.local_energy(X, edges, 1.0, 8.0, amp64)
    e16 = hubbard.local_energy(X, edges, 1.0, 8.0, amp16)
    sc = _eloc_scale(ps, X, edges, 8.0, amp64)
    d64, d16 = np.abs(eg - e64) / sc, np.abs(eg - e16) / sc
    print("E_loc rel. to term scale: vs FP64 max %.3e median %.3e; vs BF16 emulation max %.3e median %.3e"
          % (d64.max(), np.median(d64), d16.max(), np.median(d16)))
    assert (d64 <= 1e-2).all()
    assert (d16 <= 1e-3).all()


@pytest.mark.parametrize("B", [6000, 12288])
def test_mixed_row_compaction_is_exact(B):
    """The sweep's GEMMs and LU run over the walkers whose proposal changes
    them only (compact rows, slots taken atomically).  An MMA row and a
    matrix's LU do not depend on their neighbours, so a replayed sweep with
    compaction equals the one without it bit for bit: configurations, signs,
    log-amplitudes and accept counts; one walker group (6000, two chunks on
    the pipeline) and three groups (12288, k_logdet_dual)."""
    N, nf = 64, 64
    ps = om.nnbf_init(N, nf, 256, 2, seed=93)
    g = vg.SquareLattice(8, 8)
    E = len(g.sweep_edges())
    rng = np.random.default_rng(B + 7)
    rp = tuple(torch.as_tensor(a, device=DEV) for a in (rng.random((1, E, B), dtype=np.float32),
                                                         rng.integers(0, 2, (1, E, B)).astype(np.uint8),
                                                         rng.random((1, E, B), dtype=np.float32)))
    x0 = vg.init_walkers(B, N, 32, 32, seed=B, device=DEV)
    out = []
    for compact in (True, False):
        m = make_model(ps, N, nf, "mixed")
        m.compact_rows = compact
        fx = x0.clone()
        fx, (s, l) = vg.MetropolisExchangeSpinfulSamplerGB300().step(fx, m, g, use_log_amp=True, replay=rp)
        out.append((fx, s, l, m._state.n_acc.clone()))
    assert not torch.equal(out[0][0], x0)
    for a, b in zip(out[0], out[1]):
        assert torch.equal(a, b)
