"""The learned Metropolis-Hastings proposal as a sampler.

* Stationarity: on the 4x2 sector (4900 states) the learned sampler, driving
  an FP64 Slater model through the model-agnostic accept (vmc_accept_mh),
  reproduces |psi|^2 from exact enumeration: 32768 chains, 32 snapshots each
  (1.05e6 samples), chi-square over 64 equal-probability bins, next to plain
  exchange/hop Metropolis on the same chains as the control.
* Online schedule: the on_step_end hook records every SR step's samples and
  trains every ``every`` steps inside VMC_GB300.run_vmc_loop.
* Gain: after training on the chains' own samples, the learned sampler's
  ESS/s of E_loc (sampler device time) exceeds plain exchange/hop
  Metropolis's at matched energy on 6x6.
"""
import numpy as np
import pytest
import torch

from oracle import lattice, models as om
import vmc_torch_gb300 as vg
from vmc_torch_gb300.proposal import LearnedProposal, LearnedSamplerGB300, OnlineProposalTraining
from vmc_torch_gb300.stats import tau_int

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _state_index(N, n_up, n_dn):
    S = lattice.all_states(N, n_up, n_dn)
    code = (S * (4 ** np.arange(N))).sum(1)
    table = np.full(4 ** N, -1, dtype=np.int64)
    table[code] = np.arange(len(S))
    return S, table


def _chi_square(counts, p, n_bins=64):
    order = np.argsort(-p)
    cum = np.cumsum(p[order])
    bins = np.minimum((cum * n_bins).astype(np.int64), n_bins - 1)
    b_of_state = np.empty_like(bins)
    b_of_state[order] = bins
    obs = np.bincount(b_of_state, weights=counts, minlength=n_bins)
    exp = np.bincount(b_of_state, weights=p, minlength=n_bins) * counts.sum()
    keep = exp > 0
    return float(((obs[keep] - exp[keep]) ** 2 / exp[keep]).sum()), int(keep.sum()) - 1


def _sample_4x2(sampler, model, graph, table, burn, snaps, B=32768):
    fx = vg.init_walkers(B, 8, 4, 4, seed=19, device=DEV)
    for _ in range(burn):
        sampler.step(fx, model, graph)
    counts = np.zeros(table.max() + 1)
    for _ in range(snaps):
        sampler.step(fx, model, graph)
        X = fx.cpu().numpy()
        idx = table[(X * (4 ** np.arange(8))).sum(1)]
        assert (idx >= 0).all()
        counts += np.bincount(idx, minlength=len(counts))
    return counts


def test_learned_sampler_is_stationary_on_4x2():
    N, nup = 8, 4
    M = np.random.default_rng(3).normal(0, 0.5, (16, 8))
    model = vg.SlaterDeterminant_GB300(16, 8).to(DEV)
    with torch.no_grad():
        model.params[0].copy_(torch.as_tensor(M))
    model.invalidate()
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(4, 2, 1.0, 8.0, 8, n_fermions_per_spin=(nup, nup))
    S, table = _state_index(N, nup, nup)
    p = om.slater_amp(M, S) ** 2
    p /= p.sum()
    prop = LearnedProposal(N, H.edges_on(DEV), device=DEV, seed=17)
    with torch.no_grad():
        prop.params.mul_(2.0)   # a non-uniform proposal: q(x->x') != q(x'->x) matters
    prop.t += 1
    counts = _sample_4x2(LearnedSamplerGB300(prop, moves_per_step=8), model, H.graph, table, 100, 32)
    ctrl = _sample_4x2(vg.MetropolisExchangeSpinfulSamplerGB300(seed=1), model, H.graph, table, 100, 32)
    chi2, dof = _chi_square(counts, p)
    chi2c, _ = _chi_square(ctrl, p)
    tv = 0.5 * np.abs(counts / counts.sum() - p).sum()
    tvc = 0.5 * np.abs(ctrl / ctrl.sum() - p).sum()
    acc = float((prop.k_acc.sum() / prop.k_prop.sum()).item())
    kk = (prop.k_prop / prop.k_prop.sum()).cpu().numpy()
    print("4x2, %d samples: learned chi2/dof %.2f TV %.4f (acceptance %.3f, k mix %s); plain chi2/dof %.2f TV %.4f"
          % (counts.sum(), chi2 / dof, tv, acc, np.round(kk, 3), chi2c / dof, tvc))
    assert acc > 0.05 and kk[1:].sum() > 0.3   # multi-hop moves are proposed and accepted
    # snapshots one step apart are weakly correlated: chi2 up to 4x its dof; at
    # 1e6 samples over 4900 states the total variation is sampling noise
    # (~0.02), so it is held to the plain control's
    assert chi2 / dof < 4.0 and chi2c / dof < 4.0
    assert tv < 1.5 * tvc + 0.005


def test_fused_mixed_step_matches_generic_path():
    """The mixed NNBF model's fused learned-MH step (proposal evaluation, LU
    and Metropolis-Hastings accept in one call) makes the same decisions as
    the model-agnostic path whose stationarity the 4x2 test shows: same
    proposals (two proposal objects with one seed and one set of weights),
    same amplitudes, so the chains coincide up to acceptance tests within the
    FP32 rounding of the fused ratio."""
    Lx, Ly, nup, B = 6, 6, 16, 2048
    N = Lx * Ly
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, 2 * nup, n_fermions_per_spin=(nup, nup))
    model = _nnbf_6x6(21)
    props = []
    for _ in range(2):
        p = LearnedProposal(N, H.edges_on(DEV), device=DEV, seed=23)
        with torch.no_grad():
            p.params.mul_(2.0)
        p.t += 1
        props.append(p)
    x0 = vg.init_walkers(B, N, nup, nup, seed=24, device=DEV)
    xf, xg = x0.clone(), x0.clone()
    _, (sf, lf) = LearnedSamplerGB300(props[0], moves_per_step=12).step(xf, model, H.graph, use_log_amp=True)
    _, (sg, lg) = LearnedSamplerGB300(props[1], moves_per_step=12, fused=False).step(xg, model, H.graph,
                                                                                     use_log_amp=True)
    same = (xf == xg).all(1)
    print("fused vs generic learned MH: %d/%d chains identical, accepted %d / %d"
          % (int(same.sum()), B, int(props[0].kstats[4:].sum()), int(props[1].kstats[4:].sum())))
    assert not torch.equal(xf, x0)
    assert same.double().mean().item() > 0.995
    assert torch.equal(props[0].kstats, props[1].kstats) or same.double().mean().item() > 0.995
    assert (lf[same] - lg[same]).abs().max().item() < 1e-2


def _nnbf_6x6(seed=7):
    g = torch.Generator().manual_seed(seed)
    return vg.NNBF_GB300(36, 32, precision="mixed", generator=g).to(DEV)


def test_online_training_schedule_in_vmc_loop():
    Lx, Ly, nup, B = 6, 6, 16, 2048
    N = Lx * Ly
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, 2 * nup, n_fermions_per_spin=(nup, nup))
    H.precompute_hops_gpu(DEV)
    model = _nnbf_6x6()
    prop = LearnedProposal(N, H.edges_on(DEV), device=DEV, seed=3, buffer=8192)
    seen = []
    hook = OnlineProposalTraining(prop, model, every=5, epochs=1, batch=2048,
                                  then=lambda info: seen.append(info["step"]))
    smp = vg.MetropolisExchangeSpinfulSamplerGB300(seed=2)
    fx = vg.init_walkers(B, N, nup, nup, seed=4, device=DEV)
    cfg = vg.VMCLoopConfig(vmc_steps=10, ns_per_rank=B, grad_batch_size=B, n_params=model.n_params, nsites=N,
                           learning_rate=0.02, diag_shift=1e-3, burn_in_steps=5, factored_o=True)
    drv = vg.VMC_GB300(smp, vg.MinSRGB300(), vg.SGDGB300(0.02))
    hist, fx = drv.run_vmc_loop(fx, model, H, H.graph, 0, 1, cfg, on_step_end=hook)
    assert seen == list(range(10))
    assert hook.sessions == 2 and hook.train_seconds > 0
    assert prop.n_buf == 8192 and np.isfinite(hook.last_loss)
    assert all(np.isfinite(hist))


def _ess(sampler, model, H, x0, samples, discard):
    xc = x0.clone()
    Es, t = [], 0.0
    for _ in range(samples):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        sampler.step(xc, model, H.graph)
        e1.record()
        torch.cuda.synchronize()
        t += e0.elapsed_time(e1) / 1e3
        Es.append(vg.evaluate_energy(xc, model, H)[1])
    E = torch.stack(Es[discard:]).t().contiguous()
    tau = tau_int(E)
    nb, used = E.shape
    ess_s = nb * used / tau / (t * used / samples)
    se = float(E.std().item()) * (tau / (nb * used)) ** 0.5
    return ess_s, tau, float(E.mean().item()), se, 1e3 * t / samples


def test_learned_proposal_gains_ess_per_second_on_6x6():
    Lx, Ly, nup, B = 6, 6, 16, 4096
    N = Lx * Ly
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(Lx, Ly, 1.0, 8.0, 2 * nup, n_fermions_per_spin=(nup, nup))
    H.precompute_hops_gpu(DEV)
    model = _nnbf_6x6(11)
    plain = vg.MetropolisExchangeSpinfulSamplerGB300(seed=5)
    fx = vg.init_walkers(B, N, nup, nup, seed=6, device=DEV)
    plain.burn_in(fx, model, H.graph, 30)
    prop = LearnedProposal(N, H.edges_on(DEV), device=DEV, seed=13)
    for _ in range(8):
        plain.step(fx, model, H.graph)
        vg.evaluate_energy(fx, model, H)
        prop.record(model)
    prop.train(epochs=6, batch=4096)
    learned = LearnedSamplerGB300(prop, moves_per_step=16)
    ep, tp, mp, sp, msp = _ess(plain, model, H, fx, 96, 16)
    el, tl, ml, sl, msl = _ess(learned, model, H, fx, 96, 16)
    dE = abs(mp - ml) / N
    print("6x6 ESS/s plain %.3g (tau %.2f, %.1f ms/sample)  learned %.3g (tau %.2f, %.1f ms/sample)  ratio %.2f  "
          "|dE/site| %.2e (%.1f sigma)" % (ep, tp, msp, el, tl, msl, el / ep, dE, dE * N / (sp ** 2 + sl ** 2) ** 0.5))
    assert abs(mp - ml) < 5 * (sp ** 2 + sl ** 2) ** 0.5
    assert el > 1.3 * ep
