"""Benchmark of the VMC inner loop on one GB300.

Workload (the headline configuration): 8x8 OBC spinful Fermi-Hubbard, t=1,
U=8, 32 up + 32 down electrons; neural-backflow Slater determinant (128-dim
occupation -> 2 x 256 GELU -> 128 x 64 orbital correction, N(0, 1/fan_in)
init, bf_scale 0.01) with the MLP in BF16 / FP32 accumulation and the
determinant in FP32; 16384 walkers resident on the GPU.

A step is one Metropolis sweep of every walker over all 112 nearest-neighbour
edges (exchange-or-hop proposals, 25 % hops), i.e. 16384 * 112 walker-steps.
``value`` is walker-steps/s with the walkers resident in HBM; ``e2e`` is the
same metric through the public sampler API with the configurations copied
from pinned host memory before each step and the configurations plus
log-amplitudes copied back after it.  L2 is flushed (256 MB write) between
timed steps.

--impl reference times the reference's own implementation on the host CPU:
its batched sampler (MetropolisExchangeSpinfulSamplerGPU) and NNBF_GPU model,
imported from its pip install in baseline/_ref under the import shims of its
absent tensor-network / MPI dependencies, one single-thread process per core
with 16 chains each (the reference's MPI ranks run independent chains too).
Where that install is absent, the CPU port of the same sampler
(oracle/sampler.py with the FP64 NNBF amplitude of oracle/models.py) stands in.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "walker-steps/s and ESS/s, learned vs plain proposal, at |ΔE/site|<1e-3"
UNIT = "walker-steps/s"
LX, LY, NUP, NDN = 8, 8, 32, 32
B = 16384
HID = 256
BF_SCALE = 0.01


def workload_config(extra=None):
    cfg = {"workload": "8x8 OBC Fermi-Hubbard t=1 U=8 (32+32), NNBF 2x256 GELU backflow, 16384 walkers, "
                       "one exchange-or-hop Metropolis sweep (112 edges) per step",
           "lattice": "8x8", "n_up": NUP, "n_dn": NDN, "walkers": B, "hidden": "2x256", "edges_per_sweep": 112,
           "mlp_dtype": "bf16 (fp32 accumulate)", "det_dtype": "fp32", "init": "N(0,1/fan_in), M_base N(0,0.1^2)",
           "l2": "flushed (256 MB write) between timed steps", "parallelism": "replicas (1 GPU per process)"}
    if extra:
        cfg.update(extra)
    return cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def replica_rate(units, ms, dist=None, device=None):
    """Whole-job throughput of independent replicas (one per rank): the units
    all ranks processed over the slowest rank's time, so that N replicas are
    timed as one job.  Returns (units/s, max ms).  Collective calls only when
    a process group is given."""
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.barrier()
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
    ms_max = float(t.item())
    return float(u.item()) / (ms_max / 1e3), ms_max


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d.get("hbm_gbs"), "bf16_tflops": d.get("bf16_tflops"),
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


# ---------------------------------------------------------------------------
def cpu_port_rate(n_walkers=48, n_sweeps=1, seed=0):
    """The oracle (CPU port of the reference sampler + FP64 NNBF) on a bounded
    sample: returns (walker-steps/s, seconds, sample description)."""
    from oracle import lattice, models, sampler
    ps = models.nnbf_init(LX * LY, NUP + NDN, HID, 2, seed=seed)
    edges = lattice.sweep_edges(LX, LY)
    X = lattice.random_initial_configs(n_walkers, LX * LY, NUP, NDN, seed=seed + 1)
    rng = np.random.default_rng(seed + 2)
    S, E = n_sweeps, len(edges)
    um = rng.random((S, E, n_walkers), dtype=np.float32)
    hb = rng.integers(0, 2, (S, E, n_walkers)).astype(np.uint8)
    ua = rng.random((S, E, n_walkers), dtype=np.float32)
    t0 = time.perf_counter()
    sampler.sweep(X, edges, lambda y: models.nnbf_logamp(ps, y, BF_SCALE), um, hb, ua)
    dt = time.perf_counter() - t0
    steps = n_walkers * E * S
    return steps / dt, dt, "%d walkers x %d sweep(s) x %d edges of the same 8x8 NNBF workload (FP64 numpy)" % (
        n_walkers, S, E)


REF_ROOT = os.path.join(ROOT, "baseline", "_ref")
_ref = {}


def _ref_init(root, n_walkers, seed):
    """Worker set-up: the reference's own batched sampler and NNBF_GPU model
    (imported from its pip install under the import shims of its absent TN /
    MPI dependencies), one CPU thread, ``n_walkers`` seeded chains."""
    os.environ["OMP_NUM_THREADS"] = "1"
    import torch
    torch.set_num_threads(1)
    from oracle import lattice, models, refshim
    ht = refshim.load("vmc_torch.hamiltonian_torch", root)
    smp = refshim.load("vmc_torch.GPU.sampler", root)
    nn = refshim.load("vmc_torch.GPU.models.NNBF", root)
    H = ht.spinful_Fermi_Hubbard_square_lattice_torch(LX, LY, 1.0, 8.0, NUP + NDN, n_fermions_per_spin=(NUP, NDN))
    model = nn.NNBF_GPU(LX * LY, NUP + NDN, hidden_dim=HID, n_layers=2, activation="gelu", bf_scale=BF_SCALE)
    with torch.no_grad():
        for p, v in zip(model.params, models.nnbf_init(LX * LY, NUP + NDN, HID, 2, seed=0)):
            p.copy_(torch.as_tensor(v))
    fx = torch.as_tensor(lattice.random_initial_configs(n_walkers, LX * LY, NUP, NDN, seed=seed + os.getpid()))
    _ref.update(H=H, model=model, sampler=smp.MetropolisExchangeSpinfulSamplerGPU(), fx=fx, torch=torch)


def _ref_sweep(_):
    """One reference sweep (112 edges) of this worker's chains: (walker-steps, seconds)."""
    torch = _ref["torch"]
    t0 = time.perf_counter()
    with torch.inference_mode():
        _ref["fx"], _ = _ref["sampler"].step(_ref["fx"], _ref["model"], _ref["H"].graph)
    n_edges = 2 * LX * LY - LX - LY   # nearest-neighbour edges of the open LX x LY lattice: one sweep
    return _ref["fx"].shape[0] * n_edges, time.perf_counter() - t0


def reference_pool(n_procs, n_walkers):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    return ctx.Pool(n_procs, initializer=_ref_init, initargs=(REF_ROOT, n_walkers, 17))


def reference_rate(pool, n_procs):
    """One timed round: every worker runs one sweep of its own chains at once
    (independent chains, no communication, as the reference's MPI ranks);
    throughput = all walker-steps over the slowest worker's time."""
    res = pool.map(_ref_sweep, range(n_procs))
    return sum(r[0] for r in res) / max(r[1] for r in res)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    world = int(os.environ.get("WORLD_SIZE", "1"))
    cores = os.cpu_count()
    if os.path.isdir(os.path.join(REF_ROOT, "vmc_torch")):
        # the reference's own batched sampler + NNBF_GPU on every host core:
        # one single-thread process per core, 16 chains each
        nw = 16
        pool = reference_pool(cores, nw)
        try:
            for _ in range(args.warmup):
                reference_rate(pool, cores)
            rates = []
            t0 = time.perf_counter()
            for _ in range(args.steps):
                rates.append(reference_rate(pool, cores))
            tot = time.perf_counter() - t0
        finally:
            pool.close()
            pool.join()
        value = float(np.mean(rates))
        kind = "reference"
        sample = ("the reference's MetropolisExchangeSpinfulSamplerGPU + NNBF_GPU(2x256 GELU) on the host CPU: "
                  "%d single-thread processes x %d chains x 1 sweep (112 edges) per step" % (cores, nw))
        dtype = "f64 (reference defaults)"
    else:
        for _ in range(args.warmup):
            cpu_port_rate(n_walkers=16, n_sweeps=1)
        rates, tot = [], 0.0
        for k in range(args.steps):
            r, dt, sample = cpu_port_rate(n_walkers=48, n_sweeps=1, seed=k)
            rates.append(r)
            tot += dt
        value = float(np.mean(rates))
        kind = "port"
        dtype = "f64"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded)",
            "config": workload_config({"sample": sample}), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
PEPS_LX, PEPS_LY, PEPS_D, PEPS_NE, PEPS_B, PEPS_CHI = 6, 6, 4, 16, 8192, 16


def peps_flops_per_column(Lx=PEPS_LX, D=PEPS_D):
    """Algorithmic FLOP of one column step of the two-row sweep: per top-bond
    slice the four contractions (D^3 DA^2 + 2 D^5 DA + D^3 DA^2 multiply-adds),
    DA slices, plus the column's two boundary-MPS builds."""
    da = D ** (Lx // 2 - 1)
    per_slice = 2 * D ** 3 * da * da + 2 * D ** 5 * da
    build = 2 * (da * D * da) * D * (Lx // 2 - 2) if Lx > 4 else 0
    return 2.0 * (da * per_slice + build)


def peps_flops_per_amp(Lx=PEPS_LX, Ly=PEPS_LY, D=PEPS_D):
    """One exact amplitude from scratch: Ly column steps."""
    return Ly * peps_flops_per_column(Lx, D)


def peps_cpu_rate(n_walkers=6, seed=0):
    """The oracle's exact contraction driving the CPU port of the sampler on a
    bounded sample of the 6x6 fPEPS workload."""
    from oracle import lattice, peps, sampler
    T = peps.init_tensors(PEPS_LX, PEPS_LY, PEPS_D, seed=seed)
    edges = lattice.sweep_edges(PEPS_LX, PEPS_LY)
    X = lattice.random_initial_configs(n_walkers, PEPS_LX * PEPS_LY, PEPS_NE, PEPS_NE, seed=seed + 1)
    rng = np.random.default_rng(seed + 2)
    E = len(edges)
    um = rng.random((1, E, n_walkers), dtype=np.float32)
    hb = rng.integers(0, 2, (1, E, n_walkers)).astype(np.uint8)
    ua = rng.random((1, E, n_walkers), dtype=np.float32)
    t0 = time.perf_counter()
    sampler.sweep(X, edges, lambda y: peps.logamp(T, y, "rows"), um, hb, ua)
    dt = time.perf_counter() - t0
    return n_walkers * E / dt, "%d walkers x 1 sweep x %d edges of the 6x6 D=4 fPEPS (FP64 numpy, exact)" % (
        n_walkers, E)


def peps_chi_cpu_rate(n_walkers=2, seed=0, chi=PEPS_CHI):
    """The oracle's chi-truncated contraction (full-state formulation, FP64
    numpy SVDs) driving the CPU port of the sampler on a bounded sample."""
    from oracle import lattice, peps, sampler
    T = peps.init_tensors(PEPS_LX, PEPS_LY, PEPS_D, seed=seed)
    edges = lattice.sweep_edges(PEPS_LX, PEPS_LY)
    X = lattice.random_initial_configs(n_walkers, PEPS_LX * PEPS_LY, PEPS_NE, PEPS_NE, seed=seed + 1)
    rng = np.random.default_rng(seed + 2)
    E = len(edges)
    um = rng.random((1, E, n_walkers), dtype=np.float32)
    hb = rng.integers(0, 2, (1, E, n_walkers)).astype(np.uint8)
    ua = rng.random((1, E, n_walkers), dtype=np.float32)
    t0 = time.perf_counter()
    sampler.sweep(X, edges, lambda y: peps.logamp(T, y, "chi", chi=chi), um, hb, ua)
    dt = time.perf_counter() - t0
    return n_walkers * E / dt, "%d walkers x 1 sweep x %d edges of the 6x6 D=4 fPEPS, chi=%d (FP64 numpy SVD)" % (
        n_walkers, E, chi)


def _timed(stream, fn):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    out = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), out


def peps_block(dev, steps, fp32_peak_tflops, cpu=True, env_reuse=True):
    """Secondary workload: 6x6 OBC Hubbard (16+16), fPEPS D=4 with N(0,1) FP32
    site tensors, 8192 walkers, one Metropolis sweep (60 edges) per step, with
    the reference's boundary contraction truncated to chi = 16 (the headline of
    the block); the exact contraction (max_bond -> infinity, cached column
    environments) is timed beside it, and gives the O timing (the
    log-derivatives are implemented for the exact contraction)."""
    import torch
    import vmc_torch_gb300 as vg
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(PEPS_LX, PEPS_LY, 1.0, 8.0, 2 * PEPS_NE,
                                                      n_fermions_per_spin=(PEPS_NE, PEPS_NE))
    H.precompute_hops_gpu(dev)
    g = H.graph
    E = len(g.sweep_edges())
    stream = torch.cuda.current_stream(dev)

    def run(model):
        fx = vg.init_walkers(PEPS_B, PEPS_LX * PEPS_LY, PEPS_NE, PEPS_NE, seed=9, device=dev)
        smp = vg.MetropolisExchangeSpinfulSamplerGB300(seed=13)
        smp.burn_in(fx, model, g, 1)
        st = model.bind_state(fx)
        ne = torch.zeros(2, dtype=torch.int64, device=dev)
        ms = 0.0
        for k in range(steps):
            ms += _timed(stream, lambda: model.sweep(st, g, 1, 13, 100 + k, 0.25, None, n_eval=ne))[0]
        el_ms, (_, eloc) = _timed(stream, lambda: vg.evaluate_energy(fx, model, H))
        return fx, st, ms, int(ne[0].item()), int(ne[1].item()), el_ms, eloc

    mc = vg.FPEPS_GB300(PEPS_LX, PEPS_LY, PEPS_D, max_bond=PEPS_CHI,
                        generator=torch.Generator().manual_seed(5)).to(dev)
    fx, st, ms_c, ev_c, builds, el_c, eloc_c = run(mc)
    ev_ms = _timed(stream, lambda: mc._refresh(st, 0))[0]
    m = vg.FPEPS_GB300(PEPS_LX, PEPS_LY, PEPS_D, generator=torch.Generator().manual_seed(5),
                       env_reuse=env_reuse).to(dev)
    fx2, st2, ms, n_eval, n_cols, el_ms, eloc = run(m)
    gr_ms, O = _timed(stream, lambda: m.logpsi_grad(st2))
    fl = peps_flops_per_column()
    achieved = n_cols * fl / (ms / 1e3) / 1e12
    out = {"workload": "6x6 OBC Fermi-Hubbard U=8 (16+16), fPEPS D=4 N(0,1) FP32 tensors, 8192 walkers, boundary "
                       "contraction truncated to chi=%d, one 60-edge Metropolis sweep per step" % PEPS_CHI,
           "value": steps * PEPS_B * E / (ms_c / 1e3), "unit": UNIT, "ms_per_step": ms_c / steps,
           "chi": PEPS_CHI, "truncated_cuts": mc.chi_cuts,
           "evaluated_proposals_per_step": ev_c / steps, "side_states_built_per_step": builds / steps,
           "us_per_side_state": 1e3 * ms_c / max(builds, 1),
           "eval_ms": ev_ms, "local_energy_ms": el_c,
           "energy_per_site": float(eloc_c.mean().item()) / (PEPS_LX * PEPS_LY),
           "exact": {"workload": "the same sweep with the exact contraction (max_bond -> infinity)",
                     "value": steps * PEPS_B * E / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
                     "evaluated_proposals_per_step": n_eval / steps, "column_steps_per_step": n_cols / steps,
                     "column_steps_per_proposal": n_cols / max(n_eval, 1),
                     "roofline": {"bound": "fp32 CUDA-core FMA",
                                  "kernel": "k_peps_sweep_env<float,4,16>" if env_reuse else "k_peps_sweep<float,4,16>",
                                  "achieved": achieved, "peak": fp32_peak_tflops, "unit": "TFLOP/s",
                                  "frac": achieved / fp32_peak_tflops,
                                  "algorithmic": "%.4g FLOP per column step (counted on device); a from-scratch "
                                                 "amplitude is 6 column steps" % fl,
                                  "peak_source": "nominal: 152 SM x 128 FP32 lanes x 2 x sampled max SM clock"},
                     "local_energy_ms": el_ms, "logpsi_grad_ms": gr_ms, "O_shape": list(O.shape),
                     "energy_per_site": float(eloc.mean().item()) / (PEPS_LX * PEPS_LY)}}
    if cpu:
        r, sample = peps_chi_cpu_rate()
        out["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample}
        r, sample = peps_cpu_rate()
        out["exact"]["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample}
    return out


# ---------------------------------------------------------------------------
def ess_block(dev, n_walkers, samples=192, discard=32, moves=14, sr_steps=20, pre_walkers=4096, every=10, epochs=4,
              lr=0.02, burn=120):
    """ESS/s of E_loc for plain exchange/hop Metropolis (one 112-edge sweep per
    sample) vs the learned proposal (``moves`` MH moves per sample) on the 8x8
    backflow model after ``sr_steps`` SR steps (not at random init).

    Schedule: the SR steps run on ``pre_walkers`` walkers with the plain
    sampler; the learned proposal records every step's samples (ring buffer of
    the last 65536) and trains ``epochs`` epochs every ``every`` steps (the
    OnlineProposalTraining hook).  Then, at the final parameters, both
    samplers draw ``samples`` samples per chain from the same equilibrated
    ``n_walkers`` walkers (the first ``discard`` left out of the estimates).
    ESS/s is reported three ways: (a) sampler device time only; (b) with the
    proposal's training charged as on the schedule, one session per ``every``
    samples (one sample per chain per SR step); (c) with the local-energy
    device time of every sample added to both samplers; and (b)+(c).  The
    measurement walkers are first equilibrated by ``burn`` plain sweeps at the
    final parameters; the mean energies of the first and second halves of the
    used samples show any remaining drift."""
    import torch
    import vmc_torch_gb300 as vg
    from vmc_torch_gb300.proposal import LearnedProposal, LearnedSamplerGB300, OnlineProposalTraining
    from vmc_torch_gb300.stats import split_rhat, tau_int

    model = vg.NNBF_GB300(LX * LY, NUP + NDN, hidden_dim=HID, n_layers=2, bf_scale=BF_SCALE, precision="mixed",
                          generator=torch.Generator().manual_seed(4321)).to(dev)
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(LX, LY, 1.0, 8.0, NUP + NDN, n_fermions_per_spin=(NUP, NDN))
    H.precompute_hops_gpu(dev)
    graph = H.graph
    prop = LearnedProposal(LX * LY, H.edges_on(dev), device=dev, seed=5)
    # warm-up of the training path on a throwaway proposal: the first call of
    # each kernel pays for loading its module and, for the tensor library's
    # own kernels, for first-use compilation; none of that belongs to a
    # training session
    tmp = LearnedProposal(LX * LY, H.edges_on(dev), device=dev, seed=6, buffer=16384)
    tmp.buf_occ.copy_(vg.pack(vg.init_walkers(16384, LX * LY, NUP, NDN, seed=5, device=dev)))
    tmp.buf_tgt.uniform_()
    tmp.n_buf = 16384
    tmp.train(epochs=1, batch=16384)
    del tmp
    hook = OnlineProposalTraining(prop, model, every=every, epochs=epochs, batch=16384)
    plain = vg.MetropolisExchangeSpinfulSamplerGB300(seed=303)
    xp = vg.init_walkers(pre_walkers, LX * LY, NUP, NDN, seed=77, device=dev)
    cfg = vg.VMCLoopConfig(vmc_steps=sr_steps, ns_per_rank=pre_walkers, grad_batch_size=pre_walkers,
                           n_params=model.n_params, nsites=LX * LY, learning_rate=lr, diag_shift=1e-3,
                           burn_in_steps=10, factored_o=True)
    drv = vg.VMC_GB300(plain, vg.MinSRGB300(), vg.SGDGB300(lr))
    t0 = time.time()
    hist, xp = drv.run_vmc_loop(xp, model, H, graph, 0, 1, cfg, on_step_end=hook)
    torch.cuda.synchronize()
    t_pre = time.time() - t0
    t_train = hook.train_seconds / max(hook.sessions, 1)

    x = vg.init_walkers(n_walkers, LX * LY, NUP, NDN, seed=78, device=dev)
    plain.burn_in(x, model, graph, burn)
    learned = LearnedSamplerGB300(prop, moves_per_step=moves)

    def run(sampler, x0):
        xc = x0.clone()
        Es, ts, te = [], 0.0, 0.0
        for _ in range(samples):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            ev[0].record()
            sampler.step(xc, model, graph)
            ev[1].record()
            Es.append(vg.evaluate_energy(xc, model, H)[1])
            ev[2].record()
            torch.cuda.synchronize()
            ts += ev[0].elapsed_time(ev[1]) / 1e3
            te += ev[1].elapsed_time(ev[2]) / 1e3
        E = torch.stack(Es[discard:]).t().contiguous()
        tau = tau_int(E)
        nb, used = E.shape
        half = used // 2
        drift = [float(E[:, :half].mean().item()) / (LX * LY), float(E[:, half:].mean().item()) / (LX * LY)]
        ess = nb * used / tau
        f = used / samples
        return {"tau_int_samples": tau, "ess": ess, "sampler_s": ts, "eloc_s": te,
                "ms_per_sample": 1e3 * ts / samples, "eloc_ms_per_sample": 1e3 * te / samples,
                "ess_per_s": ess / (ts * f), "ess_per_s_with_eloc": ess / ((ts + te) * f),
                "energy_per_site": float(E.mean().item()) / (LX * LY),
                "stderr_per_site": float(E.std().item()) / (LX * LY) * (tau / (nb * used)) ** 0.5,
                "split_rhat": split_rhat(E), "energy_per_site_halves": drift}

    rp = run(plain, x)
    rl = run(learned, x)
    # (b): one training session per `every` samples, counted over the samples the estimate uses
    used_frac = (samples - discard) / samples
    train_s = (samples / every) * t_train * used_frac
    rl["ess_per_s_with_training"] = rl["ess"] / (rl["sampler_s"] * used_frac + train_s)
    rl["ess_per_s_with_training_and_eloc"] = rl["ess"] / ((rl["sampler_s"] + rl["eloc_s"]) * used_frac + train_s)
    rp["ess_per_s_with_training"] = rp["ess_per_s"]
    rp["ess_per_s_with_training_and_eloc"] = rp["ess_per_s_with_eloc"]
    acc = float((prop.k_acc.sum() / prop.k_prop.sum().clamp_min(1)).item())
    dE = abs(rp["energy_per_site"] - rl["energy_per_site"])
    ratio = {k: rl[k] / rp[k] for k in ("ess_per_s", "ess_per_s_with_training", "ess_per_s_with_eloc",
                                        "ess_per_s_with_training_and_eloc")}
    return {"plain": rp, "learned": rl,
            "ratio_learned_over_plain": {"a_sampler_only": ratio["ess_per_s"],
                                         "b_with_training_schedule": ratio["ess_per_s_with_training"],
                                         "c_with_local_energy": ratio["ess_per_s_with_eloc"],
                                         "b_and_c": ratio["ess_per_s_with_training_and_eloc"]},
            "ess_ratio_learned_over_plain": ratio["ess_per_s"],
            "abs_dE_per_site": dE, "matched_energy_1e-3": dE < 1e-3,
            "dE_sigma": dE / (rp["stderr_per_site"] ** 2 + rl["stderr_per_site"] ** 2) ** 0.5,
            "walkers": n_walkers, "samples_per_chain": samples, "discarded_per_chain": discard,
            "burn_in_sweeps": burn,
            "learned_moves_per_sample": moves, "learned_acceptance": acc,
            "wavefunction": {"sr_steps_before_measuring": sr_steps, "sr_walkers": pre_walkers, "lr": lr,
                             "diag_shift": 1e-3, "energy_per_site_first_last": [hist[0], hist[-1]],
                             "seconds": t_pre},
            "training": {"schedule": "every %d SR steps, %d epochs over the last %d samples, batches of 16384"
                                     % (every, epochs, prop.cap),
                         "sessions": hook.sessions, "seconds_per_session": t_train, "last_loss": hook.last_loss},
            "proposal": "MLP 128->512->512 GELU (BF16 tcgen05 inference, FP32 CUDA-core training), k<=4 hops"}


# ---------------------------------------------------------------------------
def sr_block(model, H, fxs, dev, fp32_peak_tflops, diag_shift=1e-4):
    """Configs 2-3's SR path at the headline size: the hand-written adjoint O
    (dense block + Kronecker factors of the out_w block) for every walker, the
    local energies, then minSR (centring, dense Gram on the tensor cores with
    the fixed-point digit split, the Kronecker-corrected head block, FP64
    Cholesky, solves, update); the same solve with the CUDA-core Gram is
    timed beside it with the difference of the two directions.  Device time per stage (CUDA events on the
    current stream) and the algorithmic FLOP of each: dense Gram
    2 Ns^2 Np_dense, head 2 Ns^2 (2N nf + 256) (+ the mean 2 Ns 2N nf 256),
    Cholesky Ns^3 / 3."""
    import torch
    import vmc_torch_gb300 as vg
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return r, e0.elapsed_time(e1)

    # warm-up on 1024 walkers (module loads and first-use compilation), then
    # the full size twice: the second pass is the steady state of a VMC loop
    sub = fxs[:1024].clone()
    Fw, _ = vg.compute_grads_factored(sub, model)
    _, Ew = vg.evaluate_energy(sub, model, H)
    vg.MinSRGB300().solve(local_o=Fw, local_energies=Ew, energy_mean=float(Ew.mean()), total_samples=1024,
                          n_params=model.n_params, diag_shift=diag_shift, device=dev, run_sr=True)
    del Fw, Ew, sub
    first = {}
    for rep in range(2):
        (F, _), grad_ms = timed(lambda: vg.compute_grads_factored(fxs, model))
        (_, E), eloc_ms = timed(lambda: vg.evaluate_energy(fxs, model, H))
        if rep == 0:
            first = {"logpsi_grad_ms": grad_ms, "local_energy_ms": eloc_ms}
            del F
    solver = vg.MinSRGB300(record_stages=True)
    (dp, _, info), sr_ms = timed(lambda: solver.solve(local_o=F, local_energies=E, energy_mean=float(E.mean()),
                                                      total_samples=fxs.shape[0], n_params=model.n_params,
                                                      diag_shift=diag_shift, device=dev, run_sr=True))
    Ns, Nd = F.dense.shape
    Ng, Nh = F.g.shape[1], F.h.shape[1]
    st = solver.last_stages or {}
    fl = {"gram_dense": 2.0 * Ns * Ns * Nd, "gram_head": 2.0 * Ns * Ns * (Ng + Nh) + 2.0 * Ns * Ng * Nh,
          "cholesky": Ns ** 3 / 3.0}
    stages = {}
    for k, ms in st.items():
        d = {"ms": ms}
        if k in fl:
            d["tflops"] = fl[k] / (ms / 1e3) / 1e12
            d["flop"] = fl[k]
        stages[k] = d
    if "gram_dense" in stages:
        # nine BF16 products per counted multiply-add, on the lower triangle of 128 x 128 tiles only
        nt = -(-Ns // 128)
        ex = 9 * stages["gram_dense"]["tflops"] * (nt + 1) / (2.0 * nt)
        stages["gram_dense"]["tensor_tflops_executed"] = ex
        stages["gram_dense"]["frac_of_bf16_measured"] = ex / peaks()["bf16_tflops"]
    if "cholesky" in stages:
        stages["cholesky"]["frac_of_fp64_nominal"] = stages["cholesky"]["tflops"] / 1.25
    o_bytes = Ns * (Nd + Ng + Nh) * F.dense.element_size()
    # the same solve with the Gram blocks on the CUDA cores (compensated accumulation: the exact Gram of the FP32 rows)
    tsolver = vg.MinSRGB300(record_stages=True, gram="cuda")
    tsolver.solve(local_o=F, local_energies=E, energy_mean=float(E.mean()), total_samples=Ns,
                  n_params=model.n_params, diag_shift=diag_shift, device=dev, run_sr=True)   # warm-up
    (dpt, _, tinfo), tsr_ms = timed(lambda: tsolver.solve(local_o=F, local_energies=E, energy_mean=float(E.mean()),
                                                          total_samples=Ns, n_params=model.n_params,
                                                          diag_shift=diag_shift, device=dev, run_sr=True))
    tstages = {}
    for k, ms in (tsolver.last_stages or {}).items():
        d = {"ms": ms}
        if k in fl:
            d["tflops"] = fl[k] / (ms / 1e3) / 1e12
        tstages[k] = d
    cuda_gram = {"minsr_ms": tsr_ms, "minsr_stages": tstages, "info": tinfo,
                 "dp_rel_diff_vs_tensor_gram": float((dpt - dp).norm().item() / dp.norm().item())}
    return {"workload": "8x8 NNBF, %d walkers: per-sample O (FP32, dense %d + Kronecker %d x %d), E_loc, minSR "
                        "over %d parameters (diag shift %g)" % (Ns, Nd, Ng, Nh, model.n_params, diag_shift),
            "logpsi_grad_ms": grad_ms, "first_full_size_call": first, "O_bytes_written": o_bytes,
            "O_write_gbs": o_bytes / (grad_ms / 1e3) / 1e9, "local_energy_ms": eloc_ms, "minsr_ms": sr_ms,
            "minsr_stages": stages, "info": info, "dp_norm": float(dp.norm().item()), "cuda_gram": cuda_gram,
            "peaks": "FP32 nominal %.1f TFLOP/s (152 SM x 128 lanes x 2 x max SM clock), FP64 nominal 1.25 TFLOP/s"
                     % fp32_peak_tflops}


# ---------------------------------------------------------------------------
def run_gb300(args):
    import torch
    import vmc_torch_gb300 as vg
    from vmc_torch_gb300 import build as vbuild

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if not os.path.exists(vbuild.LIB):
        vbuild.build()

    gen = torch.Generator().manual_seed(1234 + rank)
    model = vg.NNBF_GB300(LX * LY, NUP + NDN, hidden_dim=HID, n_layers=2, bf_scale=BF_SCALE, precision="mixed",
                          generator=gen).to(dev)
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(LX, LY, 1.0, 8.0, NUP + NDN, n_fermions_per_spin=(NUP, NDN))
    H.precompute_hops_gpu(dev)
    graph = H.graph
    E = len(graph.sweep_edges())
    fxs = vg.init_walkers(B, LX * LY, NUP, NDN, seed=7 + 1000 * rank, device=dev)
    smp = vg.MetropolisExchangeSpinfulSamplerGB300(seed=11 + rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # burn-in + warm-up (untimed)
    smp.burn_in(fxs, model, graph, 2, use_log_amp=True)
    for _ in range(args.warmup):
        smp.step(fxs, model, graph, use_log_amp=True)
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    instr = {}
    st = model.bind_state(fxs)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.3)
    total_ms = 0.0
    stream = torch.cuda.current_stream(dev)
    for k in range(args.steps):
        flush.fill_(float(k))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        smp.step(fxs, model, graph, use_log_amp=True)
        e1.record(stream)
        torch.cuda.synchronize()
        total_ms += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    clocks = clk.stop()
    # same steps again with CUDA events around every kernel launch (per-kernel
    # device time on the launching stream) for the roofline / kernel shares
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        smp.step(fxs, model, graph, use_log_amp=True, instrument=instr)
    torch.cuda.synchronize()
    value, total_ms = replica_rate(args.steps * B * E, total_ms, dist, dev)
    n_eval = int(instr["n_eval"].item())
    stage_ms = list(instr["stage_ms"])
    stage_n = list(instr["stage_launches"])
    eloc_check = None

    # ---- roofline of the dominant kernel (device time share inside the timed region) ----
    names = ["prep (proposal + first layer)", "hidden layer GEMM (tcgen05)", "backflow GEMM (tcgen05, persistent)",
             "LU log-det + accept (FP32 CUDA cores)"]
    pk = peaks()
    nf = NUP + NDN
    # algorithmic work per launch
    lu_flops = n_eval * (2.0 / 3.0) * nf ** 3
    bf_flops = args.steps * E * B * 2.0 * HID * (2 * LX * LY * nf)
    l1_flops = args.steps * E * B * 2.0 * HID * HID
    per_kernel = []
    for i, (nm, ms, n) in enumerate(zip(names, stage_ms, stage_n)):
        per_kernel.append({"kernel": nm, "launches": n, "ms_total": ms, "share": ms / max(sum(stage_ms), 1e-9)})
    dom = int(np.argmax(stage_ms))
    kern_flops = [0.0, l1_flops, bf_flops, lu_flops]
    achieved = kern_flops[dom] / (stage_ms[dom] / 1e3) / 1e12
    # DRAM bytes per LU launch (4096-row chunk, compacted rows) from one ncu capture
    # (cold cache) of the kernel the per-kernel pass times: read 52.58 MB + write 0.02 MB
    lu_traffic = 52.583936e6 + 0.016896e6 if dom == 3 else None
    roofline = {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": achieved / pk["bf16_tflops"], "traffic": lu_traffic,
                "traffic_note": "ncu dram__bytes_read+write per 4096-row LU launch, cold-cache capture",
                "kernel": names[dom], "peak_source": pk["source"] + " (bf16 burst, MEASURED_PEAKS.json)",
                "algorithmic": "LU: (2/3) nf^3 FLOP per evaluated proposal (nf=64); GEMMs: 2*M*N*K",
                "per_kernel": per_kernel,
                "backflow_gemm_tflops": bf_flops / (stage_ms[2] / 1e3) / 1e12 if stage_ms[2] else None,
                # per_kernel times come from a pass with the chunk pipeline and walker
                # groups off (every launch alone on the GPU); in the timed steps the LU
                # overlaps the GEMMs and the other groups' launches.  LU work completed
                # per unit of step time:
                "lu_tflops_in_step": lu_flops / args.steps / (total_ms / args.steps / 1e3) / 1e12,
                "hidden_gemm_tflops": l1_flops / (stage_ms[1] / 1e3) / 1e12 if stage_ms[1] else None}

    # ---- end-to-end through the public API with host buffers ----
    host_fx = torch.empty((B, LX * LY), dtype=torch.int64).pin_memory()
    host_fx.copy_(fxs.cpu())
    host_la = torch.empty(B, dtype=torch.float64).pin_memory()
    host_sg = torch.empty(B, dtype=torch.float64).pin_memory()
    dev_fx = torch.empty_like(fxs)
    torch.cuda.synchronize()
    e2e_ms = 0.0
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        dev_fx.copy_(host_fx, non_blocking=True)
        _, (sg, la) = smp.step(dev_fx, model, graph, use_log_amp=True)
        host_fx.copy_(dev_fx, non_blocking=True)
        host_sg.copy_(sg, non_blocking=True)
        host_la.copy_(la, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms += e0.elapsed_time(e1)
    e2e_value, _ = replica_rate(args.steps * B * E, e2e_ms, dist, dev)
    h2d = B * LX * LY * 8
    d2h = B * LX * LY * 8 + 2 * B * 8
    n_chunks = -(-B // 4096)
    # Launches of the timed steps.  The sweep runs G walker groups (the library
    # splits B >= 8192 walkers into min(VMC_GB300_SWEEP_LANES, B // 4096)
    # groups, default 4), each launching per edge a prep kernel, the hidden
    # GEMM and (backflow GEMM + LU) per 4096-row chunk of the group; per step
    # also the refresh (prep, hidden GEMM, n_chunks x (backflow GEMM + LU)) and
    # the unpack of the configurations.
    lanes = max(1, min(4, int(os.environ.get("VMC_GB300_SWEEP_LANES", "4"))))
    G = min(lanes, B // 4096) if B >= 2 * 4096 and lanes > 1 else 1
    bg = -(-B // G)
    per_edge = sum(2 + 2 * -(-min(bg, B - g * bg) // 4096) for g in range(G) if g * bg < B)
    gpu_launches = args.steps * (E * per_edge + 2 + 2 * n_chunks + 1)

    smax = clocks.get("sm_max_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * smax * 1e6 / 1e12
    sr = None
    if not args.no_sr:
        try:
            sr = sr_block(model, H, fxs, dev, fp32_peak)
        except Exception as e:   # reported in the line; the headline numbers stand
            sr = {"error": "%s: %s" % (type(e).__name__, e)}
    ess = None
    if not args.no_ess:
        try:
            ess = ess_block(dev, B)
        except Exception as e:
            ess = {"error": "%s: %s" % (type(e).__name__, e)}
    peps = peps_block(dev, 2, fp32_peak, cpu=(rank == 0 and not args.no_cpu_baseline)) if not args.no_peps else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count()
        if os.path.isdir(os.path.join(REF_ROOT, "vmc_torch")):
            pool = reference_pool(cores, 16)
            try:
                t0 = time.perf_counter()
                reference_rate(pool, cores)   # warm-up round
                rates = [reference_rate(pool, cores) for _ in range(3)]
                dt = time.perf_counter() - t0
            finally:
                pool.close()
                pool.join()
            cpu = {"value": float(np.mean(rates)), "unit": UNIT, "cores": cores, "kind": "reference",
                   "sample": "the reference's MetropolisExchangeSpinfulSamplerGPU + NNBF_GPU(2x256 GELU) on the "
                             "host CPU: %d single-thread processes x 16 chains, 3 timed sweeps" % cores,
                   "seconds": dt}
        else:
            r, dt, sample = cpu_port_rate(n_walkers=48, n_sweeps=1)
            cpu = {"value": r, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample, "seconds": dt}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "bf16 MLP / fp32 det",
                "data": "synthetic (seeded walkers and random-init weights)",
                "config": workload_config({"accepted_per_walker_per_step":
                                           float(st.n_acc.float().mean().item()) if st is not None else None,
                                           "evaluated_proposals_per_step": n_eval / args.steps}),
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": gpu_launches,
                "ess": ess, "sr": sr, "fpeps": peps}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def free_port():
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def spawn_replicas(n, argv):
    """``--gpus N`` outside a launcher: start N ranks of this script, one per
    GPU, through torch.distributed.run on 127.0.0.1, and return the launcher's
    exit status.  Each rank runs its own replica; rank 0 prints the line."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.abspath(__file__)] + list(argv)
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ess", action="store_true", help="skip the learned-vs-plain ESS/s comparison")
    ap.add_argument("--no-peps", action="store_true", help="skip the secondary 6x6 fPEPS workload")
    ap.add_argument("--no-sr", action="store_true", help="skip the O + minSR block at the headline size")
    ap.add_argument("--peps-only", action="store_true",
                    help="run only the fPEPS block (print its JSON object); for profiling")
    ap.add_argument("--peps-walkers", type=int, default=PEPS_B, help="walkers of the fPEPS block (default 8192)")
    ap.add_argument("--peps-recompute", action="store_true",
                    help="fPEPS block without cached column environments (every amplitude from scratch)")
    ap.add_argument("--walkers", type=int, default=B,
                    help="walkers per GPU (the headline workload uses 16384; smaller values are for profiling)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return spawn_replicas(args.gpus, sys.argv[1:])
    globals()["B"] = args.walkers
    if args.warmup < 3:
        args.warmup = 3
    globals()["PEPS_B"] = args.peps_walkers
    if args.impl == "reference":
        return run_reference(args)
    if args.peps_only:
        import torch
        from vmc_torch_gb300 import build as vbuild
        if not os.path.exists(vbuild.LIB):
            vbuild.build()
        print(json.dumps(peps_block(torch.device("cuda", 0), args.steps, 152 * 128 * 2 * 2070e6 / 1e12,
                                    cpu=False, env_reuse=not args.peps_recompute)), flush=True)
        return 0
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
