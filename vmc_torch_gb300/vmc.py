"""Single-GPU VMC driver with the reference's loop structure
(VMC_GPU, vmc_torch/GPU/VMC.py:151-847): the sampler, preconditioner,
optimizer, energy and gradient functions are injected exactly as in the
reference, so the same objects plug into either driver.

Per step: sampling phase (sweep -> local energy -> O, repeated until
``ns_per_rank`` samples) -> energy statistics -> SR solve -> parameter update
-> ``on_step_end`` callback.  With one GPU there is no collective: the
reference's all_reduce / broadcast become on-device reductions.
"""
import time
from dataclasses import dataclass, fields
from typing import Any, Callable, Dict, Optional

import torch

from .energy import compute_grads_factored, compute_grads_gpu, evaluate_energy
from .optimizer import FactoredO


@dataclass
class VMCLoopConfig:
    """Fields of vmc_torch/GPU/VMC.py:89-148 used on this path."""
    vmc_steps: int
    ns_per_rank: int
    grad_batch_size: int
    n_params: int
    nsites: int
    learning_rate: float = 0.1
    diag_shift: float = 1e-4
    burn_in_steps: int = 0
    run_sr: bool = True
    use_log_amp: bool = False
    outlier_clip_factor: float = 100.0
    lr_scheduler: object = None
    verbose: bool = False
    step_offset: int = 0       # global step of the first iteration (resumed runs)
    show_progress: bool = False
    factored_o: bool = False   # NNBF: Kronecker-factored out_w block of O (FactoredO)

    def __init__(self, **kwargs):
        for f in fields(self):
            setattr(self, f.name, kwargs.pop(f.name, f.default))
        for k, v in kwargs.items():
            setattr(self, k, v)


class VMC_GB300:
    def __init__(self, sampler, preconditioner=None, optimizer=None, evaluate_energy_fn: Callable = evaluate_energy,
                 compute_grads_fn: Callable = compute_grads_gpu):
        self.sampler = sampler
        self.preconditioner = preconditioner
        self.optimizer = optimizer
        self.evaluate_energy_fn = evaluate_energy_fn
        self.compute_grads_fn = compute_grads_fn

    def _run_sampling_phase(self, fxs, model, hamiltonian, graph, ns_per_rank, grad_batch_size, burn_in=False,
                            burn_in_steps=0, outlier_clip_factor=0.0, use_log_amp=False, verbose=False,
                            factored_o=False):
        B = fxs.shape[0]
        t_samp = t_locE = t_grad = 0.0
        if burn_in and burn_in_steps > 0:
            fxs = self.sampler.burn_in(fxs, model, graph, burn_in_steps, use_log_amp=use_log_amp)
        Es, Os = [], []
        count = 0
        while count < ns_per_rank:
            need = min(B, ns_per_rank - count)
            t0 = time.time()
            fxs, amps = self.sampler.step(fxs, model, graph, use_log_amp=use_log_amp)
            t_samp += time.time() - t0
            t0 = time.time()
            res = self.evaluate_energy_fn(fxs, model, hamiltonian, amps, use_log_amp=use_log_amp)
            local_E = res[1]
            t_locE += time.time() - t0
            t0 = time.time()
            if factored_o:
                grads, aux = compute_grads_factored(fxs, model)
            else:
                grads, aux = self.compute_grads_fn(fxs, model, batch_size=grad_batch_size, use_log_amp=use_log_amp)
                if not use_log_amp:
                    grads = grads / aux.to(grads.dtype).unsqueeze(1)
            t_grad += time.time() - t0
            Es.append(local_E[:need])
            Os.append(grads[:need])
            count += need
        local_E = torch.cat(Es)
        O = FactoredO.cat(Os) if factored_o else torch.cat(Os)
        if outlier_clip_factor > 0:
            norms = O.row_norms() if factored_o else O.norm(dim=1)
            keep = norms <= outlier_clip_factor * norms.median()
            if not bool(keep.all()):
                if factored_o:
                    O.zero_rows(~keep)
                else:
                    O[~keep] = 0.0
                local_E[~keep] = local_E[keep].mean()
        times = {"t_samp": t_samp, "t_locE": t_locE, "t_grad": t_grad}
        return (local_E, O), fxs, t_samp + t_locE + t_grad, times

    @staticmethod
    def compute_global_energy_stats(local_energies):
        n = local_energies.shape[0]
        m = local_energies.mean()
        var = (local_energies ** 2).mean() - m * m
        return n, float(m.item()), float(var.item())

    def run_vmc_loop(self, fxs, model, hamiltonian, graph, rank=0, world_size=1, config: VMCLoopConfig = None,
                     on_step_end: Optional[Callable[[Dict[str, Any]], None]] = None):
        """The reference's loop contract (vmc_torch/GPU/VMC.py:645-847): returns
        (energy_history, fxs) with the energy per site of every step, and calls
        on_step_end with the reference's info keys.  One process drives one GPU
        (rank 0 of 1); the per-step records with timings are kept in
        ``self.history``."""
        if config is None:
            if isinstance(rank, VMCLoopConfig):  # run_vmc_loop(fxs, model, H, graph, config)
                config, rank, world_size = rank, 0, 1
            else:
                raise ValueError("run_vmc_loop needs a VMCLoopConfig")
        if world_size != 1:
            raise ValueError("VMC_GB300 drives one GPU per process (world_size 1)")
        device = next(model.parameters()).device
        self.history = []
        energy_history = []
        for step in range(config.vmc_steps):
            t0 = time.time()
            (E, O), fxs, ts, times = self._run_sampling_phase(
                fxs, model, hamiltonian, graph, config.ns_per_rank, config.grad_batch_size, burn_in=(step == 0),
                burn_in_steps=config.burn_in_steps, outlier_clip_factor=config.outlier_clip_factor,
                use_log_amp=config.use_log_amp, verbose=config.verbose, factored_o=config.factored_o)
            n, Em, Evar = self.compute_global_energy_stats(E)
            dp, t_sr, info = self.preconditioner.solve(
                local_o=O, local_energies=E, energy_mean=Em, total_samples=n, n_params=config.n_params,
                diag_shift=config.diag_shift, device=device, run_sr=config.run_sr)
            global_step = step + config.step_offset
            if config.lr_scheduler is not None:
                config.learning_rate = config.lr_scheduler(global_step)
            self.optimizer.step(model=model, direction=dp, device=device, learning_rate=config.learning_rate)
            t_step = time.time() - t0
            e_site = Em / config.nsites
            err = (max(Evar, 0.0) / n) ** 0.5 / config.nsites
            energy_history.append(e_site)
            rec = {"step": global_step, "energy": Em, "energy_per_site": e_site, "variance": Evar,
                   "error": (max(Evar, 0.0) / n) ** 0.5, "t_step": t_step, "t_sr": t_sr, "sr_info": info, **times}
            self.history.append(rec)
            if config.show_progress:
                print("Step %3d | E/site: %.6f +/- %.6f | N=%d | T_samp=%.2fs T_locE=%.2fs T_grad=%.2fs T_SR=%.2fs"
                      % (global_step, e_site, err, n, times["t_samp"], times["t_locE"], times["t_grad"], t_sr))
            if on_step_end is not None:
                on_step_end({"step": global_step, "energy_mean": Em, "energy_var": Evar, "energy_per_site": e_site,
                             "error_per_site": err, "total_samples": n, "sample_time": ts, "phase_times": times,
                             "sr_time": t_sr, "total_time": t_step, "solver_info": info, "fxs": fxs})
        return energy_history, fxs
