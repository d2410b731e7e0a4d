"""Metropolis exchange-or-hop sampler with the reference's sampler interface
(vmc_torch/GPU/sampler.py:140-388): ``step(fxs, model, graph, ...)`` performs
one sweep over all lattice edges for every walker, mutates ``fxs`` in place and
returns ``(fxs, amps)`` or ``(fxs, (signs, log_abs))``; ``burn_in`` runs
several sweeps.

All edges of all requested sweeps run inside one kernel launch: each walker's
chain is independent, so no host round trip or device-wide barrier separates
the edges (the reference launches several torch ops per edge and syncs the
host at ``new_flags.sum().item()``).
"""
import torch

from . import _lib
from .models import floor_log


class SamplerGB300:
    """Base interface (vmc_torch/GPU/sampler.py:140-197)."""

    def step(self, fxs, model, graph, **kwargs):
        raise NotImplementedError

    def burn_in(self, fxs, model, graph, n_steps, **kwargs):
        for _ in range(n_steps):
            fxs, _ = self.step(fxs, model, graph, **kwargs)
        return fxs


class MetropolisExchangeSpinfulSamplerGB300(SamplerGB300):
    """Exchange-or-hop Metropolis sampler for spinful fermions.

    Args:
        hopping_rate: fraction of hop (vs exchange) proposals, default 0.25.
        seed: Philox key of the device random stream.
        sweeps_per_step: sweeps performed by one ``step`` call (the reference
            does one).
    Random stream: counter-based, keyed by (walker, global sweep index, edge);
    ``replay=(u_move, hop_bit, u_acc)`` CUDA tensors of shape
    (n_sweeps, E, B) replace it (deterministic replay of a recorded stream).
    """

    def __init__(self, hopping_rate=0.25, seed=0, sweeps_per_step=1):
        self.hopping_rate = hopping_rate
        self.seed = seed
        self.sweeps_per_step = sweeps_per_step
        self.sweep_counter = 0

    def _run(self, fxs, model, graph, n_sweeps, use_log_amp, replay, instrument=None):
        st = model.bind_state(fxs)
        model.check_status(st)   # a status copy of earlier work that has landed; never waits
        if instrument is None:
            model.sweep(st, graph, n_sweeps, self.seed, self.sweep_counter, self.hopping_rate, replay)
        else:
            model.sweep(st, graph, n_sweeps, self.seed, self.sweep_counter, self.hopping_rate, replay,
                        instrument=instrument)
        model._watch_err(st)
        self.sweep_counter += n_sweeps
        model.store_configs(st, fxs)
        if use_log_amp:
            return fxs, (st.sign.clone(), floor_log(st.logabs))
        return fxs, st.sign * torch.exp(st.logabs)

    @torch.inference_mode()
    def step(self, fxs, model, graph, compile=False, verbose=False, use_log_amp=False, replay=None, instrument=None,
             **kwargs):
        return self._run(fxs, model, graph, self.sweeps_per_step, use_log_amp, replay, instrument)

    @torch.inference_mode()
    def burn_in(self, fxs, model, graph, n_steps, use_log_amp=False, replay=None, **kwargs):
        if n_steps <= 0:
            return fxs
        self._run(fxs, model, graph, n_steps * self.sweeps_per_step, use_log_amp, replay)
        return fxs
