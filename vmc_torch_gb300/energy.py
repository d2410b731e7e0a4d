"""Local energy and per-sample log-derivatives with the reference's function
signatures:

  * ``evaluate_energy(fxs, model, H, current_amps, use_log_amp, verbose, ...)
    -> (E_mean, local_E)`` (vmc_torch/GPU/vmc_utils.py:322-506);
  * ``compute_grads_gpu(fxs, model, batch_size, ..., use_log_amp) ->
    (grads (B, Np), amps)`` or ``(O, (signs, log_abs))`` in log mode
    (vmc_torch/GPU/vmc_utils.py:1389-1634).  In amplitude mode the reference
    returns d psi / d theta and the driver divides by psi
    (vmc_torch/GPU/VMC.py:453); the same contract is kept.
"""
import torch


@torch.inference_mode()
def evaluate_energy(fxs, model, H, current_amps=None, use_log_amp=False, verbose=False, return_bMPS=False, **kwargs):
    st = model.bind_state(fxs)
    eloc = model.local_energy(st, H)
    return eloc.mean(), eloc


def compute_grads_factored(fxs, model, use_log_amp=True, **kwargs):
    """Log-derivatives with the NNBF output-layer block in Kronecker-factored
    form (``optimizer.FactoredO``), for sample-space SR at scale.  Always in log
    mode: returns (FactoredO, (signs, log_abs))."""
    from .optimizer import FactoredO
    with torch.inference_mode():
        st = model.bind_state(fxs)
        Od, g, h = model.logpsi_grad_factored(st)
        off = model.n_params - model.n_params_out_w - model.n_orbitals * model.n_fermions
        return FactoredO(Od, g, h, off), (st.sign.clone(), st.logabs.clone())


def compute_grads_gpu(fxs, model, batch_size=None, verbose=False, offload_to_cpu=False, use_log_amp=False,
                      vectorize=True, vmap_grad=True, bMPS_params_x=None, **kwargs):
    with torch.inference_mode():
        st = model.bind_state(fxs)
        O = model.logpsi_grad(st)
        if use_log_amp:
            aux = (st.sign.clone(), st.logabs.clone())
            if offload_to_cpu:
                return O.cpu(), (aux[0].cpu(), aux[1].cpu())
            return O, aux
        amps = st.sign * torch.exp(st.logabs)
        g = O.mul_(amps.to(O.dtype).unsqueeze(1))
        if offload_to_cpu:
            return g.cpu(), amps.cpu()
        return g, amps
