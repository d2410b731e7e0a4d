"""Drop-in proof: the reference's own driver, VMC_GPU.run_vmc_loop
(vmc_torch/GPU/VMC.py:645-847), runs three SR steps of the 4x2 Slater
workload with this library's objects injected in every slot
(vmc_torch/GPU/VMC.py:160-172): sampler, preconditioner, optimizer,
evaluate_energy_fn and compute_grads_fn.  The reference is imported from its
pip install in baseline/_ref under the import shims of its absent
tensor-network / MPI dependencies (one NCCL rank on this GPU for its
collectives).  Its energy history equals VMC_GB300.run_vmc_loop's on the same
objects, seeds and walkers, and the parameters end where this package's own
driver leaves them.
"""
import os
import socket

import numpy as np
import pytest
import torch

import vmc_torch_gb300 as vg

pytestmark = pytest.mark.gpu
DEV = "cuda"
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "baseline", "_ref")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _setup():
    gen = torch.Generator().manual_seed(0)
    model = vg.SlaterDeterminant_GB300(16, 8, init_std=0.1, generator=gen).to(DEV)
    H = vg.spinful_Fermi_Hubbard_square_lattice_torch(4, 2, 1.0, 8.0, 8, n_fermions_per_spin=(4, 4))
    H.precompute_hops_gpu(DEV)
    fx = vg.init_walkers(1024, 8, 4, 4, seed=2, device=DEV)
    objs = dict(sampler=vg.MetropolisExchangeSpinfulSamplerGB300(seed=1, sweeps_per_step=2),
                preconditioner=vg.MinSRGB300(), optimizer=vg.SGDGB300(0.1),
                evaluate_energy_fn=vg.evaluate_energy, compute_grads_fn=vg.compute_grads_gpu)
    return model, H, fx, objs


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "vmc_torch")), reason="reference not installed in baseline/_ref")
def test_reference_driver_runs_with_gb300_objects():
    from oracle import refshim
    RV = refshim.load("vmc_torch.GPU.VMC", REF)
    import torch.distributed as dist
    own_group = not dist.is_initialized()
    if own_group:
        os.environ["MASTER_ADDR"] = "127.0.0.1"
        os.environ["MASTER_PORT"] = str(_free_port())
        dist.init_process_group("nccl", rank=0, world_size=1)
    try:
        steps = 3
        model, H, fx, objs = _setup()
        drv = RV.VMC_GPU(**objs)
        cfg = RV.VMCLoopConfig(vmc_steps=steps, ns_per_rank=1024, grad_batch_size=512, n_params=model.n_params,
                               nsites=8, learning_rate=0.1, diag_shift=1e-4, burn_in_steps=20, show_progress=False,
                               outlier_clip_factor=0.0)
        seen = []
        hist, fx = drv.run_vmc_loop(fx, model, H, H.graph, 0, 1, cfg, on_step_end=lambda info: seen.append(info))
        M_ref = model.params[0].detach().clone()
        # the same objects and seeds through this package's driver
        model2, H2, fx2, objs2 = _setup()
        own = vg.VMC_GB300(**objs2)
        cfg2 = vg.VMCLoopConfig(vmc_steps=steps, ns_per_rank=1024, grad_batch_size=512, n_params=model2.n_params,
                                nsites=8, learning_rate=0.1, diag_shift=1e-4, burn_in_steps=20, outlier_clip_factor=0.0)
        hist2, fx2 = own.run_vmc_loop(fx2, model2, H2, H2.graph, 0, 1, cfg2)
    finally:
        if own_group:
            dist.destroy_process_group()
    print("reference driver E/site:", np.round(hist, 6), " VMC_GB300:", np.round(hist2, 6))
    assert len(hist) == steps and all(np.isfinite(hist))
    assert [s["step"] for s in seen] == list(range(steps)) and all(s["solver_info"] == 0 for s in seen)
    np.testing.assert_allclose(hist, hist2, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(M_ref.cpu().numpy(), model2.params[0].detach().cpu().numpy(), rtol=1e-8, atol=1e-12)
    assert torch.equal(fx, fx2)
