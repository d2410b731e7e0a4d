"""Checkpoints and run statistics in the reference's formats
(vmc_torch/GPU/run_scripts/vmcconfig.py:131-224).

A checkpoint is ``torch.save({'model_state_dict': model.state_dict(), 'fxs':
fxs.cpu()}, '<dir>/checkpoint_<model>_<step>.pt')``; loading also accepts a
bare state dict (the older format).  The models keep the reference's
parameter container (``params.0``, ``params.1``, ... in the reference's
order), so state dicts move between these models and the reference's GPU
models of the same architecture in either direction, and the saved walkers
resume the chains.  The statistics file is the reference's JSON with
``system``, ``Np``, ``sample size`` and per-step ``mean`` / ``error`` /
``variance``.
"""
import json
import os

import torch


def checkpoint_path(output_dir, model_name, step):
    return os.path.join(output_dir, f"checkpoint_{model_name}_{step}.pt")


def save_checkpoint(path, model, fxs):
    torch.save({"model_state_dict": model.state_dict(), "fxs": fxs.detach().cpu()}, path)


def load_checkpoint(model, output_dir, model_name, resume_step, device, rank=0):
    """Load ``checkpoint_<model_name>_<resume_step>.pt`` into ``model`` when
    resume_step > 0 (vmcconfig.py:131-158).  Returns the saved walkers (int64
    on ``device``) when the file has them, else None."""
    if resume_step <= 0:
        return None
    path = checkpoint_path(output_dir, model_name, resume_step)
    ckpt = torch.load(path, map_location=device, weights_only=True)
    fxs = None
    if isinstance(ckpt, dict) and "model_state_dict" in ckpt:
        model.load_state_dict(ckpt["model_state_dict"])
        if "fxs" in ckpt:
            fxs = ckpt["fxs"].to(device=device, dtype=torch.int64)
    else:
        model.load_state_dict(ckpt)
    if hasattr(model, "invalidate"):
        model.invalidate()
    if rank == 0:
        print(f"Loaded checkpoint: {path}")
    return fxs


def make_stats(system_str, n_params, ns_per_rank, world_size):
    return {"system": system_str, "Np": n_params, "sample size": ns_per_rank * world_size, "mean": [], "error": [],
            "variance": []}


def make_stats_file(output_dir, model_name, resume_step, suffix=""):
    step_tag = f"_from{resume_step}" if resume_step > 0 else ""
    return os.path.join(output_dir, f"stats_{model_name}{suffix}{step_tag}.json")


def make_on_step_end(rank, stats, stats_file, output_dir, model_name, model, save_every):
    """Callback for ``run_vmc_loop``: appends the step's statistics to the JSON
    file and saves a checkpoint every ``save_every`` steps (rank 0)."""
    def on_step_end(info):
        if rank != 0:
            return
        stats["mean"].append(info["energy_per_site"])
        stats["error"].append(info["error_per_site"])
        stats["variance"].append(info["energy_var"])
        with open(stats_file, "w") as f:
            json.dump(stats, f, indent=4)
        step = info["step"]
        if (step + 1) % save_every == 0:
            save_checkpoint(checkpoint_path(output_dir, model_name, step + 1), model, info["fxs"])

    return on_step_end
