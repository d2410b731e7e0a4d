"""Checkpoint and statistics files interchangeable with the reference's run
scripts (vmc_torch/GPU/run_scripts/vmcconfig.py:131-224): the fixtures were
written by the reference's own callback for its 4x2 NNBF_GPU and
SlaterDeterminant_GPU models (tests/golden/make_golden.py)."""
import json
import os
import shutil

import numpy as np
import torch

import vmc_torch_gb300 as vg
from vmc_torch_gb300 import checkpoint as ck
from oracle.lattice import random_initial_configs
from oracle.models import nnbf_init

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _stage(tmp_path, name, model_name, step):
    shutil.copy(os.path.join(GOLD, name), ck.checkpoint_path(str(tmp_path), model_name, step))


def test_reference_nnbf_checkpoint_loads(tmp_path):
    _stage(tmp_path, "ckpt_nnbf_4x2.pt", "NNBF", 1)
    m = vg.NNBF_GB300(8, 8, hidden_dim=256, n_layers=2, bf_scale=0.01)
    fxs = ck.load_checkpoint(m, str(tmp_path), "NNBF", 1, "cpu", rank=1)
    for p, v in zip(m.params, nnbf_init(8, 8, 256, 2, seed=5)):
        assert p.dtype == torch.float64 and np.array_equal(p.detach().numpy(), v)
    assert np.array_equal(fxs.numpy(), random_initial_configs(6, 8, 4, 4, seed=6))


def test_reference_slater_checkpoint_loads(tmp_path):
    _stage(tmp_path, "ckpt_slater_4x2.pt", "Slater", 1)
    m = vg.SlaterDeterminant_GB300(16, 8)
    ck.load_checkpoint(m, str(tmp_path), "Slater", 1, "cpu", rank=1)
    assert np.array_equal(m.params[0].detach().numpy(), np.random.default_rng(8).standard_normal((16, 8)))
    assert ck.load_checkpoint(m, str(tmp_path), "Slater", 0, "cpu") is None  # resume_step 0: nothing to load


def test_written_files_match_reference_format(tmp_path):
    ref = torch.load(os.path.join(GOLD, "ckpt_nnbf_4x2.pt"), weights_only=True)
    m = vg.NNBF_GB300(8, 8, hidden_dim=256, n_layers=2, bf_scale=0.01)
    stats = ck.make_stats("4x2 t=1 U=8 N=8", m.n_params, 6, 1)
    sf = ck.make_stats_file(str(tmp_path), "NNBF", 0)
    fxs = torch.as_tensor(random_initial_configs(6, 8, 4, 4, seed=6))
    cb = ck.make_on_step_end(0, stats, sf, str(tmp_path), "NNBF", m, 1)
    cb({"step": 0, "energy_per_site": -0.25, "error_per_site": 0.01, "energy_var": 0.5, "fxs": fxs})
    ours = torch.load(ck.checkpoint_path(str(tmp_path), "NNBF", 1), weights_only=True)
    assert set(ours) == set(ref) == {"model_state_dict", "fxs"}
    assert list(ours["model_state_dict"]) == list(ref["model_state_dict"])
    for k in ref["model_state_dict"]:
        assert ours["model_state_dict"][k].shape == ref["model_state_dict"][k].shape
        assert ours["model_state_dict"][k].dtype == ref["model_state_dict"][k].dtype
    assert torch.equal(ours["fxs"], ref["fxs"])
    assert json.load(open(sf)) == json.load(open(os.path.join(GOLD, "ckpt_nnbf_4x2_stats.json")))
    assert os.path.basename(ck.make_stats_file("d", "NNBF", 26, "_reuse")) == "stats_NNBF_reuse_from26.json"


def test_roundtrip_and_bare_state_dict(tmp_path):
    g = torch.Generator().manual_seed(3)
    a = vg.SlaterDeterminant_GB300(16, 8, generator=g)
    b = vg.SlaterDeterminant_GB300(16, 8)
    fx = torch.as_tensor(random_initial_configs(4, 8, 4, 4, seed=1))
    ck.save_checkpoint(ck.checkpoint_path(str(tmp_path), "S", 3), a, fx)
    got = ck.load_checkpoint(b, str(tmp_path), "S", 3, "cpu", rank=1)
    assert torch.equal(a.params[0], b.params[0]) and torch.equal(got, fx)
    torch.save(a.state_dict(), ck.checkpoint_path(str(tmp_path), "S", 4))  # the older bare format
    c = vg.SlaterDeterminant_GB300(16, 8)
    assert ck.load_checkpoint(c, str(tmp_path), "S", 4, "cpu", rank=1) is None
    assert torch.equal(a.params[0], c.params[0])
