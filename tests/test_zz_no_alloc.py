"""The allocation-free evaluation entry point.

vmc_nnbf_eval_noalloc serves callers that cannot allocate device memory while
they run (a fixed memory budget set up once, a real-time loop, a framework
that owns the whole device pool).  It must give the same log-amplitudes as
the workspace-taking entry point, on consecutive calls that share its fixed
scratch array, and refuse batches beyond its capacity.

This file is named so that pytest collects it after every other test file;
it passes both on its own in a fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import lattice, models as om
import vmc_torch_gb300 as vg
from vmc_torch_gb300 import _lib

pytestmark = pytest.mark.gpu
DEV = "cuda"
CAPACITY = 512


def _model():
    ps = om.nnbf_init(64, 64, 256, 2, seed=77)
    m = vg.NNBF_GB300(64, 64, precision="mixed").to(DEV)
    with torch.no_grad():
        for p, v in zip(m.params, ps):
            p.copy_(torch.as_tensor(v))
    m.invalidate()
    return m


def _noalloc(m, occ, R):
    ts, arr = m.net(occ.device)
    sign = torch.full((R,), 7.0, dtype=torch.float64, device=DEV)
    logabs = torch.full((R,), 7.0, dtype=torch.float64, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    st = _lib.load().vmc_nnbf_eval_noalloc(arr, 64, 64, 256, m.bf_scale, _lib.ptr(occ), R, _lib.ptr(sign),
                                           _lib.ptr(logabs), _lib.ptr(err), _lib.stream_of(occ.device))
    return st, sign, logabs, err


def test_noalloc_matches_workspace_entry_point_on_consecutive_calls():
    m = _model()
    for seed, R in ((3, 300), (4, CAPACITY)):  # two calls in a row, the second at full capacity
        X = torch.as_tensor(lattice.random_initial_configs(R, 64, 32, 32, seed=seed), device=DEV)
        occ = vg.pack(X)
        st, s, l, err = _noalloc(m, occ, R)
        assert st == 0
        s_ref, l_ref = m.forward_log(X)  # vmc_nnbf_eval with caller-allocated workspace
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        assert torch.equal(s, s_ref)
        np.testing.assert_allclose(l.cpu().numpy(), l_ref.cpu().numpy(), rtol=0, atol=1e-9)


def test_noalloc_rejects_batches_beyond_capacity():
    m = _model()
    X = torch.as_tensor(lattice.random_initial_configs(CAPACITY + 1, 64, 32, 32, seed=5), device=DEV)
    st, _, _, _ = _noalloc(m, vg.pack(X), CAPACITY + 1)
    assert st == _lib.VMC_ERR_CAPACITY


def test_noalloc_allocates_nothing_after_its_first_call():
    """After one warm-up call (which loads the library's module on the device,
    committing the fixed array, and resolves its address), a full-capacity call
    takes no device memory: the free memory the driver reports (which counts
    allocations made outside torch as well) does not drop, and torch's own
    allocator holds exactly the caller's tensors."""
    m = _model()
    X = torch.as_tensor(lattice.random_initial_configs(CAPACITY, 64, 32, 32, seed=6), device=DEV)
    occ = vg.pack(X)
    st, _, _, _ = _noalloc(m, occ, CAPACITY)   # warm-up
    assert st == 0
    ts, arr = m.net(occ.device)
    sign = torch.empty(CAPACITY, dtype=torch.float64, device=DEV)
    logabs = torch.empty_like(sign)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    held0 = torch.cuda.memory_allocated()
    st = _lib.load().vmc_nnbf_eval_noalloc(arr, 64, 64, 256, m.bf_scale, _lib.ptr(occ), CAPACITY, _lib.ptr(sign),
                                           _lib.ptr(logabs), _lib.ptr(err), _lib.stream_of(occ.device))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert st == 0 and int(err.item()) == 0
    assert torch.cuda.memory_allocated() == held0
    assert free1 >= free0 - (1 << 20), "the call took %d bytes of device memory" % (free0 - free1)

