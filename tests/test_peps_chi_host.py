"""Host logic of the chi-truncated fPEPS path (no GPU): the C library's
truncation schedule equals the oracle's, the model picks the exact kernels
exactly when no cut can exceed chi, and the workspace query validates its
arguments."""
import ctypes

import pytest

from oracle import peps
import vmc_torch_gb300 as vg
from vmc_torch_gb300 import _lib


@pytest.fixture(scope="module", autouse=True)
def built():
    from vmc_torch_gb300 import build
    build.build()


@pytest.mark.parametrize("Lx,Ly,D,chi", [(6, 6, 4, 16), (6, 6, 4, 8), (6, 6, 4, 64), (4, 4, 4, 3), (8, 8, 2, 4),
                                         (8, 6, 4, 16), (4, 6, 4, 8), (2, 6, 4, 1), (10, 6, 4, 16)])
def test_schedule_matches_oracle(Lx, Ly, D, chi):
    assert vg.FPEPS_GB300.chi_schedule(Lx, Ly, D, chi) == peps.chi_schedule(Lx, Ly, D, chi)


def test_model_path_selection():
    assert vg.FPEPS_GB300(6, 6, 4, max_bond=16).truncated
    assert not vg.FPEPS_GB300(6, 6, 4, max_bond=64).truncated
    assert not vg.FPEPS_GB300(6, 6, 4, max_bond=None).truncated
    assert not vg.FPEPS_GB300(6, 6, 4, max_bond=0).truncated      # the reference's chi > 0 test
    m = vg.FPEPS_GB300(10, 6, 4, max_bond=16)                        # beyond the exact kernels' Lx range
    assert m.truncated and m.chi_cuts[-1] == [3]
    with pytest.raises(ValueError):
        vg.FPEPS_GB300(8, 8, 4, max_bond=16)                         # D^Ly = 65536 states per side


def test_work_bytes_and_errors():
    nb = ctypes.c_int64(0)
    assert _lib.load().vmc_peps_chi_work_bytes(0, 6, 6, 4, 16, 1024, ctypes.byref(nb)) == _lib.VMC_OK
    assert nb.value >= 1024 * 4 * 4096 * 4
    assert _lib.load().vmc_peps_chi_work_bytes(0, 8, 8, 4, 16, 1024, ctypes.byref(nb)) == _lib.VMC_ERR_UNSUPPORTED
    assert _lib.load().vmc_peps_chi_work_bytes(2, 6, 6, 4, 16, 1024, ctypes.byref(nb)) == _lib.VMC_ERR_ARGS
    assert _lib.load().vmc_peps_chi_work_bytes(0, 6, 6, 4, 16, 0, ctypes.byref(nb)) == _lib.VMC_ERR_ARGS


def test_chi_entry_points_reject_bad_arguments():
    """The chi C entry points validate precision, lattice support, sizes and
    pointers before any GPU work (so these calls run without a GPU)."""
    L = _lib.load()
    vp = ctypes.c_void_p(1)   # never dereferenced: every call below fails its checks first
    assert L.vmc_peps_chi_eval(2, vp, 6, 6, 4, 16, vp, 4, vp, vp, vp, 8, None) == _lib.VMC_ERR_ARGS
    assert L.vmc_peps_chi_eval(0, vp, 8, 8, 4, 16, vp, 4, vp, vp, vp, 8, None) == _lib.VMC_ERR_UNSUPPORTED
    assert L.vmc_peps_chi_eval(0, vp, 6, 6, 4, 16, vp, -1, vp, vp, vp, 8, None) == _lib.VMC_ERR_ARGS
    assert L.vmc_peps_chi_eval(0, None, 6, 6, 4, 16, vp, 4, vp, vp, vp, 8, None) == _lib.VMC_ERR_ARGS
    assert L.vmc_peps_chi_eval(0, vp, 6, 6, 4, 16, vp, 0, vp, vp, vp, 8, None) == _lib.VMC_OK   # nothing to do
    # sweep: replay buffers all or none
    assert L.vmc_peps_chi_sweep(0, vp, 6, 6, 4, 16, vp, 4, vp, 60, 1, ctypes.c_float(0.25), 1, 0, vp, None, None,
                                vp, vp, None, None, vp, 8, None) == _lib.VMC_ERR_ARGS
    # local energy: host offsets must start at 0 and end at P
    offs = (ctypes.c_int32 * 3)(0, 5, 9)
    assert L.vmc_peps_chi_local_energy(0, vp, 6, 6, 4, 16, vp, 2, vp, ctypes.c_double(1.0), ctypes.c_double(8.0), vp,
                                       vp, offs, 10, vp, vp, vp, 8, None) == _lib.VMC_ERR_ARGS
    # log-derivatives: schedules with truncations before the last row are not supported
    nb = ctypes.c_int64(0)
    assert L.vmc_peps_chi_grad_work_bytes(0, 6, 6, 4, 8, 64, ctypes.byref(nb)) == _lib.VMC_ERR_UNSUPPORTED
    assert L.vmc_peps_chi_logpsi_grad(0, vp, 6, 6, 4, 8, vp, 4, vp, 36864, vp, 8, None) == _lib.VMC_ERR_UNSUPPORTED
    assert L.vmc_peps_chi_logpsi_grad(0, vp, 6, 6, 4, 16, vp, 4, vp, 100, vp, 8, None) == _lib.VMC_ERR_ARGS  # ldo


def test_gram_split_rejects_bad_arguments():
    L = _lib.load()
    vp = ctypes.c_void_p(1)
    # rows_pad not a multiple of 128, kp not a multiple of 64, missing row exponents
    assert L.vmc_split_bf16x3(vp, 100, 64, 64, vp, 100, 64, vp, None) == _lib.VMC_ERR_ARGS
    assert L.vmc_split_bf16x3(vp, 100, 64, 64, vp, 128, 60, vp, None) == _lib.VMC_ERR_ARGS
    assert L.vmc_split_bf16x3(vp, 100, 64, 64, vp, 128, 64, None, None) == _lib.VMC_ERR_ARGS
    assert L.vmc_sr_gram_tc(vp, None, 100, 128, 64, ctypes.c_double(1.0), vp, 100, None, ctypes.c_double(0.0), 0,
                            vp, None) == _lib.VMC_ERR_ARGS
