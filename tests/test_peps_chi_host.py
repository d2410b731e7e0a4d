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
