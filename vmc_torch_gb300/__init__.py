"""GB300-native VMC inner loop (spinful Fermi-Hubbard, Slater / neural-backflow
/ fPEPS amplitudes, minSR) behind the interfaces of sjdu10/vmc_torch's batched path.

All compute runs in libvmc_gb300.so (hand-written sm_103a CUDA, C ABI in
include/vmc_gb300.h).  There is no CPU fallback.
"""
from . import _lib
from .energy import compute_grads_factored, compute_grads_gpu, evaluate_energy
from .hamiltonian import SpinfulFermion, SquareLattice, spinful_Fermi_Hubbard_square_lattice_torch
from .models import FPEPS_GB300, NNBF_GB300, SlaterDeterminant_GB300, WavefunctionModel_GB300
from .optimizer import FactoredO, MinSRGB300, SGDGB300
from .sampler import MetropolisExchangeSpinfulSamplerGB300
from .symmetry import FermionSymmetryProjectedModel_GB300, build_symmetry_group
from .vmc import VMC_GB300, VMCLoopConfig
from .walkers import init_walkers, pack, unpack

__all__ = [
    "SquareLattice", "SpinfulFermion", "spinful_Fermi_Hubbard_square_lattice_torch",
    "WavefunctionModel_GB300", "SlaterDeterminant_GB300", "NNBF_GB300", "FPEPS_GB300",
    "FermionSymmetryProjectedModel_GB300", "build_symmetry_group",
    "MetropolisExchangeSpinfulSamplerGB300", "evaluate_energy", "compute_grads_gpu", "compute_grads_factored",
    "MinSRGB300", "SGDGB300", "FactoredO", "VMC_GB300", "VMCLoopConfig", "pack", "unpack", "init_walkers",
]


def load_library():
    return _lib.load()
