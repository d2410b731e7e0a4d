"""Walker encodings on the device: quimb int64 (B, N) <-> packed uint64 (B, 2)
``[up_bits, dn_bits]`` (stored as int64 tensors), and seeded sector
initialisation (role of vmc_torch/GPU/vmc_utils.py:22-39 and
vmc_torch/GPU/vmc_setup.py:139-159)."""
import torch

from . import _lib


def pack(fxs):
    """(B, N) int64 quimb configs -> (B, 2) packed occupations.  Raises
    ValueError on values outside {0,1,2,3} (reference: invalid configuration,
    vmc_torch/sampler.py:1628)."""
    _lib.require_cuda(fxs, "fxs")
    if fxs.dtype != torch.int64 or fxs.dim() != 2:
        raise ValueError("fxs must be a (B, N_sites) int64 tensor")
    x = fxs.contiguous()
    B, N = x.shape
    occ = torch.empty((B, 2), dtype=torch.int64, device=x.device)
    bad = torch.zeros(1, dtype=torch.int32, device=x.device)
    _lib.call("vmc_pack", _lib.ptr(x), B, N, _lib.ptr(occ), _lib.ptr(bad), _lib.stream_of(x.device))
    if B and int(bad.item()):
        raise ValueError("Invalid configuration: site values must be in {0, 1, 2, 3}")
    return occ


def unpack(occ, n_sites, out=None):
    """(B, 2) packed -> (B, N) int64 quimb configs (written into ``out`` if given)."""
    B = occ.shape[0]
    if out is None:
        out = torch.empty((B, n_sites), dtype=torch.int64, device=occ.device)
    if not out.is_contiguous():
        raise ValueError("output config tensor must be contiguous")
    _lib.call("vmc_unpack", _lib.ptr(occ.contiguous()), B, n_sites, _lib.ptr(out), _lib.stream_of(occ.device))
    return out


def init_walkers(B, n_sites, n_up, n_dn, seed=0, device="cuda"):
    """(B, N) int64 random sector states, seeded (Philox on the device)."""
    occ = torch.empty((B, 2), dtype=torch.int64, device=device)
    _lib.call("vmc_init_walkers", _lib.ptr(occ), B, n_sites, n_up, n_dn, int(seed) & ((1 << 64) - 1),
              _lib.stream_of(occ.device))
    return unpack(occ, n_sites)
