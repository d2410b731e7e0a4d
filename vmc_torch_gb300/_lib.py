"""ctypes binding of libvmc_gb300.so (the C ABI declared in include/vmc_gb300.h).

The library is built in-tree (``vmc_torch_gb300/build.py``).  There is no CPU
fallback: if the library is missing or a CUDA device is absent, every entry
point raises.
"""
import ctypes
import os

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libvmc_gb300.so")

(VMC_OK, VMC_ERR_ARGS, VMC_ERR_CUDA, VMC_ERR_NONFINITE, VMC_ERR_SINGULAR, VMC_ERR_TIMEOUT, VMC_ERR_UNSUPPORTED,
 VMC_ERR_CAPACITY) = range(8)
_MSG = {
    VMC_ERR_CAPACITY: "request exceeds a fixed built-in capacity",
    VMC_ERR_ARGS: "invalid arguments (sizes, null pointers or unsupported shape)",
    VMC_ERR_CUDA: "CUDA launch failed",
    VMC_ERR_NONFINITE: "non-finite amplitude or energy",
    VMC_ERR_SINGULAR: "singular orbital matrix",
    VMC_ERR_TIMEOUT: "a bounded device-side wait gave up",
    VMC_ERR_UNSUPPORTED: "configuration not supported by libvmc_gb300",
}

P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int
U64 = ctypes.c_uint64
F64 = ctypes.c_double
F32 = ctypes.c_float

# name -> argtypes (every function returns int status)
SIGNATURES = {
    "vmc_abi_version": [],
    "vmc_pack": [P, I64, I32, P, P, P],
    "vmc_unpack": [P, I64, I32, P, P],
    "vmc_init_walkers": [P, I64, I32, I32, I32, U64, P],
    "vmc_hubbard_conn": [P, I64, I32, P, I32, F64, F64, P, P, P, P],
    "vmc_slater_refresh": [P, I32, I32, P, I64, I32, P, P, P, P, P, I32, P, P],
    "vmc_slater_sweep": [P, I32, I32, P, I64, I32, P, I32, I32, F32, U64, U64, P, P, P, P, P, P, P, P, P],
    "vmc_slater_local_energy": [P, I32, I32, P, I64, I32, P, I32, F64, F64, P, P, P, P],
    "vmc_slater_logpsi_grad": [P, P, I64, I32, I32, P, I64, P],
    "vmc_nnbf_eval": [I32, P, I32, I32, I32, F64, P, I64, P, P, P, P, P, P, P, P],
    "vmc_nnbf_sweep": [I32, P, I32, I32, I32, F64, P, I64, P, I32, I32, F32, U64, U64, P, P, P, P, P, P, P, P, P,
                       P, P, P, P, P, P, P, P, P],
    "vmc_nnbf_eval_noalloc": [P, I32, I32, I32, F64, P, I64, P, P, P, P],
    "vmc_nnbf_hidden_layer": [P, I64, P, P, P, U64, I32, P, P],
    "vmc_check_finite": [P, P, I64, P, I32, I64, I64, P, P, P, P, P],
    "vmc_prop_logits": [P, I32, P, I64, P, P, P, P, P, P],
    "vmc_prop_sample": [P, I32, I32, P, P, I64, U64, U64, P, P, P],
    "vmc_prop_reverse": [P, I32, I32, P, P, I64, P, P],
    "vmc_accept_mh": [P, I64, P, P, P, P, P, P, P, P, P, P, P],
    "vmc_nnbf_mh_step": [P, I32, I32, I32, F64, P, I64, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P],
    "vmc_prop_train_step": [I32, P, I32, P, I32, P, P, P, F32, P, P, P, P, I64, F32, F32, F32, F32, I32, P, P, P],
    "vmc_prop_inputs_f32": [I32, P, I64, P, P],
    "vmc_prop_collect_targets": [P, I64, P, F64, I32, I64, P, P],
    "vmc_nnbf_logpsi_grad": [I32, P, I32, I32, I32, F64, P, I64, P, I64, P, I64, P, P, P, P, P],
    "vmc_nnbf_conn_count": [P, I64, I32, P, I32, P, P],
    "vmc_nnbf_conn_pairs": [P, I64, I32, P, I32, P, P, P],
    "vmc_nnbf_local_energy": [I32, P, I32, I32, I32, F64, P, I64, P, F64, F64, P, P, P, P, P, I64, I64, P, P, P, P,
                              P, P, P, P, P],
    "vmc_sr_center": [P, I32, I64, I64, I64, P, I64, P, P],
    "vmc_sr_gram": [P, I32, I64, I64, I64, P, I64, F64, I32, P],
    "vmc_sr_cholesky": [P, I64, I64, P, P],
    "vmc_split_bf16x3": [P, I64, I64, I64, P, I64, I64, P, P],
    "vmc_sr_gram_tc": [P, P, I64, I64, I64, F64, P, I64, P, F64, I32, P, P],
    "vmc_sr_cholesky_solve": [P, I64, I64, P, P],
    "vmc_sr_rhs": [P, I64, F64, P, P],
    "vmc_sr_update": [P, I32, I64, I64, I64, P, P, P],
    "vmc_energy_gradient": [P, I32, I64, I64, I64, P, F64, P, P],
    "vmc_gemm": [I32, I32, I64, I64, I64, F64, P, I64, P, I64, P, I32, F64, P, I64, P, I64, I32, P],
    "vmc_sr_kron_correction": [I64, P, I64, P, I64, P, I32, I64, I64, F64, F64, P, P],
    "vmc_peps_eval": [I32, P, I32, I32, I32, P, I64, P, P, P],
    "vmc_peps_sweep": [I32, P, I32, I32, I32, P, I64, P, I32, I32, F32, U64, U64, P, P, P, P, P, P, P, P, I64, P,
                       P],
    "vmc_peps_local_energy": [I32, P, I32, I32, I32, P, I64, P, F64, F64, P, P, P, P, I64, P, P, P, I64, P, P],
    "vmc_peps_logpsi_grad": [I32, P, I32, I32, I32, P, I64, P, I64, P, I64, P],
    "vmc_peps_chi_work_bytes": [I32, I32, I32, I32, I32, I64, P],
    "vmc_peps_chi_schedule": [I32, I32, I32, I32, P, I32],
    "vmc_peps_chi_eval": [I32, P, I32, I32, I32, I32, P, I64, P, P, P, I64, P],
    "vmc_peps_chi_sweep": [I32, P, I32, I32, I32, I32, P, I64, P, I32, I32, F32, U64, U64, P, P, P, P, P, P, P, P,
                           I64, P],
    "vmc_peps_chi_local_energy": [I32, P, I32, I32, I32, I32, P, I64, P, F64, F64, P, P, P, I64, P, P, P, I64, P],
    "vmc_peps_chi_grad_work_bytes": [I32, I32, I32, I32, I32, I64, P],
    "vmc_peps_chi_logpsi_grad": [I32, P, I32, I32, I32, I32, P, I64, P, I64, P, I64, P],
    "vmc_sym_images": [P, I64, I32, P, P, I32, P, P, P],
    "vmc_sym_combine": [P, P, P, P, I64, I32, P, P, P, P],
    "vmc_sym_grad_combine": [I32, P, I64, P, I64, I32, I64, P, I64, P],
    "vmc_propose_edge": [P, I64, I32, P, I32, I32, I32, F32, U64, U64, P, P, P, P, P, P, P],
    "vmc_accept_edge": [P, I64, P, P, P, P, P, P, P, P, P],
    "vmc_conn_rows": [P, I64, P, I32, P, F64, P, P, P],
    "vmc_eloc_terms": [P, I64, P, P, P, P, P, P, P],
    "vmc_eloc_reduce": [P, I64, P, P, F64, P, P],
}

_lib = None


def load():
    """Load the library (once) and declare every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "libvmc_gb300.so is not built (expected at %s); run __graft_entry__.build() or "
            "python vmc_torch_gb300/build.py" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    _lib = lib
    return lib


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream_of(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def call(name, *args):
    """Call an entry point and raise on a non-zero status."""
    st = getattr(load(), name)(*args)
    if st != VMC_OK:
        raise ValueError("%s failed: %s (status %d)" % (name, _MSG.get(st, "unknown"), st))
    return st


def call_status(name, *args, allow=()):
    """Call an entry point; return its status when it is VMC_OK or in
    ``allow`` (statuses that report a condition rather than a failure), else
    raise."""
    st = getattr(load(), name)(*args)
    if st != VMC_OK and st not in allow:
        raise ValueError("%s failed: %s (status %d)" % (name, _MSG.get(st, "unknown"), st))
    return st


def message(status):
    return _MSG.get(status, "unknown status %d" % status)


def require_cuda(t, what="tensor"):
    if not (isinstance(t, torch.Tensor) and t.is_cuda):
        raise ValueError("%s must be a CUDA tensor: the GB300 path has no CPU fallback" % what)
