"""Local energy and per-sample log-derivatives with the reference's function
signatures:

  * ``evaluate_energy(fxs, model, H, current_amps, use_log_amp, verbose, ...)
    -> (E_mean, local_E)`` (vmc_torch/GPU/vmc_utils.py:322-506);
  * ``compute_grads_gpu(fxs, model, batch_size, ..., offload_to_cpu,
    use_log_amp) -> (grads (B, Np), amps)`` or ``(O, (signs, log_abs))`` in
    log mode (vmc_torch/GPU/vmc_utils.py:1389-1634).  In amplitude mode the
    reference returns d psi / d theta and the driver divides by psi
    (vmc_torch/GPU/VMC.py:453); the same contract is kept.  ``batch_size``
    walkers are differentiated per launch; with ``offload_to_cpu`` each chunk
    goes straight to pinned host memory, so the device holds two chunks, not
    the (B, Np) matrix (vmc_torch/GPU/vmc_utils.py:1484-1609).

Both gradient functions end with the reference's checks
(``_check_grads_amps``, vmc_torch/GPU/vmc_utils.py:1330-1386): NaN or Inf in
the amplitudes (log mode: log|psi|) or in O raises ``ValueError`` with the
reference's message.  Amplitudes below the reference's 1e-45 floor report
log|psi| = log(1e-45) and zero log-derivatives, as the reference's clamped
log-amplitude does; they are counted (``last_check``), not raised.
"""
import ctypes

import torch

from . import _lib
from .models import LOG_MIN, floor_log

# counts of the last gradient check: {"zero_amplitudes": n, "samples": B}
last_check = {}


@torch.inference_mode()
def evaluate_energy(fxs, model, H, current_amps=None, use_log_amp=False, verbose=False, return_bMPS=False, **kwargs):
    st = model.bind_state(fxs)
    model.check_status(st)
    eloc = model.local_energy(st, H)
    model._watch_err(st)
    return eloc.mean(), eloc


def _count(amp, sign, O, Np, device, col_flags=False):
    """Run vmc_check_finite: (status, [nan, inf, zero, bad rows], row flags, column flags)."""
    counts = torch.empty(4, dtype=torch.int64, device=device)
    B = (amp if amp is not None else sign).shape[0] if (amp is not None or sign is not None) else O.shape[0]
    rows = cols = None
    if O is not None and col_flags:
        rows = torch.empty(O.shape[0], dtype=torch.uint8, device=device)
        cols = torch.empty(max(Np, 1), dtype=torch.uint8, device=device)
    host = (ctypes.c_ulonglong * 4)()
    dt = 0 if O is None or O.dtype == torch.float64 else 1
    st = _lib.call_status("vmc_check_finite", _lib.ptr(amp), _lib.ptr(sign), B if O is None else O.shape[0],
                          _lib.ptr(O), dt, Np if O is not None else 0, O.stride(0) if O is not None else 0,
                          _lib.ptr(counts), _lib.ptr(rows), _lib.ptr(cols), host, _lib.stream_of(device),
                          allow=(_lib.VMC_ERR_NONFINITE, _lib.VMC_ERR_SINGULAR))
    return st, [int(v) for v in host], rows, cols


def _param_ranges(model):
    out, off = [], 0
    for i, p in enumerate(model.params):
        out.append((i, off, off + p.numel(), tuple(p.shape)))
        off += p.numel()
    return out


def _raise_grads(model, n_bad, B, bad_ids, n_bad_params, Np):
    info = []
    ranges = _param_ranges(model)
    for pid in bad_ids[:10]:
        for (idx, lo, hi, shape) in ranges:
            if lo <= pid < hi:
                info.append("  flat[%d] -> params[%d]%s offset %d" % (pid, idx, list(shape), pid - lo))
                break
    raise ValueError("NaN/Inf in gradients: %d/%d samples affected, %d/%d params affected.\nFirst bad params:\n"
                     % (n_bad, B, n_bad_params, Np) + "\n".join(info))


def _check_amps(amp, sign):
    """First half of the reference's _check_grads_amps: NaN/Inf amplitudes
    (log mode: log|psi|) raise; zero amplitudes are counted."""
    B = amp.shape[0]
    _, c, _, _ = _count(amp, sign, None, 0, amp.device)
    if c[0] or c[1]:
        raise ValueError("NaN/Inf in amplitudes: %d NaN, %d Inf out of %d samples" % (c[0], c[1], B))
    last_check.clear()
    last_check.update({"zero_amplitudes": c[2], "samples": B})


def _check_grads_amps(O, amp, sign, model):
    """The reference's _check_grads_amps on the device: amplitudes first
    (log mode: log|psi|), then the O rows."""
    _check_amps(amp, sign)
    _check_O(O, model)


def _check_O(O, model):
    """Second half: NaN/Inf entries of O raise with the reference's message
    (samples and parameters affected, the first bad parameters)."""
    from .optimizer import FactoredO
    dev = O.device
    B = O.shape[0]
    if isinstance(O, FactoredO):
        parts = [O.dense, O.g, O.h]
        res = [_count(None, None, t, t.shape[1], dev) for t in parts]
        if not any(r[1][3] for r in res):
            return
        res = [_count(None, None, t, t.shape[1], dev, col_flags=True) for t in parts]
        rows = res[0][2].bool() | res[1][2].bool() | res[2][2].bool()
        cd, cg, ch = (r[3].bool().cpu() for r in res)
        Ng, Nh, off = O.g.shape[1], O.h.shape[1], O.offset
        ids = [j if j < off else j + Ng * Nh for j in torch.nonzero(cd).flatten().tolist()]
        kb = (cg[:, None] | ch[None, :]).reshape(-1)
        ids += [off + j for j in torch.nonzero(kb).flatten().tolist()]
        ids.sort()
        _raise_grads(model, int(rows.sum().item()), B, ids, len(ids), O.n_params)
    Np = O.shape[1]
    st, c, _, _ = _count(None, None, O, Np, dev)
    if c[3]:
        _, c, _, cols = _count(None, None, O, Np, dev, col_flags=True)
        bad = torch.nonzero(cols[:Np]).flatten()
        _raise_grads(model, c[3], B, bad[:10].tolist(), int(bad.numel()), Np)


def _floor_rows(O, logabs):
    """Zero the O rows of walkers below the 1e-45 amplitude floor (the
    gradient of the reference's clamp), without a host synchronisation."""
    from .optimizer import FactoredO
    small = (logabs < LOG_MIN).unsqueeze(1)
    if isinstance(O, FactoredO):
        for t in (O.dense, O.g, O.h):
            t.masked_fill_(small, 0)
    else:
        O.masked_fill_(small, 0)


def compute_grads_factored(fxs, model, use_log_amp=True, **kwargs):
    """Log-derivatives with the NNBF output-layer block in Kronecker-factored
    form (``optimizer.FactoredO``), for sample-space SR at scale.  Always in log
    mode: returns (FactoredO, (signs, log_abs))."""
    from .optimizer import FactoredO
    # no_grad, not inference mode: the returned tensors are ordinary tensors
    # that the caller may update in place (the reference's driver divides O
    # by the amplitudes in place, vmc_torch/GPU/VMC.py:453)
    with torch.no_grad():
        st = model.bind_state(fxs)
        Od, g, h = model.logpsi_grad_factored(st)
        model.check_status(st, wait=True)
        off = model.n_params - model.n_params_out_w - model.n_orbitals * model.n_fermions
        F = FactoredO(Od, g, h, off)
        _floor_rows(F, st.logabs)
        la = floor_log(st.logabs)
        _check_grads_amps(F, la, st.sign, model)
        return F, (st.sign.clone(), la)


def compute_grads_gpu(fxs, model, batch_size=None, verbose=False, offload_to_cpu=False, use_log_amp=False,
                      vectorize=True, vmap_grad=True, bMPS_params_x=None, **kwargs):
    # no_grad, not inference mode: O, the amplitudes and the log-amplitudes are
    # returned as ordinary tensors the caller may update in place (the
    # reference's driver divides O by the amplitudes in place,
    # vmc_torch/GPU/VMC.py:453)
    with torch.no_grad():
        st = model.bind_state(fxs)
        B, Np = st.B, model.n_params
        bs = int(batch_size) if batch_size else B
        if bs <= 0:
            raise ValueError("batch_size must be positive")
        la = floor_log(st.logabs)
        sign = st.sign.clone()
        amps = sign * torch.exp(st.logabs)
        small = st.logabs < LOG_MIN
        if not offload_to_cpu:
            if bs >= B:
                O = model.logpsi_grad(st)
            else:
                O = None
                for a in range(0, B, bs):
                    b = min(B, a + bs)
                    if O is None:   # the first chunk gives the dtype of O
                        Oc = model.logpsi_grad(st.view(a, b))
                        O = torch.empty((B, Np), dtype=Oc.dtype, device=st.device)
                        O[a:b].copy_(Oc)
                        del Oc
                    else:
                        model.logpsi_grad(st.view(a, b), out=O[a:b])
            model.check_status(st, wait=True)
            O.masked_fill_(small.unsqueeze(1), 0)
            _check_grads_amps(O, la if use_log_amp else amps, sign, model)
            if use_log_amp:
                return O, (sign, la)
            return O.mul_(amps.to(O.dtype).unsqueeze(1)), amps
        # offload: two device chunk buffers alternate; each chunk is counted on
        # the device, scaled (amplitude mode) and copied to pinned host memory
        _check_amps(la if use_log_amp else amps, sign)
        n_bad = 0
        Oh = None
        cur = torch.cuda.current_stream(st.device)
        done = [None, None]
        bufs = [None, None]
        for k, a in enumerate(range(0, B, bs)):
            b = min(B, a + bs)
            i = k & 1
            if done[i] is not None:
                done[i].synchronize()
            v = st.view(a, b)
            Oc = model.logpsi_grad(v, out=bufs[i][:b - a] if bufs[i] is not None else None)
            if bufs[i] is None:
                bufs[i] = Oc
            if Oh is None:
                Oh = torch.empty((B, Np), dtype=Oc.dtype, pin_memory=True)
            Oc.masked_fill_(small[a:b].unsqueeze(1), 0)
            n_bad += _count(None, None, Oc, Np, st.device)[1][3]
            if not use_log_amp:
                Oc.mul_(amps[a:b].to(Oc.dtype).unsqueeze(1))
            Oh[a:b].copy_(Oc, non_blocking=True)
            done[i] = torch.cuda.Event()
            done[i].record(cur)
        model.check_status(st, wait=True)
        torch.cuda.current_stream(st.device).synchronize()
        if n_bad:   # error path only: locate the bad entries in the host copy
            bad = ~torch.isfinite(Oh)
            cols = torch.nonzero(bad.any(0)).flatten()
            _raise_grads(model, int(bad.any(1).sum()), B, cols[:10].tolist(), int(cols.numel()), Np)
        if use_log_amp:
            return Oh, (sign.cpu(), la.cpu())
        return Oh, amps.cpu()
