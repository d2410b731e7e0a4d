"""Wavefunction models with the reference's model interface
(vmc_torch/GPU/models/_base.py:21-142): ``forward(x) -> (B,)`` amplitudes,
``forward_log(x) -> (signs, log_abs)``, single-sample ``amplitude(x,
params_list)`` and ``params`` (an ``nn.ParameterList`` whose flattened order is
the column order of O).

Behind the interface every evaluation runs in libvmc_gb300 kernels.  A model
keeps one persistent walker state (packed occupations plus the per-walker
amplitude data the kernels update in place) bound to the configuration tensor
it last saw; sampler, local energy and gradients share it.
"""
import ctypes
import math
import weakref

import torch
import torch.nn as nn

from . import _lib
from .walkers import pack, unpack

# The reference's log-amplitude is log(clamp(|psi|, min=1e-45))
# (vmc_torch/GPU/models/_base.py:101-109): zero and tiny amplitudes report this
# floor, and their log-derivatives are zero (the clamp's gradient).  The
# kernels keep the exact value (-inf for a singular orbital matrix) internally;
# every log-amplitude handed back through the reference's interfaces is
# floored the same way.
LOG_MIN = math.log(1e-45)


def floor_log(logabs):
    """Copy of a log-amplitude vector with the reference's 1e-45 floor (NaN
    stays NaN)."""
    return logabs.clamp(min=LOG_MIN)


class WalkerState:
    """Device buffers for B walkers, bound to one (B, N) config tensor."""

    def __init__(self, B, n_sites, device):
        self.B, self.n_sites, self.device = B, n_sites, device
        self.occ = torch.empty((B, 2), dtype=torch.int64, device=device)
        self.sign = torch.empty(B, dtype=torch.float64, device=device)
        self.logabs = torch.empty(B, dtype=torch.float64, device=device)
        self.n_acc = torch.zeros(B, dtype=torch.int32, device=device)
        self.key = None          # (weak reference, _version, shape) of the bound config tensor
        self.param_key = None    # model parameter fingerprint at the last refresh
        self.extra = {}

    def bound_to(self, fxs):
        """True when fxs is the very tensor last bound, unmodified since.  The
        tensor object is held by a weak reference: a data pointer alone is not
        enough, because a freed tensor's memory is handed to the next
        allocation of the same size."""
        if self.key is None:
            return False
        ref, ver, shape = self.key
        return ref() is fxs and ver == fxs._version and shape == tuple(fxs.shape)

    def bind(self, fxs):
        self.key = (weakref.ref(fxs), fxs._version, tuple(fxs.shape))

    def view(self, a, b):
        """Walkers a..b-1 as a state that shares this one's memory (every
        per-walker tensor sliced along its first axis); unbound."""
        v = WalkerState.__new__(WalkerState)
        v.B, v.n_sites, v.device = b - a, self.n_sites, self.device
        v.occ, v.sign, v.logabs, v.n_acc = self.occ[a:b], self.sign[a:b], self.logabs[a:b], self.n_acc[a:b]
        v.key = None
        v.param_key = self.param_key
        v.extra = {k: (t[a:b] if isinstance(t, torch.Tensor) and t.dim() > 0 and t.shape[0] == self.B and k != "err"
                       else t) for k, t in self.extra.items()}
        return v


class WavefunctionModel_GB300(nn.Module):
    """Base class: parameter list, state binding and the log/amp dispatch."""

    def __init__(self, params_list, n_sites):
        super().__init__()
        self.params = nn.ParameterList([p if isinstance(p, nn.Parameter) else nn.Parameter(p) for p in params_list])
        self.n_sites = n_sites
        self._state = None
        self._bump = 0

    # ---- parameter bookkeeping ----
    def invalidate(self):
        """Call after changing parameters through ``.data`` (which torch does not
        version-count); the optimizers in this package call it themselves."""
        self._bump += 1

    def param_key(self):
        return (self._bump,) + tuple((p.data_ptr(), p._version) for p in self.params)

    @property
    def n_params(self):
        return sum(p.numel() for p in self.params)

    # ---- state management ----
    def _new_state(self, B, device):
        return WalkerState(B, self.n_sites, device)

    @torch.inference_mode()
    def bind_state(self, fxs):
        """Return the walker state for ``fxs``, re-packing and re-evaluating the
        amplitudes when fxs or the parameters changed since the last use.  The
        state's tensors are inference tensors, updated in place by the kernels;
        values handed back to callers are copies."""
        _lib.require_cuda(fxs, "fxs")
        if fxs.dim() != 2 or fxs.shape[1] != self.n_sites:
            raise ValueError("fxs must be (B, %d) int64" % self.n_sites)
        st = self._state
        pk = self.param_key()
        if st is not None and st.B == fxs.shape[0] and st.device == fxs.device and st.bound_to(fxs) \
                and st.param_key == pk:
            return st
        if st is None or st.B != fxs.shape[0] or st.device != fxs.device:
            st = self._new_state(fxs.shape[0], fxs.device)
            self._state = st
        st.occ.copy_(pack(fxs))
        self._refresh(st, threshold=0)
        st.bind(fxs)
        st.param_key = pk
        return st

    @torch.inference_mode()
    def _eval_state(self, x):
        """A fresh state for arbitrary configs (not bound)."""
        st = self._new_state(x.shape[0], x.device)
        st.occ.copy_(pack(x))
        self._refresh(st, threshold=0)
        return st

    def store_configs(self, st, fxs):
        """Write the state's configurations into fxs in place and re-bind."""
        unpack(st.occ, self.n_sites, out=fxs)
        st.bind(fxs)

    # ---- device status ----
    def _err_word(self, st):
        """Device status word of the state's kernels (None for models whose
        kernels report through their return codes only)."""
        return st.extra.get("err")

    @torch.inference_mode()
    def _watch_err(self, st):
        """Queue a copy of the status word to pinned host memory behind the
        work just enqueued (no synchronisation)."""
        err = self._err_word(st)
        if err is None:
            return
        if "err_host" not in st.extra:
            st.extra["err_host"] = torch.zeros(1, dtype=torch.int32, pin_memory=True)
            st.extra["err_event"] = torch.cuda.Event()
        st.extra["err_host"].copy_(err, non_blocking=True)
        st.extra["err_event"].record(torch.cuda.current_stream(st.device))
        st.extra["err_pending"] = True

    @torch.inference_mode()
    def check_status(self, st, wait=False):
        """Raise if a kernel of this state reported an error (a bounded device
        wait that gave up, or configurations outside the model's sector).
        wait=False looks only at a status copy that has already landed, so
        the sampler never stalls the stream; wait=True reads the word now."""
        err = self._err_word(st)
        if err is None:
            return
        if wait:
            v = int(err.item())
        elif st.extra.get("err_pending") and st.extra["err_event"].query():
            st.extra["err_pending"] = False
            v = int(st.extra["err_host"].item())
        else:
            return
        if v != 0:
            err.zero_()
            raise ValueError("%s kernel reported status %d: %s" % (type(self).__name__, v, _lib.message(v)))

    # ---- reference interface ----
    def forward_log(self, x):
        if x.shape[0] == 0:
            z = torch.zeros(0, dtype=torch.float64, device=x.device)
            return z, z.clone()
        st = self._eval_state(x)
        self.check_status(st, wait=True)
        return st.sign.clone(), floor_log(st.logabs)

    def forward(self, x):
        s, la = self.forward_log(x)
        return s * torch.exp(la)

    def log_amplitude(self, x, params_list=None):
        s, la = self.forward_log(x.reshape(1, -1))
        return s[0], la[0]

    def take_singular_count(self):
        """Walkers whose orbital matrix was found singular (zero amplitude)
        since the last call; the count is reset.  Zero amplitudes are legal
        states in the reference (its sampler and energy carry on), so they are
        counted, not raised."""
        return 0

    def amplitude(self, x, params_list=None):
        """Single-sample amplitude (the model's current parameters are used; the
        reference passes them explicitly for torch.func transforms, which this
        library replaces with hand-written adjoints)."""
        return self.forward(x.reshape(1, -1))[0]

    def conn_pairs(self, st, H):
        """(pairs (P, 2) int32 [walker, hop term], offs (B+1) int32, P): every
        non-zero hop of every walker, term = 2*edge + (0 up, 1 down)."""
        edges = H.edges_on(st.device)
        cnt = torch.empty(st.B, dtype=torch.int32, device=st.device)
        _lib.call("vmc_nnbf_conn_count", _lib.ptr(st.occ), st.B, self.n_sites, _lib.ptr(edges), edges.shape[0],
                  _lib.ptr(cnt), _lib.stream_of(st.device))
        offs = torch.zeros(st.B + 1, dtype=torch.int32, device=st.device)
        offs[1:] = torch.cumsum(cnt, 0)
        P = int(offs[-1].item())
        pairs = torch.empty((max(P, 1), 2), dtype=torch.int32, device=st.device)
        _lib.call("vmc_nnbf_conn_pairs", _lib.ptr(st.occ), st.B, self.n_sites, _lib.ptr(edges), edges.shape[0],
                  _lib.ptr(offs), _lib.ptr(pairs), _lib.stream_of(st.device))
        return pairs, offs, P

    # ---- hooks implemented by subclasses ----
    def _refresh(self, st, threshold):
        raise NotImplementedError

    def sweep(self, st, graph, n_sweeps, seed, sweep_offset, hopping_rate=0.25, replay=None):
        raise NotImplementedError

    def local_energy(self, st, H):
        raise NotImplementedError

    def logpsi_grad(self, st):
        raise NotImplementedError


class SlaterDeterminant_GB300(WavefunctionModel_GB300):
    """psi(x) = det(M[ascending occupied rows]), M of shape (2N, N_f), FP64
    (vmc_torch/GPU/models/slater.py:15-61; ascending rows as in
    vmc_torch/model.py:7437-7457).

    ``init_std`` scales the N(0, 1) init of the reference (``torch.randn``);
    ``generator`` seeds it."""

    def __init__(self, n_orbitals, n_fermions, dtype=torch.float64, init_std=1.0, generator=None,
                 refresh_every=64):
        if dtype != torch.float64:
            raise ValueError("the Slater walker kernels run in FP64")
        if n_fermions > 64 or n_orbitals > 128 or n_orbitals % 2:
            raise ValueError("supports n_fermions <= 64 and n_orbitals = 2 * n_sites <= 128")
        M = torch.randn(n_orbitals, n_fermions, dtype=dtype, generator=generator) * init_std
        super().__init__([M], n_orbitals // 2)
        self.n_fermions = n_fermions
        self.n_orbitals = n_orbitals
        self.refresh_every = refresh_every

    def _new_state(self, B, device):
        st = WalkerState(B, self.n_sites, device)
        nf = self.n_fermions
        st.extra["G"] = torch.empty((B, nf, nf), dtype=torch.float64, device=device)
        st.extra["slot"] = torch.empty((B, nf), dtype=torch.uint8, device=device)
        st.extra["nsing"] = torch.zeros(1, dtype=torch.int32, device=device)
        return st

    def _M(self, device):
        M = self.params[0]
        if M.device != device:
            raise ValueError("model parameters must live on the walkers' device (call model.to(device))")
        return M.detach().contiguous()

    @torch.inference_mode()
    def take_singular_count(self):
        st = self._state
        if st is None:
            return 0
        n = int(st.extra["nsing"].item())
        st.extra["nsing"].zero_()
        return n

    def _refresh(self, st, threshold):
        M = self._M(st.device)
        _lib.call("vmc_slater_refresh", _lib.ptr(M), self.n_orbitals, self.n_fermions, _lib.ptr(st.occ), st.B,
                  self.n_sites, _lib.ptr(st.extra["G"]), _lib.ptr(st.extra["slot"]), _lib.ptr(st.sign),
                  _lib.ptr(st.logabs), _lib.ptr(st.n_acc), int(threshold), _lib.ptr(st.extra["nsing"]),
                  _lib.stream_of(st.device))

    def sweep(self, st, graph, n_sweeps, seed, sweep_offset, hopping_rate=0.25, replay=None):
        from .hamiltonian import device_sweep_edges
        M = self._M(st.device)
        edges = device_sweep_edges(graph, st.device)
        rm = rb = ra = None
        if replay is not None:
            rm, rb, ra = replay
            E = edges.shape[0]
            for a in (rm, rb, ra):
                if tuple(a.shape) != (n_sweeps, E, st.B) or not a.is_cuda or not a.is_contiguous():
                    raise ValueError("replay buffers must be contiguous CUDA tensors of shape (n_sweeps, E, B)")
        # one launch per sweep, so that the FP64 re-inversion of every walker
        # with refresh_every or more accepted moves since its last one (which
        # resets the Sherman-Morrison drift) runs between sweeps, also in a
        # long burn-in
        for k in range(int(n_sweeps)):
            part = (None, None, None) if replay is None else tuple(a[k:k + 1] for a in (rm, rb, ra))
            _lib.call("vmc_slater_sweep", _lib.ptr(M), self.n_orbitals, self.n_fermions, _lib.ptr(st.occ), st.B,
                      self.n_sites, _lib.ptr(edges), edges.shape[0], 1, float(hopping_rate),
                      int(seed) & ((1 << 64) - 1), int(sweep_offset) + k, _lib.ptr(part[0]), _lib.ptr(part[1]),
                      _lib.ptr(part[2]), _lib.ptr(st.extra["G"]), _lib.ptr(st.extra["slot"]), _lib.ptr(st.sign),
                      _lib.ptr(st.logabs), _lib.ptr(st.n_acc), _lib.stream_of(st.device))
            if self.refresh_every:
                self._refresh(st, threshold=self.refresh_every)

    def local_energy(self, st, H):
        M = self._M(st.device)
        edges = H.edges_on(st.device)
        eloc = torch.empty(st.B, dtype=torch.float64, device=st.device)
        _lib.call("vmc_slater_local_energy", _lib.ptr(M), self.n_orbitals, self.n_fermions, _lib.ptr(st.occ), st.B,
                  self.n_sites, _lib.ptr(edges), edges.shape[0], float(H.t), float(H.U), _lib.ptr(st.extra["G"]),
                  _lib.ptr(st.extra["slot"]), _lib.ptr(eloc), _lib.stream_of(st.device))
        return eloc

    def logpsi_grad(self, st, out=None):
        Np = self.n_params
        if out is None:
            out = torch.empty((st.B, Np), dtype=torch.float64, device=st.device)
        _lib.call("vmc_slater_logpsi_grad", _lib.ptr(st.extra["G"]), _lib.ptr(st.extra["slot"]), st.B,
                  self.n_orbitals, self.n_fermions, _lib.ptr(out), out.stride(0), _lib.stream_of(st.device))
        return out


_PREC = {"mixed": 0, "fp64": 1}


class NNBF_GB300(WavefunctionModel_GB300):
    """Neural-network backflow psi(x) = det((M_base + bf_scale * MLP(n))[occ])
    (vmc_torch/GPU/models/NNBF.py:36-162) with GELU hidden layers of width 256.

    Parameters (FP64 masters, reference order): M_base (2N, N_f), w_0 (H, 2N),
    b_0 (H), w_1 (H, H), b_1 (H), out_w (2N*N_f, H), out_b (2N*N_f).

    precision="mixed": BF16 tensor-core MLP with FP32 accumulation, FP32
    determinant, log|det| combined in FP64 (the production path).
    precision="fp64": every stage in FP64 (parity mode, 1e-10 against the oracle).

    init="fan_in": M_base ~ N(0, 0.1^2), weights ~ N(0, 1/fan_in), biases 0;
    init="reference": the reference's defaults (M_base ~ N(0,1), kaiming-uniform
    hidden weights, zero output layer).
    """

    def __init__(self, n_sites, n_fermions, hidden_dim=256, n_layers=2, activation="gelu", bf_scale=0.01,
                 dtype=torch.float64, precision="mixed", init="fan_in", generator=None):
        if hidden_dim != 256 or n_layers != 2 or activation != "gelu":
            raise ValueError("the GB300 NNBF kernels implement 2 GELU hidden layers of width 256")
        if precision not in _PREC:
            raise ValueError("precision must be 'mixed' or 'fp64'")
        n_orb = 2 * n_sites
        g = generator
        if init == "fan_in":
            ps = [torch.randn(n_orb, n_fermions, generator=g, dtype=torch.float64) * 0.1]
            fan = n_orb
            for _ in range(n_layers):
                ps.append(torch.randn(hidden_dim, fan, generator=g, dtype=torch.float64) / fan ** 0.5)
                ps.append(torch.zeros(hidden_dim, dtype=torch.float64))
                fan = hidden_dim
            ps.append(torch.randn(n_orb * n_fermions, fan, generator=g, dtype=torch.float64) / fan ** 0.5)
            ps.append(torch.zeros(n_orb * n_fermions, dtype=torch.float64))
        elif init == "reference":
            ps = [torch.randn(n_orb, n_fermions, generator=g, dtype=torch.float64)]
            fan = n_orb
            for _ in range(n_layers):
                w = torch.empty(hidden_dim, fan, dtype=torch.float64)
                torch.nn.init.kaiming_uniform_(w, a=0, mode="fan_in", nonlinearity="tanh", generator=g)
                ps += [w, torch.zeros(hidden_dim, dtype=torch.float64)]
                fan = hidden_dim
            ps += [torch.zeros(n_orb * n_fermions, fan, dtype=torch.float64),
                   torch.zeros(n_orb * n_fermions, dtype=torch.float64)]
        else:
            raise ValueError("init must be 'fan_in' or 'reference'")
        super().__init__(ps, n_sites)
        self.n_fermions = n_fermions
        self.n_orbitals = n_orb
        self.hidden_dim = hidden_dim
        self.n_layers = n_layers
        self.bf_scale = float(bf_scale)
        self.precision = precision
        self._net_cache = None
        self.refresh_each_sweep = True
        # sweeps evaluate only the walkers whose proposal changes them
        self.compact_rows = True

    # ---- device copies of the parameters in kernel layout ----
    def net(self, device):
        key = (self.param_key(), str(device), self.precision)
        if self._net_cache is not None and self._net_cache[0] == key:
            return self._net_cache[1]
        p = [q.detach() for q in self.params]
        if any(q.device != device for q in p):
            raise ValueError("model parameters must live on the walkers' device (call model.to(device))")
        M_base, w0, b0, w1, b1, out_w, out_b = p
        if self.precision == "mixed":
            f32, bf = torch.float32, torch.bfloat16
            ts = [w0.t().contiguous().to(f32), b0.to(f32).contiguous(), w1.to(bf).contiguous(),
                  b1.to(f32).contiguous(), out_w.to(bf).contiguous(), out_b.to(f32).contiguous(),
                  M_base.to(f32).contiguous()]
        else:
            ts = [w0.t().contiguous(), b0.contiguous(), w1.contiguous(), b1.contiguous(), out_w.contiguous(),
                  out_b.contiguous(), M_base.contiguous()]
        arr = (ctypes.c_void_p * 7)(*[t.data_ptr() for t in ts])
        self._net_cache = (key, (ts, arr))
        return ts, arr

    @property
    def _prec(self):
        return _PREC[self.precision]

    def _hdtype(self):
        return torch.bfloat16 if self.precision == "mixed" else torch.float64

    def _rdtype(self):
        return torch.float32 if self.precision == "mixed" else torch.float64

    def _new_state(self, B, device):
        st = WalkerState(B, self.n_sites, device)
        nf, H = self.n_fermions, self.hidden_dim
        x = st.extra
        x["z0"] = torch.empty((B, H), dtype=self._rdtype(), device=device)
        x["prop_occ"] = torch.zeros((B, 2), dtype=torch.int64, device=device)
        x["rec"] = torch.zeros((B, 4), dtype=torch.int32, device=device)
        x["H1"] = torch.empty((B, H), dtype=self._hdtype(), device=device)
        x["H2"] = torch.empty((B, H), dtype=self._hdtype(), device=device)
        x["A"] = torch.empty((B, nf, nf), dtype=self._rdtype(), device=device)
        x["err"] = torch.zeros(1, dtype=torch.int32, device=device)
        return st

    def _refresh(self, st, threshold):
        ts, arr = self.net(st.device)
        x = st.extra
        _lib.call("vmc_nnbf_eval", self._prec, arr, self.n_sites, self.n_fermions, self.hidden_dim, self.bf_scale,
                  _lib.ptr(st.occ), st.B, _lib.ptr(x["z0"]), _lib.ptr(x["H1"]), _lib.ptr(x["H2"]), _lib.ptr(x["A"]),
                  _lib.ptr(st.sign), _lib.ptr(st.logabs), _lib.ptr(x["err"]), _lib.stream_of(st.device))
        st.n_acc.zero_()

    def sweep(self, st, graph, n_sweeps, seed, sweep_offset, hopping_rate=0.25, replay=None, instrument=None):
        """instrument: optional dict; receives 'n_eval' (device counter) and
        accumulates 'stage_ms'/'stage_launches' (host arrays of 4) per stage."""
        from .hamiltonian import device_sweep_edges
        ts, arr = self.net(st.device)
        edges = device_sweep_edges(graph, st.device)
        rm = rb = ra = None
        if replay is not None:
            rm, rb, ra = replay
            E = edges.shape[0]
            for a in (rm, rb, ra):
                if tuple(a.shape) != (n_sweeps, E, st.B) or not a.is_cuda or not a.is_contiguous():
                    raise ValueError("replay buffers must be contiguous CUDA tensors of shape (n_sweeps, E, B)")
        if self.refresh_each_sweep:
            self._refresh(st, 0)  # recompute z0 = W0 n + b0 and psi from scratch (resets FP32 drift)
        x = st.extra
        _lib.call("vmc_nnbf_sweep", self._prec, arr, self.n_sites, self.n_fermions, self.hidden_dim, self.bf_scale,
                  _lib.ptr(st.occ), st.B, _lib.ptr(edges), edges.shape[0], int(n_sweeps), float(hopping_rate),
                  int(seed) & ((1 << 64) - 1), int(sweep_offset), _lib.ptr(rm), _lib.ptr(rb), _lib.ptr(ra),
                  _lib.ptr(x["z0"]), _lib.ptr(st.sign), _lib.ptr(st.logabs), _lib.ptr(st.n_acc),
                  _lib.ptr(x["prop_occ"]), _lib.ptr(x["rec"]), _lib.ptr(x["H1"]), _lib.ptr(x["H2"]),
                  _lib.ptr(x["A"]), _lib.ptr(x["err"]), *self._instr_args(instrument, st.device),
                  _lib.ptr(self._compact_ws(st)), _lib.stream_of(st.device))

    def _compact_ws(self, st):
        """Row-compaction workspace of the mixed 64-orbital sweep (None: off)."""
        if self.precision != "mixed" or self.n_fermions != 64 or not self.compact_rows:
            return None
        ws = st.extra.get("compact")
        if ws is None:
            n = 256 + ((4 * st.B + 15) // 16) * 16 + 16 * st.B
            ws = torch.empty(n, dtype=torch.uint8, device=st.device)
            st.extra["compact"] = ws
        return ws

    @staticmethod
    def _instr_args(instrument, device):
        if instrument is None:
            return (None, None, None)
        if "n_eval" not in instrument:
            instrument["n_eval"] = torch.zeros(1, dtype=torch.int64, device=device)
            instrument["stage_ms"] = (ctypes.c_float * 4)()
            instrument["stage_launches"] = (ctypes.c_int * 4)()
        return (_lib.ptr(instrument["n_eval"]), instrument["stage_ms"], instrument["stage_launches"])

    # ---- per-sample log-derivatives (hand-written adjoint) ----
    def grad_net(self, device):
        """Parameters in the adjoint kernel's layout and precision (FP32 for the
        mixed model, FP64 for the fp64 model)."""
        key = (self.param_key(), str(device), self.precision, "grad")
        cache = getattr(self, "_grad_cache", None)
        if cache is not None and cache[0] == key:
            return cache[1]
        dt = torch.float32 if self.precision == "mixed" else torch.float64
        M_base, w0, b0, w1, b1, out_w, out_b = [q.detach().to(device=device, dtype=dt) for q in self.params]
        ts = [w0.t().contiguous(), b0.contiguous(), w1.contiguous(), w1.t().contiguous(), b1.contiguous(),
              out_w.contiguous(), out_w.t().contiguous(), out_b.contiguous(), M_base.contiguous()]
        arr = (ctypes.c_void_p * 9)(*[t.data_ptr() for t in ts])
        self._grad_cache = (key, (ts, arr))
        return ts, arr

    @property
    def n_params_out_w(self):
        return self.n_orbitals * self.n_fermions * self.hidden_dim

    def logpsi_grad(self, st, out=None):
        """(B, Np) O rows in the reference parameter order (FP32 mixed / FP64)."""
        ts, arr = self.grad_net(st.device)
        dt = ts[0].dtype
        if out is None:
            out = torch.empty((st.B, self.n_params), dtype=dt, device=st.device)
        _lib.call("vmc_nnbf_logpsi_grad", self._prec, arr, self.n_sites, self.n_fermions, self.hidden_dim,
                  self.bf_scale, _lib.ptr(st.occ), st.B, _lib.ptr(out), out.stride(0), None, 0, None, None, None,
                  None, _lib.stream_of(st.device))
        return out

    def logpsi_grad_factored(self, st):
        """O in factored form: (O_dense (B, Np - Nw), kron_g (B, 2N*nf), kron_h (B, 256))
        where the out_w block of row b is kron_g[b] (x) kron_h[b]."""
        ts, arr = self.grad_net(st.device)
        dt = ts[0].dtype
        nd = self.n_params - self.n_params_out_w
        Od = torch.empty((st.B, nd), dtype=dt, device=st.device)
        kg = torch.empty((st.B, self.n_orbitals * self.n_fermions), dtype=dt, device=st.device)
        kh = torch.empty((st.B, self.hidden_dim), dtype=dt, device=st.device)
        _lib.call("vmc_nnbf_logpsi_grad", self._prec, arr, self.n_sites, self.n_fermions, self.hidden_dim,
                  self.bf_scale, _lib.ptr(st.occ), st.B, None, 0, _lib.ptr(Od), Od.stride(0), _lib.ptr(kg),
                  _lib.ptr(kh), None, None, _lib.stream_of(st.device))
        return Od, kg, kh

    def local_energy(self, st, H):
        ts, arr = self.net(st.device)
        edges = H.edges_on(st.device)
        pairs, offs, P = self.conn_pairs(st, H)
        x = st.extra
        chunk = st.B
        row_occ = torch.empty((chunk, 2), dtype=torch.int64, device=st.device)
        coeff = torch.empty(chunk, dtype=torch.float64, device=st.device)
        term = torch.empty(max(P, 1), dtype=torch.float64, device=st.device)
        eloc = torch.empty(st.B, dtype=torch.float64, device=st.device)
        _lib.call("vmc_nnbf_local_energy", self._prec, arr, self.n_sites, self.n_fermions, self.hidden_dim,
                  self.bf_scale, _lib.ptr(st.occ), st.B, _lib.ptr(edges), float(H.t), float(H.U), _lib.ptr(x["z0"]),
                  _lib.ptr(st.sign), _lib.ptr(st.logabs), _lib.ptr(pairs), _lib.ptr(offs), P, chunk,
                  _lib.ptr(row_occ), _lib.ptr(coeff), _lib.ptr(term), _lib.ptr(x["H1"]), _lib.ptr(x["H2"]),
                  _lib.ptr(x["A"]), _lib.ptr(eloc), _lib.ptr(x["err"]), _lib.stream_of(st.device))
        # kept for the learned proposal: per-hop amplitude ratios of this evaluation
        self.last_conn = {"pairs": pairs, "P": P, "term": term, "t": float(H.t), "occ": st.occ}
        return eloc

    def mh_step(self, st, prop_occ, rec, lg_x=None, lg_p=None, kstats=None, rows=None):
        """Metropolis-Hastings accept of learned proposals (prop_occ, rec from
        ``LearnedProposal.propose``); lg_x rows of moved walkers are replaced by
        lg_p rows; kstats (8 int32) counts proposals / acceptances by k.
        rows=(a, b): act on walkers a..b-1 only (prop_occ, rec, lg_x, lg_p are
        then that group's rows), with their own slice of every buffer, so that
        disjoint groups may run on different streams."""
        if self.precision != "mixed":
            raise ValueError("the learned-proposal step runs on the mixed-precision model")
        ts, arr = self.net(st.device)
        x = st.extra
        if "z0p" not in x:
            x["z0p"] = torch.empty_like(x["z0"])
        a, b = rows if rows is not None else (0, st.B)
        _lib.call("vmc_nnbf_mh_step", arr, self.n_sites, self.n_fermions, self.hidden_dim, self.bf_scale,
                  _lib.ptr(st.occ[a:b]), b - a, _lib.ptr(prop_occ), _lib.ptr(rec), _lib.ptr(x["z0"][a:b]),
                  _lib.ptr(x["z0p"][a:b]), _lib.ptr(st.sign[a:b]), _lib.ptr(st.logabs[a:b]), _lib.ptr(st.n_acc[a:b]),
                  _lib.ptr(x["H1"][a:b]), _lib.ptr(x["H2"][a:b]), _lib.ptr(x["A"][a:b]), _lib.ptr(lg_x),
                  _lib.ptr(lg_p), _lib.ptr(kstats), _lib.ptr(x["err"]), _lib.stream_of(st.device))


_PEPS_PREC = {"fp32": 0, "fp64": 1}


class FPEPS_GB300(WavefunctionModel_GB300):
    """Fermionic PEPS (fPEPS_Model_GPU, vmc_torch/GPU/models/pureTNS.py:24-160)
    on an Lx x Ly open square lattice, bond dimension D, physical dimension 4.

    Parameters: one tensor ``(Lx, Ly, 4, D, D, D, D)`` = [row][col][quimb
    state][left][up][right][down], Z2-graded (bond parity = index & 1, every
    tensor parity-even, legs leaving the lattice at index 0); the entries
    outside that structure are zero and stay zero (their log-derivatives are
    zero).  Sites are numbered ``row * Ly + col`` like the Hamiltonian's.

    The amplitude is the Grassmann contraction of the network (bond variables
    ordered left, up, down, right within a site) with the reference's
    boundary contraction (pureTNS.py:100-111): rows [0, Lx/2) absorbed from the
    top and rows [Lx/2, Lx) from the bottom into boundaries truncated to
    ``max_bond`` = chi after every row (cutoff 0), then contracted.  When no cut
    can exceed chi (``max_bond`` None or <= 0, as the reference's ``chi > 0``
    test, or large enough) the contraction is exact and runs on the row-boundary
    kernels (top/bottom boundary MPSs of bond D^(Lx/2-1), a column sweep through
    the two middle rows, cached column environments); otherwise on the
    chi-truncated kernels (vmc_peps_chi_*: each side's boundary as the full
    vector over its D^Ly legs, truncated by Gram/Jacobi across the scheduled
    cuts).  ``truncated`` tells which.

    precision="fp32": FP32 contraction with power-of-two rescaling per column
    (the production path); "fp64": FP64 (parity mode).
    Init: entries ~ N(0, init_std^2) (config 5 uses N(0, 1)), masked.
    env_reuse: sweeps and local energies keep each walker's left/right column
    environments (a workspace of env_rows walkers at a time) and contract only
    the columns a move touches; False recomputes every amplitude.
    """

    def __init__(self, Lx, Ly, D, max_bond=None, dtype=torch.float32, precision="fp32", init_std=1.0,
                 generator=None, tensors=None, env_reuse=True, env_rows=2048):
        if precision not in _PEPS_PREC:
            raise ValueError("precision must be 'fp32' or 'fp64'")
        chi = int(max_bond) if max_bond is not None else 0
        self.chi_cuts = self.chi_schedule(Lx, Ly, D, chi) if chi > 0 else []
        self.truncated = any(self.chi_cuts)
        if self.truncated:
            if Lx % 2 or D not in (2, 4) or D ** Ly > 4096 or Lx * Ly > 64:
                raise ValueError("chi-truncated fPEPS supports even Lx, D in {2, 4}, D**Ly <= 4096, Lx*Ly <= 64")
        elif Lx % 2 or not 4 <= Lx <= 8 or D not in (2, 4) or D ** (Lx // 2 - 1) > 16 or Lx * Ly > 64:
            raise ValueError("exact fPEPS supports even Lx in [4, 8], D in {2, 4}, D**(Lx/2-1) <= 16, Lx*Ly <= 64")
        if tensors is None:
            tensors = torch.randn((Lx, Ly, 4, D, D, D, D), generator=generator, dtype=torch.float64) * init_std
        tensors = torch.as_tensor(tensors, dtype=torch.float64).clone()
        if tuple(tensors.shape) != (Lx, Ly, 4, D, D, D, D):
            raise ValueError("tensors must have shape (Lx, Ly, 4, D, D, D, D)")
        tensors = tensors * self.structure_mask(Lx, Ly, D)
        super().__init__([tensors.to(dtype)], Lx * Ly)
        self.Lx, self.Ly, self.D = Lx, Ly, D
        self.max_bond = max_bond
        self.chi = chi
        self.precision = precision
        self.env_reuse = env_reuse
        self.env_rows = env_rows
        self.chi_rows = 8192
        self._cast = None

    @staticmethod
    def chi_schedule(Lx, Ly, D, chi):
        """Per absorbed row of a side, the cuts (columns to their left) that
        the chi-truncated contraction truncates; empty lists everywhere mean
        the contraction with max_bond = chi is exact."""
        if Lx % 2 or D not in (2, 4) or D ** Ly > 4096 or Lx * Ly > 64 or chi < 1:
            # outside the truncated kernels: exact only when no bond can exceed chi
            return [[]] * (Lx // 2) if chi >= D ** (Lx // 2) else [[-1]]
        cuts = (ctypes.c_uint32 * (Lx // 2))()
        _lib.call("vmc_peps_chi_schedule", Lx, Ly, D, chi, cuts, Lx // 2)
        return [[k for k in range(Ly - 1, 0, -1) if (cuts[a] >> k) & 1] for a in range(Lx // 2)]

    def _chi_work(self, st, rows=None):
        rows = int(rows or min(st.B, self.chi_rows))
        nbytes = ctypes.c_int64(0)
        _lib.call("vmc_peps_chi_work_bytes", self._prec, self.Lx, self.Ly, self.D, self.chi, rows,
                  ctypes.byref(nbytes))
        w = st.extra.get("chi_work")
        if w is None or w.numel() < nbytes.value:
            w = torch.empty(nbytes.value, dtype=torch.uint8, device=st.device)
            st.extra["chi_work"] = w
        return w, rows

    @staticmethod
    def structure_mask(Lx, Ly, D):
        """(Lx, Ly, 4, D, D, D, D) bool: parity-even entries with open legs at 0."""
        bp = torch.arange(D) % 2
        sp = torch.tensor([0, 1, 1, 0])
        tot = (sp[:, None, None, None, None] + bp[None, :, None, None, None] + bp[None, None, :, None, None]
               + bp[None, None, None, :, None] + bp[None, None, None, None, :])
        m = ((tot % 2) == 0).expand(Lx, Ly, 4, D, D, D, D).clone()
        m[:, 0, :, 1:, :, :, :] = False
        m[0, :, :, :, 1:, :, :] = False
        m[:, Ly - 1, :, :, :, 1:, :] = False
        m[Lx - 1, :, :, :, :, :, 1:] = False
        return m

    @property
    def _prec(self):
        return _PEPS_PREC[self.precision]

    def _tensors(self, device):
        """Contiguous kernel-dtype copy of the parameters, cached per version."""
        p = self.params[0]
        if p.device != device:
            raise ValueError("model parameters must live on the walkers' device (call model.to(device))")
        want = torch.float32 if self._prec == 0 else torch.float64
        key = (self.param_key(), str(device))
        if self._cast is None or self._cast[0] != key:
            t = p.detach()
            t = t if (t.dtype == want and t.is_contiguous()) else t.to(want).contiguous()
            self._cast = (key, t)
        return self._cast[1]

    def _shape_args(self):
        return (self.Lx, self.Ly, self.D)

    def _refresh(self, st, threshold):
        T = self._tensors(st.device)
        if self.truncated:
            work, rows = self._chi_work(st)
            _lib.call("vmc_peps_chi_eval", self._prec, _lib.ptr(T), *self._shape_args(), self.chi, _lib.ptr(st.occ),
                      st.B, _lib.ptr(st.sign), _lib.ptr(st.logabs), _lib.ptr(work), rows, _lib.stream_of(st.device))
            return
        _lib.call("vmc_peps_eval", self._prec, _lib.ptr(T), *self._shape_args(), _lib.ptr(st.occ), st.B,
                  _lib.ptr(st.sign), _lib.ptr(st.logabs), _lib.stream_of(st.device))

    def sweep(self, st, graph, n_sweeps, seed, sweep_offset, hopping_rate=0.25, replay=None, n_eval=None):
        """n_eval: optional int64 CUDA tensor of 2 counters, incremented by the
        evaluated proposals and by the column steps executed."""
        from .hamiltonian import device_sweep_edges
        if n_eval is not None and (n_eval.dtype != torch.int64 or n_eval.numel() < 2 or not n_eval.is_cuda):
            raise ValueError("n_eval must be an int64 CUDA tensor with 2 elements")
        T = self._tensors(st.device)
        edges = device_sweep_edges(graph, st.device)
        rm = rb = ra = None
        if replay is not None:
            rm, rb, ra = replay
            E = edges.shape[0]
            for a in (rm, rb, ra):
                if tuple(a.shape) != (n_sweeps, E, st.B) or not a.is_cuda or not a.is_contiguous():
                    raise ValueError("replay buffers must be contiguous CUDA tensors of shape (n_sweeps, E, B)")
        if self.truncated:
            work, rows = self._chi_work(st)
            _lib.call("vmc_peps_chi_sweep", self._prec, _lib.ptr(T), *self._shape_args(), self.chi, _lib.ptr(st.occ),
                      st.B, _lib.ptr(edges), edges.shape[0], int(n_sweeps), float(hopping_rate),
                      int(seed) & ((1 << 64) - 1), int(sweep_offset), _lib.ptr(rm), _lib.ptr(rb), _lib.ptr(ra),
                      _lib.ptr(st.sign), _lib.ptr(st.logabs), _lib.ptr(st.n_acc), _lib.ptr(n_eval), _lib.ptr(work),
                      rows, _lib.stream_of(st.device))
            return
        work, rows, err = self._env_work(st)
        _lib.call("vmc_peps_sweep", self._prec, _lib.ptr(T), *self._shape_args(), _lib.ptr(st.occ), st.B,
                  _lib.ptr(edges), edges.shape[0], int(n_sweeps), float(hopping_rate), int(seed) & ((1 << 64) - 1),
                  int(sweep_offset), _lib.ptr(rm), _lib.ptr(rb), _lib.ptr(ra), _lib.ptr(st.sign), _lib.ptr(st.logabs),
                  _lib.ptr(st.n_acc), _lib.ptr(n_eval), _lib.ptr(work), rows, _lib.ptr(err),
                  _lib.stream_of(st.device))
        self._check_err(err)

    def _env_work(self, st):
        """(workspace, rows, device error word) for environment reuse, or
        (None, 0, None) when it is off."""
        if not self.env_reuse:
            return None, 0, None
        rows = int(min(st.B, self.env_rows))
        da = self.D ** (self.Lx // 2 - 1)
        n = rows * 2 * (self.Ly + 1) * da * self.D * self.D * da
        dt = torch.float32 if self._prec == 0 else torch.float64
        w = st.extra.get("env")
        if w is None or w.numel() < n or w.dtype != dt:
            w = torch.empty(n, dtype=dt, device=st.device)
            st.extra["env"] = w
            st.extra["env_err"] = torch.zeros(1, dtype=torch.int32, device=st.device)
        return w, rows, st.extra["env_err"]

    @staticmethod
    def _check_err(err):
        if err is not None and int(err.item()) != 0:
            v = int(err.item())
            err.zero_()
            raise ValueError("fPEPS environment reuse needs nearest-neighbour edges (status %d)" % v)

    def local_energy(self, st, H):
        T = self._tensors(st.device)
        edges = H.edges_on(st.device)
        pairs, offs, P = self.conn_pairs(st, H)
        term = torch.empty(max(P, 1), dtype=torch.float64, device=st.device)
        eloc = torch.empty(st.B, dtype=torch.float64, device=st.device)
        if self.truncated:
            work, rows = self._chi_work(st)
            offs_h = offs.cpu()
            _lib.call("vmc_peps_chi_local_energy", self._prec, _lib.ptr(T), *self._shape_args(), self.chi,
                      _lib.ptr(st.occ), st.B, _lib.ptr(edges), float(H.t), float(H.U), _lib.ptr(pairs), _lib.ptr(offs),
                      ctypes.c_void_p(offs_h.data_ptr()), P, _lib.ptr(term), _lib.ptr(eloc), _lib.ptr(work), rows,
                      _lib.stream_of(st.device))
            return eloc
        work, rows, err = self._env_work(st)
        _lib.call("vmc_peps_local_energy", self._prec, _lib.ptr(T), *self._shape_args(), _lib.ptr(st.occ), st.B,
                  _lib.ptr(edges), float(H.t), float(H.U), _lib.ptr(st.sign), _lib.ptr(st.logabs), _lib.ptr(pairs),
                  _lib.ptr(offs), P, _lib.ptr(term), _lib.ptr(eloc), _lib.ptr(work), rows, _lib.ptr(err),
                  _lib.stream_of(st.device))
        self._check_err(err)
        return eloc

    def logpsi_grad(self, st, out=None, work_rows=None):
        """O (B, n_params) = d log|psi| / d tensors (flattened parameter order),
        FP32 for precision "fp32", FP64 for "fp64"; hand-written reverse
        column sweep (vmc_peps_logpsi_grad), or for a truncated model the
        truncation's cotangent and a reverse row sweep
        (vmc_peps_chi_logpsi_grad)."""
        T = self._tensors(st.device)
        if self.truncated:
            dt = torch.float32 if self._prec == 0 else torch.float64
            if out is None:
                out = torch.empty((st.B, self.n_params), dtype=dt, device=st.device)
            rows = int(work_rows or min(st.B, 2048))
            nbytes = ctypes.c_int64(0)
            status = _lib.call_status("vmc_peps_chi_grad_work_bytes", self._prec, self.Lx, self.Ly, self.D, self.chi,
                                      rows, ctypes.byref(nbytes), allow=(_lib.VMC_ERR_UNSUPPORTED,))
            if status != _lib.VMC_OK:
                raise NotImplementedError(
                    "log-derivatives through this truncation schedule are not built (%s): they need one truncated "
                    "cut after each side's last row with parity blocks of at most 32 x 32" % self.chi_cuts)
            work = torch.empty(nbytes.value, dtype=torch.uint8, device=st.device)
            _lib.call("vmc_peps_chi_logpsi_grad", self._prec, _lib.ptr(T), *self._shape_args(), self.chi,
                      _lib.ptr(st.occ), st.B, _lib.ptr(out), out.stride(0), _lib.ptr(work), rows,
                      _lib.stream_of(st.device))
            return out
        dt = torch.float32 if self._prec == 0 else torch.float64
        if out is None:
            out = torch.empty((st.B, self.n_params), dtype=dt, device=st.device)
        da = self.D ** (self.Lx // 2 - 1)
        esz = da * self.D * self.D * da
        rows = int(work_rows or min(st.B, 8192))
        work = torch.empty(rows * (self.Ly + 1) * esz, dtype=dt, device=st.device)
        _lib.call("vmc_peps_logpsi_grad", self._prec, _lib.ptr(T), *self._shape_args(), _lib.ptr(st.occ), st.B,
                  _lib.ptr(out), out.stride(0), _lib.ptr(work), rows, _lib.stream_of(st.device))
        return out
