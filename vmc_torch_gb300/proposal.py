"""Learned Metropolis-Hastings proposal and the sampler that uses it.

A small MLP over the occupation bits (2N -> 512 -> 512, GELU) emits one logit
per nearest-neighbour single-electron hop and four logits for the number k of
simultaneous hops (1..4).  A proposal draws k, then k mutually non-conflicting
valid hops without replacement; q(x -> x') sums over the k! draw orders, and the
reverse probability q(x' -> x) is evaluated with the network at x', so the
acceptance min(1, |psi'/psi|^2 q(x'->x)/q(x->x')) keeps |psi|^2 exactly
stationary (libvmc_gb300: vmc_prop_sample / vmc_prop_reverse / vmc_nnbf_mh_step).

Training (hand-written FP32 kernels, vmc_prop_train_step) fits the hop head to
the heat-bath distribution p(h | x) ~ |psi(x_h)/psi(x)|^2 of the chains' own
samples -- the ratios the local-energy pass computes anyway -- and the k head to
the measured accepted-hops-per-proposal of each k.  The last ``buffer`` samples
are kept in a ring buffer on the device.

No reference counterpart: the reference samples with local exchange / hop moves
only (vmc_torch/GPU/sampler.py:47-137); plain Metropolis stays available as the
fallback and as the baseline this proposal is measured against (tau_int of E_loc).
"""
import math
import time

import torch

from . import _lib
from .models import floor_log
from .sampler import SamplerGB300

PH, PLOG, KMAX = 512, 256, 4


class LearnedProposal:
    def __init__(self, n_sites, edges, device="cuda", seed=0, lr=1e-3, buffer=65536, kweight=0.1):
        """edges: int32 (E, 2) device tensor in the Hamiltonian's edge order
        (hop index 2e + spin matches the local-energy pairs)."""
        self.N = n_sites
        self.edges = edges.contiguous()
        self.E = int(edges.shape[0])
        self.H = 2 * self.E
        if self.H + KMAX > PLOG:
            raise ValueError("too many hops for the logits row (2E + 4 must be <= 256)")
        self.device = torch.device(device)
        self.Kin = ((2 * n_sites + 63) // 64) * 64
        g = torch.Generator().manual_seed(seed)
        W1 = torch.randn(PH, self.Kin, generator=g) / math.sqrt(2 * n_sites)
        W1[:, 2 * n_sites:] = 0
        W2 = torch.randn(PH, PH, generator=g) / math.sqrt(PH)
        Wo = torch.randn(PLOG, PH, generator=g) * (0.1 / math.sqrt(PH))
        parts = [W1, torch.zeros(PH), W2, torch.zeros(PH), Wo, torch.zeros(PLOG)]
        self.params = torch.cat([p.reshape(-1) for p in parts]).to(self.device, torch.float32)
        self.n_params = self.params.numel()
        self.grad = torch.zeros_like(self.params)
        self.m1 = torch.zeros_like(self.params)
        self.m2 = torch.zeros_like(self.params)
        self.t = 0
        self.lr, self.kweight = lr, kweight
        self.cap = buffer
        self.buf_occ = torch.zeros((buffer, 2), dtype=torch.int64, device=self.device)
        self.buf_tgt = torch.zeros((buffer, self.H), dtype=torch.float32, device=self.device)
        self.n_buf, self.pos = 0, 0
        # device counters: proposals [0:4] and acceptances [4:8] by k
        self.kstats = torch.zeros(2 * KMAX, dtype=torch.int32, device=self.device)
        self._wcache = None
        self._ws = {}
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.step_counter = 0
        self.seed = seed

    # ---- views of the flat parameter vector ----
    def _views(self, v):
        sizes = [PH * self.Kin, PH, PH * PH, PH, PLOG * PH, PLOG]
        out, o = [], 0
        for s in sizes:
            out.append(v[o:o + s])
            o += s
        W1, b1, W2, b2, Wo, bo = out
        return W1.view(PH, self.Kin), b1, W2.view(PH, PH), b2, Wo.view(PLOG, PH), bo

    def inference_weights(self):
        if self._wcache is not None and self._wcache[0] == self.t:
            return self._wcache[1]
        W1, b1, W2, b2, Wo, bo = self._views(self.params)
        ts = [W1.to(torch.bfloat16).contiguous(), b1.contiguous(), W2.to(torch.bfloat16).contiguous(),
              b2.contiguous(), Wo.to(torch.bfloat16).contiguous(), bo.contiguous()]
        import ctypes
        arr = (ctypes.c_void_p * 6)(*[t.data_ptr() for t in ts])
        self._wcache = (self.t, (ts, arr))
        return ts, arr

    def _work(self, R):
        if self._ws.get("R", 0) < R:
            d = self.device
            self._ws = {"R": R, "X": torch.empty((R, self.Kin), dtype=torch.bfloat16, device=d),
                        "H1": torch.empty((R, PH), dtype=torch.bfloat16, device=d),
                        "H2": torch.empty((R, PH), dtype=torch.bfloat16, device=d),
                        "L": torch.empty((R, PLOG), dtype=torch.float32, device=d),
                        "L2": torch.empty((R, PLOG), dtype=torch.float32, device=d),
                        "prop": torch.empty((R, 2), dtype=torch.int64, device=d),
                        "rec": torch.zeros((R, 12), dtype=torch.int32, device=d)}
        return self._ws

    def logits(self, occ, out=None, w0=0):
        """Logits at the R configurations occ; the network's workspace rows
        [w0, w0 + R) are used (disjoint row ranges may run on different streams)."""
        R = occ.shape[0]
        w = self._work(w0 + R)
        ts, arr = self.inference_weights()
        L = w["L"][w0:w0 + R] if out is None else out
        _lib.call("vmc_prop_logits", arr, self.N, _lib.ptr(occ.contiguous()), R, _lib.ptr(w["X"][w0:w0 + R]),
                  _lib.ptr(w["H1"][w0:w0 + R]), _lib.ptr(w["H2"][w0:w0 + R]), _lib.ptr(L), _lib.ptr(self.err),
                  _lib.stream_of(occ.device))
        return L

    @property
    def k_prop(self):
        return self.kstats[:KMAX].double()

    @property
    def k_acc(self):
        return self.kstats[KMAX:].double()

    def propose(self, occ, Lx=None, w0=0):
        """Returns (prop_occ (B, 2), rec (B, 12) int32 records, logits at the
        proposals) with log q both ways.  Lx: logits at occ if already known.
        w0: first workspace row (walker groups on separate streams use
        disjoint rows; every call draws from a fresh counter of the stream)."""
        B = occ.shape[0]
        w = self._work(w0 + B)
        s = _lib.stream_of(occ.device)
        if Lx is None:
            Lx = self.logits(occ, out=w["L"][w0:w0 + B], w0=w0)
        prop, rec = w["prop"][w0:w0 + B], w["rec"][w0:w0 + B]
        _lib.call("vmc_prop_sample", _lib.ptr(self.edges), self.E, self.N, _lib.ptr(Lx), _lib.ptr(occ), B,
                  int(self.seed) & ((1 << 64) - 1), self.step_counter, _lib.ptr(prop), _lib.ptr(rec), s)
        self.step_counter += 1
        Lp = self.logits(prop, out=w["L2"][w0:w0 + B], w0=w0)
        _lib.call("vmc_prop_reverse", _lib.ptr(self.edges), self.E, self.N, _lib.ptr(Lp), _lib.ptr(prop), B,
                  _lib.ptr(rec), s)
        return prop, rec, Lp

    # ---- data and training ----
    def record(self, model):
        """Append the last local-energy evaluation's samples and heat-bath hop
        targets (|psi(x_h)/psi(x)|^2) to the ring buffer."""
        lc = getattr(model, "last_conn", None)
        if lc is None:
            return
        occ = lc["occ"]
        B = occ.shape[0]
        rows = (self.pos + torch.arange(B, device=self.device)) % self.cap
        tgt = torch.zeros((B, self.H), dtype=torch.float32, device=self.device)
        _lib.call("vmc_prop_collect_targets", _lib.ptr(lc["pairs"]), lc["P"], _lib.ptr(lc["term"]), lc["t"], self.H,
                  0, _lib.ptr(tgt), _lib.stream_of(self.device))
        self.buf_occ[rows] = occ
        self.buf_tgt[rows] = tgt
        self.pos = (self.pos + B) % self.cap
        self.n_buf = min(self.cap, self.n_buf + B)

    def k_target(self):
        """p*(k) ~ k * (acceptance rate of k-hop proposals), smoothed."""
        rate = (self.k_acc + 1.0) / (self.k_prop + 2.0)
        w = torch.arange(1, KMAX + 1, device=self.device, dtype=torch.float64) * rate
        return (w / w.sum()).float()

    def train(self, epochs=1, batch=4096, generator=None):
        n = self.n_buf
        if n == 0:
            return None
        ws_need = batch * (4 * PH + 2 * PLOG)
        if self._ws.get("train_n", 0) < ws_need:
            self._ws["train"] = torch.empty(ws_need, dtype=torch.float32, device=self.device)
            self._ws["train_n"] = ws_need
            self._ws["Xf"] = torch.empty((batch, self.Kin), dtype=torch.float32, device=self.device)
            self._ws["loss"] = torch.empty(batch, dtype=torch.float32, device=self.device)
        kt = self.k_target()
        s = _lib.stream_of(self.device)
        losses = []
        for _ in range(epochs):
            perm = torch.randperm(n, device=self.device, generator=generator)
            for b0 in range(0, n - batch + 1 if n >= batch else 1, batch):
                idx = perm[b0:b0 + batch] if n >= batch else perm
                R = idx.numel()
                occ = self.buf_occ[idx].contiguous()
                tgt = self.buf_tgt[idx].contiguous()
                Xf = self._ws["Xf"][:R]
                _lib.call("vmc_prop_inputs_f32", self.N, _lib.ptr(occ), R, _lib.ptr(Xf), s)
                self.t += 1
                _lib.call("vmc_prop_train_step", self.N, _lib.ptr(self.edges), self.E, _lib.ptr(occ), R,
                          _lib.ptr(Xf), _lib.ptr(tgt), _lib.ptr(kt), float(self.kweight), _lib.ptr(self.params),
                          _lib.ptr(self.grad), _lib.ptr(self.m1), _lib.ptr(self.m2), self.n_params, float(self.lr),
                          0.9, 0.999, 1e-8, self.t, _lib.ptr(self._ws["train"]), _lib.ptr(self._ws["loss"]), s)
                losses.append(self._ws["loss"][:R].mean())
        return float(torch.stack(losses).mean().item()) if losses else None


class LearnedSamplerGB300(SamplerGB300):
    """Metropolis-Hastings sampler with the learned proposal.  One ``step``
    performs ``moves_per_step`` learned MH moves per walker; it mutates
    ``fxs`` in place like the reference sampler.  The mixed-precision NNBF
    model evaluates and accepts the proposals in one fused call
    (vmc_nnbf_mh_step); any other model evaluates them with its own kernels
    and the walkers move by the model-agnostic vmc_accept_mh, after which the
    model's per-walker state is rebuilt for the new configurations."""

    def __init__(self, proposal, moves_per_step=112, fused=None):
        """fused: None picks the fused step where the model has one; False
        forces the model-agnostic path (evaluation + vmc_accept_mh)."""
        self.proposal = proposal
        self.moves_per_step = moves_per_step
        self.fused = fused
        self._st = []

    def _streams(self, n, device):
        while len(self._st) < n:
            self._st.append(torch.cuda.Stream(device=device))
        return self._st[:n]

    GROUP = 4096   # walkers per group when the batch is split over streams

    def _native(self, model):
        if self.fused is False:
            return False
        return getattr(model, "precision", None) == "mixed" and hasattr(model, "mh_step")

    def _generic_moves(self, st, model):
        P = self.proposal
        B = st.B
        key = (id(model), B, str(st.device))
        if getattr(self, "_tmp_key", None) != key:
            self._tmp = model._new_state(B, st.device)
            self._tmp_key = key
        tmp = self._tmp
        Lx = P.logits(st.occ).clone()
        s = _lib.stream_of(st.device)
        for _ in range(self.moves_per_step):
            prop, rec, Lp = P.propose(st.occ, Lx)
            tmp.occ.copy_(prop)
            model._refresh(tmp, 0)
            _lib.call("vmc_accept_mh", _lib.ptr(st.occ), B, _lib.ptr(prop), _lib.ptr(rec), _lib.ptr(tmp.sign),
                      _lib.ptr(tmp.logabs), _lib.ptr(st.sign), _lib.ptr(st.logabs), _lib.ptr(st.n_acc),
                      _lib.ptr(Lx), _lib.ptr(Lp), _lib.ptr(P.kstats), s)
        model._refresh(st, 0)   # the model's per-walker state for the configurations reached

    @torch.inference_mode()
    def step(self, fxs, model, graph=None, use_log_amp=False, **kwargs):
        st = model.bind_state(fxs)
        P = self.proposal
        B = st.B
        P._work(B)
        if not self._native(model):
            self._generic_moves(st, model)
            model.store_configs(st, fxs)
            if use_log_amp:
                return fxs, (st.sign.clone(), floor_log(st.logabs))
            return fxs, st.sign * torch.exp(st.logabs)
        Lx = P.logits(st.occ).clone()   # logits at the current configurations
        if B < 2 * self.GROUP:
            for _ in range(self.moves_per_step):
                prop, rec, Lp = P.propose(st.occ, Lx)
                # accepted walkers take x' and its logits (one network evaluation per move)
                model.mh_step(st, prop, rec, Lx, Lp, P.kstats)
        else:
            # Independent chains: groups of <= 4096 walkers run their moves on
            # their own streams, so one group's LU overlaps another's GEMMs.
            groups = [(a, min(B, a + self.GROUP)) for a in range(0, B, self.GROUP)]
            main = torch.cuda.current_stream(st.device)
            streams = self._streams(len(groups), st.device)
            for s in streams:
                s.wait_stream(main)
            for _ in range(self.moves_per_step):
                for (a, b), s in zip(groups, streams):
                    with torch.cuda.stream(s):
                        prop, rec, Lp = P.propose(st.occ[a:b], Lx[a:b], w0=a)
                        model.mh_step(st, prop, rec, Lx[a:b], Lp, P.kstats, rows=(a, b))
            for s in streams:
                main.wait_stream(s)
        model._watch_err(st)
        model.store_configs(st, fxs)
        if use_log_amp:
            return fxs, (st.sign.clone(), floor_log(st.logabs))
        return fxs, st.sign * torch.exp(st.logabs)


class OnlineProposalTraining:
    """Online training schedule of the learned proposal inside a VMC loop, as
    an ``on_step_end(info)`` callback of either driver (``VMC_GB300.run_vmc_loop``
    or the reference's ``VMC_GPU.run_vmc_loop``, vmc_torch/GPU/VMC.py:645-847):
    after every SR step the step's samples and their heat-bath hop targets
    (from that step's local-energy pass) join the proposal's ring buffer (its
    last ``buffer`` samples), and every ``every`` steps the proposal trains
    for ``epochs`` epochs over the buffer.  ``then`` is called afterwards with
    the same info (to chain the caller's own callback).  ``train_seconds``
    accumulates the training time for the ESS accounting, measured like the
    samplers' times: CUDA events on the current stream around each session."""

    def __init__(self, proposal, model, every=10, epochs=4, batch=16384, then=None):
        self.proposal, self.model = proposal, model
        self.every, self.epochs, self.batch = int(every), int(epochs), int(batch)
        self.then = then
        self.steps = 0
        self.sessions = 0
        self.train_seconds = 0.0
        self.last_loss = None

    def __call__(self, info):
        self.proposal.record(self.model)
        self.steps += 1
        if self.steps % self.every == 0:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            self.last_loss = self.proposal.train(epochs=self.epochs, batch=self.batch)
            e1.record()
            e1.synchronize()
            self.train_seconds += e0.elapsed_time(e1) / 1e3
            self.sessions += 1
        if self.then is not None:
            self.then(info)
