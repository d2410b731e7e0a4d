"""Stochastic reconfiguration in sample space (minSR) and the parameter update,
with the reference's preconditioner / optimizer interfaces
(vmc_torch/GPU/optimizer.py:130-251, 471-614, 884-907).

minSR: O~ = (O - <O>)/sqrt(Ns); T = O~ O~^T + lambda I (Ns x Ns, FP64
accumulation); x = T^-1 (E - <E>)/sqrt(Ns); dp = O~^T x.  T is symmetric
positive definite whenever lambda > 0 and O is finite, and is then factored by
this library's FP64 Cholesky.  When the Cholesky meets a non-positive pivot (a
negative or zero shift, a rank-deficient O) the solve follows the reference
exactly (vmc_torch/GPU/optimizer.py:557-561): torch.linalg.solve (LU with
partial pivoting) with info = 0, and when that raises on an exactly singular
T, the minimum-norm least-squares solution with info = 1 (the role of the
reference's lstsq; computed from the eigendecomposition of the symmetric T,
eigenvalues below Ns * eps * max|eigenvalue| dropped).  These fallbacks are
library calls on the failure path only; the Cholesky path never leaves this
library's kernels.

``local_o`` may be a dense (Ns, Np) tensor (the reference's layout) or a
:class:`FactoredO`, in which the NNBF output-layer block of every row is the
outer product g_a (x) h_a.  For the factored form the Gram matrix of that block
is assembled without materialising it:

    (O_k - 1 mu^T)(O_k - 1 mu^T)^T = (G G^T) o (H H^T) - v 1^T - 1 v^T + |mu|^2
    mu = G^T H / Ns,  v_a = g_a^T mu h_a,
    dp_k = (G^T diag(x) H - (sum x) mu) / sqrt(Ns),

which reduces the 8x8 NNBF Gram from 2 Ns^2 * 2.2e6 to 2 Ns^2 * (1.15e5 + 8192
+ 256) flops and never stores the 145 GB out_w block of O.
"""
import time

import torch

from . import _lib


def _dtype_code(t):
    if t.dtype == torch.float64:
        return 0
    if t.dtype == torch.float32:
        return 1
    raise ValueError("O must be float64 or float32")


class FactoredO:
    """Per-sample log-derivatives with one Kronecker-factored block.

    dense: (Ns, Nd) rows of O without the factored block; g: (Ns, Ng);
    h: (Ns, Nh); the factored block occupies full-parameter indices
    [offset, offset + Ng*Nh) with row b equal to (g[b][:, None] * h[b][None, :]).ravel().
    """

    def __init__(self, dense, g, h, offset):
        self.dense, self.g, self.h, self.offset = dense, g, h, int(offset)

    @property
    def shape(self):
        return (self.dense.shape[0], self.n_params)

    @property
    def n_params(self):
        return self.dense.shape[1] + self.g.shape[1] * self.h.shape[1]

    @property
    def device(self):
        return self.dense.device

    def __getitem__(self, idx):
        return FactoredO(self.dense[idx], self.g[idx], self.h[idx], self.offset)

    @staticmethod
    def cat(parts):
        return FactoredO(torch.cat([p.dense for p in parts]), torch.cat([p.g for p in parts]),
                         torch.cat([p.h for p in parts]), parts[0].offset)

    def row_norms(self):
        d = (self.dense.double() ** 2).sum(1)
        k = (self.g.double() ** 2).sum(1) * (self.h.double() ** 2).sum(1)
        return (d + k).sqrt()

    def zero_rows(self, mask):
        self.dense[mask] = 0
        self.g[mask] = 0
        self.h[mask] = 0

    def full(self):
        """Materialise the dense (Ns, Np) matrix (small cases / tests)."""
        k = (self.g[:, :, None] * self.h[:, None, :]).reshape(self.g.shape[0], -1)
        return torch.cat([self.dense[:, :self.offset], k, self.dense[:, self.offset:]], dim=1)

    def assemble(self, dp_dense, dp_kron):
        return torch.cat([dp_dense[:self.offset], dp_kron.reshape(-1), dp_dense[self.offset:]])


class _Stages:
    """Optional per-stage device times of one solve: CUDA events recorded on
    the current stream; ``mark(name)`` closes the stage called ``name``."""

    def __init__(self, enabled):
        self.ev = [("start", self._event())] if enabled else None

    @staticmethod
    def _event():
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        return e

    def mark(self, name):
        if self.ev is not None:
            self.ev.append((name, self._event()))

    def result(self):
        if self.ev is None:
            return None
        self.ev[-1][1].synchronize()
        out = {}
        for (_, a), (name, b) in zip(self.ev[:-1], self.ev[1:]):
            out[name] = out.get(name, 0.0) + a.elapsed_time(b)
        return out


class PreconditionerGB300:
    def solve(self, *, local_o, local_energies, energy_mean, total_samples, n_params, diag_shift, device, run_sr):
        raise NotImplementedError


class MinSRGB300(PreconditionerGB300):
    """Drop-in for MinSRGPU.solve (vmc_torch/GPU/optimizer.py:884-907).

    record_stages=True keeps the device time of each stage of the last solve
    (centring, Gram blocks, Cholesky, triangular solves, update) in
    ``last_stages`` (milliseconds, CUDA events on the current stream)."""

    def __init__(self, record_stages=False, gram="tensor"):
        """gram: "tensor" (default) forms the Gram blocks of FP32 O on the
        tensor cores (vmc_sr_gram_tc: each row split
        into three 7-bit fixed-point digits under a shared power-of-two
        exponent, all nine digit products, the leading one summed exactly in
        FP32, drained into FP64 every 2048 columns): the Gram matrix of the
        rows rounded to 2^-20 of their largest entry, positive semidefinite
        up to ~2^-32 rounding.  "cuda" forms them on the CUDA cores with
        compensated (double-float) accumulation: the exact Gram of the FP32
        rows, ~10x slower.  FP64 O always uses FP64 arithmetic."""
        if gram not in ("tensor", "cuda"):
            raise ValueError("gram must be 'tensor' or 'cuda'")
        self.record_stages = record_stages
        self.last_stages = None
        self.gram = gram

    def _tc_gram(self, X, T, alpha, D, shift, accumulate, dev):
        """T [+]= alpha (X X^T) o D [+ shift I] on the tensor cores, X FP32 (Ns, K)."""
        s = _lib.stream_of(dev)
        Ns, K = X.shape
        rp, kp = -(-Ns // 128) * 128, -(-K // 64) * 64
        planes = torch.empty(3 * rp * kp, dtype=torch.bfloat16, device=dev)
        rexp = torch.empty(rp, dtype=torch.int32, device=dev)
        _lib.call("vmc_split_bf16x3", _lib.ptr(X), Ns, K, X.stride(0), _lib.ptr(planes), rp, kp, _lib.ptr(rexp), s)
        err = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("vmc_sr_gram_tc", _lib.ptr(planes), _lib.ptr(rexp), Ns, rp, kp, float(alpha), _lib.ptr(T),
                  T.stride(0), _lib.ptr(D), float(shift), int(accumulate), _lib.ptr(err), s)
        self._tc_err = err
        del planes

    def _check_tc(self):
        err = getattr(self, "_tc_err", None)
        if err is not None and int(err.item()) != 0:
            raise ValueError("vmc_sr_gram_tc: %s" % _lib.message(int(err.item())))

    def solve(self, *, local_o, local_energies, energy_mean, total_samples, n_params, diag_shift, device=None,
              run_sr=True):
        t0 = time.time()
        self._st = _Stages(self.record_stages and run_sr)
        try:
            return self._solve(local_o, local_energies, energy_mean, n_params, diag_shift, device, run_sr, t0)
        finally:
            self.last_stages = self._st.result()

    def _solve(self, local_o, local_energies, energy_mean, n_params, diag_shift, device, run_sr, t0):
        dev = torch.device(device) if device is not None else torch.device("cuda")
        E = torch.as_tensor(local_energies, device=dev, dtype=torch.float64).contiguous()
        if isinstance(local_o, FactoredO):
            return self._solve_factored(local_o, E, float(energy_mean), n_params, float(diag_shift), dev, run_sr, t0)
        O = torch.as_tensor(local_o, device=dev)
        if O.dtype not in (torch.float64, torch.float32):
            O = O.to(torch.float64)
        O = O.contiguous()
        Ns, Np = O.shape
        if Np != n_params:
            raise ValueError("local_o has %d columns, n_params is %d" % (Np, n_params))
        s = _lib.stream_of(dev)
        code = _dtype_code(O)
        if not run_sr:
            g = torch.empty(Np, dtype=torch.float64, device=dev)
            _lib.call("vmc_energy_gradient", _lib.ptr(O), code, Ns, Np, O.stride(0), _lib.ptr(E), float(energy_mean),
                      _lib.ptr(g), s)
            return g, time.time() - t0, None
        Oc = torch.empty_like(O)
        _lib.call("vmc_sr_center", _lib.ptr(O), code, Ns, Np, O.stride(0), _lib.ptr(Oc), Oc.stride(0), None, s)
        self._st.mark("center")

        def gram(T, shift):
            if code == 1 and self.gram == "tensor":
                self._tc_gram(Oc, T, 1.0, None, shift, 0, dev)
            else:
                _lib.call("vmc_sr_gram", _lib.ptr(Oc), code, Ns, Np, Oc.stride(0), _lib.ptr(T), Ns, shift, 0, s)
            self._st.mark("gram")

        gram.check = self._check_tc
        x, info = self._factor_solve(gram, E, float(energy_mean), Ns, float(diag_shift), dev, self._st)
        dp = torch.empty(Np, dtype=torch.float64, device=dev)
        _lib.call("vmc_sr_update", _lib.ptr(Oc), code, Ns, Np, Oc.stride(0), _lib.ptr(x), _lib.ptr(dp), s)
        self._st.mark("update")
        return dp, time.time() - t0, info

    # -- shared: Gram -> FP64 Cholesky -> solve (reference fallbacks on failure) --
    @staticmethod
    def _factor_solve(build_gram, E, Ebar, Ns, shift, dev, stages):
        s = _lib.stream_of(dev)
        T = torch.empty((Ns, Ns), dtype=torch.float64, device=dev)
        build_gram(T, shift)
        flag = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("vmc_sr_cholesky", _lib.ptr(T), Ns, Ns, _lib.ptr(flag), s)
        stages.mark("cholesky")
        check = getattr(build_gram, "check", None)
        if check is not None:
            check()
        x = torch.empty(Ns, dtype=torch.float64, device=dev)
        _lib.call("vmc_sr_rhs", _lib.ptr(E), Ns, Ebar, _lib.ptr(x), s)
        if int(flag.item()) == 0:
            _lib.call("vmc_sr_cholesky_solve", _lib.ptr(T), Ns, Ns, _lib.ptr(x), s)
            stages.mark("solve")
            return x, 0
        # the factorisation overwrote T: rebuild it, then solve as the reference does
        build_gram(T, shift)
        T = torch.tril(T) + torch.tril(T, -1).t()   # symmetric from the lower triangle the kernels define
        try:
            return torch.linalg.solve(T, x), 0
        except RuntimeError:
            return _min_norm_solve(T, x), 1

    def _solve_factored(self, F, E, Ebar, n_params, shift, dev, run_sr, t0):
        s = _lib.stream_of(dev)
        Od, G, H = F.dense.contiguous(), F.g.contiguous(), F.h.contiguous()
        if not (Od.dtype == G.dtype == H.dtype):
            raise ValueError("factored O blocks must share one dtype")
        code = _dtype_code(Od)
        Ns, Nd = Od.shape
        Ng, Nh = G.shape[1], H.shape[1]
        if Nd + Ng * Nh != n_params:
            raise ValueError("factored O has %d parameters, n_params is %d" % (Nd + Ng * Nh, n_params))
        # mu = G^T H / Ns  (Ng x Nh, FP64)
        mu = torch.empty((Ng, Nh), dtype=torch.float64, device=dev)
        _lib.call("vmc_gemm", 1, 0, Ng, Nh, Ns, 1.0 / Ns, _lib.ptr(G), G.stride(0), _lib.ptr(H), H.stride(0), None,
                  code, 0.0, _lib.ptr(mu), Nh, None, 0, 0, s)
        self._st.mark("gram_head")
        if not run_sr:
            g = torch.empty(Nd, dtype=torch.float64, device=dev)
            _lib.call("vmc_energy_gradient", _lib.ptr(Od), code, Ns, Nd, Od.stride(0), _lib.ptr(E), Ebar, _lib.ptr(g), s)
            # <E O_k> - <E><O_k> = G^T diag(E - Ebar) H / Ns
            w = (E - Ebar).to(G.dtype).contiguous()
            gk = torch.empty((Ng, Nh), dtype=torch.float64, device=dev)
            _lib.call("vmc_gemm", 1, 0, Ng, Nh, Ns, 1.0 / Ns, _lib.ptr(G), G.stride(0), _lib.ptr(H), H.stride(0),
                      _lib.ptr(w), code, 0.0, _lib.ptr(gk), Nh, None, 0, 0, s)
            return F.assemble(g, gk), time.time() - t0, None
        Oc = torch.empty_like(Od)
        _lib.call("vmc_sr_center", _lib.ptr(Od), code, Ns, Nd, Od.stride(0), _lib.ptr(Oc), Oc.stride(0), None, s)
        self._st.mark("center")
        HH = torch.empty((Ns, Ns), dtype=torch.float64, device=dev)
        _lib.call("vmc_gemm", 0, 1, Ns, Ns, Nh, 1.0, _lib.ptr(H), H.stride(0), _lib.ptr(H), H.stride(0), None, code,
                  0.0, _lib.ptr(HH), Ns, None, 0, 1, s)
        mu_c = mu.to(G.dtype).contiguous()
        P = torch.empty((Ns, Nh), dtype=torch.float64, device=dev)
        _lib.call("vmc_gemm", 0, 0, Ns, Nh, Ng, 1.0, _lib.ptr(G), G.stride(0), _lib.ptr(mu_c), Nh, None, code, 0.0,
                  _lib.ptr(P), Nh, None, 0, 0, s)
        mu_sq = float((mu * mu).sum().item())
        vwork = torch.empty(Ns, dtype=torch.float64, device=dev)
        self._st.mark("gram_head")

        def gram(T, sh):
            tc = code == 1 and self.gram == "tensor"
            if tc:
                self._tc_gram(Oc, T, 1.0, None, sh, 0, dev)
            else:
                _lib.call("vmc_sr_gram", _lib.ptr(Oc), code, Ns, Nd, Oc.stride(0), _lib.ptr(T), Ns, sh, 0, s)
            self._st.mark("gram_dense")
            if tc:
                self._tc_gram(G, T, 1.0 / Ns, HH, 0.0, 1, dev)
            else:
                _lib.call("vmc_gemm", 0, 1, Ns, Ns, Ng, 1.0 / Ns, _lib.ptr(G), G.stride(0), _lib.ptr(G), G.stride(0),
                          None, code, 1.0, _lib.ptr(T), Ns, _lib.ptr(HH), Ns, 1, s)
            _lib.call("vmc_sr_kron_correction", Ns, _lib.ptr(T), Ns, _lib.ptr(P), Nh, _lib.ptr(H), code, H.stride(0),
                      Nh, mu_sq, 1.0 / Ns, _lib.ptr(vwork), s)
            self._st.mark("gram_head")

        gram.check = self._check_tc
        x, info = self._factor_solve(gram, E, Ebar, Ns, shift, dev, self._st)
        dp_d = torch.empty(Nd, dtype=torch.float64, device=dev)
        _lib.call("vmc_sr_update", _lib.ptr(Oc), code, Ns, Nd, Oc.stride(0), _lib.ptr(x), _lib.ptr(dp_d), s)
        rs = Ns ** 0.5
        dp_k = (-float(x.sum().item()) / rs) * mu
        xc = x.to(G.dtype).contiguous()
        _lib.call("vmc_gemm", 1, 0, Ng, Nh, Ns, 1.0 / rs, _lib.ptr(G), G.stride(0), _lib.ptr(H), H.stride(0),
                  _lib.ptr(xc), code, 1.0, _lib.ptr(dp_k), Nh, None, 0, 0, s)
        self._st.mark("update")
        return F.assemble(dp_d, dp_k), time.time() - t0, info


def _min_norm_solve(T, b):
    """Minimum-norm least-squares solution of the symmetric system T x = b:
    x = V diag(1/w) V^T b over the eigenpairs with |w| > Ns eps max|w| (the
    cutoff numpy's lstsq uses for its singular values, which are |w| here)."""
    w, V = torch.linalg.eigh(T)
    cut = T.shape[0] * torch.finfo(T.dtype).eps * w.abs().max()
    inv = torch.where(w.abs() > cut, 1.0 / w, torch.zeros_like(w))
    return V @ (inv * (V.t() @ b))


class OptimizerGB300:
    """theta <- compute_update(theta, direction), copied in place per parameter
    (vmc_torch/GPU/optimizer.py:130-176)."""

    def __init__(self, learning_rate=1e-3):
        self.lr = learning_rate

    def compute_update(self, params_vec, direction_vec, learning_rate=None):
        raise NotImplementedError

    @torch.no_grad()
    def step(self, model, direction, device=None, learning_rate=None):
        current = torch.nn.utils.parameters_to_vector(model.parameters())
        d = torch.as_tensor(direction, device=current.device if device is None else device, dtype=current.dtype)
        updated = self.compute_update(current, d, learning_rate)
        off = 0
        for p in model.parameters():
            n = p.numel()
            p.data.copy_(updated[off:off + n].view_as(p.data))
            off += n
        if hasattr(model, "invalidate"):
            model.invalidate()

    def reset(self):
        pass


class SGDGB300(OptimizerGB300):
    """theta - lr * dp (vmc_torch/GPU/optimizer.py:178-186)."""

    def compute_update(self, params_vec, direction_vec, learning_rate=None):
        lr = self.lr if learning_rate is None else learning_rate
        return params_vec - lr * direction_vec
