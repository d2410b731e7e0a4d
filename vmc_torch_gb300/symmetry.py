"""Point-group symmetry projection with fermionic signs
(FermionSymmetryProjectedModel, vmc_torch/GPU/models/symmetry.py:770-1136):

    psi_r(n) = (1/|G|) sum_g sign(g, n) chi_r(g) psi(n[perm_g])

for any model of this package as the base.  The group is C4v on an L x L
lattice and C2v otherwise, with the reference's element order and 1D irreps
A1, A2, B1, B2 (symmetry.py:33-146).  Images and fermionic signs
(vmc_sym_images), the projection (vmc_sym_combine) and the projected
log-derivatives O_r = sum_g w_g O_g (vmc_sym_grad_combine) run in
libvmc_gb300; the base model evaluates the |G| images of every configuration
in one batch.  Sampling and local energies use the model-agnostic
vmc_propose_edge / vmc_accept_edge / vmc_conn_rows / vmc_eloc_* steps, with
the same proposals and random stream as the other models' sweeps.
"""
import torch

from . import _lib
from .models import WavefunctionModel_GB300

C4V_CHARACTERS = {"A1": [1, 1, 1, 1, 1, 1, 1, 1], "A2": [1, 1, 1, 1, -1, -1, -1, -1],
                  "B1": [1, -1, 1, -1, 1, 1, -1, -1], "B2": [1, -1, 1, -1, -1, -1, 1, 1]}
C2V_CHARACTERS = {"A1": [1, 1, 1, 1], "A2": [1, 1, -1, -1], "B1": [1, -1, 1, -1], "B2": [1, -1, -1, 1]}
C4V_ELEMENT_NAMES = ["e", "C4", "C4^2", "C4^3", "sigma_v", "sigma_v'", "sigma_d", "sigma_d'"]
C2V_ELEMENT_NAMES = ["e", "C2", "sigma_v", "sigma_v'"]


def build_symmetry_group(Lx, Ly):
    """(perms (|G|, N) int64, characters, element names): C4v for Lx == Ly
    (rotations about the lattice centre, counter-clockwise), else C2v; site
    i = row * Ly + col, image of g = x[perms[g]]."""
    i = torch.arange(Lx * Ly, dtype=torch.long)
    r, c = i // Ly, i % Ly
    if Lx == Ly:
        L = Lx
        f = lambda a, b: a * L + b  # noqa: E731
        perms = torch.stack([f(r, c), f(L - 1 - c, r), f(L - 1 - r, L - 1 - c), f(c, L - 1 - r),
                             f(r, L - 1 - c), f(L - 1 - r, c), f(c, r), f(L - 1 - c, L - 1 - r)])
        return perms, C4V_CHARACTERS, C4V_ELEMENT_NAMES
    f = lambda a, b: a * Ly + b  # noqa: E731
    perms = torch.stack([f(r, c), f(Lx - 1 - r, Ly - 1 - c), f(r, Ly - 1 - c), f(Lx - 1 - r, c)])
    return perms, C2V_CHARACTERS, C2V_ELEMENT_NAMES


class FermionSymmetryProjectedModel_GB300(WavefunctionModel_GB300):
    """Projection of ``base_model`` onto the 1D irrep ``irrep`` of the lattice's
    point group, with fermionic signs.  The parameters are the base model's
    (shared, same order), so O columns are the base's."""

    def __init__(self, base_model, Lx, Ly, irrep="A1"):
        perms, chars, names = build_symmetry_group(Lx, Ly)
        if irrep not in chars:
            raise ValueError("irrep must be one of %s" % sorted(chars))
        if Lx * Ly != base_model.n_sites:
            raise ValueError("lattice does not match the base model's sites")
        super().__init__(list(base_model.params), base_model.n_sites)
        self.base = base_model
        self.Lx, self.Ly, self.irrep = Lx, Ly, irrep
        self.element_names = names
        inv = torch.empty_like(perms)
        for g in range(perms.shape[0]):
            inv[g, perms[g]] = torch.arange(perms.shape[1])
        self.register_buffer("perms", perms.to(torch.int32).contiguous())
        self.register_buffer("inv_perms", inv.to(torch.int32).contiguous())
        self.register_buffer("characters", torch.tensor(chars[irrep], dtype=torch.float64))
        self.n_group = perms.shape[0]

    # the base model owns the parameters and their caches
    def invalidate(self):
        super().invalidate()
        self.base.invalidate()

    def param_key(self):
        return (self._bump,) + self.base.param_key()

    def _images(self, occ):
        """(occ_img (R*G, 2), fsign (R*G)) for packed configurations occ (R, 2)."""
        R, G = occ.shape[0], self.n_group
        img = torch.empty((R * G, 2), dtype=torch.int64, device=occ.device)
        fs = torch.empty(R * G, dtype=torch.float64, device=occ.device)
        _lib.call("vmc_sym_images", _lib.ptr(occ), R, self.n_sites, _lib.ptr(self.perms), _lib.ptr(self.inv_perms), G,
                  _lib.ptr(img), _lib.ptr(fs), _lib.stream_of(occ.device))
        return img, fs

    def _base_state(self, occ_img):
        """A base-model state holding the image configurations, evaluated."""
        bst = self.base._new_state(occ_img.shape[0], occ_img.device)
        bst.occ.copy_(occ_img)
        self.base._refresh(bst, threshold=0)
        return bst

    def _project(self, occ, want_weights=False):
        """(sign, logabs, weights or None, base state) of packed configurations."""
        R, G = occ.shape[0], self.n_group
        img, fs = self._images(occ)
        bst = self._base_state(img)
        sign = torch.empty(R, dtype=torch.float64, device=occ.device)
        logabs = torch.empty(R, dtype=torch.float64, device=occ.device)
        w = torch.empty(R * G, dtype=torch.float64, device=occ.device) if want_weights else None
        _lib.call("vmc_sym_combine", _lib.ptr(bst.sign), _lib.ptr(bst.logabs), _lib.ptr(fs), _lib.ptr(self.characters),
                  R, G, _lib.ptr(sign), _lib.ptr(logabs), _lib.ptr(w), _lib.stream_of(occ.device))
        return sign, logabs, w, bst

    # ---- model hooks ----
    def _refresh(self, st, threshold):
        s, la, _, _ = self._project(st.occ)
        st.sign.copy_(s)
        st.logabs.copy_(la)

    def sweep(self, st, graph, n_sweeps, seed, sweep_offset, hopping_rate=0.25, replay=None):
        from .hamiltonian import device_sweep_edges
        edges = device_sweep_edges(graph, st.device)
        E = edges.shape[0]
        rm = rb = ra = None
        if replay is not None:
            rm, rb, ra = replay
            for a in (rm, rb, ra):
                if tuple(a.shape) != (n_sweeps, E, st.B) or not a.is_cuda or not a.is_contiguous():
                    raise ValueError("replay buffers must be contiguous CUDA tensors of shape (n_sweeps, E, B)")
        prop = torch.empty_like(st.occ)
        u = torch.empty(st.B, dtype=torch.float32, device=st.device)
        flag = torch.empty(st.B, dtype=torch.uint8, device=st.device)
        s_ = _lib.stream_of(st.device)
        for s in range(int(n_sweeps)):
            for e in range(E):
                _lib.call("vmc_propose_edge", _lib.ptr(st.occ), st.B, self.n_sites, _lib.ptr(edges), E, e, s,
                          float(hopping_rate), int(seed) & ((1 << 64) - 1), int(sweep_offset) + s, _lib.ptr(rm),
                          _lib.ptr(rb), _lib.ptr(ra), _lib.ptr(prop), _lib.ptr(u), _lib.ptr(flag), s_)
                sp, lp, _, _ = self._project(prop)
                _lib.call("vmc_accept_edge", _lib.ptr(st.occ), st.B, _lib.ptr(prop), _lib.ptr(u), _lib.ptr(flag),
                          _lib.ptr(sp), _lib.ptr(lp), _lib.ptr(st.sign), _lib.ptr(st.logabs), _lib.ptr(st.n_acc), s_)

    def local_energy(self, st, H):
        edges = H.edges_on(st.device)
        pairs, offs, P = self.conn_pairs(st, H)
        term = torch.empty(max(P, 1), dtype=torch.float64, device=st.device)
        eloc = torch.empty(st.B, dtype=torch.float64, device=st.device)
        s_ = _lib.stream_of(st.device)
        chunk = max(st.B, 1)
        for p0 in range(0, P, chunk):
            R = min(chunk, P - p0)
            rows = torch.empty((R, 2), dtype=torch.int64, device=st.device)
            coeff = torch.empty(R, dtype=torch.float64, device=st.device)
            pr = pairs[p0:p0 + R]
            _lib.call("vmc_conn_rows", _lib.ptr(pr), R, _lib.ptr(st.occ), self.n_sites, _lib.ptr(edges), float(H.t),
                      _lib.ptr(rows), _lib.ptr(coeff), s_)
            sp, lp, _, _ = self._project(rows)
            _lib.call("vmc_eloc_terms", _lib.ptr(pr), R, _lib.ptr(coeff), _lib.ptr(sp), _lib.ptr(lp), _lib.ptr(st.sign),
                      _lib.ptr(st.logabs), _lib.ptr(term[p0:p0 + R]), s_)
        _lib.call("vmc_eloc_reduce", _lib.ptr(st.occ), st.B, _lib.ptr(offs), _lib.ptr(term), float(H.U), _lib.ptr(eloc),
                  s_)
        return eloc

    def logpsi_grad(self, st, out=None, max_bytes=2 << 30):
        """O_r (B, n_params) = sum_g w_g O_g over the base model's O of the
        images, in walker chunks whose image O fits max_bytes."""
        G, Np = self.n_group, self.n_params
        # one walker's images give the base O dtype and so the chunk size
        _, _, _, probe = self._project(st.occ[:1])
        esz = self.base.logpsi_grad(probe).element_size()
        cb = max(1, min(st.B, int(max_bytes // (G * Np * esz))))
        res = out
        for b0 in range(0, st.B, cb):
            b1 = min(st.B, b0 + cb)
            _, _, w, bst = self._project(st.occ[b0:b1], want_weights=True)
            Og = self.base.logpsi_grad(bst)
            if res is None:
                res = torch.empty((st.B, Np), dtype=Og.dtype, device=st.device)
            dt = 0 if Og.dtype == torch.float64 else 1
            _lib.call("vmc_sym_grad_combine", dt, _lib.ptr(Og), Og.stride(0), _lib.ptr(w), b1 - b0, G, Np,
                      _lib.ptr(res[b0:b1]), res.stride(0), _lib.stream_of(st.device))
        return res


__all__ = ["build_symmetry_group", "FermionSymmetryProjectedModel_GB300", "C4V_CHARACTERS", "C2V_CHARACTERS"]
