"""Square lattice, spinful-fermion Hilbert sector and the Fermi-Hubbard
Hamiltonian, mirroring the reference's interfaces
(vmc_torch/hamiltonian_torch.py: SpinfulFermion 109-222, SquareLattice
344-372, spinful_Fermi_Hubbard_square_lattice_torch 995-1076,
SpinfulFermionGPUMixin 553-655).

The connected set is enumerated on the GPU by ``vmc_hubbard_conn`` in integer
arithmetic (packed bits, masked popcount phases); ``get_conn_batch_gpu``
returns it in the reference's term-major order.
"""
import itertools
from math import comb

import numpy as np
import torch

from . import _lib
from .walkers import pack, unpack


class SquareLattice:
    """OBC square lattice with zig-zag site index i*Ly + j.  ``edges()`` is in
    cell order (each site's right then down neighbour); ``row_edges`` /
    ``col_edges`` group them by row / column, and the sampler sweeps all row
    edges then all column edges (vmc_torch/GPU/sampler.py:263-267)."""

    def __init__(self, Lx, Ly, pbc=False):
        if pbc:
            raise NotImplementedError("PBC not implemented (as in the reference)")
        self.Lx, self.Ly, self.pbc = Lx, Ly, pbc
        self.n_nodes = Lx * Ly
        self._edges = []
        for r in range(Lx):
            for c in range(Ly):
                if c + 1 < Ly:
                    self._edges.append((r * Ly + c, r * Ly + c + 1))
                if r + 1 < Lx:
                    self._edges.append((r * Ly + c, (r + 1) * Ly + c))
        self.row_edges, self.col_edges = {}, {}
        for (i, j) in self._edges:
            ri, ci = self.from_index_to_2dcoo(i)
            rj, cj = self.from_index_to_2dcoo(j)
            if ri == rj:
                self.row_edges.setdefault(ri, []).append((i, j))
            else:
                self.col_edges.setdefault(ci, []).append((i, j))
        self._dev_cache = {}

    def edges(self):
        return list(self._edges)

    @property
    def n_edges(self):
        return len(self._edges)

    def from_index_to_2dcoo(self, index):
        return index // self.Ly, index % self.Ly

    def sweep_edges(self):
        out = []
        for k in self.row_edges:
            out.extend(self.row_edges[k])
        for k in self.col_edges:
            out.extend(self.col_edges[k])
        return out

    def device_edges(self, device, kind="sweep"):
        """int32 (E, 2) device tensor of the sweep order (or the edges() order)."""
        key = (str(device), kind)
        if key not in self._dev_cache:
            e = self.sweep_edges() if kind == "sweep" else self.edges()
            self._dev_cache[key] = torch.tensor(e, dtype=torch.int32, device=device).reshape(-1, 2).contiguous()
        return self._dev_cache[key]


def sweep_edge_list(graph):
    """Edge list in the reference sampler's order for any graph object with
    row_edges / col_edges dicts."""
    if hasattr(graph, "sweep_edges"):
        return graph.sweep_edges()
    out = []
    for edges in graph.row_edges.values():
        out.extend(edges)
    for edges in graph.col_edges.values():
        out.extend(edges)
    return out


def device_sweep_edges(graph, device):
    if hasattr(graph, "device_edges"):
        return graph.device_edges(device, "sweep")
    cache = graph.__dict__.setdefault("_gb300_edges", {})
    key = str(device)
    if key not in cache:
        cache[key] = torch.tensor(sweep_edge_list(graph), dtype=torch.int32, device=device).reshape(-1, 2)
    return cache[key]


class SpinfulFermion:
    """Spin-1/2 fermion sector (vmc_torch/hamiltonian_torch.py:109-222)."""

    def __init__(self, n_orbitals, n_fermions=None, n_fermions_per_spin=None):
        self.n_orbitals = 2 * n_orbitals
        if n_fermions_per_spin is None:
            if n_fermions is None or n_fermions % 2:
                raise ValueError("give n_fermions_per_spin, or an even n_fermions split equally")
            n_fermions_per_spin = (n_fermions // 2, n_fermions // 2)
        self.n_fermions_per_spin = tuple(n_fermions_per_spin)
        self.n_fermions_spin_up, self.n_fermions_spin_down = self.n_fermions_per_spin
        self.n_fermions = sum(self.n_fermions_per_spin)

    @property
    def size(self):
        n = self.n_orbitals // 2
        return comb(n, self.n_fermions_spin_up) * comb(n, self.n_fermions_spin_down)

    def all_states(self):
        n = self.n_orbitals // 2
        ups = list(itertools.combinations(range(n), self.n_fermions_spin_up))
        dns = list(itertools.combinations(range(n), self.n_fermions_spin_down))
        out = np.zeros((len(ups) * len(dns), n), dtype=np.int64)
        k = 0
        for u in ups:
            for d in dns:
                out[k, list(u)] += 2
                out[k, list(d)] += 1
                k += 1
        return out

    def random_state(self, key=None):
        rng = np.random.default_rng(key)
        n = self.n_orbitals // 2
        x = np.zeros(n, dtype=np.int64)
        x[rng.choice(n, self.n_fermions_spin_up, replace=False)] += 2
        x[rng.choice(n, self.n_fermions_spin_down, replace=False)] += 1
        return x


class spinful_Fermi_Hubbard_square_lattice_torch:
    """H = -t sum_<ij>,s c+ c + U sum n_up n_dn on an OBC Lx x Ly lattice
    (vmc_torch/hamiltonian_torch.py:995-1076)."""

    def __init__(self, Lx, Ly, t, U, N_f, pbc=False, n_fermions_per_spin=None, no_u1_symmetry=False, gpu=True):
        if no_u1_symmetry:
            raise NotImplementedError("only the U(1) (n_up, n_dn) sector is on the GB300 path")
        self.Lx, self.Ly, self.t, self.U = Lx, Ly, float(t), float(U)
        self._graph = SquareLattice(Lx, Ly, pbc)
        self._hilbert = SpinfulFermion(Lx * Ly, N_f, n_fermions_per_spin)
        self.gpu = gpu
        # Hamiltonian-dict view kept for introspection (same keys as the reference)
        self._H = {}
        for (i, j) in self._graph.edges():
            for spin in (1, -1):
                self._H[(i, j, spin)] = -self.t
        for i in range(Lx * Ly):
            self._H[(i,)] = self.U

    @property
    def graph(self):
        return self._graph

    @property
    def hilbert(self):
        return self._hilbert

    @property
    def n_sites(self):
        return self.Lx * self.Ly

    def precompute_hops_gpu(self, device):
        """Uploads the edge list; sets ``_hop_list`` so that energy code that
        dispatches on it (vmc_torch/GPU/vmc_utils.py:360) takes the batched path."""
        self._gpu_device = torch.device(device)
        self._edges_dev = self._graph.device_edges(self._gpu_device, "graph")
        self._hop_list = [k for k in self._H if len(k) == 3]
        self._diag_list = [(k[0], v) for k, v in self._H.items() if len(k) == 1]

    def edges_on(self, device):
        return self._graph.device_edges(torch.device(device), "graph")

    def conn_slots(self, occ):
        """Raw per-walker slots: eta (B, T, 2) uint64-as-int64, coeff (B, T),
        valid (B, T) with T = 2E + N."""
        dev = occ.device
        B = occ.shape[0]
        N = self.n_sites
        E = self._graph.n_edges
        T = 2 * E + N
        eta = torch.empty((B, T, 2), dtype=torch.int64, device=dev)
        coeff = torch.empty((B, T), dtype=torch.float64, device=dev)
        valid = torch.empty((B, T), dtype=torch.uint8, device=dev)
        _lib.call("vmc_hubbard_conn", _lib.ptr(occ), B, N, _lib.ptr(self.edges_on(dev)), E, self.t, self.U,
                  _lib.ptr(eta), _lib.ptr(coeff), _lib.ptr(valid), _lib.stream_of(dev))
        return eta, coeff, valid

    def get_conn_batch_gpu(self, fxs):
        """(etas (T, N) int64, coeffs (T,) float64, batch_ids (T,) int64) in the
        reference's order: hop terms (edge, spin up / down) then on-site terms,
        each block listing its valid walkers in ascending order
        (vmc_torch/hamiltonian_torch.py:586-655)."""
        _lib.require_cuda(fxs, "fxs")
        occ = pack(fxs)
        eta, coeff, valid = self.conn_slots(occ)
        tb = valid.t().nonzero()  # (term, walker) pairs, term-major
        t_idx, b_idx = tb[:, 0], tb[:, 1]
        etas = unpack(eta[b_idx, t_idx].contiguous(), self.n_sites)
        return etas, coeff[b_idx, t_idx].contiguous(), b_idx.contiguous()

    def get_conn(self, sigma_quimb):
        """Connected configurations of one configuration with duplicate keys
        merged (vmc_torch/hamiltonian_torch.py:1037-1076)."""
        dev = getattr(self, "_gpu_device", torch.device("cuda"))
        x = torch.as_tensor(np.asarray(sigma_quimb), dtype=torch.int64, device=dev).reshape(1, -1)
        etas, coeffs, _ = self.get_conn_batch_gpu(x)
        merged = {}
        for e, c in zip(etas.cpu().numpy().tolist(), coeffs.cpu().numpy().tolist()):
            merged[tuple(e)] = merged.get(tuple(e), 0.0) + c
        keys = list(merged.keys())
        return np.array(keys, dtype=np.int64), np.array([merged[k] for k in keys])
