"""Lattice, Hilbert-sector and configuration encodings (oracle, test-only).

Encodings follow the reference:
  * quimb encoding per site: 0 = empty, 1 = down, 2 = up, 3 = up+down
    (vmc_torch/fermion_utils.py:1448-1498).
  * netket occupation vector ``[u_0..u_{N-1}, d_0..d_{N-1}]``
    (vmc_torch/fermion_utils.py:1473-1498; GPU inline
    vmc_torch/GPU/models/slater.py:53-56).
  * symmray interleaved order ``[d_0, u_0, d_1, u_1, ...]``
    (vmc_torch/hamiltonian_torch.py:572-576, 620-623).
  * packed bits: site ``i`` -> bit ``i`` of an up word and of a down word
    (the GB300 layout; no reference counterpart).

Edges: square lattice, zig-zag site index ``i*Ly + j``
(vmc_torch/hamiltonian_torch.py:344-372).  Sweep order is all row edges, row
by row, then all column edges, column by column
(vmc_torch/GPU/sampler.py:263-267).
"""
import numpy as np


def square_edges(Lx, Ly):
    """Nearest-neighbour OBC edges in cell order: for each site (r, c) in
    row-major order, the horizontal edge to (r, c+1) then the vertical edge to
    (r+1, c).  Mirrors ``graph.edges()`` of ``SquareLattice``
    (vmc_torch/hamiltonian_torch.py:350-352); the underlying quimb order is not
    vendored, so this cell order is the documented stand-in."""
    edges = []
    for r in range(Lx):
        for c in range(Ly):
            if c + 1 < Ly:
                edges.append((r * Ly + c, r * Ly + c + 1))
            if r + 1 < Lx:
                edges.append((r * Ly + c, (r + 1) * Ly + c))
    return edges


def sweep_edges(Lx, Ly):
    """Sweep order: ``row_edges`` (row 0, 1, ...) then ``col_edges``
    (column 0, 1, ...), as built in vmc_torch/hamiltonian_torch.py:355-367 and
    concatenated in vmc_torch/GPU/sampler.py:263-267."""
    rows, cols = {}, {}
    for (i, j) in square_edges(Lx, Ly):
        ri, ci = divmod(i, Ly)
        rj, cj = divmod(j, Ly)
        if ri == rj:
            rows.setdefault(ri, []).append((i, j))
        else:
            cols.setdefault(ci, []).append((i, j))
    out = []
    for k in rows:
        out.extend(rows[k])
    for k in cols:
        out.extend(cols[k])
    return out


def quimb_to_netket(x):
    """(…, N) quimb -> (…, 2N) netket occupations
    (vmc_torch/fermion_utils.py:1473-1498)."""
    x = np.asarray(x)
    up = ((x == 2) | (x == 3)).astype(np.int64)
    dn = ((x == 1) | (x == 3)).astype(np.int64)
    return np.concatenate([up, dn], axis=-1)


def netket_to_quimb(n):
    """(…, 2N) netket -> (…, N) quimb (vmc_torch/fermion_utils.py:1448-1471);
    the batched GPU form ``su*2 + sd`` is vmc_torch/hamiltonian_torch.py:610-613."""
    n = np.asarray(n)
    N = n.shape[-1] // 2
    return (2 * n[..., :N] + n[..., N:]).astype(np.int64)


def quimb_to_symmray(x):
    """(…, N) quimb -> (…, 2N) symmray ``[d0, u0, d1, u1, …]``
    (vmc_torch/hamiltonian_torch.py:620-623)."""
    x = np.asarray(x)
    up = ((x == 2) | (x == 3)).astype(np.int64)
    dn = ((x == 1) | (x == 3)).astype(np.int64)
    return np.stack([dn, up], axis=-1).reshape(*x.shape[:-1], 2 * x.shape[-1])


def pack(x):
    """(B, N) quimb -> (B, 2) uint64 ``[up_bits, dn_bits]``, site i -> bit i."""
    x = np.asarray(x, dtype=np.int64)
    B, N = x.shape
    assert N <= 64
    w = np.uint64(1) << np.arange(N, dtype=np.uint64)
    up = (((x == 2) | (x == 3)).astype(np.uint64) * w).sum(axis=1, dtype=np.uint64)
    dn = (((x == 1) | (x == 3)).astype(np.uint64) * w).sum(axis=1, dtype=np.uint64)
    return np.stack([up, dn], axis=1)


def unpack(occ, N):
    """(B, 2) uint64 -> (B, N) quimb int64."""
    occ = np.asarray(occ, dtype=np.uint64)
    sh = np.arange(N, dtype=np.uint64)
    up = ((occ[:, 0:1] >> sh) & np.uint64(1)).astype(np.int64)
    dn = ((occ[:, 1:2] >> sh) & np.uint64(1)).astype(np.int64)
    return 2 * up + dn


def all_states(N, n_up, n_dn):
    """All sector states in the reference's enumeration order
    (vmc_torch/hamiltonian_torch.py:157-169: itertools.product over up then
    down binary vectors).  ``generate_binary_vectors`` enumerates
    combinations in lexicographic order of positions."""
    import itertools

    def binvecs(n, k):
        out = []
        for pos in itertools.combinations(range(n), k):
            v = [0] * n
            for p in pos:
                v[p] = 1
            out.append(v)
        return out

    ups = binvecs(N, n_up)
    dns = binvecs(N, n_dn)
    nk = np.array([u + d for u in ups for d in dns], dtype=np.int64)
    return netket_to_quimb(nk)


def random_initial_configs(B, N, n_up, n_dn, seed):
    """Seeded random sector states, one per walker (role of
    vmc_torch/GPU/vmc_utils.py:22-39 and vmc_torch/GPU/vmc_setup.py:139-159:
    random placement of n_up up and n_dn down electrons)."""
    rng = np.random.default_rng(seed)
    x = np.zeros((B, N), dtype=np.int64)
    for b in range(B):
        up = rng.choice(N, size=n_up, replace=False)
        dn = rng.choice(N, size=n_dn, replace=False)
        x[b, up] += 2
        x[b, dn] += 1
    return x
