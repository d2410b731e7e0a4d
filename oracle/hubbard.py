"""Spinful Fermi-Hubbard connected set, symmray hop phases, dense H and ED
(oracle, test-only).

H = -t sum_{<ij>, s} (c+_{i s} c_{j s} + h.c.) + U sum_i n_{i up} n_{i dn}, OBC.

Follows:
  * Hamiltonian dict: hop keys (i, j, spin) for every edge and spin in
    (+1 up, -1 down), on-site keys (i,) = U
    (vmc_torch/hamiltonian_torch.py:995-1015).
  * batched connected set ``get_conn_batch_gpu``: a hop term (i, j, s) is
    valid when the netket occupations of the two spin-orbitals differ; the
    connected config swaps them; the phase is (-1)^{#occupied symmray modes
    strictly between p = 2i+s' and q = 2j+s'} (s' = 1 up, 0 down) in the
    ORIGINAL config; one diagonal entry U per doubly-occupied site
    (vmc_torch/hamiltonian_torch.py:562-655, phase rule also
    vmc_torch/fermion_utils.py:1564-1585).
  * ``to_dense`` accumulates H[eta, sigma] += coeff
    (vmc_torch/hamiltonian_torch.py:424-442).
"""
import numpy as np

from .lattice import quimb_to_netket, quimb_to_symmray, netket_to_quimb, all_states


def hop_list(edges, N, t):
    """(i_net, j_net, coeff, p_sym, q_sym) per hop term, in Hamiltonian-dict
    order (vmc_torch/hamiltonian_torch.py:562-582)."""
    out = []
    for (i, j) in edges:
        for spin in (1, -1):
            i_net = i if spin == 1 else i + N
            j_net = j if spin == 1 else j + N
            p = 2 * i + (1 if spin == 1 else 0)
            q = 2 * j + (1 if spin == 1 else 0)
            if p > q:
                p, q = q, p
            out.append((i_net, j_net, -t, p, q))
    return out


def get_conn_batch(x, edges, t, U):
    """Batched connected set, same term order as get_conn_batch_gpu
    (vmc_torch/hamiltonian_torch.py:586-655).

    Args: x (B, N) quimb int64.
    Returns: etas (T, N) int64, coeffs (T,) float64, batch_ids (T,) int64.
    """
    x = np.asarray(x, dtype=np.int64)
    B, N = x.shape
    nk = quimb_to_netket(x)
    sy = quimb_to_symmray(x)
    etas, coeffs, bids = [], [], []
    for (i_net, j_net, c, p, q) in hop_list(edges, N, t):
        valid = nk[:, i_net] != nk[:, j_net]
        idx = np.nonzero(valid)[0]
        if idx.size == 0:
            continue
        new = nk[idx].copy()
        new[:, [i_net, j_net]] = new[:, [j_net, i_net]]
        between = sy[idx, p + 1:q].sum(axis=1) % 2
        etas.append(netket_to_quimb(new))
        coeffs.append((1.0 - 2.0 * between) * c)
        bids.append(idx)
    for site in range(N):
        idx = np.nonzero(x[:, site] == 3)[0]
        if idx.size == 0:
            continue
        etas.append(x[idx])
        coeffs.append(np.full(idx.size, float(U)))
        bids.append(idx)
    if not etas:
        return (np.zeros((0, N), np.int64), np.zeros(0), np.zeros(0, np.int64))
    return np.concatenate(etas), np.concatenate(coeffs), np.concatenate(bids)


def conn_as_sets(etas, coeffs, bids, B):
    """Per-walker dict {eta tuple: summed coeff} with zeros dropped — the
    representation in which the CPU ``get_conn`` (which merges duplicate
    keys, vmc_torch/hamiltonian_torch.py:1037-1076) and the batched form
    agree."""
    out = [dict() for _ in range(B)]
    for e, c, b in zip(np.asarray(etas).tolist(), np.asarray(coeffs).tolist(),
                       np.asarray(bids).tolist()):
        k = tuple(e)
        out[b][k] = out[b].get(k, 0.0) + c
    return [{k: v for k, v in d.items() if v != 0.0} for d in out]


def local_energy(x, edges, t, U, amp_fn):
    """E_loc(x) = sum_eta H_{x,eta} psi(eta)/psi(x)
    (vmc_torch/GPU/vmc_utils.py:449-476, non-log branch).

    amp_fn: (K, N) quimb -> (K,) float64 amplitudes.
    """
    x = np.asarray(x, dtype=np.int64)
    B = x.shape[0]
    etas, coeffs, bids = get_conn_batch(x, edges, t, U)
    psi_x = amp_fn(x)
    psi_e = amp_fn(etas) if len(etas) else np.zeros(0)
    terms = coeffs * psi_e / psi_x[bids]
    eloc = np.zeros(B)
    np.add.at(eloc, bids, terms)
    return eloc


def dense_hamiltonian(N, n_up, n_dn, edges, t, U):
    """Dense H over the (n_up, n_dn) sector, reference state order
    (vmc_torch/hamiltonian_torch.py:424-442)."""
    S = all_states(N, n_up, n_dn)
    index = {tuple(s): k for k, s in enumerate(S.tolist())}
    H = np.zeros((len(S), len(S)))
    etas, coeffs, bids = get_conn_batch(S, edges, t, U)
    for e, c, b in zip(etas.tolist(), coeffs.tolist(), bids.tolist()):
        H[index[tuple(e)], b] += c
    return S, H


def exact_energy(psi, H):
    """<psi|H|psi>/<psi|psi> over the full sector (role of
    vmc_torch/variational_state.py:200-230, full_hi_expect)."""
    psi = np.asarray(psi, dtype=np.float64)
    return float(psi @ H @ psi / (psi @ psi))
