"""Exchange-or-hop Metropolis sweep under a replayed random stream
(oracle, test-only).

Follows ``propose_exchange_or_hopping_vec`` (vmc_torch/GPU/sampler.py:47-137)
and ``MetropolisExchangeSpinfulSamplerGPU.step`` (vmc_torch/GPU/sampler.py:
200-388):
  * on edge (i, j) a walker is "changed" iff x_i != x_j;
  * u_move < 1 - hopping_rate  -> exchange (swap the two site states);
  * otherwise hop: |dn| == 1 -> swap; |dn| == 0 -> (0,3) / (3,0) by one random
    bit (bit 1 -> (3,0)); |dn| == 2 -> (1,2) / (2,1) (bit 1 -> (2,1));
  * accept iff changed and u_acc < |psi'|^2/|psi|^2 (log mode:
    exp(2 (log|psi'| - log|psi|))).

The replay stream holds, per sweep, edge and walker, one float32 ``u_move``,
one bit ``hop_bit`` and one float32 ``u_acc`` — the three draws the reference
makes per edge (``torch.rand`` for the move type, ``torch.randint(0, 2)`` for
the hop target, ``torch.rand`` for acceptance).
"""
import numpy as np

N_MAP = np.array([0, 1, 1, 2], dtype=np.int64)


def propose(x, i, j, u_move, hop_bit, hopping_rate=0.25):
    """Vectorised proposal on edge (i, j). Returns (proposed, changed)."""
    x = np.asarray(x, dtype=np.int64)
    ci, cj = x[:, i].copy(), x[:, j].copy()
    diff = ci != cj
    is_ex = (np.asarray(u_move, np.float32) < np.float32(1.0 - hopping_rate)) & diff
    is_hop = (~is_ex) & diff
    dn = np.abs(N_MAP[ci] - N_MAP[cj])
    ni, nj = ci.copy(), cj.copy()
    sw = is_ex | (is_hop & (dn == 1))
    ni[sw], nj[sw] = cj[sw], ci[sw]
    bit = np.asarray(hop_bit).astype(bool)
    d0 = is_hop & (dn == 0)
    ni[d0] = np.where(bit[d0], 3, 0)
    nj[d0] = np.where(bit[d0], 0, 3)
    d2 = is_hop & (dn == 2)
    ni[d2] = np.where(bit[d2], 2, 1)
    nj[d2] = np.where(bit[d2], 1, 2)
    prop = x.copy()
    prop[:, i] = ni
    prop[:, j] = nj
    return prop, diff


def sweep(x, edges, logamp_fn, u_move, hop_bit, u_acc, hopping_rate=0.25):
    """Replay ``n_sweeps = u_move.shape[0]`` sweeps.

    logamp_fn: (K, N) -> (sign (K,), log|psi| (K,)).
    Returns final configs, (sign, log|psi|), and the per-walker accept count.
    """
    x = np.asarray(x, dtype=np.int64).copy()
    s, l = logamp_fn(x)
    s, l = np.asarray(s, np.float64).copy(), np.asarray(l, np.float64).copy()
    n_acc = np.zeros(x.shape[0], dtype=np.int64)
    for sw in range(u_move.shape[0]):
        for e, (i, j) in enumerate(edges):
            prop, changed = propose(x, i, j, u_move[sw, e], hop_bit[sw, e], hopping_rate)
            if not changed.any():
                continue
            idx = np.nonzero(changed)[0]
            ps, pl = logamp_fn(prop[idx])
            ratio = np.exp(2.0 * (np.asarray(pl) - l[idx]))
            acc = np.asarray(u_acc[sw, e][idx], np.float32).astype(np.float64) < ratio
            a = idx[acc]
            x[a] = prop[a]
            s[a] = np.asarray(ps)[acc]
            l[a] = np.asarray(pl)[acc]
            n_acc[a] += 1
    return x, (s, l), n_acc
