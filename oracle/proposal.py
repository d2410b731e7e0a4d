"""Learned Metropolis-Hastings proposal: CPU restatement (oracle, test-only).

No reference counterpart exists (the reference proposes local exchange / hop
moves only, vmc_torch/GPU/sampler.py:47-137).  This module restates the
proposal the GB300 kernels implement, by brute force: the probability of an
unordered hop set is summed over all k! draw orders explicitly
(itertools.permutations) rather than by the kernels' subset DP, and the MLP,
its loss and gradients use float64 numpy / torch autograd.

Hop h = 2e + s (s = 0 up, 1 down) on edge e = (i, j) of the edge list is valid
when exactly one of i, j holds spin s; hops conflict when they share a site and
a spin.
"""
import itertools
import math

import numpy as np
import torch

from .lattice import quimb_to_netket

PH, PLOG, KMAX = 512, 256, 4


def valid_hops(x, edges):
    x = np.asarray(x)
    up = (x == 2) | (x == 3)
    dn = (x == 1) | (x == 3)
    out = np.zeros((x.shape[0], 2 * len(edges)), dtype=bool)
    for e, (i, j) in enumerate(edges):
        out[:, 2 * e] = up[:, i] != up[:, j]
        out[:, 2 * e + 1] = dn[:, i] != dn[:, j]
    return out


def conflict(h1, h2, edges):
    if (h1 & 1) != (h2 & 1):
        return False
    return len(set(edges[h1 >> 1]) & set(edges[h2 >> 1])) > 0


def apply_hops(x, hops, edges):
    x = np.array(x, copy=True)
    for h in hops:
        i, j = edges[h >> 1]
        bit = 2 if (h & 1) == 0 else 1
        a, b = (x[i] & bit) != 0, (x[j] & bit) != 0
        assert a != b
        x[i] ^= bit
        x[j] ^= bit
    return x


def log_q(logits, x_row, hops, edges):
    """log p(k) + log sum over orders of prod_t softmax_allowed(l)[hop_t]."""
    H = 2 * len(edges)
    lg = np.asarray(logits, np.float64)
    valid = valid_hops(x_row[None], edges)[0]
    k = len(hops)
    tot = 0.0
    for order in itertools.permutations(hops):
        p = 1.0
        chosen = []
        for h in order:
            allowed = [g for g in range(H) if valid[g] and g not in chosen
                       and not any(conflict(g, c, edges) for c in chosen)]
            if h not in allowed:
                p = 0.0
                break
            w = np.exp(lg[allowed] - lg[allowed].max())
            p *= float(np.exp(lg[h] - lg[allowed].max()) / w.sum())
            chosen.append(h)
        tot += p
    kl = lg[H:H + KMAX]
    lpk = kl[k - 1] - kl.max() - math.log(np.exp(kl - kl.max()).sum())
    return lpk + math.log(tot) if tot > 0 else -math.inf


def gelu(z):
    from scipy.special import erf
    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def unpack_params(flat, n_sites):
    Kin = ((2 * n_sites + 63) // 64) * 64
    sizes = [PH * Kin, PH, PH * PH, PH, PLOG * PH, PLOG]
    out, o = [], 0
    for s in sizes:
        out.append(np.asarray(flat[o:o + s], np.float64))
        o += s
    W1, b1, W2, b2, Wo, bo = out
    return W1.reshape(PH, Kin), b1, W2.reshape(PH, PH), b2, Wo.reshape(PLOG, PH), bo, Kin


def inputs(x, n_sites, Kin):
    X = np.zeros((x.shape[0], Kin))
    X[:, :2 * n_sites] = quimb_to_netket(x)
    return X


def logits(flat, x, n_sites):
    W1, b1, W2, b2, Wo, bo, Kin = unpack_params(flat, n_sites)
    h = gelu(inputs(x, n_sites, Kin) @ W1.T + b1)
    h = gelu(h @ W2.T + b2)
    return h @ Wo.T + bo


def loss_and_grad(flat, x, tgt, ktgt, kweight, edges, n_sites):
    """Mean over rows of the masked cross entropy (hop targets normalised over
    valid hops) + kweight * CE(k); gradient w.r.t. the flat parameters (FP64)."""
    W1, b1, W2, b2, Wo, bo, Kin = [torch.tensor(a, requires_grad=True) if isinstance(a, np.ndarray) else a
                                   for a in unpack_params(flat, n_sites)]
    X = torch.tensor(inputs(x, n_sites, Kin))
    H = 2 * len(edges)
    h = torch.nn.functional.gelu(X @ W1.T + b1)
    h = torch.nn.functional.gelu(h @ W2.T + b2)
    L = h @ Wo.T + bo
    valid = torch.tensor(valid_hops(x, edges))
    t = torch.tensor(np.asarray(tgt, np.float64)) * valid
    ts = t.sum(1, keepdim=True)
    lh = L[:, :H].masked_fill(~valid, -1e300)
    logp = lh - torch.logsumexp(lh, dim=1, keepdim=True)
    ce = -(torch.where(t > 0, (t / ts.clamp_min(1e-300)) * logp, torch.zeros_like(logp))).sum(1)
    ce = torch.where(ts[:, 0] > 0, ce, torch.zeros_like(ce))
    kl = torch.log_softmax(L[:, H:H + KMAX], dim=1)
    kt = torch.tensor(np.asarray(ktgt, np.float64))
    ck = -(torch.where(kt > 0, kt * kl, torch.zeros_like(kl))).sum(1)
    loss = (ce + kweight * ck).mean()
    loss.backward()
    g = torch.cat([p.grad.reshape(-1) for p in (W1, b1, W2, b2, Wo, bo)])
    return float(loss.item()), g.numpy()


def transition_matrix(states, logits_fn, amp, edges):
    """Exact MH transition matrix of the learned proposal on an enumerable
    sector: P[x, y] = q(x->y) min(1, |psi_y|^2 q(y->x) / (|psi_x|^2 q(x->y)))."""
    index = {tuple(s): n for n, s in enumerate(states.tolist())}
    S = len(states)
    H = 2 * len(edges)
    L = logits_fn(states)
    P = np.zeros((S, S))
    for a in range(S):
        x = states[a]
        valid = np.nonzero(valid_hops(x[None], edges)[0])[0]
        for k in range(1, KMAX + 1):
            for hs in itertools.combinations(valid, k):
                if any(conflict(p, q, edges) for p, q in itertools.combinations(hs, 2)):
                    continue
                qf = math.exp(log_q(L[a], x, list(hs), edges))
                y = apply_hops(x, hs, edges)
                b = index[tuple(y)]
                qr = math.exp(log_q(L[b], y, list(hs), edges))
                ratio = (amp[b] ** 2 * qr) / (amp[a] ** 2 * qf)
                P[a, b] += qf * min(1.0, ratio)
        P[a, a] += 1.0 - P[a].sum()
    return P
