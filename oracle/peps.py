"""Fermionic PEPS amplitude (oracle, test-only; FP64).

The reference's fPEPS (vmc_torch/GPU/models/pureTNS.py:24-160) contracts
symmray Z2-graded tensors with quimb's boundary-MPS (max_bond chi; rows
[0, Lx/2-1] from xmin, rows [Lx/2, Lx-1] from xmax, pureTNS.py:103-114).
Neither library is available here, so this restatement defines the ansatz
itself, from the Grassmann tensor-network definition of a fermionic PEPS:

  * site tensors T[r][c][s][l, u, r', d], bond dimension D, physical states s
    in the quimb encoding {0, 1 = down, 2 = up, 3 = up+down}; layout
    (Lx, Ly, 4, D, D, D, D);
  * Z2 grading: bond index k has parity k mod 2, state s has parity
    (electron count) mod 2, and T[s][l,u,r',d] = 0 unless the total parity is
    even;
  * open boundaries: legs leaving the lattice carry index 0 only;
  * the state is |psi> = Int prod_i T_i, with T_i = sum T[s](l,u,r',d)
    (c+_i)^s th_l th_u th_d th_r' (Grassmann bond variables in the order
    left, up, down, right; sites in row-major order i = r*Ly + c, the order
    of the Hamiltonian's modes), each bond integrated as an adjacent pair
    (th th-bar) = 1.  psi(x) is the coefficient of prod_i (c+_i)^{x_i}|0> in
    row-major order.

``amp_grassmann`` evaluates that definition literally (enumerates every bond
assignment and takes the sign of the permutation of odd Grassmann symbols into
the target order); it is the independent ground truth for small lattices.

Reordering the symbols gives (derivation in ``sign_rule``'s docstring)
    psi(x) = (-1)^{K(K-1)/2} * Z(T~[x])
with K the number of singly-occupied sites, Z the plain (bosonic) contraction
and T~ the site tensors with the up leg of every site in rows >= 1 multiplied
by (-1)^{p(u) * (p(l) + n_left)}, n_left = electron count to the left in the
same row.  ``amp_rows`` is the exact row-boundary contraction of that network
that the GPU kernel uses (top rows into an MPS, bottom rows into an MPS, the
two middle rows swept column by column): the chi -> infinity limit of the
reference's boundary contraction.  ``amp_boundary_chi`` is the reference-style
truncated contraction (SVD compression to bond chi after each absorbed row).
"""
import itertools

import numpy as np

S_PARITY = np.array([0, 1, 1, 0])
S_COUNT = np.array([0, 1, 1, 2])


def parity_mask(D):
    b = np.arange(D) % 2
    tot = (S_PARITY[:, None, None, None, None] + b[None, :, None, None, None] + b[None, None, :, None, None]
           + b[None, None, None, :, None] + b[None, None, None, None, :])
    return (tot % 2) == 0


def boundary_mask(Lx, Ly, D):
    """(Lx, Ly, 1, D, D, D, D) mask of allowed bond indices (index 0 on open edges)."""
    m = np.ones((Lx, Ly, 1, D, D, D, D), dtype=bool)
    for r in range(Lx):
        for c in range(Ly):
            if c == 0:
                m[r, c, :, 1:, :, :, :] = False
            if r == 0:
                m[r, c, :, :, 1:, :, :] = False
            if c == Ly - 1:
                m[r, c, :, :, :, 1:, :] = False
            if r == Lx - 1:
                m[r, c, :, :, :, :, 1:] = False
    return m


def init_tensors(Lx, Ly, D, seed, scale=1.0):
    """N(0, scale^2) entries, zeroed outside the parity / boundary structure
    (the reference initialises config 5 with random N(0,1) site tensors)."""
    g = np.random.default_rng(seed)
    T = g.normal(0.0, scale, size=(Lx, Ly, 4, D, D, D, D))
    T *= parity_mask(D)[None, None]
    T *= boundary_mask(Lx, Ly, D)
    return T


# ----------------------------------------------------------------------------
# Ground truth: literal Grassmann contraction
# ----------------------------------------------------------------------------

def _bonds(Lx, Ly):
    """Internal bonds as (site_a, leg_a, site_b, leg_b), site_a < site_b;
    legs numbered 0=l, 1=u, 2=r, 3=d (tensor axis order)."""
    out = []
    for r in range(Lx):
        for c in range(Ly):
            i = r * Ly + c
            if c + 1 < Ly:
                out.append((i, 2, i + 1, 0))
            if r + 1 < Lx:
                out.append((i, 3, i + Ly, 1))
    return out


# position of each leg inside a site's Grassmann monomial: l, u, d, r
_LEG_SLOT = {0: 1, 1: 2, 3: 3, 2: 4}


def amp_grassmann(T, x, chunk=1 << 16):
    """psi(x) by enumerating all internal bond assignments (D^n_bonds terms)."""
    Lx, Ly, _, D = T.shape[:4]
    N = Lx * Ly
    x = np.asarray(x, dtype=np.int64)
    bonds = _bonds(Lx, Ly)
    nb = len(bonds)
    # symbols: physical of site i (slot 0), then two per bond
    src_key = [(i, 0) for i in range(N)]
    tgt_key = [(0, i, 0) for i in range(N)]
    for k, (a, la, b, lb) in enumerate(bonds):
        src_key += [(a, _LEG_SLOT[la]), (b, _LEG_SLOT[lb])]
        tgt_key += [(1, k, 0), (1, k, 1)]
    ns = len(src_key)
    src_rank = np.argsort(np.argsort([k[0] * 8 + k[1] for k in src_key]))
    tgt_order = sorted(range(ns), key=lambda s: tgt_key[s])
    tgt_rank = np.empty(ns, dtype=np.int64)
    tgt_rank[tgt_order] = np.arange(ns)
    inv = ((src_rank[:, None] < src_rank[None, :]) & (tgt_rank[:, None] > tgt_rank[None, :])).astype(np.int64)
    # leg -> bond column per site
    legcol = -np.ones((N, 4), dtype=np.int64)
    for k, (a, la, b, lb) in enumerate(bonds):
        legcol[a, la] = k
        legcol[b, lb] = k
    A = [T[i // Ly, i % Ly, x[i]] for i in range(N)]
    phys_par = S_PARITY[x]
    total = 0.0
    n_assign = D ** nb
    for start in range(0, n_assign, chunk):
        idx = np.arange(start, min(n_assign, start + chunk), dtype=np.int64)
        asg = np.empty((idx.size, nb), dtype=np.int64)
        rem = idx.copy()
        for k in range(nb):
            asg[:, k] = rem % D
            rem //= D
        val = np.ones(idx.size)
        for i in range(N):
            legs = [asg[:, legcol[i, g]] if legcol[i, g] >= 0 else np.zeros(idx.size, dtype=np.int64)
                    for g in range(4)]
            val *= A[i][legs[0], legs[1], legs[2], legs[3]]
        par = np.empty((idx.size, ns), dtype=np.int64)
        par[:, :N] = phys_par[None, :]
        par[:, N::2] = asg & 1
        par[:, N + 1::2] = asg & 1
        expo = ((par @ inv) * par).sum(axis=1) & 1
        total += float(np.sum(val * (1 - 2 * expo)))
    return total


# ----------------------------------------------------------------------------
# Local sign rule and the plain contractions
# ----------------------------------------------------------------------------

def sign_rule(T, x):
    """(global sign, signed tensors A[r, c] = T~[r][c][x_rc]).

    Derivation.  Moving every physical symbol to the front passes the bond
    monomials of the earlier sites, whose parity equals their site's
    electron parity (each tensor is even): sign (-1)^{sum_{j<i} p_i p_j} =
    (-1)^{K(K-1)/2}.  Bringing each bond's pair together costs (-1)^{p p'} for
    every pair of interleaved bonds.  With the slot order l, u, d, r the only
    interleaved pairs are vertical bonds (i, i+Ly), (j, j+Ly) with
    i < j < i+Ly: the same row layer (c < c') and the next layer (c' < c).
    Z2 evenness of the row segment left of column c turns the parity of the
    vertical legs left of c into horizontal-bond and electron parities, and
    the product collapses to one factor per vertical bond (r-1, c)-(r, c):
    (-1)^{p(u_rc) * (p(l_rc) + sum_{c'<c} n_{r c'})}, a sign on the up leg of
    site (r, c) fixed by its own left leg and the row's electrons to its
    left."""
    Lx, Ly, _, D = T.shape[:4]
    x = np.asarray(x, dtype=np.int64).reshape(Lx, Ly)
    K = int(np.sum(S_PARITY[x]))
    gsign = -1.0 if (K * (K - 1) // 2) % 2 else 1.0
    bp = np.arange(D) % 2
    A = np.empty((Lx, Ly, D, D, D, D))
    for r in range(Lx):
        nleft = 0
        for c in range(Ly):
            a = T[r, c, x[r, c]].copy()
            if r > 0:
                e = (bp[None, :] * (bp[:, None] + nleft)) % 2          # (l, u)
                a *= (1 - 2 * e)[:, :, None, None]
            A[r, c] = a
            nleft += int(S_COUNT[x[r, c]])
    return gsign, A


def _contract_plain(A):
    """Plain contraction of the selected-tensor network (open legs at index 0),
    site by site in row-major order through a frontier F[v_0..v_{Ly-1}][h]
    (open down legs of the last row of sites, right leg of the last site) --
    a different contraction order from ``amp_rows``."""
    Lx, Ly, D = A.shape[0], A.shape[1], A.shape[2]
    F = np.zeros((D,) * (Ly + 1))
    F[(0,) * (Ly + 1)] = 1.0
    for r in range(Lx):
        for c in range(Ly):
            if c == 0:  # the previous row's right boundary leg is index 0
                F = F[..., :1] * np.eye(D)[0]
            G = np.moveaxis(F, (c, Ly), (-2, -1))
            G = np.einsum("...ul,lurd->...dr", G, A[r, c])
            F = np.moveaxis(G, (-2, -1), (c, Ly))
    return float(F[(0,) * (Ly + 1)])


def amp_bruteforce(T, x):
    """Sign rule + whole-network einsum (small lattices)."""
    g, A = sign_rule(T, x)
    return g * _contract_plain(A)


def _boundary_mpses(A):
    """Top MPS of rows [0, Lx/2-2] as (a, u-down, b) and bottom MPS of rows
    [Lx/2+1, Lx-1] as (a, d-up, b), exact."""
    Lx, Ly, D = A.shape[0], A.shape[1], A.shape[2]
    mid = Lx // 2 - 1
    M = [A[0, c][:, 0, :, :].transpose(0, 2, 1) for c in range(Ly)]          # (l, d, r)
    for r in range(1, mid):
        M = [np.einsum("aub,lurd->aldbr", M[c], A[r, c]).reshape(M[c].shape[0] * D, D, M[c].shape[2] * D)
             for c in range(Ly)]
    N = [A[Lx - 1, c][:, :, :, 0] for c in range(Ly)]                          # (l, u, r)
    for r in range(Lx - 2, mid + 1, -1):
        N = [np.einsum("adb,lurd->alubr", N[c], A[r, c]).reshape(N[c].shape[0] * D, D, N[c].shape[2] * D)
             for c in range(Ly)]
    return M, N, mid


def col_step(E, M, A2, A3, N):
    """E(a, l2, l3, a') -> E'(b, r2, r3, b') through one column of the two middle
    rows: M(a, u2, b) top MPS, A2(l2, u2, r2, d2), A3(l3, d2, r3, d3), N(a', d3, b')."""
    X = np.einsum("apqz,aub->ubpqz", E, M)
    X = np.einsum("ubpqz,purd->brdqz", X, A2)
    X = np.einsum("brdqz,qdse->brsez", X, A3)
    return np.einsum("brsez,zew->brsw", X, N)


def amp_rows_signed(A):
    """Exact row-boundary contraction of a selected, signed network A (Lx even, >= 4)."""
    Lx, Ly, D = A.shape[0], A.shape[1], A.shape[2]
    assert Lx % 2 == 0 and Lx >= 4
    M, N, mid = _boundary_mpses(A)
    E = np.zeros((M[0].shape[0], D, D, N[0].shape[0]))
    E[0, 0, 0, 0] = 1.0
    for c in range(Ly):
        E = col_step(E, M[c], A[mid, c], A[mid + 1, c], N[c])
    return float(E[0, 0, 0, 0])


def amp_rows(T, x):
    """psi(x) by the exact row-boundary contraction (the GPU kernel's algorithm)."""
    g, A = sign_rule(T, x)
    return g * amp_rows_signed(A)


def _compress(mps, chi):
    """Left-to-right QR canonicalisation, then right-to-left SVD truncation to
    bond chi (cutoff 0): the compression quimb's boundary contraction applies
    after absorbing a row.  Tensors are (a, p, b)."""
    mps = [t.copy() for t in mps]
    L = len(mps)
    for i in range(L - 1):
        a, p, b = mps[i].shape
        q, r = np.linalg.qr(mps[i].reshape(a * p, b))
        mps[i] = q.reshape(a, p, q.shape[1])
        mps[i + 1] = np.einsum("xb,bpc->xpc", r, mps[i + 1])
    for i in range(L - 1, 0, -1):
        a, p, b = mps[i].shape
        u, s, vh = np.linalg.svd(mps[i].reshape(a, p * b), full_matrices=False)
        k = min(chi, s.size)
        mps[i] = vh[:k].reshape(k, p, b)
        mps[i - 1] = np.einsum("xpa,ak->xpk", mps[i - 1], u[:, :k] * s[:k])
    return mps


def amp_boundary_chi(T, x, chi):
    """Reference-style boundary contraction: rows [0, Lx/2-1] absorbed from
    the top and rows [Lx/2, Lx-1] from the bottom into MPSs compressed to bond
    chi after every row, then the two MPSs contracted
    (vmc_torch/GPU/models/pureTNS.py:103-114)."""
    g, A = sign_rule(T, x)
    Lx, Ly, D = A.shape[0], A.shape[1], A.shape[2]
    half = Lx // 2
    top = [A[0, c][:, 0, :, :].transpose(0, 2, 1) for c in range(Ly)]
    for r in range(1, half):
        top = [np.einsum("aub,lurd->aldbr", top[c], A[r, c]).reshape(top[c].shape[0] * D, D, top[c].shape[2] * D)
               for c in range(Ly)]
        top = _compress(top, chi)
    bot = [A[Lx - 1, c][:, :, :, 0] for c in range(Ly)]
    for r in range(Lx - 2, half - 1, -1):
        bot = [np.einsum("adb,lurd->alubr", bot[c], A[r, c]).reshape(bot[c].shape[0] * D, D, bot[c].shape[2] * D)
               for c in range(Ly)]
        bot = _compress(bot, chi)
    E = np.ones((1, 1))
    for c in range(Ly):
        E = np.einsum("ab,apc,bpd->cd", E, top[c], bot[c])
    return g * float(E[0, 0])


def chi_schedule(Lx, Ly, D, chi):
    """Cuts truncated after each absorbed row of one side (absorption order),
    from static bounds on the Schmidt rank: a row multiplies the bond across
    cut k by D, the rank never exceeds min(D^k, D^(Ly-k)), truncating cut k to
    chi bounds cut k-1 by D*chi.  Cuts whose bound is <= chi need no SVD (the
    truncation is the identity there).  Rows before the second are never
    compressed (amp_boundary_chi starts from the bare first row)."""
    b = [1] * (Ly + 1)
    out = []
    for a in range(Lx // 2):
        for k in range(1, Ly):
            b[k] = min(b[k] * D, D ** k, D ** (Ly - k))
        cuts = []
        if a >= 1:
            for k in range(Ly - 1, 0, -1):
                if b[k] > chi:
                    cuts.append(k)
                    b[k] = chi
                    if k > 1:
                        b[k - 1] = min(b[k - 1], D * chi)
        out.append(cuts)
    return out


def _truncate_cut(psi, Ly, D, k, chi):
    """Best rank-chi approximation of the state psi (D^Ly, column 0 most
    significant) across the cut after k columns."""
    M = psi.reshape(D ** k, D ** (Ly - k))
    u, s, vh = np.linalg.svd(M, full_matrices=False)
    r = min(chi, s.size)
    return ((u[:, :r] * s[:r]) @ vh[:r]).reshape(-1)


def amp_state_chi(T, x, chi, with_norms=False):
    """amp_boundary_chi restated on the full boundary state: each side's
    boundary is kept as a vector over the D^Ly open legs, a row is absorbed
    exactly, and the compression (left-to-right QR, right-to-left truncated
    SVD) becomes the sequence of best rank-chi truncations across cuts
    Ly-1, ..., 1 of that vector -- in the canonical sweep the SVD at cut k is
    the Schmidt decomposition of the whole current state across that cut.
    The algorithm of the GPU kernels (vmc_peps_chi_*)."""
    g, A = sign_rule(T, x)
    Lx, Ly, D = A.shape[0], A.shape[1], A.shape[2]
    sched = chi_schedule(Lx, Ly, D, chi)

    def side(rows, top):
        psi = np.zeros(D ** Ly)
        psi[0] = 1.0
        for a, r in enumerate(rows):
            W = psi.reshape((D,) * Ly)[..., None] * np.eye(D)[0]       # (d_0..d_{Ly-1}, h)
            for c in range(Ly):
                t = A[r, c] if top else A[r, c].transpose(0, 3, 2, 1)   # (h, old, h', new)
                W = np.moveaxis(W, c, -2)
                W = np.einsum("...oh,hopn->...np", W, t)
                W = np.moveaxis(W, -2, c)
            psi = W[..., 0].reshape(-1)
            for k in sched[a]:
                psi = _truncate_cut(psi, Ly, D, k, chi)
        return psi

    top = side(range(0, Lx // 2), True)
    bot = side(range(Lx - 1, Lx // 2 - 1, -1), False)
    if with_norms:  # (psi, |top| |bot|): the scale of the final overlap's cancellation
        return g * float(top @ bot), float(np.linalg.norm(top) * np.linalg.norm(bot))
    return g * float(top @ bot)


def logamp_grad_chi(T, x, chi):
    """d log|psi_chi| / d T (FP64) by torch autograd through the full-state
    chi-truncated contraction with torch.linalg.svd at every scheduled cut
    (the reference differentiates its quimb contraction with torch autograd,
    vmc_torch/GPU/vmc_utils.py:1389-1634, through the same truncated SVDs)."""
    import torch
    Lx, Ly, _, D = T.shape[:4]
    x = np.asarray(x, dtype=np.int64).reshape(Lx, Ly)
    Tt = torch.tensor(T, dtype=torch.float64, requires_grad=True)
    bp = np.arange(D) % 2
    A = [[None] * Ly for _ in range(Lx)]
    for r in range(Lx):
        nleft = 0
        for c in range(Ly):
            a = Tt[r, c, int(x[r, c])]
            if r > 0:
                e = (bp[None, :] * (bp[:, None] + nleft)) % 2
                a = a * torch.tensor((1 - 2 * e)[:, :, None, None], dtype=torch.float64)
            A[r][c] = a
            nleft += int(S_COUNT[x[r, c]])
    sched = chi_schedule(Lx, Ly, D, chi)
    eye0 = torch.zeros(D, dtype=torch.float64)
    eye0[0] = 1.0

    def side(rows, top):
        psi = torch.zeros(D ** Ly, dtype=torch.float64)
        psi = psi.index_put((torch.tensor([0]),), torch.tensor([1.0], dtype=torch.float64))
        for a, r in enumerate(rows):
            W = psi.reshape((D,) * Ly)[..., None] * eye0
            for c in range(Ly):
                t = A[r][c] if top else A[r][c].permute(0, 3, 2, 1)
                W = torch.movedim(W, c, -2)
                W = torch.einsum("...oh,hopn->...np", W, t)
                W = torch.movedim(W, -2, c)
            psi = W[..., 0].reshape(-1)
            for k in sched[a]:
                M = psi.reshape(D ** k, D ** (Ly - k))
                u, sv, vh = torch.linalg.svd(M, full_matrices=False)
                rk = min(chi, sv.shape[0])
                psi = ((u[:, :rk] * sv[:rk]) @ vh[:rk]).reshape(-1)
        return psi

    top = side(range(0, Lx // 2), True)
    bot = side(range(Lx - 1, Lx // 2 - 1, -1), False)
    z = top @ bot
    torch.log(torch.abs(z)).backward()
    return Tt.grad.numpy()


def trunc_adjoint(M, B, k):
    """Cotangent of the rank-k truncation P(M) = U_k S_k V_k^T against B:
    d<P(M), B> = <dM, Mbar> with
        Mbar = P_k B + sum_{i < k <= j} w_ij (q_j u_i^T + q_i u_j^T),
        w_ij = (q_j^T B u_i + q_i^T B u_j) / (s_i^2 - s_j^2),
    q the left singular vectors, u_i = s_i v_i (the first-order change of the
    kept singular subspace).  The formula vmc_peps_chi_logpsi_grad evaluates
    per parity block (FP64 numpy here, test infrastructure)."""
    u, sv, vh = np.linalg.svd(M)
    n = sv.size
    Q = u[:, :n].T                     # rows q_i
    U = sv[:, None] * vh[:n]           # rows u_i = s_i v_i
    lam = sv ** 2
    C = Q @ B
    X = C @ U.T                        # X[a][c] = q_a^T B u_c
    keep = np.arange(n) < k
    R = keep[:, None] * C
    for a in range(n):
        for c in range(n):
            if keep[a] == keep[c]:
                continue
            den = (lam[a] - lam[c]) if keep[a] else (lam[c] - lam[a])
            R[a] = R[a] + (X[a, c] + X[c, a]) / den * U[c]
    return Q.T @ R


def logamp(T, X, method="rows", chi=None):
    if method == "chi":
        a = np.array([amp_state_chi(T, x, chi) for x in np.asarray(X)])
        return np.sign(a), np.log(np.maximum(np.abs(a), 1e-300))
    f = {"rows": amp_rows, "brute": amp_bruteforce, "grassmann": amp_grassmann}[method]
    a = np.array([f(T, x) for x in np.asarray(X)])
    return np.sign(a), np.log(np.maximum(np.abs(a), 1e-300))


def all_bond_assignments(D, n):
    return np.array(list(itertools.product(range(D), repeat=n)), dtype=np.int64)


def logamp_grad(T, x):
    """d log|psi| / d T (FP64, torch autograd through the exact row contraction
    with the sign rule); shape of T, non-zero only at the selected states."""
    import torch
    Lx, Ly, _, D = T.shape[:4]
    x = np.asarray(x, dtype=np.int64).reshape(Lx, Ly)
    Tt = torch.tensor(T, dtype=torch.float64, requires_grad=True)
    bp = np.arange(D) % 2
    A = [[None] * Ly for _ in range(Lx)]
    for r in range(Lx):
        nleft = 0
        for c in range(Ly):
            a = Tt[r, c, int(x[r, c])]
            if r > 0:
                e = (bp[None, :] * (bp[:, None] + nleft)) % 2
                a = a * torch.tensor((1 - 2 * e)[:, :, None, None], dtype=torch.float64)
            A[r][c] = a
            nleft += int(S_COUNT[x[r, c]])
    mid = Lx // 2 - 1
    M = [A[0][c][:, 0, :, :].permute(0, 2, 1) for c in range(Ly)]
    for r in range(1, mid):
        M = [torch.einsum("aub,lurd->aldbr", M[c], A[r][c]).reshape(M[c].shape[0] * D, D, M[c].shape[2] * D)
             for c in range(Ly)]
    N = [A[Lx - 1][c][:, :, :, 0] for c in range(Ly)]
    for r in range(Lx - 2, mid + 1, -1):
        N = [torch.einsum("adb,lurd->alubr", N[c], A[r][c]).reshape(N[c].shape[0] * D, D, N[c].shape[2] * D)
             for c in range(Ly)]
    E = torch.zeros((M[0].shape[0], D, D, N[0].shape[0]), dtype=torch.float64)
    E[0, 0, 0, 0] = 1.0
    for c in range(Ly):
        X = torch.einsum("apqz,aub->ubpqz", E, M[c])
        X = torch.einsum("ubpqz,purd->brdqz", X, A[mid][c])
        X = torch.einsum("brdqz,qdse->brsez", X, A[mid + 1][c])
        E = torch.einsum("brsez,zew->brsw", X, N[c])
    z = E[0, 0, 0, 0]
    torch.log(torch.abs(z)).backward()
    return Tt.grad.numpy()
