"""Point-group symmetry projection with fermionic signs (oracle, test-only).

Restates vmc_torch/GPU/models/symmetry.py:
  * site permutations: C2v on an Lx x Ly lattice (identity, 180-degree
    rotation, reflections of the column and the row index;
    symmetry.py:63-90) and C4v on an L x L lattice (identity, rotations by
    90/180/270 degrees counter-clockwise, the two axis reflections, the two
    diagonal reflections; symmetry.py:112-146), site i = row * Ly + col;
    the image configuration of g is x[perm_g];
  * 1D irrep characters (symmetry.py:33-57);
  * the fermionic sign of g for configuration n: the parity of the number of
    pairs of occupied modes m1 < m2 (interleaved order 2 i + s, s = 0 down,
    1 up) whose images under the mode permutation of g^-1 are inverted
    (symmetry.py:698-760, with the inverse permutation of 788-808);
  * psi_r(n) = (1/|G|) sum_g sign(g, n) chi_r(g) psi(n[perm_g])
    (symmetry.py:902-957).
"""
import numpy as np

C4V_CHARACTERS = {"A1": [1, 1, 1, 1, 1, 1, 1, 1], "A2": [1, 1, 1, 1, -1, -1, -1, -1],
                  "B1": [1, -1, 1, -1, 1, 1, -1, -1], "B2": [1, -1, 1, -1, -1, -1, 1, 1]}
C2V_CHARACTERS = {"A1": [1, 1, 1, 1], "A2": [1, 1, -1, -1], "B1": [1, -1, 1, -1], "B2": [1, -1, -1, 1]}


def group(Lx, Ly):
    """(perms (G, N) int64, characters dict): C4v for Lx == Ly, else C2v."""
    N = Lx * Ly
    i = np.arange(N)
    r, c = i // Ly, i % Ly
    if Lx == Ly:
        L = Lx
        f = lambda a, b: a * L + b  # noqa: E731
        perms = np.stack([f(r, c), f(L - 1 - c, r), f(L - 1 - r, L - 1 - c), f(c, L - 1 - r),
                          f(r, L - 1 - c), f(L - 1 - r, c), f(c, r), f(L - 1 - c, L - 1 - r)])
        return perms.astype(np.int64), C4V_CHARACTERS
    f = lambda a, b: a * Ly + b  # noqa: E731
    perms = np.stack([f(r, c), f(Lx - 1 - r, Ly - 1 - c), f(r, Ly - 1 - c), f(Lx - 1 - r, c)])
    return perms.astype(np.int64), C2V_CHARACTERS


def inverse_perms(perms):
    inv = np.empty_like(perms)
    for g in range(perms.shape[0]):
        inv[g, perms[g]] = np.arange(perms.shape[1])
    return inv


def fermion_signs(X, perms):
    """(B, G) signs sign(g, n) for quimb configurations X (B, N)."""
    X = np.asarray(X, dtype=np.int64)
    B, N = X.shape
    inv = inverse_perms(perms)
    dn = ((X == 1) | (X == 3)).astype(np.int64)
    up = ((X == 2) | (X == 3)).astype(np.int64)
    occ = np.stack([dn, up], axis=-1).reshape(B, 2 * N)
    out = np.empty((B, perms.shape[0]))
    for g in range(perms.shape[0]):
        mp = np.empty(2 * N, dtype=np.int64)
        mp[0::2] = 2 * inv[g]
        mp[1::2] = 2 * inv[g] + 1
        inv_mask = np.triu(mp[:, None] > mp[None, :], k=1)
        cnt = np.einsum("mn,bm,bn->b", inv_mask.astype(np.int64), occ, occ)
        out[:, g] = 1.0 - 2.0 * (cnt % 2)
    return out


def projected_amp(amp_fn, X, perms, chars):
    """psi_r for configurations X given the base amplitude amp_fn((K, N)) -> (K,)."""
    X = np.asarray(X, dtype=np.int64)
    B = X.shape[0]
    G = perms.shape[0]
    fs = fermion_signs(X, perms)
    imgs = X[:, perms].reshape(B * G, -1)
    a = np.asarray(amp_fn(imgs)).reshape(B, G)
    return (a * fs * np.asarray(chars, dtype=np.float64)[None, :]).sum(axis=1) / G


def projected_O(amp_fn, O_fn, X, perms, chars):
    """d log|psi_r| / d theta = sum_g w_g O_g, w_g = sign chi psi_g / (|G| psi_r)."""
    X = np.asarray(X, dtype=np.int64)
    B = X.shape[0]
    G = perms.shape[0]
    fs = fermion_signs(X, perms)
    imgs = X[:, perms].reshape(B * G, -1)
    a = np.asarray(amp_fn(imgs)).reshape(B, G)
    Og = np.asarray(O_fn(imgs)).reshape(B, G, -1)
    c = fs * np.asarray(chars, dtype=np.float64)[None, :]
    psi = (a * c).sum(axis=1) / G
    w = c * a / (G * psi[:, None])
    return np.einsum("bg,bgp->bp", w, Og)
