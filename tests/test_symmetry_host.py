"""Host-side checks of the point-group projection (no GPU): the group built by
the model (vmc_torch/GPU/models/symmetry.py:63-146 element order) equals the
oracle's, is closed under composition, its 1D irrep characters multiply as
characters, and the model rejects bad arguments like the reference."""
import itertools

import numpy as np
import pytest

from oracle import symmetry as osym
import vmc_torch_gb300 as vg


@pytest.mark.parametrize("Lx,Ly", [(4, 4), (4, 2), (6, 6), (3, 5), (8, 8)])
def test_group_matches_oracle_and_is_a_group(Lx, Ly):
    perms, chars, names = vg.build_symmetry_group(Lx, Ly)
    ops, ochars = osym.group(Lx, Ly)
    assert np.array_equal(perms.numpy(), ops)
    assert chars == ochars
    G = perms.shape[0]
    assert G == (8 if Lx == Ly else 4) and len(names) == G
    assert all(sorted(p.tolist()) == list(range(Lx * Ly)) for p in perms)
    assert perms[0].tolist() == list(range(Lx * Ly))
    index = {tuple(p.tolist()): i for i, p in enumerate(perms)}
    # image of g is x[perm_g]: applying b then a gives x[perm_b][perm_a] = x[perm_b[perm_a]]
    for a, b in itertools.product(range(G), range(G)):
        c = index[tuple(perms[b][perms[a]].tolist())]
        for ch in chars.values():
            assert ch[c] == ch[a] * ch[b]


def test_inverse_permutations():
    perms, _, _ = vg.build_symmetry_group(4, 4)
    inv = osym.inverse_perms(perms.numpy())
    for p, q in zip(perms.numpy(), inv):
        assert np.array_equal(p[q], np.arange(16))


def test_projected_model_arguments():
    base = vg.SlaterDeterminant_GB300(32, 16)   # 16 sites
    with pytest.raises(ValueError):
        vg.FermionSymmetryProjectedModel_GB300(base, 4, 4, "E")
    with pytest.raises(ValueError):
        vg.FermionSymmetryProjectedModel_GB300(base, 4, 2, "A1")
    pm = vg.FermionSymmetryProjectedModel_GB300(base, 4, 4, "B2")
    assert pm.n_group == 8 and pm.n_params == base.n_params
    assert all(p is q for p, q in zip(pm.params, base.params))
    assert pm.characters.tolist() == vg.build_symmetry_group(4, 4)[1]["B2"]
