"""The symmetry-projection oracle against the reference's own outputs
(tests/golden/sym.npz: FermionSymmetryProjectedModel over a Slater base)."""
import numpy as np
import pytest

from oracle import models as om, symmetry as osym
from oracle.lattice import random_initial_configs


@pytest.mark.parametrize("tag,Lx,Ly", [("4x2", 4, 2), ("4x4", 4, 4)])
def test_group_signs_and_projection_match_reference(golden, tag, Lx, Ly):
    g = golden("sym.npz")
    perms, chars = osym.group(Lx, Ly)
    assert np.array_equal(perms, g[tag + "_perms"])
    X = g[tag + "_x"].astype(np.int64)
    assert np.array_equal(osym.fermion_signs(X, perms), g[tag + "_fsign"])
    M = g[tag + "_M"]
    for irrep in ("A1", "A2", "B1", "B2"):
        assert np.array_equal(np.asarray(chars[irrep], dtype=np.float64), g[tag + "_" + irrep + "_chars"])
        psi = osym.projected_amp(lambda y: om.slater_amp(M, y), X, perms, chars[irrep])
        ref = g[tag + "_" + irrep + "_sign"] * np.exp(g[tag + "_" + irrep + "_logabs"])
        np.testing.assert_allclose(psi, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


def test_projected_O_matches_finite_differences():
    perms, chars = osym.group(4, 2)
    rng = np.random.default_rng(1)
    M = rng.standard_normal((16, 8))
    X = random_initial_configs(3, 8, 4, 4, seed=4)
    O = osym.projected_O(lambda y: om.slater_amp(M, y), lambda y: om.slater_O(M, y), X, perms, chars["A1"])
    h = 1e-6
    for k in (0, 17, 63, 100):
        Mp, Mm = M.copy(), M.copy()
        Mp.flat[k] += h
        Mm.flat[k] -= h
        fp = np.log(np.abs(osym.projected_amp(lambda y: om.slater_amp(Mp, y), X, perms, chars["A1"])))
        fm = np.log(np.abs(osym.projected_amp(lambda y: om.slater_amp(Mm, y), X, perms, chars["A1"])))
        np.testing.assert_allclose(O[:, k], (fp - fm) / (2 * h), rtol=1e-5, atol=1e-7)
