"""Pin the CPU oracle against golden vectors produced by the reference's own
code (tests/golden/make_golden.py) and against the reference's shipped 4x2
example data."""
import json

import numpy as np
import pytest

from oracle import hubbard, lattice, models, sampler, sr
from oracle.lattice import pack


def canonical(etas, coeffs, bids, B):
    pk = pack(etas)
    rows = []
    for b in range(B):
        m = np.nonzero(bids == b)[0]
        key = sorted((int(pk[k, 0]), int(pk[k, 1]), float(coeffs[k])) for k in m)
        rows.extend((b, u, d, c) for (u, d, c) in key)
    return rows


@pytest.mark.parametrize("case", ["4x2", "8x8"])
def test_connected_sets_match_reference(golden, case):
    g = golden("conn.npz")
    if case == "4x2":
        X = g["states_4x2"].astype(np.int64)
        Lx, Ly = 4, 2
    else:
        X = g["x_8x8"].astype(np.int64)
        Lx, Ly = 8, 8
    e, c, b = hubbard.get_conn_batch(X, lattice.square_edges(Lx, Ly), 1.0, 8.0)
    mine = canonical(e, c, b, len(X))
    ref = [(int(bb), int(u), int(d), float(cc)) for bb, (u, d), cc in
           zip(g[f"bid_{case}"], g[f"pk_{case}"], g[f"coeff_{case}"])]
    assert mine == ref  # bit-exact: configs, multiplicities and signs


def test_encodings_roundtrip():
    X = lattice.random_initial_configs(50, 36, 16, 16, seed=1)
    assert np.array_equal(lattice.unpack(lattice.pack(X), 36), X)
    assert np.array_equal(lattice.netket_to_quimb(lattice.quimb_to_netket(X)), X)
    sy = lattice.quimb_to_symmray(X)
    nk = lattice.quimb_to_netket(X)
    assert np.array_equal(sy[:, 1::2], nk[:, :36]) and np.array_equal(sy[:, 0::2], nk[:, 36:])


def test_ed_and_checkpoints(golden):
    g = golden("ed_4x2.npz")
    S, H = hubbard.dense_hamiltonian(8, 4, 4, lattice.square_edges(4, 2), 1.0, 8.0)
    assert len(S) == 4900
    E0 = np.linalg.eigvalsh(H)[0]
    assert abs(E0 - float(g["E0"])) < 1e-10
    assert abs(E0 - (-3.025922805691)) < 1e-9
    for M, ex, mc, err in zip(g["ckpt_M"], g["ckpt_exact"], g["ckpt_mc_mean"], g["ckpt_mc_err"]):
        psi = models.slater_amp(M, S)
        E = hubbard.exact_energy(psi, H)
        assert abs(E - ex) < 1e-10
    # the last shipped MC energy agrees with the exact energy of its parameters
    assert abs(g["ckpt_exact"][-1] - g["ckpt_mc_mean"][-1]) < 3 * g["ckpt_mc_err"][-1]
    hist = json.loads(str(g["hist_json"]))
    assert len(hist["mean"]) == 50 and abs(hist["mean"][0] - g["ckpt_mc_mean"][0]) < 1e-12


def test_slater_amplitudes_match_reference(golden):
    g = golden("slater.npz")
    cg = golden("conn.npz")
    S = cg["states_4x2"].astype(np.int64)
    amp = models.slater_amp(g["M"], S)
    np.testing.assert_allclose(amp, g["amps_all"], rtol=1e-10, atol=0)


def test_slater_replayed_sweep_matches_reference(golden):
    g = golden("slater.npz")
    M = g["M"]
    fn = lambda x: models.slater_logamp(M, x)
    x, (s, l), _ = sampler.sweep(g["x0"], lattice.sweep_edges(4, 2), fn,
                                 g["u_move"], g["hop_bit"], g["u_acc"])
    assert np.array_equal(x, g["x_final"])
    np.testing.assert_allclose(s * np.exp(l), g["amps_final"], rtol=1e-10)


def test_slater_local_energy_and_O_match_reference(golden):
    g = golden("slater.npz")
    M = g["M"]
    x = g["x_final"]
    eloc = hubbard.local_energy(x, lattice.square_edges(4, 2), 1.0, 8.0,
                                lambda y: models.slater_amp(M, y))
    np.testing.assert_allclose(eloc, g["eloc"], rtol=1e-10, atol=1e-10)
    O = models.slater_O(M, x)
    np.testing.assert_allclose(O, g["O"], rtol=1e-10, atol=1e-10)


def _nnbf_params(g):
    ps = models.nnbf_init(64, 64, 256, 2, seed=int(g["seed"]))
    import hashlib
    h = hashlib.sha256()
    for p in ps:
        h.update(np.ascontiguousarray(p, dtype=np.float64).tobytes())
    if h.hexdigest() != str(g["params_sha256"]):
        pytest.skip("numpy normal stream differs from the one that made the fixture")
    return ps


def test_nnbf_logamp_matches_reference(golden):
    g = golden("nnbf.npz")
    ps = _nnbf_params(g)
    s, l = models.nnbf_logamp(ps, g["x"].astype(np.int64), 0.01)
    assert np.array_equal(s, g["sign"])
    np.testing.assert_allclose(l, g["logabs"], rtol=1e-11, atol=1e-11)


def test_nnbf_sweep_energy_and_O_match_reference(golden):
    g = golden("nnbf.npz")
    ps = _nnbf_params(g)
    fn = lambda x: models.nnbf_logamp(ps, x, 0.01)
    x, (s, l), _ = sampler.sweep(g["x0"].astype(np.int64), lattice.sweep_edges(8, 8), fn,
                                 g["u_move"], g["hop_bit"], g["u_acc"])
    assert np.array_equal(x, g["x_final"].astype(np.int64))
    assert np.array_equal(s, g["sign_final"])
    np.testing.assert_allclose(l, g["logabs_final"], rtol=1e-11, atol=1e-11)
    eloc = hubbard.local_energy(x, lattice.square_edges(8, 8), 1.0, 8.0,
                                lambda y: models.nnbf_amp(ps, y, 0.01))
    np.testing.assert_allclose(eloc, g["eloc"], rtol=1e-9, atol=1e-9)
    O = models.nnbf_O(ps, x[:4], 0.01)
    np.testing.assert_allclose(O[:, g["O_cols"]], g["O_sub"], rtol=1e-9, atol=1e-12)
    r = np.random.default_rng(int(g["proj_seed"])).standard_normal(O.shape[1])
    np.testing.assert_allclose(O @ r, g["O_proj"], rtol=1e-9)


def test_minsr_matches_reference(golden):
    g = golden("minsr.npz")
    dp = sr.minsr(g["O"], g["E"], float(g["E"].mean()), float(g["diag_shift"]))
    np.testing.assert_allclose(dp, g["dp"], rtol=1e-9, atol=1e-12)


def test_tau_int_known_answer():
    # AR(1) with coefficient a has tau_int = (1 + a) / (1 - a)
    rng = np.random.default_rng(0)
    a = 0.8
    n, L = 64, 4000
    x = np.zeros((n, L))
    e = rng.standard_normal((n, L))
    for t in range(1, L):
        x[:, t] = a * x[:, t - 1] + e[:, t]
    tau = sr.tau_int(x[:, 200:])
    assert abs(tau - 9.0) < 1.0
    assert abs(sr.tau_int(rng.standard_normal((16, 2000))) - 1.0) < 0.15
