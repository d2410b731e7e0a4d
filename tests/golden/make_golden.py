"""Generate the golden fixtures in this directory from the REFERENCE's own code.

Run where the reference sources are readable, naming their checkout in
VMC_REFERENCE_ROOT (required):

    VMC_REFERENCE_ROOT=<path to sjdu10/vmc_torch> python tests/golden/make_golden.py

The reference is imported under the shims of ``oracle/refshim.py`` (its
third-party TN/MPI dependencies are absent and are not on this path).  Every
array saved here is an output of a reference function, on inputs generated
from fixed seeds; the oracle and the CUDA path are checked against them by
``tests/test_oracle_golden.py`` and the ``-m gpu`` tests.

Fixtures:
  conn.npz      get_conn_batch_gpu on 4x2 (all 4900 sector states) and 8x8
                (48 random half-filled configs), per-walker canonical lists.
  ed_4x2.npz    ED E0 from the reference's to_dense; the shipped Slater
                checkpoints' M[:16] and stored MC energy statistics; the exact
                <H> of each checkpoint under the reference Hamiltonian.
  slater.npz    SlaterDeterminant_GPU amplitudes (4x2, all states), the
                reference sampler replayed on a recorded stream (4x2, 64
                walkers, 3 sweeps), evaluate_energy and compute_grads_gpu.
  nnbf.npz      NNBF_GPU (8x8, 2x256 GELU, bf_scale 0.01; argsort made stable)
                log-amplitudes, a replayed sweep (8 walkers, 1 sweep, log mode),
                evaluate_energy and a column subset + projection of the
                compute_grads_gpu O matrix.
  minsr.npz     minSR_solver_gpu on a seeded (64 x 96) O and energies.
  ckpt_nnbf_4x2.pt / ckpt_slater_4x2.pt (+ _stats.json)
                checkpoints and statistics files written by the reference's
                run-script callback (make_on_step_end) for 4x2 NNBF_GPU and
                SlaterDeterminant_GPU models with 6 walkers
                (``python tests/golden/make_golden.py checkpoints`` rebuilds
                only these).
  sym.npz       FermionSymmetryProjectedModel over SlaterDeterminant_GPU on 4x2
                (C2v) and 4x4 (C4v): permutations, fermionic signs and
                forward_log for the four 1D irreps (``... symmetry`` rebuilds
                only this one).
"""
import hashlib
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import refshim  # noqa: E402
from oracle.lattice import pack, sweep_edges, random_initial_configs  # noqa: E402
from oracle.models import nnbf_init  # noqa: E402

torch.set_default_dtype(torch.float64)


def params_digest(ps):
    h = hashlib.sha256()
    for p in ps:
        h.update(np.ascontiguousarray(p, dtype=np.float64).tobytes())
    return h.hexdigest()


def canonical_conn(etas, coeffs, bids, B):
    """Per walker: sorted (up_bits, dn_bits, coeff) rows, duplicates kept."""
    pk = pack(np.asarray(etas))
    out_pk, out_c, out_b = [], [], []
    bids = np.asarray(bids)
    coeffs = np.asarray(coeffs)
    for b in range(B):
        m = np.nonzero(bids == b)[0]
        key = [(int(pk[k, 0]), int(pk[k, 1]), float(coeffs[k])) for k in m]
        key.sort()
        for (u, d, c) in key:
            out_pk.append((u, d))
            out_c.append(c)
            out_b.append(b)
    return (np.array(out_pk, dtype=np.uint64).reshape(-1, 2), np.array(out_c),
            np.array(out_b, dtype=np.int64))


class Recorder:
    """Feeds the reference sampler a predefined random stream.

    ``propose_exchange_or_hopping_vec`` is wrapped to advance the (sweep,
    edge) position; inside it ``torch.rand`` returns u_move and every
    ``torch.randint`` returns hop_bit; the next ``torch.rand`` before the
    following proposal returns u_acc."""

    def __init__(self, mod, u_move, hop_bit, u_acc, n_edges):
        self.mod, self.E = mod, n_edges
        self.u_move, self.hop_bit, self.u_acc = u_move, hop_bit, u_acc
        self.pos = -1
        self.phase = None

    def __enter__(self):
        self.orig_prop = self.mod.propose_exchange_or_hopping_vec
        self.orig_rand, self.orig_randint = torch.rand, torch.randint
        rec = self

        def prop(i, j, fxs, hr=0.25):
            rec.pos += 1
            rec.phase = "move"
            out = rec.orig_prop(i, j, fxs, hr)
            rec.phase = "acc"
            return out

        def rand(*shape, **kw):
            s, e = divmod(rec.pos, rec.E)
            if rec.phase == "move":
                v = rec.u_move[s, e]
            elif rec.phase == "acc":
                v = rec.u_acc[s, e]
                rec.phase = None
            else:
                raise RuntimeError("unexpected torch.rand call")
            return torch.as_tensor(v.copy(), dtype=torch.float32)

        def randint(lo, hi, shape, **kw):
            s, e = divmod(rec.pos, rec.E)
            return torch.as_tensor(rec.hop_bit[s, e].astype(bool).copy())

        self.mod.propose_exchange_or_hopping_vec = prop
        torch.rand, torch.randint = rand, randint
        return self

    def __exit__(self, *a):
        self.mod.propose_exchange_or_hopping_vec = self.orig_prop
        torch.rand, torch.randint = self.orig_rand, self.orig_randint


def stream(seed, S, E, B):
    g = np.random.default_rng(seed)
    return (g.random((S, E, B), dtype=np.float32), g.integers(0, 2, (S, E, B)).astype(np.uint8),
            g.random((S, E, B), dtype=np.float32))


def main():
    refshim.install()
    ht = refshim.load("vmc_torch.hamiltonian_torch")
    smp = refshim.load("vmc_torch.GPU.sampler")
    vu = refshim.load("vmc_torch.GPU.vmc_utils")
    slater_mod = refshim.load("vmc_torch.GPU.models.slater")
    nnbf_mod = refshim.load("vmc_torch.GPU.models.NNBF")
    optmod = refshim.load("vmc_torch.GPU.optimizer")
    fu = refshim.load("vmc_torch.fermion_utils")

    # ---------------- connected sets ----------------
    H42 = ht.spinful_Fermi_Hubbard_square_lattice_torch(4, 2, 1.0, 8.0, 8, n_fermions_per_spin=(4, 4))
    H42.precompute_hops_gpu("cpu")
    S = np.asarray(H42.hilbert.all_states(), dtype=np.int64)
    e, c, b = H42.get_conn_batch_gpu(torch.as_tensor(S))
    c42 = canonical_conn(e.numpy(), c.numpy(), b.numpy(), len(S))
    H88 = ht.spinful_Fermi_Hubbard_square_lattice_torch(8, 8, 1.0, 8.0, 64, n_fermions_per_spin=(32, 32))
    H88.precompute_hops_gpu("cpu")
    X88 = random_initial_configs(48, 64, 32, 32, seed=11)
    e, c, b = H88.get_conn_batch_gpu(torch.as_tensor(X88))
    c88 = canonical_conn(e.numpy(), c.numpy(), b.numpy(), 48)
    np.savez_compressed(os.path.join(HERE, "conn.npz"),
                        states_4x2=S.astype(np.int8), pk_4x2=c42[0], coeff_4x2=c42[1], bid_4x2=c42[2],
                        x_8x8=X88.astype(np.int8), pk_8x8=c88[0], coeff_8x8=c88[1], bid_8x8=c88[2])
    print("conn.npz", len(c42[1]), len(c88[1]))

    # ---------------- ED + shipped checkpoints ----------------
    Hd = H42.to_dense()
    E0 = float(np.linalg.eigvalsh(Hd)[0])
    ck = os.path.join(refshim.REFERENCE_ROOT,
                      "examples/example_data/4x2/t=1.0_U=8.0/N=8/SlaterDeterminant")
    Ms, mc_mean, mc_err, exact = [], [], [], []
    for step in (1, 26, 50):
        d = torch.load(os.path.join(ck, f"model_params_step{step}.pth"), weights_only=False)
        M = np.asarray(d["model_params_vec"], dtype=np.float64).reshape(4900, 8)[:16]
        Ms.append(M)
        mc_mean.append(float(d["MC_energy_stats"]["mean"]))
        mc_err.append(float(d["MC_energy_stats"]["error"]))
        q2n = fu.from_quimb_config_to_netket_config
        psi = np.array([np.linalg.det(M[np.nonzero(q2n(s))[0]]) for s in S])
        exact.append(float(psi @ Hd @ psi / (psi @ psi)))
    import json
    hist = json.load(open(os.path.join(ck, "energy_stats_start_0.json")))
    np.savez_compressed(os.path.join(HERE, "ed_4x2.npz"), E0=E0, ckpt_steps=np.array([1, 26, 50]),
                        ckpt_M=np.stack(Ms), ckpt_mc_mean=np.array(mc_mean),
                        ckpt_mc_err=np.array(mc_err), ckpt_exact=np.array(exact),
                        hist_json=json.dumps(hist))
    print("ed_4x2.npz E0", E0, "exact", exact)

    # ---------------- Slater 4x2 ----------------
    g = torch.Generator().manual_seed(1234)
    M = torch.randn(16, 8, generator=g, dtype=torch.float64) * 0.1
    model = slater_mod.SlaterDeterminant_GPU(16, 8)
    with torch.no_grad():
        model.params[0].copy_(M)
    amps_all = model(torch.as_tensor(S)).detach().numpy()
    E42 = sweep_edges(4, 2)
    B = 64
    x0 = random_initial_configs(B, 8, 4, 4, seed=5)
    um, hb, ua = stream(77, 3, len(E42), B)
    sampler = smp.MetropolisExchangeSpinfulSamplerGPU()
    graph = H42.graph
    fx = torch.as_tensor(x0.copy())
    with Recorder(smp, um, hb, ua, len(E42)):
        for _ in range(3):
            fx, amps = sampler.step(fx, model, graph)
    x_fin = fx.numpy().copy()
    amps_fin = amps.numpy().copy()
    with torch.inference_mode():
        Em, Eloc = vu.evaluate_energy(fx, model, H42, amps)
    grads, gam = vu.compute_grads_gpu(fx, model, batch_size=32)
    O = (grads / gam.unsqueeze(1)).detach().numpy()
    np.savez_compressed(os.path.join(HERE, "slater.npz"), M=M.numpy(), amps_all=amps_all,
                        x0=x0, u_move=um, hop_bit=hb, u_acc=ua, x_final=x_fin, amps_final=amps_fin,
                        eloc=Eloc.numpy(), O=O)
    print("slater.npz accept-changed", int((x_fin != x0).any(1).sum()))

    # ---------------- NNBF 8x8 ----------------
    orig_argsort = torch.Tensor.argsort

    def stable_argsort(self, dim=-1, descending=False, stable=False):
        return orig_argsort(self, dim=dim, descending=descending, stable=True)

    torch.Tensor.argsort = stable_argsort
    ps = nnbf_init(64, 64, 256, 2, seed=2024)
    nn_model = nnbf_mod.NNBF_GPU(64, 64, hidden_dim=256, n_layers=2, activation="gelu", bf_scale=0.01)
    with torch.no_grad():
        for p, v in zip(nn_model.params, ps):
            p.copy_(torch.as_tensor(v))
    X = random_initial_configs(32, 64, 32, 32, seed=21)
    with torch.inference_mode():
        s_ref, l_ref = nn_model.forward_log(torch.as_tensor(X))
    E88 = sweep_edges(8, 8)
    Bn = 8
    xn0 = X[:Bn].copy()
    umn, hbn, uan = stream(99, 1, len(E88), Bn)
    fx = torch.as_tensor(xn0.copy())
    with Recorder(smp, umn, hbn, uan, len(E88)):
        fx, (sg, la) = sampler.step(fx, nn_model, H88.graph, use_log_amp=True)
    xn_fin = fx.numpy().copy()
    with torch.inference_mode():
        _, Eloc_n = vu.evaluate_energy(fx, nn_model, H88, (sg, la), use_log_amp=True)
    Bg = 4
    gr, (gs, gl) = vu.compute_grads_gpu(fx[:Bg], nn_model, batch_size=Bg, use_log_amp=True)
    gr = gr.detach().numpy()
    cols = np.arange(0, gr.shape[1], 997)
    proj_vec = np.random.default_rng(7).standard_normal(gr.shape[1])
    torch.Tensor.argsort = orig_argsort
    np.savez_compressed(os.path.join(HERE, "nnbf.npz"), params_sha256=params_digest(ps), seed=2024,
                        x=X.astype(np.int8), sign=s_ref.numpy(), logabs=l_ref.numpy(),
                        x0=xn0.astype(np.int8), u_move=umn, hop_bit=hbn, u_acc=uan,
                        x_final=xn_fin.astype(np.int8), sign_final=sg.numpy(), logabs_final=la.numpy(),
                        eloc=Eloc_n.numpy(), O_cols=cols, O_sub=gr[:, cols], O_proj=gr @ proj_vec,
                        proj_seed=7)
    print("nnbf.npz changed walkers", int((xn_fin != xn0).any(1).sum()))

    # ---------------- minSR ----------------
    import torch.distributed as dist
    if not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29533")
        dist.init_process_group("gloo", rank=0, world_size=1)
    rg = np.random.default_rng(3)
    Om = rg.standard_normal((64, 96)) * 0.3
    Ev = rg.standard_normal(64) - 2.0
    dp, _, info = optmod.minSR_solver_gpu(torch.as_tensor(Om), torch.as_tensor(Ev), float(Ev.mean()),
                                          64, 96, diag_shift=1e-4, device=torch.device("cpu"))
    np.savez_compressed(os.path.join(HERE, "minsr.npz"), O=Om, E=Ev, diag_shift=1e-4,
                        dp=np.asarray(dp), info=info)
    dist.destroy_process_group()
    print("minsr.npz info", info)


def make_symmetry():
    """sym.npz: FermionSymmetryProjectedModel (vmc_torch/GPU/models/symmetry.py)
    over a SlaterDeterminant_GPU base (M ~ N(0,1), seed 3) on 4x2 (C2v) and 4x4
    (C4v): site permutations, compute_fermion_signs and forward_log for every
    irrep on 24 configurations (argsort made stable, as for nnbf.npz)."""
    refshim.install()
    sym = refshim.load("vmc_torch.GPU.models.symmetry")
    slater_mod = refshim.load("vmc_torch.GPU.models.slater")
    orig_argsort = torch.Tensor.argsort

    def stable_argsort(self, dim=-1, descending=False, stable=False):
        return orig_argsort(self, dim=dim, descending=descending, stable=True)

    torch.Tensor.argsort = stable_argsort
    out = {}
    for (Lx, Ly, nup) in ((4, 2, 4), (4, 4, 8)):
        N = Lx * Ly
        tag = "%dx%d" % (Lx, Ly)
        M = np.random.default_rng(3).standard_normal((2 * N, 2 * nup))
        m = slater_mod.SlaterDeterminant_GPU(2 * N, 2 * nup)
        with torch.no_grad():
            m.params[0].copy_(torch.as_tensor(M))
        X = random_initial_configs(24, N, nup, nup, seed=2)
        perms, chars, _ = sym.build_symmetry_group(Lx, Ly)
        out[tag + "_M"] = M
        out[tag + "_x"] = X.astype(np.int8)
        out[tag + "_perms"] = perms.numpy()
        for irrep in ("A1", "A2", "B1", "B2"):
            pm = sym.FermionSymmetryProjectedModel(m, Lx, Ly, irrep=irrep)
            with torch.no_grad():
                sg, la = pm.forward_log(torch.as_tensor(X))
            out[tag + "_" + irrep + "_chars"] = np.asarray(chars[irrep], dtype=np.float64)
            out[tag + "_" + irrep + "_sign"] = sg.numpy()
            out[tag + "_" + irrep + "_logabs"] = la.numpy()
            if irrep == "A1":
                out[tag + "_fsign"] = sym.compute_fermion_signs(torch.as_tensor(X), pm.mode_inv_masks).numpy()
    torch.Tensor.argsort = orig_argsort
    np.savez_compressed(os.path.join(HERE, "sym.npz"), **out)
    print("sym.npz written")


def make_checkpoints():
    """ckpt_*.pt: checkpoints written by the reference's own run-script
    callback (vmc_torch/GPU/run_scripts/vmcconfig.py:185-213) for a 4x2 NNBF_GPU
    (parameters nnbf_init(8, 8, 256, 2, seed=5)) and a 4x2
    SlaterDeterminant_GPU (M = N(0,1) from seed 8), each with 6 walkers."""
    import shutil
    import tempfile
    refshim.install()
    vc = refshim.load("vmc_torch.GPU.run_scripts.vmcconfig")
    nnbf_mod = refshim.load("vmc_torch.GPU.models.NNBF")
    slater_mod = refshim.load("vmc_torch.GPU.models.slater")
    nn_model = nnbf_mod.NNBF_GPU(8, 8, hidden_dim=256, n_layers=2, activation="gelu", bf_scale=0.01)
    with torch.no_grad():
        for p, v in zip(nn_model.params, nnbf_init(8, 8, 256, 2, seed=5)):
            p.copy_(torch.as_tensor(v))
    sl_model = slater_mod.SlaterDeterminant_GPU(16, 8)
    with torch.no_grad():
        sl_model.params[0].copy_(torch.as_tensor(np.random.default_rng(8).standard_normal((16, 8))))
    fxs = torch.as_tensor(random_initial_configs(6, 8, 4, 4, seed=6))
    for name, m in (("NNBF", nn_model), ("Slater", sl_model)):
        with tempfile.TemporaryDirectory() as d:
            n_params = sum(p.numel() for p in m.parameters())
            stats = vc.make_stats("4x2 t=1 U=8 N=8", n_params, 6, 1)
            sf = vc.make_stats_file(d, name, 0)
            cb = vc.make_on_step_end(0, stats, sf, d, name, m, 1)
            cb({"step": 0, "energy_per_site": -0.25, "error_per_site": 0.01, "energy_var": 0.5, "fxs": fxs})
            shutil.copy(os.path.join(d, f"checkpoint_{name}_1.pt"), os.path.join(HERE, f"ckpt_{name.lower()}_4x2.pt"))
            shutil.copy(sf, os.path.join(HERE, f"ckpt_{name.lower()}_4x2_stats.json"))
    print("checkpoints written")


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "checkpoints":
        make_checkpoints()
    elif len(sys.argv) > 1 and sys.argv[1] == "symmetry":
        make_symmetry()
    else:
        main()
        make_checkpoints()
        make_symmetry()
