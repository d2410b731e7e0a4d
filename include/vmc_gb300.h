/*
 * vmc_gb300.h — C ABI of the GB300 VMC inner-loop library (libvmc_gb300.so).
 *
 * Every entry point takes raw device pointers, sizes and a cudaStream_t (passed
 * as void*), enqueues work on that stream and returns a status code; it never
 * allocates or frees caller memory.  Two calls synchronise the stream and say
 * so below: vmc_nnbf_sweep with stage timing, and vmc_check_finite with host
 * counts.  Host wrappers turn status codes into the reference's exceptions.
 *
 * Walker layout: occ[2*w] = up bits, occ[2*w+1] = down bits (site i -> bit i,
 * n_sites <= 64).  Configurations at the API boundary use the reference's
 * quimb encoding {0: empty, 1: down, 2: up, 3: up+down} as int64 (B, n_sites).
 *
 * Reference interfaces replaced (paths within sjdu10/vmc_torch):
 *   vmc_pack / vmc_unpack        — quimb <-> netket conversion,
 *                                  vmc_torch/fermion_utils.py:1448-1498 and the
 *                                  inline form in vmc_torch/GPU/models/slater.py:53-56
 *   vmc_init_walkers             — random_initial_config, vmc_torch/GPU/vmc_utils.py:22-39;
 *                                  initialize_walkers, vmc_torch/GPU/vmc_setup.py:139-159
 *   vmc_hubbard_conn             — SpinfulFermionGPUMixin.get_conn_batch_gpu,
 *                                  vmc_torch/hamiltonian_torch.py:586-655
 *   vmc_slater_refresh           — SlaterDeterminant_GPU.amplitude / forward_log,
 *                                  vmc_torch/GPU/models/slater.py:40-61, _base.py:101-130
 *   vmc_slater_sweep             — MetropolisExchangeSpinfulSamplerGPU.step,
 *                                  vmc_torch/GPU/sampler.py:217-388 (+ proposals 47-137)
 *   vmc_slater_local_energy      — _evaluate_energy_impl, vmc_torch/GPU/vmc_utils.py:322-476
 *   vmc_slater_logpsi_grad       — compute_grads_gpu, vmc_torch/GPU/vmc_utils.py:1389-1634
 *   vmc_sr_*                     — minSR_solver_gpu, vmc_torch/GPU/optimizer.py:471-614
 *   vmc_check_finite             — _check_grads_amps, vmc_torch/GPU/vmc_utils.py:1330-1386
 *   vmc_energy_gradient          — the run_sr=False branch, vmc_torch/GPU/optimizer.py:585-613
 *   vmc_peps_eval / _sweep /     — fPEPS_Model_GPU.amplitude / log_amplitude,
 *   _local_energy                  vmc_torch/GPU/models/pureTNS.py:82-146, driven by
 *                                  the same sampler and energy loop as the other models
 *                                  (exact contraction: max_bond absent or large)
 *   vmc_peps_chi_*               — the same with the boundaries truncated to max_bond
 *                                  (contract_boundary_from_xmin_/xmax_ with max_bond = chi,
 *                                  pureTNS.py:100-111), and its log-derivatives
 *   vmc_split_bf16x3 /           — the Gram matrix lpg_scaled @ lpg_scaled.T of
 *   vmc_sr_gram_tc                 minSR_solver_gpu (vmc_torch/GPU/optimizer.py:551-553)
 *                                  on the tensor cores
 *   vmc_sym_*                    — FermionSymmetryProjectedModel,
 *                                  vmc_torch/GPU/models/symmetry.py:673-1136
 *   vmc_propose_edge / _accept_edge, vmc_conn_rows, vmc_eloc_*
 *                                — the sampler and energy steps for a wrapped model
 *                                  (vmc_torch/GPU/sampler.py:217-388, vmc_utils.py:322-476)
 */
#ifndef VMC_GB300_H
#define VMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum vmc_status {
  VMC_OK = 0,
  VMC_ERR_ARGS = 1,        /* invalid sizes / null pointers / unsupported shape */
  VMC_ERR_CUDA = 2,        /* a launch failed */
  VMC_ERR_NONFINITE = 3,   /* non-finite amplitude or energy */
  VMC_ERR_SINGULAR = 4,    /* singular orbital matrix */
  VMC_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  VMC_ERR_UNSUPPORTED = 6, /* configuration not built into this library */
  VMC_ERR_CAPACITY = 7     /* request larger than a fixed built-in capacity */
};

int vmc_abi_version(void);

/* ---- walkers and the Hubbard connected set ---- */
/* fxs (B, n_sites) int64 quimb -> occ (B, 2) uint64.  *d_bad (device int) is set
 * to 1 when a value is outside {0,1,2,3}. */
int vmc_pack(const int64_t* fxs, int64_t B, int n_sites, uint64_t* occ, int* d_bad, void* stream);
int vmc_unpack(const uint64_t* occ, int64_t B, int n_sites, int64_t* fxs, void* stream);
/* Seeded uniform random sector states (n_up up, n_dn down electrons). */
int vmc_init_walkers(uint64_t* occ, int64_t B, int n_sites, int n_up, int n_dn, uint64_t seed, void* stream);
/* Connected set, T = 2*n_edges + n_sites slots per walker: for each edge (order
 * of `edges`, int32 [n_edges][2]) spin up then spin down, then one on-site slot
 * per site.  eta (B, T, 2) uint64, coeff (B, T) float64, valid (B, T) uint8. */
int vmc_hubbard_conn(const uint64_t* occ, int64_t B, int n_sites, const int32_t* edges, int n_edges, double t,
                     double U, uint64_t* eta, double* coeff, uint8_t* valid, void* stream);

/* ---- Slater determinant (FP64): psi(x) = det(M[ascending occupied rows]) ----
 * M (n_orb = 2*n_sites, nf) row-major float64.  Per-walker state: G (B, nf, nf)
 * float64 with G[k][c] = (A^-1)[c][k]; slot_orb (B, nf) uint8; sign, logabs (B)
 * float64; n_acc (B) int32 accepted moves since the last re-inversion. */
int vmc_slater_refresh(const double* M, int n_orb, int nf, const uint64_t* occ, int64_t B, int n_sites, double* G,
                       uint8_t* slot_orb, double* sign, double* logabs, int32_t* n_acc, int threshold,
                       int* d_n_singular, void* stream);
/* n_sweeps sweeps over `edges` (sweep order).  Random stream: replay buffers
 * r_move/r_bit/r_acc of shape (n_sweeps, n_edges, B) when non-null, else
 * Philox4x32-10 keyed by seed with counter (walker, sweep_offset + s, edge). */
int vmc_slater_sweep(const double* M, int n_orb, int nf, uint64_t* occ, int64_t B, int n_sites, const int32_t* edges,
                     int n_edges, int n_sweeps, float hopping_rate, uint64_t seed, uint64_t sweep_offset,
                     const float* r_move, const uint8_t* r_bit, const float* r_acc, double* G, uint8_t* slot_orb,
                     double* sign, double* logabs, int32_t* n_acc, void* stream);
int vmc_slater_local_energy(const double* M, int n_orb, int nf, const uint64_t* occ, int64_t B, int n_sites,
                            const int32_t* edges, int n_edges, double t, double U, const double* G,
                            const uint8_t* slot_orb, double* eloc, void* stream);
/* O (B, ldo) float64, O[w][o*nf + c] = d log|psi| / d M[o][c]. */
int vmc_slater_logpsi_grad(const double* G, const uint8_t* slot_orb, int64_t B, int n_orb, int nf, double* O,
                           int64_t ldo, void* stream);

/* ---- Neural-network backflow (NNBF_GPU, vmc_torch/GPU/models/NNBF.py:36-162) ----
 * psi(x) = det((M_base + s * (out_w h2(x) + out_b))[ascending occupied rows]),
 * h2 = gelu(W1 gelu(W0 n + b0) + b1), hidden width 256, two hidden layers.
 * prec 0 ("mixed"): BF16 tensor-core GEMMs (tcgen05, FP32 accumulate), FP32 LU,
 *   log|det| combined in FP64; requires nf in {32, 64} and 2*n_sites*nf % 256 == 0.
 * prec 1 ("fp64"): every stage in FP64 on CUDA cores (parity mode).
 * net_ptrs[7] (device pointers), prec 0 / prec 1 element types:
 *   [0] W0^T (2N, 256) f32/f64   [1] b0 (256) f32/f64   [2] W1 (256, 256) bf16/f64
 *   [3] b1 (256) f32/f64          [4] out_w (2N*nf, 256) bf16/f64
 *   [5] out_b (2N*nf) f32/f64     [6] M_base (2N, nf) f32/f64
 * Workspace for R rows (caller-owned): H1, H2 (R, 256) bf16/f64; A (R, nf, nf) f32/f64.
 * The workspace is scratch: its contents on return are unspecified (the LU
 * reuses consumed orbital-matrix rows).
 * d_err (device int) receives VMC_ERR_TIMEOUT if a bounded device wait gave up,
 * and VMC_ERR_ARGS if a configuration evaluated from scratch has an occupation
 * bit at or above n_sites or other than nf electrons (its result is then
 * meaningless; bits above n_sites are ignored, never used as indices).
 * Streams: work is enqueued on `stream`; for R > 4096 (mixed precision) the
 * call may fork part of it onto library-owned streams (one high-priority stream
 * for the next chunk's backflow GEMM, up to four for independent walker groups),
 * created once per device and shared by all callers, and joins them back into
 * `stream` by events before it returns, on error paths too.  Calls issued
 * concurrently from several host threads therefore share those streams.
 * Environment: VMC_GB300_SERIAL_CHUNKS=1 / VMC_GB300_SWEEP_LANES=1 keep all
 * work on `stream`.
 * Amplitude results: a singular orbital matrix gives sign 0 and logabs -inf; a
 * NaN or Inf entry (non-finite parameters) gives NaN for both, as the
 * reference's NaN amplitude.  Metropolis tests never accept a NaN ratio; from a
 * zero-amplitude walker every non-zero proposal is accepted. */
/* Evaluate R configurations from scratch: sign/logabs (R), and z0 = W0 n + b0
 * (R, 256) f32/f64 when z0_out is non-null.  Replaces forward_log / vamp_log
 * (vmc_torch/GPU/models/_base.py:101-130). */
int vmc_nnbf_eval(int prec, const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale,
                  const uint64_t* occ, int64_t R, void* z0_out, void* H1, void* H2, void* A, double* sign,
                  double* logabs, int* d_err, void* stream);
/* Metropolis sweeps (MetropolisExchangeSpinfulSamplerGPU.step,
 * vmc_torch/GPU/sampler.py:217-388): per edge, propose for all B walkers,
 * evaluate every proposal, accept with min(1, |psi'|^2/|psi|^2).  Walker state
 * occ, z0 (B, 256), sign, logabs, n_acc is updated in place.  Workspace:
 * prop_occ (B, 2) u64, rec (B, 16 bytes), H1/H2/A for B rows.  Random stream as
 * in vmc_slater_sweep.  Optional instrumentation (all nullable): d_n_eval (device
 * u64) counts evaluated proposals; stage_ms[4] / stage_launches[4] (HOST arrays)
 * accumulate the device time of the [prep, hidden layer, backflow GEMM, LU]
 * launches, measured with CUDA events on `stream` (the call then synchronises
 * the stream before returning).  compact_ws (nullable, 16-byte aligned,
 * 256 + 4 B rounded up to 16 + 16 B bytes): with it, mixed precision and 64
 * orbitals, each edge's GEMMs and LU run over the walkers whose proposal
 * changes them only (compacted on the device; results identical). */
int vmc_nnbf_sweep(int prec, const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale,
                   uint64_t* occ, int64_t B, const int32_t* edges, int n_edges, int n_sweeps, float hopping_rate,
                   uint64_t seed, uint64_t sweep_offset, const float* r_move, const uint8_t* r_bit, const float* r_acc,
                   void* z0, double* sign, double* logabs, int32_t* n_acc, uint64_t* prop_occ, void* rec, void* H1,
                   void* H2, void* A, int* d_err, unsigned long long* d_n_eval, float* stage_ms, int* stage_launches,
                   void* compact_ws, void* stream);
/* Local-energy support (vmc_torch/GPU/vmc_utils.py:322-476): per-walker count
 * of valid hop terms, then the (walker, hop-term) pair list at offsets offs
 * (B+1, exclusive scan of the counts).  Hop term = 2*edge + (0 up, 1 down). */
int vmc_nnbf_conn_count(const uint64_t* occ, int64_t B, int n_sites, const int32_t* edges, int n_edges, int32_t* cnt,
                        void* stream);
int vmc_nnbf_conn_pairs(const uint64_t* occ, int64_t B, int n_sites, const int32_t* edges, int n_edges,
                        const int32_t* offs, int32_t* pairs, void* stream);
/* E_loc(x) = U * doublons + sum_pairs H_{x,eta} psi(eta)/psi(x), evaluating
 * `chunk` connected configurations at a time with workspace row_occ (chunk, 2),
 * coeff (chunk), H1/H2/A for chunk rows; term (P) holds the per-pair terms. */
int vmc_nnbf_local_energy(int prec, const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale,
                          const uint64_t* occ, int64_t B, const int32_t* edges, double t, double U, const void* z0,
                          const double* sign, const double* logabs, const int32_t* pairs, const int32_t* offs,
                          int64_t P, int64_t chunk, uint64_t* row_occ, double* coeff, double* term, void* H1, void* H2,
                          void* A, double* eloc, int* d_err, void* stream);

/* Per-sample log-derivatives O = d log|psi| / d theta of the NNBF model
 * (compute_grads_gpu, vmc_torch/GPU/vmc_utils.py:1389-1634, which the reference
 * obtains with torch.func.grad): hand-written adjoint, forward activations
 * recomputed, A^-1 by Gauss-Jordan.  prec 0: FP32, prec 1: FP64 (all arrays of
 * that type).  gnet[9]: W0^T (2N,256), b0, W1 (256,256), W1^T, b1,
 * out_w (2N*nf,256), out_w^T (256,2N*nf), out_b, M_base (2N,nf).
 * Outputs (each nullable): O_full (B, ld_full >= Np) rows in the reference
 * parameter order; O_dense (B, ld_dense >= Np - 2N*nf*256) the same rows without
 * the out_w block; kron_g (B, 2N*nf) = s * Gbar and kron_h (B, 256) = h2, whose
 * outer product is the out_w block; logabs/sign (B). */
int vmc_nnbf_logpsi_grad(int prec, const void* const* gnet, int n_sites, int nf, int hidden, double bf_scale,
                         const uint64_t* occ, int64_t B, void* O_full, int64_t ld_full, void* O_dense,
                         int64_t ld_dense, void* kron_g, void* kron_h, double* logabs, double* sign, void* stream);

/* ---- Learned Metropolis-Hastings proposal (no reference counterpart: the
 * reference samples with local exchange/hop moves only, vmc_torch/GPU/sampler.py:47-137).
 * Network 2N -> 512 -> 512 -> 256 logits (GELU): logits[0, 2E) one per hop
 * (edge e of `edges`, index 2e up / 2e+1 down), logits[2E, 2E+4) k = 1..4.
 * rec: 48-byte record per walker {flag, k, u_acc, logq_fwd, hop[4], logq_rev}. */
/* wts[6]: W1 (512, Kin) bf16, b1 (512) f32, W2 (512, 512) bf16, b2 f32, Wo (256, 512)
 * bf16, bo (256) f32; Kin = 2N rounded up to 64.  Workspace X (R, Kin), H1, H2
 * (R, 512) bf16.  Output logits (R, 256) f32 (tcgen05 BF16 GEMMs). */
int vmc_prop_logits(const void* const* wts, int n_sites, const uint64_t* occ, int64_t R, void* X, void* H1, void* H2,
                    float* logits, int* d_err, void* stream);
/* Draw k and k non-conflicting valid hops per walker; prop_occ, rec (flag, k,
 * u_acc, hops, log q(x->x') by a DP over the 2^k orderings). */
int vmc_prop_sample(const int32_t* edges, int n_edges, int n_sites, const float* logits, const uint64_t* occ,
                    int64_t B, uint64_t seed, uint64_t step, uint64_t* prop_occ, void* rec, void* stream);
/* log q(x'->x) from the logits at the proposed configurations. */
int vmc_prop_reverse(const int32_t* edges, int n_edges, int n_sites, const float* logits_p, const uint64_t* prop_occ,
                     int64_t B, void* rec, void* stream);
/* MH accept of learned proposals for the mixed NNBF model: psi(x') evaluated with
 * its first layer z0p = z0 + the W0 columns of the orbitals the proposal changes
 * (z0: the walkers' first layer, as left by vmc_nnbf_eval; z0p workspace, copied
 * into z0 on acceptance), accept with min(1, |psi'/psi|^2 q(x'->x)/q(x->x')).
 * Optional: lg_x (B, 256) proposal logits at x, overwritten with lg_p's row when a
 * walker moves (so the next move needs only the logits at its new proposal);
 * kstats[8] device counters of proposals / acceptances by k. */
int vmc_nnbf_mh_step(const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale, uint64_t* occ,
                     int64_t B, const uint64_t* prop_occ, const void* rec4, void* z0, void* z0p, double* sign,
                     double* logabs, int32_t* n_acc, void* H1, void* H2, void* A, float* lg_x, const float* lg_p,
                     int* kstats, int* d_err, void* stream);
/* MH accept of learned proposals for any model (the proposals' sign_p /
 * logabs_p (B) come from the caller's own evaluation of prop_occ): accept with
 * min(1, |psi'/psi|^2 q(x'->x)/q(x->x')), a NaN ratio never; on accept the
 * walker takes x', sign, logabs and (lg_x / lg_p, both or neither) the
 * proposal logits at x'.  n_acc (B) and kstats[8] are nullable counters. */
int vmc_accept_mh(uint64_t* occ, int64_t B, const uint64_t* prop_occ, const void* rec4, const double* sign_p,
                  const double* logabs_p, double* sign, double* logabs, int32_t* n_acc, float* lg_x,
                  const float* lg_p, int* kstats, void* stream);
/* Training (FP32 CUDA cores): forward, masked softmax cross entropy against the
 * heat-bath hop targets tgt (R, 2E) and the k target ktgt (4), backward, Adam.
 * params/grad/m1/m2: flat FP32 [W1, b1, W2, b2, Wo, bo]; ws: R*(4*512+2*256) f32;
 * loss (R) per-row loss; grad holds this step's gradient on return. */
int vmc_prop_train_step(int n_sites, const int32_t* edges, int n_edges, const uint64_t* occ, int R, const float* Xf,
                        const float* tgt, const float* ktgt, float kweight, float* params, float* grad, float* m1,
                        float* m2, int64_t n_params, float lr, float beta1, float beta2, float eps, int t, float* ws,
                        float* loss, void* stream);
int vmc_prop_inputs_f32(int n_sites, const uint64_t* occ, int64_t R, float* Xf, void* stream);
/* tgt[row0 + w][hop] = (term / t)^2 = |psi(x_hop)/psi(x)|^2 from the local-energy pairs. */
int vmc_prop_collect_targets(const int32_t* pairs, int64_t P, const double* term, double t_abs, int n_hops,
                             int64_t row0, float* tgt, void* stream);

/* Second network layer on the tensor cores: H2 = gelu(H1 W1^T + b1), H1 (R, 256)
 * and W1 (256, 256) BF16, b1 (256) FP32, H2 (R, 256) BF16 (the stage the NNBF
 * entry points run internally; no reference counterpart as an operator of its
 * own, it is the second layer of NNBF_GPU, vmc_torch/GPU/models/NNBF.py:113-162).
 * wait_limit_ns bounds the kernel's wait for its operand tiles (0: 1 s).
 * skip_loads = 1 issues no tile load, so that the wait runs out with nothing in
 * flight: d_err then receives VMC_ERR_TIMEOUT, H2 is left untouched and the
 * context stays usable (the self-test of the bounded-wait path). */
int vmc_nnbf_hidden_layer(const void* H1, int64_t R, const void* W1, const float* b1, void* H2,
                          uint64_t wait_limit_ns, int skip_loads, int* d_err, void* stream);

/* Allocation-free variant of vmc_nnbf_eval (mixed precision only, no z0 output).
 * This entry point has no counterpart in the reference.  It is for callers that
 * cannot allocate device memory while they run (a fixed device-memory budget
 * set up once, a real-time loop, or a framework that owns the whole device
 * pool): it takes no workspace and allocates nothing; its scratch is a fixed
 * 8.5 MiB array inside the library, held by every GPU that loads the library
 * until the process exits.  At most 512 configurations per call (nf <= 64);
 * larger R returns VMC_ERR_CAPACITY.  With CUDA's lazy module loading (the
 * default) the array is committed on a device only when the library's module is
 * first loaded there: the first call on each device does that, resolves the
 * array's device address (cudaGetSymbolAddress) and sets the kernels'
 * shared-memory attributes.  A caller that may not allocate later makes one
 * warm-up call on each device first, before any no-allocation region and
 * before any stream capture.  All calls share the one array: calls whose work overlaps on
 * the GPU (different streams, or different host threads) race on it and must
 * be serialised by the caller. */
int vmc_nnbf_eval_noalloc(const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale,
                          const uint64_t* occ, int64_t R, double* sign, double* logabs, int* d_err, void* stream);

/* ---- non-finite and zero-amplitude detection (_check_grads_amps,
 * vmc_torch/GPU/vmc_utils.py:1330-1386) ----
 * Counts into d_counts (4 device u64, cleared by the call): [0] NaN and [1] Inf
 * entries of amp (B, nullable), [2] zero entries of sign (B, nullable), [3] rows
 * of O (B, Np, leading dim ldo, dtype 0 f64 / 1 f32, nullable) holding a NaN or
 * Inf.  d_row_bad (B) / d_col_bad (Np) flag those rows and columns (nullable).
 * With h_counts (host, 4) non-null the call copies the counts there,
 * synchronises the stream and returns VMC_ERR_NONFINITE if anything is NaN or
 * Inf, else VMC_ERR_SINGULAR if some amplitude is zero, else VMC_OK; with
 * h_counts null it only enqueues the work and returns VMC_OK. */
int vmc_check_finite(const double* amp, const double* sign, int64_t B, const void* O, int dtype, int64_t Np,
                     int64_t ldo, unsigned long long* d_counts, uint8_t* d_row_bad, uint8_t* d_col_bad,
                     unsigned long long* h_counts, void* stream);

/* ---- minSR in sample space (dtype: 0 = float64, 1 = float32 for O / Oc) ---- */
int vmc_sr_center(const void* O, int dtype, int64_t Ns, int64_t Np, int64_t ldo, void* Oc, int64_t ldc, double* mean,
                  void* stream);
int vmc_sr_gram(const void* Oc, int dtype, int64_t Ns, int64_t Np, int64_t ldc, double* T, int64_t ldt,
                double diag_shift, int accumulate, void* stream);
/* vmc_sr_cholesky: T = L L^T in place (lower), blocked right-looking with 64-column
 *   panels; tile factorisations and panel solves in FP64, trailing updates in
 *   double-float arithmetic on the FP32 pipes (~2^-46 relative per product sum).
 *   *d_info is set to 1 when a pivot is not positive or not finite (the caller
 *   zeroes it first); the factor is then not usable. */
int vmc_sr_cholesky(double* T, int64_t n, int64_t ldt, int* d_info, void* stream);
/* Tensor-core Gram for FP32 inputs (no reference counterpart as an operator:
 * the reference forms lpg_scaled @ lpg_scaled.T in FP64, vmc_torch/GPU/optimizer.py:551-553).
 * vmc_split_bf16x3: X (rows, K, ld ldx) FP32 -> row_exp (rows_pad ints, device):
 *   E_r with max |X[r]| < 2^E_r, and three BF16 planes hi, mid, lo holding the
 *   7-bit integer digits of x 2^-E_r times 2^-6, 2^-13, 2^-20 (to 2^-21 of the
 *   row's largest entry), each (rows_pad, kp) row-major, rows_pad a multiple
 *   of 128 >= rows, kp a multiple of 64 >= K, padding zeroed; planes holds
 *   3 * rows_pad * kp bf16.
 * vmc_sr_gram_tc: T (ns, ns, FP64, ld ldt) = [T +] alpha (X X^T) o D [+ shift I]
 *   with D (nullable, ld ldt) elementwise and `accumulate` selecting "+=";
 *   all nine digit products per element pair on tcgen05: the leading one summed
 *   exactly in FP32 (integer multiples of 2^-12, < 2^23 units per 2048
 *   columns), the others in a second FP32 accumulator; drained into FP64 every
 *   2048 columns and scaled by 2^(E_i + E_j); the full symmetric T is written.
 *   d_err (device int) receives VMC_ERR_TIMEOUT if a bounded wait gave up. */
int vmc_split_bf16x3(const float* X, int64_t rows, int64_t K, int64_t ldx, void* planes, int64_t rows_pad,
                     int64_t kp, int* row_exp, void* stream);
int vmc_sr_gram_tc(const void* planes, const int* row_exp, int64_t ns, int64_t rows_pad, int64_t kp, double alpha,
                   double* T, int64_t ldt, const double* D, double diag_shift, int accumulate, int* d_err,
                   void* stream);
int vmc_sr_cholesky_solve(const double* L, int64_t n, int64_t ldt, double* b, void* stream);
int vmc_sr_rhs(const double* E, int64_t Ns, double Ebar, double* b, void* stream);
int vmc_sr_update(const void* Oc, int dtype, int64_t Ns, int64_t Np, int64_t ldc, const double* x, double* dp,
                  void* stream);
int vmc_energy_gradient(const void* O, int dtype, int64_t Ns, int64_t Np, int64_t ldo, const double* E, double Ebar,
                        double* g, void* stream);
/* Factored (Kronecker) SR pieces for the NNBF output layer, whose O block is
 * g_a (x) h_a per sample (no reference counterpart: the reference materialises
 * the full O, vmc_torch/GPU/optimizer.py:545-563).
 * vmc_gemm: C = beta C + alpha op(A) op(B) [* D elementwise], row-major storage,
 *   ta/tb = 1 transposes A (K x M storage) / B (N x K storage); sk (length K,
 *   nullable) scales op(A)'s columns; dtype of A, B, sk: 0 f64, 1 f32; C, D f64;
 *   lower = 1 computes the lower tile triangle of a symmetric result and mirrors it.
 * vmc_sr_kron_correction: v[a] = P[a] . H[a]; T[a][b] += alpha (mu_sq - v[a] - v[b]). */
int vmc_gemm(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const void* A, int64_t lda, const void* B,
             int64_t ldb, const void* sk, int dtype, double beta, double* C, int64_t ldc, const double* D,
             int64_t ldd, int lower, void* stream);
int vmc_sr_kron_correction(int64_t n, double* T, int64_t ldt, const double* P, int64_t ldp, const void* H, int dtype,
                           int64_t ldh, int64_t K, double mu_sq, double alpha, double* v_work, void* stream);

/* ---- Fermionic PEPS (fPEPS_Model_GPU, vmc_torch/GPU/models/pureTNS.py:24-160) ----
 * tensors (Lx, Ly, 4, D, D, D, D) = [row][col][quimb state][left][up][right][down],
 * float32 (prec 0) or float64 (prec 1); Z2-graded (bond parity = index & 1, every
 * tensor even), open legs at index 0.  Sites i = row * Ly + col.  psi(x) is the
 * Grassmann contraction with bond variables ordered (left, up, down, right)
 * within a site, computed exactly (the max_bond -> infinity limit of the
 * reference's boundary contraction, pureTNS.py:103-114): top and bottom
 * boundary MPSs of bond D^(Lx/2-1) and a column sweep through the two middle
 * rows.  Supported: Lx in {4, 6, 8} even, D in {2, 4}, D^(Lx/2-1) <= 16,
 * Lx * Ly <= 64 (else VMC_ERR_UNSUPPORTED).  Zero amplitudes give sign 0 and
 * logabs -inf.
 * vmc_peps_eval         — forward_log of R configurations.
 * vmc_peps_sweep        — Metropolis sweeps as vmc_slater_sweep (same proposal,
 *                         random stream and acceptance); n_acc (B, nullable)
 *                         accumulates accepted moves, d_n_eval (nullable device
 *                         u64[2]) accumulates evaluated proposals and column
 *                         steps executed.
 * vmc_peps_local_energy — E_loc with pairs/offs from vmc_nnbf_conn_count/pairs;
 *                         term (P, nullable with env_work) receives the
 *                         per-pair hop terms.
 *   env_work (nullable): work_rows * 2 * (Ly+1) * D^(Lx-2) * D^2 elements of the
 *   tensors' dtype for cached left/right column environments (the role of the
 *   reference's bMPS environment reuse, pureTNS.py:163-2375): a move on a
 *   horizontal pair then costs two column steps and on a vertical pair one,
 *   instead of Ly; edges must be nearest-neighbour pairs (else *d_err, device
 *   int, nullable, = VMC_ERR_UNSUPPORTED).  NULL recomputes every proposal from
 *   scratch (sign/logabs are then required by the local energy).
 * vmc_peps_logpsi_grad  — O (B, ldo >= Lx*Ly*4*D^4, dtype of prec) =
 *                         d log|psi| / d tensors in the flattened tensor order
 *                         (zero except at each site's occupied state), by a
 *                         reverse column sweep over stored left environments;
 *                         work holds work_rows * (Ly+1) * D^(Lx-2) * D^2
 *                         elements of that dtype; Lx in {4, 6}. */
int vmc_peps_eval(int prec, const void* tensors, int Lx, int Ly, int D, const uint64_t* occ, int64_t R, double* sign,
                  double* logabs, void* stream);
int vmc_peps_sweep(int prec, const void* tensors, int Lx, int Ly, int D, uint64_t* occ, int64_t B,
                   const int32_t* edges, int n_edges, int n_sweeps, float hopping_rate, uint64_t seed,
                   uint64_t sweep_offset, const float* r_move, const uint8_t* r_bit, const float* r_acc, double* sign,
                   double* logabs, int32_t* n_acc, uint64_t* d_n_eval, void* env_work, int64_t work_rows, int* d_err,
                   void* stream);
int vmc_peps_local_energy(int prec, const void* tensors, int Lx, int Ly, int D, const uint64_t* occ, int64_t B,
                          const int32_t* edges, double t, double U, const double* sign, const double* logabs,
                          const int32_t* pairs, const int32_t* offs, int64_t P, double* term, double* eloc,
                          void* env_work, int64_t work_rows, int* d_err, void* stream);
int vmc_peps_logpsi_grad(int prec, const void* tensors, int Lx, int Ly, int D, const uint64_t* occ, int64_t B,
                         void* O, int64_t ldo, void* work, int64_t work_rows, void* stream);

/* ---- fPEPS with the reference's chi-truncated boundary contraction
 * (fPEPS_Model_GPU.amplitude / log_amplitude, vmc_torch/GPU/models/pureTNS.py:81-146:
 * contract_boundary_from_xmin_ over rows [0, Lx/2-1] and _from_xmax_ over
 * [Lx/2, Lx-1] with max_bond = chi, cutoff 0, then the two boundaries contracted).
 * Same tensors, sign convention and (sign, logabs) semantics as vmc_peps_*.
 * Each side's boundary is kept as the full vector over its D^Ly open legs; a row
 * is absorbed exactly and the compression after it (left-to-right QR, right-to-left
 * truncated SVD) is applied as the best rank-chi truncations across cuts
 * Ly-1, ..., 1 that static rank bounds cannot rule out (Gram matrix of the smaller
 * side, Z2 parity blocks, Jacobi eigenvectors).  Supported: Lx even >= 2,
 * D in {2, 4}, D^Ly <= 4096, Lx * Ly <= 64, chi >= 1 (else VMC_ERR_UNSUPPORTED).
 * work: *bytes from vmc_peps_chi_work_bytes(prec, Lx, Ly, D, chi, work_rows, bytes)
 * of device memory (256-byte aligned) for chunks of work_rows walkers (or hop
 * terms).
 * vmc_peps_chi_schedule     — cuts[a] (a < Lx/2): bit k set when cut k (after k
 *                             columns) is truncated after the a-th absorbed row of
 *                             a side; all zero means the contraction is exact.
 * vmc_peps_chi_eval         — forward_log of R configurations.
 * vmc_peps_chi_sweep        — Metropolis sweeps with the proposals, random stream
 *                             and acceptance of vmc_peps_sweep; per edge every
 *                             walker's proposal rebuilds only the touched sides.
 *                             sign/logabs are recomputed for the walkers first.
 *                             d_n_eval (nullable) += evaluated proposals, side
 *                             states built.
 * vmc_peps_chi_local_energy — E_loc with pairs/offs from vmc_nnbf_conn_count/pairs;
 *                             offs_host is a host copy of offs (B + 1 entries);
 *                             term (P) receives the hop terms. */
int vmc_peps_chi_work_bytes(int prec, int Lx, int Ly, int D, int chi, int64_t work_rows, int64_t* bytes);
int vmc_peps_chi_schedule(int Lx, int Ly, int D, int chi, uint32_t* cuts, int max_rows);
int vmc_peps_chi_eval(int prec, const void* tensors, int Lx, int Ly, int D, int chi, const uint64_t* occ, int64_t R,
                      double* sign, double* logabs, void* work, int64_t work_rows, void* stream);
int vmc_peps_chi_sweep(int prec, const void* tensors, int Lx, int Ly, int D, int chi, uint64_t* occ, int64_t B,
                       const int32_t* edges, int n_edges, int n_sweeps, float hopping_rate, uint64_t seed,
                       uint64_t sweep_offset, const float* r_move, const uint8_t* r_bit, const float* r_acc,
                       double* sign, double* logabs, int32_t* n_acc, uint64_t* d_n_eval, void* work,
                       int64_t work_rows, void* stream);
int vmc_peps_chi_local_energy(int prec, const void* tensors, int Lx, int Ly, int D, int chi, const uint64_t* occ,
                              int64_t B, const int32_t* edges, double t, double U, const int32_t* pairs,
                              const int32_t* offs, const int32_t* offs_host, int64_t P, double* term, double* eloc,
                              void* work, int64_t work_rows, void* stream);
/* vmc_peps_chi_logpsi_grad — O (B, ldo >= Lx*Ly*4*D^4, dtype of prec) = d log|psi| / d
 *   tensors through the truncation (the reference differentiates its truncated
 *   contraction with torch autograd, vmc_torch/GPU/vmc_utils.py:1389-1634): the
 *   cotangent of each side's rank-chi truncation against the other side's
 *   truncated state (first-order change of the kept singular subspace, weights
 *   1/(s_i^2 - s_j^2) between kept and dropped directions), then a reverse row
 *   sweep that recomputes the forward column states.  Supported when the only
 *   truncated cut is one cut after each side's last row and its parity blocks
 *   are at most 32 x 32 (6x6 D=4 chi in [16, 64), 4x4 D=4 chi in [4, 16)), else
 *   VMC_ERR_UNSUPPORTED; FP64 also needs 2 * D^(Ly+1) doubles of shared memory.
 *   work: *bytes from vmc_peps_chi_grad_work_bytes for work_rows walkers.  Rows of
 *   zero amplitude stay zero. */
int vmc_peps_chi_grad_work_bytes(int prec, int Lx, int Ly, int D, int chi, int64_t work_rows, int64_t* bytes);
int vmc_peps_chi_logpsi_grad(int prec, const void* tensors, int Lx, int Ly, int D, int chi, const uint64_t* occ,
                             int64_t B, void* O, int64_t ldo, void* work, int64_t work_rows, void* stream);

/* ---- Point-group symmetry projection with fermionic signs
 * (FermionSymmetryProjectedModel, vmc_torch/GPU/models/symmetry.py:770-1136) ----
 * psi_r(n) = (1/G) sum_g sign(g, n) chi_r(g) psi(n[perm_g]).
 * vmc_sym_images:  occ_img (B*G, 2) = the G images of each walker (image site j
 *   holds site perms[g][j]); fsign (B*G) = sign(g, n) from the inversions of the
 *   occupied interleaved modes under g^-1 (inv_perms = inverse permutations).
 * vmc_sym_combine: projected sign/logabs (B) from the images' sign/logabs (B*G)
 *   and characters (G); weights (B*G, nullable) w_g = sign chi psi_g / (G psi_r),
 *   so that O_r = sum_g w_g O_g.
 * vmc_sym_grad_combine: O (B, ldo) = sum_g w_g O_img[b*G+g]; dtype 0 f64, 1 f32. */
int vmc_sym_images(const uint64_t* occ, int64_t B, int n_sites, const int32_t* perms, const int32_t* inv_perms, int G,
                   uint64_t* occ_img, double* fsign, void* stream);
int vmc_sym_combine(const double* sign_img, const double* logabs_img, const double* fsign, const double* chars,
                    int64_t B, int G, double* sign, double* logabs, double* weights, void* stream);
int vmc_sym_grad_combine(int dtype, const void* O_img, int64_t ld_img, const double* weights, int64_t B, int G,
                         int64_t Np, void* O, int64_t ldo, void* stream);
/* Model-agnostic sweep and local-energy steps (any model that evaluates
 * batches), used for wrapped models such as the projection:
 * vmc_propose_edge: the proposal of the sweeps on edge e (same draws; replay or
 *   Philox), prop_occ (B, 2), u_acc (B), flag (B) = proposal changes the walker.
 * vmc_accept_edge: Metropolis accept of flagged walkers from the proposals'
 *   sign/logabs (MetropolisExchangeSpinfulSamplerGPU.step,
 *   vmc_torch/GPU/sampler.py:342-367).
 * vmc_conn_rows / vmc_eloc_terms / vmc_eloc_reduce: connected configuration and
 *   H element per (walker, hop) pair, the terms H psi(x')/psi(x), and
 *   E_loc = U * doublons + sum of the walker's terms
 *   (_evaluate_energy_impl, vmc_torch/GPU/vmc_utils.py:322-476). */
int vmc_propose_edge(const uint64_t* occ, int64_t B, int n_sites, const int32_t* edges, int n_edges, int e, int s,
                     float hopping_rate, uint64_t seed, uint64_t sweep_index, const float* r_move, const uint8_t* r_bit,
                     const float* r_acc, uint64_t* prop_occ, float* u_acc, uint8_t* flag, void* stream);
int vmc_accept_edge(uint64_t* occ, int64_t B, const uint64_t* prop_occ, const float* u_acc, const uint8_t* flag,
                    const double* sign_p, const double* logabs_p, double* sign, double* logabs, int32_t* n_acc,
                    void* stream);
int vmc_conn_rows(const int32_t* pairs, int64_t P, const uint64_t* occ, int n_sites, const int32_t* edges, double t,
                  uint64_t* row_occ, double* coeff, void* stream);
int vmc_eloc_terms(const int32_t* pairs, int64_t P, const double* coeff, const double* sign_p, const double* logabs_p,
                   const double* sign, const double* logabs, double* term, void* stream);
int vmc_eloc_reduce(const uint64_t* occ, int64_t B, const int32_t* offs, const double* term, double U, double* eloc,
                    void* stream);

#ifdef __cplusplus
}
#endif
#endif /* VMC_GB300_H */
