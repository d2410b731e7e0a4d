// Point-group symmetry projection with fermionic signs
// (FermionSymmetryProjectedModel, vmc_torch/GPU/models/symmetry.py:770-1136),
// and the model-agnostic Metropolis / local-energy helpers a wrapped model is
// driven with.
//
//   psi_r(n) = (1/|G|) sum_g sign(g, n) chi_r(g) psi(n[perm_g])
//
// Images: image site j of element g holds the state of site perm_g[j].  The
// fermionic sign is the parity of the pairs of occupied modes m1 < m2
// (interleaved order m = 2 i + s, s = 0 down, 1 up) whose images under the
// mode map of g^-1, m -> 2 inv_g[i] + s, are in the opposite order; one pass
// over the occupied modes counts, for each, the already-placed images above
// it in a 128-bit mask.
#include "common.cuh"
#include "vmc_gb300.h"

using namespace vmc;

namespace {

__device__ __forceinline__ int popc_above(uint64_t lo, uint64_t hi, int pm) {  // placed images > pm
  if (pm < 64) {
    const uint64_t m = pm == 63 ? 0ull : ~((1ull << (pm + 1)) - 1ull);
    return __popcll(lo & m) + __popcll(hi);
  }
  const int q = pm - 64;
  const uint64_t m = q == 63 ? 0ull : ~((1ull << (q + 1)) - 1ull);
  return __popcll(hi & m);
}

__global__ void k_sym_images(const uint64_t* __restrict__ occ, int64_t B, int N, const int32_t* __restrict__ perms,
                             const int32_t* __restrict__ inv, int G, uint64_t* __restrict__ occ_img,
                             double* __restrict__ fsign) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= B * G) return;
  const int64_t b = t / G;
  const int g = (int)(t - b * G);
  const uint64_t up = occ[2 * b], dn = occ[2 * b + 1];
  const int32_t* pg = perms + (size_t)g * N;
  const int32_t* ig = inv + (size_t)g * N;
  uint64_t iu = 0, id = 0;
  for (int j = 0; j < N; ++j) {
    const int s = pg[j];
    iu |= ((up >> s) & 1ull) << j;
    id |= ((dn >> s) & 1ull) << j;
  }
  uint64_t lo = 0, hi = 0;
  int cnt = 0;
  for (int i = 0; i < N; ++i) {
#pragma unroll
    for (int sp = 0; sp < 2; ++sp) {  // mode 2 i (down) before 2 i + 1 (up)
      if (!(((sp ? up : dn) >> i) & 1ull)) continue;
      const int pm = 2 * ig[i] + sp;
      cnt += popc_above(lo, hi, pm);
      if (pm < 64) lo |= 1ull << pm;
      else hi |= 1ull << (pm - 64);
    }
  }
  occ_img[2 * t] = iu;
  occ_img[2 * t + 1] = id;
  fsign[t] = (cnt & 1) ? -1.0 : 1.0;
}

__global__ void k_sym_combine(const double* __restrict__ sign_img, const double* __restrict__ logabs_img,
                              const double* __restrict__ fsign, const double* __restrict__ chars, int64_t B, int G,
                              double* __restrict__ sign, double* __restrict__ logabs, double* __restrict__ w) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  double mx = -INFINITY;
  for (int g = 0; g < G; ++g) {
    const int64_t k = b * G + g;
    if (sign_img[k] != 0.0 && logabs_img[k] > mx) mx = logabs_img[k];
  }
  double sum = 0.0;
  if (mx > -INFINITY) {
    for (int g = 0; g < G; ++g) {
      const int64_t k = b * G + g;
      if (sign_img[k] != 0.0) sum += fsign[k] * chars[g] * sign_img[k] * exp(logabs_img[k] - mx);
    }
  }
  double s = 0.0, la = -INFINITY;
  if (sum != 0.0 && isfinite(sum)) {
    s = sum < 0 ? -1.0 : 1.0;
    la = mx + log(fabs(sum)) - log((double)G);
  } else if (!isfinite(sum)) {
    la = NAN;
  }
  sign[b] = s;
  logabs[b] = la;
  if (w) {
    for (int g = 0; g < G; ++g) {
      const int64_t k = b * G + g;
      double v = 0.0;
      if (s != 0.0 && sign_img[k] != 0.0) v = fsign[k] * chars[g] * sign_img[k] * s * exp(logabs_img[k] - la) / G;
      w[k] = v;
    }
  }
}

template <typename T>
__global__ void k_sym_grad(const T* __restrict__ O_img, int64_t ld_img, const double* __restrict__ w, int64_t B, int G,
                           int64_t Np, T* __restrict__ O, int64_t ldo) {
  const int64_t nblk = (Np + blockDim.x - 1) / blockDim.x;
  const int64_t b = blockIdx.x / nblk;
  const int64_t p = (blockIdx.x - b * nblk) * blockDim.x + threadIdx.x;
  if (b >= B || p >= Np) return;
  double acc = 0.0;
  for (int g = 0; g < G; ++g) acc += w[b * G + g] * (double)O_img[(b * G + g) * ld_img + p];
  O[b * ldo + p] = (T)acc;
}

// Proposal on edge e for all walkers (the draw of k_prep_sweep / the sweep
// kernels): prop_occ, the walker's acceptance uniform and a changed flag.
__global__ void k_propose_edge(const uint64_t* __restrict__ occ, int64_t B, const int32_t* __restrict__ edges, int e,
                               int s_local, int E, float hop_rate, uint64_t seed, uint64_t sweep_idx,
                               const float* __restrict__ rm, const uint8_t* __restrict__ rb,
                               const float* __restrict__ ra, uint64_t* __restrict__ prop_occ,
                               float* __restrict__ u_acc, uint8_t* __restrict__ flag) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  const int i = edges[2 * e], j = edges[2 * e + 1];
  const int xi = site_state(up, dn, i), xj = site_state(up, dn, j);
  uint8_t f = 0;
  float ua = 0.f;
  if (xi != xj) {
    float um;
    int bit;
    if (rm) {
      const size_t ridx = ((size_t)s_local * E + e) * (size_t)B + (size_t)w;
      um = rm[ridx]; bit = rb[ridx] & 1; ua = ra[ridx];
    } else {
      EdgeDraw d = draw_edge(seed, (uint64_t)w, sweep_idx, (uint32_t)e);
      um = d.u_move; bit = d.bit; ua = d.u_acc;
    }
    int ni, nj;
    propose_pair(xi, xj, um, bit, hop_rate, ni, nj);
    const uint64_t mi = 1ull << i, mj = 1ull << j;
    up &= ~(mi | mj);
    dn &= ~(mi | mj);
    if (ni & 2) up |= mi;
    if (ni & 1) dn |= mi;
    if (nj & 2) up |= mj;
    if (nj & 1) dn |= mj;
    f = 1;
  }
  prop_occ[2 * w] = up;
  prop_occ[2 * w + 1] = dn;
  u_acc[w] = ua;
  flag[w] = f;
}

__global__ void k_accept_edge(uint64_t* __restrict__ occ, int64_t B, const uint64_t* __restrict__ prop_occ,
                              const float* __restrict__ u_acc, const uint8_t* __restrict__ flag,
                              const double* __restrict__ sign_p, const double* __restrict__ logabs_p,
                              double* __restrict__ sign, double* __restrict__ logabs, int32_t* __restrict__ n_acc) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B || !flag[w]) return;
  const double la1 = logabs_p[w], la0 = logabs[w];
  bool acc;
  if (!(la1 > -INFINITY) || sign_p[w] == 0.0) acc = false;
  else if (la0 == -INFINITY) acc = true;
  else acc = (double)u_acc[w] < exp(2.0 * (la1 - la0));
  if (!acc) return;
  occ[2 * w] = prop_occ[2 * w];
  occ[2 * w + 1] = prop_occ[2 * w + 1];
  sign[w] = sign_p[w];
  logabs[w] = la1;
  if (n_acc) n_acc[w] += 1;
}

// Connected configuration and matrix element of each (walker, hop term) pair.
__global__ void k_conn_rows(const int32_t* __restrict__ pairs, int64_t P, const uint64_t* __restrict__ occ, int N,
                            const int32_t* __restrict__ edges, double t, uint64_t* __restrict__ row_occ,
                            double* __restrict__ coeff) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int w = pairs[2 * p], tm = pairs[2 * p + 1];
  const uint64_t up = occ[2 * (int64_t)w], dn = occ[2 * (int64_t)w + 1];
  const int e = tm >> 1, sp = (tm & 1) ? 0 : 1;
  int i = edges[2 * e], j = edges[2 * e + 1];
  if (i > j) { const int tt = i; i = j; j = tt; }
  const uint64_t m = sp ? up : dn;
  const int oi = (int)((m >> i) & 1ull);
  const int base = sp ? 0 : N;
  uint64_t eu = up, ed = dn;
  apply_move(eu, ed, N, base + (oi ? i : j), base + (oi ? j : i));
  row_occ[2 * p] = eu;
  row_occ[2 * p + 1] = ed;
  coeff[p] = symmray_parity(up, dn, i, j, sp) ? t : -t;
}

__global__ void k_eloc_terms(const int32_t* __restrict__ pairs, int64_t P, const double* __restrict__ coeff,
                             const double* __restrict__ sign_p, const double* __restrict__ logabs_p,
                             const double* __restrict__ sign, const double* __restrict__ logabs,
                             double* __restrict__ term) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int w = pairs[2 * p];
  double v = 0.0;
  if (sign_p[p] != 0.0 && sign[w] != 0.0) v = coeff[p] * sign_p[p] * sign[w] * exp(logabs_p[p] - logabs[w]);
  term[p] = v;
}

__global__ void k_eloc_sum(int64_t B, const uint64_t* __restrict__ occ, const int32_t* __restrict__ offs,
                           const double* __restrict__ term, double U, double* __restrict__ eloc) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  double s = U * (double)__popcll(occ[2 * w] & occ[2 * w + 1]);
  for (int q = offs[w]; q < offs[w + 1]; ++q) s += term[q];
  eloc[w] = s;
}

inline unsigned grid_of(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

extern "C" {

int vmc_sym_images(const uint64_t* occ, int64_t B, int n_sites, const int32_t* perms, const int32_t* inv_perms, int G,
                   uint64_t* occ_img, double* fsign, void* stream) {
  if (B < 0 || n_sites < 1 || n_sites > 64 || G < 1 || G > 64) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!occ || !perms || !inv_perms || !occ_img || !fsign) return VMC_ERR_ARGS;
  k_sym_images<<<grid_of(B * G, 256), 256, 0, (cudaStream_t)stream>>>(occ, B, n_sites, perms, inv_perms, G, occ_img,
                                                                       fsign);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_sym_combine(const double* sign_img, const double* logabs_img, const double* fsign, const double* chars,
                    int64_t B, int G, double* sign, double* logabs, double* weights, void* stream) {
  if (B < 0 || G < 1 || G > 64) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!sign_img || !logabs_img || !fsign || !chars || !sign || !logabs) return VMC_ERR_ARGS;
  k_sym_combine<<<grid_of(B, 256), 256, 0, (cudaStream_t)stream>>>(sign_img, logabs_img, fsign, chars, B, G, sign,
                                                                    logabs, weights);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_sym_grad_combine(int dtype, const void* O_img, int64_t ld_img, const double* weights, int64_t B, int G,
                         int64_t Np, void* O, int64_t ldo, void* stream) {
  if ((dtype != 0 && dtype != 1) || B < 0 || G < 1 || G > 64 || Np < 0 || ld_img < Np || ldo < Np) return VMC_ERR_ARGS;
  if (B == 0 || Np == 0) return VMC_OK;
  if (!O_img || !weights || !O) return VMC_ERR_ARGS;
  const int64_t nblk = (Np + 255) / 256;
  if (B * nblk > 0x7fffffffLL) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == 0)
    k_sym_grad<double><<<(unsigned)(B * nblk), 256, 0, st>>>((const double*)O_img, ld_img, weights, B, G, Np,
                                                             (double*)O, ldo);
  else
    k_sym_grad<float><<<(unsigned)(B * nblk), 256, 0, st>>>((const float*)O_img, ld_img, weights, B, G, Np, (float*)O,
                                                            ldo);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_propose_edge(const uint64_t* occ, int64_t B, int n_sites, const int32_t* edges, int n_edges, int e, int s,
                     float hopping_rate, uint64_t seed, uint64_t sweep_index, const float* r_move, const uint8_t* r_bit,
                     const float* r_acc, uint64_t* prop_occ, float* u_acc, uint8_t* flag, void* stream) {
  if (B < 0 || n_sites < 1 || n_sites > 64 || e < 0 || e >= n_edges || s < 0) return VMC_ERR_ARGS;
  if ((r_move != nullptr) != (r_acc != nullptr) || (r_move != nullptr) != (r_bit != nullptr)) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!occ || !edges || !prop_occ || !u_acc || !flag) return VMC_ERR_ARGS;
  k_propose_edge<<<grid_of(B, 256), 256, 0, (cudaStream_t)stream>>>(occ, B, edges, e, s, n_edges, hopping_rate, seed,
                                                                     sweep_index, r_move, r_bit, r_acc, prop_occ,
                                                                     u_acc, flag);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_accept_edge(uint64_t* occ, int64_t B, const uint64_t* prop_occ, const float* u_acc, const uint8_t* flag,
                    const double* sign_p, const double* logabs_p, double* sign, double* logabs, int32_t* n_acc,
                    void* stream) {
  if (B < 0) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!occ || !prop_occ || !u_acc || !flag || !sign_p || !logabs_p || !sign || !logabs) return VMC_ERR_ARGS;
  k_accept_edge<<<grid_of(B, 256), 256, 0, (cudaStream_t)stream>>>(occ, B, prop_occ, u_acc, flag, sign_p, logabs_p,
                                                                    sign, logabs, n_acc);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_conn_rows(const int32_t* pairs, int64_t P, const uint64_t* occ, int n_sites, const int32_t* edges, double t,
                  uint64_t* row_occ, double* coeff, void* stream) {
  if (P < 0 || n_sites < 1 || n_sites > 64) return VMC_ERR_ARGS;
  if (P == 0) return VMC_OK;
  if (!pairs || !occ || !edges || !row_occ || !coeff) return VMC_ERR_ARGS;
  k_conn_rows<<<grid_of(P, 256), 256, 0, (cudaStream_t)stream>>>(pairs, P, occ, n_sites, edges, t, row_occ, coeff);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_eloc_terms(const int32_t* pairs, int64_t P, const double* coeff, const double* sign_p, const double* logabs_p,
                   const double* sign, const double* logabs, double* term, void* stream) {
  if (P < 0) return VMC_ERR_ARGS;
  if (P == 0) return VMC_OK;
  if (!pairs || !coeff || !sign_p || !logabs_p || !sign || !logabs || !term) return VMC_ERR_ARGS;
  k_eloc_terms<<<grid_of(P, 256), 256, 0, (cudaStream_t)stream>>>(pairs, P, coeff, sign_p, logabs_p, sign, logabs,
                                                                   term);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_eloc_reduce(const uint64_t* occ, int64_t B, const int32_t* offs, const double* term, double U, double* eloc,
                    void* stream) {
  if (B < 0) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!occ || !offs || !eloc) return VMC_ERR_ARGS;
  k_eloc_sum<<<grid_of(B, 256), 256, 0, (cudaStream_t)stream>>>(B, occ, offs, term, U, eloc);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

}  // extern "C"
