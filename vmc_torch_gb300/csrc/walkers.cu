// Walker encodings (quimb int64 <-> packed uint64 bits), seeded sector
// initialisation, and the bit-exact spinful Fermi-Hubbard connected set.
#include "common.cuh"

using namespace vmc;

namespace {

__global__ void k_pack(const int64_t* __restrict__ fxs, int64_t B, int N, uint64_t* __restrict__ occ,
                       int* __restrict__ bad) {
  int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  uint64_t up = 0, dn = 0;
  const int64_t* x = fxs + w * N;
  for (int i = 0; i < N; ++i) {
    int64_t v = x[i];
    if (v < 0 || v > 3) { atomicExch(bad, 1); v = 0; }
    up |= (uint64_t)((v >> 1) & 1) << i;
    dn |= (uint64_t)(v & 1) << i;
  }
  occ[2 * w] = up;
  occ[2 * w + 1] = dn;
}

__global__ void k_unpack(const uint64_t* __restrict__ occ, int64_t B, int N, int64_t* __restrict__ fxs) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * N) return;
  int64_t w = idx / N;
  int i = (int)(idx - w * N);
  fxs[idx] = (int64_t)site_state(occ[2 * w], occ[2 * w + 1], i);
}

// Uniformly random placement of n_up and n_dn electrons, per walker, by a
// Philox-driven partial Fisher-Yates shuffle of the site list.
__global__ void k_init(uint64_t* __restrict__ occ, int64_t B, int N, int n_up, int n_dn, uint64_t seed) {
  int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  uint64_t res[2];
  int cnt[2] = {n_up, n_dn};
  for (int s = 0; s < 2; ++s) {
    uint8_t perm[64];
    for (int i = 0; i < N; ++i) perm[i] = (uint8_t)i;
    uint64_t m = 0;
    for (int k = 0; k < cnt[s]; ++k) {
      U4 r = philox4x32_10(U4{(uint32_t)w, (uint32_t)(w >> 32), (uint32_t)(s * 64 + k), 0x5eedu},
                           (uint32_t)seed, (uint32_t)(seed >> 32));
      int j = k + (int)(((uint64_t)r.x * (uint64_t)(N - k)) >> 32);
      uint8_t t = perm[k]; perm[k] = perm[j]; perm[j] = t;
      m |= 1ull << perm[k];
    }
    res[s] = m;
  }
  occ[2 * w] = res[0];
  occ[2 * w + 1] = res[1];
}

// One thread per (walker, term).  Term order: for each edge e (the order of
// ``edges``), spin up then spin down; then on-site terms by site.
__global__ void k_conn(const uint64_t* __restrict__ occ, int64_t B, int N, const int32_t* __restrict__ edges,
                       int E, double t, double U, uint64_t* __restrict__ eta, double* __restrict__ coeff,
                       uint8_t* __restrict__ valid) {
  const int T = 2 * E + N;
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * T) return;
  int64_t w = idx / T;
  int term = (int)(idx - w * T);
  uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  uint64_t eu = up, ed = dn;
  double c = 0.0;
  uint8_t ok = 0;
  if (term < 2 * E) {
    int e = term >> 1, s = (term & 1) ? 0 : 1;  // even term: up (s=1), odd: down (s=0)
    int i = edges[2 * e], j = edges[2 * e + 1];
    if (i > j) { int tmp = i; i = j; j = tmp; }
    uint64_t m = s ? up : dn;
    int oi = (int)((m >> i) & 1ull), oj = (int)((m >> j) & 1ull);
    if (oi != oj) {
      ok = 1;
      uint64_t flip = (1ull << i) | (1ull << j);
      if (s) eu = up ^ flip; else ed = dn ^ flip;
      c = symmray_parity(up, dn, i, j, s) ? t : -t;  // coefficient -t times (-1)^parity
    }
  } else {
    int site = term - 2 * E;
    if (((up >> site) & 1ull) && ((dn >> site) & 1ull)) { ok = 1; c = U; }
  }
  eta[2 * idx] = eu;
  eta[2 * idx + 1] = ed;
  coeff[idx] = c;
  valid[idx] = ok;
}

}  // namespace

extern "C" {

int vmc_pack(const int64_t* fxs, int64_t B, int n_sites, uint64_t* occ, int* d_bad, void* stream) {
  if (B < 0 || n_sites < 1 || n_sites > 64 || (B > 0 && (!fxs || !occ || !d_bad))) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  k_pack<<<(unsigned)((B + 255) / 256), 256, 0, (cudaStream_t)stream>>>(fxs, B, n_sites, occ, d_bad);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_unpack(const uint64_t* occ, int64_t B, int n_sites, int64_t* fxs, void* stream) {
  if (B < 0 || n_sites < 1 || n_sites > 64 || (B > 0 && (!fxs || !occ))) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  int64_t n = B * n_sites;
  k_unpack<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(occ, B, n_sites, fxs);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_init_walkers(uint64_t* occ, int64_t B, int n_sites, int n_up, int n_dn, uint64_t seed, void* stream) {
  if (B < 0 || n_sites < 1 || n_sites > 64 || n_up < 0 || n_dn < 0 || n_up > n_sites || n_dn > n_sites ||
      (B > 0 && !occ))
    return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  k_init<<<(unsigned)((B + 127) / 128), 128, 0, (cudaStream_t)stream>>>(occ, B, n_sites, n_up, n_dn, seed);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_hubbard_conn(const uint64_t* occ, int64_t B, int n_sites, const int32_t* edges, int n_edges, double t,
                     double U, uint64_t* eta, double* coeff, uint8_t* valid, void* stream) {
  if (B < 0 || n_sites < 1 || n_sites > 64 || n_edges < 0 || (B > 0 && (!occ || !eta || !coeff || !valid)) ||
      (n_edges > 0 && !edges))
    return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  int64_t n = B * (2 * (int64_t)n_edges + n_sites);
  k_conn<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(occ, B, n_sites, edges, n_edges, t, U,
                                                                        eta, coeff, valid);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

}  // extern "C"

extern "C" int vmc_abi_version(void) { return 1; }
