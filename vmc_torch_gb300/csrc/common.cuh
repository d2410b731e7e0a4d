// Shared device helpers for the GB300 VMC kernels: status codes, the
// counter-based Philox4x32-10 generator, packed-occupation bit helpers and
// warp reductions.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/vmc_gb300.h"

#define VMC_FULL_MASK 0xffffffffu

namespace vmc {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with the
// published multipliers and Weyl key increments.
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// 24-bit uniform in [0, 1) as a float32 (the same value set as torch.rand).
__device__ __forceinline__ float u24(uint32_t r) { return (float)(r >> 8) * (1.0f / 16777216.0f); }

// Draws for one (walker, sweep, edge): u_move, hop bit, u_acc.
struct EdgeDraw { float u_move; int bit; float u_acc; };

__device__ __forceinline__ EdgeDraw draw_edge(uint64_t seed, uint64_t walker, uint64_t sweep, uint32_t edge) {
  U4 c{(uint32_t)walker, (uint32_t)(walker >> 32) ^ (edge << 8), (uint32_t)sweep, (uint32_t)(sweep >> 32)};
  U4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  return EdgeDraw{u24(r.x), (int)(r.y & 1u), u24(r.z)};
}

// ---------------------------------------------------------------------------
// Packed occupations: walker w holds occ[2w] = up bits, occ[2w+1] = down bits,
// site i -> bit i (n_sites <= 64).  Netket spin-orbital index: up at site i ->
// i, down at site i -> n_sites + i.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t bits_below(int i) { return i >= 64 ? ~0ull : ((1ull << i) - 1ull); }
__device__ __forceinline__ uint64_t bits_between(int i, int j) {  // strictly between, i < j
  return bits_below(j) & ~bits_below(i + 1);
}
__device__ __forceinline__ int site_state(uint64_t up, uint64_t dn, int i) {
  return (int)(((up >> i) & 1ull) << 1 | ((dn >> i) & 1ull));  // quimb: 2*up + dn
}
// Number of occupied netket orbitals with index < o.
__device__ __forceinline__ int orb_prefix(uint64_t up, uint64_t dn, int N, int o) {
  if (o < N) return __popcll(up & bits_below(o));
  return __popcll(up) + __popcll(dn & bits_below(o - N));
}
__device__ __forceinline__ bool orb_occupied(uint64_t up, uint64_t dn, int N, int o) {
  return o < N ? ((up >> o) & 1ull) : ((dn >> (o - N)) & 1ull);
}
// Parity of occupied orbitals strictly between a (occupied) and b (empty):
// the sign picked up when orbital a is replaced by b in an ascending row list.
__device__ __forceinline__ int reorder_parity(uint64_t up, uint64_t dn, int N, int a, int b) {
  int pa = orb_prefix(up, dn, N, a), pb = orb_prefix(up, dn, N, b);
  int between = (a < b) ? (pb - pa - 1) : (pa - pb);
  return between & 1;
}
// symmray hop phase parity for a hop on sites i < j with spin s (1 up, 0 down):
// occupied interleaved modes strictly between 2i+s and 2j+s.
__device__ __forceinline__ int symmray_parity(uint64_t up, uint64_t dn, int i, int j, int s) {
  uint64_t m = bits_between(i, j);
  int c = __popcll(up & m) + __popcll(dn & m);
  c += s ? (int)((dn >> j) & 1ull) : (int)((up >> i) & 1ull);
  return c & 1;
}

// Exchange-or-hop proposal on one edge (reference propose_exchange_or_hopping_vec).
// Returns the new (xi, xj); caller guarantees xi != xj.
__device__ __forceinline__ void propose_pair(int xi, int xj, float u_move, int bit, float hopping_rate,
                                             int& ni, int& nj) {
  const int nmap_i = (xi == 0) ? 0 : (xi == 3 ? 2 : 1);
  const int nmap_j = (xj == 0) ? 0 : (xj == 3 ? 2 : 1);
  const int dn = nmap_i > nmap_j ? nmap_i - nmap_j : nmap_j - nmap_i;
  const bool is_ex = u_move < (1.0f - hopping_rate);
  if (is_ex || dn == 1) { ni = xj; nj = xi; return; }
  if (dn == 0) { ni = bit ? 3 : 0; nj = bit ? 0 : 3; return; }
  ni = bit ? 2 : 1; nj = bit ? 1 : 2;  // dn == 2
}

// Electron moves implied by (xi, xj) -> (ni, nj): up to one per spin.
// Each move is (from orbital a, to orbital b) in netket indices.
struct Moves { int n; int a[2]; int b[2]; };
__device__ __forceinline__ Moves pair_moves(int i, int j, int xi, int ni, int N) {
  Moves m; m.n = 0;
  // up (bit 1 of the quimb state)
  int ui = (xi >> 1) & 1, nui = (ni >> 1) & 1;
  if (ui != nui) { if (ui) { m.a[m.n] = i; m.b[m.n] = j; } else { m.a[m.n] = j; m.b[m.n] = i; } ++m.n; }
  int di = xi & 1, ndi = ni & 1;
  if (di != ndi) { if (di) { m.a[m.n] = N + i; m.b[m.n] = N + j; } else { m.a[m.n] = N + j; m.b[m.n] = N + i; } ++m.n; }
  return m;
}
__device__ __forceinline__ void apply_move(uint64_t& up, uint64_t& dn, int N, int a, int b) {
  if (a < N) { up &= ~(1ull << a); up |= 1ull << b; }
  else { dn &= ~(1ull << (a - N)); dn |= 1ull << (b - N); }
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(VMC_FULL_MASK, v, o);
  return v;
}

}  // namespace vmc

#define VMC_CUDA_CHECK_LAUNCH()                                   \
  do {                                                            \
    cudaError_t _e = cudaGetLastError();                          \
    if (_e != cudaSuccess) return VMC_ERR_CUDA;                   \
  } while (0)
