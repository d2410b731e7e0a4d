// Learned Metropolis-Hastings proposal for spinful lattice fermions.
//
// Network (hidden width 512, GELU):  n (2N occupations) -> 512 -> 512 -> logits
//   logits[0 .. 2E)   one per single-electron hop (edge e, spin): index 2e (up), 2e+1 (down)
//   logits[2E .. 2E+4) k = 1..4 simultaneous hops
// A hop (e, s) is valid in x when exactly one endpoint of e holds spin s.  Two
// hops conflict when they move the same spin and share a site; chosen hops are
// pairwise non-conflicting, so they commute and define x'.
//
// Proposal: k ~ softmax(k logits); then k hops drawn sequentially without
// replacement, each from softmax over the valid hops not yet chosen and not
// conflicting with the chosen ones.  The probability of the unordered set S is
// the sum over the k! orders, computed by a DP over the 2^k subsets:
//   P(T) = sum_{h in T} P(T \ h) exp(l_h) / Z(T \ h),  Z(U) = sum of exp(l) over
//   valid hops outside U and not conflicting with U.
// q(x -> x') = p(k|x) P(S|x); the reverse move uses the same (edge, spin) set at
// x' (each reversed hop is valid at x' and the conflict structure is the same),
// so q(x' -> x) = p(k|x') P(S|x').  Acceptance: min(1, |psi'|^2/|psi|^2 * q(x'->x)/q(x->x')).
//
// Kernels: occupation -> BF16 input rows; a K-looping tcgen05 GEMM (BF16 in,
// FP32 accumulate in TMEM) with GELU/BF16 or bias/FP32 epilogues for inference;
// warp-per-walker sampling and reverse-probability kernels; FP32 CUDA-core
// training kernels (forward, masked cross entropy, backward, Adam).
#include <cuda_bf16.h>
#include <cuda.h>
#include <cudaTypedefs.h>
#include "common.cuh"
#include "tc.cuh"

using namespace vmc;

namespace {

constexpr int PH = 512;      // hidden width
constexpr int PLOG = 256;    // logits row width (2E + 4 <= 256)
constexpr int KMAX = 4;
constexpr int TM = 128, TN = 256, KC = 256;   // GEMM tile, K chunk (4 atoms of 64)
constexpr int SA = TM * KC * 2, SB = TN * KC * 2;
constexpr int GSMEM = SA + SB + 1024 + 128;

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_df(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * expf(-0.5f * x * x) * 0.39894228040143267794f;
}

// ---------------------------------------------------------------------------
// input rows: bf16 (R, 2N padded to Kin) 0/1 occupations [up | down]
__global__ void k_bits_bf16(int64_t R, int N, int Kin, const uint64_t* __restrict__ occ, __nv_bfloat16* __restrict__ X) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= R * Kin) return;
  const int64_t r = idx / Kin;
  const int c = (int)(idx - r * Kin);
  float v = 0.f;
  if (c < 2 * N) v = (c < N) ? (float)((occ[2 * r] >> c) & 1ull) : (float)((occ[2 * r + 1] >> (c - N)) & 1ull);
  X[idx] = __float2bfloat16(v);
}

__global__ void k_bits_f32(int64_t R, int N, int Kin, const uint64_t* __restrict__ occ, float* __restrict__ X) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= R * Kin) return;
  const int64_t r = idx / Kin;
  const int c = (int)(idx - r * Kin);
  float v = 0.f;
  if (c < 2 * N) v = (c < N) ? (float)((occ[2 * r] >> c) & 1ull) : (float)((occ[2 * r + 1] >> (c - N)) & 1ull);
  X[idx] = v;
}

// ---------------------------------------------------------------------------
// D[M x N] = A[M x K] B[N x K]^T, bf16 K-major operands (TMA, SWIZZLE_128B),
// K a multiple of 64 processed in chunks of up to 256; one 128 x 256 tile per CTA.
// EPI 0: out_bf16[m][n] = bf16(gelu(D + bias[n]));  EPI 1: out_f32[m][n] = D + bias[n].
template <int EPI>
__global__ void __launch_bounds__(128, 1)
    k_gemm_kloop(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int K,
                 int ldo, const float* __restrict__ bias, void* __restrict__ out, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = sm;
  uint8_t* sB = sm + SA;
  uint64_t* bars = (uint64_t*)(sm + SA + SB);   // [0] load, [1] mma
  uint32_t* tslot = (uint32_t*)(bars + 2);
  int* sflag = (int*)(bars + 3);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::fence_mbar_init();
    *sflag = 1;
  }
  if (warp == 0) tc::tmem_alloc(tslot, 256);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;
  if (threadIdx.x == 0) {
    constexpr uint32_t idesc = tc::idesc_bf16_f32(TM, TN);
    int phase = 0;
    for (int k0 = 0; k0 < K; k0 += KC, phase ^= 1) {
      const int natoms = min(4, (K - k0) / 64);
      if (k0 > 0) {  // previous chunk's MMAs must finish reading smem
        if (!tc::mbar_wait(&bars[1], phase ^ 1)) { *sflag = 0; atomicExch(err, VMC_ERR_TIMEOUT); break; }
      }
      tc::mbar_arrive_expect_tx(&bars[0], natoms * (TM + TN) * 128);
      for (int j = 0; j < natoms; ++j) {
        tc::tma_load_2d(sA + j * (TM * 128), &tmA, &bars[0], k0 + j * 64, row0);
        tc::tma_load_2d(sB + j * (TN * 128), &tmB, &bars[0], k0 + j * 64, n0);
      }
      if (!tc::mbar_wait(&bars[0], phase)) { *sflag = 0; atomicExch(err, VMC_ERR_TIMEOUT); break; }
      tc::fence_after_sync();
      for (int j = 0; j < natoms; ++j)
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint64_t ad = tc::sdesc_sw128(tc::smem_u32(sA + j * (TM * 128)) + kk * 32);
          const uint64_t bd = tc::sdesc_sw128(tc::smem_u32(sB + j * (TN * 128)) + kk * 32);
          tc::mma_bf16(tbase, ad, bd, idesc, (k0 | j | kk) ? 1u : 0u);
        }
      tc::mma_commit(&bars[1]);
    }
  }
  __syncthreads();
  if (*sflag) {
    const uint32_t last_par = (uint32_t)(((K + KC - 1) / KC - 1) & 1);  // parity of the last MMA commit
    const bool done = tc::mbar_wait(&bars[1], last_par);
    tc::fence_after_sync();
    if (!done) {
      if (lane == 0) atomicExch(err, VMC_ERR_TIMEOUT);
    } else {
      const int64_t row = (int64_t)row0 + warp * 32 + lane;
      const bool live = row < M;
#pragma unroll 1
      for (int cc = 0; cc < TN / 32; ++cc) {
        float v[32];
        tc::tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cc * 32), v);
        if (!live) continue;
        const int nb = n0 + cc * 32;
        if (EPI == 0) {
          uint32_t pk[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            __nv_bfloat162 h2 = __floats2bfloat162_rn(gelu_f(v[2 * q] + bias[nb + 2 * q]),
                                                      gelu_f(v[2 * q + 1] + bias[nb + 2 * q + 1]));
            pk[q] = *reinterpret_cast<uint32_t*>(&h2);
          }
          uint4* dst = reinterpret_cast<uint4*>((__nv_bfloat16*)out + row * ldo + nb);
#pragma unroll
          for (int q = 0; q < 4; ++q) dst[q] = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
        } else {
          float4* dst = reinterpret_cast<float4*>((float*)out + row * ldo + nb);
#pragma unroll
          for (int q = 0; q < 8; ++q)
            dst[q] = make_float4(v[4 * q] + bias[nb + 4 * q], v[4 * q + 1] + bias[nb + 4 * q + 1],
                                 v[4 * q + 2] + bias[nb + 4 * q + 2], v[4 * q + 3] + bias[nb + 4 * q + 3]);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

// ---------------------------------------------------------------------------
// hop bookkeeping
struct Lat {
  const int32_t* edges;  // (E, 2), i < j
  int E, N;
};

__device__ __forceinline__ bool hop_valid(uint64_t up, uint64_t dn, const Lat& L, int h) {
  const int e = h >> 1;
  const uint64_t m = (h & 1) ? dn : up;
  const int i = L.edges[2 * e], j = L.edges[2 * e + 1];
  return (((m >> i) ^ (m >> j)) & 1ull) != 0ull;
}
// two hops conflict when they move the same spin and share a site
__device__ __forceinline__ bool hop_conflict(const Lat& L, int h1, int h2) {
  if ((h1 & 1) != (h2 & 1)) return false;
  const int a0 = L.edges[2 * (h1 >> 1)], a1 = L.edges[2 * (h1 >> 1) + 1];
  const int b0 = L.edges[2 * (h2 >> 1)], b1 = L.edges[2 * (h2 >> 1) + 1];
  return a0 == b0 || a0 == b1 || a1 == b0 || a1 == b1;
}
__device__ __forceinline__ void apply_hop(uint64_t& up, uint64_t& dn, const Lat& L, int h) {
  const int e = h >> 1, i = L.edges[2 * e], j = L.edges[2 * e + 1];
  const uint64_t flip = (1ull << i) | (1ull << j);
  if (h & 1) dn ^= flip; else up ^= flip;
}
// Conflict signature of hop h against the chosen hops S[0..k): bit t is set
// when h is S[t] or moves the same spin through a site of S[t]'s edge.
__device__ __forceinline__ unsigned conflict_sig(const Lat& L, int h, const int* S, int k) {
  unsigned sig = 0;
#pragma unroll
  for (int t = 0; t < KMAX; ++t)
    if (t < k && (h == S[t] || hop_conflict(L, h, S[t]))) sig |= 1u << t;
  return sig;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(VMC_FULL_MASK, v, o));
  return v;
}

// log p(k|x) + log P(S|x), with P(S|x) summed over the k! draw orders by the
// subset DP.  Z(U) (total weight of hops allowed after drawing the subset U) is
// accumulated for all 16 subsets in one pass over the hops, each hop adding its
// weight to the subsets it does not conflict with.  Warp-cooperative.
__device__ float log_q_set(const float* __restrict__ lg, uint64_t up, uint64_t dn, const Lat& L, const int* S, int k) {
  const int lane = threadIdx.x & 31;
  const int H = 2 * L.E;
  float mx = -INFINITY;
  for (int h = lane; h < H; h += 32)
    if (hop_valid(up, dn, L, h)) mx = fmaxf(mx, lg[h]);
  mx = warp_max(mx);
  if (!(mx > -INFINITY)) return -INFINITY;
  const int nU = 1 << k;
  float Z[1 << KMAX];
#pragma unroll
  for (int U = 0; U < (1 << KMAX); ++U) Z[U] = 0.f;
  for (int h = lane; h < H; h += 32) {
    if (!hop_valid(up, dn, L, h)) continue;
    const float wgt = expf(lg[h] - mx);
    const unsigned sig = conflict_sig(L, h, S, k);
#pragma unroll
    for (int U = 0; U < (1 << KMAX); ++U)
      if (U < nU && !(sig & (unsigned)U)) Z[U] += wgt;
  }
#pragma unroll
  for (int U = 0; U < (1 << KMAX); ++U) Z[U] = warp_sum(Z[U]);
  float e[KMAX];
#pragma unroll
  for (int t = 0; t < KMAX; ++t) e[t] = (t < k) ? expf(lg[S[t]] - mx) : 0.f;
  float P[1 << KMAX];
  P[0] = 1.f;
#pragma unroll
  for (int T = 1; T < (1 << KMAX); ++T) {
    float p = 0.f;
#pragma unroll
    for (int t = 0; t < KMAX; ++t)
      if ((T >> t) & 1) {
        const int U = T & ~(1 << t);
        if (Z[U] > 0.f) p += P[U] * e[t] / Z[U];
      }
    P[T] = p;
  }
  float pt = 0.f;
#pragma unroll
  for (int T = 1; T < (1 << KMAX); ++T)
    if (T == nU - 1) pt = P[T];
  const float* kl = lg + H;
  const float km = fmaxf(fmaxf(kl[0], kl[1]), fmaxf(kl[2], kl[3]));
  const float kz = expf(kl[0] - km) + expf(kl[1] - km) + expf(kl[2] - km) + expf(kl[3] - km);
  const float lpk = kl[k - 1] - km - logf(kz);
  return pt > 0.f ? lpk + logf(pt) : -INFINITY;
}

struct PropRec4 {
  int flag;       // 1: proposal made
  int k;          // number of hops
  float u_acc;
  float logq_fwd; // log q(x -> x')
  int hop[4];
  float logq_rev; // log q(x' -> x), filled by the reverse kernel
  int pad[3];
};

constexpr int HPL = 8;  // hops per lane (2E <= 252)

// Sample a proposal per walker from logits L(x).
__global__ void k_prop_sample(int64_t B, Lat L, const float* __restrict__ logits, const uint64_t* __restrict__ occ,
                              uint64_t seed, uint64_t step, uint64_t* __restrict__ prop_occ, PropRec4* __restrict__ rec) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= B) return;
  const float* lg = logits + w * PLOG;
  const uint64_t up0 = occ[2 * w], dn0 = occ[2 * w + 1];
  const int H = 2 * L.E;
  U4 r0 = philox4x32_10(U4{(uint32_t)w, (uint32_t)(w >> 32), (uint32_t)step, 0x9a11u}, (uint32_t)seed,
                        (uint32_t)(seed >> 32));
  U4 r1 = philox4x32_10(U4{(uint32_t)w, (uint32_t)(w >> 32), (uint32_t)step, 0x9a12u}, (uint32_t)seed,
                        (uint32_t)(seed >> 32));
  const float uk = u24(r0.x), u_acc = u24(r0.y);
  const float uh[4] = {u24(r0.z), u24(r0.w), u24(r1.x), u24(r1.y)};
  const float* kl = lg + H;
  const float km = fmaxf(fmaxf(kl[0], kl[1]), fmaxf(kl[2], kl[3]));
  float kp[4], kz = 0.f;
#pragma unroll
  for (int t = 0; t < 4; ++t) { kp[t] = expf(kl[t] - km); kz += kp[t]; }
  int k = 4;
  float acc = 0.f;
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    acc += kp[t] / kz;
    if (k == 4 && uk < acc) k = t + 1;
  }
  // per-lane hop weights (lane + 32 q), zero for invalid hops
  float wv[HPL];
  bool ex[HPL];
  float mx = -INFINITY;
#pragma unroll
  for (int q = 0; q < HPL; ++q) {
    const int h = lane + 32 * q;
    const bool v = h < H && hop_valid(up0, dn0, L, h);
    wv[q] = v ? lg[h] : -INFINITY;
    ex[q] = !v;
    mx = fmaxf(mx, wv[q]);
  }
  mx = warp_max(mx);
  bool ok = mx > -INFINITY;
#pragma unroll
  for (int q = 0; q < HPL; ++q) wv[q] = ex[q] ? 0.f : expf(wv[q] - mx);
  int S[4] = {-1, -1, -1, -1};
#pragma unroll
  for (int t = 0; t < KMAX; ++t) {
    if (t >= k || !ok) break;
    float z = 0.f;
#pragma unroll
    for (int q = 0; q < HPL; ++q) z += ex[q] ? 0.f : wv[q];
    z = warp_sum(z);
    if (!(z > 0.f)) { ok = false; break; }
    const float target = uh[t] * z;
    float run = 0.f;
    int pick = -1;
    // inverse CDF in hop-index order h = 32 q + lane
#pragma unroll
    for (int q = 0; q < HPL; ++q) {
      const float wq = ex[q] ? 0.f : wv[q];
      float inc = wq;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float y = __shfl_up_sync(VMC_FULL_MASK, inc, o);
        if (lane >= o) inc += y;
      }
      const unsigned hit = __ballot_sync(VMC_FULL_MASK, wq > 0.f && run + inc > target);
      if (pick < 0 && hit) pick = 32 * q + __ffs(hit) - 1;
      run += __shfl_sync(VMC_FULL_MASK, inc, 31);
    }
    if (pick < 0) {  // rounding at the top end: the last allowed hop
      int last = -1;
#pragma unroll
      for (int q = 0; q < HPL; ++q)
        if (!ex[q] && wv[q] > 0.f) last = max(last, lane + 32 * q);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) last = max(last, __shfl_xor_sync(VMC_FULL_MASK, last, o));
      pick = last;
    }
    S[t] = pick;
#pragma unroll
    for (int q = 0; q < HPL; ++q) {
      const int h = lane + 32 * q;
      if (h < H && (h == pick || hop_conflict(L, h, pick))) ex[q] = true;
    }
  }
  PropRec4 rc{};
  rc.flag = (ok && S[k - 1] >= 0) ? 1 : 0;
  rc.k = k;
  rc.u_acc = u_acc;
  uint64_t up = up0, dn = dn0;
  if (rc.flag) {
    for (int t = 0; t < k; ++t) { rc.hop[t] = S[t]; apply_hop(up, dn, L, S[t]); }
    rc.logq_fwd = log_q_set(lg, up0, dn0, L, S, k);
  }
  if (lane == 0) {
    rec[w] = rc;
    prop_occ[2 * w] = up;
    prop_occ[2 * w + 1] = dn;
  }
}

// log q(x' -> x) from logits L(x')
__global__ void k_prop_reverse(int64_t B, Lat L, const float* __restrict__ logits_p,
                               const uint64_t* __restrict__ prop_occ, PropRec4* __restrict__ rec) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= B) return;
  PropRec4 rc = rec[w];
  if (!rc.flag) return;
  const float lq = log_q_set(logits_p + w * PLOG, prop_occ[2 * w], prop_occ[2 * w + 1], L, rc.hop, rc.k);
  if (lane == 0) rec[w].logq_rev = lq;
}

// ---------------------------------------------------------------------------
// training: FP32 CUDA cores
// C[M x N] = op(A) op(B) (+ bias[n]); row-major; EPI: 0 plain, 1 gelu(pre) with
// pre stored in aux, 2 accumulate (C += ...), 3 split-K: block z adds the
// partial product over k in [z kchunk, (z+1) kchunk) to C atomically (C
// cleared beforehand; used for the weight gradients, whose K is the batch).
template <int EPI>
__global__ void k_sgemm(int ta, int tb, int M, int N, int K, const float* __restrict__ A, int lda,
                        const float* __restrict__ Bm, int ldb, const float* __restrict__ bias, float* __restrict__ C,
                        int ldc, float* __restrict__ aux, int kchunk) {
  constexpr int T = 64, TKk = 16;
  __shared__ float As[TKk][T + 1];
  __shared__ float Bs[TKk][T + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * T, n0 = blockIdx.x * T;
  const int kb = EPI == 3 ? blockIdx.z * kchunk : 0;
  const int ke = EPI == 3 ? min(K, kb + kchunk) : K;
  float acc[4][4] = {};
  for (int k0 = kb; k0 < ke; k0 += TKk) {
    for (int idx = threadIdx.x; idx < T * TKk; idx += 256) {
      int r, kk;
      if (ta) { kk = idx / T; r = idx - kk * T; } else { r = idx / TKk; kk = idx - r * TKk; }
      const int gm = m0 + r, gk = k0 + kk;
      As[kk][r] = (gm < M && gk < ke) ? (ta ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk]) : 0.f;
    }
    for (int idx = threadIdx.x; idx < T * TKk; idx += 256) {
      int c, kk;
      if (tb) { c = idx / TKk; kk = idx - c * TKk; } else { kk = idx / T; c = idx - kk * T; }
      const int gn = n0 + c, gk = k0 + kk;
      Bs[kk][c] = (gn < N && gk < ke) ? (tb ? Bm[(size_t)gn * ldb + gk] : Bm[(size_t)gk * ldb + gn]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TKk; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) { a[q] = As[kk][ty * 4 + q]; b[q] = Bs[kk][tx * 4 + q]; }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[q][r] = fmaf(a[q], b[r], acc[q][r]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int gm = m0 + ty * 4 + q, gn = n0 + tx * 4 + r;
      if (gm >= M || gn >= N) continue;
      float v = acc[q][r] + (bias ? bias[gn] : 0.f);
      const size_t o = (size_t)gm * ldc + gn;
      if (EPI == 1) { aux[o] = v; C[o] = gelu_f(v); }
      else if (EPI == 2) C[o] += v;
      else if (EPI == 3) atomicAdd(&C[o], v);
      else C[o] = v;
    }
}

// Masked softmax cross entropy.  Targets: hop weights w_h >= 0 (heat-bath
// |psi(x_h)/psi(x)|^2 for valid hops) normalised per row; k target pk (4).
// Writes dlogits = (softmax - target)/R and the per-row loss.
__global__ void k_prop_loss(int R, Lat L, const uint64_t* __restrict__ occ, const float* __restrict__ logits,
                            const float* __restrict__ tgt, const float* __restrict__ ktgt, float kweight,
                            float* __restrict__ dlog, float* __restrict__ loss) {
  const int lane = threadIdx.x & 31;
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= R) return;
  const int H = 2 * L.E;
  const uint64_t up = occ[2 * r], dn = occ[2 * r + 1];
  const float* lg = logits + (size_t)r * PLOG;
  const float* tg = tgt + (size_t)r * H;
  float* dl = dlog + (size_t)r * PLOG;
  float mx = -INFINITY, ts = 0.f;
  for (int h = lane; h < H; h += 32)
    if (hop_valid(up, dn, L, h)) { mx = fmaxf(mx, lg[h]); ts += tg[h]; }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(VMC_FULL_MASK, mx, o));
  ts = warp_sum(ts);
  float z = 0.f;
  for (int h = lane; h < H; h += 32)
    if (hop_valid(up, dn, L, h)) z += expf(lg[h] - mx);
  z = warp_sum(z);
  const float lz = mx + logf(z);
  float ls = 0.f;
  const float inv = 1.0f / (float)R;
  for (int h = lane; h < PLOG; h += 32) {
    float g = 0.f;
    if (h < H && hop_valid(up, dn, L, h) && ts > 0.f) {
      const float p = expf(lg[h] - lz), t = tg[h] / ts;
      g = (p - t) * inv;
      if (t > 0.f) ls -= t * (lg[h] - lz);
    }
    dl[h] = g;
  }
  ls = warp_sum(ls);
  if (lane == 0) {
    const float* kl = lg + H;
    float km = fmaxf(fmaxf(kl[0], kl[1]), fmaxf(kl[2], kl[3]));
    float e[4], kz = 0.f;
    for (int t = 0; t < 4; ++t) { e[t] = expf(kl[t] - km); kz += e[t]; }
    float lk = 0.f;
    for (int t = 0; t < 4; ++t) {
      const float p = e[t] / kz;
      dl[H + t] = kweight * (p - ktgt[t]) * inv;
      if (ktgt[t] > 0.f) lk -= ktgt[t] * logf(p);
    }
    loss[r] = (ts > 0.f ? ls : 0.f) + kweight * lk;
  }
}

// dZ = dH * gelu'(pre)
__global__ void k_gelu_back(int64_t n, const float* __restrict__ pre, float* __restrict__ d) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] *= gelu_df(pre[i]);
}
// column sums (bias gradients): out[n] = sum_m D[m][n]
__global__ void k_colsum(int M, int N, const float* __restrict__ D, int ldd, float* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += D[(size_t)m * ldd + n];
  out[n] = s;
}
// Adam (bias-corrected) on a flat parameter vector
__global__ void k_adam(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}
// heat-bath targets from local-energy terms: tgt[w][hop] = (term/coeff)^2
__global__ void k_collect(int64_t P, const int32_t* __restrict__ pairs, const double* __restrict__ term,
                          double t_abs, int H, int64_t row0, float* __restrict__ tgt) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  const int64_t w = pairs[2 * p];
  const int h = pairs[2 * p + 1];
  const double r = term[p] / t_abs;
  tgt[(row0 + w) * H + h] = (float)(r * r);
}

PFN_cuTensorMapEncodeTiled_v12000 g_enc = nullptr;
bool tmap(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols, uint32_t box_rows) {
  if (!g_enc) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return false;
    g_enc = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  if (((uintptr_t)base & 15) != 0 || (cols * 2) % 16 != 0) return false;
  cuuint64_t gdim[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t gstr[1] = {(cuuint64_t)cols * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  return g_enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), gdim, gstr, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// kernel attributes are per device: set on each device the first time it is current
bool g_attr[64] = {};

int gemm_bf16(int epi, const __nv_bfloat16* A, int64_t M, int K, const __nv_bfloat16* Bw, int N, const float* bias,
              void* out, int ldo, int* err, cudaStream_t st) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return VMC_ERR_CUDA;
  if (!g_attr[dev]) {
    cudaFuncSetAttribute(k_gemm_kloop<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, GSMEM);
    cudaFuncSetAttribute(k_gemm_kloop<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, GSMEM);
    g_attr[dev] = true;
  }
  if (K % 64 != 0 || N % TN != 0) return VMC_ERR_ARGS;
  CUtensorMap ta, tb;
  if (!tmap(&ta, A, (uint64_t)M, (uint64_t)K, TM) || !tmap(&tb, Bw, (uint64_t)N, (uint64_t)K, TN))
    return VMC_ERR_UNSUPPORTED;
  dim3 g((unsigned)((M + TM - 1) / TM), (unsigned)(N / TN));
  if (epi == 0) k_gemm_kloop<0><<<g, 128, GSMEM, st>>>(ta, tb, (int)M, K, ldo, bias, out, err);
  else k_gemm_kloop<1><<<g, 128, GSMEM, st>>>(ta, tb, (int)M, K, ldo, bias, out, err);
  return VMC_OK;
}

}  // namespace

// Metropolis-Hastings accept of learned proposals for any model: the
// proposals' sign / log-amplitude come from the model's own evaluation.
// Accept with min(1, |psi'/psi|^2 q(x'->x)/q(x->x')); a NaN ratio never
// accepts, a zero-amplitude proposal never, and from a zero-amplitude walker
// every non-zero proposal with a finite reverse probability does.  On accept
// the walker takes x', its sign / log-amplitude and (when given) the proposal
// logits at x'.  One warp per walker (the logits row is 256 floats).
__global__ void k_accept_mh(int64_t B, uint64_t* __restrict__ occ, const uint64_t* __restrict__ prop_occ,
                            const PropRec4* __restrict__ rec, const double* __restrict__ sign_p,
                            const double* __restrict__ logabs_p, double* __restrict__ sign, double* __restrict__ logabs,
                            int32_t* __restrict__ n_acc, float* __restrict__ lg_x, const float* __restrict__ lg_p,
                            int* __restrict__ kstats) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= B) return;
  const PropRec4 r = rec[w];
  if (!r.flag) return;
  const double l1 = logabs_p[w], l0 = logabs[w];
  const double lr = 2.0 * (l1 - l0) + ((double)r.logq_rev - (double)r.logq_fwd);
  bool acc;
  if (!(l1 > -INFINITY) || sign_p[w] == 0.0 || !isfinite(r.logq_rev)) acc = false;
  else if (l0 == -INFINITY) acc = true;
  else acc = (lr == lr) && ((double)r.u_acc < exp(fmin(lr, 80.0)));
  const int kk = min(max(r.k, 1), 4) - 1;
  if (kstats && lane == 0) {
    atomicAdd(&kstats[kk], 1);
    if (acc) atomicAdd(&kstats[4 + kk], 1);
  }
  if (!acc) return;
  if (lg_x) {
#pragma unroll
    for (int q = 0; q < 8; ++q) lg_x[w * PLOG + lane * 8 + q] = lg_p[w * PLOG + lane * 8 + q];
  }
  if (lane == 0) {
    occ[2 * w] = prop_occ[2 * w];
    occ[2 * w + 1] = prop_occ[2 * w + 1];
    sign[w] = sign_p[w];
    logabs[w] = l1;
    if (n_acc) n_acc[w] += 1;
  }
}

extern "C" {

int vmc_accept_mh(uint64_t* occ, int64_t B, const uint64_t* prop_occ, const void* rec4, const double* sign_p,
                  const double* logabs_p, double* sign, double* logabs, int32_t* n_acc, float* lg_x,
                  const float* lg_p, int* kstats, void* stream) {
  if (B < 0 || (lg_x != nullptr) != (lg_p != nullptr)) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!occ || !prop_occ || !rec4 || !sign_p || !logabs_p || !sign || !logabs) return VMC_ERR_ARGS;
  k_accept_mh<<<(unsigned)((B * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      B, occ, prop_occ, (const PropRec4*)rec4, sign_p, logabs_p, sign, logabs, n_acc, lg_x, lg_p, kstats);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// Inference: logits (R, 256) fp32 for configurations occ (R, 2).
// wts[6]: W1 (512, Kin) bf16, b1 (512) f32, W2 (512, 512) bf16, b2 f32,
//         Wo (256, 512) bf16, bo (256) f32.  Workspace X (R, Kin) bf16,
//         H1, H2 (R, 512) bf16.  Kin = 2N rounded up to a multiple of 64.
int vmc_prop_logits(const void* const* wts, int n_sites, const uint64_t* occ, int64_t R, void* X, void* H1, void* H2,
                    float* logits, int* d_err, void* stream) {
  if (n_sites < 1 || n_sites > 64 || R < 0 || !wts || !occ || !X || !H1 || !H2 || !logits || !d_err)
    return VMC_ERR_ARGS;
  if (R == 0) return VMC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int Kin = ((2 * n_sites + 63) / 64) * 64;
  k_bits_bf16<<<(unsigned)((R * Kin + 255) / 256), 256, 0, st>>>(R, n_sites, Kin, occ, (__nv_bfloat16*)X);
  int rc = gemm_bf16(0, (const __nv_bfloat16*)X, R, Kin, (const __nv_bfloat16*)wts[0], PH, (const float*)wts[1], H1,
                     PH, d_err, st);
  if (rc) return rc;
  rc = gemm_bf16(0, (const __nv_bfloat16*)H1, R, PH, (const __nv_bfloat16*)wts[2], PH, (const float*)wts[3], H2, PH,
                 d_err, st);
  if (rc) return rc;
  rc = gemm_bf16(1, (const __nv_bfloat16*)H2, R, PH, (const __nv_bfloat16*)wts[4], PLOG, (const float*)wts[5], logits,
                 PLOG, d_err, st);
  if (rc) return rc;
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_prop_sample(const int32_t* edges, int n_edges, int n_sites, const float* logits, const uint64_t* occ,
                    int64_t B, uint64_t seed, uint64_t step, uint64_t* prop_occ, void* rec, void* stream) {
  if (n_edges < 1 || 2 * n_edges + 4 > PLOG || B < 0 || !edges || !logits || !occ || !prop_occ || !rec)
    return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  Lat L{edges, n_edges, n_sites};
  k_prop_sample<<<(unsigned)((B * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(B, L, logits, occ, seed, step,
                                                                                   prop_occ, (PropRec4*)rec);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_prop_reverse(const int32_t* edges, int n_edges, int n_sites, const float* logits_p, const uint64_t* prop_occ,
                     int64_t B, void* rec, void* stream) {
  if (n_edges < 1 || 2 * n_edges + 4 > PLOG || B < 0 || !edges || !logits_p || !prop_occ || !rec) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  Lat L{edges, n_edges, n_sites};
  k_prop_reverse<<<(unsigned)((B * 32 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(B, L, logits_p, prop_occ,
                                                                                    (PropRec4*)rec);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// One training step (forward, loss, backward, Adam) on R samples.
// params (FP32 masters, contiguous flat): [W1 (512,Kin), b1, W2 (512,512), b2, Wo (256,512), bo]
// m1, m2: Adam moments (same layout); grad: workspace of the same size.
// ws: FP32 workspace of R * (4*512 + 2*256) floats.  Xf: (R, Kin) fp32 inputs.
int vmc_prop_train_step(int n_sites, const int32_t* edges, int n_edges, const uint64_t* occ, int R, const float* Xf,
                        const float* tgt, const float* ktgt, float kweight, float* params, float* grad, float* m1,
                        float* m2, int64_t n_params, float lr, float beta1, float beta2, float eps, int t,
                        float* ws, float* loss, void* stream) {
  if (n_sites < 1 || n_sites > 64 || R <= 0 || n_edges < 1 || 2 * n_edges + 4 > PLOG || !edges || !occ || !Xf ||
      !tgt || !ktgt || !params || !grad || !m1 || !m2 || !ws || !loss || t < 1)
    return VMC_ERR_ARGS;
  const int Kin = ((2 * n_sites + 63) / 64) * 64;
  const int64_t np = (int64_t)PH * Kin + PH + (int64_t)PH * PH + PH + (int64_t)PLOG * PH + PLOG;
  if (n_params != np) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  float* W1 = params;
  float* b1 = W1 + (size_t)PH * Kin;
  float* W2 = b1 + PH;
  float* b2 = W2 + (size_t)PH * PH;
  float* Wo = b2 + PH;
  float* bo = Wo + (size_t)PLOG * PH;
  float* gW1 = grad;
  float* gb1 = gW1 + (size_t)PH * Kin;
  float* gW2 = gb1 + PH;
  float* gb2 = gW2 + (size_t)PH * PH;
  float* gWo = gb2 + PH;
  float* gbo = gWo + (size_t)PLOG * PH;
  float* Z1 = ws;                       // R x 512 pre-activations
  float* H1 = Z1 + (size_t)R * PH;      // R x 512
  float* Z2 = H1 + (size_t)R * PH;
  float* H2 = Z2 + (size_t)R * PH;
  float* LG = H2 + (size_t)R * PH;      // R x 256 logits
  float* DL = LG + (size_t)R * PLOG;    // R x 256 dlogits
  auto grid = [](int M, int N) { return dim3((unsigned)((N + 63) / 64), (unsigned)((M + 63) / 64)); };
  // weight gradients: K = R (the batch), split in chunks of 256 rows so that
  // the 512 x 512 products fill the GPU; the partial sums land atomically in
  // the cleared gradient vector
  const int kc = 256;
  const unsigned nz = (unsigned)((R + kc - 1) / kc);
  auto gridk = [nz](int M, int N) { return dim3((unsigned)((N + 63) / 64), (unsigned)((M + 63) / 64), nz); };
  if (cudaMemsetAsync(grad, 0, (size_t)np * sizeof(float), st) != cudaSuccess) return VMC_ERR_CUDA;
  // forward
  k_sgemm<1><<<grid(R, PH), 256, 0, st>>>(0, 1, R, PH, Kin, Xf, Kin, W1, Kin, b1, H1, PH, Z1, 0);
  k_sgemm<1><<<grid(R, PH), 256, 0, st>>>(0, 1, R, PH, PH, H1, PH, W2, PH, b2, H2, PH, Z2, 0);
  k_sgemm<0><<<grid(R, PLOG), 256, 0, st>>>(0, 1, R, PLOG, PH, H2, PH, Wo, PH, bo, LG, PLOG, nullptr, 0);
  Lat L{edges, n_edges, n_sites};
  k_prop_loss<<<(unsigned)((R * 32 + 255) / 256), 256, 0, st>>>(R, L, occ, LG, tgt, ktgt, kweight, DL, loss);
  // backward
  k_sgemm<3><<<gridk(PLOG, PH), 256, 0, st>>>(1, 0, PLOG, PH, R, DL, PLOG, H2, PH, nullptr, gWo, PH, nullptr, kc);
  k_colsum<<<(PLOG + 255) / 256, 256, 0, st>>>(R, PLOG, DL, PLOG, gbo);
  // dH2 = DL Wo -> stored in H2 (H2 no longer needed), then * gelu'(Z2)
  k_sgemm<0><<<grid(R, PH), 256, 0, st>>>(0, 0, R, PH, PLOG, DL, PLOG, Wo, PH, nullptr, H2, PH, nullptr, 0);
  k_gelu_back<<<(unsigned)(((int64_t)R * PH + 255) / 256), 256, 0, st>>>((int64_t)R * PH, Z2, H2);
  k_sgemm<3><<<gridk(PH, PH), 256, 0, st>>>(1, 0, PH, PH, R, H2, PH, H1, PH, nullptr, gW2, PH, nullptr, kc);
  k_colsum<<<(PH + 255) / 256, 256, 0, st>>>(R, PH, H2, PH, gb2);
  // dH1 = dZ2 W2 -> Z2 buffer, * gelu'(Z1)
  k_sgemm<0><<<grid(R, PH), 256, 0, st>>>(0, 0, R, PH, PH, H2, PH, W2, PH, nullptr, Z2, PH, nullptr, 0);
  k_gelu_back<<<(unsigned)(((int64_t)R * PH + 255) / 256), 256, 0, st>>>((int64_t)R * PH, Z1, Z2);
  k_sgemm<3><<<gridk(PH, Kin), 256, 0, st>>>(1, 0, PH, Kin, R, Z2, PH, Xf, Kin, nullptr, gW1, Kin, nullptr, kc);
  k_colsum<<<(PH + 255) / 256, 256, 0, st>>>(R, PH, Z2, PH, gb1);
  // Adam
  const float c1 = 1.0f - powf(beta1, (float)t), c2 = 1.0f - powf(beta2, (float)t);
  k_adam<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(np, params, grad, m1, m2, lr, beta1, beta2, eps, c1, c2);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// Training inputs: fp32 (R, Kin) occupations.
int vmc_prop_inputs_f32(int n_sites, const uint64_t* occ, int64_t R, float* Xf, void* stream) {
  if (n_sites < 1 || n_sites > 64 || R < 0 || !occ || !Xf) return VMC_ERR_ARGS;
  if (R == 0) return VMC_OK;
  const int Kin = ((2 * n_sites + 63) / 64) * 64;
  const int64_t n = R * Kin;
  k_bits_f32<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(R, n_sites, Kin, occ, Xf);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_prop_collect_targets(const int32_t* pairs, int64_t P, const double* term, double t_abs, int n_hops,
                             int64_t row0, float* tgt, void* stream) {
  if (P < 0 || n_hops < 1 || !tgt || !(t_abs > 0.0) || (P > 0 && (!pairs || !term))) return VMC_ERR_ARGS;
  if (P == 0) return VMC_OK;
  k_collect<<<(unsigned)((P + 255) / 256), 256, 0, (cudaStream_t)stream>>>(P, pairs, term, t_abs, n_hops, row0, tgt);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

}  // extern "C"
