// Sample-space SR Gram matrix on the tensor cores:
//
//   T (Ns x Ns, FP64) [+]= alpha * (X X^T) o D  (+ shift I)
//
// for an FP32 matrix X (Ns x K): the per-sample log-derivatives, centred and
// scaled (the dense block of O), or the Kronecker factor G of the NNBF output
// layer (with D = H H^T).  Fixed-point split (the Ozaki scheme's idea): each
// row i gets a shared power-of-two exponent E_i (its largest |x| below
// 2^E_i), and y = x 2^-E_i is written as three 7-bit integer digits,
//   y = 2^-6 a0 + 2^-13 a1 + 2^-20 a2,  a_s in [-64, 64]
// (to 2^-20 of the row's largest entry), each digit scaled by its power of two
// exactly representable in BF16.  The product y_i y_j is taken as all nine
// digit products (hi, mid, lo the three planes), so the result is exactly the
// Gram matrix of the rounded rows and stays positive semidefinite.  The
// leading term hi hi is an integer multiple of 2^-12 of magnitude <= 1, so its
// FP32 running sum over a 2048-column chunk (<= 2^23 units) is exact: it
// accumulates in its own TMEM accumulator with no rounding at all.  The eight
// small terms (2^-7 of it and below) share a second accumulator, where FP32
// rounding is ~2^-25 of 2^-7 of the result.
// Both are drained into the FP64 result every 2048 columns of K, scaled by
// 2^(E_i + E_j).
//
// Tile: 128 x 128 outputs per CTA, lower triangle of tiles only (the upper
// triangle is written as the mirror image).  K atoms of 64 BF16 (128 bytes per
// row) are staged by TMA (SWIZZLE_128B) through a 2-stage pipeline; each stage
// holds the three planes of the 128 rows of both operands (96 KB).  Warp 0
// issues the copies, warp 1 (one thread) the tcgen05 MMAs into two TMEM
// buffers used alternately per K chunk (each 2 x 128 columns: leading and
// small products), warps 2..5 add each finished chunk into T.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include "common.cuh"
#include "tc.cuh"

namespace {

constexpr int GT = 128;                       // tile rows / cols
constexpr int KA = 64;                        // bf16 per K atom (128 bytes)
constexpr int PLANE = GT * KA * 2;            // 16 KB: one plane of one operand, one atom
constexpr int STAGE = 6 * PLANE;              // A hi/mid/lo + B hi/mid/lo
constexpr int NSTAGE = 2;
constexpr int CHUNK_ATOMS = 32;               // 2048 columns of K per FP32 accumulation
constexpr int GR_THREADS = 192;
constexpr int GR_SMEM = NSTAGE * STAGE + 1024 + 256;

// Row exponents: E[r] = ilogb(max_k |X[r][k]|) + 1 (0 for a zero row or a
// padding row), one warp per row.
__global__ void k_row_exp(const float* __restrict__ X, int64_t rows, int64_t rows_pad, int64_t K, int64_t ldx,
                          int* __restrict__ E) {
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= rows_pad) return;
  float m = 0.f;
  if (r < rows)
    for (int64_t c = lane; c < K; c += 32) m = fmaxf(m, fabsf(X[r * ldx + c]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(VMC_FULL_MASK, m, o));
  if (lane == 0) E[r] = (m > 0.f && m < INFINITY) ? ilogbf(m) + 1 : 0;
}

// x -> (hi, mid, lo) planes of the fixed-point digits of x 2^-E[r] (plane p at
// P + p * plane), row-major with row stride kp; rows >= `rows` and columns >=
// K are zero.  Every step below is exact in FP32: scaling by powers of two,
// rounding to an integer, and the subtraction of that integer from a value
// within 0.5 of it.
__global__ void k_split3(const float* __restrict__ X, int64_t rows, int64_t rows_pad, int64_t K, int64_t ldx,
                         int64_t kp, const int* __restrict__ E, __nv_bfloat16* __restrict__ P) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= rows_pad * kp) return;
  const int64_t r = idx / kp, c = idx - r * kp;
  const float x = (r < rows && c < K) ? X[r * ldx + c] : 0.f;
  const float y = ldexpf(x, 6 - E[r]);       // 2^6 x 2^-E, |y| < 64
  const float a0 = rintf(y);
  const float r1 = (y - a0) * 128.f;         // |r1| <= 64
  const float a1 = rintf(r1);
  const float a2 = rintf((r1 - a1) * 128.f);
  const int64_t plane = rows_pad * kp;
  P[idx] = __float2bfloat16_rn(ldexpf(a0, -6));
  P[plane + idx] = __float2bfloat16_rn(ldexpf(a1, -13));
  P[2 * plane + idx] = __float2bfloat16_rn(ldexpf(a2, -20));
}

struct GramArgs {
  double* T;
  int64_t ldt;
  const double* D;   // nullable, ld = ldt
  const int* E;      // row exponents of the split
  double alpha, shift;
  int n;             // rows of X (order of T)
  int prow;          // rows per plane (n rounded up to the tile)
  int n_atoms, accumulate;
};

// tile index -> (bi, bj), bj <= bi, row-major over the lower triangle
__device__ __forceinline__ void tile_of(int t, int& bi, int& bj) {
  int i = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
  while ((i + 1) * (i + 2) / 2 <= t) ++i;
  while (i * (i + 1) / 2 > t) --i;
  bi = i;
  bj = t - i * (i + 1) / 2;
}

__global__ void __launch_bounds__(GR_THREADS, 1)
    k_gram_bf16x3(const __grid_constant__ CUtensorMap tmX, GramArgs ga, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bar = (uint64_t*)(sm + NSTAGE * STAGE);
  uint64_t* full = bar;          // [NSTAGE]
  uint64_t* empty = bar + 2;     // [NSTAGE]
  uint64_t* tfull = bar + 4;     // [2]
  uint64_t* tempty = bar + 6;    // [2]
  uint32_t* tslot = (uint32_t*)(bar + 8);
  volatile int* abort_flag = (volatile int*)(bar + 9);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int bi, bj;
  tile_of(blockIdx.x, bi, bj);
  const int n_chunks = (ga.n_atoms + CHUNK_ATOMS - 1) / CHUNK_ATOMS;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) { tc::mbar_init(&full[s], 1); tc::mbar_init(&empty[s], 1); }
    for (int b = 0; b < 2; ++b) { tc::mbar_init(&tfull[b], 1); tc::mbar_init(&tempty[b], 4); }
    *abort_flag = 0;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tmX);
  }
  if (warp == 0) tc::tmem_alloc(tslot, 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;
  if (warp == 0) {
    if (lane == 0) {  // ---- TMA producer: atom a -> stage a % NSTAGE ----
      for (int a = 0; a < ga.n_atoms && !*abort_flag; ++a) {
        const int s = a % NSTAGE;
        if (a >= NSTAGE && !tc::mbar_wait(&empty[s], ((a / NSTAGE) - 1) & 1)) {
          *abort_flag = 1;
          atomicExch(err, VMC_ERR_TIMEOUT);
          break;
        }
        tc::mbar_arrive_expect_tx(&full[s], STAGE);
        uint8_t* st = sm + s * STAGE;
#pragma unroll
        for (int p = 0; p < 3; ++p) {   // plane p of the rows of tile bi (A) and of tile bj (B)
          tc::tma_load_2d(st + p * PLANE, &tmX, &full[s], a * KA, p * ga.prow + bi * GT);
          tc::tma_load_2d(st + (3 + p) * PLANE, &tmX, &full[s], a * KA, p * ga.prow + bj * GT);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // ---- MMA issuer ----
      constexpr uint32_t idesc = tc::idesc_bf16_f32(GT, GT);
      // (A plane, B plane) of the nine products: the leading one, then the rest
      constexpr int pa[9] = {0, 0, 1, 0, 2, 1, 1, 2, 2};
      constexpr int pb[9] = {0, 1, 0, 2, 0, 1, 2, 1, 2};
      for (int c = 0; c < n_chunks && !*abort_flag; ++c) {
        const int buf = c & 1;
        if (c >= 2 && !tc::mbar_wait(&tempty[buf], ((c >> 1) - 1) & 1)) {
          *abort_flag = 1;
          atomicExch(err, VMC_ERR_TIMEOUT);
          break;
        }
        tc::fence_after_sync();
        const uint32_t dt = tbase + (uint32_t)(buf * 2 * GT);   // leading products; small ones at + GT
        const int a0 = c * CHUNK_ATOMS, a1 = min(ga.n_atoms, a0 + CHUNK_ATOMS);
        bool ok = true;
        for (int a = a0; a < a1; ++a) {
          const int s = a % NSTAGE;
          if (!tc::mbar_wait(&full[s], (a / NSTAGE) & 1)) { ok = false; break; }
          tc::fence_after_sync();
          const uint8_t* st = sm + s * STAGE;
#pragma unroll
          for (int q = 0; q < 9; ++q) {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint64_t ad = tc::sdesc_sw128(tc::smem_u32(st + pa[q] * PLANE) + kk * 32);
              const uint64_t bd = tc::sdesc_sw128(tc::smem_u32(st + (3 + pb[q]) * PLANE) + kk * 32);
              if (q == 0) tc::mma_bf16(dt, ad, bd, idesc, (a > a0 || kk) ? 1u : 0u);
              else tc::mma_bf16(dt + GT, ad, bd, idesc, (a > a0 || q > 1 || kk) ? 1u : 0u);
            }
          }
          tc::mma_commit(&empty[s]);   // the stage is free once these MMAs have read it
        }
        if (!ok) { *abort_flag = 1; atomicExch(err, VMC_ERR_TIMEOUT); break; }
        tc::mma_commit(&tfull[buf]);
      }
    }
  } else {  // ---- epilogue: warps 2..5, TMEM lane quadrant warp % 4 ----
    const int quad = warp & 3;
    const int r = quad * 32 + lane;          // row of the tile
    const int64_t gi = (int64_t)bi * GT + r;
    const bool live = gi < ga.n;
    for (int c = 0; c < n_chunks; ++c) {
      const int buf = c & 1;
      bool ok = tc::mbar_wait(&tfull[buf], (c >> 1) & 1);
      ok = __all_sync(VMC_FULL_MASK, ok);
      if (!ok) { if (lane == 0) { *abort_flag = 1; atomicExch(err, VMC_ERR_TIMEOUT); } break; }
      tc::fence_after_sync();
      const bool first = (c == 0) && !ga.accumulate;
      const bool last = c == n_chunks - 1;
#pragma unroll 1
      for (int cc = 0; cc < GT / 32; ++cc) {
        float v[32], w[32];
        const uint32_t ta = tbase + (uint32_t)(buf * 2 * GT) + ((uint32_t)(quad * 32) << 16) + (uint32_t)(cc * 32);
        tc::tmem_ld32(ta, v);
        tc::tmem_ld32(ta + GT, w);
        if (!live) continue;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          const int64_t gj = (int64_t)bj * GT + cc * 32 + q;
          if (gj >= ga.n || (bi == bj && gj > gi)) continue;
          double* t = ga.T + gi * ga.ldt + gj;
          double add = ga.alpha * ldexp((double)v[q] + (double)w[q], ga.E[gi] + ga.E[gj]);
          if (ga.D) add *= ga.D[gi * ga.ldt + gj];
          double val = first ? add : *t + add;
          if (last && gj == gi) val += ga.shift;
          *t = val;
          if (last && gj != gi) ga.T[gj * ga.ldt + gi] = val;
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(&tempty[buf])) : "memory");
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

PFN_cuTensorMapEncodeTiled_v12000 g_enc = nullptr;

// The three planes stacked as one (3 rows, kp) bf16 matrix: box {64, 128}, SWIZZLE_128B.
bool tmap_planes(CUtensorMap* m, const void* base, uint64_t rows3, uint64_t kp) {
  if (!g_enc) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return false;
    g_enc = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  if (((uintptr_t)base & 15) != 0 || (kp * 2) % 16 != 0) return false;
  cuuint64_t gdim[2] = {(cuuint64_t)kp, (cuuint64_t)rows3};
  cuuint64_t gstr[1] = {(cuuint64_t)kp * 2};
  cuuint32_t box[2] = {KA, GT};
  cuuint32_t es[2] = {1, 1};
  return g_enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), gdim, gstr, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

constexpr int kMaxDev = 64;
bool g_gram_attr[kMaxDev] = {};

}  // namespace

extern "C" {

// planes: 3 * rows_pad * kp bf16 workspace, rows_pad = rows rounded up to 128,
// kp = K rounded up to 64.  Rows beyond `rows` are zeroed.
int vmc_split_bf16x3(const float* X, int64_t rows, int64_t K, int64_t ldx, void* planes, int64_t rows_pad,
                     int64_t kp, int* row_exp, void* stream) {
  if (rows < 0 || K < 0 || ldx < K || rows_pad < rows || rows_pad % GT != 0 || kp < K || kp % KA != 0 ||
      (rows > 0 && (!X || !planes)) || (rows_pad > 0 && !row_exp))
    return VMC_ERR_ARGS;
  if (rows_pad == 0) return VMC_OK;
  k_row_exp<<<(unsigned)((rows_pad + 7) / 8), 256, 0, (cudaStream_t)stream>>>(X, rows, rows_pad, K, ldx, row_exp);
  VMC_CUDA_CHECK_LAUNCH();
  const int64_t n = rows_pad * kp;
  k_split3<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(X, rows, rows_pad, K, ldx, kp, row_exp,
                                                                          (__nv_bfloat16*)planes);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_sr_gram_tc(const void* planes, const int* row_exp, int64_t ns, int64_t rows_pad, int64_t kp, double alpha,
                   double* T, int64_t ldt, const double* D, double diag_shift, int accumulate, int* d_err,
                   void* stream) {
  if (ns <= 0 || rows_pad < ns || rows_pad % GT != 0 || kp <= 0 || kp % KA != 0 || ldt < ns || !planes || !T ||
      !d_err || !row_exp || ns > (1 << 30))
    return VMC_ERR_ARGS;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return VMC_ERR_CUDA;
  if (!g_gram_attr[dev]) {
    if (cudaFuncSetAttribute(k_gram_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize, GR_SMEM) != cudaSuccess)
      return VMC_ERR_CUDA;
    g_gram_attr[dev] = true;
  }
  CUtensorMap tm;
  if (!tmap_planes(&tm, planes, (uint64_t)(3 * rows_pad), (uint64_t)kp)) return VMC_ERR_UNSUPPORTED;
  const int nt = (int)(rows_pad / GT);
  GramArgs ga{T, ldt, D, row_exp, alpha, diag_shift, (int)ns, (int)rows_pad, (int)(kp / KA), accumulate};
  const int n_tiles = nt * (nt + 1) / 2;
  k_gram_bf16x3<<<(unsigned)n_tiles, GR_THREADS, GR_SMEM, (cudaStream_t)stream>>>(tm, ga, d_err);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

}  // extern "C"
