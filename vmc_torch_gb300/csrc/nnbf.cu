// Neural-network backflow (NNBF) amplitudes on GB300.
//
//   n = [up | dn] (2N spin-orbitals);  z0 = W0 n + b0;  h1 = gelu(z0);
//   h2 = gelu(W1 h1 + b1);  dM = out_w h2 + out_b  (2N x nf);
//   M = M_base + s * dM;  psi = det(M[ascending occupied rows])
//
// Evaluation pipeline over R "rows" (a row = one configuration to evaluate:
// a proposal during a sweep, a connected configuration during the local
// energy, or a walker's current configuration on refresh):
//   prep      : z0(row) from the walker's z0 plus the moved orbitals' W0
//               columns (or from scratch), h1 = gelu(z0) -> H1 (bf16 / fp64)
//   layer1    : H2 = gelu(H1 W1^T + b1)            tcgen05 GEMM 128x256x256
//   backflow  : A[row][pos] = M_base[r] + s (H2 out_w[r]^T + out_b[r]) for each
//               occupied orbital r at ascending position pos
//                                                   tcgen05 GEMM 128x256x256,
//               gather of occupied rows fused in the epilogue
//   logdet    : LU with partial pivoting, one warp per row, FP32 registers;
//               |det| accumulated as a normalised mantissa and an integer
//               exponent, combined in FP64; then Metropolis accept / local
//               energy term / refresh, fused.
// An FP64 twin of every stage (CUDA cores) gives the 1e-10 parity mode.
#include <cuda_bf16.h>
#include <cstdlib>
#include <utility>
#include <mutex>
#include <vector>
#include <cuda.h>
#include <cudaTypedefs.h>
#include "common.cuh"
#include "tc.cuh"

using namespace vmc;

namespace {

constexpr int HID = 256;
constexpr int TM = 128;          // rows per GEMM tile
constexpr int TN = 256;          // output columns per GEMM tile
constexpr int SMEM_A = TM * HID * 2;   // 64 KB
constexpr int SMEM_B = TN * HID * 2;   // 128 KB
constexpr int GEMM_SMEM = SMEM_A + SMEM_B + 1024 /*align*/ + 64 + 2 * TN * 4;

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ double gelu_d(double x) { return 0.5 * x * (1.0 + erf(x * 0.70710678118654752440)); }

// Proposal record (one per walker for sweeps): flag, packed moves, n moves, u_acc
struct __align__(16) PropRec {
  int flag;
  int moves;  // a0 | b0 << 8 | a1 << 16 | b1 << 24
  int nmov;
  float u_acc;
};

__device__ __forceinline__ void unpack_moves(const PropRec& r, int* a, int* b) {
  a[0] = r.moves & 0xff; b[0] = (r.moves >> 8) & 0xff; a[1] = (r.moves >> 16) & 0xff; b[1] = (r.moves >> 24) & 0xff;
}

// ---------------------------------------------------------------------------
// prep kernels (warp per row, lane handles 8 consecutive hidden units)
// ---------------------------------------------------------------------------
template <typename T> struct H1Store;
template <> struct H1Store<float> {
  static __device__ __forceinline__ void store(void* H1, int64_t row, int lane, const float* h) {
    __nv_bfloat162 p[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) p[q] = __floats2bfloat162_rn(h[2 * q], h[2 * q + 1]);
    reinterpret_cast<uint4*>((__nv_bfloat16*)H1 + row * HID)[lane] = *reinterpret_cast<uint4*>(p);
  }
};
template <> struct H1Store<double> {
  static __device__ __forceinline__ void store(void* H1, int64_t row, int lane, const double* h) {
    double* d = (double*)H1 + row * HID + lane * 8;
#pragma unroll
    for (int q = 0; q < 8; ++q) d[q] = h[q];
  }
};
template <typename T> __device__ __forceinline__ T gelu_t(T x);
template <> __device__ __forceinline__ float gelu_t<float>(float x) { return gelu_f(x); }
template <> __device__ __forceinline__ double gelu_t<double>(double x) { return gelu_d(x); }

// Sweep prep for edge e of sweep s: proposal, proposed occupation, moves, h1.
// Walkers [w_begin, w_end) of the B; arrays are indexed by the global walker.
// Row compaction (cnt non-null): a walker whose proposal changes it takes the
// next compact row of its group (atomic slot in *cnt, cleared before the
// launch); its hidden activations go to that row of H1, the row's walker
// (index within the group) to row_map and its proposed occupation to prop_c,
// so that the GEMMs and the LU run over the changed walkers only.  A row's
// arithmetic does not depend on which rows share its tile or warp, so the
// results do not depend on the slot order.
template <typename T>
__global__ void k_prep_sweep(int64_t B, int64_t w_begin, int64_t w_end, int N, const uint64_t* __restrict__ occ,
                             const int32_t* __restrict__ edges, int e, int s_local, int E, float hop_rate,
                             uint64_t seed, uint64_t sweep_idx, const float* __restrict__ rm,
                             const uint8_t* __restrict__ rb, const float* __restrict__ ra, const T* __restrict__ z0,
                             const T* __restrict__ w0t, uint64_t* __restrict__ prop_occ, PropRec* __restrict__ rec,
                             void* __restrict__ H1, int* __restrict__ cnt, int32_t* __restrict__ row_map,
                             uint64_t* __restrict__ prop_c, int* __restrict__ cnt_next) {
  const int lane = threadIdx.x & 31;
  // the counter of the next edge: its previous users (the launches of the
  // edge before this one) have finished, as they precede this launch
  if (cnt_next && blockIdx.x == 0 && threadIdx.x == 0) *cnt_next = 0;
  const int64_t w = w_begin + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (w >= w_end) return;
  uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  const int i = edges[2 * e], j = edges[2 * e + 1];
  const int xi = site_state(up, dn, i), xj = site_state(up, dn, j);
  PropRec r{0, 0, 0, 0.f};
  int a[2] = {0, 0}, b[2] = {0, 0};
  if (xi != xj) {
    float u_move, u_acc;
    int bit;
    if (rm) {
      size_t ridx = ((size_t)s_local * E + e) * (size_t)B + (size_t)w;
      u_move = rm[ridx]; bit = rb[ridx] & 1; u_acc = ra[ridx];
    } else {
      EdgeDraw d = draw_edge(seed, (uint64_t)w, sweep_idx, (uint32_t)e);
      u_move = d.u_move; bit = d.bit; u_acc = d.u_acc;
    }
    int ni, nj;
    propose_pair(xi, xj, u_move, bit, hop_rate, ni, nj);
    Moves mv = pair_moves(i, j, xi, ni, N);
    for (int q = 0; q < mv.n; ++q) { a[q] = mv.a[q]; b[q] = mv.b[q]; apply_move(up, dn, N, a[q], b[q]); }
    r.flag = 1;
    r.nmov = mv.n;
    r.moves = a[0] | (b[0] << 8) | (a[1] << 16) | (b[1] << 24);
    r.u_acc = u_acc;
  }
  if (lane == 0) {
    prop_occ[2 * w] = up;
    prop_occ[2 * w + 1] = dn;
    rec[w] = r;
  }
  if (!r.flag) return;
  int64_t hrow = w;
  if (cnt) {
    int slot = 0;
    if (lane == 0) {
      slot = atomicAdd(cnt, 1);
      row_map[w_begin + slot] = (int32_t)(w - w_begin);
      prop_c[2 * (w_begin + slot)] = up;
      prop_c[2 * (w_begin + slot) + 1] = dn;
    }
    hrow = w_begin + __shfl_sync(VMC_FULL_MASK, slot, 0);
  }
  T h[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) h[q] = z0[w * HID + lane * 8 + q];
  for (int m = 0; m < r.nmov; ++m) {
#pragma unroll
    for (int q = 0; q < 8; ++q) h[q] += w0t[b[m] * HID + lane * 8 + q] - w0t[a[m] * HID + lane * 8 + q];
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) h[q] = gelu_t<T>(h[q]);
  H1Store<T>::store(H1, hrow, lane, h);
}

// z0 = b0 + sum of W0 columns of the occupied orbitals (from scratch); h1 -> H1.
// A configuration with an occupation bit at or above N, or with other than nf
// electrons, sets *err = VMC_ERR_ARGS (its result is meaningless); the bits
// above N are dropped here so that W0 is never indexed past its 2N rows.
template <typename T>
__global__ void k_prep_fresh(int64_t R, int N, int nf, const uint64_t* __restrict__ occ, const T* __restrict__ w0t,
                             const T* __restrict__ b0, T* __restrict__ z0_out, void* __restrict__ H1,
                             int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= R) return;
  const uint64_t keep = bits_below(N);
  const uint64_t up_raw = occ[2 * w], dn_raw = occ[2 * w + 1];
  const uint64_t up = up_raw & keep, dn = dn_raw & keep;
  if (lane == 0 && err && (((up_raw | dn_raw) & ~keep) != 0ull || __popcll(up) + __popcll(dn) != nf))
    atomicExch(err, VMC_ERR_ARGS);
  T h[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) h[q] = b0[lane * 8 + q];
  for (int sp = 0; sp < 2; ++sp) {
    uint64_t m = sp ? dn : up;
    while (m) {
      const int site = __ffsll((long long)m) - 1;
      m &= m - 1;
      const int o = sp * N + site;
#pragma unroll
      for (int q = 0; q < 8; ++q) h[q] += w0t[o * HID + lane * 8 + q];
    }
  }
  if (z0_out) {
#pragma unroll
    for (int q = 0; q < 8; ++q) z0_out[w * HID + lane * 8 + q] = h[q];
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) h[q] = gelu_t<T>(h[q]);
  H1Store<T>::store(H1, w, lane, h);
}

// First layer of proposals that differ from the current configurations in a
// few orbitals (a learned move of k <= 4 hops changes at most 8): z0p = z0 +
// the W0 columns of the orbitals the proposal fills - those it empties, then
// GELU -> BF16 row.  z0 is the current configuration's cached first layer
// (rebuilt from scratch whenever the walkers are bound or refreshed).
template <typename T>
__global__ void k_prep_delta(int64_t R, int N, int nf, const uint64_t* __restrict__ occ,
                             const uint64_t* __restrict__ prop_occ, const T* __restrict__ z0,
                             const T* __restrict__ w0t, T* __restrict__ z0p, void* __restrict__ H1,
                             int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= R) return;
  const uint64_t keep = bits_below(N);
  const uint64_t pu_raw = prop_occ[2 * w], pd_raw = prop_occ[2 * w + 1];
  const uint64_t pu = pu_raw & keep, pd = pd_raw & keep;
  if (lane == 0 && err && (((pu_raw | pd_raw) & ~keep) != 0ull || __popcll(pu) + __popcll(pd) != nf))
    atomicExch(err, VMC_ERR_ARGS);
  const uint64_t cu = occ[2 * w] & keep, cd = occ[2 * w + 1] & keep;
  T h[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) h[q] = z0[w * HID + lane * 8 + q];
  for (int sp = 0; sp < 2; ++sp) {
    const uint64_t pm = sp ? pd : pu;
    uint64_t m = pm ^ (sp ? cd : cu);
    while (m) {
      const int site = __ffsll((long long)m) - 1;
      m &= m - 1;
      const T sg = ((pm >> site) & 1ull) ? T(1) : T(-1);
      const int o = sp * N + site;
#pragma unroll
      for (int q = 0; q < 8; ++q) h[q] += sg * w0t[o * HID + lane * 8 + q];
    }
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) z0p[w * HID + lane * 8 + q] = h[q];
#pragma unroll
  for (int q = 0; q < 8; ++q) h[q] = gelu_t<T>(h[q]);
  H1Store<T>::store(H1, w, lane, h);
}

// Local-energy prep: pair p = (walker, hop term) -> connected configuration
// occupation, coefficient, z0 + W0 column difference, h1.
template <typename T>
__global__ void k_prep_conn(int64_t P, int N, const int32_t* __restrict__ pairs /*(P,2) walker, term*/,
                            const uint64_t* __restrict__ occ, const int32_t* __restrict__ edges, double t,
                            const T* __restrict__ z0, const T* __restrict__ w0t, uint64_t* __restrict__ row_occ,
                            double* __restrict__ coeff, void* __restrict__ H1) {
  const int lane = threadIdx.x & 31;
  const int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= P) return;
  const int w = pairs[2 * p], term = pairs[2 * p + 1];
  const uint64_t up = occ[2 * (int64_t)w], dn = occ[2 * (int64_t)w + 1];
  const int e = term >> 1, s = (term & 1) ? 0 : 1;
  int i = edges[2 * e], j = edges[2 * e + 1];
  if (i > j) { int tt = i; i = j; j = tt; }
  const uint64_t m = s ? up : dn;
  const int oi = (int)((m >> i) & 1ull);
  const int base = s ? 0 : N;
  const int a = base + (oi ? i : j), b = base + (oi ? j : i);
  uint64_t eu = up, ed = dn;
  apply_move(eu, ed, N, a, b);
  if (lane == 0) {
    row_occ[2 * p] = eu;
    row_occ[2 * p + 1] = ed;
    coeff[p] = symmray_parity(up, dn, i, j, s) ? t : -t;
  }
  T h[8];
#pragma unroll
  for (int q = 0; q < 8; ++q)
    h[q] = gelu_t<T>(z0[(int64_t)w * HID + lane * 8 + q] + w0t[b * HID + lane * 8 + q] - w0t[a * HID + lane * 8 + q]);
  H1Store<T>::store(H1, p, lane, h);
}

// ---------------------------------------------------------------------------
// tcgen05 GEMM: D[128 x 256] = A[128 x 256] * B[256 x 256]^T, both K-major bf16
// in SWIZZLE_128B smem loaded by TMA; D in TMEM; fused epilogues.
// ---------------------------------------------------------------------------
enum { EPI_GELU_BF16 = 0, EPI_BACKFLOW = 1 };

struct EpiArgs {
  // EPI_GELU_BF16
  const float* bias;          // (256)
  __nv_bfloat16* out;         // (rows, 256)
  // EPI_BACKFLOW
  const uint64_t* row_occ;    // (rows, 2)
  const float* mbase;         // (n_orb, nf)
  const float* outb;          // (n_orb * nf)
  float* Aout;                // (rows, nf, nf)
  float scale;
  int n_sites, nf;
  // bounded wait for the operand tiles (0: 1 s); skip_loads issues no tile
  // load, so that the wait runs out with nothing in flight (self-test of the
  // timeout path, vmc_nnbf_hidden_layer)
  uint64_t wait_ns;
  int skip_loads;
  // compacted rows: the row count is *rows_dev (device), at most `rows`
  const int* rows_dev;
};

template <int EPI>
__global__ void __launch_bounds__(128, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int rows, EpiArgs ea,
              int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = sm;
  uint8_t* sB = sm + SMEM_A;
  uint64_t* bars = (uint64_t*)(sm + SMEM_A + SMEM_B);
  uint32_t* tslot = (uint32_t*)(bars + 2);
  int* sflag = (int*)(bars + 3);
  float* sc0 = (float*)(sm + SMEM_A + SMEM_B + 64);   // bias, or M_base slice
  float* sc1 = sc0 + TN;                               // out_b slice
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = blockIdx.x * TM;
  const int brow0 = blockIdx.y * TN;
  if (ea.rows_dev) {   // uniform over the CTA, before any barrier or allocation
    const int rr = *ea.rows_dev;
    if (row0 >= rr) return;
    rows = rows < rr ? rows : rr;
  }
  if (threadIdx.x == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
    *sflag = 1;
  }
  if (EPI == EPI_GELU_BF16) {
    for (int q = threadIdx.x; q < TN; q += blockDim.x) sc0[q] = ea.bias[brow0 + q];
  } else {
    for (int q = threadIdx.x; q < TN; q += blockDim.x) {
      sc0[q] = ea.mbase[brow0 + q];
      sc1[q] = ea.outb[brow0 + q];
    }
  }
  if (warp == 0) tc::tmem_alloc(tslot, 256);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;
  if (threadIdx.x == 0) {
    if (!ea.skip_loads) {
      tc::mbar_arrive_expect_tx(&bars[0], SMEM_A + SMEM_B);
#pragma unroll
      for (int j = 0; j < 4; ++j) tc::tma_load_2d(sA + j * (TM * 128), &tmA, &bars[0], j * 64, row0);
#pragma unroll
      for (int j = 0; j < 4; ++j) tc::tma_load_2d(sB + j * (TN * 128), &tmB, &bars[0], j * 64, brow0);
    }
    if (tc::mbar_wait(&bars[0], 0, ea.wait_ns ? ea.wait_ns : 1000000000ull)) {
      tc::fence_after_sync();
      constexpr uint32_t idesc = tc::idesc_bf16_f32(TM, TN);
#pragma unroll
      for (int ks = 0; ks < HID / 16; ++ks) {
        const int j = ks >> 2, kk = ks & 3;
        const uint64_t ad = tc::sdesc_sw128(tc::smem_u32(sA + j * (TM * 128)) + kk * 32);
        const uint64_t bd = tc::sdesc_sw128(tc::smem_u32(sB + j * (TN * 128)) + kk * 32);
        tc::mma_bf16(tbase, ad, bd, idesc, ks > 0 ? 1u : 0u);
      }
      tc::mma_commit(&bars[1]);
    } else {
      *sflag = 0;
      atomicExch(err, VMC_ERR_TIMEOUT);
    }
  }
  __syncthreads();
  if (*sflag) {
    const bool done = tc::mbar_wait(&bars[1], 0);
    tc::fence_after_sync();
    if (!done) {
      if (lane == 0) atomicExch(err, VMC_ERR_TIMEOUT);
    } else {
      const int r = warp * 32 + lane;
      const int64_t row = (int64_t)row0 + r;
      const bool live = row < rows;
      uint64_t up = 0, dn = 0;
      if (EPI == EPI_BACKFLOW && live) { up = ea.row_occ[2 * row]; dn = ea.row_occ[2 * row + 1]; }
#pragma unroll 1
      for (int cc = 0; cc < TN / 32; ++cc) {
        float v[32];
        tc::tmem_ld32(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cc * 32), v);
        if (!live) continue;
        if (EPI == EPI_GELU_BF16) {
          const int n0 = brow0 + cc * 32;
          uint32_t pk[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            __nv_bfloat162 h2 = __floats2bfloat162_rn(gelu_f(v[2 * q] + sc0[cc * 32 + 2 * q]),
                                                      gelu_f(v[2 * q + 1] + sc0[cc * 32 + 2 * q + 1]));
            pk[q] = *reinterpret_cast<uint32_t*>(&h2);
          }
          uint4* dst = reinterpret_cast<uint4*>(ea.out + row * HID + n0);
#pragma unroll
          for (int q = 0; q < 4; ++q) dst[q] = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
        } else {
          const int nf = ea.nf;
          const int col = brow0 + cc * 32;          // flat output index = orbital * nf + c
          const int orb = col / nf, c0 = col - orb * nf;
          const int N = ea.n_sites;
          if (!orb_occupied(up, dn, N, orb)) continue;
          const int pos = orb_prefix(up, dn, N, orb);
          if (pos >= nf) continue;
          float* dst = ea.Aout + ((size_t)row * nf + pos) * nf + c0;
          const float* mb = sc0 + cc * 32;   // == M_base[orb][c0 ..], staged
          const float* ob = sc1 + cc * 32;   // == out_b[orb * nf + c0 ..], staged
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            float4 o;
            o.x = mb[4 * q + 0] + ea.scale * (v[4 * q + 0] + ob[4 * q + 0]);
            o.y = mb[4 * q + 1] + ea.scale * (v[4 * q + 1] + ob[4 * q + 1]);
            o.z = mb[4 * q + 2] + ea.scale * (v[4 * q + 2] + ob[4 * q + 2]);
            o.w = mb[4 * q + 3] + ea.scale * (v[4 * q + 3] + ob[4 * q + 3]);
            reinterpret_cast<float4*>(dst)[q] = o;
          }
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

// ---------------------------------------------------------------------------
// Persistent backflow GEMM: one CTA per SM walks a contiguous range of work
// items (orbital group g, walker tile t) in g-major order.  The out_w rows of
// group g (256 x 256 bf16, 128 KB) stay resident in shared memory while the
// hidden-activation tiles (128 x 256 bf16) stream through a 4-stage pipeline
// (one stage per 64-wide K atom).  Warp roles: warp 0 = TMA producer, warp 1 =
// MMA issuer (one thread), warps 2..5 = epilogue (TMEM lane quadrants 2,3,0,1).
// Two TMEM accumulators (2 x 256 columns) let the epilogue of item i overlap
// the MMAs of item i+1.
// ---------------------------------------------------------------------------
constexpr int PB_THREADS = 192;
constexpr int PB_SMEM = SMEM_A + SMEM_B + 1024 + 256 + 2 * TN * 4;

struct PBArgs {
  const uint64_t* row_occ;  // (R, 2)
  const float* mbase;       // (n_orb * nf) flat
  const float* outb;        // (n_orb * nf)
  float* Aout;              // (R, nf, nf)
  float scale;
  int n_sites, nf, R, n_tiles, n_items;
  // compacted rows: the row count is clamp(*rows_dev - rows_off, 0, R) (device)
  const int* rows_dev;
  int64_t rows_off;
};

__global__ void __launch_bounds__(PB_THREADS, 1)
    k_backflow_persistent(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, PBArgs pa,
                          int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = sm;                 // 4 atoms x 16 KB
  uint8_t* sB = sm + SMEM_A;        // 4 atoms x 32 KB
  uint64_t* bar = (uint64_t*)(sm + SMEM_A + SMEM_B);
  uint64_t* bfull = bar + 0;
  uint64_t* bempty = bar + 1;
  uint64_t* afull = bar + 2;    // [4]
  uint64_t* aempty = bar + 6;   // [4]
  uint64_t* tfull = bar + 10;   // [2]
  uint64_t* tempty = bar + 12;  // [2]
  uint32_t* tslot = (uint32_t*)(bar + 14);
  volatile int* abort_flag = (volatile int*)(bar + 15);
  float* cM = (float*)(sm + SMEM_A + SMEM_B + 256);
  float* cO = cM + TN;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int R = pa.R, n_tiles = pa.n_tiles, n_items = pa.n_items;
  if (pa.rows_dev) {   // the same value in every thread: all roles walk the same items
    const int64_t rr = (int64_t)*pa.rows_dev - pa.rows_off;
    R = rr < 0 ? 0 : (rr < R ? (int)rr : R);
    const int n_groups = pa.n_items / pa.n_tiles;
    n_tiles = (R + TM - 1) / TM;
    n_items = n_groups * n_tiles;
  }
  const int per = (n_items + gridDim.x - 1) / gridDim.x;
  const int it0 = blockIdx.x * per;
  const int it1 = min(n_items, it0 + per);
  if (threadIdx.x == 0) {
    tc::mbar_init(bfull, 1);
    tc::mbar_init(bempty, 1);
    for (int j = 0; j < 4; ++j) { tc::mbar_init(&afull[j], 1); tc::mbar_init(&aempty[j], 1); }
    for (int b = 0; b < 2; ++b) { tc::mbar_init(&tfull[b], 1); tc::mbar_init(&tempty[b], 4); }
    *abort_flag = 0;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
  }
  if (warp == 0) tc::tmem_alloc(tslot, 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;
  if (it0 < it1) {
    if (warp == 0) {
      if (lane == 0) {  // ---------------- TMA producer ----------------
        int cur_g = -1, ng = 0;
        for (int it = it0, i = 0; it < it1 && !*abort_flag; ++it, ++i) {
          const int g = it / n_tiles, t = it - g * n_tiles;
          if (g != cur_g) {
            if (cur_g >= 0 && !tc::mbar_wait(bempty, (ng - 1) & 1)) { *abort_flag = 1; atomicExch(err, VMC_ERR_TIMEOUT); break; }
            tc::mbar_arrive_expect_tx(bfull, SMEM_B);
            for (int j = 0; j < 4; ++j) tc::tma_load_2d(sB + j * (TN * 128), &tmB, bfull, j * 64, g * TN);
            cur_g = g;
            ++ng;
          }
          for (int j = 0; j < 4; ++j) {
            if (i > 0 && !tc::mbar_wait(&aempty[j], (i - 1) & 1)) { *abort_flag = 1; atomicExch(err, VMC_ERR_TIMEOUT); break; }
            tc::mbar_arrive_expect_tx(&afull[j], TM * 128);
            tc::tma_load_2d(sA + j * (TM * 128), &tmA, &afull[j], j * 64, t * TM);
          }
        }
      }
    } else if (warp == 1) {
      if (lane == 0) {  // ---------------- MMA issuer ----------------
        constexpr uint32_t idesc = tc::idesc_bf16_f32(TM, TN);
        int cur_g = -1, ng = 0;
        for (int it = it0, i = 0; it < it1 && !*abort_flag; ++it, ++i) {
          const int g = it / n_tiles;
          if (g != cur_g) {
            if (!tc::mbar_wait(bfull, ng & 1)) { *abort_flag = 1; atomicExch(err, VMC_ERR_TIMEOUT); break; }
            cur_g = g;
            ++ng;
          }
          const int buf = i & 1;
          if (i >= 2 && !tc::mbar_wait(&tempty[buf], ((i >> 1) - 1) & 1)) { *abort_flag = 1; atomicExch(err, VMC_ERR_TIMEOUT); break; }
          tc::fence_after_sync();
          const uint32_t dt = tbase + (uint32_t)(buf * TN);
          bool ok = true;
          for (int j = 0; j < 4; ++j) {
            if (!tc::mbar_wait(&afull[j], i & 1)) { ok = false; break; }
            tc::fence_after_sync();
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint64_t ad = tc::sdesc_sw128(tc::smem_u32(sA + j * (TM * 128)) + kk * 32);
              const uint64_t bd = tc::sdesc_sw128(tc::smem_u32(sB + j * (TN * 128)) + kk * 32);
              tc::mma_bf16(dt, ad, bd, idesc, (j | kk) ? 1u : 0u);
            }
            tc::mma_commit(&aempty[j]);
          }
          if (!ok) { *abort_flag = 1; atomicExch(err, VMC_ERR_TIMEOUT); break; }
          tc::mma_commit(&tfull[buf]);
          const int gn = (it + 1 < it1) ? (it + 1) / n_tiles : -2;
          if (gn != g) tc::mma_commit(bempty);  // B of group g no longer needed
        }
      }
    } else {  // ---------------- epilogue warps 2..5 ----------------
      const int quad = warp & 3;
      const int et = threadIdx.x - 64;   // 0..127
      int cur_g = -1;
      for (int it = it0, i = 0; it < it1; ++it, ++i) {
        const int g = it / n_tiles, t = it - g * n_tiles;
        if (g != cur_g) {
          asm volatile("bar.sync 1, 128;" ::: "memory");
          for (int q = et; q < TN; q += 128) { cM[q] = pa.mbase[g * TN + q]; cO[q] = pa.outb[g * TN + q]; }
          asm volatile("bar.sync 1, 128;" ::: "memory");
          cur_g = g;
        }
        const int buf = i & 1;
        bool ok = tc::mbar_wait(&tfull[buf], (i >> 1) & 1);
        ok = __all_sync(VMC_FULL_MASK, ok);
        if (!ok) { if (lane == 0) { *abort_flag = 1; atomicExch(err, VMC_ERR_TIMEOUT); } break; }
        tc::fence_after_sync();
        const int64_t row = (int64_t)t * TM + quad * 32 + lane;
        const bool live = row < R;
        uint64_t up = 0, dn = 0;
        if (live) { up = pa.row_occ[2 * row]; dn = pa.row_occ[2 * row + 1]; }
        const int nf = pa.nf, N = pa.n_sites;
#pragma unroll 1
        for (int cc = 0; cc < TN / 32; ++cc) {
          float v[32];
          tc::tmem_ld32(tbase + (uint32_t)(buf * TN) + ((uint32_t)(quad * 32) << 16) + (uint32_t)(cc * 32), v);
          if (!live) continue;
          const int col = g * TN + cc * 32;
          const int orb = col / nf, c0 = col - orb * nf;
          if (!orb_occupied(up, dn, N, orb)) continue;
          const int pos = orb_prefix(up, dn, N, orb);
          if (pos >= nf) continue;
          float* dst = pa.Aout + ((size_t)row * nf + pos) * nf + c0;
          const float* mb = cM + cc * 32;
          const float* ob = cO + cc * 32;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const float4 m4 = reinterpret_cast<const float4*>(mb)[q];
            const float4 o4 = reinterpret_cast<const float4*>(ob)[q];
            float4 o;
            o.x = m4.x + pa.scale * (v[4 * q + 0] + o4.x);
            o.y = m4.y + pa.scale * (v[4 * q + 1] + o4.y);
            o.z = m4.z + pa.scale * (v[4 * q + 2] + o4.z);
            o.w = m4.w + pa.scale * (v[4 * q + 3] + o4.w);
            reinterpret_cast<float4*>(dst)[q] = o;
          }
        }
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(&tempty[buf])) : "memory");
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

// ---------------------------------------------------------------------------
// FP64 twins (CUDA cores): layer 1 and backflow, one block per row
// ---------------------------------------------------------------------------
__global__ void k_layer1_f64(int64_t R, const double* __restrict__ H1, const double* __restrict__ W1,
                             const double* __restrict__ b1, double* __restrict__ H2) {
  __shared__ double h[HID];
  const int64_t row = blockIdx.x;
  h[threadIdx.x] = H1[row * HID + threadIdx.x];
  __syncthreads();
  const int n = threadIdx.x;
  double acc = b1[n];
  for (int k = 0; k < HID; ++k) acc = fma(W1[(size_t)n * HID + k], h[k], acc);
  H2[row * HID + n] = gelu_d(acc);
}

__global__ void k_backflow_f64(int64_t R, int N, int nf, const uint64_t* __restrict__ row_occ,
                               const double* __restrict__ H2, const double* __restrict__ outw,
                               const double* __restrict__ outb, const double* __restrict__ mbase, double scale,
                               double* __restrict__ A) {
  __shared__ double h[HID];
  __shared__ int orbs[64];
  const int64_t row = blockIdx.x;
  const uint64_t up = row_occ[2 * row], dn = row_occ[2 * row + 1];
  h[threadIdx.x] = H2[row * HID + threadIdx.x];
  if (threadIdx.x < 2 * N && orb_occupied(up, dn, N, threadIdx.x)) {
    int pos = orb_prefix(up, dn, N, threadIdx.x);
    if (pos < 64) orbs[pos] = threadIdx.x;
  }
  __syncthreads();
  const bool ok = (__popcll(up) + __popcll(dn)) == nf;
  for (int idx = threadIdx.x; idx < nf * nf; idx += blockDim.x) {
    const int pos = idx / nf, c = idx - pos * nf;
    double val = 0.0;
    if (ok) {
      const int o = orbs[pos];
      const double* wr = outw + ((size_t)o * nf + c) * HID;
      double acc = outb[(size_t)o * nf + c];
      for (int k = 0; k < HID; ++k) acc = fma(wr[k], h[k], acc);
      val = mbase[(size_t)o * nf + c] + scale * acc;
    }
    A[(size_t)row * nf * nf + idx] = val;
  }
}

// ---------------------------------------------------------------------------
// log|det| + sign, one warp per row
// ---------------------------------------------------------------------------
struct Det { double logabs; double sign; };

// FP32 registers, rows lane and lane+32, no physical row swaps: a retired-row
// mask U tracks the pivots; the permutation parity is accumulated as the
// number of unretired rows below each pivot.
//
// Code-size-aware schedule: the elimination runs in NF/16 phases of 16 steps.
// Within a phase of width W the live columns of every row are kept at
// register indices 0..W-1, so the step bodies have only compile-time register
// indices and run in a runtime loop; each phase is a separate instantiation
// with W = NF, NF-16, ... (work per step ~ 2 W FMAs instead of the fixed
// 2 NF).  Columns are held in pairs.  The loop body is two pivot steps: the
// first eliminates column 0 and updates the pairs in place with the packed
// FP32 FMA (two correctly rounded FMAs per instruction: results equal the
// scalar form bit for bit); the second eliminates column 1 and writes every
// pair one slot lower (pair[i-1] = pair[i] - f * pivot[i]) with scalar FMAs,
// so the live window stays at the front without register moves.  Packing the
// shifting step too, or unrolling four steps, raises the register count past
// 168 (3 CTAs of 4 warps per SM) or the loop body's code size, and measured
// slower end to end.
// Register layouts of the elimination: LU_FULL = rows lane and lane + 32 (of
// a 64-row matrix; row lane of a 32-row one); LU_PAIRED = two matrices a
// warp, lanes 16 h .. 16 h + 15 holding two live rows each of matrix h (see
// warp_logdet_f32_pair).
enum { LU_FULL = 0, LU_PAIRED = 1 };

template <int NF>
struct LuRegs {
  float2 a[NF / 32][NF / 2];
  uint64_t U;
  float mant;
  int expo, neg;   // neg bit 0: sign of the determinant; bit 1: a non-finite pivot was met
  bool ok;
  unsigned key;   // pivot key of the next step (computed one step ahead)
  // paired layout: original rows of the two register rows, their bits, and
  // the half (matrix) the lane works on
  int prow_of[2];
  uint64_t pbit[2];
  int half;
};

// Resident 4-warp CTAs per SM that the LU kernel's register budget is held
// to (168 registers, no spills).
constexpr int LU_MIN_CTAS = 3;
template <int E> __device__ __forceinline__ float lu_el(const float2& v) { return E ? v.y : v.x; }

// Pivot key: max |a| over unretired rows by a single warp reduction on a packed
// key (|a| bits with the low 6 mantissa bits replaced by 63 - row: larger
// magnitude wins, ties -> smaller row).  The 6 dropped bits only matter for
// magnitudes equal to 2^-17 relative, where either choice is a valid pivot.
// The pivot column is element E of pair P; LM is the register layout.  In
// the paired layout each half reduces its own matrix's keys (two warp
// reductions, the other half's keys masked to 0).
template <int NF, int R, int P, int E, int LM>
__device__ __forceinline__ unsigned lu_pivot_key(const LuRegs<NF>& S, int lane) {
  unsigned key = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int row = LM == LU_PAIRED ? S.prow_of[r] : lane + 32 * r;
    // live test: the precomputed bit, or the 32-bit word of the lane's row
    const bool live = LM == LU_PAIRED ? (S.U & S.pbit[r]) != 0ull
                                      : ((((r == 0) ? (unsigned)S.U : (unsigned)(S.U >> 32)) >> lane) & 1u) != 0u;
    if (live) {
      const unsigned kb = (__float_as_uint(fabsf(lu_el<E>(S.a[r][P]))) & ~63u) | (unsigned)(63 - row);
      key = kb > key ? kb : key;
    }
  }
  if constexpr (LM == LU_PAIRED) {
    const unsigned k0 = __reduce_max_sync(VMC_FULL_MASK, S.half ? 0u : key);
    const unsigned k1 = __reduce_max_sync(VMC_FULL_MASK, S.half ? key : 0u);
    return S.half ? k1 : k0;
  }
  return __reduce_max_sync(VMC_FULL_MASK, key);
}

// Bookkeeping of one pivot step on the pivot value pv read back from the
// pivot row: validity, sign, retired mask, |det| as mantissa in [1, 2) times
// 2^expo (normal floats; pivots are O(1e-3..1e1) here, far from the FP32
// limits).  Returns 1 / pv.
template <int NF>
__device__ __forceinline__ float lu_pivot_update(LuRegs<NF>& S, unsigned key, int p, float pv) {
  const float best = __uint_as_float(key & ~63u);
  const bool pvalid = key != 0u && (best > 0.0f) && isfinite(best);
  // NaN and Inf keys order above every finite one, so a non-finite entry of
  // the pivot column is always the candidate that is seen here
  if (!pvalid) { S.ok = false; S.neg |= (key != 0u && !isfinite(best)) ? 2 : 0; pv = 1.0f; }
  S.neg ^= (pv < 0.0f);
  S.neg ^= __popcll(S.U & ((1ull << p) - 1ull)) & 1;
  S.U &= ~(1ull << p);
  const float m = S.mant * fabsf(pv);
  const unsigned mb = __float_as_uint(m);
  S.expo += (int)((mb >> 23) & 255u) - 127;
  S.mant = __uint_as_float((mb & 0x007FFFFFu) | 0x3F800000u);
  // elimination multipliers only: the hardware reciprocal (relative error
  // ~2^-23) is as accurate as the multiplier's own rounding; |det| uses pv
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(pv));
  return r;
}

// Pivot row (H pairs of the owning lane's register row) -> shared memory.
template <int H>
__device__ __forceinline__ void lu_store_row(const float2* a, float* prow) {
#pragma unroll
  for (int q = 0; q < H / 2; ++q)
    reinterpret_cast<float4*>(prow)[q] = make_float4(a[2 * q].x, a[2 * q].y, a[2 * q + 1].x, a[2 * q + 1].y);
}

// pair[i] -= f * pivot[i] in place for pairs I0 <= i < H, packed FMAs, the
// pivot row streamed from shared memory (16-byte loads where aligned).
// pair[i] -= f * pivot[i] in place for pairs 1 <= i < H, packed FMAs, the
// pivot row streamed from shared memory (16-byte loads where aligned).
template <int R, int H, int NP>
__device__ __forceinline__ void lu_update_inplace(float2 (*a)[NP], const float* prow, const float (&f)[R]) {
  {
    const float2 p0 = reinterpret_cast<const float2*>(prow)[1];
#pragma unroll
    for (int r = 0; r < R; ++r) a[r][1] = __ffma2_rn(make_float2(-f[r], -f[r]), p0, a[r][1]);
  }
#pragma unroll
  for (int q = 1; q < H / 2; ++q) {
    const float4 t4 = reinterpret_cast<const float4*>(prow)[q];
    const float2 p0 = make_float2(t4.x, t4.y), p1 = make_float2(t4.z, t4.w);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const float2 nf2 = make_float2(-f[r], -f[r]);
      a[r][2 * q] = __ffma2_rn(nf2, p0, a[r][2 * q]);
      a[r][2 * q + 1] = __ffma2_rn(nf2, p1, a[r][2 * q + 1]);
    }
  }
}

// pair[i-1] = pair[i] - f * pivot[i] for pairs 2 <= i < H, scalar FMAs (the
// caller has done pair 1 first: it carries the next pivot column).
template <int R, int H, int NP>
__device__ __forceinline__ void lu_update_shift(float2 (*a)[NP], const float* prow, const float (&f)[R]) {
#pragma unroll
  for (int q = 1; q < H / 2; ++q) {
    const float4 t4 = reinterpret_cast<const float4*>(prow)[q];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      a[r][2 * q - 1].x = fmaf(-f[r], t4.x, a[r][2 * q].x);
      a[r][2 * q - 1].y = fmaf(-f[r], t4.y, a[r][2 * q].y);
      a[r][2 * q].x = fmaf(-f[r], t4.z, a[r][2 * q + 1].x);
      a[r][2 * q].y = fmaf(-f[r], t4.w, a[r][2 * q + 1].y);
    }
  }
}

// One pivot step on column K (0 or 1) of a phase of width W.  The next pivot
// column is updated first so that its key reduction overlaps the rest.  The
// pivot row goes through shared slot K of the warp's two 64-float slots: a
// slot is rewritten two steps later, after every lane has passed the barrier
// of the step in between, so one barrier per step orders both the write
// before the reads and the reads before the next write.
template <int NF, int R, int W, int K, int LM>
__device__ __forceinline__ void lu_step(LuRegs<NF>& S, float* prow2, int lane) {
  constexpr int H = W / 2;
  // paired layout: each half's pivot row in its own 32-float part of the slot
  float* prow = prow2 + 64 * K + (LM == LU_PAIRED ? 32 * S.half : 0);
  const unsigned key = S.key;
  const int p = 63 - (int)(key & 63u);
  // pivot row -> shared memory (warp-uniform branch on the register row)
  if (LM == LU_PAIRED) {
    if (S.prow_of[0] == p) lu_store_row<H>(S.a[0], prow);
    else if (S.prow_of[1] == p) lu_store_row<H>(S.a[R - 1], prow);
  } else if (R > 1 && (p >> 5)) {
    if ((p & 31) == lane) lu_store_row<H>(S.a[R - 1], prow);
  } else {
    if ((p & 31) == lane) lu_store_row<H>(S.a[0], prow);
  }
  __syncwarp();
  const float ipv = lu_pivot_update<NF>(S, key, p, prow[K]);
  float f[R];
#pragma unroll
  for (int r = 0; r < R; ++r) f[r] = lu_el<K>(S.a[r][0]) * ipv;   // retired rows keep updating harmlessly
  if constexpr (K == 0) {
    const float pn = prow[1];
#pragma unroll
    for (int r = 0; r < R; ++r) S.a[r][0].y = fmaf(-f[r], pn, S.a[r][0].y);
    S.key = lu_pivot_key<NF, R, 0, 1, LM>(S, lane);
    lu_update_inplace<R, H>(S.a, prow, f);
  } else {
    const float2 pn = reinterpret_cast<const float2*>(prow)[1];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      S.a[r][0].x = fmaf(-f[r], pn.x, S.a[r][1].x);
      S.a[r][0].y = fmaf(-f[r], pn.y, S.a[r][1].y);
    }
    S.key = lu_pivot_key<NF, R, 0, 0, LM>(S, lane);
    lu_update_shift<R, H>(S.a, prow, f);
  }
}

// 16 pivot steps of width W in register layout LM.
template <int NF, int R, int W, int LM>
__device__ __forceinline__ void lu_phase(LuRegs<NF>& S, float* prow, int lane) {
#pragma unroll 1
  for (int t = 0; t < 8; ++t) {
    lu_step<NF, R, W, 0, LM>(S, prow, lane);
    lu_step<NF, R, W, 1, LM>(S, prow, lane);
  }
}

// After 32 pivot steps of a 64-row matrix exactly 32 rows are retired.  The
// live rows move into register slot 0, one per lane in ascending row order
// (lane L takes the L-th live row), ready to be parked and regrouped into the
// paired layout.  Returns the original row now held by the lane.
template <int W>
__device__ __forceinline__ int lu_compact(LuRegs<64>& S, int lane) {
  uint64_t m = S.U;
  for (int i = 0; i < lane; ++i) m &= m - 1ull;  // drop the lane's lower live rows
  const int src = m ? __ffsll((long long)m) - 1 : lane;  // m == 0 only after a failed pivot (result discarded)
  const int sl = src & 31;
  const bool s1 = (src >> 5) != 0;
#pragma unroll
  for (int i = 0; i < W / 2; ++i) {
    const float x0 = __shfl_sync(VMC_FULL_MASK, S.a[0][i].x, sl);
    const float y0 = __shfl_sync(VMC_FULL_MASK, S.a[0][i].y, sl);
    const float x1 = __shfl_sync(VMC_FULL_MASK, S.a[1][i].x, sl);
    const float y1 = __shfl_sync(VMC_FULL_MASK, S.a[1][i].y, sl);
    S.a[0][i] = s1 ? make_float2(x1, y1) : make_float2(x0, y0);
  }
  return src;
}

template <int NF>
__device__ __forceinline__ void lu_load(LuRegs<NF>& S, const float* __restrict__ A, int lane) {
  constexpr int R = NF / 32;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float4* src = reinterpret_cast<const float4*>(A + (size_t)(lane + 32 * r) * NF);
#pragma unroll
    for (int q = 0; q < NF / 4; ++q) {
      float4 t = src[q];
      S.a[r][2 * q] = make_float2(t.x, t.y);
      S.a[r][2 * q + 1] = make_float2(t.z, t.w);
    }
  }
  S.U = (NF == 64) ? ~0ull : ((1ull << NF) - 1ull);
  S.mant = 1.0f;
  S.expo = 0;
  S.neg = 0;
  S.ok = true;
  S.key = lu_pivot_key<NF, R, 0, 0, LU_FULL>(S, lane);
}

// Singular matrices give sign 0 and log|det| = -inf; a non-finite entry
// (NaN or Inf parameters upstream) gives NaN for both, like the reference's
// NaN amplitude.
__device__ __forceinline__ Det lu_det(bool ok, float mant, int expo, int neg) {
  Det d;
  if (!ok && (neg & 2)) {
    d.logabs = __longlong_as_double(0x7ff8000000000000ll);
    d.sign = d.logabs;
  } else if (ok) {
    // mantissa in [1, 2): FP32 log is accurate to ~1e-7 absolute; the exponent
    // part is exact; only the final sum is FP64 (FP64 pipes are scarce on GB300)
    d.logabs = (double)logf(mant) + (double)expo * 0.69314718055994530942;
    d.sign = neg ? -1.0 : 1.0;
  } else {
    d.logabs = -INFINITY;
    d.sign = 0.0;
  }
  return d;
}

// One 32 x 32 matrix a warp (64 x 64 matrices go two a warp through
// warp_logdet_f32_pair).
template <int NF>
__device__ __forceinline__ Det warp_logdet_f32(const float* __restrict__ A, float* prow) {
  static_assert(NF == 32, "one-matrix path: NF = 32");
  const int lane = threadIdx.x & 31;
  LuRegs<NF> S;
  lu_load<NF>(S, A, lane);
  lu_phase<NF, 1, NF, LU_FULL>(S, prow, lane);
  lu_phase<NF, 1, NF - 16, LU_FULL>(S, prow, lane);
  return lu_det(S.ok, S.mant, S.expo, S.neg);
}

// Scalar LU state word of a parked remainder: bit 0 determinant sign, bit 1
// ok, bit 2 non-finite pivot met.
__device__ __forceinline__ uint32_t park_flags(int neg, bool ok) {
  return (uint32_t)(neg & 1) | ((uint32_t)ok << 1) | ((uint32_t)(neg & 2) << 1);
}
__device__ __forceinline__ int unpark_neg(uint32_t w) { return (int)((w & 1u) | ((w >> 1) & 2u)); }

// Last 32 pivot steps of a 64 x 64 matrix whose first 32 ran on this warp
// (S after lu_compact, lane L holding live row L, orow its original row),
// together with a partner matrix when one is given.  Partner (psw != null):
// the 32 x 32 remainder parked at park (lane-major float4 rows) with its
// original rows in psw[0..31] and scalar state in psw[32..36].  The warp
// splits into halves: half 0 (lanes 0..15) carries live rows L and L + 16 of
// the own matrix, half 1 those of the partner (or of the own matrix again if
// there is none), and both tails run as one instruction stream.  A row's
// updates are the same FMAs in every layout and the pivot keys carry the
// original row numbers, so a matrix's result does not depend on its partner
// or on the pairing.  d0: own matrix, d1: partner.
__device__ __forceinline__ void lu_tail_pair(LuRegs<64>& S, int orow, const float4* park, const uint32_t* psw,
                                             float* prow, Det& d0, Det& d1) {
  const int lane = threadIdx.x & 31;
  const int half = lane >> 4;
  const int i = lane & 15;
  float2 t[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) t[k] = make_float2(__shfl_xor_sync(VMC_FULL_MASK, S.a[0][k].x, 16),
                                                  __shfl_xor_sync(VMC_FULL_MASK, S.a[0][k].y, 16));
  const int orow_x = __shfl_xor_sync(VMC_FULL_MASK, orow, 16);
  if (half == 0) {
#pragma unroll
    for (int k = 0; k < 16; ++k) S.a[1][k] = t[k];
    S.prow_of[0] = orow;
    S.prow_of[1] = orow_x;
  } else if (psw == nullptr) {
#pragma unroll
    for (int k = 0; k < 16; ++k) { S.a[1][k] = S.a[0][k]; S.a[0][k] = t[k]; }
    S.prow_of[0] = orow_x;
    S.prow_of[1] = orow;
  } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 v0 = __ldcg(park + q * 32 + i), v1 = __ldcg(park + q * 32 + i + 16);
      S.a[0][2 * q] = make_float2(v0.x, v0.y);
      S.a[0][2 * q + 1] = make_float2(v0.z, v0.w);
      S.a[1][2 * q] = make_float2(v1.x, v1.y);
      S.a[1][2 * q + 1] = make_float2(v1.z, v1.w);
    }
    S.prow_of[0] = (int)psw[i];
    S.prow_of[1] = (int)psw[i + 16];
    S.U = (uint64_t)psw[32] | ((uint64_t)psw[33] << 32);
    S.mant = __uint_as_float(psw[34]);
    S.expo = (int)psw[35];
    S.neg = unpark_neg(psw[36]);
    S.ok = (psw[36] >> 1) & 1u;
  }
  S.half = half;
  S.pbit[0] = 1ull << S.prow_of[0];
  S.pbit[1] = 1ull << S.prow_of[1];
  S.key = lu_pivot_key<64, 2, 0, 0, LU_PAIRED>(S, lane);
  lu_phase<64, 2, 32, LU_PAIRED>(S, prow, lane);
  lu_phase<64, 2, 16, LU_PAIRED>(S, prow, lane);
  // each half's state -> both results
  const float mo = __shfl_xor_sync(VMC_FULL_MASK, S.mant, 16);
  const int eo = __shfl_xor_sync(VMC_FULL_MASK, S.expo, 16);
  const int no = __shfl_xor_sync(VMC_FULL_MASK, S.neg, 16);
  const bool oo = __shfl_xor_sync(VMC_FULL_MASK, (int)S.ok, 16) != 0;
  const Det mine = lu_det(S.ok, S.mant, S.expo, S.neg), other = lu_det(oo, mo, eo, no);
  d0 = half ? other : mine;
  d1 = half ? mine : other;
}

// Two 64 x 64 matrices on one warp.  Each runs its first 32 pivot steps in
// the full layout, then parks its 32 x 32 remainder in its own first 4 KB
// (L2; the warp has consumed those rows) and its scalar state in the warp's
// shared words, so nothing but indices stays live from one matrix to the
// next.  The remainders then share the warp: half h (lanes 16 h .. 16 h + 15)
// reloads live rows i and i + 16 of matrix h, and the last 32 steps of both
// run as one instruction stream.  A row's updates are the same FMAs in either
// layout and the pivot keys carry the original row numbers, so a matrix's
// result does not depend on its partner or on the pairing.  The matrices
// are rows sw[38 + h] of A; with nm = 1 both halves carry matrix 0 and the
// second result is unused.
__device__ __forceinline__ void warp_logdet_f32_pair(float* A, float* prow, uint32_t* sw, int nm, Det& d0,
                                                     Det& d1) {
  const int lane = threadIdx.x & 31;
  LuRegs<64> S;
#pragma unroll 1
  for (int m = 0; m < nm; ++m) {
    float* Am = A + (size_t)sw[38 + m] * 4096;
    lu_load<64>(S, Am, lane);
    lu_phase<64, 2, 64, LU_FULL>(S, prow, lane);
    lu_phase<64, 2, 48, LU_FULL>(S, prow, lane);
    const int orow = lu_compact<32>(S, lane);
    __syncwarp();  // every lane's loads of the matrix precede the parking stores
    float4* park = reinterpret_cast<float4*>(Am);
#pragma unroll
    for (int q = 0; q < 8; ++q)
      __stcg(park + q * 32 + lane,
             make_float4(S.a[0][2 * q].x, S.a[0][2 * q].y, S.a[0][2 * q + 1].x, S.a[0][2 * q + 1].y));
    uint32_t* w = sw + 40 * m;   // [0, 32): original row held by each lane; [32, 37): scalar state
    w[lane] = (uint32_t)orow;
    if (lane == 0) {
      w[32] = (uint32_t)S.U;
      w[33] = (uint32_t)(S.U >> 32);
      w[34] = __float_as_uint(S.mant);
      w[35] = (uint32_t)S.expo;
      w[36] = park_flags(S.neg, S.ok);
    }
  }
  __syncwarp();  // parked rows and words visible to every lane
  const int half = lane >> 4;
  const int h = nm == 2 ? half : 0;   // matrix carried by this lane
  const int i = lane & 15;
  const uint32_t* w = sw + 40 * h;
  const float4* park = reinterpret_cast<const float4*>(A + (size_t)sw[38 + h] * 4096);
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float4 v0 = __ldcg(park + q * 32 + i), v1 = __ldcg(park + q * 32 + i + 16);
    S.a[0][2 * q] = make_float2(v0.x, v0.y);
    S.a[0][2 * q + 1] = make_float2(v0.z, v0.w);
    S.a[1][2 * q] = make_float2(v1.x, v1.y);
    S.a[1][2 * q + 1] = make_float2(v1.z, v1.w);
  }
  S.prow_of[0] = (int)w[i];
  S.prow_of[1] = (int)w[i + 16];
  S.U = (uint64_t)w[32] | ((uint64_t)w[33] << 32);
  S.mant = __uint_as_float(w[34]);
  S.expo = (int)w[35];
  S.neg = unpark_neg(w[36]);
  S.ok = (w[36] >> 1) & 1u;
  S.half = half;
  S.pbit[0] = 1ull << S.prow_of[0];
  S.pbit[1] = 1ull << S.prow_of[1];
  S.key = lu_pivot_key<64, 2, 0, 0, LU_PAIRED>(S, lane);
  lu_phase<64, 2, 32, LU_PAIRED>(S, prow, lane);
  lu_phase<64, 2, 16, LU_PAIRED>(S, prow, lane);
  // each half's state -> both results
  const float mo = __shfl_xor_sync(VMC_FULL_MASK, S.mant, 16);
  const int eo = __shfl_xor_sync(VMC_FULL_MASK, S.expo, 16);
  const int no = __shfl_xor_sync(VMC_FULL_MASK, S.neg, 16);
  const bool oo = __shfl_xor_sync(VMC_FULL_MASK, (int)S.ok, 16) != 0;
  const Det mine = lu_det(S.ok, S.mant, S.expo, S.neg), other = lu_det(oo, mo, eo, no);
  d0 = half ? other : mine;
  d1 = half ? mine : other;
}

// FP64 in shared memory (nf <= 64 at run time), same retired-row scheme.
__device__ Det warp_logdet_f64(const double* __restrict__ A, int nf, double* s /*nf*(nf+1)*/) {
  const int lane = threadIdx.x & 31;
  const int ld = nf + 1;
  for (int idx = lane; idx < nf * nf; idx += 32) s[(idx / nf) * ld + idx % nf] = A[idx];
  __syncwarp();
  uint64_t U = (nf == 64) ? ~0ull : ((1ull << nf) - 1ull);
  double la = 0.0;
  int neg = 0;
  bool ok = true, nonfinite = false;
  for (int k = 0; k < nf; ++k) {
    double best = -1.0;
    int bi = 1 << 30;
    for (int r = lane; r < nf; r += 32) {
      if ((U >> r) & 1ull) {
        double v = fabs(s[r * ld + k]);
        if (v != v) v = INFINITY;   // NaN ranks first, so that it is detected
        if (v > best) { best = v; bi = r; }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(VMC_FULL_MASK, best, o);
      const int oi = __shfl_xor_sync(VMC_FULL_MASK, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const int p = bi;
    if (p >= nf) { ok = false; break; }  // no finite pivot candidate (warp-uniform)
    double pv = s[p * ld + k];
    if (!(best > 0.0) || !isfinite(best)) {
      nonfinite |= !isfinite(best);
      ok = false;
      pv = 1.0;
    }
    neg ^= (pv < 0.0);
    neg ^= __popcll(U & ((1ull << p) - 1ull)) & 1;
    U &= ~(1ull << p);
    la += log(fabs(pv));
    __syncwarp();
    for (int r = lane; r < nf; r += 32) {
      if ((U >> r) & 1ull) {
        const double f = s[r * ld + k] / pv;
        for (int c = k + 1; c < nf; ++c) s[r * ld + c] -= f * s[p * ld + c];
      }
    }
    __syncwarp();
  }
  Det d;
  if (nonfinite) {
    d.logabs = __longlong_as_double(0x7ff8000000000000ll);
    d.sign = d.logabs;
  } else {
    d.logabs = ok ? la : -INFINITY;
    d.sign = ok ? (neg ? -1.0 : 1.0) : 0.0;
  }
  return d;
}

enum { LD_ACCEPT = 0, LD_EVAL = 1, LD_ELOC = 2, LD_ACCEPT_Q = 3 };

// Learned-proposal record (layout shared with the proposal kernels).
struct PropRec4 {
  int flag, k;
  float u_acc, logq_fwd;
  int hop[4];
  float logq_rev;
  int pad[3];
};

struct LdArgs {
  // accept
  const PropRec* rec;
  const uint64_t* prop_occ;
  uint64_t* occ;
  int32_t* nacc;
  void* z0;            // float or double (B, HID)
  const void* w0t;
  // accept / eval
  double* sign;
  double* logabs;
  unsigned long long* n_eval;  // accept mode: number of proposals evaluated (nullable)
  // learned-proposal accept
  const PropRec4* rec4;
  const void* z0p;             // (B, HID) z0 of the proposed configurations
  float* lg_x;                 // (B, 256) proposal logits at x (nullable): replaced by lg_p on accept
  const float* lg_p;           // (B, 256) proposal logits at x'
  int* kstats;                 // [4] proposals and [4] acceptances by k (nullable)
  // eloc
  const int32_t* pairs;
  const double* coeff;
  double* term;
  // compacted rows (accept mode): rows [0, clamp(*rows_dev - rows_off)) of
  // the launch are the changed walkers row_map[rows_off + local]
  const int* rows_dev;
  int64_t rows_off;
  const int32_t* row_map;
};

__device__ __forceinline__ int64_t ld_rows(const LdArgs& la, int64_t R) {
  if (!la.rows_dev) return R;
  const int64_t rr = (int64_t)*la.rows_dev - la.rows_off;
  return rr < 0 ? 0 : (rr < R ? rr : R);
}
__device__ __forceinline__ int64_t ld_row(const LdArgs& la, int64_t row0, int64_t l) {
  return la.row_map ? (int64_t)la.row_map[row0 + l] : row0 + l;
}

// What the evaluated row's log-determinant is used for: EVAL stores it, ELOC
// forms the hop term, ACCEPT / ACCEPT_Q run the Metropolis(-Hastings) test and
// apply an accepted move (whole warp).
template <typename T, int MODE>
__device__ __forceinline__ void ld_finish(int64_t row, const Det& d, const LdArgs& la, int lane) {
  if (MODE == LD_EVAL) {
    if (lane == 0) { la.sign[row] = d.sign; la.logabs[row] = d.logabs; }
  } else if (MODE == LD_ELOC) {
    if (lane == 0) {
      const int w = la.pairs[2 * row];
      double v = 0.0;
      if (d.sign != 0.0 && la.sign[w] != 0.0) v = la.coeff[row] * d.sign * la.sign[w] * exp(d.logabs - la.logabs[w]);
      la.term[row] = v;
    }
  } else if (MODE == LD_ACCEPT_Q) {
    const PropRec4 r = la.rec4[row];
    // Metropolis-Hastings with the proposal ratio q(x'->x)/q(x->x').  Every
    // lane reads the current log-amplitude before lane 0 may overwrite it.
    const double cur = __shfl_sync(VMC_FULL_MASK, lane == 0 ? la.logabs[row] : 0.0, 0);
    const float la2 = (float)(2.0 * (d.logabs - cur)) + (r.logq_rev - r.logq_fwd);
    const float prob = expf(fminf(la2, 80.0f));
    // a NaN ratio (NaN amplitude on either side) never accepts, as u < NaN is false
    const bool acc = (d.sign != 0.0) && (la2 == la2) && isfinite(r.logq_rev) && (r.u_acc < prob);
    const int kk = min(max(r.k, 1), 4) - 1;
    if (la.kstats && lane == 0) {
      atomicAdd(&la.kstats[kk], 1);
      if (acc) atomicAdd(&la.kstats[4 + kk], 1);
    }
    if (!acc) return;
    if (la.lg_x) {  // the walker moved: its proposal logits are now those of x'
#pragma unroll
      for (int q = 0; q < 8; ++q) la.lg_x[row * 256 + lane * 8 + q] = la.lg_p[row * 256 + lane * 8 + q];
    }
    if (lane == 0) {
      la.occ[2 * row] = la.prop_occ[2 * row];
      la.occ[2 * row + 1] = la.prop_occ[2 * row + 1];
      la.sign[row] = d.sign;
      la.logabs[row] = d.logabs;
      la.nacc[row] += 1;
    }
    T* z0 = reinterpret_cast<T*>(la.z0);
    const T* zp = reinterpret_cast<const T*>(la.z0p);
#pragma unroll
    for (int q = 0; q < 8; ++q) z0[row * HID + lane * 8 + q] = zp[row * HID + lane * 8 + q];
  } else {
    const PropRec r = la.rec[row];
    // |psi'|^2/|psi|^2 from the FP64 log difference, exponentiated in FP32
    // (FP32 relative accuracy is ample for comparing against a 24-bit uniform).
    // Every lane reads the current log-amplitude before lane 0 may overwrite it.
    const double cur = __shfl_sync(VMC_FULL_MASK, lane == 0 ? la.logabs[row] : 0.0, 0);
    const float dl2 = (float)(2.0 * (d.logabs - cur));
    const float prob = expf(fminf(dl2, 80.0f));
    // a NaN ratio (NaN amplitude on either side) never accepts, as u < NaN is false;
    // from a zero-amplitude walker (cur = -inf) every non-zero proposal accepts
    const bool acc = (d.sign != 0.0) && (dl2 == dl2) && (r.u_acc < prob);
    if (!acc) return;
    if (lane == 0) {
      la.occ[2 * row] = la.prop_occ[2 * row];
      la.occ[2 * row + 1] = la.prop_occ[2 * row + 1];
      la.sign[row] = d.sign;
      la.logabs[row] = d.logabs;
      la.nacc[row] += 1;
    }
    int a[2], b[2];
    unpack_moves(r, a, b);
    T* z0 = reinterpret_cast<T*>(la.z0);
    const T* w0t = reinterpret_cast<const T*>(la.w0t);
    for (int m = 0; m < r.nmov; ++m) {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int u = lane * 8 + q;
        z0[row * HID + u] += w0t[b[m] * HID + u] - w0t[a[m] * HID + u];
      }
    }
  }
}

template <typename T, int NF, int MODE>
__global__ void __launch_bounds__(128, LU_MIN_CTAS) k_logdet(int64_t R, int64_t row0, int nf, const T* __restrict__ A, LdArgs la) {
  extern __shared__ __align__(16) uint8_t lsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t local = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (local >= R) return;
  const int64_t row = row0 + local;
  if (MODE == LD_ACCEPT) {
    if (!la.rec[row].flag) return;
    if (la.n_eval && lane == 0) atomicAdd(la.n_eval, 1ull);
  }
  if (MODE == LD_ACCEPT_Q) {
    if (!la.rec4[row].flag) return;
  }
  Det d;
  if constexpr (sizeof(T) == 4) {
    float* prow = reinterpret_cast<float*>(lsm) + warp * 128;  // two pivot-row slots
    d = warp_logdet_f32<NF>(reinterpret_cast<const float*>(A) + (size_t)local * NF * NF, prow);
  } else {
    double* s = reinterpret_cast<double*>(lsm) + (size_t)warp * (64 * 65);
    d = warp_logdet_f64(reinterpret_cast<const double*>(A) + (size_t)local * nf * nf, nf, s);
  }
  ld_finish<T, MODE>(row, d, la, lane);
}

template <int MODE>
__device__ __forceinline__ bool ld_flag(const LdArgs& la, int64_t row) {
  if (MODE == LD_ACCEPT) return la.rec[row].flag != 0;
  if (MODE == LD_ACCEPT_Q) return la.rec4[row].flag != 0;
  return true;
}

// FP32 64 x 64 rows.  A CTA of 4 warps takes 4 rows and hands the ones that
// need an evaluation to its warps in order; each warp runs its matrix's first
// 32 pivot steps in the full layout (one matrix a warp, as many warps as
// rows).  Warps 2k and 2k + 1 then meet at a named barrier: the odd warp parks
// its 32 x 32 remainder in its own (consumed) orbital-matrix slot and its
// scalar state in shared memory and retires; the even warp runs both tails as
// one instruction stream (lu_tail_pair) and finishes both rows.  A warp
// without a partner runs its tail alone in the same layout.
// shared words per warp: 128 floats of pivot-row slots + parked state (k_logdet_dual: two 40-word blocks,
// k_logdet_pair: one)
constexpr int LDP_WARP_WORDS = 128 + 80;

// Named barrier of warps 2k and 2k + 1 (ids 1 and 2; 0 is __syncthreads').
__device__ __forceinline__ void pair_barrier(int warp) {
  if (warp >> 1) asm volatile("bar.sync 2, 64;" ::: "memory");
  else asm volatile("bar.sync 1, 64;" ::: "memory");
}
template <int MODE>
__global__ void __launch_bounds__(128, LU_MIN_CTAS) k_logdet_pair(int64_t R, int64_t row0, float* A, LdArgs la) {
  extern __shared__ __align__(16) uint8_t lsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t base = (int64_t)blockIdx.x * 4;
  const int64_t Reff = ld_rows(la, R);
  bool fl = false;
  if (lane < 4 && base + lane < Reff) fl = la.rows_dev ? true : ld_flag<MODE>(la, row0 + base + lane);
  const unsigned mask = __ballot_sync(VMC_FULL_MASK, fl);
  const int n = __popc(mask);
  if (warp >= n) return;
  // the warp's row: the warp-th set bit; its partner's: the (warp ^ 1)-th
  unsigned m = mask;
  for (int k = 0; k < warp; ++k) m &= m - 1u;
  const int64_t l = base + (__ffs(m) - 1);
  const bool paired = (warp ^ 1) < n;
  if (MODE == LD_ACCEPT && la.n_eval && lane == 0) atomicAdd(la.n_eval, 1ull);
  float* prow = reinterpret_cast<float*>(lsm) + warp * LDP_WARP_WORDS;
  float* Am = A + (size_t)l * 4096;
  LuRegs<64> S;
  lu_load<64>(S, Am, lane);
  lu_phase<64, 2, 64, LU_FULL>(S, prow, lane);
  lu_phase<64, 2, 48, LU_FULL>(S, prow, lane);
  const int orow = lu_compact<32>(S, lane);
  if (paired && (warp & 1)) {
    __syncwarp();  // every lane's loads of the matrix precede the parking stores
    float4* park = reinterpret_cast<float4*>(Am);
#pragma unroll
    for (int q = 0; q < 8; ++q)
      __stcg(park + q * 32 + lane,
             make_float4(S.a[0][2 * q].x, S.a[0][2 * q].y, S.a[0][2 * q + 1].x, S.a[0][2 * q + 1].y));
    uint32_t* w = reinterpret_cast<uint32_t*>(prow + 128);
    w[lane] = (uint32_t)orow;
    if (lane == 0) {
      w[32] = (uint32_t)S.U;
      w[33] = (uint32_t)(S.U >> 32);
      w[34] = __float_as_uint(S.mant);
      w[35] = (uint32_t)S.expo;
      w[36] = park_flags(S.neg, S.ok);
    }
    pair_barrier(warp);
    return;   // the even partner finishes this row
  }
  Det d0, d1;
  int64_t lp = l;
  if (paired) {
    pair_barrier(warp);
    m &= m - 1u;
    lp = base + (__ffs(m) - 1);
    const float* pw = reinterpret_cast<const float*>(lsm) + (warp + 1) * LDP_WARP_WORDS;
    lu_tail_pair(S, orow, reinterpret_cast<const float4*>(A + (size_t)lp * 4096),
                 reinterpret_cast<const uint32_t*>(pw + 128), prow, d0, d1);
  } else {
    lu_tail_pair(S, orow, nullptr, nullptr, prow, d0, d1);
  }
  const int nd = paired ? 2 : 1;
#pragma unroll 1
  for (int k = 0; k < nd; ++k) ld_finish<float, MODE>(ld_row(la, row0, k ? lp : l), k ? d1 : d0, la, lane);
}

// FP32 64 x 64 rows, two matrices a warp throughout: a CTA of 4 warps takes
// 8 rows and hands the ones that need an evaluation out in pairs (warp w: the
// (2w)-th and (2w+1)-th; at most one warp of a CTA is left with one), see
// warp_logdet_f32_pair.  Half as many warps as k_logdet_pair, each busy to
// the end: the better choice when other launches (concurrent walker groups)
// fill the SMs; alone on the GPU k_logdet_pair's warp per row wins.
template <int MODE>
__global__ void __launch_bounds__(128, LU_MIN_CTAS) k_logdet_dual(int64_t R, int64_t row0, float* A, LdArgs la) {
  extern __shared__ __align__(16) uint8_t lsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t base = (int64_t)blockIdx.x * 8;
  const int64_t Reff = ld_rows(la, R);
  bool fl = false;
  if (lane < 8 && base + lane < Reff) fl = la.rows_dev ? true : ld_flag<MODE>(la, row0 + base + lane);
  unsigned m = __ballot_sync(VMC_FULL_MASK, fl);
  for (int i = 0; i < 2 * warp; ++i) m &= m - 1u;
  if (!m) return;
  const int64_t l0 = base + (__ffs(m) - 1);
  m &= m - 1u;
  const int64_t l1 = m ? base + (__ffs(m) - 1) : -1;
  if (MODE == LD_ACCEPT && la.n_eval && lane == 0) atomicAdd(la.n_eval, l1 >= 0 ? 2ull : 1ull);
  float* prow = reinterpret_cast<float*>(lsm) + warp * LDP_WARP_WORDS;
  uint32_t* sw = reinterpret_cast<uint32_t*>(prow + 128);
  // the rows (local indices < 2^31) wait in shared memory during the elimination
  if (lane == 0) { sw[38] = (uint32_t)l0; sw[39] = (uint32_t)(l1 < 0 ? l0 : l1); }
  const int nd = l1 < 0 ? 1 : 2;
  __syncwarp();
  Det d0, d1;
  warp_logdet_f32_pair(A, prow, sw, nd, d0, d1);
#pragma unroll 1
  for (int k = 0; k < nd; ++k) ld_finish<float, MODE>(ld_row(la, row0, (int64_t)sw[38 + k]), k ? d1 : d0, la, lane);
}

// per-walker local energy: U * doublons + segmented sum of the hop terms
__global__ void k_eloc_reduce(int64_t B, const uint64_t* __restrict__ occ, const int32_t* __restrict__ offs,
                              const double* __restrict__ term, double U, double* __restrict__ eloc) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  double s = U * (double)__popcll(occ[2 * w] & occ[2 * w + 1]);
  for (int q = offs[w]; q < offs[w + 1]; ++q) s += term[q];
  eloc[w] = s;
}

// number of valid hop terms per walker (T = 2E hop slots)
__global__ void k_count_hops(int64_t B, int N, const uint64_t* __restrict__ occ, const int32_t* __restrict__ edges,
                             int E, int32_t* __restrict__ cnt) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  const uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  int c = 0;
  for (int e = 0; e < E; ++e) {
    const int i = edges[2 * e], j = edges[2 * e + 1];
    c += (int)(((up >> i) ^ (up >> j)) & 1ull) + (int)(((dn >> i) ^ (dn >> j)) & 1ull);
  }
  cnt[w] = c;
}

__global__ void k_fill_pairs(int64_t B, int N, const uint64_t* __restrict__ occ, const int32_t* __restrict__ edges,
                             int E, const int32_t* __restrict__ offs, int32_t* __restrict__ pairs) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  const uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  int q = offs[w];
  for (int e = 0; e < E; ++e) {
    const int i = edges[2 * e], j = edges[2 * e + 1];
    if (((up >> i) ^ (up >> j)) & 1ull) { pairs[2 * q] = (int)w; pairs[2 * q + 1] = 2 * e; ++q; }
    if (((dn >> i) ^ (dn >> j)) & 1ull) { pairs[2 * q] = (int)w; pairs[2 * q + 1] = 2 * e + 1; ++q; }
  }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

bool get_encoder() {
  if (g_encode) return true;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return false;
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return true;
}

// bf16 row-major (rows x 256) tensor map, box {64, box_rows}, SWIZZLE_128B
bool tmap_bf16(CUtensorMap* m, const void* base, uint64_t rows, uint32_t box_rows) {
  if (!get_encoder()) return false;
  if (((uintptr_t)base & 15) != 0) return false;
  cuuint64_t gdim[2] = {(cuuint64_t)HID, (cuuint64_t)rows};
  cuuint64_t gstr[1] = {(cuuint64_t)HID * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), gdim, gstr, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

struct NetF32 {
  const float* w0t;             // (n_orb, 256)
  const float* b0;              // (256)
  const __nv_bfloat16* w1;      // (256, 256) bf16
  const float* b1;              // (256)
  const __nv_bfloat16* outw;    // (n_orb*nf, 256) bf16
  const float* outb;            // (n_orb*nf)
  const float* mbase;           // (n_orb, nf)
};
struct NetF64 {
  const double* w0t; const double* b0; const double* w1; const double* b1; const double* outw; const double* outb;
  const double* mbase;
};

// Workspace for R rows: H1, H2 (bf16 or fp64, R x 256), A (R x nf x nf).
struct Work {
  void* H1; void* H2; void* A;
};

// Optional per-stage device timing (CUDA events on the launching stream),
// used by the benchmark to time the kernels inside its timed region.
struct StageTimer {
  cudaStream_t st = nullptr;
  float* acc = nullptr;  // host: [prep, layer1, backflow, logdet] milliseconds
  int* cnt = nullptr;    // host: launches per stage
  std::vector<cudaEvent_t> ev;
  std::vector<int> stage;
  size_t used = 0;
  void mark(int stg, bool start) {
    if (!acc) return;
    if (used == ev.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev.push_back(e);
      stage.push_back(0);
    }
    stage[used] = start ? stg : -1;
    cudaEventRecord(ev[used], st);
    ++used;
  }
  void finish() {
    if (!acc) return;
    cudaStreamSynchronize(st);
    for (size_t i = 0; i + 1 < used; i += 2) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, ev[i], ev[i + 1]) == cudaSuccess) {
        acc[stage[i]] += ms;
        cnt[stage[i]] += 1;
      }
    }
    used = 0;
  }
};
// One timer for the process: stage timing (vmc_nnbf_sweep with stage_ms) is
// a benchmarking aid and is not re-entrant across host threads.
StageTimer g_timer;
#define STAGE_BEGIN(s) g_timer.mark((s), true)
#define STAGE_END(s) g_timer.mark((s), false)

// Rows per backflow+LU chunk: 4096 x 64 x 64 FP32 orbital matrices = 64 MB,
// small enough to stay resident in L2 between the GEMM epilogue and the LU.
constexpr int64_t kChunkRows = 4096;

// Per-device state is indexed by the current device's ordinal, so that one
// process may drive several GPUs.
constexpr int kMaxDevices = 64;
int g_num_sms[kMaxDevices] = {};
int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
  return dev;
}
int num_sms() {
  const int dev = current_device();
  if (!g_num_sms[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    g_num_sms[dev] = n > 0 ? n : 148;
  }
  return g_num_sms[dev];
}

void set_attrs();

// Second stream for the chunk pipeline: the backflow GEMM of chunk c+1 runs
// on it (high priority) while the LU of chunk c runs on the caller's stream;
// the GEMM is tensor/epilogue work and the LU latency-bound CUDA-core work,
// so the two share the SMs.  Events order the slot reuse of the two A
// buffers.  VMC_GB300_SERIAL_CHUNKS=1 runs the chunks back to back instead.
struct ChunkPipe {
  int dev = -1;
  cudaStream_t aux = nullptr;
  cudaEvent_t h2 = nullptr, g[2] = {nullptr, nullptr}, lu[2] = {nullptr, nullptr};
  bool ok = false;
  // walker groups of a sweep (vmc_nnbf_sweep): one stream each, fork/join events
  static constexpr int kLanes = 4;
  cudaStream_t lane[kLanes] = {};
  cudaEvent_t fork = nullptr, join[kLanes] = {};
  bool lanes_ok = false;
};
ChunkPipe g_pipe[16];
std::mutex g_pipe_mu;

ChunkPipe* chunk_pipe() {
  static const bool serial = [] {
    const char* e = std::getenv("VMC_GB300_SERIAL_CHUNKS");
    return e && e[0] == '1';
  }();
  if (serial) return nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) return nullptr;
  std::lock_guard<std::mutex> lk(g_pipe_mu);
  ChunkPipe& p = g_pipe[dev];
  if (p.dev == dev) return p.ok ? &p : nullptr;
  p.dev = dev;
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  bool ok = cudaStreamCreateWithPriority(&p.aux, cudaStreamNonBlocking, hi) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&p.h2, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; i < 2; ++i) {
    ok = ok && cudaEventCreateWithFlags(&p.g[i], cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&p.lu[i], cudaEventDisableTiming) == cudaSuccess;
  }
  bool lok = ok && cudaEventCreateWithFlags(&p.fork, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; i < ChunkPipe::kLanes; ++i) {
    lok = lok && cudaStreamCreateWithFlags(&p.lane[i], cudaStreamNonBlocking) == cudaSuccess;
    lok = lok && cudaEventCreateWithFlags(&p.join[i], cudaEventDisableTiming) == cudaSuccess;
  }
  p.lanes_ok = lok;
  p.ok = ok;
  return ok ? &p : nullptr;
}

// Walker groups per sweep (VMC_GB300_SWEEP_LANES, 1..4; default 4).  The
// groups are independent Markov chains, so each runs its whole edge loop on
// its own stream and the groups' GEMMs, LUs and proposal kernels overlap
// without a device-wide join per edge.
int sweep_lanes() {
  static const int n = [] {
    const char* e = std::getenv("VMC_GB300_SWEEP_LANES");
    int v = e ? std::atoi(e) : 4;
    return v < 1 ? 1 : (v > ChunkPipe::kLanes ? ChunkPipe::kLanes : v);
  }();
  return n;
}

// d_count / row_map (mixed precision, nf = 64): the rows are compacted, their
// number *d_count on the device (at most R) and their walkers row_map.
int launch_eval_rows(int prec, int64_t R, int N, int nf, const uint64_t* row_occ, const void* net, double scale,
                     const Work& wk, int* err, cudaStream_t st, int ldmode, const LdArgs& la,
                     bool allow_pipe = true, bool concurrent = false, const int* d_count = nullptr,
                     const int32_t* row_map = nullptr) {
  const int n_orb = 2 * N;
  if (prec == 0) {
    const NetF32& n = *(const NetF32*)net;
    CUtensorMap tH1, tW1, tOW;
    if (!tmap_bf16(&tH1, wk.H1, (uint64_t)R, TM) || !tmap_bf16(&tW1, n.w1, HID, TN) ||
        !tmap_bf16(&tOW, n.outw, (uint64_t)n_orb * nf, TN))
      return VMC_ERR_UNSUPPORTED;
    EpiArgs e1{};
    e1.bias = n.b1;
    e1.out = (__nv_bfloat16*)wk.H2;
    e1.rows_dev = d_count;
    dim3 g1((unsigned)((R + TM - 1) / TM), 1);
    STAGE_BEGIN(1);
    k_gemm_tc<EPI_GELU_BF16><<<g1, 128, GEMM_SMEM, st>>>(tH1, tW1, (int)R, e1, err);
    STAGE_END(1);
    const int n_groups = (n_orb * nf) / TN;
    const int64_t CH = R < kChunkRows ? R : kChunkRows;
    const int64_t n_chunks = (R + CH - 1) / CH;
    const int wpb = 4;
    const size_t lsmem = wpb * 128 * sizeof(float);  // two pivot-row slots per warp
    // chunk pipeline (two A slots inside the R-row workspace) unless the
    // stages are being timed one by one
    ChunkPipe* pipe = (allow_pipe && n_chunks > 1 && !g_timer.acc) ? chunk_pipe() : nullptr;
    if (pipe) {
      if (cudaEventRecord(pipe->h2, st) != cudaSuccess || cudaStreamWaitEvent(pipe->aux, pipe->h2, 0) != cudaSuccess)
        return VMC_ERR_CUDA;
    }
    // on an error after the first chunk the caller's stream waits for what is
    // already queued on the second stream before the error is returned
    auto fail = [&](int rc) {
      if (pipe) {
        cudaEventRecord(pipe->h2, pipe->aux);
        cudaStreamWaitEvent(st, pipe->h2, 0);
      }
      return rc;
    };
    for (int64_t ci = 0; ci < n_chunks; ++ci) {
      const int64_t c0 = ci * CH;
      const int64_t Rc = (R - c0) < CH ? (R - c0) : CH;
      const int slot = pipe ? (int)(ci & 1) : 0;
      float* Ac = (float*)wk.A + (size_t)slot * (size_t)CH * nf * nf;
      CUtensorMap tH2c;
      if (!tmap_bf16(&tH2c, (const __nv_bfloat16*)wk.H2 + c0 * HID, (uint64_t)Rc, TM)) return fail(VMC_ERR_UNSUPPORTED);
      PBArgs pa{};
      pa.row_occ = row_occ + 2 * c0; pa.mbase = n.mbase; pa.outb = n.outb; pa.Aout = Ac;
      pa.scale = (float)scale; pa.n_sites = N; pa.nf = nf; pa.R = (int)Rc;
      pa.n_tiles = (int)((Rc + TM - 1) / TM);
      pa.n_items = n_groups * pa.n_tiles;
      pa.rows_dev = d_count;
      pa.rows_off = c0;
      const int grid = pa.n_items < num_sms() ? pa.n_items : num_sms();
      cudaStream_t gs = pipe ? pipe->aux : st;
      if (pipe && ci >= 2 && cudaStreamWaitEvent(gs, pipe->lu[slot], 0) != cudaSuccess) return fail(VMC_ERR_CUDA);
      STAGE_BEGIN(2);
      k_backflow_persistent<<<grid, PB_THREADS, PB_SMEM, gs>>>(tH2c, tOW, pa, err);
      STAGE_END(2);
      if (pipe) {
        if (cudaEventRecord(pipe->g[slot], gs) != cudaSuccess || cudaStreamWaitEvent(st, pipe->g[slot], 0) != cudaSuccess)
          return fail(VMC_ERR_CUDA);
      }
      STAGE_BEGIN(3);
      LdArgs lc = la;
      lc.rows_dev = d_count;
      lc.rows_off = c0;
      lc.row_map = row_map;
      const unsigned gl = (unsigned)((Rc + wpb - 1) / wpb);
      if (nf == 64 && !concurrent) {  // warp pairs share the tails (the orbital-matrix slot is scratch: the LU parks in it)
        const unsigned gp = (unsigned)((Rc + wpb - 1) / wpb);
        const size_t psmem = (size_t)wpb * LDP_WARP_WORDS * sizeof(float);
        if (ldmode == LD_ACCEPT) k_logdet_pair<LD_ACCEPT><<<gp, 32 * wpb, psmem, st>>>(Rc, c0, Ac, lc);
        else if (ldmode == LD_EVAL) k_logdet_pair<LD_EVAL><<<gp, 32 * wpb, psmem, st>>>(Rc, c0, Ac, lc);
        else if (ldmode == LD_ACCEPT_Q) k_logdet_pair<LD_ACCEPT_Q><<<gp, 32 * wpb, psmem, st>>>(Rc, c0, Ac, lc);
        else k_logdet_pair<LD_ELOC><<<gp, 32 * wpb, psmem, st>>>(Rc, c0, Ac, lc);
      } else if (nf == 64) {  // two matrices a warp (concurrent walker groups fill the SMs)
        const unsigned gp = (unsigned)((Rc + 2 * wpb - 1) / (2 * wpb));
        const size_t psmem = (size_t)wpb * LDP_WARP_WORDS * sizeof(float);
        if (ldmode == LD_ACCEPT) k_logdet_dual<LD_ACCEPT><<<gp, 32 * wpb, psmem, st>>>(Rc, c0, Ac, lc);
        else if (ldmode == LD_EVAL) k_logdet_dual<LD_EVAL><<<gp, 32 * wpb, psmem, st>>>(Rc, c0, Ac, lc);
        else if (ldmode == LD_ACCEPT_Q) k_logdet_dual<LD_ACCEPT_Q><<<gp, 32 * wpb, psmem, st>>>(Rc, c0, Ac, lc);
        else k_logdet_dual<LD_ELOC><<<gp, 32 * wpb, psmem, st>>>(Rc, c0, Ac, lc);
      } else {
        // no compaction with 32 orbitals (the caller passes none)
        if (ldmode == LD_ACCEPT) k_logdet<float, 32, LD_ACCEPT><<<gl, 32 * wpb, lsmem, st>>>(Rc, c0, nf, Ac, la);
        else if (ldmode == LD_EVAL) k_logdet<float, 32, LD_EVAL><<<gl, 32 * wpb, lsmem, st>>>(Rc, c0, nf, Ac, la);
        else if (ldmode == LD_ACCEPT_Q) k_logdet<float, 32, LD_ACCEPT_Q><<<gl, 32 * wpb, lsmem, st>>>(Rc, c0, nf, Ac, la);
        else k_logdet<float, 32, LD_ELOC><<<gl, 32 * wpb, lsmem, st>>>(Rc, c0, nf, Ac, la);
      }
      STAGE_END(3);
      if (pipe && cudaEventRecord(pipe->lu[slot], st) != cudaSuccess) return fail(VMC_ERR_CUDA);
    }
  } else {
    const NetF64& n = *(const NetF64*)net;
    k_layer1_f64<<<(unsigned)R, HID, 0, st>>>(R, (const double*)wk.H1, n.w1, n.b1, (double*)wk.H2);
    k_backflow_f64<<<(unsigned)R, 256, 0, st>>>(R, N, nf, row_occ, (const double*)wk.H2, n.outw, n.outb, n.mbase,
                                                scale, (double*)wk.A);
    const int wpb = 2;
    const unsigned gl = (unsigned)((R + wpb - 1) / wpb);
    const size_t smem = (size_t)wpb * 64 * 65 * sizeof(double);
    if (ldmode == LD_ACCEPT) {
      cudaFuncSetAttribute(k_logdet<double, 64, LD_ACCEPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_logdet<double, 64, LD_ACCEPT><<<gl, 32 * wpb, smem, st>>>(R, 0, nf, (const double*)wk.A, la);
    } else if (ldmode == LD_EVAL) {
      cudaFuncSetAttribute(k_logdet<double, 64, LD_EVAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_logdet<double, 64, LD_EVAL><<<gl, 32 * wpb, smem, st>>>(R, 0, nf, (const double*)wk.A, la);
    } else {
      cudaFuncSetAttribute(k_logdet<double, 64, LD_ELOC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_logdet<double, 64, LD_ELOC><<<gl, 32 * wpb, smem, st>>>(R, 0, nf, (const double*)wk.A, la);
    }
  }
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// Kernel attributes are per device: set once on each device the first time
// that device is current.
bool g_attr_done[kMaxDevices] = {};
std::mutex g_attr_mu;
void set_attrs() {
  const int dev = current_device();
  std::lock_guard<std::mutex> lk(g_attr_mu);
  if (g_attr_done[dev]) return;
  cudaFuncSetAttribute(k_gemm_tc<EPI_GELU_BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_SMEM);
  cudaFuncSetAttribute(k_gemm_tc<EPI_BACKFLOW>, cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_SMEM);
  cudaFuncSetAttribute(k_backflow_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, PB_SMEM);
  g_attr_done[dev] = true;
}

int check_shape(int prec, int N, int nf, int hidden) {
  if (N < 1 || N > 64 || hidden != HID || nf < 1 || nf > 64) return VMC_ERR_ARGS;
  if (prec == 0 && ((nf != 32 && nf != 64) || ((2 * N * nf) % TN) != 0)) return VMC_ERR_UNSUPPORTED;
  if (prec != 0 && prec != 1) return VMC_ERR_ARGS;
  return VMC_OK;
}

}  // namespace

extern "C" {

// net: pointer array, see include/vmc_gb300.h (vmc_nnbf_* documentation)
int vmc_nnbf_eval(int prec, const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale,
                  const uint64_t* occ, int64_t R, void* z0_out, void* H1, void* H2, void* A, double* sign,
                  double* logabs, int* d_err, void* stream) {
  int st0 = check_shape(prec, n_sites, nf, hidden);
  if (st0) return st0;
  if (R < 0 || !net_ptrs || !occ || !H1 || !H2 || !A || !sign || !logabs || !d_err) return VMC_ERR_ARGS;
  if (R == 0) return VMC_OK;
  set_attrs();
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned gw = (unsigned)((R * 32 + 255) / 256);
  NetF32 nf32; NetF64 nf64;
  const void* net;
  if (prec == 0) {
    nf32 = NetF32{(const float*)net_ptrs[0], (const float*)net_ptrs[1], (const __nv_bfloat16*)net_ptrs[2],
                  (const float*)net_ptrs[3], (const __nv_bfloat16*)net_ptrs[4], (const float*)net_ptrs[5],
                  (const float*)net_ptrs[6]};
    k_prep_fresh<float><<<gw, 256, 0, st>>>(R, n_sites, nf, occ, nf32.w0t, nf32.b0, (float*)z0_out, H1, d_err);
    net = &nf32;
  } else {
    nf64 = NetF64{(const double*)net_ptrs[0], (const double*)net_ptrs[1], (const double*)net_ptrs[2],
                  (const double*)net_ptrs[3], (const double*)net_ptrs[4], (const double*)net_ptrs[5],
                  (const double*)net_ptrs[6]};
    k_prep_fresh<double><<<gw, 256, 0, st>>>(R, n_sites, nf, occ, nf64.w0t, nf64.b0, (double*)z0_out, H1, d_err);
    net = &nf64;
  }
  VMC_CUDA_CHECK_LAUNCH();
  LdArgs la{};
  la.sign = sign;
  la.logabs = logabs;
  return launch_eval_rows(prec, R, n_sites, nf, occ, net, bf_scale, Work{H1, H2, A}, d_err, st, LD_EVAL, la);
}

int vmc_nnbf_sweep(int prec, const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale,
                   uint64_t* occ, int64_t B, const int32_t* edges, int n_edges, int n_sweeps, float hopping_rate,
                   uint64_t seed, uint64_t sweep_offset, const float* r_move, const uint8_t* r_bit, const float* r_acc,
                   void* z0, double* sign, double* logabs, int32_t* n_acc, uint64_t* prop_occ, void* rec, void* H1,
                   void* H2, void* A, int* d_err, unsigned long long* d_n_eval, float* stage_ms, int* stage_launches,
                   void* compact_ws, void* stream) {
  int st0 = check_shape(prec, n_sites, nf, hidden);
  if (st0) return st0;
  if (B < 0 || n_edges < 0 || n_sweeps < 0) return VMC_ERR_ARGS;
  if (compact_ws && ((uintptr_t)compact_ws & 15) != 0) return VMC_ERR_ARGS;
  if ((r_move != nullptr) != (r_acc != nullptr) || (r_move != nullptr) != (r_bit != nullptr)) return VMC_ERR_ARGS;
  if (B == 0 || n_edges == 0 || n_sweeps == 0) return VMC_OK;
  if (!net_ptrs || !occ || !edges || !z0 || !sign || !logabs || !n_acc || !prop_occ || !rec || !H1 || !H2 || !A ||
      !d_err)
    return VMC_ERR_ARGS;
  set_attrs();
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned gw = (unsigned)((B * 32 + 255) / 256);
  NetF32 nf32; NetF64 nf64;
  const void* net;
  if (prec == 0) {
    nf32 = NetF32{(const float*)net_ptrs[0], (const float*)net_ptrs[1], (const __nv_bfloat16*)net_ptrs[2],
                  (const float*)net_ptrs[3], (const __nv_bfloat16*)net_ptrs[4], (const float*)net_ptrs[5],
                  (const float*)net_ptrs[6]};
    net = &nf32;
  } else {
    nf64 = NetF64{(const double*)net_ptrs[0], (const double*)net_ptrs[1], (const double*)net_ptrs[2],
                  (const double*)net_ptrs[3], (const double*)net_ptrs[4], (const double*)net_ptrs[5],
                  (const double*)net_ptrs[6]};
    net = &nf64;
  }
  LdArgs la{};
  la.rec = (const PropRec*)rec;
  la.prop_occ = prop_occ;
  la.occ = occ;
  la.nacc = n_acc;
  la.z0 = z0;
  la.w0t = prec == 0 ? (const void*)nf32.w0t : (const void*)nf64.w0t;
  la.sign = sign;
  la.logabs = logabs;
  la.n_eval = d_n_eval;
  g_timer.st = st;
  g_timer.acc = stage_ms;
  g_timer.cnt = stage_launches;
  g_timer.used = 0;
  // row compaction (mixed precision, 64 orbitals): workspace = two counters
  // per walker group (alternating edges) | row_map (B int32) | prop_c (B x 2 u64)
  int* ccnt = nullptr;
  int32_t* cmap = nullptr;
  uint64_t* cprop = nullptr;
  if (compact_ws && prec == 0 && nf == 64) {
    ccnt = (int*)compact_ws;
    cmap = (int32_t*)((char*)compact_ws + 256);
    cprop = (uint64_t*)((char*)compact_ws + 256 + (((size_t)B * 4 + 15) & ~(size_t)15));
    if (cudaMemsetAsync(ccnt, 0, 2 * ChunkPipe::kLanes * sizeof(int), st) != cudaSuccess) return VMC_ERR_CUDA;
  }
  // walker groups on their own streams (mixed precision, untimed stages, B >= 2 chunks)
  ChunkPipe* pipe = nullptr;
  int G = 1;
  if (prec == 0 && !stage_ms && sweep_lanes() > 1 && B >= 2 * kChunkRows) {
    pipe = chunk_pipe();
    if (pipe && pipe->lanes_ok) {
      G = sweep_lanes();
      if ((int64_t)G > B / kChunkRows) G = (int)(B / kChunkRows);
    } else {
      pipe = nullptr;
    }
  }
  if (G > 1) {
    if (cudaEventRecord(pipe->fork, st) != cudaSuccess) return VMC_ERR_CUDA;
    const int64_t Bg = (B + G - 1) / G;
    const size_t zrow = (size_t)HID * sizeof(float);
    for (int g = 0; g < G; ++g) {
      const int64_t w0 = (int64_t)g * Bg, w1 = (w0 + Bg) < B ? (w0 + Bg) : B;
      if (w0 >= w1) continue;
      cudaStream_t gs = pipe->lane[g];
      if (cudaStreamWaitEvent(gs, pipe->fork, 0) != cudaSuccess) return VMC_ERR_CUDA;
      LdArgs lg = la;
      lg.rec = la.rec + w0;
      lg.prop_occ = prop_occ + 2 * w0;
      lg.occ = occ + 2 * w0;
      lg.nacc = n_acc + w0;
      lg.z0 = (char*)z0 + (size_t)w0 * zrow;
      lg.sign = sign + w0;
      lg.logabs = logabs + w0;
      const Work wg{(char*)H1 + (size_t)w0 * HID * 2, (char*)H2 + (size_t)w0 * HID * 2,
                    (float*)A + (size_t)w0 * nf * nf};
      const unsigned gwg = (unsigned)(((w1 - w0) * 32 + 255) / 256);
      for (int s = 0; s < n_sweeps; ++s) {
        for (int e = 0; e < n_edges; ++e) {
          const int par = (s * n_edges + e) & 1;
          int* cn = ccnt ? ccnt + 2 * g + par : nullptr;
          int* cx = ccnt ? ccnt + 2 * g + (par ^ 1) : nullptr;
          k_prep_sweep<float><<<gwg, 256, 0, gs>>>(B, w0, w1, n_sites, occ, edges, e, s, n_edges, hopping_rate, seed,
                                                   sweep_offset + (uint64_t)s, r_move, r_bit, r_acc,
                                                   (const float*)z0, nf32.w0t, prop_occ, (PropRec*)rec, H1, cn, cmap,
                                                   cprop, cx);
          int rc = launch_eval_rows(prec, w1 - w0, n_sites, nf, cn ? cprop + 2 * w0 : prop_occ + 2 * w0, net,
                                    bf_scale, wg, d_err, gs, LD_ACCEPT, lg, /*allow_pipe=*/false,
                                    /*concurrent=*/true, cn, cn ? cmap + w0 : nullptr);
          if (rc) {
            // kernels already queued on this group's stream still write the
            // caller's buffers: the caller's stream waits for them all the same
            cudaEventRecord(pipe->join[g], gs);
            cudaStreamWaitEvent(st, pipe->join[g], 0);
            g_timer.acc = nullptr;
            return rc;
          }
        }
      }
      if (cudaEventRecord(pipe->join[g], gs) != cudaSuccess || cudaStreamWaitEvent(st, pipe->join[g], 0) != cudaSuccess)
        return VMC_ERR_CUDA;
    }
    g_timer.acc = nullptr;
    VMC_CUDA_CHECK_LAUNCH();
    return VMC_OK;
  }
  for (int s = 0; s < n_sweeps; ++s) {
    for (int e = 0; e < n_edges; ++e) {
      const int par = (s * n_edges + e) & 1;
      int* cn = ccnt ? ccnt + par : nullptr;
      int* cx = ccnt ? ccnt + (par ^ 1) : nullptr;
      STAGE_BEGIN(0);
      if (prec == 0)
        k_prep_sweep<float><<<gw, 256, 0, st>>>(B, 0, B, n_sites, occ, edges, e, s, n_edges, hopping_rate, seed,
                                                sweep_offset + (uint64_t)s, r_move, r_bit, r_acc, (const float*)z0,
                                                nf32.w0t, prop_occ, (PropRec*)rec, H1, cn, cmap, cprop, cx);
      else
        k_prep_sweep<double><<<gw, 256, 0, st>>>(B, 0, B, n_sites, occ, edges, e, s, n_edges, hopping_rate, seed,
                                                 sweep_offset + (uint64_t)s, r_move, r_bit, r_acc,
                                                 (const double*)z0, nf64.w0t, prop_occ, (PropRec*)rec, H1, nullptr,
                                                 nullptr, nullptr, nullptr);
      STAGE_END(0);
      int rc = launch_eval_rows(prec, B, n_sites, nf, cn ? cprop : prop_occ, net, bf_scale, Work{H1, H2, A}, d_err,
                                st, LD_ACCEPT, la, true, false, cn, cn ? cmap : nullptr);
      if (rc) { g_timer.acc = nullptr; return rc; }
    }
  }
  g_timer.finish();
  g_timer.acc = nullptr;
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// Local energy.  pairs/offs come from vmc_nnbf_conn_pairs; chunk rows at a time
// are evaluated with the workspace (H1, H2, A sized for `chunk` rows).
int vmc_nnbf_conn_count(const uint64_t* occ, int64_t B, int n_sites, const int32_t* edges, int n_edges, int32_t* cnt,
                        void* stream) {
  if (B < 0 || n_sites < 1 || n_sites > 64 || n_edges < 0 || (B > 0 && (!occ || !cnt || !edges))) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  k_count_hops<<<(unsigned)((B + 255) / 256), 256, 0, (cudaStream_t)stream>>>(B, n_sites, occ, edges, n_edges, cnt);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_nnbf_conn_pairs(const uint64_t* occ, int64_t B, int n_sites, const int32_t* edges, int n_edges,
                        const int32_t* offs, int32_t* pairs, void* stream) {
  if (B < 0 || n_sites < 1 || n_sites > 64 || n_edges < 0 || (B > 0 && (!occ || !offs || !pairs || !edges)))
    return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  k_fill_pairs<<<(unsigned)((B + 255) / 256), 256, 0, (cudaStream_t)stream>>>(B, n_sites, occ, edges, n_edges, offs,
                                                                            pairs);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_nnbf_local_energy(int prec, const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale,
                          const uint64_t* occ, int64_t B, const int32_t* edges, double t, double U, const void* z0,
                          const double* sign, const double* logabs, const int32_t* pairs, const int32_t* offs,
                          int64_t P, int64_t chunk, uint64_t* row_occ, double* coeff, double* term, void* H1, void* H2,
                          void* A, double* eloc, int* d_err, void* stream) {
  int st0 = check_shape(prec, n_sites, nf, hidden);
  if (st0) return st0;
  if (B < 0 || P < 0 || chunk <= 0) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!net_ptrs || !occ || !z0 || !sign || !logabs || !offs || !eloc || !d_err || !row_occ || !coeff || !term ||
      !H1 || !H2 || !A || (P > 0 && (!pairs || !edges)))
    return VMC_ERR_ARGS;
  set_attrs();
  cudaStream_t st = (cudaStream_t)stream;
  NetF32 nf32; NetF64 nf64;
  const void* net;
  if (prec == 0) {
    nf32 = NetF32{(const float*)net_ptrs[0], (const float*)net_ptrs[1], (const __nv_bfloat16*)net_ptrs[2],
                  (const float*)net_ptrs[3], (const __nv_bfloat16*)net_ptrs[4], (const float*)net_ptrs[5],
                  (const float*)net_ptrs[6]};
    net = &nf32;
  } else {
    nf64 = NetF64{(const double*)net_ptrs[0], (const double*)net_ptrs[1], (const double*)net_ptrs[2],
                  (const double*)net_ptrs[3], (const double*)net_ptrs[4], (const double*)net_ptrs[5],
                  (const double*)net_ptrs[6]};
    net = &nf64;
  }
  // Mixed precision with a workspace of >= 2 chunks: the pair chunks are
  // independent, so G streams each take every G-th sub-chunk with their own
  // slice of the workspace (the walker-group scheme of vmc_nnbf_sweep).
  ChunkPipe* pipe = nullptr;
  int G = 1;
  if (prec == 0 && !g_timer.acc && sweep_lanes() > 1 && chunk >= 2 * kChunkRows && P > kChunkRows) {
    pipe = chunk_pipe();
    if (pipe && pipe->lanes_ok) {
      G = sweep_lanes();
      if ((int64_t)G > chunk / kChunkRows) G = (int)(chunk / kChunkRows);
    }
  }
  if (G > 1) {
    const int64_t sub = chunk / G;
    if (cudaEventRecord(pipe->fork, st) != cudaSuccess) return VMC_ERR_CUDA;
    for (int g = 0; g < G; ++g)
      if (cudaStreamWaitEvent(pipe->lane[g], pipe->fork, 0) != cudaSuccess) return VMC_ERR_CUDA;
    int64_t k = 0;
    for (int64_t p0 = 0; p0 < P; p0 += sub, ++k) {
      const int g = (int)(k % G);
      cudaStream_t gs = pipe->lane[g];
      const int64_t R = (P - p0) < sub ? (P - p0) : sub;
      uint64_t* ro = row_occ + 2 * (size_t)g * sub;
      double* co = coeff + (size_t)g * sub;
      const Work wg{(char*)H1 + (size_t)g * sub * HID * 2, (char*)H2 + (size_t)g * sub * HID * 2,
                    (float*)A + (size_t)g * sub * nf * nf};
      k_prep_conn<float><<<(unsigned)((R * 32 + 255) / 256), 256, 0, gs>>>(
          R, n_sites, pairs + 2 * p0, occ, edges, t, (const float*)z0, nf32.w0t, ro, co, wg.H1);
      LdArgs la{};
      la.pairs = pairs + 2 * p0;
      la.coeff = co;
      la.term = term + p0;
      la.sign = const_cast<double*>(sign);
      la.logabs = const_cast<double*>(logabs);
      int rc = launch_eval_rows(prec, R, n_sites, nf, ro, net, bf_scale, wg, d_err, gs, LD_ELOC, la,
                                /*allow_pipe=*/false, /*concurrent=*/true);
      if (rc) {
        // the caller's stream still waits for every kernel already queued on the lanes
        for (int h = 0; h < G; ++h) {
          cudaEventRecord(pipe->join[h], pipe->lane[h]);
          cudaStreamWaitEvent(st, pipe->join[h], 0);
        }
        return rc;
      }
    }
    for (int g = 0; g < G; ++g)
      if (cudaEventRecord(pipe->join[g], pipe->lane[g]) != cudaSuccess ||
          cudaStreamWaitEvent(st, pipe->join[g], 0) != cudaSuccess)
        return VMC_ERR_CUDA;
    P = 0;  // every pair is done; only the reduction below remains
  }
  for (int64_t p0 = 0; p0 < P; p0 += chunk) {
    const int64_t R = (P - p0) < chunk ? (P - p0) : chunk;
    const unsigned gw = (unsigned)((R * 32 + 255) / 256);
    if (prec == 0)
      k_prep_conn<float><<<gw, 256, 0, st>>>(R, n_sites, pairs + 2 * p0, occ, edges, t, (const float*)z0, nf32.w0t,
                                             row_occ, coeff, H1);
    else
      k_prep_conn<double><<<gw, 256, 0, st>>>(R, n_sites, pairs + 2 * p0, occ, edges, t, (const double*)z0, nf64.w0t,
                                              row_occ, coeff, H1);
    LdArgs la{};
    la.pairs = pairs + 2 * p0;
    la.coeff = coeff;
    la.term = term + p0;
    la.sign = const_cast<double*>(sign);
    la.logabs = const_cast<double*>(logabs);
    int rc = launch_eval_rows(prec, R, n_sites, nf, row_occ, net, bf_scale, Work{H1, H2, A}, d_err, st, LD_ELOC, la);
    if (rc) return rc;
  }
  k_eloc_reduce<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(B, occ, offs, term, U, eloc);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

}  // extern "C"

// ===========================================================================
// Allocation-free evaluation entry point.
//
// Some callers cannot allocate device memory while they run: a host program
// that drives the evaluation from a region where allocation is forbidden (a
// fixed device-memory budget set up once at start, a real-time loop, or a
// framework that owns the whole device pool and rejects foreign allocations).
// For them this variant of vmc_nnbf_eval (mixed precision only) keeps its
// scratch -- the two hidden-activation tiles and the per-configuration orbital
// matrices -- in a fixed array in device memory that is part of this library.
// Capacity: kNoAllocRows configurations per call with nf <= 64 (8.5 MiB).
// Every GPU that loads the library holds this array until the process exits.
// ===========================================================================
namespace {
constexpr int64_t kNoAllocRows = 512;
constexpr size_t kNoAllocH = (size_t)kNoAllocRows * HID * 2;          // one bf16 activation tile, bytes
constexpr size_t kNoAllocA = (size_t)kNoAllocRows * 64 * 64 * 4;      // orbital matrices, bytes
static __device__ __align__(256) uint8_t g_noalloc_scratch[2 * kNoAllocH + kNoAllocA];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {};  // device address of g_noalloc_scratch, per device ordinal

// Host code must not use g_noalloc_scratch as a device address: its host-side
// name is only a stand-in.  Resolve the real address once per device, with
// that device current.
int noalloc_scratch(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return VMC_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return VMC_ERR_CUDA;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return VMC_OK;
}
}  // namespace

extern "C" int vmc_nnbf_eval_noalloc(const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale,
                                     const uint64_t* occ, int64_t R, double* sign, double* logabs, int* d_err,
                                     void* stream) {
  int st0 = check_shape(0, n_sites, nf, hidden);
  if (st0) return st0;
  if (R < 0 || !net_ptrs || !occ || !sign || !logabs || !d_err) return VMC_ERR_ARGS;
  if (R > kNoAllocRows) return VMC_ERR_CAPACITY;
  if (R == 0) return VMC_OK;
  void* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  set_attrs();
  cudaStream_t st = (cudaStream_t)stream;
  // Every scratch row this call reads is written earlier in the same call (rows
  // beyond R are zero-filled by the TMA bounds check, not read from the array),
  // so nothing needs clearing between calls.
  Work wk{scratch, (uint8_t*)scratch + kNoAllocH, (uint8_t*)scratch + 2 * kNoAllocH};
  NetF32 n32{(const float*)net_ptrs[0], (const float*)net_ptrs[1], (const __nv_bfloat16*)net_ptrs[2],
             (const float*)net_ptrs[3], (const __nv_bfloat16*)net_ptrs[4], (const float*)net_ptrs[5],
             (const float*)net_ptrs[6]};
  const unsigned gw = (unsigned)((R * 32 + 255) / 256);
  k_prep_fresh<float><<<gw, 256, 0, st>>>(R, n_sites, nf, occ, n32.w0t, n32.b0, nullptr, wk.H1, d_err);
  VMC_CUDA_CHECK_LAUNCH();
  LdArgs la{};
  la.sign = sign;
  la.logabs = logabs;
  return launch_eval_rows(0, R, n_sites, nf, occ, &n32, bf_scale, wk, d_err, st, LD_EVAL, la);
}

// Second network layer on the tensor cores, H2 = gelu(H1 W1^T + b1) (BF16
// operands, FP32 accumulation, BF16 result): the stage every mixed NNBF entry
// point runs after the first layer.  It doubles as the self-test of the
// bounded-wait path: with skip_loads = 1 the kernel issues no tile load, so
// its wait for the operands runs out after wait_limit_ns with no copy or MMA
// in flight; the kernel then records VMC_ERR_TIMEOUT in *d_err, frees its
// tensor memory and returns, leaving H2 untouched and the context usable.
extern "C" int vmc_nnbf_hidden_layer(const void* H1, int64_t R, const void* W1, const float* b1, void* H2,
                                     uint64_t wait_limit_ns, int skip_loads, int* d_err, void* stream) {
  if (R < 0 || R > (int64_t)INT32_MAX || (R > 0 && (!H1 || !W1 || !b1 || !H2 || !d_err))) return VMC_ERR_ARGS;
  if (R == 0) return VMC_OK;
  set_attrs();
  CUtensorMap tH1, tW1;
  if (!tmap_bf16(&tH1, H1, (uint64_t)R, TM) || !tmap_bf16(&tW1, W1, HID, TN)) return VMC_ERR_UNSUPPORTED;
  EpiArgs e1{};
  e1.bias = b1;
  e1.out = (__nv_bfloat16*)H2;
  e1.wait_ns = wait_limit_ns;
  e1.skip_loads = skip_loads ? 1 : 0;
  dim3 g1((unsigned)((R + TM - 1) / TM), 1);
  k_gemm_tc<EPI_GELU_BF16><<<g1, 128, GEMM_SMEM, (cudaStream_t)stream>>>(tH1, tW1, (int)R, e1, d_err);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// Metropolis-Hastings step with a learned proposal (mixed precision): the
// proposals (prop_occ, rec4 from vmc_prop_sample / vmc_prop_reverse) are
// evaluated (first layer updated from the walkers' cached z0 over the changed
// orbitals, the rest in full) and accepted with
// min(1, |psi'/psi|^2 q(x'->x)/q(x->x')).
// Workspace: z0p (B, 256) f32, H1/H2/A for B rows.
extern "C" int vmc_nnbf_mh_step(const void* const* net_ptrs, int n_sites, int nf, int hidden, double bf_scale,
                                uint64_t* occ, int64_t B, const uint64_t* prop_occ, const void* rec4, void* z0,
                                void* z0p, double* sign, double* logabs, int32_t* n_acc, void* H1, void* H2, void* A,
                                float* lg_x, const float* lg_p, int* kstats, int* d_err, void* stream) {
  int st0 = check_shape(0, n_sites, nf, hidden);
  if (st0) return st0;
  if (B < 0 || !net_ptrs || !occ || !prop_occ || !rec4 || !z0 || !z0p || !sign || !logabs || !n_acc || !H1 || !H2 ||
      !A || !d_err)
    return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  set_attrs();
  cudaStream_t st = (cudaStream_t)stream;
  NetF32 n32{(const float*)net_ptrs[0], (const float*)net_ptrs[1], (const __nv_bfloat16*)net_ptrs[2],
             (const float*)net_ptrs[3], (const __nv_bfloat16*)net_ptrs[4], (const float*)net_ptrs[5],
             (const float*)net_ptrs[6]};
  const unsigned gw = (unsigned)((B * 32 + 255) / 256);
  k_prep_delta<float><<<gw, 256, 0, st>>>(B, n_sites, nf, occ, prop_occ, (const float*)z0, n32.w0t, (float*)z0p, H1,
                                          d_err);
  VMC_CUDA_CHECK_LAUNCH();
  LdArgs la{};
  la.rec4 = (const PropRec4*)rec4;
  la.prop_occ = prop_occ;
  la.occ = occ;
  la.nacc = n_acc;
  la.z0 = z0;
  la.z0p = z0p;
  la.sign = sign;
  la.logabs = logabs;
  la.lg_x = lg_x;
  la.lg_p = lg_p;
  la.kstats = kstats;
  if ((lg_x != nullptr) != (lg_p != nullptr)) return VMC_ERR_ARGS;
  return launch_eval_rows(0, B, n_sites, nf, prop_occ, &n32, bf_scale, Work{H1, H2, A}, d_err, st, LD_ACCEPT_Q, la);
}
