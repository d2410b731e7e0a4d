// Sample-space SR (minSR) linear algebra on one GPU:
//   column means and centring/scaling of O, the Gram matrix T = O~ O~^T + lambda I
//   on the CUDA cores (the tensor-core Gram is in gram.cu), a blocked right-looking
//   Cholesky of T (FP64 tiles and panels, double-float trailing updates), blocked
//   forward/backward substitution, and dp = O~^T x.  Also the plain energy
//   gradient <E O> - <E><O>.
#include "common.cuh"

namespace {

constexpr int TB = 64;   // output tile
constexpr int TK = 16;   // k chunk

// FP32 inputs: products are accumulated in FP32 over 4 consecutive k and then
// folded into a double-float (hi, lo) pair with Knuth's TwoSum, which keeps the
// Gram matrix accurate to ~FP64 level (its smallest eigenvalues sit at the
// diagonal shift, ~1e-6 of its norm) at ~2.5x the FP32 cost instead of the
// 64x of native FP64 arithmetic on GB300.  FP64 inputs accumulate natively.
template <typename TA>
struct TileAcc {
  TA acc[4][4];
  float lo[4][4];
  float hi[4][4];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int r = 0; r < 4; ++r) { acc[q][r] = 0; lo[q][r] = 0.f; hi[q][r] = 0.f; }
  }
  __device__ __forceinline__ void fold() {
    if constexpr (sizeof(TA) == 4) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const float a = hi[q][r], b = (float)acc[q][r];
          const float s = a + b;
          const float bb = s - a;
          const float err = (a - (s - bb)) + (b - bb);
          hi[q][r] = s;
          lo[q][r] += err;
          acc[q][r] = 0;
        }
    }
  }
  __device__ __forceinline__ double value(int q, int r) const {
    if constexpr (sizeof(TA) == 4) return (double)hi[q][r] + (double)lo[q][r] + (double)acc[q][r];
    return (double)acc[q][r];
  }
};

// mean[p] = (1/Ns) sum_i O[i][p];  Oc[i][p] = (O[i][p] - mean[p]) * scale
template <typename TI, typename TO>
__global__ void k_center(const TI* __restrict__ O, int64_t Ns, int64_t Np, int64_t ldo, TO* __restrict__ Oc,
                         int64_t ldc, double* __restrict__ mean, double scale) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= Np) return;
  double s = 0.0;
  for (int64_t i = 0; i < Ns; ++i) s += (double)O[i * ldo + p];
  const double m = s / (double)Ns;
  if (mean) mean[p] = m;
  if (Oc)
    for (int64_t i = 0; i < Ns; ++i) Oc[i * ldc + p] = (TO)(((double)O[i * ldo + p] - m) * scale);
}

// g[p] = (1/Ns) sum_i E[i] O[i][p] - Ebar * mean_i O[i][p]
template <typename TI>
__global__ void k_egrad(const TI* __restrict__ O, int64_t Ns, int64_t Np, int64_t ldo, const double* __restrict__ E,
                        double Ebar, double* __restrict__ g) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= Np) return;
  double se = 0.0, so = 0.0;
  for (int64_t i = 0; i < Ns; ++i) {
    double o = (double)O[i * ldo + p];
    se += E[i] * o;
    so += o;
  }
  g[p] = se / (double)Ns - Ebar * so / (double)Ns;
}

// C[i][j] (+)= sign * sum_{k<K} A[i][k] * A[j][k] for lower-triangular 64x64 tiles
// (tile row >= tile col).  A row-major with leading dim lda; rows offset by
// row0 for both operands; columns of C offset by col0 as well.  Tiles of the
// strict upper triangle are mirrored when mirror != 0.
template <typename TI, typename TA>
__global__ void k_syrk(const TI* __restrict__ A, int64_t lda, int64_t n, int64_t K, double* __restrict__ C,
                       int64_t ldc, int64_t off, double sgn, double diag, int mirror) {
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj > bi) return;
  __shared__ TA As[TK][TB + 1];
  __shared__ TA Bs[TK][TB + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = off + (int64_t)bi * TB, j0 = off + (int64_t)bj * TB;
  TileAcc<TA> T;
  T.zero();
  for (int64_t k0 = 0; k0 < K; k0 += TK) {
    for (int idx = threadIdx.x; idx < TB * TK; idx += 256) {
      int r = idx / TK, kk = idx - r * TK;
      int64_t gk = k0 + kk;
      int64_t gi = i0 + r, gj = j0 + r;
      As[kk][r] = (gi < off + n && gk < K) ? (TA)A[gi * lda + gk] : (TA)0;
      Bs[kk][r] = (gj < off + n && gk < K) ? (TA)A[gj * lda + gk] : (TA)0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      TA a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) { a[q] = As[kk][ty * 4 + q]; b[q] = Bs[kk][tx * 4 + q]; }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int r = 0; r < 4; ++r) T.acc[q][r] += a[q] * b[r];
      if ((kk & 3) == 3) T.fold();
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int64_t gi = i0 + ty * 4 + q, gj = j0 + tx * 4 + r;
      if (gi < off + n && gj < off + n && gj <= gi) {
        double v = C[gi * ldc + gj] + sgn * T.value(q, r);
        if (gi == gj) v += diag;
        C[gi * ldc + gj] = v;
        if (mirror && gi != gj) C[gj * ldc + gi] = v;
      }
    }
}

// The Cholesky's trailing update C -= A A^T for FP64 A in double-float
// arithmetic on the FP32 pipes (GB300's FP64 rate is 1/64 of FP32): each
// operand is split into FP32 x = hi + lo (to 2^-48), the leading product
// hi*hi is captured exactly (p and its FMA error term), p is summed with
// Knuth's TwoSum into a (s, c) pair and the small terms (the error term,
// hi*lo + lo*hi) into a third FP32 accumulator; lo*lo (2^-48) is dropped.
// ~12 FP32 instructions per multiply-add, relative accuracy ~2^-45 over the
// tile, far below the Gram matrix's own input rounding.  Same tiling and
// lower-triangle semantics as k_syrk.
__global__ void k_syrk_df(const double* __restrict__ A, int64_t lda, int64_t n, int64_t K, double* __restrict__ C,
                          int64_t ldc, int64_t off, double sgn) {
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj > bi) return;
  __shared__ float Ah[TK][TB + 1], Al[TK][TB + 1], Bh[TK][TB + 1], Bl[TK][TB + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = off + (int64_t)bi * TB, j0 = off + (int64_t)bj * TB;
  float hs[4][4], hc[4][4], sm[4][4];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int r = 0; r < 4; ++r) { hs[q][r] = 0.f; hc[q][r] = 0.f; sm[q][r] = 0.f; }
  for (int64_t k0 = 0; k0 < K; k0 += TK) {
    for (int idx = threadIdx.x; idx < TB * TK; idx += 256) {
      const int r = idx / TK, kk = idx - r * TK;
      const int64_t gk = k0 + kk, gi = i0 + r, gj = j0 + r;
      const double a = (gi < off + n && gk < K) ? A[gi * lda + gk] : 0.0;
      const double b = (gj < off + n && gk < K) ? A[gj * lda + gk] : 0.0;
      const float ah = (float)a, bh = (float)b;
      Ah[kk][r] = ah;
      Al[kk][r] = (float)(a - (double)ah);
      Bh[kk][r] = bh;
      Bl[kk][r] = (float)(b - (double)bh);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < TK; ++kk) {
      float ah[4], al[4], bh[4], bl[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        ah[q] = Ah[kk][ty * 4 + q]; al[q] = Al[kk][ty * 4 + q];
        bh[q] = Bh[kk][tx * 4 + q]; bl[q] = Bl[kk][tx * 4 + q];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const float p = ah[q] * bh[r];
          const float e = fmaf(ah[q], bh[r], -p);
          sm[q][r] += e + fmaf(ah[q], bl[r], al[q] * bh[r]);
          const float s2 = hs[q][r] + p;
          const float bb = s2 - hs[q][r];
          hc[q][r] += (hs[q][r] - (s2 - bb)) + (p - bb);
          hs[q][r] = s2;
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int64_t gi = i0 + ty * 4 + q, gj = j0 + tx * 4 + r;
      if (gi < off + n && gj < off + n && gj <= gi)
        C[gi * ldc + gj] += sgn * ((double)hs[q][r] + (double)hc[q][r] + (double)sm[q][r]);
    }
}

// Unblocked Cholesky of one diagonal tile (lower), in place; flags non-positive pivots.
__global__ void k_potrf_tile(double* __restrict__ C, int64_t ldc, int64_t k0, int64_t nb, int* __restrict__ info) {
  __shared__ double a[TB][TB + 1];
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
    int r = idx / nb, c = idx - r * nb;
    a[r][c] = C[(k0 + r) * ldc + k0 + c];
  }
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (threadIdx.x == 0) {
      double d = a[k][k];
      if (!(d > 0.0) || !isfinite(d)) { atomicExch(info, 1); d = 1e-300; }
      a[k][k] = sqrt(d);
    }
    __syncthreads();
    for (int r = k + 1 + threadIdx.x; r < nb; r += blockDim.x) a[r][k] /= a[k][k];
    __syncthreads();
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
      int r = idx / nb, c = idx - r * nb;
      if (c > k && r >= c) a[r][c] -= a[r][k] * a[c][k];
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
    int r = idx / nb, c = idx - r * nb;
    C[(k0 + r) * ldc + k0 + c] = (c <= r) ? a[r][c] : 0.0;
  }
}

// Panel: X = A21 * L11^{-T} for the rows below the diagonal tile; one thread per row.
__global__ void k_trsm_panel(double* __restrict__ C, int64_t ldc, int64_t n, int64_t k0, int64_t nb) {
  __shared__ double L[TB][TB + 1];
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
    int r = idx / nb, c = idx - r * nb;
    L[r][c] = C[(k0 + r) * ldc + k0 + c];
  }
  __syncthreads();
  int64_t row = k0 + nb + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  double x[TB];
  double* a = C + row * ldc + k0;
  for (int k = 0; k < nb; ++k) {
    double v = a[k];
    for (int m = 0; m < k; ++m) v -= x[m] * L[k][m];
    x[k] = v / L[k][k];
  }
  for (int k = 0; k < nb; ++k) a[k] = x[k];
}

// Blocked triangular solves (panels of TRSV_NB rows): the diagonal block is
// solved by one CTA (thread t owns row t of the block), then every remaining
// row is updated by a coalesced dot with the panel's solved values.
constexpr int TRSV_NB = 64;

// trans = 0: solve L[k0:k0+nb, k0:k0+nb] y = b[k0:k0+nb] in place (forward);
// trans = 1: solve L[k0:k0+nb, k0:k0+nb]^T x = b[k0:k0+nb] in place (backward).
__global__ void k_trsv_diag(const double* __restrict__ L, int64_t ldc, int64_t k0, int nb, double* __restrict__ b,
                            int trans) {
  __shared__ double xs[TRSV_NB];
  const int t = threadIdx.x;
  double bt = t < nb ? b[k0 + t] : 0.0;
  if (!trans) {
    for (int j = 0; j < nb; ++j) {
      if (t == j) xs[j] = bt / L[(k0 + j) * ldc + k0 + j];
      __syncthreads();
      if (t > j && t < nb) bt -= L[(k0 + t) * ldc + k0 + j] * xs[j];
    }
  } else {
    for (int j = nb - 1; j >= 0; --j) {
      if (t == j) xs[j] = bt / L[(k0 + j) * ldc + k0 + j];
      __syncthreads();
      if (t < j) bt -= L[(k0 + j) * ldc + k0 + t] * xs[j];
    }
  }
  if (t < nb) b[k0 + t] = xs[t];
}

// forward update: b[i] -= sum_{j < nb} L[i][k0 + j] b[k0 + j] for rows i >= k0 + nb, a warp per row
__global__ void k_trsv_upd_fwd(const double* __restrict__ L, int64_t ldc, int64_t n, int64_t k0, int nb,
                               double* __restrict__ b) {
  const int64_t i = k0 + nb + (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  double acc = 0.0;
  for (int j = lane; j < nb; j += 32) acc += L[i * ldc + k0 + j] * b[k0 + j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) b[i] -= acc;
}

// backward update: b[j] -= sum_{i < nb} L[k0 + i][j] b[k0 + i] for columns j < k0, a thread per column
__global__ void k_trsv_upd_bwd(const double* __restrict__ L, int64_t ldc, int64_t k0, int nb,
                               double* __restrict__ b) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k0) return;
  double acc = 0.0;
  for (int i = 0; i < nb; ++i) acc += L[(k0 + i) * ldc + j] * b[k0 + i];
  b[j] -= acc;
}

// dp[p] = sum_i Oc[i][p] * x[i]
template <typename TI>
__global__ void k_gemv_t(const TI* __restrict__ Oc, int64_t Ns, int64_t Np, int64_t ldc, const double* __restrict__ x,
                         double* __restrict__ dp) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= Np) return;
  double s = 0.0;
  for (int64_t i = 0; i < Ns; ++i) s += (double)Oc[i * ldc + p] * x[i];
  dp[p] = s;
}

__global__ void k_rhs(const double* __restrict__ E, int64_t Ns, double Ebar, double scale, double* __restrict__ b) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < Ns) b[i] = (E[i] - Ebar) * scale;
}

__global__ void k_zero(double* __restrict__ p, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.0;
}

}  // namespace

extern "C" {

// Centre and scale O (Ns x Np, ld ldo) into Oc (ld ldc): Oc = (O - mean)/sqrt(Ns).
// dtype codes: 0 = float64, 1 = float32 (for both O and Oc).
int vmc_sr_center(const void* O, int dtype, int64_t Ns, int64_t Np, int64_t ldo, void* Oc, int64_t ldc, double* mean,
                  void* stream) {
  if (Ns <= 0 || Np <= 0 || ldo < Np || ldc < Np || !O || !Oc) return VMC_ERR_ARGS;
  const double scale = 1.0 / sqrt((double)Ns);
  unsigned grid = (unsigned)((Np + 255) / 256);
  if (dtype == 0)
    k_center<double, double><<<grid, 256, 0, (cudaStream_t)stream>>>((const double*)O, Ns, Np, ldo, (double*)Oc, ldc,
                                                                      mean, scale);
  else if (dtype == 1)
    k_center<float, float><<<grid, 256, 0, (cudaStream_t)stream>>>((const float*)O, Ns, Np, ldo, (float*)Oc, ldc,
                                                                    mean, scale);
  else
    return VMC_ERR_ARGS;
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// T (Ns x Ns, FP64, ld ldt) = (accumulate ? T : 0) + Oc Oc^T (+ diag_shift on the diagonal).
int vmc_sr_gram(const void* Oc, int dtype, int64_t Ns, int64_t Np, int64_t ldc, double* T, int64_t ldt,
                double diag_shift, int accumulate, void* stream) {
  if (Ns <= 0 || Np < 0 || ldc < Np || ldt < Ns || !Oc || !T) return VMC_ERR_ARGS;
  cudaStream_t s = (cudaStream_t)stream;
  if (!accumulate) {
    int64_t n = Ns * ldt;
    k_zero<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(T, n);
  }
  int64_t nt = (Ns + TB - 1) / TB;
  if (nt > 65535) return VMC_ERR_ARGS;
  dim3 grid((unsigned)nt, (unsigned)nt);
  if (dtype == 0)
    k_syrk<double, double><<<grid, 256, 0, s>>>((const double*)Oc, ldc, Ns, Np, T, ldt, 0, 1.0, diag_shift, 1);
  else if (dtype == 1)
    k_syrk<float, float><<<grid, 256, 0, s>>>((const float*)Oc, ldc, Ns, Np, T, ldt, 0, 1.0, diag_shift, 1);
  else
    return VMC_ERR_ARGS;
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// In-place lower Cholesky of T: FP64 tiles and panels, double-float trailing
// updates.  d_info set to 1 on a non-positive pivot.
int vmc_sr_cholesky(double* T, int64_t n, int64_t ldt, int* d_info, void* stream) {
  if (n <= 0 || ldt < n || !T || !d_info) return VMC_ERR_ARGS;
  cudaStream_t s = (cudaStream_t)stream;
  for (int64_t k0 = 0; k0 < n; k0 += TB) {
    int64_t nb = (n - k0) < TB ? (n - k0) : TB;
    k_potrf_tile<<<1, 256, 0, s>>>(T, ldt, k0, nb, d_info);
    int64_t rest = n - k0 - nb;
    if (rest > 0) {
      k_trsm_panel<<<(unsigned)((rest + 63) / 64), 64, 0, s>>>(T, ldt, n, k0, nb);
      int64_t nt = (rest + TB - 1) / TB;
      dim3 grid((unsigned)nt, (unsigned)nt);
      // trailing update of the lower triangle: A22 -= L21 L21^T (double-float on the FP32 pipes)
      k_syrk_df<<<grid, 256, 0, s>>>(T + k0, ldt, rest, nb, T, ldt, k0 + nb, -1.0);
    }
  }
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// Solve L L^T x = b in place on b (L from vmc_sr_cholesky).
int vmc_sr_cholesky_solve(const double* L, int64_t n, int64_t ldt, double* b, void* stream) {
  if (n <= 0 || ldt < n || !L || !b) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  for (int64_t k0 = 0; k0 < n; k0 += TRSV_NB) {   // L y = b
    const int nb = (int)((n - k0) < TRSV_NB ? (n - k0) : TRSV_NB);
    k_trsv_diag<<<1, TRSV_NB, 0, st>>>(L, ldt, k0, nb, b, 0);
    const int64_t rest = n - k0 - nb;
    if (rest > 0) k_trsv_upd_fwd<<<(unsigned)((rest + 7) / 8), 256, 0, st>>>(L, ldt, n, k0, nb, b);
  }
  const int64_t last = ((n - 1) / TRSV_NB) * TRSV_NB;
  for (int64_t k0 = last; k0 >= 0; k0 -= TRSV_NB) {   // L^T x = y
    const int nb = (int)((n - k0) < TRSV_NB ? (n - k0) : TRSV_NB);
    k_trsv_diag<<<1, TRSV_NB, 0, st>>>(L, ldt, k0, nb, b, 1);
    if (k0 > 0) k_trsv_upd_bwd<<<(unsigned)((k0 + 255) / 256), 256, 0, st>>>(L, ldt, k0, nb, b);
  }
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// b = (E - Ebar)/sqrt(Ns)
int vmc_sr_rhs(const double* E, int64_t Ns, double Ebar, double* b, void* stream) {
  if (Ns <= 0 || !E || !b) return VMC_ERR_ARGS;
  k_rhs<<<(unsigned)((Ns + 255) / 256), 256, 0, (cudaStream_t)stream>>>(E, Ns, Ebar, 1.0 / sqrt((double)Ns), b);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// dp = Oc^T x
int vmc_sr_update(const void* Oc, int dtype, int64_t Ns, int64_t Np, int64_t ldc, const double* x, double* dp,
                  void* stream) {
  if (Ns <= 0 || Np <= 0 || ldc < Np || !Oc || !x || !dp) return VMC_ERR_ARGS;
  unsigned grid = (unsigned)((Np + 255) / 256);
  if (dtype == 0)
    k_gemv_t<double><<<grid, 256, 0, (cudaStream_t)stream>>>((const double*)Oc, Ns, Np, ldc, x, dp);
  else if (dtype == 1)
    k_gemv_t<float><<<grid, 256, 0, (cudaStream_t)stream>>>((const float*)Oc, Ns, Np, ldc, x, dp);
  else
    return VMC_ERR_ARGS;
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

// g = <E O> - Ebar <O>
int vmc_energy_gradient(const void* O, int dtype, int64_t Ns, int64_t Np, int64_t ldo, const double* E, double Ebar,
                        double* g, void* stream) {
  if (Ns <= 0 || Np <= 0 || ldo < Np || !O || !E || !g) return VMC_ERR_ARGS;
  unsigned grid = (unsigned)((Np + 255) / 256);
  if (dtype == 0)
    k_egrad<double><<<grid, 256, 0, (cudaStream_t)stream>>>((const double*)O, Ns, Np, ldo, E, Ebar, g);
  else if (dtype == 1)
    k_egrad<float><<<grid, 256, 0, (cudaStream_t)stream>>>((const float*)O, Ns, Np, ldo, E, Ebar, g);
  else
    return VMC_ERR_ARGS;
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// General GEMM for the factored (Kronecker) SR pieces, CUDA cores:
//   C = beta * C + alpha * (op(A) op(B)) [elementwise * D]
// op(A) is M x K (ta = 0: A[m][k] row-major; ta = 1: A[k][m]), op(B) is K x N
// (tb = 0: B[k][n]; tb = 1: B[n][k]); optional per-k scale s[k] on op(A).
// Inputs FP32 or FP64 (accumulated in FP64 for FP64 inputs, FP32 per 64x64x16
// tile step otherwise), C and D FP64.  lower != 0 computes only tiles with
// tile-row >= tile-col and mirrors them (symmetric results).
// ---------------------------------------------------------------------------
namespace {
template <typename TI, typename TA>
__global__ void k_gemm_gen(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const TI* __restrict__ A,
                           int64_t lda, const TI* __restrict__ Bm, int64_t ldb, const TI* __restrict__ sk,
                           double beta, double* __restrict__ C, int64_t ldc, const double* __restrict__ D,
                           int64_t ldd, int lower) {
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (lower && bj > bi) return;
  __shared__ TA As[TK][TB + 1];
  __shared__ TA Bs[TK][TB + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t m0 = (int64_t)bi * TB, n0 = (int64_t)bj * TB;
  TileAcc<TA> T;
  T.zero();
  for (int64_t k0 = 0; k0 < K; k0 += TK) {
    for (int idx = threadIdx.x; idx < TB * TK; idx += 256) {
      int r, kk;
      if (ta) { kk = idx / TB; r = idx - kk * TB; } else { r = idx / TK; kk = idx - r * TK; }
      const int64_t gm = m0 + r, gk = k0 + kk;
      TA v = 0;
      if (gm < M && gk < K) {
        v = (TA)(ta ? A[gk * lda + gm] : A[gm * lda + gk]);
        if (sk) v *= (TA)sk[gk];
      }
      As[kk][r] = v;
    }
    for (int idx = threadIdx.x; idx < TB * TK; idx += 256) {
      int c, kk;
      if (tb) { c = idx / TK; kk = idx - c * TK; } else { kk = idx / TB; c = idx - kk * TB; }
      const int64_t gn = n0 + c, gk = k0 + kk;
      Bs[kk][c] = (gn < N && gk < K) ? (TA)(tb ? Bm[gn * ldb + gk] : Bm[gk * ldb + gn]) : (TA)0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      TA a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) { a[q] = As[kk][ty * 4 + q]; b[q] = Bs[kk][tx * 4 + q]; }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int r = 0; r < 4; ++r) T.acc[q][r] += a[q] * b[r];
      if ((kk & 3) == 3) T.fold();
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int64_t gm = m0 + ty * 4 + q, gn = n0 + tx * 4 + r;
      if (gm >= M || gn >= N) continue;
      if (lower && gn > gm) continue;
      double v = alpha * T.value(q, r);
      if (D) v *= D[gm * ldd + gn];
      const double out = (beta == 0.0 ? 0.0 : beta * C[gm * ldc + gn]) + v;
      C[gm * ldc + gn] = out;
      if (lower && gm != gn) C[gn * ldc + gm] = out;
    }
}

// T[a][b] += alpha * (-v[a] - v[b] + c0)
__global__ void k_rank_corr(int64_t n, double* __restrict__ T, int64_t ldt, const double* __restrict__ v, double c0,
                            double alpha) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * n) return;
  const int64_t a = idx / n, b = idx - a * n;
  T[a * ldt + b] += alpha * (c0 - v[a] - v[b]);
}

// v[a] = sum_k P[a][k] * H[a][k]
template <typename TI>
__global__ void k_rowdot(int64_t n, int64_t K, const double* __restrict__ P, int64_t ldp, const TI* __restrict__ H,
                         int64_t ldh, double* __restrict__ v) {
  const int64_t a = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (a >= n) return;
  double s = 0.0;
  for (int64_t k = lane; k < K; k += 32) s += P[a * ldp + k] * (double)H[a * ldh + k];
  s = vmc::warp_sum(s);
  if (lane == 0) v[a] = s;
}
}  // namespace

extern "C" {

int vmc_gemm(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const void* A, int64_t lda, const void* B,
             int64_t ldb, const void* sk, int dtype, double beta, double* C, int64_t ldc, const double* D,
             int64_t ldd, int lower, void* stream) {
  if (M <= 0 || N <= 0 || K < 0 || !A || !B || !C || (dtype != 0 && dtype != 1)) return VMC_ERR_ARGS;
  if (lower && M != N) return VMC_ERR_ARGS;
  const int64_t mt = (M + TB - 1) / TB, nt = (N + TB - 1) / TB;
  if (mt > 65535) return VMC_ERR_ARGS;
  dim3 grid((unsigned)nt, (unsigned)mt);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == 0)
    k_gemm_gen<double, double><<<grid, 256, 0, s>>>(ta, tb, M, N, K, alpha, (const double*)A, lda, (const double*)B,
                                                     ldb, (const double*)sk, beta, C, ldc, D, ldd, lower);
  else
    k_gemm_gen<float, float><<<grid, 256, 0, s>>>(ta, tb, M, N, K, alpha, (const float*)A, lda, (const float*)B, ldb,
                                                   (const float*)sk, beta, C, ldc, D, ldd, lower);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_sr_kron_correction(int64_t n, double* T, int64_t ldt, const double* P, int64_t ldp, const void* H, int dtype,
                           int64_t ldh, int64_t K, double mu_sq, double alpha, double* v_work, void* stream) {
  if (n <= 0 || K <= 0 || !T || !P || !H || !v_work || (dtype != 0 && dtype != 1)) return VMC_ERR_ARGS;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == 0)
    k_rowdot<double><<<(unsigned)((n + 7) / 8), 256, 0, s>>>(n, K, P, ldp, (const double*)H, ldh, v_work);
  else
    k_rowdot<float><<<(unsigned)((n + 7) / 8), 256, 0, s>>>(n, K, P, ldp, (const float*)H, ldh, v_work);
  const int64_t nn = n * n;
  k_rank_corr<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(n, T, ldt, v_work, mu_sq, alpha);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

}  // extern "C"
