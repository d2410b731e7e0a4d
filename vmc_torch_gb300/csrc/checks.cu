// Non-finite and zero-amplitude detection for amplitudes and log-derivative
// rows: the device side of the reference's _check_grads_amps
// (vmc_torch/GPU/vmc_utils.py:1330-1386), which raises ValueError when the
// amplitudes or the per-sample gradients hold NaN or Inf.
//
// Counters (caller-owned device words, cleared by the call):
//   [0] NaN amplitudes  [1] Inf amplitudes  [2] zero amplitudes (sign == 0)
//   [3] rows of O with a NaN or Inf entry
// Optional per-row (B) and per-column (Np) flags of O mark where the bad
// entries are, for the error message.
#include "common.cuh"

namespace {

__global__ void k_check_amp(const double* __restrict__ amp, const double* __restrict__ sign, int64_t B,
                            unsigned long long* __restrict__ c) {
  unsigned n_nan = 0, n_inf = 0, n_zero = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < B; i += (int64_t)gridDim.x * blockDim.x) {
    if (amp) {
      const double a = amp[i];
      n_nan += (a != a);
      n_inf += (a == INFINITY || a == -INFINITY);
    }
    if (sign) n_zero += (sign[i] == 0.0);
  }
  n_nan = vmc::warp_sum(n_nan);
  n_inf = vmc::warp_sum(n_inf);
  n_zero = vmc::warp_sum(n_zero);
  if ((threadIdx.x & 31) == 0) {
    if (n_nan) atomicAdd(&c[0], (unsigned long long)n_nan);
    if (n_inf) atomicAdd(&c[1], (unsigned long long)n_inf);
    if (n_zero) atomicAdd(&c[2], (unsigned long long)n_zero);
  }
}

// exponent field all ones <=> NaN or Inf
__device__ __forceinline__ bool bad_bits(float v) { return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u; }
__device__ __forceinline__ bool bad_bits(double v) {
  return ((unsigned long long)__double_as_longlong(v) & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
}

// One block per row; threads stride over the columns (coalesced).
template <typename T>
__global__ void k_check_rows(const T* __restrict__ O, int64_t Np, int64_t ld, unsigned long long* __restrict__ c,
                             uint8_t* __restrict__ row_bad, uint8_t* __restrict__ col_bad) {
  const int64_t r = blockIdx.x;
  const T* row = O + r * ld;
  int bad = 0;
  for (int64_t j = threadIdx.x; j < Np; j += blockDim.x) {
    if (bad_bits(row[j])) {
      bad = 1;
      if (col_bad) col_bad[j] = 1;
    }
  }
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) {
    if (bad) atomicAdd(&c[3], 1ull);
    if (row_bad) row_bad[r] = (uint8_t)bad;
  }
}

}  // namespace

extern "C" int vmc_check_finite(const double* amp, const double* sign, int64_t B, const void* O, int dtype,
                                int64_t Np, int64_t ldo, unsigned long long* d_counts, uint8_t* d_row_bad,
                                uint8_t* d_col_bad, unsigned long long* h_counts, void* stream) {
  if (B < 0 || !d_counts || (O && (Np < 0 || ldo < Np || (dtype != 0 && dtype != 1)))) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(d_counts, 0, 4 * sizeof(unsigned long long), st) != cudaSuccess) return VMC_ERR_CUDA;
  if (d_col_bad && O && Np > 0 && cudaMemsetAsync(d_col_bad, 0, (size_t)Np, st) != cudaSuccess) return VMC_ERR_CUDA;
  if (B > 0 && (amp || sign)) {
    const int64_t blocks = (B + 255) / 256 < 1024 ? (B + 255) / 256 : 1024;
    k_check_amp<<<(unsigned)blocks, 256, 0, st>>>(amp, sign, B, d_counts);
  }
  if (B > 0 && O && Np > 0) {
    if (dtype == 0)
      k_check_rows<double><<<(unsigned)B, 256, 0, st>>>((const double*)O, Np, ldo, d_counts, d_row_bad, d_col_bad);
    else
      k_check_rows<float><<<(unsigned)B, 256, 0, st>>>((const float*)O, Np, ldo, d_counts, d_row_bad, d_col_bad);
  }
  VMC_CUDA_CHECK_LAUNCH();
  if (!h_counts) return VMC_OK;
  if (cudaMemcpyAsync(h_counts, d_counts, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return VMC_ERR_CUDA;
  if (h_counts[0] || h_counts[1] || h_counts[3]) return VMC_ERR_NONFINITE;
  if (h_counts[2]) return VMC_ERR_SINGULAR;
  return VMC_OK;
}
