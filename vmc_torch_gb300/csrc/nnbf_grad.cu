// Hand-written adjoint of the NNBF log-amplitude: per-sample
// O_k(x) = d log|psi(x)| / d theta_k for every parameter, in the reference's
// parameter order [M_base, W0, b0, W1, b1, out_w, out_b].
//
//   A = M(x)[occ] (nf x nf),  G = A^-T = d log|det A| / dA,
//   Gbar (2N x nf): G scattered into the occupied rows (zero elsewhere)
//   dM_base = Gbar;  d out_b = s Gbar;  d out_w = (s Gbar) (x) h2   (outer product)
//   dh2 = s out_w^T vec(Gbar);  dz1 = dh2 * gelu'(z1);  db1 = dz1;  dW1 = dz1 (x) h1
//   dh1 = W1^T dz1;  dz0 = dh1 * gelu'(z0);  db0 = dz0;  dW0 = dz0 (x) n
//
// One block of 256 threads per configuration; the forward activations and the
// orbital matrix are recomputed (not stored between sampling and gradient
// evaluation), A^-1 comes from a Gauss-Jordan elimination with partial pivoting
// in shared memory.  The out_w block is either written in full (reference row
// layout) or as its two Kronecker factors s*Gbar (2N*nf) and h2 (256), which is
// what the sample-space SR solver consumes at scale.
#include "common.cuh"

using namespace vmc;

namespace {

constexpr int HID = 256;

template <typename T> __device__ __forceinline__ T erf_t(T x);
template <> __device__ __forceinline__ float erf_t<float>(float x) { return erff(x); }
template <> __device__ __forceinline__ double erf_t<double>(double x) { return erf(x); }
template <typename T> __device__ __forceinline__ T exp_t(T x);
template <> __device__ __forceinline__ float exp_t<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double exp_t<double>(double x) { return exp(x); }

template <typename T>
__device__ __forceinline__ T gelu_v(T x) { return T(0.5) * x * (T(1) + erf_t<T>(x * T(0.70710678118654752440))); }
// d/dx [x Phi(x)] = Phi(x) + x phi(x)
template <typename T>
__device__ __forceinline__ T gelu_d(T x) {
  return T(0.5) * (T(1) + erf_t<T>(x * T(0.70710678118654752440))) +
         x * exp_t<T>(T(-0.5) * x * x) * T(0.39894228040143267794);
}

template <typename T>
struct GradNet {
  const T* w0t;    // (2N, 256)   W0^T
  const T* b0;     // (256)
  const T* w1;     // (256, 256)  W1 [out][in]
  const T* w1t;    // (256, 256)  W1^T [in][out]
  const T* b1;     // (256)
  const T* outw;   // (2N*nf, 256)
  const T* outwt;  // (256, 2N*nf)
  const T* outb;   // (2N*nf)
  const T* mbase;  // (2N, nf)
};

template <typename T>
__global__ void __launch_bounds__(256) k_nnbf_grad(GradNet<T> net, int N, int nf, T s, const uint64_t* __restrict__ occ,
                                                   T* __restrict__ Ofull, int64_t ldf, T* __restrict__ Odense,
                                                   int64_t ldd, T* __restrict__ kg, T* __restrict__ kh,
                                                   double* __restrict__ logabs_out, double* __restrict__ sign_out) {
  extern __shared__ __align__(16) uint8_t gsm[];
  const int tid = threadIdx.x;
  const int64_t w = blockIdx.x;
  const int n_orb = 2 * N;
  const int ldA = nf + 1;
  T* A = reinterpret_cast<T*>(gsm);           // nf x (nf+1)
  T* Ai = A + nf * ldA;                        // nf x (nf+1)
  T* z0 = Ai + nf * ldA;                       // 256
  T* h1 = z0 + HID;                            // 256
  T* z1 = h1 + HID;                            // 256
  T* h2 = z1 + HID;                            // 256
  T* dz1 = h2 + HID;                           // 256
  T* fac = dz1 + HID;                          // 64
  int* orbs = reinterpret_cast<int*>(fac + 64);   // 64
  int* piv = orbs + 64;                            // [0]=pivot row, [1]=ok

  const uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  const bool count_ok = (__popcll(up) + __popcll(dn)) == nf;
  if (tid < n_orb && orb_occupied(up, dn, N, tid)) {
    const int p = orb_prefix(up, dn, N, tid);
    if (p < 64) orbs[p] = tid;
  }
  if (tid == 0) piv[1] = count_ok ? 1 : 0;
  __syncthreads();
  // ---- forward recompute ----
  {
    T acc = net.b0[tid];
    if (count_ok)
      for (int k = 0; k < nf; ++k) acc += net.w0t[(size_t)orbs[k] * HID + tid];
    z0[tid] = acc;
    h1[tid] = gelu_v<T>(acc);
  }
  __syncthreads();
  {
    T acc = net.b1[tid];
    for (int k = 0; k < HID; ++k) acc += net.w1t[(size_t)k * HID + tid] * h1[k];
    z1[tid] = acc;
    h2[tid] = gelu_v<T>(acc);
  }
  __syncthreads();
  const int nout = n_orb * nf;
  for (int idx = tid; idx < nf * nf; idx += 256) {
    const int pos = idx / nf, c = idx - pos * nf;
    T v = 0;
    if (count_ok) {
      const int j = orbs[pos] * nf + c;
      T acc = net.outb[j];
      for (int k = 0; k < HID; ++k) acc += net.outwt[(size_t)k * nout + j] * h2[k];
      v = net.mbase[j] + s * acc;
    }
    A[pos * ldA + c] = v;
    Ai[pos * ldA + c] = (pos == c) ? T(1) : T(0);
  }
  __syncthreads();
  // ---- Gauss-Jordan inverse with partial pivoting ----
  double la = 0.0;
  int neg = 0;
  for (int k = 0; k < nf && piv[1] == 1; ++k) {
    if (tid < 32) {
      double best = -1.0;
      int bi = k;
      for (int r = k + tid; r < nf; r += 32) {
        double v = fabs((double)A[r * ldA + k]);
        if (v != v) v = INFINITY;   // NaN ranks first, so that it is detected
        if (v > best) { best = v; bi = r; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(VMC_FULL_MASK, best, o);
        const int oi = __shfl_xor_sync(VMC_FULL_MASK, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tid == 0) {
        piv[0] = bi;
        if (!(best > 0.0) || !isfinite(best)) piv[1] = isfinite(best) ? 0 : -1;
      }
    }
    __syncthreads();
    if (piv[1] != 1) break;
    const int p = piv[0];
    if (p != k) {
      for (int c = tid; c < 2 * nf; c += 256) {
        T* M = c < nf ? A : Ai;
        const int cc = c < nf ? c : c - nf;
        const T t0 = M[k * ldA + cc];
        M[k * ldA + cc] = M[p * ldA + cc];
        M[p * ldA + cc] = t0;
      }
      neg ^= 1;
    }
    __syncthreads();
    const T pv = A[k * ldA + k];
    la += log(fabs((double)pv));
    neg ^= (pv < T(0));
    __syncthreads();
    const T ipv = T(1) / pv;
    for (int c = tid; c < 2 * nf; c += 256) {
      if (c < nf) A[k * ldA + c] *= ipv; else Ai[k * ldA + c - nf] *= ipv;
    }
    for (int r = tid; r < nf; r += 256) fac[r] = (r == k) ? T(0) : A[r * ldA + k];
    __syncthreads();
    for (int idx = tid; idx < nf * 2 * nf; idx += 256) {
      const int r = idx / (2 * nf), c = idx - r * 2 * nf;
      if (r == k) continue;
      if (c < nf) A[r * ldA + c] -= fac[r] * A[k * ldA + c];
      else Ai[r * ldA + c - nf] -= fac[r] * Ai[k * ldA + c - nf];
    }
    __syncthreads();
  }
  // piv[1]: 1 regular, 0 singular (or wrong electron count), -1 non-finite entry
  const bool ok = piv[1] == 1;
  if (tid == 0) {
    const double qnan = __longlong_as_double(0x7ff8000000000000ll);
    if (logabs_out) logabs_out[w] = ok ? la : (piv[1] < 0 ? qnan : -INFINITY);
    if (sign_out) sign_out[w] = ok ? (neg ? -1.0 : 1.0) : (piv[1] < 0 ? qnan : 0.0);
  }
  // Gbar[orbs[pos]][c] = Ainv[c][pos]; stored as G[pos][c] in A (reuse)
  for (int idx = tid; idx < nf * nf; idx += 256) {
    const int pos = idx / nf, c = idx - pos * nf;
    A[pos * ldA + c] = ok ? Ai[c * ldA + pos] : T(0);
  }
  __syncthreads();
  // ---- backward through the MLP ----
  {
    // dh2[k] = s * sum_{pos,c} G[pos][c] * out_w[orbs[pos]*nf + c][k]
    T acc = 0;
    if (ok)
      for (int pos = 0; pos < nf; ++pos) {
        const T* wr = net.outw + (size_t)orbs[pos] * nf * HID + tid;
        const T* g = A + pos * ldA;
        for (int c = 0; c < nf; ++c) acc += g[c] * wr[(size_t)c * HID];
      }
    dz1[tid] = s * acc * gelu_d<T>(z1[tid]);
  }
  __syncthreads();
  T dz0;
  {
    T acc = 0;
    for (int j = 0; j < HID; ++j) acc += net.w1[(size_t)j * HID + tid] * dz1[j];
    dz0 = acc * gelu_d<T>(z0[tid]);
  }
  __syncthreads();
  // stash dz0 in z0 (z0 no longer needed)
  z0[tid] = dz0;
  __syncthreads();
  // ---- write O ----
  // offsets in the reference order
  const int64_t oM = 0, oW0 = (int64_t)n_orb * nf, ob0 = oW0 + (int64_t)HID * n_orb, oW1 = ob0 + HID,
                ob1 = oW1 + (int64_t)HID * HID, oOW = ob1 + HID, oOB = oOW + (int64_t)nout * HID;
  // the dense row omits the out_w block: same order with out_b following b1
  for (int pass = 0; pass < 2; ++pass) {
    T* row = pass == 0 ? (Ofull ? Ofull + w * ldf : nullptr) : (Odense ? Odense + w * ldd : nullptr);
    if (!row) continue;
    const int64_t obB = pass == 0 ? oOB : oOW;
    for (int idx = tid; idx < nout; idx += 256) {
      const int o = idx / nf, c = idx - o * nf;
      T g = 0;
      if (ok && orb_occupied(up, dn, N, o)) g = A[orb_prefix(up, dn, N, o) * ldA + c];
      row[oM + idx] = g;
      row[obB + idx] = s * g;
    }
    for (int idx = tid; idx < HID * n_orb; idx += 256) {
      const int j = idx / n_orb, i = idx - j * n_orb;
      row[oW0 + idx] = orb_occupied(up, dn, N, i) ? z0[j] : T(0);
    }
    row[ob0 + tid] = z0[tid];
    for (int idx = tid; idx < HID * HID; idx += 256) {
      const int j = idx / HID, k = idx - j * HID;
      row[oW1 + idx] = dz1[j] * h1[k];
    }
    row[ob1 + tid] = dz1[tid];
    if (pass == 0) {
      for (int64_t idx = tid; idx < (int64_t)nout * HID; idx += 256) {
        const int j = (int)(idx / HID), k = (int)(idx - (int64_t)j * HID);
        const int o = j / nf, c = j - o * nf;
        T g = 0;
        if (ok && orb_occupied(up, dn, N, o)) g = A[orb_prefix(up, dn, N, o) * ldA + c];
        row[oOW + idx] = s * g * h2[k];
      }
    }
  }
  if (kg) {
    for (int idx = tid; idx < nout; idx += 256) {
      const int o = idx / nf, c = idx - o * nf;
      T g = 0;
      if (ok && orb_occupied(up, dn, N, o)) g = A[orb_prefix(up, dn, N, o) * ldA + c];
      kg[w * (int64_t)nout + idx] = s * g;
    }
  }
  if (kh) kh[w * HID + tid] = h2[tid];
}

template <typename T>
size_t grad_smem(int nf) {
  return (size_t)(2 * nf * (nf + 1) + 5 * HID + 64) * sizeof(T) + 2 * 64 * sizeof(int) + 16;
}

}  // namespace

extern "C" int vmc_nnbf_logpsi_grad(int prec, const void* const* gnet, int n_sites, int nf, int hidden, double bf_scale,
                                    const uint64_t* occ, int64_t B, void* O_full, int64_t ld_full, void* O_dense,
                                    int64_t ld_dense, void* kron_g, void* kron_h, double* logabs, double* sign,
                                    void* stream) {
  if (n_sites < 1 || n_sites > 64 || nf < 1 || nf > 64 || hidden != HID || B < 0 || (prec != 0 && prec != 1))
    return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!gnet || !occ) return VMC_ERR_ARGS;
  const int64_t n_orb = 2 * n_sites, nout = n_orb * nf;
  const int64_t Np = nout + HID * n_orb + HID + HID * HID + HID + nout * HID + nout;
  const int64_t Nd = Np - nout * HID;
  if (O_full && ld_full < Np) return VMC_ERR_ARGS;
  if (O_dense && ld_dense < Nd) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  if (prec == 0) {
    GradNet<float> g{(const float*)gnet[0], (const float*)gnet[1], (const float*)gnet[2], (const float*)gnet[3],
                     (const float*)gnet[4], (const float*)gnet[5], (const float*)gnet[6], (const float*)gnet[7],
                     (const float*)gnet[8]};
    const size_t sm = grad_smem<float>(nf);
    cudaFuncSetAttribute(k_nnbf_grad<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_nnbf_grad<float><<<(unsigned)B, 256, sm, st>>>(g, n_sites, nf, (float)bf_scale, occ, (float*)O_full, ld_full,
                                                     (float*)O_dense, ld_dense, (float*)kron_g, (float*)kron_h, logabs,
                                                     sign);
  } else {
    GradNet<double> g{(const double*)gnet[0], (const double*)gnet[1], (const double*)gnet[2], (const double*)gnet[3],
                      (const double*)gnet[4], (const double*)gnet[5], (const double*)gnet[6], (const double*)gnet[7],
                      (const double*)gnet[8]};
    const size_t sm = grad_smem<double>(nf);
    cudaFuncSetAttribute(k_nnbf_grad<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_nnbf_grad<double><<<(unsigned)B, 256, sm, st>>>(g, n_sites, nf, bf_scale, occ, (double*)O_full, ld_full,
                                                      (double*)O_dense, ld_dense, (double*)kron_g, (double*)kron_h,
                                                      logabs, sign);
  }
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}
