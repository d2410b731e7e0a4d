// Fermionic PEPS amplitudes (fPEPS_Model_GPU, vmc_torch/GPU/models/pureTNS.py:24-160)
// by exact row-boundary contraction, one CTA per configuration.
//
// Ansatz.  Site tensors T[r][c][s][l][u][r'][d] (bond dimension D, quimb
// states s), Z2-graded (bond index parity = index & 1, every tensor even),
// open legs at index 0.  The Grassmann contraction with the bond variables of
// a site ordered (l, u, d, r') and sites in row-major order reduces to
//     psi(x) = (-1)^{K(K-1)/2} * Z(T~[x]),
// K = number of singly-occupied sites, Z the plain contraction, and T~ equal
// to T except that for rows r >= 1 every element is multiplied by
// (-1)^{p(u) * (p(l) + n_left)} with n_left the electrons to the left of the
// site in its row.  The sign is applied while a column is loaded.
//
// Contraction.  Rows [0, mid-1] (mid = Lx/2 - 1) form a top MPS M[a][u][b] and
// rows [mid+2, Lx-1] a bottom MPS N[a'][d][b'], both of bond DA = D^mid, built
// per column from that column's tensors.  The two middle rows are swept left
// to right with the environment E[a][l2][l3][a'] (DA*D*D*DA values):
//   Y [u2][l2][l3][a'] = sum_a     M[a][u2][b] E[a][l2][l3][a']
//   X2[r2][d2][l3][a'] = sum_l2,u2 A2[l2][u2][r2][d2] Y[u2][l2][l3][a']
//   X3[r2][r3][d3][a'] = sum_l3,d2 A3[l3][d2][r3][d3] X2[r2][d2][l3][a']
//   E'[b][r2][r3][b']  = sum_d3,a' X3[r2][r3][d3][a'] N[a'][d3][b']
// one warp per top-bond slice b, so the per-slice intermediates (D^3*DA
// values) stay in the warp's own shared-memory buffer.  After every column
// the environment is rescaled by a power of two (exact) and the exponent is
// accumulated, so FP32 never overflows.  This is the chi -> infinity limit of
// the reference's boundary contraction (which truncates the boundary MPS to
// max_bond with SVDs); at 6x6, D = 4 it costs ~12 MFLOP per amplitude.
#include <climits>
#include <type_traits>

#include "common.cuh"
#include "vmc_gb300.h"

using namespace vmc;

namespace {

template <typename T, int D, int DA>
struct Peps {
  static constexpr int D4 = D * D * D * D;
  static constexpr int ESZ = DA * D * D * DA;  // environment
  static constexpr int SL = D * D * D * DA;    // per-slice intermediate
  static constexpr int MSZ = DA * D * DA;      // boundary MPS column
  // warps per CTA (one per top-bond slice; FP64 at DA = 16 takes two slices a warp for registers)
  static constexpr int NW = (sizeof(T) == 8 && DA > 8) ? 8 : (DA < 16 ? DA : 16);
  static constexpr int NT = 32 * NW;
  static constexpr int R = (SL + 31) / 32;     // outputs per lane per step
  static constexpr bool FAST = std::is_same<T, float>::value && D == 4 && DA == 16;  // register-tiled step
  static constexpr int BUFW = FAST ? 1540 : SL;  // per-warp buffer
  // shared-memory layout (elements of T); the boundary builder's two scratch
  // columns live in the free environment buffer (ESZ >= 2 MSZ)
  static constexpr size_t off_M = 0, off_N = off_M + MSZ, off_E0 = off_N + MSZ, off_E1 = off_E0 + ESZ,
                          off_buf = off_E1 + ESZ,
                          off_red = off_buf + (size_t)NW * BUFW, off_col = off_red + 32;
  // + 4 broadcast doubles (8-byte aligned) and the environment cache's 2 x 17 exponents
  static size_t smem_bytes(int Lx) { return (off_col + (size_t)Lx * D4) * sizeof(T) + 8 + 4 * sizeof(double) + 34 * sizeof(int); }
  static __device__ double* bcast(T* sm, int Lx) {
    return reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(sm + off_col + (size_t)Lx * D4) + 7) & ~uintptr_t(7));
  }
  static __device__ int* exps(T* sm, int Lx) { return reinterpret_cast<int*>(bcast(sm, Lx) + 4); }
};

__device__ __forceinline__ uint64_t row_mask(int r, int Ly, int c) {  // sites (r, 0..c-1)
  return c == 0 ? 0ull : (bits_below(c) << (r * Ly));
}

template <typename T>
__device__ __forceinline__ int exp2_of(T m);
template <>
__device__ __forceinline__ int exp2_of<float>(float m) { return ilogbf(m); }
template <>
__device__ __forceinline__ int exp2_of<double>(double m) { return ilogb(m); }

// Build one boundary MPS column into dst: rows rows[0..nr-1] of tcol, where
// the first row contributes its (l, ., r, .) slice with the outer leg fixed
// to 0.  top = true: M[a][d][b] from row 0 down; false: N[a][u][b] from row
// Lx-1 up.  ping/pong are scratch of MSZ each.  CTA-wide, ends synchronised.
template <typename T, int D, int DA>
__device__ void build_boundary(const T* tcol, int Lx, bool top, T* dst, T* ping, T* pong, T scale,
                               bool transposed = false) {
  using P = Peps<T, D, DA>;
  const int nr = Lx / 2 - 1;
  const int r0 = top ? 0 : Lx - 1;
  // first row: (l, v, r) with v the inner vertical leg
  T* cur = (nr == 1) ? dst : ping;
  {
    const T* A = tcol + (size_t)r0 * P::D4;
    for (int o = threadIdx.x; o < D * D * D; o += blockDim.x) {
      const int l = o / (D * D), v = (o / D) % D, r = o % D;
      // top: A[l][0][r][v]; bottom: A[l][v][r][0]
      const T val = top ? A[((l * D + 0) * D + r) * D + v] : A[((l * D + v) * D + r) * D + 0];
      if (nr == 1) dst[transposed ? (r * D + l) * D + v : o] = val * scale;
      else cur[o] = val;
    }
  }
  __syncthreads();
  int da = D;
  for (int k = 1; k < nr; ++k) {
    const int rr = top ? k : Lx - 1 - k;
    const T* A = tcol + (size_t)rr * P::D4;
    T* nxt = (k == nr - 1) ? dst : (cur == ping ? pong : ping);
    const int dn = da * D;
    const bool tr = transposed && k == nr - 1;  // walk the destination order: conflict-free stores
    for (int o = threadIdx.x; o < dn * D * dn; o += blockDim.x) {
      const int an = tr ? (o / D) % dn : o / (D * dn);
      const int v2 = tr ? o % D : (o / dn) % D;
      const int bn = tr ? o / (D * dn) : o % dn;
      const int a = an / D, l = an % D, b = bn / D, r = bn % D;
      T acc = 0;
#pragma unroll
      for (int v = 0; v < D; ++v) {
        // top: sum_v M[a][v][b] A[l][v][r][v2]; bottom: sum_v N[a][v][b] A[l][v2][r][v]
        const T av = top ? A[((l * D + v) * D + r) * D + v2] : A[((l * D + v2) * D + r) * D + v];
        acc += cur[(a * D + v) * da + b] * av;
      }
      if (k == nr - 1) dst[o] = acc * scale;
      else nxt[o] = acc;
    }
    __syncthreads();
    cur = nxt;
    da = dn;
  }
}

// One top-bond slice b of the column step, thread per output (generic shapes
// and FP64).  Returns max |E'| over the slice.
template <typename T, int D, int DA>
struct SliceStep {
  static __device__ __forceinline__ T run(const T* __restrict__ Mc, const T* __restrict__ E0, const T* __restrict__ A2,
                                          const T* __restrict__ A3, const T* __restrict__ Nc, T* __restrict__ buf,
                                          T* __restrict__ E1, int b, int lane) {
    using P = Peps<T, D, DA>;
    T wmax = 0;
    T r[P::R];
    // Y[u2][l2][l3][a']
#pragma unroll
    for (int q = 0; q < P::R; ++q) {
      const int o = lane + 32 * q;
      T acc = 0;
      if (o < P::SL) {
        const int u2 = o / (D * D * DA), rest = o % (D * D * DA);
#pragma unroll 4
        for (int a = 0; a < DA; ++a) acc += Mc[(a * D + u2) * DA + b] * E0[a * (D * D * DA) + rest];
      }
      r[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < P::R; ++q)
      if (lane + 32 * q < P::SL) buf[lane + 32 * q] = r[q];
    __syncwarp();
    // X2[r2][d2][l3][a']
#pragma unroll
    for (int q = 0; q < P::R; ++q) {
      const int o = lane + 32 * q;
      T acc = 0;
      if (o < P::SL) {
        const int r2 = o / (D * D * DA), d2 = (o / (D * DA)) % D, l3a = o % (D * DA);
#pragma unroll
        for (int l2 = 0; l2 < D; ++l2)
#pragma unroll
          for (int u2 = 0; u2 < D; ++u2)
            acc += A2[((l2 * D + u2) * D + r2) * D + d2] * buf[(u2 * D + l2) * (D * DA) + l3a];
      }
      r[q] = acc;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < P::R; ++q)
      if (lane + 32 * q < P::SL) buf[lane + 32 * q] = r[q];
    __syncwarp();
    // X3[r2][r3][d3][a']
#pragma unroll
    for (int q = 0; q < P::R; ++q) {
      const int o = lane + 32 * q;
      T acc = 0;
      if (o < P::SL) {
        const int r2 = o / (D * D * DA), r3 = (o / (D * DA)) % D, d3 = (o / DA) % D, ap = o % DA;
#pragma unroll
        for (int l3 = 0; l3 < D; ++l3)
#pragma unroll
          for (int d2 = 0; d2 < D; ++d2)
            acc += A3[((l3 * D + d2) * D + r3) * D + d3] * buf[((r2 * D + d2) * D + l3) * DA + ap];
      }
      r[q] = acc;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < P::R; ++q)
      if (lane + 32 * q < P::SL) buf[lane + 32 * q] = r[q];
    __syncwarp();
    // E'[b][r2][r3][b']
    for (int o = lane; o < D * D * DA; o += 32) {
      const int rr = o / DA, bp = o % DA;
      T acc = 0;
#pragma unroll 4
      for (int d3 = 0; d3 < D; ++d3)
        for (int ap = 0; ap < DA; ++ap) acc += buf[(rr * D + d3) * DA + ap] * Nc[(ap * D + d3) * DA + bp];
      E1[b * (D * D * DA) + o] = acc;
      wmax = fmax(wmax, fabs(acc));
    }
    __syncwarp();
    return wmax;
  }
};

// Register-tiled slice step for FP32, D = 4, DA = 16 (Lx = 6 at D = 4).  Lane
// (h, a') = (lane >> 4, lane & 15) holds Y and X2 for l3 in {h, h+2}: the
// (l2, u2) contraction is lane-local; the (l3, d2) contraction takes the other
// two l3 values from lane ^ 16 (16 shuffles) with lane h keeping
// r2 in {2h, 2h+1}; the (d3, a') contraction goes through the warp's buffer
// (X3 stored [h][d3][a'][r2 r3] with 12-float rows, so that 8 consecutive
// lanes' 16-byte stores hit distinct bank groups, and the halves 772 floats
// apart, so that their broadcast reads do too).  M arrives transposed,
// [b][a][u2], for one 16-byte load per a.
template <>
struct SliceStep<float, 4, 16> {
  static constexpr int HALF = 772;
  static __device__ __forceinline__ float run(const float* __restrict__ Mc, const float* __restrict__ E0,
                                              const float* __restrict__ A2, const float* __restrict__ A3,
                                              const float* __restrict__ Nc, float* __restrict__ buf,
                                              float* __restrict__ E1, int b, int lane) {
    const int h = lane >> 4, ap = lane & 15;
    // ---- Y[u2][l2][j] (l3 = h + 2j) = sum_a M[a][u2][b] E[a][l2][l3][a'] ----
    float y[4][4][2];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int l = 0; l < 4; ++l) y[u][l][0] = y[u][l][1] = 0.f;
#pragma unroll 2
    for (int a = 0; a < 16; ++a) {
      const float4 m4 = *reinterpret_cast<const float4*>(Mc + (b * 16 + a) * 4);  // M stored [b][a][u2]
      const float m[4] = {m4.x, m4.y, m4.z, m4.w};
      const float* e = E0 + a * 256 + h * 16 + ap;
#pragma unroll
      for (int l = 0; l < 4; ++l)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const float ev = e[l * 64 + j * 32];
#pragma unroll
          for (int u = 0; u < 4; ++u) y[u][l][j] = fmaf(m[u], ev, y[u][l][j]);
        }
    }
    // ---- X2[r2][d2][j] = sum_{l2,u2} A2[l2][u2][r2][d2] Y[u2][l2][j] ----
    float x2[4][4][2];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int d = 0; d < 4; ++d) x2[r][d][0] = x2[r][d][1] = 0.f;
#pragma unroll
    for (int l = 0; l < 4; ++l)
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const float4 a4 = *reinterpret_cast<const float4*>(A2 + ((l * 4 + u) * 4 + r) * 4);
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            const float yv = y[u][l][j];
            x2[r][0][j] = fmaf(a4.x, yv, x2[r][0][j]);
            x2[r][1][j] = fmaf(a4.y, yv, x2[r][1][j]);
            x2[r][2][j] = fmaf(a4.z, yv, x2[r][2][j]);
            x2[r][3][j] = fmaf(a4.w, yv, x2[r][3][j]);
          }
        }
    // ---- exchange: keep r2 = 2h + rr; own l3 = h + 2j, partner l3 = 1 - h + 2j ----
    float zo[2][4][2], zp[2][4][2];
#pragma unroll
    for (int rr = 0; rr < 2; ++rr)
#pragma unroll
      for (int d = 0; d < 4; ++d)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const float lo = x2[rr][d][j], hi = x2[2 + rr][d][j];
          zo[rr][d][j] = h ? hi : lo;
          zp[rr][d][j] = __shfl_xor_sync(VMC_FULL_MASK, h ? lo : hi, 16);
        }
    // ---- X3[rr][r3][d3] = sum_{l3,d2} A3[l3][d2][r3][d3] X2[r2][d2][l3] ----
    float x3[2][4][4];
#pragma unroll
    for (int rr = 0; rr < 2; ++rr)
#pragma unroll
      for (int r = 0; r < 4; ++r) x3[rr][r][0] = x3[rr][r][1] = x3[rr][r][2] = x3[rr][r][3] = 0.f;
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int d2 = 0; d2 < 4; ++d2)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const float4 ao = *reinterpret_cast<const float4*>(A3 + (((h + 2 * j) * 4 + d2) * 4 + r) * 4);
          const float4 aq = *reinterpret_cast<const float4*>(A3 + (((1 - h + 2 * j) * 4 + d2) * 4 + r) * 4);
#pragma unroll
          for (int rr = 0; rr < 2; ++rr) {
            const float vo = zo[rr][d2][j], vp = zp[rr][d2][j];
            x3[rr][r][0] = fmaf(ao.x, vo, fmaf(aq.x, vp, x3[rr][r][0]));
            x3[rr][r][1] = fmaf(ao.y, vo, fmaf(aq.y, vp, x3[rr][r][1]));
            x3[rr][r][2] = fmaf(ao.z, vo, fmaf(aq.z, vp, x3[rr][r][2]));
            x3[rr][r][3] = fmaf(ao.w, vo, fmaf(aq.w, vp, x3[rr][r][3]));
          }
        }
    // ---- stage X3 as [h][d3][a'][rr*4 + r3], rows padded to 12 floats ----
    float* xb = buf + h * HALF;
#pragma unroll
    for (int d3 = 0; d3 < 4; ++d3) {
      float4* dst = reinterpret_cast<float4*>(xb + (d3 * 16 + ap) * 12);
      dst[0] = make_float4(x3[0][0][d3], x3[0][1][d3], x3[0][2][d3], x3[0][3][d3]);
      dst[1] = make_float4(x3[1][0][d3], x3[1][1][d3], x3[1][2][d3], x3[1][3][d3]);
    }
    __syncwarp();
    // ---- E'[b][2h + rr][r3][b'] = sum_{d3,a'} X3 N[a'][d3][b'], b' = ap ----
    float acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = 0.f;
#pragma unroll 4
    for (int q = 0; q < 64; ++q) {  // q = d3 * 16 + a'
      const int d3 = q >> 4, a2 = q & 15;
      const float n = Nc[(a2 * 4 + d3) * 16 + ap];
      const float4 v0 = *reinterpret_cast<const float4*>(xb + q * 12);
      const float4 v1 = *reinterpret_cast<const float4*>(xb + q * 12 + 4);
      acc[0] = fmaf(v0.x, n, acc[0]); acc[1] = fmaf(v0.y, n, acc[1]);
      acc[2] = fmaf(v0.z, n, acc[2]); acc[3] = fmaf(v0.w, n, acc[3]);
      acc[4] = fmaf(v1.x, n, acc[4]); acc[5] = fmaf(v1.y, n, acc[5]);
      acc[6] = fmaf(v1.z, n, acc[6]); acc[7] = fmaf(v1.w, n, acc[7]);
    }
    float wmax = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {  // row (r2 * 4 + r3) = 8h + (k ^ h): the halves hit different banks
      const float v = h ? acc[k ^ 1] : acc[k];
      E1[b * 256 + (8 * h + (k ^ h)) * 16 + ap] = v;
      wmax = fmaxf(wmax, fabsf(v));
    }
    __syncwarp();
    return wmax;
  }
};

constexpr int EXP_ZERO = INT_MIN, EXP_BAD = INT_MAX;

// One column step of the two-row sweep, CTA-wide: dst = f_c(src) for the
// configuration (up, dn).  mirror = true contracts from the right (the
// column's left and right legs exchanged), so right environments F_c =
// dZ/dE_c come from the same code: F_c = f_c~(F_{c+1}).  src and dst are
// distinct shared-memory environments.  dst is rescaled by 2^-e in place;
// returns e, EXP_ZERO when dst vanishes, EXP_BAD when it is not finite.
template <typename T, int D, int DA>
__device__ int col_step(const T* __restrict__ tens, int Lx, int Ly, uint64_t up, uint64_t dn, int c, bool mirror,
                        const T* src, T* dst, T* sm) {
  using P = Peps<T, D, DA>;
  T* Mc = sm + P::off_M;
  T* Nc = sm + P::off_N;
  T* red = sm + P::off_red;
  T* tcol = sm + P::off_col;
  T* scr = sm + P::off_buf;  // the warps' buffers are free outside the slice step
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* buf = sm + P::off_buf + (size_t)warp * P::BUFW;
  const int mid = Lx / 2 - 1;
  __syncthreads();  // earlier readers of tcol / M / N / the buffers / src are done
  for (int o = threadIdx.x; o < Lx * P::D4; o += blockDim.x) {
    const int r = o / P::D4, idx = o % P::D4;
    int l = idx / (D * D * D);
    const int u = (idx / (D * D)) % D, rr = (idx / D) % D, d = idx % D;
    int sidx = idx;
    if (mirror) {  // mirrored element (l, u, rr, d) is the original (rr, u, l, d)
      sidx = ((rr * D + u) * D + l) * D + d;
      l = rr;
    }
    const int site = r * Ly + c;
    T v = tens[((size_t)site * 4 + site_state(up, dn, site)) * P::D4 + sidx];
    if (r > 0) {
      const uint64_t m = row_mask(r, Ly, c);
      if (u & (l ^ (__popcll(up & m) + __popcll(dn & m))) & 1) v = -v;
    }
    tcol[o] = v;
  }
  __syncthreads();
  build_boundary<T, D, DA>(tcol, Lx, true, Mc, scr, scr + P::MSZ, T(1), P::FAST);
  build_boundary<T, D, DA>(tcol, Lx, false, Nc, scr, scr + P::MSZ, T(1));
  const T* A2 = tcol + (size_t)mid * P::D4;
  const T* A3 = tcol + (size_t)(mid + 1) * P::D4;
  T wmax = 0;
  for (int b = warp; b < DA; b += P::NW)
    wmax = fmax(wmax, SliceStep<T, D, DA>::run(Mc, src, A2, A3, Nc, buf, dst, b, lane));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) wmax = fmax(wmax, __shfl_xor_sync(VMC_FULL_MASK, wmax, o));
  if (lane == 0) red[warp] = wmax;
  __syncthreads();
  T m = 0;
  for (int k = 0; k < P::NW; ++k) m = fmax(m, red[k]);
  if (m == T(0)) return EXP_ZERO;
  if (!(m < T(INFINITY))) return EXP_BAD;
  const int e = exp2_of<T>(m);
  const T sc = (T)ldexp(1.0, -e);
  for (int o = threadIdx.x; o < P::ESZ; o += blockDim.x) dst[o] *= sc;
  return e;
}

// (sign, log|psi|) from a normalised contraction value v * 2^expo and the
// configuration's global sign (-1)^{K(K-1)/2}.
__device__ __forceinline__ void finish_amp(double v, int expo, bool bad, uint64_t up, uint64_t dn, double& sgn,
                                           double& la) {
  const int K = __popcll(up ^ dn);
  const double g = ((K * (K - 1) / 2) & 1) ? -1.0 : 1.0;
  if (bad || !isfinite(v)) {
    sgn = 0.0;
    la = NAN;
  } else if (v == 0.0) {
    sgn = 0.0;
    la = -INFINITY;
  } else {
    sgn = v < 0 ? -g : g;
    la = log(fabs(v)) + (double)expo * 0.69314718055994530942;
  }
}

// finish_amp evaluated once (thread 0) and broadcast: the FP64 log on every
// thread would occupy GB300's narrow FP64 pipe.
__device__ __forceinline__ void cta_finish(double v, int expo, bool bad, uint64_t up, uint64_t dn, double& sgn,
                                           double& la, double* bc) {
  __syncthreads();
  if (threadIdx.x == 0) {
    finish_amp(v, expo, bad, up, dn, sgn, la);
    bc[0] = sgn;
    bc[1] = la;
  }
  __syncthreads();
  sgn = bc[0];
  la = bc[1];
}

// Metropolis decision u < |psi'|^2 / |psi|^2, taken by thread 0 and broadcast.
__device__ __forceinline__ bool cta_accept(float u_acc, double la1, double la, double* bc) {
  __syncthreads();
  if (threadIdx.x == 0) {
    bool a;
    if (!(la1 > -INFINITY)) a = false;  // zero or NaN
    else if (la == -INFINITY) a = true;
    else a = (double)u_acc < exp(2.0 * (la1 - la));
    bc[2] = a ? 1.0 : 0.0;
  }
  __syncthreads();
  return bc[2] != 0.0;
}

// psi(up, dn) for the CTA by a full left-to-right sweep.  Every thread
// returns the same (sign, log|psi|).
template <typename T, int D, int DA>
__device__ void peps_amp(const T* __restrict__ tens, int Lx, int Ly, uint64_t up, uint64_t dn, T* sm, double& sgn,
                         double& la) {
  using P = Peps<T, D, DA>;
  T* E0 = sm + P::off_E0;
  T* E1 = sm + P::off_E1;
  __syncthreads();
  for (int o = threadIdx.x; o < P::ESZ; o += blockDim.x) E0[o] = (o == 0) ? T(1) : T(0);
  int expo = 0;
  bool zero = false, bad = false;
  for (int c = 0; c < Ly; ++c) {
    const int e = col_step<T, D, DA>(tens, Lx, Ly, up, dn, c, false, E0, E1, sm);
    T* t = E0; E0 = E1; E1 = t;
    if (e == EXP_ZERO) { zero = true; break; }
    if (e == EXP_BAD) { bad = true; break; }
    expo += e;
  }
  __syncthreads();
  cta_finish(zero ? 0.0 : (double)E0[0], expo, bad, up, dn, sgn, la, P::bcast(sm, Lx));
}

// ---------------------------------------------------------------------------
// Environment reuse (the role of the reference's cached boundary
// environments, vmc_torch/GPU/models/pureTNS.py:163-2375).  Per walker the
// left environments E_k (columns < k contracted) and right environments F_k
// (columns >= k) live in a global slab with validity masks; Z = <E_k, F_k>
// for every cut k.  A horizontal move on columns (c, c+1) costs two column
// steps from E_c and a dot product with F_{c+2}; a vertical move in column c
// costs one step from E_c and a dot product with F_{c+1}.  A vertical move
// that changes the electron parity of row r (and so of row r+1) flips the
// sign rule of both rows' sites right of column c; by Z2 evenness of the
// row-r segment right of a cut k that equals the diagonal sign
// (-1)^{N_r(>=k) + p(h_{r,k})} on F_k, p(h_{r,k}) the parity of the row-r
// leg of the cut index.  Horizontal moves keep every row count right of
// column c+1, so F_{c+2} stays valid as is.
// ---------------------------------------------------------------------------
template <int D>
struct Log2 { static constexpr int v = D == 4 ? 2 : 1; };

// parity of the row-r leg inside the cut index o = ((a D + l2) D + l3) DA + a'
template <int D, int DA>
__device__ __forceinline__ int cut_leg_parity(int o, int r, int mid) {
  const int ap = o % DA, l3 = (o / DA) % D, l2 = (o / (DA * D)) % D, a = o / (DA * D * D);
  if (r < mid) return (a >> (Log2<D>::v * (mid - 1 - r))) & 1;
  if (r == mid) return l2 & 1;
  if (r == mid + 1) return l3 & 1;
  return (ap >> (Log2<D>::v * (r - mid - 2))) & 1;
}

__device__ __forceinline__ int row_count_from(uint64_t up, uint64_t dn, int r, int Ly, int k) {
  const uint64_t m = (bits_below(Ly) & ~bits_below(k)) << (r * Ly);  // sites (r, k..Ly-1)
  return __popcll(up & m) + __popcll(dn & m);
}

template <typename T, int D, int DA>
struct EnvCache {
  using P = Peps<T, D, DA>;
  T* slab;        // [2 (Ly+1)][ESZ]: E_0..E_Ly, F_0..F_Ly
  int* pE;        // shared: exponents (E_k = E^_k 2^pE[k])
  int* pF;
  uint32_t vE, vF;
  int Ly;
  bool bad;
  unsigned long long ncols;  // column steps executed (uniform across the CTA)
  __device__ T* Eg(int k) const { return slab + (size_t)k * P::ESZ; }
  __device__ T* Fg(int k) const { return slab + (size_t)(Ly + 1 + k) * P::ESZ; }
};

template <typename T>
__device__ __forceinline__ void cta_copy(T* dst, const T* src, int n) {
  for (int o = threadIdx.x; o < n; o += blockDim.x) dst[o] = src[o];
}

template <typename T, int D, int DA>
__device__ void env_init(EnvCache<T, D, DA>& C) {
  using P = Peps<T, D, DA>;
  __syncthreads();
  for (int o = threadIdx.x; o < P::ESZ; o += blockDim.x) {
    C.Eg(0)[o] = (o == 0) ? T(1) : T(0);
    C.Fg(C.Ly)[o] = (o == 0) ? T(1) : T(0);
  }
  if (threadIdx.x == 0) { C.pE[0] = 0; C.pF[C.Ly] = 0; }
  C.vE = 1u;
  C.vF = 1u << C.Ly;
  C.bad = false;
  C.ncols = 0;
  __syncthreads();
}

// make E_c valid (S0, S1: shared scratch environments)
template <typename T, int D, int DA>
__device__ void env_ensure_E(EnvCache<T, D, DA>& C, const T* tens, int Lx, uint64_t up, uint64_t dn, int c, T* S0,
                             T* S1, T* sm) {
  using P = Peps<T, D, DA>;
  if ((C.vE >> c) & 1u) return;
  int k = c;
  while (!((C.vE >> k) & 1u)) --k;  // E_0 is always valid
  __syncthreads();
  cta_copy(S0, C.Eg(k), P::ESZ);
  int pc = C.pE[k];
  for (int j = k; j < c; ++j) {
    int e = col_step<T, D, DA>(tens, Lx, C.Ly, up, dn, j, false, S0, S1, sm);
    ++C.ncols;
    if (e == EXP_BAD) { C.bad = true; e = 0; }
    if (e == EXP_ZERO) e = 0;
    pc += e;
    __syncthreads();
    cta_copy(C.Eg(j + 1), S1, P::ESZ);
    if (threadIdx.x == 0) C.pE[j + 1] = pc;
    C.vE |= 1u << (j + 1);
    T* t = S0; S0 = S1; S1 = t;
  }
  __syncthreads();
}

template <typename T, int D, int DA>
__device__ void env_ensure_F(EnvCache<T, D, DA>& C, const T* tens, int Lx, uint64_t up, uint64_t dn, int c, T* S0,
                             T* S1, T* sm) {
  using P = Peps<T, D, DA>;
  if ((C.vF >> c) & 1u) return;
  int k = c;
  while (!((C.vF >> k) & 1u)) ++k;  // F_Ly is always valid
  __syncthreads();
  cta_copy(S0, C.Fg(k), P::ESZ);
  int pc = C.pF[k];
  for (int j = k - 1; j >= c; --j) {
    int e = col_step<T, D, DA>(tens, Lx, C.Ly, up, dn, j, true, S0, S1, sm);
    ++C.ncols;
    if (e == EXP_BAD) { C.bad = true; e = 0; }
    if (e == EXP_ZERO) e = 0;
    pc += e;
    __syncthreads();
    cta_copy(C.Fg(j), S1, P::ESZ);
    if (threadIdx.x == 0) C.pF[j] = pc;
    C.vF |= 1u << j;
    T* t = S0; S0 = S1; S1 = t;
  }
  __syncthreads();
}

// sum_o S[o] F[o] (-1)^{nparity + p(row-r leg of o)} (no sign when flip_row < 0),
// CTA-wide; every thread gets the sum.
template <typename T, int D, int DA>
__device__ double env_dot(const T* S, const T* F, int flip_row, int nparity, int mid, T* red, double* bc) {
  using P = Peps<T, D, DA>;
  __syncthreads();
  T acc = 0;
  for (int o = threadIdx.x; o < P::ESZ; o += blockDim.x) {
    T v = S[o] * F[o];
    if (flip_row >= 0 && ((cut_leg_parity<D, DA>(o, flip_row, mid) ^ nparity) & 1)) v = -v;
    acc += v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(VMC_FULL_MASK, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += (double)red[k];
    bc[3] = t;
  }
  __syncthreads();
  return bc[3];
}

// Electron-count parity change of row r when site (r, c) goes from state xs to ns.
__device__ __forceinline__ int row_parity_change(int xs, int ns) { return (__popc(xs) + __popc(ns)) & 1; }

// Proposal on the horizontal pair (r, c)-(r, c+1): x' = (up1, dn1).  Leaves
// S1 = E'_{c+1} (exponent e1 over E_c) and S0 = E'_{c+2} (e2 over E'_{c+1}).
template <typename T, int D, int DA>
__device__ void env_prop_h(EnvCache<T, D, DA>& C, const T* tens, int Lx, uint64_t up, uint64_t dn, uint64_t up1,
                           uint64_t dn1, int c, T* S0, T* S1, T* sm, int& e1, int& e2, double& sgn, double& la) {
  env_ensure_F(C, tens, Lx, up, dn, c + 2, S0, S1, sm);
  env_ensure_E(C, tens, Lx, up, dn, c, S0, S1, sm);
  cta_copy(S0, C.Eg(c), Peps<T, D, DA>::ESZ);
  e1 = col_step<T, D, DA>(tens, Lx, C.Ly, up1, dn1, c, false, S0, S1, sm);
  e2 = (e1 == EXP_ZERO || e1 == EXP_BAD) ? e1 : col_step<T, D, DA>(tens, Lx, C.Ly, up1, dn1, c + 1, false, S1, S0, sm);
  C.ncols += (e1 == EXP_ZERO || e1 == EXP_BAD) ? 1 : 2;
  double* bc = Peps<T, D, DA>::bcast(sm, Lx);
  if (e1 == EXP_BAD || e2 == EXP_BAD || C.bad) { cta_finish(0.0, 0, true, up1, dn1, sgn, la, bc); return; }
  if (e1 == EXP_ZERO || e2 == EXP_ZERO) { cta_finish(0.0, 0, false, up1, dn1, sgn, la, bc); return; }
  const double z = env_dot<T, D, DA>(S0, C.Fg(c + 2), -1, 0, Lx / 2 - 1, sm + Peps<T, D, DA>::off_red, bc);
  cta_finish(z, C.pE[c] + e1 + e2 + C.pF[c + 2], false, up1, dn1, sgn, la, bc);
}

// Proposal on the vertical pair (r, c)-(r+1, c).  flip: the move changes row
// r's electron parity.  Leaves S1 = E'_{c+1} (exponent e1 over E_c).
template <typename T, int D, int DA>
__device__ void env_prop_v(EnvCache<T, D, DA>& C, const T* tens, int Lx, uint64_t up, uint64_t dn, uint64_t up1,
                           uint64_t dn1, int r, int c, bool flip, T* S0, T* S1, T* sm, int& e1, double& sgn,
                           double& la) {
  env_ensure_F(C, tens, Lx, up, dn, c + 1, S0, S1, sm);
  env_ensure_E(C, tens, Lx, up, dn, c, S0, S1, sm);
  cta_copy(S0, C.Eg(c), Peps<T, D, DA>::ESZ);
  e1 = col_step<T, D, DA>(tens, Lx, C.Ly, up1, dn1, c, false, S0, S1, sm);
  ++C.ncols;
  double* bc = Peps<T, D, DA>::bcast(sm, Lx);
  if (e1 == EXP_BAD || C.bad) { cta_finish(0.0, 0, true, up1, dn1, sgn, la, bc); return; }
  if (e1 == EXP_ZERO) { cta_finish(0.0, 0, false, up1, dn1, sgn, la, bc); return; }
  const int np = flip ? (row_count_from(up, dn, r, C.Ly, c + 1) & 1) : 0;
  const double z =
      env_dot<T, D, DA>(S1, C.Fg(c + 1), flip ? r : -1, np, Lx / 2 - 1, sm + Peps<T, D, DA>::off_red, bc);
  cta_finish(z, C.pE[c] + e1 + C.pF[c + 1], false, up1, dn1, sgn, la, bc);
}

template <typename T, int D, int DA>
__device__ void env_accept_h(EnvCache<T, D, DA>& C, int c, const T* S0, const T* S1, int e1, int e2) {
  using P = Peps<T, D, DA>;
  __syncthreads();
  cta_copy(C.Eg(c + 1), S1, P::ESZ);
  cta_copy(C.Eg(c + 2), S0, P::ESZ);
  if (threadIdx.x == 0) {
    C.pE[c + 1] = C.pE[c] + e1;
    C.pE[c + 2] = C.pE[c] + e1 + e2;
  }
  C.vE = (C.vE & ((2u << c) - 1u)) | (1u << (c + 1)) | (1u << (c + 2));
  C.vF &= ~((4u << c) - 1u);  // F_k, k <= c+1, contain the changed columns
  __syncthreads();
}

// up1/dn1: the accepted configuration (row counts right of column c equal
// the old ones).
template <typename T, int D, int DA>
__device__ void env_accept_v(EnvCache<T, D, DA>& C, int Lx, int r, int c, bool flip, uint64_t up1, uint64_t dn1,
                             const T* S1, int e1) {
  using P = Peps<T, D, DA>;
  __syncthreads();
  cta_copy(C.Eg(c + 1), S1, P::ESZ);
  if (threadIdx.x == 0) C.pE[c + 1] = C.pE[c] + e1;
  C.vE = (C.vE & ((2u << c) - 1u)) | (1u << (c + 1));
  C.vF &= ~((2u << c) - 1u);  // F_k, k <= c, contain column c
  if (flip) {
    const int mid = Lx / 2 - 1;
    for (int k = c + 1; k < C.Ly; ++k) {
      if (!((C.vF >> k) & 1u)) continue;
      const int np = row_count_from(up1, dn1, r, C.Ly, k) & 1;
      T* F = C.Fg(k);
      for (int o = threadIdx.x; o < P::ESZ; o += blockDim.x)
        if ((cut_leg_parity<D, DA>(o, r, mid) ^ np) & 1) F[o] = -F[o];
    }
  }
  __syncthreads();
}

// ---- kernels ----
template <typename T, int D, int DA>
__global__ void __launch_bounds__(Peps<T, D, DA>::NT)
    k_peps_eval(const T* __restrict__ tens, int Lx, int Ly, const uint64_t* __restrict__ occ, int64_t R,
                double* __restrict__ sign, double* __restrict__ logabs) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int64_t w = blockIdx.x;
  if (w >= R) return;
  double s, la;
  peps_amp<T, D, DA>(tens, Lx, Ly, occ[2 * w], occ[2 * w + 1], sm, s, la);
  if (threadIdx.x == 0) { sign[w] = s; logabs[w] = la; }
}

template <typename T, int D, int DA>
__global__ void __launch_bounds__(Peps<T, D, DA>::NT)
    k_peps_sweep(const T* __restrict__ tens, int Lx, int Ly, uint64_t* __restrict__ occ, int64_t B,
                 const int32_t* __restrict__ edges, int E, int n_sweeps, float hopping_rate, uint64_t seed,
                 uint64_t sweep_offset, const float* __restrict__ r_move, const uint8_t* __restrict__ r_bit,
                 const float* __restrict__ r_acc, double* __restrict__ sign, double* __restrict__ logabs,
                 int32_t* __restrict__ n_acc, unsigned long long* __restrict__ n_eval) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int64_t w = blockIdx.x;
  if (w >= B) return;
  uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  double sg = sign[w], la = logabs[w];
  int acc = 0;
  unsigned long long ne = 0;
  for (int s = 0; s < n_sweeps; ++s) {
    for (int e = 0; e < E; ++e) {
      const int i = edges[2 * e], j = edges[2 * e + 1];
      const int xi = site_state(up, dn, i), xj = site_state(up, dn, j);
      if (xi == xj) continue;
      float u_move, u_acc;
      int bit;
      if (r_move) {
        const size_t ridx = ((size_t)s * E + e) * (size_t)B + (size_t)w;
        u_move = r_move[ridx]; bit = r_bit[ridx] & 1; u_acc = r_acc[ridx];
      } else {
        EdgeDraw d = draw_edge(seed, (uint64_t)w, sweep_offset + (uint64_t)s, (uint32_t)e);
        u_move = d.u_move; bit = d.bit; u_acc = d.u_acc;
      }
      int ni, nj;
      propose_pair(xi, xj, u_move, bit, hopping_rate, ni, nj);
      const uint64_t mi = 1ull << i, mj = 1ull << j;
      uint64_t up1 = up & ~(mi | mj), dn1 = dn & ~(mi | mj);
      if (ni & 2) up1 |= mi;
      if (ni & 1) dn1 |= mi;
      if (nj & 2) up1 |= mj;
      if (nj & 1) dn1 |= mj;
      double s1, la1;
      peps_amp<T, D, DA>(tens, Lx, Ly, up1, dn1, sm, s1, la1);
      ++ne;
      const bool accept = cta_accept(u_acc, la1, la, Peps<T, D, DA>::bcast(sm, Lx));
      if (accept) { up = up1; dn = dn1; sg = s1; la = la1; ++acc; }
    }
  }
  if (threadIdx.x == 0) {
    occ[2 * w] = up; occ[2 * w + 1] = dn;
    sign[w] = sg; logabs[w] = la;
    if (n_acc) n_acc[w] += acc;
    if (n_eval && ne) {
      atomicAdd(n_eval, ne);
      atomicAdd(n_eval + 1, ne * (unsigned long long)Ly);
    }
  }
}

// One CTA per (walker, hop term) pair: term = H_{x,x'} psi(x') / psi(x).
template <typename T, int D, int DA>
__global__ void __launch_bounds__(Peps<T, D, DA>::NT)
    k_peps_conn_terms(const T* __restrict__ tens, int Lx, int Ly, const uint64_t* __restrict__ occ,
                      const int32_t* __restrict__ pairs, int64_t P, const int32_t* __restrict__ edges, double t,
                      const double* __restrict__ sign, const double* __restrict__ logabs,
                      double* __restrict__ term) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int64_t p = blockIdx.x;
  if (p >= P) return;
  const int N = Lx * Ly;
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
  const double coeff = symmray_parity(up, dn, i, j, sp) ? t : -t;
  double s1, la1;
  peps_amp<T, D, DA>(tens, Lx, Ly, eu, ed, sm, s1, la1);
  if (threadIdx.x == 0) {
    const double s0 = sign[w], la0 = logabs[w];
    term[p] = (s1 == 0.0) ? 0.0 : coeff * s1 * s0 * exp(la1 - la0);
  }
}

// Sweeps with environment reuse: one CTA per walker, environments in the
// walker's slab (chunk-local slot).  Same proposals, random stream and
// acceptance as k_peps_sweep; edges must be nearest-neighbour pairs (else
// *d_err = VMC_ERR_UNSUPPORTED and the edge is skipped).
template <typename T, int D, int DA>
__global__ void __launch_bounds__(Peps<T, D, DA>::NT)
    k_peps_sweep_env(const T* __restrict__ tens, int Lx, int Ly, uint64_t* __restrict__ occ, int64_t B, int64_t w0,
                     const int32_t* __restrict__ edges, int E, int n_sweeps, float hopping_rate, uint64_t seed,
                     uint64_t sweep_offset, const float* __restrict__ r_move, const uint8_t* __restrict__ r_bit,
                     const float* __restrict__ r_acc, double* __restrict__ sign, double* __restrict__ logabs,
                     int32_t* __restrict__ n_acc, unsigned long long* __restrict__ n_eval, T* __restrict__ env,
                     int* __restrict__ d_err) {
  using P = Peps<T, D, DA>;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int64_t w = w0 + blockIdx.x;
  if (w >= B) return;
  EnvCache<T, D, DA> C;
  C.slab = env + (size_t)blockIdx.x * (size_t)(2 * (Ly + 1)) * P::ESZ;
  C.pE = P::exps(sm, Lx);
  C.pF = C.pE + 17;
  C.Ly = Ly;
  T* S0 = sm + P::off_E0;
  T* S1 = sm + P::off_E1;
  env_init(C);
  uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  double sg = sign[w], la = logabs[w];
  int acc = 0;
  unsigned long long ne = 0;
  for (int s = 0; s < n_sweeps; ++s) {
    for (int e = 0; e < E; ++e) {
      const int i = edges[2 * e], j = edges[2 * e + 1];
      const int xi = site_state(up, dn, i), xj = site_state(up, dn, j);
      if (xi == xj) continue;
      const int lo = i < j ? i : j, hi = i < j ? j : i;
      const int ri = lo / Ly, ci = lo % Ly, rj = hi / Ly, cj = hi % Ly;
      const bool horiz = (ri == rj && cj == ci + 1), vert = (ci == cj && rj == ri + 1);
      if (!horiz && !vert) {
        if (d_err && threadIdx.x == 0) atomicExch(d_err, (int)VMC_ERR_UNSUPPORTED);
        continue;
      }
      float u_move, u_acc;
      int bit;
      if (r_move) {
        const size_t ridx = ((size_t)s * E + e) * (size_t)B + (size_t)w;
        u_move = r_move[ridx]; bit = r_bit[ridx] & 1; u_acc = r_acc[ridx];
      } else {
        EdgeDraw d = draw_edge(seed, (uint64_t)w, sweep_offset + (uint64_t)s, (uint32_t)e);
        u_move = d.u_move; bit = d.bit; u_acc = d.u_acc;
      }
      int ni, nj;
      propose_pair(xi, xj, u_move, bit, hopping_rate, ni, nj);
      const uint64_t mi = 1ull << i, mj = 1ull << j;
      uint64_t up1 = up & ~(mi | mj), dn1 = dn & ~(mi | mj);
      if (ni & 2) up1 |= mi;
      if (ni & 1) dn1 |= mi;
      if (nj & 2) up1 |= mj;
      if (nj & 1) dn1 |= mj;
      double s1, la1;
      int e1 = 0, e2 = 0;
      const int xlo = (lo == i) ? xi : xj, nlo = (lo == i) ? ni : nj;
      const bool flip = vert && row_parity_change(xlo, nlo);
      if (horiz) env_prop_h(C, tens, Lx, up, dn, up1, dn1, ci, S0, S1, sm, e1, e2, s1, la1);
      else env_prop_v(C, tens, Lx, up, dn, up1, dn1, ri, ci, flip, S0, S1, sm, e1, s1, la1);
      ++ne;
      const bool accept = cta_accept(u_acc, la1, la, P::bcast(sm, Lx));
      if (accept) {
        if (horiz) env_accept_h(C, ci, S0, S1, e1, e2);
        else env_accept_v(C, Lx, ri, ci, flip, up1, dn1, S1, e1);
        up = up1; dn = dn1; sg = s1; la = la1; ++acc;
      }
    }
  }
  if (threadIdx.x == 0) {
    occ[2 * w] = up; occ[2 * w + 1] = dn;
    sign[w] = sg; logabs[w] = la;
    if (n_acc) n_acc[w] += acc;
    if (n_eval) {
      if (ne) atomicAdd(n_eval, ne);
      atomicAdd(n_eval + 1, C.ncols);
    }
  }
}

// Local energy with environment reuse: one CTA per walker; all E_k and F_k of
// x, then every hop term of the walker from them.  psi(x) is taken from the
// same environments (Z = E_Ly[0]).
template <typename T, int D, int DA>
__global__ void __launch_bounds__(Peps<T, D, DA>::NT)
    k_peps_eloc_env(const T* __restrict__ tens, int Lx, int Ly, const uint64_t* __restrict__ occ, int64_t B,
                    int64_t w0, const int32_t* __restrict__ pairs, const int32_t* __restrict__ offs,
                    const int32_t* __restrict__ edges, double t, double U, double* __restrict__ term,
                    double* __restrict__ eloc, T* __restrict__ env, int* __restrict__ d_err) {
  using P = Peps<T, D, DA>;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int64_t w = w0 + blockIdx.x;
  if (w >= B) return;
  const int N = Lx * Ly;
  EnvCache<T, D, DA> C;
  C.slab = env + (size_t)blockIdx.x * (size_t)(2 * (Ly + 1)) * P::ESZ;
  C.pE = P::exps(sm, Lx);
  C.pF = C.pE + 17;
  C.Ly = Ly;
  T* S0 = sm + P::off_E0;
  T* S1 = sm + P::off_E1;
  env_init(C);
  const uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  env_ensure_E(C, tens, Lx, up, dn, Ly, S0, S1, sm);
  double s0, la0;
  {
    __syncthreads();
    const double z = (double)C.Eg(Ly)[0];
    cta_finish(z, C.pE[Ly], C.bad, up, dn, s0, la0, P::bcast(sm, Lx));
  }
  double tot = U * (double)__popcll(up & dn);
  for (int q = offs[w]; q < offs[w + 1]; ++q) {
    const int tm = pairs[2 * q + 1];
    const int e = tm >> 1, sp = (tm & 1) ? 0 : 1;
    int i = edges[2 * e], j = edges[2 * e + 1];
    if (i > j) { const int tt = i; i = j; j = tt; }
    const int ri = i / Ly, ci = i % Ly, rj = j / Ly, cj = j % Ly;
    const bool horiz = (ri == rj && cj == ci + 1), vert = (ci == cj && rj == ri + 1);
    double v = 0.0;
    if (!horiz && !vert) {
      if (d_err && threadIdx.x == 0) atomicExch(d_err, (int)VMC_ERR_UNSUPPORTED);
    } else {
      const uint64_t m = sp ? up : dn;
      const int oi = (int)((m >> i) & 1ull);
      const int base = sp ? 0 : N;
      uint64_t eu = up, ed = dn;
      apply_move(eu, ed, N, base + (oi ? i : j), base + (oi ? j : i));
      const double coeff = symmray_parity(up, dn, i, j, sp) ? t : -t;
      double s1, la1;
      int e1 = 0, e2 = 0;
      if (horiz) env_prop_h(C, tens, Lx, up, dn, eu, ed, ci, S0, S1, sm, e1, e2, s1, la1);
      else env_prop_v(C, tens, Lx, up, dn, eu, ed, ri, ci, true, S0, S1, sm, e1, s1, la1);  // a hop moves one electron
      if (threadIdx.x == 0 && s1 != 0.0 && s0 != 0.0) v = coeff * s1 * s0 * exp(la1 - la0);
    }
    if (threadIdx.x == 0 && term) term[q] = v;
    tot += v;
  }
  if (threadIdx.x == 0) eloc[w] = tot;
}

__global__ void k_peps_eloc_reduce(int64_t B, const uint64_t* __restrict__ occ, const int32_t* __restrict__ offs,
                                   const double* __restrict__ term, double U, double* __restrict__ eloc) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  double s = U * (double)__popcll(occ[2 * w] & occ[2 * w + 1]);
  for (int q = offs[w]; q < offs[w + 1]; ++q) s += term[q];
  eloc[w] = s;
}

// ---------------------------------------------------------------------------
// Log-derivatives O = d log|psi| / d T[r][c][x_rc][l][u][r'][d] (the reference
// takes torch.func.grad of log_amplitude, vmc_torch/GPU/vmc_utils.py:1389-1634):
// a forward column sweep that stores every left environment E_c (in the
// caller's workspace), then a reverse sweep with the right environment
// F_c = dZ/dE_c.  Per column the slices b are processed one after another by
// the whole CTA: the forward intermediates Y, X2, X3 are recomputed and the
// adjoint chain
//   GX3 = F . N,  GX2 = A3^T GX3,  GY = A2^T GX2,  F_c += M^T GY
// yields dZ/dA2 = Y . GX2, dZ/dA3 = X2 . GX3, dZ/dN = X3 . F, dZ/dM = E . GY,
// which the boundary rows then receive through the MPS construction.
// Environments are kept normalised by powers of two with integer exponents
// (E_c = E^_c 2^p_c, F_c = F^_c 2^q_c, Z = Z^ 2^P), so
// O = sign-rule * dZ^/dA * 2^(p_c + q_{c+1} - P) / Z^.  Gradients are
// implemented for Lx in {4, 6}.
// ---------------------------------------------------------------------------
template <typename T, int D, int DA>
struct PepsGrad {
  using P = Peps<T, D, DA>;
  static constexpr int NT = 512;
  static constexpr int D4 = P::D4, ESZ = P::ESZ, SL = P::SL, MSZ = P::MSZ, D2A = D * D * DA;
  static constexpr size_t o_M = 0, o_N = o_M + MSZ, o_E = o_N + MSZ, o_F = o_E + ESZ, o_Fn = o_F + ESZ,
                          o_Y = o_Fn + ESZ, o_X2 = o_Y + SL, o_X3 = o_X2 + SL, o_G3 = o_X3 + SL, o_G2 = o_G3 + SL,
                          o_GY = o_G2 + SL, o_GA2 = o_GY + SL, o_GA3 = o_GA2 + D4, o_GN = o_GA3 + D4,
                          o_GM = o_GN + MSZ, o_GT = o_GM + MSZ, o_red = o_GT + 4 * D4, o_col = o_red + 32;
  static size_t smem_bytes(int Lx) { return (o_col + (size_t)Lx * D4) * sizeof(T) + 16 * sizeof(int); }
};

// CTA-wide max |v| over n values, power-of-two exponent of it (INT_MIN if 0).
template <typename T>
__device__ int cta_exp_of_max(const T* v, int n, T* red) {
  T m = 0;
  for (int o = threadIdx.x; o < n; o += blockDim.x) m = fmax(m, fabs(v[o]));
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) m = fmax(m, __shfl_xor_sync(VMC_FULL_MASK, m, s));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  T mm = 0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) mm = fmax(mm, red[k]);
  if (mm == T(0)) return INT_MIN;
  if (!(mm < T(INFINITY))) return INT_MAX;
  return exp2_of<T>(mm);
}

// Forward slice b (CTA-wide): Y, X2, X3 of slice b into smem, synchronised.
template <typename T, int D, int DA>
__device__ void grad_fwd_slice(const T* M, const T* E, const T* A2, const T* A3, T* Y, T* X2, T* X3, int b) {
  using G = PepsGrad<T, D, DA>;
  for (int o = threadIdx.x; o < G::SL; o += blockDim.x) {
    const int u2 = o / G::D2A, rest = o % G::D2A;
    T acc = 0;
    for (int a = 0; a < DA; ++a) acc += M[(a * D + u2) * DA + b] * E[a * G::D2A + rest];
    Y[o] = acc;
  }
  __syncthreads();
  for (int o = threadIdx.x; o < G::SL; o += blockDim.x) {
    const int r2 = o / G::D2A, d2 = (o / (D * DA)) % D, l3a = o % (D * DA);
    T acc = 0;
#pragma unroll
    for (int l2 = 0; l2 < D; ++l2)
#pragma unroll
      for (int u2 = 0; u2 < D; ++u2) acc += A2[((l2 * D + u2) * D + r2) * D + d2] * Y[(u2 * D + l2) * (D * DA) + l3a];
    X2[o] = acc;
  }
  __syncthreads();
  for (int o = threadIdx.x; o < G::SL; o += blockDim.x) {
    const int r2 = o / G::D2A, r3 = (o / (D * DA)) % D, d3 = (o / DA) % D, ap = o % DA;
    T acc = 0;
#pragma unroll
    for (int l3 = 0; l3 < D; ++l3)
#pragma unroll
      for (int d2 = 0; d2 < D; ++d2)
        acc += A3[((l3 * D + d2) * D + r3) * D + d3] * X2[((r2 * D + d2) * D + l3) * DA + ap];
    X3[o] = acc;
  }
  __syncthreads();
}

// Sum over 8 consecutive lanes (aligned groups).
template <typename T>
__device__ __forceinline__ T sum8(T v) {
  v += __shfl_xor_sync(VMC_FULL_MASK, v, 1);
  v += __shfl_xor_sync(VMC_FULL_MASK, v, 2);
  v += __shfl_xor_sync(VMC_FULL_MASK, v, 4);
  return v;
}

template <typename T, int D, int DA>
__global__ void __launch_bounds__(512)
    k_peps_grad(const T* __restrict__ tens, int Lx, int Ly, const uint64_t* __restrict__ occ, int64_t R,
                T* __restrict__ O, int64_t ldo, T* __restrict__ env) {
  using G = PepsGrad<T, D, DA>;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  T *M = sm + G::o_M, *Nn = sm + G::o_N, *E = sm + G::o_E, *F = sm + G::o_F, *Fn = sm + G::o_Fn;
  T *Y = sm + G::o_Y, *X2 = sm + G::o_X2, *X3 = sm + G::o_X3, *G3 = sm + G::o_G3, *G2 = sm + G::o_G2;
  T *GY = sm + G::o_GY, *GA2 = sm + G::o_GA2, *GA3 = sm + G::o_GA3, *GN = sm + G::o_GN, *GM = sm + G::o_GM;
  T *GT = sm + G::o_GT, *red = sm + G::o_red, *tcol = sm + G::o_col;
  int* pexp = reinterpret_cast<int*>(tcol + (size_t)Lx * G::D4);
  const int64_t w = blockIdx.x;
  if (w >= R) return;
  const uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  T* envw = env + (size_t)w * (size_t)(Ly + 1) * G::ESZ;
  const int mid = Lx / 2 - 1, nr = mid;
  const T* A2 = tcol + (size_t)mid * G::D4;
  const T* A3 = tcol + (size_t)(mid + 1) * G::D4;
  const int tid = threadIdx.x;

  auto load_col = [&](int c) {
    for (int o = tid; o < Lx * G::D4; o += blockDim.x) {
      const int r = o / G::D4, idx = o % G::D4;
      const int site = r * Ly + c;
      T v = tens[((size_t)site * 4 + site_state(up, dn, site)) * G::D4 + idx];
      if (r > 0) {
        const int l = idx / (D * D * D), u = (idx / (D * D)) % D;
        const uint64_t m = row_mask(r, Ly, c);
        if (u & (l ^ (__popcll(up & m) + __popcll(dn & m))) & 1) v = -v;
      }
      tcol[o] = v;
    }
    __syncthreads();
    build_boundary<T, D, DA>(tcol, Lx, true, M, Y, X2, T(1));
    build_boundary<T, D, DA>(tcol, Lx, false, Nn, Y, X2, T(1));
  };

  // ---------------- forward: store E^_c, exponents p_c ----------------
  for (int o = tid; o < G::ESZ; o += blockDim.x) E[o] = (o == 0) ? T(1) : T(0);
  int pcur = 0;
  bool dead = false;
  for (int c = 0; c < Ly; ++c) {
    __syncthreads();
    load_col(c);
    for (int o = tid; o < G::ESZ; o += blockDim.x) envw[(size_t)c * G::ESZ + o] = E[o];
    if (tid == 0) pexp[c] = pcur;
    for (int b = 0; b < DA; ++b) {
      grad_fwd_slice<T, D, DA>(M, E, A2, A3, Y, X2, X3, b);
      for (int o = tid; o < G::D2A; o += blockDim.x) {
        const int rr = o / DA, bp = o % DA;
        T acc = 0;
        for (int d3 = 0; d3 < D; ++d3)
          for (int ap = 0; ap < DA; ++ap) acc += X3[(rr * D + d3) * DA + ap] * Nn[(ap * D + d3) * DA + bp];
        Fn[b * G::D2A + o] = acc;  // Fn holds E_{c+1} during the forward
      }
    }
    __syncthreads();
    const int e = cta_exp_of_max<T>(Fn, G::ESZ, red);
    if (e == INT_MIN || e == INT_MAX) { dead = true; break; }
    const T s = (T)ldexp(1.0, -e);
    for (int o = tid; o < G::ESZ; o += blockDim.x) E[o] = Fn[o] * s;
    pcur += e;
  }
  if (dead) return;  // psi = 0 or non-finite: the O row stays zero
  __syncthreads();
  const T zhat = E[0];
  if (zhat == T(0)) return;
  const int Pexp = pcur;

  // ---------------- reverse sweep ----------------
  for (int o = tid; o < G::ESZ; o += blockDim.x) F[o] = (o == 0) ? T(1) : T(0);
  int q = 0;  // F^_{c+1} = F_{c+1} 2^-q
  for (int c = Ly - 1; c >= 0; --c) {
    __syncthreads();
    load_col(c);
    for (int o = tid; o < G::ESZ; o += blockDim.x) { E[o] = envw[(size_t)c * G::ESZ + o]; Fn[o] = 0; }
    for (int o = tid; o < G::D4; o += blockDim.x) { GA2[o] = 0; GA3[o] = 0; }
    for (int o = tid; o < G::MSZ; o += blockDim.x) GN[o] = 0;
    __syncthreads();
    for (int b = 0; b < DA; ++b) {
      grad_fwd_slice<T, D, DA>(M, E, A2, A3, Y, X2, X3, b);
      const T* Fb = F + (size_t)b * G::D2A;
      // GX3[r2][r3][d3][a'] = sum_b' F[b][r2 r3][b'] N[a'][d3][b'];  GN += X3 . F
      for (int o = tid; o < G::SL; o += blockDim.x) {
        const int rr = o / (D * DA), d3 = (o / DA) % D, ap = o % DA;
        T acc = 0;
        for (int bp = 0; bp < DA; ++bp) acc += Fb[rr * DA + bp] * Nn[(ap * D + d3) * DA + bp];
        G3[o] = acc;
      }
      for (int o = tid; o < G::MSZ; o += blockDim.x) {
        const int ap = o / (D * DA), d3 = (o / DA) % D, bp = o % DA;
        T acc = 0;
        for (int rr = 0; rr < D * D; ++rr) acc += X3[(rr * D + d3) * DA + ap] * Fb[rr * DA + bp];
        GN[o] += acc;
      }
      __syncthreads();
      // GX2[r2][d2][l3][a'] = sum_{r3,d3} A3[l3][d2][r3][d3] GX3;  GA3 += X2 . GX3
      for (int o = tid; o < G::SL; o += blockDim.x) {
        const int r2 = o / G::D2A, d2 = (o / (D * DA)) % D, l3 = (o / DA) % D, ap = o % DA;
        T acc = 0;
#pragma unroll
        for (int r3 = 0; r3 < D; ++r3)
#pragma unroll
          for (int d3 = 0; d3 < D; ++d3)
            acc += A3[((l3 * D + d2) * D + r3) * D + d3] * G3[((r2 * D + r3) * D + d3) * DA + ap];
        G2[o] = acc;
      }
      for (int t = tid; t < G::D4 * 8; t += blockDim.x) {
        const int o = t >> 3, part = t & 7;
        const int l3 = o / (D * D * D), d2 = (o / (D * D)) % D, r3 = (o / D) % D, d3 = o % D;
        T acc = 0;
        for (int k = part; k < D * DA; k += 8) {
          const int r2 = k / DA, ap = k % DA;
          acc += X2[((r2 * D + d2) * D + l3) * DA + ap] * G3[((r2 * D + r3) * D + d3) * DA + ap];
        }
        acc = sum8(acc);
        if (part == 0) GA3[o] += acc;
      }
      __syncthreads();
      // GY[u2][l2][l3][a'] = sum_{r2,d2} A2[l2][u2][r2][d2] GX2;  GA2 += Y . GX2
      for (int o = tid; o < G::SL; o += blockDim.x) {
        const int u2 = o / G::D2A, l2 = (o / (D * DA)) % D, l3a = o % (D * DA);
        T acc = 0;
#pragma unroll
        for (int r2 = 0; r2 < D; ++r2)
#pragma unroll
          for (int d2 = 0; d2 < D; ++d2)
            acc += A2[((l2 * D + u2) * D + r2) * D + d2] * G2[(r2 * D + d2) * (D * DA) + l3a];
        GY[o] = acc;
      }
      for (int t = tid; t < G::D4 * 8; t += blockDim.x) {
        const int o = t >> 3, part = t & 7;
        const int l2 = o / (D * D * D), u2 = (o / (D * D)) % D, r2 = (o / D) % D, d2 = o % D;
        T acc = 0;
        for (int k = part; k < D * DA; k += 8)  // k = l3 * DA + a'
          acc += Y[(u2 * D + l2) * (D * DA) + k] * G2[(r2 * D + d2) * (D * DA) + k];
        acc = sum8(acc);
        if (part == 0) GA2[o] += acc;
      }
      __syncthreads();
      // GM[a][u2][b] = sum E[a][.] GY[u2][.];  F_c[a][.] += sum_u2 M[a][u2][b] GY[u2][.]
      for (int t = tid; t < DA * D * 8; t += blockDim.x) {
        const int o = t >> 3, part = t & 7;
        const int a = o / D, u2 = o % D;
        T acc = 0;
        for (int k = part; k < G::D2A; k += 8) acc += E[a * G::D2A + k] * GY[u2 * G::D2A + k];
        acc = sum8(acc);
        if (part == 0) GM[(a * D + u2) * DA + b] = acc;
      }
      for (int o = tid; o < G::ESZ; o += blockDim.x) {
        const int a = o / G::D2A, k = o % G::D2A;
        T acc = 0;
#pragma unroll
        for (int u2 = 0; u2 < D; ++u2) acc += M[(a * D + u2) * DA + b] * GY[u2 * G::D2A + k];
        Fn[o] += acc;
      }
      // the next slice first rewrites Y (read above only through GY/E/M): no barrier needed
    }
    __syncthreads();
    // ---- boundary rows: dZ/dA for rows [0, nr) from GM and rows (Lx-1-nr, Lx-1] from GN ----
    const T* At0 = tcol;                                 // row 0
    const T* Ab0 = tcol + (size_t)(Lx - 1) * G::D4;     // row Lx-1
    T* gT0 = GT;                  // row 0
    T* gT1 = GT + G::D4;          // row 1 (nr == 2)
    T* gB0 = GT + 2 * G::D4;      // row Lx-1
    T* gB1 = GT + 3 * G::D4;      // row Lx-2 (nr == 2)
    for (int o = tid; o < G::D4; o += blockDim.x) {
      const int l = o / (D * D * D), u = (o / (D * D)) % D, r = (o / D) % D, d = o % D;
      if (nr == 1) {
        gT0[o] = (u == 0) ? GM[(l * D + d) * DA + r] : T(0);           // M[l][d][r] = A0[l][0][r][d]
        gB0[o] = (d == 0) ? GN[(l * D + u) * DA + r] : T(0);           // N[l][u][r] = A[l][u][r][0]
      } else {
        const T* A1 = tcol + (size_t)1 * G::D4;
        const T* A4 = tcol + (size_t)(Lx - 2) * G::D4;
        // row 0: G_A0[l][0][r][v=d] = sum_{l1,r1,d1} GM[(l l1)][d1][(r r1)] A1[l1][v][r1][d1]
        T g0 = 0, b0 = 0;
        if (u == 0) {
          for (int l1 = 0; l1 < D; ++l1)
            for (int r1 = 0; r1 < D; ++r1)
              for (int d1 = 0; d1 < D; ++d1)
                g0 += GM[((l * D + l1) * D + d1) * DA + (r * D + r1)] * A1[((l1 * D + d) * D + r1) * D + d1];
        }
        // row Lx-1: G_A5[l][v=u][r][0] = sum_{l4,u4,r4} GN[(l l4)][u4][(r r4)] A4[l4][u4][r4][v]
        if (d == 0) {
          for (int l4 = 0; l4 < D; ++l4)
            for (int u4 = 0; u4 < D; ++u4)
              for (int r4 = 0; r4 < D; ++r4)
                b0 += GN[((l * D + l4) * D + u4) * DA + (r * D + r4)] * A4[((l4 * D + u4) * D + r4) * D + u];
        }
        gT0[o] = g0;
        gB0[o] = b0;
        // row 1: G_A1[l1=l][v=u][r1=r][d1=d] = sum_{l0,r0} GM[(l0 l)][d][(r0 r)] A0[l0][0][r0][u]
        T g1 = 0, b1 = 0;
        for (int l0 = 0; l0 < D; ++l0)
          for (int r0 = 0; r0 < D; ++r0) {
            g1 += GM[((l0 * D + l) * D + d) * DA + (r0 * D + r)] * At0[((l0 * D + 0) * D + r0) * D + u];
            // row Lx-2: G_A4[l4=l][u4=u][r4=r][v=d] = sum_{l5,r5} GN[(l5 l)][u][(r5 r)] A5[l5][v][r5][0]
            b1 += GN[((l0 * D + l) * D + u) * DA + (r0 * D + r)] * Ab0[((l0 * D + d) * D + r0) * D + 0];
          }
        gT1[o] = g1;
        gB1[o] = b1;
      }
    }
    __syncthreads();
    // ---- write O for the column's sites ----
    const double scl = ldexp(1.0 / (double)zhat, pexp[c] + q - Pexp);
    T* Ow = O + (size_t)w * (size_t)ldo;
    for (int o = tid; o < Lx * G::D4; o += blockDim.x) {
      const int r = o / G::D4, idx = o % G::D4;
      const T* src;
      if (r == mid) src = GA2;
      else if (r == mid + 1) src = GA3;
      else if (r == 0) src = gT0;
      else if (r == Lx - 1) src = gB0;
      else if (r == 1) src = gT1;
      else src = gB1;
      T v = src[idx];
      const int site = r * Ly + c;
      if (r > 0) {
        const int l = idx / (D * D * D), u = (idx / (D * D)) % D;
        const uint64_t m = row_mask(r, Ly, c);
        if (u & (l ^ (__popcll(up & m) + __popcll(dn & m))) & 1) v = -v;
      }
      Ow[((size_t)site * 4 + site_state(up, dn, site)) * G::D4 + idx] = (T)((double)v * scl);
    }
    // ---- F^_c = Fn normalised ----
    const int e = cta_exp_of_max<T>(Fn, G::ESZ, red);
    if (c > 0) {
      if (e == INT_MIN || e == INT_MAX) return;  // nothing flows further left
      const T s = (T)ldexp(1.0, -e);
      for (int o = tid; o < G::ESZ; o += blockDim.x) F[o] = Fn[o] * s;
      q += e;
    }
  }
}

// ---- dispatch over the supported (D, DA) shapes ----
enum PepsOp { OP_EVAL, OP_SWEEP, OP_TERMS, OP_SWEEP_ENV, OP_ELOC_ENV };

struct PepsArgs {
  const void* tens;
  int Lx, Ly;
  uint64_t* occ;
  int64_t n;
  const int32_t* edges;
  int E, n_sweeps;
  float hopping_rate;
  uint64_t seed, sweep_offset;
  const float* r_move;
  const uint8_t* r_bit;
  const float* r_acc;
  double* sign;
  double* logabs;
  int32_t* n_acc;
  unsigned long long* n_eval;
  const int32_t* pairs;
  double t;
  double* term;
  // environment-reuse launches
  int64_t w0, rows;
  void* env;
  int* d_err;
  const int32_t* offs;
  double U;
  double* eloc;
};

template <typename T, int D, int DA>
int launch_peps(PepsOp op, const PepsArgs& a, cudaStream_t st) {
  using P = Peps<T, D, DA>;
  const size_t smem = P::smem_bytes(a.Lx);
  if (smem > 227 * 1024) return VMC_ERR_UNSUPPORTED;
  const T* tens = (const T*)a.tens;
  if (op == OP_EVAL) {
    cudaFuncSetAttribute(k_peps_eval<T, D, DA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_peps_eval<T, D, DA><<<(unsigned)a.n, P::NT, smem, st>>>(tens, a.Lx, a.Ly, a.occ, a.n, a.sign, a.logabs);
  } else if (op == OP_SWEEP) {
    cudaFuncSetAttribute(k_peps_sweep<T, D, DA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_peps_sweep<T, D, DA><<<(unsigned)a.n, P::NT, smem, st>>>(
        tens, a.Lx, a.Ly, a.occ, a.n, a.edges, a.E, a.n_sweeps, a.hopping_rate, a.seed, a.sweep_offset, a.r_move,
        a.r_bit, a.r_acc, a.sign, a.logabs, a.n_acc, a.n_eval);
  } else if (op == OP_TERMS) {
    cudaFuncSetAttribute(k_peps_conn_terms<T, D, DA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_peps_conn_terms<T, D, DA><<<(unsigned)a.n, P::NT, smem, st>>>(tens, a.Lx, a.Ly, a.occ, a.pairs, a.n,
                                                                     a.edges, a.t, a.sign, a.logabs, a.term);
  } else if (op == OP_SWEEP_ENV) {
    cudaFuncSetAttribute(k_peps_sweep_env<T, D, DA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_peps_sweep_env<T, D, DA><<<(unsigned)a.rows, P::NT, smem, st>>>(
        tens, a.Lx, a.Ly, a.occ, a.n, a.w0, a.edges, a.E, a.n_sweeps, a.hopping_rate, a.seed, a.sweep_offset,
        a.r_move, a.r_bit, a.r_acc, a.sign, a.logabs, a.n_acc, a.n_eval, (T*)a.env, a.d_err);
  } else {
    cudaFuncSetAttribute(k_peps_eloc_env<T, D, DA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_peps_eloc_env<T, D, DA><<<(unsigned)a.rows, P::NT, smem, st>>>(tens, a.Lx, a.Ly, a.occ, a.n, a.w0, a.pairs,
                                                                      a.offs, a.edges, a.t, a.U, a.term, a.eloc,
                                                                      (T*)a.env, a.d_err);
  }
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

template <typename T>
int dispatch_peps(int D, PepsOp op, const PepsArgs& a, cudaStream_t st) {
  const int mid = a.Lx / 2 - 1;
  if (D == 2) {
    if (mid == 1) return launch_peps<T, 2, 2>(op, a, st);
    if (mid == 2) return launch_peps<T, 2, 4>(op, a, st);
    if (mid == 3) return launch_peps<T, 2, 8>(op, a, st);
  } else if (D == 4) {
    if (mid == 1) return launch_peps<T, 4, 4>(op, a, st);
    if (mid == 2) return launch_peps<T, 4, 16>(op, a, st);
  }
  return VMC_ERR_UNSUPPORTED;
}

template <typename T, int D, int DA>
int launch_peps_grad(int Lx, int Ly, const void* tens, const uint64_t* occ, int64_t R, void* O, int64_t ldo,
                     void* env, cudaStream_t st) {
  using G = PepsGrad<T, D, DA>;
  const size_t smem = G::smem_bytes(Lx);
  if (smem > 227 * 1024) return VMC_ERR_UNSUPPORTED;
  cudaFuncSetAttribute(k_peps_grad<T, D, DA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_peps_grad<T, D, DA><<<(unsigned)R, G::NT, smem, st>>>((const T*)tens, Lx, Ly, occ, R, (T*)O, ldo, (T*)env);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

template <typename T>
int dispatch_peps_grad(int D, int Lx, int Ly, const void* tens, const uint64_t* occ, int64_t R, void* O,
                       int64_t ldo, void* env, cudaStream_t st) {
  const int mid = Lx / 2 - 1;
  if (D == 2 && mid == 1) return launch_peps_grad<T, 2, 2>(Lx, Ly, tens, occ, R, O, ldo, env, st);
  if (D == 2 && mid == 2) return launch_peps_grad<T, 2, 4>(Lx, Ly, tens, occ, R, O, ldo, env, st);
  if (D == 4 && mid == 1) return launch_peps_grad<T, 4, 4>(Lx, Ly, tens, occ, R, O, ldo, env, st);
  if (D == 4 && mid == 2) return launch_peps_grad<T, 4, 16>(Lx, Ly, tens, occ, R, O, ldo, env, st);
  return VMC_ERR_UNSUPPORTED;
}

int check_peps(int prec, int Lx, int Ly, int D) {
  if (prec != 0 && prec != 1) return VMC_ERR_ARGS;
  if (Lx < 4 || Lx > 8 || (Lx & 1) || Ly < 1 || Lx * Ly > 64) return VMC_ERR_UNSUPPORTED;
  if (D != 2 && D != 4) return VMC_ERR_UNSUPPORTED;
  if (D == 4 && Lx > 6) return VMC_ERR_UNSUPPORTED;
  return VMC_OK;
}

int run_peps(int prec, int D, PepsOp op, const PepsArgs& a, cudaStream_t st) {
  return prec == 0 ? dispatch_peps<float>(D, op, a, st) : dispatch_peps<double>(D, op, a, st);
}

}  // namespace

extern "C" {

int vmc_peps_eval(int prec, const void* tensors, int Lx, int Ly, int D, const uint64_t* occ, int64_t R, double* sign,
                  double* logabs, void* stream) {
  int rc = check_peps(prec, Lx, Ly, D);
  if (rc) return rc;
  if (R < 0) return VMC_ERR_ARGS;
  if (R == 0) return VMC_OK;
  if (!tensors || !occ || !sign || !logabs) return VMC_ERR_ARGS;
  PepsArgs a{};
  a.tens = tensors; a.Lx = Lx; a.Ly = Ly; a.occ = const_cast<uint64_t*>(occ); a.n = R;
  a.sign = sign; a.logabs = logabs;
  return run_peps(prec, D, OP_EVAL, a, (cudaStream_t)stream);
}

int vmc_peps_sweep(int prec, const void* tensors, int Lx, int Ly, int D, uint64_t* occ, int64_t B,
                   const int32_t* edges, int n_edges, int n_sweeps, float hopping_rate, uint64_t seed,
                   uint64_t sweep_offset, const float* r_move, const uint8_t* r_bit, const float* r_acc, double* sign,
                   double* logabs, int32_t* n_acc, uint64_t* d_n_eval, void* env_work, int64_t work_rows, int* d_err,
                   void* stream) {
  int rc = check_peps(prec, Lx, Ly, D);
  if (rc) return rc;
  if (B < 0 || n_edges < 0 || n_sweeps < 0 || (env_work && work_rows <= 0)) return VMC_ERR_ARGS;
  if ((r_move != nullptr) != (r_acc != nullptr) || (r_move != nullptr) != (r_bit != nullptr)) return VMC_ERR_ARGS;
  if (B == 0 || n_sweeps == 0 || n_edges == 0) return VMC_OK;
  if (!tensors || !occ || !edges || !sign || !logabs) return VMC_ERR_ARGS;
  PepsArgs a{};
  a.tens = tensors; a.Lx = Lx; a.Ly = Ly; a.occ = occ; a.n = B; a.edges = edges; a.E = n_edges;
  a.n_sweeps = n_sweeps; a.hopping_rate = hopping_rate; a.seed = seed; a.sweep_offset = sweep_offset;
  a.r_move = r_move; a.r_bit = r_bit; a.r_acc = r_acc; a.sign = sign; a.logabs = logabs; a.n_acc = n_acc;
  a.n_eval = (unsigned long long*)d_n_eval;
  if (!env_work) return run_peps(prec, D, OP_SWEEP, a, (cudaStream_t)stream);
  a.env = env_work; a.d_err = d_err;
  for (int64_t w0 = 0; w0 < B; w0 += work_rows) {
    a.w0 = w0;
    a.rows = (B - w0) < work_rows ? (B - w0) : work_rows;
    rc = run_peps(prec, D, OP_SWEEP_ENV, a, (cudaStream_t)stream);
    if (rc) return rc;
  }
  return VMC_OK;
}

int vmc_peps_local_energy(int prec, const void* tensors, int Lx, int Ly, int D, const uint64_t* occ, int64_t B,
                          const int32_t* edges, double t, double U, const double* sign, const double* logabs,
                          const int32_t* pairs, const int32_t* offs, int64_t P, double* term, double* eloc,
                          void* env_work, int64_t work_rows, int* d_err, void* stream) {
  int rc = check_peps(prec, Lx, Ly, D);
  if (rc) return rc;
  if (B < 0 || P < 0 || (env_work && work_rows <= 0)) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!tensors || !occ || !offs || !eloc || (P > 0 && (!pairs || !edges))) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  if (env_work) {
    PepsArgs a{};
    a.tens = tensors; a.Lx = Lx; a.Ly = Ly; a.occ = const_cast<uint64_t*>(occ); a.n = B; a.edges = edges;
    a.pairs = pairs; a.offs = offs; a.t = t; a.U = U; a.term = term; a.eloc = eloc; a.env = env_work;
    a.d_err = d_err;
    for (int64_t w0 = 0; w0 < B; w0 += work_rows) {
      a.w0 = w0;
      a.rows = (B - w0) < work_rows ? (B - w0) : work_rows;
      rc = run_peps(prec, D, OP_ELOC_ENV, a, st);
      if (rc) return rc;
    }
    return VMC_OK;
  }
  if (!sign || !logabs || (P > 0 && !term)) return VMC_ERR_ARGS;
  if (P > 0) {
    PepsArgs a{};
    a.tens = tensors; a.Lx = Lx; a.Ly = Ly; a.occ = const_cast<uint64_t*>(occ); a.n = P; a.edges = edges;
    a.pairs = pairs; a.t = t; a.sign = const_cast<double*>(sign); a.logabs = const_cast<double*>(logabs);
    a.term = term;
    rc = run_peps(prec, D, OP_TERMS, a, st);
    if (rc) return rc;
  }
  k_peps_eloc_reduce<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(B, occ, offs, term, U, eloc);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_peps_logpsi_grad(int prec, const void* tensors, int Lx, int Ly, int D, const uint64_t* occ, int64_t B,
                         void* O, int64_t ldo, void* work, int64_t work_rows, void* stream) {
  int rc = check_peps(prec, Lx, Ly, D);
  if (rc) return rc;
  if (Lx > 6) return VMC_ERR_UNSUPPORTED;
  const int64_t np = (int64_t)Lx * Ly * 4 * D * D * D * D;
  if (B < 0 || ldo < np || work_rows <= 0) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!tensors || !occ || !O || !work) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t es = prec == 0 ? sizeof(float) : sizeof(double);
  if (cudaMemset2DAsync(O, (size_t)ldo * es, 0, (size_t)np * es, (size_t)B, st) != cudaSuccess) return VMC_ERR_CUDA;
  for (int64_t w0 = 0; w0 < B; w0 += work_rows) {
    const int64_t R = (B - w0) < work_rows ? (B - w0) : work_rows;
    rc = prec == 0 ? dispatch_peps_grad<float>(D, Lx, Ly, tensors, occ + 2 * w0, R, (float*)O + w0 * ldo, ldo, work, st)
                   : dispatch_peps_grad<double>(D, Lx, Ly, tensors, occ + 2 * w0, R, (double*)O + w0 * ldo, ldo, work,
                                                st);
    if (rc) return rc;
  }
  return VMC_OK;
}

}  // extern "C"
