// Fermionic PEPS amplitudes with the reference's chi-truncated boundary
// contraction (fPEPS_Model_GPU.amplitude / log_amplitude,
// vmc_torch/GPU/models/pureTNS.py:81-146: contract_boundary_from_xmin_ over
// rows [0, Lx/2-1] and contract_boundary_from_xmax_ over [Lx/2, Lx-1], both
// with max_bond = chi and cutoff 0, then the two boundaries contracted).
//
// Formulation.  Each side's boundary is kept as the full vector over its
// D^Ly open vertical legs (index sum_c d_c D^(Ly-1-c), column 0 most
// significant).  A row is absorbed exactly, column by column, with the open
// horizontal leg h as an extra index: W[h][idx], and per column c the 16
// entries of every group (fixed other digits) map through the signed site
// tensor A[h][old][h'][new] in place.  The boundary-MPS compression after a
// row (left-to-right QR, then right-to-left SVD truncation to chi) is, in the
// canonical sweep, the sequence of best rank-chi approximations of the whole
// boundary state across cuts Ly-1, ..., 1; which cuts can exceed chi follows
// from static bounds (a row multiplies a cut's bond by D, the rank never
// exceeds min(D^k, D^(Ly-k)), truncating cut k bounds cut k-1 by D*chi), so
// the host passes a per-row schedule of cuts and the others are skipped
// (their truncation is the identity).  At 6x6, D = 4, chi = 16 each side
// truncates only the middle cut, once.
//
// Truncation at cut k: the state as a matrix M (D^k x D^(Ly-k)) is
// block-diagonal in the Z2 parity of its smaller side's index (each tensor is
// parity-even), two blocks of at most 32 rows, one warp per block.  When a
// block also has at most 32 columns (the middle cut of a 6-wide lattice): a
// pivoted LQ factorisation in the warp, then one-sided Jacobi on the rows of
// L^T (pairs (i, i xor m), m = 1..31: every pair once per sweep, 16 disjoint
// rotations a round), whose normalised final rows are the block's left
// singular vectors.  Otherwise the block's Gram matrix by two-sided Jacobi.
// The chi largest singular values over both blocks select the kept vectors U
// and the state becomes U U^T M, the SVD truncation.  Precision "fp64" runs
// everything in FP64, "fp32" the state and the Jacobi in FP32 with FP64
// accumulation of the final overlap.
//
// Log-derivatives: the cotangent of each side's truncation against the other
// side's truncated state (first-order change of the kept singular subspace),
// then a reverse row sweep over recomputed forward column states.
//
// After every absorbed row the state is rescaled by a power of two (exact)
// and the exponent accumulated, so FP32 does not overflow.
#include <climits>
#include <type_traits>

#include "common.cuh"
#include "vmc_gb300.h"

using namespace vmc;

namespace {

constexpr int CHI_NT = 256;
constexpr int CHI_MAX_NS = 4096;      // D^Ly
constexpr int CHI_MAX_ROWS = 32;      // rows per side
constexpr int CHI_EXP_ZERO = INT_MIN, CHI_EXP_BAD = INT_MAX;

struct ChiSched {
  int Lx, Ly, D, NS, chi, rows;       // rows per side = Lx / 2
  uint32_t cuts[CHI_MAX_ROWS];        // bit k: truncate cut k after this absorbed row
};

template <int D>
__device__ __forceinline__ int digit_parity(uint32_t x) {
  return D == 4 ? (__popc(x & 0x55555555u) & 1) : (__popc(x) & 1);
}

// small-side index of the i-th member of parity block b
template <int D>
__device__ __forceinline__ uint32_t block_member(int b, int i) {
  const uint32_t e = (uint32_t)i << 1;
  return e | (uint32_t)(b ^ digit_parity<D>(e));
}

template <typename T>
struct ChiSmem {
  // absorption: W (D * NS), per column of a row the two parity blocks of A ((D^2/2)^2 each), reduction scratch
  static size_t bytes(int NS, int D, int Ly) {
    return ((size_t)D * NS + (size_t)Ly * D * D * D * D / 2 + 32) * sizeof(T) + 16;
  }
};

// One warp: eigen-decomposition of the symmetric 32 x 32 matrix in S (row
// stride 33, zero-padded beyond nb) by cyclic Jacobi.  On return lam[i] holds
// the eigenvalue of lane i and V[i * 33 + j] component j of its eigenvector.
template <typename T>
__device__ void warp_jacobi(T* S, T* V, T* lam) {
  const int ln = threadIdx.x & 31;
  T g[32], v[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    g[j] = S[ln * 33 + j];
    v[j] = (j == ln) ? T(1) : T(0);
  }
  const T tol = std::is_same<T, float>::value ? T(2e-7) : T(4e-16);
  // rotations below tol * max|diag| are rounding noise of the largest entries
  T floor_ = fabs(S[ln * 33 + ln]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) floor_ = fmax(floor_, __shfl_xor_sync(VMC_FULL_MASK, floor_, o));
  floor_ *= tol;
  for (int sw = 0; sw < 20; ++sw) {
    bool rotated = false;
    for (int m = 1; m < 32; ++m) {
      const int pr = ln ^ m;
      const bool lead = ln < pr;
      T c = T(1), s = T(0);
      int need = 0;
      if (lead) {
        const T app = S[ln * 33 + ln], aqq = S[pr * 33 + pr], apq = S[ln * 33 + pr];
        if (fabs(apq) > floor_ && fabs(apq) > tol * sqrt(fabs(app * aqq))) {
          // Golub & Van Loan, sym.schur2: J = [[c, s], [-s, c]] zeroes (p, q) of J^T A J
          const T tau = (aqq - app) / (T(2) * apq);
          const T t = (tau >= T(0) ? T(1) : T(-1)) / (fabs(tau) + hypot(T(1), tau));
          c = T(1) / sqrt(T(1) + t * t);
          s = t * c;
          need = 1;
        }
      }
      const T c2 = __shfl_xor_sync(VMC_FULL_MASK, c, m), s2 = __shfl_xor_sync(VMC_FULL_MASK, s, m);
      const int n2 = __shfl_xor_sync(VMC_FULL_MASK, need, m);
      if (!lead) { c = c2; s = s2; need = n2; }
      if (!__any_sync(VMC_FULL_MASK, need)) continue;
      rotated = true;
      const T sp = lead ? -s : s;  // row p' = c p - s q, row q' = s p + c q
      // rows: H = J^T G
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const T o = __shfl_xor_sync(VMC_FULL_MASK, g[j], m);
        g[j] = fma(sp, o, c * g[j]);
      }
      __syncwarp();
#pragma unroll
      for (int j = 0; j < 32; ++j) S[ln * 33 + j] = g[j];
      __syncwarp();
#pragma unroll
      for (int j = 0; j < 32; ++j) g[j] = S[j * 33 + ln];
      __syncwarp();
      // rows of H^T = G J: J^T (G J) = G'
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const T o = __shfl_xor_sync(VMC_FULL_MASK, g[j], m);
        g[j] = fma(sp, o, c * g[j]);
      }
#pragma unroll
      for (int j = 0; j < 32; ++j) S[ln * 33 + j] = g[j];
      __syncwarp();
      // eigenvectors: V <- V J, lane i holds column i
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const T o = __shfl_xor_sync(VMC_FULL_MASK, v[j], m);
        v[j] = fma(sp, o, c * v[j]);
      }
    }
    if (!rotated) break;
  }
  lam[ln] = S[ln * 33 + ln];
#pragma unroll
  for (int j = 0; j < 32; ++j) V[ln * 33 + j] = v[j];
  __syncwarp();
}

// One warp: one-sided (Hestenes) Jacobi on the rows u_i (lane i, up to 32
// columns) of a block of the state.  Pairs (i, i xor m) are rotated until
// their rows are orthogonal; the accumulated rotation Q (lane i holds row i)
// satisfies Q A = U with orthogonal rows, so the rows of Q are the
// eigenvectors of A A^T with eigenvalues |u_i|^2.  Works on A itself, so the
// condition number is not squared as in the Gram matrix.  Output as
// warp_jacobi: lam[i], V[i * 33 + j] = Q[i][j].
template <typename T>
__device__ void warp_hestenes(T (&u)[32], T* V, T* lam) {
  const int ln = threadIdx.x & 31;
  T qv[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) qv[j] = (j == ln) ? T(1) : T(0);
  const T tol = std::is_same<T, float>::value ? T(2e-7) : T(4e-16);
  T nrm = T(0);
#pragma unroll
  for (int j = 0; j < 32; ++j) nrm = fma(u[j], u[j], nrm);
  T floor_ = nrm;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) floor_ = fmax(floor_, __shfl_xor_sync(VMC_FULL_MASK, floor_, o));
  floor_ *= tol;
  for (int sw = 0; sw < 20; ++sw) {
    bool rotated = false;
    for (int m = 1; m < 32; ++m) {
      const bool lead = ln < (ln ^ m);
      T o[32];
      T gam = T(0), alp = T(0);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        o[j] = __shfl_xor_sync(VMC_FULL_MASK, u[j], m);
        gam = fma(u[j], o[j], gam);
        alp = fma(u[j], u[j], alp);
      }
      const T bet = __shfl_xor_sync(VMC_FULL_MASK, alp, m);
      T c = T(1), s = T(0);
      int need = 0;
      if (lead && fabs(gam) > floor_ && fabs(gam) > tol * sqrt(alp * bet)) {
        const T zeta = (bet - alp) / (T(2) * gam);
        const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + hypot(T(1), zeta));
        c = T(1) / sqrt(T(1) + t * t);
        s = t * c;
        need = 1;
      }
      const T c2 = __shfl_xor_sync(VMC_FULL_MASK, c, m), s2 = __shfl_xor_sync(VMC_FULL_MASK, s, m);
      const int n2 = __shfl_xor_sync(VMC_FULL_MASK, need, m);
      if (!lead) { c = c2; s = s2; need = n2; }
      if (!__any_sync(VMC_FULL_MASK, need)) continue;
      rotated = true;
      const T sp = lead ? -s : s;
#pragma unroll
      for (int j = 0; j < 32; ++j) u[j] = fma(sp, o[j], c * u[j]);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const T oq = __shfl_xor_sync(VMC_FULL_MASK, qv[j], m);
        qv[j] = fma(sp, oq, c * qv[j]);
      }
    }
    if (!rotated) break;
  }
  nrm = T(0);
#pragma unroll
  for (int j = 0; j < 32; ++j) nrm = fma(u[j], u[j], nrm);
  lam[ln] = nrm;
#pragma unroll
  for (int j = 0; j < 32; ++j) V[ln * 33 + j] = qv[j];
  __syncwarp();
}

// One warp: the left singular vectors of a block A (lane i holds row i, nq
// <= 32 columns, rows beyond the block zero) by a pivoted LQ factorisation
// A = L Q followed by one-sided Jacobi on the rows of L^T (Drmac & Veselic:
// Jacobi on the triangular factor of a pivoted QR converges in about half the
// sweeps).  LQ: Householder reflectors from the right, the pivot row of step
// k the unprocessed row with the largest trailing norm (rows stay in their
// lanes; the order only decides which row defines reflector k).  Then L^T
// goes through shared memory (lane k holds column k of L), its rows are made
// orthogonal (no rotation matrix is kept: A A^T = L L^T, whose eigenvectors
// are the normalised final rows), and lam[k] = |row k|^2, V[k * 33 + i] =
// row k / |row k| (zero for a zero row).  S: a 32 x 33 scratch.
template <typename T>
__device__ void warp_lq_jacobi(T (&u)[32], int nq, T* S, T* V, T* lam) {
  const int ln = threadIdx.x & 31;
  bool done = false;
  for (int k = 0; k < nq; ++k) {
    T nr = T(0);
#pragma unroll
    for (int j = 0; j < 32; ++j) nr = (j >= k) ? fma(u[j], u[j], nr) : nr;
    // pivot: the unprocessed row with the largest trailing norm (ties: lower lane)
    T key = done ? T(-1) : nr;
    int p = ln;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T ok = __shfl_xor_sync(VMC_FULL_MASK, key, o);
      const int op = __shfl_xor_sync(VMC_FULL_MASK, p, o);
      if (ok > key || (ok == key && op < p)) { key = ok; p = op; }
    }
    const T pn = __shfl_sync(VMC_FULL_MASK, nr, p);
    if (!(pn > T(0))) break;   // the remaining rows vanish: A is rank k
    if (ln == p) done = true;
    // reflector v from the pivot row's trailing part: v = x - alpha e_k, alpha = -sign(x_k) |x|
    T v[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = (j >= k) ? __shfl_sync(VMC_FULL_MASK, u[j], p) : T(0);
    T vk = T(0);
#pragma unroll
    for (int j = 0; j < 32; ++j) vk = (j == k) ? v[j] : vk;
    const T alpha = (vk >= T(0)) ? -sqrt(pn) : sqrt(pn);
    const T vk2 = vk - alpha;
    const T vv = pn - vk * vk + vk2 * vk2;
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = (j == k) ? vk2 : v[j];
    T d = T(0);
#pragma unroll
    for (int j = 0; j < 32; ++j) d = fma(u[j], v[j], d);
    const T f = T(2) * d / vv;
#pragma unroll
    for (int j = 0; j < 32; ++j) u[j] = fma(-f, v[j], u[j]);
  }
  // L^T: lane k takes column k of L
  __syncwarp();
#pragma unroll
  for (int j = 0; j < 32; ++j) S[ln * 33 + j] = u[j];
  __syncwarp();
#pragma unroll
  for (int j = 0; j < 32; ++j) u[j] = S[j * 33 + ln];
  __syncwarp();
  const T tol = std::is_same<T, float>::value ? T(2e-7) : T(4e-16);
  T nrm = T(0);
#pragma unroll
  for (int j = 0; j < 32; ++j) nrm = fma(u[j], u[j], nrm);
  T floor_ = nrm;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) floor_ = fmax(floor_, __shfl_xor_sync(VMC_FULL_MASK, floor_, o));
  floor_ *= tol;
  for (int sw = 0; sw < 20; ++sw) {
    bool rotated = false;
    for (int m = 1; m < 32; ++m) {
      const bool lead = ln < (ln ^ m);
      T o[32];
      T gam = T(0), alp = T(0);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        o[j] = __shfl_xor_sync(VMC_FULL_MASK, u[j], m);
        gam = fma(u[j], o[j], gam);
        alp = fma(u[j], u[j], alp);
      }
      const T bet = __shfl_xor_sync(VMC_FULL_MASK, alp, m);
      T c = T(1), s = T(0);
      int need = 0;
      if (lead && fabs(gam) > floor_ && fabs(gam) > tol * sqrt(alp * bet)) {
        const T zeta = (bet - alp) / (T(2) * gam);
        const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + hypot(T(1), zeta));
        c = T(1) / sqrt(T(1) + t * t);
        s = t * c;
        need = 1;
      }
      const T c2 = __shfl_xor_sync(VMC_FULL_MASK, c, m), s2 = __shfl_xor_sync(VMC_FULL_MASK, s, m);
      const int n2 = __shfl_xor_sync(VMC_FULL_MASK, need, m);
      if (!lead) { c = c2; s = s2; need = n2; }
      if (!__any_sync(VMC_FULL_MASK, need)) continue;
      rotated = true;
      const T sp = lead ? -s : s;
#pragma unroll
      for (int j = 0; j < 32; ++j) u[j] = fma(sp, o[j], c * u[j]);
    }
    if (!rotated) break;
  }
  nrm = T(0);
#pragma unroll
  for (int j = 0; j < 32; ++j) nrm = fma(u[j], u[j], nrm);
  lam[ln] = nrm;
  const T inv = nrm > T(0) ? T(1) / sqrt(nrm) : T(0);
#pragma unroll
  for (int j = 0; j < 32; ++j) V[ln * 33 + j] = u[j] * inv;
  __syncwarp();
}

// Largest |x| of the CTA (thread 0's value is returned to every thread).
template <typename T>
__device__ T cta_absmax(T m, T* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(VMC_FULL_MASK, m, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  T r = red[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, red[w]);
  return r;
}

// Item -> (configuration index ci, side): sides == nullptr: ci = item >> 1,
// side = item & 1; else ci = cfg_idx[item] (or item), side = sides[item].  The
// item's state lives in slot 2 * ci + side.
__device__ __forceinline__ void chi_item(int64_t item, const int32_t* cfg_idx, const uint8_t* sides, int64_t& ci,
                                         int& side) {
  if (sides) { ci = cfg_idx ? cfg_idx[item] : item; side = sides[item]; }
  else { ci = item >> 1; side = (int)(item & 1); }
}

// Electron parity of the first n_rows rows of a side.
__device__ __forceinline__ int side_parity(uint64_t up, uint64_t dn, int Lx, int Ly, int side, int n_rows) {
  const int r0 = side ? Lx - n_rows : 0;
  const uint64_t m = bits_below((r0 + n_rows) * Ly) & ~bits_below(r0 * Ly);
  return (__popcll(up & m) + __popcll(dn & m)) & 1;
}

// Pair ia (< D^2/2) of parity class t: (d, h) with p(d) + p(h) = t.
template <int D>
__device__ __forceinline__ void class_pair(int t, int ia, int& d, int& h) {
  d = ia / (D / 2);
  h = ((t ^ (d & 1)) & 1) + 2 * (ia % (D / 2));
}

// Signed site tensors of row r in parity blocks, all columns:
// A2[c][ti][ia][ib] = A(r, c)[h][old][h'][new] for the input pair ia = (old, h)
// of class ti and the output pair ib = (new, h') of class ti ^ p(x_rc).
template <typename T, int D>
__device__ void load_row_tables(const T* __restrict__ tens, uint64_t up, uint64_t dn, int r, int Ly, int side,
                                T* A2) {
  constexpr int H = D * D / 2;
  for (int e = threadIdx.x; e < Ly * 2 * H * H; e += blockDim.x) {
    const int c = e / (2 * H * H), el = e - c * 2 * H * H;
    const int site = r * Ly + c;
    const int x = site_state(up, dn, site);
    const int px = (x ^ (x >> 1)) & 1;
    const uint64_t lm = bits_below(site) & ~bits_below(r * Ly);
    const int nleft = __popcll(up & lm) + __popcll(dn & lm);
    const int ti = el / (H * H), ia = (el / H) % H, ib = el % H;
    int o, h, n, hp;
    class_pair<D>(ti, ia, o, h);
    class_pair<D>(ti ^ px, ib, n, hp);
    const int u = side ? n : o, d = side ? o : n;
    T val = tens[((size_t)site * 4 + x) * (D * D * D * D) + ((h * D + u) * D + hp) * D + d];
    if (r >= 1 && (u & 1) && ((h + nleft) & 1)) val = -val;
    A2[e] = val;
  }
}

// Tensor index (within the site's D^4 block) and sign-rule sign of entry
// (ti, ia, ib) of a column's table; inverse of load_row_tables.
template <int D>
__device__ __forceinline__ int table_entry(int ti, int ia, int ib, int px, int side, int r, int nleft, int& sgn) {
  int o, h, n, hp;
  class_pair<D>(ti, ia, o, h);
  class_pair<D>(ti ^ px, ib, n, hp);
  const int u = side ? n : o, d = side ? o : n;
  sgn = (r >= 1 && (u & 1) && ((h + nleft) & 1)) ? -1 : 1;
  return ((h * D + u) * D + hp) * D + d;
}

// One column of a row absorption, in place on W[h][idx] (all threads).
// par: electron parity absorbed before this column; px: the site's.  The
// first half of the CTA takes the groups of parity class 0, the second half
// class 1 (class = par + digit parity of the group's other digits), so each
// warp works on one class and keeps that class's (D^2/2)^2 block of the site
// tensor in registers for the whole column.
template <typename T, int D>
__device__ void column_forward(T* W, int NS, int stride, int par, int px, const T* Ac) {
  constexpr int H = D * D / 2;
  const int half = (int)blockDim.x >> 1;
  const int ti = threadIdx.x < half ? 0 : 1, tl = threadIdx.x - ti * half, to = ti ^ px;
  T A[H * H];
#pragma unroll
  for (int k = 0; k < H * H; ++k) A[k] = Ac[ti * H * H + k];
  const int G = NS / D, Gh = (G + 1) >> 1;
  for (int i = tl; i < Gh; i += half) {
    // the i-th group of the class: other-digit index with digit parity ti ^ par
    const uint32_t e = (uint32_t)i << 1;
    const int g = (int)(e | (uint32_t)((ti ^ par ^ digit_parity<D>(e)) & 1));
    if (g >= G) continue;
    const int lo = g % stride, hi = g / stride;
    const int base = hi * stride * D + lo;
    T in[H];
    bool any = false;
#pragma unroll
    for (int ia = 0; ia < H; ++ia) {
      int o, h;
      class_pair<D>(ti, ia, o, h);
      in[ia] = W[h * NS + base + o * stride];
      any |= in[ia] != T(0);
    }
    if (!any) continue;
    T outv[H];
#pragma unroll
    for (int ib = 0; ib < H; ++ib) outv[ib] = T(0);
#pragma unroll
    for (int ia = 0; ia < H; ++ia)
#pragma unroll
      for (int ib = 0; ib < H; ++ib) outv[ib] += in[ia] * A[ia * H + ib];
    if (px) {  // the input class empties
#pragma unroll
      for (int ia = 0; ia < H; ++ia) {
        int o, h;
        class_pair<D>(ti, ia, o, h);
        W[h * NS + base + o * stride] = T(0);
      }
    }
#pragma unroll
    for (int ib = 0; ib < H; ++ib) {
      int n, hp;
      class_pair<D>(to, ib, n, hp);
      W[hp * NS + base + n * stride] = outv[ib];
    }
  }
}

// Transpose of column_forward on a cotangent Wb (in place): the output class
// cotangents map back onto the input class.
template <typename T, int D>
__device__ void column_adjoint(T* Wb, int NS, int stride, int par, int px, const T* Ac) {
  constexpr int H = D * D / 2;
  for (int gi = threadIdx.x; gi < NS / D; gi += blockDim.x) {
    const int lo = gi % stride, hi = gi / stride;
    const int base = hi * stride * D + lo;
    const int ti = (par ^ digit_parity<D>((uint32_t)base)) & 1, to = ti ^ px;
    T g[H];
    bool any = false;
#pragma unroll
    for (int ib = 0; ib < H; ++ib) {
      int n, hp;
      class_pair<D>(to, ib, n, hp);
      g[ib] = Wb[hp * NS + base + n * stride];
      any |= g[ib] != T(0);
    }
    if (!any) continue;
    const T* Ab = Ac + ti * H * H;
    T inb[H];
#pragma unroll
    for (int ia = 0; ia < H; ++ia) {
      T acc = T(0);
#pragma unroll
      for (int ib = 0; ib < H; ++ib) acc += Ab[ia * H + ib] * g[ib];
      inb[ia] = acc;
    }
    if (px) {
#pragma unroll
      for (int ib = 0; ib < H; ++ib) {
        int n, hp;
        class_pair<D>(to, ib, n, hp);
        Wb[hp * NS + base + n * stride] = T(0);
      }
    }
#pragma unroll
    for (int ia = 0; ia < H; ++ia) {
      int o, h;
      class_pair<D>(ti, ia, o, h);
      Wb[h * NS + base + o * stride] = inb[ia];
    }
  }
}

// Absorbs rows [a0, a1) of each item's side into its boundary state (slot
// 2 ci + side of state / expo; a0 == 0 starts from the empty boundary).  One
// CTA per item, W[h][idx] (D x NS) in shared memory.  Z2 structure: while a
// row is absorbed, W[h][idx] vanishes unless p(h) + p(idx) equals the parity
// of the electrons absorbed so far, and A[h][o][h'][n] unless p(h) + p(o) +
// p(h') + p(n) equals the site's; so a group's D^2 inputs hold D^2/2 non-zero
// values, mapped by a (D^2/2)^2 block of A onto the D^2/2 outputs of the
// other class when the site's parity is odd (the emptied slots are zeroed).
// keep / row_e (nullable): the normalised state after every row and the
// row's power-of-two exponent, at [(slot * rows + a)], for the adjoint.
template <typename T, int D>
__global__ void __launch_bounds__(CHI_NT)
    k_chi_absorb(const T* __restrict__ tens, ChiSched sc, const uint64_t* __restrict__ cfg,
                 const int32_t* __restrict__ cfg_idx, const uint8_t* __restrict__ sides, int64_t n_items,
                 const int* __restrict__ count, int a0, int a1, T* __restrict__ state, int* __restrict__ expo_io,
                 T* __restrict__ keep, int* __restrict__ row_e) {
  constexpr int H = D * D / 2;  // non-zero entries of a group
  extern __shared__ __align__(16) unsigned char smraw[];
  const int64_t item = blockIdx.x;
  if (item >= n_items || (count && item >= *count)) return;
  const int NS = sc.NS, Ly = sc.Ly, Lx = sc.Lx;
  T* W = reinterpret_cast<T*>(smraw);
  T* A2 = W + (size_t)D * NS;   // per column of the row: [class of (o, h)][H][H]
  T* red = A2 + (size_t)sc.Ly * 2 * H * H;
  int64_t ci;
  int side;
  chi_item(item, cfg_idx, sides, ci, side);
  const int64_t slot = 2 * ci + side;
  const uint64_t up = cfg[2 * ci], dn = cfg[2 * ci + 1];
  T* st = state + slot * (int64_t)NS;
  int expo = 0;
  bool zero = false, bad = false;
  if (a0 == 0) {
    for (int e = threadIdx.x; e < D * NS; e += blockDim.x) W[e] = (e == 0) ? T(1) : T(0);
  } else {
    expo = expo_io[slot];
    zero = expo == CHI_EXP_ZERO;
    bad = expo == CHI_EXP_BAD;
    for (int e = threadIdx.x; e < D * NS; e += blockDim.x) W[e] = (e < NS && !zero && !bad) ? st[e] : T(0);
  }
  int par = side_parity(up, dn, Lx, Ly, side, a0);
  for (int a = a0; a < a1 && !zero && !bad; ++a) {
    const int r = side ? (Lx - 1 - a) : a;
    // the row's signed tensors, all columns at once (one global-load latency per row)
    __syncthreads();
    load_row_tables<T, D>(tens, up, dn, r, Ly, side, A2);
    int stride = NS / D;
    for (int c = 0; c < Ly; ++c, stride /= D) {
      const int x = site_state(up, dn, r * Ly + c);
      const int px = (x ^ (x >> 1)) & 1;
      __syncthreads();
      column_forward<T, D>(W, NS, stride, par, px, A2 + c * 2 * H * H);
      par ^= px;
    }
    __syncthreads();
    // rescale the state (the h != 0 slices are zero after the open right edge)
    T m = T(0);
    int nonfinite = 0;
    for (int e = threadIdx.x; e < NS; e += blockDim.x) {
      const T v = fabs(W[e]);
      nonfinite |= !(v < T(INFINITY));
      m = fmax(m, v);
    }
    if (__syncthreads_or(nonfinite)) { bad = true; break; }
    m = cta_absmax<T>(m, red);
    if (m == T(0)) { zero = true; break; }
    const int e2 = (int)ilogb(m);
    expo += e2;
    __syncthreads();
    for (int e = threadIdx.x; e < NS; e += blockDim.x) W[e] = scalbn(W[e], -e2);
    if (keep) {
      __syncthreads();
      T* kp = keep + (slot * sc.rows + a) * (int64_t)NS;
      for (int e = threadIdx.x; e < NS; e += blockDim.x) kp[e] = W[e];
      if (threadIdx.x == 0) row_e[slot * sc.rows + a] = e2;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < NS; e += blockDim.x) st[e] = (zero || bad) ? T(0) : W[e];
  if (threadIdx.x == 0) expo_io[slot] = bad ? CHI_EXP_BAD : (zero ? CHI_EXP_ZERO : expo);
}

constexpr int CHI_TRUNC_ITEMS = 2;  // items per CTA, two warps (one per parity block) each

template <typename T>
struct ChiTruncSmem {
  static size_t bytes() { return (size_t)CHI_TRUNC_ITEMS * ((4 * 32 * 33 + 64) * sizeof(T) + 64 * sizeof(int)); }
};

// Best rank-chi truncation across cut k of each item's state (after the
// side's first n_rows rows): warp b of an item forms the parity block b of the
// Gram matrix on the cut's smaller side (only the big-side indices of the
// matching parity contribute), diagonalises it (warp_jacobi), and after the
// item's two warps have ranked their eigenvalues together projects its block
// of the state onto the kept eigenvectors.  The state stays in global memory
// (L2-resident).
template <typename T, int D, bool ONE_SIDED>
__global__ void __launch_bounds__(32 * 2 * CHI_TRUNC_ITEMS)
    k_chi_trunc(ChiSched sc, int k, int n_rows, const uint64_t* __restrict__ cfg,
                const int32_t* __restrict__ cfg_idx, const uint8_t* __restrict__ sides, int64_t n_items,
                const int* __restrict__ count, T* __restrict__ state, const int* __restrict__ expo_io) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int warp = threadIdx.x >> 5, ln = threadIdx.x & 31;
  const int il = warp >> 1, b = warp & 1;
  const int64_t item = (int64_t)blockIdx.x * CHI_TRUNC_ITEMS + il;
  const int64_t lim = count ? (int64_t)*count : n_items;
  const bool live = item < n_items && item < lim;
  T* base_s = reinterpret_cast<T*>(smraw) + (size_t)il * (4 * 32 * 33 + 64);
  T* S = base_s + b * 32 * 33;
  T* V = base_s + 2 * 32 * 33 + b * 32 * 33;
  T* lam = base_s + 4 * 32 * 33;  // [2][32]
  int* keep = reinterpret_cast<int*>(reinterpret_cast<T*>(smraw) + (size_t)CHI_TRUNC_ITEMS * (4 * 32 * 33 + 64)) +
              il * 64;
  const int NS = sc.NS;
  int nL = 1;
  for (int i = 0; i < k; ++i) nL *= D;
  const int nR = NS / nL;
  const bool left = nL <= nR;
  const int n = left ? nL : nR, nb = n >> 1, nq = (NS / n) >> 1;
  int64_t ci = 0;
  int side = 0, qcls = 0;
  bool on = false;
  T* st = nullptr;
  if (live) {
    chi_item(item, cfg_idx, sides, ci, side);
    const int ex = expo_io[2 * ci + side];
    on = ex != CHI_EXP_ZERO && ex != CHI_EXP_BAD;
    st = state + (2 * ci + side) * (int64_t)NS;
    qcls = side_parity(cfg[2 * ci], cfg[2 * ci + 1], sc.Lx, sc.Ly, side, n_rows) ^ b;
  }
  const uint32_t pi = block_member<D>(b, ln);
  auto at = [&](uint32_t p, uint32_t q) -> int64_t {
    return left ? (int64_t)p * nR + q : (int64_t)q * nR + p;
  };
  if constexpr (ONE_SIDED) {
    // the block fits a warp's registers (nq <= 32: the middle cut of a 6-wide lattice): one-sided Jacobi on its rows
    T u[32];
#pragma unroll
    for (int j = 0; j < 32; ++j)
      u[j] = (on && ln < nb && j < nq) ? st[at(pi, block_member<D>(qcls, j))] : T(0);
    warp_lq_jacobi<T>(u, nq, S, V, lam + b * 32);
  } else {
    // Gram block: lane i accumulates row i
    T acc[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) acc[j] = T(0);
    if (on)
      for (int iq = 0; iq < nq; ++iq) {
        const uint32_t q = block_member<D>(qcls, iq);
        const T a = (ln < nb) ? st[at(pi, q)] : T(0);
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[j] += a * __shfl_sync(VMC_FULL_MASK, a, j);
      }
#pragma unroll
    for (int j = 0; j < 32; ++j) S[ln * 33 + j] = acc[j];
    __syncwarp();
    warp_jacobi<T>(S, V, lam + b * 32);
  }
  __syncthreads();
  {
    // eigenpairs: lanes < nq (rows of L^T) on the one-sided path, < nb on the Gram path
    const int nval = ONE_SIDED ? nq : nb;
    const T l = lam[b * 32 + ln];
    int rank = 0;
    for (int e = 0; e < 64; ++e) {
      const int b2 = e >> 5, i2 = e & 31;
      if (i2 >= nval) continue;
      const T l2 = lam[e];
      rank += (l2 > l) || (l2 == l && (b2 < b || (b2 == b && i2 < ln)));
    }
    keep[b * 32 + ln] = (ln < nval) && rank < sc.chi;
  }
  __syncwarp();
  // projection of the block onto the kept eigenvectors, one big-side column at a time
  if (on) {
    const T* vi = V + ln * 33;   // eigenvector ln, read from shared memory (keeps registers for the Jacobi)
    const bool kp = keep[b * 32 + ln] != 0;
    for (int iq = 0; iq < nq; ++iq) {
      const uint32_t q = block_member<D>(qcls, iq);
      const T a = (ln < nb) ? st[at(pi, q)] : T(0);
      T y = T(0);
#pragma unroll
      for (int j = 0; j < 32; ++j) y += vi[j] * __shfl_sync(VMC_FULL_MASK, a, j);
      if (!kp) y = T(0);
      T nv = T(0);
#pragma unroll
      for (int i = 0; i < 32; ++i) nv += V[i * 33 + ln] * __shfl_sync(VMC_FULL_MASK, y, i);
      if (ln < nb) st[at(pi, q)] = nv;
    }
  }
}

// (sign, log|psi|) from <top, bottom> * 2^(et + eb) and the global sign.
__device__ __forceinline__ void chi_finish(double v, int et, int eb, uint64_t up, uint64_t dn, double& sgn,
                                           double& la) {
  const int K = __popcll(up ^ dn);
  const double g = ((K * (K - 1) / 2) & 1) ? -1.0 : 1.0;
  if (et == CHI_EXP_BAD || eb == CHI_EXP_BAD || !isfinite(v)) { sgn = 0.0; la = NAN; }
  else if (et == CHI_EXP_ZERO || eb == CHI_EXP_ZERO || v == 0.0) { sgn = 0.0; la = -INFINITY; }
  else {
    sgn = v < 0 ? -g : g;
    la = log(fabs(v)) + (double)(et + eb) * 0.69314718055994530942;
  }
}

template <typename T>
__device__ __forceinline__ double warp_dot(const T* a, const T* b, int NS) {
  double acc = 0.0;
  for (int e = threadIdx.x & 31; e < NS; e += 32) acc += (double)a[e] * (double)b[e];
  return warp_sum(acc);
}

// One warp per configuration: states at st[(2w) * NS] (top), st[(2w+1) * NS].
template <typename T>
__global__ void k_chi_dot(const T* __restrict__ st, const int* __restrict__ ex, int NS,
                          const uint64_t* __restrict__ occ, int64_t R, double* __restrict__ sign,
                          double* __restrict__ logabs) {
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= R) return;
  const double v = warp_dot(st + 2 * w * NS, st + (2 * w + 1) * NS, NS);
  if ((threadIdx.x & 31) == 0) {
    double s, la;
    chi_finish(v, ex[2 * w], ex[2 * w + 1], occ[2 * w], occ[2 * w + 1], s, la);
    sign[w] = s;
    logabs[w] = la;
  }
}


// Warp-aggregated append of k items (k in {0, 1, 2}) to a device list; returns
// the first index of this lane's items.
__device__ __forceinline__ int warp_append(int k, int* count) {
  const int ln = threadIdx.x & 31;
  int incl = k;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(VMC_FULL_MASK, incl, o);
    if (ln >= o) incl += y;
  }
  const int tot = __shfl_sync(VMC_FULL_MASK, incl, 31);
  int base = 0;
  if (ln == 31 && tot) base = atomicAdd(count, tot);
  base = __shfl_sync(VMC_FULL_MASK, base, 31);
  return base + incl - k;
}

// Sides whose boundary state a change of sites i and j touches.
__device__ __forceinline__ int touched_sides(int i, int j, int Ly, int half) {
  const int ri = i / Ly, rj = j / Ly;
  return ((ri < half || rj < half) ? 1 : 0) | ((ri >= half || rj >= half) ? 2 : 0);
}

// One proposal per walker on edge e (the draws and proposal of k_peps_sweep):
// proposed configuration, touched sides, and the side-state items to build.
__global__ void k_chi_propose(const uint64_t* __restrict__ occ, int64_t n, int64_t w0, int64_t B, int Ly, int half,
                              const int32_t* __restrict__ edges, int e, int E, int s, float hopping_rate,
                              uint64_t seed, uint64_t sweep_offset, const float* __restrict__ r_move,
                              const uint8_t* __restrict__ r_bit, const float* __restrict__ r_acc,
                              uint64_t* __restrict__ prop, uint8_t* __restrict__ flags, float* __restrict__ u_acc,
                              int32_t* __restrict__ cfg_idx, uint8_t* __restrict__ sides, int* __restrict__ count) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int f = 0;
  if (w < n) {
    const uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
    const int i = edges[2 * e], j = edges[2 * e + 1];
    const int xi = site_state(up, dn, i), xj = site_state(up, dn, j);
    if (xi != xj) {
      float um, ua;
      int bit;
      const int64_t gw = w0 + w;
      if (r_move) {
        const size_t ridx = ((size_t)s * E + e) * (size_t)B + (size_t)gw;
        um = r_move[ridx]; bit = r_bit[ridx] & 1; ua = r_acc[ridx];
      } else {
        EdgeDraw d = draw_edge(seed, (uint64_t)gw, sweep_offset + (uint64_t)s, (uint32_t)e);
        um = d.u_move; bit = d.bit; ua = d.u_acc;
      }
      int ni, nj;
      propose_pair(xi, xj, um, bit, hopping_rate, ni, nj);
      const uint64_t mi = 1ull << i, mj = 1ull << j;
      uint64_t up1 = up & ~(mi | mj), dn1 = dn & ~(mi | mj);
      if (ni & 2) up1 |= mi;
      if (ni & 1) dn1 |= mi;
      if (nj & 2) up1 |= mj;
      if (nj & 1) dn1 |= mj;
      prop[2 * w] = up1;
      prop[2 * w + 1] = dn1;
      u_acc[w] = ua;
      f = touched_sides(i, j, Ly, half);
    }
    flags[w] = (uint8_t)f;
  }
  const int k = (f & 1) + ((f >> 1) & 1);
  const int base = warp_append(k, count);
  int o = base;
  if (f & 1) { cfg_idx[o] = (int32_t)w; sides[o] = 0; ++o; }
  if (f & 2) { cfg_idx[o] = (int32_t)w; sides[o] = 1; }
}

// Metropolis decision for every walker with a proposal: amplitude from the
// rebuilt sides (new) and the kept ones (cur); on acceptance the new states
// replace the current ones.  One warp per walker.
template <typename T>
__global__ void k_chi_accept(int NS, int64_t n, T* __restrict__ cur, int* __restrict__ cur_ex,
                             const T* __restrict__ nw, const int* __restrict__ nw_ex, const uint8_t* __restrict__ flags,
                             const uint64_t* __restrict__ prop, const float* __restrict__ u_acc,
                             uint64_t* __restrict__ occ, double* __restrict__ sign, double* __restrict__ logabs,
                             int32_t* __restrict__ n_acc, unsigned long long* __restrict__ n_eval) {
  __shared__ int evals, builds;
  if (threadIdx.x == 0) { evals = 0; builds = 0; }
  __syncthreads();
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int ln = threadIdx.x & 31;
  const int f = (w < n) ? flags[w] : 0;
  if (f) {
    const T* a = ((f & 1) ? nw : cur) + 2 * w * NS;
    const T* b = ((f & 2) ? nw : cur) + (2 * w + 1) * NS;
    const int et = ((f & 1) ? nw_ex : cur_ex)[2 * w], eb = ((f & 2) ? nw_ex : cur_ex)[2 * w + 1];
    const double v = warp_dot(a, b, NS);
    int acc = 0;
    double s1 = 0.0, la1 = 0.0;
    if (ln == 0) {
      chi_finish(v, et, eb, prop[2 * w], prop[2 * w + 1], s1, la1);
      const double la = logabs[w];
      if (!(la1 > -INFINITY)) acc = 0;
      else if (la == -INFINITY) acc = 1;
      else acc = (double)u_acc[w] < exp(2.0 * (la1 - la));
      atomicAdd(&evals, 1);
      atomicAdd(&builds, (f & 1) + ((f >> 1) & 1));
    }
    acc = __shfl_sync(VMC_FULL_MASK, acc, 0);
    if (acc) {
      for (int sd = 0; sd < 2; ++sd)
        if (f & (1 << sd)) {
          const int64_t o = (2 * w + sd) * NS;
          for (int e2 = ln; e2 < NS; e2 += 32) cur[o + e2] = nw[o + e2];
          if (ln == 0) cur_ex[2 * w + sd] = nw_ex[2 * w + sd];
        }
      if (ln == 0) {
        occ[2 * w] = prop[2 * w];
        occ[2 * w + 1] = prop[2 * w + 1];
        sign[w] = s1;
        logabs[w] = la1;
        if (n_acc) n_acc[w] += 1;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && n_eval && evals) {
    atomicAdd(n_eval, (unsigned long long)evals);
    atomicAdd(n_eval + 1, (unsigned long long)builds);
  }
}

// Local-energy terms: the configuration of every hop term (the move of
// k_peps_conn_terms) and the side states it needs rebuilt.
__global__ void k_chi_term_prep(const uint64_t* __restrict__ occ, int N, int Ly, int half,
                                const int32_t* __restrict__ pairs, int64_t p0, int64_t np, int64_t w0,
                                const int32_t* __restrict__ edges, uint64_t* __restrict__ prop,
                                uint8_t* __restrict__ flags, int32_t* __restrict__ cfg_idx,
                                uint8_t* __restrict__ sides, int* __restrict__ count) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int f = 0;
  if (p < np) {
    const int w = pairs[2 * (p0 + p)], tm = pairs[2 * (p0 + p) + 1];
    const uint64_t up = occ[2 * (int64_t)w], dn = occ[2 * (int64_t)w + 1];
    const int e = tm >> 1, sp = (tm & 1) ? 0 : 1;
    int i = edges[2 * e], j = edges[2 * e + 1];
    if (i > j) { const int tt = i; i = j; j = tt; }
    const uint64_t m = sp ? up : dn;
    const int oi = (int)((m >> i) & 1ull);
    const int base = sp ? 0 : N;
    uint64_t eu = up, ed = dn;
    apply_move(eu, ed, N, base + (oi ? i : j), base + (oi ? j : i));
    prop[2 * p] = eu;
    prop[2 * p + 1] = ed;
    f = touched_sides(i, j, Ly, half);
    flags[p] = (uint8_t)f;
    (void)w0;
  }
  const int k = (f & 1) + ((f >> 1) & 1);
  const int b = warp_append(k, count);
  int o = b;
  if (f & 1) { cfg_idx[o] = (int32_t)p; sides[o] = 0; ++o; }
  if (f & 2) { cfg_idx[o] = (int32_t)p; sides[o] = 1; }
}

// term = H_{x,x'} psi(x') / psi(x) for each pair of the block; the walker's
// own states (cur, slot 2(w - w0) + side) fill in the untouched side.
template <typename T>
__global__ void k_chi_terms(int NS, int N, const uint64_t* __restrict__ occ, const int32_t* __restrict__ pairs,
                            int64_t p0, int64_t np, int64_t w0, const int32_t* __restrict__ edges, double t,
                            const T* __restrict__ cur, const int* __restrict__ cur_ex, const double* __restrict__ s0a,
                            const double* __restrict__ la0a, const T* __restrict__ nw, const int* __restrict__ nw_ex,
                            const uint8_t* __restrict__ flags, const uint64_t* __restrict__ prop,
                            double* __restrict__ term) {
  const int64_t p = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (p >= np) return;
  const int w = pairs[2 * (p0 + p)], tm = pairs[2 * (p0 + p) + 1];
  const int64_t lw = w - w0;
  const int f = flags[p];
  const T* a = (f & 1) ? nw + 2 * p * NS : cur + 2 * lw * NS;
  const T* b = (f & 2) ? nw + (2 * p + 1) * NS : cur + (2 * lw + 1) * NS;
  const int et = (f & 1) ? nw_ex[2 * p] : cur_ex[2 * lw], eb = (f & 2) ? nw_ex[2 * p + 1] : cur_ex[2 * lw + 1];
  const double v = warp_dot(a, b, NS);
  if ((threadIdx.x & 31) == 0) {
    const uint64_t up = occ[2 * (int64_t)w], dn = occ[2 * (int64_t)w + 1];
    const int e = tm >> 1, sp = (tm & 1) ? 0 : 1;
    int i = edges[2 * e], j = edges[2 * e + 1];
    if (i > j) { const int tt = i; i = j; j = tt; }
    const double coeff = symmray_parity(up, dn, i, j, sp) ? t : -t;
    double s1, la1;
    chi_finish(v, et, eb, prop[2 * p], prop[2 * p + 1], s1, la1);
    const double s0 = s0a[lw], la0 = la0a[lw];
    term[p0 + p] = (s1 == 0.0 || s0 == 0.0) ? 0.0 : coeff * s1 * s0 * exp(la1 - la0);
    (void)N;
  }
}

__global__ void k_chi_eloc_reduce(int64_t B, const uint64_t* __restrict__ occ, const int32_t* __restrict__ offs,
                                  const double* __restrict__ term, double U, double* __restrict__ eloc) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= B) return;
  double s = U * (double)__popcll(occ[2 * w] & occ[2 * w + 1]);
  for (int q = offs[w]; q < offs[w + 1]; ++q) s += term[q];
  eloc[w] = s;
}

// ---------------------------------------------------------------------------
// Log-derivatives through the truncation (schedules whose only truncated cut
// is one cut after each side's last row, with parity blocks that fit a warp:
// 6x6 D=4 chi in [16, 64), 4x4 D=4 chi in [4, 16)).  With z = <P(phi_t),
// beta_b> in the normalised units of the states (phi_t the top state before
// its truncation P, beta_b the truncated bottom state):
//   dz = <dphi_t, cot_t>,  cot_t = (dP at phi_t)^T beta_b,
// and d log|psi| / dA(r, c) = <d phi_t / dA(r, c), cot_t> / z, the hole
// contraction of the side's rows against cot_t (likewise for the bottom).
// The cotangent of the rank-k truncation of M = sum_i s_i q_i v_i^T (q, v
// singular vectors, u_i = s_i v_i the one-sided Jacobi rows) against B is
//   Mbar = P_k B + sum_{i kept, j dropped} w_ij (q_j u_i^T + q_i u_j^T),
//   w_ij = (q_j^T B u_i + q_i^T B u_j) / (s_i^2 - s_j^2),
// the first-order change of the kept subspace (it couples kept and dropped
// directions only, and only within a parity block).
// ---------------------------------------------------------------------------
template <typename T>
struct ChiAdj {
  static constexpr int ITEMS = sizeof(T) == 4 ? 4 : 2;  // items per CTA (two warps each)
  static constexpr int PER_ITEM = 2 * 4 * 32 * 33 + 64;  // T elements: per block Q, U, B/X, C/R; lam
  static size_t bytes() { return (size_t)ITEMS * (PER_ITEM * sizeof(T) + 64 * sizeof(int)); }
};

template <typename T, int D>
__global__ void __launch_bounds__(64 * ChiAdj<T>::ITEMS)
    k_chi_trunc_adj(ChiSched sc, int k, const uint64_t* __restrict__ cfg, int64_t n_items,
                    const T* __restrict__ phi_keep, const T* __restrict__ trunc_state, const int* __restrict__ ex,
                    T* __restrict__ cot) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int warp = threadIdx.x >> 5, ln = threadIdx.x & 31;
  const int il = warp >> 1, b = warp & 1;
  const int64_t item = (int64_t)blockIdx.x * ChiAdj<T>::ITEMS + il;
  const bool live = item < n_items;
  T* base_s = reinterpret_cast<T*>(smraw) + (size_t)il * ChiAdj<T>::PER_ITEM;
  T* Qs = base_s + (b * 4 + 0) * 32 * 33;
  T* Us = base_s + (b * 4 + 1) * 32 * 33;
  T* BX = base_s + (b * 4 + 2) * 32 * 33;
  T* CR = base_s + (b * 4 + 3) * 32 * 33;
  T* lam = base_s + 8 * 32 * 33;  // [2][32]
  int* keep = reinterpret_cast<int*>(reinterpret_cast<T*>(smraw) + (size_t)ChiAdj<T>::ITEMS * ChiAdj<T>::PER_ITEM) +
              il * 64;
  const int NS = sc.NS;
  int nL = 1;
  for (int i = 0; i < k; ++i) nL *= D;
  const int nR = NS / nL;
  const bool left = nL <= nR;
  const int n = left ? nL : nR, nb = n >> 1, nq = (NS / n) >> 1;
  bool on = false;
  int qcls = 0;
  const T* phi = nullptr;
  const T* bst = nullptr;
  if (live) {
    const int64_t ci = item >> 1;
    const int side = (int)(item & 1);
    on = ex[item] != CHI_EXP_ZERO && ex[item] != CHI_EXP_BAD && ex[item ^ 1] != CHI_EXP_ZERO &&
         ex[item ^ 1] != CHI_EXP_BAD;
    phi = phi_keep + (item * sc.rows + sc.rows - 1) * (int64_t)NS;
    bst = trunc_state + (item ^ 1) * (int64_t)NS;
    qcls = side_parity(cfg[2 * ci], cfg[2 * ci + 1], sc.Lx, sc.Ly, side, sc.rows) ^ b;
  }
  const uint32_t pi = block_member<D>(b, ln);
  auto at = [&](uint32_t p, uint32_t q) -> int64_t {
    return left ? (int64_t)p * nR + q : (int64_t)q * nR + p;
  };
  T u[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) u[j] = (on && ln < nb && j < nq) ? phi[at(pi, block_member<D>(qcls, j))] : T(0);
  warp_hestenes<T>(u, Qs, lam + b * 32);
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    Us[ln * 33 + j] = u[j];
    BX[ln * 33 + j] = (on && ln < nb && j < nq) ? bst[at(pi, block_member<D>(qcls, j))] : T(0);
  }
  __syncthreads();
  {
    const T l = lam[b * 32 + ln];
    int rank = 0;
    for (int e = 0; e < 64; ++e) {
      const int b2 = e >> 5, i2 = e & 31;
      if (i2 >= nb) continue;
      const T l2 = lam[e];
      rank += (l2 > l) || (l2 == l && (b2 < b || (b2 == b && i2 < ln)));
    }
    keep[b * 32 + ln] = (ln < nb) && rank < sc.chi;
  }
  __syncthreads();
  // C = Q B (lane a: row a)
  T crow[32];
  {
    T qrow[32];
#pragma unroll
    for (int p = 0; p < 32; ++p) qrow[p] = Qs[ln * 33 + p];
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      T acc = T(0);
#pragma unroll
      for (int p = 0; p < 32; ++p) acc = fma(qrow[p], BX[p * 33 + q], acc);
      crow[q] = acc;
    }
  }
  __syncwarp();
  // X[a][c] = q_a^T B u_c, into BX
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    T acc = T(0);
#pragma unroll
    for (int q = 0; q < 32; ++q) acc = fma(crow[q], Us[c * 33 + q], acc);
    BX[ln * 33 + c] = acc;
  }
  __syncwarp();
  // R[a][:] = keep_a C[a][:] + sum over mixed pairs (a, c) of w * u_c
  {
    const bool ka = keep[b * 32 + ln] != 0;
    const T la = lam[b * 32 + ln];
    T r[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) r[q] = ka ? crow[q] : T(0);
    for (int c = 0; c < nb; ++c) {
      const bool kc = keep[b * 32 + c] != 0;
      if (ka == kc || ln >= nb) continue;
      const T den = ka ? (la - lam[b * 32 + c]) : (lam[b * 32 + c] - la);
      const T w = (BX[ln * 33 + c] + BX[c * 33 + ln]) / den;
#pragma unroll
      for (int q = 0; q < 32; ++q) r[q] = fma(w, Us[c * 33 + q], r[q]);
    }
#pragma unroll
    for (int q = 0; q < 32; ++q) CR[ln * 33 + q] = r[q];
  }
  __syncwarp();
  // Mbar = Q^T R: lane p writes row p of the block
  if (on && ln < nb) {
    T* ct = cot + item * (int64_t)NS;
    for (int q = 0; q < nq; ++q) {
      T acc = T(0);
#pragma unroll
      for (int a = 0; a < 32; ++a) acc = fma(Qs[a * 33 + ln], CR[a * 33 + q], acc);
      ct[at(pi, block_member<D>(qcls, q))] = acc;
    }
  }
}

// z[w] = <top, bottom> of the normalised truncated states (FP64), 0 when a side vanished.
template <typename T>
__global__ void k_chi_zdot(const T* __restrict__ st, const int* __restrict__ ex, int NS, int64_t R,
                           double* __restrict__ z) {
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= R) return;
  const double v = warp_dot(st + 2 * w * NS, st + (2 * w + 1) * NS, NS);
  if ((threadIdx.x & 31) == 0) {
    const bool dead = ex[2 * w] == CHI_EXP_ZERO || ex[2 * w] == CHI_EXP_BAD || ex[2 * w + 1] == CHI_EXP_ZERO ||
                      ex[2 * w + 1] == CHI_EXP_BAD;
    z[w] = dead ? 0.0 : v;
  }
}

// Reverse row sweep of one side (item = 2 w + side): the cotangent of the
// side's final state goes back through its rows (each row's exponent scales
// it), column by column; the forward state before a column is recomputed from
// the row's stored input state.  Per column the site's gradient is
// sum over groups of (input entry) x (output cotangent), written to O with the
// sign rule's sign and divided by z.  W and the cotangent Wb in shared memory.
template <typename T, int D>
__global__ void __launch_bounds__(CHI_NT)
    k_chi_grad_side(const T* __restrict__ tens, ChiSched sc, const uint64_t* __restrict__ cfg, int64_t n_items,
                    const T* __restrict__ keep, const int* __restrict__ row_e, const T* __restrict__ cot,
                    const double* __restrict__ z, T* __restrict__ O, int64_t ldo) {
  constexpr int H = D * D / 2, NE = 2 * H * H;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int64_t item = blockIdx.x;
  if (item >= n_items) return;
  const int NS = sc.NS, Ly = sc.Ly, Lx = sc.Lx;
  T* W = reinterpret_cast<T*>(smraw);
  T* Wb = W + (size_t)D * NS;
  T* A2 = Wb + (size_t)D * NS;
  T* part = A2 + (size_t)Ly * NE;   // [CHI_NT / NE][NE]
  T* red = part + CHI_NT;
  const int64_t w = item >> 1;
  const int side = (int)(item & 1);
  const uint64_t up = cfg[2 * w], dn = cfg[2 * w + 1];
  const double zw = z[w];
  if (zw == 0.0 || !isfinite(zw)) return;
  T* Ow = O + w * ldo;
  for (int e = threadIdx.x; e < D * NS; e += blockDim.x) Wb[e] = (e < NS) ? cot[item * (int64_t)NS + e] : T(0);
  int fexp = 0;  // the cotangent is Wb * 2^fexp
  const int halves = CHI_NT / NE;
  for (int a = sc.rows - 1; a >= 0; --a) {
    const int r = side ? (Lx - 1 - a) : a;
    fexp -= row_e[item * sc.rows + a];
    __syncthreads();
    load_row_tables<T, D>(tens, up, dn, r, Ly, side, A2);
    const int par0 = side_parity(up, dn, Lx, Ly, side, a);
    const T* in_state = a > 0 ? keep + (item * sc.rows + a - 1) * (int64_t)NS : nullptr;
    for (int c = Ly - 1; c >= 0; --c) {
      // forward state before column c
      __syncthreads();
      for (int e = threadIdx.x; e < D * NS; e += blockDim.x)
        W[e] = (e < NS) ? (in_state ? in_state[e] : (e == 0 ? T(1) : T(0))) : T(0);
      int par = par0, stride = NS / D;
      for (int c2 = 0; c2 < c; ++c2, stride /= D) {
        const int x2 = site_state(up, dn, r * Ly + c2);
        const int px2 = (x2 ^ (x2 >> 1)) & 1;
        __syncthreads();
        column_forward<T, D>(W, NS, stride, par, px2, A2 + c2 * NE);
        par ^= px2;
      }
      __syncthreads();
      const int site = r * Ly + c;
      const int x = site_state(up, dn, site);
      const int px = (x ^ (x >> 1)) & 1;
      // gradient of the site's table: thread (half, e), e = (ti, ia, ib)
      {
        const int e = threadIdx.x % NE, hf = threadIdx.x / NE;
        const int ti = e / (H * H), ia = (e / H) % H, ib = e % H;
        int o, h, nn, hp;
        class_pair<D>(ti, ia, o, h);
        class_pair<D>(ti ^ px, ib, nn, hp);
        T acc = T(0);
        if (hf < halves)
          for (int gi = hf; gi < NS / D; gi += halves) {
            const int lo = gi % stride, hi = gi / stride;
            const int base = hi * stride * D + lo;
            if (((par ^ digit_parity<D>((uint32_t)base)) & 1) != ti) continue;
            acc = fma(W[h * NS + base + o * stride], Wb[hp * NS + base + nn * stride], acc);
          }
        part[threadIdx.x] = acc;
      }
      __syncthreads();
      if (threadIdx.x < NE) {
        T tot = T(0);
        for (int hf = 0; hf < halves; ++hf) tot += part[hf * NE + threadIdx.x];
        const int e = threadIdx.x, ti = e / (H * H), ia = (e / H) % H, ib = e % H;
        const uint64_t lm = bits_below(site) & ~bits_below(r * Ly);
        const int nleft = __popcll(up & lm) + __popcll(dn & lm);
        int sgn;
        const int idx = table_entry<D>(ti, ia, ib, px, side, r, nleft, sgn);
        const double g = (double)sgn * ldexp((double)tot, fexp) / zw;
        Ow[((int64_t)site * 4 + x) * (D * D * D * D) + idx] = (T)g;
      }
      __syncthreads();
      column_adjoint<T, D>(Wb, NS, stride, par, px, A2 + c * NE);
    }
    __syncthreads();
    // the cotangent of the row's input state: slice h = 0; renormalise by a power of two
    T m = T(0);
    for (int e = threadIdx.x; e < D * NS; e += blockDim.x) {
      if (e >= NS) Wb[e] = T(0);
      else m = fmax(m, fabs(Wb[e]));
    }
    m = cta_absmax<T>(m, red);
    if (m > T(0) && m < T(INFINITY)) {
      const int e2 = (int)ilogb(m);
      fexp += e2;
      __syncthreads();
      for (int e = threadIdx.x; e < NS; e += blockDim.x) Wb[e] = scalbn(Wb[e], -e2);
    }
  }
}


int chi_plan(int Lx, int Ly, int D, int chi, ChiSched& sc) {
  if (Lx < 2 || (Lx & 1) || Ly < 1 || Lx * Ly > 64 || (D != 2 && D != 4) || chi < 1) return VMC_ERR_UNSUPPORTED;
  int64_t NS = 1;
  for (int c = 0; c < Ly; ++c) NS *= D;
  if (NS > CHI_MAX_NS || NS < 2) return VMC_ERR_UNSUPPORTED;
  sc = ChiSched{};
  sc.Lx = Lx; sc.Ly = Ly; sc.D = D; sc.NS = (int)NS; sc.chi = chi; sc.rows = Lx / 2;
  int64_t b[16];
  for (int k = 0; k <= Ly; ++k) b[k] = 1;
  for (int a = 0; a < sc.rows; ++a) {
    for (int k = 1; k < Ly; ++k) {
      int64_t lk = 1, rk = 1;
      for (int i = 0; i < k; ++i) lk *= D;
      for (int i = k; i < Ly; ++i) rk *= D;
      int64_t nb = b[k] * D;
      if (nb > lk) nb = lk;
      if (nb > rk) nb = rk;
      b[k] = nb;
    }
    uint32_t m = 0;
    if (a >= 1)
      for (int k = Ly - 1; k >= 1; --k)
        if (b[k] > chi) {
          m |= 1u << k;
          b[k] = chi;
          if (k > 1 && b[k - 1] > (int64_t)D * chi) b[k - 1] = (int64_t)D * chi;
        }
    sc.cuts[a] = m;
  }
  return VMC_OK;
}

template <typename T, int D>
int build_sides_d(const void* tens, const ChiSched& sc, const uint64_t* cfg, const int32_t* cfg_idx,
                  const uint8_t* sides, int64_t n_items, const int* count, T* state, int* ex, cudaStream_t st,
                  T* keep = nullptr, int* row_e = nullptr) {
  const size_t smem = ChiSmem<T>::bytes(sc.NS, D, sc.Ly);
  if (cudaFuncSetAttribute(k_chi_absorb<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return VMC_ERR_CUDA;
  const size_t tsm = ChiTruncSmem<T>::bytes();
  if (cudaFuncSetAttribute(k_chi_trunc<T, D, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm) !=
          cudaSuccess ||
      cudaFuncSetAttribute(k_chi_trunc<T, D, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm) !=
          cudaSuccess)
    return VMC_ERR_CUDA;
  int a = 0;
  while (a < sc.rows) {
    int a1 = a + 1;
    while (a1 < sc.rows && sc.cuts[a1 - 1] == 0) ++a1;
    k_chi_absorb<T, D><<<(unsigned)n_items, CHI_NT, smem, st>>>((const T*)tens, sc, cfg, cfg_idx, sides, n_items,
                                                                count, a, a1, state, ex, keep, row_e);
    VMC_CUDA_CHECK_LAUNCH();
    for (int k = sc.Ly - 1; k >= 1; --k)
      if ((sc.cuts[a1 - 1] >> k) & 1u) {
        int nL = 1;
        for (int i = 0; i < k; ++i) nL *= D;
        const int n = nL <= sc.NS / nL ? nL : sc.NS / nL;
        const unsigned grid = (unsigned)((n_items + CHI_TRUNC_ITEMS - 1) / CHI_TRUNC_ITEMS);
        if ((sc.NS / n) / 2 <= 32)
          k_chi_trunc<T, D, true><<<grid, 64 * CHI_TRUNC_ITEMS, tsm, st>>>(sc, k, a1, cfg, cfg_idx, sides, n_items,
                                                                            count, state, ex);
        else
          k_chi_trunc<T, D, false><<<grid, 64 * CHI_TRUNC_ITEMS, tsm, st>>>(sc, k, a1, cfg, cfg_idx, sides, n_items,
                                                                             count, state, ex);
        VMC_CUDA_CHECK_LAUNCH();
      }
    a = a1;
  }
  return VMC_OK;
}

// Boundary states of n_items (configuration, side) items into slots
// 2 ci + side of state / ex: the rows of the schedule absorbed in runs that
// end at a row with truncated cuts, each cut then truncated.
template <typename T>
int launch_chi_side(const void* tens, const ChiSched& sc, const uint64_t* cfg, const int32_t* cfg_idx,
                    const uint8_t* sides, int64_t n_items, const int* count, T* state, int* ex, cudaStream_t st) {
  if (n_items <= 0) return VMC_OK;
  return sc.D == 4 ? build_sides_d<T, 4>(tens, sc, cfg, cfg_idx, sides, n_items, count, state, ex, st)
                   : build_sides_d<T, 2>(tens, sc, cfg, cfg_idx, sides, n_items, count, state, ex, st);
}


// Per-chunk workspace (work_rows walkers): current and new side states, their
// exponents, proposed configurations, item lists.
template <typename T>
struct ChiWork {
  T* cur; T* nw; int* cur_ex; int* nw_ex; uint64_t* prop; int32_t* cfg_idx; uint8_t* sides; uint8_t* flags;
  float* u_acc; int* count; double* s0; double* la0;
  static int64_t bytes(int NS, int64_t rows) {
    return rows * (4 * (int64_t)NS * (int64_t)sizeof(T) + 4 * 4 + 16 + 8 + 2 + 1 + 4 + 16) + 16 * 256;
  }
  ChiWork(void* base, int NS, int64_t rows) {
    char* p = (char*)base;
    auto take = [&](int64_t nbytes) { char* q = p; p += (nbytes + 255) & ~int64_t(255); return q; };
    cur = (T*)take(2 * rows * NS * (int64_t)sizeof(T));
    nw = (T*)take(2 * rows * NS * (int64_t)sizeof(T));
    prop = (uint64_t*)take(2 * rows * 8);
    s0 = (double*)take(rows * 8);
    la0 = (double*)take(rows * 8);
    cur_ex = (int*)take(2 * rows * 4);
    nw_ex = (int*)take(2 * rows * 4);
    cfg_idx = (int32_t*)take(2 * rows * 4);
    u_acc = (float*)take(rows * 4);
    count = (int*)take(256);
    sides = (uint8_t*)take(2 * rows);
    flags = (uint8_t*)take(rows);
  }
};

template <typename T>
int chi_eval(const void* tens, const ChiSched& sc, const uint64_t* occ, int64_t R, double* sign, double* logabs,
             void* work, int64_t work_rows, cudaStream_t st) {
  ChiWork<T> W(work, sc.NS, work_rows);
  for (int64_t w0 = 0; w0 < R; w0 += work_rows) {
    const int64_t n = (R - w0) < work_rows ? (R - w0) : work_rows;
    int rc = launch_chi_side<T>(tens, sc, occ + 2 * w0, nullptr, nullptr, 2 * n, nullptr, W.cur, W.cur_ex, st);
    if (rc) return rc;
    k_chi_dot<T><<<(unsigned)((n + 7) / 8), 256, 0, st>>>(W.cur, W.cur_ex, sc.NS, occ + 2 * w0, n, sign + w0,
                                                          logabs + w0);
    VMC_CUDA_CHECK_LAUNCH();
  }
  return VMC_OK;
}

template <typename T>
int chi_sweep(const void* tens, const ChiSched& sc, uint64_t* occ, int64_t B, const int32_t* edges, int E,
              int n_sweeps, float hopping_rate, uint64_t seed, uint64_t sweep_offset, const float* r_move,
              const uint8_t* r_bit, const float* r_acc, double* sign, double* logabs, int32_t* n_acc,
              unsigned long long* n_eval, void* work, int64_t work_rows, cudaStream_t st) {
  ChiWork<T> W(work, sc.NS, work_rows);
  for (int64_t w0 = 0; w0 < B; w0 += work_rows) {
    const int64_t n = (B - w0) < work_rows ? (B - w0) : work_rows;
    int rc = launch_chi_side<T>(tens, sc, occ + 2 * w0, nullptr, nullptr, 2 * n, nullptr, W.cur, W.cur_ex, st);
    if (rc) return rc;
    k_chi_dot<T><<<(unsigned)((n + 7) / 8), 256, 0, st>>>(W.cur, W.cur_ex, sc.NS, occ + 2 * w0, n, sign + w0,
                                                          logabs + w0);
    VMC_CUDA_CHECK_LAUNCH();
    for (int s = 0; s < n_sweeps; ++s)
      for (int e = 0; e < E; ++e) {
        if (cudaMemsetAsync(W.count, 0, sizeof(int), st) != cudaSuccess) return VMC_ERR_CUDA;
        k_chi_propose<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
            occ + 2 * w0, n, w0, B, sc.Ly, sc.rows, edges, e, E, s, hopping_rate, seed, sweep_offset, r_move, r_bit,
            r_acc, W.prop, W.flags, W.u_acc, W.cfg_idx, W.sides, W.count);
        VMC_CUDA_CHECK_LAUNCH();
        rc = launch_chi_side<T>(tens, sc, W.prop, W.cfg_idx, W.sides, 2 * n, W.count, W.nw, W.nw_ex, st);
        if (rc) return rc;
        k_chi_accept<T><<<(unsigned)((n + 7) / 8), 256, 0, st>>>(sc.NS, n, W.cur, W.cur_ex, W.nw, W.nw_ex, W.flags,
                                                                 W.prop, W.u_acc, occ + 2 * w0, sign + w0,
                                                                 logabs + w0, n_acc ? n_acc + w0 : nullptr, n_eval);
        VMC_CUDA_CHECK_LAUNCH();
      }
  }
  return VMC_OK;
}

// The pair range of a walker chunk comes from offs_host (a host copy of offs).
template <typename T>
int chi_local_energy(const void* tens, const ChiSched& sc, const uint64_t* occ, int64_t B, const int32_t* edges,
                     double t, double U, const int32_t* pairs, const int32_t* offs, const int32_t* offs_host,
                     double* term, double* eloc, void* work, int64_t work_rows, cudaStream_t st) {
  ChiWork<T> W(work, sc.NS, work_rows);
  const int N = sc.Lx * sc.Ly;
  for (int64_t w0 = 0; w0 < B; w0 += work_rows) {
    const int64_t n = (B - w0) < work_rows ? (B - w0) : work_rows;
    int rc = launch_chi_side<T>(tens, sc, occ + 2 * w0, nullptr, nullptr, 2 * n, nullptr, W.cur, W.cur_ex, st);
    if (rc) return rc;
    k_chi_dot<T><<<(unsigned)((n + 7) / 8), 256, 0, st>>>(W.cur, W.cur_ex, sc.NS, occ + 2 * w0, n, W.s0, W.la0);
    VMC_CUDA_CHECK_LAUNCH();
    const int64_t pa = offs_host[w0], pb = offs_host[w0 + n];
    for (int64_t p0 = pa; p0 < pb; p0 += work_rows) {
      const int64_t np = (pb - p0) < work_rows ? (pb - p0) : work_rows;
      if (cudaMemsetAsync(W.count, 0, sizeof(int), st) != cudaSuccess) return VMC_ERR_CUDA;
      k_chi_term_prep<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(occ, N, sc.Ly, sc.rows, pairs, p0, np, w0, edges,
                                                                    W.prop, W.flags, W.cfg_idx, W.sides, W.count);
      VMC_CUDA_CHECK_LAUNCH();
      rc = launch_chi_side<T>(tens, sc, W.prop, W.cfg_idx, W.sides, 2 * np, W.count, W.nw, W.nw_ex, st);
      if (rc) return rc;
      k_chi_terms<T><<<(unsigned)((np + 7) / 8), 256, 0, st>>>(sc.NS, N, occ, pairs, p0, np, w0, edges, t, W.cur,
                                                               W.cur_ex, W.s0, W.la0, W.nw, W.nw_ex, W.flags, W.prop,
                                                               term);
      VMC_CUDA_CHECK_LAUNCH();
    }
  }
  k_chi_eloc_reduce<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(B, occ, offs, term, U, eloc);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}


// Truncation schedules the adjoint supports: one truncated cut, after each
// side's last row, whose parity blocks fit a warp.  Returns that cut or 0.
int chi_grad_cut(const ChiSched& sc) {
  for (int a = 0; a + 1 < sc.rows; ++a)
    if (sc.cuts[a]) return 0;
  const uint32_t m = sc.cuts[sc.rows - 1];
  if (!m || (m & (m - 1))) return 0;
  int k = 0;
  while (!((m >> k) & 1u)) ++k;
  int nL = 1;
  for (int i = 0; i < k; ++i) nL *= sc.D;
  const int n = nL <= sc.NS / nL ? nL : sc.NS / nL;
  return (sc.NS / n) / 2 <= 32 ? k : 0;
}

template <typename T>
size_t chi_grad_smem(const ChiSched& sc) {
  const int H = sc.D * sc.D / 2;
  return ((size_t)2 * sc.D * sc.NS + (size_t)sc.Ly * 2 * H * H + CHI_NT + 32) * sizeof(T) + 16;
}

template <typename T>
int64_t chi_grad_bytes(const ChiSched& sc, int64_t rows) {
  return rows * (2 * ((int64_t)sc.rows + 2) * sc.NS * (int64_t)sizeof(T) + 2 * 4 + 2 * (int64_t)sc.rows * 4 + 8) +
         8 * 256;
}

template <typename T, int D>
int chi_logpsi_grad_d(const void* tens, const ChiSched& sc, int k, const uint64_t* occ, int64_t B, T* O, int64_t ldo,
                      void* work, int64_t work_rows, cudaStream_t st) {
  const size_t gsm = chi_grad_smem<T>(sc), asm_ = ChiAdj<T>::bytes();
  if (gsm > 227 * 1024) return VMC_ERR_UNSUPPORTED;
  if (cudaFuncSetAttribute(k_chi_grad_side<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsm) !=
          cudaSuccess ||
      cudaFuncSetAttribute(k_chi_trunc_adj<T, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)asm_) !=
          cudaSuccess)
    return VMC_ERR_CUDA;
  char* p = (char*)work;
  auto take = [&](int64_t nbytes) { char* q = p; p += (nbytes + 255) & ~int64_t(255); return q; };
  T* keep = (T*)take(2 * work_rows * sc.rows * (int64_t)sc.NS * (int64_t)sizeof(T));
  T* state = (T*)take(2 * work_rows * (int64_t)sc.NS * (int64_t)sizeof(T));
  T* cot = (T*)take(2 * work_rows * (int64_t)sc.NS * (int64_t)sizeof(T));
  int* ex = (int*)take(2 * work_rows * 4);
  int* row_e = (int*)take(2 * work_rows * sc.rows * 4);
  double* z = (double*)take(work_rows * 8);
  for (int64_t w0 = 0; w0 < B; w0 += work_rows) {
    const int64_t n = (B - w0) < work_rows ? (B - w0) : work_rows;
    const uint64_t* cfg = occ + 2 * w0;
    if (cudaMemsetAsync(cot, 0, 2 * n * (size_t)sc.NS * sizeof(T), st) != cudaSuccess) return VMC_ERR_CUDA;
    int rc = build_sides_d<T, D>(tens, sc, cfg, nullptr, nullptr, 2 * n, nullptr, state, ex, st, keep, row_e);
    if (rc) return rc;
    k_chi_zdot<T><<<(unsigned)((n + 7) / 8), 256, 0, st>>>(state, ex, sc.NS, n, z);
    VMC_CUDA_CHECK_LAUNCH();
    const int per = ChiAdj<T>::ITEMS;
    k_chi_trunc_adj<T, D><<<(unsigned)((2 * n + per - 1) / per), 64 * per, asm_, st>>>(sc, k, cfg, 2 * n, keep,
                                                                                      state, ex, cot);
    VMC_CUDA_CHECK_LAUNCH();
    k_chi_grad_side<T, D><<<(unsigned)(2 * n), CHI_NT, gsm, st>>>((const T*)tens, sc, cfg, 2 * n, keep, row_e, cot,
                                                                  z, O + w0 * ldo, ldo);
    VMC_CUDA_CHECK_LAUNCH();
  }
  return VMC_OK;
}

}  // namespace

extern "C" {

int vmc_peps_chi_work_bytes(int prec, int Lx, int Ly, int D, int chi, int64_t work_rows, int64_t* bytes) {
  ChiSched sc;
  if ((prec != 0 && prec != 1) || work_rows <= 0 || !bytes) return VMC_ERR_ARGS;
  int rc = chi_plan(Lx, Ly, D, chi, sc);
  if (rc) return rc;
  *bytes = prec == 0 ? ChiWork<float>::bytes(sc.NS, work_rows) : ChiWork<double>::bytes(sc.NS, work_rows);
  return VMC_OK;
}

int vmc_peps_chi_schedule(int Lx, int Ly, int D, int chi, uint32_t* cuts, int max_rows) {
  ChiSched sc;
  int rc = chi_plan(Lx, Ly, D, chi, sc);
  if (rc) return rc;
  if (!cuts || max_rows < sc.rows) return VMC_ERR_ARGS;
  for (int a = 0; a < sc.rows; ++a) cuts[a] = sc.cuts[a];
  return VMC_OK;
}

int vmc_peps_chi_eval(int prec, const void* tensors, int Lx, int Ly, int D, int chi, const uint64_t* occ, int64_t R,
                      double* sign, double* logabs, void* work, int64_t work_rows, void* stream) {
  ChiSched sc;
  if (prec != 0 && prec != 1) return VMC_ERR_ARGS;
  int rc = chi_plan(Lx, Ly, D, chi, sc);
  if (rc) return rc;
  if (R < 0 || work_rows <= 0) return VMC_ERR_ARGS;
  if (R == 0) return VMC_OK;
  if (!tensors || !occ || !sign || !logabs || !work) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  return prec == 0 ? chi_eval<float>(tensors, sc, occ, R, sign, logabs, work, work_rows, st)
                   : chi_eval<double>(tensors, sc, occ, R, sign, logabs, work, work_rows, st);
}

int vmc_peps_chi_sweep(int prec, const void* tensors, int Lx, int Ly, int D, int chi, uint64_t* occ, int64_t B,
                       const int32_t* edges, int n_edges, int n_sweeps, float hopping_rate, uint64_t seed,
                       uint64_t sweep_offset, const float* r_move, const uint8_t* r_bit, const float* r_acc,
                       double* sign, double* logabs, int32_t* n_acc, uint64_t* d_n_eval, void* work,
                       int64_t work_rows, void* stream) {
  ChiSched sc;
  if (prec != 0 && prec != 1) return VMC_ERR_ARGS;
  int rc = chi_plan(Lx, Ly, D, chi, sc);
  if (rc) return rc;
  if (B < 0 || n_edges < 0 || n_sweeps < 0 || work_rows <= 0) return VMC_ERR_ARGS;
  if ((r_move != nullptr) != (r_acc != nullptr) || (r_move != nullptr) != (r_bit != nullptr)) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!tensors || !occ || !sign || !logabs || !work || (n_edges > 0 && !edges)) return VMC_ERR_ARGS;
  if (B > INT32_MAX || work_rows > (INT32_MAX / 2)) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long* ne = (unsigned long long*)d_n_eval;
  return prec == 0 ? chi_sweep<float>(tensors, sc, occ, B, edges, n_edges, n_sweeps, hopping_rate, seed,
                                      sweep_offset, r_move, r_bit, r_acc, sign, logabs, n_acc, ne, work, work_rows, st)
                   : chi_sweep<double>(tensors, sc, occ, B, edges, n_edges, n_sweeps, hopping_rate, seed,
                                       sweep_offset, r_move, r_bit, r_acc, sign, logabs, n_acc, ne, work, work_rows,
                                       st);
}

int vmc_peps_chi_local_energy(int prec, const void* tensors, int Lx, int Ly, int D, int chi, const uint64_t* occ,
                              int64_t B, const int32_t* edges, double t, double U, const int32_t* pairs,
                              const int32_t* offs, const int32_t* offs_host, int64_t P, double* term, double* eloc,
                              void* work, int64_t work_rows, void* stream) {
  ChiSched sc;
  if (prec != 0 && prec != 1) return VMC_ERR_ARGS;
  int rc = chi_plan(Lx, Ly, D, chi, sc);
  if (rc) return rc;
  if (B < 0 || P < 0 || work_rows <= 0) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!tensors || !occ || !offs || !offs_host || !eloc || !work || (P > 0 && (!pairs || !edges || !term)))
    return VMC_ERR_ARGS;
  if (offs_host[0] != 0 || offs_host[B] != P || work_rows > (INT32_MAX / 2)) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  return prec == 0 ? chi_local_energy<float>(tensors, sc, occ, B, edges, t, U, pairs, offs, offs_host, term, eloc,
                                             work, work_rows, st)
                   : chi_local_energy<double>(tensors, sc, occ, B, edges, t, U, pairs, offs, offs_host, term, eloc,
                                              work, work_rows, st);
}

int vmc_peps_chi_grad_work_bytes(int prec, int Lx, int Ly, int D, int chi, int64_t work_rows, int64_t* bytes) {
  ChiSched sc;
  if ((prec != 0 && prec != 1) || work_rows <= 0 || !bytes) return VMC_ERR_ARGS;
  int rc = chi_plan(Lx, Ly, D, chi, sc);
  if (rc) return rc;
  if (!chi_grad_cut(sc)) return VMC_ERR_UNSUPPORTED;
  *bytes = prec == 0 ? chi_grad_bytes<float>(sc, work_rows) : chi_grad_bytes<double>(sc, work_rows);
  return VMC_OK;
}

int vmc_peps_chi_logpsi_grad(int prec, const void* tensors, int Lx, int Ly, int D, int chi, const uint64_t* occ,
                             int64_t B, void* O, int64_t ldo, void* work, int64_t work_rows, void* stream) {
  ChiSched sc;
  if (prec != 0 && prec != 1) return VMC_ERR_ARGS;
  int rc = chi_plan(Lx, Ly, D, chi, sc);
  if (rc) return rc;
  const int k = chi_grad_cut(sc);
  if (!k) return VMC_ERR_UNSUPPORTED;
  const int64_t np = (int64_t)Lx * Ly * 4 * D * D * D * D;
  if (B < 0 || ldo < np || work_rows <= 0) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!tensors || !occ || !O || !work) return VMC_ERR_ARGS;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t es = prec == 0 ? sizeof(float) : sizeof(double);
  if (cudaMemset2DAsync(O, (size_t)ldo * es, 0, (size_t)np * es, (size_t)B, st) != cudaSuccess) return VMC_ERR_CUDA;
  if (prec == 0)
    return D == 4 ? chi_logpsi_grad_d<float, 4>(tensors, sc, k, occ, B, (float*)O, ldo, work, work_rows, st)
                  : chi_logpsi_grad_d<float, 2>(tensors, sc, k, occ, B, (float*)O, ldo, work, work_rows, st);
  return D == 4 ? chi_logpsi_grad_d<double, 4>(tensors, sc, k, occ, B, (double*)O, ldo, work, work_rows, st)
                : chi_logpsi_grad_d<double, 2>(tensors, sc, k, occ, B, (double*)O, ldo, work, work_rows, st);
}

}  // extern "C"
