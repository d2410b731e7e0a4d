// Slater-determinant walkers: one warp per walker.
//
// Per-walker state (global memory, owned by the caller):
//   occ[2]          packed up / down bits
//   slot_orb[nf]    orbital held by each row slot of A (A[k] = M[slot_orb[k]])
//   G[nf][nf]       G[k][c] = (A^-1)[c][k]  (column k of the inverse, contiguous)
//   sign, logabs    psi(x) = sign * exp(logabs), with psi = det(M[ascending occupied rows])
//   n_acc           accepted moves since the last full re-inversion
//
// The slot order drifts away from the ascending row order as moves are
// accepted; the reordering sign is tracked combinatorially (parity of the
// occupied orbitals passed over) so that sign always refers to the ascending
// (reference) row order.  A full re-inversion resets the slots to ascending
// order.
#include "common.cuh"

using namespace vmc;

namespace {

constexpr int kMaxNf = 64;

struct WarpSmem {
  double* G;      // nf x (nf+1)
  double* tmp;    // 2 x nf
  uint8_t* slot;  // nf
};

__device__ __forceinline__ int gstride(int nf) { return nf + 1; }

// Full re-inversion by Gauss-Jordan with partial pivoting on [A | I] in
// shared memory.  Resets slots to ascending occupied order.  aug: nf x (2nf+1),
// fac: nf.  Writes G (stride nf+1) into g_out.  Returns false if singular or
// non-finite; a non-finite entry (NaN/Inf parameters) gives NaN sign and
// log-amplitude, a singular matrix sign 0 and -inf.
__device__ bool warp_refresh(const double* __restrict__ M, int nf, int N, uint64_t up, uint64_t dn, double* aug,
                             double* fac, double* g_out, uint8_t* slot, double& sign, double& logabs) {
  const int lane = threadIdx.x & 31;
  const int ld = 2 * nf + 1;
  const int gs0 = gstride(nf);
  if (__popcll(up) + __popcll(dn) != nf) {
    // wrong electron count for this orbital matrix: report singular, leave a
    // well-formed (all-zero) state so later kernels never index with garbage
    for (int k = lane; k < nf; k += 32) slot[k] = 0;
    for (int idx = lane; idx < nf * nf; idx += 32) g_out[(idx / nf) * gs0 + idx % nf] = 0.0;
    __syncwarp();
    sign = 0.0;
    logabs = -INFINITY;
    return false;
  }
  // ascending occupied orbitals -> slots
  for (int o = lane; o < 2 * N; o += 32) {
    if (orb_occupied(up, dn, N, o)) {
      int k = orb_prefix(up, dn, N, o);
      if (k < nf) slot[k] = (uint8_t)o;
    }
  }
  __syncwarp();
  for (int idx = lane; idx < nf * 2 * nf; idx += 32) {
    int r = idx / (2 * nf), c = idx - r * 2 * nf;
    aug[r * ld + c] = (c < nf) ? M[(int)slot[r] * nf + c] : (c - nf == r ? 1.0 : 0.0);
  }
  __syncwarp();
  double s = 1.0, la = 0.0;
  bool ok = true, nonfinite = false;
  for (int k = 0; k < nf; ++k) {
    // pivot search over rows >= k (smallest index wins ties; NaN ranks first)
    double best = -1.0;
    int bi = k;
    for (int r = k + lane; r < nf; r += 32) {
      double v = fabs(aug[r * ld + k]);
      if (v != v) v = INFINITY;
      if (v > best) { best = v; bi = r; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double ob = __shfl_xor_sync(VMC_FULL_MASK, best, o);
      int oi = __shfl_xor_sync(VMC_FULL_MASK, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (!(best > 0.0) || !isfinite(best)) {
      nonfinite = !isfinite(best);
      ok = false;
      break;
    }
    if (bi != k) {
      for (int c = lane; c < 2 * nf; c += 32) {
        double t0 = aug[k * ld + c];
        aug[k * ld + c] = aug[bi * ld + c];
        aug[bi * ld + c] = t0;
      }
      s = -s;
      __syncwarp();
    }
    double d = aug[k * ld + k];
    if (d < 0) s = -s;
    la += log(fabs(d));
    __syncwarp();
    double inv = 1.0 / d;
    for (int c = lane; c < 2 * nf; c += 32) aug[k * ld + c] *= inv;
    for (int r = lane; r < nf; r += 32) fac[r] = (r == k) ? 0.0 : aug[r * ld + k];
    __syncwarp();
    for (int idx = lane; idx < nf * 2 * nf; idx += 32) {
      int r = idx / (2 * nf), c = idx - r * 2 * nf;
      if (r != k) aug[r * ld + c] -= fac[r] * aug[k * ld + c];
    }
    __syncwarp();
  }
  const int gs = gstride(nf);
  for (int idx = lane; idx < nf * nf; idx += 32) {
    int k = idx / nf, c = idx - k * nf;
    g_out[k * gs + c] = ok ? aug[c * ld + nf + k] : 0.0;
  }
  __syncwarp();
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  sign = ok ? s : (nonfinite ? qnan : 0.0);
  logabs = ok ? la : (nonfinite ? qnan : -INFINITY);
  return ok;
}

__device__ __forceinline__ double dot_row(const double* __restrict__ Mrow, const double* Grow, int nf) {
  double acc = 0.0;
  for (int c = 0; c < nf; ++c) acc = fma(Mrow[c], Grow[c], acc);
  return acc;
}

__device__ __forceinline__ int find_slot(const uint8_t* slot, int nf, int orb) {
  const int lane = threadIdx.x & 31;
  unsigned b0 = __ballot_sync(VMC_FULL_MASK, lane < nf && slot[lane] == orb);
  if (b0) return __ffs(b0) - 1;
  unsigned b1 = __ballot_sync(VMC_FULL_MASK, lane + 32 < nf && slot[lane + 32] == orb);
  return b1 ? 31 + __ffs(b1) : -1;
}

// ---------------------------------------------------------------------------
__global__ void k_slater_refresh(const double* __restrict__ M, int nf, int N, const uint64_t* __restrict__ occ,
                                 int64_t B, double* __restrict__ G, uint8_t* __restrict__ slot_orb,
                                 double* __restrict__ sign, double* __restrict__ logabs, int32_t* __restrict__ n_acc,
                                 int threshold, int* __restrict__ n_singular) {
  extern __shared__ double sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (w >= B) return;
  if (threshold > 0 && n_acc && n_acc[w] < threshold) return;
  const int per = nf * (2 * nf + 1) + nf + nf * gstride(nf) + 8;
  double* aug = sm + (size_t)warp * per;
  double* fac = aug + nf * (2 * nf + 1);
  double* gs = fac + nf;
  uint8_t* sl = (uint8_t*)(gs + nf * gstride(nf));
  double s, la;
  bool ok = warp_refresh(M, nf, N, occ[2 * w], occ[2 * w + 1], aug, fac, gs, sl, s, la);
  for (int idx = lane; idx < nf * nf; idx += 32) {
    int k = idx / nf, c = idx - k * nf;
    G[w * nf * nf + idx] = gs[k * gstride(nf) + c];
  }
  for (int k = lane; k < nf; k += 32) slot_orb[w * nf + k] = sl[k];
  if (lane == 0) {
    sign[w] = s;
    logabs[w] = la;
    if (n_acc) n_acc[w] = 0;
    if (!ok && s == 0.0 && n_singular) atomicAdd(n_singular, 1);   // singular, not non-finite
  }
}

// ---------------------------------------------------------------------------
__global__ void k_slater_sweep(const double* __restrict__ M, int nf, int N, uint64_t* __restrict__ occ, int64_t B,
                               const int32_t* __restrict__ edges, int E, int n_sweeps, float hopping_rate,
                               uint64_t seed, uint64_t sweep_offset, const float* __restrict__ r_move,
                               const uint8_t* __restrict__ r_bit, const float* __restrict__ r_acc,
                               double* __restrict__ G, uint8_t* __restrict__ slot_orb, double* __restrict__ sign,
                               double* __restrict__ logabs, int32_t* __restrict__ n_acc) {
  extern __shared__ double sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  if (w >= B) return;
  const int gsd = gstride(nf);
  const int per = nf * gsd + 2 * nf + 8;
  double* g = sm + (size_t)warp * per;
  double* tmp = g + nf * gsd;
  uint8_t* sl = (uint8_t*)(tmp + 2 * nf);
  for (int idx = lane; idx < nf * nf; idx += 32) {
    int k = idx / nf, c = idx - k * nf;
    g[k * gsd + c] = G[w * nf * nf + idx];
  }
  for (int k = lane; k < nf; k += 32) sl[k] = slot_orb[w * nf + k];
  __syncwarp();
  uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  double sg = sign[w], la = logabs[w];
  int nacc = n_acc[w];
  const int j0 = lane, j1 = lane + 32;
  for (int s = 0; s < n_sweeps; ++s) {
    for (int e = 0; e < E; ++e) {
      const int i = edges[2 * e], j = edges[2 * e + 1];
      const int xi = site_state(up, dn, i), xj = site_state(up, dn, j);
      if (xi == xj) continue;
      float u_move, u_acc;
      int bit;
      if (r_move) {
        size_t ridx = ((size_t)s * E + e) * (size_t)B + (size_t)w;
        u_move = r_move[ridx]; bit = r_bit[ridx] & 1; u_acc = r_acc[ridx];
      } else {
        EdgeDraw d = draw_edge(seed, (uint64_t)w, sweep_offset + (uint64_t)s, (uint32_t)e);
        u_move = d.u_move; bit = d.bit; u_acc = d.u_acc;
      }
      int ni, nj;
      propose_pair(xi, xj, u_move, bit, hopping_rate, ni, nj);
      Moves mv = pair_moves(i, j, xi, ni, N);
      const int k1 = find_slot(sl, nf, mv.a[0]);
      const int k2 = (mv.n == 2) ? find_slot(sl, nf, mv.a[1]) : -1;
      if (k1 < 0 || (mv.n == 2 && k2 < 0)) continue;  // inconsistent slot table: never index with it
      int par = reorder_parity(up, dn, N, mv.a[0], mv.b[0]);
      uint64_t up1 = up, dn1 = dn;
      apply_move(up1, dn1, N, mv.a[0], mv.b[0]);
      if (mv.n == 2) {
        par ^= reorder_parity(up1, dn1, N, mv.a[1], mv.b[1]);
        apply_move(up1, dn1, N, mv.a[1], mv.b[1]);
      }
      const double* m1 = M + (size_t)mv.b[0] * nf;
      const double* m2 = (mv.n == 2) ? M + (size_t)mv.b[1] * nf : m1;
      double w1a = 0, w1b = 0, w2a = 0, w2b = 0;
      if (j0 < nf) { w1a = dot_row(m1, g + j0 * gsd, nf); if (mv.n == 2) w2a = dot_row(m2, g + j0 * gsd, nf); }
      if (j1 < nf) { w1b = dot_row(m1, g + j1 * gsd, nf); if (mv.n == 2) w2b = dot_row(m2, g + j1 * gsd, nf); }
      // gather R entries from the owning lanes
      auto get = [&](double va, double vb, int k) {
        double a = __shfl_sync(VMC_FULL_MASK, va, k & 31);
        double b = __shfl_sync(VMC_FULL_MASK, vb, k & 31);
        return k < 32 ? a : b;
      };
      double R00 = get(w1a, w1b, k1), R01 = 0, R10 = 0, R11 = 0, r;
      if (mv.n == 2) {
        R01 = get(w1a, w1b, k2);
        R10 = get(w2a, w2b, k1);
        R11 = get(w2a, w2b, k2);
        r = R00 * R11 - R01 * R10;
      } else {
        r = R00;
      }
      const double prob = r * r;
      if (!((double)u_acc < prob)) continue;
      // accept: rank-1 / rank-2 inverse update
      for (int c = lane; c < nf; c += 32) {
        tmp[c] = g[k1 * gsd + c];
        if (mv.n == 2) tmp[nf + c] = g[k2 * gsd + c];
      }
      __syncwarp();
      const double ir = 1.0 / r;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int jj = h ? j1 : j0;
        if (jj >= nf) continue;
        const double v1 = (h ? w1b : w1a) - (jj == k1 ? 1.0 : 0.0);
        double alpha, beta = 0.0;
        if (mv.n == 2) {
          const double v2 = (h ? w2b : w2a) - (jj == k2 ? 1.0 : 0.0);
          alpha = (R11 * v1 - R01 * v2) * ir;
          beta = (-R10 * v1 + R00 * v2) * ir;
        } else {
          alpha = v1 * ir;
        }
        double* row = g + jj * gsd;
        if (mv.n == 2) {
          for (int c = 0; c < nf; ++c) row[c] -= alpha * tmp[c] + beta * tmp[nf + c];
        } else {
          for (int c = 0; c < nf; ++c) row[c] -= alpha * tmp[c];
        }
      }
      __syncwarp();
      if (lane == 0) {
        sl[k1] = (uint8_t)mv.b[0];
        if (mv.n == 2) sl[k2] = (uint8_t)mv.b[1];
      }
      __syncwarp();
      up = up1; dn = dn1;
      sg *= ((r < 0) != (par != 0)) ? -1.0 : 1.0;
      la += log(fabs(r));
      ++nacc;
    }
  }
  for (int idx = lane; idx < nf * nf; idx += 32) {
    int k = idx / nf, c = idx - k * nf;
    G[w * nf * nf + idx] = g[k * gsd + c];
  }
  for (int k = lane; k < nf; k += 32) slot_orb[w * nf + k] = sl[k];
  if (lane == 0) {
    occ[2 * w] = up; occ[2 * w + 1] = dn;
    sign[w] = sg; logabs[w] = la; n_acc[w] = nacc;
  }
}

// ---------------------------------------------------------------------------
// E_loc(x) = U * #doublons + sum_hops (-t) (-1)^{symmray parity} psi(eta)/psi(x),
// with psi(eta)/psi(x) = (-1)^{reorder parity} * M[b] . A^-1[:, slot(a)].
__global__ void k_slater_eloc(const double* __restrict__ M, int nf, int N, const uint64_t* __restrict__ occ,
                              int64_t B, const int32_t* __restrict__ edges, int E, double t, double U,
                              const double* __restrict__ G, const uint8_t* __restrict__ slot_orb,
                              double* __restrict__ eloc) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  __shared__ int8_t orb2slot_all[8][128];
  if (w >= B) return;
  int8_t* o2s = orb2slot_all[warp];
  for (int o = lane; o < 128; o += 32) o2s[o] = -1;
  __syncwarp();
  for (int k = lane; k < nf; k += 32) {
    const int o = slot_orb[w * nf + k];
    if (o < 2 * N) o2s[o] = (int8_t)k;
  }
  __syncwarp();
  const uint64_t up = occ[2 * w], dn = occ[2 * w + 1];
  const double* g = G + (size_t)w * nf * nf;
  double acc = 0.0;
  for (int term = lane; term < 2 * E; term += 32) {
    const int e = term >> 1, s = (term & 1) ? 0 : 1;
    int i = edges[2 * e], j = edges[2 * e + 1];
    if (i > j) { int tt = i; i = j; j = tt; }
    const uint64_t m = s ? up : dn;
    const int oi = (int)((m >> i) & 1ull), oj = (int)((m >> j) & 1ull);
    if (oi == oj) continue;
    const int base = s ? 0 : N;
    const int a = base + (oi ? i : j), b = base + (oi ? j : i);
    const int k = o2s[a];
    if (k < 0) continue;  // inconsistent state (zero amplitude walker)
    double r = dot_row(M + (size_t)b * nf, g + (size_t)k * nf, nf);
    if (reorder_parity(up, dn, N, a, b)) r = -r;
    const double c = symmray_parity(up, dn, i, j, s) ? t : -t;
    acc = fma(c, r, acc);
  }
  acc = warp_sum(acc);
  if (lane == 0) eloc[w] = acc + U * (double)__popcll(up & dn);
}

// O[w][o*nf + c] = G[slot(o)][c] for occupied o, else 0.
__global__ void k_slater_grad(const double* __restrict__ G, const uint8_t* __restrict__ slot_orb, int64_t B,
                              int n_orb, int nf, double* __restrict__ O, int64_t ldo) {
  __shared__ int8_t o2s[128];
  const int64_t w = blockIdx.x;
  for (int o = threadIdx.x; o < 128; o += blockDim.x) o2s[o] = -1;
  __syncthreads();
  for (int k = threadIdx.x; k < nf; k += blockDim.x) {
    const int o = slot_orb[w * nf + k];
    if (o < n_orb) o2s[o] = (int8_t)k;
  }
  __syncthreads();
  const double* g = G + (size_t)w * nf * nf;
  for (int idx = threadIdx.x; idx < n_orb * nf; idx += blockDim.x) {
    const int o = idx / nf, c = idx - o * nf;
    const int k = o2s[o];
    O[w * ldo + idx] = (k >= 0) ? g[k * nf + c] : 0.0;
  }
}

size_t refresh_smem_per_warp(int nf) {
  return ((size_t)nf * (2 * nf + 1) + nf + (size_t)nf * (nf + 1) + 8) * sizeof(double);
}
size_t sweep_smem_per_warp(int nf) { return ((size_t)nf * (nf + 1) + 2 * nf + 8) * sizeof(double); }

int warps_per_block(size_t per_warp) {
  size_t budget = 96 * 1024;
  int wpb = (int)(budget / per_warp);
  if (wpb < 1) wpb = 1;
  if (wpb > 8) wpb = 8;
  return wpb;
}

}  // namespace

extern "C" {

int vmc_slater_refresh(const double* M, int n_orb, int nf, const uint64_t* occ, int64_t B, int n_sites, double* G,
                       uint8_t* slot_orb, double* sign, double* logabs, int32_t* n_acc, int threshold,
                       int* d_n_singular, void* stream) {
  if (B < 0 || nf < 1 || nf > kMaxNf || n_sites < 1 || n_sites > 64 || n_orb != 2 * n_sites) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!M || !occ || !G || !slot_orb || !sign || !logabs) return VMC_ERR_ARGS;
  size_t per = refresh_smem_per_warp(nf);
  int wpb = warps_per_block(per);
  size_t smem = per * wpb;
  cudaFuncSetAttribute(k_slater_refresh, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_slater_refresh<<<(unsigned)((B + wpb - 1) / wpb), 32 * wpb, smem, (cudaStream_t)stream>>>(
      M, nf, n_sites, occ, B, G, slot_orb, sign, logabs, n_acc, threshold, d_n_singular);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_slater_sweep(const double* M, int n_orb, int nf, uint64_t* occ, int64_t B, int n_sites, const int32_t* edges,
                     int n_edges, int n_sweeps, float hopping_rate, uint64_t seed, uint64_t sweep_offset,
                     const float* r_move, const uint8_t* r_bit, const float* r_acc, double* G, uint8_t* slot_orb,
                     double* sign, double* logabs, int32_t* n_acc, void* stream) {
  if (B < 0 || nf < 1 || nf > kMaxNf || n_sites < 1 || n_sites > 64 || n_orb != 2 * n_sites || n_edges < 0 ||
      n_sweeps < 0)
    return VMC_ERR_ARGS;
  if ((r_move != nullptr) != (r_acc != nullptr) || (r_move != nullptr) != (r_bit != nullptr)) return VMC_ERR_ARGS;
  if (B == 0 || n_sweeps == 0 || n_edges == 0) return VMC_OK;
  if (!M || !occ || !edges || !G || !slot_orb || !sign || !logabs || !n_acc) return VMC_ERR_ARGS;
  size_t per = sweep_smem_per_warp(nf);
  int wpb = warps_per_block(per);
  size_t smem = per * wpb;
  cudaFuncSetAttribute(k_slater_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_slater_sweep<<<(unsigned)((B + wpb - 1) / wpb), 32 * wpb, smem, (cudaStream_t)stream>>>(
      M, nf, n_sites, occ, B, edges, n_edges, n_sweeps, hopping_rate, seed, sweep_offset, r_move, r_bit, r_acc, G,
      slot_orb, sign, logabs, n_acc);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_slater_local_energy(const double* M, int n_orb, int nf, const uint64_t* occ, int64_t B, int n_sites,
                            const int32_t* edges, int n_edges, double t, double U, const double* G,
                            const uint8_t* slot_orb, double* eloc, void* stream) {
  if (B < 0 || nf < 1 || nf > kMaxNf || n_sites < 1 || n_sites > 64 || n_orb != 2 * n_sites || n_edges < 0)
    return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!M || !occ || !G || !slot_orb || !eloc || (n_edges > 0 && !edges)) return VMC_ERR_ARGS;
  const int wpb = 8;
  k_slater_eloc<<<(unsigned)((B + wpb - 1) / wpb), 32 * wpb, 0, (cudaStream_t)stream>>>(
      M, nf, n_sites, occ, B, edges, n_edges, t, U, G, slot_orb, eloc);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

int vmc_slater_logpsi_grad(const double* G, const uint8_t* slot_orb, int64_t B, int n_orb, int nf, double* O,
                           int64_t ldo, void* stream) {
  if (B < 0 || nf < 1 || nf > kMaxNf || n_orb < nf || n_orb > 128 || ldo < (int64_t)n_orb * nf) return VMC_ERR_ARGS;
  if (B == 0) return VMC_OK;
  if (!G || !slot_orb || !O) return VMC_ERR_ARGS;
  k_slater_grad<<<(unsigned)B, 128, 0, (cudaStream_t)stream>>>(G, slot_orb, B, n_orb, nf, O, ldo);
  VMC_CUDA_CHECK_LAUNCH();
  return VMC_OK;
}

}  // extern "C"
