// Products and solves with the nested Nystrom HODLR factor, and the Nystrom matvec.
//
// Replaces the per-block BLAS2 loops of the reference:
//   ldiv!(target, W::FactorHODLR, src) / ldiv!(target, W', src)   baseoverloads.jl:126-150
//   mul!(target, W::FactorHODLR, src) / mul!(target, W', src)     baseoverloads.jl:95-124
//   mul!(target, K::KernelHODLR, src)                             baseoverloads.jl:152-179
// In the nested bases every level's work is r x r per node (see km_factor.cu):
//   W_N^{-1} y :  y_c2 -= Q_c2 (z2 - L22^{-1}(z2 - Ct' z1))
//   W_N^{-T} y :  y_c1 -= Q_c1 Ct L22^{-T} z2 ;  y_c2 -= Q_c2 (z2 - L22^{-T} z2)
//   W_N y      :  y_c2 += Q_c2 (Ct' z1 + (L22 - I) z2)
//   W_N' y     :  y_c1 += Q_c1 Ct z2 ;  y_c2 += Q_c2 (L22' - I) z2
// with z_i = Q_ci' y the projections on the children's orthonormal bases.  Projections travel
// up the tree through the transfer reflectors E_N, corrections travel down through E_N, and
// only the leaves touch n-length data.
//
// Vector workspaces (per column, r doubles per slot): VP projections, VG down-going
// coefficients, VD per-node corrections (2r).  Slot s, column c: (s * k + c) * r.
#include "km_kernels.h"

namespace km {

struct NodeMats {
  const double* Ct;
  const double* L22;
  const double* Eref;
  const double* Etau;
  int r;
};

// x (2r, warp-shared) <- reflectors applied in order j = 0..r-1 (E' x, fwd) or j = r-1..0
// (E x).  Reflector j = [e_j ; Es[:, j]] with tau ts[j]; Es is r x r with leading dim ld.
__device__ __forceinline__ void apply_node_reflectors(const double* Es, const double* ts, int r, int ld,
                                                      double* x, bool fwd) {
  const int lane = threadIdx.x & 31;
  for (int q = 0; q < r; ++q) {
    const int j = fwd ? q : r - 1 - q;
    const double tj = ts[j];
    if (tj == 0.0) continue;
    const double* v = Es + j * ld;
    double acc = 0.0;
    for (int i = lane; i < r; i += 32) acc += v[i] * x[r + i];
    acc = warp_sum(acc);
    acc = (acc + x[j]) * tj;
    __syncwarp();
    if (lane == 0) x[j] -= acc;
    for (int i = lane; i < r; i += 32) x[r + i] -= acc * v[i];
    __syncwarp();
  }
}

// up-sweep modes
enum { UP_PROJ = 0, UP_FWD = 1, UP_MULT = 2, UP_SUM = 3 };
// down-sweep modes
enum { DN_FWD = 0, DN_BWD = 1, DN_MUL = 2, DN_MULT = 3, DN_NYS = 4 };

// Stages the node's Ct, L22, Eref (leading dimension r+1) and tau in shared memory.
__device__ __forceinline__ void stage_node(const NodeMats& nm, int64_t node, double* Cs, double* Ls,
                                           double* Es, double* ts) {
  const int r = nm.r, ld = r + 1;
  const int64_t off = node * (int64_t)r * r;
  for (int e = threadIdx.x; e < r * r; e += blockDim.x) {
    const int i = e % r, c = e / r;
    Cs[i + c * ld] = nm.Ct[off + e];
    Ls[i + c * ld] = nm.L22[off + e];
    Es[i + c * ld] = nm.Eref[off + e];
  }
  for (int e = threadIdx.x; e < r; e += blockDim.x) ts[e] = nm.Etau[node * r + e];
  __syncthreads();
}

// grid = (nodes at level, ceil(k/8)), block 256: one warp per (node, column); the node's
// matrices are shared by the CTA's 8 columns.
__global__ void __launch_bounds__(256) k_up(NodeMats nm, int level, int L, int64_t cslot0, int64_t nslot0,
                                            int64_t node0, double* __restrict__ VP, double* __restrict__ VD,
                                            int k, int mode) {
  extern __shared__ double sm[];
  const int r = nm.r, ld = r + 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int col = blockIdx.y * 8 + w;
  const int64_t kk = blockIdx.x;
  const int64_t node = node0 + kk;
  double* Cs = sm;
  double* Ls = Cs + r * ld;
  double* Es = Ls + r * ld;
  double* ts = Es + r * ld;
  const bool mats = (mode != UP_SUM);
  double* x = (mats ? ts + r : sm) + (size_t)w * 3 * r;  // [0,2r): x   [2r,3r): t
  double* t = x + 2 * r;
  if (mats) stage_node(nm, node, Cs, Ls, Es, ts);
  if (col >= k) return;
  const double* z1 = VP + ((cslot0 + 2 * kk) * k + col) * r;
  const double* z2 = VP + ((cslot0 + 2 * kk + 1) * k + col) * r;
  for (int i = lane; i < r; i += 32) {
    x[i] = z1[i];
    x[r + i] = z2[i];
  }
  __syncwarp();
  if (mode == UP_SUM) {
    if (level < L) {
      double* out = VP + ((nslot0 + kk) * k + col) * r;
      for (int i = lane; i < r; i += 32) out[i] = x[i] + x[r + i];
    }
    return;
  }
  if (mode == UP_FWD) {
    // t = z2 - Ct' z1
    for (int i = lane; i < r; i += 32) {
      const double* ci = Cs + i * ld;
      double acc = 0.0;
#pragma unroll 8
      for (int l = 0; l < r; ++l) acc += ci[l] * x[l];
      t[i] = x[r + i] - acc;
    }
    __syncwarp();
    // w = L22^{-1} t (in t)
    for (int l = 0; l < r; ++l) {
      const double wl = t[l] / Ls[l * ld + l];
      __syncwarp();
      if (lane == 0) t[l] = wl;
      for (int i = l + 1 + lane; i < r; i += 32) t[i] -= Ls[l * ld + i] * wl;
      __syncwarp();
    }
    double* d = VD + (node * k + col) * 2 * r;
    for (int i = lane; i < r; i += 32) {
      d[i] = x[r + i] - t[i];
      x[r + i] = t[i];
    }
    __syncwarp();
  } else if (mode == UP_MULT) {
    // D1 = Ct z2 ; D2 = L22' z2 - z2
    double* d = VD + (node * k + col) * 2 * r;
    for (int i = lane; i < r; i += 32) {
      double a1 = 0.0, a2 = 0.0;
#pragma unroll 8
      for (int l = 0; l < r; ++l) a1 += Cs[i + l * ld] * x[r + l];
      for (int l = i; l < r; ++l) a2 += Ls[l + i * ld] * x[r + l];
      a2 -= x[r + i];
      d[i] = a1;
      d[r + i] = a2;
      t[i] = a2;
      x[i] += a1;
    }
    __syncwarp();
    for (int i = lane; i < r; i += 32) x[r + i] += t[i];
    __syncwarp();
  }
  if (level < L) {
    apply_node_reflectors(Es, ts, r, ld, x, true);
    double* out = VP + ((nslot0 + kk) * k + col) * r;
    for (int i = lane; i < r; i += 32) out[i] = x[i];
  }
}

__global__ void __launch_bounds__(256) k_down(NodeMats nm, int level, int L, int64_t cslot0, int64_t nslot0,
                                              int64_t node0, const double* __restrict__ VP,
                                              double* __restrict__ VG, const double* __restrict__ VD,
                                              int k, int mode) {
  extern __shared__ double sm[];
  const int r = nm.r, ld = r + 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int col = blockIdx.y * 8 + w;
  const int64_t kk = blockIdx.x;
  const int64_t node = node0 + kk;
  const bool top = (level >= L);
  double* Cs = sm;
  double* Ls = Cs + r * ld;
  double* Es = Ls + r * ld;
  double* ts = Es + r * ld;
  const bool mats = (mode != DN_NYS);
  double* x = (mats ? ts + r : sm) + (size_t)w * 4 * r;  // [0,2r): base   [2r,4r): scratch
  double* t = x + 2 * r;
  if (mats) stage_node(nm, node, Cs, Ls, Es, ts);
  if (col >= k) return;
  const double* g = VG + ((nslot0 + kk) * k + col) * r;
  for (int i = lane; i < r; i += 32) {
    x[i] = top ? 0.0 : g[i];
    x[r + i] = 0.0;
  }
  __syncwarp();
  double* g1 = VG + ((cslot0 + 2 * kk) * k + col) * r;
  double* g2 = VG + ((cslot0 + 2 * kk + 1) * k + col) * r;
  const double* p1 = VP + ((cslot0 + 2 * kk) * k + col) * r;
  const double* p2 = VP + ((cslot0 + 2 * kk + 1) * k + col) * r;
  if (mode == DN_NYS) {
    // coefficient sums: child c1 gets parent + phi(c2), child c2 gets parent + phi(c1)
    for (int i = lane; i < r; i += 32) {
      const double b = x[i];
      g1[i] = b + p2[i];
      g2[i] = b + p1[i];
    }
    return;
  }
  if (!top) apply_node_reflectors(Es, ts, r, ld, x, false);
  if (mode == DN_FWD) {
    const double* d = VD + (node * k + col) * 2 * r;
    for (int i = lane; i < r; i += 32) {
      g1[i] = x[i];
      g2[i] = x[r + i] + d[i];
    }
  } else if (mode == DN_MULT) {
    const double* d = VD + (node * k + col) * 2 * r;
    for (int i = lane; i < r; i += 32) {
      g1[i] = x[i] + d[i];
      g2[i] = x[r + i] + d[r + i];
    }
  } else if (mode == DN_BWD) {
    // z2 = p2 - base_bot (kept in t[r..2r)), then t[0..r) = L22^{-T} z2
    for (int i = lane; i < r; i += 32) {
      const double z2 = p2[i] - x[r + i];
      t[r + i] = z2;
      t[i] = z2;
    }
    __syncwarp();
    for (int i = r - 1; i >= 0; --i) {
      const double xi = t[i] / Ls[i * ld + i];
      __syncwarp();
      if (lane == 0) t[i] = xi;
      for (int l = lane; l < i; l += 32) t[l] -= Ls[i + l * ld] * xi;
      __syncwarp();
    }
    for (int i = lane; i < r; i += 32) {
      double acc = 0.0;
#pragma unroll 8
      for (int l = 0; l < r; ++l) acc += Cs[i + l * ld] * t[l];
      g1[i] = x[i] + acc;
      g2[i] = x[r + i] + t[r + i] - t[i];
    }
  } else {  // DN_MUL
    for (int i = lane; i < r; i += 32) {
      t[i] = p1[i] + x[i];
      t[r + i] = p2[i] + x[r + i];
    }
    __syncwarp();
    for (int i = lane; i < r; i += 32) {
      double acc = 0.0;
      const double* ci = Cs + i * ld;
#pragma unroll 8
      for (int l = 0; l < r; ++l) acc += ci[l] * t[l];
      for (int l = 0; l <= i; ++l) acc += Ls[i + l * ld] * t[r + l];
      acc -= t[r + i];
      g1[i] = x[i];
      g2[i] = x[r + i] + acc;
    }
  }
}

// VP[leaf][col] = Phi_leaf' x_leaf  (r values), Phi per leaf column-major m x r.
// grid = (nleaf, ceil(k/8)), block 256, warp per column.
__global__ void __launch_bounds__(256) k_leaf_phiT(const double* __restrict__ Phi, int r, DTree t,
                                                   const double* __restrict__ X, int64_t ldx,
                                                   double* __restrict__ VP, int k) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int col = blockIdx.y * 8 + w;
  if (col >= k) return;
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  double* x = sm + (size_t)w * m;
  const double* src = X + (int64_t)col * ldx + s;
  for (int i = lane; i < m; i += 32) x[i] = src[i];
  __syncwarp();
  const double* P = Phi + s * r;
  double* out = VP + (leaf * k + col) * r;
  for (int c = 0; c < r; ++c) {
    const double* pc = P + (int64_t)c * m;
    double acc = 0.0;
    for (int i = lane; i < m; i += 32) acc += pc[i] * x[i];
    acc = warp_sum(acc);
    if (lane == 0) out[c] = acc;
  }
}

// y_leaf = K_leaf x_leaf + Phi_leaf S^{-1} a_leaf, a_leaf = VG[leaf] (sum of the siblings'
// projections along the path to the root).  This is the leaf product plus the sum over levels
// of U (V' x) and V (U' x) with U = K(rows, P), V = K(cols, P) S^{-1}
// (src/HODLR/src/baseoverloads.jl:158-169, src/factorizations.jl:86-94).
// grid = (nleaf, ceil(k/8)), block 256: x chunk (m x 8) and beta (r x 8) staged in shared.
__global__ void __launch_bounds__(256) k_leaf_nys_apply(const double* __restrict__ Kl, const double* __restrict__ Phi,
                                                        const double* __restrict__ Sc, int r, DTree t,
                                                        const double* __restrict__ X, int64_t ldx,
                                                        const double* __restrict__ VG, double* __restrict__ Y,
                                                        int64_t ldy, int k) {
  extern __shared__ double sm[];
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int c0 = blockIdx.y * 8;
  const int nc = min(8, k - c0);
  double* xs = sm;               // 8 x m
  double* bs = sm + 8 * m;       // 8 x r
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int e = threadIdx.x; e < nc * m; e += blockDim.x) {
    const int c = e / m, i = e % m;
    xs[c * m + i] = X[(int64_t)(c0 + c) * ldx + s + i];
  }
  // beta = S^{-1} a = Sc^{-T} Sc^{-1} a, one warp per column
  if (w < nc) {
    double* b = bs + w * r;
    const double* a = VG + (leaf * k + c0 + w) * r;
    for (int i = lane; i < r; i += 32) b[i] = a[i];
    __syncwarp();
    for (int l = 0; l < r; ++l) {
      const double bl = b[l] / Sc[(int64_t)l * r + l];
      __syncwarp();
      if (lane == 0) b[l] = bl;
      for (int i = l + 1 + lane; i < r; i += 32) b[i] -= Sc[(int64_t)l * r + i] * bl;
      __syncwarp();
    }
    for (int i = r - 1; i >= 0; --i) {
      const double bi = b[i] / Sc[(int64_t)i * r + i];
      __syncwarp();
      if (lane == 0) b[i] = bi;
      for (int l = lane; l < i; l += 32) b[l] -= Sc[i + (int64_t)l * r] * bi;
      __syncwarp();
    }
  }
  __syncthreads();
  const double* K = Kl + d_leaf_koff(t, leaf);
  const double* P = Phi + s * r;
  for (int e = threadIdx.x; e < nc * m; e += blockDim.x) {
    const int c = e / m, i = e % m;
    const double* xc = xs + c * m;
    double acc = 0.0;
    for (int l = 0; l < m; ++l) acc += K[i + (int64_t)l * m] * xc[l];
    const double* bc = bs + c * r;
    for (int q = 0; q < r; ++q) acc += P[i + (int64_t)q * m] * bc[q];
    Y[(int64_t)(c0 + c) * ldy + s + i] = acc;
  }
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
static inline int64_t child_slot0(const Tree& t, int level) {
  return level == 1 ? 0 : t.nleaf + t.node_off[level - 1];
}

void launch_up(const Tree& t, const NodeMatsH& h, int level, double* VP, double* VD, int k, int mode,
               cudaStream_t st) {
  NodeMats nm{h.Ct, h.L22, h.Eref, h.Etau, h.r};
  dim3 grid((unsigned)t.nodes_at(level), (unsigned)((k + 7) / 8));
  const size_t sm = ((mode != UP_SUM_) ? (size_t)3 * h.r * (h.r + 1) + h.r : 0) * sizeof(double) + (size_t)8 * 3 * h.r * sizeof(double);
  cudaFuncSetAttribute(k_up, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_up<<<grid, 256, sm, st>>>(
      nm, level, t.L, child_slot0(t, level), t.nleaf + t.node_off[level], t.node_off[level], VP, VD, k, mode);
}

void launch_down(const Tree& t, const NodeMatsH& h, int level, const double* VP, double* VG,
                 const double* VD, int k, int mode, cudaStream_t st) {
  NodeMats nm{h.Ct, h.L22, h.Eref, h.Etau, h.r};
  dim3 grid((unsigned)t.nodes_at(level), (unsigned)((k + 7) / 8));
  const size_t sm = ((mode != DN_NYS_) ? (size_t)3 * h.r * (h.r + 1) + h.r : 0) * sizeof(double) + (size_t)8 * 4 * h.r * sizeof(double);
  cudaFuncSetAttribute(k_down, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_down<<<grid, 256, sm, st>>>(
      nm, level, t.L, child_slot0(t, level), t.nleaf + t.node_off[level], t.node_off[level], VP, VG, VD, k, mode);
}

void launch_leaf_phiT(const double* Phi, int r, const Tree& t, const double* X, int64_t ldx, double* VP,
                      int k, cudaStream_t st) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 7) / 8));
  const size_t sm = (size_t)8 * t.max_leaf * sizeof(double);
  cudaFuncSetAttribute(k_leaf_phiT, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_leaf_phiT<<<grid, 256, sm, st>>>(Phi, r, dtree(t), X, ldx, VP, k);
}

void launch_leaf_nys_apply(const double* Kl, const double* Phi, const double* Sc, int r, const Tree& t,
                           const double* X, int64_t ldx, const double* VG, double* Y, int64_t ldy, int k,
                           cudaStream_t st) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 7) / 8));
  const size_t sm = (size_t)8 * (t.max_leaf + r) * sizeof(double);
  cudaFuncSetAttribute(k_leaf_nys_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_leaf_nys_apply<<<grid, 256, sm, st>>>(Kl, Phi, Sc, r, dtree(t), X, ldx, VG, Y, ldy, k);
}

}  // namespace km
