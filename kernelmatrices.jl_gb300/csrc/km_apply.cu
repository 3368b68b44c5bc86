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
#include <atomic>
#include <type_traits>

#include "km_kernels.h"

namespace km {

template <typename T>
struct NodeMats {
  const T* Ct;    // r x r
  const T* L22;   // r x r lower
  const T* L22i;  // r x r lower, inverse of L22
  const T* E;     // 2r x r explicit transfer
  int r;
  const T* CtT;   // transposes: a thread per output row reads consecutive addresses across a warp
  const T* L22T;
  const T* L22iT;
  const T* ET;    // r x 2r
};

// up-sweep modes
enum { UP_PROJ = 0, UP_FWD = 1, UP_MULT = 2, UP_SUM = 3 };
// down-sweep modes
enum { DN_FWD = 0, DN_BWD = 1, DN_MUL = 2, DN_MULT = 3 };

// sum_l a[l*sa] b[l], l < n, with four independent partial sums (term l into sum l % 4, the
// tail after the last full group of four into the first).  The node matrices come from L2.  In
// FP64 a sweep phase is bound by the round trips of these loads, so sixteen are issued before
// their terms are summed (about n / 16 round trips instead of n / 4, same order of summation:
// 1.38 -> 1.22 ms of sweeps per C2 step); the float-pair sums ran slower that way (1.15 -> 1.54
// ms), so they keep groups of four (staged launches read the matrices from shared memory).
template <typename T>
__device__ __forceinline__ T dot4(const T* __restrict__ a, int sa, const T* __restrict__ b, int n) {
  T s0 = T(0.0), s1 = T(0.0), s2 = T(0.0), s3 = T(0.0);
  int l = 0;
  if constexpr (std::is_same<T, double>::value) {
    for (; l + 15 < n; l += 16) {
      T av[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) av[u] = a[(int64_t)(l + u) * sa];
#pragma unroll
      for (int u = 0; u < 16; u += 4) {
        s0 += av[u] * b[l + u];
        s1 += av[u + 1] * b[l + u + 1];
        s2 += av[u + 2] * b[l + u + 2];
        s3 += av[u + 3] * b[l + u + 3];
      }
    }
  }
  for (; l + 3 < n; l += 4) {
    s0 += a[(int64_t)l * sa] * b[l];
    s1 += a[(int64_t)(l + 1) * sa] * b[l + 1];
    s2 += a[(int64_t)(l + 2) * sa] * b[l + 2];
    s3 += a[(int64_t)(l + 3) * sa] * b[l + 3];
  }
  for (; l < n; ++l) s0 += a[(int64_t)l * sa] * b[l];
  return (s0 + s1) + (s2 + s3);
}

constexpr int KC = 16;  // most right-hand-side columns per CTA

// Columns per CTA and block size for one level: a level with few nodes spreads its columns over
// more CTAs so that the sweep of the upper levels still covers the SMs (each CTA's dot products
// are one node's r x r products on its kcb columns).
static inline void sweep_shape(int64_t nodes, int k, int* kcb, int* threads) {
  int c = KC;
  while (c > 1 && nodes * ((k + c - 1) / c) < 2 * 152) c >>= 1;
  *kcb = c;
  *threads = c >= 8 ? 512 : (c >= 4 ? 256 : 128);
}

// Staged launches (STAGE): the node matrices a phase reads are copied into shared memory at the
// start of the kernel with asynchronous 8-byte copies (no registers held, all in flight at
// once, overlapped with the vector loads), and the dot products read them from there instead of
// waiting on L2 / DRAM round trips.  Used when the launch's CTAs fit in one wave at one CTA per
// SM (the staged matrices take 4 r^2 values of shared memory); the sums are the same.
template <typename T>
__device__ __forceinline__ void stage_async(T* dst, const T* __restrict__ src, int n, int tid, int nth) {
  static_assert(sizeof(T) == 8, "8-byte elements");
  const unsigned base = (unsigned)__cvta_generic_to_shared(dst);
  for (int e = tid; e < n; e += nth)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(base + 8u * (unsigned)e), "l"(src + e) : "memory");
}
__device__ __forceinline__ void stage_wait() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// grid = (nodes at level, ceil(k / kcb)).  Every phase is a set of independent dot products (one
// thread per output entry) separated by barriers; node matrices are read through the L1 cache,
// or from shared memory in a staged launch.
template <typename T, bool STAGE>
__global__ void __launch_bounds__(512) k_up(NodeMats<T> nm, int level, int L, int64_t cslot0, int64_t nslot0,
                                            int64_t node0, T* __restrict__ VP, T* __restrict__ VD, int k, int mode, int kcb) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* z = reinterpret_cast<T*>(smraw);   // kcb x 2r : [z1 ; z2] per column
  const int r = nm.r, r2 = 2 * r;
  T* tb = z + kcb * r2;                    // kcb x r
  T* ub = tb + kcb * r;                    // kcb x r
  const int64_t kk = blockIdx.x;
  const int64_t node = node0 + kk;
  const int c0 = blockIdx.y * kcb;
  const int kc = min(kcb, k - c0);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int64_t rr = (int64_t)r * r;
  const T* Ct = nm.Ct + node * rr;
  const T* L22i = nm.L22i + node * rr;
  const T* CtT = nm.CtT + node * rr;
  const T* L22T = nm.L22T + node * rr;
  const T* ETn = nm.ET + node * (int64_t)r2 * r;
  if constexpr (STAGE) {
    if (mode != UP_SUM) {
      T* sA = ub + kcb * r;  // r^2: CtT or Ct
      T* sB = sA + rr;       // r^2: L22i or L22T
      T* sE = sB + rr;       // 2 r^2: ET
      if (mode == UP_FWD) {
        stage_async(sA, CtT, r * r, tid, nth);
        stage_async(sB, L22i, r * r, tid, nth);
        CtT = sA;
        L22i = sB;
      } else if (mode == UP_MULT) {
        stage_async(sA, Ct, r * r, tid, nth);
        stage_async(sB, L22T, r * r, tid, nth);
        Ct = sA;
        L22T = sB;
      }
      if (level < L) {
        stage_async(sE, ETn, 2 * r * r, tid, nth);
        ETn = sE;
      }
    }
  }
  for (int e = tid; e < kc * r2; e += nth) {
    const int c = e / r2, i = e % r2;
    const int64_t slot = cslot0 + 2 * kk + (i >= r ? 1 : 0);
    z[c * r2 + i] = VP[(slot * k + c0 + c) * r + (i >= r ? i - r : i)];
  }
  if constexpr (STAGE) stage_wait();
  __syncthreads();
  if (mode == UP_SUM) {
    if (level < L)
      for (int e = tid; e < kc * r; e += nth) {
        const int c = e / r, i = e % r;
        VP[((nslot0 + kk) * k + c0 + c) * r + i] = z[c * r2 + i] + z[c * r2 + r + i];
      }
    return;
  }
  if (mode == UP_FWD) {
    // t = z2 - Ct' z1
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      const T* z1 = z + c * r2;
      tb[c * r + i] = z1[r + i] - dot4(CtT + i, r, z1, r);
    }
    __syncthreads();
    // w = L22^{-1} t
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      ub[c * r + i] = dot4(L22i + i, r, tb + c * r, i + 1);
    }
    __syncthreads();
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      const T w = ub[c * r + i];
      VD[(node * k + c0 + c) * 2 * r + i] = z[c * r2 + r + i] - w;
      z[c * r2 + r + i] = w;
    }
    __syncthreads();
  } else if (mode == UP_MULT) {
    // D1 = Ct z2 ; D2 = L22' z2 - z2
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      const T* z2 = z + c * r2 + r;
      const T a1 = dot4(Ct + i, r, z2, r);
      const T a2 = dot4(L22T + i + (int64_t)i * r, r, z2 + i, r - i) - z2[i];
      tb[c * r + i] = a1;
      ub[c * r + i] = a2;
      VD[(node * k + c0 + c) * 2 * r + i] = a1;
      VD[(node * k + c0 + c) * 2 * r + r + i] = a2;
    }
    __syncthreads();
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      z[c * r2 + i] += tb[c * r + i];
      z[c * r2 + r + i] += ub[c * r + i];
    }
    __syncthreads();
  }
  if (level < L) {
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, q = e % r;
      VP[((nslot0 + kk) * k + c0 + c) * r + q] = dot4(ETn + q, r, z + c * r2, r2);
    }
  }
}

template <typename T, bool STAGE>
__global__ void __launch_bounds__(512) k_down(NodeMats<T> nm, int level, int L, int64_t cslot0, int64_t nslot0,
                                              int64_t node0, const T* __restrict__ VP, T* __restrict__ VG,
                                              const T* __restrict__ VD, int k, int mode, int kcb) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* g = reinterpret_cast<T*>(smraw);   // kcb x r  (parent coefficient)
  const int r = nm.r, r2 = 2 * r;
  T* base = g + kcb * r;                   // kcb x 2r (E g)
  T* tb = base + kcb * r2;                 // kcb x 2r scratch
  const int64_t kk = blockIdx.x;
  const int64_t node = node0 + kk;
  const int c0 = blockIdx.y * kcb;
  const int kc = min(kcb, k - c0);
  const int tid = threadIdx.x, nth = blockDim.x;
  const bool top = (level >= L);
  const int64_t rr = (int64_t)r * r;
  const T* E = nm.E + node * (int64_t)r2 * r;
  const T* Ct = nm.Ct + node * rr;
  const T* L22 = nm.L22 + node * rr;
  const T* CtT = nm.CtT + node * rr;
  const T* L22iT = nm.L22iT + node * rr;
  if constexpr (STAGE) {
    T* sE = tb + kcb * r2;  // 2 r^2: E
    T* sA = sE + 2 * rr;    // r^2: Ct or CtT
    T* sB = sA + rr;        // r^2: L22iT or L22
    if (!top) {
      stage_async(sE, E, 2 * r * r, tid, nth);
      E = sE;
    }
    if (mode == DN_BWD) {
      stage_async(sA, Ct, r * r, tid, nth);
      stage_async(sB, L22iT, r * r, tid, nth);
      Ct = sA;
      L22iT = sB;
    } else if (mode == DN_MUL) {
      stage_async(sA, CtT, r * r, tid, nth);
      stage_async(sB, L22, r * r, tid, nth);
      CtT = sA;
      L22 = sB;
    }
  }
  for (int e = tid; e < kc * r; e += nth) {
    const int c = e / r, i = e % r;
    g[c * r + i] = top ? T(0.0) : VG[((nslot0 + kk) * k + c0 + c) * r + i];
  }
  if constexpr (STAGE) stage_wait();
  __syncthreads();
  auto child = [&](int side, int c, int i) -> int64_t { return ((cslot0 + 2 * kk + side) * k + c0 + c) * r + i; };
  for (int e = tid; e < kc * r2; e += nth) {
    const int c = e / r2, i = e % r2;
    base[c * r2 + i] = top ? T(0.0) : dot4(E + i, r2, g + c * r, r);
  }
  __syncthreads();
  if (mode == DN_FWD || mode == DN_MULT) {
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      const T* d = VD + (node * k + c0 + c) * 2 * r;
      VG[child(0, c, i)] = (mode == DN_MULT) ? base[c * r2 + i] + d[i] : base[c * r2 + i];
      VG[child(1, c, i)] = base[c * r2 + r + i] + d[(mode == DN_MULT ? r : 0) + i];
    }
  } else if (mode == DN_BWD) {
    // z2 = p2 - base_bot ; t = L22^{-T} z2 ; g1 = base_top + Ct t ; g2 = base_bot + z2 - t
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      tb[c * r2 + r + i] = VP[child(1, c, i)] - base[c * r2 + r + i];
    }
    __syncthreads();
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      const T* z2 = tb + c * r2 + r;
      tb[c * r2 + i] = dot4(L22iT + i + (int64_t)i * r, r, z2 + i, r - i);
    }
    __syncthreads();
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      const T* tc = tb + c * r2;
      const T acc = dot4(Ct + i, r, tc, r);
      VG[child(0, c, i)] = base[c * r2 + i] + acc;
      VG[child(1, c, i)] = base[c * r2 + r + i] + tc[r + i] - tc[i];
    }
  } else {  // DN_MUL: z = p + base ; D2 = Ct' z1 + L22 z2 - z2
    for (int e = tid; e < kc * r2; e += nth) {
      const int c = e / r2, i = e % r2;
      tb[c * r2 + i] = VP[child(i >= r ? 1 : 0, c, i % r)] + base[c * r2 + i];
    }
    __syncthreads();
    for (int e = tid; e < kc * r; e += nth) {
      const int c = e / r, i = e % r;
      const T* zc = tb + c * r2;
      const T acc = dot4(CtT + i, r, zc, r) + dot4(L22 + i, r, zc + r, i + 1) - zc[r + i];
      VG[child(0, c, i)] = base[c * r2 + i];
      VG[child(1, c, i)] = base[c * r2 + r + i] + acc;
    }
  }
}


// y_leaf = K_leaf x_leaf + Phi_leaf S^{-1} a_leaf, a_leaf = VG[leaf] (sum of the siblings'
// projections along the path to the root).  This is the leaf product plus the sum over levels
// of U (V' x) and V (U' x) with U = K(rows, P), V = K(cols, P) S^{-1}
// (src/HODLR/src/baseoverloads.jl:158-169, src/factorizations.jl:86-94).
// grid = (nleaf, ceil(k/8)), block 256: x chunk (m x 8) and beta (r x 8) staged in shared.
constexpr int kNaRows = 128, kNaParts = 4;  // k_leaf_nys_apply: rows a pass x parts of each row's sum

__global__ void __launch_bounds__(512) k_leaf_nys_apply(const double* __restrict__ Kl, const double* __restrict__ Phi,
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
  // y_i = sum_l K[i][l] x_l + sum_q Phi[i][q] beta_q for the nc columns: thread (row i of a block
  // of kNaRows, part p of kNaParts) takes the columns l and landmarks q of its part, each loaded
  // entry feeding the nc columns; the parts are added in order through shared memory.
  const double* K = Kl + d_leaf_koff(t, leaf);
  const double* P = Phi + s * r;
  double* red = bs + 8 * r;  // kNaParts x kNaRows x 8
  const int il = threadIdx.x % kNaRows, part = threadIdx.x / kNaRows;
  const int l0 = (int)((int64_t)m * part / kNaParts), l1 = (int)((int64_t)m * (part + 1) / kNaParts);
  const int q0 = r * part / kNaParts, q1 = r * (part + 1) / kNaParts;
  for (int i0 = 0; i0 < m; i0 += kNaRows) {
    const int i = i0 + il;
    double acc[8] = {};
    if (i < m && nc == 1) {  // one column: two independent chains, no idle column slots
      double a1 = 0.0;
      int l = l0;
      for (; l + 1 < l1; l += 2) {
        acc[0] += K[i + (int64_t)l * m] * xs[l];
        a1 += K[i + (int64_t)(l + 1) * m] * xs[l + 1];
      }
      if (l < l1) acc[0] += K[i + (int64_t)l * m] * xs[l];
      for (int q = q0; q < q1; ++q) a1 += P[i + (int64_t)q * m] * bs[q];
      acc[0] += a1;
    } else if (i < m) {
      for (int l = l0; l < l1; ++l) {
        const double kv = K[i + (int64_t)l * m];
#pragma unroll
        for (int c = 0; c < 8; ++c)
          if (c < nc) acc[c] += kv * xs[c * m + l];
      }
      for (int q = q0; q < q1; ++q) {
        const double pv = P[i + (int64_t)q * m];
#pragma unroll
        for (int c = 0; c < 8; ++c)
          if (c < nc) acc[c] += pv * bs[c * r + q];
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) red[(part * kNaRows + il) * 8 + c] = acc[c];
    __syncthreads();
    if (part == 0 && i < m)
      for (int c = 0; c < nc; ++c) {
        double v = red[il * 8 + c];
        for (int u = 1; u < kNaParts; ++u) v += red[(u * kNaRows + il) * 8 + c];
        Y[(int64_t)(c0 + c) * ldy + s + i] = v;
      }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
// Shared memory a staged sweep launch may take (below the 227 KB opt-in limit per CTA; r <= 80
// needs at most 203 KB)
constexpr size_t kStageSmemMax = 220 * 1024;

// SM count of the current device (cached per device); a staged sweep launch has at most this
// many CTAs
static int sweep_sm_count() {
  constexpr int kDevMax = 64;
  static std::atomic<int> nsm_of[kDevMax];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevMax) return 1;
  int v = nsm_of[dev].load();
  if (v == 0) {
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    v = nsm > 0 ? nsm : 1;
    nsm_of[dev].store(v);
  }
  return v;
}

static inline int64_t child_slot0(const Tree& t, int level) {
  return level == 1 ? 0 : t.nleaf + t.node_off[level - 1];
}

template <typename T>
void launch_up(const Tree& t, const NodeMatsH& h, int level, T* VP, T* VD, int k, int mode, cudaStream_t st) {
  NodeMats<T> nm{reinterpret_cast<const T*>(h.Ct),    reinterpret_cast<const T*>(h.L22),
                 reinterpret_cast<const T*>(h.L22i),  reinterpret_cast<const T*>(h.E), h.r,
                 reinterpret_cast<const T*>(h.CtT),   reinterpret_cast<const T*>(h.L22T),
                 reinterpret_cast<const T*>(h.L22iT), reinterpret_cast<const T*>(h.ET)};
  int kcb, nth;
  sweep_shape(t.nodes_at(level), k, &kcb, &nth);
  dim3 grid((unsigned)t.nodes_at(level), (unsigned)((k + kcb - 1) / kcb));
  const size_t sm = (size_t)kcb * 4 * h.r * sizeof(T);
  const size_t sms = sm + (size_t)4 * h.r * h.r * sizeof(T);
  if (mode != UP_SUM && (int64_t)grid.x * grid.y <= sweep_sm_count() && sms <= kStageSmemMax) {
    smem_limit((const void*)k_up<T, true>, sms);
    k_up<T, true><<<grid, nth, sms, st>>>(nm, level, t.L, child_slot0(t, level), t.nleaf + t.node_off[level],
                                          t.node_off[level], VP, VD, k, mode, kcb);
    return;
  }
  smem_limit((const void*)k_up<T, false>, sm);
  k_up<T, false><<<grid, nth, sm, st>>>(nm, level, t.L, child_slot0(t, level), t.nleaf + t.node_off[level],
                                        t.node_off[level], VP, VD, k, mode, kcb);
}

template <typename T>
void launch_down(const Tree& t, const NodeMatsH& h, int level, const T* VP, T* VG, const T* VD, int k, int mode,
                 cudaStream_t st) {
  NodeMats<T> nm{reinterpret_cast<const T*>(h.Ct),    reinterpret_cast<const T*>(h.L22),
                 reinterpret_cast<const T*>(h.L22i),  reinterpret_cast<const T*>(h.E), h.r,
                 reinterpret_cast<const T*>(h.CtT),   reinterpret_cast<const T*>(h.L22T),
                 reinterpret_cast<const T*>(h.L22iT), reinterpret_cast<const T*>(h.ET)};
  int kcb, nth;
  sweep_shape(t.nodes_at(level), k, &kcb, &nth);
  dim3 grid((unsigned)t.nodes_at(level), (unsigned)((k + kcb - 1) / kcb));
  const size_t sm = (size_t)kcb * 5 * h.r * sizeof(T);
  const size_t sms = sm + (size_t)4 * h.r * h.r * sizeof(T);
  if ((int64_t)grid.x * grid.y <= sweep_sm_count() && sms <= kStageSmemMax) {
    smem_limit((const void*)k_down<T, true>, sms);
    k_down<T, true><<<grid, nth, sms, st>>>(nm, level, t.L, child_slot0(t, level), t.nleaf + t.node_off[level],
                                            t.node_off[level], VP, VG, VD, k, mode, kcb);
    return;
  }
  smem_limit((const void*)k_down<T, false>, sm);
  k_down<T, false><<<grid, nth, sm, st>>>(nm, level, t.L, child_slot0(t, level), t.nleaf + t.node_off[level],
                                          t.node_off[level], VP, VG, VD, k, mode, kcb);
}

// VG[(leaf k + c) W + q] = A[c][q] - VP[(leaf k + c) W + q], A = sum over the leaves of VP: the
// landmark coefficients every leaf receives from the off-diagonal blocks of a Nystrom HODLR.
// All its off-diagonal blocks are Phi_rows S^{-1} Phi_cols' with the one landmark set
// (nystrom_uvt, src/factorizations.jl:86-94), so the blocks along a leaf's path to the root
// together hold every other leaf once and the sum of the siblings' projections is the total
// minus the leaf's own: one pass over the leaf slots in place of the up- and down-sweeps of
// the tree.  A is summed in a fixed order (warp w takes the leaves w, w + 8, ..., then the warp
// sums in order).  grid (k, ceil(W / 32)), block 256.
__global__ void k_nys_sums(const double* __restrict__ VP, double* __restrict__ VG, int64_t nleaf, int W, int k) {
  __shared__ double red[8][32];
  const int c = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int q = blockIdx.y * 32 + lane;
  double s = 0.0;
  if (q < W) {
#pragma unroll 4
    for (int64_t l = w; l < nleaf; l += 8) s += VP[(l * k + c) * W + q];
  }
  red[w][lane] = s;
  __syncthreads();
  double tot = 0.0;
#pragma unroll
  for (int u = 0; u < 8; ++u) tot += red[u][lane];
  if (q < W)
    for (int64_t l = w; l < nleaf; l += 8) {
      const int64_t e = (l * k + c) * W + q;
      VG[e] = tot - VP[e];
    }
}

// VP[e] -= VG[e] for e < count: the leaf projections of the backward solve from those of the
// forward solve (see nested_bwd_t).
template <typename T>
__global__ void k_slot_sub(T* __restrict__ VP, const T* __restrict__ VG, int64_t count) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    VP[e] = VP[e] - VG[e];
}

template <typename T>
void launch_slot_sub(T* VP, const T* VG, int64_t count, cudaStream_t st) {
  if (count <= 0) return;
  k_slot_sub<T><<<(unsigned)std::min<int64_t>((count + 255) / 256, 4096), 256, 0, st>>>(VP, VG, count);
}
template void launch_slot_sub<double>(double*, const double*, int64_t, cudaStream_t);
template void launch_slot_sub<ff>(ff*, const ff*, int64_t, cudaStream_t);

void launch_nys_sums(const double* VP, double* VG, int64_t nleaf, int W, int k, cudaStream_t st) {
  k_nys_sums<<<dim3((unsigned)k, (unsigned)((W + 31) / 32)), 256, 0, st>>>(VP, VG, nleaf, W, k);
}

void launch_leaf_nys_apply(const double* Kl, const double* Phi, const double* Sc, int r, const Tree& t,
                           const double* X, int64_t ldx, const double* VG, double* Y, int64_t ldy, int k,
                           cudaStream_t st) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 7) / 8));
  const size_t sm = ((size_t)8 * (t.max_leaf + r) + (size_t)kNaParts * kNaRows * 8) * sizeof(double);
  smem_limit((const void*)k_leaf_nys_apply, sm);
  k_leaf_nys_apply<<<grid, kNaParts * kNaRows, sm, st>>>(Kl, Phi, Sc, r, dtree(t), X, ldx, VG, Y, ldy, k);
}

template void launch_up<double>(const Tree&, const NodeMatsH&, int, double*, double*, int, int, cudaStream_t);
template void launch_up<ff>(const Tree&, const NodeMatsH&, int, ff*, ff*, int, int, cudaStream_t);
template void launch_down<double>(const Tree&, const NodeMatsH&, int, const double*, double*, const double*, int, int,
                                  cudaStream_t);
template void launch_down<ff>(const Tree&, const NodeMatsH&, int, const ff*, ff*, const ff*, int, int, cudaStream_t);

}  // namespace km
