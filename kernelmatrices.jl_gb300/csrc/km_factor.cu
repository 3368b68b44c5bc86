// FP64 factorisation kernels of the nested Nystrom HODLR factorisation.
//
// The reference (src/HODLR/src/symfact.jl:6-49) factors K = W W' with
//   W = L_leaf * W_1 * ... * W_L,  W_N = I + M X M'  (src/HODLR/src/utils.jl:29-35),
// where every W_N is built from the Householder QR of the node's transformed off-diagonal
// panels.  With Nystrom blocks every panel is a row block of the single n x r matrix
// Phi = K(X, P) (or of Phi S^{-1}, S = K(P, P)), and left-multiplication by the earlier factors
// commutes with the right factor S^{-1}.  So after the leaf stage (A = L^{-1} Phi, A_leaf =
// Q_leaf R_leaf) every transformed panel of a node N lies in the span of its children's bases:
//   A[N] = blockdiag(Q_c1, Q_c2) G_N,   G_N = [R_c1 ; L22^{-1}(R_c2 - Ct' R_c1)]   (2r x r)
// with Ct = R_c1 S^{-1} R_c2' and L22 = chol(I - Ct' Ct), and the reference's
// X = chol([I C; C' I]) - I equals [[0,0],[C', L22 - I]] in those bases.  QR(G_N) = E_N R_N
// gives the node basis Q_N = blockdiag(Q_c1, Q_c2) E_N.  Only r x r work is left above the
// leaves; the factor is the reference's up to the rounding freedom of the QR of rank-deficient
// panels.  Orthogonal factors are kept in Householder (LAPACK dgeqrf-style) form.
#include <cooperative_groups.h>

#include <atomic>
#include <cstdlib>
#include <type_traits>

#include "km_kernels.h"

namespace km {

namespace cg = cooperative_groups;

// ---------------------------------------------------------------------------------------------
// Small dense Cholesky (r x r, lower, in place, column-major) for S = K(P, P).  One CTA.
// ---------------------------------------------------------------------------------------------
__global__ void k_chol_small(double* __restrict__ A, int n, int* __restrict__ info) {
  extern __shared__ double s[];  // n x (n+1)
  const int ld = n + 1;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) s[(e % n) + (e / n) * ld] = A[e];
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    const double d = s[j + j * ld];
    if (!(d > 0.0)) {
      if (threadIdx.x == 0 && info[0] == 0) info[0] = j + 1;
      __syncthreads();
      break;
    }
    const double sd = sqrt(d);
    __syncthreads();
    for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) s[i + j * ld] /= sd;
    if (threadIdx.x == 0) s[j + j * ld] = sd;
    __syncthreads();
    // trailing lower triangle update
    const int w = n - j - 1;
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
      const int i = j + 1 + e % w, c = j + 1 + e / w;
      if (i >= c) s[i + c * ld] -= s[i + j * ld] * s[c + j * ld];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, c = e / n;
    A[e] = (i >= c) ? s[i + c * ld] : 0.0;
  }
}

// ---------------------------------------------------------------------------------------------
// Batched leaf Cholesky: Lf_j = chol(K_j) (lower), blocked right-looking, one CTA per leaf.
// The current column panel (rows below the diagonal block) lives in shared memory.
// info[j] = first failing column (1-based) of leaf j, 0 if positive definite.
// ---------------------------------------------------------------------------------------------
template <typename T, int NB, int NT>
__global__ void __launch_bounds__(NT) k_leaf_chol(const double* __restrict__ K, T* __restrict__ Lf,
                                                  DTree t, int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t off = d_leaf_koff(t, leaf);
  const double* A0 = K + off;
  T* A = Lf + off;
  constexpr int LDP = NB + 1;
  T* P = sm;                    // (m) x LDP, row-major panel rows
  T* D = sm + (size_t)m * LDP;  // NB x LDP
  const int tid = threadIdx.x, nth = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nth >> 5;
  for (int64_t e = tid; e < (int64_t)m * m; e += nth) A[e] = from_double<T>(A0[e]);
  __syncthreads();
  int bad = 0;
  for (int k0 = 0; k0 < m; k0 += NB) {
    const int kb = min(NB, m - k0);
    // (1) diagonal block -> shared, unblocked Cholesky
    for (int e = tid; e < kb * kb; e += nth) {
      const int i = e % kb, c = e / kb;
      D[i * LDP + c] = A[(int64_t)(k0 + c) * m + k0 + i];
    }
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
      const T d = D[j * LDP + j];
      const bool ok = d > 0.0;
      if (!ok && bad == 0) bad = k0 + j + 1;
      const T sd = ok ? sqrt(d) : T(1.0);
      __syncthreads();
      for (int i = j + 1 + tid; i < kb; i += nth) D[i * LDP + j] /= sd;
      if (tid == 0) D[j * LDP + j] = sd;
      __syncthreads();
      const int w = kb - j - 1;
      for (int e = tid; e < w * w; e += nth) {
        const int i = j + 1 + e % w, c = j + 1 + e / w;
        if (i >= c) D[i * LDP + c] -= D[i * LDP + j] * D[c * LDP + j];
      }
      __syncthreads();
    }
    for (int e = tid; e < kb * kb; e += nth) {
      const int i = e % kb, c = e / kb;
      if (i >= c) A[(int64_t)(k0 + c) * m + k0 + i] = D[i * LDP + c];
    }
    // (2) panel rows i >= k0+kb: x D' = a  (forward substitution per row)
    const int r0 = k0 + kb, mr = m - r0;
    for (int ii = tid; ii < mr; ii += nth) {
      const int i = r0 + ii;
      T x[NB];
#pragma unroll
      for (int c = 0; c < NB; ++c) {
        if (c < kb) {
          acc_t<T> v = A[(int64_t)(k0 + c) * m + i];
          for (int l = 0; l < c; ++l) v -= x[l] * D[c * LDP + l];
          x[c] = accv(v) / D[c * LDP + c];
        }
      }
#pragma unroll
      for (int c = 0; c < NB; ++c) {
        if (c < kb) {
          P[ii * LDP + c] = x[c];
          A[(int64_t)(k0 + c) * m + i] = x[c];
        }
      }
    }
    __syncthreads();
    // (3) trailing update of the lower triangle: A[i, c] -= sum_l P[i,l] P[c,l]
    for (int cc = warp; cc < mr; cc += nwarp) {
      T pc[NB];
#pragma unroll
      for (int l = 0; l < NB; ++l) pc[l] = (l < kb) ? P[cc * LDP + l] : T(0.0);
      T* col = A + (int64_t)(r0 + cc) * m + r0;
      for (int ii = cc + lane; ii < mr; ii += 32) {
        acc_t<T> acc{};
#pragma unroll
        for (int l = 0; l < NB; ++l) acc += P[ii * LDP + l] * pc[l];
        col[ii] -= accv(acc);
      }
    }
    __syncthreads();
  }
  if (tid == 0) info[leaf] = bad;
}

// ---------------------------------------------------------------------------------------------
// Batched Householder QR of the leaf panels A_j (m_j x r, column-major at start(j)*r), in place:
// reflector vectors below the diagonal (unit leading entry implicit), tau[j*r + c], and
// R_j (r x r column-major, zeros below the diagonal) written to Rout[j*r*r].
// Follows LAPACK dgeqr2/dlarfg: beta = -sign(alpha) ||(alpha, x)||, tau = (beta-alpha)/beta,
// v = x/(alpha-beta); a zero column x gives tau = 0 (H = I).  One CTA per leaf; the panel is
// copied to shared memory when it fits.
// ---------------------------------------------------------------------------------------------
// One CTA per leaf.  With float pairs it has 1024 threads: the panel (up to 200 KB of shared
// memory) admits one CTA per SM, so the CTA takes all the warps the SM can hold to hide the
// latency of the float-pair dot products.  The FP64 kernel is bound by the FP64 pipe and keeps
// 256 threads (and the registers that go with them).
template <typename T>
constexpr int leaf_qr_threads() { return std::is_same<T, double>::value ? 256 : 1024; }

template <typename T, bool SMEM>
__global__ void __launch_bounds__(leaf_qr_threads<T>()) k_leaf_qr(T* __restrict__ Pan, int r, DTree t,
                                                                 T* __restrict__ tau, T* __restrict__ Rout) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  __shared__ T red[32];
  __shared__ T sh_tau;
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  T* G = Pan + s * r;
  T* A = SMEM ? sm : G;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (SMEM) {
    for (int64_t e = tid; e < (int64_t)m * r; e += blockDim.x) sm[e] = G[e];
    __syncthreads();
  }
  const int kmax = min(m, r);
  // Two barriers a column: (1) thread 0 forms reflector j from alpha = a[j][j] and the norm of
  // the rest of column j, which the warp that last updated that column left in sh_sig, while the
  // other threads scale the previous reflector; (2) one warp per column c > j applies H_j with
  // the unscaled vector x = a[j+1:, j] (v = scal x), and the warp of column j + 1 then leaves the
  // norm of its rows below j + 1 for the next step.
  __shared__ T sh_sig, sh_scal;
  if (kmax > 0) {  // norm of column 0 below its first row
    T part = T(0.0);
    for (int i = 1 + tid; i < m; i += blockDim.x) part += A[i] * A[i];
    part = warp_sum_t(part);
    if (lane == 0) red[w] = part;
    __syncthreads();
    if (w == 0) {
      T v = lane < (int)(blockDim.x >> 5) ? red[lane] : T(0.0);
      v = warp_sum_t(v);
      if (lane == 0) sh_sig = v;
    }
  }
  T prev_scal = T(0.0);
  for (int j = 0; j < kmax; ++j) {
    T* aj = A + (int64_t)j * m;
    __syncthreads();
    if (j > 0) {  // the previous reflector's vector, scaled in place (nobody reads it this phase)
      T* ap = A + (int64_t)(j - 1) * m;
      for (int i = j + tid; i < m; i += blockDim.x) ap[i] *= prev_scal;
    }
    if (tid == 0) {
      const T sig = sh_sig;
      const T alpha = aj[j];
      T tj = T(0.0), beta = alpha, scal = T(0.0);
      if (sig != 0.0) {
        const T nrm = sqrt(alpha * alpha + sig);
        beta = alpha >= 0.0 ? -nrm : nrm;
        tj = (beta - alpha) / beta;
        scal = T(1.0) / (alpha - beta);
      }
      aj[j] = beta;
      sh_scal = scal;
      sh_tau = tj;
      tau[leaf * r + j] = tj;
    }
    __syncthreads();
    const T scal = sh_scal, tj = sh_tau;
    prev_scal = scal;
    if (tj != 0.0) {
      // apply H_j = I - tau v v' to columns c > j, v = scal x.  Float pairs (32 warps): a warp
      // takes the columns c and c + nwarps together, two independent dot products and updates in
      // flight; FP64 (8 warps, bound by the FP64 pipe): one column a warp
      constexpr bool kPair = std::is_same<T, ff>::value;
      const int nwarps = (int)(blockDim.x >> 5);
      for (int c = j + 1 + w; c < r; c += (kPair ? 2 : 1) * nwarps) {
        const int c2 = c + nwarps;
        const bool two = kPair && c2 < r;
        T* ac = A + (int64_t)c * m;
        T* ac2 = A + (int64_t)(two ? c2 : c) * m;
        T acc = T(0.0), acc2 = T(0.0);
        for (int i = j + 1 + lane; i < m; i += 32) {
          const T x = aj[i];
          acc += x * ac[i];
          if (two) acc2 += x * ac2[i];
        }
        acc = (warp_sum_t(acc) * scal + ac[j]) * tj;
        if (two) acc2 = (warp_sum_t(acc2) * scal + ac2[j]) * tj;
        if (lane == 0) {
          ac[j] -= acc;
          if (two) ac2[j] -= acc2;
        }
        const T f = acc * scal, f2 = acc2 * scal;
        if (c == j + 1) {  // the next column: its norm below row j + 1 on the way
          T nrm = T(0.0);
          for (int i = j + 1 + lane; i < m; i += 32) {
            const T x = aj[i];
            const T v = ac[i] - f * x;
            ac[i] = v;
            if (i > j + 1) nrm += v * v;
            if (two) ac2[i] -= f2 * x;
          }
          nrm = warp_sum_t(nrm);
          if (lane == 0) sh_sig = nrm;
        } else {
          for (int i = j + 1 + lane; i < m; i += 32) {
            const T x = aj[i];
            ac[i] -= f * x;
            if (two) ac2[i] -= f2 * x;
          }
        }
      }
    } else if (j + 1 < kmax && w == 0) {  // H_j = I: the next column's norm as it stands
      T* an = A + (int64_t)(j + 1) * m;
      T nrm = T(0.0);
      for (int i = j + 2 + lane; i < m; i += 32) nrm += an[i] * an[i];
      nrm = warp_sum_t(nrm);
      if (lane == 0) sh_sig = nrm;
    }
  }
  __syncthreads();
  if (kmax > 0) {  // the last reflector's vector
    T* ap = A + (int64_t)(kmax - 1) * m;
    for (int i = kmax + tid; i < m; i += blockDim.x) ap[i] *= prev_scal;
  }
  __syncthreads();
  for (int j = kmax + tid; j < r; j += blockDim.x) tau[leaf * r + j] = T(0.0);
  for (int e = tid; e < r * r; e += blockDim.x) {
    const int i = e % r, c = e / r;
    Rout[leaf * (int64_t)r * r + e] = (i <= c && i < m) ? A[(int64_t)c * m + i] : T(0.0);
  }
  if (SMEM) {
    __syncthreads();
    for (int64_t e = tid; e < (int64_t)m * r; e += blockDim.x) G[e] = sm[e];
  }
}


// Explicit leaf basis Q = H_0 ... H_{r-1} [I; 0] in place of the reflectors (LAPACK dorg2r).
// Runs on the side stream, overlapped with the node levels (only the solves need Q).
template <typename T, bool SMEM>
__global__ void __launch_bounds__(leaf_qr_threads<T>()) k_leaf_formq(T* __restrict__ Pan, const T* __restrict__ tau,
                                                                     int r, DTree t) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  T* G = Pan + s * r;
  T* A = SMEM ? sm : G;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (SMEM) {
    for (int64_t e = tid; e < (int64_t)m * r; e += blockDim.x) sm[e] = G[e];
  }
  const int kmax = min(m, r);
  __syncthreads();
  // explicit Q = H_0 ... H_{r-1} [I; 0] in place (LAPACK dorg2r)
  for (int j = kmax - 1; j >= 0; --j) {
    T* aj = A + (int64_t)j * m;
    const T tj = tau[leaf * r + j];
    if (j < r - 1) {
      if (tid == 0) aj[j] = T(1.0);
      __syncthreads();
      for (int c = j + 1 + w; c < r; c += (int)(blockDim.x >> 5)) {
        T* ac = A + (int64_t)c * m;
        T acc = T(0.0);
        for (int i = j + lane; i < m; i += 32) acc += aj[i] * ac[i];
        acc = warp_sum_t(acc) * tj;
        for (int i = j + lane; i < m; i += 32) ac[i] -= acc * aj[i];
      }
      __syncthreads();
    }
    for (int i = j + 1 + tid; i < m; i += blockDim.x) aj[i] = -(tj * aj[i]);
    for (int i = tid; i < j; i += blockDim.x) aj[i] = T(0.0);
    if (tid == 0) aj[j] = T(1.0) - tj;
    __syncthreads();
  }
  if (SMEM) {
    __syncthreads();
    for (int64_t e = tid; e < (int64_t)m * r; e += blockDim.x) G[e] = sm[e];
  }
}

// ---------------------------------------------------------------------------------------------
// Node factorisation, one CTA (1024 threads) per node of level l.  Given the children's R factors
// (slots c1, c2) and Sc = chol(S) (lower):
//   T1 = R1 Sc^{-T}, T2 = R2 Sc^{-T}   (upper triangular)
//   Ct = T1 T2'                        (= R1 S^{-1} R2')
//   L22 = chol(I - Ct' Ct)
//   if l < L:  G = [R1 ; L22^{-1}(R2 - Ct' R1)],  Householder QR  G = E R_N  (structured:
//              reflector j is e_j on top plus a dense bottom part, kept in Eref[:, j])
// Outputs per node: Ct, L22 (lower), Eref (r x r), Etau (r), R_N into slot N.
//
// Work mapping: the products are split into (column c, 32-row chunk s) items, one warp per
// item, lane = row, so that no index needs a division by r and the warps stay converged; sums
// use the Dot2 accumulator (km_ff.cuh).  The Cholesky runs in dataflow order over columns (one
// warp per column, shared-memory flags instead of block barriers), L22^{-1} B is then solved by
// blocks of 8 rows with all threads, and the QR is a dataflow pipeline in which each warp owns
// four columns and forms their reflectors itself.
// Shared memory: four r x (r+1) matrices, three r-vectors and r + 1 flags.
//
// Cluster form (csize = 2, 4 or 8 CTAs per node, 1-D thread-block clusters): on levels with fewer
// nodes than SMs the product phases (T1, T2, Ct, H, B) are split by columns over the CTAs of the
// node's cluster, CTA `rank` taking columns rank, rank + csize, ...  Every CTA loads the inputs;
// T1, T2 and Ct are all-gathered by storing each column into every CTA's shared memory
// (distributed shared memory), H and B are stored into CTA 0 only, and cluster barriers separate
// the phases (they also make sure that every CTA has started before the first remote store and
// that no CTA exits while others still write to it).  CTA 0 then runs the Cholesky, the solve,
// the QR and the stores alone; the other CTAs return.  With csize = 1 the kernel is the
// one-CTA form (block barriers, local stores).
// ---------------------------------------------------------------------------------------------
// Iteration bound of a spin wait on a shared-memory flag (a few tens of cycles per iteration:
// well above any legitimate wait inside one node, far below a watchdog).  The spin does not
// sleep: a sleeping waiter wakes too late for the column-to-column handoff.
constexpr int kWaitLimit = 1 << 22;

template <typename T>
__device__ __forceinline__ T sel(bool p, T a) {
  return p ? a : T(0.0);
}

// v into the same shared-memory location as p in every CTA of the cluster (locally if csize = 1)
template <typename T>
__device__ __forceinline__ void put_all(T* p, T v, int csize) {
  if (csize == 1) {
    *p = v;
    return;
  }
  cg::cluster_group cl = cg::this_cluster();
  for (int d = 0; d < csize; ++d) *cl.map_shared_rank(p, (unsigned)d) = v;
}

// v into the same shared-memory location as p in CTA 0 of the cluster (locally if csize = 1)
template <typename T>
__device__ __forceinline__ void put_rank0(T* p, T v, int csize) {
  if (csize == 1) {
    *p = v;
    return;
  }
  *cg::this_cluster().map_shared_rank(p, 0u) = v;
}

// barrier over the cluster (release/acquire for the remote stores), or over the CTA if csize = 1
__device__ __forceinline__ void node_barrier(int csize) {
  if (csize == 1) __syncthreads();
  else cg::this_cluster().sync();
}

template <typename T>
__global__ void __launch_bounds__(1024) k_node_factor(T* __restrict__ R, const T* __restrict__ SinvT,
                                                     int r, int level, int L, int64_t nleaf,
                                                     int64_t cbase, int64_t nbase, T* __restrict__ Ct_out,
                                                     T* __restrict__ L22_out, T* __restrict__ Eref,
                                                     T* __restrict__ Etau, int* __restrict__ info,
                                                     int csize, int wait_limit) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int ld = r + 1;
  // polls of a flag before a wait gives up; wait_limit 0: every wait gives up at its first poll,
  // as if its flag were never set (the test of the timeout path)
  const int lim = wait_limit < 0 ? kWaitLimit : wait_limit;
  T* X0 = sm;
  T* X1 = X0 + r * ld;
  T* X2 = X1 + r * ld;
  T* X3 = X2 + r * ld;
  T* va = X3 + r * ld;  // r values: sqrt(d_j), then the reflector betas
  T* vb = va + r;       // r values: 1 / L22[j][j], then the reflector scales
  T* vc = vb + r;       // r values: the reflector taus
  int* flags = reinterpret_cast<int*>(vc + r);  // r + 1 ints: column published / first bad pivot
  const int64_t k = blockIdx.x / csize;
  const int rank = (int)(blockIdx.x % csize);  // rank in the node's cluster (1-D clusters)
  const int64_t node = nbase + k;  // node index within all nodes (level-major)
  const T* R1 = R + (cbase + 2 * k) * (int64_t)r * r;
  const T* R2 = R + (cbase + 2 * k + 1) * (int64_t)r * r;
  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nth >> 5;
  const int nch = (r + 31) >> 5;   // 32-row chunks per column (r <= 96)
  // product items of this CTA: (column c = rank + csize * lc, 32-row chunk s)
  const int nitems = ((r - rank + csize - 1) / csize) * nch;
  for (int e = tid; e <= r; e += nth) flags[e] = (e < r) ? 0 : r + 1;
  // load: X0 = Sc^{-T} (upper), X1 = R1, X2 = R2   (element (i,c) at i + c*ld)
  for (int c = w; c < r; c += nw)
    for (int i = lane; i < r; i += 32) {
      const int e = i + c * r;
      X0[i + c * ld] = SinvT[e];
      X1[i + c * ld] = R1[e];
      X2[i + c * ld] = R2[e];
    }
  node_barrier(csize);
  // T1 = R1 Sc^{-T} -> X3: T1[i][c] = sum_{l = i..c} R1[i][l] Sinv[l][c]
  for (int q = w; q < nitems; q += nw) {
    const int lc = q / nch, s = q - lc * nch, c = rank + csize * lc, i = 32 * s + lane, ii = min(i, r - 1);
    acc_t<T> a0{}, a1{};
    int l = 32 * s;
    for (; l + 1 <= c; l += 2) {
      a0 += sel(l >= i, X1[ii + l * ld]) * X0[l + c * ld];
      a1 += sel(l + 1 >= i, X1[ii + (l + 1) * ld]) * X0[l + 1 + c * ld];
    }
    if (l <= c) a0 += sel(l >= i, X1[ii + l * ld]) * X0[l + c * ld];
    if (i < r) put_all(X3 + i + c * ld, accv(a0) + accv(a1), csize);
  }
  node_barrier(csize);
  // T2 = R2 Sc^{-T} -> X1
  for (int q = w; q < nitems; q += nw) {
    const int lc = q / nch, s = q - lc * nch, c = rank + csize * lc, i = 32 * s + lane, ii = min(i, r - 1);
    acc_t<T> a0{}, a1{};
    int l = 32 * s;
    for (; l + 1 <= c; l += 2) {
      a0 += sel(l >= i, X2[ii + l * ld]) * X0[l + c * ld];
      a1 += sel(l + 1 >= i, X2[ii + (l + 1) * ld]) * X0[l + 1 + c * ld];
    }
    if (l <= c) a0 += sel(l >= i, X2[ii + l * ld]) * X0[l + c * ld];
    if (i < r) put_all(X1 + i + c * ld, accv(a0) + accv(a1), csize);
  }
  node_barrier(csize);
  // Ct = T1 T2' -> X0: Ct[i][c] = sum_{l >= max(i, c)} T1[i][l] T2[c][l]
  for (int q = w; q < nitems; q += nw) {
    const int lc = q / nch, s = q - lc * nch, c = rank + csize * lc, i = 32 * s + lane, ii = min(i, r - 1);
    acc_t<T> a0{}, a1{};
    int l = max(32 * s, c);
    for (; l + 1 < r; l += 2) {
      a0 += sel(l >= i, X3[ii + l * ld]) * X1[c + l * ld];
      a1 += sel(l + 1 >= i, X3[ii + (l + 1) * ld]) * X1[c + (l + 1) * ld];
    }
    if (l < r) a0 += sel(l >= i, X3[ii + l * ld]) * X1[c + l * ld];
    if (i < r) put_all(X0 + i + c * ld, accv(a0) + accv(a1), csize);
  }
  node_barrier(csize);
  // H = I - Ct' Ct -> X3 of CTA 0 (lower triangle); CTA 0 reloads R1 into X1 for the QR meanwhile
  if (level < L && rank == 0)
    for (int c = w; c < r; c += nw)
      for (int i = lane; i < r; i += 32) X1[i + c * ld] = R1[i + c * r];
  for (int q = w; q < nitems; q += nw) {
    const int lc = q / nch, s = q - lc * nch, c = rank + csize * lc, i = 32 * s + lane, ii = min(i, r - 1);
    if (32 * s + 31 < c) continue;
    acc_t<T> a0{}, a1{};
    int l = 0;
    for (; l + 1 < r; l += 2) {
      a0 += X0[l + ii * ld] * X0[l + c * ld];
      a1 += X0[l + 1 + ii * ld] * X0[l + 1 + c * ld];
    }
    if (l < r) a0 += X0[l + ii * ld] * X0[l + c * ld];
    if (i < r && i >= c) put_rank0(X3 + i + c * ld, (i == c ? T(1.0) : T(0.0)) - (accv(a0) + accv(a1)), csize);
  }
  // B = R2 - Ct' R1 -> X2 of CTA 0 (column c of R1 has entries l <= c; R1 read from global memory)
  if (level < L)
    for (int q = w; q < nitems; q += nw) {
      const int lc = q / nch, s = q - lc * nch, c = rank + csize * lc, i = 32 * s + lane, ii = min(i, r - 1);
      const T* r1 = R1 + (int64_t)c * r;
      acc_t<T> a0{}, a1{};
      int l = 0;
      for (; l + 1 <= c; l += 2) {
        a0 += X0[l + ii * ld] * r1[l];
        a1 += X0[l + 1 + ii * ld] * r1[l + 1];
      }
      if (l <= c) a0 += X0[l + ii * ld] * r1[l];
      if (i < r) put_rank0(X2 + i + c * ld, X2[i + c * ld] - (accv(a0) + accv(a1)), csize);
    }
  node_barrier(csize);
  if (rank != 0) return;  // the rest runs in CTA 0; no CTA touches another's memory after the barrier
  // L22 = chol(H) by columns in dataflow order.  Warp w owns columns w, w + nw, ... and finishes
  // them in increasing order: column c accumulates the contributions of columns k < c as soon as
  // each is published (flag[k] set after its values are in shared memory), then takes its pivot
  // and publishes itself; vc[c] keeps the reciprocal pivot.  No block barrier inside the loop.
  // Waits are bounded; a wait that runs out marks the node with info = -1 (reported as a
  // timeout) and the kernel carries on.
  int bad = 0;
  {
    volatile int* vflag = flags;
    int known = 0;           // columns 0 .. known-1 are published (as seen by this warp)
    bool timed_out = false;  // after one expired wait this warp stops waiting
    for (int c = w; c < r; c += nw) {
      acc_t<T> v[3];
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const int i = 32 * s + lane;
        v[s] = (i >= c && i < r) ? X3[i + c * ld] : T(0.0);
      }
      for (int k = 0; k < c; ++k) {
        if (k >= known && !timed_out) {
          int spins = 0;
          // a warp more than two columns behind the pivot it waits for is off the critical
          // chain: it naps between polls, so that its polls do not take issue slots from the
          // warp that forms the next column
          const bool nap = c - k > 2;
          while (wait_limit == 0 || vflag[k] == 0) {
            if (++spins > lim) {
              if (lane == 0) info[node] = -1;
              timed_out = true;
              break;
            }
            if (nap) __nanosleep(32);
          }
          __threadfence_block();
          known = k + 1;
          while (known < c && vflag[known] != 0) ++known;
          __threadfence_block();
        }
        const T lck = X3[c + k * ld];
#pragma unroll
        for (int s = 0; s < 3; ++s) {
          if (32 * s + 31 < c) continue;
          const int i = 32 * s + lane;
          if (i >= c && i < r) v[s] -= X3[i + k * ld] * lck;
        }
      }
      const int cs = c >> 5;
      const T d = shfl_idx(accv(cs == 0 ? v[0] : (cs == 1 ? v[1] : v[2])), c & 31);
      if (!(d > 0.0) && bad == 0) bad = c + 1;
      const T sd = d > 0.0 ? sqrt(d) : T(1.0);
      const T inv = ff_recip(sd);
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const int i = 32 * s + lane;
        if (i == c) X3[i + c * ld] = sd;
        else if (i > c && i < r) X3[i + c * ld] = accv(v[s]) * inv;
      }
      if (lane == 0) vc[c] = inv;
      __threadfence_block();
      __syncwarp();
      if (lane == 0) vflag[c] = 1;
    }
  }
  __syncthreads();
  // B' = L22^{-1} B (element (i, c) at X2[i + c * ld]) by blocks of 8 rows: the rows of a block
  // take the contributions of all earlier rows (one output per thread, a dot product over the
  // solved rows), then a thread per column solves them with the 8 x 8 diagonal block.
  if (level < L)
    for (int k0 = 0; k0 < r; k0 += 8) {
      const int kb = min(8, r - k0);
      if (k0 > 0) {
        for (int e = tid; e < kb * r; e += nth) {
          const int jj = e % kb, c = e / kb;
          acc_t<T> acc = X2[k0 + jj + c * ld];
          for (int q = 0; q < k0; ++q) acc -= X3[k0 + jj + q * ld] * X2[q + c * ld];
          X2[k0 + jj + c * ld] = accv(acc);
        }
        __syncthreads();
      }
      if (tid < r) {
        T y[8];
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
          if (jj < kb) {
            acc_t<T> acc = X2[k0 + jj + tid * ld];
#pragma unroll
            for (int q = 0; q < jj; ++q) acc -= X3[k0 + jj + (k0 + q) * ld] * y[q];
            y[jj] = accv(acc) * vc[k0 + jj];
            X2[k0 + jj + tid * ld] = y[jj];
          }
        }
      }
      __syncthreads();
    }
  // a warp's first non-positive pivot; the smallest over the warps is written below
  if (lane == 0 && bad) atomicMin(flags + r, bad);
  __syncthreads();
  if (tid == 0 && flags[r] < r + 1 && info[node] == 0) info[node] = flags[r];
  // store Ct and L22
  for (int c = w; c < r; c += nw)
    for (int i = lane; i < r; i += 32) {
      const int64_t e = node * (int64_t)r * r + i + (int64_t)c * r;
      Ct_out[e] = X0[i + c * ld];
      L22_out[e] = (i >= c) ? X3[i + c * ld] : T(0.0);
    }
  if (level >= L) return;
  // structured Householder QR of [X1 (upper r x r) ; X2 (r x r)]: reflector j acts on row j of
  // the top and all r rows of the bottom.  Dataflow over columns: column c belongs to the group
  // of 8 lanes c & 3 of warp c >> 2 (lane q of the group holds bottom rows q, q+8, ..., so a dot
  // product is a 3-level shuffle reduction) and stays in registers.  A warp applies reflectors
  // 0, 1, ... to its four columns as they are published; when the next reflector is formed from
  // one of its own columns it forms it at once and publishes it (the unscaled vector into
  // X2[:, j], beta, scale and tau into va, vb, vc, then flag[j]).  No block barrier inside the
  // loop; three of four handoffs stay inside a warp.  The betas and the scaling of the reflector
  // columns are applied in the output loop.
  for (int e = tid; e < r; e += nth) flags[e] = 0;  // reused: the Cholesky waits ended at the barrier above
  __syncthreads();
  const int gq = lane & 7, grp = lane >> 3;
  const int rpl = (r + 7) >> 3;  // rows per lane (<= 10 for r <= 80)
  auto gsum = [&](T x) {
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) x = x + shfl_xor(x, o);
    return x;
  };
  if (w < ((r + 3) >> 2)) {
    volatile int* vflag = flags;
    const int c0 = 4 * w, cmine = c0 + grp;  // this group's column (may be >= r on the last warp)
    const int clast = min(c0 + 3, r - 1);
    T x[10];
#pragma unroll
    for (int t = 0; t < 10; ++t) {
      const int i = gq + 8 * t;
      x[t] = (t < rpl && i < r && cmine < r) ? X2[i + cmine * ld] : T(0.0);
    }
    bool timed_out = false;
    for (int j = 0; j <= clast; ++j) {
      if (j >= c0) {
        // reflector j from this warp's column j (group j - c0); every group computes its own
        // column's norm alike, the owning group publishes
        acc_t<T> part{};
#pragma unroll
        for (int t = 0; t < 10; ++t) part += x[t] * x[t];
        const T sig = gsum(accv(part));
        const T alpha = X1[j + j * ld];
        T tj = T(0.0), beta = alpha, scal = T(0.0);
        if (sig != 0.0) {
          const T nrm = sqrt(alpha * alpha + sig);
          beta = alpha >= 0.0 ? -nrm : nrm;
          tj = (beta - alpha) * ff_recip(beta);
          scal = ff_recip(alpha - beta);
        }
        if (cmine == j) {
#pragma unroll
          for (int t = 0; t < 10; ++t) {
            const int i = gq + 8 * t;
            if (t < rpl && i < r) X2[i + j * ld] = x[t];
          }
          if (gq == 0) {
            va[j] = beta;
            vb[j] = scal;
            vc[j] = tj;
            Etau[node * (int64_t)r + j] = tj;
          }
        }
        __threadfence_block();
        __syncwarp();
        if (lane == 0) vflag[j] = 1;
      } else if (!timed_out) {
        int spins = 0;
        // only the warp that owns column j + 1 forms the next reflector; the others nap between
        // polls so that their polls do not take issue slots from it
        const bool nap = j + 1 < c0;
        while (wait_limit == 0 || vflag[j] == 0) {
          if (++spins > lim) {
            if (lane == 0) info[node] = -1;
            timed_out = true;
            break;
          }
          if (nap) __nanosleep(32);
        }
        __threadfence_block();
      }
      // apply reflector j to this warp's columns c > j
      if (j < clast) {
        const T tj = vc[j];
        if (tj != 0.0) {
          const T scal = vb[j];
          T v[10];
#pragma unroll
          for (int t = 0; t < 10; ++t) {
            const int i = gq + 8 * t;
            v[t] = (t < rpl && i < r) ? X2[i + j * ld] : T(0.0);
          }
          acc_t<T> dacc{};
#pragma unroll
          for (int t = 0; t < 10; ++t) dacc += v[t] * x[t];
          const bool live = cmine > j && cmine < r;
          const T top = live ? X1[j + cmine * ld] : T(0.0);
          const T acc = (gsum(accv(dacc)) * scal + top) * tj;
          if (live) {
            if (gq == 0) X1[j + cmine * ld] = top - acc;
            const T f = acc * scal;
#pragma unroll
            for (int t = 0; t < 10; ++t) x[t] -= f * v[t];
          }
        }
      }
    }
  }
  __syncthreads();
  T* Rn = R + (nleaf + node) * (int64_t)r * r;
  for (int c = w; c < r; c += nw)
    for (int i = lane; i < r; i += 32) {
      const int64_t e = i + (int64_t)c * r;
      Rn[e] = (i < c) ? X1[i + c * ld] : (i == c ? va[c] : T(0.0));
      Eref[node * (int64_t)r * r + e] = X2[i + c * ld] * vb[c];
    }
}

// FP64 variant: thread per output entry, 256 threads.  The FP64 pipe (2 DFMA/clk/SM) bounds
// this kernel, and with few warps per CTA it keeps that pipe busier than the warp-item mapping
// of k_node_factor.
__global__ void __launch_bounds__(256) k_node_factor_f64(double* __restrict__ R, const double* __restrict__ SinvT,
                                                     int r, int level, int L, int64_t nleaf,
                                                     int64_t cbase, int64_t nbase, double* __restrict__ Ct_out,
                                                     double* __restrict__ L22_out, double* __restrict__ Eref,
                                                     double* __restrict__ Etau, int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double* sm = reinterpret_cast<double*>(smraw);
  __shared__ double red[32];
  __shared__ double sh[2];
  const int ld = r + 1;
  double* X0 = sm;
  double* X1 = X0 + r * ld;
  double* X2 = X1 + r * ld;
  double* X3 = X2 + r * ld;
  const int64_t k = blockIdx.x;
  const int64_t node = nbase + k;  // node index within all nodes (level-major)
  const double* R1 = R + (cbase + 2 * k) * (int64_t)r * r;
  const double* R2 = R + (cbase + 2 * k + 1) * (int64_t)r * r;
  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nth >> 5;
  // load: X0 = Sc^{-T} (upper), X1 = R1, X2 = R2   (element (i,c) at i + c*ld)
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    X0[i + c * ld] = SinvT[e];
    X1[i + c * ld] = R1[e];
    X2[i + c * ld] = R2[e];
  }
  __syncthreads();
  // T1 = R1 Sc^{-T} -> X3 (upper x upper: entries l in [i, c])
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    double acc = double(0.0);
    if (i <= c) {
#pragma unroll 4
      for (int l = i; l <= c; ++l) acc += X1[i + l * ld] * X0[l + c * ld];
    }
    X3[i + c * ld] = acc;
  }
  __syncthreads();
  // T2 = R2 Sc^{-T} -> X1
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    double acc = double(0.0);
    if (i <= c) {
#pragma unroll 4
      for (int l = i; l <= c; ++l) acc += X2[i + l * ld] * X0[l + c * ld];
    }
    X1[i + c * ld] = acc;
  }
  __syncthreads();
  // Ct = T1 T2' -> X0 ; Ct[i][c] = sum_{l >= max(i,c)} T1[i][l] T2[c][l]
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    double acc = double(0.0);
#pragma unroll 4
    for (int l = max(i, c); l < r; ++l) acc += X3[i + l * ld] * X1[c + l * ld];
    X0[i + c * ld] = acc;
  }
  __syncthreads();
  // H = I - Ct' Ct -> X3 (lower triangle)
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    if (i >= c) {
      double acc = double(0.0);
#pragma unroll 4
      for (int l = 0; l < r; ++l) acc += X0[l + i * ld] * X0[l + c * ld];
      X3[i + c * ld] = double(i == c ? 1.0 : 0.0) - acc;
    }
  }
  __syncthreads();
  // L22 = chol(H) in place (lower)
  int bad = 0;
  for (int j = 0; j < r; ++j) {
    const double d = X3[j + j * ld];
    const bool ok = d > 0.0;
    if (!ok && bad == 0) bad = j + 1;
    const double sd = ok ? sqrt(d) : double(1.0);
    __syncthreads();
    for (int i = j + 1 + tid; i < r; i += nth) X3[i + j * ld] /= sd;
    if (tid == 0) X3[j + j * ld] = sd;
    __syncthreads();
    const int wdt = r - j - 1;
    for (int e = tid; e < wdt * wdt; e += nth) {
      const int i = j + 1 + e % wdt, c = j + 1 + e / wdt;
      if (i >= c) X3[i + c * ld] -= X3[i + j * ld] * X3[c + j * ld];
    }
    __syncthreads();
  }
  if (tid == 0 && bad) info[node] = bad;
  // store Ct and L22
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    Ct_out[node * (int64_t)r * r + e] = X0[i + c * ld];
    L22_out[node * (int64_t)r * r + e] = (i >= c) ? X3[i + c * ld] : double(0.0);
  }
  if (level >= L) return;
  __syncthreads();
  // reload R1 -> X1 (X2 still holds R2)
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    X1[i + c * ld] = R1[e];
  }
  __syncthreads();
  // B = R2 - Ct' R1 -> X2 (column c of R1 has entries l <= c)
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    double acc = double(0.0);
#pragma unroll 4
    for (int l = 0; l <= c; ++l) acc += X0[l + i * ld] * X1[l + c * ld];
    X2[i + c * ld] -= acc;
  }
  __syncthreads();
  // B <- L22^{-1} B, row by row with the whole CTA
  for (int i = 0; i < r; ++i) {
    const double inv = double(1.0) / X3[i + i * ld];
    for (int c = tid; c < r; c += nth) X2[i + c * ld] *= inv;
    __syncthreads();
    const int rows = r - i - 1;
    for (int e = tid; e < rows * r; e += nth) {
      const int ii = i + 1 + e % rows, c = e / rows;
      X2[ii + c * ld] -= X3[ii + i * ld] * X2[i + c * ld];
    }
    __syncthreads();
  }
  // structured Householder QR of [X1 (upper r x r) ; X2 (r x r)]:
  // reflector j acts on row j of the top and all r rows of the bottom.
  for (int j = 0; j < r; ++j) {
    double part = double(0.0);
    for (int i = tid; i < r; i += nth) part += X2[i + j * ld] * X2[i + j * ld];
    part = warp_sum_t(part);
    if (lane == 0) red[w] = part;
    __syncthreads();
    if (tid == 0) {
      double sig = double(0.0);
      for (int q = 0; q < nw; ++q) sig += red[q];
      const double alpha = X1[j + j * ld];
      double tj = double(0.0), beta = alpha, scal = double(0.0);
      if (sig != 0.0) {
        const double nrm = sqrt(alpha * alpha + sig);
        beta = alpha >= 0.0 ? -nrm : nrm;
        tj = (beta - alpha) / beta;
        scal = double(1.0) / (alpha - beta);
      }
      X1[j + j * ld] = beta;
      sh[0] = scal;
      sh[1] = tj;
      Etau[node * (int64_t)r + j] = tj;
    }
    __syncthreads();
    const double scal = sh[0], tj = sh[1];
    if (tj != 0.0) {
      // scaled reflector column v = X2[:, j] * scal is formed on the fly; each warp updates
      // whole columns c > j
      for (int c = j + 1 + w; c < r; c += nw) {
        double acc = double(0.0);
        for (int i = lane; i < r; i += 32) acc += X2[i + j * ld] * X2[i + c * ld];
        acc = (warp_sum_t(acc) * scal + X1[j + c * ld]) * tj;
        if (lane == 0) X1[j + c * ld] -= acc;
        const double f = acc * scal;
        for (int i = lane; i < r; i += 32) X2[i + c * ld] -= f * X2[i + j * ld];
      }
    }
    __syncthreads();
    for (int i = tid; i < r; i += nth) X2[i + j * ld] *= scal;
    __syncthreads();
  }
  double* Rn = R + (nleaf + node) * (int64_t)r * r;
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    Rn[e] = (i <= c) ? X1[i + c * ld] : double(0.0);
    Eref[node * (int64_t)r * r + e] = X2[i + c * ld];
  }
}

// Sc^{-T} (upper triangular) from the landmark Cholesky factor Sc (lower): X = Sc^{-1} by forward
// substitution on all r columns at once, one CTA with Sc and the right-hand sides in shared
// memory.  At step l the columns j <= l take x[l][j] = b[l][j] / Sc[l][l], then the rows i > l of
// those columns take b[i][j] -= Sc[i][l] x[l][j].  Every x[i][j] sees the operations of the
// row-by-row substitution of its column in the same order (b = e_j; l = j, ..., i - 1; one
// division), two barriers a row instead of a serial chain of r^2 / 2 steps per thread.
__global__ void k_tri_inv_t(const double* __restrict__ Sc, int r, double* __restrict__ SinvT) {
  extern __shared__ double s[];
  const int ld = r + 1;
  double* L = s;           // Sc, element (i, c) at i + c * ld
  double* B = s + r * ld;  // right-hand sides, then X
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int e = tid; e < r * r; e += nth) {
    const int i = e % r, c = e / r;
    L[i + c * ld] = Sc[e];
    B[i + c * ld] = (i == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int l = 0; l < r; ++l) {
    for (int j = tid; j <= l; j += nth) B[l + j * ld] = B[l + j * ld] / L[l + l * ld];
    __syncthreads();
    const int w = r - 1 - l;
    for (int e = tid; e < w * (l + 1); e += nth) {
      const int i = l + 1 + e % w, j = e / w;
      B[i + j * ld] -= L[i + l * ld] * B[l + j * ld];
    }
    __syncthreads();
  }
  for (int e = tid; e < r * r; e += nth) {
    const int j = e % r, i = e / r;  // SinvT[j + i r] = X[i][j] for i >= j
    SinvT[e] = (i >= j) ? B[i + j * ld] : 0.0;
  }
}

// ---------------------------------------------------------------------------------------------
// log det: 2 sum log diag(L_leaf) + 2 sum log |diag(L22)|, deterministic two-pass reduction.
// ---------------------------------------------------------------------------------------------
template <typename T>
__global__ void k_logdet_partial(const T* __restrict__ Lf, DTree t, const T* __restrict__ L22,
                                 int r, int64_t nnode, double* __restrict__ partial) {
  __shared__ double red[8];
  const int64_t nleafdiag = t.n;
  const int64_t tot = nleafdiag + nnode * r;
  double acc = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    T d;
    if (e < nleafdiag) {
      // leaf containing row e
      const int64_t big = t.rem * (t.m0 + 1);
      const int64_t j = e < big ? e / (t.m0 + 1) : t.rem + (e - big) / t.m0;
      const int64_t i = e - d_leaf_start(t, j);
      const int m = d_leaf_size(t, j);
      d = Lf[d_leaf_koff(t, j) + i * m + i];
    } else {
      const int64_t q = e - nleafdiag;
      const int64_t node = q / r, i = q % r;
      d = L22[node * (int64_t)r * r + i * r + i];
    }
    acc += 2.0 * log(fabs(to_double(d)));
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    partial[blockIdx.x] = s;
  }
}

__global__ void k_sum_partials(const double* __restrict__ partial, int np, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < np; ++q) s += partial[q];
    out[0] = s;
  }
}

void launch_sum_partials(const double* partial, int np, double* out, cudaStream_t st) {
  k_sum_partials<<<1, 32, 0, st>>>(partial, np, out);
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
bool launch_chol_small(double* A, int n, int* info, cudaStream_t st) {
  const size_t sm = (size_t)n * (n + 1) * sizeof(double);
  if (sm > 200 * 1024) return false;
  smem_limit((const void*)k_chol_small, sm);
  k_chol_small<<<1, 256, sm, st>>>(A, n, info);
  return true;
}

template <typename T, int NB>
static void leaf_chol_launch(const double* K, T* Lf, const Tree& t, int* info, cudaStream_t st) {
  constexpr int NT = 256;
  const size_t sm = (size_t)(t.max_leaf + NB) * (NB + 1) * sizeof(T);
  smem_limit((const void*)k_leaf_chol<T, NB, NT>, sm);
  k_leaf_chol<T, NB, NT><<<(unsigned)t.nleaf, NT, sm, st>>>(K, Lf, dtree(t), info);
}

template <typename T>
bool launch_leaf_chol(const double* K, T* Lf, const Tree& t, int* info, cudaStream_t st) {
  const int64_t m = t.max_leaf;
  auto fits = [&](int nb) { return (size_t)(m + nb) * (nb + 1) * sizeof(T) <= 200 * 1024; };
  // float pairs need twice the registers per value: use the 16-wide panel for them
  if (sizeof(T) == sizeof(double) && std::is_same<T, double>::value && fits(32)) {
    leaf_chol_launch<T, 32>(K, Lf, t, info, st);
  } else if (fits(16)) {
    leaf_chol_launch<T, 16>(K, Lf, t, info, st);
  } else if (fits(8)) {
    leaf_chol_launch<T, 8>(K, Lf, t, info, st);
  } else {
    return false;
  }
  return true;
}

template <typename T>
void launch_leaf_qr(T* Pan, int r, const Tree& t, T* tau, T* Rout, cudaStream_t st) {
  const size_t sm = (size_t)t.max_leaf * r * sizeof(T);
  if (sm <= 200 * 1024) {
    smem_limit((const void*)k_leaf_qr<T, true>, sm);
    k_leaf_qr<T, true><<<(unsigned)t.nleaf, leaf_qr_threads<T>(), sm, st>>>(Pan, r, dtree(t), tau, Rout);
  } else {
    k_leaf_qr<T, false><<<(unsigned)t.nleaf, leaf_qr_threads<T>(), 0, st>>>(Pan, r, dtree(t), tau, Rout);
  }
}

void launch_tri_inv_t(const double* Sc, int r, double* SinvT, cudaStream_t st) {
  const size_t sm = (size_t)2 * r * (r + 1) * sizeof(double);
  smem_limit((const void*)k_tri_inv_t, sm);
  k_tri_inv_t<<<1, 512, sm, st>>>(Sc, r, SinvT);
}

// SM count of the current device (cached per device)
static int sm_count() {
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

// CTAs per node of the float-pair node kernel: the largest of 8, 4, 2 with nodes x csize <= the
// SM count and at least one such cluster schedulable (checked once per size and device), else 1.
// max_cs (the handle's setting) and KM_NODE_CLUSTER=1, 2, 4 or 8 cap it (1 gives the one-CTA
// form).
static int node_cluster_size(const void* fn, int64_t nodes, int threads, size_t smem, int max_cs) {
  static const int cap = [] {
    const char* e = std::getenv("KM_NODE_CLUSTER");
    const int v = e ? std::atoi(e) : 8;
    return v >= 8 ? 8 : v >= 4 ? 4 : v >= 2 ? 2 : 1;
  }();
  constexpr int kDevMax = 64;
  // per device and size 1, 2, 4, 8: 0 unknown, 1 schedulable, -1 not (handles on several host
  // threads may ask at once; a repeated query gives the same answer)
  static std::atomic<int> ok[kDevMax][4];
  const int nsm = sm_count();
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevMax) return 1;
  const int top = std::min(cap, max_cs);
  for (int cs = top, lg = top >= 8 ? 3 : top == 4 ? 2 : top == 2 ? 1 : 0; cs > 1; cs >>= 1, --lg) {
    if (nodes * cs > nsm) continue;
    if (ok[dev][lg].load() == 0) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)cs);
      cfg.blockDim = dim3((unsigned)threads);
      cfg.dynamicSmemBytes = smem;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)cs;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nclusters = 0;
      const cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg);
      if (e != cudaSuccess) cudaGetLastError();  // clear the query's error; the size is not used
      ok[dev][lg].store((e == cudaSuccess && nclusters > 0) ? 1 : -1);
    }
    if (ok[dev][lg].load() > 0) return cs;
  }
  return 1;
}

template <typename T>
void launch_node_factor(T* R, const T* SinvT, int r, int level, const Tree& t, T* Ct, T* L22, T* Eref,
                        T* Etau, int* info, cudaStream_t st, int max_cluster, int wait_limit) {
  const int64_t cbase = (level == 1) ? 0 : t.nleaf + t.node_off[level - 1];
  const int64_t nbase = t.node_off[level];
  if constexpr (std::is_same<T, double>::value) {
    const size_t sm = (size_t)4 * r * (r + 1) * sizeof(double);
    smem_limit((const void*)k_node_factor_f64, sm);
    k_node_factor_f64<<<(unsigned)t.nodes_at(level), 256, sm, st>>>(
        reinterpret_cast<double*>(R), reinterpret_cast<const double*>(SinvT), r, level, t.L, t.nleaf, cbase, nbase,
        reinterpret_cast<double*>(Ct), reinterpret_cast<double*>(L22), reinterpret_cast<double*>(Eref),
        reinterpret_cast<double*>(Etau), info);
  } else {
    const size_t sm = ((size_t)4 * r * (r + 1) + 3 * r) * sizeof(T) + (size_t)(r + 1) * sizeof(int);
    smem_limit((const void*)k_node_factor<T>, sm);
    const int64_t nodes = t.nodes_at(level);
    const int cs = node_cluster_size((const void*)k_node_factor<T>, nodes, 1024, sm, max_cluster);
    if (cs > 1) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)(nodes * cs));
      cfg.blockDim = dim3(1024);
      cfg.dynamicSmemBytes = sm;
      cfg.stream = st;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)cs;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      const cudaError_t prior = cudaPeekAtLastError();
      if (cudaLaunchKernelEx(&cfg, k_node_factor<T>, R, SinvT, r, level, t.L, t.nleaf, cbase, nbase, Ct, L22, Eref,
                             Etau, info, cs, wait_limit) == cudaSuccess)
        return;
      // the cluster launch was refused (nothing ran): one CTA per node instead; an error from
      // before this launch stays for the caller
      if (prior == cudaSuccess) cudaGetLastError();
    }
    {
      k_node_factor<T><<<(unsigned)nodes, 1024, sm, st>>>(R, SinvT, r, level, t.L, t.nleaf, cbase, nbase, Ct, L22,
                                                          Eref, Etau, info, 1, wait_limit);
    }
  }
}

template <typename T>
void launch_logdet(const T* Lf, const Tree& t, const T* L22, int r, double* partial, int np, double* out,
                   cudaStream_t st) {
  k_logdet_partial<T><<<np, 256, 0, st>>>(Lf, dtree(t), L22, r, t.nnode, partial);
  k_sum_partials<<<1, 32, 0, st>>>(partial, np, out);
}

// double -> float pair conversion of n values (in place allowed: same 8-byte slots)
__global__ void k_to_ff(const double* __restrict__ in, ff* __restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = ff(in[i]);
}
__global__ void k_from_ff(const ff* __restrict__ in, double* __restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}
void launch_to_ff(const double* in, ff* out, int64_t n, cudaStream_t st) {
  k_to_ff<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(in, out, n);
}
void launch_from_ff(const ff* in, double* out, int64_t n, cudaStream_t st) {
  k_from_ff<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(in, out, n);
}


// Solve operators of the nodes of one level, formed off the critical path (side stream):
// L22^{-1} (lower) and the explicit transfer E = H_0 ... H_{r-1} [I; 0] (2r x r) from the
// reflectors of QR(G_N).  One CTA per node; columns are independent.
// Per node of one level: L22^{-1} (lower) and, below the root, the explicit 2r x r factor E
// of G = E R_N from the structured reflectors.  One warp per column; the column lives in
// registers (row i in lane i % 32, slot i / 32, r <= 96), so the dependent chains need no
// block barriers.  Column c's two chains take r - c and c + 1 steps, r + 1 together, so every
// column costs the same; gridDim.y CTAs share a node's columns (warp w of CTA y takes columns
// y * nw + w, stepping gridDim.y * nw), enough on levels with few nodes for one column per warp.
// Runs on the side stream, overlapped with the next level's node kernel.
template <typename T>
__device__ __forceinline__ T slot_get(const T (&x)[3], int s) {
  return s == 0 ? x[0] : (s == 1 ? x[1] : x[2]);
}

template <typename T>
__global__ void __launch_bounds__(512) k_node_finalize(const T* __restrict__ L22, const T* __restrict__ Ct,
                                                       const T* __restrict__ Eref, const T* __restrict__ Etau, int r,
                                                       int64_t nbase, int with_e, T* __restrict__ L22i,
                                                       T* __restrict__ Eexp, T* __restrict__ CtT,
                                                       T* __restrict__ L22T, T* __restrict__ L22iT,
                                                       T* __restrict__ ET) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int ld = r + 1;
  T* Ls = sm;               // L22
  T* Vs = Ls + r * ld;      // reflector bottoms
  T* Cs = Vs + r * ld;      // Ct
  T* ts = Cs + r * ld;      // tau
  const int64_t node = nbase + blockIdx.x;
  const int64_t off = node * (int64_t)r * r;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  const int c0 = (int)blockIdx.y * nw + w, cstep = (int)gridDim.y * nw;  // this warp's columns
  for (int e = tid; e < r * r; e += blockDim.x) {
    const int i = e % r, c = e / r;
    Ls[i + c * ld] = L22[off + e];
    Cs[i + c * ld] = Ct[off + e];
    if (with_e) Vs[i + c * ld] = Eref[off + e];
  }
  if (with_e)
    for (int e = tid; e < r; e += blockDim.x) ts[e] = Etau[node * (int64_t)r + e];
  __syncthreads();
  // transposes of Ct and L22 for the sweeps (entries split over the node's CTAs)
  for (int e = (int)blockIdx.y * blockDim.x + tid; e < r * r; e += (int)gridDim.y * blockDim.x) {
    const int i = e % r, c = e / r;
    CtT[off + e] = Cs[c + i * ld];
    L22T[off + e] = Ls[c + i * ld];
  }
  // L22^{-1} e_c by forward substitution in column (axpy) order: row i accumulates
  // -L[i,p] x_p for p = c .. i-1 and is then divided by L[i,i]
  for (int c = c0; c < r; c += cstep) {
    T x[3];
#pragma unroll
    for (int s = 0; s < 3; ++s) x[s] = (lane + 32 * s) == c ? T(1.0) : T(0.0);
    for (int p = c; p < r; ++p) {
      const T xp = shfl_idx(slot_get(x, p >> 5), p & 31) / Ls[p + p * ld];
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const int i = lane + 32 * s;
        if (i == p) x[s] = xp;
        else if (i > p && i < r) x[s] -= Ls[i + p * ld] * xp;
      }
    }
    T* out = L22i + off + (int64_t)c * r;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const int i = lane + 32 * s;
      if (i < r) {
        out[i] = x[s];
        L22iT[off + c + (int64_t)i * r] = x[s];
      }
    }
  }
  if (!with_e) return;
  // column c of E: H_c ... H_0 applied in turn (j = c down to 0) to [e_c ; 0]; H_j acts on
  // top row j and the whole bottom, so top row j is final once H_j has acted
  T* Eo = Eexp + node * (int64_t)2 * r * r;
  T* Et = ET + node * (int64_t)2 * r * r;  // r x 2r: element (c, l) at c + l*r
  for (int c = c0; c < r; c += cstep) {
    T* top = Eo + (int64_t)c * 2 * r;
    T* bot = top + r;
    T b[3] = {T(0.0), T(0.0), T(0.0)};
    for (int i = c + 1 + lane; i < r; i += 32) {
      top[i] = T(0.0);
      Et[c + (int64_t)i * r] = T(0.0);
    }
    for (int j = c; j >= 0; --j) {
      const T tj = ts[j];
      const T tjtop = j == c ? T(1.0) : T(0.0);
      if (tj == 0.0) {
        if (lane == 0) {
          top[j] = tjtop;
          Et[c + (int64_t)j * r] = tjtop;
        }
        continue;
      }
      T part = T(0.0);
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const int i = lane + 32 * s;
        if (i < r) part += Vs[i + j * ld] * b[s];
      }
      const T acc = (tjtop + warp_sum_t(part)) * tj;
      if (lane == 0) {
        top[j] = tjtop - acc;
        Et[c + (int64_t)j * r] = tjtop - acc;
      }
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const int i = lane + 32 * s;
        if (i < r) b[s] -= acc * Vs[i + j * ld];
      }
    }
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      const int i = lane + 32 * s;
      if (i < r) {
        bot[i] = b[s];
        Et[c + (int64_t)(r + i) * r] = b[s];
      }
    }
  }
}

template <typename T>
void launch_leaf_formq(T* Pan, const T* tau, int r, const Tree& t, cudaStream_t st) {
  const size_t sm = (size_t)t.max_leaf * r * sizeof(T);
  if (sm <= 200 * 1024) {
    smem_limit((const void*)k_leaf_formq<T, true>, sm);
    k_leaf_formq<T, true><<<(unsigned)t.nleaf, leaf_qr_threads<T>(), sm, st>>>(Pan, tau, r, dtree(t));
  } else {
    k_leaf_formq<T, false><<<(unsigned)t.nleaf, leaf_qr_threads<T>(), 0, st>>>(Pan, tau, r, dtree(t));
  }
}

template <typename T>
void launch_node_finalize(const T* L22, const T* Ct, const T* Eref, const T* Etau, int r, int level, const Tree& t,
                          T* L22i, T* Eexp, T* CtT, T* L22T, T* L22iT, T* ET, cudaStream_t st) {
  const size_t sm = ((size_t)3 * r * (r + 1) + r) * sizeof(T);
  smem_limit((const void*)k_node_finalize<T>, sm);
  // CTAs per node: enough for one column per warp (16 warps per CTA) while nodes x CTAs stays
  // within the SM count; one per node on the wide levels
  const int64_t nodes = t.nodes_at(level);
  const int nsm = sm_count();
  const int per_node = (int)std::max<int64_t>(1, std::min<int64_t>((r + 15) / 16, nsm / std::max<int64_t>(nodes, 1)));
  k_node_finalize<T><<<dim3((unsigned)nodes, (unsigned)per_node), 512, sm, st>>>(
      L22, Ct, Eref, Etau, r, t.node_off[level], level < t.L ? 1 : 0, L22i, Eexp, CtT, L22T, L22iT, ET);
}

template void launch_leaf_formq<double>(double*, const double*, int, const Tree&, cudaStream_t);
template void launch_leaf_formq<ff>(ff*, const ff*, int, const Tree&, cudaStream_t);
template void launch_node_finalize<double>(const double*, const double*, const double*, const double*, int, int,
                                           const Tree&, double*, double*, double*, double*, double*, double*,
                                           cudaStream_t);
template void launch_node_finalize<ff>(const ff*, const ff*, const ff*, const ff*, int, int, const Tree&, ff*, ff*,
                                       ff*, ff*, ff*, ff*, cudaStream_t);

template bool launch_leaf_chol<double>(const double*, double*, const Tree&, int*, cudaStream_t);
template bool launch_leaf_chol<ff>(const double*, ff*, const Tree&, int*, cudaStream_t);
template void launch_leaf_qr<double>(double*, int, const Tree&, double*, double*, cudaStream_t);
template void launch_leaf_qr<ff>(ff*, int, const Tree&, ff*, ff*, cudaStream_t);
template void launch_node_factor<double>(double*, const double*, int, int, const Tree&, double*, double*, double*,
                                         double*, int*, cudaStream_t, int, int);
template void launch_node_factor<ff>(ff*, const ff*, int, int, const Tree&, ff*, ff*, ff*, ff*, int*, cudaStream_t,
                                     int, int);
template void launch_logdet<double>(const double*, const Tree&, const double*, int, double*, int, double*, cudaStream_t);
template void launch_logdet<ff>(const ff*, const Tree&, const ff*, int, double*, int, double*, cudaStream_t);

}  // namespace km
