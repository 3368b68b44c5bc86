// ACA assembly and the general (per-block basis) HODLR factorisation used for ACA blocks.
//
// ACA: one CTA per off-diagonal block runs the partially pivoted adaptive cross approximation of
// the reference (src/factorizations.jl:9-84) step for step: the start-row search, the pivot
// rule of restrictedmaxabs (src/utils.jl:2-15: first strict maximum of |x| outside the used set,
// the first unused index when nothing is non-zero), residual updates as a multiply followed by a
// subtract (Julia's `tmprow .-= U[j][mi]*V[j]` is not fused), the Frobenius-norm estimate update
// and the stopping rule norm(row)*norm(col) > rtol*sqrt(znorm2).  Kernel rows and columns are
// evaluated on the fly; U and V are written into per-block panels (column-major).
//
// General factorisation (src/HODLR/src/symfact.jl:6-49 without the Nystrom nesting): leaf
// Cholesky, leaf triangular solves of every panel, then per level the Householder QR of the
// node's V (rows c1) and U (rows c2) panels with explicit Q, C = R1 R2', L22 = chol(I - C'C),
// and the application of W_N^{-1} to the coarser panels.  In the QR bases W_N^{-1} only changes
// the c2 rows:  y_c2 -= Q2 (z2 - L22^{-1}(z2 - C' z1)),  z1 = Q1' y_c1, z2 = Q2' y_c2.
#include <climits>


#include "km_kernels.h"

namespace km {

// ---------------------------------------------------------------------------------------------
// CTA-wide reductions (deterministic order)
// ---------------------------------------------------------------------------------------------
__device__ double cta_sum(double v, double* sred) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  if (lane == 0) sred[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = (lane < nw) ? sred[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) sred[32] = t;
  }
  __syncthreads();
  const double t = sred[32];
  __syncthreads();
  return t;
}

// restrictedmaxabs over x[0..n) with excluded flags: returns (value, index).
__device__ void cta_restricted_argmax(const double* x, const uint8_t* excl, int64_t n, double* sval,
                                     long long* sidx, double* out_val, int64_t* out_idx) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double best = 0.0;
  long long bi = LLONG_MAX, first = LLONG_MAX;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    if (excl[i]) continue;
    if (first == LLONG_MAX) first = i;
    const double a = fabs(x[i]);
    if (a > best) {
      best = a;
      bi = i;
    }
  }
  // reduce: larger |x| wins, ties go to the smaller index; first = min over threads
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
    const long long of = __shfl_xor_sync(0xffffffffu, first, o);
    if (ob > best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
    first = min(first, of);
  }
  if (lane == 0) {
    sval[w] = best;
    sidx[w] = bi;
    sidx[32 + w] = first;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    long long ib = LLONG_MAX, f = LLONG_MAX;
    for (int q = 0; q < nw; ++q) {
      if (sval[q] > b || (sval[q] == b && sidx[q] < ib)) {
        b = sval[q];
        ib = sidx[q];
      }
      f = min(f, sidx[32 + q]);
    }
    if (b > 0.0) {
      sval[32] = x[ib];
      sidx[64] = ib;
    } else {
      sval[32] = 0.0;
      sidx[64] = (f == LLONG_MAX) ? n - 1 : f;
    }
  }
  __syncthreads();
  *out_val = sval[32];
  *out_idx = sidx[64];
  __syncthreads();
}

// ---------------------------------------------------------------------------------------------
// ACA, one CTA (1024 threads) per block.  status: 0 ok, 1 "Incompatible maxrank or matrix
// dimensions." (factorizations.jl:30), 2 rank capacity of the panel reached before convergence.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_aca(const double* __restrict__ pts, KParams kp,
                                              const AcaBlock* __restrict__ blocks, double* __restrict__ P,
                                              uint8_t* __restrict__ F, int* __restrict__ piv, double rtol,
                                              int* __restrict__ rank_out, int* __restrict__ status, int only) {
  extern __shared__ double dsm[];  // 2 * cap: dots with previous columns
  __shared__ double sred[40];
  __shared__ double sval[40];
  __shared__ long long sidx[72];
  const int bid = only >= 0 ? only : (int)blockIdx.x;
  const AcaBlock B = blocks[bid];
  if (only < 0 && B.grid) return;  // compressed by k_aca_grid
  const int64_t nro = B.nro, ncl = B.ncl;
  double* U = P + B.offU;
  double* V = P + B.offV;
  uint8_t* urow = F + B.offFlag;
  uint8_t* ucol = urow + nro;
  int* prow = piv + 2 * B.offPiv;
  int* pcol = prow + B.cap;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  const double* xr = pts + 2 * B.row0;
  const double* xc = pts + 2 * B.col0;
  for (int64_t i = tid; i < nro; i += blockDim.x) urow[i] = 0;
  for (int64_t i = tid; i < ncl; i += blockDim.x) ucol[i] = 0;
  const int maxsz = B.maxsz;
  auto eval_row = [&](int64_t i, double* out) {
    const double px = xr[2 * i], py = xr[2 * i + 1];
    for (int64_t c = tid; c < ncl; c += blockDim.x) out[c] = kernel_value(kp, px, py, xc[2 * c], xc[2 * c + 1]);
  };
  auto eval_col = [&](int64_t j, double* out) {
    const double px = xc[2 * j], py = xc[2 * j + 1];
    for (int64_t i = tid; i < nro; i += blockDim.x) out[i] = kernel_value(kp, xr[2 * i], xr[2 * i + 1], px, py);
  };
  auto sumsq = [&](const double* x, int64_t n) {
    double a = 0.0;
    for (int64_t i = tid; i < n; i += blockDim.x) a += x[i] * x[i];
    return cta_sum(a, sred);
  };
  // first row (factorizations.jl:24-30)
  int64_t strt = 0;
  eval_row(strt, V);
  __syncthreads();
  {
    double mx = 0.0;
    for (int64_t c = tid; c < ncl; c += blockDim.x) mx = fmax(mx, fabs(V[c]));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) sred[w] = mx;
    __syncthreads();
    if (tid == 0) {
      double m = 0.0;
      for (int q = 0; q < nw; ++q) m = fmax(m, sred[q]);
      sred[34] = m;
    }
    __syncthreads();
    mx = sred[34];
    __syncthreads();
    while (mx == 0.0 && strt + 1 < maxsz) {
      ++strt;
      eval_row(strt, V);
      __syncthreads();
      double m2 = 0.0;
      for (int64_t c = tid; c < ncl; c += blockDim.x) m2 = fmax(m2, fabs(V[c]));
      for (int o = 16; o > 0; o >>= 1) m2 = fmax(m2, __shfl_xor_sync(0xffffffffu, m2, o));
      if (lane == 0) sred[w] = m2;
      __syncthreads();
      if (tid == 0) {
        double m = 0.0;
        for (int q = 0; q < nw; ++q) m = fmax(m, sred[q]);
        sred[34] = m;
      }
      __syncthreads();
      mx = sred[34];
      __syncthreads();
    }
  }
  if (strt + 1 == maxsz) {
    if (tid == 0) {
      status[bid] = 1;
      rank_out[bid] = 0;
    }
    return;
  }
  if (tid == 0) {
    urow[strt] = 1;
    prow[0] = (int)strt;
  }
  __syncthreads();
  double mv;
  int64_t mi;
  cta_restricted_argmax(V, ucol, ncl, sval, sidx, &mv, &mi);
  for (int64_t c = tid; c < ncl; c += blockDim.x) V[c] = __ddiv_rn(V[c], mv);
  eval_col(mi, U);
  __syncthreads();
  double sr = sumsq(V, ncl), sc = sumsq(U, nro);
  double znorm2 = __dmul_rn(sr, sc);
  if (tid == 0) {
    ucol[mi] = 1;
    pcol[0] = (int)mi;
  }
  __syncthreads();
  int frnk = 1;
  int st = 0;
  while (__dmul_rn(sqrt(sr), sqrt(sc)) > __dmul_rn(rtol, sqrt(znorm2)) && frnk < maxsz) {
    const double* lastcol = U + (int64_t)(frnk - 1) * nro;
    int64_t ri;
    double rv;
    cta_restricted_argmax(lastcol, urow, nro, sval, sidx, &rv, &ri);
    if (tid == 0) urow[ri] = 1;
    if (frnk >= B.cap) {
      st = 2;
      break;
    }
    double* row = V + (int64_t)frnk * ncl;
    {
      const double px = xr[2 * ri], py = xr[2 * ri + 1];
      for (int64_t c = tid; c < ncl; c += blockDim.x) {
        double v = kernel_value(kp, px, py, xc[2 * c], xc[2 * c + 1]);
        for (int j = 0; j < frnk; ++j) v = __dsub_rn(v, __dmul_rn(U[ri + (int64_t)j * nro], V[c + (int64_t)j * ncl]));
        row[c] = v;
      }
    }
    __syncthreads();
    double cv;
    int64_t cj;
    cta_restricted_argmax(row, ucol, ncl, sval, sidx, &cv, &cj);
    if (cv == 0.0) break;
    if (tid == 0) ucol[cj] = 1;
    for (int64_t c = tid; c < ncl; c += blockDim.x) row[c] = __ddiv_rn(row[c], cv);
    double* col = U + (int64_t)frnk * nro;
    {
      const double px = xc[2 * cj], py = xc[2 * cj + 1];
      for (int64_t i = tid; i < nro; i += blockDim.x) {
        double v = kernel_value(kp, xr[2 * i], xr[2 * i + 1], px, py);
        for (int j = 0; j < frnk; ++j) v = __dsub_rn(v, __dmul_rn(V[cj + (int64_t)j * ncl], U[i + (int64_t)j * nro]));
        col[i] = v;
      }
    }
    __syncthreads();
    // dots with the previous columns, one warp per j
    for (int j = w; j < frnk; j += nw) {
      const double* uj = U + (int64_t)j * nro;
      const double* vj = V + (int64_t)j * ncl;
      double a = 0.0, b = 0.0;
      for (int64_t i = lane; i < nro; i += 32) a += uj[i] * col[i];
      for (int64_t c = lane; c < ncl; c += 32) b += vj[c] * row[c];
      a = warp_sum(a);
      b = warp_sum(b);
      if (lane == 0) {
        dsm[j] = a;
        dsm[B.cap + j] = b;
      }
    }
    __syncthreads();
    if (tid == 0) {
      double z = znorm2;
      for (int j = 0; j < frnk; ++j) z = __dadd_rn(z, __dmul_rn(__dmul_rn(2.0, fabs(dsm[j])), fabs(dsm[B.cap + j])));
      sred[36] = z;
      prow[frnk] = (int)ri;
      pcol[frnk] = (int)cj;
    }
    __syncthreads();
    znorm2 = sred[36];
    __syncthreads();
    sr = sumsq(row, ncl);
    sc = sumsq(col, nro);
    znorm2 = __dadd_rn(znorm2, __dmul_rn(sr, sc));
    ++frnk;
  }
  if (tid == 0) {
    rank_out[bid] = frnk;
    status[bid] = st;
  }
}

// ---------------------------------------------------------------------------------------------
// Householder QR with explicit Q of one panel per CTA, blocked (LAPACK dgeqrf / dorgqr
// structure: reflectors of kQB columns are formed by the unblocked dgeqr2 / dlarfg rules and
// applied to the rest of the panel as one compact-WY block reflector I - V T V').  The trailing
// columns are then read and written once per block instead of once per reflector.  V is staged
// in shared memory kQC rows at a time; trailing columns are processed kQT at a time.
// ---------------------------------------------------------------------------------------------
constexpr int kQB = 8;
constexpr int kQC = 256;
constexpr int kQT = 256;
constexpr int kQV = kQB + 1;  // row stride of the staged V chunk (conflict-free column reads)

// T (kQB x kQB, upper, column-major) of the block reflector of columns j0 .. j0+jb-1:
//   T[q][q] = tau_q,  T[0:q, q] = -tau_q T[0:q, 0:q] (V[:, 0:q]' v_q)
// with v_p = e_p + A[p+1:, p] (zero above row p).  G holds the dots v_p . v_q.
__device__ void panel_block_T(const double* A, int64_t m, int64_t lda, int j0, int jb, const double* tau,
                              double* G, double* Tm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int pq = w; pq < jb * jb; pq += nw) {
    const int p = pq % jb, q = pq / jb;
    if (p >= q) continue;
    const double* vp = A + (int64_t)(j0 + p) * lda;
    const double* vq = A + (int64_t)(j0 + q) * lda;
    // v_p[j0+q] * 1 + sum_{i > j0+q} v_p[i] v_q[i]
    double acc = 0.0;
    for (int64_t i = j0 + q + 1 + lane; i < m; i += 32) acc += vp[i] * vq[i];
    acc = warp_sum(acc);
    if (lane == 0) G[p + q * kQB] = acc + vp[j0 + q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < jb; ++q) {
      const double tq = tau[j0 + q];
      for (int p = 0; p < q; ++p) {
        double z = 0.0;
        for (int l = p; l < q; ++l) z += Tm[p + l * kQB] * G[l + q * kQB];
        Tm[p + q * kQB] = -tq * z;
      }
      Tm[q + q * kQB] = tq;
      for (int p = q + 1; p < kQB; ++p) Tm[p + q * kQB] = 0.0;
    }
  }
  __syncthreads();
}

// C[:, c0:c1] <- (I - V op(T) V') C[:, c0:c1] over rows j0 .. m-1, op(T) = T' (QR, transT = 1)
// or T (forming Q, transT = 0); V = the block's reflectors (columns j0 .. j0+jb-1 of A).
__device__ void panel_apply_block(double* A, int64_t m, int64_t lda, int j0, int jb, int c0, int c1,
                                  const double* Tm, int transT, double* W, double* W2, double* Vc, int wcap) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5, tid = threadIdx.x;
  for (int t0 = c0; t0 < c1; t0 += wcap) {
    const int nt = min(wcap, c1 - t0);
    for (int e = tid; e < kQB * nt; e += blockDim.x) W[e] = 0.0;
    __syncthreads();
    // W = V' C  (rows from j0 on, chunked)
    for (int64_t r0 = j0; r0 < m; r0 += kQC) {
      const int rows = (int)(m - r0 < kQC ? m - r0 : kQC);
      for (int e = tid; e < rows * kQB; e += blockDim.x) {
        const int ii = e % rows, p = e / rows;  // consecutive threads: consecutive rows of a column
        const int64_t i = r0 + ii, ip = j0 + p;
        double v = 0.0;
        if (p < jb) v = (i == ip) ? 1.0 : (i > ip ? A[(int64_t)(j0 + p) * lda + i] : 0.0);
        Vc[ii * kQV + p] = v;
      }
      __syncthreads();
      for (int c = w; c < nt; c += nw) {
        const double* col = A + (int64_t)(t0 + c) * lda + r0;
        double acc[kQB];
#pragma unroll
        for (int p = 0; p < kQB; ++p) acc[p] = 0.0;
        for (int ii = lane; ii < rows; ii += 32) {
          const double x = col[ii];
#pragma unroll
          for (int p = 0; p < kQB; ++p) acc[p] += Vc[ii * kQV + p] * x;
        }
#pragma unroll
        for (int p = 0; p < kQB; ++p) {
          const double sum = warp_sum(acc[p]);
          if (lane == 0) W[p + c * kQB] += sum;
        }
      }
      __syncthreads();
    }
    // W2 = op(T) W
    for (int e = tid; e < kQB * nt; e += blockDim.x) {
      const int q = e % kQB, c = e / kQB;
      double z = 0.0;
      if (transT) {
        for (int p = 0; p <= q; ++p) z += Tm[p + q * kQB] * W[p + c * kQB];
      } else {
        for (int p = q; p < kQB; ++p) z += Tm[q + p * kQB] * W[p + c * kQB];
      }
      W2[e] = z;
    }
    __syncthreads();
    // C -= V W2
    for (int64_t r0 = j0; r0 < m; r0 += kQC) {
      const int rows = (int)(m - r0 < kQC ? m - r0 : kQC);
      for (int e = tid; e < rows * kQB; e += blockDim.x) {
        const int ii = e % rows, p = e / rows;  // consecutive threads: consecutive rows of a column
        const int64_t i = r0 + ii, ip = j0 + p;
        double v = 0.0;
        if (p < jb) v = (i == ip) ? 1.0 : (i > ip ? A[(int64_t)(j0 + p) * lda + i] : 0.0);
        Vc[ii * kQV + p] = v;
      }
      __syncthreads();
      for (int c = w; c < nt; c += nw) {
        double* col = A + (int64_t)(t0 + c) * lda + r0;
        const double* wc = W2 + c * kQB;
        for (int ii = lane; ii < rows; ii += 32) {
          double z = 0.0;
#pragma unroll
          for (int p = 0; p < kQB; ++p) z += Vc[ii * kQV + p] * wc[p];
          col[ii] -= z;
        }
      }
      __syncthreads();
    }
  }
}

// The panel QR of a level runs as a sequence of launches per reflector block, so that the
// trailing updates of a tall panel spread over many CTAs (one FP64-bound SM per panel took
// seconds for the 32768 x 549 panels of an n = 2^16 ACA matrix):
//   k_pq_factor  (one CTA per panel)        dgeqr2 on the block's kQB columns, its T
//   k_pq_update  (panels x column tiles)    block reflector applied to kQU trailing columns each
//   k_pq_rout    (one CTA per panel)        R out
//   then, blocks from last to first: k_pq_update on the formed columns, k_pq_form (dorg2r on
//   the block's own columns).  tau and the T factors live in global scratch between launches.
constexpr int kQU = 8;  // trailing columns per update CTA (each CTA is FP64-bound: narrow tiles, more SMs)

__global__ void __launch_bounds__(512) k_pq_factor(const PanelDesc* __restrict__ descs, int j0,
                                                   double* __restrict__ taus, int ldtau, double* __restrict__ Ts,
                                                   int nblk, int skip_big = 0) {
  __shared__ double red[40];
  __shared__ double sh[2];
  __shared__ double G[kQB * kQB], Tm[kQB * kQB];
  const PanelDesc D = descs[blockIdx.x];
  const int k = D.k;
  if (j0 >= k || (skip_big && D.big)) return;
  double* A = D.A;
  const int64_t m = D.m, lda = D.lda;
  double* tau = taus + (int64_t)blockIdx.x * ldtau;
  const int jb = min(kQB, k - j0);
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  for (int j = j0; j < j0 + jb; ++j) {  // dgeqr2 / dlarfg: beta = -sign(alpha) ||.||
    double* aj = A + (int64_t)j * lda;
    double part = 0.0;
    for (int64_t i = j + 1 + tid; i < m; i += blockDim.x) part += aj[i] * aj[i];
    const double sig = cta_sum(part, red);
    if (tid == 0) {
      const double alpha = aj[j];
      double tj = 0.0, beta = alpha, scal = 0.0;
      if (sig != 0.0) {
        const double nrm = sqrt(alpha * alpha + sig);
        beta = alpha >= 0.0 ? -nrm : nrm;
        tj = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      aj[j] = beta;
      sh[0] = scal;
      sh[1] = tj;
      tau[j] = tj;
    }
    __syncthreads();
    const double scal = sh[0], tj = sh[1];
    for (int64_t i = j + 1 + tid; i < m; i += blockDim.x) aj[i] *= scal;
    __syncthreads();
    if (tj != 0.0) {
      for (int c = j + 1 + w; c < j0 + jb; c += nw) {
        double* ac = A + (int64_t)c * lda;
        double acc = (lane == 0) ? ac[j] : 0.0;
        for (int64_t i = j + 1 + lane; i < m; i += 32) acc += aj[i] * ac[i];
        acc = warp_sum(acc) * tj;
        if (lane == 0) ac[j] -= acc;
        for (int64_t i = j + 1 + lane; i < m; i += 32) ac[i] -= acc * aj[i];
      }
    }
    __syncthreads();
  }
  if (j0 + jb < k) {
    panel_block_T(A, m, lda, j0, jb, tau, G, Tm);
    double* Tout = Ts + ((int64_t)blockIdx.x * nblk + j0 / kQB) * kQB * kQB;
    for (int e = tid; e < kQB * kQB; e += blockDim.x) Tout[e] = Tm[e];
  }
}

// grid (panels, tiles): the reflector block at j0 applied to trailing columns j0+kQB + y*kQU ..
// (transT = 1: QR, I - V T' V'; transT = 0: forming Q, I - V T V').
__global__ void __launch_bounds__(256) k_pq_update(const PanelDesc* __restrict__ descs, int j0,
                                                   const double* __restrict__ Ts, int nblk, int transT) {
  extern __shared__ double smq[];
  __shared__ double Tm[kQB * kQB];
  const PanelDesc D = descs[blockIdx.x];
  const int k = D.k;
  if (j0 >= k || D.big) return;
  const int jb = min(kQB, k - j0), j1 = j0 + jb;
  const int c0 = j1 + blockIdx.y * kQU;
  if (c0 >= k) return;
  const double* Tin = Ts + ((int64_t)blockIdx.x * nblk + j0 / kQB) * kQB * kQB;
  for (int e = threadIdx.x; e < kQB * kQB; e += blockDim.x) Tm[e] = Tin[e];
  double* W = smq;               // kQB x kQU
  double* W2 = W + kQB * kQU;    // kQB x kQU
  double* Vc = W2 + kQB * kQU;   // kQC x kQV
  __syncthreads();
  panel_apply_block(D.A, D.m, D.lda, j0, jb, c0, min(c0 + kQU, k), Tm, transT, W, W2, Vc, kQU);
}

__global__ void k_pq_rout(const PanelDesc* __restrict__ descs) {
  const PanelDesc D = descs[blockIdx.x];
  const int k = D.k;
  for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
    const int i = e % k, c = e / k;
    D.R[e] = (i <= c) ? D.A[(int64_t)c * D.lda + i] : 0.0;
  }
}

// dorg2r on the block's own columns j0 .. j1-1 (the columns to its right are already formed).
__global__ void __launch_bounds__(512) k_pq_form(const PanelDesc* __restrict__ descs, int j0,
                                                 const double* __restrict__ taus, int ldtau, int skip_big = 0) {
  const PanelDesc D = descs[blockIdx.x];
  const int k = D.k;
  if (j0 >= k || (skip_big && D.big)) return;
  double* A = D.A;
  const int64_t m = D.m, lda = D.lda;
  const double* tau = taus + (int64_t)blockIdx.x * ldtau;
  const int j1 = min(j0 + kQB, k);
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  for (int j = j1 - 1; j >= j0; --j) {
    double* aj = A + (int64_t)j * lda;
    const double tj = tau[j];
    if (j < j1 - 1) {
      if (tid == 0) aj[j] = 1.0;
      __syncthreads();
      for (int c = j + 1 + w; c < j1; c += nw) {
        double* ac = A + (int64_t)c * lda;
        double acc = 0.0;
        for (int64_t i = j + lane; i < m; i += 32) acc += aj[i] * ac[i];
        acc = warp_sum(acc) * tj;
        for (int64_t i = j + lane; i < m; i += 32) ac[i] -= acc * aj[i];
      }
      __syncthreads();
    }
    for (int64_t i = j + 1 + tid; i < m; i += blockDim.x) aj[i] *= -tj;
    for (int64_t i = tid; i < j; i += blockDim.x) aj[i] = 0.0;
    if (tid == 0) aj[j] = 1.0 - tj;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------------------------
// Node capacitance of the general factorisation: C = R1 R2', L22 = chol(I - C'C) (lower), one
// CTA per node, operands in global memory.  info[node] = failing column (1-based) or 0.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(512) k_gnode(const GNodeDesc* __restrict__ nodes, int* __restrict__ info) {
  const GNodeDesc N = nodes[blockIdx.x];
  const int r = N.r;
  const double* R1 = N.R1;
  const double* R2 = N.R2;
  double* C = N.C;
  double* Lm = N.L22;
  const int tid = threadIdx.x;
  for (int e = tid; e < r * r; e += blockDim.x) {
    const int i = e % r, c = e / r;
    double acc = 0.0;
    for (int l = max(i, c); l < r; ++l) acc += R1[i + (int64_t)l * r] * R2[c + (int64_t)l * r];
    C[e] = acc;
  }
  __syncthreads();
  for (int e = tid; e < r * r; e += blockDim.x) {
    const int i = e % r, c = e / r;
    if (i >= c) {
      double acc = 0.0;
      for (int l = 0; l < r; ++l) acc += C[l + (int64_t)i * r] * C[l + (int64_t)c * r];
      Lm[e] = (i == c ? 1.0 : 0.0) - acc;
    } else {
      Lm[e] = 0.0;
    }
  }
  __syncthreads();
  __shared__ int bad;
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < r; ++j) {
    const double d = Lm[j + (int64_t)j * r];
    const bool ok = d > 0.0;
    const double sd = ok ? sqrt(d) : 1.0;
    __syncthreads();
    if (tid == 0 && !ok && bad == 0) bad = j + 1;
    for (int i = j + 1 + tid; i < r; i += blockDim.x) Lm[i + (int64_t)j * r] /= sd;
    if (tid == 0) Lm[j + (int64_t)j * r] = sd;
    __syncthreads();
    const int wdt = r - j - 1;
    for (int e = tid; e < wdt * wdt; e += blockDim.x) {
      const int i = j + 1 + e % wdt, c = j + 1 + e / wdt;
      if (i >= c) Lm[i + (int64_t)c * r] -= Lm[i + (int64_t)j * r] * Lm[c + (int64_t)j * r];
    }
    __syncthreads();
  }
  if (tid == 0) info[blockIdx.x] = bad;
}

// ---------------------------------------------------------------------------------------------
// Application of node factors to column blocks, one warp per (item, column):
//   mode 0 (W^{-1}):  y2 -= Q2 (z2 - L22^{-1}(z2 - C' z1))
//   mode 1 (W^{-T}):  t = L22^{-T} z2;  y1 -= Q1 C t;  y2 -= Q2 (z2 - t)
//   mode 2 (W):       y2 += Q2 (C' z1 + L22 z2 - z2)
//   mode 3 (W'):      y1 += Q1 C z2;  y2 += Q2 (L22' z2 - z2)
//   mode 4 (pre-factor product): y1 += V (U' y2_in), y2 += U (V' y1_in) with Q1 = V, Q2 = U
//          reading x (in) and accumulating into y (out)
// with z1 = Q1' y1, z2 = Q2' y2.  grid = (items, ceil(ncols/8)), block 256.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gapply(const GApplyItem* __restrict__ items,
                                                const GNodeDesc* __restrict__ nodes, int mode, double* X,
                                                const double* Xin, int64_t ldX, int kX) {
  extern __shared__ double sm[];
  const GApplyItem I = items[blockIdx.x];
  if (I.big) return;  // large nodes go through the library-GEMM path
  const GNodeDesc N = nodes[I.node];
  const int r = N.r;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int col = blockIdx.y * 8 + w;
  double* base = I.base ? I.base : X;
  const int64_t ld = I.base ? I.ld : ldX;
  const int ncols = I.base ? I.ncols : kX;
  if (col >= ncols) return;
  double* z1 = sm + (size_t)w * 3 * r;
  double* z2 = z1 + r;
  double* t = z2 + r;
  double* y1 = base + I.off1 + (int64_t)col * ld;
  double* y2 = base + I.off2 + (int64_t)col * ld;
  const double* x1 = (mode == 4) ? Xin + I.off1 + (int64_t)col * ldX : y1;
  const double* x2 = (mode == 4) ? Xin + I.off2 + (int64_t)col * ldX : y2;
  const double* Q1 = N.Q1;
  const double* Q2 = N.Q2;
  const int64_t s1 = N.s1, s2 = N.s2;
  // projections z1 = Q1' x1, z2 = Q2' x2 (mode 4: z1 = U' x2, z2 = V' x1)
  for (int q = 0; q < r; ++q) {
    const double* q1 = (mode == 4 ? Q2 : Q1) + (int64_t)q * (mode == 4 ? s2 : s1);
    const double* q2 = (mode == 4 ? Q1 : Q2) + (int64_t)q * (mode == 4 ? s1 : s2);
    const double* xa = (mode == 4) ? x2 : x1;
    const double* xb = (mode == 4) ? x1 : x2;
    const int64_t na = (mode == 4) ? s2 : s1, nb = (mode == 4) ? s1 : s2;
    double a = 0.0, b = 0.0;
    if (mode == 0 || mode == 2 || mode == 4)
      for (int64_t i = lane; i < na; i += 32) a += q1[i] * xa[i];
    for (int64_t i = lane; i < nb; i += 32) b += q2[i] * xb[i];
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) {
      z1[q] = a;
      z2[q] = b;
    }
  }
  __syncwarp();
  const double* C = N.C;
  const double* Lm = N.L22;
  if (mode == 4) {
    // y1 (rows c1) += V z1 ; y2 (rows c2) += U z2   (V = Q1 rows c1, U = Q2 rows c2)
    for (int64_t i = lane; i < s1; i += 32) {
      double acc = 0.0;
      for (int q = 0; q < r; ++q) acc += Q1[i + (int64_t)q * s1] * z1[q];
      y1[i] += acc;
    }
    for (int64_t i = lane; i < s2; i += 32) {
      double acc = 0.0;
      for (int q = 0; q < r; ++q) acc += Q2[i + (int64_t)q * s2] * z2[q];
      y2[i] += acc;
    }
    return;
  }
  if (mode == 0) {
    for (int i = lane; i < r; i += 32) {
      double acc = 0.0;
      for (int l = 0; l < r; ++l) acc += C[l + (int64_t)i * r] * z1[l];
      t[i] = z2[i] - acc;
    }
    __syncwarp();
    for (int l = 0; l < r; ++l) {
      const double v = t[l] / Lm[l + (int64_t)l * r];
      __syncwarp();
      if (lane == 0) t[l] = v;
      for (int i = l + 1 + lane; i < r; i += 32) t[i] -= Lm[i + (int64_t)l * r] * v;
      __syncwarp();
    }
    for (int i = lane; i < r; i += 32) t[i] = z2[i] - t[i];
    __syncwarp();
    for (int64_t i = lane; i < s2; i += 32) {
      double acc = 0.0;
      for (int q = 0; q < r; ++q) acc += Q2[i + (int64_t)q * s2] * t[q];
      y2[i] -= acc;
    }
  } else if (mode == 1) {
    for (int i = lane; i < r; i += 32) t[i] = z2[i];
    __syncwarp();
    for (int i = r - 1; i >= 0; --i) {
      const double v = t[i] / Lm[i + (int64_t)i * r];
      __syncwarp();
      if (lane == 0) t[i] = v;
      for (int l = lane; l < i; l += 32) t[l] -= Lm[i + (int64_t)l * r] * v;
      __syncwarp();
    }
    // z1 <- C t (reuse z1), z2 <- z2 - t
    for (int i = lane; i < r; i += 32) {
      double acc = 0.0;
      for (int l = 0; l < r; ++l) acc += C[i + (int64_t)l * r] * t[l];
      z1[i] = acc;
    }
    __syncwarp();
    for (int i = lane; i < r; i += 32) z2[i] -= t[i];
    __syncwarp();
    for (int64_t i = lane; i < s1; i += 32) {
      double acc = 0.0;
      for (int q = 0; q < r; ++q) acc += Q1[i + (int64_t)q * s1] * z1[q];
      y1[i] -= acc;
    }
    for (int64_t i = lane; i < s2; i += 32) {
      double acc = 0.0;
      for (int q = 0; q < r; ++q) acc += Q2[i + (int64_t)q * s2] * z2[q];
      y2[i] -= acc;
    }
  } else if (mode == 2) {
    for (int i = lane; i < r; i += 32) {
      double acc = 0.0;
      for (int l = 0; l < r; ++l) acc += C[l + (int64_t)i * r] * z1[l];
      for (int l = 0; l <= i; ++l) acc += Lm[i + (int64_t)l * r] * z2[l];
      t[i] = acc - z2[i];
    }
    __syncwarp();
    for (int64_t i = lane; i < s2; i += 32) {
      double acc = 0.0;
      for (int q = 0; q < r; ++q) acc += Q2[i + (int64_t)q * s2] * t[q];
      y2[i] += acc;
    }
  } else {
    for (int i = lane; i < r; i += 32) {
      double a1 = 0.0, a2 = 0.0;
      for (int l = 0; l < r; ++l) a1 += C[i + (int64_t)l * r] * z2[l];
      for (int l = i; l < r; ++l) a2 += Lm[l + (int64_t)i * r] * z2[l];
      z1[i] = a1;
      t[i] = a2 - z2[i];
    }
    __syncwarp();
    for (int64_t i = lane; i < s1; i += 32) {
      double acc = 0.0;
      for (int q = 0; q < r; ++q) acc += Q1[i + (int64_t)q * s1] * z1[q];
      y1[i] += acc;
    }
    for (int64_t i = lane; i < s2; i += 32) {
      double acc = 0.0;
      for (int q = 0; q < r; ++q) acc += Q2[i + (int64_t)q * s2] * t[q];
      y2[i] += acc;
    }
  }
}

// The r x r part of k_gapply (same operations in the same order) for the nodes whose
// projections and expansions run as library GEMMs: one warp per column.
__global__ void k_gsmall(const GNodeDesc* __restrict__ node, int mode, const double* __restrict__ Z1,
                         const double* __restrict__ Z2, double* __restrict__ G1, double* __restrict__ G2) {
  extern __shared__ double sm[];
  const GNodeDesc N = *node;
  const int r = N.r;
  const int lane = threadIdx.x;
  const int col = blockIdx.x;
  double* z1 = sm;
  double* z2 = z1 + r;
  double* t = z2 + r;
  for (int i = lane; i < r; i += 32) {
    z1[i] = (mode == 0 || mode == 2) ? Z1[(int64_t)col * r + i] : 0.0;
    z2[i] = Z2[(int64_t)col * r + i];
  }
  __syncwarp();
  const double* C = N.C;
  const double* Lm = N.L22;
  double* g1 = G1 + (int64_t)col * r;
  double* g2 = G2 + (int64_t)col * r;
  if (mode == 0) {
    for (int i = lane; i < r; i += 32) {
      double acc = 0.0;
      for (int l = 0; l < r; ++l) acc += C[l + (int64_t)i * r] * z1[l];
      t[i] = z2[i] - acc;
    }
    __syncwarp();
    for (int l = 0; l < r; ++l) {
      const double v = t[l] / Lm[l + (int64_t)l * r];
      __syncwarp();
      if (lane == 0) t[l] = v;
      for (int i = l + 1 + lane; i < r; i += 32) t[i] -= Lm[i + (int64_t)l * r] * v;
      __syncwarp();
    }
    for (int i = lane; i < r; i += 32) g2[i] = z2[i] - t[i];
  } else if (mode == 1) {
    for (int i = lane; i < r; i += 32) t[i] = z2[i];
    __syncwarp();
    for (int i = r - 1; i >= 0; --i) {
      const double v = t[i] / Lm[i + (int64_t)i * r];
      __syncwarp();
      if (lane == 0) t[i] = v;
      for (int l = lane; l < i; l += 32) t[l] -= Lm[i + (int64_t)l * r] * v;
      __syncwarp();
    }
    for (int i = lane; i < r; i += 32) {
      double acc = 0.0;
      for (int l = 0; l < r; ++l) acc += C[i + (int64_t)l * r] * t[l];
      g1[i] = acc;
      g2[i] = z2[i] - t[i];
    }
  } else if (mode == 2) {
    for (int i = lane; i < r; i += 32) {
      double acc = 0.0;
      for (int l = 0; l < r; ++l) acc += C[l + (int64_t)i * r] * z1[l];
      for (int l = 0; l <= i; ++l) acc += Lm[i + (int64_t)l * r] * z2[l];
      g2[i] = acc - z2[i];
    }
  } else {
    for (int i = lane; i < r; i += 32) {
      double a1 = 0.0, a2 = 0.0;
      for (int l = 0; l < r; ++l) a1 += C[i + (int64_t)l * r] * z2[l];
      for (int l = i; l < r; ++l) a2 += Lm[l + (int64_t)i * r] * z2[l];
      g1[i] = a1;
      g2[i] = a2 - z2[i];
    }
  }
}

// 2 sum log |diag(L22)| over the general nodes: one partial per node (deterministic).
__global__ void k_glogdet(const GNodeDesc* __restrict__ nodes, int nn, double* __restrict__ partial) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nn) return;
  const GNodeDesc N = nodes[q];
  double s = 0.0;
  for (int i = 0; i < N.r; ++i) s += 2.0 * log(fabs(N.L22[i + (int64_t)i * N.r]));
  partial[q] = s;
}

// ---------------------------------------------------------------------------------------------
// ACA of one large block by every SM (cooperative launch, one CTA per SM).  The steps are those
// of k_aca (factorizations.jl:9-84): each CTA owns a slice of the rows and a slice of the
// columns, evaluates its part of the residual row / column, and the argmax searches and the
// norms are reduced over the CTAs' partial results in a fixed order, so every CTA takes the
// same pivots.  Values written by other CTAs (records, pivots' entries, the published norms) are
// read with ld.global.cg (L2, the coherence point); a CTA sets the used-row/column flags of its
// own slices only.  Grid barriers spin a bounded number of times; a barrier that runs out sets the
// block's status to 3 (timeout) and the CTAs leave the loop together at the next check.
// ---------------------------------------------------------------------------------------------
constexpr long long kGridSpinLimit = 1ll << 20;  // L2 polls per barrier wait (~0.3 s)

struct GridBar {
  unsigned* count;
  volatile unsigned* gen;
  volatile int* err;
  long long limit;  // polls before a wait gives up (< 0: kGridSpinLimit; 0: at the first poll, as
                    // if the other CTAs never arrived: the test of the timeout path)
};

// Returns true when every CTA has arrived and no barrier of this launch has run out; the answer
// is the same for all threads of the CTA (thread 0's view, passed through shared memory), so the
// CTA leaves its loop as a whole.
__device__ bool grid_barrier(GridBar gb) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const long long lim = gb.limit < 0 ? kGridSpinLimit : gb.limit;
    const unsigned g = *gb.gen;
    __threadfence();
    if (atomicAdd(gb.count, 1u) == gridDim.x - 1) {
      *gb.count = 0;
      __threadfence();
      atomicExch((unsigned*)gb.gen, g + 1);
    } else {
      long long spins = 0;
      while ((gb.limit == 0 || *gb.gen == g) && *gb.err == 0) {
        if (++spins > lim) {
          atomicExch((int*)gb.err, 1);
          break;
        }
      }
    }
    __threadfence();
    s_ok = *gb.err == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

// partial argmax record of one CTA: (|x| best, its index, first unflagged index)
__device__ void slice_argmax(const double* x, const uint8_t* excl, int64_t lo, int64_t hi, double* sval,
                             long long* sidx, double* pval, long long* pidx) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double best = 0.0;
  long long bi = LLONG_MAX, first = LLONG_MAX;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    if (excl[i]) continue;
    if (first == LLONG_MAX) first = i;
    const double a = fabs(x[i]);
    if (a > best) {
      best = a;
      bi = i;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
    const long long of = __shfl_xor_sync(0xffffffffu, first, o);
    if (ob > best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
    first = min(first, of);
  }
  if (lane == 0) {
    sval[w] = best;
    sidx[w] = bi;
    sidx[32 + w] = first;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    long long ib = LLONG_MAX, f = LLONG_MAX;
    for (int q = 0; q < nw; ++q) {
      if (sval[q] > b || (sval[q] == b && sidx[q] < ib)) {
        b = sval[q];
        ib = sidx[q];
      }
      f = min(f, sidx[32 + q]);
    }
    *pval = b;
    pidx[0] = ib;
    pidx[1] = f;
  }
  __syncthreads();
}

// combine the CTAs' argmax records (same order in every CTA): restrictedmaxabs semantics.
// CTA g's record: value at pval[g * stride], indices at pidx[2 g] (best) and pidx[2 g + 1] (first).
__device__ void grid_argmax(const double* x, int64_t n, const double* pval, const long long* pidx, int stride,
                            double* sh, long long* shi, double* out_val, int64_t* out_idx) {
  if (threadIdx.x == 0) {
    double b = 0.0;
    long long ib = LLONG_MAX, f = LLONG_MAX;
    for (int g = 0; g < (int)gridDim.x; ++g) {
      const double v = __ldcg(pval + (int64_t)g * stride);
      const long long i = __ldcg(pidx + 2 * g), fi = __ldcg(pidx + 2 * g + 1);
      if (v > b || (v == b && i < ib)) {
        b = v;
        ib = i;
      }
      f = min(f, fi);
    }
    if (b > 0.0) {
      sh[0] = __ldcg(x + ib);
      shi[0] = ib;
    } else {
      sh[0] = 0.0;
      shi[0] = (f == LLONG_MAX) ? n - 1 : f;
    }
  }
  __syncthreads();
  *out_val = sh[0];
  *out_idx = shi[0];
  __syncthreads();
}

__global__ void __launch_bounds__(512) k_aca_grid(const double* __restrict__ pts, KParams kp,
                                                  const AcaBlock* __restrict__ blocks, int bidx,
                                                  double* __restrict__ P, uint8_t* __restrict__ F,
                                                  int* __restrict__ piv, double rtol, int* __restrict__ rank_out,
                                                  int* __restrict__ status, double* __restrict__ scr,
                                                  GridBar gb) {
  extern __shared__ double coef[];  // cap: U[ri, j] or V[cj, j] of the previous columns
  __shared__ double sred[40];
  __shared__ double sval[40];
  __shared__ long long sidx[72];
  __shared__ double sh[4];
  __shared__ long long shi[2];
  const AcaBlock B = blocks[bidx];
  const int64_t nro = B.nro, ncl = B.ncl;
  const int cap = B.cap;
  double* U = P + B.offU;
  double* V = P + B.offV;
  uint8_t* urow = F + B.offFlag;
  uint8_t* ucol = urow + nro;
  int* prow = piv + 2 * B.offPiv;
  int* pcol = prow + cap;
  const int G = gridDim.x, g = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  const int64_t rs = (nro + G - 1) / G, cs = (ncl + G - 1) / G;
  auto mn = [](int64_t a, int64_t b) { return a < b ? a : b; };
  const int64_t r_lo = mn(nro, (int64_t)g * rs), r_hi = mn(nro, r_lo + rs);
  const int64_t c_lo = mn(ncl, (int64_t)g * cs), c_hi = mn(ncl, c_lo + cs);
  const double* xr = pts + 2 * B.row0;
  const double* xc = pts + 2 * B.col0;
  // scratch: per CTA a record of stride S doubles: [0] argmax value, [1] sum 1, [2] sum 2,
  // [3 .. 3+cap) dots a_j, [3+cap .. 3+2cap) dots b_j; then 2 long longs per CTA; then scalars
  const int S = 3 + 2 * cap;
  double* rec = scr + (int64_t)g * S;
  long long* irec = reinterpret_cast<long long*>(scr + (int64_t)G * S);
  double* scal = scr + (int64_t)G * S + 2 * G;  // [0] znorm2, [1] sr, [2] sc
  for (int64_t i = r_lo + tid; i < r_hi; i += blockDim.x) urow[i] = 0;
  for (int64_t c = c_lo + tid; c < c_hi; c += blockDim.x) ucol[c] = 0;
  if (!grid_barrier(gb)) goto done;
  {
    const int maxsz = B.maxsz;
    auto slice_max = [&](const double* x) {
      double mx = 0.0;
      for (int64_t c = c_lo + tid; c < c_hi; c += blockDim.x) mx = fmax(mx, fabs(x[c]));
      for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (lane == 0) sred[w] = mx;
      __syncthreads();
      if (tid == 0) {
        double m = 0.0;
        for (int q = 0; q < nw; ++q) m = fmax(m, sred[q]);
        rec[0] = m;
      }
      __syncthreads();
    };
    auto all_max = [&]() {
      if (tid == 0) {
        double m = 0.0;
        for (int q = 0; q < G; ++q) m = fmax(m, __ldcg(scr + (int64_t)q * S));
        sh[2] = m;
      }
      __syncthreads();
      const double m = sh[2];
      __syncthreads();
      return m;
    };
    auto slice_sum = [&](const double* x, int64_t lo, int64_t hi) {
      double a = 0.0;
      for (int64_t i = lo + tid; i < hi; i += blockDim.x) a += x[i] * x[i];
      return cta_sum(a, sred);
    };
    // first row not all zero (factorizations.jl:24-30)
    int64_t strt = 0;
    for (;;) {
      const double px = xr[2 * strt], py = xr[2 * strt + 1];
      for (int64_t c = c_lo + tid; c < c_hi; c += blockDim.x) V[c] = kernel_value(kp, px, py, xc[2 * c], xc[2 * c + 1]);
      __syncthreads();
      slice_max(V);
      if (!grid_barrier(gb)) goto done;
      const double m = all_max();
      if (m != 0.0 || strt + 1 >= maxsz) break;
      ++strt;
      if (!grid_barrier(gb)) goto done;  // records are rewritten by the next row
    }
    if (strt + 1 == maxsz) {
      if (g == 0 && tid == 0) {
        status[bidx] = 1;
        rank_out[bidx] = 0;
      }
      goto done;
    }
    if (tid == 0 && strt >= r_lo && strt < r_hi) urow[strt] = 1;  // flags are set by their slice's owner
    if (g == 0 && tid == 0) prow[0] = (int)strt;
    double mv;
    int64_t mi;
    slice_argmax(V, ucol, c_lo, c_hi, sval, sidx, rec, irec + 2 * g);
    if (!grid_barrier(gb)) goto done;
    grid_argmax(V, ncl, scr, irec, S, sh, shi, &mv, &mi);
    if (!grid_barrier(gb)) goto done;  // V[mi] is read before the division below
    for (int64_t c = c_lo + tid; c < c_hi; c += blockDim.x) V[c] = __ddiv_rn(V[c], mv);
    {
      const double px = xc[2 * mi], py = xc[2 * mi + 1];
      for (int64_t i = r_lo + tid; i < r_hi; i += blockDim.x) U[i] = kernel_value(kp, xr[2 * i], xr[2 * i + 1], px, py);
    }
    __syncthreads();
    {
      const double a = slice_sum(V, c_lo, c_hi), b = slice_sum(U, r_lo, r_hi);
      if (tid == 0) {
        rec[1] = a;
        rec[2] = b;
      }
    }
    if (tid == 0 && mi >= c_lo && mi < c_hi) ucol[mi] = 1;
    if (g == 0 && tid == 0) pcol[0] = (int)mi;
    if (!grid_barrier(gb)) goto done;
    double sr = 0.0, sc = 0.0;
    for (int q = 0; q < G; ++q) {
      sr += __ldcg(scr + (int64_t)q * S + 1);
      sc += __ldcg(scr + (int64_t)q * S + 2);
    }
    double znorm2 = __dmul_rn(sr, sc);
    int frnk = 1, st = 0;
    while (__dmul_rn(sqrt(sr), sqrt(sc)) > __dmul_rn(rtol, sqrt(znorm2)) && frnk < maxsz) {
      // next row pivot: argmax of the last column over unused rows
      const double* lastcol = U + (int64_t)(frnk - 1) * nro;
      double rv;
      int64_t ri;
      if (!grid_barrier(gb)) goto done;  // the records of the previous step have been read
      slice_argmax(lastcol, urow, r_lo, r_hi, sval, sidx, rec, irec + 2 * g);
      if (!grid_barrier(gb)) goto done;
      grid_argmax(lastcol, nro, scr, irec, S, sh, shi, &rv, &ri);
      if (frnk >= cap) {
        st = 2;
        break;
      }
      for (int j = tid; j < frnk; j += blockDim.x) coef[j] = __ldcg(U + ri + (int64_t)j * nro);
      __syncthreads();
      double* row = V + (int64_t)frnk * ncl;
      {
        const double px = xr[2 * ri], py = xr[2 * ri + 1];
        for (int64_t c = c_lo + tid; c < c_hi; c += blockDim.x) {
          double v = kernel_value(kp, px, py, xc[2 * c], xc[2 * c + 1]);
          for (int j = 0; j < frnk; ++j) v = __dsub_rn(v, __dmul_rn(coef[j], V[c + (int64_t)j * ncl]));
          row[c] = v;
        }
      }
      if (!grid_barrier(gb)) goto done;  // urow[ri] is set after every CTA searched
      if (tid == 0 && ri >= r_lo && ri < r_hi) urow[ri] = 1;
      double cv;
      int64_t cj;
      slice_argmax(row, ucol, c_lo, c_hi, sval, sidx, rec, irec + 2 * g);
      if (!grid_barrier(gb)) goto done;
      grid_argmax(row, ncl, scr, irec, S, sh, shi, &cv, &cj);
      if (cv == 0.0) break;
      if (!grid_barrier(gb)) goto done;  // row[cj] is read before the division below
      if (tid == 0 && cj >= c_lo && cj < c_hi) ucol[cj] = 1;
      for (int64_t c = c_lo + tid; c < c_hi; c += blockDim.x) row[c] = __ddiv_rn(row[c], cv);
      for (int j = tid; j < frnk; j += blockDim.x) coef[j] = __ldcg(V + cj + (int64_t)j * ncl);
      __syncthreads();
      double* col = U + (int64_t)frnk * nro;
      {
        const double px = xc[2 * cj], py = xc[2 * cj + 1];
        for (int64_t i = r_lo + tid; i < r_hi; i += blockDim.x) {
          double v = kernel_value(kp, xr[2 * i], xr[2 * i + 1], px, py);
          for (int j = 0; j < frnk; ++j) v = __dsub_rn(v, __dmul_rn(coef[j], U[i + (int64_t)j * nro]));
          col[i] = v;
        }
      }
      __syncthreads();
      // partial dots with the previous columns and the new squared norms
      for (int j = w; j < frnk; j += nw) {
        const double* uj = U + (int64_t)j * nro;
        const double* vj = V + (int64_t)j * ncl;
        double a = 0.0, b = 0.0;
        for (int64_t i = r_lo + lane; i < r_hi; i += 32) a += uj[i] * col[i];
        for (int64_t c = c_lo + lane; c < c_hi; c += 32) b += vj[c] * row[c];
        a = warp_sum(a);
        b = warp_sum(b);
        if (lane == 0) {
          rec[3 + j] = a;
          rec[3 + cap + j] = b;
        }
      }
      {
        const double a = slice_sum(row, c_lo, c_hi), b = slice_sum(col, r_lo, r_hi);
        if (tid == 0) {
          rec[1] = a;
          rec[2] = b;
        }
      }
      if (!grid_barrier(gb)) goto done;
      if (g == 0) {
        // dots summed over the CTAs in a fixed order, one warp per j
        for (int j = w; j < frnk; j += nw) {
          double a = 0.0, b = 0.0;
          for (int q = lane; q < G; q += 32) {
            a += __ldcg(scr + (int64_t)q * S + 3 + j);
            b += __ldcg(scr + (int64_t)q * S + 3 + cap + j);
          }
          a = warp_sum(a);
          b = warp_sum(b);
          if (lane == 0) coef[j] = __dmul_rn(__dmul_rn(2.0, fabs(a)), fabs(b));
        }
        __syncthreads();
        if (tid == 0) {
          double z = znorm2;
          for (int j = 0; j < frnk; ++j) z = __dadd_rn(z, coef[j]);
          double s1 = 0.0, s2 = 0.0;
          for (int q = 0; q < G; ++q) {
            s1 += __ldcg(scr + (int64_t)q * S + 1);
            s2 += __ldcg(scr + (int64_t)q * S + 2);
          }
          scal[0] = __dadd_rn(z, __dmul_rn(s1, s2));
          scal[1] = s1;
          scal[2] = s2;
          prow[frnk] = (int)ri;
          pcol[frnk] = (int)cj;
        }
      }
      if (!grid_barrier(gb)) goto done;
      znorm2 = __ldcg(scal);
      sr = __ldcg(scal + 1);
      sc = __ldcg(scal + 2);
      ++frnk;
    }
    if (g == 0 && tid == 0) {
      rank_out[bidx] = frnk;
      status[bidx] = st;
    }
  }
done:
  if (g == 0 && tid == 0 && *gb.err) status[bidx] = 3;
}

int64_t aca_grid_scratch(int cap) {
  const int G = 152 * 2;  // upper bound of the grid
  return (int64_t)G * (3 + 2 * cap) + 2 * G + 8 + 4;
}

bool launch_aca_grid(const double* pts, KParams kp, const AcaBlock* blocks, int b, int cap, double* P, uint8_t* F,
                     int* piv, double rtol, int* rank, int* status, double* scratch, cudaStream_t st,
                     long long wait_limit) {
  int dev = 0, coop = 0, nsm = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (!coop) return false;
  const size_t sm = (size_t)std::max(cap, 1) * sizeof(double);
  smem_limit((const void*)k_aca_grid, sm);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_aca_grid, 512, sm) != cudaSuccess || per < 1) {
    cudaGetLastError();
    return false;
  }
  const int G = std::min(nsm, 152 * 2);
  // barrier words live after the records in the scratch
  unsigned* words = reinterpret_cast<unsigned*>(scratch + (int64_t)G * (3 + 2 * cap) + 2 * G + 8);
  if (cudaMemsetAsync(words, 0, 4 * sizeof(unsigned), st) != cudaSuccess) return false;
  GridBar gb{words, words + 1, reinterpret_cast<volatile int*>(words + 2), wait_limit};
  void* args[] = {(void*)&pts, (void*)&kp, (void*)&blocks, (void*)&b, (void*)&P, (void*)&F, (void*)&piv,
                  (void*)&rtol, (void*)&rank, (void*)&status, (void*)&scratch, (void*)&gb};
  if (cudaLaunchCooperativeKernel((const void*)k_aca_grid, dim3(G), dim3(512), args, sm, st) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

void launch_aca_one(const double* pts, KParams kp, const AcaBlock* blocks, int b, int maxcap, double* P,
                    uint8_t* F, int* piv, double rtol, int* rank, int* status, cudaStream_t st) {
  const size_t sm = (size_t)2 * std::max(maxcap, 1) * sizeof(double);
  smem_limit((const void*)k_aca, sm);
  k_aca<<<1, 1024, sm, st>>>(pts, kp, blocks, P, F, piv, rtol, rank, status, b);
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
void launch_aca(const double* pts, KParams kp, const AcaBlock* blocks, int nblocks, int maxcap, double* P,
                uint8_t* F, int* piv, double rtol, int* rank, int* status, cudaStream_t st) {
  const size_t sm = (size_t)2 * std::max(maxcap, 1) * sizeof(double);
  smem_limit((const void*)k_aca, sm);
  k_aca<<<nblocks, 1024, sm, st>>>(pts, kp, blocks, P, F, piv, rtol, rank, status, -1);
}

void launch_panel_qr(const PanelDesc* descs, int n, int kmax, double* taus, double* Ts, cudaStream_t st) {
  if (n <= 0 || kmax <= 0) return;
  const int nblk = (kmax + kQB - 1) / kQB;
  const int ntiles = (kmax + kQU - 1) / kQU;
  const size_t smu = ((size_t)2 * kQB * kQU + kQC * kQV) * sizeof(double);
  smem_limit((const void*)k_pq_update, smu);
  for (int b = 0; b < nblk; ++b) {
    k_pq_factor<<<n, 512, 0, st>>>(descs, b * kQB, taus, kmax, Ts, nblk);
    k_pq_update<<<dim3((unsigned)n, (unsigned)ntiles), 256, smu, st>>>(descs, b * kQB, Ts, nblk, 1);
  }
  k_pq_rout<<<n, 256, 0, st>>>(descs);
  for (int b = nblk - 1; b >= 0; --b) {
    k_pq_update<<<dim3((unsigned)n, (unsigned)ntiles), 256, smu, st>>>(descs, b * kQB, Ts, nblk, 0);
    k_pq_form<<<n, 512, 0, st>>>(descs, b * kQB, taus, kmax);
  }
}

// ---------------------------------------------------------------------------------------------
// Factor and form steps of one 8-column block of ONE tall panel by all SMs (cooperative launch):
// CTA b owns the contiguous row slice [b*rows, (b+1)*rows); every sum over rows is formed as
// per-CTA partials that all CTAs add in CTA order after a bounded grid barrier (same value in
// every CTA, same bits on every run); the partial buffers alternate between two halves so that a
// phase never overwrites partials another CTA may still be reading; every element is updated by
// the CTA that owns its row.  The operations per element are those of k_pq_factor / k_pq_form
// (dgeqr2 / dlarfg and dorg2r rules); only the order of the row sums differs.
// ---------------------------------------------------------------------------------------------
constexpr int kPqParts = 32;  // partial slots per CTA per phase

__device__ __forceinline__ double sum_parts(const double* part, int G, int slot) {
  double s = 0.0;
  for (int q = 0; q < G; ++q) s += __ldcg(part + (int64_t)q * kPqParts + slot);
  return s;
}

// CTA partial of up to 28 values in one pass: red holds nw x kPqParts doubles
__device__ void cta_parts(double (&v)[kPqParts], int nv, double* red, double* out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int t = 0; t < nv; ++t) {
    const double x = warp_sum(v[t]);
    if (lane == 0) red[w * kPqParts + t] = x;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double s = 0.0;
    for (int q = 0; q < nw; ++q) s += red[q * kPqParts + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(256) k_pq_factor_grid(const PanelDesc* __restrict__ desc, int j0,
                                                        double* __restrict__ tau, double* __restrict__ Tout,
                                                        double* __restrict__ part, GridBar gb) {
  __shared__ double red[8 * kPqParts];
  const PanelDesc D = *desc;
  double* A = D.A;
  const int64_t m = D.m, lda = D.lda;
  const int jb = min(kQB, D.k - j0), j1 = j0 + jb;
  const int G = gridDim.x, b = blockIdx.x;
  const int64_t rows = (m + G - 1) / G, r0 = (int64_t)b * rows, r1 = min(m, r0 + rows);
  int phase = 0;
  auto slot = [&]() { return part + (int64_t)(phase & 1) * G * kPqParts; };
  for (int j = j0; j < j1; ++j) {
    double* aj = A + (int64_t)j * lda;
    const bool own_j = (j >= r0 && j < r1);
    // ||x||^2 over rows j+1 .. m-1
    double v[kPqParts];
    v[0] = 0.0;
    // alpha travels in slot 1 from the CTA owning row j (the other CTAs add exact zeros): the
    // owner overwrites A[j][j] with beta once it is past the barrier
    v[1] = (own_j && threadIdx.x == 0) ? aj[j] : 0.0;
    for (int64_t i = max(r0, (int64_t)j + 1) + threadIdx.x; i < r1; i += blockDim.x) v[0] += aj[i] * aj[i];
    cta_parts(v, 2, red, slot() + (int64_t)b * kPqParts);
    if (!grid_barrier(gb)) return;
    const double sig = sum_parts(slot(), G, 0);
    const double alpha = sum_parts(slot(), G, 1);
    ++phase;
    double tj = 0.0, beta = alpha, scal = 0.0;
    if (sig != 0.0) {
      const double nrm = sqrt(alpha * alpha + sig);
      beta = alpha >= 0.0 ? -nrm : nrm;
      tj = (beta - alpha) / beta;
      scal = 1.0 / (alpha - beta);
    }
    __syncthreads();  // every thread has read alpha before its owner overwrites it
    if (own_j && threadIdx.x == 0) aj[j] = beta;
    if (b == 0 && threadIdx.x == 0) tau[j] = tj;
    for (int64_t i = max(r0, (int64_t)j + 1) + threadIdx.x; i < r1; i += blockDim.x) aj[i] *= scal;
    __syncthreads();
    if (tj == 0.0 || j + 1 >= j1) continue;
    // v . A[:, c] for the block's columns c > j (unit entry of v at row j)
    const int nc = j1 - j - 1;
    for (int t = 0; t < nc; ++t) v[t] = 0.0;
    for (int64_t i = max(r0, (int64_t)j + 1) + threadIdx.x; i < r1; i += blockDim.x) {
      const double x = aj[i];
      for (int t = 0; t < nc; ++t) v[t] += x * A[(int64_t)(j + 1 + t) * lda + i];
    }
    if (own_j && threadIdx.x == 0)
      for (int t = 0; t < nc; ++t) v[t] += A[(int64_t)(j + 1 + t) * lda + j];
    cta_parts(v, nc, red, slot() + (int64_t)b * kPqParts);
    if (!grid_barrier(gb)) return;
    double acc[kQB];
    for (int t = 0; t < nc; ++t) acc[t] = sum_parts(slot(), G, t) * tj;
    ++phase;
    for (int64_t i = max(r0, (int64_t)j + 1) + threadIdx.x; i < r1; i += blockDim.x) {
      const double x = aj[i];
      for (int t = 0; t < nc; ++t) A[(int64_t)(j + 1 + t) * lda + i] -= acc[t] * x;
    }
    if (own_j && threadIdx.x == 0)
      for (int t = 0; t < nc; ++t) A[(int64_t)(j + 1 + t) * lda + j] -= acc[t];
    __syncthreads();
  }
  if (j1 >= D.k || Tout == nullptr) return;
  // T of the block (panel_block_T): G[p][q] = v_p[j0+q] + sum_{i > j0+q} v_p[i] v_q[i], p < q
  double v[kPqParts];
  int np = 0;
  for (int q = 1; q < jb; ++q)
    for (int p2 = 0; p2 < q; ++p2) v[np++] = 0.0;
  for (int64_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
    int t = 0;
    for (int q = 1; q < jb; ++q)
      for (int p2 = 0; p2 < q; ++p2, ++t)
        if (i > j0 + q) v[t] += A[(int64_t)(j0 + p2) * lda + i] * A[(int64_t)(j0 + q) * lda + i];
  }
  if (threadIdx.x == 0) {
    int t = 0;
    for (int q = 1; q < jb; ++q)
      for (int p2 = 0; p2 < q; ++p2, ++t)
        if (j0 + q >= r0 && j0 + q < r1) v[t] += A[(int64_t)(j0 + p2) * lda + j0 + q];
  }
  cta_parts(v, np, red, slot() + (int64_t)b * kPqParts);
  if (!grid_barrier(gb)) return;
  if (b != 0 || threadIdx.x != 0) return;
  double Gm[kQB * kQB], Tm[kQB * kQB];
  {
    int t = 0;
    for (int q = 1; q < jb; ++q)
      for (int p2 = 0; p2 < q; ++p2, ++t) Gm[p2 + q * kQB] = sum_parts(slot(), G, t);
  }
  for (int q = 0; q < jb; ++q) {
    const double tq = tau[j0 + q];
    for (int p2 = 0; p2 < q; ++p2) {
      double z = 0.0;
      for (int l = p2; l < q; ++l) z += Tm[p2 + l * kQB] * Gm[l + q * kQB];
      Tm[p2 + q * kQB] = -tq * z;
    }
    Tm[q + q * kQB] = tq;
    for (int p2 = q + 1; p2 < kQB; ++p2) Tm[p2 + q * kQB] = 0.0;
  }
  for (int e = 0; e < kQB * kQB; ++e) Tout[e] = (e % kQB < jb && e / kQB < jb) ? Tm[e] : 0.0;
}

// dorg2r on the block's own columns j0 .. j1-1 of one tall panel by all SMs
__global__ void __launch_bounds__(256) k_pq_form_grid(const PanelDesc* __restrict__ desc, int j0,
                                                      const double* __restrict__ tau, double* __restrict__ part,
                                                      GridBar gb) {
  __shared__ double red[8 * kPqParts];
  const PanelDesc D = *desc;
  double* A = D.A;
  const int64_t m = D.m, lda = D.lda;
  const int j1 = min(j0 + kQB, D.k);
  const int G = gridDim.x, b = blockIdx.x;
  const int64_t rows = (m + G - 1) / G, r0 = (int64_t)b * rows, r1 = min(m, r0 + rows);
  int phase = 0;
  for (int j = j1 - 1; j >= j0; --j) {
    double* aj = A + (int64_t)j * lda;
    const double tj = tau[j];
    const bool own_j = (j >= r0 && j < r1);
    if (j < j1 - 1) {
      // v = e_j + A[j+1:, j]; c <- c - tau (v . c) v for the block's columns c > j
      const int nc = j1 - j - 1;
      double v[kPqParts];
      for (int t = 0; t < nc; ++t) v[t] = 0.0;
      for (int64_t i = max(r0, (int64_t)j + 1) + threadIdx.x; i < r1; i += blockDim.x) {
        const double x = aj[i];
        for (int t = 0; t < nc; ++t) v[t] += x * A[(int64_t)(j + 1 + t) * lda + i];
      }
      if (own_j && threadIdx.x == 0)
        for (int t = 0; t < nc; ++t) v[t] += A[(int64_t)(j + 1 + t) * lda + j];
      double* sl = part + (int64_t)(phase & 1) * G * kPqParts;
      cta_parts(v, nc, red, sl + (int64_t)b * kPqParts);
      if (!grid_barrier(gb)) return;
      double acc[kQB];
      for (int t = 0; t < nc; ++t) acc[t] = sum_parts(sl, G, t) * tj;
      ++phase;
      for (int64_t i = max(r0, (int64_t)j + 1) + threadIdx.x; i < r1; i += blockDim.x) {
        const double x = aj[i];
        for (int t = 0; t < nc; ++t) A[(int64_t)(j + 1 + t) * lda + i] -= acc[t] * x;
      }
      if (own_j && threadIdx.x == 0)
        for (int t = 0; t < nc; ++t) A[(int64_t)(j + 1 + t) * lda + j] -= acc[t];
    }
    for (int64_t i = max(r0, (int64_t)j + 1) + threadIdx.x; i < r1; i += blockDim.x) aj[i] *= -tj;
    for (int64_t i = r0 + threadIdx.x; i < min(r1, (int64_t)j); i += blockDim.x) aj[i] = 0.0;
    if (own_j && threadIdx.x == 0) aj[j] = 1.0 - tj;
    __syncthreads();
  }
}

// explicit reflector block V (rows j0 .. m-1 of columns j0 .. j0+jb-1: unit diagonal, zeros
// above it, the stored vectors below), column-major with leading dimension m - j0
__global__ void k_pq_vcopy(const PanelDesc* __restrict__ desc, int j0, double* __restrict__ V) {
  const PanelDesc D = *desc;
  const int jb = min(kQB, D.k - j0);
  const int64_t mr = D.m - j0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < mr * jb; e += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(e / mr);
    const int64_t i = e - (int64_t)p * mr;
    V[e] = (i == p) ? 1.0 : (i > p ? D.A[(int64_t)(j0 + p) * D.lda + j0 + i] : 0.0);
  }
}

int64_t panel_qr_gemm_scratch(const PanelDesc* hdescs, int n, int kmax) {
  int64_t mbig = 0;
  for (int p = 0; p < n; ++p)
    if (hdescs[p].big) mbig = std::max<int64_t>(mbig, hdescs[p].m);
  return mbig * kQB + 2 * (int64_t)kQB * std::max(kmax, 1) + 2 * 152 * kPqParts + 8 +
         dgemm_scratch(1, kQB, std::max(kmax, 1), mbig);
}

// C[:, j1:k] <- (I - V op(T) V') C[:, j1:k] for big panel p, block j0: W = V' C, W2 = op(T) W,
// C -= V W2 (op(T) = T' while factoring, T while forming Q), then the small panels' blocks by
// k_pq_update
static void panel_block_gemm(const PanelDesc* descs, const PanelDesc& D, int p, int j0, int nblk, const double* Ts,
                             double* scr, int kmax, double* split, int64_t split_len, int transT, cudaStream_t st) {
  const int k = D.k;
  if (j0 >= k) return;
  const int jb = std::min(kQB, k - j0), j1 = j0 + jb;
  const int nt = k - j1;
  if (nt <= 0) return;
  const int64_t mr = D.m - j0;
  double* V = scr;
  double* W = V + mr * kQB;
  double* W2 = W + (int64_t)kQB * kmax;
  const unsigned g = (unsigned)std::min<int64_t>((mr * jb + 255) / 256, 4096);
  k_pq_vcopy<<<g, 256, 0, st>>>(descs + p, j0, V);
  const double* Tm = Ts + ((int64_t)p * nblk + j0 / kQB) * kQB * kQB;
  double* C = D.A + (int64_t)j1 * D.lda + j0;
  launch_dgemm(1, jb, nt, mr, 1.0, V, mr, C, D.lda, 0.0, W, jb, split, split_len, st);
  launch_dgemm(transT, jb, nt, jb, 1.0, Tm, kQB, W, jb, 0.0, W2, jb, nullptr, 0, st);
  launch_dgemm(0, mr, nt, jb, -1.0, V, mr, W2, jb, 1.0, C, D.lda, nullptr, 0, st);
}

// grid size of the cooperative factor / form steps of a tall panel (0: cooperative launch
// unavailable); every CTA must be resident at once
static int pq_grid_size(int64_t m) {
  static int nsm = -1, per = 0;
  if (nsm < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    int coop = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pq_factor_grid, 256, 0) != cudaSuccess ||
        per < 1) {
      cudaGetLastError();
      per = 0;
    }
    int per2 = 0;
    if (per > 0 && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, k_pq_form_grid, 256, 0) != cudaSuccess ||
                    per2 < 1)) {
      cudaGetLastError();
      per = 0;
    }
  }
  if (per == 0) return 0;
  return (int)std::max<int64_t>(1, std::min<int64_t>(nsm, m / 512));
}

void launch_panel_qr_gemm(const PanelDesc* descs, const PanelDesc* hdescs, int n, int kmax, double* taus,
                          double* Ts, double* gemm_scratch, int* grid_err, cudaStream_t st,
                          long long wait_limit) {
  if (n <= 0 || kmax <= 0) return;
  const int nblk = (kmax + kQB - 1) / kQB;
  const int ntiles = (kmax + kQU - 1) / kQU;
  const size_t smu = ((size_t)2 * kQB * kQU + kQC * kQV) * sizeof(double);
  smem_limit((const void*)k_pq_update, smu);
  // scratch after the GEMM buffers: partials of the cooperative steps and the barrier words
  int64_t mbig = 0;
  for (int p = 0; p < n; ++p)
    if (hdescs[p].big) mbig = std::max<int64_t>(mbig, hdescs[p].m);
  double* part = gemm_scratch + mbig * kQB + 2 * (int64_t)kQB * std::max(kmax, 1);
  unsigned* words = reinterpret_cast<unsigned*>(part + 2 * 152 * kPqParts);
  double* split = part + 2 * 152 * kPqParts + 8;  // partial products of the split V'C reductions
  const int64_t split_len = dgemm_scratch(1, kQB, std::max(kmax, 1), mbig);
  cudaMemsetAsync(words, 0, 4 * sizeof(unsigned), st);
  GridBar gb{words, words + 1, grid_err, wait_limit};
  auto factor_big = [&](int p, int b) {
    const int G = pq_grid_size(hdescs[p].m);
    const PanelDesc* dp = descs + p;
    int j0 = b * kQB;
    double* tau = taus + (int64_t)p * kmax;
    double* Tout = Ts + ((int64_t)p * nblk + b) * kQB * kQB;
    if (G > 0 && G <= 152) {
      void* args[] = {(void*)&dp, (void*)&j0, (void*)&tau, (void*)&Tout, (void*)&part, (void*)&gb};
      if (cudaLaunchCooperativeKernel((const void*)k_pq_factor_grid, dim3(G), dim3(256), args, 0, st) == cudaSuccess)
        return;
      cudaGetLastError();
    }
    k_pq_factor<<<1, 512, 0, st>>>(dp, j0, tau, kmax, Ts + (int64_t)p * nblk * kQB * kQB, nblk, 0);
  };
  auto form_big = [&](int p, int b) {
    const int G = pq_grid_size(hdescs[p].m);
    const PanelDesc* dp = descs + p;
    int j0 = b * kQB;
    const double* tau = taus + (int64_t)p * kmax;
    if (G > 0 && G <= 152) {
      void* args[] = {(void*)&dp, (void*)&j0, (void*)&tau, (void*)&part, (void*)&gb};
      if (cudaLaunchCooperativeKernel((const void*)k_pq_form_grid, dim3(G), dim3(256), args, 0, st) == cudaSuccess)
        return;
      cudaGetLastError();
    }
    k_pq_form<<<1, 512, 0, st>>>(dp, j0, tau, kmax, 0);
  };
  for (int b = 0; b < nblk; ++b) {
    k_pq_factor<<<n, 512, 0, st>>>(descs, b * kQB, taus, kmax, Ts, nblk, 1);
    for (int p = 0; p < n; ++p)
      if (hdescs[p].big && b * kQB < hdescs[p].k) factor_big(p, b);
    k_pq_update<<<dim3((unsigned)n, (unsigned)ntiles), 256, smu, st>>>(descs, b * kQB, Ts, nblk, 1);
    for (int p = 0; p < n; ++p)
      if (hdescs[p].big)
        panel_block_gemm(descs, hdescs[p], p, b * kQB, nblk, Ts, gemm_scratch, kmax, split, split_len, 1, st);
  }
  k_pq_rout<<<n, 256, 0, st>>>(descs);
  for (int b = nblk - 1; b >= 0; --b) {
    k_pq_update<<<dim3((unsigned)n, (unsigned)ntiles), 256, smu, st>>>(descs, b * kQB, Ts, nblk, 0);
    for (int p = 0; p < n; ++p)
      if (hdescs[p].big)
        panel_block_gemm(descs, hdescs[p], p, b * kQB, nblk, Ts, gemm_scratch, kmax, split, split_len, 0, st);
    k_pq_form<<<n, 512, 0, st>>>(descs, b * kQB, taus, kmax, 1);
    for (int p = 0; p < n; ++p)
      if (hdescs[p].big && b * kQB < hdescs[p].k) form_big(p, b);
  }
}

int64_t panel_qr_scratch(int n, int kmax) {
  const int nblk = (kmax + kQB - 1) / kQB;
  return (int64_t)n * kmax + (int64_t)n * nblk * kQB * kQB;
}

void launch_gnode(const GNodeDesc* nodes, int n, int* info, cudaStream_t st) {
  k_gnode<<<n, 512, 0, st>>>(nodes, info);
}

void launch_gapply(const GApplyItem* items, int n, const GNodeDesc* nodes, int maxr, int maxcols, int mode,
                   double* X, const double* Xin, int64_t ldX, int kX, cudaStream_t st) {
  if (n <= 0) return;
  dim3 grid((unsigned)n, (unsigned)((maxcols + 7) / 8));
  const size_t sm = (size_t)8 * 3 * std::max(maxr, 1) * sizeof(double);
  smem_limit((const void*)k_gapply, sm);
  k_gapply<<<grid, 256, sm, st>>>(items, nodes, mode, X, Xin, ldX, kX);
}

void launch_gsmall(const GNodeDesc* node, int mode, const double* Z1, const double* Z2, double* G1, double* G2,
                   int r, int ncols, cudaStream_t st) {
  if (ncols <= 0 || r <= 0) return;
  const size_t sm = (size_t)3 * r * sizeof(double);
  smem_limit((const void*)k_gsmall, sm);
  k_gsmall<<<(unsigned)ncols, 32, sm, st>>>(node, mode, Z1, Z2, G1, G2);
}

void launch_glogdet(const GNodeDesc* nodes, int nn, double* partial, cudaStream_t st) {
  k_glogdet<<<(nn + 127) / 128, 128, 0, st>>>(nodes, nn, partial);
}

}  // namespace km
