// Kernel-entry evaluation: dense leaves, the Nystrom landmark columns Phi = K(X, P) and the
// landmark matrix S = K(P, P).  Replaces the comprehension in getindex/full
// (src/baseoverloads.jl:10-29) that KernelHODLR calls for every leaf (src/HODLR/src/
// constructor.jl:39) and nystrom_uvt calls for every block (src/factorizations.jl:86-94).
//
// Layouts (device):
//   points   : 2n doubles, (x, y) pairs (AoS, the SVector{2,Float64} layout)
//   leaves   : packed m_j x m_j column-major blocks at d_leaf_koff(j)
//   panels   : per-leaf m_j x r column-major blocks at leaf_start(j) * r
#include <algorithm>

#include "km_kernels.h"
#include "km_kfun.cuh"

namespace km {

// One 32x32 tile of one leaf per CTA; only lower-triangle tiles are evaluated and each is
// written twice (the kernel is symmetric bit for bit: |x-y| and x == y are symmetric).
// Kff (the kernel itself in float pairs, may be null): the entries of the evaluated tiles
// (every lower-triangle entry) also as float pairs, for the tensor-core leaf factorisation,
// evaluated on the split coordinates P3; the same kernel on the same points always gives the
// same pairs.  grid = (ntile, ntile, nleaf), block = (32, 8).
__global__ void k_eval_leaves(const double* __restrict__ pts, const float* __restrict__ P3, DTree t, KParams kp,
                              int deriv, bool use_ff, double* __restrict__ K, ff* __restrict__ Kff) {
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (ti < tj) return;
  const int64_t leaf = blockIdx.z;
  const int m = d_leaf_size(t, leaf);
  if (ti * 32 >= m) return;
  const int64_t s = d_leaf_start(t, leaf);
  double* A = K + d_leaf_koff(t, leaf);
  __shared__ double px[2][32], py[2][32];
  __shared__ double tile[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * 32 + tx;
  if (tid < 64) {
    const int which = tid >> 5, q = tid & 31;
    const int idx = (which == 0 ? ti : tj) * 32 + q;
    if (idx < m) {
      px[which][q] = pts[2 * (s + idx)];
      py[which][q] = pts[2 * (s + idx) + 1];
    }
  }
  __syncthreads();
  const int i = ti * 32 + tx;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int jl = ty + 8 * q;
    const int j = tj * 32 + jl;
    if (i < m && j < m) {
      double v;
      if (Kff) {
        f3 x1, y1, x2, y2;
        if (P3) {
          load_p3(P3, s + i, x1, y1);
          load_p3(P3, s + j, x2, y2);
        } else {
          x1 = split3(px[0][tx]);
          y1 = split3(py[0][tx]);
          x2 = split3(px[1][jl]);
          y2 = split3(py[1][jl]);
        }
        ff f = kernel_value_ffp(kp, x1, y1, x2, y2);
        v = to_double(f);
        if (eq3(x1, x2) && eq3(y1, y2)) {  // the diagonal: the FP64 sum with the nugget, rounded to a pair
          v = __dadd_rn(v, kp.p2);
          f = ff(v);
        }
        Kff[d_leaf_koff(t, leaf) + (int64_t)j * m + i] = f;
      } else {
        v = eval_entry(use_ff, kp, deriv, px[0][tx], py[0][tx], px[1][jl], py[1][jl]);
      }
      A[(int64_t)j * m + i] = v;
      tile[tx][jl] = v;
    }
  }
  if (ti == tj) return;
  __syncthreads();
  // mirrored write: element (row = tj*32+tx, col = ti*32+ty+8q) = tile[ty+8q][tx]
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int il = ty + 8 * q;
    const int row = tj * 32 + tx, col = ti * 32 + il;
    if (row < m && col < m) A[(int64_t)col * m + row] = tile[il][tx];
  }
}

// Phi[i, c] = k(x_i, p_c) for every point i and landmark c, stored per leaf column-major; the
// float-pair kernel (use_ff, deriv < 0) on the split coordinates P3 and L3, whose pairs also go
// to Phif when given (the same values as the FP64 copy rounded back to pairs).
// grid = (ceil(maxleaf*r / 256), nleaf), block = 256.
__global__ void k_eval_phi(const double* __restrict__ pts, const double* __restrict__ lnd,
                           const float* __restrict__ P3, const float* __restrict__ L3, int r,
                           DTree t, KParams kp, int deriv, bool use_ff, double* __restrict__ Phi,
                           ff* __restrict__ Phif) {
  extern __shared__ double sl[];  // 2r
  for (int q = threadIdx.x; q < 2 * r; q += blockDim.x) sl[q] = lnd[q];
  __syncthreads();
  const int64_t leaf = blockIdx.y;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)m * r) return;
  const int c = (int)(e / m), i = (int)(e % m);
  if (use_ff && deriv < 0 && P3) {
    f3 x1, y1, x2, y2;
    load_p3(P3, s + i, x1, y1);
    load_p3(L3, c, x2, y2);
    ff f = kernel_value_ffp(kp, x1, y1, x2, y2);
    double v = to_double(f);
    if (eq3(x1, x2) && eq3(y1, y2)) {
      v = __dadd_rn(v, kp.p2);
      f = ff(v);
    }
    Phi[s * r + (int64_t)c * m + i] = v;
    if (Phif) Phif[s * r + (int64_t)c * m + i] = f;
    return;
  }
  const double x = pts[2 * (s + i)], y = pts[2 * (s + i) + 1];
  Phi[s * r + (int64_t)c * m + i] = eval_entry(use_ff, kp, deriv, x, y, sl[2 * c], sl[2 * c + 1]);
}

// P3[8 i .. 8 i + 7] = (split3(x_i), split3(y_i), 0, 0) for n points.
__global__ void k_split_points(const double* __restrict__ pts, int64_t n, float* __restrict__ P3) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const f3 x = split3(pts[2 * i]), y = split3(pts[2 * i + 1]);
    float4* o = reinterpret_cast<float4*>(P3 + 8 * i);
    o[0] = make_float4(x.h, x.m, x.l, y.h);
    o[1] = make_float4(y.m, y.l, 0.f, 0.f);
  }
}

// Dense block out[i + j*ld] = k(a_i, b_j) (or its derivative) for small matrices such as S.
__global__ void k_eval_dense(const double* __restrict__ a, int na, const double* __restrict__ b,
                             int nb, KParams kp, int deriv, double* __restrict__ out, int ld) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= na * nb) return;
  const int i = e % na, j = e / na;
  const double v = eval_entry(false, kp, deriv, a[2 * i], a[2 * i + 1], b[2 * j], b[2 * j + 1]);
  out[i + (int64_t)j * ld] = v;
}

// Gathers the landmark points lnd[c] = pts[idx[c]].
__global__ void k_gather_points(const double* __restrict__ pts, const int64_t* __restrict__ idx,
                                int r, double* __restrict__ lnd) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < r) {
    lnd[2 * c] = pts[2 * idx[c]];
    lnd[2 * c + 1] = pts[2 * idx[c] + 1];
  }
}

void launch_eval_leaves(const double* pts, const Tree& t, KParams kp, int deriv, double* K,
                        cudaStream_t st, bool use_ff, ff* Kff, const float* P3) {
  const int nt = (int)((t.max_leaf + 31) / 32);
  dim3 grid(nt, nt, (unsigned)t.nleaf), block(32, 8);
  k_eval_leaves<<<grid, block, 0, st>>>(pts, P3, dtree(t), kp, deriv, use_ff, K,
                                        (use_ff && deriv < 0) ? Kff : nullptr);
}

void launch_eval_phi(const double* pts, const double* lnd, int r, const Tree& t, KParams kp,
                     int deriv, double* Phi, cudaStream_t st, bool use_ff, const float* P3, const float* L3,
                     ff* Phif) {
  const int64_t per = t.max_leaf * r;
  dim3 grid((unsigned)((per + 255) / 256), (unsigned)t.nleaf);
  k_eval_phi<<<grid, 256, 2 * r * sizeof(double), st>>>(pts, lnd, P3, L3, r, dtree(t), kp, deriv, use_ff, Phi,
                                                         (use_ff && deriv < 0 && P3) ? Phif : nullptr);
}

void launch_split_points(const double* pts, int64_t n, float* P3, cudaStream_t st) {
  if (n <= 0) return;
  k_split_points<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(pts, n, P3);
}

void launch_eval_dense(const double* a, int na, const double* b, int nb, KParams kp, int deriv,
                       double* out, int ld, cudaStream_t st) {
  const int tot = na * nb;
  k_eval_dense<<<(tot + 255) / 256, 256, 0, st>>>(a, na, b, nb, kp, deriv, out, ld);
}

void launch_gather_points(const double* pts, const int64_t* idx, int r, double* lnd,
                          cudaStream_t st) {
  k_gather_points<<<(r + 127) / 128, 128, 0, st>>>(pts, idx, r, lnd);
}

}  // namespace km
