// k-d ordering of 2-D points on the GPU (the input step of the path, maxlikdata,
// src/HODLR/src/constructor.jl:171-181, and data_reorder, src/utils.jl:22-25).
//
// The reference orders points with NearestNeighbors.KDTree(pts).data, whose exact permutation
// belongs to that package.  This library defines its own deterministic ordering and computes it
// here: a segment of more than `leaf` points is sorted stably by its coordinate of larger spread
// (max - min; x when the spreads are equal), its first floor(len/2) points form the left child
// and the rest the right child, and both children are ordered the same way in place; a segment
// of at most `leaf` points keeps the order its parent's sort gave it.
//
// GPU form, level-synchronous: at each level every segment (a contiguous range of positions) is
// either split or final.  (1) one CTA per segment to be split reduces min/max of x and y of its
// points and picks the axis; (2) every position gets a 64-bit key, the order-preserving bits of
// its coordinate on that axis (0 in final segments); (3) a stable LSD radix sort by (segment,
// key), 8-bit digits, carries the permutation along.  Stability makes equal coordinates keep
// their current order, as a stable sort does, and final segments keep theirs.
#include <algorithm>
#include <vector>

#include "km_kernels.h"

namespace km {

namespace {

constexpr int kChunk = 2048;  // positions per CTA in the radix passes
constexpr int kRadixThreads = 256;

// order-preserving map from a finite double to uint64 (-0.0 is taken as +0.0, so the two
// compare equal as they do for a sort on doubles)
__device__ __forceinline__ uint64_t order_bits(double v) {
  if (v == 0.0) v = 0.0;
  const uint64_t u = static_cast<uint64_t>(__double_as_longlong(v));
  return (u >> 63) ? ~u : (u | (uint64_t(1) << 63));
}

__device__ __forceinline__ uint32_t digit_of(uint64_t key, uint32_t seg, int pass) {
  return pass < 8 ? static_cast<uint32_t>(key >> (8 * pass)) & 255u
                  : (seg >> (8 * (pass - 8))) & 255u;
}

// segment id of every position (one CTA per segment)
__global__ void k_seg_fill(const KdSeg* __restrict__ segs, uint32_t* __restrict__ seg_of) {
  const KdSeg s = segs[blockIdx.x];
  for (int64_t i = threadIdx.x; i < s.len; i += blockDim.x) seg_of[s.start + i] = blockIdx.x;
}

// axis of every segment to be split: 0 when max-min of x >= max-min of y (one CTA per segment)
__global__ void k_seg_axis(const KdSeg* __restrict__ segs, const double* __restrict__ pts,
                           const int64_t* __restrict__ perm, int* __restrict__ axis) {
  const KdSeg s = segs[blockIdx.x];
  if (!s.split) return;
  double mnx = 0.0, mxx = 0.0, mny = 0.0, mxy = 0.0;
  bool any = false;
  for (int64_t i = threadIdx.x; i < s.len; i += blockDim.x) {
    const int64_t q = perm[s.start + i];
    const double x = pts[2 * q], y = pts[2 * q + 1];
    if (!any) {
      mnx = mxx = x;
      mny = mxy = y;
      any = true;
    } else {
      mnx = fmin(mnx, x);
      mxx = fmax(mxx, x);
      mny = fmin(mny, y);
      mxy = fmax(mxy, y);
    }
  }
  __shared__ double red[4][32];
  __shared__ int anyw[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // warp reduction carrying "has a value"
  for (int o = 16; o > 0; o >>= 1) {
    const double a = __shfl_xor_sync(0xffffffffu, mnx, o), b = __shfl_xor_sync(0xffffffffu, mxx, o);
    const double c = __shfl_xor_sync(0xffffffffu, mny, o), d = __shfl_xor_sync(0xffffffffu, mxy, o);
    const bool oa = __shfl_xor_sync(0xffffffffu, any, o);
    if (oa) {
      if (!any) {
        mnx = a;
        mxx = b;
        mny = c;
        mxy = d;
        any = true;
      } else {
        mnx = fmin(mnx, a);
        mxx = fmax(mxx, b);
        mny = fmin(mny, c);
        mxy = fmax(mxy, d);
      }
    }
  }
  if (lane == 0) {
    red[0][w] = mnx;
    red[1][w] = mxx;
    red[2][w] = mny;
    red[3][w] = mxy;
    anyw[w] = any;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    bool f = false;
    for (int q = 0; q < nw; ++q) {
      if (!anyw[q]) continue;
      if (!f) {
        mnx = red[0][q];
        mxx = red[1][q];
        mny = red[2][q];
        mxy = red[3][q];
        f = true;
      } else {
        mnx = fmin(mnx, red[0][q]);
        mxx = fmax(mxx, red[1][q]);
        mny = fmin(mny, red[2][q]);
        mxy = fmax(mxy, red[3][q]);
      }
    }
    axis[blockIdx.x] = (mxx - mnx >= mxy - mny) ? 0 : 1;
  }
}

__global__ void k_make_keys(const KdSeg* __restrict__ segs, const uint32_t* __restrict__ seg_of,
                            const int* __restrict__ axis, const double* __restrict__ pts,
                            const int64_t* __restrict__ perm, uint64_t* __restrict__ key, int64_t n) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t s = seg_of[p];
    key[p] = segs[s].split ? order_bits(pts[2 * perm[p] + axis[s]]) : 0;
  }
}

// digit counts of each chunk: hist[digit * nblocks + chunk]
__global__ void k_radix_hist(const uint64_t* __restrict__ key, const uint32_t* __restrict__ seg, int64_t n,
                             int pass, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  for (int d = threadIdx.x; d < 256; d += blockDim.x) h[d] = 0;
  __syncthreads();
  const int64_t b0 = (int64_t)blockIdx.x * kChunk;
  for (int i = threadIdx.x; i < kChunk; i += blockDim.x) {
    const int64_t e = b0 + i;
    if (e < n) atomicAdd(&h[digit_of(key[e], seg[e], pass)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[(int64_t)d * gridDim.x + blockIdx.x] = h[d];
}

// exclusive prefix sum of `len` counts in place, one CTA of 1024 threads
__global__ void k_exclusive_scan(uint32_t* __restrict__ a, int64_t len) {
  __shared__ uint32_t part[1024];
  const int tid = threadIdx.x;
  const int64_t per = (len + blockDim.x - 1) / blockDim.x;
  const int64_t lo = tid * per, hi = (lo + per < len) ? lo + per : len;
  uint32_t s = 0;
  for (int64_t i = lo; i < hi; ++i) s += a[i];
  part[tid] = s;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {  // inclusive Hillis-Steele scan of the parts
    const uint32_t v = tid >= o ? part[tid - o] : 0u;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  uint32_t run = part[tid] - s;  // exclusive
  for (int64_t i = lo; i < hi; ++i) {
    const uint32_t v = a[i];
    a[i] = run;
    run += v;
  }
}

// stable scatter of one pass: positions are taken in order, 256 at a time; equal digits keep
// their order through the warp match masks and the per-warp counts
__global__ void __launch_bounds__(kRadixThreads) k_radix_scatter(
    const uint64_t* __restrict__ kin, const uint32_t* __restrict__ sin, const int64_t* __restrict__ pin,
    uint64_t* __restrict__ kout, uint32_t* __restrict__ sout, int64_t* __restrict__ pout, int64_t n, int pass,
    const uint32_t* __restrict__ offs) {
  __shared__ uint32_t run[256];
  __shared__ uint32_t wcnt[kRadixThreads / 32][256];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int d = tid; d < 256; d += kRadixThreads) run[d] = offs[(int64_t)d * gridDim.x + blockIdx.x];
  const int64_t b0 = (int64_t)blockIdx.x * kChunk;
  for (int sub = 0; sub < kChunk; sub += kRadixThreads) {
    for (int e = tid; e < (kRadixThreads / 32) * 256; e += kRadixThreads) (&wcnt[0][0])[e] = 0;
    __syncthreads();
    const int64_t e = b0 + sub + tid;
    const bool valid = e < n;
    uint64_t k = 0;
    uint32_t s = 0;
    int64_t p = 0;
    uint32_t dig = 256u;  // out-of-range positions form their own group and write nothing
    if (valid) {
      k = kin[e];
      s = sin[e];
      p = pin[e];
      dig = digit_of(k, s, pass);
    }
    const unsigned mask = __match_any_sync(0xffffffffu, dig);
    const int rank = __popc(mask & ((1u << lane) - 1u));
    if (valid && rank == 0) wcnt[w][dig] = __popc(mask);
    __syncthreads();
    if (valid) {
      uint32_t before = 0;
      for (int q = 0; q < w; ++q) before += wcnt[q][dig];
      const uint32_t pos = run[dig] + before + rank;
      kout[pos] = k;
      sout[pos] = s;
      pout[pos] = p;
    }
    __syncthreads();
    for (int d = tid; d < 256; d += kRadixThreads) {
      uint32_t t = 0;
      for (int q = 0; q < kRadixThreads / 32; ++q) t += wcnt[q][d];
      run[d] += t;
    }
    __syncthreads();
  }
}

__global__ void k_iota64(int64_t* __restrict__ p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = i;
}

__global__ void k_gather_sorted(const double* __restrict__ pts, const double* __restrict__ data,
                                const int64_t* __restrict__ perm, int64_t n, double* __restrict__ pts_s,
                                double* __restrict__ data_s) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = perm[i];
    pts_s[2 * i] = pts[2 * q];
    pts_s[2 * i + 1] = pts[2 * q + 1];
    if (data) data_s[i] = data[q];
  }
}

}  // namespace

// the scratch pieces, in the order kd_order_device carves them, each rounded up to 256 bytes
static size_t kd_piece(size_t bytes) { return (bytes + 255) & ~size_t(255); }

size_t kd_scratch_bytes(int64_t n) {
  const int64_t nb = (n + kChunk - 1) / kChunk;
  return 2 * kd_piece(n * sizeof(uint64_t))        // keys
         + 2 * kd_piece(n * sizeof(uint32_t))      // segment ids
         + kd_piece(n * sizeof(int64_t))           // second permutation buffer
         + kd_piece(nb * 256 * sizeof(uint32_t))   // digit histograms
         + kd_piece(n * sizeof(KdSeg))             // segments (at most one per position)
         + kd_piece(n * sizeof(int));              // split axes
}

// Fills d_perm (n) with the k-d ordering of the n points d_pts (AoS x, y).  d_scratch holds
// kd_scratch_bytes(n) bytes.  Segment lists are formed on the host, level by level.
bool kd_order_device(const double* d_pts, int64_t n, int64_t leaf, int64_t* d_perm, void* d_scratch,
                     cudaStream_t st, std::string* err) {
  if (n < 1 || leaf < 1) {
    *err = "bad k-d ordering arguments";
    return false;
  }
  char* sp = static_cast<char*>(d_scratch);
  auto take = [&](size_t bytes) {
    char* p = sp;
    sp += kd_piece(bytes);
    return p;
  };
  const int64_t nb = (n + kChunk - 1) / kChunk;
  uint64_t* key0 = reinterpret_cast<uint64_t*>(take(n * sizeof(uint64_t)));
  uint64_t* key1 = reinterpret_cast<uint64_t*>(take(n * sizeof(uint64_t)));
  uint32_t* seg0 = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
  uint32_t* seg1 = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
  int64_t* perm1 = reinterpret_cast<int64_t*>(take(n * sizeof(int64_t)));
  uint32_t* hist = reinterpret_cast<uint32_t*>(take(nb * 256 * sizeof(uint32_t)));
  KdSeg* dsegs = reinterpret_cast<KdSeg*>(take(n * sizeof(KdSeg)));
  int* daxis = reinterpret_cast<int*>(take(n * sizeof(int)));
  if ((size_t)(sp - static_cast<char*>(d_scratch)) > kd_scratch_bytes(n)) {
    *err = "k-d scratch too small";
    return false;
  }
  k_iota64<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(d_perm, n);
  std::vector<KdSeg> segs{KdSeg{0, n, n > leaf ? 1 : 0}};
  int64_t* pcur = d_perm;
  int64_t* palt = perm1;
  std::vector<KdSeg> next;
  for (;;) {
    bool any_split = false;
    for (const KdSeg& s : segs) any_split |= s.split != 0;
    if (!any_split) break;
    const int64_t nseg = (int64_t)segs.size();
    cudaMemcpyAsync(dsegs, segs.data(), nseg * sizeof(KdSeg), cudaMemcpyHostToDevice, st);
    k_seg_fill<<<(unsigned)nseg, 256, 0, st>>>(dsegs, seg0);
    k_seg_axis<<<(unsigned)nseg, 256, 0, st>>>(dsegs, d_pts, pcur, daxis);
    k_make_keys<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(dsegs, seg0, daxis, d_pts, pcur,
                                                                                    key0, n);
    const int segbytes = nseg <= 1 ? 0 : (nseg <= 256 ? 1 : (nseg <= 65536 ? 2 : (nseg <= (1 << 24) ? 3 : 4)));
    uint64_t* kc = key0;
    uint64_t* ka = key1;
    uint32_t* sc = seg0;
    uint32_t* sa = seg1;
    for (int pass = 0; pass < 8 + segbytes; ++pass) {
      k_radix_hist<<<(unsigned)nb, 256, 0, st>>>(kc, sc, n, pass, hist);
      k_exclusive_scan<<<1, 1024, 0, st>>>(hist, nb * 256);
      k_radix_scatter<<<(unsigned)nb, kRadixThreads, 0, st>>>(kc, sc, pcur, ka, sa, palt, n, pass, hist);
      std::swap(kc, ka);
      std::swap(sc, sa);
      std::swap(pcur, palt);
    }
    // the next level's segments
    next.clear();
    for (const KdSeg& s : segs) {
      if (!s.split) {
        next.push_back(s);
        continue;
      }
      const int64_t h = s.len / 2;
      next.push_back(KdSeg{s.start, h, h > leaf ? 1 : 0});
      next.push_back(KdSeg{s.start + h, s.len - h, (s.len - h) > leaf ? 1 : 0});
    }
    segs.swap(next);
  }
  if (pcur != d_perm) cudaMemcpyAsync(d_perm, pcur, n * sizeof(int64_t), cudaMemcpyDeviceToDevice, st);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    *err = std::string("k-d ordering: ") + cudaGetErrorString(e);
    return false;
  }
  return true;
}

void launch_gather_sorted(const double* pts, const double* data, const int64_t* perm, int64_t n, double* pts_s,
                          double* data_s, cudaStream_t st) {
  k_gather_sorted<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(pts, data, perm, n, pts_s,
                                                                                      data_s);
}

}  // namespace km
