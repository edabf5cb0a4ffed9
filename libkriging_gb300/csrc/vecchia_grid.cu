// vecchia_grid.cu -- exact Vecchia ordering and neighbour sets on uniform grids, O(n log n) work instead of O(n^2).
//
// Definition (Kriging::make_vecchia_sets, src/lib/Kriging.cpp:736-804): the order starts at the point closest to the
// centroid and then repeatedly takes the point whose smallest squared distance to the points already ordered is
// largest (argmax ties to the lowest index); the neighbours of the point at position t are its min(m, t) nearest
// points among positions 0 .. t - 1, by (squared distance, index).  Squared distances are sums of (a_k - b_k)^2
// rounded term by term, as the reference's loop computes them (no fused multiply-add).
//
// Maxmin order.  The points are counting-sorted into the cells of a uniform grid.  When point p is taken with
// running distance r2 = mind2[p] (the current maximum), only points q with d2(q, p) < mind2[q] <= r2 change, so only
// the cells that intersect the cube of half-width sqrt(r2) around p are visited: a few cells per step once the
// ordering has covered the domain.  The argmax runs on a two-level 64-ary tournament tree in shared memory (level 1
// holds one (max, index) per 64 grid slots, level 2 one per 64 level-1 nodes) that is updated only where distances
// changed.  One CTA runs the steps one after another (each needs the previous argmax); a launch runs a bounded
// number of steps and rebuilds the tree from the distances it left behind.  The cell range of a query is computed
// with the same monotone floating-point map as the cells of the points, with a 1e-12 relative margin on the radius,
// so every point that can change lies in a visited cell.
//
// Neighbour sets.  For the points at positions t in (2^(j-1), 2^j] a grid over the first 2^j ordered points (about
// two per cell) holds at least half earlier points, so a ring-by-ring search around the query's cell finds the m
// nearest earlier points after O(m) visited points; it stops once the m-th best squared distance is below the
// squared distance to the next ring of cells (minus a margin for the cell rounding).  Positions t <= 2048 scan the
// earlier points directly.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "stats.hpp"
#include "vecchia.hpp"

namespace lkg {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int MAXD = 8;
constexpr int G1 = 64;                 // grid slots per level-1 node
constexpr int NG1_MAX = 16384;         // level-1 nodes in shared memory (n <= 2^20 at G1 = 64; larger n widens G1)
constexpr int NG2_MAX = 256;           // level-2 nodes (64 level-1 nodes each)
constexpr int LIST_MAX = 2048;         // dirty level-1 nodes tracked per step; more -> every node is rebuilt
constexpr int MM_THREADS = 1024;
constexpr int KNN_BRUTE = 2048;        // positions up to this scan the earlier points directly
constexpr double RADIUS_MARGIN = 1e-12;

struct GridDesc {
  int d;
  int G[MAXD];          // cells per dimension
  long long stride[MAXD];
  double lo[MAXD], inv_h[MAXD];
  double h_min;         // smallest cell width
  double slack;         // absolute margin for the rounding of the cell map
};

__device__ __forceinline__ int cell_coord(const GridDesc& g, int k, double x) {
  const double f = (x - g.lo[k]) * g.inv_h[k];  // monotone in x: the same map for points and query bounds
  int c = (f >= 0.0) ? (int)fmin(f, 2.0e9) : 0;
  return c < 0 ? 0 : (c >= g.G[k] ? g.G[k] - 1 : c);
}

__device__ __forceinline__ double sqdist(const double* a, const double* b, int d) {
  double s = 0.0;
  for (int k = 0; k < d; ++k) {
    const double dk = __dsub_rn(a[k], b[k]);
    s = __dadd_rn(s, __dmul_rn(dk, dk));
  }
  return s;
}

// (value, index) pairs: larger value wins, ties to the lower index.  Values are running squared distances (>= 0,
// +inf before the first step, -inf once ordered); for these, the IEEE bit patterns read as signed 64-bit integers
// order exactly like the doubles, so the tree compares integers (FP64 throughput is scarce on this part).
__device__ __forceinline__ long long key_of(double v) { return __double_as_longlong(v); }
__device__ __forceinline__ bool beats(long long v, int i, long long bv, int bi) { return v > bv || (v == bv && i < bi); }

__device__ __forceinline__ void warp_argmax(long long& v, int& i) {
  for (int o = 16; o > 0; o >>= 1) {
    const long long ov = __shfl_xor_sync(FULL, v, o);
    const int oi = __shfl_xor_sync(FULL, i, o);
    if (beats(ov, oi, v, i)) {
      v = ov;
      i = oi;
    }
  }
}

// ------------------------------------------------------------------------------------------------ grid building
__global__ void k_grid_cells(int n, const double* __restrict__ P, int pstride_pts, GridDesc g, int* __restrict__ cell,
                             int* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  long long c = 0;
  for (int k = 0; k < g.d; ++k) c += (long long)cell_coord(g, k, P[(int64_t)i * pstride_pts + k]) * g.stride[k];
  cell[i] = (int)c;
  atomicAdd(&count[c], 1);
}

// exclusive scan of a[0 .. len) in place, one block, 1024 threads, len any size (sequential chunks)
__global__ void __launch_bounds__(1024) k_scan_exclusive(int len, int* __restrict__ a, int* __restrict__ total) {
  __shared__ int warp_sums[32];
  __shared__ int carry_s;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int base = 0; base < len; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < len ? a[i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
      int s = warp_sums[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, s, o);
        if (lane >= o) s += y;
      }
      warp_sums[lane] = s;
    }
    __syncthreads();
    const int carry = carry_s;
    const int incl = x + (w > 0 ? warp_sums[w - 1] : 0) + carry;
    if (i < len) a[i] = incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry_s = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry_s;
}

// slot of every point: cursor starts as a copy of cell_start
__global__ void k_grid_scatter(int n, const int* __restrict__ cell, int* __restrict__ cursor, int* __restrict__ perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  perm[atomicAdd(&cursor[cell[i]], 1)] = i;
}

// slot arrays of the maxmin grid: coordinates, original index, slot of every point, running distance = +inf
__global__ void k_grid_slots(int n, int d, const double* __restrict__ Xp, const int* __restrict__ perm,
                             double* __restrict__ Xs, int* __restrict__ orig, int* __restrict__ slot_of,
                             double* __restrict__ dist) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int i = perm[s];
  for (int k = 0; k < d; ++k) Xs[(int64_t)s * d + k] = Xp[(int64_t)i * d + k];
  orig[s] = i;
  slot_of[i] = s;
  dist[s] = INFINITY;
}

// ------------------------------------------------------------------------------------------------ maxmin steps
struct MaxminArgs {
  int n, d, t0, t1, first, g1;  // steps [t0, t1); t0 == 0 takes `first` with an infinite radius
  int ng1, ng2;
  GridDesc g;
  const int* cell_start;
  const double* Xs;
  const int* orig;
  const int* slot_of;
  double* dist;
  int* order;
};

__global__ void __launch_bounds__(MM_THREADS, 1) k_maxmin_grid(MaxminArgs a) {
  extern __shared__ long long mm_smem[];
  long long* l1v = mm_smem;                                  // ng1 keys
  int* l1i = reinterpret_cast<int*>(l1v + a.ng1);            // ng1
  long long* l2v = reinterpret_cast<long long*>(l1i + ((a.ng1 + 1) & ~1));
  int* l2i = reinterpret_cast<int*>(l2v + NG2_MAX);          // 256
  unsigned* dirty1 = reinterpret_cast<unsigned*>(l2i + NG2_MAX);  // ng1 bits
  int* list1 = reinterpret_cast<int*>(dirty1 + NG1_MAX / 32);     // LIST_MAX
  __shared__ unsigned dirty2[NG2_MAX / 32];
  __shared__ int nlist1, overflow;
  // the step's scalars, computed by warp 0 and read by every warp: the point taken, its slot and coordinates, and
  // the range of cells that can hold a changing point
  __shared__ int st_snext, st_clo[MAXD], st_chi[MAXD], st_rows;
  __shared__ double st_xn[MAXD];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = MM_THREADS / 32;
  const int d = a.d, n = a.n, gs = a.g1, per = gs / 32;

  auto mark_dirty = [&](int gidx) {
    const unsigned bit = 1u << (gidx & 31);
    if (!(atomicOr(&dirty1[gidx >> 5], bit) & bit)) {
      const int pos = atomicAdd(&nlist1, 1);
      if (pos < LIST_MAX)
        list1[pos] = gidx;
      else
        overflow = 1;
    }
  };
  // level-1 node g: argmax of dist over slots [g gs, (g + 1) gs), ties to the lowest original index
  auto reduce_l1 = [&](int gidx) {
    long long bv = LLONG_MIN;
    int bi = 0x7fffffff;
    for (int q = 0; q < per; ++q) {
      const int s = gidx * gs + q * 32 + lane;
      if (s < n) {
        const long long v = key_of(a.dist[s]);
        const int i = a.orig[s];
        if (beats(v, i, bv, bi)) {
          bv = v;
          bi = i;
        }
      }
    }
    warp_argmax(bv, bi);
    if (lane == 0) {
      l1v[gidx] = bv;
      l1i[gidx] = bi;
    }
  };
  auto reduce_l2 = [&](int gidx) {
    long long bv = LLONG_MIN;
    int bi = 0x7fffffff;
    for (int q = 0; q < 2; ++q) {
      const int c = gidx * 64 + q * 32 + lane;
      if (c < a.ng1 && beats(l1v[c], l1i[c], bv, bi)) {
        bv = l1v[c];
        bi = l1i[c];
      }
    }
    warp_argmax(bv, bi);
    if (lane == 0) {
      l2v[gidx] = bv;
      l2i[gidx] = bi;
    }
  };

  // rebuild the tree from the distances of the previous launch
  for (int gidx = w; gidx < a.ng1; gidx += nw) reduce_l1(gidx);
  for (int q = tid; q < NG1_MAX / 32; q += MM_THREADS) dirty1[q] = 0u;
  if (tid < NG2_MAX / 32) dirty2[tid] = 0u;
  if (tid == 0) {
    nlist1 = 0;
    overflow = 0;
  }
  __syncthreads();
  for (int gidx = w; gidx < a.ng2; gidx += nw) reduce_l2(gidx);
  __syncthreads();

  for (int t = a.t0; t < a.t1; ++t) {
    // (a) warp 0: the next point (the root of the tree) and the cells that can hold a changing point
    if (w == 0) {
      int next;
      double r2;
      if (t == 0) {
        next = a.first;
        r2 = INFINITY;
      } else {
        long long bv = LLONG_MIN;
        int bi = 0x7fffffff;
        for (int c = lane; c < a.ng2; c += 32)
          if (beats(l2v[c], l2i[c], bv, bi)) {
            bv = l2v[c];
            bi = l2i[c];
          }
        warp_argmax(bv, bi);
        next = bi;
        r2 = __longlong_as_double(bv);
      }
      const int snext = a.slot_of[next];
      const bool all = !(r2 < INFINITY);
      double r = 0.0;
      if (lane == 0 && !all) r = sqrt(r2) * (1.0 + RADIUS_MARGIN);
      r = __shfl_sync(FULL, r, 0);
      if (lane < d) {
        const double x = a.Xs[(int64_t)snext * d + lane];
        st_xn[lane] = x;
        st_clo[lane] = all ? 0 : cell_coord(a.g, lane, x - r);
        st_chi[lane] = all ? a.g.G[lane] - 1 : cell_coord(a.g, lane, x + r);
      }
      __syncwarp();
      if (lane == 0) {
        int rows = 1;
        for (int k = 1; k < d; ++k) rows *= (st_chi[k] - st_clo[k] + 1);
        st_rows = rows;
        st_snext = snext;
        a.order[t] = next;
        a.dist[snext] = -INFINITY;
        mark_dirty(snext / gs);
      }
    }
    __syncthreads();
    // (b) distance updates, one warp per row of cells along dimension 0 (contiguous slots)
    {
      const int snext = st_snext, rows = st_rows;
      double xn[MAXD];
      for (int k = 0; k < d; ++k) xn[k] = st_xn[k];
      for (int rho = w; rho < rows; rho += nw) {
        int rem = rho;
        long long cbase = st_clo[0];
        for (int k = 1; k < d; ++k) {
          const int span = st_chi[k] - st_clo[k] + 1;
          cbase += (long long)(st_clo[k] + rem % span) * a.g.stride[k];
          rem /= span;
        }
        const int s0 = a.cell_start[cbase], s1 = a.cell_start[cbase + (st_chi[0] - st_clo[0]) + 1];
        for (int s = s0 + lane; s < s1; s += 32) {
          if (s == snext) continue;
          const long long dv = key_of(a.dist[s]);
          if (dv < 0) continue;  // already ordered (-inf)
          const double d2 = sqdist(a.Xs + (int64_t)s * d, xn, d);
          if (key_of(d2) < dv) {
            a.dist[s] = d2;
            mark_dirty(s / gs);
          }
        }
      }
    }
    __syncthreads();
    // (c) level 1 where distances changed (every node after an overflowing step)
    const bool full = overflow != 0;
    const int cnt = full ? a.ng1 : nlist1;
    for (int q = w; q < cnt; q += nw) {
      const int gidx = full ? q : list1[q];
      reduce_l1(gidx);
      if (lane == 0) atomicOr(&dirty2[(gidx >> 6) >> 5], 1u << ((gidx >> 6) & 31));
    }
    __syncthreads();
    // (d) level 2, then clear the marks
    for (int c = w; c < a.ng2; c += nw)
      if (dirty2[c >> 5] & (1u << (c & 31))) reduce_l2(c);
    if (full) {
      for (int q = tid; q < NG1_MAX / 32; q += MM_THREADS) dirty1[q] = 0u;
    } else {
      for (int q = tid; q < cnt; q += MM_THREADS) {
        const int gidx = list1[q];
        atomicAnd(&dirty1[gidx >> 5], ~(1u << (gidx & 31)));
      }
    }
    __syncthreads();
    if (tid < NG2_MAX / 32) dirty2[tid] = 0u;
    if (tid == 0) {
      nlist1 = 0;
      overflow = 0;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------------ neighbour sets
// sorted per-warp list of the best k (squared distance, index) keys: insert the qualifying lanes' candidates
__device__ __forceinline__ void knn_offer(double dj, int ij, bool valid, int k, int lane, double* kd, int* ki,
                                          int& cnt, double& thr, int& thri) {
  const bool qual = valid && (cnt < k || dj < thr || (dj == thr && ij < thri));
  unsigned mask = __ballot_sync(FULL, qual);
  while (mask) {
    const int src = __ffs(mask) - 1;
    mask &= mask - 1;
    const double cd = __shfl_sync(FULL, dj, src);
    const int ci = __shfl_sync(FULL, ij, src);
    if (lane == 0) {
      const bool fullq = cnt >= k;
      if (!fullq || cd < kd[k - 1] || (cd == kd[k - 1] && ci < ki[k - 1])) {
        int pos = fullq ? k - 1 : cnt;
        while (pos > 0 && (kd[pos - 1] > cd || (kd[pos - 1] == cd && ki[pos - 1] > ci))) {
          kd[pos] = kd[pos - 1];
          ki[pos] = ki[pos - 1];
          --pos;
        }
        kd[pos] = cd;
        ki[pos] = ci;
      }
    }
    cnt = cnt < k ? cnt + 1 : k;
    __syncwarp();
  }
  __syncwarp();
  if (cnt >= k && k > 0) {
    thr = kd[k - 1];
    thri = ki[k - 1];
  }
}

// positions t in [t0, t1) with t <= KNN_BRUTE: scan positions 0 .. t - 1
__global__ void __launch_bounds__(256) k_knn_brute(int t0, int t1, int d, int m, const double* __restrict__ Xo,
                                                   const int32_t* __restrict__ order, int32_t* __restrict__ nbr) {
  __shared__ double kd[8][VECCHIA_MAX_M];
  __shared__ int ki[8][VECCHIA_MAX_M];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = t0 + blockIdx.x * 8 + w;
  if (t >= t1) return;
  const int k = t < m ? t : m;
  double xt[MAXD];
  for (int q = 0; q < d; ++q) xt[q] = Xo[(int64_t)t * d + q];
  int cnt = 0;
  double thr = INFINITY;
  int thri = 0x7fffffff;
  for (int j0 = 0; j0 < t; j0 += 32) {
    const int j = j0 + lane;
    double dj = INFINITY;
    int ij = 0x7fffffff;
    if (j < t) {
      dj = sqdist(xt, Xo + (int64_t)j * d, d);
      ij = order[j];
    }
    knn_offer(dj, ij, j < t, k, lane, kd[w], ki[w], cnt, thr, thri);
  }
  for (int q = lane; q < m; q += 32) nbr[(int64_t)t * m + q] = (q < k) ? ki[w][q] : -1;
}

// positions t in [t0, t1) on the grid over positions 0 .. np - 1 (slots hold positions; a slot qualifies when its
// position is below t): rings of cells around the query's cell, stopping once no unvisited cell can hold a better key
__global__ void __launch_bounds__(256) k_knn_grid(int t0, int t1, int m, GridDesc g, const int* __restrict__ cell_start,
                                                  const int* __restrict__ spos, const double* __restrict__ Xo,
                                                  const int32_t* __restrict__ order, int32_t* __restrict__ nbr) {
  __shared__ double kd[8][VECCHIA_MAX_M];
  __shared__ int ki[8][VECCHIA_MAX_M];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = t0 + blockIdx.x * 8 + w;
  if (t >= t1) return;
  const int d = g.d, k = t < m ? t : m;
  double xt[MAXD];
  int cq[MAXD];
  int rmax = 0;
  for (int q = 0; q < d; ++q) {
    xt[q] = Xo[(int64_t)t * d + q];
    cq[q] = cell_coord(g, q, xt[q]);
    rmax = max(rmax, max(cq[q], g.G[q] - 1 - cq[q]));
  }
  int cnt = 0;
  double thr = INFINITY;
  int thri = 0x7fffffff;
  for (int R = 0; R <= rmax; ++R) {
    // cells of the cube [cq - R, cq + R] (clamped) on its surface: max_k |c_k - cq_k| == R
    long long cube = 1;
    int lo[MAXD], span[MAXD];
    for (int q = 0; q < d; ++q) {
      lo[q] = max(0, cq[q] - R);
      span[q] = min(g.G[q] - 1, cq[q] + R) - lo[q] + 1;
      cube *= span[q];
    }
    for (long long c0 = 0; c0 < cube; c0 += 32) {
      const long long c = c0 + lane;
      int s0 = 0, s1 = 0;
      if (c < cube) {
        long long rem = c, cid = 0;
        int cheb = 0;
        for (int q = 0; q < d; ++q) {
          const int cc = lo[q] + (int)(rem % span[q]);
          rem /= span[q];
          cheb = max(cheb, abs(cc - cq[q]));
          cid += (long long)cc * g.stride[q];
        }
        if (cheb == R) {
          s0 = cell_start[cid];
          s1 = cell_start[cid + 1];
        }
      }
      // the lanes' cells one slot at a time; lanes with fewer slots offer nothing
      int more = __any_sync(FULL, s0 < s1);
      while (more) {
        double dj = INFINITY;
        int ij = 0x7fffffff;
        bool valid = false;
        if (s0 < s1) {
          const int pos = spos[s0];
          if (pos < t) {
            dj = sqdist(xt, Xo + (int64_t)pos * d, d);
            ij = order[pos];
            valid = true;
          }
          ++s0;
        }
        knn_offer(dj, ij, valid, k, lane, kd[w], ki[w], cnt, thr, thri);
        more = __any_sync(FULL, s0 < s1);
      }
    }
    // every unvisited point is at least R cell widths away in some dimension (less the rounding of the cell map)
    if (cnt >= k) {
      const double gap = (double)R * g.h_min - g.slack;
      if (gap > 0.0 && thr < gap * gap * (1.0 - 1e-12)) break;
    }
  }
  for (int q = lane; q < m; q += 32) nbr[(int64_t)t * m + q] = (q < k) ? ki[w][q] : -1;
}

__global__ void k_points_major(int n, int d, const double* __restrict__ X, const int32_t* __restrict__ order,
                               double* __restrict__ Xp, double* __restrict__ Xo) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int q = 0; q < d; ++q) {
    if (Xp) Xp[i * d + q] = X[i + (int64_t)q * n];
    if (Xo) Xo[i * d + q] = X[order[i] + (int64_t)q * n];
  }
}

template <class P>
struct DevBuf {
  P* p = nullptr;
  explicit DevBuf(size_t count) { LKG_CUDA(cudaMalloc(&p, sizeof(P) * std::max<size_t>(count, 1))); }
  ~DevBuf() { cudaFree(p); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

// a grid over np points (point-major P with stride d) with about `per_cell` points per cell
GridDesc make_grid(int np, int d, const double* lo, const double* hi, double per_cell) {
  GridDesc g{};
  g.d = d;
  const double cells = std::max(1.0, np / per_cell);
  const int per_dim = std::max(1, (int)std::floor(std::pow(cells, 1.0 / d)));
  long long stride = 1;
  g.h_min = INFINITY;
  double ext_max = 0.0;
  for (int k = 0; k < d; ++k) {
    const double ext = hi[k] - lo[k];
    g.G[k] = ext > 0.0 ? per_dim : 1;
    g.lo[k] = lo[k];
    g.inv_h[k] = ext > 0.0 ? g.G[k] / ext : 0.0;
    g.stride[k] = stride;
    stride *= g.G[k];
    if (ext > 0.0) g.h_min = std::min(g.h_min, ext / g.G[k]);
    ext_max = std::max(ext_max, std::max(std::fabs(lo[k]), std::fabs(hi[k])));
  }
  if (!(g.h_min < INFINITY)) g.h_min = 0.0;  // all points coincide: every query scans every cell
  g.slack = 1e-9 * std::max(ext_max, 1e-300);
  return g;
}

long long grid_cells(const GridDesc& g) {
  long long c = 1;
  for (int k = 0; k < g.d; ++k) c *= g.G[k];
  return c;
}

// counting sort of np points into the cells of g: cell_start (cells + 1) and perm (slot -> point)
void grid_sort(int np, const double* P, const GridDesc& g, int* cell, int* cell_start, int* cursor, int* perm,
               cudaStream_t st) {
  const long long nc = grid_cells(g);
  LKG_CUDA(cudaMemsetAsync(cell_start, 0, sizeof(int) * (nc + 1), st));
  k_grid_cells<<<ceil_div(np, 256), 256, 0, st>>>(np, P, g.d, g, cell, cell_start);
  LKG_LAUNCH("k_grid_cells");
  k_scan_exclusive<<<1, 1024, 0, st>>>((int)nc + 1, cell_start, nullptr);
  LKG_LAUNCH("k_scan_exclusive");
  LKG_CUDA(cudaMemcpyAsync(cursor, cell_start, sizeof(int) * nc, cudaMemcpyDeviceToDevice, st));
  k_grid_scatter<<<ceil_div(np, 256), 256, 0, st>>>(np, cell, cursor, perm);
  LKG_LAUNCH("k_grid_scatter");
}

}  // namespace

void vecchia_sets_grid(int n, int d, const double* hX, const double* dX, int first, int m, int32_t* dorder,
                       int32_t* dnbr, cudaStream_t st) {
  if (d < 1 || d > MAXD) throw std::invalid_argument("Vecchia sets on the GPU support 1 <= d <= 8");
  if (m > VECCHIA_MAX_M) throw std::invalid_argument("Vecchia sets on the GPU support m <= 32");
  // bounding box of the points (the grids' extent)
  std::vector<double> lo(d, INFINITY), hi(d, -INFINITY);
  for (int k = 0; k < d; ++k)
    for (int i = 0; i < n; ++i) {
      lo[k] = std::min(lo[k], hX[i + (size_t)k * n]);
      hi[k] = std::max(hi[k], hX[i + (size_t)k * n]);
    }
  DevBuf<double> Xp((size_t)n * d), Xs((size_t)n * d), dist(n);
  DevBuf<int> cell(n), perm(n), orig(n), slot_of(n);
  k_points_major<<<ceil_div(n, 256), 256, 0, st>>>(n, d, dX, nullptr, Xp.p, nullptr);
  LKG_LAUNCH("k_points_major");

  // ---- maxmin order on a grid of about 2 points per cell
  {
    const GridDesc g = make_grid(n, d, lo.data(), hi.data(), 2.0);
    const long long nc = grid_cells(g);
    DevBuf<int> cstart(nc + 1), cursor(nc);
    grid_sort(n, Xp.p, g, cell.p, cstart.p, cursor.p, perm.p, st);
    k_grid_slots<<<ceil_div(n, 256), 256, 0, st>>>(n, d, Xp.p, perm.p, Xs.p, orig.p, slot_of.p, dist.p);
    LKG_LAUNCH("k_grid_slots");
    int gs = G1;
    while (ceil_div(n, gs) > NG1_MAX) gs *= 2;
    MaxminArgs a{};
    a.n = n;
    a.d = d;
    a.first = first;
    a.g1 = gs;
    a.ng1 = ceil_div(n, gs);
    a.ng2 = ceil_div(a.ng1, 64);
    a.g = g;
    a.cell_start = cstart.p;
    a.Xs = Xs.p;
    a.orig = orig.p;
    a.slot_of = slot_of.p;
    a.dist = dist.p;
    a.order = dorder;
    const size_t smem = sizeof(long long) * a.ng1 + sizeof(int) * ((a.ng1 + 1) & ~1) +
                        (sizeof(long long) + sizeof(int)) * NG2_MAX + sizeof(unsigned) * (NG1_MAX / 32) +
                        sizeof(int) * LIST_MAX;
    LKG_CUDA(cudaFuncSetAttribute(k_maxmin_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int chunk = 65536;  // steps per launch: each launch stays well under a second
    for (int t0 = 0; t0 < n; t0 += chunk) {
      a.t0 = t0;
      a.t1 = std::min(n, t0 + chunk);
      LaunchTimer lt("k_maxmin_grid", st, 0.0, 8.0 * (a.t1 - t0) * 64.0);
      k_maxmin_grid<<<1, MM_THREADS, smem, st>>>(a);
      LKG_LAUNCH("k_maxmin_grid");
    }
    LKG_CUDA(cudaStreamSynchronize(st));  // cstart / cursor are freed at scope exit
  }
  if (m <= 0 || n < 2) return;
  // ---- neighbour sets (rows of m = min(m, n - 1) entries): ordered coordinates, then one grid per prefix of
  // 2^j positions serving the positions in (2^(j-1), 2^j]
  const int mm = std::min(m, n - 1);
  DevBuf<double> Xo((size_t)n * d);
  k_points_major<<<ceil_div(n, 256), 256, 0, st>>>(n, d, dX, dorder, nullptr, Xo.p);
  LKG_LAUNCH("k_points_major");
  const int tb = std::min(n, KNN_BRUTE + 1);
  {
    LaunchTimer lt("k_knn_brute", st, 0.0, 8.0 * d * (double)tb * tb / 2.0);
    k_knn_brute<<<ceil_div(tb, 8), 256, 0, st>>>(0, tb, d, mm, Xo.p, dorder, dnbr);
    LKG_LAUNCH("k_knn_brute");
  }
  DevBuf<int> pos_cell(n), spos(n);
  for (long long np = 2LL * KNN_BRUTE; np / 2 + 1 < n; np *= 2) {
    const int t0 = (int)(np / 2 + 1), t1 = (int)std::min<long long>(n, np + 1);
    const GridDesc g = make_grid(t1, d, lo.data(), hi.data(), 2.0);  // positions 0 .. t1 - 1
    const long long nc = grid_cells(g);
    DevBuf<int> cstart(nc + 1), cursor(nc);
    grid_sort(t1, Xo.p, g, pos_cell.p, cstart.p, cursor.p, spos.p, st);
    LaunchTimer lt("k_knn_grid", st, 0.0, 8.0 * (d + 1) * (double)(t1 - t0) * 8.0 * mm);
    k_knn_grid<<<ceil_div(t1 - t0, 8), 256, 0, st>>>(t0, t1, mm, g, cstart.p, spos.p, Xo.p, dorder, dnbr);
    LKG_LAUNCH("k_knn_grid");
  }
  // the grids' buffers are freed at scope exit: make sure their last users have run
  LKG_CUDA(cudaStreamSynchronize(st));
}

}  // namespace lkg
