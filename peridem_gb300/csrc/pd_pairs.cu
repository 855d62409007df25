// pd_pairs.cu -- bond lists on the GPU: for every particle, all node pairs (i, j), i < j, with
// |x_i - x_j| <= r, sorted by (i, j). This is the pair list the reference's setup scripts take
// from scipy's cKDTree.query_pairs(delta) and sort (exp_dict.py:542-567). The distance test is
// ((dx*dx + dy*dy) + dz*dz <= r*r in FP64, compiled without contraction), which is how x86
// builds of scipy evaluate it: the lists equal the sorted query_pairs output there. (aarch64
// builds of scipy contract the expression into fused multiply-adds, which can move pairs that
// lie within an ulp of r.)
//
// Method: per particle, a hashed grid of cells slightly larger than r (counting sort into a
// table keyed by particle and cell), then one thread per node scans the 27 cells around it,
// counts its partners j > i (pass 1), writes them after an exclusive scan of the counts
// (pass 2) and sorts its own segment (pass 3).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <cmath>

#include <string>
#include <vector>

#include "peridem_gb300.h"

namespace {

constexpr int kThreads = 256;

struct PairsArgs {
  const double *pos;        // [N][3]
  const uint32_t *pid;      // particle of each node
  const uint64_t *g0;       // first node of each particle
  const double *r;          // radius of each particle
  const double *lo;         // [P][3] lower corner of each particle's box
  const double *cell;       // cell edge of each particle
  uint64_t N;
  uint32_t mask;            // hash table size - 1
  uint32_t *count, *start, *key, *slot, *sorted;
  uint64_t *deg;            // partners j > i per node (pass 1), then exclusive offsets
  uint32_t *out;            // [M][2] local (i, j)
};

__device__ __forceinline__ uint32_t hash_cell(uint32_t p, long long cx, long long cy, long long cz, uint32_t mask) {
  unsigned long long h = (unsigned long long)cx * 0x9E3779B97F4A7C15ull;
  h ^= (unsigned long long)cy * 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
  h ^= (unsigned long long)cz * 0x165667B19E3779F9ull + (h << 6) + (h >> 2);
  h ^= (unsigned long long)p * 0x27D4EB2F165667C5ull;
  h ^= h >> 31;
  h *= 0x7FB5D329728EA185ull;
  h ^= h >> 27;
  return (uint32_t)h & mask;
}

__device__ __forceinline__ void cell_of(const PairsArgs &a, uint64_t n, uint32_t p, long long &cx, long long &cy,
                                        long long &cz) {
  const double c = a.cell[p];
  cx = (long long)floor((a.pos[3 * n] - a.lo[3 * p]) / c);
  cy = (long long)floor((a.pos[3 * n + 1] - a.lo[3 * p + 1]) / c);
  cz = (long long)floor((a.pos[3 * n + 2] - a.lo[3 * p + 2]) / c);
}

__global__ void k_count(PairsArgs a) {
  for (uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = a.pid[n];
    long long cx, cy, cz;
    cell_of(a, n, p, cx, cy, cz);
    const uint32_t k = hash_cell(p, cx, cy, cz, a.mask);
    a.key[n] = k;
    a.slot[n] = atomicAdd(&a.count[k], 1u);
  }
}

__global__ void k_scatter(PairsArgs a) {
  for (uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += (uint64_t)gridDim.x * blockDim.x)
    a.sorted[a.start[a.key[n]] + a.slot[n]] = (uint32_t)n;
}

// Visits every j > i of node i's particle within r; WRITE selects pass 1 (count) or 2 (write).
template <bool WRITE>
__global__ void k_pairs(PairsArgs a) {
  for (uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = a.pid[n];
    const double xi = a.pos[3 * n], yi = a.pos[3 * n + 1], zi = a.pos[3 * n + 2];
    const double r2 = a.r[p] * a.r[p];
    const uint64_t base = a.g0[p];
    long long cx, cy, cz;
    cell_of(a, n, p, cx, cy, cz);
    uint64_t c = 0;
    uint64_t w = WRITE ? a.deg[n] : 0;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const uint32_t k = hash_cell(p, cx + dx, cy + dy, cz + dz, a.mask);
          const uint32_t b = a.start[k], e = b + a.count[k];
          for (uint32_t it = b; it < e; ++it) {
            const uint32_t m = a.sorted[it];
            if (m <= n || a.pid[m] != p) continue;
            // hash collisions can map two stencil cells to one bucket: count each node once
            long long mx, my, mz;
            cell_of(a, m, p, mx, my, mz);
            if (mx != cx + dx || my != cy + dy || mz != cz + dz) continue;
            const double ex = a.pos[3 * (uint64_t)m] - xi, ey = a.pos[3 * (uint64_t)m + 1] - yi,
                         ez = a.pos[3 * (uint64_t)m + 2] - zi;
            if (!((ex * ex + ey * ey) + ez * ez <= r2)) continue;
            if (WRITE) {
              a.out[2 * w] = (uint32_t)(n - base);
              a.out[2 * w + 1] = (uint32_t)(m - base);
              ++w;
            }
            ++c;
          }
        }
    if (!WRITE) a.deg[n] = c;
  }
}

// Flags every node q that lies within r of a marked node of its particle (itself included), with
// the reference's test: d = sqrt((dx*dx + dy*dy) + dz*dz), d <= r (gen_nonlocal_boundry_nodes,
// exp_dict.py:1231-1248, which scans every node for every edge node).
__global__ void k_near(PairsArgs a, const uint8_t *marked, uint8_t *near) {
  for (uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = a.pid[n];
    const double xi = a.pos[3 * n], yi = a.pos[3 * n + 1], zi = a.pos[3 * n + 2];
    const double r = a.r[p];
    long long cx, cy, cz;
    cell_of(a, n, p, cx, cy, cz);
    uint8_t hit = 0;
    for (int dz = -1; dz <= 1 && !hit; ++dz)
      for (int dy = -1; dy <= 1 && !hit; ++dy)
        for (int dx = -1; dx <= 1 && !hit; ++dx) {
          const uint32_t k = hash_cell(p, cx + dx, cy + dy, cz + dz, a.mask);
          const uint32_t b = a.start[k], e = b + a.count[k];
          for (uint32_t it = b; it < e; ++it) {
            const uint32_t m = a.sorted[it];
            if (!marked[m] || a.pid[m] != p) continue;
            const double ex = xi - a.pos[3 * (uint64_t)m], ey = yi - a.pos[3 * (uint64_t)m + 1],
                         ez = zi - a.pos[3 * (uint64_t)m + 2];
            if (sqrt((ex * ex + ey * ey) + ez * ez) <= r) {
              hit = 1;
              break;
            }
          }
        }
    near[n] = hit;
  }
}

// Sorts each node's partner segment (j ascending): rows are already grouped by i in node order.
__global__ void k_sort_rows(PairsArgs a, const uint64_t *end) {
  for (uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b = a.deg[n], e = end[n];
    for (uint64_t x = b + 1; x < e; ++x) {
      const uint32_t v = a.out[2 * x + 1];
      uint64_t y = x;
      while (y > b && a.out[2 * (y - 1) + 1] > v) {
        a.out[2 * y + 1] = a.out[2 * (y - 1) + 1];
        --y;
      }
      a.out[2 * y + 1] = v;
    }
  }
}

// Host-side exclusive scans are fine here: this runs once per setup, not per step.
struct Dev {
  std::vector<void *> ptrs;
  cudaStream_t s = nullptr;
  ~Dev() {
    for (void *p : ptrs) cudaFreeAsync(p, s);
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  }
  template <typename T>
  cudaError_t alloc(T **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, (count ? count : 1) * sizeof(T), s);
    if (e == cudaSuccess) ptrs.push_back(q);
    *p = (T *)q;
    return e;
  }
};

thread_local std::string g_pairs_error;

int fail(int rc, const std::string &m) {
  g_pairs_error = m;
  return rc;
}

// Per-particle boxes and cells a little larger than r, the hashed cell list of all nodes
// (counting sort: count on the device, exclusive scan on the host, scatter on the device), on d's
// stream; a receives the device arrays.
static int check_inputs(const double *pos, const uint64_t *node_offset, const double *radius, uint32_t n_particles) {
  if (!pos || !node_offset || !radius) return fail(PD_EINVAL, "null argument");
  if (node_offset[0] != 0) return fail(PD_EINVAL, "node_offset must start at 0");
  for (uint32_t p = 0; p < n_particles; ++p) {
    if (node_offset[p + 1] < node_offset[p]) return fail(PD_EINVAL, "node_offset not monotone");
    if (!(radius[p] > 0) || !std::isfinite(radius[p])) return fail(PD_EINVAL, "radius must be positive");
  }
  if (node_offset[n_particles] >= 0xFFFFFFF0ull) return fail(PD_EINVAL, "too many nodes");
  return PD_OK;
}

static int build_grid(const double *pos, const uint64_t *node_offset, const double *radius, uint32_t n_particles,
                      Dev &d, PairsArgs &a) {
  const uint64_t N = node_offset[n_particles];
  // per-particle boxes and cells (host: one pass over the points)
  std::vector<double> lo(3 * (size_t)n_particles, 0.0), cell(n_particles), hi(3 * (size_t)n_particles, 0.0);
  std::vector<uint32_t> pid(N);
  std::vector<uint64_t> g0(n_particles);
  for (uint32_t p = 0; p < n_particles; ++p) {
    g0[p] = node_offset[p];
    for (int c = 0; c < 3; ++c) {
      lo[3 * p + c] = INFINITY;
      hi[3 * p + c] = -INFINITY;
    }
    for (uint64_t n = node_offset[p]; n < node_offset[p + 1]; ++n) {
      pid[n] = p;
      for (int c = 0; c < 3; ++c) {
        const double x = pos[3 * n + c];
        if (!std::isfinite(x)) return fail(PD_EINVAL, "non-finite position");
        lo[3 * p + c] = std::fmin(lo[3 * p + c], x);
        hi[3 * p + c] = std::fmax(hi[3 * p + c], x);
      }
    }
    // cells a little larger than r, so that every pair within r lies in adjacent cells
    cell[p] = radius[p] * (1.0 + 1e-6);
    if (node_offset[p + 1] == node_offset[p])
      for (int c = 0; c < 3; ++c) lo[3 * p + c] = 0.0;
  }
  uint32_t bits = 10;
  while ((1ull << bits) < 2 * N) ++bits;
  if (bits > 31) return fail(PD_EINVAL, "too many nodes");
  const uint64_t T = 1ull << bits;

  if (cudaStreamCreateWithFlags(&d.s, cudaStreamNonBlocking) != cudaSuccess)
    return fail(PD_ECUDA, "stream create failed");
  a.N = N;
  a.mask = (uint32_t)(T - 1);
  double *dpos, *dr, *dlo, *dcell;
  uint32_t *dpid;
  uint64_t *dg0;
  cudaError_t e = cudaSuccess;
  auto ck = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  ck(d.alloc(&dpos, 3 * N));
  ck(d.alloc(&dpid, N));
  ck(d.alloc(&dg0, n_particles));
  ck(d.alloc(&dr, n_particles));
  ck(d.alloc(&dlo, 3 * (size_t)n_particles));
  ck(d.alloc(&dcell, n_particles));
  ck(d.alloc(&a.count, T));
  ck(d.alloc(&a.start, T));
  ck(d.alloc(&a.key, N));
  ck(d.alloc(&a.slot, N));
  ck(d.alloc(&a.sorted, N));
  ck(d.alloc(&a.deg, N));
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? PD_ENOMEM : PD_ECUDA, cudaGetErrorString(e));
  ck(cudaMemcpyAsync(dpos, pos, 3 * N * 8, cudaMemcpyHostToDevice, d.s));
  ck(cudaMemcpyAsync(dpid, pid.data(), N * 4, cudaMemcpyHostToDevice, d.s));
  ck(cudaMemcpyAsync(dg0, g0.data(), n_particles * 8, cudaMemcpyHostToDevice, d.s));
  ck(cudaMemcpyAsync(dr, radius, n_particles * 8, cudaMemcpyHostToDevice, d.s));
  ck(cudaMemcpyAsync(dlo, lo.data(), 3 * (size_t)n_particles * 8, cudaMemcpyHostToDevice, d.s));
  ck(cudaMemcpyAsync(dcell, cell.data(), n_particles * 8, cudaMemcpyHostToDevice, d.s));
  ck(cudaMemsetAsync(a.count, 0, T * 4, d.s));
  a.pos = dpos;
  a.pid = dpid;
  a.g0 = dg0;
  a.r = dr;
  a.lo = dlo;
  a.cell = dcell;
  a.out = nullptr;
  const unsigned grid = 152 * 8;
  k_count<<<grid, kThreads, 0, d.s>>>(a);
  // bucket starts: exclusive scan of the counts on the host (T is at most a few 1e7)
  std::vector<uint32_t> cnt(T);
  ck(cudaMemcpyAsync(cnt.data(), a.count, T * 4, cudaMemcpyDeviceToHost, d.s));
  ck(cudaStreamSynchronize(d.s));
  if (e != cudaSuccess) return fail(PD_ECUDA, cudaGetErrorString(e));
  uint32_t run = 0;
  for (uint64_t i = 0; i < T; ++i) {
    const uint32_t c = cnt[i];
    cnt[i] = run;
    run += c;
  }
  ck(cudaMemcpyAsync(a.start, cnt.data(), T * 4, cudaMemcpyHostToDevice, d.s));
  k_scatter<<<grid, kThreads, 0, d.s>>>(a);
  ck(cudaGetLastError());
  if (e != cudaSuccess) return fail(PD_ECUDA, cudaGetErrorString(e));
  return PD_OK;
}

}  // namespace

extern "C" {

const char *pd_pairs_error(void) { return g_pairs_error.c_str(); }

int pd_query_pairs(const double *pos, const uint64_t *node_offset, const double *radius, uint32_t n_particles,
                   uint32_t *pairs, uint64_t cap, uint64_t *pair_offset) {
  if (!pair_offset) return fail(PD_EINVAL, "null argument");
  const int bad = check_inputs(pos, node_offset, radius, n_particles);
  if (bad != PD_OK) return bad;
  const uint64_t N = node_offset[n_particles];
  pair_offset[0] = 0;
  if (N == 0) {
    for (uint32_t p = 0; p < n_particles; ++p) pair_offset[p + 1] = 0;
    return PD_OK;
  }
  Dev d;
  PairsArgs a;
  const int rc = build_grid(pos, node_offset, radius, n_particles, d, a);
  if (rc != PD_OK) return rc;
  const unsigned grid = 152 * 8;
  uint64_t *end;
  cudaError_t e = cudaSuccess;
  auto ck = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  ck(d.alloc(&end, N));
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? PD_ENOMEM : PD_ECUDA, cudaGetErrorString(e));
  k_pairs<false><<<grid, kThreads, 0, d.s>>>(a);
  std::vector<uint64_t> deg(N);
  ck(cudaMemcpyAsync(deg.data(), a.deg, N * 8, cudaMemcpyDeviceToHost, d.s));
  ck(cudaStreamSynchronize(d.s));
  if (e != cudaSuccess) return fail(PD_ECUDA, cudaGetErrorString(e));
  std::vector<uint64_t> off(N), ends(N);
  uint64_t M = 0;
  for (uint64_t n = 0; n < N; ++n) {
    off[n] = M;
    M += deg[n];
    ends[n] = M;
  }
  for (uint32_t p = 0; p < n_particles; ++p)
    pair_offset[p + 1] = node_offset[p + 1] > node_offset[p] ? ends[node_offset[p + 1] - 1] : pair_offset[p];
  if (!pairs) return PD_OK;  // counts only
  if (cap < M) return fail(PD_EINVAL, "pair buffer too small: " + std::to_string(M) + " pairs");
  uint32_t *dout;
  ck(d.alloc(&dout, 2 * M));
  ck(cudaMemcpyAsync(a.deg, off.data(), N * 8, cudaMemcpyHostToDevice, d.s));
  ck(cudaMemcpyAsync(end, ends.data(), N * 8, cudaMemcpyHostToDevice, d.s));
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? PD_ENOMEM : PD_ECUDA, cudaGetErrorString(e));
  a.out = dout;
  k_pairs<true><<<grid, kThreads, 0, d.s>>>(a);
  k_sort_rows<<<grid, kThreads, 0, d.s>>>(a, end);
  ck(cudaGetLastError());
  ck(cudaMemcpyAsync(pairs, dout, 2 * M * 4, cudaMemcpyDeviceToHost, d.s));
  ck(cudaStreamSynchronize(d.s));
  if (e != cudaSuccess) return fail(PD_ECUDA, cudaGetErrorString(e));
  return PD_OK;
}

int pd_query_near(const double *pos, const uint64_t *node_offset, const double *radius, uint32_t n_particles,
                  const uint8_t *marked, uint8_t *near) {
  if (!marked || !near) return fail(PD_EINVAL, "null argument");
  const int bad = check_inputs(pos, node_offset, radius, n_particles);
  if (bad != PD_OK) return bad;
  const uint64_t N = node_offset[n_particles];
  if (N == 0) return PD_OK;
  Dev d;
  PairsArgs a;
  const int rc = build_grid(pos, node_offset, radius, n_particles, d, a);
  if (rc != PD_OK) return rc;
  uint8_t *dmark, *dnear;
  cudaError_t e = cudaSuccess;
  auto ck = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  ck(d.alloc(&dmark, N));
  ck(d.alloc(&dnear, N));
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? PD_ENOMEM : PD_ECUDA, cudaGetErrorString(e));
  ck(cudaMemcpyAsync(dmark, marked, N, cudaMemcpyHostToDevice, d.s));
  k_near<<<152 * 8, kThreads, 0, d.s>>>(a, dmark, dnear);
  ck(cudaGetLastError());
  ck(cudaMemcpyAsync(near, dnear, N, cudaMemcpyDeviceToHost, d.s));
  ck(cudaStreamSynchronize(d.s));
  if (e != cudaSuccess) return fail(PD_ECUDA, cudaGetErrorString(e));
  return PD_OK;
}

}  // extern "C"
