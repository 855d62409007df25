// pd_sell.cu -- the SELL-32 bond arrays (pd_engine.h) built on the device from a strictly
// sorted Connectivity: every pair (i, j) has i < j and the pairs of a particle ascend in
// (i, j), so each node's row in conn2NArr's push order (load_hdf5.h:27-37) is the ascending
// list of its partners. The pairs are scattered into rows in any order, each row is sorted,
// and the rows are written slice by slice into the column-major SELL layout with their live
// bits. Integer work only; the host builds the same arrays for any other Connectivity.
#include <cuda_runtime.h>

#include "pd_engine.h"

namespace pdg {

namespace {

// Pair -> both of its rows; a row receives its partners' file indices (the sort key).
__global__ void k_sell_scatter(const uint32_t *__restrict__ conn, uint64_t npairs, const uint64_t *pair_off,
                               const uint64_t *node0, uint32_t nparts, const uint32_t *node_of,
                               const uint64_t *rowptr, uint32_t *cursor, uint32_t *rows) {
  for (uint64_t l = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; l < npairs;
       l += (uint64_t)gridDim.x * blockDim.x) {
    // the particle of pair l: the last p with pair_off[p] <= l (pair_off[0] = 0,
    // pair_off[nparts] = npairs)
    uint32_t lo = 0, hi = nparts;
    while (hi - lo > 1) {
      const uint32_t mid = lo + (hi - lo) / 2;
      if (pair_off[mid] <= l) lo = mid;
      else hi = mid;
    }
    const uint64_t g0 = node0[lo];
    const uint32_t fi = (uint32_t)(g0 + conn[2 * l]), fj = (uint32_t)(g0 + conn[2 * l + 1]);
    const uint32_t a = node_of[fi], b = node_of[fj];
    rows[rowptr[a] + atomicAdd(&cursor[a], 1u)] = fj;
    rows[rowptr[b] + atomicAdd(&cursor[b], 1u)] = fi;
  }
}

// Each row ascending, one warp per row: a row of up to 128 partners is held in registers (4
// per lane) and each partner is written at its rank, the number of smaller partners (partners
// are distinct, so the ranks are a permutation). Longer rows: an insertion sort by one lane.
__global__ void k_sell_sort(const uint64_t *rowptr, uint64_t n_nodes, uint32_t *rows) {
  const uint64_t n = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (n >= n_nodes) return;  // whole warps (the block size is a multiple of 32)
  uint32_t *r = rows + rowptr[n];
  const uint64_t d = rowptr[n + 1] - rowptr[n];
  if (d > 128) {
    if (lane == 0)
      for (uint64_t i = 1; i < d; ++i) {
        const uint32_t x = r[i];
        uint64_t j = i;
        while (j > 0 && r[j - 1] > x) {
          r[j] = r[j - 1];
          --j;
        }
        r[j] = x;
      }
    return;
  }
  uint32_t x[4], rank[4] = {0, 0, 0, 0};
#pragma unroll
  for (int k = 0; k < 4; ++k) x[k] = (lane + 32u * k < d) ? r[lane + 32 * k] : 0xFFFFFFFFu;
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) {
    if (32u * k2 >= d) break;  // uniform across the warp
    for (uint32_t src = 0; src < 32; ++src) {
      const uint32_t y = __shfl_sync(0xffffffffu, x[k2], src);
      const bool vy = src + 32u * k2 < d;
#pragma unroll
      for (int k = 0; k < 4; ++k) rank[k] += (vy && y < x[k]) ? 1u : 0u;
    }
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (lane + 32u * k < d) r[rank[k]] = x[k];
}

// One warp per slice: lane l writes its row's entry of each position (partners as engine
// indices, kNoCol past the row's end) and lane 0 the position's live bits.
__global__ void k_sell_fill(const uint64_t *slice_ptr, uint64_t nslices, const uint64_t *rowptr,
                            const uint32_t *rows, const uint32_t *node_of, uint64_t n_nodes, uint32_t *col,
                            uint32_t *mask) {
  const uint64_t s = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  if (s >= nslices) return;  // whole warps (the block size is a multiple of 32)
  const uint64_t n = s * 32 + lane;
  const uint64_t e0 = slice_ptr[s], w = (slice_ptr[s + 1] - e0) / 32;
  const uint64_t d = n < n_nodes ? rowptr[n + 1] - rowptr[n] : 0;
  const uint32_t *r = rows + (n < n_nodes ? rowptr[n] : 0);
  for (uint64_t j = 0; j < w; ++j) {
    const bool on = j < d;
    col[e0 + 32 * j + lane] = on ? node_of[r[j]] : kNoCol;
    const uint32_t bits = __ballot_sync(0xffffffffu, on);
    if (lane == 0) mask[(e0 >> 5) + j] = bits;
  }
}

}  // namespace

void launch_sell_build(const SellBuild &b, cudaStream_t s) {
  if (b.npairs) k_sell_scatter<<<152 * 8, 256, 0, s>>>(b.conn, b.npairs, b.pair_off, b.node0, b.nparts, b.node_of,
                                                       b.rowptr, b.cursor, b.rows);
  if (b.n_nodes)  // one warp per row
    k_sell_sort<<<(unsigned)((b.n_nodes * 32 + 255) / 256), 256, 0, s>>>(b.rowptr, b.n_nodes, b.rows);
  if (b.nslices)
    k_sell_fill<<<(unsigned)((b.nslices * 32 + 255) / 256), 256, 0, s>>>(b.slice_ptr, b.nslices, b.rowptr, b.rows,
                                                                          b.node_of, b.n_nodes, b.col, b.mask);
}

}  // namespace pdg
