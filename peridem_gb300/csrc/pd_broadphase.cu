// pd_broadphase.cu -- contact broad phase: hashed cell list built by counting sort, and
// per-node candidate lists (global indices, ascending) of the nodes of the same simulation
// within contact radius + skin. The reference tests every node pair of every particle
// pair whose AABBs intersect (timeloop.h:637-651, contact.h:754-769); the exact distance
// test of the reference is still made for every candidate in every step (pd_kernels.cu),
// so the lists only need to be a superset of the pairs within the contact radius. A node with
// more candidates than a list holds is marked to walk the cell list instead (CandWalk,
// pd_device.cuh): the same partners in the same order, so capacity never changes results.
//
// The lists are rebuilt only when the accumulated bound on node movement since the last
// build could exceed half the skin: every kernel here first reads the rebuild flag set by
// k_bp_decide and returns at once when no rebuild is due, so the whole sequence can sit
// in a CUDA graph that replays every step.
#include <cuda_runtime.h>

#include <algorithm>
#include <math.h>

#include "pd_bp.cuh"
#include "pd_device.cuh"
#include "pd_engine.h"
#include "pd_math.cuh"

namespace pdg {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanBlock = kScanThreads * kScanPer;

// Decide whether this step rebuilds; also zero the wall reactions of every simulation
// (Wall.setzero_reaction at the top of each step, timeloop.h:397). Inside the step graph the
// decision also sets the conditional node that runs the rebuild kernels.
__global__ void k_bp_decide(DevView v, double half_skin, cudaGraphConditionalHandle cond) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) {
    const uint32_t rebuild = bp_decide(v, half_skin);
    if (cond) cudaGraphSetConditional(cond, rebuild);
  }
  for (uint32_t s = t; s < v.S; s += gridDim.x * blockDim.x)
    for (int k = 0; k < 18; ++k) v.ss[s].react[k] = 0.0;
}

__global__ void k_bp_clear(DevView v, uint32_t *count, uint64_t T) {
  if (!v.cnt->rebuild) return;
  if (v.xcount && blockIdx.x == 0 && threadIdx.x == 0) v.xcount[0] = 0;  // contact-node list restarts
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T; i += (uint64_t)gridDim.x * blockDim.x)
    count[i] = 0;
}

__global__ void k_bp_count(DevView v, uint32_t *count, uint32_t *key, uint32_t *slot, uint32_t mask) {
  if (!v.cnt->rebuild) return;
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.N) return;
  bp_count_node(v, n, count, key, slot, mask);
}

// exclusive scan, phase 1: per-block scan, block totals
__global__ void k_scan_blocks(const DevView v, const uint32_t *in, uint32_t *out, uint32_t *sums, uint64_t T) {
  if (!v.cnt->rebuild) return;
  __shared__ uint32_t sh[kScanThreads];
  const uint64_t base = (uint64_t)blockIdx.x * kScanBlock + (uint64_t)threadIdx.x * kScanPer;
  uint32_t vals[kScanPer];
  uint32_t tot = 0;
  for (int i = 0; i < kScanPer; ++i) {
    uint64_t idx = base + i;
    vals[i] = idx < T ? in[idx] : 0u;
    tot += vals[i];
  }
  sh[threadIdx.x] = tot;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    uint32_t add = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0u;
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  uint32_t run = sh[threadIdx.x] - tot;  // exclusive prefix of this thread
  for (int i = 0; i < kScanPer; ++i) {
    uint64_t idx = base + i;
    if (idx < T) out[idx] = run;
    run += vals[i];
  }
  if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = sh[threadIdx.x];
}

// phase 2: one block scans the block totals in place (exclusive)
__global__ void k_scan_top(const DevView v, uint32_t *sums, uint32_t nb) {
  if (!v.cnt->rebuild) return;
  __shared__ uint32_t sh[kScanThreads];
  const uint32_t per = (nb + kScanThreads - 1) / kScanThreads;
  const uint32_t b0 = threadIdx.x * per;
  uint32_t tot = 0;
  for (uint32_t i = 0; i < per; ++i)
    if (b0 + i < nb) tot += sums[b0 + i];
  sh[threadIdx.x] = tot;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    uint32_t add = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0u;
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  uint32_t run = sh[threadIdx.x] - tot;
  for (uint32_t i = 0; i < per; ++i) {
    if (b0 + i < nb) {
      uint32_t x = sums[b0 + i];
      sums[b0 + i] = run;
      run += x;
    }
  }
}

// phase 3: add block offsets
__global__ void k_scan_add(const DevView v, uint32_t *out, const uint32_t *sums, uint64_t T) {
  if (!v.cnt->rebuild) return;
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < T) out[i] += sums[i / kScanBlock];
}

__global__ void k_bp_scatter(DevView v, const uint32_t *start, const uint32_t *key, const uint32_t *slot,
                             uint32_t *sorted) {
  if (!v.cnt->rebuild) return;
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.N) return;
  bp_scatter_node(n, start, key, slot, sorted);
}

__global__ void k_bp_candidates(DevView v, const uint32_t *count, const uint32_t *start, const uint32_t *sorted,
                                uint32_t mask, uint32_t *cand, uint16_t *cand_n, uint32_t cap) {
  if (!v.cnt->rebuild) return;
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.N) return;
  bp_candidates_node(v, n, count, start, sorted, mask, cand, cand_n, cap);
}

// Four nodes per warp (bp_candidates_quad): small handles, whose one-thread-per-node search is a
// long chain of dependent loads on few warps.
__global__ void __launch_bounds__(128) k_bp_candidates_w(DevView v, const uint32_t *count, const uint32_t *start,
                                                         const uint32_t *sorted, uint32_t mask, uint32_t *cand,
                                                         uint16_t *cand_n, uint32_t cap) {
  __shared__ uint32_t sh[4][kCandQuadWords];
  if (!v.cnt->rebuild) return;
  // a bounded grid whose warps take groups of four nodes in turn: in steps without a rebuild the
  // launch costs a few waves less than one warp per group would
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 4 < v.N; w += nwarps)
    bp_candidates_quad(v, w * 4, threadIdx.x & 31, count, start, sorted, mask, cand, cand_n, cap, sh[threadIdx.x >> 5]);
}

}  // namespace

void launch_broadphase(const DevView &v, BroadPhase &bp, cudaStream_t s) {
  const uint64_t T = 1ull << bp.table_bits;
  const uint32_t mask = (uint32_t)(T - 1);
  const uint32_t nb = (uint32_t)((T + kScanBlock - 1) / kScanBlock);
  const uint64_t nblk = (v.N + 255) / 256;
  k_bp_clear<<<1024, 256, 0, s>>>(v, bp.count, T);
  if (nblk) k_bp_count<<<(unsigned)nblk, 256, 0, s>>>(v, bp.count, bp.key, bp.slot, mask);
  k_scan_blocks<<<nb, kScanThreads, 0, s>>>(v, bp.count, bp.start, bp.block_sums, T);
  k_scan_top<<<1, kScanThreads, 0, s>>>(v, bp.block_sums, nb);
  k_scan_add<<<(unsigned)((T + 255) / 256), 256, 0, s>>>(v, bp.start, bp.block_sums, T);
  if (nblk) {
    k_bp_scatter<<<(unsigned)nblk, 256, 0, s>>>(v, bp.start, bp.key, bp.slot, bp.sorted);
    if (v.N <= kWarpCandNodes)
      k_bp_candidates_w<<<(unsigned)std::min<uint64_t>((v.N + 15) / 16, 152 * 8), 128, 0, s>>>(
          v, bp.count, bp.start, bp.sorted, mask, bp.cand, bp.cand_n, bp.cand_cap);
    else
      k_bp_candidates<<<(unsigned)((v.N + 127) / 128), 128, 0, s>>>(v, bp.count, bp.start, bp.sorted, mask,
                                                                    bp.cand, bp.cand_n, bp.cand_cap);
  }
}

void launch_bp_decide(const DevView &v, double half_skin, cudaStream_t s, cudaGraphConditionalHandle cond) {
  k_bp_decide<<<1, 128, 0, s>>>(v, half_skin, cond);
}

}  // namespace pdg
