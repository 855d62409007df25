// pd_bp.cuh -- per-node bodies of the contact broad phase (pd_broadphase.cu): the rebuild
// decision, the cell count, the scatter into the cell list and the candidate search. The
// per-phase kernels of pd_broadphase.cu and the persistent step of pd_fp32c.cu call the same
// code, so both build the same lists.
#ifndef PD_BP_CUH
#define PD_BP_CUH

#include <cuda_runtime.h>
#include <math.h>

#include "pd_device.cuh"
#include "pd_engine.h"
#include "pd_math.cuh"

namespace pdg {

constexpr uint32_t kNoKey = 0xFFFFFFFFu;  // node not in the cell list

// Node n's current position and cell (a cell is wider than the candidate radius, so two nodes
// within it lie in the same or adjacent cells; CandWalk computes the cell the same way).
__device__ __forceinline__ void node_cell(const DevView &v, uint64_t n, double inv_cell, long long &cx,
                                          long long &cy, long long &cz, double &x, double &y, double &z) {
  x = v.pos[n] + v.disp[n];
  y = v.pos[n + v.Ncap] + v.disp[n + v.Ncap];
  z = v.pos[n + 2 * v.Ncap] + v.disp[n + 2 * v.Ncap];
  cx = (long long)floor(__dmul_rn(x, inv_cell));
  cy = (long long)floor(__dmul_rn(y, inv_cell));
  cz = (long long)floor(__dmul_rn(z, inv_cell));
}

// Whether this step rebuilds (one thread): the accumulated movement bound against half the
// skin; the per-step counters restart.
__device__ __forceinline__ uint32_t bp_decide(const DevView &v, double half_skin) {
  DevCounters &c = *v.cnt;
  const double stepmax = __longlong_as_double((long long)c.stepmax_bits);
  c.rebuild = (c.moved + stepmax > half_skin) ? 1u : 0u;
  c.contacts = 0;
  c.live_bonds = 0;
  return c.rebuild;
}

// Node n's cell bucket and its slot in it (count must be zeroed).
__device__ __forceinline__ void bp_count_node(const DevView &v, uint64_t n, uint32_t *count, uint32_t *key,
                                              uint32_t *slot, uint32_t mask) {
  const uint32_t sim = v.S == 1 ? 0u : v.parts[v.pid[n]].sim;
  if (!v.ss[sim].active) {  // finished simulations leave the cell list
    key[n] = kNoKey;
    return;
  }
  long long cx, cy, cz;
  double x, y, z;
  node_cell(v, n, v.sp[sim].inv_cell, cx, cy, cz, x, y, z);
  const uint32_t kk = cell_hash(cx, cy, cz, sim, mask);
  key[n] = kk;
  slot[n] = atomicAdd(&count[kk], 1u);
}

__device__ __forceinline__ void bp_scatter_node(uint64_t n, const uint32_t *start, const uint32_t *key,
                                                const uint32_t *slot, uint32_t *sorted) {
  if (key[n] == kNoKey) return;
  sorted[start[key[n]] + slot[n]] = (uint32_t)n;
}

// Node n's candidate list: the nodes of its simulation within the candidate radius, ascending
// in file order.
__device__ __forceinline__ void bp_candidates_node(const DevView &v, uint64_t n, const uint32_t *count,
                                                   const uint32_t *start, const uint32_t *sorted, uint32_t mask,
                                                   uint32_t *cand, uint16_t *cand_n, uint32_t cap) {
  constexpr int kMaxCand = (int)kMaxCandCap;
  const uint32_t sim = v.parts[v.pid[n]].sim;
  if (!v.ss[sim].active) {
    cand_n[n] = 0;
    return;
  }
  const DevSimParams &sp = v.sp[sim];
  long long cx, cy, cz;
  double x, y, z;
  node_cell(v, n, sp.inv_cell, cx, cy, cz, x, y, z);
  uint32_t list[kMaxCand];  // file indices: the reference visits contact partners in its numbering
  int cnt = 0;
  bool overflow = false;
  for (int dz = -1; dz <= 1; ++dz)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        uint32_t kk = cell_hash(cx + dx, cy + dy, cz + dz, sim, mask);
        uint32_t b = start[kk], e = b + count[kk];
        for (uint32_t it = b; it < e; ++it) {
          uint32_t m = sorted[it];
          if (m == n) continue;
          if (v.parts[v.pid[m]].sim != sim) continue;
          double mx = v.pos[m] + v.disp[m];
          double my = v.pos[m + v.Ncap] + v.disp[m + v.Ncap];
          double mz = v.pos[m + 2 * v.Ncap] + v.disp[m + 2 * v.Ncap];
          double ddx = mx - x, ddy = my - y, ddz = mz - z;
          if (ddx * ddx + ddy * ddy + ddz * ddz > sp.cand_r2) continue;
          // insert keeping ascending file order; drop duplicates (hash collisions can make
          // two stencil cells share a bucket)
          const uint32_t fm = v.file_of[m];
          int pos = cnt;
          while (pos > 0 && list[pos - 1] > fm) --pos;
          if (pos > 0 && list[pos - 1] == fm) continue;
          if (cnt >= (int)cap) {
            overflow = true;
            break;
          }
          for (int q = cnt; q > pos; --q) list[q] = list[q - 1];
          list[pos] = fm;
          ++cnt;
        }
      }
  if (overflow) {
    // more partners than the list holds: the consumers walk the cell list for this node instead
    // (CandWalk), which gives the same partners in the same order; the host grows the lists
    cand_n[n] = kCandCells;
    atomicAdd(&v.cnt->cand_cells, 1u);
  } else {
    uint32_t *out = cand + n * cap;
    for (int i = 0; i < cnt; ++i) out[i] = v.node_of[list[i]];
    cand_n[n] = (uint16_t)cnt;
  }
  if (cnt && v.xnodes) v.xnodes[atomicAdd(&v.xcount[0], 1u)] = (uint32_t)n;  // FP32 form: work list
}

// Words of shared memory bp_candidates_quad takes per warp: four groups' 27 stencil buckets and
// four gather buffers of kMaxCandCap entries plus a count.
constexpr uint32_t kCandQuadWords = 4 * 27 + 4 * (kMaxCandCap + 1);

// The same lists built four nodes per warp: lane group q = lane / 8 takes node n0 + q, and its
// lane g walks stencil cells g, g + 8, g + 16 and g + 24 (those below 27; a bucket that several
// stencil cells of the node share through a hash collision is walked once, for its lowest cell).
// The qualifying nodes' file indices are gathered in the group's shared buffer and ranked into
// ascending order. Lists, overflow decisions and the work list equal bp_candidates_node's: each
// node of the simulation is found at most once, and a list overflows exactly when more than cap
// distinct nodes qualify. A small handle's search is a chain of dependent loads per node (its
// position, the buckets, their entries, the entries' positions); four chains per warp run side by
// side. All 32 lanes of the warp call it with the same n0; sh holds kCandQuadWords words.
__device__ __forceinline__ void bp_candidates_quad(const DevView &v, uint64_t n0, uint32_t lane, const uint32_t *count,
                                                   const uint32_t *start, const uint32_t *sorted, uint32_t mask,
                                                   uint32_t *cand, uint16_t *cand_n, uint32_t cap, uint32_t *sh) {
  const uint32_t q = lane >> 3, g = lane & 7u;
  const uint64_t n = n0 + q;
  uint32_t *cells = sh + 27 * q;                           // the group's stencil buckets
  uint32_t *buf = sh + 4 * 27 + (kMaxCandCap + 1) * q;     // its file indices, their count last
  const bool one_sim = v.S == 1;                           // no other simulation's nodes in a bucket
  uint32_t sim = 0;
  bool run = false;
  if (n < v.N) {
    sim = one_sim ? 0u : v.parts[v.pid[n]].sim;
    run = v.ss[sim].active != 0;
  }
  long long cx = 0, cy = 0, cz = 0;
  double x = 0.0, y = 0.0, z = 0.0, r2 = 0.0;
  uint32_t kk[4] = {0u, 0u, 0u, 0u};
  if (run) {
    const DevSimParams &sp = v.sp[sim];
    node_cell(v, n, sp.inv_cell, cx, cy, cz, x, y, z);
    r2 = sp.cand_r2;
#pragma unroll
    for (uint32_t r = 0; r < 4; ++r) {
      const uint32_t c = g + 8 * r;
      if (c < 27) {
        const int dx = (int)(c % 3u) - 1, dy = (int)((c / 3u) % 3u) - 1, dz = (int)(c / 9u) - 1;
        kk[r] = cell_hash(cx + dx, cy + dy, cz + dz, sim, mask);
        cells[c] = kk[r];
      }
    }
  }
  if (g == 0) buf[kMaxCandCap] = 0;
  __syncwarp();
  if (run) {
    bool walk[4];
#pragma unroll
    for (uint32_t r = 0; r < 4; ++r) {
      const uint32_t c = g + 8 * r;
      walk[r] = c < 27;
      for (uint32_t c2 = 0; c2 < c && walk[r]; ++c2) walk[r] = cells[c2] != kk[r];
    }
    uint32_t b[4], len[4];
#pragma unroll
    for (uint32_t r = 0; r < 4; ++r) {
      b[r] = walk[r] ? start[kk[r]] : 0u;
      len[r] = walk[r] ? count[kk[r]] : 0u;
    }
    // the lane's buckets as one sequence, in batches of 4 entries whose loads are all issued
    // before their tests
    constexpr uint32_t B = 4;
    const uint32_t tot = len[0] + len[1] + len[2] + len[3];
    for (uint32_t i = 0; i < tot; i += B) {
      uint32_t m[B];
#pragma unroll
      for (uint32_t u = 0; u < B; ++u) {
        uint32_t off = i + u, base = b[0];
        if (off >= len[0]) {
          off -= len[0];
          base = b[1];
          if (off >= len[1]) {
            off -= len[1];
            base = b[2];
            if (off >= len[2]) {
              off -= len[2];
              base = b[3];
            }
          }
        }
        m[u] = i + u < tot ? sorted[base + off] : (uint32_t)n;  // n: no entry
      }
      bool other[B];
#pragma unroll
      for (uint32_t u = 0; u < B; ++u) other[u] = m[u] == n || (!one_sim && v.parts[v.pid[m[u]]].sim != sim);
      double px[B], py[B], pz[B];
#pragma unroll
      for (uint32_t u = 0; u < B; ++u) {
        px[u] = v.pos[m[u]] + v.disp[m[u]];
        py[u] = v.pos[m[u] + v.Ncap] + v.disp[m[u] + v.Ncap];
        pz[u] = v.pos[m[u] + 2 * v.Ncap] + v.disp[m[u] + 2 * v.Ncap];
      }
#pragma unroll
      for (uint32_t u = 0; u < B; ++u) {
        if (other[u]) continue;
        const double ddx = px[u] - x, ddy = py[u] - y, ddz = pz[u] - z;
        if (ddx * ddx + ddy * ddy + ddz * ddz > r2) continue;
        const uint32_t slot = atomicAdd(&buf[kMaxCandCap], 1u);
        if (slot < cap) buf[slot] = v.file_of[m[u]];
      }
    }
  }
  __syncwarp();
  if (n < v.N) {
    if (!run) {
      if (g == 0) cand_n[n] = 0;
    } else {
      const uint32_t total = buf[kMaxCandCap];
      if (total > cap) {
        if (g == 0) {
          cand_n[n] = kCandCells;
          atomicAdd(&v.cnt->cand_cells, 1u);
        }
      } else {
        uint32_t *out = cand + n * cap;
        for (uint32_t i = g; i < total; i += 8) {
          const uint32_t fi = buf[i];
          uint32_t rk = 0;
          for (uint32_t j = 0; j < total; ++j) rk += buf[j] < fi;
          out[rk] = v.node_of[fi];
        }
        if (g == 0) cand_n[n] = (uint16_t)total;
      }
      if (g == 0 && total && v.xnodes) v.xnodes[atomicAdd(&v.xcount[0], 1u)] = (uint32_t)n;
    }
  }
  __syncwarp();
}

}  // namespace pdg
#endif
