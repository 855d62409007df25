// pd_fp32c.cu -- the FP32-compensated form of the fused step (compiled with contraction on).
//
// GB300 issues FP64 at 1/64 of the FP32 rate, so this form keeps FP64 to what needs it:
//   k_extra32  the non-bond force density of the nodes that have any this step -- contact
//              partners, a wall face within reach, extforce, torque -- in FP64 with the
//              reference's formulas (contact.h:744-942, 1057-1124; timeloop.h:582-633). A
//              float test in each particle's local frame skips faces that are out of reach.
//   k_bond32   per node: PD bond forces in FP32 with the cancellation-free stretch
//              s = (2 xi.eta + eta.eta) / ((|xi+eta| + |xi|) |xi|) on anchor-relative FP32
//              positions and displacements, Kahan-compensated FP32 sums; the stretch-vs-snot
//              decision is re-taken in FP64 inside a relative band around snot; then the
//              FP64 velocity-Verlet corrector (timeloop.h:661-781) and the particle AABB in the
//              local frame (FP32, widened outwards when converted back).
// The summation order is not the reference's (bonds, then the FP64 extras); results agree
// with the FP64 form within the stated tolerance.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

#include "pd_bp.cuh"
#include "pd_device.cuh"
#include "pd_end.cuh"
#include "pd_engine.h"
#include "pd_math.cuh"

namespace pdg {

// Whether node n has any FP64 non-bond work this step: contact candidates, a wall within the
// contact radius (FP32 test in the particle's frame, slightly widened), external force or
// torque.
__device__ __forceinline__ bool extra_needed(const DevView &v, uint64_t n, uint32_t k, const DevPart &P,
                                             const DevSimParams &sp, const DevSimState &st, const float4 &pl,
                                             const float4 &ul) {
  const bool mov = P.movable != 0;
  if (v.cand_n[n] != 0 || st.torque || (mov && P.has_ext)) return true;
  if (mov && P.stoppable && sp.allow_wall) {
    const float cx = pl.x + ul.x, cy = pl.y + ul.y, cz = pl.z + ul.z;
    const float *wl = v.wall_local + 6 * (uint64_t)k;
    const float lim = (float)sp.Rc * 1.001f;
    return fabsf(cx - wl[0]) <= lim || fabsf(cx - wl[3]) <= lim || fabsf(cy - wl[1]) <= lim ||
           fabsf(cy - wl[4]) <= lim || fabsf(cz - wl[2]) <= lim || fabsf(cz - wl[5]) <= lim;
  }
  return false;
}

// The node-level inputs of extra_force.
struct ExtraCtx {
  uint32_t k;
  bool nc, mov, wall_near, ext, bdry_i;
  D3 di, pi, vi;
  double voli;
};

__device__ __forceinline__ ExtraCtx extra_ctx(const DevView &v, uint64_t n, const DevPart &P,
                                              const DevSimParams &sp) {
  ExtraCtx c;
  c.k = v.pid[n];
  c.nc = v.cand_n[n] != 0;  // contact candidates (a list, or the cell walk)
  c.mov = P.movable != 0;
  c.wall_near = false;
  if (c.mov && P.stoppable && sp.allow_wall) {
    const float4 pl = v.rec[n].p, ul = v.rec[n].u;
    const float cx = pl.x + ul.x, cy = pl.y + ul.y, cz = pl.z + ul.z;
    const float *wl = v.wall_local + 6 * (uint64_t)c.k;
    const float lim = (float)sp.Rc * 1.001f;
    c.wall_near = fabsf(cx - wl[0]) <= lim || fabsf(cx - wl[3]) <= lim || fabsf(cy - wl[1]) <= lim ||
                  fabsf(cy - wl[4]) <= lim || fabsf(cz - wl[2]) <= lim || fabsf(cz - wl[5]) <= lim;
  }
  c.ext = c.mov && P.has_ext;
  const uint64_t C3 = v.Ncap;
  c.di = ld3(v.disp, n, C3);
  c.pi = ld3(v.pos, n, C3);
  c.vi = ld3(v.vel_in, n, C3);
  c.voli = v.vol[n];
  c.bdry_i = v.bdry[n] != 0;
  return c;
}

// One contact candidate's share of the node's force: the pair's forces and how they enter the
// sum (kind 0: not at all; 1: added, in the self-contact loop and for a partner of a later
// particle; 2: subtracted with the volume scaling, for a partner of an earlier particle).
struct CandShare {
  PairForce pf;
  double volm;
  int kind;
};

// Candidate m of node n in extra_force's self-contact loop (self) or contact loop (!self): the
// loop's tests and its pair_force call (contact.h:746-942).
__device__ __forceinline__ CandShare cand_share(const DevView &v, uint64_t n, const DevPart &P,
                                                const DevSimParams &sp, const DevSimState &st, const ExtraCtx &c,
                                                uint32_t m, bool self) {
  CandShare o;
  o.pf.fc = o.pf.fd = o.pf.ff = d3(0.0, 0.0, 0.0);
  o.pf.has_fd = o.pf.has_ff = false;
  o.volm = 0.0;
  o.kind = 0;
  const uint64_t C3 = v.Ncap;
  const bool own = m >= P.g0 && m < P.g0 + P.n;
  if (self) {  // self-contact with the particle's own nodes that are not bonded to n
    if (!own) return o;
    if (sp.nl_bdry_only && !v.bdry[m]) return o;
    D3 xi = ld3(v.pos, m, C3) - c.pi;
    D3 dir = (ld3(v.disp, m, C3) - c.di) + xi;
    const double q = sq3(dir);
    if (q >= sp.rc2_far) return o;  // outside Rc for certain: skip the square root
    double dn = sqrt(q);
    if (!(dn <= sp.Rc)) return o;
    double xin = norm3(xi);
    double len_ref = sp.Rc, sc = sp.sc;
    if (row_has_live(v, n, m)) return o;
    if (xin < sp.Rc) {
      len_ref = xin;
      sc = P.cnot;
    }
    if (!(dn < len_ref)) return o;
    pair_force(dir, dn, len_ref, sc, v.vol[m], P.rho, c.vi, ld3(v.vel_in, m, C3), sp, st, o.pf);
    if (P.stoppable) o.kind = 1;
    return o;
  }
  if (own) return o;
  const uint32_t km = v.pid[m];
  const uint32_t a = km < c.k ? km : c.k, b = km < c.k ? c.k : km;
  if (!(v.parts[a].movable || v.parts[b].movable)) return o;
  if (!intersects_fext(v.lrtb + 6 * (uint64_t)a, v.lrtb + 6 * (uint64_t)b, sp.Rc)) return o;
  if (sp.nl_bdry_only && !v.bdry[m]) return o;
  const D3 pm = ld3(v.pos, m, C3), dm = ld3(v.disp, m, C3);
  if (km > c.k) {
    D3 dir = (dm - c.di) + (pm - c.pi);
    const double q = sq3(dir);
    if (q >= sp.rc2_far) return o;
    double dn = sqrt(q);
    if (!(dn < sp.Rc)) return o;
    pair_force(dir, dn, sp.Rc, sp.sc, v.vol[m], P.rho, c.vi, ld3(v.vel_in, m, C3), sp, st, o.pf);
    o.kind = 1;
    if (v.stats) atomicAdd(&v.cnt->contacts, 1ull);
  } else {
    D3 dir = (c.di - dm) + (c.pi - pm);
    const double q = sq3(dir);
    if (q >= sp.rc2_far) return o;
    double dn = sqrt(q);
    if (!(dn < sp.Rc)) return o;
    o.volm = v.vol[m];
    pair_force(dir, dn, sp.Rc, sp.sc, c.voli, v.parts[km].rho, ld3(v.vel_in, m, C3), c.vi, sp, st, o.pf);
    o.kind = 2;
  }
  return o;
}

// Adds a candidate's share to the running sum f, in the loops' order of operations.
__device__ __forceinline__ void apply_share(D3 &f, const CandShare &s, double voli) {
  if (s.kind == 1) {
    f = f + s.pf.fc;
    if (s.pf.has_fd) f = f + s.pf.fd;
    if (s.pf.has_ff) f = f + s.pf.ff;
  } else if (s.kind == 2) {
    const double volm = s.volm;
    f = f - (s.pf.fc / voli) * volm;
    if (s.pf.has_fd) f = f - (s.pf.fd / sqrt(voli)) * sqrt(volm);
    if (s.pf.has_ff) f = f - s.pf.ff;
  }
}

// The part of extra_force between the two candidate loops: walls and external force of a
// movable node, then torque.
__device__ __forceinline__ void extra_middle(const DevView &v, uint64_t n, const DevPart &P, const DevSimParams &sp,
                                             DevSimState &st, const ExtraCtx &c, D3 &f) {
  const uint64_t C3 = v.Ncap;
  if (c.mov) {
    if (c.wall_near && !within_interior(v.lrtb + 6 * (uint64_t)c.k, st.wall, sp.Rc) &&
        (!sp.nl_bdry_only || c.bdry_i)) {
      D3 cur = c.pi + c.di;
      const bool rx = sp.compute_wall_reaction != 0;
      wall_face(cur.x - st.wall[0], 0, c.vi, c.voli, P.rho, f, st.spd[0], 0, sp, st, rx);
      wall_face(cur.x - st.wall[3], 0, c.vi, c.voli, P.rho, f, st.spd[3], 3, sp, st, rx);
      wall_face(cur.y - st.wall[1], 1, c.vi, c.voli, P.rho, f, st.spd[1], 1, sp, st, rx);
      wall_face(cur.y - st.wall[4], 1, c.vi, c.voli, P.rho, f, st.spd[4], 4, sp, st, rx);
      wall_face(cur.z - st.wall[2], 2, c.vi, c.voli, P.rho, f, st.spd[2], 2, sp, st, rx);
      wall_face(cur.z - st.wall[5], 2, c.vi, c.voli, P.rho, f, st.spd[5], 5, sp, st, rx);
    }
    if (c.ext) {
      D3 ex = ld3(v.ext, n, C3);
      if (sp.gradient_extforce) ex = st.extf_scale * ex;
      f = f + ex;
    }
  }
  if (st.torque) {
    const double *cc = v.centroid + 3 * (uint64_t)c.k;
    D3 r = (c.pi + c.di) - d3(cc[0], cc[1], cc[2]);
    double rn = norm3(r);
    double r_inv = (rn != 0.0 ? 1 / rn : 0);
    const int ta = (int)P.taxis;
    set_comp(r, ta, 0.0);
    D3 perp = d3(0.0, 0.0, 0.0);
    set_comp(perp, (ta + 1) % 3, -comp(r, (ta + 2) % 3));
    set_comp(perp, (ta + 2) % 3, comp(r, (ta + 1) % 3));
    double pn = norm3(perp);
    if (pn > 0) {
      perp = perp / pn;
    } else {
      set_comp(perp, (ta + 1) % 3, 0.0);
      set_comp(perp, (ta + 2) % 3, 0.0);
    }
    f = f + (r_inv * P.tval) * perp;
  }
}

// FP64 non-bond force density of node n in the reference's order: self-contact
// (timeloop.h:554-557), walls (contact.h:1060-1124), external force and torque
// (timeloop.h:582-633), then contact with the other particles in ascending partner order
// (timeloop.h:637-651). Kept out of line: the bond kernel calls it only for nodes that need it.
__device__ __noinline__ D3 extra_force(const DevView &v, uint64_t n) {
  const DevPart &P = v.parts[v.pid[n]];
  const DevSimParams &sp = v.sp[P.sim];
  DevSimState &st = v.ss[P.sim];
  const ExtraCtx c = extra_ctx(v, n, P, sp);
  D3 f = d3(0.0, 0.0, 0.0);
  if (c.mov && c.nc && st.fracture && P.breakable && st.self_contact && (!sp.nl_bdry_only || c.bdry_i)) {
    CandWalk walk(v, n);
    uint32_t m;
    while (walk.next(m)) {
      if (m < P.g0) continue;
      if (m >= P.g0 + P.n) break;
      apply_share(f, cand_share(v, n, P, sp, st, c, m, true), c.voli);
    }
  }
  extra_middle(v, n, P, sp, st, c, f);
  if (c.nc && P.stoppable && (!sp.nl_bdry_only || c.bdry_i)) {
    CandWalk walk(v, n);
    uint32_t m;
    while (walk.next(m)) apply_share(f, cand_share(v, n, P, sp, st, c, m, false), c.voli);
  }
  return f;
}

// Lane src's share, all lanes of mask gm taking part.
__device__ __forceinline__ CandShare shfl_share(const CandShare &s, uint32_t src, unsigned gm) {
  CandShare o;
  o.pf.fc = d3(__shfl_sync(gm, s.pf.fc.x, src), __shfl_sync(gm, s.pf.fc.y, src), __shfl_sync(gm, s.pf.fc.z, src));
  o.pf.fd = d3(__shfl_sync(gm, s.pf.fd.x, src), __shfl_sync(gm, s.pf.fd.y, src), __shfl_sync(gm, s.pf.fd.z, src));
  o.pf.ff = d3(__shfl_sync(gm, s.pf.ff.x, src), __shfl_sync(gm, s.pf.ff.y, src), __shfl_sync(gm, s.pf.ff.z, src));
  o.volm = __shfl_sync(gm, s.volm, src);
  const int bits = __shfl_sync(gm, s.kind | (s.pf.has_fd ? 4 : 0) | (s.pf.has_ff ? 8 : 0), src);
  o.kind = bits & 3;
  o.pf.has_fd = (bits & 4) != 0;
  o.pf.has_ff = (bits & 8) != 0;
  return o;
}

// extra_force by the L lanes of node n (lanes first .. first + L - 1 of the warp, all calling it
// with the same n; the result is valid on lane first) for a node whose candidates are a list:
// the candidates are dealt over the lanes, each computing its candidates' shares with
// cand_share, and lane first adds them in list order with apply_share, so the sum is
// extra_force's bit for bit. A node in contact no longer evaluates its pairs one after another
// on one lane while the node's other lanes wait (each pair is a chain of FP64 square roots and
// divisions).
template <int L>
__device__ __noinline__ D3 extra_force_lanes(const DevView &v, uint64_t n, uint32_t sub, uint32_t first) {
  const unsigned gm = ((1u << L) - 1u) << first;
  const DevPart &P = v.parts[v.pid[n]];
  const DevSimParams &sp = v.sp[P.sim];
  DevSimState &st = v.ss[P.sim];
  const ExtraCtx c = extra_ctx(v, n, P, sp);
  const uint32_t *cl = v.cand + n * v.cand_cap;
  const int ncand = (int)v.cand_n[n];
  D3 f = d3(0.0, 0.0, 0.0);
  auto loop = [&](bool self) {
    for (int i0 = 0; i0 < ncand; i0 += L) {
      const int i = i0 + (int)sub;
      CandShare s;
      s.pf.fc = s.pf.fd = s.pf.ff = d3(0.0, 0.0, 0.0);
      s.pf.has_fd = s.pf.has_ff = false;
      s.volm = 0.0;
      s.kind = 0;
      if (i < ncand) s = cand_share(v, n, P, sp, st, c, cl[i], self);
      for (int j = 0; j < L && i0 + j < ncand; ++j) {
        const CandShare t = shfl_share(s, first + (uint32_t)j, gm);
        if (sub == 0) apply_share(f, t, c.voli);
      }
    }
  };
  if (c.mov && c.nc && st.fracture && P.breakable && st.self_contact && (!sp.nl_bdry_only || c.bdry_i))
    loop(true);
  if (sub == 0) extra_middle(v, n, P, sp, st, c, f);
  if (c.nc && P.stoppable && (!sp.nl_bdry_only || c.bdry_i)) loop(false);
  return f;
}

// Separate-kernel form: the FP64 non-bond force of the nodes that have some, for the bond
// kernel to add (f_extra, extra_flag; the bond kernel clears the flag when it takes the force).
// Only listed work is visited: the nodes with contact candidates (listed when the candidate
// lists are built) and the nodes of the particles listed at the end of the previous step
// (external force, torque, or a wall nearby); the cost follows the work, not the node count.
__device__ __forceinline__ void extra_node(const DevView &v, uint64_t n) {
  const uint32_t k = v.pid[n];
  const DevPart &P = v.parts[k];
  const DevSimState &st = v.ss[P.sim];
  if (!st.active || !extra_needed(v, n, k, P, v.sp[P.sim], st, v.rec[n].p, v.rec[n].u)) return;
  st3(v.f_extra, n, v.Ncap, extra_force(v, n));
  v.extra_flag[n] = 1;
}

__global__ void __launch_bounds__(128) k_extra32(const __grid_constant__ DevView v) {
  if (v.cnt->xall) {  // after setup or a state change: every node, once
    for (uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n < v.N; n += (uint64_t)gridDim.x * blockDim.x)
      extra_node(v, n);
    return;
  }
  const uint32_t nx = v.xcount[0], np = v.xcount[1];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nx; i += gridDim.x * blockDim.x)
    extra_node(v, v.xnodes[i]);
  // the listed particles' nodes in chunks of one block's threads, spread over all blocks (one
  // block per particle left a 10k-node particle's nodes to 128 threads in turn)
  const uint64_t cpp = (v.max_part_nodes + blockDim.x - 1) / blockDim.x;  // chunks per particle
  for (uint64_t c = blockIdx.x; c < (uint64_t)np * cpp; c += gridDim.x) {
    const DevPart &P = v.parts[v.xparts[c / cpp]];
    const uint64_t l = (c % cpp) * blockDim.x + threadIdx.x;
    if (l < P.n) {
      const uint64_t n = (uint64_t)P.g0 + l;
      if (v.cand_n[n] == 0) extra_node(v, n);  // nodes with candidates are on the node list
    }
  }
}

// Breaking a bond in the FP32 form: its live bit is cleared and the broken flag (bit 31) is set
// in its column entry, which only the node's own thread writes. The bond loops read the flag
// with the column index and need no live-mask loads.
__device__ __noinline__ void cut_bond(uint32_t *word, uint32_t lane, uint32_t *cole, uint32_t q) {
  atomicAnd(word, ~(1u << lane));
  *cole = q | kColBroken;
}

// FP64 stretch of the reference formula (particle2.h:139-149) for a bond whose FP32 stretch
// lies in the band around snot; breaks the bond when it exceeds snot. Kept out of line so that
// the compiler does not predicate its FP64 work into the bond loop.
__device__ __noinline__ void band_check(const DevView &v, uint64_t n, uint32_t q, uint32_t *word, uint32_t lane,
                                        double snot, uint32_t *cole) {
  const uint64_t C3 = v.Ncap;
  const D3 di = ld3(v.disp, n, C3), pi = ld3(v.pos, n, C3);
  D3 xi64 = ld3(v.pos, q, C3) - pi;
  D3 eta = (ld3(v.disp, q, C3) - di) + xi64;
  double en = norm3(eta), xn = norm3(xi64);
  if (((en - xn) / xn) > snot) {
    atomicAnd(word, ~(1u << lane));
    *cole = q | kColBroken;
  }
}

// A column entry: read once per step, so it is not allocated in L1, which is left to the
// partner records (the bond kernel's working set). NC = 0: a coherent load, for a launch that
// writes the entries it reads in a later step (the persistent step).
template <int NC = 1>
__device__ __forceinline__ uint32_t ld_col(const uint32_t *p) {
  uint32_t r;
  if (NC)
    asm("ld.global.nc.L1::no_allocate.b32 %0, [%1];" : "=r"(r) : "l"(p));
  else
    asm volatile("ld.global.L1::no_allocate.b32 %0, [%1];" : "=r"(r) : "l"(p) : "memory");
  return r;
}

// A partner's record: one 256-bit load (W) or two 128-bit loads of the same 32-byte sector;
// NC = 0 as for ld_col.
template <int W, int NC = 1>
__device__ __forceinline__ void ld_rec(const Rec32 *r, float4 &p, float4 &u) {
  if (W && NC) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(p.x), "=f"(p.y), "=f"(p.z), "=f"(p.w), "=f"(u.x), "=f"(u.y), "=f"(u.z), "=f"(u.w)
        : "l"(r));
  } else if (W) {
    asm volatile("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(p.x), "=f"(p.y), "=f"(p.z), "=f"(p.w), "=f"(u.x), "=f"(u.y), "=f"(u.z), "=f"(u.w)
                 : "l"(r)
                 : "memory");
  } else if (NC) {
    p = __ldg(&r->p);
    u = __ldg(&r->u);
  } else {
    asm volatile("ld.global.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(p.x), "=f"(p.y), "=f"(p.z), "=f"(p.w) : "l"(&r->p) : "memory");
    asm volatile("ld.global.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(u.x), "=f"(u.y), "=f"(u.z), "=f"(u.w) : "l"(&r->u) : "memory");
  }
}

// Kahan-compensated FP32 accumulator (sum s, compensation c; the value is s - c).
struct Acc32 {
  float sx, sy, sz, cx, cy, cz;
};

// A node's bond force density is summed in up to four chains: its row of dg positions is cut
// into consecutive blocks of chain_len(dg) = 8 ceil(dg / 32) positions, each block is
// Kahan-summed from zero in row order, and the blocks' sums are merged left to right with exact
// two-sums (kahan_merge). The order depends on the row alone, so every form of the bond loop -- one
// thread walking the row, or two or four lanes per node each taking whole blocks -- gives the same
// bits. One thread holds only the running total and the current block's sum.
__device__ __forceinline__ int chain_len(int dg) { return 8 * ((dg + 31) >> 5); }

// Approximate reciprocal square root and reciprocal (one special-function instruction each;
// subnormal inputs flush to zero, which never occurs for squared bond lengths).
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The terms of one bond in FP32: cancellation-free stretch and the force coefficient g, so
// that the bond adds g * (xi + eta) to the node's force density.
struct BondTerms {
  float g, yx, yy, yz, str;
};

// xi = pq - pi (reference positions), eta = uq - ui (displacements), y = xi + eta. The stretch
// (particle2.h:139-149) s = (|y| - |xi|) / |xi| is formed as (|y|^2 - |xi|^2) / ((|y| + |xi|) |xi|)
// with |y|^2 - |xi|^2 = 2 xi.eta + eta.eta = eta.(xi + y), which has no cancellation; the force
// density term is cnot V_q s y / |y| (particle2.h:151-157), and the record's fourth float holds
// cnot V_q.
__device__ __forceinline__ BondTerms bond32_terms(const float4 &pi, const float4 &ui, const float4 &pq,
                                                  const float4 &uq) {
  const float xx = pq.x - pi.x, xy = pq.y - pi.y, xz = pq.z - pi.z;
  const float ex = uq.x - ui.x, ey = uq.y - ui.y, ez = uq.z - ui.z;
  BondTerms b;
  b.yx = xx + ex;
  b.yy = xy + ey;
  b.yz = xz + ez;
  const float x2 = fmaf(xx, xx, fmaf(xy, xy, xz * xz));
  const float y2 = fmaf(b.yx, b.yx, fmaf(b.yy, b.yy, b.yz * b.yz));
  const float num = fmaf(ex, xx + b.yx, fmaf(ey, xy + b.yy, ez * (xz + b.yz)));
  const float rx = rsqrt_approx(x2), ry = rsqrt_approx(y2);
  b.str = (num * rx) * rcp_approx(fmaf(x2, rx, y2 * ry));
  b.g = (b.str * ry) * pq.w;
  return b;
}

// Kahan-compensated accumulation of one bond (the order of these calls fixes the result).
__device__ __forceinline__ void kahan_add(Acc32 &a, float g, float yx, float yy, float yz) {
  float t, y;
  y = fmaf(g, yx, -a.cx); t = a.sx + y; a.cx = (t - a.sx) - y; a.sx = t;
  y = fmaf(g, yy, -a.cy); t = a.sy + y; a.cy = (t - a.sy) - y; a.sy = t;
  y = fmaf(g, yz, -a.cz); t = a.sz + y; a.cz = (t - a.sz) - y; a.sz = t;
}

// (s, c) + (s2, c2) -> (S, (c + c2) - e) with S + e = s + s2 exactly (Knuth's two-sum): the
// result does not depend on the order of the operands.
__device__ __forceinline__ void merge1(float &s, float &c, float s2, float c2) {
  const float S = s + s2;
  const float bb = S - s;
  const float e = (s - (S - bb)) + (s2 - bb);
  c = (c + c2) - e;
  s = S;
}
__device__ __forceinline__ void kahan_merge(Acc32 &a, const Acc32 &b) {
  merge1(a.sx, a.cx, b.sx, b.cx);
  merge1(a.sy, a.cy, b.sy, b.cy);
  merge1(a.sz, a.cz, b.sz, b.cz);
}
__device__ __forceinline__ D3 acc_value(const Acc32 &a) {
  return d3((double)a.sx - (double)a.cx, (double)a.sy - (double)a.cy, (double)a.sz - (double)a.cz);
}
// Lane src's accumulator, all lanes taking part.
__device__ __forceinline__ Acc32 acc_shfl(const Acc32 &a, uint32_t src) {
  const unsigned full = 0xffffffffu;
  return Acc32{__shfl_sync(full, a.sx, src), __shfl_sync(full, a.sy, src), __shfl_sync(full, a.sz, src),
               __shfl_sync(full, a.cx, src), __shfl_sync(full, a.cy, src), __shfl_sync(full, a.cz, src)};
}

// One load group of U positions of a node's row (U = 4 or 8, the group starting at a multiple of
// U, so inside one block of the row): the partner records are gathered, every position's terms
// evaluated (a broken or missing bond's are discarded), the live ones added to the block's sum in
// position order, and -- once per group, only when some live stretch exceeds the lower edge of the
// band around snot -- the breaking decisions taken (FP32 above the band, FP64 inside it).
// bond_group_eval is the part after the gathers, on partner records already loaded (pq, uq; U may
// also be 2); bond_group gathers them and evaluates the same way.
template <int U>
__device__ __forceinline__ void bond_group_eval(const DevView &v, uint64_t nn, const float4 &pi4, const float4 &ui4,
                                                const uint32_t (&q)[U], const float4 (&pq)[U], const float4 (&uq)[U],
                                                Acc32 &a, bool brk, float slo, float shi, double snot,
                                                uint32_t *maskp, uint32_t *colw, uint32_t lane) {
  static_assert(U == 2 || U == 4 || U == 8, "groups inside one block of the row");
  BondTerms bt[U];
#pragma unroll
  for (int u = 0; u < U; ++u) bt[u] = bond32_terms(pi4, ui4, pq[u], uq[u]);
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (!(q[u] & kColBroken)) kahan_add(a, bt[u].g, bt[u].yx, bt[u].yy, bt[u].yz);
  if (brk) {
    bool any = false;
#pragma unroll
    for (int u = 0; u < U; ++u) any |= !(q[u] & kColBroken) && bt[u].str > slo;
    if (any) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!(q[u] & kColBroken) && bt[u].str > slo) {
          if (bt[u].str > shi) cut_bond(&maskp[u], lane, colw + 32 * u, q[u]);
          else band_check(v, nn, q[u], &maskp[u], lane, snot, colw + 32 * u);
        }
      }
    }
  }
}

template <int U, int W, int NC = 1>
__device__ __forceinline__ void bond_group(const DevView &v, uint64_t nn, const Rec32 *__restrict__ rec,
                                           const float4 &pi4, const float4 &ui4, const uint32_t (&q)[U], Acc32 &a,
                                           bool brk, float slo, float shi, double snot, uint32_t *maskp,
                                           uint32_t *colw, uint32_t lane) {
  static_assert(U == 4 || U == 8, "groups inside one block of the row");
  float4 pq[U], uq[U];
#pragma unroll
  for (int u = 0; u < U; ++u) ld_rec<W, NC>(rec + (q[u] & kColIndex), pq[u], uq[u]);
  BondTerms bt[U];
#pragma unroll
  for (int u = 0; u < U; ++u) bt[u] = bond32_terms(pi4, ui4, pq[u], uq[u]);
#pragma unroll
  for (int u = 0; u < U; ++u)
    if (!(q[u] & kColBroken)) kahan_add(a, bt[u].g, bt[u].yx, bt[u].yy, bt[u].yz);
  if (brk) {
    bool any = false;
#pragma unroll
    for (int u = 0; u < U; ++u) any |= !(q[u] & kColBroken) && bt[u].str > slo;
    if (any) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!(q[u] & kColBroken) && bt[u].str > slo) {
          if (bt[u].str > shi) cut_bond(&maskp[u], lane, colw + 32 * u, q[u]);
          else band_check(v, nn, q[u], &maskp[u], lane, snot, colw + 32 * u);
        }
      }
    }
  }
}

// Live bonds of a row at the start of the step (statistics only: a second read of the row's
// column entries, outside the bond loop).
__device__ __noinline__ uint32_t row_live(const uint32_t *colp, int dg) {
  uint32_t live = 0;
  for (int j = 0; j < dg; ++j) live += !(colp[32 * j] & kColBroken);
  return live;
}

// Per-node end of the FP32-form step, given the total force density f: force store,
// velocity-Verlet corrector in FP64 (timeloop.h:670-682), clamped nodes (timeloop.h:767-774),
// the next step's predictor (timeloop.h:537-540) into disp_next / rec_next, the particle's
// local-frame AABB of this step and the broad-phase movement bound. Warp-collective.
__device__ __forceinline__ void verlet_tail(const DevView &v, uint64_t nn, uint32_t k, const DevPart &P,
                                            const DevSimState &st, bool run, D3 f, const float4 &pi4,
                                            const float4 &ui4) {
  const uint64_t C3 = v.Ncap;
  const int32_t movable = P.movable;
  float i2 = 0.f;  // squared displacement increment of the next step (broad-phase bound)
  if (run) {
    st3(v.force, nn, C3, f);
    if (nonfinite(f.x) || nonfinite(f.y) || nonfinite(f.z)) atomicOr(&v.cnt->err, PD_DERR_NONFINITE);
    const D3 vi = ld3(v.vel_in, nn, C3);
    D3 vo = vi;
    D3 an = ld3(v.acc, nn, C3);
    const DevSimParams &sp = v.sp[P.sim];
    const bool clamped = movable && v.clamp_flag[nn];
    if (movable) {
      // velocity-Verlet corrector (timeloop.h:670-682)
      const D3 ao = an;
      if (v.afd && st.vconstraint && (int32_t)(k - sp.p0) == sp.pv_particle) st3(v.afd, nn, C3, ao);
      an = P.irho * f;
      vo = vi + sp.hdt * (ao + an);
      if (clamped) {  // timeloop.h:767-774
        vo = d3(0.0, 0.0, 0.0);
        an = d3(0.0, 0.0, 0.0);
      }
      st3(v.acc, nn, C3, an);
    }
    st3(v.vel_out, nn, C3, vo);
    // predictor of the next step (timeloop.h:537-540)
    const D3 d = ld3(v.disp, nn, C3);
    D3 dn;
    if (clamped) {
      dn = d3(0.0, 0.0, 0.0);
    } else {
      const D3 inc = sp.dt * vo + sp.hdt2 * an;
      dn = d + inc;
    }
    st3(v.disp_next, nn, C3, dn);
    const float ix = (float)(dn.x - d.x), iy = (float)(dn.y - d.y), iz = (float)(dn.z - d.z);
    i2 = ix * ix + iy * iy + iz * iz;
    const double *anx = v.anchor_next + 3 * (uint64_t)k;
    v.rec_next[nn].u = make_float4((float)(dn.x - anx[0]), (float)(dn.y - anx[1]), (float)(dn.z - anx[2]), 0.f);
  }
  // particle AABB of this step's positions in the particle's local frame
  {
    const bool contrib = run && movable;
    const float px = pi4.x + ui4.x, py = pi4.y + ui4.y, pz = pi4.z + ui4.z;
    float lo[3] = {contrib ? px : INFINITY, contrib ? py : INFINITY, contrib ? pz : INFINITY};
    float hi[3] = {contrib ? px : -INFINITY, contrib ? py : -INFINITY, contrib ? pz : -INFINITY};
    const uint32_t k0 = __shfl_sync(0xffffffffu, k, 0);
    const bool uniform = __all_sync(0xffffffffu, k == k0);
    if (uniform) {
      for (int o = 16; o > 0; o >>= 1) {
        for (int c = 0; c < 3; ++c) {
          lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
          hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
        }
      }
    }
    const bool writer = uniform ? ((threadIdx.x & 31) == 0) : contrib;
    if (writer && lo[0] <= hi[0]) {
      unsigned int *L = v.lrtb_local_next + 6 * (uint64_t)k;
      for (int c = 0; c < 3; ++c) {
        atomicMin(&L[c], fkey(lo[c]));
        atomicMax(&L[3 + c], fkey(hi[c]));
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) i2 = fmaxf(i2, __shfl_xor_sync(0xffffffffu, i2, o));
  if ((threadIdx.x & 31) == 0 && i2 > 0.f) {
    const double inc = sqrt((double)i2) * (1.0 + 1e-5);
    atomicMax(&v.cnt->stepmax_bits, (unsigned long long)__double_as_longlong(inc));
  }
}

// U: positions whose loads are issued together; MINB: minimum resident blocks per SM (register
// cap); W: 256-bit record loads; PF: the column entries (index + broken flag) of the next PF
// groups are loaded ahead of this group's partner records, so that the column stream's latency
// overlaps the gathers and arithmetic of the current group; FX: the FP64 non-bond work is
// done here (extra_force) instead of in a separate k_extra32 launch.
template <int U, int W, int PF, int FX, int NC = 1>
__device__ __forceinline__ void bond_node(const DevView &v, uint64_t n) {
  const bool valid = n < v.N;
  const uint64_t nn = valid ? n : 0;
  const uint32_t k = v.pid[nn];
  const DevPart &P = v.parts[k];
  const int32_t movable = P.movable;
  const DevSimState &st = v.ss[P.sim];
  const bool run = valid && st.active;
  const uint64_t C3 = v.Ncap;
  float4 pi4, ui4;
  ld_rec<W, NC>(v.rec + nn, pi4, ui4);
  Acc32 tot = {}, a = {};  // merged blocks so far, current block
  uint32_t live = 0;
  if (run && movable) {
    const uint32_t lane = (uint32_t)(nn & 31);
    const uint64_t sbase = v.slice_ptr[nn >> 5];
    const uint32_t *colp = v.col + sbase + lane;
    uint32_t *colw = const_cast<uint32_t *>(colp);  // broken flags of this node's entries
    uint32_t *maskp = v.mask + (sbase >> 5);
    const int dg = v.deg[nn];
    const bool brk = st.fracture && P.breakable && P.break_bonds;
    const float slo = P.snot_lo32, shi = P.snot_hi32;
    const Rec32 *__restrict__ rec = v.rec;
    if (v.stats) live = row_live(colp, dg);
    const int cl = chain_len(dg);
    int next = cl, merged = 0;
    int j = 0;
    // column entries (index + broken flag) of the next PF groups, loaded ahead (static
    // indices only, so that the ring stays in registers)
    uint32_t qb[PF > 0 ? PF : 1][U];
#pragma unroll
    for (int d = 0; d < PF; ++d) {
      if ((d + 1) * U <= dg) {
#pragma unroll
        for (int u = 0; u < U; ++u) qb[d][u] = ld_col<NC>(colp + 32 * (d * U + u));
      }
    }
    for (; j + U <= dg; j += U) {
      uint32_t q[U];
      if (PF > 0) {
#pragma unroll
        for (int u = 0; u < U; ++u) q[u] = qb[0][u];
#pragma unroll
        for (int d = 0; d + 1 < PF; ++d) {
#pragma unroll
          for (int u = 0; u < U; ++u) qb[d][u] = qb[d + 1][u];
        }
        if (j + (PF + 1) * U <= dg) {
#pragma unroll
          for (int u = 0; u < U; ++u) qb[PF - 1][u] = ld_col<NC>(colp + 32 * (j + PF * U + u));
        }
      } else {
#pragma unroll
        for (int u = 0; u < U; ++u) q[u] = ld_col<NC>(colp + 32 * (j + u));
      }
      if (j == next) {  // a new block of the row
        kahan_merge(tot, a);
        a = Acc32{};
        next += cl;
        ++merged;
      }
      bond_group<U, W, NC>(v, nn, rec, pi4, ui4, q, a, brk, slo, shi, P.snot, maskp + j, colw + 32 * j, lane);
    }
    if (j < dg) {  // the row's last dg - j < U positions as one group; missing ones count as broken
      uint32_t q[U];
#pragma unroll
      for (int u = 0; u < U; ++u) q[u] = (j + u < dg) ? ld_col<NC>(colp + 32 * (j + u)) : kColBroken;
      if (j == next) {
        kahan_merge(tot, a);
        a = Acc32{};
        ++merged;
      }
      bond_group<U, W, NC>(v, nn, rec, pi4, ui4, q, a, brk, slo, shi, P.snot, maskp + j, colw + 32 * j, lane);
    }
    kahan_merge(tot, a);  // the last block, then the empty ones: four merges in every form
    for (++merged; merged < 4; ++merged) kahan_merge(tot, Acc32{});
  }
  D3 f = d3(0.0, 0.0, 0.0);
  if (run) {
    f = acc_value(tot);
    if (FX) {  // the non-bond work of k_extra32, fused (same arithmetic, same order)
      if (extra_needed(v, nn, k, P, v.sp[P.sim], st, pi4, ui4)) f = f + extra_force(v, nn);
    } else if (v.extra_flag[nn]) {
      f = f + ld3(v.f_extra, nn, C3);
      v.extra_flag[nn] = 0;
    }
  }
  verlet_tail(v, nn, k, P, st, run, f, pi4, ui4);
  if (v.stats) {
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    if ((threadIdx.x & 31) == 0 && live) atomicAdd(&v.cnt->live_bonds, (unsigned long long)live);
  }
}

// bond_node's loop with the partner records of the next load group requested before the
// current group is evaluated and its column entries two groups ahead (small handles: with few
// warps per SM the gathers' latency is not hidden by other warps). The same positions in the same
// order as bond_node, the same sums. FP64 non-bond work fused; coherent loads where NC = 0.
template <int U, int NC = 1>
__device__ __forceinline__ void bond_node_ahead(const DevView &v, uint64_t n) {
  const bool valid = n < v.N;
  const uint64_t nn = valid ? n : 0;
  const uint32_t k = v.pid[nn];
  const DevPart &P = v.parts[k];
  const int32_t movable = P.movable;
  const DevSimState &st = v.ss[v.S == 1 ? 0u : P.sim];  // one simulation: no wait for P
  const bool run = valid && st.active;
  float4 pi4, ui4;
  ld_rec<1, NC>(v.rec + nn, pi4, ui4);
  // the row's first two groups of column entries and the first group's partner records are
  // requested before the node's flags arrive (any node's row is a valid address)
  const uint32_t lane = (uint32_t)(nn & 31);
  const uint64_t sbase = v.slice_ptr[nn >> 5];
  const uint32_t *colp = v.col + sbase + lane;
  const int dg = v.deg[nn];
  const Rec32 *__restrict__ rec = v.rec;
  uint32_t qc[U], qn[U];
  float4 pc[U], uc[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    qc[u] = u < dg ? ld_col<NC>(colp + 32 * u) : kColBroken;
    qn[u] = U + u < dg ? ld_col<NC>(colp + 32 * (U + u)) : kColBroken;
  }
#pragma unroll
  for (int u = 0; u < U; ++u) ld_rec<1, NC>(rec + (qc[u] & kColIndex), pc[u], uc[u]);
  Acc32 tot = {};
  uint32_t live = 0;
  if (run && movable) {
    uint32_t *colw = const_cast<uint32_t *>(colp);
    uint32_t *maskp = v.mask + (sbase >> 5);
    const bool brk = st.fracture && P.breakable && P.break_bonds;
    const float slo = P.snot_lo32, shi = P.snot_hi32;
    if (v.stats) live = row_live(colp, dg);
    const int cl = chain_len(dg), ng = (dg + U - 1) / U;
    int next = cl, merged = 0;
    Acc32 a = {};
    for (int g = 0; g < ng; ++g) {
      const int j = g * U;
      float4 pn[U], un[U];
#pragma unroll
      for (int u = 0; u < U; ++u) ld_rec<1, NC>(rec + (qn[u] & kColIndex), pn[u], un[u]);
      uint32_t qnn[U];
#pragma unroll
      for (int u = 0; u < U; ++u) qnn[u] = j + 2 * U + u < dg ? ld_col<NC>(colp + 32 * (j + 2 * U + u)) : kColBroken;
      if (j == next) {  // a new block of the row
        kahan_merge(tot, a);
        a = Acc32{};
        next += cl;
        ++merged;
      }
      bond_group_eval<U>(v, nn, pi4, ui4, qc, pc, uc, a, brk, slo, shi, P.snot, maskp + j, colw + 32 * j, lane);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        qc[u] = qn[u];
        qn[u] = qnn[u];
        pc[u] = pn[u];
        uc[u] = un[u];
      }
    }
    kahan_merge(tot, a);  // the last block, then the empty ones: four merges in every form
    for (++merged; merged < 4; ++merged) kahan_merge(tot, Acc32{});
  }
  D3 f = d3(0.0, 0.0, 0.0);
  if (run) {
    f = acc_value(tot);
    if (extra_needed(v, nn, k, P, v.sp[P.sim], st, pi4, ui4)) f = f + extra_force(v, nn);
  }
  verlet_tail(v, nn, k, P, st, run, f, pi4, ui4);
  if (v.stats) {
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    if ((threadIdx.x & 31) == 0 && live) atomicAdd(&v.cnt->live_bonds, (unsigned long long)live);
  }
}

// The bond loop of bond_node with L = 2 or 4 lanes per node (small handles: few nodes, long rows,
// so few warps that each wait on a long chain). Global thread t serves node t / L; lane s of the
// node takes whole blocks of its row (chain_len): block s with L = 4, blocks 2s and 2s + 1 with
// L = 2, in rounds of U positions; at the end the node's first lane merges the four block sums in
// row order, as bond_node does, so the sums are bond_node's bit for bit. The breaking decisions
// are taken by the lane that evaluated the bond. All lanes of a warp run the same number of rounds
// (the warp's longest block run); positions past a block's or the row's end count as broken. The
// non-bond work and the corrector run on the node's first lane.
template <int L, int U, int FX, int NC = 1>
__device__ __forceinline__ void bond_node_split(const DevView &v, uint64_t t) {
  static_assert((L == 2 || L == 4) && (U == 4 || U == 8), "two or four lanes per node, groups inside a block");
  const unsigned full = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t sub = lane & (L - 1), first = lane - sub;
  const uint64_t n = t / L;
  const bool valid = n < v.N;
  const uint64_t nn = valid ? n : 0;
  const uint32_t k = v.pid[nn];
  const DevPart &P = v.parts[k];
  const int32_t movable = P.movable;
  const DevSimState &st = v.ss[v.S == 1 ? 0u : P.sim];  // one simulation: no wait for P
  const bool run = valid && st.active;
  const uint64_t C3 = v.Ncap;
  float4 pi4, ui4;
  ld_rec<1, NC>(v.rec + nn, pi4, ui4);
  Acc32 A = {}, C = {};  // L = 2: the lane's first block once done; the current block
  uint32_t live = 0;
  const uint32_t lane_n = (uint32_t)(nn & 31);  // the node's lane in its 32-node slice
  const uint64_t sbase = v.slice_ptr[nn >> 5];
  const uint32_t *colp = v.col + sbase + lane_n;
  uint32_t *colw = const_cast<uint32_t *>(colp);
  uint32_t *maskp = v.mask + (sbase >> 5);
  const int dg = (run && movable) ? (int)v.deg[nn] : 0;
  const int cl = chain_len(dg), len = (4 / L) * cl, base = (int)sub * len;
  const bool brk = st.fracture && P.breakable && P.break_bonds;
  const float slo = P.snot_lo32, shi = P.snot_hi32;
  const Rec32 *__restrict__ rec = v.rec;
  if (v.stats && sub == 0 && dg) live = row_live(colp, dg);
  const int rounds = (int)__reduce_max_sync(full, (unsigned)((len + U - 1) / U));
  for (int r = 0; r < rounds; ++r) {
    const int m0 = r * U;
    if (L == 2 && m0 == cl) {  // the lane's second block
      A = C;
      C = Acc32{};
    }
    uint32_t q[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int m = m0 + u, j = base + m;
      q[u] = (m < len && j < dg) ? ld_col<NC>(colp + 32 * j) : kColBroken;
    }
    float4 pq[U], uq[U];
#pragma unroll
    for (int u = 0; u < U; ++u) ld_rec<1, NC>(rec + (q[u] & kColIndex), pq[u], uq[u]);
    BondTerms bt[U];
#pragma unroll
    for (int u = 0; u < U; ++u) bt[u] = bond32_terms(pi4, ui4, pq[u], uq[u]);
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (!(q[u] & kColBroken)) kahan_add(C, bt[u].g, bt[u].yx, bt[u].yy, bt[u].yz);
    if (brk) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!(q[u] & kColBroken) && bt[u].str > slo) {
          const int j = base + m0 + u;
          if (bt[u].str > shi) cut_bond(&maskp[j], lane_n, colw + 32 * j, q[u]);
          else band_check(v, nn, q[u], &maskp[j], lane_n, P.snot, colw + 32 * j);
        }
      }
    }
  }
  // the four block sums in row order, merged from zero as bond_node does
  Acc32 tot = {};
  if (L == 4) {
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const Acc32 x = acc_shfl(C, first + b);
      kahan_merge(tot, x);
    }
  } else {
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const Acc32 x = acc_shfl(A, first + b), y = acc_shfl(C, first + b);
      kahan_merge(tot, x);
      kahan_merge(tot, y);
    }
  }
  const bool lead = run && sub == 0;
  D3 f = d3(0.0, 0.0, 0.0);
  if (lead) {
    f = acc_value(tot);
    if (!FX && v.extra_flag[nn]) {
      f = f + ld3(v.f_extra, nn, C3);
      v.extra_flag[nn] = 0;
    }
  }
  if (FX) {  // FP64 non-bond work: a node's lanes share its listed contact candidates
    const bool need = __shfl_sync(full, lead && extra_needed(v, nn, k, P, v.sp[P.sim], st, pi4, ui4), first);
    if (need) {
      if (v.cand_n[nn] == kCandCells) {  // the cell walk: one lane
        if (lead) f = f + extra_force(v, nn);
      } else {
        const D3 e = extra_force_lanes<L>(v, nn, sub, first);
        if (lead) f = f + e;
      }
    }
  }
  verlet_tail(v, nn, k, P, st, lead, f, pi4, ui4);
  if (v.stats) {
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(full, live, o);
    if (lane == 0 && live) atomicAdd(&v.cnt->live_bonds, (unsigned long long)live);
  }
}

template <int U, int MINB>
__global__ void __launch_bounds__(128, MINB) k_bond32a(const __grid_constant__ DevView v) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && v.xcount) {
    v.xcount[1] = 0;
    v.cnt->xall = 0;
  }
  bond_node_ahead<U>(v, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <int L, int U, int MINB>
__global__ void __launch_bounds__(128, MINB) k_bond32l(const __grid_constant__ DevView v) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && v.xcount) {
    v.xcount[1] = 0;
    v.cnt->xall = 0;
  }
  bond_node_split<L, U, 1>(v, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <int U, int MINB, int W, int PF, int FX>
__global__ void __launch_bounds__(128, MINB) k_bond32(const __grid_constant__ DevView v) {
  // the work lists of k_extra32 have been consumed: k_end_step builds the next particle list
  if (blockIdx.x == 0 && threadIdx.x == 0 && v.xcount) {
    v.xcount[1] = 0;
    v.cnt->xall = 0;
  }
  bond_node<U, W, PF, FX>(v, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// Staged form of the bond kernel: one block of kStageNodes nodes first copies the contiguous
// range of node records its bonds read into shared memory with bulk asynchronous copies
// (cp.async.bulk, completion on an mbarrier), then gathers every partner from shared memory
// instead of L1/L2. Blocks whose range does not fit (win_cnt == 0), or whose copy misses the
// wait limit, read global memory as the plain kernel does; results are the same either way.
constexpr uint32_t kStageWaitPolls = 1u << 22;  // bounded wait (~0.5 s) for the staging copy

template <int U, int PF>
__global__ void __launch_bounds__(kStageNodes, 1) k_bond32s(const __grid_constant__ DevView v) {
  extern __shared__ __align__(128) unsigned char stage_raw[];
  Rec32 *win = reinterpret_cast<Rec32 *>(stage_raw);
  __shared__ __align__(8) uint64_t bar;
  if (blockIdx.x == 0 && threadIdx.x == 0 && v.xcount) {  // as in k_bond32
    v.xcount[1] = 0;
    v.cnt->xall = 0;
  }
  const uint32_t wlo = v.win_lo[blockIdx.x];
  const uint32_t wcnt = v.win_cnt[blockIdx.x];
  bool staged = wcnt != 0;
  bool copy_done = true;
  if (staged) {
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      const uint32_t bytes = wcnt * (uint32_t)sizeof(Rec32);
      mbar_expect_tx(&bar, bytes);
      const char *src = reinterpret_cast<const char *>(v.rec + wlo);
      for (uint32_t off = 0; off < bytes; off += 32768u)
        bulk_g2s(stage_raw + off, src + off, bytes - off < 32768u ? bytes - off : 32768u, &bar);
    }
    __syncthreads();  // the barrier is initialised before anyone polls it
    copy_done = mbar_wait_bounded(&bar, 0, kStageWaitPolls);
    staged = __syncthreads_and(copy_done) != 0;
    if (!staged && threadIdx.x == 0) atomicOr(&v.cnt->err, PD_DERR_STAGE_TIMEOUT);
  }
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = n < v.N;
  const uint64_t nn = valid ? n : 0;
  const uint32_t k = v.pid[nn];
  const DevPart &P = v.parts[k];
  const int32_t movable = P.movable;
  const DevSimState &st = v.ss[P.sim];
  const bool run = valid && st.active;
  const uint64_t C3 = v.Ncap;
  float4 pi4, ui4;
  ld_rec<1>(v.rec + nn, pi4, ui4);
  Acc32 tot = {}, a = {};  // merged blocks so far, current block (bond_node)
  static_assert(U == 4 || U == 8, "groups inside one block of the row");
  uint32_t live = 0;
  if (run && movable) {
    const uint32_t lane = (uint32_t)(nn & 31);
    const uint64_t sbase = v.slice_ptr[nn >> 5];
    const uint32_t *colp = v.col + sbase + lane;
    uint32_t *colw = const_cast<uint32_t *>(colp);
    uint32_t *maskp = v.mask + (sbase >> 5);
    const int dg = v.deg[nn];
    const bool brk = st.fracture && P.breakable && P.break_bonds;
    const float slo = P.snot_lo32, shi = P.snot_hi32;
    const Rec32 *__restrict__ rec = v.rec;
    if (v.stats) live = row_live(colp, dg);
    // partner record: shared memory when staged (and inside the staged range), else global
    auto partner = [&](uint32_t q, float4 &p, float4 &u) {
      const uint32_t o = q - wlo;
      if (staged && o < wcnt) {
        p = win[o].p;
        u = win[o].u;
      } else {
        ld_rec<1>(rec + q, p, u);
      }
    };
    const int cl = chain_len(dg);
    int next = cl, merged = 0;
    int j = 0;
    uint32_t qb[PF][U];
#pragma unroll
    for (int d = 0; d < PF; ++d) {
      if ((d + 1) * U <= dg) {
#pragma unroll
        for (int u = 0; u < U; ++u) qb[d][u] = __ldg(colp + 32 * (d * U + u));
      }
    }
    for (; j + U <= dg; j += U) {
      uint32_t q[U];
#pragma unroll
      for (int u = 0; u < U; ++u) q[u] = qb[0][u];
#pragma unroll
      for (int d = 0; d + 1 < PF; ++d) {
#pragma unroll
        for (int u = 0; u < U; ++u) qb[d][u] = qb[d + 1][u];
      }
      if (j + (PF + 1) * U <= dg) {
#pragma unroll
        for (int u = 0; u < U; ++u) qb[PF - 1][u] = __ldg(colp + 32 * (j + PF * U + u));
      }
      if (j == next) {  // a new block of the row
        kahan_merge(tot, a);
        a = Acc32{};
        next += cl;
        ++merged;
      }
      float4 pq[U], uq[U];
#pragma unroll
      for (int u = 0; u < U; ++u) partner(q[u] & kColIndex, pq[u], uq[u]);
      BondTerms bt[U];  // as in bond_node: terms unconditionally, live ones summed in order
#pragma unroll
      for (int u = 0; u < U; ++u) bt[u] = bond32_terms(pi4, ui4, pq[u], uq[u]);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (!(q[u] & kColBroken)) {
          kahan_add(a, bt[u].g, bt[u].yx, bt[u].yy, bt[u].yz);
          if (brk && bt[u].str > slo) {
            if (bt[u].str > shi) cut_bond(&maskp[j + u], lane, colw + 32 * (j + u), q[u]);
            else band_check(v, nn, q[u], &maskp[j + u], lane, P.snot, colw + 32 * (j + u));
          }
        }
      }
    }
    for (; j < dg; ++j) {
      if (j == next) {
        kahan_merge(tot, a);
        a = Acc32{};
        next += cl;
        ++merged;
      }
      const uint32_t q = __ldg(colp + 32 * j);
      if (q & kColBroken) continue;
      float4 pq, uq;
      partner(q, pq, uq);
      const BondTerms b = bond32_terms(pi4, ui4, pq, uq);
      kahan_add(a, b.g, b.yx, b.yy, b.yz);
      const float str = b.str;
      if (brk && str > slo) {
        if (str > shi) cut_bond(&maskp[j], lane, colw + 32 * j, q);
        else band_check(v, nn, q, &maskp[j], lane, P.snot, colw + 32 * j);
      }
    }
    kahan_merge(tot, a);  // the last block, then the empty ones: four merges in every form
    for (++merged; merged < 4; ++merged) kahan_merge(tot, Acc32{});
  }
  D3 f = d3(0.0, 0.0, 0.0);
  if (run) {
    f = acc_value(tot);
    if (v.extra_flag[nn]) {
      f = f + ld3(v.f_extra, nn, C3);
      v.extra_flag[nn] = 0;
    }
  }
  verlet_tail(v, nn, k, P, st, run, f, pi4, ui4);
  if (v.stats) {
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    if ((threadIdx.x & 31) == 0 && live) atomicAdd(&v.cnt->live_bonds, (unsigned long long)live);
  }
  // a copy that missed its wait limit may still be writing shared memory: let it land
  if (!copy_done && threadIdx.x == 0) (void)mbar_wait_bounded(&bar, 0, kStageWaitPolls);
  __syncthreads();
}

// ---- the persistent step (small handles) ------------------------------------------------
//
// A handle of a few tens of thousands of nodes steps in tens of microseconds, a good part of it
// spent between the ~10 kernels of a step graph. k_persist runs all requested steps in one
// cooperative launch, its phases separated by grid-wide barriers: per step the bond phase (the
// FP32 bond loop with the FP64 non-bond work fused, the corrector and the next predictor), the
// particles' end of step, then the simulations' advance with the next step's rebuild decision;
// the broad phase runs only in the steps that rebuild (clear, count, scan, scatter, candidates).
// Every phase calls the same device code as the per-phase kernels (pd_bp.cuh, pd_end.cuh,
// bond_node), so the results are those of the step graph bit for bit. Per step: the bond phase,
// a barrier, the end of step (its last block advancing the simulations), a barrier. Records and column entries
// are written from one step to the next inside the launch, so they are read with coherent loads.
//
// The blocks meet at a barrier of their own (GridBarrier) rather than a library grid sync, so
// that every wait is bounded: a block that waits longer than kBarrierWaitNs sets
// PD_DERR_BARRIER_TIMEOUT and every block leaves the launch at its next barrier. The launch is
// cooperative, so all blocks are resident at once and every barrier is reachable.
constexpr int kPersistThreads = 512;  // one block per SM (128 registers a thread)
constexpr uint64_t kBarrierWaitNs = 2000000000ull;  // 2 s; a phase of a small handle takes microseconds

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Two words, zeroed before each launch: the arrival counter (barrier k of the launch waits until
// k * gridDim.x blocks have arrived) and the release counter of barriers with a last-block action.
// sync() and sync_last() return false when the launch must stop (a wait ran out here or in another
// block).
struct GridBarrier {
  uint32_t *count;
  uint32_t *err;
  uint32_t target;   // arrivals the next barrier waits for
  uint32_t release;  // last-block actions done so far

  // Thread 0: bounded wait until *word >= want; false when it ran out or another block's did.
  __device__ bool wait_for(const uint32_t *word, uint32_t want) {
    const uint64_t t0 = global_ns();
    uint32_t polls = 0, seen;
    asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(seen) : "l"(word) : "memory");
    while (seen < want) {
      if ((++polls & 255u) == 0) {
        if (*(volatile uint32_t *)err & PD_DERR_BARRIER_TIMEOUT) return false;
        if (global_ns() - t0 > kBarrierWaitNs) {
          atomicOr(err, PD_DERR_BARRIER_TIMEOUT);
          return false;
        }
      }
      asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(seen) : "l"(word) : "memory");
    }
    return !(*(volatile uint32_t *)err & PD_DERR_BARRIER_TIMEOUT);
  }

  // Thread 0, after a block barrier: arrive; returns the number of blocks arrived so far, this one
  // included. The release half of the atomic publishes the block's writes (ordered before it by
  // the block barrier), its acquire half lets the last arrival see every other block's.
  __device__ uint32_t arrive() {
    uint32_t seen;
    asm volatile("atom.add.acq_rel.gpu.u32 %0, [%1], 1;" : "=r"(seen) : "l"(count) : "memory");
    return seen + 1;
  }

  __device__ bool sync() {
    __shared__ uint32_t ok;
    target += gridDim.x;
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t seen = arrive();
      ok = (seen >= target || wait_for(count, target)) ? 1u : 0u;
    }
    __syncthreads();
    return ok != 0;
  }

  // A barrier whose last block to arrive runs fn (all its threads) before any block leaves.
  template <class F>
  __device__ bool sync_last(F &&fn) {
    __shared__ uint32_t last, ok;
    target += gridDim.x;
    ++release;
    __syncthreads();
    if (threadIdx.x == 0) last = arrive() == target ? 1u : 0u;
    __syncthreads();
    if (last) {
      fn();
      __syncthreads();
      if (threadIdx.x == 0) {
        asm volatile("st.release.gpu.u32 [%0], %1;" ::"l"(count + 1), "r"(release) : "memory");
        ok = !(*(volatile uint32_t *)err & PD_DERR_BARRIER_TIMEOUT);
      }
    } else if (threadIdx.x == 0) {
      ok = wait_for(count + 1, release) ? 1u : 0u;
    }
    __syncthreads();
    return ok != 0;
  }
};

// Sum over the block (every thread gets it).
__device__ __forceinline__ uint32_t block_sum(uint32_t x, uint32_t *sh) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[w] = x;
  __syncthreads();
  uint32_t s = 0;
  for (int i = 0; i < nw; ++i) s += sh[i];
  return s;
}

// Inclusive scan over the block; *total receives the block's sum.
__device__ __forceinline__ uint32_t block_incl_scan(uint32_t x, uint32_t *sh, uint32_t *total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) sh[w] = x;
  __syncthreads();
  uint32_t before = 0, tot = 0;
  for (int i = 0; i < nw; ++i) {
    if (i < w) before += sh[i];
    tot += sh[i];
  }
  *total = tot;
  return x + before;
}

// start[i] = count[0] + ... + count[i-1] over the cell table (T entries): each block sums its
// contiguous range, then (after one barrier) scans it from the sum of the ranges before it.
__device__ __forceinline__ bool persist_scan(const PersistArgs &a, GridBarrier &bar) {
  __shared__ uint32_t sh[kPersistThreads / 32];
  const uint64_t G = gridDim.x, R = (a.T + G - 1) / G;
  const uint64_t lo = min((uint64_t)a.T, (uint64_t)blockIdx.x * R), hi = min((uint64_t)a.T, lo + R);
  uint32_t s = 0;
  for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += a.count[i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) a.sums[blockIdx.x] = s;
  if (!bar.sync()) return false;
  uint32_t o = 0;
  for (uint32_t i = threadIdx.x; i < blockIdx.x; i += blockDim.x) o += a.sums[i];
  o = block_sum(o, sh);
  for (uint64_t base = lo; base < hi; base += blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    const uint32_t x = i < hi ? a.count[i] : 0u;
    uint32_t tot;
    const uint32_t incl = block_incl_scan(x, sh, &tot);
    if (i < hi) a.start[i] = o + incl - x;
    o += tot;
  }
  return true;
}

template <int L>
__global__ void __launch_bounds__(kPersistThreads, 1) k_persist(const __grid_constant__ PersistArgs a) {
  GridBarrier bar{a.bar, &a.v[0].cnt->err, 0u, 0u};
  const uint64_t gtid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t gsize = (uint64_t)gridDim.x * blockDim.x;
  // warps are dealt round-robin over the blocks (one per SM), so that a small handle's nodes
  // spread over every SM
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t gwarp = (uint64_t)(threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  const uint64_t nwarps = gsize >> 5;
  {  // the first step's rebuild decision; wall reactions restart (k_bp_decide)
    const DevView &v = a.v[a.cur0 & 1];
    if (gtid == 0) {
      bp_decide(v, a.half_skin);
      v.cnt->end_blocks = 0;  // the end-of-step tickets (a launch stopped at a barrier leaves them set)
    }
    for (uint64_t i = gtid; i < v.S; i += gsize)
      for (int k = 0; k < 18; ++k) v.ss[i].react[k] = 0.0;
  }
  if (!bar.sync()) return;
  for (uint32_t step = 0; step < a.nsteps; ++step) {
    const DevView &v = a.v[(a.cur0 + step) & 1];
    if (*(volatile const uint32_t *)&v.cnt->rebuild) {  // the broad phase (pd_bp.cuh)
      if (gtid == 0 && v.xcount) v.xcount[0] = 0;
      for (uint64_t i = gtid; i < a.T; i += gsize) a.count[i] = 0;
      if (!bar.sync()) return;
      for (uint64_t n = gtid; n < v.N; n += gsize) bp_count_node(v, n, a.count, a.key, a.slot, a.mask);
      if (!bar.sync()) return;
      if (!persist_scan(a, bar) || !bar.sync()) return;
      for (uint64_t n = gtid; n < v.N; n += gsize) bp_scatter_node(n, a.start, a.key, a.slot, a.sorted);
      if (!bar.sync()) return;
      {  // four nodes per warp
        __shared__ uint32_t csh[kPersistThreads / 32][kCandQuadWords];
        for (uint64_t w = gwarp; w * 4 < v.N; w += nwarps)
          bp_candidates_quad(v, w * 4, lane, a.count, a.start, a.sorted, a.mask, a.cand, a.cand_n, a.cap,
                             csh[threadIdx.x >> 5]);
      }
      if (!bar.sync()) return;
    }
    // bond phase: whole warps take 32 threads' worth of nodes (the bond loop is warp-collective)
    if (gtid == 0 && v.xcount) {
      v.xcount[1] = 0;
      v.cnt->xall = 0;
    }
    if constexpr (L == 1) {  // one lane per node, partner records gathered a group ahead
      for (uint64_t w = gwarp; w * 32 < v.N; w += nwarps) bond_node_ahead<4, 0>(v, w * 32 + lane);
    } else {  // L lanes per node (bond_node_split)
      for (uint64_t w = gwarp; w * 32 < v.N * L; w += nwarps)
        bond_node_split<L, 4, 1, 0>(v, w * 32 + lane);
    }
    // end of step, one warp per particle (k_end_step_w): after one more barrier over all blocks,
    // or, for a handle of at most one particle per warp of a block, in the last block to arrive
    // at the end barrier (one barrier less per step). That block then advances the simulations
    // and takes the next step's rebuild decision (k_bp_decide).
    const bool fold = v.P <= kPersistThreads / 32;
    if (!fold) {
      if (!bar.sync()) return;
      for (uint64_t k = gwarp; k < v.P; k += nwarps) end_particle_warp(v, (uint32_t)k, lane);
    }
    const bool more = step + 1 < a.nsteps;
    const DevView &vn = a.v[(a.cur0 + step + 1) & 1];
    if (!bar.sync_last([&] {
          if (fold) {
            if ((threadIdx.x >> 5) < v.P) end_particle_warp(v, threadIdx.x >> 5, lane);
            __syncthreads();
          }
          end_step_advance(v, threadIdx.x, blockDim.x, more, a.half_skin);
          if (more)  // the next step's wall reactions restart (other fields than the advance's)
            for (uint32_t i = threadIdx.x; i < vn.S; i += blockDim.x)
              for (int k = 0; k < 18; ++k) vn.ss[i].react[k] = 0.0;
        }))
      return;
  }
}

static const void *persist_kernel(int lanes) {
  switch (lanes) {
    case 2: return (const void *)k_persist<2>;
    case 4: return (const void *)k_persist<4>;
    default: return (const void *)k_persist<1>;
  }
}

int persist_threads() { return kPersistThreads; }

// Blocks of k_persist that fit on the current device at once (its grid may not exceed them).
int persist_max_blocks(int lanes) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, persist_kernel(lanes), kPersistThreads, 0) != cudaSuccess)
    return 0;
  return sms * per;
}

cudaError_t launch_persist(const PersistArgs &a, uint32_t grid, int lanes, cudaStream_t s) {
  void *args[] = {const_cast<PersistArgs *>(&a)};
  return cudaLaunchCooperativeKernel(persist_kernel(lanes), dim3(grid), dim3(kPersistThreads), args, 0, s);
}

int prepare_staged_kernels(uint32_t smem_bytes) {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void *fn) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
  };
  set((const void *)k_bond32s<4, 1>);
  set((const void *)k_bond32s<4, 2>);
  set((const void *)k_bond32s<4, 3>);
  set((const void *)k_bond32s<8, 1>);
  return e == cudaSuccess ? PD_OK : PD_ECUDA;
}


__global__ void k_stage_windows(const __grid_constant__ DevView v, uint32_t *win_lo, uint32_t *win_cnt) {
  const uint64_t b = blockIdx.x;
  const uint64_t n0 = b * kStageNodes, n1 = min(v.N, n0 + kStageNodes);
  uint32_t lo = (uint32_t)n0, hi = (uint32_t)(n1 - 1);
  const uint64_t e0 = v.slice_ptr[n0 / 32], e1 = v.slice_ptr[(n1 + 31) / 32];
  for (uint64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const uint32_t q = v.col[e];
    if (q != kNoCol) {  // a bond, live or broken
      lo = min(lo, q & kColIndex);
      hi = max(hi, q & kColIndex);
    }
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  __shared__ uint32_t slo[32], shi[32];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    slo[w] = lo;
    shi[w] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
      lo = min(lo, slo[i]);
      hi = max(hi, shi[i]);
    }
    const uint64_t cnt = (uint64_t)hi - lo + 1;
    win_lo[b] = lo;
    win_cnt[b] = cnt <= kStageMaxRecords ? (uint32_t)cnt : 0u;
  }
}

void launch_stage_windows(const DevView &v, uint32_t *win_lo, uint32_t *win_cnt, cudaStream_t s) {
  const uint64_t nb = (v.N + kStageNodes - 1) / kStageNodes;
  if (nb) k_stage_windows<<<(unsigned)nb, 256, 0, s>>>(v, win_lo, win_cnt);
}

// FP32 form: broken flags of the column entries from the live masks (after the masks were
// restored from a snapshot or set from a saved Connectivity).
__global__ void k_col_flags(const __grid_constant__ DevView v) {
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.N) return;
  const uint32_t lane = (uint32_t)(n & 31);
  const uint64_t sbase = v.slice_ptr[n >> 5];
  uint32_t *col = const_cast<uint32_t *>(v.col) + sbase + lane;
  const uint32_t *maskp = v.mask + (sbase >> 5);
  const int dg = v.deg[n];
  for (int j = 0; j < dg; ++j) {
    const uint32_t q = col[32 * j] & kColIndex;
    col[32 * j] = ((maskp[j] >> lane) & 1u) ? q : (q | kColBroken);
  }
}

void launch_col_flags(const DevView &v, cudaStream_t s) {
  if (v.N) k_col_flags<<<(unsigned)((v.N + 127) / 128), 128, 0, s>>>(v);
}

// A_next := this step's predicted displacement of each particle's anchor node.
__global__ void k_anchor_next(DevView v) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= v.P) return;
  const uint32_t a = v.parts[k].anchor;
  for (int c = 0; c < 3; ++c) v.anchor_next[3 * (uint64_t)k + c] = v.disp[a + c * v.Ncap];
}

// Shortest setup bond of every particle (FP64 reference positions), for the breaking band:
// the squared length's bits (a non-negative double orders like its bits) min-reduced per
// particle into d2min[P], which must start at all ones.
__global__ void k_xi_min(const __grid_constant__ DevView v, unsigned long long *d2min) {
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = n < v.N;
  const uint64_t nn = valid ? n : 0;
  unsigned long long m = ~0ull;
  if (valid) {
    const uint32_t lane = (uint32_t)(nn & 31);
    const uint32_t *colp = v.col + v.slice_ptr[nn >> 5] + lane;
    const int dg = v.deg[nn];
    const D3 pi = ld3(v.pos, nn, v.Ncap);
    for (int j = 0; j < dg; ++j) {
      const uint32_t q = colp[32 * j] & kColIndex;
      const D3 d = ld3(v.pos, q, v.Ncap) - pi;
      const double d2 = (d.x * d.x + d.y * d.y) + d.z * d.z;
      m = min(m, (unsigned long long)__double_as_longlong(d2));
    }
  }
  const uint32_t k = v.pid[nn];
  const uint32_t k0 = __shfl_sync(0xffffffffu, k, 0);
  if (__all_sync(0xffffffffu, k == k0)) {
    for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m != ~0ull) atomicMin(&d2min[k0], m);
  } else if (valid && m != ~0ull) {
    atomicMin(&d2min[k], m);
  }
}

__global__ void k_set_xi_min(DevView v, const unsigned long long *d2min) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= v.P) return;
  const unsigned long long m = d2min[k];
  // rounded down a little: a lower bound of every bond length of the particle
  v.parts[k].xi_min = m == ~0ull ? INFINITY : sqrt(__longlong_as_double((long long)m)) * (1.0 - 1e-12);
}

void launch_xi_min(const DevView &v, unsigned long long *d2min, cudaStream_t s) {
  if (v.N) k_xi_min<<<(unsigned)((v.N + 127) / 128), 128, 0, s>>>(v, d2min);
  if (v.P) k_set_xi_min<<<(v.P + 127) / 128, 128, 0, s>>>(v, d2min);
}

void launch_anchor_next(const DevView &v, cudaStream_t s) {
  if (v.P) k_anchor_next<<<(v.P + 127) / 128, 128, 0, s>>>(v);
}

// Bond-kernel variants the autotuner chooses from: k_bond32 <positions per load group, min
// blocks/SM, 256-bit record loads, column prefetch, fused non-bond work> with 128-thread blocks
// (0-9, 18-20) and with 32/64-thread blocks (14-17), the staged k_bond32s (10-13), k_bond32l with
// 2 or 4 lanes per node (21-24) and k_bond32a, one lane per node gathering a group ahead (25-27).
const int kNumBondVariants = 28;

int num_bond_variants() { return kNumBondVariants; }

void launch_step_fp32c(const DevView &v, int variant, cudaStream_t s) {
  const uint64_t blocks = (v.N + 127) / 128;
  if (!blocks) return;
  const unsigned b = (unsigned)blocks;
  // nothing to stage (or the ranges not computed): the plain kernel
  if (variant >= kFirstStagedVariant && variant < kFirstStagedVariant + 4 && !v.win_max) variant = 3;
  const bool fused_extra = (variant >= 6 && variant <= 9) || (variant >= 14 && variant <= 16) || variant == 19 ||
                           variant >= 21;
  if (!fused_extra) k_extra32<<<152 * 8, 128, 0, s>>>(v);
  const unsigned bs = (unsigned)((v.N + kStageNodes - 1) / kStageNodes);
  const size_t sm = (size_t)v.win_max * sizeof(Rec32);
  switch (variant) {
    case 1: k_bond32<4, 6, 1, 1, 0><<<b, 128, 0, s>>>(v); break;
    case 2: k_bond32<4, 4, 1, 2, 0><<<b, 128, 0, s>>>(v); break;
    case 3: k_bond32<4, 6, 1, 2, 0><<<b, 128, 0, s>>>(v); break;
    case 4: k_bond32<8, 4, 1, 1, 0><<<b, 128, 0, s>>>(v); break;
    case 5: k_bond32<4, 4, 1, 0, 0><<<b, 128, 0, s>>>(v); break;
    case 6: k_bond32<4, 4, 1, 1, 1><<<b, 128, 0, s>>>(v); break;
    case 7: k_bond32<4, 4, 1, 2, 1><<<b, 128, 0, s>>>(v); break;
    case 8: k_bond32<4, 6, 1, 1, 1><<<b, 128, 0, s>>>(v); break;
    case 9: k_bond32<4, 6, 1, 2, 1><<<b, 128, 0, s>>>(v); break;
    case 10: k_bond32s<4, 1><<<bs, kStageNodes, sm, s>>>(v); break;
    case 11: k_bond32s<4, 2><<<bs, kStageNodes, sm, s>>>(v); break;
    case 12: k_bond32s<4, 3><<<bs, kStageNodes, sm, s>>>(v); break;
    case 13: k_bond32s<8, 1><<<bs, kStageNodes, sm, s>>>(v); break;
    // small handles: a few hundred 128-thread blocks leave some SMs one block more than others;
    // 32- and 64-thread blocks of the same kernels spread the warps evenly
    case 14: k_bond32<4, 4, 1, 1, 1><<<(unsigned)((v.N + 31) / 32), 32, 0, s>>>(v); break;
    case 15: k_bond32<4, 4, 1, 2, 1><<<(unsigned)((v.N + 31) / 32), 32, 0, s>>>(v); break;
    case 16: k_bond32<4, 4, 1, 2, 1><<<(unsigned)((v.N + 63) / 64), 64, 0, s>>>(v); break;
    case 17: k_bond32<4, 6, 1, 2, 0><<<(unsigned)((v.N + 63) / 64), 64, 0, s>>>(v); break;
    // 5 blocks/SM (96 registers, no spills)
    case 18: k_bond32<4, 5, 1, 1, 0><<<b, 128, 0, s>>>(v); break;
    case 19: k_bond32<4, 5, 1, 1, 1><<<b, 128, 0, s>>>(v); break;
    case 20: k_bond32<8, 5, 1, 1, 0><<<b, 128, 0, s>>>(v); break;
    // L lanes per node (bond_node_split): small handles
    case 21: k_bond32l<2, 4, 4><<<(unsigned)((2 * v.N + 127) / 128), 128, 0, s>>>(v); break;
    case 22: k_bond32l<2, 8, 4><<<(unsigned)((2 * v.N + 127) / 128), 128, 0, s>>>(v); break;
    case 23: k_bond32l<4, 4, 4><<<(unsigned)((4 * v.N + 127) / 128), 128, 0, s>>>(v); break;
    case 24: k_bond32l<4, 8, 4><<<(unsigned)((4 * v.N + 127) / 128), 128, 0, s>>>(v); break;
    // one lane per node, partner records gathered a group ahead (small handles)
    case 25: k_bond32a<4, 4><<<b, 128, 0, s>>>(v); break;
    case 26: k_bond32a<4, 4><<<(unsigned)((v.N + 31) / 32), 32, 0, s>>>(v); break;
    case 27: k_bond32a<2, 4><<<b, 128, 0, s>>>(v); break;
    default: k_bond32<4, 4, 1, 1, 0><<<b, 128, 0, s>>>(v); break;
  }
}

}  // namespace pdg
