// pd_device.cuh -- device helpers shared by the step kernels: SoA loads/stores and the
// reference's contact, wall and box tests (contact.h), written in its FP64 evaluation order.
#ifndef PD_DEVICE_CUH
#define PD_DEVICE_CUH
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

#include "pd_engine.h"
#include "pd_math.cuh"

namespace pdg {


__device__ __forceinline__ D3 ld3(const double *a, uint64_t n, uint64_t cap) {
  return d3(a[n], a[n + cap], a[n + 2 * cap]);
}
__device__ __forceinline__ void st3(double *a, uint64_t n, uint64_t cap, D3 v) {
  a[n] = v.x;
  a[n + cap] = v.y;
  a[n + 2 * cap] = v.z;
}

__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// intersects_box_fext<3> (contact.h:1143-1183): only box A is extended by c.
__device__ __forceinline__ bool intersects_fext(const double *A, const double *B, double c) {
  double A_min_x = A[0] - c, A_min_y = A[1] - c, A_min_z = A[2] - c;
  double A_max_x = A[3] + c, A_max_y = A[4] + c, A_max_z = A[5] + c;
  return (A_min_x <= B[3]) && (A_max_x >= B[0]) && (A_max_y >= B[1]) && (A_min_y <= B[4]) &&
         (A_min_z <= B[5]) && (A_max_z >= B[2]);
}

// within_interior_fext (contact.h:1229-1243) with its 2D indexing of 3D boxes.
__device__ __forceinline__ bool within_interior(const double *A, const double *B, double c) {
  double A_Left = A[0] - c, A_Right = A[1] + c, A_Top = A[2] + c, A_Bottom = A[3] - c;
  return (B[0] < A_Left) && (A_Right < B[1]) && (B[2] > A_Top) && (B[3] < A_Bottom);
}

// Normal, damping and friction force densities of one node-node contact, computed from
// the point of view of the "C" node as update_contact_force_by_boundary does
// (contact.h:798-934). fc is always set; fd/ff only when has_fd/has_ff.
struct PairForce {
  D3 fc, fd, ff;
  bool has_fd, has_ff;
};

__device__ __forceinline__ void pair_force(D3 dir, double dn, double len_ref, double sc,
                                           double N_vol, double rho_C, D3 velC, D3 velN,
                                           const DevSimParams &sp, const DevSimState &st,
                                           PairForce &o) {
  D3 unit = dir / dn;
  double s = (dn - len_ref) / len_ref;
  double fmag = (sc * s) * N_vol;
  o.fc = fmag * unit;
  double fcn = norm3(o.fc);
  o.has_fd = false;
  o.has_ff = false;
  if (st.damping) {
    D3 rel = velC - velN;
    double rvp = dot3(rel, unit);
    D3 rvn = rvp * unit;
    double dc = (sp.zeta2 * sqrt(sc * rho_C)) * sqrt(N_vol);
    o.fd = (-dc) * rvn;
    o.has_fd = true;
  }
  if (st.friction) {
    D3 rel = velC - velN;
    double rd = dot3(rel, unit);
    D3 rvt = rel - rd * unit;
    double rvtn = norm3(rvt);
    if (rvtn > 0) {
      D3 tu = rvt / norm3(rvt);
      double fm = (-sp.mu) * fcn;
      if (rvtn < ((sp.mu * fcn) * sp.dt) / rho_C) fm = ((-rvtn) / rho_C) / sp.dt;
      o.ff = fm * tu;
      o.has_ff = true;
    }
  }
}

// segment_mass<3> + wall_side_force_update<3> (contact.h:14-39, 381-502) for one face.
__device__ __forceinline__ void wall_face(double dist, int dir, D3 vel, double vol, double rho,
                                          D3 &f, double wspeed, int face,
                                          const DevSimParams &sp, DevSimState &st, bool reaction) {
  const double R = sp.Rc;
  if (!(fabs(dist) <= R)) return;
  double d = fabs(dist);
  double rd = R - d;
  double area = (sp.pi3 * (rd * rd)) * (2 * R - d);
  double w = R * R - d * d;
  double I = sp.pi4 * (w * w);
  double cen = I / area;
  double crc = R - cen;
  double pcrc = (crc > 0 ? crc : 0);
  double F = (sp.Kn * pcrc) * area;
  double c_sign = (dist > 0 ? 1.0 : -1.0);
  double r0 = 0, r1 = 0, r2 = 0;  // reaction contributions in dir, t1, t2
  {
    double a = c_sign * F;
    set_comp(f, dir, comp(f, dir) + a);
    r0 -= ((vol * c_sign) * F);
  }
  D3 rel = vel;
  set_comp(rel, dir, comp(rel, dir) - wspeed);
  const int t1 = (dir + 1) % 3, t2 = (dir + 2) % 3;
  if (st.friction) {
    double v1 = comp(rel, t1), v2 = comp(rel, t2);
    double vn = sqrt(v1 * v1 + v2 * v2);
    if (vn > 0) {
      double u1 = v1 / vn, u2 = v2 / vn;
      double aF = fabs(F);
      double ff1 = ((-sp.mu) * aF) * u1;
      double ff2 = ((-sp.mu) * aF) * u2;
      if (vn < ((sp.mu * aF) * sp.dt) / rho) {
        double g = ((-vn) / rho) / sp.dt;
        ff1 = g * u1;
        ff2 = g * u2;
      }
      set_comp(f, t1, comp(f, t1) + ff1);
      set_comp(f, t2, comp(f, t2) + ff2);
      r1 -= (vol * ff1);
      r2 -= (vol * ff2);
    }
  }
  if (st.damping) {
    double dc = ((sp.zeta2) * sqrt(sp.Kn * rho)) * sqrt(fabs(area));
    double df = (-dc) * comp(rel, dir);
    set_comp(f, dir, comp(f, dir) + df);
    r0 -= (vol * df);
  }
  if (reaction) {
    atomicAdd(&st.react[3 * face + dir], r0);
    if (r1 != 0) atomicAdd(&st.react[3 * face + t1], r1);
    if (r2 != 0) atomicAdd(&st.react[3 * face + t2], r2);
  }
}

// Bucket of a broad-phase cell (hashed cell list: cells of every simulation share one table).
__device__ __forceinline__ uint32_t cell_hash(long long cx, long long cy, long long cz, uint32_t sim,
                                              uint32_t mask) {
  unsigned long long h = (unsigned long long)cx * 0x9E3779B97F4A7C15ull;
  h ^= (unsigned long long)cy * 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
  h ^= (unsigned long long)cz * 0x165667B19E3779F9ull + (h << 6) + (h >> 2);
  h ^= (unsigned long long)sim * 0x27D4EB2F165667C5ull;
  h ^= h >> 31;
  h *= 0x7FB5D329728EA185ull;
  h ^= h >> 27;
  return (uint32_t)h & mask;
}

// The contact partners of node n in ascending file-order index (the order in which the
// reference visits them): its candidate list, or, for a node whose list overflowed at the last
// rebuild, the nodes of the same simulation in the 27 cells around its current position that
// lie within the candidate radius now, taken one at a time by selection. Both are supersets of
// the partners within the contact radius (a node moves less than half the skin between
// rebuilds and cells are wider than the candidate radius), and every consumer makes the exact
// distance test, so the two give the same sums; the cell walk costs a scan of the 27 cells per
// partner, which only nodes in unusually dense contact pay.
struct CandWalk {
  const DevView &v;
  uint64_t n;
  const uint32_t *cl;
  int nc, c;
  bool cells;
  long long cx, cy, cz;
  double x, y, z, r2;
  uint32_t sim;
  long long last;  // file index of the partner returned last (-1: none yet)

  __device__ __forceinline__ CandWalk(const DevView &view, uint64_t node) : v(view), n(node), c(0), last(-1) {
    const uint16_t k = v.cand_n[n];
    cells = k == kCandCells;
    nc = cells ? 0 : (int)k;
    cl = v.cand + n * v.cand_cap;
    if (cells) {
      sim = v.parts[v.pid[n]].sim;
      const DevSimParams &sp = v.sp[sim];
      x = v.pos[n] + v.disp[n];
      y = v.pos[n + v.Ncap] + v.disp[n + v.Ncap];
      z = v.pos[n + 2 * v.Ncap] + v.disp[n + 2 * v.Ncap];
      cx = (long long)floor(__dmul_rn(x, sp.inv_cell));  // as node_cell
      cy = (long long)floor(__dmul_rn(y, sp.inv_cell));
      cz = (long long)floor(__dmul_rn(z, sp.inv_cell));
      r2 = sp.cand_r2;
    }
  }

  __device__ __noinline__ bool next_cell(uint32_t &m) {
    uint32_t best = 0, best_m = 0;
    bool found = false;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const uint32_t kk = cell_hash(cx + dx, cy + dy, cz + dz, sim, v.cell_mask);
          const uint32_t b = v.cell_start[kk], e = b + v.cell_count[kk];
          for (uint32_t it = b; it < e; ++it) {
            const uint32_t q = v.cell_sorted[it];
            if (q == n || v.parts[v.pid[q]].sim != sim) continue;
            const uint32_t fq = v.file_of[q];
            if ((long long)fq <= last || (found && fq >= best)) continue;
            const double ddx = (v.pos[q] + v.disp[q]) - x;
            const double ddy = (v.pos[q + v.Ncap] + v.disp[q + v.Ncap]) - y;
            const double ddz = (v.pos[q + 2 * v.Ncap] + v.disp[q + 2 * v.Ncap]) - z;
            if (ddx * ddx + ddy * ddy + ddz * ddz > r2) continue;
            best = fq;
            best_m = q;
            found = true;
          }
        }
    if (!found) return false;
    last = best;
    m = best_m;
    return true;
  }

  __device__ __forceinline__ bool next(uint32_t &m) {
    if (!cells) {
      if (c >= nc) return false;
      m = cl[c++];
      return true;
    }
    return next_cell(m);
  }
};

// Does row n hold a live bond to global node m? (std::find over NbdArr, contact.h:783)
__device__ __forceinline__ bool row_has_live(const DevView &v, uint64_t n, uint32_t m) {
  const uint64_t s = n >> 5;
  const uint32_t lane = (uint32_t)(n & 31);
  const uint64_t base = v.slice_ptr[s] + lane;
  const uint64_t mbase = v.slice_ptr[s] >> 5;
  const int dg = v.deg[n];
  // eight entries requested at once: the row's entries lie 128 bytes apart, one load each, and a
  // load-compare-branch chain would wait on every one of them in turn
  for (int j0 = 0; j0 < dg; j0 += 8) {
    uint32_t c[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k] = (j0 + k < dg) ? v.col[base + 32ull * (j0 + k)] : 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (c[k] == m) return (v.mask[mbase + j0 + k] >> lane) & 1u;
  }
  return false;
}


__device__ __forceinline__ unsigned int fkey(float x) {
  unsigned int u = __float_as_uint(x);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fval(unsigned int k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
__device__ __forceinline__ bool nonfinite(double x) {
  return ((__double2hiint(x) >> 20) & 0x7FF) == 0x7FF;
}

// FP32 form: the band [snot (1 - w), snot (1 + w)] in which a bond's breaking decision is
// re-taken in FP64 (outside it the FP32 stretch decides), wide enough that the FP32 stretch can
// never be on the other side of snot outside it. With eps = 2^-24 and s <= 2 snot near the band:
//  * reference positions are stored as floats relative to the anchor, |component| <= ext_p, so
//    xi is off by at most a = 2 sqrt(3) eps ext_p; displacements likewise, |component| <= u_max,
//    so eta is off by at most b = 2 sqrt(3) eps u_max. The stretch s = |xi + eta| / |xi| - 1
//    moves by at most (|b| + |y^ - (1 + s) xi^| |a|) / |xi| <= (b + (2 + s) a) / xi_min to first
//    order, whatever the rotation of the bond;
//  * the numerator eta.(xi + y) is a dot product of vectors up to (2 + s)|xi| and (4 + s)|xi| long
//    (a rotated bond): its rounding moves s by at most 4 eps (2 + s)(4 + s); the approximate
//    reciprocal square roots and reciprocal (relative error below 2^-22 each) and the remaining
//    roundings add at most 3 * 2^-22 s.
// w is 1.25 times that bound over snot (the band is set from this step's extent and used in the
// next), and at least 1e-4. xi_min is the particle's shortest setup bond: reference positions do
// not change, so no bond gets shorter. The bound is evaluated in FP32 with every operation rounded
// towards +infinity on positive quantities (inputs rounded up, divisors down), so it is an upper
// bound of the formula's exact value; the band's edges are rounded outwards. The same code runs in
// every translation unit (no contraction applies to explicitly rounded operations).
__device__ __forceinline__ void set_break_band(DevPart &P, double u_max) {
  const float eps4 = 4.0f * 5.9604644775390625e-08f, eps12 = 12.0f * 5.9604644775390625e-08f;  // exact
  const float te = 0x1.bb67b0p-23f;  // 2 sqrt(3) * 2^-24, rounded up
  const float snot_u = __double2float_ru(P.snot), snot_d = __double2float_rd(P.snot);
  const float s = __fmul_ru(2.0f, snot_u);
  const float a = __fmul_ru(te, __double2float_ru(P.ext_p)), b = __fmul_ru(te, __double2float_ru(u_max));
  const float s2 = __fadd_ru(2.0f, s), s4 = __fadd_ru(4.0f, s);
  const float lin = __fdiv_ru(__fadd_ru(b, __fmul_ru(s2, a)), __double2float_rd(P.xi_min));
  const float dot = __fmul_ru(__fmul_ru(eps4, s2), s4);
  const float rcp = __fmul_ru(eps12, s);
  const float ds = __fadd_ru(__fadd_ru(lin, dot), rcp);
  float w = __fdiv_ru(__fmul_ru(1.25f, ds), snot_d);
  if (!(w >= 0x1.a36e30p-14f)) w = 0x1.a36e30p-14f;  // at least 1e-4 (also for a particle without bonds)
  P.snot_lo32 = __fmul_rd(snot_d, __fsub_rd(1.0f, w));
  P.snot_hi32 = __fmul_ru(snot_u, __fadd_ru(1.0f, w));
}

// Largest |component| of a particle's anchor-relative displacement, bounded from the box of its
// current anchor-relative positions p + u (|u| <= |p + u| + |p|).
__device__ __forceinline__ double u_extent(const DevPart &P, double box_extent) {
  return box_extent + P.ext_p;
}

// Per-particle inputs of the FP32 form's end of step that depend only on the particle index,
// loaded together before the kernel's branches (the kernel is a short chain of dependent loads).
struct EndPre {
  unsigned int L[6];       // local-frame AABB keys of this step
  double an[3], ann[3];    // anchors of this step and of the next
  double dn[3];            // the anchor node's predicted displacement for the next step
  double apos[3];          // the anchor's reference position
  int32_t movable;
};

__device__ __forceinline__ void end_pre_fp32c(const DevView &v, uint32_t k, uint32_t g0, const DevPart &P,
                                              EndPre &e) {
  const unsigned int *L = v.lrtb_local_next + 6 * (uint64_t)k;
  for (int c = 0; c < 6; ++c) e.L[c] = L[c];
  for (int c = 0; c < 3; ++c) {
    e.an[c] = v.anchor[3 * (uint64_t)k + c];
    e.ann[c] = v.anchor_next[3 * (uint64_t)k + c];
    e.dn[c] = v.disp_next[P.anchor + c * v.Ncap];
    e.apos[c] = P.anchor_pos[c];
  }
  e.movable = P.movable;
}

// End-of-step work of the FP32 form for one particle: AABB from the local-frame keys of this
// step (widened by a few float ulps each way), anchors moved on by one step, the next step's
// wall planes (wall_next) expressed in the frame of the next step's records.
__device__ __forceinline__ void end_particle_fp32c(const DevView &v, uint32_t k, const EndPre &e,
                                                   const double *wall_next) {
  double *an = const_cast<double *>(v.anchor) + 3 * (uint64_t)k;
  double *ann = v.anchor_next + 3 * (uint64_t)k;
  unsigned int *L = v.lrtb_local_next + 6 * (uint64_t)k;
  if (e.movable) {
    double ext = 0.0;
    for (int c = 0; c < 3; ++c) {
      const float lo = fval(e.L[c]), hi = fval(e.L[3 + c]);
      const double base = e.apos[c] + e.an[c];
      const double w = __dadd_rn(__dmul_rn(8.0 * (double)FLT_EPSILON, fmax(fabs((double)lo), fabs((double)hi))), 1e-30);
      v.lrtb[6 * (uint64_t)k + c] = base + (double)lo - w;
      v.lrtb[6 * (uint64_t)k + 3 + c] = base + (double)hi + w;
      ext = fmax(ext, fmax(fabs((double)lo), fabs((double)hi)) + w);
    }
    set_break_band(v.parts[k], u_extent(v.parts[k], ext));
  }
  for (int c = 0; c < 3; ++c) {
    L[c] = fkey(INFINITY);
    L[3 + c] = fkey(-INFINITY);
  }
  // disp_next holds the next step's predicted displacement of the anchor node
  for (int c = 0; c < 3; ++c) {
    an[c] = e.ann[c];
    ann[c] = e.dn[c];
  }
  float *wl = v.wall_local + 6 * (uint64_t)k;
  for (int f = 0; f < 6; ++f) {
    const int c = f % 3;
    wl[f] = (float)(wall_next[f] - (e.apos[c] + e.ann[c]));
  }
}

// ---- bulk copies global -> shared with an mbarrier (cp.async.bulk) --------------------

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// bytes: multiple of 16; both addresses 16-byte aligned
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for phase `parity` of the barrier at most `limit` polls; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit) {
  for (uint32_t it = 0; it < limit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 32) __nanosleep(128);
  }
  return false;
}

}  // namespace pdg
#endif
