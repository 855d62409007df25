// pd_kernels.cu -- the per-step kernels (compiled with -fmad=false).
//
// One step (src/particle/timeloop.h:395-797) is:
//   k_predict        predictor for all nodes (timeloop.h:537-540), step-max displacement
//                    increment for the broad-phase rebuild test, FP32 local displacement
//   [broad phase]    pd_broadphase.cu, runs only when a rebuild is due
//   k_step           FP64 fused per-node force and corrector: PD bond sum with breaking
//                    (particle2.h:107-237), self-contact, walls, extforce, torque
//                    (timeloop.h:544-634), node-node contact of particle pairs in
//                    ascending partner order (timeloop.h:636-651, contact.h:744-942) and
//                    the velocity-Verlet corrector (timeloop.h:661-781)
//   k_end_step       AABB refresh, clamped nodes, anchors, per-particle toggles; its last
//                    block: wall motion (timeloop.h:784-797), scheduled toggles, step counter
// Each node's force is gathered by one thread in the reference's summation order, so the
// FP64 form reproduces the reference bit for bit without atomics on forces.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "pd_device.cuh"
#include "pd_end.cuh"
#include "pd_engine.h"
#include "pd_math.cuh"

namespace pdg {

// ------------------------------------------------------------------------------------
// predictor

__global__ void k_predict(DevView v) {
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float inc2 = 0.f;
  if (n < v.N) {
    const uint32_t k = v.pid[n];
    const DevPart &P = v.parts[k];
    const DevSimParams &sp = v.sp[P.sim];
    if (v.ss[P.sim].active) {
      D3 d = ld3(v.disp, n, v.Ncap), ve = ld3(v.vel_in, n, v.Ncap), a = ld3(v.acc, n, v.Ncap);
      // disp += dt*vel + (dt*dt*0.5)*acc  (timeloop.h:538, overloads.h:129-159)
      D3 dv = sp.dt * ve;
      D3 da = sp.hdt2 * a;
      D3 in = dv + da;
      d = d + in;
      st3(v.disp, n, v.Ncap, d);
      // squared increment in FP32 (only bounds the broad-phase rebuild test)
      const float ix = (float)in.x, iy = (float)in.y, iz = (float)in.z;
      inc2 = ix * ix + iy * iy + iz * iz;
      if (v.rec) {
        const double *an = v.anchor + 3 * (uint64_t)k;
        v.rec[n].u = make_float4((float)(d.x - an[0]), (float)(d.y - an[1]), (float)(d.z - an[2]), 0.f);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) inc2 = fmaxf(inc2, __shfl_xor_sync(0xffffffffu, inc2, o));
  if ((threadIdx.x & 31) == 0 && inc2 > 0.f) {
    const double inc = sqrt((double)inc2) * (1.0 + 1e-5);
    atomicMax(&v.cnt->stepmax_bits, (unsigned long long)__double_as_longlong(inc));
  }
}

void launch_predict(const DevView &v, int tpb, cudaStream_t s) {
  uint64_t blocks = (v.N + tpb - 1) / tpb;
  if (blocks) k_predict<<<(unsigned)blocks, tpb, 0, s>>>(v);
}

// ------------------------------------------------------------------------------------
// fused force + corrector

__global__ void __launch_bounds__(128) k_step(DevView v) {
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = n < v.N;
  const uint64_t nn = valid ? n : 0;
  const uint32_t k = v.pid[nn];
  const DevPart P = v.parts[k];
  const DevSimParams &sp = v.sp[P.sim];
  DevSimState &st = v.ss[P.sim];
  const bool run = valid && st.active;
  const uint64_t C3 = v.Ncap;

  D3 f = d3(0.0, 0.0, 0.0);
  D3 di = ld3(v.disp, nn, C3);
  const D3 pi = ld3(v.pos, nn, C3);
  const D3 vi = ld3(v.vel_in, nn, C3);
  const double voli = v.vol[nn];
  const bool bdry_i = v.bdry[nn] != 0;
  unsigned long long live = 0, ncontacts = 0;

  if (run && P.movable) {
    // ---- peridynamic bond force (particle2.h:117-157) and breaking (particle2.h:196-237)
    const uint64_t s = nn >> 5;
    const uint32_t lane = (uint32_t)(nn & 31);
    const uint64_t base = v.slice_ptr[s] + lane;
    const uint64_t mbase = v.slice_ptr[s] >> 5;
    const int dg = v.deg[nn];
    const bool brk = st.fracture && P.breakable && P.break_bonds;
    D3 acc = d3(0.0, 0.0, 0.0);
    for (int j = 0; j < dg; ++j) {
      const uint32_t mw = v.mask[mbase + j];
      if (!((mw >> lane) & 1u)) continue;
      const uint64_t e = base + 32ull * j;
      const uint32_t q = v.col[e];
      ++live;
      D3 dq = ld3(v.disp, q, C3);
      D3 eta = (dq - di) + d3(v.bxi[e], v.bxi[e + v.E], v.bxi[e + 2 * v.E]);
      double en = norm3(eta);
      double xn = v.bxin[e];
      double str = div_rcp(en - xn, xn, v.brxin[e]);
      double mag = (P.cnot * str) * v.vol[q];
      double ren = __drcp_rn(en);
      D3 unit = d3(div_rcp(eta.x, en, ren), div_rcp(eta.y, en, ren), div_rcp(eta.z, en, ren));
      acc = acc + mag * unit;
      if (brk && str > P.snot) atomicAnd(&v.mask[mbase + j], ~(1u << lane));
    }
    f = d3(0.0, 0.0, 0.0) + acc;

    // ---- self-contact (timeloop.h:554-557, contact.h:779-796), C side only
    if (st.fracture && P.breakable && st.self_contact && (!sp.nl_bdry_only || bdry_i)) {
      CandWalk walk(v, nn);
      uint32_t m;
      while (walk.next(m)) {
        if (m < P.g0) continue;
        if (m >= P.g0 + P.n) break;
        if (sp.nl_bdry_only && !v.bdry[m]) continue;
        D3 xi = ld3(v.pos, m, C3) - pi;
        D3 dir = (ld3(v.disp, m, C3) - di) + xi;
        const double q = sq3(dir);
        if (q >= sp.rc2_far) continue;  // outside Rc for certain: skip the square root
        double dn = sqrt(q);
        if (!(dn <= sp.Rc)) continue;
        double xin = norm3(xi);
        double len_ref = sp.Rc, sc = sp.sc;
        if (row_has_live(v, nn, m)) continue;
        if (xin < sp.Rc) {
          len_ref = xin;
          sc = P.cnot;
        }
        if (!(dn < len_ref)) continue;
        PairForce pf;
        pair_force(dir, dn, len_ref, sc, v.vol[m], P.rho, vi, ld3(v.vel_in, m, C3), sp, st, pf);
        if (P.stoppable) {
          f = f + pf.fc;
          if (pf.has_fd) f = f + pf.fd;
          if (pf.has_ff) f = f + pf.ff;
        }
      }
    }

    // ---- walls (timeloop.h:561-569, contact.h:1094-1121)
    if (P.stoppable && sp.allow_wall && !within_interior(v.lrtb + 6 * (uint64_t)k, st.wall, sp.Rc) &&
        (!sp.nl_bdry_only || bdry_i)) {
      D3 cur = pi + di;
      const bool rx = sp.compute_wall_reaction != 0;
      wall_face(cur.x - st.wall[0], 0, vi, voli, P.rho, f, st.spd[0], 0, sp, st, rx);
      wall_face(cur.x - st.wall[3], 0, vi, voli, P.rho, f, st.spd[3], 3, sp, st, rx);
      wall_face(cur.y - st.wall[1], 1, vi, voli, P.rho, f, st.spd[1], 1, sp, st, rx);
      wall_face(cur.y - st.wall[4], 1, vi, voli, P.rho, f, st.spd[4], 4, sp, st, rx);
      wall_face(cur.z - st.wall[2], 2, vi, voli, P.rho, f, st.spd[2], 2, sp, st, rx);
      wall_face(cur.z - st.wall[5], 2, vi, voli, P.rho, f, st.spd[5], 5, sp, st, rx);
    }

    // ---- external force (timeloop.h:582-597)
    D3 ex = ld3(v.ext, nn, C3);
    if (sp.gradient_extforce) ex = st.extf_scale * ex;
    f = f + ex;
  }

  // ---- torque about the centroid (timeloop.h:600-633), for movable and fixed particles
  if (run && st.torque) {
    const double *c = v.centroid + 3 * (uint64_t)k;
    D3 r = (pi + di) - d3(c[0], c[1], c[2]);
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

  // ---- node-node contact of particle pairs (timeloop.h:636-651, contact.h:754-937):
  // partners in ascending file-order global index; a partner in a lower particle index acts as
  // the "C" node of the pair (reaction form), a partner in a higher index as the "N" node.
  if (run && P.stoppable && (!sp.nl_bdry_only || bdry_i)) {
    CandWalk walk(v, nn);
    uint32_t m;
    while (walk.next(m)) {
      if (m >= P.g0 && m < P.g0 + P.n) continue;
      const uint32_t km = v.pid[m];
      const uint32_t a = km < k ? km : k, b = km < k ? k : km;
      if (!(v.parts[a].movable || v.parts[b].movable)) continue;
      if (!intersects_fext(v.lrtb + 6 * (uint64_t)a, v.lrtb + 6 * (uint64_t)b, sp.Rc)) continue;
      if (sp.nl_bdry_only && !v.bdry[m]) continue;
      const D3 pm = ld3(v.pos, m, C3), dm = ld3(v.disp, m, C3), vm = ld3(v.vel_in, m, C3);
      const double volm = v.vol[m];
      if (km > k) {
        D3 xi = pm - pi;
        D3 dir = (dm - di) + xi;
        const double q = sq3(dir);
        if (q >= sp.rc2_far) continue;
        double dn = sqrt(q);
        if (!(dn <= sp.Rc) || !(dn < sp.Rc)) continue;
        PairForce pf;
        pair_force(dir, dn, sp.Rc, sp.sc, volm, P.rho, vi, vm, sp, st, pf);
        f = f + pf.fc;
        if (pf.has_fd) f = f + pf.fd;
        if (pf.has_ff) f = f + pf.ff;
        ++ncontacts;
      } else {
        D3 xi = pi - pm;
        D3 dir = (di - dm) + xi;
        const double q = sq3(dir);
        if (q >= sp.rc2_far) continue;
        double dn = sqrt(q);
        if (!(dn <= sp.Rc) || !(dn < sp.Rc)) continue;
        PairForce pf;
        pair_force(dir, dn, sp.Rc, sp.sc, voli, v.parts[km].rho, vm, vi, sp, st, pf);
        f = f - (pf.fc / voli) * volm;
        if (pf.has_fd) {
          double sn = sqrt(voli), sv = sqrt(volm);
          f = f - (pf.fd / sn) * sv;
        }
        if (pf.has_ff) f = f - pf.ff;
      }
    }
  }

  // ---- corrector (timeloop.h:662-781)
  if (run) {
    st3(v.force, nn, C3, f);
    if (!(isfinite(f.x) && isfinite(f.y) && isfinite(f.z))) atomicOr(&v.cnt->err, PD_DERR_NONFINITE);
    D3 vo = vi;
    if (P.movable) {
      const D3 ao = ld3(v.acc, nn, C3);
      if (v.afd && st.vconstraint && (int32_t)(k - sp.p0) == sp.pv_particle) st3(v.afd, nn, C3, ao);
      const D3 an = P.irho * f;
      D3 tmp = ao + an;
      tmp = sp.hdt * tmp;
      vo = vi + tmp;
      st3(v.acc, nn, C3, an);
    }
    st3(v.vel_out, nn, C3, vo);
  }

  // ---- AABB of CurrPos for the next step (timeloop.h:779), warp-reduced
  {
    const bool contrib = run && P.movable;
    D3 cur = pi + di;
    double lo[3] = {contrib ? cur.x : INFINITY, contrib ? cur.y : INFINITY, contrib ? cur.z : INFINITY};
    double hi[3] = {contrib ? cur.x : -INFINITY, contrib ? cur.y : -INFINITY, contrib ? cur.z : -INFINITY};
    const uint32_t k0 = __shfl_sync(0xffffffffu, k, 0);
    const bool uniform = __all_sync(0xffffffffu, k == k0);
    if (uniform) {
      for (int o = 16; o > 0; o >>= 1) {
        for (int c = 0; c < 3; ++c) {
          lo[c] = fmin(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
          hi[c] = fmax(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
        }
      }
    }
    const bool writer = uniform ? ((threadIdx.x & 31) == 0) : contrib;
    if (writer && lo[0] <= hi[0]) {
      unsigned long long *L = reinterpret_cast<unsigned long long *>(v.lrtb_next) + 6 * (uint64_t)k;
      for (int c = 0; c < 3; ++c) {
        atomicMin(&L[c], ord_key(lo[c]));
        atomicMax(&L[3 + c], ord_key(hi[c]));
      }
    }
  }

  if (v.stats) {
    for (int o = 16; o > 0; o >>= 1) {
      live += __shfl_xor_sync(0xffffffffu, live, o);
      ncontacts += __shfl_xor_sync(0xffffffffu, ncontacts, o);
    }
    if ((threadIdx.x & 31) == 0) {
      if (live) atomicAdd(&v.cnt->live_bonds, live);
      if (ncontacts) atomicAdd(&v.cnt->contacts, ncontacts);
    }
  }
}

void launch_step_kernel(const DevView &v, int precision, int variant, cudaStream_t s) {
  uint64_t blocks = (v.N + 127) / 128;
  if (!blocks) return;
  if (precision == PD_FP32C)
    launch_step_fp32c(v, variant, s);
  else
    k_step<<<(unsigned)blocks, 128, 0, s>>>(v);
}

// ------------------------------------------------------------------------------------
// end of step

// Per-particle end of step, then (last block) the simulations' advance (pd_end.cuh). One kernel:
// the particles read their simulation's state of this step and derive the next step's wall
// planes and step index themselves, with the same arithmetic as the advance, which the last block
// to finish applies once every other block is done reading.
__global__ void k_end_step(DevView v, const uint32_t *clamped_ptr, const uint32_t *clamped, double *clamped_disp) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < v.P) end_step_particle(v, k, clamped_ptr, clamped, clamped_disp);
  // the last block to finish advances the simulations and the step counters
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&v.cnt->end_blocks, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  end_step_advance(v, threadIdx.x, blockDim.x);
}

// The FP32 form's end of step with one warp per particle (end_particle_warp), the last block
// advancing the simulations as in k_end_step.
__global__ void __launch_bounds__(128) k_end_step_w(DevView v) {
  const uint64_t k = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (k < v.P) end_particle_warp(v, (uint32_t)k, threadIdx.x & 31);
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(&v.cnt->end_blocks, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  end_step_advance(v, threadIdx.x, blockDim.x);
}

void launch_end_step(const DevView &v, const uint32_t *clamped, uint64_t n_clamped, double *clamped_disp,
                     cudaStream_t s) {
  if (v.rec && v.fused) {  // FP32 form (its clamped nodes are handled by the corrector)
    k_end_step_w<<<(v.P + 3) / 4, 128, 0, s>>>(v);
    return;
  }
  const uint32_t *cptr = n_clamped ? clamped : nullptr;
  const uint32_t *clist = n_clamped ? clamped + (v.P + 1) : nullptr;
  k_end_step<<<(v.P + 127) / 128, 128, 0, s>>>(v, cptr, clist, clamped_disp);
}

// ------------------------------------------------------------------------------------
// auxiliary kernels

// mean_CurrPos per particle (particle2.h:94-103): a sequential sum in file node order.
__global__ void k_centroids(DevView v) {
  const uint32_t k = blockIdx.x;
  const int c = threadIdx.x;
  if (k >= v.P || c >= 3) return;
  const DevPart &P = v.parts[k];
  if (!v.ss[P.sim].torque) return;
  double m = 0.0;
  const double *pp = v.pos + c * v.Ncap, *dd = v.disp + c * v.Ncap;
  for (uint32_t i = 0; i < P.n; ++i) {
    const uint32_t g = v.node_of[P.g0 + i];
    m = m + (pp[g] + dd[g]);
  }
  const_cast<double *>(v.centroid)[3 * (uint64_t)k + c] = m / (double)P.n;
}

void launch_centroids(const DevView &v, cudaStream_t s) {
  if (v.P) k_centroids<<<v.P, 32, 0, s>>>(v);
}

// Prescribed velocity of one particle per simulation, after the corrector (timeloop.h:684-764):
// the particle's velocity is split into its mean and the rest; the mean's x component
// (fix_velocity_mean_x) and the rest (fix_velocity_angular: rotation about z at the
// prescribed rate, about mean_CurrPos) are replaced. applied_force_density =
// rho*((2/dt)*(pv - vel) - acc_old) - force, with vel already equal to pv (as in the
// reference). The means are sequential sums in file node order, like Eigen's += loop.
__global__ void k_prescribed(DevView v) {
  const uint32_t s = blockIdx.x;
  if (s >= v.S) return;
  const DevSimParams &sp = v.sp[s];
  const DevSimState &st = v.ss[s];
  if (!st.active || !st.vconstraint || sp.pv_particle < 0) return;
  const uint32_t k = sp.p0 + (uint32_t)sp.pv_particle;
  const DevPart &P = v.parts[k];
  if (!P.movable) return;
  const uint64_t C3 = v.Ncap;
  __shared__ double sh[6];
  if (threadIdx.x == 0) {
    D3 mv = d3(0.0, 0.0, 0.0), mp = d3(0.0, 0.0, 0.0);
    for (uint32_t i = 0; i < P.n; ++i) mv = mv + ld3(v.vel_out, v.node_of[P.g0 + i], C3);
    const double nn = (double)P.n;
    mv = d3(mv.x / nn, mv.y / nn, mv.z / nn);
    if (sp.fix_angular) {  // mean_CurrPos (particle2.h:94-103)
      for (uint32_t i = 0; i < P.n; ++i) {
        const uint32_t g = v.node_of[P.g0 + i];
        mp = mp + (ld3(v.pos, g, C3) + ld3(v.disp, g, C3));
      }
      mp = d3(mp.x / nn, mp.y / nn, mp.z / nn);
    }
    sh[0] = mv.x;
    sh[1] = mv.y;
    sh[2] = mv.z;
    sh[3] = mp.x;
    sh[4] = mp.y;
    sh[5] = mp.z;
  }
  __syncthreads();
  const double two_dt = 2 / sp.dt;
  float i2 = 0.f;
  for (uint32_t i = threadIdx.x; i < P.n; i += blockDim.x) {
    const uint64_t g = P.g0 + i;
    const D3 vel = ld3(v.vel_out, g, C3);
    D3 mean = d3(sh[0], sh[1], sh[2]);
    D3 vrot = vel - mean;
    if (sp.fix_mean_x) mean.x = sp.pv_mean_x;
    if (sp.fix_angular) {
      const D3 rv = (ld3(v.pos, g, C3) + ld3(v.disp, g, C3)) - d3(sh[3], sh[4], sh[5]);
      const double r = norm3(rv);
      D3 ru = d3(0.0, 0.0, 0.0);
      if (r > 0) ru = d3(rv.x / r, rv.y / r, rv.z / r);
      const double rw = r * sp.pv_angular;
      vrot = d3(-rw * ru.y, rw * ru.x, 0.0);
    }
    const D3 pv = vrot + mean;
    const bool clamped32 = v.fused && v.clamp_flag[g];  // FP32 form: clamped nodes already at rest
    if (!clamped32) st3(v.vel_out, g, C3, pv);
    const D3 dd = pv - pv;
    const D3 a = (two_dt * dd) - ld3(v.afd, g, C3);
    st3(v.afd, g, C3, (P.rho * a) - ld3(v.force, g, C3));
    if (v.fused && !clamped32) {
      // the fused predictor of the FP32 form ran with the velocity before the overwrite
      const D3 d = ld3(v.disp, g, C3);
      const D3 an = ld3(v.acc, g, C3);
      const D3 inc = sp.dt * pv + sp.hdt2 * an;
      const D3 dn = d + inc;
      st3(v.disp_next, g, C3, dn);
      const double *anx = v.anchor_next + 3 * (uint64_t)k;
      v.rec_next[g].u = make_float4((float)(dn.x - anx[0]), (float)(dn.y - anx[1]), (float)(dn.z - anx[2]), 0.f);
      const float ix = (float)(dn.x - d.x), iy = (float)(dn.y - d.y), iz = (float)(dn.z - d.z);
      i2 = fmaxf(i2, ix * ix + iy * iy + iz * iz);
    }
  }
  for (int o = 16; o > 0; o >>= 1) i2 = fmaxf(i2, __shfl_xor_sync(0xffffffffu, i2, o));
  if ((threadIdx.x & 31) == 0 && i2 > 0.f) {
    const double inc = sqrt((double)i2) * (1.0 + 1e-5);
    atomicMax(&v.cnt->stepmax_bits, (unsigned long long)__double_as_longlong(inc));
  }
}

void launch_prescribed(const DevView &v, cudaStream_t s) {
  if (v.S && v.afd) k_prescribed<<<v.S, 256, 0, s>>>(v);
}

// reset_partzero_y at the top of step t (timeloop.h:500-535): particle 0 is lifted so that its
// mean y sits wheel_rad + contact radius above the highest node of the other particles within
// wheel_rad (in x) of its mean x. The displacement read here is the one after the previous
// corrector (clamped nodes at zero).
__device__ __forceinline__ D3 disp_after_corrector(const DevView &v, uint64_t g, uint32_t t) {
  if (v.fused) {  // FP32 form: the previous step's buffer keeps clamped nodes' prediction
    if (t > 1 && v.clamp_flag[g]) return d3(0.0, 0.0, 0.0);
    return ld3(v.disp_next, g, v.Ncap);
  }
  return ld3(v.disp, g, v.Ncap);
}

__global__ void k_reset_y(DevView v) {
  const uint32_t s = blockIdx.x;
  if (s >= v.S) return;
  const DevSimParams &sp = v.sp[s];
  const DevSimState &st = v.ss[s];
  if (!st.active || !sp.reset_y || st.t != sp.reset_y_ts) return;
  const uint64_t C3 = v.Ncap;
  const DevPart &P0 = v.parts[sp.p0];
  const DevPart &P1 = v.parts[sp.p0 + 1];
  __shared__ double m0[3];
  __shared__ unsigned long long best;
  __shared__ int found;
  __shared__ double move;
  if (threadIdx.x == 0) {
    D3 m = d3(0.0, 0.0, 0.0);
    for (uint32_t i = 0; i < P0.n; ++i) {  // file node order
      const uint32_t g = v.node_of[P0.g0 + i];
      m = m + (ld3(v.pos, g, C3) + disp_after_corrector(v, g, st.t));
    }
    const double nn = (double)P0.n;
    m0[0] = m.x / nn;
    m0[1] = m.y / nn;
    m0[2] = m.z / nn;
    best = ord_key(-INFINITY);
    found = 0;
  }
  __syncthreads();
  // highest y among the other particles' nodes near particle 0's mean x (an exact max)
  const uint64_t a = P1.g0, b = sp.node0 + sp.nnodes;
  double my = -INFINITY;
  int any = 0;
  for (uint64_t g = a + threadIdx.x; g < b; g += blockDim.x) {
    const D3 now = ld3(v.pos, g, C3) + disp_after_corrector(v, g, st.t);
    if (fabs(m0[0] - now.x) <= sp.wheel_rad) {
      any = 1;
      my = fmax(my, now.y);
    }
  }
  if (any) {
    atomicMax(&best, ord_key(my));
    found = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double max_bulk_y;
    if (found) {
      max_bulk_y = ord_val(best);
    } else {  // the reference's initial value: pos[0] of particle 1 plus disp[1] (file order)
      const uint64_t j = P1.n > 1 ? 1 : 0;
      max_bulk_y = v.pos[v.node_of[P1.g0] + C3] + disp_after_corrector(v, v.node_of[P1.g0 + j], st.t).y;
    }
    const double dest = (max_bulk_y + sp.wheel_rad) + sp.Rc;
    move = dest - m0[1];
    v.cnt->xall = 1;       // particle 0 moved: the non-bond work lists are stale for this step
    v.cnt->moved = 1e300;  // and so are the contact candidate lists: this step rebuilds them
    if (v.fused) {  // the FP32 form keeps positions relative to the particle's anchor
      DevPart &Pw = v.parts[sp.p0];
      Pw.anchor_pos[1] = Pw.anchor_pos[1] + move;
      float *wl = v.wall_local + 6 * (uint64_t)sp.p0;
      const double *an = v.anchor + 3 * (uint64_t)sp.p0;
      for (int f = 0; f < 6; ++f) {
        const int c = f % 3;
        wl[f] = (float)(st.wall[f] - (Pw.anchor_pos[c] + an[c]));
      }
    }
  }
  __syncthreads();
  double *py = const_cast<double *>(v.pos) + C3;
  for (uint32_t i = threadIdx.x; i < P0.n; i += blockDim.x) py[P0.g0 + i] = py[P0.g0 + i] + move;
}

void launch_reset_y(const DevView &v, cudaStream_t s) {
  if (v.S) k_reset_y<<<v.S, 256, 0, s>>>(v);
}

// gen_xi (particle2.h:241-257): xi = pos[q] - pos[i], |xi| and RN(1/|xi|) per SELL entry.
__global__ void k_bond_constants(DevView v, double *bxi, double *bxin, double *brxin) {
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= v.N) return;
  const uint64_t s = n >> 5;
  const uint32_t lane = (uint32_t)(n & 31);
  const uint64_t base = v.slice_ptr[s] + lane;
  const D3 pi = ld3(v.pos, n, v.Ncap);
  const int dg = v.deg[n];
  for (int j = 0; j < dg; ++j) {
    const uint64_t e = base + 32ull * j;
    const uint32_t q = v.col[e];
    D3 xi = ld3(v.pos, q, v.Ncap) - pi;
    double xn = norm3(xi);
    bxi[e] = xi.x;
    bxi[e + v.E] = xi.y;
    bxi[e + 2 * v.E] = xi.z;
    bxin[e] = xn;
    brxin[e] = __drcp_rn(xn);
  }
}

void launch_bond_constants(const DevView &v, double *bxi, double *bxin, double *brxin, cudaStream_t s) {
  uint64_t blocks = (v.N + 127) / 128;
  if (blocks) k_bond_constants<<<(unsigned)blocks, 128, 0, s>>>(v, bxi, bxin, brxin);
}

// AABBs of all particles before the loop (timeloop.h:389-393). A warp whose nodes all belong to
// one particle reduces its keys with shuffles first (min/max are exact, so the result does not
// depend on how they are combined), which keeps the atomics on a particle's six keys few.
__global__ void k_init_lrtb_acc(DevView v) {
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = n < v.N;
  const uint32_t k = valid ? v.pid[n] : 0xFFFFFFFFu;
  unsigned long long lo[3], hi[3];
  if (valid) {
    const D3 cur = ld3(v.pos, n, v.Ncap) + ld3(v.disp, n, v.Ncap);
    lo[0] = hi[0] = ord_key(cur.x);
    lo[1] = hi[1] = ord_key(cur.y);
    lo[2] = hi[2] = ord_key(cur.z);
  } else {
    for (int c = 0; c < 3; ++c) {
      lo[c] = ord_key(INFINITY);
      hi[c] = ord_key(-INFINITY);
    }
  }
  const uint32_t k0 = __shfl_sync(0xffffffffu, k, 0);
  if (__all_sync(0xffffffffu, !valid || k == k0)) {  // lanes past N carry the identity keys
    if (k0 == 0xFFFFFFFFu) return;
    for (int o = 16; o > 0; o >>= 1)
      for (int c = 0; c < 3; ++c) {
        lo[c] = min(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
        hi[c] = max(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
      }
    if ((threadIdx.x & 31) != 0) return;
  } else if (!valid) {
    return;
  }
  const uint64_t kp = valid ? k : k0;
  unsigned long long *L = reinterpret_cast<unsigned long long *>(v.lrtb_next) + 6 * kp;
  for (int c = 0; c < 3; ++c) {
    atomicMin(&L[c], lo[c]);
    atomicMax(&L[3 + c], hi[c]);
  }
}
__global__ void k_init_lrtb_fin(DevView v) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= v.P) return;
  unsigned long long *L = reinterpret_cast<unsigned long long *>(v.lrtb_next) + 6 * (uint64_t)k;
  for (int c = 0; c < 6; ++c) v.lrtb[6 * (uint64_t)k + c] = ord_val(L[c]);
  for (int c = 0; c < 3; ++c) {
    L[c] = ord_key(INFINITY);
    L[3 + c] = ord_key(-INFINITY);
  }
  if (v.rec) {
    const DevPart &P = v.parts[k];
    const DevSimState &st = v.ss[P.sim];
    double *an = const_cast<double *>(v.anchor) + 3 * (uint64_t)k;
    an[0] = v.disp[P.anchor];
    an[1] = v.disp[P.anchor + v.Ncap];
    an[2] = v.disp[P.anchor + 2 * v.Ncap];
    // the breaking band from the anchor-relative extent of the current positions
    double ext = 0.0;
    for (int c = 0; c < 3; ++c) {
      const double A = P.anchor_pos[c] + an[c];
      ext = fmax(ext, fmax(fabs(v.lrtb[6 * (uint64_t)k + c] - A), fabs(v.lrtb[6 * (uint64_t)k + 3 + c] - A)));
    }
    set_break_band(v.parts[k], u_extent(P, ext * (1.0 + 1e-6)));
    unsigned int *Lf = v.lrtb_local_next + 6 * (uint64_t)k;
    float *wl = v.wall_local + 6 * (uint64_t)k;
    for (int c = 0; c < 3; ++c) {
      Lf[c] = fkey(INFINITY);
      Lf[3 + c] = fkey(-INFINITY);
    }
    for (int f = 0; f < 6; ++f) wl[f] = (float)(st.wall[f] - (P.anchor_pos[f % 3] + an[f % 3]));
  }
}
__global__ void k_reset_lrtb_next(DevView v) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= v.P) return;
  unsigned long long *L = reinterpret_cast<unsigned long long *>(v.lrtb_next) + 6 * (uint64_t)k;
  for (int c = 0; c < 3; ++c) {
    L[c] = ord_key(INFINITY);
    L[3 + c] = ord_key(-INFINITY);
  }
}

void launch_init_lrtb(const DevView &v, cudaStream_t s) {
  if (!v.P) return;
  k_reset_lrtb_next<<<(v.P + 127) / 128, 128, 0, s>>>(v);
  uint64_t blocks = (v.N + 127) / 128;
  if (blocks) k_init_lrtb_acc<<<(unsigned)blocks, 128, 0, s>>>(v);
  k_init_lrtb_fin<<<(v.P + 127) / 128, 128, 0, s>>>(v);
}

// Readback in file order: a [3][Ncap] engine-order array (plus `add` of the same layout,
// added as add + src, when given) -> N*3 rows in file order.
__global__ void k_rows_to_file(const double *src, const double *add, uint64_t Ncap, uint64_t N,
                               const uint32_t *file_of, double *dst) {
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const uint64_t f = file_of[n];
  for (int c = 0; c < 3; ++c) {
    const double x = src[c * Ncap + n];
    dst[3 * f + c] = add ? add[c * Ncap + n] + x : x;
  }
}

// The rows of the clamped nodes: zero (FP32 form's displacement after a step), or pos + the
// predicted displacement kept for them (FP64 form's CurrPos, timeloop.h:767-774).
__global__ void k_clamped_rows(const uint32_t *clamped, uint64_t n_clamped, const uint32_t *file_of,
                               const double *pos, const double *cdisp, uint64_t Ncap, double *dst) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_clamped) return;
  const uint64_t g = clamped[i], f = file_of[g];
  for (int c = 0; c < 3; ++c) dst[3 * f + c] = cdisp ? pos[c * Ncap + g] + cdisp[3 * i + c] : 0.0;
}

void launch_rows_to_file(const double *src, const double *add, uint64_t Ncap, uint64_t N, const uint32_t *file_of,
                         double *dst, cudaStream_t s) {
  if (N) k_rows_to_file<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(src, add, Ncap, N, file_of, dst);
}

void launch_clamped_rows(const uint32_t *clamped, uint64_t n_clamped, const uint32_t *file_of, const double *pos,
                         const double *cdisp, uint64_t Ncap, double *dst, cudaStream_t s) {
  if (n_clamped)
    k_clamped_rows<<<(unsigned)((n_clamped + 127) / 128), 128, 0, s>>>(clamped, n_clamped, file_of, pos, cdisp,
                                                                       Ncap, dst);
}

// Number of particle pairs the pair loop evaluates (timeloop.h:641-649), for the
// progress line's "#contacts" column.
__global__ void k_pairwise(DevView v) {
  const uint32_t s = blockIdx.y;
  if (s >= v.S) return;
  const DevSimParams &sp = v.sp[s];
  if (!v.ss[s].active) return;
  const uint64_t np = sp.np;
  const uint64_t total = np * (np - 1) / 2;
  unsigned long long cnt = 0;
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (uint64_t)gridDim.x * blockDim.x) {
    // invert idx -> (i, j), i < j, lexicographic
    uint64_t i = (uint64_t)((2.0 * np - 1 - sqrt((2.0 * np - 1) * (2.0 * np - 1) - 8.0 * idx)) / 2);
    while (i > 0 && i * (2 * np - i - 1) / 2 > idx) --i;
    while ((i + 1) * (2 * np - i - 2) / 2 <= idx) ++i;
    uint64_t j = idx - i * (2 * np - i - 1) / 2 + i + 1;
    const uint32_t a = sp.p0 + (uint32_t)i, b = sp.p0 + (uint32_t)j;
    if (!(v.parts[a].movable || v.parts[b].movable)) continue;
    if (intersects_fext(v.lrtb + 6 * (uint64_t)a, v.lrtb + 6 * (uint64_t)b, sp.Rc)) ++cnt;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&v.cnt->pairwise, cnt);
}

void launch_pairwise_count(const DevView &v, cudaStream_t s) {
  if (!v.S) return;
  dim3 grid(64, v.S);
  k_pairwise<<<grid, 256, 0, s>>>(v);
}

}  // namespace pdg

namespace pdg {

// Live directed bonds of movable particles: popcount of each node's live bits.
__global__ void k_count_live(DevView v, unsigned long long *out) {
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long c = 0;
  if (n < v.N && v.parts[v.pid[n]].movable) {
    const uint64_t s = n >> 5;
    const uint32_t lane = (uint32_t)(n & 31);
    const uint64_t mbase = v.slice_ptr[s] >> 5;
    const int dg = v.deg[n];
    for (int j = 0; j < dg; ++j) c += (v.mask[mbase + j] >> lane) & 1u;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

void launch_count_live(const DevView &v, unsigned long long *out, cudaStream_t s) {
  uint64_t blocks = (v.N + 255) / 256;
  if (blocks) k_count_live<<<(unsigned)blocks, 256, 0, s>>>(v, out);
}

// Bonds of each node as a saved Connectivity counts them: NbdArr2conn (timeloop.h:20-44)
// keeps the live pair (i, q) for i < q only, and total_neighbors (plot3d_timestep.py:95-105)
// counts each kept pair at both ends. So row n adds every live partner above it in file
// order to both n and that partner. Nodes [n0, n0 + nn) are whole particles (the same range
// in engine and file order); now[] is indexed by file order - n0 and starts at zero.
__global__ void k_damage_count(DevView v, uint64_t n0, uint64_t nn, uint32_t *now) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nn) return;
  const uint64_t n = n0 + k;
  const uint64_t e0 = v.slice_ptr[n >> 5];
  const uint32_t lane = (uint32_t)(n & 31);
  const uint32_t fn = v.file_of[n];
  const int dg = v.deg[n];
  uint32_t own = 0;
  for (int j = 0; j < dg; ++j) {
    if (!((v.mask[(e0 >> 5) + j] >> lane) & 1u)) continue;
    const uint32_t fq = v.file_of[v.col[e0 + 32 * (uint64_t)j + lane] & kColIndex];
    if (fq > fn) {
      ++own;
      atomicAdd(&now[fq - n0], 1u);
    }
  }
  if (own) atomicAdd(&now[fn - n0], own);
}

// damage = (orig - now) / orig per node (plot3d_timestep.py:156-166), orig being the node's
// bond count in the setup's Connectivity (its row length); 0/0 gives NaN as it does there.
__global__ void k_damage_out(DevView v, uint64_t n0, uint64_t nn, const uint32_t *now, double *out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nn) return;
  const uint64_t n = n0 + k;
  const uint64_t f = v.file_of[n] - n0;
  const double orig = (double)v.deg[n];
  out[f] = (orig - (double)now[f]) / orig;
}

void launch_damage(const DevView &v, uint64_t n0, uint64_t nn, uint32_t *now, double *out, cudaStream_t s) {
  const uint64_t blocks = (nn + 255) / 256;
  if (!blocks) return;
  k_damage_count<<<(unsigned)blocks, 256, 0, s>>>(v, n0, nn, now);
  k_damage_out<<<(unsigned)blocks, 256, 0, s>>>(v, n0, nn, now, out);
}

}  // namespace pdg
