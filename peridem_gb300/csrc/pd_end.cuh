// pd_end.cuh -- the end of a step: each particle's end-of-step work and the simulations'
// advance (walls, step index, sticky toggles, broad-phase movement bookkeeping). Called by
// k_end_step (pd_kernels.cu) and by the persistent step (pd_fp32c.cu). Products and sums are
// written with explicit round-to-nearest intrinsics so that the arithmetic is the same in every
// translation unit, whatever its contraction setting: one rounding per multiply and per add, as
// in the reference's compiled CPU code.
#ifndef PD_END_CUH
#define PD_END_CUH

#include <cuda_runtime.h>
#include <math.h>

#include "pd_device.cuh"
#include "pd_engine.h"
#include "pd_math.cuh"

namespace pdg {

// Flags a simulation uses in step t (the sticky toggles of timeloop.h:405-464).
__device__ __forceinline__ void apply_sim_toggles(const DevSimParams &sp, DevSimState &st, uint32_t t) {
  if (sp.set_torque_ts != -1 && t == (uint32_t)sp.set_torque_ts) st.torque = 1;
  if (sp.set_fracture_ts != -1 && t == (uint32_t)sp.set_fracture_ts) st.fracture = 1;
  if (sp.set_self_contact_ts != -1 && t == (uint32_t)sp.set_self_contact_ts) st.self_contact = 1;
  if (sp.set_damping_ts != -1 && t == (uint32_t)sp.set_damping_ts) st.damping = 1;
  if (sp.set_zero_wall_speed_ts != -1 && t == (uint32_t)sp.set_zero_wall_speed_ts)
    for (int c = 0; c < 6; ++c) st.spd[c] = 0;
  if (sp.set_fix_velocity_ts != -1 && t == (uint32_t)sp.set_fix_velocity_ts) st.vconstraint = 1;
  if (sp.gradient_extforce) {
    double sc = (double)t / (double)sp.extforce_maxstep;
    if (sc > 1) sc = 1;
    st.extf_scale = sc;
  }
}

// One particle's end of step: its AABB (and in the FP32 form its anchors, local wall planes and
// breaking band), the FP64 form's clamped nodes, its toggles for the next step, and the FP32
// form's list of particles with FP64 non-bond work next step. It reads its simulation's state of
// this step and derives the next step's wall planes and step index with the same arithmetic as
// end_step_advance, which runs once every particle is done.
__device__ __forceinline__ void end_step_particle(const DevView &v, uint32_t k, const uint32_t *clamped_ptr,
                                                  const uint32_t *clamped, double *clamped_disp) {
  DevPart &P = v.parts[k];
  const uint32_t sim = P.sim;
  EndPre pre;
  if (v.rec) end_pre_fp32c(v, k, P.anchor, P, pre);
  const double move = __longlong_as_double((long long)v.cnt->stepmax_bits);  // this step's bound
  const DevSimState &st = v.ss[sim];
  const DevSimParams &sp = v.sp[sim];
  if (st.active) {
    double wall_next[6];
    for (int c = 0; c < 6; ++c) wall_next[c] = __dadd_rn(st.wall[c], __dmul_rn(st.spd[c], sp.dt));  // timeloop.h:791-796
    const uint32_t tn = st.t + 1;
    if (v.rec) {
      end_particle_fp32c(v, k, pre, wall_next);
    } else {
      unsigned long long *L = reinterpret_cast<unsigned long long *>(v.lrtb_next) + 6 * (uint64_t)k;
      if (P.movable) {
        for (int c = 0; c < 6; ++c) v.lrtb[6 * (uint64_t)k + c] = ord_val(L[c]);
      }
      for (int c = 0; c < 3; ++c) {
        L[c] = ord_key(INFINITY);
        L[3 + c] = ord_key(-INFINITY);
      }
    }
    // clamped nodes are zeroed after the corrector (timeloop.h:767-774); their CurrPos
    // keeps this step's predicted displacement, saved for the readback (the fused FP32 form
    // zeroes them in its corrector and keeps this step's displacement buffer intact)
    if (clamped_ptr && !v.fused) {
      double jump = 0;
      for (uint32_t c = clamped_ptr[k]; c < clamped_ptr[k + 1]; ++c) {
        uint64_t g = clamped[c];
        D3 d = ld3(v.disp, g, v.Ncap);
        clamped_disp[3 * (uint64_t)c] = d.x;
        clamped_disp[3 * (uint64_t)c + 1] = d.y;
        clamped_disp[3 * (uint64_t)c + 2] = d.z;
        if (P.movable) {
          jump = fmax(jump, norm3(d));
          st3(v.disp, g, v.Ncap, d3(0.0, 0.0, 0.0));
          st3(v.vel_out, g, v.Ncap, d3(0.0, 0.0, 0.0));
          st3(v.acc, g, v.Ncap, d3(0.0, 0.0, 0.0));
        }
      }
      if (jump > 0) atomicMax(&v.cnt->stepmax_bits, (unsigned long long)__double_as_longlong(jump));
    }
    // per-particle toggles for the next step (timeloop.h:481-498)
    const uint32_t kl = k - sp.p0;
    if (sp.set_movable_index != -1 && (uint32_t)sp.set_movable_index == kl && (uint32_t)sp.set_movable_ts == tn)
      P.movable = 1;
    if (sp.set_stoppable_index != -1 && (uint32_t)sp.set_stoppable_index == kl &&
        (uint32_t)sp.set_stoppable_ts == tn)
      P.stoppable = 1;
    // FP32 form: does any node of this particle need FP64 non-bond work next step besides
    // contact (which the contact-node list covers)? External force, torque, or a wall within
    // the contact radius of the particle's box grown by this step's movement bound
    // (k_extra32 then tests each node exactly).
    if (v.xparts) {
      const bool torque_next = st.torque || (sp.set_torque_ts != -1 && tn == (uint32_t)sp.set_torque_ts);
      bool need = (P.movable && P.has_ext) || torque_next;
      if (!need && P.movable && P.stoppable && sp.allow_wall) {
        const double lim = __dadd_rn(__dadd_rn(__dmul_rn(sp.Rc, 1.001), __dmul_rn(2.0, move)), 1e-12);
        const double *b = v.lrtb + 6 * (uint64_t)k;
        for (int f = 0; f < 6 && !need; ++f) {
          const int c = f % 3;
          need = (b[c] - lim <= wall_next[f]) && (b[3 + c] + lim >= wall_next[f]);
        }
      }
      if (need) v.xparts[atomicAdd(&v.xcount[1], 1u)] = k;
    }
  }
}

// The FP32 form's end_step_particle for particle k by one warp (all 32 lanes call it with the same
// k): lane c < 3 takes coordinate c of the box, the anchors and the extent, lane f < 6 face f of
// the box keys, the wall planes and the wall test of the work list. Every quantity is computed with
// end_step_particle's arithmetic, so both give the same state; the warp form shortens the chain
// of dependent loads and FP64 operations each particle waits on.
__device__ __forceinline__ void end_particle_warp(const DevView &v, uint32_t k, uint32_t lane) {
  const unsigned full = 0xffffffffu;
  DevPart &P = v.parts[k];
  const uint32_t sim = v.S == 1 ? 0u : P.sim;  // one simulation: its state loads need not wait for P
  const DevSimState &st = v.ss[sim];
  const DevSimParams &sp = v.sp[sim];
  unsigned int *L = v.lrtb_local_next + 6 * (uint64_t)k;
  const uint64_t k3 = 3 * (uint64_t)k;
  const unsigned int key = lane < 6 ? L[lane] : 0u;
  double an = 0.0, ann = 0.0, dn = 0.0, apos = 0.0;
  double blo = 0.0, bhi = 0.0;  // lanes < 3: coordinate lane of the particle's box, as kept below
  if (lane < 3) {
    an = v.anchor[k3 + lane];
    ann = v.anchor_next[k3 + lane];
    dn = v.disp_next[P.anchor + lane * v.Ncap];
    apos = P.anchor_pos[lane];
    blo = v.lrtb[6 * (uint64_t)k + lane];
    bhi = v.lrtb[6 * (uint64_t)k + 3 + lane];
  }
  const double move = __longlong_as_double((long long)v.cnt->stepmax_bits);  // this step's bound
  if (!st.active) return;
  const uint32_t c = lane % 3u;
  const double wn = lane < 6 ? __dadd_rn(st.wall[lane], __dmul_rn(st.spd[lane], sp.dt)) : 0.0;  // timeloop.h:791-796
  const uint32_t tn = st.t + 1;
  const int32_t movable = P.movable;
  // box from the local-frame keys (end_particle_fp32c)
  const unsigned int klo = __shfl_sync(full, key, c), khi = __shfl_sync(full, key, c + 3);
  double ext = 0.0;
  if (movable && lane < 3) {
    const float lo = fval(klo), hi = fval(khi);
    const double base = apos + an;
    const double w = __dadd_rn(__dmul_rn(8.0 * (double)FLT_EPSILON, fmax(fabs((double)lo), fabs((double)hi))), 1e-30);
    blo = base + (double)lo - w;
    bhi = base + (double)hi + w;
    v.lrtb[6 * (uint64_t)k + lane] = blo;
    v.lrtb[6 * (uint64_t)k + 3 + lane] = bhi;
    ext = fmax(fabs((double)lo), fabs((double)hi)) + w;
  }
  for (int o = 1; o < 4; o <<= 1) ext = fmax(ext, __shfl_xor_sync(full, ext, o));
  if (movable && lane == 0) set_break_band(P, u_extent(P, ext));
  if (lane < 6) L[lane] = lane < 3 ? fkey(INFINITY) : fkey(-INFINITY);
  // wall planes of the next step in the frame of the next step's anchor
  const double apos_c = __shfl_sync(full, apos, c), ann_c = __shfl_sync(full, ann, c);
  if (lane < 6) v.wall_local[6 * (uint64_t)k + lane] = (float)(wn - (apos_c + ann_c));
  if (lane < 3) {
    const_cast<double *>(v.anchor)[k3 + lane] = ann;
    v.anchor_next[k3 + lane] = dn;
  }
  // per-particle toggles for the next step (timeloop.h:481-498)
  int32_t mov = movable, stop = P.stoppable;  // the flags after the toggles
  if (lane == 0) {
    const uint32_t kl = k - sp.p0;
    if (sp.set_movable_index != -1 && (uint32_t)sp.set_movable_index == kl && (uint32_t)sp.set_movable_ts == tn) {
      P.movable = 1;
      mov = 1;
    }
    if (sp.set_stoppable_index != -1 && (uint32_t)sp.set_stoppable_index == kl &&
        (uint32_t)sp.set_stoppable_ts == tn) {
      P.stoppable = 1;
      stop = 1;
    }
  }
  mov = __shfl_sync(full, mov, 0);
  stop = __shfl_sync(full, stop, 0);
  // work list of particles with FP64 non-bond work next step (end_step_particle); the box and
  // flags come from the lanes that computed them, not back from memory
  const double lo_c = __shfl_sync(full, blo, c), hi_c = __shfl_sync(full, bhi, c);
  if (v.xparts) {
    const bool torque_next = st.torque || (sp.set_torque_ts != -1 && tn == (uint32_t)sp.set_torque_ts);
    bool need = (mov && P.has_ext) || torque_next;
    if (!need && mov && stop && sp.allow_wall) {
      const double lim = __dadd_rn(__dadd_rn(__dmul_rn(sp.Rc, 1.001), __dmul_rn(2.0, move)), 1e-12);
      const bool hit = lane < 6 && (lo_c - lim <= wn) && (hi_c + lim >= wn);
      need = __any_sync(full, hit);
    }
    if (need && lane == 0) v.xparts[atomicAdd(&v.xcount[1], 1u)] = k;
  }
}

// After every particle's end of step: the simulations advance (walls, step index, sticky
// toggles, timeloop.h:785-797) and the broad phase's movement bookkeeping. Threads tid of
// nthreads share the simulations; the last of them takes the counters, beside the first's
// simulation. With decide, the counters also take the next step's rebuild decision and restart
// its per-step counts, as bp_decide would at the start of that step (this step's bound having
// just restarted at 0).
__device__ __forceinline__ void end_step_advance(const DevView &v, uint32_t tid, uint32_t nthreads,
                                                 bool decide = false, double half_skin = 0.0) {
  for (uint32_t s = tid; s < v.S; s += nthreads) {
    const DevSimParams &sp = v.sp[s];
    DevSimState &st = v.ss[s];
    if (st.active) {
      for (int c = 0; c < 6; ++c) st.wall[c] = __dadd_rn(st.wall[c], __dmul_rn(st.spd[c], sp.dt));  // timeloop.h:791-796
      st.t += 1;
      apply_sim_toggles(sp, st, st.t);
    }
  }
  if (tid == nthreads - 1) {
    DevCounters &c = *v.cnt;
    const double stepmax = __longlong_as_double((long long)c.stepmax_bits);
    double moved;
    if (c.rebuild) {
      // with the fused predictor, stepmax already bounds the next step's movement
      moved = v.fused ? stepmax : 0.0;
      c.rebuilds += 1;
    } else {
      moved = c.moved + stepmax;
    }
    c.moved = moved;
    c.last_stepmax = stepmax;
    c.stepmax_bits = 0;
    c.rebuild = decide && moved > half_skin ? 1u : 0u;  // bp_decide: moved + 0 against half the skin
    if (decide) {
      c.contacts = 0;
      c.live_bonds = 0;
    }
    c.end_blocks = 0;
  }
}

}  // namespace pdg
#endif
