// pd_oracle.cpp -- TEST INFRASTRUCTURE (the checker, never the product).
//
// CPU restatement of PeriDEM's explicit step for the oracle: every function names the
// reference lines it restates. FP64 throughout, compiled with -ffp-contract=off so that no
// multiply-add is fused; the order of every sum follows the reference:
//   * Eigen 3.3's norm()/dot() on a 1x3 double row reduce as (x0 + x1) + x2 (one SSE2/NEON
//     packet of two lanes, then the tail), so norm(v) = sqrt((x*x + y*y) + z*z);
//   * vector<Matrix> arithmetic of src/compat/overloads.h:21-159 is element-wise, in order;
//   * the force on a node is accumulated in the order of timeloop.h:544-651 (PD sum,
//     self-contact, walls, extforce, torque, then particle pairs in lexicographic order).
#include "pd_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct V3 {
  double c[3];
};
inline V3 v3(double x, double y, double z) { return V3{{x, y, z}}; }
inline V3 vzero() { return v3(0.0, 0.0, 0.0); }
inline V3 vsub(const V3 &a, const V3 &b) { return v3(a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]); }
inline V3 vadd(const V3 &a, const V3 &b) { return v3(a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]); }
inline V3 vscale(double s, const V3 &a) { return v3(s * a.c[0], s * a.c[1], s * a.c[2]); }
inline V3 vdiv(const V3 &a, double s) { return v3(a.c[0] / s, a.c[1] / s, a.c[2] / s); }
inline void vacc(V3 &a, const V3 &b) {
  a.c[0] += b.c[0];
  a.c[1] += b.c[1];
  a.c[2] += b.c[2];
}
// Eigen norm()/dot() reduction order (see file header).
inline double vnorm(const V3 &a) { return std::sqrt((a.c[0] * a.c[0] + a.c[1] * a.c[1]) + a.c[2] * a.c[2]); }
inline double vdot(const V3 &a, const V3 &b) { return (a.c[0] * b.c[0] + a.c[1] * b.c[1]) + a.c[2] * b.c[2]; }

struct Part {
  uint32_t n = 0, g0 = 0;
  std::vector<V3> pos, disp, cur, vel, acc, force, ext, afd;
  std::vector<double> vol;
  std::vector<uint32_t> bdry, clamped;
  std::vector<std::vector<uint32_t>> nbr;   // NbdArr
  std::vector<std::vector<V3>> xi;          // xi[i][j] = pos[q] - pos[i]
  std::vector<std::vector<double>> xin;     // |xi|
  std::vector<std::vector<double>> str;     // last stretch per bond
  double delta = 0, rho = 0, cnot = 0, snot = 0, tval = 0;
  int movable = 1, breakable = 1, stoppable = 1;
  uint32_t taxis = 2;
  bool break_bonds = true;
  double lrtb[6] = {0, 0, 0, 0, 0, 0};
};

struct Contact {
  double Rc, Kn, zeta, mu;
  int allow_damping, allow_friction, nl_bdry_only, self_contact, compute_wall_reaction;
  int cell_search = 0;  // visit only node pairs in neighbouring cells (see contact_force)
};

struct Wall {
  int allow;
  double w[6];    // x_min y_min z_min x_max y_max z_max (lrtb() order, contact.h:221-238)
  double spd[6];  // speeds in the same order
  V3 react[6];    // reactions in get_reaction() order (contact.h:256-273)
};

struct Worker {
  std::vector<V3> gf;
  V3 react[6];
  uint64_t pw = 0, contacts = 0;
};

}  // namespace

struct or_sim {
  std::vector<Part> P;
  uint32_t Ntot = 0;
  Contact cn{};
  Wall wall{};
  pd_config cfg{};
  // Timeloop fields (timeloop.h:71-115) after apply_config (timeloop.h:184-225)
  double dt = 0;
  int enable_fracture = 0, gradient_extforce = 0, enable_torque = 0, enable_velocity_constraint = 0;
  uint32_t extforce_maxstep = 0;
  uint32_t t = 0;
  int threads = 1;
  std::vector<Worker> workers;
  uint64_t last_pw = 0, last_contacts = 0, last_live = 0;
};

namespace {

// ParticleN::gen_xi (particle2.h:241-257).
void gen_xi(Part &p) {
  p.xi.assign(p.n, {});
  p.xin.assign(p.n, {});
  p.str.assign(p.n, {});
  for (uint32_t i = 0; i < p.n; ++i) {
    size_t ss = p.nbr[i].size();
    p.xi[i].resize(ss);
    p.xin[i].resize(ss);
    p.str[i].assign(ss, 0.0);
    for (size_t j = 0; j < ss; ++j) {
      uint32_t q = p.nbr[i][j];
      p.xi[i][j] = vsub(p.pos[q], p.pos[i]);
      p.xin[i][j] = vnorm(p.xi[i][j]);
    }
  }
}

// get_minmax<3> (contact.h:1187-1225); std::min(a,b) = (b<a)?b:a, std::max(a,b) = (a<b)?b:a.
void get_minmax(const std::vector<V3> &P, double out[6]) {
  out[0] = P[0].c[0];
  out[1] = P[0].c[1];
  out[2] = P[0].c[2];
  out[3] = P[0].c[0];
  out[4] = P[0].c[1];
  out[5] = P[0].c[2];
  for (size_t i = 0; i < P.size(); ++i) {
    for (int k = 0; k < 3; ++k) {
      double v = P[i].c[k];
      out[k] = (v < out[k]) ? v : out[k];
      out[3 + k] = (out[3 + k] < v) ? v : out[3 + k];
    }
  }
}

// intersects_box_fext<3> (contact.h:1143-1183): only box A is extended by c.
bool intersects_box_fext(const double *A, const double *B, double c) {
  double A_min_x = A[0] - c, A_min_y = A[1] - c, A_min_z = A[2] - c;
  double A_max_x = A[3] + c, A_max_y = A[4] + c, A_max_z = A[5] + c;
  return (A_min_x <= B[3]) && (A_max_x >= B[0]) && (A_max_y >= B[1]) && (A_min_y <= B[4]) &&
         (A_min_z <= B[5]) && (A_max_z >= B[2]);
}

// within_interior_fext (contact.h:1229-1243), which indexes its 6-entry 3D boxes as if
// they were 2D [left, right, top, bottom] boxes.
bool within_interior_fext(const double *A, const double *B, double c) {
  double A_Left = A[0] - c, A_Right = A[1] + c, A_Top = A[2] + c, A_Bottom = A[3] - c;
  return (B[0] < A_Left) && (A_Right < B[1]) && (B[2] > A_Top) && (B[3] < A_Bottom);
}

// ParticleN::mean_CurrPos (particle2.h:94-103).
V3 mean_currpos(const Part &p) {
  V3 m = vzero();
  for (uint32_t i = 0; i < p.n; ++i) vacc(m, vadd(p.pos[i], p.disp[i]));
  double nn = (double)p.n;
  return v3(m.c[0] / nn, m.c[1] / nn, m.c[2] / nn);
}

// ParticleN::get_peridynamic_force (particle2.h:107-193), added into gf[g0 + i]
// (timeloop.h:546-549).
void peridynamic_force(Part &p, std::vector<V3> &gf) {
  for (uint32_t i = 0; i < p.n; ++i) {
    V3 v = vzero();
    const std::vector<uint32_t> &nb = p.nbr[i];
    for (size_t j = 0; j < nb.size(); ++j) {
      uint32_t q = nb[j];
      V3 eta = vadd(vsub(p.disp[q], p.disp[i]), p.xi[i][j]);
      double en = vnorm(eta);
      double xn = p.xin[i][j];
      double diff = en - xn;
      double s = diff / xn;
      double mag = (p.cnot * s) * p.vol[q];
      V3 unit = vdiv(eta, en);
      vacc(v, vscale(mag, unit));
      p.str[i][j] = s;
    }
    vacc(gf[p.g0 + i], v);
  }
}

// ParticleN::remove_bonds (particle2.h:196-237): drop bonds with stretch > snot.
void remove_bonds(Part &p) {
  if (!p.break_bonds) return;
  for (uint32_t i = 0; i < p.n; ++i) {
    size_t w = 0;
    for (size_t j = 0; j < p.nbr[i].size(); ++j) {
      if (p.str[i][j] > p.snot) continue;
      p.nbr[i][w] = p.nbr[i][j];
      p.xi[i][w] = p.xi[i][j];
      p.xin[i][w] = p.xin[i][j];
      p.str[i][w] = p.str[i][j];
      ++w;
    }
    p.nbr[i].resize(w);
    p.xi[i].resize(w);
    p.xin[i].resize(w);
    p.str[i].resize(w);
  }
}

// update_contact_force_by_boundary<3> (contact.h:744-942). `pair` is the loop body for node
// i of C and node j of N; the reference visits every (i, j), i outer, both ascending in the
// iteration lists. With cn.cell_search the same pairs are visited in the same order, but only
// those whose current positions lie in neighbouring cells of edge > Rc: every other pair fails
// the first test (|dir| <= Rc), so the sums are bit-identical and the cost follows the pairs in
// reach instead of nC * nN (the checker of large cases; timing runs use the plain loops).
uint64_t contact_force(const Part &C, const Part &N, const Contact &cn, double dt,
                       std::vector<V3> &gf, bool self) {
  uint64_t contacts = 0;
  uint32_t tn_i = cn.nl_bdry_only ? (uint32_t)C.bdry.size() : C.n;
  uint32_t tn_j = cn.nl_bdry_only ? (uint32_t)N.bdry.size() : N.n;
  auto pair = [&](uint32_t i, uint32_t j) {
    V3 xi_ij = vsub(N.pos[j], C.pos[i]);
    V3 dir = vadd(vsub(N.disp[j], C.disp[i]), xi_ij);
    double dn = vnorm(dir);
    if (!(dn <= cn.Rc)) return;
    bool do_compute = true;
    double xin = vnorm(xi_ij);
    double len_ref = cn.Rc;
    double sc = cn.Kn * cn.Rc;
    if (self) {
      if (i == j) {
        do_compute = false;
      } else if (std::find(C.nbr[i].begin(), C.nbr[i].end(), j) != C.nbr[i].end()) {
        do_compute = false;
      } else if (xin < cn.Rc) {
        len_ref = xin;
        sc = N.cnot;
      } else {
        len_ref = cn.Rc;
      }
    }
    if (!(do_compute && (dn < len_ref))) return;
    ++contacts;
    double N_vol = N.vol[j];
    V3 unit = vdiv(dir, dn);
    double s = (dn - len_ref) / len_ref;
    double fmag = (sc * s) * N_vol;
    V3 fc = vscale(fmag, unit);
    double fcn = vnorm(fc);
    uint32_t gi = C.g0 + i, gj = N.g0 + j;
    if (C.stoppable) vacc(gf[gi], fc);
    if (!self && N.stoppable) {
      double cv = C.vol[i];
      for (int k = 0; k < 3; ++k) gf[gj].c[k] -= (fc.c[k] / N_vol) * cv;
    }
    if (cn.allow_damping) {
      V3 rel = vsub(C.vel[i], N.vel[j]);
      double rvp = vdot(rel, unit);
      V3 rvn = vscale(rvp, unit);
      double dc = ((2.0 * cn.zeta) * std::sqrt(sc * C.rho)) * std::sqrt(N_vol);
      V3 fd = vscale(-dc, rvn);
      if (C.stoppable) vacc(gf[gi], fd);
      if (!self && N.stoppable) {
        double sn = std::sqrt(N_vol), sv = std::sqrt(C.vol[i]);
        for (int k = 0; k < 3; ++k) gf[gj].c[k] -= (fd.c[k] / sn) * sv;
      }
    }
    if (cn.allow_friction) {
      V3 rel = vsub(C.vel[i], N.vel[j]);
      double rd = vdot(rel, unit);
      V3 rvt = vsub(rel, vscale(rd, unit));
      double rvtn = vnorm(rvt);
      if (rvtn > 0) {
        V3 tu = vdiv(rvt, vnorm(rvt));
        V3 ff = vscale((-cn.mu) * fcn, tu);
        if (rvtn < ((cn.mu * fcn) * dt) / C.rho) ff = vscale(((-rvtn) / C.rho) / dt, tu);
        if (C.stoppable) vacc(gf[gi], ff);
        if (!self && N.stoppable) {
          for (int k = 0; k < 3; ++k) gf[gj].c[k] -= ff.c[k];
        }
      }
    }
  };
  if (!cn.cell_search || (uint64_t)tn_i * tn_j <= 4096) {
    for (uint32_t pp = 0; pp < tn_i; ++pp) {
      uint32_t i = cn.nl_bdry_only ? C.bdry[pp] : pp;
      for (uint32_t qq = 0; qq < tn_j; ++qq) pair(i, cn.nl_bdry_only ? N.bdry[qq] : qq);
    }
    return contacts;
  }
  // cells of edge h > Rc over N's iterated nodes (current positions pos + disp); a pair with
  // |dir| <= Rc has |cur_j - cur_i| <= Rc up to rounding (1e-15 relative), so it lies in
  // neighbouring cells
  const double h = cn.Rc * 1.001;
  double lo[3] = {INFINITY, INFINITY, INFINITY};
  for (uint32_t qq = 0; qq < tn_j; ++qq) {
    const V3 &x = N.cur[cn.nl_bdry_only ? N.bdry[qq] : qq];
    for (int c = 0; c < 3; ++c) lo[c] = std::min(lo[c], x.c[c]);
  }
  auto cell = [&](const V3 &x, int64_t *k) {
    for (int c = 0; c < 3; ++c) k[c] = (int64_t)std::floor((x.c[c] - lo[c]) / h);
  };
  auto key = [](int64_t a, int64_t b, int64_t c) {
    return ((uint64_t)(a + (1 << 20)) << 42) | ((uint64_t)(b + (1 << 20)) << 21) | (uint64_t)(c + (1 << 20));
  };
  std::vector<std::pair<uint64_t, uint32_t>> grid(tn_j);
  for (uint32_t qq = 0; qq < tn_j; ++qq) {
    int64_t k[3];
    cell(N.cur[cn.nl_bdry_only ? N.bdry[qq] : qq], k);
    grid[qq] = {key(k[0], k[1], k[2]), qq};
  }
  std::sort(grid.begin(), grid.end());
  std::vector<uint32_t> cand;
  for (uint32_t pp = 0; pp < tn_i; ++pp) {
    uint32_t i = cn.nl_bdry_only ? C.bdry[pp] : pp;
    int64_t k[3];
    cell(C.cur[i], k);
    if (k[0] < -2 || k[1] < -2 || k[2] < -2 || k[0] > (1 << 19) || k[1] > (1 << 19) || k[2] > (1 << 19)) continue;
    cand.clear();
    for (int64_t a = k[0] - 1; a <= k[0] + 1; ++a)
      for (int64_t b2 = k[1] - 1; b2 <= k[1] + 1; ++b2)
        for (int64_t c = k[2] - 1; c <= k[2] + 1; ++c) {
          if (a < -1 || b2 < -1 || c < -1) continue;
          const uint64_t kk = key(a, b2, c);
          auto it = std::lower_bound(grid.begin(), grid.end(), std::make_pair(kk, 0u));
          for (; it != grid.end() && it->first == kk; ++it) cand.push_back(it->second);
        }
    std::sort(cand.begin(), cand.end());
    for (uint32_t qq : cand) pair(i, cn.nl_bdry_only ? N.bdry[qq] : qq);
  }
  return contacts;
}

// segment_mass<3> (contact.h:14-39): spherical-cap volume and centroid; pow(x,2) is x*x.
inline void segment_mass(double R, double d, double &centroid, double &area) {
  double rd = R - d;
  area = ((M_PI / 3) * (rd * rd)) * (2 * R - d);
  double w = R * R - d * d;
  double I = (M_PI / 4) * (w * w);
  centroid = I / area;
}

// wall_side_force_update<3> (contact.h:381-502).
void wall_side(double dist, const Contact &cn, unsigned dir, const V3 &vel_i, double vol_i,
               double rho, V3 &f, double dt, double wspeed, V3 &react) {
  if (!(std::fabs(dist) <= cn.Rc)) return;
  double cen, area;
  segment_mass(cn.Rc, std::fabs(dist), cen, area);
  double crc = cn.Rc - cen;
  double pcrc = (crc > 0 ? crc : 0);
  double F = (cn.Kn * pcrc) * area;
  double c_sign = (dist > 0 ? 1 : -1);
  f.c[dir] += (c_sign * F);
  react.c[dir] -= ((vol_i * c_sign) * F);
  V3 rel = vel_i;
  rel.c[dir] -= wspeed;
  if (cn.allow_friction) {
    unsigned t1 = (dir + 1) % 3, t2 = (dir + 2) % 3;
    double v1 = rel.c[t1], v2 = rel.c[t2];
    double vn = std::sqrt(v1 * v1 + v2 * v2);
    if (vn > 0) {
      double u1 = v1 / vn, u2 = v2 / vn;
      double ff1 = ((-cn.mu) * std::fabs(F)) * u1;
      double ff2 = ((-cn.mu) * std::fabs(F)) * u2;
      if (vn < ((cn.mu * std::fabs(F)) * dt) / rho) {
        ff1 = (((-vn) / rho) / dt) * u1;
        ff2 = (((-vn) / rho) / dt) * u2;
      }
      f.c[t1] += ff1;
      f.c[t2] += ff2;
      react.c[t1] -= (vol_i * ff1);
      react.c[t2] -= (vol_i * ff2);
    }
  }
  if (cn.allow_damping) {
    double dc = ((2 * cn.zeta) * std::sqrt(cn.Kn * rho)) * std::sqrt(std::fabs(area));
    double df = (-dc) * rel.c[dir];
    f.c[dir] += df;
    react.c[dir] -= (vol_i * df);
  }
}

// update_wall_contact_force_by_boundary<3> (contact.h:1057-1124): faces in the order
// x_min, x_max, y_min, y_max, z_min, z_max.
void wall_contact(const Part &p, Wall &wall, V3 *react, const Contact &cn, double dt,
                  std::vector<V3> &gf) {
  uint32_t tn = cn.nl_bdry_only ? (uint32_t)p.bdry.size() : p.n;
  static const int face_of[6] = {0, 3, 1, 4, 2, 5};  // lrtb index of each face in call order
  for (uint32_t pp = 0; pp < tn; ++pp) {
    uint32_t i = cn.nl_bdry_only ? p.bdry[pp] : pp;
    V3 &f = gf[p.g0 + i];
    for (int k = 0; k < 6; ++k) {
      int fi = face_of[k];
      unsigned dir = (unsigned)(fi % 3);
      double dist = p.cur[i].c[dir] - wall.w[fi];
      wall_side(dist, cn, dir, p.vel[i], p.vol[i], p.rho, f, dt, wall.spd[fi], react[fi]);
    }
  }
}

// External torque about the centroid (timeloop.h:600-633).
void torque(const Part &p, std::vector<V3> &gf) {
  V3 c = mean_currpos(p);
  unsigned ta = p.taxis;
  for (uint32_t nn = 0; nn < p.n; ++nn) {
    V3 r = vsub(p.cur[nn], c);
    double rn = vnorm(r);
    double r_inv = (rn != 0.0 ? 1 / rn : 0);
    r.c[ta] = 0;
    V3 perp = vzero();
    perp.c[ta] = 0;
    perp.c[(ta + 1) % 3] = -r.c[(ta + 2) % 3];
    perp.c[(ta + 2) % 3] = r.c[(ta + 1) % 3];
    double pn = vnorm(perp);
    if (pn > 0) {
      perp = vdiv(perp, pn);
    } else {
      perp.c[(ta + 1) % 3] = 0;
      perp.c[(ta + 2) % 3] = 0;
    }
    double s = r_inv * p.tval;
    vacc(gf[p.g0 + nn], vscale(s, perp));
  }
}

void reset_partzero_y(or_sim &S) {
  // timeloop.h:500-535 (uses particle 1's pos[0] and disp[1] for the initial value).
  std::vector<Part> &P = S.P;
  if (P.size() < 2) return;
  double max_bulk_y = P[1].pos[0].c[1] + P[1].disp[1 < P[1].n ? 1 : 0].c[1];
  bool init = true;
  V3 m0 = mean_currpos(P[0]);
  for (size_t i = 1; i < P.size(); ++i) {
    for (uint32_t j = 0; j < P[i].n; ++j) {
      double now_x = P[i].pos[j].c[0] + P[i].disp[j].c[0];
      double now_y = P[i].pos[j].c[1] + P[i].disp[j].c[1];
      if (std::fabs(m0.c[0] - now_x) <= S.cfg.wheel_rad) {
        if (init) {
          max_bulk_y = now_y;
          init = !init;
        } else if (now_y > max_bulk_y) {
          max_bulk_y = now_y;
        }
      }
    }
  }
  double dest = max_bulk_y + S.cfg.wheel_rad + S.cn.Rc;
  double to_move_by = dest - mean_currpos(P[0]).c[1];
  for (uint32_t j = 0; j < P[0].n; ++j) P[0].pos[j].c[1] += to_move_by;
}

// Prescribed-velocity handling of one particle (timeloop.h:684-764).
void prescribed_velocity(or_sim &S, Part &p, const std::vector<V3> &acc_old) {
  const pd_config &cf = S.cfg;
  V3 mean_vel = vzero();
  for (uint32_t k = 0; k < p.n; ++k) vacc(mean_vel, p.vel[k]);
  double nn = (double)p.n;
  mean_vel = v3(mean_vel.c[0] / nn, mean_vel.c[1] / nn, mean_vel.c[2] / nn);
  std::vector<V3> vrot(p.n);
  for (uint32_t k = 0; k < p.n; ++k) vrot[k] = vsub(p.vel[k], mean_vel);
  if (cf.fix_velocity_mean_x) mean_vel.c[0] = cf.prescribed_velocity_mean_x;
  if (cf.fix_velocity_angular) {
    V3 mpos = mean_currpos(p);
    for (uint32_t k = 0; k < p.n; ++k) {
      V3 rv = vsub(p.cur[k], mpos);
      double r = vnorm(rv);
      V3 ru = vzero();
      if (r > 0) ru = vdiv(rv, r);
      V3 pvt = vzero();
      pvt.c[0] = -(r * cf.prescribed_angular_vel) * ru.c[1];
      pvt.c[1] = (r * cf.prescribed_angular_vel) * ru.c[0];
      vrot[k] = pvt;
    }
  }
  std::vector<V3> pv(p.n);
  for (uint32_t k = 0; k < p.n; ++k) pv[k] = vadd(vrot[k], mean_vel);
  p.vel = pv;
  double two_dt = 2 / S.dt;
  for (uint32_t k = 0; k < p.n; ++k) {
    V3 d = vsub(pv[k], p.vel[k]);
    V3 a = vsub(vscale(two_dt, d), acc_old[k]);
    p.afd[k] = vsub(vscale(p.rho, a), p.force[k]);
  }
}

// Lexicographic pair index -> (i, j), i < j (timeloop.h:244-255).
void step_once(or_sim &S) {
  std::vector<Part> &P = S.P;
  const uint32_t np = (uint32_t)P.size();
  const uint32_t t = ++S.t;
  const pd_config &cf = S.cfg;
  Wall &wall = S.wall;
  for (int k = 0; k < 6; ++k) wall.react[k] = vzero();  // timeloop.h:397

  // scheduled toggles (timeloop.h:405-535)
  if (cf.set_torque_timestep != -1 && t == (unsigned)cf.set_torque_timestep) S.enable_torque = 1;
  if (cf.set_fix_velocity_timestep != -1 && t == (unsigned)cf.set_fix_velocity_timestep)
    S.enable_velocity_constraint = 1;
  if (cf.set_fracture_timestep != -1 && t == (unsigned)cf.set_fracture_timestep) S.enable_fracture = 1;
  if (cf.set_self_contact_timestep != -1 && t == (unsigned)cf.set_self_contact_timestep)
    S.cn.self_contact = 1;
  if (cf.set_damping_timestep != -1 && t == (unsigned)cf.set_damping_timestep) S.cn.allow_damping = 1;
  if (cf.set_zero_wall_speed_timestep != -1 && t == (unsigned)cf.set_zero_wall_speed_timestep)
    for (int k = 0; k < 6; ++k) wall.spd[k] = 0;
  // brazil-nut toggles (timeloop.h:467-479) only touch the 2D wall fields: no 3D effect.
  if (cf.set_movable_index != -1 && (unsigned)cf.set_movable_timestep == t &&
      (unsigned)cf.set_movable_index < np)
    P[(unsigned)cf.set_movable_index].movable = 1;
  if (cf.set_stoppable_index != -1 && (unsigned)cf.set_stoppable_timestep == t &&
      (unsigned)cf.set_stoppable_index < np)
    P[(unsigned)cf.set_stoppable_index].stoppable = 1;
  if (cf.reset_partzero_y && cf.reset_partzero_y_timestep == t) reset_partzero_y(S);

  // predictor for all particles (timeloop.h:537-540)
  const double dt = S.dt;
  const double hdt2 = (dt * dt) * 0.5;
  for (uint32_t i = 0; i < np; ++i) {
    Part &p = P[i];
    for (uint32_t k = 0; k < p.n; ++k) {
      for (int c = 0; c < 3; ++c) {
        p.disp[k].c[c] = p.disp[k].c[c] + ((dt * p.vel[k].c[c]) + (hdt2 * p.acc[k].c[c]));
        p.cur[k].c[c] = p.pos[k].c[c] + p.disp[k].c[c];
      }
    }
  }

  uint64_t live = 0;
  for (uint32_t i = 0; i < np; ++i)
    if (P[i].movable)
      for (uint32_t k = 0; k < P[i].n; ++k) live += P[i].nbr[k].size();
  S.last_live = live;

  const int R = S.threads;
  for (int r = 0; r < R; ++r) {
    Worker &w = S.workers[r];
    std::fill(w.gf.begin(), w.gf.end(), vzero());
    for (int k = 0; k < 6; ++k) w.react[k] = vzero();
    w.pw = 0;
    w.contacts = 0;
  }
  const uint64_t npairs = (uint64_t)np * (np - 1) / 2;

#pragma omp parallel num_threads(R) if (R > 1)
  {
    int r = 0;
#ifdef _OPENMP
    r = omp_get_thread_num();
#endif
    Worker &w = S.workers[r];
    // per-particle phase, rank-strided (timeloop.h:544-634)
    for (uint32_t i = (uint32_t)r; i < np; i += (uint32_t)R) {
      Part &p = P[i];
      if (p.movable) {
        peridynamic_force(p, w.gf);
        if (S.enable_fracture && p.breakable) {
          remove_bonds(p);
          if (S.cn.self_contact) contact_force(p, p, S.cn, dt, w.gf, true);
        }
        if (p.stoppable) {
          if (wall.allow && !within_interior_fext(p.lrtb, wall.w, S.cn.Rc))
            wall_contact(p, wall, w.react, S.cn, dt, w.gf);
        }
        if (S.gradient_extforce) {
          double sc = (double)t / (double)S.extforce_maxstep;
          if (sc > 1) sc = 1;
          for (uint32_t k = 0; k < p.n; ++k) vacc(w.gf[p.g0 + k], vscale(sc, p.ext[k]));
        } else {
          for (uint32_t k = 0; k < p.n; ++k) vacc(w.gf[p.g0 + k], p.ext[k]);
        }
      }
      if (S.enable_torque) torque(p, w.gf);
    }
    // particle-pair phase, rank-strided over the lexicographic pair list (timeloop.h:636-651)
    uint64_t pidx = 0;
    for (uint32_t i = 0; i < np; ++i) {
      for (uint32_t j = i + 1; j < np; ++j, ++pidx) {
        if ((pidx % (uint64_t)R) != (uint64_t)r) continue;
        if (P[i].movable || P[j].movable) {
          if (intersects_box_fext(P[i].lrtb, P[j].lrtb, S.cn.Rc)) {
            w.contacts += contact_force(P[i], P[j], S.cn, dt, w.gf, false);
            w.pw++;
          }
        }
      }
    }
  }
  (void)npairs;

  // force reduction (MPI_Allreduce, timeloop.h:658-659): rank order sum
  std::vector<V3> &gf = S.workers[0].gf;
  for (int r = 1; r < R; ++r) {
    const std::vector<V3> &o = S.workers[r].gf;
    for (uint32_t k = 0; k < S.Ntot; ++k) vacc(gf[k], o[k]);
  }
  S.last_pw = 0;
  S.last_contacts = 0;
  for (int r = 0; r < R; ++r) {
    for (int k = 0; k < 6; ++k) vacc(wall.react[k], S.workers[r].react[k]);
    S.last_pw += S.workers[r].pw;
    S.last_contacts += S.workers[r].contacts;
  }

  // corrector (timeloop.h:661-781)
  const double hdt = 0.5 * dt;
#pragma omp parallel for num_threads(R) if (R > 1) schedule(dynamic)
  for (uint32_t i = 0; i < np; ++i) {
    Part &p = P[i];
    for (uint32_t k = 0; k < p.n; ++k) p.force[k] = gf[p.g0 + k];
    if (!p.movable) continue;
    std::vector<V3> acc_old = p.acc;
    const double irho = 1 / p.rho;
    for (uint32_t k = 0; k < p.n; ++k) {
      for (int c = 0; c < 3; ++c) {
        double an = irho * p.force[k].c[c];
        p.acc[k].c[c] = an;
        double tmp = acc_old[k].c[c] + an;
        tmp = tmp * hdt;
        p.vel[k].c[c] = p.vel[k].c[c] + tmp;
      }
    }
    if ((int64_t)i == (int64_t)(unsigned)cf.particle_w_fixed_velocity && S.enable_velocity_constraint)
      prescribed_velocity(S, p, acc_old);
    for (uint32_t cid : p.clamped) {
      p.disp[cid] = vzero();
      p.vel[cid] = vzero();
      p.acc[cid] = vzero();
    }
    get_minmax(p.cur, p.lrtb);
  }

  // wall boundary update (timeloop.h:790-797)
  for (int k = 0; k < 6; ++k) wall.w[k] += wall.spd[k] * dt;
}

}  // namespace

extern "C" {

// ConfigVal's defaults: the in-class initialisers (read_config.h:36-99) and the constructor
// (read_config.h:102-167). The oracle keeps its own copy so that its callers never need the
// engine library.
int or_config_default(pd_config *c) {
  if (!c) return PD_EINVAL;
  std::memset(c, 0, sizeof(*c));
  c->timesteps = 8000;
  c->modulo = 100;
  c->dt = 0.02 / 1e5;
  c->is_parallel = 1;
  c->resume_ind = 50;
  c->save_file = 1;
  c->allow_damping = 1;
  c->allow_friction = 1;
  c->self_contact = 1;
  c->self_contact_rad = -1;
  c->cohesion_scaling = 1;
  c->set_torque_timestep = -1;
  c->set_fracture_timestep = -1;
  c->set_self_contact_timestep = -1;
  c->set_zero_wall_speed_timestep = -1;
  c->set_damping_timestep = -1;
  c->set_movable_index = -1;
  c->set_movable_timestep = -1;
  c->set_stoppable_index = -1;
  c->set_stoppable_timestep = -1;
  c->particle_w_fixed_velocity = -1;
  c->set_fix_velocity_timestep = -1;
  c->prescribed_angular_vel = -999;
  c->prescribed_velocity_mean_x = -999;
  c->normal_stiffness = -1;
  c->damping_ratio = -1;
  c->friction_coefficient = -1;
  c->new_snot = -1;
  c->wall_left = c->wall_right = c->wall_top = c->wall_bottom = -999;
  c->wall_x_min = c->wall_y_min = c->wall_z_min = -999;
  c->wall_x_max = c->wall_y_max = c->wall_z_max = -999;
  c->brazil_reset_wall_bottom_freq = -1;
  c->brazil_nonzero_wall_bottom_speed_freq = -1;
  c->brazil_reset_wall_bottom_y = -999;
  c->forcefield_scaling = 1e9;
  std::strncpy(c->setup_filename, "data/hdf5/all.h5", sizeof(c->setup_filename) - 1);
  std::strncpy(c->output_dir, "output/hdf5/", sizeof(c->output_dir) - 1);
  return PD_OK;
}

or_sim *or_create(const pd_setup_arrays *su, const pd_config *cfg) {
  if (!su || !cfg || su->n_particles == 0) return nullptr;
  or_sim *S = new or_sim();
  S->cfg = *cfg;
  const uint32_t np = su->n_particles;
  S->P.resize(np);
  uint32_t g = 0;
  for (uint32_t pi = 0; pi < np; ++pi) {
    Part &p = S->P[pi];
    uint64_t a = su->node_offset[pi], b = su->node_offset[pi + 1];
    p.n = (uint32_t)(b - a);
    p.g0 = g;
    g += p.n;
    p.pos.resize(p.n);
    p.disp.resize(p.n);
    p.cur.resize(p.n);
    p.vel.resize(p.n);
    p.acc.resize(p.n);
    p.force.assign(p.n, vzero());
    p.ext.resize(p.n);
    p.afd.assign(p.n, vzero());
    p.vol.resize(p.n);
    for (uint32_t k = 0; k < p.n; ++k) {
      uint64_t n = a + k;
      p.pos[k] = v3(su->pos[3 * n], su->pos[3 * n + 1], su->pos[3 * n + 2]);
      p.disp[k] = v3(su->disp[3 * n], su->disp[3 * n + 1], su->disp[3 * n + 2]);
      p.vel[k] = v3(su->vel[3 * n], su->vel[3 * n + 1], su->vel[3 * n + 2]);
      p.acc[k] = v3(su->acc[3 * n], su->acc[3 * n + 1], su->acc[3 * n + 2]);
      p.ext[k] = v3(su->extforce[3 * n], su->extforce[3 * n + 1], su->extforce[3 * n + 2]);
      p.vol[k] = su->vol[n];
    }
    // conn2NArr (load_hdf5.h:27-37): row order of Connectivity decides neighbour order.
    p.nbr.assign(p.n, {});
    for (uint64_t l = su->conn_offset[pi]; l < su->conn_offset[pi + 1]; ++l) {
      uint32_t i = su->conn[2 * l], j = su->conn[2 * l + 1];
      p.nbr[i].push_back(j);
      p.nbr[j].push_back(i);
    }
    gen_xi(p);
    if (su->bdry_offset)
      for (uint64_t l = su->bdry_offset[pi]; l < su->bdry_offset[pi + 1]; ++l) p.bdry.push_back(su->bdry[l]);
    if (su->clamped_offset)
      for (uint64_t l = su->clamped_offset[pi]; l < su->clamped_offset[pi + 1]; ++l)
        p.clamped.push_back(su->clamped[l]);
    p.delta = su->delta[pi];
    p.rho = su->rho[pi];
    p.cnot = su->cnot[pi];
    p.snot = su->snot[pi];
    p.movable = su->movable[pi];
    p.breakable = su->breakable[pi];
    p.stoppable = su->stoppable[pi];
    p.taxis = su->torque_axis[pi];
    p.tval = su->torque_val[pi];
    p.break_bonds = true;  // simulate3d.cpp:137-139
  }
  S->Ntot = g;

  // Contact: load_contact (load_hdf5.h:115-127) then Contact::apply_config (contact.h:151-179)
  Contact &cn = S->cn;
  cn.Rc = su->contact_radius;
  cn.Kn = su->normal_stiffness;
  cn.zeta = su->damping_ratio;
  cn.mu = su->friction_coefficient;
  cn.allow_damping = cfg->allow_damping;
  cn.allow_friction = cfg->allow_friction;
  cn.nl_bdry_only = cfg->nl_bdry_only;
  if (cfg->damping_ratio != -1) cn.zeta = cfg->damping_ratio;
  if (cfg->friction_coefficient != -1) cn.mu = cfg->friction_coefficient;
  if (cfg->normal_stiffness != -1) cn.Kn = cfg->normal_stiffness;
  cn.self_contact = cfg->self_contact;
  cn.compute_wall_reaction = cfg->compute_wall_reaction;

  // Wall: load_wall<3> (load_hdf5.h:150-181) then RectWall::apply_config (contact.h:325-372)
  Wall &w = S->wall;
  w.allow = su->allow_wall ? 1 : 0;
  for (int k = 0; k < 6; ++k) w.w[k] = (su->n_geom_wall != 1) ? su->geom_wall_info[k] : 0.0;
  if (cfg->wall_top != -999) w.w[5] = cfg->wall_top;
  if (cfg->wall_right != -999) w.w[4] = cfg->wall_right;
  if (cfg->wall_x_min != -999) w.w[0] = cfg->wall_x_min;
  if (cfg->wall_y_min != -999) w.w[1] = cfg->wall_y_min;
  if (cfg->wall_z_min != -999) w.w[2] = cfg->wall_z_min;
  if (cfg->wall_x_max != -999) w.w[3] = cfg->wall_x_max;
  if (cfg->wall_y_max != -999) w.w[4] = cfg->wall_y_max;
  if (cfg->wall_z_max != -999) w.w[5] = cfg->wall_z_max;
  w.spd[0] = cfg->speed_wall_x_min;
  w.spd[1] = cfg->speed_wall_y_min;
  w.spd[2] = cfg->speed_wall_z_min;
  w.spd[3] = cfg->speed_wall_x_max;
  w.spd[4] = cfg->speed_wall_y_max;
  w.spd[5] = cfg->speed_wall_z_max;
  for (int k = 0; k < 6; ++k) w.react[k] = vzero();

  // Timeloop::apply_config (timeloop.h:184-225) and the snot override (timeloop.h:314-318)
  S->dt = cfg->dt;
  S->enable_fracture = cfg->enable_fracture;
  S->gradient_extforce = cfg->gradient_extforce;
  S->extforce_maxstep = cfg->extforce_maxstep;
  S->enable_torque = cfg->enable_torque;
  S->enable_velocity_constraint = 0;
  if (cfg->new_snot != -1)
    for (Part &p : S->P) p.snot = cfg->new_snot;

  // CurrPos and AABBs before the loop (timeloop.h:389-393)
  for (Part &p : S->P) {
    for (uint32_t k = 0; k < p.n; ++k) p.cur[k] = vadd(p.pos[k], p.disp[k]);
    if (p.n) get_minmax(p.cur, p.lrtb);
  }
  or_set_threads(S, 1);
  return S;
}

void or_set_cell_search(or_sim *S, int on) { S->cn.cell_search = on ? 1 : 0; }

void or_set_threads(or_sim *S, int threads) {
  if (threads < 1) threads = 1;
  S->threads = threads;
  S->workers.assign(threads, Worker{});
  for (Worker &w : S->workers) w.gf.assign(S->Ntot, vzero());
}

int or_step(or_sim *S, uint32_t nsteps) {
  if (!S) return PD_EINVAL;
  for (uint32_t k = 0; k < nsteps; ++k) step_once(*S);
  return PD_OK;
}

static void put3(double *dst, uint64_t n, const V3 &v) {
  dst[3 * n] = v.c[0];
  dst[3 * n + 1] = v.c[1];
  dst[3 * n + 2] = v.c[2];
}

int or_get_state(or_sim *S, double *curpos, double *vel, double *acc, double *force) {
  for (const Part &p : S->P) {
    for (uint32_t k = 0; k < p.n; ++k) {
      uint64_t n = p.g0 + k;
      if (curpos) put3(curpos, n, p.cur[k]);
      if (vel) put3(vel, n, p.vel[k]);
      if (acc) put3(acc, n, p.acc[k]);
      if (force) put3(force, n, p.force[k]);
    }
  }
  return PD_OK;
}

int or_get_disp(or_sim *S, double *disp) {
  for (const Part &p : S->P)
    for (uint32_t k = 0; k < p.n; ++k) put3(disp, p.g0 + k, p.disp[k]);
  return PD_OK;
}

int or_get_afd(or_sim *S, double *afd) {
  for (const Part &p : S->P)
    for (uint32_t k = 0; k < p.n; ++k) put3(afd, p.g0 + k, p.afd[k]);
  return PD_OK;
}

// NbdArr2conn (timeloop.h:20-44)
int or_get_connectivity(or_sim *S, uint32_t particle, uint32_t *pairs, uint64_t cap, uint64_t *n) {
  if (particle >= S->P.size()) return PD_EINVAL;
  const Part &p = S->P[particle];
  uint64_t c = 0;
  for (uint32_t i = 0; i < p.n; ++i) {
    for (uint32_t q : p.nbr[i]) {
      if (i < q) {
        if (pairs && c < cap) {
          pairs[2 * c] = i;
          pairs[2 * c + 1] = q;
        }
        ++c;
      }
    }
  }
  *n = c;
  return (pairs && c > cap) ? PD_EINVAL : PD_OK;
}

int or_get_wall(or_sim *S, double *wall_info, double *reaction) {
  for (int k = 0; k < 6; ++k) {
    if (wall_info) wall_info[k] = S->wall.w[k];
    if (reaction) put3(reaction, (uint64_t)k, S->wall.react[k]);
  }
  return PD_OK;
}

int or_get_aabb(or_sim *S, double *lrtb) {
  for (size_t i = 0; i < S->P.size(); ++i)
    for (int k = 0; k < 6; ++k) lrtb[6 * i + k] = S->P[i].lrtb[k];
  return PD_OK;
}

int or_get_counts(or_sim *S, uint64_t *counts) {
  counts[0] = S->last_pw;
  counts[1] = S->last_contacts;
  counts[2] = S->last_live;
  counts[3] = S->t;
  return PD_OK;
}

uint64_t or_get_stretch(or_sim *S, uint32_t particle, double *out, uint64_t cap) {
  if (particle >= S->P.size()) return 0;
  const Part &p = S->P[particle];
  uint64_t c = 0;
  for (uint32_t i = 0; i < p.n; ++i)
    for (double s : p.str[i]) {
      if (out && c < cap) out[c] = s;
      ++c;
    }
  return c;
}

// Resume support (timeloop.h:274-293): new disp/vel/acc (N*3, any may be NULL), then the
// CurrPos/AABB initialisation that precedes the loop (timeloop.h:389-393).
int or_set_state(or_sim *S, const double *disp, const double *vel, const double *acc) {
  for (Part &p : S->P) {
    for (uint32_t k = 0; k < p.n; ++k) {
      const uint64_t n = p.g0 + k;
      for (int c = 0; c < 3; ++c) {
        if (disp) p.disp[k].c[c] = disp[3 * n + c];
        if (vel) p.vel[k].c[c] = vel[3 * n + c];
        if (acc) p.acc[k].c[c] = acc[3 * n + c];
      }
    }
    for (uint32_t k = 0; k < p.n; ++k) p.cur[k] = vadd(p.pos[k], p.disp[k]);
    if (p.n) get_minmax(p.cur, p.lrtb);
  }
  return PD_OK;
}

// Connectivity of one particle replaced: conn2NArr + gen_xi (timeloop.h:285-291).
int or_set_connectivity(or_sim *S, uint32_t particle, const uint32_t *pairs, uint64_t n) {
  if (particle >= S->P.size()) return PD_EINVAL;
  Part &p = S->P[particle];
  p.nbr.assign(p.n, {});
  for (uint64_t l = 0; l < n; ++l) {
    const uint32_t i = pairs[2 * l], j = pairs[2 * l + 1];
    if (i >= p.n || j >= p.n) return PD_EINVAL;
    p.nbr[i].push_back(j);
    p.nbr[j].push_back(i);
  }
  gen_xi(p);
  return PD_OK;
}

void or_destroy(or_sim *S) { delete S; }

}  // extern "C"
