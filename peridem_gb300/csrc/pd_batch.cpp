// pd_batch.cpp -- batches of independent simulations in one engine, and the extern "C"
// entry points a serving loop uses on them.
//
// A batch concatenates the nodes, particles and bonds of S simulations in the layout of
// pd_engine.h; every phase of a step is one launch over all of them, and the per-node work
// looks up its simulation's constants (DevSimParams) and state (DevSimState). Nothing in a
// step couples two simulations: bonds stay inside a particle, contact candidates come from
// cells hashed with the simulation index, walls are per simulation. A simulation of a batch
// therefore computes exactly what it computes alone.
//
// Simulations of a batch may need different step counts. The host stops one with
// finish_sim() at a step boundary: its state is read back and kept on the host, and its
// `active` flag is cleared so the kernels skip its nodes from then on. The reference runs one
// simulation per process (run/simulate3d.cpp); none of this has a counterpart there.
#include <algorithm>
#include <cstddef>
#include <cstring>

#include "pd_engine.h"
#include "pd_sim.h"

#define PD_TRY(expr)              \
  do {                            \
    int _rc = (expr);             \
    if (_rc != PD_OK) return _rc; \
  } while (0)

namespace pdg {

namespace {
inline uint64_t up32(uint64_t x) { return (x + 31) / 32 * 32; }
inline uint64_t atleast1(uint64_t x) { return x ? x : 1; }
}  // namespace

// Mirrors every allocation of Engine::init (alloc_and_upload, upload_bonds,
// alloc_candidates) for the same setups, without touching the device.
uint64_t Engine::estimate_bytes(const std::vector<HostSim> &sims, int precision, uint32_t cand_cap, int64_t *bad) {
  uint64_t N = 0, P = 0, S = sims.size(), ncl = 0;
  for (auto &s : sims) {
    N += s.node_offset[s.np];
    P += s.np;
    ncl += s.clamped.size();
  }
  const uint64_t C = up32(N), nsl = C / 32;
  std::vector<uint32_t> file_of, node_of, deg_file;
  order_nodes(sims, file_of, node_of, deg_file, bad, nullptr, order_bin(precision));
  std::vector<uint32_t> deg(C, 0);
  for (uint64_t n = 0; n < N; ++n) deg[n] = deg_file[file_of[n]];
  uint64_t E = 0;
  for (uint64_t sl = 0; sl < nsl; ++sl) {
    uint32_t w = 0;
    for (int l = 0; l < 32; ++l) w = std::max(w, deg[sl * 32 + l]);
    E += 32ull * w;
  }
  uint64_t b = 0;
  // bonds
  b += (nsl + 1) * 8 + C * 2 + atleast1(E) * 4 + atleast1(E / 32) * 4;
  // node state, particles, simulations
  b += 7 * 3 * C * 8 + C * 8 + C * 4 + C;
  b += 2 * C * 4;  // node order maps
  b += P * sizeof(DevPart) + 6 * P * 8 * 2 + 3 * P * 8;
  b += S * sizeof(DevSimParams) + S * sizeof(DevSimState) + sizeof(DevCounters);
  if (ncl) b += (P + 1 + ncl) * 4 + 3 * ncl * 8;
  if (precision == PD_FP64) {
    b += 3 * atleast1(E) * 8 + 2 * atleast1(E) * 8;
  } else {
    b += 2 * C * 32 + 3 * C * 8 + 2 * 3 * P * 8 + C + 3 * C * 8 + C + 2 * 6 * P * 4;
    b += 2 * 4 * atleast1((N + kStageNodes - 1) / kStageNodes);  // staged-kernel record ranges
    b += C * 4 + atleast1(P) * 4 + 2 * 4;                          // non-bond work lists
  }
  // broad phase
  uint32_t bits = 10;
  while ((1ull << bits) < 2 * N) ++bits;
  const uint64_t T = 1ull << bits;
  b += 2 * T * 4 + 3 * C * 4 + ((T + 4095) / 4096 + 1) * 4;
  b += C * (cand_cap ? cand_cap : 32) * 4 + C * 2;
  return b;
}

int Engine::sim_range(uint32_t sim, uint64_t *node0, uint64_t *n_nodes, uint32_t *particle0,
                      uint32_t *n_particles) const {
  if (sim >= S_) return PD_EINVAL;
  if (node0) *node0 = sim_node0_[sim];
  if (n_nodes) *n_nodes = sim_node0_[sim + 1] - sim_node0_[sim];
  if (particle0) *particle0 = sim_p0_[sim];
  if (n_particles) *n_particles = sim_p0_[sim + 1] - sim_p0_[sim];
  return PD_OK;
}

// [3][Ncap] device array, engine nodes [node0, node0+nn) -> nn*3 row vectors in file order
// (a simulation's node range is the same in both numberings).
int Engine::read_nodes(const double *d, uint64_t node0, uint64_t nn, double *dst) {
  std::vector<double> buf(3 * nn);
  for (int c = 0; c < 3; ++c)
    PD_TRY(check(cudaMemcpyAsync(buf.data() + c * nn, d + c * Ncap_ + node0, nn * 8, cudaMemcpyDeviceToHost, stream_),
                 "read state"));
  PD_TRY(check(cudaStreamSynchronize(stream_), "read state"));
  rows_to_file(buf.data(), nn, node0, nn, dst);
  return PD_OK;
}

int Engine::get_sim_state(uint32_t sim, double *curpos, double *vel, double *acc, double *force, double *disp) {
  if (sim >= S_) {
    err = "simulation index out of range";
    return PD_EINVAL;
  }
  const uint64_t n0 = sim_node0_[sim], nn = sim_node0_[sim + 1] - n0;
  double *outs[5] = {curpos, vel, acc, force, disp};
  if (finished_[sim]) {
    for (int k = 0; k < 5; ++k)
      if (outs[k]) std::memcpy(outs[k], final_[sim].data() + k * 3 * nn, 3 * nn * 8);
    return PD_OK;
  }
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  const bool fused = precision_ == PD_FP32C;
  // clamped nodes of this simulation (h_clamped_ lists them particle by particle)
  std::vector<uint64_t> cl;
  for (uint64_t i = 0; i < h_clamped_.size(); ++i)
    if (h_clamped_[i] >= n0 && h_clamped_[i] < n0 + nn) cl.push_back(i);
  if (curpos || disp) {
    std::vector<double> dsp(3 * nn);
    PD_TRY(read_nodes(fused ? d_dispb_[cur_ ^ 1] : d_disp_, n0, nn, dsp.data()));
    if (disp) {
      std::memcpy(disp, dsp.data(), 3 * nn * 8);
      if (fused && sim_steps_[sim] > 0)  // clamped nodes end each step at zero (timeloop.h:767-774)
        for (uint64_t i : cl)
          for (int c = 0; c < 3; ++c) disp[3 * (h_clamped_[i] - n0) + c] = 0.0;
    }
    if (curpos) {
      if (!cl.empty() && sim_steps_[sim] > 0 && !fused) {
        // CurrPos of clamped nodes keeps the predicted displacement (zeroed afterwards)
        std::vector<double> cd(3 * n_clamped_);
        PD_TRY(cpy(cd.data(), d_clamped_disp_, cd.size() * 8, "read clamped"));
        for (uint64_t i : cl)
          for (int c = 0; c < 3; ++c) dsp[3 * (h_clamped_[i] - n0) + c] = cd[3 * i + c];
      }
      if (reset_possible_) {  // reset_partzero_y moves reference positions on the device
        std::vector<double> p(3 * nn);
        PD_TRY(read_nodes(d_pos_, n0, nn, p.data()));
        for (uint64_t k = 0; k < 3 * nn; ++k) curpos[k] = p[k] + dsp[k];
      } else {
        const HostSim &s = sims_[sim];
        for (uint64_t k = 0; k < 3 * nn; ++k) curpos[k] = s.pos[k] + dsp[k];
      }
    }
  }
  if (vel) PD_TRY(read_nodes(d_vel_[cur_], n0, nn, vel));
  if (acc) PD_TRY(read_nodes(d_acc_, n0, nn, acc));
  if (force) PD_TRY(read_nodes(d_force_, n0, nn, force));
  return PD_OK;
}

int Engine::finish_sim(uint32_t sim) {
  if (sim >= S_) {
    err = "simulation index out of range";
    return PD_EINVAL;
  }
  if (finished_[sim]) return PD_OK;
  const uint64_t nn = sim_node0_[sim + 1] - sim_node0_[sim];
  std::vector<double> keep(15 * nn + 24);
  PD_TRY(get_sim_state(sim, keep.data(), keep.data() + 3 * nn, keep.data() + 6 * nn, keep.data() + 9 * nn,
                       keep.data() + 12 * nn));
  PD_TRY(get_wall(sim, keep.data() + 15 * nn, keep.data() + 15 * nn + 6));
  const int32_t off = 0;
  PD_TRY(cpy((char *)(d_ss_ + sim) + offsetof(DevSimState, active), &off, sizeof(off), "deactivate"));
  final_[sim].swap(keep);
  finished_[sim] = 1;
  return PD_OK;
}

// ---- per-simulation checkpoints (eviction and re-admission) ----------------------------
//
// A simulation's nodes occupy one contiguous engine range whose internal order depends only on
// its own setup (order_nodes sorts inside each particle), and its particles one contiguous
// range; so the simulation's slices of every per-node and per-particle array are copied as
// they are. What depends on the handle -- global node indices in the bond columns and the
// SELL slices' live masks, the contact lists, the cell list, the work lists -- is not copied:
// the live bonds travel as each particle's Connectivity and the rest is rebuilt by the next
// step. The FP32 form's two displacement buffers, records and velocity buffer are saved by
// role (completed step, predicted next step), since the two handles' buffer parity may differ.
namespace {
constexpr uint32_t kCkptMagic = 0x4B434450u;  // "PDCK"
constexpr uint32_t kCkptVersion = 1;

struct CkptHeader {
  uint32_t magic, version;
  int32_t precision, flags;  // flags: 1 pos saved (reset_partzero_y), 2 afd saved, 4 clamped disp
  uint64_t nn, np, ncl, steps;
  DevSimParams sp;           // the target's constants must be equal (layout fields zeroed)
};

// Mutable fields of a particle (toggles, the moving reference frame and the breaking band).
struct CkptPart {
  int32_t movable, breakable, stoppable, break_bonds;
  double anchor_pos[3];
  float snot_lo32, snot_hi32;
  uint64_t n_nodes, n_pairs;  // the particle's size and its live pairs that follow the fixed part
};

struct Writer {
  std::vector<uint8_t> &b;
  void put(const void *p, size_t n) {
    const uint8_t *c = static_cast<const uint8_t *>(p);
    b.insert(b.end(), c, c + n);
  }
};
struct Reader {
  const uint8_t *p;
  uint64_t n, off = 0;
  bool get(void *dst, size_t k) {
    if (off + k > n) return false;
    std::memcpy(dst, p + off, k);
    off += k;
    return true;
  }
};

// The simulation's constants without what depends on the handle: its place in the layout and
// the broad phase's cell size (the contact skin, which does not change results).
DevSimParams layout_free(DevSimParams sp) {
  sp.p0 = 0;
  sp.np = 0;
  sp.node0 = 0;
  sp.nnodes = 0;
  sp.cell = 0;
  sp.inv_cell = 0;
  sp.cand_r2 = 0;
  return sp;
}

// Optional sections, from the simulation's own config: 1 reference positions (reset_partzero_y
// moves them), 2 applied_force_density (a prescribed-velocity particle), 4 the FP64 form's
// predicted displacement of clamped nodes.
int ckpt_flags(const DevSimParams &sp, bool fused, uint64_t ncl) {
  return (sp.reset_y ? 1 : 0) | (sp.pv_particle >= 0 ? 2 : 0) | (!fused && ncl ? 4 : 0);
}
}  // namespace

int Engine::save_sim(uint32_t sim, std::vector<uint8_t> &out) {
  if (sim >= S_) {
    err = "simulation index out of range";
    return PD_EINVAL;
  }
  if (finished_[sim]) {
    err = "simulation " + std::to_string(sim) + " is finished: its device state is gone";
    return PD_ESTATE;
  }
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  const uint64_t n0 = sim_node0_[sim], nn = sim_node0_[sim + 1] - n0;
  const uint32_t p0 = sim_p0_[sim], np = sim_p0_[sim + 1] - p0;
  const bool fused = precision_ == PD_FP32C;
  uint64_t c0 = 0, ncl = 0;  // the simulation's entries of the clamped list
  for (uint64_t i = 0; i < h_clamped_.size(); ++i)
    if (h_clamped_[i] >= n0 && h_clamped_[i] < n0 + nn) {
      if (!ncl) c0 = i;
      ++ncl;
    }
  CkptHeader h;
  std::memset(&h, 0, sizeof(h));
  h.magic = kCkptMagic;
  h.version = kCkptVersion;
  h.precision = precision_;
  h.nn = nn;
  h.np = np;
  h.ncl = ncl;
  h.steps = sim_steps_[sim];
  PD_TRY(cpy(&h.sp, d_sp_ + sim, sizeof(DevSimParams), "read params"));
  h.flags = ckpt_flags(h.sp, fused, ncl);
  h.sp = layout_free(h.sp);
  out.clear();
  Writer w{out};
  w.put(&h, sizeof(h));
  std::vector<double> buf(3 * nn);
  auto node3 = [&](const double *d) -> int {  // [3][Ncap] slice, engine order
    for (int c = 0; c < 3; ++c)
      PD_TRY(check(cudaMemcpyAsync(buf.data() + c * nn, d + c * Ncap_ + n0, nn * 8, cudaMemcpyDeviceToHost, stream_),
                   "save"));
    PD_TRY(check(cudaStreamSynchronize(stream_), "save"));
    w.put(buf.data(), 3 * nn * 8);
    return PD_OK;
  };
  PD_TRY(node3(fused ? d_dispb_[cur_ ^ 1] : d_disp_));  // the completed step
  if (fused) PD_TRY(node3(d_dispb_[cur_]));              // the next step's prediction
  PD_TRY(node3(d_vel_[cur_]));
  PD_TRY(node3(d_acc_));
  PD_TRY(node3(d_force_));
  if (h.flags & 1) PD_TRY(node3(d_pos_));
  if (h.flags & 2) PD_TRY(node3(d_afd_));
  if (fused) {
    std::vector<Rec32> r(nn);
    PD_TRY(cpy(r.data(), d_rec_[cur_] + n0, nn * sizeof(Rec32), "save records"));
    w.put(r.data(), nn * sizeof(Rec32));
  }
  std::vector<DevPart> parts(np);
  PD_TRY(cpy(parts.data(), d_parts_ + p0, np * sizeof(DevPart), "save particles"));
  std::vector<double> lrtb(6 * np);
  PD_TRY(cpy(lrtb.data(), d_lrtb_ + 6ull * p0, 6 * np * 8, "save boxes"));
  w.put(lrtb.data(), 6 * np * 8);
  if (fused) {
    std::vector<double> an(3 * np), ann(3 * np);
    std::vector<float> wl(6 * np);
    PD_TRY(cpy(an.data(), d_anchor_ + 3ull * p0, 3 * np * 8, "save anchors"));
    PD_TRY(cpy(ann.data(), d_anchor_next_ + 3ull * p0, 3 * np * 8, "save anchors"));
    PD_TRY(cpy(wl.data(), d_wall_local_ + 6ull * p0, 6 * np * 4, "save walls"));
    w.put(an.data(), 3 * np * 8);
    w.put(ann.data(), 3 * np * 8);
    w.put(wl.data(), 6 * np * 4);
  }
  DevSimState ss;
  PD_TRY(cpy(&ss, d_ss_ + sim, sizeof(ss), "save sim state"));
  w.put(&ss, sizeof(ss));
  if (h.flags & 4) {
    std::vector<double> cd(3 * ncl);
    PD_TRY(cpy(cd.data(), d_clamped_disp_ + 3 * c0, 3 * ncl * 8, "save clamped"));
    w.put(cd.data(), 3 * ncl * 8);
  }
  std::vector<uint32_t> pairs;
  for (uint32_t k = 0; k < np; ++k) {
    uint64_t npairs = 0;
    PD_TRY(get_connectivity(p0 + k, nullptr, 0, &npairs));
    pairs.resize(2 * std::max<uint64_t>(npairs, 1));
    PD_TRY(get_connectivity(p0 + k, pairs.data(), npairs, &npairs));
    const DevPart &P = parts[k];
    CkptPart cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.movable = P.movable;
    cp.breakable = P.breakable;
    cp.stoppable = P.stoppable;
    cp.break_bonds = P.break_bonds;
    for (int c = 0; c < 3; ++c) cp.anchor_pos[c] = P.anchor_pos[c];
    cp.snot_lo32 = P.snot_lo32;
    cp.snot_hi32 = P.snot_hi32;
    cp.n_nodes = P.n;
    cp.n_pairs = npairs;
    w.put(&cp, sizeof(cp));
    w.put(pairs.data(), 2 * npairs * 4);
  }
  return PD_OK;
}

int Engine::load_sim(uint32_t sim, const uint8_t *buf, uint64_t n) {
  if (sim >= S_) {
    err = "simulation index out of range";
    return PD_EINVAL;
  }
  Reader r{buf, n};
  CkptHeader h;
  if (!r.get(&h, sizeof(h)) || h.magic != kCkptMagic || h.version != kCkptVersion) {
    err = "not a simulation checkpoint of this library";
    return PD_EINVAL;
  }
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  const uint64_t n0 = sim_node0_[sim], nn = sim_node0_[sim + 1] - n0;
  const uint32_t p0 = sim_p0_[sim], np = sim_p0_[sim + 1] - p0;
  const bool fused = precision_ == PD_FP32C;
  uint64_t c0 = 0, ncl = 0;
  for (uint64_t i = 0; i < h_clamped_.size(); ++i)
    if (h_clamped_[i] >= n0 && h_clamped_[i] < n0 + nn) {
      if (!ncl) c0 = i;
      ++ncl;
    }
  DevSimParams sp;
  PD_TRY(cpy(&sp, d_sp_ + sim, sizeof(sp), "read params"));
  const int flags = ckpt_flags(sp, fused, ncl);
  sp = layout_free(sp);
  if (h.precision != precision_ || h.nn != nn || h.np != np || h.ncl != ncl || h.flags != flags ||
      std::memcmp(&sp, &h.sp, sizeof(sp)) != 0) {
    err = "checkpoint of another setup, config or precision form than simulation " + std::to_string(sim);
    return PD_EINVAL;
  }
  std::vector<double> nodebuf(3 * nn);
  auto node3 = [&](double *d) -> int {
    if (!r.get(nodebuf.data(), 3 * nn * 8)) return PD_EINVAL;
    for (int c = 0; c < 3; ++c)
      PD_TRY(check(cudaMemcpyAsync(d + c * Ncap_ + n0, nodebuf.data() + c * nn, nn * 8, cudaMemcpyHostToDevice,
                                   stream_), "load"));
    return check(cudaStreamSynchronize(stream_), "load");
  };
  auto take = [&](void *dst_dev, size_t bytes, const char *what) -> int {
    std::vector<uint8_t> tmp(bytes);
    if (!r.get(tmp.data(), bytes)) return PD_EINVAL;
    return cpy(dst_dev, tmp.data(), bytes, what);
  };
  int rc = PD_OK;
  auto bad = [&]() {
    err = "truncated or corrupt simulation checkpoint";
    return PD_EINVAL;
  };
  if ((rc = node3(fused ? d_dispb_[cur_ ^ 1] : d_disp_)) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  if (fused && (rc = node3(d_dispb_[cur_])) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  if ((rc = node3(d_vel_[cur_])) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  if ((rc = node3(d_acc_)) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  if ((rc = node3(d_force_)) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  if ((h.flags & 1) && (rc = node3(d_pos_)) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  if ((h.flags & 2) && (rc = node3(d_afd_)) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  if (fused && (rc = take(d_rec_[cur_] + n0, nn * sizeof(Rec32), "load records")) != PD_OK)
    return rc == PD_EINVAL ? bad() : rc;
  if ((rc = take(d_lrtb_ + 6ull * p0, 6 * np * 8, "load boxes")) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  if (fused) {
    if ((rc = take(d_anchor_ + 3ull * p0, 3 * np * 8, "load anchors")) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
    if ((rc = take(d_anchor_next_ + 3ull * p0, 3 * np * 8, "load anchors")) != PD_OK)
      return rc == PD_EINVAL ? bad() : rc;
    if ((rc = take(d_wall_local_ + 6ull * p0, 6 * np * 4, "load walls")) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  }
  if ((rc = take(d_ss_ + sim, sizeof(DevSimState), "load sim state")) != PD_OK) return rc == PD_EINVAL ? bad() : rc;
  if ((h.flags & 4) && (rc = take(d_clamped_disp_ + 3 * c0, 3 * ncl * 8, "load clamped")) != PD_OK)
    return rc == PD_EINVAL ? bad() : rc;
  std::vector<DevPart> parts(np);
  PD_TRY(cpy(parts.data(), d_parts_ + p0, np * sizeof(DevPart), "read particles"));
  std::vector<uint32_t> pairs;
  for (uint32_t k = 0; k < np; ++k) {
    CkptPart cp;
    if (!r.get(&cp, sizeof(cp)) || cp.n_nodes != parts[k].n) return bad();
    pairs.resize(2 * std::max<uint64_t>(cp.n_pairs, 1));
    if (!r.get(pairs.data(), 2 * cp.n_pairs * 4)) return bad();
    DevPart &P = parts[k];
    P.movable = cp.movable;
    P.breakable = cp.breakable;
    P.stoppable = cp.stoppable;
    P.break_bonds = cp.break_bonds;
    for (int c = 0; c < 3; ++c) P.anchor_pos[c] = cp.anchor_pos[c];
    P.snot_lo32 = cp.snot_lo32;
    P.snot_hi32 = cp.snot_hi32;
    PD_TRY(set_connectivity(p0 + k, pairs.data(), cp.n_pairs));
  }
  PD_TRY(cpy(d_parts_ + p0, parts.data(), np * sizeof(DevPart), "load particles"));
  // contact lists, cell list and work lists follow from the loaded positions at the next step
  const double big = 1e300;
  PD_TRY(cpy(&d_cnt_->moved, &big, 8, "force rebuild"));
  if (fused) {
    const uint32_t one = 1;
    PD_TRY(cpy(&d_cnt_->xall, &one, 4, "work lists"));
  }
  sim_steps_[sim] = h.steps;
  finished_[sim] = 0;
  final_[sim].clear();
  return PD_OK;
}

}  // namespace pdg

namespace {
int fail(int rc, const std::string &m) { return pdg::set_global_error(rc, m); }
}  // namespace

extern "C" {

int pd_create_batch(const pd_setup_arrays *setups, const pd_config *cfgs, uint32_t n_sims, int precision,
                    pd_sim **out) {
  if (!out) return fail(PD_EINVAL, "null output handle");
  *out = nullptr;
  if (!setups || !cfgs || n_sims == 0) return fail(PD_EINVAL, "empty batch");
  if (precision != PD_FP64 && precision != PD_FP32C) return fail(PD_EINVAL, "unknown precision form");
  std::vector<pdg::HostSim> sims(n_sims);
  for (uint32_t i = 0; i < n_sims; ++i) {
    std::string err;
    int rc = pdg::host_sim_from_arrays(&setups[i], &cfgs[i], sims[i], err);
    if (rc != PD_OK) return fail(rc, "simulation " + std::to_string(i) + ": " + err);
  }
  pd_sim *s = new pd_sim();
  s->cfg = cfgs[0];
  int rc = s->eng.init(sims, precision);
  if (rc != PD_OK) {
    std::string e = s->eng.err;
    delete s;
    return fail(rc, e);
  }
  *out = s;
  return PD_OK;
}

int pd_estimate_bytes(const pd_setup_arrays *setups, uint32_t n_sims, int precision, uint64_t *bytes) {
  if (!setups || !bytes || n_sims == 0) return fail(PD_EINVAL, "null argument");
  std::vector<pdg::HostSim> sims(n_sims);
  pd_config cfg;
  pd_config_default(&cfg);
  for (uint32_t i = 0; i < n_sims; ++i) {
    std::string err;
    int rc = pdg::host_sim_from_arrays(&setups[i], &cfg, sims[i], err);
    if (rc != PD_OK) return fail(rc, "simulation " + std::to_string(i) + ": " + err);
  }
  int64_t bad = -1;
  const uint64_t b = pdg::Engine::estimate_bytes(sims, precision, 0, &bad);
  if (bad >= 0) return fail(PD_EINVAL, "Connectivity index out of range in particle " + std::to_string(bad));
  *bytes = b;
  return PD_OK;
}

int pd_device_bytes(const pd_sim *s, uint64_t *bytes) {
  if (!s || !bytes) return fail(PD_EINVAL, "null argument");
  *bytes = s->eng.device_bytes();
  return PD_OK;
}

int pd_device_memory(uint64_t *free_bytes, uint64_t *total_bytes) {
  size_t f = 0, t = 0;
  cudaError_t e = cudaMemGetInfo(&f, &t);
  if (e != cudaSuccess) return fail(PD_ECUDA, std::string("cudaMemGetInfo: ") + cudaGetErrorString(e));
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return PD_OK;
}

int pd_num_sims(const pd_sim *s, uint32_t *n) {
  if (!s || !n) return fail(PD_EINVAL, "null argument");
  *n = s->eng.num_sims();
  return PD_OK;
}

int pd_sim_range(const pd_sim *s, uint32_t sim, uint64_t *node0, uint64_t *n_nodes, uint32_t *particle0,
                 uint32_t *n_particles) {
  if (!s) return fail(PD_EINVAL, "null handle");
  int rc = s->eng.sim_range(sim, node0, n_nodes, particle0, n_particles);
  return rc == PD_OK ? rc : fail(rc, "simulation index out of range");
}

int pd_sim_steps(const pd_sim *s, uint32_t sim, uint64_t *steps) {
  if (!s || !steps) return fail(PD_EINVAL, "null argument");
  if (sim >= s->eng.num_sims()) return fail(PD_EINVAL, "simulation index out of range");
  *steps = s->eng.sim_steps(sim);
  return PD_OK;
}

int pd_finish_sim(pd_sim *s, uint32_t sim) {
  if (!s) return fail(PD_EINVAL, "null handle");
  return s->eng.finish_sim(sim);
}

int pd_get_sim_state(pd_sim *s, uint32_t sim, double *curpos, double *vel, double *acc, double *force) {
  if (!s) return fail(PD_EINVAL, "null handle");
  return s->eng.get_sim_state(sim, curpos, vel, acc, force, nullptr);
}

int pd_get_sim_disp(pd_sim *s, uint32_t sim, double *disp) {
  if (!s) return fail(PD_EINVAL, "null handle");
  return s->eng.get_sim_state(sim, nullptr, nullptr, nullptr, nullptr, disp);
}

int pd_get_sim_damage(pd_sim *s, uint32_t sim, double *damage) {
  if (!s || !damage) return fail(PD_EINVAL, "null argument");
  uint64_t n0 = 0, nn = 0;
  uint32_t p0 = 0, np = 0;
  if (s->eng.sim_range(sim, &n0, &nn, &p0, &np) != PD_OK) return fail(PD_EINVAL, "simulation index out of range");
  return s->eng.get_damage(damage, n0, nn);
}

int pd_save_sim(pd_sim *s, uint32_t sim, void *buf, uint64_t cap, uint64_t *bytes) {
  if (!s || !bytes) return fail(PD_EINVAL, "null argument");
  std::vector<uint8_t> out;
  int rc = s->eng.save_sim(sim, out);
  if (rc != PD_OK) return fail(rc, s->eng.err);
  *bytes = out.size();
  if (!buf) return PD_OK;
  if (cap < out.size()) return fail(PD_EINVAL, "checkpoint buffer too small");
  std::memcpy(buf, out.data(), out.size());
  return PD_OK;
}

int pd_load_sim(pd_sim *s, uint32_t sim, const void *buf, uint64_t bytes) {
  if (!s || !buf) return fail(PD_EINVAL, "null argument");
  int rc = s->eng.load_sim(sim, static_cast<const uint8_t *>(buf), bytes);
  return rc == PD_OK ? rc : fail(rc, s->eng.err);
}

int pd_get_sim_wall(pd_sim *s, uint32_t sim, double *wall_info, double *reaction) {
  if (!s) return fail(PD_EINVAL, "null handle");
  if (sim >= s->eng.num_sims()) return fail(PD_EINVAL, "simulation index out of range");
  return s->eng.get_wall(sim, wall_info, reaction);
}

}  // extern "C"
