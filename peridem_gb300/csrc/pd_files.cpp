// pd_files.cpp -- the file boundary: setup.h5 in (load_particles/load_contact/load_wall,
// src/read/load_hdf5.h:41-181), plotinfo.h5 / tc_%05u.h5 / wall_%05u.h5 / run_time.h5 out
// (src/particle/timeloop.h:321-350, 801-964), the resume path (timeloop.h:262-312), the
// whole time loop with saves and the progress table (timeloop.h:352-369, 909-947), plus a
// small C API over h5lite so that scripts can write setup files and read frames.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <deque>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>

#include "h5lite.h"
#include "pd_sim.h"

namespace {

thread_local std::string g_ferr;

int fail(int rc, const std::string &m) {
  g_ferr = m;
  return rc;
}

std::string pnum(unsigned p) {
  char b[32];
  std::snprintf(b, sizeof(b), "P_%05u", p);
  return b;
}

bool read_col_f64(const h5lite::Reader &r, const std::string &path, std::vector<double> &v, std::string &err) {
  std::vector<uint64_t> dims;
  return r.read_vec<double>(path, h5lite::F64, v, dims, err);
}

template <typename T>
bool read_any(const h5lite::Reader &r, const std::string &path, int dt, std::vector<T> &v, std::string &err) {
  std::vector<uint64_t> dims;
  return r.read_vec<T>(path, dt, v, dims, err);
}

// load_particles<3> + load_contact + load_wall<3> (load_hdf5.h:41-181)
int load_setup(const std::string &fn, pdg::HostSim &hs, std::string &err) {
  h5lite::Reader r;
  if (!r.open(fn, err)) return PD_EIO;
  std::vector<uint32_t> tp;
  if (!read_any<uint32_t>(r, "total_particles_univ", h5lite::U32, tp, err) || tp.empty()) return PD_EIO;
  const uint32_t np = tp[0];
  hs.np = np;
  hs.node_offset.assign(1, 0);
  hs.conn_offset.assign(1, 0);
  hs.bdry_offset.assign(1, 0);
  hs.clamped_offset.assign(1, 0);
  for (uint32_t p = 0; p < np; ++p) {
    const std::string g = pnum(p) + "/";
    std::vector<double> pos, vol, disp, vel, acc, ext, sc;
    std::vector<uint64_t> dims;
    if (!r.read_vec<double>(g + "Pos", h5lite::F64, pos, dims, err)) return PD_EIO;
    if (dims.size() != 2 || dims[1] != 3) {
      err = g + "Pos is not an (N,3) array";
      return PD_EIO;
    }
    const uint64_t n = dims[0];
    if (!read_col_f64(r, g + "Vol", vol, err) || vol.size() != n) {
      if (err.empty()) err = g + "Vol size mismatch";
      return PD_EIO;
    }
    for (const char *k : {"disp", "vel", "acc", "extforce"}) {
      std::vector<double> *dst = (std::strcmp(k, "disp") == 0) ? &disp
                                 : (std::strcmp(k, "vel") == 0) ? &vel
                                 : (std::strcmp(k, "acc") == 0) ? &acc : &ext;
      if (!r.read_vec<double>(g + k, h5lite::F64, *dst, dims, err)) return PD_EIO;
      if (dst->size() != 3 * n) {
        err = g + k + " size mismatch";
        return PD_EIO;
      }
    }
    std::vector<uint32_t> conn, bdry, clamped;
    if (!r.read_vec<uint32_t>(g + "Connectivity", h5lite::U32, conn, dims, err)) return PD_EIO;
    if (!conn.empty() && (dims.size() != 2 || dims[1] != 2)) {
      err = g + "Connectivity is not an (M,2) array";
      return PD_EIO;
    }
    if (r.has(g + "bdry_nodes") && !r.read_vec<uint32_t>(g + "bdry_nodes", h5lite::U32, bdry, dims, err)) return PD_EIO;
    if (r.has(g + "clamped_nodes") && !r.read_vec<uint32_t>(g + "clamped_nodes", h5lite::U32, clamped, dims, err))
      return PD_EIO;
    auto scalar = [&](const char *k, double &out) -> bool {
      std::vector<double> v;
      if (!read_col_f64(r, g + k, v, err) || v.empty()) {
        if (err.empty()) err = g + k + " is empty";
        return false;
      }
      out = v[0];
      return true;
    };
    double delta, rho, cnot, snot, tval = 0, mov = 1, brk = 1, stp = 1, tax = 2;
    if (!scalar("delta", delta) || !scalar("rho", rho) || !scalar("cnot", cnot) || !scalar("snot", snot) ||
        !scalar("movable", mov) || !scalar("breakable", brk) || !scalar("stoppable", stp) ||
        !scalar("torque_axis", tax) || !scalar("torque_val", tval))
      return PD_EIO;
    hs.pos.insert(hs.pos.end(), pos.begin(), pos.end());
    hs.vol.own.insert(hs.vol.own.end(), vol.begin(), vol.end());
    hs.disp.own.insert(hs.disp.own.end(), disp.begin(), disp.end());
    hs.vel.own.insert(hs.vel.own.end(), vel.begin(), vel.end());
    hs.acc.own.insert(hs.acc.own.end(), acc.begin(), acc.end());
    hs.ext.own.insert(hs.ext.own.end(), ext.begin(), ext.end());
    hs.conn.own.insert(hs.conn.own.end(), conn.begin(), conn.end());
    hs.bdry.insert(hs.bdry.end(), bdry.begin(), bdry.end());
    hs.clamped.insert(hs.clamped.end(), clamped.begin(), clamped.end());
    hs.node_offset.push_back(hs.node_offset.back() + n);
    hs.conn_offset.push_back(hs.conn_offset.back() + conn.size() / 2);
    hs.bdry_offset.push_back(hs.bdry_offset.back() + bdry.size());
    hs.clamped_offset.push_back(hs.clamped_offset.back() + clamped.size());
    hs.delta.push_back(delta);
    hs.rho.push_back(rho);
    hs.cnot.push_back(cnot);
    hs.snot.push_back(snot);
    hs.tval.push_back(tval);
    hs.movable.push_back((int32_t)mov);
    hs.breakable.push_back((int32_t)brk);
    hs.stoppable.push_back((int32_t)stp);
    hs.taxis.push_back((uint32_t)tax);
  }
  std::vector<double> v;
  if (!read_col_f64(r, "pairwise/contact_radius", v, err) || v.empty()) return PD_EIO;
  hs.Rc = v[0];
  if (!read_col_f64(r, "pairwise/normal_stiffness", v, err) || v.empty()) return PD_EIO;
  hs.Kn = v[0];
  if (!read_col_f64(r, "pairwise/friction_coefficient", v, err) || v.empty()) return PD_EIO;
  hs.mu = v[0];
  if (!read_col_f64(r, "pairwise/damping_ratio", v, err) || v.empty()) return PD_EIO;
  hs.zeta = v[0];
  std::vector<uint32_t> aw;
  if (!read_any<uint32_t>(r, "wall/allow_wall", h5lite::U32, aw, err) || aw.empty()) return PD_EIO;
  hs.allow_wall = aw[0] != 0;
  if (!read_col_f64(r, "wall/geom_wall_info", v, err)) return PD_EIO;
  hs.n_geom_wall = (int32_t)v.size();
  if (v.size() != 1) {
    if (v.size() < 6) {
      err = "wall/geom_wall_info has " + std::to_string(v.size()) + " entries (3D needs 6)";
      return PD_EIO;
    }
    for (int k = 0; k < 6; ++k) hs.geom[k] = v[k];
  }
  return PD_OK;
}

bool is_dir(const std::string &p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

std::string format_ms(int ms) {
  int s = ms / 1000, mi = s / 60, rs = s % 60, hr = mi / 60, rm = mi % 60;
  std::stringstream ss;
  ss << hr << ":" << std::setfill('0') << std::setw(2) << rm << ":" << std::setfill('0') << std::setw(2) << rs;
  return ss.str();
}

}  // namespace

extern "C" {

const char *pd_files_error(void) { return g_ferr.c_str(); }

int pd_open(const char *conf, const char *setup_h5, const char *outdir, int precision, pd_sim **out) {
  if (!out) return fail(PD_EINVAL, "null output handle");
  *out = nullptr;
  pd_config cfg;
  pd_config_default(&cfg);
  if (setup_h5) std::strncpy(cfg.setup_filename, setup_h5, sizeof(cfg.setup_filename) - 1);
  if (outdir) std::strncpy(cfg.output_dir, outdir, sizeof(cfg.output_dir) - 1);
  if (conf) {
    int rc = pd_config_read(conf, &cfg);
    if (rc != PD_OK && rc != PD_ECONFIG) return fail(rc, "config read failed");
    if (rc == PD_ECONFIG) {
      // the reference carries on with defaults when the file cannot be opened
      std::ifstream probe(conf);
      if (probe.good()) return fail(PD_ECONFIG, std::string("bad value in config file ") + conf);
    }
  }
  std::vector<pdg::HostSim> sims(1);
  std::string err;
  int rc = load_setup(cfg.setup_filename, sims[0], err);
  if (rc != PD_OK) return fail(rc, "setup: " + err);
  sims[0].cfg = cfg;
  pd_sim *s = new pd_sim();
  s->cfg = cfg;
  s->outdir = cfg.output_dir;
  rc = s->eng.init(sims, precision);
  if (rc != PD_OK) {
    std::string e = s->eng.err;
    delete s;
    return fail(rc, e);
  }
  *out = s;
  return PD_OK;
}

}  // extern "C"

namespace {

// tc_%05u.h5 and wall_%05u.h5 of one frame from host arrays (timeloop.h:801-953).
int write_frame_files(pd_sim *s, uint32_t counter, const double *cur, const double *vel, const double *acc,
                      const double *force, const double *afd,
                      const std::function<int(uint32_t, std::vector<uint32_t> &)> &conn, const double *wall,
                      const double *react) {
  const uint32_t P = s->eng.num_particles();
  const auto &hs = s->eng.sims()[0];
  const int32_t pvp = s->cfg.particle_w_fixed_velocity;
  h5lite::Writer w;
  std::vector<uint32_t> pairs;
  for (uint32_t p = 0; p < P; ++p) {
    const uint64_t a = hs.node_offset[p], n = hs.node_offset[p + 1] - a;
    const std::string g = pnum(p) + "/";
    w.add(g + "CurrPos", h5lite::F64, {n, 3}, cur + 3 * a);
    w.add(g + "vel", h5lite::F64, {n, 3}, vel + 3 * a);
    w.add(g + "acc", h5lite::F64, {n, 3}, acc + 3 * a);
    w.add(g + "force", h5lite::F64, {n, 3}, force + 3 * a);
    // applied_force_density of the prescribed-velocity particle (timeloop.h:844-848)
    if (afd && pvp >= 0 && p == (uint32_t)pvp) w.add(g + "applied_force_density", h5lite::F64, {n, 3}, afd + 3 * a);
    int rc = conn(p, pairs);
    if (rc != PD_OK) return rc;
    w.add(g + "Connectivity", h5lite::U32, {pairs.size() / 2, 2}, pairs.data());
  }
  char buf[64];
  std::snprintf(buf, sizeof(buf), "/tc_%05u.h5", counter);
  std::string err;
  if (!w.write(s->outdir + buf, err)) return fail(PD_EIO, err);
  h5lite::Writer ww;
  ww.add("wall_info", h5lite::F64, {6, 1}, wall);
  if (s->cfg.compute_wall_reaction) ww.add("reaction", h5lite::F64, {6, 3}, react);
  std::snprintf(buf, sizeof(buf), "/wall_%05u.h5", counter);
  if (!ww.write(s->outdir + buf, err)) return fail(PD_EIO, err);
  return PD_OK;
}

// Frames of pd_run off the critical path: the main thread stages a frame (copies enqueued on
// the engine's stream, pinned destination) and goes on stepping; this thread waits for the
// copies, builds the arrays of the frame on the host and writes the files. Two staging slots.
class FrameWriter {
 public:
  using Done = std::function<void(uint32_t counter, uint32_t t, const pdg::HostFrame &)>;
  FrameWriter(pd_sim *s, Done done) : s_(s), done_(std::move(done)) {}
  ~FrameWriter() { finish(); }

  int start(int nslots) {
    slots_.resize(nslots);
    for (auto &f : slots_) {
      int rc = s_->eng.frame_alloc(f);
      if (rc != PD_OK) return fail(rc, s_->eng.err);
      free_.push_back(&f);
    }
    th_ = std::thread([this] { run(); });
    return PD_OK;
  }

  // Main thread: stage the engine's current state as frame `counter` (after step t).
  int submit(uint32_t counter, uint32_t t) {
    pdg::HostFrame *f = nullptr;
    {
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] { return !free_.empty() || rc_ != PD_OK; });
      if (rc_ != PD_OK) return rc_;
      f = free_.front();
      free_.pop_front();
    }
    int rc = s_->eng.frame_stage(*f);
    if (rc != PD_OK) return fail(rc, s_->eng.err);
    {
      std::lock_guard<std::mutex> lk(m_);
      jobs_.push_back({f, counter, t});
    }
    cv_.notify_all();
    return PD_OK;
  }

  // Waits for every staged frame to be written; returns the first error.
  int finish() {
    if (th_.joinable()) {
      {
        std::lock_guard<std::mutex> lk(m_);
        stop_ = true;
      }
      cv_.notify_all();
      th_.join();
    }
    for (auto &f : slots_) s_->eng.frame_free(f);
    slots_.clear();
    return rc_;
  }

 private:
  struct Job {
    pdg::HostFrame *f;
    uint32_t counter, t;
  };

  void run() {
    const uint64_t N = s_->eng.num_nodes();
    std::vector<double> cur(3 * N), vel(3 * N), acc(3 * N), force(3 * N), afd;
    for (;;) {
      Job j;
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return !jobs_.empty() || stop_; });
        if (jobs_.empty()) return;
        j = jobs_.front();
        jobs_.pop_front();
      }
      int rc = PD_OK;
      if (cudaEventSynchronize(j.f->done) != cudaSuccess) rc = fail(PD_ECUDA, "staged frame copy failed");
      if (rc == PD_OK && j.f->cnt->err)  // the device error word (non-finite force, list overflow)
        rc = fail(PD_EDEVICE, "device error word " + std::to_string(j.f->cnt->err) + " at step " + std::to_string(j.t));
      if (rc == PD_OK) {
        const pdg::HostFrame &f = *j.f;
        if (f.afd) afd.resize(3 * N);
        s_->eng.frame_state(f, cur.data(), vel.data(), acc.data(), force.data(), f.afd ? afd.data() : nullptr);
        double wall[6], react[18];
        s_->eng.frame_wall(f, 0, wall, react);
        rc = write_frame_files(
            s_, j.counter, cur.data(), vel.data(), acc.data(), force.data(), f.afd ? afd.data() : nullptr,
            [&](uint32_t p, std::vector<uint32_t> &pairs) {
              s_->eng.frame_connectivity(f, p, pairs);
              return PD_OK;
            },
            wall, react);
        if (rc == PD_OK) done_(j.counter, j.t, f);
      }
      {
        std::lock_guard<std::mutex> lk(m_);
        if (rc != PD_OK && rc_ == PD_OK) rc_ = rc;
        free_.push_back(j.f);
      }
      cv_.notify_all();
    }
  }

  pd_sim *s_;
  Done done_;
  std::vector<pdg::HostFrame> slots_;
  std::deque<pdg::HostFrame *> free_;
  std::deque<Job> jobs_;
  std::mutex m_;
  std::condition_variable cv_;
  std::thread th_;
  bool stop_ = false;
  int rc_ = PD_OK;
};

}  // namespace

extern "C" {

int pd_write_frame(pd_sim *s, uint32_t counter) {
  if (!s) return fail(PD_EINVAL, "null handle");
  const uint64_t N = s->eng.num_nodes();
  const uint32_t P = s->eng.num_particles();
  std::vector<double> cur(3 * N), vel(3 * N), acc(3 * N), force(3 * N);
  int rc = s->eng.get_state(cur.data(), vel.data(), acc.data(), force.data(), nullptr);
  if (rc != PD_OK) return rc;
  const int32_t pvp = s->cfg.particle_w_fixed_velocity;
  std::vector<double> afd;
  if (pvp >= 0 && (uint32_t)pvp < P) {
    afd.resize(3 * N);
    rc = s->eng.get_afd(afd.data());
    if (rc != PD_OK) return rc;
  }
  double wall[6], react[18];
  rc = s->eng.get_wall(0, wall, react);
  if (rc != PD_OK) return rc;
  return write_frame_files(
      s, counter, cur.data(), vel.data(), acc.data(), force.data(), afd.empty() ? nullptr : afd.data(),
      [&](uint32_t p, std::vector<uint32_t> &pairs) {
        uint64_t m = 0;
        int r = s->eng.get_connectivity(p, nullptr, 0, &m);
        if (r != PD_OK) return r;
        pairs.resize(2 * m);
        return s->eng.get_connectivity(p, pairs.data(), m, &m);
      },
      wall, react);
}

// Sets the kinematic state (and, with enable_fracture, the surviving bonds) from a saved
// frame, like the resume branch of run_timeloop (timeloop.h:262-312).
int pd_resume(pd_sim *s, uint32_t resume_ind, int wall_resume) {
  if (!s) return fail(PD_EINVAL, "null handle");
  char buf[64];
  std::snprintf(buf, sizeof(buf), "/tc_%05u.h5", resume_ind);
  h5lite::Reader r;
  std::string err;
  if (!r.open(s->outdir + buf, err)) return fail(PD_EIO, err);
  const auto &hs = s->eng.sims()[0];
  const uint64_t N = s->eng.num_nodes();
  std::vector<double> disp(3 * N), vel(3 * N), acc(3 * N);
  for (uint32_t p = 0; p < hs.np; ++p) {
    const std::string g = pnum(p) + "/";
    const uint64_t a = hs.node_offset[p], n = hs.node_offset[p + 1] - a;
    std::vector<double> cp, v, ac;
    std::vector<uint64_t> dims;
    if (!r.read_vec<double>(g + "CurrPos", h5lite::F64, cp, dims, err) || cp.size() != 3 * n ||
        !r.read_vec<double>(g + "vel", h5lite::F64, v, dims, err) || v.size() != 3 * n ||
        !r.read_vec<double>(g + "acc", h5lite::F64, ac, dims, err) || ac.size() != 3 * n)
      return fail(PD_EIO, "resume frame: " + (err.empty() ? g + " size mismatch" : err));
    for (uint64_t k = 0; k < 3 * n; ++k) {
      disp[3 * a + k] = cp[k] - hs.pos[3 * a + k];  // disp = CurrPos - pos (timeloop.h:279-281)
      vel[3 * a + k] = v[k];
      acc[3 * a + k] = ac[k];
    }
    if (s->cfg.enable_fracture) {
      std::vector<uint32_t> conn;
      if (!r.read_vec<uint32_t>(g + "Connectivity", h5lite::U32, conn, dims, err))
        return fail(PD_EIO, "resume frame: " + err);
      int rc = s->eng.set_connectivity(p, conn.data(), conn.size() / 2);
      if (rc != PD_OK) return rc;
    }
  }
  int rc = s->eng.set_state(disp.data(), vel.data(), acc.data());
  if (rc != PD_OK) return rc;
  if (wall_resume) {
    std::snprintf(buf, sizeof(buf), "/wall_%05u.h5", resume_ind);
    h5lite::Reader rw;
    if (!rw.open(s->outdir + buf, err)) return fail(PD_EIO, err);
    std::vector<double> wi;
    std::vector<uint64_t> dims;
    if (!rw.read_vec<double>("wall_info", h5lite::F64, wi, dims, err) || wi.size() < 6)
      return fail(PD_EIO, "wall resume: " + err);
    rc = s->eng.set_wall(0, wi.data());
    if (rc != PD_OK) return rc;
  }
  return PD_OK;
}

// run_timeloop's loop with saves, progress table and run_time.h5 (timeloop.h:314-964).
int pd_run(pd_sim *s) {
  if (!s) return fail(PD_EINVAL, "null handle");
  pd_config &cf = s->cfg;
  const std::string out = s->outdir;
  if (!is_dir(out)) return fail(PD_EIO, "output directory does not exist: " + out);
  std::cout << "Output data dir: " << out << std::endl;
  uint32_t counter, first_counter, last_counter;
  if (cf.do_resume) {
    counter = cf.resume_ind + 1;
    first_counter = counter;
    last_counter = cf.resume_ind + cf.timesteps / cf.modulo;
    char b[64];
    std::snprintf(b, sizeof(b), "/tc_%05u.h5", cf.resume_ind);
    std::cout << "Loading from file: " << out + b << std::endl;
    int rc = pd_resume(s, cf.resume_ind, cf.wall_resume);
    if (rc != PD_OK) return rc;
    std::cout << "Resuming from counter " << counter << std::endl;
  } else {
    counter = 1;
    first_counter = counter;
    last_counter = cf.timesteps / cf.modulo;
  }
  {  // plotinfo.h5 (timeloop.h:320-350)
    double wall[6];
    s->eng.get_wall(0, wall, nullptr);
    h5lite::Writer w;
    uint32_t flc[2] = {first_counter, last_counter}, dim = 3, mod = cf.modulo;
    int32_t aw = s->eng.sims()[0].allow_wall ? 1 : 0;
    w.add("f_l_counter", h5lite::U32, {2, 1}, flc);
    w.add("dimension", h5lite::U32, {1, 1}, &dim);
    w.add("dt", h5lite::F64, {1, 1}, &cf.dt);
    w.add("modulo", h5lite::U32, {1, 1}, &mod);
    w.add("wall/allow_wall", h5lite::I32, {1, 1}, &aw);
    w.add("wall/geom_wall_info", h5lite::F64, {6, 1}, wall);
    std::string err;
    std::cout << "Output plotinfo: " << out + "/plotinfo.h5" << std::endl;
    if (!w.write(out + "/plotinfo.h5", err)) return fail(PD_EIO, err);
  }
  const unsigned cw = 12;
  time_t now = time(nullptr);
  char sc[64];
  std::snprintf(sc, sizeof(sc), "ct[%d:%d]", (int)first_counter, (int)last_counter);
  std::cout << "----------------------------------------------------------------------" << std::endl;
  std::cout << "Starting time loop (Parallel=" << cf.is_parallel << "): " << ctime(&now);
  std::cout << std::left << std::setw(cw) << "t " << std::setw(cw) << std::string(sc) << std::setw(cw + 5)
            << "duration(s)" << std::setw(cw) << "rem(h:m:s)" << std::setw(cw) << "#contacts" << std::setw(cw)
            << "time" << std::endl;
  s->eng.set_tuning(0, 0, 0, cf.save_file ? 1 : 0, -1);
  auto t0 = std::chrono::system_clock::now();
  std::vector<double> run_time, t_ind;
  std::vector<uint32_t> pw_vec;
  // progress row of each written frame (timeloop.h:909-947), printed by the writer thread
  FrameWriter fw(s, [&](uint32_t ctr, uint32_t t, const pdg::HostFrame &f) {
    auto t1 = std::chrono::system_clock::now();
    const int ms = (int)std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count();
    t0 = t1;
    double avg = 0;
    const int start = (int)run_time.size() - 10;
    if (start > 0)
      for (int c = start; c < (int)run_time.size(); ++c) avg += run_time[c];
    avg /= 10;
    const int rem = (int)((int)(last_counter - ctr) * avg);
    char ts[80];
    time_t nt = time(nullptr);
    strftime(ts, sizeof(ts), "%F-%T", localtime(&nt));
    std::cout << std::left << std::setw(cw) << t << std::setw(cw) << ctr << std::setw(cw + 5) << (double)ms / 1000
              << std::setw(cw) << format_ms(rem) << std::setw(cw) << f.cnt->pairwise << std::setw(cw) << ts
              << std::endl;
    run_time.push_back(ms);
    t_ind.push_back(t);
    pw_vec.push_back((uint32_t)f.cnt->pairwise);
  });
  if (cf.save_file && cf.modulo) {
    int rc = fw.start(2);
    if (rc != PD_OK) return rc;
  }
  uint32_t t = 0;
  while (t < cf.timesteps) {
    uint32_t n = cf.timesteps - t;
    if (cf.save_file && cf.modulo) n = std::min<uint32_t>(n, cf.modulo - (t % cf.modulo));
    int rc = s->eng.step(n);
    if (rc != PD_OK) {
      fw.finish();
      return rc;
    }
    t += n;
    if (cf.save_file && cf.modulo && t % cf.modulo == 0) {
      rc = fw.submit(counter, t);
      if (rc != PD_OK) {
        fw.finish();
        return rc;
      }
      ++counter;
    }
  }
  int rc = s->eng.sync(-1);
  const int wrc = fw.finish();
  if (rc != PD_OK) return rc;
  if (wrc != PD_OK) return wrc;
  if (is_dir("output/hdf5")) {  // run_time.h5 at the reference's fixed path (timeloop.h:957-964)
    h5lite::Writer w;
    w.add("run_time", h5lite::F64, {run_time.size(), 1}, run_time.data());
    w.add("t_ind", h5lite::F64, {t_ind.size(), 1}, t_ind.data());
    w.add("pairwise_computations", h5lite::U32, {pw_vec.size(), 1}, pw_vec.data());
    std::string err;
    w.write("output/hdf5/run_time.h5", err);
  }
  return PD_OK;
}

// ---- generic HDF5 access for scripts (setup writing, frame reading) -------------------

void *pd_h5_writer_new(void) { return new h5lite::Writer(); }
int pd_h5_writer_add(void *w, const char *path, int dtype, int rank, const uint64_t *dims, const void *data) {
  if (!w || !path || rank < 0 || rank > 8) return PD_EINVAL;
  static_cast<h5lite::Writer *>(w)->add(path, dtype, std::vector<uint64_t>(dims, dims + rank), data);
  return PD_OK;
}
int pd_h5_writer_write(void *w, const char *filename) {
  std::string err;
  if (!w || !filename) return PD_EINVAL;
  if (!static_cast<h5lite::Writer *>(w)->write(filename, err)) return fail(PD_EIO, err);
  return PD_OK;
}
void pd_h5_writer_free(void *w) { delete static_cast<h5lite::Writer *>(w); }

void *pd_h5_open(const char *filename) {
  auto *r = new h5lite::Reader();
  std::string err;
  if (!filename || !r->open(filename, err)) {
    g_ferr = err;
    delete r;
    return nullptr;
  }
  return r;
}
// Newline-separated dataset paths; returns the length needed (including the NUL).
size_t pd_h5_list(void *h, char *buf, size_t cap) {
  if (!h) return 0;
  std::string all;
  for (auto &p : static_cast<h5lite::Reader *>(h)->paths()) all += p + "\n";
  if (buf && cap) {
    size_t n = std::min(all.size(), cap - 1);
    std::memcpy(buf, all.data(), n);
    buf[n] = 0;
  }
  return all.size() + 1;
}
int pd_h5_info(void *h, const char *path, int *rank, uint64_t *dims) {
  if (!h || !path) return PD_EINVAL;
  const h5lite::Info *in = static_cast<h5lite::Reader *>(h)->info(path);
  if (!in) return fail(PD_EIO, std::string("no dataset ") + path);
  *rank = in->rank;
  for (int i = 0; i < in->rank && i < 8; ++i) dims[i] = in->dims[i];
  return PD_OK;
}
int pd_h5_read(void *h, const char *path, int dtype, void *out, uint64_t cap_bytes) {
  if (!h || !path) return PD_EINVAL;
  std::vector<uint8_t> b;
  std::vector<uint64_t> dims;
  std::string err;
  if (!static_cast<h5lite::Reader *>(h)->read(path, dtype, b, dims, err)) return fail(PD_EIO, err);
  if (b.size() > cap_bytes) return fail(PD_EINVAL, "buffer too small");
  if (!b.empty()) std::memcpy(out, b.data(), b.size());
  return PD_OK;
}
void pd_h5_close(void *h) { delete static_cast<h5lite::Reader *>(h); }

}  // extern "C"
