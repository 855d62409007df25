// pd_frames.cpp -- output frames off the critical path: the state a frame needs is copied to
// pinned host memory in stream order (no synchronisation of the step pipeline), and the host
// turns it into the arrays of a tc_%05u.h5 / wall_%05u.h5 frame (timeloop.h:801-953) later,
// on another thread, with the same arithmetic as get_state / get_connectivity / get_wall.
#include <cstring>

#include "pd_engine.h"

#define PD_TRY(expr)              \
  do {                            \
    int _rc = (expr);             \
    if (_rc != PD_OK) return _rc; \
  } while (0)

namespace pdg {

int Engine::frame_alloc(HostFrame &f) {
  const size_t a3 = 3 * Ncap_ * sizeof(double);
  auto pin = [&](void **p, size_t b) { return check(cudaMallocHost(p, b ? b : 8), "pinned frame buffer"); };
  PD_TRY(pin((void **)&f.disp, a3));
  PD_TRY(pin((void **)&f.vel, a3));
  PD_TRY(pin((void **)&f.acc, a3));
  PD_TRY(pin((void **)&f.force, a3));
  if (reset_possible_) PD_TRY(pin((void **)&f.pos, a3));
  if (n_clamped_) PD_TRY(pin((void **)&f.cdisp, 3 * n_clamped_ * sizeof(double)));
  if (d_afd_) PD_TRY(pin((void **)&f.afd, a3));
  PD_TRY(pin((void **)&f.mask, std::max<uint64_t>(E_ / 32, 1) * 4));
  PD_TRY(pin((void **)&f.ss, S_ * sizeof(DevSimState)));
  PD_TRY(pin((void **)&f.cnt, sizeof(DevCounters)));
  PD_TRY(check(cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming), "frame event"));
  if (h_col_.empty()) {  // column indices never change: read them back once
    h_col_.resize(std::max<uint64_t>(E_, 1));
    PD_TRY(cpy(h_col_.data(), d_col_, h_col_.size() * 4, "read columns"));
  }
  return PD_OK;
}

void Engine::frame_free(HostFrame &f) {
  if (f.done) cudaEventSynchronize(f.done);
  for (void *p : {(void *)f.disp, (void *)f.vel, (void *)f.acc, (void *)f.force, (void *)f.pos, (void *)f.cdisp,
                  (void *)f.afd, (void *)f.mask, (void *)f.ss, (void *)f.cnt})
    if (p) cudaFreeHost(p);
  if (f.done) cudaEventDestroy(f.done);
  f = HostFrame();
}

int Engine::frame_stage(HostFrame &f) {
  const size_t a3 = 3 * Ncap_ * sizeof(double);
  cudaStream_t s = stream_;
  auto d2h = [&](void *dst, const void *src, size_t b) {
    return check(cudaMemcpyAsync(dst, src, b, cudaMemcpyDeviceToHost, s), "stage frame");
  };
  const bool fused = precision_ == PD_FP32C;
  PD_TRY(d2h(f.disp, fused ? d_dispb_[cur_ ^ 1] : d_disp_, a3));
  PD_TRY(d2h(f.vel, d_vel_[cur_], a3));
  PD_TRY(d2h(f.acc, d_acc_, a3));
  PD_TRY(d2h(f.force, d_force_, a3));
  if (f.pos) PD_TRY(d2h(f.pos, d_pos_, a3));
  if (f.cdisp) PD_TRY(d2h(f.cdisp, d_clamped_disp_, 3 * n_clamped_ * sizeof(double)));
  if (f.afd) PD_TRY(d2h(f.afd, d_afd_, a3));
  PD_TRY(d2h(f.mask, d_mask_, std::max<uint64_t>(E_ / 32, 1) * 4));
  PD_TRY(d2h(f.ss, d_ss_, S_ * sizeof(DevSimState)));
  PD_TRY(d2h(f.cnt, d_cnt_, sizeof(DevCounters)));
  // the pairwise count restarts for the next save interval (get_stats does the same)
  PD_TRY(check(cudaMemsetAsync(&d_cnt_->pairwise, 0, sizeof(unsigned long long), s), "reset pairwise"));
  f.steps = steps_done_;
  return check(cudaEventRecord(f.done, s), "frame event");
}

void Engine::frame_state(const HostFrame &f, double *curpos, double *vel, double *acc, double *force,
                         double *afd) const {
  const uint64_t C = Ncap_;
  const bool fused = precision_ == PD_FP32C;
  auto rows = [&](const double *src, double *dst) { rows_to_file(src, C, 0, N_, dst); };
  if (curpos) {
    std::vector<double> dsp(3 * N_);
    rows(f.disp, dsp.data());
    if (n_clamped_ && f.steps > 0 && !fused)  // CurrPos of clamped nodes: the predicted displacement
      for (uint64_t i = 0; i < n_clamped_; ++i)
        for (int c = 0; c < 3; ++c) dsp[3 * (uint64_t)h_clamped_[i] + c] = f.cdisp[3 * i + c];
    if (f.pos) {
      rows(f.pos, curpos);
      for (uint64_t k = 0; k < 3 * N_; ++k) curpos[k] = curpos[k] + dsp[k];
    } else {
      uint64_t off = 0;
      for (auto &s : sims_) {
        const uint64_t ns = s.node_offset[s.np];
        for (uint64_t k = 0; k < 3 * ns; ++k) curpos[3 * off + k] = s.pos[k] + dsp[3 * off + k];
        off += ns;
      }
    }
  }
  if (vel) rows(f.vel, vel);
  if (acc) rows(f.acc, acc);
  if (force) rows(f.force, force);
  if (afd) {
    if (f.afd)
      rows(f.afd, afd);
    else
      std::memset(afd, 0, 3 * N_ * sizeof(double));
  }
}

// NbdArr2conn (timeloop.h:20-44) from the staged live masks.
void Engine::frame_connectivity(const HostFrame &f, uint32_t particle, std::vector<uint32_t> &pairs) const {
  pairs.clear();
  if (particle >= P_) return;
  const uint64_t g0 = h_g0_[particle];
  uint64_t nloc = 0;
  {
    uint32_t pacc = 0;
    for (auto &s : sims_) {
      if (particle < pacc + s.np) {
        nloc = s.node_offset[particle - pacc + 1] - s.node_offset[particle - pacc];
        break;
      }
      pacc += s.np;
    }
  }
  for (uint64_t i = 0; i < nloc; ++i) {  // file order
    const uint64_t g = node_of_[g0 + i];
    const uint64_t base = h_slice_ptr_[g >> 5] + (g & 31);
    const uint64_t mbase = h_slice_ptr_[g >> 5] >> 5;
    for (uint32_t j = 0; j < h_deg_[g]; ++j) {
      if (!((f.mask[mbase + j] >> (g & 31)) & 1u)) continue;
      const uint64_t q = file_of_[h_col_[base + 32ull * j] & kColIndex] - g0;
      if (i < q) {
        pairs.push_back((uint32_t)i);
        pairs.push_back((uint32_t)q);
      }
    }
  }
}

void Engine::frame_wall(const HostFrame &f, uint32_t sim, double *wall_info, double *reaction) const {
  if (sim >= S_) return;
  if (wall_info) std::memcpy(wall_info, f.ss[sim].wall, 6 * sizeof(double));
  if (reaction) std::memcpy(reaction, f.ss[sim].react, 18 * sizeof(double));
}

}  // namespace pdg
