// pd_engine.cu -- host side of the explicit-step engine: builds the HBM layout described in
// pd_engine.h from one or more simulations, captures one step as a CUDA graph and replays
// it, and reads results back in the reference's shapes.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <thread>

#include "pd_engine.h"
#include "pd_math.cuh"

namespace pdg {

#define PD_TRY(expr)             \
  do {                           \
    int _rc = (expr);            \
    if (_rc != PD_OK) return _rc; \
  } while (0)

namespace {
inline uint64_t round_up(uint64_t x, uint64_t m) { return (x + m - 1) / m * m; }
}  // namespace

// Device memory comes from the stream-ordered allocator and goes back to it in stream order:
// neither creating nor closing a handle waits for other handles' queued work, so a server
// can admit and retire simulations while others keep the GPU busy.
Engine::~Engine() {
  if (stream_) cudaStreamSynchronize(stream_);
  if (h_stage_) cudaFreeHost(h_stage_);
  for (int i = 0; i < 2; ++i)
    if (graph_[i]) cudaGraphExecDestroy(graph_[i]);
  for (void *p : allocs_) cudaFreeAsync(p, capture_stream_);
  if (own_stream_ && capture_stream_) cudaStreamDestroy(capture_stream_);
}

int Engine::check(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return PD_OK;
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? PD_ENOMEM : PD_ECUDA;
}

int Engine::raw_alloc(void **p, size_t bytes) {
  cudaError_t e = cudaMallocAsync(p, bytes, capture_stream_);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    err = std::string("device allocation of ") + std::to_string(bytes) + " B: " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? PD_ENOMEM : PD_ECUDA;
  }
  device_bytes_ += bytes;
  return PD_OK;
}

int Engine::cpy(void *dst, const void *src, size_t bytes, const char *what) {
  PD_TRY(check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, stream_), what));
  return check(cudaStreamSynchronize(stream_), what);
}

int Engine::mset(void *dst, int value, size_t bytes, const char *what) {
  return check(cudaMemsetAsync(dst, value, bytes, stream_), what);
}

template <typename T>
static int dalloc(Engine *E, std::vector<void *> &allocs, T **p, uint64_t count, std::string &err) {
  (void)err;
  *p = nullptr;
  if (count == 0) count = 1;
  void *q = nullptr;
  PD_TRY(E->raw_alloc(&q, count * sizeof(T)));
  *p = (T *)q;
  allocs.push_back(q);
  return PD_OK;
}

DevView Engine::view(int cur) const {
  DevView v;
  std::memset(&v, 0, sizeof(v));
  v.N = N_;
  v.Ncap = Ncap_;
  v.P = P_;
  v.S = S_;
  v.pos = d_pos_;
  v.disp = d_disp_;
  v.vel_in = d_vel_[cur];
  v.vel_out = d_vel_[cur ^ 1];
  v.acc = d_acc_;
  v.force = d_force_;
  v.ext = d_ext_;
  v.vol = d_vol_;
  v.pid = d_pid_;
  v.node_of = d_node_of_;
  v.file_of = d_file_of_;
  v.bdry = d_bdry_;
  v.slice_ptr = d_slice_ptr_;
  v.deg = d_deg_;
  v.col = d_col_;
  v.mask = d_mask_;
  v.bxi = d_bxi_;
  v.bxin = d_bxin_;
  v.brxin = d_brxin_;
  v.E = E_;
  v.anchor = d_anchor_;
  if (precision_ == PD_FP32C) {
    v.disp = d_dispb_[cur];
    v.disp_next = d_dispb_[cur ^ 1];
    v.rec = d_rec_[cur];
    v.rec_next = d_rec_[cur ^ 1];
    v.anchor_next = d_anchor_next_;
    v.clamp_flag = d_clamp_flag_;
    v.fused = 1;
  }
  v.break_band = 1e-4;
  v.f_extra = d_f_extra_;
  v.win_lo = d_win_lo_;
  v.win_cnt = d_win_cnt_;
  v.win_max = win_max_;
  v.xnodes = bp_.xnodes;
  v.xparts = bp_.xparts;
  v.xcount = bp_.xcount;
  v.max_part_nodes = max_part_nodes_;
  v.extra_flag = d_extra_flag_;
  v.wall_local = d_wall_local_;
  v.lrtb_local_next = d_lrtb_local_;
  v.parts = d_parts_;
  v.lrtb = d_lrtb_;
  v.lrtb_next = d_lrtb_next_;
  v.sp = d_sp_;
  v.ss = d_ss_;
  v.cand = bp_.cand;
  v.cand_n = bp_.cand_n;
  v.cand_cap = bp_.cand_cap;
  v.cell_count = bp_.count;
  v.cell_start = bp_.start;
  v.cell_sorted = bp_.sorted;
  v.cell_mask = bp_.table_bits ? (uint32_t)((1ull << bp_.table_bits) - 1) : 0u;
  v.centroid = d_centroid_;
  v.afd = d_afd_;
  if (n_clamped_) {
    v.clamped_ptr = d_clamped_;
    v.clamped_list = d_clamped_ + (P_ + 1);
    v.clamped_disp = d_clamped_disp_;
  }
  v.cnt = d_cnt_;
  v.stats = stats_ ? 1 : 0;
  return v;
}

// Host mirror of the sticky toggles of timeloop.h:405-464 for the first step.
static void host_sim_toggles(const DevSimParams &sp, DevSimState &st, uint32_t t) {
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

int Engine::init(std::vector<HostSim> &sims, int precision) {
  sims_.swap(sims);
  precision_ = precision;
  S_ = (uint32_t)sims_.size();
  P_ = 0;
  N_ = 0;
  for (auto &s : sims_) {
    P_ += s.np;
    N_ += s.node_offset[s.np];
  }
  if (N_ == 0 || P_ == 0) {
    err = "empty setup";
    return PD_EINVAL;
  }
  if (N_ > 0x7FFFFFE0ull) {  // node indices use 31 bits (bit 31 of a column entry is a flag)
    err = "too many nodes for 31-bit node indices";
    return PD_EINVAL;
  }
  Ncap_ = round_up(N_, 32);
  nslices_ = Ncap_ / 32;
  // default bond-kernel variant: the autotuner's choice on small and on large handles (small
  // handles are launch-latency bound and gain most from doing the non-bond work in the bond
  // kernel, one launch less per step)
  variant_ = N_ < 131072 ? 25 : 18;
  // and the step graph: on large handles the broad phase's kernels are worth skipping in
  // steps without a rebuild (a conditional node); small handles replay them, exiting at once.
  // Small FP32 handles step in persistent launches (where the handle's features allow it,
  // persist_eligible), faster than either graph on every small workload measured.
  use_conditional_ = N_ >= 131072;
  use_persist_ = precision_ == PD_FP32C && N_ < 131072;
  sim_node0_.assign(S_ + 1, 0);
  sim_p0_.assign(S_ + 1, 0);
  for (uint32_t i = 0; i < S_; ++i) {
    sim_node0_[i + 1] = sim_node0_[i] + sims_[i].node_offset[sims_[i].np];
    sim_p0_[i + 1] = sim_p0_[i] + sims_[i].np;
  }
  sim_steps_.assign(S_, 0);
  finished_.assign(S_, 0);
  final_.assign(S_, std::vector<double>());
  {
    int64_t bad = -1;
    order_nodes(sims_, file_of_, node_of_, deg_file_, &bad, &conn_sorted_, order_bin(precision_));
    if (bad >= 0) {
      err = "Connectivity index out of range in particle " + std::to_string(bad);
      return PD_EINVAL;
    }
  }
  PD_TRY(check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate"));
  own_stream_ = true;
  capture_stream_ = stream_;
  const int rc = alloc_and_upload();
  std::vector<uint32_t>().swap(deg_file_);
  // arrays read only while building (possibly views of the caller's buffers)
  for (auto &s : sims_) {
    s.vol.release();
    s.disp.release();
    s.vel.release();
    s.acc.release();
    s.ext.release();
    s.conn.release();
  }
  return rc;
}


void Engine::order_nodes(const std::vector<HostSim> &sims, std::vector<uint32_t> &file_of,
                         std::vector<uint32_t> &node_of, std::vector<uint32_t> &deg_file, int64_t *bad,
                         bool *sorted, uint32_t deg_bin) {
  // The SELL-32 layout pads every row of a slice to the slice's longest row. In file order a
  // slice mixes interior nodes (full neighbourhoods) with surface nodes (truncated ones);
  // sorting by bond count makes the rows of a slice nearly equal (crush512: padded entries
  // 1.23x the bonds in file order, 1.03x sorted). Sorting by count / deg_bin keeps more of the
  // file's lattice order among nodes of nearly equal counts (deg_bin 16: 1.07x padding). The sort runs inside windows of
  // kOrderWindow consecutive nodes of a particle and is stable, so a node moves less than a
  // window and interior nodes keep their lattice order: partners stay close in memory (a
  // whole-particle sort of a 1.5 M-node plate made the FP32 bond kernel slower).
  // Per-node results do not depend on the order: each node's sums keep the reference's row
  // order, and every sequence that the reference takes in node order (contact partners,
  // particle means) is taken in file order through node_of / file_of.
  struct PartRef {
    const HostSim *s;
    uint32_t p;
    uint64_t g0;
  };
  std::vector<PartRef> parts;
  uint64_t N = 0;
  for (auto &s : sims) {
    for (uint32_t p = 0; p < s.np; ++p) parts.push_back({&s, p, N + s.node_offset[p]});
    N += s.node_offset[s.np];
  }
  deg_file.assign(N, 0);
  file_of.assign(N, 0);
  node_of.assign(N, 0);
  std::atomic<int64_t> bad_p(-1);
  std::atomic<bool> all_sorted(true);
  parallel_items(parts.size(), [&](uint64_t x) {
    const HostSim &s = *parts[x].s;
    const uint32_t p = parts[x].p;
    const uint64_t g0 = parts[x].g0;
    const uint64_t nloc = s.node_offset[p + 1] - s.node_offset[p];
    uint32_t *dg = deg_file.data() + g0;
    bool srt = true;  // pairs i < j in strictly increasing (i, j) order: every row ascending
    uint64_t prev = 0;
    for (uint64_t l = s.conn_offset[p]; l < s.conn_offset[p + 1]; ++l) {
      const uint32_t i = s.conn[2 * l], j = s.conn[2 * l + 1];
      if (i < nloc && j < nloc) {
        dg[i]++;
        dg[j]++;
      } else {
        bad_p = (int64_t)p;
      }
      const uint64_t key = ((uint64_t)i << 32) | j;
      srt = srt && i < j && (l == s.conn_offset[p] || key > prev);
      prev = key;
    }
    if (!srt) all_sorted = false;
    std::vector<uint32_t> idx(nloc);
    std::vector<uint32_t> hist;
    for (uint64_t w0 = 0; w0 < nloc; w0 += kOrderWindow) {
      const uint64_t w1 = std::min<uint64_t>(nloc, w0 + kOrderWindow);
      uint32_t dmax = 0;
      for (uint64_t k = w0; k < w1; ++k) dmax = std::max(dmax, (dg[k] / deg_bin));
      if (dmax < 4096) {  // stable counting sort by descending count
        hist.assign(dmax + 2, 0);
        for (uint64_t k = w0; k < w1; ++k) hist[dmax - (dg[k] / deg_bin) + 1]++;
        for (uint32_t d = 1; d <= dmax + 1; ++d) hist[d] += hist[d - 1];
        for (uint64_t k = w0; k < w1; ++k) idx[w0 + hist[dmax - (dg[k] / deg_bin)]++] = (uint32_t)k;
      } else {
        for (uint64_t k = w0; k < w1; ++k) idx[k] = (uint32_t)k;
        std::stable_sort(idx.begin() + w0, idx.begin() + w1, [&](uint32_t a, uint32_t b) { return dg[a] / deg_bin > dg[b] / deg_bin; });
      }
    }
    for (uint64_t k = 0; k < nloc; ++k) {
      file_of[g0 + k] = (uint32_t)(g0 + idx[k]);
      node_of[g0 + idx[k]] = (uint32_t)(g0 + k);
    }
  });
  if (bad) *bad = bad_p.load();
  if (sorted) *sorted = all_sorted.load();
}

int Engine::build_bonds_host(SellHost &h) {
  // conn2NArr (load_hdf5.h:27-37): for every Connectivity row (i, j) push j onto row i and
  // i onto row j; rows keep that push order. Particles own disjoint rows, so they are filled
  // in parallel; the live masks (all bonds live at the start) follow from the degrees alone.
  // Host work only (it runs beside the node arrays' staging and upload).
  struct PartRef {
    const HostSim *s;
    uint32_t p;
    uint64_t g0;
  };
  std::vector<PartRef> parts;
  {
    uint64_t gnode = 0;
    for (auto &s : sims_) {
      for (uint32_t p = 0; p < s.np; ++p) parts.push_back({&s, p, gnode + s.node_offset[p]});
      gnode += s.node_offset[s.np];
    }
  }
  std::vector<uint32_t> deg;
  {
    const int rc = bond_counts(deg, nullptr);
    if (rc != PD_OK) {
      h.err = "node degree above 65535";
      return rc;
    }
  }
  const uint64_t ncol = std::max<uint64_t>(E_, 1), nmask = std::max<uint64_t>(E_ / 32, 1);
  h.ncol = ncol;
  h.nmask = nmask;
  h.col.reset(new uint32_t[ncol]);  // every entry set below
  h.mask.reset(new uint32_t[nmask]);
  uint32_t *col = h.col.get(), *mask = h.mask.get();
  col[0] = kNoCol;
  mask[0] = 0u;
  parallel_items((nslices_ + 63) / 64, [&](uint64_t chunk) {
    // padding entries, and the live bits: position j of lane l is a bond iff j < deg (below the
    // slice's shortest row every lane has a bond)
    for (uint64_t sl = chunk * 64; sl < std::min<uint64_t>(nslices_, chunk * 64 + 64); ++sl) {
      const uint64_t e0 = h_slice_ptr_[sl], e1 = h_slice_ptr_[sl + 1];
      const uint64_t w = (e1 - e0) / 32;
      uint64_t dmin = w;
      for (int l = 0; l < 32; ++l) dmin = std::min<uint64_t>(dmin, deg[sl * 32 + l]);
      for (uint64_t j = 0; j < dmin; ++j) mask[(e0 >> 5) + j] = 0xFFFFFFFFu;
      for (uint64_t j = dmin; j < w; ++j) {
        uint32_t bits = 0;
        for (int l = 0; l < 32; ++l)
          if (j < deg[sl * 32 + l]) {
            bits |= 1u << l;
          } else {
            col[e0 + 32 * j + l] = kNoCol;
          }
        mask[(e0 >> 5) + j] = bits;
      }
    }
  });
  std::vector<uint32_t> fill(Ncap_, 0);
  parallel_items(parts.size(), [&](uint64_t x) {
    const HostSim &s = *parts[x].s;
    const uint32_t p = parts[x].p;
    const uint64_t g0 = parts[x].g0;
    for (uint64_t l = s.conn_offset[p]; l < s.conn_offset[p + 1]; ++l) {
      const uint64_t a = node_of_[g0 + s.conn[2 * l]], b = node_of_[g0 + s.conn[2 * l + 1]];
      col[h_slice_ptr_[a >> 5] + 32ull * fill[a] + (a & 31)] = (uint32_t)b;
      fill[a]++;
      col[h_slice_ptr_[b >> 5] + 32ull * fill[b] + (b & 31)] = (uint32_t)a;
      fill[b]++;
    }
  });
  return PD_OK;
}

int Engine::bond_counts(std::vector<uint32_t> &deg, std::vector<uint64_t> *rowptr) {
  // bond counts per engine node (counted by order_nodes, which also checked the indices),
  // slice widths, and the row starts of a row-contiguous layout when asked for
  deg.assign(Ncap_, 0);
  const uint64_t nchunk = (Ncap_ + 65535) / 65536;
  std::vector<uint32_t> cmax(nchunk, 0);
  std::vector<uint64_t> csum(nchunk + 1, 0);
  parallel_items(nchunk, [&](uint64_t c) {
    uint32_t m = 0;
    for (uint64_t g = c * 65536; g < std::min<uint64_t>(N_, c * 65536 + 65536); ++g) {
      deg[node_of_[g]] = deg_file_[g];
      m = std::max(m, deg_file_[g]);
    }
    cmax[c] = m;
  });
  uint32_t maxdeg = 0;
  for (uint32_t m : cmax) maxdeg = std::max(maxdeg, m);
  if (maxdeg > 65535) return PD_EINVAL;
  h_deg_.assign(Ncap_, 0);
  if (rowptr) rowptr->assign(Ncap_ + 1, 0);
  parallel_items(nchunk, [&](uint64_t c) {
    uint64_t t = 0;
    for (uint64_t n = c * 65536; n < std::min<uint64_t>(Ncap_, c * 65536 + 65536); ++n) {
      h_deg_[n] = (uint16_t)deg[n];
      if (rowptr) (*rowptr)[n] = t;  // offset inside the chunk for now
      t += deg[n];
    }
    csum[c + 1] = t;
  });
  for (uint64_t c = 0; c < nchunk; ++c) csum[c + 1] += csum[c];
  initial_bonds_ = csum[nchunk];
  if (rowptr) {
    parallel_items(nchunk, [&](uint64_t c) {
      for (uint64_t n = c * 65536; n < std::min<uint64_t>(Ncap_, c * 65536 + 65536); ++n) (*rowptr)[n] += csum[c];
    });
    (*rowptr)[Ncap_] = csum[nchunk];
  }
  h_slice_ptr_.assign(nslices_ + 1, 0);
  parallel_items((nslices_ + 4095) / 4096, [&](uint64_t c) {
    for (uint64_t sl = c * 4096; sl < std::min<uint64_t>(nslices_, c * 4096 + 4096); ++sl) {
      uint32_t w = 0;
      for (int l = 0; l < 32; ++l) w = std::max(w, deg[sl * 32 + l]);
      h_slice_ptr_[sl + 1] = 32ull * w;  // widths for now
    }
  });
  for (uint64_t sl = 0; sl < nslices_; ++sl) h_slice_ptr_[sl + 1] += h_slice_ptr_[sl];
  E_ = h_slice_ptr_[nslices_];
  return PD_OK;
}

int Engine::alloc_bond_arrays() {
  const uint64_t ncol = std::max<uint64_t>(E_, 1), nmask = std::max<uint64_t>(E_ / 32, 1);
  if (precision_ == PD_FP32C) {
    // record ranges of the staged bond kernel: computed on the device the first time a staged
    // variant is chosen (prepare_windows)
    const uint64_t nb = (N_ + kStageNodes - 1) / kStageNodes;
    PD_TRY(dalloc(this, allocs_, &d_win_lo_, nb, err));
    PD_TRY(dalloc(this, allocs_, &d_win_cnt_, nb, err));
    win_max_ = 0;
    windows_ready_ = false;
  }
  PD_TRY(dalloc(this, allocs_, &d_slice_ptr_, nslices_ + 1, err));
  PD_TRY(dalloc(this, allocs_, &d_deg_, Ncap_, err));
  PD_TRY(dalloc(this, allocs_, &d_col_, ncol, err));
  PD_TRY(dalloc(this, allocs_, &d_mask_, nmask, err));
  PD_TRY(cpy(d_slice_ptr_, h_slice_ptr_.data(), (nslices_ + 1) * 8, "upload slice_ptr"));
  PD_TRY(cpy(d_deg_, h_deg_.data(), Ncap_ * 2, "upload deg"));
  return PD_OK;
}

int Engine::build_bonds_gpu(const std::vector<uint64_t> &rowptr, bool &fallback) {
  fallback = false;
  // per-particle pair offsets and first nodes, particles of all simulations concatenated
  std::vector<uint64_t> pair_off(1, 0), node0;
  uint64_t gnode = 0;
  for (auto &s : sims_) {
    for (uint32_t p = 0; p < s.np; ++p) {
      pair_off.push_back(pair_off.back() + (s.conn_offset[p + 1] - s.conn_offset[p]));
      node0.push_back(gnode + s.node_offset[p]);
    }
    gnode += s.node_offset[s.np];
  }
  const uint64_t npairs = pair_off.back();
  // scratch (not part of the handle's memory): freed before this returns
  void *t_conn = nullptr, *t_off = nullptr, *t_node0 = nullptr, *t_rowptr = nullptr, *t_cursor = nullptr,
       *t_rows = nullptr;
  auto tfree = [&] {
    for (void *q : {t_conn, t_off, t_node0, t_rowptr, t_cursor, t_rows})
      if (q) cudaFreeAsync(q, stream_);
  };
  auto talloc = [&](void **q, size_t bytes) {
    if (cudaMallocAsync(q, bytes ? bytes : 8, stream_) != cudaSuccess) {
      cudaGetLastError();
      *q = nullptr;
      return false;
    }
    return true;
  };
  if (!talloc(&t_conn, npairs * 8) || !talloc(&t_off, pair_off.size() * 8) ||
      !talloc(&t_node0, node0.size() * 8) || !talloc(&t_rowptr, rowptr.size() * 8) ||
      !talloc(&t_cursor, Ncap_ * 4) || !talloc(&t_rows, initial_bonds_ * 4)) {
    tfree();
    fallback = true;  // no room for the scratch: the host builds the arrays
    return PD_OK;
  }
  int rc = PD_OK;
  {
    uint64_t at = 0;
    for (auto &s : sims_) {
      const uint64_t m = s.conn_offset[s.np];
      if (m && rc == PD_OK)
        rc = check(cudaMemcpyAsync((char *)t_conn + at * 8, s.conn.data(), m * 8, cudaMemcpyHostToDevice,
                                   stream_), "upload Connectivity");
      at += m;
    }
  }
  auto h2d = [&](void *dst, const void *src, size_t bytes, const char *what) {
    if (rc == PD_OK) rc = check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream_), what);
  };
  h2d(t_off, pair_off.data(), pair_off.size() * 8, "upload pair offsets");
  h2d(t_node0, node0.data(), node0.size() * 8, "upload node offsets");
  h2d(t_rowptr, rowptr.data(), rowptr.size() * 8, "upload row starts");
  if (rc == PD_OK) rc = check(cudaMemsetAsync(t_cursor, 0, Ncap_ * 4, stream_), "zero row cursors");
  if (rc == PD_OK) rc = alloc_bond_arrays();
  if (rc == PD_OK) {
    SellBuild b;
    b.conn = (const uint32_t *)t_conn;
    b.npairs = npairs;
    b.pair_off = (const uint64_t *)t_off;
    b.node0 = (const uint64_t *)t_node0;
    b.nparts = (uint32_t)node0.size();
    b.node_of = d_node_of_;
    b.rowptr = (const uint64_t *)t_rowptr;
    b.cursor = (uint32_t *)t_cursor;
    b.rows = (uint32_t *)t_rows;
    b.n_nodes = N_;
    b.slice_ptr = d_slice_ptr_;
    b.nslices = nslices_;
    b.col = d_col_;
    b.mask = d_mask_;
    launch_sell_build(b, stream_);
    rc = check(cudaGetLastError(), "bond build kernels");
  }
  tfree();
  if (rc == PD_OK) rc = check(cudaStreamSynchronize(stream_), "bond build");
  return rc;
}

int Engine::upload_bonds(SellHost &h) {
  const uint64_t ncol = h.ncol, nmask = h.nmask;
  PD_TRY(alloc_bond_arrays());
  PD_TRY(cpy(d_col_, h.col.get(), ncol * 4, "upload col"));
  PD_TRY(cpy(d_mask_, h.mask.get(), nmask * 4, "upload mask"));
  return PD_OK;
}

int Engine::alloc_and_upload() {
  const uint64_t C = Ncap_;
  // The SELL-32 bond arrays: from a sorted Connectivity they are built on the device once the
  // node arrays (node_of among them) are uploaded, the bond counts being computed on a host
  // thread meanwhile; from any other Connectivity the whole build runs on a host thread beside
  // the node arrays' staging and upload.
  SellHost sell;
  int sell_rc = PD_OK;
  auto host_build = [&] {
    try {
      sell_rc = build_bonds_host(sell);
    } catch (const std::bad_alloc &) {  // an exception must not leave the thread
      sell.err = "host memory exhausted while building the bond lists";
      sell_rc = PD_ENOMEM;
    }
  };
  std::vector<uint64_t> rowptr;  // row starts for the device build
  int counts_rc = PD_OK;
  auto counts = [&] {
    try {
      std::vector<uint32_t> deg;
      counts_rc = bond_counts(deg, &rowptr);
    } catch (const std::bad_alloc &) {
      counts_rc = PD_ENOMEM;
    }
  };
  std::thread sell_thread;
  if (!conn_sorted_) sell_thread = std::thread(host_build);
  else sell_thread = std::thread(counts);
  struct Joiner {
    std::thread &t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  } sell_join{sell_thread};
  // [3][Ncap] staging in engine order; every entry is written below (padding nodes zero)
  std::unique_ptr<double[]> pos(new double[3 * C]), disp(new double[3 * C]), vel(new double[3 * C]),
      acc(new double[3 * C]), ext(new double[3 * C]), vol(new double[C]);
  for (uint64_t g = N_; g < C; ++g) {
    for (int c = 0; c < 3; ++c)
      pos[c * C + g] = disp[c * C + g] = vel[c * C + g] = acc[c * C + g] = ext[c * C + g] = 0.0;
    vol[g] = 0.0;
  }
  std::vector<int32_t> part_ext(P_, 0);  // any non-zero extforce in the particle
  h_pid_.assign(C, 0);
  std::vector<uint8_t> bdry(C, 0);
  std::vector<DevPart> parts(P_);
  std::vector<DevSimParams> sps(S_);
  std::vector<DevSimState> sss(S_);
  std::vector<uint32_t> clamped_ptr(P_ + 1, 0), clamped_list, clamped_file;
  h_g0_.assign(P_, 0);
  uint64_t gnode = 0;
  uint32_t gpart = 0;
  torque_possible_ = false;
  double min_half_skin = 1e300;
  for (uint32_t si = 0; si < S_; ++si) {
    HostSim &s = sims_[si];
    const pd_config &cf = s.cfg;
    const uint64_t ns = s.node_offset[s.np];
    parallel_items((ns + 65535) / 65536, [&](uint64_t chunk) {
      const uint64_t k0 = chunk * 65536, k1 = std::min<uint64_t>(ns, k0 + 65536);
      uint32_t p = (uint32_t)(std::upper_bound(s.node_offset.begin(), s.node_offset.begin() + s.np + 1, k0) -
                              s.node_offset.begin() - 1);
      for (uint64_t k = k0; k < k1; ++k) {
        while (k >= s.node_offset[p + 1]) ++p;
        const uint64_t g = node_of_[gnode + k];
        int32_t any = 0;
        for (int c = 0; c < 3; ++c) {
          pos[c * C + g] = s.pos[3 * k + c];
          disp[c * C + g] = s.disp[3 * k + c];
          vel[c * C + g] = s.vel[3 * k + c];
          acc[c * C + g] = s.acc[3 * k + c];
          const double e = s.ext[3 * k + c];
          ext[c * C + g] = e;
          any |= e != 0.0;
        }
        vol[g] = s.vol[k];
        if (any) __atomic_store_n(&part_ext[gpart + p], 1, __ATOMIC_RELAXED);
      }
    });
    for (uint32_t p = 0; p < s.np; ++p) {
      uint32_t gp = gpart + p;
      DevPart &P = parts[gp];
      P.g0 = (uint32_t)(gnode + s.node_offset[p]);
      P.n = (uint32_t)(s.node_offset[p + 1] - s.node_offset[p]);
      max_part_nodes_ = std::max(max_part_nodes_, P.n);
      P.sim = si;
      P.taxis = s.taxis[p];
      P.rho = s.rho[p];
      P.irho = 1 / s.rho[p];
      P.cnot = s.cnot[p];
      P.snot = (cf.new_snot != -1) ? cf.new_snot : s.snot[p];  // timeloop.h:314-318
      P.tval = s.tval[p];
      P.movable = s.movable[p];
      P.breakable = s.breakable[p];
      P.stoppable = s.stoppable[p];
      P.break_bonds = 1;  // simulate3d.cpp:137-139
      P.has_ext = part_ext[gp];
      if (P.n == 0) {
        err = "particle " + std::to_string(p) + " has no nodes";
        return PD_EINVAL;
      }
      h_g0_[gp] = P.g0;
      if (!s.bdry_offset.empty())
        for (uint64_t l = s.bdry_offset[p]; l < s.bdry_offset[p + 1]; ++l) {
          if (s.bdry[l] >= P.n) {
            err = "bdry_nodes index out of range in particle " + std::to_string(p);
            return PD_EINVAL;
          }
          bdry[node_of_[P.g0 + s.bdry[l]]] = 1;
        }
      clamped_ptr[gp + 1] = clamped_ptr[gp];
      if (!s.clamped_offset.empty())
        for (uint64_t l = s.clamped_offset[p]; l < s.clamped_offset[p + 1]; ++l) {
          if (s.clamped[l] >= P.n) {
            err = "clamped_nodes index out of range in particle " + std::to_string(p);
            return PD_EINVAL;
          }
          clamped_list.push_back(node_of_[P.g0 + s.clamped[l]]);
          clamped_file.push_back(P.g0 + s.clamped[l]);
          clamped_ptr[gp + 1]++;
        }
    }
    // Contact: setup values, then Contact::apply_config overrides (contact.h:151-179)
    DevSimParams &sp = sps[si];
    std::memset(&sp, 0, sizeof(sp));
    double Kn = s.Kn, zeta = s.zeta, mu = s.mu;
    if (cf.damping_ratio != -1) zeta = cf.damping_ratio;
    if (cf.friction_coefficient != -1) mu = cf.friction_coefficient;
    if (cf.normal_stiffness != -1) Kn = cf.normal_stiffness;
    sp.dt = cf.dt;
    sp.hdt2 = (cf.dt * cf.dt) * 0.5;
    sp.hdt = 0.5 * cf.dt;
    sp.Rc = s.Rc;
    sp.rc2_far = (s.Rc * s.Rc) * (1.0 + 1e-12);
    sp.Kn = Kn;
    sp.sc = Kn * s.Rc;
    sp.zeta2 = 2 * zeta;
    sp.mu = mu;
    sp.pi3 = M_PI / 3;
    sp.pi4 = M_PI / 4;
    const double skin = bp_.skin_frac * s.Rc;
    const double rcand = (s.Rc + skin) * (1.0 + 1e-9);
    sp.cell = rcand * (1.0 + 1e-9);
    sp.inv_cell = 1.0 / sp.cell;
    sp.cand_r2 = rcand * rcand;
    min_half_skin = std::min(min_half_skin, 0.5 * skin);
    sp.nl_bdry_only = cf.nl_bdry_only;
    sp.compute_wall_reaction = cf.compute_wall_reaction;
    sp.gradient_extforce = cf.gradient_extforce;
    sp.allow_wall = s.allow_wall ? 1 : 0;
    sp.extforce_maxstep = cf.extforce_maxstep;
    sp.set_torque_ts = cf.set_torque_timestep;
    sp.set_fracture_ts = cf.set_fracture_timestep;
    sp.set_self_contact_ts = cf.set_self_contact_timestep;
    sp.set_damping_ts = cf.set_damping_timestep;
    sp.set_zero_wall_speed_ts = cf.set_zero_wall_speed_timestep;
    sp.set_movable_index = cf.set_movable_index;
    sp.set_movable_ts = cf.set_movable_timestep;
    sp.set_stoppable_index = cf.set_stoppable_index;
    sp.set_stoppable_ts = cf.set_stoppable_timestep;
    sp.p0 = gpart;
    sp.np = s.np;
    sp.node0 = gnode;
    sp.nnodes = ns;
    // prescribed velocity and reset_partzero_y (timeloop.h:412-420, 500-535, 684-764)
    sp.pv_particle = (cf.particle_w_fixed_velocity >= 0 && (uint32_t)cf.particle_w_fixed_velocity < s.np)
                         ? cf.particle_w_fixed_velocity
                         : -1;
    sp.set_fix_velocity_ts = cf.set_fix_velocity_timestep;
    sp.fix_mean_x = cf.fix_velocity_mean_x;
    sp.fix_angular = cf.fix_velocity_angular;
    sp.pv_mean_x = cf.prescribed_velocity_mean_x;
    sp.pv_angular = cf.prescribed_angular_vel;
    sp.reset_y = (cf.reset_partzero_y && s.np >= 2) ? 1 : 0;
    sp.reset_y_ts = cf.reset_partzero_y_timestep;
    sp.wheel_rad = cf.wheel_rad;
    if (sp.pv_particle >= 0) pv_possible_ = true;
    if (sp.reset_y) reset_possible_ = true;
    // Wall: load_wall<3> then RectWall::apply_config (contact.h:325-372)
    DevSimState &st = sss[si];
    std::memset(&st, 0, sizeof(st));
    for (int c = 0; c < 6; ++c) st.wall[c] = (s.n_geom_wall != 1) ? s.geom[c] : 0.0;
    if (cf.wall_top != -999) st.wall[5] = cf.wall_top;
    if (cf.wall_right != -999) st.wall[4] = cf.wall_right;
    if (cf.wall_x_min != -999) st.wall[0] = cf.wall_x_min;
    if (cf.wall_y_min != -999) st.wall[1] = cf.wall_y_min;
    if (cf.wall_z_min != -999) st.wall[2] = cf.wall_z_min;
    if (cf.wall_x_max != -999) st.wall[3] = cf.wall_x_max;
    if (cf.wall_y_max != -999) st.wall[4] = cf.wall_y_max;
    if (cf.wall_z_max != -999) st.wall[5] = cf.wall_z_max;
    st.spd[0] = cf.speed_wall_x_min;
    st.spd[1] = cf.speed_wall_y_min;
    st.spd[2] = cf.speed_wall_z_min;
    st.spd[3] = cf.speed_wall_x_max;
    st.spd[4] = cf.speed_wall_y_max;
    st.spd[5] = cf.speed_wall_z_max;
    st.extf_scale = 1.0;
    st.t = 1;
    st.fracture = cf.enable_fracture;
    st.self_contact = cf.self_contact;
    st.damping = cf.allow_damping;
    st.friction = cf.allow_friction;
    st.torque = cf.enable_torque;
    st.active = 1;
    host_sim_toggles(sp, st, 1);
    for (uint32_t p = 0; p < s.np; ++p) {
      DevPart &P = parts[gpart + p];
      if (cf.set_movable_index != -1 && (uint32_t)cf.set_movable_index == p && (uint32_t)cf.set_movable_timestep == 1u)
        P.movable = 1;
      if (cf.set_stoppable_index != -1 && (uint32_t)cf.set_stoppable_index == p &&
          (uint32_t)cf.set_stoppable_timestep == 1u)
        P.stoppable = 1;
    }
    if (cf.enable_torque || cf.set_torque_timestep != -1) torque_possible_ = true;
    gnode += ns;
    gpart += s.np;
  }
  half_skin_ = min_half_skin;

  parallel_items(P_, [&](uint64_t gp) {  // particle of each node
    for (uint32_t k = 0; k < parts[gp].n; ++k) h_pid_[parts[gp].g0 + k] = (uint32_t)gp;
  });
  PD_TRY(dalloc(this, allocs_, &d_pos_, 3 * C, err));
  PD_TRY(dalloc(this, allocs_, &d_disp_, 3 * C, err));
  PD_TRY(dalloc(this, allocs_, &d_vel_[0], 3 * C, err));
  PD_TRY(dalloc(this, allocs_, &d_vel_[1], 3 * C, err));
  PD_TRY(dalloc(this, allocs_, &d_acc_, 3 * C, err));
  PD_TRY(dalloc(this, allocs_, &d_force_, 3 * C, err));
  PD_TRY(dalloc(this, allocs_, &d_ext_, 3 * C, err));
  PD_TRY(dalloc(this, allocs_, &d_vol_, C, err));
  PD_TRY(dalloc(this, allocs_, &d_pid_, C, err));
  PD_TRY(dalloc(this, allocs_, &d_node_of_, C, err));
  PD_TRY(dalloc(this, allocs_, &d_file_of_, C, err));
  PD_TRY(dalloc(this, allocs_, &d_bdry_, C, err));
  PD_TRY(dalloc(this, allocs_, &d_parts_, P_, err));
  PD_TRY(dalloc(this, allocs_, &d_lrtb_, 6ull * P_, err));
  PD_TRY(dalloc(this, allocs_, &d_lrtb_next_, 6ull * P_, err));
  PD_TRY(dalloc(this, allocs_, &d_centroid_, 3ull * P_, err));
  PD_TRY(dalloc(this, allocs_, &d_sp_, S_, err));
  PD_TRY(dalloc(this, allocs_, &d_ss_, S_, err));
  PD_TRY(dalloc(this, allocs_, &d_cnt_, 1, err));
  // FP32 form: each particle's records are relative to an anchor node, the node nearest the
  // centre of the particle's box (the FP32 rounding of a record grows with its distance from the
  // anchor); ext_p bounds the reference positions' rounding (set_break_band). xi_min is measured
  // on the device once the bonds are built.
  parallel_items(P_, [&](uint64_t k) {
    DevPart &P = parts[k];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint64_t g = P.g0; g < (uint64_t)P.g0 + P.n; ++g)
      for (int c = 0; c < 3; ++c) {
        lo[c] = std::min(lo[c], pos[c * C + g]);
        hi[c] = std::max(hi[c], pos[c * C + g]);
      }
    double best = INFINITY;
    uint32_t a = P.g0;
    for (uint64_t g = P.g0; g < (uint64_t)P.g0 + P.n; ++g) {
      double d2 = 0;
      for (int c = 0; c < 3; ++c) {
        const double d = pos[c * C + g] - 0.5 * (lo[c] + hi[c]);
        d2 += d * d;
      }
      if (d2 < best) {
        best = d2;
        a = (uint32_t)g;
      }
    }
    P.anchor = a;
    double ep = 0;
    for (int c = 0; c < 3; ++c) P.anchor_pos[c] = pos[c * C + a];
    for (uint64_t g = P.g0; g < (uint64_t)P.g0 + P.n; ++g)
      for (int c = 0; c < 3; ++c) ep = std::max(ep, std::fabs(pos[c * C + g] - P.anchor_pos[c]));
    P.ext_p = ep;
    P.xi_min = INFINITY;
    P.snot_lo32 = (float)P.snot;
    P.snot_hi32 = (float)P.snot;
  });
  auto up = [&](void *d, const void *h, size_t b, const char *w) { return cpy(d, h, b, w); };
  PD_TRY(up(d_pos_, pos.get(), 3 * C * 8, "upload pos"));
  PD_TRY(up(d_disp_, disp.get(), 3 * C * 8, "upload disp"));
  PD_TRY(up(d_vel_[0], vel.get(), 3 * C * 8, "upload vel"));
  PD_TRY(up(d_vel_[1], vel.get(), 3 * C * 8, "upload vel"));
  PD_TRY(up(d_acc_, acc.get(), 3 * C * 8, "upload acc"));
  PD_TRY(mset(d_force_, 0, 3 * C * 8, "memset force"));
  PD_TRY(up(d_ext_, ext.get(), 3 * C * 8, "upload extforce"));
  PD_TRY(up(d_vol_, vol.get(), C * 8, "upload vol"));
  PD_TRY(up(d_pid_, h_pid_.data(), C * 4, "upload pid"));
  {
    std::vector<uint32_t> no(C), fo(C);
    for (uint64_t g = 0; g < C; ++g) {
      no[g] = g < N_ ? node_of_[g] : (uint32_t)g;
      fo[g] = g < N_ ? file_of_[g] : (uint32_t)g;
    }
    PD_TRY(up(d_node_of_, no.data(), C * 4, "upload node order"));
    PD_TRY(up(d_file_of_, fo.data(), C * 4, "upload node order"));
  }
  PD_TRY(up(d_bdry_, bdry.data(), C, "upload bdry"));
  PD_TRY(up(d_parts_, parts.data(), P_ * sizeof(DevPart), "upload particles"));
  PD_TRY(up(d_sp_, sps.data(), S_ * sizeof(DevSimParams), "upload sim params"));
  PD_TRY(up(d_ss_, sss.data(), S_ * sizeof(DevSimState), "upload sim state"));
  PD_TRY(mset(d_centroid_, 0, 3ull * P_ * 8, "memset centroid"));
  DevCounters cnt;
  std::memset(&cnt, 0, sizeof(cnt));
  cnt.moved = 1e300;  // forces the first broad-phase build
  PD_TRY(up(d_cnt_, &cnt, sizeof(cnt), "upload counters"));
  n_clamped_ = clamped_list.size();
  if (n_clamped_) {
    std::vector<uint32_t> cl(clamped_ptr);
    cl.insert(cl.end(), clamped_list.begin(), clamped_list.end());
    PD_TRY(dalloc(this, allocs_, &d_clamped_, cl.size(), err));
    PD_TRY(up(d_clamped_, cl.data(), cl.size() * 4, "upload clamped"));
    PD_TRY(dalloc(this, allocs_, &d_clamped_disp_, 3 * n_clamped_, err));
    h_clamped_ = clamped_file;
  }

  if (pv_possible_) {
    PD_TRY(dalloc(this, allocs_, &d_afd_, 3 * C, err));
    PD_TRY(mset(d_afd_, 0, 3 * C * 8, "memset applied force density"));
  }

  bool host_bonds = !conn_sorted_;
  if (conn_sorted_) {
    sell_thread.join();
    if (counts_rc != PD_OK) {
      err = counts_rc == PD_ENOMEM ? "host memory exhausted while counting bonds"
                                   : "node degree above 65535";
      return counts_rc;
    }
    bool fallback = false;
    PD_TRY(build_bonds_gpu(rowptr, fallback));
    if (fallback) {  // no device room for the build's scratch
      host_bonds = true;
      host_build();
    }
  } else {
    sell_thread.join();
  }
  if (host_bonds) {
    if (sell_rc != PD_OK) {
      err = sell.err;
      return sell_rc;
    }
    PD_TRY(upload_bonds(sell));
  }

  if (precision_ == PD_FP64) {
    PD_TRY(dalloc(this, allocs_, &d_bxi_, 3 * std::max<uint64_t>(E_, 1), err));
    PD_TRY(dalloc(this, allocs_, &d_bxin_, std::max<uint64_t>(E_, 1), err));
    PD_TRY(dalloc(this, allocs_, &d_brxin_, std::max<uint64_t>(E_, 1), err));
  } else {
    std::unique_ptr<Rec32[]> r32(new Rec32[C]);  // every entry written below
    parallel_items((C + 65535) / 65536, [&](uint64_t chunk) {
      for (uint64_t g = chunk * 65536; g < std::min<uint64_t>(C, chunk * 65536 + 65536); ++g) {
        Rec32 &r = r32[g];
        r.u = make_float4(0.f, 0.f, 0.f, 0.f);
        if (g < N_) {
          const DevPart &P = parts[h_pid_[g]];
          // the bond kernels' force coefficient of this node as a partner: cnot * volume (a
          // bond's partner is in the same particle)
          r.p = make_float4((float)(pos[g] - P.anchor_pos[0]), (float)(pos[C + g] - P.anchor_pos[1]),
                            (float)(pos[2 * C + g] - P.anchor_pos[2]), (float)(P.cnot * vol[g]));
        } else {
          r.p = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
    });
    for (int b = 0; b < 2; ++b) {
      PD_TRY(dalloc(this, allocs_, &d_rec_[b], C, err));
      if (reinterpret_cast<uintptr_t>(d_rec_[b]) % 32) {  // the bond kernel reads records with 256-bit loads
        err = "node records not 32-byte aligned";
        return PD_ECUDA;
      }
      PD_TRY(up(d_rec_[b], r32.get(), C * sizeof(Rec32), "upload rec32"));
    }
    d_dispb_[0] = d_disp_;
    PD_TRY(dalloc(this, allocs_, &d_dispb_[1], 3 * C, err));
    PD_TRY(dalloc(this, allocs_, &d_anchor_, 3ull * P_, err));
    PD_TRY(dalloc(this, allocs_, &d_anchor_next_, 3ull * P_, err));
    {
      std::vector<uint8_t> cf(C, 0);
      for (uint32_t g : clamped_list) cf[g] = 1;
      PD_TRY(dalloc(this, allocs_, &d_clamp_flag_, C, err));
      PD_TRY(up(d_clamp_flag_, cf.data(), C, "upload clamp flags"));
    }
    PD_TRY(dalloc(this, allocs_, &d_f_extra_, 3 * C, err));
    PD_TRY(dalloc(this, allocs_, &d_extra_flag_, C, err));
    PD_TRY(dalloc(this, allocs_, &d_wall_local_, 6ull * P_, err));
    PD_TRY(dalloc(this, allocs_, &d_lrtb_local_, 6ull * P_, err));
    PD_TRY(mset(d_extra_flag_, 0, C, "memset extra flag"));
  }

  // broad phase
  uint32_t bits = 10;
  while ((1ull << bits) < 2 * N_) ++bits;
  if (bits > 31) {
    err = "too many nodes for the broad-phase cell table";
    return PD_EINVAL;
  }
  bp_.table_bits = bits;
  const uint64_t T = 1ull << bits;
  if (bp_.cand_cap == 0) bp_.cand_cap = 32;
  PD_TRY(dalloc(this, allocs_, &bp_.count, T, err));
  PD_TRY(dalloc(this, allocs_, &bp_.start, T, err));
  PD_TRY(dalloc(this, allocs_, &bp_.key, C, err));
  PD_TRY(dalloc(this, allocs_, &bp_.slot, C, err));
  PD_TRY(dalloc(this, allocs_, &bp_.sorted, C, err));
  PD_TRY(dalloc(this, allocs_, &bp_.block_sums, (T + 4095) / 4096 + 1, err));
  if (precision_ == PD_FP32C) {
    PD_TRY(dalloc(this, allocs_, &bp_.xnodes, C, err));
    PD_TRY(dalloc(this, allocs_, &bp_.xparts, P_, err));
    PD_TRY(dalloc(this, allocs_, &bp_.xcount, 2, err));
    PD_TRY(mset(bp_.xcount, 0, 8, "work lists"));
  }
  PD_TRY(alloc_candidates());

  if (precision_ == PD_FP64) {
    DevView v = view(0);
    launch_bond_constants(v, d_bxi_, d_bxin_, d_brxin_, stream_);
    launch_init_lrtb(v, stream_);
    PD_TRY(check(cudaGetLastError(), "init kernels"));
  } else {
    // each particle's shortest bond, for the breaking band that prepare_fused sets
    unsigned long long *d2min = nullptr;
    PD_TRY(check(cudaMallocAsync((void **)&d2min, 8ull * std::max<uint32_t>(P_, 1), stream_), "xi_min scratch"));
    int rc = check(cudaMemsetAsync(d2min, 0xFF, 8ull * P_, stream_), "xi_min scratch");
    if (rc == PD_OK) {
      launch_xi_min(view(0), d2min, stream_);
      rc = check(cudaGetLastError(), "xi_min");
    }
    cudaFreeAsync(d2min, stream_);
    PD_TRY(rc);
    cur_ = 1;
    PD_TRY(prepare_fused(cur_));
  }
  PD_TRY(check(cudaStreamSynchronize(stream_), "init sync"));
  return PD_OK;
}

// FP32 form: disp[cur^1] holds the displacement of the last completed step (or the initial
// one); derive this step's AABBs, anchors and wall frames from it, then run the predictor
// into disp[cur]/rec[cur] and set the anchors of the next step's records.
int Engine::prepare_fused(int cur) {
  // AABBs from pos + disp (timeloop.h:389-393), anchors := disp of each anchor node, walls in
  // the anchors' frame
  launch_init_lrtb(view(cur ^ 1), stream_);
  PD_TRY(check(cudaMemcpyAsync(d_dispb_[cur], d_dispb_[cur ^ 1], 3 * Ncap_ * 8, cudaMemcpyDeviceToDevice, stream_),
               "copy disp"));
  DevView v = view(cur);
  launch_predict(v, tpb_, stream_);
  launch_anchor_next(v, stream_);
  // the next step's non-bond kernel visits every node (the work lists are rebuilt by then)
  PD_TRY(check(cudaMemsetAsync(&d_cnt_->xall, 1, sizeof(uint32_t), stream_), "work lists"));
  return check(cudaGetLastError(), "prepare fused");
}

int Engine::alloc_candidates() {
  if (bp_.cand) {
    cudaFreeAsync(bp_.cand, stream_);
    cudaFreeAsync(bp_.cand_n, stream_);
    device_bytes_ -= cand_bytes_;
    allocs_.erase(std::remove(allocs_.begin(), allocs_.end(), (void *)bp_.cand), allocs_.end());
    allocs_.erase(std::remove(allocs_.begin(), allocs_.end(), (void *)bp_.cand_n), allocs_.end());
    bp_.cand = nullptr;
    bp_.cand_n = nullptr;
  }
  PD_TRY(dalloc(this, allocs_, &bp_.cand, Ncap_ * bp_.cand_cap, err));
  PD_TRY(dalloc(this, allocs_, &bp_.cand_n, Ncap_, err));
  cand_bytes_ = Ncap_ * bp_.cand_cap * 4 + Ncap_ * 2;
  PD_TRY(mset(bp_.cand_n, 0, Ncap_ * 2, "memset cand_n"));
  return PD_OK;
}

int Engine::launch_step_seq(int cur, cudaStream_t s) {
  DevView v = view(cur);
  if (reset_possible_) launch_reset_y(v, s);
  if (precision_ == PD_FP64) launch_predict(v, tpb_, s);
  if (torque_possible_) launch_centroids(v, s);
  launch_bp_decide(v, half_skin_, s);
  launch_broadphase(v, bp_, s);
  launch_step_kernel(v, precision_, variant_, s);
  if (pv_possible_) launch_prescribed(v, s);
  if (stats_) launch_pairwise_count(v, s);
  launch_end_step(v, d_clamped_, n_clamped_, d_clamped_disp_, s);
  return check(cudaGetLastError(), "step launch");
}

int Engine::capture_conditional(int cur, cudaGraphExec_t *out) {
  cudaStream_t cs = capture_stream_;
  DevView v = view(cur);
  // the rebuild kernels as a graph of their own
  cudaGraph_t gb = nullptr, g = nullptr;
  PD_TRY(check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture"));
  launch_broadphase(v, bp_, cs);
  PD_TRY(check(cudaStreamEndCapture(cs, &gb), "end capture"));
  cudaError_t e = cudaGraphCreate(&g, 0);
  cudaGraphConditionalHandle h = 0;
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
  if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  bool capturing = e == cudaSuccess;
  if (capturing) {
    if (reset_possible_) launch_reset_y(v, cs);
    if (precision_ == PD_FP64) launch_predict(v, tpb_, cs);
    if (torque_possible_) launch_centroids(v, cs);
    launch_bp_decide(v, half_skin_, cs, h);
    cudaStreamCaptureStatus st;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *ed = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(cs, &st, nullptr, nullptr, &deps, &ed, &nd);
    std::vector<cudaGraphNode_t> dv(deps, deps + nd);
    cudaGraphNode_t cond = nullptr;
    if (e == cudaSuccess) {
      // zeroed storage: the struct's union makes its default constructor unavailable
      alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
      std::memset(raw, 0, sizeof(raw));
      cudaGraphNodeParams &cp = *reinterpret_cast<cudaGraphNodeParams *>(raw);
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeIf;
      cp.conditional.size = 1;
      e = cudaGraphAddNode(&cond, g, dv.data(), nullptr, dv.size(), &cp);
      if (e == cudaSuccess) {
        cudaGraphNode_t child;
        e = cudaGraphAddChildGraphNode(&child, cp.conditional.phGraph_out[0], nullptr, 0, gb);
      }
    }
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(cs, &cond, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e == cudaSuccess) {
      launch_step_kernel(v, precision_, variant_, cs);
      if (pv_possible_) launch_prescribed(v, cs);
      if (stats_) launch_pairwise_count(v, cs);
      launch_end_step(v, d_clamped_, n_clamped_, d_clamped_disp_, cs);
    }
    cudaGraph_t done = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cs, &done);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
  if (g) cudaGraphDestroy(g);
  cudaGraphDestroy(gb);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return PD_ECUDA;
  }
  return PD_OK;
}

int Engine::capture_graphs() {
  for (int i = 0; i < 2; ++i) {
    if (graph_[i]) {
      cudaGraphExecDestroy(graph_[i]);
      graph_[i] = nullptr;
    }
  }
  bool cond_ok = use_conditional_;
  for (int i = 0; i < 2 && cond_ok; ++i)
    if (capture_conditional(i, &graph_[i]) != PD_OK) cond_ok = false;
  if (cond_ok) {
    graphs_ok_ = true;
    return PD_OK;
  }
  for (int i = 0; i < 2; ++i) {
    if (graph_[i]) {
      cudaGraphExecDestroy(graph_[i]);
      graph_[i] = nullptr;
    }
  }
  use_conditional_ = false;
  for (int i = 0; i < 2; ++i) {
    cudaGraph_t g;
    PD_TRY(check(cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal), "begin capture"));
    int rc = launch_step_seq(i, capture_stream_);
    cudaError_t e = cudaStreamEndCapture(capture_stream_, &g);
    if (rc != PD_OK) return rc;
    PD_TRY(check(e, "end capture"));
    e = cudaGraphInstantiate(&graph_[i], g, 0);
    cudaGraphDestroy(g);
    PD_TRY(check(e, "graph instantiate"));
  }
  graphs_ok_ = true;
  return PD_OK;
}

// Steps per persistent launch: a launch of a small handle stays within tens of milliseconds.
constexpr uint32_t kPersistMaxSteps = 1024;

int Engine::launch_persist_steps(uint32_t n) {
  if (persist_grid_lanes_ != persist_lanes_ + 1) {  // (re)size the grid for these lanes
    if (persist_lanes_ == 0) {  // four lanes per node where all threads fit at once, else one
      const uint64_t resident = (uint64_t)persist_threads() * (uint64_t)std::max(0, persist_max_blocks(4));
      persist_kernel_lanes_ = 4 * N_ <= resident ? 4 : 1;
    } else {
      persist_kernel_lanes_ = persist_lanes_;
    }
    const int mb = persist_max_blocks(persist_kernel_lanes_);
    if (mb <= 0) {
      err = "persistent step: no resident blocks";
      return PD_ECUDA;
    }
    const uint64_t warps = (N_ * (uint64_t)persist_kernel_lanes_ + 31) / 32;
    // one block per SM, or fewer where the handle has fewer warps of work than SMs
    persist_blocks_ = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)mb, warps));
    persist_grid_lanes_ = persist_lanes_ + 1;
  }
  int dev = 0, sms = 0;
  PD_TRY(check(cudaGetDevice(&dev), "device"));
  PD_TRY(check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"));
  // two barrier words + one scan word per block; a block holds at least 32 threads, an SM 2048
  const uint64_t max_blocks = 64ull * (uint64_t)sms;
  if (!persist_ws_) PD_TRY(dalloc(this, allocs_, &persist_ws_, 2 + max_blocks, err));
  if (persist_blocks_ > max_blocks) {
    err = "persistent step: grid larger than its scratch";
    return PD_ECUDA;
  }
  PersistArgs a;
  a.v[0] = view(0);
  a.v[1] = view(1);
  a.cur0 = (uint32_t)cur_;
  a.nsteps = n;
  a.half_skin = half_skin_;
  a.count = bp_.count;
  a.start = bp_.start;
  a.key = bp_.key;
  a.slot = bp_.slot;
  a.sorted = bp_.sorted;
  a.bar = persist_ws_;
  a.sums = persist_ws_ + 2;
  a.T = 1ull << bp_.table_bits;
  a.mask = (uint32_t)(a.T - 1);
  a.cand = bp_.cand;
  a.cand_n = bp_.cand_n;
  a.cap = bp_.cand_cap;
  a.clamped_ptr = n_clamped_ ? d_clamped_ : nullptr;
  a.clamped = n_clamped_ ? d_clamped_ + (P_ + 1) : nullptr;
  a.clamped_disp = d_clamped_disp_;
  PD_TRY(check(cudaMemsetAsync(persist_ws_, 0, 8, stream_), "persistent barrier reset"));
  PD_TRY(check(launch_persist(a, persist_blocks_, persist_kernel_lanes_, stream_), "persistent step launch"));
  cur_ ^= (int)(n & 1);
  steps_done_ += n;
  return PD_OK;
}

int Engine::step(uint32_t nsteps) {
  if (grow_cand_) {  // some node walked the cell list since the last grow: longer lists from now on
    grow_cand_ = false;
    const uint32_t cap = std::min<uint32_t>(kMaxCandCap, 2 * bp_.cand_cap);
    if (cap > bp_.cand_cap) PD_TRY(set_tuning(0.0, cap, 0, -1, -1));
    uint32_t z = 0;
    PD_TRY(cpy(&d_cnt_->cand_cells, &z, 4, "reset cell-walk count"));
  }
  if (use_persist_ && persist_eligible()) {
    for (uint32_t done = 0; done < nsteps;) {
      const uint32_t n = std::min(nsteps - done, kPersistMaxSteps);
      PD_TRY(launch_persist_steps(n));
      done += n;
    }
    for (uint32_t i = 0; i < S_; ++i)
      if (!finished_[i]) sim_steps_[i] += nsteps;
    return PD_OK;
  }
  if (!graphs_ok_ && use_graphs_) PD_TRY(capture_graphs());
  for (uint32_t i = 0; i < nsteps; ++i) {
    if (use_graphs_) {
      PD_TRY(check(cudaGraphLaunch(graph_[cur_], stream_), "graph launch"));
    } else {
      PD_TRY(launch_step_seq(cur_, stream_));
    }
    cur_ ^= 1;
    ++steps_done_;
  }
  for (uint32_t i = 0; i < S_; ++i)
    if (!finished_[i]) sim_steps_[i] += nsteps;
  return PD_OK;
}

int Engine::sync(int timeout_ms) {
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(stream_);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) return check(e, "stream");
    if (timeout_ms == 0) {
      err = "pd_sync: work still queued";
      return PD_ETIMEOUT;
    }
    if (timeout_ms > 0) {
      auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
      if (ms > timeout_ms) {
        err = "pd_sync: timed out after " + std::to_string(timeout_ms) + " ms";
        return PD_ETIMEOUT;
      }
    }
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  DevCounters c;
  PD_TRY(cpy(&c, d_cnt_, sizeof(c), "read counters"));
  if (c.cand_cells && bp_.cand_cap < kMaxCandCap) grow_cand_ = true;
  if (c.err) {
    err = "device error word 0x" + std::to_string(c.err);
    if (c.err & PD_DERR_NONFINITE) err += " (non-finite force density)";
    return PD_EDEVICE;
  }
  return PD_OK;
}

int Engine::set_stream(cudaStream_t s) {
  PD_TRY(sync(-1));
  if (s == nullptr) {
    stream_ = capture_stream_;
  } else {
    stream_ = s;
  }
  return PD_OK;
}

void Engine::rows_to_file(const double *src, uint64_t stride, uint64_t node0, uint64_t nn, double *dst) const {
  parallel_items((nn + 65535) / 65536, [&](uint64_t chunk) {
    for (uint64_t k = chunk * 65536; k < std::min<uint64_t>(nn, chunk * 65536 + 65536); ++k) {
      const uint64_t f = file_of_[node0 + k] - node0;
      for (int c = 0; c < 3; ++c) dst[3 * f + c] = src[c * stride + k];
    }
  });
}

int Engine::get_state(double *curpos, double *vel, double *acc, double *force, double *disp) {
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  // each array put in file order on the device, then copied straight to the caller
  double *rows = nullptr;
  if (cudaMallocAsync((void **)&rows, std::max<uint64_t>(3 * N_, 1) * 8, stream_) != cudaSuccess) {
    cudaGetLastError();
    return get_state_host(curpos, vel, acc, force, disp);  // no room for the scratch
  }
  const bool fused = precision_ == PD_FP32C;
  const double *dcur = fused ? d_dispb_[cur_ ^ 1] : d_disp_;
  const uint32_t *clist = n_clamped_ ? d_clamped_ + (P_ + 1) : nullptr;
  // Large handles copy through a pinned staging buffer and fill the caller's (pageable) arrays
  // from it on all host cores: a pageable device-to-host copy runs at a few GB/s.
  if (N_ >= kPinnedStageNodes && !h_stage_ && cudaMallocHost((void **)&h_stage_, 3 * N_ * 8) != cudaSuccess) {
    cudaGetLastError();
    h_stage_ = nullptr;
  }
  int rc = PD_OK;
  auto out = [&](const double *src, const double *add, int clamped_mode, double *dst) {
    if (!dst || rc != PD_OK) return;
    launch_rows_to_file(src, add, Ncap_, N_, d_file_of_, rows, stream_);
    if (clamped_mode == 1) launch_clamped_rows(clist, n_clamped_, d_file_of_, nullptr, nullptr, Ncap_, rows, stream_);
    if (clamped_mode == 2)
      launch_clamped_rows(clist, n_clamped_, d_file_of_, d_pos_, d_clamped_disp_, Ncap_, rows, stream_);
    rc = check(cudaGetLastError(), "read state");
    double *to = h_stage_ ? h_stage_ : dst;
    if (rc == PD_OK) rc = check(cudaMemcpyAsync(to, rows, 3 * N_ * 8, cudaMemcpyDeviceToHost, stream_), "read state");
    if (rc == PD_OK) rc = check(cudaStreamSynchronize(stream_), "read state");
    if (rc == PD_OK && h_stage_) {
      const uint64_t n = 3 * N_, chunk = 1ull << 17;  // 1 MB per item
      parallel_items((n + chunk - 1) / chunk, [&](uint64_t i) {
        const uint64_t a = i * chunk, b = std::min(n, a + chunk);
        std::memcpy(dst + a, h_stage_ + a, (b - a) * 8);
      });
    }
  };
  const bool stepped = steps_done_ > 0 && n_clamped_;
  // clamped nodes end each step at zero (timeloop.h:767-774); the FP64 form's CurrPos keeps
  // their predicted displacement (the FP32 form's displacement buffer already holds it)
  out(dcur, nullptr, fused && stepped ? 1 : 0, disp);
  out(dcur, d_pos_, !fused && stepped ? 2 : 0, curpos);
  out(d_vel_[cur_], nullptr, 0, vel);
  out(d_acc_, nullptr, 0, acc);
  out(d_force_, nullptr, 0, force);
  cudaFreeAsync(rows, stream_);
  return rc;
}

int Engine::get_state_host(double *curpos, double *vel, double *acc, double *force, double *disp) {
  const uint64_t C = Ncap_;
  std::unique_ptr<double[]> buf(new double[3 * C]);  // staging, overwritten by each copy
  auto scatter = [&](double *dst) { rows_to_file(buf.get(), C, 0, N_, dst); };
  auto fetch = [&](const double *d, double *dst) -> int {
    PD_TRY(cpy(buf.get(), d, 3 * C * 8, "read state"));
    scatter(dst);
    return PD_OK;
  };
  if (curpos || disp) {
    std::unique_ptr<double[]> dsp_buf(new double[3 * N_]);  // every entry written by fetch
    double *dsp = dsp_buf.get();
    const bool fused = precision_ == PD_FP32C;
    PD_TRY(fetch(fused ? d_dispb_[cur_ ^ 1] : d_disp_, dsp));
    if (disp) {
      std::memcpy(disp, dsp, 3 * N_ * 8);
      if (fused && steps_done_ > 0)  // clamped nodes end each step at zero (timeloop.h:767-774)
        for (uint32_t g : h_clamped_)
          for (int c = 0; c < 3; ++c) disp[3 * (uint64_t)g + c] = 0.0;
    }
    if (curpos) {
      if (n_clamped_ && steps_done_ > 0 && !fused) {
        // CurrPos of clamped nodes keeps the predicted displacement (zeroed afterwards)
        std::vector<double> cd(3 * n_clamped_);
        PD_TRY(cpy(cd.data(), d_clamped_disp_, 3 * n_clamped_ * 8, "read clamped"));
        for (uint64_t i = 0; i < n_clamped_; ++i)
          for (int c = 0; c < 3; ++c) dsp[3 * (uint64_t)h_clamped_[i] + c] = cd[3 * i + c];
      }
      if (reset_possible_) {  // reset_partzero_y moves reference positions on the device
        std::vector<double> p(3 * N_);
        PD_TRY(fetch(d_pos_, p.data()));
        for (uint64_t k = 0; k < 3 * N_; ++k) curpos[k] = p[k] + dsp[k];
      } else {
        uint64_t off = 0;
        for (auto &s : sims_) {
          const uint64_t n3 = 3 * s.node_offset[s.np];
          const double *sp = s.pos.data(), *dp = dsp + 3 * off;
          double *cp = curpos + 3 * off;
          parallel_items((n3 + 65535) / 65536, [&](uint64_t chunk) {
            for (uint64_t k = chunk * 65536; k < std::min<uint64_t>(n3, chunk * 65536 + 65536); ++k)
              cp[k] = sp[k] + dp[k];
          });
          off += n3 / 3;
        }
      }
    }
  }
  if (vel) PD_TRY(fetch(d_vel_[cur_], vel));
  if (acc) PD_TRY(fetch(d_acc_, acc));
  if (force) PD_TRY(fetch(d_force_, force));
  return PD_OK;
}

int Engine::set_state(const double *disp, const double *vel, const double *acc) {
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  const uint64_t C = Ncap_;
  std::vector<double> buf(3 * C, 0.0);
  auto put = [&](double *d, const double *src) -> int {
    for (uint64_t n = 0; n < N_; ++n)
      for (int c = 0; c < 3; ++c) buf[c * C + node_of_[n]] = src[3 * n + c];
    return cpy(d, buf.data(), 3 * C * 8, "write state");
  };
  const bool fused = precision_ == PD_FP32C;
  if (disp) PD_TRY(put(fused ? d_dispb_[cur_ ^ 1] : d_disp_, disp));
  if (vel) PD_TRY(put(d_vel_[cur_], vel));
  if (acc) PD_TRY(put(d_acc_, acc));
  // a resumed state re-derives CurrPos/AABBs (timeloop.h:389-393) and the contact lists
  if (fused) {
    PD_TRY(prepare_fused(cur_));
  } else {
    launch_init_lrtb(view(cur_), stream_);
  }
  double big = 1e300;
  PD_TRY(cpy(&d_cnt_->moved, &big, 8, "force rebuild"));
  return check(cudaStreamSynchronize(stream_), "set_state");
}

int Engine::get_connectivity(uint32_t particle, uint32_t *pairs, uint64_t cap, uint64_t *n) {
  if (particle >= P_) {
    err = "particle index out of range";
    return PD_EINVAL;
  }
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  const uint64_t g0 = h_g0_[particle];
  uint64_t nloc = 0;
  {
    uint64_t off = 0;
    uint32_t pacc = 0;
    for (auto &s : sims_) {
      if (particle < pacc + s.np) {
        uint32_t p = particle - pacc;
        nloc = s.node_offset[p + 1] - s.node_offset[p];
        break;
      }
      pacc += s.np;
      off += s.node_offset[s.np];
    }
  }
  const uint64_t s0 = g0 >> 5, s1 = (g0 + nloc + 31) >> 5;
  const uint64_t e0 = h_slice_ptr_[s0], e1 = h_slice_ptr_[std::min<uint64_t>(s1, nslices_)];
  std::vector<uint32_t> col(e1 - e0), mask((e1 - e0) / 32);
  if (e1 > e0) {
    PD_TRY(cpy(col.data(), d_col_ + e0, (e1 - e0) * 4, "read col"));
    PD_TRY(cpy(mask.data(), d_mask_ + e0 / 32, (e1 - e0) / 32 * 4, "read mask"));
  }
  uint64_t c = 0;
  for (uint64_t i = 0; i < nloc; ++i) {  // file order
    const uint64_t g = node_of_[g0 + i];
    const uint64_t base = h_slice_ptr_[g >> 5] - e0 + (g & 31);
    const uint64_t mbase = (h_slice_ptr_[g >> 5] - e0) >> 5;
    for (uint32_t j = 0; j < h_deg_[g]; ++j) {
      if (!((mask[mbase + j] >> (g & 31)) & 1u)) continue;
      uint64_t q = file_of_[col[base + 32ull * j] & kColIndex] - g0;
      if (i < q) {
        if (pairs && c < cap) {
          pairs[2 * c] = (uint32_t)i;
          pairs[2 * c + 1] = (uint32_t)q;
        }
        ++c;
      }
    }
  }
  *n = c;
  if (pairs && c > cap) {
    err = "connectivity buffer too small";
    return PD_EINVAL;
  }
  return PD_OK;
}

int Engine::get_wall(uint32_t sim, double *wall_info, double *reaction) {
  if (sim >= S_) return PD_EINVAL;
  if (finished_[sim]) {  // kept by finish_sim
    const double *w = final_[sim].data() + 15 * (sim_node0_[sim + 1] - sim_node0_[sim]);
    if (wall_info) std::memcpy(wall_info, w, 6 * 8);
    if (reaction) std::memcpy(reaction, w + 6, 18 * 8);
    return PD_OK;
  }
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  DevSimState st;
  PD_TRY(cpy(&st, d_ss_ + sim, sizeof(st), "read wall"));
  if (wall_info) std::memcpy(wall_info, st.wall, 6 * 8);
  if (reaction) std::memcpy(reaction, st.react, 18 * 8);
  return PD_OK;
}

int Engine::get_aabb(double *lrtb) {
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  return cpy(lrtb, d_lrtb_, 6ull * P_ * 8, "read aabb");
}

int Engine::get_stats(pd_stats *st) {
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  DevCounters c;
  PD_TRY(cpy(&c, d_cnt_, sizeof(c), "read counters"));
  DevSimState s0;
  PD_TRY(cpy(&s0, d_ss_, sizeof(s0), "read sim"));
  st->step = s0.t - 1;
  st->live_bonds = stats_ ? c.live_bonds : initial_bonds_;
  st->pairwise_computations = c.pairwise;
  st->contacts = c.contacts;
  st->rebuilds = c.rebuilds;
  st->device_errors = c.err;
  unsigned long long z = 0;
  PD_TRY(cpy(&d_cnt_->pairwise, &z, 8, "reset pairwise"));
  return PD_OK;
}

int Engine::set_tuning(double skin_frac, uint32_t cand_cap, int tpb, int stats, int use_graphs) {
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  bool relaunch = false;
  if (skin_frac > 0 && skin_frac != bp_.skin_frac) {
    bp_.skin_frac = skin_frac;
    std::vector<DevSimParams> sps(S_);
    PD_TRY(cpy(sps.data(), d_sp_, S_ * sizeof(DevSimParams), "read params"));
    double mh = 1e300;
    for (auto &sp : sps) {
      const double skin = skin_frac * sp.Rc;
      const double rcand = (sp.Rc + skin) * (1.0 + 1e-9);
      sp.cell = rcand * (1.0 + 1e-9);
      sp.inv_cell = 1.0 / sp.cell;
      sp.cand_r2 = rcand * rcand;
      mh = std::min(mh, 0.5 * skin);
    }
    half_skin_ = mh;
    PD_TRY(cpy(d_sp_, sps.data(), S_ * sizeof(DevSimParams), "write params"));
    double big = 1e300;
    PD_TRY(cpy(&d_cnt_->moved, &big, 8, "force rebuild"));
    relaunch = true;
  }
  if (cand_cap > 0 && cand_cap != bp_.cand_cap) {
    if (cand_cap > kMaxCandCap) {
      err = "cand_cap above " + std::to_string(kMaxCandCap);
      return PD_EINVAL;
    }
    bp_.cand_cap = cand_cap;
    PD_TRY(alloc_candidates());
    double big = 1e300;
    PD_TRY(cpy(&d_cnt_->moved, &big, 8, "force rebuild"));
    relaunch = true;
  }
  if (tpb > 0 && tpb != tpb_) {
    tpb_ = tpb;
    relaunch = true;
  }
  if (stats >= 0 && (stats != 0) != stats_) {
    stats_ = stats != 0;
    relaunch = true;
  }
  if (use_graphs >= 0) {  // 0: separate launches, 1: plain step graph, 2: conditional broad phase,
                         // 3: persistent launches (where eligible; the graph of mode 2 otherwise)
    if (use_graphs > 3) {
      err = "launch mode above 3";
      return PD_EINVAL;
    }
    use_graphs_ = use_graphs != 0;
    use_conditional_ = use_graphs >= 2;
    use_persist_ = use_graphs == 3;
    graphs_ok_ = false;
  }
  if (relaunch) graphs_ok_ = false;
  return PD_OK;
}

int Engine::clear_device_errors() {
  uint32_t z = 0;
  return cpy(&d_cnt_->err, &z, 4, "clear errors");
}

double Engine::step_bytes(uint64_t live) const {
  return 4.125 * (double)live + 224.0 * (double)N_;
}

}  // namespace pdg

namespace pdg {

int Engine::profile(uint32_t nsteps, double *phase_ms) {
  cudaEvent_t ev[5];
  for (int i = 0; i < 5; ++i)
    if (cudaEventCreate(&ev[i]) != cudaSuccess) return check(cudaGetLastError(), "event create");
  int rc = PD_OK;
  for (uint32_t k = 0; k < nsteps && rc == PD_OK; ++k) {
    DevView v = view(cur_);
    cudaStream_t s = stream_;
    cudaEventRecord(ev[0], s);
    if (reset_possible_) launch_reset_y(v, s);
    if (precision_ == PD_FP64) launch_predict(v, tpb_, s);
    if (torque_possible_) launch_centroids(v, s);
    cudaEventRecord(ev[1], s);
    launch_bp_decide(v, half_skin_, s);
    launch_broadphase(v, bp_, s);
    cudaEventRecord(ev[2], s);
    launch_step_kernel(v, precision_, variant_, s);
    if (pv_possible_) launch_prescribed(v, s);
    cudaEventRecord(ev[3], s);
    if (stats_) launch_pairwise_count(v, s);
    launch_end_step(v, d_clamped_, n_clamped_, d_clamped_disp_, s);
    cudaEventRecord(ev[4], s);
    rc = check(cudaEventSynchronize(ev[4]), "profile step");
    if (rc != PD_OK) break;
    for (int i = 0; i < 4; ++i) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
      phase_ms[i] += ms;
    }
    cur_ ^= 1;
    ++steps_done_;
    for (uint32_t i = 0; i < S_; ++i)
      if (!finished_[i]) sim_steps_[i] += 1;
  }
  for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]);
  return rc;
}

int Engine::get_afd(double *afd) {
  if (!d_afd_) {
    std::memset(afd, 0, 3 * N_ * 8);
    return PD_OK;
  }
  std::unique_ptr<double[]> buf(new double[3 * Ncap_]);
  PD_TRY(cpy(buf.get(), d_afd_, 3 * Ncap_ * 8, "read applied force density"));
  rows_to_file(buf.get(), Ncap_, 0, N_, afd);
  return PD_OK;
}

int Engine::count_live_bonds(uint64_t *live) {
  unsigned long long *d = nullptr;
  PD_TRY(check(cudaMallocAsync((void **)&d, 8, stream_), "alloc"));
  cudaMemsetAsync(d, 0, 8, stream_);
  launch_count_live(view(cur_), d, stream_);
  unsigned long long h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, stream_);
  cudaFreeAsync(d, stream_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  PD_TRY(check(e, "count live bonds"));
  *live = h;
  return PD_OK;
}

int Engine::get_damage(double *damage, uint64_t n0, uint64_t nn) {
  if (nn == UINT64_MAX) nn = N_ - n0;
  if (n0 > N_ || nn > N_ - n0) {
    err = "get_damage: node range out of bounds";
    return PD_EINVAL;
  }
  if (!nn) return PD_OK;
  // scratch: the file-ordered bond counts (4 B/node, padded to 8 B) and the damage field
  const uint64_t bytes = 4 * (nn + (nn & 1)) + 8 * nn;
  uint32_t *now = nullptr;
  if (cudaMallocAsync((void **)&now, bytes, stream_) != cudaSuccess) {
    cudaGetLastError();
    err = "get_damage: no device room for " + std::to_string(bytes) + " bytes of scratch";
    return PD_ENOMEM;
  }
  double *out = reinterpret_cast<double *>(now + nn + (nn & 1));  // 8-byte aligned
  cudaError_t e = cudaMemsetAsync(now, 0, 4 * nn, stream_);
  if (e == cudaSuccess) {
    launch_damage(view(cur_), n0, nn, now, out, stream_);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(damage, out, 8 * nn, cudaMemcpyDeviceToHost, stream_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  cudaFreeAsync(now, stream_);
  PD_TRY(check(e, "read damage"));
  return PD_OK;
}

}  // namespace pdg

namespace pdg {

int Engine::set_connectivity(uint32_t particle, const uint32_t *pairs, uint64_t n) {
  if (particle >= P_) {
    err = "particle index out of range";
    return PD_EINVAL;
  }
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
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
  std::vector<uint64_t> keys(n);
  for (uint64_t l = 0; l < n; ++l) {
    uint64_t a = pairs[2 * l], b = pairs[2 * l + 1];
    if (a >= nloc || b >= nloc) {
      err = "connectivity index out of range";
      return PD_EINVAL;
    }
    if (a > b) std::swap(a, b);
    keys[l] = a * nloc + b;
  }
  std::sort(keys.begin(), keys.end());
  const uint64_t s0 = g0 >> 5, s1 = std::min<uint64_t>((g0 + nloc + 31) >> 5, nslices_);
  const uint64_t e0 = h_slice_ptr_[s0], e1 = h_slice_ptr_[s1];
  if (e1 == e0) return PD_OK;
  std::vector<uint32_t> col(e1 - e0), mask((e1 - e0) / 32);
  PD_TRY(cpy(col.data(), d_col_ + e0, (e1 - e0) * 4, "read col"));
  PD_TRY(cpy(mask.data(), d_mask_ + e0 / 32, (e1 - e0) / 32 * 4, "read mask"));
  for (uint64_t i = 0; i < nloc; ++i) {
    const uint64_t g = node_of_[g0 + i];
    const uint64_t base = h_slice_ptr_[g >> 5] - e0 + (g & 31);
    const uint64_t mbase = (h_slice_ptr_[g >> 5] - e0) >> 5;
    const uint32_t bit = 1u << (g & 31);
    for (uint32_t j = 0; j < h_deg_[g]; ++j) {
      uint64_t q = file_of_[col[base + 32ull * j] & kColIndex] - g0;
      uint64_t a = std::min<uint64_t>(i, q), b = std::max<uint64_t>(i, q);
      const bool live = std::binary_search(keys.begin(), keys.end(), a * nloc + b);
      if (live)
        mask[mbase + j] |= bit;
      else
        mask[mbase + j] &= ~bit;
    }
  }
  PD_TRY(cpy(d_mask_ + e0 / 32, mask.data(), (e1 - e0) / 32 * 4, "write mask"));
  if (precision_ == PD_FP32C) {  // broken flags of the column entries from the new masks
    launch_col_flags(view(cur_), stream_);
    PD_TRY(check(cudaGetLastError(), "set connectivity"));
    PD_TRY(check(cudaStreamSynchronize(stream_), "set connectivity"));
  }
  return PD_OK;
}

int Engine::set_wall(uint32_t sim, const double *wall_info) {
  if (sim >= S_) return PD_EINVAL;
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  DevSimState st;
  PD_TRY(cpy(&st, d_ss_ + sim, sizeof(st), "read sim state"));
  for (int k = 0; k < 6; ++k) st.wall[k] = wall_info[k];
  PD_TRY(cpy(d_ss_ + sim, &st, sizeof(st), "write sim state"));
  if (precision_ == PD_FP32C) PD_TRY(prepare_fused(cur_));  // walls in the local frames
  return check(cudaStreamSynchronize(stream_), "set_wall");
}

}  // namespace pdg

namespace pdg {

int Engine::snapshot() {
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  const uint64_t C = Ncap_;
  mutable_.clear();
  auto reg = [&](void *p, size_t b) {
    if (p && b) mutable_.push_back({p, b});
  };
  reg(d_disp_, 3 * C * 8);
  if (d_dispb_[1]) reg(d_dispb_[1], 3 * C * 8);
  reg(d_vel_[0], 3 * C * 8);
  reg(d_vel_[1], 3 * C * 8);
  reg(d_acc_, 3 * C * 8);
  reg(d_force_, 3 * C * 8);
  reg(d_mask_, std::max<uint64_t>(E_ / 32, 1) * 4);
  reg(d_lrtb_, 6ull * P_ * 8);
  reg(d_lrtb_next_, 6ull * P_ * 8);
  reg(d_parts_, (size_t)P_ * sizeof(DevPart));
  reg(d_ss_, (size_t)S_ * sizeof(DevSimState));
  reg(d_cnt_, sizeof(DevCounters));
  reg(d_centroid_, 3ull * P_ * 8);
  if (reset_possible_) reg(d_pos_, 3 * C * 8);
  if (d_afd_) reg(d_afd_, 3 * C * 8);
  if (d_clamped_disp_) reg(d_clamped_disp_, 3 * n_clamped_ * 8);
  if (precision_ == PD_FP32C) {
    reg(d_rec_[0], C * sizeof(Rec32));
    reg(d_rec_[1], C * sizeof(Rec32));
    reg(d_anchor_, 3ull * P_ * 8);
    reg(d_anchor_next_, 3ull * P_ * 8);
    reg(d_wall_local_, 6ull * P_ * 4);
    reg(d_lrtb_local_, 6ull * P_ * 4);
    reg(d_extra_flag_, C);
    reg(d_f_extra_, 3 * C * 8);
  }
  // the contact candidate lists, the cell list and the FP32 form's contact-node list are
  // derived from the positions: restore() has the next step rebuild them instead
  if (bp_.xcount) {
    reg(bp_.xparts, (size_t)P_ * 4);
    reg(bp_.xcount, 8);
  }
  size_t total = 0;
  for (auto &m : mutable_) total += (m.second + 255) & ~(size_t)255;
  if (total > backup_bytes_) {
    if (backup_) {
      cudaFreeAsync(backup_, stream_);
      device_bytes_ -= backup_bytes_;
      allocs_.erase(std::remove(allocs_.begin(), allocs_.end(), backup_), allocs_.end());
      backup_ = nullptr;
    }
    char *b = nullptr;
    PD_TRY(dalloc(this, allocs_, &b, total, err));
    backup_ = b;
    backup_bytes_ = total;
  }
  size_t off = 0;
  for (auto &m : mutable_) {
    PD_TRY(check(cudaMemcpyAsync((char *)backup_ + off, m.first, m.second, cudaMemcpyDeviceToDevice, stream_),
                 "snapshot"));
    off += (m.second + 255) & ~(size_t)255;
  }
  backup_cur_ = cur_;
  backup_steps_ = steps_done_;
  backup_sim_steps_ = sim_steps_;
  backup_finished_ = finished_;
  return check(cudaStreamSynchronize(stream_), "snapshot");
}

int Engine::restore() {
  if (!backup_) {
    err = "restore without a snapshot";
    return PD_ESTATE;
  }
  PD_TRY(check(cudaStreamSynchronize(stream_), "sync"));
  size_t off = 0;
  for (auto &m : mutable_) {
    PD_TRY(check(cudaMemcpyAsync(m.first, (char *)backup_ + off, m.second, cudaMemcpyDeviceToDevice, stream_),
                 "restore"));
    off += (m.second + 255) & ~(size_t)255;
  }
  if (precision_ == PD_FP32C) launch_col_flags(view(cur_), stream_);  // broken flags from the masks
  PD_TRY(check(cudaGetLastError(), "restore"));
  {  // the next step rebuilds the broad phase from the restored positions (results do not depend
     // on when it is rebuilt); the FP32 non-bond kernel visits every node once meanwhile
    const double big = 1e300;
    const uint32_t one = 1;
    PD_TRY(check(cudaMemcpyAsync(&d_cnt_->moved, &big, 8, cudaMemcpyHostToDevice, stream_), "restore"));
    PD_TRY(check(cudaMemcpyAsync(&d_cnt_->xall, &one, 4, cudaMemcpyHostToDevice, stream_), "restore"));
  }
  cur_ = backup_cur_;
  steps_done_ = backup_steps_;
  sim_steps_ = backup_sim_steps_;
  // a simulation finished after the snapshot is live again (its active flag came back)
  for (uint32_t i = 0; i < S_; ++i)
    if (finished_[i] && !backup_finished_[i]) {
      finished_[i] = 0;
      final_[i].clear();
    }
  return check(cudaStreamSynchronize(stream_), "restore");
}

int Engine::prepare_windows() {
  if (windows_ready_ || precision_ != PD_FP32C) return PD_OK;
  const uint64_t nb = (N_ + kStageNodes - 1) / kStageNodes;
  launch_stage_windows(view(cur_), d_win_lo_, d_win_cnt_, stream_);
  PD_TRY(check(cudaGetLastError(), "stage windows"));
  std::vector<uint32_t> wcnt(nb);
  PD_TRY(cpy(wcnt.data(), d_win_cnt_, nb * 4, "read windows"));
  win_max_ = 0;
  for (uint32_t c : wcnt) win_max_ = std::max(win_max_, c);
  if (win_max_) PD_TRY(prepare_staged_kernels(win_max_ * (uint32_t)sizeof(Rec32)));
  windows_ready_ = true;
  graphs_ok_ = false;  // the kernels' view carries win_max
  return PD_OK;
}

int Engine::set_persist_lanes(int lanes) {
  if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4) {
    err = "persistent lanes per node must be 0, 1, 2 or 4";
    return PD_EINVAL;
  }
  persist_lanes_ = lanes;
  persist_grid_lanes_ = 0;
  return PD_OK;
}

int Engine::set_variant(int variant) {
  if (variant < 0 || variant >= num_bond_variants()) {
    err = "bond kernel variant out of range";
    return PD_EINVAL;
  }
  if (variant >= kFirstStagedVariant) PD_TRY(prepare_windows());
  variant_ = variant;
  graphs_ok_ = false;
  return PD_OK;
}

int Engine::autotune(uint32_t steps_per_variant, int *chosen, double *variant_ms) {
  const int nv = precision_ == PD_FP32C ? num_bond_variants() : 1;
  if (steps_per_variant == 0) steps_per_variant = 8;
  if (nv > kFirstStagedVariant) PD_TRY(prepare_windows());
  PD_TRY(snapshot());
  int best = variant_;
  double best_ms = 1e300;
  for (int v = 0; v < nv; ++v) {
    variant_ = v;
    double ph[4] = {0, 0, 0, 0};
    PD_TRY(profile(2, ph));  // first launches of a variant
    double pm[4] = {0, 0, 0, 0};
    PD_TRY(profile(steps_per_variant, pm));
    const double ms = pm[2] / steps_per_variant;
    if (variant_ms) variant_ms[v] = ms;
    if (ms < best_ms) {
      best_ms = ms;
      best = v;
    }
    PD_TRY(restore());  // every variant starts from the same state
  }
  variant_ = best;
  graphs_ok_ = false;
  if (chosen) *chosen = best;
  // launch mode: the plain step graph, the one with the conditional broad phase or (where
  // eligible) the persistent launch, each timed from the same snapshot
  if (use_graphs_) {
    cudaEvent_t e0, e1;
    PD_TRY(check(cudaEventCreate(&e0), "event"));
    PD_TRY(check(cudaEventCreate(&e1), "event"));
    float best_mode_ms = 1e30f;
    bool best_cond = use_conditional_, best_persist = use_persist_;
    int best_lanes = persist_lanes_;
    // modes 1 and 2, then (where eligible) the persistent step with 1, 2 and 4 lanes per node
    const int last_mode = persist_eligible() ? 5 : 2;
    for (int mode = 1; mode <= last_mode; ++mode) {
      const int lanes = mode >= 3 ? (1 << (mode - 3)) : 0;
      use_conditional_ = mode >= 2;
      use_persist_ = mode >= 3;
      if (mode >= 3) PD_TRY(set_persist_lanes(lanes));
      graphs_ok_ = false;
      int rc = step(2);
      if (rc == PD_OK) rc = check(cudaEventRecord(e0, stream_), "event");
      if (rc == PD_OK) rc = step(steps_per_variant);
      if (rc == PD_OK) rc = check(cudaEventRecord(e1, stream_), "event");
      if (rc == PD_OK) rc = check(cudaEventSynchronize(e1), "event");
      float ms = 0;
      if (rc == PD_OK) cudaEventElapsedTime(&ms, e0, e1);
      // the conditional graph counts only if it was really captured (it falls back otherwise)
      if (rc == PD_OK && (mode == 1 || use_conditional_) && ms < best_mode_ms) {
        best_mode_ms = ms;
        best_cond = mode >= 2;
        best_persist = mode >= 3;
        best_lanes = lanes;
      }
      if (rc != PD_OK && mode >= 3) {  // a device that cannot hold the cooperative grid: not a candidate
        cudaGetLastError();
        rc = PD_OK;
      }
      if (rc == PD_OK) rc = restore();
      if (rc != PD_OK) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rc;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    use_conditional_ = best_cond;
    use_persist_ = best_persist;
    PD_TRY(set_persist_lanes(best_persist ? best_lanes : 0));
    graphs_ok_ = false;
  }
  // contact skin: a wider skin rebuilds the candidate lists less often but makes them longer.
  // Where the lists were rebuilt while the chosen mode stepped, 1.5 and 2 times the skin are timed
  // as well, each from the same snapshot over enough steps to span several rebuilds (results do
  // not depend on the skin)
  {
    cudaEvent_t e0, e1;
    PD_TRY(check(cudaEventCreate(&e0), "event"));
    PD_TRY(check(cudaEventCreate(&e1), "event"));
    const uint32_t ks = std::max<uint32_t>(steps_per_variant, 24);
    const double skin0 = bp_.skin_frac;
    double best_skin = skin0;
    float best_skin_ms = 0;
    bool rebuilt = false;
    int rc = PD_OK;
    for (int i = 0; i < 3 && rc == PD_OK; ++i) {
      if (i > 0 && !rebuilt) break;
      const double skin = skin0 * (i == 0 ? 1.0 : i == 1 ? 1.5 : 2.0);
      unsigned long long r0 = 0, r1 = 0;
      rc = set_tuning(skin, 0, 0, -1, -1);
      if (rc == PD_OK) rc = step(2);
      if (rc == PD_OK) rc = check(cudaStreamSynchronize(stream_), "sync");
      if (rc == PD_OK) rc = cpy(&r0, &d_cnt_->rebuilds, sizeof(r0), "read rebuilds");
      if (rc == PD_OK) rc = check(cudaEventRecord(e0, stream_), "event");
      if (rc == PD_OK) rc = step(ks);
      if (rc == PD_OK) rc = check(cudaEventRecord(e1, stream_), "event");
      if (rc == PD_OK) rc = check(cudaEventSynchronize(e1), "event");
      if (rc == PD_OK) rc = cpy(&r1, &d_cnt_->rebuilds, sizeof(r1), "read rebuilds");
      float ms = 0;
      if (rc == PD_OK) cudaEventElapsedTime(&ms, e0, e1);
      if (rc == PD_OK) {
        if (i == 0) rebuilt = r1 > r0;
        if (i == 0 || ms < best_skin_ms) {
          best_skin_ms = ms;
          best_skin = skin;
        }
      }
      if (rc == PD_OK) rc = restore();
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    PD_TRY(rc);
    PD_TRY(set_tuning(best_skin, 0, 0, -1, -1));
  }
  return PD_OK;
}

}  // namespace pdg
