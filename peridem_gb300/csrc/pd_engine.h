// pd_engine.h -- device data layout and host engine of the GB300 explicit step.
//
// Layout in HBM (all particles of all simulations of a batch concatenated in file order; the
// nodes of particle p occupy the engine indices [node_offset[p], node_offset[p+1]) as in the
// file, but inside each window of kOrderWindow of them they are sorted by descending bond
// count (stable), so that the 32 rows of a SELL slice have nearly equal lengths; node_of /
// file_of map the two numberings and every host-facing array is in file order):
//   * node state, FP64 structure-of-arrays: pos/disp/vel/acc/force/extforce as [3][Ncap]
//     (x block, y block, z block), vol[N]; vel is double-buffered (the fused kernel reads
//     partners' step-start velocity while it writes the corrected one);
//   * bonds, SELL-32: nodes are grouped in slices of 32 consecutive nodes (one warp); a
//     slice stores its rows column-major, entry (slice s, position j, lane l) at
//     slice_ptr[s] + 32*j + l, so the 32 lanes of a warp read 128 contiguous bytes of
//     column indices per position. Each row keeps the reference's neighbour order
//     (conn2NArr push order, ascending for a sorted Connectivity). One 32-bit word per
//     (slice, position) holds the live bits of the 32 lanes: bit l of
//     mask[slice_ptr[s]/32 + j]. Breaking clears a bit; bonds are never re-added;
//   * FP32-compensated form: bit 31 of a column entry mirrors a cleared live bit (set by the
//     FP32 kernels when they break the bond, re-derived from the masks after a restore or a
//     set Connectivity), so that the FP32 bond loops read liveness with the column index;
//     the masks stay the record every other reader uses;
//   * FP64 form only: per-entry constants xi = pos[q]-pos[i] (3 doubles), |xi| and the
//     correctly rounded reciprocal of |xi| (gen_xi, particle2.h:241-257);
//   * FP32-compensated form only: a 32-byte record per node, float4 (local position,
//     cnot * volume) + float4 (local displacement), double-buffered; local = relative to the
//     particle's anchor node;
//   * contact broad phase: hashed cell list (counting sort) rebuilt only when the nodes may
//     have moved more than half the skin since the last build; per-node candidate lists
//     (fixed capacity, ascending file index) of nodes within contact radius + skin.
#ifndef PD_ENGINE_H
#define PD_ENGINE_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "peridem_gb300.h"

namespace pdg {

// Runs f(i) for i in [0, n) on the host's cores (work handed out one index at a time).
template <class F>
void parallel_items(uint64_t n, F f) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const unsigned T = (unsigned)std::min<uint64_t>(std::min(hw, 32u), n);
  if (T <= 1) {
    for (uint64_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<uint64_t> next(0);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < T; ++t)
    th.emplace_back([&] {
      for (uint64_t i = next++; i < n; i = next++) f(i);
    });
  for (auto &x : th) x.join();
}

constexpr int kSlice = 32;
constexpr int kStageNodes = 512;          // nodes per block of the staged bond kernel
constexpr uint32_t kStageMaxRecords = 6400;  // 200 KB of 32-byte records per block
constexpr uint32_t kNoCol = 0xFFFFFFFFu;
constexpr uint16_t kCandCells = 0xFFFFu;  // cand_n of a node whose contact partners come from the cell list
constexpr uint32_t kMaxCandCap = 64;      // largest per-node candidate list
constexpr uint32_t kColBroken = 0x80000000u;  // FP32 form: broken flag in a column entry
constexpr uint32_t kColIndex = 0x7FFFFFFFu;   // the partner index in a column entry
constexpr uint64_t kOrderWindow = 1024;     // nodes per window of the bond-count sort (order_nodes)

// Per-particle parameters (ParticleN scalars, particle2.h:51-59).
struct DevPart {
  uint32_t g0, n, sim, taxis;
  double rho, irho, cnot, snot, tval;
  int32_t movable, breakable, stoppable, break_bonds;
  double anchor_pos[3];  // FP32 form: position of the anchor node
  int32_t has_ext;       // any non-zero extforce in this particle
  uint32_t anchor;       // FP32 form: the anchor node (the node nearest the particle's box centre)
  double ext_p;          // FP32 form: largest |component| of a node's position relative to the anchor
  double xi_min;         // FP32 form: shortest bond of the particle's setup (reference positions)
  float snot_lo32, snot_hi32;  // FP32 form: the band around snot where FP64 decides (set_break_band)
};

// Per-simulation constants (Contact, RectWall and Timeloop fields after apply_config).
struct DevSimParams {
  double dt, hdt2, hdt;       // dt, (dt*dt)*0.5, 0.5*dt
  double Rc, Kn, sc, zeta2, mu;  // contact radius, stiffness, Kn*Rc, 2*damping, friction
  double rc2_far;             // Rc^2 (1 + 1e-12): a pair whose squared distance reaches it fails both
                              // contact tests (dn < Rc, dn <= Rc), so its square root is skipped
  double pi3, pi4;            // M_PI/3, M_PI/4 (segment_mass)
  double cell;                // broad-phase cell edge (Rc + skin, slightly enlarged)
  double inv_cell;            // 1 / cell: cell coordinates are floor(x * inv_cell) everywhere
  double cand_r2;             // squared candidate radius
  int32_t nl_bdry_only, compute_wall_reaction, gradient_extforce, allow_wall;
  uint32_t extforce_maxstep;
  int32_t set_torque_ts, set_fracture_ts, set_self_contact_ts, set_damping_ts;
  int32_t set_zero_wall_speed_ts, set_movable_index, set_movable_ts;
  int32_t set_stoppable_index, set_stoppable_ts;
  uint32_t p0, np;            // particle range of this simulation
  uint64_t node0, nnodes;     // node range of this simulation
  // prescribed velocity of one particle (timeloop.h:684-764); pv_particle -1 = none
  int32_t pv_particle, set_fix_velocity_ts, fix_mean_x, fix_angular;
  double pv_mean_x, pv_angular;
  // reset_partzero_y (timeloop.h:500-535)
  int32_t reset_y;
  uint32_t reset_y_ts;
  double wheel_rad;
};

// Per-simulation state that changes from step to step.
struct DevSimState {
  double wall[6];   // x_min y_min z_min x_max y_max z_max
  double spd[6];
  double react[18]; // 6 faces x 3, get_reaction() order
  double extf_scale;
  uint32_t t;       // index of the step about to run (1-based, like timeloop.h:395)
  int32_t fracture, self_contact, damping, friction, torque, active;
  int32_t vconstraint;  // enable_velocity_constraint
};

// Global counters (one block of device memory, read back by pd_get_stats).
struct DevCounters {
  unsigned long long stepmax_bits;  // max |disp increment| of the current step (double bits)
  double moved;                     // accumulated bound since the last rebuild
  uint32_t rebuild;                 // set when this step rebuilt the broad phase
  uint32_t err;                     // PD_DERR_* bits
  unsigned long long contacts;
  unsigned long long pairwise;
  unsigned long long rebuilds;
  unsigned long long live_bonds;
  double last_stepmax;              // movement bound of the step that just ended
  uint32_t end_blocks;              // blocks of k_end_step done (the last one advances the sims)
  uint32_t xall;                    // FP32 form: k_extra32 visits every node this step (no lists)
  uint32_t cand_cells;              // nodes whose candidate list overflowed (they walk the cells)
};

// FP32 form: one 32-byte record per node, so that a bond gathers its partner with a single
// 256-bit load: p = (anchor-relative position, cnot * volume), u = (anchor-relative
// displacement, 0).
struct __align__(32) Rec32 {
  float4 p, u;
};

// Everything a kernel needs, passed by value.
struct DevView {
  uint64_t N;            // nodes
  uint64_t Ncap;         // stride of the [3][Ncap] arrays
  uint32_t P, S;         // particles, simulations
  const double *pos;     // [3][Ncap]
  double *disp;
  const double *vel_in;
  double *vel_out;
  double *acc, *force;
  const double *ext, *vol;
  const uint32_t *pid;   // particle of each node
  const uint32_t *node_of;  // file-order global index -> engine index
  const uint32_t *file_of;  // engine index -> file-order global index
  const uint8_t *bdry;   // 1 if node is in its particle's bdry_nodes list
  // bonds
  const uint64_t *slice_ptr;
  const uint16_t *deg;
  const uint32_t *col;
  uint32_t *mask;
  const double *bxi, *bxin, *brxin;  // FP64 form, [3][E], [E], [E]
  uint64_t E;
  // FP32-compensated form (the predictor of the next step runs in the bond kernel's tail:
  // disp/rec are read for this step while disp_next/rec_next receive the next one)
  Rec32 *rec, *rec_next;
  double *disp_next;
  const uint8_t *clamp_flag;  // FP32 form: 1 for nodes listed in clamped_nodes
  int fused;                  // 1: FP32 form with the fused predictor
  const double *anchor;       // [P][3] anchor of rec[].u (this step)
  double *anchor_next;        // [P][3] anchor of rec_next[].u
  double break_band;     // relative band around snot where the FP64 stretch decides
  double *f_extra;       // [3][Ncap] FP64 non-bond force density of flagged nodes
  // FP32 form, staged bond kernel: per block of kStageNodes nodes, the contiguous range of
  // node records its bonds read ([win_lo, win_lo + win_cnt); win_cnt 0 = not staged)
  const uint32_t *win_lo, *win_cnt;
  uint32_t win_max;      // largest staged range (records): the kernel's shared-memory size
  // FP32 form: work lists of k_extra32 (see BroadPhase)
  uint32_t *xnodes, *xparts, *xcount;
  uint32_t max_part_nodes;  // nodes of the largest particle
  uint8_t *extra_flag;   // 1 where f_extra holds this step's contribution
  float *wall_local;     // [P][6] wall planes in each particle's local frame
  unsigned int *lrtb_local_next;  // [P][6] ordered float keys of the local-frame AABB
  // particles / sims
  DevPart *parts;
  double *lrtb, *lrtb_next;  // [P][6]; lrtb_next holds ordered-integer min/max keys
  const DevSimParams *sp;
  DevSimState *ss;
  // contact
  const uint32_t *cand;  // [N][cap]
  const uint16_t *cand_n;  // list length, or kCandCells: walk the cell list (the list overflowed)
  uint32_t cand_cap;
  // the broad phase's hashed cell list (valid from one rebuild to the next)
  const uint32_t *cell_count, *cell_start, *cell_sorted;
  uint32_t cell_mask;
  // torque centroids [P][3]
  const double *centroid;
  DevCounters *cnt;
  int stats;
  // prescribed velocity: the corrector stores the old acceleration of the particle's nodes
  // here, k_prescribed turns it into applied_force_density ([3][Ncap], or null)
  double *afd;
  // clamped nodes ([P+1] offsets, global node ids) and their predicted displacement (FP64 form)
  const uint32_t *clamped_ptr, *clamped_list;
  const double *clamped_disp;
};

// Broad-phase scratch (hashed cell list).
struct BroadPhase {
  uint32_t table_bits = 0;
  uint32_t *count = nullptr, *start = nullptr, *key = nullptr, *slot = nullptr, *sorted = nullptr;
  uint32_t *block_sums = nullptr;
  uint32_t *cand = nullptr;
  uint16_t *cand_n = nullptr;
  uint32_t cand_cap = 0;
  double skin_frac = 0.5;
  // FP32 form: the nodes that have contact candidates (rebuilt with the lists), the particles
  // that need FP64 non-bond work next step, and their counts ([0] nodes, [1] particles)
  uint32_t *xnodes = nullptr, *xparts = nullptr, *xcount = nullptr;
};

// A frame's worth of device state in pinned host memory, copied in stream order: the copies
// run after the step that produced the state and before later steps overwrite it, so the
// step pipeline does not stop for output (timeloop.h:801-953 writes synchronously).
struct HostFrame {
  double *disp = nullptr, *vel = nullptr, *acc = nullptr, *force = nullptr;  // [3][Ncap]
  double *pos = nullptr;    // [3][Ncap], only when reference positions can move
  double *cdisp = nullptr;  // [n_clamped][3] predicted displacement of clamped nodes
  double *afd = nullptr;    // [3][Ncap], only with a prescribed-velocity particle
  uint32_t *mask = nullptr; // live masks
  struct DevSimState *ss = nullptr;
  struct DevCounters *cnt = nullptr;
  uint64_t steps = 0;       // steps done when staged
  cudaEvent_t done = nullptr;
};

// An array the engine reads only while it is built (Engine::init, estimate_bytes): it either
// owns its elements or views the caller's, which then must stay valid until the call that
// builds the engine returns. Engine::init releases it afterwards.
template <class T>
struct InitArray {
  std::vector<T> own;
  const T *ext = nullptr;
  size_t n_ext = 0;
  const T *data() const { return ext ? ext : own.data(); }
  size_t size() const { return ext ? n_ext : own.size(); }
  bool empty() const { return size() == 0; }
  const T &operator[](size_t i) const { return data()[i]; }
  void view(const T *p, size_t n) {
    own.clear();
    ext = p;
    n_ext = n;
  }
  void release() {
    std::vector<T>().swap(own);
    ext = nullptr;
    n_ext = 0;
  }
};

// Host-side description of one simulation (setup + resolved config).
struct HostSim {
  pd_config cfg;
  uint32_t np = 0;
  std::vector<uint64_t> node_offset;
  std::vector<double> pos;                        // N*3, kept (CurrPos = pos + disp on output)
  InitArray<double> vol, disp, vel, acc, ext;     // N / N*3
  std::vector<uint64_t> conn_offset;
  InitArray<uint32_t> conn;
  std::vector<uint64_t> bdry_offset, clamped_offset;
  std::vector<uint32_t> bdry, clamped;
  std::vector<double> delta, rho, cnot, snot, tval;
  std::vector<int32_t> movable, breakable, stoppable;
  std::vector<uint32_t> taxis;
  double Rc = 0, Kn = 0, zeta = 0, mu = 0;
  int32_t allow_wall = 0, n_geom_wall = 6;
  double geom[6] = {0, 0, 0, 0, 0, 0};
};

class Engine {
 public:
  Engine() = default;
  ~Engine();
  int init(std::vector<HostSim> &sims, int precision);
  int step(uint32_t nsteps);
  int sync(int timeout_ms);
  int set_stream(cudaStream_t s);
  int get_state(double *curpos, double *vel, double *acc, double *force, double *disp);
  // The same through host staging (when the device has no room for get_state's scratch).
  int get_state_host(double *curpos, double *vel, double *acc, double *force, double *disp);
  int set_state(const double *disp, const double *vel, const double *acc);
  int get_connectivity(uint32_t particle, uint32_t *pairs, uint64_t cap, uint64_t *n);
  // Keeps exactly the listed bonds (local i<q pairs) of a particle alive (resume).
  int set_connectivity(uint32_t particle, const uint32_t *pairs, uint64_t n);
  int set_wall(uint32_t sim, const double *wall_info);
  int get_wall(uint32_t sim, double *wall_info, double *reaction);
  int get_aabb(double *lrtb);
  int get_stats(pd_stats *st);
  // skin_frac <= 0, cand_cap == 0, tpb <= 0, stats < 0, use_graphs < 0 keep the setting
  int set_tuning(double skin_frac, uint32_t cand_cap, int tpb, int stats, int use_graphs);
  int clear_device_errors();
  // Bond-kernel variant (FP32 form); autotune() times each on the live state and restores it.
  int set_variant(int variant);
  // lanes per node of the persistent step's bond phase: 0 chooses by size, else 1, 2 or 4
  int set_persist_lanes(int lanes);
  int persist_lanes() const { return persist_lanes_; }
  int autotune(uint32_t steps_per_variant, int *chosen, double *variant_ms);
  // Copy of every mutable device buffer (and the host step counters), and its restore.
  int snapshot();
  int restore();
  // Runs nsteps steps as separate launches with CUDA events between the phases and adds the
  // per-phase device time (ms) to phase_ms[0..3]: predictor, broad phase, fused step
  // kernel, end-of-step kernels.
  int profile(uint32_t nsteps, double *phase_ms);
  // Live directed bonds of movable particles (popcount of the live masks).
  int count_live_bonds(uint64_t *live);
  // applied_force_density (N*3, file order); zeros when no particle has a prescribed velocity.
  int get_afd(double *afd);
  // Damage per node (N, file order) as plot3d_timestep.py:156-166 derives it from a saved
  // Connectivity: (setup bonds - live bonds) / setup bonds, NaN for a node without bonds.
  // Nodes [n0, n0 + nn) only when nn is given (whole simulations of a batch).
  int get_damage(double *damage, uint64_t n0 = 0, uint64_t nn = UINT64_MAX);
  // ---- output frames off the critical path (pd_frames.cpp) ----
  int frame_alloc(HostFrame &f);
  void frame_free(HostFrame &f);
  // Enqueues the copies of the current state into f and an event after them; also restarts
  // the pairwise counter (as get_stats does). Returns at once.
  int frame_stage(HostFrame &f);
  // After f.done: the arrays get_state / get_connectivity / get_wall / get_afd would return.
  void frame_state(const HostFrame &f, double *curpos, double *vel, double *acc, double *force,
                   double *afd) const;
  void frame_connectivity(const HostFrame &f, uint32_t particle, std::vector<uint32_t> &pairs) const;
  void frame_wall(const HostFrame &f, uint32_t sim, double *wall_info, double *reaction) const;
  // ---- batches of independent simulations (one launch per phase covers all of them) ----
  uint32_t num_sims() const { return S_; }
  int sim_range(uint32_t sim, uint64_t *node0, uint64_t *n_nodes, uint32_t *particle0, uint32_t *n_particles) const;
  uint64_t sim_steps(uint32_t sim) const { return sim < S_ ? sim_steps_[sim] : 0; }
  // Reads the simulation's state back, keeps it on the host and stops stepping it: the
  // kernels skip its nodes from the next launch on and its device state is not kept.
  int finish_sim(uint32_t sim);
  bool sim_finished(uint32_t sim) const { return sim < S_ && finished_[sim]; }
  // N*3 arrays of one simulation (its own node order); any pointer may be NULL.
  int get_sim_state(uint32_t sim, double *curpos, double *vel, double *acc, double *force, double *disp);
  // Checkpoint of one simulation at a step boundary (everything stepping changes, in a form that
  // does not depend on the handle's layout), and its load into simulation `sim` of a handle
  // created from the same setup and config: stepping on from the load computes what stepping on
  // from the save would have. A finished simulation cannot be saved (its device state is gone).
  int save_sim(uint32_t sim, std::vector<uint8_t> &out);
  int load_sim(uint32_t sim, const uint8_t *buf, uint64_t n);
  // Bytes of device memory this engine holds, and the same figure computed from a setup
  // before anything is allocated.
  uint64_t device_bytes() const { return device_bytes_; }
  // *bad (if given): a particle whose Connectivity has an index out of range, or -1 (the
  // setups pd_create_batch would refuse).
  static uint64_t estimate_bytes(const std::vector<HostSim> &sims, int precision, uint32_t cand_cap,
                                 int64_t *bad = nullptr);
  // Engine node order: inside each window of kOrderWindow nodes of a particle, nodes by
  // descending bond count bin (stable: equal bins keep their file order). file_of[engine index] = file index, node_of = its inverse,
  // deg_file = bond count of each node in file order (indices out of range are not counted).
  static void order_nodes(const std::vector<HostSim> &sims, std::vector<uint32_t> &file_of,
                          std::vector<uint32_t> &node_of, std::vector<uint32_t> &deg_file,
                          int64_t *bad = nullptr,   // a particle with an index out of range, or -1
                          bool *sorted = nullptr,   // every Connectivity strictly (i, j)-sorted, i < j
                          uint32_t deg_bin = 1);    // sort by bond count / deg_bin (order_bin)
  // Bond-count bin of the node order for a precision form: exact counts for the FP64 form (its
  // padded SELL lanes idle through FP64 arithmetic), bins of 16 for the FP32 form (its record
  // gathers keep more of the file's lattice locality, at a few per cent more padding).
  static uint32_t order_bin(int precision) { return precision == PD_FP32C ? 16u : 1u; }
  int raw_alloc(void **p, size_t bytes);
  double step_bytes(uint64_t live_bonds) const;
  uint64_t initial_bonds() const { return initial_bonds_; }
  uint64_t num_nodes() const { return N_; }
  uint32_t num_particles() const { return P_; }
  uint64_t steps_done() const { return steps_done_; }
  // 0: separate launches, 1: step graph, 2: step graph with the conditional broad phase,
  // 3: persistent launches
  int graph_mode() const {
    if (use_persist_ && persist_eligible()) return 3;
    return !use_graphs_ ? 0 : (graphs_ok_ && use_conditional_ ? 2 : 1);
  }
  // The persistent step covers the FP32 form's step without the phases it leaves out.
  bool persist_eligible() const {
    return precision_ == PD_FP32C && N_ > 0 && !reset_possible_ && !pv_possible_ && !torque_possible_ && !stats_;
  }
  cudaStream_t stream() const { return stream_; }
  int precision() const { return precision_; }
  // Device view of the state between steps (what the next step reads).
  DevView current_view() const { return view(cur_); }
  std::string err;
  const std::vector<HostSim> &sims() const { return sims_; }

 private:
  int alloc_and_upload();
  int alloc_candidates();
  // Host-side SELL-32 arrays of the bonds, built by build_bonds_host and uploaded by upload_bonds.
  struct SellHost {
    std::unique_ptr<uint32_t[]> col, mask;
    uint64_t ncol = 0, nmask = 0;
    std::string err;
  };
  int build_bonds_host(SellHost &h);
  int upload_bonds(SellHost &h);
  // Bond counts per engine node (deg), h_deg_, h_slice_ptr_, E_, initial_bonds_, and the row
  // starts of a row-contiguous layout when rowptr is given.
  int bond_counts(std::vector<uint32_t> &deg, std::vector<uint64_t> *rowptr);
  int alloc_bond_arrays();  // device SELL arrays (+ staged-kernel ranges), slice_ptr and deg uploaded
  // Device build from a sorted Connectivity, after bond_counts (rowptr: its row starts);
  // fallback = true when its scratch does not fit.
  int build_bonds_gpu(const std::vector<uint64_t> &rowptr, bool &fallback);
  int launch_step_seq(int cur, cudaStream_t s);
  int prepare_fused(int cur);  // FP32 form: predicted state for the next step from disp[cur^1]
  int capture_graphs();
  // FP32 form: record ranges of the staged bond kernel (win_lo / win_cnt / win_max), computed
  // on the device the first time a staged variant is needed.
  int prepare_windows();
  // One step graph whose broad-phase rebuild kernels sit in a conditional node set by
  // k_bp_decide (0 on success; falls back to the plain graph when unsupported).
  int capture_conditional(int cur, cudaGraphExec_t *out);
  int check(cudaError_t e, const char *what);
  // Copy / memset ordered on the engine's stream, then a wait for that stream only (never
  // the legacy default stream, so other handles' work keeps running).
  int cpy(void *dst, const void *src, size_t bytes, const char *what);
  int mset(void *dst, int value, size_t bytes, const char *what);
  int read_nodes(const double *d, uint64_t node0, uint64_t nn, double *dst);
  // Host copy of a [3][stride] array holding engine nodes node0 .. node0+nn-1 at columns
  // 0 .. nn-1 -> nn*3 row vectors in file order (relative to node0).
  void rows_to_file(const double *src, uint64_t stride, uint64_t node0, uint64_t nn, double *dst) const;
  DevView view(int cur) const;

  std::vector<HostSim> sims_;
  int precision_ = PD_FP64;
  uint64_t N_ = 0, Ncap_ = 0, E_ = 0, nslices_ = 0;
  uint32_t P_ = 0, S_ = 0;
  uint32_t max_part_nodes_ = 0;
  cudaStream_t stream_ = nullptr;          // stream work is enqueued on
  cudaStream_t capture_stream_ = nullptr;  // the handle's own stream (graphs are captured here)
  bool own_stream_ = false;
  int tpb_ = 128;
  int cur_ = 0;  // which vel buffer holds the current velocity
  bool torque_possible_ = false;
  bool stats_ = false;
  bool use_graphs_ = true;
  bool grow_cand_ = false;  // a sync saw nodes walking the cell list: double the lists at the next step
  bool use_persist_ = false;        // launch mode 3 (persistent step, FP32 form)
  uint32_t *persist_ws_ = nullptr;  // its barrier counter and scan scratch
  uint32_t persist_blocks_ = 0;     // its grid
  int persist_lanes_ = 0;           // lanes per node of its bond phase (0: by size)
  int persist_kernel_lanes_ = 1;    // the lanes of the kernel launched
  int persist_grid_lanes_ = 0;      // 1 + the lanes persist_blocks_ was sized for (0: not yet)
  int launch_persist_steps(uint32_t n);
  bool use_conditional_ = false;  // broad phase in a conditional graph node (pd_set_tuning
                                  // mode 2); init() picks by size
  int variant_ = 18;  // FP32 bond-kernel variant; init() picks by size (the autotuner's usual choices)
  std::vector<std::pair<void *, size_t>> mutable_;  // device buffers that change while stepping
  void *backup_ = nullptr;
  size_t backup_bytes_ = 0;
  int backup_cur_ = 0;
  uint64_t backup_steps_ = 0;
  std::vector<uint64_t> backup_sim_steps_;
  std::vector<uint8_t> backup_finished_;
  uint64_t steps_done_ = 0;
  uint64_t initial_bonds_ = 0;
  uint64_t device_bytes_ = 0;
  uint64_t cand_bytes_ = 0;
  std::vector<uint64_t> sim_node0_, sim_steps_;
  std::vector<uint32_t> sim_p0_;
  std::vector<uint8_t> finished_;
  std::vector<std::vector<double>> final_;  // [sim]: curpos, vel, acc, force, disp (N*3 each)
  double half_skin_ = 0;

  // host mirrors used when reading results back
  std::vector<uint32_t> file_of_, node_of_;  // see order_nodes
  std::vector<uint32_t> deg_file_;           // bond counts in file order, while building
  bool conn_sorted_ = false;                 // rows in push order are ascending (GPU bond build)
  std::vector<uint32_t> h_pid_;
  std::vector<uint64_t> h_slice_ptr_;
  std::vector<uint16_t> h_deg_;
  std::vector<uint32_t> h_g0_;
  std::vector<uint32_t> h_clamped_;  // clamped nodes, file-order global indices
  std::vector<uint32_t> h_col_;  // SELL column indices, read back once for staged frames

  // device buffers
  double *d_pos_ = nullptr, *d_disp_ = nullptr, *d_vel_[2] = {nullptr, nullptr}, *d_acc_ = nullptr;
  double *d_dispb_[2] = {nullptr, nullptr};  // FP32 form: double-buffered displacement
  Rec32 *d_rec_[2] = {nullptr, nullptr};
  double *d_anchor_next_ = nullptr;
  uint8_t *d_clamp_flag_ = nullptr;
  double *d_force_ = nullptr, *d_ext_ = nullptr, *d_vol_ = nullptr;
  uint32_t *d_pid_ = nullptr;
  uint32_t *d_node_of_ = nullptr, *d_file_of_ = nullptr;
  uint8_t *d_bdry_ = nullptr;
  uint64_t *d_slice_ptr_ = nullptr;
  uint16_t *d_deg_ = nullptr;
  uint32_t *d_col_ = nullptr, *d_mask_ = nullptr;
  double *d_bxi_ = nullptr, *d_bxin_ = nullptr, *d_brxin_ = nullptr;
  double *d_anchor_ = nullptr;
  double *d_f_extra_ = nullptr;
  uint32_t *d_win_lo_ = nullptr, *d_win_cnt_ = nullptr;
  uint32_t win_max_ = 0;
  bool windows_ready_ = false;
  uint8_t *d_extra_flag_ = nullptr;
  float *d_wall_local_ = nullptr;
  unsigned int *d_lrtb_local_ = nullptr;
  DevPart *d_parts_ = nullptr;
  double *d_lrtb_ = nullptr, *d_lrtb_next_ = nullptr, *d_centroid_ = nullptr;
  DevSimParams *d_sp_ = nullptr;
  DevSimState *d_ss_ = nullptr;
  DevCounters *d_cnt_ = nullptr;
  uint32_t *d_clamped_ = nullptr;  // [P+1] offsets followed by engine node indices
  double *d_clamped_disp_ = nullptr;
  double *h_stage_ = nullptr;  // pinned host staging of state reads on large handles (3 N doubles)
  uint64_t n_clamped_ = 0;
  double *d_afd_ = nullptr;
  bool pv_possible_ = false, reset_possible_ = false;
  BroadPhase bp_;
  std::vector<void *> allocs_;
  cudaGraphExec_t graph_[2] = {nullptr, nullptr};
  bool graphs_ok_ = false;
};

// Handles up to this many nodes search contact candidates with four nodes per warp
// (bp_candidates_quad), larger ones with one thread per node; the lists are the same.
constexpr uint64_t kWarpCandNodes = 1ull << 20;
// Handles of at least this many nodes read their state back through pinned host memory.
constexpr uint64_t kPinnedStageNodes = 1ull << 18;

// Arguments of the persistent step (k_persist, pd_fp32c.cu): the views of the two buffer
// parities, the steps to run and the broad phase's buffers.
struct PersistArgs {
  DevView v[2];
  uint32_t cur0, nsteps;
  double half_skin;
  uint32_t *count, *start, *key, *slot, *sorted;
  uint32_t *sums;  // [grid] scan scratch
  uint32_t *bar;   // barrier arrival and release counters, zero at launch
  uint64_t T;
  uint32_t mask;
  uint32_t *cand;
  uint16_t *cand_n;
  uint32_t cap;
  const uint32_t *clamped_ptr, *clamped;
  double *clamped_disp;
};
// Blocks of the persistent step with `lanes` lanes per node in its bond phase (1, 2 or 4) that
// fit on the current device at once (0 on error), and its cooperative launch.
int persist_max_blocks(int lanes);
int persist_threads();  // threads per block of the persistent step
cudaError_t launch_persist(const PersistArgs &a, uint32_t grid, int lanes, cudaStream_t s);

// Device build of the SELL-32 bond arrays from a strictly sorted Connectivity (pd_sell.cu).
struct SellBuild {
  const uint32_t *conn;      // [npairs][2] local pair indices, particles concatenated
  uint64_t npairs;
  const uint64_t *pair_off;  // [nparts+1] first pair of each particle
  const uint64_t *node0;     // [nparts] first file-order node of each particle
  uint32_t nparts;
  const uint32_t *node_of;   // file index -> engine index
  const uint64_t *rowptr;    // [n_nodes+1] row starts, engine order
  uint32_t *cursor;          // [n_nodes], zeroed
  uint32_t *rows;            // [rowptr[n_nodes]] scratch
  uint64_t n_nodes;
  const uint64_t *slice_ptr;
  uint64_t nslices;
  uint32_t *col, *mask;      // outputs
};
void launch_sell_build(const SellBuild &b, cudaStream_t s);

// kernel launchers (pd_kernels.cu / pd_broadphase.cu)
void launch_predict(const DevView &v, int tpb, cudaStream_t s);
void launch_step_kernel(const DevView &v, int precision, int variant, cudaStream_t s);
void launch_step_fp32c(const DevView &v, int variant, cudaStream_t s);
int num_bond_variants();
// Raises the dynamic shared-memory limit of the staged bond kernels (once per engine).
int prepare_staged_kernels(uint32_t smem_bytes);
constexpr int kFirstStagedVariant = 10;  // variants >= this use the staged bond kernel
// Per block of kStageNodes nodes, the smallest contiguous range of node records that holds the
// block's own nodes and every partner of their bonds (win_cnt 0 when above kStageMaxRecords).
void launch_stage_windows(const DevView &v, uint32_t *win_lo, uint32_t *win_cnt, cudaStream_t s);
void launch_end_step(const DevView &v, const uint32_t *clamped, uint64_t n_clamped, double *clamped_disp,
                     cudaStream_t s);
void launch_centroids(const DevView &v, cudaStream_t s);
void launch_bond_constants(const DevView &v, double *bxi, double *bxin, double *brxin, cudaStream_t s);
void launch_broadphase(const DevView &v, BroadPhase &bp, cudaStream_t s);
void launch_bp_decide(const DevView &v, double half_skin, cudaStream_t s, cudaGraphConditionalHandle cond = 0);
void launch_pairwise_count(const DevView &v, cudaStream_t s);
void launch_init_lrtb(const DevView &v, cudaStream_t s);
void launch_count_live(const DevView &v, unsigned long long *out, cudaStream_t s);
// k_damage_count + k_damage_out over nodes [n0, n0 + nn) (whole particles): now[nn] (file
// order - n0) must be zeroed; out[nn] in file order - n0.
void launch_damage(const DevView &v, uint64_t n0, uint64_t nn, uint32_t *now, double *out, cudaStream_t s);
void launch_anchor_next(const DevView &v, cudaStream_t s);
// FP32 form: each particle's shortest setup bond into DevPart::xi_min (d2min: [P] scratch set to
// all ones).
void launch_xi_min(const DevView &v, unsigned long long *d2min, cudaStream_t s);
void launch_col_flags(const DevView &v, cudaStream_t s);
void launch_rows_to_file(const double *src, const double *add, uint64_t Ncap, uint64_t N, const uint32_t *file_of,
                         double *dst, cudaStream_t s);
void launch_clamped_rows(const uint32_t *clamped, uint64_t n_clamped, const uint32_t *file_of, const double *pos,
                         const double *cdisp, uint64_t Ncap, double *dst, cudaStream_t s);
void launch_prescribed(const DevView &v, cudaStream_t s);
void launch_reset_y(const DevView &v, cudaStream_t s);

}  // namespace pdg
#endif
