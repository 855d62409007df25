/*
 * peridem_gb300.h -- C-ABI of the GB300 explicit-step engine for PeriDEM.
 *
 * PeriDEM (DavoodDamircheli/PeriDEM) runs its time loop behind two boundaries:
 *   1. a process/file boundary: `simulate3d -c <main.conf> -i <setup.h5> -o <outdir>`
 *      (run/simulate3d.cpp:86-105) reading the `main.conf` grammar
 *      (src/read/read_config.h:170-435) and the setup schema of
 *      src/read/load_hdf5.h:41-181, writing plotinfo.h5 / tc_%05u.h5 / wall_%05u.h5
 *      (src/particle/timeloop.h:321-350, 801-953);
 *   2. an in-process C++ boundary:
 *      run_timeloop<dim>(vector<ParticleN<dim>>&, Timeloop, Contact, RectWall<dim>, ConfigVal)
 *      (src/particle/timeloop.h:231-965), which mutates the particles in place.
 * This header replaces both with plain C entry points: no C++ exceptions and no torch
 * types cross it; every function returns an int status (PD_OK == 0, negative on error).
 *
 * Ownership: device memory belongs to the handle; caller buffers are copied and never
 * retained. A handle is not thread-safe. Work is enqueued on the handle's CUDA stream.
 */
#ifndef PERIDEM_GB300_H
#define PERIDEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------------- */
#define PD_OK 0
#define PD_EINVAL (-1)    /* bad argument / inconsistent setup arrays               */
#define PD_ECUDA (-2)     /* a CUDA runtime call failed (no GPU, launch error, ...)  */
#define PD_ENOMEM (-3)    /* device or host allocation failed                       */
#define PD_EIO (-4)       /* file missing, unreadable or not in the expected schema */
#define PD_ETIMEOUT (-5)  /* pd_sync: the bounded wait ran out                      */
#define PD_EDEVICE (-6)   /* the device raised its error word (NaN, list overflow)  */
#define PD_ECONFIG (-7)   /* config file could not be opened                        */
#define PD_ESTATE (-8)    /* call not valid in the handle's current state           */

/* ---- precision forms ------------------------------------------------------------ */
#define PD_FP64 0         /* plain FP64, same operation order as the reference        */
#define PD_FP32C 1        /* FP32 bond forces, cancellation-free stretch, Kahan sums  */

/* ---- device error word bits (pd_device_errors) ----------------------------------- */
#define PD_DERR_NONFINITE 1u      /* a NaN/Inf force density was produced             */
#define PD_DERR_CAND_OVERFLOW 2u  /* not raised: a node with more contact candidates than
                                     its list holds takes them from the cell list (same
                                     results) and the lists grow at the next pd_step      */
#define PD_DERR_CONTACT_OVERFLOW 4u /* more in-range contacts than the per-node cap   */
#define PD_DERR_STAGE_TIMEOUT 8u    /* a shared-memory staging copy missed its wait limit
                                       (the block used global loads; results unaffected) */
#define PD_DERR_BARRIER_TIMEOUT 16u /* a block of the persistent step (launch mode 3) waited
                                       longer than 2 s at a grid barrier; the launch stopped
                                       there and the state is not a step boundary's */

/*
 * pd_config: the run parameters of `main.conf`. Field names, meanings, defaults and
 * sentinels (-1 = "not set" for the contact overrides and new_snot, -999 = "not set"
 * for wall positions) follow ConfigVal (src/read/read_config.h:14-167). Booleans are
 * int32 (0/1).
 */
typedef struct pd_config {
  uint32_t timesteps;                 /* default 8000 */
  uint32_t modulo;                    /* default 100  */
  double dt;                          /* default 0.02/1e5 */
  int32_t is_parallel;
  int32_t do_resume, wall_resume;
  uint32_t resume_ind;                /* default 50 */
  int32_t save_file;                  /* default 1 */
  int32_t enable_fracture;            /* default 0 */
  int32_t nl_bdry_only;               /* default 0 */
  int32_t allow_damping, allow_friction; /* default 1, 1 */
  double normal_stiffness, damping_ratio, friction_coefficient; /* -1: use setup file */
  double new_snot;                    /* -1: keep per-particle snot */
  int32_t self_contact;               /* default 1 */
  double self_contact_rad;            /* -1 (parsed, unused on the path) */
  int32_t enable_cohesion;            /* parsed, unused on the path */
  double cohesion_scaling;
  int32_t enable_torque;
  int32_t set_torque_timestep, set_fracture_timestep, set_self_contact_timestep;
  int32_t set_zero_wall_speed_timestep, set_damping_timestep;
  int32_t set_movable_index, set_movable_timestep;
  int32_t set_stoppable_index, set_stoppable_timestep;
  int32_t reset_partzero_y;
  uint32_t reset_partzero_y_timestep;
  double wheel_rad;
  int32_t particle_w_fixed_velocity, set_fix_velocity_timestep;
  int32_t fix_velocity_angular;
  double prescribed_angular_vel;
  int32_t fix_velocity_mean_x;
  double prescribed_velocity_mean_x;
  double wall_left, wall_right, wall_top, wall_bottom;            /* 2D names, -999 */
  double wall_x_min, wall_y_min, wall_z_min, wall_x_max, wall_y_max, wall_z_max;
  double speed_wall_left, speed_wall_right, speed_wall_top, speed_wall_bottom;
  double speed_wall_x_min, speed_wall_y_min, speed_wall_z_min;
  double speed_wall_x_max, speed_wall_y_max, speed_wall_z_max;
  int32_t brazil;
  int32_t brazil_reset_wall_bottom_freq, brazil_nonzero_wall_bottom_speed_freq;
  double brazil_reset_wall_bottom_y;
  int32_t forcefield_type;
  double forcefield_scaling;
  int32_t gradient_extforce;
  uint32_t extforce_maxstep;
  int32_t compute_wall_reaction;
  char setup_filename[1024];          /* default "data/hdf5/all.h5"  (-i) */
  char output_dir[1024];              /* default "output/hdf5/"      (-o) */
  uint32_t n_unknown_keys;            /* keys the parser reported as "Wrong config name" */
} pd_config;

/*
 * pd_setup_arrays: the setup schema (exp_dict.py:2119-2185, read by
 * src/read/load_hdf5.h:41-181) as caller-owned host arrays. Particles are concatenated
 * in file order (P_00000, P_00001, ...): particle p owns nodes
 * [node_offset[p], node_offset[p+1]) of every per-node array. Connectivity rows use
 * particle-local node indices (i < j, sorted, as written by exp_dict.py:567).
 */
typedef struct pd_setup_arrays {
  uint32_t n_particles;
  const uint64_t *node_offset;      /* n_particles+1 */
  const double *pos;                /* N*3 */
  const double *vol;                /* N   */
  const double *disp, *vel, *acc;   /* N*3 initial data */
  const double *extforce;           /* N*3 */
  const uint64_t *conn_offset;      /* n_particles+1, rows of Connectivity */
  const uint32_t *conn;             /* M*2 local pairs */
  const uint64_t *bdry_offset;      /* n_particles+1 (may be NULL: no bdry lists) */
  const uint32_t *bdry;             /* local node ids */
  const uint64_t *clamped_offset;   /* n_particles+1 (may be NULL) */
  const uint32_t *clamped;          /* local node ids */
  const double *delta, *rho, *cnot, *snot, *torque_val; /* per particle */
  const int32_t *movable, *breakable, *stoppable;        /* per particle */
  const uint32_t *torque_axis;                           /* per particle */
  double contact_radius, normal_stiffness, damping_ratio, friction_coefficient;
  int32_t allow_wall;
  int32_t n_geom_wall;              /* 6 in 3D; 1 means "no wall geometry" */
  double geom_wall_info[6];         /* x_min y_min z_min x_max y_max z_max */
} pd_setup_arrays;

typedef struct pd_sim pd_sim;

/* Per-step counters read back by pd_get_stats. */
typedef struct pd_stats {
  uint64_t step;                 /* the step counter t of the last completed step     */
  uint64_t live_bonds;           /* live directed bonds at the start of the last step */
  uint64_t pairwise_computations;/* particle pairs evaluated, summed since last read  */
  uint64_t contacts;             /* node-node contact pairs applied in the last step  */
  uint64_t rebuilds;             /* contact broad-phase rebuilds so far               */
  uint32_t device_errors;        /* PD_DERR_* bits                                    */
} pd_stats;

/* ---- configuration (replaces ConfigVal + read_file, read_config.h:102-435) -------- */
int pd_config_default(pd_config *cfg);
/* Parses `key = value` lines (whitespace removed, '#' comments). Unknown keys print
 * "[Error]: Wrong config name: <key> !!" to stderr and are counted, like read_config.h:425. */
int pd_config_read(const char *path, pd_config *cfg);

/* ---- simulation handles ----------------------------------------------------------- */
/* Copies the arrays to the device, applies the config the way simulate3d.cpp:125-139
 * and the apply_config methods (timeloop.h:184-225, contact.h:151-179, 325-372) do,
 * builds the bond lists (load_hdf5.h:27-37 + particle2.h:241-257) and initial AABBs
 * (timeloop.h:389-393). `precision` is PD_FP64 or PD_FP32C. The arrays are read during
 * the call only; the handle keeps no pointer to them. Every per-node array in and out of
 * a handle is in the setup's node order (the device layout's own order is internal). */
int pd_create_from_arrays(const pd_setup_arrays *setup, const pd_config *cfg,
                          int precision, pd_sim **out);
/* Reads main.conf + setup.h5 and prepares outdir, like simulate3d -c -i -o. */
int pd_open(const char *conf, const char *setup_h5, const char *outdir, int precision,
            pd_sim **out);
/* Runs the whole configured time loop with saves (run_timeloop, timeloop.h:395-965). */
int pd_run(pd_sim *sim);
/* Enqueues `nsteps` explicit steps (timeloop.h:395-797) on the handle's stream. */
int pd_step(pd_sim *sim, uint32_t nsteps);
/* Bounded wait for the handle's stream; PD_ETIMEOUT when timeout_ms passes first,
 * PD_EDEVICE when the device error word is set. timeout_ms < 0 waits without limit;
 * timeout_ms == 0 only polls (PD_ETIMEOUT while work is still queued). */
int pd_sync(pd_sim *sim, int timeout_ms);
/* Uses an external CUDA stream (cudaStream_t passed as void*; NULL = handle's own). */
int pd_set_stream(pd_sim *sim, void *cuda_stream);

/* ---- state access (all arrays N*3 in particle file order; any pointer may be NULL) -- */
int pd_num_nodes(const pd_sim *sim, uint64_t *n_nodes, uint32_t *n_particles);
int pd_get_state(pd_sim *sim, double *curpos, double *vel, double *acc, double *force);
int pd_get_disp(pd_sim *sim, double *disp);
/* pd_get_state and pd_get_disp in one call (the displacement is read from the device once). */
int pd_get_node_state(pd_sim *sim, double *curpos, double *vel, double *acc, double *force, double *disp);
/* applied_force_density (N*3): non-zero on the particle_w_fixed_velocity particle once the
 * velocity constraint is on (timeloop.h:760-764, saved at timeloop.h:844-848). */
int pd_get_applied_force_density(pd_sim *sim, double *afd);
/* Damage per node (N, file order), the field the reference's plotting derives from a saved
 * frame (examples/3D-HPC-aggregate-particle-breakage/plot3d_timestep.py:95-105, 156-166):
 * (bonds in the setup's Connectivity - bonds in the Connectivity pd_get_connectivity would
 * return) / bonds in the setup's Connectivity, each pair counted at both of its nodes. A node
 * without bonds in the setup gets NaN (0/0), as it does there. Computed on the device. */
int pd_get_damage(pd_sim *sim, double *damage);
/* Overwrites the kinematic state (resume from a frame, timeloop.h:262-312). */
int pd_set_state(pd_sim *sim, const double *disp, const double *vel, const double *acc);
/* Connectivity (local i<q pairs of live bonds) of one particle, as NbdArr2conn
 * (timeloop.h:20-44). With pairs == NULL only *n is returned. */
int pd_get_connectivity(pd_sim *sim, uint32_t particle, uint32_t *pairs, uint64_t cap,
                        uint64_t *n);
/* Wall geometry lrtb() (6) and reaction (6*3, x_min..z_max order of get_reaction). */
int pd_get_wall(pd_sim *sim, double *wall_info, double *reaction);
/* Particle AABBs as used by the next step (get_minmax, contact.h:1187-1225): P*6. */
int pd_get_aabb(pd_sim *sim, double *lrtb);
int pd_get_stats(pd_sim *sim, pd_stats *stats);
/* Writes tc_%05u.h5 and wall_%05u.h5 for `counter` into the output dir. */
int pd_write_frame(pd_sim *sim, uint32_t counter);
/* Loads CurrPos/vel/acc (and, with enable_fracture, Connectivity) of tc_%05u.h5 and, with
 * wall_resume, wall_%05u.h5 from the output dir (run_timeloop's resume, timeloop.h:262-312). */
int pd_resume(pd_sim *sim, uint32_t resume_ind, int wall_resume);
/* Text of the last error of pd_open / pd_run / pd_write_frame / pd_resume / pd_h5_*. */
const char *pd_files_error(void);

/* ---- HDF5 files of the schema (subset reader/writer, no libhdf5 needed) ---------------
 * dtype codes: 1 f64, 2 i32, 3 u32, 4 i64, 5 u64, 6 f32. Paths like "P_00000/Pos". */
void *pd_h5_writer_new(void);
int pd_h5_writer_add(void *w, const char *path, int dtype, int rank, const uint64_t *dims, const void *data);
int pd_h5_writer_write(void *w, const char *filename);
void pd_h5_writer_free(void *w);
void *pd_h5_open(const char *filename);
size_t pd_h5_list(void *h, char *buf, size_t cap);
int pd_h5_info(void *h, const char *path, int *rank, uint64_t *dims);
int pd_h5_read(void *h, const char *path, int dtype, void *out, uint64_t cap_bytes);
void pd_h5_close(void *h);
/* Text of the last error on this handle (never NULL). */
const char *pd_last_error(const pd_sim *sim);
/* Text of the last error of a call that could not return a handle. */
const char *pd_global_error(void);
int pd_close(pd_sim *sim);

/* Tuning knobs: contact skin as a fraction of the contact radius (<= 0 keeps it), per-node
 * candidate capacity (0 keeps it, at most 64; capacity never changes results: a node with more
 * candidates walks the broad phase's cell list instead, and after a pd_sync that saw one the
 * next pd_step doubles the capacity, up to 64), threads per block (<= 0 keeps it), per-step
 * statistics on/off (< 0 keeps it; on adds the pair-count kernel), step launch mode
 * (< 0 keeps it; 0 separate launches, 1 one CUDA graph per step, the FP64 default below 131,072
 * nodes, 2 the same graph with the broad-phase rebuild kernels in a conditional node, the
 * default above: fewer launches per step, but the conditional node itself costs a few
 * microseconds, which small handles feel; 3 all steps of a pd_step call in persistent
 * cooperative launches of one block per SM (up to 1024 steps each), the FP32C default below
 * 131,072 nodes, for handles without reset_partzero_y, prescribed-velocity or torque particles
 * and with statistics off -- others step as in mode 2. A persistent launch occupies every SM
 * while it runs: handles stepping concurrently on other streams wait for it, so small handles
 * that step at the same time (a server's cohorts) should use mode 1. Its grid barriers wait at
 * most 2 s each (PD_DERR_BARRIER_TIMEOUT). All modes give the same results). */
int pd_set_tuning(pd_sim *sim, double skin_frac, uint32_t cand_cap, int threads_per_block,
                  int stats, int use_graphs);
/* Clears the device error word after the caller has handled it. */
int pd_clear_device_errors(pd_sim *sim);

/* Algorithmic byte count of one step (4.125 B per live directed bond + 224 B per node). */
double pd_step_bytes(const pd_sim *sim);
/* Phase timing (the reference's per-block wall clock, timeloop.h:909-947, per kernel
 * phase): runs nsteps real steps as separate launches with CUDA events between phases and
 * returns the summed device milliseconds in phase_ms[4] = {predictor, broad phase, fused
 * force+corrector kernel, end-of-step}. */
int pd_profile_steps(pd_sim *sim, uint32_t nsteps, double *phase_ms);
/* Autotuner: times every bond-kernel variant (loads issued per group, minimum blocks per SM,
 * lanes per node) for steps_per_variant steps from the same snapshot of the live state, restores
 * the state and keeps the fastest; then times the launch modes of pd_set_tuning the same way (the
 * persistent step with 1, 2 and 4 lanes per node, where it applies); then, where the contact
 * candidate lists were rebuilt while the chosen mode stepped, the contact skin at 1.5 and 2 times
 * its value (over at least 24 steps each). Results do not depend on the variant or the mode: every form sums a node's bonds in
 * the same four blocks of its row, merged in the same order. variant_ms (may be NULL) receives
 * pd_num_variants() timings in ms per step. */
int pd_autotune(pd_sim *sim, uint32_t steps_per_variant, int *chosen, double *variant_ms);
int pd_set_variant(pd_sim *sim, int variant);
int pd_num_variants(void);
/* Lanes per node in the bond phase of the persistent step (launch mode 3): 1, 2 or 4, or 0 (the
 * default) to choose by size: 4 where four threads per node all fit on the device at once, else
 * 1 (one lane per node, each partner record requested one group of bonds ahead of its use). More
 * lanes shorten a node's chain of gathers on handles too small to fill the GPU; results do not
 * depend on it (each node's bond sum is taken in four blocks of its row, merged in a fixed
 * order). pd_autotune times 1, 2 and 4. */
int pd_set_persist_lanes(pd_sim *sim, int lanes);
int pd_persist_lanes(const pd_sim *sim);
/* How steps are launched: 0 separate launches, 1 one CUDA graph per step, 2 a step graph whose
 * broad-phase rebuild kernels sit in a conditional node, 3 persistent launches of up to 1024
 * steps each (see pd_set_tuning). */
int pd_graph_mode(const pd_sim *sim);
/* Copy of all device state that stepping changes, and its restore (checkpoint in HBM). */
int pd_snapshot(pd_sim *sim);
int pd_restore(pd_sim *sim);
/* Live directed bonds of movable particles (the bond-update count of the next step). */
int pd_count_live_bonds(pd_sim *sim, uint64_t *live);
/* Same count as pd_count_live_bonds, but allocating nothing: for callers that must not call
 * cudaMalloc -- a monitor polling a running simulation (cudaMalloc would synchronise the
 * device under the step pipeline) or an application that has handed all free HBM to resident
 * simulations. Scratch lives in a static 32 KB device array shared by all calls on a device
 * (concurrent calls race; each call overwrites what it reads). At most 1,048,576 nodes, larger
 * handles get PD_EINVAL. The first call on a device looks up the array's address; make it
 * before any stream capture, with the simulation's device current. This entry point has no
 * counterpart in the reference. */
int pd_count_live_bonds_noalloc(pd_sim *sim, uint64_t *live);

/* ---- batches of independent simulations (serving) -------------------------------------
 * The reference runs one simulation per process (run/simulate3d.cpp:37-176); these entry
 * points have no counterpart there. A batch handle holds n_sims simulations, each with its
 * own setup and main.conf values, concatenated in one device layout: every phase of a step
 * is one launch over all of them and nothing couples two of them, so each computes exactly
 * what it computes in a handle of its own. pd_step advances every simulation that is not
 * finished. Simulation i's nodes are [node0, node0+n_nodes) of the handle's nodes and
 * its particles [particle0, particle0+n_particles) (pd_get_connectivity takes handle
 * particle indices). Errors of these calls are reported by pd_global_error(). */
int pd_create_batch(const pd_setup_arrays *setups, const pd_config *cfgs, uint32_t n_sims,
                    int precision, pd_sim **out);
/* Device bytes pd_create_batch would allocate for these setups (host work only: it runs
 * without a GPU). PD_EINVAL where pd_create_batch would refuse a Connectivity index out of
 * range. */
int pd_estimate_bytes(const pd_setup_arrays *setups, uint32_t n_sims, int precision,
                      uint64_t *bytes);
/* Device bytes a handle holds; free and total memory of the current device. */
int pd_device_bytes(const pd_sim *sim, uint64_t *bytes);
int pd_device_memory(uint64_t *free_bytes, uint64_t *total_bytes);
int pd_num_sims(const pd_sim *sim, uint32_t *n_sims);
int pd_sim_range(const pd_sim *sim, uint32_t i, uint64_t *node0, uint64_t *n_nodes,
                 uint32_t *particle0, uint32_t *n_particles);
/* Steps simulation i has taken. */
int pd_sim_steps(const pd_sim *sim, uint32_t i, uint64_t *steps);
/* Ends simulation i at the current step boundary: waits for the handle's stream, reads its
 * state and walls back into host memory (kept by the handle) and stops stepping it. Later
 * reads of simulation i return that state. */
int pd_finish_sim(pd_sim *sim, uint32_t i);
/* State of simulation i alone (N_i*3 arrays in its own node order; pointers may be NULL). */
int pd_get_sim_state(pd_sim *sim, uint32_t i, double *curpos, double *vel, double *acc,
                     double *force);
int pd_get_sim_disp(pd_sim *sim, uint32_t i, double *disp);
int pd_get_sim_wall(pd_sim *sim, uint32_t i, double *wall_info, double *reaction);
/* Damage of simulation i alone (N_i, its own node order; pd_get_damage's definition). */
int pd_get_sim_damage(pd_sim *sim, uint32_t i, double *damage);
/* Eviction and re-admission. pd_save_sim writes a checkpoint of simulation i at the current
 * step boundary into host memory: everything stepping changes (displacement, velocity,
 * acceleration, force, each particle's live bonds as its Connectivity, walls and their
 * reactions, step counter, scheduled toggles, the FP32 form's records and predicted step).
 * *bytes receives its size; with buf == NULL only the size is returned, else cap must hold it.
 * It extends the reference's resume (timeloop.h:262-312, which reloads CurrPos, vel, acc,
 * Connectivity and the wall from a frame) to an exact continuation: the displacement is saved
 * as such (not as CurrPos - pos) together with the rest of the state. A finished simulation
 * (pd_finish_sim) cannot be saved (PD_ESTATE). The handle may be closed afterwards: its device
 * memory returns at pd_close. */
int pd_save_sim(pd_sim *sim, uint32_t i, void *buf, uint64_t cap, uint64_t *bytes);
/* Loads such a checkpoint into simulation i of a handle (a batch or single handle) whose
 * simulation i was created from the same setup and config in the same precision form
 * (PD_EINVAL otherwise), at a step boundary of that handle. From then on simulation i computes
 * exactly what the saved simulation would have computed had it stepped on; the other
 * simulations of the handle are not touched. */
int pd_load_sim(pd_sim *sim, uint32_t i, const void *buf, uint64_t bytes);

/* ---- bond lists on the GPU (setup generation) -----------------------------------------
 * For each particle p (nodes [node_offset[p], node_offset[p+1]) of pos, N*3), every node pair
 * (i, j), i < j, particle-local indices, with ((dx*dx + dy*dy) + dz*dz) <= r*r, r = radius[p],
 * sorted by (i, j): the Connectivity the reference's setup scripts build with
 * sorted(cKDTree(pos).query_pairs(delta)) (exp_dict.py:542-567), pair for pair where scipy
 * evaluates that expression without fused multiply-adds (its x86 builds).
 * pair_offset (n_particles+1) receives the pair count prefix; with pairs == NULL only the
 * counts are computed, otherwise cap must hold pair_offset[n_particles] pairs (PD_EINVAL if
 * not). Runs on the current device. Errors: pd_pairs_error(). */
int pd_query_pairs(const double *pos, const uint64_t *node_offset, const double *radius,
                   uint32_t n_particles, uint32_t *pairs, uint64_t cap, uint64_t *pair_offset);
/* near[q] = 1 for every node q within radius[p] of a node of its particle p with marked[] set
 * (the marked nodes themselves included), else 0: the nonlocal boundary nodes the reference's
 * setup scripts find by scanning every node for every edge node (gen_nonlocal_boundry_nodes,
 * exp_dict.py:1231-1248), with its test sqrt((dx*dx + dy*dy) + dz*dz) <= r in FP64 without
 * contraction. marked and near hold one byte per node; same inputs and errors as pd_query_pairs. */
int pd_query_near(const double *pos, const uint64_t *node_offset, const double *radius, uint32_t n_particles,
                  const uint8_t *marked, uint8_t *near);
const char *pd_pairs_error(void);

#ifdef __cplusplus
}
#endif
#endif /* PERIDEM_GB300_H */
