/* ldo.h - C ABI of the GB300 lattice DNA-origami Monte Carlo engine.
 *
 * The reference (cumberworth/LatticeDNAOrigami) is one C++ program with no
 * plugin or FFI layer; its hot path is reached through C++ classes.  Each
 * entry point below replaces one of those calls for a batch of replicas that
 * live on one GPU:
 *
 *   ldo_create_from_inp   origami::setup_origami + GCMCSimulation ctor
 *                         (src/origami_system.cpp:991, src/simulation.cpp:182)
 *   ldo_set_controls      OrigamiSystem::update_temp / update_staple_us
 *                         (src/origami_system.cpp:618-628)
 *   ldo_run               GCMCSimulation::simulate (src/simulation.cpp:568)
 *   ldo_get_observables   OrigamiSystem counters + energy + SystemBiases
 *                         (include/.../origami_system.hpp:99-130)
 *   ldo_get_config        OrigamiSystem::chains (src/origami_system.cpp:175)
 *   ldo_set_config(s)     OrigamiSystem ctor from given chains
 *                         (src/origami_system.cpp:588-615, 991-1003)
 *   ldo_read_trj_frame    OrigamiTrajInputFile::read_config (src/files.cpp:129)
 *   ldo_checkpoint_*      restart_traj_file + .randstate + .swp restart
 *                         (src/origami_system.cpp:1000, src/simulation.cpp:204,
 *                         src/ptmc_simulation.cpp:62)
 *   ldo_pt_run            PTGCMCSimulation::run (src/ptmc_simulation.cpp:106)
 *
 * Conventions: every call is synchronous at return; input buffers are
 * copied; output buffers are caller-allocated; no C++ exception crosses the
 * ABI; the engine is not thread-safe (one host thread per engine).  Random
 * numbers follow one Philox4x32-10 stream per replica, key (seed, replica).
 */
#ifndef LDO_H
#define LDO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ldo_engine ldo_engine;

typedef enum {
    LDO_OK = 0,
    LDO_EINVAL = 1,      /* bad argument or input file (reference: FileError, OrigamiMisuse at load) */
    LDO_ENOMEM = 2,      /* device or host allocation failed */
    LDO_ECUDA = 3,       /* CUDA runtime error */
    LDO_EINVARIANT = 4,  /* a replica hit a state the reference throws on (OrigamiMisuse, SimulationMisuse) */
    LDO_EITERCAP = 5,    /* a data-dependent loop reached its iteration cap */
    LDO_ECAPACITY = 6    /* a replica needed more staple or lattice slots than allocated */
} ldo_status;

/* Per-replica observables, as the reference's log block reports them
 * (src/simulation.cpp:667-704). */
typedef struct {
    double energy;            /* OrigamiSystem::energy(), kT units            */
    double total_bias;        /* SystemBiases::get_total_bias()               */
    double temp;              /* current temperature (K)                      */
    double enthalpy;          /* update_enthalpy_and_entropy: H / T           */
    double entropy;           /*                              S               */
    double stacking;          /*                              stacking energy */
    int64_t draws;            /* random numbers consumed                      */
    int32_t num_staples;
    int32_t num_fully_bound;  /* NumBoundDomainPairs order parameter          */
    int32_t num_bound;        /* bound + misbound pairs                       */
    int32_t num_self_bound;
    int32_t num_stacked;
    int32_t num_unassigned;
    int32_t current_c_i;      /* next unique chain index - 1                  */
    int32_t status;           /* ldo_status of this replica                   */
} ldo_observables;

/* Creates n_replicas copies of the system described by a reference .inp file
 * (key=value, src/parser.cpp option names).  `overrides` holds extra
 * key=value lines applied after the file (may be NULL).  Replica r draws from
 * Philox key (seed, r). */
ldo_status ldo_create_from_inp(const char* inp_path, const char* overrides, int n_replicas, uint32_t seed,
                               ldo_engine** out);

/* Like ldo_create_from_inp, but replica r is a copy of system
 * sys_of_replica[r] taken from inp_paths[] (uneven sizes in one batch). */
ldo_status ldo_create_multi(const char* const* inp_paths, int n_systems, const char* overrides,
                            const int* sys_of_replica, int n_replicas, uint32_t seed, ldo_engine** out);

void ldo_destroy(ldo_engine* e);

/* Last error message of this engine (or of the last failed create if e is NULL). */
const char* ldo_last_error(const ldo_engine* e);

int ldo_num_replicas(const ldo_engine* e);

/* Per-replica temperature, stacking multiplier and staple chemical-potential
 * multiplier.  Rebuilds the energy tables and recomputes every replica's
 * energy by unassigning and reassigning all domains, like
 * OrigamiSystem::update_temp (src/origami_system.cpp:618).  NULL arrays keep
 * the current values. */
ldo_status ldo_set_controls(ldo_engine* e, const double* temps, const double* stacking_mults,
                            const double* staple_u_mults, int n);

/* Each replica performs n_steps move attempts (GCMCSimulation::simulate).
 * If device_ms is non-NULL it receives the kernel time measured with CUDA
 * events on the engine's stream. */
ldo_status ldo_run(ldo_engine* e, int64_t n_steps, double* device_ms);

/* Each replica performs n_sweeps sweeps of n_scaffold move attempts (its own
 * scaffold length); sampling intervals then count sweeps. */
ldo_status ldo_run_sweeps(ldo_engine* e, int64_t n_sweeps, double* device_ms);

/* Bytes of device state per replica (the shared-memory footprint of one warp). */
int ldo_state_bytes(const ldo_engine* e);

ldo_status ldo_get_observables(ldo_engine* e, ldo_observables* out, int n);

/* Configuration of one replica: n_chains, then per chain (index, identity,
 * length, length x (x, y, z, ox, oy, oz, state)).  *written receives the
 * number of ints; LDO_EINVAL if cap is too small. */
ldo_status ldo_get_config(ldo_engine* e, int replica, int32_t* buf, int cap, int* written);

/* Replaces one replica's configuration with buf (ldo_get_config's format;
 * the states are ignored): the replica is rebuilt as the OrigamiSystem
 * constructor builds a system from given chains (energy, counters, order
 * parameters and biases of the new configuration) and keeps its
 * random-number position, step counter and move statistics.  A
 * configuration that violates a constraint returns LDO_EINVAL ("Constaints
 * in violation after move complete") and leaves the replica unchanged. */
ldo_status ldo_set_config(ldo_engine* e, int replica, const int32_t* buf, int n);

/* Annealing (AnnealingGCMCSimulation::run, src/annealing_simulation.cpp:40):
 * temperatures max_temp, max_temp - temp_interval, ... down to min_temp; at
 * each, every replica gets that temperature (stacking multiplier 1; staple
 * chemical-potential multiplier 1 unless constant_staple_M) and runs
 * steps_per_temp steps.  LDO_EINVAL "Bad temperature interval" when
 * temp_interval does not divide max_temp - min_temp, as the reference throws.
 * The .inp keys of the same names hold the reference's values. */
ldo_status ldo_anneal_run(ldo_engine* e, double max_temp, double min_temp, double temp_interval,
                          int64_t steps_per_temp, int constant_staple_M, double* device_ms);

/* Every replica at once, with one device launch: bufs holds n_replicas
 * configurations in ldo_get_config's format, replica r's in
 * [offsets[r], offsets[r+1]) (offsets has n_replicas + 1 entries).  All or
 * nothing: a violating configuration returns LDO_EINVAL naming the replica
 * and leaves every replica unchanged. */
ldo_status ldo_set_configs(ldo_engine* e, const int32_t* bufs, const int32_t* offsets, int n_replicas);

/* Frame `frame` (0 = first written) of a .trj trajectory file in
 * ldo_get_config's format, states 0 (OrigamiTrajInputFile::read_config,
 * src/files.cpp:129).  Host only; error text via ldo_last_error(NULL).
 * The .inp keys restart_traj_file / restart_step start every replica of a
 * system from such a frame, as the reference's setup_origami does. */
ldo_status ldo_read_trj_frame(const char* path, int frame, int32_t* buf, int cap, int* written);

/* Checkpoint / resume: one binary file with every replica's state
 * (configuration, counters, random-number position, move statistics), its
 * controls (temperature, multipliers, windows, centres, grid biases, seed),
 * the learned proposal's table and network, and a parallel-tempering
 * ladder's permutation, swap counter, swap random-number positions and
 * statistics.  An engine created from the same input files with the same
 * replica count loads it and continues bit for bit as the saved engine
 * would have; LDO_EINVAL for a file of other systems, or one that is
 * truncated or corrupt (the header carries the payload's length and FNV-1a
 * hash).  Sample and trace
 * buffers, the .swp history and umbrella-sampling iterations are not saved. */
ldo_status ldo_checkpoint_save(ldo_engine* e, const char* path);
ldo_status ldo_checkpoint_load(ldo_engine* e, const char* path);

/* Order-parameter sampling: every `interval` steps each replica appends
 * (num_fully_bound, num_staples) to a ring of `capacity` samples. */
ldo_status ldo_set_sampling(ldo_engine* e, int interval, int capacity);
/* Copies samples[replica][k][2] (int16) for the first min(count, capacity). */
ldo_status ldo_get_samples(ldo_engine* e, int16_t* out, int capacity, int* count);

/* Work counters since the engine was created (no reference counterpart: the
 * end-to-end accounting of a caller): kernel launches of the MC, exchange,
 * status and enumeration kernels (a replayed CUDA graph counts the kernels
 * it holds; network training is not counted), and bytes copied host to
 * device and device to host.  Any pointer may be NULL. */
ldo_status ldo_get_counters(ldo_engine* e, int64_t* launches, int64_t* h2d_bytes, int64_t* d2h_bytes);

/* Step trace for replicas [0, n_trace): per step 8 doubles (step, energy,
 * staples, fully bound, bound, stacked, total bias, draws). */
ldo_status ldo_set_trace(ldo_engine* e, int n_trace, int max_steps);
ldo_status ldo_get_trace(ldo_engine* e, double* out, int n_trace, int max_steps);

/* Per-move attempts/accepts summed over replicas: out[2*m], out[2*m+1]. */
ldo_status ldo_get_move_stats(ldo_engine* e, int64_t* out, int n_moves);

/* Grid-bias values for bias function `tag` (1-D over the order parameter
 * value 0..n-1) of one replica, or of all replicas if replica < 0
 * (GridBiasFunction::replace_biases, src/bias_functions.cpp:237). */
ldo_status ldo_set_grid_bias(ldo_engine* e, const char* tag, int replica, const double* values, int n);

/* Window restraint of one replica for a SquareWell bias `tag`
 * (SquareWellBiasFunction::set_min_op/set_max_op, src/bias_functions.cpp:218-220). */
ldo_status ldo_set_window(ldo_engine* e, const char* tag, int replica, int min_op, int max_op);

/* Centre of one replica's Harmonic bias `tag` (engine extension: the
 * reference has no harmonic bias; 0.5 k (x - centre)^2 restrains an umbrella
 * window).  Like ldo_set_window, the new bias enters at the next move. */
ldo_status ldo_set_bias_centre(ldo_engine* e, const char* tag, int replica, double centre);

/* Parallel tempering: `swaps` rounds of (update controls, exchange_interval
 * steps, exchange attempt between neighbouring control slots), the 1-D
 * even/odd schedule of PTGCMCSimulation::run / OneDPTGCMCSimulation::
 * attempt_exchange (src/ptmc_simulation.cpp:106-412).  Replicas are split
 * into n_ladders independent ladders of n_rungs consecutive replicas.
 * `exchange_q` selects the exchanged controls as a bit set:
 * 1 = temperature, 2 = staple chemical potential, 4 = bias multiplier,
 * 8 = stacking multiplier (T: 1, uT: 3, HuT: 7, ST: 9). */
ldo_status ldo_pt_run(ldo_engine* e, int n_rungs, int64_t swaps, int exchange_interval, int exchange_q,
                      double* device_ms);

/* Two-dimensional parallel tempering over temperature x stacking multiplier
 * (TwoDPTGCMCSimulation, src/ptmc_simulation.cpp:428-560): the .inp's temps
 * and stacking_mults span n_temps x n_stacking slots (slot i * n_stacking + j),
 * pairs are attempted in the reference's four alternating sets (even / odd
 * along temperature, even / odd along stacking), and temperature, staple
 * chemical potential and stacking multiplier are exchanged.  Replicas form
 * ladders of n_temps * n_stacking consecutive replicas. */
ldo_status ldo_pt2d_run(ldo_engine* e, int n_temps, int n_stacking, int64_t swaps, int exchange_interval,
                        double* device_ms);

/* Current control-slot to replica permutation (the .swp file row) for all
 * ladders: out[ladder * n_rungs + slot] = replica. */
ldo_status ldo_pt_get_permutation(ldo_engine* e, int32_t* out, int n);
/* Swap attempts and acceptances summed over ladders: per neighbouring slot
 * pair i (n_pairs = n_rungs - 1) for a 1-D ladder; for a 2-D ladder per
 * direction v (0 temperature, 1 stacking) and lower slot (i, j),
 * index v * n_temps * n_stacking + i * n_stacking + j (n_pairs =
 * 2 * n_temps * n_stacking, the reference's m_attempt_count[v][i][j]). */
ldo_status ldo_pt_get_stats(ldo_engine* e, int64_t* attempts, int64_t* accepts, int n_pairs);

/* Multi-window umbrella sampling with adaptive grid biases
 * (MWUSGCMCSimulation::run / PTMWUSGCMCSimulation::run with the updates of
 * SimpleUSGCMCSimulation, src/us_simulation.cpp:84-434, 454-864).  Window w
 * starts on replica w; the windows and their square-well bias come from the
 * system's windows_file (none: one unrestrained window per replica).  After
 * equil_steps, each of n_iters iterations runs iter_steps steps, counting the
 * grid point of `grid_tag` after every step, then sets each visited point's
 * bias to ln of its reweighted probability, changes limited to max_D_bias.
 * exchange_interval > 0 attempts neighbouring-window exchanges every that
 * many steps (PTMWUS); window assignments move, configurations stay.  A
 * second call with the same grid_tag continues the iterations (biases,
 * visited points, windows and exchange stream kept; ldo_us_reset starts
 * over); ldo_checkpoint_save/load carry that state between processes, as the
 * reference's restart_us_iter archives do. */
ldo_status ldo_us_run(ldo_engine* e, const char* grid_tag, int n_iters, int64_t equil_steps, int64_t iter_steps,
                      double max_D_bias, int exchange_interval, double* device_ms);
/* USGCMCSimulation::output_weights (src/us_simulation.cpp:208): the grid
 * biases of window `window` (every point visited or read) as a .biases JSON
 * file in the reference's layout. */
ldo_status ldo_us_write_biases(ldo_engine* e, int window, const char* path);
/* USGCMCSimulation::read_weights (src/us_simulation.cpp:192, the read_biases
 * restart): the grid biases of window `window` from a .biases file; sets up
 * the umbrella state of grid bias grid_tag if there is none.  The .inp keys
 * read_biases / biases_file / biases_filebase do the same for every window
 * when ldo_us_run sets up (biases_filebase + "_win-<min>--<max>.biases" with
 * a windows file, as MWUSGCMCSimulation::setup_window_sims names them). */
ldo_status ldo_us_read_biases(ldo_engine* e, const char* grid_tag, int window, const char* path);
/* Drops the umbrella-sampling state: the next ldo_us_run starts from zero
 * biases (ldo_us_run otherwise continues the iterations of the last one). */
ldo_status ldo_us_reset(ldo_engine* e);
/* read_weights without an engine: n entries of dimension dim; points[i*dim+j],
 * biases[i] (pass NULL buffers to get n and dim only). */
ldo_status ldo_read_biases(const char* path, int32_t* points, double* biases, int cap, int* n, int* dim);
/* Grid biases per window: out[w * grid_len + point]. */
ldo_status ldo_us_get_biases(ldo_engine* e, double* out, int n_windows, int grid_len);
/* Window held by each replica, and the grid length. */
ldo_status ldo_us_get_windows(ldo_engine* e, int32_t* window_of_replica, int n, int* grid_len);

/* enumerate_main with enumerate_staples_only (src/enumerate.cpp:19-81): the
 * exact partition function of replica 0's system at its temperature over
 * every staple configuration on the fixed scaffold, with min_total..max_total
 * staples and at most max_type of a type (the .inp's min_total_staples,
 * max_total_staples, max_type_staples), the reference's growth-point sets
 * and overcount corrections.  The staple sets times growth-point sets are
 * enumerated on the GPU in parallel.  weights[k1 * n2 + k2] receives the
 * normalised weight of (op1, op2) = (k1, k2) (order parameter tags), the
 * reference's .weights entries; num_configs its number of configurations.
 * The system starts without staples and has no bias functions. */
ldo_status ldo_enumerate(ldo_engine* e, int32_t min_total, int32_t max_total, int32_t max_type, const char* op1_tag,
                         const char* op2_tag, int32_t n1, int32_t n2, double* weights, double* num_configs,
                         int32_t* n_units, double* device_ms);

/* enumerate_main without enumerate_staples_only (src/enumerate.cpp:19-81,
 * ConformationalEnumerator::enumerate, :218): the scaffold is unassigned and
 * enumerated too, from its first domain at the origin, as the reference's
 * full enumeration does, with the same staple sets, growth-point sets and
 * overcount corrections.  Each unit is split into 6^split_levels parts (0..4)
 * by the branch its recursion takes at its first split_levels choices
 * (sites and orientations), which run in parallel. */
ldo_status ldo_enumerate_full(ldo_engine* e, int32_t min_total, int32_t max_total, int32_t max_type,
                              const char* op1_tag, const char* op2_tag, int32_t n1, int32_t n2, int32_t split_levels,
                              double* weights, double* num_configs, int32_t* n_units, double* device_ms);

/* The last enumeration's weights unit by unit: out[(u * n1 + k1) * n2 + k2]
 * the unnormalised weight of (op1, op2) = (k1, k2) within unit u (cap: room
 * for n_units * n1 * n2 doubles; NULL out: count only). */
ldo_status ldo_enumerate_unit_weights(ldo_engine* e, double* out, int64_t cap, int32_t* n_units);

/* The last ldo_enumerate's work units (the reference's growth-point sets, in
 * its enumeration order): out[2u] the unit's partition-function sum before
 * normalisation, out[2u+1] its number of configurations (NULL out: count
 * only). */
ldo_status ldo_enumerate_units(ldo_engine* e, double* out, int32_t cap, int32_t* n_units);

/* The work units an enumeration of the system in inp_path (with overrides,
 * as ldo_create takes them) would run, listed on the host without a GPU:
 * StapleEnumerator::enumerate (src/enumerate.cpp:1082) over the staple sets
 * and GrowthpointEnumerator::enumerate (:819) over the growth-point sets
 * without repeats, in the reference's order.  out[2u] the number of staples
 * of unit u, out[2u+1] its number of growth points (cap: room for 2 *
 * n_units; NULL out: count only).  Error text via ldo_last_error(NULL). */
ldo_status ldo_enumeration_plan(const char* inp_path, const char* overrides, int32_t min_total, int32_t max_total,
                                int32_t max_type, int32_t* out, int32_t cap, int32_t* n_units);

/* No counterpart in the reference: the engine's autotuner of the MC kernel's
 * launch shape (the reference runs one replica per MPI process and has no
 * launch shape).  Times probe_sweeps sweeps of this engine's own batch for
 * every candidate -- 1, 2 or 4 replicas (warps) per block, each number of
 * resident blocks per SM the occupancy calculator allows (set through extra
 * shared memory per block), replicas in the given order or interleaved over
 * the systems -- best of two probes each, restores the replicas' state after
 * every probe (tuning changes no trajectory), and keeps the fastest shape for
 * the following runs.  With use_cache, a shape found before in this process
 * for the same capacity class, systems and replica count is reused without
 * probing. */
typedef struct {
    int32_t warps_per_block;
    int32_t smem_pad_bytes;
    int32_t blocks_per_sm;      /* resident blocks per SM of the chosen shape */
    int32_t interleaved;        /* 1: replicas interleaved over the systems */
    double best_ms;             /* probe time of the chosen shape */
    double default_ms;          /* probe time of the shape before tuning */
    int32_t n_candidates;
} ldo_tune_report;
ldo_status ldo_autotune(ldo_engine* e, int32_t probe_sweeps, int32_t use_cache, ldo_tune_report* out);
/* The candidates of the last probing autotune: shape[4k..4k+3] = warps per
 * block, padding bytes, blocks per SM, interleaved; ms[k] its probe time. */
ldo_status ldo_autotune_candidates(ldo_engine* e, int32_t* shape, double* ms, int32_t cap);

/* No counterpart in the reference.  Status of every replica without
 * allocating: for a caller that may not allocate device memory at this point
 * (its own pool allocator owns all device memory, or its step loop must not
 * stall the device on cudaMalloc/cudaFree).  Writes each replica's status
 * (an ldo_status code) to status_of_replica[n] (may be NULL), the largest to
 * *worst and the number of nonzero ones to *n_bad; n must equal the replica
 * count and be at most 65536 (LDO_EINVAL otherwise).  Its scratch is a fixed
 * 256 KiB device array of the library, shared by every call.  Each call looks
 * up the array's device address anew (a device reset can move it); the first
 * call on a device may also load the library's device code, so make that
 * first call before any stream capture.  Do not let two calls overlap on the
 * GPU (they race on the array).  Returns after the results are in host
 * memory. */
ldo_status ldo_replica_status_noalloc(ldo_engine* e, int32_t* status_of_replica, int n, int32_t* worst,
                                      int32_t* n_bad);

/* No counterpart in the reference.  The engine's exponential, y[i] =
 * exp(x[i]) for i < n, evaluated on the GPU: the function every acceptance
 * probability and Rosenbluth weight of the engine uses (Tang's table-driven
 * method, about half a unit in the last place), with the same bits as its
 * host version, so that host code can repeat the engine's decisions exactly.
 * The reference uses the C library's exp instead.  Allocates and frees two
 * device buffers of n doubles. */
ldo_status ldo_engine_exp(const double* x, double* y, int n);

/* Learned proposals (movetypes "LearnedStapleExchange" and
 * "LearnedStapleRegrowth"; engine extensions with no counterpart in the
 * reference, which only proposes uniformly: src/movetypes.cpp:98-140).  A
 * network of three 256-wide GELU layers scores growth-point targets from their
 * chain neighbourhood and the temperature, and the six sites a regrown staple
 * domain can take from what they hold; ldo_learn.h describes the input
 * encoding.  Until trained, every input weighs 1. */

/* Adds every replica's current bound / unbound domains and the sites of its
 * placed staple domains to the training counts (per network input). */
ldo_status ldo_learn_collect(ldo_engine* e);
ldo_status ldo_learn_reset_counts(ldo_engine* e);
/* Training counts per network input (n = LDO_LEARN_TABLE = 524544: 524288
 * insertion inputs, then 256 regrowth-direction inputs, ldo_learn.h). */
ldo_status ldo_learn_get_counts(ldo_engine* e, float* cnt_bound, float* cnt_total, int n);
/* Full-batch Adam (lr) on the weighted logistic loss of the counts, starting
 * from seeded parameters the first time; then the proposal's weight table.
 * Loss before the first and after the last step (either may be NULL). */
ldo_status ldo_learn_train(ldo_engine* e, int iters, double lr, uint32_t seed, double* loss_first, double* loss_last);
/* Network parameters (n = LDO_LEARN_NPARAM = 148481 floats); setting them
 * recomputes the weight table. */
ldo_status ldo_learn_set_params(ldo_engine* e, const float* params, int n);
ldo_status ldo_learn_get_params(ldo_engine* e, float* params, int n);
/* Proposal weight exp(clamped logit) of every network input (n = 524544). */
ldo_status ldo_learn_get_table(ldo_engine* e, double* weights, int n);
ldo_status ldo_learn_set_table(ldo_engine* e, const double* weights, int n);
/* Loss and gradient of the network for given parameters on a batch of n
 * network inputs with bound / total counts (no engine; the GPU kernels the
 * trainer uses). */
ldo_status ldo_learn_loss_grad(const float* params, const int32_t* idx, const float* cnt_bound, const float* cnt_total,
                               int n, double* loss, float* grad);

/* Output files of one replica in the reference's formats and file names
 * (setup_output_files, src/simulation.cpp:47-147; writers src/files.cpp:
 * 519-789): <filebase>.vsf at open, then on every ldo_writer_write the
 * replica's current state, for the kinds set in `kinds`: 1 .trj, 2 .vcf
 * .states .ores, 4 .counts .staples .staplestates, 8 .ene, 16 .ops (the
 * .inp's ops_to_output, or every order parameter), 32 .times (wall seconds
 * since the writer was opened, as the reference's seconds since the start of
 * its run). */
typedef struct ldo_writer ldo_writer;
ldo_status ldo_writer_open(ldo_engine* e, int replica, const char* filebase, uint32_t kinds, ldo_writer** out);
ldo_status ldo_writer_write(ldo_writer* w, int64_t step);
void ldo_writer_close(ldo_writer* w);

/* The .swp file of one ladder of parallel tempering
 * (PTGCMCSimulation::initialize_swap_file / write_swap_entry,
 * src/ptmc_simulation.cpp:91,315): opens <filebase>.swp and writes the
 * header (the exchanged controls of every slot, as the reference's
 * "temp/u/ " columns), sets up the ladder as ldo_pt_run(n_rungs, exchange_q)
 * would and starts recording the permutation (slot -> replica within the
 * ladder) before every exchange attempt of later ldo_pt_run calls.
 * ldo_writer_write(w, step) appends the recorded rows whose step is a
 * multiple of freq (the reference's configs_output_freq) and, when step >= 0
 * and a multiple of freq, the current permutation as the end-of-run row (the
 * reference writes it once at the end of its run; pass -1 to only append the
 * recorded rows).  The device keeps the last 4096 rows per ladder: write at
 * least that often.  Close with ldo_writer_close. */
ldo_status ldo_swap_writer_open(ldo_engine* e, int n_rungs, int exchange_q, int ladder, const char* filebase,
                                int64_t freq, ldo_writer** out);

/* Batches split by capacity class (no reference counterpart: the reference
 * runs one system per process).  A batch holds replicas of several systems
 * like ldo_create_multi, but groups them by the state-layout class each
 * system needs on its own (small, medium, large) and gives every group its
 * own engine: its own layout, kernel instantiation (scaffold moves compiled
 * in only where a group's systems use them) and launch shape.  A run forks
 * one MC launch per group from the batch's stream onto the groups' streams
 * and joins them, so the groups run concurrently.  Replica r keeps the
 * random stream of replica r of one engine holding the whole batch: the
 * trajectories equal those of ldo_create_multi with the same arguments. */
typedef struct ldo_batch ldo_batch;
ldo_status ldo_batch_create(const char* const* inp_paths, int n_systems, const char* overrides,
                            const int* sys_of_replica, int n_replicas, uint32_t seed, ldo_batch** out);
void ldo_batch_destroy(ldo_batch* b);
const char* ldo_batch_last_error(const ldo_batch* b);   /* NULL batch: last failed create */
int ldo_batch_num_groups(const ldo_batch* b);
/* Group g: its class (LDO_CLASS_S/M/L = 0/1/2), replica count, the batch
 * indices of its replicas (n_rep entries; may be NULL) and its engine, owned
 * by the batch, for every other engine call on that group. */
ldo_status ldo_batch_group(ldo_batch* b, int g, int* cls, int* n_rep, int32_t* replicas, ldo_engine** engine);
/* As ldo_set_controls / ldo_run / ldo_run_sweeps / ldo_set_sampling /
 * ldo_get_samples / ldo_get_counters over the whole batch (arrays indexed by
 * batch replica); device_ms spans the fork and join of all groups. */
ldo_status ldo_batch_set_controls(ldo_batch* b, const double* temps, const double* stacking_mults,
                                  const double* staple_u_mults, int n);
ldo_status ldo_batch_run(ldo_batch* b, int64_t n_steps, double* device_ms);
ldo_status ldo_batch_run_sweeps(ldo_batch* b, int64_t n_sweeps, double* device_ms);
ldo_status ldo_batch_set_sampling(ldo_batch* b, int interval, int capacity);
ldo_status ldo_batch_get_samples(ldo_batch* b, int16_t* out, int capacity, int* count);
ldo_status ldo_batch_get_counters(ldo_batch* b, int64_t* launches, int64_t* h2d_bytes, int64_t* d2h_bytes);
/* ldo_autotune of every group on its own replicas: out[g] for g < n groups. */
ldo_status ldo_batch_autotune(ldo_batch* b, int32_t probe_sweeps, int32_t use_cache, ldo_tune_report* out, int n);

/* Host-only helpers (no GPU needed). */

/* Reduced hybridisation enthalpy H/(RT) and entropy S/R of a fully paired
 * duplex with top strand `seq` (nearestNeighbour::
 * calc_unitless_hybridization_thermo, src/nearest_neighbour.cpp:34). */
ldo_status ldo_nn_duplex_thermo(const char* seq, double temp, double cation_M, double* h, double* s);

/* Energy tables of the system of an .inp file at (temp, stacking_mult), as
 * OrigamiPotential::calc_energies builds them (src/origami_potential.cpp:1057):
 * dense (2*imax+1)^2 row-major arrays over identity pairs (i+imax, j+imax) of
 * hybridisation free energy, enthalpy, entropy and stacking energy (kT units),
 * and init[3] = initiation enthalpy, entropy, free energy.  *imax receives the
 * largest |identity|; arrays must hold cap doubles. */
ldo_status ldo_energy_tables(const char* inp_path, double temp, double stacking_mult, int* imax, double* hyb_e,
                             double* hyb_h, double* hyb_s, double* stack, double* init, int cap);

#ifdef __cplusplus
}
#endif
#endif /* LDO_H */
