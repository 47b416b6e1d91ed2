/*
 * brawl_gpu.h -- C ABI of the GB300 (sm_103a) implementation of BraWl's
 * lattice-sampling hot path.
 *
 * The entry points replace, call for call, the procedures that BraWl's
 * Fortran host reaches through its procedure pointers and its one existing
 * C binding.  Each declaration names the reference interface it replaces
 * (paths relative to the BraWl repository root).  Everything is plain C:
 * pointers, sizes and int status codes; no CUDA or C++ types cross the
 * boundary, and every call is synchronous unless its name ends in _async.
 *
 * Data layouts are the reference's own (Fortran, column-major):
 *   config  int8  config(1, 2*n_1, 2*n_2, 2*n_3), x fastest; empty sites 0,
 *                 species 1..n_species (src/initialise.F90:286-298)
 *   V_ex    double V_ex(n_species, n_species, interaction_range) in Ry
 *                 (src/shared_data.f90:37, read by src/io.f90:389-402)
 *   sites   int[4] (b, i, j, k), 1-based, as returned by *_random_site
 *   rho     double rho(n_species, n_species, wc_range)
 *
 * Errors: the reference stops the program (e.g. src/initialise.F90:168,
 * :205, :237); these functions return a status instead and leave their
 * outputs untouched.  brawl_last_error() describes the most recent failure
 * on the calling thread.
 */
#ifndef BRAWL_GPU_H
#define BRAWL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define BRAWL_OK 0
#define BRAWL_EINVAL 1        /* unsupported lattice / shells / sizes / species */
#define BRAWL_ENOMEM 2        /* device memory exhausted */
#define BRAWL_ECUDA 3         /* CUDA runtime failure (no device, launch error) */
#define BRAWL_ETIMEDOUT 4     /* a serving request did not finish in time */
#define BRAWL_ECANCELLED 5    /* a serving request was cancelled */
#define BRAWL_ESTATE 6        /* a device-side consistency check failed */
#define BRAWL_EAGAIN 7        /* a serving request has not finished yet */

/* ---- lattice codes (setup%lattice, src/initialise.F90:157-243) ----------- */
#define BRAWL_SIMPLE_CUBIC 0  /* interaction_range 1-2 */
#define BRAWL_BCC 1           /* interaction_range 1-10 */
#define BRAWL_FCC 2           /* interaction_range 1-6 */

/* The subset of run_params (src/derived_types.f90:56-100) the path needs. */
typedef struct brawl_setup {
    int lattice;              /* BRAWL_SIMPLE_CUBIC / BRAWL_BCC / BRAWL_FCC */
    int n_1, n_2, n_3;        /* conventional cells per direction */
    int n_species;            /* 1..15 */
    int interaction_range;    /* coordination shells in the Hamiltonian */
} brawl_setup;

/* Counters returned per chain (all 64-bit):
 *   [0] trials  [1] trials whose species differed  [2] 32-bit words drawn
 *   [3] accepted  [4] trials that drew the acceptance uniform
 *   [5] trials decided with the FP64 reference-order sums
 *   [6] exp/log decisions that needed the FP64 libm value
 *   [7] ... and the double-double value */
#define BRAWL_NUM_COUNTERS 8

const char *brawl_last_error(void);
int brawl_version(void);

/* ====================================================================== */
/* Single chain: one simulation as the reference runs it in one process. */
/* ====================================================================== */
typedef struct brawl_ctx brawl_ctx;

/* initialise_function_pointers + initialise_interaction + read_exchange
 * (src/initialise.F90:153-257, :267-273; src/io.f90:389-402): validates the
 * lattice and shell count and keeps V_ex on the device. */
int brawl_ctx_create(const brawl_setup *setup, const double *V_ex, brawl_ctx **out);
int brawl_ctx_destroy(brawl_ctx *ctx);
/* Replace V_ex (same shape). */
int brawl_set_interactions(brawl_ctx *ctx, const double *V_ex);

/* init_genrand(seed) (src/mt19937ar.c:63-78) on the chain's own stream. */
int brawl_seed(brawl_ctx *ctx, uint32_t seed);
/* f90_init_genrand (src/mt19937ar.c:127-142): static seed 110179+11*rank or
 * a time-based one; returns the seed used. */
int brawl_f90_init_genrand(brawl_ctx *ctx, int seedtime, int my_rank, uint32_t job_id,
                           uint32_t *seed_out);
/* The generator state as the reference holds it: mt[624] then mti. */
int brawl_rng_get(brawl_ctx *ctx, uint32_t state[625]);
int brawl_rng_set(brawl_ctx *ctx, const uint32_t state[625]);
/* n calls of genrand() (src/mt19937ar.c:121-125) from the chain's stream. */
int brawl_genrand(brawl_ctx *ctx, int64_t n, double *out);

/* config in and out, reference layout (see above). */
int brawl_set_config(brawl_ctx *ctx, const int8_t *config);
int brawl_get_config(brawl_ctx *ctx, int8_t *config);

/* initial_setup (src/initialise.F90:434-617) on the device, consuming the
 * chain's stream exactly as the reference does.  species_concentrations has
 * n_species+1 entries with [0] = 0 (the reference's 0:n_species array) and
 * is rewritten, as the reference rewrites it, when species_numbers (may be
 * NULL) sums to the number of atoms. */
int brawl_initial_setup(brawl_ctx *ctx, double *species_concentrations,
                        const int64_t *species_numbers);

/* total_energy (src/bw_hamiltonian.f90:58-81), bit-identical. */
int brawl_total_energy(brawl_ctx *ctx, double *energy);
/* nbr_energy of one site (the setup%nbr_energy pointer,
 * src/derived_types.f90:90-98), 1-based (b, i, j, k). */
int brawl_site_energy(brawl_ctx *ctx, const int idx[4], double *energy);
/* pair_energy (src/bw_hamiltonian.f90:99-114). */
int brawl_pair_energy(brawl_ctx *ctx, const int idx1[4], const int idx2[4], double *energy);

/* n_trials calls of monte_carlo_step_lattice (nbr_swap = 0) or
 * monte_carlo_step_nbr (nbr_swap = 1) at inverse temperature beta
 * (src/metropolis.F90:751-891).  accepted (may be NULL) receives the sum of
 * their accept results, i.e. what the reference adds to `acceptance`. */
int brawl_metropolis_run(brawl_ctx *ctx, double beta, int64_t n_trials, int nbr_swap,
                         int64_t *accepted);
/* The sweep loop of metropolis_simulated_annealing with its energy samples
 * (src/metropolis.F90:348-367): n_sweeps blocks of sweep_trials trials at
 * inverse temperature beta, and after each block the chain's total_energy,
 * written to energies[n_sweeps] (may be NULL: no energies).  The blocks run
 * back to back on the device; each block's energy is taken from a copy of
 * the lattice while the next block runs.  accepted (may be NULL) receives
 * the accepted moves of all blocks.  Trajectory and results are what
 * n_sweeps pairs of brawl_metropolis_run + brawl_total_energy give. */
int brawl_anneal_sweeps(brawl_ctx *ctx, double beta, int64_t n_sweeps, int64_t sweep_trials, int nbr_swap,
                        double *energies, int64_t *accepted);

/* lattice_shells (src/analytics.f90:205-275) of the current config. */
int brawl_lattice_shells(brawl_ctx *ctx, int wc_range, double *shells);
/* radial_densities (src/analytics.f90:293-404), bit-identical. */
int brawl_radial_densities(brawl_ctx *ctx, int wc_range, const double *shells, double *rho);
/* ALRO (store_state, src/analytics.f90:43-64): add the configuration's
 * occupancies to a device accumulator; read it as
 * order(species, basis, 2n1, 2n2, 2n3) (species fastest, empty cells 0);
 * zero it (the reference zeroes it at every temperature). */
int brawl_alro_add(brawl_ctx *ctx);
int brawl_alro_get(brawl_ctx *ctx, double *order);
int brawl_alro_reset(brawl_ctx *ctx);

/* Cumulative counters of this chain (BRAWL_NUM_COUNTERS values). */
int brawl_counters(brawl_ctx *ctx, int64_t *counters);

/* No counterpart in the reference.  The shared-memory bandwidth of the
 * current device in bytes/s (a streaming 16-byte-load kernel on every SM,
 * the best of three timed launches): the ceiling the sampling kernels,
 * whose lattices and tables live in shared memory, are measured against. */
int brawl_smem_bandwidth(double *bytes_per_s);

/* No counterpart in the reference.  The total energy of brawl_total_energy,
 * bit-identical, for callers that cannot allocate device memory -- a host
 * that gives all device memory to its own pool at start-up, or one that
 * records its GPU work into a CUDA graph and must finish allocating before
 * recording.  d_V_ex, d_config (reference layout) and d_energy (one double)
 * are device memory the caller owns; nothing is allocated or freed.  The
 * per-site scratch is one fixed array of 524288 doubles (4 MiB) inside the
 * library, held by every device that loads it until the process exits;
 * lattices with more sites are rejected with BRAWL_EINVAL.  The work is
 * queued on `stream` (a cudaStream_t, NULL for the default stream) and the
 * call returns without waiting.  The first call made with a given CUDA
 * context current (per device, its primary context for runtime-API callers)
 * does a one-time set-up of that context, so make it before any stream
 * capture.  Calls share the scratch array: calls that overlap on the GPU
 * race.  The config must hold species 1..n_species on every lattice site. */
int brawl_total_energy_noalloc(const brawl_setup *setup, const double *d_V_ex,
                               const int8_t *d_config, double *d_energy, void *stream);

/* ====================================================================== */
/* Batches: many independent chains (replicas, temperatures, walkers) of  */
/* uneven lattice, species and shell counts, run together -- the          */
/* reference's MPI replica ensemble (src/comms.F90:122-160) on one GPU.   */
/* ====================================================================== */
typedef struct brawl_batch brawl_batch;

typedef struct brawl_chain_desc {
    brawl_setup setup;
    const double *V_ex;                    /* copied at create */
    uint32_t seed;                         /* init_genrand seed of this chain */
    double beta;                           /* 1/(k_B T) in 1/Ry */
    int nbr_swap;
    const double *species_concentrations;  /* n_species+1 ([0] = 0) */
    const int64_t *species_numbers;        /* n_species or NULL */
    const int8_t *config;                  /* start config, or NULL for initial_setup */
} brawl_chain_desc;

/* Seeds every chain, then sets its configuration (copying `config`, or by
 * initial_setup on the device when config is NULL). */
int brawl_batch_create(const brawl_chain_desc *chains, int n_chains, brawl_batch **out);
int brawl_batch_destroy(brawl_batch *batch);
int brawl_batch_size(brawl_batch *batch, int *n_chains);
/* New inverse temperatures, one per chain. */
int brawl_batch_set_beta(brawl_batch *batch, const double *beta);
/* Trials per speculative round of the fcc/bcc Metropolis kernel (1-4, 1 =
 * one trial at a time, the default).  Speed only: the trajectory is the same. */
int brawl_batch_set_speculation(brawl_batch *batch, int trials_per_round);
/* Picks the trials per round by measurement: n_trials[c] trials of every
 * chain are timed at each depth 1..max_depth (<= 4) from the same state,
 * which is restored after each run, so the batch's chains, streams and
 * counters are as before the call.  ms (max_depth entries, may be NULL)
 * gets each depth's time; chosen (may be NULL) the depth kept. */
int brawl_batch_autotune(brawl_batch *batch, const int64_t *n_trials, int max_depth, double *ms,
                         int *chosen);
/* Shared-memory chains are grouped in classes (same lattice, n1, n2, n3,
 * species and shells); after this call every class runs in its own launch,
 * concurrently with the others, with its own shared memory, unrolling and
 * trials per round.  The depths are picked per class by timing the whole
 * batch (n_trials[c] trials of every chain, three runs per try, from the
 * same state, restored after each): the classes in order of decreasing
 * work, each class's depths 1..max_depth with the others fixed, a deeper
 * round kept only when 2% faster.  depths (n_classes entries, may be NULL)
 * gets the choice, ms (n_classes * max_depth, may be NULL) the median time
 * of every try, n_classes (may be NULL) the class count.  Speed only: the
 * trajectories do not depend on the depths. */
int brawl_batch_autotune_classes(brawl_batch *batch, const int64_t *n_trials, int max_depth,
                                 int *depths, double *ms, int *n_classes);
/* Trials per round of every class (n_classes entries, 1-4 each), set by
 * the caller; every class then runs in its own launch as above. */
int brawl_batch_set_class_depths(brawl_batch *batch, const int *depths);
/* The class of every chain (-1: not a shared-memory chain). */
int brawl_batch_chain_classes(brawl_batch *batch, int *classes);
/* n_trials[c] Metropolis trials on every chain c, all chains in one launch.
 * accepted (may be NULL) receives each chain's accept sum for this call. */
int brawl_batch_metropolis_run(brawl_batch *batch, const int64_t *n_trials, int64_t *accepted);
/* Same, queued on `stream` (a cudaStream_t, or NULL for the batch's own
 * stream) without waiting; brawl_batch_sync waits for it. */
int brawl_batch_metropolis_run_async(brawl_batch *batch, const int64_t *n_trials, void *stream);
int brawl_batch_sync(brawl_batch *batch);
/* The plain path: chains run one at a time, one launch per chain. */
int brawl_batch_metropolis_run_serial(brawl_batch *batch, const int64_t *n_trials,
                                      int64_t *accepted);
int brawl_batch_total_energy(brawl_batch *batch, double *energies);
int brawl_batch_get_config(brawl_batch *batch, int chain, int8_t *config);
int brawl_batch_set_config(brawl_batch *batch, int chain, const int8_t *config);
/* Every chain's config at once: the reference-layout grids of all chains
 * concatenated in chain order (the host side of the ensemble). */
int brawl_batch_get_configs(brawl_batch *batch, int8_t *configs);
int brawl_batch_set_configs(brawl_batch *batch, const int8_t *configs);
/* Sampling sums of metropolis_simulated_annealing kept on the device for
 * every chain (src/metropolis.F90:360-430): the FP64 sums step_E and
 * step_Esq of the sampled total energies, the sums r_densities of the
 * sampled radial densities (wc_range >= 1; every chain must then have the
 * same species count) and the accepted count at the start of the sampling
 * loop.  brawl_batch_sampling_reset zeroes them (call it after a
 * temperature's burn-in); brawl_batch_energy_sample adds every chain's
 * total_energy (returned in energies[n] when not NULL, for trajectories);
 * brawl_batch_asro_sample adds chain c's radial_densities (rho, optional,
 * gets them in the layout of brawl_batch_radial_densities). */
int brawl_batch_sampling_reset(brawl_batch *batch, int wc_range);
int brawl_batch_energy_sample(brawl_batch *batch, double *energies);
/* brawl_anneal_sweeps for every chain of a batch (each at its own beta and
 * nbr_swap): n_sweeps blocks of sweep_trials trials per chain; after each
 * block every chain's total_energy goes to energies[sweep * n + chain]
 * (when not NULL) and, with accumulate = 1, into the sampling sums as
 * brawl_batch_energy_sample adds it.  accepted[n] (may be NULL) receives
 * each chain's accepted moves over all blocks. */
int brawl_batch_anneal_sweeps(brawl_batch *batch, int64_t n_sweeps, int64_t sweep_trials, int accumulate,
                              double *energies, int64_t *accepted);
int brawl_batch_asro_sample(brawl_batch *batch, int chain, const double *shells, double *rho);
/* The temperature's results (src/metropolis.F90:410-428): per_chain[3n] =
 * energies_of_T (n), C_of_T (n), acceptance_of_T (n), computed on the
 * device from the sums with the reference's arithmetic; average[3] = each
 * summed over the chains in chain order and divided by real(n), as
 * comms_reduce_metropolis_results averages the ranks (src/comms.F90:
 * 122-160).  with_energies = 0: energies_of_T and C_of_T are 0. */
int brawl_batch_temperature_stats(brawl_batch *batch, int64_t n_save_energy, int64_t n_mc_steps,
                                  double temp, double sim_temp, int with_energies,
                                  double *per_chain, double *average);
/* rho_of_T = r_densities / n_save_asro per chain (per_chain[n * wc*ns*ns])
 * and its average over the chains (average[wc*ns*ns]), as above. */
int brawl_batch_asro_stats(brawl_batch *batch, int64_t n_save_asro, double *per_chain,
                           double *average);

/* set_configs, metropolis_run and get_configs as one call from host
 * buffers (every chain's grid, as set_configs takes them; configs_out may be
 * configs_in): page-locked buffers are read and written in place by the
 * kernels (no staging copy), others go through a device copy.  One wait at
 * the end.  A bad species in configs_in fails the call (BRAWL_ESTATE)
 * before any trial runs. */
int brawl_batch_metropolis_host(brawl_batch *batch, const int8_t *configs_in, const int64_t *n_trials,
                                int8_t *configs_out, int64_t *accepted);
int brawl_batch_rng_get(brawl_batch *batch, int chain, uint32_t state[625]);
int brawl_batch_counters(brawl_batch *batch, int64_t *counters /* n_chains * 8 */);
int brawl_batch_lattice_shells(brawl_batch *batch, int chain, int wc_range, double *shells);
int brawl_batch_alro_add(brawl_batch *batch);                       /* every chain */
int brawl_batch_alro_get(brawl_batch *batch, int chain, double *order);
int brawl_batch_alro_reset(brawl_batch *batch);
int brawl_batch_radial_densities(brawl_batch *batch, int chain, int wc_range,
                                 const double *shells, double *rho);

/* ====================================================================== */
/* Nested sampling (src/nested_sampling.f90:45-206): independent runs,   */
/* each with its own stream, walkers resident on the device.             */
/* ====================================================================== */
typedef struct brawl_ns brawl_ns;

typedef struct brawl_ns_desc {
    brawl_setup setup;
    const double *V_ex;
    uint32_t seed;                         /* init_genrand seed of the run */
    int n_walkers;                         /* ns_params%n_walkers */
    int n_steps;                           /* ns_params%n_steps */
    const double *species_concentrations;  /* n_species+1 ([0] = 0) */
    const int64_t *species_numbers;        /* n_species or NULL */
} brawl_ns_desc;

/* Seeds each run and draws its walkers as the reference does: for every
 * walker initial_setup then one genrand() for the 1e-8 energy jitter; the
 * walker energies are total_energy + jitter (nested_sampling.f90:78-98). */
int brawl_ns_create(const brawl_ns_desc *runs, int n_runs, brawl_ns **out);
int brawl_ns_destroy(brawl_ns *ns);
/* n_iter iterations of every run (nested_sampling.f90:114-200); limits
 * receives each iteration's ceiling, run-major (n_runs x n_iter). */
int brawl_ns_iterate(brawl_ns *ns, int n_iter, double *limits);
/* The walkers' energies of one run (n_walkers doubles). */
int brawl_ns_energies(brawl_ns *ns, int run, double *energies);
/* One walker's configuration, reference layout. */
int brawl_ns_walker_config(brawl_ns *ns, int run, int walker, int8_t *config);
/* Counters of one run (BRAWL_NUM_COUNTERS values: [0] walk steps,
 * [2] words drawn, [3] accepted steps, [5] steps that needed the FP64 sums). */
int brawl_ns_counters(brawl_ns *ns, int run, int64_t *counters);

/* ====================================================================== */
/* Wang-Landau walkers (src/wang-landau.F90): sweeps of every walker and  */
/* the in-window average that follows them, with ln g, the histograms,    */
/* the configurations and the streams resident on the device.             */
/* ====================================================================== */
typedef struct brawl_wl brawl_wl;

typedef struct brawl_wl_desc {
    brawl_setup setup;
    const double *V_ex;
    uint32_t seed;                         /* the walker's (rank's) stream */
    const int8_t *config;                  /* start config (reference layout) */
    int start_idx, end_idx;                /* 1-based window bins (window_indices) */
    int window;                            /* walkers of a window are averaged together */
    int nbr_swap;                          /* wl_params%nbr_swap: site 2 a random nearest
                                              neighbour of site 1 (select_sites_nbr,
                                              src/wang-landau.F90:1527-1532) */
} brawl_wl_desc;

/* Walkers of one Wang-Landau simulation; bin_edges has bins+1 entries
 * (create_energy_bins, src/wang-landau.F90:969-992).  Walkers of the same
 * window must be consecutive; ln g starts at zero. */
int brawl_wl_create(const brawl_wl_desc *walkers, int n_walkers, int bins,
                    const double *bin_edges, brawl_wl **out);
int brawl_wl_destroy(brawl_wl *wl);
/* sweeps() on every walker (src/wang-landau.F90:539-632): e_unswapped from
 * full_energy, n_trials = mc_sweeps*n_atoms trials adding wl_f to ln g, a
 * histogram tick every hist_period trials, then ln g and the histograms
 * averaged over the walkers of each window.  accepted (may be NULL)
 * receives each walker's accepted moves.  BRAWL_ESTATE if a walker's
 * energy is outside its window (the reference would index outside its
 * histogram). */
int brawl_wl_sweeps(brawl_wl *wl, int64_t n_trials, double wl_f, int hist_period,
                    int64_t *accepted);  /* n_trials < 2^31 */
/* dos_average (src/wang-landau.F90:1127-1133): ln g averaged over the
 * walkers of each window (histograms untouched). */
int brawl_wl_average(brawl_wl *wl);
/* replica_exchange (src/wang-landau.F90:1392-1501, shuffle_rows :1513-1525)
 * with walker w in the role of MPI rank w: every window must hold the same
 * number of walkers and windows must be in ascending energy order.  The
 * candidate lists are shuffled on walker 0's stream; a matched lower walker
 * draws genrand() < exp(lng(i) - lng(j)) from its own stream; accepted
 * pairs swap configurations.  partner / exchanged (n_walkers each, may be
 * NULL): the walker paired with each walker (-1 for none) and whether its
 * configuration was swapped; n_accepted (may be NULL): accepted pairs. */
int brawl_wl_replica_exchange(brawl_wl *wl, int *partner, int *exchanged, int *n_accepted);
/* Per-walker flatness minval(hist)/(sum(hist)/window_bins)
 * (src/wang-landau.F90:222). */
int brawl_wl_flatness(brawl_wl *wl, double *flatness);
/* dos_combine (src/wang-landau.F90:1147-1194): the windows' ln g (first
 * walker of each window) stitched where the slopes agree best and shifted
 * to a zero minimum; every walker's ln g becomes the result (the
 * reference's MPI_BCAST).  lng (bins, may be NULL) receives it.
 * BRAWL_ESTATE when a window has no overlap with the previous one. */
int brawl_wl_dos_combine(brawl_wl *wl, double *lng);
/* mpi_wl_hist = 0 for every walker. */
int brawl_wl_reset_hist(brawl_wl *wl);
int brawl_wl_get_lng(brawl_wl *wl, int walker, double *lng);        /* bins */
int brawl_wl_set_lng(brawl_wl *wl, int walker, const double *lng);
int brawl_wl_get_hist(brawl_wl *wl, int walker, double *hist);      /* window bins */
int brawl_wl_set_hist(brawl_wl *wl, int walker, const double *hist);
int brawl_wl_energies(brawl_wl *wl, double *energies);              /* full_energy per walker */
int brawl_wl_get_config(brawl_wl *wl, int walker, int8_t *config);
int brawl_wl_set_config(brawl_wl *wl, int walker, const int8_t *config);
/* Exchange the configurations of two walkers (replica_exchange's swap). */
int brawl_wl_swap_configs(brawl_wl *wl, int a, int b);
/* n genrand() draws from a walker's stream (exchange shuffles and tests). */
int brawl_wl_genrand(brawl_wl *wl, int walker, int64_t n, double *out);
int brawl_wl_counters(brawl_wl *wl, int walker, int64_t *counters);
/* enter_energy_window (src/wang-landau.F90:643-741) for every walker: the
 * biased walk into the inner 80% of the walker's window (energy_min /
 * energy_max the wl_input range in meV/atom, single-precision values as the
 * reference reads them, which set the bias width), on
 * the walker's own stream; with initial != 0 the walk starts from
 * initial_setup(conc, numbers) (numbers may be NULL), which also draws the
 * redraws every n_atoms*250 steps.  steps (n, may be NULL) gets each
 * walker's loop iterations.  The MPI hand-over (the first walker of a window
 * in sends its configuration to the others) is left to the caller.
 * BRAWL_ESTATE when a walker has not entered after max_steps. */
int brawl_wl_enter_windows(brawl_wl *wl, double energy_min, double energy_max, const double *conc,
                           const int64_t *numbers, int initial, int64_t max_steps, int64_t *steps);
/* Radial-density samples inside sweeps() (src/wang-landau.F90:566-586):
 * while a bin's radial_record is under MAX(radial_samples / num_walkers, 1)
 * and its radial_record_bool is unset, every n_atoms-th trial that proposes
 * that bin adds radial_densities(wc_range, shells) of the trial
 * configuration to the walker's rho_of_E(:, :, :, bin).  All walkers must
 * share the lattice.  Enabling zeroes radial_record, rho_of_E,
 * radial_mc_steps and radial_record_bool. */
int brawl_wl_radial_enable(brawl_wl *wl, int wc_range, const double *shells, int radial_samples,
                           int num_walkers);
/* radial_record_bool (bins bytes, 0/1), as save_rho_E sets it; when every
 * bin is set, sampling stops (rho_saved). */
int brawl_wl_radial_set_done(brawl_wl *wl, const uint8_t *done);
/* One walker's radial_record (bins), rho_of_E (bins * wc * ns * ns, i
 * fastest; may be NULL) and radial_mc_steps (may be NULL). */
int brawl_wl_radial_get(brawl_wl *wl, int walker, int32_t *record, double *rho_of_E, int32_t *steps);
/* The configuration store of sweeps() (config_per_bin / config_store,
 * src/wang-landau.F90:60-61, 605-622, 1042-1043, 1109-1110): every walker
 * gets bins slots (bins * n_sites bytes, zeroed) and their flags, all open;
 * from then on, at every histogram tick the walker's configuration goes to
 * the slot of the tick's bin if that bin is still open, which closes it.
 * BRAWL_ENOMEM when the slots do not fit. */
int brawl_wl_store_enable(brawl_wl *wl);
/* The flags (n_walkers * bins bytes, walker-major; 1 = open, i.e. the
 * reference's config_store(bin) = .True.). */
int brawl_wl_store_flags(brawl_wl *wl, uint8_t *open);
/* merge_configs (src/wang-landau.F90:1556-1615) after the caller's draw:
 * pick[bin-1] is the walker whose slot every walker takes for that bin (the
 * rank drawn among those holding it) or -1 when none holds it; the bin's
 * flag becomes closed, or open for -1, in every walker.  The draw is the
 * caller's (the reference uses gfortran's random_number).  All walkers must
 * share the lattice. */
int brawl_wl_store_merge(brawl_wl *wl, const int *pick);
/* load_window_config (src/wang-landau.F90:1541-1554) after the caller's
 * draw of the 1-based bin: the walker's configuration becomes its slot for
 * that bin.  BRAWL_ESTATE when the slot is still open. */
int brawl_wl_store_load(brawl_wl *wl, int walker, int bin);
/* One stored configuration in the config(1, 2n1, 2n2, 2n3) layout. */
int brawl_wl_store_get(brawl_wl *wl, int walker, int bin, int8_t *config);
/* New windows after mpi_window_optimise (src/wang-landau.F90:1211-1328):
 * start_idx / end_idx per window (1-based bins, overlap included as
 * create_overlap gives it), applied to every walker of the window; the
 * histograms restart from 0 as mpi_arrays reallocates them (:1351-1379).
 * ln g is kept.  A walker whose energy then lies outside its window needs
 * a configuration from it (brawl_wl_store_load) before the next sweeps. */
int brawl_wl_set_windows(brawl_wl *wl, const int *start_idx, const int *end_idx);

/* ====================================================================== */
/* Serving: a request loop that admits anneal, Wang-Landau and nested-    */
/* sampling jobs as they arrive and runs every resident job's next        */
/* quantum of work in shared launches (continuous batching).  No          */
/* counterpart in the reference, whose drivers run one simulation per     */
/* process; each job's results equal those of the same job run alone.     */
/* ====================================================================== */
typedef struct brawl_server brawl_server;

typedef struct brawl_server_opts {
    size_t hbm_budget;          /* device bytes for resident jobs (0: 60% of the
                                   memory free at creation) */
    int max_active;             /* resident jobs at most (0: 4096) */
    double round_ms;            /* device time each job's quantum of work aims at,
                                   from the job's measured cost (0: 20 ms) */
    int64_t max_trials;         /* cap on a job's Metropolis / Wang-Landau trials
                                   per round (0: none) */
    int max_iterations;         /* cap on a nested-sampling job's iterations per
                                   round (0: none) */
    int max_active_wl;          /* resident Wang-Landau jobs at most (0: 64) */
    int max_active_ns;          /* resident nested-sampling jobs at most (0: 64);
                                   queued jobs of a kind at its cap wait while
                                   later jobs of other kinds are admitted */
} brawl_server_opts;

#define BRAWL_JOB_ANNEAL 1
#define BRAWL_JOB_WL 2
#define BRAWL_JOB_NS 3

typedef struct brawl_job_desc {
    int kind;                              /* BRAWL_JOB_* */
    brawl_setup setup;
    const double *V_ex;                    /* copied at submission */
    uint32_t seed;
    const double *species_concentrations;  /* n_species+1 ([0] = 0), copied */
    const int64_t *species_numbers;        /* n_species or NULL, copied */
    /* anneal (metropolis_simulated_annealing, src/metropolis.F90:84-558):
     * T_steps temperatures T_start + k*delta_T, sweeps_per_T*n_atoms trials
     * each; the energy is sampled at the end of every temperature. */
    double T_start, delta_T;
    int T_steps;
    int64_t sweeps_per_T;
    /* Wang-Landau window: wl_walkers walkers on one window of wl_bins bins
     * spanning Ec -/+ h (Ry; Ec = the mean of the walkers' initial energies in
     * walker order, h = wl_half_width or 1.25 times the largest |E_k - Ec|
     * when that is larger);
     * wl_calls sweeps() calls of wl_trials trials, ln f starting at wl_f and
     * halved whenever every walker's histogram is flatter than wl_flatness
     * (the histograms then reset); stops early once ln f < wl_tolerance. */
    int wl_walkers, wl_bins, wl_calls;
    int64_t wl_trials;
    double wl_half_width, wl_f, wl_flatness, wl_tolerance;
    /* nested sampling (src/nested_sampling.f90:45-206) */
    int ns_walkers, ns_steps, ns_iter;
} brawl_job_desc;

typedef struct brawl_job_result {
    int status;                 /* BRAWL_OK or the error that ended the job */
    int kind;
    double t_submit, t_admit, t_finish;  /* seconds since the server started */
    double t_ready;             /* device objects built (after admission) */
    int64_t trials;             /* Metropolis trials / WL trials / NS walk steps */
    int64_t accepted;
    double energy;              /* anneal: final energy; WL: walker 0's; NS: last ceiling */
    double wl_f;                /* WL: ln f at the end */
    int wl_halvings;
    int n_values;               /* length of the job's value array */
} brawl_job_result;

int brawl_serve_create(const brawl_server_opts *opts, brawl_server **out);
/* Stops the loop; jobs still queued or running end with BRAWL_ECANCELLED. */
int brawl_serve_destroy(brawl_server *server);
/* Queues a job (its inputs are copied); *id names it in later calls. */
int brawl_serve_submit(brawl_server *server, const brawl_job_desc *job, uint64_t *id);
/* BRAWL_OK with *result filled once the job has ended, BRAWL_EAGAIN before. */
int brawl_serve_poll(brawl_server *server, uint64_t id, brawl_job_result *result);
/* Waits up to timeout_s seconds (< 0: no limit); BRAWL_ETIMEDOUT if the
 * job has not ended by then. */
int brawl_serve_wait(brawl_server *server, uint64_t id, double timeout_s,
                     brawl_job_result *result);
/* The job's values (n_values doubles): anneal -- energy at the end of every
 * temperature then the acceptance ratio of every temperature; WL -- ln g
 * of walker 0 (wl_bins) then the bin edges (wl_bins+1); NS -- the ceiling
 * of every iteration. */
int brawl_serve_values(brawl_server *server, uint64_t id, double *values);
/* The final configuration (reference layout; WL: walker 0; NS: walker 1). */
int brawl_serve_config(brawl_server *server, uint64_t id, int8_t *config);
/* Forgets an ended job. */
int brawl_serve_release(brawl_server *server, uint64_t id);
/* Rounds run and jobs resident/queued/ended so far. */
int brawl_serve_stats(brawl_server *server, int64_t stats[4]);
/* Per pipeline (anneal, Wang-Landau, nested sampling), 5 values each:
 * rounds, seconds from launch to completion seen, seconds spent launching,
 * seconds spent settling, trials handed out (Wang-Landau: summed over the
 * walkers; nested sampling: walk steps at n_steps per iteration, adaptive
 * extra steps not counted). */
int brawl_serve_profile(brawl_server *server, double profile[15]);

#ifdef __cplusplus
}
#endif

#endif /* BRAWL_GPU_H */
