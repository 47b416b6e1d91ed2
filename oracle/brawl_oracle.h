/*
 * brawl_oracle.h -- CPU restatement of BraWl's lattice-sampling hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against (tests/, the smoke check and bench.py's CPU-baseline
 * leg).  Nothing in the brawl_gb300 package links, loads or calls it.
 *
 * Parity status: pinned.  The restatement reproduces the reference's own
 * golden outputs byte-for-byte (tests/99_ref/01_serial_metropolis and
 * tests/99_ref/02_parallel_metropolis of the reference repository), and its
 * Mersenne Twister is cross-checked word-for-word against the reference's
 * src/mt19937ar.c compiled from source.  The nested-sampling golden
 * (tests/99_ref/03_serial_nested_sampling) is not reproduced by the
 * reference's current source with its committed input; the nested-sampling
 * restatement is checked against it statistically, its primitives by the
 * Metropolis goldens.
 *
 * Conventions shared with the reference (Fortran, column-major):
 *   config(1, x, y, z) int8 on the doubled grid 2n1 x 2n2 x 2n3, stored with
 *   x fastest: index = x + 2n1*(y + 2n2*z), all coordinates 0-based here.
 *   V(a, b, shell) double in Ry, index = a + ns*(b + ns*shell), 0-based.
 */
#ifndef BRAWL_ORACLE_H
#define BRAWL_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { BO_SC = 0, BO_BCC = 1, BO_FCC = 2 };

/* ---- mt19937ar (src/mt19937ar.c) ---------------------------------------- */
typedef struct {
    uint32_t mt[624];
    int mti;
} bo_rng;

void bo_rng_seed(bo_rng *r, uint32_t seed);
uint32_t bo_rng_u32(bo_rng *r);
double bo_rng_uniform(bo_rng *r);
uint32_t bo_static_seed(int rank);

/* ---- model --------------------------------------------------------------- */
typedef struct {
    int lattice;            /* BO_SC / BO_BCC / BO_FCC */
    int n1, n2, n3;         /* conventional cells per direction */
    int nsh;                /* interaction_range */
    int ns;                 /* n_species */
    const double *V;        /* V_ex, Ry */
} bo_model;

int bo_n_atoms(const bo_model *m);
int bo_grid_size(const bo_model *m);
int bo_max_shells(int lattice);
int bo_shell_size(int lattice, int shell /* 1-based */);
int bo_shell_offset(int lattice, int shell, int k, int d[3]);

double bo_site_energy(const bo_model *m, const int8_t *cfg, int x, int y, int z);
double bo_pair_energy(const bo_model *m, const int8_t *cfg, const int s1[3], const int s2[3]);
double bo_total_energy(const bo_model *m, const int8_t *cfg);

void bo_random_site(const bo_model *m, bo_rng *r, int site[3]);
void bo_random_nbr(const bo_model *m, bo_rng *r, const int site[3], int nbr[3]);

typedef struct {
    int64_t trials;         /* monte_carlo_step calls */
    int64_t evaluated;      /* trials whose two species differed */
    int64_t draws;          /* 32-bit words drawn */
    int64_t accepted;       /* accept == 1 (includes same-species trials) */
    int64_t exp_tests;      /* trials that drew the acceptance uniform */
} bo_counters;

int bo_mc_step(const bo_model *m, int8_t *cfg, bo_rng *r, double beta,
               int nbr_swap, bo_counters *c);
int64_t bo_mc_run(const bo_model *m, int8_t *cfg, bo_rng *r, double beta,
                  int64_t n_trials, int nbr_swap, bo_counters *c);
/* Same trials, but also returns the per-trial accept flag and the delta-E
 * (NaN for same-species trials), for trial-by-trial comparisons. */
int64_t bo_mc_trace(const bo_model *m, int8_t *cfg, bo_rng *r, double beta,
                    int64_t n_trials, int nbr_swap, int8_t *accept_out,
                    double *de_out, bo_counters *c);

/* initial_setup: conc has ns+1 entries with conc[0] = 0 (index 0..ns as in
 * the reference); it is rewritten when numbers[] sums to n_atoms.  numbers
 * may be NULL.  Returns 0, or -1 when the species counts cannot be made to
 * sum to the number of sites. */
int bo_initial_setup(const bo_model *m, double *conc, const int64_t *numbers,
                     bo_rng *r, int8_t *cfg);

/* ---- analytics ----------------------------------------------------------- */
void bo_lattice_shells(const bo_model *m, const int8_t *cfg, int wc_range,
                       double *shells);
/* rho(i, j, l), index i + ns*(j + ns*l); counts (optional) get the raw
 * integer pair counts in the same layout. */
void bo_radial_densities(const bo_model *m, const int8_t *cfg, int wc_range,
                         const double *shells, double *rho, int64_t *counts);

/* ---- Metropolis simulated annealing (src/metropolis.F90:84-558) ---------- */
typedef struct {
    double T, delta_T;
    int T_steps;
    int64_t n_mc_steps, n_burn_in_steps;
    int64_t n_sample_steps, n_sample_steps_asro, n_sample_steps_alro;
    int64_t n_sample_steps_trajectory;
    int burn_in, burn_in_start;
    int calculate_energies, calculate_asro;
    int nbr_swap;
    int wc_range;
} bo_anneal_params;

typedef struct {
    /* per temperature (T_steps) */
    double *temperature, *energies_of_T, *C_of_T, *acceptance_of_T;
    double *rho_of_T;           /* ns*ns*wc_range*T_steps (may be NULL) */
    /* trajectory, written when n_sample_steps_trajectory divides the step;
     * capacity in rows; rows filled returned in traj_rows */
    int64_t traj_capacity;
    int64_t traj_rows;
    int64_t *traj_step;
    double *traj_energy;        /* traj_capacity */
    double *traj_asro;          /* traj_capacity * ns*ns*wc (may be NULL) */
    /* configurations at start / end of each temperature (may be NULL) */
    int8_t *initial_configs;    /* T_steps * grid */
    int8_t *final_configs;      /* T_steps * grid */
    double *shells;             /* wc_range */
} bo_anneal_out;

int bo_anneal(const bo_model *m, const bo_anneal_params *p, int8_t *cfg,
              bo_rng *r, bo_anneal_out *o);

/* ---- nested sampling (src/nested_sampling.f90:45-206) -------------------- */
typedef struct {
    int n_walkers, n_steps, n_iter;
} bo_ns_params;

/* Runs initialisation + n_iter iterations.  walkers: n_walkers*grid bytes of
 * scratch (filled); energies: n_walkers; limits: n_iter (the ener_limit
 * written at each iteration).  Returns 0. */
int bo_ns_run(const bo_model *m, const bo_ns_params *p, double *conc,
              const int64_t *numbers, bo_rng *r, int8_t *walkers,
              double *energies, double *limits, int64_t *accepted_steps);

/* One NS random walk of n_steps on one walker (inner loop of
 * src/nested_sampling.f90:157-192).  Returns accepted steps. */
int64_t bo_ns_walk(const bo_model *m, int8_t *cfg, bo_rng *r, double *energy,
                   double ener_limit, int64_t n_steps, bo_counters *c);

/* ---- Wang-Landau walker update (src/wang-landau.F90:515-632) ------------- */
int bo_wl_bin_index(double energy, const double *bin_edges, int bins);

typedef struct {
    int bins;                   /* global number of bins */
    int start_idx, end_idx;     /* 1-based window [start, end] */
    int64_t n_trials;           /* mc_sweeps * n_atoms */
    double wl_f;
    int hist_period;            /* INT(0.02*REAL(n_atoms)) */
    int nbr_swap;               /* select_sites_nbr: site 2 a random neighbour of site 1 */
} bo_wl_params;

/* One walker's sweeps() trial loop.  lng: bins entries (global indexing),
 * hist: window-local (end-start+1).  energy in/out is the walker's running
 * e_unswapped (the reference recomputes it with full_energy at entry; the
 * caller passes that value).  Returns accepted moves. */
/* The radial-density samples sweeps() takes per bin (src/wang-landau.F90:
 * 566-586): while the bin's radial_record is under cap and radial_record_bool
 * is unset, every n_atoms-th such trial adds radial_densities of the trial
 * configuration (the swap applied, before the decision) to rho_of_E. */
typedef struct {
    int wc_range;               /* 0: no sampling (rho_saved) */
    const double *shells;       /* wc_range distances */
    int cap;                    /* MAX(radial_samples / num_walkers, 1) */
    const unsigned char *done;  /* radial_record_bool, bins */
    int32_t *record;            /* radial_record, bins (this walker) */
    double *rho_of_E;           /* rho_of_E(i, j, l, bin), i fastest */
    int32_t *steps;             /* radial_mc_steps, carried between calls */
} bo_wl_radial;

int64_t bo_wl_sweep_radial(const bo_model *m, const bo_wl_params *p, int8_t *cfg,
                           bo_rng *r, const double *bin_edges, double *lng,
                           double *hist, double *energy, bo_counters *c,
                           const bo_wl_radial *rad);
/* The configuration store of sweeps() (config_per_bin / config_store,
 * src/wang-landau.F90:605-622): at a histogram tick whose bin is still
 * open, the configuration goes to that bin's slot and the bin closes. */
typedef struct {
    int8_t *slots;          /* bins x cfg_bytes, bin 1 first */
    unsigned char *open;    /* bins; 1 = open (config_store = .True.) */
    size_t cfg_bytes;
} bo_wl_store;
int64_t bo_wl_sweep_store(const bo_model *m, const bo_wl_params *p, int8_t *cfg,
                          bo_rng *r, const double *bin_edges, double *lng,
                          double *hist, double *energy, bo_counters *c,
                          const bo_wl_radial *rad, const bo_wl_store *store);
/* enter_energy_window (src/wang-landau.F90:643-741) for one walker,
 * without the MPI hand-over between walkers of a window: the biased walk
 * towards the middle of [min_e, max_e] until the energy is inside the inner
 * 80% (checked with full_energy).  sig2x2 = 2 (0.0025 |E_max - E_min| n_atoms
 * / (Ry_to_eV 1000))^2.  Every n_atoms*50*5 steps the configuration is drawn
 * again with initial_setup (conc / numbers as initial_setup takes them); the
 * running energy is not recomputed then, as in the reference.  Returns the
 * loop iterations taken, or -1 after max_steps; energy_out gets the final
 * full_energy. */
int64_t bo_wl_enter_window(const bo_model *m, int8_t *cfg, bo_rng *r, const double *conc,
                           const int64_t *numbers, double min_e, double max_e, double sig2x2,
                           int64_t max_steps, double *energy_out);
int64_t bo_wl_sweep(const bo_model *m, const bo_wl_params *p, int8_t *cfg,
                    bo_rng *r, const double *bin_edges, double *lng,
                    double *hist, double *energy, bo_counters *c);

/* ---- Wang-Landau exchange and stitching (src/wang-landau.F90) ------------ */
/* replica_exchange (:1392-1501) with shuffle_rows (:1513-1525).  Walkers are
 * ordered by window, per_window each (walker w plays MPI rank w, window
 * w/per_window + 1); win_start/win_end: 1-based bins of every window;
 * energies: full energies at the call; lng: n x bins; rngs: n streams (the
 * shuffles draw from rngs[0], rank 0's); cfgs: n x cfg_bytes, swapped on
 * acceptance.  partner[w]: walker paired with w or -1; accepted[w]: 1 when
 * w's configuration was exchanged.  Returns the accepted exchanges. */
int bo_wl_replica_exchange(int n_windows, int per_window, const int *win_start,
                           const int *win_end, const double *bin_edges, int bins,
                           const double *energies, const double *lng, bo_rng *rngs,
                           int8_t *cfgs, size_t cfg_bytes, int *partner, int *accepted);

/* dos_combine (:1147-1194): lng_windows holds each window's ln g (n_windows
 * x bins, after the in-window average); out: the stitched, min-shifted ln g.
 * Returns -1 when a window has no overlap with the previous one. */
int bo_wl_dos_combine(int n_windows, const int *win_start, const int *win_end, int bins,
                      const double *lng_windows, double *out);

/* flatness (:222): minval(hist)/(sum(hist)/n). */
double bo_wl_flatness(const double *hist, int n);

#ifdef __cplusplus
}
#endif

#endif
