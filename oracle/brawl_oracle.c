/*
 * brawl_oracle.c -- CPU restatement of BraWl's lattice-sampling hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (see
 * brawl_oracle.h).  Each function cites the reference file:line it restates
 * (paths are relative to the BraWl repository root).
 *
 * Build with -ffp-contract=off and without -ffast-math: every floating-point
 * operation below is meant to round exactly as the reference's does
 * (gfortran on x86-64 emits no FMA and never reassociates).
 */
#include "brawl_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ========================================================================= */
/* mt19937ar: src/mt19937ar.c:63-142 (Matsumoto & Nishimura's published
 * MT19937, 32-bit output, genrand = int32 * 2^-32).                          */
/* ========================================================================= */
#define MT_N 624
#define MT_M 397

void bo_rng_seed(bo_rng *r, uint32_t seed)
{
    /* src/mt19937ar.c:63-78 */
    r->mt[0] = seed;
    for (int i = 1; i < MT_N; i++) {
        uint32_t p = r->mt[i - 1];
        r->mt[i] = 1812433253u * (p ^ (p >> 30)) + (uint32_t)i;
    }
    r->mti = MT_N;
}

static void mt_twist(bo_rng *r)
{
    /* src/mt19937ar.c:90-107 */
    uint32_t *mt = r->mt;
    for (int k = 0; k < MT_N; k++) {
        uint32_t y = (mt[k] & 0x80000000u) | (mt[(k + 1) % MT_N] & 0x7fffffffu);
        mt[k] = mt[(k + MT_M) % MT_N] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    r->mti = 0;
}

uint32_t bo_rng_u32(bo_rng *r)
{
    /* src/mt19937ar.c:82-118; an unseeded generator uses seed 5489 */
    if (r->mti > MT_N) bo_rng_seed(r, 5489u);
    if (r->mti >= MT_N) mt_twist(r);
    uint32_t y = r->mt[r->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

double bo_rng_uniform(bo_rng *r)
{
    /* src/mt19937ar.c:121-125 */
    return (double)bo_rng_u32(r) * (1.0 / 4294967296.0);
}

uint32_t bo_static_seed(int rank)
{
    /* src/mt19937ar.c:137-139 */
    return (uint32_t)(110179 + 11 * rank);
}

/* ========================================================================= */
/* Neighbour lists, in the order the reference sums them.                    */
/* Offsets (dx, dy, dz) on the doubled grid, transcribed from               */
/*   src/bw_hamiltonian.f90:134-877   (bcc shells 1-10)                      */
/*   src/bw_hamiltonian.f90:1282-1691 (fcc shells 1-6)                       */
/*   src/bw_hamiltonian.f90:1930-2038 (simple cubic shells 1-2)              */
/* bcc shell 8 keeps its two (0,4,0)/(-4,0,0) entries and bcc shell 10 its   */
/* repeated entries: the reference sums them that way.                       */
/* ========================================================================= */
static const signed char sc_s1[6][3] = {{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1}};
static const signed char sc_s2[12][3] = {{0,1,-1},{-1,0,-1},{1,0,-1},{0,-1,-1},{1,1,0},{-1,1,0},
    {1,-1,0},{-1,-1,0},{0,1,1},{-1,0,1},{1,0,1},{0,-1,1}};

static const signed char bcc_s1[8][3] = {{1,1,1},{1,1,-1},{1,-1,1},{1,-1,-1},{-1,1,1},{-1,1,-1},
    {-1,-1,1},{-1,-1,-1}};
static const signed char bcc_s2[6][3] = {{2,0,0},{-2,0,0},{0,-2,0},{0,2,0},{0,0,2},{0,0,-2}};
static const signed char bcc_s3[12][3] = {{0,-2,-2},{2,0,-2},{-2,0,-2},{0,2,-2},{2,-2,0},{-2,-2,0},
    {2,2,0},{-2,2,0},{0,-2,2},{2,0,2},{-2,0,2},{0,2,2}};
static const signed char bcc_s4[24][3] = {{1,1,3},{-1,1,3},{1,-1,3},{-1,-1,3},{1,1,-3},{-1,1,-3},
    {1,-1,-3},{-1,-1,-3},{1,3,1},{-1,3,1},{1,3,-1},{-1,3,-1},{1,-3,1},{-1,-3,1},{1,-3,-1},
    {-1,-3,-1},{3,1,1},{3,-1,1},{3,1,-1},{3,-1,-1},{-3,1,1},{-3,-1,1},{-3,1,-1},{-3,-1,-1}};
static const signed char bcc_s5[8][3] = {{2,2,2},{-2,2,2},{2,-2,2},{-2,-2,2},{2,2,-2},{-2,2,-2},
    {2,-2,-2},{-2,-2,-2}};
static const signed char bcc_s6[6][3] = {{4,0,0},{-4,0,0},{0,4,0},{0,-4,0},{0,0,4},{0,0,-4}};
static const signed char bcc_s7[24][3] = {{1,3,3},{-1,3,3},{3,1,3},{-3,1,3},{3,-1,3},{-3,-1,3},
    {1,-3,3},{-1,-3,3},{3,3,1},{-3,3,1},{3,-3,1},{-3,-3,1},{3,3,-1},{-3,3,-1},{3,-3,-1},
    {-3,-3,-1},{1,3,-3},{-1,3,-3},{3,1,-3},{-3,1,-3},{3,-1,-3},{-3,-1,-3},{1,-3,-3},{-1,-3,-3}};
static const signed char bcc_s8[24][3] = {{0,2,4},{2,0,4},{-2,0,4},{0,-2,4},{0,4,2},{-4,0,2},
    {4,0,2},{0,-4,2},{2,4,0},{-2,4,0},{4,2,0},{-4,2,0},{4,-2,0},{-4,-2,0},{0,4,0},{-4,0,0},
    {0,4,-2},{-4,0,-2},{4,0,-2},{0,-4,-2},{0,2,-4},{2,0,-4},{-2,0,-4},{0,-2,-4}};
static const signed char bcc_s9[24][3] = {{2,2,4},{-2,2,4},{2,-2,4},{-2,-2,4},{2,4,2},{-2,4,2},
    {4,2,2},{-4,2,2},{4,-2,2},{-4,-2,2},{2,-4,2},{-2,-4,2},{2,4,-2},{-2,4,-2},{4,2,-2},
    {-4,2,-2},{4,-2,-2},{-4,-2,-2},{2,-4,-2},{-2,-4,-2},{2,2,-4},{-2,2,-4},{2,-2,-4},{-2,-2,-4}};
static const signed char bcc_s10[32][3] = {{1,1,5},{-1,1,5},{1,-1,5},{-1,-1,5},{3,3,3},{-3,3,3},
    {3,-3,3},{-3,-3,3},{1,-5,1},{-1,-5,1},{5,-1,1},{-5,-1,1},{5,1,1},{-5,1,1},{1,-5,1},
    {-1,-5,1},{1,-5,-1},{-1,-5,-1},{5,-1,-1},{-5,-1,-1},{5,1,-1},{-5,1,-1},{1,-5,-1},
    {-1,-5,-1},{3,3,-3},{-3,3,-3},{3,-3,-3},{-3,-3,-3},{1,1,-5},{-1,1,-5},{1,-1,-5},{-1,-1,-5}};

static const signed char fcc_s1[12][3] = {{0,-1,1},{0,-1,-1},{0,1,1},{0,1,-1},{1,-1,0},{1,1,0},
    {1,0,1},{1,0,-1},{-1,-1,0},{-1,1,0},{-1,0,1},{-1,0,-1}};
static const signed char fcc_s2[6][3] = {{2,0,0},{-2,0,0},{0,2,0},{0,-2,0},{0,0,2},{0,0,-2}};
static const signed char fcc_s3[24][3] = {{-2,1,1},{-2,1,-1},{-2,-1,1},{-2,-1,-1},{2,1,1},{2,1,-1},
    {2,-1,1},{2,-1,-1},{1,2,1},{-1,2,1},{1,2,-1},{-1,2,-1},{1,-2,1},{-1,-2,1},{1,-2,-1},
    {-1,-2,-1},{1,1,2},{-1,1,2},{1,-1,2},{-1,-1,2},{1,1,-2},{-1,1,-2},{1,-1,-2},{-1,-1,-2}};
static const signed char fcc_s4[12][3] = {{2,0,-2},{-2,0,-2},{0,2,-2},{0,-2,-2},{2,2,0},{-2,2,0},
    {2,-2,0},{-2,-2,0},{2,0,2},{-2,0,2},{0,2,2},{0,-2,2}};
static const signed char fcc_s5[24][3] = {{1,0,-3},{-1,0,-3},{0,-1,-3},{0,1,-3},{0,3,-1},{3,0,-1},
    {-3,0,-1},{0,-3,-1},{1,3,0},{-1,3,0},{3,1,0},{-3,1,0},{3,-1,0},{-3,-1,0},{1,-3,0},
    {-1,-3,0},{0,3,1},{3,0,1},{-3,0,1},{0,-3,1},{1,0,3},{-1,0,3},{0,-1,3},{0,1,3}};
static const signed char fcc_s6[8][3] = {{2,2,-2},{-2,2,-2},{2,-2,-2},{-2,-2,-2},{2,2,2},{-2,2,2},
    {2,-2,2},{-2,-2,2}};

typedef struct { int n; const signed char (*d)[3]; } shell_list;

static const shell_list SC_SHELLS[2] = {{6, sc_s1}, {12, sc_s2}};
static const shell_list BCC_SHELLS[10] = {{8, bcc_s1}, {6, bcc_s2}, {12, bcc_s3}, {24, bcc_s4},
    {8, bcc_s5}, {6, bcc_s6}, {24, bcc_s7}, {24, bcc_s8}, {24, bcc_s9}, {32, bcc_s10}};
static const shell_list FCC_SHELLS[6] = {{12, fcc_s1}, {6, fcc_s2}, {24, fcc_s3}, {12, fcc_s4},
    {24, fcc_s5}, {8, fcc_s6}};

static const shell_list *shells_of(int lattice)
{
    switch (lattice) {
    case BO_SC: return SC_SHELLS;
    case BO_BCC: return BCC_SHELLS;
    case BO_FCC: return FCC_SHELLS;
    }
    return NULL;
}

int bo_max_shells(int lattice)
{
    /* src/initialise.F90:160-241: sc 1-2, bcc 1-10, fcc 1-6 */
    switch (lattice) {
    case BO_SC: return 2;
    case BO_BCC: return 10;
    case BO_FCC: return 6;
    }
    return 0;
}

int bo_shell_size(int lattice, int shell)
{
    if (shell < 1 || shell > bo_max_shells(lattice)) return 0;
    return shells_of(lattice)[shell - 1].n;
}

int bo_shell_offset(int lattice, int shell, int k, int d[3])
{
    if (shell < 1 || shell > bo_max_shells(lattice)) return -1;
    const shell_list *s = &shells_of(lattice)[shell - 1];
    if (k < 0 || k >= s->n) return -1;
    d[0] = s->d[k][0];
    d[1] = s->d[k][1];
    d[2] = s->d[k][2];
    return 0;
}

int bo_n_atoms(const bo_model *m)
{
    /* src/initialise.F90:162,175,214 */
    int cells = m->n1 * m->n2 * m->n3;
    switch (m->lattice) {
    case BO_SC: return 8 * cells;
    case BO_BCC: return 2 * cells;
    case BO_FCC: return 4 * cells;
    }
    return 0;
}

int bo_grid_size(const bo_model *m)
{
    return 8 * m->n1 * m->n2 * m->n3;
}

static inline int fmod_pos(int a, int n)
{
    int r = a % n;
    return r < 0 ? r + n : r;
}

/* Neighbour coordinate along one axis.  fcc/bcc wrap on the doubled grid
 * (modulo(i+d, 2n)); the simple-cubic routines wrap on n, not 2n
 * (src/bw_hamiltonian.f90:1944-1949), and an axis with zero offset keeps the
 * site's own index (site_i is used directly). */
static inline int nbr_coord(int lattice, int c, int d, int n)
{
    if (d == 0) return c;
    return fmod_pos(c + d, lattice == BO_SC ? n : 2 * n);
}

static inline int cfg_index(const bo_model *m, int x, int y, int z)
{
    return x + 2 * m->n1 * (y + 2 * m->n2 * z);
}

static inline double vex(const bo_model *m, int a, int b, int shell0)
{
    /* V_ex(a, b, shell) with 1-based species a, b */
    return m->V[(a - 1) + m->ns * ((b - 1) + m->ns * shell0)];
}

double bo_site_energy(const bo_model *m, const int8_t *cfg, int x, int y, int z)
{
    /* {fcc,bcc,simple_cubic}_energy_Nshells: shell1 + shell2 + ... left to
     * right (src/bw_hamiltonian.f90:898-1262, 1712-1910, 2059-2106); each
     * shell sum starts from 0.0 and adds V_ex(species, nbr, shell) in list
     * order (e.g. src/bw_hamiltonian.f90:171-173). */
    const shell_list *sl = shells_of(m->lattice);
    int species = cfg[cfg_index(m, x, y, z)];
    double total = 0.0;
    for (int sh = 0; sh < m->nsh; sh++) {
        double e = 0.0;
        for (int k = 0; k < sl[sh].n; k++) {
            int nx = nbr_coord(m->lattice, x, sl[sh].d[k][0], m->n1);
            int ny = nbr_coord(m->lattice, y, sl[sh].d[k][1], m->n2);
            int nz = nbr_coord(m->lattice, z, sl[sh].d[k][2], m->n3);
            e = e + vex(m, species, cfg[cfg_index(m, nx, ny, nz)], sh);
        }
        total = (sh == 0) ? e : total + e;
    }
    return total;
}

double bo_pair_energy(const bo_model *m, const int8_t *cfg, const int s1[3], const int s2[3])
{
    /* src/bw_hamiltonian.f90:99-114 */
    return bo_site_energy(m, cfg, s1[0], s1[1], s1[2]) + bo_site_energy(m, cfg, s2[0], s2[1], s2[2]);
}

double bo_total_energy(const bo_model *m, const int8_t *cfg)
{
    /* src/bw_hamiltonian.f90:58-81: loop z, y, x; skip empty sites; x 0.5 */
    double energy = 0.0;
    for (int z = 0; z < 2 * m->n3; z++)
        for (int y = 0; y < 2 * m->n2; y++)
            for (int x = 0; x < 2 * m->n1; x++) {
                if (cfg[cfg_index(m, x, y, z)] == 0) continue;
                energy = energy + bo_site_energy(m, cfg, x, y, z);
            }
    return 0.5 * energy;
}

/* ========================================================================= */
/* Proposals: src/random_site.f90                                            */
/* ========================================================================= */
static inline int fmod2(int a) { return ((a % 2) + 2) % 2; }

void bo_random_site(const bo_model *m, bo_rng *r, int site[3])
{
    /* Returned 0-based as (x, y, z); the reference's site(2:4). */
    int x1, y1, z1;
    switch (m->lattice) {
    case BO_SC: /* src/random_site.f90:74-84: x, y, z */
        x1 = (int)floor(bo_rng_uniform(r) * 2.0 * (double)m->n1) + 1;
        y1 = (int)floor(bo_rng_uniform(r) * 2.0 * (double)m->n2) + 1;
        z1 = (int)floor(bo_rng_uniform(r) * 2.0 * (double)m->n3) + 1;
        break;
    case BO_BCC: /* src/random_site.f90:127-139: z, x, y */
        z1 = (int)floor(2.0 * bo_rng_uniform(r) * (double)m->n3) + 1;
        x1 = 2 * (int)floor(bo_rng_uniform(r) * (double)m->n1) + 2 - fmod2(z1);
        y1 = 2 * (int)floor(bo_rng_uniform(r) * (double)m->n2) + 2 - fmod2(z1);
        break;
    default: /* BO_FCC, src/random_site.f90:182-193: z, x, y */
        z1 = (int)floor(2.0 * bo_rng_uniform(r) * (double)m->n3) + 1;
        x1 = (int)floor(2.0 * bo_rng_uniform(r) * (double)m->n1) + 1;
        y1 = 2 * (int)floor(bo_rng_uniform(r) * (double)m->n2) + 1 + fmod2(x1 - fmod2(z1));
        break;
    }
    site[0] = x1 - 1;
    site[1] = y1 - 1;
    site[2] = z1 - 1;
}

/* Nearest-neighbour vectors used by the nbr_swap proposals, in the
 * reference's order (sc_nbrs, bcc_nbrs, fcc_nbrs, src/random_site.f90:29-61). */
static const signed char sc_nbrs[6][3] = {{0,0,1},{0,1,0},{1,0,0},{0,0,-1},{0,-1,0},{-1,0,0}};
static const signed char bcc_nbrs[8][3] = {{1,1,1},{1,1,-1},{1,-1,1},{1,-1,-1},{-1,1,1},{-1,1,-1},
    {-1,-1,1},{-1,-1,-1}};
static const signed char fcc_nbrs[12][3] = {{0,1,1},{0,1,-1},{0,-1,1},{0,-1,-1},{1,1,0},{1,-1,0},
    {1,0,1},{1,0,-1},{-1,1,0},{-1,-1,0},{-1,0,1},{-1,0,-1}};

void bo_random_nbr(const bo_model *m, bo_rng *r, const int site[3], int nbr[3])
{
    /* src/random_site.f90:97-116, 152-171, 206-225: n = floor(k*genrand())+1,
     * then wrap on the doubled grid for every lattice. */
    const signed char (*tab)[3];
    int k;
    switch (m->lattice) {
    case BO_SC:
        k = (int)floor(6.0 * bo_rng_uniform(r));
        tab = sc_nbrs;
        break;
    case BO_BCC:
        k = (int)floor(8.0 * bo_rng_uniform(r));
        tab = bcc_nbrs;
        break;
    default:
        k = (int)floor(12.0 * bo_rng_uniform(r));
        tab = fcc_nbrs;
        break;
    }
    nbr[0] = fmod_pos(site[0] + tab[k][0], 2 * m->n1);
    nbr[1] = fmod_pos(site[1] + tab[k][1], 2 * m->n2);
    nbr[2] = fmod_pos(site[2] + tab[k][2], 2 * m->n3);
}

static inline void pair_swap(const bo_model *m, int8_t *cfg, const int a[3], const int b[3])
{
    /* src/random_site.f90:238-250 */
    int ia = cfg_index(m, a[0], a[1], a[2]);
    int ib = cfg_index(m, b[0], b[1], b[2]);
    int8_t t = cfg[ia];
    cfg[ia] = cfg[ib];
    cfg[ib] = t;
}

/* ========================================================================= */
/* Metropolis step: src/metropolis.F90:751-813 (lattice), :829-891 (nbr)    */
/* ========================================================================= */
static int mc_step_de(const bo_model *m, int8_t *cfg, bo_rng *r, double beta,
                      int nbr_swap, bo_counters *c, double *de_out)
{
    int a[3], b[3];
    bo_random_site(m, r, a);
    if (nbr_swap) bo_random_nbr(m, r, a, b);
    else bo_random_site(m, r, b);
    if (c) {
        c->trials++;
        c->draws += nbr_swap ? 4 : 6;
    }
    int8_t s1 = cfg[cfg_index(m, a[0], a[1], a[2])];
    int8_t s2 = cfg[cfg_index(m, b[0], b[1], b[2])];
    if (de_out) *de_out = NAN;
    if (s1 == s2) {
        if (c) c->accepted++;
        return 1;
    }
    if (c) c->evaluated++;
    double e_unswapped = bo_pair_energy(m, cfg, a, b);
    pair_swap(m, cfg, a, b);
    double e_swapped = bo_pair_energy(m, cfg, a, b);
    double delta_e = e_swapped - e_unswapped;
    if (de_out) *de_out = delta_e;
    if (delta_e < 0.0) {
        if (c) c->accepted++;
        return 1;
    }
    if (c) {
        c->draws++;
        c->exp_tests++;
    }
    if (bo_rng_uniform(r) < exp(-beta * delta_e)) {
        if (c) c->accepted++;
        return 1;
    }
    pair_swap(m, cfg, a, b);
    return 0;
}

int bo_mc_step(const bo_model *m, int8_t *cfg, bo_rng *r, double beta,
               int nbr_swap, bo_counters *c)
{
    return mc_step_de(m, cfg, r, beta, nbr_swap, c, NULL);
}

int64_t bo_mc_run(const bo_model *m, int8_t *cfg, bo_rng *r, double beta,
                  int64_t n_trials, int nbr_swap, bo_counters *c)
{
    int64_t acc = 0;
    for (int64_t i = 0; i < n_trials; i++) acc += mc_step_de(m, cfg, r, beta, nbr_swap, c, NULL);
    return acc;
}

int64_t bo_mc_trace(const bo_model *m, int8_t *cfg, bo_rng *r, double beta,
                    int64_t n_trials, int nbr_swap, int8_t *accept_out,
                    double *de_out, bo_counters *c)
{
    int64_t acc = 0;
    for (int64_t i = 0; i < n_trials; i++) {
        int a = mc_step_de(m, cfg, r, beta, nbr_swap, c, de_out ? &de_out[i] : NULL);
        if (accept_out) accept_out[i] = (int8_t)a;
        acc += a;
    }
    return acc;
}

/* ========================================================================= */
/* initial_setup: src/initialise.F90:434-617                                 */
/* ========================================================================= */
static double seq_sum(const double *a, int lo, int hi)
{
    /* gfortran SUM(a(lo:hi)): sequential from the first element */
    double s = 0.0;
    for (int i = lo; i <= hi; i++) s = s + a[i];
    return s;
}

int bo_initial_setup(const bo_model *m, double *conc, const int64_t *numbers,
                     bo_rng *r, int8_t *cfg)
{
    const int ns = m->ns;
    const int n_atoms = bo_n_atoms(m);
    const int n_sites = n_atoms;
    int64_t count[64], check[64];
    if (ns < 1 || ns > 63) return -1;
    int64_t sum_numbers = 0;
    if (numbers)
        for (int i = 0; i < ns; i++) sum_numbers += numbers[i];
    if (numbers && sum_numbers == n_atoms) {
        /* :468-472, concentrations recomputed in single precision */
        for (int i = 0; i < ns; i++) {
            count[i] = numbers[i];
            conc[i + 1] = (double)((float)count[i] / (float)n_atoms);
        }
    } else {
        /* :480-506 */
        int64_t total = 0;
        for (int i = 0; i < ns; i++) {
            double prod = (double)(float)n_sites * conc[i + 1];
            count[i] = (int64_t)lround(prod);
            total += count[i];
        }
        int64_t round_err = total - n_sites;
        int64_t inc = (-round_err >= 0) ? 1 : -1;
        int64_t round_check = round_err;
        int guard = 0;
        while (round_check != 0) {
            for (int j = 0; j < ns; j++) {
                if (count[j] == 0) continue;
                if (round_check == 0) continue;
                count[j] += inc;
                round_check += inc;
            }
            if (++guard > 1000000) return -1;
        }
    }
    int64_t sum = 0;
    for (int i = 0; i < ns; i++) sum += count[i];
    if (sum != n_sites) return -1;

    memset(cfg, 0, (size_t)bo_grid_size(m));
    memset(check, 0, sizeof(check));
    double lo[64], hi[64];
    for (int l = 1; l <= ns; l++) {
        lo[l] = seq_sum(conc, 0, l - 1);
        hi[l] = seq_sum(conc, 0, l);
    }
    const int gx = 2 * m->n1, gy = 2 * m->n2, gz = 2 * m->n3;

#define FILL_SITE(X, Y, Z)                                                  \
    do {                                                                    \
        int idx_ = cfg_index(m, (X), (Y), (Z));                             \
        while (cfg[idx_] == 0) {                                            \
            double rnd_ = bo_rng_uniform(r);                                \
            for (int l_ = 1; l_ <= ns; l_++) {                              \
                if (rnd_ >= lo[l_] && rnd_ <= hi[l_]) {                     \
                    if (check[l_ - 1] < count[l_ - 1]) {                    \
                        cfg[idx_] = (int8_t)l_;                             \
                        check[l_ - 1]++;                                    \
                    }                                                       \
                }                                                           \
            }                                                               \
        }                                                                   \
    } while (0)

    if (m->lattice == BO_SC) {
        /* :525-544 */
        for (int k = 0; k < gz; k++)
            for (int j = 0; j < gy; j++)
                for (int i = 0; i < gx; i++) FILL_SITE(i, j, k);
    } else if (m->lattice == BO_BCC) {
        /* :546-573: z odd (1-based) -> odd x, y; z even -> even x, y */
        for (int k1 = 1; k1 <= gz; k1++)
            for (int j1 = 1; j1 <= gy / 2; j1++)
                for (int i1 = 1; i1 <= gx / 2; i1++) {
                    int x1 = (k1 % 2 == 1) ? 2 * i1 - 1 : 2 * i1;
                    int y1 = (k1 % 2 == 1) ? 2 * j1 - 1 : 2 * j1;
                    FILL_SITE(x1 - 1, y1 - 1, k1 - 1);
                }
    } else {
        /* :575-610 */
        for (int k1 = 1; k1 <= gz; k1++)
            for (int j1 = 1; j1 <= gy; j1++)
                for (int i1 = 1; i1 <= gx / 2; i1++) {
                    int x1 = 2 * i1 - (k1 % 2) * (j1 % 2) - ((k1 + 1) % 2) * ((j1 + 1) % 2);
                    FILL_SITE(x1 - 1, j1 - 1, k1 - 1);
                }
    }
#undef FILL_SITE
    return 0;
}

/* ========================================================================= */
/* Analytics: src/analytics.f90:205-404                                      */
/* ========================================================================= */
static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

void bo_lattice_shells(const bo_model *m, const int8_t *cfg, int wc_range, double *shells)
{
    /* src/analytics.f90:205-275: single-precision distances of occupied
     * sites from the origin, sorted, de-duplicated at 1e-3; the array has
     * 8 n1 n2 n3 + 1 slots and the unfilled slots stay 0. */
    int total = bo_grid_size(m) + 1;
    double *all = (double *)calloc((size_t)total, sizeof(double));
    int l = 0;
    for (int k = 0; k < 2 * m->n3; k++)
        for (int j = 0; j < 2 * m->n2; j++)
            for (int i = 0; i < 2 * m->n1; i++) {
                if (cfg[cfg_index(m, i, j, k)] == 0) continue;
                float d2 = (float)(k * k) + (float)(j * j) + (float)(i * i);
                all[l++] = (double)sqrtf(d2);
            }
    qsort(all, (size_t)total, sizeof(double), cmp_double);
    for (int i = 0; i < wc_range; i++) shells[i] = 0.0;
    int out = 0;
    for (int i = 0; i < total - 1; i++) {
        if (fabs(all[i] - all[i + 1]) < 1e-3) continue;
        shells[out++] = all[i];
        if (out >= wc_range) break;
    }
    free(all);
}

void bo_radial_densities(const bo_model *m, const int8_t *cfg, int wc_range,
                         const double *shells, double *rho, int64_t *counts_out)
{
    /* src/analytics.f90:293-404 */
    const int ns = m->ns;
    const int gx = 2 * m->n1, gy = 2 * m->n2, gz = 2 * m->n3;
    int64_t pc[64] = {0};
    size_t nrho = (size_t)ns * ns * wc_range;
    int64_t *cnt = (int64_t *)calloc(nrho, sizeof(int64_t));
    for (int z = 0; z < gz; z++)
        for (int y = 0; y < gy; y++)
            for (int x = 0; x < gx; x++) {
                int s = cfg[cfg_index(m, x, y, z)];
                if (s >= 1 && s <= ns) pc[s - 1]++;
            }
    int l1 = m->n1 < 5 ? m->n1 : 5;
    int l2 = m->n2 < 5 ? m->n2 : 5;
    int l3 = m->n3 < 5 ? m->n3 : 5;
    for (int i3 = 0; i3 < gz; i3++)
        for (int i2 = 0; i2 < gy; i2++)
            for (int i1 = 0; i1 < gx; i1++) {
                int si = cfg[cfg_index(m, i1, i2, i3)];
                if (si == 0) continue;
                for (int jj3 = i3 - l3; jj3 <= i3 + l3; jj3++) {
                    int j3 = fmod_pos(jj3, gz);
                    for (int jj2 = i2 - l2; jj2 <= i2 + l2; jj2++) {
                        int j2 = fmod_pos(jj2, gy);
                        for (int jj1 = i1 - l1; jj1 <= i1 + l1; jj1++) {
                            int j1 = fmod_pos(jj1, gx);
                            int sj = cfg[cfg_index(m, j1, j2, j3)];
                            if (sj == 0) continue;
                            /* minimum image with nint(d / float(2n)) */
                            double dx = (double)(float)(i1 - j1);
                            double dy = (double)(float)(i2 - j2);
                            double dz = (double)(float)(i3 - j3);
                            dx = dx - (double)((float)gx * (float)lround(dx / (double)(float)gx));
                            dy = dy - (double)((float)gy * (float)lround(dy / (double)(float)gy));
                            dz = dz - (double)((float)gz * (float)lround(dz / (double)(float)gz));
                            double dist = sqrt(dx * dx + dy * dy + dz * dz);
                            for (int l = 0; l < wc_range; l++)
                                if (fabs(dist - shells[l]) < 1e-3)
                                    cnt[(si - 1) + ns * ((sj - 1) + ns * l)]++;
                        }
                    }
                }
            }
    for (int l = 0; l < wc_range; l++)
        for (int j = 0; j < ns; j++)
            for (int i = 0; i < ns; i++) {
                size_t idx = (size_t)i + ns * ((size_t)j + ns * l);
                rho[idx] = (double)cnt[idx] / (double)pc[i];
            }
    if (counts_out) memcpy(counts_out, cnt, nrho * sizeof(int64_t));
    free(cnt);
}

/* ========================================================================= */
/* Simulated annealing driver: src/metropolis.F90:84-558                     */
/* k_b_in_Ry = 8.167333262e-5/13.605693122990 (src/constants.f90:41-46)     */
/* ========================================================================= */
static const double K_B_IN_RY = 8.167333262e-5 / 13.605693122990;

int bo_anneal(const bo_model *m, const bo_anneal_params *p, int8_t *cfg,
              bo_rng *r, bo_anneal_out *o)
{
    const int ns = m->ns, wc = p->wc_range;
    const size_t nrho = (size_t)ns * ns * wc;
    const size_t grid = (size_t)bo_grid_size(m);
    double *r_dens = (double *)calloc(nrho ? nrho : 1, sizeof(double));
    double *asro = (double *)calloc(nrho ? nrho : 1, sizeof(double));
    /* n_save_* = floor(real(n_mc_steps)/real(n_sample_steps_*)) in single
     * precision (src/metropolis.F90:156-166) */
    int64_t n_save_energy = (int64_t)floorf((float)p->n_mc_steps / (float)p->n_sample_steps);
    int64_t n_save_asro = (int64_t)floorf((float)p->n_mc_steps / (float)p->n_sample_steps_asro);
    bo_lattice_shells(m, cfg, wc, o->shells);
    o->traj_rows = 0;
    for (int j = 0; j < p->T_steps; j++) {
        memset(r_dens, 0, nrho * sizeof(double));
        double step_E = 0.0, step_Esq = 0.0, acceptance = 0.0;
        double temp = p->T + (double)j * p->delta_T;
        double sim_temp = temp * K_B_IN_RY;
        double beta = 1.0 / sim_temp;
        o->temperature[j] = temp;
        int do_burn = (j == 0) ? p->burn_in_start : p->burn_in;
        if (do_burn)
            for (int64_t i = 0; i < p->n_burn_in_steps; i++)
                acceptance += bo_mc_step(m, cfg, r, beta, p->nbr_swap, NULL);
        double current_energy = 0.0;
        if (p->calculate_energies) current_energy = bo_total_energy(m, cfg);
        if (p->calculate_asro) bo_radial_densities(m, cfg, wc, o->shells, asro, NULL);
        if (o->traj_rows < o->traj_capacity) {
            int64_t row = o->traj_rows++;
            o->traj_step[row] = 0;
            o->traj_energy[row] = current_energy;
            if (o->traj_asro) memcpy(o->traj_asro + row * nrho, asro, nrho * sizeof(double));
        }
        if (o->initial_configs) memcpy(o->initial_configs + (size_t)j * grid, cfg, grid);
        int64_t n_sweeps = p->n_mc_steps / p->n_sample_steps;
        int64_t n_sweep_steps = p->n_mc_steps / n_sweeps;
        acceptance = 0.0;
        for (int64_t i = 1; i <= n_sweeps; i++) {
            for (int64_t k = 0; k < n_sweep_steps; k++)
                acceptance = acceptance + (double)bo_mc_step(m, cfg, r, beta, p->nbr_swap, NULL);
            int64_t step_n = i * n_sweep_steps;
            if (p->calculate_energies) {
                current_energy = bo_total_energy(m, cfg);
                step_E = step_E + current_energy;
                step_Esq = step_Esq + current_energy * current_energy;
            }
            if (p->calculate_asro) {
                if (step_n % p->n_sample_steps_asro == 0) {
                    bo_radial_densities(m, cfg, wc, o->shells, asro, NULL);
                    for (size_t q = 0; q < nrho; q++) r_dens[q] = r_dens[q] + asro[q];
                }
            }
            if (step_n % p->n_sample_steps_trajectory == 0 && o->traj_rows < o->traj_capacity) {
                int64_t row = o->traj_rows++;
                o->traj_step[row] = step_n;
                o->traj_energy[row] = current_energy;
                if (o->traj_asro) memcpy(o->traj_asro + row * nrho, asro, nrho * sizeof(double));
            }
        }
        o->acceptance_of_T[j] = acceptance / (double)(float)p->n_mc_steps;
        if (p->calculate_energies) {
            double ne = (double)n_save_energy;
            o->energies_of_T[j] = step_E / ne / (double)bo_n_atoms(m);
            double mean = step_E / ne;
            double C = (step_Esq / ne - mean * mean) / (sim_temp * temp) / (double)bo_n_atoms(m);
            if (C < 0.0) C = 0.0;
            if (temp <= 0.0) C = 0.0;
            o->C_of_T[j] = C;
        }
        if (p->calculate_asro && o->rho_of_T)
            for (size_t q = 0; q < nrho; q++)
                o->rho_of_T[(size_t)j * nrho + q] = r_dens[q] / (double)n_save_asro;
        if (o->final_configs) memcpy(o->final_configs + (size_t)j * grid, cfg, grid);
    }
    free(r_dens);
    free(asro);
    return 0;
}

/* ========================================================================= */
/* Nested sampling: src/nested_sampling.f90:45-206                           */
/* ========================================================================= */
int64_t bo_ns_walk(const bo_model *m, int8_t *cfg, bo_rng *r, double *energy,
                   double ener_limit, int64_t n_steps, bo_counters *c)
{
    /* src/nested_sampling.f90:157-192 */
    int64_t n_acc = 0;
    for (int64_t i = 0; i < n_steps; i++) {
        int a[3], b[3];
        bo_random_site(m, r, a);
        int8_t s1 = cfg[cfg_index(m, a[0], a[1], a[2])];
        int8_t s2;
        if (c) { c->trials++; c->draws += 3; }
        do {
            bo_random_site(m, r, b);
            if (c) c->draws += 3;
            s2 = cfg[cfg_index(m, b[0], b[1], b[2])];
        } while (s1 == s2);
        if (c) c->evaluated++;
        double e_unswapped = bo_pair_energy(m, cfg, a, b);
        pair_swap(m, cfg, a, b);
        double e_swapped = bo_pair_energy(m, cfg, a, b);
        double delta_e = e_swapped - e_unswapped;
        if (*energy + delta_e < ener_limit) {
            *energy = *energy + delta_e;
            n_acc++;
            if (c) c->accepted++;
        } else {
            pair_swap(m, cfg, a, b);
        }
    }
    return n_acc;
}

int bo_ns_run(const bo_model *m, const bo_ns_params *p, double *conc,
              const int64_t *numbers, bo_rng *r, int8_t *walkers,
              double *energies, double *limits, int64_t *accepted_steps)
{
    const size_t grid = (size_t)bo_grid_size(m);
    const int K = p->n_walkers;
    /* n_at = n_1*n_2*n_3*n_basis*n_species (src/nested_sampling.f90:82) */
    const int n_at = m->n1 * m->n2 * m->n3 * 1 * m->ns;
    for (int w = 0; w < K; w++) {
        /* :88-96; the 1e-8 literal is single precision */
        if (bo_initial_setup(m, conc, numbers, r, walkers + (size_t)w * grid) != 0) return -1;
        double rnde = bo_rng_uniform(r);
        energies[w] = bo_total_energy(m, walkers + (size_t)w * grid) + rnde * (double)1e-8f;
    }
    int extra_steps = 0;
    int64_t n_acc = 0, total_acc = 0;
    int half = (int)((float)K / 2.0f);
    for (int it = 1; it <= p->n_iter; it++) {
        /* maxloc: first index of the maximum */
        int imax = 0;
        for (int w = 1; w < K; w++)
            if (energies[w] > energies[imax]) imax = w;
        double ener_limit = energies[imax];
        limits[it - 1] = ener_limit;
        if (half > 0 && it % half == 0) {
            /* :129-144 */
            if (((float)n_acc < (float)n_at * 0.05f) && (extra_steps < p->n_steps * 100))
                extra_steps = extra_steps + p->n_steps;
        }
        /* :149-152; ceiling(rnd*K) is 0 only when rnd == 0, where the
         * reference indexes out of bounds: clamp to the first walker */
        double rnd = bo_rng_uniform(r);
        int irnd = (int)ceil(rnd * (double)K);
        if (irnd < 1) irnd = 1;
        memcpy(walkers + (size_t)imax * grid, walkers + (size_t)(irnd - 1) * grid, grid);
        energies[imax] = energies[irnd - 1];
        n_acc = bo_ns_walk(m, walkers + (size_t)imax * grid, r, &energies[imax], ener_limit,
                           (int64_t)p->n_steps + extra_steps, NULL);
        total_acc += n_acc;
    }
    if (accepted_steps) *accepted_steps = total_acc;
    return 0;
}

/* ========================================================================= */
/* Wang-Landau walker update: src/wang-landau.F90:515-632                    */
/* ========================================================================= */
int bo_wl_bin_index(double energy, const double *bin_edges, int bins)
{
    /* src/wang-landau.F90:515-523: int() truncates toward zero */
    double bin_range = bin_edges[bins] - bin_edges[0];
    double t = ((energy - bin_edges[0]) / bin_range) * (double)bins;
    return (int)t + 1;
}

int64_t bo_wl_sweep(const bo_model *m, const bo_wl_params *p, int8_t *cfg,
                    bo_rng *r, const double *bin_edges, double *lng,
                    double *hist, double *energy, bo_counters *c)
{
    return bo_wl_sweep_radial(m, p, cfg, r, bin_edges, lng, hist, energy, c, NULL);
}

int64_t bo_wl_sweep_radial(const bo_model *m, const bo_wl_params *p, int8_t *cfg,
                           bo_rng *r, const double *bin_edges, double *lng,
                           double *hist, double *energy, bo_counters *c,
                           const bo_wl_radial *rad)
{
    return bo_wl_sweep_store(m, p, cfg, r, bin_edges, lng, hist, energy, c, rad, NULL);
}

int64_t bo_wl_sweep_store(const bo_model *m, const bo_wl_params *p, int8_t *cfg,
                          bo_rng *r, const double *bin_edges, double *lng,
                          double *hist, double *energy, bo_counters *c,
                          const bo_wl_radial *rad, const bo_wl_store *store)
{
    const int n_atoms = bo_n_atoms(m);
    const int per_bin = rad ? m->ns * m->ns * rad->wc_range : 0;
    double rho_buf[15 * 15 * 64];
    int64_t accepted = 0;
    double e_unswapped = *energy;
    for (int64_t i = 1; i <= p->n_trials; i++) {
        int a[3], b[3];
        /* mc_select: select_sites or select_sites_nbr (src/wang-landau.F90:1527-1539) */
        bo_random_site(m, r, a);
        if (p->nbr_swap) bo_random_nbr(m, r, a, b);
        else bo_random_site(m, r, b);
        if (c) { c->trials++; c->draws += p->nbr_swap ? 4 : 6; }
        int8_t s1 = cfg[cfg_index(m, a[0], a[1], a[2])];
        int8_t s2 = cfg[cfg_index(m, b[0], b[1], b[2])];
        double e_swapped = e_unswapped;
        double pair_unswapped = bo_pair_energy(m, cfg, a, b);
        pair_swap(m, cfg, a, b);
        if (s1 != s2) {
            double pair_swapped = bo_pair_energy(m, cfg, a, b);
            e_swapped = e_unswapped - pair_unswapped + pair_swapped;
            if (c) c->evaluated++;
        }
        int ibin = bo_wl_bin_index(e_unswapped, bin_edges, p->bins);
        int jbin = bo_wl_bin_index(e_swapped, bin_edges, p->bins);
        int hist_tick = (p->hist_period > 0) && (i % p->hist_period == 0);
        if (rad && rad->wc_range > 0 && jbin < p->bins + 1 && jbin > 0 &&
            rad->record[jbin - 1] < rad->cap && !rad->done[jbin - 1]) {
            *rad->steps += 1;
            if (*rad->steps >= n_atoms) {
                *rad->steps = 0;
                rad->record[jbin - 1] += 1;
                bo_radial_densities(m, cfg, rad->wc_range, rad->shells, rho_buf, NULL);
                double *dst = rad->rho_of_E + (size_t)(jbin - 1) * per_bin;
                for (int k = 0; k < per_bin; k++) dst[k] = dst[k] + rho_buf[k];
            }
        }
        if (jbin > p->start_idx - 1 && jbin < p->end_idx + 1) {
            if (c) { c->draws++; c->exp_tests++; }
            if (log(bo_rng_uniform(r)) < (lng[ibin - 1] - lng[jbin - 1])) {
                accepted++;
                e_unswapped = e_swapped;
            } else {
                pair_swap(m, cfg, a, b);
                jbin = ibin;
            }
        } else {
            jbin = ibin;
            pair_swap(m, cfg, a, b);
        }
        if (hist_tick) {
            hist[jbin - p->start_idx] = hist[jbin - p->start_idx] + 1.0;
            if (store && store->open[jbin - 1]) {
                store->open[jbin - 1] = 0;
                memcpy(store->slots + (size_t)(jbin - 1) * store->cfg_bytes, cfg, store->cfg_bytes);
            }
        }
        lng[jbin - 1] = lng[jbin - 1] + p->wl_f;
    }
    if (c) c->accepted += accepted;
    *energy = e_unswapped;
    return accepted;
}

/* shuffle_rows (src/wang-landau.F90:1513-1525): rows i = n..2, partner
 * MIN(1+int(genrand()*i), n), on the stream it is given. */
static void wl_shuffle_rows(int rows[][2], int n, bo_rng *r)
{
    for (int i = n; i >= 2; i--) {
        int k = 1 + (int)(bo_rng_uniform(r) * (double)i);
        if (k > n) k = n;
        int t0 = rows[i - 1][0], t1 = rows[i - 1][1];
        rows[i - 1][0] = rows[k - 1][0];
        rows[i - 1][1] = rows[k - 1][1];
        rows[k - 1][0] = t0;
        rows[k - 1][1] = t1;
    }
}

int bo_wl_replica_exchange(int n_windows, int per_window, const int *win_start,
                           const int *win_end, const double *bin_edges, int bins,
                           const double *energies, const double *lng, bo_rng *rngs,
                           int8_t *cfgs, size_t cfg_bytes, int *partner, int *accepted)
{
    /* src/wang-landau.F90:1403-1435: every walker's bin and the overlap it
     * lies in (the lower window's index, 0 for none); the walker index plays
     * the MPI rank (rank r is walker r, window r/per_window + 1). */
    const int n = n_windows * per_window;
    int *ibin = (int *)malloc(sizeof(int) * (size_t)n);
    int (*ov)[2] = malloc(sizeof(int[2]) * (size_t)n);
    int (*lo)[2] = malloc(sizeof(int[2]) * (size_t)per_window);
    int (*up)[2] = malloc(sizeof(int[2]) * (size_t)per_window);
    int (*pairs)[2] = malloc(sizeof(int[2]) * (size_t)per_window);
    int8_t *tmp = (int8_t *)malloc(cfg_bytes);
    int n_acc = 0;
    for (int w = 0; w < n; w++) {
        int idx = w / per_window + 1;
        int ib = bo_wl_bin_index(energies[w], bin_edges, bins);
        int lower = 0, upper = 0;
        if (idx > 1)
            lower = ib < win_end[idx - 2] + 1 && ib > win_start[idx - 1] - 1;
        if (idx < n_windows)
            upper = ib > win_start[idx] - 1 && ib < win_end[idx - 1] + 1;
        ibin[w] = ib;
        ov[w][0] = w;
        ov[w][1] = upper ? idx : (lower ? idx - 1 : 0);
        partner[w] = -1;
        accepted[w] = 0;
    }
    /* :1437-1494: per adjacent pair of windows, shuffle both lists on the
     * first walker's stream, match equal overlaps, then every matched lower
     * walker draws against its own ln g and the pair swap configurations */
    for (int i = 1; i <= n_windows - 1; i++) {
        memcpy(lo, ov + (size_t)(i - 1) * per_window, sizeof(int[2]) * (size_t)per_window);
        memcpy(up, ov + (size_t)i * per_window, sizeof(int[2]) * (size_t)per_window);
        wl_shuffle_rows(lo, per_window, &rngs[0]);
        wl_shuffle_rows(up, per_window, &rngs[0]);
        int np = 0;
        for (int j = 0; j < per_window; j++) {
            if (lo[j][1] == 0) continue;
            for (int k = 0; k < per_window; k++) {
                if (up[k][1] == 0) continue;
                if (lo[j][1] == up[k][1]) {
                    pairs[np][0] = lo[j][0];
                    pairs[np][1] = up[k][0];
                    np++;
                    lo[j][0] = lo[j][1] = 0;
                    up[k][0] = up[k][1] = 0;
                }
            }
        }
        for (int p = 0; p < np; p++) {
            int a = pairs[p][0], b = pairs[p][1];
            int jb = bo_wl_bin_index(energies[b], bin_edges, bins);
            const double *la = lng + (size_t)a * bins;
            partner[a] = b;
            partner[b] = a;
            if (bo_rng_uniform(&rngs[a]) < exp(la[ibin[a] - 1] - la[jb - 1])) {
                int8_t *ca = cfgs + (size_t)a * cfg_bytes, *cb = cfgs + (size_t)b * cfg_bytes;
                memcpy(tmp, ca, cfg_bytes);
                memcpy(ca, cb, cfg_bytes);
                memcpy(cb, tmp, cfg_bytes);
                accepted[a] = accepted[b] = 1;
                n_acc++;
            }
        }
    }
    free(ibin); free(ov); free(lo); free(up); free(pairs); free(tmp);
    return n_acc;
}

int bo_wl_dos_combine(int n_windows, const int *win_start, const int *win_end, int bins,
                      const double *lng_windows, double *out)
{
    /* src/wang-landau.F90:1147-1194: start from window 1's ln g; for every
     * next window find, in the overlap, the bin where the two slopes differ
     * least (first such bin), shift the window's ln g to meet the combined
     * one there and overwrite from that bin to the window's end; then
     * subtract the minimum.  beta_index carries over between windows as in
     * the reference (it is initialised once). */
    memcpy(out, lng_windows, sizeof(double) * (size_t)bins);
    int beta_index = 0;
    for (int i = 2; i <= n_windows; i++) {
        const double *buf = lng_windows + (size_t)(i - 1) * bins;
        const int s = win_start[i - 1], e = win_end[i - 1];
        double beta_diff = DBL_MAX;
        for (int j = 0; j <= win_end[i - 2] - win_start[i - 1] - 1; j++) {
            double bo = out[s + j] - out[s + j - 1];
            double bm = buf[s + j] - buf[s + j - 1];
            if (fabs(bo - bm) < beta_diff) {
                beta_diff = fabs(bo - bm);
                beta_index = s + j + 1;
            }
        }
        if (beta_index < 1) return -1;     /* no overlap: the reference indexes bin 0 */
        for (int j = beta_index; j <= e; j++)
            out[j - 1] = buf[j - 1] + out[beta_index - 1] - buf[beta_index - 1];
    }
    double mn = 0.0;
    int have = 0;
    for (int b = 0; b < bins; b++)
        if (out[b] == out[b] && (!have || out[b] < mn)) { mn = out[b]; have = 1; }
    for (int b = 0; b < bins; b++) out[b] = out[b] - mn;
    return 0;
}

double bo_wl_flatness(const double *hist, int n)
{
    /* src/wang-landau.F90:222: minval(hist)/(sum(hist)/mpi_bins) */
    double mn = hist[0], s = 0.0;
    for (int b = 0; b < n; b++) {
        if (hist[b] < mn) mn = hist[b];
        s = s + hist[b];
    }
    return mn / (s / (double)n);
}

/* enter_energy_window (src/wang-landau.F90:643-741), one walker. */
int64_t bo_wl_enter_window(const bo_model *m, int8_t *cfg, bo_rng *r, const double *conc,
                           const int64_t *numbers, double min_e, double max_e, double sig2x2,
                           int64_t max_steps, double *energy_out)
{
    const double target = (min_e + max_e) / 2.0;
    const double condition = fabs(max_e - min_e) * 0.1;
    const int64_t reinit = (int64_t)bo_n_atoms(m) * 50 * 5;
    double conc_buf[16];
    double e_un = bo_total_energy(m, cfg);
    int64_t i_steps = 0;
    for (int64_t it = 1; it <= max_steps; it++) {
        i_steps++;
        if (i_steps % reinit == 0) {
            i_steps = 0;
            for (int k = 0; k <= m->ns; k++) conc_buf[k] = conc[k];
            if (bo_initial_setup(m, conc_buf, numbers, r, cfg) != 0) return -1;
        }
        if (e_un < max_e - condition && e_un > min_e + condition) {
            e_un = bo_total_energy(m, cfg);
            if (e_un < max_e - condition && e_un > min_e + condition) {
                *energy_out = e_un;
                return it;
            }
            continue;
        }
        int a[3], b[3];
        bo_random_site(m, r, a);
        bo_random_site(m, r, b);
        const int8_t s1 = cfg[cfg_index(m, a[0], a[1], a[2])];
        const int8_t s2 = cfg[cfg_index(m, b[0], b[1], b[2])];
        if (s1 != s2) {
            const double p_un = bo_pair_energy(m, cfg, a, b);
            pair_swap(m, cfg, a, b);
            const double p_sw = bo_pair_energy(m, cfg, a, b);
            const double e_sw = e_un - p_un + p_sw;
            const double delta_e = ((e_sw - target) * (e_sw - target) -
                                    (e_un - target) * (e_un - target)) / sig2x2;
            if (log(bo_rng_uniform(r)) < -delta_e) e_un = e_sw;
            else pair_swap(m, cfg, a, b);
        }
    }
    *energy_out = e_un;
    return -1;
}
