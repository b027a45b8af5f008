/*
 * pimc_oracle.h -- CPU oracle for the PIMC Monte Carlo sweep.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * package's (oameye/PIMC.jl) sweep: action pieces, Levy staging, the
 * permutation swap, the centre-of-mass moves, the estimators and the run!
 * driver.  It is the checker for the CUDA engine and the timed CPU baseline.
 * Nothing in the product links it; the product fails loudly without its
 * CUDA library.
 *
 * Parity status: the reference is Julia and no Julia toolchain exists on the
 * build or GPU machines, so the reference cannot be run.  The restatement is
 * pinned against the reference's own known answers (exact N=1 energy
 * constant, the Z_N recursion energies, density normalisation and the
 * beads-in-box test); draw-for-draw identity with Julia's RNG is
 * "parity unpinned" and injected draws are used on both sides instead.
 *
 * Conventions: slices are 0-based here (reference slice j = our j+1);
 * positions are SoA x[d*N*M + n*M + j]; cached link actions V[n*M + j] hold
 * lnV(bead j, next bead) exactly like Particle.V (src/system.jl:1-6).
 */
#ifndef PIMC_ORACLE_H
#define PIMC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_SEM_REFERENCE = 0, ORC_SEM_PHYSICAL = 1 };

/* move outcome codes */
enum {
  ORC_REJECT = 0,
  ORC_ACCEPT = 1,
  ORC_SKIP = 2,      /* attempt returned before proposing (n1==n2, no singles, N<=1) */
  ORC_HARDCORE = 3,  /* hard-core retry cap reached: counts as a reject */
  ORC_EDRAWS = -1,   /* injected draw arrays ran out */
  ORC_EARG = -2,
  ORC_ESTATE = -3    /* init_world could not place the hard spheres */
};

typedef struct orc_params {
  int dim, N, M;
  double L;        /* half-width: box is [-L, L)^dim */
  double beta, tau, lambda, mu;
  /* external potential: hcoef*(x^2+y^2) + V0*(sin^2(lat_k x)+sin^2(lat_k y)) */
  double hcoef, V0, lat_k;
  /* pair: lnU(r1,r2) = -tau/2 (v(|r1|)+v(|r2|)), v(r) = g exp(-r^2 inv2s2) */
  int interactions;
  double g, inv2s2;
  int nbins;       /* neighbour grid cells per dimension, floor(2L/r_a) */
  double rc;       /* neighbour radius 2L/nbins */
  double hardcore_a;
  int ctr;         /* hard-core retry cap (s.ctr) */
  int semantics;   /* ORC_SEM_REFERENCE or ORC_SEM_PHYSICAL */
  /* tabulated contact propagator (build_prop_int, src/propagator.jl:74-89):
   * when ct_tab is set and interactions is on, lnU comes from the table
   * T[i1*ct_n + i2] on r_i = 1e-20 + i (ct_range - 1e-20)/(ct_n - 1) */
  const double *ct_tab;
  int ct_n;
  double ct_range;
  /* optical lattice (examples/tools/potentialtools.jl:1-39): V += beam_depth
   * * normalized_intensity(r, beam_angle[0..nbeam), beam_scale; helical) */
  int nbeam, beam_helical;
  double beam_depth, beam_scale;
  double beam_angle[16];
} orc_params;

typedef struct orc_rng {
  uint32_t key[2];
  uint32_t ctr[4];
  uint32_t buf[4];
  int pos;
  int have_spare;
  double spare;
} orc_rng;

typedef struct orc_draws {
  const double *normals; long n_normals; long normal_pos;
  const double *uniforms; long n_uniforms; long uniform_pos;
  orc_rng *rng;    /* when non-NULL, draws come from the generator */
  int exhausted;
} orc_draws;

typedef struct orc_state {
  orc_params p;
  double *x;       /* [dim][N][M] */
  double *V;       /* [N][M] */
  int *next;       /* [N] */
  /* per-slice cell lists (doubly linked) */
  int ncell;       /* nbins^dim */
  int *cell_head;  /* [M][ncell] */
  int *cell_nxt;   /* [M][N] */
  int *cell_prv;   /* [M][N] */
  int *bins;       /* [N][M] */
  /* scratch */
  double *scratch;
  long scratch_len;
} orc_state;

/* ---- parameters / state ---- */
void orc_params_init(orc_params *p, int dim, int N, int M, double L, double T,
                     double lambda);
orc_state *orc_create(const orc_params *p);
void orc_destroy(orc_state *st);
/* copy positions in and recompute V (lnV(bead, next bead) using next) and cells */
int orc_set_state(orc_state *st, const double *x, const int *next);
/* set positions and cached link actions verbatim (V may be stale on purpose) */
int orc_set_raw(orc_state *st, const double *x, const double *V, const int *next);
void orc_get_state(const orc_state *st, double *x, double *V, int *next);
/* init_world (src/system.jl:36-78): uniform start + Levy loop per particle */
int orc_init_world(orc_state *st, orc_draws *dr);

/* ---- action pieces (src/propagator.jl) ---- */
double orc_distance(double x1, double x2, double L);
double orc_teleport(double x, double L);
double orc_lnK(const orc_params *p, const double *r1, const double *r2, double tau_eff);
double orc_Vext(const orc_params *p, const double *r);
double orc_lnV(const orc_params *p, const double *r1, const double *r2);
double orc_lnU(const orc_params *p, const double *d1, const double *d2);

/* total action pieces on the current configuration:
 * out[0] = sum lnK over all links, out[1] = sum lnV (recomputed), out[2] =
 * pair sum (link formulation, each unordered pair once), out[3] = sum of the
 * cached V */
void orc_eval_action(const orc_state *st, double out[4]);
/* the staging move's w_initial / w_updated for a given proposed window
 * rp[(m+1)*dim] (bead-major), without drawing (src/updates/reshape.jl:66-77) */
void orc_staging_weights(orc_state *st, int n, int j0, int m, const double *rp,
                         double *w_init, double *w_upd);

/* ---- moves (src/updates/reshape.jl, src/updates/com.jl) ---- */
int orc_staging(orc_state *st, int n, int j0, int m, orc_draws *dr, double *rp_out);
int orc_swap(orc_state *st, int j0, int m, int n1, double u_pick, orc_draws *dr,
             int *n2_out, double *rp_out);
int orc_com(orc_state *st, int n, double maxd, orc_draws *dr);
int orc_polymer_com(orc_state *st, int n, double maxd, orc_draws *dr);

/* ---- estimators (src/measurement.jl) ---- */
/* out[0] = E_th, out[1] = E_v (reference formulas), out[2] = pair energy term,
 * out[3] = pair virial term (both zero without interactions) */
void orc_energy(const orc_state *st, double out[4]);
/* Density: hist[nb*nb] (dim 2, column-major like dens[ix,iy]) += counts */
void orc_density(const orc_state *st, int nb, double *hist);
/* superfluid estimators (the TODO of src/measurement.jl:126): out[0] = W^2,
 * |sum over links of the signed minimum-image displacement|^2; out[1] = A_z =
 * 1/2 sum over links (x dy - y dx); out[2] = sum r^2 / M */
void orc_superfluid(const orc_state *st, double out[3]);
/* radial distribution (the TODO of src/measurement.jl:125): adds, for every
 * slice, every unordered pair with minimum-image distance r to bin
 * floor(r / dr) when that is below nb */
void orc_radial(const orc_state *st, int nb, double dr, double *hist);

/* ---- generator ---- */
void orc_rng_init(orc_rng *r, uint64_t seed, uint64_t stream);
double orc_rng_uniform(orc_rng *r);   /* [0,1) 53 bit */
double orc_rng_normal(orc_rng *r);    /* Box-Muller, FP64 */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ---- run! driver (src/simulation.jl:29-42) ---- */
typedef struct orc_update {
  int kind;        /* 0 staging, 1 swap, 2 single CoM, 3 polymer CoM */
  int every;
  /* NumbOfSlices / Step */
  double var;      /* m (slices) or step size */
  double minvar, maxvar, minacc, maxacc;
  int adj, range;
  /* counter_var queue state */
  unsigned char *queue; int qlen, qhead; long qsum; long tries;
  long attempts, accepts;
} orc_update;

typedef struct orc_run_stats {
  long attempts[4], accepts[4];
  double bead_updates;
  long measurements;
} orc_run_stats;

/* n attempts; energy series appended to e_out (cap e_cap) every ncycle
 * attempts (ncycle<=0: no measurement); density accumulated when hist != NULL */
int orc_run(orc_state *st, long n, orc_update *ups, int nups, orc_rng *rng,
            int ncycle, double *e_out, long e_cap, long *e_count,
            int dens_nb, double *hist, long *ndata, orc_run_stats *stats);

void orc_update_init(orc_update *u, int kind, int every, double var,
                     double minvar, double maxvar, double minacc, double maxacc,
                     int adj, int range);
void orc_update_free(orc_update *u);

/* multi-chain timing: nchains independent chains of identical parameters
 * (seeded per chain), nthreads host threads, each chain runs `attempts`
 * run! attempts with the sweep mix (staging l, swap l, CoM step).  Returns
 * elapsed seconds, bead updates through *bead_updates. */
double orc_bench_chains(const orc_params *p, int nchains, int nthreads,
                        long attempts, int ell, double com_step, uint64_t seed,
                        double *bead_updates);

/* sweeps in the engine's schedule (pimc_run / pimc_batch_run), with the
 * reference's moves: per sweep one staging phase -- a random offset o, the
 * imaginary-time circle cut into k = ceil(M/ell) slots starting at o + s ell,
 * one window per (slot, particle) of m = min(slot length, 2 + floor(u (ell -
 * 1))) slices from the slot's start (ReshapeLinear) -- then `swaps` swap
 * attempts (ReshapeSwapLinear: j0, m, n1 and the partner uniform drawn per
 * attempt), then one SingleCenterOfMass attempt per particle with next == n
 * in particle order; the centre-of-mass step adapts once per sweep on that
 * sweep's acceptance (x0.9 below com_minacc, x1.1 above com_maxacc, clamped
 * to [com_min, com_max]).  Measurements (Energy, and Density when dens_nb >
 * 0) at the end of every measure_every-th sweep.  The reference's run!
 * interleaves the same moves at random instead; under the reference's
 * acceptance rules, which are not reversible, the two schedules sample
 * different distributions, so the engine's implementation of those rules is
 * checked against this schedule.  Returns 0 or a negative ORC_* code. */
int orc_run_sweeps(orc_state *st, long nsweeps, int ell, int swaps, double *com_step,
                   double com_min, double com_max, double com_minacc, double com_maxacc,
                   orc_rng *rng, int measure_every, double *e_out, long e_cap, long *e_count,
                   int dens_nb, double *hist, long *ndata, orc_run_stats *stats);

/* time-budgeted timing of a list of chains (parameters ps[c], staging and
 * swap window ells[c]) on nthreads host threads: the chains are dealt to the
 * threads longest first (cost N M (4 with the pair interaction) + N^2 / 2,
 * each to the least-loaded thread), every thread runs one sweep's worth of
 * run! attempts (N (k + 2)) on each of its chains in turn, in chunks of 256
 * attempts, until budget_s seconds have passed since the common start, so
 * that no thread idles while another finishes.  Chains are created and
 * initialised (init_world) before the start.  Returns the wall seconds of the
 * timed region (the last thread's stop), bead updates through
 * *bead_updates and completed sweeps through *sweeps. */
double orc_bench_budget(const orc_params *ps, const int *ells, int nchains, int nthreads,
                        double budget_s, double com_step, uint64_t seed, double *bead_updates,
                        double *sweeps);

#ifdef __cplusplus
}
#endif
#endif
