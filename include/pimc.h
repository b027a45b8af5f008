/*
 * pimc.h -- C ABI of the GB300 engine for the PIMC.jl Monte Carlo sweep.
 *
 * The reference package (oameye/PIMC.jl) has no FFI; its boundary is the
 * Julia API: System(...), the update callables, run!, and the Density/Energy
 * measurements.  Each entry point below names the reference interface it
 * stands in for (file:line within the reference project).  A host wrapper
 * (Julia via ccall, Python via ctypes) reproduces that API on top of it.
 *
 * Conventions
 *   - Every call returns 0 on success or a negative PIMC_E* code; the text of
 *     the last error on the calling host thread is pimc_last_error().
 *   - Positions are caller-owned host buffers in structure-of-arrays order
 *     x[d][n][j] (d < dim, n < N particles, j < M slices, slice 0-based);
 *     they are copied in and out.  Device memory belongs to the handle.
 *   - A handle holds one or more independent chains (a batch).  The
 *     single-chain calls act on chain 0; the pimc_batch_* calls take a chain
 *     index.  A handle is not re-entrant; distinct handles may be used from
 *     distinct host threads.  Each handle owns one CUDA stream.
 */
#ifndef PIMC_H
#define PIMC_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PIMC_ABI_VERSION 5
/* columns of an observable row (pimc_get_observables) */
#define PIMC_NOBS 8

enum {
  PIMC_OK = 0,
  PIMC_EARG = -1,     /* invalid argument */
  PIMC_ECUDA = -2,    /* CUDA runtime error */
  PIMC_ESTATE = -3,   /* invalid state (e.g. next is not a permutation) */
  PIMC_EDEVICE = -4,  /* device-side error flag (capacity, retry cap, ...) */
  PIMC_EDRAWS = -5,   /* injected draw arrays ran out */
  PIMC_ENOMEM = -6
};

/* acceptance semantics */
enum {
  PIMC_SEM_REFERENCE = 0, /* bug-compatible with the reference's updates */
  PIMC_SEM_PHYSICAL = 1   /* same action, applied consistently (detailed balance) */
};

/* outcome of one attempted move */
enum { PIMC_REJECT = 0, PIMC_ACCEPT = 1, PIMC_SKIP = 2, PIMC_HARDCORE = 3 };

/* System(potential; dV, dim, M, N, mu, L, T, lambda, interactions, propint,
 *        g, r_a, length_measurement_cycle, measure_scheme)
 * (src/system.jl:129-167).  Closures cannot cross the ABI, so the potential
 * and the pair propagator are engine-known forms:
 *   V(r)  = 1/2 omega^2 |r|^2 + V0 sum_d sin^2(pi r_d / a)
 *   lnU   = -tau/2 (v(|r1|) + v(|r2|)),  v(r) = g exp(-r^2 / (2 sigma^2))
 * The optical lattices of generate_V (pimc_set_beams) and the tabulated
 * contact propagator of build_prop_int (pimc_set_contact_propagator,
 * pimc_set_contact_table) are attached to a chain after creation.  The
 * hard-core radius is the reference's a = exp(-2 pi / g_contact) when
 * interacting (src/system.jl:151), passed explicitly here. */
typedef struct pimc_params {
  int dim;               /* 1 or 2 */
  int N;                 /* particles */
  int M;                 /* imaginary-time slices */
  double L;              /* half-width: box [-L, L)^dim */
  double T;              /* temperature, beta = 1/T, tau = beta/M */
  double lambda;         /* hbar^2 / 2m */
  double mu;             /* chemical potential (used by lnU when propint < 0) */
  double harmonic_omega; /* 0 = no trap */
  double lattice_V0;     /* 0 = no lattice */
  double lattice_a;
  int interactions;      /* pair propagator on */
  double pair_g, pair_sigma;
  double r_a;            /* neighbour range; 0 -> L/4 (src/system.jl:18-24) */
  double hardcore_a;     /* 0 = off */
  int semantics;         /* PIMC_SEM_* */
  uint64_t seed;         /* Philox key */
  int density_nbins;     /* Density(s; nbins); 0 = no histogram */
  int energy_capacity;   /* Energy(s, n): stored measurements per chain */
  int retry_cap;         /* hard-core retries (s.ctr); 0 -> 10000 */
} pimc_params;

/* The update list of run!(s, n, updates) (src/simulation.jl:29-42) mapped
 * onto a sweep.  One sweep = staging_phases staging phases (every particle's
 * imaginary-time circle cut into windows of up to stage_slices slices,
 * ReshapeLinear, src/updates/reshape.jl:31-91), swaps_per_sweep swap attempts
 * (ReshapeSwapLinear, reshape.jl:123-283), com_phases single-path
 * centre-of-mass phases (SingleCenterOfMass, src/updates/com.jl:136-224) and
 * polymer_com_phases cycle centre-of-mass phases (PolymerCenterOfMass,
 * com.jl:31-104).  Adaptation follows adjust! (src/updates/helper.jl:22-52)
 * once per sweep when adapt != 0. */
typedef struct pimc_move_mix {
  int staging_phases;
  int stage_slices, stage_min, stage_max;
  double stage_minacc, stage_maxacc;
  int swaps_per_sweep;
  int swap_slices, swap_min, swap_max;
  double swap_minacc, swap_maxacc;
  int com_phases;
  double com_step, com_minstep, com_maxstep, com_minacc, com_maxacc;
  int polymer_com_phases;
  double pcom_step, pcom_minstep, pcom_maxstep, pcom_minacc, pcom_maxacc;
  int adapt;
  int measure_every;     /* sweeps between measurements (measurement_Z_sector,
                            src/measurement.jl:1-17); 0 = none */
} pimc_move_mix;

typedef struct pimc_stats {
  unsigned long long attempts[4];  /* staging, swap, com, polymer com */
  unsigned long long accepts[4];
  unsigned long long skips;        /* swap with n1 == n2 */
  double bead_updates;             /* proposed bead positions */
  unsigned long long sweeps;
  unsigned long long measurements;
  int stage_slices, swap_slices;   /* current adaptive var.m */
  double com_step, pcom_step;      /* current adaptive step */
  double bead_updates_kind[4];     /* bead_updates by move kind */
} pimc_stats;

/* ---------------- lifecycle: System constructor (src/system.jl:129-167) */
int pimc_create(const pimc_params *p, void **handle);
/* the parameters a chain was created with */
int pimc_get_params(void *handle, int chain, pimc_params *out);
/* one handle with nchains independent chains (params[c], mix[c]) */
int pimc_batch_create(const pimc_params *params, int nchains, void **handle);
int pimc_destroy(void *handle);
int pimc_num_chains(void *handle, int *nchains);

/* ---------------- state I/O: s.world[n].r / .next (src/system.jl:1-6) */
/* set positions; recomputes the cached link actions (Particle.V) and grids */
int pimc_set_beads(void *handle, const double *x);
int pimc_get_beads(void *handle, double *x);
int pimc_set_next(void *handle, const int *next);
int pimc_get_next(void *handle, int *next);
/* positions, cached link actions V[n][j] and next verbatim */
int pimc_set_raw(void *handle, const double *x, const double *V, const int *next);
int pimc_get_links(void *handle, double *V);
/* init_world (src/system.jl:36-78) on the device: uniform start + Levy loop;
 * with a hard core (hardcore_a > 0) each particle is drawn again while a
 * bead overlaps an earlier particle's bead at the same slice, at most 10000
 * times (system.jl:44-64); a world that cannot be made returns PIMC_ESTATE.
 * pimc_create and pimc_batch_create run it for every chain. */
int pimc_init_world(void *handle);
int pimc_batch_set_beads(void *handle, int chain, const double *x);
int pimc_batch_get_beads(void *handle, int chain, double *x);
int pimc_batch_get_next(void *handle, int chain, int *next);
/* every chain at once: x_all is the concatenation of each chain's
 * x[d][n][j] in chain order.  A page-locked x_all (cudaHostAlloc,
 * cudaHostRegister) is read or written by the GPU in place, the copy fused
 * with the layout transpose; a pageable one takes one staged copy. */
int pimc_batch_set_beads_all(void *handle, const double *x_all);
int pimc_batch_get_beads_all(void *handle, double *x_all);
/* running energy sums of every chain: sum[c][4], sumsq[c][4], count[c] */
int pimc_batch_energy_sums_all(void *handle, double *sum, double *sumsq,
                               unsigned long long *count);

/* ---------------- sweep: run!(s, n, updates) (src/simulation.jl:29-42) */
int pimc_set_move_mix(void *handle, int chain, const pimc_move_mix *mix); /* chain<0: all */
int pimc_run(void *handle, long long n_sweeps);
/* all chains, one persistent launch per sweep block from a device work
 * queue, captured in a CUDA graph */
int pimc_batch_run(void *handle, long long n_sweeps);
/* the same sweeps issued as one plain launch per chain (no queue, no graph) */
int pimc_batch_run_plain(void *handle, long long n_sweeps);
/* pimc_batch_set_beads_all(x_in), pimc_batch_run(n_sweeps),
 * pimc_batch_get_beads_all(x_out) as one call with no host round trip in
 * between.  When both buffers are page-locked, the layout transposes read
 * x_in and write x_out in place over the host link (chunks is ignored).
 * Otherwise the positions move through a staging buffer in `chunks`
 * contiguous groups of about equal bytes (chunks <= 0: 4), one group's copy
 * on its own copy stream while the compute stream transposes another.  All
 * chains sweep together in between, as pimc_batch_run does.  The chains
 * reach the same states as by the three calls.  x_in and x_out may be the
 * same buffer.  pimc_last_run_ms gives the device time of the whole call. */
int pimc_batch_run_io(void *handle, const double *x_in, double *x_out, long long n_sweeps,
                      int chunks);
/* launch shape of pimc_batch_run.  warp_per_chain = 0: one CTA of `block`
 * threads per chain, the chain's state staged in shared memory when it fits
 * state_smem_bytes.  warp_per_chain = 1: every warp of a `block`-thread CTA
 * runs its own chain (block <= 256, state_smem_bytes ignored).  Both shapes
 * give the same chains bit for bit; they differ in speed only. */
typedef struct {
  int warp_per_chain;
  int block;
  int sweeps_per_launch;
  int state_smem_bytes;
  /* 0: every phase of a sweep in one launch; 1 (one CTA per chain only):
   * staging, swaps and the rest as three launches per sweep, each phase
   * finished by every chain before the next starts */
  int split_phases;
  /* with split_phases: CTA size of the staging, swap and remaining launches
   * (0: block) */
  int phase_block[3];
  /* with split_phases: 1 runs that phase with one warp per chain (every warp
   * of a phase_block-thread CTA its own chain, phase_block <= 256); the swap
   * phase (index 1) only */
  int phase_warp[3];
  /* with split_phases, the swap phase (index 1) with one CTA of at most 64
   * threads per chain: its kernel compiled for at most 170 or 255 registers
   * a thread (6 or 4 resident CTAs per SM) instead of 128 (0 or 128) */
  int phase_regs[3];
  /* the neighbour queries' candidates: 0 leaves PIMC_OPT_CELL_LISTS as it
   * is; 1 + a value of it (1 off, 2 auto, 3 always) sets it for every chain.
   * pimc_batch_get_launch reports 1 + the current value.  The chains are the
   * same either way; only the speed differs. */
  int cell_lists;
} pimc_launch;
/* time candidate launch shapes on the handle's own chains and keep the
 * fastest; the chains are restored afterwards.  For chains with cell lists
 * it also times the chosen shape with the lists on (the handle's setting)
 * and off, and keeps the faster (cell_lists of chosen).  chosen may be
 * NULL. */
int pimc_batch_tune(void *handle, int sweeps_per_trial, pimc_launch *chosen);
int pimc_batch_set_launch(void *handle, const pimc_launch *launch);
int pimc_batch_get_launch(void *handle, pimc_launch *launch);

/* ---------------- single moves with injected draws (parity level b) */
/* (u::ReshapeLinear)(s) with n, j0, m given (reshape.jl:31-91).  normals are
 * consumed d per interior bead in order; uniforms[0] is the Metropolis
 * uniform, read only when delta < 1.  proposal (optional) receives the
 * teleported window (m+1)*dim, bead-major. */
int pimc_attempt_staging(void *handle, int n, int j0, int m, const double *normals,
                         int n_normals, const double *uniforms, int n_uniforms, int *result,
                         double *proposal);
/* (u::ReshapeSwapLinear)(s) with j0, m, n1 and the partner-selection uniform
 * given (reshape.jl:123-283, helper.jl:224-267) */
int pimc_attempt_swap(void *handle, int j0, int m, int n1, double u_pick, const double *normals,
                      int n_normals, const double *uniforms, int n_uniforms, int *result,
                      int *n2, double *proposal);
/* (u::SingleCenterOfMass)(s) on particle n (com.jl:136-224); uniforms: dim
 * shift uniforms then the Metropolis uniform */
int pimc_attempt_com(void *handle, int n, double step, const double *uniforms, int n_uniforms,
                     int *result);
/* PolymerCenterOfMass on the cycle containing n (com.jl:31-104, working) */
int pimc_attempt_polymer_com(void *handle, int n, double step, const double *uniforms,
                             int n_uniforms, int *result);

/* ---------------- action evaluation (parity level a) */
/* out[0] = sum lnK, out[1] = sum lnV (recomputed), out[2] = pair sum lnU
 * (each unordered pair once; Gaussian pair or contact table), out[3] = sum
 * of cached V (src/propagator.jl:16-28, src/system.jl:26-28) */
int pimc_eval_action(void *handle, double out[4]);
/* w_initial / w_updated of a staging move for a given proposed window
 * rp[(m+1)*dim] (reshape.jl:66-77) */
int pimc_eval_staging_weights(void *handle, int n, int j0, int m, const double *rp,
                              double *w_init, double *w_upd);

/* ---------------- estimators (src/measurement.jl) */
int pimc_measure(void *handle);  /* one measurement of every chain now */
/* Energy (measurement.jl:92-122): rows of 4: E_th, E_v (reference
 * formulas), pair energy term, pair virial term */
int pimc_get_energies(void *handle, int chain, double *out, int cap, int *count);
/* running sums per chain: sum[4], sumsq[4], count */
int pimc_get_energy_sums(void *handle, int chain, double *sum, double *sumsq,
                         unsigned long long *count);
/* Density (measurement.jl:45-55): nb^dim counts (column-major) and ndata */
int pimc_get_density(void *handle, int chain, double *hist, unsigned long long *ndata);
/* the estimators the reference leaves as TODOs (measurement.jl:125-127),
 * measured with every Energy row: rows of PIMC_NOBS = E_th, E_v, pair
 * energy, pair virial energy, W^2 (squared total minimum-image displacement
 * of all links: the winding estimator, rho_s/rho = <W^2> / (2 dim lambda
 * beta N) in a periodic box), A_z (1/2 sum over links of x dy - y dx: the
 * area estimator about the origin, rho_s/rho = 2 <A_z^2> / (lambda beta
 * <sum r^2 / M>) in a trap), sum r^2 / M, 0 */
int pimc_get_observables(void *handle, int chain, double *out, int cap, int *count);
/* running sums of the observables: sum[PIMC_NOBS], sumsq[PIMC_NOBS], count */
int pimc_get_observable_sums(void *handle, int chain, double *sum, double *sumsq,
                             unsigned long long *count);
/* radial distribution: every measurement adds, for each slice, every
 * unordered pair with minimum-image distance r to bin floor(r / dr),
 * dr = rmax / nbins (rmax 0: L), bins past nbins dropped.  chain < 0: every
 * chain; nbins 0 switches it off.  Setting it clears the histograms. */
int pimc_set_radial(void *handle, int chain, int nbins, double rmax);
/* the pair counts (nbins) and the number of measurements they hold; g(r) =
 * hist[k] / (nmeas M N(N-1)/2 * shell(k) / (2L)^dim) */
int pimc_get_radial(void *handle, int chain, double *hist, unsigned long long *nmeas);
int pimc_reset_measurements(void *handle);

/* the optical-lattice potentials of the reference's examples
 * (examples/tools/potentialtools.jl:1-39): adds depth * I(r) to V, with
 * I = |(1/K) sum_k exp(i phi_k)|^2, phi_k = 2 pi scale (x sin a_k + y cos a_k),
 * plus a_k when helical; K = nangles <= 16 beams (0 removes it); 2D chains
 * only; chain < 0: every chain.  generate_V(scale, depth, sym; attractive)
 * is depth -> -depth with the named angle sets.  The cached link actions are
 * recomputed.  The adjoint's parameter derivatives do not cover depth. */
int pimc_set_beams(void *handle, int chain, const double *angles, int nangles, double scale,
                   double depth, int helical);

/* ---------------- adjoint: per-bead dS_pot/dr and dS/d(V0, omega, g) */
/* dSdr [dim][N][M] (optional), dSdtheta[3] = d/dV0, d/domega, d/dg,
 * extra[4] = S_ext, S_pair, virial energy (external + pair), sum r.dS/dr */
int pimc_adjoint(void *handle, int chain, double *dSdr, double *dSdtheta, double *extra);
/* The same adjoint, same arguments and results, with no device allocation:
 * its scratch is a static 3.2 MB device array instead of a buffer that
 * pimc_adjoint grows with cudaMalloc.  No reference counterpart (PIMC.jl
 * has no adjoint).  For callers that must not allocate device memory while
 * they run: an optimisation loop whose host framework owns the GPU's memory
 * through its own pool (CUDA.jl, a caching allocator) that a cudaMalloc
 * behind its back would fragment or push past its limit, or a process
 * already at the edge of device memory where a late cudaMalloc can fail in
 * the middle of a run.
 * Limit: chains of at most 65536 beads (N*M) and 8192 particles; larger
 * chains return PIMC_EARG and must use pimc_adjoint.  The handle's device
 * must be the current device.  The array's address on a device is looked up
 * when a handle is created on it (set-up, with that device current), so the
 * calls themselves make no lookup; after a cudaDeviceReset, which destroys
 * every handle made before it, the first handle created again repeats the
 * set-up.  The array is shared by all handles of the process and keeps the
 * last call's contents: calls that overlap in time (from several threads, on
 * any handles of one device) race on it. */
int pimc_adjoint_noalloc(void *handle, int chain, double *dSdr, double *dSdtheta,
                         double *extra);
/* pimc_adjoint for every chain of the batch at once (four launches over all
 * chains, scratch carved from a pool the handle allocates on the first call
 * and keeps): dSdtheta[c][3], extra[c][4] as pimc_adjoint per chain c, and
 * dSdr_all (optional) in the layout of pimc_batch_get_beads_all, each
 * chain's [dim][N][M] in chain order.  pimc_last_run_ms then gives the
 * device time of the four launches.  No reference counterpart (PIMC.jl has
 * no adjoint); the examples' pmap over systems is what it batches. */
int pimc_batch_adjoint(void *handle, double *dSdtheta, double *extra, double *dSdr_all);
/* change (V0, omega, g) in place; cached links are recomputed */
int pimc_set_potential(void *handle, int chain, double V0, double omega, double g);

/* ---------------- diagnostics, checkpoint */
int pimc_get_stats(void *handle, int chain, pimc_stats *out);
/* aggregate over chains */
int pimc_get_total_stats(void *handle, pimc_stats *out);
/* opaque, versioned snapshot of every chain: beads, links, next, counters,
 * adaptive variables, generator position, density and pair-distance
 * histograms; restoring it reproduces the following sweeps bit for bit.  A
 * snapshot restores only into a handle of the same shape, including the
 * pair-distance bins of pimc_set_radial (else PIMC_ESTATE, nothing written) */
int pimc_state_size(void *handle, size_t *bytes);
int pimc_get_state(void *handle, void *buf, size_t bytes);
int pimc_set_state(void *handle, const void *buf, size_t bytes);

/* ---------------- files (examples/tools/savetools.jl) */
/* save_paths (savetools.jl:4-35): a CSV with columns tau, "p<n> x"[, "p<n> y"]
 * and M + 1 rows (tau = j beta/M; the last row closes each path with the
 * first bead of the next particle of its cycle), numbers printed as Julia
 * prints a Float64 */
int pimc_write_paths_csv(void *handle, int chain, const char *path);
/* save_density (savetools.jl:37-65): counts / ((2L/nbins) ndata) with a pos
 * column range(-L, L, length = nbins); 2D: columns x1..x<nbins>, counts
 * column-major (x index first) as pimc_get_density returns them */
int pimc_write_density_csv(const char *path, int dim, int nbins, double L, const double *counts,
                           unsigned long long ndata);
/* the pimc_get_state snapshot in a file: "PIMCCKPT", ABI version, size,
 * state, FNV-1a checksum; loading checks all four and the handle's shape */
int pimc_save_checkpoint(void *handle, const char *path);
int pimc_load_checkpoint(void *handle, const char *path);
/* x printed as Julia prints a Float64 ("0.5", "1.0e-5", "1.234567e6") */
int pimc_format_float(double x, char *out, size_t cap);
/* prop_rel_interpolate_terms (src/propagator.jl:36-73): the integral terms
 * T[i1][i2] = -I1 - I2 + I3 of the contact-interaction propagator on the
 * reference's grid r_i = 1e-20 + i (range - 1e-20)/(n - 1), n = 600 there,
 * computed on the device (row-major, symmetric) */
int pimc_contact_table(double g0, double tau, double range, int n, double *out);
/* build_prop_int(range, g0, tau) attached as the pair propagator of a chain
 * (chain < 0: every chain) that was created with interactions = 1:
 *   lnU(r1, r2) = log(1 + T(|r1|, |r2|) / prop_rel0(r1, r2, tau)), or -mu
 *   where the argument is negative (src/system.jl:26-28,
 *   src/propagator.jl:74-89), T bilinear in the table above (n = 0 -> 600).
 * tau is the chain's own; chains with equal (g0, tau, range, n) share one
 * device table.  It replaces the Gaussian pair in every move and in
 * pimc_eval_action; the pair energy columns of the estimators read 0 for it,
 * and pimc_adjoint refuses it.  Radii outside [1e-20, range] are clamped to
 * the grid, where the reference raises a BoundsError. */
int pimc_set_contact_propagator(void *handle, int chain, double g0, double range, int n);
/* the same with a caller-made table T[i1][i2] (row-major n*n, on the grid
 * above), e.g. one stored by the reference's precompute_int_prop.jl */
int pimc_set_contact_table(void *handle, int chain, const double *table, int n, double range);
/* the chain's contact table: *n = 0 when it has none; out (optional) receives
 * n*n values and must hold cap >= n*n */
int pimc_get_contact_table(void *handle, int chain, double *out, size_t cap, int *n,
                           double *range);
/* back to the Gaussian pair of pimc_params (chain < 0: every chain) */
int pimc_clear_contact(void *handle, int chain);
/* measurement utility, no reference counterpart: FP64 fused multiply-add
 * throughput of the handle's device in TFLOP/s (eight independent DFMA
 * chains per thread over the whole GPU, best of three timed launches) --
 * the denominator of the sweep's FP64 roofline */
int pimc_fp64_peak(void *handle, double *tflops);
/* measurement utility: n sweeps of every chain as separately issued phase
 * launches (staging, swaps, rest; one launch when the launch shape is not
 * split) with CUDA events around each phase; ms[3] receives the device time
 * of each phase summed over the sweeps */
int pimc_batch_phase_times(void *handle, long long n_sweeps, double ms[3]);
/* device time of the last run call or pimc_batch_adjoint (CUDA events on
 * the handle's stream) */
int pimc_last_run_ms(void *handle, double *ms);
/* the handle's device: its name (NUL-terminated, at most cap bytes) and SM
 * count; no reference counterpart (keys the tuner's cache of launch shapes) */
int pimc_device_info(void *handle, char *name, size_t cap, int *num_sms);
/* diagnostics, no reference counterpart: in the profiling build (nvcc
 * -DPIMC_PROFILE=1) the permutation swap adds the clock cycles of its
 * sections (0 heat-bath exponents, 1 partner search, 2 physical ratio, 3
 * bridges, 4 new beads, 5 pair-free sums and early accept, 6 bounded pair
 * estimates, 7 exact pair sums, 8 decision, 9 accepted write-back) to
 * out[0..15] and counts outcomes in out[16..31] (16 attempts, 17 n2 == n1,
 * 18 early accepts, 19 decided by the estimates, 20 exact sums, 21
 * accepted, 22 rejected), summed over every CTA; reset != 0 clears them
 * after the read.  Other builds return PIMC_EARG. */
int pimc_swap_profile(void *handle, unsigned long long *out, int reset);
/* kernel launches issued by the last run call */
int pimc_last_run_launches(void *handle, long long *launches);
/* engine options: PIMC_OPT_FORCE_WARP_WINDOW routes pair-free staging
 * attempts through the warp-cooperative window as well (parity coverage);
 * PIMC_OPT_EXACT_DECISIONS makes sweeps take every accept/reject decision
 * from the exact FP64 sums, without the bounded shortcuts (pair-sum
 * estimates from the position mirror, FP32 log-space Metropolis tests, the
 * reference rules' pair-free early accept).  Both ways give the same chains
 * bit for bit; the option exists to show it.
 * PIMC_OPT_CELL_LISTS: the sweeps' neighbour queries (the cell grid of
 * find_nns, src/nearest_neighbours.jl:26-154) take their candidates from
 * per-slice cell lists (value 2), from a scan of the whole slice (0), or
 * from the lists except on slices whose cells are too crowded for them to
 * pay (1, the default): 3^dim sum over cells of n_c^2 above the crowding
 * bound times N^2.  PIMC_OPT_CELL_CROWDING sets that bound in thousandths
 * (default 500).  The neighbour sets are the same every way; the order in
 * which a query sums its pairs is not, so the exact sums may differ in
 * their last bits.  Chains whose cells would be fewer than 5 per axis
 * always scan. */
enum {
  PIMC_OPT_FORCE_WARP_WINDOW = 1, PIMC_OPT_EXACT_DECISIONS = 2, PIMC_OPT_CELL_LISTS = 3,
  PIMC_OPT_CELL_CROWDING = 4
};
int pimc_set_option(void *handle, int key, long long value);
const char *pimc_last_error(void);
int pimc_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
