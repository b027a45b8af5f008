// pimc_types.h -- host/device shared descriptors of the GB300 sweep engine.
#pragma once
#include <stdint.h>

namespace pimc {

// chain flags
enum : int {
  PF_PAIR = 1,      // pair propagator on (System interactions=true)
  PF_PHYS = 2,      // physical semantics (pair action in every move, swap ratio)
  PF_HARD = 4,      // hard-core radius > 0
  PF_LATT = 8,      // square lattice term in V
  PF_HARM = 16,     // harmonic trap term in V
  PF_EXACT = 32,    // sweeps decide every move from exact FP64 sums (no bounded shortcuts)
  PF_CONTACT = 64,  // pair link action from the tabulated contact propagator (with PF_PAIR)
  PF_BEAM = 128,    // optical-lattice term depth * normalized_intensity in V (2D)
};

constexpr int MAX_BEAMS = 16;  // laser beams of an optical-lattice potential
constexpr int kMaxParticles = 8192;  // particles per chain (pimc_params.N)

// observables of one measurement (a row of the series): E_th, E_v, pair
// energy, pair virial energy, squared winding W^2, signed area A_z, sum r^2/M,
// and one spare column
constexpr int NOBS = 8;

// move kinds for counters
enum : int { MV_STAGE = 0, MV_SWAP = 1, MV_COM = 2, MV_PCOM = 3 };

// stream phases (Philox counter word 3, high byte)
enum : unsigned {
  PH_STAGE = 1, PH_STAGE_OFF = 2, PH_SWAP = 3, PH_COM = 4, PH_PCOM = 5, PH_INIT = 6,
  PH_ORDER = 7
};

// constant per chain
struct ChainDesc {
  int N, M, dim, nbins, ncell, flags, ctr, dens_nb;
  int ldn;          // particle stride of a slice row in global memory (== N)
  int wtab;         // bridge-coefficient table covers windows m < wtab
  double L, tau, lambda, beta;
  double hcoef, V0, lat_k;
  double g, inv2s2, rc, hard_a, mu;
  double dens_bw;
  double L2;            // 2L
  double inv2L;         // 1 / (2L), the IEEE quotient
  double rc2;           // rc^2
  double mhtau_g;       // -tau g / 2: weight of a link's pair exponentials
  double q_scale;       // 65536 / (2L): box coordinate -> 16-bit mirror units
  float q_unit2;        // (2L / 65536)^2: squared mirror unit
  unsigned q_lim_rc;    // mirror prefilter bound (squared units) for rc
  unsigned q_lim_hard;  // the same for the hard-core radius
  // bounded pair estimates from the mirror: u^2 / (2 sigma^2), and the
  // squared-unit bounds below which a pair is surely within rc and above
  // which it is surely beyond (kQErr units of mirror error on a distance)
  float q_u2i;
  unsigned q_lim_lo, q_lim_hi;
  // the sweeps' FP32 heat-bath exponent scale per window length m:
  // hb_unit / m = (squared mirror unit) / (4 lambda m tau)
  float hb_unit;
  // L and q_scale rounded to FP32 (the mirror words are formed in FP32)
  float q_Lf, q_scalef;
  long long x_off;      // doubles: x[j][n][d] (slice-major) at dpool + x_off
  long long V_off;      // doubles: V[j][n]
  long long xq_off;     // doubles: 16-bit fixed-point mirror [j][n] (x | y << 16, u32)
  long long host_off;   // doubles: offset of the chain in a host-layout batch buffer
  long long tab_off;    // double2: bridge table (alpha, sigma)[m*wtab + t]
  long long next_off;   // ints: next[n]
  long long dens_off;   // u64: hist[nb^dim]
  long long eser_off;   // doubles: observable series [cap][NOBS]
  // per-slice cell lists (ints at ipool + cl_off, cell_layout below): cl_nc
  // cells per axis (0: no lists, every query scans its slice row), cl_cap
  // moved particles a slice's list tracks before its queries fall back to
  // the row scan, cl_mode 1 (a slice whose build finds its cells too crowded,
  // 9 sum n_c^2 > cl_frac N^2 in 2D, scans its row) or 2 (lists always)
  long long cl_off;
  int cl_nc, cl_cap, cl_mode;
  float cl_frac;
  int eser_cap;
  int smem_bytes;       // bytes to stage x, V, mirror, next in shared memory
  unsigned key0, key1;  // Philox key
  unsigned chain_tag;   // chain id (low 24 bits of counter word 3)
  int pad_;
  // tabulated contact propagator (PF_CONTACT): the Bessel-integral terms
  // T(r1, r2) on the grid r_i = ct_r0 + i ct_h, i < ct_n, row-major
  // ct_tab[i1 * ct_n + i2]
  const double *ct_tab;
  int ct_n, ct_pad_;
  double ct_r0, ct_h, ct_rmax;
  // pair-distance histogram (rdf_nb > 0): counts of unordered pairs per
  // slice with floor(r / rdf_dr) = k, k < rdf_nb
  unsigned long long *rdf;
  int rdf_nb, rdf_pad_;
  double rdf_dr;
  // optical lattice (PF_BEAM): beam k has direction (sin a_k, cos a_k), phase
  // a_k when helical; V = depth |(1/K) sum exp(i phi_k)|^2, phi_k =
  // 2 pi scale (x sin a_k + y cos a_k) (+ a_k)
  int nbeam, beam_helical;
  double beam_depth, beam_scale;
  double beam_sin[MAX_BEAMS], beam_cos[MAX_BEAMS];
};

// ints of a chain's cell lists: end[M][ncq+1] (end of each cell's entries in
// items), dn[M] (moved particles per slice since its build), moved bitmask
// [M][nw], then as 16-bit words items[M][N] (the slice's particles in cell
// order), pos[M][N] (a particle's index in items) and dl[M][cap] (the
// slice's moved particles)
struct CellLayout {
  long long end, dn, moved, items, pos, dl, total;
};
#ifdef __CUDACC__
__host__ __device__
#endif
inline CellLayout cell_layout(int N, int M, int ncq, int cap) {
  CellLayout c;
  const long long nw = (N + 31) / 32;
  c.end = 0;
  c.dn = c.end + (long long)M * (ncq + 1);
  c.moved = c.dn + M;
  c.items = c.moved + (long long)M * nw;
  c.pos = c.items + ((long long)M * N + 1) / 2;
  c.dl = c.pos + ((long long)M * N + 1) / 2;
  c.total = c.dl + ((long long)M * cap + 1) / 2;
  return c;
}

// move mix as seen by the device
struct MixDev {
  int staging_phases;
  int stage_min, stage_max;
  double stage_minacc, stage_maxacc;
  int swaps_per_sweep;
  int swap_min, swap_max;
  double swap_minacc, swap_maxacc;
  int com_phases;
  double com_minstep, com_maxstep, com_minacc, com_maxacc;
  int polymer_com_phases;
  double pcom_minstep, pcom_maxstep, pcom_minacc, pcom_maxacc;
  int adapt;
  int measure_every;
};

// mutable per chain
struct ChainVar {
  unsigned long long sweep;
  int stage_m, swap_m;
  double com_step, pcom_step;
  unsigned long long att[4], acc[4];
  unsigned long long skips;
  double bead_updates;
  unsigned long long n_meas, ndata, eser_count;
  double esum[NOBS], esum2[NOBS];
  int err;
  int cl_hold;  // sweeps left during which the chain's crowded cell lists are not built
  unsigned long long rdf_meas;  // measurements in the pair-distance histogram
  double beads_kind[4];         // bead updates by move kind
};

// device error codes (ChainVar::err and, in PIMC_CHECK builds, the device
// check word; first error wins).  DERR_STATE: next is not a permutation.  The
// others are raised only by the bounds checks of a PIMC_CHECK build:
// DERR_WINDOW a window or slice index out of range, DERR_SCRATCH a shared
// scratch carve past the launch's dynamic shared memory, DERR_QUEUE a
// neighbour-queue push past its capacity, DERR_INDEX a particle index out of
// range.  DERR_INIT: init_world could not place the hard spheres.
enum : int {
  DERR_NONE = 0, DERR_WINDOW = 1, DERR_STATE = 2, DERR_SCRATCH = 3, DERR_QUEUE = 4, DERR_INDEX = 5,
  DERR_INIT = 6
};

}  // namespace pimc
