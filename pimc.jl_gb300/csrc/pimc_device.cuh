// pimc_device.cuh -- device building blocks of the sweep: counter-based
// random numbers, the action pieces, neighbour scans, and the staging
// window written once and shared by the sweep kernels and the injected-draw
// attempt kernels.
//
// Layout: positions are slice-major on the device, x[j][n][d] (all particles
// of one imaginary-time slice contiguous, a bead's coordinates in one 16-byte
// unit, so that gathering a neighbour touches one sector), cached links
// V[j][n].  Thread-per-window staging reads slices of consecutive particles
// (coalesced).  Every chain keeps a 16-bit fixed-point mirror xq[j][n] of the
// positions (one 32-bit word per bead): a neighbour query tests candidates
// with integer arithmetic and a bound that covers the rounding, and evaluates
// the few that pass exactly in FP64, so the neighbour set is exactly the
// reference's (every bead within 2L/nbins, src/nearest_neighbours.jl:131-154).
// The candidates come from per-slice cell lists (the reference's cell grid,
// src/nearest_neighbours.jl:26-104: a counting sort of the slice's mirror
// words, rebuilt at the start of every phase that queries, moved beads
// tracked on the side) or, for slices whose cells are too crowded to pay,
// from a scan of the whole slice row.
//
// Reference correspondence (oameye/PIMC.jl):
//   distance / lnK / lnV / teleport      src/propagator.jl:6-32
//   lnU (Gaussian propint)               src/system.jl:26-28
//   neighbour set                        src/nearest_neighbours.jl:106-179
//   metropolis                           src/updates/helper.jl:3-5
//   hardspherelevy!                      src/updates/helper.jl:141-222
//   ReshapeLinear                        src/updates/reshape.jl:31-91
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pimc_types.h"

namespace pimc {

constexpr int WMAX = 64;     // largest staging / swap window m handled on the device
constexpr int TWMAX = 32;    // thread-per-window variant handles m <= TWMAX
// doubles of per-warp scratch of window_warp: new beads x, y, their external
// potential, normals (2 per bead), the neighbour queue (96 entries), the
// new beads' mirror words, and 4 doubles through which the warps of a
// staging team exchange their partial sums
constexpr int TEAM_SLOT_D = 5 * (WMAX + 1) + 96 + (WMAX + 2) / 2;
constexpr int WARP_SCRATCH_D = TEAM_SLOT_D + 4;

// move outcomes (PIMC_REJECT / ACCEPT / SKIP / HARDCORE of pimc.h)
constexpr int RES_REJECT = 0, RES_ACCEPT = 1, RES_SKIP = 2, RES_HARDCORE = 3;

// ---------------------------------------------------------------------------
// bounds checks of the PIMC_CHECK build (nvcc -DPIMC_CHECK=1).  A window or
// slice index, a particle index, a shared-scratch carve or a neighbour-queue
// push that falls outside its range records (code << 32 | chain) in
// g_check_word, first error wins, and the access is skipped; the host reads
// the word after every run and reports PIMC_EDEVICE.  Nothing traps.  In the
// default build check_ok() is a constant true and compiles away.
// ---------------------------------------------------------------------------
#ifndef PIMC_CHECK
#define PIMC_CHECK 0
#endif
// one per kernel translation unit (static), read by the host through each
// unit's accessor
static __device__ unsigned long long g_check_word;

__device__ __forceinline__ bool check_ok(bool cond, int code, const ChainDesc &d) {
#if PIMC_CHECK
  if (!cond) {
    atomicCAS(&g_check_word, 0ull, ((unsigned long long)code << 32) | (d.chain_tag & 0xFFFFFFu));
    return false;
  }
#endif
  return true;
}

// ---------------------------------------------------------------------------
// per-section clock counters of the permutation swap (nvcc -DPIMC_PROFILE=1):
// thread 0 of the group adds the clock64() cycles between section marks to
// g_prof[0..15] and counts outcomes in g_prof[16..31].  Compiled out in the
// default build.
// ---------------------------------------------------------------------------
#ifndef PIMC_PROFILE
#define PIMC_PROFILE 0
#endif
// one per kernel translation unit (static)
static __device__ unsigned long long g_prof[32];
#if PIMC_PROFILE
#define PROF_DECL long long prof_t_ = clock64()
#define PROF_MARK(slot)                                                              \
  do {                                                                               \
    const long long n_ = clock64();                                                  \
    if (threadIdx.x == 0) atomicAdd(&g_prof[slot], (unsigned long long)(n_ - prof_t_)); \
    prof_t_ = n_;                                                                    \
  } while (0)
#define PROF_COUNT(slot)                                          \
  do {                                                            \
    if (threadIdx.x == 0) atomicAdd(&g_prof[16 + (slot)], 1ull); \
  } while (0)
#else
#define PROF_DECL
#define PROF_MARK(slot) \
  do {                  \
  } while (0)
#define PROF_COUNT(slot) \
  do {                   \
  } while (0)
#endif

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and draws derived from it
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k.x += 0x9E3779B9u; k.y += 0xBB67AE85u; }
    const unsigned hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const unsigned hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  return c;
}

// 53-bit uniform in [0, 1)
__device__ __forceinline__ double u53(unsigned a, unsigned b) {
  const unsigned long long x = ((((unsigned long long)a) << 32) | b) >> 11;
  return (double)x * 0x1.0p-53;
}

// Box-Muller pair from two 53-bit uniforms.  The transcendental functions
// run in FP32 (CUDA's logf / sincospif / sqrtf as library calls): the FP64
// pipe of this part issues 2 lanes per SM clock, and a normal's relative
// error of about 1e-7 distorts the sampled Gaussian far below any Monte Carlo
// error.  u1 keeps its 53-bit range (as a float, exponent intact), so the
// tails reach 8.6 sigma.  Injected-draw attempts take their normals as given.
__device__ __forceinline__ void normal2(uint4 r, double &z0, double &z1) {
  const unsigned long long x1 = ((((unsigned long long)r.x) << 32) | r.y) >> 11;
  const unsigned long long x2 = ((((unsigned long long)r.z) << 32) | r.w) >> 11;
  const float u1 = __ull2float_rn((1ull << 53) - x1) * 0x1.0p-53f;  // (0, 1]
  const float u2 = __ull2float_rn(x2) * 0x1.0p-53f;                 // [0, 1]
  const float rad = sqrtf(-2.f * logf(u1));
  float s, c;
  sincospif(2.f * u2, &s, &c);
  z0 = (double)(rad * c);
  z1 = (double)(rad * s);
}

struct Stream {
  uint2 key;
  unsigned item, sweep, tag;
  __device__ __forceinline__ uint4 at(unsigned draw) const {
    return philox10(make_uint4(draw, item, sweep, tag), key);
  }
  __device__ __forceinline__ double uni(unsigned draw) const {
    const uint4 r = at(draw);
    return u53(r.x, r.y);
  }
};

__device__ __forceinline__ Stream make_stream(const ChainDesc &d, unsigned long long sweep,
                                              unsigned phase, unsigned item) {
  Stream s;
  s.key = make_uint2(d.key0, d.key1);
  s.item = item;
  s.sweep = (unsigned)sweep;
  s.tag = (phase << 24) | (d.chain_tag & 0xFFFFFFu);
  return s;
}

// draw indices inside one move's stream
constexpr unsigned DRAW_SEQ = 0x40000000u;     // sequential normals (hard-core retries)
constexpr unsigned DRAW_UNI = 0x80000000u;     // sequential uniforms (CoM shifts)
constexpr unsigned DRAW_CHOICE = 0xA0000000u;  // move choices (window, partner)
constexpr unsigned DRAW_ACCEPT = 0xC0000000u;  // Metropolis uniform

// Generator-backed draws for one move.  bead_normals(k) is a pure function of
// the bead index so lanes may evaluate beads in parallel.
struct GenDraws {
  static constexpr bool kSweep = true;  // counter-based: decisions may use bounded estimates
  Stream s;
  unsigned seq;
  int have;
  double spare;
  __device__ __forceinline__ void bead_normals(int k, int dim, double *z) const {
    double a, b;
    normal2(s.at((unsigned)k), a, b);
    z[0] = a;
    if (dim > 1) z[1] = b;
  }
  __device__ __forceinline__ void consumed(int) {}
  __device__ __forceinline__ double normal() {
    if (have) { have = 0; return spare; }
    double a, b;
    normal2(s.at(DRAW_SEQ + seq++), a, b);
    spare = b;
    have = 1;
    return a;
  }
  __device__ __forceinline__ double uniform() { return s.uni(DRAW_UNI + seq++); }
  __device__ __forceinline__ double uniform_accept() { return s.uni(DRAW_ACCEPT); }
};

__device__ __forceinline__ GenDraws gen_draws(const Stream &s) {
  GenDraws g;
  g.s = s;
  g.seq = 0;
  g.have = 0;
  g.spare = 0.0;
  return g;
}

// Injected draws (parity level b): normals bead-major, d per bead, in the
// order the reference draws them; uniforms consumed sequentially.
struct InjDraws {
  static constexpr bool kSweep = false;  // injected draws: exact decisions only
  const double *nrm;
  int n_nrm, pn;
  const double *uni;
  int n_uni, pu;
  int exh;
  __device__ __forceinline__ void bead_normals(int k, int dim, double *z) const {
    for (int d = 0; d < dim; ++d) {
      const int i = pn + k * dim + d;
      z[d] = i < n_nrm ? nrm[i] : 0.0;
    }
  }
  __device__ __forceinline__ void consumed(int cnt) { pn += cnt; }
  __device__ __forceinline__ double normal() {
    if (pn < n_nrm) return nrm[pn++];
    exh = 1;
    return 0.0;
  }
  __device__ __forceinline__ double uniform() {
    if (pu < n_uni) return uni[pu++];
    exh = 1;
    return 0.5;
  }
  __device__ __forceinline__ double uniform_accept() { return uniform(); }
};

// ---------------------------------------------------------------------------
// 16-bit fixed-point mirror of the positions: a coordinate x of the periodic
// box [-L, L) is stored as round((x + L) 65536 / 2L) mod 65536, x in the low
// and y in the high half of a 32-bit word.  A wrapped 16-bit difference is
// the minimum-image separation in mirror units, so a neighbour prefilter is
// integer arithmetic on one word per bead (half the bytes of an FP32 copy).
// ---------------------------------------------------------------------------
// formed in FP32: the roundings of x, L, the sum, q_scale and the product
// move the value by at most 2^-24 (4 L s + 2 L s + 2^16) = 2^-6 units (L s =
// 2^15), so a word lies within 0.516 units of the exact position instead of
// 0.5.  Two such words and a shifted centre differ from the exact
// separation by at most 1.55 units per axis, 2.2 in distance, inside the
// prefilter bounds' 4 units and the estimates' kQErr = 3.  The FP64 pipe
// does one conversion instead of an addition, a product and a conversion
__device__ __forceinline__ unsigned qcoord(const ChainDesc &d, double x) {
  return (unsigned)__float2int_rn(((float)x + d.q_Lf) * d.q_scalef) & 0xffffu;
}
__device__ __forceinline__ unsigned qpos(const ChainDesc &d, double x, double y) {
  return qcoord(d, x) | (d.dim > 1 ? qcoord(d, y) << 16 : 0u);
}
// squared minimum-image separation of two mirror words, in squared units
__device__ __forceinline__ unsigned qdist2(unsigned a, unsigned b) {
  const unsigned dd = __vsub2(a, b);
  const int dx = ((int)(dd << 16)) >> 16, dy = ((int)dd) >> 16;
  return (unsigned)(dx * dx) + (unsigned)(dy * dy);
}

// ---------------------------------------------------------------------------
// per-slice cell lists (the cell grid of src/nearest_neighbours.jl:26-104)
//
// A slice's particles sorted by the cell of their mirror word, nc cells per
// axis on the 16-bit periodic mirror, each at least as wide as the largest
// prefilter radius in mirror units: a particle that passes a prefilter
// around a centre lies in the 3 x 3 block of cells (3 in 1D) around the
// centre's cell.  The lists are built (a stable counting sort: the particles
// of a cell in index order) at the start of every phase that queries them;
// a particle whose bead moves afterwards is flagged in items (bit 15: its
// cell is stale, queries skip the entry) and appended to the slice's list of
// moved particles, which every query of the slice takes in full.  Each
// slice's moves are marked by one thread in a fixed order, so the lists, and
// with them the order in which a query visits candidates, are a function of
// the chain's history.  A slice whose moved list overflows, or whose build
// found the cells too crowded to pay (dn = kCellOff), is scanned row-wise.
// ---------------------------------------------------------------------------
constexpr int kCellOff = 1 << 30;
// sweeps for which a chain whose build found most slices crowded scans rows
// without building
constexpr int kCellHold = 8;

struct CellLists {
  int N, nc, ncq, cap, nw;
  int *end;              // end[j*(ncq+1) + c]: end of cell c's entries (begin: end[c-1], or 0)
  int *dn;               // dn[j]: moved particles since the build (kCellOff: row scan)
  unsigned *moved;       // moved[j*nw + w]: bitmask of the moved particles
  unsigned short *items; // items[j*N + k]: particles in cell order; bit 15 = moved
  unsigned short *pos;   // pos[j*N + n]: the index of particle n in items
  unsigned short *dl;    // dl[j*cap + k]: moved particles, in the order of their first move
  __device__ __forceinline__ void bind(const ChainDesc &d, int *ipool) {
    N = d.N;
    nc = d.cl_nc;
    ncq = d.dim > 1 ? nc * nc : nc;
    cap = d.cl_cap;
    nw = (d.N + 31) >> 5;
    const CellLayout l = cell_layout(d.N, d.M, ncq, cap);
    int *b = ipool + d.cl_off;
    end = b + l.end;
    dn = b + l.dn;
    moved = (unsigned *)(b + l.moved);
    items = (unsigned short *)(b + l.items);
    pos = (unsigned short *)(b + l.pos);
    dl = (unsigned short *)(b + l.dl);
  }
  __device__ __forceinline__ int cx(unsigned q) const {
    return (int)(((q & 0xffffu) * (unsigned)nc) >> 16);
  }
  __device__ __forceinline__ int cy(unsigned q) const {
    return ncq == nc ? 0 : (int)(((q >> 16) * (unsigned)nc) >> 16);
  }
  __device__ __forceinline__ int cell(unsigned q) const { return cx(q) + nc * cy(q); }
  // particle n's bead at slice j has moved since the build.  The marks of a
  // slice within one move come from one thread (plain loads and stores: the
  // three reads are independent, one round trip)
  __device__ __forceinline__ void mark(int n, int j) const {
    unsigned *w = moved + (size_t)j * nw + (n >> 5);
    const unsigned bit = 1u << (n & 31);
    const unsigned old = *w;
    const int k = dn[j];
    const unsigned short p = pos[(size_t)j * N + n];
    if (old & bit) return;
    *w = old | bit;
    dn[j] = k + 1;
    if (k < cap) {
      items[(size_t)j * N + p] = (unsigned short)(n | 0x8000);  // the entry of n, flagged
      dl[(size_t)j * cap + k] = (unsigned short)n;
    }
  }
  // particles a and b trade their beads at slice j.  When neither has moved
  // since the build the lists stay exact by trading the two entries (the
  // set of positions is unchanged); otherwise both are marked.
  __device__ __forceinline__ void trade(int a, int b, int j) const {
    const unsigned *mw = moved + (size_t)j * nw;
    const unsigned wa = mw[a >> 5], wb = mw[b >> 5];
    unsigned short *it = items + (size_t)j * N, *ps = pos + (size_t)j * N;
    const unsigned short pa = ps[a], pb = ps[b];
    if (((wa >> (a & 31)) & 1u) == 0u && ((wb >> (b & 31)) & 1u) == 0u) {
      it[pa] = (unsigned short)b;
      it[pb] = (unsigned short)a;
      ps[a] = pb;
      ps[b] = pa;
      return;
    }
    mark(a, j);
    mark(b, j);
  }
  // whether queries of slice j use the lists (uniform across the warp)
  __device__ __forceinline__ bool usable(int j) const { return dn[j] <= cap; }
};

// ---------------------------------------------------------------------------
// chain view: x/V/next/xq may live in shared or global memory (generic pointers)
// ---------------------------------------------------------------------------
struct CV {
  const ChainDesc *d;
  double *x;          // x[(j*ldn + n)*dim + k]: a bead's coordinates in one 16-byte unit
  double *V;          // V[j*ldn + n]
  int *next;
  unsigned *xq;       // fixed-point mirror [j*ldn + n]
  const double2 *tab; // (alpha, sigma)[m*wtab + t]
  const double2 *tabw; // (w, k)[m*wtab + t] of the closed form (bridge_w)
  unsigned long long *hist;
  double *eser;
  // the chain's cell lists while a phase maintains them (moves mark, queries
  // use them); nullptr: every query scans its row, moves mark nothing
  const CellLists *cl;
  int N, M, dim, ldn;
  __device__ __forceinline__ double &X(int k, int n, int j) const {
    return x[((size_t)j * ldn + n) * dim + k];
  }
  __device__ __forceinline__ double &Vl(int n, int j) const { return V[(size_t)j * ldn + n]; }
  __device__ __forceinline__ double Xd(int k, int n, int j) const {
    return k < dim ? X(k, n, j) : 0.0;
  }
  __device__ __forceinline__ unsigned Q(int n, int j) const { return xq[(size_t)j * ldn + n]; }
  // every position write goes through here so that the mirror and the cell
  // lists follow; the writes of one slice within a move come from one thread
  __device__ __forceinline__ void set_pos(int n, int j, double px, double py) const {
    X(0, n, j) = px;
    if (dim > 1) X(1, n, j) = py;
    xq[(size_t)j * ldn + n] = qpos(*d, px, py);
    if (cl) cl->mark(n, j);
  }
  // the same with the mirror word already computed (qpos of px, py)
  __device__ __forceinline__ void set_pos_q(int n, int j, double px, double py, unsigned q) const {
    X(0, n, j) = px;
    if (dim > 1) X(1, n, j) = py;
    xq[(size_t)j * ldn + n] = q;
    if (cl) cl->mark(n, j);
  }
  // exchange the beads of particles a and b at slice j, mirror and cached
  // link included, with every load issued before the first store: the
  // compiler cannot know that a != b, so exchanging the arrays one after
  // another would cost one memory round trip each
  __device__ __forceinline__ void exchange_linked(int a, int b, int j) const {
    double *pa = &X(0, a, j), *pb = &X(0, b, j);
    unsigned *r = xq + (size_t)j * ldn;
    double *v = V + (size_t)j * ldn;
    const double xa = pa[0], xb = pb[0];
    const double ya = dim > 1 ? pa[1] : 0.0, yb = dim > 1 ? pb[1] : 0.0;
    const unsigned qa = r[a], qb = r[b];
    const double va = v[a], vb = v[b];
    pa[0] = xb;
    pb[0] = xa;
    if (dim > 1) {
      pa[1] = yb;
      pb[1] = ya;
    }
    r[a] = qb;
    r[b] = qa;
    v[a] = vb;
    v[b] = va;
    if (cl) cl->trade(a, b, j);
  }
};

// ---------------------------------------------------------------------------
// cell-list queries.  Every lane of the warp calls them; f(b, valid, sides)
// is called by every lane, 32 candidates at a time (valid: the lane holds
// candidate b; sides: bit 0 the query's first centre, bit 1 its second).
// ---------------------------------------------------------------------------
// the candidates of slice j in the periodic block of cells [x0, x0+nx) x
// [y0, y0+ny) (nx <= nc, ny <= min(nc, 4)), skipping moved entries, then the
// slice's moved particles
template <class F>
__device__ __forceinline__ void cell_block(const CellLists &L, int j, int x0, int nx, int y0, int ny,
                                           unsigned sides, int lane, F &&f) {
  const int *E = L.end + (size_t)j * (L.ncq + 1);
  // lane k < 2 ny holds segment k: row k/2, its columns up to the wrap
  // (part 0) and past it (part 1): first entry and length
  int st = 0, len = 0;
  if (lane < 2 * ny) {
    const int r = lane >> 1, part = lane & 1;
    int y = y0 + r;
    if (y >= L.nc) y -= L.nc;
    const int xe = x0 + nx - 1;
    int xa, xb;
    if (xe < L.nc) {
      xa = part ? 1 : x0;
      xb = part ? 0 : xe;
    } else {
      xa = part ? 0 : x0;
      xb = part ? xe - L.nc : L.nc - 1;
    }
    if (xa <= xb) {
      const int c0 = y * L.nc + xa, c1 = y * L.nc + xb;
      st = c0 ? E[c0 - 1] : 0;
      len = E[c1] - st;
    }
  }
  int incl = len;
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int S = __shfl_sync(0xffffffffu, incl, 7);
  const int excl = incl - len;
  const int D = L.dn[j];
  const unsigned short *items = L.items + (size_t)j * L.N, *dl = L.dl + (size_t)j * L.cap;
  for (int f0 = 0; f0 < S + D; f0 += 32) {
    const int fl = f0 + lane;
    // the segment of entry fl: the last one that starts at or before it
    int k = 0;
#pragma unroll
    for (int kk = 1; kk < 8; ++kk)
      if (fl >= __shfl_sync(0xffffffffu, excl, kk)) k = kk;
    const int sk = __shfl_sync(0xffffffffu, st, k), ek = __shfl_sync(0xffffffffu, excl, k);
    int b = -1;
    if (fl < S) {
      const unsigned it = items[sk + fl - ek];
      if (!(it & 0x8000u)) b = (int)it;
    } else if (fl < S + D) {
      b = (int)dl[fl - S];
    }
    f(b, b >= 0, sides);
  }
}

// the cell-list candidates of a query at slice j around the mirror words qa
// and qb (the old and the new position of a moving bead; qa == qb for one
// centre).  Centres in the same or in adjacent cells share one block of
// cells (sides 3 for every candidate); farther apart each has its own.
// use: L->usable(j), which callers read ahead of the query.  Returns false,
// having called nothing, when slice j has no usable lists.
template <class F>
__device__ __forceinline__ bool cell_query(const CellLists *L, bool use, int j, unsigned qa,
                                           unsigned qb, int lane, F &&f) {
  if (!L || !use) return false;
  const int nc = L->nc, h = nc >> 1;
  const int ax = L->cx(qa), ay = L->cy(qa), bx = L->cx(qb), by = L->cy(qb);
  int dx = bx - ax, dy = by - ay;
  if (dx > h) dx -= nc; else if (dx < -h) dx += nc;
  if (dy > h) dy -= nc; else if (dy < -h) dy += nc;
  const bool two = L->ncq != nc;
  auto wrap = [&](int v) { return v < 0 ? v + nc : (v >= nc ? v - nc : v); };
  const bool joint = abs(dx) <= 1 && abs(dy) <= 1;
  // one call site: the block is inlined once
  for (int k = 0; k < (joint ? 1 : 2); ++k) {
    int x0, nx, y0, ny;
    unsigned sides;
    if (joint) {
      x0 = wrap(min(ax, ax + dx) - 1);
      nx = 3 + abs(dx);
      y0 = two ? wrap(min(ay, ay + dy) - 1) : 0;
      ny = two ? 3 + abs(dy) : 1;
      sides = 3u;
    } else {
      x0 = wrap((k ? bx : ax) - 1);
      nx = 3;
      y0 = two ? wrap((k ? by : ay) - 1) : 0;
      ny = two ? 3 : 1;
      sides = k ? 2u : 1u;
    }
    cell_block(*L, j, x0, nx, y0, ny, sides, lane, f);
  }
  return true;
}

// ---------------------------------------------------------------------------
// action pieces (src/propagator.jl)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dist1(double a, double b, double L) {
  const double dx = fabs(a - b);
  const double o = (2.0 * L) - dx;
  return o < dx ? o : dx;
}

// teleport(x, L) = (x+L) - floor(x/2L + 1/2) 2L - L (src/propagator.jl:30-32).
// The quotient is formed by a multiplication; when it lands within 1e-9 of an
// integer the IEEE division of the reference is used instead, so the floor is
// always the reference's.
// Inside the box the floor is 0 and the result is (x + L) - L, the same bits
// as the full expression; that path skips the floor and its guard.
__device__ __forceinline__ double teleport(double x, double L, double inv2L) {
  if (fabs(x) < 0.999999 * L) return (x + L) - L;
  const double q = x * inv2L + 0.5;
  double f = floor(q);
  const double fr = q - f;
  if (fr < 1e-9 || fr > 1.0 - 1e-9) f = floor(x / (2.0 * L) + 0.5);
  return (x + L) - f * (2.0 * L) - L;
}

// teleport in the sweeps (SWEEP): a coordinate inside the box is kept as it
// is.  The reference's (x + L) - L can only round its last bits, which no
// statistic of a sweep sees, and skipping it spares two FP64 additions per
// coordinate on this part's narrow FP64 pipe.  Injected-draw attempts keep
// the reference's bits.
template <bool SWEEP>
__device__ __forceinline__ double teleport_s(double x, double L, double inv2L) {
  if (SWEEP && fabs(x) < L) return x;
  return teleport(x, L, inv2L);
}

__device__ __forceinline__ double sgn(double v) { return v > 0.0 ? 1.0 : (v < 0.0 ? -1.0 : 0.0); }

// engine-known external potential: hcoef |r|^2 + V0 sum sin^2(pi r_d / a)
// the optical lattice's normalized intensity (examples/tools/potentialtools.jl:1-16):
// with phi_k = 2 pi scale (x sin a_k + y cos a_k) (+ a_k when helical),
// S = (1/K) sum sin phi_k, C = (1/K) sum cos phi_k, I = S^2 + C^2; optionally
// the gradient of I
static __device__ __noinline__ double beam_intensity(const ChainDesc &d, double x, double y, double *gx,
                                              double *gy) {
  double S = 0.0, Cc = 0.0, sx = 0.0, sy = 0.0, cx = 0.0, cy = 0.0;
  for (int k = 0; k < d.nbeam; ++k) {
    const double sa = d.beam_sin[k], ca = d.beam_cos[k];
    double s, c;
    sincospi(2.0 * d.beam_scale * (x * sa + y * ca), &s, &c);
    if (d.beam_helical) {  // rotate by the beam's own angle a_k
      const double s2 = s * ca + c * sa, c2 = c * ca - s * sa;
      s = s2;
      c = c2;
    }
    S += s;
    Cc += c;
    // d(sin phi) = cos phi dphi, d(cos phi) = -sin phi dphi, dphi/dx = 2 pi scale sin a_k
    sx += c * sa;
    sy += c * ca;
    cx -= s * sa;
    cy -= s * ca;
  }
  const double inv = 1.0 / d.nbeam;
  S *= inv;
  Cc *= inv;
  if (gx) {
    const double w = 2.0 * 3.141592653589793 * d.beam_scale * inv;
    *gx = 2.0 * w * (S * sx + Cc * cx);
    *gy = 2.0 * w * (S * sy + Cc * cy);
  }
  return S * S + Cc * Cc;
}

__device__ __forceinline__ double vext(const ChainDesc &d, double x, double y) {
  double v = 0.0;
  if (d.flags & PF_BEAM) v += d.beam_depth * beam_intensity(d, x, y, nullptr, nullptr);
  if (d.flags & PF_HARM) {
    double s = x * x;
    if (d.dim > 1) s += y * y;
    v += d.hcoef * s;
  }
  if (d.flags & PF_LATT) {
    const double a = sinpi(x * d.lat_k);
    double s = a * a;
    if (d.dim > 1) {
      const double b = sinpi(y * d.lat_k);
      s += b * b;
    }
    v += d.V0 * s;
  }
  return v;
}

// gradient of vext along one coordinate, separable terms only
__device__ __forceinline__ double dvext(const ChainDesc &d, double x) {
  double g = 0.0;
  if (d.flags & PF_HARM) g += 2.0 * d.hcoef * x;
  if (d.flags & PF_LATT) g += d.V0 * (d.lat_k * 3.141592653589793) * sinpi(2.0 * x * d.lat_k);
  return g;
}

// full gradient of vext (the optical lattice is not separable)
__device__ __forceinline__ void grad_vext(const ChainDesc &d, double x, double y, double &gx,
                                          double &gy) {
  gx = dvext(d, x);
  gy = d.dim > 1 ? dvext(d, y) : 0.0;
  if (d.flags & PF_BEAM) {
    double bx, by;
    beam_intensity(d, x, y, &bx, &by);
    gx += d.beam_depth * bx;
    gy += d.beam_depth * by;
  }
}

// exp(x) for x <= 0 by a table of exp(-k/64), k = 0..2560 (filled from the
// host's libm at handle creation), times the degree-5 Taylor polynomial of
// exp(f) on |f| <= 1/128 (Tang's table-driven method, ACM TOMS 15, 1989):
// truncation <= (1/128)^6/720 = 3.2e-16 relative, about 9 FP64 operations
// against the library's longer range reduction and polynomial.  Arguments
// below -40 (pair terms of far-away next beads) go to the library exp.
constexpr int EXPTAB_N = 2560;
// one per kernel translation unit (static), both filled by the host
static __device__ double g_exptab[EXPTAB_N + 1];

__device__ __forceinline__ double exp_neg(double x) {
  if (!(x >= -40.0)) return exp(x);
  const int k = __double2int_rn(x * -64.0);
  const double f = fma((double)k, 0.015625, x);
  double p = fma(f, 1.0 / 120.0, 1.0 / 24.0);
  p = fma(p, f, 1.0 / 6.0);
  p = fma(p, f, 0.5);
  p = fma(p, f, 1.0);
  p = fma(p, f, 1.0);
  return __ldg(&g_exptab[k]) * p;
}

__device__ __forceinline__ double vpair(const ChainDesc &d, double r2) {
  return d.g * exp_neg(-r2 * d.inv2s2);
}

__device__ __forceinline__ double lnU2(const ChainDesc &d, double r2a, double r2b) {
  return -0.5 * d.tau * (vpair(d, r2a) + vpair(d, r2b));
}

// bridge coefficients alpha_t = (m-t)/(m+1-t), sigma_t = sqrt(2 lambda alpha tau)
// (src/updates/helper.jl:154,165); tabulated per chain with the same
// expression for m < wtab
__device__ __forceinline__ double2 bridge_coef(const CV &c, int m, int t) {
  if (m < c.d->wtab) return c.tab[m * c.d->wtab + t];
  const double a = (double)(m - t) / (double)(m + 1 - t);
  return make_double2(a, sqrt(2.0 * c.d->lambda * a * c.d->tau));
}

// the sweeps' closed form of the same bridge.  With q_t = p_t - e and
// a_t = (m-t)/(m+1-t), q_t = a_t q_(t-1) + sigma_t z_t becomes
// u_t = u_(t-1) + w_t z_t for u_t = q_t / (m-t), so
//   p_t = e + (m-t) (q_0/m + sum_(s<=t) w_s z_s),   w_t = sigma_t / (m-t):
// a prefix sum in place of the recursion (two FP64 operations a coordinate
// per bead, or a plain scan across lanes).  bridge_w(c, m, t) = (w_t, m-t)
// for t >= 1 and (1/m, m) for t = 0; tabulated per chain for m < wtab
__device__ __forceinline__ double2 bridge_w(const CV &c, int m, int t) {
  if (m < c.d->wtab) return c.tabw[m * c.d->wtab + t];
  if (t == 0) return make_double2(1.0 / m, (double)m);
  const double a = (double)(m - t) / (double)(m + 1 - t);
  return make_double2(sqrt(2.0 * c.d->lambda * a * c.d->tau) / (m - t), (double)(m - t));
}

// minimum-image difference a - b: the same magnitude as dist1 (|a-b| when it
// is at most L, else 2L - |a-b|, both exactly rounded), with one subtraction
// and a rarely taken wrap
__device__ __forceinline__ double mi1(double a, double b, double L, double L2) {
  double dx = a - b;
  if (fabs(dx) > L) dx -= copysign(L2, dx);
  return dx;
}

__device__ __forceinline__ double mi2(const ChainDesc &d, double ax, double ay, double bx,
                                      double by) {
  const double dx = mi1(ax, bx, d.L, d.L2);
  double s = dx * dx;
  if (d.dim > 1) {
    const double dy = mi1(ay, by, d.L, d.L2);
    s = fma(dy, dy, s);
  }
  return s;
}

// grid position of a radius in the contact table: cell i and weight of
// cell i + 1 of the linear B-spline (Interpolations.jl's scaled linear
// interpolation: (x - first)/step, the last cell for x at the end).  Radii
// outside [r0, rmax] are clamped, where the reference raises a BoundsError.
__device__ __forceinline__ int contact_cell(const ChainDesc &d, double r, double &w) {
  r = fmin(fmax(r, d.ct_r0), d.ct_rmax);
  const double p = (r - d.ct_r0) / d.ct_h;
  double f = floor(p);
  if (f > (double)(d.ct_n - 2)) f = (double)(d.ct_n - 2);
  w = p - f;
  return (int)f;
}

// the pair link action of the tabulated contact propagator between two
// particles whose minimum-image differences are d1 (slice j) and d2 (slice
// j+1): prop_int = 1 + T(|d1|, |d2|) / prop_rel0(d1, d2, tau) with
// prop_rel0 = exp(-|d1 - d2|^2 / (4 tau)) / (4 pi tau), and lnU = log(prop_int),
// or -mu where prop_int < 0 (src/propagator.jl:74-89, src/system.jl:26-28).
// The reference passes per-component absolute differences (distance.(),
// src/propagator.jl:6-9), so its |d1 - d2| is taken between the absolute
// vectors; the physical rules use the signed differences, their own
// difference wrapped to the minimum image.  Products and sums are rounded
// separately as in the reference (no fused multiply-add).
__device__ __forceinline__ double contact_lnU(const ChainDesc &d, double d1x, double d1y,
                                              double d2x, double d2y) {
  const double ax = fabs(d1x), ay = fabs(d1y), bx = fabs(d2x), by = fabs(d2y);
  const double n1 = __dsqrt_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)));
  const double n2 = __dsqrt_rn(__dadd_rn(__dmul_rn(bx, bx), __dmul_rn(by, by)));
  double ex, ey;
  if (d.flags & PF_PHYS) {
    ex = mi1(d1x, d2x, d.L, d.L2);
    ey = mi1(d1y, d2y, d.L, d.L2);
  } else {
    ex = ax - bx;
    ey = ay - by;
  }
  double wx, wy;
  const int ix = contact_cell(d, n1, wx), iy = contact_cell(d, n2, wy);
  const int n = d.ct_n;
  const double *r0 = d.ct_tab + (size_t)ix * n + iy, *r1 = r0 + n;
  const double c0 = __dadd_rn(__dmul_rn(1.0 - wy, __ldg(r0)), __dmul_rn(wy, __ldg(r0 + 1)));
  const double c1 = __dadd_rn(__dmul_rn(1.0 - wy, __ldg(r1)), __dmul_rn(wy, __ldg(r1 + 1)));
  const double T = __dadd_rn(__dmul_rn(1.0 - wx, c0), __dmul_rn(wx, c1));
  const double dd = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
  const double rel0 = exp(-dd / (4.0 * d.tau)) / (12.566370614359172 * d.tau);
  const double p = 1.0 + T / rel0;
  return p < 0.0 ? -d.mu : log(p);
}

// contact_lnU from the four beads of a link pair (a, b at slice j; an, bn at
// slice j+1), kept out of line: the Gaussian pair path does not carry its code
static __device__ __noinline__ double contact_link(const ChainDesc &d, double ax, double ay, double bx,
                                            double by, double anx, double any, double bnx,
                                            double bny) {
  const bool two = d.dim > 1;
  return contact_lnU(d, mi1(ax, bx, d.L, d.L2), two ? mi1(ay, by, d.L, d.L2) : 0.0,
                     mi1(anx, bnx, d.L, d.L2), two ? mi1(any, bny, d.L, d.L2) : 0.0);
}

// ---------------------------------------------------------------------------
// neighbour scans over one slice
// ---------------------------------------------------------------------------
// neighbour prefilter on the mirror: every bead within R (exact FP64
// minimum-image distance) of the centre passes; lim is the chain's bound for
// R (q_lim_rc or q_lim_hard)
struct Prefilter {
  unsigned c, lim;
  __device__ __forceinline__ void init(const ChainDesc &d, double px, double py, unsigned lim_) {
    c = qpos(d, px, py);
    lim = lim_;
  }
  __device__ __forceinline__ void init_q(unsigned centre, unsigned lim_) {
    c = centre;
    lim = lim_;
  }
  __device__ __forceinline__ bool pass(unsigned p) const { return qdist2(c, p) <= lim; }
};

// ---------------------------------------------------------------------------
// pair terms of a moving path segment, old and new configurations, with
// every lane busy.  A segment is a list of links t: bead t at slice(t) and
// the next bead along the path (at slice(t)+1).  Pass 1: lanes test the
// particles of the slice against the old and the new bead in FP32 and push
// the survivors (b, t, side) onto a warp-private queue in shared memory
// (ballot + popc).  Pass 2: whenever 32 entries are queued, each lane takes
// one and evaluates it exactly in FP64.  The warp's divergent FP64 work is
// then proportional to the neighbours found, not to the particles scanned.
//
// Seg provides: slice(t), cur(side, t, &x, &y), nxt(side, t, &x, &y),
// curq(side, t) (the bead's mirror word), skip(side, t, b).  side 0 = old
// configuration, 1 = new.
// ---------------------------------------------------------------------------
constexpr int PQ_CAP = 96;  // queue entries per warp (64-bit)

// one queued entry: the link's two pair exponentials exp(-r^2/2s^2) at its
// ends, added to the lane's old (so) or new (sn) sum; the caller applies the
// link weight -tau g / 2 once per segment.  With the contact table the entry
// is the link's pair action itself (weight 1).
// CT = false: the chains this code runs for have no contact table (a
// specialised kernel), so its branch is compiled out
template <bool CT = true, class Seg>
__device__ __forceinline__ void pq_eval(const CV &c, const Seg &s, unsigned long long e,
                                        double &so, double &sn) {
  const ChainDesc &d = *c.d;
  const int M = c.M;
  const int b = (int)(e >> 32), t = (int)((e >> 1) & 0x7fffffffu), side = (int)(e & 1u);
  const int j = s.slice(t), jn = j + 1 == M ? 0 : j + 1;
  double ax, ay, anx, any;
  s.cur(side, t, ax, ay);
  const double bx = c.X(0, b, j), by = c.Xd(1, b, j);
  const double r2a = mi2(d, ax, ay, bx, by);
  if (r2a > d.rc2) return;
  s.nxt(side, t, anx, any);
  const int bn = j == M - 1 ? c.next[b] : b;
  const double bnx = c.X(0, bn, jn), bny = c.Xd(1, bn, jn);
  double v;
  if (CT && (d.flags & PF_CONTACT)) {
    v = contact_link(d, ax, ay, bx, by, anx, any, bnx, bny);
  } else {
    const double r2b = mi2(d, anx, any, bnx, bny);
    v = exp_neg(-r2a * d.inv2s2) + exp_neg(-r2b * d.inv2s2);
  }
  if (side) sn += v; else so += v;
}

// evaluate the first min(qn, 32) queued entries and move the rest up
template <bool CT = true, class Seg>
__device__ __forceinline__ void pq_flush(const CV &c, const Seg &s, unsigned long long *q, int &qn,
                                         double &wo, double &wn, int lane) {
  const int k = qn < 32 ? qn : 32;
  if (lane < k) pq_eval<CT>(c, s, q[lane], wo, wn);
  __syncwarp();
  unsigned long long rest[3];
  const int nr = qn - k;
  for (int r = 0; r < 3; ++r) {
    const int i = 32 + lane + 32 * r;
    rest[r] = (lane + 32 * r < nr) ? q[i] : 0ull;
  }
  __syncwarp();
  for (int r = 0; r < 3; ++r)
    if (lane + 32 * r < nr) q[lane + 32 * r] = rest[r];
  __syncwarp();
  qn = nr;
}

// the lane's sums of the links' pair exponentials, old and new configuration
template <bool CT = true, class Seg>
__device__ void segment_sums(const CV &c, const Seg &s, int t0, int t1, bool do_old, bool do_new,
                             unsigned long long *q, double &wo, double &wn, int lane) {
  const ChainDesc &d = *c.d;
  const int N = c.N, dim = c.dim;
  const unsigned lt = (1u << lane) - 1u;
  int qn = 0;
  const CellLists *L = c.cl;
  bool use_next = L && t0 < t1 && L->usable(s.slice(t0));
  for (int t = t0; t < t1; ++t) {
    const bool use = use_next;
    if (L && t + 1 < t1) use_next = L->usable(s.slice(t + 1));
    const int j = s.slice(t);
    const unsigned co = s.curq(0, t), cn = s.curq(1, t);
    Prefilter fo, fn;
    fo.init_q(co, d.q_lim_rc);
    fn.init_q(cn, d.q_lim_rc);
    const unsigned *row = c.xq + (size_t)j * c.ldn;
    // every lane calls push with its candidate's outcome, old and new side
    auto push = [&](int b, bool po, bool pn) {
      const unsigned mo = __ballot_sync(0xffffffffu, po), mn = __ballot_sync(0xffffffffu, pn);
      const unsigned long long base = ((unsigned long long)(unsigned)b << 32) | ((unsigned)t << 1);
      if (po) {
        const int k = qn + __popc(mo & lt);
        if (check_ok(k < PQ_CAP, DERR_QUEUE, d)) q[k] = base;
      }
      qn += __popc(mo);
      if (pn) {
        const int k = qn + __popc(mn & lt);
        if (check_ok(k < PQ_CAP, DERR_QUEUE, d)) q[k] = base | 1ull;
      }
      qn += __popc(mn);
#if PIMC_CHECK
      if (qn > PQ_CAP) qn = PQ_CAP;
#endif
      __syncwarp();
      // a block of 32 candidates queues up to 64 entries (old and new):
      // drain to fewer than 32 before the next block, so that the queue
      // holds at most 31 + 64 = 95 < PQ_CAP entries at any time
      while (qn >= 32) pq_flush<CT>(c, s, q, qn, wo, wn, lane);
    };
    const bool listed = cell_query(L, use, j, co, cn, lane, [&](int b, bool v, unsigned sides) {
      bool po = false, pn = false;
      if (v) {
        const unsigned pb = row[b];
        po = (sides & 1u) && do_old && fo.pass(pb) && !s.skip(0, t, b);
        pn = (sides & 2u) && do_new && fn.pass(pb) && !s.skip(1, t, b);
      }
      push(b, po, pn);
    });
    if (listed) continue;
    for (int b0 = 0; b0 < N; b0 += 32) {
      const int b = b0 + lane;
      bool po = false, pn = false;
      if (b < N) {
        const unsigned pb = row[b];
        po = do_old && fo.pass(pb) && !s.skip(0, t, b);
        pn = do_new && fn.pass(pb) && !s.skip(1, t, b);
      }
      push(b, po, pn);
    }
  }
  while (qn > 0) pq_flush<CT>(c, s, q, qn, wo, wn, lane);
}

// adds the links' pair terms -tau/2 (v(r_a) + v(r_b)) of the old (wo) and the
// new (wn) configuration; every lane of the warp calls it
template <bool CT = true, class Seg>
__device__ void segment_pairs(const CV &c, const Seg &s, int t0, int t1, bool do_old, bool do_new,
                              unsigned long long *q, double &wo, double &wn, int lane) {
  double so = 0.0, sn = 0.0;
  segment_sums<CT>(c, s, t0, t1, do_old, do_new, q, so, sn, lane);
  if (CT && (c.d->flags & PF_CONTACT)) {
    wo += so;
    wn += sn;
  } else {
    wo = fma(c.d->mhtau_g, so, wo);
    wn = fma(c.d->mhtau_g, sn, wn);
  }
}

// ---------------------------------------------------------------------------
// bounded estimate of a segment's pair sums, from the mirror alone.  For
// every link it gives the lane's sum of exp(-r_a^2/2s^2) + exp(-r_b^2/2s^2)
// over the neighbours within rc, old (so) and new (sn) configuration, and a
// bound (bo, bn) on its distance from the exact FP64 sum: a mirror distance
// is within kQErr units of the exact one, __expf is within (3 + 1.2 y) ulp
// (CUDA's documented 2 + floor(1.16 |y|)), and a pair whose mirror distance
// cannot settle the cut-off contributes the midpoint of [0, its value].
// Only the decision of a move is taken from it, and only when the whole
// interval lies on one side of the Metropolis threshold.
// ---------------------------------------------------------------------------
constexpr float kQErr = 3.f;

struct PairEst {
  float so, bo, sn, bn;  // sums and bounds, old and new configuration
  int ko, kn;            // terms added (for the FP32 accumulation error)
};

// squared mirror distance, and whether an axis lies within 4 units of the
// half box, where the exact minimum image may fold the other way
__device__ __forceinline__ unsigned qdist2_w(unsigned a, unsigned b, bool &edge) {
  const unsigned dd = __vsub2(a, b);
  const int dx = ((int)(dd << 16)) >> 16, dy = ((int)dd) >> 16;
  edge = abs(dx) > 32763 || abs(dy) > 32763;
  return (unsigned)(dx * dx) + (unsigned)(dy * dy);
}

// The relative error of a term exp(-y) whose end lies at squared mirror
// distance d2 is at most  c1 (2 sqrt(d2) + kQErr) + (3 + 1.2 y) 1.2e-7 :
// the argument error from the mirror (c1 = 1.01 u^2/(2 sigma^2) kQErr, the
// 1.01 covering FP32 rounding) plus __expf's own.  The bound grows with d2,
// so for the first end, which the callers take within q_lim_hi, the value at
// q_lim_hi (eps_a) bounds every term.  For the second end, which may lie
// anywhere, 2 sqrt(d2) <= d2 / s + s for any s > 0 (s = sqrt(q_lim_hi),
// tight where it matters); past q_lim_hi the looser bound only touches
// terms exp(-y) below exp(-y_hi).  Neither needs a square root per term.
struct EstConst {
  float c1, inv_s, s, eps_a;
  __device__ __forceinline__ explicit EstConst(const ChainDesc &d) {
    c1 = 1.01f * d.q_u2i * kQErr;
    const float lim = (float)d.q_lim_hi;
    s = sqrtf(lim);
    inv_s = 1.f / s;
    eps_a = c1 * (2.f * s + kQErr) + (3.f + 1.2f * (lim * d.q_u2i)) * 1.2e-7f;
  }
};

__device__ __forceinline__ void est_term(const ChainDesc &d, const EstConst &K, unsigned d2a,
                                         unsigned d2b, bool edge_b, float &sum, float &bnd, int &k) {
  const float ya = (float)d2a * d.q_u2i, yb = (float)d2b * d.q_u2i;
  const float ea = __expf(-ya), eb = __expf(-yb);
  // relative error of each exponential (EstConst)
  const float da = K.eps_a;
  const float db = fmaf(K.c1, fmaf((float)d2b, K.inv_s, K.s + kQErr), (3.f + 1.2f * yb) * 1.2e-7f);
  // an end next to the half box: anything in [0, 1]
  const float vb = edge_b ? 0.5f : eb, eb_err = edge_b ? 0.5f : eb * db;
  const float v = ea + vb, err = ea * da + eb_err + 2e-30f;
  if (d2a < d.q_lim_lo) {
    sum += v;
    bnd += err;
  } else {
    // the exact cut-off may keep or drop the link: [0, v + err]
    sum += 0.5f * v;
    bnd += 0.5f * v + err;
  }
  ++k;
}

// no early stop
struct NoStop {
  __device__ __forceinline__ bool operator()(const PairEst &) const { return false; }
};

// stop(e), called by the whole warp after every link, ends the scan early;
// returns whether it did
template <class Seg, class Stop = NoStop>
__device__ bool segment_estimate(const CV &c, const Seg &s, int t0, int t1, PairEst &e, int lane,
                                 const Stop &stop = Stop()) {
  const ChainDesc &d = *c.d;
  const int N = c.N, M = c.M;
  const EstConst K(d);
  // whether a slice's lists are usable is read one link ahead
  const CellLists *L = c.cl;
  bool use_next = L && t0 < t1 && L->usable(s.slice(t0));
  for (int t = t0; t < t1; ++t) {
    const bool use = use_next;
    if (L && t + 1 < t1) use_next = L->usable(s.slice(t + 1));
    const int j = s.slice(t), jn = j + 1 == M ? 0 : j + 1;
    const bool wrap = j == M - 1;
    const unsigned co = s.curq(0, t), cn = s.curq(1, t);
    const unsigned no = s.nxtq(0, t), nn = s.nxtq(1, t);
    const unsigned *row = c.xq + (size_t)j * c.ldn, *rown = c.xq + (size_t)jn * c.ldn;
    // one candidate b: its mirror words at slices j (pb) and j+1 (pbn)
    auto cand = [&](int b, unsigned pb, unsigned pbn) {
      const unsigned d2o = qdist2(co, pb), d2n = qdist2(cn, pb);
      const bool io = d2o <= d.q_lim_hi && !s.skip(0, t, b);
      const bool in = d2n <= d.q_lim_hi && !s.skip(1, t, b);
      bool edge;
      if (io) {
        const unsigned d2b = qdist2_w(no, pbn, edge);
        est_term(d, K, d2o, d2b, edge, e.so, e.bo, e.ko);
      }
      if (in) {
        const unsigned d2b = qdist2_w(nn, pbn, edge);
        est_term(d, K, d2n, d2b, edge, e.sn, e.bn, e.kn);
      }
    };
    // a cell-list candidate: the sides its block serves, the word at slice
    // j+1 read only for a pair that passes
    const bool listed = cell_query(L, use, j, co, cn, lane, [&](int b, bool v, unsigned sides) {
      if (!v) return;
      const unsigned pb = row[b];
      const unsigned d2o = qdist2(co, pb), d2n = qdist2(cn, pb);
      const bool io = (sides & 1u) && d2o <= d.q_lim_hi && !s.skip(0, t, b);
      const bool in = (sides & 2u) && d2n <= d.q_lim_hi && !s.skip(1, t, b);
      if (!io && !in) return;
      const unsigned pbn = rown[wrap ? c.next[b] : b];
      bool edge;
      if (io) {
        const unsigned d2b = qdist2_w(no, pbn, edge);
        est_term(d, K, d2o, d2b, edge, e.so, e.bo, e.ko);
      }
      if (in) {
        const unsigned d2b = qdist2_w(nn, pbn, edge);
        est_term(d, K, d2n, d2b, edge, e.sn, e.bn, e.kn);
      }
    });
    if (listed) {
    } else if (!wrap) {
      // the words at both slices are read together, two blocks of 32
      // candidates at a time, so that one round trip to memory serves four
      // loads (the latency, not the bytes, bounds this scan); the lane's
      // candidates are visited in the same order as one block at a time
      for (int b0 = lane; b0 < N; b0 += 64) {
        const int b1 = b0 + 32;
        const unsigned pa0 = row[b0], pn0 = rown[b0];
        const unsigned pa1 = b1 < N ? row[b1] : 0u, pn1 = b1 < N ? rown[b1] : 0u;
        cand(b0, pa0, pn0);
        if (b1 < N) cand(b1, pa1, pn1);
      }
    } else {
      // past slice M the partner's next bead belongs to next[b]
      for (int b = lane; b < N; b += 32) {
        const unsigned pb = row[b];
        const unsigned d2o = qdist2(co, pb), d2n = qdist2(cn, pb);
        const bool io = d2o <= d.q_lim_hi && !s.skip(0, t, b);
        const bool in = d2n <= d.q_lim_hi && !s.skip(1, t, b);
        if (io || in) cand(b, pb, rown[c.next[b]]);
      }
    }
    if (stop(e)) return true;
  }
  return false;
}

// a lane's estimates in FP64, with the error of its FP32 accumulation (two
// ulp per addition of non-negative terms, on the sum and on the bound) added
// to the bounds; the caller sums them over the group
__device__ __forceinline__ void est_reduce_lanes(const PairEst &e, double (&v)[4]) {
  const double ro = 2.4e-7 * (e.ko + 1), rn = 2.4e-7 * (e.kn + 1);
  v[0] = (double)e.so;
  v[1] = (double)e.bo * (1.0 + ro) + ro * (double)e.so + 1e-30;
  v[2] = (double)e.sn;
  v[3] = (double)e.bn * (1.0 + rn) + rn * (double)e.sn + 1e-30;
}

// log u in FP32 (logf within a few ulp, u a 53-bit uniform in (0, 1)) and
// a margin that covers its error
__device__ __forceinline__ double log_u_margin(double u, double &margin) {
  const double lu = (double)logf((float)u);
  margin = 1e-5 * (1.0 + fabs(lu));
  return lu;
}

// the Metropolis decision from an interval [lo, hi] of the log acceptance
// ratio: 1 accept, 0 reject, -1 undecided.  Decided only where exp(dS) > u
// (accept) or exp(dS) < u < 1 (reject) holds for every dS in the interval,
// so the outcome is the FP64 formula's for the exact dS.
__device__ __forceinline__ int decide_interval(double lo, double hi, double u) {
  if (u <= 0.0) return lo > -700.0 ? 1 : -1;
  double margin;
  const double lu = log_u_margin(u, margin);
  margin += 1e-9 * (fabs(lo) + fabs(hi));
  if (lo > lu + margin) return 1;
  if (hi < lu - margin) return 0;
  return -1;
}

// Metropolis acceptance of a log ratio dS (helper.jl:3-5: delta >= 1 ||
// delta > rand()).  A sweep's uniform is a pure function of the move's
// stream, so away from the threshold the comparison runs in FP32 log space
// and the FP64 exponential settles only the rest; the outcome is the FP64
// formula's.  Injected draws keep the reference's order: the uniform is read
// only when delta < 1.
template <class D>
__device__ __forceinline__ bool metropolis(const ChainDesc &d, double dS, D &dr) {
  if (D::kSweep && !(d.flags & PF_EXACT)) {
    const double u = dr.uniform_accept();
    const int k = decide_interval(dS, dS, u);
    if (k >= 0) return k == 1;
    const double delta = exp(dS);
    return delta >= 1.0 || delta > u;
  }
  const double delta = exp(dS);
  return (delta >= 1.0) || (delta > dr.uniform_accept());
}

// a staging window: bead t at absolute slice j0+t of particle n (next(n)
// past slice M); new beads in shared arrays; the moving path is excluded
struct WindowSeg {
  const CV *c;
  int n, nx, j0, M;
  const double *px, *py;
  const unsigned *pq;   // mirror words of the new beads
  __device__ __forceinline__ int own(int t) const { return j0 + t < M ? n : nx; }
  __device__ __forceinline__ unsigned curq(int side, int t) const {
    return side ? pq[t] : c->Q(own(t), slice(t));
  }
  __device__ __forceinline__ unsigned nxtq(int side, int t) const { return curq(side, t + 1); }
  __device__ __forceinline__ int slice(int t) const { return j0 + t < M ? j0 + t : j0 + t - M; }
  __device__ __forceinline__ void cur(int side, int t, double &x, double &y) const {
    if (side) { x = px[t]; y = py[t]; }
    else { x = c->X(0, own(t), slice(t)); y = c->Xd(1, own(t), slice(t)); }
  }
  __device__ __forceinline__ void nxt(int side, int t, double &x, double &y) const {
    cur(side, t + 1, x, y);
  }
  __device__ __forceinline__ bool skip(int, int t, int b) const { return b == own(t); }
};

// any bead other than e1/e2 at slice j closer than the hard-core radius
// (find_nn + distance < a, src/updates/helper.jl:167-169); per-lane result
__device__ __forceinline__ bool hard_hit_lanes(const CV &c, double x, double y, int j, int e1,
                                               int e2, int lane, int lanes) {
  const ChainDesc &d = *c.d;
  const int N = c.N, dim = c.dim;
  const double a2 = d.hard_a * d.hard_a;
  Prefilter f;
  f.init(d, x, y, d.q_lim_hard);
  const unsigned *row = c.xq + (size_t)j * c.ldn;
  bool hit = false;
  // the cell lists serve whole warps only
  if (lanes == 32 && cell_query(c.cl, c.cl && c.cl->usable(j), j, f.c, f.c, lane, [&](int b, bool v, unsigned) {
        if (!v || hit || b == e1 || b == e2 || !f.pass(row[b])) return;
        if (mi2(d, x, y, c.X(0, b, j), c.Xd(1, b, j)) < a2) hit = true;
      }))
    return hit;
  for (int b = lane; b < N && !hit; b += lanes) {
    if (b == e1 || b == e2 || !f.pass(row[b])) continue;
    if (mi2(d, x, y, c.X(0, b, j), c.Xd(1, b, j)) < a2) hit = true;
  }
  return hit;
}

// ---------------------------------------------------------------------------
// warp helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ---------------------------------------------------------------------------
// Levy staging window, one thread (pair-free acceptance, no hard core)
// ReshapeLinear (src/updates/reshape.jl:31-91) with hardspherelevy! for a = 0
// ---------------------------------------------------------------------------
template <class D>
__device__ int window_thread(const CV &c, int n, int j0, int m, D &dr, bool rewrite_start,
                             double *prop) {
  const ChainDesc &d = *c.d;
  if (!check_ok(m >= 2 && m <= TWMAX && m < c.M && j0 >= 0 && j0 < c.M, DERR_WINDOW, d) ||
      !check_ok(n >= 0 && n < c.N, DERR_INDEX, d))
    return RES_REJECT;
  const int M = c.M, dim = c.dim;
  const double L = d.L, inv2L = d.inv2L, mhtau = -0.5 * d.tau;
  const int nx = c.next[n];
  const int jend = j0 + m;
  const int oe = jend < M ? n : nx, je = jend < M ? jend : jend - M;
  double bx[TWMAX + 1], by[TWMAX + 1], vp[TWMAX];
  const double sx = c.X(0, n, j0), sy = c.Xd(1, n, j0);
  double ex = c.X(0, oe, je), ey = c.Xd(1, oe, je);
  if (fabs(sx - ex) > L) ex += sgn(sx) * (2.0 * L);
  if (dim > 1 && fabs(sy - ey) > L) ey += sgn(sy) * (2.0 * L);
  double px = sx, py = sy;
  bx[0] = sx;
  by[0] = sy;
  // sweeps take the bridge's closed form (bridge_w); attempts keep the
  // reference's recursion a p' + (1 - a) e + z sigma and its bits
  const double inv_m = D::kSweep ? bridge_w(c, m, 0).x : 0.0;
  double ux = (sx - ex) * inv_m, uy = (sy - ey) * inv_m;
  for (int t = 1; t < m; ++t) {
    double z[2];
    dr.bead_normals(t - 1, dim, z);
    if (D::kSweep) {
      const double2 wk = bridge_w(c, m, t);
      ux = fma(z[0], wk.x, ux);
      bx[t] = fma(wk.y, ux, ex);
      if (dim > 1) {
        uy = fma(z[1], wk.x, uy);
        by[t] = fma(wk.y, uy, ey);
      }
    } else {
      const double2 ab = bridge_coef(c, m, t);
      px = ab.x * px + (1.0 - ab.x) * ex + z[0] * ab.y;
      bx[t] = px;
      if (dim > 1) {
        py = ab.x * py + (1.0 - ab.x) * ey + z[1] * ab.y;
        by[t] = py;
      }
    }
  }
  dr.consumed((m - 1) * dim);
  bx[m] = ex;
  by[m] = ey;
  double wi = 0.0, wu = 0.0, vprev = 0.0;
  for (int t = 0; t <= m; ++t) {
    bx[t] = teleport_s<D::kSweep>(bx[t], L, inv2L);
    if (dim > 1) by[t] = teleport_s<D::kSweep>(by[t], L, inv2L);
    const double vb = vext(d, bx[t], by[t]);
    // sweeps keep the links' sums and scale once (the write-back scales each)
    if (t > 0) vp[t - 1] = D::kSweep ? vprev + vb : mhtau * (vprev + vb);
    vprev = vb;
  }
  for (int t = 0; t < m; ++t) {
    const int a = j0 + t;
    wi += c.Vl(a < M ? n : nx, a < M ? a : a - M);
  }
  for (int t = 0; t < m; ++t) wu += vp[t];
  if (D::kSweep) wu *= mhtau;
  if (prop)
    for (int t = 0; t <= m; ++t) {
      prop[t * dim] = bx[t];
      if (dim > 1) prop[t * dim + 1] = by[t];
    }
  const bool acc = metropolis(d, wu - wi, dr);
  if (acc) {
    for (int t = 0; t < m; ++t) {
      const int a = j0 + t;
      const int o = a < M ? n : nx, j = a < M ? a : a - M;
      if (t > 0 || rewrite_start) c.set_pos(o, j, bx[t], by[t]);
      c.Vl(o, j) = D::kSweep ? mhtau * vp[t] : vp[t];
    }
  }
  return acc ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Levy staging window, one warp: pair terms (physical semantics) and the
// hard-core retry loop.  sb: per-warp shared scratch of 5*(WMAX+1) doubles
// followed by a PQ_CAP-entry neighbour queue.
// ---------------------------------------------------------------------------
template <class D>
__device__ int window_warp(const CV &c, int n, int j0, int m, D &dr, bool rewrite_start,
                           double *sb, double *prop) {
  const ChainDesc &d = *c.d;
  if (!check_ok(m >= 2 && m <= WMAX && m < c.M && j0 >= 0 && j0 < c.M, DERR_WINDOW, d) ||
      !check_ok(n >= 0 && n < c.N, DERR_INDEX, d))
    return RES_REJECT;
  const int lane = threadIdx.x & 31;
  const int M = c.M, dim = c.dim;
  const double L = d.L, inv2L = d.inv2L, mhtau = -0.5 * d.tau;
  const bool phys_pair = (d.flags & PF_PAIR) && (d.flags & PF_PHYS);
  const bool hard = (d.flags & PF_HARD) != 0;
  double *sx_ = sb, *sy_ = sb + (WMAX + 1), *svb = sb + 2 * (WMAX + 1);
  double *sz = sb + 3 * (WMAX + 1);  // 2*(WMAX+1): normals
  unsigned *sq = (unsigned *)(sb + 5 * (WMAX + 1) + 96);
  const int nx = c.next[n];
  const int jend = j0 + m;
  const int oe = jend < M ? n : nx, je = jend < M ? jend : jend - M;
  const double sx = c.X(0, n, j0), sy = c.Xd(1, n, j0);
  double ex = c.X(0, oe, je), ey = c.Xd(1, oe, je);
  if (fabs(sx - ex) > L) ex += sgn(sx) * (2.0 * L);
  if (dim > 1 && fabs(sy - ey) > L) ey += sgn(sy) * (2.0 * L);
  int fail = 0;
  if (!hard) {
    for (int t = 1 + lane; t < m; t += 32) {
      double z[2];
      dr.bead_normals(t - 1, dim, z);
      sz[2 * t] = z[0];
      sz[2 * t + 1] = dim > 1 ? z[1] : 0.0;
    }
    dr.consumed((m - 1) * dim);
    __syncwarp();
    if (lane < dim) {
      double p = lane == 0 ? sx : sy;
      const double e = lane == 0 ? ex : ey;
      double *dst = lane == 0 ? sx_ : sy_;
      for (int t = 1; t < m; ++t) {
        const double2 ab = bridge_coef(c, m, t);
        p = ab.x * p + (1.0 - ab.x) * e + sz[2 * t + lane] * ab.y;
        dst[t] = p;
      }
    }
  } else {
    // sequential retries in the reference's draw order (lane 0 draws, the warp
    // scans the slice); the reference excludes the start particle (fpcycle of
    // the wrapped slice) in its find_nn, the physical semantics the true owner
    double px = sx, py = sy;
    for (int t = 1; t < m && !fail; ++t) {
      const double2 ab = bridge_coef(c, m, t);
      const int a = j0 + t, j = a < M ? a : a - M;
      const int exc = (d.flags & PF_PHYS) ? (a < M ? n : nx) : n;
      int tries = 0;
      while (true) {
        if (++tries > d.ctr) { fail = 1; break; }
        double qx = 0.0, qy = 0.0;
        if (lane == 0) {
          const double z0 = dr.normal(), z1 = dim > 1 ? dr.normal() : 0.0;
          qx = ab.x * px + (1.0 - ab.x) * ex + z0 * ab.y;
          qy = dim > 1 ? ab.x * py + (1.0 - ab.x) * ey + z1 * ab.y : 0.0;
        }
        qx = __shfl_sync(0xffffffffu, qx, 0);
        qy = __shfl_sync(0xffffffffu, qy, 0);
        const double tx = teleport_s<D::kSweep>(qx, L, inv2L);
        const double ty = dim > 1 ? teleport_s<D::kSweep>(qy, L, inv2L) : 0.0;
        const bool hit = __any_sync(0xffffffffu, hard_hit_lanes(c, tx, ty, j, exc, -1, lane, 32));
        if (!hit) { px = qx; py = qy; break; }
      }
      if (lane == 0) {
        sx_[t] = px;
        sy_[t] = py;
      }
    }
  }
  __syncwarp();
  if (fail) return RES_HARDCORE;
  for (int t = lane; t <= m; t += 32) {
    double qx = t == 0 ? sx : (t == m ? ex : sx_[t]);
    double qy = t == 0 ? sy : (t == m ? ey : sy_[t]);
    qx = teleport_s<D::kSweep>(qx, L, inv2L);
    if (dim > 1) qy = teleport_s<D::kSweep>(qy, L, inv2L);
    sx_[t] = qx;
    sy_[t] = qy;
    svb[t] = vext(d, qx, qy);
    if (phys_pair) sq[t] = qpos(d, qx, qy);
  }
  __syncwarp();
  double wi = 0.0, wu = 0.0;
  for (int t = lane; t < m; t += 32) {
    const int a = j0 + t;
    wi += c.Vl(a < M ? n : nx, a < M ? a : a - M);
    wu += mhtau * (svb[t] + svb[t + 1]);
  }
  int dec = -1;
  if (phys_pair) {
    WindowSeg seg{&c, n, nx, j0, M, sx_, sy_, sq};
    if (D::kSweep && !(d.flags & (PF_EXACT | PF_CONTACT))) {
      // bounded estimate from the mirror; the exact sums only when its
      // interval straddles the Metropolis threshold
      PairEst e = {0.f, 0.f, 0.f, 0.f, 0, 0};
      segment_estimate(c, seg, 0, m, e, lane);
      double v[4];
      est_reduce_lanes(e, v);
      for (int k = 0; k < 4; ++k) v[k] = warp_sum(v[k]);
      const double h = d.mhtau_g;
      const double centre = warp_sum(wu) - warp_sum(wi) + h * (v[2] - v[0]);
      const double radius = fabs(h) * (v[1] + v[3]);
      dec = decide_interval(centre - radius, centre + radius, dr.uniform_accept());
    }
    if (dec == -1)
      segment_pairs(c, seg, 0, m, true, true, (unsigned long long *)(sb + 5 * (WMAX + 1)), wi, wu,
                    lane);
  }
  wi = warp_sum(wi);
  wu = warp_sum(wu);
  if (prop)
    for (int t = lane; t <= m; t += 32) {
      prop[t * dim] = sx_[t];
      if (dim > 1) prop[t * dim + 1] = sy_[t];
    }
  int acc = dec;
  if (dec == -1) {
    if (lane == 0) acc = metropolis(d, wu - wi, dr);
    acc = __shfl_sync(0xffffffffu, acc, 0);
  }
  if (acc) {
    for (int t = lane; t < m; t += 32) {
      const int a = j0 + t;
      const int o = a < M ? n : nx, j = a < M ? a : a - M;
      if (t > 0 || rewrite_start) c.set_pos(o, j, sx_[t], sy_[t]);
      c.Vl(o, j) = mhtau * (svb[t] + svb[t + 1]);
    }
  }
  __syncwarp();
  return acc;
}

// ---------------------------------------------------------------------------
// a staging window by a team of warps (pair action, no hard core): the warps
// of the team split the window's links for the pair scans, each with its own
// neighbour queue; the first warp draws the bridge and decides.  Warp w of
// the team has the scratch tb + w * tstride (the first warp's holds the
// window).  Every thread of the team calls it; the team synchronises on
// named barrier `bar`.
// ---------------------------------------------------------------------------
constexpr int kMaxTeams = 7;  // named barriers 1..7 (barrier 0 is the CTA's)
struct Team {
  int w, nw, bar;  // warp in the team, warps in the team, barrier 1..kMaxTeams
  __device__ __forceinline__ void sync() const {
    // immediate barrier ids, so that a CTA reserves kMaxTeams + 1 barriers
    // (not all 16), which keeps CTAs per SM from being limited by barriers
    const int cnt = nw * 32;
    switch (bar) {
      case 1: asm volatile("bar.sync 1, %0;" ::"r"(cnt) : "memory"); break;
      case 2: asm volatile("bar.sync 2, %0;" ::"r"(cnt) : "memory"); break;
      case 3: asm volatile("bar.sync 3, %0;" ::"r"(cnt) : "memory"); break;
      case 4: asm volatile("bar.sync 4, %0;" ::"r"(cnt) : "memory"); break;
      case 5: asm volatile("bar.sync 5, %0;" ::"r"(cnt) : "memory"); break;
      case 6: asm volatile("bar.sync 6, %0;" ::"r"(cnt) : "memory"); break;
      default: asm volatile("bar.sync 7, %0;" ::"r"(cnt) : "memory"); break;
    }
  }
};

template <class D>
__device__ int window_team(const CV &c, const Team &tm, int n, int j0, int m, D &dr, double *tb,
                           int tstride) {
  auto sb = [&](int w) { return tb + (size_t)w * tstride; };
  const ChainDesc &d = *c.d;
  const int lane = threadIdx.x & 31, tid = tm.w * 32 + lane, nt = tm.nw * 32;
  const int M = c.M, dim = c.dim;
  const double L = d.L, inv2L = d.inv2L, mhtau = -0.5 * d.tau;
  double *b0 = sb(0);
  double *sx_ = b0, *sy_ = b0 + (WMAX + 1), *svb = b0 + 2 * (WMAX + 1);
  double *sz = b0 + 3 * (WMAX + 1);
  unsigned *sq = (unsigned *)(b0 + 5 * (WMAX + 1) + 96);
  const int nx = c.next[n];
  const int jend = j0 + m;
  const int oe = jend < M ? n : nx, je = jend < M ? jend : jend - M;
  const double sx = c.X(0, n, j0), sy = c.Xd(1, n, j0);
  double ex = c.X(0, oe, je), ey = c.Xd(1, oe, je);
  if (fabs(sx - ex) > L) ex += sgn(sx) * (2.0 * L);
  if (dim > 1 && fabs(sy - ey) > L) ey += sgn(sy) * (2.0 * L);
  for (int t = 1 + tid; t < m; t += nt) {
    double z[2];
    dr.bead_normals(t - 1, dim, z);
    sz[2 * t] = z[0];
    sz[2 * t + 1] = dim > 1 ? z[1] : 0.0;
  }
  tm.sync();
  if (tm.w == 0 && lane < dim) {
    double p = lane == 0 ? sx : sy;
    const double e = lane == 0 ? ex : ey;
    double *dst = lane == 0 ? sx_ : sy_;
    for (int t = 1; t < m; ++t) {
      const double2 ab = bridge_coef(c, m, t);
      p = ab.x * p + (1.0 - ab.x) * e + sz[2 * t + lane] * ab.y;
      dst[t] = p;
    }
  }
  tm.sync();
  for (int t = tid; t <= m; t += nt) {
    double qx = t == 0 ? sx : (t == m ? ex : sx_[t]);
    double qy = t == 0 ? sy : (t == m ? ey : sy_[t]);
    qx = teleport_s<D::kSweep>(qx, L, inv2L);
    if (dim > 1) qy = teleport_s<D::kSweep>(qy, L, inv2L);
    sx_[t] = qx;
    sy_[t] = qy;
    svb[t] = vext(d, qx, qy);
    sq[t] = qpos(d, qx, qy);
  }
  tm.sync();
  double wi = 0.0, wu = 0.0;
  for (int t = tid; t < m; t += nt) {
    const int a = j0 + t;
    wi += c.Vl(a < M ? n : nx, a < M ? a : a - M);
    wu += mhtau * (svb[t] + svb[t + 1]);
  }
  {
    const int per = (m + tm.nw - 1) / tm.nw;
    const int t0 = min(m, tm.w * per), t1 = min(m, t0 + per);
    if (t0 < t1) {
      WindowSeg seg{&c, n, nx, j0, M, sx_, sy_, sq};
      segment_pairs(c, seg, t0, t1, true, true, (unsigned long long *)(sb(tm.w) + 5 * (WMAX + 1)),
                    wi, wu, lane);
    }
  }
  wi = warp_sum(wi);
  wu = warp_sum(wu);
  double *slot = sb(tm.w) + TEAM_SLOT_D;
  if (lane == 0) {
    slot[0] = wi;
    slot[1] = wu;
  }
  tm.sync();
  double *lead = b0 + TEAM_SLOT_D;
  if (tid == 0) {
    double si = 0.0, su = 0.0;
    for (int w = 0; w < tm.nw; ++w) {
      si += sb(w)[TEAM_SLOT_D];
      su += sb(w)[TEAM_SLOT_D + 1];
    }
    lead[2] = metropolis(d, su - si, dr) ? 1.0 : 0.0;
  }
  tm.sync();
  const int acc = lead[2] != 0.0;
  if (acc) {
    for (int t = 1 + tid; t < m; t += nt) {
      const int a = j0 + t;
      c.set_pos(a < M ? n : nx, a < M ? a : a - M, sx_[t], sy_[t]);
    }
    for (int t = tid; t < m; t += nt) {
      const int a = j0 + t;
      c.Vl(a < M ? n : nx, a < M ? a : a - M) = mhtau * (svb[t] + svb[t + 1]);
    }
  }
  tm.sync();
  return acc;
}

}  // namespace pimc
