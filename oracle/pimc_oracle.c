/*
 * pimc_oracle.c -- CPU oracle (test infrastructure only) for the PIMC sweep.
 *
 * A plain-C restatement of oameye/PIMC.jl's Monte Carlo sweep.  Each function
 * cites the reference file:line it follows.  Two acceptance semantics:
 *   ORC_SEM_REFERENCE  bug-compatible with the reference:
 *     - interaction_action! is a no-op in staging and CoM moves
 *       (src/updates/helper.jl:306-366 rebinds a by-value Float64);
 *     - the swap adds the NEW paths' pair terms to w_initial
 *       (src/updates/reshape.jl:224,239) and double counts the old
 *       path1-path2 pair (166-199);
 *     - the swap applies no partner-selection normalisation ratio;
 *     - the swap leaves the cached link action of link j_m stale when the
 *       window does not wrap (tail swap starts at j_m+1, reshape.jl:269-275).
 *   ORC_SEM_PHYSICAL   the same action, applied consistently: pair terms in
 *     every move, the cross term between the two swapped paths, the
 *     heat-bath normalisation ratio, and the j_m link moved with the tail.
 * Nothing here is used by the product library.
 */
#include "pimc_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define XI(st, d, n, j) ((size_t)(d) * (size_t)(st)->p.N * (size_t)(st)->p.M + (size_t)(n) * (size_t)(st)->p.M + (size_t)(j))
#define VI(st, n, j) ((size_t)(n) * (size_t)(st)->p.M + (size_t)(j))
#define MAXDIM 2

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), restated from the paper */
/* ------------------------------------------------------------------------ */
void orc_philox4x32_10(const uint32_t c_in[4], const uint32_t k_in[2], uint32_t out[4]) {
  uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3];
  uint32_t k0 = k_in[0], k1 = k_in[1];
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void orc_rng_init(orc_rng *r, uint64_t seed, uint64_t stream) {
  r->key[0] = (uint32_t)seed; r->key[1] = (uint32_t)(seed >> 32);
  r->ctr[0] = 0; r->ctr[1] = 0; r->ctr[2] = (uint32_t)stream; r->ctr[3] = (uint32_t)(stream >> 32);
  r->pos = 4; r->have_spare = 0; r->spare = 0.0;
}

static uint32_t rng_u32(orc_rng *r) {
  if (r->pos >= 4) {
    orc_philox4x32_10(r->ctr, r->key, r->buf);
    if (++r->ctr[0] == 0) ++r->ctr[1];
    r->pos = 0;
  }
  return r->buf[r->pos++];
}

double orc_rng_uniform(orc_rng *r) {
  uint64_t a = rng_u32(r), b = rng_u32(r);
  uint64_t x = ((a << 32) | b) >> 11;
  return (double)x * 0x1.0p-53;
}

double orc_rng_normal(orc_rng *r) {
  if (r->have_spare) { r->have_spare = 0; return r->spare; }
  double u1 = 1.0 - orc_rng_uniform(r); /* (0,1] */
  double u2 = orc_rng_uniform(r);
  double rad = sqrt(-2.0 * log(u1));
  double th = 6.283185307179586476925 * u2;
  r->spare = rad * sin(th); r->have_spare = 1;
  return rad * cos(th);
}

static double draw_normal(orc_draws *dr) {
  if (dr->rng) return orc_rng_normal(dr->rng);
  if (dr->normal_pos >= dr->n_normals) { dr->exhausted = 1; return 0.0; }
  return dr->normals[dr->normal_pos++];
}
static double draw_uniform(orc_draws *dr) {
  if (dr->rng) return orc_rng_uniform(dr->rng);
  if (dr->uniform_pos >= dr->n_uniforms) { dr->exhausted = 1; return 0.5; }
  return dr->uniforms[dr->uniform_pos++];
}

/* ------------------------------------------------------------------------ */
/* action pieces: src/propagator.jl                                          */
/* ------------------------------------------------------------------------ */
/* src/propagator.jl:6-9 */
double orc_distance(double x1, double x2, double L) {
  double dx = fabs(x1 - x2);
  double o = (2.0 * L) - dx;
  return o < dx ? o : dx;
}
/* src/propagator.jl:30-32 */
double orc_teleport(double x, double L) {
  return (x + L) - floor(x / (2.0 * L) + 0.5) * (2.0 * L) - L;
}
/* src/propagator.jl:16-19, called through the System closure with lambda and
 * tau in swapped positions (src/system.jl:163): denominator (4 tau) lambda */
double orc_lnK(const orc_params *p, const double *r1, const double *r2, double tau_eff) {
  double s = 0.0;
  for (int d = 0; d < p->dim; ++d) { double q = orc_distance(r1[d], r2[d], p->L); s += q * q; }
  return -s / (4.0 * tau_eff * p->lambda);
}
/* normalized_intensity (examples/tools/potentialtools.jl:1-16): plane waves
 * of every beam, r_k = x sin(a) + y cos(a), sin/cos of 2 pi r_k scale (+ a when
 * helical), their means squared and added; optionally the gradient */
static double beam_intensity(const orc_params *p, const double *r, double *grad) {
  double s = 0.0, c = 0.0, sx = 0.0, sy = 0.0, cx = 0.0, cy = 0.0;
  for (int k = 0; k < p->nbeam; ++k) {
    double a = p->beam_angle[k], sa = sin(a), ca = cos(a);
    double rk = r[0] * sa + r[1] * ca;
    double ph = p->beam_helical ? 2.0 * 3.141592653589793 * rk * p->beam_scale + a
                                : 2.0 * 3.141592653589793 * rk * p->beam_scale;
    double sp = sin(ph), cp = cos(ph);
    s += sp;
    c += cp;
    sx += cp * sa; sy += cp * ca;
    cx -= sp * sa; cy -= sp * ca;
  }
  s /= p->nbeam;
  c /= p->nbeam;
  if (grad) {
    double w = 2.0 * 3.141592653589793 * p->beam_scale / p->nbeam;
    grad[0] = 2.0 * w * (s * sx + c * cx);
    grad[1] = 2.0 * w * (s * sy + c * cy);
  }
  return s * s + c * c;
}

/* engine-known potentials: Harmonic (hcoef = omega^2/2) + SquareLattice +
 * optical lattice */
double orc_Vext(const orc_params *p, const double *r) {
  double v = 0.0;
  if (p->nbeam > 0 && p->beam_depth != 0.0) v += p->beam_depth * beam_intensity(p, r, NULL);
  if (p->hcoef != 0.0) {
    double s = 0.0;
    for (int d = 0; d < p->dim; ++d) s += r[d] * r[d];
    v += p->hcoef * s;
  }
  if (p->V0 != 0.0) {
    double s = 0.0;
    for (int d = 0; d < p->dim; ++d) { double q = sin(p->lat_k * r[d]); s += q * q; }
    v += p->V0 * s;
  }
  return v;
}
static void orc_dVext(const orc_params *p, const double *r, double *g) {
  for (int d = 0; d < p->dim; ++d) {
    double q = 0.0;
    if (p->hcoef != 0.0) q += 2.0 * p->hcoef * r[d];
    if (p->V0 != 0.0) q += p->V0 * p->lat_k * sin(2.0 * p->lat_k * r[d]);
    g[d] = q;
  }
  if (p->nbeam > 0 && p->beam_depth != 0.0) {
    double bg[2];
    beam_intensity(p, r, bg);
    g[0] += p->beam_depth * bg[0];
    g[1] += p->beam_depth * bg[1];
  }
}
/* src/propagator.jl:26-28 */
double orc_lnV(const orc_params *p, const double *r1, const double *r2) {
  return -0.5 * p->tau * (orc_Vext(p, r1) + orc_Vext(p, r2));
}
static double vpair_r2(const orc_params *p, double r2) { return p->g * exp(-r2 * p->inv2s2); }
/* src/system.jl:26-28 with the Gaussian pair propagator
 * propint(r1,r2,tau) = exp(-tau/2 (v(|r1|)+v(|r2|))), so log(propint) is the
 * primitive pair link action; d1, d2 are per-component min-image distances */
static double contact_lnU(const orc_params *p, const double *d1, const double *d2);
double orc_lnU(const orc_params *p, const double *d1, const double *d2) {
  if (p->ct_tab) return contact_lnU(p, d1, d2);
  double a = 0.0, b = 0.0;
  for (int d = 0; d < p->dim; ++d) { a += d1[d] * d1[d]; b += d2[d] * d2[d]; }
  return -0.5 * p->tau * (vpair_r2(p, a) + vpair_r2(p, b));
}

/* Linear B-spline of the table scaled onto the grid (Interpolations.jl's
 * scale(interpolate(A, BSpline(Linear())), r, r), src/propagator.jl:68-70):
 * position (x - first)/step, the last cell for x at the end.  The reference
 * raises a BoundsError outside [1e-20, range]; the engine clamps. */
static int contact_cell(const orc_params *p, double r, double *w) {
  const double r0 = 1e-20, h = (p->ct_range - r0) / (double)(p->ct_n - 1);
  if (r < r0) r = r0;
  if (r > p->ct_range) r = p->ct_range;
  double pos = (r - r0) / h, f = floor(pos);
  if (f > (double)(p->ct_n - 2)) f = (double)(p->ct_n - 2);
  *w = pos - f;
  return (int)f;
}
static double contact_T(const orc_params *p, double r1, double r2) {
  double wx, wy;
  int ix = contact_cell(p, r1, &wx), iy = contact_cell(p, r2, &wy), n = p->ct_n;
  const double *a = p->ct_tab + (size_t)ix * n + iy, *b = a + n;
  double c0 = (1.0 - wy) * a[0] + wy * a[1];
  double c1 = (1.0 - wy) * b[0] + wy * b[1];
  return (1.0 - wx) * c0 + wx * c1;
}
/* minimum-image wrap of a difference of two minimum-image vectors */
static double wrap1(double x, double L) {
  if (fabs(x) > L) x -= (x > 0 ? 2.0 * L : -2.0 * L);
  return x;
}
/* lnU = log(prop_int) or -mu when prop_int < 0 (src/system.jl:26-28) with
 * prop_int(r1, r2) = 1 + T(|r1|, |r2|) / prop_rel0(r1, r2, tau),
 * prop_rel0 = exp(-|r1 - r2|^2 / (4 tau)) / (4 pi tau) (propagator.jl:74-89).
 * d1, d2 are signed minimum-image differences; the reference passes their
 * per-component absolute values (distance.()), the physical rules the signed
 * vectors with their difference wrapped. */
static double contact_lnU(const orc_params *p, const double *d1, const double *d2) {
  double n1 = 0.0, n2 = 0.0, dd = 0.0;
  for (int d = 0; d < p->dim; ++d) {
    double a = fabs(d1[d]), b = fabs(d2[d]);
    n1 += a * a;
    n2 += b * b;
    double e = p->semantics == ORC_SEM_PHYSICAL ? wrap1(d1[d] - d2[d], p->L) : a - b;
    dd += e * e;
  }
  double T = contact_T(p, sqrt(n1), sqrt(n2));
  double rel0 = exp(-dd / (4.0 * p->tau)) / (4.0 * 3.141592653589793 * p->tau);
  double pi = 1.0 + T / rel0;
  return pi < 0.0 ? -p->mu : log(pi);
}

/* ------------------------------------------------------------------------ */
/* cell grid: src/nearest_neighbours.jl                                      */
/* ------------------------------------------------------------------------ */
/* src/nearest_neighbours.jl:26-33, clamped to the grid (a bead rounded onto
 * +L would index past the grid in the reference) */
static int cell_of(const orc_params *p, const double *r) {
  double w = 2.0 * p->L / p->nbins;
  int c = 0, mul = 1;
  for (int d = 0; d < p->dim; ++d) {
    int i = (int)floor((r[d] + p->L) / w);
    if (i < 0) i = 0;
    if (i >= p->nbins) i = p->nbins - 1;
    c += i * mul; mul *= p->nbins;
  }
  return c;
}
static int use_cells(const orc_state *st) { return st->p.interactions || st->p.hardcore_a > 0.0; }

static void bead_pos(const orc_state *st, int n, int j, double *r) {
  for (int d = 0; d < st->p.dim; ++d) r[d] = st->x[XI(st, d, n, j)];
}
static void cell_unlink(orc_state *st, int n, int j) {
  int M = st->p.M, N = st->p.N;
  int c = st->bins[VI(st, n, j)];
  int *nx = st->cell_nxt + (size_t)j * N, *pv = st->cell_prv + (size_t)j * N;
  if (pv[n] >= 0) nx[pv[n]] = nx[n]; else st->cell_head[(size_t)j * st->ncell + c] = nx[n];
  if (nx[n] >= 0) pv[nx[n]] = pv[n];
  nx[n] = pv[n] = -1;
  (void)M;
}
static void cell_link(orc_state *st, int n, int j, int c) {
  int N = st->p.N;
  int *nx = st->cell_nxt + (size_t)j * N, *pv = st->cell_prv + (size_t)j * N;
  int *h = st->cell_head + (size_t)j * st->ncell + c;
  nx[n] = *h; pv[n] = -1;
  if (*h >= 0) pv[*h] = n;
  *h = n;
  st->bins[VI(st, n, j)] = c;
}
/* update_nn_bead! (src/nearest_neighbours.jl:198-209) */
static void cell_refresh(orc_state *st, int n, int j) {
  if (!use_cells(st)) return;
  double r[MAXDIM]; bead_pos(st, n, j, r);
  int c = cell_of(&st->p, r);
  if (c == st->bins[VI(st, n, j)]) return;
  cell_unlink(st, n, j); cell_link(st, n, j, c);
}
static void cells_rebuild(orc_state *st) {
  if (!use_cells(st)) return;
  int N = st->p.N, M = st->p.M;
  for (size_t i = 0; i < (size_t)M * st->ncell; ++i) st->cell_head[i] = -1;
  for (int j = 0; j < M; ++j)
    for (int n = N - 1; n >= 0; --n) {
      double r[MAXDIM]; bead_pos(st, n, j, r);
      cell_link(st, n, j, cell_of(&st->p, r));
    }
}
/* 3x3 (or 3) stencil of src/nearest_neighbours.jl:55-65; duplicates removed */
static int stencil(const orc_params *p, int c, int *out) {
  int nb = p->nbins, k = 0;
  if (p->dim == 1) {
    int cand[3] = {c, (c - 1 + nb) % nb, (c + 1) % nb};
    for (int i = 0; i < 3; ++i) {
      int dup = 0;
      for (int q = 0; q < k; ++q) dup |= out[q] == cand[i];
      if (!dup) out[k++] = cand[i];
    }
    return k;
  }
  int x = c % nb, y = c / nb;
  static const int dx[9] = {0, -1, 0, 1, -1, 1, -1, 0, 1};
  static const int dy[9] = {0, 1, 1, 1, 0, 0, -1, -1, -1};
  for (int i = 0; i < 9; ++i) {
    int cc = ((x + dx[i] + nb) % nb) + nb * ((y + dy[i] + nb) % nb);
    int dup = 0;
    for (int q = 0; q < k; ++q) dup |= out[q] == cc;
    if (!dup) out[k++] = cc;
  }
  return k;
}

/* squared minimum-image distance; dv (optional) receives the signed
 * minimum-image difference a - b, of magnitude distance(a, b) */
static double mi_dist2(const orc_params *p, const double *a, const double *b, double *dv) {
  double s = 0.0;
  for (int d = 0; d < p->dim; ++d) {
    double q = orc_distance(a[d], b[d], p->L);
    if (dv) {
      double x = a[d] - b[d];
      dv[d] = (fabs(x) > p->L) == (x > 0) ? -q : q;
    }
    s += q * q;
  }
  return s;
}

/* sum over neighbours b (not excluded) of the bead at position `a` on slice j
 * with min-image distance <= rc: lnU(d(a, b_j), d(an, b_next)), where an is
 * the next bead along the moving path.  This is the body of
 * interaction_action! / the swap's pair loops (src/updates/helper.jl:306-347,
 * src/updates/reshape.jl:166-240) with the neighbour set of find_nns
 * (src/nearest_neighbours.jl:131-154: 3x3 stencil, inrange <= 2L/nbins). */
static double pair_link(const orc_state *st, const double *a, const double *an, int j,
                        int e1, int e2) {
  const orc_params *p = &st->p;
  int N = p->N, M = p->M;
  int cells[9];
  int nc = stencil(p, cell_of(p, a), cells);
  double rc2 = p->rc * p->rc, w = 0.0;
  for (int ci = 0; ci < nc; ++ci) {
    for (int b = st->cell_head[(size_t)j * st->ncell + cells[ci]]; b >= 0;
         b = st->cell_nxt[(size_t)j * N + b]) {
      if (b == e1 || b == e2) continue;
      double rb[MAXDIM], d1[MAXDIM], d2[MAXDIM], rbn[MAXDIM];
      bead_pos(st, b, j, rb);
      if (mi_dist2(p, a, rb, d1) > rc2) continue;
      int bn = (j == M - 1) ? st->next[b] : b;
      bead_pos(st, bn, (j + 1) % M, rbn);
      mi_dist2(p, an, rbn, d2);
      w += orc_lnU(p, d1, d2);
    }
  }
  return w;
}
/* cross pair term between two moving paths at one link */
static double pair_cross(const orc_params *p, const double *a, const double *an,
                         const double *b, const double *bn) {
  double d1[MAXDIM], d2[MAXDIM];
  if (mi_dist2(p, a, b, d1) > p->rc * p->rc) return 0.0;
  mi_dist2(p, an, bn, d2);
  return orc_lnU(p, d1, d2);
}

/* hard-core test of find_nn + distance < a (src/updates/helper.jl:167-169) */
static int hardcore_hit(const orc_state *st, const double *r, int j, int e1, int e2) {
  const orc_params *p = &st->p;
  if (p->hardcore_a <= 0.0) return 0;
  double a2 = p->hardcore_a * p->hardcore_a;
  int cells[9];
  int nc = stencil(p, cell_of(p, r), cells);
  for (int ci = 0; ci < nc; ++ci)
    for (int b = st->cell_head[(size_t)j * st->ncell + cells[ci]]; b >= 0;
         b = st->cell_nxt[(size_t)j * st->p.N + b]) {
      if (b == e1 || b == e2) continue;
      double rb[MAXDIM]; bead_pos(st, b, j, rb);
      if (mi_dist2(p, r, rb, NULL) < a2) return 1;
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* state                                                                     */
/* ------------------------------------------------------------------------ */
void orc_params_init(orc_params *p, int dim, int N, int M, double L, double T, double lambda) {
  memset(p, 0, sizeof(*p));
  p->dim = dim; p->N = N; p->M = M; p->L = L;
  p->beta = 1.0 / T; p->tau = p->beta / M; p->lambda = lambda;
  p->nbins = (int)floor((2.0 * L) / (L / 4.0)); /* r_a = L/4 when unset (src/system.jl:18-24) */
  p->rc = 2.0 * L / p->nbins;
  p->ctr = 10000;
  p->semantics = ORC_SEM_REFERENCE;
}

orc_state *orc_create(const orc_params *p) {
  if (p->dim < 1 || p->dim > 2 || p->N < 1 || p->M < 3 || p->nbins < 1) return NULL;
  orc_state *st = (orc_state *)calloc(1, sizeof(orc_state));
  st->p = *p;
  int N = p->N, M = p->M;
  st->x = (double *)calloc((size_t)p->dim * N * M, sizeof(double));
  st->V = (double *)calloc((size_t)N * M, sizeof(double));
  st->next = (int *)malloc(sizeof(int) * N);
  for (int n = 0; n < N; ++n) st->next[n] = n;
  st->ncell = p->dim == 2 ? p->nbins * p->nbins : p->nbins;
  st->cell_head = (int *)malloc(sizeof(int) * (size_t)M * st->ncell);
  st->cell_nxt = (int *)malloc(sizeof(int) * (size_t)M * N);
  st->cell_prv = (int *)malloc(sizeof(int) * (size_t)M * N);
  st->bins = (int *)malloc(sizeof(int) * (size_t)N * M);
  st->scratch_len = (long)(8 * (M + 2) * MAXDIM + 8 * (M + 2) + 4 * (size_t)N + 64);
  st->scratch = (double *)malloc(sizeof(double) * st->scratch_len);
  return st;
}

void orc_destroy(orc_state *st) {
  if (!st) return;
  free(st->x); free(st->V); free(st->next); free(st->cell_head); free(st->cell_nxt);
  free(st->cell_prv); free(st->bins); free(st->scratch); free(st);
}

static void recompute_V(orc_state *st) {
  int N = st->p.N, M = st->p.M;
  for (int n = 0; n < N; ++n)
    for (int j = 0; j < M; ++j) {
      double a[MAXDIM], b[MAXDIM];
      bead_pos(st, n, j, a);
      bead_pos(st, j == M - 1 ? st->next[n] : n, (j + 1) % M, b);
      st->V[VI(st, n, j)] = orc_lnV(&st->p, a, b);
    }
}

int orc_set_state(orc_state *st, const double *x, const int *next) {
  size_t nx = (size_t)st->p.dim * st->p.N * st->p.M;
  memcpy(st->x, x, nx * sizeof(double));
  if (next) memcpy(st->next, next, sizeof(int) * st->p.N);
  recompute_V(st);
  cells_rebuild(st);
  return 0;
}

int orc_set_raw(orc_state *st, const double *x, const double *V, const int *next) {
  size_t nx = (size_t)st->p.dim * st->p.N * st->p.M;
  memcpy(st->x, x, nx * sizeof(double));
  memcpy(st->V, V, sizeof(double) * (size_t)st->p.N * st->p.M);
  memcpy(st->next, next, sizeof(int) * st->p.N);
  cells_rebuild(st);
  return 0;
}

void orc_get_state(const orc_state *st, double *x, double *V, int *next) {
  if (x) memcpy(x, st->x, sizeof(double) * (size_t)st->p.dim * st->p.N * st->p.M);
  if (V) memcpy(V, st->V, sizeof(double) * (size_t)st->p.N * st->p.M);
  if (next) memcpy(next, st->next, sizeof(int) * st->p.N);
}

/* levy! (src/updates/helper.jl:118-139) on a full closed row r[M][dim] */
static void levy_rows(orc_state *st, double *r, int rows, orc_draws *dr) {
  const orc_params *p = &st->p;
  int dim = p->dim;
  double *e = r + (size_t)(rows - 1) * dim;
  for (int d = 0; d < dim; ++d)
    if (fabs(r[d] - e[d]) > p->L) e[d] += (r[d] > 0 ? 1.0 : (r[d] < 0 ? -1.0 : 0.0)) * (2.0 * p->L);
  int mm = rows - 2;
  for (int j = 1; j <= mm; ++j) {
    double alpha = (double)(mm + 1 - j) / (double)(mm + 2 - j);
    double sig = sqrt(2.0 * p->lambda * alpha * p->tau);
    double z[MAXDIM];
    for (int d = 0; d < dim; ++d) z[d] = draw_normal(dr);
    for (int d = 0; d < dim; ++d)
      r[(size_t)j * dim + d] = alpha * r[(size_t)(j - 1) * dim + d] + (1.0 - alpha) * e[d] + z[d] * sig;
  }
  for (int i = 0; i < rows * dim; ++i) r[i] = orc_teleport(r[i], p->L);
}

/* any bead of the new path r (M rows) closer than the hard-core radius to a
 * bead of particles 0..n-1 at the same slice (system.jl:54-62: norm of the
 * per-component minimum-image distances, strictly below a) */
static int init_overlap(const orc_state *st, const double *r, int n) {
  const orc_params *p = &st->p;
  int M = p->M, dim = p->dim;
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int d = 0; d < dim; ++d) {
        double dd = orc_distance(st->x[XI(st, d, i, j)], r[(size_t)j * dim + d], p->L);
        s += dd * dd;
      }
      if (sqrt(s) < p->hardcore_a) return 1;
    }
  return 0;
}

/* init_world (src/system.jl:36-78): per particle a uniform start, the last
 * row equal to the first, a Levy loop through the rows between; with a hard
 * core, particle n > 0 is drawn again (start and loop) while one of its beads
 * overlaps a bead of an earlier particle at the same slice, at most 10000
 * times, after which the world cannot be made (ORC_ESTATE; the reference
 * logs an error and returns an empty world) */
int orc_init_world(orc_state *st, orc_draws *dr) {
  const orc_params *p = &st->p;
  int N = p->N, M = p->M, dim = p->dim;
  double *r = (double *)malloc(sizeof(double) * (size_t)M * dim);
  int rc = 0;
  for (int n = 0; n < N && rc == 0; ++n) {
    int tries = 0;
    while (1) {
      if (++tries > 10000) { rc = ORC_ESTATE; break; }
      for (int d = 0; d < dim; ++d) r[d] = 2.0 * p->L * (draw_uniform(dr) - 0.5);
      for (int d = 0; d < dim; ++d) r[(size_t)(M - 1) * dim + d] = r[d];
      levy_rows(st, r, M, dr);
      if (!(p->hardcore_a > 0.0) || n == 0 || !init_overlap(st, r, n)) break;
    }
    if (rc) break;
    for (int j = 0; j < M; ++j)
      for (int d = 0; d < dim; ++d) st->x[XI(st, d, n, j)] = r[(size_t)j * dim + d];
    st->next[n] = n;
  }
  free(r);
  if (rc) return rc;
  recompute_V(st);
  cells_rebuild(st);
  return dr->exhausted ? ORC_EDRAWS : 0;
}

/* ------------------------------------------------------------------------ */
/* Levy bridge with hard-core retry: hardspherelevy! (helper.jl:141-222)     */
/* rp holds m+1 beads (bead-major); exclusions per bead via own arrays       */
/* ------------------------------------------------------------------------ */
static int bridge(orc_state *st, double *rp, int m, int j0, const int *exc1, const int *exc2,
                  orc_draws *dr) {
  const orc_params *p = &st->p;
  int dim = p->dim, M = p->M;
  double L = p->L;
  double *e = rp + (size_t)m * dim;
  for (int d = 0; d < dim; ++d)
    if (fabs(rp[d] - e[d]) > L) e[d] += (rp[d] > 0 ? 1.0 : (rp[d] < 0 ? -1.0 : 0.0)) * (2.0 * L);
  int mm = m - 1;
  for (int j = 1; j <= mm; ++j) {
    double alpha = (double)(mm + 1 - j) / (double)(mm + 2 - j);
    double sig = sqrt(2.0 * p->lambda * alpha * p->tau);
    int tries = 0, bad = 1;
    while (bad) {
      bad = 0;
      if (++tries > p->ctr) return ORC_HARDCORE;
      double z[MAXDIM];
      for (int d = 0; d < dim; ++d) z[d] = draw_normal(dr);
      for (int d = 0; d < dim; ++d)
        rp[(size_t)j * dim + d] = alpha * rp[(size_t)(j - 1) * dim + d] + (1.0 - alpha) * e[d] + z[d] * sig;
      if (p->hardcore_a > 0.0) {
        double tp[MAXDIM];
        for (int d = 0; d < dim; ++d) tp[d] = orc_teleport(rp[(size_t)j * dim + d], L);
        if (hardcore_hit(st, tp, (j0 + j) % M, exc1[j], exc2 ? exc2[j] : -1)) bad = 1;
      }
    }
  }
  for (int i = 0; i < (m + 1) * dim; ++i) rp[i] = orc_teleport(rp[i], L);
  return ORC_ACCEPT;
}

static int metropolis(double delta, orc_draws *dr) {
  /* src/updates/helper.jl:3-5: a uniform is drawn only when delta < 1 */
  if (delta >= 1.0) return 1;
  return delta > draw_uniform(dr);
}

/* ------------------------------------------------------------------------ */
/* ReshapeLinear (src/updates/reshape.jl:31-91)                              */
/* ------------------------------------------------------------------------ */
static inline int own_of(const orc_state *st, int n, int j0, int t) {
  return (j0 + t < st->p.M) ? n : st->next[n];
}

static void staging_w(orc_state *st, int n, int j0, int m, const double *rp, const int *own,
                      double *Vp, double *w_init, double *w_upd) {
  const orc_params *p = &st->p;
  int dim = p->dim, M = p->M;
  double wi = 0.0, wu = 0.0;
  for (int t = 0; t < m; ++t) {
    int j = (j0 + t) % M;
    wi += st->V[VI(st, own[t], j)];
    Vp[t] = orc_lnV(p, rp + (size_t)t * dim, rp + (size_t)(t + 1) * dim);
  }
  for (int t = 0; t < m; ++t) wu += Vp[t];
  if (p->interactions && p->semantics == ORC_SEM_PHYSICAL) {
    for (int t = 0; t < m; ++t) {
      int j = (j0 + t) % M;
      double a[MAXDIM], an[MAXDIM];
      bead_pos(st, own[t], j, a);
      bead_pos(st, own[t + 1], (j + 1) % M, an);
      wi += pair_link(st, a, an, j, own[t], -1);
      wu += pair_link(st, rp + (size_t)t * dim, rp + (size_t)(t + 1) * dim, j, own[t], -1);
    }
  }
  (void)n;
  *w_init = wi; *w_upd = wu;
}

void orc_staging_weights(orc_state *st, int n, int j0, int m, const double *rp, double *w_init,
                         double *w_upd) {
  int own[2 * 4096 + 2];
  double *Vp = st->scratch;
  for (int t = 0; t <= m; ++t) own[t] = own_of(st, n, j0, t);
  staging_w(st, n, j0, m, rp, own, Vp, w_init, w_upd);
}

int orc_staging(orc_state *st, int n, int j0, int m, orc_draws *dr, double *rp_out) {
  const orc_params *p = &st->p;
  int dim = p->dim, M = p->M;
  if (n < 0 || n >= p->N || j0 < 0 || j0 >= M || m < 2 || m > M - 1) return ORC_EARG;
  double *rp = st->scratch;                    /* (m+1)*dim */
  double *Vp = rp + (size_t)(M + 2) * MAXDIM;  /* m */
  int own[4096 + 2], exc[4096 + 2];
  if (m + 1 > 4096) return ORC_EARG;
  for (int t = 0; t <= m; ++t) {
    own[t] = own_of(st, n, j0, t);
    /* the reference excludes fpcycle(mod1(j0+j, M)), i.e. always the start
     * particle (helper.jl:167); the physical mode excludes the true owner */
    exc[t] = p->semantics == ORC_SEM_REFERENCE ? n : own[t];
  }
  for (int d = 0; d < dim; ++d) {
    rp[d] = st->x[XI(st, d, n, j0)];
    rp[(size_t)m * dim + d] = st->x[XI(st, d, own[m], (j0 + m) % M)];
  }
  int rc = bridge(st, rp, m, j0, exc, NULL, dr);
  if (rp_out) memcpy(rp_out, rp, sizeof(double) * (size_t)(m + 1) * dim);
  if (rc == ORC_HARDCORE) return dr->exhausted ? ORC_EDRAWS : ORC_HARDCORE;
  double wi, wu;
  staging_w(st, n, j0, m, rp, own, Vp, &wi, &wu);
  int acc = metropolis(exp(wu - wi), dr);
  if (dr->exhausted) return ORC_EDRAWS;
  if (acc) {
    for (int t = 0; t < m; ++t) {
      int j = (j0 + t) % M;
      for (int d = 0; d < dim; ++d) st->x[XI(st, d, own[t], j)] = rp[(size_t)t * dim + d];
      st->V[VI(st, own[t], j)] = Vp[t];
      cell_refresh(st, own[t], j);
    }
  }
  return acc ? ORC_ACCEPT : ORC_REJECT;
}

/* ------------------------------------------------------------------------ */
/* ReshapeSwapLinear (src/updates/reshape.jl:123-283) with sampleparticles    */
/* (src/updates/helper.jl:224-267)                                           */
/* ------------------------------------------------------------------------ */
static double logaddexp(double a, double b) {
  double mx = a > b ? a : b;
  if (mx == -INFINITY) return -INFINITY;
  return mx + log(exp(a - mx) + exp(b - mx));
}

/* log of sum_i exp(lnK(x_a(j0), E(i)) + lnK(x_i(j0), E(a))) with ends E */
static double log_sigma(orc_state *st, int a, int j0, double taum, const double *E) {
  const orc_params *p = &st->p;
  int N = p->N, dim = p->dim;
  double ra[MAXDIM], ri[MAXDIM];
  bead_pos(st, a, j0, ra);
  double *w = st->scratch + (size_t)(p->M + 2) * MAXDIM * 4;
  double mx = -INFINITY;
  for (int i = 0; i < N; ++i) {
    bead_pos(st, i, j0, ri);
    w[i] = orc_lnK(p, ra, E + (size_t)i * dim, taum) + orc_lnK(p, ri, E + (size_t)a * dim, taum);
    if (w[i] > mx) mx = w[i];
  }
  double s = 0.0;
  for (int i = 0; i < N; ++i) s += exp(w[i] - mx);
  return mx + log(s);
}

int orc_swap(orc_state *st, int j0, int m, int n1, double u_pick, orc_draws *dr, int *n2_out,
             double *rp_out) {
  const orc_params *p = &st->p;
  int N = p->N, M = p->M, dim = p->dim;
  if (n2_out) *n2_out = -1;
  if (N <= 1) return ORC_SKIP;
  if (n1 < 0 || n1 >= N || j0 < 0 || j0 >= M || m < 2 || m > M - 1) return ORC_EARG;
  int se = (j0 + m) % M, wrap = (j0 + m) >= M;
  double taum = m * p->tau;
  /* ends E(i) = bead at absolute slice j0+m on i's path */
  double *E = (double *)malloc(sizeof(double) * (size_t)N * dim);
  double *q = (double *)malloc(sizeof(double) * (size_t)N);
  for (int i = 0; i < N; ++i) {
    int ei = wrap ? st->next[i] : i;
    bead_pos(st, ei, se, E + (size_t)i * dim);
  }
  /* heat-bath weights exp(t_i + y_i) (helper.jl:233-263); shifted by the max
   * so that they cannot all underflow */
  double ra[MAXDIM], ri[MAXDIM];
  bead_pos(st, n1, j0, ra);
  double mx = -INFINITY;
  for (int i = 0; i < N; ++i) {
    bead_pos(st, i, j0, ri);
    q[i] = orc_lnK(p, ra, E + (size_t)i * dim, taum) + orc_lnK(p, ri, E + (size_t)n1 * dim, taum);
    if (q[i] > mx) mx = q[i];
  }
  double nrm = 0.0;
  for (int i = 0; i < N; ++i) { q[i] = exp(q[i] - mx); nrm += q[i]; }
  double wsum = 0.0;
  for (int i = 0; i < N; ++i) { q[i] = q[i] / nrm; wsum += q[i]; }
  /* StatsBase.sample(a, Weights): first i with cumulative weight >= u*sum */
  double tt = u_pick * wsum, cw = q[0];
  int n2 = 0;
  while (cw < tt && n2 < N - 1) { ++n2; cw += q[n2]; }
  if (n2_out) *n2_out = n2;
  if (n1 == n2) { free(E); free(q); return ORC_SKIP; }

  int *own1 = (int *)malloc(sizeof(int) * (size_t)(m + 1) * 4);
  int *own2 = own1 + (m + 1), *exc1 = own1 + 2 * (m + 1), *exc2 = own1 + 3 * (m + 1);
  for (int t = 0; t <= m; ++t) {
    own1[t] = own_of(st, n1, j0, t);
    own2[t] = own_of(st, n2, j0, t);
  }
  double *r1 = (double *)malloc(sizeof(double) * (size_t)(m + 1) * dim * 2 + sizeof(double) * 2 * m);
  double *r2 = r1 + (size_t)(m + 1) * dim;
  double *V1 = r2 + (size_t)(m + 1) * dim, *V2 = V1 + m;
  for (int d = 0; d < dim; ++d) {
    r1[d] = st->x[XI(st, d, n1, j0)];
    r2[d] = st->x[XI(st, d, n2, j0)];
    r1[(size_t)m * dim + d] = E[(size_t)n2 * dim + d];
    r2[(size_t)m * dim + d] = E[(size_t)n1 * dim + d];
  }
  int rc1, rc2;
  if (p->semantics == ORC_SEM_REFERENCE) {
    for (int t = 0; t <= m; ++t) { exc1[t] = n2; exc2[t] = n1; }
    rc1 = bridge(st, r1, m, j0, exc1, NULL, dr);
    rc2 = bridge(st, r2, m, j0, exc2, NULL, dr);
  } else {
    rc1 = bridge(st, r1, m, j0, own1, own2, dr);
    rc2 = bridge(st, r2, m, j0, own1, own2, dr);
  }
  if (rp_out) {
    memcpy(rp_out, r1, sizeof(double) * (size_t)(m + 1) * dim);
    memcpy(rp_out + (size_t)(m + 1) * dim, r2, sizeof(double) * (size_t)(m + 1) * dim);
  }
  int result;
  if (rc1 == ORC_HARDCORE || rc2 == ORC_HARDCORE) {
    result = ORC_HARDCORE;
    goto done;
  }
  {
    double wi = 0.0, wu = 0.0;
    for (int t = 0; t < m; ++t) {
      int j = (j0 + t) % M;
      wi += st->V[VI(st, own1[t], j)] + st->V[VI(st, own2[t], j)];
      V1[t] = orc_lnV(p, r1 + (size_t)t * dim, r1 + (size_t)(t + 1) * dim);
      V2[t] = orc_lnV(p, r2 + (size_t)t * dim, r2 + (size_t)(t + 1) * dim);
    }
    double s1 = 0.0, s2 = 0.0;
    for (int t = 0; t < m; ++t) { s1 += V1[t]; s2 += V2[t]; }
    wu = s1 + s2;
    double log_ratio = 0.0;
    if (p->interactions) {
      for (int t = 0; t < m; ++t) {
        int j = (j0 + t) % M;
        double a1[MAXDIM], a1n[MAXDIM], a2[MAXDIM], a2n[MAXDIM];
        bead_pos(st, own1[t], j, a1); bead_pos(st, own1[t + 1], (j + 1) % M, a1n);
        bead_pos(st, own2[t], j, a2); bead_pos(st, own2[t + 1], (j + 1) % M, a2n);
        const double *b1 = r1 + (size_t)t * dim, *b1n = r1 + (size_t)(t + 1) * dim;
        const double *b2 = r2 + (size_t)t * dim, *b2n = r2 + (size_t)(t + 1) * dim;
        if (p->semantics == ORC_SEM_REFERENCE) {
          wi += pair_link(st, a1, a1n, j, own1[t], -1);
          wi += pair_link(st, a2, a2n, j, own2[t], -1);
          wi += pair_link(st, b1, b1n, j, own1[t], own2[t]);
          wi += pair_link(st, b2, b2n, j, own1[t], own2[t]);
        } else {
          wi += pair_link(st, a1, a1n, j, own1[t], own2[t]);
          wi += pair_link(st, a2, a2n, j, own1[t], own2[t]);
          wi += pair_cross(p, a1, a1n, a2, a2n);
          wu += pair_link(st, b1, b1n, j, own1[t], own2[t]);
          wu += pair_link(st, b2, b2n, j, own1[t], own2[t]);
          wu += pair_cross(p, b1, b1n, b2, b2n);
        }
      }
    }
    if (p->semantics == ORC_SEM_PHYSICAL) {
      /* heat-bath partner choice needs (1/S'_1 + 1/S'_2) / (1/S_1 + 1/S_2) */
      double l1 = log_sigma(st, n1, j0, taum, E), l2 = log_sigma(st, n2, j0, taum, E);
      double tmp[MAXDIM];
      for (int d = 0; d < dim; ++d) {
        tmp[d] = E[(size_t)n1 * dim + d];
        E[(size_t)n1 * dim + d] = E[(size_t)n2 * dim + d];
        E[(size_t)n2 * dim + d] = tmp[d];
      }
      double l1p = log_sigma(st, n1, j0, taum, E), l2p = log_sigma(st, n2, j0, taum, E);
      log_ratio = logaddexp(-l1p, -l2p) - logaddexp(-l1, -l2);
    }
    int acc = metropolis(exp(wu - wi + log_ratio), dr);
    if (dr->exhausted) { result = ORC_EDRAWS; goto done; }
    if (!acc) { result = ORC_REJECT; goto done; }
    /* accept: swap next, write the bridges along the new cycles, swap tails */
    int tn = st->next[n1]; st->next[n1] = st->next[n2]; st->next[n2] = tn;
    for (int t = 1; t <= m; ++t) {
      int j = (j0 + t) % M;
      int o1 = own_of(st, n1, j0, t), o2 = own_of(st, n2, j0, t);
      for (int d = 0; d < dim; ++d) {
        st->x[XI(st, d, o1, j)] = r1[(size_t)t * dim + d];
        st->x[XI(st, d, o2, j)] = r2[(size_t)t * dim + d];
      }
    }
    for (int t = 0; t < m; ++t) {
      int j = (j0 + t) % M;
      st->V[VI(st, own_of(st, n1, j0, t), j)] = V1[t];
      st->V[VI(st, own_of(st, n2, j0, t), j)] = V2[t];
    }
    if (j0 + m < M - 1) {
      for (int j = j0 + m + 1; j < M; ++j) {
        for (int d = 0; d < dim; ++d) {
          double a = st->x[XI(st, d, n1, j)];
          st->x[XI(st, d, n1, j)] = st->x[XI(st, d, n2, j)];
          st->x[XI(st, d, n2, j)] = a;
        }
        double v = st->V[VI(st, n1, j)];
        st->V[VI(st, n1, j)] = st->V[VI(st, n2, j)];
        st->V[VI(st, n2, j)] = v;
      }
    }
    if (p->semantics == ORC_SEM_PHYSICAL && j0 + m <= M - 1) {
      int j = j0 + m;
      double v = st->V[VI(st, n1, j)];
      st->V[VI(st, n1, j)] = st->V[VI(st, n2, j)];
      st->V[VI(st, n2, j)] = v;
    }
    if (use_cells(st)) {
      for (int t = 1; t <= m; ++t) {
        int j = (j0 + t) % M;
        cell_refresh(st, own_of(st, n1, j0, t), j);
        cell_refresh(st, own_of(st, n2, j0, t), j);
      }
      for (int j = j0 + m + 1; j < M; ++j) { cell_refresh(st, n1, j); cell_refresh(st, n2, j); }
    }
    result = ORC_ACCEPT;
  }
done:
  free(E); free(q); free(own1); free(r1);
  return result;
}

/* ------------------------------------------------------------------------ */
/* SingleCenterOfMass / PolymerCenterOfMass (src/updates/com.jl) with        */
/* move_polymer! (src/updates/helper.jl:368-395)                             */
/* ------------------------------------------------------------------------ */
static int com_core(orc_state *st, const int *pol, int npol, double maxd, orc_draws *dr) {
  const orc_params *p = &st->p;
  int M = p->M, dim = p->dim, N = p->N;
  size_t nb = (size_t)npol * M;
  double *rp = (double *)malloc(sizeof(double) * nb * dim + sizeof(double) * nb);
  double *Vp = rp + nb * dim;
  int *inpol = (int *)calloc(N, sizeof(int));
  int *idx = (int *)malloc(sizeof(int) * N);
  for (int i = 0; i < npol; ++i) { inpol[pol[i]] = 1; idx[pol[i]] = i; }
  int tries = 0, bad = 1, result;
  double shift[MAXDIM];
  while (bad) {
    bad = 0;
    if (++tries > p->ctr) { result = ORC_HARDCORE; goto out; }
    for (int d = 0; d < dim; ++d) shift[d] = maxd * 2.0 * (draw_uniform(dr) - 0.5);
    for (int i = 0; i < npol && !bad; ++i)
      for (int j = 0; j < M; ++j) {
        double *r = rp + ((size_t)i * M + j) * dim;
        for (int d = 0; d < dim; ++d) r[d] = orc_teleport(st->x[XI(st, d, pol[i], j)] + shift[d], p->L);
        if (p->hardcore_a > 0.0 && hardcore_hit(st, r, j, pol[i], -1)) { bad = 1; break; }
      }
  }
  {
    double wi = 0.0, wu = 0.0;
    for (int i = 0; i < npol; ++i)
      for (int j = 0; j < M; ++j) wi += st->V[VI(st, pol[i], j)];
    for (int i = 0; i < npol; ++i)
      for (int j = 0; j < M; ++j) {
        int ii = (j == M - 1) ? idx[st->next[pol[i]]] : i;
        Vp[(size_t)i * M + j] = orc_lnV(p, rp + ((size_t)i * M + j) * dim, rp + ((size_t)ii * M + (j + 1) % M) * dim);
        wu += Vp[(size_t)i * M + j];
      }
    if (p->interactions && p->semantics == ORC_SEM_PHYSICAL) {
      /* pairs with particles outside the moved cycle; pairs inside it are
       * unchanged by a rigid shift */
      for (int i = 0; i < npol; ++i)
        for (int j = 0; j < M; ++j) {
          int n = pol[i], nn = (j == M - 1) ? st->next[n] : n, ii = idx[nn];
          double a[MAXDIM], an[MAXDIM];
          bead_pos(st, n, j, a); bead_pos(st, nn, (j + 1) % M, an);
          const double *b = rp + ((size_t)i * M + j) * dim, *bn = rp + ((size_t)ii * M + (j + 1) % M) * dim;
          int cells[9], nc;
          for (int side = 0; side < 2; ++side) {
            const double *P = side ? b : a, *Pn = side ? bn : an;
            double w = 0.0;
            nc = stencil(p, cell_of(p, P), cells);
            for (int ci = 0; ci < nc; ++ci)
              for (int q = st->cell_head[(size_t)j * st->ncell + cells[ci]]; q >= 0;
                   q = st->cell_nxt[(size_t)j * N + q]) {
                if (inpol[q]) continue;
                double rq[MAXDIM], rqn[MAXDIM];
                bead_pos(st, q, j, rq);
                bead_pos(st, j == M - 1 ? st->next[q] : q, (j + 1) % M, rqn);
                w += pair_cross(p, P, Pn, rq, rqn);
              }
            if (side) wu += w; else wi += w;
          }
        }
    }
    int acc = metropolis(exp(wu - wi), dr);
    if (dr->exhausted) { result = ORC_EDRAWS; goto out; }
    if (acc) {
      for (int i = 0; i < npol; ++i)
        for (int j = 0; j < M; ++j) {
          for (int d = 0; d < dim; ++d) st->x[XI(st, d, pol[i], j)] = rp[((size_t)i * M + j) * dim + d];
          st->V[VI(st, pol[i], j)] = Vp[(size_t)i * M + j];
          cell_refresh(st, pol[i], j);
        }
    }
    result = acc ? ORC_ACCEPT : ORC_REJECT;
  }
out:
  free(rp); free(inpol); free(idx);
  return result;
}

int orc_com(orc_state *st, int n, double maxd, orc_draws *dr) {
  if (n < 0 || n >= st->p.N || st->next[n] != n) return ORC_EARG;
  return com_core(st, &n, 1, maxd, dr);
}

int orc_polymer_com(orc_state *st, int n, double maxd, orc_draws *dr) {
  int N = st->p.N;
  if (n < 0 || n >= N) return ORC_EARG;
  int *pol = (int *)malloc(sizeof(int) * N);
  int np = 0, i = n;
  do { pol[np++] = i; i = st->next[i]; } while (i != n && np <= N);
  int r = np > N ? ORC_EARG : com_core(st, pol, np, maxd, dr);
  free(pol);
  return r;
}

/* ------------------------------------------------------------------------ */
/* estimators (src/measurement.jl)                                           */
/* ------------------------------------------------------------------------ */
/* pair energy / virial terms of the link-formulated pair action:
 * E_pair = S_pair / (M tau), virial = (1/(2 M tau)) sum d . dS/dd */
static void pair_terms(const orc_state *st, double *epair, double *evir) {
  const orc_params *p = &st->p;
  int N = p->N, M = p->M, dim = p->dim;
  double s = 0.0, v = 0.0, c = p->inv2s2, rc2 = p->rc * p->rc;
  for (int j = 0; j < M; ++j)
    for (int a = 0; a < N; ++a) {
      double ra[MAXDIM], ran[MAXDIM];
      bead_pos(st, a, j, ra);
      bead_pos(st, j == M - 1 ? st->next[a] : a, (j + 1) % M, ran);
      for (int b = a + 1; b < N; ++b) {
        double rb[MAXDIM], rbn[MAXDIM];
        bead_pos(st, b, j, rb);
        double d1 = mi_dist2(p, ra, rb, NULL);
        if (d1 > rc2) continue;
        bead_pos(st, j == M - 1 ? st->next[b] : b, (j + 1) % M, rbn);
        double d2 = mi_dist2(p, ran, rbn, NULL);
        double v1 = vpair_r2(p, d1), v2 = vpair_r2(p, d2);
        s += 0.5 * p->tau * (v1 + v2);
        v += 0.5 * p->tau * (-2.0 * c * d1 * v1 - 2.0 * c * d2 * v2);
      }
    }
  (void)dim;
  *epair = s / (M * p->tau);
  *evir = *epair + v / (2.0 * M * p->tau);
}

/* signed minimum-image difference b - a, of magnitude distance(a, b) */
static double mi_signed1(double b, double a, double L) {
  double q = orc_distance(a, b, L), x = b - a;
  return (fabs(x) > L) == (x > 0) ? -q : q;
}

void orc_superfluid(const orc_state *st, double out[3]) {
  const orc_params *p = &st->p;
  int N = p->N, M = p->M, dim = p->dim;
  double w[MAXDIM] = {0.0, 0.0}, area = 0.0, rsq = 0.0;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < M; ++j) {
      int inext = (j == M - 1) ? st->next[i] : i, jn = (j + 1) % M;
      double a[MAXDIM] = {0.0, 0.0}, b[MAXDIM] = {0.0, 0.0}, dv[MAXDIM] = {0.0, 0.0};
      bead_pos(st, i, j, a);
      bead_pos(st, inext, jn, b);
      for (int d = 0; d < dim; ++d) { dv[d] = mi_signed1(b[d], a[d], p->L); w[d] += dv[d]; }
      area += 0.5 * (a[0] * dv[1] - a[1] * dv[0]);
      rsq += a[0] * a[0] + a[1] * a[1];
    }
  out[0] = w[0] * w[0] + w[1] * w[1];
  out[1] = area;
  out[2] = rsq / M;
}

void orc_radial(const orc_state *st, int nb, double dr, double *hist) {
  const orc_params *p = &st->p;
  int N = p->N, M = p->M, dim = p->dim;
  for (int j = 0; j < M; ++j)
    for (int a = 0; a < N; ++a)
      for (int b = a + 1; b < N; ++b) {
        double ra[MAXDIM], rb[MAXDIM];
        bead_pos(st, a, j, ra);
        bead_pos(st, b, j, rb);
        double s = 0.0;
        for (int d = 0; d < dim; ++d) { double q = orc_distance(ra[d], rb[d], p->L); s += q * q; }
        double k = floor(sqrt(s) / dr);
        if (k < (double)nb) hist[(int)k] += 1.0;
      }
}

void orc_energy(const orc_state *st, double out[4]) {
  const orc_params *p = &st->p;
  int N = p->N, M = p->M, dim = p->dim;
  double link = 0.0, pot = 0.0, vkin = 0.0, vpot = 0.0;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < M; ++j) {
      int inext = (j == M - 1) ? st->next[i] : i, jn = (j + 1) % M;
      double a[MAXDIM], b[MAXDIM], g[MAXDIM];
      bead_pos(st, i, j, a); bead_pos(st, inext, jn, b);
      double l = 0.0;
      for (int d = 0; d < dim; ++d) { double q = orc_distance(a[d], b[d], p->L); l += q * q; }
      link += l;
      double va = orc_Vext(p, a), vb = orc_Vext(p, b);
      pot += va + vb;
      orc_dVext(p, a, g);
      double k = 0.0;
      for (int d = 0; d < dim; ++d) k += a[d] * g[d];
      vkin += k;
      vpot += va + vb;
    }
  double tau = p->tau;
  out[0] = (double)(dim * N) / (2.0 * tau) - 1.0 / (4.0 * p->lambda * (tau * tau) * M) * link + 1.0 / (2.0 * M) * pot;
  out[1] = 1.0 / (2.0 * M) * vkin + 1.0 / (2.0 * M) * vpot;
  out[2] = out[3] = 0.0;
  /* the contact table has no tau derivative: no pair energy for it */
  if (p->interactions && !p->ct_tab) pair_terms(st, &out[2], &out[3]);
}

/* Density (src/measurement.jl:45-55): bin floor((r+L)/bin), counted only for
 * 1 <= ibin <= nbins, so the first row/column is dropped as in the reference */
void orc_density(const orc_state *st, int nb, double *hist) {
  const orc_params *p = &st->p;
  double bw = (2.0 * p->L) / nb;
  for (int n = 0; n < p->N; ++n)
    for (int j = 0; j < p->M; ++j) {
      int ok = 1, idx = 0, mul = 1;
      for (int d = 0; d < p->dim; ++d) {
        long ib = (long)floor((st->x[XI(st, d, n, j)] + p->L) / bw);
        if (ib < 1 || ib > nb) { ok = 0; break; }
        idx += (int)(ib - 1) * mul; mul *= nb;
      }
      if (ok) hist[idx] += 1.0;
    }
}

void orc_eval_action(const orc_state *st, double out[4]) {
  const orc_params *p = &st->p;
  int N = p->N, M = p->M;
  double k = 0.0, v = 0.0, u = 0.0, c = 0.0;
  for (int n = 0; n < N; ++n)
    for (int j = 0; j < M; ++j) {
      double a[MAXDIM], b[MAXDIM];
      bead_pos(st, n, j, a);
      bead_pos(st, j == M - 1 ? st->next[n] : n, (j + 1) % M, b);
      k += orc_lnK(p, a, b, p->tau);
      v += orc_lnV(p, a, b);
      c += st->V[VI(st, n, j)];
    }
  if (p->interactions) {
    double rc2 = p->rc * p->rc;
    for (int j = 0; j < M; ++j)
      for (int a = 0; a < N; ++a) {
        double ra[MAXDIM], ran[MAXDIM];
        bead_pos(st, a, j, ra);
        bead_pos(st, j == M - 1 ? st->next[a] : a, (j + 1) % M, ran);
        for (int b = a + 1; b < N; ++b) {
          double rb[MAXDIM], rbn[MAXDIM], d1[MAXDIM], d2[MAXDIM];
          bead_pos(st, b, j, rb);
          if (mi_dist2(p, ra, rb, d1) > rc2) continue;
          bead_pos(st, j == M - 1 ? st->next[b] : b, (j + 1) % M, rbn);
          mi_dist2(p, ran, rbn, d2);
          u += orc_lnU(p, d1, d2);
        }
      }
  }
  out[0] = k; out[1] = v; out[2] = u; out[3] = c;
}

/* ------------------------------------------------------------------------ */
/* run! driver (src/simulation.jl:1-42) with Counter/adjust! (helper.jl:6-52) */
/* ------------------------------------------------------------------------ */
void orc_update_init(orc_update *u, int kind, int every, double var, double minvar,
                     double maxvar, double minacc, double maxacc, int adj, int range) {
  memset(u, 0, sizeof(*u));
  u->kind = kind; u->every = every; u->var = var; u->minvar = minvar; u->maxvar = maxvar;
  u->minacc = minacc; u->maxacc = maxacc; u->adj = adj; u->range = range;
  u->queue = (unsigned char *)calloc(range > 0 ? range : 1, 1);
}
void orc_update_free(orc_update *u) { free(u->queue); u->queue = NULL; }

static void queue_push(orc_update *u, int acc) {
  u->tries++;
  if (u->qlen < u->range) {
    u->queue[(u->qhead + u->qlen) % u->range] = (unsigned char)acc;
    u->qlen++;
  } else {
    u->qsum -= u->queue[u->qhead];
    u->queue[u->qhead] = (unsigned char)acc;
    u->qhead = (u->qhead + 1) % u->range;
  }
  u->qsum += acc;
}

static void adjust(orc_update *u) {
  double acc = u->qlen ? (double)u->qsum / u->qlen : NAN;
  if (u->kind == 0 || u->kind == 1) {
    if (acc < u->minacc) u->var -= 1; else if (acc > u->maxacc) u->var += 1;
  } else {
    if (acc < u->minacc) u->var *= 0.9; else if (acc > u->maxacc) u->var *= 1.1;
  }
  if (u->var < u->minvar) u->var = u->minvar;
  if (u->var > u->maxvar) u->var = u->maxvar;
}

static int rand_range(orc_rng *r, int lo, int hi) { /* uniform integer in [lo, hi] */
  return lo + (int)floor(orc_rng_uniform(r) * (hi - lo + 1));
}

int orc_run(orc_state *st, long n, orc_update *ups, int nups, orc_rng *rng, int ncycle,
            double *e_out, long e_cap, long *e_count, int dens_nb, double *hist, long *ndata,
            orc_run_stats *stats) {
  const orc_params *p = &st->p;
  int N = p->N, M = p->M;
  orc_draws dr; memset(&dr, 0, sizeof(dr)); dr.rng = rng;
  double wsum = 0.0;
  for (int k = 0; k < nups; ++k) wsum += 1.0 / ups[k].every;
  int *singles = (int *)malloc(sizeof(int) * N);
  long nctr = 0;
  for (long it = 0; it < n; ++it) {
    double t = orc_rng_uniform(rng) * wsum, cw = 1.0 / ups[0].every;
    int k = 0;
    while (cw < t && k < nups - 1) { ++k; cw += 1.0 / ups[k].every; }
    orc_update *u = &ups[k];
    int rc = ORC_SKIP;
    double beads = 0.0;
    if (u->kind == 0) {
      int nn = rand_range(rng, 0, N - 1), j0 = rand_range(rng, 0, M - 1);
      int m = rand_range(rng, 2, (int)u->var);
      if (m > (int)u->maxvar) m = (int)u->maxvar;
      rc = orc_staging(st, nn, j0, m, &dr, NULL);
      if (rc != ORC_HARDCORE) beads = m - 1;
    } else if (u->kind == 1) {
      if (N > 1) {
        int j0 = rand_range(rng, 0, M - 1);
        int m = rand_range(rng, 2, (int)u->var);
        if (m > (int)u->maxvar) m = (int)u->maxvar;
        int n1 = rand_range(rng, 0, N - 1);
        double up = orc_rng_uniform(rng);
        rc = orc_swap(st, j0, m, n1, up, &dr, NULL, NULL);
        if (rc == ORC_ACCEPT || rc == ORC_REJECT) beads = 2.0 * (m - 1);
      }
    } else if (u->kind == 2) {
      int ns = 0;
      for (int i = 0; i < N; ++i) if (st->next[i] == i) singles[ns++] = i;
      if (ns > 0) {
        int nn = singles[rand_range(rng, 0, ns - 1)];
        rc = orc_com(st, nn, u->var, &dr);
        if (rc != ORC_HARDCORE) beads = M;
      }
    } else {
      int nn = rand_range(rng, 0, N - 1);
      int np = 0, i = nn;
      do { ++np; i = st->next[i]; } while (i != nn && np <= N);
      rc = orc_polymer_com(st, nn, u->var, &dr);
      if (rc != ORC_HARDCORE) beads = (double)M * np;
    }
    if (rc < 0) { free(singles); return rc; }
    int acc = rc == ORC_ACCEPT;
    if (rc != ORC_SKIP) queue_push(u, acc);
    if (stats) {
      stats->attempts[u->kind]++; stats->accepts[u->kind] += acc; stats->bead_updates += beads;
    }
    u->attempts++; u->accepts += acc;
    if (u->adj > 0 && u->tries % u->adj == 0) adjust(u);
    if (ncycle > 0) {
      if (++nctr == ncycle) {
        nctr = 0;
        if (e_out && e_count && *e_count < e_cap) {
          double e[4]; orc_energy(st, e);
          for (int q = 0; q < 4; ++q) e_out[*e_count * 4 + q] = e[q];
          (*e_count)++;
        }
        if (hist) { orc_density(st, dens_nb, hist); if (ndata) *ndata += M; }
        if (stats) stats->measurements++;
      }
    }
  }
  free(singles);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* multi-chain CPU timing (one chain per host thread at a time)              */
/* ------------------------------------------------------------------------ */
typedef struct {
  const orc_params *p; int c0, c1; long attempts; int ell; double com_step; uint64_t seed;
  double beads;
} bench_job;

static void *bench_worker(void *arg) {
  bench_job *jb = (bench_job *)arg;
  const orc_params *p = jb->p;
  for (int c = jb->c0; c < jb->c1; ++c) {
    orc_state *st = orc_create(p);
    orc_rng rng; orc_rng_init(&rng, jb->seed, (uint64_t)c);
    orc_draws dr; memset(&dr, 0, sizeof(dr)); dr.rng = &rng;
    orc_init_world(st, &dr);
    int k = (p->M + jb->ell - 1) / jb->ell;
    orc_update ups[3];
    int maxs = p->M - 2;
    int l = jb->ell < maxs ? jb->ell : maxs;
    orc_update_init(&ups[0], 0, 1, l, 2, maxs, 0.0, 1.0, 10, 10000);
    orc_update_init(&ups[1], 1, k, l, 2, maxs, 0.0, 1.0, 10, 10000);
    orc_update_init(&ups[2], 2, k, jb->com_step, 0.1, p->L / 2, 0.4, 0.6, 10, 10000);
    orc_run_stats s; memset(&s, 0, sizeof(s));
    orc_run(st, jb->attempts, ups, 3, &rng, 0, NULL, 0, NULL, 0, NULL, NULL, &s);
    jb->beads += s.bead_updates;
    for (int q = 0; q < 3; ++q) orc_update_free(&ups[q]);
    orc_destroy(st);
  }
  return NULL;
}

double orc_bench_chains(const orc_params *p, int nchains, int nthreads, long attempts, int ell,
                        double com_step, uint64_t seed, double *bead_updates) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > nchains) nthreads = nchains;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  bench_job *jobs = (bench_job *)calloc(nthreads, sizeof(bench_job));
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int i = 0; i < nthreads; ++i) {
    jobs[i].p = p; jobs[i].c0 = (int)((long)nchains * i / nthreads);
    jobs[i].c1 = (int)((long)nchains * (i + 1) / nthreads);
    jobs[i].attempts = attempts; jobs[i].ell = ell; jobs[i].com_step = com_step; jobs[i].seed = seed;
    pthread_create(&th[i], NULL, bench_worker, &jobs[i]);
  }
  double beads = 0.0;
  for (int i = 0; i < nthreads; ++i) { pthread_join(th[i], NULL); beads += jobs[i].beads; }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  free(th); free(jobs);
  if (bead_updates) *bead_updates = beads;
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* ------------------------------------------------------------------------ */
/* time-budgeted multi-chain timing                                          */
/* ------------------------------------------------------------------------ */
typedef struct {
  orc_state *st; orc_update ups[3]; orc_rng rng; long per; double cost;
} budget_chain;

typedef struct {
  budget_chain **mine; int n; double budget; struct timespec t0;
  double beads, sweeps, stop;
  pthread_barrier_t *bar;
} budget_job;

static double secs_since(const struct timespec *t0) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)(t.tv_sec - t0->tv_sec) + 1e-9 * (double)(t.tv_nsec - t0->tv_nsec);
}

static void *budget_worker(void *arg) {
  budget_job *jb = (budget_job *)arg;
  pthread_barrier_wait(jb->bar);
  int done = jb->n == 0;
  while (!done) {
    for (int c = 0; c < jb->n && !done; ++c) {
      budget_chain *bc = jb->mine[c];
      long left = bc->per;
      while (left > 0) {
        long chunk = left < 256 ? left : 256;
        orc_run_stats s; memset(&s, 0, sizeof(s));
        orc_run(bc->st, chunk, bc->ups, 3, &bc->rng, 0, NULL, 0, NULL, 0, NULL, NULL, &s);
        jb->beads += s.bead_updates;
        left -= chunk;
        if (secs_since(&jb->t0) >= jb->budget) { done = 1; break; }
      }
      if (left == 0) jb->sweeps += 1.0;
    }
  }
  jb->stop = secs_since(&jb->t0);
  return NULL;
}

double orc_bench_budget(const orc_params *ps, const int *ells, int nchains, int nthreads,
                        double budget_s, double com_step, uint64_t seed, double *bead_updates,
                        double *sweeps) {
  if (nthreads < 1) nthreads = 1;
  budget_chain *bc = (budget_chain *)calloc(nchains > 0 ? nchains : 1, sizeof(budget_chain));
  int *order = (int *)malloc(sizeof(int) * (nchains > 0 ? nchains : 1));
  for (int c = 0; c < nchains; ++c) {
    const orc_params *p = &ps[c];
    bc[c].st = orc_create(p);
    orc_rng_init(&bc[c].rng, seed, (uint64_t)c);
    orc_draws dr; memset(&dr, 0, sizeof(dr)); dr.rng = &bc[c].rng;
    orc_init_world(bc[c].st, &dr);
    int ell = ells[c], maxs = p->M - 2;
    int l = ell < maxs ? ell : maxs;
    int k = (p->M + ell - 1) / ell;
    orc_update_init(&bc[c].ups[0], 0, 1, l, 2, maxs, 0.0, 1.0, 10, 10000);
    orc_update_init(&bc[c].ups[1], 1, k, l, 2, maxs, 0.0, 1.0, 10, 10000);
    orc_update_init(&bc[c].ups[2], 2, k, com_step, 0.1, p->L / 2, 0.4, 0.6, 10, 10000);
    bc[c].per = (long)p->N * (k + 2);
    bc[c].cost = (double)p->N * p->M * (p->interactions ? 4.0 : 1.0) + 0.5 * (double)p->N * p->N;
    order[c] = c;
  }
  /* longest first (insertion sort keeps it dependency-free), each chain to
     the least-loaded thread */
  for (int a = 1; a < nchains; ++a) {
    int v = order[a], b = a - 1;
    while (b >= 0 && bc[order[b]].cost < bc[v].cost) { order[b + 1] = order[b]; --b; }
    order[b + 1] = v;
  }
  budget_job *jobs = (budget_job *)calloc(nthreads, sizeof(budget_job));
  double *load = (double *)calloc(nthreads, sizeof(double));
  for (int t = 0; t < nthreads; ++t) jobs[t].mine = (budget_chain **)malloc(sizeof(budget_chain *) * (nchains > 0 ? nchains : 1));
  for (int a = 0; a < nchains; ++a) {
    int best = 0;
    for (int t = 1; t < nthreads; ++t) if (load[t] < load[best]) best = t;
    jobs[best].mine[jobs[best].n++] = &bc[order[a]];
    load[best] += bc[order[a]].cost;
  }
  pthread_barrier_t bar;
  pthread_barrier_init(&bar, NULL, (unsigned)nthreads + 1);
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  for (int t = 0; t < nthreads; ++t) {
    jobs[t].budget = budget_s; jobs[t].bar = &bar;
    pthread_create(&th[t], NULL, budget_worker, &jobs[t]);
  }
  struct timespec t0;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int t = 0; t < nthreads; ++t) jobs[t].t0 = t0;
  pthread_barrier_wait(&bar);
  double beads = 0.0, sw = 0.0, wall = 0.0;
  for (int t = 0; t < nthreads; ++t) {
    pthread_join(th[t], NULL);
    beads += jobs[t].beads; sw += jobs[t].sweeps;
    if (jobs[t].stop > wall) wall = jobs[t].stop;
    free(jobs[t].mine);
  }
  pthread_barrier_destroy(&bar);
  for (int c = 0; c < nchains; ++c) {
    for (int q = 0; q < 3; ++q) orc_update_free(&bc[c].ups[q]);
    orc_destroy(bc[c].st);
  }
  free(th); free(jobs); free(load); free(bc); free(order);
  if (bead_updates) *bead_updates = beads;
  if (sweeps) *sweeps = sw;
  return wall;
}

/* ------------------------------------------------------------------------ */
/* the engine's sweep schedule with the reference's moves                     */
/* ------------------------------------------------------------------------ */
int orc_run_sweeps(orc_state *st, long nsweeps, int ell, int swaps, double *com_step,
                   double com_min, double com_max, double com_minacc, double com_maxacc,
                   orc_rng *rng, int measure_every, double *e_out, long e_cap, long *e_count,
                   int dens_nb, double *hist, long *ndata, orc_run_stats *stats) {
  const orc_params *p = &st->p;
  const int N = p->N, M = p->M;
  orc_draws dr; memset(&dr, 0, sizeof(dr)); dr.rng = rng;
  int l = ell;
  if (l > M - 1) l = M - 1;
  if (l > 64) l = 64;
  if (l < 2) l = 2;
  const int k = (M + l - 1) / l;
  for (long sw = 0; sw < nsweeps; ++sw) {
    /* staging phase */
    const int o = (int)fmin((double)(M - 1), floor(orc_rng_uniform(rng) * M));
    for (int s = 0; s < k; ++s) {
      const int len = s < k - 1 ? l : M - (k - 1) * l;
      if (len < 2) continue;
      const int j0 = (o + s * l) % M;
      for (int n = 0; n < N; ++n) {
        int m = 2 + (int)floor(orc_rng_uniform(rng) * (l - 1));
        if (m > len) m = len;
        const int rc = orc_staging(st, n, j0, m, &dr, NULL);
        if (rc < 0) return rc;
        if (stats) {
          stats->attempts[0]++; stats->accepts[0] += rc == ORC_ACCEPT;
          if (rc != ORC_HARDCORE) stats->bead_updates += m - 1;
        }
      }
    }
    /* swaps */
    if (N > 1)
      for (int a = 0; a < swaps; ++a) {
        const int j0 = (int)fmin((double)(M - 1), floor(orc_rng_uniform(rng) * M));
        int m = 2 + (int)floor(orc_rng_uniform(rng) * (l - 1));
        if (m > l) m = l;
        const int n1 = (int)fmin((double)(N - 1), floor(orc_rng_uniform(rng) * N));
        const double up = orc_rng_uniform(rng);
        const int rc = orc_swap(st, j0, m, n1, up, &dr, NULL, NULL);
        if (rc < 0) return rc;
        if (stats && rc != ORC_SKIP) {
          stats->attempts[1]++; stats->accepts[1] += rc == ORC_ACCEPT;
          if (rc != ORC_HARDCORE) stats->bead_updates += 2.0 * (m - 1);
        }
      }
    /* centre of mass: one attempt per single path */
    long catt = 0, cacc = 0;
    for (int n = 0; n < N; ++n) {
      if (st->next[n] != n) continue;
      const int rc = orc_com(st, n, *com_step, &dr);
      if (rc < 0) return rc;
      ++catt; cacc += rc == ORC_ACCEPT;
      if (stats) {
        stats->attempts[2]++; stats->accepts[2] += rc == ORC_ACCEPT;
        if (rc != ORC_HARDCORE) stats->bead_updates += M;
      }
    }
    if (catt > 0) {
      const double r = (double)cacc / (double)catt;
      if (r < com_minacc) *com_step *= 0.9;
      else if (r > com_maxacc) *com_step *= 1.1;
      if (*com_step < com_min) *com_step = com_min;
      if (*com_step > com_max) *com_step = com_max;
    }
    if (measure_every > 0 && (sw + 1) % measure_every == 0) {
      if (e_out && e_count && *e_count < e_cap) {
        double e[4]; orc_energy(st, e);
        for (int q = 0; q < 4; ++q) e_out[*e_count * 4 + q] = e[q];
        (*e_count)++;
      }
      if (hist) { orc_density(st, dens_nb, hist); if (ndata) *ndata += M; }
      if (stats) stats->measurements++;
    }
  }
  return dr.exhausted ? ORC_EDRAWS : 0;
}
