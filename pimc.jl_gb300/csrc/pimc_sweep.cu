// pimc_sweep.cu -- kernels of the GB300 sweep engine.
//
// One CTA (or one warp) owns one chain for the duration of a sweep, of a
// block of sweeps, or of one phase of a sweep (staging, swaps, the rest as
// three launches).  Chains that fit are staged in shared memory (x, V, the
// 16-bit position mirror and next); larger ones are updated in place in
// HBM/L2.  The same kernels serve the plain path (one launch per chain) and
// the batched path (persistent grid pulling chains from a device work queue
// in LPT order, captured in a CUDA graph).  Also here: the layout
// transposes, init_world, the estimators' launch, the adjoint, the contact
// table and the FP64 throughput probe.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>

#include "pimc_sweep.cuh"

namespace pimc {

// the sweep's phases as separate launches (staging, swaps, the rest), each
// compiled and scheduled on its own: every chain of the batch finishes one
// phase before any starts the next, so the longest chain of each phase, not
// the longest sum over phases, sets a sweep's time
__global__ void __launch_bounds__(512, 1) k_sweep_stage(SweepArgs a) { sweep_cta<SW_STAGE>(a); }
__global__ void __launch_bounds__(512, 1) k_sweep_rest(SweepArgs a) { sweep_cta<SW_REST>(a); }

// ---------------------------------------------------------------------------
// state maintenance: layout transposes, init_world, cached links + mirror,
// measurements
// ---------------------------------------------------------------------------
// host layout x[d][n][j] (a batch buffer at d.host_off) -> device x[j][n][d]
__global__ void k_import(const ChainDesc *desc, double *dpool, const double *src, int chain0) {
  const ChainDesc &d = desc[chain0 + blockIdx.y];
  const size_t tot = (size_t)d.dim * d.N * d.M;
  double *x = dpool + d.x_off;
  const double *s = src + d.host_off;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t row = (size_t)d.N * d.dim;
    const size_t j = e / row, r = e % row;
    const size_t n = r / d.dim, k = r % d.dim;
    x[e] = s[(k * d.N + n) * d.M + j];
  }
}

__global__ void k_export(const ChainDesc *desc, const double *dpool, double *dst, int chain0) {
  const ChainDesc &d = desc[chain0 + blockIdx.y];
  const size_t tot = (size_t)d.dim * d.N * d.M;
  const double *x = dpool + d.x_off;
  double *o = dst + d.host_off;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t k = e / ((size_t)d.M * d.N), r = e % ((size_t)d.M * d.N);
    const size_t n = r / d.M, j = r % d.M;
    o[e] = x[(j * d.N + n) * d.dim + k];
  }
}

// The same transposes through 32 x 32 tiles of (particle, slice), over a
// flat list of every chain's tiles (tile_off[c] = first tile of chain c), so
// that both sides are read and written in whole rows: the host layout
// x[d][n][j] in runs of 32 slices, the device layout x[j][n][d] in runs of
// 32 particles.  The host-layout side may be the caller's pinned host buffer,
// which the GPU reads and writes directly over the coherent CPU-GPU link
// (Grace-Blackwell NVLink-C2C): the copy and the transpose are one pass.
// Persistent grid; each block walks tiles t = blockIdx.x, += gridDim.x.
__device__ __forceinline__ int tile_chain(const int *tile_off, int c_lo, int c_hi, int t) {
  int lo = c_lo, hi = c_hi;  // tile_off[lo] <= t < tile_off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (tile_off[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

template <bool IMPORT>
__global__ void __launch_bounds__(256) k_transpose_tiles(const ChainDesc *desc, double *dpool,
                                                          double *host, const int *tile_off,
                                                          int c_lo, int c_hi) {
  __shared__ double tile[2][32][33];
  const int t_end = tile_off[c_hi];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = tile_off[c_lo] + blockIdx.x; t < t_end; t += gridDim.x) {
    const int c = tile_chain(tile_off, c_lo, c_hi, t);
    const ChainDesc &d = desc[c];
    const int N = d.N, M = d.M, dim = d.dim;
    const int tj = (M + 31) >> 5, lt = t - tile_off[c];
    const int n0 = (lt / tj) * 32, j0 = (lt % tj) * 32;
    const int nn = min(32, N - n0), nj = min(32, M - j0);
    double *x = dpool + d.x_off;
    double *hx = host + d.host_off;
    if (IMPORT) {
      // host rows (k, n): 32 consecutive slices per warp-wide read
      for (int r = w; r < dim * nn; r += 8) {
        const int k = r / nn, n = r % nn;
        if (lane < nj) tile[k][n][lane] = hx[((size_t)k * N + n0 + n) * M + j0 + lane];
      }
      __syncthreads();
      // device rows j: 32 particles x dim consecutive doubles each
      const int row = nn * dim;
      for (int q = threadIdx.x; q < nj * row; q += blockDim.x) {
        const int jj = q / row, e = q % row;
        const int n = e / dim, k = e % dim;
        x[((size_t)(j0 + jj) * N + n0) * dim + e] = tile[k][n][jj];
      }
      __syncthreads();
    } else {
      const int row = nn * dim;
      for (int q = threadIdx.x; q < nj * row; q += blockDim.x) {
        const int jj = q / row, e = q % row;
        const int n = e / dim, k = e % dim;
        tile[k][n][jj] = x[((size_t)(j0 + jj) * N + n0) * dim + e];
      }
      __syncthreads();
      for (int r = w; r < dim * nn; r += 8) {
        const int k = r / nn, n = r % nn;
        if (lane < nj) hx[((size_t)k * N + n0 + n) * M + j0 + lane] = tile[k][n][lane];
      }
      __syncthreads();
    }
  }
}

// init_world (src/system.jl:36-78): uniform start, closed Levy loop through
// M rows whose first and last rows coincide, teleport
__global__ void k_init_world(const ChainDesc *desc, double *dpool, int *ipool, int chain0) {
  const ChainDesc &d = desc[chain0 + blockIdx.y];
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= d.N) return;
  CV c = make_cv(&d, dpool, ipool, nullptr);
  const int M = d.M, dim = d.dim;
  GenDraws dr = gen_draws(make_stream(d, 0, PH_INIT, (unsigned)n));
  const double L = d.L, inv2L = 1.0 / (2.0 * L);
  double st[2] = {0.0, 0.0};
  for (int k = 0; k < dim; ++k) {
    st[k] = 2.0 * L * (dr.uniform() - 0.5);
    c.X(k, n, 0) = st[k];
    c.X(k, n, M - 1) = st[k];
  }
  const int mm = M - 2;
  double p[2] = {st[0], st[1]};
  for (int j = 1; j <= mm; ++j) {
    const double al = (double)(mm + 1 - j) / (double)(mm + 2 - j);
    const double sg = sqrt(2.0 * d.lambda * al * d.tau);
    double z[2];
    for (int k = 0; k < dim; ++k) z[k] = dr.normal();
    for (int k = 0; k < dim; ++k) {
      p[k] = al * p[k] + (1.0 - al) * st[k] + z[k] * sg;
      c.X(k, n, j) = p[k];
    }
  }
  for (int k = 0; k < dim; ++k)
    for (int j = 0; j < M; ++j) c.X(k, n, j) = teleport(c.X(k, n, j), L, inv2L);
  c.next[n] = n;
}

// init_world with a hard core (src/system.jl:44-64): one warp per chain, the
// particles in order.  Lane 0 draws a particle's start and Levy loop from the
// particle's own stream in k_init_world's order (so a particle that fits at
// once gets k_init_world's path); the warp then checks every bead against the
// beads of the earlier particles at its slice (norm of the per-component
// minimum-image distances below a).  A particle that overlaps is drawn again
// from its continuing stream, at most 10000 times, after which the chain gets
// ChainVar::err = DERR_INIT and the world is not made.
__global__ void k_init_world_hard(const ChainDesc *desc, ChainVar *var, double *dpool, int *ipool,
                                  int chain0) {
  const int ch = chain0 + blockIdx.x;
  const ChainDesc &d = desc[ch];
  if (!(d.flags & PF_HARD)) return;
  const int lane = threadIdx.x & 31;
  CV c = make_cv(&d, dpool, ipool, nullptr);
  const int N = d.N, M = d.M, dim = d.dim;
  const double L = d.L, inv2L = 1.0 / (2.0 * L);
  for (int n = 0; n < N; ++n) {
    GenDraws dr = gen_draws(make_stream(d, 0, PH_INIT, (unsigned)n));
    bool placed = false;
    for (int tries = 0; tries < 10000 && !placed; ++tries) {
      if (lane == 0) {
        double st[2] = {0.0, 0.0};
        for (int k = 0; k < dim; ++k) {
          st[k] = 2.0 * L * (dr.uniform() - 0.5);
          c.X(k, n, 0) = st[k];
          c.X(k, n, M - 1) = st[k];
        }
        const int mm = M - 2;
        double pp[2] = {st[0], st[1]};
        for (int j = 1; j <= mm; ++j) {
          const double al = (double)(mm + 1 - j) / (double)(mm + 2 - j);
          const double sg = sqrt(2.0 * d.lambda * al * d.tau);
          double z[2];
          for (int k = 0; k < dim; ++k) z[k] = dr.normal();
          for (int k = 0; k < dim; ++k) {
            pp[k] = al * pp[k] + (1.0 - al) * st[k] + z[k] * sg;
            c.X(k, n, j) = pp[k];
          }
        }
        for (int k = 0; k < dim; ++k)
          for (int j = 0; j < M; ++j) c.X(k, n, j) = teleport(c.X(k, n, j), L, inv2L);
      }
      __syncwarp();
      int hit = 0;
      for (int q = lane; q < M * n && !hit; q += 32) {
        const int j = q / n, i = q % n;
        double s2 = 0.0;
        for (int k = 0; k < dim; ++k) {
          const double dd = dist1(c.X(k, i, j), c.X(k, n, j), L);
          s2 = __dadd_rn(s2, __dmul_rn(dd, dd));
        }
        if (__dsqrt_rn(s2) < d.hard_a) hit = 1;
      }
      placed = !__any_sync(0xffffffffu, hit);
    }
    if (!placed) {
      if (lane == 0) var[ch].err = DERR_INIT;
      return;
    }
    if (lane == 0) c.next[n] = n;
    __syncwarp();
  }
}

// cached link actions V[j][n] = lnV(bead, next bead) and the 16-bit mirror
__global__ void k_links(const ChainDesc *desc, double *dpool, int *ipool, int chain0) {
  const ChainDesc &d = desc[chain0 + blockIdx.y];
  CV c = make_cv(&d, dpool, ipool, nullptr);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.N * d.M; k += gridDim.x * blockDim.x) {
    const int j = k / d.N, i = k % d.N;
    const int in = j == d.M - 1 ? c.next[i] : i, jn = j + 1 == d.M ? 0 : j + 1;
    const double ax = c.X(0, i, j), ay = c.Xd(1, i, j);
    const double bx = c.X(0, in, jn), by = c.Xd(1, in, jn);
    c.Vl(i, j) = -0.5 * d.tau * (vext(d, ax, ay) + vext(d, bx, by));
    c.xq[(size_t)j * c.ldn + i] = qpos(d, ax, ay);
  }
}

// the 16-bit mirror alone (after verbatim state uploads)
__global__ void k_mirror(const ChainDesc *desc, double *dpool, int chain0) {
  const ChainDesc &d = desc[chain0 + blockIdx.y];
  CV c = make_cv(&d, dpool, nullptr, nullptr);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.N * d.M; k += gridDim.x * blockDim.x) {
    const int j = k / d.N, i = k % d.N;
    c.xq[(size_t)j * c.ldn + i] = qpos(d, c.X(0, i, j), c.Xd(1, i, j));
  }
}

__global__ void __launch_bounds__(256) k_measure(const ChainDesc *desc, ChainVar *var, double *dpool,
                                                 int *ipool, unsigned long long *upool, int chain0) {
  __shared__ SmemCtl sc;
  __shared__ double red[256];
  const int ch = chain0 + blockIdx.x;
  if (threadIdx.x == 0) {
    sc.d = desc[ch];
    sc.v = var[ch];
  }
  __syncthreads();
  CV c = make_cv(&sc.d, dpool, ipool, upool);
  __shared__ unsigned long long qbuf[8 * PQ_CAP];
  __shared__ unsigned bits[(kMaxParticles + 31) / 32];
  if (sc.v.err != 0 || !next_is_permutation<false>(c.next, sc.d.N, bits)) {
    if (threadIdx.x == 0) {
      if (sc.v.err == 0) sc.v.err = DERR_STATE;
      var[ch] = sc.v;
    }
    return;
  }
  measure_group<false>(c, red, sc.e4, c.hist != nullptr, qbuf);
  if (threadIdx.x == 0) {
    record_measurement(sc.d, sc.v, c, sc.e4, c.hist != nullptr);
    var[ch] = sc.v;
  }
}

// ---------------------------------------------------------------------------
// adjoint of the potential action S_pot = -sum lnV - sum lnU:
// per-bead dS/dr and dS/d(V0, omega, g).  Bead-parallel over one chain;
// consecutive threads are consecutive particles of one slice, so the slice
// row they scan is shared.
// part[block][8]: S_ext, dV0, domega, S_pair, dg, pair virial, r.g_ext, 0
// ---------------------------------------------------------------------------
__device__ __forceinline__ double mi_signed(double a, double b, double L) {
  double s = a - b;
  if (s > L) s -= 2.0 * L;
  else if (s < -L) s += 2.0 * L;
  return s;
}

// adjoint terms of bead k (slice-major k = j N + i) of one chain: v[8] the
// block partials above, ga the bead's gradient from the external potential
// and from the pair terms of the link it starts, gb the gradient of the next
// bead of its path (in_, jn) from the pair terms of that link
__device__ __forceinline__ void adjoint_bead(const ChainDesc &d, const CV &c, int k, double omega,
                                             double (&v)[8], double (&ga)[2], double (&gb)[2]) {
  const int N = c.N, M = c.M, dim = c.dim;
  const int j = k / N, i = k % N;
  const int in = j == M - 1 ? c.next[i] : i, jn = j + 1 == M ? 0 : j + 1;
  const double tau = d.tau;
  const double ax = c.X(0, i, j), ay = c.Xd(1, i, j);
  const double anx = c.X(0, in, jn), any = c.Xd(1, in, jn);
  double ge[2];
  grad_vext(d, ax, ay, ge[0], ge[1]);
  ge[0] *= tau;
  ge[1] *= tau;
  v[0] = tau * vext(d, ax, ay);
  if (d.flags & PF_LATT) {
    const double sx = sinpi(ax * d.lat_k), sy = dim > 1 ? sinpi(ay * d.lat_k) : 0.0;
    v[1] = tau * (sx * sx + sy * sy);
  }
  if (d.flags & PF_HARM) v[2] = tau * omega * (ax * ax + ay * ay);
  v[6] = ax * ge[0] + ay * ge[1];
  double go[2] = {0.0, 0.0}, gn[2] = {0.0, 0.0};
  if (d.flags & PF_PAIR) {
    const double rc2 = d.rc * d.rc, cg = d.inv2s2, h = 0.5 * tau;
    Prefilter f;
    f.init_q(c.Q(i, j), d.q_lim_rc);
    const unsigned *row = c.xq + (size_t)j * c.ldn;
    for (int b = 0; b < N; ++b) {
      if (b == i || !f.pass(row[b])) continue;
      const double bxv = c.X(0, b, j), byv = c.Xd(1, b, j);
      const double d1x = mi_signed(ax, bxv, d.L), d1y = dim > 1 ? mi_signed(ay, byv, d.L) : 0.0;
      const double r2a = mi2(d, ax, ay, bxv, byv);
      if (r2a > rc2) continue;
      const int bn = j == M - 1 ? c.next[b] : b;
      const double bnx = c.X(0, bn, jn), bny = c.Xd(1, bn, jn);
      const double d2x = mi_signed(anx, bnx, d.L), d2y = dim > 1 ? mi_signed(any, bny, d.L) : 0.0;
      const double r2b = mi2(d, anx, any, bnx, bny);
      const double e1 = exp_neg(-r2a * cg), e2 = exp_neg(-r2b * cg);
      const double v1 = d.g * e1, v2 = d.g * e2;
      go[0] += h * (-2.0 * cg * v1) * d1x;
      go[1] += h * (-2.0 * cg * v1) * d1y;
      gn[0] += h * (-2.0 * cg * v2) * d2x;
      gn[1] += h * (-2.0 * cg * v2) * d2y;
      // each unordered pair is visited from both sides
      v[3] += 0.5 * h * (v1 + v2);
      v[4] += 0.5 * h * (e1 + e2);
      v[5] += 0.5 * h * (-2.0 * cg) * (r2a * v1 + r2b * v2);
    }
  }
  ga[0] = ge[0] + go[0];
  ga[1] = ge[1] + go[1];
  gb[0] = gn[0];
  gb[1] = gn[1];
}

__global__ void __launch_bounds__(256) k_adjoint_beads(AdjArgs a) {
  __shared__ double red[256];
  __shared__ ChainDesc d;
  if (threadIdx.x == 0) d = a.desc[a.chain];
  __syncthreads();
  CV c = make_cv(&d, a.dpool, a.ipool, nullptr);
  const int N = c.N, M = c.M;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (k < N * M) {
    double ga[2], gb[2];
    adjoint_bead(d, c, k, a.omega, v, ga, gb);
    // per-bead buffers in the chain's [i][j] order (k2 = i*M + j)
    const int j = k / N, i = k % N;
    const size_t k2 = (size_t)i * M + j;
    for (int q = 0; q < 2; ++q) {
      a.gA[k2 * 2 + q] = ga[q];
      a.gB[k2 * 2 + q] = gb[q];
    }
  }
  block_sum_k<8>(v, red);
  if (threadIdx.x == 0)
    for (int q = 0; q < 8; ++q) a.part[(size_t)blockIdx.x * 8 + q] = v[q];
}

__global__ void k_inverse_next(AdjArgs a) {
  const ChainDesc &d = a.desc[a.chain];
  const int *next = a.ipool + d.next_off;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.N; i += gridDim.x * blockDim.x)
    a.inv[next[i]] = i;
}

__global__ void __launch_bounds__(256) k_adjoint_finish(AdjArgs a) {
  __shared__ double red[256];
  __shared__ ChainDesc d;
  if (threadIdx.x == 0) d = a.desc[a.chain];
  __syncthreads();
  CV c = make_cv(&d, a.dpool, a.ipool, nullptr);
  const int N = c.N, M = c.M, dim = c.dim;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;  // k = i*M + j
  double rg[1] = {0.0};
  if (k < N * M) {
    const int i = k / M, j = k % M;
    const int kp = j > 0 ? k - 1 : a.inv[i] * M + (M - 1);
    for (int q = 0; q < dim; ++q) {
      const double g = a.gA[(size_t)k * 2 + q] + a.gB[(size_t)kp * 2 + q];
      if (a.dSdr) a.dSdr[(size_t)q * N * M + k] = g;
      rg[0] += c.X(q, i, j) * g;
    }
  }
  block_sum_k<1>(rg, red);
  if (threadIdx.x == 0) atomicAdd(a.sum_rg, rg[0]);
  if (blockIdx.x == 0) {
    double t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = threadIdx.x; b < a.nblocks; b += blockDim.x)
      for (int q = 0; q < 8; ++q) t[q] += a.part[(size_t)b * 8 + q];
    block_sum_k<8>(t, red);
    if (threadIdx.x == 0)
      for (int q = 0; q < 8; ++q) a.totals[q] = t[q];
  }
}

// ---------------------------------------------------------------------------
// batched adjoint: every chain of a batch in one launch per stage.  Blocks of
// 256 beads are laid out chain after chain (blk_first[c] is chain c's first
// block, blk_chain[b] the chain of block b), so one grid covers chains of any
// size; each block works on one chain only and writes its partial sums to
// its own row of part, which k_adjoint_totals_b reduces per chain.
// ---------------------------------------------------------------------------
__global__ void k_adjoint_inv_b(AdjBatchArgs a) {
  const int ch = blockIdx.y;
  const ChainDesc &d = a.desc[ch];
  const int *next = a.ipool + d.next_off;
  int *inv = a.inv + a.inv_off[ch];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.N; i += gridDim.x * blockDim.x)
    inv[next[i]] = i;
}

__global__ void __launch_bounds__(256) k_adjoint_beads_b(AdjBatchArgs a) {
  __shared__ double red[256];
  __shared__ ChainDesc d;
  __shared__ int ch, lb;
  if (threadIdx.x == 0) {
    ch = a.blk_chain[blockIdx.x];
    lb = blockIdx.x - a.blk_first[ch];
    d = a.desc[ch];
  }
  __syncthreads();
  CV c = make_cv(&d, a.dpool, a.ipool, nullptr);
  const int N = c.N, M = c.M;
  const int k = lb * blockDim.x + threadIdx.x;
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (k < N * M) {
    double ga[2], gb[2];
    adjoint_bead(d, c, k, a.omega[ch], v, ga, gb);
    const int j = k / N, i = k % N;
    const size_t k2 = (size_t)a.bead_off[ch] + (size_t)i * M + j;
    for (int q = 0; q < 2; ++q) {
      a.gA[k2 * 2 + q] = ga[q];
      a.gB[k2 * 2 + q] = gb[q];
    }
  }
  block_sum_k<8>(v, red);
  if (threadIdx.x == 0)
    for (int q = 0; q < 8; ++q) a.part[(size_t)blockIdx.x * 9 + q] = v[q];
}

// the pair terms and the external potential of one slice of one chain per
// CTA (blocks slice_first[c] .. slice_first[c] + M - 1 are chain c's slices):
// warps take particles i, lanes scan the higher-numbered partners b of the
// slice through the mirror prefilter and queue the survivors, and every
// queued pair is evaluated once in FP64, 32 at a time on full warps; its
// force goes to both particles through accumulators in shared memory
// (4 doubles per particle: the bead's gradient from the link it starts, and
// the gradient of its next bead from the same link).  Needs 32 N bytes of
// dynamic shared memory.  The accumulators add the pair forces in the order
// the atomics land, so results repeat to rounding, not bit for bit.  Partial
// sums to part_s[cta][8] as k_adjoint_beads.
__global__ void __launch_bounds__(256) k_adjoint_slice_b(AdjBatchArgs a) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ double red[256];
  __shared__ ChainDesc d;
  __shared__ int ch, j;
  __shared__ unsigned long long qbuf[8 * PQ_CAP];
  if (threadIdx.x == 0) {
    int lo = 0, hi = a.nchains;  // slice_first[lo] <= blockIdx.x < slice_first[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (a.slice_first[mid] <= (int)blockIdx.x) lo = mid; else hi = mid;
    }
    ch = lo;
    j = blockIdx.x - a.slice_first[lo];
    d = a.desc[lo];
  }
  __syncthreads();
  CV c = make_cv(&d, a.dpool, a.ipool, nullptr);
  const int N = c.N, M = c.M, dim = c.dim, jn = j + 1 == M ? 0 : j + 1;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = nt >> 5;
  double *acc = reinterpret_cast<double *>(dsm);  // [4][N]: ga.x, ga.y, gb.x, gb.y
  for (int e = tid; e < 4 * N; e += nt) acc[e] = 0.0;
  __syncthreads();
  const double tau = d.tau;
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (d.flags & PF_PAIR) {
    const double cg = d.inv2s2, h = 0.5 * tau, rc2 = d.rc * d.rc;
    unsigned long long *q = qbuf + (size_t)warp * PQ_CAP;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned *row = c.xq + (size_t)j * c.ldn;
    int qn = 0;
    auto flush = [&]() {
      const int k = qn < 32 ? qn : 32;
      if (lane < k) {
        const unsigned long long e = q[lane];
        const int i = (int)(e >> 32), b = (int)(e & 0xffffffffu);
        const double ax = c.X(0, i, j), ay = c.Xd(1, i, j);
        const double bx = c.X(0, b, j), by = c.Xd(1, b, j);
        const double r2a = mi2(d, ax, ay, bx, by);
        if (r2a <= rc2) {
          const int in = j == M - 1 ? c.next[i] : i, bn = j == M - 1 ? c.next[b] : b;
          const double anx = c.X(0, in, jn), any = c.Xd(1, in, jn);
          const double bnx = c.X(0, bn, jn), bny = c.Xd(1, bn, jn);
          const double d1x = mi_signed(ax, bx, d.L), d1y = dim > 1 ? mi_signed(ay, by, d.L) : 0.0;
          const double d2x = mi_signed(anx, bnx, d.L), d2y = dim > 1 ? mi_signed(any, bny, d.L) : 0.0;
          const double r2b = mi2(d, anx, any, bnx, bny);
          const double e1 = exp_neg(-r2a * cg), e2 = exp_neg(-r2b * cg);
          const double v1 = d.g * e1, v2 = d.g * e2;
          const double f1 = h * (-2.0 * cg * v1), f2 = h * (-2.0 * cg * v2);
          atomicAdd(&acc[i], f1 * d1x);
          atomicAdd(&acc[b], -f1 * d1x);
          atomicAdd(&acc[2 * N + i], f2 * d2x);
          atomicAdd(&acc[2 * N + b], -f2 * d2x);
          if (dim > 1) {
            atomicAdd(&acc[N + i], f1 * d1y);
            atomicAdd(&acc[N + b], -f1 * d1y);
            atomicAdd(&acc[3 * N + i], f2 * d2y);
            atomicAdd(&acc[3 * N + b], -f2 * d2y);
          }
          v[3] += h * (v1 + v2);
          v[4] += h * (e1 + e2);
          v[5] += h * (-2.0 * cg) * (r2a * v1 + r2b * v2);
        }
      }
      __syncwarp();
      unsigned long long rest[2];
      const int nr = qn - k;
      for (int r = 0; r < 2; ++r) rest[r] = (lane + 32 * r < nr) ? q[32 + lane + 32 * r] : 0ull;
      __syncwarp();
      for (int r = 0; r < 2; ++r)
        if (lane + 32 * r < nr) q[lane + 32 * r] = rest[r];
      __syncwarp();
      qn = nr;
    };
    for (int i = warp; i < N; i += nwarps) {
      Prefilter f;
      f.init_q(row[i], d.q_lim_rc);
      for (int b0 = i + 1; b0 < N; b0 += 32) {
        const int b = b0 + lane;
        const bool p = b < N && f.pass(row[b]);
        const unsigned mk = __ballot_sync(0xffffffffu, p);
        if (p) q[qn + __popc(mk & lt)] = ((unsigned long long)(unsigned)i << 32) | (unsigned)b;
        qn += __popc(mk);
        __syncwarp();
        if (qn >= 32) flush();
      }
    }
    while (qn > 0) flush();
  }
  __syncthreads();
  // the external potential per bead, and the per-bead buffers in the
  // chain's [i][j] order (k2 = i M + j)
  for (int i = tid; i < N; i += nt) {
    const double ax = c.X(0, i, j), ay = c.Xd(1, i, j);
    double ge[2];
    grad_vext(d, ax, ay, ge[0], ge[1]);
    ge[0] *= tau;
    ge[1] *= tau;
    v[0] += tau * vext(d, ax, ay);
    if (d.flags & PF_LATT) {
      const double sx = sinpi(ax * d.lat_k), sy = dim > 1 ? sinpi(ay * d.lat_k) : 0.0;
      v[1] += tau * (sx * sx + sy * sy);
    }
    if (d.flags & PF_HARM) v[2] += tau * a.omega[ch] * (ax * ax + ay * ay);
    v[6] += ax * ge[0] + ay * ge[1];
    const size_t k2 = (size_t)a.bead_off[ch] + (size_t)i * M + j;
    a.gA[k2 * 2] = ge[0] + acc[i];
    a.gA[k2 * 2 + 1] = ge[1] + acc[N + i];
    a.gB[k2 * 2] = acc[2 * N + i];
    a.gB[k2 * 2 + 1] = acc[3 * N + i];
  }
  block_sum_k<8>(v, red);
  if (tid == 0)
    for (int q = 0; q < 8; ++q) a.part_s[(size_t)blockIdx.x * 8 + q] = v[q];
}

// per bead the full gradient gA[k] + gB[prev(k)]: dS/dr (host layout
// x[d][n][j] of the chain at desc.host_off, when requested) and r . dS/dr
__global__ void __launch_bounds__(256) k_adjoint_finish_b(AdjBatchArgs a) {
  __shared__ double red[256];
  __shared__ int ch, lb;
  if (threadIdx.x == 0) {
    ch = a.blk_chain[blockIdx.x];
    lb = blockIdx.x - a.blk_first[ch];
  }
  __syncthreads();
  const ChainDesc &d = a.desc[ch];
  const int N = d.N, M = d.M, dim = d.dim;
  const double *x = a.dpool + d.x_off;
  const int k = lb * blockDim.x + threadIdx.x;  // k = i*M + j
  double rg[1] = {0.0};
  if (k < N * M) {
    const int i = k / M, j = k % M;
    const size_t base = (size_t)a.bead_off[ch];
    const int kp = j > 0 ? k - 1 : a.inv[a.inv_off[ch] + i] * M + (M - 1);
    for (int q = 0; q < dim; ++q) {
      const double g = a.gA[(base + k) * 2 + q] + a.gB[(base + kp) * 2 + q];
      if (a.dSdr) a.dSdr[(size_t)d.host_off + (size_t)q * N * M + k] = g;
      rg[0] += x[((size_t)j * N + i) * dim + q] * g;
    }
  }
  block_sum_k<1>(rg, red);
  if (threadIdx.x == 0) a.part[(size_t)blockIdx.x * 9 + 8] = rg[0];
}

// totals[c][9]: the partial rows of chain c's blocks summed (its slice CTAs'
// rows when the slice kernel ran)
__global__ void __launch_bounds__(256) k_adjoint_totals_b(AdjBatchArgs a) {
  __shared__ double red[256];
  const int ch = blockIdx.x;
  const int b0 = a.blk_first[ch];
  const int b1 = ch + 1 < a.nchains ? a.blk_first[ch + 1] : a.nblocks;
  double t[8] = {0, 0, 0, 0, 0, 0, 0, 0}, r[1] = {0.0};
  for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
    if (!a.use_slices)
      for (int q = 0; q < 8; ++q) t[q] += a.part[(size_t)b * 9 + q];
    r[0] += a.part[(size_t)b * 9 + 8];
  }
  if (a.use_slices) {
    const int s0 = a.slice_first[ch], s1 = s0 + a.desc[ch].M;
    for (int b = s0 + threadIdx.x; b < s1; b += blockDim.x)
      for (int q = 0; q < 8; ++q) t[q] += a.part_s[(size_t)b * 8 + q];
  }
  block_sum_k<8>(t, red);
  block_sum_k<1>(r, red);
  if (threadIdx.x == 0) {
    for (int q = 0; q < 8; ++q) a.totals[(size_t)ch * 9 + q] = t[q];
    a.totals[(size_t)ch * 9 + 8] = r[0];
  }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

// scratch sizes of the device move routines, for the host's shared-memory plans
size_t swap_scratch_bytes(int N, int nwarps) { return SwapScratch::bytes(N, nwarps); }
size_t com_scratch_bytes(int N, int M, int nwarps) { return ComScratch::bytes(N, M, nwarps); }
int window_scratch_doubles() { return WARP_SCRATCH_D; }

// the exp table of exp_neg for the current device, in every kernel unit
cudaError_t upload_exp_table() {
  static double tab[EXPTAB_N + 1];
  for (int k = 0; k <= EXPTAB_N; ++k) tab[k] = std::exp(-k / 64.0);
  cudaError_t e = tu_upload_exp_table(tab, sizeof(tab));
  if (e == cudaSuccess) e = swap_upload_exp_table(tab, sizeof(tab));
  if (e == cudaSuccess) e = fused_upload_exp_table(tab, sizeof(tab));
  if (e == cudaSuccess) e = attempt_upload_exp_table(tab, sizeof(tab));
  return e;
}

// phase kernels: 0 staging, 1 swaps (pimc_swap.cu), 2 the rest; warp = 1
// (swaps only): one warp per chain; spec = 1 (swaps in CTA mode): the
// reference-rules swap kernel
static const void *phase_kernel(int phase, int warp, int spec, int regs) {
  if (phase == 1) return swap_kernel(warp, spec, regs);
  return phase == 0 ? (const void *)k_sweep_stage : (const void *)k_sweep_rest;
}
cudaError_t launch_sweep_phase(const SweepArgs &a, int phase, int warp, int spec, int regs,
                               int grid, int block, size_t smem, cudaStream_t s) {
  if (phase == 1) return launch_swap(a, warp, spec, regs, grid, block, smem, s);
  if (phase == 0) k_sweep_stage<<<grid, block, smem, s>>>(a);
  else k_sweep_rest<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t sweep_phase_set_smem(int phase, int warp, int spec, int regs, size_t smem) {
  return cudaFuncSetAttribute(phase_kernel(phase, warp, spec, regs),
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t sweep_phase_occupancy(int phase, int warp, int spec, int regs, int block, size_t smem,
                                  int *blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      blocks_per_sm, phase_kernel(phase, warp, spec, regs), block, smem);
}

size_t sweep_ctl_bytes() { return (sizeof(SmemCtl) + 15) & ~(size_t)15; }
cudaError_t launch_import(const ChainDesc *desc, double *dpool, const double *src, int chain0,
                          int nchains, size_t maxn, cudaStream_t s) {
  dim3 g((unsigned)std::min<size_t>((maxn + 255) / 256, 1024), nchains);
  k_import<<<g, 256, 0, s>>>(desc, dpool, src, chain0);
  return cudaGetLastError();
}
cudaError_t launch_export(const ChainDesc *desc, const double *dpool, double *dst, int chain0,
                          int nchains, size_t maxn, cudaStream_t s) {
  dim3 g((unsigned)std::min<size_t>((maxn + 255) / 256, 1024), nchains);
  k_export<<<g, 256, 0, s>>>(desc, dpool, dst, chain0);
  return cudaGetLastError();
}
cudaError_t launch_transpose_tiles(bool import, const ChainDesc *desc, double *dpool,
                                   double *host, const int *tile_off, int c_lo, int c_hi,
                                   int ntiles, int grid, cudaStream_t s) {
  const int g = std::max(1, std::min(grid, ntiles));
  if (import) k_transpose_tiles<true><<<g, 256, 0, s>>>(desc, dpool, host, tile_off, c_lo, c_hi);
  else k_transpose_tiles<false><<<g, 256, 0, s>>>(desc, dpool, host, tile_off, c_lo, c_hi);
  return cudaGetLastError();
}
cudaError_t launch_init_world(const ChainDesc *desc, double *dpool, int *ipool, int chain0,
                              int nchains, int maxN, cudaStream_t s) {
  dim3 g((maxN + 127) / 128, nchains);
  k_init_world<<<g, 128, 0, s>>>(desc, dpool, ipool, chain0);
  return cudaGetLastError();
}
cudaError_t launch_init_world_hard(const ChainDesc *desc, ChainVar *var, double *dpool, int *ipool,
                                   int chain0, int nchains, cudaStream_t s) {
  k_init_world_hard<<<nchains, 32, 0, s>>>(desc, var, dpool, ipool, chain0);
  return cudaGetLastError();
}
cudaError_t launch_links(const ChainDesc *desc, double *dpool, int *ipool, int chain0, int nchains,
                         int maxNM, cudaStream_t s) {
  dim3 g((unsigned)std::min((maxNM + 255) / 256, 1024), nchains);
  k_links<<<g, 256, 0, s>>>(desc, dpool, ipool, chain0);
  return cudaGetLastError();
}
cudaError_t launch_mirror(const ChainDesc *desc, double *dpool, int chain0, int nchains, int maxNM,
                          cudaStream_t s) {
  dim3 g((unsigned)std::min((maxNM + 255) / 256, 1024), nchains);
  k_mirror<<<g, 256, 0, s>>>(desc, dpool, chain0);
  return cudaGetLastError();
}
cudaError_t launch_measure(const ChainDesc *desc, ChainVar *var, double *dpool, int *ipool,
                           unsigned long long *upool, int chain0, int nchains, cudaStream_t s) {
  k_measure<<<nchains, 256, 0, s>>>(desc, var, dpool, ipool, upool, chain0);
  return cudaGetLastError();
}
// ---------------------------------------------------------------------------
// contact-interaction propagator table (build_prop_int, src/propagator.jl:35-89):
// T(r1, r2) = -I1 - I2 + I3 on the reference's 600 x 600 grid r = 1e-20 + i h,
// with I = (1/2pi) int_0^inf k exp(-tau k^2) w(k) (Bessel products) dk
// (Gautier et al., supplementary S28), t(k) = 1/((2/pi)(gamma + log(k/2)) - 4/g0):
//   I1: w = t^2/(1+t^2), J0(k r1) J0(k r2)
//   I2: w = t/(1+t^2),   J0(k r1) Y0(k r2) + J0(k r2) Y0(k r1)
//   I3: w = t^2/(1+t^2), Y0(k r1) Y0(k r2)
// Composite 8-point Gauss-Legendre in FP64: geometric panels from 1e-10 to 0.5
// (the log behaviour at k -> 0), then uniform panels of a quarter of the
// shortest oscillation period up to K with exp(-tau K^2) = 1e-18.  CUDA's j0 /
// y0 are library calls.  One thread per entry of the upper triangle.
// ---------------------------------------------------------------------------
struct ContactQuad {
  double tau, g0, K, k0, du;
  int ngraded, nuniform;
};

// the integrand of the three Bessel integrals (Gautier et al., supplementary
// S28; src/propagator.jl:50-64) combined, T = (-I1 - I2 + I3) / (2 pi).  With
// t(k) = 1/s(k), s = (2/pi)(gamma + log(k/2)) - 4/g0, the weights
// t^2/(1+t^2) = 1/(1+s^2) and t/(1+t^2) = s/(1+s^2) are taken in s, which
// stays finite where t has its pole.
__device__ __forceinline__ double contact_integrand(double k, double r1, double r2, const ContactQuad &q) {
  const double sk = (2.0 / 3.141592653589793) * (0.5772156649015329 + log(0.5 * k)) - 4.0 / q.g0;
  const double den = 1.0 / (1.0 + sk * sk), wa = den, wb = sk * den;
  const double J1 = j0(k * r1), J2 = j0(k * r2), Y1 = y0(k * r1), Y2 = y0(k * r2);
  return k * exp(-q.tau * k * k) * (-wa * J1 * J2 - wb * (J1 * Y2 + J2 * Y1) + wa * Y1 * Y2);
}

__device__ double contact_entry(double r1, double r2, const ContactQuad &q) {
  const double xs[4] = {0.18343464249564978, 0.525532409916329, 0.7966664774136267, 0.9602898564975362};
  const double ws[4] = {0.36268378337836166, 0.3137066458778869, 0.22238103445337443, 0.10122853629037706};
  double sum = 0.0;
  auto panel = [&](double a, double b) {
    const double c = 0.5 * (a + b), hw = 0.5 * (b - a);
    double ps = 0.0;
    for (int i = 0; i < 4; ++i)
      ps += ws[i] * (contact_integrand(c - hw * xs[i], r1, r2, q) + contact_integrand(c + hw * xs[i], r1, r2, q));
    sum += hw * ps;
  };
  double a = 1e-10;
  for (int p = 0; p < q.ngraded; ++p) {
    const double b = p + 1 == q.ngraded ? q.k0 : 2.0 * a;
    panel(a, b);
    a = b;
  }
  for (int p = 0; p < q.nuniform; ++p) panel(q.k0 + p * q.du, q.k0 + (p + 1) * q.du);
  return sum / (2.0 * 3.141592653589793);
}

__global__ void k_contact_table(double *tab, int n, double r0, double h, ContactQuad q) {
  const long long ntri = (long long)n * (n + 1) / 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ntri;
       e += (long long)gridDim.x * blockDim.x) {
    // row i1 of the upper triangle holds n - i1 entries
    int i1 = (int)((2.0 * n + 1.0 - sqrt((2.0 * n + 1.0) * (2.0 * n + 1.0) - 8.0 * (double)e)) / 2.0);
    if (i1 < 0) i1 = 0;
    while (i1 > 0 && (long long)i1 * (2 * n - i1 + 1) / 2 > e) --i1;
    while ((long long)(i1 + 1) * (2 * n - i1) / 2 <= e) ++i1;
    const int i2 = i1 + (int)(e - (long long)i1 * (2 * n - i1 + 1) / 2);
    const double v = contact_entry(r0 + i1 * h, r0 + i2 * h, q);
    tab[(size_t)i1 * n + i2] = v;
    tab[(size_t)i2 * n + i1] = v;
  }
}

cudaError_t launch_contact_table(double *dtab, int n, double range, double g0, double tau,
                                 cudaStream_t s) {
  ContactQuad q;
  q.tau = tau;
  q.g0 = g0;
  q.K = sqrt(41.5 / tau);
  q.k0 = 0.5;
  q.ngraded = 33;  // 1e-10 * 2^32 > 0.5
  // the Bessel products oscillate with period >= 2 pi / (2 range): quarter
  // periods per panel
  const double period = 2.0 * 3.141592653589793 / (2.0 * range);
  q.nuniform = (int)ceil((q.K - q.k0) / (0.25 * period));
  if (q.nuniform < 1) q.nuniform = 1;
  q.du = (q.K - q.k0) / q.nuniform;
  const double r0 = 1e-20, h = (range - r0) / (n - 1);
  const long long ntri = (long long)n * (n + 1) / 2;
  const int blocks = (int)std::min<long long>((ntri + 127) / 128, 65535);
  k_contact_table<<<blocks, 128, 0, s>>>(dtab, n, r0, h, q);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP64 pipe throughput probe: eight independent DFMA chains per thread
// ---------------------------------------------------------------------------
static __device__ double g_fp64_sink[256];

__global__ void __launch_bounds__(256) k_fp64_peak(int iters, double b, double c) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = 1.0 + 1e-3 * k + 1e-9 * threadIdx.x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == -1.0) g_fp64_sink[threadIdx.x] = s;  // never true; keeps the chains live
}

cudaError_t fp64_peak(int num_sms, cudaStream_t st, double *tflops) {
  const int iters = 1 << 14, blocks = num_sms * 8, threads = 256;
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e != cudaSuccess) return e;
  e = cudaEventCreate(&e1);
  if (e != cudaSuccess) {
    cudaEventDestroy(e0);
    return e;
  }
  float best = 1e30f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
    cudaEventRecord(e0, st);
    k_fp64_peak<<<blocks, threads, 0, st>>>(iters, 0.9999999, 1e-7);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && ms < best) best = ms;  // rep 0 warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return e;
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// adjoint scratch in static device memory (pimc_adjoint_noalloc): room for a
// chain of up to kNoAllocBeads beads and kNoAllocParticles particles in the
// layout of the allocating adjoint (gA, gB, partials, totals, dS/dr, inverse
// permutation), 3.2 MB per device
// ---------------------------------------------------------------------------
static __device__ __align__(256) double g_adj_static[kNoAllocDoubles];

// The array's device address, per device, in an atomic slot.  Handle
// creation takes it (with the handle's device current: the set-up) and every
// later creation on that device takes it again, so the slot always holds the
// address in the device's current context: a cudaDeviceReset destroys the
// handles made before it, and the first handle made after it refreshes the
// slot before any call can use it.  Concurrent set-ups store the same value;
// readers never see a half-written entry.
namespace {
constexpr int kMaxDevices = 64;
std::atomic<double *> g_adj_addr[kMaxDevices];
}  // namespace

cudaError_t adjoint_static_setup() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  void *p = nullptr;
  e = cudaGetSymbolAddress(&p, g_adj_static);
  if (e != cudaSuccess) return e;
  g_adj_addr[dev].store(static_cast<double *>(p), std::memory_order_release);
  return cudaSuccess;
}

cudaError_t adjoint_static_scratch(double **ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  double *a = g_adj_addr[dev].load(std::memory_order_acquire);
  if (!a) {
    e = adjoint_static_setup();
    if (e != cudaSuccess) return e;
    a = g_adj_addr[dev].load(std::memory_order_acquire);
  }
  *ptr = a;
  return cudaSuccess;
}

// the PIMC_PROFILE build's swap counters (g_prof of every kernel unit,
// summed): read, then cleared on request; cudaErrorNotSupported in other
// builds
cudaError_t profile_take(unsigned long long *out, bool reset, cudaStream_t s) {
#if PIMC_PROFILE
  for (int k = 0; k < 32; ++k) out[k] = 0;
  cudaError_t e = tu_profile_take(out, reset, s);
  if (e == cudaSuccess) e = swap_profile_take(out, reset, s);
  if (e == cudaSuccess) e = fused_profile_take(out, reset, s);
  if (e == cudaSuccess) e = attempt_profile_take(out, reset, s);
  return e;
#else
  (void)out;
  (void)reset;
  (void)s;
  return cudaErrorNotSupported;
#endif
}

// the PIMC_CHECK build's device check word of every kernel unit (the first
// nonzero): read and cleared (0 in the default build, which has no bounds
// checks)
cudaError_t check_word_take(cudaStream_t s, unsigned long long *w) {
  cudaError_t (*const take[3])(cudaStream_t, unsigned long long *) = {
      swap_check_word_take, fused_check_word_take, attempt_check_word_take};
  cudaError_t e = tu_check_word_take(s, w);
  for (int u = 0; u < 3 && e == cudaSuccess; ++u) {
    unsigned long long w2 = 0;
    e = take[u](s, &w2);
    if (*w == 0) *w = w2;
  }
  return e;
}

cudaError_t launch_adjoint_batch(const AdjBatchArgs &a, int maxN, cudaStream_t s) {
  dim3 gi((unsigned)std::max(1, (maxN + 255) / 256), (unsigned)a.nchains);
  k_adjoint_inv_b<<<gi, 256, 0, s>>>(a);
  if (a.use_slices) {
    const size_t sm = 32 * (size_t)maxN;
    cudaError_t e = cudaFuncSetAttribute(k_adjoint_slice_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_adjoint_slice_b<<<a.nslices, 256, sm, s>>>(a);
  } else {
    k_adjoint_beads_b<<<a.nblocks, 256, 0, s>>>(a);
  }
  k_adjoint_finish_b<<<a.nblocks, 256, 0, s>>>(a);
  k_adjoint_totals_b<<<a.nchains, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adjoint(const AdjArgs &a, int nbeads, cudaStream_t s) {
  const int nb = (nbeads + 255) / 256;
  k_inverse_next<<<4, 256, 0, s>>>(a);
  k_adjoint_beads<<<nb, 256, 0, s>>>(a);
  k_adjoint_finish<<<nb, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace pimc
