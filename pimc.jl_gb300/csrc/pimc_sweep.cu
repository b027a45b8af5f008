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

#include "pimc_kernels.cuh"
#include "pimc_launch.h"

namespace pimc {

__device__ __forceinline__ CV make_cv(const ChainDesc *d, double *dpool, int *ipool,
                                      unsigned long long *upool) {
  CV c;
  c.d = d;
  c.N = d->N;
  c.M = d->M;
  c.dim = d->dim;
  c.ldn = d->N;
  c.x = dpool + d->x_off;
  c.V = dpool + d->V_off;
  c.xq = (unsigned *)(dpool + d->xq_off);
  c.next = ipool + d->next_off;
  c.tab = (const double2 *)(dpool + d->tab_off);
  c.hist = (d->dens_off >= 0 && upool) ? upool + d->dens_off : nullptr;
  c.eser = d->eser_off >= 0 ? dpool + d->eser_off : nullptr;
  return c;
}

// moves whose acceptance depends on other paths at the same slice
__device__ __forceinline__ bool chain_serial_local(const ChainDesc &d) {
  return ((d.flags & PF_PAIR) && (d.flags & PF_PHYS)) || (d.flags & PF_HARD);
}

// next[] of a chain must be a permutation of 0..N-1: every value in range
// (the host refuses out-of-range values before they reach the device) and no
// value twice.  The group marks each value in a bitmap of (N + 31) / 32 words
// of shared memory; a chain that fails gets ChainVar::err = DERR_STATE and is
// skipped by every kernel until its state is replaced.
template <bool WARP>
__device__ bool next_is_permutation(const int *next, int N, unsigned *bits) {
  const int tid = WARP ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
  const int nt = WARP ? 32 : (int)blockDim.x;
  const int nw = (N + 31) >> 5;
  for (int w = tid; w < nw; w += nt) bits[w] = 0u;
  if (WARP) __syncwarp(); else __syncthreads();
  int bad = 0;
  for (int i = tid; i < N; i += nt) {
    const int v = next[i];
    if (v < 0 || v >= N) {
      bad = 1;
    } else {
      const unsigned m = 1u << (v & 31);
      if (atomicOr(&bits[v >> 5], m) & m) bad = 1;
    }
  }
  return WARP ? !__any_sync(0xffffffffu, bad) : !__syncthreads_or(bad);
}

__device__ void record_measurement(const ChainDesc &d, ChainVar &v, const CV &c, const double *e,
                                   bool density) {
  if (c.eser && v.eser_count < (unsigned long long)d.eser_cap) {
    for (int q = 0; q < NOBS; ++q) c.eser[v.eser_count * NOBS + q] = e[q];
    v.eser_count++;
  }
  for (int q = 0; q < NOBS; ++q) {
    v.esum[q] += e[q];
    v.esum2[q] += e[q] * e[q];
  }
  v.n_meas++;
  if (d.rdf_nb > 0) v.rdf_meas++;
  if (density) v.ndata += d.M;
}

// adjust! (src/updates/helper.jl:22-52) from this sweep's acceptance
__device__ void adapt_slices(int &m, double acc_ratio, int mn, int mx, double minacc,
                             double maxacc) {
  if (acc_ratio < minacc) m -= 1;
  else if (acc_ratio > maxacc) m += 1;
  m = max(mn, m);
  m = min(mx, m);
}
__device__ void adapt_step(double &s, double acc_ratio, double mn, double mx, double minacc,
                           double maxacc) {
  if (acc_ratio < minacc) s *= 0.9;
  else if (acc_ratio > maxacc) s *= 1.1;
  s = fmax(mn, s);
  s = fmin(mx, s);
}

struct SmemCtl {
  ChainDesc d;
  ChainVar v;
  MixDev mix;
  double shift[2];
  double e4[NOBS];
  int iflag[8];
  int chain;
  int scratch_bytes;  // bytes of shared scratch the group's moves may carve
};

// bytes of dynamic shared memory of the running launch
__device__ __forceinline__ unsigned dyn_smem_bytes() {
  unsigned r;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
  return r;
}

// one sweep of one chain by a group: the whole CTA, or one warp on its own
// the phases of a sweep; a kernel runs the ones its mask names, so that each
// phase can run as its own launch with its own register budget
enum : int { SW_STAGE = 1, SW_SWAP = 2, SW_REST = 4, SW_ALL = 7 };

// closes one phase of move kind q: adds its tallies (attempts, accepts,
// skips, bead updates) to the chain's counters and adapts the phase's own
// variable (adjust!, src/updates/helper.jl:22-52) from this sweep's
// acceptance.  Only the phase itself reads that variable, so adapting at its
// end is the same as adapting at the end of the sweep.
template <bool WARP>
__device__ void close_phase(SmemCtl &sc, double *red, int q, double (&t)[4]) {
  using G = Group<WARP>;
  G::template sum<4>(t, red);
  if (G::rank() == 0) {
    ChainVar &v = sc.v;
    const MixDev &mix = sc.mix;
    v.att[q] += (unsigned long long)t[0];
    v.acc[q] += (unsigned long long)t[1];
    v.skips += (unsigned long long)t[2];
    v.bead_updates += t[3];
    v.beads_kind[q] += t[3];
    // the reference divides by an empty queue (NaN) and leaves var alone
    if (mix.adapt && t[0] > 0) {
      const double r = t[1] / t[0];
      if (q == MV_STAGE)
        adapt_slices(v.stage_m, r, mix.stage_min, mix.stage_max, mix.stage_minacc, mix.stage_maxacc);
      else if (q == MV_SWAP)
        adapt_slices(v.swap_m, r, mix.swap_min, mix.swap_max, mix.swap_minacc, mix.swap_maxacc);
      else if (q == MV_COM)
        adapt_step(v.com_step, r, mix.com_minstep, mix.com_maxstep, mix.com_minacc, mix.com_maxacc);
      else
        adapt_step(v.pcom_step, r, mix.pcom_minstep, mix.pcom_maxstep, mix.pcom_minacc,
                   mix.pcom_maxacc);
    }
  }
  G::sync();
}

template <bool WARP, int PH, int SPEC = SWAP_ANY>
__device__ void sweep_one(SmemCtl &sc, double *red, const CV &c, unsigned char *scratch,
                          int warp_scratch_d, bool teams) {
  using G = Group<WARP>;
  const ChainDesc &d = sc.d;
  const MixDev &mix = sc.mix;
  const int tid = G::rank(), nt = G::size(), lane = threadIdx.x & 31;
  const int warp = WARP ? 0 : (int)(threadIdx.x >> 5), nwarps = WARP ? 1 : (int)(blockDim.x >> 5);
  const int N = c.N, M = c.M;
  const bool serial_local = chain_serial_local(d);
  const unsigned long long sweep = sc.v.sweep;
  double *wsb = (double *)scratch + (size_t)warp * warp_scratch_d;
  // every carve below must fit the group's scratch (PIMC_CHECK builds)
  if (!check_ok((size_t)nwarps * warp_scratch_d * sizeof(double) <= (size_t)sc.scratch_bytes &&
                    SwapScratch::bytes(N, nwarps) <= (size_t)sc.scratch_bytes &&
                    ComScratch::bytes(N, M, nwarps) <= (size_t)sc.scratch_bytes,
                DERR_SCRATCH, d))
    return;

  // ---- staging phases (ReshapeLinear)
  if (PH & SW_STAGE) {
  // per-thread tallies: attempts, accepts, skips, bead updates
  double tal[4] = {0, 0, 0, 0};
  for (int ph = 0; ph < mix.staging_phases; ++ph) {
    int ell = sc.v.stage_m;
    ell = max(2, min(ell, min(M - 1, WMAX)));
    const int k = (M + ell - 1) / ell;
    const Stream so = make_stream(d, sweep, PH_STAGE_OFF, (unsigned)ph);
    const int o = min(M - 1, (int)(so.uni(0) * M));
    const int items = N * k;
    if (!serial_local) {
      // every window of the phase is independent: slot s of particle n moves
      // the beads strictly inside its slot; item order s*N + n makes
      // neighbouring threads touch neighbouring particles of one slice
      if (ell <= TWMAX) {
        for (int it = tid; it < items; it += nt) {
          const int s = it / N, n = it % N;
          const int len = s < k - 1 ? ell : M - (k - 1) * ell;
          if (len < 2) continue;
          const int st = (o + s * ell) % M;
          GenDraws dr = gen_draws(make_stream(d, sweep, PH_STAGE, (unsigned)(ph * items + it)));
          const int m = min(len, 2 + (int)(dr.s.uni(DRAW_CHOICE) * (ell - 1)));
          const int r = window_thread(c, n, st, m, dr, false, nullptr);
          tal[0] += 1.0;
          tal[1] += r;
          tal[3] += m - 1;
        }
      } else {
        for (int it = warp; it < items; it += nwarps) {
          const int s = it / N, n = it % N;
          const int len = s < k - 1 ? ell : M - (k - 1) * ell;
          if (len < 2) continue;
          const int st = (o + s * ell) % M;
          GenDraws dr = gen_draws(make_stream(d, sweep, PH_STAGE, (unsigned)(ph * items + it)));
          const int m = min(len, 2 + (int)(dr.s.uni(DRAW_CHOICE) * (ell - 1)));
          const int r = window_warp(c, n, st, m, dr, false, wsb, nullptr);
          if (lane == 0) {
            tal[0] += 1.0;
            tal[1] += r == RES_ACCEPT;
            tal[3] += m - 1;
          }
        }
      }
    } else if (!WARP && teams && !(d.flags & PF_HARD) && 2 * k <= nwarps && k <= kMaxTeams) {
      // fewer slots than warps: a team of T warps walks each slot, the
      // warps splitting every window's links (named barrier 1 + team)
      const int T = min(nwarps / k, 8), team = warp / T;
      if (team < k) {
        const Team tm{warp - team * T, T, 1 + team};
        double *tb = (double *)scratch + (size_t)(team * T) * warp_scratch_d;
        const int len = team < k - 1 ? ell : M - (k - 1) * ell;
        const int st = (o + team * ell) % M;
        if (len >= 2)
          for (int n = 0; n < N; ++n) {
            GenDraws dr = gen_draws(make_stream(d, sweep, PH_STAGE, (unsigned)(ph * items + team * N + n)));
            const int m = min(len, 2 + (int)(dr.s.uni(DRAW_CHOICE) * (ell - 1)));
            const int r = window_team(c, tm, n, st, m, dr, tb, warp_scratch_d);
            if (tm.w == 0 && lane == 0) {
              tal[0] += 1.0;
              tal[1] += r == RES_ACCEPT;
              tal[3] += m - 1;
            }
          }
      }
    } else {
      // windows of one slot interact through the pair action or the hard
      // core: a warp walks the particles of its slot in order; distinct
      // slots share only their fixed end slices and run concurrently
      for (int s = warp; s < k; s += nwarps) {
        const int len = s < k - 1 ? ell : M - (k - 1) * ell;
        if (len < 2) continue;
        const int st = (o + s * ell) % M;
        for (int n = 0; n < N; ++n) {
          GenDraws dr = gen_draws(make_stream(d, sweep, PH_STAGE, (unsigned)(ph * items + s * N + n)));
          const int m = min(len, 2 + (int)(dr.s.uni(DRAW_CHOICE) * (ell - 1)));
          const int r = window_warp(c, n, st, m, dr, false, wsb, nullptr);
          if (lane == 0) {
            tal[0] += 1.0;
            tal[1] += r == RES_ACCEPT;
            if (r != RES_HARDCORE) tal[3] += m - 1;
          }
        }
      }
    }
    G::sync();
  }
  if (mix.staging_phases > 0) close_phase<WARP>(sc, red, MV_STAGE, tal);
  }

  // ---- permutation swaps (ReshapeSwapLinear), one at a time by the group
  if ((PH & SW_SWAP) && N > 1 && mix.swaps_per_sweep > 0) {
    double tal[4] = {0, 0, 0, 0};
    SwapScratch S;
    S.carve(scratch, N, nwarps);
    const int mmax = max(2, min(mix.swap_max, min(M - 1, WMAX)));
    const int sm = max(2, sc.v.swap_m);
    for (int a = 0; a < mix.swaps_per_sweep; ++a) {
      const Stream ss = make_stream(d, sweep, PH_SWAP, (unsigned)a);
      const uint4 r0 = ss.at(DRAW_CHOICE), r1 = ss.at(DRAW_CHOICE + 1);
      const int j0 = min(M - 1, (int)(u53(r0.x, r0.y) * M));
      const int m = min(mmax, 2 + (int)(u53(r0.z, r0.w) * (sm - 1)));
      const int n1 = min(N - 1, (int)(u53(r1.x, r1.y) * N));
      const double upick = u53(r1.z, r1.w);
      GenDraws dr = gen_draws(ss);
      const int r = swap_group<WARP, true, GenDraws, SPEC>(c, j0, m, n1, upick, dr, S, red, nullptr,
                                                           nullptr);
      if (tid == 0) {
        if (r == RES_SKIP) {
          tal[2] += 1.0;
        } else {
          tal[0] += 1.0;
          tal[1] += r == RES_ACCEPT;
          if (r != RES_HARDCORE) tal[3] += 2.0 * (m - 1);
        }
      }
    }
    G::sync();
    close_phase<WARP>(sc, red, MV_SWAP, tal);
  }

  if (!(PH & SW_REST)) return;

  // ---- single-path centre of mass
  double tal[4] = {0, 0, 0, 0};
  for (int ph = 0; ph < mix.com_phases; ++ph) {
    const double step = sc.v.com_step;
    if (!serial_local) {
      for (int n = tid; n < N; n += nt) {
        if (c.next[n] != n) continue;
        GenDraws dr = gen_draws(make_stream(d, sweep, PH_COM, (unsigned)(ph * N + n)));
        const int r = com_thread(c, n, step, dr);
        tal[0] += 1.0;
        tal[1] += r;
        tal[3] += M;
      }
      G::sync();
    } else {
      ComScratch cs;
      cs.carve(scratch, N, M);
      for (int n = 0; n < N; ++n) {
        if (c.next[n] != n) continue;
        GenDraws dr = gen_draws(make_stream(d, sweep, PH_COM, (unsigned)(ph * N + n)));
        const int r = com_group<WARP>(c, n, false, step, dr, cs, red, sc.shift, &sc.iflag[2], nullptr);
        if (tid == 0) {
          tal[0] += 1.0;
          tal[1] += r == RES_ACCEPT;
          if (r != RES_HARDCORE) tal[3] += M;
        }
        G::sync();
      }
    }
  }

  if (mix.com_phases > 0) close_phase<WARP>(sc, red, MV_COM, tal);

  // ---- cycle centre of mass, one attempt per cycle (led by its lowest index)
  double tlp[4] = {0, 0, 0, 0};
  for (int ph = 0; ph < mix.polymer_com_phases; ++ph) {
    ComScratch cs;
    cs.carve(scratch, N, M);
    for (int n = 0; n < N; ++n) {
      if (tid == 0) {
        int lead = 1, i = c.next[n], guard = 0;
        while (i != n && guard++ <= N) {
          if (i < n) { lead = 0; break; }
          i = c.next[i];
        }
        sc.iflag[1] = lead;
      }
      G::sync();
      if (!sc.iflag[1]) continue;
      GenDraws dr = gen_draws(make_stream(d, sweep, PH_PCOM, (unsigned)(ph * N + n)));
      const int r = com_group<WARP>(c, n, true, sc.v.pcom_step, dr, cs, red, sc.shift, &sc.iflag[2],
                                    &sc.iflag[3]);
      const int np = sc.iflag[3];
      if (tid == 0) {
        tlp[0] += 1.0;
        tlp[1] += r == RES_ACCEPT;
        if (r != RES_HARDCORE) tlp[3] += (double)M * np;
      }
      G::sync();
    }
  }
  if (mix.polymer_com_phases > 0) close_phase<WARP>(sc, red, MV_PCOM, tlp);

  // ---- measurement cadence (measurement_Z_sector)
  if (mix.measure_every > 0 && ((sweep + 1) % (unsigned long long)mix.measure_every) == 0) {
    measure_group<WARP>(c, red, sc.e4, c.hist != nullptr, (unsigned long long *)scratch);
    if (tid == 0) record_measurement(d, sc.v, c, sc.e4, c.hist != nullptr);
  }
  if (tid == 0) sc.v.sweep++;
  G::sync();
}

// warp per chain: every warp of the grid pulls chains from the queue (or
// takes chain0 + its global warp index once) and sweeps them alone; its
// control block and scratch live in its own slice of dynamic shared memory.
// PH names the phases of the sweep it runs (all of them, or the swaps alone
// as the swap launch of a split sweep).
template <int PH>
__device__ __forceinline__ void sweep_warp(const SweepArgs &a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const size_t ctl = (sizeof(SmemCtl) + 15) & ~(size_t)15;
  unsigned char *mine = smem + (size_t)w * (ctl + a.warp_bytes);
  SmemCtl &sc = *reinterpret_cast<SmemCtl *>(mine);
  unsigned char *scratch = mine + ctl;
  const int gw = blockIdx.x * (blockDim.x >> 5) + w;
  int iter = 0;
  while (true) {
    int ci = a.nchains;
    if (lane == 0) {
      if (a.queue) ci = atomicAdd(a.queue, 1);
      else ci = iter == 0 ? gw : a.nchains;
      if (ci < a.nchains) {
        const int ch = a.order ? a.order[ci] : a.chain0 + ci;
        sc.chain = ch;
        sc.d = a.desc[ch];
        sc.v = a.var[ch];
        sc.mix = a.mix[ch];
        sc.scratch_bytes = a.warp_bytes;
      }
    }
    ci = __shfl_sync(0xffffffffu, ci, 0);
    __syncwarp();
    ++iter;
    if (ci >= a.nchains) break;
    CV c = make_cv(&sc.d, a.dpool, a.ipool, a.upool);
    // the warp's scratch (at least N doubles) holds the bitmap of the check
    const bool ok = sc.v.err == 0 && next_is_permutation<true>(c.next, sc.d.N, (unsigned *)scratch);
    if (!ok && lane == 0 && sc.v.err == 0) sc.v.err = DERR_STATE;
    __syncwarp();
    if (ok)
      for (int s = 0; s < a.sweeps; ++s) sweep_one<true, PH>(sc, nullptr, c, scratch, a.warp_scratch_d, false);
    if (lane == 0) a.var[sc.chain] = sc.v;
    __syncwarp();
  }
}

__global__ void __launch_bounds__(256, 2) k_sweep_warp(SweepArgs a) { sweep_warp<SW_ALL>(a); }
// the swap phase of a split sweep with one warp per chain: twice the chains
// in flight of a two-warp CTA per chain at the same registers per SM
__global__ void __launch_bounds__(256, 2) k_sweep_swap_warp(SweepArgs a) { sweep_warp<SW_SWAP>(a); }

template <int PH, int SPEC = SWAP_ANY>
__device__ __forceinline__ void sweep_cta(const SweepArgs &a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ SmemCtl sc;
  __shared__ double red[256];
  const int tid = threadIdx.x, nt = blockDim.x;
  int iter = 0;
  while (true) {
    if (tid == 0) {
      int ci;
      if (a.queue) ci = atomicAdd(a.queue, 1);
      else ci = iter == 0 ? (int)blockIdx.x : a.nchains;
      if (ci < a.nchains) {
        const int ch = a.order ? a.order[ci] : a.chain0 + ci;
        sc.chain = ch;
        sc.d = a.desc[ch];
        sc.v = a.var[ch];
        sc.mix = a.mix[ch];
        sc.scratch_bytes = (int)dyn_smem_bytes() - a.state_bytes;
      } else {
        sc.chain = -1;
      }
    }
    __syncthreads();
    ++iter;
    if (sc.chain < 0) break;
    const ChainDesc &d = sc.d;
    CV c = make_cv(&sc.d, a.dpool, a.ipool, a.upool);
    {
      __shared__ unsigned bits[(kMaxParticles + 31) / 32];
      const bool ok = sc.v.err == 0 && next_is_permutation<false>(c.next, d.N, bits);
      if (!ok) {
        if (tid == 0) {
          if (sc.v.err == 0) sc.v.err = DERR_STATE;
          a.var[sc.chain] = sc.v;
        }
        __syncthreads();
        continue;
      }
    }
    const int N = d.N, M = d.M, dim = d.dim;
    const bool staged = d.smem_bytes > 0 && d.smem_bytes <= a.state_bytes;
    const size_t nx = (size_t)dim * M * N, nv = (size_t)M * N;
    if (staged) {
      double *sx = (double *)smem;
      double *sV = sx + nx;
      unsigned *sq = (unsigned *)(sV + nv);
      int *snx = (int *)(sq + nv);
      for (size_t e = tid; e < nx; e += nt) sx[e] = c.x[e];
      for (size_t e = tid; e < nv; e += nt) sV[e] = c.V[e];
      for (size_t e = tid; e < nv; e += nt) sq[e] = c.xq[e];
      for (int e = tid; e < N; e += nt) snx[e] = c.next[e];
      c.x = sx;
      c.V = sV;
      c.xq = sq;
      c.next = snx;
      __syncthreads();
    }
    unsigned char *scratch = smem + a.state_bytes;
    for (int s = 0; s < a.sweeps; ++s)
      sweep_one<false, PH, SPEC>(sc, red, c, scratch, a.warp_scratch_d, a.teams != 0);
    if (staged) {
      double *gx = a.dpool + d.x_off, *gV = a.dpool + d.V_off;
      unsigned *gq = (unsigned *)(a.dpool + d.xq_off);
      int *gn = a.ipool + d.next_off;
      for (size_t e = tid; e < nx; e += nt) gx[e] = c.x[e];
      for (size_t e = tid; e < nv; e += nt) gV[e] = c.V[e];
      for (size_t e = tid; e < nv; e += nt) gq[e] = c.xq[e];
      for (int e = tid; e < N; e += nt) gn[e] = c.next[e];
    }
    if (tid == 0) a.var[sc.chain] = sc.v;
    __syncthreads();
  }
}

// one CTA per chain, every phase of the sweep in one launch
__global__ void __launch_bounds__(512) k_sweep(SweepArgs a) { sweep_cta<SW_ALL>(a); }

// the sweep's phases as separate launches (staging, swaps, the rest), each
// compiled and scheduled on its own: every chain of the batch finishes one
// phase before any starts the next, so the longest chain of each phase, not
// the longest sum over phases, sets a sweep's time
__global__ void __launch_bounds__(512) k_sweep_stage(SweepArgs a) { sweep_cta<SW_STAGE>(a); }
__global__ void __launch_bounds__(512) k_sweep_swap(SweepArgs a) { sweep_cta<SW_SWAP>(a); }
// the swap launch for batches whose every chain follows the reference's
// rules without a hard core or a contact table (swap_group SWAP_REF)
__global__ void __launch_bounds__(512) k_sweep_swap_ref(SweepArgs a) {
  sweep_cta<SW_SWAP, SWAP_REF>(a);
}
__global__ void __launch_bounds__(512) k_sweep_rest(SweepArgs a) { sweep_cta<SW_REST>(a); }

// ---------------------------------------------------------------------------
// single moves with injected draws (one CTA, state in global memory)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_attempt(AttemptArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ SmemCtl sc;
  __shared__ double red[256];
  const int tid = threadIdx.x;
  if (tid == 0) {
    sc.d = a.desc[a.chain];
    sc.v = a.var[a.chain];
  }
  __syncthreads();
  const ChainDesc &d = sc.d;
  CV c = make_cv(&sc.d, a.dpool, a.ipool, a.upool);
  InjDraws dr;
  dr.nrm = a.normals;
  dr.n_nrm = a.n_normals;
  dr.pn = 0;
  dr.uni = a.uniforms;
  dr.n_uni = a.n_uniforms;
  dr.pu = 0;
  dr.exh = 0;
  int res = 0, extra = -1;
  const bool serial = chain_serial_local(d);
  if (a.kind == MV_STAGE) {
    const bool use_warp = serial || a.force_warp || a.m > TWMAX;
    if (use_warp) {
      if (tid < 32) res = window_warp(c, a.n, a.j0, a.m, dr, true, (double *)smem, a.prop);
    } else {
      if (tid == 0) res = window_thread(c, a.n, a.j0, a.m, dr, true, a.prop);
    }
  } else if (a.kind == MV_SWAP) {
    if (tid < 32) {
      SwapScratch S;
      S.carve(smem, d.N, 1);
      res = swap_warp<false>(c, a.j0, a.m, a.n, a.u_pick, dr, S, a.prop, &sc.iflag[4]);
    }
    __syncthreads();
    extra = sc.iflag[4];
  } else if (a.kind == MV_COM && !serial && !a.force_warp) {
    if (tid == 0) res = com_thread(c, a.n, a.step, dr);
  } else {
    ComScratch cs;
    cs.carve(smem, d.N, d.M);
    res = com_group<false>(c, a.n, a.kind == MV_PCOM, a.step, dr, cs, red, sc.shift, &sc.iflag[2],
                           &sc.iflag[3]);
    extra = sc.iflag[3];
  }
  __syncthreads();
  if (tid == 0) {
    a.out[0] = res;
    a.out[1] = extra;
    a.out[2] = dr.pn;
    a.out[3] = dr.pu;
    a.out[4] = dr.exh;
  }
}

// ---------------------------------------------------------------------------
// action evaluation (parity level a) and staging weights of a given window
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_eval_action(EvalArgs a) {
  __shared__ SmemCtl sc;
  __shared__ double red[256];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = nt >> 5;
  if (tid == 0) sc.d = a.desc[a.chain];
  __syncthreads();
  const ChainDesc &d = sc.d;
  CV c = make_cv(&sc.d, a.dpool, a.ipool, a.upool);
  const int N = c.N, M = c.M, dim = c.dim;
  const double den = 4.0 * d.tau * d.lambda, mhtau = -0.5 * d.tau, rc2 = d.rc * d.rc;
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k = tid; k < N * M; k += nt) {
    const int j = k / N, i = k % N;
    const int in = j == M - 1 ? c.next[i] : i, jn = j + 1 == M ? 0 : j + 1;
    const double ax = c.X(0, i, j), ay = c.Xd(1, i, j);
    const double bx = c.X(0, in, jn), by = c.Xd(1, in, jn);
    s[0] += -mi2(d, ax, ay, bx, by) / den;
    s[1] += mhtau * (vext(d, ax, ay) + vext(d, bx, by));
    s[3] += c.Vl(i, j);
  }
  if (d.flags & PF_PAIR) {
    for (int k = warp; k < N * M; k += nwarps) {
      const int j = k / N, i = k % N;
      const int in = j == M - 1 ? c.next[i] : i, jn = j + 1 == M ? 0 : j + 1;
      const double ax = c.X(0, i, j), ay = c.Xd(1, i, j);
      const double bx = c.X(0, in, jn), by = c.Xd(1, in, jn);
      Prefilter f;
      f.init_q(c.Q(i, j), d.q_lim_rc);
      const unsigned *row = c.xq + (size_t)j * c.ldn;
      for (int b = i + 1 + lane; b < N; b += 32) {
        if (!f.pass(row[b])) continue;
        const double r2a = mi2(d, ax, ay, c.X(0, b, j), c.Xd(1, b, j));
        if (r2a > rc2) continue;
        const int bn = j == M - 1 ? c.next[b] : b;
        if (d.flags & PF_CONTACT)
          s[2] += contact_link(d, ax, ay, c.X(0, b, j), c.Xd(1, b, j), bx, by, c.X(0, bn, jn),
                               c.Xd(1, bn, jn));
        else
          s[2] += lnU2(d, r2a, mi2(d, bx, by, c.X(0, bn, jn), c.Xd(1, bn, jn)));
      }
    }
  }
  block_sum_k<4>(s, red);
  if (tid == 0)
    for (int q = 0; q < 4; ++q) a.out[q] = s[q];
}

__global__ void k_eval_weights(EvalArgs a) {
  __shared__ ChainDesc d;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) d = a.desc[a.chain];
  __syncthreads();
  CV c = make_cv(&d, a.dpool, a.ipool, a.upool);
  const int M = c.M, dim = c.dim, n = a.n, j0 = a.j0, m = a.m;
  const int nx = c.next[n];
  const double mhtau = -0.5 * d.tau;
  const double *rp = a.rp;
  auto px = [&](int t) { return rp[t * dim]; };
  auto py = [&](int t) { return dim > 1 ? rp[t * dim + 1] : 0.0; };
  double wi = 0.0, wu = 0.0;
  if (lane == 0) {
    for (int t = 0; t < m; ++t) {
      const int ab = j0 + t;
      wi += c.Vl(ab < M ? n : nx, ab < M ? ab : ab - M);
    }
    for (int t = 0; t < m; ++t) wu += mhtau * (vext(d, px(t), py(t)) + vext(d, px(t + 1), py(t + 1)));
  }
  if ((d.flags & PF_PAIR) && (d.flags & PF_PHYS)) {
    __shared__ double wx[WMAX + 1], wy[WMAX + 1];
    __shared__ unsigned wq[WMAX + 1];
    __shared__ unsigned long long q[PQ_CAP];
    for (int t = lane; t <= m; t += 32) {
      wx[t] = px(t);
      wy[t] = py(t);
      wq[t] = qpos(d, wx[t], wy[t]);
    }
    __syncwarp();
    WindowSeg seg{&c, n, nx, j0, M, wx, wy, wq};
    segment_pairs(c, seg, 0, m, true, true, q, wi, wu, lane);
  }
  wi = warp_sum(wi);
  wu = warp_sum(wu);
  if (threadIdx.x == 0) {
    a.out[0] = wi;
    a.out[1] = wu;
  }
}

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
__device__ __forceinline__ int tile_chain(const int *tile_off, int nchains, int t) {
  int lo = 0, hi = nchains;  // tile_off[lo] <= t < tile_off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (tile_off[mid] <= t) lo = mid; else hi = mid;
  }
  return lo;
}

template <bool IMPORT>
__global__ void __launch_bounds__(256) k_transpose_tiles(const ChainDesc *desc, double *dpool,
                                                          double *host, const int *tile_off,
                                                          int nchains) {
  __shared__ double tile[2][32][33];
  const int ntiles = tile_off[nchains];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int c = tile_chain(tile_off, nchains, t);
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

// the exp table of exp_neg for the current device
// scratch sizes of the device move routines, for the host's shared-memory plans
size_t swap_scratch_bytes(int N, int nwarps) { return SwapScratch::bytes(N, nwarps); }
size_t com_scratch_bytes(int N, int M, int nwarps) { return ComScratch::bytes(N, M, nwarps); }
int window_scratch_doubles() { return WARP_SCRATCH_D; }

cudaError_t upload_exp_table() {
  static double tab[EXPTAB_N + 1];
  for (int k = 0; k <= EXPTAB_N; ++k) tab[k] = std::exp(-k / 64.0);
  return cudaMemcpyToSymbol(g_exptab, tab, sizeof(tab));
}

cudaError_t launch_sweep(const SweepArgs &a, int mode, int grid, int block, size_t smem,
                         cudaStream_t s) {
  if (mode == 1) k_sweep_warp<<<grid, block, smem, s>>>(a);
  else k_sweep<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}
// phase kernels: 0 staging, 1 swaps, 2 the rest; warp = 1 (swaps only): one
// warp per chain
// warp = 1 (swaps only): one warp per chain; spec = 1 (swaps in CTA mode):
// the reference-rules swap kernel
static const void *phase_kernel(int phase, int warp, int spec) {
  if (phase == 1) {
    if (warp) return (const void *)k_sweep_swap_warp;
    return spec ? (const void *)k_sweep_swap_ref : (const void *)k_sweep_swap;
  }
  return phase == 0 ? (const void *)k_sweep_stage : (const void *)k_sweep_rest;
}
cudaError_t launch_sweep_phase(const SweepArgs &a, int phase, int warp, int spec, int grid,
                               int block, size_t smem, cudaStream_t s) {
  if (phase == 0) k_sweep_stage<<<grid, block, smem, s>>>(a);
  else if (phase == 1 && warp) k_sweep_swap_warp<<<grid, block, smem, s>>>(a);
  else if (phase == 1 && spec) k_sweep_swap_ref<<<grid, block, smem, s>>>(a);
  else if (phase == 1) k_sweep_swap<<<grid, block, smem, s>>>(a);
  else k_sweep_rest<<<grid, block, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t sweep_phase_set_smem(int phase, int warp, int spec, size_t smem) {
  return cudaFuncSetAttribute(phase_kernel(phase, warp, spec),
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t sweep_phase_occupancy(int phase, int warp, int spec, int block, size_t smem,
                                  int *blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm,
                                                       phase_kernel(phase, warp, spec), block, smem);
}

cudaError_t sweep_set_smem(int mode, size_t smem) {
  if (mode == 1)
    return cudaFuncSetAttribute(k_sweep_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaFuncSetAttribute(k_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
size_t sweep_ctl_bytes() { return (sizeof(SmemCtl) + 15) & ~(size_t)15; }
cudaError_t sweep_occupancy(int mode, int block, size_t smem, int *blocks_per_sm) {
  if (mode == 1)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep_warp, block, smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_sweep, block, smem);
}
cudaError_t launch_attempt(const AttemptArgs &a, size_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_attempt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_attempt<<<1, 128, smem, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_eval_action(const EvalArgs &a, cudaStream_t s) {
  k_eval_action<<<1, 256, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t launch_eval_weights(const EvalArgs &a, cudaStream_t s) {
  k_eval_weights<<<1, 32, 0, s>>>(a);
  return cudaGetLastError();
}
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
                                   double *host, const int *tile_off, int nchains, int ntiles,
                                   int grid, cudaStream_t s) {
  const int g = std::max(1, std::min(grid, ntiles));
  if (import) k_transpose_tiles<true><<<g, 256, 0, s>>>(desc, dpool, host, tile_off, nchains);
  else k_transpose_tiles<false><<<g, 256, 0, s>>>(desc, dpool, host, tile_off, nchains);
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

// the PIMC_PROFILE build's swap counters (g_prof): read, then cleared on
// request; cudaErrorNotSupported in other builds
cudaError_t profile_take(unsigned long long *out, bool reset, cudaStream_t s) {
#if PIMC_PROFILE
  cudaError_t e = cudaMemcpyFromSymbolAsync(out, g_prof, sizeof(g_prof), 0, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && reset) {
    static const unsigned long long z[32] = {};
    e = cudaMemcpyToSymbolAsync(g_prof, z, sizeof(z), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return e;
#else
  (void)out;
  (void)reset;
  (void)s;
  return cudaErrorNotSupported;
#endif
}

// the PIMC_CHECK build's device check word: read and cleared (0 in the
// default build, which has no bounds checks)
cudaError_t check_word_take(cudaStream_t s, unsigned long long *w) {
  *w = 0;
#if PIMC_CHECK
  cudaError_t e = cudaMemcpyFromSymbolAsync(w, g_check_word, sizeof(*w), 0, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && *w) {
    const unsigned long long z = 0;
    e = cudaMemcpyToSymbolAsync(g_check_word, &z, sizeof(z), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return e;
#else
  (void)s;
  return cudaSuccess;
#endif
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
