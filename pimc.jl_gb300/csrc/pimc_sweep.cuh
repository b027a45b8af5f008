// pimc_sweep.cuh -- the sweep of one chain by a group (a CTA or one warp)
// and the persistent drivers that pull chains from the batch's work queue,
// shared by the kernel translation units, compiled in parallel:
// pimc_sweep.cu (the staging and rest phases and the other kernels),
// pimc_swap.cu (the swap phase), pimc_fused.cu (whole sweeps in one launch)
// and pimc_attempt.cu (single moves with injected draws).  Device globals of
// the headers are per translation unit (static); each unit gives the host
// its own accessors (tu_* below, exported by PIMC_UNIT_ACCESSORS).
#pragma once
#include <cuda_runtime.h>

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
  c.tabw = c.tab + (size_t)d->wtab * d->wtab;
  c.hist = (d->dens_off >= 0 && upool) ? upool + d->dens_off : nullptr;
  c.eser = d->eser_off >= 0 ? dpool + d->eser_off : nullptr;
  c.cl = nullptr;
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

static __device__ void record_measurement(const ChainDesc &d, ChainVar &v, const CV &c, const double *e,
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
static __device__ void adapt_slices(int &m, double acc_ratio, int mn, int mx, double minacc,
                             double maxacc) {
  if (acc_ratio < minacc) m -= 1;
  else if (acc_ratio > maxacc) m += 1;
  m = max(mn, m);
  m = min(mx, m);
}
static __device__ void adapt_step(double &s, double acc_ratio, double mn, double mx, double minacc,
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
  CellLists cl;       // the chain's cell lists (d.cl_nc > 0)
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
  // the view with the chain's cell lists: a phase that queries neighbours
  // builds them at its start and its moves keep them current; the phases
  // that do not query run on c, whose moves mark nothing
  CV cq = c;
  cq.cl = d.cl_nc > 0 && d.cl_mode > 0 ? &sc.cl : nullptr;
  // builds the lists for a phase that queries (every thread calls it); false
  // (row scans, no marks) while the chain is held off, or when fewer than
  // half of its slices have usable lists, which holds it off for the next
  // kCellHold sweeps
  auto build_lists = [&]() -> bool {
    if (!cq.cl || sc.v.cl_hold > 0) return false;
    if (tid == 0) sc.iflag[5] = 0;
    G::sync();
    cells_build<WARP>(cq, sc.cl, (int *)scratch, sc.scratch_bytes / 4, &sc.iflag[5]);
    G::sync();
    const bool use = 2 * sc.iflag[5] >= M;
    G::sync();
    if (!use && tid == 0) sc.v.cl_hold = kCellHold;
    return use;
  };
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
    const bool lists = serial_local && build_lists();
    const CV &cw = lists ? cq : c;
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
            const int r = window_team(cw, tm, n, st, m, dr, tb, warp_scratch_d);
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
          const int r = window_warp(cw, n, st, m, dr, false, wsb, nullptr);
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
    const bool lists = (d.flags & (PF_PAIR | PF_HARD)) && build_lists();
    const CV &cs = lists ? cq : c;
    for (int a = 0; a < mix.swaps_per_sweep; ++a) {
      const Stream ss = make_stream(d, sweep, PH_SWAP, (unsigned)a);
      const uint4 r0 = ss.at(DRAW_CHOICE), r1 = ss.at(DRAW_CHOICE + 1);
      const int j0 = min(M - 1, (int)(u53(r0.x, r0.y) * M));
      const int m = min(mmax, 2 + (int)(u53(r0.z, r0.w) * (sm - 1)));
      const int n1 = min(N - 1, (int)(u53(r1.x, r1.y) * N));
      const double upick = u53(r1.z, r1.w);
      GenDraws dr = gen_draws(ss);
      const int r = swap_group<WARP, true, GenDraws, SPEC>(cs, j0, m, n1, upick, dr, S, red, nullptr,
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
      const bool lists = build_lists();
      const CV &cw = lists ? cq : c;
      for (int n = 0; n < N; ++n) {
        if (c.next[n] != n) continue;
        GenDraws dr = gen_draws(make_stream(d, sweep, PH_COM, (unsigned)(ph * N + n)));
        const int r = com_group<WARP>(cw, n, false, step, dr, cs, red, sc.shift, &sc.iflag[2], nullptr);
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
    const bool lists = serial_local && build_lists();
    const CV &cp = lists ? cq : c;
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
      const int r = com_group<WARP>(cp, n, true, sc.v.pcom_step, dr, cs, red, sc.shift, &sc.iflag[2],
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
    const bool lists = (d.flags & PF_PAIR) && !(d.flags & PF_CONTACT) && build_lists();
    measure_group<WARP, true>(lists ? cq : c, red, sc.e4, c.hist != nullptr, (unsigned long long *)scratch);
    if (tid == 0) record_measurement(d, sc.v, c, sc.e4, c.hist != nullptr);
  }
  if (tid == 0) {
    sc.v.sweep++;
    if (sc.v.cl_hold > 0) --sc.v.cl_hold;
  }
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
        if (sc.d.cl_nc > 0) sc.cl.bind(sc.d, a.ipool);
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
        if (sc.d.cl_nc > 0) sc.cl.bind(sc.d, a.ipool);
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

// ---------------------------------------------------------------------------
// host accessors of this translation unit's device globals
// ---------------------------------------------------------------------------
static inline cudaError_t tu_upload_exp_table(const double *tab, size_t bytes) {
  return cudaMemcpyToSymbol(g_exptab, tab, bytes);
}
// adds this unit's swap-profile counters to out[32], clearing them on reset
static inline cudaError_t tu_profile_take(unsigned long long *out, bool reset, cudaStream_t s) {
#if PIMC_PROFILE
  unsigned long long v[32];
  cudaError_t e = cudaMemcpyFromSymbolAsync(v, g_prof, sizeof(v), 0, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  for (int k = 0; k < 32; ++k) out[k] += v[k];
  if (reset) {
    const unsigned long long z[32] = {};
    e = cudaMemcpyToSymbolAsync(g_prof, z, sizeof(z), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return e;
#else
  (void)out;
  (void)reset;
  (void)s;
  return cudaSuccess;
#endif
}
// this unit's bounds-check word (first error), cleared once read
static inline cudaError_t tu_check_word_take(cudaStream_t s, unsigned long long *w) {
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

// the accessors a kernel unit exports under its own prefix
#define PIMC_UNIT_ACCESSORS(unit)                                                              \
  cudaError_t unit##_upload_exp_table(const double *tab, size_t bytes) {                       \
    return tu_upload_exp_table(tab, bytes);                                                     \
  }                                                                                             \
  cudaError_t unit##_profile_take(unsigned long long *out, bool reset, cudaStream_t s) {       \
    return tu_profile_take(out, reset, s);                                                      \
  }                                                                                             \
  cudaError_t unit##_check_word_take(cudaStream_t s, unsigned long long *w) {                  \
    return tu_check_word_take(s, w);                                                            \
  }

}  // namespace pimc
