// pimc_kernels.cuh -- warp/CTA-level moves (permutation swap, centre-of-mass
// shifts) and the estimators.
#pragma once
#include <type_traits>

#include "pimc_device.cuh"

namespace pimc {

// ---------------------------------------------------------------------------
// block reductions (red: >= 256 doubles of shared memory; K <= 8)
// ---------------------------------------------------------------------------
template <int K, class T>
__device__ __forceinline__ void block_sum_k(T (&v)[K], double *red_) {
  T *red = reinterpret_cast<T *>(red_);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) red[k * 32 + w] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    T s = lane < nw ? red[k * 32 + lane] : T(0);
    v[k] = warp_sum(s);
  }
  __syncthreads();
}

template <int K, class T>
__device__ __forceinline__ void block_max_k(T (&v)[K], double *red_) {
  T *red = reinterpret_cast<T *>(red_);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_max(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) red[k * 32 + w] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_max(lane < nw ? red[k * 32 + lane] : T(-INFINITY));
  __syncthreads();
}

__device__ __forceinline__ double logaddexp(double a, double b) {
  const double mx = fmax(a, b);
  if (mx == -INFINITY) return -INFINITY;
  return mx + log(exp(a - mx) + exp(b - mx));
}

// exclusive prefix over the warp of one value per lane
template <class T>
__device__ __forceinline__ T warp_exclusive_scan(T v) {
  const int lane = threadIdx.x & 31;
  T incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  return incl - v;
}

__device__ __forceinline__ int warp_min_int(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// shared scratch of the swap
struct SwapScratch {
  double *w;                                   // N heat-bath weights
  double *r1x, *r1y, *r2x, *r2y, *vb1, *vb2;   // WMAX+1 each
  double *z;                                   // 4*WMAX normals
  unsigned long long *q;                       // PQ_CAP neighbour queue per warp
  unsigned *q1, *q2;                           // WMAX+1 mirror words each
  int *iv;                                     // 4 ints: group broadcasts
  static __host__ __device__ size_t bytes(int N, int nwarps) {
    return sizeof(double) * ((size_t)N + 6 * (WMAX + 1) + 4 * WMAX) +
           sizeof(unsigned long long) * PQ_CAP * (size_t)nwarps +
           sizeof(unsigned) * 2 * (WMAX + 1) + sizeof(int) * 4;
  }
  __device__ void carve(void *base, int N, int nwarps) {
    double *p = (double *)base;
    w = p; p += N;
    r1x = p; p += WMAX + 1; r1y = p; p += WMAX + 1;
    r2x = p; p += WMAX + 1; r2y = p; p += WMAX + 1;
    vb1 = p; p += WMAX + 1; vb2 = p; p += WMAX + 1;
    z = p; p += 4 * WMAX;
    q = (unsigned long long *)p;
    q1 = (unsigned *)(q + (size_t)PQ_CAP * nwarps);
    q2 = q1 + (WMAX + 1);
    iv = (int *)(q2 + (WMAX + 1));
  }
};

// scratch of a centre-of-mass move: cycle members and their index, the
// shifted single path (x, y, external potential, mirror words), and one
// neighbour queue per warp
struct ComScratch {
  int *pol, *idx;
  double *q;
  unsigned *qq;
  unsigned long long *qbuf;
  static __host__ __device__ size_t bytes(int N, int M, int nwarps) {
    return sizeof(int) * 2 * (size_t)N + sizeof(double) * 3 * (size_t)M +
           sizeof(unsigned) * 2 * (size_t)((M + 1) / 2) +
           sizeof(unsigned long long) * PQ_CAP * (size_t)nwarps;
  }
  __device__ void carve(void *base, int N, int M) {
    pol = (int *)base;
    idx = pol + N;
    q = (double *)(pol + 2 * N);
    qq = (unsigned *)(q + 3 * M);
    qbuf = (unsigned long long *)(qq + 2 * ((M + 1) / 2));
  }
};

// one bridge of a swap: old path (start particle na, next nxa) and its new
// beads; old terms of the reference see the other moving path
struct SwapSeg {
  const CV *c;
  int j0, M, na, nxa, n1, nx1, n2, nx2;
  const double *px, *py;
  bool ref;
  const unsigned *pq;   // mirror words of the new beads
  __device__ __forceinline__ int slice(int t) const { return j0 + t < M ? j0 + t : j0 + t - M; }
  __device__ __forceinline__ int own(int t) const { return j0 + t < M ? na : nxa; }
  __device__ __forceinline__ unsigned curq(int side, int t) const {
    return side ? pq[t] : c->Q(own(t), slice(t));
  }
  __device__ __forceinline__ unsigned nxtq(int side, int t) const { return curq(side, t + 1); }
  __device__ __forceinline__ void cur(int side, int t, double &x, double &y) const {
    if (side) { x = px[t]; y = py[t]; }
    else { x = c->X(0, own(t), slice(t)); y = c->Xd(1, own(t), slice(t)); }
  }
  __device__ __forceinline__ void nxt(int side, int t, double &x, double &y) const {
    cur(side, t + 1, x, y);
  }
  __device__ __forceinline__ bool skip(int side, int t, int b) const {
    if (ref && side == 0) return b == own(t);
    const bool w = j0 + t >= M;
    return b == (w ? nx1 : n1) || b == (w ? nx2 : n2);
  }
};

// links of particles moved by a rigid shift: link t is slice t % M of member
// pol[t / M] (a single path when np == 1); new beads are the shifted old
// beads (precomputed for a single path, recomputed for a cycle); particles
// of the moved cycle are excluded
struct ComSeg {
  const CV *c;
  const int *pol, *idx;
  int M;
  const double *q;   // single path: new x[M], y[M]; null for a cycle
  double shx, shy, L, inv2L;
  const unsigned *qq;  // single path: the new beads' mirror words
  unsigned qsh;        // the shift in mirror units (a cycle's new centres)
  __device__ __forceinline__ int slice(int t) const { return t % M; }
  __device__ __forceinline__ unsigned beadq(int side, int i, int j) const {
    if (!side) return c->Q(i, j);
    if (q) return qq[j];
    return __vadd2(c->Q(i, j), qsh);
  }
  __device__ __forceinline__ unsigned curq(int side, int t) const {
    return beadq(side, pol[t / M], t % M);
  }
  __device__ __forceinline__ unsigned nxtq(int side, int t) const {
    const int i = pol[t / M], j = t % M;
    return j + 1 < M ? beadq(side, i, j + 1) : beadq(side, c->next[i], 0);
  }
  __device__ __forceinline__ void bead(int side, int i, int j, double &x, double &y) const {
    if (!side) { x = c->X(0, i, j); y = c->Xd(1, i, j); return; }
    if (q) { x = q[j]; y = q[M + j]; return; }
    x = teleport(c->X(0, i, j) + shx, L, inv2L);
    y = c->dim > 1 ? teleport(c->X(1, i, j) + shy, L, inv2L) : 0.0;
  }
  __device__ __forceinline__ void cur(int side, int t, double &x, double &y) const {
    bead(side, pol[t / M], t % M, x, y);
  }
  __device__ __forceinline__ void nxt(int side, int t, double &x, double &y) const {
    const int i = pol[t / M], j = t % M;
    if (j + 1 < M) bead(side, i, j + 1, x, y);
    else bead(side, c->next[i], 0, x, y);
  }
  __device__ __forceinline__ bool skip(int, int, int b) const { return idx[b] >= 0; }
};

// a warp (WARP) or the whole CTA working on one chain
template <bool WARP>
struct Group {
  __device__ __forceinline__ static int rank() { return WARP ? (int)(threadIdx.x & 31) : (int)threadIdx.x; }
  __device__ __forceinline__ static int size() { return WARP ? 32 : (int)blockDim.x; }
  __device__ __forceinline__ static void sync() {
    if (WARP) __syncwarp(); else __syncthreads();
  }
  __device__ __forceinline__ static int any(int p) {
    return WARP ? __any_sync(0xffffffffu, p) : __syncthreads_or(p);
  }
  template <int K, class T>
  __device__ __forceinline__ static void max(T (&v)[K], double *red) {
    if (WARP) {
#pragma unroll
      for (int k = 0; k < K; ++k) v[k] = warp_max(v[k]);
    } else {
      block_max_k<K>(v, red);
    }
  }
  template <int K, class T>
  __device__ __forceinline__ static void sum(T (&v)[K], double *red) {
    if (WARP) {
#pragma unroll
      for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    } else {
      block_sum_k<K>(v, red);
    }
  }
};

// ---------------------------------------------------------------------------
// build of a chain's cell lists from its mirror, every slice, by the whole
// group (warps take slices).  Per slice a stable counting sort: pass 1 counts
// the particles of each cell 32 at a time (lanes of one cell found by
// match_any, the lowest adds), a scan turns the counts into starts, pass 2
// places each particle at its cell's cursor plus its rank among the lanes of
// its cell.  After pass 2 the cursors hold each cell's end, which is what
// end[] keeps.  The counts live in the warp's share of the shared scratch ws
// (ws_ints ints for the group) when it has room for ncq + 1 of them, else in
// end[] itself.  cl_mode 1: a slice whose cells hold 3^dim sum n_c^2 >
// cl_frac N^2 pairs (the block around a particle would hold most of the
// slice) is marked for the row scan.  nusable (shared) counts the slices
// whose lists are usable.
// ---------------------------------------------------------------------------
template <bool WARP>
__device__ void cells_build(const CV &c, const CellLists &L, int *ws, int ws_ints, int *nusable) {
  const ChainDesc &d = *c.d;
  const int lane = threadIdx.x & 31, warp = WARP ? 0 : (int)(threadIdx.x >> 5);
  const int nwarps = WARP ? 1 : (int)(blockDim.x >> 5);
  const int N = c.N, M = c.M, ne = L.ncq + 1;
  const unsigned lt = (1u << lane) - 1u;
  const bool local = ws && ws_ints >= ne;
  // warps that build: with shared counts, as many as the scratch holds
  const int nb = local ? min(nwarps, ws_ints / ne) : nwarps;
  if (warp >= nb) return;
  int *E = local ? ws + (size_t)warp * ne : nullptr;
  for (int j = warp; j < M; j += nb) {
    int *Eg = L.end + (size_t)j * ne;
    if (!local) E = Eg;
    for (int k = lane; k < ne; k += 32) E[k] = 0;
    for (int w = lane; w < L.nw; w += 32) L.moved[(size_t)j * L.nw + w] = 0u;
    __syncwarp();
    const unsigned *row = c.xq + (size_t)j * c.ldn;
    unsigned short *items = L.items + (size_t)j * N, *pos = L.pos + (size_t)j * N;
    double sq = 0.0;  // sum over cells of n_c^2 (the lowest lanes' shares)
    for (int b0 = 0; b0 < N; b0 += 32) {
      const int b = b0 + lane;
      const bool v = b < N;
      const int ce = v ? L.cell(row[b]) : 0;
      const unsigned act = __ballot_sync(0xffffffffu, v);
      if (v) {
        const unsigned peers = __match_any_sync(act, ce);
        if ((peers & lt) == 0) {
          const int old = E[ce + 1], k = __popc(peers);
          E[ce + 1] = old + k;
          sq += (double)k * (double)(2 * old + k);
        }
      }
      __syncwarp();
    }
    // inclusive scan of the counts E[1..ncq]: E[c] = start of cell c
    int carry = 0;
    for (int k0 = 1; k0 < ne; k0 += 32) {
      const int k = k0 + lane;
      int v = k < ne ? E[k] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
      }
      v += carry;
      if (k < ne) E[k] = v;
      carry = __shfl_sync(0xffffffffu, v, 31);
    }
    __syncwarp();
    for (int b0 = 0; b0 < N; b0 += 32) {
      const int b = b0 + lane;
      const bool v = b < N;
      const int ce = v ? L.cell(row[b]) : 0;
      const unsigned act = __ballot_sync(0xffffffffu, v);
      int base = 0, rank = 0, k = 0;
      if (v) {
        const unsigned peers = __match_any_sync(act, ce);
        rank = __popc(peers & lt);
        k = __popc(peers);
        base = E[ce];
      }
      __syncwarp();
      if (v) {
        const int p = base + rank;
        if (check_ok(p >= 0 && p < N, DERR_INDEX, d)) {
          items[p] = (unsigned short)b;
          pos[b] = (unsigned short)p;
        }
        if (rank == 0) E[ce] = base + k;
      }
      __syncwarp();
    }
    if (local)
      for (int k = lane; k < ne; k += 32) Eg[k] = E[k];
    sq = warp_sum(sq);
    if (lane == 0) {
      const double pairs = (L.ncq == L.nc ? 3.0 : 9.0) * sq;
      const bool crowded = d.cl_mode == 1 && pairs > (double)d.cl_frac * N * N;
      L.dn[j] = crowded ? kCellOff : 0;
      if (!crowded) atomicAdd(nusable, 1);
    }
    __syncwarp();
  }
}

// heat-bath exponent -(|s - E|^2 + |x_i(j0) - f|^2) / (4 lambda m tau) with
// E the end bead of particle i's path (or an explicit end): FP64 as the
// reference (attempt parity), or FP32 from the position mirror (sweeps: the
// proposal weights are then a deterministic FP32 function of the
// configuration, and the physical ratio uses the same function, so detailed
// balance is exact)
// a bead for the heat bath: FP64 position and its mirror word
struct HBead {
  double x, y;
  unsigned q;
};

template <bool FAST>
struct HeatBath {
  using W = typename std::conditional<FAST, float, double>::type;  // weight arithmetic
  const CV *c;
  double inv_den;
  float inv_denf;   // 1 / (4 lambda m tau) times the squared mirror unit
  int se, j0;
  bool wrap;
  __device__ __forceinline__ int endp(int i) const { return wrap ? c->next[i] : i; }
  __device__ __forceinline__ HBead bead(int n, int j) const {
    return {c->X(0, n, j), c->Xd(1, n, j), c->Q(n, j)};
  }
  // E = bead (endp(i), se) unless e is given
  __device__ __forceinline__ W expo(int i, const HBead &s, const HBead &f,
                                    const HBead *e = nullptr) const {
    const ChainDesc &d = *c->d;
    if (!FAST) {
      double ex, ey;
      if (!e) {
        const int ei = endp(i);
        ex = c->X(0, ei, se);
        ey = c->Xd(1, ei, se);
      } else {
        ex = e->x;
        ey = e->y;
      }
      const double t1 = mi2(d, s.x, s.y, ex, ey);
      const double t2 = mi2(d, c->X(0, i, j0), c->Xd(1, i, j0), f.x, f.y);
      return -(t1 + t2) * inv_den;
    } else {
      const unsigned eq = e ? e->q : c->Q(endp(i), se);
      const float s2 = (float)qdist2(s.q, eq) + (float)qdist2(c->Q(i, j0), f.q);
      return (W)(-s2 * inv_denf);
    }
  }
  __device__ __forceinline__ W ex_(W v) const {
    if (FAST) return (W)__expf((float)v);
    return (W)exp((double)v);
  }
};

// ---------------------------------------------------------------------------
// permutation swap: (u::ReshapeSwapLinear)(s) with the heat-bath partner
// choice sampleparticles (src/updates/reshape.jl:123-283,
// src/updates/helper.jl:224-267), by a warp (WARP) or a whole CTA.  Every
// thread of the group calls it.  The group forms the heat-bath exponents and
// splits the pair scans of the two moving paths by links; the partner
// search, the bridges and the decision are the first warp's (thread 0 draws
// the Metropolis uniform).  Returns RES_*; n2_out receives n2.
// ---------------------------------------------------------------------------
// SPEC = SWAP_REF: every chain this code runs for follows the reference's
// rules with the Gaussian pair (or none), no hard core and no contact table;
// the other rules' code is compiled out, so the kernel needs fewer registers
// and less instruction cache (the host picks it when the whole batch
// qualifies)
constexpr int SWAP_ANY = 0, SWAP_REF = 1;

template <bool WARP, bool FAST, class D, int SPEC = SWAP_ANY>
__device__ int swap_group(const CV &c, int j0, int m, int n1, double u_pick, D &dr,
                          SwapScratch &S, double *red, double *prop, int *n2_out) {
  using G = Group<WARP>;
  const ChainDesc &d = *c.d;
  constexpr bool GEN = SPEC == SWAP_ANY;
  const bool f_phys = GEN && (d.flags & PF_PHYS), f_hard = GEN && (d.flags & PF_HARD);
  const bool f_contact = GEN && (d.flags & PF_CONTACT);
  const int N = c.N, M = c.M, dim = c.dim, lane = threadIdx.x & 31;
  const int tid = G::rank(), nt = G::size();
  const int warp = WARP ? 0 : (int)(threadIdx.x >> 5), nwarps = WARP ? 1 : (int)(blockDim.x >> 5);
  const bool lead = warp == 0;
  const double L = d.L, inv2L = d.inv2L, mhtau = -0.5 * d.tau;
  if (!check_ok(m >= 2 && m <= WMAX && m < M && j0 >= 0 && j0 < M, DERR_WINDOW, d) ||
      !check_ok(n1 >= 0 && n1 < N, DERR_INDEX, d))
    return RES_SKIP;
  PROF_DECL;
  PROF_COUNT(0);
  HeatBath<FAST> hb;
  hb.c = &c;
  hb.j0 = j0;
  hb.wrap = (j0 + m) >= M;
  hb.se = hb.wrap ? j0 + m - M : j0 + m;
  if (FAST) {
    // sweeps weigh in FP32 alone: no FP64 division per attempt
    hb.inv_den = 0.0;
    hb.inv_denf = d.hb_unit / (float)m;
  } else {
    hb.inv_den = 1.0 / (4.0 * (m * d.tau) * d.lambda);
    hb.inv_denf = (float)hb.inv_den * d.q_unit2;
  }
  const int se = hb.se;
  const bool wrap = hb.wrap;
  const HBead A = hb.bead(n1, j0);
  const double ax = A.x, ay = A.y;
  const int e1p = hb.endp(n1);
  const HBead E1 = hb.bead(e1p, se);
  const double e1x = E1.x, e1y = E1.y;
  // weights exp(t_i + y_i) shifted by their maximum (the reference normalises
  // them, helper.jl:260-263; the shift keeps them from underflowing).  The
  // group forms the exponents (coalesced reads of the two slices); the first
  // warp sums them and searches the cumulative weights over contiguous
  // per-lane chunks, so that the search order is the particle order
  // sweeps (FAST) weigh in FP32 from the position mirror: a deterministic
  // function of the configuration used for both directions of the move;
  // injected-draw attempts weigh in FP64 as the reference
  using W = typename HeatBath<FAST>::W;
  W *Sw = reinterpret_cast<W *>(S.w);
  const int chunk = (N + 31) / 32;
  const int i0 = min(N, lane * chunk), i1 = min(N, i0 + chunk);
  // the bridges' normals depend on the move's stream alone: draw them first,
  // so that their arithmetic overlaps the heat bath's memory reads
  const bool early_normals = FAST && !f_hard;
  if (early_normals) {
    for (int k = tid; k < 2 * (m - 1); k += nt) {
      double zz[2];
      dr.bead_normals(k, dim, zz);
      S.z[2 * k] = zz[0];
      S.z[2 * k + 1] = dim > 1 ? zz[1] : 0.0;
    }
  }
  W wm[1] = {W(-INFINITY)};
  if (FAST) {
    // four candidates per thread at a time: their next[] and mirror words are
    // loaded before any is used, one round trip for four (the same
    // arithmetic as HeatBath::expo, in the same order)
    constexpr int U = 4;
    for (int i0 = tid; i0 < N; i0 += U * nt) {
      int ie[U];
      unsigned qa[U], qe[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + u * nt;
        ie[u] = i < N ? (wrap ? c.next[i] : i) : 0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + u * nt;
        qa[u] = i < N ? c.Q(i, j0) : 0u;
        qe[u] = i < N ? c.Q(ie[u], se) : 0u;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + u * nt;
        if (i < N) {
          const float s2 = (float)qdist2(A.q, qe[u]) + (float)qdist2(qa[u], E1.q);
          // the weight itself: exp of a non-positive exponent, unshifted (a
          // batch whose every weight underflows takes the shifted form below)
          Sw[i] = __expf((float)(W)(-s2 * hb.inv_denf));
        }
      }
    }
  } else {
    for (int i = tid; i < N; i += nt) {
      const W v = hb.expo(i, A, E1);
      Sw[i] = v;
      wm[0] = v > wm[0] ? v : wm[0];
    }
  }
  if (!FAST) G::template max<1>(wm, red);
  G::sync();
  PROF_MARK(0);
  W wmax = FAST ? W(0) : wm[0];
  W ssum = W(0);
  if (lead) {
    W ls = W(0);
    if (FAST) {
      for (int i = i0; i < i1; ++i) ls += Sw[i];
      ssum = warp_sum(ls);
      if (!(ssum > W(0))) {
        // every weight underflowed: exponents shifted by their largest
        W mx = W(-INFINITY);
        for (int i = i0; i < i1; ++i) {
          const W v = hb.expo(i, A, E1);
          Sw[i] = v;
          mx = v > mx ? v : mx;
        }
        wmax = warp_max(mx);
        ls = W(0);
        for (int i = i0; i < i1; ++i) {
          const W e = hb.ex_(Sw[i] - wmax);
          Sw[i] = e;
          ls += e;
        }
        ssum = warp_sum(ls);
      }
    } else {
      for (int i = i0; i < i1; ++i) {
        const W e = hb.ex_(Sw[i] - wmax);
        Sw[i] = e;
        ls += e;
      }
      ssum = warp_sum(ls);
    }
    W lq = ls, target;
    if (FAST) {
      // sweeps search the unnormalised weights against u times their sum
      target = (W)u_pick * ssum;
    } else {
      // attempts normalise first, as StatsBase.sample does
      const W inv_s = W(1) / ssum;
      lq = W(0);
      for (int i = i0; i < i1; ++i) {
        const W q = Sw[i] * inv_s;
        Sw[i] = q;
        lq += q;
      }
      target = (W)u_pick * warp_sum(lq);
    }
    // first i with cumulative weight >= target (StatsBase.sample)
    W cw = warp_exclusive_scan(lq);
    int cand = 0x7fffffff;
    for (int i = i0; i < i1; ++i) {
      cw += Sw[i];
      if (cw >= target) { cand = i; break; }
    }
    int n2 = warp_min_int(cand);
    if (n2 >= N) n2 = N - 1;
    if (lane == 0) S.iv[0] = n2;
  }
  G::sync();
  const int n2 = S.iv[0];
  if (n2_out && tid == 0) *n2_out = n2;
  G::sync();
  PROF_MARK(1);
  if (n2 == n1 || !check_ok(n2 >= 0 && n2 < N, DERR_INDEX, d)) {
    PROF_COUNT(1);
    return RES_SKIP;
  }
  // the partner is known: start the reads the rest of the attempt waits on
  const int nx1 = c.next[n1], nx2 = c.next[n2];
  auto own1 = [&](int t) { return (j0 + t < M) ? n1 : nx1; };
  auto own2 = [&](int t) { return (j0 + t < M) ? n2 : nx2; };
  auto slc = [&](int t) { return (j0 + t < M) ? j0 + t : j0 + t - M; };
  // the old paths' cached links (w_initial below), read now
  double vold = 0.0;
  for (int k = tid; k < 2 * m; k += nt) {
    const int b = k / m, t = k % m;
    vold += c.Vl(b == 0 ? own1(t) : own2(t), slc(t));
  }

  double log_ratio = 0.0;
  if (f_phys) {
    // (1/S'_1 + 1/S'_2) / (1/S_1 + 1/S_2): S_a sums the heat-bath weights
    // with a chosen first; primes after the ends of n1 and n2 are exchanged
    const HBead B = hb.bead(n2, j0);
    const HBead E2 = hb.bead(hb.endp(n2), se);
    // expo(i) with E(i) replaced by E'(i): the ends of n1 and n2 exchanged
    auto expo_p = [&](int i, const HBead &s_, const HBead &f_) {
      if (i != n1 && i != n2) return hb.expo(i, s_, f_);
      return hb.expo(i, s_, f_, i == n1 ? &E2 : &E1);
    };
    W mx[3] = {W(-INFINITY), W(-INFINITY), W(-INFINITY)};
    for (int i = tid; i < N; i += nt) {
      const W a0 = hb.expo(i, B, E2), a1 = expo_p(i, A, E2), a2 = expo_p(i, B, E1);
      mx[0] = a0 > mx[0] ? a0 : mx[0];
      mx[1] = a1 > mx[1] ? a1 : mx[1];
      mx[2] = a2 > mx[2] ? a2 : mx[2];
    }
    G::template max<3>(mx, red);
    W s3[4] = {W(0), W(0), W(0), W(0)};
    for (int i = tid; i < N; i += nt) {
      s3[0] += hb.ex_(hb.expo(i, B, E2) - mx[0]);
      s3[1] += hb.ex_(expo_p(i, A, E2) - mx[1]);
      s3[2] += hb.ex_(expo_p(i, B, E1) - mx[2]);
    }
    // the first warp's S_1 rides along in the fourth slot
    s3[3] = (lead && lane == 0) ? ssum : W(0);
    G::template sum<4>(s3, red);
    const double l1 = (double)wmax + log((double)s3[3]);
    const double l2 = (double)mx[0] + log((double)s3[0]);
    const double l1p = (double)mx[1] + log((double)s3[1]);
    const double l2p = (double)mx[2] + log((double)s3[2]);
    log_ratio = logaddexp(-l1p, -l2p) - logaddexp(-l1, -l2);
  }

  PROF_MARK(2);
  // two bridges with exchanged ends
  const double s1x = ax, s1y = ay, s2x = c.X(0, n2, j0), s2y = c.Xd(1, n2, j0);
  const int e2p = hb.endp(n2);
  double f1x = c.X(0, e2p, se), f1y = c.Xd(1, e2p, se);  // r1 ends at E(n2)
  double f2x = e1x, f2y = e1y;                            // r2 ends at E(n1)
  if (fabs(s1x - f1x) > L) f1x += sgn(s1x) * (2.0 * L);
  if (dim > 1 && fabs(s1y - f1y) > L) f1y += sgn(s1y) * (2.0 * L);
  if (fabs(s2x - f2x) > L) f2x += sgn(s2x) * (2.0 * L);
  if (dim > 1 && fabs(s2y - f2y) > L) f2y += sgn(s2y) * (2.0 * L);
  const bool hard = f_hard;
  if (!hard) {
    if (!early_normals)
      for (int k = tid; k < 2 * (m - 1); k += nt) {
        double zz[2];
        dr.bead_normals(k, dim, zz);
        S.z[2 * k] = zz[0];
        S.z[2 * k + 1] = dim > 1 ? zz[1] : 0.0;
      }
    dr.consumed(2 * (m - 1) * dim);
    G::sync();
    if (FAST) {
      // sweeps: each bridge coordinate in the closed form (bridge_w),
      // p_t = e + (m-t) u_t with u_t = (p_0 - e)/m + the sum of w_r z_r over
      // r <= t, that sum a prefix scan over 32-lane chunks of t (five FP64
      // additions a chunk); sequence q = b dim + k (bridge b, coordinate k)
      // goes to warp q mod nwarps, with the same arithmetic in every launch
      // shape
      const double inv_m = bridge_w(c, m, 0).x;
      for (int q = warp; q < 2 * dim; q += nwarps) {
        const int b = q / dim, k = q % dim;
        const double s0 = b == 0 ? (k == 0 ? s1x : s1y) : (k == 0 ? s2x : s2y);
        const double e = b == 0 ? (k == 0 ? f1x : f1y) : (k == 0 ? f2x : f2y);
        double *dst = b == 0 ? (k == 0 ? S.r1x : S.r1y) : (k == 0 ? S.r2x : S.r2y);
        double carry = (s0 - e) * inv_m;
        for (int c0 = 1; c0 < m; c0 += 32) {
          const int t = c0 + lane;
          const bool act = t < m;
          double v = 0.0, kt = 0.0;
          if (act) {
            const double2 wk = bridge_w(c, m, t);
            v = S.z[2 * (b * (m - 1) + t - 1) + k] * wk.x;
            kt = wk.y;
          }
#pragma unroll
          for (int off = 1; off < 32; off <<= 1) {
            const double vp = __shfl_up_sync(0xffffffffu, v, off);
            if (lane >= off) v += vp;
          }
          const double u = carry + v;
          if (act) dst[t] = fma(kt, u, e);
          carry = __shfl_sync(0xffffffffu, u, 31);
        }
      }
    } else if (lead && lane < 2 * dim) {
      const int b = lane / dim, k = lane % dim;
      double p = b == 0 ? (k == 0 ? s1x : s1y) : (k == 0 ? s2x : s2y);
      const double e = b == 0 ? (k == 0 ? f1x : f1y) : (k == 0 ? f2x : f2y);
      double *dst = b == 0 ? (k == 0 ? S.r1x : S.r1y) : (k == 0 ? S.r2x : S.r2y);
      for (int t = 1; t < m; ++t) {
        const double2 ab = bridge_coef(c, m, t);
        p = ab.x * p + (1.0 - ab.x) * e + S.z[2 * (b * (m - 1) + t - 1) + k] * ab.y;
        dst[t] = p;
      }
    }
    if (tid == 0) S.iv[1] = 0;
  } else if (lead) {
    int fail = 0;
    for (int b = 0; b < 2 && !fail; ++b) {
      double px = b == 0 ? s1x : s2x, py = b == 0 ? s1y : s2y;
      const double ex = b == 0 ? f1x : f2x, ey = b == 0 ? f1y : f2y;
      double *dx = b == 0 ? S.r1x : S.r2x, *dy = b == 0 ? S.r1y : S.r2y;
      for (int t = 1; t < m && !fail; ++t) {
        const double2 ab = bridge_coef(c, m, t);
        const int j = slc(t);
        const int ea = f_phys ? own1(t) : (b == 0 ? n2 : n1);
        const int eb = f_phys ? own2(t) : -1;
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
          if (!__any_sync(0xffffffffu, hard_hit_lanes(c, tx, ty, j, ea, eb, lane, 32))) {
            px = qx;
            py = qy;
            break;
          }
        }
        if (lane == 0) {
          dx[t] = px;
          dy[t] = py;
        }
      }
    }
    if (lane == 0) S.iv[1] = fail;
  }
  G::sync();
  PROF_MARK(3);
  if (S.iv[1]) return RES_HARDCORE;
  for (int k = tid; k < 2 * (m + 1); k += nt) {
    const int b = k / (m + 1), t = k % (m + 1);
    double qx, qy;
    if (b == 0) {
      qx = t == 0 ? s1x : (t == m ? f1x : S.r1x[t]);
      qy = t == 0 ? s1y : (t == m ? f1y : S.r1y[t]);
    } else {
      qx = t == 0 ? s2x : (t == m ? f2x : S.r2x[t]);
      qy = t == 0 ? s2y : (t == m ? f2y : S.r2y[t]);
    }
    qx = teleport_s<D::kSweep>(qx, L, inv2L);
    qy = dim > 1 ? teleport_s<D::kSweep>(qy, L, inv2L) : 0.0;
    (b == 0 ? S.r1x : S.r2x)[t] = qx;
    (b == 0 ? S.r1y : S.r2y)[t] = qy;
    (b == 0 ? S.vb1 : S.vb2)[t] = vext(d, qx, qy);
    if (d.flags & PF_PAIR) (b == 0 ? S.q1 : S.q2)[t] = qpos(d, qx, qy);
  }
  G::sync();
  PROF_MARK(4);
  const bool any_pair = (d.flags & PF_PAIR) != 0, phys = f_phys;
  double w2[2] = {vold, 0.0};  // w_initial, w_update
  for (int k = tid; k < 2 * m; k += nt) {
    const int b = k / m, t = k % m;
    w2[1] += mhtau * ((b == 0 ? S.vb1 : S.vb2)[t] + (b == 0 ? S.vb1 : S.vb2)[t + 1]);
  }
  // Under the reference's rules every pair term (-tau/2 g (..) <= 0 for
  // g >= 0) enters w_initial, so it can only raise w_update - w_initial: when
  // the pair-free part already accepts, the pair sums cannot change the
  // decision and a sweep skips them (its Metropolis uniform is a pure function
  // of the move's stream).  Injected-draw attempts always evaluate them.
  bool pairs = any_pair;
  const bool shortcuts = FAST && !(d.flags & PF_EXACT) && !f_contact;
  int early = 0;  // 1: accepted on the pair-free sums, which are then the final sums
  // reference rules, g >= 0: dS = dS_pf + (tau g / 2)(So + Sn) with So, Sn >= 0,
  // so any lower bound of the pair sums that reaches `need` accepts the move
  bool monotone = false;
  double need = 0.0;
  if (shortcuts && any_pair && !phys && d.g >= 0.0) {
    if (tid == 0) S.iv[3] = 0;
    double c2[2] = {w2[0], w2[1]};
    G::template sum<2>(c2, red);
    const double dpf = c2[1] - c2[0] + log_ratio;
    if (metropolis(d, dpf, dr)) {
      pairs = false;
      early = 1;
    } else {
      double margin;
      const double lu = log_u_margin(dr.uniform_accept(), margin);
      need = lu + margin + 1e-9 * (fabs(lu) + fabs(dpf)) - dpf;
      monotone = d.g > 0.0;
    }
  }
  PROF_MARK(5);
  if (early) PROF_COUNT(2);
  // the pair of the two moving paths, old and new (physical rules), exact
  if (pairs && phys)
    for (int t = tid; t < m; t += nt) {
      const int j = slc(t), jn = slc(t + 1);
      const int o1 = own1(t), o1n = own1(t + 1), o2 = own2(t), o2n = own2(t + 1);
      const double ox = c.X(0, o1, j), oy = c.Xd(1, o1, j);
      const double r2o = mi2(d, ox, oy, c.X(0, o2, j), c.Xd(1, o2, j));
      if (r2o <= d.rc2) {
        if (f_contact)
          w2[0] += contact_link(d, ox, oy, c.X(0, o2, j), c.Xd(1, o2, j), c.X(0, o1n, jn),
                                c.Xd(1, o1n, jn), c.X(0, o2n, jn), c.Xd(1, o2n, jn));
        else
          w2[0] += lnU2(d, r2o, mi2(d, c.X(0, o1n, jn), c.Xd(1, o1n, jn), c.X(0, o2n, jn), c.Xd(1, o2n, jn)));
      }
      const double r2n = mi2(d, S.r1x[t], S.r1y[t], S.r2x[t], S.r2y[t]);
      if (r2n <= d.rc2) {
        if (f_contact)
          w2[1] += contact_link(d, S.r1x[t], S.r1y[t], S.r2x[t], S.r2y[t], S.r1x[t + 1],
                                S.r1y[t + 1], S.r2x[t + 1], S.r2y[t + 1]);
        else
          w2[1] += lnU2(d, r2n, mi2(d, S.r1x[t + 1], S.r1y[t + 1], S.r2x[t + 1], S.r2y[t + 1]));
      }
    }
  // the 2m links of the two moving paths in contiguous ranges per warp
  const int per = (2 * m + nwarps - 1) / nwarps;
  const int a0 = min(2 * m, warp * per), a1 = min(2 * m, a0 + per);
  auto seg_of = [&](int b) {
    return SwapSeg{&c, j0, M, b == 0 ? n1 : n2, b == 0 ? nx1 : nx2, n1, nx1, n2, nx2,
                   b == 0 ? S.r1x : S.r2x, b == 0 ? S.r1y : S.r2y, !phys, b == 0 ? S.q1 : S.q2};
  };
  int dec = early ? 1 : (pairs ? -1 : 2);  // 2: decided by the exact sums at hand
  if (shortcuts && pairs) {
    // bounded estimate from the mirror: decides the move unless the log
    // acceptance ratio's interval straddles the threshold
    PairEst e = {0.f, 0.f, 0.f, 0.f, 0, 0};
    // under the monotone rules a warp whose own lower bound of the pair sums
    // already accepts raises a flag in shared memory, and every warp stops at
    // its next link (no group reduction inside the scan); a warp stops only
    // once the flag is up, so without it every warp has scanned all its links
    const double gh = 0.5 * d.tau * d.g;
    volatile int *flag = S.iv + 3;
    // the warp's lower bound is formed in FP32 (the FP64 pipe of this part
    // is narrow, and this runs after every link): the lane's estimate minus
    // its bounds, widened by the FP32 accumulation error as est_reduce_lanes
    // does, summed over the warp; the FP32 rounding of these few operations
    // and of the warp sum stays below 4e-6 of the sum of the magnitudes, which
    // is taken off, so the bound used is never above the FP64 one and an
    // early accept is always one the exact sums would make
    auto stop = [&](const PairEst &pe) -> bool {
      if (!monotone) return false;
      if (*flag) return true;
      const float ro = 2.4e-7f * (float)(pe.ko + 1), rn = 2.4e-7f * (float)(pe.kn + 1);
      const float lf = (pe.so * (1.f - ro) - pe.bo * (1.f + ro)) + (pe.sn * (1.f - rn) - pe.bn * (1.f + rn));
      const float af = (pe.so + pe.bo) + (pe.sn + pe.bn);
      const float slf = warp_sum(lf), saf = warp_sum(af);
      const double lb = (double)slf - 4e-6 * (double)saf - 1e-30;
      if (gh * lb > need) {
        if (lane == 0) *flag = 1;
        return true;
      }
      return false;
    };
    for (int b = 0; b < 2; ++b) {
      const int t0 = max(a0 - b * m, 0), t1 = min(a1 - b * m, m);
      if (t0 < t1 && segment_estimate(c, seg_of(b), t0, t1, e, lane, stop)) break;
    }
    if (monotone) {
      G::sync();
      if (*flag) dec = 1;
      G::sync();
    }
    if (dec == -1) {
      double v[6], l4[4];
      est_reduce_lanes(e, l4);
      for (int k = 0; k < 4; ++k) v[k] = l4[k];
      v[4] = w2[0];
      v[5] = w2[1];
      G::template sum<6>(v, red);
      // w_initial gets h*So and, under the reference's rules, h*Sn; the
      // physical rules put h*Sn into w_update (h = -tau g / 2)
      const double h = d.mhtau_g;
      const double centre = v[5] - v[4] + log_ratio - h * v[0] + (phys ? h : -h) * v[2];
      const double radius = fabs(h) * (v[1] + v[3]);
      dec = decide_interval(centre - radius, centre + radius, dr.uniform_accept());
    }
    if (dec != -1) PROF_COUNT(3);
  }
  PROF_MARK(6);
  if (dec == -1) PROF_COUNT(4);
  if (dec == -1) {
    for (int b = 0; b < 2; ++b) {
      const int t0 = max(a0 - b * m, 0), t1 = min(a1 - b * m, m);
      if (t0 >= t1) continue;
      double wo = 0.0, wn = 0.0;
      segment_pairs<GEN>(c, seg_of(b), t0, t1, true, true, S.q + (size_t)warp * PQ_CAP, wo, wn, lane);
      // the reference adds the new paths' pair terms to w_initial and lets
      // the old ones see the other moving path (reshape.jl:166-240)
      w2[0] += wo;
      if (phys) w2[1] += wn; else w2[0] += wn;
    }
  }
  PROF_MARK(7);
  int acc;
  if (dec == 0 || dec == 1) {
    acc = dec;
  } else {
    G::template sum<2>(w2, red);
    if (prop)
      for (int k = tid; k < 2 * (m + 1); k += nt) {
        const int b = k / (m + 1), t = k % (m + 1);
        prop[k * dim] = (b == 0 ? S.r1x : S.r2x)[t];
        if (dim > 1) prop[k * dim + 1] = (b == 0 ? S.r1y : S.r2y)[t];
      }
    if (D::kSweep) {
      // every thread holds the same sums and the move's uniform is a pure
      // function of its stream: each decides alone, no broadcast
      acc = metropolis(d, w2[1] - w2[0] + log_ratio, dr);
    } else {
      if (tid == 0) S.iv[2] = metropolis(d, w2[1] - w2[0] + log_ratio, dr);
      G::sync();
      acc = S.iv[2];
      G::sync();
    }
  }
  PROF_MARK(8);
  if (!acc) {
    PROF_COUNT(6);
    return RES_REJECT;
  }
  PROF_COUNT(5);
  // accept: exchange next, write the bridges along the new cycles, exchange
  // the tails (reshape.jl:247-279)
  const int nn1 = nx2, nn2 = nx1;
  auto nown1 = [&](int t) { return (j0 + t < M) ? n1 : nn1; };
  auto nown2 = [&](int t) { return (j0 + t < M) ? n2 : nn2; };
  for (int t = 1 + tid; t <= m; t += nt) {
    const int j = slc(t);
    if (any_pair) {  // the new beads' mirror words are at hand
      c.set_pos_q(nown1(t), j, S.r1x[t], S.r1y[t], S.q1[t]);
      c.set_pos_q(nown2(t), j, S.r2x[t], S.r2y[t], S.q2[t]);
    } else {
      c.set_pos(nown1(t), j, S.r1x[t], S.r1y[t]);
      c.set_pos(nown2(t), j, S.r2x[t], S.r2y[t]);
    }
  }
  for (int t = tid; t < m; t += nt) {
    const int j = slc(t);
    c.Vl(nown1(t), j) = mhtau * (S.vb1[t] + S.vb1[t + 1]);
    c.Vl(nown2(t), j) = mhtau * (S.vb2[t] + S.vb2[t + 1]);
  }
  if (j0 + m < M - 1)
    for (int j = se + 1 + tid; j < M; j += nt) c.exchange_linked(n1, n2, j);
  G::sync();
  if (tid == 0) {
    c.next[n1] = nn1;
    c.next[n2] = nn2;
    if (phys && !wrap) {
      // the link leaving the end bead moves with the tail
      const double v = c.Vl(n1, se);
      c.Vl(n1, se) = c.Vl(n2, se);
      c.Vl(n2, se) = v;
    }
  }
  G::sync();
  PROF_MARK(9);
  return RES_ACCEPT;
}

// the swap by one warp (injected-draw attempts)
template <bool FAST, class D>
__device__ int swap_warp(const CV &c, int j0, int m, int n1, double u_pick, D &dr,
                         SwapScratch &S, double *prop, int *n2_out) {
  return swap_group<true, FAST>(c, j0, m, n1, u_pick, dr, S, nullptr, prop, n2_out);
}

// ---------------------------------------------------------------------------
// single-path centre of mass, one thread per particle (pair-free acceptance,
// no hard core): (u::SingleCenterOfMass)(s) with move_polymer!
// (src/updates/com.jl:136-224, src/updates/helper.jl:368-395).  The shifted
// path is recomputed for the write-back instead of being stored.
// ---------------------------------------------------------------------------
template <class D>
__device__ int com_thread(const CV &c, int n, double step, D &dr) {
  const ChainDesc &d = *c.d;
  const int M = c.M, dim = c.dim;
  const double L = d.L, inv2L = d.inv2L, mhtau = -0.5 * d.tau;
  const double shx = step * 2.0 * (dr.uniform() - 0.5);
  const double shy = dim > 1 ? step * 2.0 * (dr.uniform() - 0.5) : 0.0;
  double wi = 0.0, wu = 0.0;
  const double q0x = teleport_s<D::kSweep>(c.X(0, n, 0) + shx, L, inv2L);
  const double q0y = dim > 1 ? teleport_s<D::kSweep>(c.X(1, n, 0) + shy, L, inv2L) : 0.0;
  const double v0 = vext(d, q0x, q0y);
  double vprev = v0;
  for (int j = 1; j <= M; ++j) {
    double vj = v0;
    if (j < M) {
      const double qx = teleport_s<D::kSweep>(c.X(0, n, j) + shx, L, inv2L);
      const double qy = dim > 1 ? teleport_s<D::kSweep>(c.X(1, n, j) + shy, L, inv2L) : 0.0;
      vj = vext(d, qx, qy);
    }
    wi += c.Vl(n, j - 1);
    // sweeps sum the links and scale once
    if (D::kSweep) wu += vprev + vj;
    else wu += mhtau * (vprev + vj);
    vprev = vj;
  }
  if (D::kSweep) wu *= mhtau;
  const bool acc = metropolis(d, wu - wi, dr);
  if (acc) {
    vprev = v0;
    double px = q0x, py = q0y;
    for (int j = 1; j <= M; ++j) {
      double qx = q0x, qy = q0y, vj = v0;
      if (j < M) {
        qx = teleport_s<D::kSweep>(c.X(0, n, j) + shx, L, inv2L);
        qy = dim > 1 ? teleport_s<D::kSweep>(c.X(1, n, j) + shy, L, inv2L) : 0.0;
        vj = vext(d, qx, qy);
      }
      c.set_pos(n, j - 1, px, py);
      c.Vl(n, j - 1) = mhtau * (vprev + vj);
      vprev = vj;
      px = qx;
      py = qy;
    }
  }
  return acc ? 1 : 0;
}

// ---------------------------------------------------------------------------
// centre of mass of a whole cycle (npol members; npol = 1 is the single-path
// move), whole CTA: pair terms with every particle outside the cycle, hard-
// core retries, PolymerCenterOfMass (src/updates/com.jl:31-104) without the
// worm fields that make the reference's version fail.  pol/idx: int scratch
// of 2N; q: shared scratch of 3*M doubles (single-path case); qbuf: one
// PQ_CAP-entry neighbour queue per warp.
// ---------------------------------------------------------------------------
// the threads that run a move: a whole CTA, or one warp on its own

template <bool WARP, class D>
__device__ int com_group(const CV &c, int n, bool polymer, double step, D &dr, const ComScratch &cs,
                         double *red, double *shift, int *sflag, int *np_out) {
  int *pol = cs.pol, *idx = cs.idx;
  double *q = cs.q;
  unsigned long long *qbuf = cs.qbuf;
  using G = Group<WARP>;
  const ChainDesc &d = *c.d;
  const int N = c.N, M = c.M, dim = c.dim, tid = G::rank(), nt = G::size();
  const int lane = threadIdx.x & 31, warp = WARP ? 0 : (int)(threadIdx.x >> 5);
  const int nwarps = WARP ? 1 : (int)(blockDim.x >> 5);
  const double L = d.L, inv2L = d.inv2L, mhtau = -0.5 * d.tau;
  const bool hard = (d.flags & PF_HARD) != 0;
  const bool phys_pair = (d.flags & PF_PAIR) && (d.flags & PF_PHYS);
  for (int i = tid; i < N; i += nt) idx[i] = -1;
  G::sync();
  if (tid == 0) {
    int np = 0, i = n;
    if (polymer) {
      do {
        pol[np++] = i;
        i = c.next[i];
      } while (i != n && np <= N);
    } else {
      pol[np++] = n;
    }
    *sflag = np;
  }
  G::sync();
  const int np = *sflag;
  G::sync();
  if (np_out && tid == 0) *np_out = np;
  if (np > N) return -1;
  for (int i = tid; i < np; i += nt) idx[pol[i]] = i;
  G::sync();
  int tries = 0;
  while (true) {
    if (tid == 0) {
      if (++tries > d.ctr) {
        *sflag = -1;
      } else {
        shift[0] = step * 2.0 * (dr.uniform() - 0.5);
        shift[1] = dim > 1 ? step * 2.0 * (dr.uniform() - 0.5) : 0.0;
        *sflag = 0;
      }
    }
    G::sync();
    const int fl = *sflag;
    G::sync();
    if (fl < 0) return RES_HARDCORE;
    if (!hard) break;
    // a warp per bead, lanes over the slice
    int hit = 0;
    for (int k = warp; k < np * M; k += nwarps) {
      const int i = pol[k / M], j = k % M;
      const double qx = teleport(c.X(0, i, j) + shift[0], L, inv2L);
      const double qy = dim > 1 ? teleport(c.X(1, i, j) + shift[1], L, inv2L) : 0.0;
      if (hard_hit_lanes(c, qx, qy, j, i, -1, lane, 32)) hit = 1;
    }
    if (!G::any(hit)) break;
  }
  const double shx = shift[0], shy = shift[1];
  auto shifted = [&](int i, int j, double &qx, double &qy) {
    qx = teleport(c.X(0, i, j) + shx, L, inv2L);
    qy = dim > 1 ? teleport(c.X(1, i, j) + shy, L, inv2L) : 0.0;
  };
  if (!polymer) {
    for (int j = tid; j < M; j += nt) {
      double qx, qy;
      shifted(n, j, qx, qy);
      q[j] = qx;
      q[M + j] = qy;
      q[2 * M + j] = vext(d, qx, qy);
      if (phys_pair) cs.qq[j] = qpos(d, qx, qy);
    }
    G::sync();
  }
  double ws[2] = {0.0, 0.0};
  for (int k = tid; k < np * M; k += nt) {
    const int i = pol[k / M], j = k % M;
    const int jn = j + 1 == M ? 0 : j + 1, in = j == M - 1 ? c.next[i] : i;
    ws[0] += c.Vl(i, j);
    if (!polymer) {
      ws[1] += mhtau * (q[2 * M + j] + q[2 * M + jn]);
    } else {
      double qx, qy, qnx, qny;
      shifted(i, j, qx, qy);
      shifted(in, jn, qnx, qny);
      ws[1] += mhtau * (vext(d, qx, qy) + vext(d, qnx, qny));
    }
  }
  int dec = -1;
  if (phys_pair) {
    // warps split the links, lanes the particles of each slice; pairs inside
    // the cycle keep their relative positions under the rigid shift
    // a cycle's shifted centres: the mirror words plus the shift in mirror
    // units (one more rounding, inside the prefilter bound)
    const unsigned qsh = ((unsigned)__double2ll_rn(shx * d.q_scale) & 0xffffu) |
                         (dim > 1 ? ((unsigned)__double2ll_rn(shy * d.q_scale) & 0xffffu) << 16 : 0u);
    ComSeg seg{&c, pol, idx, M, polymer ? nullptr : q, shx, shy, L, inv2L, cs.qq, qsh};
    const int tot = np * M, per = (tot + nwarps - 1) / nwarps;
    const int t0 = min(tot, warp * per), t1 = min(tot, t0 + per);
    if (D::kSweep && !(d.flags & (PF_EXACT | PF_CONTACT))) {
      // bounded estimate from the mirror; the exact sums only when its
      // interval straddles the Metropolis threshold
      PairEst e = {0.f, 0.f, 0.f, 0.f, 0, 0};
      if (t0 < t1) segment_estimate(c, seg, t0, t1, e, lane);
      double v[6], l4[4];
      est_reduce_lanes(e, l4);
      for (int k = 0; k < 4; ++k) v[k] = l4[k];
      v[4] = ws[0];
      v[5] = ws[1];
      G::template sum<6>(v, red);
      const double h = d.mhtau_g;
      const double centre = v[5] - v[4] + h * (v[2] - v[0]);
      const double radius = fabs(h) * (v[1] + v[3]);
      dec = decide_interval(centre - radius, centre + radius, dr.uniform_accept());
    }
    if (dec == -1)
      segment_pairs(c, seg, t0, t1, true, true, qbuf + (size_t)warp * PQ_CAP, ws[0], ws[1], lane);
  }
  int acc = dec;
  if (dec == -1) {
    G::template sum<2>(ws, red);
    if (tid == 0) {
      *sflag = metropolis(d, ws[1] - ws[0], dr);
    }
    G::sync();
    acc = *sflag;
    G::sync();
  }
  if (!acc) return RES_REJECT;
  // links first (they read the unshifted neighbours), then positions
  for (int k = tid; k < np * M; k += nt) {
    const int i = pol[k / M], j = k % M;
    const int jn = j + 1 == M ? 0 : j + 1, in = j == M - 1 ? c.next[i] : i;
    if (!polymer) {
      c.Vl(i, j) = mhtau * (q[2 * M + j] + q[2 * M + jn]);
    } else {
      double qx, qy, qnx, qny;
      shifted(i, j, qx, qy);
      shifted(in, jn, qnx, qny);
      c.Vl(i, j) = mhtau * (vext(d, qx, qy) + vext(d, qnx, qny));
    }
  }
  G::sync();
  // one thread writes a slice's beads, in cycle order (the order in which
  // the cell lists record the moves is then fixed)
  for (int j = tid; j < M; j += nt)
    for (int p = 0; p < np; ++p) {
      const int i = pol[p];
      double qx, qy;
      if (!polymer) {
        qx = q[j];
        qy = q[M + j];
      } else {
        shifted(i, j, qx, qy);
      }
      c.set_pos(i, j, qx, qy);
    }
  G::sync();
  return RES_ACCEPT;
}

// floor((x + L) / w) with the division replaced by a multiplication unless
// the quotient lies within 1e-9 of an integer (then the IEEE division decides)
__device__ __forceinline__ long long bin_floor(double x, double L, double w, double inv_w) {
  const double q = (x + L) * inv_w;
  double f = floor(q);
  const double fr = q - f;
  if (fr < 1e-9 || fr > 1.0 - 1e-9) f = floor((x + L) / w);
  return (long long)f;
}

// ---------------------------------------------------------------------------
// estimators, whole CTA (src/measurement.jl:45-55, 92-122, and the radial
// distribution and superfluid estimators its TODOs name, 125-127)
// out[0] E_th, out[1] E_v, out[2] pair energy, out[3] pair virial energy,
// out[4] W^2 = |sum over links of the minimum-image displacement|^2 (winding),
// out[5] A_z = 1/2 sum over links (x dy - y dx) (signed area about the origin),
// out[6] sum r^2 / M (classical moment of inertia / m), out[7] 0;
// qbuf: one PQ_CAP-entry queue per warp (pair chains).
// FAST (the sweeps' measurements): a neighbour pair's exponentials are FP32
// expf of the FP64 squared distances (relative error about 1e-7 per term,
// far below any Monte Carlo error), so that the FP64 pipe only forms the
// distances, the exact cut-off test and the sums; the neighbour set is the
// same.  Otherwise (pimc_measure) every term is FP64.
// ---------------------------------------------------------------------------
template <bool WARP, bool FAST = false>
__device__ void measure_group(const CV &c, double *red, double *out, bool density,
                              unsigned long long *qbuf) {
  using G = Group<WARP>;
  const ChainDesc &d = *c.d;
  const int N = c.N, M = c.M, dim = c.dim, tid = G::rank(), nt = G::size();
  const int lane = threadIdx.x & 31, warp = WARP ? 0 : (int)(threadIdx.x >> 5);
  const int nwarps = WARP ? 1 : (int)(blockDim.x >> 5);
  // the contact table carries no tau derivative: no pair energy for it
  const bool pair = (d.flags & PF_PAIR) != 0 && !(d.flags & PF_CONTACT);
  const double rc2 = d.rc * d.rc, cg = d.inv2s2;
  double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // link, pot, vkin, pair, pair virial
  double sf[4] = {0.0, 0.0, 0.0, 0.0};       // winding x, y, area, sum r^2
  const double inv_bw = density ? 1.0 / d.dens_bw : 0.0;
  for (int k = tid; k < N * M; k += nt) {
    const int j = k / N, i = k % N;
    const int in = j == M - 1 ? c.next[i] : i, jn = j + 1 == M ? 0 : j + 1;
    const double ax = c.X(0, i, j), ay = c.Xd(1, i, j);
    const double bx = c.X(0, in, jn), by = c.Xd(1, in, jn);
    s[0] += mi2(d, ax, ay, bx, by);
    s[1] += vext(d, ax, ay) + vext(d, bx, by);
    {
      double gx, gy;
      grad_vext(d, ax, ay, gx, gy);
      s[2] += ax * gx + (dim > 1 ? ay * gy : 0.0);
    }
    {
      const double dx = mi1(bx, ax, d.L, d.L2), dy = dim > 1 ? mi1(by, ay, d.L, d.L2) : 0.0;
      sf[0] += dx;
      sf[1] += dy;
      sf[2] += 0.5 * __dsub_rn(__dmul_rn(ax, dy), __dmul_rn(ay, dx));
      sf[3] += __dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay));
    }
    if (density) {
      const long long ib = bin_floor(ax, d.L, d.dens_bw, inv_bw);
      bool ok = ib >= 1 && ib <= d.dens_nb;
      long long idx = ib - 1;
      if (dim > 1) {
        const long long jb = bin_floor(ay, d.L, d.dens_bw, inv_bw);
        ok = ok && jb >= 1 && jb <= d.dens_nb;
        idx += (jb - 1) * d.dens_nb;
      }
      if (ok) atomicAdd(c.hist + idx, 1ull);
    }
  }
  if (pair && qbuf) {
    // warps split the beads; lanes test the higher-numbered particles of the
    // slice in FP32 and queue the survivors, evaluated 32 at a time in FP64
    unsigned long long *q = qbuf + (size_t)warp * PQ_CAP;
    const unsigned lt = (1u << lane) - 1u;
    const int tot = N * M, per = (tot + nwarps - 1) / nwarps;
    const int k0 = min(tot, warp * per), k1 = min(tot, k0 + per);
    int qn = 0;
    auto flush = [&]() {
      const int k = qn < 32 ? qn : 32;
      if (lane < k) {
        const unsigned long long e = q[lane];
        const int b = (int)(e >> 32), kk = (int)(e & 0xffffffffu);
        const int j = kk / N, i = kk % N;
        const int in = j == M - 1 ? c.next[i] : i, jn = j + 1 == M ? 0 : j + 1;
        const double r2a = mi2(d, c.X(0, i, j), c.Xd(1, i, j), c.X(0, b, j), c.Xd(1, b, j));
        if (r2a <= rc2) {
          const int bn = j == M - 1 ? c.next[b] : b;
          // the pair exponentials e = exp(x), x = -r^2/(2 s^2), and x e; the
          // factors g tau/2 are applied once at the end
          if (FAST) {
            const float dxb = (float)mi1(c.X(0, in, jn), c.X(0, bn, jn), d.L, d.L2);
            const float dyb = dim > 1 ? (float)mi1(c.Xd(1, in, jn), c.Xd(1, bn, jn), d.L, d.L2) : 0.f;
            const float cgf = (float)cg;
            const float xa = -(float)r2a * cgf, xb = -fmaf(dxb, dxb, dyb * dyb) * cgf;
            const float ea = expf(xa), eb = expf(xb);
            s[3] += (double)(ea + eb);
            s[4] += (double)fmaf(xa, ea, xb * eb);
          } else {
            const double r2b =
                mi2(d, c.X(0, in, jn), c.Xd(1, in, jn), c.X(0, bn, jn), c.Xd(1, bn, jn));
            const double xa = -r2a * cg, xb = -r2b * cg;
            const double ea = exp_neg(xa), eb = exp_neg(xb);
            s[3] += ea + eb;
            s[4] = fma(xa, ea, fma(xb, eb, s[4]));
          }
        }
      }
      __syncwarp();
      unsigned long long rest[3];
      const int nr = qn - k;
      for (int r = 0; r < 3; ++r) rest[r] = (lane + 32 * r < nr) ? q[32 + lane + 32 * r] : 0ull;
      __syncwarp();
      for (int r = 0; r < 3; ++r)
        if (lane + 32 * r < nr) q[lane + 32 * r] = rest[r];
      __syncwarp();
      qn = nr;
    };
    for (int kk = k0; kk < k1; ++kk) {
      const int j = kk / N, i = kk % N;
      Prefilter f;
      f.init_q(c.Q(i, j), d.q_lim_rc);
      const unsigned *row = c.xq + (size_t)j * c.ldn;
      // every lane calls push with whether its candidate b passed
      auto push = [&](int b, bool p) {
        const unsigned mk = __ballot_sync(0xffffffffu, p);
        if (p) {
          const int k = qn + __popc(mk & lt);
          if (check_ok(k < PQ_CAP, DERR_QUEUE, d))
            q[k] = ((unsigned long long)(unsigned)b << 32) | (unsigned)kk;
        }
        qn += __popc(mk);
#if PIMC_CHECK
        if (qn > PQ_CAP) qn = PQ_CAP;
#endif
        __syncwarp();
        if (qn >= 32) flush();
      };
      // partners of higher index: from the cell lists, or the rest of the row
      if (cell_query(c.cl, c.cl && c.cl->usable(j), j, f.c, f.c, lane,
                     [&](int b, bool v, unsigned) { push(b, v && b > i && f.pass(row[b])); }))
        continue;
      // two blocks of 32 partners at a time: both rows' words are loaded
      // before either is tested, and the queue takes both blocks with one
      // warp synchronisation (at most 31 + 64 = 95 < PQ_CAP entries before
      // it drains below 32 again)
      for (int b0 = i + 1; b0 < N; b0 += 64) {
        const int ba = b0 + lane, bb = ba + 32;
        const unsigned wa = ba < N ? row[ba] : 0u, wb = bb < N ? row[bb] : 0u;
        const bool pa = ba < N && f.pass(wa), pb = bb < N && f.pass(wb);
        const unsigned ma = __ballot_sync(0xffffffffu, pa), mb = __ballot_sync(0xffffffffu, pb);
        const unsigned long long tag = (unsigned)kk;
        if (pa) {
          const int k = qn + __popc(ma & lt);
          if (check_ok(k < PQ_CAP, DERR_QUEUE, d)) q[k] = ((unsigned long long)(unsigned)ba << 32) | tag;
        }
        if (pb) {
          const int k = qn + __popc(ma) + __popc(mb & lt);
          if (check_ok(k < PQ_CAP, DERR_QUEUE, d)) q[k] = ((unsigned long long)(unsigned)bb << 32) | tag;
        }
        qn += __popc(ma) + __popc(mb);
#if PIMC_CHECK
        if (qn > PQ_CAP) qn = PQ_CAP;
#endif
        __syncwarp();
        while (qn >= 32) flush();
      }
    }
    while (qn > 0) flush();
  }
  if (d.rdf_nb > 0) {
    // pair-distance histogram: warps split the beads, lanes the partners of
    // higher index; lanes with the same bin add once (match_any)
    const int tot = N * M;
    const int gw = WARP ? 0 : warp, ngw = WARP ? 1 : nwarps;
    const int ib_max = d.rdf_nb;
    for (int kk = gw; kk < tot; kk += ngw) {
      const int j = kk / N, i = kk % N;
      const double ax = c.X(0, i, j), ay = c.Xd(1, i, j);
      for (int b0 = i + 1; b0 < N; b0 += 32) {
        const int b = b0 + lane;
        int bin = -1;
        if (b < N) {
          const double dx = fabs(mi1(ax, c.X(0, b, j), d.L, d.L2));
          const double dy = dim > 1 ? fabs(mi1(ay, c.Xd(1, b, j), d.L, d.L2)) : 0.0;
          const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
          const double f = floor(r / d.rdf_dr);
          if (f < (double)ib_max) bin = (int)f;
        }
        const unsigned act = __ballot_sync(0xffffffffu, bin >= 0);
        if (bin >= 0) {
          const unsigned peers = __match_any_sync(act, bin);
          if (lane == __ffs(peers) - 1) atomicAdd(d.rdf + bin, (unsigned long long)__popc(peers));
        }
      }
    }
  }
  G::template sum<5>(s, red);
  G::template sum<4>(sf, red);
  if (tid == 0) {
    const double tau = d.tau;
    out[4] = sf[0] * sf[0] + sf[1] * sf[1];
    out[5] = sf[2];
    out[6] = sf[3] / M;
    out[7] = 0.0;
    out[0] = (double)(dim * N) / (2.0 * tau) - 1.0 / (4.0 * d.lambda * (tau * tau) * M) * s[0] +
             1.0 / (2.0 * M) * s[1];
    out[1] = 1.0 / (2.0 * M) * s[2] + 1.0 / (2.0 * M) * s[1];
    // pair energy sum (tau/2) g (e_a + e_b) / (M tau) and its virial part
    // sum (tau/2) g (-2 r^2/(2 s^2)) (e_a, e_b) / (2 M tau)
    out[2] = pair ? d.g * s[3] / (2.0 * M) : 0.0;
    out[3] = pair ? out[2] + d.g * s[4] / (2.0 * M) : 0.0;
  }
}

}  // namespace pimc
