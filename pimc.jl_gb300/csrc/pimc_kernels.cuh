// pimc_kernels.cuh -- CTA-level moves (permutation swap, centre-of-mass
// shifts), estimators, and the sweep driver executed by one CTA per chain.
#pragma once
#include "pimc_device.cuh"

namespace pimc {

// ---------------------------------------------------------------------------
// block reductions (red: >= 256 doubles of shared memory; K <= 6)
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void block_sum_k(double (&v)[K], double *red) {
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
    double s = lane < nw ? red[k * 32 + lane] : 0.0;
    v[k] = warp_sum(s);
  }
  __syncthreads();
}

template <int K>
__device__ __forceinline__ void block_max_k(double (&v)[K], double *red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_max(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) red[k * 32 + w] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double s = lane < nw ? red[k * 32 + lane] : -INFINITY;
    v[k] = warp_max(s);
  }
  __syncthreads();
}

__device__ __forceinline__ int block_min_int(int v, int *ired) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) ired[w] = v;
  __syncthreads();
  int s = lane < nw ? ired[lane] : 0x7fffffff;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s = min(s, __shfl_xor_sync(0xffffffffu, s, o));
  __syncthreads();
  return s;
}

// exclusive prefix over the block of one double per thread
__device__ __forceinline__ double block_exclusive_scan(double v, double *red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  double incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  __syncthreads();
  if (lane == 31) red[w] = incl;
  __syncthreads();
  double base = 0.0;
  for (int q = 0; q < w && q < nw; ++q) base += red[q];
  __syncthreads();
  return base + incl - v;
}

__device__ __forceinline__ double logaddexp(double a, double b) {
  const double mx = fmax(a, b);
  if (mx == -INFINITY) return -INFINITY;
  return mx + log(exp(a - mx) + exp(b - mx));
}

// shared scratch of the swap: doubles then ints
struct SwapScratch {
  double *w;              // N heat-bath weights
  double *r1x, *r1y, *r2x, *r2y, *vb1, *vb2;  // WMAX+1 each
  double *z;              // 2*WMAX*2 normals
  int *pa, *pb, *ca, *cb; // M each
  static __host__ __device__ size_t bytes(int N, int M) {
    return sizeof(double) * ((size_t)N + 6 * (WMAX + 1) + 4 * WMAX) + sizeof(int) * 4 * (size_t)M;
  }
  __device__ void carve(void *base, int N, int M) {
    double *p = (double *)base;
    w = p; p += N;
    r1x = p; p += WMAX + 1; r1y = p; p += WMAX + 1;
    r2x = p; p += WMAX + 1; r2y = p; p += WMAX + 1;
    vb1 = p; p += WMAX + 1; vb2 = p; p += WMAX + 1;
    z = p; p += 4 * WMAX;
    int *q = (int *)p;
    pa = q; q += M; pb = q; q += M; ca = q; q += M; cb = q;
  }
};

// ---------------------------------------------------------------------------
// permutation swap, whole CTA: (u::ReshapeSwapLinear)(s) with the heat-bath
// partner choice sampleparticles (src/updates/reshape.jl:123-283,
// src/updates/helper.jl:224-267).  Returns RES_*; *n2_out receives n2.
// ---------------------------------------------------------------------------
template <class D>
__device__ int swap_cta(const CV &c, int j0, int m, int n1, double u_pick, D &dr, SwapScratch &S,
                        double *red, int *ired, int *sflag, double *prop, int *n2_out,
                        bool update_cells) {
  const ChainDesc &d = *c.d;
  const int N = c.N, M = c.M, dim = c.dim, tid = threadIdx.x, nt = blockDim.x;
  const double L = d.L, inv2L = 1.0 / (2.0 * L), mhtau = -0.5 * d.tau;
  const bool wrap = (j0 + m) >= M;
  const int se = wrap ? j0 + m - M : j0 + m;
  const double taum = m * d.tau;
  const double den = 4.0 * taum * d.lambda;
  auto endp = [&](int i) { return wrap ? c.next[i] : i; };
  auto Xd = [&](int k, int n, int j) { return k < dim ? c.X(k, n, j) : 0.0; };
  const double ax = c.X(0, n1, j0), ay = Xd(1, n1, j0);
  const int e1p = endp(n1);
  const double e1x = c.X(0, e1p, se), e1y = Xd(1, e1p, se);
  // heat-bath weights exp(t_i + y_i), shifted by the maximum
  double vm[1] = {-INFINITY};
  for (int i = tid; i < N; i += nt) {
    const int ei = endp(i);
    const double t1 = -mi2(d, ax, ay, c.X(0, ei, se), Xd(1, ei, se)) / den;
    const double t2 = -mi2(d, c.X(0, i, j0), Xd(1, i, j0), e1x, e1y) / den;
    S.w[i] = t1 + t2;
    vm[0] = fmax(vm[0], t1 + t2);
  }
  block_max_k<1>(vm, red);
  const double wmax = vm[0];
  double vs[1] = {0.0};
  for (int i = tid; i < N; i += nt) {
    const double e = exp(S.w[i] - wmax);
    S.w[i] = e;
    vs[0] += e;
  }
  block_sum_k<1>(vs, red);
  const double ssum = vs[0];
  double vq[1] = {0.0};
  for (int i = tid; i < N; i += nt) {
    const double q = S.w[i] / ssum;
    S.w[i] = q;
    vq[0] += q;
  }
  block_sum_k<1>(vq, red);
  const double target = u_pick * vq[0];
  // first i with cumulative weight >= target (StatsBase.sample)
  const int chunk = (N + nt - 1) / nt;
  const int i0 = min(N, tid * chunk), i1 = min(N, i0 + chunk);
  double loc = 0.0;
  for (int i = i0; i < i1; ++i) loc += S.w[i];
  double cw = block_exclusive_scan(loc, red);
  int cand = 0x7fffffff;
  for (int i = i0; i < i1; ++i) {
    cw += S.w[i];
    if (cw >= target) { cand = i; break; }
  }
  int n2 = block_min_int(cand, ired);
  if (n2 >= N) n2 = N - 1;
  if (n2_out && tid == 0) *n2_out = n2;
  if (n2 == n1) return RES_SKIP;

  double log_ratio = 0.0;
  if (d.flags & PF_PHYS) {
    // (1/S'_1 + 1/S'_2) / (1/S_1 + 1/S_2): S_a sums the heat-bath weights
    // with a chosen first; primes after the ends of n1 and n2 are exchanged
    const double l1 = wmax + log(ssum);
    const double bx = c.X(0, n2, j0), by = Xd(1, n2, j0);
    const int e2p = endp(n2);
    const double e2x = c.X(0, e2p, se), e2y = Xd(1, e2p, se);
    double wv[3];
    double mx3[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = tid; i < N; i += nt) {
      const int ei = endp(i);
      const double ex = c.X(0, ei, se), ey = Xd(1, ei, se);
      const double epx = i == n1 ? e2x : (i == n2 ? e1x : ex);
      const double epy = i == n1 ? e2y : (i == n2 ? e1y : ey);
      const double xi = c.X(0, i, j0), yi = Xd(1, i, j0);
      wv[0] = -mi2(d, bx, by, ex, ey) / den - mi2(d, xi, yi, e2x, e2y) / den;
      wv[1] = -mi2(d, ax, ay, epx, epy) / den - mi2(d, xi, yi, e2x, e2y) / den;
      wv[2] = -mi2(d, bx, by, epx, epy) / den - mi2(d, xi, yi, e1x, e1y) / den;
#pragma unroll
      for (int k = 0; k < 3; ++k) mx3[k] = fmax(mx3[k], wv[k]);
    }
    block_max_k<3>(mx3, red);
    double s3[3] = {0.0, 0.0, 0.0};
    for (int i = tid; i < N; i += nt) {
      const int ei = endp(i);
      const double ex = c.X(0, ei, se), ey = Xd(1, ei, se);
      const double epx = i == n1 ? e2x : (i == n2 ? e1x : ex);
      const double epy = i == n1 ? e2y : (i == n2 ? e1y : ey);
      const double xi = c.X(0, i, j0), yi = Xd(1, i, j0);
      s3[0] += exp(-mi2(d, bx, by, ex, ey) / den - mi2(d, xi, yi, e2x, e2y) / den - mx3[0]);
      s3[1] += exp(-mi2(d, ax, ay, epx, epy) / den - mi2(d, xi, yi, e2x, e2y) / den - mx3[1]);
      s3[2] += exp(-mi2(d, bx, by, epx, epy) / den - mi2(d, xi, yi, e1x, e1y) / den - mx3[2]);
    }
    block_sum_k<3>(s3, red);
    const double l2 = mx3[0] + log(s3[0]);
    const double l1p = mx3[1] + log(s3[1]);
    const double l2p = mx3[2] + log(s3[2]);
    log_ratio = logaddexp(-l1p, -l2p) - logaddexp(-l1, -l2);
  }

  // two bridges with exchanged ends
  const int nx1 = c.next[n1], nx2 = c.next[n2];
  auto own1 = [&](int t) { return (j0 + t < M) ? n1 : nx1; };
  auto own2 = [&](int t) { return (j0 + t < M) ? n2 : nx2; };
  auto slc = [&](int t) { return (j0 + t < M) ? j0 + t : j0 + t - M; };
  const double s1x = ax, s1y = ay, s2x = c.X(0, n2, j0), s2y = Xd(1, n2, j0);
  const int e2p = endp(n2);
  double f1x = c.X(0, e2p, se), f1y = Xd(1, e2p, se);  // r1 ends at E(n2)
  double f2x = e1x, f2y = e1y;                            // r2 ends at E(n1)
  if (fabs(s1x - f1x) > L) f1x += sgn(s1x) * (2.0 * L);
  if (dim > 1 && fabs(s1y - f1y) > L) f1y += sgn(s1y) * (2.0 * L);
  if (fabs(s2x - f2x) > L) f2x += sgn(s2x) * (2.0 * L);
  if (dim > 1 && fabs(s2y - f2y) > L) f2y += sgn(s2y) * (2.0 * L);
  const bool hard = (d.flags & PF_HARD) != 0;
  if (!hard) {
    for (int k = tid; k < 2 * (m - 1); k += nt) {
      double zz[2];
      dr.bead_normals(k, dim, zz);
      S.z[2 * k] = zz[0];
      S.z[2 * k + 1] = dim > 1 ? zz[1] : 0.0;
    }
    dr.consumed(2 * (m - 1) * dim);
    __syncthreads();
    if (tid < 2 * dim) {
      const int b = tid / dim, k = tid % dim;
      double p = b == 0 ? (k == 0 ? s1x : s1y) : (k == 0 ? s2x : s2y);
      const double e = b == 0 ? (k == 0 ? f1x : f1y) : (k == 0 ? f2x : f2y);
      double *dst = b == 0 ? (k == 0 ? S.r1x : S.r1y) : (k == 0 ? S.r2x : S.r2y);
      for (int t = 1; t < m; ++t) {
        const double2 ab = bridge_coef(c, m, t);
        p = ab.x * p + (1.0 - ab.x) * e + S.z[2 * (b * (m - 1) + t - 1) + k] * ab.y;
        dst[t] = p;
      }
    }
    if (tid == 0) *sflag = 0;
  } else if (tid == 0) {
    int fail = 0;
    for (int b = 0; b < 2 && !fail; ++b) {
      double px = b == 0 ? s1x : s2x, py = b == 0 ? s1y : s2y;
      const double ex = b == 0 ? f1x : f2x, ey = b == 0 ? f1y : f2y;
      double *dx = b == 0 ? S.r1x : S.r2x, *dy = b == 0 ? S.r1y : S.r2y;
      for (int t = 1; t < m && !fail; ++t) {
        const double2 ab = bridge_coef(c, m, t);
        const int j = slc(t);
        const int ea = (d.flags & PF_PHYS) ? own1(t) : (b == 0 ? n2 : n1);
        const int eb = (d.flags & PF_PHYS) ? own2(t) : -1;
        int tries = 0;
        while (true) {
          if (++tries > d.ctr) { fail = 1; break; }
          const double z0 = dr.normal(), z1 = dim > 1 ? dr.normal() : 0.0;
          const double qx = ab.x * px + (1.0 - ab.x) * ex + z0 * ab.y;
          const double qy = dim > 1 ? ab.x * py + (1.0 - ab.x) * ey + z1 * ab.y : 0.0;
          if (!hard_hit(c, teleport(qx, L, inv2L), dim > 1 ? teleport(qy, L, inv2L) : 0.0, j, ea,
                        eb)) {
            px = qx; py = qy;
            break;
          }
        }
        dx[t] = px;
        dy[t] = py;
      }
    }
    *sflag = fail;
  }
  __syncthreads();
  if (*sflag) return RES_HARDCORE;
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
    qx = teleport(qx, L, inv2L);
    if (dim > 1) qy = teleport(qy, L, inv2L); else qy = 0.0;
    (b == 0 ? S.r1x : S.r2x)[t] = qx;
    (b == 0 ? S.r1y : S.r2y)[t] = qy;
    (b == 0 ? S.vb1 : S.vb2)[t] = vext(d, qx, qy);
  }
  __syncthreads();
  const bool any_pair = (d.flags & PF_PAIR) != 0, phys = (d.flags & PF_PHYS) != 0;
  double ws[2] = {0.0, 0.0};
  for (int k = tid; k < 2 * m; k += nt) {
    const int b = k / m, t = k % m;
    const int j = slc(t), o = b == 0 ? own1(t) : own2(t);
    const int on = b == 0 ? own1(t + 1) : own2(t + 1), jn = slc(t + 1);
    const double *bxs = b == 0 ? S.r1x : S.r2x, *bys = b == 0 ? S.r1y : S.r2y;
    const double *vb = b == 0 ? S.vb1 : S.vb2;
    ws[0] += c.Vl(o, j);
    ws[1] += mhtau * (vb[t] + vb[t + 1]);
    if (any_pair) {
      const double ox = c.X(0, o, j), oy = Xd(1, o, j), onx = c.X(0, on, jn), ony = Xd(1, on, jn);
      if (!phys) {
        // the reference: old pairs exclude only the path's own particle,
        // the new paths' pair terms are added to w_initial
        ws[0] += pair_link(c, ox, oy, onx, ony, j, o, -1);
        ws[0] += pair_link(c, bxs[t], bys[t], bxs[t + 1], bys[t + 1], j, own1(t), own2(t));
      } else {
        ws[0] += pair_link(c, ox, oy, onx, ony, j, own1(t), own2(t));
        ws[1] += pair_link(c, bxs[t], bys[t], bxs[t + 1], bys[t + 1], j, own1(t), own2(t));
        if (b == 0) {
          const int o2 = own2(t), o2n = own2(t + 1);
          ws[0] += pair_cross(d, ox, oy, onx, ony, c.X(0, o2, j), Xd(1, o2, j), c.X(0, o2n, jn),
                              Xd(1, o2n, jn));
          ws[1] += pair_cross(d, S.r1x[t], S.r1y[t], S.r1x[t + 1], S.r1y[t + 1], S.r2x[t],
                              S.r2y[t], S.r2x[t + 1], S.r2y[t + 1]);
        }
      }
    }
  }
  block_sum_k<2>(ws, red);
  if (prop)
    for (int k = tid; k < 2 * (m + 1); k += nt) {
      const int b = k / (m + 1), t = k % (m + 1);
      prop[k * dim] = (b == 0 ? S.r1x : S.r2x)[t];
      if (dim > 1) prop[k * dim + 1] = (b == 0 ? S.r1y : S.r2y)[t];
    }
  if (tid == 0) {
    const double delta = exp(ws[1] - ws[0] + log_ratio);
    *sflag = (delta >= 1.0) || (delta > dr.uniform_accept());
  }
  __syncthreads();
  const int acc = *sflag;
  if (!acc) return RES_REJECT;
  // accept: exchange next, write the bridges along the new cycles, exchange
  // the tails (reshape.jl:247-279)
  const int nn1 = nx2, nn2 = nx1;  // next after the exchange
  auto nown1 = [&](int t) { return (j0 + t < M) ? n1 : nn1; };
  auto nown2 = [&](int t) { return (j0 + t < M) ? n2 : nn2; };
  const bool tail = (j0 + m) < M - 1;
  if (update_cells) {
    for (int j = tid; j < M; j += nt) {
      const int t = (j - j0 + M) % M;
      int pa = -1, pb = -1;
      if (t >= 1 && t <= m) { pa = nown1(t); pb = nown2(t); }
      else if (tail && j > se) { pa = n1; pb = n2; }
      S.pa[j] = pa;
      S.pb[j] = pb;
      S.ca[j] = pa >= 0 ? cell_of(d, c.X(0, pa, j), Xd(1, pa, j)) : -1;
      S.cb[j] = pb >= 0 ? cell_of(d, c.X(0, pb, j), Xd(1, pb, j)) : -1;
    }
  }
  __syncthreads();
  if (tid == 0) {
    c.next[n1] = nn1;
    c.next[n2] = nn2;
  }
  for (int t = 1 + tid; t <= m; t += nt) {
    const int j = slc(t);
    c.X(0, nown1(t), j) = S.r1x[t];
    c.X(0, nown2(t), j) = S.r2x[t];
    if (dim > 1) {
      c.X(1, nown1(t), j) = S.r1y[t];
      c.X(1, nown2(t), j) = S.r2y[t];
    }
  }
  for (int t = tid; t < m; t += nt) {
    const int j = slc(t);
    c.Vl(nown1(t), j) = mhtau * (S.vb1[t] + S.vb1[t + 1]);
    c.Vl(nown2(t), j) = mhtau * (S.vb2[t] + S.vb2[t + 1]);
  }
  if (tail)
    for (int j = se + 1 + tid; j < M; j += nt) {
      for (int k = 0; k < dim; ++k) {
        const double a = c.X(k, n1, j);
        c.X(k, n1, j) = c.X(k, n2, j);
        c.X(k, n2, j) = a;
      }
      const double v = c.Vl(n1, j);
      c.Vl(n1, j) = c.Vl(n2, j);
      c.Vl(n2, j) = v;
    }
  if (phys && !wrap && tid == 0) {
    // the link leaving the end bead moves with the tail
    const double v = c.Vl(n1, se);
    c.Vl(n1, se) = c.Vl(n2, se);
    c.Vl(n2, se) = v;
  }
  __syncthreads();
  if (update_cells) {
    for (int j = tid; j < M; j += nt) {
      if (S.pa[j] >= 0)
        cell_move(c, S.pa[j], j, S.ca[j], cell_of(d, c.X(0, S.pa[j], j), Xd(1, S.pa[j], j)));
      if (S.pb[j] >= 0)
        cell_move(c, S.pb[j], j, S.cb[j], cell_of(d, c.X(0, S.pb[j], j), Xd(1, S.pb[j], j)));
    }
    __syncthreads();
  }
  return RES_ACCEPT;
}

// ---------------------------------------------------------------------------
// single-path centre of mass, one warp: (u::SingleCenterOfMass)(s) with
// move_polymer! (src/updates/com.jl:136-224, src/updates/helper.jl:368-395).
// sb: per-warp shared scratch of 3*M doubles.
// ---------------------------------------------------------------------------
template <class D>
__device__ int com_warp(const CV &c, int n, double step, D &dr, double *sb, bool update_cells) {
  const ChainDesc &d = *c.d;
  const int lane = threadIdx.x & 31, M = c.M, dim = c.dim;
  const double L = d.L, inv2L = 1.0 / (2.0 * L), mhtau = -0.5 * d.tau;
  const bool hard = (d.flags & PF_HARD) != 0;
  const bool phys_pair = (d.flags & PF_PAIR) && (d.flags & PF_PHYS);
  double *qx_ = sb, *qy_ = sb + M, *vb = sb + 2 * M;
  int tries = 0, fail = 0;
  double shx = 0.0, shy = 0.0;
  while (true) {
    if (lane == 0) {
      if (++tries > d.ctr) {
        fail = 1;
      } else {
        shx = step * 2.0 * (dr.uniform() - 0.5);
        shy = dim > 1 ? step * 2.0 * (dr.uniform() - 0.5) : 0.0;
      }
    }
    fail = __shfl_sync(0xffffffffu, fail, 0);
    if (fail) break;
    shx = __shfl_sync(0xffffffffu, shx, 0);
    shy = __shfl_sync(0xffffffffu, shy, 0);
    bool hit = false;
    for (int j = lane; j < M; j += 32) {
      const double qx = teleport(c.X(0, n, j) + shx, L, inv2L);
      const double qy = dim > 1 ? teleport(c.X(1, n, j) + shy, L, inv2L) : 0.0;
      qx_[j] = qx;
      qy_[j] = qy;
      if (hard && hard_hit(c, qx, qy, j, n, -1)) hit = true;
    }
    if (!__any_sync(0xffffffffu, hit)) break;
  }
  if (fail) return RES_HARDCORE;
  for (int j = lane; j < M; j += 32) vb[j] = vext(d, qx_[j], qy_[j]);
  __syncwarp();
  double wi = 0.0, wu = 0.0;
  for (int j = lane; j < M; j += 32) {
    const int jn = j + 1 == M ? 0 : j + 1;
    wi += c.Vl(n, j);
    wu += mhtau * (vb[j] + vb[jn]);
    if (phys_pair) {
      wi += pair_link(c, c.X(0, n, j), dim > 1 ? c.X(1, n, j) : 0.0, c.X(0, n, jn),
                      dim > 1 ? c.X(1, n, jn) : 0.0, j, n, -1);
      wu += pair_link(c, qx_[j], qy_[j], qx_[jn], qy_[jn], j, n, -1);
    }
  }
  wi = warp_sum(wi);
  wu = warp_sum(wu);
  int acc = 0;
  if (lane == 0) {
    const double delta = exp(wu - wi);
    acc = (delta >= 1.0) || (delta > dr.uniform_accept());
  }
  acc = __shfl_sync(0xffffffffu, acc, 0);
  if (acc) {
    for (int j = lane; j < M; j += 32) {
      const int jn = j + 1 == M ? 0 : j + 1;
      if (update_cells)
        cell_move(c, n, j, cell_of(d, c.X(0, n, j), dim > 1 ? c.X(1, n, j) : 0.0),
                  cell_of(d, qx_[j], qy_[j]));
      c.X(0, n, j) = qx_[j];
      if (dim > 1) c.X(1, n, j) = qy_[j];
      c.Vl(n, j) = mhtau * (vb[j] + vb[jn]);
    }
  }
  __syncwarp();
  return acc;
}

// ---------------------------------------------------------------------------
// cycle centre of mass, whole CTA: PolymerCenterOfMass (src/updates/com.jl:31-104)
// without the worm fields that make the reference's version fail.
// pol/idx: int scratch of 2N.
// ---------------------------------------------------------------------------
template <class D>
__device__ int pcom_cta(const CV &c, int n, double step, D &dr, int *pol, int *idx, double *red,
                        int *sflag, int *np_out, bool update_cells) {
  const ChainDesc &d = *c.d;
  const int N = c.N, M = c.M, dim = c.dim, tid = threadIdx.x, nt = blockDim.x;
  const double L = d.L, inv2L = 1.0 / (2.0 * L), mhtau = -0.5 * d.tau;
  const bool hard = (d.flags & PF_HARD) != 0;
  const bool phys_pair = (d.flags & PF_PAIR) && (d.flags & PF_PHYS);
  for (int i = tid; i < N; i += nt) idx[i] = -1;
  __syncthreads();
  if (tid == 0) {
    int np = 0, i = n;
    do {
      pol[np++] = i;
      i = c.next[i];
    } while (i != n && np <= N);
    *sflag = np;
  }
  __syncthreads();
  const int np = *sflag;
  if (np_out && tid == 0) *np_out = np;
  if (np > N) return -1;
  for (int i = tid; i < np; i += nt) idx[pol[i]] = i;
  __syncthreads();
  double *shift = red + 224;  // two doubles beyond the reduction slots
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
    __syncthreads();
    if (*sflag < 0) return RES_HARDCORE;
    if (!hard) break;
    int hit = 0;
    for (int k = tid; k < np * M; k += nt) {
      const int i = pol[k / M], j = k % M;
      const double qx = teleport(c.X(0, i, j) + shift[0], L, inv2L);
      const double qy = dim > 1 ? teleport(c.X(1, i, j) + shift[1], L, inv2L) : 0.0;
      if (hard_hit(c, qx, qy, j, i, -1)) hit = 1;
    }
    if (!__syncthreads_or(hit)) break;
  }
  const double shx = shift[0], shy = shift[1];
  double ws[2] = {0.0, 0.0};
  for (int k = tid; k < np * M; k += nt) {
    const int i = pol[k / M], j = k % M;
    const int jn = j + 1 == M ? 0 : j + 1, in = j == M - 1 ? c.next[i] : i;
    const double ox = c.X(0, i, j), oy = dim > 1 ? c.X(1, i, j) : 0.0;
    const double onx = c.X(0, in, jn), ony = dim > 1 ? c.X(1, in, jn) : 0.0;
    const double qx = teleport(ox + shx, L, inv2L), qy = dim > 1 ? teleport(oy + shy, L, inv2L) : 0.0;
    const double qnx = teleport(onx + shx, L, inv2L);
    const double qny = dim > 1 ? teleport(ony + shy, L, inv2L) : 0.0;
    ws[0] += c.Vl(i, j);
    ws[1] += mhtau * (vext(d, qx, qy) + vext(d, qnx, qny));
    if (phys_pair) {
      // pairs with particles outside the cycle; pairs inside it keep their
      // relative positions under the rigid shift
      int cells[9];
      for (int side = 0; side < 2; ++side) {
        const double px = side ? qx : ox, py = side ? qy : oy;
        const double pnx = side ? qnx : onx, pny = side ? qny : ony;
        const int nc = stencil(d, cell_of(d, px, py), cells);
        double w = 0.0;
        for (int ci = 0; ci < nc; ++ci)
          for (int b = c.head[(size_t)j * d.ncell + cells[ci]]; b >= 0; b = c.cn[(size_t)j * N + b]) {
            if (idx[b] >= 0) continue;
            const int bn = j == M - 1 ? c.next[b] : b;
            w += pair_cross(d, px, py, pnx, pny, c.X(0, b, j), dim > 1 ? c.X(1, b, j) : 0.0,
                            c.X(0, bn, jn), dim > 1 ? c.X(1, bn, jn) : 0.0);
          }
        ws[side] += w;
      }
    }
  }
  block_sum_k<2>(ws, red);
  if (tid == 0) {
    const double delta = exp(ws[1] - ws[0]);
    *sflag = (delta >= 1.0) || (delta > dr.uniform_accept());
  }
  __syncthreads();
  const int acc = *sflag;
  if (!acc) return RES_REJECT;
  // links first (they read the unshifted neighbours), then positions per slice
  for (int k = tid; k < np * M; k += nt) {
    const int i = pol[k / M], j = k % M;
    const int jn = j + 1 == M ? 0 : j + 1, in = j == M - 1 ? c.next[i] : i;
    const double qx = teleport(c.X(0, i, j) + shx, L, inv2L);
    const double qy = dim > 1 ? teleport(c.X(1, i, j) + shy, L, inv2L) : 0.0;
    const double qnx = teleport(c.X(0, in, jn) + shx, L, inv2L);
    const double qny = dim > 1 ? teleport(c.X(1, in, jn) + shy, L, inv2L) : 0.0;
    c.Vl(i, j) = mhtau * (vext(d, qx, qy) + vext(d, qnx, qny));
  }
  __syncthreads();
  for (int j = tid; j < M; j += nt)
    for (int q = 0; q < np; ++q) {
      const int i = pol[q];
      const double qx = teleport(c.X(0, i, j) + shx, L, inv2L);
      const double qy = dim > 1 ? teleport(c.X(1, i, j) + shy, L, inv2L) : 0.0;
      if (update_cells)
        cell_move(c, i, j, cell_of(d, c.X(0, i, j), dim > 1 ? c.X(1, i, j) : 0.0),
                  cell_of(d, qx, qy));
      c.X(0, i, j) = qx;
      if (dim > 1) c.X(1, i, j) = qy;
    }
  __syncthreads();
  return RES_ACCEPT;
}

// ---------------------------------------------------------------------------
// estimators, whole CTA (src/measurement.jl:45-55, 92-122)
// out[0] E_th, out[1] E_v, out[2] pair energy, out[3] pair virial energy
// ---------------------------------------------------------------------------
__device__ void measure_cta(const CV &c, double *red, double *out, bool density) {
  const ChainDesc &d = *c.d;
  const int N = c.N, M = c.M, dim = c.dim, tid = threadIdx.x, nt = blockDim.x;
  const bool pair = (d.flags & PF_PAIR) != 0;
  const double rc2 = d.rc * d.rc, cg = d.inv2s2;
  double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // link, pot, vkin, pair, pair virial
  for (int k = tid; k < N * M; k += nt) {
    const int i = k / M, j = k % M;
    const int in = j == M - 1 ? c.next[i] : i, jn = j + 1 == M ? 0 : j + 1;
    const double ax = c.X(0, i, j), ay = dim > 1 ? c.X(1, i, j) : 0.0;
    const double bx = c.X(0, in, jn), by = dim > 1 ? c.X(1, in, jn) : 0.0;
    s[0] += mi2(d, ax, ay, bx, by);
    s[1] += vext(d, ax, ay) + vext(d, bx, by);
    s[2] += ax * dvext(d, ax) + (dim > 1 ? ay * dvext(d, ay) : 0.0);
    if (pair) {
      int cells[9];
      const int nc = stencil(d, cell_of(d, ax, ay), cells);
      for (int ci = 0; ci < nc; ++ci)
        for (int b = c.head[(size_t)j * d.ncell + cells[ci]]; b >= 0; b = c.cn[(size_t)j * N + b]) {
          if (b <= i) continue;
          const double r2a = mi2(d, ax, ay, c.X(0, b, j), dim > 1 ? c.X(1, b, j) : 0.0);
          if (r2a > rc2) continue;
          const int bn = j == M - 1 ? c.next[b] : b;
          const double r2b = mi2(d, bx, by, c.X(0, bn, jn), dim > 1 ? c.X(1, bn, jn) : 0.0);
          const double v1 = vpair(d, r2a), v2 = vpair(d, r2b);
          s[3] += 0.5 * d.tau * (v1 + v2);
          s[4] += 0.5 * d.tau * (-2.0 * cg * r2a * v1 - 2.0 * cg * r2b * v2);
        }
    }
    if (density) {
      const double bw = d.dens_bw;
      const long long ib = (long long)floor((ax + d.L) / bw);
      bool ok = ib >= 1 && ib <= d.dens_nb;
      long long idx = ib - 1;
      if (dim > 1) {
        const long long jb = (long long)floor((ay + d.L) / bw);
        ok = ok && jb >= 1 && jb <= d.dens_nb;
        idx += (jb - 1) * d.dens_nb;
      }
      if (ok) atomicAdd(c.hist + idx, 1ull);
    }
  }
  block_sum_k<5>(s, red);
  if (tid == 0) {
    const double tau = d.tau;
    out[0] = (double)(dim * N) / (2.0 * tau) - 1.0 / (4.0 * d.lambda * (tau * tau) * M) * s[0] +
             1.0 / (2.0 * M) * s[1];
    out[1] = 1.0 / (2.0 * M) * s[2] + 1.0 / (2.0 * M) * s[1];
    out[2] = pair ? s[3] / (M * tau) : 0.0;
    out[3] = pair ? out[2] + s[4] / (2.0 * M * tau) : 0.0;
  }
}

}  // namespace pimc
