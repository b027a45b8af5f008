// pimc_attempt.cu -- single moves with injected draws and the action
// evaluation kernels (the parity entry points), in a translation unit of
// their own so that they compile in parallel with the sweep kernels.
#include <cuda_runtime.h>

#include "pimc_sweep.cuh"

namespace pimc {

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
PIMC_UNIT_ACCESSORS(attempt)

}  // namespace pimc
