// pimc_launch.h -- kernel argument blocks and host launchers of the engine.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "pimc_types.h"

namespace pimc {

struct SweepArgs {
  const ChainDesc *desc;
  ChainVar *var;
  const MixDev *mix;
  double *dpool;
  int *ipool;
  unsigned long long *upool;
  int nchains;        // chains in this launch
  int chain0;         // first chain when no queue/order is used
  const int *order;   // chain order (LPT), or null
  int *queue;         // device work-queue head, or null (one chain per CTA)
  int sweeps;         // sweeps per chain per launch
  int state_bytes;    // shared bytes reserved for staging a chain's state
  int warp_scratch_d; // doubles of scratch per warp
  int warp_bytes;     // warp-per-chain mode: scratch bytes of each warp
  int teams;          // 1: staging slots walked by teams of warps (latency-bound
                      // launches whose chains all fit on the GPU at once)
};

struct AttemptArgs {
  const ChainDesc *desc;
  ChainVar *var;
  double *dpool;
  int *ipool;
  unsigned long long *upool;
  int chain, kind, n, j0, m;
  double u_pick, step;
  const double *normals;
  int n_normals;
  const double *uniforms;
  int n_uniforms;
  double *prop;
  int *out;           // result, extra, normals used, uniforms used, exhausted
  int force_warp;
};

struct EvalArgs {
  const ChainDesc *desc;
  double *dpool;
  int *ipool;
  unsigned long long *upool;
  int chain, n, j0, m;
  const double *rp;
  double *out;
};

struct AdjArgs {
  const ChainDesc *desc;
  double *dpool;
  int *ipool;
  int chain;
  double omega;
  double *gA, *gB;    // [N*M][2] scratch
  int *inv;           // [N] scratch
  double *part;       // [nblocks][8] scratch
  int nblocks;
  double *dSdr;       // [dim][N][M] or null
  double *totals;     // [8]
  double *sum_rg;     // [1], zeroed before the launch
};

// mode 0: one CTA per chain (k_sweep); mode 1: one warp per chain (k_sweep_warp)
cudaError_t launch_sweep(const SweepArgs &a, int mode, int grid, int block, size_t smem,
                         cudaStream_t s);
cudaError_t sweep_set_smem(int mode, size_t smem);
// the sweep as three launches per sweep (phase 0 staging, 1 swaps, 2 the
// rest), one CTA per chain; a.sweeps must be 1
cudaError_t launch_sweep_phase(const SweepArgs &a, int phase, int grid, int block, size_t smem,
                               cudaStream_t s);
cudaError_t sweep_phase_set_smem(int phase, size_t smem);
cudaError_t sweep_phase_occupancy(int phase, int block, size_t smem, int *blocks_per_sm);
size_t sweep_ctl_bytes();
cudaError_t sweep_occupancy(int mode, int block, size_t smem, int *blocks_per_sm);
cudaError_t launch_attempt(const AttemptArgs &a, size_t smem, cudaStream_t s);
cudaError_t launch_eval_action(const EvalArgs &a, cudaStream_t s);
cudaError_t launch_eval_weights(const EvalArgs &a, cudaStream_t s);
cudaError_t launch_init_world(const ChainDesc *desc, double *dpool, int *ipool, int chain0,
                              int nchains, int maxN, cudaStream_t s);
cudaError_t launch_links(const ChainDesc *desc, double *dpool, int *ipool, int chain0, int nchains,
                         int maxNM, cudaStream_t s);
cudaError_t launch_import(const ChainDesc *desc, double *dpool, const double *src, int chain0,
                          int nchains, size_t maxn, cudaStream_t s);
cudaError_t launch_export(const ChainDesc *desc, const double *dpool, double *dst, int chain0,
                          int nchains, size_t maxn, cudaStream_t s);
cudaError_t launch_mirror(const ChainDesc *desc, double *dpool, int chain0, int nchains, int maxNM,
                          cudaStream_t s);
cudaError_t launch_measure(const ChainDesc *desc, ChainVar *var, double *dpool, int *ipool,
                           unsigned long long *upool, int chain0, int nchains, cudaStream_t s);
cudaError_t launch_adjoint(const AdjArgs &a, int nbeads, cudaStream_t s);
cudaError_t upload_exp_table();
// static adjoint scratch: kNoAllocDoubles doubles, enough for a chain of
// kNoAllocBeads beads (N*M) and kNoAllocParticles particles
constexpr int kNoAllocBeads = 65536;
constexpr int kNoAllocParticles = 8192;
constexpr size_t kNoAllocDoubles = 6 * (size_t)kNoAllocBeads +
                                   8 * (size_t)((kNoAllocBeads + 255) / 256) + 16 +
                                   (size_t)kNoAllocParticles;
// its device address on the current device (looked up on the first call)
cudaError_t adjoint_static_scratch(double **ptr);
// the contact-interaction propagator table T[n][n] for (range, g0, tau)
cudaError_t launch_contact_table(double *dtab, int n, double range, double g0, double tau,
                                 cudaStream_t s);
// measured FP64 FMA throughput of the current device (TFLOP/s)
cudaError_t fp64_peak(int num_sms, cudaStream_t st, double *tflops);
// shared scratch of the device move routines (bytes; doubles for a window)
size_t swap_scratch_bytes(int N, int nwarps);
size_t com_scratch_bytes(int N, int M, int nwarps);
int window_scratch_doubles();

}  // namespace pimc
