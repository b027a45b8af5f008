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

// the adjoint of every chain of a batch (pimc_batch_adjoint): beads in
// blocks of 256, chain after chain
struct AdjBatchArgs {
  const ChainDesc *desc;
  double *dpool;
  int *ipool;
  const double *omega;        // [nchains] trap frequency (d/domega)
  const int *blk_chain;       // [nblocks] chain of each block
  const int *blk_first;       // [nchains] first block of each chain
  const long long *bead_off;  // [nchains] first bead of each chain in gA / gB
  const int *inv_off;         // [nchains] offset of each chain's inverse permutation
  double *gA, *gB;            // [total beads][2]
  int *inv;                   // [sum of N]
  double *part;               // [nblocks][9]
  double *dSdr;               // host layout of every chain (desc.host_off), or null
  double *totals;             // [nchains][9]: S_ext, dV0, domega, S_pair, dg, pair
                              // virial, r.g_ext, 0, r.dS/dr
  int nblocks, nchains;
  // the slice kernel (one CTA per chain slice, 32 maxN bytes of shared
  // memory): used when use_slices != 0
  int use_slices, nslices;
  const int *slice_first;     // [nchains] first slice CTA of each chain
  double *part_s;             // [nslices][8]
};

// mode 0: one CTA per chain (k_sweep); mode 1: one warp per chain (k_sweep_warp)
cudaError_t launch_sweep(const SweepArgs &a, int mode, int grid, int block, size_t smem,
                         cudaStream_t s);
cudaError_t sweep_set_smem(int mode, size_t smem);
// the sweep as three launches per sweep (phase 0 staging, 1 swaps, 2 the
// rest), one CTA per chain, or for the swaps (warp = 1) one warp per chain;
// spec = 1 selects the swap kernel compiled for the reference's rules alone
// (every chain of the launch without physical rules, hard core or contact
// table); a.sweeps must be 1
// regs (swap phase in CTA mode): 0 the 128-register kernel, 170 or 255 the
// kernels compiled for CTAs of at most 64 threads with that many registers
cudaError_t launch_sweep_phase(const SweepArgs &a, int phase, int warp, int spec, int regs,
                               int grid, int block, size_t smem, cudaStream_t s);
cudaError_t sweep_phase_set_smem(int phase, int warp, int spec, int regs, size_t smem);
cudaError_t sweep_phase_occupancy(int phase, int warp, int spec, int regs, int block, size_t smem,
                                  int *blocks_per_sm);
size_t sweep_ctl_bytes();
cudaError_t sweep_occupancy(int mode, int block, size_t smem, int *blocks_per_sm);
cudaError_t launch_attempt(const AttemptArgs &a, size_t smem, cudaStream_t s);
cudaError_t launch_eval_action(const EvalArgs &a, cudaStream_t s);
cudaError_t launch_eval_weights(const EvalArgs &a, cudaStream_t s);
cudaError_t launch_init_world(const ChainDesc *desc, double *dpool, int *ipool, int chain0,
                              int nchains, int maxN, cudaStream_t s);
// the hard-core redraw of init_world for the chains with a hard core (one
// warp per chain; others return at once); failures set ChainVar::err
cudaError_t launch_init_world_hard(const ChainDesc *desc, ChainVar *var, double *dpool, int *ipool,
                                   int chain0, int nchains, cudaStream_t s);
cudaError_t launch_links(const ChainDesc *desc, double *dpool, int *ipool, int chain0, int nchains,
                         int maxNM, cudaStream_t s);
cudaError_t launch_import(const ChainDesc *desc, double *dpool, const double *src, int chain0,
                          int nchains, size_t maxn, cudaStream_t s);
cudaError_t launch_export(const ChainDesc *desc, const double *dpool, double *dst, int chain0,
                          int nchains, size_t maxn, cudaStream_t s);
cudaError_t launch_mirror(const ChainDesc *desc, double *dpool, int chain0, int nchains, int maxNM,
                          cudaStream_t s);
// the positions of chains [c_lo, c_hi) between the host layout (at
// desc.host_off of `host`, which may be pinned host memory the GPU reaches
// directly) and the device layout, in 32 x 32 tiles; tile_off[nchains + 1]
// on the device, ntiles the range's tile count
cudaError_t launch_transpose_tiles(bool import, const ChainDesc *desc, double *dpool,
                                   double *host, const int *tile_off, int c_lo, int c_hi,
                                   int ntiles, int grid, cudaStream_t s);
cudaError_t launch_measure(const ChainDesc *desc, ChainVar *var, double *dpool, int *ipool,
                           unsigned long long *upool, int chain0, int nchains, cudaStream_t s);
cudaError_t launch_adjoint(const AdjArgs &a, int nbeads, cudaStream_t s);
// four launches over every chain (inverse permutations, beads, gradients,
// per-chain totals)
cudaError_t launch_adjoint_batch(const AdjBatchArgs &a, int maxN, cudaStream_t s);
cudaError_t upload_exp_table();
// PIMC_CHECK builds: the device check word (code << 32 | chain of the first
// failed bounds check, 0 if none), cleared by the read; always 0 otherwise
cudaError_t check_word_take(cudaStream_t s, unsigned long long *w);
// PIMC_PROFILE builds: the swap's section cycles [0..15] and outcome counts
// [16..31]; cudaErrorNotSupported otherwise
cudaError_t profile_take(unsigned long long *out, bool reset, cudaStream_t s);
// static adjoint scratch: kNoAllocDoubles doubles, enough for a chain of
// kNoAllocBeads beads (N*M) and kNoAllocParticles particles
constexpr int kNoAllocBeads = 65536;
constexpr int kNoAllocParticles = 8192;
constexpr size_t kNoAllocDoubles = 6 * (size_t)kNoAllocBeads +
                                   8 * (size_t)((kNoAllocBeads + 255) / 256) + 16 +
                                   (size_t)kNoAllocParticles;
// set-up: look up the array's address on the current device (every handle
// creation calls it with its device current)
cudaError_t adjoint_static_setup();
// its address on the current device, as the last set-up on it found it
cudaError_t adjoint_static_scratch(double **ptr);
// the contact-interaction propagator table T[n][n] for (range, g0, tau)
cudaError_t launch_contact_table(double *dtab, int n, double range, double g0, double tau,
                                 cudaStream_t s);
// measured FP64 FMA throughput of the current device (TFLOP/s)
cudaError_t fp64_peak(int num_sms, cudaStream_t st, double *tflops);
// the swap-phase kernels' translation unit (pimc_swap.cu): its kernel for a
// launch shape and its launcher
const void *swap_kernel(int warp, int spec, int regs);
cudaError_t launch_swap(const SweepArgs &a, int warp, int spec, int regs, int grid, int block,
                        size_t smem, cudaStream_t s);
// accessors of each kernel unit's device globals (swap_, fused_, attempt_)
#define PIMC_UNIT_DECL(unit)                                                              \
  cudaError_t unit##_upload_exp_table(const double *tab, size_t bytes);                   \
  cudaError_t unit##_profile_take(unsigned long long *out, bool reset, cudaStream_t s);  \
  cudaError_t unit##_check_word_take(cudaStream_t s, unsigned long long *w);
PIMC_UNIT_DECL(swap)
PIMC_UNIT_DECL(fused)
PIMC_UNIT_DECL(attempt)
#undef PIMC_UNIT_DECL
// shared scratch of the device move routines (bytes; doubles for a window)
size_t swap_scratch_bytes(int N, int nwarps);
size_t com_scratch_bytes(int N, int M, int nwarps);
int window_scratch_doubles();

}  // namespace pimc
