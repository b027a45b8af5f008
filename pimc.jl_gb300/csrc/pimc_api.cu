// pimc_api.cu -- extern "C" boundary of the engine (include/pimc.h).
//
// Host side of the System / run! / Density / Energy API: parameter checks,
// device pools, state I/O, the plain and batched sweep drivers (work queue,
// LPT chain order, CUDA graph of a sweep block, launch-shape tuner),
// injected-draw attempts, estimators, adjoint and checkpoints.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pimc.h"
#include "pimc_internal.h"
#include "pimc_launch.h"
#include "pimc_types.h"

using namespace pimc;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(PIMC_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

constexpr unsigned kStateMagic = 0x50494D43u;   // "PIMC"
constexpr int kStateBudget = 100 * 1024;        // shared bytes for a staged chain

// one launch shape of the sweep kernel and its shared-memory layout
struct Plan {
  int mode = 0;                // 0: one CTA per chain, 1: one warp per chain
  int block = 256;
  int spl = 1;                 // sweeps per launch
  int state_cap = kStateBudget;
  int state_bytes = 0;         // shared bytes for a staged chain (CTA mode)
  int warp_scratch_d = window_scratch_doubles();
  int warp_bytes = 0;          // scratch bytes of one warp's chain (warp mode)
  size_t dyn_smem = 0;
  int split = 0;               // CTA mode: 1 = staging, swaps, rest as three launches
  int pblock[3] = {0, 0, 0};   // split: CTA size per phase (0: block)
  size_t psmem[3] = {0, 0, 0}; // split: dynamic shared bytes per phase
  int pwarp[3] = {0, 0, 0};    // split: 1 = that phase with one warp per chain
  int pwarp_bytes[3] = {0, 0, 0};  // ... and the scratch bytes of each warp
  int pregs[3] = {0, 0, 0};    // split, swap phase: register variant (0, 170, 255)
};

// CTA size and dynamic shared bytes of phase ph of a plan
int phase_block(const Plan &p, int ph) { return p.pblock[ph] > 0 ? p.pblock[ph] : p.block; }
size_t phase_smem(const Plan &p, int ph) {
  return (p.pblock[ph] > 0 || p.pwarp[ph]) ? p.psmem[ph] : p.dyn_smem;
}

struct Handle {
  int nchains = 0;
  std::vector<pimc_params> params;
  std::vector<ChainDesc> desc;
  std::vector<MixDev> mix;
  std::vector<pimc_move_mix> umix;
  ChainDesc *d_desc = nullptr;
  ChainVar *d_var = nullptr;
  MixDev *d_mix = nullptr;
  double *d_dpool = nullptr;
  size_t n_dpool = 0;
  int *d_ipool = nullptr;
  size_t n_ipool = 0;
  unsigned long long *d_upool = nullptr;
  size_t n_upool = 0;
  int *d_queue = nullptr;
  int *d_order = nullptr;
  int *d_iout = nullptr;
  double *d_buf = nullptr;
  size_t n_buf = 0;
  double *d_adj = nullptr;
  size_t n_adj = 0;
  double *d_stage = nullptr;   // host-layout positions of every chain (transposes)
  size_t n_stage = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  long long last_launches = 0;
  int maxN = 0, maxM = 0, maxNM = 0;
  Plan bat;                    // batched launch shape (tuned or set)
  Plan one;                    // plain per-chain launches: one CTA each
  int num_sms = 0;
  int device = 0;              // the device current at creation
  int max_dyn_smem = 0;         // opt-in shared bytes per CTA, less static use
  cudaGraphExec_t gexec = nullptr;
  long long graph_launches = 0;  // kernel launches in one replay of gexec
  int force_warp = 0;
  // contact-propagator tables on the device, shared by the chains whose
  // (g0, tau, range, n) agree; tables given by the caller are never shared
  struct ContactTab {
    double g0, tau, range;
    int n;
    bool given;
    double *d;
  };
  std::vector<ContactTab> ctabs;
  unsigned long long *d_rdf = nullptr;  // pair-distance histograms of every chain
  size_t n_rdf = 0;
  // the batched adjoint's pool and block maps, made on its first call (the
  // chains' shapes are fixed for the handle's lifetime)
  double *d_badj = nullptr;
  AdjBatchArgs badj{};
  bool badj_ready = false;
  // the batch's 32 x 32 (particle, slice) tiles: first tile of each chain
  int *d_tile_off = nullptr;
  int ntiles = 0;
  std::vector<int> tile_off;  // the same on the host
  // pimc_batch_run_io: copy streams, per-chunk events and the chunks' chain
  // ranges, made on first use for a chunk count
  cudaStream_t s_up = nullptr, s_down = nullptr;
  std::vector<cudaEvent_t> io_ev;
  std::vector<int> io_cut;     // chunk k holds chains [io_cut[k], io_cut[k + 1])
};

// the LPT cost of a chain (staging and CoM ~ N M, swaps ~ N^2)
double chain_cost(const pimc_params &p) {
  return (double)p.N * p.M * (p.interactions ? 4.0 : 1.0) + 0.5 * (double)p.N * p.N;
}

int check_params(const pimc_params &p) {
  if (p.dim < 1 || p.dim > 2) return fail(PIMC_EARG, "dim must be 1 or 2");
  if (p.N < 1 || p.N > 8192) return fail(PIMC_EARG, "N must be in [1, 8192]");
  if (p.M < 4 || p.M > 4096) return fail(PIMC_EARG, "M must be in [4, 4096]");
  if (!(p.L > 0.0)) return fail(PIMC_EARG, "L must be positive");
  if (!(p.T > 0.0)) return fail(PIMC_EARG, "T must be positive");
  if (!(p.lambda > 0.0)) return fail(PIMC_EARG, "lambda must be positive");
  if (p.lattice_V0 != 0.0 && !(p.lattice_a > 0.0)) return fail(PIMC_EARG, "lattice_a must be positive");
  if (p.interactions && !(p.pair_sigma > 0.0)) return fail(PIMC_EARG, "pair_sigma must be positive");
  if (p.interactions && !(p.r_a > 0.0))
    return fail(PIMC_EARG, "interactions need r_a > 0 (the neighbour range is not searched for)");
  if (p.semantics != PIMC_SEM_REFERENCE && p.semantics != PIMC_SEM_PHYSICAL)
    return fail(PIMC_EARG, "semantics must be PIMC_SEM_REFERENCE or PIMC_SEM_PHYSICAL");
  if (p.density_nbins < 0 || p.energy_capacity < 0) return fail(PIMC_EARG, "negative capacity");
  if (p.hardcore_a < 0.0) return fail(PIMC_EARG, "hardcore_a must be >= 0");
  return PIMC_OK;
}

// System constructor's derived constants (src/system.jl:129-167)
ChainDesc make_desc(const pimc_params &p, int chain) {
  ChainDesc d;
  memset(&d, 0, sizeof(d));
  d.N = p.N;
  d.M = p.M;
  d.dim = p.dim;
  d.ldn = p.N;
  d.L = p.L;
  d.beta = 1.0 / p.T;
  d.tau = d.beta / p.M;
  d.lambda = p.lambda;
  d.mu = p.mu;
  d.hcoef = 0.5 * p.harmonic_omega * p.harmonic_omega;
  d.V0 = p.lattice_V0;
  d.lat_k = p.lattice_V0 != 0.0 ? 1.0 / p.lattice_a : 0.0;
  d.g = p.pair_g;
  d.inv2s2 = p.interactions ? 1.0 / (2.0 * p.pair_sigma * p.pair_sigma) : 0.0;
  const double ra = p.r_a > 0.0 ? p.r_a : p.L / 4.0;
  d.nbins = (int)std::floor((2.0 * p.L) / ra);
  if (d.nbins < 1) d.nbins = 1;
  d.rc = 2.0 * p.L / d.nbins;
  d.ncell = p.dim == 2 ? d.nbins * d.nbins : d.nbins;
  d.L2 = 2.0 * d.L;
  d.inv2L = 1.0 / (2.0 * d.L);
  d.rc2 = d.rc * d.rc;
  d.mhtau_g = -0.5 * d.tau * d.g;
  // 16-bit fixed-point mirror of the positions on the periodic box: a pair
  // within R of each other has mirror coordinates within R/u + 1 (u the unit)
  // per axis; the bound adds 4 units so that a shifted mirror centre (one
  // more rounding) is covered as well
  {
    const double u = 2.0 * p.L / 65536.0;
    d.q_scale = 65536.0 / (2.0 * p.L);
    d.q_unit2 = (float)(u * u);
    auto lim = [&](double R) {
      const double v = std::ceil((R / u + 4.0) * (R / u + 4.0));
      return v >= 4294967295.0 ? 0xffffffffu : (unsigned)v;  // squares stay <= 2^31
    };
    d.q_lim_rc = lim(d.rc);
    d.q_lim_hard = lim(p.hardcore_a);
    // a mirror distance differs from the exact one by at most 3 units: two
    // roundings per axis (each within 0.516 units, the words being formed in
    // FP32), plus one more for a shifted centre (cycle moves)
    const double rq = d.rc / u, e = 3.0;
    d.q_u2i = (float)(u * u * d.inv2s2);
    d.q_lim_lo = rq > e ? (unsigned)std::floor((rq - e) * (rq - e)) : 0u;
    d.q_lim_hi = (unsigned)std::min(std::ceil((rq + e) * (rq + e)), (double)d.q_lim_rc);
    d.hb_unit = (float)((double)d.q_unit2 / (4.0 * d.tau * d.lambda));
    d.q_Lf = (float)p.L;
    d.q_scalef = (float)d.q_scale;
  }
  d.hard_a = p.hardcore_a;
  d.ctr = p.retry_cap > 0 ? p.retry_cap : 10000;
  d.flags = 0;
  if (p.interactions) d.flags |= PF_PAIR;
  if (p.semantics == PIMC_SEM_PHYSICAL) d.flags |= PF_PHYS;
  if (p.hardcore_a > 0.0) d.flags |= PF_HARD;
  if (p.lattice_V0 != 0.0) d.flags |= PF_LATT;
  if (p.harmonic_omega != 0.0) d.flags |= PF_HARM;
  d.dens_nb = p.density_nbins;
  d.dens_bw = p.density_nbins > 0 ? (2.0 * p.L) / p.density_nbins : 0.0;
  d.eser_cap = p.energy_capacity;
  d.wtab = std::min(p.M - 1, 32) + 1;
  d.key0 = (unsigned)(p.seed & 0xffffffffu);
  d.key1 = (unsigned)(p.seed >> 32);
  d.chain_tag = (unsigned)chain;
  const size_t nm = (size_t)p.N * p.M;
  const size_t sb = 8 * (size_t)(p.dim + 1) * nm + 4 * nm + 4 * (size_t)p.N;
  d.smem_bytes = sb > (size_t)(1 << 30) ? (1 << 30) : (int)((sb + 15) & ~(size_t)15);
  return d;
}

// cells per axis of a chain's cell lists: each cell at least as wide as the
// largest mirror prefilter radius (pair range, hard core), no more than about
// four cells per particle; 0 (no lists) below 5 per axis, where the block of
// cells around a centre covers most of the box
int cell_count(const ChainDesc &d) {
  if (!(d.flags & (PF_PAIR | PF_HARD))) return 0;
  unsigned lim = 0;
  if (d.flags & PF_PAIR) lim = std::max(lim, d.q_lim_rc);
  if (d.flags & PF_HARD) lim = std::max(lim, d.q_lim_hard);
  unsigned long long r = (unsigned long long)std::ceil(std::sqrt((double)lim));
  while (r * r < lim) ++r;
  if (r < 1) r = 1;
  long long nc = 65536 / (long long)r;
  const long long most = d.dim == 2 ? (long long)std::floor(std::sqrt(4.0 * d.N)) : 4LL * d.N;
  nc = std::min(nc, std::max(most, 5LL));
  return nc >= 5 ? (int)nc : 0;
}

pimc_move_mix default_mix(const pimc_params &p) {
  pimc_move_mix m;
  memset(&m, 0, sizeof(m));
  m.staging_phases = 1;
  m.stage_slices = std::min(16, p.M - 2);
  m.stage_min = 2;
  m.stage_max = p.M - 2;
  m.stage_minacc = 0.6;
  m.stage_maxacc = 0.8;
  m.swaps_per_sweep = p.N > 1 ? p.N : 0;
  m.swap_slices = std::min(16, p.M - 2);
  m.swap_min = 2;
  m.swap_max = p.M - 2;
  m.swap_minacc = 0.6;
  m.swap_maxacc = 0.8;
  m.com_phases = 1;
  m.com_step = 1.0;
  m.com_minstep = 1e-1;
  m.com_maxstep = p.L / 2;
  m.com_minacc = 0.4;
  m.com_maxacc = 0.6;
  m.polymer_com_phases = 0;
  m.pcom_step = 1.0;
  m.pcom_minstep = 1e-1;
  m.pcom_maxstep = p.L / 2;
  m.pcom_minacc = 0.4;
  m.pcom_maxacc = 0.6;
  m.adapt = 1;
  m.measure_every = 0;
  return m;
}

int check_mix(const pimc_move_mix &m, const pimc_params &p) {
  if (m.staging_phases < 0 || m.swaps_per_sweep < 0 || m.com_phases < 0 || m.polymer_com_phases < 0)
    return fail(PIMC_EARG, "negative move counts");
  if (m.stage_slices < 2 || m.stage_min < 2 || m.stage_max < m.stage_min || m.stage_max > p.M - 1)
    return fail(PIMC_EARG, "staging slices must satisfy 2 <= min <= max <= M-1");
  if (m.swap_slices < 2 || m.swap_min < 2 || m.swap_max < m.swap_min || m.swap_max > p.M - 1)
    return fail(PIMC_EARG, "swap slices must satisfy 2 <= min <= max <= M-1");
  if (m.stage_max > 64 || m.swap_max > 64)
    return fail(PIMC_EARG, "windows longer than 64 slices are not supported on the device");
  if (m.measure_every < 0) return fail(PIMC_EARG, "measure_every must be >= 0");
  return PIMC_OK;
}

MixDev to_dev(const pimc_move_mix &m) {
  MixDev d;
  memset(&d, 0, sizeof(d));
  d.staging_phases = m.staging_phases;
  d.stage_min = m.stage_min;
  d.stage_max = m.stage_max;
  d.stage_minacc = m.stage_minacc;
  d.stage_maxacc = m.stage_maxacc;
  d.swaps_per_sweep = m.swaps_per_sweep;
  d.swap_min = m.swap_min;
  d.swap_max = m.swap_max;
  d.swap_minacc = m.swap_minacc;
  d.swap_maxacc = m.swap_maxacc;
  d.com_phases = m.com_phases;
  d.com_minstep = m.com_minstep;
  d.com_maxstep = m.com_maxstep;
  d.com_minacc = m.com_minacc;
  d.com_maxacc = m.com_maxacc;
  d.polymer_com_phases = m.polymer_com_phases;
  d.pcom_minstep = m.pcom_minstep;
  d.pcom_maxstep = m.pcom_maxstep;
  d.pcom_minacc = m.pcom_minacc;
  d.pcom_maxacc = m.pcom_maxacc;
  d.adapt = m.adapt;
  d.measure_every = m.measure_every;
  return d;
}

Handle *H(void *h) { return reinterpret_cast<Handle *>(h); }

int ensure_buf(Handle *h, size_t n) {
  if (n <= h->n_buf) return PIMC_OK;
  if (h->d_buf) cudaFree(h->d_buf);
  h->d_buf = nullptr;
  h->n_buf = 0;
  CK(cudaMalloc(&h->d_buf, n * sizeof(double)));
  h->n_buf = n;
  return PIMC_OK;
}

int sync_check(Handle *h) {
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaGetLastError());
  return PIMC_OK;
}

// shared-memory layout of a launch shape.  CTA mode: staged chain state (the
// largest chain that fits state_cap) followed by the CTA's scratch.  Warp
// mode: per warp, its chain's control block and the scratch of a one-warp
// group; chain state stays in global memory.
Plan plan_smem(const Handle *h, int mode, int block, int spl, int state_cap) {
  Plan p;
  p.mode = mode;
  p.block = block;
  p.spl = spl;
  p.state_cap = state_cap;
  p.warp_scratch_d = window_scratch_doubles();
  if (mode == 1) {
    size_t w = std::max(swap_scratch_bytes(h->maxN, 1), (size_t)window_scratch_doubles() * sizeof(double));
    w = std::max(w, com_scratch_bytes(h->maxN, h->maxM, 1));
    w = (w + 15) & ~(size_t)15;
    p.state_bytes = 0;
    p.state_cap = 0;
    p.warp_bytes = (int)w;
    p.dyn_smem = (size_t)(block / 32) * (sweep_ctl_bytes() + w);
    return p;
  }
  const int nw = block / 32;
  size_t scratch = std::max(swap_scratch_bytes(h->maxN, nw),
                            (size_t)nw * p.warp_scratch_d * sizeof(double));
  scratch = std::max(scratch, com_scratch_bytes(h->maxN, h->maxM, nw));
  scratch = (scratch + 15) & ~(size_t)15;
  int need_state = 0;
  for (const auto &d : h->desc)
    if (d.smem_bytes <= state_cap) need_state = std::max(need_state, d.smem_bytes);
  need_state = (need_state + 15) & ~15;
  p.state_bytes = need_state;
  p.dyn_smem = (size_t)need_state + scratch;
  return p;
}

// the chain descriptors to the device; the captured sweep graph is dropped,
// since which kernels it launches depends on the chains' flags
int upload_desc(Handle *h) {
  CK(cudaMemcpyAsync(h->d_desc, h->desc.data(), sizeof(ChainDesc) * h->nchains,
                     cudaMemcpyHostToDevice, h->stream));
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  return PIMC_OK;
}

// cached links V and the 16-bit position mirror from the positions
int refresh_links(Handle *h, int chain0, int nch) {
  CK(launch_links(h->d_desc, h->d_dpool, h->d_ipool, chain0, nch, h->maxNM, h->stream));
  return PIMC_OK;
}

// init_world on the device for every chain: the uniform start and Levy loop
// of each particle, the hard-core redraw for the chains that have one, then
// the cached links.  A chain whose hard spheres cannot be placed fails the
// call (the reference logs an error and returns an empty world,
// src/system.jl:47-49).
int init_world_impl(Handle *h) {
  const int nc = h->nchains;
  CK(launch_init_world(h->d_desc, h->d_dpool, h->d_ipool, 0, nc, h->maxN, h->stream));
  bool any_hard = false;
  for (const auto &d : h->desc) any_hard = any_hard || (d.flags & PF_HARD);
  if (any_hard) {
    CK(launch_init_world_hard(h->d_desc, h->d_var, h->d_dpool, h->d_ipool, 0, nc, h->stream));
    std::vector<ChainVar> v(nc);
    CK(cudaMemcpyAsync(v.data(), h->d_var, sizeof(ChainVar) * nc, cudaMemcpyDeviceToHost, h->stream));
    int rc = sync_check(h);
    if (rc) return rc;
    for (int c = 0; c < nc; ++c)
      if (v[c].err == DERR_INIT) {
        const ChainDesc &d = h->desc[c];
        char vol[64];
        snprintf(vol, sizeof vol, "%g", std::pow(2.0 * d.L, d.dim));
        // the failed chain's flag is cleared so that a retry starts clean
        v[c].err = 0;
        cudaMemcpyAsync(h->d_var, v.data(), sizeof(ChainVar) * nc, cudaMemcpyHostToDevice, h->stream);
        cudaStreamSynchronize(h->stream);
        return fail(PIMC_ESTATE, "chain " + std::to_string(c) + ": creating world of " +
                                     std::to_string(d.N) + " particles with hardspheres of length " +
                                     std::to_string(d.hard_a) + " in the volume " + vol + " failed");
      }
  }
  if (refresh_links(h, 0, nc)) return PIMC_ECUDA;
  return PIMC_OK;
}

int create_impl(const pimc_params *params, int nchains, void **out) {
  if (!params || !out || nchains < 1) return fail(PIMC_EARG, "null argument or nchains < 1");
  if (nchains > (1 << 24)) return fail(PIMC_EARG, "too many chains");
  for (int c = 0; c < nchains; ++c) {
    int rc = check_params(params[c]);
    if (rc) return fail(rc, "chain " + std::to_string(c) + ": " + g_err);
    if (params[c].interactions) {
      const double ra = params[c].r_a;
      const int nb = (int)std::floor((2.0 * params[c].L) / ra);
      if (nb < 3) return fail(PIMC_EARG, "interactions need at least 3 neighbour cells per dimension");
    }
  }
  Handle *h = new Handle();
  h->nchains = nchains;
  h->params.assign(params, params + nchains);
  size_t dp = 0, ip = 0, up = 0;
  for (int c = 0; c < nchains; ++c) {
    const pimc_params &p = params[c];
    ChainDesc d = make_desc(p, c);
    const size_t NM = (size_t)p.N * p.M;
    d.x_off = (long long)dp; dp += (size_t)p.dim * NM;
    d.V_off = (long long)dp; dp += NM;
    d.xq_off = (long long)dp; dp += (NM + 1) / 2;
    dp = (dp + 1) & ~(size_t)1;
    d.host_off = (long long)h->n_stage;
    h->n_stage += (size_t)p.dim * NM;
    d.tab_off = (long long)dp; dp += 4 * (size_t)d.wtab * d.wtab;  // (alpha, sigma), then (w, k)
    d.eser_off = p.energy_capacity > 0 ? (long long)dp : -1;
    dp += (size_t)NOBS * p.energy_capacity;
    d.next_off = (long long)ip; ip += p.N;
    d.cl_nc = cell_count(d);
    d.cl_cap = std::min(p.N, std::max(32, p.N / 4));
    d.cl_mode = 1;
    d.cl_frac = 0.5f;
    if (d.cl_nc > 0) {
      const CellLayout cl = cell_layout(p.N, p.M, p.dim == 2 ? d.cl_nc * d.cl_nc : d.cl_nc, d.cl_cap);
      d.cl_off = (long long)ip;
      ip += (size_t)cl.total;
    } else {
      d.cl_off = -1;
    }
    if (p.density_nbins > 0) {
      d.dens_off = (long long)up;
      up += p.dim == 2 ? (size_t)p.density_nbins * p.density_nbins : (size_t)p.density_nbins;
    } else {
      d.dens_off = -1;
    }
    h->desc.push_back(d);
    pimc_move_mix m = default_mix(p);
    h->umix.push_back(m);
    h->mix.push_back(to_dev(m));
    h->maxN = std::max(h->maxN, p.N);
    h->maxM = std::max(h->maxM, p.M);
    h->maxNM = std::max(h->maxNM, (int)NM);
  }
  h->n_dpool = dp;
  h->n_ipool = std::max<size_t>(ip, 1);
  h->n_upool = std::max<size_t>(up, 1);
  auto cleanup = [&](int rc) {
    pimc_destroy(h);
    return rc;
  };
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cleanup(fail(PIMC_ECUDA, "no CUDA device"));
  h->device = dev;
  cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&h->max_dyn_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  h->max_dyn_smem -= 4096;  // the CTA kernel's static control block and reduction buffer
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
    return cleanup(fail(PIMC_ECUDA, "stream/event creation failed"));
  if (cudaMalloc(&h->d_desc, sizeof(ChainDesc) * nchains) != cudaSuccess ||
      cudaMalloc(&h->d_var, sizeof(ChainVar) * nchains) != cudaSuccess ||
      cudaMalloc(&h->d_mix, sizeof(MixDev) * nchains) != cudaSuccess ||
      cudaMalloc(&h->d_dpool, sizeof(double) * h->n_dpool) != cudaSuccess ||
      cudaMalloc(&h->d_ipool, sizeof(int) * h->n_ipool) != cudaSuccess ||
      cudaMalloc(&h->d_upool, sizeof(unsigned long long) * h->n_upool) != cudaSuccess ||
      cudaMalloc(&h->d_queue, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&h->d_order, sizeof(int) * nchains) != cudaSuccess ||
      cudaMalloc(&h->d_iout, sizeof(int) * 16) != cudaSuccess ||
      cudaMalloc(&h->d_stage, sizeof(double) * std::max<size_t>(h->n_stage, 1)) != cudaSuccess)
    return cleanup(fail(PIMC_ENOMEM, "device allocation failed"));
  cudaMemsetAsync(h->d_dpool, 0, sizeof(double) * h->n_dpool, h->stream);
  cudaMemsetAsync(h->d_upool, 0, sizeof(unsigned long long) * h->n_upool, h->stream);
  // bridge coefficient tables: alpha = (m-t)/(m+1-t), sigma = sqrt(2 lambda
  // alpha tau); then the sweeps' closed form of the same bridge, (w, k) =
  // (sigma / (m-t), m-t) at t >= 1 and (1/m, m) at t = 0
  std::vector<double> tab;
  for (int c = 0; c < nchains; ++c) {
    const ChainDesc &d = h->desc[c];
    const size_t ww = (size_t)d.wtab * d.wtab;
    tab.assign(4 * ww, 0.0);
    for (int m = 2; m < d.wtab; ++m) {
      tab[2 * (ww + (size_t)m * d.wtab)] = 1.0 / m;
      tab[2 * (ww + (size_t)m * d.wtab) + 1] = (double)m;
      for (int t = 1; t < m; ++t) {
        const double a = (double)(m - t) / (double)(m + 1 - t);
        const double sig = std::sqrt(2.0 * d.lambda * a * d.tau);
        tab[2 * ((size_t)m * d.wtab + t)] = a;
        tab[2 * ((size_t)m * d.wtab + t) + 1] = sig;
        tab[2 * (ww + (size_t)m * d.wtab + t)] = sig / (m - t);
        tab[2 * (ww + (size_t)m * d.wtab + t) + 1] = (double)(m - t);
      }
    }
    cudaMemcpyAsync(h->d_dpool + d.tab_off, tab.data(), sizeof(double) * tab.size(),
                    cudaMemcpyHostToDevice, h->stream);
  }
  std::vector<ChainVar> vars(nchains);
  for (int c = 0; c < nchains; ++c) {
    memset(&vars[c], 0, sizeof(ChainVar));
    vars[c].stage_m = std::min(h->umix[c].stage_slices, h->umix[c].stage_max);
    vars[c].swap_m = std::min(h->umix[c].swap_slices, h->umix[c].swap_max);
    vars[c].com_step = h->umix[c].com_step;
    vars[c].pcom_step = h->umix[c].pcom_step;
  }
  cudaMemcpyAsync(h->d_var, vars.data(), sizeof(ChainVar) * nchains, cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(h->d_mix, h->mix.data(), sizeof(MixDev) * nchains, cudaMemcpyHostToDevice, h->stream);
  // LPT order: most expensive chains first (staging/CoM ~ N M, swaps ~ N^2)
  std::vector<int> order(nchains);
  for (int c = 0; c < nchains; ++c) order[c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return chain_cost(h->params[a]) > chain_cost(h->params[b]);
  });
  cudaMemcpyAsync(h->d_order, order.data(), sizeof(int) * nchains, cudaMemcpyHostToDevice, h->stream);
  if (upload_desc(h)) return cleanup(PIMC_ECUDA);
  if (upload_exp_table() != cudaSuccess) return cleanup(fail(PIMC_ECUDA, "exp table upload failed"));
  // the address of pimc_adjoint_noalloc's static scratch on this device
  if (adjoint_static_setup() != cudaSuccess)
    return cleanup(fail(PIMC_ECUDA, "static adjoint scratch lookup failed"));
  // System(): init_world, cached links, neighbour grid
  {
    const int rc = init_world_impl(h);
    if (rc) return cleanup(rc);
  }
  h->bat = plan_smem(h, 0, 256, 1, kStateBudget);
  h->one = h->bat;
  if (sync_check(h)) return cleanup(PIMC_ECUDA);
  *out = h;
  return PIMC_OK;
}

int check_chain(Handle *h, int chain) {
  if (!h) return fail(PIMC_EARG, "null handle");
  if (chain < 0 || chain >= h->nchains) return fail(PIMC_EARG, "chain index out of range");
  return PIMC_OK;
}

int set_beads_impl(Handle *h, int chain, const double *x) {
  if (check_chain(h, chain)) return PIMC_EARG;
  if (!x) return fail(PIMC_EARG, "null positions");
  const ChainDesc &d = h->desc[chain];
  for (size_t i = 0; i < (size_t)d.dim * d.N * d.M; ++i)
    if (!std::isfinite(x[i])) return fail(PIMC_EARG, "non-finite position");
  const size_t n = (size_t)d.dim * d.N * d.M;
  CK(cudaMemcpyAsync(h->d_stage + d.host_off, x, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  CK(launch_import(h->d_desc, h->d_dpool, h->d_stage, chain, 1, n, h->stream));
  if (refresh_links(h, chain, 1)) return PIMC_ECUDA;
  return sync_check(h);
}

int get_beads_impl(Handle *h, int chain, double *x) {
  if (check_chain(h, chain)) return PIMC_EARG;
  if (!x) return fail(PIMC_EARG, "null output");
  const ChainDesc &d = h->desc[chain];
  const size_t n = (size_t)d.dim * d.N * d.M;
  CK(launch_export(h->d_desc, h->d_dpool, h->d_stage, chain, 1, n, h->stream));
  CK(cudaMemcpyAsync(x, h->d_stage + d.host_off, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
  return sync_check(h);
}

int check_perm(const int *next, int N) {
  std::vector<char> seen(N, 0);
  for (int i = 0; i < N; ++i) {
    if (next[i] < 0 || next[i] >= N || seen[next[i]]) return fail(PIMC_ESTATE, "next is not a permutation");
    seen[next[i]] = 1;
  }
  return PIMC_OK;
}

int read_var(Handle *h, int chain, ChainVar *v) {
  CK(cudaMemcpyAsync(v, h->d_var + chain, sizeof(ChainVar), cudaMemcpyDeviceToHost, h->stream));
  return sync_check(h);
}

void fill_stats(const ChainVar &v, pimc_stats *o) {
  for (int q = 0; q < 4; ++q) {
    o->attempts[q] = v.att[q];
    o->accepts[q] = v.acc[q];
  }
  o->skips = v.skips;
  o->bead_updates = v.bead_updates;
  o->sweeps = v.sweep;
  o->measurements = v.n_meas;
  o->stage_slices = v.stage_m;
  o->swap_slices = v.swap_m;
  o->com_step = v.com_step;
  o->pcom_step = v.pcom_step;
  for (int q = 0; q < 4; ++q) o->bead_updates_kind[q] = v.beads_kind[q];
}

SweepArgs sweep_args(Handle *h, const Plan &p) {
  SweepArgs a;
  a.desc = h->d_desc;
  a.var = h->d_var;
  a.mix = h->d_mix;
  a.dpool = h->d_dpool;
  a.ipool = h->d_ipool;
  a.upool = h->d_upool;
  a.nchains = h->nchains;
  a.chain0 = 0;
  a.order = nullptr;
  a.queue = nullptr;
  a.sweeps = 1;
  a.state_bytes = p.state_bytes;
  a.warp_scratch_d = p.warp_scratch_d;
  a.warp_bytes = p.warp_bytes;
  a.teams = 0;
  return a;
}

// plain path: one launch of one CTA per chain per sweep, no queue, no graph
int run_plain(Handle *h, long long n) {
  const Plan &p = h->one;
  CK(sweep_set_smem(p.mode, p.dyn_smem));
  SweepArgs a = sweep_args(h, p);
  a.nchains = 1;
  a.teams = 1;  // a lone chain is latency-bound: idle warps join its slots
  CK(cudaEventRecord(h->ev0, h->stream));
  long long launches = 0;
  for (long long s = 0; s < n; ++s)
    for (int c = 0; c < h->nchains; ++c) {
      a.chain0 = c;
      CK(launch_sweep(a, p.mode, 1, p.block, p.dyn_smem, h->stream));
      ++launches;
    }
  CK(cudaEventRecord(h->ev1, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  h->last_launches = launches;
  return PIMC_OK;
}

// persistent grid: every resident CTA (CTA mode) or resident warp (warp mode)
// pulls chains from the work queue
// 1 when every chain follows the reference's rules without a hard core or
// a contact table: the swap phase then runs the kernel compiled for those
// rules alone (the CUDA graph is rebuilt whenever a chain's flags change)
int swap_spec(const Handle *h) {
  for (const auto &d : h->desc)
    if (d.flags & (PF_PHYS | PF_HARD | PF_CONTACT)) return 0;
  return 1;
}

// resident CTAs (or warps) for a launch of the plan's kernel; phase >= 0
// names a phase kernel of a split plan
int grid_for(Handle *h, const Plan &p, int phase = -1, int nch = -1) {
  int per_sm = 0;
  const cudaError_t e = phase >= 0
                            ? sweep_phase_occupancy(phase, p.pwarp[phase], swap_spec(h), p.pregs[phase],
                                                    phase_block(p, phase), phase_smem(p, phase), &per_sm)
                            : sweep_occupancy(p.mode, p.block, p.dyn_smem, &per_sm);
  if (e != cudaSuccess || per_sm < 1) per_sm = 1;
  const bool warp = phase >= 0 ? p.pwarp[phase] != 0 : p.mode == 1;
  const int units_per_cta = warp ? phase_block(p, phase >= 0 ? phase : 0) / 32 : 1;
  const int chains = nch >= 0 ? nch : h->nchains;
  const int need = (chains + units_per_cta - 1) / units_per_cta;
  return std::max(1, std::min(need, per_sm * h->num_sms));
}

// teams of warps pay off only when every chain of the launch is resident at
// once (the launch is latency-bound); with more chains than resident CTAs
// the idle warps' issue slots are used by other chains anyway
bool launch_teams(Handle *h, const Plan &p) {
  int per_sm = 0;
  if (p.mode != 0) return false;
  const cudaError_t e = p.split ? sweep_phase_occupancy(0, 0, 0, 0, phase_block(p, 0), phase_smem(p, 0), &per_sm)
                                : sweep_occupancy(p.mode, p.block, p.dyn_smem, &per_sm);
  if (e != cudaSuccess) return false;
  return h->nchains <= per_sm * h->num_sms;
}

// the dynamic shared-memory attribute of every kernel the plan launches
cudaError_t plan_set_smem(const Handle *h, const Plan &p) {
  if (!p.split) return sweep_set_smem(p.mode, p.dyn_smem);
  for (int ph = 0; ph < 3; ++ph) {
    const cudaError_t e = sweep_phase_set_smem(ph, p.pwarp[ph], swap_spec(h), p.pregs[ph], phase_smem(p, ph));
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// n sweeps of every chain as launches on the stream: one launch of n sweeps,
// or for a split plan n rounds of (staging, swaps, rest), each from a reset
// work queue
// a.queue: the work-queue counter of the launches (a.order names a.nchains
// chains)
cudaError_t issue_sweeps(Handle *h, const Plan &p, SweepArgs a, int n, long long *launches) {
  if (!p.split) {
    a.sweeps = n;
    cudaError_t e = cudaMemsetAsync(a.queue, 0, sizeof(int), h->stream);
    if (e == cudaSuccess)
      e = launch_sweep(a, p.mode, grid_for(h, p, -1, a.nchains), p.block, p.dyn_smem, h->stream);
    if (launches) *launches += 1;
    return e;
  }
  a.sweeps = 1;
  for (int s = 0; s < n; ++s)
    for (int ph = 0; ph < 3; ++ph) {
      SweepArgs b = a;
      if (p.pwarp[ph]) b.warp_bytes = p.pwarp_bytes[ph];
      cudaError_t e = cudaMemsetAsync(a.queue, 0, sizeof(int), h->stream);
      if (e == cudaSuccess)
        e = launch_sweep_phase(b, ph, p.pwarp[ph], swap_spec(h), p.pregs[ph], grid_for(h, p, ph, a.nchains),
                               phase_block(p, ph), phase_smem(p, ph), h->stream);
      if (e != cudaSuccess) return e;
      if (launches) *launches += 1;
    }
  return cudaSuccess;
}

int build_graph(Handle *h) {
  if (h->gexec) return PIMC_OK;
  const Plan &p = h->bat;
  SweepArgs a = sweep_args(h, p);
  a.order = h->d_order;
  a.queue = h->d_queue;
  a.teams = launch_teams(h, p);
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  long long nl = 0;
  issue_sweeps(h, p, a, p.spl, &nl);
  h->graph_launches = nl;
  CK(cudaStreamEndCapture(h->stream, &g));
  cudaError_t e = cudaGraphInstantiate(&h->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(PIMC_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return PIMC_OK;
}

// n sweeps of every chain on the handle stream: replays of the captured
// graph, the remainder issued directly; adds the kernel launches to *launches
int issue_batched(Handle *h, long long n, long long *launches) {
  const Plan &p = h->bat;
  CK(plan_set_smem(h, p));
  const int spl = std::max(1, p.spl);
  int rc = build_graph(h);
  if (rc) return rc;
  const long long full = n / spl, rem = n % spl;
  for (long long i = 0; i < full; ++i) {
    CK(cudaGraphLaunch(h->gexec, h->stream));
    *launches += h->graph_launches;
  }
  if (rem) {
    SweepArgs a = sweep_args(h, p);
    a.order = h->d_order;
    a.queue = h->d_queue;
    a.teams = launch_teams(h, p);
    CK(issue_sweeps(h, p, a, (int)rem, launches));
  }
  return PIMC_OK;
}

int run_batched(Handle *h, long long n) {
  CK(cudaEventRecord(h->ev0, h->stream));
  long long launches = 0;
  int rc = issue_batched(h, n, &launches);
  if (rc) return rc;
  CK(cudaEventRecord(h->ev1, h->stream));
  rc = sync_check(h);
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  h->last_launches = launches;
  return PIMC_OK;
}

int check_device_errors(Handle *h) {
  unsigned long long w = 0;
  CK(check_word_take(h->stream, &w));
  if (w)
    return fail(PIMC_EDEVICE, "device bounds check failed: code " + std::to_string((int)(w >> 32)) +
                                  " on chain " + std::to_string((int)(w & 0xFFFFFFu)) +
                                  " (1 window, 3 scratch, 4 neighbour queue, 5 particle index)");
  std::vector<ChainVar> v(h->nchains);
  CK(cudaMemcpyAsync(v.data(), h->d_var, sizeof(ChainVar) * h->nchains, cudaMemcpyDeviceToHost, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  for (int c = 0; c < h->nchains; ++c)
    if (v[c].err)
      return fail(PIMC_EDEVICE, "device error " + std::to_string(v[c].err) +
                                    (v[c].err == DERR_STATE ? " (next is not a permutation)" : "") +
                                    " on chain " + std::to_string(c) +
                                    "; the chain is skipped until its state is replaced");
  return PIMC_OK;
}

// ---------------------------------------------------------------- attempts

int attempt_impl(Handle *h, int kind, int n, int j0, int m, double u_pick, double step,
                 const double *normals, int n_normals, const double *uniforms, int n_uniforms,
                 int *result, int *extra, double *proposal) {
  if (!h) return fail(PIMC_EARG, "null handle");
  const ChainDesc &d = h->desc[0];
  if (n < 0 || n >= d.N) return fail(PIMC_EARG, "particle index out of range");
  if (kind == MV_STAGE || kind == MV_SWAP) {
    if (j0 < 0 || j0 >= d.M) return fail(PIMC_EARG, "slice index out of range");
    if (m < 2 || m > d.M - 1 || m > 64) return fail(PIMC_EARG, "window m must be in [2, min(M-1, 64)]");
  }
  if (n_normals < 0 || n_uniforms < 0 || (n_normals && !normals) || (n_uniforms && !uniforms))
    return fail(PIMC_EARG, "bad draw arrays");
  if (!(d.flags & PF_HARD)) {
    const int need = kind == MV_STAGE ? (m - 1) * d.dim : (kind == MV_SWAP ? 2 * (m - 1) * d.dim : 0);
    if (n_normals < need) return fail(PIMC_EDRAWS, "not enough injected normals");
  }
  if (kind == MV_SWAP && d.N <= 1) {
    if (result) *result = PIMC_SKIP;
    return PIMC_OK;
  }
  if (kind == MV_COM) {
    int nx = -1;
    CK(cudaMemcpyAsync(&nx, h->d_ipool + d.next_off + n, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (sync_check(h)) return PIMC_ECUDA;
    if (nx != n) return fail(PIMC_EARG, "SingleCenterOfMass needs a particle with next == itself");
  }
  // snapshot of the chain so that a run-out of injected draws leaves no trace
  // x, V and the mirror are contiguous in the pool
  const size_t nsnap = (size_t)(d.tab_off - d.x_off);
  std::vector<double> sx(nsnap);
  std::vector<int> sn(d.N);
  CK(cudaMemcpyAsync(sx.data(), h->d_dpool + d.x_off, nsnap * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(sn.data(), h->d_ipool + d.next_off, d.N * 4, cudaMemcpyDeviceToHost, h->stream));
  const size_t nprop = (size_t)2 * (m + 1) * d.dim + 8;
  if (ensure_buf(h, (size_t)n_normals + n_uniforms + nprop + 8)) return PIMC_ENOMEM;
  double *dn = h->d_buf, *du = dn + n_normals, *dprop = du + n_uniforms;
  if (n_normals) CK(cudaMemcpyAsync(dn, normals, 8 * (size_t)n_normals, cudaMemcpyHostToDevice, h->stream));
  if (n_uniforms) CK(cudaMemcpyAsync(du, uniforms, 8 * (size_t)n_uniforms, cudaMemcpyHostToDevice, h->stream));
  AttemptArgs a;
  a.desc = h->d_desc;
  a.var = h->d_var;
  a.dpool = h->d_dpool;
  a.ipool = h->d_ipool;
  a.upool = h->d_upool;
  a.chain = 0;
  a.kind = kind;
  a.n = n;
  a.j0 = j0;
  a.m = m;
  a.u_pick = u_pick;
  a.step = step;
  a.normals = dn;
  a.n_normals = n_normals;
  a.uniforms = du;
  a.n_uniforms = n_uniforms;
  a.prop = proposal ? dprop : nullptr;
  a.out = h->d_iout;
  a.force_warp = h->force_warp;
  size_t smem = std::max(swap_scratch_bytes(d.N, 1), (size_t)window_scratch_doubles() * 8);
  smem = std::max(smem, com_scratch_bytes(d.N, d.M, 4));
  CK(launch_attempt(a, smem, h->stream));
  int out[5] = {0, 0, 0, 0, 0};
  CK(cudaMemcpyAsync(out, h->d_iout, sizeof(out), cudaMemcpyDeviceToHost, h->stream));
  if (proposal) {
    const size_t np = (kind == MV_SWAP ? 2 : 1) * (size_t)(m + 1) * d.dim;
    CK(cudaMemcpyAsync(proposal, dprop, np * 8, cudaMemcpyDeviceToHost, h->stream));
  }
  int rc = sync_check(h);
  if (rc) return rc;
  unsigned long long w = 0;
  CK(check_word_take(h->stream, &w));
  if (w)
    return fail(PIMC_EDEVICE, "device bounds check failed: code " + std::to_string((int)(w >> 32)) +
                                  " in an injected-draw attempt");
  if (out[4]) {
    CK(cudaMemcpyAsync(h->d_dpool + d.x_off, sx.data(), nsnap * 8, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_ipool + d.next_off, sn.data(), d.N * 4, cudaMemcpyHostToDevice, h->stream));
    sync_check(h);
    return fail(PIMC_EDRAWS, "injected draws ran out; state restored");
  }
  if (out[0] < 0) return fail(PIMC_ESTATE, "invalid cycle structure");
  if (result) *result = out[0];
  if (extra) *extra = out[1];
  return PIMC_OK;
}

}  // namespace

int pimc_fail(int code, const std::string &msg) { return fail(code, msg); }

// ===================================================================== C ABI
// pimc_batch_run_io's chunks: contiguous chain ranges of about equal bytes
// in the host layout, and an upload and a transposed-back event per chunk
int io_prepare(Handle *h, int chunks) {
  if ((int)h->io_cut.size() == chunks + 1) return PIMC_OK;
  std::vector<int> cut(chunks + 1, 0);
  cut[chunks] = h->nchains;
  const double total = (double)h->n_stage;
  for (int k = 1; k < chunks; ++k) {
    const double target = total * k / chunks;
    int c = cut[k - 1] + 1;
    while (c < h->nchains - (chunks - k) && (double)h->desc[c].host_off < target) ++c;
    cut[k] = c;
  }
  if (!h->s_up) {
    CK(cudaStreamCreateWithFlags(&h->s_up, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&h->s_down, cudaStreamNonBlocking));
  }
  for (cudaEvent_t e : h->io_ev) cudaEventDestroy(e);
  h->io_ev.assign(2 * chunks + 2, nullptr);  // per chunk upload and done; start; end
  for (auto &e : h->io_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  h->io_cut = cut;
  return PIMC_OK;
}

extern "C" {

const char *pimc_last_error(void) { return g_err.c_str(); }

int pimc_abi_version(void) { return PIMC_ABI_VERSION; }

int pimc_create(const pimc_params *p, void **handle) { return create_impl(p, 1, handle); }

int pimc_batch_create(const pimc_params *params, int nchains, void **handle) {
  return create_impl(params, nchains, handle);
}

int pimc_destroy(void *handle) {
  Handle *h = H(handle);
  if (!h) return PIMC_OK;
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->d_desc);
  cudaFree(h->d_var);
  cudaFree(h->d_mix);
  cudaFree(h->d_dpool);
  cudaFree(h->d_ipool);
  cudaFree(h->d_upool);
  cudaFree(h->d_queue);
  cudaFree(h->d_order);
  cudaFree(h->d_iout);
  cudaFree(h->d_buf);
  cudaFree(h->d_adj);
  cudaFree(h->d_stage);
  for (cudaEvent_t e : h->io_ev) cudaEventDestroy(e);
  if (h->s_up) cudaStreamDestroy(h->s_up);
  if (h->s_down) cudaStreamDestroy(h->s_down);
  for (auto &t : h->ctabs) cudaFree(t.d);
  cudaFree(h->d_rdf);
  cudaFree(h->d_badj);
  cudaFree(h->d_tile_off);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return PIMC_OK;
}

int pimc_get_params(void *handle, int chain, pimc_params *out) {
  Handle *h = H(handle);
  if (check_chain(h, chain) || !out) return fail(PIMC_EARG, "bad argument");
  *out = h->params[chain];
  return PIMC_OK;
}

int pimc_num_chains(void *handle, int *n) {
  if (!handle || !n) return fail(PIMC_EARG, "null argument");
  *n = H(handle)->nchains;
  return PIMC_OK;
}

int pimc_set_beads(void *handle, const double *x) { return set_beads_impl(H(handle), 0, x); }
int pimc_get_beads(void *handle, double *x) { return get_beads_impl(H(handle), 0, x); }
int pimc_batch_set_beads(void *handle, int chain, const double *x) {
  return set_beads_impl(H(handle), chain, x);
}
int pimc_batch_get_beads(void *handle, int chain, double *x) {
  return get_beads_impl(H(handle), chain, x);
}

// the tile list of the batch (once per handle)
static int ensure_tiles(Handle *h) {
  if (h->d_tile_off) return PIMC_OK;
  std::vector<int> off(h->nchains + 1, 0);
  long long t = 0;
  for (int c = 0; c < h->nchains; ++c) {
    off[c] = (int)t;
    t += (long long)((h->desc[c].N + 31) / 32) * ((h->desc[c].M + 31) / 32);
    if (t > 0x7fffffffLL) return fail(PIMC_EARG, "batch too large for the transpose tiles");
  }
  off[h->nchains] = (int)t;
  int *d = nullptr;
  CK(cudaMalloc(&d, sizeof(int) * off.size()));
  cudaError_t e = cudaMemcpyAsync(d, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    cudaFree(d);
    return fail(PIMC_ECUDA, std::string("tile list: ") + cudaGetErrorString(e));
  }
  h->d_tile_off = d;
  h->ntiles = (int)t;
  h->tile_off = off;
  return PIMC_OK;
}

// the device address of a host buffer that the GPU can read and write in
// place (page-locked memory: cudaHostAlloc, cudaHostRegister, a pinned torch
// tensor), or null for pageable memory
static double *device_view(const void *host) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return static_cast<double *>(a.devicePointer);
}

// the whole batch (host layout, chain order) in one pass: from a pinned host
// buffer the tiled transpose reads the caller's memory directly; a pageable
// buffer goes through one copy into the staging buffer first.  Then one link
// refresh launch for all chains.
int pimc_batch_set_beads_all(void *handle, const double *x_all) {
  Handle *h = H(handle);
  if (!h || !x_all) return fail(PIMC_EARG, "null argument");
  int rc = ensure_tiles(h);
  if (rc) return rc;
  double *src = device_view(x_all);
  if (!src) {
    CK(cudaMemcpyAsync(h->d_stage, x_all, h->n_stage * 8, cudaMemcpyHostToDevice, h->stream));
    src = h->d_stage;
  }
  CK(launch_transpose_tiles(true, h->d_desc, h->d_dpool, src, h->d_tile_off, 0, h->nchains,
                            h->ntiles, 8 * h->num_sms, h->stream));
  if (refresh_links(h, 0, h->nchains)) return PIMC_ECUDA;
  return sync_check(h);
}

int pimc_batch_get_beads_all(void *handle, double *x_all) {
  Handle *h = H(handle);
  if (!h || !x_all) return fail(PIMC_EARG, "null argument");
  int rc = ensure_tiles(h);
  if (rc) return rc;
  double *dst = device_view(x_all);
  CK(launch_transpose_tiles(false, h->d_desc, h->d_dpool, dst ? dst : h->d_stage, h->d_tile_off, 0,
                            h->nchains, h->ntiles, 8 * h->num_sms, h->stream));
  if (!dst)
    CK(cudaMemcpyAsync(x_all, h->d_stage, h->n_stage * 8, cudaMemcpyDeviceToHost, h->stream));
  return sync_check(h);
}

// upload, sweep and download the batch with the copies in chunks of chains:
// chunk k's positions go host -> staging buffer on the upload stream while
// the compute stream transposes chunk k - 1 into the device layout and
// refreshes its links; once every chunk is in, all chains sweep n times
// together (the batched launch shape and its graph, so that the sweep keeps
// the whole batch's load balance); then the compute stream transposes the
// chunks back one by one and the download stream copies each to x_out as
// soon as it is out.  With page-locked buffers the copies are DMA transfers
// that run beside the transposes.  x_in and x_out may be the same buffer.
int pimc_batch_run_io(void *handle, const double *x_in, double *x_out, long long n_sweeps, int chunks) {
  Handle *h = H(handle);
  if (!h || !x_in || !x_out || n_sweeps < 0) return fail(PIMC_EARG, "bad argument");
  if (chunks <= 0) chunks = 4;
  chunks = std::max(1, std::min(chunks, h->nchains));
  int rc = ensure_tiles(h);
  if (rc) return rc;
  long long launches = 0;
  double *vin = device_view(x_in), *vout = device_view(x_out);
  if (vin && vout) {
    // page-locked buffers: the tiled transposes read and write them in place
    // over the host link, which beats staging copies plus device transposes
    CK(cudaEventRecord(h->ev0, h->stream));
    CK(launch_transpose_tiles(true, h->d_desc, h->d_dpool, vin, h->d_tile_off, 0, h->nchains,
                              h->ntiles, 8 * h->num_sms, h->stream));
    CK(launch_links(h->d_desc, h->d_dpool, h->d_ipool, 0, h->nchains, h->maxNM, h->stream));
    launches += 2;
    if (n_sweeps > 0 && (rc = issue_batched(h, n_sweeps, &launches))) return rc;
    CK(launch_transpose_tiles(false, h->d_desc, h->d_dpool, vout, h->d_tile_off, 0, h->nchains,
                              h->ntiles, 8 * h->num_sms, h->stream));
    launches += 1;
    CK(cudaEventRecord(h->ev1, h->stream));
    rc = sync_check(h);
    if (rc) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->last_ms = ms;
    h->last_launches = launches;
    return check_device_errors(h);
  }
  if ((rc = io_prepare(h, chunks))) return rc;
  CK(cudaEventRecord(h->ev0, h->stream));
  cudaEvent_t start = h->io_ev[2 * chunks];
  CK(cudaEventRecord(start, h->stream));
  CK(cudaStreamWaitEvent(h->s_up, start, 0));
  auto span = [&](int k, size_t *off, size_t *n) {
    const int c0 = h->io_cut[k], c1 = h->io_cut[k + 1];
    *off = (size_t)h->desc[c0].host_off;
    *n = (c1 < h->nchains ? (size_t)h->desc[c1].host_off : h->n_stage) - *off;
  };
  for (int k = 0; k < chunks; ++k) {
    size_t off, n;
    span(k, &off, &n);
    CK(cudaMemcpyAsync(h->d_stage + off, x_in + off, n * sizeof(double), cudaMemcpyHostToDevice,
                       h->s_up));
    CK(cudaEventRecord(h->io_ev[2 * k], h->s_up));
  }
  for (int k = 0; k < chunks; ++k) {
    const int c0 = h->io_cut[k], c1 = h->io_cut[k + 1];
    const int nt = h->tile_off[c1] - h->tile_off[c0];
    CK(cudaStreamWaitEvent(h->stream, h->io_ev[2 * k], 0));
    CK(launch_transpose_tiles(true, h->d_desc, h->d_dpool, h->d_stage, h->d_tile_off, c0, c1, nt,
                              8 * h->num_sms, h->stream));
    CK(launch_links(h->d_desc, h->d_dpool, h->d_ipool, c0, c1 - c0, h->maxNM, h->stream));
    launches += 2;
  }
  if (n_sweeps > 0 && (rc = issue_batched(h, n_sweeps, &launches))) return rc;
  for (int k = 0; k < chunks; ++k) {
    const int c0 = h->io_cut[k], c1 = h->io_cut[k + 1];
    const int nt = h->tile_off[c1] - h->tile_off[c0];
    CK(launch_transpose_tiles(false, h->d_desc, h->d_dpool, h->d_stage, h->d_tile_off, c0, c1, nt,
                              8 * h->num_sms, h->stream));
    launches += 1;
    CK(cudaEventRecord(h->io_ev[2 * k + 1], h->stream));
    size_t off, n;
    span(k, &off, &n);
    CK(cudaStreamWaitEvent(h->s_down, h->io_ev[2 * k + 1], 0));
    CK(cudaMemcpyAsync(x_out + off, h->d_stage + off, n * sizeof(double), cudaMemcpyDeviceToHost,
                       h->s_down));
  }
  CK(cudaEventRecord(h->io_ev[2 * chunks + 1], h->s_down));
  CK(cudaStreamWaitEvent(h->stream, h->io_ev[2 * chunks + 1], 0));
  CK(cudaEventRecord(h->ev1, h->stream));
  rc = sync_check(h);
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  h->last_launches = launches;
  return check_device_errors(h);
}

int pimc_batch_energy_sums_all(void *handle, double *sum, double *sumsq, unsigned long long *count) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  std::vector<ChainVar> v(h->nchains);
  CK(cudaMemcpyAsync(v.data(), h->d_var, sizeof(ChainVar) * h->nchains, cudaMemcpyDeviceToHost, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  for (int c = 0; c < h->nchains; ++c) {
    for (int q = 0; q < 4; ++q) {
      if (sum) sum[4 * c + q] = v[c].esum[q];
      if (sumsq) sumsq[4 * c + q] = v[c].esum2[q];
    }
    if (count) count[c] = v[c].n_meas;
  }
  return PIMC_OK;
}

int pimc_set_next(void *handle, const int *next) {
  Handle *h = H(handle);
  if (!h || !next) return fail(PIMC_EARG, "null argument");
  const ChainDesc &d = h->desc[0];
  if (check_perm(next, d.N)) return PIMC_ESTATE;
  CK(cudaMemcpyAsync(h->d_ipool + d.next_off, next, sizeof(int) * d.N, cudaMemcpyHostToDevice, h->stream));
  if (refresh_links(h, 0, 1)) return PIMC_ECUDA;
  return sync_check(h);
}

int pimc_batch_get_next(void *handle, int chain, int *next) {
  Handle *h = H(handle);
  if (check_chain(h, chain) || !next) return fail(PIMC_EARG, "bad argument");
  const ChainDesc &d = h->desc[chain];
  CK(cudaMemcpyAsync(next, h->d_ipool + d.next_off, sizeof(int) * d.N, cudaMemcpyDeviceToHost, h->stream));
  return sync_check(h);
}
int pimc_get_next(void *handle, int *next) { return pimc_batch_get_next(handle, 0, next); }

int pimc_set_raw(void *handle, const double *x, const double *V, const int *next) {
  Handle *h = H(handle);
  if (!h || !x || !V || !next) return fail(PIMC_EARG, "null argument");
  const ChainDesc &d = h->desc[0];
  if (check_perm(next, d.N)) return PIMC_ESTATE;
  const size_t n = (size_t)d.dim * d.N * d.M;
  std::vector<double> vt((size_t)d.N * d.M);
  for (int i = 0; i < d.N; ++i)
    for (int j = 0; j < d.M; ++j) vt[(size_t)j * d.N + i] = V[(size_t)i * d.M + j];
  CK(cudaMemcpyAsync(h->d_stage + d.host_off, x, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  CK(launch_import(h->d_desc, h->d_dpool, h->d_stage, 0, 1, n, h->stream));
  CK(cudaMemcpyAsync(h->d_dpool + d.V_off, vt.data(), sizeof(double) * vt.size(), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->d_ipool + d.next_off, next, sizeof(int) * d.N, cudaMemcpyHostToDevice, h->stream));
  CK(launch_mirror(h->d_desc, h->d_dpool, 0, 1, h->maxNM, h->stream));
  return sync_check(h);
}

int pimc_get_links(void *handle, double *V) {
  Handle *h = H(handle);
  if (!h || !V) return fail(PIMC_EARG, "null argument");
  const ChainDesc &d = h->desc[0];
  std::vector<double> vt((size_t)d.N * d.M);
  CK(cudaMemcpyAsync(vt.data(), h->d_dpool + d.V_off, sizeof(double) * vt.size(), cudaMemcpyDeviceToHost, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  for (int i = 0; i < d.N; ++i)
    for (int j = 0; j < d.M; ++j) V[(size_t)i * d.M + j] = vt[(size_t)j * d.N + i];
  return PIMC_OK;
}

int pimc_init_world(void *handle) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  int rc = init_world_impl(h);
  if (rc) return rc;
  return sync_check(h);
}

int pimc_set_move_mix(void *handle, int chain, const pimc_move_mix *mix) {
  Handle *h = H(handle);
  if (!h || !mix) return fail(PIMC_EARG, "null argument");
  if (chain >= h->nchains) return fail(PIMC_EARG, "chain index out of range");
  const int c0 = chain < 0 ? 0 : chain, c1 = chain < 0 ? h->nchains : chain + 1;
  for (int c = c0; c < c1; ++c)
    if (check_mix(*mix, h->params[c])) return PIMC_EARG;
  std::vector<ChainVar> v(h->nchains);
  CK(cudaMemcpyAsync(v.data(), h->d_var, sizeof(ChainVar) * h->nchains, cudaMemcpyDeviceToHost, h->stream));
  if (sync_check(h)) return PIMC_ECUDA;
  for (int c = c0; c < c1; ++c) {
    h->umix[c] = *mix;
    h->mix[c] = to_dev(*mix);
    v[c].stage_m = std::min(mix->stage_slices, mix->stage_max);
    v[c].swap_m = std::min(mix->swap_slices, mix->swap_max);
    v[c].com_step = mix->com_step;
    v[c].pcom_step = mix->pcom_step;
  }
  CK(cudaMemcpyAsync(h->d_var, v.data(), sizeof(ChainVar) * h->nchains, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->d_mix, h->mix.data(), sizeof(MixDev) * h->nchains, cudaMemcpyHostToDevice, h->stream));
  return sync_check(h);
}

int pimc_run(void *handle, long long n_sweeps) {
  Handle *h = H(handle);
  if (!h || n_sweeps < 0) return fail(PIMC_EARG, "bad argument");
  int rc = h->nchains == 1 ? run_plain(h, n_sweeps) : run_batched(h, n_sweeps);
  if (rc) return rc;
  return check_device_errors(h);
}

int pimc_batch_run(void *handle, long long n_sweeps) {
  Handle *h = H(handle);
  if (!h || n_sweeps < 0) return fail(PIMC_EARG, "bad argument");
  int rc = run_batched(h, n_sweeps);
  if (rc) return rc;
  return check_device_errors(h);
}

int pimc_batch_run_plain(void *handle, long long n_sweeps) {
  Handle *h = H(handle);
  if (!h || n_sweeps < 0) return fail(PIMC_EARG, "bad argument");
  int rc = run_plain(h, n_sweeps);
  if (rc) return rc;
  return check_device_errors(h);
}

int check_launch(const Handle *h, const pimc_launch &l, Plan *out) {
  if (l.warp_per_chain != 0 && l.warp_per_chain != 1)
    return fail(PIMC_EARG, "warp_per_chain must be 0 or 1");
  const int bmax = l.warp_per_chain ? 256 : 512;
  if (l.block < 32 * (1 + !l.warp_per_chain) || l.block > bmax || l.block % 32)
    return fail(PIMC_EARG, l.warp_per_chain ? "block must be a multiple of 32 in [32, 256]"
                                            : "block must be a multiple of 32 in [64, 512]");
  if (l.sweeps_per_launch < 1) return fail(PIMC_EARG, "sweeps_per_launch must be >= 1");
  if (l.cell_lists < 0 || l.cell_lists > 3)
    return fail(PIMC_EARG, "cell_lists must be 0 (keep), 1 (off), 2 (auto) or 3 (always)");
  if (l.state_smem_bytes < 0 || l.state_smem_bytes > 160 * 1024)
    return fail(PIMC_EARG, "state_smem_bytes must be in [0, 160 KiB]");
  if (l.split_phases < 0 || l.split_phases > 1 || (l.split_phases && l.warp_per_chain))
    return fail(PIMC_EARG, "split_phases must be 0, or 1 with one CTA per chain");
  Plan p = plan_smem(h, l.warp_per_chain, l.block, l.sweeps_per_launch, l.state_smem_bytes);
  p.split = l.split_phases;
  for (int ph = 0; ph < 3; ++ph) {
    const int b = l.phase_block[ph];
    const int w = l.phase_warp[ph];
    const int rg = l.phase_regs[ph] == 128 ? 0 : l.phase_regs[ph];
    if (w != 0 && w != 1) return fail(PIMC_EARG, "phase_warp must be 0 or 1");
    if (rg != 0 && rg != 170 && rg != 255) return fail(PIMC_EARG, "phase_regs must be 0, 128, 170 or 255");
    if (rg && (!l.split_phases || ph != 1 || w || (b > 0 ? b : l.block) > 64))
      return fail(PIMC_EARG,
                  "phase_regs: 170 and 255 are offered for the swap phase of a split sweep in CTAs of 64 threads");
    p.pregs[ph] = rg;
    if (w && (!l.split_phases || ph != 1))
      return fail(PIMC_EARG, "phase_warp: one warp per chain is offered for the swap phase of a split sweep");
    if (w) {
      const int bw = b > 0 ? b : l.block;
      if (bw < 32 || bw > 256 || bw % 32)
        return fail(PIMC_EARG, "a warp-per-chain phase needs a CTA of 32 to 256 threads, a multiple of 32");
      const Plan q = plan_smem(h, 1, bw, 1, 0);
      if (h->max_dyn_smem > 0 && q.dyn_smem > (size_t)h->max_dyn_smem)
        return fail(PIMC_EARG, "phase launch needs more shared memory than the device offers");
      p.pblock[ph] = bw;
      p.psmem[ph] = q.dyn_smem;
      p.pwarp[ph] = 1;
      p.pwarp_bytes[ph] = q.warp_bytes;
      continue;
    }
    if (b == 0) continue;
    if (!l.split_phases || b < 64 || b > 512 || b % 32)
      return fail(PIMC_EARG, "phase_block needs split_phases and a multiple of 32 in [64, 512]");
    const Plan q = plan_smem(h, 0, b, 1, l.state_smem_bytes);
    if (h->max_dyn_smem > 0 && q.dyn_smem > (size_t)h->max_dyn_smem)
      return fail(PIMC_EARG, "phase launch needs more shared memory than the device offers");
    p.pblock[ph] = b;
    p.psmem[ph] = q.dyn_smem;
  }
  if (h->max_dyn_smem > 0 && p.dyn_smem > (size_t)h->max_dyn_smem)
    return fail(PIMC_EARG, "launch shape needs " + std::to_string(p.dyn_smem) +
                               " shared bytes per CTA, more than the device offers");
  *out = p;
  return PIMC_OK;
}

int pimc_batch_phase_times(void *handle, long long n, double ms[3]) {
  Handle *h = H(handle);
  if (!h || !ms || n < 1) return fail(PIMC_EARG, "bad argument");
  const Plan &p = h->bat;
  CK(plan_set_smem(h, p));
  SweepArgs a = sweep_args(h, p);
  a.order = h->d_order;
  a.queue = h->d_queue;
  a.teams = launch_teams(h, p);
  const int nph = p.split ? 3 : 1;
  cudaEvent_t ev[4];
  for (int k = 0; k <= nph; ++k) CK(cudaEventCreate(&ev[k]));
  double acc[3] = {0.0, 0.0, 0.0};
  cudaError_t e = cudaSuccess;
  for (long long s = 0; s < n && e == cudaSuccess; ++s) {
    cudaEventRecord(ev[0], h->stream);
    for (int ph = 0; ph < nph && e == cudaSuccess; ++ph) {
      e = cudaMemsetAsync(h->d_queue, 0, sizeof(int), h->stream);
      if (e != cudaSuccess) break;
      if (p.split) {
        SweepArgs b = a;
        b.sweeps = 1;
        if (p.pwarp[ph]) b.warp_bytes = p.pwarp_bytes[ph];
        e = launch_sweep_phase(b, ph, p.pwarp[ph], swap_spec(h), p.pregs[ph], grid_for(h, p, ph),
                               phase_block(p, ph), phase_smem(p, ph), h->stream);
      } else {
        a.sweeps = 1;
        e = launch_sweep(a, p.mode, grid_for(h, p), p.block, p.dyn_smem, h->stream);
      }
      if (e == cudaSuccess) e = cudaEventRecord(ev[ph + 1], h->stream);
    }
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[nph]);
    for (int ph = 0; ph < nph && e == cudaSuccess; ++ph) {
      float t = 0.f;
      e = cudaEventElapsedTime(&t, ev[ph], ev[ph + 1]);
      acc[ph] += t;
    }
  }
  for (int k = 0; k <= nph; ++k) cudaEventDestroy(ev[k]);
  if (e != cudaSuccess) return fail(PIMC_ECUDA, std::string("phase timing: ") + cudaGetErrorString(e));
  for (int k = 0; k < 3; ++k) ms[k] = acc[k];
  return sync_check(h);
}

int pimc_batch_set_launch(void *handle, const pimc_launch *launch) {
  Handle *h = H(handle);
  if (!h || !launch) return fail(PIMC_EARG, "null argument");
  Plan p;
  int rc = check_launch(h, *launch, &p);
  if (rc) return rc;
  h->bat = p;
  if (h->gexec) {
    cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
  }
  if (launch->cell_lists) return pimc_set_option(h, PIMC_OPT_CELL_LISTS, launch->cell_lists - 1);
  return PIMC_OK;
}

int pimc_batch_get_launch(void *handle, pimc_launch *launch) {
  Handle *h = H(handle);
  if (!h || !launch) return fail(PIMC_EARG, "null argument");
  launch->warp_per_chain = h->bat.mode;
  launch->block = h->bat.block;
  launch->sweeps_per_launch = h->bat.spl;
  launch->state_smem_bytes = h->bat.state_cap;
  launch->split_phases = h->bat.split;
  for (int ph = 0; ph < 3; ++ph) {
    launch->phase_block[ph] = h->bat.pblock[ph];
    launch->phase_warp[ph] = h->bat.pwarp[ph];
    launch->phase_regs[ph] = h->bat.pregs[ph];
  }
  launch->cell_lists = 1 + h->desc[0].cl_mode;
  return PIMC_OK;
}

int pimc_get_state(void *handle, void *buf, size_t bytes);
int pimc_set_state(void *handle, const void *buf, size_t bytes);
int pimc_state_size(void *handle, size_t *bytes);

// project-written tuner: time every launch shape -- one CTA per chain with
// (threads, sweeps per launch, shared-memory staging budget), or one warp per
// chain with (warps per CTA, sweeps per launch) -- on the handle's own chains
// and keep the fastest.  Smaller staging budgets trade shared-memory residency
// of small chains for more resident CTAs per SM; warp mode trades threads per
// chain for chains in flight.
static int tune_impl(Handle *h, int sweeps_per_trial, pimc_launch *chosen);

// The trials run with measurements off: a trial of a sweep or two that
// happened to hold a measurement sweep (several times a plain sweep's cost
// with the pair energy) would lose whatever shape it timed.  The chains' move
// mixes are restored afterwards, as their states are.
int pimc_batch_tune(void *handle, int sweeps_per_trial, pimc_launch *chosen) {
  Handle *h = H(handle);
  if (!h || sweeps_per_trial < 1) return fail(PIMC_EARG, "bad argument");
  const std::vector<MixDev> saved = h->mix;
  for (MixDev &m : h->mix) m.measure_every = 0;
  CK(cudaMemcpyAsync(h->d_mix, h->mix.data(), sizeof(MixDev) * h->nchains, cudaMemcpyHostToDevice,
                     h->stream));
  const int rc = tune_impl(h, sweeps_per_trial, chosen);
  h->mix = saved;
  CK(cudaMemcpyAsync(h->d_mix, h->mix.data(), sizeof(MixDev) * h->nchains, cudaMemcpyHostToDevice,
                     h->stream));
  const int rs = sync_check(h);
  return rc ? rc : rs;
}

static int tune_impl(Handle *h, int sweeps_per_trial, pimc_launch *chosen) {
  // trials advance the chains; the snapshot puts them back afterwards
  size_t nb = 0;
  int rc = pimc_state_size(h, &nb);
  if (rc) return rc;
  std::vector<char> snap(nb);
  if ((rc = pimc_get_state(h, snap.data(), nb))) return rc;
  std::vector<pimc_launch> cand;
  for (int s : {1, 2}) {
    if (s > sweeps_per_trial) continue;
    for (int b : {64, 128, 256})
      for (int m : {0, 32 * 1024, kStateBudget}) cand.push_back({0, b, s, m});
    for (int b : {64, 128, 256}) cand.push_back({1, b, s, 0});
    // the phases as separate launches
    for (int b : {64, 128, 256})
      for (int m : {0, 32 * 1024}) cand.push_back({0, b, s, m, 1});
  }
  pimc_launch keep;
  pimc_batch_get_launch(h, &keep);
  std::vector<std::pair<double, pimc_launch>> timed;
  for (const pimc_launch &l : cand) {
    Plan p;
    if (check_launch(h, l, &p)) continue;  // does not fit this device
    if ((rc = pimc_batch_set_launch(h, &l))) return rc;
    if ((rc = run_batched(h, l.sweeps_per_launch))) return rc;  // warm (graph build)
    if ((rc = run_batched(h, sweeps_per_trial))) return rc;
    timed.push_back({h->last_ms / sweeps_per_trial, l});
  }
  // the chains keep moving during the trials, so early and late candidates
  // see different configurations: the three fastest are timed again, in
  // turn, twice each, and the lowest total wins
  std::stable_sort(timed.begin(), timed.end(),
                   [](const std::pair<double, pimc_launch> &a, const std::pair<double, pimc_launch> &b) {
                     return a.first < b.first;
                   });
  if (!timed.empty()) keep = timed[0].second;
  const size_t nduel = std::min<size_t>(3, timed.size());
  if (nduel > 1) {
    std::vector<double> tot(nduel, 0.0);
    for (int round = 0; round < 2; ++round)
      for (size_t k = 0; k < nduel; ++k) {
        const pimc_launch &l = timed[k].second;
        if ((rc = pimc_batch_set_launch(h, &l))) return rc;
        if ((rc = run_batched(h, l.sweeps_per_launch))) return rc;
        if ((rc = run_batched(h, sweeps_per_trial))) return rc;
        tot[k] += h->last_ms;
      }
    size_t kb = 0;
    for (size_t k = 1; k < nduel; ++k)
      if (tot[k] < tot[kb]) kb = k;
    keep = timed[kb].second;
  }
  // a split shape: time each phase under every CTA size (events between
  // the phases) and give each phase its fastest size, kept if the whole
  // sweep gets faster
  if (keep.split_phases) {
    double pbest[3] = {1e300, 1e300, 1e300};
    pimc_launch ref = keep;
    for (int b : {64, 128, 256}) {
      pimc_launch l = keep;
      l.block = b;
      for (int ph = 0; ph < 3; ++ph) l.phase_block[ph] = l.phase_warp[ph] = l.phase_regs[ph] = 0;
      Plan p;
      if (check_launch(h, l, &p)) continue;
      if ((rc = pimc_batch_set_launch(h, &l))) return rc;
      double ms[3];
      if ((rc = pimc_batch_phase_times(h, 1, ms))) return rc;  // warm
      if ((rc = pimc_batch_phase_times(h, sweeps_per_trial, ms))) return rc;
      for (int ph = 0; ph < 3; ++ph)
        if (ms[ph] < pbest[ph]) {
          pbest[ph] = ms[ph];
          ref.phase_block[ph] = b;
          ref.phase_warp[ph] = 0;
          ref.phase_regs[ph] = 0;
        }
    }
    // the swap phase with one warp per chain, 2 to 8 chains per CTA
    for (int b : {64, 128, 256}) {
      pimc_launch l = keep;
      for (int ph = 0; ph < 3; ++ph) l.phase_block[ph] = l.phase_warp[ph] = l.phase_regs[ph] = 0;
      l.phase_block[1] = b;
      l.phase_warp[1] = 1;
      Plan p;
      if (check_launch(h, l, &p)) continue;
      if ((rc = pimc_batch_set_launch(h, &l))) return rc;
      double ms[3];
      if ((rc = pimc_batch_phase_times(h, 1, ms))) return rc;  // warm
      if ((rc = pimc_batch_phase_times(h, sweeps_per_trial, ms))) return rc;
      if (ms[1] < pbest[1]) {
        pbest[1] = ms[1];
        ref.phase_block[1] = b;
        ref.phase_warp[1] = 1;
        ref.phase_regs[1] = 0;
      }
    }
    // the swap phase in CTAs of 64 threads with the kernels compiled for 170
    // and 255 registers a thread (fewer spills, fewer chains per SM)
    for (int rg : {170, 255}) {
      pimc_launch l = keep;
      for (int ph = 0; ph < 3; ++ph) l.phase_block[ph] = l.phase_warp[ph] = l.phase_regs[ph] = 0;
      l.phase_block[1] = 64;
      l.phase_regs[1] = rg;
      Plan p;
      if (check_launch(h, l, &p)) continue;
      if ((rc = pimc_batch_set_launch(h, &l))) return rc;
      double ms[3];
      if ((rc = pimc_batch_phase_times(h, 1, ms))) return rc;  // warm
      if ((rc = pimc_batch_phase_times(h, sweeps_per_trial, ms))) return rc;
      if (ms[1] < pbest[1]) {
        pbest[1] = ms[1];
        ref.phase_block[1] = 64;
        ref.phase_warp[1] = 0;
        ref.phase_regs[1] = rg;
      }
    }
    Plan p;
    if (!check_launch(h, ref, &p)) {
      if ((rc = pimc_batch_set_launch(h, &ref))) return rc;
      if ((rc = run_batched(h, ref.sweeps_per_launch))) return rc;
      if ((rc = run_batched(h, sweeps_per_trial))) return rc;
      const double t_ref = h->last_ms;
      if ((rc = pimc_batch_set_launch(h, &keep))) return rc;
      if ((rc = run_batched(h, keep.sweeps_per_launch))) return rc;
      if ((rc = run_batched(h, sweeps_per_trial))) return rc;
      if (t_ref < h->last_ms) keep = ref;
    }
  }
  // the cell lists against the row scans on the chosen shape: the same
  // chains either way, timed in turn, twice each
  keep.cell_lists = 1 + h->desc[0].cl_mode;
  bool lists = false;
  for (const ChainDesc &d : h->desc) lists = lists || d.cl_nc > 0;
  if (lists && keep.cell_lists != 1) {
    double tot[2] = {0.0, 0.0};
    pimc_launch lc[2] = {keep, keep};
    lc[1].cell_lists = 1;
    for (int round = 0; round < 2; ++round)
      for (int k = 0; k < 2; ++k) {
        if ((rc = pimc_batch_set_launch(h, &lc[k]))) return rc;
        if ((rc = run_batched(h, lc[k].sweeps_per_launch))) return rc;
        if ((rc = run_batched(h, sweeps_per_trial))) return rc;
        tot[k] += h->last_ms;
      }
    if (tot[1] < tot[0]) keep = lc[1];
  }
  if ((rc = pimc_batch_set_launch(h, &keep))) return rc;
  if ((rc = pimc_set_state(h, snap.data(), nb))) return rc;
  if (chosen) *chosen = keep;
  return PIMC_OK;
}

int pimc_attempt_staging(void *handle, int n, int j0, int m, const double *normals, int n_normals,
                         const double *uniforms, int n_uniforms, int *result, double *proposal) {
  return attempt_impl(H(handle), MV_STAGE, n, j0, m, 0.0, 0.0, normals, n_normals, uniforms,
                      n_uniforms, result, nullptr, proposal);
}

int pimc_attempt_swap(void *handle, int j0, int m, int n1, double u_pick, const double *normals,
                      int n_normals, const double *uniforms, int n_uniforms, int *result, int *n2,
                      double *proposal) {
  return attempt_impl(H(handle), MV_SWAP, n1, j0, m, u_pick, 0.0, normals, n_normals, uniforms,
                      n_uniforms, result, n2, proposal);
}

int pimc_attempt_com(void *handle, int n, double step, const double *uniforms, int n_uniforms,
                     int *result) {
  return attempt_impl(H(handle), MV_COM, n, 0, 2, 0.0, step, nullptr, 0, uniforms, n_uniforms,
                      result, nullptr, nullptr);
}

int pimc_attempt_polymer_com(void *handle, int n, double step, const double *uniforms,
                             int n_uniforms, int *result) {
  return attempt_impl(H(handle), MV_PCOM, n, 0, 2, 0.0, step, nullptr, 0, uniforms, n_uniforms,
                      result, nullptr, nullptr);
}

int pimc_eval_action(void *handle, double out[4]) {
  Handle *h = H(handle);
  if (!h || !out) return fail(PIMC_EARG, "null argument");
  if (ensure_buf(h, 8)) return PIMC_ENOMEM;
  EvalArgs a;
  memset(&a, 0, sizeof(a));
  a.desc = h->d_desc;
  a.dpool = h->d_dpool;
  a.ipool = h->d_ipool;
  a.upool = h->d_upool;
  a.chain = 0;
  a.out = h->d_buf;
  CK(launch_eval_action(a, h->stream));
  CK(cudaMemcpyAsync(out, h->d_buf, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return sync_check(h);
}

int pimc_eval_staging_weights(void *handle, int n, int j0, int m, const double *rp, double *w_init,
                              double *w_upd) {
  Handle *h = H(handle);
  if (!h || !rp || !w_init || !w_upd) return fail(PIMC_EARG, "null argument");
  const ChainDesc &d = h->desc[0];
  if (n < 0 || n >= d.N || j0 < 0 || j0 >= d.M || m < 2 || m > d.M - 1 || m > 64)
    return fail(PIMC_EARG, "window out of range (m must be in [2, min(M-1, 64)])");
  const size_t nrp = (size_t)(m + 1) * d.dim;
  if (ensure_buf(h, nrp + 8)) return PIMC_ENOMEM;
  CK(cudaMemcpyAsync(h->d_buf + 8, rp, nrp * 8, cudaMemcpyHostToDevice, h->stream));
  EvalArgs a;
  memset(&a, 0, sizeof(a));
  a.desc = h->d_desc;
  a.dpool = h->d_dpool;
  a.ipool = h->d_ipool;
  a.upool = h->d_upool;
  a.chain = 0;
  a.n = n;
  a.j0 = j0;
  a.m = m;
  a.rp = h->d_buf + 8;
  a.out = h->d_buf;
  CK(launch_eval_weights(a, h->stream));
  double o[2];
  CK(cudaMemcpyAsync(o, h->d_buf, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  *w_init = o[0];
  *w_upd = o[1];
  return PIMC_OK;
}

int pimc_measure(void *handle) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  CK(launch_measure(h->d_desc, h->d_var, h->d_dpool, h->d_ipool, h->d_upool, 0, h->nchains, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  return check_device_errors(h);
}

int pimc_get_energies(void *handle, int chain, double *out, int cap, int *count) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  ChainVar v;
  int rc = read_var(h, chain, &v);
  if (rc) return rc;
  const ChainDesc &d = h->desc[chain];
  const int have = (int)std::min<unsigned long long>(v.eser_count, (unsigned long long)d.eser_cap);
  const int k = std::min(have, std::max(cap, 0));
  if (k > 0 && out) {
    std::vector<double> rows((size_t)NOBS * k);
    CK(cudaMemcpyAsync(rows.data(), h->d_dpool + d.eser_off, sizeof(double) * NOBS * k,
                       cudaMemcpyDeviceToHost, h->stream));
    rc = sync_check(h);
    if (rc) return rc;
    for (int r = 0; r < k; ++r)
      for (int q = 0; q < 4; ++q) out[4 * r + q] = rows[(size_t)NOBS * r + q];
  }
  if (count) *count = have;
  return PIMC_OK;
}

int pimc_get_observables(void *handle, int chain, double *out, int cap, int *count) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  ChainVar v;
  int rc = read_var(h, chain, &v);
  if (rc) return rc;
  const ChainDesc &d = h->desc[chain];
  const int have = (int)std::min<unsigned long long>(v.eser_count, (unsigned long long)d.eser_cap);
  const int k = std::min(have, std::max(cap, 0));
  if (k > 0 && out) {
    CK(cudaMemcpyAsync(out, h->d_dpool + d.eser_off, sizeof(double) * NOBS * k,
                       cudaMemcpyDeviceToHost, h->stream));
    rc = sync_check(h);
    if (rc) return rc;
  }
  if (count) *count = have;
  return PIMC_OK;
}

int pimc_get_observable_sums(void *handle, int chain, double *sum, double *sumsq,
                             unsigned long long *count) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  ChainVar v;
  int rc = read_var(h, chain, &v);
  if (rc) return rc;
  for (int q = 0; q < NOBS; ++q) {
    if (sum) sum[q] = v.esum[q];
    if (sumsq) sumsq[q] = v.esum2[q];
  }
  if (count) *count = v.n_meas;
  return PIMC_OK;
}

int pimc_set_radial(void *handle, int chain, int nbins, double rmax) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  if (chain < -1 || chain >= h->nchains) return fail(PIMC_EARG, "chain out of range");
  if (nbins < 0 || nbins > (1 << 20)) return fail(PIMC_EARG, "nbins must be in [0, 2^20]");
  if (nbins > 0 && !(rmax >= 0.0 && std::isfinite(rmax)))
    return fail(PIMC_EARG, "rmax must be finite and >= 0 (0: the half-width L)");
  const int c0 = chain < 0 ? 0 : chain, c1 = chain < 0 ? h->nchains : chain + 1;
  CK(cudaStreamSynchronize(h->stream));
  for (int c = c0; c < c1; ++c) {
    ChainDesc &d = h->desc[c];
    d.rdf_nb = nbins;
    d.rdf_dr = nbins > 0 ? (rmax > 0.0 ? rmax : d.L) / nbins : 0.0;
  }
  // one buffer for every chain's histogram, laid out afresh and zeroed
  size_t tot = 0;
  for (const auto &d : h->desc) tot += (size_t)std::max(d.rdf_nb, 0);
  unsigned long long *buf = nullptr;
  if (tot > 0) {
    CK(cudaMalloc(&buf, sizeof(unsigned long long) * tot));
    CK(cudaMemsetAsync(buf, 0, sizeof(unsigned long long) * tot, h->stream));
  }
  size_t off = 0;
  for (auto &d : h->desc) {
    d.rdf = d.rdf_nb > 0 ? buf + off : nullptr;
    off += (size_t)std::max(d.rdf_nb, 0);
  }
  std::vector<ChainVar> v(h->nchains);
  CK(cudaMemcpyAsync(v.data(), h->d_var, sizeof(ChainVar) * h->nchains, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (auto &x : v) x.rdf_meas = 0;
  CK(cudaMemcpyAsync(h->d_var, v.data(), sizeof(ChainVar) * h->nchains, cudaMemcpyHostToDevice, h->stream));
  if (upload_desc(h)) return PIMC_ECUDA;
  int rc = sync_check(h);
  cudaFree(h->d_rdf);
  h->d_rdf = buf;
  h->n_rdf = tot;
  return rc;
}

int pimc_get_radial(void *handle, int chain, double *hist, unsigned long long *nmeas) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  const ChainDesc &d = h->desc[chain];
  if (d.rdf_nb <= 0) return fail(PIMC_EARG, "no pair-distance histogram (pimc_set_radial)");
  std::vector<unsigned long long> u((size_t)d.rdf_nb);
  CK(cudaMemcpyAsync(u.data(), d.rdf, 8 * u.size(), cudaMemcpyDeviceToHost, h->stream));
  ChainVar v;
  CK(cudaMemcpyAsync(&v, h->d_var + chain, sizeof(ChainVar), cudaMemcpyDeviceToHost, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  if (hist)
    for (size_t i = 0; i < u.size(); ++i) hist[i] = (double)u[i];
  if (nmeas) *nmeas = v.rdf_meas;
  return PIMC_OK;
}

int pimc_get_energy_sums(void *handle, int chain, double *sum, double *sumsq,
                         unsigned long long *count) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  ChainVar v;
  int rc = read_var(h, chain, &v);
  if (rc) return rc;
  for (int q = 0; q < 4; ++q) {
    if (sum) sum[q] = v.esum[q];
    if (sumsq) sumsq[q] = v.esum2[q];
  }
  if (count) *count = v.n_meas;
  return PIMC_OK;
}

int pimc_get_density(void *handle, int chain, double *hist, unsigned long long *ndata) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  const ChainDesc &d = h->desc[chain];
  if (d.dens_off < 0) return fail(PIMC_EARG, "no density histogram (density_nbins == 0)");
  const size_t nb = d.dim == 2 ? (size_t)d.dens_nb * d.dens_nb : (size_t)d.dens_nb;
  std::vector<unsigned long long> u(nb);
  CK(cudaMemcpyAsync(u.data(), h->d_upool + d.dens_off, nb * 8, cudaMemcpyDeviceToHost, h->stream));
  ChainVar v;
  CK(cudaMemcpyAsync(&v, h->d_var + chain, sizeof(ChainVar), cudaMemcpyDeviceToHost, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  if (hist)
    for (size_t i = 0; i < nb; ++i) hist[i] = (double)u[i];
  if (ndata) *ndata = v.ndata;
  return PIMC_OK;
}

int pimc_reset_measurements(void *handle) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  std::vector<ChainVar> v(h->nchains);
  CK(cudaMemcpyAsync(v.data(), h->d_var, sizeof(ChainVar) * h->nchains, cudaMemcpyDeviceToHost, h->stream));
  if (sync_check(h)) return PIMC_ECUDA;
  for (auto &x : v) {
    x.n_meas = x.ndata = x.eser_count = x.rdf_meas = 0;
    for (int q = 0; q < NOBS; ++q) x.esum[q] = x.esum2[q] = 0.0;
  }
  CK(cudaMemcpyAsync(h->d_var, v.data(), sizeof(ChainVar) * h->nchains, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemsetAsync(h->d_upool, 0, sizeof(unsigned long long) * h->n_upool, h->stream));
  if (h->d_rdf) CK(cudaMemsetAsync(h->d_rdf, 0, sizeof(unsigned long long) * h->n_rdf, h->stream));
  return sync_check(h);
}

int pimc_adjoint(void *handle, int chain, double *dSdr, double *dSdtheta, double *extra) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  const ChainDesc &d = h->desc[chain];
  if (d.flags & PF_CONTACT)
    return fail(PIMC_EARG, "the adjoint covers the Gaussian pair; chain " + std::to_string(chain) +
                               " uses the contact table, which has no parameter derivative");
  const size_t nbd = (size_t)d.N * d.M;
  const int nblocks = (int)((nbd + 255) / 256);
  const size_t need = 4 * nbd + (size_t)d.N + 8 * (size_t)nblocks + 16 + (size_t)d.dim * nbd;
  if (need > h->n_adj) {
    if (h->d_adj) cudaFree(h->d_adj);
    h->d_adj = nullptr;
    h->n_adj = 0;
    CK(cudaMalloc(&h->d_adj, need * sizeof(double)));
    h->n_adj = need;
  }
  AdjArgs a;
  a.desc = h->d_desc;
  a.dpool = h->d_dpool;
  a.ipool = h->d_ipool;
  a.chain = chain;
  a.omega = h->params[chain].harmonic_omega;
  a.gA = h->d_adj;
  a.gB = a.gA + 2 * nbd;
  a.part = a.gB + 2 * nbd;
  a.nblocks = nblocks;
  a.totals = a.part + 8 * (size_t)nblocks;
  a.sum_rg = a.totals + 8;
  a.dSdr = a.sum_rg + 8;
  a.inv = (int *)(a.dSdr + (size_t)d.dim * nbd);
  // inv needs N ints: the buffer has N doubles of room after dSdr
  CK(cudaMemsetAsync(a.sum_rg, 0, sizeof(double), h->stream));
  CK(launch_adjoint(a, (int)nbd, h->stream));
  double tot[9];
  CK(cudaMemcpyAsync(tot, a.totals, 8 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(tot + 8, a.sum_rg, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (dSdr) CK(cudaMemcpyAsync(dSdr, a.dSdr, sizeof(double) * d.dim * nbd, cudaMemcpyDeviceToHost, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  // totals: S_ext, dV0, domega, S_pair, dg, pair virial, r.g_ext
  if (dSdtheta) {
    dSdtheta[0] = tot[1];
    dSdtheta[1] = tot[2];
    dSdtheta[2] = tot[4];
  }
  if (extra) {
    const double Mt = d.M * d.tau;
    extra[0] = tot[0];
    extra[1] = tot[3];
    extra[2] = (tot[0] + 0.5 * tot[6]) / Mt + (tot[3] + 0.5 * tot[5]) / Mt;
    extra[3] = tot[8];
  }
  return PIMC_OK;
}

// the adjoint with its scratch in static device memory instead of a buffer
// grown by cudaMalloc: for callers that must not allocate device memory
// while they run (see pimc.h)
int pimc_adjoint_noalloc(void *handle, int chain, double *dSdr, double *dSdtheta, double *extra) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  const ChainDesc &d = h->desc[chain];
  if (d.flags & PF_CONTACT)
    return fail(PIMC_EARG, "the adjoint covers the Gaussian pair; chain " + std::to_string(chain) +
                               " uses the contact table, which has no parameter derivative");
  const size_t nbd = (size_t)d.N * d.M;
  const int nblocks = (int)((nbd + 255) / 256);
  const size_t need = 4 * nbd + (size_t)d.N + 8 * (size_t)nblocks + 16 + (size_t)d.dim * nbd;
  if (nbd > (size_t)kNoAllocBeads || d.N > kNoAllocParticles || need > kNoAllocDoubles)
    return fail(PIMC_EARG, "pimc_adjoint_noalloc serves chains of at most " +
                               std::to_string(kNoAllocBeads) + " beads (N*M) and " +
                               std::to_string(kNoAllocParticles) + " particles; chain " +
                               std::to_string(chain) + " has N*M = " + std::to_string(nbd) +
                               " (use pimc_adjoint)");
  int cur = -1;
  CK(cudaGetDevice(&cur));
  if (cur != h->device)
    return fail(PIMC_EARG, "pimc_adjoint_noalloc: the handle's device (" +
                               std::to_string(h->device) + ") is not the current device (" +
                               std::to_string(cur) + ")");
  double *base = nullptr;
  CK(adjoint_static_scratch(&base));
  AdjArgs a;
  a.desc = h->d_desc;
  a.dpool = h->d_dpool;
  a.ipool = h->d_ipool;
  a.chain = chain;
  a.omega = h->params[chain].harmonic_omega;
  a.gA = base;
  a.gB = a.gA + 2 * nbd;
  a.part = a.gB + 2 * nbd;
  a.nblocks = nblocks;
  a.totals = a.part + 8 * (size_t)nblocks;
  a.sum_rg = a.totals + 8;
  a.dSdr = a.sum_rg + 8;
  a.inv = (int *)(a.dSdr + (size_t)d.dim * nbd);
  // the only accumulator the kernels do not overwrite
  CK(cudaMemsetAsync(a.sum_rg, 0, sizeof(double), h->stream));
  CK(launch_adjoint(a, (int)nbd, h->stream));
  double tot[9];
  CK(cudaMemcpyAsync(tot, a.totals, 8 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(tot + 8, a.sum_rg, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (dSdr) CK(cudaMemcpyAsync(dSdr, a.dSdr, sizeof(double) * d.dim * nbd, cudaMemcpyDeviceToHost, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  if (dSdtheta) {
    dSdtheta[0] = tot[1];
    dSdtheta[1] = tot[2];
    dSdtheta[2] = tot[4];
  }
  if (extra) {
    const double Mt = d.M * d.tau;
    extra[0] = tot[0];
    extra[1] = tot[3];
    extra[2] = (tot[0] + 0.5 * tot[6]) / Mt + (tot[3] + 0.5 * tot[5]) / Mt;
    extra[3] = tot[8];
  }
  return PIMC_OK;
}

// the batched adjoint's pool: per bead gA, gB (2 doubles each), per block a
// row of 9 partials, per chain 9 totals, dS/dr in the host layout of every
// chain, per chain omega, then the int maps (block -> chain, first block,
// inverse-permutation offsets, the inverse permutations) and the bead
// offsets.  One cudaMalloc for the handle's lifetime.
static int batch_adjoint_setup(Handle *h) {
  if (h->badj_ready) return PIMC_OK;
  const int nc = h->nchains;
  std::vector<int> blk_chain, blk_first(nc), inv_off(nc);
  std::vector<long long> bead_off(nc);
  std::vector<double> omega(nc);
  long long tb = 0;
  int ninv = 0;
  for (int c = 0; c < nc; ++c) {
    const ChainDesc &d = h->desc[c];
    const long long nm = (long long)d.N * d.M;
    blk_first[c] = (int)blk_chain.size();
    for (long long b = 0; b < (nm + 255) / 256; ++b) blk_chain.push_back(c);
    bead_off[c] = tb;
    tb += nm;
    inv_off[c] = ninv;
    ninv += d.N;
    omega[c] = h->params[c].harmonic_omega;
  }
  const size_t nblocks = blk_chain.size();
  if (nblocks > (size_t)0x7fffffff) return fail(PIMC_EARG, "batch too large for the adjoint");
  // one CTA per chain slice when every chain's accumulators (32 N bytes, and
  // 12 KB for the kernel's static reduction buffer, queues and descriptor)
  // fit the device's shared memory
  std::vector<int> slice_first(nc);
  long long ns = 0;
  for (int c = 0; c < nc; ++c) {
    slice_first[c] = (int)ns;
    ns += h->desc[c].M;
  }
  const bool slices = 32LL * h->maxN + 12288 <= (long long)h->max_dyn_smem && ns < 0x7fffffffLL;
  const size_t nd = 4 * (size_t)tb + 9 * nblocks + 9 * (size_t)nc + h->n_stage + (size_t)nc +
                    8 * (size_t)ns;
  const size_t ni = nblocks + 3 * (size_t)nc + (size_t)ninv;
  const size_t bytes = 8 * nd + 4 * ((ni + 1) & ~(size_t)1) + 8 * (size_t)nc;
  double *pool = nullptr;
  if (cudaMalloc(&pool, bytes) != cudaSuccess)
    return fail(PIMC_ENOMEM, "batched adjoint pool of " + std::to_string(bytes) + " bytes");
  AdjBatchArgs &a = h->badj;
  a.desc = h->d_desc;
  a.dpool = h->d_dpool;
  a.ipool = h->d_ipool;
  a.gA = pool;
  a.gB = a.gA + 2 * (size_t)tb;
  a.part = a.gB + 2 * (size_t)tb;
  a.totals = a.part + 9 * nblocks;
  a.dSdr = a.totals + 9 * (size_t)nc;
  double *om = a.dSdr + h->n_stage;
  a.part_s = om + nc;
  int *ip = (int *)(a.part_s + 8 * (size_t)ns);
  int *bc = ip, *bf = bc + nblocks, *io = bf + nc, *sf = io + nc, *inv = sf + nc;
  long long *bo = (long long *)(ip + ((ni + 1) & ~(size_t)1));
  a.omega = om;
  a.blk_chain = bc;
  a.blk_first = bf;
  a.inv_off = io;
  a.inv = inv;
  a.bead_off = bo;
  a.nblocks = (int)nblocks;
  a.nchains = nc;
  a.use_slices = slices ? 1 : 0;
  a.nslices = (int)ns;
  a.slice_first = sf;
  h->d_badj = pool;
  CK(cudaMemcpyAsync(om, omega.data(), 8 * (size_t)nc, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(bc, blk_chain.data(), 4 * nblocks, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(bf, blk_first.data(), 4 * (size_t)nc, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(io, inv_off.data(), 4 * (size_t)nc, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(sf, slice_first.data(), 4 * (size_t)nc, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(bo, bead_off.data(), 8 * (size_t)nc, cudaMemcpyHostToDevice, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  h->badj_ready = true;
  return PIMC_OK;
}

int pimc_batch_adjoint(void *handle, double *dSdtheta, double *extra, double *dSdr_all) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  for (int c = 0; c < h->nchains; ++c)
    if (h->desc[c].flags & PF_CONTACT)
      return fail(PIMC_EARG, "the adjoint covers the Gaussian pair; chain " + std::to_string(c) +
                                 " uses the contact table, which has no parameter derivative");
  int rc = batch_adjoint_setup(h);
  if (rc) return rc;
  AdjBatchArgs a = h->badj;
  if (!dSdr_all) a.dSdr = nullptr;
  CK(cudaEventRecord(h->ev0, h->stream));
  CK(launch_adjoint_batch(a, h->maxN, h->stream));
  CK(cudaEventRecord(h->ev1, h->stream));
  std::vector<double> tot(9 * (size_t)h->nchains);
  CK(cudaMemcpyAsync(tot.data(), a.totals, 8 * tot.size(), cudaMemcpyDeviceToHost, h->stream));
  if (dSdr_all)
    CK(cudaMemcpyAsync(dSdr_all, a.dSdr, 8 * h->n_stage, cudaMemcpyDeviceToHost, h->stream));
  rc = sync_check(h);
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  h->last_launches = 4;
  for (int c = 0; c < h->nchains; ++c) {
    const double *t = tot.data() + 9 * (size_t)c;
    const ChainDesc &d = h->desc[c];
    if (dSdtheta) {
      dSdtheta[3 * c] = t[1];
      dSdtheta[3 * c + 1] = t[2];
      dSdtheta[3 * c + 2] = t[4];
    }
    if (extra) {
      const double Mt = d.M * d.tau;
      extra[4 * c] = t[0];
      extra[4 * c + 1] = t[3];
      extra[4 * c + 2] = (t[0] + 0.5 * t[6]) / Mt + (t[3] + 0.5 * t[5]) / Mt;
      extra[4 * c + 3] = t[8];
    }
  }
  return PIMC_OK;
}

int pimc_contact_table(double g0, double tau, double range, int n, double *out) {
  if (!(g0 != 0.0) || !std::isfinite(g0) || !(tau > 0.0) || !(range > 0.0) || n < 2 || n > 4096 ||
      !out)
    return fail(PIMC_EARG, "contact table needs g0 != 0, tau > 0, range > 0, 2 <= n <= 4096");
  double *d = nullptr;
  CK(cudaMalloc(&d, sizeof(double) * (size_t)n * n));
  cudaError_t e = launch_contact_table(d, n, range, g0, tau, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(out, d, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return fail(PIMC_ECUDA, std::string("contact table: ") + cudaGetErrorString(e));
  return PIMC_OK;
}

namespace {
// the reference's grid: range(1e-20, range, n) (src/propagator.jl:39-45)
constexpr double kContactR0 = 1e-20;

int contact_targets(Handle *h, int chain, int *c0, int *c1) {
  if (!h) return fail(PIMC_EARG, "null handle");
  if (chain < -1 || chain >= h->nchains) return fail(PIMC_EARG, "chain out of range");
  *c0 = chain < 0 ? 0 : chain;
  *c1 = chain < 0 ? h->nchains : chain + 1;
  for (int c = *c0; c < *c1; ++c)
    if (!(h->desc[c].flags & PF_PAIR))
      return fail(PIMC_EARG, "chain " + std::to_string(c) +
                                 " has no pair propagator (create it with interactions = 1)");
  return PIMC_OK;
}

void attach_contact(ChainDesc &d, const double *tab, int n, double range) {
  d.ct_tab = tab;
  d.ct_n = n;
  d.ct_r0 = kContactR0;
  d.ct_rmax = range;
  d.ct_h = (range - kContactR0) / (double)(n - 1);
  d.flags |= PF_CONTACT;
}

// drop device tables no chain refers to any more
void release_contact_tables(Handle *h) {
  for (size_t i = 0; i < h->ctabs.size();) {
    bool used = false;
    for (const auto &d : h->desc) used = used || ((d.flags & PF_CONTACT) && d.ct_tab == h->ctabs[i].d);
    if (used) { ++i; continue; }
    cudaFree(h->ctabs[i].d);
    h->ctabs.erase(h->ctabs.begin() + (long)i);
  }
}

int contact_args(double range, int n) {
  if (!(range > kContactR0) || !std::isfinite(range) || n < 2 || n > 4096)
    return fail(PIMC_EARG, "contact table needs range > 0 and 2 <= n <= 4096");
  return PIMC_OK;
}
}  // namespace

int pimc_set_contact_propagator(void *handle, int chain, double g0, double range, int n) {
  Handle *h = H(handle);
  int c0, c1;
  if (contact_targets(h, chain, &c0, &c1)) return PIMC_EARG;
  if (n == 0) n = 600;
  if (!(g0 != 0.0) || !std::isfinite(g0)) return fail(PIMC_EARG, "contact propagator needs g0 != 0");
  if (contact_args(range, n)) return PIMC_EARG;
  CK(cudaStreamSynchronize(h->stream));
  for (int c = c0; c < c1; ++c) {
    const double tau = h->desc[c].tau;
    const double *tab = nullptr;
    for (const auto &t : h->ctabs)
      if (!t.given && t.g0 == g0 && t.tau == tau && t.range == range && t.n == n) tab = t.d;
    if (!tab) {
      double *d = nullptr;
      CK(cudaMalloc(&d, sizeof(double) * (size_t)n * n));
      h->ctabs.push_back({g0, tau, range, n, false, d});
      CK(launch_contact_table(d, n, range, g0, tau, h->stream));
      tab = d;
    }
    attach_contact(h->desc[c], tab, n, range);
  }
  if (upload_desc(h)) return PIMC_ECUDA;
  int rc = sync_check(h);
  release_contact_tables(h);
  return rc;
}

int pimc_set_contact_table(void *handle, int chain, const double *tab, int n, double range) {
  Handle *h = H(handle);
  int c0, c1;
  if (contact_targets(h, chain, &c0, &c1)) return PIMC_EARG;
  if (!tab) return fail(PIMC_EARG, "null table");
  if (contact_args(range, n)) return PIMC_EARG;
  const size_t cnt = (size_t)n * n;
  for (size_t i = 0; i < cnt; ++i)
    if (std::isnan(tab[i])) return fail(PIMC_EARG, "contact table holds NaN");
  CK(cudaStreamSynchronize(h->stream));
  double *d = nullptr;
  CK(cudaMalloc(&d, sizeof(double) * cnt));
  h->ctabs.push_back({0.0, 0.0, range, n, true, d});
  CK(cudaMemcpy(d, tab, sizeof(double) * cnt, cudaMemcpyHostToDevice));
  for (int c = c0; c < c1; ++c) attach_contact(h->desc[c], d, n, range);
  if (upload_desc(h)) return PIMC_ECUDA;
  int rc = sync_check(h);
  release_contact_tables(h);
  return rc;
}

int pimc_get_contact_table(void *handle, int chain, double *out, size_t cap, int *n, double *range) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  const ChainDesc &d = h->desc[chain];
  if (!(d.flags & PF_CONTACT)) {
    if (n) *n = 0;
    if (range) *range = 0.0;
    return PIMC_OK;
  }
  if (n) *n = d.ct_n;
  if (range) *range = d.ct_rmax;
  if (out) {
    const size_t cnt = (size_t)d.ct_n * d.ct_n;
    if (cap < cnt) return fail(PIMC_EARG, "output holds fewer than n*n values");
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(out, d.ct_tab, sizeof(double) * cnt, cudaMemcpyDeviceToHost));
  }
  return PIMC_OK;
}

int pimc_clear_contact(void *handle, int chain) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  if (chain < -1 || chain >= h->nchains) return fail(PIMC_EARG, "chain out of range");
  const int c0 = chain < 0 ? 0 : chain, c1 = chain < 0 ? h->nchains : chain + 1;
  for (int c = c0; c < c1; ++c) {
    ChainDesc &d = h->desc[c];
    d.flags &= ~PF_CONTACT;
    d.ct_tab = nullptr;
    d.ct_n = 0;
  }
  CK(cudaStreamSynchronize(h->stream));
  if (upload_desc(h)) return PIMC_ECUDA;
  int rc = sync_check(h);
  release_contact_tables(h);
  return rc;
}

int pimc_fp64_peak(void *handle, double *tflops) {
  Handle *h = H(handle);
  if (!h || !tflops) return fail(PIMC_EARG, "null argument");
  CK(fp64_peak(h->num_sms, h->stream, tflops));
  return PIMC_OK;
}

int pimc_set_potential(void *handle, int chain, double V0, double omega, double g) {
  Handle *h = H(handle);
  if (check_chain(h, chain)) return PIMC_EARG;
  pimc_params &p = h->params[chain];
  if (V0 != 0.0 && !(p.lattice_a > 0.0)) return fail(PIMC_EARG, "lattice_a must be positive");
  p.lattice_V0 = V0;
  p.harmonic_omega = omega;
  p.pair_g = g;
  ChainDesc &d = h->desc[chain];
  d.V0 = V0;
  d.lat_k = V0 != 0.0 ? 1.0 / p.lattice_a : 0.0;
  d.hcoef = 0.5 * omega * omega;
  d.g = g;
  d.mhtau_g = -0.5 * d.tau * d.g;
  d.flags &= ~(PF_LATT | PF_HARM);
  if (V0 != 0.0) d.flags |= PF_LATT;
  if (omega != 0.0) d.flags |= PF_HARM;
  if (upload_desc(h)) return PIMC_ECUDA;
  CK(launch_links(h->d_desc, h->d_dpool, h->d_ipool, chain, 1, h->maxNM, h->stream));
  return sync_check(h);
}

int pimc_set_beams(void *handle, int chain, const double *angles, int nangles, double scale,
                   double depth, int helical) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  if (chain < -1 || chain >= h->nchains) return fail(PIMC_EARG, "chain out of range");
  if (nangles < 0 || nangles > MAX_BEAMS || (nangles > 0 && !angles))
    return fail(PIMC_EARG, "between 0 and " + std::to_string(MAX_BEAMS) + " beam angles");
  if (nangles > 0 && !(std::isfinite(scale) && std::isfinite(depth)))
    return fail(PIMC_EARG, "scale and depth must be finite");
  for (int k = 0; k < nangles; ++k)
    if (!std::isfinite(angles[k])) return fail(PIMC_EARG, "beam angles must be finite");
  const int c0 = chain < 0 ? 0 : chain, c1 = chain < 0 ? h->nchains : chain + 1;
  for (int c = c0; c < c1; ++c)
    if (nangles > 0 && h->desc[c].dim != 2)
      return fail(PIMC_EARG, "the optical lattice is two-dimensional (chain " + std::to_string(c) + ")");
  CK(cudaStreamSynchronize(h->stream));
  for (int c = c0; c < c1; ++c) {
    ChainDesc &d = h->desc[c];
    d.nbeam = nangles;
    d.beam_helical = helical ? 1 : 0;
    d.beam_scale = scale;
    d.beam_depth = depth;
    for (int k = 0; k < MAX_BEAMS; ++k) {
      d.beam_sin[k] = k < nangles ? std::sin(angles[k]) : 0.0;
      d.beam_cos[k] = k < nangles ? std::cos(angles[k]) : 0.0;
    }
    if (nangles > 0 && depth != 0.0) d.flags |= PF_BEAM;
    else d.flags &= ~PF_BEAM;
  }
  if (upload_desc(h)) return PIMC_ECUDA;
  CK(launch_links(h->d_desc, h->d_dpool, h->d_ipool, c0, c1 - c0, h->maxNM, h->stream));
  return sync_check(h);
}

int pimc_get_stats(void *handle, int chain, pimc_stats *out) {
  Handle *h = H(handle);
  if (check_chain(h, chain) || !out) return fail(PIMC_EARG, "bad argument");
  ChainVar v;
  int rc = read_var(h, chain, &v);
  if (rc) return rc;
  fill_stats(v, out);
  return PIMC_OK;
}

int pimc_get_total_stats(void *handle, pimc_stats *out) {
  Handle *h = H(handle);
  if (!h || !out) return fail(PIMC_EARG, "null argument");
  std::vector<ChainVar> v(h->nchains);
  CK(cudaMemcpyAsync(v.data(), h->d_var, sizeof(ChainVar) * h->nchains, cudaMemcpyDeviceToHost, h->stream));
  int rc = sync_check(h);
  if (rc) return rc;
  memset(out, 0, sizeof(*out));
  for (auto &x : v) {
    for (int q = 0; q < 4; ++q) {
      out->attempts[q] += x.att[q];
      out->accepts[q] += x.acc[q];
    }
    out->skips += x.skips;
    out->bead_updates += x.bead_updates;
    for (int q = 0; q < 4; ++q) out->bead_updates_kind[q] += x.beads_kind[q];
    out->sweeps += x.sweep;
    out->measurements += x.n_meas;
  }
  if (!v.empty()) {
    out->stage_slices = v[0].stage_m;
    out->swap_slices = v[0].swap_m;
    out->com_step = v[0].com_step;
    out->pcom_step = v[0].pcom_step;
  }
  return PIMC_OK;
}

// checkpoint layout: magic, version, nchains, then per chain ChainVar, the
// raw device regions (positions, links and 16-bit mirror, next, density,
// observable series), the number of pair-distance bins and those counts.
// ChainVar::rdf_meas counts the measurements in the pair-distance histogram,
// so both travel together: a restored chain's g(r) normalisation matches its
// counts.
int pimc_state_size(void *handle, size_t *bytes) {
  Handle *h = H(handle);
  if (!h || !bytes) return fail(PIMC_EARG, "null argument");
  size_t b = 3 * sizeof(unsigned);
  for (const auto &d : h->desc) {
    b += sizeof(ChainVar) + 8 * (size_t)(d.tab_off - d.x_off) + 4 * (size_t)d.N;
    if (d.dens_off >= 0) b += 8 * (d.dim == 2 ? (size_t)d.dens_nb * d.dens_nb : (size_t)d.dens_nb);
    if (d.eser_off >= 0) b += 8 * (size_t)NOBS * d.eser_cap;
    b += sizeof(int) + 8 * (size_t)std::max(d.rdf_nb, 0);
  }
  *bytes = b;
  return PIMC_OK;
}

static int state_io(Handle *h, char *buf, size_t bytes, bool save) {
  size_t need = 0;
  pimc_state_size(h, &need);
  if (!buf || bytes < need) return fail(PIMC_EARG, "state buffer too small");
  char *p = buf;
  unsigned hdr[3] = {kStateMagic, (unsigned)PIMC_ABI_VERSION, (unsigned)h->nchains};
  if (save) {
    memcpy(p, hdr, sizeof(hdr));
  } else {
    unsigned in[3];
    memcpy(in, p, sizeof(in));
    if (in[0] != hdr[0] || in[1] != hdr[1] || in[2] != hdr[2])
      return fail(PIMC_ESTATE, "state does not belong to a handle of this shape");
  }
  p += sizeof(hdr);
  const auto kind = save ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice;
  auto io = [&](void *dev, size_t n) -> cudaError_t {
    cudaError_t e = save ? cudaMemcpyAsync(p, dev, n, kind, h->stream) : cudaMemcpyAsync(dev, p, n, kind, h->stream);
    p += n;
    return e;
  };
  // every chain's next values (in range: a kernel indexes with them) and
  // radial bin count are checked before anything is written to the device,
  // so a refused snapshot leaves the handle untouched.  Whether next is a
  // permutation is the device's check (ChainVar::err, PIMC_EDEVICE).
  if (!save) {
    const char *q = p;
    for (int c = 0; c < h->nchains; ++c) {
      const ChainDesc &d = h->desc[c];
      q += sizeof(ChainVar) + 8 * (size_t)(d.tab_off - d.x_off);
      for (int i = 0; i < d.N; ++i) {
        int v = 0;
        memcpy(&v, q + 4 * (size_t)i, sizeof(int));
        if (v < 0 || v >= d.N)
          return fail(PIMC_ESTATE, "state has next[" + std::to_string(i) + "] = " +
                                       std::to_string(v) + " out of range on chain " +
                                       std::to_string(c));
      }
      q += 4 * (size_t)d.N;
      if (d.dens_off >= 0) q += 8 * (d.dim == 2 ? (size_t)d.dens_nb * d.dens_nb : (size_t)d.dens_nb);
      if (d.eser_off >= 0) q += 8 * (size_t)NOBS * d.eser_cap;
      int nb = 0;
      memcpy(&nb, q, sizeof(int));
      if (nb != std::max(d.rdf_nb, 0))
        return fail(PIMC_ESTATE, "state has " + std::to_string(nb) + " pair-distance bins on chain " +
                                     std::to_string(c) + ", the handle " +
                                     std::to_string(std::max(d.rdf_nb, 0)) + " (pimc_set_radial)");
      q += sizeof(int) + 8 * (size_t)nb;
    }
  }
  for (int c = 0; c < h->nchains; ++c) {
    const ChainDesc &d = h->desc[c];
    CK(io(h->d_var + c, sizeof(ChainVar)));
    CK(io(h->d_dpool + d.x_off, 8 * (size_t)(d.tab_off - d.x_off)));
    CK(io(h->d_ipool + d.next_off, 4 * (size_t)d.N));
    if (d.dens_off >= 0) CK(io(h->d_upool + d.dens_off, 8 * (d.dim == 2 ? (size_t)d.dens_nb * d.dens_nb : (size_t)d.dens_nb)));
    if (d.eser_off >= 0) CK(io(h->d_dpool + d.eser_off, 8 * (size_t)NOBS * d.eser_cap));
    const int nb = std::max(d.rdf_nb, 0);
    if (save) memcpy(p, &nb, sizeof(int));
    p += sizeof(int);
    if (nb > 0) CK(io(d.rdf, 8 * (size_t)nb));
  }
  return sync_check(h);
}

int pimc_get_state(void *handle, void *buf, size_t bytes) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  return state_io(h, (char *)buf, bytes, true);
}

int pimc_set_state(void *handle, const void *buf, size_t bytes) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  return state_io(h, (char *)const_cast<void *>(buf), bytes, false);
}

int pimc_device_info(void *handle, char *name, size_t cap, int *num_sms) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, h->device));
  if (name && cap > 0) {
    strncpy(name, prop.name, cap - 1);
    name[cap - 1] = '\0';
  }
  if (num_sms) *num_sms = h->num_sms;
  return PIMC_OK;
}

int pimc_swap_profile(void *handle, unsigned long long *out, int reset) {
  Handle *h = H(handle);
  if (!h || !out) return fail(PIMC_EARG, "null argument");
  const cudaError_t e = profile_take(out, reset != 0, h->stream);
  if (e == cudaErrorNotSupported)
    return fail(PIMC_EARG, "pimc_swap_profile needs the profiling build (nvcc -DPIMC_PROFILE=1)");
  if (e != cudaSuccess) return fail(PIMC_ECUDA, std::string("swap profile: ") + cudaGetErrorString(e));
  return PIMC_OK;
}

int pimc_last_run_ms(void *handle, double *ms) {
  if (!handle || !ms) return fail(PIMC_EARG, "null argument");
  *ms = H(handle)->last_ms;
  return PIMC_OK;
}

int pimc_last_run_launches(void *handle, long long *launches) {
  if (!handle || !launches) return fail(PIMC_EARG, "null argument");
  *launches = H(handle)->last_launches;
  return PIMC_OK;
}

int pimc_set_option(void *handle, int key, long long value) {
  Handle *h = H(handle);
  if (!h) return fail(PIMC_EARG, "null handle");
  if (key == PIMC_OPT_FORCE_WARP_WINDOW) {
    h->force_warp = value != 0;
    return PIMC_OK;
  }
  if (key == PIMC_OPT_CELL_LISTS || key == PIMC_OPT_CELL_CROWDING) {
    if (key == PIMC_OPT_CELL_LISTS && (value < 0 || value > 2))
      return fail(PIMC_EARG, "cell lists: 0 off, 1 auto, 2 always");
    if (key == PIMC_OPT_CELL_CROWDING && (value < 1 || value > 1000000))
      return fail(PIMC_EARG, "cell crowding bound in thousandths must be in [1, 1e6]");
    for (auto &d : h->desc) {
      if (key == PIMC_OPT_CELL_LISTS) d.cl_mode = (int)value;
      else d.cl_frac = (float)(value / 1000.0);
    }
    if (upload_desc(h)) return PIMC_ECUDA;
    return sync_check(h);
  }
  if (key == PIMC_OPT_EXACT_DECISIONS) {
    for (auto &d : h->desc) d.flags = value ? (d.flags | PF_EXACT) : (d.flags & ~PF_EXACT);
    if (upload_desc(h)) return PIMC_ECUDA;
    if (h->gexec) {
      cudaGraphExecDestroy(h->gexec);
      h->gexec = nullptr;
    }
    return sync_check(h);
  }
  return fail(PIMC_EARG, "unknown option");
}

}  // extern "C"
