// Host side of the fused ROF path: validation, workspace layout, dispatch
// over (dtype, D, C) and the per-iteration launch sequence.
#include <string.h>

#include <mutex>

#include "rof_kernels.cuh"
#include "rof_vec.cuh"
#include "rof_pipe.cuh"
#include "rof_sweep.cuh"
#include "rof_sweep3.cuh"
#include "rof_sweep1.cuh"

namespace opyx {
namespace rof {

// Workspace layout (bytes): [0, 256) adaptive state, [256, 512) info record,
// [512, 512 + kPartials) FP64 block partials, then 256 bytes of ticket
// counters (one word, or 1 + kTicketGroups for the grouped arrivals of the
// FP32 gap reductions), zeroed by opyx_rof_init.
constexpr size_t kStateOff = 0;
constexpr size_t kInfoOff = 256;
constexpr int kMaxBlocks = 4096;
constexpr size_t kPartialsOff = 512;
constexpr size_t kPartialsBytes = (size_t)kMaxBlocks * 5 * sizeof(double);
constexpr size_t kTicketOff = kPartialsOff + kPartialsBytes;
constexpr size_t kWsBytes = kTicketOff + 256;
static_assert((1 + kTicketGroups) * sizeof(unsigned) <= 256, "ticket counters");

static_assert(sizeof(opyx_adaptive_state) <= 256, "state record too large");
static_assert(sizeof(opyx_rof_info) <= 256, "info record too large");

// Problems with more than 2^40 dual values (N * D * C) are rejected: far
// beyond any device memory, and it keeps every product of the dims, the
// channel count and an element size inside int64.
constexpr int64_t kMaxValues = (int64_t)1 << 40;

// N = prod(dims) for ndim in [1, 3] and nchannels in [1, OPYX_ROF_MAX_C];
// false if a dim is < 1 or N * ndim * nchannels exceeds kMaxValues (checked
// before each multiplication, so nothing wraps).
static bool count_pixels(const opyx_rof_problem* p, int64_t* n_out) {
  int64_t n = 1;
  for (int t = 0; t < p->ndim; ++t) {
    if (p->dims[t] < 1 || p->dims[t] > kMaxValues / n) return false;
    n *= p->dims[t];
  }
  if (n > kMaxValues / ((int64_t)p->ndim * p->nchannels)) return false;
  *n_out = n;
  return true;
}

static int validate(const opyx_rof_problem* p, const opyx_rof_buffers* b) {
  if (!p || !b) return OPYX_ERR_ARG;
  if (p->dtype != OPYX_F32 && p->dtype != OPYX_F64) return OPYX_ERR_ARG;
  if (p->ndim < 1 || p->ndim > 3) return OPYX_ERR_UNSUPPORTED;
  if (p->nchannels < 1 || p->nchannels > OPYX_ROF_MAX_C) return OPYX_ERR_UNSUPPORTED;
  if (p->steps < OPYX_STEPS_CONST || p->steps > OPYX_STEPS_PRECOND) return OPYX_ERR_ARG;
  int64_t npix = 0;
  if (!count_pixels(p, &npix)) return OPYX_ERR_ARG;
  for (int t = 0; t < p->ndim; ++t)
    if (!(p->h[t] > 0)) return OPYX_ERR_ARG;
  for (int k = 0; k < p->nchannels; ++k)
    if (!(p->vol[k] > 0)) return OPYX_ERR_ARG;
  if (!(p->lbd > 0) || p->huber_alpha < 0 || !(p->theta > 0)) return OPYX_ERR_ARG;
  if (p->term_mode < 0 || p->term_mode > 2) return OPYX_ERR_ARG;
  if (p->term_mode == 2 && p->steps != OPYX_STEPS_ADAPTIVE) return OPYX_ERR_ARG;
  if (p->steps != OPYX_STEPS_PRECOND && (!(p->tau > 0) || !(p->sigma > 0))) return OPYX_ERR_ARG;
  if (p->steps == OPYX_STEPS_ADAPTIVE &&
      (!(p->alpha0 > 0) || !(p->alpha0 < 1) || !(p->Delta > 1) || !(p->eta > 0)))
    return OPYX_ERR_ARG;
  if (!b->x || !b->xbar || !b->y || !b->f || !b->ws) return OPYX_ERR_ARG;
  if (p->steps == OPYX_STEPS_ADAPTIVE && (!b->xgrad || !b->gp)) return OPYX_ERR_ARG;
  if (((uintptr_t)b->ws) & 255) return OPYX_ERR_WORKSPACE;
  const size_t al = p->dtype == OPYX_F32 ? 4 : 8;
  if (((uintptr_t)b->x | (uintptr_t)b->xbar | (uintptr_t)b->y | (uintptr_t)b->f) & (al - 1))
    return OPYX_ERR_ARG;
  return OPYX_OK;
}

template <typename T>
static Geo<T> make_geo(const opyx_rof_problem* p) {
  Geo<T> g;
  memset(&g, 0, sizeof(g));
  const int D = p->ndim;
  double invh[3] = {1.0, 1.0, 1.0};
  g.N = 1;
  for (int t = 0; t < 3; ++t) { g.n[t] = 1; g.s[t] = 1; }
  for (int t = 0; t < D; ++t) { g.n[t] = p->dims[t]; invh[t] = 1.0 / p->h[t]; g.N *= p->dims[t]; }
  int64_t s = 1;
  for (int t = D - 1; t >= 0; --t) { g.s[t] = s; s *= g.n[t]; }
  g.nl = g.n[D - 1];
  g.rows = g.N / g.nl;
  for (int t = 0; t < 3; ++t) {
    g.invh[t] = (T)invh[t];
    for (int k = 0; k < OPYX_ROF_MAX_C; ++k) {
      const double w = k < p->nchannels ? p->weights[k] : 1.0;
      g.coef[t][k] = (T)(w * invh[t]);
      g.absc[t][k] = (T)(fabs(w) * invh[t]);
      const double rs = 2.0 * fabs(w) * invh[t];
      g.sig_pre[t][k] = (T)(rs > 2.220446049250313e-16 ? 1.0 / rs : 0.0);
    }
  }
  for (int k = 0; k < OPYX_ROF_MAX_C; ++k) {
    const double w = k < p->nchannels ? p->weights[k] : 1.0;
    const double v = k < p->nchannels ? p->vol[k] : 1.0;
    g.w[k] = (T)w;
    g.vol[k] = (T)v;
    g.half_rvol[k] = (T)(0.5 / v);
  }
  g.lbd = (T)p->lbd;
  g.lbd2 = (T)(p->lbd * p->lbd);
  g.lbd_d = p->lbd;
  g.huber_d = p->huber_alpha;
  g.use_huber = p->huber_alpha > 0;
  g.huber = (T)p->huber_alpha;
  g.half_huber = (T)(0.5 * p->huber_alpha);
  g.half_rhuber = (T)(p->huber_alpha > 0 ? 0.5 / p->huber_alpha : 0.0);
  g.hub_ratio = (T)(p->huber_alpha / p->lbd);
  g.theta = (T)p->theta;
  g.theta1 = (T)(1.0 + p->theta);
  g.steps = p->steps;
  g.term_mode = p->term_mode;
  g.term_relgap = p->term_relgap;
  g.term_infeas = p->term_infeas;
  // preconditioner tables: neighbour counts (n_last, n_row, n_z) -> tau etc.
  for (int cb = 0; cb < 27; ++cb) {
    const int nl_ = cb % 3, nr = (cb / 3) % 3, nz = cb / 9;
    for (int k = 0; k < OPYX_ROF_MAX_C; ++k) {
      const double w = fabs(k < p->nchannels ? p->weights[k] : 1.0);
      const double v = k < p->nchannels ? p->vol[k] : 1.0;
      double cs = w * invh[D - 1] * nl_;
      if (D >= 2) cs += w * invh[D - 2] * nr;
      if (D == 3) cs += w * invh[0] * nz;
      const double tau = cs > 2.220446049250313e-16 ? 1.0 / cs : 0.0;
      g.tau_tab[cb][k] = (T)tau;
      g.tv_tab[cb][k] = (T)(tau * v);
      g.a_tab[cb][k] = (T)(1.0 / (1.0 + tau * v));
    }
  }
  for (int t = 0; t < 3; ++t)
    for (int k = 0; k < OPYX_ROF_MAX_C; ++k) {
      const double w = k < p->nchannels ? p->weights[k] : 1.0;
      const double rs = 2.0 * fabs(w) * invh[t];
      const double sig = rs > 2.220446049250313e-16 ? 1.0 / rs : 0.0;
      g.hub_pre[t][k] = (T)(1.0 / (1.0 + sig * (p->huber_alpha / p->lbd)));
    }
  return g;
}

template <typename T>
static Args<T> make_args(const opyx_rof_problem* p, const opyx_rof_buffers* b) {
  Args<T> a;
  a.x = (T*)b->x;
  a.xbar = (T*)b->xbar;
  a.y = (T*)b->y;
  a.f = (const T*)b->f;
  a.mask = b->mask;
  a.xgrad = (T*)b->xgrad;
  a.gp = (T*)b->gp;
  a.x2 = (T*)b->xbar;
  a.y2 = (T*)b->y2;
  char* ws = (char*)b->ws;
  a.st = (opyx_adaptive_state*)(ws + kStateOff);
  a.info = (opyx_rof_info*)(ws + kInfoOff);
  a.partials = (double*)(ws + kPartialsOff);
  a.ticket = (unsigned*)(ws + kTicketOff);
  a.tau = p->tau;
  a.sigma = p->sigma;
  return a;
}

// Launch shape: 32 x 8 threads; x covers the contiguous axis, y-blocks run
// grid-stride over the remaining rows.  Reduction kernels cap the number of
// blocks at kMaxBlocks (their partials buffer).
template <typename T>
static void shape(const Geo<T>& g, dim3* grid, dim3* block, bool reduce) {
  *block = dim3(32, 8, 1);
  const int64_t cap_total = reduce ? kMaxBlocks : (int64_t)sm_count() * 64;
  int64_t gx = (g.nl + 31) / 32;
  if (gx > cap_total) gx = cap_total;          // the kernels grid-stride along x too
  int64_t gy = (g.rows + 7) / 8;
  int64_t cap_y = cap_total / gx;
  if (cap_y < 1) cap_y = 1;
  if (gy > cap_y) gy = cap_y;
  if (gy > 65535) gy = 65535;
  *grid = dim3((unsigned)gx, (unsigned)gy, 1);   // gx * gy <= cap_total
}

// The vectorised FP32 kernels need the contiguous axis to be a multiple of 4
// and 16-byte aligned arrays (4-byte aligned mask).
template <typename T>
static bool vec_ok(const opyx_rof_problem* p, const opyx_rof_buffers* b) {
  if (p->dtype != OPYX_F32 || (p->flags & 1)) return false;
  if (p->dims[p->ndim - 1] % 4 != 0) return false;
  // the gap reduction has at most kMaxBlocks blocks and the vectorised
  // kernels do not stride along the contiguous axis
  if ((p->dims[p->ndim - 1] / 4 + kVecThreads - 1) / kVecThreads > kMaxBlocks) return false;
  const uintptr_t al = (uintptr_t)b->x | (uintptr_t)b->xbar | (uintptr_t)b->y | (uintptr_t)b->f;
  if (al & 15) return false;
  if (b->mask && ((uintptr_t)b->mask & 3)) return false;
  return true;
}

// Rows per thread of the vectorised kernels: enough warps to fill the GPU
// (about 48 per SM), at most 16 rows; `p->rows_per_thread` > 0 overrides.
template <typename T>
static int rows_per_thread(const opyx_rof_problem* p, const Geo<T>& g) {
  if (p->rows_per_thread > 0) return p->rows_per_thread;
  const int64_t warps_per_row = ((g.nl >> 2) + 31) / 32;
  const int64_t target = (int64_t)sm_count() * 48;
  int64_t R = g.rows * warps_per_row / (target > 0 ? target : 1);
  if (R < 1) R = 1;
  if (R > 16) R = 16;
  return (int)R;
}

template <typename T, int D, int C>
struct VecLaunch {
  static void run(const Geo<T>&, const Args<T>&, int, int, double, cudaStream_t) {}
};

template <int D, int C>
struct VecLaunch<float, D, C> {
  static void run(const Geo<float>& g, const Args<float>& a, int which, int R, double shift,
                  cudaStream_t s) {
    const int64_t Q = g.nl >> 2;
    const int64_t gx = (Q + kVecThreads - 1) / kVecThreads;
    int64_t gy = (g.rows + R - 1) / R;
    const int64_t cap = which == 3 ? kMaxBlocks : (int64_t)sm_count() * 256;
    int64_t cap_y = cap / gx;
    if (cap_y < 1) cap_y = 1;
    if (gy > cap_y) gy = cap_y;
    if (gy > 65535) gy = 65535;
    const dim3 grid((unsigned)gx, (unsigned)gy, 1), block(kVecThreads, 1, 1);
    if (which == 0) k_passA_v<D, C><<<grid, block, 0, s>>>(g, a, R);
    else if (which == 1) k_passB_v<D, C><<<grid, block, 0, s>>>(g, a, R);
    else k_gap_v<D, C><<<grid, block, 0, s>>>(g, a, R, shift);
  }
};

// Row-streaming kernels (rof_pipe.cuh): 2-D and 3-D FP32 problems whose
// arrays satisfy the vector requirements; flag bit 1 turns them off.
template <typename T>
static bool pipe_ok(const opyx_rof_problem* p, const opyx_rof_buffers* b) {
  return p->ndim >= 2 && !(p->flags & 2) && vec_ok<T>(p, b);
}

template <typename T, int D, int C>
struct PipeLaunch {
  static void run(const Geo<T>&, const Args<T>&, int, double, cudaStream_t) {}
};

template <typename K>
static int pipe_blocks_per_sm(K kernel, int smem, int threads = kPipeThreads) {
  int n = 0;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess)
    return 0;
  return n;
}

template <int D, int C>
struct PipeLaunch<float, D, C> {
  // Grid: ceil(nl / TW) tiles across x; enough row runs for one full wave
  // of resident CTAs.  Rows of at most 256 pixels use 256-pixel tiles (64
  // threads), so no CTA carries an idle half.
  template <int TW, typename K>
  static void go(K kernel, int smem, const Geo<float>& g, const Args<float>& a, bool reduce,
                 double shift, cudaStream_t s, int which) {
    static int per_sm[3] = {-1, -1, -1};
    if (per_sm[which] < 0) per_sm[which] = pipe_blocks_per_sm(kernel, smem, TW / 4);
    const int64_t gx = (g.nl + TW - 1) / TW;
    int64_t target = (int64_t)(per_sm[which] > 0 ? per_sm[which] : 1) * sm_count();
    if (reduce && target > kMaxBlocks) target = kMaxBlocks;
    int64_t gy = target / gx;
    if (gy < 1) gy = 1;
    if (gy > g.rows) gy = g.rows;
    const int RB = (int)((g.rows + gy - 1) / gy);
    gy = (g.rows + RB - 1) / RB;
    const dim3 grid((unsigned)gx, (unsigned)gy, 1);
    if (which == 0) k_passA_p<D, C, TW><<<grid, TW / 4, smem, s>>>(g, a, RB);
    else if (which == 1) k_passB_p<D, C, TW><<<grid, TW / 4, smem, s>>>(g, a, RB);
    else k_gap_p<D, C, TW><<<grid, TW / 4, smem, s>>>(g, a, RB, shift);
  }
  template <int TW>
  static void run_tw(const Geo<float>& g, const Args<float>& a, int which, double shift,
                     cudaStream_t s) {
    using S = PipeSmem<D, C, TW>;
    if (which == 0) go<TW>(k_passA_p<D, C, TW>, S::A, g, a, false, shift, s, 0);
    else if (which == 1) go<TW>(k_passB_p<D, C, TW>, S::B, g, a, false, shift, s, 1);
    else go<TW>(k_gap_p<D, C, TW>, S::G, g, a, true, shift, s, 2);
  }
  static void run(const Geo<float>& g, const Args<float>& a, int which, double shift,
                  cudaStream_t s) {
    if (g.nl <= 256) run_tw<256>(g, a, which, shift, s);
    else run_tw<kPipeTW>(g, a, which, shift, s);
  }
};

// Single-sweep iterations (rof_sweep.cuh, rof_sweep3.cuh): FP32 problems
// with constant or preconditioned steps whose caller gave the second dual
// buffer y2; 2-D any channel count, 3-D one channel, rows of 128, 256 or
// 512 pixels, no mask.
template <typename T, int D>
static bool sweep_ok(const opyx_rof_problem* p, const opyx_rof_buffers* b) {
  if (p->steps == OPYX_STEPS_ADAPTIVE || !b->y2 || (((uintptr_t)b->y2) & 15) || !pipe_ok<T>(p, b))
    return false;
  if (D == 2) return true;
  const int64_t nl = p->dims[2];
  return D == 3 && p->nchannels == 1 && !b->mask && (nl == 128 || nl == 256 || nl == 512);
}

template <typename T, int D, int C>
struct SweepLaunch {
  static void run(const Geo<T>&, const Args<T>&, cudaStream_t) {}
  static bool run_gap(const Geo<T>&, const Args<T>&, double, cudaStream_t) { return false; }
};

template <int C>
struct SweepLaunch<float, 2, C> {
  // GAP: the sweep that also computes the gap of its input state; false if
  // its grid would need more CTAs than the reduction has partials for.
  template <int TW, bool GAP>
  static bool go(const Geo<float>& g, const Args<float>& a, double shift, cudaStream_t s) {
    constexpr int P = sweep_p(C), DP = sweep_depth(C);
    constexpr int smem = SweepSmem<C, TW, DP>::bytes;
    static int per_sm = -1;
    if (per_sm < 0) per_sm = pipe_blocks_per_sm(k_sweep<C, TW, P, DP, GAP>, smem, TW / P);
    const int64_t gx = (g.nl + TW - 1) / TW;
    int64_t target = (int64_t)(per_sm > 0 ? per_sm : 1) * sm_count();
    if (GAP && target > kMaxBlocks) target = kMaxBlocks;
    int64_t gy = target / gx;
    if (gy < 1) gy = 1;
    if (gy > g.rows) gy = g.rows;
    const int RB = (int)((g.rows + gy - 1) / gy);
    gy = (g.rows + RB - 1) / RB;
    if (GAP && gx * gy > kMaxBlocks) return false;
    launch_chained(k_sweep<C, TW, P, DP, GAP>, dim3((unsigned)gx, (unsigned)gy, 1), dim3(TW / P),
                   smem, s, g, a, RB, shift);
    return true;
  }
  // narrow rows get narrow tiles, so that no CTA carries idle threads
  static void run(const Geo<float>& g, const Args<float>& a, cudaStream_t s) {
    if (g.nl <= 128) go<128, false>(g, a, 0.0, s);
    else if (g.nl <= 256) go<256, false>(g, a, 0.0, s);
    else go<kPipeTW, false>(g, a, 0.0, s);
  }
  static bool run_gap(const Geo<float>& g, const Args<float>& a, double shift, cudaStream_t s) {
    if (g.nl <= 128) return go<128, true>(g, a, shift, s);
    if (g.nl <= 256) return go<256, true>(g, a, shift, s);
    return go<kPipeTW, true>(g, a, shift, s);
  }
};

// 3-D sweep: TY = 3 rows per plane tile (measured on 256^3: TY = 1, 2, 3,
// 4, 8 gave 151, 121, 109, 127, 148 us -- three rows keep three CTAs per SM
// at 70 KB of shared memory); the planes are cut into ranges so that the
// work items fill whole waves of resident CTAs, traded against the halo
// plane each range recomputes.
constexpr int kSweep3TY = 3;

template <int C>
struct SweepLaunch<float, 3, C> {
  template <int TW>
  static void go(const Geo<float>& g, const Args<float>& a, cudaStream_t s) {
    constexpr int TY = kSweep3TY, P = 4;
    constexpr int threads = (TY + 1) * (TW / P);
    constexpr int smem = Sweep3Smem<TW, TY>::bytes;
    static int per_sm = -1;
    if (per_sm < 0) per_sm = pipe_blocks_per_sm(k_sweep3<TW, TY, P>, smem, threads);
    const int64_t R = (int64_t)(per_sm > 0 ? per_sm : 1) * sm_count();
    const int64_t Z = g.n[0];
    const int nyt = (int)((g.n[1] + TY - 1) / TY);
    int best_nc = 1;
    double best = 1e30;
    for (int64_t nc = 1; nc <= Z; ++nc) {
      const int64_t zc = (Z + nc - 1) / nc;
      if (nc > 1 && zc < 4) break;
      const double items = (double)nyt * (double)((Z + zc - 1) / zc);
      const double waves = items / (double)R;
      const double fill = waves >= 1.0 ? ceil(waves) / waves : 1.0 / waves;
      const double cost = fill * (1.0 + 1.0 / (double)zc);
      if (cost < best) { best = cost; best_nc = (int)nc; }
    }
    const int ZC = (int)((Z + best_nc - 1) / best_nc);
    const int64_t items = (int64_t)nyt * ((Z + ZC - 1) / ZC);
    const int64_t grid = items < R ? items : R;
    launch_chained(k_sweep3<TW, TY, P>, dim3((unsigned)grid), dim3(threads), smem, s, g, a, ZC, nyt);
  }
  static bool run_gap(const Geo<float>&, const Args<float>&, double, cudaStream_t) { return false; }
  static void run(const Geo<float>& g, const Args<float>& a, cudaStream_t s) {
    if (C != 1) return;
    if (g.nl == 128) go<128>(g, a, s);
    else if (g.nl == 256) go<256>(g, a, s);
    else go<512>(g, a, s);
  }
};

// Args of the second iteration of a pair: read (xbar, y2), write (x, y).
template <typename T>
static __host__ __device__ Args<T> swapped(const Args<T>& a) {
  Args<T> b = a;
  b.x = a.x2;
  b.x2 = a.x;
  b.y = a.y2;
  b.y2 = a.y;
  return b;
}

template <typename T, int D, int C>
struct Runner {
  static int init(const opyx_rof_problem* p, const opyx_rof_buffers* b, cudaStream_t s) {
    Geo<T> g = make_geo<T>(p);
    Args<T> a = make_args<T>(p, b);
    if (p->steps == OPYX_STEPS_ADAPTIVE) {
      dim3 grid, block;
      shape(g, &grid, &block, false);
      k_passR<T, D, C, 0><<<grid, block, 0, s>>>(g, a);
      return check_launch();
    }
    return OPYX_OK;
  }

  // which: 0 = pass A, 1 = pass B, 2 = pass R (adaptive), 3 = gap
  static void launch(const opyx_rof_problem* p, const Geo<T>& g, const Args<T>& a, int which,
                     bool use_vec, int R, cudaStream_t s, bool use_pipe = false) {
    const bool ad = p->steps == OPYX_STEPS_ADAPTIVE;
    if (use_pipe && (which == 3 || !ad) && D >= 2) {
      PipeLaunch<T, D, C>::run(g, a, which == 3 ? 2 : which, p->ssd_shift, s);
      return;
    }
    if (use_vec && (which == 3 || !ad)) {
      VecLaunch<T, D, C>::run(g, a, which, R, p->ssd_shift, s);
      return;
    }
    dim3 grid, block;
    shape(g, &grid, &block, ad || which == 3);
    if (which == 0) {
      if (ad) k_passA<T, D, C, 1><<<grid, block, 0, s>>>(g, a);
      else k_passA<T, D, C, 0><<<grid, block, 0, s>>>(g, a);
    } else if (which == 1) {
      if (ad) k_passB<T, D, C, 1><<<grid, block, 0, s>>>(g, a);
      else k_passB<T, D, C, 0><<<grid, block, 0, s>>>(g, a);
    } else if (which == 2) {
      k_passR<T, D, C, 1><<<grid, block, 0, s>>>(g, a);
    } else {
      k_gap<T, D, C><<<grid, block, 0, s>>>(g, a, p->ssd_shift);
    }
  }

  static int iterate(const opyx_rof_problem* p, const opyx_rof_buffers* b, int iters,
                     cudaStream_t s) {
    Geo<T> g = make_geo<T>(p);
    Args<T> a = make_args<T>(p, b);
    const bool v = vec_ok<T>(p, b), pp = pipe_ok<T>(p, b);
    const int R = rows_per_thread(p, g);
    int rest = iters;
    if (sweep_ok<T, D>(p, b)) {
      // pairs of sweeps return the state to (x, y); an odd count ends with
      // one two-pass iteration in place
      const Args<T> a2 = swapped(a);
      for (; rest >= 2; rest -= 2) {
        SweepLaunch<T, D, C>::run(g, a, s);
        SweepLaunch<T, D, C>::run(g, a2, s);
      }
    }
    for (int it = 0; it < rest; ++it) {
      launch(p, g, a, 0, v, R, s, pp);
      launch(p, g, a, 1, v, R, s, pp);
      if (p->steps == OPYX_STEPS_ADAPTIVE) launch(p, g, a, 2, v, R, s, pp);
    }
    return check_launch();
  }

  static int pass(const opyx_rof_problem* p, const opyx_rof_buffers* b, int which,
                  cudaStream_t s) {
    if (which < 0 || which > 3 || (which == 2 && p->steps != OPYX_STEPS_ADAPTIVE))
      return OPYX_ERR_ARG;
    if (which == 3 && !sweep_ok<T, D>(p, b)) return OPYX_ERR_UNSUPPORTED;
    Geo<T> g = make_geo<T>(p);
    Args<T> a = make_args<T>(p, b);
    if (which == 3) {
      SweepLaunch<T, D, C>::run(g, a, s);
      return check_launch();
    }
    launch(p, g, a, which, vec_ok<T>(p, b), rows_per_thread(p, g), s, pipe_ok<T>(p, b));
    return check_launch();
  }

  static int gap(const opyx_rof_problem* p, const opyx_rof_buffers* b, cudaStream_t s) {
    Geo<T> g = make_geo<T>(p);
    Args<T> a = make_args<T>(p, b);
    launch(p, g, a, 3, vec_ok<T>(p, b), rows_per_thread(p, g), s, pipe_ok<T>(p, b));
    return check_launch();
  }

  // The gap of the current state, then `iters` iterations.  With single
  // sweeps the first sweep computes the gap from the rows it reads (into
  // the second buffers, so a passing stop test leaves (x, y) as checked and
  // the remaining launches return at once); else opyx_rof_gap first.
  static int gap_iterate(const opyx_rof_problem* p, const opyx_rof_buffers* b, int iters,
                         cudaStream_t s) {
    if (iters >= 2 && sweep_ok<T, D>(p, b)) {
      Geo<T> g = make_geo<T>(p);
      Args<T> a = make_args<T>(p, b);
      if (SweepLaunch<T, D, C>::run_gap(g, a, p->ssd_shift, s)) {
        SweepLaunch<T, D, C>::run(g, swapped(a), s);
        int st = check_launch();
        if (st) return st;
        return iterate(p, b, iters - 2, s);
      }
    }
    int st = gap(p, b, s);
    if (st) return st;
    return iterate(p, b, iters, s);
  }
};

template <typename F>
static int dispatch(const opyx_rof_problem* p, F&& f) {
#define OPYX_ROF_CASE(TT, DD, CC)                                            \
  if (p->ndim == DD && p->nchannels == CC) return f(Runner<TT, DD, CC>());
#define OPYX_ROF_CASES(TT)                                                   \
  OPYX_ROF_CASE(TT, 1, 1) OPYX_ROF_CASE(TT, 1, 2) OPYX_ROF_CASE(TT, 1, 3) OPYX_ROF_CASE(TT, 1, 4) \
  OPYX_ROF_CASE(TT, 2, 1) OPYX_ROF_CASE(TT, 2, 2) OPYX_ROF_CASE(TT, 2, 3) OPYX_ROF_CASE(TT, 2, 4) \
  OPYX_ROF_CASE(TT, 3, 1) OPYX_ROF_CASE(TT, 3, 2) OPYX_ROF_CASE(TT, 3, 3) OPYX_ROF_CASE(TT, 3, 4)
  if (p->dtype == OPYX_F32) { OPYX_ROF_CASES(float) }
  else { OPYX_ROF_CASES(double) }
#undef OPYX_ROF_CASES
#undef OPYX_ROF_CASE
  return OPYX_ERR_UNSUPPORTED;
}

__global__ void k_write_state(opyx_adaptive_state* dst, opyx_adaptive_state v) { *dst = v; }

// Device state record written at init.
static void host_state(const opyx_rof_problem* p, opyx_adaptive_state* st) {
  memset(st, 0, sizeof(*st));
  st->tau = p->tau;
  st->sigma = p->sigma;
  st->alpha = p->alpha0;
  st->eta = p->eta;
  st->Delta = p->Delta;
  st->theta = p->theta;
  for (int j = 0; j < 4; ++j) st->eps[j] = p->eps[j];
  int64_t N = 1;
  for (int t = 0; t < p->ndim; ++t) N *= p->dims[t];
  st->xsize = (double)(N * p->nchannels);
  st->ysize = (double)(N * p->nchannels * p->ndim);
}

}  // namespace rof
}  // namespace opyx

using namespace opyx;
using namespace opyx::rof;

extern "C" {

size_t opyx_rof_workspace_size(void) { return kWsBytes; }
size_t opyx_rof_info_offset(void) { return kInfoOff; }

int opyx_rof_init(const opyx_rof_problem* p, const opyx_rof_buffers* b, void* stream) {
  int st = validate(p, b);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  // The state record is passed by value through a kernel argument so that
  // init stays capturable and needs no pinned staging buffer.
  opyx_adaptive_state hs;
  host_state(p, &hs);
  if (cudaMemsetAsync((char*)b->ws + kInfoOff, 0, 256, s) != cudaSuccess) return OPYX_ERR_LAUNCH;
  if (cudaMemsetAsync((char*)b->ws + kTicketOff, 0, 256, s) != cudaSuccess) return OPYX_ERR_LAUNCH;
  k_write_state<<<1, 1, 0, s>>>((opyx_adaptive_state*)((char*)b->ws + kStateOff), hs);
  st = check_launch();
  if (st) return st;
  return dispatch(p, [&](auto r) { return decltype(r)::init(p, b, s); });
}

int opyx_rof_uses_sweep(const opyx_rof_problem* p, const opyx_rof_buffers* b) {
  if (!p || !b || validate(p, b)) return 0;
  if (p->dtype != OPYX_F32) return 0;
  if (p->ndim == 2) return sweep_ok<float, 2>(p, b) ? 1 : 0;
  if (p->ndim == 3) return sweep_ok<float, 3>(p, b) ? 1 : 0;
  return 0;
}

int opyx_rof_iterate(const opyx_rof_problem* p, const opyx_rof_buffers* b, int iters,
                     void* stream) {
  int st = validate(p, b);
  if (st) return st;
  if (iters < 0) return OPYX_ERR_ARG;
  if (iters == 0) return OPYX_OK;
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch(p, [&](auto r) { return decltype(r)::iterate(p, b, iters, s); });
}

int opyx_rof_pass(const opyx_rof_problem* p, const opyx_rof_buffers* b, int which,
                  void* stream) {
  int st = validate(p, b);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch(p, [&](auto r) { return decltype(r)::pass(p, b, which, s); });
}

int opyx_rof_gap(const opyx_rof_problem* p, const opyx_rof_buffers* b, void* stream) {
  int st = validate(p, b);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch(p, [&](auto r) { return decltype(r)::gap(p, b, s); });
}

int opyx_rof_gap_iterate(const opyx_rof_problem* p, const opyx_rof_buffers* b, int iters,
                         void* stream) {
  int st = validate(p, b);
  if (st) return st;
  if (iters < 0) return OPYX_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  return dispatch(p, [&](auto r) { return decltype(r)::gap_iterate(p, b, iters, s); });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free entry point.
//
// Some callers of this path cannot allocate device memory themselves: code
// that runs inside another framework's memory pool or a host process that
// is only handed device pointers for the image and the iterates.  For them
// the scratch of the fused iteration -- the step/info/reduction workspace,
// the extrapolated primal xbar and, for adaptive steps, A^T y and the
// residual part -- lives in one file-scope __device__ array of
// OPYX_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library holds
// until the process exits.
// ---------------------------------------------------------------------------

static __device__ __align__(256) unsigned char g_noalloc_scratch[OPYX_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch for the current device, looked up once
// per device with that device current (host code may not use the symbol's
// name as an address).
static int noalloc_scratch(char** out) {
  static std::mutex mu;
  static char* addr[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return OPYX_ERR_LAUNCH;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr)
      return OPYX_ERR_LAUNCH;
    addr[dev] = (char*)ptr;
  }
  *out = addr[dev];
  return OPYX_OK;
}

static size_t round256(size_t n) { return (n + 255) & ~(size_t)255; }

extern "C" int opyx_rof_iterate_noalloc(const opyx_rof_problem* p, void* x, void* y,
                                        const void* f, const uint8_t* mask, int iters,
                                        double* gap_out, void* stream) {
  if (!p || iters < 0) return OPYX_ERR_ARG;
  if (p->ndim < 1 || p->ndim > 3 || p->nchannels < 1 || p->nchannels > OPYX_ROF_MAX_C)
    return OPYX_ERR_UNSUPPORTED;
  for (int t = 0; t < p->ndim; ++t)
    if (p->dims[t] < 1) return OPYX_ERR_ARG;
  int64_t N = 0;
  if (!count_pixels(p, &N)) return OPYX_ERR_SCRATCH_LIMIT;
  const size_t esz = p->dtype == OPYX_F64 ? 8 : 4;
  const size_t field = round256((size_t)N * p->nchannels * esz);
  const int nfields = p->steps == OPYX_STEPS_ADAPTIVE ? 3 : 1;   // xbar [, xgrad, gp]
  if (N > (int64_t)(OPYX_NOALLOC_SCRATCH_BYTES / 4) ||
      round256(kWsBytes) + nfields * field > (size_t)OPYX_NOALLOC_SCRATCH_BYTES)
    return OPYX_ERR_SCRATCH_LIMIT;
  char* base = nullptr;
  int st = noalloc_scratch(&base);
  if (st) return st;
  opyx_rof_buffers b;
  b.x = x;
  b.y = y;
  b.f = f;
  b.mask = mask;
  b.ws = base;
  b.xbar = base + round256(kWsBytes);
  b.xgrad = nfields > 1 ? base + round256(kWsBytes) + field : nullptr;
  b.gp = nfields > 1 ? base + round256(kWsBytes) + 2 * field : nullptr;
  b.y2 = nullptr;
  // opyx_rof_init clears the info record and the reduction ticket, which the
  // previous call left behind, and rewrites the step state.
  st = opyx_rof_init(p, &b, stream);
  if (st) return st;
  st = opyx_rof_iterate(p, &b, iters, stream);
  if (st) return st;
  if (gap_out) {
    st = opyx_rof_gap(p, &b, stream);
    if (st) return st;
    if (cudaMemcpyAsync(gap_out, base + kInfoOff, 6 * sizeof(double), cudaMemcpyDeviceToDevice,
                        (cudaStream_t)stream) != cudaSuccess)
      return OPYX_ERR_LAUNCH;
  }
  return OPYX_OK;
}

// ---------------------------------------------------------------------------
// Batched solves: many independent 2-D FP32 problems with constant or
// preconditioned steps, one launch per iteration for all of them.
//
// The host fills a descriptor (opyx_rof_batch_describe): per instance its
// geometry/coefficients, buffer pointers and step state; a list of work
// items (instance, row run, 512-pixel column tile) over the active
// instances.  The sweep kernel walks the items (grid-stride) with the body of
// the single-instance sweep; small instances then cost a few CTAs instead of
// a launch each.  Gaps: per-item FP64 partial sums, folded per instance in
// item order (deterministic) into the instance's info record with the stop
// test.  Per-instance step state and info records are 512-byte records in
// one caller array.
// ---------------------------------------------------------------------------
namespace opyx {
namespace rof {

constexpr size_t kBatchRecord = 512;   // [0, 256) step state, [256, 512) info

// Work items come in three tile-width classes (128, 256, 512 pixels; see
// batch_tiles for the choice per image), so narrow images do not leave most
// of a 512-pixel CTA idle; the sweep launches once per class.
constexpr int kBatchClasses = 3;
constexpr int kStripW = 128;   // pixels per work item of the persistent solve (one warp)
constexpr int kBatchTW[kBatchClasses] = {128, 256, 512};

// Column tiles of an instance with rows of nl pixels: n tiles of equal width
// tw (a multiple of 4, the last one possibly narrower) in the width class
// whose CTAs leave the fewest lanes idle, n * TW_class pixel slots per row
// (ties to the wider class).  On the 512-instance mixed-size batch this
// fills 0.92 of the lanes against 0.76 for tiles of the class width (4.10 s
// against 5.10 s to solve it).
static int batch_tiles(int64_t nl, int64_t* tw) {
  int best = kBatchClasses - 1;
  int64_t best_cost = INT64_MAX;
  for (int c = kBatchClasses - 1; c >= 0; --c) {
    const int64_t n = (nl + kBatchTW[c] - 1) / kBatchTW[c];
    const int64_t cost = n * kBatchTW[c];
    if (cost < best_cost) { best_cost = cost; best = c; }
  }
  const int64_t n = (nl + kBatchTW[best] - 1) / kBatchTW[best];
  *tw = ((nl + n - 1) / n + 3) / 4 * 4;
  return best;
}

struct BatchHeader {
  int32_t ninst, nitems, nchannels, rows_per_item;
  int32_t class_beg[kBatchClasses + 1];   // items of class c: [class_beg[c], class_beg[c+1])
  int32_t witems, pad;                    // strips of the persistent solve (all instances)
};

struct BatchInst {
  Geo<float> g;
  Args<float> a;
  opyx_adaptive_state st0;
  double ssd_shift;
  int32_t item_beg, item_end;
  // the persistent solve's work items: strips of 128 pixels by runs of
  // rows_per_item rows, w_ntx across and w_nty down, numbered from w_beg
  int32_t w_beg, w_ntx, w_nty, w_pad;
};

struct BatchItem {
  int32_t inst, r0, r1, q_beg, q_end;
};

static size_t batch_inst_off() { return (sizeof(BatchHeader) + 255) & ~(size_t)255; }
static size_t batch_item_off(int ninst) {
  return (batch_inst_off() + (size_t)ninst * sizeof(BatchInst) + 255) & ~(size_t)255;
}

// Cooperative copy of an instance's geometry and arguments into shared memory.
OPYX_D void load_inst(const BatchInst* src, BatchInst* dst) {
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  constexpr int nw = (int)(sizeof(BatchInst) / 4);
  for (int i = threadIdx.x; i < nw; i += blockDim.x) d[i] = s[i];
}

template <int C, int TW, int P = sweep_p(C), int DP = sweep_depth(C)>
__global__ void __launch_bounds__(TW / P, sweep_min_blocks(TW, P))
k_sweep_batch(const BatchInst* __restrict__ insts, const BatchItem* __restrict__ items,
              int nitems, int flip) {
  extern __shared__ float4 smem4[];
  __shared__ __align__(8) uint64_t mbar[kSweepMaxBars];
  __shared__ __align__(16) BatchInst cur;
  float* sm = reinterpret_cast<float*>(smem4);
  const bool lead = threadIdx.x == 0;
  if (lead) {
    for (int i = 0; i < kSweepMaxBars; ++i) mbar_init(&mbar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  unsigned st = 0;
  int loaded = -1;
  // a contiguous share of the item list per CTA; runs of vertically adjacent
  // items of one tile column are swept as one range of rows (one prologue,
  // no halo row between them)
  const int64_t lo = (int64_t)nitems * blockIdx.x / gridDim.x;
  const int64_t hi = (int64_t)nitems * (blockIdx.x + 1) / gridDim.x;
  for (int64_t it = lo; it < hi;) {
    const BatchItem item = items[it];
    int32_t r1 = item.r1;
    for (++it; it < hi; ++it) {
      const BatchItem nx = items[it];
      if (nx.inst != item.inst || nx.q_beg != item.q_beg || nx.r0 != r1) break;
      r1 = nx.r1;
    }
    if (item.inst != loaded) {
      __syncthreads();   // nobody still reads the previous instance
      load_inst(&insts[item.inst], &cur);
      __syncthreads();
      loaded = item.inst;
    }
    if (cur.a.info->done != 0.0) continue;   // uniform: read by every thread alike
    const Args<float> a = flip ? swapped(cur.a) : cur.a;
    if (!sweep_rows<C, TW, P, DP>(cur.g, a, item.q_beg, item.q_end, item.r0, r1, mbar, st, sm))
      return;
  }
  if (lead) bulk_wait_all();
}

// Per-item partial sums of the gap (as k_gap_p): {G, |Ax|, G*, |y|^2,
// max(|y| - lbd)}.  A thread owns one quad (4 pixels along the row) of a run
// of consecutive rows of the item, carries x of the next row and y of the
// current row into the following row, and accumulates in FP32 over its
// pixels; FP64 across the block.
template <int C>
__global__ void __launch_bounds__(256)
k_gap_batch(const BatchInst* __restrict__ insts, const BatchItem* __restrict__ items,
            int nitems, double* partials) {
  constexpr int D = 2, M = D * C;
  __shared__ __align__(16) BatchInst cur;
  __shared__ double red[5][8];
  int loaded = -1;
  // a contiguous share of the items per CTA: consecutive items mostly belong
  // to one instance, whose coefficients are then loaded once
  const int64_t lo = (int64_t)nitems * blockIdx.x / gridDim.x;
  const int64_t hi = (int64_t)nitems * (blockIdx.x + 1) / gridDim.x;
  for (int64_t it = lo; it < hi; ++it) {
    const BatchItem item = items[it];
    if (item.inst != loaded) {
      __syncthreads();
      load_inst(&insts[item.inst], &cur);
      __syncthreads();
      loaded = item.inst;
    }
    const Geo<float>& g = cur.g;
    const Args<float>& a = cur.a;
    float pG = 0.f, pF = 0.f, pGs = 0.f, pFs = 0.f, pinf = -INFINITY;
    const int nq = (int)((item.q_end - item.q_beg) >> 2);     // quads per row, <= 128
    const int rstep = (int)blockDim.x / nq;                     // row runs per block
    const int tq = (int)threadIdx.x % nq, tr = (int)threadIdx.x / nq;
    const int nr = item.r1 - item.r0;
    const int rpt = (nr + rstep - 1) / rstep;
    const int64_t rb = item.r0 + (int64_t)tr * rpt;
    const int64_t re = rb + rpt < item.r1 ? rb + rpt : item.r1;
    if (a.info->done == 0.0 && tr < rstep && rb < re) {
      const int64_t q0 = item.q_beg + 4 * tq;
      const int64_t nl = g.nl, nrow = g.n[0];
      const bool has_r = q0 + 4 < nl, has_l = q0 > 0;
      float qx[4 * C], qn[4 * C], qf[4 * C], qy[4 * M], qu[4 * M], xr[C], yl[C];
      ldv(qx, a.x + (rb * nl + q0) * C);
      if (rb > 0) ldv(qu, a.y + ((rb - 1) * nl + q0) * M);
      else zero(qu);
      for (int64_t r = rb; r < re; ++r) {
        const int64_t i0 = r * nl + q0;
        const bool has_up = r > 0, has_dn = r < nrow - 1;
        if (has_dn) ldv(qn, a.x + (i0 + nl) * C);
        else zero(qn);
        ldv(qy, a.y + i0 * M);
        ldv(qf, a.f + i0 * C);
#pragma unroll
        for (int k2 = 0; k2 < C; ++k2) {
          xr[k2] = has_r ? a.x[(i0 + 4) * C + k2] : 0.f;
          yl[k2] = has_l ? a.y[(i0 - 1) * M + (D - 1) * C + k2] : 0.f;
        }
        unsigned mk = 0xffffffffu;
        if (a.mask) mk = *reinterpret_cast<const unsigned*>(a.mask + i0);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          const int64_t q = q0 + p;
          const bool on = (mk >> (8 * p)) & 0xffu;
          const bool inx = q < nl - 1;
          float n2 = 0.f, y2 = 0.f;
#pragma unroll
          for (int k2 = 0; k2 < C; ++k2) {
            const float xk = qx[p * C + k2], fk = qf[p * C + k2];
            float s = 0.f;
            const float ihl = g.invh[D - 1], ihr = g.invh[D - 2];
            if (inx) s -= qy[p * M + (D - 1) * C + k2] * ihl;
            if (q > 0) s += (p > 0 ? qy[(p - 1) * M + (D - 1) * C + k2] : yl[k2]) * ihl;
            if (has_dn) s -= qy[p * M + (D - 2) * C + k2] * ihr;
            if (has_up) s += qu[p * M + (D - 2) * C + k2] * ihr;
            const float ak = g.w[k2] * s;
            if (on) {
              const float d = xk - fk;
              pG += g.vol[k2] * d * d;
              pGs += ak * ak * g.half_rvol[k2] - fk * ak;
            }
            const float nb = p < 3 ? qx[(p + 1) * C + k2] : xr[k2];
            const float gl = inx ? g.coef[D - 1][k2] * (nb - xk) : 0.f;
            const float gr = has_dn ? g.coef[D - 2][k2] * (qn[p * C + k2] - xk) : 0.f;
            n2 += gl * gl + gr * gr;
          }
#pragma unroll
          for (int j = 0; j < M; ++j) y2 += qy[p * M + j] * qy[p * M + j];
          const float nrm = sqrtf(n2);
          pF += g.use_huber ? (nrm <= g.huber ? n2 * g.half_rhuber : nrm - g.half_huber) : nrm;
          pFs += y2;
          pinf = fmaxf(pinf, sqrtf(y2) - g.lbd);
        }
#pragma unroll
        for (int j = 0; j < 4 * C; ++j) qx[j] = qn[j];
#pragma unroll
        for (int j = 0; j < 4 * M; ++j) qu[j] = qy[j];
      }
    }
    double v[5] = {0.5 * (double)pG, (double)pF, (double)pGs, (double)pFs, (double)pinf};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      double r = warp_reduce(k == 4 ? RED_MAX : RED_SUM, v[k]);
      if (lane == 0) red[k][warp] = r;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
      const int k = threadIdx.x;
      double r = k == 4 ? -INFINITY : 0.0;
      for (int w2 = 0; w2 < (int)(blockDim.x >> 5); ++w2)
        r = k == 4 ? fmax(r, red[k][w2]) : r + red[k][w2];
      partials[(size_t)it * 5 + k] = r;
    }
    __syncthreads();
  }
}

// Per instance (one CTA each): fold its items' partials -- thread t takes
// items t, t + 128, ..., then a fixed-order block reduction, so the result
// does not depend on timing -- and write its info record (objectives, gap,
// stop test) as the single-instance gap kernels do.
__global__ void __launch_bounds__(128)
k_gap_fold(const BatchInst* __restrict__ insts, int ninst, const double* __restrict__ partials) {
  const int i = blockIdx.x;
  if (i >= ninst) return;
  const BatchInst& b = insts[i];
  if (b.item_end <= b.item_beg || b.a.info->done != 0.0) return;   // uniform per CTA
  double tot[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int it = b.item_beg + (int)threadIdx.x; it < b.item_end; it += blockDim.x)
    for (int k = 0; k < 5; ++k)
      tot[k] = k == 4 ? fmax(tot[k], partials[(size_t)it * 5 + k]) : tot[k] + partials[(size_t)it * 5 + k];
  __shared__ double red[5][4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const double r = warp_reduce(k == 4 ? RED_MAX : RED_SUM, tot[k]);
    if (lane == 0) red[k][warp] = r;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[5];
    for (int k = 0; k < 5; ++k) {
      t[k] = red[k][0];
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
        t[k] = k == 4 ? fmax(t[k], red[k][w]) : t[k] + red[k][w];
    }
    write_info(b.g, b.a, t, b.ssd_shift);
  }
}

__global__ void k_batch_init(const BatchInst* __restrict__ insts, int ninst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ninst) return;
  *insts[i].a.st = insts[i].st0;
  opyx_rof_info* info = insts[i].a.info;
  memset(info, 0, sizeof(opyx_rof_info));
}

// ---------------------------------------------------------------------------
// Persistent batched solve (one channel): one cooperative launch runs every
// iteration, gap check and retirement of the batch.  Each iteration, the
// warps take work items -- strips of 128 pixels by runs of rows of the
// active instances -- from a counter and sweep them (sweep_strip1); a grid
// barrier ends the iteration.  Every `gran` iterations the warps write each
// strip's partial gap sums, the CTAs fold each active instance's sums into
// its info record with the reference's stop test (pdhg.py:287-305), and CTA
// 0 rebuilds the list of active instances.  Waits are bounded: a barrier
// that does not fill within kPersistSpin polls sets the error word and every
// CTA returns.
// ---------------------------------------------------------------------------
constexpr int kPersistThreads = 256;
constexpr int kPersistSpin = 1 << 25;   // polls of 64 ns and more per barrier: > 2 s

// The control record (opyx_rof_persist_ctl): barrier arrivals (monotone),
// work counters of the grabbing phases (mod 4), the error word, the active
// instances and their strips, the iterations at the last check.
using PersistCtl = opyx_rof_persist_ctl;
static_assert(sizeof(opyx_rof_persist_ctl) == 48, "control record layout");

// Workspace: the control record, then act_inst (ninst), act_off and
// act_goff (ninst + 1 each: sweep-item and gap-strip offsets of the active
// instances), then the strips' gap partials.
static size_t persist_align(size_t n) { return (n + 255) & ~(size_t)255; }
static size_t persist_act_off(int ninst) { return 256 + persist_align(4 * (size_t)ninst); }
static size_t persist_act_goff(int ninst) {
  return persist_act_off(ninst) + persist_align(4 * ((size_t)ninst + 1));
}
static size_t persist_part_off(int ninst) {
  return persist_act_goff(ninst) + persist_align(4 * ((size_t)ninst + 1));
}

OPYX_D unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Bounded grid barrier: returns false (every thread of the CTA alike) if it
// timed out or another CTA reported an error.
OPYX_D bool grid_sync(PersistCtl* ctl, unsigned long long& nbar) {
  __shared__ int ok_s;
  __syncthreads();
  ++nbar;
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd((unsigned long long*)&ctl->arrive, 1ull);
    const unsigned long long target = nbar * gridDim.x;
    int ok = 1;
    for (int i = 0;; ++i) {
      if (ld_acquire_u64((const unsigned long long*)&ctl->arrive) >= target) break;
      if (*(volatile int*)&ctl->error || i >= kPersistSpin) {
        atomicExch(&ctl->error, 1);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// The next work item of a grabbing phase for this warp (the same for all its
// lanes), or -1 when the phase's nwork items are taken.
OPYX_D int grab_item(PersistCtl* ctl, unsigned ph, int nwork) {
  int w = 0;
  if ((threadIdx.x & 31) == 0) w = (int)atomicAdd((unsigned*)&ctl->grab[ph & 3u], 1u);
  w = __shfl_sync(0xffffffffu, w, 0);
  return w < nwork ? w : -1;
}

// Active instance j holding work item w (act_off ascending, binary search).
OPYX_D int item_owner(const int* act_off, int nact, int w) {
  int lo = 0, hi = nact - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldcg(act_off + mid) <= w) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Partial gap sums of one strip (rows [r0, r1), 128 pixels from q_beg) by
// one warp, with the per-pixel terms of k_gap_batch: {G, |Ax|, G*, |y|^2,
// max(|y| - lbd)}; each lane sums its quad of a row in FP32 and adds that
// into FP64 (the objectives are large sums whose difference is the gap),
// FP64 across the warp in a fixed order.
OPYX_D void gap_strip1(const Geo<float>& g, const Args<float>& a, int64_t q_beg, int64_t r0,
                       int64_t r1, double* out) {
  const int lane = threadIdx.x & 31;
  const int64_t q0 = q_beg + 4 * lane;
  const bool act = q0 < g.nl;
  const int64_t nl = g.nl, nrow = g.n[0];
  const bool has_r = q0 + 4 < nl, has_l = q0 > 0;
  double sG = 0.0, sF = 0.0, sGs = 0.0, sFs = 0.0;
  float pinf = -INFINITY;
  if (act) {
    float qx[4], qn[4], qf[4], qy[8], qu[8], xr = 0.f, yl = 0.f;
    auto ld4 = [](float* d, const float* s) {
      const float4 v = __ldcg(reinterpret_cast<const float4*>(s));
      d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
    };
    ld4(qx, a.x + r0 * nl + q0);
    if (r0 > 0) { ld4(qu, a.y + ((r0 - 1) * nl + q0) * 2); ld4(qu + 4, a.y + ((r0 - 1) * nl + q0) * 2 + 4); }
    else { for (int j = 0; j < 8; ++j) qu[j] = 0.f; }
    for (int64_t r = r0; r < r1; ++r) {
      const int64_t i0 = r * nl + q0;
      const bool has_up = r > 0, has_dn = r < nrow - 1;
      if (has_dn) ld4(qn, a.x + i0 + nl);
      else { for (int j = 0; j < 4; ++j) qn[j] = 0.f; }
      ld4(qy, a.y + i0 * 2);
      ld4(qy + 4, a.y + i0 * 2 + 4);
      {
        const float4 v = __ldg(reinterpret_cast<const float4*>(a.f + i0));
        qf[0] = v.x; qf[1] = v.y; qf[2] = v.z; qf[3] = v.w;
      }
      xr = has_r ? __ldcg(a.x + i0 + 4) : 0.f;
      yl = has_l ? __ldcg(a.y + (i0 - 1) * 2 + 1) : 0.f;
      unsigned mk = 0xffffffffu;
      if (a.mask) mk = __ldg(reinterpret_cast<const unsigned*>(a.mask + i0));
      float pG = 0.f, pF = 0.f, pGs = 0.f, pFs = 0.f;
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int64_t q = q0 + p;
        const bool on = (mk >> (8 * p)) & 0xffu;
        const bool inx = q < nl - 1;
        float n2 = 0.f, y2 = 0.f;
        const float xk = qx[p], fk = qf[p];
        float s = 0.f;
        const float ihl = g.invh[1], ihr = g.invh[0];
        if (inx) s -= qy[p * 2 + 1] * ihl;
        if (q > 0) s += (p > 0 ? qy[(p - 1) * 2 + 1] : yl) * ihl;
        if (has_dn) s -= qy[p * 2] * ihr;
        if (has_up) s += qu[p * 2] * ihr;
        const float ak = g.w[0] * s;
        if (on) {
          const float d = xk - fk;
          pG += g.vol[0] * d * d;
          pGs += ak * ak * g.half_rvol[0] - fk * ak;
        }
        const float nb = p < 3 ? qx[p + 1] : xr;
        const float gl = inx ? g.coef[1][0] * (nb - xk) : 0.f;
        const float gr = has_dn ? g.coef[0][0] * (qn[p] - xk) : 0.f;
        n2 += gl * gl + gr * gr;
        y2 += qy[p * 2] * qy[p * 2];
        y2 += qy[p * 2 + 1] * qy[p * 2 + 1];
        const float nrm = sqrtf(n2);
        pF += g.use_huber ? (nrm <= g.huber ? n2 * g.half_rhuber : nrm - g.half_huber) : nrm;
        pFs += y2;
        pinf = fmaxf(pinf, sqrtf(y2) - g.lbd);
      }
      sG += 0.5 * (double)pG;
      sF += (double)pF;
      sGs += (double)pGs;
      sFs += (double)pFs;
#pragma unroll
      for (int j = 0; j < 4; ++j) qx[j] = qn[j];
#pragma unroll
      for (int j = 0; j < 8; ++j) qu[j] = qy[j];
    }
  }
  double v[5] = {sG, sF, sGs, sFs, (double)pinf};
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const double r = warp_reduce(k == 4 ? RED_MAX : RED_SUM, v[k]);
    if (lane == 0) out[k] = r;
  }
}

// CTA-wide fold of instance b's strip partials (fixed order) and its info
// record with the stop test.
OPYX_D void fold_inst(const BatchInst& b, const double* partials) {
  __shared__ double red[5][kPersistThreads / 32];
  const int n = b.w_ntx * b.w_nty;
  double tot[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int it = (int)threadIdx.x; it < n; it += blockDim.x)
    for (int k = 0; k < 5; ++k) {
      const double v = __ldcg(partials + (size_t)(b.w_beg + it) * 5 + k);
      tot[k] = k == 4 ? fmax(tot[k], v) : tot[k] + v;
    }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const double r = warp_reduce(k == 4 ? RED_MAX : RED_SUM, tot[k]);
    if (lane == 0) red[k][warp] = r;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t[5];
    for (int k = 0; k < 5; ++k) {
      t[k] = red[k][0];
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
        t[k] = k == 4 ? fmax(t[k], red[k][w]) : t[k] + red[k][w];
    }
    write_info(b.g, b.a, t, b.ssd_shift);
  }
  __syncthreads();
}

// CTA 0, thread 0: the instances whose info record is not done, the rows
// of the sweep items (R halved, down to 2, until there are at least
// kPersistItemsPerWarp items per warp), their sweep-item and gap-strip
// offsets, and the counts.
#ifndef OPYX_PERSIST_ITEMS_PER_WARP
#define OPYX_PERSIST_ITEMS_PER_WARP 4
#endif
constexpr int kPersistItemsPerWarp = OPYX_PERSIST_ITEMS_PER_WARP;

OPYX_D void rebuild_active(const BatchInst* insts, int ninst, int R, PersistCtl* ctl, int* act_inst,
                           int* act_off, int* act_goff, int iters) {
  if (threadIdx.x != 0) return;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  int n = 0, goff = 0;
  for (int i = 0; i < ninst; ++i) {
    if (*(volatile double*)&insts[i].a.info->done != 0.0) continue;
    act_inst[n] = i;
    act_goff[n] = goff;
    goff += insts[i].w_ntx * insts[i].w_nty;
    ++n;
  }
  act_goff[n] = goff;
  int re = R;
  for (;;) {
    int64_t items = 0;
    for (int j = 0; j < n; ++j) {
      const BatchInst& b = insts[act_inst[j]];
      items += (int64_t)b.w_ntx * ((b.g.rows + re - 1) / re);
    }
    if (re <= 2 || items >= kPersistItemsPerWarp * warps) break;
    re = (re + 1) / 2;
  }
  int off = 0;
  for (int j = 0; j < n; ++j) {
    const BatchInst& b = insts[act_inst[j]];
    act_off[j] = off;
    off += b.w_ntx * (int)((b.g.rows + re - 1) / re);
  }
  act_off[n] = off;
  ctl->nact = n;
  ctl->nwork = off;
  ctl->nwork_gap = goff;
  ctl->rows = re;
  ctl->iters = iters;
}

template <bool PRE, bool MASK>
__global__ void __launch_bounds__(kPersistThreads, 2)
k_batch_persist(const BatchInst* __restrict__ insts, int ninst, int R, PersistCtl* ctl,
                int* act_inst, int* act_off, int* act_goff, double* partials, int gran,
                int maxiter) {
  unsigned long long nbar = 0;
  unsigned ph = 0;
  if (blockIdx.x == 0) rebuild_active(insts, ninst, R, ctl, act_inst, act_off, act_goff, 0);
  if (!grid_sync(ctl, nbar)) return;
  for (int k = 0; k < maxiter; ++k) {
    const int nwork = __ldcg(&ctl->nwork), nact = __ldcg(&ctl->nact);
    const int re = __ldcg(&ctl->rows);
    if (nwork == 0) break;
    // ---- iteration k of every active instance
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->grab[(ph + 2) & 3u] = 0u;
    for (int w = grab_item(ctl, ph, nwork); w >= 0; w = grab_item(ctl, ph, nwork)) {
      const int j = item_owner(act_off, nact, w);
      const BatchInst& b = insts[__ldcg(act_inst + j)];
      const int loc = w - __ldcg(act_off + j);
      const int tx = loc % b.w_ntx, ty = loc / b.w_ntx;
      const int64_t r0 = (int64_t)ty * re;
      const int64_t r1 = r0 + re < b.g.rows ? r0 + re : b.g.rows;
      const Args<float> a = (k & 1) ? swapped(b.a) : b.a;
      sweep_strip1<PRE, MASK>(b.g, a, (int64_t)tx * kStripW, r0, r1);
    }
    ++ph;
    if (!grid_sync(ctl, nbar)) return;
    if ((k + 1) % gran != 0) continue;
    // ---- gap check after iteration k (an even count: the iterate is in x, y)
    const int ngap = __ldcg(&ctl->nwork_gap);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->grab[(ph + 2) & 3u] = 0u;
    for (int w = grab_item(ctl, ph, ngap); w >= 0; w = grab_item(ctl, ph, ngap)) {
      const int j = item_owner(act_goff, nact, w);
      const BatchInst& b = insts[__ldcg(act_inst + j)];
      const int loc = w - __ldcg(act_goff + j);
      const int tx = loc % b.w_ntx, ty = loc / b.w_ntx;
      const int64_t r0 = (int64_t)ty * R;
      const int64_t r1 = r0 + R < b.g.rows ? r0 + R : b.g.rows;
      gap_strip1(b.g, b.a, (int64_t)tx * kStripW, r0, r1, partials + (size_t)(b.w_beg + loc) * 5);
    }
    ++ph;
    if (!grid_sync(ctl, nbar)) return;
    for (int j = blockIdx.x; j < nact; j += gridDim.x) fold_inst(insts[__ldcg(act_inst + j)], partials);
    if (!grid_sync(ctl, nbar)) return;
    if (blockIdx.x == 0) rebuild_active(insts, ninst, R, ctl, act_inst, act_off, act_goff, k + 1);
    if (!grid_sync(ctl, nbar)) return;
  }
}

static int batch_check(const opyx_rof_problem* p, const opyx_rof_buffers* b) {
  int st = validate(p, b);
  if (st) return st;
  if (p->dtype != OPYX_F32 || p->ndim != 2 || p->steps == OPYX_STEPS_ADAPTIVE)
    return OPYX_ERR_UNSUPPORTED;
  if (!b->y2 || (((uintptr_t)b->y2) & 15) || !pipe_ok<float>(p, b)) return OPYX_ERR_ARG;
  if (p->dims[0] > INT32_MAX || p->dims[1] > INT32_MAX) return OPYX_ERR_UNSUPPORTED;
  return OPYX_OK;
}

template <int C, int TW>
static int batch_launch_sweep(const BatchInst* insts, const BatchItem* items, int nitems,
                              int flip, cudaStream_t s) {
  constexpr int P = sweep_p(C), DP = sweep_depth(C);
  constexpr int smem = SweepSmem<C, TW, DP>::bytes;
  static int per_sm = -1;
  if (per_sm < 0) per_sm = pipe_blocks_per_sm(k_sweep_batch<C, TW, P, DP>, smem, TW / P);
  int64_t grid = (int64_t)(per_sm > 0 ? per_sm : 1) * sm_count();
  if (grid > nitems) grid = nitems;
  k_sweep_batch<C, TW, P, DP><<<(unsigned)grid, TW / P, smem, s>>>(insts, items, nitems, flip);
  return check_launch();
}

template <int C>
static int batch_sweep_all(const BatchHeader& h, const BatchInst* insts, const BatchItem* items,
                           int flip, cudaStream_t s) {
  int st = OPYX_OK;
  const int n0 = h.class_beg[1] - h.class_beg[0], n1 = h.class_beg[2] - h.class_beg[1];
  const int n2 = h.class_beg[3] - h.class_beg[2];
  if (n0) st = batch_launch_sweep<C, 128>(insts, items + h.class_beg[0], n0, flip, s);
  if (!st && n1) st = batch_launch_sweep<C, 256>(insts, items + h.class_beg[1], n1, flip, s);
  if (!st && n2) st = batch_launch_sweep<C, 512>(insts, items + h.class_beg[2], n2, flip, s);
  return st;
}

template <int C>
static int batch_sweep_class(const BatchHeader& h, const BatchInst* insts, const BatchItem* items,
                             int cls, int flip, cudaStream_t s) {
  const int n = h.class_beg[cls + 1] - h.class_beg[cls];
  if (!n) return OPYX_OK;
  const BatchItem* it = items + h.class_beg[cls];
  if (cls == 0) return batch_launch_sweep<C, 128>(insts, it, n, flip, s);
  if (cls == 1) return batch_launch_sweep<C, 256>(insts, it, n, flip, s);
  return batch_launch_sweep<C, 512>(insts, it, n, flip, s);
}

}  // namespace rof
}  // namespace opyx

extern "C" {

size_t opyx_rof_batch_record_bytes(void) { return kBatchRecord; }

size_t opyx_rof_batch_desc_bytes(int ninst, int nitems) {
  if (ninst < 0 || nitems < 0) return 0;
  return batch_item_off(ninst) + (size_t)nitems * sizeof(BatchItem);
}

int opyx_rof_batch_describe(const opyx_rof_problem* probs, const opyx_rof_buffers* bufs,
                            int ninst, void* records, const uint8_t* active, int rows_per_item,
                            void* host_desc, size_t host_bytes, int* nitems_out) {
  if (!probs || !bufs || ninst < 1 || !records || rows_per_item < 1 || (!host_desc && host_bytes) ||
      !nitems_out)
    return OPYX_ERR_ARG;
  if (((uintptr_t)records) & 255) return OPYX_ERR_WORKSPACE;
  const int C = probs[0].nchannels;
  int64_t nitems = 0;
  for (int i = 0; i < ninst; ++i) {
    opyx_rof_buffers bb = bufs[i];
    bb.ws = records;   // the batch keeps step state and info in `records`
    int st = batch_check(&probs[i], &bb);
    if (st) return st;
    if (probs[i].nchannels != C) return OPYX_ERR_ARG;
    if (active && !active[i]) continue;
    int64_t tw;
    batch_tiles(probs[i].dims[1], &tw);
    const int64_t gx = (probs[i].dims[1] + tw - 1) / tw;
    const int64_t gy = (probs[i].dims[0] + rows_per_item - 1) / rows_per_item;
    nitems += gx * gy;
  }
  if (nitems > INT32_MAX) return OPYX_ERR_UNSUPPORTED;
  *nitems_out = (int)nitems;   // also on OPYX_ERR_WORKSPACE: the size to allocate
  if (host_bytes < opyx_rof_batch_desc_bytes(ninst, (int)nitems)) return OPYX_ERR_WORKSPACE;
  char* base = (char*)host_desc;
  BatchHeader* h = (BatchHeader*)base;
  h->ninst = ninst;
  h->nitems = (int)nitems;
  h->nchannels = C;
  h->rows_per_item = rows_per_item;
  h->witems = 0;
  h->pad = 0;
  BatchInst* insts = (BatchInst*)(base + batch_inst_off());
  BatchItem* items = (BatchItem*)(base + batch_item_off(ninst));
  for (int i = 0; i < ninst; ++i) {
    const opyx_rof_problem* p = &probs[i];
    BatchInst& bi = insts[i];
    memset(&bi, 0, sizeof(bi));
    opyx_rof_buffers bb = bufs[i];
    bb.ws = records;
    bi.g = make_geo<float>(p);
    bi.a = make_args<float>(p, &bb);
    char* rec = (char*)records + (size_t)i * kBatchRecord;
    bi.a.st = (opyx_adaptive_state*)rec;
    bi.a.info = (opyx_rof_info*)(rec + 256);
    bi.a.partials = nullptr;
    bi.a.ticket = nullptr;
    host_state(p, &bi.st0);
    bi.ssd_shift = p->ssd_shift;
    bi.item_beg = bi.item_end = 0;
    bi.w_ntx = (int32_t)((p->dims[1] + kStripW - 1) / kStripW);
    bi.w_nty = (int32_t)((p->dims[0] + rows_per_item - 1) / rows_per_item);
  }
  // strips of the persistent solve: every instance, active or not
  int64_t w = 0;
  for (int i = 0; i < ninst; ++i) {
    insts[i].w_beg = (int32_t)w;
    w += (int64_t)insts[i].w_ntx * insts[i].w_nty;
  }
  if (w > INT32_MAX) return OPYX_ERR_UNSUPPORTED;
  h->witems = (int32_t)w;
  // items grouped by tile class; an image's items are consecutive
  int32_t k = 0;
  for (int c = 0; c < kBatchClasses; ++c) {
    h->class_beg[c] = k;
    for (int i = 0; i < ninst; ++i) {
      const opyx_rof_problem* p = &probs[i];
      int64_t tw;
      if ((active && !active[i]) || batch_tiles(p->dims[1], &tw) != c) continue;
      const int64_t rows = p->dims[0], nl = p->dims[1];
      insts[i].item_beg = k;
      // tile columns outer: vertically adjacent items are consecutive, so a
      // CTA whose share holds several sweeps them as one run of rows
      for (int64_t q = 0; q < nl; q += tw)
        for (int64_t r0 = 0; r0 < rows; r0 += rows_per_item) {
          BatchItem& it = items[k++];
          it.inst = i;
          it.r0 = (int32_t)r0;
          it.r1 = (int32_t)(r0 + rows_per_item < rows ? r0 + rows_per_item : rows);
          it.q_beg = (int32_t)q;
          it.q_end = (int32_t)(q + tw < nl ? q + tw : nl);
        }
      insts[i].item_end = k;
    }
  }
  h->class_beg[kBatchClasses] = k;
  *nitems_out = (int)nitems;
  return OPYX_OK;
}

int opyx_rof_batch_init(const void* host_desc, const void* dev_desc, void* stream) {
  if (!host_desc || !dev_desc) return OPYX_ERR_ARG;
  const BatchHeader& h = *(const BatchHeader*)host_desc;
  if (h.ninst < 1) return OPYX_ERR_ARG;
  const BatchInst* insts = (const BatchInst*)((const char*)dev_desc + batch_inst_off());
  k_batch_init<<<(h.ninst + 127) / 128, 128, 0, (cudaStream_t)stream>>>(insts, h.ninst);
  return check_launch();
}

int opyx_rof_batch_iterate(const void* host_desc, const void* dev_desc, int iters, void* stream) {
  if (!host_desc || !dev_desc || iters < 0 || (iters & 1)) return OPYX_ERR_ARG;
  const BatchHeader& h = *(const BatchHeader*)host_desc;
  if (h.ninst < 1 || h.nitems < 0) return OPYX_ERR_ARG;
  if (h.nitems == 0 || iters == 0) return OPYX_OK;
  const BatchInst* insts = (const BatchInst*)((const char*)dev_desc + batch_inst_off());
  const BatchItem* items = (const BatchItem*)((const char*)dev_desc + batch_item_off(h.ninst));
  cudaStream_t s = (cudaStream_t)stream;
  for (int it = 0; it < iters; ++it) {
    int st;
    switch (h.nchannels) {
      case 1: st = batch_sweep_all<1>(h, insts, items, it & 1, s); break;
      case 2: st = batch_sweep_all<2>(h, insts, items, it & 1, s); break;
      case 3: st = batch_sweep_all<3>(h, insts, items, it & 1, s); break;
      case 4: st = batch_sweep_all<4>(h, insts, items, it & 1, s); break;
      default: return OPYX_ERR_UNSUPPORTED;
    }
    if (st) return st;
  }
  return OPYX_OK;
}

int opyx_rof_batch_iterate_class(const void* host_desc, const void* dev_desc, int cls, int iters,
                                 void* stream) {
  if (!host_desc || !dev_desc || iters < 0 || (iters & 1) || cls < 0 || cls >= kBatchClasses)
    return OPYX_ERR_ARG;
  const BatchHeader& h = *(const BatchHeader*)host_desc;
  if (h.ninst < 1 || h.nitems < 0) return OPYX_ERR_ARG;
  if (h.nitems == 0 || iters == 0) return OPYX_OK;
  const BatchInst* insts = (const BatchInst*)((const char*)dev_desc + batch_inst_off());
  const BatchItem* items = (const BatchItem*)((const char*)dev_desc + batch_item_off(h.ninst));
  cudaStream_t s = (cudaStream_t)stream;
  for (int it = 0; it < iters; ++it) {
    int st;
    switch (h.nchannels) {
      case 1: st = batch_sweep_class<1>(h, insts, items, cls, it & 1, s); break;
      case 2: st = batch_sweep_class<2>(h, insts, items, cls, it & 1, s); break;
      case 3: st = batch_sweep_class<3>(h, insts, items, cls, it & 1, s); break;
      case 4: st = batch_sweep_class<4>(h, insts, items, cls, it & 1, s); break;
      default: return OPYX_ERR_UNSUPPORTED;
    }
    if (st) return st;
  }
  return OPYX_OK;
}

size_t opyx_rof_batch_persist_ws_bytes(const void* host_desc) {
  if (!host_desc) return 0;
  const BatchHeader& h = *(const BatchHeader*)host_desc;
  if (h.ninst < 1 || h.witems < 0) return 0;
  return persist_part_off(h.ninst) + (size_t)h.witems * 5 * sizeof(double);
}

int opyx_rof_batch_persist(const void* host_desc, const void* dev_desc, void* ws, int gran,
                           int maxiter, void* stream) {
  if (!host_desc || !dev_desc || !ws || gran < 2 || (gran & 1) || maxiter < 0 || (maxiter & 1))
    return OPYX_ERR_ARG;
  if (((uintptr_t)ws) & 255) return OPYX_ERR_WORKSPACE;
  const BatchHeader& h = *(const BatchHeader*)host_desc;
  if (h.ninst < 1 || h.witems < 0 || h.rows_per_item < 1) return OPYX_ERR_ARG;
  if (h.nchannels != 1) return OPYX_ERR_UNSUPPORTED;
  const BatchInst* hinst = (const BatchInst*)((const char*)host_desc + batch_inst_off());
  const int steps = hinst[0].g.steps;
  for (int i = 1; i < h.ninst; ++i)
    if (hinst[i].g.steps != steps) return OPYX_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(ws, 0, persist_part_off(h.ninst), s) != cudaSuccess) return OPYX_ERR_LAUNCH;
  if (maxiter == 0 || h.witems == 0) return OPYX_OK;
  const BatchInst* insts = (const BatchInst*)((const char*)dev_desc + batch_inst_off());
  PersistCtl* ctl = (PersistCtl*)ws;
  int* act_inst = (int*)((char*)ws + 256);
  int* act_off = (int*)((char*)ws + persist_act_off(h.ninst));
  int* act_goff = (int*)((char*)ws + persist_act_goff(h.ninst));
  double* partials = (double*)((char*)ws + persist_part_off(h.ninst));
  int ninst = h.ninst, R = h.rows_per_item;
  void* args[] = {(void*)&insts, &ninst, &R, &ctl, &act_inst, &act_off, &act_goff, &partials,
                  &gran, &maxiter};
  bool mask = false;
  for (int i = 0; i < h.ninst; ++i) mask |= hinst[i].a.mask != nullptr;
  const bool pre = steps == OPYX_STEPS_PRECOND;
  const void* fn = pre ? (mask ? (const void*)k_batch_persist<true, true>
                               : (const void*)k_batch_persist<true, false>)
                       : (mask ? (const void*)k_batch_persist<false, true>
                               : (const void*)k_batch_persist<false, false>);
  static int per_sm[4] = {-1, -1, -1, -1};
  int& ps = per_sm[(pre ? 2 : 0) + (mask ? 1 : 0)];
  if (ps < 0 && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, fn, kPersistThreads, 0) !=
                    cudaSuccess)
    return OPYX_ERR_LAUNCH;
  if (ps < 1) return OPYX_ERR_LAUNCH;
  const unsigned grid = (unsigned)(ps * sm_count());
  if (cudaLaunchCooperativeKernel(fn, grid, kPersistThreads, args, 0, s) != cudaSuccess)
    return OPYX_ERR_LAUNCH;
  return check_launch();
}

int opyx_rof_batch_gap(const void* host_desc, const void* dev_desc, double* partials,
                       void* stream) {
  if (!host_desc || !dev_desc) return OPYX_ERR_ARG;
  const BatchHeader& h = *(const BatchHeader*)host_desc;
  if (h.ninst < 1 || h.nitems < 0 || (h.nitems > 0 && !partials)) return OPYX_ERR_ARG;
  if (((uintptr_t)partials) & 7) return OPYX_ERR_WORKSPACE;
  if (h.nitems == 0) return OPYX_OK;
  const BatchInst* insts = (const BatchInst*)((const char*)dev_desc + batch_inst_off());
  const BatchItem* items = (const BatchItem*)((const char*)dev_desc + batch_item_off(h.ninst));
  cudaStream_t s = (cudaStream_t)stream;
  const int nitems = h.nitems;
  unsigned grid = (unsigned)(nitems < sm_count() * 8 ? nitems : sm_count() * 8);
  switch (h.nchannels) {
    case 1: k_gap_batch<1><<<grid, 256, 0, s>>>(insts, items, nitems, partials); break;
    case 2: k_gap_batch<2><<<grid, 256, 0, s>>>(insts, items, nitems, partials); break;
    case 3: k_gap_batch<3><<<grid, 256, 0, s>>>(insts, items, nitems, partials); break;
    case 4: k_gap_batch<4><<<grid, 256, 0, s>>>(insts, items, nitems, partials); break;
    default: return OPYX_ERR_UNSUPPORTED;
  }
  int st = check_launch();
  if (st) return st;
  k_gap_fold<<<h.ninst, 128, 0, s>>>(insts, h.ninst, partials);
  return check_launch();
}

}  // extern "C"
