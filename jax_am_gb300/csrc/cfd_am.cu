// Implicit CFD / energy solver of JAX-AM's AM_3d (jax_am/cfd/cfd_am.py), float64.
//
// Layout: fields are (nx, ny, nz) C order, z fastest (cell c = (i ny + j) nz
// + k); vel, conv, grad_p0 carry three components per cell.  A stencil
// operator is the reference's per-cell Jacobian rows (cfd_am.py:474-484):
// seven planes (cell, x-, x+, y-, y+, z-, z+) of n values, applied to the
// mirrored neighbour list of mesh3d (a boundary cell's missing neighbour is
// the cell itself, cfd_am.py:697-706).
//
// BiCGSTAB follows jax.scipy.sparse.linalg.bicgstab (preconditioned
// van der Vorst with JAX's stopping rule |r|^2 <= max(tol^2 |b|^2, atol^2),
// its early exit on |s|^2 and its breakdown codes).  One iteration is six
// launches: two elementwise updates, two stencil applications with fused dot
// products, one elementwise update with two fused dot products, and a
// single-block scalar step that advances rho, alpha, omega, k and the stop
// flag.  Dot products are per-block partial sums reduced in a fixed order, so
// results do not depend on scheduling.  The host enqueues iterations in
// chunks and reads the stop flag after each chunk; launches after the stop
// return at once, so the iteration count is exactly JAX's.  No kernel waits
// on another.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "pfg_host.h"

namespace pfg {
int g_cfd_cells_per_thread = 4;  // pfg_tune key 6

namespace cfd {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 1024;  // partial sums per dot product
constexpr int kSlots = 8;         // dot products with partials in flight

struct Dims {
  int nx, ny, nz;
  long long n;
  double D[6], dS[6], dV;  // mesh3d's signed face distances and areas (cfd_am.py:681-690)
  double g[6];             // dS / D per face, computed once on the host
  double invD[6];          // 1 / D: the kernels multiply (float64 division is slow on GB300)
};

static Dims make_dims(const pfg_cfd_grid& g) {
  Dims d{};
  d.nx = g.nx;
  d.ny = g.ny;
  d.nz = g.nz;
  d.n = (long long)g.nx * g.ny * g.nz;
  const double dx = g.dx, dy = g.dy, dz = g.dz;
  const double D[6] = {-dx, dx, -dy, dy, -dz, dz};
  const double S[6] = {-dy * dz, dy * dz, -dz * dx, dz * dx, -dx * dy, dx * dy};
  for (int f = 0; f < 6; ++f) {
    d.D[f] = D[f];
    d.dS[f] = S[f];
    d.g[f] = S[f] / D[f];
    d.invD[f] = 1.0 / D[f];
  }
  d.dV = dx * dy * dz;
  return d;
}

// Neighbour of cell (i, j, k) across face f, mirrored at the boundary.
__device__ __forceinline__ long long nb_index(const Dims& d, long long c, int i, int j, int k,
                                              int f) {
  const long long sx = (long long)d.ny * d.nz, sy = d.nz;
  switch (f) {
    case 0: return i > 0 ? c - sx : c;
    case 1: return i < d.nx - 1 ? c + sx : c;
    case 2: return j > 0 ? c - sy : c;
    case 3: return j < d.ny - 1 ? c + sy : c;
    case 4: return k > 0 ? c - 1 : c;
    default: return k < d.nz - 1 ? c + 1 : c;
  }
}
__device__ __forceinline__ bool on_face(const Dims& d, int i, int j, int k, int f) {
  switch (f) {
    case 0: return i == 0;
    case 1: return i == d.nx - 1;
    case 2: return j == 0;
    case 3: return j == d.ny - 1;
    case 4: return k == 0;
    default: return k == d.nz - 1;
  }
}
// cell -> (i, j, k); the host keeps n below 2^31, so 32-bit division suffices
__device__ __forceinline__ void ijk(const Dims& d, long long c, int& i, int& j, int& k) {
  const unsigned cu = (unsigned)c, nz = (unsigned)d.nz, ny = (unsigned)d.ny;
  const unsigned r = cu / nz;
  k = (int)(cu - r * nz);
  const unsigned q = r / ny;
  j = (int)(r - q * ny);
  i = (int)q;
}

// np.clip: min(max(T, lo), hi), NaN passes through
__device__ __forceinline__ double clip(double T, double lo, double hi) {
  return T < lo ? lo : (T > hi ? hi : T);
}
__device__ __forceinline__ double linclip(const pfg_linclip& f, double T) {
  return f.a * clip(T, f.lo, f.hi) + f.b;
}
// derivative as jax.jacrev gives it: a inside, a/2 at a tie, 0 outside
__device__ __forceinline__ double linclip_d(const pfg_linclip& f, double T) {
  const double w = (T > f.lo && T < f.hi) ? 1.0 : ((T == f.lo || T == f.hi) ? 0.5 : 0.0);
  return f.a * w;
}
// mesh3d cell centres: midpoints of numpy.linspace(0, L, n + 1) nodes
__device__ __forceinline__ double centre(int i, int n, double h, double L) {
  const double a = (double)i * h;
  const double b = (i + 1 == n) ? L : (double)(i + 1) * h;
  return (b + a) / 2.0;
}

// ---- reductions (fixed order) ---------------------------------------------
__device__ double block_allsum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (l == 0) sh[32] = t;
  }
  __syncthreads();
  const double r = sh[32];
  __syncthreads();
  return r;
}
__device__ __forceinline__ void put_partial(double v, double* P, double* sh) {
  const double t = block_allsum(v, sh);
  if (threadIdx.x == 0) P[blockIdx.x] = t;
}
__device__ double sum_partials(const double* P, int nb, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) v += P[i];
  return block_allsum(v, sh);
}

// ---- BiCGSTAB --------------------------------------------------------------
// Scalars live in device memory.  A dot product is a partial sum per block;
// the block that completes the slot's counter (an atomic increment after
// its partial is fenced) adds the partials in block order and stores the
// result, so every value is reduced once and in a fixed order.
struct KState {
  double atol2, rho, alpha, omega;  // previous iteration's scalars
  double rho_new;                   // <rhat, r> for the coming iteration
  double rs;                        // <r, r>
  double alpha_cur, ss, omega_cur;  // this iteration's alpha, <s, s>, omega
  double bb;                        // <b, b> (setup) or a residual norm^2
  long long k, maxiter;
  int done, pad;
  unsigned cnt[8];                  // last-block counters, one per slot
};
enum { P_RQ = 0, P_SS, P_TS, P_TT, P_RR, P_RHR, P_BB, P_AUX };

struct Work {
  double* vals;  // 7 n
  double* diag;  // n: Jacobi reciprocals 1 / precond_values
  double* b;
  double* x;
  double* r;
  double* rhat;
  double* p;
  double* phat;
  double* q;
  double* s;
  double* shat;
  double* t;
  double* velL;  // 3 nL (flow step)
  double* P;     // kSlots * kMaxBlocks partials
  KState* st;
};

// Blocks for n cells: about four cells per thread, at most four blocks per
// SM.  GB300 issues about two float64 FMAs per clock per SM, so a block's
// reduction tree (a few float64 adds per lane) must be amortised over several
// cells per thread; four blocks of 256 threads per SM still keep enough loads
// in flight for the HBM-bound solves.
static int nblocks(long long n) {
  const int sm = std::max(1, device_info().sm_count);
  const long long cpt = std::max(1, g_cfd_cells_per_thread);
  const long long cap = std::min<long long>((16 / cpt + 1) * (long long)sm, kMaxBlocks);
  const long long b = (n + cpt * kThreads - 1) / (cpt * kThreads);
  return (int)std::max(1LL, std::min(b, cap));
}

#define GRID_LOOP(c, n) \
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < (n); \
       c += (long long)gridDim.x * blockDim.x)

// Post this block's partial of slot `slot`; true in the one block that
// arrives last (it may then read every partial of the slot).
__device__ bool post_partial(double v, double* P, int slot, unsigned* cnt, double* sh) {
  __shared__ bool last;
  const double t = block_allsum(v, sh);
  if (threadIdx.x == 0) {
    P[slot * kMaxBlocks + blockIdx.x] = t;
    __threadfence();
    last = atomicAdd(&cnt[slot], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}
// Two sums posted together under the counter of slot `s1`.
__device__ bool post_pair(double v1, double v2, double* P, int s1, int s2, unsigned* cnt,
                          double* sh) {
  __shared__ bool last;
  const double a1 = block_allsum(v1, sh);
  const double a2 = block_allsum(v2, sh);
  if (threadIdx.x == 0) {
    P[s1 * kMaxBlocks + blockIdx.x] = a1;
    P[s2 * kMaxBlocks + blockIdx.x] = a2;
    __threadfence();
    last = atomicAdd(&cnt[s1], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}
// In the last block: the slot's partials added in block order; resets the
// slot's counter (a slot read through another slot's counter leaves its own
// counter at zero, where it already is).
__device__ double total(const double* P, int slot, unsigned* cnt, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
    v += __ldcg(P + slot * kMaxBlocks + i);
  const double r = block_allsum(v, sh);
  if (threadIdx.x == 0) cnt[slot] = 0u;
  return r;
}

__device__ __forceinline__ double apply_row(const Dims& d, const double* vals, const double* u,
                                            long long c) {
  int i, j, k;
  ijk(d, c, i, j, k);
  double acc = vals[c] * u[c];
#pragma unroll
  for (int f = 0; f < 6; ++f) acc += vals[(1 + f) * d.n + c] * u[nb_index(d, c, i, j, k, f)];
  return acc;
}

// x = 0, r = rhat = p = q = b; the last block sets up the scalars
__global__ void k_setup(long long n, const double* b, double* x, double* r, double* rhat,
                        double* p, double* q, double* P, KState* st, double tol, double atol,
                        long long maxiter) {
  __shared__ double sh[33];
  double bb = 0.0;
  GRID_LOOP(c, n) {
    const double v = b[c];
    x[c] = 0.0;
    r[c] = v;
    rhat[c] = v;
    p[c] = v;
    q[c] = v;
    bb += v * v;
  }
  if (!post_partial(bb, P, P_BB, st->cnt, sh)) return;
  const double bs = total(P, P_BB, st->cnt, sh);
  if (threadIdx.x == 0) {
    const double a2 = tol * tol * bs, b2 = atol * atol;
    st->atol2 = a2 > b2 ? a2 : b2;
    st->rho = st->alpha = st->omega = 1.0;
    st->rho_new = bs;  // <rhat, r> with rhat = r = b
    st->rs = bs;
    st->bb = bs;
    st->k = 0;
    st->maxiter = maxiter;
    st->done = !(bs > st->atol2 && 0 < maxiter);
  }
}

// p = r + beta (p - omega q); phat = M p (dinv: the Jacobi reciprocals, or NULL)
__global__ void k_a(long long n, const KState* st, const double* r, double* p, const double* q,
                    double* phat, const double* dinv) {
  if (st->done) return;
  const double beta = st->rho_new / st->rho * st->alpha / st->omega;
  const double om = st->omega;
  GRID_LOOP(c, n) {
    const double v = r[c] + beta * (p[c] - om * q[c]);
    p[c] = v;
    phat[c] = dinv ? dinv[c] * v : v;
  }
}

// q = A phat; alpha = rho / <rhat, q>
__global__ void k_b(Dims d, KState* st, const double* vals, const double* phat, double* q,
                    const double* rhat, double* P) {
  if (st->done) return;
  __shared__ double sh[33];
  double acc = 0.0;
  GRID_LOOP(c, d.n) {
    const double v = apply_row(d, vals, phat, c);
    q[c] = v;
    acc += rhat[c] * v;
  }
  if (!post_partial(acc, P, P_RQ, st->cnt, sh)) return;
  const double rq = total(P, P_RQ, st->cnt, sh);
  if (threadIdx.x == 0) st->alpha_cur = st->rho_new / rq;
}

// s = r - alpha q; shat = M s; <s, s>
__global__ void k_c(long long n, KState* st, const double* r, const double* q, double* s,
                    double* shat, const double* dinv, double* P) {
  if (st->done) return;
  __shared__ double sh[33];
  const double alpha = st->alpha_cur;
  double acc = 0.0;
  GRID_LOOP(c, n) {
    const double v = r[c] - alpha * q[c];
    s[c] = v;
    shat[c] = dinv ? dinv[c] * v : v;
    acc += v * v;
  }
  if (!post_partial(acc, P, P_SS, st->cnt, sh)) return;
  const double ss = total(P, P_SS, st->cnt, sh);
  if (threadIdx.x == 0) st->ss = ss;
}

// t = A shat; omega = <t, s> / <t, t>
__global__ void k_d(Dims d, KState* st, const double* vals, const double* shat, double* t,
                    const double* s, double* P) {
  if (st->done) return;
  __shared__ double sh[33];
  double ts = 0.0, tt = 0.0;
  GRID_LOOP(c, d.n) {
    const double v = apply_row(d, vals, shat, c);
    t[c] = v;
    ts += v * s[c];
    tt += v * v;
  }
  if (!post_pair(ts, tt, P, P_TS, P_TT, st->cnt, sh)) return;
  const double tsv = total(P, P_TS, st->cnt, sh);
  const double ttv = total(P, P_TT, st->cnt, sh);
  if (threadIdx.x == 0) st->omega_cur = tsv / ttv;
}

// x, r update (early exit when <s, s> < atol2); <r, r>, <rhat, r>; the
// scalar step of the iteration (JAX's k, breakdown codes and stop test)
__global__ void k_e(long long n, KState* st, double* P, double* x, double* r, const double* s,
                    const double* t, const double* phat, const double* shat, const double* rhat) {
  if (st->done) return;
  __shared__ double sh[33];
  const double alpha = st->alpha_cur, omega = st->omega_cur;
  const bool exit_early = st->ss < st->atol2;
  double rr = 0.0, rhr = 0.0;
  GRID_LOOP(c, n) {
    double rn;
    if (exit_early) {
      x[c] = x[c] + alpha * phat[c];
      rn = s[c];
    } else {
      x[c] = x[c] + (alpha * phat[c] + omega * shat[c]);
      rn = s[c] - omega * t[c];
    }
    r[c] = rn;
    rr += rn * rn;
    rhr += rhat[c] * rn;
  }
  if (!post_pair(rr, rhr, P, P_RR, P_RHR, st->cnt, sh)) return;
  const double rs = total(P, P_RR, st->cnt, sh);
  const double rh = total(P, P_RHR, st->cnt, sh);
  if (threadIdx.x == 0) {
    const double rho_ = st->rho_new;
    long long k = (omega == 0.0 || alpha == 0.0) ? -11 : st->k + 1;
    if (rho_ == 0.0) k = -10;
    st->rho = rho_;
    st->alpha = alpha;
    st->omega = omega;
    st->rho_new = rh;
    st->rs = rs;
    st->k = k;
    st->done = !(rs > st->atol2 && k < st->maxiter && k >= 0);
  }
}

static cudaError_t read_state(const KState* dst, KState* host, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(host, dst, sizeof(KState), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

// One chunk of kChunk iterations, launched directly ...
constexpr int kChunk = 8;
static void launch_chunk(const Dims& d, const double* vals, const double* dinv, double* x,
                         const Work& w, int nb, cudaStream_t s) {
  const long long n = d.n;
  for (int it = 0; it < kChunk; ++it) {
    k_a<<<nb, kThreads, 0, s>>>(n, w.st, w.r, w.p, w.q, w.phat, dinv);
    k_b<<<nb, kThreads, 0, s>>>(d, w.st, vals, w.phat, w.q, w.rhat, w.P);
    k_c<<<nb, kThreads, 0, s>>>(n, w.st, w.r, w.q, w.s, w.shat, dinv, w.P);
    k_d<<<nb, kThreads, 0, s>>>(d, w.st, vals, w.shat, w.t, w.s, w.P);
    k_e<<<nb, kThreads, 0, s>>>(n, w.st, w.P, x, w.r, w.s, w.t, w.phat, w.shat, w.rhat);
  }
}

// ... or as a CUDA graph captured once per argument set (operator, reciprocals,
// solution and scratch buffers, grid) and replayed.  The cache only grows: an
// executable is never destroyed, so one in flight on another thread stays
// valid; past kMaxGraphs argument sets the chunks are launched directly.
struct GraphKey {
  const void *vals, *dinv, *x, *r, *P;  // r and P fix the scratch layout
  long long n;
  int nx, ny, nz, dev, nb;
  bool operator==(const GraphKey& o) const {
    return vals == o.vals && dinv == o.dinv && x == o.x && r == o.r && P == o.P && n == o.n &&
           nx == o.nx && ny == o.ny && nz == o.nz && dev == o.dev && nb == o.nb;
  }
};
constexpr int kMaxGraphs = 64;
static std::mutex g_graph_mu;
static GraphKey g_graph_keys[kMaxGraphs];
static cudaGraphExec_t g_graph_execs[kMaxGraphs];
static int g_graph_count = 0;

static cudaGraphExec_t chunk_graph(const Dims& d, const double* vals, const double* dinv,
                                   double* x, const Work& w, int nb) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  const GraphKey key{vals, dinv, x, w.r, w.P, d.n, d.nx, d.ny, d.nz, dev, nb};
  std::lock_guard<std::mutex> lock(g_graph_mu);
  for (int i = 0; i < g_graph_count; ++i)
    if (g_graph_keys[i] == key) return g_graph_execs[i];
  if (g_graph_count == kMaxGraphs) return nullptr;
  cudaStream_t cap = nullptr;
  if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    launch_chunk(d, vals, dinv, x, w, nb, cap);
    if (cudaStreamEndCapture(cap, &g) == cudaSuccess && g) {
      if (cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) exec = nullptr;
      cudaGraphDestroy(g);
    }
  }
  cudaStreamDestroy(cap);
  cudaGetLastError();  // a failed capture falls back to direct launches
  if (!exec) return nullptr;
  g_graph_keys[g_graph_count] = key;
  g_graph_execs[g_graph_count] = exec;
  ++g_graph_count;
  return exec;
}

// Solve vals x = b (dinv: Jacobi reciprocals or NULL); *iters = JAX's k.
static int krylov(const Dims& d, const double* vals, const double* dinv, const double* b,
                  double* x, double tol, double atol, long long maxiter, Work& w,
                  cudaStream_t s, long long* iters) {
  const long long n = d.n;
  const int nb = nblocks(n);
  // the scalars and the last-block counters start from zero in every solve
  cudaError_t e = cudaMemsetAsync(w.st, 0, sizeof(KState), s);
  if (e != cudaSuccess) return record_cuda(e);
  k_setup<<<nb, kThreads, 0, s>>>(n, b, x, w.r, w.rhat, w.p, w.q, w.P, w.st, tol, atol, maxiter);
  e = cudaGetLastError();
  if (e != cudaSuccess) return record_cuda(e);
  KState h{};
  e = read_state(w.st, &h, s);
  if (e != cudaSuccess) return record_cuda(e);
  if (h.done) {
    *iters = h.k;
    return PFG_OK;
  }
  cudaGraphExec_t exec = chunk_graph(d, vals, dinv, x, w, nb);
  long long launched = 0;
  int reps = 1;
  // at most maxiter iterations run; the stop flag is set no later than that;
  // chunks launched after the stop return at once
  while (!h.done && launched < maxiter + 1) {
    for (int r = 0; r < reps; ++r) {
      if (exec) {
        e = cudaGraphLaunch(exec, s);
        if (e != cudaSuccess) return record_cuda(e);
      } else {
        launch_chunk(d, vals, dinv, x, w, nb, s);
      }
    }
    launched += (long long)reps * kChunk;
    e = cudaGetLastError();
    if (e != cudaSuccess) return record_cuda(e);
    e = read_state(w.st, &h, s);
    if (e != cudaSuccess) return record_cuda(e);
    reps = std::min(reps * 2, 8);
  }
  *iters = h.k;
  return PFG_OK;
}

// ---- energy equation ---------------------------------------------------------
struct EnergyK {
  pfg_cfd_energy e;
  double Lx, Ly, Lz;  // domain lengths: the last mesh node (centre coordinates)
  double dx, dy, dz;
};

__device__ __forceinline__ double cp_eff(const pfg_cfd_energy& e, double T0) {
  const double bump = e.latent_heat / (e.Tl - e.Ts);
  return linclip(e.cp, T0) + bump * ((T0 > e.Ts && T0 < e.Tl) ? 1.0 : 0.0);
}

// b = -residual(U) (cfd_am.py:446-454 with the energy source :497-500 and
// the Neumann top flux :334-358); partial <b, b>
__global__ void k_energy_residual(Dims d, EnergyK K, const double* U, const double* T0,
                                  const double* conv, double* b, double* P) {
  __shared__ double sh[33];
  const pfg_cfd_energy& e = K.e;
  double acc = 0.0;
  GRID_LOOP(c, d.n) {
    int i, j, k;
    ijk(d, c, i, j, k);
    const double u = U[c];
    const double ku = linclip(e.k, u);
    double lap = 0.0;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const double un = U[nb_index(d, c, i, j, k, f)];
      const double kn = linclip(e.k, un);
      const double mu = 2.0 * ku * kn / (kn + ku);
      lap += (un - u) * d.invD[f] * mu * d.dS[f];
    }
    const double t0 = T0[c];
    const double cp0 = cp_eff(e, t0);
    double Q = 0.0;
    const double xc = centre(i, d.nx, K.dx, K.Lx), yc = centre(j, d.ny, K.dy, K.Ly);
    const double r2 = e.rb * e.rb;
    if (e.heat_source == 1) {  // Gaussian cylinder (cfd_am.py:224-233)
      const double zc = centre(k, d.nz, K.dz, K.Lz);
      const double dep = e.phi * e.P / e.speed / r2;
      Q = 2.0 * e.P * e.eta / dep / M_PI / r2 *
          exp(-2.0 * ((xc - e.xl) * (xc - e.xl) + (yc - e.yl) * (yc - e.yl)) / r2);
      Q = Q * (((e.zl - zc) <= dep) ? 1.0 : 0.0);
    }
    const double src = -e.rho * (u - t0) * cp0 / e.dt - e.rho * cp0 * conv[c] + Q;
    double res = -lap - src * d.dV;
    if (k == d.nz - 1) {
      const double t2 = t0 * t0, rr = e.T_ref * e.T_ref;  // x**4 as (x*x)*(x*x), as JAX does
      const double t4 = t2 * t2, r4 = rr * rr;
      double q = -(e.h_conv * (t0 - e.T_ref)) - e.sigma * e.emissivity * (t4 - r4);
      if (e.heat_source == 0)  // Gaussian surface flux (cfd_am.py:326-332)
        q = q + 2.0 * e.P * e.eta / M_PI / r2 *
                    exp(-2.0 * ((xc - e.xl) * (xc - e.xl) + (yc - e.yl) * (yc - e.yl)) / r2);
      res -= q * fabs(d.dS[5]);
    }
    b[c] = -res;
    acc += res * res;
  }
  put_partial(acc, P + P_AUX * kMaxBlocks, sh);
}

// Jacobian rows of the energy residual and the Jacobi diagonal
__global__ void k_energy_jacobian(Dims d, EnergyK K, const double* U, const double* T0,
                                  double* vals, double* diag) {
  const pfg_cfd_energy& e = K.e;
  GRID_LOOP(c, d.n) {
    int i, j, k;
    ijk(d, c, i, j, k);
    const double u = U[c];
    const double ku = linclip(e.k, u), dku = linclip_d(e.k, u);
    double v0 = 0.0, dg = 0.0;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const double un = U[nb_index(d, c, i, j, k, f)];
      const double kn = linclip(e.k, un), dkn = linclip_d(e.k, un);
      const double rden = 1.0 / (kn + ku);  // one float64 division per face
      const double mu = 2.0 * ku * kn * rden;
      const double dmu_p = 2.0 * dku * kn * kn * (rden * rden);
      const double dmu_n = 2.0 * dkn * ku * ku * (rden * rden);
      const double g = d.g[f];
      v0 += g * mu - (un - u) * g * dmu_p;
      const double vf = -(g * mu + (un - u) * g * dmu_n);
      vals[(1 + f) * d.n + c] = vf;
      if (on_face(d, i, j, k, f)) dg += vf;
    }
    v0 += e.rho * cp_eff(e, T0[c]) / e.dt * d.dV;
    vals[c] = v0;
    diag[c] = 1.0 / (v0 + dg);  // the reference applies M as 1./precond_values * U
  }
}

__global__ void k_copy(long long n, const double* a, double* b) {
  GRID_LOOP(c, n) b[c] = a[c];
}
__global__ void k_axpy(long long n, double* U, const double* inc) {
  GRID_LOOP(c, n) U[c] = U[c] + inc[c];
}
__global__ void k_norm(const double* P, int nb, double* out) {
  __shared__ double sh[33];
  const double v = sum_partials(P + P_AUX * kMaxBlocks, nb, sh);
  if (threadIdx.x == 0) *out = v;
}

// ---- velocity equation (local box) ------------------------------------------
struct FlowK {
  pfg_cfd_flow f;
  int gnx, gny, gnz;  // global grid
  double ldx, ldy;    // local cell size (Marangoni gradient)
};

__device__ __forceinline__ long long gidx(const FlowK& F, int i, int j, int k) {
  return ((long long)(F.f.x0 + i) * F.gny + (F.f.y0 + j)) * F.gnz + (F.f.z0 + k);
}
__device__ __forceinline__ double fluid_frac(double T, double Ts, double Tl) {
  return (clip(T, Ts, Tl) - Ts) / (Tl - Ts);
}

// momentum component `comp`: b = -residual(0) and Jacobian rows
// (cfd_am.py:530-536, 426-472, solver_linear :748-778)
__global__ void k_momentum(Dims d, FlowK F, int comp, const double* T, const double* vel0,
                           const double* conv, const double* gp, double* b, double* vals,
                           double* diag) {
  const pfg_cfd_flow& f = F.f;
  GRID_LOOP(c, d.n) {
    int i, j, k;
    ijk(d, c, i, j, k);
    const long long g = gidx(F, i, j, k);
    const double u0 = vel0[3 * g + comp];
    const double fl = fluid_frac(T[g], f.Ts, f.Tl);
    const double src0 = -f.rho * (0.0 - u0) / f.dt - f.rho * conv[3 * g + comp] - gp[3 * g + comp];
    double res = -src0 * d.dV;
    if (k == d.nz - 1 && comp < 2) {  // Marangoni shear, Neumann (cfd_am.py:291-317)
      const int im = i > 0 ? i - 1 : 0, ip = i < d.nx - 1 ? i + 1 : i;
      const int jm = j > 0 ? j - 1 : 0, jp = j < d.ny - 1 ? j + 1 : j;
      const double flt = fluid_frac(T[g], f.Ts, f.Tl);
      double m;
      if (comp == 0)
        m = (T[gidx(F, ip, j, k)] - T[gidx(F, im, j, k)]) / 2.0 / F.ldx * f.marangoni / f.visco * flt;
      else
        m = (T[gidx(F, i, jp, k)] - T[gidx(F, i, jm, k)]) / 2.0 / F.ldy * f.marangoni / f.visco * flt;
      res -= m * f.visco * fabs(d.dS[5]);
    }
    b[c] = -res;
    const double darcy = 1e7 * f.rho * (1.0 - fl) * (1.0 - fl) / (fl * fl * fl + 1e-5);
    double v0 = 0.0, dg = 0.0;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const double gq = d.g[q];
      v0 += gq * f.visco;
      const double vq = -gq * f.visco;
      vals[(1 + q) * d.n + c] = vq;
      if (on_face(d, i, j, k, q)) {
        dg += vq;
        // Dirichlet walls: all faces but the top for u and v (cfd_am.py:304-310)
        if (q < 5 || comp == 2) v0 += f.visco * 2.0 * d.invD[q] * d.dS[q];
      }
    }
    v0 += (f.rho / f.dt + darcy) * d.dV;
    vals[c] = v0;
    diag[c] = 1.0 / (v0 + dg);
  }
}

// pressure Poisson rows (mu = 1, no boundary terms: cfd_am.py:538-547)
__global__ void k_pressure_vals(Dims d, double* vals) {
  GRID_LOOP(c, d.n) {
    double v0 = 0.0;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const double gq = d.g[q];
      v0 += gq;
      vals[(1 + q) * d.n + c] = -gq;
    }
    vals[c] = v0;
  }
}

// face velocity between cells a-1 and a along an axis of extent n: zero on
// the box's faces (get_face_vels with the wall ghosts, cfd_am.py:94-112)
__device__ __forceinline__ double face_u(const double* u, long long c, long long stride, int a,
                                         int n) {
  if (a == 0 || a == n) return 0.0;
  return (u[c] + u[c - stride]) / 2.0;
}

// b = -div(vel*) dV / dt * rho (cfd_am.py:578-584); velL is SoA (3, nL)
__global__ void k_pressure_rhs(Dims d, FlowK F, const double* velL, double* b, double ldz) {
  const long long sx = (long long)d.ny * d.nz, sy = d.nz;
  GRID_LOOP(c, d.n) {
    int i, j, k;
    ijk(d, c, i, j, k);
    const double* u = velL;
    const double* v = velL + d.n;
    const double* w = velL + 2 * d.n;
    const double dxl = -d.D[0], dyl = -d.D[2];
    const double div = ((face_u(u, c + sx, sx, i + 1, d.nx) - face_u(u, c, sx, i, d.nx)) / dxl +
                        (face_u(v, c + sy, sy, j + 1, d.ny) - face_u(v, c, sy, j, d.ny)) / dyl +
                        (face_u(w, c + 1, 1, k + 1, d.nz) - face_u(w, c, 1, k, d.nz)) / ldz) /
                       F.f.dt * F.f.rho;
    b[c] = -(div * d.dV);
  }
}

// gradient of p (zero-gradient ghosts, cfd_am.py:82-91), projection and
// pressure-gradient update written into the global arrays
__global__ void k_project(Dims d, FlowK F, const double* p, const double* velL, double* vel,
                          double* grad_p0, double ldz) {
  const long long sx = (long long)d.ny * d.nz, sy = d.nz;
  GRID_LOOP(c, d.n) {
    int i, j, k;
    ijk(d, c, i, j, k);
    const double pc = p[c];
    const double pxm = i > 0 ? p[c - sx] : pc, pxp = i < d.nx - 1 ? p[c + sx] : pc;
    const double pym = j > 0 ? p[c - sy] : pc, pyp = j < d.ny - 1 ? p[c + sy] : pc;
    const double pzm = k > 0 ? p[c - 1] : pc, pzp = k < d.nz - 1 ? p[c + 1] : pc;
    const double dxl = -d.D[0], dyl = -d.D[2];
    const double g3[3] = {((pxp - pc) + (pc - pxm)) / dxl / 2.0, ((pyp - pc) + (pc - pym)) / dyl / 2.0,
                          ((pzp - pc) + (pc - pzm)) / ldz / 2.0};
    const long long g = gidx(F, i, j, k);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      vel[3 * g + q] = velL[q * d.n + c] - F.f.dt * g3[q] / F.f.rho;
      grad_p0[3 * g + q] = grad_p0[3 * g + q] + g3[q];
    }
  }
}

// face value of the theta-blended upwind scheme (cfd_am.py:61-72): cells
// l2, l1 | r1, r2 around the face, uf the face velocity
__device__ __forceinline__ double upwind_face(double l2, double l1, double r1, double r2,
                                              double uf) {
  const double th = 0.125;
  return th * (l1 / 2.0 + r1 / 2.0) + (1.0 - th) * (3.0 * l1 / 2.0 - l2 / 2.0) * (uf >= 0.0 ? 1.0 : 0.0) +
         (1.0 - th) * (3.0 * r1 / 2.0 - r2 / 2.0) * (uf < 0.0 ? 1.0 : 0.0);
}

// div(f, vel_f) on the box for f = T and the three velocity components
// (update_convective_terms, cfd_am.py:254-259), global cell size
__global__ void k_convective(Dims d, FlowK F, double gdx, double gdy, double gdz, const double* T,
                             const double* vel, double* conv_T, double* conv) {
  GRID_LOOP(c, d.n) {
    int i, j, k;
    ijk(d, c, i, j, k);
    const int n3[3] = {d.nx, d.ny, d.nz};
    const int a3[3] = {i, j, k};
    const double h3[3] = {gdx, gdy, gdz};
    double out[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      // cells a-2 .. a+2 along the axis, clamped to the box
      int idx[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        int a = a3[ax] + m - 2;
        a = a < 0 ? 0 : (a > n3[ax] - 1 ? n3[ax] - 1 : a);
        idx[m] = a;
      }
      long long gc[5];
#pragma unroll
      for (int m = 0; m < 5; ++m)
        gc[m] = ax == 0 ? gidx(F, idx[m], j, k) : (ax == 1 ? gidx(F, i, idx[m], k) : gidx(F, i, j, idx[m]));
      // face velocities of the low and high faces of the cell (component ax)
      const double ulo = (a3[ax] == 0) ? 0.0 : (vel[3 * gc[1] + ax] + vel[3 * gc[2] + ax]) / 2.0;
      const double uhi = (a3[ax] == n3[ax] - 1) ? 0.0 : (vel[3 * gc[2] + ax] + vel[3 * gc[3] + ax]) / 2.0;
#pragma unroll
      for (int fld = 0; fld < 4; ++fld) {
        double v[5];
#pragma unroll
        for (int m = 0; m < 5; ++m) v[m] = fld == 0 ? T[gc[m]] : vel[3 * gc[m] + (fld - 1)];
        const double flo = upwind_face(v[0], v[1], v[2], v[3], ulo);
        const double fhi = upwind_face(v[1], v[2], v[3], v[4], uhi);
        out[fld] += (fhi * uhi - flo * ulo) / h3[ax];
      }
    }
    const long long g = gidx(F, i, j, k);
    conv_T[g] = out[0];
    conv[3 * g + 0] = out[1];
    conv[3 * g + 1] = out[2];
    conv[3 * g + 2] = out[3];
  }
}

__global__ void k_solid(long long n, double Ts, double Tl, const double* T, double* solid) {
  GRID_LOOP(c, n) {
    const double fl = fluid_frac(T[c], Ts, Tl);
    const double s = solid[c];
    solid[c] = (s > fl || s != s) ? s : fl;  // np.maximum propagates NaN
  }
}

// ---- host side ---------------------------------------------------------------
static long long cells(const pfg_cfd_grid* g) { return (long long)g->nx * g->ny * g->nz; }

static int check_grid(const pfg_cfd_grid* g) {
  if (!g) return PFG_ERR_NULL;
  if (g->nx < 1 || g->ny < 1 || g->nz < 1) return PFG_ERR_SHAPE;
  if ((long long)g->nx * g->ny * g->nz >= (1LL << 31)) return PFG_ERR_SHAPE;  // 32-bit cell math
  if (!(g->dx > 0.0) || !(g->dy > 0.0) || !(g->dz > 0.0)) return PFG_ERR_PARAM;
  if (!(g->lx > 0.0) || !(g->ly > 0.0) || !(g->lz > 0.0)) return PFG_ERR_PARAM;
  return PFG_OK;
}

static int64_t workspace_bytes(long long n, long long nl) {
  const long long m = std::max(n, nl);
  return (int64_t)((18 * m + 3 * nl + (long long)kSlots * kMaxBlocks) * 8 + 256);
}

static bool carve(void* ws, int64_t bytes, long long n, long long nl, Work& w) {
  if (!ws || ((uintptr_t)ws & 7) || bytes < workspace_bytes(n, nl)) return false;
  const long long m = std::max(n, nl);
  double* p = static_cast<double*>(ws);
  w.vals = p; p += 7 * m;
  w.diag = p; p += m;
  w.b = p; p += m;
  w.x = p; p += m;
  w.r = p; p += m;
  w.rhat = p; p += m;
  w.p = p; p += m;
  w.phat = p; p += m;
  w.q = p; p += m;
  w.s = p; p += m;
  w.shat = p; p += m;
  w.t = p; p += m;
  w.velL = p; p += 3 * nl;
  w.P = p; p += (long long)kSlots * kMaxBlocks;
  w.st = reinterpret_cast<KState*>(p);
  return true;
}

}  // namespace cfd
}  // namespace pfg

using namespace pfg;
using namespace pfg::cfd;

extern "C" int64_t pfg_cfd_workspace_bytes(const pfg_cfd_grid* global, const pfg_cfd_grid* local) {
  if (!global) return -PFG_ERR_NULL;
  return workspace_bytes(cells(global), local ? cells(local) : 0);
}

extern "C" int pfg_cfd_energy_solve(const pfg_cfd_grid* g, const pfg_cfd_energy* e,
                                    const double* T0, const double* conv_T, double* T_out,
                                    void* ws, int64_t ws_bytes, pfg_cfd_stats* stats,
                                    void* stream) {
  int st = check_grid(g);
  if (st) return st;
  if (!e || !T0 || !conv_T || !T_out) return PFG_ERR_NULL;
  if (!(e->dt > 0.0) || !(e->Tl > e->Ts) || e->max_newton < 0 ||
      (e->heat_source != 0 && e->heat_source != 1))
    return PFG_ERR_PARAM;
  const long long n = cells(g);
  Work w{};
  if (!carve(ws, ws_bytes, n, 0, w)) return PFG_ERR_CAPACITY;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const Dims d = make_dims(*g);
  EnergyK K{};
  K.e = *e;
  K.dx = g->dx;
  K.dy = g->dy;
  K.dz = g->dz;
  K.Lx = g->lx;
  K.Ly = g->ly;
  K.Lz = g->lz;
  const int nb = nblocks(n);
  // the Newton residual norm^2 sits after the solver state, inside the 256-byte reserve
  static_assert(sizeof(KState) <= 192, "solver state outgrew its reserve");
  double* norm = reinterpret_cast<double*>(w.st) + 24;
  k_copy<<<nb, kThreads, 0, s>>>(n, T0, T_out);
  k_energy_residual<<<nb, kThreads, 0, s>>>(d, K, T_out, T0, conv_T, w.b, w.P);
  k_norm<<<1, kThreads, 0, s>>>(w.P, nb, norm);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return record_cuda(ce);
  double bb0 = 0.0;
  ce = cudaMemcpyAsync(&bb0, norm, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return record_cuda(ce);
  const double res_init = std::sqrt(bb0);
  double bb = bb0;
  int it = 0;
  long long lin = 0;
  while (std::sqrt(bb) / res_init > e->newton_tol && it < e->max_newton) {
    k_energy_jacobian<<<nb, kThreads, 0, s>>>(d, K, T_out, T0, w.vals, w.diag);
    long long k = 0;
    st = krylov(d, w.vals, w.diag, w.b, w.x, 1e-5, 0.0, 10 * n, w, s, &k);
    if (st) return st;
    lin += k;
    k_axpy<<<nb, kThreads, 0, s>>>(n, T_out, w.x);
    k_energy_residual<<<nb, kThreads, 0, s>>>(d, K, T_out, T0, conv_T, w.b, w.P);
    k_norm<<<1, kThreads, 0, s>>>(w.P, nb, norm);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) return record_cuda(ce);
    ce = cudaMemcpyAsync(&bb, norm, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return record_cuda(ce);
    ++it;
  }
  if (stats) {
    stats->newton_iters = it;
    stats->energy_krylov = lin;
  }
  return PFG_OK;
}

extern "C" int pfg_cfd_solid_update(const pfg_cfd_grid* g, double Ts, double Tl, const double* T,
                                    double* solidID, void* stream) {
  int st = check_grid(g);
  if (st) return st;
  if (!T || !solidID) return PFG_ERR_NULL;
  if (!(Tl > Ts)) return PFG_ERR_PARAM;
  const long long n = cells(g);
  k_solid<<<nblocks(n), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(n, Ts, Tl, T, solidID);
  return record_cuda(cudaGetLastError());
}

extern "C" int pfg_cfd_flow_step(const pfg_cfd_grid* global, const pfg_cfd_grid* local,
                                 const pfg_cfd_flow* f, const double* T, double* vel,
                                 double* conv, double* grad_p0, double* conv_T, void* ws,
                                 int64_t ws_bytes, pfg_cfd_stats* stats, void* stream) {
  int st = check_grid(global);
  if (st) return st;
  st = check_grid(local);
  if (st) return st;
  if (!f || !T || !vel || !conv || !grad_p0 || !conv_T) return PFG_ERR_NULL;
  if (f->x0 < 0 || f->y0 < 0 || f->z0 < 0 || f->x0 + local->nx > global->nx ||
      f->y0 + local->ny > global->ny || f->z0 + local->nz > global->nz)
    return PFG_ERR_SHAPE;
  if (!(f->dt > 0.0) || !(f->rho > 0.0) || !(f->visco > 0.0) || !(f->Tl > f->Ts))
    return PFG_ERR_PARAM;
  const long long n = cells(global), nl = cells(local);
  Work w{};
  if (!carve(ws, ws_bytes, n, nl, w)) return PFG_ERR_CAPACITY;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const Dims d = make_dims(*local);
  FlowK F{};
  F.f = *f;
  F.gnx = global->nx;
  F.gny = global->ny;
  F.gnz = global->nz;
  F.ldx = local->dx;
  F.ldy = local->dy;
  const int nb = nblocks(nl);
  for (int comp = 0; comp < 3; ++comp) {
    k_momentum<<<nb, kThreads, 0, s>>>(d, F, comp, T, vel, conv, grad_p0, w.b, w.vals, w.diag);
    long long k = 0;
    st = krylov(d, w.vals, w.diag, w.b, w.velL + comp * nl, 1e-10, 0.0, 10000, w, s, &k);
    if (st) return st;
    if (stats) stats->momentum_krylov[comp] = k;
  }
  k_pressure_rhs<<<nb, kThreads, 0, s>>>(d, F, w.velL, w.b, local->dz);
  k_pressure_vals<<<nb, kThreads, 0, s>>>(d, w.vals);
  long long k = 0;
  st = krylov(d, w.vals, nullptr, w.b, w.x, 1e-10, 0.0, 10000, w, s, &k);
  if (st) return st;
  if (stats) stats->pressure_krylov = k;
  k_project<<<nb, kThreads, 0, s>>>(d, F, w.x, w.velL, vel, grad_p0, local->dz);
  k_convective<<<nb, kThreads, 0, s>>>(d, F, global->dx, global->dy, global->dz, T, vel, conv_T,
                                       conv);
  return record_cuda(cudaGetLastError());
}
