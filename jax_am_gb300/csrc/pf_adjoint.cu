// Hand-written discrete adjoint of the fused heat + phase-field step.
//
// Forward step k (pfg_heat_pf_step): eta' = eta + dt R(eta, T) with
//   R_i = -Lg(T) (m_g/ad_hoc) g_i + Lg(T) kappa_g ad_hoc a_i(e_i) L_i,
//   g_i = eta_i (K - 3 eta_i^2), K = 4 S + 2 (1 - zeta(T))^2 - 1, S = sum eta^2,
//   L_i = sum_d w_d (eta_i(+d) + eta_i(-d) - 2 eta_i), e_i = central differences,
// and T' = H(T; P, x_laser) (explicit heat step whose ghost faces are state).
// Given the adjoints of step k+1 (lam' = dJ/d eta', Tb' = dJ/dTg' including
// the ghost faces) and the forward state of step k, the kernels below produce
// the adjoints of step k and add this step's dJ/dP and dJ/dv.
//
// Transposes used (derived for the reference's edge-replicate Neumann
// boundary, allen_cahn.py:61-66): the Laplacian term transposes to the same
// Laplacian applied to u = lam Lg kappa' a (even extension at a Neumann face);
// the anisotropy term (a depends on e = eta(+d) - eta(-d)) transposes to minus
// the central difference of v_d = lam Lg kappa' L da/de_d with an odd
// extension at a Neumann face; periodic axes wrap in both.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "pfg_device.cuh"
#include "pfg_host.h"
#include "pfg_step.cuh"

namespace pfg {

struct AdjArgs {
  int nx, ny, nz, n;
  int bcx, bcy, bcz;
  float dt;
  PFConsts pc;
  HeatConsts hc;
  float xl, yl, P, dxl_dv;  // beam at mid-step and d x_laser / d v
  int beam_on;
  const float* eta;    // forward eta at step k (nz, ny, nx, n)
  const float* Tg;     // forward ghosted T at step k
  const float* lam_in; // dJ/d eta^{k+1}
  const float* Tb_in;  // dJ/d Tg^{k+1} (ghosted)
  float* lam_out;      // dJ/d eta^k
  float* Tb_out;       // dJ/d Tg^k (ghosted; interior and faces written)
  float* u;            // (N, n)
  float* v;            // 3 x (N, n)
  float* loc;          // (N, n)
  float* muPF;         // (N) dt * sum_i lam_i dR_i/dT
  float* mask;         // (N) 0 where liquid forcing zeroed the cell, else 1
  double* grads;       // [dJ/dP, dJ/dv]
  float dirs[3 * PFG_MAX_ORIS * 3];
};

__device__ __forceinline__ int nbr(int i, int d, int n, int periodic) {
  return bc_index(i + d, n, periodic);
}

// d zeta / dT of zeta = (1 - tanh(1e10 (T / T_liq - 1))) / 2 evaluated as the
// float32 step kernel does: the float32 tanh is exactly +-1 unless x == 0.
__device__ __forceinline__ float dzeta_dT(const PFConsts& c, float x) {
  return (x == 0.f) ? -0.5f * 1e10f / c.T_liq : 0.f;
}

// Lane layout of kernels A and B: a cell takes tpc = ceil(n / 2) lanes, each
// lane two consecutive orientations, so a warp holds 32 / tpc cells (for
// n = 10: six cells, 30 of 32 lanes busy).
struct AdjLanes {
  int tpc, cpw, cw, g;
  bool active;
};
__device__ __forceinline__ AdjLanes adj_lanes(int n) {
  AdjLanes l;
  const int lane = threadIdx.x & 31;
  l.tpc = (n + 1) >> 1;
  l.cpw = 32 / l.tpc;
  l.cw = lane / l.tpc;
  l.g = lane - l.cw * l.tpc;
  l.active = l.cw < l.cpw;
  return l;
}
// Sum of v over the tpc lanes of this lane's cell, returned to every lane of
// the cell (a guarded shfl-down tree leaves the sum in the cell's lane 0).
__device__ __forceinline__ float cell_sum(float v, const AdjLanes& l) {
  for (int o = 1; o < l.tpc; o <<= 1) {
    const float t = __shfl_down_sync(0xffffffffu, v, o);
    if (l.g + o < l.tpc) v += t;
  }
  const int lane = threadIdx.x & 31;
  return __shfl_sync(0xffffffffu, v, min(lane - l.g, 31));
}

// ---- kernel A: u, v, the local term and the temperature sensitivity --------
// ANISO = false (A = 0): v is identically zero and is neither written nor read.
template <bool ANISO>
__global__ void __launch_bounds__(256) adj_pf_local_kernel(const __grid_constant__ AdjArgs a) {
  const int ncell = a.nx * a.ny * a.nz;  // host checks < 2^31
  const int n = a.n;
  const AdjLanes ln = adj_lanes(n);
  const int warp_id = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  const float mg = a.pc.mg_ad, kap = a.pc.kappa_ad, A = a.pc.aniso;
  const int64_t Nn = (int64_t)ncell * n;
  const int xy = a.nx * a.ny;
  const int64_t sy = (int64_t)a.nx * n, sz = (int64_t)xy * n;
  const int64_t gsy = a.nx + 2, gsz = (int64_t)(a.ny + 2) * (a.nx + 2);
  for (int cb = warp_id * ln.cpw; cb < ncell; cb += nwarps * ln.cpw) {
    const int c = cb + ln.cw;
    const bool valid = ln.active && c < ncell;
    const int cc = valid ? c : 0;
    const int z = cc / xy, r = cc - z * xy, y = r / a.nx, x = r - y * a.nx;
    // temperature-only quantities (as in the forward fast kernels)
    const float T = a.Tg[(int64_t)(z + 1) * gsz + (int64_t)(y + 1) * gsy + x + 1];
    const bool clipped = T > 2000.f;
    const float Tc = clipped ? 2000.f : T;
    const float xz = Tc / a.pc.T_liq - 1.f;
    const float zeta = (xz > 0.f) ? 0.f : (xz < 0.f) ? 1.f : (xz == 0.f) ? 0.5f : xz;
    const float om = 1.f - zeta;
    const float Lg = a.pc.L0 * expf(a.pc.neg_Qg_over_R / Tc);
    const float dLg = clipped ? 0.f : Lg * (-a.pc.neg_Qg_over_R) / (Tc * Tc);
    const float dz = clipped ? 0.f : dzeta_dT(a.pc, xz);
    const bool liquid = a.pc.force && T > a.pc.liquid_limit;
    const int64_t base = (int64_t)z * sz + (int64_t)y * sy + (int64_t)x * n;
    // per-cell sums
    float s = 0.f, ld = 0.f;
    if (valid) {
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int i = 2 * ln.g + j;
        if (i < n) {
          const float ei = a.eta[base + i], li = a.lam_in[base + i];
          s = fmaf(ei, ei, s);
          ld = fmaf(li, ei, ld);
        }
      }
    }
    s = cell_sum(s, ln);
    ld = cell_sum(ld, ln);
    const float K = 4.f * s + 2.f * om * om - 1.f;
    const int xm = nbr(x, -1, a.nx, a.bcx), xp = nbr(x, 1, a.nx, a.bcx);
    const int ym = nbr(y, -1, a.ny, a.bcy), yp = nbr(y, 1, a.ny, a.bcy);
    const int zm = nbr(z, -1, a.nz, a.bcz), zp = nbr(z, 1, a.nz, a.bcz);
    const int64_t oxm = (int64_t)z * sz + (int64_t)y * sy + (int64_t)xm * n;
    const int64_t oxp = (int64_t)z * sz + (int64_t)y * sy + (int64_t)xp * n;
    const int64_t oym = (int64_t)z * sz + (int64_t)ym * sy + (int64_t)x * n;
    const int64_t oyp = (int64_t)z * sz + (int64_t)yp * sy + (int64_t)x * n;
    const int64_t ozm = (int64_t)zm * sz + (int64_t)y * sy + (int64_t)x * n;
    const int64_t ozp = (int64_t)zp * sz + (int64_t)y * sy + (int64_t)x * n;
    float mu = 0.f;
    if (valid) {
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int i = 2 * ln.g + j;
        if (i >= n) continue;
        const float e = a.eta[base + i], lam = liquid ? 0.f : a.lam_in[base + i];
        const float vxm = a.eta[oxm + i], vxp = a.eta[oxp + i];
        const float vym = a.eta[oym + i], vyp = a.eta[oyp + i];
        const float vzm = a.eta[ozm + i], vzp = a.eta[ozp + i];
        const float L = a.pc.wx * ((vxp - e) + (vxm - e)) + a.pc.wy * ((vyp - e) + (vym - e)) +
                        a.pc.wz * ((vzp - e) + (vzm - e));
        float an = 1.f, dax = 0.f, day = 0.f, daz = 0.f;
        if (ANISO) {
          const float ex = vxp - vxm, ey = vyp - vym, ez = vzp - vzm;
          const float ee = ex * ex + ey * ey + ez * ez;
          float pbest = 0.f, m = -1.f;
          int kbest = 0;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const float* d = &a.dirs[(k * n + i) * 3];
            const float pk = d[0] * ex + d[1] * ey + d[2] * ez;
            if (pk * pk > m) { m = pk * pk; pbest = pk; kbest = k; }
          }
          const float c2 = (ee > 0.f) ? m / ee : 1.f;
          if (c2 < 1.f) {
            const float s2 = 1.f - c2;
            an = 1.f + A * (c2 * c2 + s2 * s2);
            // da/de = A (4 c2 - 2) * 2 (p* d* - c2 e) / ee
            const float f = A * (4.f * c2 - 2.f) * 2.f / ee;
            const float* d = &a.dirs[(kbest * n + i) * 3];
            dax = f * (pbest * d[0] - c2 * ex);
            day = f * (pbest * d[1] - c2 * ey);
            daz = f * (pbest * d[2] - c2 * ez);
          } else {
            an = 1.f + A;
          }
        }
        const float gg = e * (K - 3.f * e * e);
        const float Q = Lg * kap;
        a.u[base + i] = lam * Q * an;
        if (ANISO) {
          a.v[base + i] = lam * Q * L * dax;
          a.v[Nn + base + i] = lam * Q * L * day;
          a.v[2 * Nn + base + i] = lam * Q * L * daz;
        }
        a.loc[base + i] = liquid ? 0.f : -Lg * mg * (lam * (K - 9.f * e * e) + 8.f * e * ld);
        mu += lam * (dLg * (-mg * gg + kap * an * L) + Lg * mg * 4.f * om * e * dz);
      }
    }
    mu = cell_sum(mu, ln);
    if (valid && ln.g == 0) {
      a.muPF[c] = a.dt * mu;
      a.mask[c] = liquid ? 0.f : 1.f;
    }
  }
}

// ---- kernel B: the adjoint of the stencil terms, gathered per element --------
template <bool ANISO>
__global__ void __launch_bounds__(256) adj_pf_gather_kernel(const __grid_constant__ AdjArgs a) {
  const int ncell = a.nx * a.ny * a.nz;
  const int n = a.n;
  const AdjLanes ln = adj_lanes(n);
  const int warp_id = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)(((long long)gridDim.x * blockDim.x) >> 5);
  const int64_t Nn = (int64_t)ncell * n;
  const int xy = a.nx * a.ny;
  const int64_t sy = (int64_t)a.nx * n, sz = (int64_t)xy * n;
  for (int cb = warp_id * ln.cpw; cb < ncell; cb += nwarps * ln.cpw) {
    const int c = cb + ln.cw;
    if (!ln.active || c >= ncell) continue;  // no shuffles below
    const int z = c / xy, r = c - z * xy, y = r / a.nx, x = r - y * a.nx;
    const int64_t base = (int64_t)z * sz + (int64_t)y * sy + (int64_t)x * n;
    // neighbour offsets and the sign of v at each (odd extension at a Neumann face)
    int64_t off[6];
    float sgn[6];
    const int dims[3] = {a.nx, a.ny, a.nz};
    const int bcs[3] = {a.bcx, a.bcy, a.bcz};
    const int pos[3] = {x, y, z};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      int q[3] = {x, y, z};
      const int ax = k >> 1, step = (k & 1) ? 1 : -1;
      const int raw = pos[ax] + step;
      q[ax] = bc_index(raw, dims[ax], bcs[ax]);
      sgn[k] = (!bcs[ax] && (raw < 0 || raw >= dims[ax])) ? -1.f : 1.f;
      off[k] = (int64_t)q[2] * sz + (int64_t)q[1] * sy + (int64_t)q[0] * n;
    }
    const float m = a.mask[c];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int i = 2 * ln.g + j;
      if (i >= n) continue;
      const float uc = a.u[base + i];
      const float lapu = a.pc.wx * (a.u[off[0] + i] + a.u[off[1] + i] - 2.f * uc) +
                         a.pc.wy * (a.u[off[2] + i] + a.u[off[3] + i] - 2.f * uc) +
                         a.pc.wz * (a.u[off[4] + i] + a.u[off[5] + i] - 2.f * uc);
      float dvx = 0.f, dvy = 0.f, dvz = 0.f;
      if (ANISO) {
        dvx = sgn[1] * a.v[off[1] + i] - sgn[0] * a.v[off[0] + i];
        dvy = sgn[3] * a.v[Nn + off[3] + i] - sgn[2] * a.v[Nn + off[2] + i];
        dvz = sgn[5] * a.v[2 * Nn + off[5] + i] - sgn[4] * a.v[2 * Nn + off[4] + i];
      }
      a.lam_out[base + i] =
          m * a.lam_in[base + i] + a.dt * (a.loc[base + i] + lapu - (dvx + dvy + dvz));
    }
  }
}

// ---- kernel C: heat transpose, one thread per interior cell -------------------
struct HeatLocal {
  float k, dk, cp, dcp, alpha, dalpha;
};
__device__ __forceinline__ HeatLocal heat_local(const HeatConsts& H, float T) {
  HeatLocal r;
  const bool in = T > 300.f && T < H.Tl;
  const float Tk = fminf(fmaxf(T, 300.f), H.Tl);
  r.k = 0.0163f * Tk + 4.5847f;
  r.dk = in ? 0.0163f : 0.f;
  r.cp = 0.2441f * Tk + 338.39f + (heat_mushy(H, T) ? H.latent : 0.f);
  r.dcp = in ? 0.2441f : 0.f;
  r.alpha = r.k / H.rho / r.cp;
  r.dalpha = (r.dk * r.cp - r.k * r.dcp) / (H.rho * r.cp * r.cp);
  return r;
}

__global__ void __launch_bounds__(256) adj_heat_kernel(const __grid_constant__ AdjArgs a) {
  const HeatConsts& H = a.hc;
  const long long ncell = (long long)a.nx * a.ny * a.nz;
  const int64_t sx = 1, sy = a.nx + 2, sz = (int64_t)(a.ny + 2) * (a.nx + 2);
  const float R2 = a.hc.two_over_r2;
  double gP = 0.0, gv = 0.0;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(c % a.nx), y = (int)((c / a.nx) % a.ny), z = (int)(c / ((long long)a.nx * a.ny));
    const int64_t idx = (int64_t)(z + 1) * sz + (int64_t)(y + 1) * sy + x + 1;
    const float Tc = a.Tg[idx];
    const HeatLocal hl = heat_local(H, Tc);
    const float dt = a.dt;
    const float mu_c = a.Tb_in[idx];
    // neighbours: value used in the forward Laplacian and its adjoint route
    const int64_t st[6] = {-sx, sx, -sy, sy, -sz, sz};
    const bool face[6] = {x == 0, x == a.nx - 1, y == 0, y == a.ny - 1, z == 0, z == a.nz - 1};
    const float d[6] = {H.dx, H.dx, H.dy, H.dy, H.dz, H.dz};
    const float r2[6] = {1.f / H.dx2, 1.f / H.dx2, 1.f / H.dy2, 1.f / H.dy2, 1.f / H.dz2, 1.f / H.dz2};
    float Nv[6], dGdT[6], dGdG[6], dGdB[6], B[6];
    for (int f = 0; f < 6; ++f) {
      const float Gold = a.Tg[idx + st[f]];
      dGdT[f] = dGdG[f] = dGdB[f] = 0.f;
      B[f] = 0.f;
      if (face[f]) {
        const float Tf = 0.5f * (Tc + Gold);
        const float Rf = heat_robin(H, Tf);
        const float dR = H.h + 4.f * H.sb_eps * Tf * Tf * Tf;
        float beam = 0.f;
        if (f == 5 && a.beam_on) {
          const float px = H.x_first + (float)x * H.dx - a.xl;
          const float py = H.y_first + (float)y * H.dy - a.yl;
          beam = a.P * H.beam_coef * expf(-(px * px + py * py) * R2);
          B[f] = beam;
        }
        const float q = Rf - beam;
        Nv[f] = Tc - q / hl.k * d[f];
        dGdT[f] = 1.f - d[f] * (0.5f * dR / hl.k - q * hl.dk / (hl.k * hl.k));
        dGdG[f] = -d[f] * 0.5f * dR / hl.k;
        dGdB[f] = d[f] / hl.k;
      } else {
        Nv[f] = Gold;  // an interior neighbour (old value)
      }
    }
    const float lap = (Nv[0] - 2.f * Tc + Nv[1]) * r2[0] + (Nv[2] - 2.f * Tc + Nv[3]) * r2[2] +
                      (Nv[4] - 2.f * Tc + Nv[5]) * r2[4];
    float mu = mu_c * (1.f + dt * hl.dalpha * lap -
                       2.f * dt * hl.alpha * (r2[0] + r2[2] + r2[4]));
    for (int f = 0; f < 6; ++f) {
      if (face[f]) {
        const float w = mu_c * dt * hl.alpha * r2[f] + a.Tb_in[idx + st[f]];
        mu += w * dGdT[f];
        a.Tb_out[idx + st[f]] = w * dGdG[f];
        if (f == 5 && a.beam_on) {
          // B = P coef exp(...): dB/dP = B / P, dB/dxl = B * 4 (x - xl) / r^2
          const float px = H.x_first + (float)x * H.dx - a.xl;
          gP += (double)(w * dGdB[f]) * (double)(B[f] / a.P);
          gv += (double)(w * dGdB[f]) * (double)(B[f] * 2.f * R2 * px) * (double)a.dxl_dv;
        }
      } else {
        // this cell is the neighbour m's Laplacian input with weight dt alpha_m / d^2
        const float Tm = Nv[f];
        const HeatLocal hm = heat_local(H, Tm);
        mu += a.Tb_in[idx + st[f]] * dt * hm.alpha * r2[f];
      }
    }
    a.Tb_out[idx] = mu + a.muPF[c];
  }
  // block reduction of the two gradient components, one atomic per block
  __shared__ double sP[8], sv[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gP += __shfl_xor_sync(0xffffffffu, gP, o);
    gv += __shfl_xor_sync(0xffffffffu, gv, o);
  }
  if (lane == 0) { sP[w] = gP; sv[w] = gv; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tP = 0.0, tv = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { tP += sP[i]; tv += sv[i]; }
    atomicAdd(&a.grads[0], tP);
    atomicAdd(&a.grads[1], tv);
  }
}

// ---- objective J = mean over cells of sum_i w_i eta_i^2 and its seed ----------
__global__ void __launch_bounds__(256)
objective_kernel(const float* __restrict__ eta, const float* __restrict__ w, long long ncell, int n,
                 double* __restrict__ J, float* __restrict__ lam) {
  double acc = 0.0;
  const long long total = ncell * n;
  const float inv = 1.f / (float)ncell;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n);
    const float v = eta[e];
    acc += (double)w[i] * (double)v * (double)v;
    if (lam) lam[e] = 2.f * w[i] * v * inv;
  }
  __shared__ double s[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += s[i];
    atomicAdd(J, t / (double)ncell);
  }
}

}  // namespace pfg

using namespace pfg;

extern "C" int64_t pfg_adjoint_scratch_bytes(const pfg_pf_params* p) {
  if (check_pf_params(p)) return -1;
  const int64_t N = (int64_t)p->nx * p->ny * p->nz;
  return (5 * N * p->num_oris + 2 * N) * (int64_t)sizeof(float);
}

extern "C" int pfg_adjoint_step(const pfg_pf_params* p, const pfg_heat_params* h,
                                const float* eta, const float* Tg, double t, float dt,
                                const float* lam_in, const float* Tb_in, float* lam_out,
                                float* Tb_out, void* scratch, int64_t scratch_bytes,
                                double* grads, float dxl_dv, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  st = check_heat_params(h);
  if (st) return st;
  if (h->nx != p->nx || h->ny != p->ny || h->nz != p->nz) return PFG_ERR_SHAPE;
  if (!eta || !Tg || !lam_in || !Tb_in || !lam_out || !Tb_out || !scratch || !grads)
    return PFG_ERR_NULL;
  if (scratch_bytes < pfg_adjoint_scratch_bytes(p)) return PFG_ERR_CAPACITY;
  // 32-bit cell indices (with room for the grid-stride look-ahead)
  if ((int64_t)p->nx * p->ny * p->nz >= ((int64_t)1 << 31) - ((int64_t)1 << 22))
    return PFG_ERR_SHAPE;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  AdjArgs a{};
  a.nx = p->nx; a.ny = p->ny; a.nz = p->nz; a.n = p->num_oris;
  a.bcx = p->bc_x; a.bcy = p->bc_y; a.bcz = p->bc_z;
  a.dt = dt;
  a.pc = make_pf_consts(*p);
  a.hc = make_heat_consts(*h);
  float xl = 0.f, yl = 0.f, P = 0.f;
  // the beam at the mid-step time, as the forward step places it
  for (int s = 0; s < h->num_segments; ++s) {
    const pfg_segment& g = h->path[s];
    const double tm = t + 0.5 * (double)dt;
    if (tm >= (double)g.t0 && tm < (double)g.t1) {
      const double f = (tm - (double)g.t0) / ((double)g.t1 - (double)g.t0);
      xl = (float)((double)g.x0 + f * ((double)g.x1 - (double)g.x0));
      yl = (float)((double)g.y0 + f * ((double)g.y1 - (double)g.y0));
      P = g.power;
      break;
    }
  }
  a.xl = xl; a.yl = yl; a.P = P; a.beam_on = P != 0.f; a.dxl_dv = dxl_dv;
  a.eta = eta; a.Tg = Tg; a.lam_in = lam_in; a.Tb_in = Tb_in;
  a.lam_out = lam_out; a.Tb_out = Tb_out;
  const int64_t N = (int64_t)p->nx * p->ny * p->nz, Nn = N * p->num_oris;
  float* sc = static_cast<float*>(scratch);
  a.u = sc;
  a.v = sc + Nn;
  a.loc = sc + 4 * Nn;
  a.muPF = sc + 5 * Nn;
  a.mask = sc + 5 * Nn + N;
  a.grads = grads;
  for (int i = 0; i < 3 * p->num_oris * 3; ++i) a.dirs[i] = p->grain_dirs[i];
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const DeviceInfo& d = device_info();
  const int cpw = 32 / ((p->num_oris + 1) / 2);  // cells per warp of kernels A and B
  const int warps_blocks =
      (int)std::min<int64_t>((N + 8 * cpw - 1) / (8 * cpw), (int64_t)d.sm_count * 16);
  const bool aniso = a.pc.aniso > 0.f;
  if (aniso) adj_pf_local_kernel<true><<<warps_blocks, 256, 0, s>>>(a);
  else adj_pf_local_kernel<false><<<warps_blocks, 256, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return record_cuda(e);
  if (aniso) adj_pf_gather_kernel<true><<<warps_blocks, 256, 0, s>>>(a);
  else adj_pf_gather_kernel<false><<<warps_blocks, 256, 0, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return record_cuda(e);
  const int cell_blocks = (int)std::min<int64_t>((N + 255) / 256, (int64_t)d.sm_count * 16);
  adj_heat_kernel<<<cell_blocks, 256, 0, s>>>(a);
  return record_cuda(cudaGetLastError());
}

extern "C" int pfg_objective(const pfg_pf_params* p, const float* eta, const float* w, double* J,
                             float* lam_seed, void* stream) {
  int st = check_pf_params(p);
  if (st) return st;
  if (!eta || !w || !J) return PFG_ERR_NULL;
  if (!device_info().ok) return PFG_ERR_NO_DEVICE;
  const long long ncell = (long long)p->nx * p->ny * p->nz;
  const int blocks = (int)std::min<long long>((ncell * p->num_oris + 255) / 256,
                                              (long long)device_info().sm_count * 8);
  objective_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      eta, w, ncell, p->num_oris, J, lam_seed);
  return record_cuda(cudaGetLastError());
}
