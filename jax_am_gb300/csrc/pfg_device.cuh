// Device-side helpers shared by the phase-field, heat, diagnostics, batch and
// adjoint kernels.  Internal to the library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pf_gb300.h"
#include "pfg_df.cuh"

namespace pfg {

constexpr int kThreads = 256;  // threads per CTA of every stencil kernel

// ---------------------------------------------------------------------------
// cp.async (LDGSTS) wrappers: global -> shared copies that bypass registers.
// ---------------------------------------------------------------------------
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if constexpr (BYTES == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
  } else if constexpr (BYTES == 8) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait(int pending) {
  // wait_group takes an immediate
  if (pending <= 0) asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  else if (pending == 1) asm volatile("cp.async.wait_group 1;\n" ::: "memory");
  else asm volatile("cp.async.wait_group 2;\n" ::: "memory");
}

// Reciprocal to within 1 ulp (one MUFU instruction, denormal inputs flushed).
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Vector of V floats moved as one 4/8/16-byte access.
template <int V>
struct VecF {
  float v[V];
  __device__ __forceinline__ void load(const float* p) {
    if constexpr (V == 4) {
      const float4 t = *reinterpret_cast<const float4*>(p);
      v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else if constexpr (V == 2) {
      const float2 t = *reinterpret_cast<const float2*>(p);
      v[0] = t.x; v[1] = t.y;
    } else {
      v[0] = *p;
    }
  }
  __device__ __forceinline__ void store(float* p) const {
    if constexpr (V == 4) {
      *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else if constexpr (V == 2) {
      *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    } else {
      *p = v[0];
    }
  }
  __device__ __forceinline__ void store_stream(float* p) const {
    if constexpr (V == 4) {
      __stcs(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
    } else if constexpr (V == 2) {
      __stcs(reinterpret_cast<float2*>(p), make_float2(v[0], v[1]));
    } else {
      __stcs(p, v[0]);
    }
  }
};

// Index of a neighbour plane/row/column under the boundary condition:
// Neumann replicates the edge cell (allen_cahn.py:61-66), periodic wraps.
__device__ __forceinline__ int bc_index(int i, int n, int periodic) {
  if (i < 0) return periodic ? i + n : 0;
  if (i >= n) return periodic ? i - n : n - 1;
  return i;
}

// ---------------------------------------------------------------------------
// Phase-field per-cell constants.
// With S = sum_j eta_j^2 and gamma = 1 (allen_cahn.py:43) the energy gradient
// m_g [eta^3 - eta + 4 eta (S - eta^2) + 2 (1 - zeta)^2 eta] / ad_hoc
// (allen_cahn.py:42-51,58) equals (m_g/ad_hoc) eta (K - 3 eta^2) with
// K = 4 S + 2 (1 - zeta)^2 - 1, and one Euler step is
//   eta' = eta + cg * eta (K - 3 eta^2) + cl * a * Lap(eta),
//   cg = -dt Lg m_g / ad_hoc,   cl = dt Lg kappa_g ad_hoc,
// where Lap sums (eta_+ - eta) + (eta_- - eta) over axes weighted by 1/h^2.
// ---------------------------------------------------------------------------
struct PFConsts {
  float wx, wy, wz;          // 1/h^2 per axis
  float T_liq, inv_T_liq;    // liquidus
  // the float32 quotient Tc / T_liq is above 1 exactly when Tc >= zeta_hi and
  // below 1 exactly when Tc <= zeta_lo (both found on the host by stepping
  // through the floats next to T_liq with the same IEEE division)
  float zeta_hi, zeta_lo;
  float neg_Qg_over_R;       // -Qg / gas_const
  float L0;
  float mg_ad;               // m_g / ad_hoc
  float kappa_ad;            // kappa_g * ad_hoc
  float aniso;               // anisotropy strength A
  float liquid_limit;        // T_liquidus + liquid_shift
  int force;                 // liquid forcing on/off
};

struct CellCoef {
  float cg, cl, K, liquid;  // liquid: 1.0 when forcing zeroes this cell
};

// The temperature-only part of a cell's coefficients.
struct TempCoef {
  float cg, cl;   // see above
  float om2;      // 2 (1 - zeta)^2
  float liquid;   // 1.0 when liquid forcing zeroes the cell
};

__device__ __forceinline__ TempCoef temp_coefficients(const PFConsts& c, float T, float dt) {
  // T > 2000 is clipped (allen_cahn.py:56); written as a select so that NaN passes through
  const float Tc = (T > 2000.f) ? 2000.f : T;
  const float zeta = 0.5f * (1.f - tanhf(1e10f * (Tc / c.T_liq - 1.f)));  // allen_cahn.py:57
  const float Lg = c.L0 * expf(c.neg_Qg_over_R / Tc);                      // allen_cahn.py:83
  const float om = 1.f - zeta;
  TempCoef r;
  r.cg = -dt * Lg * c.mg_ad;
  r.cl = dt * Lg * c.kappa_ad;
  r.om2 = 2.f * om * om;
  // forcing compares the unclipped start-of-step T (allen_cahn.py:124-126)
  r.liquid = (c.force && T > c.liquid_limit) ? 1.f : 0.f;
  return r;
}

// The same coefficients for the fast kernel, with cheaper arithmetic:
//  * zeta = (1 - tanh(1e10 x)) / 2 with x = Tc / T_liq - 1 rounded to float32.
//    Tc / T_liq is a float32, so x is 0 or at least 2^-24 in magnitude, and
//    1e10 |x| >= 596: the float32 tanh is exactly +-1 unless x == 0.  zeta is
//    therefore 0 (x > 0), 1 (x < 0) or 1/2 (x == 0), and NaN propagates.
//    The sign of x is read from two precomputed thresholds instead of a
//    division (same result for every float Tc).
//  * Lg uses the fast exponential (relative error ~1e-6 at the Arrhenius
//    arguments of this model, |Qg / (R T)| <= 60).
__device__ __forceinline__ TempCoef temp_coefficients_fast(const PFConsts& c, float T, float dt) {
  const float Tc = (T > 2000.f) ? 2000.f : T;
  const float zeta = (Tc >= c.zeta_hi) ? 0.f
                     : (Tc <= c.zeta_lo) ? 1.f
                     : (Tc == Tc) ? 0.5f : Tc;  // Tc == Tc is false only for NaN
  const float Lg = c.L0 * __expf(c.neg_Qg_over_R * rcp_approx(Tc));
  const float om = 1.f - zeta;
  TempCoef r;
  r.cg = -dt * Lg * c.mg_ad;
  r.cl = dt * Lg * c.kappa_ad;
  r.om2 = 2.f * om * om;
  r.liquid = (c.force && T > c.liquid_limit) ? 1.f : 0.f;
  return r;
}

// temp_coefficients_fast for a compensated temperature Th + Tl: zeta from
// the exact sign of Th + Tl - T_liquidus (the float64 reference's tanh of
// 1e10 (T / T_liq - 1) is +-1 unless |T - T_liq| < ~1e-6 K), Lg from Th.
__device__ __forceinline__ TempCoef temp_coefficients_pair(const PFConsts& c, float Th, float Tl,
                                                           float dt) {
  TempCoef r = temp_coefficients_fast(c, Th, dt);
  if (Th <= 2000.f && Th == c.T_liq && Tl != 0.f) {
    const float om = (Tl > 0.f) ? 1.f : 0.f;  // 1 - zeta
    r.om2 = 2.f * om * om;
  } else if (Th <= 2000.f && Th > c.zeta_lo && Th < c.zeta_hi && Th != c.T_liq) {
    const float om = (Th > c.T_liq) ? 1.f : 0.f;
    r.om2 = 2.f * om * om;
  }
  return r;
}

__device__ __forceinline__ CellCoef cell_coefficients(const TempCoef& t, float S) {
  CellCoef r;
  r.cg = t.cg;
  r.cl = t.cl;
  r.K = 4.f * S + t.om2 - 1.f;
  r.liquid = t.liquid;
  return r;
}

// Cubic anisotropy factor 1 + A (cos^4 t + sin^4 t) where t is the smallest
// folded angle between the central-difference vector e and the orientation's
// three rotated cube axes (allen_cahn.py:28-39).  cos t = max_k |d_k.e|/|e|,
// so with c2 = cos^2 t: cos^4 + sin^4 = c2^2 + (1 - c2)^2.  A zero (or
// non-finite) |e| makes the reference's angles NaN, which it maps to 0, i.e.
// c2 = 1; rounding above 1 is clamped the same way.
__device__ __forceinline__ float aniso_factor(float A, float ex, float ey, float ez,
                                              const float* d /* 9: 3 axes x (x,y,z) */) {
  const float ee = ex * ex + ey * ey + ez * ez;
  const float p0 = d[0] * ex + d[1] * ey + d[2] * ez;
  const float p1 = d[3] * ex + d[4] * ey + d[5] * ez;
  const float p2 = d[6] * ex + d[7] * ey + d[8] * ez;
  const float m = fmaxf(fmaxf(p0 * p0, p1 * p1), p2 * p2);
  float c2 = (ee > 0.f) ? fminf(m / ee, 1.f) : 1.f;
  const float s2 = 1.f - c2;
  return 1.f + A * (c2 * c2 + s2 * s2);
}

// ---------------------------------------------------------------------------
// Heat equation (jax_am/cfd/gamma.py) per interior cell.
// ---------------------------------------------------------------------------
struct HeatConsts {
  int nx, ny, nz;
  float dx, dy, dz;
  float dx2, dy2, dz2;       // d^2
  float rdx2, rdy2, rdz2;    // 1/d^2
  float inv_rho;             // 1/rho
  float rho, h, sb_eps, T0, T0_4, Ts, Tl, latent;
  float beam_coef;           // 2 * absorptivity / pi / r^2  (times P gives the peak flux)
  float two_over_r2;         // 2 / r^2
  float x_first, y_first;
};

__device__ __forceinline__ float heat_k(const HeatConsts& H, float T) {
  return fmaf(0.0163f, fminf(fmaxf(T, 300.f), H.Tl), 4.5847f);  // gamma.py:14
}

// Whether the latent heat enters cp (gamma.py:12,15): the liquid fraction
// fl = (clip(T, Ts, Tl) - Ts) / (Tl - Ts) lies strictly inside (0, 1).  In
// float32 that is exactly Ts < T < Tl whenever Tl <= 2 Ts (every alloy):
// clip(T) - Ts is then exact (Sterbenz), and a correctly rounded quotient
// x / y of floats 0 < x < y is positive and below 1.  For Tl > 2 Ts the two
// tests can differ only for T within one ulp of Tl.
__device__ __forceinline__ bool heat_mushy(const HeatConsts& H, float T) {
  return T > H.Ts && T < H.Tl;
}

// Robin + radiation flux magnitude h (Tf - T0) + SB eps (Tf^4 - T0^4)
// evaluated at the face temperature Tf (gamma.py:23-34).
__device__ __forceinline__ float heat_robin(const HeatConsts& H, float Tf) {
  const float t2 = Tf * Tf;
  // one explicit fused multiply-add: with a * b + c * d the compiler may fuse
  // either product, and which one can depend on the surrounding code
  return fmaf(H.h, Tf - H.T0, H.sb_eps * fmaf(t2, t2, -H.T0_4));
}

// Evaluate the beam position and power at time t from the tool path.
__device__ __forceinline__ void laser_at(const pfg_heat_params& hp, double t, float* xl,
                                         float* yl, float* P) {
  *xl = 0.f; *yl = 0.f; *P = 0.f;
  for (int s = 0; s < hp.num_segments && s < PFG_MAX_SEGMENTS; ++s) {
    const pfg_segment& g = hp.path[s];
    if (t >= (double)g.t0 && t < (double)g.t1) {
      const double f = (t - (double)g.t0) / ((double)g.t1 - (double)g.t0);
      *xl = (float)((double)g.x0 + f * ((double)g.x1 - (double)g.x0));
      *yl = (float)((double)g.y0 + f * ((double)g.y1 - (double)g.y0));
      *P = g.power;
      return;
    }
  }
}

// laser_at with the beam centre in float64.
__device__ __forceinline__ void laser_at_d(const pfg_heat_params& hp, double t, double* xl,
                                           double* yl, float* P) {
  *xl = 0.0; *yl = 0.0; *P = 0.f;
  for (int s = 0; s < hp.num_segments && s < PFG_MAX_SEGMENTS; ++s) {
    const pfg_segment& g = hp.path[s];
    if (t >= (double)g.t0 && t < (double)g.t1) {
      const double f = (t - (double)g.t0) / ((double)g.t1 - (double)g.t0);
      *xl = (double)g.x0 + f * ((double)g.x1 - (double)g.x0);
      *yl = (double)g.y0 + f * ((double)g.y1 - (double)g.y0);
      *P = g.power;
      return;
    }
  }
}

// New ghosts of the domain faces that interior cell (gx, gy, gz) touches,
// computed from the old ghost (gamma.py:18-43), written to Tg_out and
// substituted for the matching neighbour value.  rk = 1 / k(Tc).
template <typename IDX>
__device__ __forceinline__ void heat_faces(const HeatConsts& H, float Tc, float rk, float& Txm,
                                           float& Txp, float& Tym, float& Typ, float& Tzm,
                                           float& Tzp, int gx, int gy, int gz, float xl,
                                           float yl, float P, float* Tg_out, IDX idx, IDX sx,
                                           IDX sy, IDX sz) {
  // Every a * b + c expression below is written as an explicit fmaf: left
  // to the compiler, which product it fuses can depend on the surrounding
  // code (which operands are loop-invariant), and the kernels that call
  // this promise identical results in either axis order.
  if (gx == 0) {
    Txm = fmaf(-(heat_robin(H, (Tc + Txm) * 0.5f) * rk), H.dx, Tc);
    Tg_out[idx - sx] = Txm;
  }
  if (gx == H.nx - 1) {
    Txp = fmaf(-(heat_robin(H, (Tc + Txp) * 0.5f) * rk), H.dx, Tc);
    Tg_out[idx + sx] = Txp;
  }
  if (gy == 0) {
    Tym = fmaf(-(heat_robin(H, (Tc + Tym) * 0.5f) * rk), H.dy, Tc);
    Tg_out[idx - sy] = Tym;
  }
  if (gy == H.ny - 1) {
    Typ = fmaf(-(heat_robin(H, (Tc + Typ) * 0.5f) * rk), H.dy, Tc);
    Tg_out[idx + sy] = Typ;
  }
  if (gz == 0) {
    Tzm = fmaf(-(heat_robin(H, (Tc + Tzm) * 0.5f) * rk), H.dz, Tc);
    Tg_out[idx - sz] = Tzm;
  }
  if (gz == H.nz - 1) {
    // top face: convection + radiation minus the Gaussian beam flux (gamma.py:33-35)
    const float x = fmaf((float)gx, H.dx, H.x_first);
    const float y = fmaf((float)gy, H.dy, H.y_first);
    const float ddx = x - xl, ddy = y - yl;
    const float e = expf(-fmaf(ddx, ddx, ddy * ddy) * H.two_over_r2);
    const float q = fmaf(-(P * H.beam_coef), e, heat_robin(H, (Tc + Tzp) * 0.5f));
    Tzp = fmaf(-(q * rk), H.dz, Tc);
    Tg_out[idx + sz] = Tzp;
  }
}

// One explicit heat update of interior cell (gx, gy, gz) given its old value
// and its six old neighbours in the ghosted field (a neighbour across a
// domain face is the old ghost).  idx is the cell's index in the ghosted
// array and sx, sy, sz its element strides.  New ghosts of the faces this cell touches
// are computed from the old ghost and written to Tg_out (gamma.py:18-43);
// the Laplacian uses them (gamma.py:58-60).  Returns the new interior value.
// FACES = false is for callers that know the cell touches no domain face.
template <typename IDX, bool FACES = true>
__device__ __forceinline__ float heat_cell_update(const HeatConsts& H, float Tc, float Txm,
                                                  float Txp, float Tym, float Typ, float Tzm,
                                                  float Tzp, int gx, int gy, int gz, float xl,
                                                  float yl, float P, float dt, float* Tg_out,
                                                  IDX idx, IDX sx, IDX sy, IDX sz) {
  const float k = heat_k(H, Tc);
  const float cp = fmaf(0.2441f, fminf(fmaxf(Tc, 300.f), H.Tl), 338.39f) +
                   (heat_mushy(H, Tc) ? H.latent : 0.f);  // gamma.py:12-15
  if constexpr (FACES)
    heat_faces(H, Tc, rcp_approx(k), Txm, Txp, Tym, Typ, Tzm, Tzp, gx, gy, gz, xl, yl, P, Tg_out,
               idx, sx, sy, sz);
  // gamma.py:49-51, with explicit fused multiply-adds (see heat_faces)
  const float ax = fmaf(-2.f, Tc, Txm) + Txp;
  const float ay = fmaf(-2.f, Tc, Tym) + Typ;
  const float az = fmaf(-2.f, Tc, Tzm) + Tzp;
  const float lap = fmaf(ax, H.rdx2, fmaf(ay, H.rdy2, az * H.rdz2));
  return fmaf(dt, (k * H.inv_rho) * rcp_approx(cp) * lap, Tc);
}

// ---------------------------------------------------------------------------
// Compensated (double-float) heat update.  The temperature is stored as two
// float32 fields, T = h + l.  A float32 update rounds T to ulp(T) ~ 1e-3 K
// every step at T ~ 1e4 K, and the rounded coefficients k / (rho cp) and
// the rounded beam flux make a run drift from the float64 reference by up
// to ~1e-2 K over thousands of steps; a cell near Ts, Tl (the latent-heat
// switch) or T_liquidus then takes the other branch of the step function
// and differs by O(1 K).  The compensated update keeps the state to ~48
// bits, forms the Laplacian from exact differences, and, wherever the
// temperature is far from ambient (or on a domain face), evaluates the
// coefficients, the Robin/radiation flux and the Gaussian beam in DF.
// ---------------------------------------------------------------------------
struct HeatDF {
  DF k1, k0;          // k = k1 clip(T, 300, Tl) + k0        (gamma.py:14)
  DF c1, c0, latent;  // cp = c1 clip(T, 300, Tl) + c0 [+ L] (gamma.py:12-15)
  DF beam_coef;       // 2 absorptivity / (pi r^2)
  DF two_over_r2;     // 2 / r^2
  DF sb_eps, T0_4;    // sigma eps, T0^4
  DF rd2[3];          // 1 / d^2 per axis
  DF dt;              // the step (a float32 value)
  float hot;          // a warp with a cell or neighbour above this takes the DF path
};

// Robin + radiation flux h (Tf - T0) + sigma eps (Tf^4 - T0^4) in DF
// (gamma.py:23-34), Tf the face temperature.
__device__ __forceinline__ DF heat_robin_df(const HeatConsts& H, const HeatDF& D, DF Tf) {
  const DF t2 = df_mul(Tf, Tf);
  const DF rad = df_mul(D.sb_eps, df_sub(df_mul(t2, t2), D.T0_4));
  return df_add(df_mul_f(df_add_f(Tf, -H.T0), H.h), rad);
}

// k(T) and cp(T) in DF (gamma.py:12-15)
__device__ __forceinline__ void heat_k_cp_df(const HeatConsts& H, const HeatDF& D, DF T, DF& k,
                                             DF& cp) {
  const DF clip = df_gt(T, H.Tl) ? df_from(H.Tl) : (df_lt(T, 300.f) ? df_from(300.f) : T);
  k = df_add(df_mul(D.k1, clip), D.k0);
  cp = df_add(df_mul(D.c1, clip), D.c0);
  if (df_gt(T, H.Ts) && df_lt(T, H.Tl)) cp = df_add(cp, D.latent);
}

// New ghosts of the domain faces the cell touches (gamma.py:18-43), in DF,
// written to (Th_out, Tl_out) and substituted for the neighbour: ghost =
// T - q dx / k.  n[] = xm, xp, ym, yp, zm, zp.  (xl, yl): beam centre.
__device__ __forceinline__ void heat_faces_df(const HeatConsts& H, const HeatDF& D, DF Tc, DF k,
                                              DF* n, int gx, int gy, int gz, DF xl, DF yl,
                                              float P, float* Th_out, float* Tl_out, int idx,
                                              int sx, int sy, int sz) {
  const int face_idx[6] = {idx - sx, idx + sx, idx - sy, idx + sy, idx - sz, idx + sz};
  const bool on[6] = {gx == 0, gx == H.nx - 1, gy == 0, gy == H.ny - 1, gz == 0, gz == H.nz - 1};
  const float d[3] = {H.dx, H.dy, H.dz};
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    if (!on[f]) continue;
    DF Tf = df_add(Tc, n[f]);
    Tf.h *= 0.5f;
    Tf.l *= 0.5f;
    DF q = heat_robin_df(H, D, Tf);
    if (f == 5) {
      // top face: minus the Gaussian beam (gamma.py:33-35), positions exact
      const DF x = df_add_f(two_prod((float)gx, H.dx), H.x_first);
      const DF y = df_add_f(two_prod((float)gy, H.dy), H.y_first);
      const DF ddx = df_sub(x, xl), ddy = df_sub(y, yl);
      const DF r2 = df_add(df_mul(ddx, ddx), df_mul(ddy, ddy));
      const DF e = df_exp_neg(df_neg(df_mul(r2, D.two_over_r2)));
      q = df_sub(q, df_mul_f(df_mul(e, D.beam_coef), P));
    }
    const DF g = df_sub(Tc, df_div(df_mul_f(q, d[f >> 1]), k));
    Th_out[face_idx[f]] = g.h;
    Tl_out[face_idx[f]] = g.l;
    n[f] = g;
  }
}

// The compensated explicit heat update of one interior cell, all in DF:
// k and cp, the new ghosts of the faces the cell touches (Robin/radiation
// and the Gaussian beam), the Laplacian and the update.  For cells far from
// ambient and the beam-heated top plane; kept out of line so that the
// stencil loop stays small.
static __device__ __noinline__ DF heat_update_df_accurate(const HeatConsts& H, const HeatDF& D,
                                                          DF Tc, DF* n, int gx, int gy, int gz,
                                                          DF xl, DF yl, float P, float* Th_out,
                                                          float* Tl_out, int idx, int sx, int sy,
                                                          int sz) {
  DF k, cp;
  heat_k_cp_df(H, D, Tc, k, cp);
  heat_faces_df(H, D, Tc, k, n, gx, gy, gz, xl, yl, P, Th_out, Tl_out, idx, sx, sy, sz);
  DF lap = df_from(0.f);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const DF s2 = df_add(df_sub(n[2 * a], Tc), df_sub(n[2 * a + 1], Tc));
    lap = df_add(lap, df_mul(s2, D.rd2[a]));
  }
  const DF coef = df_div(df_mul(k, D.dt), df_mul_f(cp, H.rho));
  return df_add(Tc, df_mul(coef, lap));
}

// The compensated update of a cell near ambient: float32 coefficients and
// face fluxes (their rounding, ~1e-7 of the increment, is far below 1e-6 K
// when T - T0 < 50 K), the Laplacian from exact differences of the pairs,
// and the state and the new ghosts kept as pairs.  FACES: the cell may
// touch a domain face.
template <bool FACES>
__device__ __forceinline__ DF heat_update_df_near_ambient(const HeatConsts& H, DF Tc, DF* n,
                                                         int gx, int gy, int gz, float xl,
                                                         float yl, float P, float dt,
                                                         float* Th_out, float* Tl_out, int idx,
                                                         int sx, int sy, int sz) {
  const float k = heat_k(H, Tc.h);
  const float cp = fmaf(0.2441f, fminf(fmaxf(Tc.h, 300.f), H.Tl), 338.39f) +
                   (heat_mushy(H, Tc.h) ? H.latent : 0.f);
  if constexpr (FACES) {
    const float rk = rcp_approx(k);
    const int fidx[6] = {idx - sx, idx + sx, idx - sy, idx + sy, idx - sz, idx + sz};
    const bool on[6] = {gx == 0, gx == H.nx - 1, gy == 0, gy == H.ny - 1, gz == 0, gz == H.nz - 1};
    const float d[3] = {H.dx, H.dy, H.dz};
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      if (!on[f]) continue;
      float q = heat_robin(H, (Tc.h + n[f].h) * 0.5f);
      if (f == 5) {
        const float x = fmaf((float)gx, H.dx, H.x_first);
        const float y = fmaf((float)gy, H.dy, H.y_first);
        const float ddx = x - xl, ddy = y - yl;
        q = fmaf(-(P * H.beam_coef), expf(-fmaf(ddx, ddx, ddy * ddy) * H.two_over_r2), q);
      }
      const DF g = df_add_f(Tc, -q * rk * d[f >> 1]);
      Th_out[fidx[f]] = g.h;
      Tl_out[fidx[f]] = g.l;
      n[f] = g;
    }
  }
  const float rd[3] = {H.rdx2, H.rdy2, H.rdz2};
  float lap = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float s2 = ((n[2 * a].h - Tc.h) + (n[2 * a + 1].h - Tc.h)) +
                     ((n[2 * a].l - Tc.l) + (n[2 * a + 1].l - Tc.l));
    lap = fmaf(s2, rd[a], lap);
  }
  return df_add_f(Tc, dt * ((k * H.inv_rho) * rcp_approx(cp) * lap));
}

// ---------------------------------------------------------------------------
// Moving point source (Rosenthal), per cell.
// ---------------------------------------------------------------------------
struct PointConsts {
  float T_ambient, inv_2pi_kappa, inv_2alpha, T_clip;
  float x_first, y_first, z_first;
  float hx, hy, hz;
  const pfg_point_source* table;
  int64_t num_records;
};

// The record a step starting at step count `step` uses.
__device__ __forceinline__ pfg_point_source point_record(const PointConsts& c, int64_t step) {
  const int64_t k = step < 0 ? 0 : (step < c.num_records ? step : c.num_records - 1);
  return c.table[k];
}

// T at the centre of cell (gx, gy, gz) (simple/example.py:28-36,
// multi_scan/example.py:38-48), float32 with the accurate sqrt and exp.
__device__ __forceinline__ float point_source_T(const PointConsts& c, const pfg_point_source& r,
                                                int gx, int gy, int gz) {
  const float X = fmaf((float)gx, c.hx, c.x_first) - r.x;
  const float Y = fmaf((float)gy, c.hy, c.y_first) - r.y;
  const float Z = fmaf((float)gz, c.hz, c.z_first) - r.z;
  const float R = sqrtf(fmaf(X, X, fmaf(Y, Y, Z * Z)));
  const float proj = fmaf(X, r.ux, fmaf(Y, r.uy, Z * r.uz));
  const float T =
      c.T_ambient + (r.Q * c.inv_2pi_kappa) / R * expf(-(r.vel * c.inv_2alpha) * (R + proj));
  return (T > c.T_clip) ? c.T_clip : T;  // NaN passes through
}

// Weight of T_past for a step ending at t_end (coupled/example.py:38-42).
__device__ __forceinline__ float interp_weight(double t_future, double dt_coarse, double t_end) {
  return (float)((t_future - t_end) / dt_coarse);
}

HeatConsts make_heat_consts(const pfg_heat_params& h);
HeatDF make_heat_df(const pfg_heat_params& h, float dt);
PointConsts make_point_consts(const pfg_point_sources& s, const pfg_pf_params& p);
PFConsts make_pf_consts(const pfg_pf_params& p);

}  // namespace pfg
