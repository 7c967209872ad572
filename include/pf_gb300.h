/*
 * pf_gb300.h -- C ABI of the GB300 (sm_103a) phase-field grain-growth library.
 *
 * The library advances JAX-AM's multi-order-parameter Allen-Cahn grain-growth
 * model (jax_am/phase_field/allen_cahn.py) and its explicit finite-difference
 * heat equation with a moving Gaussian laser (jax_am/cfd/gamma.py) on one GPU.
 *
 * Conventions shared by every entry point:
 *  - All array arguments are DEVICE pointers owned by the caller.  Nothing is
 *    allocated inside the library unless an entry point says so.
 *  - eta is float32, shape (nz, ny, nx, num_oris), C order: x fastest among
 *    the cells, orientation innermost -- the reference's (N, num_oris) array
 *    with cells in z-major order (allen_cahn.py:60, phase_field/utils.py:188).
 *  - A per-cell temperature T is float32 (nz, ny, nx) -- the reference's
 *    (N, 1) ode_params array.
 *  - The heat state Tg is float32 (nz+2, ny+2, nx+2) with one ghost layer,
 *    x fastest.  The reference holds the same ghosted field as
 *    (nx+2, ny+2, nz+2), x slowest (applications/cfd/gamma/example.py:85);
 *    pfg_heat_step also accepts that order (pfg_heat_params.layout), so no
 *    transpose is needed at the boundary.  Ghost faces are part of
 *    the state: each step reads the previous ghosts and writes new ones
 *    (gamma.py:23-42).  Edge and corner ghosts are never read or written.
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy
 *    default stream.  Work is enqueued on it and the call returns without
 *    synchronising.
 *  - The return value is 0 (PFG_OK) or a pfg_status code; no exception ever
 *    crosses the ABI.  pfg_status_string() names a code.
 *  - input and output buffers of one step must not overlap.
 */
#ifndef PF_GB300_H
#define PF_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PFG_ABI_VERSION 1
#define PFG_MAX_ORIS 64      /* orientations per cell */
#define PFG_MAX_SEGMENTS 16  /* laser tool-path segments */

typedef enum pfg_status {
  PFG_OK = 0,
  PFG_ERR_SHAPE = 1,        /* a grid extent < 1, or num_oris outside [1, PFG_MAX_ORIS] */
  PFG_ERR_NULL = 2,         /* a required pointer is NULL */
  PFG_ERR_ALIGN = 3,        /* a device pointer is not 16-byte aligned */
  PFG_ERR_PARAM = 4,        /* a parameter is out of its domain (h <= 0, bad bc code, ...) */
  PFG_ERR_LAUNCH = 5,       /* the CUDA launch failed; see pfg_last_cuda_error() */
  PFG_ERR_TIMEOUT = 6,      /* a bounded device-side wait ran out */
  PFG_ERR_CAPACITY = 7,     /* a job table or scratch buffer is too small */
  PFG_ERR_NO_DEVICE = 8     /* no usable sm_103 device */
} pfg_status;

typedef enum pfg_bc { PFG_BC_NEUMANN = 0, PFG_BC_PERIODIC = 1 } pfg_bc;

typedef enum pfg_layout { PFG_LAYOUT_ZYX = 0, PFG_LAYOUT_XYZ = 1 } pfg_layout;

/* Phase-field parameters: the reference pf_args keys (pf_params.yaml) plus the
 * polycrystal's cell size and grain directions (phase_field/utils.py:55-62,
 * 104-109). */
typedef struct pfg_pf_params {
  int32_t nx, ny, nz;      /* cells along x, y, z (pf_args Nx, Ny, Nz) */
  int32_t num_oris;        /* orientations per cell (pf_args num_oris) */
  float h_x, h_y, h_z;     /* cell size [m] (Field.mesh_h_xyz) */
  float T_liquidus;        /* [K] */
  float gas_const;         /* [J/(mol K)] */
  float Qg;                /* [J/mol] */
  float L0;                /* [m^3/(J s)] */
  float kappa_g;           /* [J/m] */
  float m_g;               /* [J/m^3] */
  float anisotropy;        /* 0 disables the anisotropy term, as the reference does */
  float ad_hoc;
  int32_t bc_x, bc_y, bc_z;   /* pfg_bc per axis; the reference is Neumann on all faces */
  int32_t force_liquid_zero;  /* 1: eta = 0 where T > T_liquidus + liquid_shift after the
                                 step (allen_cahn.py:117-128; off in the reference stepper) */
  float liquid_shift;         /* [K], 1.0 in the reference */
  float grain_dirs[3 * PFG_MAX_ORIS * 3];  /* (3, num_oris, 3): rotated cube axes */
} pfg_pf_params;

/* One straight tool-path segment: between times t0 and t1 the beam moves
 * linearly from (x0, y0) to (x1, y1) at `power` watts.  Outside every
 * segment the beam is off. */
typedef struct pfg_segment {
  float t0, t1, x0, y0, x1, y1, power, reserved;
} pfg_segment;

/* Heat-equation parameters: the reference gamma_args dict
 * (applications/cfd/gamma/example.py:67-79) plus the grid. */
typedef struct pfg_heat_params {
  int32_t nx, ny, nz;      /* interior cells */
  float dx, dy, dz;        /* [m] */
  float rho;               /* density (gamma_args rho) */
  float h_conv;            /* convection coefficient (gamma_args h) */
  float emissivity;        /* (gamma_args eps) */
  float sigma_sb;          /* Stefan-Boltzmann constant (gamma_args SB) */
  float T0;                /* ambient temperature (gamma_args T0) */
  float Ts, Tl;            /* solidus / liquidus (gamma_args Ts, Tl) */
  float latent;            /* latent heat per kelvin of mushy range (gamma_args L) */
  float absorptivity;      /* (gamma_args eta) */
  float beam_radius;       /* (gamma_args r) */
  float x_first, y_first;  /* centre of the first cell along x and y (dx/2, dy/2 in the
                              reference driver, applications/cfd/gamma/example.py:61-62) */
  int32_t layout;          /* PFG_LAYOUT_ZYX: Tg is (nz+2, ny+2, nx+2), x fastest (required by
                              pfg_heat_pf_step); PFG_LAYOUT_XYZ: the reference's (nx+2, ny+2,
                              nz+2), z fastest (accepted by pfg_heat_step) */
  int32_t num_segments;    /* tool path used by pfg_heat_pf_step; 0..PFG_MAX_SEGMENTS */
  pfg_segment path[PFG_MAX_SEGMENTS];
} pfg_heat_params;

/* Simulation clock kept on the device so that a captured CUDA graph of fused
 * steps advances time without the host. */
typedef struct pfg_clock {
  double t;       /* time at the start of the step [s] */
  int64_t step;   /* steps taken */
} pfg_clock;

/* Moving linear temperature gradient of the directional-solidification
 * driver (applications/phase_field/solidification/example.py:21-34):
 *   T(z, t) = T_base + grad * (z - z0) - grad * vel * t
 * with z the cell-centre height z_first + iz * h_z.  The reference has
 * z0 = 0 and T_base = T_liquidus. */
typedef struct pfg_quench {
  double T_base;   /* [K] */
  double grad;     /* [K/m] */
  double vel;      /* [m/s] */
  double z0;       /* [m] */
  double z_first;  /* centre of the first cell along z [m] */
} pfg_quench;

/* Analytic moving point source (Rosenthal solution) of the phase-field
 * drivers (applications/phase_field/simple/example.py:21-37,
 * simple/example_grf.py:21-46, multi_scan/example.py:33-49):
 *   T = T_ambient + Q / (2 pi kappa) / R * exp(-vel / (2 alpha) (R + proj)),
 * R the distance from the source to the cell centre, proj the projection of
 * (cell centre - source) on the moving direction, then T = min(T, T_clip).
 * The source state is one record per step: a step that starts with
 * clk_in->step = k uses record min(k, num_records - 1), so the tool path,
 * power and speed can follow any schedule (the drivers' read_path samples,
 * a ramp) with no host work per step. */
typedef struct pfg_point_source {
  double t;         /* time of the record [s] (informational) */
  float x, y, z;    /* source position [m] */
  float ux, uy, uz; /* unit moving direction */
  float Q;          /* absorbed power [W] */
  float vel;        /* speed in the exponent [m/s] */
} pfg_point_source;
typedef struct pfg_point_sources {
  float T_ambient;  /* [K] */
  float alpha;      /* thermal diffusivity [m^2/s] */
  float kappa;      /* conductivity [W/(m K)] */
  float T_clip;     /* clip above this temperature (INFINITY: none) [K] */
  float x_first, y_first, z_first;  /* centre of cell (0, 0, 0) [m] */
  int32_t reserved;
  const pfg_point_source* table;    /* device array of num_records records, 8-byte aligned */
  int64_t num_records;
} pfg_point_sources;

/* Linear time interpolation between two temperature fields of a coarser
 * solver, as the coupled driver does (applications/phase_field/coupled/
 * example.py:38-42): a phase-field step ending at t = clk_in->t + dt uses
 *   T = r T_past + (1 - r) T_future,  r = (t_future - t) / dt_coarse. */
typedef struct pfg_interp {
  double t_future;   /* time of T_future [s] */
  double dt_coarse;  /* time between T_past and T_future [s] */
} pfg_interp;

/* Results of pfg_pf_diag (device memory, written by the call). */
typedef struct pfg_diag {
  double energy;                 /* total free energy [J], compensated accumulation */
  double max_T;                  /* max over cells of T */
  int64_t n_cells;
  int64_t n_ori_changed;         /* cells whose argmax orientation differs from argmax0 */
  int64_t n_liquid;              /* cells with T >= T_liquidus */
  int64_t n_nonfinite;           /* eta entries that are NaN or Inf */
  double mass[PFG_MAX_ORIS];     /* sum over cells of eta_i, compensated accumulation */
} pfg_diag;

/* ---- library information ----------------------------------------------- */
int pfg_abi_version(void);
const char* pfg_status_string(int status);
/* The last CUDA error string seen by an entry point on this thread. */
const char* pfg_last_cuda_error(void);
/* sizeof() of the ABI structs, so bindings can check their mirrors:
 * 0 pfg_pf_params, 1 pfg_segment, 2 pfg_heat_params, 3 pfg_clock, 4 pfg_diag,
 * 5 pfg_quench, 6 pfg_batch_job, 7 pfg_grain, 8 pfg_point_source,
 * 9 pfg_point_sources, 10 pfg_interp, 11 pfg_cfd_grid, 12 pfg_linclip,
 * 13 pfg_cfd_energy, 14 pfg_cfd_flow, 15 pfg_cfd_stats. */
int64_t pfg_struct_size(int which);

/* Kernel selection for the stencil steps (process-wide; all compute the same
 * update):
 *  0 (default) the TMA-fed kernel when num_oris % 4 == 0, else the
 *    cp.async warp-per-cells kernel when num_oris / VEC <= 32 (VEC = 4, 2 or
 *    1: the largest width dividing num_oris), else the generic kernel;
 *  1 always the generic kernel;
 *  2 the cp.async warp-per-cells kernel where it applies, else generic;
 *  3 the same order as 0. */
int pfg_set_kernel_variant(int variant);

/* The device error flag: 0, or PFG_ERR_TIMEOUT once a bounded device-side
 * wait of a stencil kernel ran out (the kernel then stopped early and its
 * output is invalid).  Synchronises with the device.  clear != 0 resets it. */
int pfg_device_error(int clear);

/* Tile-plan overrides of the warp-per-cells kernel for tuning sweeps
 * (value 0 restores the automatic choice): key 0 = warps along x (1 .. 16),
 * 1 = rows per warp (1..32), 2 = shared-memory plane slots (4..6),
 * 3 = z chunks per tile column, 5 = consumer threads of the TMA-fed kernel
 * (256: two CTAs per SM; 512: one larger CTA per SM), 6 = cells per thread of
 * the CFD solver's kernels (1..16, default 4), 7 = 1 to run the TMA-fed
 * kernel's compile-time plans (pfg_fixed_plan) through its run-time-plan
 * instance instead, 8 = the wait probe (cycles; 0 = off): each CTA of the
 * TMA-fed and cell-per-lane kernels first waits that long on a barrier that
 * nothing completes, so the launch takes its timeout path (the CTA waits for
 * its copies in flight and returns; PFG_ERR_TIMEOUT in pfg_device_error)
 * without any fault; its output is then invalid.  Process-wide; the stencil
 * steps' results do not change; the CFD solver's dot products are summed in
 * another order (float64 rounding only). */
int pfg_tune(int key, int value);

/* The launch plan a step with these parameters would use on the current
 * device, as 12 int32: kernel, VEC, lanes per
 * cell, tile x, tile y, warps along x, rows per warp, plane slots, planes per
 * unit, CTAs, dynamic shared memory bytes, SM count.  kernel: 1 generic,
 * 2 cp.async warp-per-cells, 3 TMA-fed, 4 cell-per-lane (one cell per
 * lane: a warp owns 8 x 4 cells, so warps along x = tile x / 8 and rows per
 * warp = 4). */
int pfg_describe_plan(const pfg_pf_params* p, int32_t* out);

/* Which compile-time tile plan the TMA-fed kernel runs for these parameters
 * on the current device: 1 (num_oris = 20, 24 x 10 tiles), 2 (num_oris = 30,
 * 16 x 9 tiles), or 0 (the plan is read at run time; also when another
 * kernel runs).  A negative value is -pfg_status. */
int pfg_fixed_plan(const pfg_pf_params* p);

/* ---- phase field --------------------------------------------------------
 * One explicit Euler step of the Allen-Cahn grain-growth model with the
 * temperature held at T (the start-of-step value):
 *   eta_out = eta_in + dt * rhs(eta_in, T).
 * Replaces explicit_euler + state_rhs (allen_cahn.py:53-85, 106-114) as
 * called by PFSolver.stepper (allen_cahn.py:139-143).  T is (nz, ny, nx). */
int pfg_pf_step(const pfg_pf_params* p, const float* eta_in, float* eta_out,
                const float* T, float dt, void* stream);

/* The same step with T taken from the moving gradient q at the start-of-step
 * time clk_in->t (the solidification driver refreshes T after each step,
 * solidification/example.py:84-86), evaluated per z plane inside the kernel
 * so no temperature array is read.  Writes clk_out = {t + dt, step + 1};
 * clk_out must not alias clk_in. */
int pfg_pf_step_quench(const pfg_pf_params* p, const pfg_quench* q, const float* eta_in,
                       float* eta_out, const pfg_clock* clk_in, pfg_clock* clk_out, float dt,
                       void* stream);

/* The same step with T from the moving point source at the start-of-step
 * step count (the drivers refresh T after each step, simple/example.py:
 * 62-66, multi_scan/example.py:103-106), evaluated per cell inside the
 * kernel so that no temperature array exists.  Writes clk_out = {t + dt,
 * step + 1}; clk_out must not alias clk_in. */
int pfg_pf_step_point_source(const pfg_pf_params* p, const pfg_point_sources* src,
                             const float* eta_in, float* eta_out, const pfg_clock* clk_in,
                             pfg_clock* clk_out, float dt, void* stream);
/* The (nz, ny, nx) temperature that pfg_pf_step_point_source uses for a step
 * starting at clk (what the drivers pass to inspect_sol and write_sols). */
int pfg_point_source_T(const pfg_pf_params* p, const pfg_point_sources* src,
                       const pfg_clock* clk, float* T_out, void* stream);

/* The same step with T interpolated in time between T_past and T_future
 * (both (nz, ny, nx), the phase-field cell order) at the end-of-step time,
 * per cell inside the kernel (coupled/example.py:38-42,108-109).  Writes
 * clk_out = {t + dt, step + 1}; clk_out must not alias clk_in. */
int pfg_pf_step_interp(const pfg_pf_params* p, const pfg_interp* w, const float* T_past,
                       const float* T_future, const float* eta_in, float* eta_out,
                       const pfg_clock* clk_in, pfg_clock* clk_out, float dt, void* stream);
/* A temperature field of a solver that orders cells (nx, ny, nz), z fastest
 * (the CFD solver's T[:, :, :, 0]), into the phase-field order (nz, ny, nx):
 * the coupled driver's convert_temperature (coupled/example.py:31-36). */
int pfg_transpose_xyz(int32_t nx, int32_t ny, int32_t nz, const float* T_xyz, float* T_zyx,
                      void* stream);

/* ---- heat ----------------------------------------------------------------
 * One explicit heat step on the ghosted field, beam at (xl, yl) with the
 * given power.  Replaces gamma.update_T (gamma.py:55-61).  Tg_in and Tg_out
 * are ghosted in h->layout (either order); interior cells and the six ghost
 * faces of Tg_out are written, edge/corner ghosts are left untouched. */
int pfg_heat_step(const pfg_heat_params* h, const float* Tg_in, float* Tg_out,
                  float xl, float yl, float power, float dt, void* stream);

/* ---- fused heat + phase field -------------------------------------------
 * One pass that reads eta and the ghosted temperature and writes both:
 *   eta_out = eta_in + dt * rhs(eta_in, T_in interior)     (phase field at the
 *             start-of-step temperature, as the reference drivers do)
 *   Tg_out  = update_T(Tg_in) with the beam taken from h->path at the
 *             mid-step time clk_in->t + dt/2.
 * The clock is read from clk_in and clk_out = {t + dt, step + 1} is written,
 * so alternating (in, out) buffers inside a CUDA graph advance time on the
 * device.  The grids of p and h must agree. */
int pfg_heat_pf_step(const pfg_pf_params* p, const pfg_heat_params* h,
                     const float* eta_in, float* eta_out,
                     const float* Tg_in, float* Tg_out,
                     const pfg_clock* clk_in, pfg_clock* clk_out,
                     float dt, void* stream);

/* The same fused step with a compensated temperature: the ghosted field is
 * held as two float32 arrays whose sum is the temperature (Tg + Tlo, |Tlo|
 * at most half an ulp of Tg; start from Tlo = 0), and the heat update is
 * evaluated in double-float arithmetic (pairs of float32) wherever the
 * temperature is far from ambient and on every domain face.  A float32
 * temperature rounds to ~1e-3 K per step at 1e4 K and drifts from a
 * float64 run by ~1e-2 K over 2000 steps of the laser-track workload; the
 * compensated one stays within ~2e-6 K (1.1e-6 K measured over those 2000
 * steps).  The phase field reads Tg, and zeta the exact pair.
 * The cell-per-lane kernel (num_oris = 20) evaluates the heat update inside
 * the stencil; where the TMA-fed kernel runs instead (num_oris a multiple of
 * 4, or even with even nx and Neumann x faces) the step is two launches: the
 * compensated heat update, then the phase field with the start-of-step
 * pair (both read only the old state; 16 more bytes of traffic per cell).
 * Otherwise PFG_ERR_PARAM (see pfg_heat_pf_step_comp_supported).  Tg_in/Tg_out
 * and Tlo_in/Tlo_out must not alias.  Same reference functions as
 * pfg_heat_pf_step (allen_cahn.py:106-114, gamma.py:9-61). */
int pfg_heat_pf_step_comp(const pfg_pf_params* p, const pfg_heat_params* h,
                          const float* eta_in, float* eta_out,
                          const float* Tg_in, const float* Tlo_in,
                          float* Tg_out, float* Tlo_out,
                          const pfg_clock* clk_in, pfg_clock* clk_out,
                          float dt, void* stream);
/* 1 if pfg_heat_pf_step_comp runs for these parameters on the current
 * device, 0 if not; a negative value is -pfg_status. */
int pfg_heat_pf_step_comp_supported(const pfg_pf_params* p);

/* ---- batched serving ------------------------------------------------------
 * Many independent directional-solidification solves (each with its own
 * grid, orientation count, parameters and step count) advanced together: one
 * pfg_batch_step launch advances every active job by one step, so a CUDA
 * graph of K launches (k = 0 .. K-1) replayed from the host advances all of
 * them by K steps.  No counterpart in the reference, which solves one
 * polycrystal per Python process (applications/phase_field/solidification/
 * example.py:63-90); each job's step is the reference's stepper with the
 * driver's moving gradient (pfg_pf_step_quench). */
typedef struct pfg_batch_job {
  pfg_pf_params params;  /* grid and physics of this job */
  pfg_quench quench;     /* its moving temperature gradient */
  float* eta[2];         /* device double buffer, each (nz, ny, nx, num_oris) */
  double t0;             /* simulation time at step 0 */
  float dt;              /* explicit Euler step */
  int32_t reserved;
  int64_t base_step;     /* steps completed before launch k = 0 of the next replay */
  int64_t target_steps;  /* the job's total step count */
} pfg_batch_job;

/* Bytes of an encoded table for num_jobs jobs (host and device copies). */
int64_t pfg_batch_table_bytes(int num_jobs);
/* Encode jobs into `table` (host memory, table_bytes long); the caller then
 * copies it to a device buffer of the same size.  total_units receives the
 * number of work units (CTA tasks) of one batched step. */
int pfg_batch_encode(const pfg_batch_job* jobs, int num_jobs, void* table, int64_t table_bytes,
                     int64_t* total_units);
/* Launch k of a replay: every job with base_step + k < target_steps takes
 * one step from eta[(base_step + k) & 1] into the other buffer, at time
 * t0 + (base_step + k) dt.  device_table: the encoded table in device
 * memory; the launch uses a work counter in its header and leaves it at zero
 * when it ends (launches on one table must not overlap).  The grid is fixed
 * (persistent CTAs), so the launch can be captured once and replayed while
 * the table's contents change.  Jobs are stored in the table by unit cost,
 * largest first, not in the caller's order. */
int pfg_batch_step(void* device_table, int k, void* stream);
/* Add k_steps to every job's base_step in the device table (the end of a
 * replay of k_steps launches), so replays need no host-side table writes. */
int pfg_batch_advance(void* device_table, int k_steps, void* stream);

/* ---- adjoint ----------------------------------------------------------------
 * Reverse-mode derivative of the fused heat + phase-field step, hand-written
 * (the reference differentiates with jax.grad; it has no adjoint of the coupled
 * run).  Given the forward state of step k (eta, Tg at time t) and the
 * adjoints of step k+1 (lam_in = dJ/d eta^{k+1}, Tb_in = dJ/d Tg^{k+1}, both
 * ghost faces and interior of the ghosted layout), writes lam_out = dJ/d eta^k
 * and Tb_out = dJ/d Tg^k (interior and the six ghost faces; the caller zeroes
 * edge/corner entries once) and adds this step's contributions to grads[0]
 * (dJ/d beam power) and grads[1] (dJ/d scan speed, with dxl_dv = d x_beam / d v
 * at the mid-step time).  scratch: pfg_adjoint_scratch_bytes(p) bytes. */
int64_t pfg_adjoint_scratch_bytes(const pfg_pf_params* p);
int pfg_adjoint_step(const pfg_pf_params* p, const pfg_heat_params* h, const float* eta,
                     const float* Tg, double t, float dt, const float* lam_in, const float* Tb_in,
                     float* lam_out, float* Tb_out, void* scratch, int64_t scratch_bytes,
                     double* grads, float dxl_dv, void* stream);
/* Objective of the differentiable run: J += mean over cells of
 * sum_i w_i eta_i^2 (float64 accumulation into *J, which the caller zeroes),
 * and, if lam_seed is not NULL, dJ/d eta = 2 w_i eta_i / N. */
int pfg_objective(const pfg_pf_params* p, const float* eta, const float* w, double* J,
                  float* lam_seed, void* stream);

/* ---- grain segmentation ---------------------------------------------------
 * The grains of a solution, as the reference's post-processing finds them
 * (jax_am/phase_field/utils.py:181-310: compute_edges_in_order, BFS,
 * get_aspect_ratio_inputs): two face-adjacent cells (no wrap) are in the same
 * grain when both are solid (T < T_liquidus) and have the same orientation
 * index.  Each grain record carries the exact integer moments of its cells'
 * (x, y, z) indices; volume = cells * hx * hy * hz and the PCA aspect ratio
 * (utils.py:286-310) follow from them on the host.
 *  ori:           (nz, ny, nx) int32 orientation index per cell (the argmax
 *                 map, e.g. argmax_out of pfg_pf_diag).
 *  T:             per-cell (nz, ny, nx) when T_ghosted == 0, else the ghosted
 *                 heat state.
 *  grain_of_cell: (nz, ny, nx) int32 grain number per cell (-1 liquid), or NULL.
 *  grains:        device array of max_grains records, 8-byte aligned; grain g is
 *                 the g-th grain in increasing order of its smallest cell index
 *                 (the reference lists grains by orientation first, then in this
 *                 order: sort the records by (ori, first_cell)).
 *  num_grains:    device int64 receiving the number of grains; when it exceeds
 *                 max_grains only the first max_grains records are filled and
 *                 grain_of_cell may hold numbers >= max_grains: call again with
 *                 a larger array.
 *  scratch:       device buffer of at least pfg_grain_scratch_bytes(p) bytes.
 * Fewer than 2^31 - 2^22 cells. */
typedef struct pfg_grain {
  int64_t first_cell;  /* smallest cell index of the grain (where the reference's search starts it) */
  int32_t ori;         /* its orientation index */
  int32_t reserved;
  int64_t cells;       /* number of cells */
  int64_t sum[3];      /* sums of the cells' x, y, z indices */
  int64_t sum2[6];     /* sums of xx, yy, zz, xy, xz, yz */
} pfg_grain;
int64_t pfg_grain_scratch_bytes(const pfg_pf_params* p);
int pfg_grains(const pfg_pf_params* p, const int32_t* ori, const float* T, int T_ghosted,
               int32_t* grain_of_cell, pfg_grain* grains, int64_t max_grains, int64_t* num_grains,
               void* scratch, int64_t scratch_bytes, void* stream);

/* ---- diagnostics ----------------------------------------------------------
 * The metrics PFSolver.inspect_sol prints (allen_cahn.py:165-180) plus the
 * free energy and per-orientation mass, reduced on the device.  The mass is
 * a compensated (error-free) sum returned as float64; the energy sums
 * float32 per-cell energy densities (relative error ~1e-7 per cell) with
 * compensated accumulation.  Fewer than 2^31 cells.
 *  T:         per-cell (nz, ny, nx) when T_ghosted == 0, else the ghosted
 *             (nz+2, ny+2, nx+2) heat state.
 *  argmax0:   (nz, ny, nx) int32 reference orientation map, or NULL (then
 *             n_ori_changed is 0).
 *  argmax_out:(nz, ny, nx) int32 argmax orientation per cell (first maximum,
 *             all-zero cells give 0, as np.argmax), or NULL.
 *  scratch:   device buffer of at least pfg_pf_diag_scratch_bytes(p) bytes.
 *  out:       device pointer to one pfg_diag. */
int64_t pfg_pf_diag_scratch_bytes(const pfg_pf_params* p);
int pfg_pf_diag(const pfg_pf_params* p, const float* eta, const float* T, int T_ghosted,
                const int32_t* argmax0, int32_t* argmax_out,
                void* scratch, int64_t scratch_bytes, pfg_diag* out, void* stream);

/* Only the metrics of PFSolver.inspect_sol (allen_cahn.py:165-180): argmax
 * changes, liquid cells, max T, non-finite count and the argmax map; energy
 * and mass are returned as 0.  Same arguments and scratch as pfg_pf_diag;
 * one read of eta and no per-orientation sums. */
int pfg_pf_inspect(const pfg_pf_params* p, const float* eta, const float* T, int T_ghosted,
                   const int32_t* argmax0, int32_t* argmax_out, void* scratch,
                   int64_t scratch_bytes, pfg_diag* out, void* stream);

/* ---- diagnostics without allocation -------------------------------------
 * No counterpart in the reference.  The same results as pfg_pf_diag for
 * callers that can neither call cudaMalloc nor pass a scratch buffer: a host
 * framework that owns all device memory and gives a plugin only the buffers
 * it planned in advance (for example an XLA custom call), or a fixed-budget
 * real-time loop.  The per-block partial sums live in a static device array
 * of PFG_DIAG_NOALLOC_RECORDS records (165,760 bytes) that every GPU loading
 * the library holds until the process exits.
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current; make that first call
 *    before any stream capture.  The address is kept for the life of the
 *    process, so do not reset the device (cudaDeviceReset, or a reset of
 *    its primary context) while the library is loaded: the array would move
 *    and the kept address would point at freed memory.
 *  - Every call on a device shares the one array: calls whose work overlaps
 *    on the GPU (different streams, no ordering between them) race and give
 *    wrong results.  Order them on one stream or with events.
 *  - A parameter set whose reduction needs more records than the array holds
 *    returns PFG_ERR_CAPACITY (the reduction uses at most 296 blocks, so any
 *    grid size fits today).
 * Inputs and outputs are as for pfg_pf_diag; the caller still owns them. */
#define PFG_DIAG_NOALLOC_RECORDS 296
int pfg_pf_diag_noalloc(const pfg_pf_params* p, const float* eta, const float* T, int T_ghosted,
                        const int32_t* argmax0, int32_t* argmax_out, pfg_diag* out,
                        void* stream);

/* ---- implicit CFD / energy solver (jax_am/cfd/cfd_am.py, AM_3d) ----------
 * The finite-volume solver the reference's coupled and CFD drivers advance
 * (applications/phase_field/coupled/example.py:81-111,
 * applications/cfd/simple/example.py:44-55): per time step an implicit
 * energy solve (Newton + Jacobi-preconditioned BiCGSTAB), then inside a local
 * box that follows the laser a projection-method velocity solve (three
 * momentum solves with Darcy damping and Marangoni shear, a pressure
 * Poisson) and the explicit convective terms for the next step.
 *  - float64 throughout (the reference enables jax_enable_x64, cfd_am.py:10).
 *  - Fields are (nx, ny, nz) C order, z fastest -- the reference's
 *    (Nx, Ny, Nz, 1) arrays; vel, conv and grad_p0 are (nx, ny, nz, 3).
 *  - The solves are iterative with data-dependent iteration counts, so these
 *    entry points synchronise with `stream` to read convergence flags (a few
 *    bytes per chunk of iterations); they return when the step's results
 *    are complete on the device.
 *  - `ws` is caller-owned device scratch of pfg_cfd_workspace_bytes() bytes,
 *    8-byte aligned; its contents are not preserved between calls. */
typedef struct pfg_cfd_grid {
  int32_t nx, ny, nz, pad;
  double dx, dy, dz;             /* cell size: domain / N (cfd_am.py:677-679) */
  double lx, ly, lz;             /* domain lengths: the last mesh node (cfd_am.py:672-674) */
} pfg_cfd_grid;

typedef struct pfg_linclip {     /* a * clip(T, lo, hi) + b: the drivers' cp(T) and k(T) */
  double a, b, lo, hi;
} pfg_linclip;

typedef struct pfg_cfd_energy {  /* energy_eqn + AM_3d's energy boundary condition */
  pfg_linclip cp, k;
  double rho, latent_heat, Ts, Tl, dt;
  double T_ref, h_conv, emissivity, sigma;  /* top face: -h (T - T_ref) - sigma eps (T^4 - T_ref^4) */
  int32_t heat_source;           /* 0: Gaussian surface flux, 1: Gaussian cylinder body source */
  int32_t max_newton;            /* solver_nonlinear max_it (50) */
  double P, eta, rb, phi, speed; /* laser power (already 0 after t_OFF), absorptivity, radius, ... */
  double xl, yl, zl;             /* beam position at the step's time (AM_3d.toolpath) */
  double newton_tol;             /* solver_nonlinear tol (1e-5) */
} pfg_cfd_energy;

typedef struct pfg_cfd_flow {    /* velocity_eqn + AM_3d's moving box */
  double rho, visco, dt, marangoni, Ts, Tl;
  int32_t x0, y0, z0, pad;       /* the local box's origin in the global grid */
} pfg_cfd_flow;

typedef struct pfg_cfd_stats {   /* iteration counts of the last call (-10/-11: breakdown) */
  int32_t newton_iters, pad;
  int64_t energy_krylov;         /* BiCGSTAB iterations summed over the Newton steps */
  int64_t momentum_krylov[3];
  int64_t pressure_krylov;
} pfg_cfd_stats;

/* Scratch bytes for a global grid and a local box (either solve). */
int64_t pfg_cfd_workspace_bytes(const pfg_cfd_grid* global, const pfg_cfd_grid* local);

/* energy_eqn.update + solver_nonlinear (cfd_am.py:516-525, 780-812) with
 * AM_3d's boundary condition and heat source at the step's time
 * (cfd_am.py:223-235, 325-358): T_out = the new temperature from T0 (the
 * previous one; its top layer gives the radiation/convection flux) and the
 * explicit convection conv_T. */
int pfg_cfd_energy_solve(const pfg_cfd_grid* g, const pfg_cfd_energy* e, const double* T0,
                         const double* conv_T, double* T_out, void* ws, int64_t ws_bytes,
                         pfg_cfd_stats* stats, void* stream);

/* solidID = max(solidID, fluid fraction of T) (cfd_am.py:172-175, 360-363). */
int pfg_cfd_solid_update(const pfg_cfd_grid* g, double Ts, double Tl, const double* T,
                         double* solidID, void* stream);

/* velocity_eqn.update on the local box at f->x0/y0/z0 (cfd_am.py:557-590,
 * 287-323) followed by update_convective_terms (cfd_am.py:254-259): reads T
 * and the box's vel, conv and grad_p0 from the global arrays, writes the
 * box's vel, grad_p0, conv and conv_T back.  The convective terms use the
 * global cell size, the solves the local box's (as the reference does). */
int pfg_cfd_flow_step(const pfg_cfd_grid* global, const pfg_cfd_grid* local,
                      const pfg_cfd_flow* f, const double* T, double* vel, double* conv,
                      double* grad_p0, double* conv_T, void* ws, int64_t ws_bytes,
                      pfg_cfd_stats* stats, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PF_GB300_H */
