/*
 * lbm_gb300.h - C ABI of the GB300 (sm_103a) D3Q19 stream-and-collide solver.
 *
 * This is the boundary a host binding (ctypes, cuda-python, cffi) calls in
 * place of tack-lbm's Tack-compiled kernels and its Solver plumbing. It takes
 * plain pointers and sizes only; every function returns an lbm_status and
 * never throws. lbm_last_error() gives a message for the last failure on the
 * calling thread.
 *
 * Populations live on the GPU in one structure-of-arrays buffer that is
 * updated in place (AA pattern), so there is no A/B pair to swap. Host-side
 * exchange of populations always uses the reference layout f[q*n + idx],
 * idx = (z*ny + y)*nx + x (lbm.py:397-402, lbm.py:426), whatever storage
 * precision is used on the device.
 *
 * Reference interfaces replaced (paths inside the tack-lbm project):
 *   lbm_create/lbm_destroy  Solver.__init__ buffers and composition (lbm.py:551-584)
 *   lbm_init                lbm_init kernel (lbm.py:383-394)
 *   lbm_step                Solver.step -> lbm_step kernel + buffer swap (lbm.py:639-647, 397-513)
 *   lbm_monitors            Solver.monitors (lbm.py:649-661)
 *   lbm_field               ManagedArray fields (lbm.py:525-541, 567)
 *   lbm_set_physics         Solver.set_physics (lbm.py:613-616)
 *   lbm_set_obstacle        Solver.set_obstacle (lbm.py:628-637)
 *   lbm_set_actuation       Solver.set_actuation / omega_rot (lbm.py:618-624)
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lbm_status {
    LBM_OK = 0,
    LBM_ERR_ARG = 1,        /* bad argument: unknown model/obstacle (the reference's KeyError), bad size */
    LBM_ERR_CUDA = 2,       /* a CUDA call failed (the reference's RuntimeError, lbm.py:533-534) */
    LBM_ERR_NONFINITE = 3,  /* a monitor sum is NaN or Inf: the run diverged (collision_check.py:19) */
    LBM_ERR_STATE = 4       /* call not valid in the solver's current state */
} lbm_status;

/* collision models: the COLLISIONS registry (lbm.py:544) */
enum { LBM_BGK = 0, LBM_TRT = 1, LBM_LES = 2 };
/* obstacles (lbm.py:144-276); LBM_NO_OBSTACLE has no solid cell; LBM_HEATSINK is the
 * finned sink on the floor of a duct with walls at y = 0 and y = ny - 1 (HeatSink) */
enum { LBM_NO_OBSTACLE = 0, LBM_CYLINDER = 1, LBM_SPHERE = 2, LBM_BOX = 3, LBM_HEATSINK = 4 };
/* temperature fields of a heat run (Solver.heat_fields, lbm.py:586-604): the solid's
 * temperature (input), the summed fluid temperature on each wetted sink voxel, the
 * temperature (report steps) */
enum { LBM_T_SOLID = 0, LBM_Q_SOLID = 1, LBM_TEMP = 2, LBM_NUM_HEAT_FIELDS = 3 };
/* output grid fields: ux, uy, uz, p, vmag, and temp when the run has heat */
enum { LBM_OUT_TEMP = 5, LBM_MAX_OUTPUTS = 6 };
/* y boundaries: PeriodicY / SlipY (lbm.py:342-369); LID adds a moving no-slip top wall (new) */
enum { LBM_PERIODIC = 0, LBM_SLIP = 1, LBM_LID = 2 };
/* population storage on the device: FP32, FP16/BF16 deviations f - w_q, FP64 (oracle runs) */
enum { LBM_F32 = 0, LBM_F16 = 1, LBM_BF16 = 2, LBM_F64 = 3 };
/* diagnostic fields, in the reference's FIELDS order (lbm.py:545) */
enum {
    LBM_UX = 0, LBM_UY, LBM_UZ, LBM_P, LBM_VMAG, LBM_R_RHO, LBM_R_UX, LBM_R_UY, LBM_R_UZ,
    LBM_R_KE, LBM_FX, LBM_FY, LBM_FZ, LBM_NUM_FIELDS
};
/* lbm_monitors output order: the keys of Solver.monitors (lbm.py:655-660) */
enum {
    LBM_MON_CONTINUITY = 0, LBM_MON_MOMENTUM_X, LBM_MON_MOMENTUM_Y, LBM_MON_MOMENTUM_Z,
    LBM_MON_ENERGY, LBM_MON_DRAG, LBM_MON_LIFT, LBM_NUM_MONITORS
};
/* where a host/device buffer lives */
enum { LBM_HOST = 0, LBM_DEVICE = 1 };

typedef struct lbm_config {
    int32_t nx, ny, nz;          /* lattice (lbm.py:42-44) */
    int32_t collision;           /* LBM_BGK | LBM_TRT | LBM_LES */
    int32_t obstacle;            /* LBM_NO_OBSTACLE | LBM_CYLINDER | LBM_SPHERE | LBM_BOX */
    int32_t lateral;             /* y: LBM_PERIODIC | LBM_SLIP | LBM_LID */
    int32_t vertical;            /* z: LBM_PERIODIC | LBM_SLIP (the reference is periodic, lbm.py:415) */
    int32_t storage;             /* LBM_F32 | LBM_F16 | LBM_BF16 | LBM_F64 */
    double nu;                   /* kinematic viscosity, tau0 = 3 nu + 1/2 (lbm.py:63, 110, 131) */
    double cs;                   /* Smagorinsky constant for TRT/LES (reference: 0.16, lbm.py:107, 128) */
    double magic;                /* TRT magic parameter (reference: 0.1875, lbm.py:106) */
    double ox, oy, oz;           /* obstacle centre (lbm.py:630-637) */
    double r;                    /* cylinder/sphere radius */
    double hx, hy, hz;           /* box half sizes */
    double u0;                   /* inflow / sponge target velocity (lbm.py:372-380) */
    double sponge_start;         /* first sponge plane, reference 0.75 nx (lbm.py:561) */
    double sponge_strength;      /* reference 1.0 */
    double u_lid;                /* x velocity of the LBM_LID top wall */
    double omega_rot;            /* cylinder surface speed (lbm.py:618-620) */
    int32_t device;              /* CUDA device ordinal */
    int32_t flags;               /* LBM_FLAG_* */
    /* LBM_HEATSINK geometry in cells, the HeatSink arguments (lbm.py:235-244)
     * Solver.set_obstacle passes (lbm.py:635-637): x0, length, z0, width, base,
     * fin_height, fin_thickness, fin_pitch */
    double sink[8];
    /* heat != 0 adds the D3Q7 temperature (lbm.py:457-492; FP32 storage and the
     * per-cell kernels only): alpha is the molecular diffusivity, heat_nu the
     * viscosity its subgrid part subtracts (Heat(arrays, nu/prandtl, nu), lbm.py:596-599) */
    int32_t heat;
    int32_t reserved;
    double alpha;
    double heat_nu;
} lbm_config;

/* lbm_config.flags: LBM_FLAG_BULKCOPY selects the bulk-copy (TMA) staged step
 * kernel instead of the default per-cell kernel; it needs rows that split into
 * 16-byte pieces (nx*sizeof(storage) % 16 == 0), otherwise the per-cell kernel
 * runs. LBM_FLAG_SIMT asks for the per-cell kernel explicitly. */
#define LBM_FLAG_SIMT 1
#define LBM_FLAG_BULKCOPY 2
/* LBM_FLAG_SLOT_POINTERS keeps the populations in 19 slot rows of n cells
 * and makes the per-cell step kernels address them through 19 pointers, as
 * they must when 32-bit element offsets do not reach (19 n >= 2^32).
 * Otherwise FP32, FP16 and BF16 populations sit in 32-cell blocks of 19
 * slots and FP64 populations in slot rows, both addressed by 32-bit offsets
 * from one base pointer (faster). The results are the same either way;
 * lbm_get/set_populations always exchange the reference layout
 * f[q*n + idx]. */
#define LBM_FLAG_SLOT_POINTERS 4

typedef struct lbm_solver lbm_solver;

/* Create a solver: validate cfg, allocate the population buffer (device
 * memory) and the 13 diagnostic fields (CUDA managed memory, zeroed, stable for
 * the handle's lifetime so Conduit/NumPy may alias them). Populations are
 * undefined until lbm_init / lbm_init_random / lbm_set_populations.
 * Replaces Solver.__init__ allocation and composition (lbm.py:551-584). */
lbm_status lbm_create(const lbm_config *cfg, lbm_solver **out);
lbm_status lbm_destroy(lbm_solver *s);

/* Equilibrium at rho = 1, u = (u0*fluid, seed_amp*u0*fluid*sin(2 pi x/nx)*cos(2 pi z/nz), 0)
 * (lbm_init, lbm.py:383-394). Resets the step counter. */
lbm_status lbm_init(lbm_solver *s, double seed_amp);

/* Equilibrium at rho = 1 + rho_sigma*N(0,1), u = (u0, 0, 0) + U(-u_noise, u_noise)^3 in
 * fluid cells, rest elsewhere, from a counter-based generator keyed by seed.
 * (No reference counterpart: the configurations' seeded start states.) */
lbm_status lbm_init_random(lbm_solver *s, double rho_sigma, double u_noise, uint64_t seed);

/* One step of the fused stream-collide kernel; report != 0 also writes the 13
 * fields and the FP64 monitor sums (lbm_step with Report, lbm.py:493-513).
 * Asynchronous on `stream` (a cudaStream_t; NULL = the legacy default stream).
 * Replaces Solver.step (lbm.py:639-647). */
lbm_status lbm_step(lbm_solver *s, int32_t report, void *stream);

/* `count` quiet steps, the last one a report step when report_last != 0. Pairs
 * of quiet steps are launched as one CUDA graph (captured once per parity and
 * kept until an argument of the step changes: lbm_set_physics, lbm_set_sponge,
 * lbm_set_actuation, lbm_set_obstacle, lbm_set_sink); not while lbm_timing is on. */
lbm_status lbm_run(lbm_solver *s, int32_t count, int32_t report_last, void *stream);

/* Synchronise and return the monitors of the last report step, in
 * LBM_MON_* order: residuals sqrt(sum/n)/max(interval,1) and drag/lift
 * sum(f)/(0.5 u0^2 diameter nz) (Solver.monitors, lbm.py:649-661). The sums
 * are reduced on the GPU in FP64; no field page is touched by the host.
 * Returns LBM_ERR_NONFINITE (with the values filled in) when a sum is not finite. */
lbm_status lbm_monitors(lbm_solver *s, int32_t interval, double diameter, double out[7]);

/* The raw FP64 sums of the last report step: r_rho, r_ux, r_uy, r_uz, r_ke, fx, fy, fz. */
lbm_status lbm_field_sums(lbm_solver *s, double out[8]);

/* Managed pointer to field `id` (n floats), valid until lbm_destroy (lbm.py:525-541). */
lbm_status lbm_field(lbm_solver *s, int32_t id, float **ptr);

/* Change collision model and viscosity; cs < 0 keeps the current constant (lbm.py:613-616). */
lbm_status lbm_set_physics(lbm_solver *s, int32_t collision, double nu, double cs);

/* Change the obstacle: geo = {ox, oy, oz, r, hx, hy, hz} (LBM_HEATSINK takes its
 * geometry from lbm_config.sink). The populations are carried over as the
 * reference does (lbm.py:628-637). */
lbm_status lbm_set_obstacle(lbm_solver *s, int32_t kind, const double geo[7]);

/* Set the heat-sink geometry (lbm_config.sink order); when the obstacle is
 * LBM_HEATSINK the new sink takes effect as lbm_set_obstacle would. */
lbm_status lbm_set_sink(lbm_solver *s, const double sink[8]);

/* Cylinder surface speed, stream-ordered with the steps (lbm.py:618-624). */
lbm_status lbm_set_actuation(lbm_solver *s, double omega_rot);
lbm_status lbm_get_actuation(lbm_solver *s, double *omega_rot);

/* Sponge start plane and strength (Flow, lbm.py:372-380). */
lbm_status lbm_set_sponge(lbm_solver *s, double start, double strength);

/* Copy populations in/out in the reference layout f[q*n + idx] (19*n values).
 * dtype: LBM_F32 or LBM_F64 values; where: LBM_HOST or LBM_DEVICE pointer.
 * lbm_set_populations leaves the solver at the start of a step; solid cells
 * read back as w_q, the value every reference step gives them (lbm.py:449-456). */
lbm_status lbm_set_populations(lbm_solver *s, const void *f, int32_t dtype, int32_t where);
lbm_status lbm_get_populations(lbm_solver *s, void *f, int32_t dtype, int32_t where);

/* Output grid: the fields ux, uy, uz, p, vmag subsampled by `stride` along each
 * axis, (d + stride - 1)/stride points per axis, in managed memory
 * (lbm.py:574-581). stride 1 aliases the full-resolution fields. */
lbm_status lbm_set_output_stride(lbm_solver *s, int32_t stride);
/* Managed pointer to output field `id` (LBM_UX .. LBM_VMAG, LBM_OUT_TEMP with heat)
 * and its point count. */
lbm_status lbm_output(lbm_solver *s, int32_t id, float **ptr, int64_t *count);
/* Copy output field `id` into `host` (its point count of floats; pinned host memory
 * makes it an asynchronous copy-engine transfer) on `stream`, ordered after the
 * steps and lbm_update_output on that stream. For consumers that want a host copy
 * rather than reading the managed field in place. (No reference counterpart.) */
lbm_status lbm_read_output(lbm_solver *s, int32_t id, float *host, void *stream);

/* Refresh the output fields from the full-resolution ones: the coarsen kernel
 * (lbm.py:516-522) for every output field (Solver.update_output, lbm.py:606-611). */
lbm_status lbm_update_output(lbm_solver *s, void *stream);

/* Velocity gradient on the output grid (derived.py:52-89): jac receives 9 floats
 * per output point, jac[9 p + 3 c + d] = d u_c / d x_d, central differences and
 * one-sided at the grid's faces, scaled by inv_h (the reference passes
 * diameter / stride, derived.py:101-103). Reads the output fields as the last
 * lbm_update_output left them. jac: device or managed memory. */
lbm_status lbm_velocity_gradient(lbm_solver *s, float *jac, double inv_h, void *stream);

/* |curl u| and the Q-criterion -1/2 J_ij J_ji from such a gradient (the default
 * derived fields, derived.py:27-30), one value per output point (at_cells = 0)
 * or per cell centre (at_cells = 1: (mx-1)(my-1)(mz-1) values from the mean of
 * the eight corner gradients). Either output may be NULL. */
lbm_status lbm_vorticity_q(lbm_solver *s, const float *jac, float *vorticity, float *q, int32_t at_cells,
                           void *stream);

/* The same two fields straight from the output grid's velocity, with no
 * gradient buffer: the gradient of lbm_velocity_gradient (inv_h as there) is
 * formed where it is used, so the results equal lbm_velocity_gradient
 * followed by lbm_vorticity_q bit for bit (derived.py:27-30, 52-89).
 * Either output may be NULL. */
lbm_status lbm_vorticity_q_direct(lbm_solver *s, double inv_h, float *vorticity, float *q, int32_t at_cells,
                                  void *stream);

/* Overwrite one diagnostic field from a buffer of n floats (host or managed). */
lbm_status lbm_set_field(lbm_solver *s, int32_t id, const float *host);

/* Solid mask (1 inside the obstacle) as n bytes on the host. */
lbm_status lbm_mask(lbm_solver *s, uint8_t *host_out);

/* Number of steps taken since the last init / set_populations. */
lbm_status lbm_step_count(lbm_solver *s, int64_t *count);

/* Device bytes held by the solver (populations + fields + scratch). */
lbm_status lbm_memory(lbm_solver *s, int64_t *bytes);

/* A zeroed CUDA managed float array of `count` elements, readable from the
 * host and the GPU (ManagedArray, lbm.py:525-541); free with lbm_managed_free. */
lbm_status lbm_managed_alloc(int64_t count, float **ptr);
lbm_status lbm_managed_free(float *ptr);

/* Kernel timing: when enabled, every step records CUDA events on the launching
 * stream around the main step kernel (step_kernel, or stream_kernel with
 * LBM_FLAG_BULKCOPY) and after the step's remaining work (the lid rows'
 * general_kernel joined from its side stream, the monitor sums on report
 * steps). lbm_timing_read synchronises and returns {main kernel ms total, main
 * kernel launches, cells per main launch, ms total of the rest, its launches,
 * cells per general_kernel launch, ms from the first timed step's start to the
 * last one's end} since the last enable (at most 4096 steps are timed).
 * (No reference counterpart: measurement support.) */
lbm_status lbm_timing(lbm_solver *s, int32_t enable);
lbm_status lbm_timing_read(lbm_solver *s, double out[7]);

/* lbm_run between two CUDA events on `stream`; *ms = their elapsed time
 * (synchronous). (No reference counterpart: measurement support.) */
lbm_status lbm_run_timed(lbm_solver *s, int32_t count, int32_t report_last, void *stream, double *ms);

/* Synchronise the solver's device work (tack.sync, lbm.py:651). Returns
 * LBM_ERR_CUDA when a bulk-copy step gave up waiting for its copies since the
 * last check (the populations are then invalid), and clears that state. */
lbm_status lbm_sync(lbm_solver *s);

/* Test hook of the bulk-copy kernel's bounded waits (LBM_FLAG_BULKCOPY): the
 * next lbm_step issues no copies, so every wait of its consumers runs out
 * after wait_polls polls. Nothing is read or written in HBM by that step; the
 * next lbm_sync returns LBM_ERR_CUDA. LBM_ERR_STATE for a solver without the
 * bulk-copy kernel; lbm_run refuses to run while the hook is pending.
 * (No reference counterpart: failure-path testing.) */
lbm_status lbm_test_bulkcopy_stall(lbm_solver *s, int64_t wait_polls);

/* Largest n accepted by lbm_field_sums_static: 2^28 cells. */
#define LBM_STATIC_SUMS_MAX_CELLS 268435456LL

/* The eight FP64 monitor sums (r_rho, r_ux, r_uy, r_uz, r_ke, fx, fy, fz, the
 * totals Solver.monitors turns into residuals and drag/lift) of caller-owned
 * report fields, WITHOUT ANY DEVICE ALLOCATION. There is no counterpart in the
 * reference. It exists for callers that cannot allocate device memory while
 * they run: an in-situ pipeline or host framework that owns every device
 * buffer and forbids allocation mid-run (cudaMalloc synchronises the device and
 * can fail under memory pressure), or a deployment with a fixed device
 * footprint. fields: 8 arrays of n floats the GPU can read (device or
 * managed memory); sums: 8 doubles the GPU can write. n must be in
 * [1, LBM_STATIC_SUMS_MAX_CELLS], otherwise LBM_ERR_ARG. Runs asynchronously on
 * `stream` of the current device. The per-block partial sums go to a static
 * 1 MiB device array that every GPU loading the library holds until exit; the
 * first call on a device looks up that array's address, so make it before any
 * stream capture. All calls share the array: calls that overlap on the GPU race. */
lbm_status lbm_field_sums_static(const float *const fields[8], int64_t n, double *sums, void *stream);

/* ---------------------------------------------------------------------------
 * Gradients of time-averaged drag (no reference counterpart).
 *
 * A differentiable form of the LES step: the cylinder along z is the smoothed
 * solid fraction phi = (1 + tanh((r - d)/width))/2 (d: distance to the axis
 * (ox, oy)), used wherever the reference step uses its 0/1 solid test
 * (bounce-back blend, momentum exchange, u = fluid j/rho, sponge sigma), all
 * boundaries periodic, start state lbm_init (lbm.py:383-394). Runs on its own
 * A/B population buffers in FP32 or FP64, holding the deviations f_q - w_q
 * from the float32 lattice weights, with the production step's pair-sum
 * arithmetic (the stress and the density keep their digits in FP32). The loss is
 *   L = sum_{t = loss_start..steps} F_x(t) / (N_l 0.5 U^2 diameter nz),
 * F_x(t) the momentum-exchange x force of step t, N_l the number of those
 * steps. lbm_adj_backward runs the hand-written adjoint kernel backwards over
 * the steps, recomputing each interval of `checkpoint` steps from the state
 * the forward run kept at its start, and returns dL/d(U, tau0, Cs, r).
 */
typedef struct lbm_adj_config {
    int32_t nx, ny, nz;
    int32_t precision;           /* LBM_F32 | LBM_F64: storage and arithmetic */
    int32_t steps;               /* steps of one forward run */
    int32_t loss_start;          /* first step (1-based) whose force enters the loss */
    int32_t checkpoint;          /* K: a state is kept every K steps */
    int32_t device;
    double u0, tau0, cs, r;      /* the parameters: inflow U, tau0 = 3 nu + 1/2, Cs, radius */
    double ox, oy, width;        /* cylinder axis and tanh width */
    double diameter;             /* length in the drag normalisation (a constant) */
    double sponge_start, sponge_strength;
    double seed_amp;             /* lbm_init's wave amplitude */
} lbm_adj_config;

typedef struct lbm_adj lbm_adj;

/* Allocate the run: (steps/K + 1) checkpoints, K - 1 recompute states and the
 * adjoint buffers, each 19 n values. */
lbm_status lbm_adj_create(const lbm_adj_config *cfg, lbm_adj **out);
lbm_status lbm_adj_destroy(lbm_adj *h);
/* par = {U, tau0, Cs, r}; invalidates the last forward run. */
lbm_status lbm_adj_set_params(lbm_adj *h, const double par[4]);
/* Forward run from the start state; the loss (synchronous). */
lbm_status lbm_adj_forward(lbm_adj *h, double *loss);
/* dL/d(U, tau0, Cs, r) of the last forward run (synchronous). */
lbm_status lbm_adj_backward(lbm_adj *h, double grad[4]);
/* The state after `step` steps (a multiple of K, or 0) as 19 n values f_q of
 * the run's precision in the layout f[q*n + idx], to a host buffer (the kept
 * deviations plus the weights, added in that precision). */
lbm_status lbm_adj_state(lbm_adj *h, int32_t step, void *host);
/* {forward ms, backward ms (CUDA events), sum of F_x over the loss steps, device bytes}. */
lbm_status lbm_adj_info(lbm_adj *h, double out[4]);

/* Managed pointer to heat field `id` (LBM_T_SOLID, LBM_Q_SOLID, LBM_TEMP; n floats),
 * valid until lbm_destroy. LBM_ERR_STATE when the run has no heat. Report steps zero
 * q_solid before they add to it (Solver.step, lbm.py:641-642). */
lbm_status lbm_heat_field(lbm_solver *s, int32_t id, float **ptr);

/* Copy the temperature populations in/out in the layout g[q*n + idx] (7*n values,
 * D3Q7 order of lbm.py:20-25). They start at zero (lbm.py:592). */
lbm_status lbm_set_heat_populations(lbm_solver *s, const void *g, int32_t dtype, int32_t where);
lbm_status lbm_get_heat_populations(lbm_solver *s, void *g, int32_t dtype, int32_t where);

/* ---------------------------------------------------------------------------
 * Pitch-plunge wing (tack-lbm flutter.py:20-130): a rigid NACA 0012 section
 * spanning z on a lattice periodic in x, y and z, moving with the plunge h
 * and pitch alpha about its elastic axis (x_ea, y_ea) at chord fraction ea.
 * The structure is integrated by the caller; every step takes the state
 * {h, alpha, dh/dt, dalpha/dt} and returns the momentum-exchange force and its
 * moment about the displaced elastic axis, summed over the lattice (not per
 * unit span). FP32 populations on A/B buffers.
 */
typedef struct lbm_wing_config {
    int32_t nx, ny, nz;
    int32_t collision;           /* LBM_BGK | LBM_TRT | LBM_LES */
    double nu, cs, magic;
    double chord, x_ea, y_ea, ea;
    double u0, sponge_start, sponge_strength;
    int32_t device;
    int32_t reserved;
} lbm_wing_config;

typedef struct lbm_wing lbm_wing;

lbm_status lbm_wing_create(const lbm_wing_config *cfg, lbm_wing **out);
lbm_status lbm_wing_destroy(lbm_wing *w);
/* wing_init (flutter.py:51-58): equilibrium at rho = 1, u = (u0 (1 - solid), 0, 0). */
lbm_status lbm_wing_init(lbm_wing *w, const double state[4]);
/* wing_step (flutter.py:61-130); report != 0 writes ux, uy, uz, p, vmag.
 * Synchronous: load = {fx, fy, mz}. */
lbm_status lbm_wing_step(lbm_wing *w, int32_t report, const double state[4], double load[3]);
lbm_status lbm_wing_set_physics(lbm_wing *w, int32_t collision, double nu);
/* Managed pointer to field id (0..4: ux, uy, uz, p, vmag; n floats). */
lbm_status lbm_wing_field(lbm_wing *w, int32_t id, float **ptr);
/* Copy the current populations (19 n floats, f[q*n + idx]) from (set = 0) or to (set = 1) `host`. */
lbm_status lbm_wing_populations(lbm_wing *w, float *host, int32_t set);
/* The solid mask (n bytes) at `state`: the section test of flutter.py:30-42 with
 * float64 results (a float32 prefilter decides the points away from the outline,
 * the rest run in float64), as every step uses it. */
lbm_status lbm_wing_mask(lbm_wing *w, const double state[4], uint8_t *host);
/* Output grid: the five fields subsampled by `stride` (flutter.py:207-211). */
lbm_status lbm_wing_set_output_stride(lbm_wing *w, int32_t stride);
lbm_status lbm_wing_output(lbm_wing *w, int32_t id, float **ptr, int64_t *count);
lbm_status lbm_wing_update_output(lbm_wing *w);

/* ---------------------------------------------------------------------------
 * Cantilever-wing FSI (tack-lbm fsi.py:25-186): an elastic NACA 0012 wing from
 * a mirror root plane below z = 0 to z = span; inflow at x = 0, outflow at
 * x = nx - 1, periodic y, mirror plane above z = nz - 1. Every step takes the
 * kinematics of each layer z, kin[4 z .. 4 z + 3] = {h, alpha, dh/dt, dalpha/dt},
 * and returns each layer's momentum-exchange force and moment,
 * load[3 z .. 3 z + 2] = {fx, fy, mz} (relative to the fluid at rest).
 * Wetted links use the interpolated (Bouzidi) bounce-back. FP32 populations.
 */
typedef struct lbm_fsi_config {
    int32_t nx, ny, nz;
    int32_t collision;           /* LBM_BGK | LBM_TRT | LBM_LES */
    double nu, cs, magic;
    double chord, x_ea, y_ea, ea, span;
    double u0, sponge_start, sponge_strength;
    int32_t device;
    int32_t reserved;
} lbm_fsi_config;

typedef struct lbm_fsi lbm_fsi;

lbm_status lbm_fsi_create(const lbm_fsi_config *cfg, lbm_fsi **out);
lbm_status lbm_fsi_destroy(lbm_fsi *w);
/* fsi_init (fsi.py:71-78) at the layer kinematics kin (4 nz values). */
lbm_status lbm_fsi_init(lbm_fsi *w, const double *kin);
/* fsi_step (fsi.py:81-186). Synchronous: load receives 3 nz values. */
lbm_status lbm_fsi_step(lbm_fsi *w, int32_t report, const double *kin, double *load);
lbm_status lbm_fsi_set_physics(lbm_fsi *w, int32_t collision, double nu);
lbm_status lbm_fsi_field(lbm_fsi *w, int32_t id, float **ptr);
lbm_status lbm_fsi_populations(lbm_fsi *w, float *host, int32_t set);
/* The solid mask (n bytes) at the layer kinematics kin (fsi.py:35-47), with
 * float64 results as in lbm_wing_mask; kin becomes the handle's kinematics. */
lbm_status lbm_fsi_mask(lbm_fsi *w, const double *kin, uint8_t *host);
lbm_status lbm_fsi_set_output_stride(lbm_fsi *w, int32_t stride);
lbm_status lbm_fsi_output(lbm_fsi *w, int32_t id, float **ptr, int64_t *count);
lbm_status lbm_fsi_update_output(lbm_fsi *w);

/* Message of the last error on this thread ("" when none). */
const char *lbm_last_error(void);

/* ABI version: bump when a signature or struct changes. */
int32_t lbm_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
