/*
 * sopht_gb300.h — C ABI of the GB300-native SophT flow-step library.
 *
 * Scope: the flow-step hot path of SophT — the Eulerian grid operators of the
 * unbounded vorticity Navier-Stokes step (2D: forcing curl, ENO3 conservative
 * advection, diffusion, boundary penalisation, velocity recovery; 3D: forcing
 * curl, rotational-form u x w update, diffusion, optional Laplacian filter,
 * penalisation, velocity recovery), the unbounded domain-doubled FFT Poisson
 * solve, and the immersed-boundary interpolation/spreading with
 * virtual-boundary forcing.
 *
 * Conventions
 *  - Every function returns SG_OK (0) or an SG_ERR_* code; sg_last_error()
 *    returns a thread-local message for the last failure.
 *  - Pointers are raw CUDA device pointers unless stated otherwise.  Arrays are
 *    C-ordered: 2D (ny, nx), 3D (nz, ny, nx); vector fields put the component
 *    first with component 0 = x (sopht/utils/field.py).
 *  - `dtype` selects the real type of every Eulerian/Lagrangian field of the
 *    call: SG_F32 (float) or SG_F64 (double).  Marker positions and body
 *    velocities are always double, as the reference's forcing grids hold them.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Only the *_create functions and sg_ib_bind allocate memory (and the
 *    *_create functions synchronise).  Step and operator calls never allocate
 *    and never synchronise, so they can be recorded in a CUDA graph; the host
 *    reads (sg_flow_host_max, sg_flow_read_device_time, sg_ib_binding_wait)
 *    block and say so.
 *
 * Each declaration cites the reference interface it replaces (file:line within
 * the SophT repository).
 */
#ifndef SOPHT_GB300_H
#define SOPHT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SG_OK 0
#define SG_ERR_INVALID_ARG 1   /* bad dtype, null pointer, bad flag          */
#define SG_ERR_SHAPE 2         /* grid too small / unsupported extent        */
#define SG_ERR_CUDA 3          /* a CUDA runtime call failed                 */
#define SG_ERR_UNSUPPORTED 4   /* FFT length with a prime factor above 7     */
#define SG_ERR_OUT_OF_DOMAIN 5 /* an IB marker support leaves the grid       */

#define SG_F32 0
#define SG_F64 1

typedef struct sg_poisson_plan_s* sg_poisson_plan;
typedef struct sg_flow_plan_s* sg_flow_plan;

/* Per-step scalar prefactors, rounded to the field precision by the caller
 * exactly as the reference computes them (navier_stokes_flow_simulators.py:
 * 175-186, 203-207, 461-471).  Fields unused by a call are ignored. */
typedef struct sg_step_scalars {
    double dt;              /* time step                                        */
    double forcing_prefac;  /* dt / (2 dx rho)            (forcing curl update)  */
    double advection_prefac;/* 2D: dt / dx (ENO3);  3D: dt / (2 dx) (u x w curl) */
    double diffusion_prefac;/* nu dt / dx^2                                      */
    double free_stream[3];  /* free-stream velocity added after the curl         */
} sg_step_scalars;

/* ---------------------------------------------------------------- general */
/* No reference counterpart: the calling thread's message for its last failed
 * call, and the library version (major * 100 + minor). */
const char* sg_last_error(void);
int sg_version(void);

/* ------------------------------------------------- unbounded Poisson solve */
/* Replaces UnboundedPoissonSolverPYFFTW2D.__init__ (poisson_solver_2d/
 * UnboundedPoissonSolverPYFFTW2D.py:11-45) and UnboundedPoissonSolverPYFFTW3D.
 * __init__ (poisson_solver_3d/UnboundedPoissonSolverPYFFTW3D.py:12-54): builds
 * the Green's function table in FP64 on the GPU and the FFT workspace for up to
 * `max_comp` components.  dim = 2 ignores nz.  nx must be even; nx, 2*ny and
 * 2*nz must factor into 2, 3, 5 and 7. */
int sg_poisson_plan_create(int dim, int nz, int ny, int nx, double x_range, int dtype,
                           int max_comp, sg_poisson_plan* plan_out);
int sg_poisson_plan_destroy(sg_poisson_plan plan);
/* Device bytes held by the plan (workspace + tables). */
int64_t sg_poisson_plan_bytes(sg_poisson_plan plan);
/* Replaces UnboundedPoissonSolverPYFFTW2D.solve (:95-129), ...3D.solve
 * (:111-149) and ...3D.vector_field_solve (:151-172): solves -lap(sol) = rhs
 * on the unbounded domain for `ncomp` components spaced `comp_stride` elements
 * apart in both rhs and sol. */
int sg_poisson_solve(sg_poisson_plan plan, const void* rhs, void* sol, int ncomp,
                     int64_t comp_stride, void* stream);

/* Allocation-free variant of the 2D solve (no counterpart in the reference).
 * For callers that cannot allocate device memory: code running inside CUDA
 * graph capture, hosts whose device memory is owned by another framework's
 * pool, and embeddings that forbid allocation after start-up.  It solves the
 * same problem as sg_poisson_solve with ncomp = 1, fp32 only, using a fixed
 * ~10 MB file-scope device array instead of a plan (every GPU that loads the
 * library holds it until the process exits).  Limit: ny <= 256, even
 * nx <= 512; larger grids return SG_ERR_SHAPE.  The first call on a device
 * (and a call with a new ny, nx or x_range) looks up the array's address and
 * rebuilds the Green's table into it, so make that first call before any
 * stream capture; a rebuild asked for on a capturing stream returns
 * SG_ERR_INVALID_ARG and leaves the array as it was.  The array holds the table
 * of the last grid: a call on a new grid replaces it for every later reader,
 * graphs captured earlier on another grid included (they then read the new
 * grid's table; replay them only after a call on their own grid).
 * All calls share the array: calls whose GPU work overlaps (other streams,
 * other host threads) race and must be serialised by the caller. */
int sg_poisson2d_solve_noalloc(int ny, int nx, double x_range, const float* rhs, float* sol,
                               void* stream);

/* --------------------------------------------------------- flow step plan */
/* Replaces the kernel compilation of UnboundedNavierStokesFlowSimulator2D/3D
 * (navier_stokes_flow_simulators.py:89-162, 327-440).  pen_coef_{x,y,z} are
 * host arrays of length nx, ny, nz holding the penalisation factor of each
 * index (sin ramp inside the band, exactly 1 outside), computed by the caller
 * as penalise_field_boundary_{2,3}d.py does; NULL means no penalisation.
 * filter_type: 0 none, 1 multiplicative, 2 convolution (laplacian_filter_3d.py).
 */
int sg_flow_plan_create(int dim, int nz, int ny, int nx, double x_range, int dtype,
                        int penalty_width, const void* pen_coef_x, const void* pen_coef_y,
                        const void* pen_coef_z, int filter_type, int filter_order,
                        sg_flow_plan* plan_out);
int sg_flow_plan_destroy(sg_flow_plan plan);
int64_t sg_flow_plan_bytes(sg_flow_plan plan);
/* Measurement hook (no reference counterpart): arms `n_events` (<= 16)
 * cudaEvent_t handles that the next sg_flow_step records between its passes,
 * event i before pass i and the last one after the final pass.  2D passes:
 * sweep, Poisson load, column convolution, row C2R, curl (6 events).  3D
 * passes: stencils (forcing curl, u x w update, diffusion; + filter),
 * Poisson load, y FFT, z convolution, y IFFT, x C2R, curl (8 events).
 * One-shot. */
int sg_flow_set_timing_events(sg_flow_plan plan, int n_events, void* const* events);

/* One flow time step, in place on the caller's fields.  Replaces
 * _navier_stokes_with_forcing_time_step / _navier_stokes_time_step
 * (navier_stokes_flow_simulators.py:171-209 in 2D, :449-498 in 3D).
 * forcing may be NULL (no body forcing); it is read, then set to zero.
 * Scalars come from `scalars` or, when `dev_scalars` is not NULL, from that
 * device struct (written by sg_flow_device_dt).  The max over cells of
 * sum_d |u_d| of the new velocity is left in the plan for sg_flow_device_dt. */
int sg_flow_step(sg_flow_plan plan, void* vorticity, void* velocity, void* forcing,
                 void* stream_func, const sg_step_scalars* scalars,
                 const sg_step_scalars* dev_scalars, void* stream);

/* max over cells of sum_d |u_d| (passive_transport_flow_simulators.py:149-151).
 * Written as a double to the device pointer `out` (an 8-byte slot).  */
int sg_max_abs_sum(int dtype, int dim, int64_t n_cells, const void* velocity, double* out,
                   void* stream);
/* The same max of the plan's grid for a host-side stable dt
 * (navier_stokes_flow_simulators.py:212-223 read the max on the host):
 * reduced into the plan's slot, copied through a plan-owned pinned word and
 * returned in *host_out after `stream` has drained (synchronous). */
int sg_flow_host_max(sg_flow_plan plan, const void* velocity, double* host_out, void* stream);
/* Device-resident stable dt: recomputes the plan's max from `velocity` when it
 * is not NULL, then evaluates compute_advection_diffusion_stable_timestep
 * (passive_transport_flow_simulators.py:139-155) times dt_prefac, and the step
 * prefactors, into the plan's device scalar struct.  *dev_scalars_out receives
 * its device address. */
int sg_flow_device_dt(sg_flow_plan plan, const void* velocity, double cfl, double nu,
                      double flow_density, double dt_prefac, const double* free_stream,
                      const sg_step_scalars** dev_scalars_out, void* stream);
/* No reference counterpart: the device address of the plan's accumulated
 * device time (seconds added by sg_flow_device_dt since the plan was made;
 * the flow's time is the host time at creation plus this), for kernels that
 * read the time of the current step on the GPU. */
int sg_flow_device_time_slot(sg_flow_plan plan, const double** slot_out);
/* No reference counterpart (measurement hook): records a timing event on
 * `stream`; while the stream is being captured the record becomes a node of
 * the graph, so a replay times the work between two such records. */
int sg_event_record(void* event, void* stream);

/* ----------------------------------------------------- batched 2D instances */
/* Many independent 2D simulators (uneven grids and Reynolds numbers, one
 * virtual-boundary body each) advanced together: one persistent launch per
 * fused operator for the whole batch, dt evaluated per instance on the GPU.
 * No reference counterpart (the reference steps one simulator at a time,
 * navier_stokes_flow_simulators.py:200-209, with its interactor,
 * VirtualBoundaryForcing.py:232-283).  Every member references an existing 2D
 * fp32 flow plan and its fields; nx and 2 ny must be 256, 512, 768 or 1024. */
typedef struct sg_batch2d_s* sg_batch2d;
typedef struct sg_batch2d_member {
    sg_flow_plan plan;
    void* vorticity;
    void* velocity;
    void* forcing;
    void* stream_func;
    double cfl, nu, flow_density, dt_prefac;
    double free_stream[2];
    int n_lag;              /* 0: no immersed body */
    int kernel_type;        /* 0 cosine, 1 Peskin */
    double dx, shift;
    const double* position;       /* (2, n_lag) device, double */
    const double* body_velocity;  /* (2, n_lag) device, double */
    int32_t* nearest;
    void* weights;
    void* flow_velocity;
    void* velocity_mismatch;
    void* position_mismatch;
    void* lag_forcing;
    double stiffness, damping;
    int32_t* status;
} sg_batch2d_member;
int sg_batch2d_create(int n, const sg_batch2d_member* members, sg_batch2d* batch_out);
/* Tuning knobs (picked by the Python autotuner): sweep tile height 8 or 16;
 * persistent blocks per SM (0 = one block per work item); block size of the
 * FFT passes, 256 or 512 threads (512: twice the lines per work item). */
int sg_batch2d_set_tuning(sg_batch2d batch, int sweep_tile_y, int blocks_per_sm, int fft_threads);
/* One coupled step of every member (8 launches).  Each member's velocity max
 * must be primed once (sg_flow_prime_max) before the first step. */
int sg_batch2d_step(sg_batch2d batch, void* stream);
int sg_batch2d_destroy(sg_batch2d batch);

/* Record max over cells of sum_d |u_d| of `velocity` in the plan (the value
 * the next sg_flow_device_dt with velocity = NULL, or the next batched step,
 * turns into dt) without evaluating dt or advancing the device time. */
int sg_flow_prime_max(sg_flow_plan plan, const void* velocity, void* stream);

/* Simulated time accumulated on the GPU by sg_flow_device_dt / the batched
 * step (the device-resident counterpart of FlowSimulator.time,
 * flow_simulators.py:126-128).  Synchronous read into *host_out. */
int sg_flow_read_device_time(sg_flow_plan plan, double* host_out);

/* ------------------------------------------------ single operators (2D) */
/* stencil_ops_2d/advection_timestep_2d.py:10-55 (flux buffer internal). */
int sg_advection_eno3_step_2d(int dtype, int ny, int nx, const void* field_in, void* field_out,
                              const void* velocity, double dt_by_dx, void* stream);
/* stencil_ops_2d/diffusion_timestep_2d.py:10-43 */
int sg_diffusion_step_2d(int dtype, int ny, int nx, const void* field_in, void* field_out,
                         double nu_dt_by_dx2, void* stream);
/* stencil_ops_2d/update_vorticity_from_velocity_forcing_2d.py:12-71 */
int sg_forcing_curl_update_2d(int dtype, int ny, int nx, const void* field_in, void* field_out,
                              const void* forcing, double prefactor, void* stream);
/* stencil_ops_2d/outplane_field_curl_2d.py:13-100 */
int sg_outplane_curl_2d(int dtype, int ny, int nx, const void* psi, void* curl,
                        double prefactor, void* stream);
/* stencil_ops_2d/penalise_field_boundary_2d.py:12-142 (out of place) */
int sg_penalise_2d(int dtype, int ny, int nx, const void* field_in, void* field_out,
                   int width, const void* coef_x, const void* coef_y, void* stream);

/* ------------------------------------------------ single operators (3D) */
/* stencil_ops_3d/curl_3d.py:13-132 */
int sg_curl_3d(int dtype, int nz, int ny, int nx, const void* field, void* curl,
               double prefactor, void* stream);
/* stencil_ops_3d/update_vorticity_from_velocity_forcing_3d.py:12-132 */
int sg_forcing_curl_update_3d(int dtype, int nz, int ny, int nx, const void* field_in,
                              void* field_out, const void* forcing, double prefactor,
                              void* stream);
/* stencil_ops_3d/elementwise_ops_3d.py:390-449 */
int sg_cross_3d(int dtype, int64_t n_cells, const void* a, const void* b, void* out,
                void* stream);
/* stencil_ops_3d/diffusion_timestep_3d.py:12-80 (vector field) */
int sg_diffusion_step_3d(int dtype, int nz, int ny, int nx, const void* field_in,
                         void* field_out, double nu_dt_by_dx2, void* stream);
/* stencil_ops_3d/divergence_3d.py */
int sg_divergence_3d(int dtype, int nz, int ny, int nx, const void* field, void* div,
                     double inv_dx, void* stream);
/* stencil_ops_3d/penalise_field_boundary_3d.py:13-240 (vector field, out of place) */
int sg_penalise_3d(int dtype, int nz, int ny, int nx, const void* field_in, void* field_out,
                   int width, const void* coef_x, const void* coef_y, const void* coef_z,
                   void* stream);
/* stencil_ops_3d/laplacian_filter_3d.py:13-194 (vector field, in place; the
 * two scratch buffers hold one scalar field each) */
int sg_laplacian_filter_3d(int dtype, int nz, int ny, int nx, void* field, int filter_type,
                           int filter_order, void* scratch_a, void* scratch_b, void* stream);

/* ------------------------------------- elementwise and flux-form operators */
/* The lower-level factories of stencil_ops_{2,3}d/elementwise_ops_{2,3}d.py on
 * n contiguous values: op 0 set (out = alpha), 1 add a fixed value
 * (out = a + alpha), 2 copy (out = a), 3 sum (out = a + b), 4 saxpby
 * (out = alpha a + beta b), 5 complex product of n interleaved complex values
 * (re = ar br - ai bi, im = ar bi + ai br).  alpha and beta are rounded to the
 * field type first, as pystencils passes them. */
int sg_elementwise(int dtype, int op, int64_t n, const void* a, const void* b, void* out,
                   double alpha, double beta, void* stream);
/* gen_set_fixed_val_at_boundaries_pyst_kernel_{2,3}d (elementwise_ops_2d.py:
 * 193-253, elementwise_ops_3d.py:200-268): every cell within `width` of a face
 * of the grid set to `value` (dim 2 ignores nz). */
int sg_set_boundary_zone(int dtype, int dim, int nz, int ny, int nx, int width, void* field,
                         double value, void* stream);
/* gen_diffusion_flux_pyst_kernel_{2,3}d (diffusion_flux_2d.py:13-72,
 * diffusion_flux_3d.py:14-115): flux = k lap(field) on [1:-1] in the
 * reference's term order; with reset_ghost_zone the ring is set to 0, without
 * it the ring is left unchanged.  field and flux must not alias. */
int sg_diffusion_flux(int dtype, int dim, int nz, int ny, int nx, const void* field, void* flux,
                      double k, int reset_ghost_zone, void* stream);
/* gen_advection_flux_conservative_eno3_pyst_kernel_2d (advection_flux_2d.py:
 * 12-165): flux += the four ENO3 face fluxes of a 2D scalar field on [2:-2]^2 in
 * the reference's pass order (in place on `flux`). */
int sg_advection_eno3_flux_2d(int dtype, int ny, int nx, const void* field, void* flux,
                              const void* velocity, double inv_dx, void* stream);

/* ------------------------------------------------------ passive transport */
/* Replaces the 3D conservative ENO3 advection timestep
 * (stencil_ops_3d/advection_timestep_3d.py:38-96 with advection_flux_3d.py:
 * 12-233): out = in + flux on [2:-2]^3 (out = in elsewhere), inv_dx = -dt_by_dx,
 * for `ncomp` components spaced nz*ny*nx apart (all advected by the same
 * (3, nz, ny, nx) velocity; with ncomp = 3 one thread advects all three,
 * loading the velocity once).  in and out must not alias. */
int sg_advection_eno3_step_3d(int dtype, int nz, int ny, int nx, int ncomp, const void* in,
                              void* out, const void* velocity, double dt_by_dx, void* stream);
/* Replaces gen_advection_flux_conservative_eno3_pyst_kernel_3d
 * (advection_flux_3d.py:12-233): flux += the six face fluxes of a scalar field,
 * in the reference's pass order, on [2:-2]^3 (in place on `flux`). */
int sg_advection_eno3_flux_3d(int dtype, int nz, int ny, int nx, const void* field, void* flux,
                              const void* velocity, double inv_dx, void* stream);
/* Replaces PassiveTransportFlowSimulator._advection_and_diffusion_time_step
 * (simulator/flow/passive_transport_flow_simulators.py:104-118): each of the
 * `ncomp` components of `field` (1 in 2D; 1 or 3 in 3D) is advected by ENO3
 * with dt_by_dx and then diffused with nu_dt_by_dx2, in place.  `scratch`
 * holds ncomp fields of the grid (a scalar field: the simulator's
 * buffer_scalar_field).  2D: one fused sweep; 3D: one advection launch and
 * one diffusion launch for all components. */
int sg_passive_transport_step(int dtype, int dim, int nz, int ny, int nx, int ncomp, void* field,
                              void* scratch, const void* velocity, double dt_by_dx,
                              double nu_dt_by_dx2, void* stream);

/* ------------------------------------------------------ immersed boundary */
/* Replaces VirtualBoundaryForcing.compute_interaction_force_on_lag_grid
 * (immersed_boundary_ops/VirtualBoundaryForcing.py:187-230) with the
 * support/weights/interpolation kernels of EulerianLagrangianGridCommunicator
 * {2,3}D.py.  Optionally first applies VirtualBoundaryForcing.time_step
 * (:276-283), xi += dt * dU, with dt taken from `xi_dt` or from
 * dev_scalars->dt.
 *   position, body_velocity: (dim, n_lag) double.
 *   nearest (dim, n_lag) int32 and weights ((2w)^dim, n_lag) are outputs kept
 *   for the spreading call; flow_velocity, velocity_mismatch, forcing are
 *   (dim, n_lag) real outputs; position_mismatch (dim, n_lag) is in/out.
 *   kernel_type: 0 cosine, 1 Peskin.  Markers whose support leaves the grid
 *   are skipped and reported with SG_ERR_OUT_OF_DOMAIN through *status_dev. */
int sg_ib_interaction(int dtype, int dim, int nz, int ny, int nx, double dx, double shift,
                      int n_lag, int kernel_type, const double* position,
                      const double* body_velocity, const void* eul_velocity,
                      int32_t* nearest, void* weights, void* flow_velocity,
                      void* velocity_mismatch, void* position_mismatch, void* forcing,
                      double stiffness, double damping, int do_xi_step, double xi_dt,
                      const sg_step_scalars* dev_scalars, int32_t* status_dev, void* stream);
/* Replaces the Lagrangian-to-Eulerian spreading of VirtualBoundaryForcing
 * (:232-274) and EulerianLagrangianGridCommunicator{2,3}D
 * (lagrangian_to_eulerian_grid_interpolation_kernel): eul_forcing += sum_i
 * F_i phi_i, each cell summing its markers in index order (deterministic, no
 * atomics).  reset != 0 zeroes eul_forcing first (the *_with_eul_grid_forcing_
 * reset variant). */
int sg_ib_spread(int dtype, int dim, int nz, int ny, int nx, int n_lag,
                 const int32_t* nearest, const void* weights, const void* forcing,
                 void* eul_forcing, int reset, void* stream);
/* The same spreading for many markers, in O(n log n): every (marker, window
 * cell) pair keyed by its cell, a stable radix sort by key, then one thread per
 * cell summing its pairs in ascending marker order -- the sums are bitwise
 * those of sg_ib_spread, whose owner test scans the lower-index markers and so
 * grows quadratically (surface grids, batch-wide rod grids).  `scratch` is
 * caller-owned device memory of sg_ib_spread_sorted_scratch_bytes bytes (< 0:
 * unsupported sizes); the call allocates nothing. */
int64_t sg_ib_spread_sorted_scratch_bytes(int dim, int nz, int ny, int nx, int n_lag);
int sg_ib_spread_sorted(int dtype, int dim, int nz, int ny, int nx, int n_lag,
                        const int32_t* nearest, const void* weights, const void* forcing,
                        void* eul_forcing, int reset, void* scratch, int64_t scratch_bytes,
                        void* stream);
/* VirtualBoundaryForcing.time_step (:276-283): xi += dt * dU. */
int sg_ib_mismatch_step(int dtype, int n, void* position_mismatch,
                        const void* velocity_mismatch, double dt, void* stream);

/* Bound coupling of one interactor: the per-step call of an immersed body,
 * ImmersedBodyFlowInteraction.__call__ (immersed_body_flow_interaction.py:
 * 113-122: upload the marker kinematics, interact, spread), as one host call.
 * sg_ib_bind records the interactor's fixed arguments (those of
 * sg_ib_interaction, the Eulerian extent, and a (2, dim, n_lag) float64
 * device buffer receiving positions then velocities) and allocates two
 * pinned staging slots of that layout plus a pinned (dim, n_lag) buffer of
 * the field type for the Lagrangian forcing; sg_ib_binding_buffers returns
 * their host addresses. */
typedef struct sg_ib_binding_s* sg_ib_binding;
int sg_ib_bind(int dtype, int dim, int nz, int ny, int nx, double dx, double shift, int n_lag,
               int kernel_type, int32_t* nearest, void* weights, void* flow_velocity,
               void* velocity_mismatch, void* position_mismatch, void* forcing,
               int32_t* status_dev, double* dev_kinematics, sg_ib_binding* binding_out);
int sg_ib_binding_buffers(sg_ib_binding binding, double** kin_slot0, double** kin_slot1,
                          void** forcing_host);
/* Blocks until staging slot `which` (0 or 1) may be overwritten (its upload
 * has run), or, for which = 2, until the last queued forcing copy has landed. */
int sg_ib_binding_wait(sg_ib_binding binding, int which);
/* On `stream`: when kin_slot is 0 or 1, copy that staging slot to the device
 * kinematics buffer; then sg_ib_interaction on it (xi step as there, host dt
 * only); then, when spread_mode >= 0, sg_ib_spread with reset = spread_mode;
 * then, when copy_forcing != 0, copy the Lagrangian forcing to the pinned
 * forcing buffer (completion: sg_ib_binding_wait(binding, 2)).  Outside stream
 * capture the work is a graph captured on first use of each (kin_slot,
 * spread_mode, copy_forcing, eul_velocity, eul_forcing) and replayed, with the
 * per-call scalars written to a binding-owned device block just before; the
 * results are those of direct launches. */
int sg_ib_bound_step(sg_ib_binding binding, int kin_slot, const void* eul_velocity,
                     void* eul_forcing, int spread_mode, double stiffness, double damping,
                     int do_xi_step, double xi_dt, int copy_forcing, void* stream);
int sg_ib_unbind(sg_ib_binding binding);
/* Host-side (no GPU work) CosseratRodElementCentricForcingGrid kinematics
 * (simulator/immersed_body/cosserat_rod/cosserat_rod_forcing_grids.py:82-130):
 * element centres and mass-weighted element velocities of a rod with
 * n_elems + 1 nodes (node arrays of 3 rows of n_elems + 1 float64, rows
 * `*_row_stride` elements apart; mass (n_elems + 1) contiguous),
 * in numpy's operation order without fused multiply-adds, written to the
 * grid's (grid_dim, n_elems) position and velocity arrays and, when `staging`
 * is not NULL, to a staging slot of sg_ib_binding_buffers. */
int sg_rod_element_kinematics(int grid_dim, int n_elems, const double* node_position,
                              int64_t position_row_stride, const double* node_velocity,
                              int64_t velocity_row_stride, const double* mass,
                              double* position_out, double* velocity_out, double* staging);

/* ------------------------------------------------------------- adjoints */
/* Transposes of the 2D step's operators and of the virtual-boundary
 * coupling, for gradients of time-integrated body forces.  The reference has
 * no adjoint; each entry names the forward operator it transposes.  The ENO3
 * upwind branch of each face is held at its forward choice.  All adjoint
 * kernels are gathers without atomics (bitwise reproducible).  `*_bar` arrays
 * have the layout of the forward quantity they are the adjoint of. */

/* Number of doubles a `partials` buffer needs for the 2D adjoint entries
 * (one per 32 x 8 tile; the fused reverse sweep needs fewer). */
int64_t sg_adj_partials_count_2d(int ny, int nx);
/* acc[0] += sum(partials[0:n]) in a fixed order (device pointers). */
int sg_sum_partials(int64_t n, const double* partials, double* acc, void* stream);

/* Transpose of outplane_field_curl_2d.py (sg_outplane_curl_2d):
 * psi_bar = curl^T(curl_bar); the free stream adds no term. */
int sg_outplane_curl_adj_2d(int dtype, int ny, int nx, const void* curl_bar, void* psi_bar,
                            double prefactor, void* stream);
/* Transpose of penalise_field_boundary_2d.py (sg_penalise_2d), same tables. */
int sg_penalise_adj_2d(int dtype, int ny, int nx, const void* in_bar, void* out_bar, int width,
                       const void* cx, const void* cy, void* stream);
/* Transpose of diffusion_timestep_2d.py (sg_diffusion_step_2d with prefactor k):
 * out_bar = in_bar + k lap^T(m in_bar).  With `field` (the forward input) and
 * `partials`, per-tile partials of sum m lap(field) in_bar (= d loss / d k) are
 * written; reduce them with sg_sum_partials. */
int sg_diffusion_adj_2d(int dtype, int ny, int nx, const void* in_bar, void* out_bar, double k,
                        const void* field, double* partials, void* stream);
/* Transpose of the linearised advection_timestep_2d.py / advection_flux_2d.py
 * (sg_advection_eno3_step_2d) at (field, velocity):
 * out_bar = in_bar + (d flux / d field)^T in_bar, and velocity_bar (2, ny, nx)
 * += (d flux / d velocity)^T in_bar when not NULL. */
int sg_advection_eno3_adj_2d(int dtype, int ny, int nx, const void* field, const void* velocity,
                             double dt_by_dx, const void* in_bar, void* out_bar, void* velocity_bar,
                             void* stream);
/* Transpose of update_vorticity_from_velocity_forcing_2d.py
 * (sg_forcing_curl_update_2d): forcing_bar (2, ny, nx) += p curl^T(in_bar);
 * the vorticity adjoint passes through unchanged. */
int sg_forcing_curl_adj_2d(int dtype, int ny, int nx, const void* in_bar, void* forcing_bar,
                           double prefactor, void* stream);
/* Transpose of UnboundedPoissonSolverPYFFTW{2,3}D.solve (sg_poisson_solve).
 * The domain-doubled convolution with a real, even Green's function is
 * symmetric, so this is the same solve. */
int sg_poisson_solve_adj(sg_poisson_plan plan, const void* sol_bar, void* rhs_bar, int ncomp,
                         int64_t comp_stride, void* stream);
/* The Poisson plan owned by a flow plan (valid while the flow plan lives). */
sg_poisson_plan sg_flow_poisson_plan(sg_flow_plan plan);

/* Arm a one-shot tape for the next 2D sg_flow_step: the vorticity after the
 * forcing curl and after the advection update are written to the two
 * buffers (ny, nx).  Both NULL disarms. */
int sg_flow_set_tape(sg_flow_plan plan, void* w_after_forcing, void* w_after_advection);
/* Transpose of one 2D step's sweep chain (forcing curl, ENO3 advection,
 * diffusion, penalisation) in one pass, given the adjoint of the vorticity
 * after the step (w_bar_after, plus poisson_bar when not NULL) and the step's
 * tape and velocity.  Writes w_bar_before, velocity_bar (advection part,
 * overwritten), forcing_bar (overwritten, may be NULL) and, when
 * w_after_advection is given, viscosity partials (d loss / d diffusion
 * prefactor, reduce with sg_sum_partials).  `scalars` are the forward step's
 * host scalars. */
int sg_ns2d_reverse_sweep(sg_flow_plan plan, const void* w_bar_after, const void* poisson_bar,
                          const void* w_after_forcing, const void* w_after_advection,
                          const void* velocity, const sg_step_scalars* scalars, void* w_bar_before,
                          void* velocity_bar, void* forcing_bar, double* partials, void* stream);
/* Transpose of one virtual-boundary call (VirtualBoundaryForcing.py:132-185,
 * 232-283 with the spreading of EulerianLagrangianGridCommunicator{2,3}D):
 * F_bar = spread^T(eul_forcing_bar) + lag_forcing_bar_const[d] (host, may be
 * NULL); position_mismatch_bar += K F_bar; dU_bar = C F_bar +
 * velocity_mismatch_bar_carry; body_velocity_bar (device float64) -= dU_bar;
 * flow_velocity_bar = dx^dim dU_bar; then velocity_mismatch_bar_carry =
 * xi_dt * position_mismatch_bar (the transpose of time_step(xi_dt) before the
 * call).  nearest and weights are those of the forward call. */
int sg_ib_interaction_adj(int dtype, int dim, int nz, int ny, int nx, double dx, int n_lag,
                          const int32_t* nearest, const void* weights, const void* eul_forcing_bar,
                          const double* lag_forcing_bar_const, double stiffness, double damping,
                          double xi_dt, void* position_mismatch_bar,
                          void* velocity_mismatch_bar_carry, double* body_velocity_bar,
                          void* flow_velocity_bar, void* stream);
/* Transpose of the Eulerian-to-Lagrangian interpolation
 * (eulerian_to_lagrangian_grid_interpolation_kernel): eul_velocity_bar +=
 * sum_i phi_i flow_velocity_bar_i (deterministic spreading). */
int sg_ib_interp_adj(int dtype, int dim, int nz, int ny, int nx, int n_lag,
                     const int32_t* nearest, const void* weights, const void* flow_velocity_bar,
                     void* eul_velocity_bar, void* stream);
/* acc[0] (device double) += sum_d weights3[d] sum_i lag_field[d, i] (fixed order). */
int sg_lag_weighted_sum(int dtype, int dim, int n_lag, const void* lag_field,
                        const double* weights3, double* acc, void* stream);

/* ------------------------------------------------------------ Cosserat rods
 * A batch of rods with the same element count n, every array FP64 on the
 * device and C-ordered with the rod index first: nodes (n_rods, 3, n+1),
 * elements (n_rods, 3, n) or (n_rods, 3, 3, n) for matrices, Voronoi regions
 * (n_rods, 3, n-1) or (n_rods, 3, 3, n-1).  Directors are rows d1, d2, d3 (a
 * lab vector v has local components Q v); omega and external_torques are in
 * the local frame.  This is the layout of pyelastica's CosseratRod
 * (elastica/rod/cosserat_rod.py), which SophT couples through
 * cosserat_rod_flow_interaction.py:9-58 and flow_forces.py:12-25. */
typedef struct sg_rod_batch {
    int n_rods, n_elems;
    double* position;                     /* (n_rods, 3, n+1) */
    double* velocity;                     /* (n_rods, 3, n+1) */
    double* directors;                    /* (n_rods, 3, 3, n) */
    double* omega;                        /* (n_rods, 3, n)   */
    const double* mass;                   /* (n_rods, n+1)    */
    const double* rest_lengths;           /* (n_rods, n)      */
    const double* rest_voronoi_lengths;   /* (n_rods, n-1)    */
    const double* shear_matrix;           /* (n_rods, 3, 3, n)   */
    const double* bend_matrix;            /* (n_rods, 3, 3, n-1) */
    const double* mass_second_moment;     /* (n_rods, 3, 3, n)   */
    const double* inv_mass_second_moment; /* (n_rods, 3, 3, n)   */
    const double* rest_sigma;             /* (n_rods, 3, n)   */
    const double* rest_kappa;             /* (n_rods, 3, n-1) */
    double* external_forces;              /* (n_rods, 3, n+1) */
    double* external_torques;             /* (n_rods, 3, n)   */
    const int* clamped;                   /* (n_rods) 1 = node 0 and element 0's directors fixed, or NULL */
    const double* clamp_position;         /* (n_rods, 3)      */
    const double* clamp_directors;        /* (n_rods, 3, 3)   */
} sg_rod_batch;

/* n_substeps position-Verlet steps of dt for every rod of the batch, in one
 * launch (one CTA per rod): the discrete Cosserat model of Gazzola et al.
 * (2018) that pyelastica's PositionVerlet stepper integrates
 * (flow_past_rod_case.py:231-250 runs it rod_time_steps times per flow step).
 * External loads stay fixed over the call; damping_rate > 0 multiplies
 * velocities and angular velocities by exp(-damping_rate dt) each sub-step.
 * 1 <= n_elems <= 1024.  The batch struct is read on the host. */
int sg_rod_batch_step(const sg_rod_batch* batch, int n_substeps, double dt, double damping_rate,
                      void* stream);
/* The element-centric forcing grid of every rod of the batch at once
 * (cosserat_rod_forcing_grids.py:82-130), in the marker layout of one
 * VirtualBoundaryForcing over the batch: (dim, n_rods * n), marker r * n + e.
 * sg_rod_batch_element_markers writes the markers' positions (the element
 * centres) and velocities (the mass-weighted mean of the two nodes), float64
 * device arrays; sg_rod_batch_element_loads turns the Lagrangian forcing of
 * those markers (dtype SG_F32 or SG_F64) into each rod's external_forces (the
 * reaction -F/2 on both nodes of an element, components past dim 0) and sets
 * external_torques to 0, as transfer_forcing_from_grid_to_body and
 * FlowForces.apply_forces (flow_forces.py:22-25) do for a rod whose only load
 * is the flow. */
int sg_rod_batch_element_markers(const sg_rod_batch* batch, int dim, double* position, double* velocity,
                                 void* stream);
int sg_rod_batch_element_loads(const sg_rod_batch* batch, int dim, int dtype, const void* lag_forcing,
                               void* stream);

/* The flow coupling of a rod batch over one flow step, 3D.  Replaces the rod
 * loop of the reference examples (flow_past_rod_case.py:231-243,
 * immersed_magnetic_cilia_carpet.py:231-240): rod_time_steps =
 * int(flow_dt / min(flow_dt, max_rod_dt)) sub-steps of flow_dt /
 * rod_time_steps, each one pyelastica's position-Verlet do_step with
 * FlowForces.apply_forces (flow_forces.py:22-25) evaluated at the half-step
 * configuration -- the element-centric markers (cosserat_rod_forcing_grids.py:
 * 82-130), the interaction force of VirtualBoundaryForcing.
 * compute_interaction_force_on_lag_grid (VirtualBoundaryForcing.py:187-230)
 * and its reaction as the rods' external forces -- followed by
 * VirtualBoundaryForcing.time_step (xi += dt dU, :276-283).  One launch, one
 * CTA per rod, 1 to 256 elements per rod (one thread per element and marker;
 * more return SG_ERR_SHAPE); the sub-step count is read on the device, so the call can be
 * part of a step whose dt never leaves the GPU.  Lagrangian fields are
 * (3, n_rods * n_elems) in the flow precision `dtype`; marker positions and
 * velocities float64.  A driven clamp (drive_phase not NULL) turns each
 * clamped rod's element 0 about the lab axis drive_axis by
 * theta(t) = drive_amplitude sin(2 pi drive_frequency t + drive_phase[rod]),
 * its node 0 held in place.  damping_rate as in sg_rod_batch_step.  Markers
 * whose support leaves the grid set *status to SG_ERR_OUT_OF_DOMAIN. */
typedef struct sg_rod_coupling {
    int dtype;                      /* SG_F32 or SG_F64 */
    int nz, ny, nx;
    double dx, shift;               /* Eulerian spacing and coordinate shift (dx / 2) */
    int kernel_type;                /* 0 cosine, 1 Peskin */
    const void* flow_velocity;      /* (3, nz, ny, nx), read only */
    double* marker_position;        /* (3, n_markers) float64, written */
    double* marker_velocity;        /* (3, n_markers) float64, written */
    int32_t* nearest;               /* (3, n_markers) */
    void* weights;                  /* (64, n_markers) */
    void* flow_velocity_lag;        /* (3, n_markers) */
    void* velocity_mismatch;        /* (3, n_markers) */
    void* position_mismatch;        /* (3, n_markers) */
    void* lag_forcing;              /* (3, n_markers) */
    double stiffness, damping;      /* K, C after the Lagrangian-spacing rescale */
    double flow_dt;                 /* the flow step's dt when dev_scalars is NULL */
    double flow_time;               /* time at the start of the step; with dev_scalars, the time
                                       the device time slot counts from */
    const sg_step_scalars* dev_scalars; /* device dt of the flow step, or NULL */
    const double* dev_time_end;     /* with dev_scalars: the device time slot, which already
                                       holds the end of this step */
    double max_rod_dt;
    double damping_rate;
    const double* drive_phase;      /* (n_rods) device, or NULL */
    double drive_amplitude, drive_frequency;
    double drive_axis[3];
    int32_t* status;                /* device status word */
} sg_rod_coupling;
int sg_rod_batch_coupled_substeps(const sg_rod_batch* batch, const sg_rod_coupling* coupling, void* stream);

/* The 3D step's rotational-form vorticity update w2 = w1 + prefactor curl(u x w1)
 * on [1:-1]^3 (w1 elsewhere), as one operator: the reference forms it from
 * elementwise_cross_product (elementwise_ops_3d.py:406-448) and the curl
 * kernel (curl_3d.py), navier_stokes_flow_simulators.py:461-471.  staged = 0:
 * the direct-load kernel; staged = 1: inputs staged in shared memory by tensor
 * copies (fp32, nx a multiple of 4, 16-byte aligned fields), the same bits; a
 * copy wait that runs out writes SG_ERR_CUDA to *status (device word). */
int sg_rotational_update_3d(int dtype, int nz, int ny, int nx, const void* w1, const void* u, void* out,
                            double prefactor, int staged, int32_t* status, void* stream);
/* No reference counterpart: the plan's device status word (0, or SG_ERR_CUDA
 * after a bounded wait inside a step's kernels ran out; sticky); blocks. */
int sg_flow_kernel_status(sg_flow_plan plan, int32_t* host_out);
/* Replaces diffusion_timestep_3d.py:12-80 for 1 or 3 components with the
 * kernel chosen: staged = 0 the direct-load kernel (sg_diffusion_step_3d's),
 * staged = 1 the input staged in shared memory by tensor copies (fp32, nx a
 * multiple of 4, 16-byte aligned fields), the same bits; a copy wait that runs
 * out writes SG_ERR_CUDA to *status (device word). */
int sg_diffusion_3d_staged(int dtype, int nz, int ny, int nx, int ncomp, const void* in, void* out, double k,
                           int staged, int32_t* status, void* stream);
/* Replaces update_vorticity_from_velocity_forcing_3d.py:12-132 with the
 * kernel chosen: staged = 0 sg_forcing_curl_update_3d's direct-load kernel,
 * staged = 1 the forcing staged in shared memory by tensor copies (fp32, nx a
 * multiple of 4, 16-byte aligned fields), the same bits; *status as above. */
int sg_forcing_curl_3d_staged(int dtype, int nz, int ny, int nx, const void* in, void* out, const void* forcing,
                              double prefactor, int staged, int32_t* status, void* stream);
/* Replaces curl_3d.py:13-132 with elementwise_ops_3d.py's add_fixed_val and
 * the max of sum |u_d| (navier_stokes_flow_simulators.py:212-223) in one pass,
 * the kernel chosen: u = prefactor curl(psi) on [1:-1]^3 (0 on the ring) +
 * free_stream (3 host values, or NULL), max into *umax (device, or NULL; not
 * reset); staged = 0 the direct-load kernel, staged = 1 psi staged by tensor
 * copies (fp32, nx a multiple of 4, 16-byte aligned fields), the same bits. */
int sg_curl_3d_staged(int dtype, int nz, int ny, int nx, const void* psi, void* u, double prefactor,
                      const double* free_stream, void* umax, int staged, int32_t* status, void* stream);
/* No reference counterpart: the device status word of the operator entries'
 * staged kernels (sg_passive_transport_step takes them on fp32 grids); 0, or
 * SG_ERR_CUDA after a bounded wait ran out (sticky); blocks. */
int sg_ops_kernel_status(int32_t* host_out);

#ifdef __cplusplus
}
#endif
#endif /* SOPHT_GB300_H */
