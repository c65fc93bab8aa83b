// Batched Cosserat rod sub-steps: one CTA per rod, every sub-step of the call in one launch.
//
// The physics is rod.cuh's (the same functions a host driver runs in sequence); this file only
// maps its passes onto a block: threads stride over nodes, elements and Voronoi regions, and a
// barrier separates the passes that read neighbours from the ones that write them.  The per-rod
// work arrays live in shared memory.
#include "common.cuh"
#include "ib.cuh"
#include "rod.cuh"

namespace sg {

__global__ void __launch_bounds__(256) rod_batch_kernel(sg_rod_batch b, int n_substeps, double dt, double decay) {
    extern __shared__ double rod_smem[];
    rod::View v = rod::view_of(b, blockIdx.x);
    const rod::Scratch s = rod::carve(rod_smem, b.n_elems);
    const int n = b.n_elems, t = threadIdx.x, nt = blockDim.x;
    const double h = 0.5 * dt;
    for (int k = 0; k < n_substeps; ++k) {
        for (int i = t; i <= n; i += nt) rod::drift_node(v, i, h);
        for (int e = t; e < n; e += nt) rod::rotate_element(v, e, h);
        __syncthreads();
        for (int e = t; e < n; e += nt) rod::element_pass(v, s, e);
        __syncthreads();
        for (int q = t; q < n - 1; q += nt) rod::voronoi_pass(v, s, q);
        __syncthreads();
        for (int i = t; i <= n; i += nt) rod::node_update(v, s, i, dt, decay);
        for (int e = t; e < n; e += nt) rod::element_update(v, s, e, dt, decay);
        __syncthreads();
        for (int i = t; i <= n; i += nt) rod::drift_node(v, i, h);
        for (int e = t; e < n; e += nt) rod::rotate_element(v, e, h);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) rod_markers_kernel(sg_rod_batch b, int dim, double* pos, double* vel) {
    const int n = b.n_elems;
    const int64_t total = (int64_t)b.n_rods * n;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(k / n), e = (int)(k % n);
        const rod::View v = rod::view_of(b, r);
        rod::element_marker(v, r, e, dim, total, pos, vel);
    }
}

template <typename F>
__global__ void __launch_bounds__(256) rod_loads_kernel(sg_rod_batch b, int dim, const F* forcing) {
    const int n = b.n_elems, nn = n + 1;
    const int64_t total = (int64_t)b.n_rods * nn, n_markers = (int64_t)b.n_rods * n;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(k / nn), i = (int)(k % nn);
        rod::View v = rod::view_of(b, r);
        rod::element_reaction(v, r, i, dim, n_markers, forcing, b.external_forces + (int64_t)r * 3 * nn,
                              b.external_torques + (int64_t)r * 3 * n);
    }
}

// ------------------------------------------------------------------ flow coupling
// One flow step of the rod loop of the reference examples for every rod of a batch (one CTA per
// rod): rod_time_steps = int(dt / min(dt, max_rod_dt)) position-Verlet sub-steps of dt /
// rod_time_steps, each with the flow forces of the half-step configuration (the element-centric
// markers, the virtual-boundary interaction of ib_interaction_thread on those markers, the reaction
// on the nodes) and followed by xi += dt_sub dU.  The sub-step count comes from the device dt, so
// a captured step needs no host value.
template <typename T> struct RodCouplingArgs {
    IBParams<T> ib;           // marker arrays of the whole batch (n_lag = n_rods * n_elems)
    double* marker_pos;       // == ib.pos, written here
    double* marker_vel;       // == ib.body_vel
    double host_dt, host_time;
    const sg_step_scalars* dev;
    const double* dev_time_end;
    double max_rod_dt, damping_rate;
    const double* drive_phase;
    double drive_amp, drive_freq;
    double axis[3];
};

// The passes of a sub-step, each ended by a barrier: the markers with their interaction, in the same
// thread (and the next sub-step's driven-clamp frames); the reaction loads and the element pass;
// the Voronoi pass; the node and element updates; drift, rotate and the mismatch step -- the
// closing half drift of one sub-step and the opening half drift of the next in one pass.  Thread e owns marker e for the whole launch and keeps its position mismatch in
// registers.  The clamp frames of sub-step k + 1 are computed during sub-step k into the other half
// of a double buffer, by the first lanes of two warps that hold no nodes when the block has such
// warps (they would only wait at the barriers otherwise), in the longest pass.
template <typename T>
__global__ void __launch_bounds__(256) rod_coupled_kernel(sg_rod_batch b, RodCouplingArgs<T> c) {
    extern __shared__ double rod_smem[];
    const int r = blockIdx.x, n = b.n_elems, t = threadIdx.x, nt = blockDim.x;
    rod::View v = rod::view_of(b, r);
    const rod::Scratch s = rod::carve(rod_smem, n);
    // [sub-step parity][half step, end of sub-step][q (9), w (3)] of a driven clamp, then the
    // reciprocals of the masses (n + 1), rest lengths (n) and rest Voronoi lengths (n - 1)
    double* clamp = rod_smem + rod::scratch_doubles(n);
    double* recip = clamp + 48;
    for (int i = t; i <= n; i += nt) recip[i] = 1.0 / v.mass[i];
    for (int e = t; e < n; e += nt) recip[n + 1 + e] = 1.0 / v.l0[e];
    for (int q = t; q < n - 1; q += nt) recip[2 * n + 1 + q] = 1.0 / v.d0[q];
    v.inv_mass = recip;
    v.inv_l0 = recip + n + 1;
    v.inv_d0 = recip + 2 * n + 1;
    // the rod's state and loads live in shared memory for the launch (each pass reads what other
    // threads of the block wrote in the one before), copied back at the end
    double* const gx = v.x;
    double* const gv = v.v;
    double* const gq = v.q;
    double* const gw = v.w;
    double* const gf = b.external_forces + (int64_t)r * 3 * (n + 1);
    double* const gc = b.external_torques + (int64_t)r * 3 * n;
    double* const sx = recip + 3 * n;
    double* const sv = sx + 3 * (n + 1);
    double* const sq = sv + 3 * (n + 1);
    double* const sw = sq + 9 * n;
    double* const sf = sw + 3 * n;
    double* const sc = sf + 3 * (n + 1);
    for (int i = t; i < 3 * (n + 1); i += nt) {
        sx[i] = gx[i];
        sv[i] = gv[i];
    }
    for (int i = t; i < 9 * n; i += nt) sq[i] = gq[i];
    for (int i = t; i < 3 * n; i += nt) sw[i] = gw[i];
    v.x = sx;
    v.v = sv;
    v.q = sq;
    v.w = sw;
    v.f_ext = sf;
    v.c_ext = sc;
    const bool driven = c.drive_phase != nullptr && v.clamped;
    const double dt = c.dev ? c.dev->dt : c.host_dt;
    const double t0 = c.dev ? c.host_time + (*c.dev_time_end - dt) : c.host_time;
    const int n_sub = dt > c.max_rod_dt ? (int)(dt / c.max_rod_dt) : 1;
    const double h = dt / n_sub;
    const double decay = c.damping_rate != 0.0 ? exp(-c.damping_rate * h) : 1.0;
    const int64_t n_markers = (int64_t)b.n_rods * n;
    const double* q0 = b.clamp_directors + r * 9;
    const double phase = driven ? c.drive_phase[r] : 0.0;
    const int fa = n + 1 <= nt - 64 ? nt - 64 : 0;  // the frame threads: fa and fa + 32
    const T hT = (T)h;
    auto frames = [&](int k) {
        if (driven && (t == fa || t == fa + 32)) {
            double* fr = clamp + (k & 1) * 24 + (t == fa ? 0 : 12);
            const double tk = t0 + k * h;
            rod::driven_clamp(q0, c.axis, c.drive_amp, c.drive_freq, phase, tk + (t == fa ? 0.5 * h : h), fr, fr + 9);
        }
    };
    frames(0);
    // the position mismatch of the thread's marker (n <= 256 = blockDim: one marker per thread)
    T xi[3] = {T(0), T(0), T(0)};
    const int64_t own = (int64_t)r * n + t;
    if (t < n)
        for (int d = 0; d < 3; ++d) xi[d] = c.ib.pos_mismatch[d * n_markers + own];
    const double inv_dx = 1.0 / c.ib.dx;
    __syncthreads();
    // the first sub-step's opening half drift
    if (driven) {
        v.clamp_q = clamp;
        v.clamp_w = clamp + 9;
    }
    for (int i = t; i <= n; i += nt) rod::drift_node(v, i, 0.5 * h);
    for (int e = t; e < n; e += nt) rod::rotate_element(v, e, 0.5 * h);
    __syncthreads();
    for (int k = 0; k < n_sub; ++k) {
        const bool last = k + 1 == n_sub;
        // FlowForces.apply_forces at the half step: each marker, then its interaction
        if (!last) frames(k + 1);
        T dU[3] = {T(0), T(0), T(0)};
        if (t < n) {
            double X[3], V[3];
            rod::element_marker_at(v, t, 3, X, V);
            for (int d = 0; d < 3; ++d) {
                c.marker_pos[d * n_markers + own] = X[d];
                c.marker_vel[d * n_markers + own] = V[d];
            }
            ib_interaction_thread<T, 3>(c.ib, (int)own, X, V, xi, dU, last, inv_dx);
        }
        __syncthreads();
        // the reaction on the nodes, and the element pass (which reads neither the loads nor the markers)
        for (int i = t; i <= n; i += nt) rod::element_reaction(v, r, i, 3, n_markers, c.ib.forcing, sf, sc);
        for (int e = t; e < n; e += nt) rod::element_pass(v, s, e);
        __syncthreads();
        for (int q = t; q < n - 1; q += nt) rod::voronoi_pass(v, s, q);
        __syncthreads();
        for (int i = t; i <= n; i += nt) rod::node_update(v, s, i, h, decay);
        for (int e = t; e < n; e += nt) rod::element_update(v, s, e, h, decay);
        __syncthreads();
        // this sub-step's closing half drift and the next one's opening half drift in one pass (the
        // same arithmetic as the two, one rotation exponential), element 0 left at the next
        // half-step frame; the last sub-step closes with one half drift at the end-of-step frame
        double* const next = clamp + ((k + 1) & 1) * 24;
        if (driven) {
            v.clamp_q = last ? clamp + (k & 1) * 24 + 12 : next;
            v.clamp_w = last ? clamp + (k & 1) * 24 + 21 : next + 9;
        }
        if (last) {
            for (int i = t; i <= n; i += nt) rod::drift_node(v, i, 0.5 * h);
            for (int e = t; e < n; e += nt) rod::rotate_element(v, e, 0.5 * h);
        } else {
            for (int i = t; i <= n; i += nt) rod::drift_node_twice(v, i, 0.5 * h);
            for (int e = t; e < n; e += nt) rod::rotate_element_twice(v, e, 0.5 * h);
        }
        // VirtualBoundaryForcing.time_step(local_rod_dt) of the thread's marker
        if (t < n)
            for (int d = 0; d < 3; ++d) xi[d] = xi[d] + hT * dU[d];
        __syncthreads();  // the next sub-step's frames are written, and this one's no longer read
    }
    if (t < n)
        for (int d = 0; d < 3; ++d) c.ib.pos_mismatch[d * n_markers + own] = xi[d];
    for (int i = t; i < 3 * (n + 1); i += nt) {
        gx[i] = sx[i];
        gv[i] = sv[i];
        gf[i] = sf[i];
    }
    for (int i = t; i < 9 * n; i += nt) gq[i] = sq[i];
    for (int i = t; i < 3 * n; i += nt) {
        gw[i] = sw[i];
        gc[i] = sc[i];
    }
}

static int rod_grid_blocks(int64_t items) {
    const int64_t blocks = (items + 255) / 256;
    return (int)(blocks < 152 * 8 ? blocks : 152 * 8);
}

}  // namespace sg

static int rod_batch_check(const sg_rod_batch* batch, int dim) {
    SG_REQUIRE(batch, SG_ERR_INVALID_ARG, "rod batch: null batch");
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "rod batch: dim must be 2 or 3");
    SG_REQUIRE(batch->n_rods >= 1 && batch->n_elems >= 1, SG_ERR_SHAPE, "rod batch: empty batch");
    SG_REQUIRE(batch->position && batch->velocity && batch->mass && batch->external_forces &&
                   batch->external_torques,
               SG_ERR_INVALID_ARG, "rod batch: null array");
    return SG_OK;
}

extern "C" int sg_rod_batch_element_markers(const sg_rod_batch* batch, int dim, double* position, double* velocity,
                                            void* stream) {
    SG_TRY(rod_batch_check(batch, dim));
    SG_REQUIRE(position && velocity, SG_ERR_INVALID_ARG, "rod markers: null output");
    const int64_t items = (int64_t)batch->n_rods * batch->n_elems;
    sg::rod_markers_kernel<<<sg::rod_grid_blocks(items), 256, 0, (cudaStream_t)stream>>>(*batch, dim, position,
                                                                                        velocity);
    return sg::launch_status("rod batch element markers");
}

extern "C" int sg_rod_batch_element_loads(const sg_rod_batch* batch, int dim, int dtype, const void* lag_forcing,
                                          void* stream) {
    SG_TRY(rod_batch_check(batch, dim));
    SG_REQUIRE(lag_forcing, SG_ERR_INVALID_ARG, "rod loads: null forcing");
    SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, SG_ERR_INVALID_ARG, "rod loads: bad dtype");
    const int64_t items = (int64_t)batch->n_rods * (batch->n_elems + 1);
    auto s = (cudaStream_t)stream;
    if (dtype == SG_F32)
        sg::rod_loads_kernel<float><<<sg::rod_grid_blocks(items), 256, 0, s>>>(*batch, dim, (const float*)lag_forcing);
    else
        sg::rod_loads_kernel<double><<<sg::rod_grid_blocks(items), 256, 0, s>>>(*batch, dim,
                                                                               (const double*)lag_forcing);
    return sg::launch_status("rod batch element loads");
}

extern "C" int sg_rod_batch_step(const sg_rod_batch* batch, int n_substeps, double dt, double damping_rate,
                                 void* stream) {
    SG_REQUIRE(batch, SG_ERR_INVALID_ARG, "rod batch: null batch");
    const sg_rod_batch& b = *batch;
    SG_REQUIRE(b.n_rods >= 1 && b.n_elems >= 1 && b.n_elems <= 1024, SG_ERR_SHAPE,
               "rod batch: %d rods of %d elements (1 to 1024 elements)", b.n_rods, b.n_elems);
    SG_REQUIRE(n_substeps >= 0, SG_ERR_INVALID_ARG, "rod batch: negative sub-step count");
    SG_REQUIRE(b.position && b.velocity && b.directors && b.omega && b.mass && b.rest_lengths && b.shear_matrix &&
                   b.mass_second_moment && b.inv_mass_second_moment && b.rest_sigma && b.external_forces &&
                   b.external_torques,
               SG_ERR_INVALID_ARG, "rod batch: null array");
    SG_REQUIRE(b.n_elems == 1 || (b.rest_voronoi_lengths && b.bend_matrix && b.rest_kappa), SG_ERR_INVALID_ARG,
               "rod batch: null Voronoi array");
    SG_REQUIRE(!b.clamped || (b.clamp_position && b.clamp_directors), SG_ERR_INVALID_ARG,
               "rod batch: clamped rods need the clamp position and directors");
    if (n_substeps == 0) return SG_OK;
    const double decay = damping_rate != 0.0 ? exp(-damping_rate * dt) : 1.0;
    const size_t smem = (size_t)sg::rod::scratch_doubles(b.n_elems) * sizeof(double);
    if (smem > 48 * 1024)
        SG_TRY(sg::cuda_status(cudaFuncSetAttribute(sg::rod_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)smem),
                               "rod batch smem"));
    const int threads = (b.n_elems + 1 + 31) / 32 * 32 < 256 ? (b.n_elems + 1 + 31) / 32 * 32 : 256;
    sg::rod_batch_kernel<<<b.n_rods, threads, smem, (cudaStream_t)stream>>>(b, n_substeps, dt, decay);
    return sg::launch_status("rod batch step");
}

namespace sg {
template <typename T>
static int rod_coupled_launch(const sg_rod_batch& b, const sg_rod_coupling& cp, cudaStream_t stream) {
    RodCouplingArgs<T> c{};
    IBParams<T>& ip = c.ib;
    ip.dim = 3;
    ip.nz = cp.nz;
    ip.ny = cp.ny;
    ip.nx = cp.nx;
    ip.n_lag = b.n_rods * b.n_elems;
    ip.kernel = cp.kernel_type;
    ip.dx = cp.dx;
    ip.shift = cp.shift;
    ip.pos = cp.marker_position;
    ip.body_vel = cp.marker_velocity;
    ip.u = (const T*)cp.flow_velocity;
    ip.nearest = cp.nearest;
    ip.weights = (T*)cp.weights;
    ip.flow_vel = (T*)cp.flow_velocity_lag;
    ip.vel_mismatch = (T*)cp.velocity_mismatch;
    ip.pos_mismatch = (T*)cp.position_mismatch;
    ip.forcing = (T*)cp.lag_forcing;
    ip.K = cp.stiffness;
    ip.C = cp.damping;
    ip.xi_step = 0;
    ip.dev = nullptr;
    ip.status = cp.status;
    ip.dyn = nullptr;
    c.marker_pos = cp.marker_position;
    c.marker_vel = cp.marker_velocity;
    c.host_dt = cp.flow_dt;
    c.host_time = cp.flow_time;
    c.dev = cp.dev_scalars;
    c.dev_time_end = cp.dev_time_end;
    c.max_rod_dt = cp.max_rod_dt;
    c.damping_rate = cp.damping_rate;
    c.drive_phase = cp.drive_phase;
    c.drive_amp = cp.drive_amplitude;
    c.drive_freq = cp.drive_frequency;
    for (int a = 0; a < 3; ++a) c.axis[a] = cp.drive_axis[a];
    // pass scratch, clamp frames, reciprocals, then x, v (3 (n + 1) each), Q (9 n), w (3 n), the
    // external forces (3 (n + 1)) and torques (3 n)
    const int ne = b.n_elems;
    const size_t smem = (size_t)(rod::scratch_doubles(ne) + 48 + 3 * ne + 9 * (ne + 1) + 15 * ne) * sizeof(double);
    if (smem > 48 * 1024)
        SG_TRY(cuda_status(cudaFuncSetAttribute(rod_coupled_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem),
                           "rod coupled smem"));
    rod_coupled_kernel<T><<<b.n_rods, 256, smem, stream>>>(b, c);
    return launch_status("rod coupled sub-steps");
}
}  // namespace sg

extern "C" int sg_rod_batch_coupled_substeps(const sg_rod_batch* batch, const sg_rod_coupling* cp, void* stream) {
    SG_TRY(rod_batch_check(batch, 3));
    SG_REQUIRE(cp, SG_ERR_INVALID_ARG, "rod coupling: null coupling");
    const sg_rod_batch& b = *batch;
    SG_REQUIRE(b.n_elems <= 256, SG_ERR_SHAPE, "rod coupling: 1 to 256 elements per rod");
    SG_REQUIRE(b.directors && b.omega && b.rest_lengths && b.shear_matrix && b.mass_second_moment &&
                   b.inv_mass_second_moment && b.rest_sigma,
               SG_ERR_INVALID_ARG, "rod coupling: null rod array");
    SG_REQUIRE(b.n_elems == 1 || (b.rest_voronoi_lengths && b.bend_matrix && b.rest_kappa), SG_ERR_INVALID_ARG,
               "rod coupling: null Voronoi array");
    SG_REQUIRE(!b.clamped || (b.clamp_position && b.clamp_directors), SG_ERR_INVALID_ARG,
               "rod coupling: clamped rods need the clamp position and directors");
    SG_REQUIRE(cp->dtype == SG_F32 || cp->dtype == SG_F64, SG_ERR_INVALID_ARG, "rod coupling: bad dtype");
    SG_REQUIRE(cp->kernel_type == 0 || cp->kernel_type == 1, SG_ERR_INVALID_ARG, "rod coupling: bad kernel type");
    SG_REQUIRE(cp->nz >= 4 && cp->ny >= 4 && cp->nx >= 4 && cp->dx > 0, SG_ERR_SHAPE, "rod coupling: bad grid");
    SG_REQUIRE(cp->flow_velocity && cp->marker_position && cp->marker_velocity && cp->nearest && cp->weights &&
                   cp->flow_velocity_lag && cp->velocity_mismatch && cp->position_mismatch && cp->lag_forcing &&
                   cp->status,
               SG_ERR_INVALID_ARG, "rod coupling: null marker or field array");
    SG_REQUIRE(cp->dev_scalars ? cp->dev_time_end != nullptr : cp->flow_dt > 0, SG_ERR_INVALID_ARG,
               "rod coupling: a positive host dt, or the device dt and time");
    SG_REQUIRE(cp->max_rod_dt > 0, SG_ERR_INVALID_ARG, "rod coupling: max_rod_dt must be positive");
    if (cp->drive_phase) {
        const double* a = cp->drive_axis;
        const double norm = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        SG_REQUIRE(fabs(norm - 1.0) < 1e-12, SG_ERR_INVALID_ARG, "rod coupling: drive_axis must be a unit vector");
    }
    auto s = (cudaStream_t)stream;
    return cp->dtype == SG_F32 ? sg::rod_coupled_launch<float>(b, *cp, s) : sg::rod_coupled_launch<double>(b, *cp, s);
}
