// Immersed-boundary coupling: Eulerian <-> Lagrangian transfer with
// virtual-boundary forcing (immersed_boundary_ops/VirtualBoundaryForcing.py,
// EulerianLagrangianGridCommunicator{2,3}D.py).
//
// sg_ib_interaction: one warp per marker.  Lanes compute the nearest grid
// index (numpy floor division of (X - shift) / dx in double), the per-axis
// support and delta weights, then the windowed interpolation of the flow
// velocity (4^dim cells, warp-shuffle reduction), the velocity mismatch and the
// feedback force F = K xi + C dU.
//
// sg_ib_spread: deterministic spreading without floating-point atomics.  One
// thread per (marker, window cell); the thread whose marker is the lowest-index
// marker touching that cell owns the cell and accumulates, in marker index
// order, every marker's F * phi into it -- the same per-cell summation order as
// the reference's serial marker loop.
#include "ib.cuh"


using namespace sg;

template <typename T>
static void ib_interaction_launch(const IBParams<T>& p, cudaStream_t stream) {
    // two markers (warps) per block: bodies of ~100 markers spread over many SMs
    const unsigned blocks = ceil_div((int64_t)p.n_lag * 32, 64);
    if (p.dim == 2) ib_interaction_kernel<T, 2><<<blocks, 64, 0, stream>>>(p);
    else ib_interaction_kernel<T, 3><<<blocks, 64, 0, stream>>>(p);
}

static int ib_interaction_impl(int dtype, int dim, int nz, int ny, int nx, double dx, double shift, int n_lag,
                               int kernel_type, const double* position, const double* body_velocity,
                               const void* eul_velocity, int32_t* nearest, void* weights, void* flow_velocity,
                               void* velocity_mismatch, void* position_mismatch, void* forcing, double stiffness,
                               double damping, int do_xi_step, double xi_dt, const sg_step_scalars* dev_scalars,
                               int32_t* status_dev, cudaStream_t stream, const IBDynArgs* dyn = nullptr) {
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "ib interaction: dim must be 2 or 3");
    SG_REQUIRE(n_lag >= 1, SG_ERR_INVALID_ARG, "ib interaction: n_lag must be >= 1");
    SG_REQUIRE(kernel_type == 0 || kernel_type == 1, SG_ERR_INVALID_ARG, "ib interaction: bad kernel type");
    SG_REQUIRE(position && body_velocity && eul_velocity && nearest && weights && flow_velocity &&
                   velocity_mismatch && position_mismatch && forcing && status_dev,
               SG_ERR_INVALID_ARG, "ib interaction: null argument");
    SG_REQUIRE(dx > 0, SG_ERR_INVALID_ARG, "ib interaction: dx must be positive");
    if (dim == 2) nz = 1;
    if (dtype == SG_F32) {
        IBParams<float> p{dim, nz, ny, nx, n_lag, kernel_type, dx, shift, position, body_velocity,
                          (const float*)eul_velocity, nearest, (float*)weights, (float*)flow_velocity,
                          (float*)velocity_mismatch, (float*)position_mismatch, (float*)forcing,
                          stiffness, damping, do_xi_step, xi_dt, dev_scalars, status_dev, dyn};
        ib_interaction_launch<float>(p, stream);
    } else {
        SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "ib interaction: bad dtype");
        IBParams<double> p{dim, nz, ny, nx, n_lag, kernel_type, dx, shift, position, body_velocity,
                           (const double*)eul_velocity, nearest, (double*)weights, (double*)flow_velocity,
                           (double*)velocity_mismatch, (double*)position_mismatch, (double*)forcing,
                           stiffness, damping, do_xi_step, xi_dt, dev_scalars, status_dev, dyn};
        ib_interaction_launch<double>(p, stream);
    }
    return launch_status("ib_interaction");
}

extern "C" int sg_ib_interaction(int dtype, int dim, int nz, int ny, int nx, double dx, double shift, int n_lag,
                                 int kernel_type, const double* position, const double* body_velocity,
                                 const void* eul_velocity, int32_t* nearest, void* weights, void* flow_velocity,
                                 void* velocity_mismatch, void* position_mismatch, void* forcing, double stiffness,
                                 double damping, int do_xi_step, double xi_dt, const sg_step_scalars* dev_scalars,
                                 int32_t* status_dev, void* stream_) {
    return ib_interaction_impl(dtype, dim, nz, ny, nx, dx, shift, n_lag, kernel_type, position, body_velocity,
                               eul_velocity, nearest, weights, flow_velocity, velocity_mismatch, position_mismatch,
                               forcing, stiffness, damping, do_xi_step, xi_dt, dev_scalars, status_dev,
                               (cudaStream_t)stream_);
}

template <typename T>
static void ib_spread_launch(const SpreadParams<T>& p, cudaStream_t stream) {
    const int cells = p.dim == 2 ? 16 : 64;
    const int64_t threads = (int64_t)p.n_lag * cells;
    // one warp per (marker, window cell) with the markers' nearest indices
    // staged in shared memory, when they fit in 48 KB
    const size_t staged = (size_t)p.dim * p.n_lag * sizeof(int);
    if (staged <= 48 * 1024) {
        const unsigned blocks = ceil_div(threads * 32, 256);
        if (p.dim == 2) ib_spread_warp_kernel<T, 2><<<blocks, 256, staged, stream>>>(p);
        else ib_spread_warp_kernel<T, 3><<<blocks, 256, staged, stream>>>(p);
    } else {
        const unsigned blocks = ceil_div(threads, 256);
        if (p.dim == 2) ib_spread_kernel<T, 2><<<blocks, 256, 0, stream>>>(p);
        else ib_spread_kernel<T, 3><<<blocks, 256, 0, stream>>>(p);
    }
}

static int ib_spread_impl(int dtype, int dim, int nz, int ny, int nx, int n_lag, const int32_t* nearest,
                          const void* weights, const void* forcing, void* eul_forcing, int reset, cudaStream_t stream) {
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "ib spread: dim must be 2 or 3");
    SG_REQUIRE(nearest && weights && forcing && eul_forcing && n_lag >= 1, SG_ERR_INVALID_ARG,
               "ib spread: bad argument");
    if (dim == 2) nz = 1;
    const int64_t ncell = (int64_t)nz * ny * nx;
    if (dtype == SG_F32) {
        if (reset) {
            zero_kernel<float><<<ceil_div(dim * ncell, 256), 256, 0, stream>>>(dim * ncell, (float*)eul_forcing);
        }
        SpreadParams<float> p{dim, nz, ny, nx, n_lag, 0, nearest, (const float*)weights, (const float*)forcing,
                              (float*)eul_forcing};
        ib_spread_launch<float>(p, stream);
    } else {
        SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "ib spread: bad dtype");
        if (reset) {
            zero_kernel<double><<<ceil_div(dim * ncell, 256), 256, 0, stream>>>(dim * ncell, (double*)eul_forcing);
        }
        SpreadParams<double> p{dim, nz, ny, nx, n_lag, 0, nearest, (const double*)weights, (const double*)forcing,
                               (double*)eul_forcing};
        ib_spread_launch<double>(p, stream);
    }
    return launch_status("ib_spread");
}

extern "C" int sg_ib_spread(int dtype, int dim, int nz, int ny, int nx, int n_lag, const int32_t* nearest,
                            const void* weights, const void* forcing, void* eul_forcing, int reset, void* stream_) {
    return ib_spread_impl(dtype, dim, nz, ny, nx, n_lag, nearest, weights, forcing, eul_forcing, reset,
                          (cudaStream_t)stream_);
}

extern "C" int sg_ib_mismatch_step(int dtype, int n, void* xi, const void* du, double dt, void* stream_) {
    SG_REQUIRE(xi && du && n >= 1, SG_ERR_INVALID_ARG, "ib mismatch step: bad argument");
    auto stream = (cudaStream_t)stream_;
    if (dtype == SG_F32) mismatch_step_kernel<float><<<ceil_div(n, 256), 256, 0, stream>>>(n, (float*)xi, (const float*)du, dt);
    else mismatch_step_kernel<double><<<ceil_div(n, 256), 256, 0, stream>>>(n, (double*)xi, (const double*)du, dt);
    return launch_status("ib_mismatch_step");
}

// ---------------------------------------------------------------- bound coupling
// One interactor's fixed arguments, its pinned staging and its events, so that
// the per-step host call (VirtualBoundaryForcing.__call__ of an immersed body:
// upload the marker kinematics, interact, spread, and queue the copy of the
// Lagrangian forcing a host body integrator reads) is one call of few arguments.
struct sg_ib_binding_s {
    int dtype = SG_F32, dim = 2, nz = 1, ny = 0, nx = 0, n_lag = 0, kernel = 0;
    double dx = 0.0, shift = 0.0;
    int32_t* nearest = nullptr;
    void* weights = nullptr;
    void* flow_velocity = nullptr;
    void* vel_mismatch = nullptr;
    void* pos_mismatch = nullptr;
    void* lag_forcing = nullptr;
    int32_t* status = nullptr;
    double* dev_kin = nullptr;          // (2, dim, n_lag) float64 on the device: positions, velocities
    double* kin_host[2] = {nullptr, nullptr};  // pinned staging slots, same layout
    cudaEvent_t kin_done[2] = {nullptr, nullptr};
    void* forcing_host = nullptr;       // pinned (dim, n_lag) of the field type
    cudaEvent_t forcing_done = nullptr;
    // graphs of the per-call work, one per (staging slot, spread mode, forcing copy, Eulerian fields),
    // captured on first use; the per-call scalars come from `dyn`
    IBDynArgs* dyn = nullptr;
    cudaStream_t capture_stream = nullptr;
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        int slot = 0, spread_mode = 0, copy = 0;
        const void* u = nullptr;
        void* f = nullptr;
    } graphs[8];
    int n_graphs = 0, builds = 0;
    bool graphs_off = false;
};

static void ib_binding_free(sg_ib_binding_s* b) {
    if (!b) return;
    for (int k = 0; k < b->n_graphs; ++k)
        if (b->graphs[k].exec) cudaGraphExecDestroy(b->graphs[k].exec);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    cudaFree(b->dyn);
    for (int k = 0; k < 2; ++k) {
        if (b->kin_done[k]) cudaEventDestroy(b->kin_done[k]);
        cudaFreeHost(b->kin_host[k]);
    }
    if (b->forcing_done) cudaEventDestroy(b->forcing_done);
    cudaFreeHost(b->forcing_host);
    delete b;
}

extern "C" int sg_ib_bind(int dtype, int dim, int nz, int ny, int nx, double dx, double shift, int n_lag,
                          int kernel_type, int32_t* nearest, void* weights, void* flow_velocity,
                          void* velocity_mismatch, void* position_mismatch, void* forcing, int32_t* status_dev,
                          double* dev_kinematics, sg_ib_binding* out) {
    SG_REQUIRE(out, SG_ERR_INVALID_ARG, "ib bind: null output");
    *out = nullptr;
    SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, SG_ERR_INVALID_ARG, "ib bind: bad dtype");
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "ib bind: dim must be 2 or 3");
    SG_REQUIRE(n_lag >= 1 && ny >= 1 && nx >= 1 && (dim == 2 || nz >= 1), SG_ERR_INVALID_ARG, "ib bind: bad size");
    SG_REQUIRE(kernel_type == 0 || kernel_type == 1, SG_ERR_INVALID_ARG, "ib bind: bad kernel type");
    SG_REQUIRE(dx > 0, SG_ERR_INVALID_ARG, "ib bind: dx must be positive");
    SG_REQUIRE(nearest && weights && flow_velocity && velocity_mismatch && position_mismatch && forcing &&
                   status_dev && dev_kinematics,
               SG_ERR_INVALID_ARG, "ib bind: null argument");
    auto* b = new sg_ib_binding_s();
    b->dtype = dtype;
    b->dim = dim;
    b->nz = dim == 2 ? 1 : nz;
    b->ny = ny;
    b->nx = nx;
    b->n_lag = n_lag;
    b->kernel = kernel_type;
    b->dx = dx;
    b->shift = shift;
    b->nearest = nearest;
    b->weights = weights;
    b->flow_velocity = flow_velocity;
    b->vel_mismatch = velocity_mismatch;
    b->pos_mismatch = position_mismatch;
    b->lag_forcing = forcing;
    b->status = status_dev;
    b->dev_kin = dev_kinematics;
    const size_t kin_bytes = (size_t)2 * dim * n_lag * sizeof(double);
    const size_t f_bytes = (size_t)dim * n_lag * (dtype == SG_F32 ? sizeof(float) : sizeof(double));
    int st = SG_OK;
    for (int k = 0; k < 2 && st == SG_OK; ++k) {
        st = cuda_status(cudaMallocHost((void**)&b->kin_host[k], kin_bytes), "ib bind: pinned staging");
        if (st == SG_OK)
            st = cuda_status(cudaEventCreateWithFlags(&b->kin_done[k], cudaEventDisableTiming), "ib bind: event");
    }
    if (st == SG_OK) st = cuda_status(cudaMallocHost(&b->forcing_host, f_bytes), "ib bind: pinned forcing");
    if (st == SG_OK)
        st = cuda_status(cudaEventCreateWithFlags(&b->forcing_done, cudaEventDisableTiming), "ib bind: event");
    if (st == SG_OK) st = cuda_status(cudaMalloc((void**)&b->dyn, sizeof(IBDynArgs)), "ib bind: argument block");
    if (st != SG_OK) {
        ib_binding_free(b);
        return st;
    }
    *out = b;
    return SG_OK;
}

extern "C" int sg_ib_binding_buffers(sg_ib_binding b, double** kin_slot0, double** kin_slot1, void** forcing_host) {
    SG_REQUIRE(b && kin_slot0 && kin_slot1 && forcing_host, SG_ERR_INVALID_ARG, "ib buffers: null argument");
    *kin_slot0 = b->kin_host[0];
    *kin_slot1 = b->kin_host[1];
    *forcing_host = b->forcing_host;
    return SG_OK;
}

extern "C" int sg_ib_binding_wait(sg_ib_binding b, int which) {
    SG_REQUIRE(b && which >= 0 && which <= 2, SG_ERR_INVALID_ARG, "ib wait: bad argument");
    return cuda_status(cudaEventSynchronize(which < 2 ? b->kin_done[which] : b->forcing_done), "ib wait");
}

// The per-call work of a bound interactor on `stream`.  dyn: the interaction reads K, C and the xi
// step from the binding's device block (a graph being recorded); capturing: the event records
// become nodes of the graph being captured.
static int ib_bound_work(sg_ib_binding_s* b, int kin_slot, const void* eul_velocity, void* eul_forcing,
                         int spread_mode, double stiffness, double damping, int do_xi_step, double xi_dt,
                         int copy_forcing, bool dyn, bool capturing, cudaStream_t stream) {
    const int64_t nk = (int64_t)b->dim * b->n_lag;
    const unsigned rec = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (kin_slot >= 0) {
        SG_TRY(cuda_status(cudaMemcpyAsync(b->dev_kin, b->kin_host[kin_slot], (size_t)2 * nk * sizeof(double),
                                           cudaMemcpyHostToDevice, stream),
                           "ib bound step: kinematics upload"));
        SG_TRY(cuda_status(cudaEventRecordWithFlags(b->kin_done[kin_slot], stream, rec), "ib bound step: event"));
    }
    SG_TRY(ib_interaction_impl(b->dtype, b->dim, b->nz, b->ny, b->nx, b->dx, b->shift, b->n_lag, b->kernel,
                               b->dev_kin, b->dev_kin + nk, eul_velocity, b->nearest, b->weights, b->flow_velocity,
                               b->vel_mismatch, b->pos_mismatch, b->lag_forcing, stiffness, damping, do_xi_step,
                               xi_dt, nullptr, b->status, stream, dyn ? b->dyn : nullptr));
    if (spread_mode >= 0)
        SG_TRY(ib_spread_impl(b->dtype, b->dim, b->nz, b->ny, b->nx, b->n_lag, b->nearest, b->weights,
                              b->lag_forcing, eul_forcing, spread_mode, stream));
    if (copy_forcing) {
        const size_t f_bytes = (size_t)nk * (b->dtype == SG_F32 ? sizeof(float) : sizeof(double));
        SG_TRY(cuda_status(cudaMemcpyAsync(b->forcing_host, b->lag_forcing, f_bytes, cudaMemcpyDeviceToHost, stream),
                           "ib bound step: forcing copy"));
        SG_TRY(cuda_status(cudaEventRecordWithFlags(b->forcing_done, stream, rec), "ib bound step: event"));
    }
    return SG_OK;
}

__global__ void set_ib_dyn_kernel(IBDynArgs v, IBDynArgs* dst) { *dst = v; }

static void ib_graphs_off(sg_ib_binding_s* b) {
    cudaGetLastError();  // a failed capture leaves no sticky error: direct launches follow
    b->graphs_off = true;
}

// The captured graph of one call variant, captured now if it is new; null when graphs are off.
static cudaGraphExec_t ib_bound_graph(sg_ib_binding_s* b, int kin_slot, const void* u, void* f, int spread_mode,
                                      int copy_forcing) {
    if (b->graphs_off) return nullptr;
    for (int k = 0; k < b->n_graphs; ++k) {
        const auto& e = b->graphs[k];
        if (e.slot == kin_slot && e.spread_mode == spread_mode && e.copy == copy_forcing && e.u == u && e.f == f)
            return e.exec;
    }
    if (b->builds >= 16) {  // fields that keep moving: direct launches from now on
        ib_graphs_off(b);
        return nullptr;
    }
    ++b->builds;
    if (!b->capture_stream && cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
        b->capture_stream = nullptr;
        ib_graphs_off(b);
        return nullptr;
    }
    if (cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        ib_graphs_off(b);
        return nullptr;
    }
    const int st = ib_bound_work(b, kin_slot, u, f, spread_mode, 0.0, 0.0, 0, 0.0, copy_forcing, true, true,
                                 b->capture_stream);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->capture_stream, &g);
    cudaGraphExec_t exec = nullptr;
    if (st != SG_OK || e != cudaSuccess || !g || cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        ib_graphs_off(b);
        return nullptr;
    }
    cudaGraphDestroy(g);
    const int k = b->n_graphs < 8 ? b->n_graphs++ : b->builds % 8;
    if (b->graphs[k].exec) cudaGraphExecDestroy(b->graphs[k].exec);
    b->graphs[k] = sg_ib_binding_s::Graph{exec, kin_slot, spread_mode, copy_forcing, u, f};
    return exec;
}

extern "C" int sg_ib_bound_step(sg_ib_binding b, int kin_slot, const void* eul_velocity, void* eul_forcing,
                                int spread_mode, double stiffness, double damping, int do_xi_step, double xi_dt,
                                int copy_forcing, void* stream_) {
    SG_REQUIRE(b && eul_velocity, SG_ERR_INVALID_ARG, "ib bound step: null argument");
    SG_REQUIRE(kin_slot >= -1 && kin_slot <= 1, SG_ERR_INVALID_ARG, "ib bound step: bad staging slot");
    SG_REQUIRE(spread_mode >= -1 && spread_mode <= 1, SG_ERR_INVALID_ARG, "ib bound step: bad spread mode");
    SG_REQUIRE(spread_mode < 0 || eul_forcing, SG_ERR_INVALID_ARG, "ib bound step: no Eulerian forcing");
    auto stream = (cudaStream_t)stream_;
    copy_forcing = copy_forcing ? 1 : 0;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess) {
        cudaGetLastError();
        cs = cudaStreamCaptureStatusActive;  // unknown: take the direct path, events as graph nodes
    }
    if (cs == cudaStreamCaptureStatusNone) {
        // one replay of the captured call: 2 launches instead of 4 to 6
        const cudaGraphExec_t g = ib_bound_graph(b, kin_slot, eul_velocity, eul_forcing, spread_mode, copy_forcing);
        if (g) {
            set_ib_dyn_kernel<<<1, 1, 0, stream>>>(IBDynArgs{stiffness, damping, do_xi_step, xi_dt}, b->dyn);
            SG_TRY(launch_status("ib bound step arguments"));
            return cuda_status(cudaGraphLaunch(g, stream), "ib bound step graph launch");
        }
    }
    return ib_bound_work(b, kin_slot, eul_velocity, eul_forcing, spread_mode, stiffness, damping, do_xi_step, xi_dt,
                         copy_forcing, false, cs != cudaStreamCaptureStatusNone, stream);
}

extern "C" int sg_ib_unbind(sg_ib_binding b) {
    ib_binding_free(b);
    return SG_OK;
}

// ------------------------------------------------------------ host-side forcing-grid kinematics
// CosseratRodElementCentricForcingGrid (cosserat_rod_forcing_grids.py:82-130) on the host:
// element centres (x_i + x_{i+1}) / 2 and the mass-weighted element velocities of pyelastica's
// _node_to_element_velocity, (m_{i+1} v_{i+1} + m_i v_i) / (m_{i+1} + m_i), with the operations in
// numpy's order and without fused multiply-adds, written to the grid's position/velocity arrays and,
// when given, to a (2, grid_dim, n_elems) staging slot of sg_ib_binding_buffers.  Node-array rows
// may be strided (views into a larger block of rods).
extern "C" int sg_rod_element_kinematics(int grid_dim, int n_elems, const double* node_position,
                                         int64_t position_row_stride, const double* node_velocity,
                                         int64_t velocity_row_stride, const double* mass, double* position_out,
                                         double* velocity_out, double* staging) {
    SG_REQUIRE(grid_dim == 2 || grid_dim == 3, SG_ERR_INVALID_ARG, "rod kinematics: dim must be 2 or 3");
    SG_REQUIRE(n_elems >= 1, SG_ERR_INVALID_ARG, "rod kinematics: n_elems must be >= 1");
    SG_REQUIRE(node_position && node_velocity && mass && position_out && velocity_out, SG_ERR_INVALID_ARG,
               "rod kinematics: null argument");
    SG_REQUIRE(position_row_stride >= n_elems + 1 && velocity_row_stride >= n_elems + 1, SG_ERR_INVALID_ARG,
               "rod kinematics: row stride shorter than a row");
    for (int d = 0; d < grid_dim; ++d) {
        const double* p = node_position + (int64_t)d * position_row_stride;
        const double* v = node_velocity + (int64_t)d * velocity_row_stride;
        for (int e = 0; e < n_elems; ++e) {
            const double x = (p[e + 1] + p[e]) / 2.0;
            const double a = mass[e + 1] * v[e + 1];
            const double b = mass[e] * v[e];
            const double u = (a + b) / (mass[e + 1] + mass[e]);
            position_out[(int64_t)d * n_elems + e] = x;
            velocity_out[(int64_t)d * n_elems + e] = u;
            if (staging) {
                staging[(int64_t)d * n_elems + e] = x;
                staging[(int64_t)(grid_dim + d) * n_elems + e] = u;
            }
        }
    }
    return SG_OK;
}
