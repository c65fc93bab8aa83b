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

extern "C" int sg_ib_interaction(int dtype, int dim, int nz, int ny, int nx, double dx, double shift, int n_lag,
                                 int kernel_type, const double* position, const double* body_velocity,
                                 const void* eul_velocity, int32_t* nearest, void* weights, void* flow_velocity,
                                 void* velocity_mismatch, void* position_mismatch, void* forcing, double stiffness,
                                 double damping, int do_xi_step, double xi_dt, const sg_step_scalars* dev_scalars,
                                 int32_t* status_dev, void* stream_) {
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "ib interaction: dim must be 2 or 3");
    SG_REQUIRE(n_lag >= 1, SG_ERR_INVALID_ARG, "ib interaction: n_lag must be >= 1");
    SG_REQUIRE(kernel_type == 0 || kernel_type == 1, SG_ERR_INVALID_ARG, "ib interaction: bad kernel type");
    SG_REQUIRE(position && body_velocity && eul_velocity && nearest && weights && flow_velocity &&
                   velocity_mismatch && position_mismatch && forcing && status_dev,
               SG_ERR_INVALID_ARG, "ib interaction: null argument");
    SG_REQUIRE(dx > 0, SG_ERR_INVALID_ARG, "ib interaction: dx must be positive");
    if (dim == 2) nz = 1;
    auto stream = (cudaStream_t)stream_;
    if (dtype == SG_F32) {
        IBParams<float> p{dim, nz, ny, nx, n_lag, kernel_type, dx, shift, position, body_velocity,
                          (const float*)eul_velocity, nearest, (float*)weights, (float*)flow_velocity,
                          (float*)velocity_mismatch, (float*)position_mismatch, (float*)forcing,
                          stiffness, damping, do_xi_step, xi_dt, dev_scalars, status_dev};
        ib_interaction_launch<float>(p, stream);
    } else {
        SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "ib interaction: bad dtype");
        IBParams<double> p{dim, nz, ny, nx, n_lag, kernel_type, dx, shift, position, body_velocity,
                           (const double*)eul_velocity, nearest, (double*)weights, (double*)flow_velocity,
                           (double*)velocity_mismatch, (double*)position_mismatch, (double*)forcing,
                           stiffness, damping, do_xi_step, xi_dt, dev_scalars, status_dev};
        ib_interaction_launch<double>(p, stream);
    }
    return launch_status("ib_interaction");
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

extern "C" int sg_ib_spread(int dtype, int dim, int nz, int ny, int nx, int n_lag, const int32_t* nearest,
                            const void* weights, const void* forcing, void* eul_forcing, int reset, void* stream_) {
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "ib spread: dim must be 2 or 3");
    SG_REQUIRE(nearest && weights && forcing && eul_forcing && n_lag >= 1, SG_ERR_INVALID_ARG,
               "ib spread: bad argument");
    if (dim == 2) nz = 1;
    auto stream = (cudaStream_t)stream_;
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

extern "C" int sg_ib_mismatch_step(int dtype, int n, void* xi, const void* du, double dt, void* stream_) {
    SG_REQUIRE(xi && du && n >= 1, SG_ERR_INVALID_ARG, "ib mismatch step: bad argument");
    auto stream = (cudaStream_t)stream_;
    if (dtype == SG_F32) mismatch_step_kernel<float><<<ceil_div(n, 256), 256, 0, stream>>>(n, (float*)xi, (const float*)du, dt);
    else mismatch_step_kernel<double><<<ceil_div(n, 256), 256, 0, stream>>>(n, (double*)xi, (const double*)du, dt);
    return launch_status("ib_mismatch_step");
}
