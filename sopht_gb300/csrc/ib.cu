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
#include <cmath>

#include "common.cuh"
#include "flow_kernels.cuh"

namespace sg {

// numpy floor_divide for doubles (divmod-based: fmod, exact quotient
// adjustment, then floor with a round-to-nearest correction).
__device__ __forceinline__ double np_floor_divide(double a, double b) {
    double mod = fmod(a, b);
    double div = (a - mod) / b;
    if (mod != 0.0) {
        if ((b < 0) != (mod < 0)) div -= 1.0;
    }
    double fl;
    if (div != 0.0) {
        fl = floor(div);
        if (div - fl > 0.5) fl += 1.0;
    } else {
        fl = copysign(0.0, a / b);
    }
    return fl;
}

template <typename T> __device__ __forceinline__ T dev_cos(T x);
template <> __device__ __forceinline__ float dev_cos<float>(float x) { return cosf(x); }
template <> __device__ __forceinline__ double dev_cos<double>(double x) { return cos(x); }

// Peskin (2002, eq. 6.27) one-dimensional 4-point delta of |r|/dx.
template <typename T> __device__ __forceinline__ T peskin_phi(T a) {
    T v = T(0);
    if (a < T(1)) v = T(3) - T(2) * a + sqrt(fabs(T(1) + T(4) * a - T(4) * a * a));
    else if (a < T(2)) v = T(5) - T(2) * a - sqrt(fabs(T(-7) + T(12) * a - T(4) * a * a));
    return v;
}

template <typename T> struct IBParams {
    int dim, nz, ny, nx, n_lag, kernel;
    double dx, shift;
    const double* pos;
    const double* body_vel;
    const T* u;
    int32_t* nearest;
    T* weights;
    T* flow_vel;
    T* vel_mismatch;
    T* pos_mismatch;
    T* forcing;
    double K, C;
    int xi_step;
    double xi_dt;
    const sg_step_scalars* dev;
    int32_t* status;
};

template <typename T>
__global__ void __launch_bounds__(256) ib_interaction_kernel(IBParams<T> p) {
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= p.n_lag) return;
    const int dim = p.dim;
    const int n = p.n_lag;
    const T dxT = (T)p.dx;
    int near[3] = {0, 0, 0};
    T phi[3][4];
    const int ext[3] = {p.nx, p.ny, p.nz};
    bool inside = true;
    for (int d = 0; d < dim; ++d) {
        const double X = p.pos[d * n + i];
        const double nd = np_floor_divide(X - p.shift, p.dx);
        near[d] = (int)nd;
        if (near[d] - 1 < 0 || near[d] + 2 > ext[d] - 1) inside = false;
        for (int k = 0; k < 4; ++k) {
            // support: stored in the field precision, then scaled by 1/dx in it
            const T r = (T)((double)(near[d] + k - 1) * p.dx + p.shift - X);
            const T rn = r / dxT;
            if (p.kernel == 0) phi[d][k] = T(1) + dev_cos<T>((T)(0.5 * 3.14159265358979323846) * rn);
            else phi[d][k] = peskin_phi<T>(fabs(rn));
        }
    }
    if (lane < dim) p.nearest[lane * n + i] = near[lane];
    // optional VirtualBoundaryForcing.time_step: xi += dt * dU (previous dU)
    if (p.xi_step && lane < dim) {
        const T dt = (T)(p.dev ? p.dev->dt : p.xi_dt);
        p.pos_mismatch[lane * n + i] = p.pos_mismatch[lane * n + i] + dt * p.vel_mismatch[lane * n + i];
    }
    if (!inside) {
        if (lane == 0) atomicExch(p.status, SG_ERR_OUT_OF_DOMAIN);
        const int cells = dim == 2 ? 16 : 64;
        for (int c = lane; c < cells; c += 32) p.weights[c * n + i] = T(0);
        return;
    }
    T pref;
    if (p.kernel == 0) {
        const T q = T(0.25) / dxT;
        pref = dim == 2 ? q * q : (T)((double)q * (double)q * (double)q);
    } else {
        const T q = T(0.125) / dxT;
        pref = dim == 2 ? q * q : (T)((double)q * (double)q * (double)q);
    }
    const int cells = dim == 2 ? 16 : 64;
    const int64_t plane = (int64_t)p.ny * p.nx;
    const int64_t ncell = plane * (dim == 3 ? p.nz : 1);
    T acc[3] = {T(0), T(0), T(0)};
    for (int c = lane; c < cells; c += 32) {
        const int bx = c & 3, by = (c >> 2) & 3, bz = c >> 4;
        T w = pref * phi[0][bx] * phi[1][by];
        if (dim == 3) w = w * phi[2][bz];
        p.weights[c * n + i] = w;
        const int gx = near[0] - 1 + bx, gy = near[1] - 1 + by;
        const int gz = dim == 3 ? near[2] - 1 + bz : 0;
        const int64_t g = (int64_t)gz * plane + (int64_t)gy * p.nx + gx;
        for (int d = 0; d < dim; ++d) acc[d] += p.u[d * ncell + g] * w;
    }
    for (int d = 0; d < dim; ++d)
        for (int o = 16; o > 0; o >>= 1) acc[d] += __shfl_xor_sync(0xffffffffu, acc[d], o);
    if (lane < dim) {
        const int d = lane;
        const T dxd = dim == 2 ? dxT * dxT : dxT * dxT * dxT;
        const T U = acc[d] * dxd;
        p.flow_vel[d * n + i] = U;
        const T dU = (T)((double)U - p.body_vel[d * n + i]);
        p.vel_mismatch[d * n + i] = dU;
        p.forcing[d * n + i] = (T)(p.K * (double)p.pos_mismatch[d * n + i] + p.C * (double)dU);
    }
}

template <typename T> struct SpreadParams {
    int dim, nz, ny, nx, n_lag, reset;
    const int32_t* nearest;
    const T* weights;
    const T* forcing;
    T* eul;
};

template <typename T>
__global__ void __launch_bounds__(256) ib_spread_kernel(SpreadParams<T> p) {
    const int cells = p.dim == 2 ? 16 : 64;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)p.n_lag * cells) return;
    const int i = (int)(t / cells), c = (int)(t % cells);
    const int n = p.n_lag;
    const int dim = p.dim;
    int cell[3];
    cell[0] = p.nearest[i] - 1 + (c & 3);
    cell[1] = p.nearest[n + i] - 1 + ((c >> 2) & 3);
    cell[2] = dim == 3 ? p.nearest[2 * n + i] - 1 + (c >> 4) : 0;
    const int ext[3] = {p.nx, p.ny, dim == 3 ? p.nz : 1};
    for (int d = 0; d < dim; ++d)
        if (cell[d] < 0 || cell[d] >= ext[d]) return;  // marker reported out of domain
    auto offset_in = [&](int j, int& k) -> bool {
        int o[3] = {0, 0, 0};
        for (int d = 0; d < dim; ++d) {
            o[d] = cell[d] - (p.nearest[d * n + j] - 1);
            if (o[d] < 0 || o[d] > 3) return false;
        }
        k = o[0] + 4 * o[1] + 16 * o[2];
        return true;
    };
    int k;
    for (int j = 0; j < i; ++j)
        if (offset_in(j, k)) return;  // a lower-index marker owns this cell
    const int64_t plane = (int64_t)p.ny * p.nx;
    const int64_t ncell = plane * (dim == 3 ? p.nz : 1);
    const int64_t g = (int64_t)cell[2] * plane + (int64_t)cell[1] * p.nx + cell[0];
    T acc[3];
    for (int d = 0; d < dim; ++d) acc[d] = p.reset ? T(0) : p.eul[d * ncell + g];
    for (int j = i; j < n; ++j) {
        if (!offset_in(j, k)) continue;
        const T w = p.weights[k * n + j];
        for (int d = 0; d < dim; ++d) acc[d] = acc[d] + p.forcing[d * n + j] * w;
    }
    for (int d = 0; d < dim; ++d) p.eul[d * ncell + g] = acc[d];
}

template <typename T>
__global__ void __launch_bounds__(256) mismatch_step_kernel(int n, T* xi, const T* du, double dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) xi[i] = xi[i] + (T)dt * du[i];
}

template <typename T>
__global__ void __launch_bounds__(256) zero_kernel(int64_t n, T* f) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) f[i] = T(0);
}

}  // namespace sg

using namespace sg;

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
    const unsigned blocks = ceil_div((int64_t)n_lag * 32, 256);
    if (dtype == SG_F32) {
        IBParams<float> p{dim, nz, ny, nx, n_lag, kernel_type, dx, shift, position, body_velocity,
                          (const float*)eul_velocity, nearest, (float*)weights, (float*)flow_velocity,
                          (float*)velocity_mismatch, (float*)position_mismatch, (float*)forcing,
                          stiffness, damping, do_xi_step, xi_dt, dev_scalars, status_dev};
        ib_interaction_kernel<float><<<blocks, 256, 0, stream>>>(p);
    } else {
        SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "ib interaction: bad dtype");
        IBParams<double> p{dim, nz, ny, nx, n_lag, kernel_type, dx, shift, position, body_velocity,
                           (const double*)eul_velocity, nearest, (double*)weights, (double*)flow_velocity,
                           (double*)velocity_mismatch, (double*)position_mismatch, (double*)forcing,
                           stiffness, damping, do_xi_step, xi_dt, dev_scalars, status_dev};
        ib_interaction_kernel<double><<<blocks, 256, 0, stream>>>(p);
    }
    return launch_status("ib_interaction");
}

extern "C" int sg_ib_spread(int dtype, int dim, int nz, int ny, int nx, int n_lag, const int32_t* nearest,
                            const void* weights, const void* forcing, void* eul_forcing, int reset, void* stream_) {
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "ib spread: dim must be 2 or 3");
    SG_REQUIRE(nearest && weights && forcing && eul_forcing && n_lag >= 1, SG_ERR_INVALID_ARG,
               "ib spread: bad argument");
    if (dim == 2) nz = 1;
    auto stream = (cudaStream_t)stream_;
    const int cells = dim == 2 ? 16 : 64;
    const int64_t ncell = (int64_t)nz * ny * nx;
    const unsigned blocks = ceil_div((int64_t)n_lag * cells, 256);
    if (dtype == SG_F32) {
        if (reset) {
            zero_kernel<float><<<ceil_div(dim * ncell, 256), 256, 0, stream>>>(dim * ncell, (float*)eul_forcing);
        }
        SpreadParams<float> p{dim, nz, ny, nx, n_lag, 0, nearest, (const float*)weights, (const float*)forcing,
                              (float*)eul_forcing};
        ib_spread_kernel<float><<<blocks, 256, 0, stream>>>(p);
    } else {
        SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "ib spread: bad dtype");
        if (reset) {
            zero_kernel<double><<<ceil_div(dim * ncell, 256), 256, 0, stream>>>(dim * ncell, (double*)eul_forcing);
        }
        SpreadParams<double> p{dim, nz, ny, nx, n_lag, 0, nearest, (const double*)weights, (const double*)forcing,
                               (double*)eul_forcing};
        ib_spread_kernel<double><<<blocks, 256, 0, stream>>>(p);
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
