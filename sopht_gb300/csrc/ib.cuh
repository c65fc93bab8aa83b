// Immersed-boundary device code shared by the single-instance entry points
// (ib.cu) and the batched 2D step (batch2d.cu).
#pragma once

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

// marker i is handled by one whole warp (lane = threadIdx.x & 31)
template <typename T>
__device__ __forceinline__ void ib_interaction_body(const IBParams<T>& p, int i) {
    const int lane = threadIdx.x & 31;
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

template <typename T>
__global__ void __launch_bounds__(256) ib_interaction_kernel(IBParams<T> p) {
    ib_interaction_body<T>(p, (blockIdx.x * blockDim.x + threadIdx.x) >> 5);
}

template <typename T> struct SpreadParams {
    int dim, nz, ny, nx, n_lag, reset;
    const int32_t* nearest;
    const T* weights;
    const T* forcing;
    T* eul;
};

// thread t owns (marker t / 4^dim, window cell t % 4^dim)
template <typename T>
__device__ __forceinline__ void ib_spread_body(const SpreadParams<T>& p, int64_t t) {
    const int cells = p.dim == 2 ? 16 : 64;
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
__global__ void __launch_bounds__(256) ib_spread_kernel(SpreadParams<T> p) {
    ib_spread_body<T>(p, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
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
