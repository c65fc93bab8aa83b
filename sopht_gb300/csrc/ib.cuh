// Immersed-boundary device code shared by the single-instance entry points
// (ib.cu) and the batched 2D step (batch2d.cu).
#pragma once

#include <cmath>

#include "common.cuh"
#include "flow_kernels.cuh"

namespace sg {

// numpy's floor_divide of doubles (b > 0): the exact floor of the real quotient a / b.  numpy
// forms it from fmod (an exact remainder) and a rounding correction; here the rounded quotient's
// floor is corrected by the signs of two exactly rounded remainders a - q b (fused multiply-adds
// keep the sign of the exact value), which needs no fmod loop -- the double-precision pipe of
// this GPU is narrow, and the IB kernels evaluate this once per marker axis.
__device__ __forceinline__ double np_floor_divide(double a, double b) {
    double q = floor(a / b);
    if (fma(-q, b, a) < 0.0) q -= 1.0;
    else if (fma(-(q + 1.0), b, a) >= 0.0) q += 1.0;
    return q;
}

// The same floor from a * (1 / b): the product is within two units in the last place of a / b, so
// its floor is off by at most one, and the two corrections give the exact floor again (the same
// integer as np_floor_divide) with a multiplication in place of the division.
__device__ __forceinline__ double np_floor_divide_recip(double a, double b, double inv_b) {
    double q = floor(a * inv_b);
    if (fma(-q, b, a) < 0.0) q -= 1.0;
    else if (fma(-(q + 1.0), b, a) >= 0.0) q += 1.0;
    return q;
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

// Per-call scalars of a bound interactor read from device memory, so that one captured graph
// serves every call (written by a one-thread kernel before each replay).
struct IBDynArgs {
    double K, C;
    int xi_step;
    double xi_dt;
};

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
    const IBDynArgs* dyn;  // when not null, K, C, xi_step and xi_dt come from here
};

// Marker i is handled by one whole warp.  Lane 4 d + k (d < DIM, k < 4)
// evaluates axis d's nearest index and the 1D weight of offset k - 1; the other
// lanes read them by shuffles, so each value is computed once per marker.  DIM
// is a template parameter so every per-axis array stays in registers.
template <typename T, int DIM>
__device__ __forceinline__ void ib_interaction_body(const IBParams<T>& p, int i) {
    constexpr int CELLS = DIM == 2 ? 16 : 64;
    const int lane = threadIdx.x & 31;
    if (i >= p.n_lag) return;
    const int n = p.n_lag;
    const T dxT = (T)p.dx;
    int my_near = 0;
    T my_phi = T(0);
    if (lane < 4 * DIM) {
        const int d = lane >> 2, k = lane & 3;
        const double X = p.pos[d * n + i];
        my_near = (int)np_floor_divide(X - p.shift, p.dx);
        // support: stored in the field precision, then scaled by 1/dx in it
        const T r = (T)((double)(my_near + k - 1) * p.dx + p.shift - X);
        const T rn = r / dxT;
        if (p.kernel == 0) my_phi = T(1) + dev_cos<T>((T)(0.5 * 3.14159265358979323846) * rn);
        else my_phi = peskin_phi<T>(fabs(rn));
    }
    int near[DIM];
    bool inside = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        near[d] = __shfl_sync(0xffffffffu, my_near, 4 * d);
        const int ext = d == 0 ? p.nx : (d == 1 ? p.ny : p.nz);
        if (near[d] - 1 < 0 || near[d] + 2 > ext - 1) inside = false;
    }
    if ((lane & 3) == 0 && (lane >> 2) < DIM) p.nearest[(lane >> 2) * n + i] = my_near;
    // optional VirtualBoundaryForcing.time_step: xi += dt * dU (previous dU)
    const int xi_step = p.dyn ? p.dyn->xi_step : p.xi_step;
    if (xi_step && lane < DIM) {
        const T dt = (T)(p.dev ? p.dev->dt : (p.dyn ? p.dyn->xi_dt : p.xi_dt));
        p.pos_mismatch[lane * n + i] = p.pos_mismatch[lane * n + i] + dt * p.vel_mismatch[lane * n + i];
    }
    if (!inside) {
        if (lane == 0) atomicExch(p.status, SG_ERR_OUT_OF_DOMAIN);
        for (int c = lane; c < CELLS; c += 32) p.weights[c * n + i] = T(0);
        return;
    }
    T pref;
    if (p.kernel == 0) {
        const T q = T(0.25) / dxT;
        pref = DIM == 2 ? q * q : (T)((double)q * (double)q * (double)q);
    } else {
        const T q = T(0.125) / dxT;
        pref = DIM == 2 ? q * q : (T)((double)q * (double)q * (double)q);
    }
    const int64_t plane = (int64_t)p.ny * p.nx;
    const int64_t ncell = plane * (DIM == 3 ? p.nz : 1);
    T acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = T(0);
#pragma unroll
    for (int c0 = 0; c0 < CELLS; c0 += 32) {
        const int c = c0 + lane;
        const int bx = c & 3, by = (c >> 2) & 3, bz = (c >> 4) & 3;
        const T px = __shfl_sync(0xffffffffu, my_phi, bx);
        const T py = __shfl_sync(0xffffffffu, my_phi, 4 + by);
        T pz = T(0);
        if constexpr (DIM == 3) pz = __shfl_sync(0xffffffffu, my_phi, 8 + bz);
        if (c < CELLS) {
            T w = pref * px * py;
            int gz = 0;
            if constexpr (DIM == 3) {
                w = w * pz;
                gz = near[2] - 1 + bz;
            }
            p.weights[c * n + i] = w;
            const int gx = near[0] - 1 + bx, gy = near[1] - 1 + by;
            const int64_t g = (int64_t)gz * plane + (int64_t)gy * p.nx + gx;
#pragma unroll
            for (int d = 0; d < DIM; ++d) acc[d] += p.u[d * ncell + g] * w;
        }
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        for (int o = 16; o > 0; o >>= 1) acc[d] += __shfl_xor_sync(0xffffffffu, acc[d], o);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        if (lane != d) continue;
        const T dxd = DIM == 2 ? dxT * dxT : dxT * dxT * dxT;
        const T U = acc[d] * dxd;
        p.flow_vel[d * n + i] = U;
        const T dU = (T)((double)U - p.body_vel[d * n + i]);
        p.vel_mismatch[d * n + i] = dU;
        const double K = p.dyn ? p.dyn->K : p.K, C = p.dyn ? p.dyn->C : p.C;
        p.forcing[d * n + i] = (T)(K * (double)p.pos_mismatch[d * n + i] + C * (double)dU);
    }
}

// The same interaction with one thread per marker, for kernels that hold only a few warps (the
// coupled rod sub-steps: one block per rod).  The warp-per-marker form leaves 20 of 32 lanes idle in
// the double-precision nearest-index and feedback arithmetic, which on this GPU's narrow FP64 pipe
// costs as much as full warps (a warp's double-precision instruction holds its SM sub-partition's
// FP64 unit for about 64 cycles, however many lanes are active); here every lane works on its own
// marker and the 4^dim window is
// summed in cell order (the warp form sums it as a shuffle tree, so the two round differently).
//
// The form the rod sub-steps take: X and V are the marker's position and body velocity, xi its
// position mismatch, all in the caller's registers (the caller owns the marker for the whole launch
// and keeps xi += dt dU itself, so p.xi_step is not read); dU returns the velocity mismatch.  Only
// the forcing is stored every call: the reaction of the neighbouring nodes reads it.  The nearest
// indices, weights, interpolated velocity and velocity mismatch are stored when `keep` is set (the
// last sub-step: they are the interactor's state the reference leaves after its rod loop).  The
// flow velocity is read through the read-only path, 16 cells (48 loads) at a time.  inv_dx is
// 1 / p.dx, computed once by the caller.
template <typename T, int DIM>
__device__ __forceinline__ void ib_interaction_thread(const IBParams<T>& p, int i, const double* Xs,
                                                      const double* Vs, const T* xi, T* dU_out, bool keep,
                                                      double inv_dx) {
    constexpr int CELLS = DIM == 2 ? 16 : 64;
    if (i >= p.n_lag) return;
    const int n = p.n_lag;
    const T dxT = (T)p.dx;
    int near[DIM];
    T phi[DIM][4];
    bool inside = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const double X = Xs[d];
        near[d] = (int)np_floor_divide_recip(X - p.shift, p.dx, inv_dx);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const T r = (T)((double)(near[d] + k - 1) * p.dx + p.shift - X);
            const T rn = r / dxT;
            phi[d][k] = p.kernel == 0 ? T(1) + dev_cos<T>((T)(0.5 * 3.14159265358979323846) * rn)
                                      : peskin_phi<T>(fabs(rn));
        }
        const int ext = d == 0 ? p.nx : (d == 1 ? p.ny : p.nz);
        if (near[d] - 1 < 0 || near[d] + 2 > ext - 1) inside = false;
        if (keep) p.nearest[d * n + i] = near[d];
    }
    if (!inside) {
        atomicExch(p.status, SG_ERR_OUT_OF_DOMAIN);
        for (int c = 0; c < CELLS; ++c) p.weights[c * n + i] = T(0);
        for (int d = 0; d < DIM; ++d) dU_out[d] = T(0);
        return;
    }
    T pref;
    if (p.kernel == 0) {
        const T q = T(0.25) / dxT;
        pref = DIM == 2 ? q * q : (T)((double)q * (double)q * (double)q);
    } else {
        const T q = T(0.125) / dxT;
        pref = DIM == 2 ? q * q : (T)((double)q * (double)q * (double)q);
    }
    const int64_t plane = (int64_t)p.ny * p.nx;
    const int64_t ncell = plane * (DIM == 3 ? p.nz : 1);
    // the window's first cell, per component
    const int64_t g0 = (DIM == 3 ? (int64_t)(near[DIM - 1] - 1) * plane : 0) + (int64_t)(near[1] - 1) * p.nx +
                       (near[0] - 1);
    const T* ud[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) ud[d] = p.u + d * ncell + g0;
    T acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = T(0);
#pragma unroll 16
    for (int c = 0; c < CELLS; ++c) {
        const int bx = c & 3, by = (c >> 2) & 3, bz = (c >> 4) & 3;
        T w = pref * phi[0][bx] * phi[1][by];
        int64_t off = (int64_t)by * p.nx + bx;
        if constexpr (DIM == 3) {
            w = w * phi[2][bz];
            off += bz * plane;
        }
        if (keep) p.weights[c * n + i] = w;
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] += __ldg(ud[d] + off) * w;
    }
    const T dxd = DIM == 2 ? dxT * dxT : dxT * dxT * dxT;
    const double K = p.dyn ? p.dyn->K : p.K, C = p.dyn ? p.dyn->C : p.C;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const T U = acc[d] * dxd;
        const T dU = (T)((double)U - Vs[d]);
        dU_out[d] = dU;
        if (keep) {
            p.flow_vel[d * n + i] = U;
            p.vel_mismatch[d * n + i] = dU;
        }
        p.forcing[d * n + i] = (T)(K * (double)xi[d] + C * (double)dU);
    }
}

template <typename T, int DIM>
__global__ void __launch_bounds__(256) ib_interaction_kernel(IBParams<T> p) {
    ib_interaction_body<T, DIM>(p, (blockIdx.x * blockDim.x + threadIdx.x) >> 5);
}

template <typename T> struct SpreadParams {
    int dim, nz, ny, nx, n_lag, reset;
    const int32_t* nearest;
    const T* weights;
    const T* forcing;
    T* eul;
};

// Cell c of marker i's window: the thread whose marker is the lowest-index
// marker touching the cell owns it and sums every marker's F * phi into it in
// marker index order (the per-cell order of the reference's serial loop), so
// no atomics are needed and the result is bitwise repeatable.  near(d, j) gives
// marker j's nearest index along axis d.
template <typename T, int DIM, typename NearF>
__device__ __forceinline__ void ib_spread_at(const SpreadParams<T>& p, int i, int c, NearF near) {
    const int n = p.n_lag;
    int cell[DIM];
    cell[0] = near(0, i) - 1 + (c & 3);
    cell[1] = near(1, i) - 1 + ((c >> 2) & 3);
    if constexpr (DIM == 3) cell[2] = near(2, i) - 1 + (c >> 4);
    // a marker whose window leaves the grid was reported out of domain
    if (cell[0] < 0 || cell[0] >= p.nx || cell[1] < 0 || cell[1] >= p.ny) return;
    if constexpr (DIM == 3)
        if (cell[2] < 0 || cell[2] >= p.nz) return;
    auto offset_in = [&](int j, int& k) -> bool {
        const int o0 = cell[0] - (near(0, j) - 1);
        if (o0 < 0 || o0 > 3) return false;
        const int o1 = cell[1] - (near(1, j) - 1);
        if (o1 < 0 || o1 > 3) return false;
        int o2 = 0;
        if constexpr (DIM == 3) {
            o2 = cell[2] - (near(2, j) - 1);
            if (o2 < 0 || o2 > 3) return false;
        }
        k = o0 + 4 * o1 + 16 * o2;
        return true;
    };
    int k;
    for (int j = 0; j < i; ++j)
        if (offset_in(j, k)) return;  // a lower-index marker owns this cell
    const int64_t plane = (int64_t)p.ny * p.nx;
    const int64_t ncell = plane * (DIM == 3 ? p.nz : 1);
    const int64_t g = (int64_t)(DIM == 3 ? cell[DIM - 1] : 0) * plane + (int64_t)cell[1] * p.nx + cell[0];
    T acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = p.reset ? T(0) : p.eul[d * ncell + g];
    for (int j = i; j < n; ++j) {
        if (!offset_in(j, k)) continue;
        const T w = p.weights[k * n + j];
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] = acc[d] + p.forcing[d * n + j] * w;
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d) p.eul[d * ncell + g] = acc[d];
}

// thread t owns (marker t / 4^DIM, window cell t % 4^DIM); nearest read from global memory
template <typename T, int DIM>
__device__ __forceinline__ void ib_spread_body(const SpreadParams<T>& p, int64_t t) {
    constexpr int CELLS = DIM == 2 ? 16 : 64;
    if (t >= (int64_t)p.n_lag * CELLS) return;
    const int n = p.n_lag;
    ib_spread_at<T, DIM>(p, (int)(t / CELLS), (int)(t % CELLS),
                         [&](int d, int j) { return (int)p.nearest[d * n + j]; });
}

template <typename T, int DIM>
__global__ void __launch_bounds__(256) ib_spread_kernel(SpreadParams<T> p) {
    ib_spread_body<T, DIM>(p, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// The same spreading with one warp per (marker i, window cell c), the markers'
// nearest indices read from `s_near` (shared memory, DIM * n_lag ints).  The
// lanes scan 32 markers at a time: a ballot tells whether a lower-index marker
// touches the cell (then another warp owns it), and lane 0 adds the touching
// markers' F * phi in ascending marker order -- the order of ib_spread_at, so
// the sums are the same to the bit.  Every lane of the warp must call it.
template <typename T, int DIM>
__device__ __forceinline__ void ib_spread_warp_pair(const SpreadParams<T>& p, const int* s_near, int i, int c,
                                                    int lane) {
    const int n = p.n_lag;
    int cell[DIM];
    cell[0] = s_near[i] - 1 + (c & 3);
    cell[1] = s_near[n + i] - 1 + ((c >> 2) & 3);
    if constexpr (DIM == 3) cell[2] = s_near[2 * n + i] - 1 + (c >> 4);
    if (cell[0] < 0 || cell[0] >= p.nx || cell[1] < 0 || cell[1] >= p.ny) return;
    if constexpr (DIM == 3)
        if (cell[2] < 0 || cell[2] >= p.nz) return;
    auto offset_in = [&](int j, int& k) -> bool {
        const int o0 = cell[0] - (s_near[j] - 1);
        if (o0 < 0 || o0 > 3) return false;
        const int o1 = cell[1] - (s_near[n + j] - 1);
        if (o1 < 0 || o1 > 3) return false;
        int o2 = 0;
        if constexpr (DIM == 3) {
            o2 = cell[2] - (s_near[2 * n + j] - 1);
            if (o2 < 0 || o2 > 3) return false;
        }
        k = o0 + 4 * o1 + 16 * o2;
        return true;
    };
    for (int j0 = 0; j0 < i; j0 += 32) {
        const int j = j0 + lane;
        int k;
        const bool hit = j < i && offset_in(j, k);
        if (__any_sync(0xffffffffu, hit)) return;  // a lower-index marker owns this cell
    }
    const int64_t plane = (int64_t)p.ny * p.nx;
    const int64_t ncell = plane * (DIM == 3 ? p.nz : 1);
    const int64_t g = (int64_t)(DIM == 3 ? cell[DIM - 1] : 0) * plane + (int64_t)cell[1] * p.nx + cell[0];
    T acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = p.reset ? T(0) : p.eul[d * ncell + g];
    for (int j0 = i; j0 < n; j0 += 32) {
        const int j = j0 + lane;
        int k = 0;
        const bool hit = j < n && offset_in(j, k);
        unsigned mask = __ballot_sync(0xffffffffu, hit);
        while (mask) {
            const int b = __ffs(mask) - 1;
            mask &= mask - 1;
            const int kb = __shfl_sync(0xffffffffu, k, b);
            if (lane == 0) {
                const int jb = j0 + b;
                const T w = p.weights[kb * n + jb];
#pragma unroll
                for (int d = 0; d < DIM; ++d) acc[d] = acc[d] + p.forcing[d * n + jb] * w;
            }
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) p.eul[d * ncell + g] = acc[d];
    }
}

template <typename T, int DIM>
__global__ void __launch_bounds__(256) ib_spread_warp_kernel(SpreadParams<T> p) {
    extern __shared__ int s_near[];
    constexpr int CELLS = DIM == 2 ? 16 : 64;
    const int n = p.n_lag;
    for (int e = threadIdx.x; e < DIM * n; e += blockDim.x) s_near[e] = p.nearest[e];
    __syncthreads();
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wid >= (int64_t)n * CELLS) return;  // uniform over the warp
    ib_spread_warp_pair<T, DIM>(p, s_near, (int)(wid / CELLS), (int)(wid % CELLS), threadIdx.x & 31);
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
