// Stencil kernels of the unbounded vorticity Navier-Stokes step.
//
// Boundary conventions follow the reference's pystencils kernels, which
// iterate the interior with as many ghost layers as the largest stencil offset
// on every axis:
//   forcing curl update   [1:-1]   ring unchanged  (update_vorticity_from_velocity_forcing_{2,3}d.py)
//   ENO3 advection flux   [2:-2]   zero elsewhere  (advection_flux_2d.py)
//   diffusion flux        [1:-1]   zero ring       (diffusion_flux_{2,3}d.py)
//   curl                  [1:-1]   zero ring       (outplane_field_curl_2d.py, curl_3d.py)
#pragma once

#include "common.cuh"
#include "fft_fast.cuh"

namespace sg {

// Step scalars: from the device struct when given, else the by-value copy.
struct ScalarSrc {
    sg_step_scalars host;
    const sg_step_scalars* dev;
    __device__ __forceinline__ double dt() const { return dev ? dev->dt : host.dt; }
    __device__ __forceinline__ double forcing() const { return dev ? dev->forcing_prefac : host.forcing_prefac; }
    __device__ __forceinline__ double advection() const { return dev ? dev->advection_prefac : host.advection_prefac; }
    __device__ __forceinline__ double diffusion() const { return dev ? dev->diffusion_prefac : host.diffusion_prefac; }
    __device__ __forceinline__ double free_stream(int c) const { return dev ? dev->free_stream[c] : host.free_stream[c]; }
};

// ---------------------------------------------------------------- 2D sweep
// One fused pass: w1 = w + pf curl(f) ; w2 = w1 + ENO3 flux(w1, u) ;
// w3 = w2 + k lap(w2).  Output w3 goes to a separate buffer (the caller's
// vorticity is rewritten by the Poisson load pass) because neighbouring tiles
// still read the input halo.
enum { SWEEP_ADVECT = 1, SWEEP_DIFFUSE = 2 };

template <typename T> struct Sweep2DParams {
    int ny, nx;
    const T* w;
    const T* u;   // (2, ny, nx), may be null without SWEEP_ADVECT
    const T* f;   // (2, ny, nx) or null
    T* out;
    ScalarSrc sc;
    int flags;    // SWEEP_ADVECT | SWEEP_DIFFUSE
    T* tape_w1;   // optional: w1 (after the forcing curl) on the tile, for the adjoint
    T* tape_w2;   // optional: w2 (after advection)
};

// advection_flux_2d.py:35-47: left-biased when u_0 > -u_{+1}.  The two fused multiply-adds are
// written out, so every kernel that uses the face (and every launch shape of one kernel) rounds it
// the same way whatever the compiler's contraction choices around the call.
template <typename T>
__device__ __forceinline__ T eno3_face(T qm1, T q0, T qp1, T qp2, T u0, T up1) {
    const T third = T(1.0 / 3.0), five6 = T(5.0 / 6.0), sixth = T(1.0 / 6.0);
    if (u0 > -up1) return fma(-sixth, qm1, fma(five6, q0, third * qp1));
    return fma(-sixth, qp2, fma(five6, qp1, third * q0));
}

template <typename T, int TX, int TY>
__device__ __forceinline__ void sweep2d_body(const Sweep2DParams<T>& p, int bx, int by) {
    constexpr int HW = 3, HF = 4;
    constexpr int WX = TX + 2 * HW, WY = TY + 2 * HW;
    constexpr int FX = TX + 2 * HF, FY = TY + 2 * HF;
    constexpr int W2X = TX + 2, W2Y = TY + 2;
    __shared__ T s_fx[FY * FX];
    __shared__ T s_fy[FY * FX];
    __shared__ T s_w[WY * WX];
    __shared__ T s_ux[WY * WX];
    __shared__ T s_uy[WY * WX];
    __shared__ T s_w1[WY * WX];
    __shared__ T s_w2[W2Y * W2X];
    const int nthr = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int x0 = bx * TX, y0 = by * TY;
    const int ny = p.ny, nx = p.nx;
    const int64_t plane = (int64_t)ny * nx;
    const bool forcing = p.f != nullptr;
    // load
    for (int e = tid; e < WY * WX; e += nthr) {
        const int gy = y0 - HW + e / WX, gx = x0 - HW + e % WX;
        T w = T(0), ux = T(0), uy = T(0);
        if (gy >= 0 && gy < ny && gx >= 0 && gx < nx) {
            const int64_t g = (int64_t)gy * nx + gx;
            w = p.w[g];
            if (p.u) {
                ux = p.u[g];
                uy = p.u[plane + g];
            }
        }
        s_w[e] = w;
        s_ux[e] = ux;
        s_uy[e] = uy;
    }
    if (forcing) {
        for (int e = tid; e < FY * FX; e += nthr) {
            const int gy = y0 - HF + e / FX, gx = x0 - HF + e % FX;
            T fx = T(0), fy = T(0);
            if (gy >= 0 && gy < ny && gx >= 0 && gx < nx) {
                const int64_t g = (int64_t)gy * nx + gx;
                fx = p.f[g];
                fy = p.f[plane + g];
            }
            s_fx[e] = fx;
            s_fy[e] = fy;
        }
    }
    __syncthreads();
    // w1 on the halo-3 region
    const T pf = (T)p.sc.forcing();
    for (int e = tid; e < WY * WX; e += nthr) {
        const int ly = e / WX, lx = e % WX;
        const int gy = y0 - HW + ly, gx = x0 - HW + lx;
        T w1 = s_w[e];
        if (forcing && gy >= 1 && gy <= ny - 2 && gx >= 1 && gx <= nx - 2) {
            const int fe = (ly + 1) * FX + (lx + 1);
            const T curl = s_fy[fe + 1] - s_fy[fe - 1] - s_fx[fe + FX] + s_fx[fe - FX];
            w1 = w1 + curl * pf;
        }
        s_w1[e] = w1;
    }
    __syncthreads();
    // w2 = w1 + ENO3 flux on the halo-1 region
    const T inv_dx = -(T)p.sc.advection();
    for (int e = tid; e < W2Y * W2X; e += nthr) {
        const int ly = e / W2X + 2, lx = e % W2X + 2;  // coordinates in the halo-3 frame
        const int gy = y0 - HW + ly, gx = x0 - HW + lx;
        const int c = ly * WX + lx;
        T w2 = s_w1[c];
        if ((p.flags & SWEEP_ADVECT) && gy >= 2 && gy <= ny - 3 && gx >= 2 && gx <= nx - 3) {
            auto qx = [&](int d) { return s_w1[c + d] * s_ux[c + d]; };
            auto qy = [&](int d) { return s_w1[c + d * WX] * s_uy[c + d * WX]; };
            const T east = eno3_face(qx(-1), qx(0), qx(1), qx(2), s_ux[c], s_ux[c + 1]);
            const T west = eno3_face(qx(-2), qx(-1), qx(0), qx(1), s_ux[c - 1], s_ux[c]);
            const T north = eno3_face(qy(-1), qy(0), qy(1), qy(2), s_uy[c], s_uy[c + WX]);
            const T south = eno3_face(qy(-2), qy(-1), qy(0), qy(1), s_uy[c - WX], s_uy[c]);
            T flux = inv_dx * east;
            flux = flux - inv_dx * west;
            flux = flux + inv_dx * north;
            flux = flux - inv_dx * south;
            w2 = w2 + flux;
        }
        s_w2[e] = w2;
    }
    __syncthreads();
    // w3 = w2 + k lap(w2) on the tile
    const T k = (T)p.sc.diffusion();
    for (int e = tid; e < TY * TX; e += nthr) {
        const int ly = e / TX, lx = e % TX;
        const int gy = y0 + ly, gx = x0 + lx;
        if (gy >= ny || gx >= nx) continue;
        const int c = (ly + 1) * W2X + (lx + 1);
        T w3 = s_w2[c];
        if ((p.flags & SWEEP_DIFFUSE) && gy >= 1 && gy <= ny - 2 && gx >= 1 && gx <= nx - 2) {
            const T lap = s_w2[c + W2X] + s_w2[c - W2X] + s_w2[c + 1] + s_w2[c - 1] - T(4) * s_w2[c];
            w3 = w3 + k * lap;
        }
        p.out[(int64_t)gy * nx + gx] = w3;
        if (p.tape_w1) {
            p.tape_w1[(int64_t)gy * nx + gx] = s_w1[(ly + HW) * WX + (lx + HW)];
            p.tape_w2[(int64_t)gy * nx + gx] = s_w2[c];
        }
    }
}

template <typename T, int TX, int TY>
__global__ void __launch_bounds__(TX * 8) sweep2d_kernel(Sweep2DParams<T> p) {
    sweep2d_body<T, TX, TY>(p, blockIdx.x, blockIdx.y);
}

// --------------------------------------------- fused Poisson load (x rows R2C)
// Row q of component c (3D: q -> (c, z, y); 2D: q -> y).  Reads the swept
// vorticity `src`, applies the boundary penalisation by index clamping and the
// per-index sine factors (X pass, then Y, then Z, as penalise_field_boundary_
// {2,3}d.py orders them), writes the result back to the caller's vorticity,
// zeroes the forcing row, and emits the M+1 bins of the zero-padded row.
template <typename T> struct FlowLoadParams {
    int dim, nz, ny, nx;
    int width;               // penalty zone width (0: none)
    const T* src;            // swept vorticity, same layout as dst
    T* dst;                  // caller's vorticity (penalised copy)
    T* forcing;              // zeroed when not null
    int zero_ncomp;          // forcing rows zeroed per row: the row's component and the next ones
    const T* cx;             // penalisation factors per index (null if width 0)
    const T* cy;
    const T* cz;
    int64_t comp_stride;     // elements between components of src/dst/forcing
    cplx_t<T>* spec;
    RowMap spec_map;
    int n_rows;
    FFTStages st;
    const cplx_t<T>* tw_m;
    const cplx_t<T>* tw_l;
    int prefetch_ahead;      // register load pass: > 0 asks L2 for the rows of the block this far ahead
};

__device__ __forceinline__ int clamp_band(int i, int n, int w) {
    if (w <= 0) return i;
    return i < w - 1 ? w - 1 : (i > n - w ? n - w : i);
}

template <typename T>
__global__ void __launch_bounds__(256) flow_load_kernel(FlowLoadParams<T> p) {
    using C = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = p.st.n;
    const int rb = blockDim.y;
    C* buf0 = reinterpret_cast<C*>(smem_raw);
    C* buf1 = buf0 + rb * M;
    const int row0 = blockIdx.x * rb;
    const int nthr = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nx = p.nx;
    for (int e = tid; e < rb * M; e += nthr) {
        const int r = e / M, n = e % M;
        const int q = row0 + r;
        C z = cmake<C>(T(0), T(0));
        if (q < p.n_rows && 2 * n < nx) {
            int y = q % p.ny, c, zi;
            if (p.dim == 3) {
                zi = (q / p.ny) % p.nz;
                c = q / (p.ny * p.nz);
            } else {
                zi = 0;
                c = q / p.ny;
            }
            const int sy = clamp_band(y, p.ny, p.width);
            const int sz = p.dim == 3 ? clamp_band(zi, p.nz, p.width) : 0;
            const int64_t src_row = (int64_t)c * p.comp_stride + ((int64_t)sz * p.ny + sy) * nx;
            const int64_t dst_row = (int64_t)c * p.comp_stride + ((int64_t)zi * p.ny + y) * nx;
            T v[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int x = 2 * n + h;
                T val = T(0);
                if (x < nx) {
                    const int sx = clamp_band(x, nx, p.width);
                    val = p.src[src_row + sx];
                    if (p.width > 0) {
                        val = val * p.cx[x];
                        val = val * p.cy[y];
                        if (p.dim == 3) val = val * p.cz[zi];
                    }
                    p.dst[dst_row + x] = val;
                    if (p.forcing)
                        for (int zc = 0; zc < p.zero_ncomp; ++zc) p.forcing[dst_row + zc * p.comp_stride + x] = T(0);
                }
                v[h] = val;
            }
            z = cmake<C>(v[0], v[1]);
        }
        buf0[r * M + n] = z;
    }
    __syncthreads();
    C* Z = fft_smem<false, false>(buf0, buf1, p.st, rb, 1, M, p.tw_m);
    for (int e = tid; e < rb * (M + 1); e += nthr) {
        const int r = e / (M + 1), k = e % (M + 1);
        const int q = row0 + r;
        if (q >= p.n_rows) continue;
        const C zk = Z[r * M + (k == M ? 0 : k)];
        const C zc = cconj(Z[r * M + (k == 0 ? 0 : M - k)]);
        const C w = p.tw_l[k];
        const C s = cadd(zk, zc);
        const C wd = cmul(w, csub(zk, zc));
        p.spec[p.spec_map.offset(q) + k] = cmake<C>(T(0.5) * (s.x + wd.y), T(0.5) * (s.y - wd.x));
    }
}

// Size-specialised variant of flow_load_kernel (M = nx in the fast set).  Per
// block, the W rows' source/destination offsets and y/z boundary factors are
// computed once into shared memory; each element then costs a clamp on x only.
template <int M, int W> struct FlowLoadSmem {
    template <typename T> static constexpr size_t bytes() {
        using C = cplx_t<T>;
        return sizeof(C) * ((size_t)M * (W + 1) + M + (M + 1)) + sizeof(int64_t) * 3 * W + sizeof(T) * 2 * W + 32;
    }
};

// The row's packed complex points M/2 .. M-1 are the zero padding (2n >= nx),
// so they are not loaded and the first stage skips them.
template <typename T, int M, int W, int E = FastElems<M>::E>
__device__ __forceinline__ void fast_flow_load_body(const FlowLoadParams<T>& p, int bid, unsigned char* smem_raw,
                                                    bool stage_tw = true) {
    using C = cplx_t<T>;
    using S = FastShape<M, W, E>;
    constexpr int LS = S::LS, NT = S::NT, PER = M * W / NT;
    constexpr bool SKIP_LOAD = FastEnds<M>::first_even;
    C* buf = reinterpret_cast<C*>(smem_raw);
    C* tw_m = buf + M * LS;
    C* tw_l = tw_m + M;
    int64_t* src_off = reinterpret_cast<int64_t*>(
        (reinterpret_cast<uintptr_t>(tw_l + M + 1) + 15) & ~uintptr_t(15));
    int64_t* dst_off = src_off + W;
    int64_t* spec_off = dst_off + W;
    T* fy = reinterpret_cast<T*>(spec_off + W);
    T* fz = fy + W;
    const int tid = threadIdx.x;
    const int row0 = bid * W;
    const int nx = p.nx;  // == M
    if (tid < W) {
        const int q = row0 + tid;
        const int y = q % p.ny;
        int c, zi;
        if (p.dim == 3) {
            zi = (q / p.ny) % p.nz;
            c = q / (p.ny * p.nz);
        } else {
            zi = 0;
            c = q / p.ny;
        }
        const int sy = clamp_band(y, p.ny, p.width);
        const int sz = p.dim == 3 ? clamp_band(zi, p.nz, p.width) : 0;
        src_off[tid] = (int64_t)c * p.comp_stride + ((int64_t)sz * p.ny + sy) * nx;
        dst_off[tid] = (int64_t)c * p.comp_stride + ((int64_t)zi * p.ny + y) * nx;
        spec_off[tid] = p.spec_map.offset(q);
        fy[tid] = p.width > 0 ? p.cy[y] : T(1);
        fz[tid] = (p.width > 0 && p.dim == 3) ? p.cz[zi] : T(1);
    }
    if (stage_tw) {
        stage_table(tw_m, p.tw_m, M, tid, NT);
        stage_table(tw_l, p.tw_l, M + 1, tid, NT);
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int e = tid + b * NT;
        const int r = e / M, n = e % M;
        if (SKIP_LOAD && n >= M / 2) continue;
        C z = cmake<C>(T(0), T(0));
        if (row0 + r < p.n_rows && 2 * n < nx) {
            const int x0 = 2 * n;
            const int s0 = clamp_band(x0, nx, p.width), s1 = clamp_band(x0 + 1, nx, p.width);
            const T* src = p.src + src_off[r];
            if (s0 == x0 && s1 == x0 + 1) {
                z = *reinterpret_cast<const C*>(src + x0);
            } else {
                z.x = src[s0];
                z.y = src[s1];
            }
            if (p.width > 0) {
                // penalise_field_boundary_{2,3}d.py order: X factor, then Y, then Z
                z.x = z.x * p.cx[x0];
                z.y = z.y * p.cx[x0 + 1];
                z.x = z.x * fy[r];
                z.y = z.y * fy[r];
                if (p.dim == 3) {
                    z.x = z.x * fz[r];
                    z.y = z.y * fz[r];
                }
            }
            const int64_t d = dst_off[r] + x0;
            *reinterpret_cast<C*>(p.dst + d) = z;
            if (p.forcing)
                for (int zc = 0; zc < p.zero_ncomp; ++zc)
                    *reinterpret_cast<C*>(p.forcing + d + zc * p.comp_stride) = cmake<C>(T(0), T(0));
        }
        buf[n * LS + r] = z;
    }
    __syncthreads();
    fast_fft<M, W, false, E, true, false>(buf, tw_m, tid);
    r2c_post_store<T, M, W, E>(buf, tw_l, p.spec, spec_off, row0, p.n_rows, tid);
}

template <typename T, int M, int W, int E>
__global__ void __launch_bounds__(FastShape<M, W, E>::NT) fast_flow_load_kernel(FlowLoadParams<T> p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    fast_flow_load_body<T, M, W, E>(p, blockIdx.x, smem_raw);
}

// ---------------------------------------- curl + free stream + max |u| (2D)
// Non-negative values order like their bit patterns, so an integer atomicMax on the bits is the float max.
template <typename T>
__device__ __forceinline__ void atomic_max_nonneg(T* slot, T v);
template <>
__device__ __forceinline__ void atomic_max_nonneg<float>(float* slot, float v) {
    atomicMax(reinterpret_cast<int*>(slot), __float_as_int(v));
}
template <>
__device__ __forceinline__ void atomic_max_nonneg<double>(double* slot, double v) {
    atomicMax(reinterpret_cast<unsigned long long*>(slot), (unsigned long long)__double_as_longlong(v));
}

// The same for grids of many blocks: a value not above the slot's current content cannot change the
// max and skips the atomic, so after the first blocks most of the grid reads the slot instead of
// queueing on one address (3D curl: 65 536 blocks at 256^3).  Small grids (under one wave) keep the
// plain atomic: there the read only lengthens each block's tail.
template <typename T>
__device__ __forceinline__ void atomic_max_nonneg_filtered(T* slot, T v);
template <>
__device__ __forceinline__ void atomic_max_nonneg_filtered<float>(float* slot, float v) {
    const int bits = __float_as_int(v);
    if (bits > *reinterpret_cast<volatile int*>(slot)) atomicMax(reinterpret_cast<int*>(slot), bits);
}
template <>
__device__ __forceinline__ void atomic_max_nonneg_filtered<double>(double* slot, double v) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    if (bits > *reinterpret_cast<volatile unsigned long long*>(slot))
        atomicMax(reinterpret_cast<unsigned long long*>(slot), bits);
}

template <typename T>
__device__ __forceinline__ T block_max(T v) {
    __shared__ T warp_max[32];
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nw = (blockDim.x * blockDim.y + 31) / 32;
    if ((tid & 31) == 0) warp_max[tid >> 5] = v;
    __syncthreads();
    if (tid < 32) {
        v = tid < nw ? warp_max[tid] : T(0);
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;  // valid in thread 0
}

template <typename T> struct Curl2DParams {
    int ny, nx;
    const T* psi;
    T* u;
    T prefactor;
    ScalarSrc sc;
    int add_free_stream;
    T* umax;   // may be null
};

// one 32 x 8 tile of the 2D curl (block shape 32 x 8)
template <typename T>
__device__ __forceinline__ void curl2d_body(const Curl2DParams<T>& p, int bx, int by) {
    const int gx = bx * 32 + threadIdx.x;
    const int gy = by * 8 + threadIdx.y;
    const int ny = p.ny, nx = p.nx;
    T m = T(0);
    if (gx < nx && gy < ny) {
        const int64_t g = (int64_t)gy * nx + gx;
        T ux = T(0), uy = T(0);
        if (gy >= 1 && gy <= ny - 2 && gx >= 1 && gx <= nx - 2) {
            ux = (p.psi[g + nx] - p.psi[g - nx]) * p.prefactor;
            uy = (p.psi[g - 1] - p.psi[g + 1]) * p.prefactor;
        }
        if (p.add_free_stream) {
            ux = ux + (T)p.sc.free_stream(0);
            uy = uy + (T)p.sc.free_stream(1);
        }
        p.u[g] = ux;
        p.u[(int64_t)ny * nx + g] = uy;
        m = fabs(ux) + fabs(uy);
    }
    if (p.umax) {
        m = block_max(m);
        if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg(p.umax, m);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) curl2d_kernel(Curl2DParams<T> p) {
    curl2d_body<T>(p, blockIdx.x, blockIdx.y);
}

// ------------------------------------------------------------ 3D kernels
// Direct-load stencils; neighbour reuse is served by L1/L2.
struct Grid3 {
    int nz, ny, nx;
    __device__ __forceinline__ int64_t n() const { return (int64_t)nz * ny * nx; }
    __device__ __forceinline__ bool interior(int z, int y, int x) const {
        return z >= 1 && z <= nz - 2 && y >= 1 && y <= ny - 2 && x >= 1 && x <= nx - 2;
    }
};

// Launch shape of the cell-wise 3D kernels: 32 x 8 threads over (x, y) of one z-plane per block, so a
// thread's cell comes from its block and thread coordinates (no 64-bit division per thread).
constexpr int kCell3X = 32, kCell3Y = 8;
inline dim3 cell3_grid(const Grid3& G) {
    return dim3((unsigned)((G.nx + kCell3X - 1) / kCell3X), (unsigned)((G.ny + kCell3Y - 1) / kCell3Y),
                (unsigned)G.nz);
}
inline dim3 cell3_block() { return dim3(kCell3X, kCell3Y); }
__device__ __forceinline__ bool cell3(const Grid3& G, int& x, int& y, int& z, int64_t& g) {
    x = blockIdx.x * kCell3X + threadIdx.x;
    y = blockIdx.y * kCell3Y + threadIdx.y;
    z = blockIdx.z;
    g = ((int64_t)z * G.ny + y) * G.nx + x;
    return x < G.nx && y < G.ny;
}

// Step scalars in the field precision for every thread of a block, converted once: thread 0
// converts and the block reads them from shared memory.  A double-to-float conversion runs on this
// GPU's narrow double-precision pipe, and one per thread kept that pipe busy a fifth (one scalar)
// to two thirds (three) of the time in the 3D cell kernels; converting once made the forcing curl,
// rotational update and diffusion 1.8 % faster together (0.445 -> 0.437 ms at 256^3).  Every thread of the block calls it at
// the same point, before any early return (it holds a barrier); get(i) is called by thread 0 only.
// The kernels call it after issuing their loads, so that the barrier waits with the loads in
// flight.  The values are the same roundings as a conversion in each thread.
template <typename T, int N, typename F>
__device__ __forceinline__ void block_scalars(F get, T (&out)[N]) {
    if constexpr (sizeof(T) == sizeof(double)) {
#pragma unroll
        for (int i = 0; i < N; ++i) out[i] = (T)get(i);
    } else {
        __shared__ T s[N];
        if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0)
            for (int i = 0; i < N; ++i) s[i] = (T)get(i);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < N; ++i) out[i] = s[i];
    }
}

// out = w + pf * curl_h(v) on [1:-1]^3 (w elsewhere)  — per component as
// update_vorticity_from_velocity_forcing_3d.py:29-94 writes it.
template <typename T>
__device__ __forceinline__ void curl3_at(const T* v, int64_t g, int64_t n, int64_t sy, int64_t sz, T out[3]) {
    const T* vx = v;
    const T* vy = v + n;
    const T* vz = v + 2 * n;
    out[0] = vz[g + sy] - vz[g - sy] - vy[g + sz] + vy[g - sz];
    out[1] = vx[g + sz] - vx[g - sz] - vz[g + 1] + vz[g - 1];
    out[2] = vy[g + 1] - vy[g - 1] - vx[g + sy] + vx[g - sy];
}

template <typename T> struct Stencil3DParams {
    Grid3 grid;
    const T* a;      // primary input (vector)
    const T* b;      // secondary input (vector) or null
    T* out;          // output (vector)
    ScalarSrc sc;
    T prefactor;
    int mode;
    int ncomp;       // components of the diffusion, 1 to 3 (0 means 3)
};

// w1 = w + pf curl(f)  (mode 0; f may be null -> copy)
template <typename T>
__global__ void __launch_bounds__(256) forcing_curl3d_kernel(Stencil3DParams<T> p) {
    const Grid3 G = p.grid;
    const int64_t n = G.n();
    int x, y, z;
    int64_t g;
    const bool live = cell3(G, x, y, z, g);
    const bool in = live && p.b && G.interior(z, y, x);
    const int64_t sy = G.nx, sz = (int64_t)G.nx * G.ny;
    T w0 = T(0), w1 = T(0), w2 = T(0), c[3] = {T(0), T(0), T(0)};
    if (live) {
        w0 = p.a[g];
        w1 = p.a[n + g];
        w2 = p.a[2 * n + g];
    }
    if (in) curl3_at(p.b, g, n, sy, sz, c);
    T pfs[1];
    block_scalars<T, 1>([&](int) { return p.mode == 0 ? p.sc.forcing() : (double)p.prefactor; }, pfs);
    if (!live) return;
    if (in) {
        const T pf = pfs[0];
        w0 = w0 + pf * c[0];
        w1 = w1 + pf * c[1];
        w2 = w2 + pf * c[2];
    }
    p.out[g] = w0;
    p.out[n + g] = w1;
    p.out[2 * n + g] = w2;
}

// w2 = w1 + pc curl(u x w1) on [1:-1]^3 (a = w1, b = u)
template <typename T>
__device__ __forceinline__ void cross_at(const T* u, const T* w, int64_t g, int64_t n, T c[3]) {
    const T ux = u[g], uy = u[n + g], uz = u[2 * n + g];
    const T wx = w[g], wy = w[n + g], wz = w[2 * n + g];
    // elementwise_ops_3d.py:406-448: r_i = a_j b_k - b_j a_k
    c[0] = uy * wz - wy * uz;
    c[1] = uz * wx - wz * ux;
    c[2] = ux * wy - wx * uy;
}

template <typename T>
__global__ void __launch_bounds__(256) rotational_update3d_kernel(Stencil3DParams<T> p) {
    const Grid3 G = p.grid;
    const int64_t n = G.n();
    int x, y, z;
    int64_t g;
    const bool live = cell3(G, x, y, z, g);
    const bool in = live && G.interior(z, y, x);
    const int64_t sy = G.nx, sz = (int64_t)G.nx * G.ny;
    T w0 = T(0), w1 = T(0), w2 = T(0), r0 = T(0), r1 = T(0), r2 = T(0);
    if (live) {
        w0 = p.a[g];
        w1 = p.a[n + g];
        w2 = p.a[2 * n + g];
    }
    if (in) {
        T cyp[3], cym[3], czp[3], czm[3], cxp[3], cxm[3];
        cross_at(p.b, p.a, g + sy, n, cyp);
        cross_at(p.b, p.a, g - sy, n, cym);
        cross_at(p.b, p.a, g + sz, n, czp);
        cross_at(p.b, p.a, g - sz, n, czm);
        cross_at(p.b, p.a, g + 1, n, cxp);
        cross_at(p.b, p.a, g - 1, n, cxm);
        r0 = cyp[2] - cym[2] - czp[1] + czm[1];
        r1 = czp[0] - czm[0] - cxp[2] + cxm[2];
        r2 = cxp[1] - cxm[1] - cyp[0] + cym[0];
    }
    T pcs[1];
    block_scalars<T, 1>([&](int) { return p.sc.advection(); }, pcs);
    if (!live) return;
    if (in) {
        const T pc = pcs[0];
        w0 = w0 + pc * r0;
        w1 = w1 + pc * r1;
        w2 = w2 + pc * r2;
    }
    p.out[g] = w0;
    p.out[n + g] = w1;
    p.out[2 * n + g] = w2;
}

// The same update with its inputs staged by tensor copies (stencil_tma.cu; fp32, nx a multiple of
// 4, 16-byte aligned fields), bitwise the kernel above; a copy wait that runs out writes
// SG_ERR_CUDA to *status.
bool rot_update_tma_ok(const Grid3& G, const void* w1, const void* u, const void* out);
int launch_rot_update_tma(const Grid3& G, const float* w1, const float* u, float* out, const ScalarSrc& sc,
                          int32_t* status, cudaStream_t stream);

// The velocity curl (curl3d_kernel, below) with psi staged by tensor copies (stencil_tma.cu; fp32,
// nx a multiple of 4, 16-byte aligned fields), bitwise the direct kernel, the same max.
bool velocity_curl_tma_ok(const Grid3& G, const void* psi, const void* u);
int launch_velocity_curl_tma(const Grid3& G, const float* psi, float* u, float prefactor, const ScalarSrc& sc,
                             int add_free_stream, float* umax, int32_t* status, cudaStream_t stream);

// The forcing curl above with the forcing staged by tensor copies (stencil_tma.cu; fp32, nx a
// multiple of 4, 16-byte aligned fields), bitwise forcing_curl3d_kernel with a forcing field.
bool forcing_curl_tma_ok(const Grid3& G, const void* w, const void* f, const void* out);
int launch_forcing_curl_tma(const Grid3& G, const float* w, const float* f, float* out, const ScalarSrc& sc,
                            int32_t* status, cudaStream_t stream);

// The diffusion below with its input staged by tensor copies (stencil_tma.cu; fp32, 1 or 3
// components, nx a multiple of 4, 16-byte aligned fields), bitwise the direct kernel.
bool diffusion_tma_ok(const Grid3& G, int ncomp, const void* in, const void* out);
int launch_diffusion_tma(const Grid3& G, int ncomp, const float* in, float* out, const ScalarSrc& sc,
                         int32_t* status, cudaStream_t stream);

// w3 = w2 + k lap(w2) on [1:-1]^3 per component (diffusion_timestep_3d.py)
template <typename T>
__global__ void __launch_bounds__(256) diffusion3d_kernel(Stencil3DParams<T> p) {
    const Grid3 G = p.grid;
    const int64_t n = G.n();
    int x, y, z;
    int64_t g;
    const bool live = cell3(G, x, y, z, g);
    const bool in = live && G.interior(z, y, x);
    const int64_t sy = G.nx, sz = (int64_t)G.nx * G.ny;
    const int nc = p.ncomp ? p.ncomp : 3;
    T v[3] = {T(0), T(0), T(0)}, lap[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (c >= nc || !live) continue;
        const T* f = p.a + c * n;
        v[c] = f[g];
        // diffusion_flux_3d.py:34-43 term order: z+1, z-1, y+1, y-1, x+1, x-1
        if (in) lap[c] = f[g + sz] + f[g - sz] + f[g + sy] + f[g - sy] + f[g + 1] + f[g - 1] - T(6) * f[g];
    }
    T ks[1];
    block_scalars<T, 1>([&](int) { return p.mode == 0 ? p.sc.diffusion() : (double)p.prefactor; }, ks);
    if (!live) return;
    const T k = ks[0];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (c >= nc) continue;
        p.out[c * n + g] = in ? v[c] + k * lap[c] : v[c];
    }
}

// 3D conservative ENO3 advection (advection_flux_3d.py:12-233, advection_timestep_3d.py:38-96).
// On [2:-2]^3 the six face fluxes are accumulated in the reference's pass order (x front, x back,
// y front, y back, z front, z back) onto a start value:
//   flux mode (add_field = 0): start = base, out = the accumulated flux (the flux kernel adds into
//     its buffer; base may equal out);
//   step mode (add_field = 1): start = 0, out = field + flux (the zeroed buffer, then the sum).
// Outside the interior out = base (flux mode) or field (step mode).  The velocity (3 components) is
// shared by every advected component.  NC = 3: one thread advects all three components of a vector
// field (the velocity and the upwind choices are loaded once); NC = 1: one component per thread, the
// component being blockIdx.z / nz.  Neighbours are addressed from per-thread base pointers with
// 32-bit strides (the launcher checks that two planes fit).
template <typename T> struct Eno3D3Params {
    Grid3 grid;
    const T* field;
    const T* base;
    T* out;
    const T* u;      // velocity (3, nz, ny, nx)
    T inv_dx;
    int add_field;
};

template <typename T, int NC>
__global__ void __launch_bounds__(256) eno3_3d_kernel(Eno3D3Params<T> p) {
    const Grid3 G = p.grid;
    const int64_t n = G.n();
    const int comp0 = NC == 1 ? (int)(blockIdx.z / G.nz) : 0;
    const int x = blockIdx.x * kCell3X + threadIdx.x, y = blockIdx.y * kCell3Y + threadIdx.y;
    const int z = blockIdx.z - comp0 * G.nz;
    if (x >= G.nx || y >= G.ny) return;
    const int64_t g = ((int64_t)z * G.ny + y) * G.nx + x;
    const T* f[NC];
    T acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        f[c] = p.field + (int64_t)(comp0 + c) * n + g;
        acc[c] = p.add_field ? T(0) : p.base[(int64_t)(comp0 + c) * n + g];
    }
    const bool in = z >= 2 && z <= G.nz - 3 && y >= 2 && y <= G.ny - 3 && x >= 2 && x <= G.nx - 3;
    if (in) {
        const int strides[3] = {1, G.nx, G.nx * G.ny};
#pragma unroll
        for (int axis = 0; axis < 3; ++axis) {
            const int s = strides[axis];
            const T* ua = p.u + axis * n + g;
            const T um2 = ua[-2 * s], um1 = ua[-s], u0 = ua[0], up1 = ua[s], up2 = ua[2 * s];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const T* fc = f[c];
                const T qm2 = fc[-2 * s] * um2, qm1 = fc[-s] * um1, q0 = fc[0] * u0;
                const T qp1 = fc[s] * up1, qp2 = fc[2 * s] * up2;
                const T front = eno3_face(qm1, q0, qp1, qp2, u0, up1);
                const T back = eno3_face(qm2, qm1, q0, qp1, um1, u0);
                acc[c] = fma(p.inv_dx, front, acc[c]);
                acc[c] = fma(-p.inv_dx, back, acc[c]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) p.out[(int64_t)(comp0 + c) * n + g] = p.add_field ? f[c][0] + acc[c] : acc[c];
}

// One 1D Laplacian filter pass g = 0.25 (2 f - f[+s] - f[-s]) on [1:-1]^3,
// zero ring (laplacian_filter_3d.py:55-73), scalar field.
template <typename T>
__global__ void __launch_bounds__(256) filter_pass3d_kernel(Grid3 G, const T* in, T* out, int axis) {
    int x, y, z;
    int64_t g;
    if (!cell3(G, x, y, z, g)) return;
    const int64_t s = axis == 0 ? 1 : (axis == 1 ? (int64_t)G.nx : (int64_t)G.nx * G.ny);
    T v = T(0);
    if (G.interior(z, y, x)) v = T(0.25) * (-in[g + s] - in[g - s] + T(2) * in[g]);
    out[g] = v;
}

// f -= g (elementwise) over n cells
template <typename T>
__global__ void __launch_bounds__(256) subtract_kernel(int64_t n, T* f, const T* g) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) f[i] = f[i] - g[i];
}

template <typename T>
__global__ void __launch_bounds__(256) copy_kernel(int64_t n, T* dst, const T* src) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

// u = 0.5/dx curl(psi) on [1:-1]^3 (zero ring) + U_inf, with the max of
// sum |u_d| (curl_3d.py:13-132, elementwise_ops_3d.py add_fixed_val)
template <typename T> struct Curl3DParams {
    Grid3 grid;
    const T* psi;
    T* u;
    T prefactor;
    ScalarSrc sc;
    int add_free_stream;
    T* umax;
};

template <typename T>
__global__ void __launch_bounds__(256) curl3d_kernel(Curl3DParams<T> p) {
    const Grid3 G = p.grid;
    const int64_t n = G.n();
    int x, y, z;
    int64_t g;
    T m = T(0);
    // the free stream is converted in every thread: a block-wide conversion (block_scalars) made this
    // kernel slower (0.128 -> 0.133 ms at 256^3), its barrier costing more than the conversions
    if (cell3(G, x, y, z, g)) {
        T c[3] = {T(0), T(0), T(0)};
        if (G.interior(z, y, x)) {
            curl3_at(p.psi, g, n, (int64_t)G.nx, (int64_t)G.nx * G.ny, c);
            c[0] = p.prefactor * c[0];
            c[1] = p.prefactor * c[1];
            c[2] = p.prefactor * c[2];
        }
        if (p.add_free_stream) {
#pragma unroll
            for (int d = 0; d < 3; ++d) c[d] = c[d] + (T)p.sc.free_stream(d);
        }
        p.u[g] = c[0];
        p.u[n + g] = c[1];
        p.u[2 * n + g] = c[2];
        m = fabs(c[0]) + fabs(c[1]) + fabs(c[2]);
    }
    if (p.umax) {
        m = block_max(m);
        if (threadIdx.x == 0 && threadIdx.y == 0) atomic_max_nonneg_filtered(p.umax, m);
    }
}

}  // namespace sg
