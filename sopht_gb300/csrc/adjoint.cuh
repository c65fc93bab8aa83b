// Adjoint (transpose) kernels of the 2D unbounded vorticity step and of the
// virtual-boundary coupling.
//
// Forward step n (navier_stokes_flow_simulators.py:171-209, with the forcing
// of immersed_body_flow_interaction.py / VirtualBoundaryForcing.py):
//   w_a = w   + pf curl_f(f)            forcing curl, interior [1:-1]
//   w_b = w_a + ENO3 flux(w_a, u)       interior [2:-2], inv_dx = -dt/dx
//   w_c = w_b + k lap(w_b)              interior [1:-1]
//   w_d = Pen(w_c)                      X pass then Y pass
//   psi = Poisson(w_d) ; u' = curl(psi) + U_inf
// Every map is linear in the field except the advection, which is bilinear in
// (w_a, u) for a fixed choice of the ENO3 upwind branch per face; the branch
// choice (u_j > -u_{j+1}) is held fixed (its derivative is zero almost
// everywhere).  Each kernel below is the exact transpose of its forward
// counterpart, written as a gather (one thread per output cell, no atomics), so
// adjoint results are bitwise reproducible.
#pragma once

#include "common.cuh"
#include "flow_kernels.cuh"
#include "ib.cuh"

namespace sg {

__device__ __forceinline__ bool inner(int y, int x, int ny, int nx, int g) {
    return y >= g && y <= ny - 1 - g && x >= g && x <= nx - 1 - g;
}

// ------------------------------------------------ deterministic block sums
// Sum of one double per thread over the block, in a fixed order; the result
// is valid in thread 0.
__device__ __forceinline__ double block_sum_fixed(double v) {
    __shared__ double warp_sum[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int nw = (blockDim.x * blockDim.y + 31) / 32;
    if ((tid & 31) == 0) warp_sum[tid >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (tid == 0)
        for (int w = 0; w < nw; ++w) s += warp_sum[w];
    return s;
}

// acc[0] += sum(partials[0:n]) in index order (one warp, fixed tree).
__global__ void __launch_bounds__(32) sum_partials_kernel(int64_t n, const double* partials, double* acc) {
    double v = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += 32) v += partials[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) acc[0] += v;
}

// ------------------------------------------------ curl adjoint (2D)
// Forward (outplane_field_curl_2d.py): on [1:-1]^2
//   u_x[y,x] = p (psi[y+1,x] - psi[y-1,x]),  u_y[y,x] = p (psi[y,x-1] - psi[y,x+1]),
// zero ring.  Transpose: psi_bar = curl^T(u_bar).
template <typename T>
__global__ void __launch_bounds__(256) curl2d_adj_kernel(int ny, int nx, T p, const T* ubar, T* psibar) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const int64_t plane = (int64_t)ny * nx;
    const T* ux = ubar;
    const T* uy = ubar + plane;
    T acc = T(0);
    if (inner(y - 1, x, ny, nx, 1)) acc += ux[(int64_t)(y - 1) * nx + x];
    if (inner(y + 1, x, ny, nx, 1)) acc -= ux[(int64_t)(y + 1) * nx + x];
    if (inner(y, x + 1, ny, nx, 1)) acc += uy[(int64_t)y * nx + x + 1];
    if (inner(y, x - 1, ny, nx, 1)) acc -= uy[(int64_t)y * nx + x - 1];
    psibar[(int64_t)y * nx + x] = acc * p;
}

// ------------------------------------------------ penalisation adjoint
// Forward (penalise_field_boundary_2d.py, as a clamped gather):
//   out[y,x] = cy[y] cx[x] in[clamp(y), clamp(x)],  clamp(i) in [w-1, n-w].
// Transpose at a source index s gathers every i with clamp(i) == s.
__device__ __forceinline__ void band_sources(int s, int n, int w, int& lo, int& hi) {
    if (w <= 0) {
        lo = hi = s;
        return;
    }
    if (s < w - 1 || s > n - w) {  // overwritten band cells receive nothing
        lo = 0;
        hi = -1;
        return;
    }
    lo = s == w - 1 ? 0 : s;
    hi = s == n - w ? n - 1 : s;
}

template <typename T>
__device__ __forceinline__ T pen_adj_at(int y, int x, int ny, int nx, int w, const T* cx, const T* cy, const T* g0,
                                        const T* g1) {
    auto g = [&](int64_t i) { return g1 ? g0[i] + g1[i] : g0[i]; };
    if (w <= 0) return g((int64_t)y * nx + x);
    int ylo, yhi, xlo, xhi;
    band_sources(y, ny, w, ylo, yhi);
    band_sources(x, nx, w, xlo, xhi);
    T acc = T(0);
    for (int yy = ylo; yy <= yhi; ++yy) {
        T row = T(0);
        for (int xx = xlo; xx <= xhi; ++xx) row += cx[xx] * g((int64_t)yy * nx + xx);
        acc += cy[yy] * row;
    }
    return acc;
}

template <typename T>
__global__ void __launch_bounds__(256) pen2d_adj_kernel(int ny, int nx, int w, const T* cx, const T* cy, const T* g,
                                                        T* out) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= nx || y >= ny) return;
    out[(int64_t)y * nx + x] = pen_adj_at<T>(y, x, ny, nx, w, cx, cy, g, nullptr);
}

// ------------------------------------------------ diffusion adjoint
// Forward (diffusion_flux_2d.py / diffusion_timestep_2d.py):
//   out = in + k m (5-point Laplacian of in),  m = interior [1:-1]^2.
// Transpose: in_bar = g + k (sum_nbr m g - 4 m g).  With `field` (the forward
// input), block partials of sum_c m lap(field) g (d loss / d k) are written.
template <typename T>
__global__ void __launch_bounds__(256) diffusion2d_adj_kernel(int ny, int nx, T k, const T* g, T* out, const T* field,
                                                              double* partials) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    double dk = 0.0;
    if (x < nx && y < ny) {
        const int64_t c = (int64_t)y * nx + x;
        auto mg = [&](int yy, int xx) { return inner(yy, xx, ny, nx, 1) ? g[(int64_t)yy * nx + xx] : T(0); };
        const T lap_t = mg(y - 1, x) + mg(y + 1, x) + mg(y, x - 1) + mg(y, x + 1) - T(4) * mg(y, x);
        out[c] = g[c] + k * lap_t;
        if (field && inner(y, x, ny, nx, 1)) {
            const T lap = field[c + nx] + field[c - nx] + field[c + 1] + field[c - 1] - T(4) * field[c];
            dk = (double)lap * (double)g[c];
        }
    }
    if (partials) {
        const double s = block_sum_fixed(dk);
        if (threadIdx.x == 0 && threadIdx.y == 0) partials[blockIdx.y * gridDim.x + blockIdx.x] = s;
    }
}

// ------------------------------------------------ ENO3 advection adjoint
// Forward (advection_flux_2d.py:12-165): for the face j+1/2 between cells j and
// j+1 along an axis, with q = u_axis * w,
//   Phi_j = 1/3 q_{j+1} + 5/6 q_j - 1/6 q_{j-1}     if u_j > -u_{j+1}
//         = 1/3 q_j + 5/6 q_{j+1} - 1/6 q_{j+2}     otherwise,
// and flux[c] = inv_dx (Phi_c - Phi_{c-1}) per axis on the interior [2:-2]^2.
// With g the adjoint of w + flux:
//   Phi_bar_j = inv_dx (m2_j g_j - m2_{j+1} g_{j+1})
//   q_bar_c   = sum_{j=c-2}^{c+1} dPhi_j/dq_c Phi_bar_j
//   w_bar_c   = g_c + u_x q_bar_x + u_y q_bar_y ;  u_bar_c += w_c q_bar_c.
// Coefficient of q_c in Phi_j by offset c - j (left branch, right branch):
//   -1: (-1/6, 0)   0: (5/6, 1/3)   +1: (1/3, 5/6)   +2: (0, -1/6)
template <typename T>
__device__ __forceinline__ T eno3_coef(int off, bool left) {
    const T third = T(1.0 / 3.0), five6 = T(5.0 / 6.0), sixth = T(1.0 / 6.0);
    switch (off) {
        case -1: return left ? -sixth : T(0);
        case 0: return left ? five6 : third;
        case 1: return left ? third : five6;
        default: return left ? T(0) : -sixth;
    }
}

// q_bar along one axis at a cell.  `G(o)`, `U(o)` read g and the axis velocity
// at offset o along the axis; `M(o)` is the advection interior mask there.
template <typename T, typename GF, typename UF, typename MF>
__device__ __forceinline__ T eno3_qbar(T inv_dx, GF G, UF U, MF M) {
    T acc = T(0);
#pragma unroll
    for (int j = -2; j <= 1; ++j) {  // face between offsets j and j+1
        const bool mj = M(j), mj1 = M(j + 1);
        if (!mj && !mj1) continue;
        const T gj = mj ? G(j) : T(0), gj1 = mj1 ? G(j + 1) : T(0);
        const T phibar = inv_dx * (gj - gj1);
        const bool left = U(j) > -U(j + 1);
        acc += eno3_coef<T>(-j, left) * phibar;
    }
    return acc;
}

template <typename T>
__global__ void __launch_bounds__(256) eno3_2d_adj_kernel(int ny, int nx, T inv_dx, const T* w, const T* u,
                                                          const T* g, T* out, T* ubar) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const int64_t plane = (int64_t)ny * nx;
    const int64_t c = (int64_t)y * nx + x;
    const T* ux = u;
    const T* uy = u + plane;
    // offsets that would leave the grid only occur next to masked faces
    auto clampx = [&](int o) { return min(max(x + o, 0), nx - 1); };
    auto clampy = [&](int o) { return min(max(y + o, 0), ny - 1); };
    const T qx = eno3_qbar<T>(
        inv_dx, [&](int o) { return g[(int64_t)y * nx + clampx(o)]; },
        [&](int o) { return ux[(int64_t)y * nx + clampx(o)]; }, [&](int o) { return inner(y, x + o, ny, nx, 2); });
    const T qy = eno3_qbar<T>(
        inv_dx, [&](int o) { return g[(int64_t)clampy(o) * nx + x]; },
        [&](int o) { return uy[(int64_t)clampy(o) * nx + x]; }, [&](int o) { return inner(y + o, x, ny, nx, 2); });
    out[c] = g[c] + ux[c] * qx + uy[c] * qy;
    if (ubar) {
        ubar[c] = ubar[c] + w[c] * qx;
        ubar[plane + c] = ubar[plane + c] + w[c] * qy;
    }
}

// ------------------------------------------------ forcing-curl adjoint
// Forward (update_vorticity_from_velocity_forcing_2d.py:28-44): on [1:-1]^2
//   w[y,x] += p (f_y[y,x+1] - f_y[y,x-1] - f_x[y+1,x] + f_x[y-1,x]).
// Transpose: f_bar += p curl_f^T(g); w passes through unchanged.
template <typename T>
__global__ void __launch_bounds__(256) fcurl2d_adj_kernel(int ny, int nx, T p, const T* g, T* fbar) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const int64_t plane = (int64_t)ny * nx;
    const int64_t c = (int64_t)y * nx + x;
    auto mg = [&](int yy, int xx) { return inner(yy, xx, ny, nx, 1) ? g[(int64_t)yy * nx + xx] : T(0); };
    fbar[c] = fbar[c] + p * (mg(y + 1, x) - mg(y - 1, x));
    fbar[plane + c] = fbar[plane + c] + p * (mg(y, x - 1) - mg(y, x + 1));
}

// ------------------------------------------------ fused reverse sweep (2D)
// The transpose of Pen . diffusion . advection . forcing-curl in one pass over
// 32 x 16 tiles with a 4-cell halo:
//   g_d = g0 + g1 (adjoint of w after the step plus Poisson(psi_bar))
//   g_c = Pen^T g_d             (halo 4, gathered from global memory)
//   g_b = g_c + k lap^T(m g_c)  (halo 3) ; partial of sum m lap(w_b) g_c
//   g_a = g_b + u q_bar(g_b)    (halo 1) ; u_bar = w_a q_bar on the tile
//   f_bar = pf curl_f^T(g_a)    (tile)   ; w_bar = g_a on the tile
template <typename T> struct RSweep2DParams {
    int ny, nx, width;
    const T* g0;
    const T* g1;   // may be null
    const T* cx;
    const T* cy;
    T k;
    const T* w_b;  // forward diffusion input (null: no viscosity partials)
    double* partials;
    T inv_dx;
    const T* w_a;  // forward advection input
    const T* u;    // forward velocity (2, ny, nx)
    T pf;
    T* w_bar;      // out
    T* u_bar;      // out (2, ny, nx), overwritten
    T* f_bar;      // out (2, ny, nx), overwritten; may be null
};

template <typename T, int TX, int TY>
__global__ void __launch_bounds__(256) rsweep2d_kernel(RSweep2DParams<T> p) {
    constexpr int H4X = TX + 8, H4Y = TY + 8;
    constexpr int H3X = TX + 6, H3Y = TY + 6;
    constexpr int H1X = TX + 2, H1Y = TY + 2;
    __shared__ T s_c[H4Y * H4X];
    __shared__ T s_b[H3Y * H3X];
    __shared__ T s_ux[H3Y * H3X];
    __shared__ T s_uy[H3Y * H3X];
    __shared__ T s_wa[H1Y * H1X];
    __shared__ T s_a[H1Y * H1X];
    const int nthr = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    const int ny = p.ny, nx = p.nx;
    const int64_t plane = (int64_t)ny * nx;
    auto in_grid = [&](int y, int x) { return y >= 0 && y < ny && x >= 0 && x < nx; };
    // A: g_c on halo 4; velocity on halo 3; w_a on halo 1
    for (int e = tid; e < H4Y * H4X; e += nthr) {
        const int y = y0 - 4 + e / H4X, x = x0 - 4 + e % H4X;
        s_c[e] = in_grid(y, x) ? pen_adj_at<T>(y, x, ny, nx, p.width, p.cx, p.cy, p.g0, p.g1) : T(0);
    }
    for (int e = tid; e < H3Y * H3X; e += nthr) {
        const int y = y0 - 3 + e / H3X, x = x0 - 3 + e % H3X;
        T ux = T(0), uy = T(0);
        if (in_grid(y, x)) {
            const int64_t g = (int64_t)y * nx + x;
            ux = p.u[g];
            uy = p.u[plane + g];
        }
        s_ux[e] = ux;
        s_uy[e] = uy;
    }
    for (int e = tid; e < H1Y * H1X; e += nthr) {
        const int y = y0 - 1 + e / H1X, x = x0 - 1 + e % H1X;
        s_wa[e] = in_grid(y, x) ? p.w_a[(int64_t)y * nx + x] : T(0);
    }
    __syncthreads();
    // B: g_b on halo 3 (+ viscosity partial on the tile)
    double dk = 0.0;
    for (int e = tid; e < H3Y * H3X; e += nthr) {
        const int ly = e / H3X, lx = e % H3X;
        const int y = y0 - 3 + ly, x = x0 - 3 + lx;
        const int c = (ly + 1) * H4X + (lx + 1);
        T v = T(0);
        if (in_grid(y, x)) {
            auto mg = [&](int dy, int dx) {
                return inner(y + dy, x + dx, ny, nx, 1) ? s_c[c + dy * H4X + dx] : T(0);
            };
            const T lap_t = mg(-1, 0) + mg(1, 0) + mg(0, -1) + mg(0, 1) - T(4) * mg(0, 0);
            v = s_c[c] + p.k * lap_t;
            if (p.w_b && ly >= 3 && ly < 3 + TY && lx >= 3 && lx < 3 + TX && inner(y, x, ny, nx, 1)) {
                const int64_t g = (int64_t)y * nx + x;
                const T lap = p.w_b[g + nx] + p.w_b[g - nx] + p.w_b[g + 1] + p.w_b[g - 1] - T(4) * p.w_b[g];
                dk += (double)lap * (double)s_c[c];
            }
        }
        s_b[e] = v;
    }
    __syncthreads();
    // C: g_a on halo 1; u_bar on the tile
    for (int e = tid; e < H1Y * H1X; e += nthr) {
        const int ly = e / H1X, lx = e % H1X;
        const int y = y0 - 1 + ly, x = x0 - 1 + lx;
        const int c = (ly + 2) * H3X + (lx + 2);
        T ga = T(0);
        if (in_grid(y, x)) {
            const T qx = eno3_qbar<T>(
                p.inv_dx, [&](int o) { return s_b[c + o]; }, [&](int o) { return s_ux[c + o]; },
                [&](int o) { return inner(y, x + o, ny, nx, 2); });
            const T qy = eno3_qbar<T>(
                p.inv_dx, [&](int o) { return s_b[c + o * H3X]; }, [&](int o) { return s_uy[c + o * H3X]; },
                [&](int o) { return inner(y + o, x, ny, nx, 2); });
            ga = s_b[c] + s_ux[c] * qx + s_uy[c] * qy;
            if (ly >= 1 && ly <= TY && lx >= 1 && lx <= TX) {
                const int64_t g = (int64_t)y * nx + x;
                const T wa = s_wa[e];
                p.u_bar[g] = wa * qx;
                p.u_bar[plane + g] = wa * qy;
            }
        }
        s_a[e] = ga;
    }
    __syncthreads();
    // D: f_bar and w_bar on the tile
    for (int e = tid; e < TY * TX; e += nthr) {
        const int ly = e / TX, lx = e % TX;
        const int y = y0 + ly, x = x0 + lx;
        if (!in_grid(y, x)) continue;
        const int c = (ly + 1) * H1X + (lx + 1);
        const int64_t g = (int64_t)y * nx + x;
        p.w_bar[g] = s_a[c];
        if (p.f_bar) {
            auto ma = [&](int dy, int dx) {
                return inner(y + dy, x + dx, ny, nx, 1) ? s_a[c + dy * H1X + dx] : T(0);
            };
            p.f_bar[g] = p.pf * (ma(1, 0) - ma(-1, 0));
            p.f_bar[plane + g] = p.pf * (ma(0, -1) - ma(0, 1));
        }
    }
    if (p.partials) {
        const double s = block_sum_fixed(dk);
        if (tid == 0) p.partials[blockIdx.y * gridDim.x + blockIdx.x] = s;
    }
}

// ------------------------------------------------ virtual-boundary adjoint
// Forward per marker i (VirtualBoundaryForcing.py:132-185, 232-283):
//   xi_i  = xi_i + dt_n dU_i(previous call)               (time_step)
//   U_i   = dx^dim sum_window phi_i u ;  dU_i = U_i - V_i
//   F_i   = K xi_i + C dU_i ;  f += sum_i phi_i F_i        (spread)
// Reverse of one call (one warp per marker):
//   F_bar   = sum_window phi_i f_bar + F_const            (spread^T + loss)
//   xi_bar += K F_bar
//   dU_bar  = C F_bar + carry_i   (carry = dt_{n+1} xi_bar from the next step)
//   V_bar  -= dU_bar ; U_bar_scaled = dx^dim dU_bar       (spread onto u_bar next)
//   carry   = dt_n xi_bar                                 (time_step^T)
template <typename T> struct IBAdjParams {
    int dim, nz, ny, nx, n_lag;
    const int32_t* nearest;
    const T* weights;
    const T* f_bar;      // Eulerian forcing adjoint (dim, cells) or null
    double F_const[3];   // direct adjoint of F per component (loss weights)
    double K, C, dt, dxd;
    T* xi_bar;
    T* carry;
    double* v_bar;       // (dim, n_lag) float64, accumulated
    T* u_flow_bar;       // (dim, n_lag) out: dx^dim dU_bar
};

template <typename T>
__global__ void __launch_bounds__(256) ib_adj_kernel(IBAdjParams<T> p) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= p.n_lag) return;
    const int n = p.n_lag, dim = p.dim;
    T acc[3] = {T(0), T(0), T(0)};
    if (p.f_bar) {
        const int cells = dim == 2 ? 16 : 64;
        const int64_t plane = (int64_t)p.ny * p.nx;
        const int64_t ncell = plane * (dim == 3 ? p.nz : 1);
        const int ex = p.nearest[i] - 1, ey = p.nearest[n + i] - 1, ez = dim == 3 ? p.nearest[2 * n + i] - 1 : 0;
        const bool inside = ex >= 0 && ex + 3 < p.nx && ey >= 0 && ey + 3 < p.ny &&
                            (dim == 2 || (ez >= 0 && ez + 3 < p.nz));
        if (inside) {
            for (int c = lane; c < cells; c += 32) {
                const int64_t g = (int64_t)(ez + (c >> 4)) * plane + (int64_t)(ey + ((c >> 2) & 3)) * p.nx +
                                  ex + (c & 3);
                const T w = p.weights[c * n + i];
                for (int d = 0; d < dim; ++d) acc[d] += p.f_bar[d * ncell + g] * w;
            }
        }
        for (int d = 0; d < dim; ++d)
            for (int o = 16; o > 0; o >>= 1) acc[d] += __shfl_xor_sync(0xffffffffu, acc[d], o);
    }
    if (lane < dim) {
        const int d = lane;
        const int64_t j = (int64_t)d * n + i;
        const double Fb = (double)acc[d] + p.F_const[d];
        const double xb = (double)p.xi_bar[j] + p.K * Fb;
        const double dUb = p.C * Fb + (double)p.carry[j];
        p.xi_bar[j] = (T)xb;
        p.v_bar[j] -= dUb;
        p.u_flow_bar[j] = (T)(p.dxd * dUb);
        p.carry[j] = (T)(p.dt * xb);
    }
}

// acc[0] += sum_d wgt[d] sum_i F[d, i] (one warp, fixed order)
template <typename T>
__global__ void __launch_bounds__(32) lag_weighted_sum_kernel(int dim, int n_lag, const T* F, double w0, double w1,
                                                              double w2, double* acc) {
    const double wgt[3] = {w0, w1, w2};
    double v = 0.0;
    for (int d = 0; d < dim; ++d)
        for (int i = threadIdx.x; i < n_lag; i += 32) v += wgt[d] * (double)F[d * n_lag + i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) acc[0] += v;
}

}  // namespace sg
