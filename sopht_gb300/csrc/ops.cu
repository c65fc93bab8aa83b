// Single-operator entry points: the reference's individual stencil kernels,
// exposed one by one for the lower-level kernel-factory API and for per-operator
// parity tests.  The fused flow step does not go through these.
#include "flow_kernels.cuh"

namespace sg {

template <typename T>
int launch_sweep2d(const Sweep2DParams<T>& p, cudaStream_t stream);
template <typename T>
int launch_curl2d(const Curl2DParams<T>& p, cudaStream_t stream);
template <typename T>
int filter3d(Grid3 G, T* field, int filter_type, int order, T* a, T* b, cudaStream_t stream);

template <typename T>
__global__ void __launch_bounds__(256) penalise_kernel(int dim, int nz, int ny, int nx, int width, const T* in,
                                                        T* out, const T* cx, const T* cy, const T* cz, int ncomp) {
    const int64_t n = (int64_t)nz * ny * nx;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * ncomp) return;
    const int64_t g = t % n;
    const int c = (int)(t / n);
    const int x = (int)(g % nx), y = (int)((g / nx) % ny), z = (int)(g / ((int64_t)nx * ny));
    const int sx = clamp_band(x, nx, width), sy = clamp_band(y, ny, width);
    const int sz = dim == 3 ? clamp_band(z, nz, width) : 0;
    T v = in[c * n + ((int64_t)sz * ny + sy) * nx + sx];
    if (width > 0) {
        v = v * cx[x];
        v = v * cy[y];
        if (dim == 3) v = v * cz[z];
    }
    out[c * n + g] = v;
}

template <typename T>
__global__ void __launch_bounds__(256) cross3d_kernel(int64_t n, const T* a, const T* b, T* out) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    T c[3];
    cross_at(a, b, g, n, c);
    out[g] = c[0];
    out[n + g] = c[1];
    out[2 * n + g] = c[2];
}

template <typename T>
__global__ void __launch_bounds__(256) divergence3d_kernel(Grid3 G, const T* f, T* div, T inv_dx) {
    const int64_t n = G.n();
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const int x = (int)(g % G.nx), y = (int)((g / G.nx) % G.ny), z = (int)(g / ((int64_t)G.nx * G.ny));
    const int64_t sy = G.nx, sz = (int64_t)G.nx * G.ny;
    T v = T(0);
    if (G.interior(z, y, x)) {
        // divergence_3d.py: (dfx/dx + dfy/dy + dfz/dz) * 0.5 * inv_dx
        v = (f[g + 1] - f[g - 1] + f[n + g + sy] - f[n + g - sy] + f[2 * n + g + sz] - f[2 * n + g - sz]) *
            T(0.5) * inv_dx;
    }
    div[g] = v;
}

template <typename T>
static int sweep_op(int ny, int nx, const void* in, void* out, const void* u, const void* f, double pf, double adv,
                    double diff, int flags, cudaStream_t stream) {
    Sweep2DParams<T> s{};
    s.ny = ny;
    s.nx = nx;
    s.w = (const T*)in;
    s.u = (const T*)u;
    s.f = (const T*)f;
    s.out = (T*)out;
    s.sc.host.forcing_prefac = pf;
    s.sc.host.advection_prefac = adv;
    s.sc.host.diffusion_prefac = diff;
    s.flags = flags;
    return launch_sweep2d<T>(s, stream);
}

}  // namespace sg

using namespace sg;

#define SG_DTYPE_DISPATCH(dtype, CALL_F, CALL_D)                                     \
    do {                                                                              \
        if ((dtype) == SG_F32) return CALL_F;                                         \
        SG_REQUIRE((dtype) == SG_F64, SG_ERR_INVALID_ARG, "bad dtype %d", (int)(dtype)); \
        return CALL_D;                                                                \
    } while (0)

static int check2d(int ny, int nx, const void* a, const void* b) {
    SG_REQUIRE(a && b, SG_ERR_INVALID_ARG, "null field pointer");
    SG_REQUIRE(ny >= 1 && nx >= 1, SG_ERR_SHAPE, "bad 2D extent (%d, %d)", ny, nx);
    SG_REQUIRE(a != b, SG_ERR_INVALID_ARG, "input and output must not alias (stencil halo)");
    return SG_OK;
}

extern "C" int sg_advection_eno3_step_2d(int dtype, int ny, int nx, const void* in, void* out, const void* velocity,
                                         double dt_by_dx, void* stream) {
    SG_TRY(check2d(ny, nx, in, out));
    SG_REQUIRE(velocity, SG_ERR_INVALID_ARG, "null velocity");
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, sweep_op<float>(ny, nx, in, out, velocity, nullptr, 0, dt_by_dx, 0, SWEEP_ADVECT, s),
                      sweep_op<double>(ny, nx, in, out, velocity, nullptr, 0, dt_by_dx, 0, SWEEP_ADVECT, s));
}

extern "C" int sg_diffusion_step_2d(int dtype, int ny, int nx, const void* in, void* out, double k, void* stream) {
    SG_TRY(check2d(ny, nx, in, out));
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, sweep_op<float>(ny, nx, in, out, nullptr, nullptr, 0, 0, k, SWEEP_DIFFUSE, s),
                      sweep_op<double>(ny, nx, in, out, nullptr, nullptr, 0, 0, k, SWEEP_DIFFUSE, s));
}

extern "C" int sg_forcing_curl_update_2d(int dtype, int ny, int nx, const void* in, void* out, const void* forcing,
                                         double prefactor, void* stream) {
    SG_TRY(check2d(ny, nx, in, out));
    SG_REQUIRE(forcing, SG_ERR_INVALID_ARG, "null forcing");
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, sweep_op<float>(ny, nx, in, out, nullptr, forcing, prefactor, 0, 0, 0, s),
                      sweep_op<double>(ny, nx, in, out, nullptr, forcing, prefactor, 0, 0, 0, s));
}

template <typename T>
static int curl2d_op(int ny, int nx, const void* psi, void* curl, double pref, cudaStream_t s) {
    Curl2DParams<T> c{};
    c.ny = ny;
    c.nx = nx;
    c.psi = (const T*)psi;
    c.u = (T*)curl;
    c.prefactor = (T)pref;
    c.add_free_stream = 0;
    c.umax = nullptr;
    return launch_curl2d<T>(c, s);
}

extern "C" int sg_outplane_curl_2d(int dtype, int ny, int nx, const void* psi, void* curl, double prefactor,
                                   void* stream) {
    SG_TRY(check2d(ny, nx, psi, curl));
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, curl2d_op<float>(ny, nx, psi, curl, prefactor, s),
                      curl2d_op<double>(ny, nx, psi, curl, prefactor, s));
}

template <typename T>
static int penalise_op(int dim, int nz, int ny, int nx, const void* in, void* out, int width, const void* cx,
                       const void* cy, const void* cz, int ncomp, cudaStream_t s) {
    const int64_t n = (int64_t)nz * ny * nx * ncomp;
    penalise_kernel<T><<<ceil_div(n, 256), 256, 0, s>>>(dim, nz, ny, nx, width, (const T*)in, (T*)out,
                                                        (const T*)cx, (const T*)cy, (const T*)cz, ncomp);
    return launch_status("penalise");
}

extern "C" int sg_penalise_2d(int dtype, int ny, int nx, const void* in, void* out, int width, const void* cx,
                              const void* cy, void* stream) {
    SG_TRY(check2d(ny, nx, in, out));
    SG_REQUIRE(width >= 0 && 2 * width <= nx && 2 * width <= ny, SG_ERR_SHAPE, "penalty width does not fit");
    SG_REQUIRE(width == 0 || (cx && cy), SG_ERR_INVALID_ARG, "null penalisation table");
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, penalise_op<float>(2, 1, ny, nx, in, out, width, cx, cy, nullptr, 1, s),
                      penalise_op<double>(2, 1, ny, nx, in, out, width, cx, cy, nullptr, 1, s));
}

// The status word of the operator entries' kernels (a bounded wait that ran out), one per device.
static __device__ int32_t ops_status_word;

static int32_t* ops_status() {
    static int32_t* addr[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    if (!addr[dev]) {
        void* a = nullptr;
        if (cudaGetSymbolAddress(&a, ops_status_word) != cudaSuccess) return nullptr;
        addr[dev] = static_cast<int32_t*>(a);
    }
    return addr[dev];
}

extern "C" int sg_ops_kernel_status(int32_t* host_out) {
    SG_REQUIRE(host_out, SG_ERR_INVALID_ARG, "ops kernel status: null output");
    return cuda_status(cudaMemcpyFromSymbol(host_out, ops_status_word, sizeof(int32_t)), "read ops kernel status");
}

static int check3d(int nz, int ny, int nx, const void* a, const void* b) {
    SG_REQUIRE(a && b, SG_ERR_INVALID_ARG, "null field pointer");
    SG_REQUIRE(nz >= 1 && ny >= 1 && nx >= 1, SG_ERR_SHAPE, "bad 3D extent");
    SG_REQUIRE(a != b, SG_ERR_INVALID_ARG, "input and output must not alias (stencil halo)");
    return SG_OK;
}

template <typename T>
static int stencil3d_op(int which, int nz, int ny, int nx, const void* a, const void* b, void* out, double pref,
                        cudaStream_t s) {
    Stencil3DParams<T> p{};
    p.grid = Grid3{nz, ny, nx};
    p.a = (const T*)a;
    p.b = (const T*)b;
    p.out = (T*)out;
    p.prefactor = (T)pref;
    p.mode = 1;
    if (which == 0) forcing_curl3d_kernel<T><<<cell3_grid(p.grid), cell3_block(), 0, s>>>(p);
    else if (which == 1) diffusion3d_kernel<T><<<cell3_grid(p.grid), cell3_block(), 0, s>>>(p);
    else {
        Curl3DParams<T> c{};
        c.grid = p.grid;
        c.psi = (const T*)a;
        c.u = (T*)out;
        c.prefactor = (T)pref;
        curl3d_kernel<T><<<cell3_grid(c.grid), cell3_block(), 0, s>>>(c);
    }
    return launch_status("stencil3d op");
}

extern "C" int sg_curl_3d(int dtype, int nz, int ny, int nx, const void* field, void* curl, double prefactor,
                          void* stream) {
    SG_TRY(check3d(nz, ny, nx, field, curl));
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, stencil3d_op<float>(2, nz, ny, nx, field, nullptr, curl, prefactor, s),
                      stencil3d_op<double>(2, nz, ny, nx, field, nullptr, curl, prefactor, s));
}

extern "C" int sg_forcing_curl_update_3d(int dtype, int nz, int ny, int nx, const void* in, void* out,
                                         const void* forcing, double prefactor, void* stream) {
    SG_TRY(check3d(nz, ny, nx, in, out));
    SG_REQUIRE(forcing, SG_ERR_INVALID_ARG, "null forcing");
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, stencil3d_op<float>(0, nz, ny, nx, in, forcing, out, prefactor, s),
                      stencil3d_op<double>(0, nz, ny, nx, in, forcing, out, prefactor, s));
}

extern "C" int sg_diffusion_step_3d(int dtype, int nz, int ny, int nx, const void* in, void* out, double k,
                                    void* stream) {
    SG_TRY(check3d(nz, ny, nx, in, out));
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, stencil3d_op<float>(1, nz, ny, nx, in, nullptr, out, k, s),
                      stencil3d_op<double>(1, nz, ny, nx, in, nullptr, out, k, s));
}

// w2 = w1 + pc curl(u x w1) on [1:-1]^3 (w1 elsewhere), the 3D step's rotational-form update
template <typename T>
static int rotational_update_op(int nz, int ny, int nx, const void* w1, const void* u, void* out, double pc,
                                int staged, int32_t* status, cudaStream_t s) {
    Stencil3DParams<T> p{};
    p.grid = Grid3{nz, ny, nx};
    p.a = (const T*)w1;
    p.b = (const T*)u;
    p.out = (T*)out;
    p.sc.host.advection_prefac = pc;
    if (staged) {
        if constexpr (sizeof(T) == 4) {
            SG_REQUIRE(rot_update_tma_ok(p.grid, w1, u, out), SG_ERR_INVALID_ARG,
                       "rotational update: the staged form needs fp32, nx a multiple of 4 and 16-byte aligned fields");
            return launch_rot_update_tma(p.grid, (const float*)w1, (const float*)u, (float*)out, p.sc, status, s);
        }
        SG_REQUIRE(false, SG_ERR_INVALID_ARG, "rotational update: the staged form is fp32 only");
    }
    rotational_update3d_kernel<T><<<cell3_grid(p.grid), cell3_block(), 0, s>>>(p);
    return launch_status("rotational update");
}

// u = prefactor curl(psi) on [1:-1]^3 (0 on the ring) + free_stream (host, 3 values, or null),
// with max sum |u_d| into *umax (device, or null; not reset here): staged = 0 the direct-load
// kernel, 1 psi staged by tensor copies (fp32), the same bits
extern "C" int sg_curl_3d_staged(int dtype, int nz, int ny, int nx, const void* psi, void* u, double prefactor,
                                 const double* free_stream, void* umax, int staged, int32_t* status, void* stream) {
    SG_TRY(check3d(nz, ny, nx, psi, u));
    auto s = (cudaStream_t)stream;
    const Grid3 G{nz, ny, nx};
    ScalarSrc sc{};
    if (free_stream)
        for (int d = 0; d < 3; ++d) sc.host.free_stream[d] = free_stream[d];
    if (staged) {
        SG_REQUIRE(dtype == SG_F32 && status && velocity_curl_tma_ok(G, psi, u), SG_ERR_INVALID_ARG,
                   "curl: the staged form needs fp32, a status word, nx a multiple of 4 and 16-byte aligned fields");
        return launch_velocity_curl_tma(G, (const float*)psi, (float*)u, (float)prefactor, sc, free_stream != nullptr,
                                        (float*)umax, status, s);
    }
    auto direct = [&](auto tag) {
        using T = decltype(tag);
        Curl3DParams<T> c{};
        c.grid = G;
        c.psi = (const T*)psi;
        c.u = (T*)u;
        c.prefactor = (T)prefactor;
        c.sc = sc;
        c.add_free_stream = free_stream != nullptr;
        c.umax = (T*)umax;
        curl3d_kernel<T><<<cell3_grid(c.grid), cell3_block(), 0, s>>>(c);
        return launch_status("curl3d");
    };
    SG_DTYPE_DISPATCH(dtype, direct(float{}), direct(double{}));
}

// w1 = w + pf curl(f) on [1:-1]^3: staged = 0 the direct-load kernel, 1 the forcing staged by
// tensor copies (fp32), the same bits
extern "C" int sg_forcing_curl_3d_staged(int dtype, int nz, int ny, int nx, const void* in, void* out,
                                         const void* forcing, double prefactor, int staged, int32_t* status,
                                         void* stream) {
    SG_TRY(check3d(nz, ny, nx, in, out));
    SG_REQUIRE(forcing && forcing != out, SG_ERR_INVALID_ARG, "forcing curl: null forcing or forcing aliasing out");
    auto s = (cudaStream_t)stream;
    const Grid3 G{nz, ny, nx};
    if (staged) {
        SG_REQUIRE(dtype == SG_F32 && status && forcing_curl_tma_ok(G, in, forcing, out), SG_ERR_INVALID_ARG,
                   "forcing curl: the staged form needs fp32, a status word, nx a multiple of 4 and 16-byte aligned "
                   "fields");
        ScalarSrc sc{};
        sc.host.forcing_prefac = prefactor;
        return launch_forcing_curl_tma(G, (const float*)in, (const float*)forcing, (float*)out, sc, status, s);
    }
    SG_DTYPE_DISPATCH(dtype, stencil3d_op<float>(0, nz, ny, nx, in, forcing, out, prefactor, s),
                      stencil3d_op<double>(0, nz, ny, nx, in, forcing, out, prefactor, s));
}

// w3 = w2 + k lap(w2) on [1:-1]^3 for ncomp (1 or 3) components: staged = 0 the direct-load kernel,
// 1 the tensor-copy-staged one (fp32), the same bits
extern "C" int sg_diffusion_3d_staged(int dtype, int nz, int ny, int nx, int ncomp, const void* in, void* out,
                                      double k, int staged, int32_t* status, void* stream) {
    SG_TRY(check3d(nz, ny, nx, in, out));
    SG_REQUIRE(ncomp == 1 || ncomp == 3, SG_ERR_INVALID_ARG, "diffusion: 1 or 3 components");
    auto s = (cudaStream_t)stream;
    const Grid3 G{nz, ny, nx};
    if (staged) {
        SG_REQUIRE(dtype == SG_F32 && status && diffusion_tma_ok(G, ncomp, in, out), SG_ERR_INVALID_ARG,
                   "diffusion: the staged form needs fp32, a status word, nx a multiple of 4 and 16-byte aligned fields");
        ScalarSrc sc{};
        sc.host.diffusion_prefac = k;
        return launch_diffusion_tma(G, ncomp, (const float*)in, (float*)out, sc, status, s);
    }
    auto direct = [&](auto tag) {
        using T = decltype(tag);
        Stencil3DParams<T> p{};
        p.grid = G;
        p.a = (const T*)in;
        p.out = (T*)out;
        p.prefactor = (T)k;
        p.mode = 1;
        p.ncomp = ncomp;
        diffusion3d_kernel<T><<<cell3_grid(p.grid), cell3_block(), 0, s>>>(p);
        return launch_status("diffusion3d");
    };
    SG_DTYPE_DISPATCH(dtype, direct(float{}), direct(double{}));
}

extern "C" int sg_rotational_update_3d(int dtype, int nz, int ny, int nx, const void* w1, const void* u, void* out,
                                       double prefactor, int staged, int32_t* status, void* stream) {
    SG_TRY(check3d(nz, ny, nx, w1, out));
    SG_REQUIRE(u && u != out, SG_ERR_INVALID_ARG, "rotational update: null velocity or velocity aliasing out");
    SG_REQUIRE(!staged || status, SG_ERR_INVALID_ARG, "rotational update: the staged form needs a status word");
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, rotational_update_op<float>(nz, ny, nx, w1, u, out, prefactor, staged, status, s),
                      rotational_update_op<double>(nz, ny, nx, w1, u, out, prefactor, staged, status, s));
}

template <typename T>
static int cross_op(int64_t n, const void* a, const void* b, void* out, cudaStream_t s) {
    cross3d_kernel<T><<<ceil_div(n, 256), 256, 0, s>>>(n, (const T*)a, (const T*)b, (T*)out);
    return launch_status("cross3d");
}

extern "C" int sg_cross_3d(int dtype, int64_t n, const void* a, const void* b, void* out, void* stream) {
    SG_REQUIRE(a && b && out && n >= 1, SG_ERR_INVALID_ARG, "cross: bad argument");
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, cross_op<float>(n, a, b, out, s), cross_op<double>(n, a, b, out, s));
}

template <typename T>
static int div_op(int nz, int ny, int nx, const void* f, void* div, double inv_dx, cudaStream_t s) {
    Grid3 G{nz, ny, nx};
    divergence3d_kernel<T><<<ceil_div((int64_t)nz * ny * nx, 256), 256, 0, s>>>(G, (const T*)f, (T*)div, (T)inv_dx);
    return launch_status("divergence3d");
}

extern "C" int sg_divergence_3d(int dtype, int nz, int ny, int nx, const void* field, void* div, double inv_dx,
                                void* stream) {
    SG_TRY(check3d(nz, ny, nx, field, div));
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, div_op<float>(nz, ny, nx, field, div, inv_dx, s),
                      div_op<double>(nz, ny, nx, field, div, inv_dx, s));
}

extern "C" int sg_penalise_3d(int dtype, int nz, int ny, int nx, const void* in, void* out, int width,
                              const void* cx, const void* cy, const void* cz, void* stream) {
    SG_TRY(check3d(nz, ny, nx, in, out));
    SG_REQUIRE(width >= 0 && 2 * width <= nx && 2 * width <= ny && 2 * width <= nz, SG_ERR_SHAPE,
               "penalty width does not fit");
    SG_REQUIRE(width == 0 || (cx && cy && cz), SG_ERR_INVALID_ARG, "null penalisation table");
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, penalise_op<float>(3, nz, ny, nx, in, out, width, cx, cy, cz, 3, s),
                      penalise_op<double>(3, nz, ny, nx, in, out, width, cx, cy, cz, 3, s));
}

extern "C" int sg_laplacian_filter_3d(int dtype, int nz, int ny, int nx, void* field, int filter_type,
                                      int filter_order, void* a, void* b, void* stream) {
    SG_REQUIRE(field && a && b, SG_ERR_INVALID_ARG, "filter: null pointer");
    SG_REQUIRE(filter_type >= 0 && filter_type <= 2 && filter_order >= 0, SG_ERR_INVALID_ARG, "filter: bad setting");
    auto s = (cudaStream_t)stream;
    Grid3 G{nz, ny, nx};
    SG_DTYPE_DISPATCH(dtype, filter3d<float>(G, (float*)field, filter_type, filter_order, (float*)a, (float*)b, s),
                      filter3d<double>(G, (double*)field, filter_type, filter_order, (double*)a, (double*)b, s));
}

// ------------------------------------------------------------ passive transport
namespace sg {

// ncomp components; vector_threads: one thread per cell advects all three (ncomp must be 3)
template <typename T>
static int eno3_3d_launch(int nz, int ny, int nx, int ncomp, const void* field, const void* base, void* out,
                          const void* u, double inv_dx, int add_field, bool vector_threads, cudaStream_t s) {
    SG_REQUIRE((int64_t)nx * ny <= (int64_t)1 << 29, SG_ERR_SHAPE, "eno3 3d: plane of %d x %d too large", ny, nx);
    Eno3D3Params<T> p{};
    p.grid = Grid3{nz, ny, nx};
    p.field = (const T*)field;
    p.base = (const T*)base;
    p.out = (T*)out;
    p.u = (const T*)u;
    p.inv_dx = (T)inv_dx;
    p.add_field = add_field;
    dim3 grid = cell3_grid(p.grid);
    if (vector_threads) {
        SG_REQUIRE(ncomp == 3, SG_ERR_INVALID_ARG, "eno3 3d: vector threads need 3 components");
        eno3_3d_kernel<T, 3><<<grid, cell3_block(), 0, s>>>(p);
    } else {
        grid.z = (unsigned)nz * (unsigned)ncomp;
        eno3_3d_kernel<T, 1><<<grid, cell3_block(), 0, s>>>(p);
    }
    return launch_status("eno3_3d");
}

template <typename T>
static int diffusion3d_comps_launch(int nz, int ny, int nx, int ncomp, const void* in, void* out, double k,
                                    cudaStream_t s) {
    if constexpr (sizeof(T) == 4) {
        const Grid3 G{nz, ny, nx};
        int32_t* status = ops_status();
        if (status && diffusion_tma_ok(G, ncomp, in, out)) {
            ScalarSrc sc{};
            sc.host.diffusion_prefac = k;
            return launch_diffusion_tma(G, ncomp, (const float*)in, (float*)out, sc, status, s);
        }
    }
    Stencil3DParams<T> p{};
    p.grid = Grid3{nz, ny, nx};
    p.a = (const T*)in;
    p.out = (T*)out;
    p.prefactor = (T)k;
    p.mode = 1;
    p.ncomp = ncomp;
    diffusion3d_kernel<T><<<cell3_grid(p.grid), cell3_block(), 0, s>>>(p);
    return launch_status("diffusion3d");
}

// PassiveTransportFlowSimulator._advection_and_diffusion_time_step: advection then diffusion of
// every component, in place on `field`, through a scratch field of the same components.
template <typename T>
static int passive_step(int dim, int nz, int ny, int nx, int ncomp, void* field, void* scratch, const void* u,
                        double dt_by_dx, double k, cudaStream_t s) {
    if (dim == 2) {
        // one fused sweep (ENO3 on [2:-2]^2, then diffusion of the advected field on [1:-1]^2)
        SG_TRY(sweep_op<T>(ny, nx, field, scratch, u, nullptr, 0.0, dt_by_dx, k, SWEEP_ADVECT | SWEEP_DIFFUSE, s));
        return cuda_status(cudaMemcpyAsync(field, scratch, (size_t)ny * nx * sizeof(T), cudaMemcpyDeviceToDevice, s),
                           "passive step copy back");
    }
    SG_TRY(eno3_3d_launch<T>(nz, ny, nx, ncomp, field, nullptr, scratch, u, -dt_by_dx, 1, ncomp == 3, s));
    return diffusion3d_comps_launch<T>(nz, ny, nx, ncomp, scratch, field, k, s);
}

}  // namespace sg

extern "C" int sg_advection_eno3_step_3d(int dtype, int nz, int ny, int nx, int ncomp, const void* in, void* out,
                                         const void* velocity, double dt_by_dx, void* stream) {
    SG_TRY(check3d(nz, ny, nx, in, out));
    SG_REQUIRE(velocity, SG_ERR_INVALID_ARG, "null velocity");
    SG_REQUIRE(ncomp >= 1 && (int64_t)nz * ncomp <= 65535, SG_ERR_SHAPE, "eno3 3d: bad component count %d", ncomp);
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype,
                      eno3_3d_launch<float>(nz, ny, nx, ncomp, in, nullptr, out, velocity, -dt_by_dx, 1, ncomp == 3, s),
                      eno3_3d_launch<double>(nz, ny, nx, ncomp, in, nullptr, out, velocity, -dt_by_dx, 1, ncomp == 3,
                                             s));
}

extern "C" int sg_advection_eno3_flux_3d(int dtype, int nz, int ny, int nx, const void* field, void* flux,
                                         const void* velocity, double inv_dx, void* stream) {
    SG_TRY(check3d(nz, ny, nx, field, flux));
    SG_REQUIRE(velocity, SG_ERR_INVALID_ARG, "null velocity");
    SG_REQUIRE(nz <= 65535, SG_ERR_SHAPE, "eno3 3d: nz too large");
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, eno3_3d_launch<float>(nz, ny, nx, 1, field, flux, flux, velocity, inv_dx, 0, false, s),
                      eno3_3d_launch<double>(nz, ny, nx, 1, field, flux, flux, velocity, inv_dx, 0, false, s));
}

extern "C" int sg_passive_transport_step(int dtype, int dim, int nz, int ny, int nx, int ncomp, void* field,
                                         void* scratch, const void* velocity, double dt_by_dx, double nu_dt_by_dx2,
                                         void* stream) {
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "passive step: dim must be 2 or 3");
    SG_REQUIRE(velocity, SG_ERR_INVALID_ARG, "null velocity");
    if (dim == 2) {
        SG_REQUIRE(ncomp == 1, SG_ERR_UNSUPPORTED, "passive step: a 2D field is a scalar");
        SG_TRY(check2d(ny, nx, field, scratch));
    } else {
        SG_TRY(check3d(nz, ny, nx, field, scratch));
        SG_REQUIRE(ncomp == 1 || ncomp == 3, SG_ERR_INVALID_ARG, "passive step: 1 or 3 components");
    }
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype,
                      passive_step<float>(dim, nz, ny, nx, ncomp, field, scratch, velocity, dt_by_dx, nu_dt_by_dx2, s),
                      passive_step<double>(dim, nz, ny, nx, ncomp, field, scratch, velocity, dt_by_dx, nu_dt_by_dx2,
                                           s));
}

// ------------------------------------------------------ elementwise and flux-form operators
// The lower-level factories of elementwise_ops_{2,3}d.py, diffusion_flux_{2,3}d.py and
// advection_flux_2d.py, each one launch over contiguous arrays.
namespace sg {

enum { EW_SET = 0, EW_ADD_FIXED = 1, EW_COPY = 2, EW_SUM = 3, EW_SAXPBY = 4, EW_COMPLEX_PRODUCT = 5 };

template <typename T>
__global__ void __launch_bounds__(256) elementwise_kernel(int op, int64_t n, const T* a, const T* b, T* out, T alpha,
                                                          T beta) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    switch (op) {
        case EW_SET: out[i] = alpha; break;
        case EW_ADD_FIXED: out[i] = a[i] + alpha; break;
        case EW_COPY: out[i] = a[i]; break;
        case EW_SUM: out[i] = a[i] + b[i]; break;
        case EW_SAXPBY: out[i] = alpha * a[i] + beta * b[i]; break;
        default: {  // n interleaved complex values (real, imaginary)
            const T ar = a[2 * i], ai = a[2 * i + 1], br = b[2 * i], bi = b[2 * i + 1];
            out[2 * i] = ar * br - ai * bi;
            out[2 * i + 1] = ar * bi + ai * br;
        }
    }
}

// cells within `width` of any face of the grid (2D: nz = 1, no z faces) set to `value`
template <typename T>
__global__ void __launch_bounds__(256) boundary_zone_kernel(int dim, int nz, int ny, int nx, int width, T* f, T value) {
    const int x = blockIdx.x * kCell3X + threadIdx.x, y = blockIdx.y * kCell3Y + threadIdx.y, z = blockIdx.z;
    if (x >= nx || y >= ny) return;
    bool edge = x < width || x >= nx - width || y < width || y >= ny - width;
    if (dim == 3) edge = edge || z < width || z >= nz - width;
    if (edge) f[((int64_t)z * ny + y) * nx + x] = value;
}

// flux = k lap(field) on the interior [1:-1]; the ring is set to 0 when reset, else left as it is
template <typename T>
__global__ void __launch_bounds__(256) diffusion_flux_kernel(int dim, int nz, int ny, int nx, const T* f, T* flux, T k,
                                                             int reset) {
    const int x = blockIdx.x * kCell3X + threadIdx.x, y = blockIdx.y * kCell3Y + threadIdx.y, z = blockIdx.z;
    if (x >= nx || y >= ny) return;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    const int64_t g = (int64_t)z * sz + (int64_t)y * nx + x;
    const bool in = x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2 && (dim == 2 || (z >= 1 && z <= nz - 2));
    if (in) {
        if (dim == 2) {
            // diffusion_flux_2d.py:36-38 term order: y+1, y-1, x+1, x-1
            flux[g] = k * (f[g + sy] + f[g - sy] + f[g + 1] + f[g - 1] - T(4) * f[g]);
        } else {
            // diffusion_flux_3d.py:34-43 term order: z+1, z-1, y+1, y-1, x+1, x-1
            flux[g] = k * (f[g + sz] + f[g - sz] + f[g + sy] + f[g - sy] + f[g + 1] + f[g - 1] - T(6) * f[g]);
        }
    } else if (reset) {
        flux[g] = T(0);
    }
}

// flux += the four ENO3 face fluxes of a 2D scalar field on [2:-2]^2, in the passes' order
// (advection_flux_2d.py:28-128: x front, x back, y front, y back)
template <typename T>
__global__ void __launch_bounds__(256) eno3_2d_flux_kernel(int ny, int nx, const T* f, const T* u, T* flux, T inv_dx) {
    const int x = blockIdx.x * kCell3X + threadIdx.x, y = blockIdx.y * kCell3Y + threadIdx.y;
    if (x < 2 || y < 2 || x > nx - 3 || y > ny - 3) return;
    const int64_t n = (int64_t)ny * nx;
    const int64_t g = (int64_t)y * nx + x;
    T acc = flux[g];
#pragma unroll
    for (int axis = 0; axis < 2; ++axis) {
        const int64_t s = axis == 0 ? 1 : nx;
        const T* ua = u + axis * n;
        auto q = [&](int k) { return f[g + k * s] * ua[g + k * s]; };
        const T front = eno3_face(q(-1), q(0), q(1), q(2), ua[g], ua[g + s]);
        const T back = eno3_face(q(-2), q(-1), q(0), q(1), ua[g - s], ua[g]);
        acc = fma(inv_dx, front, acc);
        acc = fma(-inv_dx, back, acc);
    }
    flux[g] = acc;
}

template <typename T>
static int elementwise_op(int op, int64_t n, const void* a, const void* b, void* out, double alpha, double beta,
                          cudaStream_t s) {
    if (n == 0) return SG_OK;
    elementwise_kernel<T><<<ceil_div(n, 256), 256, 0, s>>>(op, n, (const T*)a, (const T*)b, (T*)out, (T)alpha,
                                                           (T)beta);
    return launch_status("elementwise");
}

}  // namespace sg

extern "C" int sg_elementwise(int dtype, int op, int64_t n, const void* a, const void* b, void* out, double alpha,
                              double beta, void* stream) {
    SG_REQUIRE(op >= EW_SET && op <= EW_COMPLEX_PRODUCT, SG_ERR_INVALID_ARG, "elementwise: bad op %d", op);
    SG_REQUIRE(n >= 0 && out, SG_ERR_INVALID_ARG, "elementwise: bad argument");
    SG_REQUIRE(op == EW_SET || a, SG_ERR_INVALID_ARG, "elementwise: null input");
    SG_REQUIRE((op != EW_SUM && op != EW_SAXPBY && op != EW_COMPLEX_PRODUCT) || b, SG_ERR_INVALID_ARG,
               "elementwise: null second input");
    auto s = (cudaStream_t)stream;
    SG_DTYPE_DISPATCH(dtype, elementwise_op<float>(op, n, a, b, out, alpha, beta, s),
                      elementwise_op<double>(op, n, a, b, out, alpha, beta, s));
}

extern "C" int sg_set_boundary_zone(int dtype, int dim, int nz, int ny, int nx, int width, void* field, double value,
                                    void* stream) {
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "boundary zone: dim must be 2 or 3");
    SG_REQUIRE(field && width > 0, SG_ERR_INVALID_ARG, "boundary zone: bad argument");
    if (dim == 2) nz = 1;
    SG_REQUIRE(nz >= 1 && ny >= 1 && nx >= 1, SG_ERR_SHAPE, "boundary zone: bad extent");
    auto s = (cudaStream_t)stream;
    const dim3 grid = cell3_grid(Grid3{nz, ny, nx});
    if (dtype == SG_F32)
        boundary_zone_kernel<float><<<grid, cell3_block(), 0, s>>>(dim, nz, ny, nx, width, (float*)field, (float)value);
    else {
        SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "boundary zone: bad dtype");
        boundary_zone_kernel<double><<<grid, cell3_block(), 0, s>>>(dim, nz, ny, nx, width, (double*)field, value);
    }
    return launch_status("boundary zone");
}

extern "C" int sg_diffusion_flux(int dtype, int dim, int nz, int ny, int nx, const void* field, void* flux, double k,
                                 int reset_ghost_zone, void* stream) {
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "diffusion flux: dim must be 2 or 3");
    if (dim == 2) nz = 1;
    SG_TRY(check3d(nz, ny, nx, field, flux));
    auto s = (cudaStream_t)stream;
    const dim3 grid = cell3_grid(Grid3{nz, ny, nx});
    if (dtype == SG_F32)
        diffusion_flux_kernel<float><<<grid, cell3_block(), 0, s>>>(dim, nz, ny, nx, (const float*)field, (float*)flux,
                                                                    (float)k, reset_ghost_zone);
    else {
        SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "diffusion flux: bad dtype");
        diffusion_flux_kernel<double><<<grid, cell3_block(), 0, s>>>(dim, nz, ny, nx, (const double*)field,
                                                                     (double*)flux, k, reset_ghost_zone);
    }
    return launch_status("diffusion flux");
}

extern "C" int sg_advection_eno3_flux_2d(int dtype, int ny, int nx, const void* field, void* flux, const void* velocity,
                                         double inv_dx, void* stream) {
    SG_TRY(check2d(ny, nx, field, flux));
    SG_REQUIRE(velocity, SG_ERR_INVALID_ARG, "null velocity");
    auto s = (cudaStream_t)stream;
    const dim3 grid = cell3_grid(Grid3{1, ny, nx});
    if (dtype == SG_F32)
        eno3_2d_flux_kernel<float><<<grid, cell3_block(), 0, s>>>(ny, nx, (const float*)field, (const float*)velocity,
                                                                  (float*)flux, (float)inv_dx);
    else {
        SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "eno3 2d flux: bad dtype");
        eno3_2d_flux_kernel<double><<<grid, cell3_block(), 0, s>>>(ny, nx, (const double*)field,
                                                                   (const double*)velocity, (double*)flux, inv_dx);
    }
    return launch_status("eno3 2d flux");
}
