// Flow-step plan and the fused 2D/3D time step of the unbounded vorticity
// Navier-Stokes simulators (navier_stokes_flow_simulators.py:171-209, 449-498).
//
// 2D step (5 kernels):  sweep (forcing curl + ENO3 + diffusion) -> Poisson load
//   (penalise, write vorticity back, zero forcing, x R2C) -> column convolution
//   -> x C2R -> curl + free stream + max|u|.
// 3D step: forcing curl -> u x w curl update -> diffusion [-> filter] ->
//   Poisson load (penalise, write back, zero forcing, x R2C, all 3 components)
//   -> y FFT -> z FFT * G * IFFT -> y IFFT -> x C2R -> curl + free stream + max.
#include <algorithm>
#include <cfloat>
#include <cstring>

#include "flow_plan.cuh"
#include "flow_load_reg.cuh"



namespace sg {

// Record timing event `i` of the armed set (no-op when none is armed).
// While `stream` is being captured the external flag makes the record a node of
// the graph (a plain record during capture only orders streams); outside capture
// the record is a plain one (the external flag is refused there).
static inline void mark(sg_flow_plan_s* p, int i, cudaStream_t stream) {
    if (i >= p->n_events || !p->events[i]) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(p->events[i], stream, cudaEventRecordExternal);
    else
        cudaEventRecord(p->events[i], stream);
}

static void flow_plan_free(sg_flow_plan_s* p) {
    if (!p) return;
    poisson_plan_free(p->poisson);
    cudaFree(p->scratch_a);
    cudaFree(p->scratch_b);
    cudaFree(p->filt_a);
    cudaFree(p->filt_b);
    cudaFree(p->coef_x);
    cudaFree(p->coef_y);
    cudaFree(p->coef_z);
    cudaFree(p->dev_block);
    cudaFreeHost(p->host_word);
    if (p->step_exec) cudaGraphExecDestroy(p->step_exec);
    if (p->capture_stream) cudaStreamDestroy(p->capture_stream);
    delete p;
}

static int alloc_into(void** dst, size_t bytes, int64_t* total, const char* what) {
    SG_TRY(cuda_status(cudaMalloc(dst, bytes), what));
    *total += (int64_t)bytes;
    return SG_OK;
}

static int upload_coef(void** dst, const void* host, int n, int esz, int64_t* total) {
    if (!host) return SG_OK;
    SG_TRY(alloc_into(dst, (size_t)n * esz, total, "penalisation table alloc"));
    return cuda_status(cudaMemcpy(*dst, host, (size_t)n * esz, cudaMemcpyHostToDevice), "penalisation upload");
}

// ---------------------------------------------------------------- launchers
template <typename T>
int launch_sweep2d(const Sweep2DParams<T>& p, cudaStream_t stream) {
    constexpr int TX = 32;
    constexpr int TY = sizeof(T) == 4 ? 16 : 8;
    dim3 grid(ceil_div(p.nx, TX), ceil_div(p.ny, TY));
    sweep2d_kernel<T, TX, TY><<<grid, dim3(TX, 8), 0, stream>>>(p);
    return launch_status("sweep2d");
}

template <typename T, int N, int W>
int launch_fast_flow_load(const FlowLoadParams<T>& p, cudaStream_t stream) {
    constexpr int E = FastPickRows<N, W>::E;
    const size_t smem = FlowLoadSmem<N, W>::template bytes<T>();
    auto kern = fast_flow_load_kernel<T, N, W, E>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "fast flow_load smem attribute"));
    SG_TRY(fast_max_carveout(kern, "fast flow_load carveout attribute"));
    kern<<<ceil_div(p.n_rows, W), FastShape<N, W, E>::NT, smem, stream>>>(p);
    return launch_status("fast flow_load");
}

template <typename T>
int launch_flow_load(FlowLoadParams<T> p, cudaStream_t stream) {
    // 3D fp32 rows of 256 reals: the register load pass (flow_load_reg.cuh)
    if constexpr (sizeof(T) == 4)
        if (p.dim == 3 && p.nx == rl::kRowM && p.st.n == rl::kRowM) return launch_reg_flow_load(p, stream);
#define SG_CALL(NN, WW) launch_fast_flow_load<T, NN, WW>(p, stream)
    SG_FAST_DISPATCH(p.st.n, p.n_rows, SG_CALL)
#undef SG_CALL
    const int esz = sizeof(cplx_t<T>);
    const int rb = rows_per_block_for(p.st.n, esz);
    const size_t smem = 2ull * rb * p.st.n * esz;
    auto kern = flow_load_kernel<T>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "flow_load smem attribute"));
    kern<<<ceil_div(p.n_rows, rb), dim3(256 / rb, rb), smem, stream>>>(p);
    return launch_status("flow_load");
}

template <typename T>
int launch_curl2d(const Curl2DParams<T>& p, cudaStream_t stream) {
    dim3 block(32, 8);
    dim3 grid(ceil_div(p.nx, 32), ceil_div(p.ny, 8));
    curl2d_kernel<T><<<grid, block, 0, stream>>>(p);
    return launch_status("curl2d");
}

template <typename T>
int launch_curl3d(const Curl3DParams<T>& p, int64_t n, cudaStream_t stream) {
    curl3d_kernel<T><<<cell3_grid(p.grid), cell3_block(), 0, stream>>>(p);
    return launch_status("curl3d");
}

template <typename T>
int filter3d(Grid3 G, T* field, int filter_type, int order, T* a, T* b, cudaStream_t stream) {
    if (filter_type == 0 || order <= 0) return SG_OK;
    const int64_t n = (int64_t)G.nz * G.ny * G.nx;
    const unsigned blocks = ceil_div(n, 256);
    for (int c = 0; c < 3; ++c) {
        T* phi = field + c * n;
        if (filter_type == 1) {
            // multiplicative: (Lz Ly Lx)^order phi, subtracted once
            const T* src = phi;
            T* bufs[2] = {a, b};
            int which = 0;
            for (int it = 0; it < order; ++it) {
                for (int axis = 0; axis < 3; ++axis) {
                    T* dst = bufs[which];
                    filter_pass3d_kernel<T><<<cell3_grid(G), cell3_block(), 0, stream>>>(G, src, dst, axis);
                    src = dst;
                    which ^= 1;
                }
            }
            subtract_kernel<T><<<blocks, 256, 0, stream>>>(n, phi, src);
        } else {
            // convolution: per axis, L_axis^order phi subtracted before the next axis
            for (int axis = 0; axis < 3; ++axis) {
                const T* src = phi;
                T* bufs[2] = {a, b};
                int which = 0;
                for (int it = 0; it < order; ++it) {
                    T* dst = bufs[which];
                    filter_pass3d_kernel<T><<<cell3_grid(G), cell3_block(), 0, stream>>>(G, src, dst, axis);
                    src = dst;
                    which ^= 1;
                }
                subtract_kernel<T><<<blocks, 256, 0, stream>>>(n, phi, src);
            }
        }
    }
    return launch_status("laplacian filter");
}

template int filter3d<float>(Grid3, float*, int, int, float*, float*, cudaStream_t);
template int filter3d<double>(Grid3, double*, int, int, double*, double*, cudaStream_t);

template <typename T>
static FlowLoadParams<T> load_params(sg_flow_plan_s* p, const T* src, T* dst, T* forcing) {
    sg_poisson_plan_s* pp = p->poisson;
    FlowLoadParams<T> l{};
    l.dim = p->dim;
    l.nz = p->nz;
    l.ny = p->ny;
    l.nx = p->nx;
    l.width = p->width;
    l.src = src;
    l.dst = dst;
    l.forcing = forcing;
    l.zero_ncomp = 1;
    l.cx = (const T*)p->coef_x;
    l.cy = (const T*)p->coef_y;
    l.cz = (const T*)p->coef_z;
    l.comp_stride = p->cells();
    l.spec = reinterpret_cast<cplx_t<T>*>(pp->spec);
    if (p->dim == 2) {
        l.spec_map = row_map(p->ny, p->nx + 1, 1, 0, pp->spec_comp_elems);
        l.n_rows = p->ny;
    } else {
        l.spec_map = row_map(p->ny, p->nx + 1, p->nz, (int64_t)2 * p->ny * (p->nx + 1), pp->spec_comp_elems);
        l.n_rows = 3 * p->nz * p->ny;
    }
    l.st = pp->st_x;
    l.tw_m = (const cplx_t<T>*)pp->tw_x;
    l.tw_l = (const cplx_t<T>*)pp->tw_xl;
    return l;
}

template <typename T>
int flow_step_2d(sg_flow_plan_s* p, T* w, T* u, T* f, T* psi, const ScalarSrc& sc, bool free_stream,
                 cudaStream_t stream) {
    Sweep2DParams<T> s{};
    s.ny = p->ny;
    s.nx = p->nx;
    s.w = w;
    s.u = u;
    s.f = f;
    s.out = (T*)p->scratch_a;
    s.sc = sc;
    s.flags = SWEEP_ADVECT | SWEEP_DIFFUSE;
    s.tape_w1 = (T*)p->tape_w1;
    s.tape_w2 = (T*)p->tape_w2;
    mark(p, 0, stream);
    SG_TRY(launch_sweep2d<T>(s, stream));
    mark(p, 1, stream);
    FlowLoadParams<T> l = load_params<T>(p, (const T*)p->scratch_a, w, f);
    l.zero_ncomp = 2;  // one vorticity row zeroes the row of both forcing components
    SG_TRY(launch_flow_load<T>(l, stream));
    mark(p, 2, stream);
    SG_TRY(poisson_spectral_passes<T>(p->poisson, 1, stream));
    mark(p, 3, stream);
    SG_TRY(poisson_store_rows<T>(p->poisson, psi, 1, 0, stream));
    mark(p, 4, stream);
    SG_TRY(cuda_status(cudaMemsetAsync(p->umax_slot(), 0, 8, stream), "umax reset"));
    Curl2DParams<T> c{};
    c.ny = p->ny;
    c.nx = p->nx;
    c.psi = psi;
    c.u = u;
    c.prefactor = T(0.5) / (T)p->dx;
    c.sc = sc;
    c.add_free_stream = free_stream;
    c.umax = (T*)p->umax_slot();
    SG_TRY(launch_curl2d<T>(c, stream));
    mark(p, 5, stream);
    return SG_OK;
}

// The three spectral passes of the 3D solve with timing marks 5 and 6 between them.
template <typename T>
int poisson_spectral_passes_marked(sg_flow_plan_s* p, int ncomp, cudaStream_t stream) {
    SG_TRY(poisson_spectral_pass3d<T>(p->poisson, ncomp, 0, stream));
    mark(p, 3, stream);
    SG_TRY(poisson_spectral_pass3d<T>(p->poisson, ncomp, 1, stream));
    mark(p, 4, stream);
    return poisson_spectral_pass3d<T>(p->poisson, ncomp, 2, stream);
}

template <typename T>
int flow_step_3d(sg_flow_plan_s* p, T* w, T* u, T* f, T* psi, const ScalarSrc& sc, bool free_stream,
                 cudaStream_t stream) {
    const int64_t n = p->cells();
    Grid3 G{p->nz, p->ny, p->nx};
    T* A = (T*)p->scratch_a;
    T* B = (T*)p->scratch_b;
    // timing marks: 0 forcing curl, u x w update, diffusion (+ filter) 1 Poisson load 2 y FFT 3 z conv
    // 4 y IFFT 5 x C2R 6 curl 7
    mark(p, 0, stream);
    const T* w1 = w;
    if (f) {
        if (sizeof(T) == 4 && forcing_curl_tma_ok(G, w, f, A)) {
            SG_TRY(launch_forcing_curl_tma(G, (const float*)w, (const float*)f, (float*)A, sc, p->kernel_status(),
                                           stream));
        } else {
            Stencil3DParams<T> s{};
            s.grid = G;
            s.a = w;
            s.b = f;
            s.out = A;
            s.sc = sc;
            s.mode = 0;
            forcing_curl3d_kernel<T><<<cell3_grid(G), cell3_block(), 0, stream>>>(s);
            SG_TRY(launch_status("forcing_curl3d"));
        }
        w1 = A;
    }
    if (sizeof(T) == 4 && rot_update_tma_ok(G, w1, u, B)) {
        SG_TRY(launch_rot_update_tma(G, (const float*)w1, (const float*)u, (float*)B, sc, p->kernel_status(), stream));
    } else {
        Stencil3DParams<T> s{};
        s.grid = G;
        s.a = w1;
        s.b = u;
        s.out = B;
        s.sc = sc;
        rotational_update3d_kernel<T><<<cell3_grid(G), cell3_block(), 0, stream>>>(s);
        SG_TRY(launch_status("rotational_update3d"));
    }
    if (sizeof(T) == 4 && diffusion_tma_ok(G, 3, B, A)) {
        SG_TRY(launch_diffusion_tma(G, 3, (const float*)B, (float*)A, sc, p->kernel_status(), stream));
    } else {
        Stencil3DParams<T> s{};
        s.grid = G;
        s.a = B;
        s.out = A;
        s.sc = sc;
        s.mode = 0;
        diffusion3d_kernel<T><<<cell3_grid(G), cell3_block(), 0, stream>>>(s);
        SG_TRY(launch_status("diffusion3d"));
    }
    SG_TRY(filter3d<T>(G, A, p->filter_type, p->filter_order, (T*)p->filt_a, (T*)p->filt_b, stream));
    mark(p, 1, stream);
    FlowLoadParams<T> l = load_params<T>(p, A, w, f);
    SG_TRY(launch_flow_load<T>(l, stream));
    mark(p, 2, stream);
    SG_TRY(poisson_spectral_passes_marked<T>(p, 3, stream));
    mark(p, 5, stream);
    SG_TRY(poisson_store_rows<T>(p->poisson, psi, 3, n, stream));
    mark(p, 6, stream);
    SG_TRY(cuda_status(cudaMemsetAsync(p->umax_slot(), 0, 8, stream), "umax reset"));
    Curl3DParams<T> c{};
    c.grid = G;
    c.psi = psi;
    c.u = u;
    c.prefactor = T(0.5) / (T)p->dx;
    c.sc = sc;
    c.add_free_stream = free_stream;
    c.umax = (T*)p->umax_slot();
    if (sizeof(T) == 4 && velocity_curl_tma_ok(G, psi, u))
        SG_TRY(launch_velocity_curl_tma(G, (const float*)psi, (float*)u, (float)c.prefactor, sc, free_stream,
                                        (float*)c.umax, p->kernel_status(), stream));
    else
        SG_TRY(launch_curl3d<T>(c, n, stream));
    mark(p, 7, stream);
    return SG_OK;
}

// max over cells of sum_d |v_d| into a field-typed slot (atomic, order free)
template <typename T>
__global__ void __launch_bounds__(256) max_abs_sum_kernel(int64_t n, int dim, const T* v, T* slot) {
    T m = T(0);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        T s = fabs(v[i]);
        for (int d = 1; d < dim; ++d) s = s + fabs(v[d * n + i]);
        m = fmax(m, s);
    }
    m = block_max(m);
    if (threadIdx.x == 0) atomic_max_nonneg(slot, m);
}

template <typename T>
int launch_max_abs_sum(int64_t n, int dim, const T* v, T* slot, cudaStream_t stream) {
    SG_TRY(cuda_status(cudaMemsetAsync(slot, 0, sizeof(T), stream), "max slot reset"));
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n, 256), 152 * 8);
    max_abs_sum_kernel<T><<<blocks, 256, 0, stream>>>(n, dim, v, slot);
    return launch_status("max_abs_sum");
}

template <typename T>
__global__ void slot_to_double_kernel(const T* slot, double* out) {
    *out = (double)*slot;
}

// compute_advection_diffusion_stable_timestep (passive_transport_flow_simulators.
// py:139-155) evaluated in the field precision with numpy's promotion rules:
// Python scalars take the field type, so every operation rounds to T.
template <typename T>
__global__ void device_dt_kernel(const T* umax_slot, sg_step_scalars* sc, double* time, int dim, T dx, double cfl,
                                 double nu, double rho, double dt_prefac, double fs0, double fs1, double fs2) {
    const T eps = sizeof(T) == 4 ? (T)FLT_EPSILON : (T)DBL_EPSILON;
    const T tol = T(10) * eps;
    const T umax = *umax_slot;
    const T a = (T)cfl * dx / (umax + tol);
    const T b = (T)0.9 * (dx * dx) / (T)(2 * dim) / (T)nu + tol;
    T dt = b < a ? b : a;
    dt = dt * (T)dt_prefac;
    sc->dt = (double)dt;
    T d2 = T(2) * dx;
    d2 = d2 * (T)rho;
    sc->forcing_prefac = (double)(dt / d2);
    sc->advection_prefac = dim == 2 ? (double)(dt / dx) : (double)(dt / (T(2) * dx));
    const T nudt = (T)nu * dt;
    sc->diffusion_prefac = (double)(nudt / dx / dx);
    sc->free_stream[0] = fs0;
    sc->free_stream[1] = fs1;
    sc->free_stream[2] = fs2;
    *time += (double)dt;
}

template <typename T>
int device_dt(sg_flow_plan_s* p, const void* velocity, double cfl, double nu, double rho, double prefac,
              const double* fs, cudaStream_t stream) {
    if (velocity)
        SG_TRY(launch_max_abs_sum<T>(p->cells(), p->dim, (const T*)velocity, (T*)p->umax_slot(), stream));
    device_dt_kernel<T><<<1, 1, 0, stream>>>((const T*)p->umax_slot(), p->dev_scalars(), p->time_slot(), p->dim,
                                             (T)p->dx, cfl, nu, rho, prefac, fs ? fs[0] : 0.0, fs ? fs[1] : 0.0,
                                             fs ? fs[2] : 0.0);
    return launch_status("device_dt");
}

}  // namespace sg

using namespace sg;

extern "C" int sg_flow_plan_create(int dim, int nz, int ny, int nx, double x_range, int dtype, int width,
                                   const void* cx, const void* cy, const void* cz, int filter_type,
                                   int filter_order, sg_flow_plan* out) {
    SG_REQUIRE(out != nullptr, SG_ERR_INVALID_ARG, "flow plan: null output pointer");
    *out = nullptr;
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "flow plan: dim must be 2 or 3");
    SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, SG_ERR_INVALID_ARG, "flow plan: bad dtype");
    if (dim == 2) nz = 1;
    SG_REQUIRE(nx >= 6 && ny >= 6 && (dim == 2 || nz >= 6), SG_ERR_SHAPE,
               "flow plan: each extent must be >= 6 (got %d, %d, %d)", nz, ny, nx);
    SG_REQUIRE(width >= 0 && 2 * width <= nx && 2 * width <= ny && (dim == 2 || 2 * width <= nz), SG_ERR_SHAPE,
               "flow plan: penalty width %d does not fit the grid", width);
    SG_REQUIRE(width == 0 || (cx && cy && (dim == 2 || cz)), SG_ERR_INVALID_ARG,
               "flow plan: penalisation tables required for width > 0");
    SG_REQUIRE(filter_type >= 0 && filter_type <= 2 && filter_order >= 0, SG_ERR_INVALID_ARG,
               "flow plan: bad filter setting");
    SG_REQUIRE(dim == 3 || filter_type == 0, SG_ERR_INVALID_ARG, "flow plan: the filter is 3D only");
    auto* p = new sg_flow_plan_s();
    p->dim = dim;
    p->nz = nz;
    p->ny = ny;
    p->nx = nx;
    p->dtype = dtype;
    p->width = width;
    p->filter_type = filter_type;
    p->filter_order = filter_order;
    p->x_range = x_range;
    p->dx = dtype == SG_F32 ? (double)(float)(x_range / nx) : x_range / nx;
    const int esz = dtype_size(dtype);
    const int64_t n = p->cells();
    int st = SG_OK;
    do {
        if ((st = poisson_plan_create_impl(dim, nz, ny, nx, x_range, dtype, dim == 3 ? 3 : 1, &p->poisson))) break;
        p->bytes += p->poisson->bytes;
        if ((st = alloc_into(&p->scratch_a, (size_t)dim * n * esz, &p->bytes, "flow scratch alloc"))) break;
        if (dim == 3 && (st = alloc_into(&p->scratch_b, (size_t)3 * n * esz, &p->bytes, "flow scratch alloc"))) break;
        if (filter_type != 0) {
            if ((st = alloc_into(&p->filt_a, (size_t)n * esz, &p->bytes, "filter scratch alloc"))) break;
            if ((st = alloc_into(&p->filt_b, (size_t)n * esz, &p->bytes, "filter scratch alloc"))) break;
        }
        if (width > 0) {
            if ((st = upload_coef(&p->coef_x, cx, nx, esz, &p->bytes))) break;
            if ((st = upload_coef(&p->coef_y, cy, ny, esz, &p->bytes))) break;
            if (dim == 3 && (st = upload_coef(&p->coef_z, cz, nz, esz, &p->bytes))) break;
        }
        if ((st = alloc_into((void**)&p->dev_block, 128, &p->bytes, "flow device block alloc"))) break;
        if ((st = cuda_status(cudaMemset(p->dev_block, 0, 128), "flow device block init"))) break;
        if ((st = cuda_status(cudaMallocHost(&p->host_word, 16), "flow pinned word alloc"))) break;
        st = cuda_status(cudaDeviceSynchronize(), "flow plan create");
    } while (0);
    if (st != SG_OK) {
        flow_plan_free(p);
        return st;
    }
    *out = p;
    return SG_OK;
}

extern "C" int sg_flow_set_timing_events(sg_flow_plan p, int n_events, void* const* events) {
    SG_REQUIRE(p && n_events >= 0 && n_events <= 16 && (n_events == 0 || events), SG_ERR_INVALID_ARG,
               "timing events: bad argument");
    p->n_events = n_events;
    for (int i = 0; i < 16; ++i) p->events[i] = i < n_events ? (cudaEvent_t)events[i] : nullptr;
    return SG_OK;
}

extern "C" int sg_flow_set_tape(sg_flow_plan p, void* w_after_forcing, void* w_after_advection) {
    SG_REQUIRE(p, SG_ERR_INVALID_ARG, "tape: null plan");
    SG_REQUIRE(p->dim == 2, SG_ERR_UNSUPPORTED, "tape: only the 2D step records a tape");
    SG_REQUIRE((w_after_forcing == nullptr) == (w_after_advection == nullptr), SG_ERR_INVALID_ARG,
               "tape: give both buffers or neither");
    p->tape_w1 = w_after_forcing;
    p->tape_w2 = w_after_advection;
    return SG_OK;
}

extern "C" int sg_flow_prime_max(sg_flow_plan p, const void* velocity, void* stream_) {
    SG_REQUIRE(p && velocity, SG_ERR_INVALID_ARG, "prime max: null argument");
    auto stream = (cudaStream_t)stream_;
    if (p->dtype == SG_F32)
        return launch_max_abs_sum<float>(p->cells(), p->dim, (const float*)velocity, (float*)p->umax_slot(), stream);
    return launch_max_abs_sum<double>(p->cells(), p->dim, (const double*)velocity, (double*)p->umax_slot(), stream);
}

extern "C" int sg_flow_host_max(sg_flow_plan p, const void* velocity, double* host_out, void* stream_) {
    SG_REQUIRE(p && velocity && host_out, SG_ERR_INVALID_ARG, "host max: null argument");
    auto stream = (cudaStream_t)stream_;
    const size_t esz = p->dtype == SG_F32 ? sizeof(float) : sizeof(double);
    if (p->dtype == SG_F32)
        SG_TRY(launch_max_abs_sum<float>(p->cells(), p->dim, (const float*)velocity, (float*)p->umax_slot(), stream));
    else
        SG_TRY(launch_max_abs_sum<double>(p->cells(), p->dim, (const double*)velocity, (double*)p->umax_slot(),
                                          stream));
    SG_TRY(cuda_status(cudaMemcpyAsync(p->host_word, p->umax_slot(), esz, cudaMemcpyDeviceToHost, stream),
                       "host max copy"));
    SG_TRY(cuda_status(cudaStreamSynchronize(stream), "host max sync"));
    *host_out = p->dtype == SG_F32 ? (double)*(const float*)p->host_word : *(const double*)p->host_word;
    return SG_OK;
}

extern "C" int sg_flow_read_device_time(sg_flow_plan p, double* host_out) {
    SG_REQUIRE(p && host_out, SG_ERR_INVALID_ARG, "read device time: null argument");
    return cuda_status(cudaMemcpy(host_out, p->time_slot(), sizeof(double), cudaMemcpyDeviceToHost),
                       "read device time");
}

extern "C" int sg_flow_kernel_status(sg_flow_plan p, int32_t* host_out) {
    SG_REQUIRE(p && host_out, SG_ERR_INVALID_ARG, "kernel status: null argument");
    return cuda_status(cudaMemcpy(host_out, p->kernel_status(), sizeof(int32_t), cudaMemcpyDeviceToHost),
                       "read kernel status");
}

extern "C" int sg_event_record(void* event, void* stream_) {
    SG_REQUIRE(event, SG_ERR_INVALID_ARG, "event record: null event");
    auto stream = (cudaStream_t)stream_;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e;
    if (cudaStreamIsCapturing(stream, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
        e = cudaEventRecordWithFlags((cudaEvent_t)event, stream, cudaEventRecordExternal);
    else
        e = cudaEventRecord((cudaEvent_t)event, stream);
    return cuda_status(e, "event record");
}

extern "C" int sg_flow_device_time_slot(sg_flow_plan p, const double** slot_out) {
    SG_REQUIRE(p && slot_out, SG_ERR_INVALID_ARG, "device time slot: null argument");
    *slot_out = p->time_slot();
    return SG_OK;
}

extern "C" int sg_flow_plan_destroy(sg_flow_plan p) {
    flow_plan_free(p);
    return SG_OK;
}

extern "C" int64_t sg_flow_plan_bytes(sg_flow_plan p) { return p ? p->bytes : 0; }

static int flow_step_dispatch(sg_flow_plan_s* p, void* w, void* u, void* f, void* psi, const ScalarSrc& sc, bool fs,
                              cudaStream_t stream) {
    if (p->dtype == SG_F32)
        return p->dim == 2 ? flow_step_2d<float>(p, (float*)w, (float*)u, (float*)f, (float*)psi, sc, fs, stream)
                           : flow_step_3d<float>(p, (float*)w, (float*)u, (float*)f, (float*)psi, sc, fs, stream);
    return p->dim == 2 ? flow_step_2d<double>(p, (double*)w, (double*)u, (double*)f, (double*)psi, sc, fs, stream)
                       : flow_step_3d<double>(p, (double*)w, (double*)u, (double*)f, (double*)psi, sc, fs, stream);
}

__global__ void set_step_scalars_kernel(sg_step_scalars v, sg_step_scalars* dst) { *dst = v; }

static void flow_graph_disable(sg_flow_plan_s* p) {
    cudaGetLastError();  // a failed capture leaves no sticky error: the direct launches follow
    p->graph_disabled = true;
    if (p->step_exec) cudaGraphExecDestroy(p->step_exec);
    p->step_exec = nullptr;
}

// The host-scalar step as one graph replay (2 launches instead of 6 to 10).  The graph is the
// device-scalar form of the same step, so every kernel gets the same scalars and pointers as a direct
// launch.  *used = false leaves the step to the direct launches (caller stream being captured,
// graphs disabled, capture failed).
static int flow_step_graph(sg_flow_plan_s* p, void* w, void* u, void* f, void* psi, const sg_step_scalars& host,
                           bool fs, cudaStream_t stream, bool* used) {
    *used = false;
    if (p->graph_disabled) return SG_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess) {
        cudaGetLastError();
        return SG_OK;
    }
    if (cs != cudaStreamCaptureStatusNone) return SG_OK;
    const bool match = p->step_exec && p->graph_fields[0] == w && p->graph_fields[1] == u &&
                       p->graph_fields[2] == f && p->graph_fields[3] == psi && p->graph_free_stream == fs;
    if (!match) {
        if (p->graph_builds >= 8) {  // fields that keep moving: direct launches from now on
            flow_graph_disable(p);
            return SG_OK;
        }
        ++p->graph_builds;
        if (p->step_exec) cudaGraphExecDestroy(p->step_exec);
        p->step_exec = nullptr;
        if (!p->capture_stream && cudaStreamCreateWithFlags(&p->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
            p->capture_stream = nullptr;
            flow_graph_disable(p);
            return SG_OK;
        }
        if (cudaStreamBeginCapture(p->capture_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            flow_graph_disable(p);
            return SG_OK;
        }
        ScalarSrc dsc{};
        dsc.dev = p->dev_scalars();
        const int st = flow_step_dispatch(p, w, u, f, psi, dsc, fs, p->capture_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(p->capture_stream, &g);
        if (st != SG_OK || e != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            flow_graph_disable(p);
            return SG_OK;
        }
        const cudaError_t ei = cudaGraphInstantiate(&p->step_exec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            p->step_exec = nullptr;
            flow_graph_disable(p);
            return SG_OK;
        }
        p->graph_fields[0] = w;
        p->graph_fields[1] = u;
        p->graph_fields[2] = f;
        p->graph_fields[3] = psi;
        p->graph_free_stream = fs;
    }
    set_step_scalars_kernel<<<1, 1, 0, stream>>>(host, p->dev_scalars());
    SG_TRY(launch_status("flow step scalars"));
    SG_TRY(cuda_status(cudaGraphLaunch(p->step_exec, stream), "flow step graph launch"));
    *used = true;
    return SG_OK;
}

extern "C" int sg_flow_step(sg_flow_plan p, void* w, void* u, void* f, void* psi, const sg_step_scalars* scalars,
                            const sg_step_scalars* dev_scalars, void* stream_) {
    SG_REQUIRE(p && w && u && psi, SG_ERR_INVALID_ARG, "flow step: null argument");
    SG_REQUIRE(scalars || dev_scalars, SG_ERR_INVALID_ARG, "flow step: no step scalars");
    ScalarSrc sc{};
    if (scalars) sc.host = *scalars;
    sc.dev = dev_scalars;
    const bool fs = dev_scalars != nullptr || (scalars && (scalars->free_stream[0] != 0.0 ||
                                                          scalars->free_stream[1] != 0.0 ||
                                                          scalars->free_stream[2] != 0.0));
    auto stream = (cudaStream_t)stream_;
    int st = SG_OK;
    bool done = false;
    if (!dev_scalars && p->n_events == 0 && !p->tape_w1)
        st = flow_step_graph(p, w, u, f, psi, *scalars, fs, stream, &done);
    if (st == SG_OK && !done) st = flow_step_dispatch(p, w, u, f, psi, sc, fs, stream);
    p->n_events = 0;  // timing events and the tape are armed for one step only
    p->tape_w1 = p->tape_w2 = nullptr;
    return st;
}

extern "C" int sg_max_abs_sum(int dtype, int dim, int64_t n, const void* v, double* out, void* stream_) {
    SG_REQUIRE(v && out && n > 0 && dim >= 1 && dim <= 3, SG_ERR_INVALID_ARG, "max_abs_sum: bad argument");
    auto stream = (cudaStream_t)stream_;
    if (dtype == SG_F32) {
        float* slot = reinterpret_cast<float*>(out);
        SG_TRY(launch_max_abs_sum<float>(n, dim, (const float*)v, slot, stream));
        slot_to_double_kernel<float><<<1, 1, 0, stream>>>(slot, out);
        return launch_status("max_abs_sum finalize");
    }
    SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "max_abs_sum: bad dtype");
    return launch_max_abs_sum<double>(n, dim, (const double*)v, reinterpret_cast<double*>(out), stream);
}

extern "C" int sg_flow_device_dt(sg_flow_plan p, const void* velocity, double cfl, double nu, double rho,
                                 double dt_prefac, const double* free_stream, const sg_step_scalars** dev_out,
                                 void* stream_) {
    SG_REQUIRE(p, SG_ERR_INVALID_ARG, "device dt: null plan");
    auto stream = (cudaStream_t)stream_;
    int st = p->dtype == SG_F32 ? device_dt<float>(p, velocity, cfl, nu, rho, dt_prefac, free_stream, stream)
                                : device_dt<double>(p, velocity, cfl, nu, rho, dt_prefac, free_stream, stream);
    if (dev_out) *dev_out = p->dev_scalars();
    return st;
}

namespace sg {
template int launch_sweep2d<float>(const Sweep2DParams<float>&, cudaStream_t);
template int launch_sweep2d<double>(const Sweep2DParams<double>&, cudaStream_t);
template int launch_curl2d<float>(const Curl2DParams<float>&, cudaStream_t);
template int launch_curl2d<double>(const Curl2DParams<double>&, cudaStream_t);
}  // namespace sg
