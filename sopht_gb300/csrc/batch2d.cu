// Batched 2D flow step: many independent 2D instances of uneven grid size and
// Reynolds number advanced together, one persistent launch per fused operator.
//
// Each instance is a regular flow plan (its own Poisson workspace, Green's
// table, scratch, device step scalars) plus one virtual-boundary interactor.
// A device table holds every instance's kernel parameters; for each operator a
// prefix sum over instances of that operator's work items (tiles, row chunks,
// line chunks, marker groups) lets a block map a work index to its instance by
// binary search.  Blocks loop over work items with a grid stride, so one launch
// covers the whole batch whatever the mix of sizes.
//
// Step (8 launches for the whole batch):
//   stable dt per instance -> IB interaction (xi step first) -> spreading ->
//   sweep (forcing curl + ENO3 + diffusion) -> Poisson load (penalise, write
//   back, zero forcing, x R2C) -> column convolution -> x C2R -> curl + U_inf
//   + max|u|.
// The FFT passes dispatch on each instance's length to the size-specialised
// bodies with a common 256-thread block: N = 256 (16 lines), 512 (8), 768 (8),
// 1024 (4).
#include <algorithm>
#include <cfloat>
#include <vector>

#include "flow_plan.cuh"
#include "ib.cuh"

namespace sg {

enum { BK_IB = 0, BK_SPREAD, BK_SWEEP, BK_LOAD, BK_CONV, BK_C2R, BK_CURL, BK_SWEEP8, BK_COUNT };

struct BatchDt {
    float* umax;
    sg_step_scalars* sc;
    double* time;
    float dx;
    double cfl, nu, rho, dt_prefac, fs0, fs1;
};

struct BatchInst {
    int ny, nx, sweep_tiles_x, curl_tiles_x, n_lag;
    Sweep2DParams<float> sweep;
    FlowLoadParams<float> load;
    LinesParams<float> conv;
    RowsC2RParams<float> c2r;
    Curl2DParams<float> curl;
    IBParams<float> ib;
    SpreadParams<float> spread;
    BatchDt dt;
};

__device__ __forceinline__ int batch_find(const int* off, int n, int w) {
    int lo = 0, hi = n;  // off[lo] <= w < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= w) lo = mid;
        else hi = mid;
    }
    return lo;
}

// compute_advection_diffusion_stable_timestep in float (numpy float32
// promotion), then the step prefactors; the max slot is reset for this step.
__global__ void batch_dt_kernel(BatchInst* insts, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BatchDt& d = insts[i].dt;
    const float tol = 10.0f * FLT_EPSILON;
    const float dx = d.dx;
    const float umax = *d.umax;
    const float a = (float)d.cfl * dx / (umax + tol);
    const float b = 0.9f * (dx * dx) / 4.0f / (float)d.nu + tol;
    float dt = b < a ? b : a;
    dt = dt * (float)d.dt_prefac;
    float d2 = 2.0f * dx;
    d2 = d2 * (float)d.rho;
    d.sc->dt = dt;
    d.sc->forcing_prefac = dt / d2;
    d.sc->advection_prefac = dt / dx;
    const float nudt = (float)d.nu * dt;
    d.sc->diffusion_prefac = nudt / dx / dx;
    d.sc->free_stream[0] = d.fs0;
    d.sc->free_stream[1] = d.fs1;
    d.sc->free_stream[2] = 0.0;
    *d.time += (double)dt;
    *d.umax = 0.0f;
}

__global__ void __launch_bounds__(256) batch_ib_kernel(const BatchInst* insts, const int* off, int n, int total) {
    const int* o = off + BK_IB * (n + 1);
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int i = batch_find(o, n, w);
        const int marker = (w - o[i]) * 8 + (threadIdx.x >> 5);
        if (marker < insts[i].n_lag) ib_interaction_body<float>(insts[i].ib, marker);
    }
}

__global__ void __launch_bounds__(256) batch_spread_kernel(const BatchInst* insts, const int* off, int n,
                                                           int total) {
    const int* o = off + BK_SPREAD * (n + 1);
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int i = batch_find(o, n, w);
        const int64_t t = (int64_t)(w - o[i]) * 256 + threadIdx.x;
        if (t < (int64_t)insts[i].n_lag * 16) ib_spread_body<float>(insts[i].spread, t);
    }
}

template <int TY>
__global__ void __launch_bounds__(256) batch_sweep_kernel(const BatchInst* insts, const int* off, int n,
                                                          int total) {
    const int* o = off + (TY == 16 ? BK_SWEEP : BK_SWEEP8) * (n + 1);
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int i = batch_find(o, n, w);
        const int local = w - o[i];
        const int tx = insts[i].sweep_tiles_x;
        sweep2d_body<float, 32, TY>(insts[i].sweep, local % tx, local / tx);
        __syncthreads();
    }
}

#define SG_BATCH_SIZES(CALL) \
    CALL(256, 16)            \
    CALL(512, 8)             \
    CALL(768, 8)             \
    CALL(1024, 4)

__global__ void __launch_bounds__(256) batch_load_kernel(const BatchInst* insts, const int* off, int n, int total) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int* o = off + BK_LOAD * (n + 1);
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int i = batch_find(o, n, w);
        const int local = w - o[i];
        switch (insts[i].nx) {
#define SG_CASE(NN, WW) \
    case NN: fast_flow_load_body<float, NN, WW>(insts[i].load, local, smem_raw); break;
            SG_BATCH_SIZES(SG_CASE)
#undef SG_CASE
            default: break;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) batch_conv_kernel(const BatchInst* insts, const int* off, int n, int total) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int* o = off + BK_CONV * (n + 1);
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int i = batch_find(o, n, w);
        const int local = w - o[i];
        switch (2 * insts[i].ny) {
#define SG_CASE(NN, WW) \
    case NN: fast_lines_body<float, NN, WW, LINE_CONV>(insts[i].conv, local, smem_raw); break;
            SG_BATCH_SIZES(SG_CASE)
#undef SG_CASE
            default: break;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) batch_c2r_kernel(const BatchInst* insts, const int* off, int n, int total) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int* o = off + BK_C2R * (n + 1);
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int i = batch_find(o, n, w);
        const int local = w - o[i];
        switch (insts[i].nx) {
#define SG_CASE(NN, WW) \
    case NN: fast_rows_c2r_body<float, NN, WW>(insts[i].c2r, local, smem_raw); break;
            SG_BATCH_SIZES(SG_CASE)
#undef SG_CASE
            default: break;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) batch_curl_kernel(const BatchInst* insts, const int* off, int n, int total) {
    const int* o = off + BK_CURL * (n + 1);
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int i = batch_find(o, n, w);
        const int local = w - o[i];
        const int tx = insts[i].curl_tiles_x;
        curl2d_body<float>(insts[i].curl, local % tx, local / tx);
        __syncthreads();
    }
}

// lines per block of the batched FFT passes for length n (256 threads)
static int batch_width(int n) {
    switch (n) {
        case 256: return 16;
        case 512: return 8;
        case 768: return 8;
        case 1024: return 4;
        default: return 0;
    }
}

static size_t batch_fft_smem(int n) {
    const int W = batch_width(n);
    const size_t c = sizeof(float2);
    const size_t rows = c * ((size_t)n * (W + 1) + n + (n + 1)) + sizeof(int64_t) * 3 * W + sizeof(float) * 2 * W + 32;
    const size_t lines = c * ((size_t)n * (W + 1) + n);
    return std::max(rows, lines);
}

}  // namespace sg

using namespace sg;

struct sg_batch2d_s {
    int n = 0;
    BatchInst* d_inst = nullptr;
    int* d_off = nullptr;
    int total[BK_COUNT] = {};
    size_t fft_smem = 0;
    int sweep_ty = 16;       // sweep tile height (8 or 16)
    int blocks_per_sm = 8;   // persistent grid size per SM (0: one block per work item)
};

static unsigned batch_grid(const sg_batch2d_s* b, int total) {
    if (total <= 0) return 0;
    if (b->blocks_per_sm <= 0) return (unsigned)total;
    return (unsigned)std::min<long long>(total, 152LL * b->blocks_per_sm);
}

extern "C" int sg_batch2d_create(int n, const sg_batch2d_member* m, sg_batch2d* out) {
    SG_REQUIRE(out && m && n >= 1 && n <= 4096, SG_ERR_INVALID_ARG, "batch2d: bad argument");
    *out = nullptr;
    std::vector<BatchInst> h(n);
    std::vector<int> off((size_t)BK_COUNT * (n + 1), 0);
    size_t smem = 0;
    for (int i = 0; i < n; ++i) {
        const sg_batch2d_member& mm = m[i];
        sg_flow_plan_s* p = mm.plan;
        SG_REQUIRE(p && p->dim == 2 && p->dtype == SG_F32, SG_ERR_INVALID_ARG,
                   "batch2d: member %d needs a 2D fp32 flow plan", i);
        SG_REQUIRE(mm.vorticity && mm.velocity && mm.forcing && mm.stream_func, SG_ERR_INVALID_ARG,
                   "batch2d: member %d has a null field", i);
        SG_REQUIRE(batch_width(p->nx) > 0 && batch_width(2 * p->ny) > 0, SG_ERR_SHAPE,
                   "batch2d: member %d grid (%d, %d): nx and 2 ny must be 256, 512, 768 or 1024", i, p->ny, p->nx);
        sg_poisson_plan_s* pp = p->poisson;
        BatchInst& b = h[i];
        b.ny = p->ny;
        b.nx = p->nx;
        b.sweep_tiles_x = (int)ceil_div(p->nx, 32);
        b.curl_tiles_x = (int)ceil_div(p->nx, 32);
        b.n_lag = mm.n_lag;
        ScalarSrc sc{};
        sc.dev = p->dev_scalars();
        float* w = (float*)mm.vorticity;
        float* u = (float*)mm.velocity;
        float* f = (float*)mm.forcing;
        float* psi = (float*)mm.stream_func;
        b.sweep = Sweep2DParams<float>{p->ny, p->nx, w, u, f, (float*)p->scratch_a, sc, SWEEP_ADVECT | SWEEP_DIFFUSE};
        FlowLoadParams<float> l{};
        l.dim = 2;
        l.nz = 1;
        l.ny = p->ny;
        l.nx = p->nx;
        l.width = p->width;
        l.src = (const float*)p->scratch_a;
        l.dst = w;
        l.forcing = f;
        l.zero_ncomp = 2;
        l.cx = (const float*)p->coef_x;
        l.cy = (const float*)p->coef_y;
        l.comp_stride = p->cells();
        l.spec = reinterpret_cast<float2*>(pp->spec);
        l.spec_map = row_map(p->ny, p->nx + 1, 1, 0, pp->spec_comp_elems);
        l.n_rows = p->ny;
        l.st = pp->st_x;
        l.tw_m = (const float2*)pp->tw_x;
        l.tw_l = (const float2*)pp->tw_xl;
        b.load = l;
        LinesParams<float> c{};
        c.in = reinterpret_cast<float2*>(pp->spec);
        c.out = reinterpret_cast<float2*>(pp->spec);
        c.n_in = p->ny;
        c.n_out = p->ny;
        c.inner = p->nx + 1;
        c.line_stride = p->nx + 1;
        c.outer_stride = 0;
        c.n_outer = 1;
        c.W = batch_width(2 * p->ny);
        c.st = pp->st_y;
        c.tw = (const float2*)pp->tw_y;
        c.g.table = (const float*)pp->greens;
        c.g.k_stride = p->nx + 1;
        c.g.inner_div = p->nx + 1;
        c.g.m_mod = 0;
        c.g.m_stride = 0;
        b.conv = c;
        RowsC2RParams<float> r{};
        r.in = reinterpret_cast<const float2*>(pp->spec);
        r.in_map = row_map(p->ny, p->nx + 1, 1, 0, pp->spec_comp_elems);
        r.out = psi;
        r.out_map = row_map(p->ny, p->nx);
        r.n_out = p->nx;
        r.n_rows = p->ny;
        r.st = pp->st_x;
        r.tw_m = (const float2*)pp->tw_x;
        r.tw_l = (const float2*)pp->tw_xl;
        b.c2r = r;
        Curl2DParams<float> cu{};
        cu.ny = p->ny;
        cu.nx = p->nx;
        cu.psi = psi;
        cu.u = u;
        cu.prefactor = 0.5f / (float)p->dx;
        cu.sc = sc;
        cu.add_free_stream = 1;
        cu.umax = (float*)p->umax_slot();
        b.curl = cu;
        if (mm.n_lag > 0) {
            SG_REQUIRE(mm.position && mm.body_velocity && mm.nearest && mm.weights && mm.flow_velocity &&
                           mm.velocity_mismatch && mm.position_mismatch && mm.lag_forcing && mm.status,
                       SG_ERR_INVALID_ARG, "batch2d: member %d has a null immersed-boundary buffer", i);
            b.ib = IBParams<float>{2, 1, p->ny, p->nx, mm.n_lag, mm.kernel_type, mm.dx, mm.shift, mm.position,
                                   mm.body_velocity, u, mm.nearest, (float*)mm.weights, (float*)mm.flow_velocity,
                                   (float*)mm.velocity_mismatch, (float*)mm.position_mismatch,
                                   (float*)mm.lag_forcing, mm.stiffness, mm.damping, 1, 0.0, p->dev_scalars(),
                                   mm.status};
            b.spread = SpreadParams<float>{2, 1, p->ny, p->nx, mm.n_lag, 0, mm.nearest, (const float*)mm.weights,
                                           (const float*)mm.lag_forcing, f};
        }
        b.dt = BatchDt{(float*)p->umax_slot(), p->dev_scalars(), p->time_slot(), (float)p->dx, mm.cfl, mm.nu,
                       mm.flow_density, mm.dt_prefac, mm.free_stream[0], mm.free_stream[1]};
        const int work[BK_COUNT] = {
            (mm.n_lag + 7) / 8,
            (int)ceil_div((int64_t)mm.n_lag * 16, 256),
            (int)(ceil_div(p->nx, 32) * ceil_div(p->ny, 16)),
            (int)ceil_div(p->ny, batch_width(p->nx)),
            (int)ceil_div(p->nx + 1, batch_width(2 * p->ny)),
            (int)ceil_div(p->ny, batch_width(p->nx)),
            (int)(ceil_div(p->nx, 32) * ceil_div(p->ny, 8)),
            (int)(ceil_div(p->nx, 32) * ceil_div(p->ny, 8)),
        };
        for (int k = 0; k < BK_COUNT; ++k) off[(size_t)k * (n + 1) + i + 1] = off[(size_t)k * (n + 1) + i] + work[k];
        smem = std::max(smem, std::max(batch_fft_smem(p->nx), batch_fft_smem(2 * p->ny)));
    }
    auto* b = new sg_batch2d_s();
    b->n = n;
    b->fft_smem = smem;
    for (int k = 0; k < BK_COUNT; ++k) b->total[k] = off[(size_t)k * (n + 1) + n];
    int st = SG_OK;
    do {
        if ((st = cuda_status(cudaMalloc(&b->d_inst, sizeof(BatchInst) * n), "batch2d table alloc"))) break;
        if ((st = cuda_status(cudaMalloc(&b->d_off, sizeof(int) * off.size()), "batch2d offsets alloc"))) break;
        if ((st = cuda_status(cudaMemcpy(b->d_inst, h.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice),
                              "batch2d table upload")))
            break;
        if ((st = cuda_status(cudaMemcpy(b->d_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice),
                              "batch2d offsets upload")))
            break;
        for (auto kern : {batch_load_kernel, batch_conv_kernel, batch_c2r_kernel}) {
            if ((st = cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                                  "batch2d smem attribute")))
                break;
        }
    } while (0);
    if (st != SG_OK) {
        cudaFree(b->d_inst);
        cudaFree(b->d_off);
        delete b;
        return st;
    }
    *out = b;
    return SG_OK;
}

extern "C" int sg_batch2d_set_tuning(sg_batch2d b, int sweep_tile_y, int blocks_per_sm) {
    SG_REQUIRE(b, SG_ERR_INVALID_ARG, "batch2d tuning: null batch");
    SG_REQUIRE(sweep_tile_y == 8 || sweep_tile_y == 16, SG_ERR_INVALID_ARG, "batch2d tuning: tile height 8 or 16");
    SG_REQUIRE(blocks_per_sm >= 0 && blocks_per_sm <= 32, SG_ERR_INVALID_ARG, "batch2d tuning: bad blocks per SM");
    b->sweep_ty = sweep_tile_y;
    b->blocks_per_sm = blocks_per_sm;
    return SG_OK;
}

extern "C" int sg_batch2d_step(sg_batch2d b, void* stream_) {
    SG_REQUIRE(b, SG_ERR_INVALID_ARG, "batch2d step: null batch");
    auto stream = (cudaStream_t)stream_;
    const int n = b->n;
    batch_dt_kernel<<<ceil_div(n, 64), 64, 0, stream>>>(b->d_inst, n);
    unsigned g;
    if ((g = batch_grid(b, b->total[BK_IB]))) batch_ib_kernel<<<g, 256, 0, stream>>>(b->d_inst, b->d_off, n, b->total[BK_IB]);
    if ((g = batch_grid(b, b->total[BK_SPREAD])))
        batch_spread_kernel<<<g, 256, 0, stream>>>(b->d_inst, b->d_off, n, b->total[BK_SPREAD]);
    if (b->sweep_ty == 16)
        batch_sweep_kernel<16><<<batch_grid(b, b->total[BK_SWEEP]), dim3(32, 8), 0, stream>>>(b->d_inst, b->d_off, n,
                                                                                            b->total[BK_SWEEP]);
    else
        batch_sweep_kernel<8><<<batch_grid(b, b->total[BK_SWEEP8]), dim3(32, 8), 0, stream>>>(b->d_inst, b->d_off, n,
                                                                                            b->total[BK_SWEEP8]);
    batch_load_kernel<<<batch_grid(b, b->total[BK_LOAD]), 256, b->fft_smem, stream>>>(b->d_inst, b->d_off, n,
                                                                                      b->total[BK_LOAD]);
    batch_conv_kernel<<<batch_grid(b, b->total[BK_CONV]), 256, b->fft_smem, stream>>>(b->d_inst, b->d_off, n,
                                                                                      b->total[BK_CONV]);
    batch_c2r_kernel<<<batch_grid(b, b->total[BK_C2R]), 256, b->fft_smem, stream>>>(b->d_inst, b->d_off, n,
                                                                                    b->total[BK_C2R]);
    batch_curl_kernel<<<batch_grid(b, b->total[BK_CURL]), dim3(32, 8), 0, stream>>>(b->d_inst, b->d_off, n,
                                                                                    b->total[BK_CURL]);
    return launch_status("batch2d step");
}

extern "C" int sg_batch2d_destroy(sg_batch2d b) {
    if (!b) return SG_OK;
    cudaFree(b->d_inst);
    cudaFree(b->d_off);
    delete b;
    return SG_OK;
}
