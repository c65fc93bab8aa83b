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
// bodies with a common 256-thread block: column convolution N = 256 (16 lines),
// 512 (8), 768 (8), 1024 (4); row passes (8 elements per thread) 256 (8),
// 512 (4), 768 (8), 1024 (2).
#include <algorithm>
#include <cfloat>
#include <vector>

#include "flow_plan.cuh"
#include "ib.cuh"

namespace sg {

enum { BK_IB = 0, BK_SPREAD, BK_SWEEP, BK_LOAD, BK_CONV, BK_C2R, BK_CURL, BK_SWEEP8, BK_LOAD512, BK_CONV512,
       BK_C2R512, BK_COUNT };

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
        if (marker < insts[i].n_lag) ib_interaction_body<float, 2>(insts[i].ib, marker);
    }
}

// A work item is 64 (marker, window cell) pairs of one instance, 8 per warp;
// the instance's nearest indices are staged in shared memory per item.
constexpr int kSpreadPairsPerItem = 64;

__global__ void __launch_bounds__(256) batch_spread_kernel(const BatchInst* insts, const int* off, int n,
                                                           int total) {
    extern __shared__ int s_near[];
    const int* o = off + BK_SPREAD * (n + 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int i = batch_find(o, n, w);
        const int local = w - o[i];
        const SpreadParams<float>& sp = insts[i].spread;
        const int n_lag = sp.n_lag;
        __syncthreads();  // the previous item's warps are done with s_near
        for (int e = threadIdx.x; e < 2 * n_lag; e += blockDim.x) s_near[e] = sp.nearest[e];
        __syncthreads();
        for (int q = warp; q < kSpreadPairsPerItem; q += 8) {
            const int pair = local * kSpreadPairsPerItem + q;
            if (pair < n_lag * 16) ib_spread_warp_pair<float, 2>(sp, s_near, pair / 16, pair % 16, lane);
        }
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

// The FFT passes run blocks of NT = 256 or 512 threads (picked by the
// autotuner).  Column convolution: 16 elements per thread (24 for the radix-3
// length); row passes (load, C2R): 8 (24), so half the lines per block.
template <int NT> struct BatchWidths;
template <> struct BatchWidths<256> {
    static constexpr int conv(int n) { return n == 256 ? 16 : n == 512 ? 8 : n == 768 ? 8 : n == 1024 ? 4 : 0; }
    static constexpr int rows(int n) { return n == 256 ? 8 : n == 512 ? 4 : n == 768 ? 8 : n == 1024 ? 2 : 0; }
};
template <> struct BatchWidths<512> {
    static constexpr int conv(int n) { return n == 256 ? 32 : n == 512 ? 16 : n == 768 ? 16 : n == 1024 ? 8 : 0; }
    static constexpr int rows(int n) { return n == 256 ? 16 : n == 512 ? 8 : n == 768 ? 16 : n == 1024 ? 4 : 0; }
};
template <int NN> constexpr int batch_row_elems() { return NN == 768 ? 24 : 8; }

#define SG_BATCH_SIZES(CALL) CALL(256) CALL(512) CALL(768) CALL(1024)

template <int NT>
__global__ void __launch_bounds__(NT) batch_load_kernel(const BatchInst* insts, const int* off, int n, int total) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int* o = off + (NT == 256 ? BK_LOAD : BK_LOAD512) * (n + 1);
    // a contiguous chunk of work items per block; the twiddles are staged again
    // only when the transform length changes
    const int chunk = (total + gridDim.x - 1) / gridDim.x;
    const int w_end = min(total, (blockIdx.x + 1) * chunk);
    int staged_len = 0;
    for (int w = blockIdx.x * chunk; w < w_end; ++w) {
        const int i = batch_find(o, n, w);
        const int local = w - o[i];
        const int len = insts[i].nx;
        const bool stage = len != staged_len;
        staged_len = len;
        switch (insts[i].nx) {
#define SG_CASE(NN)                                                                              \
    case NN:                                                                                     \
        fast_flow_load_body<float, NN, BatchWidths<NT>::rows(NN), batch_row_elems<NN>()>(insts[i].load, local, \
                                                                                         smem_raw, stage); \
        break;
            SG_BATCH_SIZES(SG_CASE)
#undef SG_CASE
            default: break;
        }
        __syncthreads();
    }
}

template <int NT>
__global__ void __launch_bounds__(NT) batch_conv_kernel(const BatchInst* insts, const int* off, int n, int total) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int* o = off + (NT == 256 ? BK_CONV : BK_CONV512) * (n + 1);
    // a contiguous chunk of work items per block; the twiddles are staged again
    // only when the transform length changes
    const int chunk = (total + gridDim.x - 1) / gridDim.x;
    const int w_end = min(total, (blockIdx.x + 1) * chunk);
    int staged_len = 0;
    for (int w = blockIdx.x * chunk; w < w_end; ++w) {
        const int i = batch_find(o, n, w);
        const int local = w - o[i];
        const int len = 2 * insts[i].ny;
        const bool stage = len != staged_len;
        staged_len = len;
        switch (2 * insts[i].ny) {
#define SG_CASE(NN)                                                                              \
    case NN:                                                                                     \
        fast_lines_body<float, NN, BatchWidths<NT>::conv(NN), LINE_CONV, FastElems<NN>::E, true, true>( \
            insts[i].conv, local, smem_raw, stage);                                              \
        break;
            SG_BATCH_SIZES(SG_CASE)
#undef SG_CASE
            default: break;
        }
        __syncthreads();
    }
}

template <int NT>
__global__ void __launch_bounds__(NT) batch_c2r_kernel(const BatchInst* insts, const int* off, int n, int total) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int* o = off + (NT == 256 ? BK_C2R : BK_C2R512) * (n + 1);
    // a contiguous chunk of work items per block; the twiddles are staged again
    // only when the transform length changes
    const int chunk = (total + gridDim.x - 1) / gridDim.x;
    const int w_end = min(total, (blockIdx.x + 1) * chunk);
    int staged_len = 0;
    for (int w = blockIdx.x * chunk; w < w_end; ++w) {
        const int i = batch_find(o, n, w);
        const int local = w - o[i];
        const int len = insts[i].nx;
        const bool stage = len != staged_len;
        staged_len = len;
        switch (insts[i].nx) {
#define SG_CASE(NN)                                                                              \
    case NN:                                                                                     \
        fast_rows_c2r_body<float, NN, BatchWidths<NT>::rows(NN), batch_row_elems<NN>(), true>(insts[i].c2r, local, \
                                                                                              smem_raw, stage); \
        break;
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

static int batch_row_width(int n, int nt) { return nt == 256 ? BatchWidths<256>::rows(n) : BatchWidths<512>::rows(n); }
static int batch_width(int n, int nt) { return nt == 256 ? BatchWidths<256>::conv(n) : BatchWidths<512>::conv(n); }

// dynamic shared memory of the row passes (load, C2R) and of the column convolution
static size_t batch_rows_smem(int n, int nt) {
    const int W = batch_row_width(n, nt);
    const size_t c = sizeof(float2);
    return c * ((size_t)n * (W + 1) + n + (n + 1)) + sizeof(int64_t) * 3 * W + sizeof(float) * 2 * W + 32;
}
static size_t batch_conv_smem(int n, int nt) {
    const int W = batch_width(n, nt);
    return sizeof(float2) * ((size_t)n * (W + 1) + n);
}

}  // namespace sg

using namespace sg;

struct sg_batch2d_s {
    int n = 0;
    BatchInst* d_inst = nullptr;
    int* d_off = nullptr;
    int total[BK_COUNT] = {};
    size_t rows_smem[2] = {};  // per FFT block size (256, 512)
    size_t conv_smem[2] = {};
    size_t near_smem = 0;    // staged nearest indices of the largest body
    int fft_threads = 256;   // block size of the FFT passes (256 or 512)
    int sweep_ty = 16;       // sweep tile height (8 or 16)
    int blocks_per_sm = 8;   // persistent grid size per SM (0: one block per work item)
};

static unsigned batch_grid(const sg_batch2d_s* b, int total) {
    if (total <= 0) return 0;
    if (b->blocks_per_sm <= 0) return (unsigned)total;
    return (unsigned)std::min<long long>(total, 152LL * b->blocks_per_sm);
}

// the FFT passes' blocks are twice as large: half the persistent blocks per SM
static unsigned batch_fft_grid(const sg_batch2d_s* b, int total) {
    if (total <= 0) return 0;
    if (b->blocks_per_sm <= 0) return (unsigned)total;
    return (unsigned)std::min<long long>(total, 152LL * std::max(1, b->blocks_per_sm / 2));
}

extern "C" int sg_batch2d_create(int n, const sg_batch2d_member* m, sg_batch2d* out) {
    SG_REQUIRE(out && m && n >= 1 && n <= 4096, SG_ERR_INVALID_ARG, "batch2d: bad argument");
    *out = nullptr;
    std::vector<BatchInst> h(n);
    std::vector<int> off((size_t)BK_COUNT * (n + 1), 0);
    size_t rows_smem[2] = {}, conv_smem[2] = {}, near_smem = 0;
    for (int i = 0; i < n; ++i) {
        const sg_batch2d_member& mm = m[i];
        sg_flow_plan_s* p = mm.plan;
        SG_REQUIRE(p && p->dim == 2 && p->dtype == SG_F32, SG_ERR_INVALID_ARG,
                   "batch2d: member %d needs a 2D fp32 flow plan", i);
        SG_REQUIRE(mm.vorticity && mm.velocity && mm.forcing && mm.stream_func, SG_ERR_INVALID_ARG,
                   "batch2d: member %d has a null field", i);
        SG_REQUIRE(batch_width(p->nx, 256) > 0 && batch_width(2 * p->ny, 256) > 0, SG_ERR_SHAPE,
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
        c.W = 0;  // set by the body's compile-time width
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
            (int)ceil_div((int64_t)mm.n_lag * 16, kSpreadPairsPerItem),
            (int)(ceil_div(p->nx, 32) * ceil_div(p->ny, 16)),
            (int)ceil_div(p->ny, batch_row_width(p->nx, 256)),
            (int)ceil_div(p->nx + 1, batch_width(2 * p->ny, 256)),
            (int)ceil_div(p->ny, batch_row_width(p->nx, 256)),
            (int)(ceil_div(p->nx, 32) * ceil_div(p->ny, 8)),
            (int)(ceil_div(p->nx, 32) * ceil_div(p->ny, 8)),
            (int)ceil_div(p->ny, batch_row_width(p->nx, 512)),
            (int)ceil_div(p->nx + 1, batch_width(2 * p->ny, 512)),
            (int)ceil_div(p->ny, batch_row_width(p->nx, 512)),
        };
        for (int k = 0; k < BK_COUNT; ++k) off[(size_t)k * (n + 1) + i + 1] = off[(size_t)k * (n + 1) + i] + work[k];
        for (int v = 0; v < 2; ++v) {
            const int nt = v == 0 ? 256 : 512;
            rows_smem[v] = std::max(rows_smem[v], batch_rows_smem(p->nx, nt));
            conv_smem[v] = std::max(conv_smem[v], batch_conv_smem(2 * p->ny, nt));
        }
        near_smem = std::max(near_smem, (size_t)2 * mm.n_lag * sizeof(int));
    }
    auto* b = new sg_batch2d_s();
    b->n = n;
    for (int v = 0; v < 2; ++v) {
        b->rows_smem[v] = rows_smem[v];
        b->conv_smem[v] = conv_smem[v];
    }
    b->near_smem = near_smem;
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
        auto attr = [&](const void* kern, size_t bytes) {
            return cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
                               "batch2d smem attribute");
        };
        if ((st = attr((const void*)batch_load_kernel<256>, rows_smem[0]))) break;
        if ((st = attr((const void*)batch_c2r_kernel<256>, rows_smem[0]))) break;
        if ((st = attr((const void*)batch_conv_kernel<256>, conv_smem[0]))) break;
        if ((st = attr((const void*)batch_load_kernel<512>, rows_smem[1]))) break;
        if ((st = attr((const void*)batch_c2r_kernel<512>, rows_smem[1]))) break;
        if ((st = attr((const void*)batch_conv_kernel<512>, conv_smem[1]))) break;
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

extern "C" int sg_batch2d_set_tuning(sg_batch2d b, int sweep_tile_y, int blocks_per_sm, int fft_threads) {
    SG_REQUIRE(b, SG_ERR_INVALID_ARG, "batch2d tuning: null batch");
    SG_REQUIRE(sweep_tile_y == 8 || sweep_tile_y == 16, SG_ERR_INVALID_ARG, "batch2d tuning: tile height 8 or 16");
    SG_REQUIRE(blocks_per_sm >= 0 && blocks_per_sm <= 32, SG_ERR_INVALID_ARG, "batch2d tuning: bad blocks per SM");
    SG_REQUIRE(fft_threads == 256 || fft_threads == 512, SG_ERR_INVALID_ARG, "batch2d tuning: FFT block 256 or 512");
    b->sweep_ty = sweep_tile_y;
    b->blocks_per_sm = blocks_per_sm;
    b->fft_threads = fft_threads;
    return SG_OK;
}

extern "C" int sg_batch2d_step(sg_batch2d b, void* stream_) {
    SG_REQUIRE(b, SG_ERR_INVALID_ARG, "batch2d step: null batch");
    SG_REQUIRE(b->near_smem <= 48 * 1024, SG_ERR_UNSUPPORTED, "batch2d step: a body has more than 6144 markers");
    auto stream = (cudaStream_t)stream_;
    const int n = b->n;
    batch_dt_kernel<<<ceil_div(n, 64), 64, 0, stream>>>(b->d_inst, n);
    unsigned g;
    if ((g = batch_grid(b, b->total[BK_IB]))) batch_ib_kernel<<<g, 256, 0, stream>>>(b->d_inst, b->d_off, n, b->total[BK_IB]);
    if ((g = batch_grid(b, b->total[BK_SPREAD])))
        batch_spread_kernel<<<g, 256, b->near_smem, stream>>>(b->d_inst, b->d_off, n, b->total[BK_SPREAD]);
    if (b->sweep_ty == 16)
        batch_sweep_kernel<16><<<batch_grid(b, b->total[BK_SWEEP]), dim3(32, 8), 0, stream>>>(b->d_inst, b->d_off, n,
                                                                                            b->total[BK_SWEEP]);
    else
        batch_sweep_kernel<8><<<batch_grid(b, b->total[BK_SWEEP8]), dim3(32, 8), 0, stream>>>(b->d_inst, b->d_off, n,
                                                                                            b->total[BK_SWEEP8]);
    if (b->fft_threads == 256) {
        const int tl = b->total[BK_LOAD], tc = b->total[BK_CONV], tr = b->total[BK_C2R];
        batch_load_kernel<256><<<batch_grid(b, tl), 256, b->rows_smem[0], stream>>>(b->d_inst, b->d_off, n, tl);
        batch_conv_kernel<256><<<batch_grid(b, tc), 256, b->conv_smem[0], stream>>>(b->d_inst, b->d_off, n, tc);
        batch_c2r_kernel<256><<<batch_grid(b, tr), 256, b->rows_smem[0], stream>>>(b->d_inst, b->d_off, n, tr);
    } else {
        const int tl = b->total[BK_LOAD512], tc = b->total[BK_CONV512], tr = b->total[BK_C2R512];
        batch_load_kernel<512><<<batch_fft_grid(b, tl), 512, b->rows_smem[1], stream>>>(b->d_inst, b->d_off, n, tl);
        batch_conv_kernel<512><<<batch_fft_grid(b, tc), 512, b->conv_smem[1], stream>>>(b->d_inst, b->d_off, n, tc);
        batch_c2r_kernel<512><<<batch_fft_grid(b, tr), 512, b->rows_smem[1], stream>>>(b->d_inst, b->d_off, n, tr);
    }
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
