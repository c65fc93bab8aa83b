// Register-resident line FFTs for the strided passes of the 3D Poisson solve (fp32, N = 256, 512).
//
// The line kernels of fft_fast.cuh stage every line in shared memory and run each radix stage
// through it, so a point crosses shared memory 12-16 times per convolution; at 256^3 the z
// convolution was bound by the shared-memory request queue at under a quarter of the HBM
// bandwidth.  Here a line of N = 16 E points is factored as
//     n = g + 16 j   (g < 16: the thread of the line, j < E: the thread's points),
//     k = k2 + E k1  (k2 < E, k1 < 16),
//     X[k2 + E k1] = sum_g w16^(g k1) [ w_N^(g k2) sum_j w_E^(j k2) x[g + 16 j] ],
// and a block of 256 threads owns 16 adjacent lines (16 threads per line):
//   stage A:  thread (line, g) loads its E points straight from global memory (16 adjacent lines
//             make two contiguous 128-byte runs per warp access), takes their length-E DFT in
//             registers and multiplies point k2 by w_N^(g k2);
//   exchange: the E values go to shared memory [g][k2][line] once, and come back transposed;
//   stage B:  thread (line, t) takes the E/16 length-16 DFTs over g for k2 = t + 16 b, holding
//             the spectrum points k2 + E k1 in registers, from where they are stored (forward),
//             or multiplied by the Green's table and transformed back (convolution).
// The inverse runs the same network transposed: stage B inverse, one exchange, stage A inverse.
// A point therefore crosses shared memory once per direction.  The zero padding of the doubled
// domain (input points >= N/2 are zero) halves the loads and the first DFT layer of stage A, and
// the crop (only points < N/2 kept) halves the stores and the last layer of the inverse.
//
// The per-thread phases are __host__ __device__ so that a host driver can run a block's threads
// phase by phase (barriers between phases) and check the index arithmetic without a GPU.
#pragma once

#include <algorithm>

#include "fft_fast.cuh"

#ifdef __CUDACC__
#define SG_RL_FN __host__ __device__ __forceinline__
#else
#define SG_RL_FN inline
#endif

namespace sg {

// Parameters of one strided-line pass.  Line q (0 <= q < n_lines) lies in slab q / slab_lines at
// position w = q % slab_lines; its point k is element (q / slab_lines) * slab_stride + w +
// k * stride.  Lines of one slab are adjacent in memory.
struct RegLinesParams {
    const float2* in;
    float2* out;          // may alias `in`: each block reads and writes only its own lines
    int n_lines;
    int slab_lines;
    int64_t slab_stride;
    int64_t stride;
    int n_in;             // input points < n_in may be non-zero
    int n_out;            // output points < n_out are stored
    const float2* tw;     // exp(-2 pi i m / N), m < N
    // Green's factor of the convolution: g[ks * g_kstride + ms * g_mstride + kx] with
    // ks = min(k, N - k), w = m * g_div + kx, ms = min(m, g_mmod - m) (ms = 0 when g_mmod == 0)
    const float* g;
    int64_t g_kstride;
    int64_t g_mstride;
    int g_div;
    int g_mmod;
    // > 1: consecutive blocks take the same 16 lines of `interleave` consecutive slabs (the three
    // components of the z pass share their Green's table rows through L2); needs slab_lines % 16 == 0
    // and n_lines == interleave * slab_lines
    int interleave;
    // forward and convolution passes with a zero-padded input: the persistent kernel that streams
    // each block's next line group into shared memory while it transforms the current one
    int persistent;
};

enum { RL_FWD = 0, RL_INV = 1, RL_CONV = 2 };

namespace rl {

constexpr int kLines = 16;    // lines per block
constexpr int kThreads = 256; // 16 threads per line

template <int N> struct Shape {
    static_assert(N == 256 || N == 512, "register line FFT lengths: 256 and 512");
    static constexpr int E = N / 16;  // points per thread
    static constexpr int B = E / 16;  // length-16 DFTs per thread in stage B
    static constexpr int TW = 16 * E;  // stage-A twiddles w_N^(g k2), [g][k2]
    static constexpr size_t smem_bytes = sizeof(float2) * ((size_t)N * kLines + TW);
};

// cos and sin of 2 pi m / 32, m < 16 (the twiddles inside a 32-point DFT)
SG_RL_FN constexpr double w32_cos(int m) {
    return m == 0 ? 1.0 : m == 1 ? 0.98078528040323044913 : m == 2 ? 0.92387953251128675613
         : m == 3 ? 0.83146961230254523708 : m == 4 ? 0.70710678118654752440 : m == 5 ? 0.55557023301960222474
         : m == 6 ? 0.38268343236508977173 : m == 7 ? 0.19509032201612826785 : m == 8 ? 0.0
         : m == 9 ? -0.19509032201612826785 : m == 10 ? -0.38268343236508977173 : m == 11 ? -0.55557023301960222474
         : m == 12 ? -0.70710678118654752440 : m == 13 ? -0.83146961230254523708 : m == 14 ? -0.92387953251128675613
         : -0.98078528040323044913;
}
SG_RL_FN constexpr double w32_sin(int m) { return m <= 8 ? w32_cos(8 - m) : w32_cos(m - 8); }

// Length-32 DFT in natural order as two length-16 DFTs of the even and odd points.  HALF_IN:
// points 16..31 are zero (so are the upper halves of both halves).  HALF_OUT: only outputs
// 0..15 are formed.
template <bool INV, bool HALF_IN, bool HALF_OUT>
SG_RL_FN void dft32(float2* v) {
    float2 e[16], o[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) {
        e[m] = v[2 * m];
        o[m] = v[2 * m + 1];
    }
    dft16<INV, HALF_IN>(e);
    dft16<INV, HALF_IN>(o);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        float2 t = o[k];
        if (k == 8) {
            t = INV ? cmake<float2>(-t.y, t.x) : cmake<float2>(t.y, -t.x);
        } else if (k != 0) {
            const float c = (float)w32_cos(k), s = (float)w32_sin(k);
            t = cmul(t, cmake<float2>(c, INV ? s : -s));
        }
        v[k] = cadd(e[k], t);
        if (!HALF_OUT) v[k + 16] = csub(e[k], t);
    }
}

template <int E, bool INV, bool HALF_IN, bool HALF_OUT>
SG_RL_FN void dft_e(float2* v) {
    if constexpr (E == 32) dft32<INV, HALF_IN, HALF_OUT>(v);
    else dft16<INV, HALF_IN>(v);
}

// Shared-memory slot of (g, k2, line): line fastest, so each half-warp touches 128 contiguous bytes.
template <int N> SG_RL_FN int sidx(int g, int k2, int l) { return (g * Shape<N>::E + k2) * kLines + l; }

struct Line {
    int64_t base;  // element of point 0
    int w;         // position within the slab
    bool live;
};

SG_RL_FN Line line_of(const RegLinesParams& p, int block, int l) {
    Line L;
    if (p.interleave > 1) {
        const int grp = block / p.interleave, slab = block - grp * p.interleave;
        L.w = grp * kLines + l;
        L.live = L.w < p.slab_lines;
        if (!L.live) L.w = 0;
        L.base = (int64_t)slab * p.slab_stride + L.w;
        return L;
    }
    const int q = block * kLines + l;
    L.live = q < p.n_lines;
    const int qq = L.live ? q : 0;
    const int slab = qq / p.slab_lines;
    L.w = qq - slab * p.slab_lines;
    L.base = (int64_t)slab * p.slab_stride + L.w;
    return L;
}

// The stage-A twiddle table of a block: tw_a[g * E + k2] = w_N^(g k2), g < 16, k2 < E (g k2 < N).
template <int N> SG_RL_FN void stage_twiddles(const RegLinesParams& p, float2* tw_a, int tid, int nt) {
    constexpr int E = Shape<N>::E;
    for (int i = tid; i < 16 * E; i += nt) tw_a[i] = p.tw[(i / E) * (i % E)];
}

// ---- stage A (thread (l, g)): points g + 16 j
template <int N, bool HIN>
SG_RL_FN void load_a(const RegLinesParams& p, const Line& L, int g, float2* v) {
    constexpr int E = Shape<N>::E;
#pragma unroll
    for (int j = 0; j < E; ++j) {
        const int n = g + 16 * j;
        v[j] = cmake<float2>(0.f, 0.f);
        if (!(HIN && j >= E / 2) && L.live && n < p.n_in) v[j] = p.in[L.base + (int64_t)n * p.stride];
    }
}

template <int N, bool HIN>
SG_RL_FN void fwd_a(const float2* tw_a, int g, float2* v) {
    constexpr int E = Shape<N>::E;
    dft_e<E, false, HIN, false>(v);
    const float2* w = tw_a + g * E;
#pragma unroll
    for (int k2 = 1; k2 < E; ++k2) v[k2] = cmul(v[k2], w[k2]);
}

template <int N, bool HOUT>
SG_RL_FN void inv_a(const float2* tw_a, int g, float2* v) {
    constexpr int E = Shape<N>::E;
    const float2* w = tw_a + g * E;
#pragma unroll
    for (int k2 = 1; k2 < E; ++k2) v[k2] = cmul(v[k2], cconj(w[k2]));
    dft_e<E, true, false, HOUT>(v);
}

template <int N, bool HOUT>
SG_RL_FN void store_a(const RegLinesParams& p, const Line& L, int g, const float2* v) {
    constexpr int E = Shape<N>::E;
#pragma unroll
    for (int j = 0; j < (HOUT ? E / 2 : E); ++j) {
        const int n = g + 16 * j;
        if (L.live && n < p.n_out) p.out[L.base + (int64_t)n * p.stride] = v[j];
    }
}

template <int N> SG_RL_FN void write_a(float2* buf, int l, int g, const float2* v) {
#pragma unroll
    for (int k2 = 0; k2 < Shape<N>::E; ++k2) buf[sidx<N>(g, k2, l)] = v[k2];
}

template <int N> SG_RL_FN void read_a(const float2* buf, int l, int g, float2* v) {
#pragma unroll
    for (int k2 = 0; k2 < Shape<N>::E; ++k2) v[k2] = buf[sidx<N>(g, k2, l)];
}

// ---- stage B (thread (l, t)): register b * 16 + r holds index r of the length-16 DFT for
// k2 = t + 16 b; after the forward DFT that is spectrum point k2 + E r.
template <int N> SG_RL_FN int point_b(int t, int b, int r) { return t + 16 * b + Shape<N>::E * r; }

template <int N> SG_RL_FN void read_b(const float2* buf, int l, int t, float2* v) {
#pragma unroll
    for (int b = 0; b < Shape<N>::B; ++b)
#pragma unroll
        for (int gg = 0; gg < 16; ++gg) v[b * 16 + gg] = buf[sidx<N>(gg, t + 16 * b, l)];
}

template <int N> SG_RL_FN void write_b(float2* buf, int l, int t, const float2* v) {
#pragma unroll
    for (int b = 0; b < Shape<N>::B; ++b)
#pragma unroll
        for (int gg = 0; gg < 16; ++gg) buf[sidx<N>(gg, t + 16 * b, l)] = v[b * 16 + gg];
}

template <int N, bool INV> SG_RL_FN void dft_b(float2* v) {
#pragma unroll
    for (int b = 0; b < Shape<N>::B; ++b) dft16<INV>(v + 16 * b);
}

template <int N>
SG_RL_FN void load_b(const RegLinesParams& p, const Line& L, int t, float2* v) {
#pragma unroll
    for (int b = 0; b < Shape<N>::B; ++b)
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const int k = point_b<N>(t, b, r);
            v[b * 16 + r] = cmake<float2>(0.f, 0.f);
            if (L.live && k < p.n_in) v[b * 16 + r] = p.in[L.base + (int64_t)k * p.stride];
        }
}

template <int N>
SG_RL_FN void store_b(const RegLinesParams& p, const Line& L, int t, const float2* v) {
#pragma unroll
    for (int b = 0; b < Shape<N>::B; ++b)
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const int k = point_b<N>(t, b, r);
            if (L.live && k < p.n_out) p.out[L.base + (int64_t)k * p.stride] = v[b * 16 + r];
        }
}

template <int N>
SG_RL_FN void green_b(const RegLinesParams& p, const Line& L, int t, float2* v) {
    const int m = L.w / p.g_div;
    const int kx = L.w - m * p.g_div;
    const int ms = p.g_mmod > 0 ? (m < p.g_mmod - m ? m : p.g_mmod - m) : 0;
    const float* gl = p.g + (int64_t)ms * p.g_mstride + kx;
    // point k = t + 16 b + E r; for r < 8, k < N/2 and the folded index is k, else N - k
    const int64_t kst = p.g_kstride;
    const float* lo = gl + (int64_t)t * kst;
    const float* hi = gl + (int64_t)(N - t) * kst;
#pragma unroll
    for (int b = 0; b < Shape<N>::B; ++b)
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const int64_t off = (int64_t)(16 * b + Shape<N>::E * r) * kst;
            const float gv = L.live ? (r < 8 ? lo[off] : hi[-off]) : 0.f;
            v[b * 16 + r] = cscale(v[b * 16 + r], gv);
        }
}

// ---- prefetched input of the persistent kernels: stage[n * 16 + l] holds point n < N/2 of line l
// of the next group, copied asynchronously while the current group is transformed.
template <int N> struct Pipe {
    static constexpr int NIN = N / 2;                 // zero-padded input: points >= N/2 are zero
    static constexpr int COPIES = NIN * kLines / kThreads;  // 8-byte copies per thread
    static constexpr size_t smem_bytes = Shape<N>::smem_bytes + sizeof(float2) * (size_t)NIN * kLines;
};

// Copy c of thread tid for line group grp: the destination slot and the source element, or
// src = -1 where the point is zero (a dead line, or n >= n_in).
template <int N> SG_RL_FN void stage_copy(const RegLinesParams& p, int grp, int tid, int c, int& slot,
                                          int64_t& src) {
    const int idx = tid + c * kThreads;
    const int l = idx & (kLines - 1), n = idx / kLines;
    const Line L = line_of(p, grp, l);
    slot = n * kLines + l;
    src = (L.live && n < p.n_in) ? L.base + (int64_t)n * p.stride : -1;
}

template <int N> SG_RL_FN void load_a_staged(const float2* stage, int l, int g, float2* v) {
    constexpr int E = Shape<N>::E;
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = j < E / 2 ? stage[(g + 16 * j) * kLines + l] : cmake<float2>(0.f, 0.f);
}

}  // namespace rl

#ifdef __CUDACC__
// One pass over 16 lines per block.  RL_FWD: forward transform, spectrum stored (HIN prunes a
// zero upper input half).  RL_INV: inverse transform of a full spectrum (HOUT keeps the lower
// output half).  RL_CONV: forward, Green's factor, inverse, in registers between the exchanges.
template <int N, int MODE, bool HIN, bool HOUT>
__global__ void __launch_bounds__(rl::kThreads, (N == 512 ? 2 : 3)) reg_lines_kernel(RegLinesParams p) {
    extern __shared__ __align__(16) float2 rl_buf[];
    float2* tw_a = rl_buf + N * rl::kLines;
    const int tid = threadIdx.x, l = tid & (rl::kLines - 1), q = tid / rl::kLines;
    const rl::Line L = rl::line_of(p, blockIdx.x, l);
    float2 v[rl::Shape<N>::E];
    rl::stage_twiddles<N>(p, tw_a, tid, rl::kThreads);
    if constexpr (MODE == RL_INV) {
        rl::load_b<N>(p, L, q, v);
        rl::dft_b<N, true>(v);
        rl::write_b<N>(rl_buf, l, q, v);
        __syncthreads();
        rl::read_a<N>(rl_buf, l, q, v);
        rl::inv_a<N, HOUT>(tw_a, q, v);
        rl::store_a<N, HOUT>(p, L, q, v);
    } else {
        rl::load_a<N, HIN>(p, L, q, v);
        __syncthreads();  // the twiddle table
        rl::fwd_a<N, HIN>(tw_a, q, v);
        rl::write_a<N>(rl_buf, l, q, v);
        __syncthreads();
        rl::read_b<N>(rl_buf, l, q, v);
        rl::dft_b<N, false>(v);
        if constexpr (MODE == RL_FWD) {
            rl::store_b<N>(p, L, q, v);
        } else {
            rl::green_b<N>(p, L, q, v);
            rl::dft_b<N, true>(v);
            __syncthreads();
            rl::write_b<N>(rl_buf, l, q, v);
            __syncthreads();
            rl::read_a<N>(rl_buf, l, q, v);
            rl::inv_a<N, HOUT>(tw_a, q, v);
            rl::store_a<N, HOUT>(p, L, q, v);
        }
    }
}

namespace rl {
__device__ __forceinline__ void cp_async8(float2* dst, const float2* src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 8 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <int N> __device__ __forceinline__ void prefetch(const RegLinesParams& p, int grp, float2* stage) {
#pragma unroll
    for (int c = 0; c < Pipe<N>::COPIES; ++c) {
        int slot;
        int64_t src;
        stage_copy<N>(p, grp, threadIdx.x, c, slot, src);
        cp_async8(stage + slot, p.in + (src < 0 ? 0 : src), src >= 0);
    }
    cp_async_commit();
}
}  // namespace rl

// Persistent form of the forward and convolution passes with a zero-padded input (n_in <= N/2):
// each block walks line groups grp = blockIdx.x, blockIdx.x + gridDim.x, ..., and while it
// transforms one group the input of its next group streams into shared memory with cp.async, so
// the global-load latency is hidden behind the arithmetic instead of stalling every block at its
// start.  The arithmetic is the per-block kernel's, phase for phase.
template <int N, int MODE, bool HOUT>
__global__ void __launch_bounds__(rl::kThreads, 2) reg_lines_pipe_kernel(RegLinesParams p, int n_groups) {
    static_assert(MODE != RL_INV, "the persistent form prefetches a zero-padded input");
    extern __shared__ __align__(16) float2 rl_buf[];
    float2* tw_a = rl_buf + N * rl::kLines;
    float2* stage = tw_a + rl::Shape<N>::TW;
    const int tid = threadIdx.x, l = tid & (rl::kLines - 1), q = tid / rl::kLines;
    float2 v[rl::Shape<N>::E];
    int grp = blockIdx.x;
    if (grp < n_groups) rl::prefetch<N>(p, grp, stage);
    rl::stage_twiddles<N>(p, tw_a, tid, rl::kThreads);
    for (; grp < n_groups; grp += gridDim.x) {
        const rl::Line L = rl::line_of(p, grp, l);
        rl::cp_async_wait_all();
        __syncthreads();  // this group's input (and, first time, the twiddles) in place
        rl::load_a_staged<N>(stage, l, q, v);
        __syncthreads();  // the stage is free for the next group
        if (grp + (int)gridDim.x < n_groups) rl::prefetch<N>(p, grp + gridDim.x, stage);
        rl::fwd_a<N, true>(tw_a, q, v);
        rl::write_a<N>(rl_buf, l, q, v);
        __syncthreads();
        rl::read_b<N>(rl_buf, l, q, v);
        rl::dft_b<N, false>(v);
        if constexpr (MODE == RL_FWD) {
            rl::store_b<N>(p, L, q, v);
        } else {
            rl::green_b<N>(p, L, q, v);
            rl::dft_b<N, true>(v);
            __syncthreads();
            rl::write_b<N>(rl_buf, l, q, v);
            __syncthreads();
            rl::read_a<N>(rl_buf, l, q, v);
            rl::inv_a<N, HOUT>(tw_a, q, v);
            rl::store_a<N, HOUT>(p, L, q, v);
        }
    }
    rl::cp_async_wait_all();  // nothing left in flight when the block exits
}

// Launches the pass when N is one of the register lengths; returns SG_ERR_UNSUPPORTED otherwise so
// the caller can take the shared-memory kernels.
template <int MODE>
int launch_reg_lines(const RegLinesParams& p, int N, cudaStream_t stream) {
    const bool hin = MODE != RL_INV && 2 * p.n_in <= N;
    const bool hout = MODE != RL_FWD && 2 * p.n_out <= N;
    const bool inter_ok = p.interleave <= 1 || (p.slab_lines % rl::kLines == 0 &&
                                               (int64_t)p.interleave * p.slab_lines == p.n_lines);
    SG_REQUIRE(inter_ok, SG_ERR_INVALID_ARG, "register lines: interleave needs whole 16-line groups");
    const unsigned blocks = ceil_div(p.n_lines, rl::kLines);
    if (p.n_lines <= 0) return SG_OK;
    auto run = [&](auto kern, size_t smem) -> int {
        SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                           "register lines smem attribute"));
        SG_TRY(fast_max_carveout(kern, "register lines carveout attribute"));
        kern<<<blocks, rl::kThreads, smem, stream>>>(p);
        return launch_status("register lines");
    };
#define SG_RL_PICK(NN)                                                                                      \
    {                                                                                                       \
        constexpr size_t smem = rl::Shape<NN>::smem_bytes;                                                  \
        if (hin && hout) return run(reg_lines_kernel<NN, MODE, MODE != RL_INV, MODE != RL_FWD>, smem);      \
        if (hin) return run(reg_lines_kernel<NN, MODE, MODE != RL_INV, false>, smem);                      \
        if (hout) return run(reg_lines_kernel<NN, MODE, false, MODE != RL_FWD>, smem);                     \
        return run(reg_lines_kernel<NN, MODE, false, false>, smem);                                         \
    }
    if constexpr (MODE != RL_INV) if (hin && p.persistent) {
        // one block per pair of resident slots: the grid is sized to the GPU, not to the lines
        auto run_pipe = [&](auto kern, size_t smem) -> int {
            SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                               "register lines smem attribute"));
            SG_TRY(fast_max_carveout(kern, "register lines carveout attribute"));
            int dev = 0, sms = 0, per_sm = 0;
            SG_TRY(cuda_status(cudaGetDevice(&dev), "register lines device"));
            SG_TRY(cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"));
            SG_TRY(cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, rl::kThreads, smem),
                               "register lines occupancy"));
            const int grid = (int)std::min<long long>((long long)sms * (per_sm > 0 ? per_sm : 1), blocks);
            kern<<<grid, rl::kThreads, smem, stream>>>(p, (int)blocks);
            return launch_status("register lines (persistent)");
        };
        if (N == 512)
            return hout ? run_pipe(reg_lines_pipe_kernel<512, MODE, MODE != RL_FWD>, rl::Pipe<512>::smem_bytes)
                        : run_pipe(reg_lines_pipe_kernel<512, MODE, false>, rl::Pipe<512>::smem_bytes);
        if (N == 256)
            return hout ? run_pipe(reg_lines_pipe_kernel<256, MODE, MODE != RL_FWD>, rl::Pipe<256>::smem_bytes)
                        : run_pipe(reg_lines_pipe_kernel<256, MODE, false>, rl::Pipe<256>::smem_bytes);
    }
    if (N == 512) SG_RL_PICK(512)
    if (N == 256) SG_RL_PICK(256)
#undef SG_RL_PICK
    return SG_ERR_UNSUPPORTED;
}
#endif

}  // namespace sg
