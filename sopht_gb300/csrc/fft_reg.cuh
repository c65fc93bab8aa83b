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
    // > 0: each block also asks L2 for the input of block blockIdx + prefetch_ahead (about one
    // wave of resident blocks later), so that block's loads find it there
    int prefetch_ahead;
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

// The input points load_a (HIN: the lower half) or load_b would load for line L, asked of L2.
template <int N, bool HIN, bool STAGE_B>
SG_RL_FN void prefetch_input(const RegLinesParams& p, const Line& L, int q) {
#ifdef __CUDA_ARCH__
    if (!L.live) return;
    constexpr int E = Shape<N>::E;
    if constexpr (STAGE_B) {
#pragma unroll
        for (int b = 0; b < Shape<N>::B; ++b)
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int k = point_b<N>(q, b, r);
                if (k < p.n_in) asm volatile("prefetch.global.L2 [%0];" ::"l"(p.in + L.base + (int64_t)k * p.stride));
            }
    } else {
#pragma unroll
        for (int j = 0; j < (HIN ? E / 2 : E); ++j) {
            const int n = q + 16 * j;
            if (n < p.n_in) asm volatile("prefetch.global.L2 [%0];" ::"l"(p.in + L.base + (int64_t)n * p.stride));
        }
    }
#endif
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

// ---- rows: the x pass's complex-to-real transform (M = 256 complex points of a 512-real row), 16
// rows per block, 16 threads per row.  Thread (row, t) reads bins k = t + 16 k1 and M - k, forms
// the packed spectrum Z[k] of the half-length transform, takes the inverse length-16 DFTs over k1,
// one exchange ([g][row][k2], a one-point pad per g so the stage-A reads hit distinct banks), and
// thread (row, g) finishes the inverse over k2 with the twiddles w_M^(-g k2), holding z[g + 16 j]
// = x[2n] + i x[2n+1], n = g + 16 j.  Only n < n_out / 2 is stored (the crop).
constexpr int kRowM = 256;
SG_RL_FN int row_slot(int g, int row, int k2) { return g * (kLines * 16 + 1) + row * 16 + k2; }
constexpr int kRowSlots = 16 * (kLines * 16 + 1);

struct RowLine {
    int64_t in_off, out_off;
    bool live;
};

SG_RL_FN RowLine row_of(const RowsC2RParams<float>& p, int block, int row) {
    RowLine R;
    const int q = block * kLines + row;
    R.live = q < p.n_rows;
    R.in_off = R.live ? p.in_map.offset(q) : 0;
    R.out_off = R.live ? p.out_map.offset(q) : 0;
    return R;
}

// w_M^(g k2) for the row transform: tw_m[m] = exp(-2 pi i m / M).
SG_RL_FN void stage_row_twiddles(const RowsC2RParams<float>& p, float2* tw_a, int tid, int nt) {
    for (int i = tid; i < 256; i += nt) tw_a[i] = p.tw_m[(i / 16) * (i % 16)];
}

SG_RL_FN void c2r_load_b(const RowsC2RParams<float>& p, const RowLine& R, int t, float2* v) {
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) {
        const int k = t + 16 * k1;
        v[k1] = cmake<float2>(0.f, 0.f);
        if (!R.live) continue;
        float2 xk = p.in[R.in_off + k];
        float2 xm = p.in[R.in_off + kRowM - k];
        if (k == 0) {
            xk.y = 0.f;
            xm.y = 0.f;
        }
        const float2 xc = cconj(xm);
        float2 w = p.tw_l[k];
        w.y = -w.y;
        const float2 sm = cadd(xk, xc);
        const float2 wd = cmul(w, csub(xk, xc));
        v[k1] = cmake<float2>(sm.x - wd.y, sm.y + wd.x);
    }
}

SG_RL_FN void c2r_write_b(float2* buf, int row, int t, const float2* v) {
#pragma unroll
    for (int gg = 0; gg < 16; ++gg) buf[row_slot(gg, row, t)] = v[gg];
}

SG_RL_FN void c2r_read_a(const float2* buf, int row, int g, float2* v) {
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) v[k2] = buf[row_slot(g, row, k2)];
}

SG_RL_FN void c2r_inv_a(const float2* tw_a, int g, float2* v) {
#pragma unroll
    for (int k2 = 1; k2 < 16; ++k2) v[k2] = cmul(v[k2], cconj(tw_a[g * 16 + k2]));
    dft16<true>(v);
}

SG_RL_FN void c2r_store_a(const RowsC2RParams<float>& p, const RowLine& R, int g, const float2* v) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int n = g + 16 * j;
        if (R.live && 2 * n < p.n_out) *reinterpret_cast<float2*>(p.out + R.out_off + 2 * n) = v[j];
    }
}

}  // namespace rl

#ifdef __CUDACC__
// The x pass's complex-to-real rows (M = 256, n_out <= M reals kept) in registers.
static __global__ void __launch_bounds__(rl::kThreads, 3) reg_rows_c2r_kernel(RowsC2RParams<float> p) {
    __shared__ __align__(16) float2 buf[rl::kRowSlots];
    __shared__ __align__(16) float2 tw_a[256];
    const int tid = threadIdx.x, row = tid / 16, q = tid & 15;
    const rl::RowLine R = rl::row_of(p, blockIdx.x, row);
    float2 v[16];
    rl::stage_row_twiddles(p, tw_a, tid, rl::kThreads);
    rl::c2r_load_b(p, R, q, v);
    dft16<true>(v);
    rl::c2r_write_b(buf, row, q, v);
    __syncthreads();
    rl::c2r_read_a(buf, row, q, v);
    rl::c2r_inv_a(tw_a, q, v);
    rl::c2r_store_a(p, R, q, v);
}

inline int launch_reg_rows_c2r(const RowsC2RParams<float>& p, cudaStream_t stream) {
    if (p.n_rows <= 0) return SG_OK;
    reg_rows_c2r_kernel<<<ceil_div(p.n_rows, rl::kLines), rl::kThreads, 0, stream>>>(p);
    return launch_status("register rows c2r");
}

// One pass over 16 lines per block.  RL_FWD: forward transform, spectrum stored (HIN prunes a
// zero upper input half).  RL_INV: inverse transform of a full spectrum (HOUT keeps the lower
// output half).  RL_CONV: forward, Green's factor, inverse, in registers between the exchanges.
// Three blocks per SM (80 registers): with the packed complex sums the 512-point inverse and
// convolution spill 8 and 16 bytes there, and run faster than at two blocks (256^3 z convolution
// 0.713 -> 0.689 ms, y inverse 0.368 -> 0.354 ms).
template <int N, int MODE, bool HIN, bool HOUT>
__global__ void __launch_bounds__(rl::kThreads, 3) reg_lines_kernel(RegLinesParams p) {
    extern __shared__ __align__(16) float2 rl_buf[];
    float2* tw_a = rl_buf + N * rl::kLines;
    const int tid = threadIdx.x, l = tid & (rl::kLines - 1), q = tid / rl::kLines;
    const rl::Line L = rl::line_of(p, blockIdx.x, l);
    float2 v[rl::Shape<N>::E];
    rl::stage_twiddles<N>(p, tw_a, tid, rl::kThreads);
    if (MODE != RL_CONV && p.prefetch_ahead > 0 && blockIdx.x + p.prefetch_ahead < gridDim.x)
        rl::prefetch_input<N, HIN, MODE == RL_INV>(p, rl::line_of(p, blockIdx.x + p.prefetch_ahead, l), q);
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
    if (N == 512) SG_RL_PICK(512)
    if (N == 256) SG_RL_PICK(256)
#undef SG_RL_PICK
    return SG_ERR_UNSUPPORTED;
}
#endif

}  // namespace sg
