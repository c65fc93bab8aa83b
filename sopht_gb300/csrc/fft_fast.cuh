// Size-specialised FFT kernels (compile-time length N) for the common extents.
//
// Same passes and parameter structs as fft.cuh, but every transform length,
// radix schedule, stride and butterfly count is a compile-time constant, so
// index arithmetic folds away and all loops unroll.  Layout in shared memory
// is point-major / line-minor with an odd line pitch LS = W + 1 (in complex
// elements): consecutive threads of a stage touch consecutive lines, and the
// row kernels' coalesced loads (consecutive points of one row) hit distinct
// banks.  Each stage is in place: a thread reads its E = N W / NT elements into
// registers, the block synchronises, and the thread writes its butterfly
// outputs back -- one buffer, so twice the resident blocks of a ping-pong.
#pragma once

#include "fft.cuh"

namespace sg {

// ------------------------------------------------------ compile-time schedule
__host__ __device__ constexpr int sched_count(int n) {
    int c = 0;
    while (n % 8 == 0) { n /= 8; ++c; }
    while (n % 4 == 0) { n /= 4; ++c; }
    while (n % 2 == 0) { n /= 2; ++c; }
    while (n % 3 == 0) { n /= 3; ++c; }
    return n == 1 ? c : -1;
}
__host__ __device__ constexpr int sched_radix(int n, int s) {
    int c = 0;
    while (n % 8 == 0) { if (c++ == s) return 8; n /= 8; }
    while (n % 4 == 0) { if (c++ == s) return 4; n /= 4; }
    while (n % 2 == 0) { if (c++ == s) return 2; n /= 2; }
    while (n % 3 == 0) { if (c++ == s) return 3; n /= 3; }
    return 1;
}
__host__ __device__ constexpr int sched_ns(int n, int s) {
    int p = 1;
    for (int i = 0; i < s; ++i) p *= sched_radix(n, i);
    return p;
}

// Per-length launch shape: W lines per block, NT threads, E elements per thread.
template <int N> struct FastShape;
#define SG_FAST_SHAPE(NN, WW, NTT)                                          \
    template <> struct FastShape<NN> {                                     \
        static constexpr int W = WW, NT = NTT, E = NN * WW / NTT, LS = WW + 1; \
    };
SG_FAST_SHAPE(64, 32, 128)
SG_FAST_SHAPE(128, 16, 128)
SG_FAST_SHAPE(256, 16, 256)
SG_FAST_SHAPE(512, 16, 512)
SG_FAST_SHAPE(1024, 8, 512)
SG_FAST_SHAPE(192, 16, 128)
SG_FAST_SHAPE(384, 16, 256)
SG_FAST_SHAPE(768, 8, 256)
#undef SG_FAST_SHAPE

inline bool fast_length(int n) {
    switch (n) {
        case 64: case 128: case 256: case 512: case 1024: case 192: case 384: case 768: return true;
        default: return false;
    }
}

template <int N, int S, int NS, bool INV, int W, int LS, int NT, typename C>
__device__ __forceinline__ void fast_stage(C* buf, const C* __restrict__ tw, int tid) {
    constexpr int R = sched_radix(N, S);
    constexpr int NB = N / R;
    constexpr int TOT = NB * W;
    static_assert(TOT % NT == 0, "butterflies must divide evenly over the block");
    constexpr int PER = TOT / NT;
    constexpr int TSTRIDE = N / (NS * R);
    C v[PER][R];
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int t = tid + b * NT;
        const int line = t % W, j = t / W;
#pragma unroll
        for (int r = 0; r < R; ++r) v[b][r] = buf[(j + r * NB) * LS + line];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int t = tid + b * NT;
        const int line = t % W, j = t / W;
        const int k = j % NS;
        if (NS > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                C w = tw[r * k * TSTRIDE];
                if (INV) w.y = -w.y;
                v[b][r] = cmul(v[b][r], w);
            }
        }
        dft_r<R, INV>(v[b]);
        const int base = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) buf[(base + r * NS) * LS + line] = v[b][r];
    }
    __syncthreads();
}

template <int N, int S, int NS, bool INV, int W, int LS, int NT, typename C>
__device__ __forceinline__ void fast_stages(C* buf, const C* __restrict__ tw, int tid) {
    if constexpr (S < sched_count(N)) {
        fast_stage<N, S, NS, INV, W, LS, NT>(buf, tw, tid);
        fast_stages<N, S + 1, NS * sched_radix(N, S), INV, W, LS, NT>(buf, tw, tid);
    }
}

// Whole in-place transform of the W lines in `buf` (ends synchronised).
template <int N, bool INV, typename C>
__device__ __forceinline__ void fast_fft(C* buf, const C* __restrict__ tw, int tid) {
    using S = FastShape<N>;
    fast_stages<N, 0, 1, INV, S::W, S::LS, S::NT>(buf, tw, tid);
}

// ----------------------------------------------------------- strided lines
template <typename T, int N, int MODE>
__global__ void __launch_bounds__(FastShape<N>::NT) fast_lines_kernel(LinesParams<T> p) {
    using C = cplx_t<T>;
    using S = FastShape<N>;
    constexpr int W = S::W, LS = S::LS, NT = S::NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* buf = reinterpret_cast<C*>(smem_raw);
    const int tid = threadIdx.x;
    const int chunks = (p.inner + W - 1) / W;
    const int outer = blockIdx.x / chunks;
    const int c0 = (blockIdx.x % chunks) * W;
    const int wcount = min(W, p.inner - c0);
    const C* src = p.in + (int64_t)outer * p.outer_stride + c0;
    constexpr int PER = N * W / NT;
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int e = tid + b * NT;
        const int pt = e / W, w = e % W;
        C v = cmake<C>(T(0), T(0));
        if (pt < p.n_in && w < wcount) v = src[(int64_t)pt * p.line_stride + w];
        buf[pt * LS + w] = v;
    }
    __syncthreads();
    if (MODE == LINE_INV) {
        fast_fft<N, true>(buf, p.tw, tid);
    } else {
        fast_fft<N, false>(buf, p.tw, tid);
        if (MODE == LINE_CONV) {
#pragma unroll
            for (int b = 0; b < PER; ++b) {
                const int e = tid + b * NT;
                const int k = e / W, w = e % W;
                const int ks = min(k, N - k);
                const T gv = (w < wcount) ? p.g.at(ks, c0 + w) : T(0);
                buf[k * LS + w] = cscale(buf[k * LS + w], gv);
            }
            __syncthreads();
            fast_fft<N, true>(buf, p.tw, tid);
        }
    }
    C* dst = p.out + (int64_t)outer * p.outer_stride + c0;
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int e = tid + b * NT;
        const int pt = e / W, w = e % W;
        if (pt < p.n_out && w < wcount) dst[(int64_t)pt * p.line_stride + w] = buf[pt * LS + w];
    }
}

// -------------------------------------------------------------- row kernels
// Rows of the x axis: W rows per block, element (row r, point n) at buf[n*LS + r].

template <typename T, int M>
__device__ __forceinline__ void r2c_post_store(const cplx_t<T>* buf, const cplx_t<T>* __restrict__ tw_l,
                                               cplx_t<T>* out, const RowMap& map, int row0, int n_rows,
                                               int tid) {
    using C = cplx_t<T>;
    using S = FastShape<M>;
    constexpr int W = S::W, LS = S::LS, NT = S::NT;
    // each row emits M + 1 bins; threads walk bins of one row (coalesced store)
    for (int e = tid; e < W * (M + 1); e += NT) {
        const int r = e / (M + 1), k = e % (M + 1);
        const int q = row0 + r;
        if (q >= n_rows) continue;
        const C zk = buf[(k == M ? 0 : k) * LS + r];
        const C zc = cconj(buf[(k == 0 ? 0 : M - k) * LS + r]);
        const C w = tw_l[k];
        const C s = cadd(zk, zc);
        const C wd = cmul(w, csub(zk, zc));
        out[map.offset(q) + k] = cmake<C>(T(0.5) * (s.x + wd.y), T(0.5) * (s.y - wd.x));
    }
}

template <typename T, int M>
__global__ void __launch_bounds__(FastShape<M>::NT) fast_rows_r2c_kernel(RowsR2CParams<T> p) {
    using C = cplx_t<T>;
    using S = FastShape<M>;
    constexpr int W = S::W, LS = S::LS, NT = S::NT, PER = M * W / NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* buf = reinterpret_cast<C*>(smem_raw);
    const int tid = threadIdx.x;
    const int row0 = blockIdx.x * W;
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int e = tid + b * NT;
        const int r = e / M, n = e % M;
        const int q = row0 + r;
        C z = cmake<C>(T(0), T(0));
        if (q < p.n_rows) {
            const T* src = p.in + p.in_map.offset(q);
            if (2 * n + 1 < p.n_in) z = *reinterpret_cast<const C*>(src + 2 * n);
            else if (2 * n < p.n_in) z.x = src[2 * n];
        }
        buf[n * LS + r] = z;
    }
    __syncthreads();
    fast_fft<M, false>(buf, p.tw_m, tid);
    r2c_post_store<T, M>(buf, p.tw_l, p.out, p.out_map, row0, p.n_rows, tid);
}

template <typename T, int M>
__global__ void __launch_bounds__(FastShape<M>::NT) fast_rows_c2r_kernel(RowsC2RParams<T> p) {
    using C = cplx_t<T>;
    using S = FastShape<M>;
    constexpr int W = S::W, LS = S::LS, NT = S::NT, PER = M * W / NT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* buf = reinterpret_cast<C*>(smem_raw);
    const int tid = threadIdx.x;
    const int row0 = blockIdx.x * W;
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int e = tid + b * NT;
        const int r = e / M, k = e % M;
        const int q = row0 + r;
        C Zk = cmake<C>(T(0), T(0));
        if (q < p.n_rows) {
            const C* src = p.in + p.in_map.offset(q);
            C xk = src[k];
            C xm = src[M - k];
            if (k == 0) { xk.y = T(0); xm.y = T(0); }
            const C xc = cconj(xm);
            C w = p.tw_l[k];
            w.y = -w.y;
            const C s = cadd(xk, xc);
            const C wd = cmul(w, csub(xk, xc));
            Zk = cmake<C>(s.x - wd.y, s.y + wd.x);
        }
        buf[k * LS + r] = Zk;
    }
    __syncthreads();
    fast_fft<M, true>(buf, p.tw_m, tid);
    // n_out real points = n_out/2 complex values per row (n_out even)
    const int half = p.n_out >> 1;
    for (int e = tid; e < W * half; e += NT) {
        const int r = e / half, n = e % half;
        const int q = row0 + r;
        if (q >= p.n_rows) continue;
        *reinterpret_cast<C*>(p.out + p.out_map.offset(q) + 2 * n) = buf[n * LS + r];
    }
}

// ------------------------------------------------------------- dispatch
template <int N> inline size_t fast_smem_bytes(int esz) { return (size_t)N * FastShape<N>::LS * esz; }

template <typename T, int N>
int launch_fast_rows_r2c(const RowsR2CParams<T>& p, cudaStream_t stream) {
    const size_t smem = fast_smem_bytes<N>(sizeof(cplx_t<T>));
    auto kern = fast_rows_r2c_kernel<T, N>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "fast rows_r2c smem attribute"));
    kern<<<ceil_div(p.n_rows, FastShape<N>::W), FastShape<N>::NT, smem, stream>>>(p);
    return launch_status("fast rows_r2c");
}

template <typename T, int N>
int launch_fast_rows_c2r(const RowsC2RParams<T>& p, cudaStream_t stream) {
    const size_t smem = fast_smem_bytes<N>(sizeof(cplx_t<T>));
    auto kern = fast_rows_c2r_kernel<T, N>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "fast rows_c2r smem attribute"));
    kern<<<ceil_div(p.n_rows, FastShape<N>::W), FastShape<N>::NT, smem, stream>>>(p);
    return launch_status("fast rows_c2r");
}

template <typename T, int N, int MODE>
int launch_fast_lines(LinesParams<T> p, cudaStream_t stream) {
    const size_t smem = fast_smem_bytes<N>(sizeof(cplx_t<T>));
    auto kern = fast_lines_kernel<T, N, MODE>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "fast lines smem attribute"));
    p.W = FastShape<N>::W;
    const long long blocks = (long long)p.n_outer * ((p.inner + p.W - 1) / p.W);
    SG_REQUIRE(blocks < (1LL << 31), SG_ERR_SHAPE, "lines: too many blocks (%lld)", blocks);
    kern<<<(unsigned)blocks, FastShape<N>::NT, smem, stream>>>(p);
    return launch_status("fast lines");
}

#define SG_FAST_SWITCH(N_, CALL)                                                  \
    switch (N_) {                                                                 \
        case 64: return CALL(64);                                                 \
        case 128: return CALL(128);                                               \
        case 256: return CALL(256);                                               \
        case 512: return CALL(512);                                               \
        case 1024: return CALL(1024);                                             \
        case 192: return CALL(192);                                               \
        case 384: return CALL(384);                                               \
        case 768: return CALL(768);                                               \
        default: break;                                                           \
    }

template <typename T>
int launch_rows_r2c(RowsR2CParams<T> p, cudaStream_t stream) {
#define SG_CALL(NN) launch_fast_rows_r2c<T, NN>(p, stream)
    SG_FAST_SWITCH(p.st.n, SG_CALL)
#undef SG_CALL
    return launch_rows_r2c_generic<T>(p, stream);
}

template <typename T>
int launch_rows_c2r(RowsC2RParams<T> p, cudaStream_t stream) {
    if (p.n_out % 2 == 0) {
#define SG_CALL(NN) launch_fast_rows_c2r<T, NN>(p, stream)
        SG_FAST_SWITCH(p.st.n, SG_CALL)
#undef SG_CALL
    }
    return launch_rows_c2r_generic<T>(p, stream);
}

template <typename T, int MODE>
int launch_lines(LinesParams<T> p, cudaStream_t stream) {
#define SG_CALL(NN) launch_fast_lines<T, NN, MODE>(p, stream)
    SG_FAST_SWITCH(p.st.n, SG_CALL)
#undef SG_CALL
    return launch_lines_generic<T, MODE>(p, stream);
}

}  // namespace sg
