// Size-specialised FFT kernels (compile-time length N and lines per block W).
//
// Same passes and parameter structs as fft.cuh, but the transform length, the
// radix schedule, strides and butterfly counts are compile-time constants, so
// index arithmetic folds away and all loops unroll.
//  * Shared layout: point-major / line-minor with an odd line pitch LS = W + 1
//    (in complex elements).  Consecutive threads of a stage touch consecutive
//    lines, and the row kernels' coalesced loads (consecutive points of one
//    row) hit distinct banks.
//  * Stages are in place: a thread reads its E = N W / NT elements into
//    registers, the block synchronises, and the thread writes its butterfly
//    outputs back (one buffer instead of a ping-pong pair).
//  * Twiddles are staged into shared memory once per block.
//  * Per-row metadata of the row kernels (global offsets, boundary factors) is
//    computed once per block, not per element.
//  * Each length has a wide shape (16 lines, 128-byte runs for the strided
//    passes) and a narrow one (1-8 lines) chosen when the wide shape would not
//    give every SM at least two blocks.
#pragma once

#include "fft.cuh"

namespace sg {

// ------------------------------------------------------ compile-time schedule
// Radix schedule of a length: 16s first when R16 (fewer stages for 128, 256
// and 1024), then 8s, 4s, 2s, 3s.
__host__ __device__ constexpr int sched_count(int n, bool r16 = false) {
    int c = 0;
    while (r16 && n % 16 == 0) { n /= 16; ++c; }
    while (n % 8 == 0) { n /= 8; ++c; }
    while (n % 4 == 0) { n /= 4; ++c; }
    while (n % 2 == 0) { n /= 2; ++c; }
    while (n % 3 == 0) { n /= 3; ++c; }
    return n == 1 ? c : -1;
}
__host__ __device__ constexpr int sched_radix(int n, int s, bool r16 = false) {
    int c = 0;
    while (r16 && n % 16 == 0) { if (c++ == s) return 16; n /= 16; }
    while (n % 8 == 0) { if (c++ == s) return 8; n /= 8; }
    while (n % 4 == 0) { if (c++ == s) return 4; n /= 4; }
    while (n % 2 == 0) { if (c++ == s) return 2; n /= 2; }
    while (n % 3 == 0) { if (c++ == s) return 3; n /= 3; }
    return 1;
}

// E complex elements per thread: a multiple of every radix of the schedule
template <int N> struct FastElems {
    static constexpr int E = (N % 3 == 0) ? 24 : 16;
};


template <int N, int W, int E_ = FastElems<N>::E> struct FastShape {
    static constexpr int E = E_;
    static constexpr int NT = N * W / E;
    static constexpr int LS = W + 1;
    static_assert(NT >= 32 && NT <= 1024 && NT % 32 == 0, "block size must be whole warps");
};

// wide / narrow line counts per length
template <int N> struct FastWidth;
#define SG_FAST_WIDTH(NN, WIDE, NARROW) \
    template <> struct FastWidth<NN> { static constexpr int wide = WIDE, narrow = NARROW; };
SG_FAST_WIDTH(64, 32, 8)
SG_FAST_WIDTH(128, 16, 4)
SG_FAST_WIDTH(256, 16, 2)
SG_FAST_WIDTH(512, 16, 2)
SG_FAST_WIDTH(1024, 8, 1)
SG_FAST_WIDTH(192, 16, 4)
SG_FAST_WIDTH(384, 16, 2)
SG_FAST_WIDTH(768, 8, 1)
#undef SG_FAST_WIDTH

// Elements per thread of the standalone kernels (E must be a multiple of every
// radix of N's schedule; radix-3 lengths keep 24).  Measured on GB300: the row
// kernels (x R2C, flow load, x C2R) run faster with E = 8 (twice the threads,
// half the registers) at every power-of-two length; the strided line kernels
// run faster with E = 8 only at their narrow width, and with E = 16 at the
// wide one, where E = 8 lost 10-15 % at N = 256 and 512.
template <int N, int W> struct FastPickRows {
    static constexpr int E = (N % 3 == 0) ? 24 : ((N * W / 8 <= 1024) ? 8 : 16);
};
template <int N, int W> struct FastPickLines {
    static constexpr int E = (N % 3 == 0) ? 24 : ((W == FastWidth<N>::narrow && N * W / 8 >= 32) ? 8 : 16);
};

// Length-R DFT of inputs whose upper half (v[R/2 .. R-1]) is zero, for the
// even radices.  Same operations as dft_r without the additions of zero, so
// every non-zero result is bitwise the same.
template <int R, bool INV, typename C> __device__ __forceinline__ void dft_r_half_in(C* v) {
    auto rot = [](C e) { return INV ? cmake<C>(-e.y, e.x) : cmake<C>(e.y, -e.x); };  // dft4's d
    if constexpr (R == 16) {
        dft16<INV, true>(v);
    } else if constexpr (R == 2) {
        v[1] = v[0];
    } else if constexpr (R == 4) {
        const C x0 = v[0], x1 = v[1];
        v[0] = cadd(x0, x1);
        v[1] = cadd(x0, rot(x1));
        v[2] = csub(x0, x1);
        v[3] = csub(x0, rot(x1));
    } else {
        static_assert(R == 8, "half-input DFT for radices 2, 4, 8, 16");
        using T = typename Cx<C>::T;
        const C e0 = v[0], e1 = v[2], o0 = v[1], o1 = v[3];
        C E0 = cadd(e0, e1), E1 = cadd(e0, rot(e1)), E2 = csub(e0, e1), E3 = csub(e0, rot(e1));
        C O0 = cadd(o0, o1), O1 = cadd(o0, rot(o1)), O2 = csub(o0, o1), O3 = csub(o0, rot(o1));
        const T r = T(0.70710678118654752440);
        const C w1 = INV ? cmake<C>(r, r) : cmake<C>(r, -r);
        const C w3 = INV ? cmake<C>(-r, r) : cmake<C>(-r, -r);
        O1 = cmul(O1, w1);
        O2 = INV ? cmake<C>(-O2.y, O2.x) : cmake<C>(O2.y, -O2.x);
        O3 = cmul(O3, w3);
        v[0] = cadd(E0, O0); v[4] = csub(E0, O0);
        v[1] = cadd(E1, O1); v[5] = csub(E1, O1);
        v[2] = cadd(E2, O2); v[6] = csub(E2, O2);
        v[3] = cadd(E3, O3); v[7] = csub(E3, O3);
    }
}

// v[r] *= w^r, r = 1 .. R-1, with w = tw[step] (conjugated for the inverse).
// The powers of two are read from the table and the other powers are formed
// as products of at most two of them, each used as soon as it exists: a
// radix-8 butterfly reads 3 twiddles (not 7) and a radix-16 one 4 (not 15).
// In the line passes the twiddle reads had been as many shared-memory
// accesses as the butterfly data itself.
template <int R, bool INV, typename C>
__device__ __forceinline__ void apply_stage_twiddles(C* v, const C* tw, int step) {
    auto ld = [&](int r) {
        C w = tw[r * step];
        if (INV) w.y = -w.y;
        return w;
    };
    if constexpr (R == 3 || R == 5 || R == 7) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[r] = cmul(v[r], ld(r));
    } else {
        const C w1 = ld(1);
        v[1] = cmul(v[1], w1);
        if constexpr (R >= 4) {
            const C w2 = ld(2);
            v[2] = cmul(v[2], w2);
            const C w3 = cmul(w2, w1);
            v[3] = cmul(v[3], w3);
            if constexpr (R >= 8) {
                const C w4 = ld(4);
                v[4] = cmul(v[4], w4);
                v[5] = cmul(v[5], cmul(w4, w1));
                v[6] = cmul(v[6], cmul(w4, w2));
                v[7] = cmul(v[7], cmul(w4, w3));
                if constexpr (R >= 16) {
                    const C w8 = ld(8);
                    v[8] = cmul(v[8], w8);
                    v[9] = cmul(v[9], cmul(w8, w1));
                    v[10] = cmul(v[10], cmul(w8, w2));
                    v[11] = cmul(v[11], cmul(w8, w3));
                    const C w12 = cmul(w8, w4);
                    v[12] = cmul(v[12], w12);
                    v[13] = cmul(v[13], cmul(w12, w1));
                    v[14] = cmul(v[14], cmul(w12, w2));
                    v[15] = cmul(v[15], cmul(w12, w3));
                }
            }
        }
    }
}

struct IdentityPost {
    template <typename C> __device__ __forceinline__ C operator()(int, C v) const { return v; }
};

// The first stage reads points j + r N/R: with HIN (points N/2 .. N-1 zero,
// an even first radix) the upper half is neither read nor summed.  The last
// stage writes point base + r N/R: with HOUT (only points < N/2 wanted, an even
// last radix) the upper half is not written.  `post(k, v)` is applied to every
// value the last stage writes (point k of the thread's line).
template <int N, bool R16 = false> struct FastEnds {
    static constexpr bool first_even = sched_radix(N, 0, R16) % 2 == 0;
    static constexpr bool last_even = sched_radix(N, sched_count(N, R16) - 1, R16) % 2 == 0;
};

template <int N, int S, int NS, bool INV, int W, int LS, int NT, bool HIN, bool HOUT, bool R16, bool TWP,
          typename C, typename Post>
__device__ __forceinline__ void fast_stage(C* buf, const C* tw, int tid, const Post& post) {
    constexpr int R = sched_radix(N, S, R16);
    constexpr int NB = N / R;
    constexpr int TOT = NB * W;
    static_assert(TOT % NT == 0, "butterflies must divide evenly over the block");
    constexpr int PER = TOT / NT;
    constexpr int TSTRIDE = N / (NS * R);
    constexpr bool LAST = S == sched_count(N, R16) - 1;
    constexpr bool SKIP_IN = HIN && S == 0 && R % 2 == 0;
    constexpr bool SKIP_OUT = HOUT && LAST && R % 2 == 0;
    C v[PER][R];
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int t = tid + b * NT;
        const int line = t % W, j = t / W;
#pragma unroll
        for (int r = 0; r < (SKIP_IN ? R / 2 : R); ++r) v[b][r] = buf[(j + r * NB) * LS + line];
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int t = tid + b * NT;
        const int line = t % W, j = t / W;
        const int k = j % NS;
        if (NS > 1) {
            if constexpr (TWP) {
                apply_stage_twiddles<R, INV>(v[b], tw, k * TSTRIDE);
            } else {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    C w = tw[r * k * TSTRIDE];
                    if (INV) w.y = -w.y;
                    v[b][r] = cmul(v[b][r], w);
                }
            }
        }
        if constexpr (SKIP_IN) dft_r_half_in<R, INV>(v[b]);
        else dft_r<R, INV>(v[b]);
        const int base = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < (SKIP_OUT ? R / 2 : R); ++r) {
            C o = v[b][r];
            if constexpr (LAST) o = post(base + r * NS, o);
            buf[(base + r * NS) * LS + line] = o;
        }
    }
    __syncthreads();
}

template <int N, int S, int NS, bool INV, int W, int LS, int NT, bool HIN, bool HOUT, bool R16, bool TWP,
          typename C, typename Post>
__device__ __forceinline__ void fast_stages(C* buf, const C* tw, int tid, const Post& post) {
    if constexpr (S < sched_count(N, R16)) {
        fast_stage<N, S, NS, INV, W, LS, NT, HIN, HOUT, R16, TWP>(buf, tw, tid, post);
        fast_stages<N, S + 1, NS * sched_radix(N, S, R16), INV, W, LS, NT, HIN, HOUT, R16, TWP>(buf, tw, tid, post);
    }
}

// Whole in-place transform of the W lines in `buf` (ends synchronised).  R16
// selects the schedule with radix-16 stages (E a multiple of 16).  TWP forms
// the stage twiddles from their powers of two (apply_stage_twiddles): measured
// on GB300 it helps the shared-memory-bound line passes and slows the row
// passes, which read the whole table.
template <int N, int W, bool INV, int E = FastElems<N>::E, bool HIN = false, bool HOUT = false, bool R16 = false,
          bool TWP = false, typename C, typename Post = IdentityPost>
__device__ __forceinline__ void fast_fft(C* buf, const C* tw, int tid, const Post& post = Post()) {
    using S = FastShape<N, W, E>;
    static_assert(!R16 || E % 16 == 0, "radix-16 stages need 16 elements per thread");
    fast_stages<N, 0, 1, INV, W, S::LS, S::NT, HIN && FastEnds<N, R16>::first_even,
                HOUT && FastEnds<N, R16>::last_even, R16, TWP>(buf, tw, tid, post);
}

// Line kernels with 16 elements per thread take radix-16 stages where that
// removes a stage (N = 128, 256, 1024).  The batched 2D step and the 2D
// single-instance column pass keep the radix-8 schedule (the same rounding
// in both, so they stay bitwise equal).
template <int N, int E> struct FastR16 {
    static constexpr bool value =
        E % 16 == 0 && N % 3 != 0 && sched_count(N, true) < sched_count(N, false);
};

template <typename C>
__device__ __forceinline__ void stage_table(C* dst, const C* __restrict__ src, int n, int tid, int nt) {
    for (int i = tid; i < n; i += nt) dst[i] = src[i];
}

// ----------------------------------------------------------- strided lines
// HIN: the points n_in .. N-1 of each line are zero with n_in <= N/2 (the
// zero padding of the doubled domain), so the upper half is neither loaded nor
// transformed.  HOUT: only the points < n_out <= N/2 are stored (the crop), so
// the inverse transform's last stage computes only those.  In LINE_CONV the
// Green's factor multiplies the forward transform's last-stage outputs in
// registers.
// stage_tw = false: the block staged this length's twiddles for an earlier
// work item (persistent batched kernels) and they are still in shared memory.
template <typename T, int N, int W, int MODE, int E = FastElems<N>::E, bool HIN = false, bool HOUT = false,
          bool R16 = false>
__device__ __forceinline__ void fast_lines_body(const LinesParams<T>& p, int bid, unsigned char* smem_raw,
                                                bool stage_tw = true) {
    using C = cplx_t<T>;
    using S = FastShape<N, W, E>;
    constexpr int LS = S::LS, NT = S::NT, PER = N * W / NT;
    constexpr bool SKIP_LOAD = HIN && FastEnds<N, R16>::first_even;
    C* buf = reinterpret_cast<C*>(smem_raw);
    C* tw = buf + N * LS;
    const int tid = threadIdx.x;
    const int chunks = (p.inner + W - 1) / W;
    const int outer = bid / chunks;
    const int c0 = (bid % chunks) * W;
    const int wcount = min(W, p.inner - c0);
    if (stage_tw) stage_table(tw, p.tw, N, tid, NT);
    const C* src = p.in + (int64_t)outer * p.outer_stride + c0;
#pragma unroll
    for (int b = 0; b < (SKIP_LOAD ? PER / 2 : PER); ++b) {
        const int e = tid + b * NT;
        const int pt = e / W, w = e % W;
        C v = cmake<C>(T(0), T(0));
        if (pt < p.n_in && w < wcount) v = src[(int64_t)pt * p.line_stride + w];
        buf[pt * LS + w] = v;
    }
    __syncthreads();
    if (MODE == LINE_INV) {
        fast_fft<N, W, true, E, false, HOUT, R16, true>(buf, tw, tid);
    } else if (MODE == LINE_FWD) {
        fast_fft<N, W, false, E, HIN, false, R16, true>(buf, tw, tid);
    } else {
        // every element a thread touches has the same line w, so the table row
        // of that line is computed once
        const int w = tid % W;
        int64_t gbase = 0;
        if (w < wcount) {
            const int inner = c0 + w;
            const int m = inner / p.g.inner_div;
            const int kx = inner - m * p.g.inner_div;
            const int ms = p.g.m_mod > 0 ? min(m, p.g.m_mod - m) : 0;
            gbase = (int64_t)ms * p.g.m_stride + kx;
        }
        const T* table = p.g.table;
        const int64_t k_stride = p.g.k_stride;
        const bool live = w < wcount;
        auto green = [&](int k, C v) {
            const int ks = min(k, N - k);
            const T gv = live ? table[(int64_t)ks * k_stride + gbase] : T(0);
            return cscale(v, gv);
        };
        fast_fft<N, W, false, E, HIN, false, R16, true>(buf, tw, tid, green);
        fast_fft<N, W, true, E, false, HOUT, R16, true>(buf, tw, tid);
    }
    C* dst = p.out + (int64_t)outer * p.outer_stride + c0;
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int e = tid + b * NT;
        const int pt = e / W, w = e % W;
        if (pt < p.n_out && w < wcount) dst[(int64_t)pt * p.line_stride + w] = buf[pt * LS + w];
    }
}

// Occupancy of the fp32 line kernels with E <= 16: registers capped at 64 per
// thread (two 512-thread or four 256-thread blocks per SM), and every FFT
// kernel asks for the largest shared-memory carveout.  Measured on GB300 the
// 512-thread convolution and inverse passes otherwise run one block per SM
// (256^3 z convolution 1.26 -> 1.14 ms, y IFFT 0.47 -> 0.43 ms); giving the
// carveout to only some of the step's FFT kernels was slower than giving it to
// all of them (the SMs reconfigure shared memory between kernels).  fp64 and
// E = 24 kernels keep their registers: a cap would spill them.
template <typename T, int NT, int E> struct FastOccupancy {
    static constexpr int min_blocks =
        (sizeof(T) == 8 || E > 16) ? 1 : (NT >= 512 ? 2048 / NT / 2 : (NT >= 256 ? 4 : 1));
};

template <typename K> inline int fast_max_carveout(K kern, const char* what) {
    return cuda_status(
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared),
        what);
}

template <typename T, int N, int W, int MODE, int E, bool HIN, bool HOUT>
__global__ void __launch_bounds__(FastShape<N, W, E>::NT, FastOccupancy<T, FastShape<N, W, E>::NT, E>::min_blocks)
    fast_lines_kernel(LinesParams<T> p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    fast_lines_body<T, N, W, MODE, E, HIN, HOUT, FastR16<N, E>::value>(p, blockIdx.x, smem_raw);
}

// -------------------------------------------------------------- row kernels
// Rows of the x axis: W rows per block, element (row r, point n) at buf[n*LS + r].
// Shared: buf [M][LS], twiddles tw_m [M] and tw_l [M + 1], row offsets [2 W].

template <int M, int W> struct RowSmem {
    static constexpr int LS = W + 1;
    template <typename C> static constexpr size_t bytes() {
        return sizeof(C) * ((size_t)M * LS + M + (M + 1)) + sizeof(int64_t) * 2 * W + 16;
    }
};

template <typename T, int M, int W, int E = FastElems<M>::E>
__device__ __forceinline__ void r2c_post_store(const cplx_t<T>* buf, const cplx_t<T>* tw_l, cplx_t<T>* out,
                                               const int64_t* out_off, int row0, int n_rows, int tid) {
    using C = cplx_t<T>;
    using S = FastShape<M, W, E>;
    constexpr int LS = S::LS, NT = S::NT;
    // each row emits M + 1 bins; threads walk bins of one row (coalesced store)
    for (int e = tid; e < W * (M + 1); e += NT) {
        const int r = e / (M + 1), k = e - r * (M + 1);
        if (row0 + r >= n_rows) continue;
        const C zk = buf[(k == M ? 0 : k) * LS + r];
        const C zc = cconj(buf[(k == 0 ? 0 : M - k) * LS + r]);
        const C w = tw_l[k];
        const C s = cadd(zk, zc);
        const C wd = cmul(w, csub(zk, zc));
        out[out_off[r] + k] = cmake<C>(T(0.5) * (s.x + wd.y), T(0.5) * (s.y - wd.x));
    }
}

// HIN: the row's real input is zero beyond n_in <= M, so the packed complex
// points M/2 .. M-1 are zero and the first stage skips them.
template <typename T, int M, int W, int E = FastElems<M>::E, bool HIN = false>
__device__ __forceinline__ void fast_rows_r2c_body(const RowsR2CParams<T>& p, int bid, unsigned char* smem_raw) {
    using C = cplx_t<T>;
    using S = FastShape<M, W, E>;
    constexpr int LS = S::LS, NT = S::NT, PER = M * W / NT;
    constexpr bool SKIP_LOAD = HIN && FastEnds<M>::first_even;
    C* buf = reinterpret_cast<C*>(smem_raw);
    C* tw_m = buf + M * LS;
    C* tw_l = tw_m + M;
    int64_t* in_off = reinterpret_cast<int64_t*>(
        (reinterpret_cast<uintptr_t>(tw_l + M + 1) + 15) & ~uintptr_t(15));
    int64_t* out_off = in_off + W;
    const int tid = threadIdx.x;
    const int row0 = bid * W;
    if (tid < W) {
        in_off[tid] = p.in_map.offset(row0 + tid);
        out_off[tid] = p.out_map.offset(row0 + tid);
    }
    stage_table(tw_m, p.tw_m, M, tid, NT);
    stage_table(tw_l, p.tw_l, M + 1, tid, NT);
    __syncthreads();
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int e = tid + b * NT;
        const int r = e / M, n = e % M;
        if (SKIP_LOAD && n >= M / 2) continue;
        C z = cmake<C>(T(0), T(0));
        if (row0 + r < p.n_rows) {
            const T* src = p.in + in_off[r];
            if (2 * n + 1 < p.n_in) z = *reinterpret_cast<const C*>(src + 2 * n);
            else if (2 * n < p.n_in) z.x = src[2 * n];
        }
        buf[n * LS + r] = z;
    }
    __syncthreads();
    fast_fft<M, W, false, E, HIN, false>(buf, tw_m, tid);
    r2c_post_store<T, M, W, E>(buf, tw_l, p.out, out_off, row0, p.n_rows, tid);
}

template <typename T, int M, int W, int E, bool HIN>
__global__ void __launch_bounds__(FastShape<M, W, E>::NT) fast_rows_r2c_kernel(RowsR2CParams<T> p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    fast_rows_r2c_body<T, M, W, E, HIN>(p, blockIdx.x, smem_raw);
}

// HOUT: only the first n_out = M real points (M/2 packed complex points) are
// stored, so the inverse transform's last stage computes only those.
template <typename T, int M, int W, int E = FastElems<M>::E, bool HOUT = false>
__device__ __forceinline__ void fast_rows_c2r_body(const RowsC2RParams<T>& p, int bid, unsigned char* smem_raw,
                                                   bool stage_tw = true) {
    using C = cplx_t<T>;
    using S = FastShape<M, W, E>;
    constexpr int LS = S::LS, NT = S::NT, PER = M * W / NT;
    C* buf = reinterpret_cast<C*>(smem_raw);
    C* tw_m = buf + M * LS;
    C* tw_l = tw_m + M;
    int64_t* in_off = reinterpret_cast<int64_t*>(
        (reinterpret_cast<uintptr_t>(tw_l + M + 1) + 15) & ~uintptr_t(15));
    int64_t* out_off = in_off + W;
    const int tid = threadIdx.x;
    const int row0 = bid * W;
    if (tid < W) {
        in_off[tid] = p.in_map.offset(row0 + tid);
        out_off[tid] = p.out_map.offset(row0 + tid);
    }
    if (stage_tw) {
        stage_table(tw_m, p.tw_m, M, tid, NT);
        stage_table(tw_l, p.tw_l, M + 1, tid, NT);
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int e = tid + b * NT;
        const int r = e / M, k = e % M;
        C Zk = cmake<C>(T(0), T(0));
        if (row0 + r < p.n_rows) {
            const C* src = p.in + in_off[r];
            C xk = src[k];
            C xm = src[M - k];
            if (k == 0) { xk.y = T(0); xm.y = T(0); }
            const C xc = cconj(xm);
            C w = tw_l[k];
            w.y = -w.y;
            const C s = cadd(xk, xc);
            const C wd = cmul(w, csub(xk, xc));
            Zk = cmake<C>(s.x - wd.y, s.y + wd.x);
        }
        buf[k * LS + r] = Zk;
    }
    __syncthreads();
    fast_fft<M, W, true, E, false, HOUT>(buf, tw_m, tid);
    // n_out real points = n_out/2 complex values per row (n_out even)
    const int half = p.n_out >> 1;
    for (int e = tid; e < W * half; e += NT) {
        const int r = e / half, n = e - r * half;
        if (row0 + r >= p.n_rows) continue;
        *reinterpret_cast<C*>(p.out + out_off[r] + 2 * n) = buf[n * LS + r];
    }
}

template <typename T, int M, int W, int E, bool HOUT>
__global__ void __launch_bounds__(FastShape<M, W, E>::NT) fast_rows_c2r_kernel(RowsC2RParams<T> p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    fast_rows_c2r_body<T, M, W, E, HOUT>(p, blockIdx.x, smem_raw);
}

// ------------------------------------------------------------- dispatch
inline int fast_pick_width(long long units, int wide, int narrow) {
    // the wide shape when it still gives every SM two blocks, else the narrow one
    return (units + wide - 1) / wide >= 2 * 152 ? wide : narrow;
}

template <typename T, int N, int W>
int launch_fast_rows_r2c(const RowsR2CParams<T>& p, cudaStream_t stream) {
    constexpr int E = FastPickRows<N, W>::E;
    const size_t smem = RowSmem<N, W>::template bytes<cplx_t<T>>();
    // real input zero beyond n_in <= N: the upper half of the packed points is zero
    auto kern = p.n_in <= N ? fast_rows_r2c_kernel<T, N, W, E, true> : fast_rows_r2c_kernel<T, N, W, E, false>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "fast rows_r2c smem attribute"));
    SG_TRY(fast_max_carveout(kern, "fast rows_r2c carveout attribute"));
    kern<<<ceil_div(p.n_rows, W), FastShape<N, W, E>::NT, smem, stream>>>(p);
    return launch_status("fast rows_r2c");
}

template <typename T, int N, int W>
int launch_fast_rows_c2r(const RowsC2RParams<T>& p, cudaStream_t stream) {
    constexpr int E = FastPickRows<N, W>::E;
    const size_t smem = RowSmem<N, W>::template bytes<cplx_t<T>>();
    // cropped output: only n_out <= N real points (N/2 packed points) are stored
    auto kern = p.n_out <= N ? fast_rows_c2r_kernel<T, N, W, E, true> : fast_rows_c2r_kernel<T, N, W, E, false>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "fast rows_c2r smem attribute"));
    SG_TRY(fast_max_carveout(kern, "fast rows_c2r carveout attribute"));
    kern<<<ceil_div(p.n_rows, W), FastShape<N, W, E>::NT, smem, stream>>>(p);
    return launch_status("fast rows_c2r");
}

template <typename T, int N, int W, int MODE>
int launch_fast_lines(LinesParams<T> p, cudaStream_t stream) {
    constexpr int E = FastPickLines<N, W>::E;
    const size_t smem = sizeof(cplx_t<T>) * ((size_t)N * FastShape<N, W, E>::LS + N);
    // zero-padded input (n_in <= N/2) and cropped output (n_out <= N/2) select the pruned transforms
    const bool hin = 2 * p.n_in <= N, hout = 2 * p.n_out <= N;
    auto kern = hin ? (hout ? fast_lines_kernel<T, N, W, MODE, E, true, true>
                            : fast_lines_kernel<T, N, W, MODE, E, true, false>)
                    : (hout ? fast_lines_kernel<T, N, W, MODE, E, false, true>
                            : fast_lines_kernel<T, N, W, MODE, E, false, false>);
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "fast lines smem attribute"));
    SG_TRY(fast_max_carveout(kern, "fast lines carveout attribute"));
    p.W = W;
    const long long blocks = (long long)p.n_outer * ((p.inner + W - 1) / W);
    SG_REQUIRE(blocks < (1LL << 31), SG_ERR_SHAPE, "lines: too many blocks (%lld)", blocks);
    kern<<<(unsigned)blocks, FastShape<N, W, E>::NT, smem, stream>>>(p);
    return launch_status("fast lines");
}

// Calls CALL(N, W) with compile-time N from the runtime length and the wide or
// narrow width for `units` independent lines/rows; falls through otherwise.
#define SG_FAST_DISPATCH(N_, UNITS, CALL)                                                          \
    switch (N_) {                                                                                  \
        case 64: return fast_pick_width(UNITS, 32, 8) == 32 ? CALL(64, 32) : CALL(64, 8);          \
        case 128: return fast_pick_width(UNITS, 16, 4) == 16 ? CALL(128, 16) : CALL(128, 4);       \
        case 256: return fast_pick_width(UNITS, 16, 2) == 16 ? CALL(256, 16) : CALL(256, 2);       \
        case 512: return fast_pick_width(UNITS, 16, 2) == 16 ? CALL(512, 16) : CALL(512, 2);       \
        case 1024: return fast_pick_width(UNITS, 8, 1) == 8 ? CALL(1024, 8) : CALL(1024, 1);       \
        case 192: return fast_pick_width(UNITS, 16, 4) == 16 ? CALL(192, 16) : CALL(192, 4);       \
        case 384: return fast_pick_width(UNITS, 16, 2) == 16 ? CALL(384, 16) : CALL(384, 2);       \
        case 768: return fast_pick_width(UNITS, 8, 1) == 8 ? CALL(768, 8) : CALL(768, 1);          \
        default: break;                                                                            \
    }

template <typename T>
int launch_rows_r2c(RowsR2CParams<T> p, cudaStream_t stream) {
#define SG_CALL(NN, WW) launch_fast_rows_r2c<T, NN, WW>(p, stream)
    SG_FAST_DISPATCH(p.st.n, p.n_rows, SG_CALL)
#undef SG_CALL
    return launch_rows_r2c_generic<T>(p, stream);
}

template <typename T>
int launch_rows_c2r(RowsC2RParams<T> p, cudaStream_t stream) {
    if (p.n_out % 2 == 0) {
#define SG_CALL(NN, WW) launch_fast_rows_c2r<T, NN, WW>(p, stream)
        SG_FAST_DISPATCH(p.st.n, p.n_rows, SG_CALL)
#undef SG_CALL
    }
    return launch_rows_c2r_generic<T>(p, stream);
}

template <typename T, int MODE>
int launch_lines(LinesParams<T> p, cudaStream_t stream) {
    const long long units = (long long)p.n_outer * p.inner;
#define SG_CALL(NN, WW) launch_fast_lines<T, NN, WW, MODE>(p, stream)
    SG_FAST_DISPATCH(p.st.n, units, SG_CALL)
#undef SG_CALL
    return launch_lines_generic<T, MODE>(p, stream);
}

}  // namespace sg
