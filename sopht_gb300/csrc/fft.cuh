// Batched shared-memory FFT kernels for the domain-doubled Poisson solve.
//
// Algorithm: mixed-radix (2, 3, 4, 8) Stockham autosort, decimation in time.
// For a length N = R_1 R_2 ... R_s, stage t reads points j + r N/R (r < R) of
// the previous buffer, multiplies point r by w_{Ns R}^{r (j mod Ns)} (Ns = the
// product of the radices already applied), applies a length-R DFT in registers
// and writes point r to ((j / Ns) Ns R + j mod Ns) + r Ns of the other buffer.
// The output is in natural order.  Twiddles come from a table of
// exp(-2 pi i m / N), m < N, evaluated in double precision on the GPU.
//
// Real transforms of even length L = 2M use the half-length complex transform
// of z[n] = x[2n] + i x[2n+1] with the standard split step:
//   X[k] = (Z[k] + Z*[M-k])/2 - (i/2) e^{-2 pi i k/L} (Z[k] - Z*[M-k]),
// and its inverse  Z[k] = (X[k] + X*[M-k]) + i e^{+2 pi i k/L} (X[k] - X*[M-k]).
//
// Three kernel shapes cover every pass of the solve:
//  * rows_r2c  — contiguous rows, real in (zero padded beyond n_in) -> M+1 bins
//  * lines     — strided lines (points `line_stride` apart), W adjacent lines
//                per block so every global access is a contiguous W-run:
//                forward, inverse, or forward * G * inverse with a crop
//  * rows_c2r  — M+1 bins -> real row, first n_out points kept
#pragma once

#include "common.cuh"

namespace sg {

constexpr int kMaxStages = 24;

struct FFTStages {
    int n;                 // transform length
    int nstages;
    int radix[kMaxStages];
};

// Factor n into radices 8, 4, 2, 3, 5, 7.  Returns false when n has a prime
// factor above 7.
inline bool fft_factor(int n, FFTStages& st) {
    st.n = n;
    st.nstages = 0;
    if (n < 1) return false;
    int m = n;
    while (m % 8 == 0) { st.radix[st.nstages++] = 8; m /= 8; }
    while (m % 4 == 0) { st.radix[st.nstages++] = 4; m /= 4; }
    while (m % 2 == 0) { st.radix[st.nstages++] = 2; m /= 2; }
    while (m % 3 == 0) { st.radix[st.nstages++] = 3; m /= 3; }
    while (m % 5 == 0) { st.radix[st.nstages++] = 5; m /= 5; }
    while (m % 7 == 0) { st.radix[st.nstages++] = 7; m /= 7; }
    if (st.nstages > kMaxStages) return false;
    return m == 1;
}

// ----------------------------------------------------------------- radix DFTs
template <typename C> struct Cx {
    using T = decltype(C::x);
};

template <bool INV, typename C> __host__ __device__ __forceinline__ void dft2(C& a, C& b) {
    C t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV, typename C> __device__ __forceinline__ void dft3(C& a, C& b, C& c) {
    using T = typename Cx<C>::T;
    const T h = T(0.5);
    const T s3 = INV ? T(0.86602540378443864676) : T(-0.86602540378443864676);
    C t = cadd(b, c);
    C d = csub(b, c);
    C m = cmake<C>(a.x - h * t.x, a.y - h * t.y);
    a = cadd(a, t);
    // (+/- i sqrt(3)/2) * d
    C r = cmake<C>(-s3 * d.y, s3 * d.x);
    b = cadd(m, r);
    c = csub(m, r);
}

template <bool INV, typename C> __host__ __device__ __forceinline__ void dft4(C& v0, C& v1, C& v2, C& v3) {
    C a = cadd(v0, v2), b = csub(v0, v2), c = cadd(v1, v3), e = csub(v1, v3);
    // forward: d = -i * e ; inverse: d = +i * e
    C d = INV ? cmake<C>(-e.y, e.x) : cmake<C>(e.y, -e.x);
    v0 = cadd(a, c);
    v1 = cadd(b, d);
    v2 = csub(a, c);
    v3 = csub(b, d);
}

template <bool INV, typename C> __device__ __forceinline__ void dft8(C* v) {
    using T = typename Cx<C>::T;
    C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    const T r = T(0.70710678118654752440);
    // w8^q with w8 = exp(-/+ i pi/4)
    C w1 = INV ? cmake<C>(r, r) : cmake<C>(r, -r);
    C w3 = INV ? cmake<C>(-r, r) : cmake<C>(-r, -r);
    o1 = cmul(o1, w1);
    o2 = INV ? cmake<C>(-o2.y, o2.x) : cmake<C>(o2.y, -o2.x);
    o3 = cmul(o3, w3);
    v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1); v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2); v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3); v[7] = csub(e3, o3);
}

// cos and sin of 2 pi k / R for the prime radices 5 and 7
__host__ __device__ constexpr double root_cos(int R, int k) {
    return R == 5 ? (k == 0 ? 1.0 : k == 1 ? 0.30901699437494745 : k == 2 ? -0.8090169943749473
                     : k == 3 ? -0.8090169943749476 : 0.30901699437494723)
                  : (k == 0 ? 1.0 : k == 1 ? 0.6234898018587336 : k == 2 ? -0.22252093395631434
                     : k == 3 ? -0.900968867902419 : k == 4 ? -0.9009688679024191
                     : k == 5 ? -0.2225209339563146 : 0.6234898018587334);
}
__host__ __device__ constexpr double root_sin(int R, int k) {
    return R == 5 ? (k == 0 ? 0.0 : k == 1 ? 0.9510565162951535 : k == 2 ? 0.5877852522924732
                     : k == 3 ? -0.587785252292473 : -0.9510565162951536)
                  : (k == 0 ? 0.0 : k == 1 ? 0.7818314824680298 : k == 2 ? 0.9749279121818236
                     : k == 3 ? 0.43388373911755823 : k == 4 ? -0.433883739117558
                     : k == 5 ? -0.9749279121818236 : -0.7818314824680299);
}

// Direct length-R DFT for the prime radices (R^2 complex multiply-adds).
template <int R, bool INV, typename C> __device__ __forceinline__ void dft_prime(C* v) {
    using T = typename Cx<C>::T;
    C out[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
        C acc = v[0];
#pragma unroll
        for (int m = 1; m < R; ++m) {
            const int idx = (m * q) % R;
            const T wr = (T)root_cos(R, idx);
            const T wi = INV ? (T)root_sin(R, idx) : -(T)root_sin(R, idx);
            acc = cadd(acc, cmul(v[m], cmake<C>(wr, wi)));
        }
        out[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = out[q];
}

// cos and sin of 2 pi m / 16 for the twiddles inside a 16-point DFT
__host__ __device__ constexpr double w16_cos(int m) {
    return m == 0 ? 1.0 : m == 1 ? 0.92387953251128674 : m == 2 ? 0.70710678118654752 : m == 3 ? 0.38268343236508977
         : m == 4 ? 0.0 : m == 6 ? -0.70710678118654752 : -0.92387953251128674;  // m == 9
}
__host__ __device__ constexpr double w16_sin(int m) {
    return m == 0 ? 0.0 : m == 1 ? 0.38268343236508977 : m == 2 ? 0.70710678118654752 : m == 3 ? 0.92387953251128674
         : m == 4 ? 1.0 : m == 6 ? 0.70710678118654752 : -0.38268343236508977;  // m == 9
}

// 16-point DFT as 4 x 4: DFT-4 over n1 for each n2 (input n = 4 n1 + n2), the
// twiddles w16^(n2 k1), then DFT-4 over n2 (output k = k1 + 4 k2).  HALF_IN:
// inputs 8..15 are zero and the first DFT-4s skip them.
template <bool INV, bool HALF_IN = false, typename C> __host__ __device__ __forceinline__ void dft16(C* v) {
    using T = typename Cx<C>::T;
    C y[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
        if constexpr (HALF_IN) {
            const C x0 = v[n2], x1 = v[n2 + 4];
            const C r1 = INV ? cmake<C>(-x1.y, x1.x) : cmake<C>(x1.y, -x1.x);
            y[n2][0] = cadd(x0, x1);
            y[n2][1] = cadd(x0, r1);
            y[n2][2] = csub(x0, x1);
            y[n2][3] = csub(x0, r1);
        } else {
            y[n2][0] = v[n2];
            y[n2][1] = v[n2 + 4];
            y[n2][2] = v[n2 + 8];
            y[n2][3] = v[n2 + 12];
            dft4<INV>(y[n2][0], y[n2][1], y[n2][2], y[n2][3]);
        }
    }
#pragma unroll
    for (int n2 = 1; n2 < 4; ++n2) {
#pragma unroll
        for (int k1 = 1; k1 < 4; ++k1) {
            const int m = n2 * k1;
            if (m == 4) {
                const C a = y[n2][k1];  // w16^4 = -i (forward), +i (inverse)
                y[n2][k1] = INV ? cmake<C>(-a.y, a.x) : cmake<C>(a.y, -a.x);
            } else {
                const T c = (T)w16_cos(m), sn = (T)w16_sin(m);
                y[n2][k1] = cmul(y[n2][k1], cmake<C>(c, INV ? sn : -sn));
            }
        }
    }
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        C z0 = y[0][k1], z1 = y[1][k1], z2 = y[2][k1], z3 = y[3][k1];
        dft4<INV>(z0, z1, z2, z3);
        v[k1] = z0;
        v[k1 + 4] = z1;
        v[k1 + 8] = z2;
        v[k1 + 12] = z3;
    }
}

template <int R, bool INV, typename C> __device__ __forceinline__ void dft_r(C* v) {
    if constexpr (R == 16) dft16<INV>(v);
    else if constexpr (R == 2) dft2<INV>(v[0], v[1]);
    else if constexpr (R == 3) dft3<INV>(v[0], v[1], v[2]);
    else if constexpr (R == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 5 || R == 7) dft_prime<R, INV>(v);
    else dft8<INV>(v);
}

// One Stockham stage over `nlines` transforms held in shared memory.  Element
// (line l, point p) lives at buf[p * ps + l * ls].  LINES_FAST selects whether
// consecutive threads walk lines (strided layout) or points (row layout).
template <int R, bool INV, bool LINES_FAST, typename C>
__device__ __forceinline__ void stockham_stage(const C* __restrict__ src, C* __restrict__ dst, int N,
                                               int Ns, int nlines, int ps, int ls,
                                               const C* __restrict__ tw) {
    const int nb = N / R;
    const int total = nb * nlines;
    const int tstride = N / (Ns * R);
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int line, j;
        if (LINES_FAST) { line = t % nlines; j = t / nlines; }
        else { j = t % nb; line = t / nb; }
        const int k = j % Ns;
        C v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[(j + r * nb) * ps + line * ls];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                C w = tw[r * k * tstride];
                if (INV) w.y = -w.y;
                v[r] = cmul(v[r], w);
            }
        }
        dft_r<R, INV>(v);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[(base + r * Ns) * ps + line * ls] = v[r];
    }
}

// Full transform; data starts in buf0 and the result pointer is returned
// (buf0 or buf1).  Ends with a __syncthreads().
template <bool INV, bool LINES_FAST, typename C>
__device__ C* fft_smem(C* buf0, C* buf1, const FFTStages& st, int nlines, int ps, int ls,
                       const C* __restrict__ tw) {
    C* src = buf0;
    C* dst = buf1;
    int Ns = 1;
    for (int s = 0; s < st.nstages; ++s) {
        const int R = st.radix[s];
        switch (R) {
            case 2: stockham_stage<2, INV, LINES_FAST>(src, dst, st.n, Ns, nlines, ps, ls, tw); break;
            case 3: stockham_stage<3, INV, LINES_FAST>(src, dst, st.n, Ns, nlines, ps, ls, tw); break;
            case 4: stockham_stage<4, INV, LINES_FAST>(src, dst, st.n, Ns, nlines, ps, ls, tw); break;
            case 5: stockham_stage<5, INV, LINES_FAST>(src, dst, st.n, Ns, nlines, ps, ls, tw); break;
            case 7: stockham_stage<7, INV, LINES_FAST>(src, dst, st.n, Ns, nlines, ps, ls, tw); break;
            default: stockham_stage<8, INV, LINES_FAST>(src, dst, st.n, Ns, nlines, ps, ls, tw); break;
        }
        __syncthreads();
        Ns *= R;
        C* t = src;
        src = dst;
        dst = t;
    }
    return src;
}

// --------------------------------------------------------------- kernels

// Row addressing shared by the row kernels: row q -> (group, slab, row) with
// row = q % rows_per_slab, slab = (q / rows_per_slab) % slabs_per_group and
// group = q / (rows_per_slab * slabs_per_group).  A 2D field is one slab; a 3D
// component is a group of nz slabs.
struct RowMap {
    int rows_per_slab;
    int slabs_per_group;
    int64_t group_stride;  // elements
    int64_t slab_stride;   // elements
    int64_t row_stride;    // elements
    __host__ __device__ __forceinline__ int64_t offset(int q) const {
        const int row = q % rows_per_slab;
        const int sq = q / rows_per_slab;
        const int slab = sq % slabs_per_group;
        const int group = sq / slabs_per_group;
        return (int64_t)group * group_stride + (int64_t)slab * slab_stride + (int64_t)row * row_stride;
    }
};

inline RowMap row_map(int rows_per_slab, int64_t row_stride, int slabs_per_group = 1,
                      int64_t slab_stride = 0, int64_t group_stride = 0) {
    RowMap m;
    m.rows_per_slab = rows_per_slab;
    m.slabs_per_group = slabs_per_group;
    m.group_stride = group_stride;
    m.slab_stride = slab_stride;
    m.row_stride = row_stride;
    return m;
}

template <typename T> struct RowsR2CParams {
    const T* in;
    RowMap in_map;
    int n_in;             // leading real points that are non-zero (<= 2M)
    cplx_t<T>* out;
    RowMap out_map;       // complex elements
    int n_rows;
    FFTStages st;         // length M
    const cplx_t<T>* tw_m;  // exp(-2 pi i m/M)
    const cplx_t<T>* tw_l;  // exp(-2 pi i k/L), k <= M
};

// Real rows of length L = 2M (zero beyond n_in) -> M+1 bins.
template <typename T>
__global__ void __launch_bounds__(256) rows_r2c_kernel(RowsR2CParams<T> p) {
    using C = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = p.st.n;
    const int rows_per_block = blockDim.y;
    C* buf0 = reinterpret_cast<C*>(smem_raw);
    C* buf1 = buf0 + rows_per_block * M;
    const int row0 = blockIdx.x * rows_per_block;
    const int nthr = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int e = tid; e < rows_per_block * M; e += nthr) {
        const int r = e / M, n = e % M;
        const int q = row0 + r;
        C z = cmake<C>(T(0), T(0));
        if (q < p.n_rows) {
            const T* src = p.in + p.in_map.offset(q);
            const int i0 = 2 * n;
            if (i0 < p.n_in) z.x = src[i0];
            if (i0 + 1 < p.n_in) z.y = src[i0 + 1];
        }
        buf0[r * M + n] = z;
    }
    __syncthreads();
    C* Z = fft_smem<false, false>(buf0, buf1, p.st, rows_per_block, 1, M, p.tw_m);
    for (int e = tid; e < rows_per_block * (M + 1); e += nthr) {
        const int r = e / (M + 1), k = e % (M + 1);
        const int q = row0 + r;
        if (q >= p.n_rows) continue;
        const C zk = Z[r * M + (k == M ? 0 : k)];
        const C zc = cconj(Z[r * M + (k == 0 ? 0 : M - k)]);
        const C w = p.tw_l[k];
        const C s = cadd(zk, zc);
        const C d = csub(zk, zc);
        // X = s/2 - (i/2) w d
        const C wd = cmul(w, d);
        C X = cmake<C>(T(0.5) * (s.x + wd.y), T(0.5) * (s.y - wd.x));
        p.out[p.out_map.offset(q) + k] = X;
    }
}

template <typename T> struct RowsC2RParams {
    const cplx_t<T>* in;
    RowMap in_map;
    T* out;
    RowMap out_map;
    int n_out;            // leading real points written
    int n_rows;
    FFTStages st;         // length M
    const cplx_t<T>* tw_m;
    const cplx_t<T>* tw_l;
};

// M+1 bins -> real row of length 2M (unnormalised), first n_out points kept.
template <typename T>
__global__ void __launch_bounds__(256) rows_c2r_kernel(RowsC2RParams<T> p) {
    using C = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = p.st.n;
    const int rows_per_block = blockDim.y;
    C* buf0 = reinterpret_cast<C*>(smem_raw);
    C* buf1 = buf0 + rows_per_block * M;
    const int row0 = blockIdx.x * rows_per_block;
    const int nthr = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int e = tid; e < rows_per_block * M; e += nthr) {
        const int r = e / M, k = e % M;
        const int q = row0 + r;
        C Zk = cmake<C>(T(0), T(0));
        if (q < p.n_rows) {
            const C* src = p.in + p.in_map.offset(q);
            C xk = src[k];
            C xm = src[M - k];
            if (k == 0) { xk.y = T(0); xm.y = T(0); }  // DC and Nyquist bins are real
            const C xc = cconj(xm);
            C w = p.tw_l[k];
            w.y = -w.y;  // exp(+2 pi i k / L)
            const C s = cadd(xk, xc);
            const C wd = cmul(w, csub(xk, xc));
            Zk = cmake<C>(s.x - wd.y, s.y + wd.x);  // s + i * wd
        }
        buf0[r * M + k] = Zk;
    }
    __syncthreads();
    C* z = fft_smem<true, false>(buf0, buf1, p.st, rows_per_block, 1, M, p.tw_m);
    for (int e = tid; e < rows_per_block * p.n_out; e += nthr) {
        const int r = e / p.n_out, i = e % p.n_out;
        const int q = row0 + r;
        if (q >= p.n_rows) continue;
        const C v = z[r * M + (i >> 1)];
        p.out[p.out_map.offset(q) + i] = (i & 1) ? v.y : v.x;
    }
}

enum LineMode { LINE_FWD = 0, LINE_INV = 1, LINE_CONV = 2 };

// Real symmetric Green's table lookup for the convolution mode.  The table is
// indexed [k_s][m_s][kx] with k_s = min(k, N - k) along the transformed axis
// and, for an inner index i = m * inner_div + kx, m_s = min(m, m_mod - m).
template <typename T> struct GreensMap {
    const T* table;
    int64_t k_stride;     // elements per k_s
    int inner_div;        // kx extent (Nx + 1)
    int m_mod;            // 2 * Ny for the 3D z pass (0 when unused)
    int64_t m_stride;     // elements per m_s
    __device__ __forceinline__ T at(int ks, int inner) const {
        const int m = inner / inner_div;
        const int kx = inner - m * inner_div;
        const int ms = m_mod > 0 ? min(m, m_mod - m) : 0;
        return table[(int64_t)ks * k_stride + (int64_t)ms * m_stride + kx];
    }
};

template <typename T> struct LinesParams {
    const cplx_t<T>* in;
    cplx_t<T>* out;       // may alias `in` (each block owns its lines)
    int n_in;             // non-zero leading points
    int n_out;            // points written
    int inner;            // number of adjacent lines (contiguous extent)
    int64_t line_stride;  // elements between consecutive points of a line
    int64_t outer_stride; // elements between outer batches
    int n_outer;
    int W;                // lines per block (adjacent)
    FFTStages st;
    const cplx_t<T>* tw;  // exp(-2 pi i m/N)
    GreensMap<T> g;
};

template <typename T, int MODE>
__global__ void __launch_bounds__(256) lines_kernel(LinesParams<T> p) {
    using C = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = p.st.n;
    const int W = p.W;
    C* buf0 = reinterpret_cast<C*>(smem_raw);
    C* buf1 = buf0 + N * W;
    const int chunks = (p.inner + W - 1) / W;
    const int outer = blockIdx.x / chunks;
    const int c0 = (blockIdx.x % chunks) * W;
    const int wcount = min(W, p.inner - c0);
    const C* src = p.in + (int64_t)outer * p.outer_stride + c0;
    for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
        const int pt = e / W, w = e % W;
        C v = cmake<C>(T(0), T(0));
        if (pt < p.n_in && w < wcount) v = src[(int64_t)pt * p.line_stride + w];
        buf0[e] = v;
    }
    __syncthreads();
    C* res;
    if (MODE == LINE_INV) {
        res = fft_smem<true, true>(buf0, buf1, p.st, W, W, 1, p.tw);
    } else {
        res = fft_smem<false, true>(buf0, buf1, p.st, W, W, 1, p.tw);
        if (MODE == LINE_CONV) {
            for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
                const int k = e / W, w = e % W;
                const int ks = min(k, N - k);
                const T gv = (w < wcount) ? p.g.at(ks, c0 + w) : T(0);
                res[e] = cscale(res[e], gv);
            }
            __syncthreads();
            C* other = (res == buf0) ? buf1 : buf0;
            res = fft_smem<true, true>(res, other, p.st, W, W, 1, p.tw);
        }
    }
    C* dst = p.out + (int64_t)outer * p.outer_stride + c0;
    for (int e = threadIdx.x; e < p.n_out * W; e += blockDim.x) {
        const int pt = e / W, w = e % W;
        if (w < wcount) dst[(int64_t)pt * p.line_stride + w] = res[e];
    }
}

// --------------------------------------------------------- host launchers

inline int rows_per_block_for(int M, int elem_bytes) {
    // two ping-pong buffers of rows_per_block * M complex values, <= 96 KiB
    int rb = 8;
    while (rb > 1 && 2LL * rb * M * elem_bytes > 96 * 1024) rb >>= 1;
    return rb;
}

inline int lines_per_block_for(int N, int elem_bytes) {
    int w = 16;
    while (w > 1 && 2LL * w * N * elem_bytes > 112 * 1024) w >>= 1;
    return w;
}

template <typename T>
int launch_rows_r2c_generic(RowsR2CParams<T> p, cudaStream_t stream) {
    const int esz = sizeof(cplx_t<T>);
    const int rb = rows_per_block_for(p.st.n, esz);
    const size_t smem = 2ull * rb * p.st.n * esz;
    auto kern = rows_r2c_kernel<T>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "rows_r2c smem attribute"));
    dim3 block(256 / rb, rb);
    kern<<<ceil_div(p.n_rows, rb), block, smem, stream>>>(p);
    return launch_status("rows_r2c launch");
}

template <typename T>
int launch_rows_c2r_generic(RowsC2RParams<T> p, cudaStream_t stream) {
    const int esz = sizeof(cplx_t<T>);
    const int rb = rows_per_block_for(p.st.n, esz);
    const size_t smem = 2ull * rb * p.st.n * esz;
    auto kern = rows_c2r_kernel<T>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "rows_c2r smem attribute"));
    dim3 block(256 / rb, rb);
    kern<<<ceil_div(p.n_rows, rb), block, smem, stream>>>(p);
    return launch_status("rows_c2r launch");
}

template <typename T, int MODE>
int launch_lines_generic(LinesParams<T> p, cudaStream_t stream) {
    const int esz = sizeof(cplx_t<T>);
    if (p.W <= 0) p.W = lines_per_block_for(p.st.n, esz);
    const size_t smem = 2ull * p.W * p.st.n * esz;
    auto kern = lines_kernel<T, MODE>;
    SG_TRY(cuda_status(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                       "lines smem attribute"));
    const long long blocks = (long long)p.n_outer * ((p.inner + p.W - 1) / p.W);
    SG_REQUIRE(blocks < (1LL << 31), SG_ERR_SHAPE, "lines: too many blocks (%lld)", blocks);
    kern<<<(unsigned)blocks, 256, smem, stream>>>(p);
    return launch_status("lines launch");
}

}  // namespace sg
