// The 3D Poisson load pass with the x real-to-complex transform in registers (fp32, nx = 256).
//
// One row of vorticity (256 reals, zero-padded to 512) becomes the 257 bins of its real transform,
// through the half-length complex transform of z[n] = x[2n] + i x[2n+1] (M = 256 points, of which
// n < 128 are non-zero).  On the way in, each point is penalised (the clamped gathers and sine
// factors of penalise_field_boundary_3d.py, X then Y then Z, as fast_flow_load_body applies them),
// written back to the caller's vorticity, and the row of the forcing field is zeroed.  16 rows per
// block and 16 threads per row:
//   stage A: thread (row, g) loads points n = g + 16 j (j < 8), takes their length-16 DFT and the
//            twiddles w_M^(g k2);
//   exchange: [g][row][k2] in shared memory, a one-point pad per g (conflict-free both ways);
//   stage B: thread (row, t) takes the length-16 DFT over g, holding Z[t + 16 k1];
//   split:   X[k] = (Z[k] + Z*[M-k]) / 2 - (i/2) w_2M^k (Z[k] - Z*[M-k]); Z[M-k] sits in lane
//            16 - t of the row's half-warp (register 15 - k1), so one shuffle per register brings it.
// The phases are __host__ __device__ (the shuffle behind a fetch function), so a host driver can run
// them thread by thread.
#pragma once

#include "fft_reg.cuh"
#include "flow_kernels.cuh"

namespace sg {
namespace rl {

struct LoadRow {
    int64_t src_off, dst_off, spec_off;
    float fy, fz;
    bool live;
};

SG_RL_FN LoadRow load_row_of(const FlowLoadParams<float>& p, int block, int row) {
    LoadRow R;
    const int q = block * kLines + row;
    R.live = q < p.n_rows;
    const int qq = R.live ? q : 0;
    const int y = qq % p.ny;
    const int zi = (qq / p.ny) % p.nz;
    const int c = qq / (p.ny * p.nz);
    const int w = p.width;
    const int sy = w <= 0 ? y : (y < w - 1 ? w - 1 : (y > p.ny - w ? p.ny - w : y));
    const int sz = w <= 0 ? zi : (zi < w - 1 ? w - 1 : (zi > p.nz - w ? p.nz - w : zi));
    R.src_off = (int64_t)c * p.comp_stride + ((int64_t)sz * p.ny + sy) * p.nx;
    R.dst_off = (int64_t)c * p.comp_stride + ((int64_t)zi * p.ny + y) * p.nx;
    R.spec_off = p.spec_map.offset(qq);
    R.fy = w > 0 ? p.cy[y] : 1.f;
    R.fz = w > 0 ? p.cz[zi] : 1.f;
    return R;
}

SG_RL_FN int band(int i, int n, int w) { return w <= 0 ? i : (i < w - 1 ? w - 1 : (i > n - w ? n - w : i)); }

// Stage A input: the penalised points n = g + 16 j of the row (written back, forcing zeroed).  All
// loads are issued before the first store: a store to the vorticity or forcing could alias a later
// load, which would otherwise keep the compiler from having more than one load in flight.
SG_RL_FN void load_row_a(const FlowLoadParams<float>& p, const LoadRow& R, int g, float2* v) {
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = cmake<float2>(0.f, 0.f);
    if (!R.live) return;
    const float* src = p.src + R.src_off;
    float2 c[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int x0 = 2 * (g + 16 * j);
        const int s0 = band(x0, p.nx, p.width), s1 = band(x0 + 1, p.nx, p.width);
        if (s0 == x0 && s1 == x0 + 1) {
            v[j] = *reinterpret_cast<const float2*>(src + x0);
        } else {
            v[j].x = src[s0];
            v[j].y = src[s1];
        }
        c[j] = p.width > 0 ? *reinterpret_cast<const float2*>(p.cx + x0) : cmake<float2>(1.f, 1.f);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int x0 = 2 * (g + 16 * j);
        float2 z = v[j];
        if (p.width > 0) {
            z.x = z.x * c[j].x;
            z.y = z.y * c[j].y;
            z.x = z.x * R.fy;
            z.y = z.y * R.fy;
            z.x = z.x * R.fz;
            z.y = z.y * R.fz;
        }
        v[j] = z;
        *reinterpret_cast<float2*>(p.dst + R.dst_off + x0) = z;
        if (p.forcing)
            for (int zc = 0; zc < p.zero_ncomp; ++zc)
                *reinterpret_cast<float2*>(p.forcing + R.dst_off + x0 + zc * p.comp_stride) = cmake<float2>(0.f, 0.f);
    }
}

// w_M^(g k2) for the rows: tw_m[m] = exp(-2 pi i m / M).
SG_RL_FN void stage_load_twiddles(const FlowLoadParams<float>& p, float2* tw_a, int tid, int nt) {
    for (int i = tid; i < 256; i += nt) tw_a[i] = p.tw_m[(i / 16) * (i % 16)];
}

SG_RL_FN void r2c_fwd_a(const float2* tw_a, int g, float2* v) {
    dft16<false, true>(v);
#pragma unroll
    for (int k2 = 1; k2 < 16; ++k2) v[k2] = cmul(v[k2], tw_a[g * 16 + k2]);
}

SG_RL_FN void r2c_write_a(float2* buf, int row, int g, const float2* v) {
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) buf[row_slot(g, row, k2)] = v[k2];
}

SG_RL_FN void r2c_read_b(const float2* buf, int row, int t, float2* v) {
#pragma unroll
    for (int gg = 0; gg < 16; ++gg) v[gg] = buf[row_slot(gg, row, t)];
}

// The split and the stores.  v holds Z[t + 16 k1]; fetch(r) returns register r of the row's lane
// 16 - t (lane 0 of the row asks itself).
template <typename Fetch>
SG_RL_FN void r2c_split_store(const FlowLoadParams<float>& p, const LoadRow& R, int t, const float2* v, Fetch fetch) {
    constexpr int M = kRowM;
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) {
        const float2 other = fetch(15 - k1);  // every lane takes part in the exchange
        const int k = t + 16 * k1;
        // Z[M - k]: lane 16 - t's register 15 - k1, or, in lane 0, its own register (16 - k1) mod 16
        const float2 zm = t == 0 ? v[(16 - k1) & 15] : other;
        const float2 zk = v[k1];
        const float2 zc = cconj(zm);
        const float2 w = p.tw_l[k];
        const float2 sm = cadd(zk, zc);
        const float2 wd = cmul(w, csub(zk, zc));
        if (R.live) p.spec[R.spec_off + k] = cmake<float2>(0.5f * (sm.x + wd.y), 0.5f * (sm.y - wd.x));
        if (k1 == 0 && t == 0 && R.live) {  // bin M from Z[0]
            const float2 zc0 = cconj(zk);
            const float2 wM = p.tw_l[M];
            const float2 s0 = cadd(zk, zc0);
            const float2 d0 = cmul(wM, csub(zk, zc0));
            p.spec[R.spec_off + M] = cmake<float2>(0.5f * (s0.x + d0.y), 0.5f * (s0.y - d0.x));
        }
    }
}

}  // namespace rl

#ifdef __CUDACC__
static __global__ void __launch_bounds__(rl::kThreads, 3) reg_flow_load_kernel(FlowLoadParams<float> p) {
    __shared__ __align__(16) float2 buf[rl::kRowSlots];
    __shared__ __align__(16) float2 tw_a[256];
    const int tid = threadIdx.x, row = tid / 16, q = tid & 15;
    const rl::LoadRow R = rl::load_row_of(p, blockIdx.x, row);
    float2 v[16];
    // the source rows of the block one wave ahead, asked of L2: 256 floats, 8 lines of 128 bytes
    if (p.prefetch_ahead > 0 && blockIdx.x + p.prefetch_ahead < gridDim.x && q < 8) {
        const rl::LoadRow Ra = rl::load_row_of(p, blockIdx.x + p.prefetch_ahead, row);
        if (Ra.live) asm volatile("prefetch.global.L2 [%0];" ::"l"(p.src + Ra.src_off + q * 32));
    }
    rl::stage_load_twiddles(p, tw_a, tid, rl::kThreads);
    rl::load_row_a(p, R, q, v);
    __syncthreads();  // the twiddle table
    rl::r2c_fwd_a(tw_a, q, v);
    rl::r2c_write_a(buf, row, q, v);
    __syncthreads();
    rl::r2c_read_b(buf, row, q, v);
    dft16<false>(v);
    const int lane = tid & 31, partner = (lane & 16) | ((16 - q) & 15);
    rl::r2c_split_store(p, R, q, v, [&](int r) {
        float2 o;
        o.x = __shfl_sync(0xffffffffu, v[r].x, partner);
        o.y = __shfl_sync(0xffffffffu, v[r].y, partner);
        return o;
    });
}

inline int launch_reg_flow_load(FlowLoadParams<float> p, cudaStream_t stream) {
    if (p.n_rows <= 0) return SG_OK;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    p.prefetch_ahead = 3 * sms;  // one wave of resident blocks (three per SM)
    reg_flow_load_kernel<<<ceil_div(p.n_rows, rl::kLines), rl::kThreads, 0, stream>>>(p);
    return launch_status("register flow load");
}
#endif

}  // namespace sg
