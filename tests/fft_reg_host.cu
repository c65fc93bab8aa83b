// Test infrastructure: the register line FFT kernels of sopht_gb300/csrc/fft_reg.cuh run on the
// host.  For every block, each phase of the kernel runs for all 256 threads before the next phase
// starts (the kernel's barriers), with each thread's registers kept between phases, so the index
// arithmetic (line addressing, the stage A / stage B split, the shared-memory slots, pruning and
// the Green's lookup) is checked against a numpy FFT without a GPU.  Built by
// tests/test_fft_reg_host.py with nvcc as host code; nothing here runs on a device.
#include <vector>

#include "../sopht_gb300/csrc/fft_reg.cuh"
#include "../sopht_gb300/csrc/flow_load_reg.cuh"

namespace {

using namespace sg;

template <int N, int MODE, bool HIN, bool HOUT>
void run_pass(const RegLinesParams& p) {
    constexpr int E = rl::Shape<N>::E;
    const int blocks = (p.n_lines + rl::kLines - 1) / rl::kLines;
    std::vector<float2> buf((size_t)N * rl::kLines);
    std::vector<float2> regs((size_t)rl::kThreads * E);
    std::vector<float2> tw_a(rl::Shape<N>::TW);
    rl::stage_twiddles<N>(p, tw_a.data(), 0, 1);
    for (int blk = 0; blk < blocks; ++blk) {
        auto each = [&](auto&& phase) {
            for (int tid = 0; tid < rl::kThreads; ++tid) {
                const int l = tid % rl::kLines, q = tid / rl::kLines;
                phase(l, q, rl::line_of(p, blk, l), regs.data() + (size_t)tid * E);
            }
        };
        if (MODE == RL_INV) {
            each([&](int l, int q, const rl::Line& L, float2* v) {
                rl::load_b<N>(p, L, q, v);
                rl::dft_b<N, true>(v);
                rl::write_b<N>(buf.data(), l, q, v);
            });
            each([&](int l, int q, const rl::Line& L, float2* v) {
                rl::read_a<N>(buf.data(), l, q, v);
                rl::inv_a<N, HOUT>(tw_a.data(), q, v);
                rl::store_a<N, HOUT>(p, L, q, v);
            });
        } else {
            each([&](int l, int q, const rl::Line& L, float2* v) {
                rl::load_a<N, HIN>(p, L, q, v);
                rl::fwd_a<N, HIN>(tw_a.data(), q, v);
                rl::write_a<N>(buf.data(), l, q, v);
            });
            if (MODE == RL_FWD) {
                each([&](int l, int q, const rl::Line& L, float2* v) {
                    rl::read_b<N>(buf.data(), l, q, v);
                    rl::dft_b<N, false>(v);
                    rl::store_b<N>(p, L, q, v);
                });
            } else {
                each([&](int l, int q, const rl::Line& L, float2* v) {
                    rl::read_b<N>(buf.data(), l, q, v);
                    rl::dft_b<N, false>(v);
                    rl::green_b<N>(p, L, q, v);
                    rl::dft_b<N, true>(v);
                });
                each([&](int l, int q, const rl::Line&, float2* v) { rl::write_b<N>(buf.data(), l, q, v); });
                each([&](int l, int q, const rl::Line& L, float2* v) {
                    rl::read_a<N>(buf.data(), l, q, v);
                    rl::inv_a<N, HOUT>(tw_a.data(), q, v);
                    rl::store_a<N, HOUT>(p, L, q, v);
                });
            }
        }
    }
}

template <int N, int MODE>
int dispatch(const RegLinesParams& p) {
    const bool hin = MODE != RL_INV && 2 * p.n_in <= N;
    const bool hout = MODE != RL_FWD && 2 * p.n_out <= N;
    if (hin && hout) run_pass<N, MODE, MODE != RL_INV, MODE != RL_FWD>(p);
    else if (hin) run_pass<N, MODE, MODE != RL_INV, false>(p);
    else if (hout) run_pass<N, MODE, false, MODE != RL_FWD>(p);
    else run_pass<N, MODE, false, false>(p);
    return 0;
}

}  // namespace

// mode: 0 forward, 1 inverse, 2 convolution; complex arrays interleaved (re, im) float32.
extern "C" int rl_host_pass(int mode, int N, const float* in, float* out, int n_lines, int slab_lines,
                            long long slab_stride, long long stride, int n_in, int n_out, const float* tw,
                            const float* g, long long g_kstride, long long g_mstride, int g_div, int g_mmod,
                            int interleave) {
    RegLinesParams p{};
    p.in = reinterpret_cast<const float2*>(in);
    p.out = reinterpret_cast<float2*>(out);
    p.n_lines = n_lines;
    p.slab_lines = slab_lines;
    p.slab_stride = slab_stride;
    p.stride = stride;
    p.n_in = n_in;
    p.n_out = n_out;
    p.tw = reinterpret_cast<const float2*>(tw);
    p.g = g;
    p.g_kstride = g_kstride;
    p.g_mstride = g_mstride;
    p.g_div = g_div;
    p.g_mmod = g_mmod;
    p.interleave = interleave;
    if (N == 512) {
        if (mode == RL_FWD) return dispatch<512, RL_FWD>(p);
        if (mode == RL_INV) return dispatch<512, RL_INV>(p);
        return dispatch<512, RL_CONV>(p);
    }
    if (N == 256) {
        if (mode == RL_FWD) return dispatch<256, RL_FWD>(p);
        if (mode == RL_INV) return dispatch<256, RL_INV>(p);
        return dispatch<256, RL_CONV>(p);
    }
    return -1;
}

// The register complex-to-real row kernel: rows of M + 1 = 257 bins (pitch 257) to rows of n_out
// reals (pitch out_pitch), phase by phase.
extern "C" int rl_host_rows_c2r(const float* in, float* out, int n_rows, int out_pitch, int n_out, const float* tw_m,
                                const float* tw_l) {
    RowsC2RParams<float> p{};
    p.in = reinterpret_cast<const float2*>(in);
    p.in_map = row_map(n_rows, rl::kRowM + 1);
    p.out = out;
    p.out_map = row_map(n_rows, out_pitch);
    p.n_out = n_out;
    p.n_rows = n_rows;
    p.tw_m = reinterpret_cast<const float2*>(tw_m);
    p.tw_l = reinterpret_cast<const float2*>(tw_l);
    std::vector<float2> buf(rl::kRowSlots), tw_a(256), regs((size_t)rl::kThreads * 16);
    rl::stage_row_twiddles(p, tw_a.data(), 0, 1);
    const int blocks = (n_rows + rl::kLines - 1) / rl::kLines;
    for (int blk = 0; blk < blocks; ++blk) {
        for (int tid = 0; tid < rl::kThreads; ++tid) {
            float2* v = regs.data() + (size_t)tid * 16;
            const int row = tid / 16, q = tid & 15;
            rl::c2r_load_b(p, rl::row_of(p, blk, row), q, v);
            dft16<true>(v);
            rl::c2r_write_b(buf.data(), row, q, v);
        }
        for (int tid = 0; tid < rl::kThreads; ++tid) {
            float2* v = regs.data() + (size_t)tid * 16;
            const int row = tid / 16, q = tid & 15;
            rl::c2r_read_a(buf.data(), row, q, v);
            rl::c2r_inv_a(tw_a.data(), q, v);
            rl::c2r_store_a(p, rl::row_of(p, blk, row), q, v);
        }
    }
    return 0;
}

// The register load pass of the 3D flow step (penalise, write back, zero the forcing, x R2C) on a
// (3, nz, ny, 256) field, phase by phase; the split's shuffle reads the partner thread's registers.
extern "C" int rl_host_flow_load(int nz, int ny, int width, const float* src, float* dst, float* forcing,
                                 const float* cx, const float* cy, const float* cz, float* spec, const float* tw_m,
                                 const float* tw_l) {
    const int nx = rl::kRowM;
    FlowLoadParams<float> p{};
    p.dim = 3;
    p.nz = nz;
    p.ny = ny;
    p.nx = nx;
    p.width = width;
    p.src = src;
    p.dst = dst;
    p.forcing = forcing;
    p.zero_ncomp = 1;
    p.cx = cx;
    p.cy = cy;
    p.cz = cz;
    p.comp_stride = (int64_t)nz * ny * nx;
    p.spec = reinterpret_cast<float2*>(spec);
    p.spec_map = row_map(ny, nx + 1, nz, (int64_t)2 * ny * (nx + 1), (int64_t)nz * 2 * ny * (nx + 1));
    p.n_rows = 3 * nz * ny;
    p.st.n = nx;
    p.tw_m = reinterpret_cast<const float2*>(tw_m);
    p.tw_l = reinterpret_cast<const float2*>(tw_l);
    std::vector<float2> buf(rl::kRowSlots), tw_a(256), regs((size_t)rl::kThreads * 16);
    rl::stage_load_twiddles(p, tw_a.data(), 0, 1);
    const int blocks = (p.n_rows + rl::kLines - 1) / rl::kLines;
    for (int blk = 0; blk < blocks; ++blk) {
        for (int tid = 0; tid < rl::kThreads; ++tid) {
            float2* v = regs.data() + (size_t)tid * 16;
            const int row = tid / 16, q = tid & 15;
            rl::load_row_a(p, rl::load_row_of(p, blk, row), q, v);
            rl::r2c_fwd_a(tw_a.data(), q, v);
            rl::r2c_write_a(buf.data(), row, q, v);
        }
        for (int tid = 0; tid < rl::kThreads; ++tid) {
            float2* v = regs.data() + (size_t)tid * 16;
            const int row = tid / 16, q = tid & 15;
            rl::r2c_read_b(buf.data(), row, q, v);
            dft16<false>(v);
        }
        for (int tid = 0; tid < rl::kThreads; ++tid) {
            const float2* v = regs.data() + (size_t)tid * 16;
            const int row = tid / 16, q = tid & 15;
            const int partner = row * 16 + ((16 - q) & 15);
            const float2* pv = regs.data() + (size_t)partner * 16;
            rl::r2c_split_store(p, rl::load_row_of(p, blk, row), q, v, [&](int r) { return pv[r]; });
        }
    }
    return 0;
}
