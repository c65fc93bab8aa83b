// The 3D rotational update w2 = w1 + pc curl(u x w1) with its inputs staged by TMA (fp32).
//
// The direct-load kernel (rotational_update3d_kernel) reads u and w1 at the six neighbours of a
// cell and forms u x w1 six times per cell, 36 loads and six cross products where one of each
// would do.  Here a block owns a 32 x 8 tile of (x, y) and marches along z through 32 planes (16
// or 8 on grids too small to give every SM four blocks otherwise):
//   * the tile's (u, w1) plane with a halo of one cell in y and of four cells before and eight
//     after in x (the copy starts on a 16-byte boundary) comes into shared memory by one tensor
//     copy per field, three planes in flight through a ring of stages, each stage completing
//     an mbarrier;
//   * u x w1 is formed once per point of the plane (the tile and a one-cell halo) into a ring of
//     three cross-product planes;
//   * each output cell then reads its six neighbouring cross products and its own w1 from shared
//     memory and writes w2 in the direct kernel's arithmetic order, so the two kernels agree to
//     the bit.
// Cells outside the grid read as zero (the copies' out-of-range fill) and only interior cells
// are updated, as in the direct kernel.  Every mbarrier wait is bounded: a wait that runs out
// records SG_ERR_CUDA in the caller's status word, lets the copies already issued land (again
// bounded) and leaves the block.
#include <cuda.h>

#include "flow_kernels.cuh"

namespace sg {
namespace {

constexpr int kTX = 32, kTY = 8;                // output tile (z planes per block: RotTmaParams::zc)
constexpr int kBX = 40, kBY = 10;               // copied box: x from x0 - 4, y from y0 - 1
constexpr int kBoxFloats = 3 * kBY * kBX;       // one field's box, [c][y][x]
constexpr int kFieldBytes = 4864;               // 4800 bytes of box, padded to 128
constexpr int kStageBytes = 2 * kFieldBytes;    // w1, then u
constexpr int kStages = 3;
constexpr int kCrossFloats = 3 * kBY * kBX;     // u x w1 of one plane on the box grid
constexpr int kCrossPoints = kBY * (kTX + 2);   // the tile and a one-cell halo in x and y
// + 64 for the mbarriers, + 128 to align the stages for the copies (under the 48 KB default)
constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + 3 * kCrossFloats * sizeof(float) + 64 + 128;
static_assert(kSmemBytes <= 48 * 1024, "no dynamic shared-memory attribute needed");
constexpr int kWaitLimit = 1 << 20;
static_assert(kBoxFloats * 4 <= kFieldBytes && kFieldBytes % 128 == 0, "stage layout");

struct RotTmaParams {
    Grid3 grid;
    float* out;
    ScalarSrc sc;      // pc = the advection prefactor
    int32_t* status;
    int zc;            // z planes per block
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// true when the phase completed within the limit
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (int i = 0; i < kWaitLimit; ++i) {
        if (mbar_try(bar, parity)) return true;
        if (i > 32) __nanosleep(64);
    }
    return false;
}

__device__ __forceinline__ void copy_box(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];"
        :
        : "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(0), "r"(bar)
        : "memory");
}

__global__ void __launch_bounds__(kTX * kTY) rot_update_tma_kernel(const __grid_constant__ CUtensorMap map_w,
                                                                   const __grid_constant__ CUtensorMap map_u,
                                                                   RotTmaParams p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // the copies' destinations on 128-byte boundaries of the shared window
    unsigned char* smem = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    float* cross = reinterpret_cast<float*>(smem + kStages * kStageBytes);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes + 3 * kCrossFloats * sizeof(float));
    const Grid3 G = p.grid;
    const int64_t n = G.n();
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTX + tx;
    const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
    const int zb = blockIdx.z * p.zc, ze = min(G.nz, zb + p.zc);
    const int nplanes = ze - zb + 2;  // input plane j is z = zb - 1 + j
    float pcs[1];
    block_scalars<float, 1>([&](int) { return p.sc.advection(); }, pcs);
    const float pc = pcs[0];
    auto stage = [&](int j) { return reinterpret_cast<float*>(smem + (j % kStages) * kStageBytes); };
    auto bar = [&](int j) { return smem_addr(bars + j % kStages); };
    auto issue = [&](int j) {  // thread 0: plane j of w1 and u into its stage
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar(j)), "r"(2 * kBoxFloats * 4)
                     : "memory");
        float* s = stage(j);
        copy_box(smem_addr(s), &map_w, x0 - 4, y0 - 1, zb - 1 + j, bar(j));
        copy_box(smem_addr(s) + kFieldBytes, &map_u, x0 - 4, y0 - 1, zb - 1 + j, bar(j));
    };
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bars + s)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0)
        for (int j = 0; j < kStages && j < nplanes; ++j) issue(j);
    int issued = min(kStages, nplanes), waited = 0;
    // u x w1 of plane j on the tile and its halo, into cross slot j % 3
    auto form_cross = [&](int j) {
        const float* w = stage(j);
        const float* u = w + kFieldBytes / 4;
        float* c = cross + (j % 3) * kCrossFloats;
        for (int k = tid; k < kCrossPoints; k += kTX * kTY) {
            const int yy = k / (kTX + 2), xx = 3 + k % (kTX + 2);
            const int o = yy * kBX + xx, pl = kBY * kBX;
            const float ux = u[o], uy = u[pl + o], uz = u[2 * pl + o];
            const float wx = w[o], wy = w[pl + o], wz = w[2 * pl + o];
            // elementwise_ops_3d.py:406-448: r_i = a_j b_k - b_j a_k, as cross_at
            c[o] = uy * wz - wy * uz;
            c[pl + o] = uz * wx - wz * ux;
            c[2 * pl + o] = ux * wy - wx * uy;
        }
    };
    // waits for plane j; false (in every thread) when a wait ran out
    auto arrive = [&](int j) {
        const bool ok = mbar_wait(bar(j), (uint32_t)((j / kStages) & 1));
        waited = j + 1;
        return ok;
    };
    bool ok = arrive(0);
    ok = ok && arrive(1);
    const bool bad0 = __syncthreads_or(!ok);
    if (!bad0) {
        form_cross(0);
        form_cross(1);
    }
    bool bad = bad0;
    if (!bad) {
        __syncthreads();
        if (tid == 0 && 3 < nplanes) issue(3);
        issued = min(4, nplanes);
        for (int j = 1; j + 1 < nplanes; ++j) {
            const bool got = arrive(j + 1);
            if (__syncthreads_or(!got)) {
                bad = true;
                break;
            }
            form_cross(j + 1);
            __syncthreads();
            // output plane j: z = zb - 1 + j
            const int z = zb - 1 + j, x = x0 + tx, y = y0 + ty;
            if (x < G.nx && y < G.ny) {
                const int xx = tx + 4, yy = ty + 1, pl = kBY * kBX, o = yy * kBX + xx;
                const float* w = stage(j);
                float w0 = w[o], w1 = w[pl + o], w2 = w[2 * pl + o];
                if (G.interior(z, y, x)) {
                    const float* cm = cross + ((j + 2) % 3) * kCrossFloats;  // plane j - 1
                    const float* c0 = cross + (j % 3) * kCrossFloats;
                    const float* cp = cross + ((j + 1) % 3) * kCrossFloats;  // plane j + 1
                    float cyp[3], cym[3], czp[3], czm[3], cxp[3], cxm[3];
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        cyp[d] = c0[d * pl + o + kBX];
                        cym[d] = c0[d * pl + o - kBX];
                        czp[d] = cp[d * pl + o];
                        czm[d] = cm[d * pl + o];
                        cxp[d] = c0[d * pl + o + 1];
                        cxm[d] = c0[d * pl + o - 1];
                    }
                    const float r0 = cyp[2] - cym[2] - czp[1] + czm[1];
                    const float r1 = czp[0] - czm[0] - cxp[2] + cxm[2];
                    const float r2 = cxp[1] - cxm[1] - cyp[0] + cym[0];
                    w0 = w0 + pc * r0;
                    w1 = w1 + pc * r1;
                    w2 = w2 + pc * r2;
                }
                const int64_t g = ((int64_t)z * G.ny + y) * G.nx + x;
                p.out[g] = w0;
                p.out[n + g] = w1;
                p.out[2 * n + g] = w2;
            }
            __syncthreads();
            if (j + 3 < nplanes) {
                if (tid == 0) issue(j + 3);
                issued = j + 4;
            }
        }
    }
    if (bad) {
        // a copy did not land in time: record it, give the issued copies a bounded wait, leave
        if (tid == 0) {
            atomicExch(p.status, SG_ERR_CUDA);
            for (int j = waited; j < issued; ++j) mbar_wait(bar(j), (uint32_t)((j / kStages) & 1));
        }
        __syncthreads();
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<EncodeTiled>(f);
    }();
    return fn;
}

// the (3, nz, ny, nx) fp32 field as a 4D tensor, boxes of 40 x 10 x 1 x 3
int encode_field(CUtensorMap* m, const float* base, const Grid3& G, int ncomp = 3) {
    EncodeTiled fn = encode_fn();
    SG_REQUIRE(fn, SG_ERR_CUDA, "tensor copies: cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[4] = {(cuuint64_t)G.nx, (cuuint64_t)G.ny, (cuuint64_t)G.nz, (cuuint64_t)ncomp};
    const cuuint64_t strides[3] = {(cuuint64_t)G.nx * 4, (cuuint64_t)G.nx * G.ny * 4,
                                   (cuuint64_t)G.nx * G.ny * G.nz * 4};
    const cuuint32_t box[4] = {kBX, kBY, 1, (cuuint32_t)ncomp};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    SG_REQUIRE(r == CUDA_SUCCESS, SG_ERR_CUDA, "tensor copies: cuTensorMapEncodeTiled failed (%d)", (int)r);
    return SG_OK;
}

// ---------------------------------------------------------------- diffusion
// w3 = w2 + k lap(w2) on [1:-1]^3 per component, the (1 or 3 components of a) plane of the tile
// with its halo copied as above; five stages: planes j - 1, j, j + 1 in use while plane j is
// written, two more in flight.
constexpr int kDStages = 5;
constexpr size_t kDSmemBytes = (size_t)kDStages * kFieldBytes + 64 + 128;
static_assert(kDSmemBytes <= 48 * 1024, "no dynamic shared-memory attribute needed");

struct DiffTmaParams {
    Grid3 grid;
    float* out;
    ScalarSrc sc;      // k = the diffusion prefactor (pf = the forcing prefactor for the curl)
    int ncomp;
    int32_t* status;
    int zc;
    const float* w;    // the forcing curl's vorticity (read at the cell), or null
    float prefactor;   // the velocity curl's 0.5 / dx
    int add_free_stream;
    float* umax;       // the velocity curl's max of sum |u_d|, or null
};

enum { PLANE_DIFFUSE = 0, PLANE_FORCING_CURL = 1, PLANE_VELOCITY_CURL = 2 };

// PLANE_DIFFUSE: out = f + k lap(f) per component.  PLANE_FORCING_CURL: out = w + pf curl(f), the
// copied field f the forcing and w read at the cell (forcing_curl3d_kernel's arithmetic).
// PLANE_VELOCITY_CURL: out = prefactor curl(f) on [1:-1]^3 (0 on the ring) + the free stream, with
// the max over the block's cells of sum |out_d| into *umax (curl3d_kernel's arithmetic; the max
// is the same whichever cells a block holds).
// NC: the components (3, or 1 for a scalar diffusion), fixed so that the per-component loop unrolls.
template <int OP, int NC = 3>
__global__ void __launch_bounds__(kTX * kTY) diffusion_tma_kernel(const __grid_constant__ CUtensorMap map,
                                                                  DiffTmaParams p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kDStages * kFieldBytes);
    const Grid3 G = p.grid;
    const int64_t n = G.n();
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTX + tx;
    const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
    const int zb = blockIdx.z * p.zc, ze = min(G.nz, zb + p.zc);
    const int nplanes = ze - zb + 2;  // input plane j is z = zb - 1 + j
    constexpr int nc = NC;
    float ks[1];
    block_scalars<float, 1>([&](int) { return OP == PLANE_DIFFUSE ? p.sc.diffusion() : p.sc.forcing(); }, ks);
    const float k = ks[0];
    float m = 0.f;  // PLANE_VELOCITY_CURL: the thread's max of sum |u_d|
    // the free stream in fp32, converted once per block (a double-to-float conversion per cell
    // and plane would hold the double-precision units for as long as the whole pass)
    float fs[3] = {0.f, 0.f, 0.f};
    if constexpr (OP == PLANE_VELOCITY_CURL)
        block_scalars<float, 3>([&](int d) { return p.add_free_stream ? p.sc.free_stream(d) : 0.0; }, fs);
    auto stage = [&](int j) { return reinterpret_cast<const float*>(smem + (j % kDStages) * kFieldBytes); };
    auto bar = [&](int j) { return smem_addr(bars + j % kDStages); };
    auto issue = [&](int j) {  // thread 0
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar(j)), "r"(nc * kBY * kBX * 4)
                     : "memory");
        copy_box(smem_addr(stage(j)), &map, x0 - 4, y0 - 1, zb - 1 + j, bar(j));
    };
    if (tid == 0) {
        for (int s = 0; s < kDStages; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bars + s)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0)
        for (int j = 0; j < kDStages && j < nplanes; ++j) issue(j);
    int issued = min(kDStages, nplanes), waited = 0;
    auto arrive = [&](int j) {
        const bool ok = mbar_wait(bar(j), (uint32_t)((j / kDStages) & 1));
        waited = j + 1;
        return ok;
    };
    bool ok = arrive(0);
    bool bad = __syncthreads_or(!ok);
    for (int j = 1; !bad && j + 1 < nplanes; ++j) {
        // planes j - 1 and j are in (waited for in the iterations before); wait for j + 1
        const bool got = (j == 1 ? arrive(1) : true) && arrive(j + 1);
        if (__syncthreads_or(!got)) {
            bad = true;
            break;
        }
        const int z = zb - 1 + j, x = x0 + tx, y = y0 + ty;
        if (OP == PLANE_FORCING_CURL && x < G.nx && y < G.ny) {
            const int xx = tx + 4, yy = ty + 1, pl = kBY * kBX, o = yy * kBX + xx;
            const float *cm = stage(j - 1), *c0 = stage(j), *cp = stage(j + 1);
            const int64_t g = ((int64_t)z * G.ny + y) * G.nx + x;
            float w0 = p.w[g], w1 = p.w[n + g], w2 = p.w[2 * n + g];
            if (G.interior(z, y, x)) {
                // curl3_at's terms: f at y +- 1, z +- 1 and x +- 1 from the three planes
                const float c0v = c0[2 * pl + o + kBX] - c0[2 * pl + o - kBX] - cp[pl + o] + cm[pl + o];
                const float c1v = cp[o] - cm[o] - c0[2 * pl + o + 1] + c0[2 * pl + o - 1];
                const float c2v = c0[pl + o + 1] - c0[pl + o - 1] - c0[o + kBX] + c0[o - kBX];
                w0 = w0 + k * c0v;
                w1 = w1 + k * c1v;
                w2 = w2 + k * c2v;
            }
            p.out[g] = w0;
            p.out[n + g] = w1;
            p.out[2 * n + g] = w2;
        }
        if (OP == PLANE_VELOCITY_CURL && x < G.nx && y < G.ny) {
            const int xx = tx + 4, yy = ty + 1, pl = kBY * kBX, o = yy * kBX + xx;
            const float *cm = stage(j - 1), *c0 = stage(j), *cp = stage(j + 1);
            const int64_t g = ((int64_t)z * G.ny + y) * G.nx + x;
            float c[3] = {0.f, 0.f, 0.f};
            if (G.interior(z, y, x)) {
                c[0] = c0[2 * pl + o + kBX] - c0[2 * pl + o - kBX] - cp[pl + o] + cm[pl + o];
                c[1] = cp[o] - cm[o] - c0[2 * pl + o + 1] + c0[2 * pl + o - 1];
                c[2] = c0[pl + o + 1] - c0[pl + o - 1] - c0[o + kBX] + c0[o - kBX];
                c[0] = p.prefactor * c[0];
                c[1] = p.prefactor * c[1];
                c[2] = p.prefactor * c[2];
            }
            if (p.add_free_stream) {
#pragma unroll
                for (int d = 0; d < 3; ++d) c[d] = c[d] + fs[d];
            }
            p.out[g] = c[0];
            p.out[n + g] = c[1];
            p.out[2 * n + g] = c[2];
            m = fmaxf(m, fabsf(c[0]) + fabsf(c[1]) + fabsf(c[2]));
        }
        if (OP == PLANE_DIFFUSE && x < G.nx && y < G.ny) {
            const int xx = tx + 4, yy = ty + 1, pl = kBY * kBX, o = yy * kBX + xx;
            const float *cm = stage(j - 1), *c0 = stage(j), *cp = stage(j + 1);
            const bool in = G.interior(z, y, x);
            const int64_t g = ((int64_t)z * G.ny + y) * G.nx + x;
#pragma unroll
            for (int c = 0; c < nc; ++c) {
                const float v = c0[c * pl + o];
                float r = v;
                if (in) {
                    // diffusion_flux_3d.py:34-43 term order: z+1, z-1, y+1, y-1, x+1, x-1
                    const float lap = cp[c * pl + o] + cm[c * pl + o] + c0[c * pl + o + kBX] + c0[c * pl + o - kBX] +
                                      c0[c * pl + o + 1] + c0[c * pl + o - 1] - 6.f * v;
                    r = v + k * lap;
                }
                p.out[c * n + g] = r;
            }
        }
        __syncthreads();
        // plane j - 1 is no longer read: its stage takes plane j + kDStages - 1
        if (j + kDStages - 1 < nplanes) {
            if (tid == 0) issue(j + kDStages - 1);
            issued = j + kDStages;
        }
    }
    if (bad) {
        if (tid == 0) {
            atomicExch(p.status, SG_ERR_CUDA);
            for (int j = waited; j < issued; ++j) mbar_wait(bar(j), (uint32_t)((j / kDStages) & 1));
        }
        __syncthreads();
    } else if (OP == PLANE_VELOCITY_CURL && p.umax) {
        m = block_max(m);
        if (tid == 0) atomic_max_nonneg_filtered(p.umax, m);
    }
}

// the longest z run per block (32, 16 or 8 planes: each block also copies the two planes around its
// run) that still gives every SM four blocks
int z_run(const Grid3& G) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t tiles = (int64_t)((G.nx + kTX - 1) / kTX) * ((G.ny + kTY - 1) / kTY);
    int zc = 32;
    while (zc > 8 && tiles * ((G.nz + zc - 1) / zc) < 4LL * sms) zc /= 2;
    return zc;
}

}  // namespace

bool diffusion_tma_ok(const Grid3& G, int ncomp, const void* in, const void* out) {
    const auto aligned = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
    return (ncomp == 1 || ncomp == 3) && G.nx % 4 == 0 && G.nx >= 4 && G.ny >= 3 && G.nz >= 3 && aligned(in) &&
           aligned(out) && encode_fn() != nullptr;
}

int launch_diffusion_tma(const Grid3& G, int ncomp, const float* in, float* out, const ScalarSrc& sc,
                         int32_t* status, cudaStream_t stream) {
    SG_REQUIRE(diffusion_tma_ok(G, ncomp, in, out), SG_ERR_INVALID_ARG,
               "tensor-copy diffusion: 1 or 3 components, nx a multiple of 4, 16-byte aligned fields");
    SG_REQUIRE(status, SG_ERR_INVALID_ARG, "tensor-copy diffusion: null status word");
    CUtensorMap m;
    SG_TRY(encode_field(&m, in, G, ncomp));
    DiffTmaParams p{};
    p.grid = G;
    p.out = out;
    p.sc = sc;
    p.ncomp = ncomp;
    p.status = status;
    p.zc = z_run(G);
    const dim3 grid((unsigned)((G.nx + kTX - 1) / kTX), (unsigned)((G.ny + kTY - 1) / kTY),
                    (unsigned)((G.nz + p.zc - 1) / p.zc));
    if (ncomp == 1) diffusion_tma_kernel<PLANE_DIFFUSE, 1><<<grid, dim3(kTX, kTY), kDSmemBytes, stream>>>(m, p);
    else diffusion_tma_kernel<PLANE_DIFFUSE, 3><<<grid, dim3(kTX, kTY), kDSmemBytes, stream>>>(m, p);
    return launch_status("tensor-copy diffusion");
}

bool velocity_curl_tma_ok(const Grid3& G, const void* psi, const void* u) {
    return diffusion_tma_ok(G, 3, psi, u);
}

int launch_velocity_curl_tma(const Grid3& G, const float* psi, float* u, float prefactor, const ScalarSrc& sc,
                             int add_free_stream, float* umax, int32_t* status, cudaStream_t stream) {
    SG_REQUIRE(velocity_curl_tma_ok(G, psi, u), SG_ERR_INVALID_ARG,
               "tensor-copy curl: nx a multiple of 4, 16-byte aligned fields");
    SG_REQUIRE(status, SG_ERR_INVALID_ARG, "tensor-copy curl: null status word");
    CUtensorMap m;
    SG_TRY(encode_field(&m, psi, G, 3));
    DiffTmaParams p{};
    p.grid = G;
    p.out = u;
    p.sc = sc;
    p.ncomp = 3;
    p.status = status;
    p.zc = z_run(G);
    p.prefactor = prefactor;
    p.add_free_stream = add_free_stream;
    p.umax = umax;
    const dim3 grid((unsigned)((G.nx + kTX - 1) / kTX), (unsigned)((G.ny + kTY - 1) / kTY),
                    (unsigned)((G.nz + p.zc - 1) / p.zc));
    diffusion_tma_kernel<PLANE_VELOCITY_CURL><<<grid, dim3(kTX, kTY), kDSmemBytes, stream>>>(m, p);
    return launch_status("tensor-copy curl");
}

bool forcing_curl_tma_ok(const Grid3& G, const void* w, const void* f, const void* out) {
    return diffusion_tma_ok(G, 3, f, out) && (reinterpret_cast<uintptr_t>(w) & 15) == 0;
}

int launch_forcing_curl_tma(const Grid3& G, const float* w, const float* f, float* out, const ScalarSrc& sc,
                            int32_t* status, cudaStream_t stream) {
    SG_REQUIRE(forcing_curl_tma_ok(G, w, f, out), SG_ERR_INVALID_ARG,
               "tensor-copy forcing curl: nx a multiple of 4, 16-byte aligned fields");
    SG_REQUIRE(status, SG_ERR_INVALID_ARG, "tensor-copy forcing curl: null status word");
    CUtensorMap m;
    SG_TRY(encode_field(&m, f, G, 3));
    DiffTmaParams p{};
    p.grid = G;
    p.out = out;
    p.sc = sc;
    p.ncomp = 3;
    p.status = status;
    p.zc = z_run(G);
    p.w = w;
    const dim3 grid((unsigned)((G.nx + kTX - 1) / kTX), (unsigned)((G.ny + kTY - 1) / kTY),
                    (unsigned)((G.nz + p.zc - 1) / p.zc));
    diffusion_tma_kernel<PLANE_FORCING_CURL><<<grid, dim3(kTX, kTY), kDSmemBytes, stream>>>(m, p);
    return launch_status("tensor-copy forcing curl");
}

bool rot_update_tma_ok(const Grid3& G, const void* w1, const void* u, const void* out) {
    const auto aligned = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
    return G.nx % 4 == 0 && G.nx >= 4 && G.ny >= 3 && G.nz >= 3 && aligned(w1) && aligned(u) && aligned(out) &&
           encode_fn() != nullptr;
}

int launch_rot_update_tma(const Grid3& G, const float* w1, const float* u, float* out, const ScalarSrc& sc,
                          int32_t* status, cudaStream_t stream) {
    SG_REQUIRE(rot_update_tma_ok(G, w1, u, out), SG_ERR_INVALID_ARG,
               "tensor-copy rotational update: nx a multiple of 4, 16-byte aligned fields");
    SG_REQUIRE(status, SG_ERR_INVALID_ARG, "tensor-copy rotational update: null status word");
    CUtensorMap mw, mu;
    SG_TRY(encode_field(&mw, w1, G));
    SG_TRY(encode_field(&mu, u, G));
    RotTmaParams p{};
    p.grid = G;
    p.out = out;
    p.sc = sc;
    p.status = status;
    p.zc = z_run(G);
    const dim3 grid((unsigned)((G.nx + kTX - 1) / kTX), (unsigned)((G.ny + kTY - 1) / kTY),
                    (unsigned)((G.nz + p.zc - 1) / p.zc));
    rot_update_tma_kernel<<<grid, dim3(kTX, kTY), kSmemBytes, stream>>>(mw, mu, p);
    return launch_status("tensor-copy rotational update");
}

}  // namespace sg
