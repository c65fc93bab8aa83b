// Batched Cosserat rod sub-steps: one CTA per rod, every sub-step of the call in one launch.
//
// The physics is rod.cuh's (the same functions a host driver runs in sequence); this file only
// maps its passes onto a block: threads stride over nodes, elements and Voronoi regions, and a
// barrier separates the passes that read neighbours from the ones that write them.  The per-rod
// work arrays live in shared memory.
#include "common.cuh"
#include "rod.cuh"

namespace sg {

__global__ void __launch_bounds__(256) rod_batch_kernel(sg_rod_batch b, int n_substeps, double dt, double decay) {
    extern __shared__ double rod_smem[];
    rod::View v = rod::view_of(b, blockIdx.x);
    const rod::Scratch s = rod::carve(rod_smem, b.n_elems);
    const int n = b.n_elems, t = threadIdx.x, nt = blockDim.x;
    const double h = 0.5 * dt;
    for (int k = 0; k < n_substeps; ++k) {
        for (int i = t; i <= n; i += nt) rod::drift_node(v, i, h);
        for (int e = t; e < n; e += nt) rod::rotate_element(v, e, h);
        __syncthreads();
        for (int e = t; e < n; e += nt) rod::element_pass(v, s, e);
        __syncthreads();
        for (int q = t; q < n - 1; q += nt) rod::voronoi_pass(v, s, q);
        __syncthreads();
        for (int i = t; i <= n; i += nt) rod::node_update(v, s, i, dt, decay);
        for (int e = t; e < n; e += nt) rod::element_update(v, s, e, dt, decay);
        __syncthreads();
        for (int i = t; i <= n; i += nt) rod::drift_node(v, i, h);
        for (int e = t; e < n; e += nt) rod::rotate_element(v, e, h);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) rod_markers_kernel(sg_rod_batch b, int dim, double* pos, double* vel) {
    const int n = b.n_elems;
    const int64_t total = (int64_t)b.n_rods * n;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(k / n), e = (int)(k % n);
        const rod::View v = rod::view_of(b, r);
        rod::element_marker(v, r, e, dim, total, pos, vel);
    }
}

template <typename F>
__global__ void __launch_bounds__(256) rod_loads_kernel(sg_rod_batch b, int dim, const F* forcing) {
    const int n = b.n_elems, nn = n + 1;
    const int64_t total = (int64_t)b.n_rods * nn, n_markers = (int64_t)b.n_rods * n;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(k / nn), i = (int)(k % nn);
        rod::View v = rod::view_of(b, r);
        rod::element_reaction(v, r, i, dim, n_markers, forcing, b.external_forces + (int64_t)r * 3 * nn,
                              b.external_torques + (int64_t)r * 3 * n);
    }
}

static int rod_grid_blocks(int64_t items) {
    const int64_t blocks = (items + 255) / 256;
    return (int)(blocks < 152 * 8 ? blocks : 152 * 8);
}

}  // namespace sg

static int rod_batch_check(const sg_rod_batch* batch, int dim) {
    SG_REQUIRE(batch, SG_ERR_INVALID_ARG, "rod batch: null batch");
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "rod batch: dim must be 2 or 3");
    SG_REQUIRE(batch->n_rods >= 1 && batch->n_elems >= 1, SG_ERR_SHAPE, "rod batch: empty batch");
    SG_REQUIRE(batch->position && batch->velocity && batch->mass && batch->external_forces &&
                   batch->external_torques,
               SG_ERR_INVALID_ARG, "rod batch: null array");
    return SG_OK;
}

extern "C" int sg_rod_batch_element_markers(const sg_rod_batch* batch, int dim, double* position, double* velocity,
                                            void* stream) {
    SG_TRY(rod_batch_check(batch, dim));
    SG_REQUIRE(position && velocity, SG_ERR_INVALID_ARG, "rod markers: null output");
    const int64_t items = (int64_t)batch->n_rods * batch->n_elems;
    sg::rod_markers_kernel<<<sg::rod_grid_blocks(items), 256, 0, (cudaStream_t)stream>>>(*batch, dim, position,
                                                                                        velocity);
    return sg::launch_status("rod batch element markers");
}

extern "C" int sg_rod_batch_element_loads(const sg_rod_batch* batch, int dim, int dtype, const void* lag_forcing,
                                          void* stream) {
    SG_TRY(rod_batch_check(batch, dim));
    SG_REQUIRE(lag_forcing, SG_ERR_INVALID_ARG, "rod loads: null forcing");
    SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, SG_ERR_INVALID_ARG, "rod loads: bad dtype");
    const int64_t items = (int64_t)batch->n_rods * (batch->n_elems + 1);
    auto s = (cudaStream_t)stream;
    if (dtype == SG_F32)
        sg::rod_loads_kernel<float><<<sg::rod_grid_blocks(items), 256, 0, s>>>(*batch, dim, (const float*)lag_forcing);
    else
        sg::rod_loads_kernel<double><<<sg::rod_grid_blocks(items), 256, 0, s>>>(*batch, dim,
                                                                               (const double*)lag_forcing);
    return sg::launch_status("rod batch element loads");
}

extern "C" int sg_rod_batch_step(const sg_rod_batch* batch, int n_substeps, double dt, double damping_rate,
                                 void* stream) {
    SG_REQUIRE(batch, SG_ERR_INVALID_ARG, "rod batch: null batch");
    const sg_rod_batch& b = *batch;
    SG_REQUIRE(b.n_rods >= 1 && b.n_elems >= 1 && b.n_elems <= 1024, SG_ERR_SHAPE,
               "rod batch: %d rods of %d elements (1 to 1024 elements)", b.n_rods, b.n_elems);
    SG_REQUIRE(n_substeps >= 0, SG_ERR_INVALID_ARG, "rod batch: negative sub-step count");
    SG_REQUIRE(b.position && b.velocity && b.directors && b.omega && b.mass && b.rest_lengths && b.shear_matrix &&
                   b.mass_second_moment && b.inv_mass_second_moment && b.rest_sigma && b.external_forces &&
                   b.external_torques,
               SG_ERR_INVALID_ARG, "rod batch: null array");
    SG_REQUIRE(b.n_elems == 1 || (b.rest_voronoi_lengths && b.bend_matrix && b.rest_kappa), SG_ERR_INVALID_ARG,
               "rod batch: null Voronoi array");
    SG_REQUIRE(!b.clamped || (b.clamp_position && b.clamp_directors), SG_ERR_INVALID_ARG,
               "rod batch: clamped rods need the clamp position and directors");
    if (n_substeps == 0) return SG_OK;
    const double decay = damping_rate != 0.0 ? exp(-damping_rate * dt) : 1.0;
    const size_t smem = (size_t)sg::rod::scratch_doubles(b.n_elems) * sizeof(double);
    if (smem > 48 * 1024)
        SG_TRY(sg::cuda_status(cudaFuncSetAttribute(sg::rod_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)smem),
                               "rod batch smem"));
    const int threads = (b.n_elems + 1 + 31) / 32 * 32 < 256 ? (b.n_elems + 1 + 31) / 32 * 32 : 256;
    sg::rod_batch_kernel<<<b.n_rods, threads, smem, (cudaStream_t)stream>>>(b, n_substeps, dt, decay);
    return sg::launch_status("rod batch step");
}
