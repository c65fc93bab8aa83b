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

}  // namespace sg

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
