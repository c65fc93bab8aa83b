// Internal definition of the unbounded Poisson plan, shared with the flow step.
#pragma once

#include "fft_fast.cuh"

struct sg_poisson_plan_s {
    int dim = 2;
    int nz = 1, ny = 0, nx = 0;
    int dtype = SG_F32;
    int max_comp = 1;
    double x_range = 1.0;
    double dx = 0.0;  // the real_t-rounded grid spacing, as double
    sg::FFTStages st_x{};  // complex length nx (rows of 2 nx reals)
    sg::FFTStages st_y{};  // 2 ny
    sg::FFTStages st_z{};  // 2 nz (3D)
    void* tw_x = nullptr;   // nx entries: exp(-2 pi i m / nx)
    void* tw_xl = nullptr;  // nx+1 entries: exp(-2 pi i k / (2 nx))
    void* tw_y = nullptr;   // 2 ny entries
    void* tw_z = nullptr;   // 2 nz entries
    void* greens = nullptr; // real table, 2D (ny+1)(nx+1), 3D (nz+1)(ny+1)(nx+1)
    void* spec = nullptr;   // complex workspace, max_comp * spec_comp_elems
    int64_t spec_comp_elems = 0;
    int64_t bytes = 0;
};

namespace sg {

// Passes of the solve, exposed so the flow step can replace the first pass by
// its fused penalise/write-back/forcing-reset variant.
template <typename T>
int poisson_spectral_passes(sg_poisson_plan_s* p, int ncomp, cudaStream_t stream);
// 3D only: pass 0 = y forward, 1 = z convolution, 2 = y inverse
template <typename T>
int poisson_spectral_pass3d(sg_poisson_plan_s* p, int ncomp, int pass, cudaStream_t stream);
template <typename T>
int poisson_load_rows(sg_poisson_plan_s* p, const T* rhs, int ncomp, int64_t comp_stride,
                      cudaStream_t stream);
template <typename T>
int poisson_store_rows(sg_poisson_plan_s* p, T* sol, int ncomp, int64_t comp_stride,
                       cudaStream_t stream);

}  // namespace sg
