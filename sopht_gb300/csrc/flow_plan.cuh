// Internal definition of the flow-step plan, shared by the single-instance
// step (flow.cu) and the batched 2D step (batch2d.cu).
#pragma once

#include "flow_kernels.cuh"
#include "poisson.cuh"

struct sg_flow_plan_s {
    int dim = 2, nz = 1, ny = 0, nx = 0, dtype = SG_F32;
    int width = 0, filter_type = 0, filter_order = 0;
    double x_range = 1.0, dx = 0.0;
    sg_poisson_plan_s* poisson = nullptr;
    void* scratch_a = nullptr;  // vector field
    void* scratch_b = nullptr;  // vector field (3D)
    void* filt_a = nullptr;     // scalar field (3D filter)
    void* filt_b = nullptr;
    void* coef_x = nullptr;
    void* coef_y = nullptr;
    void* coef_z = nullptr;
    // device block: [0, 64) sg_step_scalars, [64, 72) umax (field type), [72, 80) time,
    // [80, 84) kernel status (a bounded wait that ran out)
    unsigned char* dev_block = nullptr;
    // pinned host word the host-side stable dt reads the max through
    void* host_word = nullptr;
    int64_t bytes = 0;
    // optional one-shot timing events recorded between the passes of the next step
    int n_events = 0;
    cudaEvent_t events[16] = {};
    // optional one-shot tape of the next 2D step's sweep intermediates (adjoint)
    void* tape_w1 = nullptr;
    void* tape_w2 = nullptr;
    // CUDA graph of the step with host scalars: captured once per set of field pointers from the
    // device-scalar form of the step (the scalars are written to dev_scalars() by a one-thread
    // kernel before each replay); disabled after repeated rebuilds or a failed capture
    cudaStream_t capture_stream = nullptr;
    cudaGraphExec_t step_exec = nullptr;
    void* graph_fields[4] = {nullptr, nullptr, nullptr, nullptr};
    bool graph_free_stream = false;
    bool graph_disabled = false;
    int graph_builds = 0;
    sg_step_scalars* dev_scalars() const { return reinterpret_cast<sg_step_scalars*>(dev_block); }
    void* umax_slot() const { return dev_block + 64; }
    double* time_slot() const { return reinterpret_cast<double*>(dev_block + 72); }
    int32_t* kernel_status() const { return reinterpret_cast<int32_t*>(dev_block + 80); }
    int64_t cells() const { return (int64_t)nz * ny * nx; }
};

namespace sg {
int poisson_plan_create_impl(int, int, int, int, double, int, int, sg_poisson_plan_s**);
void poisson_plan_free(sg_poisson_plan_s*);
}  // namespace sg
