// Test infrastructure: the rod passes of sopht_gb300/csrc/rod.cuh run in sequence on the host, in the
// order the batched kernel runs them (one rod after another; within a rod, each pass over all its
// nodes, elements or Voronoi regions before the next), so the kernel's arithmetic can be checked
// against the numpy rod model without a GPU.  Built by tests/test_rod_batch_host.py with g++.
#include <vector>

#include "../sopht_gb300/csrc/rod.cuh"

extern "C" int rod_host_step(const sg_rod_batch* b, int n_substeps, double dt, double decay) {
    using namespace sg::rod;
    const int n = b->n_elems;
    std::vector<double> work(scratch_doubles(n));
    for (int r = 0; r < b->n_rods; ++r) {
        View v = view_of(*b, r);
        const Scratch s = carve(work.data(), n);
        const double h = 0.5 * dt;
        for (int k = 0; k < n_substeps; ++k) {
            for (int i = 0; i <= n; ++i) drift_node(v, i, h);
            for (int e = 0; e < n; ++e) rotate_element(v, e, h);
            for (int e = 0; e < n; ++e) element_pass(v, s, e);
            for (int q = 0; q < n - 1; ++q) voronoi_pass(v, s, q);
            for (int i = 0; i <= n; ++i) node_update(v, s, i, dt, decay);
            for (int e = 0; e < n; ++e) element_update(v, s, e, dt, decay);
            for (int i = 0; i <= n; ++i) drift_node(v, i, h);
            for (int e = 0; e < n; ++e) rotate_element(v, e, h);
        }
    }
    return 0;
}

// The same sub-steps with the coupled kernel's pass structure: the closing half drift of one
// sub-step and the opening half drift of the next in one pass (drift_node_twice,
// rotate_element_twice), a lone half drift at either end.
extern "C" int rod_host_step_merged(const sg_rod_batch* b, int n_substeps, double dt, double decay) {
    using namespace sg::rod;
    const int n = b->n_elems;
    std::vector<double> work(scratch_doubles(n));
    for (int r = 0; r < b->n_rods; ++r) {
        View v = view_of(*b, r);
        const Scratch s = carve(work.data(), n);
        const double h = 0.5 * dt;
        for (int i = 0; i <= n; ++i) drift_node(v, i, h);
        for (int e = 0; e < n; ++e) rotate_element(v, e, h);
        for (int k = 0; k < n_substeps; ++k) {
            for (int e = 0; e < n; ++e) element_pass(v, s, e);
            for (int q = 0; q < n - 1; ++q) voronoi_pass(v, s, q);
            for (int i = 0; i <= n; ++i) node_update(v, s, i, dt, decay);
            for (int e = 0; e < n; ++e) element_update(v, s, e, dt, decay);
            if (k + 1 < n_substeps) {
                for (int i = 0; i <= n; ++i) drift_node_twice(v, i, h);
                for (int e = 0; e < n; ++e) rotate_element_twice(v, e, h);
            } else {
                for (int i = 0; i <= n; ++i) drift_node(v, i, h);
                for (int e = 0; e < n; ++e) rotate_element(v, e, h);
            }
        }
    }
    return 0;
}

// The element-centric markers and reaction loads of the batch, in the kernels' order.
extern "C" int rod_host_markers(const sg_rod_batch* b, int dim, double* pos, double* vel) {
    using namespace sg::rod;
    const int64_t total = (int64_t)b->n_rods * b->n_elems;
    for (int r = 0; r < b->n_rods; ++r) {
        const View v = view_of(*b, r);
        for (int e = 0; e < b->n_elems; ++e) element_marker(v, r, e, dim, total, pos, vel);
    }
    return 0;
}

extern "C" int rod_host_loads(const sg_rod_batch* b, int dim, const double* forcing) {
    using namespace sg::rod;
    const int n = b->n_elems, nn = n + 1;
    const int64_t n_markers = (int64_t)b->n_rods * n;
    for (int r = 0; r < b->n_rods; ++r) {
        View v = view_of(*b, r);
        for (int i = 0; i <= n; ++i)
            element_reaction(v, r, i, dim, n_markers, forcing, b->external_forces + (int64_t)r * 3 * nn,
                             b->external_torques + (int64_t)r * 3 * n);
    }
    return 0;
}
