// Adjoint entry points: the transpose of every operator of the 2D step and of
// the virtual-boundary coupling (see adjoint.cuh for the forward maps), plus
// the fused reverse sweep used by the step-level adjoint.
#include "adjoint.cuh"
#include "flow_plan.cuh"

using namespace sg;

#define SG_ADJ_DISPATCH(dtype, CALL_F, CALL_D)                                             \
    do {                                                                                  \
        if ((dtype) == SG_F32) {                                                          \
            CALL_F;                                                                       \
        } else {                                                                          \
            SG_REQUIRE((dtype) == SG_F64, SG_ERR_INVALID_ARG, "bad dtype %d", (int)(dtype)); \
            CALL_D;                                                                       \
        }                                                                                 \
    } while (0)

static dim3 grid2d(int ny, int nx) { return dim3(ceil_div(nx, 32), ceil_div(ny, 8)); }

static int check_grid2d(int ny, int nx) {
    SG_REQUIRE(ny >= 1 && nx >= 1, SG_ERR_SHAPE, "bad 2D extent (%d, %d)", ny, nx);
    return SG_OK;
}

extern "C" int64_t sg_adj_partials_count_2d(int ny, int nx) {
    if (ny < 1 || nx < 1) return 0;
    return (int64_t)ceil_div(nx, 32) * ceil_div(ny, 8);
}

extern "C" int sg_sum_partials(int64_t n, const double* partials, double* acc, void* stream) {
    SG_REQUIRE(n >= 1 && partials && acc, SG_ERR_INVALID_ARG, "sum partials: bad argument");
    sum_partials_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(n, partials, acc);
    return launch_status("sum_partials");
}

extern "C" int sg_outplane_curl_adj_2d(int dtype, int ny, int nx, const void* curl_bar, void* psi_bar,
                                       double prefactor, void* stream_) {
    SG_TRY(check_grid2d(ny, nx));
    SG_REQUIRE(curl_bar && psi_bar && curl_bar != psi_bar, SG_ERR_INVALID_ARG, "curl adjoint: bad pointers");
    auto s = (cudaStream_t)stream_;
    SG_ADJ_DISPATCH(dtype,
                    (curl2d_adj_kernel<float><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(ny, nx, (float)prefactor,
                                                                                  (const float*)curl_bar,
                                                                                  (float*)psi_bar)),
                    (curl2d_adj_kernel<double><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(ny, nx, prefactor,
                                                                                   (const double*)curl_bar,
                                                                                   (double*)psi_bar)));
    return launch_status("outplane curl adjoint");
}

extern "C" int sg_penalise_adj_2d(int dtype, int ny, int nx, const void* in_bar, void* out_bar, int width,
                                  const void* cx, const void* cy, void* stream_) {
    SG_TRY(check_grid2d(ny, nx));
    SG_REQUIRE(in_bar && out_bar && in_bar != out_bar, SG_ERR_INVALID_ARG, "penalise adjoint: bad pointers");
    SG_REQUIRE(width >= 0 && 2 * width <= nx && 2 * width <= ny, SG_ERR_SHAPE, "penalty width does not fit");
    SG_REQUIRE(width != 1, SG_ERR_INVALID_ARG, "penalty width 1 has no forward map");
    SG_REQUIRE(width == 0 || (cx && cy), SG_ERR_INVALID_ARG, "null penalisation table");
    auto s = (cudaStream_t)stream_;
    SG_ADJ_DISPATCH(dtype,
                    (pen2d_adj_kernel<float><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(
                        ny, nx, width, (const float*)cx, (const float*)cy, (const float*)in_bar, (float*)out_bar)),
                    (pen2d_adj_kernel<double><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(
                        ny, nx, width, (const double*)cx, (const double*)cy, (const double*)in_bar,
                        (double*)out_bar)));
    return launch_status("penalise adjoint");
}

extern "C" int sg_diffusion_adj_2d(int dtype, int ny, int nx, const void* in_bar, void* out_bar, double k,
                                   const void* field, double* partials, void* stream_) {
    SG_TRY(check_grid2d(ny, nx));
    SG_REQUIRE(in_bar && out_bar && in_bar != out_bar, SG_ERR_INVALID_ARG, "diffusion adjoint: bad pointers");
    SG_REQUIRE((field == nullptr) == (partials == nullptr), SG_ERR_INVALID_ARG,
               "diffusion adjoint: give the forward field and the partials buffer together");
    auto s = (cudaStream_t)stream_;
    SG_ADJ_DISPATCH(dtype,
                    (diffusion2d_adj_kernel<float><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(
                        ny, nx, (float)k, (const float*)in_bar, (float*)out_bar, (const float*)field, partials)),
                    (diffusion2d_adj_kernel<double><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(
                        ny, nx, k, (const double*)in_bar, (double*)out_bar, (const double*)field, partials)));
    return launch_status("diffusion adjoint");
}

extern "C" int sg_advection_eno3_adj_2d(int dtype, int ny, int nx, const void* field, const void* velocity,
                                        double dt_by_dx, const void* in_bar, void* out_bar, void* velocity_bar,
                                        void* stream_) {
    SG_TRY(check_grid2d(ny, nx));
    SG_REQUIRE(field && velocity && in_bar && out_bar && in_bar != out_bar, SG_ERR_INVALID_ARG,
               "advection adjoint: bad pointers");
    auto s = (cudaStream_t)stream_;
    SG_ADJ_DISPATCH(dtype,
                    (eno3_2d_adj_kernel<float><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(
                        ny, nx, -(float)dt_by_dx, (const float*)field, (const float*)velocity,
                        (const float*)in_bar, (float*)out_bar, (float*)velocity_bar)),
                    (eno3_2d_adj_kernel<double><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(
                        ny, nx, -dt_by_dx, (const double*)field, (const double*)velocity, (const double*)in_bar,
                        (double*)out_bar, (double*)velocity_bar)));
    return launch_status("advection adjoint");
}

extern "C" int sg_forcing_curl_adj_2d(int dtype, int ny, int nx, const void* in_bar, void* forcing_bar,
                                      double prefactor, void* stream_) {
    SG_TRY(check_grid2d(ny, nx));
    SG_REQUIRE(in_bar && forcing_bar, SG_ERR_INVALID_ARG, "forcing curl adjoint: null pointer");
    auto s = (cudaStream_t)stream_;
    SG_ADJ_DISPATCH(dtype,
                    (fcurl2d_adj_kernel<float><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(
                        ny, nx, (float)prefactor, (const float*)in_bar, (float*)forcing_bar)),
                    (fcurl2d_adj_kernel<double><<<grid2d(ny, nx), dim3(32, 8), 0, s>>>(
                        ny, nx, prefactor, (const double*)in_bar, (double*)forcing_bar)));
    return launch_status("forcing curl adjoint");
}

// The domain-doubled solve is P^T C P with C circulant over a real, even
// Green's function, hence symmetric: its adjoint is the same solve.
extern "C" int sg_poisson_solve_adj(sg_poisson_plan p, const void* sol_bar, void* rhs_bar, int ncomp,
                                    int64_t comp_stride, void* stream) {
    return sg_poisson_solve(p, sol_bar, rhs_bar, ncomp, comp_stride, stream);
}

extern "C" sg_poisson_plan sg_flow_poisson_plan(sg_flow_plan p) { return p ? p->poisson : nullptr; }

template <typename T>
static int rsweep_launch(sg_flow_plan p, const void* g0, const void* g1, const void* w_a, const void* w_b,
                         const void* u, double k, double dt_by_dx, double pf, void* w_bar, void* u_bar, void* f_bar,
                         double* partials, cudaStream_t s) {
    RSweep2DParams<T> r{};
    r.ny = p->ny;
    r.nx = p->nx;
    r.width = p->width;
    r.g0 = (const T*)g0;
    r.g1 = (const T*)g1;
    r.cx = (const T*)p->coef_x;
    r.cy = (const T*)p->coef_y;
    r.k = (T)k;
    r.w_b = (const T*)w_b;
    r.partials = partials;
    r.inv_dx = -(T)dt_by_dx;
    r.w_a = (const T*)w_a;
    r.u = (const T*)u;
    r.pf = (T)pf;
    r.w_bar = (T*)w_bar;
    r.u_bar = (T*)u_bar;
    r.f_bar = (T*)f_bar;
    constexpr int TX = 32, TY = 16;
    rsweep2d_kernel<T, TX, TY><<<dim3(ceil_div(p->nx, TX), ceil_div(p->ny, TY)), dim3(32, 8), 0, s>>>(r);
    return launch_status("reverse sweep 2d");
}

extern "C" int sg_ns2d_reverse_sweep(sg_flow_plan p, const void* w_bar_after, const void* poisson_bar,
                                     const void* w_after_forcing, const void* w_after_advection, const void* velocity,
                                     const sg_step_scalars* scalars, void* w_bar_before, void* velocity_bar,
                                     void* forcing_bar, double* partials, void* stream_) {
    SG_REQUIRE(p && p->dim == 2, SG_ERR_INVALID_ARG, "reverse sweep: needs a 2D flow plan");
    SG_REQUIRE(w_bar_after && w_after_forcing && velocity && scalars && w_bar_before && velocity_bar,
               SG_ERR_INVALID_ARG, "reverse sweep: null argument");
    SG_REQUIRE(w_bar_before != w_bar_after && w_bar_before != poisson_bar, SG_ERR_INVALID_ARG,
               "reverse sweep: output must not alias an input (halo)");
    SG_REQUIRE((w_after_advection == nullptr) == (partials == nullptr), SG_ERR_INVALID_ARG,
               "reverse sweep: give w_after_advection and the partials buffer together");
    auto s = (cudaStream_t)stream_;
    const sg_step_scalars& sc = *scalars;
    if (p->dtype == SG_F32)
        return rsweep_launch<float>(p, w_bar_after, poisson_bar, w_after_forcing, w_after_advection, velocity,
                                    sc.diffusion_prefac, sc.advection_prefac, sc.forcing_prefac, w_bar_before,
                                    velocity_bar, forcing_bar, partials, s);
    return rsweep_launch<double>(p, w_bar_after, poisson_bar, w_after_forcing, w_after_advection, velocity,
                                 sc.diffusion_prefac, sc.advection_prefac, sc.forcing_prefac, w_bar_before,
                                 velocity_bar, forcing_bar, partials, s);
}

template <typename T>
static int ib_adj_launch(int dim, int nz, int ny, int nx, int n_lag, const int32_t* nearest, const void* weights,
                         const void* eul_forcing_bar, const double* F_const, double K, double C, double dt, double dx,
                         void* xi_bar, void* carry, double* v_bar, void* u_flow_bar, cudaStream_t s) {
    IBAdjParams<T> q{};
    q.dim = dim;
    q.nz = nz;
    q.ny = ny;
    q.nx = nx;
    q.n_lag = n_lag;
    q.nearest = nearest;
    q.weights = (const T*)weights;
    q.f_bar = (const T*)eul_forcing_bar;
    for (int d = 0; d < 3; ++d) q.F_const[d] = F_const ? F_const[d] : 0.0;
    q.K = K;
    q.C = C;
    q.dt = dt;
    q.dxd = dim == 2 ? dx * dx : dx * dx * dx;
    q.xi_bar = (T*)xi_bar;
    q.carry = (T*)carry;
    q.v_bar = v_bar;
    q.u_flow_bar = (T*)u_flow_bar;
    ib_adj_kernel<T><<<ceil_div((int64_t)n_lag * 32, 256), 256, 0, s>>>(q);
    return launch_status("ib interaction adjoint");
}

extern "C" int sg_ib_interaction_adj(int dtype, int dim, int nz, int ny, int nx, double dx, int n_lag,
                                     const int32_t* nearest, const void* weights, const void* eul_forcing_bar,
                                     const double* lag_forcing_bar_const, double stiffness, double damping,
                                     double xi_dt, void* position_mismatch_bar, void* velocity_mismatch_bar_carry,
                                     double* body_velocity_bar, void* flow_velocity_bar, void* stream_) {
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "ib adjoint: dim must be 2 or 3");
    SG_REQUIRE(n_lag >= 1 && nearest && weights && position_mismatch_bar && velocity_mismatch_bar_carry &&
                   body_velocity_bar && flow_velocity_bar,
               SG_ERR_INVALID_ARG, "ib adjoint: bad argument");
    if (dim == 2) nz = 1;
    auto s = (cudaStream_t)stream_;
    SG_ADJ_DISPATCH(dtype,
                    return ib_adj_launch<float>(dim, nz, ny, nx, n_lag, nearest, weights, eul_forcing_bar,
                                                lag_forcing_bar_const, stiffness, damping, xi_dt, dx,
                                                position_mismatch_bar, velocity_mismatch_bar_carry, body_velocity_bar,
                                                flow_velocity_bar, s),
                    return ib_adj_launch<double>(dim, nz, ny, nx, n_lag, nearest, weights, eul_forcing_bar,
                                                 lag_forcing_bar_const, stiffness, damping, xi_dt, dx,
                                                 position_mismatch_bar, velocity_mismatch_bar_carry,
                                                 body_velocity_bar, flow_velocity_bar, s));
    return SG_OK;
}

// Adjoint of the interpolation U = dx^dim sum phi u: u_bar += sum_i phi_i U_bar_i,
// with U_bar already scaled by dx^dim (sg_ib_interaction_adj does that).  It is
// the deterministic spreading kernel applied to U_bar, accumulating.
extern "C" int sg_ib_interp_adj(int dtype, int dim, int nz, int ny, int nx, int n_lag, const int32_t* nearest,
                                const void* weights, const void* flow_velocity_bar, void* eul_velocity_bar,
                                void* stream) {
    return sg_ib_spread(dtype, dim, nz, ny, nx, n_lag, nearest, weights, flow_velocity_bar, eul_velocity_bar, 0,
                        stream);
}

extern "C" int sg_lag_weighted_sum(int dtype, int dim, int n_lag, const void* lag_field, const double* weights3,
                                   double* acc, void* stream_) {
    SG_REQUIRE((dim == 2 || dim == 3) && n_lag >= 1 && lag_field && weights3 && acc, SG_ERR_INVALID_ARG,
               "lag weighted sum: bad argument");
    auto s = (cudaStream_t)stream_;
    SG_ADJ_DISPATCH(dtype,
                    (lag_weighted_sum_kernel<float><<<1, 32, 0, s>>>(dim, n_lag, (const float*)lag_field,
                                                                      weights3[0], weights3[1], weights3[2], acc)),
                    (lag_weighted_sum_kernel<double><<<1, 32, 0, s>>>(dim, n_lag, (const double*)lag_field,
                                                                       weights3[0], weights3[1], weights3[2], acc)));
    return launch_status("lag weighted sum");
}
