// Unbounded (free-space) Poisson solve by domain doubling, GB300-native.
//
// The reference (poisson_solver_{2,3}d/UnboundedPoissonSolverPYFFTW{2,3}D.py)
// zero-pads the right-hand side into a doubled box, takes a full R2C FFT,
// multiplies by the FFT of the even-reflected Green's function times dx^dim,
// takes the normalised C2R FFT and crops.  Here the same convolution is done
// without materialising the doubled box:
//   2D: rows R2C (zero-pad implicit) -> columns: FFT, * G, IFFT, crop -> rows C2R
//   3D: x rows R2C -> y lines FFT (expand to 2ny) -> z lines FFT * G IFFT crop
//       -> y lines IFFT crop -> x rows C2R (crop)
// The Green's function is real and even in every axis, so its transform is
// real and symmetric; it is stored once for k <= n per axis, with the 1/N
// normalisation and dx^dim folded in.  It is built in FP64 on the GPU with the
// same kernels instantiated for double, then rounded to the field precision.
#include <cmath>
#include <vector>

#include "poisson.cuh"
#include "fft_reg.cuh"

namespace sg {

template <typename T>
__global__ void twiddle_kernel(cplx_t<T>* out, int count, int n) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= count) return;
    double s, c;
    // exp(-2 pi i m / n)
    sincospi(-2.0 * (double)m / (double)n, &s, &c);
    out[m] = cmake<cplx_t<T>>((T)c, (T)s);
}

template <typename T>
static int make_twiddles(void** dst, int count, int n, cudaStream_t stream, int64_t* bytes) {
    const size_t sz = (size_t)count * sizeof(cplx_t<T>);
    SG_TRY(cuda_status(cudaMalloc(dst, sz), "twiddle alloc"));
    if (bytes) *bytes += (int64_t)sz;
    twiddle_kernel<T><<<ceil_div(count, 256), 256, 0, stream>>>(reinterpret_cast<cplx_t<T>*>(*dst), count, n);
    return launch_status("twiddle kernel");
}

// numpy.linspace(0, stop, num)[i] in double (the endpoint is set exactly)
__device__ __forceinline__ double linspace_at(int i, int num, double stop) {
    if (i == num - 1) return stop;
    return (double)i * (stop / (double)(num - 1));
}

// Even-reflected Green's function on the doubled 2D grid
// (UnboundedPoissonSolverPYFFTW2D.py:47-64), in double.
__global__ void greens_2d_kernel(double* g, int ny2, int nx2, double x_range, double y_range, double dx) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)ny2 * nx2) return;
    const int i = (int)(idx % nx2), j = (int)(idx / nx2);
    const double x = linspace_at(i, nx2, 2.0 * x_range - dx);
    const double y = linspace_at(j, ny2, 2.0 * y_range - dx);
    const double rx = fmin(x, 2.0 * x_range - x), ry = fmin(y, 2.0 * y_range - y);
    const double r = sqrt(rx * rx + ry * ry);
    const double pi = 3.14159265358979323846;
    double v = -log(r) / (2.0 * pi);
    if (idx == 0) v = -(2.0 * log(dx / sqrt(pi)) - 1.0) / (4.0 * pi);
    g[idx] = v;
}

// Even-reflected 1/(4 pi r) on the doubled 3D grid, G(0) = 1/(4 pi dx)
// (UnboundedPoissonSolverPYFFTW3D.py:56-79), in double.
__global__ void greens_3d_kernel(double* g, int nz2, int ny2, int nx2, double x_range, double y_range,
                                 double z_range, double dx) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)nz2 * ny2 * nx2) return;
    const int i = (int)(idx % nx2);
    const int j = (int)((idx / nx2) % ny2);
    const int k = (int)(idx / ((int64_t)nx2 * ny2));
    const double x = linspace_at(i, nx2, 2.0 * x_range - dx);
    const double y = linspace_at(j, ny2, 2.0 * y_range - dx);
    const double z = linspace_at(k, nz2, 2.0 * z_range - dx);
    const double rx = fmin(x, 2.0 * x_range - x), ry = fmin(y, 2.0 * y_range - y),
                 rz = fmin(z, 2.0 * z_range - z);
    const double r = sqrt(rx * rx + ry * ry + rz * rz);
    const double pi = 3.14159265358979323846;
    double v = (1.0 / r) / (4.0 * pi);
    if (idx == 0) v = 1.0 / (4.0 * pi * dx);
    g[idx] = v;
}

// table[ks][(ms)][kx] = Re(spec) * scale for ks <= nk, ms <= nm, kx <= nx
template <typename T>
__global__ void greens_extract_kernel(T* table, const double2* spec, int nk, int nm, int nxp1,
                                      int64_t spec_k_stride, int64_t spec_m_stride, double scale) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)(nk + 1) * (nm + 1) * nxp1;
    if (idx >= total) return;
    const int kx = (int)(idx % nxp1);
    const int m = (int)((idx / nxp1) % (nm + 1));
    const int k = (int)(idx / ((int64_t)nxp1 * (nm + 1)));
    table[idx] = (T)(spec[k * spec_k_stride + m * spec_m_stride + kx].x * scale);
}

template <typename T>
static int build_greens(sg_poisson_plan_s* p, cudaStream_t stream) {
    const int nx = p->nx, ny = p->ny, nz = p->dim == 3 ? p->nz : 1;
    const double dx = p->dx;
    const double y_range = p->x_range * ((double)ny / nx);
    const double z_range = p->x_range * ((double)nz / nx);
    void *twx = nullptr, *twxl = nullptr, *twy = nullptr, *twz = nullptr;
    double* g = nullptr;
    double2* spec = nullptr;
    int status = SG_OK;
    const int64_t nreal = (int64_t)(p->dim == 3 ? 2 * nz : 1) * 2 * ny * 2 * nx;
    const int64_t ncplx = (int64_t)(p->dim == 3 ? 2 * nz : 1) * 2 * ny * (nx + 1);
    do {
        if ((status = make_twiddles<double>(&twx, nx, nx, stream, nullptr))) break;
        if ((status = make_twiddles<double>(&twxl, nx + 1, 2 * nx, stream, nullptr))) break;
        if ((status = make_twiddles<double>(&twy, 2 * ny, 2 * ny, stream, nullptr))) break;
        if (p->dim == 3 && (status = make_twiddles<double>(&twz, 2 * nz, 2 * nz, stream, nullptr))) break;
        if ((status = cuda_status(cudaMalloc(&g, nreal * sizeof(double)), "greens alloc"))) break;
        if ((status = cuda_status(cudaMalloc(&spec, ncplx * sizeof(double2)), "greens spectrum alloc"))) break;
        if (p->dim == 2) {
            greens_2d_kernel<<<ceil_div(nreal, 256), 256, 0, stream>>>(g, 2 * ny, 2 * nx, p->x_range, y_range, dx);
        } else {
            greens_3d_kernel<<<ceil_div(nreal, 256), 256, 0, stream>>>(g, 2 * nz, 2 * ny, 2 * nx, p->x_range,
                                                                      y_range, z_range, dx);
        }
        if ((status = launch_status("greens kernel"))) break;
        RowsR2CParams<double> r{};
        r.in = g;
        r.in_map = row_map(2 * ny, 2 * nx, p->dim == 3 ? 2 * nz : 1, (int64_t)2 * ny * 2 * nx);
        r.n_in = 2 * nx;
        r.out = spec;
        r.out_map = row_map(2 * ny, nx + 1, p->dim == 3 ? 2 * nz : 1, (int64_t)2 * ny * (nx + 1));
        r.n_rows = (p->dim == 3 ? 2 * nz : 1) * 2 * ny;
        r.st = p->st_x;
        r.tw_m = (const double2*)twx;
        r.tw_l = (const double2*)twxl;
        if ((status = launch_rows_r2c<double>(r, stream))) break;
        LinesParams<double> ly{};
        ly.in = spec;
        ly.out = spec;
        ly.n_in = 2 * ny;
        ly.n_out = 2 * ny;
        ly.inner = nx + 1;
        ly.line_stride = nx + 1;
        ly.outer_stride = (int64_t)2 * ny * (nx + 1);
        ly.n_outer = p->dim == 3 ? 2 * nz : 1;
        ly.st = p->st_y;
        ly.tw = (const double2*)twy;
        if ((status = launch_lines<double, LINE_FWD>(ly, stream))) break;
        if (p->dim == 3) {
            LinesParams<double> lz{};
            lz.in = spec;
            lz.out = spec;
            lz.n_in = 2 * nz;
            lz.n_out = 2 * nz;
            lz.inner = 2 * ny * (nx + 1);
            lz.line_stride = (int64_t)2 * ny * (nx + 1);
            lz.outer_stride = 0;
            lz.n_outer = 1;
            lz.st = p->st_z;
            lz.tw = (const double2*)twz;
            if ((status = launch_lines<double, LINE_FWD>(lz, stream))) break;
        }
        // fold dx^dim and the 1/N of the unnormalised inverse into the table
        double scale;
        int64_t table_elems;
        if (p->dim == 2) {
            scale = dx * dx / (4.0 * ny * nx);
            table_elems = (int64_t)(ny + 1) * (nx + 1);
        } else {
            scale = dx * dx * dx / (8.0 * nz * ny * nx);
            table_elems = (int64_t)(nz + 1) * (ny + 1) * (nx + 1);
        }
        if ((status = cuda_status(cudaMalloc(&p->greens, table_elems * sizeof(T)), "greens table alloc"))) break;
        p->bytes += table_elems * sizeof(T);
        if (p->dim == 2) {
            greens_extract_kernel<T><<<ceil_div(table_elems, 256), 256, 0, stream>>>(
                (T*)p->greens, spec, 0, ny, nx + 1, 0, nx + 1, scale);
        } else {
            greens_extract_kernel<T><<<ceil_div(table_elems, 256), 256, 0, stream>>>(
                (T*)p->greens, spec, nz, ny, nx + 1, (int64_t)2 * ny * (nx + 1), nx + 1, scale);
        }
        if ((status = launch_status("greens extract"))) break;
        status = cuda_status(cudaStreamSynchronize(stream), "greens build sync");
    } while (0);
    cudaFree(twx);
    cudaFree(twxl);
    cudaFree(twy);
    cudaFree(twz);
    cudaFree(g);
    cudaFree(spec);
    return status;
}

template <typename T>
static int plan_init(sg_poisson_plan_s* p, cudaStream_t stream) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    SG_TRY(make_twiddles<T>(&p->tw_x, nx, nx, stream, &p->bytes));
    SG_TRY(make_twiddles<T>(&p->tw_xl, nx + 1, 2 * nx, stream, &p->bytes));
    SG_TRY(make_twiddles<T>(&p->tw_y, 2 * ny, 2 * ny, stream, &p->bytes));
    if (p->dim == 3) SG_TRY(make_twiddles<T>(&p->tw_z, 2 * nz, 2 * nz, stream, &p->bytes));
    p->spec_comp_elems = p->dim == 2 ? (int64_t)ny * (nx + 1) : (int64_t)nz * 2 * ny * (nx + 1);
    const size_t spec_bytes = (size_t)p->max_comp * p->spec_comp_elems * sizeof(cplx_t<T>);
    SG_TRY(cuda_status(cudaMalloc(&p->spec, spec_bytes), "spectrum workspace alloc"));
    p->bytes += (int64_t)spec_bytes;
    return build_greens<T>(p, stream);
}

template <typename T>
int poisson_load_rows(sg_poisson_plan_s* p, const T* rhs, int ncomp, int64_t comp_stride, cudaStream_t stream) {
    RowsR2CParams<T> r{};
    r.in = rhs;
    r.n_in = p->nx;
    r.out = reinterpret_cast<cplx_t<T>*>(p->spec);
    r.st = p->st_x;
    r.tw_m = (const cplx_t<T>*)p->tw_x;
    r.tw_l = (const cplx_t<T>*)p->tw_xl;
    if (p->dim == 2) {
        r.in_map = row_map(p->ny, p->nx, 1, 0, comp_stride);
        r.out_map = row_map(p->ny, p->nx + 1, 1, 0, p->spec_comp_elems);
        r.n_rows = ncomp * p->ny;
    } else {
        r.in_map = row_map(p->ny, p->nx, p->nz, (int64_t)p->ny * p->nx, comp_stride);
        r.out_map = row_map(p->ny, p->nx + 1, p->nz, (int64_t)2 * p->ny * (p->nx + 1), p->spec_comp_elems);
        r.n_rows = ncomp * p->nz * p->ny;
    }
    return launch_rows_r2c<T>(r, stream);
}

template <typename T>
int poisson_spectral_passes(sg_poisson_plan_s* p, int ncomp, cudaStream_t stream) {
    using C = cplx_t<T>;
    C* spec = reinterpret_cast<C*>(p->spec);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    if (p->dim == 2) {
        LinesParams<T> l{};
        l.in = spec;
        l.out = spec;
        l.n_in = ny;
        l.n_out = ny;
        l.inner = nx + 1;
        l.line_stride = nx + 1;
        l.outer_stride = p->spec_comp_elems;
        l.n_outer = ncomp;
        l.st = p->st_y;
        l.tw = (const C*)p->tw_y;
        l.g.table = (const T*)p->greens;
        l.g.k_stride = nx + 1;
        l.g.inner_div = nx + 1;
        l.g.m_mod = 0;
        l.g.m_stride = 0;
        return launch_lines<T, LINE_CONV>(l, stream);
    }
    for (int pass = 0; pass < 3; ++pass) SG_TRY(poisson_spectral_pass3d<T>(p, ncomp, pass, stream));
    return SG_OK;
}

// fp32 y and z passes of lengths 256 and 512 on the register line kernels (fft_reg.cuh): y lines
// are slabs of nx + 1 adjacent lines per (component, z plane), z lines one slab of 2 ny (nx + 1)
// lines per component.  Returns SG_ERR_UNSUPPORTED for the other lengths.
static int reg_pass3d(sg_poisson_plan_s* p, int ncomp, int pass, cudaStream_t stream) {
    float2* spec = reinterpret_cast<float2*>(p->spec);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    RegLinesParams r{};
    r.in = spec;
    r.out = spec;
    if (pass == 1) {
        const int64_t plane = (int64_t)2 * ny * (nx + 1);
        SG_REQUIRE((int64_t)ncomp * plane < (1LL << 31), SG_ERR_SHAPE, "z pass: too many lines");
        r.n_lines = (int)(ncomp * plane);
        r.slab_lines = (int)plane;
        r.slab_stride = p->spec_comp_elems;
        r.stride = plane;
        r.n_in = nz;
        r.n_out = nz;
        r.tw = (const float2*)p->tw_z;
        r.g = (const float*)p->greens;
        r.g_kstride = (int64_t)(ny + 1) * (nx + 1);
        r.g_mstride = nx + 1;
        r.g_div = nx + 1;
        r.g_mmod = 2 * ny;
        // the components of one 16-line group in consecutive blocks: their Green's rows are shared
        r.interleave = (ncomp > 1 && plane % rl::kLines == 0) ? ncomp : 1;
        return launch_reg_lines<RL_CONV>(r, 2 * nz, stream);
    }
    SG_REQUIRE((int64_t)ncomp * nz * (nx + 1) < (1LL << 31), SG_ERR_SHAPE, "y pass: too many lines");
    r.n_lines = ncomp * nz * (nx + 1);
    r.slab_lines = nx + 1;
    r.slab_stride = (int64_t)2 * ny * (nx + 1);
    r.stride = nx + 1;
    r.tw = (const float2*)p->tw_y;
    // the y passes wait on their own input (long-scoreboard bound): each block asks L2 for the
    // block two thirds of a wave of resident blocks (three per SM) ahead -- at 256^3 the y inverse
    // took 0.280 ms with 2 x SMs, 0.288 with 3 x SMs and 0.388 with 6 x SMs
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    r.prefetch_ahead = 2 * sms;
    if (pass == 0) {
        r.n_in = ny;
        r.n_out = 2 * ny;
        return launch_reg_lines<RL_FWD>(r, 2 * ny, stream);
    }
    r.n_in = 2 * ny;
    r.n_out = ny;
    return launch_reg_lines<RL_INV>(r, 2 * ny, stream);
}

static bool reg_length(int n) { return n == 256 || n == 512; }

template <typename T>
int poisson_spectral_pass3d(sg_poisson_plan_s* p, int ncomp, int pass, cudaStream_t stream) {
    using C = cplx_t<T>;
    C* spec = reinterpret_cast<C*>(p->spec);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    if constexpr (sizeof(T) == 4) {
        if (reg_length(pass == 1 ? 2 * nz : 2 * ny)) return reg_pass3d(p, ncomp, pass, stream);
    }
    // y lines: forward (Ny non-zero points -> 2 Ny bins) or inverse (keep Ny)
    LinesParams<T> ly{};
    ly.in = spec;
    ly.out = spec;
    ly.n_in = ny;
    ly.n_out = 2 * ny;
    ly.inner = nx + 1;
    ly.line_stride = nx + 1;
    ly.outer_stride = (int64_t)2 * ny * (nx + 1);
    ly.n_outer = ncomp * nz;
    ly.st = p->st_y;
    ly.tw = (const C*)p->tw_y;
    if (pass == 0) return launch_lines<T, LINE_FWD>(ly, stream);
    if (pass == 2) {
        ly.n_in = 2 * ny;
        ly.n_out = ny;
        return launch_lines<T, LINE_INV>(ly, stream);
    }
    // z: forward (Nz non-zero), * G, inverse, keep Nz
    LinesParams<T> lz{};
    lz.in = spec;
    lz.out = spec;
    lz.n_in = nz;
    lz.n_out = nz;
    lz.inner = 2 * ny * (nx + 1);
    lz.line_stride = (int64_t)2 * ny * (nx + 1);
    lz.outer_stride = p->spec_comp_elems;
    lz.n_outer = ncomp;
    lz.st = p->st_z;
    lz.tw = (const C*)p->tw_z;
    lz.g.table = (const T*)p->greens;
    lz.g.k_stride = (int64_t)(ny + 1) * (nx + 1);
    lz.g.inner_div = nx + 1;
    lz.g.m_mod = 2 * ny;
    lz.g.m_stride = nx + 1;
    return launch_lines<T, LINE_CONV>(lz, stream);
}

template <typename T>
int poisson_store_rows(sg_poisson_plan_s* p, T* sol, int ncomp, int64_t comp_stride, cudaStream_t stream) {
    RowsC2RParams<T> r{};
    r.in = reinterpret_cast<const cplx_t<T>*>(p->spec);
    r.out = sol;
    r.n_out = p->nx;
    r.st = p->st_x;
    r.tw_m = (const cplx_t<T>*)p->tw_x;
    r.tw_l = (const cplx_t<T>*)p->tw_xl;
    if (p->dim == 2) {
        r.in_map = row_map(p->ny, p->nx + 1, 1, 0, p->spec_comp_elems);
        r.out_map = row_map(p->ny, p->nx, 1, 0, comp_stride);
        r.n_rows = ncomp * p->ny;
    } else {
        r.in_map = row_map(p->ny, p->nx + 1, p->nz, (int64_t)2 * p->ny * (p->nx + 1), p->spec_comp_elems);
        r.out_map = row_map(p->ny, p->nx, p->nz, (int64_t)p->ny * p->nx, comp_stride);
        r.n_rows = ncomp * p->nz * p->ny;
        // 3D fp32 rows of 256 complex points: the register row kernel (fft_reg.cuh)
        if constexpr (sizeof(T) == 4)
            if (p->nx == rl::kRowM && r.n_out <= p->nx) return launch_reg_rows_c2r(r, stream);
    }
    return launch_rows_c2r<T>(r, stream);
}

template int poisson_load_rows<float>(sg_poisson_plan_s*, const float*, int, int64_t, cudaStream_t);
template int poisson_load_rows<double>(sg_poisson_plan_s*, const double*, int, int64_t, cudaStream_t);
template int poisson_spectral_passes<float>(sg_poisson_plan_s*, int, cudaStream_t);
template int poisson_spectral_passes<double>(sg_poisson_plan_s*, int, cudaStream_t);
template int poisson_spectral_pass3d<float>(sg_poisson_plan_s*, int, int, cudaStream_t);
template int poisson_spectral_pass3d<double>(sg_poisson_plan_s*, int, int, cudaStream_t);
template int poisson_store_rows<float>(sg_poisson_plan_s*, float*, int, int64_t, cudaStream_t);
template int poisson_store_rows<double>(sg_poisson_plan_s*, double*, int, int64_t, cudaStream_t);

static void plan_free(sg_poisson_plan_s* p) {
    if (!p) return;
    cudaFree(p->tw_x);
    cudaFree(p->tw_xl);
    cudaFree(p->tw_y);
    cudaFree(p->tw_z);
    cudaFree(p->greens);
    cudaFree(p->spec);
    delete p;
}

int poisson_plan_create_impl(int dim, int nz, int ny, int nx, double x_range, int dtype, int max_comp,
                             sg_poisson_plan_s** out) {
    SG_REQUIRE(out != nullptr, SG_ERR_INVALID_ARG, "poisson plan: null output pointer");
    *out = nullptr;
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "poisson plan: dim must be 2 or 3 (got %d)", dim);
    SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, SG_ERR_INVALID_ARG, "poisson plan: bad dtype %d", dtype);
    if (dim == 2) nz = 1;
    SG_REQUIRE(nx >= 2 && ny >= 2 && nz >= 1 && nx % 2 == 0, SG_ERR_SHAPE,
               "poisson plan: need even nx >= 2 and ny >= 2 (got nz=%d ny=%d nx=%d)", nz, ny, nx);
    SG_REQUIRE(max_comp >= 1 && max_comp <= 3, SG_ERR_INVALID_ARG, "poisson plan: max_comp must be 1..3");
    SG_REQUIRE(x_range > 0, SG_ERR_INVALID_ARG, "poisson plan: x_range must be positive");
    auto* p = new sg_poisson_plan_s();
    p->dim = dim;
    p->nz = nz;
    p->ny = ny;
    p->nx = nx;
    p->dtype = dtype;
    p->max_comp = max_comp;
    p->x_range = x_range;
    p->dx = dtype == SG_F32 ? (double)(float)(x_range / nx) : x_range / nx;
    bool ok = fft_factor(nx, p->st_x) && fft_factor(2 * ny, p->st_y) && (dim == 2 || fft_factor(2 * nz, p->st_z));
    if (!ok) {
        delete p;
        set_last_error("poisson plan: FFT lengths (nx=%d, 2ny=%d, 2nz=%d) must factor into 2, 3, 5 and 7", nx, 2 * ny,
                       2 * nz);
        return SG_ERR_UNSUPPORTED;
    }
    cudaStream_t stream = nullptr;
    int status = dtype == SG_F32 ? plan_init<float>(p, stream) : plan_init<double>(p, stream);
    if (status == SG_OK) status = cuda_status(cudaDeviceSynchronize(), "poisson plan create");
    if (status != SG_OK) {
        plan_free(p);
        return status;
    }
    *out = p;
    return SG_OK;
}

void poisson_plan_free(sg_poisson_plan_s* p) { plan_free(p); }

}  // namespace sg

extern "C" int sg_poisson_plan_create(int dim, int nz, int ny, int nx, double x_range, int dtype, int max_comp,
                                      sg_poisson_plan* plan_out) {
    return sg::poisson_plan_create_impl(dim, nz, ny, nx, x_range, dtype, max_comp, plan_out);
}

extern "C" int sg_poisson_plan_destroy(sg_poisson_plan plan) {
    sg::poisson_plan_free(plan);
    return SG_OK;
}

extern "C" int64_t sg_poisson_plan_bytes(sg_poisson_plan plan) { return plan ? plan->bytes : 0; }

extern "C" int sg_poisson_solve(sg_poisson_plan p, const void* rhs, void* sol, int ncomp, int64_t comp_stride,
                                void* stream_) {
    SG_REQUIRE(p && rhs && sol, SG_ERR_INVALID_ARG, "poisson solve: null argument");
    SG_REQUIRE(ncomp >= 1 && ncomp <= p->max_comp, SG_ERR_INVALID_ARG,
               "poisson solve: ncomp %d outside 1..%d", ncomp, p->max_comp);
    auto stream = (cudaStream_t)stream_;
    if (p->dtype == SG_F32) {
        SG_TRY(sg::poisson_load_rows<float>(p, (const float*)rhs, ncomp, comp_stride, stream));
        SG_TRY(sg::poisson_spectral_passes<float>(p, ncomp, stream));
        return sg::poisson_store_rows<float>(p, (float*)sol, ncomp, comp_stride, stream);
    }
    SG_TRY(sg::poisson_load_rows<double>(p, (const double*)rhs, ncomp, comp_stride, stream));
    SG_TRY(sg::poisson_spectral_passes<double>(p, ncomp, stream));
    return sg::poisson_store_rows<double>(p, (double*)sol, ncomp, comp_stride, stream);
}

// ===========================================================================
// Allocation-free 2D solve.
//
// Some callers cannot call cudaMalloc at all: code that runs while a CUDA
// graph is being captured, a host application whose memory pools are owned by
// another framework and must not grow, or an embedding that forbids device
// allocation after start-up.  For them sg_poisson2d_solve_noalloc solves the
// same unbounded 2D Poisson problem as sg_poisson_solve without any allocation:
// its FFT workspace, Green's table and twiddles, and the FP64 buffers used to
// build the table, live in one file-scope __device__ array of fixed size,
// which every GPU that loads this library holds until the process exits.
//
// Limits: fp32 only, ny <= 256 and nx <= 512 (nx even; nx, 2 ny with prime
// factors 2, 3, 5, 7 only).  Larger grids are rejected with SG_ERR_SHAPE.
// ===========================================================================
namespace sg {

constexpr int kNoAllocMaxNy = 256;
constexpr int kNoAllocMaxNx = 512;

// byte offsets inside the static scratch (each region 256-byte aligned)
constexpr size_t na_align(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kNaGreens64 = 0;  // double G, (2 ny) x (2 nx)
constexpr size_t kNaSpec64 = na_align(kNaGreens64 + sizeof(double) * 2 * kNoAllocMaxNy * 2 * kNoAllocMaxNx);
constexpr size_t kNaTw64 = na_align(kNaSpec64 + sizeof(double2) * 2 * kNoAllocMaxNy * (kNoAllocMaxNx + 1));
// double twiddles: nx, nx + 1, 2 ny entries
constexpr size_t kNaTable = na_align(kNaTw64 + sizeof(double2) * (2 * kNoAllocMaxNx + 1 + 2 * kNoAllocMaxNy));
constexpr size_t kNaSpec = na_align(kNaTable + sizeof(float) * (kNoAllocMaxNy + 1) * (kNoAllocMaxNx + 1));
constexpr size_t kNaTw = na_align(kNaSpec + sizeof(float2) * kNoAllocMaxNy * (kNoAllocMaxNx + 1));
constexpr size_t kNaBytes = na_align(kNaTw + sizeof(float2) * (2 * kNoAllocMaxNx + 1 + 2 * kNoAllocMaxNy));

// The scratch.  Host code must not use this name as an address: it is a host
// stand-in; the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

struct NoAllocState {
    unsigned char* base = nullptr;  // device address of g_noalloc_scratch
    bool table_ready = false;
    int ny = 0, nx = 0;
    double x_range = 0.0;
};
constexpr int kNoAllocMaxDevices = 64;
static NoAllocState g_noalloc_state[kNoAllocMaxDevices];

static int noalloc_build(NoAllocState& st, sg_poisson_plan_s& p, cudaStream_t stream) {
    unsigned char* b = st.base;
    const int nx = p.nx, ny = p.ny;
    double* g = reinterpret_cast<double*>(b + kNaGreens64);
    double2* spec64 = reinterpret_cast<double2*>(b + kNaSpec64);
    double2* tw64x = reinterpret_cast<double2*>(b + kNaTw64);
    double2* tw64xl = tw64x + nx;
    double2* tw64y = tw64xl + (nx + 1);
    float2* twx = reinterpret_cast<float2*>(b + kNaTw);
    float2* twxl = twx + nx;
    float2* twy = twxl + (nx + 1);
    twiddle_kernel<double><<<ceil_div(nx, 256), 256, 0, stream>>>(tw64x, nx, nx);
    twiddle_kernel<double><<<ceil_div(nx + 1, 256), 256, 0, stream>>>(tw64xl, nx + 1, 2 * nx);
    twiddle_kernel<double><<<ceil_div(2 * ny, 256), 256, 0, stream>>>(tw64y, 2 * ny, 2 * ny);
    twiddle_kernel<float><<<ceil_div(nx, 256), 256, 0, stream>>>(twx, nx, nx);
    twiddle_kernel<float><<<ceil_div(nx + 1, 256), 256, 0, stream>>>(twxl, nx + 1, 2 * nx);
    twiddle_kernel<float><<<ceil_div(2 * ny, 256), 256, 0, stream>>>(twy, 2 * ny, 2 * ny);
    SG_TRY(launch_status("noalloc twiddles"));
    const int64_t nreal = (int64_t)2 * ny * 2 * nx;
    const double y_range = p.x_range * ((double)ny / nx);
    greens_2d_kernel<<<ceil_div(nreal, 256), 256, 0, stream>>>(g, 2 * ny, 2 * nx, p.x_range, y_range, p.dx);
    SG_TRY(launch_status("noalloc greens"));
    RowsR2CParams<double> r{};
    r.in = g;
    r.in_map = row_map(2 * ny, 2 * nx);
    r.n_in = 2 * nx;
    r.out = spec64;
    r.out_map = row_map(2 * ny, nx + 1);
    r.n_rows = 2 * ny;
    r.st = p.st_x;
    r.tw_m = tw64x;
    r.tw_l = tw64xl;
    SG_TRY(launch_rows_r2c<double>(r, stream));
    LinesParams<double> ly{};
    ly.in = spec64;
    ly.out = spec64;
    ly.n_in = 2 * ny;
    ly.n_out = 2 * ny;
    ly.inner = nx + 1;
    ly.line_stride = nx + 1;
    ly.outer_stride = 0;
    ly.n_outer = 1;
    ly.st = p.st_y;
    ly.tw = tw64y;
    SG_TRY((launch_lines<double, LINE_FWD>(ly, stream)));
    const int64_t table_elems = (int64_t)(ny + 1) * (nx + 1);
    greens_extract_kernel<float><<<ceil_div(table_elems, 256), 256, 0, stream>>>(
        reinterpret_cast<float*>(b + kNaTable), spec64, 0, ny, nx + 1, 0, nx + 1, p.dx * p.dx / (4.0 * ny * nx));
    return launch_status("noalloc greens extract");
}

}  // namespace sg

extern "C" int sg_poisson2d_solve_noalloc(int ny, int nx, double x_range, const float* rhs, float* sol,
                                          void* stream_) {
    using namespace sg;
    SG_REQUIRE(rhs && sol, SG_ERR_INVALID_ARG, "poisson2d noalloc: null field pointer");
    SG_REQUIRE(ny >= 2 && nx >= 2 && nx % 2 == 0 && ny <= kNoAllocMaxNy && nx <= kNoAllocMaxNx, SG_ERR_SHAPE,
               "poisson2d noalloc: grid (%d, %d) outside the static scratch limit (ny <= %d, even nx <= %d)", ny,
               nx, kNoAllocMaxNy, kNoAllocMaxNx);
    SG_REQUIRE(x_range > 0, SG_ERR_INVALID_ARG, "poisson2d noalloc: x_range must be positive");
    sg_poisson_plan_s p;
    p.dim = 2;
    p.nz = 1;
    p.ny = ny;
    p.nx = nx;
    p.dtype = SG_F32;
    p.max_comp = 1;
    p.x_range = x_range;
    p.dx = (double)(float)(x_range / nx);
    if (!(fft_factor(nx, p.st_x) && fft_factor(2 * ny, p.st_y))) {
        set_last_error("poisson2d noalloc: nx=%d and 2ny=%d must factor into 2, 3, 5 and 7", nx, 2 * ny);
        return SG_ERR_UNSUPPORTED;
    }
    int dev = 0;
    SG_TRY(cuda_status(cudaGetDevice(&dev), "poisson2d noalloc: cudaGetDevice"));
    SG_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, SG_ERR_INVALID_ARG, "poisson2d noalloc: device %d", dev);
    NoAllocState& st = g_noalloc_state[dev];
    if (st.base == nullptr) {
        // once per device, with that device current
        void* addr = nullptr;
        SG_TRY(cuda_status(cudaGetSymbolAddress(&addr, g_noalloc_scratch), "poisson2d noalloc: symbol address"));
        st.base = static_cast<unsigned char*>(addr);
    }
    auto stream = (cudaStream_t)stream_;
    if (!st.table_ready || st.ny != ny || st.nx != nx || st.x_range != x_range) {
        // A rebuild queued on a capturing stream would only be recorded, not run: refuse it rather
        // than mark a table ready that no eager work has built.
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        SG_TRY(cuda_status(cudaStreamIsCapturing(stream, &cs), "poisson2d noalloc: capture status"));
        SG_REQUIRE(cs == cudaStreamCaptureStatusNone, SG_ERR_INVALID_ARG,
                   "poisson2d noalloc: the grid (%d, %d, x_range %g) needs a table rebuild, which cannot be "
                   "queued while the stream is capturing; call once on this grid outside capture first",
                   ny, nx, x_range);
        st.table_ready = false;
        SG_TRY(noalloc_build(st, p, stream));
        st.table_ready = true;
        st.ny = ny;
        st.nx = nx;
        st.x_range = x_range;
    }
    unsigned char* b = st.base;
    float2* twx = reinterpret_cast<float2*>(b + kNaTw);
    p.tw_x = twx;
    p.tw_xl = twx + nx;
    p.tw_y = twx + nx + (nx + 1);
    p.greens = b + kNaTable;
    p.spec = b + kNaSpec;
    p.spec_comp_elems = (int64_t)ny * (nx + 1);
    SG_TRY(poisson_load_rows<float>(&p, rhs, 1, 0, stream));
    SG_TRY(poisson_spectral_passes<float>(&p, 1, stream));
    return poisson_store_rows<float>(&p, sol, 1, 0, stream);
}
