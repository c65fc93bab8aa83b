// Spreading of many markers (VirtualBoundaryForcing.py:232-274 with
// EulerianLagrangianGridCommunicator{2,3}D.py:267-384), deterministic and without
// floating-point atomics, in O(n log n).
//
// The reference adds every marker's F * phi into its 4^dim window serially in marker order, so
// each cell receives its contributions in ascending marker order.  sg_ib_spread keeps that order
// by letting the lowest-index marker touching a cell own it; deciding ownership scans the
// lower-index markers, which is quadratic in the marker count.  Here every (marker, window cell)
// pair becomes a key (the cell's linear index) and a value (the pair's index j * 4^dim + k, j the
// marker); a stable radix sort by key groups the pairs of each cell with their markers still in
// ascending order, and one thread per cell then sums the group into the cell in that order.  The
// sums are therefore the same to the bit as sg_ib_spread's.
#include <cub/device/device_radix_sort.cuh>

#include "ib.cuh"

namespace sg {

struct SortedScratch {
    int* keys_in;
    int* keys_out;
    int* vals_in;
    int* vals_out;
    void* temp;
    size_t temp_bytes;
};

static size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

static int end_bit_for(int64_t ncell) {
    int bits = 1;
    while (bits < 31 && ((int64_t)1 << bits) <= ncell) ++bits;
    return bits;
}

static size_t cub_temp_bytes(int64_t pairs, int end_bit) {
    size_t bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const int*)nullptr, (int*)nullptr, (const int*)nullptr,
                                    (int*)nullptr, (int)pairs, 0, end_bit);
    return bytes;
}

// The scratch for `pairs` (marker, cell) pairs: four int arrays and the sort's temporary storage.
static size_t sorted_scratch_bytes(int64_t pairs, int end_bit) {
    return 4 * align256(sizeof(int) * (size_t)pairs) + align256(cub_temp_bytes(pairs, end_bit));
}

static SortedScratch carve_scratch(void* base, int64_t pairs, int end_bit) {
    SortedScratch s;
    unsigned char* b = static_cast<unsigned char*>(base);
    const size_t arr = align256(sizeof(int) * (size_t)pairs);
    s.keys_in = reinterpret_cast<int*>(b);
    s.keys_out = reinterpret_cast<int*>(b + arr);
    s.vals_in = reinterpret_cast<int*>(b + 2 * arr);
    s.vals_out = reinterpret_cast<int*>(b + 3 * arr);
    s.temp = b + 4 * arr;
    s.temp_bytes = align256(cub_temp_bytes(pairs, end_bit));
    return s;
}

// Pair p = j * CELLS + k: window cell k of marker j; cells outside the grid (a marker reported out
// of domain) get the key ncell and sort past every real cell.
template <int DIM>
__global__ void __launch_bounds__(256) spread_pairs_kernel(int nz, int ny, int nx, int n_lag, const int32_t* nearest,
                                                           int* keys, int* vals) {
    constexpr int CELLS = DIM == 2 ? 16 : 64;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (int64_t)n_lag * CELLS) return;
    const int j = (int)(p / CELLS), k = (int)(p % CELLS);
    const int x = nearest[j] - 1 + (k & 3);
    const int y = nearest[n_lag + j] - 1 + ((k >> 2) & 3);
    const int z = DIM == 3 ? nearest[2 * n_lag + j] - 1 + (k >> 4) : 0;
    const bool inside = x >= 0 && x < nx && y >= 0 && y < ny && z >= 0 && z < nz;
    const int64_t ncell = (int64_t)nz * ny * nx;
    keys[p] = (int)(inside ? ((int64_t)z * ny + y) * nx + x : ncell);
    vals[p] = (int)p;
}

// Thread s heads the group of its key when the key before it differs; it adds the group's pairs,
// ascending in marker index, to the cell (or to zero when the field was reset).
template <typename T, int DIM>
__global__ void __launch_bounds__(256) spread_groups_kernel(int64_t pairs, int64_t ncell, int n_lag, int reset,
                                                            const int* keys, const int* vals, const T* weights,
                                                            const T* forcing, T* eul) {
    constexpr int CELLS = DIM == 2 ? 16 : 64;
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= pairs) return;
    const int key = keys[s];
    if (key >= ncell || (s > 0 && keys[s - 1] == key)) return;
    T acc[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = reset ? T(0) : eul[d * ncell + key];
    for (int64_t t = s; t < pairs && keys[t] == key; ++t) {
        const int p = vals[t];
        const int j = p / CELLS, k = p - j * CELLS;
        const T w = weights[(int64_t)k * n_lag + j];
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] = acc[d] + forcing[(int64_t)d * n_lag + j] * w;
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d) eul[d * ncell + key] = acc[d];
}

template <typename T>
static int spread_sorted(int dim, int nz, int ny, int nx, int n_lag, const int32_t* nearest, const T* weights,
                         const T* forcing, T* eul, int reset, void* scratch, int64_t scratch_bytes,
                         cudaStream_t stream) {
    const int cells = dim == 2 ? 16 : 64;
    const int64_t pairs = (int64_t)n_lag * cells;
    const int64_t ncell = (int64_t)nz * ny * nx;
    const int end_bit = end_bit_for(ncell);
    SG_REQUIRE((size_t)scratch_bytes >= sorted_scratch_bytes(pairs, end_bit), SG_ERR_INVALID_ARG,
               "ib sorted spread: scratch of %lld bytes, %zu needed", (long long)scratch_bytes,
               sorted_scratch_bytes(pairs, end_bit));
    SortedScratch s = carve_scratch(scratch, pairs, end_bit);
    if (reset) zero_kernel<T><<<ceil_div(dim * ncell, 256), 256, 0, stream>>>(dim * ncell, eul);
    const unsigned blocks = ceil_div(pairs, 256);
    if (dim == 2) spread_pairs_kernel<2><<<blocks, 256, 0, stream>>>(nz, ny, nx, n_lag, nearest, s.keys_in, s.vals_in);
    else spread_pairs_kernel<3><<<blocks, 256, 0, stream>>>(nz, ny, nx, n_lag, nearest, s.keys_in, s.vals_in);
    SG_TRY(launch_status("ib sorted spread: pairs"));
    size_t temp = s.temp_bytes;
    SG_TRY(cuda_status(cub::DeviceRadixSort::SortPairs(s.temp, temp, s.keys_in, s.keys_out, s.vals_in, s.vals_out,
                                                       (int)pairs, 0, end_bit, stream),
                       "ib sorted spread: sort"));
    if (dim == 2)
        spread_groups_kernel<T, 2><<<blocks, 256, 0, stream>>>(pairs, ncell, n_lag, reset, s.keys_out, s.vals_out,
                                                               weights, forcing, eul);
    else
        spread_groups_kernel<T, 3><<<blocks, 256, 0, stream>>>(pairs, ncell, n_lag, reset, s.keys_out, s.vals_out,
                                                               weights, forcing, eul);
    return launch_status("ib sorted spread: groups");
}

}  // namespace sg

extern "C" int64_t sg_ib_spread_sorted_scratch_bytes(int dim, int nz, int ny, int nx, int n_lag) {
    if ((dim != 2 && dim != 3) || n_lag < 1) return -1;
    if (dim == 2) nz = 1;
    const int64_t pairs = (int64_t)n_lag * (dim == 2 ? 16 : 64);
    if (pairs >= (1LL << 31)) return -1;
    return (int64_t)sg::sorted_scratch_bytes(pairs, sg::end_bit_for((int64_t)nz * ny * nx));
}

extern "C" int sg_ib_spread_sorted(int dtype, int dim, int nz, int ny, int nx, int n_lag, const int32_t* nearest,
                                   const void* weights, const void* forcing, void* eul_forcing, int reset,
                                   void* scratch, int64_t scratch_bytes, void* stream_) {
    using namespace sg;
    SG_REQUIRE(dim == 2 || dim == 3, SG_ERR_INVALID_ARG, "ib sorted spread: dim must be 2 or 3");
    SG_REQUIRE(nearest && weights && forcing && eul_forcing && scratch && n_lag >= 1, SG_ERR_INVALID_ARG,
               "ib sorted spread: bad argument");
    if (dim == 2) nz = 1;
    SG_REQUIRE((int64_t)nz * ny * nx < (1LL << 31) - 1, SG_ERR_SHAPE, "ib sorted spread: grid too large");
    SG_REQUIRE((int64_t)n_lag * (dim == 2 ? 16 : 64) < (1LL << 31), SG_ERR_SHAPE, "ib sorted spread: too many markers");
    auto stream = (cudaStream_t)stream_;
    if (dtype == SG_F32)
        return spread_sorted<float>(dim, nz, ny, nx, n_lag, nearest, (const float*)weights, (const float*)forcing,
                                    (float*)eul_forcing, reset, scratch, scratch_bytes, stream);
    SG_REQUIRE(dtype == SG_F64, SG_ERR_INVALID_ARG, "ib sorted spread: bad dtype");
    return spread_sorted<double>(dim, nz, ny, nx, n_lag, nearest, (const double*)weights, (const double*)forcing,
                                 (double*)eul_forcing, reset, scratch, scratch_bytes, stream);
}
