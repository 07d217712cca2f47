// Particle positions in id order, written into caller memory, with no
// allocation by the library.
//
// The same three steps as the context's readback (flag the ids, exclusive
// scan of the flags, scatter), but working in one file-scope device array
// instead of buffers allocated with the context, so that a caller whose
// device memory all comes from its own allocator, or who must not let a
// cudaMalloc stall the device in the middle of a frame loop, can still order
// the particles it holds.
#include <string>

#include "../../include/flip3d.h"
#include "flip_device.cuh"

namespace flip {
int record_error(int code, const std::string &msg);   // sets flip_last_error()
}

// Scratch shared by every call on a device: one rank word per id (plus the
// total), then the per-tile sums of the scan.  Sized for FLIP_NOALLOC_MAX_IDS
// ids: (2^20 + 1 + 1026) ints, about 4 MiB, held by every GPU that loads the
// library until the process exits.
#define NA_TILE 1024
#define NA_MAX_TILES ((FLIP_NOALLOC_MAX_IDS + 1 + NA_TILE - 1) / NA_TILE + 1)
static __device__ __align__(256) int g_noalloc_scratch[FLIP_NOALLOC_MAX_IDS + 1 + NA_MAX_TILES];

namespace {

constexpr int TPB = 256;   // 4 ids per thread per scan tile

__global__ void k_na_clear(int *rank, int count) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) rank[t] = 0;
}

__global__ void k_na_flag(const unsigned int *ids, int n, int idSpace, int *rank) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n && ids[t] < (unsigned int)idSpace) rank[ids[t]] = 1;
}

// exclusive scan of one tile of NA_TILE words in place; its total to sums[tile]
__global__ void k_na_scan_tile(int *v, int count, int *sums) {
    __shared__ int warpSums[TPB / 32];
    const int base = blockIdx.x * NA_TILE + threadIdx.x * 4;
    int x[4], own = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        x[q] = base + q < count ? v[base + q] : 0;
        own += x[q];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = own;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warpSums[warp] = inc;
    __syncthreads();
    int before = 0, total = 0;
    for (int q = 0; q < TPB / 32; q++) {
        if (q < warp) before += warpSums[q];
        total += warpSums[q];
    }
    int run = before + inc - own;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if (base + q < count) v[base + q] = run;
        run += x[q];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// exclusive scan of the tile sums in place (one block)
__global__ void k_na_scan_sums(int *sums, int ntiles) {
    __shared__ int sh[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b = 0; b < ntiles; b += 1024) {
        const int t = b + threadIdx.x;
        sh[threadIdx.x] = t < ntiles ? sums[t] : 0;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            int y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += y;
            __syncthreads();
        }
        const int inc = sh[threadIdx.x];
        const int own = t < ntiles ? sums[t] : 0;
        if (t < ntiles) sums[t] = carry + inc - own;
        __syncthreads();
        if (threadIdx.x == 1023) carry += inc;
        __syncthreads();
    }
}

__global__ void k_na_scan_add(int *v, int count, const int *sums) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) v[t] += sums[t / NA_TILE];
}

__global__ void k_na_scatter(const float *px, const float *py, const float *pz, const unsigned int *ids, int n,
                             int idSpace, const int *rank, float *out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n || ids[t] >= (unsigned int)idSpace) return;
    const long long o = 3LL * rank[ids[t]];
    out[o] = px[t];
    out[o + 1] = py[t];
    out[o + 2] = pz[t];
}

// Device address of the scratch array in the current context.  The address
// belongs to the context that loaded this module, not to the device
// ordinal: a host that makes its own driver contexts, or calls
// cudaDeviceReset, gets a new one.  So it is looked up on every call; once
// the module is loaded in the context the lookup allocates nothing.  Under
// lazy module loading the array's 4 MiB are reserved at the first call in a
// context, not when the library loads.
int scratch_for_current_context(int **out) {
    int *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
        return flip::record_error(FLIP_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *out = ptr;
    return FLIP_OK;
}

}  // namespace

extern "C" int flip_order_particles_by_id_noalloc(const float *d_px, const float *d_py, const float *d_pz,
                                                  const unsigned int *d_ids, int n, int id_space,
                                                  float *d_out_xyz, void *stream) {
    if (n < 0 || id_space < 0) return flip::record_error(FLIP_E_DOMAIN, "negative particle count or id space");
    if (id_space > FLIP_NOALLOC_MAX_IDS)
        return flip::record_error(FLIP_E_OUT_OF_RANGE, "id_space " + std::to_string(id_space) +
                                                           " exceeds the no-allocation limit of " +
                                                           std::to_string(FLIP_NOALLOC_MAX_IDS) + " ids");
    if (n > id_space) return flip::record_error(FLIP_E_DOMAIN, "more particles than distinct ids below id_space");
    if (n == 0) return FLIP_OK;
    if (!d_px || !d_py || !d_pz || !d_ids || !d_out_xyz) return flip::record_error(FLIP_E_NULL, "null device pointer");
    int *rank = nullptr;
    int rc = scratch_for_current_context(&rank);
    if (rc) return rc;
    int *sums = rank + FLIP_NOALLOC_MAX_IDS + 1;
    cudaStream_t s = (cudaStream_t)stream;
    const int count = id_space + 1;   // ranks of every id, then the total
    const int ntiles = (count + NA_TILE - 1) / NA_TILE;
    { FLIP_COUNT(1); k_na_clear<<<flip::div_up(count, TPB), TPB, 0, s>>>(rank, count); }
    { FLIP_COUNT(1); k_na_flag<<<flip::div_up(n, TPB), TPB, 0, s>>>(d_ids, n, id_space, rank); }
    { FLIP_COUNT(1); k_na_scan_tile<<<ntiles, TPB, 0, s>>>(rank, count, sums); }
    { FLIP_COUNT(1); k_na_scan_sums<<<1, 1024, 0, s>>>(sums, ntiles); }
    { FLIP_COUNT(1); k_na_scan_add<<<flip::div_up(count, TPB), TPB, 0, s>>>(rank, count, sums); }
    { FLIP_COUNT(1); k_na_scatter<<<flip::div_up(n, TPB), TPB, 0, s>>>(d_px, d_py, d_pz, d_ids, n, id_space, rank, d_out_xyz); }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return flip::record_error(FLIP_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return FLIP_OK;
}
