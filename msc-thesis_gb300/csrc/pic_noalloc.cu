// pic_noalloc.cu -- a charge deposit that allocates no device memory.
//
// pic_deposit_grid accumulates into an int64 scratch grid that it allocates
// with cudaMalloc and frees with cudaFree on every call.  Some callers cannot
// do that: a host framework that owns all of the GPU's memory through its
// own pool allocator (an extra cudaMalloc can fail there even though the
// pool has room), a process that runs under a fixed device-memory budget
// decided at start-up, or a service loop that must not stall other streams
// (cudaFree synchronises the whole device).  pic_deposit_grid_noalloc gives
// them the same result from a scratch grid that lives in this library's
// static device memory instead: every GPU that loads the library holds
// PIC_NOALLOC_MAX_CELLS int64 words (8 MiB) until the process exits.
//
// The scratch array is shared by every call in the process: each call clears
// the part it uses before depositing, and calls whose work overlaps on the GPU
// (different streams, or different host threads) race on it and give wrong
// results.  Every call looks up the array's device address on the current
// device (cudaGetSymbolAddress) instead of keeping it: a cudaDeviceReset or a
// re-created primary context reloads the module at another address, and a
// kept pointer would then be stale.  The first call on a device also loads
// the module there; make it before any stream capture on that device.
//
// The call is asynchronous: it only enqueues work on the caller's stream.
// Synchronise that stream before reading rho_dev or reusing the particle
// arrays.  Entries with cell < 0 (empty slots) and cells off the grid are
// skipped without a report: a stateless call that returns before its kernel
// runs has no error word to set (the handle's kernels report off-grid cells
// as PIC_DEVERR_CELL).
#include <cuda_runtime.h>

#include <string>

#include "pic_internal.cuh"

// the scratch grid: one int64 accumulator per cell, in 2^-32 charge units
static __device__ __align__(256) unsigned long long g_noalloc_scratch[PIC_NOALLOC_MAX_CELLS];

namespace {

__global__ void noalloc_zero_kernel(unsigned long long *acc, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        acc[i] = 0ull;
}

// fixed-point CIC of one particle per thread, as pic_deposit_grid computes it
__global__ void noalloc_deposit_kernel(const int32_t *__restrict__ cell,
                                       const float *__restrict__ ox,
                                       const float *__restrict__ oy, long long n, int nx, int ny,
                                       unsigned long long *acc)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int c = cell[i];
        if (c < 0) continue;
        const int cx = c & 0xFFFF, cy = c >> 16;
        if (cx >= nx || cy >= ny) continue;
        const unsigned long long fx = __float2uint_rn(ox[i] * 65536.0f);
        const unsigned long long fy = __float2uint_rn(oy[i] * 65536.0f);
        const unsigned long long gx = 65536ull - fx, gy = 65536ull - fy;
        const int cx1 = (cx + 1 == nx) ? 0 : cx + 1;
        const int cy1 = (cy + 1 == ny) ? 0 : cy + 1;
        atomicAdd(acc + (size_t)cy * nx + cx, gx * gy);
        atomicAdd(acc + (size_t)cy * nx + cx1, fx * gy);
        atomicAdd(acc + (size_t)cy1 * nx + cx, gx * fy);
        atomicAdd(acc + (size_t)cy1 * nx + cx1, fx * fy);
    }
}

__global__ void noalloc_to_double_kernel(const unsigned long long *__restrict__ acc, long long n,
                                         double scale, double *__restrict__ dst)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        dst[i] = (double)(long long)acc[i] * scale;
}

// Device address of the scratch array on the current device.  In host code
// g_noalloc_scratch names a host-side stand-in, never the device array.
pic_status scratch_for_current_device(unsigned long long **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return pic::cuda_fail(e, "pic_deposit_grid_noalloc: cudaGetSymbolAddress");
    *out = (unsigned long long *)p;
    return PIC_OK;
}

}  // namespace

extern "C" pic_status pic_deposit_grid_noalloc(int nx, int ny, long long n,
                                               const int32_t *cell_dev, const float *ox_dev,
                                               const float *oy_dev, int q_int, double scale,
                                               double *rho_dev, void *stream)
{
    if (nx < 1 || ny < 1 || nx > 32768 || ny > 32768 || n < 0 || !rho_dev ||
        (n > 0 && (!cell_dev || !ox_dev || !oy_dev))) {
        pic::set_error("pic_deposit_grid_noalloc: bad grid size, count or pointer");
        return PIC_ERR_INVALID_ARG;
    }
    const long long ng = (long long)nx * ny;
    if (ng > PIC_NOALLOC_MAX_CELLS) {
        pic::set_error("pic_deposit_grid_noalloc: nx*ny = " + std::to_string(ng) +
                       " exceeds the fixed scratch grid of " +
                       std::to_string(PIC_NOALLOC_MAX_CELLS) + " cells");
        return PIC_ERR_INVALID_ARG;
    }
    unsigned long long *acc = nullptr;
    PIC_TRY(scratch_for_current_device(&acc));
    cudaStream_t st = (cudaStream_t)stream;
    const int block = 256;
    const int gz = (int)((ng + block - 1) / block);
    noalloc_zero_kernel<<<gz, block, 0, st>>>(acc, ng);
    PIC_CUDA(cudaGetLastError());
    if (n > 0) {
        noalloc_deposit_kernel<<<pic::grid_for(n, block), block, 0, st>>>(cell_dev, ox_dev, oy_dev,
                                                                        n, nx, ny, acc);
        PIC_CUDA(cudaGetLastError());
    }
    noalloc_to_double_kernel<<<gz, block, 0, st>>>(acc, ng, (double)q_int * scale / 4294967296.0,
                                                   rho_dev);
    PIC_CUDA(cudaGetLastError());
    return PIC_OK;
}
