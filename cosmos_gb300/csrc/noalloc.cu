// Allocation-free conservation sums.
//
// Some callers cannot allocate device memory at the point where they need the sums: a foreign
// runtime or framework that owns the device allocator and its memory pool (a cudaMalloc beside
// it fragments or overdraws the pool it manages), an embedded caller with a fixed memory budget
// set at start-up, and a pipeline that must not stall (cudaMalloc and cudaFree can synchronise
// the device).  cosmos_field_sums_noalloc serves them: it takes the caller's device state and
// output pointers and keeps its reduction scratch in a file-scope device array instead of
// calling cudaMalloc.
//
// Limits and sharing: the scratch holds one row of partial sums per grid row, so grids taller
// than COSMOS_NOALLOC_MAX_ROWS rows are rejected.  The array lives as long as the library is
// loaded, on every device that loads it (640 KB each).  All calls share it, so calls whose
// kernels overlap on the GPU (concurrent streams, several host threads) race and must be
// serialised by the caller.  The scratch's device address is looked up on the first call on each
// device and kept; a cudaDeviceReset invalidates it, so do not call this entry point again in a
// process after resetting the device.
#include <mutex>
#include <string>

#include "../../include/cosmos_gb300.h"
#include "launch.h"

namespace cg {

void set_error(const char* msg);  // capi.cu: sets the text returned by cosmos_last_error()

static __device__ __align__(256) double g_noalloc_rows[COSMOS_NOALLOC_MAX_ROWS * 5];
static __device__ __align__(256) unsigned int g_noalloc_done;

namespace {

// One block per grid row: compensated (Neumaier) sums of the row's five fields into the
// scratch row; the last block to finish adds the rows in row order, so the result does not
// depend on block scheduling.
__global__ void noalloc_sums_kernel(const void* __restrict__ state, int precision, int nx, int ny, int pitch,
                                    size_t fstride, double* rows, unsigned int* done, double* out5) {
    const int r = blockIdx.x;
    __shared__ double part[5][256];
    double s[5] = {0, 0, 0, 0, 0}, c[5] = {0, 0, 0, 0, 0};
    for (int j = threadIdx.x; j < nx; j += blockDim.x) {
        const size_t k = (size_t)r * pitch + j;
#pragma unroll
        for (int f = 0; f < 5; f++) {
            const double v = precision == COSMOS_FP32 ? (double)((const float*)state)[f * fstride + k]
                                                      : ((const double*)state)[f * fstride + k];
            const double t = s[f] + v;
            c[f] += (fabs(s[f]) >= fabs(v)) ? ((s[f] - t) + v) : ((v - t) + s[f]);
            s[f] = t;
        }
    }
#pragma unroll
    for (int f = 0; f < 5; f++) part[f][threadIdx.x] = s[f] + c[f];
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int f = 0; f < 5; f++) {
        double a = 0.0, ca = 0.0;
        for (unsigned q = 0; q < blockDim.x; q++) {
            const double v = part[f][q], t = a + v;
            ca += (fabs(a) >= fabs(v)) ? ((a - t) + v) : ((v - t) + a);
            a = t;
        }
        rows[(size_t)r * 5 + f] = a + ca;
    }
    __threadfence();
    if (atomicAdd(done, 1u) != (unsigned)ny - 1) return;
    __threadfence();
    for (int f = 0; f < 5; f++) {
        double a = 0.0, ca = 0.0;
        for (int q = 0; q < ny; q++) {
            const double v = ((volatile double*)rows)[(size_t)q * 5 + f], t = a + v;
            ca += (fabs(a) >= fabs(v)) ? ((a - t) + v) : ((v - t) + a);
            a = t;
        }
        out5[f] = a + ca;
    }
}

// Per-device addresses of the scratch symbols, looked up once per device.
struct ScratchAddr {
    double* rows = nullptr;
    unsigned int* done = nullptr;
};
std::mutex g_mu;
ScratchAddr g_addr[64];

}  // namespace
}  // namespace cg

using namespace cg;

extern "C" int cosmos_field_sums_noalloc(const void* state, int precision, int nx, int ny, int pitch,
                                         size_t field_stride, double* out5, void* stream) {
    if (!state || !out5) { set_error("cosmos_field_sums_noalloc: null state or output pointer"); return COSMOS_EINVAL; }
    if (precision != COSMOS_FP64 && precision != COSMOS_FP32) {
        set_error("cosmos_field_sums_noalloc: precision must be COSMOS_FP64 or COSMOS_FP32");
        return COSMOS_EINVAL;
    }
    if (nx < 1 || ny < 1 || pitch < nx || field_stride < (size_t)pitch * ny) {
        set_error("cosmos_field_sums_noalloc: need nx, ny >= 1, pitch >= nx and field_stride >= pitch * ny");
        return COSMOS_EINVAL;
    }
    if (ny > COSMOS_NOALLOC_MAX_ROWS) {
        set_error("cosmos_field_sums_noalloc: grid has more rows than the fixed scratch holds "
                  "(COSMOS_NOALLOC_MAX_ROWS = 16384); use cosmos_grid_field_sums for larger grids");
        return COSMOS_EINVAL;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        set_error("cosmos_field_sums_noalloc: no usable current device");
        return COSMOS_ECUDA;
    }
    ScratchAddr a;
    {
        // set-up on this device's first call: host code must ask the runtime for the device
        // address of the scratch array (its host-side name is not a device address)
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_addr[dev].rows) {
            void* p = nullptr;
            void* q = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_rows) != cudaSuccess ||
                cudaGetSymbolAddress(&q, g_noalloc_done) != cudaSuccess) {
                set_error("cosmos_field_sums_noalloc: cudaGetSymbolAddress failed for the scratch array");
                return COSMOS_ECUDA;
            }
            g_addr[dev].rows = (double*)p;
            g_addr[dev].done = (unsigned int*)q;
        }
        a = g_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    // an error left pending by earlier, unrelated work is reported as such, not as this call's
    const cudaError_t pending = cudaGetLastError();
    if (pending != cudaSuccess) {
        set_error((std::string("cosmos_field_sums_noalloc: a CUDA error was already pending before the call: ") +
                   cudaGetErrorString(pending)).c_str());
        return COSMOS_ECUDA;
    }
    // the completion counter must start at zero on every call
    if (cudaMemsetAsync(a.done, 0, sizeof(unsigned int), st) != cudaSuccess) {
        set_error("cosmos_field_sums_noalloc: clearing the completion counter failed");
        return COSMOS_ECUDA;
    }
    noalloc_sums_kernel<<<ny, 256, 0, st>>>(state, precision, nx, ny, pitch, field_stride, a.rows, a.done, out5);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(cudaGetErrorString(e));
        return COSMOS_ECUDA;
    }
    return COSMOS_OK;
}
