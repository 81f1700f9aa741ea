// CFL time step from caller-owned device arrays, without allocating.
//
// Some callers cannot call cudaMalloc: frameworks that own all device memory
// through their own pool allocator and forbid allocations behind their back,
// and latency-critical loops where a cudaMalloc/cudaFree would synchronise
// the device. For them f2d_cfl_dt_noalloc computes Model.set_dt's CFL step
// with its reduction scratch (per-block partial maxima and a ticket counter)
// in a fixed array that is part of the library image, so a call allocates
// nothing. A NaN in U.x or U.y gives NaN maxima and a NaN time step, as
// numpy's max and Python's min give in the reference's set_dt.
//
// The scratch array holds 8192 blocks' partials (128 KiB + 256 B) and stays
// resident on every GPU that loads the library until the process exits. It
// bounds the array size: rows * pitch <= 33,554,432 points (8192 blocks of
// 256 threads, 16 points per thread), enough for a 4096 x 4096 grid with its
// halo. All calls on a device share the one array: calls that may overlap on
// the GPU (different streams, or other threads) race on it and give wrong
// results; serialise them on one stream. The ticket counter is cleared at the
// start of each call; the partials are fully rewritten by every call.
// The device address of the array is looked up on the first call on each
// device and kept for the life of the process: a cudaDeviceReset after that
// first call is not supported (the kept address would belong to the
// destroyed context).
#include <mutex>
#include <string>

#include "../../include/fluids2d_gb300.h"
#include "common.cuh"

int f2d_internal_fail(int code, const char* msg);

namespace f2d {
namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_POINTS_PER_THREAD = 16;
constexpr int NA_MAX_BLOCKS = 8192;
constexpr long long NA_MAX_POINTS =
    (long long)NA_MAX_BLOCKS * NA_THREADS * NA_POINTS_PER_THREAD;

struct NoAllocScratch {
    double partials[2 * NA_MAX_BLOCKS];  // per-block max|U.x|, max|U.y|
    unsigned int ticket;                 // last-block ticket, must start at 0
    unsigned int pad[63];
};

static __device__ __align__(256) NoAllocScratch g_cfl_scratch;

// device address of g_cfl_scratch per device, looked up once per device
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_mu;
NoAllocScratch* g_addr[NA_MAX_DEVICES] = {};

// max |U.x|, max |U.y| over rows x cols of pitched arrays, then the CFL step
// of model.py:71-87: dt = min(cfl / (max|U.x| + max|U.y| + 1e-99), dtmax).
__global__ void __launch_bounds__(NA_THREADS)
k_cfl_dt_noalloc(const double* __restrict__ Ux, const double* __restrict__ Uy,
                 long long rows, long long cols, long long pitch, double cfl,
                 double dtmax, double* __restrict__ out, NoAllocScratch* scr)
{
    double m[2] = {0.0, 0.0};
    const long long n = rows * pitch;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += stride) {
        const long long j = k / pitch;
        if (k - j * pitch < cols) {
            m[0] = nanmax(m[0], fabs(Ux[k]));
            m[1] = nanmax(m[1], fabs(Uy[k]));
        }
    }
    if (grid_reduce<2, true>(m, scr->partials, &scr->ticket)) {
        out[0] = m[0];
        out[1] = m[1];
        out[2] = pymin(cfl / (m[0] + m[1] + 1e-99), dtmax);
    }
}

}  // namespace
}  // namespace f2d

extern "C" int f2d_cfl_dt_noalloc(const double* Ux, const double* Uy, int64_t rows,
                                  int64_t cols, int64_t pitch, double cfl, double dtmax,
                                  double* out, void* stream)
{
    using namespace f2d;
    if (!Ux || !Uy || !out) return f2d_internal_fail(1, "null pointer argument");
    if (rows < 1 || cols < 1 || pitch < cols)
        return f2d_internal_fail(1, "bad sizes: need rows >= 1, cols >= 1, pitch >= cols");
    if (rows > NA_MAX_POINTS / pitch)
        return f2d_internal_fail(
            1, ("array too large for the fixed scratch of f2d_cfl_dt_noalloc: rows * pitch = " +
                std::to_string((long long)rows * pitch) + " > " +
                std::to_string(NA_MAX_POINTS) + " points")
                   .c_str());
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return f2d_internal_fail((int)e, cudaGetErrorString(e));
    if (dev < 0 || dev >= NA_MAX_DEVICES)
        return f2d_internal_fail(1, "device ordinal beyond the supported 64");
    NoAllocScratch* scr = nullptr;
    {
        // set-up, once per device, with that device current
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_cfl_scratch);
            if (e != cudaSuccess)
                return f2d_internal_fail(
                    (int)e, (std::string("cudaGetSymbolAddress(scratch): ") +
                             cudaGetErrorString(e)).c_str());
            g_addr[dev] = (NoAllocScratch*)p;
        }
        scr = g_addr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    // the ticket must start at zero (a call that was cut short leaves it set)
    e = cudaMemsetAsync(&scr->ticket, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return f2d_internal_fail((int)e, cudaGetErrorString(e));
    const long long n = (long long)rows * pitch;
    const long long per_block = (long long)NA_THREADS * NA_POINTS_PER_THREAD;
    const int blocks = (int)((n + per_block - 1) / per_block);
    k_cfl_dt_noalloc<<<blocks, NA_THREADS, 0, s>>>(Ux, Uy, rows, cols, pitch, cfl, dtmax,
                                                     out, scr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return f2d_internal_fail((int)e, cudaGetErrorString(e));
    return 0;
}
