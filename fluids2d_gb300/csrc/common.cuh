// Shared definitions of the fluids2d_gb300 CUDA library: array geometry,
// per-point mask/order codes, device scalars, TMA/mbarrier helpers and
// deterministic grid reductions.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace f2d {

// ---------------------------------------------------------------------------
// Array geometry. Every field is a (NY, NX) = (ny+6, nx+6) array as in the
// reference (meshes.py:122-132), stored on the device with a row pitch P >= NX
// (a multiple of 16 elements, so rows start on 128-byte boundaries and TMA
// strides are legal).
// ---------------------------------------------------------------------------
struct Geom {
    int NY, NX;      // rows, columns including the 3-cell halo
    int ny, nx;      // interior size
    long long P;     // device row pitch in elements
    int xper;        // x-periodic: halo columns hold copies (meshes.py:135-143)
};

// Per-point code word packing the int8 masks and stencil orders of the
// reference mesh (meshes.py:77-104): six 2-bit order levels and six flags.
enum : uint32_t {
    SH_OCX = 0, SH_OCY = 2, SH_OVX = 4, SH_OVY = 6, SH_OKX = 8, SH_OKY = 10,
    B_MSK = 1u << 12, B_MSKX = 1u << 13, B_MSKY = 1u << 14,
    B_MSKV = 1u << 15, B_SLIP = 1u << 16, B_GV = 1u << 17,
};
__host__ __device__ inline int lev(uint32_t c, int sh) { return (c >> sh) & 3; }

// Status bits reported back to the host (f2d_last_error).
enum : int {
    ST_TMA_TIMEOUT = 1,    // a TMA tile load did not complete within 1 s
    ST_PCG_MAXIT = 2,      // the Poisson solve stopped at max iterations
    ST_NONFINITE = 4,      // a non-finite value reached a reduction
    ST_STAGE_ALIGN = 8,    // a TMA staging buffer was not 128-byte aligned (nothing loaded)
};

// min(x, cap) with Python's min semantics (the reference's set_dt,
// model.py:87: min(cfl/maxU, dtmax)): x unless cap < x, so a NaN x stays NaN
__host__ __device__ __forceinline__ double pymin(double x, double cap)
{
    return cap < x ? cap : x;
}

// Device-resident scalars of one model: the time line (timeline.py:4-35),
// the CFL reduction and the Poisson-solver state.
struct DevScalars {
    double t, c, dt;        // time, Kahan compensation, time step
    long long ite;
    double maxUx, maxUy;    // max |U.x|, max |U.y| of the last diagnostic
    double cfl, dtmax;      // set_dt parameters (model.py:71-87)
    int status;
    int pad0;
    // Poisson solver (one at a time per model)
    double bb, rr, rz, pq, alpha, beta;
    double tol2;            // (relative tolerance)^2
    int iter, maxit, converged, pad1;
    long long total_iters;  // summed over solves, for diagnostics
    unsigned int counter[8];  // last-block reduction tickets
    // iterative refinement: FP32 inner CG for the correction of the FP64 x
    double rr0, tol_in2;      // inner start residual^2, (inner tolerance)^2
    int iter_in, maxit_in;    // inner iterations of the current round
    int outer, maxouter;      // refinement rounds of the current solve
    int conv_in, zero;        // inner loop done; right-hand side is zero
    long long total_outer;    // refinement rounds summed over solves
    // Robert-Asselin filter coefficient of the leap-frog integrator
    // (param.py:50 RAgamma, integrators.py:39-55)
    double ragamma;
    // time step of the step whose stage increments the warm start keeps
    // (0: none yet); the next step scales them by dt / dt_warm
    double dt_warm;
    // step lengths (FP32) of the inner iterations of the current refinement
    // round: the round's correction is sum alpha_i p_i (solver.cu)
    float ahist[32];
};

// ---------------------------------------------------------------------------
// Small PTX helpers: TMA tile loads through an mbarrier, with a time-bounded
// wait so that a copy that never lands turns into a status bit, not a hang.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(count)
                 : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                     smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map,
                                            int x, int y, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may be scheduled while its predecessor drains; it waits here
// (for the predecessor's completion and memory) before touching anything the
// predecessor writes. Without such a launch this returns at once.
__device__ __forceinline__ void pdl_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for phase `parity` of the barrier; gives up after `limit_ns`.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          uint64_t limit_ns = 1000000000ull)
{
    const uint32_t a = smem_u32(bar);
    uint64_t t0 = 0;
    for (int spin = 0;; ++spin) {
        uint32_t ok;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;"
            " selp.u32 %0, 1, 0, p; }"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if (spin == 0) t0 = globaltimer_ns();
        else if (globaltimer_ns() - t0 > limit_ns) return false;
    }
}

// ---------------------------------------------------------------------------
// binary64 <-> binary32 conversions on the integer pipe. GB300 runs FP64
// instructions, the hardware conversions between FP64 and FP32 among them, at
// 1/64 of the FP32 rate, and in the FP32 form's FP64 kernels (refinement
// residual, perpgrad, correction, centers-to-vertices) the conversions are a
// large share of that pipe. These follow the IEEE 754 definitions of the two
// formats (sign, biased exponent, significand; conversion to binary32 rounds
// to nearest, ties to even, with gradual underflow, overflow to infinity and
// NaN kept quiet) and give the same bits as the hardware conversions
// (tests/test_conversions.py checks every class of input on the GPU).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float f64_to_f32_rn(double x)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const unsigned m20 = hi & 0xfffffu;  // significand bits 51..32
    if (e == 0x7ff) {  // infinity, or NaN (quiet, top payload bits kept)
        const bool nan = (m20 | lo) != 0u;
        const unsigned pay = (m20 << 3) | (lo >> 29);
        return __uint_as_float(sign | 0x7f800000u | (nan ? (0x400000u | pay) : 0u));
    }
    const int ef = e - 1023 + 127;
    if (ef >= 255) return __uint_as_float(sign | 0x7f800000u);
    if (ef >= 1) {
        // 23 result bits and the 29 bits below them
        const unsigned mf = (m20 << 3) | (lo >> 29);
        const unsigned rem = lo & 0x1fffffffu;
        unsigned bits = sign | ((unsigned)ef << 23) | mf;
        if (rem > 0x10000000u || (rem == 0x10000000u && (mf & 1u))) bits += 1u;  // may carry to inf
        return __uint_as_float(bits);
    }
    // binary32 subnormal (or zero): the significand with its leading 1,
    // shifted right by 1 - ef more places, rounded to nearest even
    if (ef < -24 || e == 0) return __uint_as_float(sign);  // below half the smallest subnormal
    const unsigned long long sig = (1ull << 52) | ((unsigned long long)m20 << 32) | lo;
    const int sh = 29 + 1 - ef;  // 30 .. 54
    const unsigned long long q = sig >> sh;
    const unsigned long long r = sig & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    unsigned bits = sign | (unsigned)q;
    if (r > half || (r == half && (q & 1ull))) bits += 1u;  // may round up to the smallest normal
    return __uint_as_float(bits);
}

__device__ __forceinline__ double f32_to_f64(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned sign = b & 0x80000000u;
    const unsigned e = (b >> 23) & 0xffu;
    unsigned m = b & 0x7fffffu;
    unsigned hi, lo;
    if (e == 0xffu) {  // infinity or NaN (payload kept, quiet bit set for NaN)
        hi = sign | 0x7ff00000u | (m ? (0x80000u | (m >> 3)) : 0u);
        lo = m << 29;
    } else if (e != 0u) {
        hi = sign | ((e + 896u) << 20) | (m >> 3);
        lo = m << 29;
    } else if (m == 0u) {
        hi = sign;
        lo = 0u;
    } else {  // subnormal m 2^-149: normalise to 1.f 2^(p-149), p its leading bit
        const int p = 31 - __clz(m);
        m = (m << (23 - p)) & 0x7fffffu;
        hi = sign | ((unsigned)(p + 874) << 20) | (m >> 3);
        lo = m << 29;
    }
    return __hiloint2double((int)hi, (int)lo);
}

// conversions between the working precisions through the functions above
template <typename To, typename From>
__device__ __forceinline__ To conv(From x)
{
    if constexpr (std::is_same<To, float>::value && std::is_same<From, double>::value)
        return f64_to_f32_rn(x);
    else if constexpr (std::is_same<To, double>::value && std::is_same<From, float>::value)
        return f32_to_f64(x);
    else
        return To(x);
}

// Maximum that propagates NaN, as numpy's max does (the reference's set_dt,
// model.py:83-87, turns a NaN velocity into a NaN time step).
__host__ __device__ __forceinline__ double nanmax(double a, double b)
{
    return (a > b || a != a) ? a : b;
}
__host__ __device__ __forceinline__ float nanmaxf(float a, float b)
{
    return (a > b || a != a) ? a : b;
}
// the same for float operands: without it float maxima were promoted to
// double, two conversions and an FP64 compare per call on GB300's 1/64-rate
// FP64 pipe
__host__ __device__ __forceinline__ float nanmax(float a, float b)
{
    return nanmaxf(a, b);
}

// ---------------------------------------------------------------------------
// Deterministic grid-wide reductions of up to N doubles: every block writes
// its partial sums, the last block to finish (ticket counter) adds the
// partials in a fixed order, so results do not depend on block scheduling.
// ---------------------------------------------------------------------------
template <int N>
__device__ __forceinline__ void warp_sum(double (&v)[N])
{
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

template <int N>
__device__ __forceinline__ void warp_max(double (&v)[N])
{
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v[k] = nanmax(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
}

// Block-wide reduction; result valid in thread 0. `sh` needs 32*N doubles.
template <int N, bool MAX>
__device__ __forceinline__ void block_reduce(double (&v)[N], double* sh)
{
    const int nt = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    if (MAX) warp_max<N>(v); else warp_sum<N>(v);
    const int w = tid >> 5, lane = tid & 31, nw = (nt + 31) >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; ++k) sh[w * N + k] = v[k];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k)
            v[k] = lane < nw ? sh[lane * N + k] : (MAX ? -INFINITY : 0.0);
        if (MAX) warp_max<N>(v); else warp_sum<N>(v);
    }
}

// Per-thread part of the final sum over partials[t0 .. t0+n) (N values
// each): thread `tid` of `nth` adds entries tid, tid+nth, ... with four
// independent accumulators (loads in flight), combined in a fixed order.
template <int N, bool MAX>
__device__ __forceinline__ void final_sum(double (&acc)[N], const double* partials, int t0,
                                          int n, int tid, int nth)
{
    double a[4][N];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int k = 0; k < N; ++k) a[u][k] = MAX ? -INFINITY : 0.0;
    int i = tid;
    for (; i + 3 * nth < n; i += 4 * nth)
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int k = 0; k < N; ++k) {
                const double p = __ldcg(&partials[(size_t)(t0 + i + u * nth) * N + k]);
                a[u][k] = MAX ? nanmax(a[u][k], p) : a[u][k] + p;
            }
    for (int u = 0; i < n; i += nth, ++u)
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const double p = __ldcg(&partials[(size_t)(t0 + i) * N + k]);
            a[u & 3][k] = MAX ? nanmax(a[u & 3][k], p) : a[u & 3][k] + p;
        }
#pragma unroll
    for (int k = 0; k < N; ++k)
        acc[k] = MAX ? nanmax(nanmax(a[0][k], a[1][k]), nanmax(a[2][k], a[3][k]))
                     : (a[0][k] + a[1][k]) + (a[2][k] + a[3][k]);
}

// Grid reduction of N values. Returns true in the single thread (thread 0
// of the last block) that holds the grid result in `v`.
template <int N, bool MAX, bool PRE = false>
__device__ __forceinline__ bool grid_reduce(double (&v)[N], double* partials,
                                            unsigned int* ticket)
{
    __shared__ double sh[32 * N];
    __shared__ int s_last;
    if (!PRE) block_reduce<N, MAX>(v, sh);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const unsigned nb = gridDim.x * gridDim.y;
    const unsigned b = blockIdx.y * gridDim.x + blockIdx.x;
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) partials[(size_t)b * N + k] = v[k];
        __threadfence();
        unsigned prev = atomicAdd(ticket, 1u);
        s_last = (prev == nb - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    const int nt = blockDim.x * blockDim.y;
    double acc[N];
    final_sum<N, MAX>(acc, partials, 0, (int)nb, tid, nt);
    block_reduce<N, MAX>(acc, sh);
    if (tid == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) v[k] = acc[k];
        *ticket = 0;  // ready for the next launch
        return true;
    }
    return false;
}

// Block total of per-thread FP32 values: warp sums in FP32 (shuffles), the
// warp sums combined in FP64 by thread 0 in a fixed order. Result in thread 0.
template <int N, bool MAX = false>
__device__ __forceinline__ void block_total_f(const float (&a)[N], double (&out)[N])
{
    __shared__ float shf[32 * N];
    float v[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        v[k] = a[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float u = __shfl_xor_sync(0xffffffffu, v[k], o);
            v[k] = MAX ? nanmaxf(v[k], u) : v[k] + u;
        }
    }
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int w = tid >> 5, lane = tid & 31, nw = (blockDim.x * blockDim.y + 31) >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; ++k) shf[w * N + k] = v[k];
    __syncthreads();
    if (tid == 0)
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double t = MAX ? -INFINITY : 0.0;
            for (int i = 0; i < nw; ++i)
                t = MAX ? nanmax(t, (double)shf[i * N + k]) : t + (double)shf[i * N + k];
            out[k] = t;
        }
}

}  // namespace f2d
