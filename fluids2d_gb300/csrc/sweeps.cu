// Flat-index sweep kernels: the CUDA counterparts of the reference's numba
// kernels CompFlux / VortexForce / InnerProduct (weno.py:346-446), with the
// same signature semantics: 1-D views of the (NY, NX) arrays, stride s (1 for
// x, NX for y), int8 stencil orders o, index range [i0, i1).
//
// These are the drop-in for the reference's kernel plug point; the model
// itself runs the fused stage kernels of stage.cu.
#include "common.cuh"
#include "weno.cuh"

namespace f2d {

template <typename T, int M>
__global__ void k_compflux(T* __restrict__ flx, const T* __restrict__ U,
                           const T* __restrict__ q, const int8_t* __restrict__ o,
                           long long s, long long i0, long long i1)
{
    const long long i = i0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i1) return;
    const int L = order_level(o[i]);
    T f = T(0);
    if (L == 3) {
        const T u = U[i];
        f = flux6<M, T>(u, q[i - 3 * s], q[i - 2 * s], q[i - s], q[i], q[i + s],
                        q[i + 2 * s]) * u;
    } else if (L == 2) {
        const T u = U[i];
        f = flux4<M, T>(u, q[i - 2 * s], q[i - s], q[i], q[i + s]) * u;
    } else if (L == 1) {
        const T u = U[i];
        f = flux2<M, T>(u, q[i - s], q[i]) * u;
    }
    flx[i] = f;
}

template <typename T, int M>
__global__ void k_vortexforce(T* __restrict__ du, const T* __restrict__ V,
                              const T* __restrict__ q, const int8_t* __restrict__ o,
                              long long s, long long s2, int sign, long long i0,
                              long long i1)
{
    const long long i = i0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i1) return;
    const int L = order_level(o[i]);
    T r = T(0);
    if (L) {
        const T Vm = T(0.25) * (((V[i] + V[i + s]) + V[i - s2]) + V[i + s - s2]);
        T f;
        if (L == 3)
            f = flux6<M, T>(Vm, q[i - 2 * s], q[i - s], q[i], q[i + s], q[i + 2 * s],
                            q[i + 3 * s]);
        else if (L == 2)
            f = flux4<M, T>(Vm, q[i - s], q[i], q[i + s], q[i + 2 * s]);
        else
            f = flux2<M, T>(Vm, q[i], q[i + s]);
        r = T(sign) * f * Vm;
    }
    du[i] = r;
}

template <typename T, int M>
__global__ void k_innerproduct(T* __restrict__ ke, const T* __restrict__ U,
                               const T* __restrict__ q, const int8_t* __restrict__ o,
                               long long s, long long i0, long long i1)
{
    const long long i = i0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i1) return;
    const int L = order_level(o[i]);
    if (!L) return;
    const T Um = T(0.5) * (U[i] + U[i + s]);
    T f;
    if (L == 3)
        f = flux6<M, T>(Um, q[i - 2 * s], q[i - s], q[i], q[i + s], q[i + 2 * s],
                        q[i + 3 * s]);
    else if (L == 2)
        f = flux4<M, T>(Um, q[i - s], q[i], q[i + s], q[i + 2 * s]);
    else
        f = flux2<M, T>(Um, q[i], q[i + s]);
    ke[i] += f * Um;
}

#define F2D_METHOD_SWITCH(method, CALL)                  \
    switch (method) {                                    \
    case METHOD_WENO: CALL(METHOD_WENO); break;          \
    case METHOD_UPWIND: CALL(METHOD_UPWIND); break;      \
    case METHOD_CENTERED: CALL(METHOD_CENTERED); break;  \
    case METHOD_CWENO: CALL(METHOD_CWENO); break;        \
    default: return 1;                                   \
    }

static unsigned nblk(long long n) { return (unsigned)((n + 255) / 256); }

int launch_compflux(int method, double* flx, const double* U, const double* q,
                    const int8_t* o, long long s, long long i0, long long i1,
                    cudaStream_t st)
{
    if (i1 <= i0) return 0;
#define CALL(M) k_compflux<double, M><<<nblk(i1 - i0), 256, 0, st>>>(flx, U, q, o, s, i0, i1)
    F2D_METHOD_SWITCH(method, CALL)
#undef CALL
    return (int)cudaGetLastError();
}

int launch_vortexforce(int method, double* du, const double* V, const double* q,
                       const int8_t* o, long long s, long long s2, int sign,
                       long long i0, long long i1, cudaStream_t st)
{
    if (i1 <= i0) return 0;
#define CALL(M) \
    k_vortexforce<double, M><<<nblk(i1 - i0), 256, 0, st>>>(du, V, q, o, s, s2, sign, i0, i1)
    F2D_METHOD_SWITCH(method, CALL)
#undef CALL
    return (int)cudaGetLastError();
}

int launch_innerproduct(int method, double* ke, const double* U, const double* q,
                        const int8_t* o, long long s, long long i0, long long i1,
                        cudaStream_t st)
{
    if (i1 <= i0) return 0;
#define CALL(M) k_innerproduct<double, M><<<nblk(i1 - i0), 256, 0, st>>>(ke, U, q, o, s, i0, i1)
    F2D_METHOD_SWITCH(method, CALL)
#undef CALL
    return (int)cudaGetLastError();
}

}  // namespace f2d
