// Launchers of the discrete-adjoint kernels of the eulerpsi step (adjoint.cu).
#pragma once
#include <algorithm>

#include "common.cuh"

namespace f2d {

// snapshot (w, U.x, U.y) of a stage state into arena slot *slot (3 arrays of
// fsz elements per slot, the forward precision)
int launch_adj_snap(int prec, const void* w, const void* ux, const void* uy, void* arena,
                    long long fsz, const int* slot, cudaStream_t s);
int launch_adj_slot(int* slot, int delta, cudaStream_t s);
// the per-stage streamfunction cache: store (store != 0) cache[*slot] = psi
// or restore psi = cache[*slot]
int launch_adj_psi(double* psi, double* cache, long long fsz, const int* slot, int store,
                   cudaStream_t s);
// adjoint RK3 combinations (mode 0: set d3,d2,d1; 1: d1,d2 +=; 2: d1 +=)
int launch_adj_comb(const Geom& g, const double* yb, double* d1, double* d2, double* d3,
                    int mode, double c1, double c2, double c3, cudaStream_t s);
// first half of a tendency VJP at snapshot slot *slot + soff: face gradients
// (6 planes each for x and y), face-velocity adjoints and the right-hand
// side psib of the adjoint Poisson solve
int launch_adj_vjp_pre(int method, int prec, const Geom& g, const uint32_t* code,
                       const void* arena, long long fsz, const int* slot, int soff,
                       const double* db, double* gx, double* gy, double* ubx, double* uby,
                       double rdx2, double rdy2, double* psib, cudaStream_t s);
// second half: yb += window gathers + c2v^T(rb), rb = the adjoint solve's solution
int launch_adj_vjp_post(const Geom& g, const uint32_t* code, const double* gx, const double* gy,
                        long long fsz, const double* rb, double* yb, cudaStream_t s);

}  // namespace f2d
