// Multigrid-preconditioned CG for the masked cell-centred Poisson operator
// with Neumann walls (the pressure projection of the euler model). See
// nsolver.cu.
#pragma once
#include <vector>

#include "common.cuh"

namespace f2d {

// One level: cells (J, I) of nyn x nxn at off + J*pitch + I; face couplings
// fx(J, I) between cells (J, I-1) and (J, I) (column 0: the periodic wrap
// face, else 0), fy(J, I) between (J-1, I) and (J, I) (row 0: 0).
struct NLevel {
    void* x;           // the level's precision (FP64; FP32 in the FP32 cycle)
    void* b;
    const void* fx;
    const void* fy;
    const uint8_t* m;
    int nyn, nxn;
    long long pitch, off;
    int per, pad;
};

struct NGlobals {
    unsigned int ticket[4];
    int status, pad;
    long long iters;
};

struct NSolver {
    std::vector<NLevel> lev;       // host copy
    NLevel* dlev = nullptr;
    NGlobals* eg = nullptr;
    DevScalars* sc = nullptr;     // iteration state (own)
    double* partials = nullptr;
    double *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;  // level-0 layout
    float *r32 = nullptr, *z32 = nullptr;  // the FP32 cycle's level 0
    NLevel prob;                  // the Krylov level: FP64 couplings, level-0 layout
    int prec = 0;                 // 0: FP64 cycle; 1: FP32 cycle
    double* lev_x0 = nullptr;     // the problem: x (the pressure) and b
    double* lev_b0 = nullptr;
    long long nfluid = 0;
    int ksweeps = 16;             // (R,B)^k (B,R)^k on the coarsest level
    int nu = 2;                   // sweeps per leg
    double tol = 1e-12;
    int maxit = 200;
    std::vector<void*> owned;
};

// Build from the level-0 fluid mask (host, (J, I) at hoff + J*pitch + I) for
// the cells of the model layout: x = the pressure field, b = the right-hand
// side (both FP64, level-0 layout). cx = dy/dx (E-W), cy = dx/dy (N-S).
int ns_build(NSolver& s, int nyn, int nxn, long long pitch, long long off, int per,
             const uint8_t* hmask, double* x, double* b, double cx, double cy, int prec);
void ns_free(NSolver& s);
// Record a solve on `st` (conditional WHILE body on st2 under capture, or
// host-driven loops otherwise): b is made zero-mean over the fluid cells (the
// compatibility projection of the singular problem), x (warm start) is
// iterated to |r| <= tol |b| and finally made zero-mean.
int ns_record(NSolver& s, cudaStream_t st, cudaStream_t st2, bool eager, int* launches);

}  // namespace f2d
