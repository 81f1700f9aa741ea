// Geometric multigrid-preconditioned conjugate gradients for the masked
// 5-point vertex operator of the reference (elliptic.py:114-195: Dirichlet
// at non-fluid vertices, optional Helmholtz diagonal, x-periodic wrap).
#pragma once
#include <vector>

#include "common.cuh"

namespace f2d {

// One grid level. Node (J, I), 0 <= J < nyn, 0 <= I < nxn, lives at
// base[off + J*pitch + I] of the level's arrays. Level 0 is the model's
// vertex array (node (J,I) = array point (3+J, 3+I)).
struct MGLevel {
    void* x;            // level unknown (level 0: the preconditioned residual z)
    void* xa;           // x after the pre-smoothing (read by the up leg)
    void* b;            // level right-hand side (level 0: the CG residual r)
    const uint8_t* m;   // 1 = fluid node
    int nyn, nxn;
    long long pitch, off;
    int per;            // x-periodic wrap over nxn nodes
    int pad;
    double cx, cy;      // east-west and north-south couplings (dy/dx, dx/dy)
    double diag, idiag; // -2(cx+cy) - maindiag and its inverse
    float fcx, fcy, fdiag, fidiag;  // the same in FP32 (no conversions in FP32 kernels)
    double md;          // maindiag of the level: diag = -2 (cx + cy) - md
    float fmd;
};

// bytes of one level's arrays (x, b: element size es; mask) in the
// single-block tail's shared memory, stored with a one-node border
__host__ __device__ inline size_t tail_level_bytes(int nyn, int nxn, size_t es)
{
    const size_t n = (size_t)(nyn + 2) * (nxn + 2);
    return 2 * ((n * es + 15) / 16 * 16) + (n + 15) / 16 * 16;
}

struct MGHost {
    std::vector<MGLevel> lev;
    std::vector<void*> owned;  // device allocations of coarse levels
    MGLevel* dlev = nullptr;   // device copy of lev
    int ltail = 0;             // first level handled by the single-block tail
    int ncoarse_sweeps = 4;    // (R,B)^k (B,R)^k on the coarsest level
    size_t tail_smem = 0;      // dynamic shared memory of the tail kernel
    int prec = 0;              // 0 = double, 1 = float
    std::vector<std::vector<uint8_t>> hmask;  // host fluid masks, dense nyn x nxn per level
};

int mg_build(MGHost& mg, int nyn0, int nxn0, long long pitch0, long long off0,
             int per, const uint8_t* hmask0 /* host, level-0 layout */, long long hoff0,
             const uint8_t* dmask0 /* device copy */, void* z0, void* za0, void* r0,
             double cx, double cy, double maindiag, int prec);
void mg_free(MGHost& mg);

}  // namespace f2d
