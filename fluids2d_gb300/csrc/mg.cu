// Multigrid hierarchy of the masked vertex Poisson/Helmholtz operator (the
// reference factorises it with SuperLU, elliptic.py:71-87; here it is solved
// matrix-free by solver.cu).
//
// Operator at a fluid node: A x = cx (xW + xE) + cy (xS + xN) + diag x, with
// non-fluid neighbours contributing 0 (Dirichlet), cx = dy/dx, cy = dx/dy and
// diag = -2 (cx + cy) - maindiag, exactly the matrix of
// get_Laplacian_sparse (elliptic.py:138-189). A is negative definite; the
// V-cycle approximates its inverse, so plain PCG applies without sign flips.
//
// Preconditioner: one V-cycle with red-black Gauss-Seidel, pre (red, black)
// and post (black, red); restriction = transpose of bilinear prolongation
// (full weighting with weights 1, 1/2, 1/4); coarse operators re-discretised
// with the same couplings and maindiag scaled by 4 per level; coarse masks
// injected from the fine mask. The cycle is symmetric, so PCG converges.
// Levels with at most ~1100 nodes run in one thread block (the "tail").
#include <algorithm>
#include <cstring>

#include "mg_ops.cuh"

namespace f2d {

// shared-memory bytes of the tail levels l0..nl-1
static size_t tail_smem(const std::vector<MGLevel>& lev, int l0, size_t es)
{
    size_t off = 0;
    for (size_t l = l0; l < lev.size(); ++l) off += tail_level_bytes(lev[l].nyn, lev[l].nxn, es);
    return off;
}

// Build the level hierarchy from the level-0 fluid mask (host copy).
int mg_build(MGHost& mg, int nyn0, int nxn0, long long pitch0, long long off0, int per,
             const uint8_t* hmask0, long long hoff0, const uint8_t* dmask0, void* z0, void* za0,
             void* r0, double cx,
             double cy, double maindiag, int prec)
{
    mg_free(mg);
    mg.prec = prec;
    const size_t es = prec == 0 ? sizeof(double) : sizeof(float);
    MGLevel L0;
    memset(&L0, 0, sizeof(L0));
    L0.x = z0;
    L0.xa = za0;
    L0.b = r0;
    L0.m = dmask0;
    L0.nyn = nyn0;
    L0.nxn = nxn0;
    L0.pitch = pitch0;
    L0.off = off0;
    L0.per = per;
    L0.cx = cx;
    L0.cy = cy;
    L0.diag = -2 * (cx + cy) - maindiag;
    L0.idiag = 1.0 / L0.diag;
    L0.fcx = (float)L0.cx;
    L0.fcy = (float)L0.cy;
    L0.fdiag = (float)L0.diag;
    L0.fidiag = (float)L0.idiag;
    L0.md = maindiag;
    L0.fmd = (float)maindiag;
    mg.lev.push_back(L0);

    // host masks of each level, dense nyn x nxn
    std::vector<uint8_t> cur((size_t)nyn0 * nxn0);
    for (int J = 0; J < nyn0; ++J)
        for (int I = 0; I < nxn0; ++I)
            cur[(size_t)J * nxn0 + I] = hmask0[hoff0 + (long long)J * pitch0 + I] ? 1 : 0;
    mg.hmask.push_back(cur);
    int nyn = nyn0, nxn = nxn0;
    double md = maindiag;
    const int max_levels = 16;
    while ((int)mg.lev.size() < max_levels) {
        // coarsen while the level is big enough; periodic needs an even count
        if (nyn < 6 || nxn < 6) break;
        if (per && (nxn % 2)) break;
        const int cyn = (nyn - 1 + 1) / 2 + 1;
        const int cxn = per ? nxn / 2 : (nxn - 1 + 1) / 2 + 1;
        std::vector<uint8_t> cm((size_t)cyn * cxn, 0);
        size_t nfluid = 0;
        for (int J = 0; J < cyn; ++J)
            for (int I = 0; I < cxn; ++I) {
                const int fj = 2 * J, fi = 2 * I;
                uint8_t v = 0;
                if (fj < nyn && fi < nxn) v = cur[(size_t)fj * nxn + fi];
                if (J == 0 || J == cyn - 1) v = 0;
                if (!per && (I == 0 || I == cxn - 1)) v = 0;
                cm[(size_t)J * cxn + I] = v;
                nfluid += v;
            }
        if (nfluid == 0) break;
        md *= 4.0;
        MGLevel C;
        memset(&C, 0, sizeof(C));
        C.nyn = cyn;
        C.nxn = cxn;
        // node (J, I) at element 1 + J*pitch + I: an odd offset, like level
        // 0's (node (J, I) of the model's array at (3+J)*P + 3+I, P even), so
        // that node pairs starting on odd columns are 8/16-byte aligned on
        // every level (the paired loads of the level kernels); the pitch
        // holds the offset too, so every node row lies inside its own
        // 32-aligned pitch row (the row the TMA loads of the pipelined level
        // kernels see)
        C.off = 1;
        C.pitch = (cxn + C.off + 31) / 32 * 32;
        C.per = per;
        C.cx = cx;
        C.cy = cy;
        C.diag = -2 * (cx + cy) - md;
        C.idiag = 1.0 / C.diag;
        C.fcx = (float)C.cx;
        C.fcy = (float)C.cy;
        C.fdiag = (float)C.diag;
        C.fidiag = (float)C.idiag;
        C.md = md;
        C.fmd = (float)md;
        const size_t n = (size_t)C.pitch * cyn + 32;  // + the offset
        void *x, *xa, *b, *m;
        if (cudaMalloc(&x, n * es) != cudaSuccess) return 2;
        mg.owned.push_back(x);
        if (cudaMalloc(&xa, n * es) != cudaSuccess) return 2;
        mg.owned.push_back(xa);
        if (cudaMalloc(&b, n * es) != cudaSuccess) return 2;
        mg.owned.push_back(b);
        if (cudaMalloc(&m, n) != cudaSuccess) return 2;
        mg.owned.push_back(m);
        cudaMemset(x, 0, n * es);
        cudaMemset(xa, 0, n * es);
        cudaMemset(b, 0, n * es);
        std::vector<uint8_t> hm(n, 0);
        for (int J = 0; J < cyn; ++J)
            memcpy(&hm[C.off + (size_t)J * C.pitch], &cm[(size_t)J * cxn], cxn);
        if (cudaMemcpy(m, hm.data(), n, cudaMemcpyHostToDevice) != cudaSuccess) return 2;
        C.x = x;
        C.xa = xa;
        C.b = b;
        C.m = (const uint8_t*)m;
        mg.lev.push_back(C);
        mg.hmask.push_back(cm);
        cur.swap(cm);
        nyn = cyn;
        nxn = cxn;
    }
    // first level from which all coarser levels fit in one block's shared
    // memory (at most 160 KB; 16 levels), starting at <= 1100 nodes: the tail
    // runs on one SM, so larger levels are cheaper as grid kernels.
    const int nl = (int)mg.lev.size();
    const size_t budget = 160 * 1024;
    const long long max_first = 1100;
    mg.ltail = nl - 1;
    for (int l = 0; l < nl; ++l)
        if (nl - l <= 16 && tail_smem(mg.lev, l, es) <= budget &&
            (long long)mg.lev[l].nyn * mg.lev[l].nxn <= max_first) {
            mg.ltail = l;
            break;
        }
    mg.tail_smem = tail_smem(mg.lev, mg.ltail, es);
    if (mg.tail_smem > budget) return 3;  // coarsest level alone too large
    const MGLevel& last = mg.lev[nl - 1];
    mg.ncoarse_sweeps = std::max(2, std::min(32, std::max(last.nyn, last.nxn) / 2));
    if (cudaMalloc(&mg.dlev, sizeof(MGLevel) * nl) != cudaSuccess) return 2;
    if (cudaMemcpy(mg.dlev, mg.lev.data(), sizeof(MGLevel) * nl, cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return 2;
    return 0;
}

void mg_free(MGHost& mg)
{
    for (void* p : mg.owned) cudaFree(p);
    mg.owned.clear();
    if (mg.dlev) cudaFree(mg.dlev);
    mg.dlev = nullptr;
    mg.lev.clear();
    mg.hmask.clear();
}

}  // namespace f2d
