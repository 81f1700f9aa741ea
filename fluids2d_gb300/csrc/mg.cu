// Multigrid-preconditioned CG for the masked vertex Poisson/Helmholtz
// operator (the reference factorises it with SuperLU, elliptic.py:71-87;
// here it is solved matrix-free).
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

#include "mg.cuh"

namespace f2d {

template <typename S>
__device__ __forceinline__ S* lx(const MGLevel& L) { return (S*)L.x; }
template <typename S>
__device__ __forceinline__ S* lb(const MGLevel& L) { return (S*)L.b; }

__device__ __forceinline__ long long nidx(const MGLevel& L, int J, int I)
{
    return L.off + (long long)J * L.pitch + I;
}

// value of a neighbour node, 0 outside the level or at non-fluid nodes
template <typename S>
__device__ __forceinline__ S nbv(const MGLevel& L, const S* __restrict__ x, int J,
                                 int I)
{
    if (J < 0 || J >= L.nyn) return S(0);
    if (I < 0 || I >= L.nxn) {
        if (!L.per) return S(0);
        I = I < 0 ? I + L.nxn : I - L.nxn;
    }
    const long long k = nidx(L, J, I);
    return L.m[k] ? x[k] : S(0);
}

template <typename S>
__device__ __forceinline__ S apply_off(const MGLevel& L, const S* __restrict__ x,
                                       int J, int I)
{
    return S(L.cx) * (nbv(L, x, J, I - 1) + nbv(L, x, J, I + 1)) +
           S(L.cy) * (nbv(L, x, J - 1, I) + nbv(L, x, J + 1, I));
}

// ---- node operations (shared by the grid kernels and the tail block) ------

// Gauss-Seidel half sweep of one colour. zero_init (red only): x = b/diag on
// red nodes and x = 0 elsewhere (the sweep that starts from a zero guess).
template <typename S>
__device__ __forceinline__ void op_smooth(const MGLevel& L, int J, int I, int color,
                                          bool zero_init)
{
    const long long k = nidx(L, J, I);
    S* x = lx<S>(L);
    const S* b = lb<S>(L);
    const bool mine = ((J + I) & 1) == color;
    if (zero_init) {
        x[k] = (mine && L.m[k]) ? b[k] * S(L.idiag) : S(0);
        return;
    }
    if (!mine || !L.m[k]) return;
    x[k] = (b[k] - apply_off<S>(L, x, J, I)) * S(L.idiag);
}

// residual of the fine level at node (J, I) (0 at non-fluid nodes)
template <typename S>
__device__ __forceinline__ S fine_res(const MGLevel& F, int J, int I)
{
    if (J < 0 || J >= F.nyn) return S(0);
    if (I < 0 || I >= F.nxn) {
        if (!F.per) return S(0);
        I = I < 0 ? I + F.nxn : I - F.nxn;
    }
    const long long k = nidx(F, J, I);
    if (!F.m[k]) return S(0);
    const S* x = lx<S>(F);
    return lb<S>(F)[k] - (apply_off<S>(F, x, J, I) + S(F.diag) * x[k]);
}

// coarse right-hand side = P^T (fine residual). After the pre-smoothing
// (red from a zero guess, then black) the residual of every black node is
// zero, and the fine nodes of full weighting that are black are exactly the
// four edge neighbours of (2J, 2I); only the centre and the four corners
// (all red) contribute.
template <typename S>
__device__ __forceinline__ void op_restrict(const MGLevel& F, const MGLevel& C, int J,
                                            int I)
{
    const long long k = nidx(C, J, I);
    S v = S(0);
    if (C.m[k]) {
        const int fj = 2 * J, fi = 2 * I;
        const S c = (fine_res<S>(F, fj - 1, fi - 1) + fine_res<S>(F, fj - 1, fi + 1)) +
                    (fine_res<S>(F, fj + 1, fi - 1) + fine_res<S>(F, fj + 1, fi + 1));
        v = fine_res<S>(F, fj, fi) + S(0.25) * c;
    }
    lb<S>(C)[k] = v;
}

// coarse node value for prolongation (0 outside / non-fluid: x is 0 there)
template <typename S>
__device__ __forceinline__ S cval(const MGLevel& C, int J, int I)
{
    if (J < 0 || J >= C.nyn) return S(0);
    if (I >= C.nxn) {
        if (!C.per) return S(0);
        I -= C.nxn;
    }
    return lx<S>(C)[nidx(C, J, I)];
}

// fine x += P (coarse x), bilinear
template <typename S>
__device__ __forceinline__ void op_prolong(const MGLevel& C, const MGLevel& F, int J,
                                           int I)
{
    const long long k = nidx(F, J, I);
    if (!F.m[k]) return;
    const int cj = J >> 1, ci = I >> 1;
    const int oj = J & 1, oi = I & 1;
    S v;
    if (!oj && !oi) v = cval<S>(C, cj, ci);
    else if (!oj) v = S(0.5) * (cval<S>(C, cj, ci) + cval<S>(C, cj, ci + 1));
    else if (!oi) v = S(0.5) * (cval<S>(C, cj, ci) + cval<S>(C, cj + 1, ci));
    else
        v = S(0.25) * ((cval<S>(C, cj, ci) + cval<S>(C, cj, ci + 1)) +
                       (cval<S>(C, cj + 1, ci) + cval<S>(C, cj + 1, ci + 1)));
    lx<S>(F)[k] += v;
}

// ---- grid kernels --------------------------------------------------------
template <typename S>
__global__ void k_mg_smooth(MGLevel L, int color, int zero_init)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    if (J < L.nyn && I < L.nxn) op_smooth<S>(L, J, I, color, zero_init != 0);
}

// Pre-smoothing from a zero guess in one pass: red nodes x = b/diag, black
// nodes one Gauss-Seidel update against those red values, which are
// recomputed from b instead of read back (same result as two half sweeps).
template <typename S>
__device__ __forceinline__ S red_from_zero(const MGLevel& L, int J, int I)
{
    if (J < 0 || J >= L.nyn) return S(0);
    if (I < 0 || I >= L.nxn) {
        if (!L.per) return S(0);
        I = I < 0 ? I + L.nxn : I - L.nxn;
    }
    const long long k = nidx(L, J, I);
    return L.m[k] ? lb<S>(L)[k] * S(L.idiag) : S(0);
}

template <typename S>
__global__ void k_mg_presmooth(MGLevel L)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    if (J >= L.nyn || I >= L.nxn) return;
    const long long k = nidx(L, J, I);
    S v = S(0);
    if (L.m[k]) {
        const S* b = lb<S>(L);
        if (((J + I) & 1) == 0) {
            v = b[k] * S(L.idiag);
        } else {
            const S off = S(L.cx) * (red_from_zero<S>(L, J, I - 1) + red_from_zero<S>(L, J, I + 1)) +
                          S(L.cy) * (red_from_zero<S>(L, J - 1, I) + red_from_zero<S>(L, J + 1, I));
            v = (b[k] - off) * S(L.idiag);
        }
    }
    lx<S>(L)[k] = v;
}

template <typename S>
__global__ void k_mg_restrict(MGLevel F, MGLevel C)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    if (J < C.nyn && I < C.nxn) op_restrict<S>(F, C, J, I);
}

template <typename S>
__global__ void k_mg_prolong(MGLevel C, MGLevel F)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    if (J < F.nyn && I < F.nxn) op_prolong<S>(C, F, J, I);
}

// ---- the single-block tail: levels l0..nl-1 of the V-cycle ---------------
template <typename S, typename F>
__device__ __forceinline__ void block_for(const MGLevel& L, F f)
{
    const int n = L.nyn * L.nxn;
    for (int k = threadIdx.x; k < n; k += blockDim.x) f(k / L.nxn, k % L.nxn);
    __syncthreads();
}

template <typename S>
__global__ void __launch_bounds__(1024) k_mg_tail(const MGLevel* __restrict__ lev,
                                                  int l0, int nl, int ksweeps)
{
    // All tail levels live in shared memory (dense nyn x nxn, x, b, mask);
    // only b of level l0 comes from global memory and only x of level l0 goes
    // back, so each phase costs a barrier, not a global-memory round trip.
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ MGLevel sl[16];
    if (threadIdx.x == 0) {
        size_t off = 0;
        for (int l = l0; l < nl; ++l) {
            MGLevel D = lev[l];
            const size_t n = (size_t)D.nyn * D.nxn;
            D.pitch = D.nxn;
            D.off = 0;
            D.x = smem_raw + off;
            off += (n * sizeof(S) + 15) / 16 * 16;
            D.b = smem_raw + off;
            off += (n * sizeof(S) + 15) / 16 * 16;
            D.m = (const uint8_t*)(smem_raw + off);
            off += (n + 15) / 16 * 16;
            sl[l - l0] = D;
        }
    }
    __syncthreads();
    for (int l = l0; l < nl; ++l) {
        const MGLevel& L = lev[l];
        const MGLevel& D = sl[l - l0];
        const int n = L.nyn * L.nxn;
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            const long long g = nidx(L, k / L.nxn, k % L.nxn);
            ((uint8_t*)D.m)[k] = L.m[g];
            if (l == l0) ((S*)D.b)[k] = ((const S*)L.b)[g];
        }
    }
    __syncthreads();
    const int nt = nl - l0;
    // down: pre-smooth (red from zero, black) and restrict
    for (int q = 0; q < nt - 1; ++q) {
        const MGLevel L = sl[q], C = sl[q + 1];
        block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 0, true); });
        block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 1, false); });
        block_for<S>(C, [&](int J, int I) { op_restrict<S>(L, C, J, I); });
    }
    // coarsest: (R,B)^k (B,R)^k from a zero guess (palindromic = symmetric)
    {
        const MGLevel L = sl[nt - 1];
        block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 0, true); });
        block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 1, false); });
        for (int s = 1; s < ksweeps; ++s) {
            block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 0, false); });
            block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 1, false); });
        }
        for (int s = 0; s < ksweeps; ++s) {
            block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 1, false); });
            block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 0, false); });
        }
    }
    // up: prolongate, post-smooth (black, red)
    for (int q = nt - 2; q >= 0; --q) {
        const MGLevel L = sl[q], C = sl[q + 1];
        block_for<S>(L, [&](int J, int I) { op_prolong<S>(C, L, J, I); });
        block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 1, false); });
        block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 0, false); });
    }
    // level l0's x back to global memory
    {
        const MGLevel G = lev[l0];
        const MGLevel L = sl[0];
        const int n = L.nyn * L.nxn;
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            ((S*)G.x)[nidx(G, k / L.nxn, k % L.nxn)] = ((const S*)L.x)[k];
    }
}

// shared-memory bytes of the tail levels l0..nl-1
static size_t tail_smem(const std::vector<MGLevel>& lev, int l0, size_t es)
{
    size_t off = 0;
    for (size_t l = l0; l < lev.size(); ++l) {
        const size_t n = (size_t)lev[l].nyn * lev[l].nxn;
        off += 2 * ((n * es + 15) / 16 * 16) + (n + 15) / 16 * 16;
    }
    return off;
}

// ---- PCG kernels on level 0 ----------------------------------------------
// The Krylov vectors x, r, p, q and all dot products are FP64. The V-cycle
// (type S) works on its own level-0 copies: rmg = (S) r as its right-hand
// side and zmg as its result. With S = float this is the mixed-precision
// form: the FP64 residual recurrence refines the FP32-preconditioned
// iterate to FP64 accuracy. With S = double, rmg aliases r.
__device__ __forceinline__ double applyA64(const MGLevel& L, const double* __restrict__ x,
                                           int J, int I, long long k)
{
    return apply_off<double>(L, x, J, I) + L.diag * x[k];
}

template <typename S>
__device__ __forceinline__ void store_rmg(S* rmg, const double* r, long long k, double v)
{
    if ((const void*)rmg != (const void*)r) rmg[k] = S(v);
}

// r = b - A x, reductions <b,b>, <r,r>
template <typename S>
__global__ void k_pcg_init(MGLevel L, const double* __restrict__ x,
                           const double* __restrict__ b, double* r, S* rmg,
                           DevScalars* sc, double* partials,
                           cudaGraphConditionalHandle cond)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    double v[2] = {0.0, 0.0};
    if (J < L.nyn && I < L.nxn) {
        const long long k = nidx(L, J, I);
        double rv = 0.0;
        if (L.m[k]) {
            const double bv = b[k];
            rv = bv - applyA64(L, x, J, I, k);
            v[0] = bv * bv;
            v[1] = rv * rv;
        }
        r[k] = rv;
        store_rmg<S>(rmg, r, k, rv);
    }
    if (grid_reduce<2, false>(v, partials, &sc->counter[1])) {
        sc->bb = v[0];
        sc->rr = v[1];
        sc->iter = 0;
        // b = 0: the solution is 0, reached by one pass of the loop body
        const int zero = (v[0] == 0.0);
        sc->converged = zero ? 0 : (v[1] <= sc->tol2 * v[0]);
        sc->pad1 = zero;
        if (cond) cudaGraphSetConditional(cond, sc->converged ? 0u : 1u);
    }
}

// rz = <r, z>; beta = rz/rz_old (0 on the first iteration)
template <typename S>
__global__ void k_pcg_rz(MGLevel L, const double* __restrict__ r, const S* __restrict__ z,
                         DevScalars* sc, double* partials)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    double v[1] = {0.0};
    if (J < L.nyn && I < L.nxn) {
        const long long k = nidx(L, J, I);
        if (L.m[k]) v[0] = r[k] * (double)z[k];
    }
    if (grid_reduce<1, false>(v, partials, &sc->counter[2])) {
        sc->beta = sc->iter == 0 ? 0.0 : v[0] / sc->rz;
        sc->rz = v[0];
    }
}

// Last red half sweep of the V-cycle on level 0 fused with rz = <r, z>
// (r the FP64 CG residual) and beta = rz / rz_old.
template <typename S>
__global__ void k_mg_red_dot(MGLevel L, const double* __restrict__ r64, DevScalars* sc,
                             double* partials)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    double v[1] = {0.0};
    if (J < L.nyn && I < L.nxn) {
        const long long k = nidx(L, J, I);
        if (L.m[k]) {
            S* x = lx<S>(L);
            const S* b = lb<S>(L);
            S z = x[k];
            if (((J + I) & 1) == 0) {
                z = (b[k] - apply_off<S>(L, x, J, I)) * S(L.idiag);
                x[k] = z;
            }
            v[0] = r64[k] * (double)z;
        }
    }
    if (grid_reduce<1, false>(v, partials, &sc->counter[2])) {
        sc->beta = sc->iter == 0 ? 0.0 : v[0] / sc->rz;
        sc->rz = v[0];
    }
}

// p = z + beta p
template <typename S>
__global__ void k_pcg_p(MGLevel L, const S* __restrict__ z, double* __restrict__ p,
                        const DevScalars* sc)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    if (J >= L.nyn || I >= L.nxn) return;
    const long long k = nidx(L, J, I);
    const double beta = sc->beta;
    p[k] = L.m[k] ? (double)z[k] + beta * p[k] : 0.0;
}

// q = A p, pq = <p, q>, alpha = rz / pq
__global__ void k_pcg_spmv(MGLevel L, const double* __restrict__ p, double* __restrict__ q,
                           DevScalars* sc, double* partials)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    double v[1] = {0.0};
    if (J < L.nyn && I < L.nxn) {
        const long long k = nidx(L, J, I);
        double qv = 0.0;
        if (L.m[k]) {
            qv = applyA64(L, p, J, I, k);
            v[0] = p[k] * qv;
        }
        q[k] = qv;
    }
    if (grid_reduce<1, false>(v, partials, &sc->counter[3])) {
        sc->pq = v[0];
        sc->alpha = sc->rz / v[0];
    }
}

// x += alpha p, r -= alpha q, rr = <r,r>, convergence test, loop condition
template <typename S>
__global__ void k_pcg_xr(MGLevel L, double* __restrict__ x, double* r, S* rmg,
                         const double* __restrict__ p, const double* __restrict__ q,
                         DevScalars* sc, double* partials,
                         cudaGraphConditionalHandle cond)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    double v[1] = {0.0};
    const int zero = sc->pad1;
    if (J < L.nyn && I < L.nxn) {
        const long long k = nidx(L, J, I);
        if (L.m[k]) {
            if (zero) {
                x[k] = 0.0;
                r[k] = 0.0;
                store_rmg<S>(rmg, r, k, 0.0);
            } else {
                const double a = sc->alpha;
                x[k] += a * p[k];
                const double rv = r[k] - a * q[k];
                r[k] = rv;
                store_rmg<S>(rmg, r, k, rv);
                v[0] = rv * rv;
            }
        }
    }
    if (grid_reduce<1, false>(v, partials, &sc->counter[4])) {
        sc->rr = v[0];
        sc->iter += 1;
        sc->total_iters += 1;
        int conv = zero || (v[0] <= sc->tol2 * sc->bb);
        if (!(v[0] == v[0])) {  // NaN residual: stop and report
            conv = 1;
            atomicOr(&sc->status, ST_NONFINITE);
        }
        sc->converged = conv;
        sc->pad1 = 0;
        const int more = !conv && sc->iter < sc->maxit;
        if (!conv && !more) atomicOr(&sc->status, ST_PCG_MAXIT);
        if (cond) cudaGraphSetConditional(cond, more ? 1u : 0u);
    }
}

__global__ void k_pcg_setup(DevScalars* sc, double tol2, int maxit)
{
    sc->tol2 = tol2;
    sc->maxit = maxit;
}

// ---- host side -------------------------------------------------------------
static dim3 lvl_grid(const MGLevel& L) { return dim3((L.nxn + 31) / 32, (L.nyn + 7) / 8); }

// One V-cycle on levels 0..nl-1. With r64, the final red half sweep of
// level 0 also forms rz = <r, z> (needs ltail > 0).
template <typename S>
static int vcycle_record(MGHost& mg, cudaStream_t s, const double* r64, DevScalars* sc,
                         double* partials)
{
    const int nl = (int)mg.lev.size();
    const dim3 blk(32, 8);
    for (int l = 0; l < mg.ltail; ++l) {
        const MGLevel& L = mg.lev[l];
        k_mg_presmooth<S><<<lvl_grid(L), blk, 0, s>>>(L);
        k_mg_restrict<S><<<lvl_grid(mg.lev[l + 1]), blk, 0, s>>>(L, mg.lev[l + 1]);
    }
    k_mg_tail<S><<<1, 1024, mg.tail_smem, s>>>(mg.dlev, mg.ltail, nl, mg.ncoarse_sweeps);
    for (int l = mg.ltail - 1; l >= 0; --l) {
        const MGLevel& L = mg.lev[l];
        k_mg_prolong<S><<<lvl_grid(L), blk, 0, s>>>(mg.lev[l + 1], L);
        k_mg_smooth<S><<<lvl_grid(L), blk, 0, s>>>(L, 1, 0);
        if (l == 0 && r64)
            k_mg_red_dot<S><<<lvl_grid(L), blk, 0, s>>>(L, r64, sc, partials);
        else
            k_mg_smooth<S><<<lvl_grid(L), blk, 0, s>>>(L, 0, 0);
    }
    return (int)cudaGetLastError();
}

template <typename S>
static int body_record(MGHost& mg, const PCGVecs& v, DevScalars* sc,
                       cudaGraphConditionalHandle cond, cudaStream_t s)
{
    const MGLevel& L = mg.lev[0];
    const dim3 g = lvl_grid(L), blk(32, 8);
    const bool fuse = mg.ltail > 0;
    int e = vcycle_record<S>(mg, s, fuse ? (const double*)v.r : nullptr, sc, v.partials);
    if (e) return e;
    if (!fuse)
        k_pcg_rz<S><<<g, blk, 0, s>>>(L, (const double*)v.r, (const S*)v.z, sc, v.partials);
    k_pcg_p<S><<<g, blk, 0, s>>>(L, (const S*)v.z, (double*)v.p, sc);
    k_pcg_spmv<<<g, blk, 0, s>>>(L, (const double*)v.p, (double*)v.q, sc, v.partials);
    k_pcg_xr<S><<<g, blk, 0, s>>>(L, (double*)v.x, (double*)v.r, (S*)v.rmg,
                                  (const double*)v.p, (const double*)v.q, sc, v.partials,
                                  cond);
    return (int)cudaGetLastError();
}

template <typename S>
static int pcg_record_t(MGHost& mg, const PCGVecs& v, DevScalars* sc, double tol,
                        int maxit, cudaStream_t s, cudaStream_t s2)
{
    const MGLevel& L = mg.lev[0];
    const dim3 g = lvl_grid(L), blk(32, 8);
    cudaStreamCaptureStatus st;
    cudaGraph_t graph = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaError_t ce = cudaStreamGetCaptureInfo(s, &st, nullptr, &graph, &deps, nullptr, &ndeps);
    if (ce != cudaSuccess) return (int)ce;
    k_pcg_setup<<<1, 1, 0, s>>>(sc, tol * tol, maxit);
    if (st != cudaStreamCaptureStatusActive) {
        // host-driven loop (used outside graphs): one sync per iteration
        k_pcg_init<S><<<g, blk, 0, s>>>(L, (const double*)v.x, (const double*)v.b,
                                         (double*)v.r, (S*)v.rmg, sc, v.partials, 0);
        for (int it = 0; it < maxit + 1; ++it) {
            DevScalars h;
            if ((ce = cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
                return (int)ce;
            if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return (int)ce;
            if (h.converged || h.iter >= maxit) break;
            int e = body_record<S>(mg, v, sc, 0, s);
            if (e) return e;
        }
        return (int)cudaGetLastError();
    }
    // graph: the loop condition lives in the captured graph
    cudaGraphConditionalHandle cond;
    ce = cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault);
    if (ce != cudaSuccess) return (int)ce;
    k_pcg_init<S><<<g, blk, 0, s>>>(L, (const double*)v.x, (const double*)v.b, (double*)v.r,
                                     (S*)v.rmg, sc, v.partials, cond);
    if ((ce = cudaGetLastError()) != cudaSuccess) return (int)ce;
    ce = cudaStreamGetCaptureInfo(s, &st, nullptr, &graph, &deps, nullptr, &ndeps);
    if (ce != cudaSuccess) return (int)ce;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    ce = cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp);
    if (ce != cudaSuccess) return (int)ce;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    ce = cudaStreamBeginCaptureToGraph(s2, body, nullptr, nullptr, 0,
                                       cudaStreamCaptureModeRelaxed);
    if (ce != cudaSuccess) return (int)ce;
    int e = body_record<S>(mg, v, sc, cond, s2);
    cudaGraph_t body_out;
    ce = cudaStreamEndCapture(s2, &body_out);
    if (e) return e;
    if (ce != cudaSuccess) return (int)ce;
    ce = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                             cudaStreamSetCaptureDependencies);
    return (int)ce;
}

int pcg_record(MGHost& mg, const PCGVecs& v, DevScalars* sc, double tol, int maxit,
               cudaStream_t s, cudaStream_t s2)
{
    if (mg.prec == 0) return pcg_record_t<double>(mg, v, sc, tol, maxit, s, s2);
    return pcg_record_t<float>(mg, v, sc, tol, maxit, s, s2);
}

// Build the level hierarchy from the level-0 fluid mask (host copy).
int mg_build(MGHost& mg, int nyn0, int nxn0, long long pitch0, long long off0, int per,
             const uint8_t* hmask0, const uint8_t* dmask0, void* z0, void* r0, double cx,
             double cy, double maindiag, int prec)
{
    mg_free(mg);
    mg.prec = prec;
    const size_t es = prec == 0 ? sizeof(double) : sizeof(float);
    MGLevel L0;
    memset(&L0, 0, sizeof(L0));
    L0.x = z0;
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
    mg.lev.push_back(L0);

    // host masks of each level, dense nyn x nxn
    std::vector<uint8_t> cur((size_t)nyn0 * nxn0);
    for (int J = 0; J < nyn0; ++J)
        for (int I = 0; I < nxn0; ++I)
            cur[(size_t)J * nxn0 + I] = hmask0[off0 + (long long)J * pitch0 + I];
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
        C.pitch = (cxn + 31) / 32 * 32;
        C.off = 0;
        C.per = per;
        C.cx = cx;
        C.cy = cy;
        C.diag = -2 * (cx + cy) - md;
        C.idiag = 1.0 / C.diag;
        const size_t n = (size_t)C.pitch * cyn;
        void *x, *b, *m;
        if (cudaMalloc(&x, n * es) != cudaSuccess) return 2;
        mg.owned.push_back(x);
        if (cudaMalloc(&b, n * es) != cudaSuccess) return 2;
        mg.owned.push_back(b);
        if (cudaMalloc(&m, n) != cudaSuccess) return 2;
        mg.owned.push_back(m);
        cudaMemset(x, 0, n * es);
        cudaMemset(b, 0, n * es);
        std::vector<uint8_t> hm(n, 0);
        for (int J = 0; J < cyn; ++J)
            memcpy(&hm[(size_t)J * C.pitch], &cm[(size_t)J * cxn], cxn);
        if (cudaMemcpy(m, hm.data(), n, cudaMemcpyHostToDevice) != cudaSuccess) return 2;
        C.x = x;
        C.b = b;
        C.m = (const uint8_t*)m;
        mg.lev.push_back(C);
        cur.swap(cm);
        nyn = cyn;
        nxn = cxn;
    }
    // first level from which all coarser levels fit in one block's shared
    // memory (at most 160 KB; 16 levels). In FP64 the tail starts at <= 1100
    // nodes: one SM's FP64 rate makes larger levels cheaper as grid kernels.
    const int nl = (int)mg.lev.size();
    const size_t budget = 160 * 1024;
    const long long max_first = prec == 0 ? 1100 : 4500;
    mg.ltail = nl - 1;
    for (int l = 0; l < nl; ++l)
        if (nl - l <= 16 && tail_smem(mg.lev, l, es) <= budget &&
            (long long)mg.lev[l].nyn * mg.lev[l].nxn <= max_first) {
            mg.ltail = l;
            break;
        }
    mg.tail_smem = tail_smem(mg.lev, mg.ltail, es);
    if (mg.tail_smem > budget) return 3;  // coarsest level alone too large
    cudaError_t fe = prec == 0
        ? cudaFuncSetAttribute(k_mg_tail<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)mg.tail_smem)
        : cudaFuncSetAttribute(k_mg_tail<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)mg.tail_smem);
    if (fe != cudaSuccess) return 4;
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
}

}  // namespace f2d
