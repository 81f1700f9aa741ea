// Node operations of the multigrid cycle (used by solver.cu).
#pragma once
#include "mg.cuh"

namespace f2d {

template <typename S>
__device__ __forceinline__ S* lx(const MGLevel& L) { return (S*)L.x; }
template <typename S>
__device__ __forceinline__ S* lb(const MGLevel& L) { return (S*)L.b; }

// operator coefficients in the working precision
template <typename S> struct Coef;
template <> struct Coef<double> {
    static __device__ __forceinline__ double cx(const MGLevel& L) { return L.cx; }
    static __device__ __forceinline__ double cy(const MGLevel& L) { return L.cy; }
    static __device__ __forceinline__ double diag(const MGLevel& L) { return L.diag; }
    static __device__ __forceinline__ double idiag(const MGLevel& L) { return L.idiag; }
    static __device__ __forceinline__ double md(const MGLevel& L) { return L.md; }
};
template <> struct Coef<float> {
    static __device__ __forceinline__ float cx(const MGLevel& L) { return L.fcx; }
    static __device__ __forceinline__ float cy(const MGLevel& L) { return L.fcy; }
    static __device__ __forceinline__ float diag(const MGLevel& L) { return L.fdiag; }
    static __device__ __forceinline__ float idiag(const MGLevel& L) { return L.fidiag; }
    static __device__ __forceinline__ float md(const MGLevel& L) { return L.fmd; }
};

// A x at a fluid node from its value c and the four neighbour values (0 at
// non-fluid nodes), written with differences to the centre:
//   cx ((xW - c) + (xE - c)) + cy ((xS - c) + (xN - c)) - md c,
// which equals cx (xW + xE) + cy (xS + xN) + diag c for diag = -2(cx+cy) - md
// but, for the smooth fields of a converging solve, loses far fewer digits
// to cancellation (the plain form's rounding error grows with the condition
// number, this one's with its square root) - what limits the accuracy of the
// FP32 Krylov products and of the refinement residual.
template <typename S>
__device__ __forceinline__ S apply_diff(S cx, S cy, S md, S c, S w, S e, S s, S n)
{
    return (cx * ((w - c) + (e - c)) + cy * ((s - c) + (n - c))) - md * c;
}

__device__ __forceinline__ long long nidx(const MGLevel& L, int J, int I)
{
    return L.off + (long long)J * L.pitch + I;
}

// value of a neighbour node, 0 outside the level or at non-fluid nodes. The
// index is clamped into the level and both loads are issued unconditionally
// (then selected), so the four neighbour loads of a stencil can be in flight
// together; non-fluid values are never used, whatever they hold.
template <typename S>
__device__ __forceinline__ S nbv(const MGLevel& L, const S* __restrict__ x, int J,
                                 int I)
{
    bool ok = (unsigned)J < (unsigned)L.nyn;
    if (I < 0 || I >= L.nxn) {
        if (L.per) I = I < 0 ? I + L.nxn : I - L.nxn;
        else ok = false;
    }
    const int Jc = min(max(J, 0), L.nyn - 1), Ic = min(max(I, 0), L.nxn - 1);
    const long long k = nidx(L, Jc, Ic);
    const S v = x[k];
    const uint8_t m = L.m[k];
    return (ok && m) ? v : S(0);
}

template <typename S>
__device__ __forceinline__ S apply_off(const MGLevel& L, const S* __restrict__ x,
                                       int J, int I)
{
    return Coef<S>::cx(L) * (nbv(L, x, J, I - 1) + nbv(L, x, J, I + 1)) +
           Coef<S>::cy(L) * (nbv(L, x, J - 1, I) + nbv(L, x, J + 1, I));
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
        x[k] = (mine && L.m[k]) ? b[k] * Coef<S>::idiag(L) : S(0);
        return;
    }
    if (!mine || !L.m[k]) return;
    x[k] = (b[k] - apply_off<S>(L, x, J, I)) * Coef<S>::idiag(L);
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
    return lb<S>(F)[k] - (apply_off<S>(F, x, J, I) + Coef<S>::diag(F) * x[k]);
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
    return L.m[k] ? lb<S>(L)[k] * Coef<S>::idiag(L) : S(0);
}

// ---- the single-block tail: levels l0..nl-1 of the V-cycle ---------------
template <typename S, typename F>
__device__ __forceinline__ void block_for(const MGLevel& L, F f)
{
    const int n = L.nyn * L.nxn;
    for (int k = threadIdx.x; k < n; k += blockDim.x) f(k / L.nxn, k % L.nxn);
    __syncthreads();
}

// Pre-smoothing of one node from a zero guess (red from zero, then one black
// update against those red values, recomputed from b).
template <typename S>
__device__ __forceinline__ void op_presmooth(const MGLevel& L, int J, int I)
{
    const long long k = nidx(L, J, I);
    S v = S(0);
    if (L.m[k]) {
        const S* b = lb<S>(L);
        if (((J + I) & 1) == 0) {
            v = b[k] * Coef<S>::idiag(L);
        } else {
            const S off = Coef<S>::cx(L) * (red_from_zero<S>(L, J, I - 1) + red_from_zero<S>(L, J, I + 1)) +
                          Coef<S>::cy(L) * (red_from_zero<S>(L, J - 1, I) + red_from_zero<S>(L, J + 1, I));
            v = (b[k] - off) * Coef<S>::idiag(L);
        }
    }
    lx<S>(L)[k] = v;
}

// The V-cycle on levels l0..nl-1 of `lev`, run by one thread block. All
// these levels live in shared memory (dense nyn x nxn, x, b, mask); only b of
// level l0 comes from global memory and only x of level l0 goes back, so each
// phase costs a barrier, not a global-memory round trip.
template <typename S>
__device__ __forceinline__ void tail_vcycle(const MGLevel* __restrict__ lev, int l0,
                                            int nl, int ksweeps,
                                            unsigned char* smem_raw, MGLevel* sl, int nu = 1)
{
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
        for (int k = 1; k < nu; ++k) {
            block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 0, false); });
            block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 1, false); });
        }
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
        for (int k = 0; k < nu; ++k) {
            block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 1, false); });
            block_for<S>(L, [&](int J, int I) { op_smooth<S>(L, J, I, 0, false); });
        }
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


}  // namespace f2d
