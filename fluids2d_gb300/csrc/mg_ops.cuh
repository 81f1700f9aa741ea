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

// ---- the single-block tail: levels l0..nl-1 of the V-cycle ---------------
// One level in shared memory: x, b and the fluid mask of nyn x nxn nodes with
// a one-node border (row pitch P = nxn + 2, node (J, I) at (J+1) P + I+1).
// The border of x is 0, or on an x-periodic level the copy of the opposite
// edge column (written by whichever thread writes that edge node; the two
// share a colour since a periodic level has an even nxn), so the sweeps read
// their neighbours without bounds checks.
template <typename S>
struct TailLev {
    S* x;
    S* b;
    uint8_t* m;
    int nyn, nxn, P, per;
    int hw;           // colour slots per row, (nxn + 1) / 2
    float rhw, rnx;   // 1/hw and 1/nxn (row of a slot index without a division)
    S cx, cy, id, dg;
};

// row of slot k of a row-major table of rows of width w (k < 2^20): the
// fractional part of (k + 0.5)/w is at least 0.5/w away from an integer,
// far above the FP32 rounding of the product
__device__ __forceinline__ int tail_row(int k, float rw)
{
    return __float2int_rz((k + 0.5f) * rw);
}

template <typename S>
__device__ __forceinline__ void tail_put(const TailLev<S>& L, int e, int I, S v)
{
    L.x[e] = v;
    if (L.per) {
        if (I == 0) L.x[e + L.nxn] = v;
        else if (I == L.nxn - 1) L.x[e - L.nxn] = v;
    }
}

// Gauss-Seidel half sweep of colour COL ((J + I) & 1 == COL); ZERO: from a
// zero guess (x = b/diag on the colour; the other colour is 0 already)
template <typename S, int COL, bool ZERO>
__device__ __forceinline__ void tail_half(const TailLev<S>& L)
{
    const int n = L.nyn * L.hw;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int J = tail_row(k, L.rhw);
        const int I = 2 * (k - J * L.hw) + ((J + COL) & 1);
        if (I >= L.nxn) continue;
        const int e = (J + 1) * L.P + I + 1;
        S v = S(0);
        if (L.m[e]) {
            if (ZERO) v = L.b[e] * L.id;
            else
                v = (L.b[e] - (L.cx * (L.x[e - 1] + L.x[e + 1]) +
                               L.cy * (L.x[e - L.P] + L.x[e + L.P]))) *
                    L.id;
        }
        tail_put(L, e, I, v);
    }
    __syncthreads();
}

// residual b - A x at fine node (j, i), 0 outside the level or at non-fluid
// nodes; i may lie one node outside an x-periodic level (wrapped)
template <typename S>
__device__ __forceinline__ S tail_res(const TailLev<S>& F, int j, int i)
{
    if (j < 0 || j >= F.nyn) return S(0);
    if (i < 0 || i >= F.nxn) {
        if (!F.per) return S(0);
        i = i < 0 ? i + F.nxn : i - F.nxn;
    }
    const int e = (j + 1) * F.P + i + 1;
    if (!F.m[e]) return S(0);
    return F.b[e] - ((F.cx * (F.x[e - 1] + F.x[e + 1]) + F.cy * (F.x[e - F.P] + F.x[e + F.P])) +
                     F.dg * F.x[e]);
}

// coarse b = P^T (fine residual): after the pre-smoothing (ending with a
// black half sweep) every black residual is zero, and the fine nodes of full
// weighting that are black are exactly the four edge neighbours of (2J, 2I);
// only the centre and the four corners (all red) contribute
template <typename S>
__device__ __forceinline__ void tail_restrict(const TailLev<S>& F, const TailLev<S>& C)
{
    const int n = C.nyn * C.nxn;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int J = tail_row(k, C.rnx), I = k - J * C.nxn;
        const int e = (J + 1) * C.P + I + 1;
        S v = S(0);
        if (C.m[e]) {
            const int fj = 2 * J, fi = 2 * I;
            const S c = (tail_res(F, fj - 1, fi - 1) + tail_res(F, fj - 1, fi + 1)) +
                        (tail_res(F, fj + 1, fi - 1) + tail_res(F, fj + 1, fi + 1));
            v = tail_res(F, fj, fi) + S(0.25) * c;
        }
        C.b[e] = v;
    }
    __syncthreads();
}

// fine x += P (coarse x), bilinear, at the fluid nodes (the coarse border
// supplies 0 outside the level, or the wrapped column)
template <typename S>
__device__ __forceinline__ void tail_prolong(const TailLev<S>& C, const TailLev<S>& F)
{
    const int n = F.nyn * F.nxn;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int J = tail_row(k, F.rnx), I = k - J * F.nxn;
        const int e = (J + 1) * F.P + I + 1;
        if (!F.m[e]) continue;
        const int cj = J >> 1, ci = I >> 1, oj = J & 1, oi = I & 1;
        const int c0 = (cj + 1) * C.P + ci + 1;
        S v;
        if (!oj && !oi) v = C.x[c0];
        else if (!oj) v = S(0.5) * (C.x[c0] + C.x[c0 + 1]);
        else if (!oi) v = S(0.5) * (C.x[c0] + C.x[c0 + C.P]);
        else
            v = S(0.25) * ((C.x[c0] + C.x[c0 + 1]) + (C.x[c0 + C.P] + C.x[c0 + C.P + 1]));
        tail_put(F, e, I, F.x[e] + v);
    }
    __syncthreads();
}

// The V-cycle on levels l0..nl-1 of `lev` (nt = nl - l0 <= 16), run by one
// thread block: red-black Gauss-Seidel, nu sweeps per leg, (R,B)^k (B,R)^k
// on the coarsest level. All these levels live in shared memory; only b of
// level l0 comes from global memory and only x of level l0 goes back, so each
// phase costs a barrier, not a global-memory round trip. On return sl[0]
// describes level l0 in shared memory.
template <typename S>
__device__ __forceinline__ void tail_vcycle(const MGLevel* __restrict__ lev, int l0,
                                            int nl, int ksweeps,
                                            unsigned char* smem_raw, TailLev<S>* sl, int nu = 1)
{
    const int nt = nl - l0;
    if (threadIdx.x == 0) {
        size_t off = 0;
        for (int q = 0; q < nt; ++q) {
            const MGLevel& G = lev[l0 + q];
            TailLev<S>& D = sl[q];
            D.nyn = G.nyn;
            D.nxn = G.nxn;
            D.P = G.nxn + 2;
            D.per = G.per;
            D.hw = (G.nxn + 1) / 2;
            D.rhw = 1.0f / (float)D.hw;
            D.rnx = 1.0f / (float)G.nxn;
            D.cx = Coef<S>::cx(G);
            D.cy = Coef<S>::cy(G);
            D.id = Coef<S>::idiag(G);
            D.dg = Coef<S>::diag(G);
            const size_t n = (size_t)(G.nyn + 2) * D.P;
            D.x = (S*)(smem_raw + off);
            off += (n * sizeof(S) + 15) / 16 * 16;
            D.b = (S*)(smem_raw + off);
            off += (n * sizeof(S) + 15) / 16 * 16;
            D.m = smem_raw + off;
            off += (n + 15) / 16 * 16;
        }
    }
    __syncthreads();
    for (int q = 0; q < nt; ++q) {
        const MGLevel& G = lev[l0 + q];
        const TailLev<S>& D = sl[q];
        const int n = (D.nyn + 2) * D.P;
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const int J = tail_row(e, 1.0f / (float)D.P) - 1, I = e - (J + 1) * D.P - 1;
            const bool in = J >= 0 && J < D.nyn && I >= 0 && I < D.nxn;
            uint8_t mv = 0;
            S bv = S(0);
            if (in) {
                const long long g = nidx(G, J, I);
                mv = G.m[g];
                if (q == 0) bv = ((const S*)G.b)[g];
            }
            D.x[e] = S(0);
            D.b[e] = bv;
            D.m[e] = mv;
        }
    }
    __syncthreads();
    // down: pre-smooth (red from zero, black, nu - 1 more (red, black)),
    // restrict
    for (int q = 0; q < nt - 1; ++q) {
        const TailLev<S> L = sl[q];
        tail_half<S, 0, true>(L);
        tail_half<S, 1, false>(L);
        for (int k = 1; k < nu; ++k) {
            tail_half<S, 0, false>(L);
            tail_half<S, 1, false>(L);
        }
        tail_restrict<S>(L, sl[q + 1]);
    }
    // coarsest: (R,B)^k (B,R)^k from a zero guess (palindromic = symmetric)
    {
        const TailLev<S> L = sl[nt - 1];
        tail_half<S, 0, true>(L);
        tail_half<S, 1, false>(L);
        for (int s = 1; s < ksweeps; ++s) {
            tail_half<S, 0, false>(L);
            tail_half<S, 1, false>(L);
        }
        for (int s = 0; s < ksweeps; ++s) {
            tail_half<S, 1, false>(L);
            tail_half<S, 0, false>(L);
        }
    }
    // up: prolongate, post-smooth (black, red) x nu
    for (int q = nt - 2; q >= 0; --q) {
        const TailLev<S> L = sl[q];
        tail_prolong<S>(sl[q + 1], L);
        for (int k = 0; k < nu; ++k) {
            tail_half<S, 1, false>(L);
            tail_half<S, 0, false>(L);
        }
    }
    // level l0's x back to global memory
    {
        const MGLevel& G = lev[l0];
        const TailLev<S>& D = sl[0];
        const int n = D.nyn * D.nxn;
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            const int J = tail_row(k, D.rnx), I = k - J * D.nxn;
            ((S*)G.x)[nidx(G, J, I)] = D.x[(J + 1) * D.P + I + 1];
        }
    }
}

}  // namespace f2d
