// Multigrid-preconditioned CG for the masked cell-centred Poisson operator
// with Neumann walls: Poisson2D(mesh, "c") of the reference (elliptic.py:
// 71-87, 114-195), the pressure solve of pressure_projection
// (operators.py:114-119). The reference factorises the singular matrix with
// SuperLU; here it is solved matrix-free.
//
// Operator at a fluid cell c, with face couplings f (dy/dx across x-faces,
// dx/dy across y-faces, 0 where either side is not fluid):
//     (A x)_c = sum_faces f (x_n - x_c)
// which is the reference's matrix (off-diagonals for present neighbours,
// diagonal minus their sum), in difference form. A is singular (constants),
// so the right-hand side is projected to zero mean over the fluid cells (the
// compatibility condition; for a divergence it is zero up to rounding) and
// the solution is returned with zero mean: the pressure is defined up to a
// constant, and only its gradient enters the model.
//
// Preconditioner: cell-centred V-cycle with red-black Gauss-Seidel (nu sweeps
// per leg, symmetric order), coarse cells = 2x2 agglomerates (fluid if any
// child is), restriction = sum of the children's residuals, prolongation =
// the parent's value, coarse couplings = half the sum of the fine face
// couplings a coarse face contains. (The sum itself is the Galerkin operator
// R A P for this R and P; with piecewise-constant P it is twice too stiff for
// smooth errors, and the coarse correction comes out halved - half the sum is
// the re-discretised coupling where the face is fully open and keeps the
// partial openings of masked faces.) Coarsest level by (R,B)^k (B,R)^k in one
// thread block. The FP32 form runs the cycle in FP32 (levels, couplings and
// smoothing in float; its right-hand side is the FP64 Krylov residual
// rounded, its result converted back), while the Krylov vectors, the
// operator products, the dot products and the zero-mean projections stay
// FP64. Single component assumed (a
// fluid domain made of several disconnected parts would need a projection
// per part).
#include <algorithm>
#include <cstring>

#include "graph_while.cuh"
#include "nsolver.cuh"

namespace f2d {

__device__ __forceinline__ long long cidx(const NLevel& L, int J, int I)
{
    return L.off + (long long)J * L.pitch + I;
}

// A x at fluid cell (J, I); also the sum of its couplings. S: the value
// and coupling type of the level (the FP32 cycle's levels are float)
template <typename S>
__device__ __forceinline__ S n_apply(const NLevel& L, const S* __restrict__ x, int J, int I,
                                     S* csum)
{
    const S* __restrict__ fx = (const S*)L.fx;
    const S* __restrict__ fy = (const S*)L.fy;
    const long long k = cidx(L, J, I);
    const S xc = x[k];
    const S cw = fx[k], cs = fy[k];
    S ce = S(0), cn = S(0), xw = S(0), xe = S(0), xs = S(0), xn = S(0);
    if (I > 0) xw = x[k - 1];
    else if (L.per) xw = x[cidx(L, J, L.nxn - 1)];
    if (I + 1 < L.nxn) {
        ce = fx[k + 1];
        xe = x[k + 1];
    } else if (L.per) {
        const long long k0 = cidx(L, J, 0);
        ce = fx[k0];
        xe = x[k0];
    }
    if (J > 0) xs = x[k - L.pitch];
    if (J + 1 < L.nyn) {
        cn = fy[k + L.pitch];
        xn = x[k + L.pitch];
    }
    if (csum) *csum = (cw + ce) + (cs + cn);
    return (cw * (xw - xc) + ce * (xe - xc)) + (cs * (xs - xc) + cn * (xn - xc));
}

__device__ __forceinline__ bool cell(const NLevel& L, int& J, int& I)
{
    I = blockIdx.x * blockDim.x + threadIdx.x;
    J = blockIdx.y * blockDim.y + threadIdx.y;
    return J < L.nyn && I < L.nxn;
}

// ---- multigrid -------------------------------------------------------------
template <typename S>
__device__ __forceinline__ void n_smooth_cell(const NLevel& L, int J, int I)
{
    S* __restrict__ x = (S*)L.x;
    const S* __restrict__ b = (const S*)L.b;
    const long long k = cidx(L, J, I);
    if (!L.m[k]) return;
    S cs;
    const S ax = n_apply<S>(L, x, J, I, &cs);
    // A x = sum c_n x_n - cs x_c = b  ->  x_c = (sum c_n x_n - b) / cs
    if (cs > S(0)) x[k] = ((ax + cs * x[k]) - b[k]) / cs;
}

// one thread per cell of the colour: thread column I' of row J takes cell
// I = 2 I' + ((J + color) & 1)
template <typename S>
__global__ void k_ns_smooth(const NLevel* __restrict__ levs, int l, int color)
{
    const NLevel L = levs[l];
    const int J = blockIdx.y * blockDim.y + threadIdx.y;
    const int I = 2 * (blockIdx.x * blockDim.x + threadIdx.x) + ((J + color) & 1);
    if (J >= L.nyn || I >= L.nxn) return;
    n_smooth_cell<S>(L, J, I);
}

// coarse b = sum of the fluid children's residuals; coarse x = 0
template <typename S>
__global__ void k_ns_restrict(const NLevel* __restrict__ levs, int l)
{
    const NLevel F = levs[l], C = levs[l + 1];
    int J, I;
    if (!cell(C, J, I)) return;
    const S* __restrict__ fxv = (const S*)F.x;
    const S* __restrict__ fb = (const S*)F.b;
    S v = S(0);
    for (int a = 0; a < 2; ++a)
        for (int c = 0; c < 2; ++c) {
            const int fj = 2 * J + a, fi = 2 * I + c;
            if (fj >= F.nyn || fi >= F.nxn) continue;
            const long long k = cidx(F, fj, fi);
            if (F.m[k]) v += fb[k] - n_apply<S>(F, fxv, fj, fi, nullptr);
        }
    const long long kc = cidx(C, J, I);
    ((S*)C.b)[kc] = C.m[kc] ? v : S(0);
    ((S*)C.x)[kc] = S(0);
}

template <typename S>
__global__ void k_ns_prolong(const NLevel* __restrict__ levs, int l)
{
    const NLevel F = levs[l], C = levs[l + 1];
    int J, I;
    if (!cell(F, J, I)) return;
    const long long k = cidx(F, J, I);
    if (F.m[k]) ((S*)F.x)[k] += ((const S*)C.x)[cidx(C, J >> 1, I >> 1)];
}

template <typename S>
__global__ void k_ns_zero(const NLevel* __restrict__ levs, int l)
{
    const NLevel L = levs[l];
    int J, I;
    if (cell(L, J, I)) ((S*)L.x)[cidx(L, J, I)] = S(0);
}

// coarsest level: (R,B)^k (B,R)^k from x = 0, one block
template <typename S>
__global__ void __launch_bounds__(1024) k_ns_coarse(const NLevel* __restrict__ levs, int l,
                                                    int ksweeps)
{
    const NLevel L = levs[l];
    const int n = L.nyn * L.nxn;
    for (int e = threadIdx.x; e < n; e += blockDim.x)
        ((S*)L.x)[cidx(L, e / L.nxn, e % L.nxn)] = S(0);
    __syncthreads();
    for (int s = 0; s < 2 * ksweeps; ++s) {
        for (int h = 0; h < 2; ++h) {
            const int color = s < ksweeps ? h : 1 - h;
            for (int e = threadIdx.x; e < n; e += blockDim.x) {
                const int J = e / L.nxn, I = e % L.nxn;
                if (((J + I) & 1) == color) n_smooth_cell<S>(L, J, I);
            }
            __syncthreads();
        }
    }
}

// FP32 cycle: its level-0 right-hand side from the FP64 Krylov residual, and
// the preconditioned residual back in FP64
__global__ void k_ns_to32(NLevel L, const double* __restrict__ r, float* __restrict__ r32)
{
    int J, I;
    if (!cell(L, J, I)) return;
    const long long k = cidx(L, J, I);
    r32[k] = (float)r[k];
}

__global__ void k_ns_to64(NLevel L, const float* __restrict__ z32, double* __restrict__ z)
{
    int J, I;
    if (!cell(L, J, I)) return;
    const long long k = cidx(L, J, I);
    z[k] = (double)z32[k];
}

// ---- Krylov ----------------------------------------------------------------
__global__ void k_ns_sum(NLevel L, const double* __restrict__ a, DevScalars* sc,
                         double* partials)
{
    int J, I;
    double w[1] = {0.0};
    if (cell(L, J, I)) {
        const long long k = cidx(L, J, I);
        if (L.m[k]) w[0] = a[k];
    }
    if (grid_reduce<1, false>(w, partials, &sc->counter[0])) sc->t = w[0];  // the sum
}

// b -= mean(b); r = b - A x; <b,b>, <r,r>; start state
__global__ void k_ns_init(NLevel L, double* __restrict__ r, DevScalars* sc, double* partials,
                          NGlobals* eg, long long nfluid, cudaGraphConditionalHandle cond)
{
    int J, I;
    double w[2] = {0.0, 0.0};
    const double mean = sc->t / (double)nfluid;
    if (cell(L, J, I)) {
        const long long k = cidx(L, J, I);
        double rv = 0.0;
        if (L.m[k]) {
            double* b = (double*)L.b;
            const double bv = b[k] - mean;
            b[k] = bv;
            rv = bv - n_apply<double>(L, (const double*)L.x, J, I, nullptr);
            w[0] = bv * bv;
            w[1] = rv * rv;
        }
        r[k] = rv;
    }
    if (grid_reduce<2, false>(w, partials, &sc->counter[1])) {
        sc->bb = w[0];
        sc->rr = w[1];
        sc->iter = 0;
        const int zero = w[0] == 0.0;
        sc->converged = zero || w[1] <= sc->tol2 * w[0];
        if (cond) cudaGraphSetConditional(cond, sc->converged ? 0u : 1u);
    }
}

// rz = <r, z>, beta
__global__ void k_ns_rz(NLevel L, const double* __restrict__ r, const double* __restrict__ z,
                        DevScalars* sc, double* partials)
{
    int J, I;
    double w[1] = {0.0};
    if (cell(L, J, I)) {
        const long long k = cidx(L, J, I);
        if (L.m[k]) w[0] = r[k] * z[k];
    }
    if (grid_reduce<1, false>(w, partials, &sc->counter[2])) {
        sc->beta = sc->iter == 0 ? 0.0 : w[0] / sc->rz;
        sc->rz = w[0];
    }
}

// p = z + beta p
__global__ void k_ns_p(NLevel L, const double* __restrict__ z, double* __restrict__ p,
                       const DevScalars* sc)
{
    int J, I;
    if (!cell(L, J, I)) return;
    const long long k = cidx(L, J, I);
    const double beta = sc->beta;
    p[k] = L.m[k] ? (sc->iter == 0 ? z[k] : z[k] + beta * p[k]) : 0.0;
}

// q = A p, <p, q>, alpha
__global__ void k_ns_q(NLevel L, const double* __restrict__ p, double* __restrict__ q,
                       DevScalars* sc, double* partials)
{
    int J, I;
    double w[1] = {0.0};
    if (cell(L, J, I)) {
        const long long k = cidx(L, J, I);
        double qv = 0.0;
        if (L.m[k]) {
            qv = n_apply<double>(L, p, J, I, nullptr);
            w[0] = p[k] * qv;
        }
        q[k] = qv;
    }
    if (grid_reduce<1, false>(w, partials, &sc->counter[3])) {
        sc->pq = w[0];
        sc->alpha = sc->rz / w[0];
    }
}

// x += alpha p, r -= alpha q, <r,r>, convergence, loop condition
__global__ void k_ns_xr(NLevel L, const double* __restrict__ p, const double* __restrict__ q,
                        double* __restrict__ r, DevScalars* sc, double* partials, NGlobals* eg,
                        cudaGraphConditionalHandle cond)
{
    int J, I;
    double w[1] = {0.0};
    const double a = sc->alpha;
    if (cell(L, J, I)) {
        const long long k = cidx(L, J, I);
        if (L.m[k]) {
            ((double*)L.x)[k] += a * p[k];
            const double rv = r[k] - a * q[k];
            r[k] = rv;
            w[0] = rv * rv;
        }
    }
    if (grid_reduce<1, false>(w, partials, &sc->counter[4])) {
        sc->rr = w[0];
        sc->iter += 1;
        sc->total_iters += 1;
        eg->iters += 1;
        const bool bad = !(w[0] == w[0]);
        bool conv = bad || w[0] <= sc->tol2 * sc->bb;
        if (bad) eg->status |= ST_NONFINITE;
        if (!conv && sc->iter >= sc->maxit) {
            eg->status |= ST_PCG_MAXIT;
            conv = true;
        }
        sc->converged = conv;
        if (cond) cudaGraphSetConditional(cond, conv ? 0u : 1u);
    }
}

// x -= mean(x) over the fluid cells (mean = sc->t / nfluid)
__global__ void k_ns_center(NLevel L, const DevScalars* sc, long long nfluid)
{
    int J, I;
    if (!cell(L, J, I)) return;
    const long long k = cidx(L, J, I);
    if (L.m[k]) ((double*)L.x)[k] -= sc->t / (double)nfluid;
}

__global__ void k_ns_setup(DevScalars* sc, double tol2, int maxit)
{
    sc->tol2 = tol2;
    sc->maxit = maxit;
    sc->converged = 0;
    sc->iter = 0;
}

// ---- host ----------------------------------------------------------------------
static dim3 ngrid(const NLevel& L) { return dim3((L.nxn + 31) / 32, (L.nyn + 7) / 8); }
// the cells of one colour: half the columns
static dim3 ngrid_half(const NLevel& L)
{
    return dim3(((L.nxn + 1) / 2 + 31) / 32, (L.nyn + 7) / 8);
}

template <typename S>
static int ns_vcycle_t(NSolver& s, cudaStream_t st)
{
    const dim3 blk(32, 8);
    const int nl = (int)s.lev.size();
    int cnt = 0;
    // level 0 of the cycle: x = z (from zero), b = r
    for (int l = 0; l < nl - 1; ++l) {
        // x = 0 before the pre-smoothing (coarse levels: set by the restriction)
        if (l == 0) k_ns_zero<S><<<ngrid(s.lev[l]), blk, 0, st>>>(s.dlev, l);
        for (int k = 0; k < s.nu; ++k) {
            k_ns_smooth<S><<<ngrid_half(s.lev[l]), blk, 0, st>>>(s.dlev, l, 0);
            k_ns_smooth<S><<<ngrid_half(s.lev[l]), blk, 0, st>>>(s.dlev, l, 1);
        }
        k_ns_restrict<S><<<ngrid(s.lev[l + 1]), blk, 0, st>>>(s.dlev, l);
        cnt += (l == 0 ? 2 : 1) + 2 * s.nu;
    }
    k_ns_coarse<S><<<1, 1024, 0, st>>>(s.dlev, nl - 1, s.ksweeps);
    cnt += 1;
    for (int l = nl - 2; l >= 0; --l) {
        k_ns_prolong<S><<<ngrid(s.lev[l]), blk, 0, st>>>(s.dlev, l);
        for (int k = 0; k < s.nu; ++k) {
            k_ns_smooth<S><<<ngrid_half(s.lev[l]), blk, 0, st>>>(s.dlev, l, 1);
            k_ns_smooth<S><<<ngrid_half(s.lev[l]), blk, 0, st>>>(s.dlev, l, 0);
        }
        cnt += 1 + 2 * s.nu;
    }
    return cnt;
}

// z = M r: the FP64 cycle works on z and r in place; the FP32 cycle on
// FP32 copies (r -> r32, cycle, z32 -> z)
static int ns_vcycle(NSolver& s, cudaStream_t st)
{
    if (s.prec == 0) return ns_vcycle_t<double>(s, st);
    const dim3 blk(32, 8), gr = ngrid(s.prob);
    k_ns_to32<<<gr, blk, 0, st>>>(s.prob, s.r, s.r32);
    const int c = ns_vcycle_t<float>(s, st);
    k_ns_to64<<<gr, blk, 0, st>>>(s.prob, s.z32, s.z);
    return c + 2;
}

static int ns_body(NSolver& s, cudaStream_t st, cudaGraphConditionalHandle cond, int* cnt)
{
    const dim3 blk(32, 8);
    const NLevel& P = s.prob;  // the Krylov level: FP64 couplings, level-0 layout
    NLevel prob = P;           // the problem (x = the pressure)
    prob.x = s.lev_x0;
    const dim3 gr = ngrid(P);
    int c = ns_vcycle(s, st);
    k_ns_rz<<<gr, blk, 0, st>>>(P, s.r, s.z, s.sc, s.partials);
    k_ns_p<<<gr, blk, 0, st>>>(P, s.z, s.p, s.sc);
    k_ns_q<<<gr, blk, 0, st>>>(P, s.p, s.q, s.sc, s.partials);
    k_ns_xr<<<gr, blk, 0, st>>>(prob, s.p, s.q, s.r, s.sc, s.partials, s.eg, cond);
    c += 4;
    if (cnt) *cnt = c;
    return (int)cudaGetLastError();
}

int ns_record(NSolver& s, cudaStream_t st, cudaStream_t st2, bool eager, int* launches)
{
    const dim3 blk(32, 8);
    NLevel prob = s.prob;
    prob.x = s.lev_x0;
    prob.b = s.lev_b0;
    const dim3 gr = ngrid(prob);
    int fixed = 0;
    k_ns_setup<<<1, 1, 0, st>>>(s.sc, s.tol * s.tol, s.maxit);
    k_ns_sum<<<gr, blk, 0, st>>>(prob, (const double*)prob.b, s.sc, s.partials);
    fixed += 2;
    cudaGraphConditionalHandle cond = 0;
    if (!eager) {
        cudaStreamCaptureStatus cs;
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, nullptr, nullptr,
                                                 nullptr);
        if (e != cudaSuccess) return (int)e;
        if (cs != cudaStreamCaptureStatusActive) return 1;
        e = cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return (int)e;
    }
    k_ns_init<<<gr, blk, 0, st>>>(prob, s.r, s.sc, s.partials, s.eg, s.nfluid, cond);
    fixed += 1;
    if (!eager) {
        int r = add_while(st, st2, &cond, 1, [&](cudaStream_t sb) {
            return ns_body(s, sb, cond, nullptr);
        });
        if (r) return r;
    } else {
        for (int it = 0; it <= s.maxit; ++it) {
            DevScalars h;
            if (cudaMemcpyAsync(&h, s.sc, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)
                return 2;
            if (h.converged) break;
            int r = ns_body(s, st, 0, nullptr);
            if (r) return r;
        }
    }
    // zero-mean solution
    k_ns_sum<<<gr, blk, 0, st>>>(prob, (const double*)prob.x, s.sc, s.partials);
    k_ns_center<<<gr, blk, 0, st>>>(prob, s.sc, s.nfluid);
    fixed += 2;
    if (launches) *launches = fixed;
    return (int)cudaGetLastError();
}

int ns_build(NSolver& s, int nyn, int nxn, long long pitch, long long off, int per,
             const uint8_t* hmask, double* x, double* b, double cx, double cy, int prec)
{
    ns_free(s);
    s.prec = prec;
    const size_t es = prec == 0 ? 8 : 4;
    // host couplings in the cycle's precision
    auto conv = [&](const std::vector<double>& v) {
        std::vector<unsigned char> out(v.size() * es);
        for (size_t k = 0; k < v.size(); ++k) {
            if (es == 8) memcpy(&out[k * 8], &v[k], 8);
            else {
                const float f = (float)v[k];
                memcpy(&out[k * 4], &f, 4);
            }
        }
        return out;
    };
    auto dal = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, bytes);
        s.owned.push_back(p);
        return p;
    };
    // level 0 in the model layout; coarse levels dense with 32-element pitch
    std::vector<uint8_t> m((size_t)nyn * nxn);
    long long nf = 0;
    for (int J = 0; J < nyn; ++J)
        for (int I = 0; I < nxn; ++I) {
            m[(size_t)J * nxn + I] = hmask[off + (long long)J * pitch + I] ? 1 : 0;
            nf += m[(size_t)J * nxn + I];
        }
    if (nf == 0) return 6;
    s.nfluid = nf;
    std::vector<double> fx((size_t)nyn * nxn, 0.0), fy((size_t)nyn * nxn, 0.0);
    for (int J = 0; J < nyn; ++J)
        for (int I = 0; I < nxn; ++I) {
            const bool c = m[(size_t)J * nxn + I];
            if (!c) continue;
            if (I > 0 && m[(size_t)J * nxn + I - 1]) fx[(size_t)J * nxn + I] = cx;
            if (I == 0 && per && m[(size_t)J * nxn + nxn - 1]) fx[(size_t)J * nxn] = cx;
            if (J > 0 && m[(size_t)(J - 1) * nxn + I]) fy[(size_t)J * nxn + I] = cy;
        }
    const size_t n0 = (size_t)(off + (long long)nyn * pitch);
    s.r = (double*)dal(n0 * 8);
    s.z = (double*)dal(n0 * 8);
    s.p = (double*)dal(n0 * 8);
    s.q = (double*)dal(n0 * 8);
    double* fx0 = (double*)dal(n0 * 8);
    double* fy0 = (double*)dal(n0 * 8);
    uint8_t* m0 = (uint8_t*)dal(n0);
    if (!s.r || !s.z || !s.p || !s.q || !fx0 || !fy0 || !m0) return 2;
    {
        std::vector<double> hx(n0, 0.0), hy(n0, 0.0);
        std::vector<uint8_t> hm(n0, 0);
        for (int J = 0; J < nyn; ++J)
            for (int I = 0; I < nxn; ++I) {
                const size_t k = (size_t)(off + (long long)J * pitch + I);
                hx[k] = fx[(size_t)J * nxn + I];
                hy[k] = fy[(size_t)J * nxn + I];
                hm[k] = m[(size_t)J * nxn + I];
            }
        if (cudaMemcpy(fx0, hx.data(), n0 * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(fy0, hy.data(), n0 * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(m0, hm.data(), n0, cudaMemcpyHostToDevice) != cudaSuccess)
            return 2;
    }
    NLevel L0;
    memset(&L0, 0, sizeof(L0));
    L0.fx = fx0;
    L0.fy = fy0;
    L0.m = m0;
    L0.nyn = nyn;
    L0.nxn = nxn;
    L0.pitch = pitch;
    L0.off = off;
    L0.per = per;
    s.prob = L0;  // the Krylov level (x, b set per record)
    if (prec == 0) {
        L0.x = s.z;  // the cycle's level 0: x = z, b = r
        L0.b = s.r;
    } else {
        // FP32 cycle: its own x, b and couplings in the level-0 layout
        s.r32 = (float*)dal(n0 * 4);
        s.z32 = (float*)dal(n0 * 4);
        void* f32x = dal(n0 * 4);
        void* f32y = dal(n0 * 4);
        if (!s.r32 || !s.z32 || !f32x || !f32y) return 2;
        std::vector<double> hx(n0, 0.0), hy(n0, 0.0);
        for (int J = 0; J < nyn; ++J)
            for (int I = 0; I < nxn; ++I) {
                const size_t k = (size_t)(off + (long long)J * pitch + I);
                hx[k] = fx[(size_t)J * nxn + I];
                hy[k] = fy[(size_t)J * nxn + I];
            }
        const std::vector<unsigned char> cx4 = conv(hx), cy4 = conv(hy);
        if (cudaMemcpy(f32x, cx4.data(), n0 * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(f32y, cy4.data(), n0 * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return 2;
        L0.x = s.z32;
        L0.b = s.r32;
        L0.fx = f32x;
        L0.fy = f32y;
    }
    s.lev.push_back(L0);
    s.lev_x0 = x;
    s.lev_b0 = b;
    // coarse levels (2x2 agglomerates; Galerkin couplings)
    int ny = nyn, nxc = nxn;
    while (ny > 8 && nxc > 8 && (!per || nxc % 2 == 0) && s.lev.size() < 16) {
        const int cy_n = (ny + 1) / 2, cx_n = (nxc + 1) / 2;
        std::vector<uint8_t> cm((size_t)cy_n * cx_n, 0);
        std::vector<double> cfx((size_t)cy_n * cx_n, 0.0), cfy((size_t)cy_n * cx_n, 0.0);
        for (int J = 0; J < cy_n; ++J)
            for (int I = 0; I < cx_n; ++I) {
                uint8_t v = 0;
                double sx = 0.0, sy = 0.0;
                for (int a = 0; a < 2; ++a)
                    for (int c = 0; c < 2; ++c) {
                        const int fj = 2 * J + a, fi = 2 * I + c;
                        if (fj < ny && fi < nxc) v |= m[(size_t)fj * nxc + fi];
                    }
                // faces crossing the coarse west face: fine x-faces at column 2I
                for (int a = 0; a < 2; ++a) {
                    const int fj = 2 * J + a;
                    if (fj < ny && 2 * I < nxc) sx += fx[(size_t)fj * nxc + 2 * I];
                }
                // faces crossing the coarse south face: fine y-faces at row 2J
                for (int c = 0; c < 2; ++c) {
                    const int fi = 2 * I + c;
                    if (2 * J < ny && fi < nxc) sy += fy[(size_t)(2 * J) * nxc + fi];
                }
                cm[(size_t)J * cx_n + I] = v;
                cfx[(size_t)J * cx_n + I] = 0.5 * sx;
                cfy[(size_t)J * cx_n + I] = 0.5 * sy;
            }
        NLevel C;
        memset(&C, 0, sizeof(C));
        C.nyn = cy_n;
        C.nxn = cx_n;
        C.pitch = (cx_n + 31) / 32 * 32;
        C.off = 0;
        C.per = per;
        const size_t n = (size_t)C.pitch * cy_n;
        void* dx_ = dal(n * es);
        void* db_ = dal(n * es);
        void* dfx = dal(n * es);
        void* dfy = dal(n * es);
        uint8_t* dm = (uint8_t*)dal(n);
        if (!dx_ || !db_ || !dfx || !dfy || !dm) return 2;
        std::vector<double> hx(n, 0.0), hy(n, 0.0);
        std::vector<uint8_t> hm(n, 0);
        for (int J = 0; J < cy_n; ++J)
            for (int I = 0; I < cx_n; ++I) {
                hx[(size_t)J * C.pitch + I] = cfx[(size_t)J * cx_n + I];
                hy[(size_t)J * C.pitch + I] = cfy[(size_t)J * cx_n + I];
                hm[(size_t)J * C.pitch + I] = cm[(size_t)J * cx_n + I];
            }
        const std::vector<unsigned char> hxs = conv(hx), hys = conv(hy);
        if (cudaMemcpy(dfx, hxs.data(), n * es, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dfy, hys.data(), n * es, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dm, hm.data(), n, cudaMemcpyHostToDevice) != cudaSuccess)
            return 2;
        C.x = dx_;
        C.b = db_;
        C.fx = dfx;
        C.fy = dfy;
        C.m = dm;
        s.lev.push_back(C);
        m.swap(cm);
        fx.swap(cfx);
        fy.swap(cfy);
        ny = cy_n;
        nxc = cx_n;
    }
    s.ksweeps = std::min(64, std::max(4, std::max(ny, nxc)));
    s.dlev = (NLevel*)dal(sizeof(NLevel) * s.lev.size());
    s.eg = (NGlobals*)dal(sizeof(NGlobals));
    s.sc = (DevScalars*)dal(sizeof(DevScalars));
    const size_t nb = (size_t)((nxn + 31) / 32) * ((nyn + 7) / 8) + 64;
    s.partials = (double*)dal(nb * 2 * sizeof(double));
    if (!s.dlev || !s.eg || !s.sc || !s.partials) return 2;
    if (cudaMemcpy(s.dlev, s.lev.data(), sizeof(NLevel) * s.lev.size(),
                   cudaMemcpyHostToDevice) != cudaSuccess)
        return 2;
    return 0;
}

void ns_free(NSolver& s)
{
    for (void* p : s.owned) cudaFree(p);
    s.owned.clear();
    s.lev.clear();
    s.dlev = nullptr;
    s.eg = nullptr;
    s.sc = nullptr;
    s.partials = nullptr;
    s.r = s.z = s.p = s.q = nullptr;
    s.r32 = s.z32 = nullptr;
}

}  // namespace f2d
