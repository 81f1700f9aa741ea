// Batched multigrid-preconditioned solver of the masked vertex operator
// (the reference factorises it with SuperLU: elliptic.py:71-87, 114-195).
//
// Operator at a fluid node: A x = cx (xW + xE) + cy (xS + xN) + diag x,
// non-fluid neighbours Dirichlet 0, diag = -2 (cx + cy) - maindiag. Every
// member of the batch has its own multigrid hierarchy (mg.cu: mg_build);
// grid levels are covered by tables of 32x32-node tiles spanning all
// members, the coarse tail runs one block per member, dot products are
// reduced per member with deterministic segmented reductions, and the
// iteration loops are CUDA-graph conditional WHILE nodes that run until every
// member has converged (converged members' blocks return at once).
//
// Two forms:
//  * mode 0 (FP64): preconditioned CG in FP64 with an FP64 V-cycle.
//  * mode 1 (FP32 + FP64 refinement): the outer loop forms the FP64 residual
//    r = b - A x (FP64 matrix-vector product and norms), the inner loop runs
//    CG in FP32 vectors with an FP32 V-cycle (dot products accumulated in
//    FP64) to reduce that residual by tol_in, and x += e in FP64. On GB300,
//    where FP64 arithmetic is scarce, this confines FP64 to one residual per
//    refinement round while the solution reaches FP64 accuracy.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "mg_ops.cuh"
#include "solver.cuh"

namespace f2d {

// node loop of a tile: tl.w rows per thread (a tile is 32 x 8*tl.w nodes)
template <typename F>
__device__ __forceinline__ void tile_nodes(const int4& tl, const MGLevel& L, F f)
{
    for (int r = 0; r < tl.w; ++r) {
        const int J = tl.z + threadIdx.y + 8 * r, I = tl.y + threadIdx.x;
        if (J < L.nyn && I < L.nxn) f(J, I);
    }
}

// per-thread dot-product partial -> what seg_reduce2 expects: FP32 values
// are summed per warp in FP32 and combined in FP64 (block total in thread 0);
// FP64 values go to seg_reduce2's own FP64 block reduction.
template <typename V>
__device__ __forceinline__ void block_dot(V acc, double (&w)[1]);
template <>
__device__ __forceinline__ void block_dot<double>(double acc, double (&w)[1])
{
    w[0] = acc;
}
template <>
__device__ __forceinline__ void block_dot<float>(float acc, double (&w)[1])
{
    const float a[1] = {acc};
    w[0] = 0.0;
    block_total_f<1>(a, w);
}

__device__ __forceinline__ bool bs_skip(const DevScalars& sc, int ir)
{
    return sc.converged || (ir && sc.conv_in);
}

// Completion of a kernel over all members, counted per member: exactly one
// block of every member calls this with mine = true (the last block of its
// segmented reduction, or the first tile of a member whose work is skipped),
// so the global ticket sees n increments, not one per block. True in the
// thread that completes the count.
__device__ __forceinline__ bool members_done(bool mine, unsigned int* ticket, int n)
{
    if (!mine) return false;
    __threadfence();
    if (atomicAdd(ticket, 1u) == (unsigned)n - 1) {
        __threadfence();
        *ticket = 0;
        return true;
    }
    return false;
}

// ---- multigrid --------------------------------------------------------------
template <typename S>
__global__ void __launch_bounds__(256)
k_bs_presmooth(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
               const MGLevel* __restrict__ levs, int l, const DevScalars* __restrict__ scs,
               int ir)
{
    const int4 tl = tiles[blockIdx.x];
    if (info[tl.x].ltail <= l || bs_skip(scs[tl.x], ir)) return;
    const MGLevel L = levs[tl.x * BS_LMAX + l];
    tile_nodes(tl, L, [&](int J, int I) { op_presmooth<S>(L, J, I); });
}

template <typename S>
__global__ void __launch_bounds__(256)
k_bs_restrict(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
              const MGLevel* __restrict__ levs, int l, const DevScalars* __restrict__ scs,
              int ir)
{
    const int4 tl = tiles[blockIdx.x];
    if (info[tl.x].ltail <= l || bs_skip(scs[tl.x], ir)) return;
    const MGLevel F = levs[tl.x * BS_LMAX + l], C = levs[tl.x * BS_LMAX + l + 1];
    tile_nodes(tl, C, [&](int J, int I) { op_restrict<S>(F, C, J, I); });
}

template <typename S>
__global__ void __launch_bounds__(256)
k_bs_prolong(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
             const MGLevel* __restrict__ levs, int l, const DevScalars* __restrict__ scs,
             int ir)
{
    const int4 tl = tiles[blockIdx.x];
    if (info[tl.x].ltail <= l || bs_skip(scs[tl.x], ir)) return;
    const MGLevel F = levs[tl.x * BS_LMAX + l], C = levs[tl.x * BS_LMAX + l + 1];
    tile_nodes(tl, F, [&](int J, int I) { op_prolong<S>(C, F, J, I); });
}

template <typename S>
__global__ void __launch_bounds__(256)
k_bs_smooth(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
            const MGLevel* __restrict__ levs, int l, int color,
            const DevScalars* __restrict__ scs, int ir)
{
    const int4 tl = tiles[blockIdx.x];
    if (info[tl.x].ltail <= l || bs_skip(scs[tl.x], ir)) return;
    const MGLevel L = levs[tl.x * BS_LMAX + l];
    tile_nodes(tl, L, [&](int J, int I) { op_smooth<S>(L, J, I, color, false); });
}

template <typename S>
__global__ void __launch_bounds__(1024)
k_bs_tail(const BSInfo* __restrict__ info, const MGLevel* __restrict__ levs,
          const DevScalars* __restrict__ scs, int ir, int nu)
{
    const int b = blockIdx.x;
    if (bs_skip(scs[b], ir)) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ MGLevel sl[16];
    const BSInfo in = info[b];
    tail_vcycle<S>(&levs[b * BS_LMAX], in.ltail, in.nl, in.ksweeps, smem_raw, sl, nu);
}

// ---- Krylov kernels on level 0 ------------------------------------------------
template <typename V>
__device__ __forceinline__ V applyA(const MGLevel& L, const V* __restrict__ x, int J, int I,
                                    long long k)
{
    return apply_off<V>(L, x, J, I) + Coef<V>::diag(L) * x[k];
}

// rz = <r, z>, beta = rz / rz_old (0 on the first iteration of a loop)
template <typename S, typename V>
__global__ void __launch_bounds__(256)
k_bs_rz(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
        const MGLevel* __restrict__ levs, const V* __restrict__ r, const S* __restrict__ z,
        DevScalars* scs, double* partials, double* gpart, unsigned int* gtick, int ir)
{
    const int4 tl = tiles[blockIdx.x];
    DevScalars& sc = scs[tl.x];
    if (bs_skip(sc, ir)) return;
    const MGLevel L = levs[tl.x * BS_LMAX];
    V acc = V(0);
    tile_nodes(tl, L, [&](int J, int I) {
        const long long k = nidx(L, J, I);
        if (L.m[k]) acc += r[k] * V(z[k]);
    });
    double w[1];
    block_dot<V>(acc, w);
    const BSInfo in = info[tl.x];
    if (seg_reduce2<1, std::is_same<V, float>::value>(w, partials, gpart, gtick, blockIdx.x,
                                                      in.n0, in.nn, in.g0, &sc.counter[2])) {
        const int first = ir ? sc.iter_in == 0 : sc.iter == 0;
        sc.beta = first ? 0.0 : w[0] / sc.rz;
        sc.rz = w[0];
    }
}

// p = z (first iteration) or z + beta p
template <typename S, typename V>
__global__ void __launch_bounds__(256)
k_bs_p(const int4* __restrict__ tiles, const MGLevel* __restrict__ levs,
       const S* __restrict__ z, V* __restrict__ p, const DevScalars* __restrict__ scs, int ir)
{
    const int4 tl = tiles[blockIdx.x];
    const DevScalars& sc = scs[tl.x];
    if (bs_skip(sc, ir)) return;
    const MGLevel L = levs[tl.x * BS_LMAX];
    const int first = ir ? sc.iter_in == 0 : sc.iter == 0;
    const V beta = V(sc.beta);
    tile_nodes(tl, L, [&](int J, int I) {
        const long long k = nidx(L, J, I);
        V v = V(0);
        if (L.m[k]) v = first ? V(z[k]) : V(z[k]) + beta * p[k];
        p[k] = v;
    });
}

// q = A p, pq = <p, q>, alpha = rz / pq
template <typename V>
__global__ void __launch_bounds__(256)
k_bs_spmv(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
          const MGLevel* __restrict__ levs, const V* __restrict__ p, V* __restrict__ q,
          DevScalars* scs, double* partials, double* gpart, unsigned int* gtick, int ir)
{
    const int4 tl = tiles[blockIdx.x];
    DevScalars& sc = scs[tl.x];
    if (bs_skip(sc, ir)) return;
    const MGLevel L = levs[tl.x * BS_LMAX];
    V acc = V(0);
    tile_nodes(tl, L, [&](int J, int I) {
        const long long k = nidx(L, J, I);
        V qv = V(0);
        if (L.m[k]) {
            qv = applyA<V>(L, p, J, I, k);
            acc += p[k] * qv;
        }
        q[k] = qv;
    });
    double w[1];
    block_dot<V>(acc, w);
    const BSInfo in = info[tl.x];
    if (seg_reduce2<1, std::is_same<V, float>::value>(w, partials, gpart, gtick, blockIdx.x,
                                                      in.n0, in.nn, in.g0, &sc.counter[3])) {
        sc.pq = w[0];
        sc.alpha = sc.rz / w[0];
    }
}

// x += alpha p, r -= alpha q, rr = <r, r>, per-member convergence, loop
// condition. FP64 form: x is the solution. Refinement form: x is the inner
// correction e (started from 0) and convergence is relative to the round's
// starting residual.
template <typename V>
__global__ void __launch_bounds__(256)
k_bs_xr(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
        const MGLevel* __restrict__ levs, V* __restrict__ x, V* __restrict__ r,
        const V* __restrict__ p, const V* __restrict__ q, DevScalars* scs, double* partials,
        double* gpart, unsigned int* gtick, BSGlobals* eg, cudaGraphConditionalHandle cond,
        int ir, int nmem)
{
    const int4 tl = tiles[blockIdx.x];
    DevScalars& sc = scs[tl.x];
    bool mine = false;
    if (bs_skip(sc, ir)) {
        mine = threadIdx.x == 0 && threadIdx.y == 0 && (int)blockIdx.x == info[tl.x].n0;
    } else {
        const MGLevel L = levs[tl.x * BS_LMAX];
        const int zero = ir ? 0 : sc.pad1;
        const int first = ir && sc.iter_in == 0;
        const V a = V(sc.alpha);
        V acc = V(0);
        tile_nodes(tl, L, [&](int J, int I) {
            const long long k = nidx(L, J, I);
            if (!L.m[k]) return;
            if (zero) {
                x[k] = V(0);
                r[k] = V(0);
                return;
            }
            x[k] = (first ? V(0) : x[k]) + a * p[k];
            const V rv = r[k] - a * q[k];
            r[k] = rv;
            acc += rv * rv;
        });
        double w[1];
        block_dot<V>(acc, w);
        const BSInfo in = info[tl.x];
        mine = seg_reduce2<1, std::is_same<V, float>::value>(w, partials, gpart, gtick,
                                                             blockIdx.x, in.n0, in.nn, in.g0,
                                                             &sc.counter[4]);
        if (mine) {
            sc.total_iters += 1;
            const bool bad = !(w[0] == w[0]);
            if (bad) atomicOr(&eg->status, ST_NONFINITE);
            if (ir) {
                sc.iter_in += 1;
                const int done = bad || w[0] <= sc.tol_in2 * sc.rr0 || sc.iter_in >= sc.maxit_in;
                if (done) {
                    sc.conv_in = 1;
                    atomicSub(&eg->active_in, 1);
                }
            } else {
                sc.rr = w[0];
                sc.iter += 1;
                const int conv = bad || zero || (w[0] <= sc.tol2 * sc.bb);
                sc.pad1 = 0;
                const int more = !conv && sc.iter < sc.maxit;
                if (!conv && !more) atomicOr(&eg->status, ST_PCG_MAXIT);
                if (!more) {
                    sc.converged = 1;
                    atomicSub(&eg->active_out, 1);
                }
            }
        }
    }
    if (members_done(mine, &eg->ticket[1], nmem)) {
        eg->loops_in += 1;
        const int act = ir ? *(volatile int*)&eg->active_in : *(volatile int*)&eg->active_out;
        if (cond) cudaGraphSetConditional(cond, act > 0 ? 1u : 0u);
    }
}

// FP64 form: r = b - A x, <b,b>, <r,r>, per-member start state
__global__ void __launch_bounds__(256)
k_bs_init(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
          const MGLevel* __restrict__ levs, const double* __restrict__ x,
          const double* __restrict__ b, double* __restrict__ r, DevScalars* scs,
          double* partials, double* gpart, unsigned int* gtick, BSGlobals* eg,
          cudaGraphConditionalHandle cond, int nmem)
{
    const int4 tl = tiles[blockIdx.x];
    DevScalars& sc = scs[tl.x];
    const MGLevel L = levs[tl.x * BS_LMAX];
    double w[2] = {0.0, 0.0};
    tile_nodes(tl, L, [&](int J, int I) {
        const long long k = nidx(L, J, I);
        double rv = 0.0;
        if (L.m[k]) {
            const double bv = b[k];
            rv = bv - applyA<double>(L, x, J, I, k);
            w[0] += bv * bv;
            w[1] += rv * rv;
        }
        r[k] = rv;
    });
    const BSInfo in = info[tl.x];
    const bool mine = seg_reduce2<2>(w, partials, gpart, gtick, blockIdx.x, in.n0, in.nn, in.g0, &sc.counter[1]);
    if (mine) {
        sc.bb = w[0];
        sc.rr = w[1];
        sc.iter = 0;
        const int zero = (w[0] == 0.0);
        sc.converged = zero ? 0 : (w[1] <= sc.tol2 * w[0]);
        sc.pad1 = zero;
        if (!sc.converged) atomicAdd(&eg->active_out, 1);
    }
    if (members_done(mine, &eg->ticket[0], nmem)) {
        eg->loops_out += 1;
        if (cond) cudaGraphSetConditional(cond, *(volatile int*)&eg->active_out > 0 ? 1u : 0u);
    }
}

// Refinement form: r64 = b - A x (FP64), the FP32 copy that drives the next
// inner solve, <b,b> and <r,r>; per member: converged, or start a new round.
__global__ void __launch_bounds__(256)
k_bs_refine(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
            const MGLevel* __restrict__ levs, const double* __restrict__ x,
            const double* __restrict__ b, double* __restrict__ r, float* __restrict__ rin,
            DevScalars* scs, double* partials, double* gpart, unsigned int* gtick,
            BSGlobals* eg, int first, cudaGraphConditionalHandle cond, int nmem)
{
    const int4 tl = tiles[blockIdx.x];
    DevScalars& sc = scs[tl.x];
    bool mine = false;
    if (sc.converged) {
        mine = threadIdx.x == 0 && threadIdx.y == 0 && (int)blockIdx.x == info[tl.x].n0;
    } else {
        const MGLevel L = levs[tl.x * BS_LMAX];
        double w[2] = {0.0, 0.0};
        tile_nodes(tl, L, [&](int J, int I) {
            const long long k = nidx(L, J, I);
            double rv = 0.0;
            if (L.m[k]) {
                const double bv = b[k];
                rv = bv - applyA<double>(L, x, J, I, k);
                w[0] += bv * bv;
                w[1] += rv * rv;
            }
            r[k] = rv;
            rin[k] = float(rv);
        });
        const BSInfo in = info[tl.x];
        mine = seg_reduce2<2>(w, partials, gpart, gtick, blockIdx.x, in.n0, in.nn, in.g0, &sc.counter[1]);
        if (mine) {
            const double rr_prev = sc.rr;
            sc.bb = w[0];
            sc.rr = w[1];
            const int zero = (w[0] == 0.0);
            sc.zero = zero;
            int conv = zero ? (w[1] == 0.0) : (w[1] <= sc.tol2 * w[0]);
            // the FP64 residual of a round cannot fall below its rounding
            // floor (about eps * cond(A) relative); a round that no longer
            // reduces it by 10x has reached that floor
            if (!first && !conv && w[1] > 0.01 * rr_prev) conv = 1;
            if (!(w[1] == w[1])) {
                conv = 1;
                atomicOr(&eg->status, ST_NONFINITE);
            }
            if (!first) {
                sc.outer += 1;
                sc.total_outer += 1;
            }
            if (!conv && sc.outer >= sc.maxouter) {
                conv = 1;
                atomicOr(&eg->status, ST_PCG_MAXIT);
            }
            sc.converged = conv;
            if (!conv) {
                atomicAdd(&eg->active_out, 1);
                sc.iter_in = 0;
                sc.rr0 = w[1];
                sc.conv_in = zero ? 1 : 0;
                if (!zero) atomicAdd(&eg->active_in, 1);
            }
        }
    }
    if (members_done(mine, &eg->ticket[0], nmem)) {
        eg->loops_out += 1;
        if (cond) cudaGraphSetConditional(cond, *(volatile int*)&eg->active_out > 0 ? 1u : 0u);
    }
}

// x += e (FP64); a member with a zero right-hand side gets x = 0
__global__ void __launch_bounds__(256)
k_bs_correct(const int4* __restrict__ tiles, const MGLevel* __restrict__ levs,
             double* __restrict__ x, const float* __restrict__ e,
             const DevScalars* __restrict__ scs)
{
    const int4 tl = tiles[blockIdx.x];
    const DevScalars& sc = scs[tl.x];
    if (sc.converged) return;
    const MGLevel L = levs[tl.x * BS_LMAX];
    const int zero = sc.zero;
    tile_nodes(tl, L, [&](int J, int I) {
        const long long k = nidx(L, J, I);
        if (L.m[k]) x[k] = zero ? 0.0 : x[k] + (double)e[k];
    });
}

__global__ void k_bs_setup(DevScalars* scs, int n, double tol2, int maxit, double tol_in2,
                           int maxit_in, int maxouter, BSGlobals* eg)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b == 0) {
        eg->active_out = 0;
        eg->active_in = 0;
        for (int k = 0; k < 4; ++k) eg->ticket[k] = 0;
    }
    if (b < n) {
        DevScalars& s = scs[b];
        s.tol2 = tol2;
        s.maxit = maxit;
        s.tol_in2 = tol_in2;
        s.maxit_in = maxit_in;
        s.maxouter = maxouter;
        s.converged = 0;
        s.conv_in = 0;
        s.iter = 0;
        s.iter_in = 0;
        s.outer = 0;
        s.pad1 = 0;
        s.zero = 0;
    }
}

__global__ void k_bs_reset(BSGlobals* eg)
{
    eg->active_out = 0;
    eg->active_in = 0;
}

__global__ void k_bs_arm(const BSGlobals* eg, cudaGraphConditionalHandle cond)
{
    cudaGraphSetConditional(cond, *(volatile const int*)&eg->active_in > 0 ? 1u : 0u);
}

// ---- host side -----------------------------------------------------------------
static bool bs_eager()
{
    static int v = -1;
    if (v < 0) {
        const char* x = getenv("F2D_EAGER");
        v = (x && *x && *x != '0') ? 1 : 0;
    }
    return v == 1;
}

// one V-cycle for all members still iterating
template <typename S>
static int vcycle(BatchSolver& s, cudaStream_t st, int ir)
{
    const dim3 blk(32, 8);
    int cnt = 0;
    for (int l = 0; l < s.maxl; ++l) {
        k_bs_presmooth<S><<<s.ntiles[l], blk, 0, st>>>(s.tiles[l], s.dinfo, s.dlevs, l, s.scs, ir);
        for (int k = 1; k < s.nu; ++k) {
            k_bs_smooth<S><<<s.ntiles[l], blk, 0, st>>>(s.tiles[l], s.dinfo, s.dlevs, l, 0, s.scs, ir);
            k_bs_smooth<S><<<s.ntiles[l], blk, 0, st>>>(s.tiles[l], s.dinfo, s.dlevs, l, 1, s.scs, ir);
        }
        k_bs_restrict<S><<<s.ntiles[l + 1], blk, 0, st>>>(s.tiles[l + 1], s.dinfo, s.dlevs, l,
                                                          s.scs, ir);
        cnt += 2 + 2 * (s.nu - 1);
    }
    k_bs_tail<S><<<s.n, 1024, s.tail_smem, st>>>(s.dinfo, s.dlevs, s.scs, ir, s.nu);
    cnt += 1;
    for (int l = s.maxl - 1; l >= 0; --l) {
        k_bs_prolong<S><<<s.ntiles[l], blk, 0, st>>>(s.tiles[l], s.dinfo, s.dlevs, l, s.scs, ir);
        for (int k = 0; k < s.nu; ++k) {
            k_bs_smooth<S><<<s.ntiles[l], blk, 0, st>>>(s.tiles[l], s.dinfo, s.dlevs, l, 1, s.scs, ir);
            k_bs_smooth<S><<<s.ntiles[l], blk, 0, st>>>(s.tiles[l], s.dinfo, s.dlevs, l, 0, s.scs, ir);
        }
        cnt += 1 + 2 * s.nu;
    }
    return cnt;
}

// the CG loop body; FP64 form (S = V = double) or the inner FP32 loop
template <typename S, typename V>
static int cg_body(BatchSolver& s, cudaStream_t st, cudaGraphConditionalHandle cond, int ir)
{
    const dim3 blk(32, 8);
    const int nt = s.nrtiles;
    V* r = (V*)(ir ? s.v.rin : s.v.r64);
    V* x = (V*)(ir ? s.v.e : s.v.x64);
    int cnt = vcycle<S>(s, st, ir);
    k_bs_rz<S, V><<<nt, blk, 0, st>>>(s.rtiles, s.dinfo, s.dlevs, r, (const S*)s.v.z, s.scs,
                                      s.partials, s.gpart, s.gtick, ir);
    k_bs_p<S, V><<<nt, blk, 0, st>>>(s.rtiles, s.dlevs, (const S*)s.v.z, (V*)s.v.p, s.scs, ir);
    k_bs_spmv<V><<<nt, blk, 0, st>>>(s.rtiles, s.dinfo, s.dlevs, (const V*)s.v.p, (V*)s.v.q,
                                     s.scs, s.partials, s.gpart, s.gtick, ir);
    k_bs_xr<V><<<nt, blk, 0, st>>>(s.rtiles, s.dinfo, s.dlevs, x, r, (const V*)s.v.p,
                                   (const V*)s.v.q, s.scs, s.partials, s.gpart, s.gtick, s.eg, cond, ir,
                                   s.n);
    cnt += 4;
    s.body_launches = cnt;
    return (int)cudaGetLastError();
}

// add a WHILE node at the current capture position of `st` and capture its
// body with `rec(stream)` on `sb`
template <typename R>
static int add_while(cudaStream_t st, cudaStream_t sb, cudaGraphConditionalHandle* cond,
                     unsigned dflt, R rec)
{
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return (int)e;
    if (!*cond) {
        e = cudaGraphConditionalHandleCreate(cond, graph, dflt, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return (int)e;
    }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = *cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp);
    if (e != cudaSuccess) return (int)e;
    e = cudaStreamBeginCaptureToGraph(sb, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return (int)e;
    int r = rec(sb);
    cudaGraph_t out;
    e = cudaStreamEndCapture(sb, &out);
    if (r) return r;
    if (e != cudaSuccess) return (int)e;
    return (int)cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                                    cudaStreamSetCaptureDependencies);
}

static int read_globals(const BatchSolver& s, cudaStream_t st, BSGlobals* h)
{
    cudaError_t e = cudaMemcpyAsync(h, s.eg, sizeof(*h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return (int)e;
}

static cudaStream_t g_third = nullptr;  // body stream of nested loops

int bs_record(BatchSolver& s, cudaStream_t st, cudaStream_t st2, int* launches)
{
    const dim3 blk(32, 8);
    const int nt = s.nrtiles;
    int fixed = 0;
    k_bs_setup<<<(s.n + 127) / 128, 128, 0, st>>>(s.scs, s.n, s.tol * s.tol, s.maxit,
                                                   s.tol_in * s.tol_in, s.maxit_in, s.maxouter,
                                                   s.eg);
    fixed += 1;
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, nullptr, nullptr, nullptr);
    if (e != cudaSuccess) return (int)e;
    const bool capturing = cs == cudaStreamCaptureStatusActive && !bs_eager();
    if (cs == cudaStreamCaptureStatusActive && bs_eager()) return 1;  // not mixed
    BSGlobals h;
    if (s.mode == 0) {
        cudaGraphConditionalHandle cond = 0;
        if (capturing) {
            e = cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault);
            if (e != cudaSuccess) return (int)e;
        }
        k_bs_init<<<nt, blk, 0, st>>>(s.rtiles, s.dinfo, s.dlevs, (const double*)s.v.x64,
                                      (const double*)s.v.b64, (double*)s.v.r64, s.scs,
                                      s.partials, s.gpart, s.gtick, s.eg, cond, s.n);
        fixed += 1;
        if (capturing) {
            int r = add_while(st, st2, &cond, 1, [&](cudaStream_t sb) {
                return cg_body<double, double>(s, sb, cond, 0);
            });
            if (r) return r;
        } else {
            for (int it = 0; it <= s.maxit; ++it) {
                int r = read_globals(s, st, &h);
                if (r) return r;
                if (h.active_out <= 0) break;
                r = cg_body<double, double>(s, st, 0, 0);
                if (r) return r;
            }
        }
        if (launches) *launches = fixed;
        return (int)cudaGetLastError();
    }
    // refinement form
    if (!g_third) {
        e = cudaStreamCreateWithFlags(&g_third, cudaStreamNonBlocking);
        if (e != cudaSuccess) return (int)e;
    }
    cudaGraphConditionalHandle cond_o = 0;
    if (capturing) {
        e = cudaGraphConditionalHandleCreate(&cond_o, graph, 1, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return (int)e;
    }
    k_bs_reset<<<1, 1, 0, st>>>(s.eg);
    k_bs_refine<<<nt, blk, 0, st>>>(s.rtiles, s.dinfo, s.dlevs, (const double*)s.v.x64,
                                    (const double*)s.v.b64, (double*)s.v.r64, (float*)s.v.rin,
                                    s.scs, s.partials, s.gpart, s.gtick, s.eg, 1, cond_o,
                                    s.n);
    fixed += 2;
    auto round_tail = [&](cudaStream_t sb) {
        k_bs_correct<<<nt, blk, 0, sb>>>(s.rtiles, s.dlevs, (double*)s.v.x64,
                                         (const float*)s.v.e, s.scs);
        k_bs_reset<<<1, 1, 0, sb>>>(s.eg);
        k_bs_refine<<<nt, blk, 0, sb>>>(s.rtiles, s.dinfo, s.dlevs, (const double*)s.v.x64,
                                        (const double*)s.v.b64, (double*)s.v.r64,
                                        (float*)s.v.rin, s.scs, s.partials, s.gpart, s.gtick,
                                        s.eg, 0, cond_o, s.n);
    };
    if (capturing) {
        int r = add_while(st, st2, &cond_o, 1, [&](cudaStream_t sb) {
            cudaGraphConditionalHandle cond_i = 0;
            // the inner condition is re-armed at the top of every round
            cudaStreamCaptureStatus cs2;
            cudaGraph_t g2 = nullptr;
            cudaError_t e2 = cudaStreamGetCaptureInfo(sb, &cs2, nullptr, &g2, nullptr, nullptr,
                                                      nullptr);
            if (e2 != cudaSuccess) return (int)e2;
            e2 = cudaGraphConditionalHandleCreate(&cond_i, g2, 0, 0);
            if (e2 != cudaSuccess) return (int)e2;
            k_bs_arm<<<1, 1, 0, sb>>>(s.eg, cond_i);
            int r2 = add_while(sb, g_third, &cond_i, 0, [&](cudaStream_t sc3) {
                return cg_body<float, float>(s, sc3, cond_i, 1);
            });
            if (r2) return r2;
            round_tail(sb);
            return (int)cudaGetLastError();
        });
        if (r) return r;
    } else {
        for (int round = 0; round <= s.maxouter; ++round) {
            int r = read_globals(s, st, &h);
            if (r) return r;
            if (h.active_out <= 0) break;
            for (int it = 0; it <= s.maxit_in; ++it) {
                r = read_globals(s, st, &h);
                if (r) return r;
                if (h.active_in <= 0) break;
                r = cg_body<float, float>(s, st, 0, 1);
                if (r) return r;
            }
            round_tail(st);
        }
    }
    if (launches) *launches = fixed;
    return (int)cudaGetLastError();
}

int bs_build(BatchSolver& s, const std::vector<BSMemberDesc>& members, const uint8_t* dmask,
             int mode, const BSVecs& v, DevScalars* scs)
{
    bs_free(s);
    s.n = (int)members.size();
    s.mode = mode;
    s.v = v;
    s.scs = scs;
    s.mg.resize(s.n);
    std::vector<MGLevel> levs((size_t)s.n * BS_LMAX);
    std::vector<BSInfo> info(s.n);
    s.maxl = 0;
    s.tail_smem = 0;
    for (int b = 0; b < s.n; ++b) {
        const BSMemberDesc& d = members[b];
        // level 0 of the multigrid: x = z, b = the residual driving the cycle
        void* r0 = mode == 0 ? v.r64 : v.rin;
        int e = mg_build(s.mg[b], d.nyn, d.nxn, d.pitch, d.off0, d.per, d.hmask, d.hoff0, dmask,
                         v.z, r0, d.cx, d.cy, d.maindiag, mode == 0 ? 0 : 1);
        if (e) return e;
        const int nl = (int)s.mg[b].lev.size();
        if (nl > BS_LMAX) return 5;
        memset(&info[b], 0, sizeof(BSInfo));
        info[b].nl = nl;
        info[b].ltail = s.mg[b].ltail;
        info[b].ksweeps = s.mg[b].ncoarse_sweeps;
        s.maxl = std::max(s.maxl, info[b].ltail);
        s.tail_smem = std::max(s.tail_smem, s.mg[b].tail_smem);
        for (int l = 0; l < nl; ++l) levs[(size_t)b * BS_LMAX + l] = s.mg[b].lev[l];
    }
    // Tiles of 32 x 8R nodes (R rows per thread): R = 4 when a level holds
    // enough nodes to fill the GPU several times over (fewer, fuller blocks),
    // R = 1 otherwise (more blocks for small levels).
    std::vector<std::vector<int4>> tiles(s.maxl + 1);
    for (int l = 0; l <= s.maxl; ++l) {
        long long nodes = 0;
        for (int b = 0; b < s.n; ++b)
            if (l <= info[b].ltail)
                nodes += (long long)levs[(size_t)b * BS_LMAX + l].nyn *
                         levs[(size_t)b * BS_LMAX + l].nxn;
        const int R = nodes >= 4ll * 1024 * 1024 ? 4 : 1;
        for (int b = 0; b < s.n; ++b) {
            if (l > info[b].ltail) continue;
            const MGLevel& L = levs[(size_t)b * BS_LMAX + l];
            for (int J0 = 0; J0 < L.nyn; J0 += 8 * R)
                for (int I0 = 0; I0 < L.nxn; I0 += BS_TW) tiles[l].push_back(make_int4(b, I0, J0, R));
        }
    }
    // Level-0 tiles of the Krylov kernels (32 x 8 nodes), with the member's
    // reduction groups of 64 tiles.
    std::vector<int4> rt;
    int ngroups = 0;
    for (int b = 0; b < s.n; ++b) {
        const MGLevel& L = levs[(size_t)b * BS_LMAX];
        const long long cols = (L.nxn + BS_TW - 1) / BS_TW;
        const long long rows8 = (L.nyn + 7) / 8;
        const int R = 1;
        (void)cols;
        (void)rows8;
        info[b].n0 = (int)rt.size();
        for (int J0 = 0; J0 < L.nyn; J0 += 8 * R)
            for (int I0 = 0; I0 < L.nxn; I0 += BS_TW) rt.push_back(make_int4(b, I0, J0, R));
        info[b].nn = (int)rt.size() - info[b].n0;
        info[b].g0 = ngroups;
        ngroups += (info[b].nn + RED_GROUP - 1) / RED_GROUP;
    }
    auto dal = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        s.owned.push_back(p);
        return p;
    };
    s.tiles.assign(s.maxl + 1, nullptr);
    s.ntiles.assign(s.maxl + 1, 0);
    for (int l = 0; l <= s.maxl; ++l) {
        s.ntiles[l] = (int)tiles[l].size();
        s.tiles[l] = (int4*)dal(std::max<size_t>(1, tiles[l].size()) * sizeof(int4));
        if (!s.tiles[l]) return 2;
        if (cudaMemcpy(s.tiles[l], tiles[l].data(), tiles[l].size() * sizeof(int4),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return 2;
    }
    s.nrtiles = (int)rt.size();
    s.rtiles = (int4*)dal(rt.size() * sizeof(int4));
    if (!s.rtiles ||
        cudaMemcpy(s.rtiles, rt.data(), rt.size() * sizeof(int4), cudaMemcpyHostToDevice) !=
            cudaSuccess)
        return 2;
    s.dlevs = (MGLevel*)dal(levs.size() * sizeof(MGLevel));
    s.dinfo = (BSInfo*)dal(info.size() * sizeof(BSInfo));
    s.eg = (BSGlobals*)dal(sizeof(BSGlobals));
    s.partials = (double*)dal((rt.size() * 2 + 64) * sizeof(double));
    s.gpart = (double*)dal(((size_t)ngroups * 2 + 64) * sizeof(double));
    s.gtick = (unsigned int*)dal(((size_t)ngroups + 64) * sizeof(unsigned int));
    if (!s.gpart || !s.gtick ||
        cudaMemset(s.gtick, 0, ((size_t)ngroups + 64) * sizeof(unsigned int)) != cudaSuccess)
        return 2;
    if (!s.dlevs || !s.dinfo || !s.eg || !s.partials) return 2;
    if (cudaMemcpy(s.dlevs, levs.data(), levs.size() * sizeof(MGLevel), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(s.dinfo, info.data(), info.size() * sizeof(BSInfo), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemset(s.eg, 0, sizeof(BSGlobals)) != cudaSuccess)
        return 2;
    cudaError_t fe = mode == 0
        ? cudaFuncSetAttribute(k_bs_tail<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)s.tail_smem)
        : cudaFuncSetAttribute(k_bs_tail<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)s.tail_smem);
    if (fe != cudaSuccess) return 4;
    return 0;
}

void bs_free(BatchSolver& s)
{
    for (auto& m : s.mg) mg_free(m);
    s.mg.clear();
    for (void* p : s.owned) cudaFree(p);
    s.owned.clear();
    s.tiles.clear();
    s.ntiles.clear();
    s.dlevs = nullptr;
    s.dinfo = nullptr;
    s.eg = nullptr;
    s.partials = nullptr;
}

}  // namespace f2d
