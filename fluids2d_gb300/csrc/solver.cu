// Batched multigrid-preconditioned solver of the masked vertex operator
// (the reference factorises it with SuperLU: elliptic.py:71-87, 114-195).
//
// Operator at a fluid node: A x = cx (xW + xE) + cy (xS + xN) + diag x,
// non-fluid neighbours Dirichlet 0, diag = -2 (cx + cy) - maindiag. Every
// member of the batch has its own multigrid hierarchy (mg.cu: mg_build);
// tile tables spanning all members cover the grid levels (the level kernels:
// 54x70-node tiles; the Krylov kernels on level 0: 32 columns x 32 or 64
// rows), the coarse tail runs one block per member, dot products are reduced
// per member deterministically (per-tile totals summed in a fixed order by
// one block per member), and the iteration loops are CUDA-graph conditional
// WHILE nodes that run until every member has converged (converged members'
// tiles are skipped).
//
// Two forms:
//  * mode 0 (FP64): preconditioned CG in FP64 with an FP64 V-cycle.
//  * mode 1 (FP32 + FP64 refinement): the outer loop forms the FP64 residual
//    r = b - A x (FP64 matrix-vector product and norms), the inner loop runs
//    CG in FP32 vectors with an FP32 V-cycle (dot products accumulated in
//    FP64) to reduce that residual by tol_in, and x += e in FP64. On GB300,
//    where FP64 arithmetic is scarce, this confines FP64 to one residual per
//    refinement round while the solution reaches FP64 accuracy.
#include <cudaTypedefs.h>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "graph_while.cuh"
#include "mg_ops.cuh"
#include "solver.cuh"

namespace f2d {

// ---- tiles staged in shared memory ---------------------------------------------
// Grid kernels work on tiles of 32 x 64 nodes (columns x rows) of one level of
// one member (the int4 of a tile table: member, first column, first row,
// unused), run by 32 x 8 threads; thread (tx, ty) owns tile rows ty + 8 q,
// q = 0..7. A kernel that needs neighbours stages the tile and a halo of H
// nodes in shared memory (rows J0-H .. J0+63+H, columns I0-H .. I0+31+H); nodes
// outside the level read as non-fluid 0, and x-periodic levels wrap. Each
// node is then loaded once per kernel with coalesced rows, all loads of a
// thread in flight together, and the red-black sweeps of a V-cycle level run
// on the staged region: a half sweep on nodes at distance >= s from the
// region edge only needs the region, so the smoothing, residual and transfer
// steps of a level fuse into one kernel with a halo as wide as the chain.
// staged region of halo H around a tile of TH rows: WX columns, WY rows
template <int H, int TH> struct Reg {
    static constexpr int WX = BS_TW + 2 * H, WY = TH + 2 * H, N = WX * WY;
};

__device__ __forceinline__ int tid256() { return threadIdx.y * 32 + threadIdx.x; }

// wrap (J, I) into the level; false outside it
__device__ __forceinline__ bool in_level(const MGLevel& L, int J, int& I)
{
    if (J < 0 || J >= L.nyn) return false;
    if (I < 0) {
        if (!L.per) return false;
        I += L.nxn;
    } else if (I >= L.nxn) {
        if (!L.per) return false;
        I -= L.nxn;
    }
    return I >= 0 && I < L.nxn;
}

// Stage mask and up to two arrays of a level on the region of halo H around
// the tile at (J0, I0). Values at non-fluid nodes are staged as 0.
template <int H, int TH, typename S, typename T2>
__device__ __forceinline__ void stage_region(const MGLevel& L, int J0, int I0,
                                             const S* __restrict__ ga, S* sa,
                                             const T2* __restrict__ gb, T2* sb, uint8_t* sm)
{
    constexpr int W = Reg<H, TH>::WX, N = Reg<H, TH>::N, IT = (N + 255) / 256;
    const int t = tid256();
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int e = t + it * 256;
        if (e < N) {
            const int r = e / W, c = e - r * W;
            const int J = J0 - H + r;
            int I = I0 - H + c;
            uint8_t mv = 0;
            S av = S(0);
            T2 bv = T2(0);
            if (in_level(L, J, I)) {
                const long long k = nidx(L, J, I);
                mv = L.m[k];
                if (ga) av = ga[k];
                if (gb) bv = gb[k];
            }
            sm[e] = mv;
            if (sa) sa[e] = mv ? av : S(0);
            if (sb) sb[e] = mv ? bv : T2(0);
        }
    }
}

__device__ __forceinline__ bool bs_skip(const DevScalars& sc, int ir)
{
    return sc.converged || (ir && sc.conv_in);
}

// Block total of per-thread values in thread 0 (FP32: warp sums in FP32,
// combined in FP64; FP64: block_reduce), fixed order.
template <typename V>
__device__ __forceinline__ double block_sum(V acc)
{
    double w[1];
    if constexpr (std::is_same<V, float>::value) {
        const float a[1] = {acc};
        block_total_f<1>(a, w);
    } else {
        __shared__ double sh[32];
        w[0] = acc;
        block_reduce<1, false>(w, sh);
    }
    return w[0];
}

// Completion of a kernel over all members, counted per member: the kernels
// that call it run one block per member, whose thread 0 calls it with
// mine = true, so the global ticket sees n increments. True in the thread
// that completes the count.
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

// rz = <r, z> of a member, beta = rz / rz_old (0 on the first iteration of
// a loop); run by the thread that holds the member's total
__device__ __forceinline__ void set_rz(DevScalars& sc, int ir, double rz)
{
    const int first = ir ? sc.iter_in == 0 : sc.iter == 0;
    sc.beta = first ? 0.0 : rz / sc.rz;
    sc.rz = rz;
}

// <r, z> of every member from the tile totals of the level-0 up leg
// (tpart[mn0 .. mn0 + mnn), summed in a fixed order), then rz and beta. The
// up leg writes one total per tile and no more, so its blocks never wait on
// a fence or a ticket; members whose level 0 is in the tail (mnn = 0) get
// theirs from k_bs_tail.
__global__ void __launch_bounds__(256)
k_bs_rz(const BSInfo* __restrict__ info, DevScalars* scs, const double* __restrict__ tpart,
        int ir)
{
    pdl_wait();
    const int b = blockIdx.x;
    const BSInfo in = info[b];
    DevScalars& sc = scs[b];
    if (in.mnn == 0 || bs_skip(sc, ir)) return;
    double acc[1] = {0.0};
    final_sum<1, false>(acc, tpart, in.mn0, in.mnn, threadIdx.x, blockDim.x);
    __shared__ double sh[32];
    block_reduce<1, false>(acc, sh);
    if (threadIdx.x == 0) set_rz(sc, ir, acc[0]);
}

// ---- multigrid level kernels (register-blocked; mg_reg.cuh) ----------------
}  // namespace f2d
#include "mg_reg.cuh"
#include "mg_pipe.cuh"
namespace f2d {

// Coarse levels of every member in one block each (tail_vcycle). A member
// whose level 0 is already in the tail also forms <r, z> here.
template <typename S>
__global__ void __launch_bounds__(1024)
k_bs_tail(const BSInfo* __restrict__ info, const MGLevel* __restrict__ levs, DevScalars* scs,
          int ir, int nu)
{
    pdl_wait();
    const int b = blockIdx.x;
    DevScalars& sc = scs[b];
    if (bs_skip(sc, ir)) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ TailLev<S> sl[16];
    const BSInfo in = info[b];
    tail_vcycle<S>(&levs[b * BS_LMAX], in.ltail, in.nl, in.ksweeps, smem_raw, sl, nu);
    if (in.ltail != 0) return;
    const TailLev<S>& D = sl[0];
    const int n = (D.nyn + 2) * D.P;
    S acc = S(0);
    for (int e = threadIdx.x; e < n; e += blockDim.x)
        if (D.m[e]) acc += D.b[e] * D.x[e];  // border: mask 0
    double w[1];
    if constexpr (std::is_same<S, float>::value) {
        const float a[1] = {acc};
        block_total_f<1>(a, w);
    } else {
        __shared__ double sh[32];
        w[0] = acc;
        block_reduce<1, false>(w, sh);
    }
    if (threadIdx.x == 0) set_rz(sc, ir, w[0]);
}

// ---- Krylov kernels on level 0 ------------------------------------------------
// p = z (first iteration) or z + beta p_old, q = A p, the tile's part of
// <p, q> (k_bs_alpha forms alpha = rz / <p, q>). p is formed on the tile and
// a one-node halo (the halo redundantly, from z and p_old), so A p needs no
// second pass; p_old and p live in two buffers chosen by the parity of the
// member's iteration count, or in the refinement form's direction ring (p_old
// of the halo belongs to other blocks and must not be overwritten meanwhile).
template <typename S, typename V, int TH>
__device__ __forceinline__ void pq_tile(const int4& tl, int tix, const MGLevel* __restrict__ levs,
                                        const S* __restrict__ z, V* __restrict__ p0,
                                        V* __restrict__ p1, V* __restrict__ q,
                                        const DevScalars* __restrict__ scs, double* partials,
                                        int ir, V* ring, long long rstride)
{
    constexpr int H = 1, W = Reg<H, TH>::WX, N = Reg<H, TH>::N, IT = (N + 255) / 256;
    constexpr int TQ = TH / 8;
    __shared__ V sp[N];
    __shared__ uint8_t sm[N];
    const DevScalars& sc = scs[tl.x];
    if (bs_skip(sc, ir)) return;
    const MGLevel L = levs[tl.x * BS_LMAX];
    const int it = ir ? sc.iter_in : sc.iter;
    const bool first = it == 0;
    // the direction ring (refinement form: p_it into slot it) or the two
    // buffers alternating with the iteration's parity (FP64 form)
    const V* __restrict__ pold =
        ring ? ring + (long long)max(it - 1, 0) * rstride : ((it & 1) ? p1 : p0);
    V* __restrict__ pnew = ring ? ring + (long long)it * rstride : ((it & 1) ? p0 : p1);
    const V beta = V(sc.beta);
    const int I0 = tl.y, J0 = tl.z, t = tid256();
    // the region in batches of PB elements per thread: the loads of a batch
    // (index of a node outside the level clamped to node (0, 0), its values
    // dropped after) are in flight together before any shared-memory write
    constexpr int PB = 3;
#pragma unroll
    for (int k0 = 0; k0 < IT; k0 += PB) {
        bool ok[PB];
        uint8_t mv[PB];
        S zv[PB];
        V pv[PB];
#pragma unroll
        for (int u = 0; u < PB; ++u) {
            const int e = t + (k0 + u) * 256;
            const int r = e / W, c = e - r * W;
            const int J = J0 - H + r;
            int I = I0 - H + c;
            ok[u] = k0 + u < IT && e < N && in_level(L, J, I);
            const long long k = ok[u] ? nidx(L, J, I) : L.off;
            mv[u] = L.m[k];
            zv[u] = z[k];
            pv[u] = first ? V(0) : pold[k];
        }
#pragma unroll
        for (int u = 0; u < PB; ++u) {
            const int e = t + (k0 + u) * 256;
            if (k0 + u < IT && e < N) {
                const uint8_t m = ok[u] ? mv[u] : 0;
                const V zz = V(zv[u]);
                sm[e] = m;
                sp[e] = m ? (first ? zz : zz + beta * pv[u]) : V(0);
            }
        }
    }
    __syncthreads();
    const V cx = Coef<V>::cx(L), cy = Coef<V>::cy(L), md = Coef<V>::md(L);
    V acc = V(0);
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr) {
        const int r = threadIdx.y + 8 * qr, c = threadIdx.x;
        const int J = J0 + r, I = I0 + c;
        const int e = (r + H) * W + c + H;
        const V pv = sp[e];
        V qv = V(0);
        if (sm[e]) qv = apply_diff<V>(cx, cy, md, pv, sp[e - 1], sp[e + 1], sp[e - W], sp[e + W]);
        if (J < L.nyn && I < L.nxn) {  // (a wrapped periodic column is not the tile's)
            const long long k = nidx(L, J, I);
            pnew[k] = pv;
            q[k] = qv;
            acc += pv * qv;
        }
    }
    const double tot = block_sum<V>(acc);
    if (t == 0) partials[tix] = tot;
}

// Persistent blocks walk the tile table with the grid's stride; the next
// tile's record is loaded before the current tile is processed, so a block
// starts each tile with its record at hand (a block per tile waited on that
// load, then on the member's scalars, before its first vector load). A
// converged member's tiles cost one check each. Per-tile totals and their
// order are those of a block per tile.
template <typename S, typename V, int TH>
__global__ void __launch_bounds__(256)
k_bs_pq(const int4* __restrict__ tiles, int ntiles, const MGLevel* __restrict__ levs,
        const S* __restrict__ z, V* __restrict__ p0, V* __restrict__ p1, V* __restrict__ q,
        const DevScalars* __restrict__ scs, double* partials, int ir, V* ring,
        long long rstride)
{
    pdl_wait();
    int b = blockIdx.x;
    if (b >= ntiles) return;
    int4 tl = tiles[b];
    for (;;) {
        const int bn = b + gridDim.x;
        const int4 tn = bn < ntiles ? tiles[bn] : tl;
        pq_tile<S, V, TH>(tl, b, levs, z, p0, p1, q, scs, partials, ir, ring, rstride);
        if (bn >= ntiles) break;
        b = bn;
        tl = tn;
    }
}

// <p, q> of every member from k_bs_pq's tile totals (fixed order), alpha =
// rz / <p, q>. The tile kernels write their totals and no more (no fence or
// ticket per block); one block per member sums them here.
__global__ void __launch_bounds__(256)
k_bs_alpha(const BSInfo* __restrict__ info, DevScalars* scs, const double* __restrict__ tpart,
           int ir)
{
    pdl_wait();
    const BSInfo in = info[blockIdx.x];
    DevScalars& sc = scs[blockIdx.x];
    if (bs_skip(sc, ir)) return;
    double acc[1] = {0.0};
    final_sum<1, false>(acc, tpart, in.n0, in.nn, threadIdx.x, blockDim.x);
    __shared__ double sh[32];
    block_reduce<1, false>(acc, sh);
    if (threadIdx.x == 0) {
        sc.pq = acc[0];
        sc.alpha = sc.rz / acc[0];
        if (ir) sc.ahist[sc.iter_in] = f64_to_f32_rn(sc.alpha);
    }
}

// x += alpha p (FP64 form, x the solution; x == nullptr in the refinement
// form, whose correction k_bs_correct forms from the direction ring),
// r -= alpha q, the tile's part of <r, r> (k_bs_conv decides).
template <typename V, int TH>
__device__ __forceinline__ void xr_tile(const int4& tl, int tix, const MGLevel* __restrict__ levs,
                                        V* __restrict__ x, V* __restrict__ r,
                                        const V* __restrict__ p0, const V* __restrict__ p1,
                                        const V* __restrict__ q,
                                        const DevScalars* __restrict__ scs, double* partials,
                                        int ir)
{
    const DevScalars& sc = scs[tl.x];
    if (bs_skip(sc, ir)) return;
    const MGLevel L = levs[tl.x * BS_LMAX];
    const int zero = ir ? 0 : sc.pad1;
    const int it = ir ? sc.iter_in : sc.iter;
    const bool first = ir && it == 0;
    const V* __restrict__ p = (it & 1) ? p0 : p1;  // written by k_bs_pq
    const V a = V(sc.alpha);
    V acc = V(0);
    // rows in batches of 4: the loads of a batch are in flight together,
    // without the register cost of holding all rows of the tile
    constexpr int QB = 4;
#pragma unroll
    for (int q0 = 0; q0 < TH / 8; q0 += QB) {
        long long k[QB];
        bool ok[QB];
        uint8_t mv[QB];
        V xv[QB], pv[QB], rv[QB], qv[QB];
#pragma unroll
        for (int qr = 0; qr < QB; ++qr) {
            const int J = tl.z + threadIdx.y + 8 * (q0 + qr), I = tl.y + threadIdx.x;
            ok[qr] = J < L.nyn && I < L.nxn;
            k[qr] = nidx(L, min(J, L.nyn - 1), min(I, L.nxn - 1));
            mv[qr] = L.m[k[qr]];
            xv[qr] = (first || !x) ? V(0) : x[k[qr]];
            pv[qr] = x ? p[k[qr]] : V(0);
            rv[qr] = r[k[qr]];
            qv[qr] = q[k[qr]];
        }
#pragma unroll
        for (int qr = 0; qr < QB; ++qr) {
            if (!ok[qr] || !mv[qr]) continue;
            if (zero) {
                if (x) x[k[qr]] = V(0);
                r[k[qr]] = V(0);
                continue;
            }
            if (x) x[k[qr]] = xv[qr] + a * pv[qr];
            const V rn = rv[qr] - a * qv[qr];
            r[k[qr]] = rn;
            acc += rn * rn;
        }
    }
    const double tot = block_sum<V>(acc);
    if (threadIdx.x == 0 && threadIdx.y == 0) partials[tix] = tot;
}

// persistent over the tile table, as k_bs_pq
template <typename V, int TH>
__global__ void __launch_bounds__(256)
k_bs_xr(const int4* __restrict__ tiles, int ntiles, const MGLevel* __restrict__ levs,
        V* __restrict__ x, V* __restrict__ r, const V* __restrict__ p0, const V* __restrict__ p1,
        const V* __restrict__ q, const DevScalars* __restrict__ scs, double* partials, int ir)
{
    pdl_wait();
    int b = blockIdx.x;
    if (b >= ntiles) return;
    int4 tl = tiles[b];
    for (;;) {
        const int bn = b + gridDim.x;
        const int4 tn = bn < ntiles ? tiles[bn] : tl;
        xr_tile<V, TH>(tl, b, levs, x, r, p0, p1, q, scs, partials, ir);
        if (bn >= ntiles) break;
        b = bn;
        tl = tn;
    }
}

// <r, r> of every member from k_bs_xr's tile totals (fixed order), the
// member's convergence, and the loop condition (the block that completes
// the count over all members sets it).
__global__ void __launch_bounds__(256)
k_bs_conv(const BSInfo* __restrict__ info, DevScalars* scs, const double* __restrict__ tpart,
          BSGlobals* eg, cudaGraphConditionalHandle cond, int ir, int nmem)
{
    pdl_wait();
    const BSInfo in = info[blockIdx.x];
    DevScalars& sc = scs[blockIdx.x];
    const bool skip = bs_skip(sc, ir);
    double w[1] = {0.0};
    if (!skip) {
        final_sum<1, false>(w, tpart, in.n0, in.nn, threadIdx.x, blockDim.x);
        __shared__ double sh[32];
        block_reduce<1, false>(w, sh);
    }
    const bool mine = threadIdx.x == 0;
    if (mine && !skip) {
        const int zero = ir ? 0 : sc.pad1;
        sc.total_iters += 1;
        const bool bad = !(w[0] == w[0]);
        if (bad) atomicOr(&eg->status, ST_NONFINITE);
        if (ir) {
            sc.iter_in += 1;
            // a round stops at its relative tolerance, or as soon as its
            // residual is a tenth of what the whole solve must reach (the
            // last round of a solve needs only the digits missing, not
            // tol_in more)
            const double goal = fmax(sc.tol_in2 * sc.rr0, 0.01 * sc.tol2 * sc.bb);
            const int done = bad || w[0] <= goal || sc.iter_in >= sc.maxit_in;
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
    if (members_done(mine, &eg->ticket[1], nmem)) {
        eg->loops_in += 1;
        const int act = ir ? *(volatile int*)&eg->active_in : *(volatile int*)&eg->active_out;
        if (cond) cudaGraphSetConditional(cond, act > 0 ? 1u : 0u);
    }
}

// FP64 residual r = b - A x of the tile (x staged with a one-node halo);
// the per-thread sums of b*b (BB) and r*r; r and its FP32 copy rin where
// given. GB300 runs FP64 at 1/64 of its FP32 rate and this is the FP64
// kernel of the FP32 form, so the variants are compile-time (a runtime
// select would issue both sides): HELM, an operator with a main-diagonal
// term (maindiag != 0; exact for members without one too); UNIT, square
// cells (cx = cy = 1: the same sums without the multiplies).
template <int TH, bool HELM, bool UNIT, bool BB>
__device__ __forceinline__ void residual64(const int4& tl, const MGLevel& L,
                                           const double* __restrict__ x,
                                           const double* __restrict__ b, double* __restrict__ r,
                                           float* __restrict__ rin, double (&w)[2])
{
    constexpr int H = 1, W = Reg<H, TH>::WX, N = Reg<H, TH>::N, TQ = TH / 8;
    __shared__ double sx[N];
    __shared__ uint8_t sm[N];
    stage_region<H, TH, double, double>(L, tl.z, tl.y, x, sx, (const double*)nullptr,
                                        (double*)nullptr, sm);
    double bv[TQ];
    long long k[TQ];
    bool ok[TQ];
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr) {
        const int J = tl.z + threadIdx.y + 8 * qr, I = tl.y + threadIdx.x;
        ok[qr] = J < L.nyn && I < L.nxn;
        k[qr] = nidx(L, min(J, L.nyn - 1), min(I, L.nxn - 1));
        bv[qr] = b[k[qr]];
    }
    __syncthreads();
    const double cx = L.cx, cy = L.cy, md = L.md;
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr) {
        const int rr = threadIdx.y + 8 * qr, c = threadIdx.x;
        const int e = (rr + H) * W + c + H;
        double rv = 0.0;
        if (sm[e] && ok[qr]) {
            const double c = sx[e];
            const double sxw = (sx[e - 1] - c) + (sx[e + 1] - c);
            const double syw = (sx[e - W] - c) + (sx[e + W] - c);
            double ax;
            if constexpr (UNIT) ax = sxw + syw;
            else ax = cx * sxw + cy * syw;
            if constexpr (HELM) ax = ax - md * c;
            rv = bv[qr] - ax;
            if constexpr (BB) w[0] += bv[qr] * bv[qr];
            w[1] += rv * rv;
        }
        if (ok[qr]) {
            if (r) r[k[qr]] = rv;
            if (rin) rin[k[qr]] = f64_to_f32_rn(rv);
        }
    }
}

// FP64 form: r = b - A x, <b,b>, <r,r>, per-member start state
template <int TH, bool HELM, bool UNIT>
__global__ void __launch_bounds__(256)
k_bs_init(const int4* __restrict__ tiles, const MGLevel* __restrict__ levs,
          const double* __restrict__ x, const double* __restrict__ b, double* __restrict__ r,
          double* partials)
{
    const int4 tl = tiles[blockIdx.x];
    const MGLevel L = levs[tl.x * BS_LMAX];
    double w[2] = {0.0, 0.0};
    residual64<TH, HELM, UNIT, true>(tl, L, x, b, r, nullptr, w);
    __shared__ double sh[64];
    block_reduce<2, false>(w, sh);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        partials[2 * (size_t)blockIdx.x] = w[0];
        partials[2 * (size_t)blockIdx.x + 1] = w[1];
    }
}

// FP64 form, per member from k_bs_init's tile sums: <b,b>, <r,r>, the start
// state of the solve; the loop condition (the block completing the count)
__global__ void __launch_bounds__(256)
k_bs_init_fin(const BSInfo* __restrict__ info, DevScalars* scs,
              const double* __restrict__ tpart, BSGlobals* eg,
              cudaGraphConditionalHandle cond, int nmem)
{
    const BSInfo in = info[blockIdx.x];
    DevScalars& sc = scs[blockIdx.x];
    double w[2];
    final_sum<2, false>(w, tpart, in.n0, in.nn, threadIdx.x, blockDim.x);
    __shared__ double sh[64];
    block_reduce<2, false>(w, sh);
    const bool mine = threadIdx.x == 0;
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

// Refinement form: r = b - A x (FP64) of the tile, its FP32 copy that drives
// the next inner solve, and the tile's sums of b*b (first call of a solve)
// and r*r; members already converged are skipped.
template <int TH, bool HELM, bool UNIT, bool FIRST>
__global__ void __launch_bounds__(256)
k_bs_refine(const int4* __restrict__ tiles, const MGLevel* __restrict__ levs,
            const double* __restrict__ x, const double* __restrict__ b,
            float* __restrict__ rin, const DevScalars* __restrict__ scs, double* partials)
{
    const int4 tl = tiles[blockIdx.x];
    if (scs[tl.x].converged) return;
    const MGLevel L = levs[tl.x * BS_LMAX];
    double w[2] = {0.0, 0.0};
    // <b, b> once per solve (the first call); the FP64 residual itself is
    // not stored (the inner solve reads its FP32 copy)
    residual64<TH, HELM, UNIT, FIRST>(tl, L, x, b, nullptr, rin, w);
    __shared__ double sh[64];
    block_reduce<2, false>(w, sh);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        partials[2 * (size_t)blockIdx.x] = w[0];
        partials[2 * (size_t)blockIdx.x + 1] = w[1];
    }
}

// Refinement form, per member from k_bs_refine's tile sums: converged, or
// start a new round; the outer loop condition.
__global__ void __launch_bounds__(256)
k_bs_refine_fin(const BSInfo* __restrict__ info, DevScalars* scs,
                const double* __restrict__ tpart, BSGlobals* eg, int first,
                cudaGraphConditionalHandle cond, int nmem)
{
    const BSInfo in = info[blockIdx.x];
    DevScalars& sc = scs[blockIdx.x];
    const bool skip = sc.converged != 0;
    double w[2] = {0.0, 0.0};
    if (!skip) {
        final_sum<2, false>(w, tpart, in.n0, in.nn, threadIdx.x, blockDim.x);
        __shared__ double sh[64];
        block_reduce<2, false>(w, sh);
    }
    const bool mine = threadIdx.x == 0;
    if (mine && !skip) {
        const double rr_prev = sc.rr;
        if (first) sc.bb = w[0];
        else w[0] = sc.bb;
        sc.rr = w[1];
        const int zero = (w[0] == 0.0);
        sc.zero = zero;
        int conv = zero ? (w[1] == 0.0) : (w[1] <= sc.tol2 * w[0]);
        // the FP64 residual of a round cannot fall below its rounding floor
        // (about eps * cond(A) relative); a round that no longer reduces it
        // by 10x has reached that floor
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
    if (members_done(mine, &eg->ticket[0], nmem)) {
        eg->loops_out += 1;
        if (cond) cudaGraphSetConditional(cond, *(volatile int*)&eg->active_out > 0 ? 1u : 0u);
    }
}

// x += e (FP64); a member with a zero right-hand side gets x = 0
template <int TH>
__global__ void __launch_bounds__(256)
k_bs_correct(const int4* __restrict__ tiles, const MGLevel* __restrict__ levs,
             double* __restrict__ x, const float* __restrict__ ring, long long rstride,
             const DevScalars* __restrict__ scs)
{
    const int4 tl = tiles[blockIdx.x];
    const DevScalars& sc = scs[tl.x];
    if (sc.converged) return;
    const MGLevel L = levs[tl.x * BS_LMAX];
    const int zero = sc.zero;
    const int kit = sc.iter_in;  // inner iterations of the round
    constexpr int TQ = TH / 8;
    long long k[TQ];
    float ev[TQ];
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr) {
        const int J = tl.z + threadIdx.y + 8 * qr, I = tl.y + threadIdx.x;
        k[qr] = nidx(L, min(J, L.nyn - 1), min(I, L.nxn - 1));
        ev[qr] = 0.f;
    }
    // e = sum alpha_i p_i in the order of the iterations, as the iterations
    // would have accumulated it (e_{i+1} = e_i + alpha_i p_i, FP32); four
    // directions' loads in flight before their FMAs
    constexpr int CH = 4;
    for (int i0 = 0; i0 < kit; i0 += CH) {
        float pv[CH][TQ];
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            const float* __restrict__ p = ring + (long long)min(i0 + c, kit - 1) * rstride;
#pragma unroll
            for (int qr = 0; qr < TQ; ++qr) pv[c][qr] = p[k[qr]];
        }
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            if (i0 + c >= kit) break;
            const float a = sc.ahist[i0 + c];
#pragma unroll
            for (int qr = 0; qr < TQ; ++qr) ev[qr] = fmaf(a, pv[c][qr], ev[qr]);
        }
    }
    uint8_t mv[TQ];
    double xv[TQ];
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr) {
        mv[qr] = L.m[k[qr]];
        xv[qr] = x[k[qr]];
    }
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr) {
        const int J = tl.z + threadIdx.y + 8 * qr, I = tl.y + threadIdx.x;
        if (J < L.nyn && I < L.nxn && mv[qr])
            x[k[qr]] = zero ? 0.0 : xv[qr] + f32_to_f64(ev[qr]);
    }
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

// one V-cycle for all members still iterating: a down kernel per grid level,
// the tail, an up kernel per grid level (the level-0 one also forms <r, z>)
// Launch with programmatic stream serialization (the kernel calls pdl_wait()
// before touching its predecessor's output): its blocks can be scheduled
// while the predecessor on the stream drains, which hides part of the launch
// gap between the many short kernels of the CG loop.
template <typename... KA, typename... A>
static void launch_pdl(void (*k)(KA...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       A... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, args...);
}

// Grid of a persistent 256-thread kernel: the blocks that fit on the device
// at once (occupancy of this kernel, computed on first use), at most one per
// tile.
template <auto KERN>
static int resident_grid(int ntiles)
{
    static int resident = 0;
    if (resident == 0) {
        int dev = 0, nsm = 0, nb = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, KERN, 256, 0);
        resident = std::max(1, nsm * nb);
    }
    return std::max(1, std::min(ntiles, resident));
}

// the same with the pipelined FP32 level kernels (persistent blocks)
template <int NU>
static int vcycle_pipe(BatchSolver& s, cudaStream_t st, int ir)
{
    const dim3 blk(32, MR_NW);
    const CUtensorMap* maps = (const CUtensorMap*)s.mmaps;
    int* status = &s.eg->status;
    int cnt = 0;
    for (int l = 0; l < s.maxl; ++l) {
        const int n = s.nmtiles[l];
        if (n == 0) continue;
        launch_pdl(k_mgp_down<NU>, dim3(std::min(n, s.pipe_gdown)), blk, sizeof(MPDown), st,
                   (const int4*)s.mtiles[l], n, (const MGLevel*)s.dlevs, maps, l,
                   (const DevScalars*)s.scs, ir, status);
        cnt += 1;
    }
    launch_pdl(k_bs_tail<float>, dim3(s.n), dim3(s.tail_threads), s.tail_smem, st,
               (const BSInfo*)s.dinfo, (const MGLevel*)s.dlevs, s.scs, ir, NU);
    cnt += 1;
    for (int l = s.maxl - 1; l >= 0; --l) {
        const int n = s.nmtiles[l];
        if (n == 0) continue;
        if (l > 0)
            launch_pdl(k_mgp_up<NU, false>, dim3(std::min(n, s.pipe_gup)), blk, sizeof(MPUp), st,
                       (const int4*)s.mtiles[l], n, (const MGLevel*)s.dlevs, maps, l,
                       (const DevScalars*)s.scs, ir, (double*)nullptr, status);
        else
            launch_pdl(k_mgp_up<NU, true>, dim3(std::min(n, s.pipe_gup)), blk, sizeof(MPUp), st,
                       (const int4*)s.mtiles[0], n, (const MGLevel*)s.dlevs, maps, 0,
                       (const DevScalars*)s.scs, ir, s.mpartials, status);
        cnt += 1;
    }
    return cnt;
}

template <typename S, int NU, int TH>
static int vcycle_nu(BatchSolver& s, cudaStream_t st, int ir)
{
    if constexpr (std::is_same<S, float>::value)
        if (s.pipe) return vcycle_pipe<NU>(s, st, ir);
    const dim3 blk(32, MR_NW);
    int cnt = 0;
    for (int l = 0; l < s.maxl; ++l) {
        k_mg_down<S, NU><<<s.nmtiles[l], blk, 0, st>>>(s.mtiles[l], s.dinfo, s.dlevs, l,
                                                       s.scs, ir);
        cnt += 1;
    }
    k_bs_tail<S><<<s.n, s.tail_threads, s.tail_smem, st>>>(s.dinfo, s.dlevs, s.scs, ir, NU);
    cnt += 1;
    for (int l = s.maxl - 1; l >= 1; --l) {
        k_mg_up<S, NU, false><<<s.nmtiles[l], blk, 0, st>>>(s.mtiles[l], s.dinfo, s.dlevs, l,
                                                           s.scs, ir, nullptr);
        cnt += 1;
    }
    if (s.maxl > 0) {
        k_mg_up<S, NU, true><<<s.nmtiles[0], blk, 0, st>>>(s.mtiles[0], s.dinfo, s.dlevs, 0,
                                                          s.scs, ir, s.mpartials);
        cnt += 1;
    }
    return cnt;
}

template <typename S, int TH>
static int vcycle(BatchSolver& s, cudaStream_t st, int ir)
{
    return s.nu >= 2 ? vcycle_nu<S, 2, TH>(s, st, ir) : vcycle_nu<S, 1, TH>(s, st, ir);
}

// the CG loop body; FP64 form (S = V = double) or the inner FP32 loop
template <typename S, typename V, int TH>
static int cg_body(BatchSolver& s, cudaStream_t st, cudaGraphConditionalHandle cond, int ir)
{
    const dim3 blk(32, 8);
    const int nt = s.nrtiles;
    V* r = (V*)(ir ? s.v.rin : s.v.r64);
    V* x = ir ? (V*)nullptr : (V*)s.v.x64;  // the refinement form's x is the ring
    int cnt = vcycle<S, TH>(s, st, ir);
    if (s.maxl > 0) {
        launch_pdl(k_bs_rz, dim3(s.n), dim3(256), 0, st, (const BSInfo*)s.dinfo, s.scs,
                   (const double*)s.mpartials, ir);
        cnt += 1;
    }
    V* ring = ir ? (V*)s.pring : (V*)nullptr;
    launch_pdl(k_bs_pq<S, V, TH>, dim3(resident_grid<k_bs_pq<S, V, TH>>(nt)), blk, 0, st,
               (const int4*)s.rtiles, nt, (const MGLevel*)s.dlevs, (const S*)s.v.z, (V*)s.v.p,
               (V*)s.v.p2, (V*)s.v.q, (const DevScalars*)s.scs, s.partials, ir, ring,
               (long long)s.v.nelem);
    launch_pdl(k_bs_alpha, dim3(s.n), dim3(256), 0, st, (const BSInfo*)s.dinfo, s.scs,
               (const double*)s.partials, ir);
    launch_pdl(k_bs_xr<V, TH>, dim3(resident_grid<k_bs_xr<V, TH>>(nt)), blk, 0, st,
               (const int4*)s.rtiles, nt, (const MGLevel*)s.dlevs, x, r, (const V*)s.v.p,
               (const V*)s.v.p2, (const V*)s.v.q, (const DevScalars*)s.scs, s.partials, ir);
    launch_pdl(k_bs_conv, dim3(s.n), dim3(256), 0, st, (const BSInfo*)s.dinfo, s.scs,
               (const double*)s.partials, s.eg, cond, ir, s.n);
    cnt += 4;
    s.body_launches = cnt;
    return (int)cudaGetLastError();
}


static int read_globals(const BatchSolver& s, cudaStream_t st, BSGlobals* h)
{
    cudaError_t e = cudaMemcpyAsync(h, s.eg, sizeof(*h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return (int)e;
}

// the FP64 residual kernels in the solver's operator variant (bs_build:
// helm = a member has a main-diagonal term, unit = every member has square
// cells)
template <int TH, bool FIRST>
static void launch_refine(const BatchSolver& s, cudaStream_t st)
{
    const dim3 blk(32, 8);
    const int nt = s.nrtiles;
    const double* x = (const double*)s.v.x64;
    const double* b = (const double*)s.v.b64;
    float* rin = (float*)s.v.rin;
    if (s.helm) {
        if (s.unit) k_bs_refine<TH, true, true, FIRST><<<nt, blk, 0, st>>>(s.rtiles, s.dlevs, x, b, rin, s.scs, s.partials);
        else k_bs_refine<TH, true, false, FIRST><<<nt, blk, 0, st>>>(s.rtiles, s.dlevs, x, b, rin, s.scs, s.partials);
    } else {
        if (s.unit) k_bs_refine<TH, false, true, FIRST><<<nt, blk, 0, st>>>(s.rtiles, s.dlevs, x, b, rin, s.scs, s.partials);
        else k_bs_refine<TH, false, false, FIRST><<<nt, blk, 0, st>>>(s.rtiles, s.dlevs, x, b, rin, s.scs, s.partials);
    }
}

template <int TH>
static void launch_init(const BatchSolver& s, cudaStream_t st)
{
    const dim3 blk(32, 8);
    const int nt = s.nrtiles;
    const double* x = (const double*)s.v.x64;
    const double* b = (const double*)s.v.b64;
    double* r = (double*)s.v.r64;
    if (s.helm) {
        if (s.unit) k_bs_init<TH, true, true><<<nt, blk, 0, st>>>(s.rtiles, s.dlevs, x, b, r, s.partials);
        else k_bs_init<TH, true, false><<<nt, blk, 0, st>>>(s.rtiles, s.dlevs, x, b, r, s.partials);
    } else {
        if (s.unit) k_bs_init<TH, false, true><<<nt, blk, 0, st>>>(s.rtiles, s.dlevs, x, b, r, s.partials);
        else k_bs_init<TH, false, false><<<nt, blk, 0, st>>>(s.rtiles, s.dlevs, x, b, r, s.partials);
    }
}

template <int TH>
static int bs_record_t(BatchSolver& s, cudaStream_t st, cudaStream_t st2, int* launches)
{
    const dim3 blk(32, 8);
    const int nt = s.nrtiles;
    int fixed = 0;
    k_bs_setup<<<(s.n + 127) / 128, 128, 0, st>>>(s.scs, s.n, s.tol * s.tol, s.maxit,
                                                   s.tol_in * s.tol_in,
                                                   std::min(s.maxit_in, BS_RING), s.maxouter,
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
        launch_init<TH>(s, st);
        k_bs_init_fin<<<s.n, 256, 0, st>>>(s.dinfo, s.scs, s.partials, s.eg, cond, s.n);
        fixed += 2;
        if (capturing) {
            int r = add_while(st, st2, &cond, 1, [&](cudaStream_t sb) {
                return cg_body<double, double, TH>(s, sb, cond, 0);
            });
            if (r) return r;
        } else {
            for (int it = 0; it <= s.maxit; ++it) {
                int r = read_globals(s, st, &h);
                if (r) return r;
                if (h.active_out <= 0) break;
                r = cg_body<double, double, TH>(s, st, 0, 0);
                if (r) return r;
            }
        }
        if (launches) *launches = fixed;
        return (int)cudaGetLastError();
    }
    // refinement form
    if (!s.s3) {  // the solver's own body stream of the nested loop
        e = cudaStreamCreateWithFlags(&s.s3, cudaStreamNonBlocking);
        if (e != cudaSuccess) return (int)e;
    }
    cudaGraphConditionalHandle cond_o = 0;
    if (capturing) {
        e = cudaGraphConditionalHandleCreate(&cond_o, graph, 1, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return (int)e;
    }
    k_bs_reset<<<1, 1, 0, st>>>(s.eg);
    launch_refine<TH, true>(s, st);
    k_bs_refine_fin<<<s.n, 256, 0, st>>>(s.dinfo, s.scs, s.partials, s.eg, 1, cond_o, s.n);
    fixed += 3;
    auto round_tail = [&](cudaStream_t sb) {
        k_bs_correct<TH><<<nt, blk, 0, sb>>>(s.rtiles, s.dlevs, (double*)s.v.x64,
                                             (const float*)s.pring, (long long)s.v.nelem,
                                             s.scs);
        k_bs_reset<<<1, 1, 0, sb>>>(s.eg);
        launch_refine<TH, false>(s, sb);
        k_bs_refine_fin<<<s.n, 256, 0, sb>>>(s.dinfo, s.scs, s.partials, s.eg, 0, cond_o, s.n);
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
            int r2 = add_while(sb, s.s3, &cond_i, 0, [&](cudaStream_t sc3) {
                return cg_body<float, float, TH>(s, sc3, cond_i, 1);
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
                r = cg_body<float, float, TH>(s, st, 0, 1);
                if (r) return r;
            }
            round_tail(st);
        }
    }
    if (launches) *launches = fixed;
    return (int)cudaGetLastError();
}

// Measurement hook: time `reps` launches of the level-0 down kernel (the
// largest share of the solver's time) on the current level-0 right-hand side
// of every member, L2 flushed between launches when asked. Every member's
// convergence flags are cleared first so that no block returns early; the
// next solve's set-up resets them. *nodes = level-0 nodes of all members,
// *es = element size of the multigrid vectors.
__global__ void k_bs_activate(DevScalars* scs, int n)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < n) {
        scs[b].converged = 0;
        scs[b].conv_in = 0;
    }
}

template <typename S, int NU>
static void launch_down0(BatchSolver& s, cudaStream_t st, int ir)
{
    if constexpr (std::is_same<S, float>::value)
        if (s.pipe) {
            k_mgp_down<NU><<<std::min(s.nmtiles[0], s.pipe_gdown), dim3(32, MR_NW),
                             sizeof(MPDown), st>>>(s.mtiles[0], s.nmtiles[0], s.dlevs,
                                                   (const CUtensorMap*)s.mmaps, 0, s.scs, ir,
                                                   &s.eg->status);
            return;
        }
    k_mg_down<S, NU><<<s.nmtiles[0], dim3(32, MR_NW), 0, st>>>(s.mtiles[0], s.dinfo, s.dlevs, 0,
                                                              s.scs, ir);
}

int bs_time_down(BatchSolver& s, cudaStream_t st, int reps, int flush_l2, double* avg_ms,
                 long long* nodes, int* es)
{
    if (s.maxl < 1 || reps < 1) return 1;
    long long n0 = 0;
    for (const MGHost& g : s.mg) n0 += (long long)g.lev[0].nyn * g.lev[0].nxn;
    if (nodes) *nodes = n0;
    if (es) *es = s.mode == 0 ? 8 : 4;
    const size_t flush_bytes = 256ull << 20;
    void* fl = nullptr;
    if (flush_l2 && cudaMalloc(&fl, flush_bytes) != cudaSuccess) return 2;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_bs_activate<<<(s.n + 127) / 128, 128, 0, st>>>(s.scs, s.n);
    const int ir = s.mode == 1 ? 1 : 0;
    double total = 0.0;
    int err = 0;
    for (int r = 0; r < reps && !err; ++r) {
        if (fl) cudaMemsetAsync(fl, r & 0xff, flush_bytes, st);
        cudaEventRecord(a, st);
        const bool two = s.nu >= 2;
        if (s.mode == 0) two ? launch_down0<double, 2>(s, st, ir) : launch_down0<double, 1>(s, st, ir);
        else two ? launch_down0<float, 2>(s, st, ir) : launch_down0<float, 1>(s, st, ir);
        cudaEventRecord(b, st);
        if (cudaEventSynchronize(b) != cudaSuccess) err = 3;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        total += ms;
    }
    if (!err && cudaGetLastError() != cudaSuccess) err = 3;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (fl) cudaFree(fl);
    if (err) return err;
    *avg_ms = total / reps;
    return 0;
}

int bs_record(BatchSolver& s, cudaStream_t st, cudaStream_t st2, int* launches)
{
    return s.th == 64 ? bs_record_t<64>(s, st, st2, launches)
                      : bs_record_t<32>(s, st, st2, launches);
}

// ---- pipelined FP32 level kernels (mg_pipe.cuh): layout checks, TMA maps ----
static PFN_cuTensorMapEncodeTiled_v12000 bs_encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)ptr;
    }
    return fn;
}

// What the pipelined kernels assume of the layout: every level's rows start
// 16 elements aligned (c0 = off mod 16 the column of node 0, node columns
// inside the pitch, pitch a multiple of 16, coarse levels at off = 1, 16-byte
// aligned arrays); on a closed level 0 the mask bytes of a node row outside
// its node columns are 0 (the TMA row spans the whole pitch); the coarse
// fluid flags are the fine centre nodes' (the restriction takes them from
// there).
static bool bs_pipe_layout_ok(BatchSolver& s, const std::vector<MGLevel>& levs,
                              const std::vector<BSInfo>& info)
{
    for (int b = 0; b < s.n; ++b) {
        const int nl = info[b].nl;
        for (int l = 0; l < nl; ++l) {
            const MGLevel& L = levs[(size_t)b * BS_LMAX + l];
            const long long c0 = L.off & 15;
            if (L.pitch % 16 || c0 + L.nxn > L.pitch || (l > 0 && L.off != 1)) return false;
            for (const void* p : {(const void*)L.x, (const void*)L.xa, (const void*)L.b,
                                  (const void*)L.m})
                if ((uintptr_t)p % 16) return false;
        }
        BSMemberDesc& d = s.descs[b];
        const MGLevel& L0 = levs[(size_t)b * BS_LMAX];
        const long long c0 = L0.off & 15;
        if (d.hwin) {
            bool ok = d.hoff0 >= c0 && (d.hoff0 & 15) == c0;
            for (int J = 0; ok && !L0.per && J < L0.nyn; ++J) {
                const uint8_t* row = d.hmask + (d.hoff0 - c0) + (long long)J * L0.pitch;
                for (long long c = 0; c < L0.pitch; ++c)
                    if ((c < c0 || c >= c0 + L0.nxn) && row[c]) {
                        ok = false;
                        break;
                    }
            }
            d.win_ok = ok ? 1 : 0;
        }
        if (!d.win_ok) return false;
        for (int l = 0; l < info[b].ltail && l + 1 < nl; ++l) {
            const MGLevel& F = levs[(size_t)b * BS_LMAX + l];
            const MGLevel& C = levs[(size_t)b * BS_LMAX + l + 1];
            const std::vector<uint8_t>& fm = s.mg[b].hmask[l];
            const std::vector<uint8_t>& cm = s.mg[b].hmask[l + 1];
            for (int J = 0; J < C.nyn; ++J)
                for (int I = 0; I < C.nxn; ++I) {
                    const uint8_t f = 2 * J < F.nyn && 2 * I < F.nxn
                                          ? fm[(size_t)(2 * J) * F.nxn + 2 * I] : 0;
                    if ((cm[(size_t)J * C.nxn + I] != 0) != (f != 0)) return false;
                }
        }
    }
    return true;
}

template <typename DAL>
static int bs_pipe_setup(BatchSolver& s, const std::vector<MGLevel>& levs,
                         const std::vector<BSInfo>& info, DAL& dal)
{
    s.pipe = false;
    s.mmaps = nullptr;
    if (s.mode != 1 || s.maxl < 1) return 0;
    auto enc = bs_encode_fn();
    if (!enc || !bs_pipe_layout_ok(s, levs, info)) return 0;
    // grid sizes: resident blocks per SM x SMs (persistent blocks)
    static int gdown = 0, gup = 0;
    if (!gdown) {
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        int lo_d = 1 << 30, lo_u = 1 << 30;
        auto occ = [&](const void* fn, size_t smem, int& lo) {
            cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            int nb = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 32 * MR_NW, smem);
            lo = std::min(lo, nb);
        };
        occ((const void*)k_mgp_down<1>, sizeof(MPDown), lo_d);
        occ((const void*)k_mgp_down<2>, sizeof(MPDown), lo_d);
        occ((const void*)k_mgp_up<1, false>, sizeof(MPUp), lo_u);
        occ((const void*)k_mgp_up<1, true>, sizeof(MPUp), lo_u);
        occ((const void*)k_mgp_up<2, false>, sizeof(MPUp), lo_u);
        occ((const void*)k_mgp_up<2, true>, sizeof(MPUp), lo_u);
        if (cudaGetLastError() != cudaSuccess || nsm < 1 || lo_d < 1 || lo_u < 1) return 0;
        gdown = lo_d * nsm;
        gup = lo_u * nsm;
    }
    const size_t nmap = (size_t)s.n * BS_LMAX * MP_NMAP;
    std::vector<CUtensorMap> maps(nmap);
    memset(maps.data(), 0, nmap * sizeof(CUtensorMap));
    for (int b = 0; b < s.n; ++b)
        for (int l = 0; l < info[b].nl; ++l) {
            const MGLevel& L = levs[(size_t)b * BS_LMAX + l];
            const long long base = L.off - (L.off & 15);
            CUtensorMap* mp = &maps[((size_t)b * BS_LMAX + l) * MP_NMAP];
            auto one = [&](CUtensorMap* m, const void* arr, bool u8, int bw, int bh) {
                const size_t es = u8 ? 1 : 4;
                cuuint64_t dims[2] = {(cuuint64_t)L.pitch, (cuuint64_t)L.nyn};
                cuuint64_t strides[1] = {(cuuint64_t)(L.pitch * es)};
                cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
                cuuint32_t estr[2] = {1, 1};
                return enc(m, u8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                           2, (void*)((const char*)arr + base * es), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
            };
            if (!one(mp + MP_B, L.b, false, MP_BW, MR_WY) ||
                !one(mp + MP_M, L.m, true, MP_MW, MR_WY) ||
                !one(mp + MP_XA, L.xa, false, MP_BW, MR_WY) ||
                !one(mp + MP_X, L.x, false, MP_CW, MP_CH))
                return 0;  // keep the one-tile-per-block kernels
        }
    void* d = dal(nmap * sizeof(CUtensorMap));
    if (!d) return 2;
    if (cudaMemcpy(d, maps.data(), nmap * sizeof(CUtensorMap), cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return 2;
    s.mmaps = d;
    s.pipe_gdown = gdown;
    s.pipe_gup = gup;
    s.pipe = true;
    return 0;
}

int bs_build(BatchSolver& s, const std::vector<BSMemberDesc>& members, const uint8_t* dmask,
             int mode, const BSVecs& v, DevScalars* scs)
{
    bs_free(s);
    s.n = (int)members.size();
    s.mode = mode;
    s.v = v;
    s.scs = scs;
    s.descs = members;
    s.dmask = dmask;
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
                         v.z, v.za, r0, d.cx, d.cy, d.maindiag, mode == 0 ? 0 : 1);
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
    // Tile height: 64 rows when level 0 holds enough nodes to fill the GPU
    // many times over (fewer, fuller blocks), else 32 (more blocks for small
    // problems, which are latency-bound).
    {
        long long n0 = 0;
        for (int b = 0; b < s.n; ++b)
            n0 += (long long)levs[(size_t)b * BS_LMAX].nyn * levs[(size_t)b * BS_LMAX].nxn;
        s.th = s.th_force ? s.th_force : n0 >= 2ll * 1024 * 1024 ? 64 : 32;
    }
    const int TH = s.th;
    // Tile table of 32 x TH level-0 nodes for the Krylov kernels (all
    // members; member b's tiles n0 .. n0+nn, whose per-tile sums the
    // member's finishing kernels add up). Tiles
    // without a fluid node are left out (their nodes stay 0 in every
    // vector), but every member keeps at least one tile for its reductions.
    auto has_fluid = [&](int b, int l, int J0, int I0) {
        const std::vector<uint8_t>& hm = s.mg[b].hmask[l];
        const MGLevel& L = levs[(size_t)b * BS_LMAX + l];
        for (int J = J0; J < std::min(L.nyn, J0 + TH); ++J)
            for (int I = I0; I < std::min(L.nxn, I0 + BS_TW); ++I)
                if (hm[(size_t)J * L.nxn + I]) return true;
        return false;
    };
    std::vector<std::vector<int4>> tiles(1);
    std::vector<int4>& rt = tiles[0];
    for (int b = 0; b < s.n; ++b) {
        const MGLevel& L = levs[(size_t)b * BS_LMAX];
        info[b].n0 = (int)rt.size();
        for (int J0 = 0; J0 < L.nyn; J0 += TH)
            for (int I0 = 0; I0 < L.nxn; I0 += BS_TW)
                if (has_fluid(b, 0, J0, I0)) rt.push_back(make_int4(b, I0, J0, 0));
        if ((int)rt.size() == info[b].n0) rt.push_back(make_int4(b, 0, 0, 0));
        info[b].nn = (int)rt.size() - info[b].n0;
    }
    // Tile tables of the multigrid level kernels (MR_TW x MR_TH nodes,
    // register-blocked, mg_reg.cuh) for every grid level below a member's
    // tail; tiles without a fluid node are left out.
    auto has_fluid_m = [&](int b, int l, int J0, int I0) {
        const std::vector<uint8_t>& hm = s.mg[b].hmask[l];
        const MGLevel& L = levs[(size_t)b * BS_LMAX + l];
        for (int J = J0; J < std::min(L.nyn, J0 + MR_TH); ++J)
            for (int I = I0; I < std::min(L.nxn, I0 + MR_TW); ++I)
                if (hm[(size_t)J * L.nxn + I]) return true;
        return false;
    };
    // Level 0 also carries the members' ranges of the level-0 up leg's
    // <r, z> tile totals (mn0, mnn): every member that reaches below level 0
    // keeps at least one tile there.
    // The record's .w serves the pipelined kernels: the column of node 0 in
    // its row (c0) and MP_SLOW for a region that wraps around the level.
    auto tile_w = [&](const MGLevel& L, int I0) {
        const int slow = L.per && (I0 - MR_H < 0 || I0 - MR_H + MR_W > L.nxn) ? MP_SLOW : 0;
        return (int)(L.off & 15) | slow;
    };
    std::vector<std::vector<int4>> mt(std::max(1, s.maxl));
    for (int l = 0; l < s.maxl; ++l)
        for (int b = 0; b < s.n; ++b) {
            if (info[b].ltail <= l) continue;
            const MGLevel& L = levs[(size_t)b * BS_LMAX + l];
            const int first = (int)mt[l].size();
            for (int J0 = 0; J0 < L.nyn; J0 += MR_TH)
                for (int I0 = 0; I0 < L.nxn; I0 += MR_TW)
                    if (has_fluid_m(b, l, J0, I0))
                        mt[l].push_back(make_int4(b, I0, J0, tile_w(L, I0)));
            if (l == 0) {
                if ((int)mt[0].size() == first) mt[0].push_back(make_int4(b, 0, 0, tile_w(L, 0)));
                info[b].mn0 = first;
                info[b].mnn = (int)mt[0].size() - first;
            }
        }
    auto dal = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        s.owned.push_back(p);
        return p;
    };
    s.mtiles.assign(mt.size(), nullptr);
    s.nmtiles.assign(mt.size(), 0);
    for (size_t l = 0; l < mt.size(); ++l) {
        s.nmtiles[l] = (int)mt[l].size();
        s.mtiles[l] = (int4*)dal(std::max<size_t>(1, mt[l].size()) * sizeof(int4));
        if (!s.mtiles[l]) return 2;
        if (!mt[l].empty() &&
            cudaMemcpy(s.mtiles[l], mt[l].data(), mt[l].size() * sizeof(int4),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return 2;
    }
    const int ntab = (int)tiles.size();
    s.tiles.assign(ntab, nullptr);
    s.ntiles.assign(ntab, 0);
    for (int l = 0; l < ntab; ++l) {
        s.ntiles[l] = (int)tiles[l].size();
        s.tiles[l] = (int4*)dal(std::max<size_t>(1, tiles[l].size()) * sizeof(int4));
        if (!s.tiles[l]) return 2;
        if (!tiles[l].empty() &&
            cudaMemcpy(s.tiles[l], tiles[l].data(), tiles[l].size() * sizeof(int4),
                       cudaMemcpyHostToDevice) != cudaSuccess)
            return 2;
    }
    s.nrtiles = s.ntiles[0];
    s.rtiles = s.tiles[0];
    s.dlevs = (MGLevel*)dal(levs.size() * sizeof(MGLevel));
    s.dinfo = (BSInfo*)dal(info.size() * sizeof(BSInfo));
    s.eg = (BSGlobals*)dal(sizeof(BSGlobals));
    s.partials = (double*)dal((rt.size() * 2 + 64) * sizeof(double));
    s.mpartials = (double*)dal((mt[0].size() + 64) * sizeof(double));
    if (!s.mpartials) return 2;
    if (!s.dlevs || !s.dinfo || !s.eg || !s.partials) return 2;
    // operator variant of the FP64 residual kernels
    s.helm = false;
    s.unit = true;
    for (int b = 0; b < s.n; ++b) {
        const MGLevel& L = levs[(size_t)b * BS_LMAX];
        if (L.md != 0.0) s.helm = true;
        if (!(L.cx == 1.0 && L.cy == 1.0)) s.unit = false;
    }
    // the tail's block: 1024 threads while every member has an SM of its own,
    // else 512 (two blocks per SM: the members' tails run in one wave)
    {
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        s.tail_threads = s.n > nsm ? 512 : 1024;
    }
    {
        const int e = bs_pipe_setup(s, levs, info, dal);
        if (e) return e;
    }
    if (mode == 1) {
        if (v.nelem <= 0) return 1;
        s.pring = (float*)dal((size_t)BS_RING * v.nelem * sizeof(float));
        if (!s.pring) return 2;
    }
    if (cudaMemcpy(s.dlevs, levs.data(), levs.size() * sizeof(MGLevel), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(s.dinfo, info.data(), info.size() * sizeof(BSInfo), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemset(s.eg, 0, sizeof(BSGlobals)) != cudaSuccess)
        return 2;
    // The dynamic shared-memory limit is an attribute of the tail kernel, not
    // of this solver: raise it to the largest tail any solver of the process
    // needs and never lower it, or the launches (and new graph captures) of
    // an existing solver with a larger tail would fail. (One host thread and
    // one device per process, as everywhere in this library.)
    static size_t tail_attr[2] = {0, 0};
    const int ti = mode == 0 ? 0 : 1;
    if (s.tail_smem > tail_attr[ti]) {
        cudaError_t fe = mode == 0
            ? cudaFuncSetAttribute(k_bs_tail<double>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)s.tail_smem)
            : cudaFuncSetAttribute(k_bs_tail<float>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)s.tail_smem);
        if (fe != cudaSuccess) return 4;
        tail_attr[ti] = s.tail_smem;
    }
    return 0;
}

// x = f * src over n doubles (the autotuner's warm start)
__global__ void k_bs_scale(double* __restrict__ x, const double* __restrict__ src, double f,
                           size_t n)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
         k += (size_t)gridDim.x * blockDim.x)
        x[k] = f * src[k];
}

// the same members with tile rows th: level-0 masks from the multigrid
// hierarchy, the device layout and settings unchanged
static int bs_rebuild(BatchSolver& s, int th)
{
    std::vector<BSMemberDesc> descs = s.descs;
    std::vector<std::vector<uint8_t>> hm(s.n);
    for (int b = 0; b < s.n; ++b) {
        BSMemberDesc& d = descs[b];
        const std::vector<uint8_t>& m0 = s.mg[b].hmask[0];
        hm[b].assign((size_t)(d.nyn - 1) * d.pitch + d.nxn, 0);
        for (int J = 0; J < d.nyn; ++J)
            for (int I = 0; I < d.nxn; ++I)
                hm[b][(size_t)J * d.pitch + I] = m0[(size_t)J * d.nxn + I];
        d.hmask = hm[b].data();
        d.hoff0 = 0;
        d.hwin = 0;  // dense node masks: win_ok from the first build stands
    }
    const BSVecs v = s.v;
    DevScalars* scs = s.scs;
    const uint8_t* dmask = s.dmask;
    const double tol = s.tol, tol_in = s.tol_in;
    const int maxit = s.maxit, maxit_in = s.maxit_in, maxouter = s.maxouter, nu = s.nu;
    s.th_force = th;
    const int e = bs_build(s, descs, dmask, s.mode, v, scs);
    s.tol = tol;
    s.tol_in = tol_in;
    s.maxit = maxit;
    s.maxit_in = maxit_in;
    s.maxouter = maxouter;
    s.nu = nu;
    return e;
}

int bs_autotune(BatchSolver& s, cudaStream_t st, cudaStream_t st2, void* x, const void* b,
                size_t xbytes, int reps, BSTune* out)
{
    if (s.n == 0 || s.mg.empty()) return 9;
    const size_t n = xbytes / sizeof(double);
    double* saved = nullptr;
    if (cudaMalloc(&saved, xbytes) != cudaSuccess) return 2;
    cudaMemcpyAsync(saved, x, xbytes, cudaMemcpyDeviceToDevice, st);
    cudaEvent_t ea, eb;
    cudaEventCreate(&ea);
    cudaEventCreate(&eb);
    const bool eager = bs_eager();
    const double tin[5] = {1e-8, 1e-7, 1e-6, 1e-5, 1e-4};
    const int ntin = s.mode == 1 ? 5 : 1;
    BSTune best{0, 0, 0.0, 1e300, 0};
    int err = 0;
    for (int th : {32, 64}) {
        if (th != s.th && (err = bs_rebuild(s, th))) break;
        for (int nu : {1, 2}) {
            for (int k = 0; k < ntin && !err; ++k) {
                s.nu = nu;
                s.tol_in = s.mode == 1 ? tin[k] : s.tol_in;
                s.v.x64 = x;
                s.v.b64 = (void*)b;
                cudaGraph_t g = nullptr;
                cudaGraphExec_t gx = nullptr;
                int fixed = 0;
                // the eager profiling mode runs the solve's loops from the
                // host (no capture); otherwise the solve is one graph
                if (!eager) {
                    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
                        err = 3;
                        break;
                    }
                    int e = bs_record(s, st, st2, &fixed);
                    cudaError_t ce = cudaStreamEndCapture(st, &g);
                    if (e || ce != cudaSuccess || cudaGraphInstantiate(&gx, g, 0) != cudaSuccess) {
                        if (g) cudaGraphDestroy(g);
                        err = e ? e : 3;
                        break;
                    }
                    cudaGraphDestroy(g);
                }
                BSGlobals zero;
                memset(&zero, 0, sizeof(zero));
                cudaMemcpyAsync(s.eg, &zero, sizeof(zero), cudaMemcpyHostToDevice, st);
                double total = 0.0;
                // one untimed solve, then the timed ones
                for (int r = -1; r < reps; ++r) {
                    k_bs_scale<<<1024, 256, 0, st>>>((double*)x, saved, 0.999, n);
                    cudaEventRecord(ea, st);
                    if (eager) {
                        const int e = bs_record(s, st, st2, &fixed);
                        if (e) {
                            err = e;
                            break;
                        }
                    } else {
                        cudaGraphLaunch(gx, st);
                    }
                    cudaEventRecord(eb, st);
                    if (cudaEventSynchronize(eb) != cudaSuccess) {
                        err = 3;
                        break;
                    }
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, ea, eb);
                    if (r >= 0) total += ms;
                }
                if (gx) cudaGraphExecDestroy(gx);
                if (err) break;
                BSGlobals hg;
                cudaMemcpy(&hg, s.eg, sizeof(hg), cudaMemcpyDeviceToHost);
                const double ms = total / std::max(1, reps);
                ++best.ncand;
                if (hg.status == 0 && ms < best.ms) best = BSTune{th, nu, s.tol_in, ms, best.ncand};
            }
            if (err) break;
        }
        if (err) break;
    }
    const int ncand = best.ncand;
    if (!err && best.th == 0) err = 10;  // no candidate converged
    best.ncand = ncand;
    if (!err) {
        if (best.th != s.th) err = bs_rebuild(s, best.th);
        s.nu = best.nu;
        s.tol_in = best.tol_in;
    }
    BSGlobals zero;
    memset(&zero, 0, sizeof(zero));
    if (s.eg) cudaMemcpyAsync(s.eg, &zero, sizeof(zero), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(x, saved, xbytes, cudaMemcpyDeviceToDevice, st);
    cudaStreamSynchronize(st);
    cudaFree(saved);
    cudaEventDestroy(ea);
    cudaEventDestroy(eb);
    if (out) *out = best;
    return err;
}

int bs_set_schedule(BatchSolver& s, int th, int nu, double tol_in)
{
    if ((th != 32 && th != 64) || (nu != 1 && nu != 2) || !(tol_in > 0 && tol_in < 1))
        return 1;
    if (th != s.th) {
        const int e = bs_rebuild(s, th);
        if (e) return e;
    }
    s.nu = nu;
    s.tol_in = tol_in;
    return 0;
}

void bs_free(BatchSolver& s)
{
    if (s.s3) {
        cudaStreamDestroy(s.s3);
        s.s3 = nullptr;
    }
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
    s.pipe = false;
    s.mmaps = nullptr;
    s.pring = nullptr;
}

}  // namespace f2d
