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

// true when the staged region of halo H around the tile at (J0, I0) lies
// inside the level (no periodic wrap, no out-of-level node)
template <int H, int W, int WY>
__device__ __forceinline__ bool region_inside(const MGLevel& L, int J0, int I0)
{
    return J0 - H >= 0 && J0 - H + WY <= L.nyn && I0 - H >= 0 && I0 - H + W <= L.nxn;
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

// Paired red-black layout of a staged region of WY rows x 2*PR columns: each
// row is cut into PR pairs of adjacent nodes (columns 2j, 2j+1), one of each
// colour; colour k's node of pair j of row r sits at packed index r*HWP + j
// of colour k's arrays. HWP = PR rounded up to even, so that packed index
// pairs (j, j+1), j even, are 8-byte (FP32) / 16-byte (FP64) aligned and a
// half sweep moves two nodes per shared-memory access. The padding slot of a
// row (when PR is odd) holds mask 0 and x 0. The x arrays of the two colours
// are 64 bytes apart modulo 128, so that a warp reading alternate colours of
// consecutive nodes touches each bank once. Layout: x red, x black, b red,
// b black, mask red, mask black.
template <typename S, int PR, int WY>
struct PRL {
    static constexpr int HWP = (PR + 1) / 2 * 2;
    static constexpr int NP = WY * HWP;
    static constexpr size_t CS = ((NP * sizeof(S) + 127) / 128) * 128 + 64;
    static constexpr size_t CM = ((NP + 127) / 128) * 128;
    static constexpr size_t BYTES = 4 * CS + 2 * CM;
};

template <typename S, int PR, int WY>
struct PRegion {
    unsigned char* base;
    using L = PRL<S, PR, WY>;
    __device__ __forceinline__ explicit PRegion(unsigned char* p) : base(p) {}
    __device__ __forceinline__ S* x(int k) const { return (S*)(base + k * L::CS); }
    __device__ __forceinline__ S* b(int k) const { return (S*)(base + (2 + k) * L::CS); }
    __device__ __forceinline__ uint8_t* m(int k) const { return base + 4 * L::CS + k * L::CM; }
};

template <typename S> struct Pair;
template <> struct Pair<float> { using T = float2; };
template <> struct Pair<double> { using T = double2; };

template <typename S>
__device__ __forceinline__ typename Pair<S>::T ld2(const S* p)
{
    return *reinterpret_cast<const typename Pair<S>::T*>(p);
}
template <typename S>
__device__ __forceinline__ void st2(S* p, S a, S b)
{
    typename Pair<S>::T v;
    v.x = a;
    v.y = b;
    *reinterpret_cast<typename Pair<S>::T*>(p) = v;
}
__device__ __forceinline__ unsigned ld_m2(const uint8_t* p)
{
    return *reinterpret_cast<const unsigned short*>(p);
}

// Stage a region whose first column is I0 - HX (HX odd) and first row
// J0 - HY, colour of region node (r, c) = (r + c + HX + HY) & 1 (the tile
// origin is even). Down leg (XA = false): b, the mask, and the pre-smoothing
// start x = b/diag on colour 0, x = 0 on colour 1. Up leg (XA = true, HY
// even): b, the mask, and x = xa + P (coarse x) from the staged coarse region
// sc2 (CW = PR + 1 columns from coarse column (I0-HX)>>1, rows from
// (J0-HY)>>1); bilinear P written as the average of two row averages, an
// even index repeating its node, so the weights 1, 1/2, 1/4 come out exactly.
// b and x are 0 at non-fluid nodes. A region inside the level is read in
// node pairs: node (J, I) of every level sits at an element index of the
// parity of I + 1 (odd level offsets, even pitches), so a pair that starts
// at the odd column I0 - HX + 2j starts on an even element (8/16-byte
// aligned). Regions that cross the level's edge (out-of-level nodes read as
// non-fluid 0, x-periodic levels wrap) go node by node.
template <typename S, int HX, int HY, int PR, int WY, bool XA>
__device__ __forceinline__ void stage_pairs(const PRegion<S, PR, WY>& R, const MGLevel& F,
                                            int J0, int I0, S id, const S* __restrict__ gxa,
                                            const S* __restrict__ sc2)
{
    static_assert(HX % 2 == 1, "the region starts on an odd column");
    static_assert(!XA || HY % 2 == 0, "the up leg's region starts on an even row");
    constexpr int HWP = PRL<S, PR, WY>::HWP, NPAIR = WY * PR, W = 2 * PR;
    constexpr int CP = (HX + HY) & 1, CW = PR + 1;
    const int t = tid256();
    const S* __restrict__ gb = lb<S>(F);
    if (HWP != PR && t < WY) {
        // padding slot of row t: mask 0, x 0, b 0
        const int q = t * HWP + PR;
        R.m(0)[q] = 0;
        R.m(1)[q] = 0;
        R.x(0)[q] = S(0);
        R.x(1)[q] = S(0);
        R.b(0)[q] = S(0);
        R.b(1)[q] = S(0);
    }
    const bool inner = J0 - HY >= 0 && J0 - HY + WY <= F.nyn && I0 - HX >= 0 &&
                       I0 - HX + W <= F.nxn;
    if (inner) {
        const long long base = F.off + (long long)(J0 - HY) * F.pitch + (I0 - HX);
        const int pitch = (int)F.pitch;
#pragma unroll
        for (int it = 0; it < (NPAIR + 255) / 256; ++it) {
            const int e = t + 256 * it;
            if (NPAIR % 256 != 0 && e >= NPAIR) break;
            const int r = e / PR, j = e - r * PR;
            const long long k = base + (r * pitch + 2 * j);
            const typename Pair<S>::T bv = ld2<S>(gb + k);
            const unsigned mv = ld_m2(F.m + k);
            const unsigned m0 = mv & 0xffu, m1 = mv >> 8;
            const S b0 = m0 ? bv.x : S(0), b1 = m1 ? bv.y : S(0);
            S x0, x1;
            if (XA) {
                // first node: odd column (between coarse columns j, j+1),
                // second: even column (on coarse column j+1); row r: on
                // coarse row r/2 (r even) or between r/2 and r/2 + 1
                const typename Pair<S>::T a = ld2<S>(gxa + k);
                const int qc = (r >> 1) * CW + j, oj = (r & 1) * CW;
                const S A = sc2[qc], B = sc2[qc + 1], Cc = sc2[qc + oj], D = sc2[qc + oj + 1];
                const S h0 = S(0.5) * (A + B), h1 = S(0.5) * (Cc + D);
                const S g0 = S(0.5) * (B + B), g1 = S(0.5) * (D + D);
                x0 = m0 ? a.x + S(0.5) * (h0 + h1) : S(0);
                x1 = m1 ? a.y + S(0.5) * (g0 + g1) : S(0);
            }
            const int q = r * HWP + j;
            // the pair's first node has colour (r + CP) & 1
            const bool f0 = ((r + CP) & 1) == 0;
            const S br = f0 ? b0 : b1;
            R.b(0)[q] = br;
            R.b(1)[q] = f0 ? b1 : b0;
            R.m(0)[q] = (uint8_t)(f0 ? m0 : m1);
            R.m(1)[q] = (uint8_t)(f0 ? m1 : m0);
            if (XA) {
                R.x(0)[q] = f0 ? x0 : x1;
                R.x(1)[q] = f0 ? x1 : x0;
            } else {
                R.x(0)[q] = br * id;
                R.x(1)[q] = S(0);
            }
        }
    } else {
        constexpr int N = WY * W;
        const int cj0 = (J0 - HY) >> 1, ci0 = (I0 - HX) >> 1;
#pragma unroll 4
        for (int e = t; e < N; e += 256) {
            const int r = e / W, c = e - r * W;
            const int J = J0 - HY + r, Iu = I0 - HX + c;
            int I = Iu;
            uint8_t mv = 0;
            S bv = S(0), xv = S(0);
            if (in_level(F, J, I)) {
                const long long k = nidx(F, J, I);
                mv = F.m[k];
                bv = gb[k];
                if (XA) xv = gxa[k];
            }
            bv = mv ? bv : S(0);
            const int col = (r + c + CP) & 1, q = r * HWP + (c >> 1);
            R.m(col)[q] = mv;
            R.b(col)[q] = bv;
            if (XA) {
                // coarse indices relative to the staged coarse region
                const int qc = ((J >> 1) - cj0) * CW + ((Iu >> 1) - ci0);
                const int oj = (J & 1) * CW, oi = Iu & 1;
                const S h0 = S(0.5) * (sc2[qc] + sc2[qc + oi]);
                const S h1 = S(0.5) * (sc2[qc + oj] + sc2[qc + oj + oi]);
                R.x(col)[q] = mv ? xv + S(0.5) * (h0 + h1) : S(0);
            } else {
                R.x(col)[q] = col == 0 ? bv * id : S(0);
            }
        }
    }
}

// Red-black half sweep of colour `col` on rows R0..R1 of a paired region
// (colour of node (r, c) = (r + c + CP) & 1): every node of that colour gets
// x = (b - offdiag(x)) / diag at fluid nodes, 0 elsewhere. A thread updates
// the two packed nodes j, j+1 (j even) of a row: in row rr the colour's nodes
// sit at columns 2j + p, p = (col + rr + CP) & 1, so their west/east
// neighbours are the other colour's packed nodes j-1+p, j+p, j+1+p (one
// pair load and one scalar load) and their north/south ones the other
// colour's packed pairs of rows rr -+ 1. Nodes within s of the region edge
// are updated from neighbours that are no longer exact; by induction the
// nodes at distance >= s from the edge are exact after half sweep s, and the
// callers sweep rows s .. WY-1-s only and read only exact nodes afterwards.
template <typename S, int PR, int WY, int CP, int R0, int R1>
__device__ __forceinline__ void sweep_pairs(const PRegion<S, PR, WY>& R, int col, S cx, S cy,
                                            S id)
{
    constexpr int HWP = PRL<S, PR, WY>::HWP, NPR = HWP / 2, n = (R1 - R0 + 1) * NPR;
    const int t = tid256();
    S* __restrict__ xo = R.x(col);
    const S* __restrict__ xn = R.x(col ^ 1);
    const S* __restrict__ bo = R.b(col);
    const uint8_t* __restrict__ mo = R.m(col);
#pragma unroll
    for (int it = 0; it < (n + 255) / 256; ++it) {
        const int e = t + 256 * it;
        if (n % 256 != 0 && e >= n) break;
        const int rr = R0 + e / NPR;
        const int q = rr * HWP + 2 * (e - (rr - R0) * NPR);
        const int p = (col + rr + CP) & 1;
        const typename Pair<S>::T a = ld2<S>(xn + q);
        const S sx = xn[p ? q + 2 : q - 1];
        const typename Pair<S>::T nn = ld2<S>(xn + q - HWP), ss = ld2<S>(xn + q + HWP);
        const typename Pair<S>::T bb = ld2<S>(bo + q);
        const unsigned mm = ld_m2(mo + q);
        const S w0 = p ? a.x : sx, e0 = p ? a.y : a.x;
        const S w1 = p ? a.y : a.x, e1 = p ? sx : a.y;
        const S v0 = (bb.x - (cx * (w0 + e0) + cy * (nn.x + ss.x))) * id;
        const S v1 = (bb.y - (cx * (w1 + e1) + cy * (nn.y + ss.y))) * id;
        st2<S>(xo + q, (mm & 0xffu) ? v0 : S(0), (mm >> 8) ? v1 : S(0));
    }
}

// residual r = b - A x at the colour-0 nodes of rows R0..R1 (in place of b;
// 0 at non-fluid nodes), two packed nodes per thread as in sweep_pairs
template <typename S, int PR, int WY, int CP, int R0, int R1>
__device__ __forceinline__ void residual_pairs(const PRegion<S, PR, WY>& R, S cx, S cy, S md)
{
    constexpr int HWP = PRL<S, PR, WY>::HWP, NPR = HWP / 2, n = (R1 - R0 + 1) * NPR;
    const int t = tid256();
    const S* __restrict__ xr = R.x(0);
    const S* __restrict__ xb = R.x(1);
    S* __restrict__ br = R.b(0);
    const uint8_t* __restrict__ mr = R.m(0);
#pragma unroll
    for (int it = 0; it < (n + 255) / 256; ++it) {
        const int e = t + 256 * it;
        if (n % 256 != 0 && e >= n) break;
        const int rr = R0 + e / NPR;
        const int q = rr * HWP + 2 * (e - (rr - R0) * NPR);
        const int p = (rr + CP) & 1;
        const typename Pair<S>::T c = ld2<S>(xr + q);
        const typename Pair<S>::T a = ld2<S>(xb + q);
        const S sx = xb[p ? q + 2 : q - 1];
        const typename Pair<S>::T ss = ld2<S>(xb + q - HWP), nn = ld2<S>(xb + q + HWP);
        const typename Pair<S>::T bb = ld2<S>(br + q);
        const unsigned mm = ld_m2(mr + q);
        const S w0 = p ? a.x : sx, e0 = p ? a.y : a.x;
        const S w1 = p ? a.y : a.x, e1 = p ? sx : a.y;
        const S r0 = bb.x - apply_diff<S>(cx, cy, md, c.x, w0, e0, ss.x, nn.x);
        const S r1 = bb.y - apply_diff<S>(cx, cy, md, c.y, w1, e1, ss.y, nn.y);
        st2<S>(br + q, (mm & 0xffu) ? r0 : S(0), (mm >> 8) ? r1 : S(0));
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

template <typename V>
__device__ __forceinline__ bool member_dot(V acc, double (&w)[1], double* partials,
                                           double* gpart, unsigned int* gtick,
                                           const BSInfo& in, unsigned int* ticket)
{
    block_dot<V>(acc, w);
    return seg_reduce2<1, std::is_same<V, float>::value>(w, partials, gpart, gtick, blockIdx.x,
                                                         in.n0, in.nn, in.g0, ticket);
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

// rz = <r, z> of a member, beta = rz / rz_old (0 on the first iteration of
// a loop); run by the thread that holds the member's total
__device__ __forceinline__ void set_rz(DevScalars& sc, int ir, double rz)
{
    const int first = ir ? sc.iter_in == 0 : sc.iter == 0;
    sc.beta = first ? 0.0 : rz / sc.rz;
    sc.rz = rz;
}

// ---- multigrid --------------------------------------------------------------
// Down leg of level l (l below the member's tail): pre-smoothing from a zero
// guess - red x = b/diag, black Gauss-Seidel, then NU-1 more (red, black)
// sweeps - and restriction of the residual to level l+1 (transpose of the
// bilinear prolongation). After a black half sweep the black residuals are
// zero, so only the red fine nodes (centre and corners of a coarse node)
// contribute. Writes the pre-smoothed x of the tile (to xa) and the coarse
// right-hand side of the coarse nodes whose centre lies in the tile. The
// staged region has a halo of 2NU+1 nodes (paired layout, PRL).
template <typename S, int NU, int TH>
__global__ void __launch_bounds__(256)
k_bs_down(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
          const MGLevel* __restrict__ levs, int l, const DevScalars* __restrict__ scs, int ir)
{
    constexpr int H = 2 * NU + 1, PR = (BS_TW + 2 * H) / 2, WY = TH + 2 * H, TQ = TH / 8;
    constexpr int HWP = PRL<S, PR, WY>::HWP;
    extern __shared__ __align__(128) unsigned char dsm[];
    const PRegion<S, PR, WY> R(dsm);
    const int4 tl = tiles[blockIdx.x];
    if (info[tl.x].ltail <= l || bs_skip(scs[tl.x], ir)) return;
    const MGLevel F = levs[tl.x * BS_LMAX + l];
    const int I0 = tl.y, J0 = tl.z, t = tid256();
    const S cx = Coef<S>::cx(F), cy = Coef<S>::cy(F), id = Coef<S>::idiag(F);
    stage_pairs<S, H, H, PR, WY, false>(R, F, J0, I0, id, nullptr, nullptr);
    __syncthreads();
    // black, then (red, black) NU-1 times; rows s .. WY-1-s at half sweep s
    sweep_pairs<S, PR, WY, 0, 1, WY - 2>(R, 1, cx, cy, id);
    __syncthreads();
    if constexpr (NU >= 2) {
        sweep_pairs<S, PR, WY, 0, 2, WY - 3>(R, 0, cx, cy, id);
        __syncthreads();
        sweep_pairs<S, PR, WY, 0, 3, WY - 4>(R, 1, cx, cy, id);
        __syncthreads();
    }
    // residual at the red nodes at distance >= 2 NU from the region edge
    // (exact there; all the restriction reads)
    residual_pairs<S, PR, WY, 0, 2 * NU, WY - 1 - 2 * NU>(R, cx, cy, Coef<S>::md(F));
    __syncthreads();
    {
        // coarse nodes with their centre in the tile: (TH/2) x (BS_TW/2);
        // the centre and its four diagonal neighbours are red
        const MGLevel C = levs[tl.x * BS_LMAX + l + 1];
        const S* __restrict__ br = R.b(0);
        static_assert((TH / 2) * (BS_TW / 2) % 256 == 0, "coarse nodes per thread");
#pragma unroll
        for (int k2 = 0; k2 < (TH / 2) * (BS_TW / 2) / 256; ++k2) {
            const int e = t + 256 * k2;
            const int a = e / (BS_TW / 2), b = e % (BS_TW / 2);
            const int cJ = (J0 >> 1) + a, cI = (I0 >> 1) + b;
            if (cJ < C.nyn && cI < C.nxn) {
                const long long k = nidx(C, cJ, cI);
                S v = S(0);
                if (C.m[k]) {
                    const int r0 = H + 2 * a, c0 = H + 2 * b;
                    // c0 odd: the corners (columns c0 -+ 1) are the red
                    // nodes of packed slots c0>>1 and c0>>1 + 1 of rows r0 -+ 1
                    const int qc = r0 * HWP + (c0 >> 1);
                    const int qn = qc - HWP, qs = qc + HWP;
                    const S c4 = (br[qn] + br[qn + 1]) + (br[qs] + br[qs + 1]);
                    v = br[qc] + S(0.25) * c4;
                }
                lb<S>(C)[k] = v;
            }
        }
    }
    S* xa = (S*)F.xa;
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr) {
        const int r = threadIdx.y + 8 * qr, c = threadIdx.x;
        const int J = J0 + r, I = I0 + c;
        if (J < F.nyn && I < F.nxn)
            xa[nidx(F, J, I)] = R.x((r + c) & 1)[(r + H) * HWP + ((c + H) >> 1)];
    }
}

// Up leg of level l: x = xa + P (coarse x), then NU (black, red)
// post-smoothing sweeps; writes x of the tile. The staged region has a halo
// of 2NU rows and 2NU+1 columns (the paired layout starts on the odd column
// I0-2NU-1); the coarse nodes it interpolates from (columns (I0-2NU-1)/2 ..,
// rows (J0-2NU)/2 ..) are staged first: 0 outside the coarse level and at
// non-fluid nodes, wrapped when x-periodic (an even fine period makes the
// wrapped fine node's coarse neighbours the wrapped coarse ones). On level 0
// (RZ) the block also forms its part of <r, z> (r = b, z = x) and the
// member's last block sets rz and beta.
template <typename S, int NU, bool RZ, int TH>
__global__ void __launch_bounds__(256)
k_bs_up(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
        const MGLevel* __restrict__ levs, int l, DevScalars* scs, int ir, double* partials,
        double* gpart, unsigned int* gtick)
{
    constexpr int HX = 2 * NU + 1, HY = 2 * NU, PR = (BS_TW + 2 * HX) / 2, WY = TH + 2 * HY;
    constexpr int CP = (HX + HY) & 1, TQ = TH / 8, HWP = PRL<S, PR, WY>::HWP;
    constexpr int CW = PR + 1, CWY = WY / 2 + 1, CN = CW * CWY, CIT = (CN + 255) / 256;
    extern __shared__ __align__(128) unsigned char dsm[];
    const PRegion<S, PR, WY> R(dsm);
    S* sc2 = (S*)(dsm + PRL<S, PR, WY>::BYTES);
    const int4 tl = tiles[blockIdx.x];
    DevScalars& sc = scs[tl.x];
    const BSInfo in = info[tl.x];
    if (in.ltail <= l || bs_skip(sc, ir)) return;
    const MGLevel F = levs[tl.x * BS_LMAX + l];
    const MGLevel C = levs[tl.x * BS_LMAX + l + 1];
    const int I0 = tl.y, J0 = tl.z, t = tid256();
    const int cj0 = (J0 - HY) >> 1, ci0 = (I0 - HX) >> 1;
    {
        const S* __restrict__ cxg = lx<S>(C);
#pragma unroll
        for (int k2 = 0; k2 < CIT; ++k2) {
            const int e = t + k2 * 256;
            if (e < CN) {
                const int r = e / CW, c = e - r * CW;
                int I = ci0 + c;
                S v = S(0);
                if (in_level(C, cj0 + r, I)) v = cxg[nidx(C, cj0 + r, I)];
                sc2[e] = v;
            }
        }
    }
    __syncthreads();
    const S cx = Coef<S>::cx(F), cy = Coef<S>::cy(F), id = Coef<S>::idiag(F);
    stage_pairs<S, HX, HY, PR, WY, true>(R, F, J0, I0, id, (const S*)F.xa, sc2);
    __syncthreads();
    // (black, red) NU times; rows s .. WY-1-s at half sweep s
    sweep_pairs<S, PR, WY, CP, 1, WY - 2>(R, 1, cx, cy, id);
    __syncthreads();
    sweep_pairs<S, PR, WY, CP, 2, WY - 3>(R, 0, cx, cy, id);
    __syncthreads();
    if constexpr (NU >= 2) {
        sweep_pairs<S, PR, WY, CP, 3, WY - 4>(R, 1, cx, cy, id);
        __syncthreads();
        sweep_pairs<S, PR, WY, CP, 4, WY - 5>(R, 0, cx, cy, id);
        __syncthreads();
    }
    S* x = lx<S>(F);
    S acc = S(0);
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr) {
        const int r = threadIdx.y + 8 * qr, c = threadIdx.x;
        const int J = J0 + r, I = I0 + c;
        const int col = (r + c + HX + HY + CP) & 1;
        const int q = (r + HY) * HWP + ((c + HX) >> 1);
        if (J < F.nyn && I < F.nxn) {
            const S xv = R.x(col)[q];
            x[nidx(F, J, I)] = xv;
            if (RZ) acc += R.b(col)[q] * xv;  // 0 at non-fluid nodes
        }
    }
    if (RZ) {
        double w[1];
        if (member_dot<S>(acc, w, partials, gpart, gtick, in, &sc.counter[2])) set_rz(sc, ir, w[0]);
    }
}

// Coarse levels of every member in one block each (tail_vcycle). A member
// whose level 0 is already in the tail also forms <r, z> here.
template <typename S>
__global__ void __launch_bounds__(1024)
k_bs_tail(const BSInfo* __restrict__ info, const MGLevel* __restrict__ levs, DevScalars* scs,
          int ir, int nu)
{
    const int b = blockIdx.x;
    DevScalars& sc = scs[b];
    if (bs_skip(sc, ir)) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ MGLevel sl[16];
    const BSInfo in = info[b];
    tail_vcycle<S>(&levs[b * BS_LMAX], in.ltail, in.nl, in.ksweeps, smem_raw, sl, nu);
    if (in.ltail != 0) return;
    const MGLevel D = sl[0];
    const int n = D.nyn * D.nxn;
    S acc = S(0);
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        if (D.m[k]) acc += ((const S*)D.b)[k] * ((const S*)D.x)[k];
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
// p = z (first iteration) or z + beta p_old, q = A p, <p, q>, alpha = rz/<p,q>.
// p is formed on the tile and a one-node halo (the halo redundantly, from
// z and p_old), so A p needs no second pass; p_old and p live in two
// buffers chosen by the parity of the member's iteration count (p_old of
// the halo belongs to other blocks and must not be overwritten meanwhile).
template <typename S, typename V, int TH>
__global__ void __launch_bounds__(256)
k_bs_pq(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
        const MGLevel* __restrict__ levs, const S* __restrict__ z, V* __restrict__ p0,
        V* __restrict__ p1, V* __restrict__ q, DevScalars* scs, double* partials, double* gpart,
        unsigned int* gtick, int ir)
{
    constexpr int H = 1, W = Reg<H, TH>::WX, N = Reg<H, TH>::N, IT = (N + 255) / 256;
    constexpr int TQ = TH / 8;
    __shared__ V sp[N];
    __shared__ uint8_t sm[N];
    const int4 tl = tiles[blockIdx.x];
    DevScalars& sc = scs[tl.x];
    if (bs_skip(sc, ir)) return;
    const BSInfo in = info[tl.x];
    const MGLevel L = levs[tl.x * BS_LMAX];
    const int it = ir ? sc.iter_in : sc.iter;
    const bool first = it == 0;
    const V* __restrict__ pold = (it & 1) ? p1 : p0;
    V* __restrict__ pnew = (it & 1) ? p0 : p1;
    const V beta = V(sc.beta);
    const int I0 = tl.y, J0 = tl.z, t = tid256();
#pragma unroll
    for (int k2 = 0; k2 < IT; ++k2) {
        const int e = t + k2 * 256;
        if (e < N) {
            const int r = e / W, c = e - r * W;
            const int J = J0 - H + r;
            int I = I0 - H + c;
            uint8_t mv = 0;
            V zv = V(0), pv = V(0);
            if (in_level(L, J, I)) {
                const long long k = nidx(L, J, I);
                mv = L.m[k];
                zv = V(z[k]);
                if (!first) pv = pold[k];
            }
            sm[e] = mv;
            sp[e] = mv ? (first ? zv : zv + beta * pv) : V(0);
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
    double w[1];
    if (member_dot<V>(acc, w, partials, gpart, gtick, in, &sc.counter[3])) {
        sc.pq = w[0];
        sc.alpha = sc.rz / w[0];
    }
}

// x += alpha p, r -= alpha q, rr = <r, r>, per-member convergence, loop
// condition. FP64 form: x is the solution. Refinement form: x is the inner
// correction e (started from 0) and convergence is relative to the round's
// starting residual.
template <typename V, int TH>
__global__ void __launch_bounds__(256)
k_bs_xr(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
        const MGLevel* __restrict__ levs, V* __restrict__ x, V* __restrict__ r,
        const V* __restrict__ p0, const V* __restrict__ p1, const V* __restrict__ q,
        DevScalars* scs, double* partials, double* gpart, unsigned int* gtick, BSGlobals* eg,
        cudaGraphConditionalHandle cond, int ir, int nmem)
{
    const int4 tl = tiles[blockIdx.x];
    DevScalars& sc = scs[tl.x];
    const BSInfo in = info[tl.x];
    bool mine = false;
    if (bs_skip(sc, ir)) {
        mine = threadIdx.x == 0 && threadIdx.y == 0 && (int)blockIdx.x == in.n0;
    } else {
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
                xv[qr] = first ? V(0) : x[k[qr]];
                pv[qr] = p[k[qr]];
                rv[qr] = r[k[qr]];
                qv[qr] = q[k[qr]];
            }
#pragma unroll
            for (int qr = 0; qr < QB; ++qr) {
                if (!ok[qr] || !mv[qr]) continue;
                if (zero) {
                    x[k[qr]] = V(0);
                    r[k[qr]] = V(0);
                    continue;
                }
                x[k[qr]] = xv[qr] + a * pv[qr];
                const V rn = rv[qr] - a * qv[qr];
                r[k[qr]] = rn;
                acc += rn * rn;
            }
        }
        double w[1];
        mine = member_dot<V>(acc, w, partials, gpart, gtick, in, &sc.counter[4]);
        if (mine) {
            sc.total_iters += 1;
            const bool bad = !(w[0] == w[0]);
            if (bad) atomicOr(&eg->status, ST_NONFINITE);
            if (ir) {
                sc.iter_in += 1;
                // a round stops at its relative tolerance, or as soon as its
                // residual is a tenth of what the whole solve must reach
                // (the last round of a solve needs only the digits missing,
                // not tol_in more)
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
    }
    if (members_done(mine, &eg->ticket[1], nmem)) {
        eg->loops_in += 1;
        const int act = ir ? *(volatile int*)&eg->active_in : *(volatile int*)&eg->active_out;
        if (cond) cudaGraphSetConditional(cond, act > 0 ? 1u : 0u);
    }
}

// FP64 residual r = b - A x of the tile (x staged with a one-node halo);
// the per-thread sums of b*b and r*r; optionally the FP32 copy of r.
template <int TH>
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
            rv = bv[qr] - apply_diff<double>(cx, cy, md, sx[e], sx[e - 1], sx[e + 1], sx[e - W],
                                             sx[e + W]);
            w[0] += bv[qr] * bv[qr];
            w[1] += rv * rv;
        }
        if (ok[qr]) {
            r[k[qr]] = rv;
            if (rin) rin[k[qr]] = float(rv);
        }
    }
}

// FP64 form: r = b - A x, <b,b>, <r,r>, per-member start state
template <int TH>
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
    residual64<TH>(tl, L, x, b, r, nullptr, w);
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
template <int TH>
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
        residual64<TH>(tl, L, x, b, r, rin, w);
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
template <int TH>
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
    constexpr int TQ = TH / 8;
    long long k[TQ];
    bool ok[TQ];
    uint8_t mv[TQ];
    double xv[TQ];
    float ev[TQ];
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr) {
        const int J = tl.z + threadIdx.y + 8 * qr, I = tl.y + threadIdx.x;
        ok[qr] = J < L.nyn && I < L.nxn;
        k[qr] = nidx(L, min(J, L.nyn - 1), min(I, L.nxn - 1));
        mv[qr] = L.m[k[qr]];
        xv[qr] = x[k[qr]];
        ev[qr] = e[k[qr]];
    }
#pragma unroll
    for (int qr = 0; qr < TQ; ++qr)
        if (ok[qr] && mv[qr]) x[k[qr]] = zero ? 0.0 : xv[qr] + (double)ev[qr];
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

// dynamic shared memory of the down and up kernels (staged region, coarse
// region, mask)
template <typename S, int NU, int TH>
static size_t down_smem()
{
    constexpr int H = 2 * NU + 1;
    return PRL<S, (BS_TW + 2 * H) / 2, TH + 2 * H>::BYTES;
}
template <typename S, int NU, int TH>
static size_t up_smem()
{
    constexpr int HX = 2 * NU + 1, HY = 2 * NU, PR = (BS_TW + 2 * HX) / 2, WY = TH + 2 * HY;
    constexpr size_t CN = (size_t)(PR + 1) * (WY / 2 + 1);
    return PRL<S, PR, WY>::BYTES + CN * sizeof(S);
}

template <typename S, int NU, int TH>
static int set_level_attrs()
{
    cudaError_t e = cudaFuncSetAttribute(k_bs_down<S, NU, TH>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)down_smem<S, NU, TH>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_bs_up<S, NU, false, TH>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)up_smem<S, NU, TH>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_bs_up<S, NU, true, TH>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)up_smem<S, NU, TH>());
    return (int)e;
}

// one V-cycle for all members still iterating: a down kernel per grid level,
// the tail, an up kernel per grid level (the level-0 one also forms <r, z>)
template <typename S, int NU, int TH>
static int vcycle_nu(BatchSolver& s, cudaStream_t st, int ir)
{
    const dim3 blk(32, 8);
    int cnt = 0;
    for (int l = 0; l < s.maxl; ++l) {
        k_bs_down<S, NU, TH><<<s.ntiles[l], blk, down_smem<S, NU, TH>(), st>>>(
            s.tiles[l], s.dinfo, s.dlevs, l, s.scs, ir);
        cnt += 1;
    }
    k_bs_tail<S><<<s.n, 1024, s.tail_smem, st>>>(s.dinfo, s.dlevs, s.scs, ir, NU);
    cnt += 1;
    for (int l = s.maxl - 1; l >= 1; --l) {
        k_bs_up<S, NU, false, TH><<<s.ntiles[l], blk, up_smem<S, NU, TH>(), st>>>(
            s.tiles[l], s.dinfo, s.dlevs, l, s.scs, ir, s.partials, s.gpart, s.gtick);
        cnt += 1;
    }
    if (s.maxl > 0) {
        k_bs_up<S, NU, true, TH><<<s.ntiles[0], blk, up_smem<S, NU, TH>(), st>>>(
            s.tiles[0], s.dinfo, s.dlevs, 0, s.scs, ir, s.partials, s.gpart, s.gtick);
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
    V* x = (V*)(ir ? s.v.e : s.v.x64);
    int cnt = vcycle<S, TH>(s, st, ir);
    k_bs_pq<S, V, TH><<<nt, blk, 0, st>>>(s.rtiles, s.dinfo, s.dlevs, (const S*)s.v.z,
                                          (V*)s.v.p, (V*)s.v.p2, (V*)s.v.q, s.scs, s.partials,
                                          s.gpart, s.gtick, ir);
    k_bs_xr<V, TH><<<nt, blk, 0, st>>>(s.rtiles, s.dinfo, s.dlevs, x, r, (const V*)s.v.p,
                                       (const V*)s.v.p2, (const V*)s.v.q, s.scs, s.partials,
                                       s.gpart, s.gtick, s.eg, cond, ir, s.n);
    cnt += 2;
    s.body_launches = cnt;
    return (int)cudaGetLastError();
}


static int read_globals(const BatchSolver& s, cudaStream_t st, BSGlobals* h)
{
    cudaError_t e = cudaMemcpyAsync(h, s.eg, sizeof(*h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return (int)e;
}

template <int TH>
static int bs_record_t(BatchSolver& s, cudaStream_t st, cudaStream_t st2, int* launches)
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
        k_bs_init<TH><<<nt, blk, 0, st>>>(s.rtiles, s.dinfo, s.dlevs, (const double*)s.v.x64,
                                      (const double*)s.v.b64, (double*)s.v.r64, s.scs,
                                      s.partials, s.gpart, s.gtick, s.eg, cond, s.n);
        fixed += 1;
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
    k_bs_refine<TH><<<nt, blk, 0, st>>>(s.rtiles, s.dinfo, s.dlevs, (const double*)s.v.x64,
                                    (const double*)s.v.b64, (double*)s.v.r64, (float*)s.v.rin,
                                    s.scs, s.partials, s.gpart, s.gtick, s.eg, 1, cond_o,
                                    s.n);
    fixed += 2;
    auto round_tail = [&](cudaStream_t sb) {
        k_bs_correct<TH><<<nt, blk, 0, sb>>>(s.rtiles, s.dlevs, (double*)s.v.x64,
                                         (const float*)s.v.e, s.scs);
        k_bs_reset<<<1, 1, 0, sb>>>(s.eg);
        k_bs_refine<TH><<<nt, blk, 0, sb>>>(s.rtiles, s.dinfo, s.dlevs, (const double*)s.v.x64,
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

template <typename S, int NU, int TH>
static void launch_down0(BatchSolver& s, cudaStream_t st, int ir)
{
    k_bs_down<S, NU, TH><<<s.ntiles[0], dim3(32, 8), down_smem<S, NU, TH>(), st>>>(
        s.tiles[0], s.dinfo, s.dlevs, 0, s.scs, ir);
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
        const bool two = s.nu >= 2, big = s.th == 64;
        if (s.mode == 0) {
            if (two) big ? launch_down0<double, 2, 64>(s, st, ir) : launch_down0<double, 2, 32>(s, st, ir);
            else big ? launch_down0<double, 1, 64>(s, st, ir) : launch_down0<double, 1, 32>(s, st, ir);
        } else {
            if (two) big ? launch_down0<float, 2, 64>(s, st, ir) : launch_down0<float, 2, 32>(s, st, ir);
            else big ? launch_down0<float, 1, 64>(s, st, ir) : launch_down0<float, 1, 32>(s, st, ir);
        }
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
    // Tile tables of 32 x TH nodes. Level 0 (all members; the Krylov
    // kernels and the first multigrid level) with the members' reduction
    // groups of RED_GROUP tiles; level l >= 1 for the members whose grid
    // levels reach below it. Tiles without a fluid node are left out (their
    // nodes stay 0 in every vector), but every member keeps at least one
    // level-0 tile for its reductions.
    auto has_fluid = [&](int b, int l, int J0, int I0) {
        const std::vector<uint8_t>& hm = s.mg[b].hmask[l];
        const MGLevel& L = levs[(size_t)b * BS_LMAX + l];
        for (int J = J0; J < std::min(L.nyn, J0 + TH); ++J)
            for (int I = I0; I < std::min(L.nxn, I0 + BS_TW); ++I)
                if (hm[(size_t)J * L.nxn + I]) return true;
        return false;
    };
    std::vector<std::vector<int4>> tiles(std::max(1, s.maxl));
    std::vector<int4>& rt = tiles[0];
    int ngroups = 0;
    for (int b = 0; b < s.n; ++b) {
        const MGLevel& L = levs[(size_t)b * BS_LMAX];
        info[b].n0 = (int)rt.size();
        for (int J0 = 0; J0 < L.nyn; J0 += TH)
            for (int I0 = 0; I0 < L.nxn; I0 += BS_TW)
                if (has_fluid(b, 0, J0, I0)) rt.push_back(make_int4(b, I0, J0, 0));
        if ((int)rt.size() == info[b].n0) rt.push_back(make_int4(b, 0, 0, 0));
        info[b].nn = (int)rt.size() - info[b].n0;
        info[b].g0 = ngroups;
        ngroups += (info[b].nn + RED_GROUP - 1) / RED_GROUP;
    }
    for (int l = 1; l < s.maxl; ++l)
        for (int b = 0; b < s.n; ++b) {
            if (info[b].ltail <= l) continue;
            const MGLevel& L = levs[(size_t)b * BS_LMAX + l];
            for (int J0 = 0; J0 < L.nyn; J0 += TH)
                for (int I0 = 0; I0 < L.nxn; I0 += BS_TW)
                    if (has_fluid(b, l, J0, I0)) tiles[l].push_back(make_int4(b, I0, J0, 0));
        }
    auto dal = [&](size_t bytes) -> void* {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        s.owned.push_back(p);
        return p;
    };
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
    // The dynamic shared-memory limit is an attribute of the tail kernel, not
    // of this solver: raise it to the largest tail any solver of the process
    // needs and never lower it, or the launches (and new graph captures) of
    // an existing solver with a larger tail would fail. (One host thread and
    // one device per process, as everywhere in this library.)
    static bool level_attrs = false;  // constant per kernel instantiation: once
    if (!level_attrs) {
        if (set_level_attrs<float, 1, 32>() || set_level_attrs<float, 2, 32>() ||
            set_level_attrs<double, 1, 32>() || set_level_attrs<double, 2, 32>() ||
            set_level_attrs<float, 1, 64>() || set_level_attrs<float, 2, 64>() ||
            set_level_attrs<double, 1, 64>() || set_level_attrs<double, 2, 64>())
            return 4;
        level_attrs = true;
    }
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
    const double tin[3] = {1e-6, 1e-5, 1e-4};
    const int ntin = s.mode == 1 ? 3 : 1;
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
}

}  // namespace f2d
