// Register-blocked multigrid level kernels (the V-cycle's down and up legs
// on every grid level finer than a member's tail), used by solver.cu in the
// FP64 form and where the pipelined FP32 kernels (mg_pipe.cuh) do not apply.
//
// A block stages a region of MR_WY x MR_W nodes (a tile of MR_TH x MR_TW
// nodes and a halo of MR_H nodes) in registers: warp w holds region rows
// w*MR_R .. w*MR_R + MR_R-1, lane L holds columns 2L and 2L+1 of them. A
// red-black half sweep then updates one colour from the other colour's
// values: the west/east neighbours in the thread's own registers or the
// adjacent lane's (one warp shuffle per row), the north/south ones in the
// thread's registers, except the first and last row of a warp's strip, which
// come from the neighbouring warps through a small shared-memory exchange
// (double-buffered by half sweep, one barrier per half sweep). The region is
// loaded once (node pairs, coalesced rows) and no node value makes a
// shared-memory round trip inside a sweep. Nodes within s of the region edge
// are updated from neighbours that are no longer exact (or from 0 outside the
// region); by induction the nodes at distance >= s from the edge are exact
// after half sweep s, and only those are used afterwards: the halo of 5 nodes
// covers the down leg's 2NU-1 half sweeps and residual and the up leg's 2NU
// half sweeps for NU <= 2.
#pragma once
#include "mg_ops.cuh"
#include "solver.cuh"

namespace f2d {

constexpr int MR_R = 10;                  // region rows per warp (even)
constexpr int MR_NW = 8;                  // warps per block
constexpr int MR_W = 64;                  // region columns (2 per lane)
constexpr int MR_WY = MR_R * MR_NW;       // region rows
constexpr int MR_H = 5;                   // halo (odd: the region starts on an odd column)
constexpr int MR_TW = MR_W - 2 * MR_H;    // tile columns (54)
constexpr int MR_TH = MR_WY - 2 * MR_H;   // tile rows (70)
static_assert(MR_R % 2 == 0 && MR_H % 2 == 1 && MR_TW % 2 == 0 && MR_TH % 2 == 0,
              "region geometry");

template <typename S> struct MRPair;
template <> struct MRPair<float> { using T = float2; };
template <> struct MRPair<double> { using T = double2; };

// The thread's part of a staged region: rows w*MR_R + i, columns 2L + j.
template <typename S>
struct MRRegs {
    S x[MR_R][2];
    S b[MR_R][2];
    unsigned m;  // fluid flags, bit 2i + j
};

// Load b and the mask of the thread's nodes; the region's first row is
// J0 - MR_H, its first column I0 - MR_H (odd, so a lane's node pair starts
// on an even element of every level: 8/16-byte aligned). Out-of-level nodes
// are non-fluid 0; x-periodic levels wrap. XA: also xa into x (up leg).
template <typename S, bool XA>
__device__ __forceinline__ void mr_load(MRRegs<S>& R, const MGLevel& F, int J0, int I0)
{
    const int L = threadIdx.x, w = threadIdx.y;
    const int RJ = J0 - MR_H, RI = I0 - MR_H;
    const S* __restrict__ gb = lb<S>(F);
    const S* __restrict__ gx = (const S*)F.xa;
    R.m = 0u;
    const bool inner = RJ >= 0 && RJ + MR_WY <= F.nyn && RI >= 0 && RI + MR_W <= F.nxn;
    if (inner) {
        const long long base = F.off + (long long)(RJ + w * MR_R) * F.pitch + RI + 2 * L;
#pragma unroll
        for (int i = 0; i < MR_R; ++i) {
            const long long k = base + (long long)i * F.pitch;
            const typename MRPair<S>::T bv = *reinterpret_cast<const typename MRPair<S>::T*>(gb + k);
            const unsigned mv = *reinterpret_cast<const unsigned short*>(F.m + k);
            const unsigned m0 = mv & 0xffu, m1 = mv >> 8;
            R.b[i][0] = m0 ? bv.x : S(0);
            R.b[i][1] = m1 ? bv.y : S(0);
            R.m |= (m0 ? 1u : 0u) << (2 * i);
            R.m |= (m1 ? 1u : 0u) << (2 * i + 1);
            if (XA) {
                const typename MRPair<S>::T xv =
                    *reinterpret_cast<const typename MRPair<S>::T*>(gx + k);
                R.x[i][0] = m0 ? xv.x : S(0);
                R.x[i][1] = m1 ? xv.y : S(0);
            }
        }
    } else {
#pragma unroll
        for (int i = 0; i < MR_R; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int J = RJ + w * MR_R + i;
                int I = RI + 2 * L + j;
                uint8_t mv = 0;
                S bv = S(0), xv = S(0);
                if (in_level(F, J, I)) {
                    const long long k = nidx(F, J, I);
                    mv = F.m[k];
                    bv = gb[k];
                    if (XA) xv = gx[k];
                }
                R.b[i][j] = mv ? bv : S(0);
                R.m |= (mv ? 1u : 0u) << (2 * i + j);
                if (XA) R.x[i][j] = mv ? xv : S(0);
            }
    }
}

// Publish the first and last row of the warp's strip (both columns of every
// lane) into exchange buffer `buf`.
template <typename S>
__device__ __forceinline__ void mr_publish(const MRRegs<S>& R, S (*xch)[MR_NW][2][MR_W], int buf)
{
    const int L = threadIdx.x, w = threadIdx.y;
    typename MRPair<S>::T top, bot;
    top.x = R.x[0][0];
    top.y = R.x[0][1];
    bot.x = R.x[MR_R - 1][0];
    bot.y = R.x[MR_R - 1][1];
    *reinterpret_cast<typename MRPair<S>::T*>(&xch[buf][w][0][2 * L]) = top;
    *reinterpret_cast<typename MRPair<S>::T*>(&xch[buf][w][1][2 * L]) = bot;
}

// The north (row r-1) and south (row r+1) values of column j of the thread's
// row i: registers, or the neighbouring warps' published rows (0 outside the
// region).
template <typename S, int I, int J>
__device__ __forceinline__ void mr_ns(const MRRegs<S>& R, S (*xch)[MR_NW][2][MR_W], int buf,
                                      S& up, S& dn)
{
    const int L = threadIdx.x, w = threadIdx.y;
    if constexpr (I > 0) up = R.x[I - 1][J];
    else up = w > 0 ? xch[buf][w - 1][1][2 * L + J] : S(0);
    if constexpr (I < MR_R - 1) dn = R.x[I + 1][J];
    else dn = w < MR_NW - 1 ? xch[buf][w + 1][0][2 * L + J] : S(0);
}

// West/east neighbours of the node of column j of row i: the other column
// of the pair, or the adjacent lane's (0 outside the region).
template <typename S, int I, int J>
__device__ __forceinline__ void mr_we(const MRRegs<S>& R, S& we, S& ea)
{
    const int L = threadIdx.x;
    if constexpr (J == 0) {
        const S v = __shfl_up_sync(0xffffffffu, R.x[I][1], 1);
        we = L > 0 ? v : S(0);
        ea = R.x[I][1];
    } else {
        const S v = __shfl_down_sync(0xffffffffu, R.x[I][0], 1);
        we = R.x[I][0];
        ea = L < 31 ? v : S(0);
    }
}

// Red-black half sweep of colour COL over the thread's rows: the node of
// colour COL in region row r is column (r + COL) & 1 of the lane's pair
// (region row parity = parity of i, MR_R even), so every index is a
// compile-time constant.
template <typename S, int COL, int I = 0>
__device__ __forceinline__ void mr_sweep_rows(MRRegs<S>& R, S (*xch)[MR_NW][2][MR_W], int buf,
                                              S cx, S cy, S id)
{
    if constexpr (I < MR_R) {
        constexpr int J = (I + COL) & 1;
        S we, ea, up, dn;
        mr_we<S, I, J>(R, we, ea);
        mr_ns<S, I, J>(R, xch, buf, up, dn);
        const S v = (R.b[I][J] - (cx * (we + ea) + cy * (up + dn))) * id;
        R.x[I][J] = (R.m >> (2 * I + J)) & 1u ? v : S(0);
        mr_sweep_rows<S, COL, I + 1>(R, xch, buf, cx, cy, id);
    }
}

template <typename S, int COL>
__device__ __forceinline__ void mr_half_sweep(MRRegs<S>& R, S (*xch)[MR_NW][2][MR_W], int buf,
                                              S cx, S cy, S id)
{
    mr_publish<S>(R, xch, buf);
    __syncthreads();
    mr_sweep_rows<S, COL>(R, xch, buf, cx, cy, id);
}

// residual b - A x of the red nodes of the thread's rows into rs[r][L]
// (0 at non-fluid nodes); the red node of row r is column r & 1 of the pair
template <typename S, int I = 0>
__device__ __forceinline__ void mr_residual_rows(const MRRegs<S>& R, S (*xch)[MR_NW][2][MR_W],
                                                 int buf, S cx, S cy, S md, S (*rs)[32])
{
    if constexpr (I < MR_R) {
        constexpr int J = I & 1;
        S we, ea, up, dn;
        mr_we<S, I, J>(R, we, ea);
        mr_ns<S, I, J>(R, xch, buf, up, dn);
        const S v = R.b[I][J] - apply_diff<S>(cx, cy, md, R.x[I][J], we, ea, up, dn);
        rs[threadIdx.y * MR_R + I][threadIdx.x] = (R.m >> (2 * I + J)) & 1u ? v : S(0);
        mr_residual_rows<S, I + 1>(R, xch, buf, cx, cy, md, rs);
    }
}

// Write x of the thread's tile nodes (rows and columns MR_H .. of the region)
// to the level array y; RZ: the thread's sum of b x over them.
template <typename S, bool RZ>
__device__ __forceinline__ S mr_store(const MRRegs<S>& R, const MGLevel& F, S* __restrict__ y,
                                      int J0, int I0)
{
    const int L = threadIdx.x, w = threadIdx.y;
    S acc = S(0);
#pragma unroll
    for (int i = 0; i < MR_R; ++i) {
        const int r = w * MR_R + i;
        const int J = J0 - MR_H + r;
        if (r < MR_H || r >= MR_H + MR_TH || J >= F.nyn) continue;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int c = 2 * L + j;
            const int I = I0 - MR_H + c;
            if (c < MR_H || c >= MR_H + MR_TW || I >= F.nxn) continue;
            y[nidx(F, J, I)] = R.x[i][j];
            if (RZ) acc += R.b[i][j] * R.x[i][j];  // 0 at non-fluid nodes
        }
    }
    return acc;
}

// Down leg of level l (l below the member's tail), one tile per block:
// pre-smoothing from a zero guess (red x = b/diag, black, then NU-1 more
// (red, black) sweeps), the residual at the red nodes and its restriction
// to level l+1 (transpose of the bilinear prolongation; after a black half
// sweep the black residuals are zero, so only the red centre and corners of
// a coarse node contribute). Writes the pre-smoothed x of the tile (xa) and
// the coarse right-hand side of the coarse nodes whose centre lies in the
// tile.
template <typename S, int NU>
__global__ void __launch_bounds__(256)
k_mg_down(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
          const MGLevel* __restrict__ levs, int l, const DevScalars* __restrict__ scs, int ir)
{
    __shared__ __align__(16) S xch[2][MR_NW][2][MR_W];
    __shared__ S rs[MR_WY][32];
    const int4 tl = tiles[blockIdx.x];
    if (info[tl.x].ltail <= l || bs_skip(scs[tl.x], ir)) return;
    const MGLevel F = levs[tl.x * BS_LMAX + l];
    const int I0 = tl.y, J0 = tl.z;
    const S cx = Coef<S>::cx(F), cy = Coef<S>::cy(F), id = Coef<S>::idiag(F);
    MRRegs<S> R;
    mr_load<S, false>(R, F, J0, I0);
#pragma unroll
    for (int i = 0; i < MR_R; ++i) {
        // red (the column i & 1 of the pair) from a zero guess
        R.x[i][i & 1] = R.b[i][i & 1] * id;
        R.x[i][(i & 1) ^ 1] = S(0);
    }
    mr_half_sweep<S, 1>(R, xch, 0, cx, cy, id);
    if constexpr (NU >= 2) {
        mr_half_sweep<S, 0>(R, xch, 1, cx, cy, id);
        mr_half_sweep<S, 1>(R, xch, 0, cx, cy, id);
    }
    mr_publish<S>(R, xch, 1);
    __syncthreads();
    mr_residual_rows<S>(R, xch, 1, cx, cy, Coef<S>::md(F), rs);
    __syncthreads();
    {
        // coarse nodes with their centre in the tile; centre (r0, c0) and
        // corners are red: row r0 odd, column c0 = 2 L0 + 1 (slot L0 of rs),
        // corner rows even, columns 2 L0 and 2 L0 + 2 (slots L0, L0 + 1)
        const MGLevel C = levs[tl.x * BS_LMAX + l + 1];
        constexpr int CX = MR_TW / 2, NC = (MR_TH / 2) * CX;
        const int t = threadIdx.y * 32 + threadIdx.x;
        for (int e = t; e < NC; e += 256) {
            const int a = e / CX, bb = e - a * CX;
            const int cJ = (J0 >> 1) + a, cI = (I0 >> 1) + bb;
            if (cJ < C.nyn && cI < C.nxn) {
                const long long k = nidx(C, cJ, cI);
                S v = S(0);
                if (C.m[k]) {
                    const int r0 = MR_H + 2 * a, L0 = (MR_H - 1) / 2 + bb;
                    const S c4 = (rs[r0 - 1][L0] + rs[r0 - 1][L0 + 1]) +
                                 (rs[r0 + 1][L0] + rs[r0 + 1][L0 + 1]);
                    v = rs[r0][L0] + S(0.25) * c4;
                }
                lb<S>(C)[k] = v;
            }
        }
    }
    mr_store<S, false>(R, F, (S*)F.xa, J0, I0);
}

// Up leg of level l: x = xa + P (coarse x), then NU (black, red)
// post-smoothing sweeps; writes x of the tile. The coarse nodes the region
// interpolates from are staged in shared memory first: 0 outside the coarse
// level and at non-fluid nodes, wrapped when x-periodic (an even fine period
// makes the wrapped fine node's coarse neighbours the wrapped coarse ones).
// On level 0 (RZ) the block also forms its tile's part of <r, z> (r = b,
// z = x) into tpart[tile] (k_bs_rz sums a member's tiles).
template <typename S, int NU, bool RZ>
__global__ void __launch_bounds__(256)
k_mg_up(const int4* __restrict__ tiles, const BSInfo* __restrict__ info,
        const MGLevel* __restrict__ levs, int l, DevScalars* scs, int ir, double* tpart)
{
    constexpr int CW = MR_W / 2 + 1, CWY = MR_WY / 2 + 1;
    __shared__ __align__(16) S xch[2][MR_NW][2][MR_W];
    __shared__ S sc2[CWY][CW];
    const int4 tl = tiles[blockIdx.x];
    DevScalars& sc = scs[tl.x];
    const BSInfo in = info[tl.x];
    if (in.ltail <= l || bs_skip(sc, ir)) return;
    const MGLevel F = levs[tl.x * BS_LMAX + l];
    const MGLevel C = levs[tl.x * BS_LMAX + l + 1];
    const int I0 = tl.y, J0 = tl.z, t = threadIdx.y * 32 + threadIdx.x;
    {
        // region row r (node J0-5+r, J0-5 odd) lies on coarse rows
        // cj0 + (r+1)/2 (and + 1 when r is even); column c on coarse columns
        // ci0 + (c+1)/2 (and + 1 when c is even)
        const int cj0 = (J0 - MR_H) >> 1, ci0 = (I0 - MR_H) >> 1;
        const S* __restrict__ cxg = lx<S>(C);
        for (int e = t; e < CWY * CW; e += 256) {
            const int r = e / CW, c = e - r * CW;
            int I = ci0 + c;
            S v = S(0);
            if (in_level(C, cj0 + r, I)) v = cxg[nidx(C, cj0 + r, I)];
            sc2[r][c] = v;
        }
    }
    MRRegs<S> R;
    mr_load<S, true>(R, F, J0, I0);
    __syncthreads();
    {
        // x += P (coarse x) at the fluid nodes: bilinear, written as the
        // average of two row averages (an even index repeats its node, so the
        // weights 1, 1/2, 1/4 come out exactly). Rows of the thread: coarse
        // rows 5w .. 5w + 5, columns L (oi = 1) and L + 1.
        const int L = threadIdx.x, w = threadIdx.y;
        S cv[MR_R / 2 + 1][2];
#pragma unroll
        for (int q = 0; q <= MR_R / 2; ++q) {
            cv[q][0] = sc2[w * (MR_R / 2) + q][L];
            cv[q][1] = sc2[w * (MR_R / 2) + q][L + 1];
        }
#pragma unroll
        for (int i = 0; i < MR_R; ++i) {
            const int lr = (1 + i) >> 1, oj = (1 + i) & 1;
            // column 2L: between coarse columns L and L+1
            const S h0 = S(0.5) * (cv[lr][0] + cv[lr][1]);
            const S h1 = S(0.5) * (cv[lr + oj][0] + cv[lr + oj][1]);
            // column 2L+1: on coarse column L+1
            const S g0 = S(0.5) * (cv[lr][1] + cv[lr][1]);
            const S g1 = S(0.5) * (cv[lr + oj][1] + cv[lr + oj][1]);
            R.x[i][0] += (R.m >> (2 * i)) & 1u ? S(0.5) * (h0 + h1) : S(0);
            R.x[i][1] += (R.m >> (2 * i + 1)) & 1u ? S(0.5) * (g0 + g1) : S(0);
        }
    }
    mr_half_sweep<S, 1>(R, xch, 0, Coef<S>::cx(F), Coef<S>::cy(F), Coef<S>::idiag(F));
    mr_half_sweep<S, 0>(R, xch, 1, Coef<S>::cx(F), Coef<S>::cy(F), Coef<S>::idiag(F));
    if constexpr (NU >= 2) {
        mr_half_sweep<S, 1>(R, xch, 0, Coef<S>::cx(F), Coef<S>::cy(F), Coef<S>::idiag(F));
        mr_half_sweep<S, 0>(R, xch, 1, Coef<S>::cx(F), Coef<S>::cy(F), Coef<S>::idiag(F));
    }
    const S acc = mr_store<S, RZ>(R, F, lx<S>(F), J0, I0);
    if (RZ) {
        const double tot = block_sum<S>(acc);
        if (t == 0) tpart[blockIdx.x] = tot;
    }
}

}  // namespace f2d
