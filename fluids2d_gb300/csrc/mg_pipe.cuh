// Pipelined FP32 multigrid level kernels: the down and up legs of the
// V-cycle on the grid levels finer than a member's tail, in the FP32 refinement
// form (solver.cu launches them when the level arrays pass the layout checks
// of bs_build; the FP64 form and the other cases keep mg_reg.cuh's kernels).
//
// Same smoothing arithmetic and region geometry as mg_reg.cuh (a block
// smooths a tile of MR_TH x MR_TW nodes from a region of MR_WY x MR_W nodes
// held in registers, MR_R rows per warp, two columns per lane), organised
// around the latency of the loads, which bound the one-tile-per-block form:
// * persistent blocks walk the level's tile table with the grid's stride;
//   while a block smooths tile k from registers, the TMA engine stages tile
//   k + stride in shared memory: b, the fluid mask and, for the up leg, xa
//   and the coarse x the tile interpolates from (2D tensor loads), with the
//   fine and coarse level descriptors (one 1D bulk copy), all completing on
//   one mbarrier (bounded wait);
// * a tile's region goes from shared memory to registers first, which frees
//   the staging buffer for the next tile's loads;
// * the sweeps carry bid = b/diag, so a Gauss-Seidel update is two adds and
//   two FMAs, and the residual is diag (GS update - x);
// * the restriction reads the residual from registers (a shuffle for the
//   east corners, one shared row per warp for the strip's last row) and
//   takes the coarse node's fluid flag from its fine centre node, which is
//   how mg.cu builds the coarse masks (bs_build checks it);
// * neighbours outside the region are whatever value is at hand (a lane's
//   own value in the region's side columns, 0 above and below it): like the
//   halo nodes themselves they reach only halo nodes, which are never stored.
//
// Level arrays are 2D tensors for the TMA: rows of `pitch` elements starting
// at the row of node (0, 0), nyn rows, node (J, I) at (c0 + I, J) with c0 =
// off mod 16 (3 on level 0, the model arrays' halo; 1 on coarse levels).
// Elements outside the tensor read as 0, mask bytes of a row outside its
// node columns are 0 (checked by bs_build), so the tiles at a level's closed
// edges need no special case; a region that wraps around an x-periodic
// level (MP_SLOW) is loaded element by element.
#pragma once
#include "mg_reg.cuh"

namespace f2d {

constexpr int MP_BW = MR_W + 4;          // staged columns of b and xa (x aligned down to 4)
constexpr int MP_MW = MR_W + 16;         // staged mask columns (x aligned down to 16)
constexpr int MP_CH = MR_WY / 2 + 1;     // staged coarse rows
constexpr int MP_CW = MR_W / 2 + 1 + 3;  // staged coarse columns (x aligned down to 4)
constexpr int MP_SLOW = 1 << 8;          // tile flag (.w): region wraps around the level
enum { MP_B = 0, MP_M = 1, MP_XA = 2, MP_X = 3, MP_NMAP = 4 };  // maps per member and level
constexpr uint32_t MP_BYTES_B = MR_WY * MP_BW * 4;
constexpr uint32_t MP_BYTES_M = MR_WY * MP_MW;
constexpr uint32_t MP_BYTES_C = MP_CH * MP_CW * 4;
static_assert(sizeof(MGLevel) == 128, "level descriptors travel as one 256-byte bulk copy");
static_assert(MP_BW * 4 % 16 == 0 && MP_MW % 16 == 0 && MP_CW * 4 % 16 == 0,
              "TMA box rows are multiples of 16 bytes");

struct MPDown {
    alignas(128) float b[MR_WY][MP_BW];
    alignas(128) uint8_t m[MR_WY][MP_MW];
    alignas(16) MGLevel lv[2][2];  // [slot][fine, coarse]
    int4 rec[2];                   // tile record of each slot
    int skip[2];                   // the slot's member is not iterating
    uint64_t bar;
};
struct MPUp {
    alignas(128) float b[MR_WY][MP_BW];
    alignas(128) float xa[MR_WY][MP_BW];
    alignas(128) uint8_t m[MR_WY][MP_MW];
    alignas(128) float c[MP_CH][MP_CW];
    alignas(16) MGLevel lv[2][2];
    int4 rec[2];
    int skip[2];
    uint64_t bar;
};

typedef float (*MPX)[MR_NW + 2][2][MR_W];  // exchange rows: [buffer][warp + 1][top, bottom][col]

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Thread 0: stage tile `tl` of level l into slot `slot` (descriptors) and the
// staging buffer (region), on st.bar.
template <bool UP, typename ST>
__device__ __forceinline__ void mp_issue(ST& st, int slot, int4 tl, const MGLevel* levs,
                                         const CUtensorMap* maps, int l)
{
    const size_t li = (size_t)tl.x * BS_LMAX + l;
    const bool fast = !(tl.w & MP_SLOW);
    // the staging buffer may hold generic-proxy writes (the MP_SLOW path)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    uint32_t bytes = 2 * sizeof(MGLevel);
    if (fast) bytes += MP_BYTES_B + MP_BYTES_M + (UP ? MP_BYTES_B + MP_BYTES_C : 0u);
    mbar_expect_tx(&st.bar, bytes);
    bulk_load(&st.lv[slot][0], levs + li, 2 * sizeof(MGLevel), &st.bar);
    if (fast) {
        const int gx = (tl.w & 0xff) + tl.y - MR_H, gy = tl.z - MR_H;
        const CUtensorMap* mp = maps + li * MP_NMAP;
        tma_load_2d(&st.b[0][0], mp + MP_B, gx & ~3, gy, &st.bar);
        tma_load_2d(&st.m[0][0], mp + MP_M, gx & ~15, gy, &st.bar);
        if constexpr (UP) {
            tma_load_2d(&st.xa[0][0], mp + MP_XA, gx & ~3, gy, &st.bar);
            // coarse level (c0 = 1): region columns from (I0 - MR_H) / 2
            const int cx = 1 + ((tl.y - MR_H) >> 1);
            tma_load_2d(&st.c[0][0], mp + MP_NMAP + MP_X, cx & ~3, (tl.z - MR_H) >> 1,
                        &st.bar);
        }
    }
}

// The staged region to registers: bid = b/diag and x = xa (XA) at the fluid
// nodes, 0 elsewhere; fluid flags into R.m. ob/om: column of region column 0
// in the staged b/xa and mask rows (even: the pairs stay aligned).
template <bool XA>
__device__ __forceinline__ void mp_take(MRRegs<float>& R, const float (*sb)[MP_BW],
                                        const float (*sxa)[MP_BW], const uint8_t (*sm)[MP_MW],
                                        int ob, int om, float id)
{
    const int L = threadIdx.x, w = threadIdx.y;
    R.m = 0u;
#pragma unroll
    for (int i = 0; i < MR_R; ++i) {
        const int r = w * MR_R + i;
        const float2 bv = *reinterpret_cast<const float2*>(&sb[r][ob + 2 * L]);
        const unsigned mv = *reinterpret_cast<const unsigned short*>(&sm[r][om + 2 * L]);
        const unsigned m0 = mv & 0xffu, m1 = mv >> 8;
        R.b[i][0] = m0 ? bv.x * id : 0.f;
        R.b[i][1] = m1 ? bv.y * id : 0.f;
        R.m |= (m0 ? 1u : 0u) << (2 * i);
        R.m |= (m1 ? 1u : 0u) << (2 * i + 1);
        if (XA) {
            const float2 xv = *reinterpret_cast<const float2*>(&sxa[r][ob + 2 * L]);
            R.x[i][0] = m0 ? xv.x : 0.f;
            R.x[i][1] = m1 ? xv.y : 0.f;
        }
    }
}

// The same from global memory with the x-periodic wrap (MP_SLOW tiles).
template <bool XA>
__device__ __forceinline__ void mp_take_global(MRRegs<float>& R, const MGLevel& F, int J0,
                                               int I0, float id)
{
    const int L = threadIdx.x, w = threadIdx.y;
    const float* __restrict__ gb = lb<float>(F);
    const float* __restrict__ gx = (const float*)F.xa;
    R.m = 0u;
#pragma unroll
    for (int i = 0; i < MR_R; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int J = J0 - MR_H + w * MR_R + i;
            int I = I0 - MR_H + 2 * L + j;
            uint8_t mv = 0;
            float bv = 0.f, xv = 0.f;
            if (in_level(F, J, I)) {
                const long long k = nidx(F, J, I);
                mv = F.m[k];
                bv = gb[k];
                if (XA) xv = gx[k];
            }
            R.b[i][j] = mv ? bv * id : 0.f;
            R.m |= (mv ? 1u : 0u) << (2 * i + j);
            if (XA) R.x[i][j] = mv ? xv : 0.f;
        }
}

__device__ __forceinline__ void mp_publish(const MRRegs<float>& R, MPX xch, int buf)
{
    const int L = threadIdx.x, w = threadIdx.y;
    *reinterpret_cast<float2*>(&xch[buf][w + 1][0][2 * L]) = make_float2(R.x[0][0], R.x[0][1]);
    *reinterpret_cast<float2*>(&xch[buf][w + 1][1][2 * L]) =
        make_float2(R.x[MR_R - 1][0], R.x[MR_R - 1][1]);
}

// north / south neighbours: registers, or the adjacent warps' published rows
// (the outer slots 0 and MR_NW + 1 hold 0)
template <int I, int J>
__device__ __forceinline__ void mp_ns(const MRRegs<float>& R, MPX xch, int buf, float& up,
                                      float& dn)
{
    const int L = threadIdx.x, w = threadIdx.y;
    if constexpr (I > 0) up = R.x[I - 1][J];
    else up = xch[buf][w][1][2 * L + J];
    if constexpr (I < MR_R - 1) dn = R.x[I + 1][J];
    else dn = xch[buf][w + 2][0][2 * L + J];
}

// west / east neighbours: the pair's other node or the adjacent lane's (at
// the region's side columns the lane's own value, see above)
template <int I, int J>
__device__ __forceinline__ void mp_we(const MRRegs<float>& R, float& we, float& ea)
{
    if constexpr (J == 0) {
        we = __shfl_up_sync(0xffffffffu, R.x[I][1], 1);
        ea = R.x[I][1];
    } else {
        we = R.x[I][0];
        ea = __shfl_down_sync(0xffffffffu, R.x[I][0], 1);
    }
}

// half sweep of colour COL over the thread's rows (node of colour COL in row
// i: column (i + COL) & 1 of the pair); cxi = cx/diag, cyi = cy/diag
template <int COL, int I = 0>
__device__ __forceinline__ void mp_sweep_rows(MRRegs<float>& R, MPX xch, int buf, float cxi,
                                              float cyi)
{
    if constexpr (I < MR_R) {
        constexpr int J = (I + COL) & 1;
        float we, ea, up, dn;
        mp_we<I, J>(R, we, ea);
        mp_ns<I, J>(R, xch, buf, up, dn);
        const float v = fmaf(-cxi, we + ea, fmaf(-cyi, up + dn, R.b[I][J]));
        R.x[I][J] = (R.m >> (2 * I + J)) & 1u ? v : 0.f;
        mp_sweep_rows<COL, I + 1>(R, xch, buf, cxi, cyi);
    }
}

template <int COL>
__device__ __forceinline__ void mp_half_sweep(MRRegs<float>& R, MPX xch, int buf, float cxi,
                                              float cyi)
{
    mp_publish(R, xch, buf);
    __syncthreads();
    mp_sweep_rows<COL>(R, xch, buf, cxi, cyi);
}

// residual b - A x = diag (GS update - x) at the red node of each row (column
// i & 1), 0 at non-fluid nodes
template <int I = 0>
__device__ __forceinline__ void mp_residual_rows(const MRRegs<float>& R, MPX xch, int buf,
                                                 float cxi, float cyi, float dg,
                                                 float (&res)[MR_R])
{
    if constexpr (I < MR_R) {
        constexpr int J = I & 1;
        float we, ea, up, dn;
        mp_we<I, J>(R, we, ea);
        mp_ns<I, J>(R, xch, buf, up, dn);
        const float v = fmaf(-cxi, we + ea, fmaf(-cyi, up + dn, R.b[I][J]));
        res[I] = (R.m >> (2 * I + J)) & 1u ? dg * (v - R.x[I][J]) : 0.f;
        mp_residual_rows<I + 1>(R, xch, buf, cxi, cyi, dg, res);
    }
}

// x of the thread's tile nodes to y (node pairs as one 8-byte store where
// both lie in the tile and the level); RZ: the thread's sum of bid x
template <bool RZ>
__device__ __forceinline__ float mp_store(const MRRegs<float>& R, const MGLevel& F,
                                          float* __restrict__ y, int J0, int I0)
{
    const int L = threadIdx.x, w = threadIdx.y;
    const int I = I0 - MR_H + 2 * L;
    const bool in0 = 2 * L >= MR_H && 2 * L < MR_H + MR_TW && I < F.nxn;
    const bool in1 = 2 * L + 1 >= MR_H && 2 * L + 1 < MR_H + MR_TW && I + 1 < F.nxn;
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < MR_R; ++i) {
        const int r = w * MR_R + i;
        const int J = J0 - MR_H + r;
        if (r < MR_H || r >= MR_H + MR_TH || J >= F.nyn) continue;
        float* p = y + nidx(F, J, I);
        if (in0 && in1) {
            *reinterpret_cast<float2*>(p) = make_float2(R.x[i][0], R.x[i][1]);
        } else {
            if (in0) p[0] = R.x[i][0];
            if (in1) p[1] = R.x[i][1];
        }
        if (RZ) {
            if (in0) acc = fmaf(R.b[i][0], R.x[i][0], acc);
            if (in1) acc = fmaf(R.b[i][1], R.x[i][1], acc);
        }
    }
    return acc;
}

// Restriction to the coarse level: the coarse node whose centre is the red
// node (r0, 2L + 1), r0 odd in the tile and L - 2 in [0, MR_TW/2), gets the
// residual there plus a quarter of the four red corners (r0 +- 1, 2L and
// 2L + 2); 0 when the centre is not a fluid node. xr[w + 1] holds warp w's
// row-0 residuals.
__device__ __forceinline__ void mp_restrict(const float (&res)[MR_R], unsigned m,
                                            const float (*xr)[32], const MGLevel& C, int J0,
                                            int I0)
{
    const int L = threadIdx.x, w = threadIdx.y;
    float* __restrict__ cb = lb<float>(C);
    const int cI = (I0 >> 1) + L - (MR_H - 1) / 2;
    const bool colin = L >= (MR_H - 1) / 2 && L < (MR_H - 1) / 2 + MR_TW / 2 && cI < C.nxn;
#pragma unroll
    for (int i = 1; i < MR_R; i += 2) {
        const float up1 = res[i - 1];
        const float dn1 = i + 1 < MR_R ? res[i + 1] : xr[w + 2][L];
        const float up2 = __shfl_down_sync(0xffffffffu, up1, 1);
        const float dn2 = __shfl_down_sync(0xffffffffu, dn1, 1);
        const int r0 = w * MR_R + i;
        const int cJ = (J0 >> 1) + ((r0 - MR_H) >> 1);
        if (colin && r0 >= MR_H && r0 < MR_H + MR_TH && cJ < C.nyn) {
            const float c4 = (up1 + up2) + (dn1 + dn2);
            const float v = res[i] + 0.25f * c4;
            cb[nidx(C, cJ, cI)] = (m >> (2 * i + 1)) & 1u ? v : 0.f;
        }
    }
}

__device__ __forceinline__ void mp_zero_outer(MPX xch, int t)
{
    // slots 0 and MR_NW + 1 of both buffers, both rows: 2 x 2 x 2 x MR_W floats
    for (int e = t; e < 8 * MR_W; e += MR_NW * 32) {
        const int buf = e / (4 * MR_W), s = (e / (2 * MR_W)) & 1, row = (e / MR_W) & 1;
        xch[buf][s ? MR_NW + 1 : 0][row][e % MR_W] = 0.f;
    }
}

// Give up on a staged load that did not land: record the time-out, wait once
// more (bounded) for the copy in flight so that it does not outlive the
// block, return.
template <typename ST>
__device__ __forceinline__ void mp_fail(ST& st, uint32_t parity, int* status, int t)
{
    if (t == 0) {
        atomicOr(status, ST_TMA_TIMEOUT);
        mbar_wait(&st.bar, parity);
    }
}

__device__ __forceinline__ bool mp_skip(int converged, int conv_in, int ir)
{
    return converged || (ir && conv_in);
}

// Down leg of level l: pre-smoothing from a zero guess (red x = bid, black,
// then NU-1 more (red, black) sweeps), xa = x on the tile, the residual at
// the red nodes and its restriction to level l+1's b.
template <int NU>
__global__ void __launch_bounds__(256, 4)
k_mgp_down(const int4* __restrict__ tiles, int ntiles, const MGLevel* __restrict__ levs,
           const CUtensorMap* __restrict__ maps, int l, const DevScalars* __restrict__ scs,
           int ir, int* status)
{
    pdl_wait();
    extern __shared__ __align__(128) unsigned char mp_dyn[];
    MPDown& st = *reinterpret_cast<MPDown*>(mp_dyn);
    // after a staging failure the rest of the solve is void: skip the work
    // (the loop ends at its iteration limit without further waits)
    if (*(volatile int*)status & (ST_TMA_TIMEOUT | ST_STAGE_ALIGN)) return;
    if (smem_u32(mp_dyn) & 127u) {
        if (threadIdx.x == 0 && threadIdx.y == 0) atomicOr(status, ST_STAGE_ALIGN);
        return;
    }
    __shared__ __align__(16) float xch[2][MR_NW + 2][2][MR_W];
    __shared__ float xr[MR_NW + 2][32];
    const int L = threadIdx.x, w = threadIdx.y, t = w * 32 + L;
    const int G = gridDim.x;
    mp_zero_outer(xch, t);
    int4 nrec = make_int4(0, 0, 0, 0);  // thread 0: record of the tile after the staged one
    int ncv = 0, nci = 0;               // and its member's convergence flags
    if (t == 0) {
        mbar_init(&st.bar, 1);
        const int4 r0 = tiles[blockIdx.x];
        const bool sk = mp_skip(scs[r0.x].converged, scs[r0.x].conv_in, ir);
        st.rec[0] = r0;
        st.skip[0] = sk;
        if (!sk) mp_issue<false>(st, 0, r0, levs, maps, l);
        if ((int)blockIdx.x + G < ntiles) {
            nrec = tiles[blockIdx.x + G];
            ncv = scs[nrec.x].converged;
            nci = scs[nrec.x].conv_in;
        }
    }
    __syncthreads();
    uint32_t ph = 0;
    for (int k = blockIdx.x, it = 0; k < ntiles; k += G, ++it) {
        const int slot = it & 1;
        const int4 tl = st.rec[slot];
        const bool skip = st.skip[slot] != 0;
        MRRegs<float> R;
        if (!skip) {
            const bool ok = mbar_wait(&st.bar, ph);
            if (__syncthreads_or(!ok)) {
                mp_fail(st, ph, status, t);
                return;
            }
            ph ^= 1u;
            const MGLevel& F = st.lv[slot][0];
            const float id = F.fidiag;
            if (!(tl.w & MP_SLOW)) {
                const int gx = (tl.w & 0xff) + tl.y - MR_H;
                mp_take<false>(R, st.b, nullptr, st.m, gx & 3, gx & 15, id);
            } else {
                mp_take_global<false>(R, F, tl.z, tl.y, id);
            }
        }
        __syncthreads();  // staging buffer free
        if (t == 0 && k + G < ntiles) {
            const bool sk = mp_skip(ncv, nci, ir);
            st.rec[slot ^ 1] = nrec;
            st.skip[slot ^ 1] = sk;
            if (!sk) mp_issue<false>(st, slot ^ 1, nrec, levs, maps, l);
            if (k + 2 * G < ntiles) nrec = tiles[k + 2 * G];
        }
        if (!skip) {
            const MGLevel& F = st.lv[slot][0];
            const float id = F.fidiag, dg = F.fdiag;
            const float cxi = F.fcx * id, cyi = F.fcy * id;
            const int I0 = tl.y, J0 = tl.z;
#pragma unroll
            for (int i = 0; i < MR_R; ++i) {
                // red (column i & 1 of the pair) from a zero guess
                R.x[i][i & 1] = R.b[i][i & 1];
                R.x[i][(i & 1) ^ 1] = 0.f;
            }
            mp_half_sweep<1>(R, xch, 0, cxi, cyi);
            if constexpr (NU >= 2) {
                mp_half_sweep<0>(R, xch, 1, cxi, cyi);
                mp_half_sweep<1>(R, xch, 0, cxi, cyi);
            }
            mp_publish(R, xch, 1);
            __syncthreads();
            float res[MR_R];
            mp_residual_rows(R, xch, 1, cxi, cyi, dg, res);
            mp_store<false>(R, F, (float*)F.xa, J0, I0);
            xr[w + 1][L] = res[0];
            __syncthreads();
            mp_restrict(res, R.m, xr, st.lv[slot][1], J0, I0);
        } else {
            __syncthreads();  // the next slot's record is visible
        }
        if (t == 0 && k + 2 * G < ntiles) {
            ncv = scs[nrec.x].converged;
            nci = scs[nrec.x].conv_in;
        }
    }
}

// Up leg of level l: x = xa + P (coarse x) at the fluid nodes, then NU
// (black, red) sweeps; x of the tile to level l's x. RZ (level 0): the
// tile's part of <r, z> (r = b, z = x) into tpart[k] (k_bs_rz sums a
// member's tiles: no fence or ticket holds the block up here).
template <int NU, bool RZ>
__global__ void __launch_bounds__(256, 3)
k_mgp_up(const int4* __restrict__ tiles, int ntiles, const MGLevel* __restrict__ levs,
         const CUtensorMap* __restrict__ maps, int l, const DevScalars* __restrict__ scs,
         int ir, double* tpart, int* status)
{
    pdl_wait();
    extern __shared__ __align__(128) unsigned char mp_dyn[];
    MPUp& st = *reinterpret_cast<MPUp*>(mp_dyn);
    // after a staging failure the rest of the solve is void: skip the work
    // (the loop ends at its iteration limit without further waits)
    if (*(volatile int*)status & (ST_TMA_TIMEOUT | ST_STAGE_ALIGN)) return;
    if (smem_u32(mp_dyn) & 127u) {
        if (threadIdx.x == 0 && threadIdx.y == 0) atomicOr(status, ST_STAGE_ALIGN);
        return;
    }
    __shared__ __align__(16) float xch[2][MR_NW + 2][2][MR_W];
    const int L = threadIdx.x, w = threadIdx.y, t = w * 32 + L;
    const int G = gridDim.x;
    mp_zero_outer(xch, t);
    int4 nrec = make_int4(0, 0, 0, 0);
    int ncv = 0, nci = 0;
    if (t == 0) {
        mbar_init(&st.bar, 1);
        const int4 r0 = tiles[blockIdx.x];
        const bool sk = mp_skip(scs[r0.x].converged, scs[r0.x].conv_in, ir);
        st.rec[0] = r0;
        st.skip[0] = sk;
        if (!sk) mp_issue<true>(st, 0, r0, levs, maps, l);
        if ((int)blockIdx.x + G < ntiles) {
            nrec = tiles[blockIdx.x + G];
            ncv = scs[nrec.x].converged;
            nci = scs[nrec.x].conv_in;
        }
    }
    __syncthreads();
    uint32_t ph = 0;
    for (int k = blockIdx.x, it = 0; k < ntiles; k += G, ++it) {
        const int slot = it & 1;
        const int4 tl = st.rec[slot];
        const bool skip = st.skip[slot] != 0;
        MRRegs<float> R;
        if (!skip) {
            const bool ok = mbar_wait(&st.bar, ph);
            if (__syncthreads_or(!ok)) {
                mp_fail(st, ph, status, t);
                return;
            }
            ph ^= 1u;
            const MGLevel& F = st.lv[slot][0];
            const float id = F.fidiag;
            const bool slow = tl.w & MP_SLOW;
            int oc = 0;
            if (!slow) {
                const int gx = (tl.w & 0xff) + tl.y - MR_H;
                mp_take<true>(R, st.b, st.xa, st.m, gx & 3, gx & 15, id);
                oc = (1 + ((tl.y - MR_H) >> 1)) & 3;
            } else {
                mp_take_global<true>(R, F, tl.z, tl.y, id);
                // the coarse region: 0 outside the coarse level, wrapped
                const MGLevel& C = st.lv[slot][1];
                const int cj0 = (tl.z - MR_H) >> 1, ci0 = (tl.y - MR_H) >> 1;
                const float* __restrict__ cxg = lx<float>(C);
                constexpr int CW = MR_W / 2 + 1;
                for (int e = t; e < MP_CH * CW; e += 256) {
                    const int r = e / CW, c = e - r * CW;
                    int I = ci0 + c;
                    float v = 0.f;
                    if (in_level(C, cj0 + r, I)) v = cxg[nidx(C, cj0 + r, I)];
                    st.c[r][c] = v;
                }
                __syncthreads();
            }
            // x += P (coarse x) at the fluid nodes, as mg_reg.cuh's up leg:
            // the average of two row averages; thread rows lie on coarse rows
            // 5w .. 5w + 5, columns L (oi = 1) and L + 1
            float cv[MR_R / 2 + 1][2];
#pragma unroll
            for (int q = 0; q <= MR_R / 2; ++q) {
                cv[q][0] = st.c[w * (MR_R / 2) + q][oc + L];
                cv[q][1] = st.c[w * (MR_R / 2) + q][oc + L + 1];
            }
#pragma unroll
            for (int i = 0; i < MR_R; ++i) {
                const int lr = (1 + i) >> 1, oj = (1 + i) & 1;
                const float h0 = 0.5f * (cv[lr][0] + cv[lr][1]);
                const float h1 = 0.5f * (cv[lr + oj][0] + cv[lr + oj][1]);
                const float g0 = 0.5f * (cv[lr][1] + cv[lr][1]);
                const float g1 = 0.5f * (cv[lr + oj][1] + cv[lr + oj][1]);
                R.x[i][0] += (R.m >> (2 * i)) & 1u ? 0.5f * (h0 + h1) : 0.f;
                R.x[i][1] += (R.m >> (2 * i + 1)) & 1u ? 0.5f * (g0 + g1) : 0.f;
            }
        }
        __syncthreads();  // staging buffer free
        if (t == 0 && k + G < ntiles) {
            const bool sk = mp_skip(ncv, nci, ir);
            st.rec[slot ^ 1] = nrec;
            st.skip[slot ^ 1] = sk;
            if (!sk) mp_issue<true>(st, slot ^ 1, nrec, levs, maps, l);
            if (k + 2 * G < ntiles) nrec = tiles[k + 2 * G];
        }
        if (!skip) {
            const MGLevel& F = st.lv[slot][0];
            const float id = F.fidiag;
            const float cxi = F.fcx * id, cyi = F.fcy * id;
            mp_half_sweep<1>(R, xch, 0, cxi, cyi);
            mp_half_sweep<0>(R, xch, 1, cxi, cyi);
            if constexpr (NU >= 2) {
                mp_half_sweep<1>(R, xch, 0, cxi, cyi);
                mp_half_sweep<0>(R, xch, 1, cxi, cyi);
            }
            const float acc = mp_store<RZ>(R, F, lx<float>(F), tl.z, tl.y);
            if (RZ) {
                // b x = diag bid x, summed per warp in FP32, combined in FP64
                const double tot = block_sum<float>(acc);
                if (t == 0) tpart[k] = (double)F.fdiag * tot;
            }
        } else {
            __syncthreads();
        }
        if (t == 0 && k + 2 * G < ntiles) {
            ncv = scs[nrec.x].converged;
            nci = scs[nrec.x].conv_in;
        }
    }
}

}  // namespace f2d
