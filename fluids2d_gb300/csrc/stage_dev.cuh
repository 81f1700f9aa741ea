// Device pieces of the fused stage kernels shared by the single-model kernels
// (stage.cu) and the batched ensemble kernels (ensemble.cu).
#pragma once
#include "common.cuh"
#include "weno.cuh"

namespace f2d {

constexpr int TX = 32, TY = 8;           // cells per tile (32 x 8 threads)
constexpr int SW = TX + 8, SH = TY + 6;  // staged tile: cols i0-4.., rows j0-3..
constexpr int OX = 4, OY = 3;            // offset of cell (j0,i0) in the tile
// The flux-form stage runs 32 x 32-cell tiles (4 rows per thread): a quarter
// of the blocks, each waiting once for its TMA tile, and 1.48x instead of
// 2.19x staged cells per cell.
constexpr int FRT = 4, FTY = 8 * FRT, FSH = FTY + 6;

// Test hook of the failure detection (f2d_test_tma_wait). When enabled,
// every stage kernel, once its TMA tile has landed, also waits for the next
// phase of the tile's barrier, which nothing completes (no thread arrives
// again), so that wait runs out after limit_ns: the kernel sets
// ST_TMA_TIMEOUT and returns with no copy in flight. One copy of the switch
// per translation unit.
struct TmaWaitTest {
    unsigned int enabled;
    unsigned int pad;
    unsigned long long limit_ns;
};
static __device__ TmaWaitTest g_tma_wait_test;

__device__ __forceinline__ bool tma_wait_test(uint64_t* bar)
{
    if (!g_tma_wait_test.enabled) return true;
    return mbar_wait(bar, 1, g_tma_wait_test.limit_ns);
}

template <typename T>
__device__ __forceinline__ T ldz(const T* __restrict__ a, int j, int i,
                                 const Geom& g)
{
    return (j >= 0 && j < g.NY && i >= 0 && i < g.NX) ? a[(long long)j * g.P + i]
                                                      : T(0);
}

// Load with the reference's flattened-array semantics (its WENO loops index
// the raveled (NY, NX) array, weno.py:349-411): a column outside [0, NX)
// continues in the previous / next row; outside the array: 0.
template <typename T>
__device__ __forceinline__ T ldw(const T* __restrict__ a, int j, int i, const Geom& g)
{
    if (i < 0) {
        i += g.NX;
        j -= 1;
    } else if (i >= g.NX) {
        i -= g.NX;
        j += 1;
    }
    return (j >= 0 && j < g.NY && i >= 0 && i < g.NX) ? a[(long long)j * g.P + i] : T(0);
}

// The RK3 increment of stage k (1, 2, 3) in the reference's evaluation order:
// y += ((0 + c1*ds1) + c2*ds2) + c3*ds3 with (c) = (dt), (-3dt/4, dt/4),
// (-dt/12, -dt/12, 2dt/3).
// The coefficients are computed once per block (one thread, into shared
// memory): per-thread FP64 divisions would load the FP64 pipe of the FP32
// kernels.
template <typename T>
__device__ __forceinline__ void rk3_coefs(int stage, double dt, T* c, double gamma = 0.0)
{
    // stage = k | (integrator << 4); the coefficients of ef (integrators.py:
    // 116-123) and enrk3 (140-155) in the reference's evaluation order; LFRA
    // (39-55): dt, 2 dt and the filter coefficient
    const int integ = (stage >> 4) & 15;
    stage &= 15;
    if (integ == 3) {
        c[0] = T(dt);
        c[1] = T(2 * dt);
        c[2] = T(gamma);
        return;
    }
    if (integ == 1) {
        c[0] = T(dt);
        c[1] = c[2] = T(0);
        return;
    }
    if (integ == 2) {
        if (stage == 1) {
            c[0] = T(dt / 3);
            c[1] = c[2] = T(0);
        } else if (stage == 2) {
            c[0] = T(-dt / 3 - 5 * dt / 48);
            c[1] = T(15 * dt / 16);
            c[2] = T(0);
        } else {
            c[0] = T(5 * dt / 48 + dt / 10);
            c[1] = T(-7 * dt / 16);
            c[2] = T(2 * dt / 5);
        }
        return;
    }
    if (stage == 1) {
        c[0] = T(dt);
        c[1] = c[2] = T(0);
    } else if (stage == 2) {
        c[0] = T(-3 * dt / 4);
        c[1] = T(dt / 4);
        c[2] = T(0);
    } else {
        c[0] = c[1] = T(-dt / 12);
        c[2] = T(2 * dt / 3);
    }
}

template <typename T>
__device__ __forceinline__ T rk3_increment(int stage, const T* c, T d1, T d2, T d3)
{
    if (stage == 1) return c[0] * d1;
    if (stage == 2) return c[0] * d1 + c[1] * d2;
    return (c[0] * d1 + c[1] * d2) + c[2] * d3;
}

// Leap-frog step with the Robert-Asselin filter at one point (integrators.py:
// 39-55) from the current value q, the filtered previous value pv and the
// tendency ds; c = {dt, 2 dt, gamma}. The first step (ite == 0) is Euler
// forward and keeps q as the previous value; afterwards the new value is
// pv + 2 dt ds and the filtered current value q + gamma (new + pv - 2 q) is
// the next step's previous value (rightpermute leaves sa == sb == it).
template <typename T>
__device__ __forceinline__ void lfra_update(bool first, const T* c, T q, T pv, T ds, T& qn,
                                            T& pn)
{
    if (first) {
        qn = q + c[0] * ds;
        pn = q;
    } else {
        qn = pv + c[1] * ds;
        pn = q + ((c[2] * qn + c[2] * pv) + (T(-2) * c[2]) * q);
    }
}

// Store v at (j,i) and, in an x-periodic domain, at its halo copy.
// Returns false for points that belong to the halo copy of another thread.
__device__ __forceinline__ bool periodic_owner(const Geom& g, int i)
{
    return !g.xper || (i >= 3 && i < g.nx + 3);
}

template <typename T>
__device__ __forceinline__ void store_filled(T* __restrict__ a, const Geom& g,
                                             int j, int i, T v)
{
    const long long r = (long long)j * g.P;
    a[r + i] = v;
    if (g.xper) {
        if (i < 6) a[r + i + g.nx] = v;
        else if (i >= g.nx) a[r + i - g.nx] = v;
    }
}

// Issue the TMA loads of up to two (SH x SW) tiles and wait for them. All
// threads wait on the barrier; returns false (uniformly) on timeout.
template <typename T, int SHR = SH>
__device__ __forceinline__ bool stage_tiles(T (*s0)[SW], const CUtensorMap* m0,
                                            T (*s1)[SW], const CUtensorMap* m1,
                                            int i0, int j0, uint64_t* bar,
                                            int* status)
{
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    if (t == 0) mbar_init(bar, 1);
    __syncthreads();
    if (t == 0) {
        const uint32_t bytes = (uint32_t)(sizeof(T) * SW * SHR * (s1 ? 2 : 1));
        mbar_expect_tx(bar, bytes);
        tma_load_2d(&s0[0][0], m0, i0 - OX, j0 - OY, bar);
        if (s1) tma_load_2d(&s1[0][0], m1, i0 - OX, j0 - OY, bar);
    }
    bool ok = mbar_wait(bar, 0) && tma_wait_test(bar);
    int all = __syncthreads_and(ok ? 1 : 0);
    if (!all && t == 0) atomicOr(status, ST_TMA_TIMEOUT);
    return all != 0;
}

// ---------------------------------------------------------------------------
// Flux-form stage on one tile: dq = -div(U q) * msk (divflux/div,
// operators.py:21-29, 104-107) for eulerpsi (q = omega) and qg (q = pv), then
// the RK3 update. `tq` is the TMA map of qin (param or global memory).
// Returns after the (uniform) TMA timeout check; all threads must call it.
// ---------------------------------------------------------------------------
template <typename T, int M>
struct FluxformSmem {
    alignas(128) T sq[FSH][SW];
    T sfx[FTY][TX + 1];
    T sfy[FTY + 1][TX];
    T rk[3];
    uint64_t bar;
};

// Integrator code of the tendency-only mode of the stage kernels (the
// reference's rhs(s, ds) alone, equations.py:73-136): the kernel writes the
// tendency (with its halo fill and any forcing term) to the tendency output
// and leaves the state alone.
constexpr int INTEG_TENDENCY = 15;

// FRC: the kernel takes a forcing field `frc` (may be null at run time),
// added to the tendency after the right-hand side (addforcingterm,
// equations.py:229-238).
template <typename T, int M, bool FRC = false>
__device__ __forceinline__ void fluxform_tile(
    FluxformSmem<T, M>& sm, const CUtensorMap* tq, const T* __restrict__ qin,
    T* __restrict__ qout, const T* __restrict__ Ux, const T* __restrict__ Uy,
    const uint32_t* __restrict__ code, T* __restrict__ ds_out, const T* __restrict__ ds1,
    const T* __restrict__ ds2, const T* __restrict__ frc, int stage, const Geom& g,
    double dt, double gamma, int* status, int i0, int j0)
{
    auto& sq = sm.sq;
    auto& sfx = sm.sfx;
    auto& sfy = sm.sfy;
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
    const int sk = stage;  // stage | integrator << 4 | first LFRA step << 8
    const bool lf = ((sk >> 4) & 15) == 3;
    const bool tend = ((sk >> 4) & 15) == INTEG_TENDENCY;
    const bool hasf = FRC && frc != nullptr;
    stage &= 15;
    (void)qin;
    // 1. the TMA load of the staged tile (q with its 3-cell halo) ...
    if (t == 0) mbar_init(&sm.bar, 1);
    __syncthreads();
    if (t == 0) {
        mbar_expect_tx(&sm.bar, (uint32_t)(sizeof(T) * SW * FSH));
        tma_load_2d(&sq[0][0], tq, i0 - OX, j0 - OY, &sm.bar);
    }
    // 2. ... overlapped with this thread's plain loads: the code word and
    // face velocities of its cells (faces (j,i) of x and y share the index
    // of cell (j,i)), the earlier stage tendencies, and the extra column of
    // x-faces / row of y-faces of the tile edge; all unconditional (clamped
    // index, then masked), so they are in flight together.
    const int i = i0 + tx;
    uint32_t cd[FRT];
    T ux[FRT], uy[FRT], d1[FRT], d2[FRT], fq[FRT];
#pragma unroll
    for (int q = 0; q < FRT; ++q) {
        const int j = j0 + ty + 8 * q;
        const bool in = j < g.NY && i < g.NX;
        const long long o = (long long)min(j, g.NY - 1) * g.P + min(i, g.NX - 1);
        const uint32_t c = code[o];
        const T u = Ux[o], v = Uy[o];
        cd[q] = in ? c : 0u;
        ux[q] = u;
        uy[q] = v;
        d1[q] = (stage >= 2 || lf) && !tend ? ds1[o] : T(0);
        d2[q] = stage == 3 && !tend ? ds2[o] : T(0);
        fq[q] = hasf ? frc[o] : T(0);
    }
    uint32_t ce = 0u;
    T ue = T(0);
    int er = 0, ec = 0, ex = 0;  // edge face: x (ex = 1) at (t, TX) or y (ex = 2) at (FTY, t-FTY)
    if (t < FTY + TX) {
        ex = t < FTY ? 1 : 2;
        er = t < FTY ? t : FTY;
        ec = t < FTY ? TX : t - FTY;
        const int j = j0 + er, ii = i0 + ec;
        const bool in = j < g.NY && ii < g.NX;
        const long long o = (long long)min(j, g.NY - 1) * g.P + min(ii, g.NX - 1);
        const uint32_t c = code[o];
        const T u = ex == 1 ? Ux[o] : Uy[o];
        ce = in ? c : 0u;
        ue = u;
    }
    // 3. wait for the tile (bounded; uniform time-out exit)
    {
        const bool ok = mbar_wait(&sm.bar, 0) && tma_wait_test(&sm.bar);
        const int all = __syncthreads_and(ok ? 1 : 0);
        if (!all) {
            if (t == 0) atomicOr(status, ST_TMA_TIMEOUT);
            return;
        }
    }
    // 4. fluxes at the faces, each evaluated once (zero without an order)
    auto xflux = [&](int r, int c, uint32_t cw, T U) {
        const int L = lev(cw, SH_OCX);
        T f = T(0);
        if (L) {
            const T* w = &sq[r + OY][c + OX - 3];
            f = face_value<M, T>(L, U, w[0], w[1], w[2], w[3], w[4], w[5]) * U;
        }
        sfx[r][c] = f;
    };
    auto yflux = [&](int r, int c, uint32_t cw, T U) {
        const int L = lev(cw, SH_OCY);
        T f = T(0);
        if (L) {
            const int cc = c + OX;
            f = face_value<M, T>(L, U, sq[r][cc], sq[r + 1][cc], sq[r + 2][cc], sq[r + 3][cc],
                                 sq[r + 4][cc], sq[r + 5][cc]) *
                U;
        }
        sfy[r][c] = f;
    };
#pragma unroll
    for (int q = 0; q < FRT; ++q) {
        xflux(ty + 8 * q, tx, cd[q], ux[q]);
        yflux(ty + 8 * q, tx, cd[q], uy[q]);
    }
    if (ex == 1) xflux(er, ec, ce, ue);
    else if (ex == 2) yflux(er, ec, ce, ue);
    if (t == 0) rk3_coefs<T>(sk, dt, sm.rk, gamma);
    __syncthreads();

    // 5. tendency, RK3 update and stores of this thread's cells
    if (i >= g.NX || !periodic_owner(g, i)) return;
#pragma unroll
    for (int q = 0; q < FRT; ++q) {
        const int r = ty + 8 * q, j = j0 + r;
        if (j >= g.NY) break;
        const T msk = (cd[q] & B_MSK) ? T(1) : T(0);
        T ds = (-(sfx[r][tx + 1] - sfx[r][tx]) - (sfy[r + 1][tx] - sfy[r][tx])) * msk;
        if (hasf) ds += fq[q];
        if (tend) {
            store_filled(ds_out, g, j, i, ds);
            continue;
        }
        if (lf) {
            // LFRA: ds1 = the filtered previous state in, ds_out = out
            T qn, pn;
            lfra_update<T>(sk & 256, sm.rk, sq[r + OY][tx + OX], d1[q], ds, qn, pn);
            store_filled(qout, g, j, i, qn);
            store_filled(ds_out, g, j, i, pn);
            continue;
        }
        T inc;
        if (stage == 1) inc = rk3_increment<T>(1, sm.rk, ds, T(0), T(0));
        else if (stage == 2) inc = rk3_increment<T>(2, sm.rk, d1[q], ds, T(0));
        else inc = rk3_increment<T>(3, sm.rk, d1[q], d2[q], ds);
        const T qv = sq[r + OY][tx + OX];
        store_filled(qout, g, j, i, qv + inc);
        if (ds_out) store_filled(ds_out, g, j, i, ds);
    }
}

}  // namespace f2d
