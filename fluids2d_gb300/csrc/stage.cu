// Fused time-stepping kernels and the element-wise kernels around them.
//
// One launch per RK stage computes the right-hand side of the reference's
// equation set AND applies the integrator's update (SSP-RK3, ef, enrk3 or
// the LFRA step; integrators.py:20-155, addto 154-196) over a tile (32x32
// cells for the flux-form models and the tracer, 32x8 for the momentum
// kernel of rsw, euler, boussinesq and qgrsw), with the stencil inputs
// staged in shared memory by TMA (halo of 3 cells) and every face flux
// evaluated once. qgrsw's momentum launch writes the raw tendency; its
// projection around the Helmholtz solve and the update follow in
// k_qgrsw_pv / k_qgrsw_update. Also here: the diagnostics (vertex average,
// perpgrad, rsw/euler diagnostics, max|U|), the euler pressure projection
// around the Neumann solve, the Bulk reduction and the float32 snapshot.
//
// Every array point is produced with the numpy-slice semantics of the
// reference operators, including the halo rows and columns (the reference
// applies the Coriolis and gradient terms there too, and those values feed
// back into the interior). In an x-periodic domain the halo columns are the
// reference's halo fill (meshes.py:135-143): the threads owning columns
// [3,6) and [nx,nx+3) also write the copies, so no separate fill pass runs.
#include <algorithm>

#include "stage.cuh"
#include "stage_dev.cuh"

namespace f2d {

// ---------------------------------------------------------------------------
// Flux-form stage kernel of one model (tile = block index).
// ---------------------------------------------------------------------------
template <typename T, int M>
__global__ void __launch_bounds__(TX * TY, sizeof(T) == 4 ? 5 : 3)
k_fluxform_stage(const __grid_constant__ CUtensorMap tq, const T* __restrict__ qin,
                 T* __restrict__ qout, const T* __restrict__ Ux,
                 const T* __restrict__ Uy, const uint32_t* __restrict__ code,
                 T* __restrict__ ds_out, const T* __restrict__ ds1,
                 const T* __restrict__ ds2, const T* __restrict__ frc, int stage, Geom g,
                 DevScalars* sc)
{
    __shared__ FluxformSmem<T, M> sm;
    if (((stage >> 4) & 15) == 3 && sc->ite == 0) stage |= 256;  // first LFRA step
    fluxform_tile<T, M, true>(sm, &tq, qin, qout, Ux, Uy, code, ds_out, ds1, ds2, frc, stage,
                              g, sc->dt, sc->ragamma, &sc->status, blockIdx.x * TX,
                              blockIdx.y * FTY);
}

// ---------------------------------------------------------------------------
// Rotating shallow water right-hand side (equations.py:139-148) + RK3 update
// of (u.x, u.y, h): vortex force (weno.vortexforce), Coriolis, gradients of
// ke and p, mass flux divergence. The same kernel steps the euler model
// (vortex force and grad ke, equations.py:11-15) and the boussinesq model
// (euler + buoyancy, with the flux divergence of b in place of h,
// equations.py:29-35).
// ---------------------------------------------------------------------------
template <typename T, int M>
__global__ void __launch_bounds__(TX * TY)
k_rsw_stage(const __grid_constant__ CUtensorMap th,
            const __grid_constant__ CUtensorMap tw, RswIn a,
            const uint32_t* __restrict__ code, int stage, Geom g, DevScalars* sc)
{
    __shared__ alignas(128) T sh[SH][SW];
    __shared__ alignas(128) T sw[SH][SW];
    __shared__ T sfx[TY][TX + 1];
    __shared__ T sfy[TY + 1][TX];
    __shared__ T srk[4];  // RK3 coefficients, Coriolis parameter
    __shared__ uint64_t bar;
    const int sk = stage;  // stage | integrator << 4
    const bool lf = ((sk >> 4) & 15) == 3;
    stage &= 15;
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const T* __restrict__ Ux = (const T*)a.Ux;
    const T* __restrict__ Uy = (const T*)a.Uy;

    if (!stage_tiles<T>(sh, &th, sw, &tw, i0, j0, &bar, &sc->status)) return;
    // qgrsw consumes the raw tendency of the x-periodic halo columns (its PV
    // is formed before the halo fill, operators.py:179-180), where the
    // reference's stencils over the raveled array run into the neighbouring
    // row: the edge tiles take those values in place of the out-of-array 0
    const bool wrap = a.euler == 3 && g.xper;
    if (wrap && (i0 < OX || i0 - OX + SW > g.NX)) {
        const T* __restrict__ hg = (const T*)a.h;
        const T* __restrict__ wg = (const T*)a.w;
        for (int e = t; e < SH * SW; e += TX * TY) {
            const int r = e / SW, c = e % SW;
            const int gj = j0 - OY + r, gi = i0 - OX + c;
            if (gi >= 0 && gi < g.NX) continue;
            sh[r][c] = ldw(hg, gj, gi, g);
            sw[r][c] = ldw(wg, gj, gi, g);
        }
        __syncthreads();
    }

    // mass fluxes U*h at the faces (compflux, weno.py:349-363)
    auto xface = [&](int r, int c) {
        const int j = j0 + r, i = i0 + c;
        T f = T(0);
        if (j < g.NY && i < g.NX) {
            const long long o = (long long)j * g.P + i;
            const int L = lev(code[o], SH_OCX);
            if (L) {
                const T U = Ux[o];
                const T* w = &sh[r + OY][c + OX - 3];
                f = face_value<M, T>(L, U, w[0], w[1], w[2], w[3], w[4], w[5]) * U;
            }
        }
        sfx[r][c] = f;
    };
    auto yface = [&](int r, int c) {
        const int j = j0 + r, i = i0 + c;
        T f = T(0);
        if (j < g.NY && i < g.NX) {
            const long long o = (long long)j * g.P + i;
            const int L = lev(code[o], SH_OCY);
            if (L) {
                const T U = Uy[o];
                const int cc = c + OX;
                f = face_value<M, T>(L, U, sh[r][cc], sh[r + 1][cc], sh[r + 2][cc],
                                     sh[r + 3][cc], sh[r + 4][cc], sh[r + 5][cc]) *
                    U;
            }
        }
        sfy[r][c] = f;
    };
    if (a.euler != 1) {
        xface(ty, tx);
        yface(ty, tx);
        if (t < TY) xface(t, TX);
        else if (t < TY + TX) yface(TY, t - TY);
    }

    // The vortex force needs no shared fluxes: it is evaluated before the
    // barrier, so warps with fewer faces above do not idle at it.
    const int j = j0 + ty, i = i0 + tx;
    // qgrsw's raw tendency is consumed before any halo fill (the reference
    // forms the PV from it, operators.py:179-180): every point, halo columns
    // included, is evaluated locally with the numpy-slice semantics
    const bool live = j < g.NY && i < g.NX && (a.euler == 3 || periodic_owner(g, i));
    const long long o = (long long)j * g.P + i;
    const uint32_t cd = live ? code[o] : 0u;
    const T* __restrict__ ke = (const T*)a.ke;
    const T* __restrict__ p = (const T*)a.p;

    // du.x: vortex force along y (sign +1), weno.py:370-384 with s = row
    // length, s2 = 1: omega window rows j-2..j+3 at column i.
    T dux = T(0);
    {
        const int L = lev(cd, SH_OVY);
        if (L) {
            const T Vm = wrap ? T(0.25) * (((Uy[o] + ldw(Uy, j + 1, i, g)) +
                                            ldw(Uy, j, i - 1, g)) +
                                           ldw(Uy, j + 1, i - 1, g))
                              : T(0.25) * (((Uy[o] + ldz(Uy, j + 1, i, g)) +
                                            ldz(Uy, j, i - 1, g)) +
                                           ldz(Uy, j + 1, i - 1, g));
            const int c = tx + OX, r = ty + OY;
            dux = face_value<M, T>(L, Vm, sw[r - 2][c], sw[r - 1][c], sw[r][c],
                                   sw[r + 1][c], sw[r + 2][c], sw[r + 3][c]) *
                  Vm;
        }
    }
    // du.y: vortex force along x (sign -1), s = 1, s2 = row length
    T duy = T(0);
    {
        const int L = lev(cd, SH_OVX);
        if (L) {
            const T Vm = wrap ? T(0.25) * (((Ux[o] + ldw(Ux, j, i + 1, g)) +
                                            ldw(Ux, j - 1, i, g)) +
                                           ldw(Ux, j - 1, i + 1, g))
                              : T(0.25) * (((Ux[o] + ldz(Ux, j, i + 1, g)) +
                                            ldz(Ux, j - 1, i, g)) +
                                           ldz(Ux, j - 1, i + 1, g));
            const T* w = &sw[ty + OY][tx + OX - 2];
            duy = -face_value<M, T>(L, Vm, w[0], w[1], w[2], w[3], w[4], w[5]) * Vm;
        }
    }
    if (tx == 0 && ty == 0) {
        rk3_coefs<T>(sk, sc->dt, srk, sc->ragamma);
        srk[3] = T(a.fc);
    }
    __syncthreads();
    if (!live) return;

    // Coriolis (addcoriolis, operators.py:32-39); the euler and boussinesq
    // models (equations.py:11-15, 29-35) have neither Coriolis nor a pressure
    // gradient here, qgrsw (106-125) has Coriolis but no gradient forces
    const T fc = srk[3];
    const bool cor = a.euler == 0 || a.euler == 3;
    if (cor && j <= g.NY - 2 && i >= 1 && i <= g.NX - 2)
        dux += fc * (((ldz(Uy, j, i - 1, g) + ldz(Uy, j + 1, i - 1, g)) + Uy[o]) +
                     ldz(Uy, j + 1, i, g));
    if (cor && j >= 1 && j <= g.NY - 2 && i <= g.NX - 2)
        duy -= fc * (((ldz(Ux, j - 1, i, g) + ldz(Ux, j - 1, i + 1, g)) + Ux[o]) +
                     ldz(Ux, j, i + 1, g));
    // gradients of ke then p (addgrad, operators.py:49-56)
    if (i >= 1 && a.euler != 3) {
        const T mx = (cd & B_MSKX) ? T(1) : T(0);
        dux -= (ke[o] - ke[o - 1]) * mx;
        if (a.euler == 0) dux -= (p[o] - p[o - 1]) * mx;
    }
    if (j >= 1 && a.euler != 3) {
        const T my = (cd & B_MSKY) ? T(1) : T(0);
        duy -= (ke[o] - ke[o - g.P]) * my;
        if (a.euler == 0) duy -= (p[o] - p[o - g.P]) * my;
        // boussinesq buoyancy (operators.py:152-153), after the gradients
        if (a.euler == 2)
            duy += (T(a.bdy) * (sh[ty + OY][tx + OX] + sh[ty + OY - 1][tx + OX])) * my;
    }
    // mass: dh = -div(flux) * msk
    const T msk = (cd & B_MSK) ? T(1) : T(0);
    T dh = (-(sfx[ty][tx + 1] - sfx[ty][tx]) - (sfy[ty + 1][tx] - sfy[ty][tx])) * msk;
    const bool hm = a.euler != 1;  // mass (rsw) or buoyancy (boussinesq) equation
    if (a.fx && a.euler != 3) {
        // the forcing term after the right-hand side (equations.py:229-238)
        dux += ((const T*)a.fx)[o];
        duy += ((const T*)a.fy)[o];
        if (hm) dh += ((const T*)a.fh)[o];
    }
    if (((sk >> 4) & 15) == INTEG_TENDENCY && a.euler != 3) {
        // the tendency alone, with the halo fill of the reference's rhs
        store_filled((T*)a.dux, g, j, i, dux);
        store_filled((T*)a.duy, g, j, i, duy);
        if (hm) store_filled((T*)a.dh, g, j, i, dh);
        return;
    }
    if (a.euler == 3) {
        // qgrsw: the raw tendency, projected by the Helmholtz solve before
        // the integrator update
        ((T*)a.dux)[o] = dux;
        ((T*)a.duy)[o] = duy;
        ((T*)a.dh)[o] = dh;
        return;
    }

    const T* dt = srk;
    T ix, iy, ih = T(0);
    if (lf) {
        // leap-frog + Robert-Asselin: dux1.. = filtered previous state in,
        // dux.. = out (buffers alternating with the parity)
        const bool first = sc->ite == 0;
        T qn, pn;
        lfra_update<T>(first, srk, ((const T*)a.ux)[o], ((const T*)a.dux1)[o], dux, qn, pn);
        store_filled((T*)a.uxo, g, j, i, qn);
        store_filled((T*)a.dux, g, j, i, pn);
        lfra_update<T>(first, srk, ((const T*)a.uy)[o], ((const T*)a.duy1)[o], duy, qn, pn);
        store_filled((T*)a.uyo, g, j, i, qn);
        store_filled((T*)a.duy, g, j, i, pn);
        if (hm) {
            lfra_update<T>(first, srk, sh[ty + OY][tx + OX], ((const T*)a.dh1)[o], dh, qn, pn);
            store_filled((T*)a.ho, g, j, i, qn);
            store_filled((T*)a.dh, g, j, i, pn);
        }
        return;
    }
    if (stage == 1) {
        ix = rk3_increment<T>(1, dt, dux, T(0), T(0));
        iy = rk3_increment<T>(1, dt, duy, T(0), T(0));
        if (hm) ih = rk3_increment<T>(1, dt, dh, T(0), T(0));
    } else if (stage == 2) {
        ix = rk3_increment<T>(2, dt, ((const T*)a.dux1)[o], dux, T(0));
        iy = rk3_increment<T>(2, dt, ((const T*)a.duy1)[o], duy, T(0));
        if (hm) ih = rk3_increment<T>(2, dt, ((const T*)a.dh1)[o], dh, T(0));
    } else {
        ix = rk3_increment<T>(3, dt, ((const T*)a.dux1)[o], ((const T*)a.dux2)[o], dux);
        iy = rk3_increment<T>(3, dt, ((const T*)a.duy1)[o], ((const T*)a.duy2)[o], duy);
        if (hm) ih = rk3_increment<T>(3, dt, ((const T*)a.dh1)[o], ((const T*)a.dh2)[o], dh);
    }
    store_filled((T*)a.uxo, g, j, i, ((const T*)a.ux)[o] + ix);
    store_filled((T*)a.uyo, g, j, i, ((const T*)a.uy)[o] + iy);
    if (hm) store_filled((T*)a.ho, g, j, i, sh[ty + OY][tx + OX] + ih);
    if (a.dux) {
        store_filled((T*)a.dux, g, j, i, dux);
        store_filled((T*)a.duy, g, j, i, duy);
        if (hm) store_filled((T*)a.dh, g, j, i, dh);
    }
}

// ---------------------------------------------------------------------------
// Rotating shallow water diagnostics (equations.py:150-155): sharp, vorticity
// (times slip coefficient), WENO kinetic energy, pressure; omega and ke get
// the halo fill.
// ---------------------------------------------------------------------------
template <typename T, int M>
__global__ void __launch_bounds__(TX * TY)
k_rsw_diag(const __grid_constant__ CUtensorMap tux,
           const __grid_constant__ CUtensorMap tuy, RswDiag a,
           const uint32_t* __restrict__ code, Geom g, DevScalars* sc)
{
    __shared__ alignas(128) T sx[SH][SW];
    __shared__ alignas(128) T sy[SH][SW];
    __shared__ uint64_t bar;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    if (!stage_tiles<T>(sx, &tux, sy, &tuy, i0, j0, &bar, &sc->status)) return;

    const int j = j0 + ty, i = i0 + tx;
    if (j >= g.NY || i >= g.NX) return;
    const long long o = (long long)j * g.P + i;
    const int r = ty + OY, c = tx + OX;
    const T rdx2 = T(a.rdx2), rdy2 = T(a.rdy2);
    const T ux = sx[r][c], uy = sy[r][c];
    // sharp: U = u / dx^2 everywhere (no fill in the reference; u is filled)
    ((T*)a.Ux)[o] = ux * rdx2;
    ((T*)a.Uy)[o] = uy * rdy2;
    if (!a.euler) ((T*)a.p)[o] = T(a.goa) * ((const T*)a.h)[o];
    if (!periodic_owner(g, i)) return;  // omega and ke: halo fill copies
    const uint32_t cd = code[o];
    // vorticity: omega[1:,:] = -diff(u.x, 0); omega[:,1:] += diff(u.y, 1)
    T om = T(0);
    if (j >= 1) om = -(ux - sx[r - 1][c]);
    if (i >= 1) om += uy - sy[r][c - 1];
    om *= (cd & B_SLIP) ? T(1) : T(0);
    if (a.noke) {
        store_filled((T*)a.omega, g, j, i, om);
        return;
    }
    T ke = T(0);
    if constexpr (M == METHOD_CLASSIC) {
        // innerproduct="classic" (operators.py:86-90): u.x U.x at the cell's
        // two x-faces (ke[:, :-1]), plus u.y U.y at its two y-faces
        // (ke[:-1, :]), times msk*0.25; U is the sharp of u as stored above
        if (i <= g.NX - 2) {
            const T a = sx[r][c + 1];
            ke = a * (a * rdx2) + ux * (ux * rdx2);
        }
        if (j <= g.NY - 2) {
            const T b = sy[r + 1][c];
            ke += b * (b * rdy2) + uy * (uy * rdy2);
        }
        ke *= (cd & B_MSK) ? T(0.25) : T(0);
    } else {
        // kinetic energy: innerproduct x then y, times msk*0.5 (operators.py:94-96)
        {
            const int L = lev(cd, SH_OKX);
            if (L) {
                const T Um = T(0.5) * (ux * rdx2 + sx[r][c + 1] * rdx2);
                const T* w = &sx[r][c - 2];
                ke = face_value<M, T>(L, Um, w[0], w[1], w[2], w[3], w[4], w[5]) * Um;
            }
        }
        {
            const int L = lev(cd, SH_OKY);
            if (L) {
                const T Um = T(0.5) * (uy * rdy2 + sy[r + 1][c] * rdy2);
                ke += face_value<M, T>(L, Um, sy[r - 2][c], sy[r - 1][c], sy[r][c],
                                       sy[r + 1][c], sy[r + 2][c], sy[r + 3][c]) *
                      Um;
            }
        }
        ke *= (cd & B_MSK) ? T(0.5) : T(0);
    }
    store_filled((T*)a.omega, g, j, i, om);
    store_filled((T*)a.ke, g, j, i, ke);
}

// ---------------------------------------------------------------------------
// Vertex diagnostics of eulerpsi/qg.
// ---------------------------------------------------------------------------

// centerstovertices (operators.py:126-133) and, for qg with beta != 0, the
// subtraction of the vertex Coriolis term (qg_inversion, operators.py:186-191)
// (the average is formed in the output precision: FP64 right-hand side of
// the Poisson solve from an FP32 state in the mixed-precision form)
template <typename Tin, typename T>
__global__ void k_c2v(const Tin* __restrict__ q, T* __restrict__ v,
                      const uint32_t* __restrict__ code, const T* __restrict__ fv,
                      Geom g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.NX) return;
    // the loads of all the thread's rows first (clamped indices, the mask
    // applied after): one memory round trip
    uint32_t cd[FRT];
    Tin a0[FRT], a1[FRT], a2[FRT], a3[FRT];
#pragma unroll
    for (int r = 0; r < FRT; ++r) {
        const int j = min(blockIdx.y * FTY + threadIdx.y + 8 * r, g.NY - 1);
        const int jm = max(j - 1, 0), im = max(i - 1, 0);
        const long long o = (long long)j * g.P + i, om = (long long)jm * g.P;
        cd[r] = code[o];
        a0[r] = q[om + im];
        a1[r] = q[(long long)j * g.P + im];
        a2[r] = q[om + i];
        a3[r] = q[o];
    }
#pragma unroll
    for (int r = 0; r < FRT; ++r) {
        const int j = blockIdx.y * FTY + threadIdx.y + 8 * r;
        if (j >= g.NY) break;
        const long long o = (long long)j * g.P + i;
        Tin a = Tin(0);
        if (j >= 1 && i >= 1 && (cd[r] & B_MSKV))
            a = Tin(0.25) * (((a0[r] + a1[r]) + a2[r]) + a3[r]);
        T b = conv<T>(a);
        if (fv) b -= fv[o];
        v[o] = b;
    }
}

// perpgrad with contravariant scaling (operators.py:144-149), optional halo
// fill of U (eulerpsi fills, qg does not), and max|U.x|, max|U.y| for set_dt.
template <typename P, typename T>
__global__ void k_perpgrad(const P* __restrict__ psi, T* __restrict__ Ux,
                           T* __restrict__ Uy, const uint32_t* __restrict__ code,
                           T rdy2, T rdx2, int fillU, Geom g,
                           DevScalars* sc, double* partials)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    T m[2] = {T(0), T(0)};
    // the loads of all the thread's rows first (clamped indices): one round trip
    const int ic = min(i, g.NX - 1);
    uint32_t cdv[FRT];
    P p0[FRT], pn[FRT], pe[FRT];
#pragma unroll
    for (int r = 0; r < FRT; ++r) {
        const int jc = min(blockIdx.y * FTY + threadIdx.y + 8 * r, g.NY - 1);
        const long long o = (long long)jc * g.P + ic;
        cdv[r] = code[o];
        p0[r] = psi[o];
        pn[r] = psi[(long long)min(jc + 1, g.NY - 1) * g.P + ic];
        pe[r] = psi[(long long)jc * g.P + min(ic + 1, g.NX - 1)];
    }
#pragma unroll
    for (int r = 0; r < FRT; ++r) {
        const int j = blockIdx.y * FTY + threadIdx.y + 8 * r;
        if (j >= g.NY || i >= g.NX) continue;
        const long long o = (long long)j * g.P + i;
        const bool own = !fillU || periodic_owner(g, i);
        if (own) {
            // the difference in the precision of psi, the scaling in that of U
            const uint32_t cd = cdv[r];
            T ux = T(0), uy = T(0);
            if (j <= g.NY - 2 && (cd & B_MSKX)) ux = -conv<T>(pn[r] - p0[r]) * rdy2;
            if (i <= g.NX - 2 && (cd & B_MSKY)) uy = conv<T>(pe[r] - p0[r]) * rdx2;
            if (fillU) {
                store_filled(Ux, g, j, i, ux);
                store_filled(Uy, g, j, i, uy);
            } else {
                Ux[o] = ux;
                Uy[o] = uy;
            }
            m[0] = nanmax(m[0], fabs(ux));
            m[1] = nanmax(m[1], fabs(uy));
        }
    }
    // the block's maxima only (no fence or ticket: k_umax_finish combines)
    double w[2];
    if constexpr (std::is_same<T, float>::value) {
        block_total_f<2, true>(m, w);
    } else {
        __shared__ double sh[64];
        w[0] = m[0];
        w[1] = m[1];
        block_reduce<2, true>(w, sh);
    }
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        const size_t b = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
        partials[2 * b] = w[0];
        partials[2 * b + 1] = w[1];
    }
}

// max|U.x|, max|U.y| from k_perpgrad's nb block maxima (NaN propagates)
__global__ void __launch_bounds__(256) k_umax_finish(const double* __restrict__ partials,
                                                      int nb, DevScalars* sc)
{
    double acc[2];
    final_sum<2, true>(acc, partials, 0, nb, threadIdx.x, blockDim.x);
    __shared__ double sh[64];
    block_reduce<2, true>(acc, sh);
    if (threadIdx.x == 0) {
        sc->maxUx = acc[0];
        sc->maxUy = acc[1];
    }
}

// max |U.x|, max |U.y| of fields written by the host
template <typename T>
__global__ void k_maxabs2(const T* __restrict__ Ux, const T* __restrict__ Uy,
                          Geom g, DevScalars* sc, double* partials)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    double m[2] = {0.0, 0.0};
    if (j < g.NY && i < g.NX) {
        const long long o = (long long)j * g.P + i;
        m[0] = fabs((double)Ux[o]);
        m[1] = fabs((double)Uy[o]);
    }
    if (grid_reduce<2, true>(m, partials, &sc->counter[0])) {
        sc->maxUx = m[0];
        sc->maxUy = m[1];
    }
}

// precision conversion between pitched arrays (field I/O of FP32 models)
template <typename Tin, typename Tout>
__global__ void k_convert(const Tin* __restrict__ in, Tout* __restrict__ out, Geom g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= g.NY || i >= g.NX) return;
    const long long o = (long long)j * g.P + i;
    out[o] = Tout(in[o]);
}

// periodic halo fill (meshes.py:135-143) of one array
template <typename T>
__global__ void k_fill_periodic(T* __restrict__ a, Geom g)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;  // 0..5 per row
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= g.NY || k >= 6) return;
    const long long r = (long long)j * g.P;
    if (k < 3) a[r + k] = a[r + g.NX - 6 + k];
    else a[r + g.NX - 6 + k] = a[r + k];  // columns NX-3.. <- 3..
}

// set_dt (model.py:71-87) from the device-side max|U|
__global__ void k_set_dt(DevScalars* sc)
{
    const double maxU = sc->maxUx + sc->maxUy + 1e-99;
    const double dt = pymin(sc->cfl / maxU, sc->dtmax);
    sc->dt = dt;
    if (!(dt == dt)) sc->status |= ST_NONFINITE;  // a NaN velocity
}

// Time.pushforward (timeline.py:20-35): Kahan-summed t, ite += 1
__global__ void k_pushforward(DevScalars* sc)
{
    const double y = sc->dt - sc->c;
    const double t = sc->t + y;
    sc->c = (t - sc->t) - y;
    sc->t = t;
    sc->ite += 1;
}

// ---------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------
static dim3 tile_grid(const Geom& g)
{
    return dim3((g.NX + TX - 1) / TX, (g.NY + TY - 1) / TY);
}

static dim3 ftile_grid(const Geom& g)
{
    return dim3((g.NX + TX - 1) / TX, (g.NY + FTY - 1) / FTY);
}

int launch_fluxform_stage(int method, int prec, const CUtensorMap* tq,
                          const void* qin, void* qout, const void* Ux,
                          const void* Uy, const uint32_t* code, void* ds_out,
                          const void* ds1, const void* ds2, const void* frc, int stage,
                          const Geom& g, DevScalars* sc, cudaStream_t s)
{
    dim3 grid = ftile_grid(g), block(TX, TY);
#define F2D_FF(T, M)                                                              \
    k_fluxform_stage<T, M><<<grid, block, 0, s>>>(                                \
        *tq, (const T*)qin, (T*)qout, (const T*)Ux, (const T*)Uy, code, (T*)ds_out, \
        (const T*)ds1, (const T*)ds2, (const T*)frc, stage, g, sc)
#define F2D_DISPATCH(T)                                                  \
    switch (method) {                                                    \
    case METHOD_WENO: F2D_FF(T, METHOD_WENO); break;                     \
    case METHOD_UPWIND: F2D_FF(T, METHOD_UPWIND); break;                 \
    case METHOD_CENTERED: F2D_FF(T, METHOD_CENTERED); break;             \
    default: F2D_FF(T, METHOD_CWENO); break;                             \
    }
    if (prec == 0) { F2D_DISPATCH(double) } else { F2D_DISPATCH(float) }
#undef F2D_DISPATCH
#undef F2D_FF
    return (int)cudaGetLastError();
}

int launch_rsw_stage(int method, int prec, const CUtensorMap* th,
                     const CUtensorMap* tw, const RswIn& a, const uint32_t* code,
                     int stage, const Geom& g, DevScalars* sc, cudaStream_t s)
{
    dim3 grid = tile_grid(g), block(TX, TY);
#define F2D_RS(T, M) k_rsw_stage<T, M><<<grid, block, 0, s>>>(*th, *tw, a, code, stage, g, sc)
#define F2D_DISPATCH(T)                                      \
    switch (method) {                                        \
    case METHOD_WENO: F2D_RS(T, METHOD_WENO); break;         \
    case METHOD_UPWIND: F2D_RS(T, METHOD_UPWIND); break;     \
    case METHOD_CENTERED: F2D_RS(T, METHOD_CENTERED); break; \
    default: F2D_RS(T, METHOD_CWENO); break;                 \
    }
    if (prec == 0) { F2D_DISPATCH(double) } else { F2D_DISPATCH(float) }
#undef F2D_DISPATCH
#undef F2D_RS
    return (int)cudaGetLastError();
}

int launch_rsw_diag(int method, int prec, const CUtensorMap* tux,
                    const CUtensorMap* tuy, const RswDiag& a, const uint32_t* code,
                    const Geom& g, DevScalars* sc, cudaStream_t s)
{
    dim3 grid = tile_grid(g), block(TX, TY);
#define F2D_RD(T, M) k_rsw_diag<T, M><<<grid, block, 0, s>>>(*tux, *tuy, a, code, g, sc)
#define F2D_DISPATCH(T)                                      \
    switch (method) {                                        \
    case METHOD_WENO: F2D_RD(T, METHOD_WENO); break;         \
    case METHOD_UPWIND: F2D_RD(T, METHOD_UPWIND); break;     \
    case METHOD_CENTERED: F2D_RD(T, METHOD_CENTERED); break; \
    case METHOD_CLASSIC: F2D_RD(T, METHOD_CLASSIC); break;   \
    default: F2D_RD(T, METHOD_CWENO); break;                 \
    }
    if (prec == 0) { F2D_DISPATCH(double) } else { F2D_DISPATCH(float) }
#undef F2D_DISPATCH
#undef F2D_RD
    return (int)cudaGetLastError();
}

static dim3 pt_grid(const Geom& g) { return dim3((g.NX + 31) / 32, (g.NY + 7) / 8); }
// 32 x 32 points per block, FRT rows per thread
static dim3 pt4_grid(const Geom& g) { return dim3((g.NX + 31) / 32, (g.NY + FTY - 1) / FTY); }

int launch_c2v(int prec_in, int prec_out, const void* q, void* v, const uint32_t* code,
               const void* fv, const Geom& g, cudaStream_t s)
{
    const dim3 gr = pt4_grid(g), bl(32, 8);
    if (prec_in == 0 && prec_out == 0)
        k_c2v<double, double><<<gr, bl, 0, s>>>((const double*)q, (double*)v, code,
                                                (const double*)fv, g);
    else if (prec_in == 1 && prec_out == 0)
        k_c2v<float, double><<<gr, bl, 0, s>>>((const float*)q, (double*)v, code,
                                               (const double*)fv, g);
    else
        k_c2v<float, float><<<gr, bl, 0, s>>>((const float*)q, (float*)v, code,
                                              (const float*)fv, g);
    return (int)cudaGetLastError();
}

int launch_perpgrad(int prec_psi, int prec_U, const void* psi, void* Ux, void* Uy,
                    const uint32_t* code, double rdy2, double rdx2, int fillU,
                    const Geom& g, DevScalars* sc, double* partials, cudaStream_t s)
{
    const dim3 gr = pt4_grid(g), bl(32, 8);
    if (prec_psi == 0 && prec_U == 0)
        k_perpgrad<double, double><<<gr, bl, 0, s>>>((const double*)psi, (double*)Ux,
                                                     (double*)Uy, code, rdy2, rdx2, fillU,
                                                     g, sc, partials);
    else if (prec_psi == 0 && prec_U == 1)
        k_perpgrad<double, float><<<gr, bl, 0, s>>>((const double*)psi, (float*)Ux,
                                                    (float*)Uy, code, rdy2, rdx2, fillU, g,
                                                    sc, partials);
    else
        k_perpgrad<float, float><<<gr, bl, 0, s>>>((const float*)psi, (float*)Ux,
                                                   (float*)Uy, code, rdy2, rdx2, fillU, g,
                                                   sc, partials);
    k_umax_finish<<<1, 256, 0, s>>>(partials, (int)(gr.x * gr.y), sc);
    return (int)cudaGetLastError();
}

int launch_convert(int prec_in, int prec_out, const void* in, void* out, const Geom& g,
                   cudaStream_t s)
{
    const dim3 gr = pt_grid(g), bl(32, 8);
    if (prec_in == 0 && prec_out == 1)
        k_convert<double, float><<<gr, bl, 0, s>>>((const double*)in, (float*)out, g);
    else if (prec_in == 1 && prec_out == 0)
        k_convert<float, double><<<gr, bl, 0, s>>>((const float*)in, (double*)out, g);
    else
        return 1;
    return (int)cudaGetLastError();
}

int launch_maxabs2(int prec, const void* Ux, const void* Uy, const Geom& g,
                   DevScalars* sc, double* partials, cudaStream_t s)
{
    if (prec == 0)
        k_maxabs2<double><<<pt_grid(g), dim3(32, 8), 0, s>>>(
            (const double*)Ux, (const double*)Uy, g, sc, partials);
    else
        k_maxabs2<float><<<pt_grid(g), dim3(32, 8), 0, s>>>(
            (const float*)Ux, (const float*)Uy, g, sc, partials);
    return (int)cudaGetLastError();
}

int launch_fill_periodic(int prec, void* a, const Geom& g, cudaStream_t s)
{
    if (!g.xper) return 0;
    dim3 grid(1, (g.NY + 31) / 32), block(8, 32);
    if (prec == 0) k_fill_periodic<double><<<grid, block, 0, s>>>((double*)a, g);
    else k_fill_periodic<float><<<grid, block, 0, s>>>((float*)a, g);
    return (int)cudaGetLastError();
}

// Warm start of the Poisson solve of SSP-RK3 stage mode+1 (psi_warm_point,
// stage.cuh): a grid-stride loop over every element.
__global__ void k_psi_warm(int mode, WarmArrays w, long long n, DevScalars* sc)
{
    const bool hist = sc->dt_warm > 0.0;
    const double rho = hist ? sc->dt / sc->dt_warm : 0.0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        psi_warm_point(mode, w, k, hist, rho);
    if (mode == 2 && blockIdx.x == 0 && threadIdx.x == 0) sc->dt_warm = sc->dt;
}

int launch_psi_warm(int mode, const WarmArrays& w, long long n, DevScalars* sc, cudaStream_t s)
{
    const int nb = (int)std::min<long long>((n + 255) / 256, 152 * 8);
    k_psi_warm<<<nb, 256, 0, s>>>(mode, w, n, sc);
    return (int)cudaGetLastError();
}

// the TMA wait test switch of this translation unit's stage kernels
int tma_wait_test_set_stage(int enabled, unsigned long long limit_ns)
{
    TmaWaitTest v;
    v.enabled = enabled ? 1u : 0u;
    v.pad = 0;
    v.limit_ns = limit_ns;
    return (int)cudaMemcpyToSymbol(g_tma_wait_test, &v, sizeof(v));
}

int launch_set_dt(DevScalars* sc, cudaStream_t s)
{
    k_set_dt<<<1, 1, 0, s>>>(sc);
    return (int)cudaGetLastError();
}

int launch_pushforward(DevScalars* sc, cudaStream_t s)
{
    k_pushforward<<<1, 1, 0, s>>>(sc);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// euler model: the pressure projection around the Neumann solve
// (pressure_projection, operators.py:114-119).
// ---------------------------------------------------------------------------

// U = sharp(u) (computed on the fly), delta = div(U) * msk into dv - whose
// last column keeps its previous value, like the reference's div
// (operators.py:104-107) - and the solve's right-hand side -delta * area
template <typename T>
__global__ void k_euler_div(const T* __restrict__ ux, const T* __restrict__ uy, T* dv,
                            double* __restrict__ rhs, const uint32_t* __restrict__ code,
                            T rdx2, T rdy2, double area, Geom g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= g.NY || i >= g.NX) return;
    const long long o = (long long)j * g.P + i;
    T d = i <= g.NX - 2 ? -(ux[o + 1] * rdx2 - ux[o] * rdx2) : dv[o];
    if (j <= g.NY - 2) d -= uy[o + g.P] * rdy2 - uy[o] * rdy2;
    d *= (code[o] & B_MSK) ? T(1) : T(0);
    dv[o] = d;
    rhs[o] = -(double)d * area;
}

// u -= grad p (addgrad, operators.py:49-53), then the halo fill of u
template <typename T>
__global__ void k_euler_project(T* ux, T* uy, const double* __restrict__ p,
                                const uint32_t* __restrict__ code, Geom g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= g.NY || i >= g.NX || !periodic_owner(g, i)) return;
    const long long o = (long long)j * g.P + i;
    const uint32_t cd = code[o];
    T vx = ux[o], vy = uy[o];
    if (i >= 1) vx -= T((p[o] - p[o - 1]) * ((cd & B_MSKX) ? 1.0 : 0.0));
    if (j >= 1) vy -= T((p[o] - p[o - g.P]) * ((cd & B_MSKY) ? 1.0 : 0.0));
    store_filled(ux, g, j, i, vx);
    store_filled(uy, g, j, i, vy);
}

int launch_euler_div(int prec, const void* ux, const void* uy, void* dv, double* rhs,
                     const uint32_t* code, double rdx2, double rdy2, double area,
                     const Geom& g, cudaStream_t s)
{
    const dim3 gr = pt_grid(g), bl(32, 8);
    if (prec == 0)
        k_euler_div<double><<<gr, bl, 0, s>>>((const double*)ux, (const double*)uy, (double*)dv,
                                              rhs, code, rdx2, rdy2, area, g);
    else
        k_euler_div<float><<<gr, bl, 0, s>>>((const float*)ux, (const float*)uy, (float*)dv, rhs,
                                             code, (float)rdx2, (float)rdy2, area, g);
    return (int)cudaGetLastError();
}

int launch_euler_project(int prec, void* ux, void* uy, const double* p, const uint32_t* code,
                         const Geom& g, cudaStream_t s)
{
    const dim3 gr = pt_grid(g), bl(32, 8);
    if (prec == 0)
        k_euler_project<double><<<gr, bl, 0, s>>>((double*)ux, (double*)uy, p, code, g);
    else
        k_euler_project<float><<<gr, bl, 0, s>>>((float*)ux, (float*)uy, p, code, g);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// qgrsw: projection of the RSW tendency on the QG manifold (qg_projection,
// operators.py:176-211) around the Helmholtz solve of the vertex PV.
// ---------------------------------------------------------------------------

// pv = compute_vorticity(u) * slipcoef (operators.py:67-77), then
// pv[1:, 1:] += 0.25 * sum of the four (h - h0) * cs around the vertex and
// pv *= mskv (add_stretching, 194-201 with centerstovertices(addto), 126-133);
// cs = -f0/H. Row 0 is 0 (slipcoef is 0 there). FP64 out.
template <typename T>
__global__ void k_qgrsw_pv(const T* __restrict__ ux, const T* __restrict__ uy,
                           const T* __restrict__ h, double* __restrict__ pv,
                           const uint32_t* __restrict__ code, double cs, double h0, Geom g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= g.NY || i >= g.NX) return;
    const long long o = (long long)j * g.P + i;
    const uint32_t cd = code[o];
    double v = 0.0;
    if (j >= 1) v = -((double)ux[o] - (double)ux[o - g.P]);
    if (i >= 1) v += (double)uy[o] - (double)uy[o - 1];
    v *= (cd & B_SLIP) ? 1.0 : 0.0;
    if (j >= 1 && i >= 1) {
        const double a00 = ((double)h[o - g.P - 1] - h0) * cs;
        const double a10 = ((double)h[o - 1] - h0) * cs;
        const double a01 = ((double)h[o - g.P] - h0) * cs;
        const double a11 = ((double)h[o] - h0) * cs;
        v += 0.25 * (((a00 + a10) + a01) + a11);
    }
    pv[o] = v * ((cd & B_MSKV) ? 1.0 : 0.0);
}

// From the solution psi: u = perpgrad(psi) (operators.py:144-146, not
// contravariant), h = verticestocenters(psi * c2) (136-141; + h0 in the state
// form) times msk (thickness_from_psi, 204-211). Points the reference does
// not assign (the last row of u.x, the last column of u.y, the last row and
// column of h) keep their incoming value. A cell with no wet vertex gets 0
// where the reference's (1/0) * 0 gives nan (a land cell).
// Mode 0: the projected tendency is filled (equations.py:124: x-periodic
// halo columns are copies of the interior columns), and the integrator (RK3
// increment, or the LFRA step) updates EVERY point of the state from its own
// value, as the reference's addto does over the whole array: the state's
// halo columns are not refilled (they need not be copies of the interior).
// Mode 1 (the state form, no fill): every point evaluated locally, in place.
template <typename T>
__device__ __forceinline__ void qg_project_point(const QgProj& a, const double* psi,
                                                 const uint32_t* code, const Geom& g,
                                                 int j, int i, T& dux, T& duy, T& dh)
{
    const long long o = (long long)j * g.P + i;
    const uint32_t cd = code[o];
    dux = ((const T*)a.cx)[o];
    duy = ((const T*)a.cy)[o];
    dh = ((const T*)a.ch)[o];
    if (j <= g.NY - 2) dux = T(-(psi[o + g.P] - psi[o]) * ((cd & B_MSKX) ? 1.0 : 0.0));
    if (i <= g.NX - 2) duy = T((psi[o + 1] - psi[o]) * ((cd & B_MSKY) ? 1.0 : 0.0));
    double hv = (double)dh;
    if (j <= g.NY - 2 && i <= g.NX - 2) {
        const int coef = ((code[o] & B_MSKV) ? 1 : 0) + ((code[o + g.P] & B_MSKV) ? 1 : 0) +
                         ((code[o + 1] & B_MSKV) ? 1 : 0) +
                         ((code[o + g.P + 1] & B_MSKV) ? 1 : 0);
        const double sum = ((psi[o] * a.c2 + psi[o + g.P] * a.c2) + psi[o + 1] * a.c2) +
                           psi[o + g.P + 1] * a.c2;
        hv = coef ? (1.0 / coef) * sum : 0.0;
    }
    dh = T((hv + a.h0) * ((cd & B_MSK) ? 1.0 : 0.0));
}

template <typename T>
__global__ void k_qgrsw_update(QgProj a, const double* __restrict__ psi,
                               const uint32_t* __restrict__ code, int sk, Geom g,
                               DevScalars* sc)
{
    __shared__ T c[3];
    const bool lf = ((sk >> 4) & 15) == 3;
    const int stage = sk & 15;
    if (threadIdx.x == 0 && threadIdx.y == 0 && a.mode == 0)
        rk3_coefs<T>(sk, sc->dt, c, sc->ragamma);
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= g.NY || i >= g.NX) return;
    const long long o = (long long)j * g.P + i;
    T dux, duy, dh;
    if (a.mode == 1) {
        qg_project_point<T>(a, psi, code, g, j, i, dux, duy, dh);
        ((T*)a.cx)[o] = dux;
        ((T*)a.cy)[o] = duy;
        ((T*)a.ch)[o] = dh;
        return;
    }
    // the filled tendency: a periodic halo column takes its interior copy's
    const int io = !g.xper ? i : i < 3 ? i + g.nx : i >= g.nx + 3 ? i - g.nx : i;
    qg_project_point<T>(a, psi, code, g, j, io, dux, duy, dh);
    if (a.fx) {
        // the forcing term after the projected right-hand side
        // (equations.py:229-238), at every point as the reference adds it
        dux += ((const T*)a.fx)[o];
        duy += ((const T*)a.fy)[o];
        dh += ((const T*)a.fh)[o];
    }
    if (a.mode == 2) {
        // the projected tendency alone (the reference's qgrsw rhs)
        ((T*)a.sx)[o] = dux;
        ((T*)a.sy)[o] = duy;
        ((T*)a.sh)[o] = dh;
        return;
    }
    const T ux = ((const T*)a.ux)[o], uy = ((const T*)a.uy)[o], h = ((const T*)a.h)[o];
    if (lf) {
        const bool first = sc->ite == 0;
        T qn, pn;
        lfra_update<T>(first, c, ux, ((const T*)a.d1x)[o], dux, qn, pn);
        ((T*)a.uxo)[o] = qn;
        ((T*)a.px)[o] = pn;
        lfra_update<T>(first, c, uy, ((const T*)a.d1y)[o], duy, qn, pn);
        ((T*)a.uyo)[o] = qn;
        ((T*)a.py)[o] = pn;
        lfra_update<T>(first, c, h, ((const T*)a.d1h)[o], dh, qn, pn);
        ((T*)a.ho)[o] = qn;
        ((T*)a.ph)[o] = pn;
        return;
    }
    T ix, iy, ih;
    if (stage == 1) {
        ix = rk3_increment<T>(1, c, dux, T(0), T(0));
        iy = rk3_increment<T>(1, c, duy, T(0), T(0));
        ih = rk3_increment<T>(1, c, dh, T(0), T(0));
    } else if (stage == 2) {
        ix = rk3_increment<T>(2, c, ((const T*)a.d1x)[o], dux, T(0));
        iy = rk3_increment<T>(2, c, ((const T*)a.d1y)[o], duy, T(0));
        ih = rk3_increment<T>(2, c, ((const T*)a.d1h)[o], dh, T(0));
    } else {
        ix = rk3_increment<T>(3, c, ((const T*)a.d1x)[o], ((const T*)a.d2x)[o], dux);
        iy = rk3_increment<T>(3, c, ((const T*)a.d1y)[o], ((const T*)a.d2y)[o], duy);
        ih = rk3_increment<T>(3, c, ((const T*)a.d1h)[o], ((const T*)a.d2h)[o], dh);
    }
    ((T*)a.uxo)[o] = ux + ix;
    ((T*)a.uyo)[o] = uy + iy;
    ((T*)a.ho)[o] = h + ih;
    if (a.store) {
        ((T*)a.sx)[o] = dux;
        ((T*)a.sy)[o] = duy;
        ((T*)a.sh)[o] = dh;
    }
}

int launch_qgrsw_pv(int prec, const void* ux, const void* uy, const void* h, double* pv,
                    const uint32_t* code, double cs, double h0, const Geom& g, cudaStream_t s)
{
    const dim3 gr = pt_grid(g), bl(32, 8);
    if (prec == 0)
        k_qgrsw_pv<double><<<gr, bl, 0, s>>>((const double*)ux, (const double*)uy,
                                             (const double*)h, pv, code, cs, h0, g);
    else
        k_qgrsw_pv<float><<<gr, bl, 0, s>>>((const float*)ux, (const float*)uy,
                                            (const float*)h, pv, code, cs, h0, g);
    return (int)cudaGetLastError();
}

int launch_qgrsw_update(int prec, const QgProj& a, const double* psi, const uint32_t* code,
                        int stage, const Geom& g, DevScalars* sc, cudaStream_t s)
{
    const dim3 gr = pt_grid(g), bl(32, 8);
    if (prec == 0) k_qgrsw_update<double><<<gr, bl, 0, s>>>(a, psi, code, stage, g, sc);
    else k_qgrsw_update<float><<<gr, bl, 0, s>>>(a, psi, code, stage, g, sc);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Bulk diagnostics (Bulk.__call__, diagnostics.py:39-57): domain sums over
// the whole array of ke, omega^2, omega, U.y * xv and U.x * yu (xv, yu: the
// y-face x and x-face y coordinates, meshes.py:57-68), divided by sum(msk);
// the last block appends {t, ke, ens, vort, angular} to the device ring.
// The grid strides over rows so that 5 partials per block fit the model's
// reduction scratch.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_bulk(BulkArgs a, Geom g, DevScalars* sc, double* partials)
{
    double w[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g.NX) {
        const T* ke = (const T*)a.ke;
        const T* om = (const T*)a.omega;
        const T* ux = (const T*)a.Ux;
        const T* uy = (const T*)a.Uy;
        const double xv = (i - 3 + 0.5) * a.dx;
        for (int j = blockIdx.y * blockDim.y + threadIdx.y; j < g.NY;
             j += gridDim.y * blockDim.y) {
            const long long o = (long long)j * g.P + i;
            const double yu = (j - 3 + 0.5) * a.dy;
            const double w0 = (double)om[o];
            w[0] += (double)ke[o];
            w[1] += w0 * w0;
            w[2] += w0;
            w[3] += (double)uy[o] * xv;
            w[4] += (double)ux[o] * yu;
        }
    }
    if (grid_reduce<5, false>(w, partials, &sc->counter[6])) {
        const int k = *a.count;
        if (k < a.cap) {
            double* r = a.ring + 5 * (size_t)k;
            const double S = a.summsk;
            r[0] = sc->t;
            r[1] = w[0] / S;
            r[2] = 0.5 * (w[1] / S) / (a.area * a.area);
            r[3] = (w[2] / S) / a.area;
            r[4] = (w[3] / S) * a.dx - (w[4] / S) * a.dy;
            *a.count = k + 1;
        }
    }
}

int launch_bulk(int prec, const BulkArgs& a, const Geom& g, DevScalars* sc, double* partials,
                cudaStream_t s)
{
    const dim3 full = pt_grid(g);
    const dim3 gr(full.x, max(1u, full.y / 2)), bl(32, 8);
    if (prec == 0) k_bulk<double><<<gr, bl, 0, s>>>(a, g, sc, partials);
    else k_bulk<float><<<gr, bl, 0, s>>>(a, g, sc, partials);
    return (int)cudaGetLastError();
}

template <typename T>
__global__ void k_to_f32(const T* __restrict__ in, float* __restrict__ out, Geom g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (j >= g.NY || i >= g.NX) return;
    out[(long long)j * g.NX + i] = (float)in[(long long)j * g.P + i];
}

int launch_to_f32(int prec, const void* in, float* out, const Geom& g, cudaStream_t s)
{
    const dim3 gr = pt_grid(g), bl(32, 8);
    if (prec == 0) k_to_f32<double><<<gr, bl, 0, s>>>((const double*)in, out, g);
    else k_to_f32<float><<<gr, bl, 0, s>>>((const float*)in, out, g);
    return (int)cudaGetLastError();
}

size_t pt_grid_blocks(const Geom& g)
{
    dim3 d = pt_grid(g);
    return (size_t)d.x * d.y;
}

}  // namespace f2d
